#include "host_io.h"

#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <sys/stat.h>
#include <sys/types.h>

#include "../../include/c2graph.h"

namespace c2g {

static thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

const char* last_error() { return g_err.c_str(); }
void clear_error() { g_err.clear(); }

bool file_exists(const std::string& path) {
    struct stat st;
    return stat(path.c_str(), &st) == 0;
}

template <typename T>
static int read_impl(const std::string& path, std::vector<T>& out) {
    static_assert(sizeof(T) == 4, "4-byte elements");
    struct stat st;
    if (stat(path.c_str(), &st) != 0)
        return fail(C2G_ERR_IO, "file:%s not exist.", path.c_str());
    if (st.st_size % 4 != 0)
        return fail(C2G_ERR_FORMAT, "file:%s size %lld is not a multiple of 4", path.c_str(),
                    (long long)st.st_size);
    size_t n = (size_t)st.st_size / 4;
    out.resize(n);
    FILE* fp = fopen(path.c_str(), "rb");
    if (!fp) return fail(C2G_ERR_IO, "cannot open %s: %s", path.c_str(), strerror(errno));
    size_t got = n ? fread(out.data(), 4, n, fp) : 0;
    fclose(fp);
    if (got != n) return fail(C2G_ERR_IO, "short read on %s (%zu of %zu)", path.c_str(), got, n);
    return C2G_OK;
}

int read_array4(const std::string& path, std::vector<int32_t>& out) { return read_impl(path, out); }
int read_array4(const std::string& path, std::vector<float>& out) { return read_impl(path, out); }

int write_array4(const std::string& path, const void* data, size_t n) {
    FILE* fp = fopen(path.c_str(), "wb");
    if (!fp) return fail(C2G_ERR_IO, "cannot create %s: %s", path.c_str(), strerror(errno));
    size_t put = n ? fwrite(data, 4, n, fp) : 0;
    int rc = fclose(fp);
    if (put != n || rc != 0) return fail(C2G_ERR_IO, "short write on %s", path.c_str());
    return C2G_OK;
}

int make_dir(const std::string& path) {
    if (mkdir(path.c_str(), 0755) != 0 && errno != EEXIST)
        return fail(C2G_ERR_IO, "cannot create directory %s: %s", path.c_str(), strerror(errno));
    return C2G_OK;
}

int check_rows(const std::vector<int32_t>& vlist) {
    if (vlist.empty()) return fail(C2G_ERR_FORMAT, "vlist is empty (needs V+1 entries)");
    const int64_t V = (int64_t)vlist.size() - 1;
    if (vlist[0] != 0) return fail(C2G_ERR_FORMAT, "vlist[0] = %d, expected 0", vlist[0]);
    for (int64_t i = 0; i < V; ++i)
        if (vlist[i + 1] < vlist[i]) return fail(C2G_ERR_FORMAT, "vlist not monotone at %lld", (long long)i);
    return C2G_OK;
}

int check_csr(const std::vector<int32_t>& vlist, const std::vector<int32_t>& elist) {
    if (vlist.empty()) return fail(C2G_ERR_FORMAT, "vlist is empty (needs V+1 entries)");
    const int64_t V = (int64_t)vlist.size() - 1;
    const int64_t E = (int64_t)elist.size();
    if (vlist[0] != 0) return fail(C2G_ERR_FORMAT, "vlist[0] = %d, expected 0", vlist[0]);
    for (int64_t i = 0; i < V; ++i)
        if (vlist[i + 1] < vlist[i])
            return fail(C2G_ERR_FORMAT, "vlist not monotone at %lld", (long long)i);
    if ((int64_t)vlist[V] != E)
        return fail(C2G_ERR_FORMAT, "vlist[V] = %d but elist has %lld entries", vlist[V],
                    (long long)E);
    for (int64_t e = 0; e < E; ++e)
        if (elist[e] < 0 || elist[e] >= V)
            return fail(C2G_ERR_FORMAT, "elist[%lld] = %d out of range [0,%lld)", (long long)e,
                        elist[e], (long long)V);
    return C2G_OK;
}

}  // namespace c2g
