// Streaming ingest of the reference's binary edge arrays (the files core/io.hpp:25-40
// reads whole with fread, and DeviceMemory::CudaMemcpyGraph then copies through more
// host vectors, src/sssp/purn/DeviceMemory.cuh:48-67).
//
// Here the edge files (elist and the weight kinds present) are memory-mapped and streamed
// in chunks through two page-locked staging buffers: host threads copy chunk k+1 out of
// the mappings while the device interleaves chunk k, reading the staging buffer directly
// through its mapped device address (over NVLink-C2C on Grace), into the (target, weight)
// records of adj_w / adj_f.  No full-size host vector or device temporary is made, every
// byte of a file is read once, and the target range check runs on the device.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <climits>
#include <cstring>
#include <string>

#include "internal.h"

namespace c2g {

int launch_interleave_chunk(c2g_graph* g, const int* col, const int* w, const int* f, int2* adj_w, int2* adj_f,
                            long long base, long long n, long long* bad);

namespace {

struct Mapped {
    void* p = MAP_FAILED;
    size_t bytes = 0;
    int fd = -1;
    ~Mapped() {
        if (p != MAP_FAILED && bytes) munmap(p, bytes);
        if (fd >= 0) close(fd);
    }
    const int32_t* data() const { return static_cast<const int32_t*>(p); }
    size_t count() const { return bytes / 4; }
};

int map_file(const std::string& path, Mapped& m) {
    m.fd = open(path.c_str(), O_RDONLY);
    if (m.fd < 0) return fail(C2G_ERR_IO, "file:%s not exist.", path.c_str());
    struct stat st;
    if (fstat(m.fd, &st) != 0) return fail(C2G_ERR_IO, "cannot stat %s: %s", path.c_str(), strerror(errno));
    if (st.st_size % 4 != 0)
        return fail(C2G_ERR_FORMAT, "file:%s size %lld is not a multiple of 4", path.c_str(), (long long)st.st_size);
    m.bytes = (size_t)st.st_size;
    if (m.bytes == 0) return C2G_OK;
    m.p = mmap(nullptr, m.bytes, PROT_READ, MAP_PRIVATE, m.fd, 0);
    if (m.p == MAP_FAILED) return fail(C2G_ERR_IO, "cannot map %s: %s", path.c_str(), strerror(errno));
    madvise(m.p, m.bytes, MADV_SEQUENTIAL);
    return C2G_OK;
}

// Page-locked staging: two buffers, each holding one chunk of every streamed array.
struct Staging {
    void* host[2] = {nullptr, nullptr};
    void* dev[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    long long* bad = nullptr;  // device: first edge with a target outside [0, V), LLONG_MAX if none
    ~Staging() {
        for (int b = 0; b < 2; ++b) {
            if (done[b]) cudaEventDestroy(done[b]);
            if (host[b]) cudaFreeHost(host[b]);
        }
        if (bad) cudaFree(bad);
    }
};

}  // namespace

// Chunk size of the stream: 4M edges (16 MB per array per buffer).
constexpr size_t kStreamChunk = size_t(1) << 22;

int stream_graph(c2g_graph* g, const std::string& elist_path, const std::string* w_path, const std::string* f_path) {
    Mapped me, mw, mf;
    int rc;
    if ((rc = map_file(elist_path, me))) return rc;
    if (w_path && (rc = map_file(*w_path, mw))) return rc;
    if (f_path && (rc = map_file(*f_path, mf))) return rc;
    const size_t E = me.count();
    if ((int64_t)E != (int64_t)g->h_row.back())
        return fail(C2G_ERR_FORMAT, "vlist[V] = %d but elist has %zu entries", g->h_row.back(), E);
    if ((w_path && mw.count() < E) || (f_path && mf.count() < E))
        return fail(C2G_ERR_FORMAT, "weight file shorter than elist");
    g->E = (int64_t)E;
    if (w_path) C2G_CUDA(cudaMalloc(&g->adj_w, sizeof(int2) * (E ? E : 1)));
    if (f_path) C2G_CUDA(cudaMalloc(&g->adj_f, sizeof(int2) * (E ? E : 1)));
    if (E == 0) return C2G_OK;
    const int arrays = 1 + (w_path ? 1 : 0) + (f_path ? 1 : 0);
    const size_t chunk = std::min(kStreamChunk, E);
    Staging st;
    for (int b = 0; b < 2; ++b) {
        C2G_CUDA(cudaHostAlloc(&st.host[b], sizeof(int32_t) * chunk * (size_t)arrays, cudaHostAllocMapped));
        C2G_CUDA(cudaHostGetDevicePointer(&st.dev[b], st.host[b], 0));
        C2G_CUDA(cudaEventCreateWithFlags(&st.done[b], cudaEventDisableTiming));
    }
    C2G_CUDA(cudaMalloc(&st.bad, sizeof(long long)));
    const long long none = LLONG_MAX;
    C2G_CUDA(cudaMemcpyAsync(st.bad, &none, sizeof(none), cudaMemcpyHostToDevice, g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    const int32_t* src[3] = {me.data(), w_path ? mw.data() : nullptr, f_path ? mf.data() : nullptr};
    for (size_t base = 0, k = 0; base < E; base += chunk, ++k) {
        const int b = (int)(k & 1);
        const size_t n = std::min(chunk, E - base);
        if (k >= 2) C2G_CUDA(cudaEventSynchronize(st.done[b]));  // its previous chunk is consumed
        int32_t* h = static_cast<int32_t*>(st.host[b]);
        // host threads copy the chunk out of the mappings (page faults read the files)
        int slot = 0;
        int32_t* dst[3] = {nullptr, nullptr, nullptr};
        for (int a = 0; a < 3; ++a)
            if (src[a]) dst[a] = h + (size_t)(slot++) * chunk;
        const long long pieces = (long long)((n + 65535) / 65536);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < pieces * 3; ++i) {
            const int a = (int)(i % 3);
            if (!src[a]) continue;
            const size_t o = (size_t)(i / 3) * 65536;
            std::memcpy(dst[a] + o, src[a] + base + o, sizeof(int32_t) * std::min<size_t>(65536, n - o));
        }
        const int32_t* d = static_cast<const int32_t*>(st.dev[b]);
        slot = 0;
        const int* dcol = d + (size_t)(slot++) * chunk;
        const int* dw = w_path ? d + (size_t)(slot++) * chunk : nullptr;
        const int* df = f_path ? d + (size_t)(slot++) * chunk : nullptr;
        if ((rc = launch_interleave_chunk(g, dcol, dw, df, g->adj_w, g->adj_f, (long long)base, (long long)n, st.bad)))
            return rc;
        C2G_CUDA(cudaEventRecord(st.done[b], g->stream));
    }
    long long bad = LLONG_MAX;
    C2G_CUDA(cudaMemcpyAsync(&bad, st.bad, sizeof(bad), cudaMemcpyDeviceToHost, g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    if (bad != LLONG_MAX)
        return fail(C2G_ERR_FORMAT, "elist[%lld] = %d out of range [0,%d)", bad, me.data()[bad], g->V);
    return C2G_OK;
}

}  // namespace c2g
