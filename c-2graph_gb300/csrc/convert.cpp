// Text edge lists to the reference's binary graph (utils/convert2binary.cpp:10-137): the
// origin/ files every program here reads.  Same bytes as the reference converter for the
// inputs it accepts:
//   * a line is read as `iss >> src >> dstPart` (an int, then the next whitespace-free
//     token); a line without both is skipped, as is one whose int does not fit;
//   * the token is split at ':' and each piece read as stoi reads it (sign, decimal digits,
//     anything after them ignored);
//   * V is the largest id seen plus one; self-loops are dropped; each row is sorted and its
//     repeats removed;
//   * weights: rand() % 100 + 1 per edge in row order from an unseeded rand() (seed 1),
//     flist = (double)w / (row sum of w), rounded to float.
// Where the reference stops with an uncaught exception (a piece stoi rejects: empty, no
// digits, out of int range) or indexes out of range (a negative id), this converter returns
// C2G_ERR_FORMAT naming the line, and writes nothing.  The lines are parsed in parallel;
// only the set of (src, dst) pairs matters, since rows are sorted and deduplicated.
#include <fcntl.h>
#include <omp.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/c2graph.h"
#include "host_io.h"

namespace c2g {
namespace {

// glibc's rand(): the additive feedback generator of random(3) with a 31-word state (TYPE_3):
// the state is seeded by the Park-Miller generator r[k] = 16807 r[k-1] mod (2^31 - 1), then
// r[k] = r[k-31] + r[k-3] (mod 2^32) with the first 310 values dropped; rand() returns
// r[k] >> 1.  Restated from the published description of the algorithm; the tests compare
// it with the C library's rand() on this machine.
class GlibcRand {
  public:
    explicit GlibcRand(uint32_t seed) {
        int64_t r = seed ? seed : 1;
        buf_[0] = (uint32_t)r;
        for (int k = 1; k < 31; ++k) {
            r = (16807 * r) % 2147483647;
            buf_[k] = (uint32_t)r;
        }
        for (int k = 31; k < 34; ++k) buf_[k] = buf_[k - 31];
        n_ = 34;
        for (int k = 34; k < 344; ++k) step();
    }
    int next() { return (int)(step() >> 1); }

  private:
    uint32_t step() {
        const uint32_t v = buf_[(n_ - 31) % 34] + buf_[(n_ - 3) % 34];
        buf_[n_ % 34] = v;
        ++n_;
        return v;
    }
    uint32_t buf_[34];
    uint64_t n_;
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

// istream >> int: whitespace, an optional sign, at least one digit; false (the line is
// skipped) when there are no digits or the value does not fit in an int.
bool read_int_stream(const char*& s, const char* e, int64_t& out) {
    while (s < e && is_space(*s)) ++s;
    const char* p = s;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    if (p >= e || *p < '0' || *p > '9') return false;
    int64_t v = 0;
    bool over = false;
    while (p < e && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p++ - '0');
        if (v > (int64_t)INT_MAX + 1) over = true, v = (int64_t)INT_MAX + 1;
    }
    v = neg ? -v : v;
    if (over || v > INT_MAX || v < INT_MIN) return false;
    s = p;
    out = v;
    return true;
}

// stoi on one ':'-separated piece: 1 and the value, or 0 where stoi throws.
int read_int_stoi(const char* s, const char* e, int64_t& out) {
    bool neg = false;
    if (s < e && (*s == '+' || *s == '-')) neg = *s++ == '-';
    if (s >= e || *s < '0' || *s > '9') return 0;
    int64_t v = 0;
    while (s < e && *s >= '0' && *s <= '9') {
        v = v * 10 + (*s++ - '0');
        if (v > (int64_t)INT_MAX + 1) return 0;
    }
    v = neg ? -v : v;
    if (v > INT_MAX || v < INT_MIN) return 0;
    out = v;
    return 1;
}

struct Part {
    std::vector<std::pair<int32_t, int32_t>> pairs;
    int64_t maxid = 0;
    int64_t bad_line = -1;  // first line of the chunk the reference would stop on (chunk-local)
    int64_t lines = 0;
};

// Parse [s, e) (whole lines) into p.
void parse_chunk(const char* s, const char* e, Part& p) {
    while (s < e) {
        const char* nl = static_cast<const char*>(memchr(s, '\n', (size_t)(e - s)));
        const char* le = nl ? nl : e;
        const char* c = s;
        int64_t src = 0;
        if (read_int_stream(c, le, src)) {
            while (c < le && is_space(*c)) ++c;
            const char* t = c;
            while (c < le && !is_space(*c)) ++c;
            if (c > t) {  // the token [t, c), split at ':' (a trailing ':' ends no piece)
                const char* q = t;
                bool ok = src >= 0;
                std::vector<int32_t> dst;
                while (ok && q < c) {
                    const char* r = q;
                    while (r < c && *r != ':') ++r;
                    int64_t d = 0;
                    if (!read_int_stoi(q, r, d) || d < 0) ok = false;
                    dst.push_back((int32_t)d);
                    q = r < c ? r + 1 : r;
                }
                if (!ok) {
                    if (p.bad_line < 0) p.bad_line = p.lines;
                } else {
                    p.maxid = std::max(p.maxid, src);
                    for (int32_t d : dst) {
                        p.maxid = std::max<int64_t>(p.maxid, d);
                        if (d != src) p.pairs.emplace_back((int32_t)src, d);
                    }
                }
            }
        }
        ++p.lines;
        s = nl ? nl + 1 : e;
    }
}

int convert_text(const std::string& text, const std::string& dir, int64_t* vertices, int64_t* edges) {
    const int fd = open(text.c_str(), O_RDONLY);
    if (fd < 0) return fail(C2G_ERR_IO, "Error opening file: %s", text.c_str());
    struct stat st;
    if (fstat(fd, &st) != 0) {
        close(fd);
        return fail(C2G_ERR_IO, "cannot stat %s", text.c_str());
    }
    std::string buf((size_t)st.st_size, '\0');
    size_t got = 0;
    while (got < buf.size()) {
        const ssize_t k = read(fd, &buf[got], buf.size() - got);
        if (k <= 0) break;
        got += (size_t)k;
    }
    close(fd);
    if (got != buf.size()) return fail(C2G_ERR_IO, "short read on %s", text.c_str());
    // chunks of whole lines, one per thread
    const int T = std::max(1, std::min(omp_get_max_threads(), 64));
    std::vector<size_t> cut((size_t)T + 1, buf.size());
    cut[0] = 0;
    for (int t = 1; t < T; ++t) {
        size_t x = std::max(cut[t - 1], buf.size() * (size_t)t / (size_t)T);
        while (x < buf.size() && x > 0 && buf[x - 1] != '\n') ++x;
        cut[t] = x;
    }
    std::vector<Part> parts((size_t)T);
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) parse_chunk(buf.data() + cut[t], buf.data() + cut[t + 1], parts[t]);
    std::string().swap(buf);
    int64_t maxid = 0, line0 = 0;
    for (const Part& p : parts) {
        if (p.bad_line >= 0)
            return fail(C2G_ERR_FORMAT, "%s: line %lld has a destination that is not a non-negative int",
                        text.c_str(), (long long)(line0 + p.bad_line + 1));
        line0 += p.lines;
        maxid = std::max(maxid, p.maxid);
    }
    if (maxid >= INT_MAX) return fail(C2G_ERR_RANGE, "%s: vertex id %lld is too large", text.c_str(), (long long)maxid);
    const int32_t V = (int32_t)maxid + 1;
    // rows: a counting sort of the pairs by source, then each row sorted and deduplicated
    std::vector<int64_t> cnt((size_t)V + 1, 0);
    for (const Part& p : parts)
        for (const auto& e : p.pairs) ++cnt[(size_t)e.first + 1];
    for (int32_t v = 0; v < V; ++v) cnt[(size_t)v + 1] += cnt[v];
    std::vector<int32_t> col((size_t)cnt[V]);
    {
        std::vector<int64_t> at(cnt.begin(), cnt.end() - 1);
        for (Part& p : parts) {
            for (const auto& e : p.pairs) col[(size_t)at[e.first]++] = e.second;
            std::vector<std::pair<int32_t, int32_t>>().swap(p.pairs);
        }
    }
    std::vector<int32_t> vlist((size_t)V + 1, 0), keep((size_t)V, 0);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int32_t v = 0; v < V; ++v) {
        int32_t* r = col.data() + cnt[v];
        const int64_t n = cnt[(size_t)v + 1] - cnt[v];
        std::sort(r, r + n);
        keep[v] = (int32_t)(std::unique(r, r + n) - r);
    }
    for (int32_t v = 0; v < V; ++v) {
        if ((int64_t)vlist[v] + keep[v] > INT_MAX) return fail(C2G_ERR_RANGE, "%s: more than 2^31 - 1 edges", text.c_str());
        vlist[(size_t)v + 1] = vlist[v] + keep[v];
    }
    const size_t E = (size_t)vlist[V];
    std::vector<int32_t> elist(E), wlist(E);
    std::vector<float> flist(E);
    GlibcRand rnd(1);
    for (int32_t v = 0; v < V; ++v) {
        const int32_t* r = col.data() + cnt[v];
        int sum = 0;
        for (int32_t x = 0; x < keep[v]; ++x) {
            const size_t j = (size_t)vlist[v] + x;
            elist[j] = r[x];
            wlist[j] = rnd.next() % 100 + 1;
            sum += wlist[j];
        }
        for (int32_t x = 0; x < keep[v]; ++x) {
            const size_t j = (size_t)vlist[v] + x;
            flist[j] = (float)(1.0 * wlist[j] / sum);
        }
    }
    int rc;
    if ((rc = make_dir(dir))) return rc;
    if ((rc = make_dir(dir + "/origin"))) return rc;
    const std::string o = dir + "/origin/";
    if ((rc = write_array4(o + "vlist.bin", vlist.data(), vlist.size()))) return rc;
    if ((rc = write_array4(o + "elist.bin", elist.data(), elist.size()))) return rc;
    if ((rc = write_array4(o + "wlist.bin", wlist.data(), wlist.size()))) return rc;
    if ((rc = write_array4(o + "flist.bin", flist.data(), flist.size()))) return rc;
    if (vertices) *vertices = V;
    if (edges) *edges = (int64_t)E;
    return C2G_OK;
}

}  // namespace
}  // namespace c2g

extern "C" int c2g_convert_text(const char* text_path, const char* dir, int64_t* max_vertex, int64_t* vertices,
                                int64_t* edges) {
    if (!text_path || !dir) return c2g::fail(C2G_ERR_ARG, "convert: path is NULL");
    int64_t V = 0, E = 0;
    const int rc = c2g::convert_text(text_path, dir, &V, &E);
    if (rc) return rc;
    if (max_vertex) *max_vertex = V - 1;
    if (vertices) *vertices = V;
    if (edges) *edges = E;
    return C2G_OK;
}
