// gbs_ingest.cu -- graph ingest on the GPU (sm_103a): the reference's text
// and binary CSR readers (graph/csr.c:4-299), duplicate-edge removal
// (partition/csr_partition_bin_mpi.c:47-105) and the build of a resident
// graph, all on the device.
//
// Text (scan_csr_idx + read_graph_csr, graph/csr.c:4-202): "p <name> v_num
// e_num offset g_v_size" then "a v_id v_to weight" lines (other lines, e.g.
// "c" comments, are skipped); the first e_num "a" lines are read.  SEND:
// row = v_id - offset, column = v_to - 1; RECV: row = v_to - offset, column =
// v_id - 1.  Rows keep their edges in file order (the reference fills them in
// file order).  The weight is (double)v_to / (double)v_num with the file's
// v_to, and the reference stores the k-th line's weight at CSR position k
// (edge_info[e_num_read], :46), not at that edge's position: the two agree
// only for a file sorted by row.  Both are kept here as the reference has
// them; the third number of an "a" line is read and ignored, as there.
//
// Binary (read_csr_bin, graph/csr.c:211-299): int64 v_num, e_num, offset,
// g_v_size, then e_num int64 (from, to) pairs.  SEND: row = from - offset,
// column = to - target_offset; RECV: row = to - offset, column = from -
// target_offset (target_offset is the reference's OFFSET: 1, or 0 in its
// Graph500 build).  The weight of CSR position p is 0.1 for even p and 0.2 for
// odd p (:293-298).  With dedup, a (from, to) pair seen earlier in the file is
// dropped first, as remove_duplicate does.
//
// Device work: the text is cut into 512-byte chunks; each chunk counts and
// then lists the "a" lines that start in it (one exclusive scan between), and
// one thread per line parses its numbers.  The CSR is a stable radix sort of
// the edges by row (CUB), so rows keep file order; the resident graph's rows
// are then sorted by (weight, column) with two or three more stable passes.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbs_host.hpp"

namespace gbs {
namespace {

constexpr uint64_t kChunk = 512;     // bytes of text per counting thread

enum IngestErr : uint32_t {
    kIngOk = 0,
    kIngSyntax = 1,      // an "a" line without three integers
    kIngRange = 2,       // a row or column outside [0, v_num)
    kIngDupRange = 3,    // a pair outside [0, 2^32) (duplicate removal)
};

struct DevErr {
    uint32_t code;
    uint32_t pad;
    unsigned long long where;   // edge index (file order)
};

__device__ __forceinline__ void set_err(DevErr *e, uint32_t code, unsigned long long where) {
    if (atomicCAS(&e->code, 0u, code) == 0u) e->where = where;
}

__device__ __forceinline__ bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\r'; }

// An "a" record starts at byte i: i is the start of a line (after optional
// blanks) whose first token is exactly "a".
__device__ __forceinline__ bool a_line_at(const char *buf, unsigned long long len, unsigned long long i) {
    if (i != 0 && buf[i - 1] != '\n') return false;
    while (i < len && is_blank(buf[i])) ++i;
    return i + 1 < len && buf[i] == 'a' && (buf[i + 1] == ' ' || buf[i + 1] == '\t');
}

__global__ void k_count_lines(const char *__restrict__ buf, unsigned long long len, unsigned long long chunks,
                              unsigned long long *__restrict__ cnt) {
    for (unsigned long long c = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; c < chunks;
         c += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long b = c * kChunk, e = min(len, b + kChunk);
        unsigned long long k = 0;
        for (unsigned long long i = b; i < e; ++i) k += a_line_at(buf, len, i) ? 1ull : 0ull;
        cnt[c] = k;
    }
}

__global__ void k_list_lines(const char *__restrict__ buf, unsigned long long len, unsigned long long chunks,
                             const unsigned long long *__restrict__ base, unsigned long long *__restrict__ pos,
                             unsigned long long cap) {
    for (unsigned long long c = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; c < chunks;
         c += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long b = c * kChunk, e = min(len, b + kChunk);
        unsigned long long k = base[c];
        for (unsigned long long i = b; i < e && k < cap; ++i)
            if (a_line_at(buf, len, i)) pos[k++] = i;
    }
}

// Reads a decimal integer (optional sign) after blanks; false if none.
__device__ __forceinline__ bool read_int(const char *buf, unsigned long long len, unsigned long long &i,
                                         long long &out) {
    while (i < len && is_blank(buf[i])) ++i;
    bool neg = false;
    if (i < len && (buf[i] == '-' || buf[i] == '+')) {
        neg = buf[i] == '-';
        ++i;
    }
    if (i >= len || buf[i] < '0' || buf[i] > '9') return false;
    unsigned long long v = 0;
    while (i < len && buf[i] >= '0' && buf[i] <= '9') v = v * 10ull + (unsigned long long)(buf[i++] - '0');
    out = neg ? -(long long)v : (long long)v;
    return true;
}

// One thread per "a" record: v_id and v_to (the weight token is checked and
// ignored, as the reference ignores it).
__global__ void k_parse_lines(const char *__restrict__ buf, unsigned long long len,
                              const unsigned long long *__restrict__ pos, unsigned long long count,
                              long long *__restrict__ x, long long *__restrict__ y, DevErr *err) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < count;
         k += (unsigned long long)gridDim.x * blockDim.x) {
        unsigned long long i = pos[k];
        while (is_blank(buf[i])) ++i;
        ++i;   // the 'a'
        long long a = 0, b = 0, w = 0;
        if (!read_int(buf, len, i, a) || !read_int(buf, len, i, b) || !read_int(buf, len, i, w)) {
            set_err(err, kIngSyntax, k);
            continue;
        }
        x[k] = a;
        y[k] = b;
    }
}

// Row and column of every edge (file order), checked against [0, v_num).
__global__ void k_rows(const long long *__restrict__ x, const long long *__restrict__ y, unsigned long long m,
                       long long row_shift, long long col_shift, bool by_y, long long v_num,
                       uint32_t *__restrict__ row, uint32_t *__restrict__ col, uint32_t *__restrict__ idx,
                       DevErr *err) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < m;
         k += (unsigned long long)gridDim.x * blockDim.x) {
        const long long r = (by_y ? y[k] : x[k]) - row_shift;
        const long long c = (by_y ? x[k] : y[k]) - col_shift;
        if (r < 0 || r >= v_num || c < 0 || c >= v_num) {
            set_err(err, kIngRange, k);
            row[k] = 0;
            col[k] = 0;
        } else {
            row[k] = (uint32_t)r;
            col[k] = (uint32_t)c;
        }
        idx[k] = (uint32_t)k;
    }
}

__global__ void k_degrees(const uint32_t *__restrict__ row, unsigned long long m, unsigned long long *__restrict__ deg) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < m;
         k += (unsigned long long)gridDim.x * blockDim.x)
        atomicAdd(deg + row[k], 1ull);
}

// CSR position p: the column of the p-th edge in (row, file order); the
// weight as the reference stores it (text: the p-th line's v_to / v_num;
// binary: 0.1 / 0.2 by the parity of p).
__global__ void k_place(const uint32_t *__restrict__ sorted_idx, const uint32_t *__restrict__ col,
                        const long long *__restrict__ raw_to, unsigned long long m, bool text, double v_num,
                        uint32_t *__restrict__ out_col, double *__restrict__ out_w) {
    for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < m;
         p += (unsigned long long)gridDim.x * blockDim.x) {
        out_col[p] = col[sorted_idx[p]];
        out_w[p] = text ? (double)raw_to[p] / v_num : ((p & 1ull) ? 0.2 : 0.1);
    }
}

// Duplicate removal: key = (from << 32) | to of the raw pair.
__global__ void k_pair_keys(const long long *__restrict__ x, const long long *__restrict__ y, unsigned long long m,
                            unsigned long long *__restrict__ key, uint32_t *__restrict__ idx, DevErr *err) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < m;
         k += (unsigned long long)gridDim.x * blockDim.x) {
        const long long a = x[k], b = y[k];
        if (a < 0 || b < 0 || a > 0xFFFFFFFFll || b > 0xFFFFFFFFll) {
            set_err(err, kIngDupRange, k);
            key[k] = 0;
        } else {
            key[k] = ((unsigned long long)a << 32) | (unsigned long long)b;
        }
        idx[k] = (uint32_t)k;
    }
}

// keep[original index] = 1 for the first occurrence of each pair (the sort is
// stable, so the first of a run of equal keys is the earliest in the file).
__global__ void k_first_of_run(const unsigned long long *__restrict__ key, const uint32_t *__restrict__ idx,
                               unsigned long long m, uint32_t *__restrict__ keep) {
    for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < m;
         p += (unsigned long long)gridDim.x * blockDim.x)
        keep[idx[p]] = (p == 0 || key[p] != key[p - 1]) ? 1u : 0u;
}

__global__ void k_compact(const long long *__restrict__ x, const long long *__restrict__ y,
                          const uint32_t *__restrict__ keep, const unsigned long long *__restrict__ at,
                          unsigned long long m, long long *__restrict__ ox, long long *__restrict__ oy) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < m;
         k += (unsigned long long)gridDim.x * blockDim.x)
        if (keep[k]) {
            ox[at[k]] = x[k];
            oy[at[k]] = y[k];
        }
}

__global__ void k_widen(const uint32_t *__restrict__ in, unsigned long long m, unsigned long long *__restrict__ out) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k <= m;
         k += (unsigned long long)gridDim.x * blockDim.x)
        out[k] = k < m ? in[k] : 0ull;
}

__global__ void k_split(const long long *__restrict__ pairs, unsigned long long m, long long *__restrict__ x,
                        long long *__restrict__ y) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < m;
         k += (unsigned long long)gridDim.x * blockDim.x) {
        x[k] = pairs[2 * k];
        y[k] = pairs[2 * k + 1];
    }
}

// ------------------------------------------------- resident graph build
__global__ void k_row_of(const unsigned long long *__restrict__ row, uint32_t n, uint32_t *__restrict__ row_of) {
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps)
        for (unsigned long long e = row[v] + lane; e < row[v + 1]; e += 32ull) row_of[e] = v;
}

// Weight bits of the resident graph; flags bit 0: a weight is negative or not
// finite, bit 1: not an integer in [0, 2^32) (uint32 graphs), bit 2: zero.
template <int WT>
__global__ void k_weight_bits(const double *__restrict__ w, unsigned long long m, unsigned long long *__restrict__ bits,
                              uint32_t *flags) {
    uint32_t f = 0;
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < m;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        double x = w[e];
        if (!(x >= 0.0) || isinf(x)) {
            f |= 1u;
            x = 0.0;
        }
        if (x == 0.0) {
            f |= 4u;
            x = 0.0;   // -0 as +0
        }
        if (WT == 2) {
            bits[e] = (unsigned long long)__double_as_longlong(x);
        } else if (WT == 1) {
            bits[e] = __float_as_uint(__double2float_rn(x));
        } else {
            if (x != floor(x) || x > 4294967295.0) f |= 2u;
            bits[e] = (unsigned long long)(uint32_t)x;
        }
    }
    if (f) atomicOr(flags, f);
}

__global__ void k_key_row_w(const uint32_t *__restrict__ row_of, const unsigned long long *__restrict__ wbits,
                            const uint32_t *__restrict__ id, unsigned long long m, unsigned long long *__restrict__ key) {
    for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < m;
         p += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t e = id[p];
        key[p] = ((unsigned long long)row_of[e] << 32) | wbits[e];
    }
}

template <typename K>
__global__ void k_gather_key(const K *__restrict__ src, const uint32_t *__restrict__ id, unsigned long long m,
                             K *__restrict__ key) {
    for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < m;
         p += (unsigned long long)gridDim.x * blockDim.x)
        key[p] = src[id[p]];
}

__global__ void k_adj(const uint32_t *__restrict__ id, const uint32_t *__restrict__ col,
                      const unsigned long long *__restrict__ wbits, unsigned long long m, bool f64, uint2 *__restrict__ adj,
                      unsigned long long *__restrict__ w64) {
    for (unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; p < m;
         p += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t e = id[p];
        adj[p] = make_uint2(col[e], f64 ? 0u : (uint32_t)wbits[e]);
        if (f64) w64[p] = wbits[e];
    }
}

__global__ void k_row32(const unsigned long long *__restrict__ row, uint32_t n, uint32_t *__restrict__ row32) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x)
        row32[v] = (uint32_t)row[v];
}

// ----------------------------------------------------------------- host
// Device buffers of one ingest call, released on every exit path.
struct Bufs {
    std::vector<void *> p;
    template <typename T> cudaError_t get(T **out, size_t count) {
        void *q = nullptr;
        const cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
        if (e == cudaSuccess) p.push_back(q);
        *out = static_cast<T *>(q);
        return e;
    }
    void release(void *q) {
        for (auto &x : p)
            if (x == q) {
                cudaFree(x);
                x = nullptr;
            }
    }
    ~Bufs() {
        for (void *q : p) cudaFree(q);
    }
};

#define ING_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(e_ == cudaErrorMemoryAllocation ? GBS_ERR_NO_MEMORY : GBS_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                 \
    } while (0)

int grid_for(unsigned long long items, int sms) {
    const unsigned long long b = (items + 255) / 256;
    return (int)std::max<unsigned long long>(1, std::min<unsigned long long>(b, (unsigned long long)sms * 16));
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

gbs_status check_err(const DevErr &e, const char *what) {
    if (e.code == kIngOk) return GBS_OK;
    const char *why = e.code == kIngSyntax    ? "an \"a\" line without three integers"
                      : e.code == kIngRange   ? "a row or column outside [0, v_num)"
                                              : "a vertex id outside [0, 2^32)";
    return fail(GBS_ERR_INVALID_ARG, std::string(what) + ": edge " + std::to_string(e.where) + ": " + why);
}

// CUB radix sort of (key, value) pairs, stable; out buffers given.
template <typename K>
gbs_status sort_pairs(const K *kin, K *kout, const uint32_t *vin, uint32_t *vout, unsigned long long m,
                      cudaStream_t s, Bufs &bufs, int end_bit = (int)sizeof(K) * 8) {
    size_t tmp = 0;
    ING_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, kin, kout, vin, vout, (int64_t)m, 0, end_bit, s));
    void *t = nullptr;
    ING_CUDA(bufs.get(reinterpret_cast<char **>(&t), tmp));
    ING_CUDA(cub::DeviceRadixSort::SortPairs(t, tmp, kin, kout, vin, vout, (int64_t)m, 0, end_bit, s));
    bufs.release(t);
    return GBS_OK;
}

gbs_status excl_sum(const unsigned long long *in, unsigned long long *out, unsigned long long count, cudaStream_t s,
                    Bufs &bufs) {
    size_t tmp = 0;
    ING_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, (int64_t)count, s));
    void *t = nullptr;
    ING_CUDA(bufs.get(reinterpret_cast<char **>(&t), tmp));
    ING_CUDA(cub::DeviceScan::ExclusiveSum(t, tmp, in, out, (int64_t)count, s));
    bufs.release(t);
    return GBS_OK;
}

// Edges (x, y) in file order -> CSR in the reference's layout.
gbs_status build_csr(const long long *dx, const long long *dy, unsigned long long m, long long v_num, long long row_shift,
                     long long col_shift, bool by_y, bool text, cudaStream_t s, int sms, Bufs &bufs,
                     gbs_device_csr *out) {
    DevErr *d_err = nullptr;
    ING_CUDA(bufs.get(&d_err, 1));
    ING_CUDA(cudaMemsetAsync(d_err, 0, sizeof(DevErr), s));
    uint32_t *row = nullptr, *col = nullptr, *idx = nullptr, *row_s = nullptr, *idx_s = nullptr;
    ING_CUDA(bufs.get(&row, m));
    ING_CUDA(bufs.get(&col, m));
    ING_CUDA(bufs.get(&idx, m));
    const int gb = grid_for(m, sms);
    k_rows<<<gb, 256, 0, s>>>(dx, dy, m, row_shift, col_shift, by_y, v_num, row, col, idx, d_err);
    ING_CUDA(cudaGetLastError());
    DevErr he{};
    ING_CUDA(cudaMemcpyAsync(&he, d_err, sizeof(he), cudaMemcpyDeviceToHost, s));
    ING_CUDA(cudaStreamSynchronize(s));
    gbs_status st = check_err(he, text ? "text graph" : "binary graph");
    if (st != GBS_OK) return st;
    unsigned long long *deg = nullptr;
    ING_CUDA(bufs.get(&deg, (size_t)v_num + 1));
    ING_CUDA(cudaMemsetAsync(deg, 0, sizeof(unsigned long long) * ((size_t)v_num + 1), s));
    k_degrees<<<gb, 256, 0, s>>>(row, m, deg);
    ING_CUDA(cudaGetLastError());
    ING_CUDA(cudaMalloc(&out->d_row, sizeof(unsigned long long) * ((size_t)v_num + 1)));
    st = excl_sum(deg, out->d_row, (unsigned long long)v_num + 1, s, bufs);
    if (st != GBS_OK) return st;
    ING_CUDA(bufs.get(&row_s, m));
    ING_CUDA(bufs.get(&idx_s, m));
    int bits = 1;
    while (bits < 32 && (1ll << bits) < v_num) ++bits;
    st = sort_pairs<uint32_t>(row, row_s, idx, idx_s, m, s, bufs, bits);
    if (st != GBS_OK) return st;
    ING_CUDA(cudaMalloc(&out->d_col, sizeof(uint32_t) * (m ? m : 1)));
    ING_CUDA(cudaMalloc(&out->d_w, sizeof(double) * (m ? m : 1)));
    // text weights come from the raw v_to of each line, in file order
    k_place<<<gb, 256, 0, s>>>(idx_s, col, dy, m, text, (double)v_num, out->d_col, out->d_w);
    ING_CUDA(cudaGetLastError());
    ING_CUDA(cudaStreamSynchronize(s));
    out->n = (uint32_t)v_num;
    out->m = m;
    return GBS_OK;
}

// File bytes into a pinned host buffer.
gbs_status read_file(const char *path, std::vector<char> &host, char **pinned, size_t &len) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(GBS_ERR_INVALID_ARG, std::string("cannot open ") + path);
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(f);
        return fail(GBS_ERR_INVALID_ARG, std::string("cannot size ") + path);
    }
    len = (size_t)sz;
    char *p = nullptr;
    if (cudaHostAlloc(reinterpret_cast<void **>(&p), len ? len : 1, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        host.resize(len ? len : 1);
        p = host.data();
    } else {
        *pinned = p;
    }
    const size_t got = len ? std::fread(p, 1, len, f) : 0;
    std::fclose(f);
    if (got != len) return fail(GBS_ERR_INVALID_ARG, std::string("short read of ") + path);
    if (!*pinned) *pinned = nullptr;
    return GBS_OK;
}

struct PinnedFree {
    char *p = nullptr;
    ~PinnedFree() {
        if (p) cudaFreeHost(p);
    }
};

// The "p" record: the first line whose first token is "p", before any "a".
gbs_status text_header(const char *buf, size_t len, long long hdr[4]) {
    size_t i = 0;
    while (i < len) {
        size_t j = i;
        while (j < len && (buf[j] == ' ' || buf[j] == '\t' || buf[j] == '\r')) ++j;
        size_t e = j;
        while (e < len && buf[e] != '\n') ++e;
        if (j + 1 < len && buf[j] == 'a' && (buf[j + 1] == ' ' || buf[j + 1] == '\t'))
            return fail(GBS_ERR_INVALID_ARG, "text graph: an \"a\" line before the \"p\" line");
        if (j + 1 < len && buf[j] == 'p' && (buf[j + 1] == ' ' || buf[j + 1] == '\t')) {
            std::string line(buf + j + 1, buf + e);
            char name[64] = {0};
            long long v[4];
            if (std::sscanf(line.c_str(), " %63s %lld %lld %lld %lld", name, &v[0], &v[1], &v[2], &v[3]) != 5)
                return fail(GBS_ERR_INVALID_ARG, "text graph: malformed \"p\" line");
            for (int k = 0; k < 4; ++k) hdr[k] = v[k];
            return GBS_OK;
        }
        i = e + 1;
    }
    return fail(GBS_ERR_INVALID_ARG, "text graph: no \"p\" line");
}

gbs_status check_header(const long long h[4]) {
    if (h[0] < 1 || h[0] > 0x7FFFFFFFll) return fail(GBS_ERR_INVALID_ARG, "v_num must be in [1, 2^31)");
    if (h[1] < 0 || h[1] >= 0xFFFFFFFFll) return fail(GBS_ERR_UNSUPPORTED, "e_num must be in [0, 2^32 - 1)");
    return GBS_OK;
}

}  // namespace

// Parses text already in memory (host bytes).
gbs_status ingest_text(const char *bytes, size_t len, int direction, gbs_device_csr *out, gbs_ingest_info *info) {
    long long hdr[4];
    gbs_status st = text_header(bytes, len, hdr);
    if (st != GBS_OK) return st;
    st = check_header(hdr);
    if (st != GBS_OK) return st;
    int dev = 0, sms = 0;
    ING_CUDA(cudaGetDevice(&dev));
    ING_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s;
    ING_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamFree {
        cudaStream_t s;
        ~StreamFree() { cudaStreamDestroy(s); }
    } sf{s};
    Bufs bufs;
    cudaEvent_t ev[3];
    for (auto &e : ev) ING_CUDA(cudaEventCreate(&e));
    struct EvFree {
        cudaEvent_t *e;
        ~EvFree() {
            for (int i = 0; i < 3; ++i) cudaEventDestroy(e[i]);
        }
    } ef{ev};
    char *dbuf = nullptr;
    ING_CUDA(bufs.get(&dbuf, len + 1));
    ING_CUDA(cudaEventRecord(ev[0], s));
    ING_CUDA(cudaMemcpyAsync(dbuf, bytes, len, cudaMemcpyHostToDevice, s));
    const unsigned long long chunks = (len + kChunk - 1) / kChunk;
    unsigned long long *cnt = nullptr, *base = nullptr;
    ING_CUDA(bufs.get(&cnt, chunks + 1));
    ING_CUDA(bufs.get(&base, chunks + 1));
    ING_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (chunks + 1), s));
    k_count_lines<<<grid_for(chunks, sms), 256, 0, s>>>(dbuf, len, chunks, cnt);
    ING_CUDA(cudaGetLastError());
    st = excl_sum(cnt, base, chunks + 1, s, bufs);
    if (st != GBS_OK) return st;
    unsigned long long lines = 0;
    ING_CUDA(cudaMemcpyAsync(&lines, base + chunks, sizeof(lines), cudaMemcpyDeviceToHost, s));
    ING_CUDA(cudaStreamSynchronize(s));
    // the reference stops after e_num records
    const unsigned long long m = std::min<unsigned long long>(lines, (unsigned long long)hdr[1]);
    unsigned long long *pos = nullptr;
    ING_CUDA(bufs.get(&pos, m));
    k_list_lines<<<grid_for(chunks, sms), 256, 0, s>>>(dbuf, len, chunks, base, pos, m);
    ING_CUDA(cudaGetLastError());
    long long *dx = nullptr, *dy = nullptr;
    ING_CUDA(bufs.get(&dx, m));
    ING_CUDA(bufs.get(&dy, m));
    DevErr *d_err = nullptr;
    ING_CUDA(bufs.get(&d_err, 1));
    ING_CUDA(cudaMemsetAsync(d_err, 0, sizeof(DevErr), s));
    k_parse_lines<<<grid_for(m, sms), 256, 0, s>>>(dbuf, len, pos, m, dx, dy, d_err);
    ING_CUDA(cudaGetLastError());
    DevErr he{};
    ING_CUDA(cudaMemcpyAsync(&he, d_err, sizeof(he), cudaMemcpyDeviceToHost, s));
    ING_CUDA(cudaEventRecord(ev[1], s));
    ING_CUDA(cudaStreamSynchronize(s));
    st = check_err(he, "text graph");
    if (st != GBS_OK) return st;
    bufs.release(dbuf);
    bufs.release(pos);
    const bool send = direction != GBS_DIR_RECV;
    // SEND: row = v_id - offset, col = v_to - 1; RECV: row = v_to - offset, col = v_id - 1
    st = build_csr(dx, dy, m, hdr[0], hdr[2], 1, !send, true, s, sms, bufs, out);
    if (st != GBS_OK) return st;
    ING_CUDA(cudaEventRecord(ev[2], s));
    ING_CUDA(cudaEventSynchronize(ev[2]));
    if (info) {
        float a = 0.f, b = 0.f;
        ING_CUDA(cudaEventElapsedTime(&a, ev[0], ev[1]));
        ING_CUDA(cudaEventElapsedTime(&b, ev[1], ev[2]));
        info->v_num = hdr[0];
        info->e_num = hdr[1];
        info->offset = hdr[2];
        info->g_v_size = hdr[3];
        info->records = lines;
        info->edges = m;
        info->duplicates = 0;
        info->parse_ms = a;
        info->build_ms = b;
    }
    return GBS_OK;
}

gbs_status ingest_bin(const char *bytes, size_t len, int direction, long long target_offset, int dedup,
                      gbs_device_csr *out, gbs_ingest_info *info) {
    if (len < 32) return fail(GBS_ERR_INVALID_ARG, "binary graph: shorter than its 32-byte header");
    long long hdr[4];
    std::memcpy(hdr, bytes, 32);
    gbs_status st = check_header(hdr);
    if (st != GBS_OK) return st;
    const unsigned long long m0 = (unsigned long long)hdr[1];
    if (len < 32 + 16 * m0) return fail(GBS_ERR_INVALID_ARG, "binary graph: fewer pairs than e_num");
    int dev = 0, sms = 0;
    ING_CUDA(cudaGetDevice(&dev));
    ING_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s;
    ING_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamFree {
        cudaStream_t s;
        ~StreamFree() { cudaStreamDestroy(s); }
    } sf{s};
    Bufs bufs;
    cudaEvent_t ev[3];
    for (auto &e : ev) ING_CUDA(cudaEventCreate(&e));
    struct EvFree {
        cudaEvent_t *e;
        ~EvFree() {
            for (int i = 0; i < 3; ++i) cudaEventDestroy(e[i]);
        }
    } ef{ev};
    // pairs are interleaved (from, to): copy both into one array, then split
    long long *pairs = nullptr, *dx = nullptr, *dy = nullptr;
    ING_CUDA(bufs.get(&pairs, 2 * m0));
    ING_CUDA(bufs.get(&dx, m0));
    ING_CUDA(bufs.get(&dy, m0));
    ING_CUDA(cudaEventRecord(ev[0], s));
    ING_CUDA(cudaMemcpyAsync(pairs, bytes + 32, 16 * m0, cudaMemcpyHostToDevice, s));
    k_split<<<grid_for(m0, sms), 256, 0, s>>>(pairs, m0, dx, dy);
    ING_CUDA(cudaGetLastError());
    ING_CUDA(cudaStreamSynchronize(s));
    bufs.release(pairs);
    unsigned long long m = m0, dups = 0;
    if (dedup && m0) {
        unsigned long long *key = nullptr, *key_s = nullptr, *at = nullptr;
        uint32_t *idx = nullptr, *idx_s = nullptr, *keep = nullptr;
        DevErr *d_err = nullptr;
        ING_CUDA(bufs.get(&d_err, 1));
        ING_CUDA(cudaMemsetAsync(d_err, 0, sizeof(DevErr), s));
        ING_CUDA(bufs.get(&key, m0));
        ING_CUDA(bufs.get(&key_s, m0));
        ING_CUDA(bufs.get(&idx, m0));
        ING_CUDA(bufs.get(&idx_s, m0));
        const int gb = grid_for(m0, sms);
        k_pair_keys<<<gb, 256, 0, s>>>(dx, dy, m0, key, idx, d_err);
        ING_CUDA(cudaGetLastError());
        DevErr he{};
        ING_CUDA(cudaMemcpyAsync(&he, d_err, sizeof(he), cudaMemcpyDeviceToHost, s));
        ING_CUDA(cudaStreamSynchronize(s));
        st = check_err(he, "binary graph");
        if (st != GBS_OK) return st;
        st = sort_pairs<unsigned long long>(key, key_s, idx, idx_s, m0, s, bufs);
        if (st != GBS_OK) return st;
        ING_CUDA(bufs.get(&keep, m0));
        k_first_of_run<<<gb, 256, 0, s>>>(key_s, idx_s, m0, keep);
        ING_CUDA(cudaGetLastError());
        bufs.release(key);
        bufs.release(key_s);
        bufs.release(idx);
        bufs.release(idx_s);
        // keep flags widened to 64-bit counts, one more slot for the total
        unsigned long long *keep64 = nullptr;
        ING_CUDA(bufs.get(&keep64, m0 + 1));
        k_widen<<<gb, 256, 0, s>>>(keep, m0, keep64);
        ING_CUDA(cudaGetLastError());
        ING_CUDA(bufs.get(&at, m0 + 1));
        st = excl_sum(keep64, at, m0 + 1, s, bufs);
        if (st != GBS_OK) return st;
        unsigned long long kept = 0;
        ING_CUDA(cudaMemcpyAsync(&kept, at + m0, sizeof(kept), cudaMemcpyDeviceToHost, s));
        long long *ox = nullptr, *oy = nullptr;
        ING_CUDA(bufs.get(&ox, m0));
        ING_CUDA(bufs.get(&oy, m0));
        k_compact<<<gb, 256, 0, s>>>(dx, dy, keep, at, m0, ox, oy);
        ING_CUDA(cudaGetLastError());
        ING_CUDA(cudaStreamSynchronize(s));
        dx = ox;
        dy = oy;
        m = kept;
        dups = m0 - kept;
    }
    ING_CUDA(cudaEventRecord(ev[1], s));
    const bool send = direction != GBS_DIR_RECV;
    // SEND: row = from - offset, col = to - target_offset; RECV: row = to - offset, col = from - target_offset
    st = build_csr(dx, dy, m, hdr[0], hdr[2], target_offset, !send, false, s, sms, bufs, out);
    if (st != GBS_OK) return st;
    ING_CUDA(cudaEventRecord(ev[2], s));
    ING_CUDA(cudaEventSynchronize(ev[2]));
    if (info) {
        float a = 0.f, b = 0.f;
        ING_CUDA(cudaEventElapsedTime(&a, ev[0], ev[1]));
        ING_CUDA(cudaEventElapsedTime(&b, ev[1], ev[2]));
        info->v_num = hdr[0];
        info->e_num = hdr[1];
        info->offset = hdr[2];
        info->g_v_size = hdr[3];
        info->records = m0;
        info->edges = m;
        info->duplicates = dups;
        info->parse_ms = a;
        info->build_ms = b;
    }
    return GBS_OK;
}

__global__ void k_iota(uint32_t *__restrict__ id, unsigned long long m) {
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < m;
         k += (unsigned long long)gridDim.x * blockDim.x)
        id[k] = (uint32_t)k;
}

// A resident graph from a device CSR: rows sorted by (weight, column) with
// stable radix passes from the least significant key up.
gbs_status graph_from_csr(const gbs_device_csr *c, gbs_weight_type wtype, gbs_graph **out) {
    if (wtype != GBS_WEIGHT_U32 && wtype != GBS_WEIGHT_F32 && wtype != GBS_WEIGHT_F64)
        return fail(GBS_ERR_INVALID_ARG, "unknown weight type");
    const unsigned long long m = c->m;
    const uint32_t n = c->n;
    int dev = 0, sms = 0;
    ING_CUDA(cudaGetDevice(&dev));
    ING_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s;
    ING_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamFree {
        cudaStream_t s;
        ~StreamFree() { cudaStreamDestroy(s); }
    } sf{s};
    Bufs bufs;
    const int gb = grid_for(m, sms);
    uint32_t *row_of = nullptr, *flags = nullptr, *id0 = nullptr, *id1 = nullptr, *col_s = nullptr;
    unsigned long long *wbits = nullptr, *key = nullptr, *key_s = nullptr;
    ING_CUDA(bufs.get(&row_of, m));
    ING_CUDA(bufs.get(&flags, 1));
    ING_CUDA(bufs.get(&wbits, m));
    ING_CUDA(cudaMemsetAsync(flags, 0, sizeof(uint32_t), s));
    k_row_of<<<std::max(1, std::min<int>((n + 7) / 8, sms * 16)), 256, 0, s>>>(c->d_row, n, row_of);
    ING_CUDA(cudaGetLastError());
    if (wtype == GBS_WEIGHT_F64) k_weight_bits<2><<<gb, 256, 0, s>>>(c->d_w, m, wbits, flags);
    else if (wtype == GBS_WEIGHT_F32) k_weight_bits<1><<<gb, 256, 0, s>>>(c->d_w, m, wbits, flags);
    else k_weight_bits<0><<<gb, 256, 0, s>>>(c->d_w, m, wbits, flags);
    ING_CUDA(cudaGetLastError());
    uint32_t hf = 0;
    ING_CUDA(cudaMemcpyAsync(&hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, s));
    ING_CUDA(cudaStreamSynchronize(s));
    if (hf & 1u) return fail(GBS_ERR_INVALID_ARG, "weights must be finite and >= 0");
    if (hf & 2u) return fail(GBS_ERR_INVALID_ARG, "uint32 graphs need integer weights below 2^32");
    // pass 1: by column
    ING_CUDA(bufs.get(&id0, m));
    ING_CUDA(bufs.get(&id1, m));
    ING_CUDA(bufs.get(&col_s, m));
    k_iota<<<gb, 256, 0, s>>>(id0, m);
    ING_CUDA(cudaGetLastError());
    gbs_status st = sort_pairs<uint32_t>(c->d_col, col_s, id0, id1, m, s, bufs);
    if (st != GBS_OK) return st;
    ING_CUDA(bufs.get(&key, m));
    ING_CUDA(bufs.get(&key_s, m));
    if (wtype == GBS_WEIGHT_F64) {
        // pass 2: by weight bits; pass 3: by row
        k_gather_key<unsigned long long><<<gb, 256, 0, s>>>(wbits, id1, m, key);
        ING_CUDA(cudaGetLastError());
        st = sort_pairs<unsigned long long>(key, key_s, id1, id0, m, s, bufs);
        if (st != GBS_OK) return st;
        uint32_t *rk = reinterpret_cast<uint32_t *>(key), *rk_s = reinterpret_cast<uint32_t *>(key_s);
        k_gather_key<uint32_t><<<gb, 256, 0, s>>>(row_of, id0, m, rk);
        ING_CUDA(cudaGetLastError());
        st = sort_pairs<uint32_t>(rk, rk_s, id0, id1, m, s, bufs);
        if (st != GBS_OK) return st;
    } else {
        // pass 2: by (row, weight bits)
        k_key_row_w<<<gb, 256, 0, s>>>(row_of, wbits, id1, m, key);
        ING_CUDA(cudaGetLastError());
        st = sort_pairs<unsigned long long>(key, key_s, id1, id0, m, s, bufs);
        if (st != GBS_OK) return st;
        std::swap(id0, id1);
    }
    // id1: the edge at each sorted position
    double hmax = 0.0, hsum = 0.0;
    double *dred = nullptr;
    ING_CUDA(bufs.get(&dred, 2));
    {
        size_t t1 = 0, t2 = 0;
        ING_CUDA(cub::DeviceReduce::Max(nullptr, t1, c->d_w, dred, (int64_t)m, s));
        ING_CUDA(cub::DeviceReduce::Sum(nullptr, t2, c->d_w, dred + 1, (int64_t)m, s));
        char *t = nullptr;
        ING_CUDA(bufs.get(&t, std::max(t1, t2)));
        if (m) {
            ING_CUDA(cub::DeviceReduce::Max(t, t1, c->d_w, dred, (int64_t)m, s));
            ING_CUDA(cub::DeviceReduce::Sum(t, t2, c->d_w, dred + 1, (int64_t)m, s));
            ING_CUDA(cudaMemcpyAsync(&hmax, dred, sizeof(double), cudaMemcpyDeviceToHost, s));
            ING_CUDA(cudaMemcpyAsync(&hsum, dred + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
        }
    }
    gbs_graph *g = nullptr;
    ING_CUDA(cudaStreamSynchronize(s));
    const double max_w = wtype == GBS_WEIGHT_F32 ? (double)(float)hmax : hmax;
    st = graph_shell(n, m, wtype, max_w, m ? hsum / (double)m : 0.0, (hf & 4u) != 0u, &g);
    if (st != GBS_OK) return st;
    cudaError_t e;
    if ((e = cudaMalloc(&g->d_row, sizeof(uint32_t) * ((size_t)n + 1))) != cudaSuccess ||
        (e = cudaMalloc(&g->d_adj, sizeof(uint2) * (m ? m : 1))) != cudaSuccess ||
        (wtype == GBS_WEIGHT_F64 && (e = cudaMalloc(&g->d_w64, sizeof(unsigned long long) * (m ? m : 1))) != cudaSuccess)) {
        free_graph(g);
        return fail(e == cudaErrorMemoryAllocation ? GBS_ERR_NO_MEMORY : GBS_ERR_CUDA, cudaGetErrorString(e));
    }
    k_row32<<<std::max(1, std::min<int>((n + 256) / 256, sms * 8)), 256, 0, s>>>(c->d_row, n, g->d_row);
    k_adj<<<gb, 256, 0, s>>>(id1, c->d_col, wbits, m, wtype == GBS_WEIGHT_F64, g->d_adj, g->d_w64);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        free_graph(g);
        return fail(GBS_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = g;
    return GBS_OK;
}

}  // namespace gbs

// ===================================================================== C ABI
extern "C" {

gbs_status gbs_parse_text(const char *bytes, size_t len, int direction, gbs_device_csr **out, gbs_ingest_info *info) {
    if (!out || (len && !bytes)) return gbs::fail(GBS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    gbs_device_csr *c = new gbs_device_csr();
    const gbs_status st = gbs::ingest_text(bytes, len, direction, c, info);
    if (st != GBS_OK) {
        gbs_device_csr_destroy(c);
        return st;
    }
    *out = c;
    return GBS_OK;
}

gbs_status gbs_parse_bin(const void *bytes, size_t len, int direction, int64_t target_offset, int dedup,
                         gbs_device_csr **out, gbs_ingest_info *info) {
    if (!out || (len && !bytes)) return gbs::fail(GBS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    gbs_device_csr *c = new gbs_device_csr();
    const gbs_status st = gbs::ingest_bin(static_cast<const char *>(bytes), len, direction, target_offset, dedup, c, info);
    if (st != GBS_OK) {
        gbs_device_csr_destroy(c);
        return st;
    }
    *out = c;
    return GBS_OK;
}

static gbs_status read_whole(const char *path, char **pinned, std::vector<char> &host, size_t &len, double &ms) {
    const auto t0 = std::chrono::steady_clock::now();
    const gbs_status st = gbs::read_file(path, host, pinned, len);
    ms = gbs::ms_since(t0);
    return st;
}

gbs_status gbs_read_text(const char *path, int direction, gbs_device_csr **out, gbs_ingest_info *info) {
    if (!path || !out) return gbs::fail(GBS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    gbs::PinnedFree pf;
    std::vector<char> host;
    size_t len = 0;
    double ms = 0.0;
    gbs_status st = read_whole(path, &pf.p, host, len, ms);
    if (st != GBS_OK) return st;
    st = gbs_parse_text(pf.p ? pf.p : host.data(), len, direction, out, info);
    if (st == GBS_OK && info) info->read_ms = ms;
    return st;
}

gbs_status gbs_read_bin(const char *path, int direction, int64_t target_offset, int dedup, gbs_device_csr **out,
                        gbs_ingest_info *info) {
    if (!path || !out) return gbs::fail(GBS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    gbs::PinnedFree pf;
    std::vector<char> host;
    size_t len = 0;
    double ms = 0.0;
    gbs_status st = read_whole(path, &pf.p, host, len, ms);
    if (st != GBS_OK) return st;
    st = gbs_parse_bin(pf.p ? pf.p : host.data(), len, direction, target_offset, dedup, out, info);
    if (st == GBS_OK && info) info->read_ms = ms;
    return st;
}

gbs_status gbs_device_csr_info(const gbs_device_csr *c, uint32_t *n, uint64_t *m) {
    if (!c) return gbs::fail(GBS_ERR_INVALID_ARG, "csr is NULL");
    if (n) *n = c->n;
    if (m) *m = c->m;
    return GBS_OK;
}

gbs_status gbs_device_csr_export(const gbs_device_csr *c, uint64_t *row_offsets, uint32_t *cols, double *weights) {
    if (!c) return gbs::fail(GBS_ERR_INVALID_ARG, "csr is NULL");
    if (row_offsets)
        GBS_CUDA(cudaMemcpy(row_offsets, c->d_row, sizeof(uint64_t) * ((size_t)c->n + 1), cudaMemcpyDeviceToHost));
    if (cols && c->m) GBS_CUDA(cudaMemcpy(cols, c->d_col, sizeof(uint32_t) * c->m, cudaMemcpyDeviceToHost));
    if (weights && c->m) GBS_CUDA(cudaMemcpy(weights, c->d_w, sizeof(double) * c->m, cudaMemcpyDeviceToHost));
    return GBS_OK;
}

gbs_status gbs_graph_from_device_csr(const gbs_device_csr *c, gbs_weight_type wtype, gbs_graph **out) {
    if (!c || !out) return gbs::fail(GBS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    return gbs::graph_from_csr(c, wtype, out);
}

gbs_status gbs_device_csr_destroy(gbs_device_csr *c) {
    if (!c) return gbs::fail(GBS_ERR_INVALID_ARG, "csr is NULL");
    cudaFree(c->d_row);
    cudaFree(c->d_col);
    cudaFree(c->d_w);
    delete c;
    return GBS_OK;
}

}  // extern "C"
