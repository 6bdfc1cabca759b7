// Internal declarations of the cigpu library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/cigpu.h"

namespace cigpu {

// SparseMatrix_CRS::_zero (SparseMatrix_CRS.cpp:44): |v| <= 1e-14 is not stored.
constexpr double kZero = 1e-14;
constexpr int kMaxL = 63;       // FCI / DOCI spaces (64-bit strings)
constexpr int kMaxLDets = 128;  // Hamiltonians and determinant lists (two 64-bit words per string)

enum Kind : uint32_t { kSelf = 0, kSingle = 1, kDouble = 2 };

extern std::atomic<int64_t> g_launches;
inline void count_launch(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

struct CudaError {
    cudaError_t err;
    const char *what;
};

#define CIGPU_CUDA(call)                                                        \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) throw ::cigpu::CudaError{e_, #call};            \
    } while (0)

void *dev_alloc(size_t bytes);          // throws std::bad_alloc on failure
void dev_free(void *p, size_t bytes);   // returns the block to the cache
// Bytes currently held by live DevBufs (not counting the cache).
size_t dev_bytes_in_use();

// The stream the calling thread's library work is ordered on. Entry points set it
// for their duration; a block released while it is set is handed to another
// stream only after an event recorded on it has completed (stream-ordered reuse).
// A block released with no stream set waits for the whole device first, as
// cudaFree would.
struct StreamScope {
    cudaStream_t prev;
    bool prev_set;
    // set = false: no stream (e.g. synchronous legacy-stream copies follow)
    explicit StreamScope(cudaStream_t s, bool set = true);
    ~StreamScope();
};

// Device buffer with RAII; allocation failure throws std::bad_alloc. Blocks come
// from a caching allocator: cudaFree synchronises the whole device, which would
// serialise concurrent solves on different streams.
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count);
    void release() {
        if (p) dev_free(p, n * sizeof(T));
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

// Phase timer: with CIGPU_TRACE=1 in the environment, mark() synchronises the
// stream and prints the time since the previous mark to stderr.
struct Trace {
    const char *scope;
    cudaStream_t s;
    bool on;
    double t0;
    Trace(const char *sc, cudaStream_t st);
    ~Trace();
    Trace(const Trace &) = delete;
    Trace &operator=(const Trace &) = delete;
    void mark(const char *what);
};

template <typename T>
void DevBuf<T>::alloc(size_t count) {
    release();
    if (count == 0) return;
    p = static_cast<T *>(dev_alloc(count * sizeof(T)));
    n = count;
}

// ---------------------------------------------------------------------------
// Per-spin string tables for FCI (host side, uploaded once per CRS).
// Strings are ranked in colex order, the order of Permutator_Bit
// (Permutator.cpp:113-153) and of determine_weight (CIMethod.cpp:689-747).
// FP32 split (hi = fl32(v), lo = fl32(v - hi)); both zero when |v| <= 1e-14.
__host__ __device__ inline void split_fp32(double v, float &hi, float &lo) {
    if (!(v > kZero || v < -kZero)) {
        hi = lo = 0.0f;
        return;
    }
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

struct SpinTables {
    int L = 0, n = 0;
    int64_t D = 0;
    int ns = 0;      // single excitations per string: n (L - n)
    int nd = 0;      // same-spin doubles per string: C(n,2) C(L-n,2)
    int nfull = 0;   // 1 + ns + nd
    int nsing = 0;   // 1 + ns
    std::vector<uint64_t> strings;   // [D]
    std::vector<uint8_t> occ;        // [D][n] occupied orbitals, ascending
    std::vector<double> diag;        // [D] get_diag_cont_one_bitstring (CIMethod.cpp:329-342)
    std::vector<uint32_t> s_target;  // [D][ns]
    std::vector<double> s_part;      // [D][ns] T(lo,hi) + sum_common (V - V), reference order
    std::vector<uint32_t> s_info;    // [D][ns] lo | hi<<6 | row<<12 | col<<18 | odd<<24
    std::vector<uint32_t> d_target;  // [D][nd]
    std::vector<double> d_val;       // [D][nd] signed element (min-rank perspective)
    std::vector<float> d_hi, d_lo;   // [D][nd] FP32 split of d_val, zero where |v| <= 1e-14
    std::vector<uint64_t> nb_full;   // [D][nfull] sorted by target: target | kind<<32 | idx<<34
    std::vector<uint64_t> nb_sing;   // [D][nsing] sorted {self} + singles
};

// Builds the tables; eri is chemist (pq|rs) L^4, h L*L.
void build_spin_tables(int L, int n, const double *h, const double *eri, SpinTables &t);

struct SpinDev {
    int64_t D;
    int n, ns, nd, nfull, nsing;
    const uint8_t *occ;
    const double *diag;
    const uint32_t *s_target;
    const double *s_part;
    const uint32_t *s_info;
    const uint32_t *d_target;
    const double *d_val;
    const float *d_hi, *d_lo;
    const uint64_t *nb_full;
    const uint64_t *nb_sing;
};

struct SpinDevStore {
    DevBuf<uint8_t> occ;
    DevBuf<double> diag, s_part, d_val;
    DevBuf<float> d_hi, d_lo;
    DevBuf<uint32_t> s_target, s_info, d_target;
    DevBuf<uint64_t> nb_full, nb_sing;
    SpinDev view{};
    void upload(const SpinTables &t, cudaStream_t s);
};

}  // namespace cigpu

// Opaque handle definitions.
struct cigpu_ham {
    int L, nup, ndown;
    double econst;
    std::vector<double> h;    // host copy, L*L
    std::vector<double> eri;  // host copy, L^4 chemist
    // false: h/eri are not filled (a Hamiltonian made on the device for a DOCI
    // build, which reads the device tables only); the device tables are current
    bool host_valid = true;
    cigpu::DevBuf<double> d_h;
    cigpu::DevBuf<double> d_eri;
    cigpu::DevBuf<float> d_eri_hi, d_eri_lo;  // FP32 split, zero where |v| <= 1e-14
};
