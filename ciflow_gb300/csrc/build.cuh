// Device-side parameter blocks and launchers of the CRS build.
#pragma once

#include "cigpu_internal.h"

namespace cigpu {

enum BuildMode { kCount = 0, kFill64 = 1, kFill32 = 2 };

constexpr int kFciThreads = 256;
constexpr int kFciRowsPerBlock = 64;
constexpr size_t kFciMaxSmem = 112 * 1024;  // two blocks per SM at most this size
constexpr int kDociThreads = 128;

struct FciParams {
    int L;
    int64_t Db;
    SpinDev a, b;
    const double *eri;  // chemist (pq|rs), L^4
    const float *eri_hi, *eri_lo;  // FP32 split of eri, zero where |v| <= 1e-14
    int staged;         // alpha-single integral slices fit in shared memory
    int fly = 0;        // FP64 slot tiles without the alpha-single x beta-single block (formed in the matvec)
    const double *diag; // [dim] row diagonals
    const float *diag_hi, *diag_lo;  // FP32 split of diag (MIXED)
    // single-excitation elements per row: [dim][ns_a + ns_b], alpha singles first
    // (FP64, and the FP32 split zeroed where |v| <= 1e-14 for MIXED)
    const double *sgl64;
    const float *sgl_hi, *sgl_lo;
    // COUNT outputs
    uint32_t *row_count;
    uint32_t *upper_off;
    // FILL inputs / outputs
    const int64_t *row_ptr;
    uint32_t *col;
    double *val64;
    float *val32;
    float *val32lo;  // v - (double)hi, rounded to FP32 (FP32 fill only)
    // slot-tile matvecs: each alpha string's slot descriptors [Da][Wp] and each
    // beta tile's single targets [tiles][ns_b][kTileRows] (slot_tables_launch)
    const uint64_t *desc_tab = nullptr;
    const uint32_t *st_tab = nullptr;
};

struct DociParams {
    int L, n, W;
    int64_t D;
    uint64_t fullmask;
    const uint64_t *strings;
    const double *h;
    const double *eri;
    const double *diag;
    uint32_t *row_count;
    uint32_t *upper_off;
    const int64_t *row_ptr;
    uint32_t *col;
    double *val64;
    float *val32;
    float *val32lo;
};

// C(n, k) exactly while it fits in int64, else INT64_MAX (saturated). Each step
// r <- r (n-k+i) / i is exact (i divides r (n-k+i)); it runs in 64 bits while
// r (n-k+i) fits, and otherwise as (r/g) ((n-k+i)/(i/g)) with g = gcd(r, i), whose
// factors are at most the result, so nothing overflows for any n (Hamiltonians go
// up to 128 orbitals).
__host__ __device__ inline int64_t d_binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    uint64_t r = 1;
    for (int i = 1; i <= k; ++i) {
        const uint64_t m = (uint64_t)(n - k + i);
        if (r <= UINT64_MAX / m) {
            r = r * m / (uint64_t)i;
        } else {
            uint64_t g = r, b = (uint64_t)i;
            while (b) {
                const uint64_t t = g % b;
                g = b;
                b = t;
            }
            const uint64_t a = r / g, f = m / ((uint64_t)i / g);
            if (a > UINT64_MAX / f) return INT64_MAX;
            r = a * f;
        }
        if (r > (uint64_t)INT64_MAX) return INT64_MAX;
    }
    return (int64_t)r;
}

// Determinants of an FCI space (alpha x beta strings) or a DOCI space (pair
// strings); -1 for impossible electron counts or a count beyond int64.
__host__ __device__ inline int64_t space_dim(int method, int L, int nup, int ndown) {
    if (L < 0 || nup < 0 || ndown < 0 || nup > L || ndown > L) return -1;
    const int64_t a = d_binom(L, nup);
    if (a == INT64_MAX) return -1;
    if (method == 1 /* CIGPU_DOCI */) return a;
    const int64_t b = d_binom(L, ndown);
    if (b == INT64_MAX || (b != 0 && a > INT64_MAX / b)) return -1;
    return a * b;
}

// Position of the a-th (0-based) set bit of x.
__device__ __forceinline__ int nth_set(uint64_t x, int a) {
    for (int i = 0; i < a; ++i) x &= x - 1;
    return __ffsll((long long)x) - 1;
}

size_t fci_smem_bytes(const FciParams &p);
// structural slots per FCI row: nfull_b + ns_a * nsing_b + nd_a
__host__ __device__ inline int fci_row_width(const FciParams &p) { return p.b.nfull + p.a.ns * p.b.nsing + p.a.nd; }
void fci_launch(int mode, const FciParams &p, cudaStream_t s);
void fci_diag_launch(const FciParams &p, double *diag, cudaStream_t s);
// Row singles table (and FP32 splits of it and of diag when hi/lo are non-null).
void fci_singles_launch(const FciParams &p, double *sgl64, float *sgl_hi, float *sgl_lo, float *diag_hi,
                        float *diag_lo, cudaStream_t s);
size_t doci_smem_bytes(int W, int warps);
void doci_strings_launch(int L, int n, int64_t D, uint64_t *strings, cudaStream_t s);
void doci_diag_launch(const DociParams &p, double *diag, cudaStream_t s);
void doci_launch(int mode, const DociParams &p, cudaStream_t s);
void upper_counts_launch(int64_t dim, const int64_t *row_ptr, const uint32_t *upper_off, uint32_t *ucnt,
                         cudaStream_t s);
void extract_upper_launch(int64_t dim, const int64_t *row_ptr, const uint32_t *upper_off, const uint32_t *col,
                          const double *val64, const float *val32, const int64_t *urow, uint32_t *ucol, double *uval,
                          cudaStream_t s);
// out[0] = 0, out[i+1] = in[0] + ... + in[i]; out has n+1 entries.
void exclusive_scan_u32(const uint32_t *in, int64_t *out, int64_t n, cudaStream_t s);
// The same without waiting: the caller keeps `sums` (the tile sums) alive until s has run it.
void exclusive_scan_u32_async(const uint32_t *in, int64_t *out, int64_t n, DevBuf<int64_t> &sums, cudaStream_t s);
int sm_count();

}  // namespace cigpu
