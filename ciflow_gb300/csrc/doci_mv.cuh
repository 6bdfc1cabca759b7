// Matrix-free DOCI matvec (doci_mv.cu).
#pragma once

#include "build.cuh"
#include "checked.cuh"

namespace cigpu {

struct DociMv {
    int L, n;                  // orbitals, electron pairs (n <= 32)
    int64_t D;                 // pair strings (rows)
    const uint64_t *strings;   // [D], colex order
    unsigned long long *err = nullptr;  // checked build: the error word
};

// K_jk = (jk|jk) for j != k, zero where |v| <= 1e-14 (and on the diagonal): the
// pair-hop values, FP64 and FP32 (L*L each, device).
void doci_pair_table_launch(int L, const double *eri, double *K64, float *K32, cudaStream_t s);
// Entries of v with |v| > 1e-14 (synchronises s).
int64_t count_nonzero(const double *v, int64_t n, cudaStream_t s);
// y = H x: FP64 (K64, FP64 diag/x/y) and FP32 (K32, FP32 diag/x/y, FP32 accumulation).
void doci_mv64(const DociMv &p, const double *K, const double *diag, const double *x, double *y, cudaStream_t s);
void doci_mv32(const DociMv &p, const float *K, const float *diag, const float *x, float *y, cudaStream_t s);

}  // namespace cigpu
