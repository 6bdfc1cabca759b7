// FP32 product of the mixed method for FCI from a factorised two-electron part
// (sigma.cu): a direct-CI sigma vector in place of the stored-matrix product.
#pragma once

#include "build.cuh"

namespace cigpu {

constexpr int kSigmaChunk = 16;      // factors per pass (the rank is padded to a multiple)
constexpr int kSigmaMaxRank = 128;   // padded rank limit
constexpr int kSigmaMaxL = 24;       // orbitals limit (the factorisation is an L^2 x L^2 eigenproblem on the host)

struct SigmaOp {
    int L = 0;
    int rank = 0;  // eigenpairs kept
    int R = 0;     // rank padded to a multiple of kSigmaChunk; 0: the operator is not in use
    int64_t Da = 0, Db = 0;
    DevBuf<float> F, G, K1;              // [L*L][R] factors, [L*L][R] scaled factors, [L*L] one-body matrix
    DevBuf<float> fa, fb, ga, gb;        // per-string diagonal sums, factor-major: [R][Da], [R][Db]
    DevBuf<float> ka, kb;                // per-string one-body diagonal sums: [Da], [Db]
    DevBuf<float> xT, Ya, Yb, kx;        // work: x transposed, A_k x in two layouts, the one-body product
    size_t smem_a = 0, smem_b = 0;       // dynamic shared memory of the two kernels
};

// Whether a space of L orbitals can use the operator (before the rank is known).
inline bool sigma_applies(int L) { return L >= 1 && L <= kSigmaMaxL; }

// Factorises (pq|rs) = sum_k s_k F^k_pq F^k_rs (a pivoted Cholesky factor of the
// pair matrix to 1e-10 of its largest diagonal; eigenpairs when it is indefinite),
// forms the one-body matrix and the per-string tables, and allocates the work
// buffers. False (op.R = 0) when the space does not qualify (too many orbitals,
// or fewer 32 x 32 string tiles than SMs unless any_grid) or the rank exceeds
// kSigmaMaxRank.
bool sigma_prepare(SigmaOp &op, int L, const double *h, const double *eri, const SpinTables &ta,
                   const SpinTables &tb, bool any_grid, cudaStream_t s);

// Device bytes of the operator's tables and work buffers at the padded rank R.
size_t sigma_bytes(int L, int64_t Da, int64_t Db, int R);

// y = H x in FP32 (x, y: [Da][Db] device vectors), H = K + 1/2 sum_k s_k A_k^2.
void sigma_mv32(SigmaOp &op, const FciParams &p, const float *x, float *y, cudaStream_t s);

}  // namespace cigpu
