// GPU-resident eigensolver (thick-restart Lanczos + mixed-precision corrections).
#pragma once

#include <functional>

#include "cigpu_internal.h"

namespace cigpu {

// y = H x on stream s (device pointers).
using Matvec64 = std::function<void(const double *x, double *y, cudaStream_t s)>;
using Matvec32 = std::function<void(const float *x, float *y, cudaStream_t s)>;

struct SolveOptions {
    double tol = 1e-8;          // FP64 residual norm target
    int64_t max_matvec = 0;     // 0: 3 * dim (ARPACK iparam[2] of the reference)
    int basis = 42;             // Krylov basis size (ARPACK ncv of the reference)
    int keep = 14;              // Ritz vectors kept at a thick restart
    int corr_steps = 24;        // FP32 Krylov steps per FP64 correction (mixed)
    int max_corrections = 12;   // FP64 correction cycles (mixed)
    int dav_basis = 30;         // FP32 correction vectors before folding into the anchor (mixed)
    uint64_t seed = 12345;      // random start vector
};

struct SolveProblem {
    int64_t n = 0;
    Matvec64 mv64;              // always present (FP64 matvec)
    Matvec32 mv32;              // mixed only
    const double *diag = nullptr;  // device, [n], H_ii (Davidson-type preconditioner)
    // mixed cold starts: the first anchor from the FP32 product (worth it where that is
    // several times cheaper than the FP64 one: the FCI sigma vector)
    bool fp32_first_anchor = false;
    cudaStream_t stream = nullptr;
};

// Plain FP64 thick-restart Lanczos. c_dev: [n] output (and optional start when
// `have_start`). Returns CIGPU_OK or CIGPU_ENOCONV; fills info (without Econst).
int solve_fp64(const SolveProblem &P, const SolveOptions &o, double *c_dev, bool have_start, cigpu_solve_info &info);
// Mixed: anchored Davidson -- FP32 correction vectors and FP32 CRS matvecs, FP64
// projected problem and diagonal preconditioner, FP64 residual-correction restarts.
int solve_mixed(const SolveProblem &P, const SolveOptions &o, double *c_dev, bool have_start, cigpu_solve_info &info);

// Symmetric eigen-decomposition of a small dense matrix (Householder + implicit QR, small_eigh.h):
// a is n*n row-major (destroyed), w ascending, z columns are eigenvectors (z[i*n+k] = vec_k[i]).
void small_eigh(int n, std::vector<double> &a, std::vector<double> &w, std::vector<double> &z);

// Device vector helpers used by the solver and the RDM code.
void dev_fill_random(double *v, int64_t n, uint64_t seed, cudaStream_t s);
void dev_convert(const double *src, float *dst, int64_t n, cudaStream_t s);
void dev_convert(const float *src, double *dst, int64_t n, cudaStream_t s);

}  // namespace cigpu
