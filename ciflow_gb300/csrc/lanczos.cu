// GPU-resident lowest-eigenpair solver.
//
// Replaces CIMethod::solve -> SparseMatrix_CRS::arpackDiagonalize
// (CIMethod.cpp:241-264, SparseMatrix_CRS.cpp:360-481), where ARPACK's
// implicitly restarted Lanczos (which='SA', ncv=42, tol=0) calls the serial
// matvec through reverse communication. Here the Krylov basis lives in HBM and
// every vector operation is a device kernel; the host only holds the small
// projected matrix (<= 43 x 43) and diagonalises it.
//
// Plain (FP64): thick-restart Lanczos (Wu & Simon) with full classical
// Gram-Schmidt re-orthogonalisation done twice per step; FP64 vectors and matvec.
//
// Mixed: the same Lanczos with FP32 vectors and the FP32 CRS (FP32 row
// accumulation), FP64 dot products / recurrence / projected eigensolve. The
// FP32 Ritz vector is then refined in FP64: w = H c with an FP64 matvec,
// E = c.w (Rayleigh quotient), r = w - E c; while ||r|| > tol a correction cycle
// runs an FP32 Krylov space from the diagonally preconditioned residual
// t = r / (E - H_ii) and does the Rayleigh-Ritz step over [c, K(t)] in FP64
// (the coupling column uses the FP64 product H c). The FP32 error only enters
// the small correction, so each cycle gains several digits.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <mutex>

#include "lanczos.cuh"
#include "small_eigh.h"
#include <type_traits>

namespace cigpu {

int sm_count();

namespace {

// Host-side time accounting of a solve (printed with CIGPU_TRACE=1).
struct SolveClock {
    double eigh = 0, wait = 0;
    int64_t n_eigh = 0, n_wait = 0;
};
thread_local SolveClock g_clk;
inline double wall() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

constexpr int kVecThreads = 256;
constexpr int kMaxBasis = 64;
constexpr int kDotChunk = 8;
constexpr int kMaxKeep = 32;
constexpr int kStartSteps = 4;  // FP32 Lanczos steps of the mixed solver's Krylov start

int vec_grid() { return sm_count() * 4; }
// blocks for an n-element basis kernel (dots, updates, combinations): one element
// per thread up to 8 resident blocks per SM. These kernels read many basis vectors
// per element, so a thread's loads, not the bytes, set their time on small vectors
// (tens of thousands of elements): spreading them over every SM instead of a few
// elements per thread on a quarter of the SMs cut a 30-vector update from ~19 us to
// a few us at n = 63,504.
int vec_grid_for(int64_t n) {
    const int64_t b = (n + kVecThreads - 1) / kVecThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sm_count() * 8, b));
}
// blocks per chunk of the dot kernels: about four elements per thread (the grid has
// one row of blocks per chunk of eight vectors, and fewer partials shorten the
// reduction that ends the kernel)
int dot_grid_for(int64_t n) {
    const int64_t b = (n + kVecThreads * 4 - 1) / (kVecThreads * 4);
    return (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sm_count() * 4, b));
}

// Ends a kernel that wrote per-block partial sums partial[v*G + b] (G = gridDim.x):
// the last block to finish reduces them into out[v], v < nvec, one warp per entry in
// a fixed order (run-to-run reproducible), and resets the ticket for the next kernel
// on the stream. Saves a separate reduction launch per dot product.
__device__ __forceinline__ bool reduce_in_last_block(const double *partial, int nvec, double *out,
                                                     unsigned *ticket) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x * gridDim.y - 1;
    __syncthreads();
    if (!last) return false;
    __threadfence();
    const int G = gridDim.x, lane = threadIdx.x & 31;
    for (int v = threadIdx.x >> 5; v < nvec; v += blockDim.x >> 5) {
        double s = 0;
        for (int b = lane; b < G; b += 32) s += __ldcg(partial + (int64_t)v * G + b);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[v] = s;
    }
    if (threadIdx.x == 0) *ticket = 0;
    return true;
}

// The last of the gridDim.x blocks of one chunk (blockIdx.y) reduces the chunk's nv
// rows of block partials partial[i * G + b] into out[i], warp i for row i (a fixed
// order: lanes over b, four running sums, then the warp tree), and resets the
// chunk's ticket. A ticket per chunk keeps the atomics spread and puts each chunk's
// reduction on its own block instead of one block reducing every vector.
__device__ __forceinline__ void reduce_chunk_in_last_block(const double *partial, int nv, double *out,
                                                           unsigned *ticket) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int G = gridDim.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp < nv) {
        const double *p = partial + (int64_t)warp * G;
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        int b = lane;
        for (; b + 96 < G; b += 128) {
            s0 += __ldcg(p + b);
            s1 += __ldcg(p + b + 32);
            s2 += __ldcg(p + b + 64);
            s3 += __ldcg(p + b + 96);
        }
        for (; b < G; b += 32) s0 += __ldcg(p + b);
        double s = (s0 + s1) + (s2 + s3);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[warp] = s;
    }
    if (threadIdx.x == 0) *ticket = 0;
}

// Per-block partial dots V_i . w (i < nvec, chunks of kDotChunk on blockIdx.y, one
// ticket per chunk). AT is the arithmetic type of the products and of the
// per-thread sums (float for FP32 vectors: GB300 issues FP64 at 1/64 of the FP32
// rate); block partials are reduced in FP64. Each thread walks its elements two at
// a time, so 18 loads are in flight per step of the loop.
template <typename VT, typename WT, typename AT = double>
__global__ void __launch_bounds__(kVecThreads) k_multidot(const VT *__restrict__ V, int64_t ld, int nvec,
                                                          const WT *__restrict__ w, int64_t n,
                                                          double *__restrict__ partial, double *__restrict__ out,
                                                          unsigned *__restrict__ tickets, const double *__restrict__ skip) {
    if (skip && *skip != 0.0) return;  // a second orthogonalisation pass that the first made unnecessary
    static_assert(kDotChunk <= kVecThreads / 32, "one warp per vector of a chunk");
    const int G = gridDim.x;
    const int v0 = blockIdx.y * kDotChunk;
    const int nv = min(kDotChunk, nvec - v0);
    AT acc[kDotChunk];
#pragma unroll
    for (int i = 0; i < kDotChunk; ++i) acc[i] = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; r + stride < n; r += 2 * stride) {
        const AT wa = (AT)w[r], wb = (AT)w[r + stride];
        AT va[kDotChunk], vb[kDotChunk];
#pragma unroll
        for (int i = 0; i < kDotChunk; ++i)
            if (i < nv) {
                va[i] = (AT)V[(int64_t)(v0 + i) * ld + r];
                vb[i] = (AT)V[(int64_t)(v0 + i) * ld + r + stride];
            }
#pragma unroll
        for (int i = 0; i < kDotChunk; ++i)
            if (i < nv) acc[i] += va[i] * wa + vb[i] * wb;
    }
    if (r < n) {
        const AT wr = (AT)w[r];
#pragma unroll
        for (int i = 0; i < kDotChunk; ++i)
            if (i < nv) acc[i] += (AT)V[(int64_t)(v0 + i) * ld + r] * wr;
    }
    __shared__ double sh[kDotChunk][kVecThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < kDotChunk; ++i) {
        // warp tree in the accumulation type (FP64 adds here would run on GB300's
        // slow FP64 pipe, 5 per thread and vector); block and grid sums are FP64
        AT a = acc[i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) sh[i][warp] = (double)a;
    }
    __syncthreads();
    if (threadIdx.x < nv) {
        double s = 0;
        for (int k = 0; k < kVecThreads / 32; ++k) s += sh[threadIdx.x][k];
        partial[(int64_t)(v0 + threadIdx.x) * G + blockIdx.x] = s;
    }
    reduce_chunk_in_last_block(partial + (int64_t)v0 * G, nv, out + v0, tickets + blockIdx.y);
}

// The FP32 dots of k_multidot<float, float, float> with 16-byte loads: V rows and w
// as float4 (a length divisible by 4, rows 16-byte aligned), four elements per
// thread and step (at most 64 registers: the grid is four blocks per SM).
__global__ void __launch_bounds__(kVecThreads, 4) k_multidot_f4(const float4 *__restrict__ V, int64_t ld4, int nvec,
                                                             const float4 *__restrict__ w, int64_t n4,
                                                             double *__restrict__ partial, double *__restrict__ out,
                                                             unsigned *__restrict__ tickets,
                                                             const double *__restrict__ skip) {
    if (skip && *skip != 0.0) return;  // a second orthogonalisation pass that the first made unnecessary
    const int G = gridDim.x;
    const int v0 = blockIdx.y * kDotChunk;
    const int nv = min(kDotChunk, nvec - v0);
    float acc[kDotChunk];
#pragma unroll
    for (int i = 0; i < kDotChunk; ++i) acc[i] = 0.f;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n4; r += (int64_t)gridDim.x * blockDim.x) {
        const float4 wr = w[r];
        float4 va[kDotChunk];
#pragma unroll
        for (int i = 0; i < kDotChunk; ++i)
            if (i < nv) va[i] = V[(int64_t)(v0 + i) * ld4 + r];
#pragma unroll
        for (int i = 0; i < kDotChunk; ++i)
            if (i < nv) acc[i] += (va[i].x * wr.x + va[i].y * wr.y) + (va[i].z * wr.z + va[i].w * wr.w);
    }
    __shared__ double sh[kDotChunk][kVecThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < kDotChunk; ++i) {
        float a = acc[i];  // warp tree in FP32, block and grid sums in FP64
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) sh[i][warp] = (double)a;
    }
    __syncthreads();
    if (threadIdx.x < nv) {
        double t = 0;
        for (int k = 0; k < kVecThreads / 32; ++k) t += sh[threadIdx.x][k];
        partial[(int64_t)(v0 + threadIdx.x) * G + blockIdx.x] = t;
    }
    reduce_chunk_in_last_block(partial + (int64_t)v0 * G, nv, out + v0, tickets + blockIdx.y);
}

// k_update<float, float, float> with 16-byte loads (the same per-element order of
// subtractions; see k_multidot_f4 for the shapes).
__global__ void __launch_bounds__(kVecThreads) k_update_f4(const float4 *__restrict__ V, int64_t ld4, int nvec,
                                                           const double *__restrict__ coef, float4 *__restrict__ w,
                                                           int64_t n4, double *__restrict__ nrm,
                                                           double *__restrict__ nrm_out, unsigned *__restrict__ ticket,
                                                           const double *__restrict__ skip,
                                                           const double *__restrict__ gate_ref,
                                                           double *__restrict__ gate_out) {
    if (skip && *skip != 0.0) return;
    __shared__ float c[kMaxBasis + 1];
    for (int i = threadIdx.x; i < nvec; i += blockDim.x) c[i] = (float)coef[i];
    __syncthreads();
    float acc = 0.f;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n4; r += (int64_t)gridDim.x * blockDim.x) {
        float4 x = w[r];
        int i = 0;
        for (; i + 4 <= nvec; i += 4) {  // four vectors' loads in flight, products subtracted in order
            float4 v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = V[(int64_t)(i + q) * ld4 + r];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float cq = c[i + q];
                x.x -= v[q].x * cq;
                x.y -= v[q].y * cq;
                x.z -= v[q].z * cq;
                x.w -= v[q].w * cq;
            }
        }
        for (; i < nvec; ++i) {
            const float4 v = V[(int64_t)i * ld4 + r];
            const float ci = c[i];
            x.x -= v.x * ci;
            x.y -= v.y * ci;
            x.z -= v.z * ci;
            x.w -= v.w * ci;
        }
        w[r] = x;
        acc += (x.x * x.x + x.y * x.y) + (x.z * x.z + x.w * x.w);
    }
    if (nrm) {
        __shared__ double sh[kVecThreads / 32];
        float a = acc;
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)a;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int k = 0; k < kVecThreads / 32; ++k) t += sh[k];
            nrm[blockIdx.x] = t;
        }
        if (reduce_in_last_block(nrm, 1, nrm_out, ticket) && gate_out && threadIdx.x == 0)
            *gate_out = (*nrm_out >= 0.5 * *gate_ref) ? 1.0 : 0.0;
    }
}

// w -= sum_{i<nvec} V_i coef_i (arithmetic in AT); partial ||w||^2 per block when nrm != nullptr.
template <typename VT, typename WT, typename AT = double>
__global__ void __launch_bounds__(kVecThreads) k_update(const VT *__restrict__ V, int64_t ld, int nvec,
                                                        const double *__restrict__ coef, WT *__restrict__ w, int64_t n,
                                                        double *__restrict__ nrm, double *__restrict__ nrm_out,
                                                        unsigned *__restrict__ ticket, const double *__restrict__ skip,
                                                        const double *__restrict__ gate_ref, double *__restrict__ gate_out) {
    if (skip && *skip != 0.0) return;  // see k_multidot
    __shared__ AT c[kMaxBasis + 1];
    for (int i = threadIdx.x; i < nvec; i += blockDim.x) c[i] = (AT)coef[i];
    __syncthreads();
    AT acc = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        AT x = (AT)w[r];
        int i = 0;
        for (; i + 8 <= nvec; i += 8) {  // eight loads in flight, products subtracted in order
            AT v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = (AT)V[(int64_t)(i + q) * ld + r];
#pragma unroll
            for (int q = 0; q < 8; ++q) x -= v[q] * c[i + q];
        }
        for (; i < nvec; ++i) x -= (AT)V[(int64_t)i * ld + r] * c[i];
        const WT xv = (WT)x;
        w[r] = xv;
        acc += (AT)xv * (AT)xv;
    }
    if (nrm) {
        __shared__ double sh[kVecThreads / 32];
        AT a = acc;  // warp tree in the accumulation type, block sum in FP64
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)a;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0;
            for (int k = 0; k < kVecThreads / 32; ++k) s += sh[k];
            nrm[blockIdx.x] = s;
        }
        // with a gate: 1 when the projection kept at least half of ||w||^2 (the
        // DGKS test with eta = 1/sqrt 2), so that a second pass is not needed
        if (reduce_in_last_block(nrm, 1, nrm_out, ticket) && gate_out && threadIdx.x == 0)
            *gate_out = (*nrm_out >= 0.5 * *gate_ref) ? 1.0 : 0.0;
    }
}

// out = (OT)(t / sqrt(nrm2))
template <typename IT, typename OT>
__global__ void k_scale_to(const IT *__restrict__ t, int64_t n, const double *__restrict__ nrm2, OT *__restrict__ out) {
    const double inv = 1.0 / sqrt(*nrm2);
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        out[r] = (OT)((double)t[r] * inv);
}

// FP32 Davidson residual of u = a0 c + sum_i y_i v_i, written straight into the
// next basis slot as the preconditioned direction:
//   ru = a0 r + a0 (E - theta) c + sum_i y_i (HV_i - theta V_i)   (FP32 arithmetic;
//        r = H c - E c is the exact FP64 anchor residual)
//   t  = ru / (sigma - H_ii), sigma = min(theta, min_i H_ii)       (guarded)
// and the partial ||ru||^2 (FP64 block sums). The shift is held at or below the
// lowest diagonal element (*dmin) so that sigma - H_ii keeps one sign: with a start
// far above the ground state (a warm start after a large orbital rotation, theta
// 14 Eh high on a DOCI L=16 problem) theta - H_ii passes through zero on the
// determinants whose diagonal lies near theta, the directions pile onto them, and
// Davidson crawled (117 matvecs, residual 0.3); held, the same start converged in
// 15. Near convergence theta lies below every H_ii and the shift is theta.
__global__ void __launch_bounds__(kVecThreads) k_dav_residual32(const float *__restrict__ r32,
                                                                const float *__restrict__ c32,
                                                                const float *__restrict__ V, const float *__restrict__ HV,
                                                                int64_t ld, int k, const double *__restrict__ y,
                                                                double a0, double a0_de, double theta,
                                                                const double *__restrict__ dmin,
                                                                const float *__restrict__ diag32, float *__restrict__ t,
                                                                int64_t n, double *__restrict__ nrm,
                                                                double *__restrict__ nrm_out, unsigned *__restrict__ ticket) {
    __shared__ float ys[kMaxBasis + 1];
    for (int i = threadIdx.x; i < k; i += blockDim.x) ys[i] = (float)y[i];
    __syncthreads();
    const float fa0 = (float)a0, fa0de = (float)a0_de, fth = (float)theta, fsig = (float)fmin(theta, *dmin);
    float acc = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        float ru = fa0 * r32[r] + fa0de * c32[r];
        int i = 0;
        for (; i + 4 <= k; i += 4) {  // eight loads in flight, terms added in order
            float hv[4], vv[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t o = (int64_t)(i + q + 1) * ld + r;  // corrections live in slots 1..k
                hv[q] = HV[o];
                vv[q] = V[o];
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) ru += ys[i + q] * (hv[q] - fth * vv[q]);
        }
        for (; i < k; ++i) {
            const int64_t o = (int64_t)(i + 1) * ld + r;
            ru += ys[i] * (HV[o] - fth * V[o]);
        }
        acc += ru * ru;
        float d = fsig - diag32[r];  // FP32 (no per-element FP64 or conversion work)
        if (fabsf(d) < 1e-2f) d = d < 0 ? -1e-2f : 1e-2f;
        t[r] = ru / d;
    }
    __shared__ double sh[kVecThreads / 32];
    float a = acc;  // warp tree in FP32, block sum in FP64
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0;
        for (int q = 0; q < kVecThreads / 32; ++q) sum += sh[q];
        nrm[blockIdx.x] = sum;
    }
    reduce_in_last_block(nrm, 1, nrm_out, ticket);
}

// k_dav_residual32 with 16-byte loads: every vector as float4 (a length divisible by
// 4, 16-byte aligned rows); the same per-element order of terms.
__device__ __forceinline__ float dav_precond(float ru, float fsig, float dg) {
    float d = fsig - dg;
    if (fabsf(d) < 1e-2f) d = d < 0 ? -1e-2f : 1e-2f;
    return ru / d;
}

__global__ void __launch_bounds__(kVecThreads) k_dav_residual32_f4(const float4 *__restrict__ r32,
                                                                   const float4 *__restrict__ c32,
                                                                   const float4 *__restrict__ V,
                                                                   const float4 *__restrict__ HV, int64_t ld4, int k,
                                                                   const double *__restrict__ y, double a0,
                                                                   double a0_de, double theta,
                                                                   const double *__restrict__ dmin,
                                                                   const float4 *__restrict__ diag32,
                                                                   float4 *__restrict__ t, int64_t n4,
                                                                   double *__restrict__ nrm,
                                                                   double *__restrict__ nrm_out,
                                                                   unsigned *__restrict__ ticket) {
    __shared__ float ys[kMaxBasis + 1];
    for (int i = threadIdx.x; i < k; i += blockDim.x) ys[i] = (float)y[i];
    __syncthreads();
    const float fa0 = (float)a0, fa0de = (float)a0_de, fth = (float)theta, fsig = (float)fmin(theta, *dmin);
    float acc = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n4; r += (int64_t)gridDim.x * blockDim.x) {
        const float4 rr = r32[r], cc = c32[r];
        float4 ru = make_float4(fa0 * rr.x + fa0de * cc.x, fa0 * rr.y + fa0de * cc.y, fa0 * rr.z + fa0de * cc.z,
                                fa0 * rr.w + fa0de * cc.w);
        int i = 0;
        for (; i + 2 <= k; i += 2) {  // four 16-byte loads in flight, terms added in order
            float4 hv[2], vv[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int64_t o = (int64_t)(i + q + 1) * ld4 + r;  // corrections live in slots 1..k
                hv[q] = HV[o];
                vv[q] = V[o];
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float yq = ys[i + q];
                ru.x += yq * (hv[q].x - fth * vv[q].x);
                ru.y += yq * (hv[q].y - fth * vv[q].y);
                ru.z += yq * (hv[q].z - fth * vv[q].z);
                ru.w += yq * (hv[q].w - fth * vv[q].w);
            }
        }
        for (; i < k; ++i) {
            const int64_t o = (int64_t)(i + 1) * ld4 + r;
            const float4 hv = HV[o], vv = V[o];
            ru.x += ys[i] * (hv.x - fth * vv.x);
            ru.y += ys[i] * (hv.y - fth * vv.y);
            ru.z += ys[i] * (hv.z - fth * vv.z);
            ru.w += ys[i] * (hv.w - fth * vv.w);
        }
        acc += (ru.x * ru.x + ru.y * ru.y) + (ru.z * ru.z + ru.w * ru.w);
        const float4 dg = diag32[r];
        t[r] = make_float4(dav_precond(ru.x, fsig, dg.x), dav_precond(ru.y, fsig, dg.y),
                           dav_precond(ru.z, fsig, dg.z), dav_precond(ru.w, fsig, dg.w));
    }
    __shared__ double sh[kVecThreads / 32];
    float a = acc;  // warp tree in FP32, block sum in FP64
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0;
        for (int q = 0; q < kVecThreads / 32; ++q) sum += sh[q];
        nrm[blockIdx.x] = sum;
    }
    reduce_in_last_block(nrm, 1, nrm_out, ticket);
}

// t = r / (sigma - H_ii) in FP32 (first direction after an anchor update), sigma =
// min(E, min_i H_ii) (*dmin): see the shift of k_dav_residual32.
__global__ void k_precond32(const double *__restrict__ r, const double *__restrict__ diag, double E,
                            const double *__restrict__ dmin, float *__restrict__ t, int64_t n) {
    const double sig = fmin(E, *dmin);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float d = (float)(sig - diag[i]);
        if (fabsf(d) < 1e-2f) d = d < 0 ? -1e-2f : 1e-2f;
        t[i] = (float)r[i] / d;
    }
}

// Block-wise (min value, index) of diag, then a single-block reduction.
__global__ void k_argmin_partial(const double *__restrict__ d, int64_t n, double *__restrict__ pv,
                                 int64_t *__restrict__ pi) {
    double best = 1e308;
    int64_t bi = 0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        if (d[r] < best || (d[r] == best && r < bi)) {
            best = d[r];
            bi = r;
        }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob < best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    __shared__ double sv[kVecThreads / 32];
    __shared__ int64_t si[kVecThreads / 32];
    if ((threadIdx.x & 31) == 0) {
        sv[threadIdx.x >> 5] = best;
        si[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < kVecThreads / 32; ++q)
            if (sv[q] < best || (sv[q] == best && si[q] < bi)) {
                best = sv[q];
                bi = si[q];
            }
        pv[blockIdx.x] = best;
        pi[blockIdx.x] = bi;
    }
}

// One warp: the (value, index) minimum over the G block partials, ties to the lower
// index; the index goes to pi[0] and the value to pv[0] (after every read of pv).
__global__ void k_argmin_final(double *__restrict__ pv, int64_t *__restrict__ pi, int G) {
    double best = 1e308;
    int64_t bi = INT64_MAX;
    for (int b = threadIdx.x; b < G; b += 32)
        if (pv[b] < best || (pv[b] == best && pi[b] < bi)) {
            best = pv[b];
            bi = pi[b];
        }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob < best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    if (threadIdx.x == 0) {
        pi[0] = bi;
        pv[0] = best;
    }
}

// v = e_at + keep * v with at = *pi (v holds a random vector on entry).
__global__ void k_add_unit_at(const int64_t *__restrict__ pi, double keep, double *__restrict__ v, int64_t n) {
    const int64_t at = *pi;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        v[r] = keep * v[r] + ((r == at) ? 1.0 : 0.0);
}

template <typename VT>
__global__ void k_scale(VT *__restrict__ w, int64_t n, const double *__restrict__ nrm2) {
    __shared__ VT inv_s;  // one FP64 divide and square root per block, not per thread
    if (threadIdx.x == 0) inv_s = (VT)(1.0 / sqrt(*nrm2));
    __syncthreads();
    const VT inv = inv_s;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        w[r] = w[r] * inv;
}

// out_i = sum_{l<m} V_l Y[l + m*i], i < k (Y column-major on the device).
// KMAX bounds k at compile time: the single-vector form (a Ritz vector) keeps one
// accumulator instead of kMaxKeep.
template <typename VT, typename OT, int KMAX = kMaxKeep>
__global__ void __launch_bounds__(kVecThreads) k_combine(const VT *__restrict__ V, int64_t ld, int m,
                                                         const double *__restrict__ Y, int k, OT *__restrict__ out,
                                                         int64_t ldo, int64_t n) {
    __shared__ double y[kMaxBasis * KMAX];
    for (int i = threadIdx.x; i < m * k; i += blockDim.x) y[i] = Y[i];
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double acc[KMAX];
#pragma unroll
        for (int i = 0; i < KMAX; ++i) acc[i] = 0;
        int l = 0;
        for (; l + 4 <= m; l += 4) {  // four loads in flight, terms added in order
            double v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = (double)V[(int64_t)(l + q) * ld + r];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int i = 0; i < KMAX; ++i)
                    if (i < k) acc[i] += v[q] * y[l + q + m * i];
        }
        for (; l < m; ++l) {
            const double v = (double)V[(int64_t)l * ld + r];
#pragma unroll
            for (int i = 0; i < KMAX; ++i)
                if (i < k) acc[i] += v * y[l + m * i];
        }
#pragma unroll
        for (int i = 0; i < KMAX; ++i)
            if (i < k) out[(int64_t)i * ldo + r] = (OT)acc[i];
    }
}

// r = w - E c; partial ||r||^2.
__global__ void __launch_bounds__(kVecThreads) k_residual(const double *__restrict__ w, const double *__restrict__ c,
                                                          double E, double *__restrict__ r, int64_t n,
                                                          double *__restrict__ nrm, double *__restrict__ nrm_out,
                                                          unsigned *__restrict__ ticket) {
    double acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = w[i] - E * c[i];
        r[i] = x;
        acc += x * x;
    }
    __shared__ double sh[kVecThreads / 32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < kVecThreads / 32; ++k) s += sh[k];
        nrm[blockIdx.x] = s;
    }
    reduce_in_last_block(nrm, 1, nrm_out, ticket);
}

__global__ void k_axpby64(double a, const double *__restrict__ x, double b, double *__restrict__ y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__global__ void k_random(double *v, int64_t n, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t h = splitmix64(seed * 0x100000001B3ull ^ (uint64_t)i);
        v[i] = (double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    }
}

template <typename S, typename D>
__global__ void k_convert(const S *__restrict__ s, D *__restrict__ d, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (D)s[i];
}

// ---------------------------------------------------------------------------
// Host-side helpers around the kernels.

// Pinned result buffers are pooled for the life of the process: cudaFreeHost
// synchronises the whole device, which would stall every concurrent solve.
constexpr size_t kPinnedDoubles = 4 * (kMaxBasis + 2);
std::mutex g_pinned_mutex;
std::vector<double *> g_pinned_pool;

double *pinned_get() {
    {
        std::lock_guard<std::mutex> lock(g_pinned_mutex);
        if (!g_pinned_pool.empty()) {
            double *p = g_pinned_pool.back();
            g_pinned_pool.pop_back();
            return p;
        }
    }
    double *p = nullptr;
    CIGPU_CUDA(cudaMallocHost(&p, sizeof(double) * kPinnedDoubles));
    return p;
}

void pinned_put(double *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_pinned_mutex);
    g_pinned_pool.push_back(p);
}

// FP32 vectors the 16-byte-load kernels take: length and row stride divisible by 4,
// 16-byte aligned start.
inline bool vec4_ok(const float *p, int64_t ld, int64_t n) {
    return n % 4 == 0 && ld % 4 == 0 && (reinterpret_cast<uintptr_t>(p) & 15) == 0;
}

struct VecOps {
    static constexpr int kTickets = (kMaxBasis + 2 + kDotChunk - 1) / kDotChunk;
    cudaStream_t s;
    int G;                   // blocks of the elementwise and update kernels: one element per thread
    int Gd;                  // blocks (per chunk) of the dot kernels: about four elements per thread
    DevBuf<double> partial;  // [(kMaxBasis+2) * max(G, Gd)]
    DevBuf<double> out;      // [4 * (kMaxBasis+2)]
    DevBuf<unsigned> ticket; // last-block counters of the fused reductions (one per dot chunk)
    double *h_out = nullptr; // pinned
    VecOps(cudaStream_t st, int64_t n)
        : s(st), G(vec_grid_for(n)), Gd(dot_grid_for(n)),
          partial((size_t)(kMaxBasis + 2) * std::max(vec_grid_for(n), dot_grid_for(n))), out(4 * (kMaxBasis + 2)),
          ticket(kTickets) {
        CIGPU_CUDA(cudaMemsetAsync(ticket.p, 0, sizeof(unsigned) * kTickets, s));
        h_out = pinned_get();
    }
    ~VecOps() {
        // normally every copy into h_out has been waited for; on an error path wait here
        if (std::uncaught_exceptions() > 0) cudaStreamSynchronize(s);
        pinned_put(h_out);
    }
    // out[dst .. dst+nvec) = V_i . w   (AT: arithmetic type of the products)
    // skip_at >= 0: the kernel does nothing when out[skip_at] != 0
    template <typename VT, typename WT, typename AT = double>
    void dots(const VT *V, int64_t ld, int nvec, const WT *w, int64_t n, int dst, int skip_at = -1) {
        dim3 grid(Gd, (nvec + kDotChunk - 1) / kDotChunk);
        if constexpr (std::is_same<VT, float>::value && std::is_same<WT, float>::value &&
                      std::is_same<AT, float>::value) {
            if (vec4_ok(V, ld, n) && vec4_ok(w, 0, n)) {
                k_multidot_f4<<<grid, kVecThreads, 0, s>>>(reinterpret_cast<const float4 *>(V), ld / 4, nvec,
                                                           reinterpret_cast<const float4 *>(w), n / 4, partial.p,
                                                           out.p + dst, ticket.p,
                                                           skip_at >= 0 ? out.p + skip_at : nullptr);
                CIGPU_CUDA(cudaGetLastError());
                count_launch();
                return;
            }
        }
        k_multidot<VT, WT, AT><<<grid, kVecThreads, 0, s>>>(V, ld, nvec, w, n, partial.p, out.p + dst, ticket.p,
                                                            skip_at >= 0 ? out.p + skip_at : nullptr);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
    }
    // skip_at >= 0: nothing when out[skip_at] != 0; gate_at >= 0 (with nrm_at):
    // out[gate_at] = 1 when ||w||^2 after the update is at least half of out[ref_at]
    template <typename VT, typename WT, typename AT = double>
    void update(const VT *V, int64_t ld, int nvec, int coef_at, WT *w, int64_t n, int nrm_at, int skip_at = -1,
                int ref_at = -1, int gate_at = -1) {
        if constexpr (std::is_same<VT, float>::value && std::is_same<WT, float>::value &&
                      std::is_same<AT, float>::value) {
            if (vec4_ok(V, ld, n) && vec4_ok(w, 0, n)) {
                k_update_f4<<<vec_grid_for(n / 4), kVecThreads, 0, s>>>(
                    reinterpret_cast<const float4 *>(V), ld / 4, nvec, out.p + coef_at, reinterpret_cast<float4 *>(w),
                    n / 4, nrm_at >= 0 ? partial.p : nullptr, nrm_at >= 0 ? out.p + nrm_at : nullptr, ticket.p,
                    skip_at >= 0 ? out.p + skip_at : nullptr, ref_at >= 0 ? out.p + ref_at : nullptr,
                    gate_at >= 0 ? out.p + gate_at : nullptr);
                CIGPU_CUDA(cudaGetLastError());
                count_launch();
                return;
            }
        }
        k_update<VT, WT, AT><<<G, kVecThreads, 0, s>>>(V, ld, nvec, out.p + coef_at, w, n,
                                                       nrm_at >= 0 ? partial.p : nullptr,
                                                       nrm_at >= 0 ? out.p + nrm_at : nullptr, ticket.p,
                                                       skip_at >= 0 ? out.p + skip_at : nullptr,
                                                       ref_at >= 0 ? out.p + ref_at : nullptr,
                                                       gate_at >= 0 ? out.p + gate_at : nullptr);
        count_launch();
        CIGPU_CUDA(cudaGetLastError());
    }
    template <typename VT>
    void scale(VT *w, int64_t n, int nrm_at) {
        k_scale<VT><<<G, kVecThreads, 0, s>>>(w, n, out.p + nrm_at);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
    }
    // fetch out[0..cnt) to the host (synchronises the stream)
    const double *fetch(int cnt) {
        CIGPU_CUDA(cudaMemcpyAsync(h_out, out.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s));
        const double t0 = wall();
        CIGPU_CUDA(cudaStreamSynchronize(s));
        g_clk.wait += wall() - t0;
        ++g_clk.n_wait;
        return h_out;
    }
    double residual(const double *w, const double *c, double E, double *r, int64_t n) {
        k_residual<<<G, kVecThreads, 0, s>>>(w, c, E, r, n, partial.p, out.p, ticket.p);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
        return std::sqrt(fetch(1)[0]);
    }
};

}  // namespace

// ---------------------------------------------------------------------------
void small_eigh(int n, std::vector<double> &a, std::vector<double> &w, std::vector<double> &z) {
    struct Acc {
        double t0 = wall();
        ~Acc() { g_clk.eigh += wall() - t0; ++g_clk.n_eigh; }
    } acc_;
    symmetric_eigh(n, a, w, z);
}

void dev_fill_random(double *v, int64_t n, uint64_t seed, cudaStream_t s) {
    k_random<<<vec_grid(), kVecThreads, 0, s>>>(v, n, seed);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}
void dev_convert(const double *src, float *dst, int64_t n, cudaStream_t s) {
    k_convert<double, float><<<vec_grid(), kVecThreads, 0, s>>>(src, dst, n);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}
void dev_convert(const float *src, double *dst, int64_t n, cudaStream_t s) {
    k_convert<float, double><<<vec_grid(), kVecThreads, 0, s>>>(src, dst, n);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

namespace {

// Thick-restart Lanczos on storage type VT.
template <typename VT>
struct TRLanczos {
    int64_t n;
    int m, keep;
    cudaStream_t s;
    VecOps &ops;
    DevBuf<VT> V;     // (m+1) vectors of n
    DevBuf<VT> tmp;   // keep vectors
    DevBuf<double> Yd;
    std::vector<double> T;  // (m+1) x (m+1) row-major
    int j = 0;              // next vector to expand; V[0..j] valid, T columns [0, j) known
    int64_t matvecs = 0;
    int restarts = 0;
    double theta0 = 0, theta1 = 0, resid_est = 1e300;
    std::vector<double> y0;  // lowest Ritz vector of T[0..j)
    std::function<void(const VT *, VT *, cudaStream_t)> mv;

    TRLanczos(int64_t n_, int m_, int keep_, cudaStream_t s_, VecOps &o)
        : n(n_), m(m_), keep(keep_), s(s_), ops(o), V((size_t)(m_ + 1) * n_), tmp((size_t)keep_ * n_),
          Yd((size_t)m_ * keep_), T((size_t)(m_ + 1) * (m_ + 1), 0.0) {}

    double &t(int i, int k) { return T[(size_t)i * (m + 1) + k]; }
    VT *vec(int i) { return V.p + (size_t)i * n; }

    // V[0] = normalised start
    void start(const VT *v0) {
        CIGPU_CUDA(cudaMemcpyAsync(vec(0), v0, sizeof(VT) * n, cudaMemcpyDeviceToDevice, s));
        ops.dots(vec(0), n, 1, vec(0), n, 0);
        ops.scale(vec(0), n, 0);
        std::fill(T.begin(), T.end(), 0.0);
        j = 0;
    }

    // One Lanczos step, split in two so the next step can run on the device while
    // the host analyses the projected matrix: enqueue() expands V[j] -> V[j+1] and
    // queues the copy of the coefficients; finish() waits and records them.
    static constexpr int H1 = 0, H2 = kMaxBasis + 1, NR = 2 * (kMaxBasis + 1);
    void enqueue() {
        VT *w = vec(j + 1);
        mv(vec(j), w, s);
        ++matvecs;
        const int nv = j + 1;
        ops.dots(V.p, n, nv, w, n, H1);
        ops.update(V.p, n, nv, H1, w, n, -1);
        ops.dots(V.p, n, nv, w, n, H2);
        ops.update(V.p, n, nv, H2, w, n, NR);
        ops.scale(w, n, NR);
        CIGPU_CUDA(cudaMemcpyAsync(ops.h_out, ops.out.p, sizeof(double) * (NR + 1), cudaMemcpyDeviceToHost, s));
    }
    double finish() {
        const double t0 = wall();
        CIGPU_CUDA(cudaStreamSynchronize(s));
        g_clk.wait += wall() - t0;
        ++g_clk.n_wait;
        const double *h = ops.h_out;
        for (int i = 0; i <= j; ++i) {
            const double v = h[H1 + i] + h[H2 + i];
            t(i, j) = v;
            t(j, i) = v;
        }
        const double beta = std::sqrt(h[NR]);
        t(j + 1, j) = beta;
        t(j, j + 1) = beta;
        ++j;
        return beta;
    }
    double step() {
        enqueue();
        return finish();
    }

    // Ritz analysis of T[0..j); updates theta0/theta1/y0/resid_est.
    void analyse(std::vector<double> *W = nullptr, std::vector<double> *Z = nullptr) {
        std::vector<double> a((size_t)j * j), w, z;
        for (int i = 0; i < j; ++i)
            for (int k = 0; k < j; ++k) a[(size_t)i * j + k] = t(i, k);
        small_eigh(j, a, w, z);
        theta0 = w[0];
        theta1 = j > 1 ? w[1] : w[0];
        y0.resize(j);
        for (int i = 0; i < j; ++i) y0[i] = z[(size_t)i * j];
        resid_est = std::fabs(t(j, j - 1) * y0[j - 1]);
        if (W) *W = w;
        if (Z) *Z = z;
    }

    void restart() {
        std::vector<double> w, z;
        analyse(&w, &z);
        const int kk = std::min(keep, m - 1);
        std::vector<double> Y((size_t)m * kk);
        for (int i = 0; i < kk; ++i)
            for (int l = 0; l < m; ++l) Y[(size_t)i * m + l] = z[(size_t)l * m + i];
        CIGPU_CUDA(cudaMemcpyAsync(Yd.p, Y.data(), sizeof(double) * Y.size(), cudaMemcpyHostToDevice, s));
        k_combine<VT, VT><<<ops.G, kVecThreads, 0, s>>>(V.p, n, m, Yd.p, kk, tmp.p, n, n);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
        CIGPU_CUDA(cudaMemcpyAsync(vec(0), tmp.p, sizeof(VT) * n * kk, cudaMemcpyDeviceToDevice, s));
        CIGPU_CUDA(cudaMemcpyAsync(vec(kk), vec(m), sizeof(VT) * n, cudaMemcpyDeviceToDevice, s));
        const double beta = t(m, m - 1);
        std::fill(T.begin(), T.end(), 0.0);
        for (int i = 0; i < kk; ++i) {
            t(i, i) = w[i];
            t(kk, i) = t(i, kk) = beta * z[(size_t)(m - 1) * m + i];
        }
        j = kk;
        ++restarts;
        CIGPU_CUDA(cudaStreamSynchronize(s));  // Y staging buffer is host memory
    }

    // c = V[0..j) y0 (FP64 output)
    void ritz_vector(double *c_dev) {
        CIGPU_CUDA(cudaMemcpyAsync(Yd.p, y0.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s));
        k_combine<VT, double, 1><<<ops.G, kVecThreads, 0, s>>>(V.p, n, j, Yd.p, 1, c_dev, n, n);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
        CIGPU_CUDA(cudaStreamSynchronize(s));
    }

    // Iterate until resid_est <= max(abs_target, rel_target * max(1, |theta0|)), the
    // matvec budget is spent, breakdown, or stagnation (no 10% gain in 3 cycles).
    // The step after the current one is already running on the device while the host
    // diagonalises T; when the target is met that speculative step is discarded
    // (V[0..j) and T are untouched by it). Returns true when the target was met.
    bool run(double abs_target, double rel_target, int64_t budget) {
        double best = 1e300;
        int64_t best_at = matvecs;
        auto target = [&] { return std::max(abs_target, rel_target * std::max(1.0, std::fabs(theta0))); };
        bool inflight = false;
        if (matvecs < budget && j < m && j < n) {
            enqueue();
            inflight = true;
        }
        while (inflight) {
            const double beta = finish();
            inflight = false;
            const bool breakdown = beta <= 1e-13 * std::max(1.0, std::fabs(theta0));
            if (!breakdown && j < m && j < n && matvecs < budget) {
                enqueue();  // overlaps with the analysis below
                inflight = true;
            }
            analyse();
            if (breakdown) resid_est = 0.0;
            bool stop = resid_est <= target();
            if (!stop) {
                if (resid_est < 0.9 * best) {
                    best = resid_est;
                    best_at = matvecs;
                } else if (matvecs - best_at > 3 * m) {
                    stop = true;  // stagnated
                }
            }
            if (stop || j >= n || breakdown) {
                if (inflight) {  // discard the speculative step
                    CIGPU_CUDA(cudaStreamSynchronize(s));
                    inflight = false;
                }
                return resid_est <= target() || j >= n;
            }
            if (!inflight && j == m) {
                restart();
                if (matvecs < budget) {
                    enqueue();
                    inflight = true;
                }
            }
        }
        analyse();
        return resid_est <= target();
    }
};

// FP64 Rayleigh quotient and residual of c (normalised in place).
struct Refine {
    int64_t n;
    cudaStream_t s;
    VecOps &ops;
    DevBuf<double> w, r, t;
    Refine(int64_t n_, cudaStream_t s_, VecOps &o) : n(n_), s(s_), ops(o), w(n_), r(n_), t(n_) {}
    // returns (E, ||r||) with w = H c, r = w - E c
    std::pair<double, double> eval(const SolveProblem &P, double *c) {
        ops.dots(c, n, 1, c, n, 0);
        ops.scale(c, n, 0);
        P.mv64(c, w.p, s);
        ops.dots(c, n, 1, w.p, n, 0);
        const double E = ops.fetch(1)[0];
        const double rn = ops.residual(w.p, c, E, r.p, n);
        return {E, rn};
    }
    // the same from the FP32 product (c32, w32: FP32 scratch vectors): w = H c to
    // FP32 accuracy, E and r as above
    std::pair<double, double> eval32(const SolveProblem &P, double *c, float *c32, float *w32) {
        ops.dots(c, n, 1, c, n, 0);
        ops.scale(c, n, 0);
        dev_convert(c, c32, n, s);
        P.mv32(c32, w32, s);
        dev_convert(w32, w.p, n, s);
        ops.dots(c, n, 1, w.p, n, 0);
        const double E = ops.fetch(1)[0];
        const double rn = ops.residual(w.p, c, E, r.p, n);
        return {E, rn};
    }
};

}  // namespace

static void trace_report(const char *what, const cigpu_solve_info &info, double t0) {
    const char *e = std::getenv("CIGPU_TRACE");
    if (!(e && e[0] == '1')) return;
    std::fprintf(stderr, "[cigpu solve] %s: %.3f ms total, host eigensolves %lld (%.3f ms), waits %lld (%.3f ms), mv64 %lld mv32 %lld\n",
                 what, (wall() - t0) * 1e3, (long long)g_clk.n_eigh, g_clk.eigh * 1e3, (long long)g_clk.n_wait,
                 g_clk.wait * 1e3, (long long)info.matvecs_fp64, (long long)info.matvecs_fp32);
}

int solve_fp64(const SolveProblem &P, const SolveOptions &o, double *c_dev, bool have_start, cigpu_solve_info &info) {
    g_clk = SolveClock{};
    const double tstart = wall();
    const int64_t n = P.n;
    const int64_t budget = o.max_matvec > 0 ? o.max_matvec : 3 * n;
    const int m = (int)std::min<int64_t>(std::min(o.basis, kMaxBasis), std::max<int64_t>(n, 1));
    const int keep = std::max(1, std::min({o.keep, m - 1, kMaxKeep}));
    cudaStream_t s = P.stream;
    VecOps ops(s, n);
    if (!have_start) dev_fill_random(c_dev, n, o.seed, s);
    Refine ref(n, s, ops);
    if (n == 1) {
        auto er = ref.eval(P, c_dev);
        info.e0 = er.first;
        info.residual = er.second;
        info.matvecs_fp64 = 1;
        info.converged = 1;
        return CIGPU_OK;
    }
    TRLanczos<double> lz(n, m, keep, s, ops);
    lz.mv = [&](const double *x, double *y, cudaStream_t st) { P.mv64(x, y, st); };
    lz.start(c_dev);
    double target = o.tol;
    std::pair<double, double> er{0, 1e300};
    for (int attempt = 0; attempt < 8; ++attempt) {
        const bool ok = lz.run(target, 0.0, budget);
        lz.ritz_vector(c_dev);
        er = ref.eval(P, c_dev);
        if (er.second <= o.tol || !ok) break;
        // the estimate was optimistic: tighten it and keep iterating
        target = std::max(target * 0.1, 1e-15);
    }
    info.e0 = er.first;
    info.residual = er.second;
    info.gap = lz.theta1 - lz.theta0;
    info.error_bound = info.gap > 0 ? er.second * er.second / info.gap : er.second;
    info.matvecs_fp64 = lz.matvecs + 1 + 0;
    info.restarts = lz.restarts;
    info.converged = er.second <= o.tol;
    trace_report("fp64 lanczos", info, tstart);
    return info.converged ? CIGPU_OK : CIGPU_ENOCONV;
}

int solve_mixed(const SolveProblem &P, const SolveOptions &o, double *c_dev, bool have_start, cigpu_solve_info &info) {
    // Anchored mixed-precision Davidson.
    //   anchor c (FP64) with w = H c from an FP64 matvec, E = c.w, r = w - E c (exact);
    //   corrections v_1..v_k stored in FP32 with H v_i from the FP32 CRS matvec; all
    //   per-iteration vector arithmetic is FP32 with FP64 reductions;
    //   projected matrix over [c, v_i - eta_i c] (eta_i = c.v_i):
    //       G = [[E, r.v_j], [r.v_i, v_i.H32 v_j]]
    //   new direction t = ru / (theta - H_ii) (diagonal preconditioner) where ru is the
    //   Davidson residual assembled from FP32 vectors. The FP32 error in ru scales with
    //   the correction size |y_v|, so once ru approaches eps32 |H| |y_v| (or the basis is
    //   full) the correction is folded into the anchor and the residual is recomputed
    //   exactly with an FP64 matvec (residual-correction restart).
    //   A fold keeps one direction besides the new anchor: the previous step's Ritz
    //   vector, orthogonalised against the current one (a "GD+1" restart). Its
    //   image under H is the same combination of H c (kept in FP32) and the H v_i,
    //   so it costs no matvec, and the restarted basis keeps the recurrence that a
    //   collapse to the anchor alone loses: on an L=11 4a4b problem whose 30-vector
    //   cycles only halved the residual this cut the matvecs from ~250 to ~105.
    // Basis slots: 0 = fp32(c) (orthogonalisation; HV slot 0 = fp32(H c)),
    // 1..k = corrections, k+1 = new.
    const int64_t n = P.n;
    const int64_t budget = o.max_matvec > 0 ? o.max_matvec : 3 * n;
    cudaStream_t s = P.stream;
    g_clk = SolveClock{};
    const double tstart = wall();
    if (n <= 2 || !P.mv32 || !P.diag) {
        if (!have_start) dev_fill_random(c_dev, n, o.seed, s);
        return solve_fp64(P, o, c_dev, true, info);
    }
    VecOps ops(s, n);
    Refine ref(n, s, ops);
    const int mmax = (int)std::min<int64_t>(std::min(o.dav_basis, kMaxBasis - 2), n - 2);
    DevBuf<float> V((size_t)(mmax + 2) * n), HV((size_t)(mmax + 2) * n), cr32((size_t)2 * n), diag32(n);
    dev_convert(P.diag, diag32.p, n, s);  // FP32 diagonal for the preconditioner
    DevBuf<double> yd(kMaxBasis + 1), dd(kMaxBasis + 2);
    int64_t mv32 = 0, mv64 = 0;
    // the lowest diagonal element (value in pv[0], index in pi[0]): the preconditioner's
    // shift bound and the cold start's determinant
    DevBuf<double> pv(ops.G);
    DevBuf<int64_t> pi(ops.G);
    k_argmin_partial<<<ops.G, kVecThreads, 0, s>>>(P.diag, n, pv.p, pi.p);
    k_argmin_final<<<1, 32, 0, s>>>(pv.p, pi.p, ops.G);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(2);
    const double *dmin = pv.p;
    if (!have_start) {
        // Krylov start. Davidson from the lowest-diagonal determinant alone can settle
        // on an excited state when that determinant overlaps the ground state weakly
        // (few electrons in many orbitals, strong two-electron terms). Instead take
        // q0 = e_argmin + g (g uniform random, |g| ~ 1), run kStartSteps FP32 Lanczos
        // steps with full reorthogonalisation, and start from the lowest Ritz vector.
        dev_fill_random(c_dev, n, o.seed, s);
        k_add_unit_at<<<ops.G, kVecThreads, 0, s>>>(pi.p, std::sqrt(3.0 / (double)n), c_dev, n);
        CIGPU_CUDA(cudaGetLastError());
        count_launch(1);
        const int m0 = (int)std::min<int64_t>(kStartSteps, std::min<int64_t>(n - 1, mmax + 1));
        constexpr int kCol = 44, kNrm = 100;  // out[] slots: T columns, norms (coefficients at 0)
        dev_convert(c_dev, V.p, n, s);
        ops.dots<float, float, float>(V.p, n, 1, V.p, n, kNrm);
        ops.scale(V.p, n, kNrm);
        for (int j = 0; j < m0; ++j) {
            float *w = V.p + (size_t)(j + 1) * n;
            P.mv32(V.p + (size_t)j * n, w, s);
            ++mv32;
            ops.dots<float, float, float>(V.p, n, j + 1, w, n, kCol + 8 * j);  // column j of T
            if (j + 1 == m0) break;
            ops.update<float, float, float>(V.p, n, j + 1, kCol + 8 * j, w, n, -1);
            ops.dots<float, float, float>(V.p, n, j + 1, w, n, 0);
            ops.update<float, float, float>(V.p, n, j + 1, 0, w, n, kNrm + 1 + j);
            ops.scale(w, n, kNrm + 1 + j);
        }
        const double *h = ops.fetch(kNrm + 1 + m0);
        // an invariant Krylov space ends the start early (later slots hold no basis vectors)
        int m = m0;
        for (int j = 0; j + 1 < m0; ++j) {
            const double d = h[kCol + 8 * j + j];
            if (!(h[kNrm + 1 + j] > 1e-24 * (1.0 + d * d))) {
                m = j + 1;
                break;
            }
        }
        std::vector<double> T((size_t)m * m), tw, tz;
        for (int j = 0; j < m; ++j)
            for (int i = 0; i <= j; ++i) T[(size_t)i * m + j] = T[(size_t)j * m + i] = h[kCol + 8 * j + i];
        small_eigh(m, T, tw, tz);
        std::vector<double> y0(m);
        for (int i = 0; i < m; ++i) y0[i] = tz[(size_t)i * m];
        CIGPU_CUDA(cudaMemcpyAsync(yd.p, y0.data(), sizeof(double) * m, cudaMemcpyHostToDevice, s));
        k_combine<float, double, 1><<<ops.G, kVecThreads, 0, s>>>(V.p, n, m, yd.p, 1, c_dev, n, n);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
    }
    std::vector<double> A((size_t)kMaxBasis * kMaxBasis, 0.0), eta(kMaxBasis, 0.0), bvec(kMaxBasis, 0.0);
    int collapses = 0;
    double E = 0, rho = 0, gap = 0, last_rho = 1e300;
    auto anchor = [&](bool fp32) {  // anchor evaluation: exact FP64, or the cold start's FP32 one
        const auto er = fp32 ? ref.eval32(P, c_dev, V.p, HV.p) : ref.eval(P, c_dev);
        ++(fp32 ? mv32 : mv64);
        E = er.first;
        rho = er.second;
        dev_convert(c_dev, V.p, n, s);          // slot 0
        dev_convert(ref.w.p, HV.p, n, s);       // H c, for the restart direction
        dev_convert(c_dev, cr32.p, n, s);       // c32, r32 for the couplings
        dev_convert(ref.r.p, cr32.p + n, n, s);
    };
    // A cold start's first anchor only turns the start vector (residual of order
    // |H|) into the first basis, so the FP32 product can serve it where it is much
    // cheaper than the FP64 one (FCI L=12 6a6b: 0.35 against 2.7 ms; one more FP32
    // product per solve); every later anchor, and so the residual the solve reports,
    // is the exact FP64 one. Where the two cost about the same (the DOCI pair hops:
    // 1.1 against 1.7 ms) the FP32 anchor's error floor, relative to |E|, cost more
    // FP32 steps than it saved (L=24 12 pairs: 24 + 2 against 21 + 3 products). A
    // warm start may already be near the tolerance and takes the FP64 product.
    anchor(!have_start && P.fp32_first_anchor);
    int k = 0;  // corrections in the basis
    double theta = E, a0 = 1.0, yv = 0;
    std::vector<double> y(kMaxBasis + 1, 0.0), yp(kMaxBasis + 1, 0.0), d(kMaxBasis + 1, 0.0);
    int ky = -1, kp = -1;  // corrections behind y and yp (-1: not of the current basis)
    double a0p = 0;
    int kept = 0;
    const int SLOT_R = 3 * (kMaxBasis + 1), SLOT_N = SLOT_R + 1, SLOT_G = SLOT_R + 2;
    while (rho > o.tol && mv32 + mv64 < budget) {
        float *vnew = V.p + (size_t)(k + 1) * n;
        float *hvnew = HV.p + (size_t)(k + 1) * n;
        // preconditioned direction into slot k+1 (and ||ru||^2 into SLOT_R)
        if (k == 0) {
            k_precond32<<<ops.G, kVecThreads, 0, s>>>(ref.r.p, P.diag, E, dmin, vnew, n);
            count_launch();
        } else {
            CIGPU_CUDA(cudaMemcpyAsync(yd.p, y.data() + 1, sizeof(double) * k, cudaMemcpyHostToDevice, s));
            if (vec4_ok(cr32.p + n, n, n) && vec4_ok(V.p, n, n) && vec4_ok(HV.p, n, n) && vec4_ok(diag32.p, 0, n) &&
                vec4_ok(vnew, 0, n)) {
                using F4 = const float4 *;
                k_dav_residual32_f4<<<vec_grid_for(n / 4), kVecThreads, 0, s>>>(
                    F4(cr32.p + n), F4(cr32.p), F4(V.p), F4(HV.p), n / 4, k, yd.p, a0, a0 * (E - theta), theta, dmin,
                    F4(diag32.p), reinterpret_cast<float4 *>(vnew), n / 4, ops.partial.p, ops.out.p + SLOT_R,
                    ops.ticket.p);
            } else {
                k_dav_residual32<<<ops.G, kVecThreads, 0, s>>>(cr32.p + n, cr32.p, V.p, HV.p, n, k, yd.p, a0,
                                                                a0 * (E - theta), theta, dmin, diag32.p, vnew, n,
                                                                ops.partial.p, ops.out.p + SLOT_R, ops.ticket.p);
            }
            CIGPU_CUDA(cudaGetLastError());
            count_launch();
        }
        // orthonormalise against slots 0..k (FP32 arithmetic, FP64 reductions): one
        // classical Gram-Schmidt pass, and a second one only when the first removed
        // more than half of ||t||^2 (DGKS, decided on the device: the second pass's
        // kernels return at once otherwise). The first dots include t itself (slot
        // k + 1), giving ||t||^2 in out[k + 1].
        ops.dots<float, float, float>(V.p, n, k + 2, vnew, n, 0);
        ops.update<float, float, float>(V.p, n, k + 1, 0, vnew, n, SLOT_N, -1, k + 1, SLOT_G);
        ops.dots<float, float, float>(V.p, n, k + 1, vnew, n, 0, SLOT_G);
        ops.update<float, float, float>(V.p, n, k + 1, 0, vnew, n, SLOT_N, SLOT_G);
        ops.scale(vnew, n, SLOT_N);
        P.mv32(vnew, hvnew, s);
        ++mv32;
        // projection column and couplings: V[1..k+1].Hv_new, then c32.v_new, r32.v_new
        ops.dots<float, float, float>(V.p + n, n, k + 1, hvnew, n, 0);
        ops.dots<float, float, float>(cr32.p, n, 2, vnew, n, k + 1);
        const double *h = ops.fetch(SLOT_N + 1);
        const double tn2 = h[SLOT_N];
        const double rho_u = (k > 0) ? std::sqrt(h[SLOT_R]) : 1e300;
        if (!(tn2 > 1e-28)) {
            // the search space is invariant: fold what we have and stop expanding
            if (k == 0) break;
        } else {
            for (int i = 0; i <= k; ++i) {
                A[(size_t)i * kMaxBasis + k] = h[i];
                A[(size_t)k * kMaxBasis + i] = h[i];
            }
            eta[k] = h[k + 1];
            bvec[k] = h[k + 2];
            ++k;
        }
        // Rayleigh-Ritz over [c, v_1..v_k]
        const int q = k + 1;
        std::vector<double> G((size_t)q * q, 0.0), wv, zv;
        G[0] = E;
        for (int i = 0; i < k; ++i) G[(size_t)(i + 1)] = G[(size_t)(i + 1) * q] = bvec[i];
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) G[(size_t)(i + 1) * q + (j + 1)] = A[(size_t)i * kMaxBasis + j];
        small_eigh(q, G, wv, zv);
        if (ky >= 0) {  // the previous Ritz vector, for a restart
            std::copy(y.begin(), y.begin() + ky + 1, yp.begin());
            a0p = a0;
        }
        kp = ky;
        theta = wv[0];
        if (q > 1) gap = wv[1] - wv[0];
        for (int i = 0; i < q; ++i) y[i] = zv[(size_t)i * q];
        a0 = y[0];
        for (int i = 1; i <= k; ++i) a0 -= y[i] * eta[i - 1];
        ky = k;
        // fold when the previous approximate residual reached the FP32 floor of the
        // correction (the new solution, with one more vector, is at least as good),
        // when the basis is full, or on breakdown
        const double floor = 30.0 * 6e-8 * std::max(1.0, std::fabs(theta)) * yv;
        const bool fold = rho_u <= std::max(0.5 * o.tol, floor) || k >= mmax || !(tn2 > 1e-28);
        yv = 0;
        for (int i = 1; i <= k; ++i) yv += y[i] * y[i];
        yv = std::sqrt(yv);
        if (fold) {
            // restart direction: the previous Ritz vector p minus its component along
            // the current one u, in the basis [c, v_1..v_k] (coefficients (a0, y_i)),
            // formed with its H image in the spare slot k+1 before the anchor moves
            // only a fold of a full basis keeps it: a fold at the FP32 floor of the
            // correction restarts clean (the kept direction would carry that floor
            // into the next cycle, and at tight tolerances the cycles then stall)
            bool keep = false;
            if (kp >= 0 && kp <= k && k >= mmax && !(rho_u <= std::max(0.5 * o.tol, floor)) && tn2 > 1e-28) {
                double uu = a0 * a0, up = a0 * a0p;
                for (int i = 1; i <= k; ++i) {
                    uu += y[i] * y[i];
                    if (i <= kp) up += y[i] * yp[i];
                }
                const double f = up / uu;
                double dn = 0;
                for (int i = 0; i <= k; ++i) {
                    const double pi = i == 0 ? a0p : (i <= kp ? yp[i] : 0.0);
                    d[i] = pi - f * (i == 0 ? a0 : y[i]);
                    dn += d[i] * d[i];
                }
                dn = std::sqrt(dn);
                if (dn > 1e-8) {
                    for (int i = 0; i <= k; ++i) d[i] /= dn;
                    CIGPU_CUDA(cudaMemcpyAsync(dd.p, d.data(), sizeof(double) * (k + 1), cudaMemcpyHostToDevice, s));
                    float *vs = V.p + (size_t)(k + 1) * n, *hs = HV.p + (size_t)(k + 1) * n;
                    k_combine<float, float, 1><<<ops.G, kVecThreads, 0, s>>>(V.p, n, k + 1, dd.p, 1, vs, n, n);
                    k_combine<float, float, 1><<<ops.G, kVecThreads, 0, s>>>(HV.p, n, k + 1, dd.p, 1, hs, n, n);
                    CIGPU_CUDA(cudaGetLastError());
                    count_launch(2);
                    keep = true;
                }
            }
            // c <- a0 c + sum_i y_i v_i  (FP64)
            CIGPU_CUDA(cudaMemcpyAsync(yd.p, y.data() + 1, sizeof(double) * k, cudaMemcpyHostToDevice, s));
            k_combine<float, double, 1><<<ops.G, kVecThreads, 0, s>>>(V.p + n, n, k, yd.p, 1, ref.t.p, n, n);
            k_axpby64<<<ops.G, kVecThreads, 0, s>>>(1.0, ref.t.p, a0, c_dev, n);
            CIGPU_CUDA(cudaGetLastError());
            count_launch(2);
            const int kf = k;
            anchor(false);
            ++collapses;
            k = 0;
            yv = 0;
            ky = kp = -1;
            if (rho > 0.7 * last_rho && collapses > 3) break;  // no progress between folds
            last_rho = rho;
            if (keep && rho > o.tol) {
                // the kept direction becomes v_1: one projection against the new
                // anchor (H v_1 follows with H c), normalised, then its couplings
                float *v1 = V.p + n, *h1 = HV.p + n;
                CIGPU_CUDA(cudaMemcpyAsync(v1, V.p + (size_t)(kf + 1) * n, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
                CIGPU_CUDA(cudaMemcpyAsync(h1, HV.p + (size_t)(kf + 1) * n, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
                ops.dots<float, float, float>(V.p, n, 1, v1, n, 0);
                ops.update<float, float, float>(V.p, n, 1, 0, v1, n, SLOT_N);
                ops.update<float, float, float>(HV.p, n, 1, 0, h1, n, -1);
                ops.scale(v1, n, SLOT_N);
                ops.scale(h1, n, SLOT_N);
                ops.dots<float, float, float>(v1, n, 1, h1, n, 1);
                ops.dots<float, float, float>(cr32.p, n, 2, v1, n, 2);
                const double *hr = ops.fetch(4);
                if (hr[1] == hr[1] && hr[2] == hr[2] && hr[3] == hr[3]) {
                    A[0] = hr[1];
                    eta[0] = hr[2];
                    bvec[0] = hr[3];
                    k = 1;
                    std::vector<double> G2 = {E, bvec[0], bvec[0], A[0]}, w2, z2;
                    small_eigh(2, G2, w2, z2);
                    theta = w2[0];
                    gap = w2[1] - w2[0];
                    y[0] = z2[0];
                    y[1] = z2[2];
                    a0 = y[0] - y[1] * eta[0];
                    yv = std::fabs(y[1]);
                    ky = 1;
                    ++kept;
                }
            }
        }
    }
    info.e0 = E;
    info.residual = rho;
    info.gap = gap;
    info.error_bound = gap > 0 ? rho * rho / gap : rho;
    info.matvecs_fp64 = mv64;
    info.matvecs_fp32 = mv32;
    info.restarts = kept;
    info.corrections = collapses;
    info.converged = rho <= o.tol;
    trace_report("mixed davidson", info, tstart);
    return info.converged ? CIGPU_OK : CIGPU_ENOCONV;
}

}  // namespace cigpu
