// Batched lowest eigenpairs of many independent problems (cigpu_solve_batch).
//
// The served analogue of a loop of CIMethod::solve calls over many Hamiltonians
// (CIMethod.cpp:241-264; the orbital optimisers' set_ham -> solve loop,
// SimulatedAnnealing.cpp:72-86). Solved one at a time, a small problem is
// latency-bound: each Lanczos step is a handful of tiny kernels and a host round
// trip. Here every problem up to max_batched_dim determinants is built with the
// usual FP64 CRS generator, the matrices are concatenated into one block-diagonal
// CRS, and all problems run an FP64 Lanczos in lockstep:
//   * one step = 9 kernel launches plus one SpMV launch per row-length class, each
//     serving every problem (the problems are ordered by mean row length, so each
//     class is one row range of the concatenated matrix with its own SpMV shape;
//     segmented dot products and updates over row chunks that never straddle two
//     problems; a warp per problem for the tridiagonal analysis), captured once
//     as a CUDA graph and replayed;
//   * full two-pass Gram-Schmidt against the problem's own basis, kBatchSteps
//     vectors per cycle, then an explicit restart from the Ritz vector;
//   * the lowest Ritz value of each tridiagonal matrix by 32-way multisection on
//     Sturm counts (one warp), its eigenvector by inverse iteration, and the
//     residual estimate beta * |s_last| — no host work per step;
//   * per-problem state on the device; a converged problem idles while the
//     others continue; the host reads one counter every 8 graph launches.
// The SpMV shape of each row-length class (lanes per row, grid) is picked by
// timing candidates on the batch's own rows (autotuner, cached by range size).
// Problems above max_batched_dim go through cigpu_solve with their requested
// precision, on worker streams that overlap with each other.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <tuple>
#include <vector>

#include "crs.cuh"
#include "spmv.cuh"

namespace cigpu {

namespace {

constexpr int kBatchSteps = 40;      // Lanczos vectors per cycle
constexpr int kChunkRows = 2048;     // rows per chunk of the segmented kernels
constexpr int kRowThreads = 256;
constexpr int kDotVecs = 8;          // basis vectors per dot-product block
constexpr int64_t kDefaultMaxBatchedDim = 65536;
// Worker threads (one stream each) for the problems above the batching limit.
constexpr int kBigWorkers = 3;
constexpr int64_t kMaxBatchRows = int64_t(1) << 22;  // rows per batch (basis: 40 x 4M doubles)

// action codes written by the analysis kernel
enum : int { kContinue = 0, kRestart = 1, kDone = 2, kIdle = 3, kFailed = 4 };

struct Batch {
    int P, C;
    int64_t N;
    const int64_t *rp;
    const uint32_t *col;
    const double *val;
    const int *chunk_prob;
    const int64_t *chunk_r0, *chunk_r1;
    const int *pc0, *pc1;  // chunks of problem p: [pc0[p], pc1[p])
    double *Q, *V, *W;     // basis [kBatchSteps][N], current vector, work vector
    double *part;          // [kBatchSteps][C] dot partials
    double *npart;         // [C] squared-norm partials
    double *h1, *h2;       // [kBatchSteps][P] Gram-Schmidt coefficients of the two passes
    double *alpha, *beta, *sv;  // [P][kBatchSteps] tridiagonal and Ritz coefficients
    double *theta, *res_est, *inv_beta;  // [P]
    int *j, *status, *action, *restarts, *mv, *budget;  // [P]; status 0 active, 1 converged, 2 budget spent
    int *n_active;
    double tol;
};

__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    return s;  // valid in thread 0
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__global__ void k_batch_random(double *v, int64_t n, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = (double)(mix64(seed * 0x100000001B3ull ^ (uint64_t)i) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// npart[c] = sum over the chunk of x^2
__global__ void __launch_bounds__(kRowThreads) k_chunk_norm2(Batch B, const double *x) {
    __shared__ double sh[kRowThreads / 32];
    const int c = blockIdx.x;
    double a = 0;
    for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) a += x[r] * x[r];
    a = block_sum(a, sh);
    if (threadIdx.x == 0) B.npart[c] = a;
}

// row_prob[r] = the problem of row r
__global__ void __launch_bounds__(kRowThreads) k_row_prob(Batch B, int *row_prob) {
    const int c = blockIdx.x, p = B.chunk_prob[c];
    for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) row_prob[r] = p;
}

// V = V / |V_p| per problem, Q[0] = V
__global__ void __launch_bounds__(kRowThreads) k_batch_start(Batch B) {
    const int c = blockIdx.x, p = B.chunk_prob[c];
    double s = 0;
    for (int q = B.pc0[p]; q < B.pc1[p]; ++q) s += B.npart[q];
    const double inv = s > 0 ? 1.0 / sqrt(s) : 0.0;
    for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) {
        const double v = B.V[r] * inv;
        B.V[r] = v;
        B.Q[r] = v;
    }
}

// part[k][c] = Q_k . W over chunk c for k <= j_p (kDotVecs basis vectors per block)
__global__ void __launch_bounds__(kRowThreads) k_batch_dots(Batch B) {
    __shared__ double sh[kDotVecs][kRowThreads / 32];
    const int c = blockIdx.x, p = B.chunk_prob[c];
    const int jp = B.j[p], k0 = blockIdx.y * kDotVecs;
    if (B.status[p] != 0 || k0 > jp) return;  // uniform per block
    const int nk = min(kDotVecs, jp + 1 - k0);
    double acc[kDotVecs];
#pragma unroll
    for (int i = 0; i < kDotVecs; ++i) acc[i] = 0;
    for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) {
        const double w = B.W[r];
#pragma unroll
        for (int i = 0; i < kDotVecs; ++i)
            if (i < nk) acc[i] += B.Q[(int64_t)(k0 + i) * B.N + r] * w;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < kDotVecs; ++i) {
        double a = acc[i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) sh[i][warp] = a;
    }
    __syncthreads();
    if (threadIdx.x < nk) {
        double s = 0;
        for (int w = 0; w < kRowThreads / 32; ++w) s += sh[threadIdx.x][w];
        B.part[(int64_t)(k0 + threadIdx.x) * B.C + c] = s;
    }
}

// h[k][p] = sum over p's chunks of part[k][c], fixed order
__global__ void k_batch_reduce(Batch B, double *h) {
    const int p = blockIdx.x;
    if (B.status[p] != 0) return;
    const int jp = B.j[p];
    for (int k = threadIdx.x; k <= jp; k += blockDim.x) {
        double s = 0;
        for (int q = B.pc0[p]; q < B.pc1[p]; ++q) s += B.part[(int64_t)k * B.C + q];
        h[(int64_t)k * B.P + p] = s;
    }
}

// W -= sum_{k <= j_p} h[k][p] Q_k; npart[c] = |W|^2 over the chunk
__global__ void __launch_bounds__(kRowThreads) k_batch_update(Batch B, const double *h) {
    __shared__ double cf[kBatchSteps];
    __shared__ double sh[kRowThreads / 32];
    const int c = blockIdx.x, p = B.chunk_prob[c];
    if (B.status[p] != 0) return;
    const int jp = B.j[p];
    for (int k = threadIdx.x; k <= jp; k += blockDim.x) cf[k] = h[(int64_t)k * B.P + p];
    __syncthreads();
    double a = 0;
    for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) {
        double w = B.W[r];
        for (int k = 0; k <= jp; ++k) w -= cf[k] * B.Q[(int64_t)k * B.N + r];
        B.W[r] = w;
        a += w * w;
    }
    a = block_sum(a, sh);
    if (threadIdx.x == 0) B.npart[c] = a;
}

// Number of eigenvalues of the tridiagonal (a, b) below sigma (Sturm count).
__device__ __forceinline__ int sturm_count(const double *a, const double *b, int m, double sigma) {
    int cnt = 0;
    double d = a[0] - sigma;
    if (d < 0) ++cnt;
    for (int i = 1; i < m; ++i) {
        if (d == 0) d = 1e-300;
        d = (a[i] - sigma) - b[i - 1] * b[i - 1] / d;
        if (d < 0) ++cnt;
    }
    return cnt;
}

// One warp per problem: record alpha_j, beta_j; lowest Ritz value of T_{j+1} by
// multisection; its eigenvector by inverse iteration; residual estimate; action.
__global__ void __launch_bounds__(256) k_batch_analyse(Batch B) {
    __shared__ double ta[8][kBatchSteps], tb[8][kBatchSteps], ts[8][kBatchSteps];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p = blockIdx.x * 8 + wib;
    if (p >= B.P) return;
    if (B.status[p] != 0) {
        if (lane == 0) B.action[p] = kIdle;
        return;
    }
    const int jp = B.j[p];
    double bsq = 0;
    for (int q = B.pc0[p] + lane; q < B.pc1[p]; q += 32) bsq += B.npart[q];
    for (int o = 16; o > 0; o >>= 1) bsq += __shfl_xor_sync(0xffffffffu, bsq, o);
    const double bnew = sqrt(bsq);
    const double anew = B.h1[(int64_t)jp * B.P + p] + B.h2[(int64_t)jp * B.P + p];
    const int m = jp + 1;
    double *a = ta[wib], *b = tb[wib], *s = ts[wib];
    for (int i = lane; i < m; i += 32) {
        a[i] = i == jp ? anew : B.alpha[(int64_t)p * kBatchSteps + i];
        b[i] = i == jp ? bnew : B.beta[(int64_t)p * kBatchSteps + i];
    }
    __syncwarp();
    // Gershgorin interval of T_m (couplings b[0..m-2])
    double lo = 1e300, hi = -1e300;
    for (int i = lane; i < m; i += 32) {
        const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i < m - 1 ? fabs(b[i]) : 0.0);
        lo = fmin(lo, a[i] - r);
        hi = fmax(hi, a[i] + r);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    // widen by a margin that survives rounding (a 1 x 1 matrix has lo == hi)
    const double scale = fmax(1.0, fmax(fabs(lo), fabs(hi)));
    const double margin = 1e-12 * fmax(hi - lo, 0.0) + 1e-13 * scale;
    lo -= margin;
    hi += margin;
    for (int round = 0; round < 12; ++round) {
        const double step = (hi - lo) / 33.0;
        if (!(step > 0)) break;
        const double sig = lo + step * (lane + 1);
        const unsigned ok = __ballot_sync(0xffffffffu, sturm_count(a, b, m, sig) >= 1);
        if (!ok) {  // cannot happen for a valid interval; keep the upper part
            lo = lo + step * 32;
            continue;
        }
        const int l = __ffs(ok) - 1;
        const double nlo = l == 0 ? lo : lo + step * l;
        hi = lo + step * (l + 1);
        lo = nlo;
    }
    if (lane == 0) {
        const double theta = 0.5 * (lo + hi);
        // inverse iteration on T - lo I (positive semi-definite: lo <= lambda_min)
        const double tiny = 1e-15 * scale;  // pivot floor, relative to |T|
        for (int i = 0; i < m; ++i) s[i] = 1.0;
        for (int it = 0; it < 3; ++it) {
            // (T - lo I) x = s by LDL^T (no pivoting needed: the matrix is positive
            // semi-definite), forward L y = s and backward D L^T x = y in place
            double dv[kBatchSteps];
            dv[0] = a[0] - lo;
            if (fabs(dv[0]) < tiny) dv[0] = tiny;
            for (int i = 1; i < m; ++i) {
                const double li = b[i - 1] / dv[i - 1];
                double di = (a[i] - lo) - li * b[i - 1];
                if (fabs(di) < tiny) di = tiny;
                dv[i] = di;
                s[i] -= li * s[i - 1];
            }
            s[m - 1] /= dv[m - 1];
            for (int i = m - 2; i >= 0; --i) s[i] = s[i] / dv[i] - (b[i] / dv[i]) * s[i + 1];
            // normalise without overflow: by the largest entry first
            double mx = 0;
            for (int i = 0; i < m; ++i) mx = fmax(mx, fabs(s[i]));
            const double imx = mx > 0 ? 1.0 / mx : 0.0;
            double nrm = 0;
            for (int i = 0; i < m; ++i) {
                s[i] *= imx;
                nrm += s[i] * s[i];
            }
            const double inv = nrm > 0 ? 1.0 / sqrt(nrm) : 0.0;
            for (int i = 0; i < m; ++i) s[i] *= inv;
        }
        const double res = fabs(bnew * s[m - 1]);
        const int mvp = B.mv[p] + 1;
        const bool invariant = bnew <= 1e-12 * fmax(1.0, fabs(theta)) || !(bnew == bnew);
        int act;
        if (res <= B.tol || invariant) act = kDone;
        else if (mvp >= B.budget[p]) act = kFailed;
        else if (m == kBatchSteps) act = kRestart;
        else act = kContinue;
        B.alpha[(int64_t)p * kBatchSteps + jp] = anew;
        B.beta[(int64_t)p * kBatchSteps + jp] = bnew;
        for (int i = 0; i < m; ++i) B.sv[(int64_t)p * kBatchSteps + i] = s[i];
        B.theta[p] = theta;
        B.res_est[p] = res;
        B.inv_beta[p] = act == kContinue ? 1.0 / bnew : 0.0;
        B.mv[p] = mvp;
        B.action[p] = act;
    }
}

// Continue: V = Q_{j+1} = W / beta. Restart / done: V = sum_k s_k Q_k (Ritz vector;
// it becomes Q_0 on a restart).
__global__ void __launch_bounds__(kRowThreads) k_batch_advance(Batch B) {
    __shared__ double cf[kBatchSteps];
    const int c = blockIdx.x, p = B.chunk_prob[c];
    const int act = B.action[p];
    if (act == kIdle) return;
    const int jp = B.j[p];
    if (act == kContinue) {
        const double ib = B.inv_beta[p];
        for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) {
            const double v = B.W[r] * ib;
            B.V[r] = v;
            B.Q[(int64_t)(jp + 1) * B.N + r] = v;
        }
        return;
    }
    for (int k = threadIdx.x; k <= jp; k += blockDim.x) cf[k] = B.sv[(int64_t)p * kBatchSteps + k];
    __syncthreads();
    for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) {
        double v = 0;
        for (int k = 0; k <= jp; ++k) v += cf[k] * B.Q[(int64_t)k * B.N + r];
        B.V[r] = v;
        if (act == kRestart) B.Q[r] = v;
    }
}

// Per-problem bookkeeping after a step, and the count of active problems.
__global__ void k_batch_finish(Batch B) {
    __shared__ int sh[32];
    int active = 0;
    for (int p = threadIdx.x; p < B.P; p += blockDim.x) {
        const int act = B.action[p];
        if (act == kContinue) {
            ++B.j[p];
        } else if (act == kRestart) {
            B.j[p] = 0;
            ++B.restarts[p];
        } else if (act == kDone) {
            B.status[p] = 1;
        } else if (act == kFailed) {
            B.status[p] = 2;
        }
        active += B.status[p] == 0;
    }
    for (int o = 16; o > 0; o >>= 1) active += __shfl_xor_sync(0xffffffffu, active, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = active;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        *B.n_active = t;
    }
}

// Final check: per chunk partials of V.W and V.V, then of |W - E V|^2.
__global__ void __launch_bounds__(kRowThreads) k_batch_rq_parts(Batch B) {
    __shared__ double sh[kRowThreads / 32];
    const int c = blockIdx.x;
    double vw = 0, vv = 0;
    for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) {
        vw += B.V[r] * B.W[r];
        vv += B.V[r] * B.V[r];
    }
    vw = block_sum(vw, sh);
    vv = block_sum(vv, sh);
    if (threadIdx.x == 0) {
        B.part[c] = vw;
        B.part[(int64_t)B.C + c] = vv;
    }
}

__global__ void __launch_bounds__(kRowThreads) k_batch_res_parts(Batch B, const double *E, const double *vv) {
    __shared__ double sh[kRowThreads / 32];
    const int c = blockIdx.x, p = B.chunk_prob[c];
    const double e = E[p], inv = vv[p] > 0 ? 1.0 / sqrt(vv[p]) : 0.0;
    double a = 0;
    for (int64_t r = B.chunk_r0[c] + threadIdx.x; r < B.chunk_r1[c]; r += blockDim.x) {
        const double d = (B.W[r] - e * B.V[r]) * inv;
        a += d * d;
    }
    a = block_sum(a, sh);
    if (threadIdx.x == 0) B.npart[c] = a;
}

__global__ void k_batch_rq(Batch B, double *E, double *vv) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < B.P; p += gridDim.x * blockDim.x) {
        double a = 0, b = 0;
        for (int q = B.pc0[p]; q < B.pc1[p]; ++q) {
            a += B.part[q];
            b += B.part[(int64_t)B.C + q];
        }
        vv[p] = b;
        E[p] = b > 0 ? a / b : 0.0;
    }
}

__global__ void k_batch_res(Batch B, double *res) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < B.P; p += gridDim.x * blockDim.x) {
        double a = 0;
        for (int q = B.pc0[p]; q < B.pc1[p]; ++q) a += B.npart[q];
        res[p] = sqrt(a);
    }
}

// Concatenation: problem p's CRS (local columns) into the block-diagonal CRS.
struct Part {
    const int64_t *rp;
    const uint32_t *col;
    const double *val;
    int64_t n, nnz, row0, nz0;
};

__global__ void k_concat(const Part *parts, int P, int64_t *rp, uint32_t *col, double *val) {
    const int p = blockIdx.y;
    if (p >= P) return;
    const Part q = parts[p];
    const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, ts = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = t0; i < q.nnz; i += ts) {
        col[q.nz0 + i] = (uint32_t)(q.col[i] + q.row0);
        val[q.nz0 + i] = q.val[i];
    }
    for (int64_t r = t0; r < q.n; r += ts) rp[q.row0 + r] = q.rp[r] + q.nz0;
}

// --------------------------------------------------------------------------
// Autotuned SpMV shape per matrix size.
std::mutex g_tune_mutex;
std::map<std::pair<int64_t, int64_t>, std::pair<int, int>> g_tuned;

// Candidates: lanes per row around the row-length class, grids of 4..16 blocks per SM.
std::pair<int, int> tune_spmv(int64_t n, int64_t nnz, int lanes0, const int64_t *rp, const uint32_t *col,
                              const double *val, const double *x, double *y, cudaStream_t s, bool *tuned_now) {
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tuned.find({n, nnz});
        if (it != g_tuned.end()) {
            *tuned_now = false;
            return it->second;
        }
    }
    const int sms = sm_count();
    const int per_sm_c[] = {4, 8, 16};
    cudaEvent_t e0, e1;
    CIGPU_CUDA(cudaEventCreate(&e0));
    CIGPU_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    std::pair<int, int> pick{lanes0, sms * 8};
    for (int lanes : {lanes0 / 2, lanes0, lanes0 * 2}) {
        if (lanes < 4 || lanes > 32) continue;
        for (int per_sm : per_sm_c) {
            const int64_t need = std::max<int64_t>(1, (n * lanes + kSpmvThreads - 1) / kSpmvThreads);
            const int grid = (int)std::min<int64_t>((int64_t)sms * per_sm, need);
            spmv_f64_shape(n, rp, col, val, x, y, lanes, grid, s);  // warm
            CIGPU_CUDA(cudaEventRecord(e0, s));
            for (int rep = 0; rep < 3; ++rep) spmv_f64_shape(n, rp, col, val, x, y, lanes, grid, s);
            CIGPU_CUDA(cudaEventRecord(e1, s));
            CIGPU_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            CIGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                pick = {lanes, grid};
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tuned[{n, nnz}] = pick;
    *tuned_now = true;
    return pick;
}

// Lanes per row for a mean row length (the starting point of the tuner).
int lanes_for(double mean_row) { return mean_row >= 160 ? 32 : mean_row >= 48 ? 16 : mean_row >= 16 ? 8 : 4; }

struct Item {
    int idx;
    cigpu_ham *ham = nullptr;
    cigpu_crs *crs = nullptr;
    int64_t dim = 0;
    int status = CIGPU_OK;
};

// Lockstep FP64 Lanczos over the problems of `items` (all built, FP64 CRS).
void solve_lockstep(std::vector<Item *> &items, double tol, cudaStream_t s, double *e0, cigpu_solve_info *info,
                    cigpu_batch_stats *st) {
    const int P = (int)items.size();
    if (P == 0) return;
    // order by mean row length so that each row-length class is one contiguous row
    // range: the SpMV runs one launch per class with its own shape
    auto mean_row = [](const Item *it) { return (double)it->crs->nnz_full / (double)std::max<int64_t>(1, it->crs->dim); };
    std::stable_sort(items.begin(), items.end(), [&](const Item *a, const Item *b) { return mean_row(a) < mean_row(b); });
    struct Seg {
        int64_t r0, r1, nnz;
        int lanes, grid;
    };
    std::vector<Seg> segs;
    int64_t N = 0, NNZ = 0;
    std::vector<Part> parts(P);
    std::vector<int> chunk_prob, pc0(P), pc1(P), budget(P);
    std::vector<int64_t> chunk_r0, chunk_r1;
    for (int p = 0; p < P; ++p) {
        cigpu_crs &c = *items[p]->crs;
        if (c.precision != CIGPU_FP64 || c.slots || (c.nnz_full > 0 && (!c.col.p || !c.val64.p)))
            throw std::invalid_argument("lockstep batch needs FP64 CRS matrices");
        parts[p] = Part{c.row_ptr.p, c.col.p, c.val64.p, c.dim, c.nnz_full, N, NNZ};
        pc0[p] = (int)chunk_prob.size();
        for (int64_t r = 0; r < c.dim; r += kChunkRows) {
            chunk_prob.push_back(p);
            chunk_r0.push_back(N + r);
            chunk_r1.push_back(N + std::min<int64_t>(c.dim, r + kChunkRows));
        }
        pc1[p] = (int)chunk_prob.size();
        budget[p] = (int)std::min<int64_t>(4000, std::max<int64_t>(300, 3 * c.dim));
        const int cls = lanes_for(mean_row(items[p]));
        if (segs.empty() || segs.back().lanes != cls) segs.push_back(Seg{N, N, 0, cls, 0});
        segs.back().r1 = N + c.dim;
        segs.back().nnz += c.nnz_full;
        N += c.dim;
        NNZ += c.nnz_full;
    }
    const int C = (int)chunk_prob.size();
    DevBuf<int64_t> rp(N + 1), cr0(C), cr1(C);
    DevBuf<uint32_t> col(std::max<int64_t>(NNZ, 1));
    DevBuf<double> val(std::max<int64_t>(NNZ, 1));
    DevBuf<Part> dparts(P);
    DevBuf<int> cprob(C), dpc0(P), dpc1(P), dbudget(P);
    CIGPU_CUDA(cudaMemcpyAsync(dparts.p, parts.data(), sizeof(Part) * P, cudaMemcpyHostToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(cprob.p, chunk_prob.data(), sizeof(int) * C, cudaMemcpyHostToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(cr0.p, chunk_r0.data(), sizeof(int64_t) * C, cudaMemcpyHostToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(cr1.p, chunk_r1.data(), sizeof(int64_t) * C, cudaMemcpyHostToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(dpc0.p, pc0.data(), sizeof(int) * P, cudaMemcpyHostToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(dpc1.p, pc1.data(), sizeof(int) * P, cudaMemcpyHostToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(dbudget.p, budget.data(), sizeof(int) * P, cudaMemcpyHostToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(rp.p + N, &NNZ, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    k_concat<<<dim3(64, P), 256, 0, s>>>(dparts.p, P, rp.p, col.p, val.p);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
    CIGPU_CUDA(cudaStreamSynchronize(s));  // the host copies above read stack vectors
    // the per-problem matrices are no longer needed
    for (Item *it : items) {
        cigpu_crs_destroy(it->crs);
        it->crs = nullptr;
    }

    DevBuf<double> Q((size_t)kBatchSteps * N), V(N), W(N), part((size_t)kBatchSteps * std::max(C, 2)), npart(C);
    DevBuf<double> h1((size_t)kBatchSteps * P), h2((size_t)kBatchSteps * P);
    DevBuf<double> alpha((size_t)kBatchSteps * P), beta((size_t)kBatchSteps * P), sv((size_t)kBatchSteps * P);
    DevBuf<double> theta(P), res_est(P), inv_beta(P), E(P), vv(P), res(P);
    DevBuf<int> j(P), status(P), action(P), restarts(P), mv(P), n_active(1), row_prob(N);
    for (auto *b : {&j, &status, &action, &restarts, &mv})
        CIGPU_CUDA(cudaMemsetAsync(b->p, 0, sizeof(int) * P, s));
    Batch B{P, C, N, rp.p, col.p, val.p, cprob.p, cr0.p, cr1.p, dpc0.p, dpc1.p, Q.p, V.p, W.p, part.p, npart.p,
            h1.p, h2.p, alpha.p, beta.p, sv.p, theta.p, res_est.p, inv_beta.p, j.p, status.p, action.p,
            restarts.p, mv.p, dbudget.p, n_active.p, tol};

    // start vectors: seeded random, normalised per problem
    k_row_prob<<<C, kRowThreads, 0, s>>>(B, row_prob.p);
    k_batch_random<<<sm_count() * 4, 256, 0, s>>>(V.p, N, 0x5EEDull);
    k_chunk_norm2<<<C, kRowThreads, 0, s>>>(B, V.p);
    k_batch_start<<<C, kRowThreads, 0, s>>>(B);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(4);

    // CIGPU_TRACE=1: the first problems' state after the start and the first steps
    const char *tr_env = std::getenv("CIGPU_TRACE");
    const bool trace = tr_env && tr_env[0] == '1';
    auto trace_state = [&](const char *what) {
        if (!trace) return;
        const int np = std::min(P, 3);
        std::vector<double> hv(std::min<int64_t>(N, 2)), hw(std::min<int64_t>(N, 2)), hn(1), ha(np * kBatchSteps),
            hb(np * kBatchSteps), ht(np), hr(np);
        std::vector<int> hj(np), hs(np), hact(np);
        cudaMemcpyAsync(hv.data(), V.p, sizeof(double) * hv.size(), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hw.data(), W.p, sizeof(double) * hw.size(), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hn.data(), npart.p, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(ha.data(), alpha.p, sizeof(double) * ha.size(), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hb.data(), beta.p, sizeof(double) * hb.size(), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(ht.data(), theta.p, sizeof(double) * np, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hr.data(), res_est.p, sizeof(double) * np, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hj.data(), j.p, sizeof(int) * np, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hs.data(), status.p, sizeof(int) * np, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hact.data(), action.p, sizeof(int) * np, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        std::fprintf(stderr, "[cigpu batch] %s: V %g %g W %g %g npart0 %g\n", what, hv[0], hv.size() > 1 ? hv[1] : 0.0,
                     hw[0], hw.size() > 1 ? hw[1] : 0.0, hn[0]);
        for (int q = 0; q < np; ++q)
            std::fprintf(stderr, "  p%d j %d status %d action %d alpha0 %g beta0 %g theta %g res %g\n", q, hj[q],
                         hs[q], hact[q], ha[q * kBatchSteps], hb[q * kBatchSteps], ht[q], hr[q]);
    };
    trace_state("start");
    bool tuned_now = false;
    for (Seg &g : segs) {
        bool t = false;
        const auto shape = tune_spmv(g.r1 - g.r0, g.nnz, g.lanes, rp.p + g.r0, col.p, val.p, V.p, W.p + g.r0, s, &t);
        g.lanes = shape.first;
        g.grid = shape.second;
        tuned_now = tuned_now || t;
    }
    trace_state("tuned");
    // rows of finished problems are skipped inside the step (their W is not read)
    auto spmv_all = [&](bool active_only) {
        for (const Seg &g : segs)
            spmv_f64_shape(g.r1 - g.r0, rp.p + g.r0, col.p, val.p, V.p, W.p + g.r0, g.lanes, g.grid, s,
                           active_only ? row_prob.p + g.r0 : nullptr, active_only ? status.p : nullptr);
    };
    const Seg &main_seg = *std::max_element(segs.begin(), segs.end(),
                                            [](const Seg &a, const Seg &b) { return a.nnz < b.nnz; });
    const int lanes = main_seg.lanes, sgrid = main_seg.grid;
    const unsigned dot_y = (kBatchSteps + kDotVecs - 1) / kDotVecs;

    // one Lanczos step of every problem, captured once
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    CIGPU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    spmv_all(true);
    k_batch_dots<<<dim3(C, dot_y), kRowThreads, 0, s>>>(B);
    k_batch_reduce<<<P, 64, 0, s>>>(B, h1.p);
    k_batch_update<<<C, kRowThreads, 0, s>>>(B, h1.p);
    k_batch_dots<<<dim3(C, dot_y), kRowThreads, 0, s>>>(B);
    k_batch_reduce<<<P, 64, 0, s>>>(B, h2.p);
    k_batch_update<<<C, kRowThreads, 0, s>>>(B, h2.p);
    k_batch_analyse<<<(P + 7) / 8, 256, 0, s>>>(B);
    k_batch_advance<<<C, kRowThreads, 0, s>>>(B);
    k_batch_finish<<<1, 1024, 0, s>>>(B);
    const cudaError_t cap = cudaStreamEndCapture(s, &graph);
    CIGPU_CUDA(cap);
    CIGPU_CUDA(cudaGetLastError());
    const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
    if (inst != cudaSuccess) {
        cudaGraphDestroy(graph);
        CIGPU_CUDA(inst);
    }
    int max_steps = 0;
    for (int p = 0; p < P; ++p) max_steps = std::max(max_steps, budget[p]);
    int steps = 0, launches = 0;
    int h_active = P;
    try {
        while (steps < max_steps + 1) {
            for (int k = 0; k < 8; ++k) {
                CIGPU_CUDA(cudaGraphLaunch(exec, s));
                count_launch(9 + (int)segs.size());
                ++launches;
                if (trace && launches <= 2) trace_state("after step");
            }
            steps += 8;
            CIGPU_CUDA(cudaMemcpyAsync(&h_active, n_active.p, sizeof(int), cudaMemcpyDeviceToHost, s));
            CIGPU_CUDA(cudaStreamSynchronize(s));
            if (h_active == 0) break;
        }
    } catch (...) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);

    // exact Rayleigh quotient and residual of every Ritz vector
    spmv_all(false);
    k_batch_rq_parts<<<C, kRowThreads, 0, s>>>(B);
    k_batch_rq<<<(P + 255) / 256, 256, 0, s>>>(B, E.p, vv.p);
    k_batch_res_parts<<<C, kRowThreads, 0, s>>>(B, E.p, vv.p);
    k_batch_res<<<(P + 255) / 256, 256, 0, s>>>(B, res.p);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(5);
    std::vector<double> hE(P), hres(P);
    std::vector<int> hmv(P), hrs(P), hst(P);
    CIGPU_CUDA(cudaMemcpyAsync(hE.data(), E.p, sizeof(double) * P, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaMemcpyAsync(hres.data(), res.p, sizeof(double) * P, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaMemcpyAsync(hmv.data(), mv.p, sizeof(int) * P, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaMemcpyAsync(hrs.data(), restarts.p, sizeof(int) * P, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaMemcpyAsync(hst.data(), status.p, sizeof(int) * P, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaStreamSynchronize(s));
    for (int p = 0; p < P; ++p) {
        Item &it = *items[p];
        const double ec = it.ham->econst;
        if (e0) e0[it.idx] = hE[p] + ec;
        if (info) {
            cigpu_solve_info &in = info[it.idx];
            std::memset(&in, 0, sizeof(in));
            in.e0 = hE[p] + ec;
            in.residual = hres[p];
            in.error_bound = hres[p];
            in.matvecs_fp64 = hmv[p] + 1;
            in.restarts = hrs[p];
            in.converged = hres[p] <= tol;
            in.precision = CIGPU_FP64;
        }
        it.status = hres[p] <= tol ? CIGPU_OK : CIGPU_ENOCONV;
    }
    if (st) {
        st->batched += P;
        st->lanes = lanes;
        st->grid = sgrid;
        st->steps = std::max(st->steps, steps);
        st->graph_launches += launches;
        st->tuned += tuned_now ? 1 : 0;
    }
}

}  // namespace
}  // namespace cigpu

using namespace cigpu;

extern "C" int cigpu_solve_batch(int count, const cigpu_request *req, int64_t max_batched_dim, double *e0,
                                 cigpu_solve_info *info, int *status, cigpu_batch_stats *stats) {
    if (count < 0 || (count > 0 && !req)) return CIGPU_EINVAL;
    if (max_batched_dim == 0) max_batched_dim = kDefaultMaxBatchedDim;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    const auto t0 = std::chrono::steady_clock::now();
    try {
        std::vector<Item> items(count);
        for (int i = 0; i < count; ++i) {
            const cigpu_request &q = req[i];
            if (!(q.tol > 0) || (q.method != CIGPU_FCI && q.method != CIGPU_DOCI) ||
                (q.precision != CIGPU_FP64 && q.precision != CIGPU_MIXED))
                return CIGPU_EINVAL;
            if (q.method == CIGPU_DOCI && q.nup != q.ndown) return CIGPU_EINVAL;
            if (q.L < 1 || q.L > kMaxL || q.nup < 0 || q.ndown < 0 || q.nup > q.L || q.ndown > q.L) return CIGPU_EINVAL;
            if (q.rot && (q.L < 1 || q.L > kMaxL || validate_rotation(q.L, q.rot) != CIGPU_OK)) return CIGPU_EINVAL;
            items[i].idx = i;
        }
        std::vector<int> small_idx, big_idx;
        for (int i = 0; i < count; ++i) {
            const cigpu_request &q = req[i];
            items[i].dim = space_dim(q.method, q.L, q.nup, q.ndown);
            (items[i].dim <= max_batched_dim ? small_idx : big_idx).push_back(i);
        }
        int hw = (int)std::thread::hardware_concurrency();
        const int nthreads = std::max(1, std::min({8, hw > 0 ? hw : 4, (int)small_idx.size()}));
        // problems above the limit: the largest first, on kBigWorkers streams
        std::stable_sort(big_idx.begin(), big_idx.end(), [&](int a, int b) { return items[a].dim > items[b].dim; });
        const int nbig = std::max(1, std::min(kBigWorkers, (int)big_idx.size()));
        int device = 0;
        CIGPU_CUDA(cudaGetDevice(&device));
        // streams live until the call returns: the built matrices keep them
        std::vector<cudaStream_t> wstreams(nthreads + nbig, nullptr);
        struct StreamsGuard {
            std::vector<cudaStream_t> &v;
            ~StreamsGuard() {
                for (cudaStream_t w : v)
                    if (w) {
                        cudaStreamSynchronize(w);
                        cudaStreamDestroy(w);
                    }
            }
        } wguard{wstreams};
        for (auto &w : wstreams) CIGPU_CUDA(cudaStreamCreateWithFlags(&w, cudaStreamNonBlocking));
        std::vector<int> failed(nthreads + nbig, CIGPU_OK);
        // Problems above the limit, in their requested precision: each worker thread
        // takes the largest one left and solves it on its own stream, so the
        // host-side parts (tables, the projected eigenproblems, the per-iteration
        // reads) of one overlap the matvecs of another, and the batched problems
        // (latency-bound) overlap them all.
        std::atomic<size_t> next_big{0};
        auto big_worker = [&](int wk) {
            cudaSetDevice(device);
            cudaStream_t s = wstreams[nthreads + wk];
            StreamScope scope(s);
            for (size_t nb = next_big.fetch_add(1); nb < big_idx.size(); nb = next_big.fetch_add(1)) {
                const int i = big_idx[nb];
                Item &it = items[i];
                const cigpu_request &q = req[i];
                int stc = cigpu_ham_create(q.L, q.nup, q.ndown, q.econst, q.h, q.eri, &it.ham);
                if (stc == CIGPU_OK && q.rot) {  // orbital rotation on the device
                    cigpu_ham *rotated = nullptr;
                    stc = cigpu_ham_rotate(it.ham, q.rot, s, &rotated);
                    cigpu_ham_destroy(it.ham);
                    it.ham = rotated;
                }
                // concurrent workers: the sigma FP32 product on any grid (as the server)
                if (stc == CIGPU_OK) stc = build_handle(it.ham, q.method, q.precision, s, true, &it.crs, true);
                if (stc == CIGPU_OK) {
                    cigpu_solve_info in{};
                    stc = cigpu_solve(it.crs, q.tol, 0, q.c0, nullptr, &in);
                    if (e0) e0[i] = in.e0;
                    if (info) info[i] = in;
                }
                if (it.crs) cigpu_crs_destroy(it.crs);
                it.crs = nullptr;
                if (it.ham) cigpu_ham_destroy(it.ham);
                it.ham = nullptr;
                it.status = stc;
                if (stc != CIGPU_OK && stc != CIGPU_ENOCONV && failed[nthreads + wk] == CIGPU_OK)
                    failed[nthreads + wk] = stc;
            }
            cudaStreamSynchronize(s);
        };
        std::vector<std::thread> big_threads;
        struct Joiner {
            std::vector<std::thread> &t;
            ~Joiner() {
                for (auto &th : t)
                    if (th.joinable()) th.join();
            }
        } big_join{big_threads};
        for (int wk = 0; wk < nbig && !big_idx.empty(); ++wk) big_threads.emplace_back(big_worker, wk);
        // build the batched problems on worker streams
        auto worker = [&](int t) {
            cudaSetDevice(device);
            cudaStream_t s = wstreams[t];
            StreamScope scope(s);
            for (size_t k = t; k < small_idx.size(); k += nthreads) {
                const int i = small_idx[k];
                Item &it = items[i];
                const cigpu_request &q = req[i];
                int stc = cigpu_ham_create(q.L, q.nup, q.ndown, q.econst, q.h, q.eri, &it.ham);
                if (stc == CIGPU_OK && q.rot) {  // orbital rotation on the device
                    cigpu_ham *rotated = nullptr;
                    stc = cigpu_ham_rotate(it.ham, q.rot, s, &rotated);
                    cigpu_ham_destroy(it.ham);
                    it.ham = rotated;
                }
                if (stc == CIGPU_OK) stc = build_handle(it.ham, q.method, CIGPU_FP64, s, false, &it.crs);
                it.status = stc;
                if (stc != CIGPU_OK && failed[t] == CIGPU_OK) failed[t] = stc;
            }
            cudaStreamSynchronize(s);
        };
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads && !small_idx.empty(); ++t) pool.emplace_back(worker, t);
        for (auto &th : pool) th.join();
        int first_err = CIGPU_OK;
        for (int t = 0; t < nthreads; ++t)
            if (failed[t] != CIGPU_OK && first_err == CIGPU_OK) first_err = failed[t];
        const double t_build = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        // batched problems, in batches of at most kMaxBatchRows rows (one tolerance per batch)
        cudaStream_t s = nullptr;
        CIGPU_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        std::unique_ptr<std::remove_pointer_t<cudaStream_t>, decltype(&cudaStreamDestroy)> sguard(s, cudaStreamDestroy);
        StreamScope scope(s);
        std::map<double, std::vector<Item *>> by_tol;
        // only the batched problems: the large-problem thread owns its items until joined
        for (int i : small_idx)
            if (items[i].crs && items[i].status == CIGPU_OK) by_tol[req[i].tol].push_back(&items[i]);
        for (auto &kv : by_tol) {
            std::vector<Item *> cur;
            int64_t rows = 0;
            for (size_t k = 0; k <= kv.second.size(); ++k) {
                if (k == kv.second.size() || rows + kv.second[k]->dim > kMaxBatchRows) {
                    solve_lockstep(cur, kv.first, s, e0, info, stats);
                    cur.clear();
                    rows = 0;
                }
                if (k < kv.second.size()) {
                    cur.push_back(kv.second[k]);
                    rows += kv.second[k]->dim;
                }
            }
        }
        for (auto &th : big_threads) th.join();
        for (int f : failed)
            if (f != CIGPU_OK && first_err == CIGPU_OK) first_err = f;
        for (auto &it : items) {
            if (it.crs) cigpu_crs_destroy(it.crs);
            if (it.ham) cigpu_ham_destroy(it.ham);
            if (status) status[it.idx] = it.status;
            if (stats && it.dim > max_batched_dim) ++stats->individual;
        }
        if (stats) {
            stats->seconds_build = t_build;
            stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        return first_err;
    } catch (...) {
        return status_from_exception();
    }
}
