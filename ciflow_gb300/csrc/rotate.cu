// Orbital rotation of a Hamiltonian on the device (cigpu_ham_rotate) and the
// unitary exp(X) of an antisymmetric generator (cigpu_unitary_exp).
//
// Replaces OrbitalTransform::fillHamCI and the one-body rotate_old_to_new
// (OrbitalTransform.cpp:64-135, 139-170): with a unitary U (row-major,
// U[a * L + p]) the rotated integrals are
//     h'_ab = sum_pq U_ap U_bq h_pq,    (ab|cd)' = sum_pqrs U_ap U_bq U_cr U_ds (pq|rs),
// the reference's four dgemm quarter-transforms with its unitary block as U. Here
// each quarter is one kernel over the L^4 tensor (a thread per output element, U
// in shared memory, one FP64 sum of L terms per element: 4 L^5 DFMA in all, 0.1 ms
// at L = 24), followed by a kernel that makes the result exactly 8-fold symmetric
// (every permutation takes the value of its canonical representative, the rule of
// cigpu_ham_create) and writes the FP32 hi/lo split the mixed build reads. The
// rotated integrals are also copied back to the host, where the string tables are
// built. exp(X) follows UnitaryMatrix::updateUnitary (UnitaryMatrix.cpp:229-290) in
// what it computes; here by scaling and squaring of a Taylor series.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "crs.cuh"

namespace cigpu {

namespace {

constexpr int kRotThreads = 256;

// out = in with tensor index `pos` (0 = slowest) rotated by U
__global__ void __launch_bounds__(kRotThreads) k_rotate_index(int L, int pos, const double *__restrict__ U,
                                                              const double *__restrict__ in, double *__restrict__ out) {
    extern __shared__ double u[];
    const int L2 = L * L;
    for (int i = threadIdx.x; i < L2; i += blockDim.x) u[i] = U[i];
    __syncthreads();
    int64_t stride = 1;
    for (int k = 3; k > pos; --k) stride *= L;
    const int64_t total = (int64_t)L2 * L2;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)((idx / stride) % L);
        const int64_t base = idx - (int64_t)a * stride;
        double s = 0;
        for (int p = 0; p < L; ++p) s = fma(u[a * L + p], in[base + (int64_t)p * stride], s);
        out[idx] = s;
    }
}

// h' = U h U^T, upper triangle computed and mirrored (exactly symmetric)
__global__ void k_rotate_h(int L, const double *__restrict__ U, const double *__restrict__ h, double *__restrict__ out) {
    const int L2 = L * L;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < L2; idx += gridDim.x * blockDim.x) {
        const int a = idx / L, b = idx - a * L;
        if (a > b) continue;
        double s = 0;
        for (int p = 0; p < L; ++p) {
            double t = 0;
            for (int q = 0; q < L; ++q) t = fma(h[p * L + q], U[b * L + q], t);
            s = fma(U[a * L + p], t, s);
        }
        out[a * L + b] = s;
        out[b * L + a] = s;
    }
}

// exact 8-fold symmetry (canonical representative p>=q, r>=s, pq>=rs) and the FP32 split
__global__ void k_canonical(int L, const double *__restrict__ in, double *__restrict__ eri, float *__restrict__ hi,
                            float *__restrict__ lo) {
    const int64_t L1 = L, L2 = L1 * L1, L3 = L2 * L1, total = L2 * L2;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(idx / L3), q = (int)((idx / L2) % L1), r = (int)((idx / L1) % L1), s = (int)(idx % L1);
        int a = max(p, q), b = min(p, q), c = max(r, s), d = min(r, s);
        if (a * L + b < c * L + d) {
            int t = a;
            a = c;
            c = t;
            t = b;
            b = d;
            d = t;
        }
        const double v = in[a * L3 + b * L2 + c * L1 + d];
        eri[idx] = v;
        split_fp32(v, hi[idx], lo[idx]);
    }
}

int rot_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(sm_count() * 8, (n + kRotThreads - 1) / kRotThreads)); }

}  // namespace

void rotate_ham(const cigpu_ham &base, const double *U, cigpu_ham &H, cudaStream_t s) {
    const int L = base.L;
    const size_t L1 = L, L2 = L1 * L1, L4 = L2 * L2;
    H.L = L;
    H.nup = base.nup;
    H.ndown = base.ndown;
    H.econst = base.econst;
    DevBuf<double> dU(L2), t1(L4), t2(L4);
    CIGPU_CUDA(cudaMemcpyAsync(dU.p, U, L2 * sizeof(double), cudaMemcpyHostToDevice, s));
    const size_t sm = L2 * sizeof(double);
    const int g = rot_grid((int64_t)L4);
    k_rotate_index<<<g, kRotThreads, sm, s>>>(L, 0, dU.p, base.d_eri.p, t1.p);
    k_rotate_index<<<g, kRotThreads, sm, s>>>(L, 1, dU.p, t1.p, t2.p);
    k_rotate_index<<<g, kRotThreads, sm, s>>>(L, 2, dU.p, t2.p, t1.p);
    k_rotate_index<<<g, kRotThreads, sm, s>>>(L, 3, dU.p, t1.p, t2.p);
    H.d_eri.alloc(L4);
    H.d_eri_hi.alloc(L4);
    H.d_eri_lo.alloc(L4);
    H.d_h.alloc(L2);
    k_canonical<<<g, kRotThreads, 0, s>>>(L, t2.p, H.d_eri.p, H.d_eri_hi.p, H.d_eri_lo.p);
    k_rotate_h<<<rot_grid((int64_t)L2), kRotThreads, 0, s>>>(L, dU.p, base.d_h.p, H.d_h.p);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(6);
    H.h.resize(L2);
    H.eri.resize(L4);
    CIGPU_CUDA(cudaMemcpyAsync(H.h.data(), H.d_h.p, L2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaMemcpyAsync(H.eri.data(), H.d_eri.p, L4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaStreamSynchronize(s));
}

// exp(X) for antisymmetric X (row-major): scaling by 2^-s so that |X|_1 2^-s <= 1/2,
// Taylor series to order 16 (remainder below 1e-19), then s squarings.
void unitary_exp(int L, const double *X, double *U) {
    const size_t n = L, N = n * n;
    double norm1 = 0;
    for (size_t j = 0; j < n; ++j) {
        double c = 0;
        for (size_t i = 0; i < n; ++i) c += std::fabs(X[i * n + j]);
        norm1 = std::max(norm1, c);
    }
    int sq = 0;
    while (norm1 > 0.5 && sq < 60) {
        norm1 *= 0.5;
        ++sq;
    }
    const double scale = std::ldexp(1.0, -sq);
    std::vector<double> Y(N), term(N), next(N), E(N, 0.0);
    for (size_t i = 0; i < N; ++i) Y[i] = X[i] * scale;
    for (size_t i = 0; i < n; ++i) E[i * n + i] = 1.0;
    term = E;
    for (int k = 1; k <= 16; ++k) {
        std::fill(next.begin(), next.end(), 0.0);
        for (size_t i = 0; i < n; ++i)
            for (size_t m = 0; m < n; ++m) {
                const double t = term[i * n + m];
                if (t == 0) continue;
                for (size_t j = 0; j < n; ++j) next[i * n + j] += t * Y[m * n + j];
            }
        for (size_t i = 0; i < N; ++i) {
            term[i] = next[i] / k;
            E[i] += term[i];
        }
    }
    for (int k = 0; k < sq; ++k) {
        std::fill(next.begin(), next.end(), 0.0);
        for (size_t i = 0; i < n; ++i)
            for (size_t m = 0; m < n; ++m) {
                const double t = E[i * n + m];
                for (size_t j = 0; j < n; ++j) next[i * n + j] += t * E[m * n + j];
            }
        E.swap(next);
    }
    std::memcpy(U, E.data(), N * sizeof(double));
}

int validate_rotation(int L, const double *U) {
    for (int i = 0; i < L * L; ++i)
        if (!std::isfinite(U[i])) return CIGPU_EINVAL;
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j) {
            double s = 0;
            for (int k = 0; k < L; ++k) s += U[i * L + k] * U[j * L + k];
            if (std::fabs(s - (i == j ? 1.0 : 0.0)) > 1e-10) return CIGPU_EINVAL;
        }
    return CIGPU_OK;
}

}  // namespace cigpu

using namespace cigpu;

extern "C" {

int cigpu_unitary_exp(int L, const double *X, double *U) {
    if (L < 1 || L > kMaxL || !X || !U) return CIGPU_EINVAL;
    double mx = 0;
    for (int i = 0; i < L * L; ++i) {
        if (!std::isfinite(X[i])) return CIGPU_EINVAL;
        mx = std::max(mx, std::fabs(X[i]));
    }
    for (int i = 0; i < L; ++i)
        for (int j = 0; j <= i; ++j)
            if (std::fabs(X[i * L + j] + X[j * L + i]) > 1e-12 * std::max(1.0, mx)) return CIGPU_EINVAL;
    unitary_exp(L, X, U);
    return CIGPU_OK;
}

int cigpu_ham_export(const cigpu_ham *ham, double *h, double *eri) {
    if (!ham) return CIGPU_EINVAL;
    if (!ham->host_valid) {
        // device-only Hamiltonian: its producer synchronised its stream, so plain copies are ordered
        try {
            const size_t L2 = (size_t)ham->L * ham->L;
            if (h) CIGPU_CUDA(cudaMemcpy(h, ham->d_h.p, sizeof(double) * L2, cudaMemcpyDeviceToHost));
            if (eri) CIGPU_CUDA(cudaMemcpy(eri, ham->d_eri.p, sizeof(double) * L2 * L2, cudaMemcpyDeviceToHost));
            return CIGPU_OK;
        } catch (...) {
            return status_from_exception();
        }
    }
    if (h) std::memcpy(h, ham->h.data(), sizeof(double) * ham->h.size());
    if (eri) std::memcpy(eri, ham->eri.data(), sizeof(double) * ham->eri.size());
    return CIGPU_OK;
}

int cigpu_ham_rotate(const cigpu_ham *base, const double *U, cigpu_stream stream, cigpu_ham **out) {
    if (!base || !U || !out) return CIGPU_EINVAL;
    *out = nullptr;
    if (base->L > kMaxL) return CIGPU_ENOTSUP;  // U is staged in shared memory
    if (validate_rotation(base->L, U) != CIGPU_OK) return CIGPU_EINVAL;  // orthogonal to 1e-10
    try {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        bool own = false;
        if (!s) {
            CIGPU_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            own = true;
        }
        std::unique_ptr<std::remove_pointer_t<cudaStream_t>, decltype(&cudaStreamDestroy)> sg(own ? s : nullptr,
                                                                                             cudaStreamDestroy);
        std::unique_ptr<cigpu_ham> H(new cigpu_ham);
        {
            StreamScope scope(s);
            rotate_ham(*base, U, *H, s);
        }
        *out = H.release();
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

}  // extern "C"
