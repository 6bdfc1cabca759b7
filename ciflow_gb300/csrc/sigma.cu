// FP32 product of the mixed method for FCI: a direct-CI sigma vector from a
// factorised two-electron part.
//
// With E_pq = sum over spins of a+_p a_q and real orbitals,
//   H = sum_pq k_pq E_pq + 1/2 sum_pqrs (pq|rs) E_pq E_rs,   k_ps = h_ps - 1/2 sum_q (pq|qs),
// and a factorisation (pq|rs) = sum_k s_k F^k_pq F^k_rs with symmetric F^k (a
// pivoted Cholesky factor of the pair matrix, s_k = 1; eigenpairs with their signs
// when the integrals are indefinite) gives
//   1/2 sum (pq|rs) E_pq E_rs = 1/2 sum_k s_k A_k A_k,   A_k = sum_pq F^k_pq E_pq.
// So y = H x is two one-body passes:
//   (1) y_k = A_k x for every factor k, and K x;
//   (2) y = K x + sum_k A_k (1/2 s_k y_k).
// A one-body pass visits, for every determinant I = (Ia, Ib), its single
// excitations (Ia -> Ja with Ib fixed, Ib -> Jb with Ia fixed; sign and orbital
// pair from the string tables) and its diagonal (occupations). Against the stored
// matrix (about 1,800 elements per row at L=12 6a6b, 4 bytes each) a determinant
// costs n_a (L - n_a) + n_b (L - n_b) excitations times the rank, and the data it
// reads (x, the A_k x vectors) stay in L2.
//
// This replaces only the mixed method's FP32 correction products: the operator
// equals the reference Hamiltonian up to FP32 rounding and the factorisation's
// truncation (a remaining pair diagonal below 1e-10 of the largest), while the FP64 anchor
// products and residuals keep using the stored matrix, whose elements are the
// reference's bit for bit; the residual the solver reports is that exact one.
//
// Both passes run on tiles of 32 alpha x 32 beta strings (8 warps in the first
// pass, 16 in the second). In the alpha
// phase warp w takes alpha rows of the tile with its lanes on consecutive beta
// strings: every lane of the warp walks the same alpha excitations (uniform
// coefficients, broadcast from shared memory) and reads x at consecutive beta
// strings (coalesced). In the beta phase the warp takes beta columns with its
// lanes on consecutive alpha strings and reads the transposed vectors. The two
// phases meet in a shared-memory tile; the A_k x vectors are written in both
// string orders, in blocks of 32 strings with the factors in groups of four
// outside the 32 ([Da][Db/32][R/4][32][4] and [Db][Da/32][R/4][32][4]): in the
// second pass a lane reads four factors of its determinant with one 16-byte load
// and the warp's load covers 512 contiguous bytes, so one excitation is R/4 loads
// and its factors one contiguous block. (Measured at L=11: factors innermost per
// determinant, each 16-byte load of a warp spread over 16 cache lines, 156 us;
// one factor of 32 strings per 4-byte load, 66 us.) The tile's excitation lists
// (target, orbital pair, sign) are staged in shared memory.
#include <algorithm>
#include <cmath>
#include <vector>

#include "checked.cuh"
#include "sigma.cuh"
#include "small_eigh.h"

namespace cigpu {

namespace {

constexpr int kTile = 32;
constexpr int kThreads = 256;   // pass 1: 8 warps, 4 rows (columns) of the tile each
constexpr int kWarps = kThreads / 32;
constexpr int kThreadsB = 512;  // pass 2: 16 warps, 2 rows (columns) each
constexpr int kWarpsB = kThreadsB / 32;
constexpr int kYtRow = kSigmaChunk * (kTile + 1) + 1;  // staging tile row (odd: the column phase is conflict-free)

struct SigmaArgs {
    int L, R, nsa, nsb;
    int64_t Da, Db;
    int64_t nTa, nTb;  // 32-string tiles of each spin (the factor blocks of Ya, Yb)
    const uint32_t *sa_t, *sa_i, *sb_t, *sb_i;  // single excitations: targets and packed info per string
    unsigned long long *err;                    // checked build: the error word
};

// The single excitations of the tile's 32 strings s0.. in shared memory, as
// {target J, (lo * L + hi) << 1 | negative}: the orbital pair of E_pq and the sign
// of <S|E_pq|J> (odd number of electrons between the two orbitals). Strings past
// the space get {0, 0}.
// (The checked build tests each target against the string count and stages a
// failing one as {0, 0}.)
__device__ __forceinline__ void stage_excitations(const uint32_t *__restrict__ tgt, const uint32_t *__restrict__ info,
                                                  int64_t s0, int64_t D, int ns, int L, uint2 *dst,
                                                  unsigned long long *err) {
    for (int i = threadIdx.x; i < kTile * ns; i += blockDim.x) {
        const int r = i / ns;
        const int64_t S = s0 + r;
        uint2 v = make_uint2(0u, 0u);
        if (S < D) {
            const int64_t at = S * ns + (i - r * ns);
            const uint32_t inf = __ldg(info + at);
            v.x = __ldg(tgt + at);
            v.y = (((inf & 63u) * (uint32_t)L + ((inf >> 6) & 63u)) << 1) | ((inf >> 24) & 1u);
            if (!CIGPU_CHECK(err, index_ok(v.x, (uint64_t)D), kCheckColumn, v.x)) v = make_uint2(0u, 0u);
        }
        dst[i] = v;
    }
    (void)err;
}
__device__ __forceinline__ float exc_sign(uint32_t packed) { return (packed & 1u) ? -1.f : 1.f; }
__device__ __forceinline__ float dot4(const float4 a, const float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }

__global__ void k_transpose32(const float *__restrict__ a, int64_t rows, int64_t cols, float *__restrict__ t) {
    __shared__ float tile[kTile][kTile + 1];
    const int64_t r0 = (int64_t)blockIdx.y * kTile, c0 = (int64_t)blockIdx.x * kTile;
    for (int i = threadIdx.y; i < kTile; i += blockDim.y) {
        const int64_t r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[i][threadIdx.x] = a[r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < kTile; i += blockDim.y) {
        const int64_t c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) t[c * rows + r] = tile[threadIdx.x][i];
    }
}

// Pass 1: (A_k x)(Ia, Ib) into Ya at (((Ia * nTb + Ib / 32) * R / 4 + k / 4) * 32 + Ib % 32) * 4 + k % 4
// and into Yb with the spins exchanged, and kx = K x.
// Per-string diagonal sums fa, fb are factor-major ([R][D]).
__global__ void __launch_bounds__(kThreads, 2)  // shared memory holds it to two blocks per SM
    k_sigma_a(const SigmaArgs a, const float *__restrict__ F, const float *__restrict__ K1,
              const float *__restrict__ fa, const float *__restrict__ fb, const float *__restrict__ ka,
              const float *__restrict__ kb, const float *__restrict__ x, const float *__restrict__ xT,
              float *__restrict__ Ya, float *__restrict__ Yb, float *__restrict__ kx) {
    extern __shared__ __align__(16) float sm[];
    const int L2 = a.L * a.L, R = a.R;
    float *Fs = sm;                                                 // [L2][R]
    float *Ks = Fs + (size_t)L2 * R;                                // [L2] (padded to 4)
    uint2 *ea = reinterpret_cast<uint2 *>(Ks + ((L2 + 3) & ~3));    // [kTile][nsa]
    uint2 *eb = ea + kTile * a.nsa;                                 // [kTile][nsb]
    float *yt = reinterpret_cast<float *>(eb + kTile * a.nsb);      // [kTile][kYtRow]
    float *kt = yt + kTile * kYtRow;                                // [kTile][kTile + 1]
    for (int i = threadIdx.x; i < L2 * R; i += kThreads) Fs[i] = F[i];
    for (int i = threadIdx.x; i < L2; i += kThreads) Ks[i] = K1[i];
    const int64_t ta = (int64_t)blockIdx.y * kTile, tb = (int64_t)blockIdx.x * kTile;
    stage_excitations(a.sa_t, a.sa_i, ta, a.Da, a.nsa, a.L, ea, a.err);
    stage_excitations(a.sb_t, a.sb_i, tb, a.Db, a.nsb, a.L, eb, a.err);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = 0; c < R; c += kSigmaChunk) {
        __syncthreads();  // tables staged / the previous chunk's tile written out
        // alpha phase: warp rows r, lanes on beta strings
        for (int r = warp; r < kTile; r += kWarps) {
            const int64_t Ia = ta + r, Ib = tb + lane;
            const bool ok = Ia < a.Da && Ib < a.Db;
            float acc[kSigmaChunk], kacc = 0.f;
#pragma unroll
            for (int k = 0; k < kSigmaChunk; ++k) acc[k] = 0.f;
            if (ok) {
                const float xi = x[Ia * a.Db + Ib];
#pragma unroll
                for (int k = 0; k < kSigmaChunk; ++k)
                    acc[k] = xi * (fa[(int64_t)(c + k) * a.Da + Ia] + fb[(int64_t)(c + k) * a.Db + Ib]);
                if (c == 0) kacc = xi * (ka[Ia] + kb[Ib]);
                const uint2 *ex = ea + r * a.nsa;
                for (int e = 0; e < a.nsa; ++e) {
                    const uint2 v = ex[e];
                    const float xv = exc_sign(v.y) * x[(int64_t)v.x * a.Db + Ib];
                    const float4 *f4 = reinterpret_cast<const float4 *>(Fs + (size_t)(v.y >> 1) * R + c);
#pragma unroll
                    for (int q = 0; q < kSigmaChunk / 4; ++q) {
                        const float4 f = f4[q];
                        acc[4 * q] += f.x * xv;
                        acc[4 * q + 1] += f.y * xv;
                        acc[4 * q + 2] += f.z * xv;
                        acc[4 * q + 3] += f.w * xv;
                    }
                    if (c == 0) kacc += Ks[v.y >> 1] * xv;
                }
            }
#pragma unroll
            for (int k = 0; k < kSigmaChunk; ++k) yt[r * kYtRow + k * (kTile + 1) + lane] = acc[k];
            if (c == 0) kt[r * (kTile + 1) + lane] = kacc;
        }
        __syncthreads();
        // beta phase: warp columns cl, lanes on alpha strings
        for (int cl = warp; cl < kTile; cl += kWarps) {
            const int64_t Ib = tb + cl, Ia = ta + lane;
            const bool ok = Ib < a.Db && Ia < a.Da;
            float acc[kSigmaChunk], kacc = 0.f;
#pragma unroll
            for (int k = 0; k < kSigmaChunk; ++k) acc[k] = 0.f;
            if (ok) {
                const uint2 *ex = eb + cl * a.nsb;
                for (int e = 0; e < a.nsb; ++e) {
                    const uint2 v = ex[e];
                    const float xv = exc_sign(v.y) * xT[(int64_t)v.x * a.Da + Ia];
                    const float4 *f4 = reinterpret_cast<const float4 *>(Fs + (size_t)(v.y >> 1) * R + c);
#pragma unroll
                    for (int q = 0; q < kSigmaChunk / 4; ++q) {
                        const float4 f = f4[q];
                        acc[4 * q] += f.x * xv;
                        acc[4 * q + 1] += f.y * xv;
                        acc[4 * q + 2] += f.z * xv;
                        acc[4 * q + 3] += f.w * xv;
                    }
                    if (c == 0) kacc += Ks[v.y >> 1] * xv;
                }
            }
#pragma unroll
            for (int k = 0; k < kSigmaChunk; ++k) yt[lane * kYtRow + k * (kTile + 1) + cl] += acc[k];
            if (c == 0) kt[lane * (kTile + 1) + cl] += kacc;
        }
        __syncthreads();
        // write out both orders: per string of the tile, this chunk's four groups of
        // four factors for 32 strings (512 contiguous bytes per warp store)
        for (int row = warp; row < kTile * (kSigmaChunk / 4); row += kWarps) {
            const int r = row / (kSigmaChunk / 4), q = row - r * (kSigmaChunk / 4);
            const int g = c / 4 + q;  // factor group
            {
                const int64_t Ia = ta + r, Ib = tb + lane;
                if (Ia < a.Da && Ib < a.Db) {
                    const float *src = yt + r * kYtRow + 4 * q * (kTile + 1) + lane;
                    reinterpret_cast<float4 *>(Ya)[((Ia * a.nTb + blockIdx.x) * (R / 4) + g) * kTile + lane] =
                        make_float4(src[0], src[kTile + 1], src[2 * (kTile + 1)], src[3 * (kTile + 1)]);
                }
            }
            {
                const int64_t Ib = tb + r, Ia = ta + lane;  // r is a beta column here
                if (Ia < a.Da && Ib < a.Db) {
                    const float *src = yt + lane * kYtRow + 4 * q * (kTile + 1) + r;
                    reinterpret_cast<float4 *>(Yb)[((Ib * a.nTa + blockIdx.y) * (R / 4) + g) * kTile + lane] =
                        make_float4(src[0], src[kTile + 1], src[2 * (kTile + 1)], src[3 * (kTile + 1)]);
                }
            }
        }
        if (c == 0)
            for (int r = warp; r < kTile; r += kWarps) {
                const int64_t Ia = ta + r, Ib = tb + lane;
                if (Ia < a.Da && Ib < a.Db) kx[Ia * a.Db + Ib] = kt[r * (kTile + 1) + lane];
            }
    }
}

// sum_k G^k_pq y_k(J): g the factor row pq (shared memory), yj this lane's first
// group of four factors in string J's block (group q at yj[32 q]).
__device__ __forceinline__ float excitation_term(const float4 *__restrict__ g, const float4 *__restrict__ yj, int R4) {
    float t = 0.f;
#pragma unroll 4
    for (int q = 0; q < R4; ++q) t += dot4(g[q], yj[q * kTile]);
    return t;
}

// Pass 2: y = K x + sum_k A_k (1/2 s_k y_k), the scaled factors G = 1/2 s_k F^k;
// ga, gb factor-major ([R][D]).
__global__ void __launch_bounds__(kThreadsB, 2)
    k_sigma_b(const SigmaArgs a, const float *__restrict__ G, const float *__restrict__ ga,
              const float *__restrict__ gb, const float *__restrict__ Ya, const float *__restrict__ Yb,
              const float *__restrict__ kx, float *__restrict__ y) {
    extern __shared__ __align__(16) float sm[];
    const int L2 = a.L * a.L, R = a.R, R4 = R / 4;
    float *Gs = sm;                                              // [L2][R]
    uint2 *ea = reinterpret_cast<uint2 *>(Gs + (size_t)L2 * R);  // [kTile][nsa]
    uint2 *eb = ea + kTile * a.nsa;                              // [kTile][nsb]
    float *st = reinterpret_cast<float *>(eb + kTile * a.nsb);   // [kTile][kTile + 1]
    for (int i = threadIdx.x; i < L2 * R; i += kThreadsB) Gs[i] = G[i];
    const int64_t ta = (int64_t)blockIdx.y * kTile, tb = (int64_t)blockIdx.x * kTile;
    stage_excitations(a.sa_t, a.sa_i, ta, a.Da, a.nsa, a.L, ea, a.err);
    stage_excitations(a.sb_t, a.sb_i, tb, a.Db, a.nsb, a.L, eb, a.err);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float4 *G4 = reinterpret_cast<const float4 *>(Gs);
    // alpha phase with the diagonal and K x
    for (int r = warp; r < kTile; r += kWarpsB) {
        const int64_t Ia = ta + r, Ib = tb + lane;
        float acc = 0.f;
        if (Ia < a.Da && Ib < a.Db) {
            acc = kx[Ia * a.Db + Ib];
            const float4 *yi = reinterpret_cast<const float4 *>(Ya) + (Ia * a.nTb + blockIdx.x) * R4 * kTile + lane;
            for (int q = 0; q < R4; ++q) {
                const float4 v = yi[q * kTile];
                const int k = 4 * q;
                acc += v.x * (ga[(int64_t)k * a.Da + Ia] + gb[(int64_t)k * a.Db + Ib]) +
                       v.y * (ga[(int64_t)(k + 1) * a.Da + Ia] + gb[(int64_t)(k + 1) * a.Db + Ib]) +
                       v.z * (ga[(int64_t)(k + 2) * a.Da + Ia] + gb[(int64_t)(k + 2) * a.Db + Ib]) +
                       v.w * (ga[(int64_t)(k + 3) * a.Da + Ia] + gb[(int64_t)(k + 3) * a.Db + Ib]);
            }
            const uint2 *ex = ea + r * a.nsa;
            // string J's block: yb + J * js
            const float4 *yb = reinterpret_cast<const float4 *>(Ya) + (int64_t)blockIdx.x * R4 * kTile + lane;
            const int64_t js = a.nTb * R4 * kTile;
            int e = 0;
            for (; e + 1 < a.nsa; e += 2) {  // two excitations' loads in flight together
                const uint2 v0 = ex[e], v1 = ex[e + 1];
                const float t0 = excitation_term(G4 + (size_t)(v0.y >> 1) * R4, yb + v0.x * js, R4);
                const float t1 = excitation_term(G4 + (size_t)(v1.y >> 1) * R4, yb + v1.x * js, R4);
                acc += exc_sign(v0.y) * t0 + exc_sign(v1.y) * t1;
            }
            if (e < a.nsa) {
                const uint2 v0 = ex[e];
                acc += exc_sign(v0.y) * excitation_term(G4 + (size_t)(v0.y >> 1) * R4, yb + v0.x * js, R4);
            }
        }
        st[r * (kTile + 1) + lane] = acc;
    }
    __syncthreads();
    for (int cl = warp; cl < kTile; cl += kWarpsB) {
        const int64_t Ib = tb + cl, Ia = ta + lane;
        float acc = 0.f;
        if (Ib < a.Db && Ia < a.Da) {
            const uint2 *ex = eb + cl * a.nsb;
            const float4 *yb = reinterpret_cast<const float4 *>(Yb) + (int64_t)blockIdx.y * R4 * kTile + lane;
            const int64_t js = a.nTa * R4 * kTile;
            int e = 0;
            for (; e + 1 < a.nsb; e += 2) {
                const uint2 v0 = ex[e], v1 = ex[e + 1];
                const float t0 = excitation_term(G4 + (size_t)(v0.y >> 1) * R4, yb + v0.x * js, R4);
                const float t1 = excitation_term(G4 + (size_t)(v1.y >> 1) * R4, yb + v1.x * js, R4);
                acc += exc_sign(v0.y) * t0 + exc_sign(v1.y) * t1;
            }
            if (e < a.nsb) {
                const uint2 v0 = ex[e];
                acc += exc_sign(v0.y) * excitation_term(G4 + (size_t)(v0.y >> 1) * R4, yb + v0.x * js, R4);
            }
        }
        st[lane * (kTile + 1) + cl] += acc;
    }
    __syncthreads();
    for (int r = warp; r < kTile; r += kWarpsB) {
        const int64_t Ia = ta + r, Ib = tb + lane;
        if (Ia < a.Da && Ib < a.Db) y[Ia * a.Db + Ib] = st[r * (kTile + 1) + lane];
    }
}

size_t smem_a_bytes(int L, int R, int nsa, int nsb) {
    const int L2 = L * L;
    return sizeof(float) * ((size_t)L2 * R + ((L2 + 3) & ~3)) + sizeof(uint2) * (size_t)kTile * (nsa + nsb) +
           sizeof(float) * ((size_t)kTile * kYtRow + (size_t)kTile * (kTile + 1));
}
size_t smem_b_bytes(int L, int R, int nsa, int nsb) {
    return sizeof(float) * (size_t)L * L * R + sizeof(uint2) * (size_t)kTile * (nsa + nsb) +
           sizeof(float) * (size_t)kTile * (kTile + 1);
}
constexpr size_t kSigmaMaxSmem = 200 * 1024;

}  // namespace

size_t sigma_bytes(int L, int64_t Da, int64_t Db, int R) {
    const int64_t dim = Da * Db, padded = Da * ((Db + kTile - 1) / kTile) * kTile + Db * ((Da + kTile - 1) / kTile) * kTile;
    return sizeof(float) * ((size_t)padded * R + 2 * (size_t)dim + (size_t)(Da + Db) * (2 * R + 1) +
                            (size_t)L * L * (2 * R + 1));
}

bool sigma_prepare(SigmaOp &op, int L, const double *h, const double *eri, const SpinTables &ta,
                   const SpinTables &tb, bool any_grid, cudaStream_t s) {
    op.R = 0;
    if (!sigma_applies(L) || ta.D < 1 || tb.D < 1) return false;
    // a grid of fewer tiles than SMs leaves the GPU part idle: the stored FP32 slot
    // values are faster there (L=10 5a5b, 64 tiles: 0.13 against 0.07 ms)
    if (!any_grid && ((ta.D + kTile - 1) / kTile) * ((tb.D + kTile - 1) / kTile) < sm_count()) return false;
    const int L2 = L * L;
    const size_t N = (size_t)L2;
    // The factors, in the space of orbital pairs p >= q: with c = 1 on the diagonal
    // pairs and sqrt 2 off it, V[P][Q] = c_P c_Q (pq|rs) is the two-electron part in
    // the operators (E_pq + E_qp) / c_P. A pivoted incomplete Cholesky factor of V
    // (two-electron integrals are positive semidefinite as a pair matrix) stops
    // when the largest remaining diagonal falls below 1e-10 of the largest; an
    // indefinite V takes its eigenpairs instead. A factor v gives the symmetric
    // F_pq = F_qp = v_P / c_P.
    const int P = L * (L + 1) / 2;
    std::vector<int> pp(P), pq_(P);
    std::vector<double> cP(P);
    for (int p = 0, i = 0; p < L; ++p)
        for (int q = 0; q <= p; ++q, ++i) {
            pp[i] = p;
            pq_[i] = q;
            cP[i] = p == q ? 1.0 : std::sqrt(2.0);
        }
    const size_t L1 = L, L3 = N * L1;
    auto eri_at = [&](int p, int q, int r, int t) { return eri[p * L3 + q * N + r * L1 + t]; };
    std::vector<double> V((size_t)P * P);
    for (int i = 0; i < P; ++i)
        for (int j = 0; j < P; ++j) V[(size_t)i * P + j] = cP[i] * cP[j] * eri_at(pp[i], pq_[i], pp[j], pq_[j]);
    std::vector<std::vector<double>> vecs;  // factors in the pair space
    std::vector<double> sgn;
    {
        std::vector<double> d(P);
        double d0 = 0;
        for (int i = 0; i < P; ++i) d0 = std::max(d0, d[i] = V[(size_t)i * P + i]);
        bool psd = true;
        while ((int)vecs.size() < P && d0 > 0) {
            int k = 0;
            for (int i = 1; i < P; ++i)
                if (d[i] > d[k]) k = i;
            if (d[k] <= 1e-10 * d0) break;
            std::vector<double> l(P);
            for (int i = 0; i < P; ++i) {
                double v = V[(size_t)i * P + k];
                for (const auto &u : vecs) v -= u[i] * u[k];
                l[i] = v;
            }
            const double r = std::sqrt(d[k]);
            for (int i = 0; i < P; ++i) {
                l[i] /= r;
                d[i] -= l[i] * l[i];
                if (d[i] < -1e-8 * d0) psd = false;
            }
            vecs.push_back(std::move(l));
            sgn.push_back(1.0);
            if (!psd) break;
        }
        if (!psd) {  // indefinite: eigenpairs of the pair matrix
            vecs.clear();
            sgn.clear();
            std::vector<double> A = V, w, z;
            symmetric_eigh(P, A, w, z);
            double wmax = 0;
            for (double v : w) wmax = std::max(wmax, std::fabs(v));
            for (int k = 0; k < P; ++k)
                if (std::fabs(w[k]) > 1e-10 * wmax) {
                    std::vector<double> l(P);
                    const double sc = std::sqrt(std::fabs(w[k]));
                    for (int i = 0; i < P; ++i) l[i] = sc * z[(size_t)i * P + k];
                    vecs.push_back(std::move(l));
                    sgn.push_back(w[k] < 0 ? -1.0 : 1.0);
                }
        }
    }
    const int rank = (int)vecs.size();
    const int R = std::max(kSigmaChunk, (rank + kSigmaChunk - 1) / kSigmaChunk * kSigmaChunk);
    if (R > kSigmaMaxRank || smem_a_bytes(L, R, ta.ns, tb.ns) > kSigmaMaxSmem ||
        smem_b_bytes(L, R, ta.ns, tb.ns) > kSigmaMaxSmem)
        return false;
    std::vector<float> F(N * R, 0.f), G(N * R, 0.f), K1(N);
    for (int j = 0; j < rank; ++j)
        for (int i = 0; i < P; ++i) {
            const double f = vecs[j][i] / cP[i];
            const size_t a = (size_t)(pp[i] * L + pq_[i]) * R + j, b = (size_t)(pq_[i] * L + pp[i]) * R + j;
            F[a] = F[b] = (float)f;
            G[a] = G[b] = (float)(0.5 * sgn[j] * f);
        }
    for (int p = 0; p < L; ++p)
        for (int q = 0; q < L; ++q) {
            double k = h[p * L1 + q];
            for (int r = 0; r < L; ++r) k -= 0.5 * eri[p * L3 + r * N + r * L1 + q];  // (pr|rq)
            K1[(size_t)p * L + q] = (float)k;
        }
    // per-string diagonal sums over occupied orbitals, factor-major
    auto diag_sums = [&](const SpinTables &t, std::vector<float> &fs, std::vector<float> &gs, std::vector<float> &ks) {
        fs.assign((size_t)R * t.D, 0.f);
        gs.assign((size_t)R * t.D, 0.f);
        ks.assign((size_t)t.D, 0.f);
        for (int64_t S = 0; S < t.D; ++S) {
            double kk = 0;
            for (int m = 0; m < t.n; ++m) {
                const int p = t.occ[(size_t)S * t.n + m];
                kk += K1[(size_t)p * L + p];
            }
            ks[S] = (float)kk;
            for (int j = 0; j < R; ++j) {
                double f = 0, g = 0;
                for (int m = 0; m < t.n; ++m) {
                    const int p = t.occ[(size_t)S * t.n + m];
                    f += F[(size_t)(p * L + p) * R + j];
                    g += G[(size_t)(p * L + p) * R + j];
                }
                fs[(size_t)j * t.D + S] = (float)f;
                gs[(size_t)j * t.D + S] = (float)g;
            }
        }
    };
    std::vector<float> fa, ga, kav, fb, gb, kbv;
    diag_sums(ta, fa, ga, kav);
    diag_sums(tb, fb, gb, kbv);
    auto up = [&](DevBuf<float> &buf, const std::vector<float> &v) {
        buf.alloc(v.size());
        if (!v.empty()) CIGPU_CUDA(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    };
    up(op.F, F);
    up(op.G, G);
    up(op.K1, K1);
    up(op.fa, fa);
    up(op.fb, fb);
    up(op.ga, ga);
    up(op.gb, gb);
    up(op.ka, kav);
    up(op.kb, kbv);
    const int64_t dim = ta.D * tb.D;
    op.xT.alloc((size_t)dim);
    const int64_t nTa = (ta.D + kTile - 1) / kTile, nTb = (tb.D + kTile - 1) / kTile;
    op.Ya.alloc((size_t)ta.D * nTb * kTile * R);  // factor blocks of 32 strings, the last one padded
    op.Yb.alloc((size_t)tb.D * nTa * kTile * R);
    op.kx.alloc((size_t)dim);
    op.L = L;
    op.rank = rank;
    op.Da = ta.D;
    op.Db = tb.D;
    op.smem_a = smem_a_bytes(L, R, ta.ns, tb.ns);
    op.smem_b = smem_b_bytes(L, R, ta.ns, tb.ns);
    op.R = R;
    return true;
}

void sigma_mv32(SigmaOp &op, const FciParams &p, const float *x, float *y, cudaStream_t s) {
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_sigma_a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSigmaMaxSmem);
        cudaFuncSetAttribute(k_sigma_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSigmaMaxSmem);
        return true;
    }();
    (void)attr_set;
    const SigmaArgs a{op.L,
                      op.R,
                      p.a.ns,
                      p.b.ns,
                      op.Da,
                      op.Db,
                      (op.Da + kTile - 1) / kTile,
                      (op.Db + kTile - 1) / kTile,
                      p.a.s_target,
                      p.a.s_info,
                      p.b.s_target,
                      p.b.s_info,
                      check_word_device()};
    const dim3 tgrid((unsigned)((op.Db + kTile - 1) / kTile), (unsigned)((op.Da + kTile - 1) / kTile));
    k_transpose32<<<tgrid, dim3(kTile, 8), 0, s>>>(x, op.Da, op.Db, op.xT.p);
    k_sigma_a<<<tgrid, kThreads, op.smem_a, s>>>(a, op.F.p, op.K1.p, op.fa.p, op.fb.p, op.ka.p, op.kb.p, x, op.xT.p,
                                                  op.Ya.p, op.Yb.p, op.kx.p);
    k_sigma_b<<<tgrid, kThreadsB, op.smem_b, s>>>(a, op.G.p, op.ga.p, op.gb.p, op.Ya.p, op.Yb.p, op.kx.p, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(3);
}

}  // namespace cigpu
