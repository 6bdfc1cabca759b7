// Matrix-free DOCI matvec: y = H x over the seniority-zero pair space without a
// stored matrix.
//
// Replaces SparseMatrix_CRS_Sym::mvprod (SparseMatrix_CRS.cpp:700-723) on the DOCI
// matrix of DOCI::construct_CI_matrix (CIMethod.cpp:611-660). Every off-diagonal
// element of that matrix is a pair hop: row I (pair string S) couples to
// J = S - j + k (j occupied, k empty) with the value K_jk = <jj|kk> = (jk|jk),
// which depends on the two orbitals only (the phase of a pair hop is even), and
// elements with |K_jk| <= 1e-14 are not stored. So a row is generated from its
// string, the L x L table K (shared memory) and the string's rank prefixes:
//
//   y_I = H_II x_I + sum_{j in S, k not in S} K_jk x_J.
//
// The rank of J costs O(1). With p_1 < ... < p_n the occupied orbitals of S and
// rank(S) = sum_m C(p_m, m) (colex, CIMethod.cpp:689-747), j = p_{a+1} and b the
// number of occupied orbitals below k:
//   k > j:  rank(J) = I - C(j, a+1) + (P_b - P_{a+1}) + C(k, b),
//           P_m = sum_{i <= m} (C(p_i, i-1) - C(p_i, i))
//   k < j:  rank(J) = I - C(j, a+1) + C(k, b+1) + (Q_a - Q_b),
//           Q_m = sum_{i <= m} (C(p_i, i+1) - C(p_i, i))
// (the electrons between j and k shift one place), evaluated modulo 2^32: the
// result is a rank below 2^32, so the wrap cancels.
//
// A group of 8-32 lanes per row (about 16 hops per lane). The group writes the
// row's occupied / empty orbital lists and the prefixes (a scan over the group) to
// shared memory, then takes the n (L - n) hops in rounds of up to 8 per lane:
// ranks first, then the round's gathers of x together (L2-resident: 2.7 M FP32
// entries are 10.8 MB at L=24), then one multiply-add each, all lanes on the same
// instruction stream (an FP64
// multiply-add issued for part of a warp would occupy GB300's FP64 pipe for the
// whole warp). The group's sums meet in a fixed shuffle tree and the diagonal term
// is added last, so the order is fixed (bit-reproducible run to run).
//
// Bytes per matvec: the pair strings (8 per row), the diagonal and x read once, y
// written once; the hop gathers hit x in L2. The matrix the CRS form streams
// (145 elements per row at L=24, 12 bytes each in FP64) is not stored at all.
#include "doci_mv.cuh"

namespace cigpu {

namespace {

constexpr int kMvThreads = 256;
constexpr int kMvWarps = kMvThreads / 32;
constexpr int kBW = 34;  // binomial table row: C(nn, kk) for kk <= 33 (n <= 32)

struct RowScratch {
    uint8_t occ[32];
    uint8_t emp[64];
    uint32_t P[33], Q[33];
};

// Hops a lane takes per round: their ranks are formed first and their x gathers
// issued together, so each lane keeps up to kHopBatch L2 loads in flight.
constexpr int kHopBatch = 8;

// G lanes per row, 32 / G rows per warp. Every row of a space has the same n (L - n)
// hops, so the rounds are the same for every group of the warp: no lane runs a
// round that is empty for it except in the last one. Fewer lanes per row mean
// fewer steps in the lanes' final sum (on GB300's FP64 pipe a shuffle-add of the
// FP64 form costs as much as a round of hops).
template <typename T, int G>
__global__ void __launch_bounds__(kMvThreads) k_doci_mv(const DociMv p, const T *__restrict__ K,
                                                        const T *__restrict__ diag, const T *__restrict__ x,
                                                        T *__restrict__ y) {
    constexpr int R = 32 / G;  // rows per warp
    constexpr int kChunk = 32 / G;  // prefix entries per lane (n <= 32)
    __shared__ uint32_t binom[64 * kBW];  // C(nn, kk) mod 2^32
    __shared__ RowScratch rs[kMvWarps][R];
    extern __shared__ __align__(16) unsigned char smem[];
    T *Ks = reinterpret_cast<T *>(smem);  // K[j * L + k]
    const int L = p.L, n = p.n, nv = L - n;
    for (int i = threadIdx.x; i < 64 * kBW; i += blockDim.x) {
        const int nn = i / kBW, kk = i % kBW;
        binom[i] = (nn <= L && kk <= n + 1) ? (uint32_t)d_binom(nn, kk) : 0u;
    }
    for (int i = threadIdx.x; i < L * L; i += blockDim.x) Ks[i] = K[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = lane / G, gl = lane % G;
    RowScratch &w = rs[warp][grp];
    const int nh = n * nv;
    // h / nv as umulhi(h, ceil(2^32 / nv)): exact for h < 4096 and nv < 64 (nh <= 992)
    const uint32_t inv_nv = nv > 0 ? (uint32_t)((0x100000000ull + nv - 1) / nv) : 0u;
    const int64_t rows_per_pass = (int64_t)gridDim.x * kMvWarps * R;
    for (int64_t r0 = ((int64_t)blockIdx.x * kMvWarps + warp) * R; r0 < p.D; r0 += rows_per_pass) {
        const int64_t r = r0 + grp;
        const bool live = r < p.D;
        const uint64_t s = live ? __ldg(p.strings + r) : 0;
        // occupied / empty lists
        if (live)
            for (int i = gl; i < L; i += G) {
                const int below = __popcll(s & ((((uint64_t)1) << i) - 1));
                if ((s >> i) & 1)
                    w.occ[below] = (uint8_t)i;
                else
                    w.emp[i - below] = (uint8_t)i;
            }
        __syncwarp();
        // rank prefixes over the occupied orbitals: lane gl owns indices
        // gl * kChunk .. gl * kChunk + kChunk - 1 (0-based m holds p_{m+1})
        uint32_t dP[kChunk], dQ[kChunk], sP = 0, sQ = 0;
#pragma unroll
        for (int c = 0; c < kChunk; ++c) {
            const int m = gl * kChunk + c;
            uint32_t a = 0, b = 0;
            if (live && m < n) {
                const int pm = w.occ[m];
                a = binom[pm * kBW + m] - binom[pm * kBW + m + 1];
                b = binom[pm * kBW + m + 2] - binom[pm * kBW + m + 1];
            }
            sP += a;
            sQ += b;
            dP[c] = sP;
            dQ[c] = sQ;
        }
        uint32_t eP = sP, eQ = sQ;  // inclusive scan of the chunk sums over the group
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const uint32_t uP = __shfl_up_sync(0xffffffffu, eP, o, G), uQ = __shfl_up_sync(0xffffffffu, eQ, o, G);
            if (gl >= o) {
                eP += uP;
                eQ += uQ;
            }
        }
        if (live) {
#pragma unroll
            for (int c = 0; c < kChunk; ++c) {
                const int m = gl * kChunk + c;
                if (m < n) {
                    w.P[m + 1] = eP - sP + dP[c];
                    w.Q[m + 1] = eQ - sQ + dQ[c];
                }
            }
            if (gl == 0) w.P[0] = w.Q[0] = 0;
        }
        __syncwarp();
        const uint32_t I = (uint32_t)r;
        T acc = 0;
        for (int h0 = 0; h0 < nh; h0 += G * kHopBatch) {
            const int nu = min(kHopBatch, (nh - h0 + G - 1) / G);  // the same for every group
            uint32_t J[kHopBatch];
            T kv[kHopBatch];
#pragma unroll
            for (int u = 0; u < kHopBatch; ++u) {
                if (u < nu) {
                    const int h = h0 + G * u + gl;
                    J[u] = 0xFFFFFFFFu;
                    kv[u] = 0;
                    if (live && h < nh) {
                        const int a = (int)__umulhi((uint32_t)h, inv_nv), bi = h - a * nv;
                        const int j = w.occ[a], k = w.emp[bi];
                        const int b = __popcll(s & ((((uint64_t)1) << k) - 1));
                        uint32_t t = I - binom[j * kBW + a + 1];
                        if (k > j)
                            t += w.P[b] - w.P[a + 1] + binom[k * kBW + b];
                        else
                            t += binom[k * kBW + b + 1] + w.Q[a] - w.Q[b];
                        J[u] = t;
                        kv[u] = Ks[j * L + k];
                    }
                }
            }
            T xv[kHopBatch];
#pragma unroll
            for (int u = 0; u < kHopBatch; ++u)
                if (u < nu) {
                    // 0xFFFFFFFF marks a lane without a hop this round; any other rank
                    // outside the space is a violation (skipped in every build)
                    bool ok = index_ok(J[u], (uint64_t)p.D);
                    if (J[u] != 0xFFFFFFFFu) ok = CIGPU_CHECK(p.err, ok, kCheckHopRank, J[u]) && ok;
                    xv[u] = ok ? __ldg(x + J[u]) : (T)0;
                }
#pragma unroll
            for (int u = 0; u < kHopBatch; ++u)
                if (u < nu) acc += kv[u] * xv[u];
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (live && gl == 0) y[r] = acc + __ldg(diag + r) * __ldg(x + r);
        __syncwarp();  // the scratch is rewritten by the next rows
    }
}

// K_jk = (jk|jk) (chemist), zero where |v| <= 1e-14 and on the diagonal; FP64 and FP32.
__global__ void k_doci_pair_table(int L, const double *__restrict__ eri, double *__restrict__ K64,
                                  float *__restrict__ K32) {
    const int L1 = L;
    const int64_t L2 = (int64_t)L * L, L3 = L2 * L;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < L * L; t += gridDim.x * blockDim.x) {
        const int j = t / L, k = t % L;
        const int lo = j < k ? j : k, hi = j < k ? k : j;
        double v = (j == k) ? 0.0 : eri[lo * L3 + hi * L2 + lo * L1 + hi];
        if (!(v > kZero || v < -kZero)) v = 0.0;
        K64[t] = v;
        K32[t] = (float)v;
    }
}

__global__ void k_count_nonzero(const double *__restrict__ v, int64_t n, unsigned long long *__restrict__ out) {
    unsigned long long c = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        c += (v[i] > kZero || v[i] < -kZero) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

template <typename T, int G>
void launch_mv_g(const DociMv &p0, const T *K, const T *diag, const T *x, T *y, cudaStream_t s) {
    DociMv p = p0;
    p.err = check_word_device();
    const size_t sm = sizeof(T) * (size_t)p.L * p.L;
    static const bool attr_set = [] {  // thread-safe one-time init (L = 63: 31 KB of FP64 K)
        cudaFuncSetAttribute(k_doci_mv<T, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        return true;
    }();
    (void)attr_set;
    constexpr int rows_per_block = kMvWarps * (32 / G);
    const int64_t blocks = std::min<int64_t>((p.D + rows_per_block - 1) / rows_per_block, (int64_t)sm_count() * 8);
    k_doci_mv<T, G><<<(unsigned)std::max<int64_t>(blocks, 1), kMvThreads, sm, s>>>(p, K, diag, x, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

// Lanes per row from the hop count: about 16 hops per lane (at least 8 lanes).
template <typename T>
void launch_mv(const DociMv &p, const T *K, const T *diag, const T *x, T *y, cudaStream_t s) {
    const int nh = p.n * (p.L - p.n);
    if (nh > 384)
        launch_mv_g<T, 32>(p, K, diag, x, y, s);
    else if (nh > 192)
        launch_mv_g<T, 16>(p, K, diag, x, y, s);
    else
        launch_mv_g<T, 8>(p, K, diag, x, y, s);
}

}  // namespace

void doci_pair_table_launch(int L, const double *eri, double *K64, float *K32, cudaStream_t s) {
    k_doci_pair_table<<<(L * L + 255) / 256, 256, 0, s>>>(L, eri, K64, K32);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

int64_t count_nonzero(const double *v, int64_t n, cudaStream_t s) {
    DevBuf<unsigned long long> out(1);
    CIGPU_CUDA(cudaMemsetAsync(out.p, 0, sizeof(unsigned long long), s));
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
    k_count_nonzero<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(v, n, out.p);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
    unsigned long long h = 0;
    CIGPU_CUDA(cudaMemcpyAsync(&h, out.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaStreamSynchronize(s));
    return (int64_t)h;
}

void doci_mv64(const DociMv &p, const double *K, const double *diag, const double *x, double *y, cudaStream_t s) {
    launch_mv<double>(p, K, diag, x, y, s);
}

void doci_mv32(const DociMv &p, const float *K, const float *diag, const float *x, float *y, cudaStream_t s) {
    launch_mv<float>(p, K, diag, x, y, s);
}

}  // namespace cigpu
