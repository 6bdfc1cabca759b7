// CRS Hamiltonian construction on the device (FCI and DOCI).
//
// Replaces FCI::construct_CI_matrix (CIMethod.cpp:749-888) and
// DOCI::construct_CI_matrix (CIMethod.cpp:611-660) together with the sorted row
// insertion of SparseMatrix_CRS::PushToRow/PushToRownoadd (SparseMatrix_CRS.cpp:
// 240-322). Instead of sorted inserts, each row is generated directly in
// ascending column order:
//   FCI row (Ia, Ib), column Ja*Db + Jb. The alpha neighbours of Ia (itself,
//   its singles, its same-spin doubles) are visited in rank order; each alpha
//   neighbour expands to a sorted run of beta columns:
//     Ja == Ia      -> Jb over {Ib} U singles(Ib) U doubles(Ib)   (diag, beta single, beta-beta double)
//     Ja single     -> Jb over {Ib} U singles(Ib)                 (alpha single, alpha-beta double)
//     Ja double     -> Jb = Ib                                    (alpha-alpha double)
//   DOCI row I: {I} plus every pair hop j -> k, sorted by rank in shared memory.
// A warp owns one row; each lane evaluates one structural slot, and a ballot
// keeps the elements with |v| > 1e-14 in order. Three passes use the same
// generator: COUNT (row lengths) and FILL (columns + values; FP64, or FP32 hi
// and lo parts for the mixed method).
//
// Values are bit-identical to the reference: every element is a chain of FP64
// additions in the reference order (no multiplications, so no FMA contraction),
// and lower-triangle entries are evaluated from the perspective the reference
// uses for the mirrored upper entry.
#include "build.cuh"

namespace cigpu {

__device__ __forceinline__ double ld_eri(const double *eri, int L, int i, int j, int k, int l) {
    return __ldg(eri + (((size_t)i * L + j) * L + k) * L + l);
}

// ---------------------------------------------------------------------------
// Row diagonals. FCI: CIMethod::diagonal (CIMethod.cpp:398-407) =
// (diag(alpha) + diag(beta)) + sum_{k in a, l in b} V(k,l,k,l).
__global__ void k_fci_diag(FciParams p, double *diag) {
    const int64_t dim = p.a.D * p.Db;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ia = r / p.Db, ib = r - ia * p.Db;
        double tot = p.a.diag[ia];
        tot += p.b.diag[ib];
        double mix = 0;
        const uint8_t *oa = p.a.occ + ia * p.a.n;
        const uint8_t *ob = p.b.occ + ib * p.b.n;
        for (int k = 0; k < p.a.n; ++k) {
            const int u = oa[k];
            for (int l = 0; l < p.b.n; ++l) {
                const int d = ob[l];
                mix += ld_eri(p.eri, p.L, u, u, d, d);  // <ud|ud> = (uu|dd)
            }
        }
        tot += mix;
        diag[r] = tot;
    }
}

// |v| > 1e-14 on the bit pattern (integer compare; GB300's FP64 pipe is slow).
__device__ __forceinline__ bool keep_bits(uint64_t b) {
    return (b & 0x7FFFFFFFFFFFFFFFull) > 0x3D06849B86A12B9Bull;  // bits of 1e-14
}
__device__ __forceinline__ uint64_t flip_if(uint64_t b, uint32_t odd) { return b ^ ((uint64_t)odd << 63); }
__device__ __forceinline__ float flipf_if(float f, uint32_t odd) {
    return __uint_as_float(__float_as_uint(f) ^ (odd << 31));
}

// One FCI row per warp; the block owns one alpha string Ia and kFciRowsPerBlock
// beta strings. Shared memory: the alpha neighbour list, group starts, the slot ->
// group map, and the integral slices (ar ac|. .) of the alpha singles of Ia
// (FP64 for COUNT/FILL64/MATVEC; FP32 hi/lo for FILL32, zeroed where |v| <= 1e-14).
// Single-excitation elements of every row, one thread per (row, single):
// one_diff_orbital (CIMethod.cpp:409-427) = same-spin part (host, s_part) + the
// opposite-spin terms added in ascending orbital order, then the phase. Done
// here without divergence so the row generator only loads them.
__global__ void k_fci_singles(FciParams p, double *__restrict__ sgl64, float *__restrict__ sgl_hi,
                              float *__restrict__ sgl_lo, float *__restrict__ diag_hi, float *__restrict__ diag_lo) {
    const int ns = p.a.ns + p.b.ns;
    const int64_t dim = p.a.D * p.Db;
    const int64_t total = dim * ns;
    const size_t L1 = p.L, L2 = L1 * L1, L3 = L2 * L1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / ns;
        const int q = (int)(i - r * ns);
        const int64_t ia = r / p.Db, ib = r - ia * p.Db;
        double v;
        uint32_t info;
        if (q < p.a.ns) {  // alpha single, beta spectators
            const size_t at = ia * p.a.ns + q;
            v = p.a.s_part[at];
            info = p.a.s_info[at];
            const double *e = p.eri + (info & 63) * L3 + ((info >> 6) & 63) * L2;
            const uint8_t *occ = p.b.occ + ib * p.b.n;
            for (int z = 0; z < p.b.n; ++z) v += __ldg(e + occ[z] * (L1 + 1));  // (lo hi|z z)
        } else {  // beta single, alpha spectators
            const size_t at = ib * p.b.ns + (q - p.a.ns);
            v = p.b.s_part[at];
            info = p.b.s_info[at];
            const double *e = p.eri + (info & 63) * L3 + ((info >> 6) & 63) * L2;
            const uint8_t *occ = p.a.occ + ia * p.a.n;
            for (int z = 0; z < p.a.n; ++z) v += __ldg(e + occ[z] * (L1 + 1));
        }
        if ((info >> 24) & 1) v = -v;
        sgl64[i] = v;
        if (sgl_hi) {
            float hi, lo;
            split_fp32(v, hi, lo);
            sgl_hi[i] = hi;
            sgl_lo[i] = lo;
        }
    }
    if (diag_hi)
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x)
            split_fp32(p.diag[r], diag_hi[r], diag_lo[r]);
}

template <int MODE>
__global__ void __launch_bounds__(kFciThreads) k_fci_rows(FciParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nga = p.a.nfull;
    const int L = p.L, L2 = L * L;
    const int nsa = p.a.ns;
    const int W = p.b.nfull + nsa * p.b.nsing + p.a.nd;
    constexpr bool F32 = MODE == kFill32;
    uint64_t *nbA = reinterpret_cast<uint64_t *>(smem);
    uint32_t *gstart = reinterpret_cast<uint32_t *>(nbA + nga);
    uint16_t *gmap = reinterpret_cast<uint16_t *>(gstart + nga + 1);
    unsigned char *after = reinterpret_cast<unsigned char *>(gmap + W);
    after = reinterpret_cast<unsigned char *>(((uintptr_t)after + 15) & ~(uintptr_t)15);
    uint64_t *sl64 = reinterpret_cast<uint64_t *>(after);  // [nsa][L2] FP64 bits
    float *slhi = reinterpret_cast<float *>(after);       // [nsa][L2]
    float *sllo = slhi + (size_t)nsa * L2;                // [nsa][L2]

    const int64_t nchunks = (p.Db + kFciRowsPerBlock - 1) / kFciRowsPerBlock;
    const int64_t ia = blockIdx.x / nchunks;
    const int64_t chunk = blockIdx.x - ia * nchunks;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;

    for (int g = tid; g < nga; g += blockDim.x) nbA[g] = p.a.nb_full[ia * nga + g];
    if (p.staged) {
        for (int i = tid; i < nsa * L2; i += blockDim.x) {
            const int xa = i / L2, t = i - xa * L2;
            const uint32_t info = __ldg(p.a.s_info + ia * nsa + xa);
            const int ar = (info >> 12) & 63, ac = (info >> 18) & 63;
            const size_t at = ((size_t)ar * L + ac) * L2 + t;  // (ar ac|br bc)
            if (F32) {
                slhi[i] = __ldg(p.eri_hi + at);
                sllo[i] = __ldg(p.eri_lo + at);
            } else {
                sl64[i] = __double_as_longlong(__ldg(p.eri + at));
            }
        }
    }
    __syncthreads();
    if (warp == 0) {
        uint32_t run = 0;
        for (int g0 = 0; g0 < nga; g0 += 32) {
            const int g = g0 + lane;
            uint32_t sz = 0;
            if (g < nga) {
                const uint32_t kind = (uint32_t)(nbA[g] >> 32) & 3u;
                sz = kind == kSelf ? (uint32_t)p.b.nfull : (kind == kSingle ? (uint32_t)p.b.nsing : 1u);
            }
            uint32_t incl = sz;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (g < nga) gstart[g] = run + incl - sz;
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) gstart[nga] = run;
    }
    __syncthreads();
    for (int g = tid; g < nga; g += blockDim.x)
        for (uint32_t k = gstart[g]; k < gstart[g + 1]; ++k) gmap[k] = (uint16_t)g;
    __syncthreads();

    for (int rr = warp; rr < kFciRowsPerBlock; rr += nwarps) {
        const int64_t ib = chunk * kFciRowsPerBlock + rr;
        if (ib >= p.Db) break;
        const int64_t r = ia * p.Db + ib;
        const uint64_t *nbF = p.b.nb_full + ib * p.b.nfull;
        const uint64_t *nbS = p.b.nb_sing + ib * p.b.nsing;
        int64_t base = 0;
        if (MODE == kFill64 || MODE == kFill32) base = p.row_ptr[r];
        uint32_t running = 0, nlow = 0;
        for (int k0 = 0; k0 < W; k0 += 32) {
            const int k = k0 + lane;
            uint64_t vb = 0;       // FP64 bits (COUNT / FILL64 / MATVEC, and computed elements)
            float hi = 0, lo = 0;  // FILL32
            bool keep = false, low = false;
            uint32_t col = 0;
            if (k < W) {
                const int g = gmap[k];
                const int q = k - (int)gstart[g];
                const uint64_t ea = nbA[g];
                const uint32_t kindA = (uint32_t)(ea >> 32) & 3u;
                const uint32_t Ja = (uint32_t)ea;
                const uint32_t xa = (uint32_t)(ea >> 34);
                if (kindA == kSelf) {
                    const uint64_t eb = __ldg(nbF + q);
                    const uint32_t kindB = (uint32_t)(eb >> 32) & 3u;
                    const uint32_t Jb = (uint32_t)eb;
                    const uint32_t xb = (uint32_t)(eb >> 34);
                    col = (uint32_t)(ia * p.Db + Jb);
                    low = Jb < (uint32_t)ib;
                    if (kindB == kSelf) {
                        if (F32) {
                            hi = p.diag_hi[r];
                            lo = p.diag_lo[r];
                        } else {
                            vb = __double_as_longlong(p.diag[r]);
                        }
                    } else if (kindB == kSingle) {
                        // beta single (one_diff_orbital(down1, down2, up1)), precomputed per row
                        const size_t at = (size_t)r * (nsa + p.b.ns) + nsa + xb;
                        if (F32) {
                            hi = __ldg(p.sgl_hi + at);
                            lo = __ldg(p.sgl_lo + at);
                        } else {
                            vb = __double_as_longlong(__ldg(p.sgl64 + at));
                        }
                    } else {
                        const size_t at = ib * p.b.nd + xb;
                        if (F32) {
                            hi = __ldg(p.b.d_hi + at);
                            lo = __ldg(p.b.d_lo + at);
                        } else {
                            vb = __double_as_longlong(__ldg(p.b.d_val + at));
                        }
                    }
                } else if (kindA == kSingle) {
                    const uint64_t eb = __ldg(nbS + q);
                    const uint32_t kindB = (uint32_t)(eb >> 32) & 3u;
                    const uint32_t Jb = (uint32_t)eb;
                    const uint32_t xb = (uint32_t)(eb >> 34);
                    col = (uint32_t)((int64_t)Ja * p.Db + Jb);
                    low = Ja < (uint32_t)ia;
                    const uint32_t infoA = __ldg(p.a.s_info + ia * nsa + xa);
                    if (kindB == kSelf) {
                        // alpha single (one_diff_orbital(up1, up2, down1)), precomputed per row
                        const size_t at = (size_t)r * (nsa + p.b.ns) + xa;
                        if (F32) {
                            hi = __ldg(p.sgl_hi + at);
                            lo = __ldg(p.sgl_lo + at);
                        } else {
                            vb = __double_as_longlong(__ldg(p.sgl64 + at));
                        }
                    } else {
                        // two_diff_orbitals(up1,up2,down1,down2) (CIMethod.cpp:444-457):
                        // V(a_row, b_row, a_col, b_col) = (ar ac|br bc); exact 8-fold symmetry
                        // of the stored integrals makes it independent of which side is the row.
                        const uint32_t infoB = __ldg(p.b.s_info + ib * p.b.ns + xb);
                        const int br = (infoB >> 12) & 63, bc = (infoB >> 18) & 63;
                        const uint32_t odd = ((infoA ^ infoB) >> 24) & 1;
                        const int t = br * L + bc;
                        if (F32) {
                            if (p.staged) {
                                hi = slhi[xa * L2 + t];
                                lo = sllo[xa * L2 + t];
                            } else {
                                const int ar = (infoA >> 12) & 63, ac = (infoA >> 18) & 63;
                                const size_t at = ((size_t)ar * L + ac) * L2 + t;
                                hi = __ldg(p.eri_hi + at);
                                lo = __ldg(p.eri_lo + at);
                            }
                            hi = flipf_if(hi, odd);
                            lo = flipf_if(lo, odd);
                        } else {
                            uint64_t b;
                            if (p.staged) {
                                b = sl64[xa * L2 + t];
                            } else {
                                const int ar = (infoA >> 12) & 63, ac = (infoA >> 18) & 63;
                                b = __double_as_longlong(__ldg(p.eri + ((size_t)ar * L + ac) * L2 + t));
                            }
                            vb = flip_if(b, odd);
                        }
                    }
                } else {
                    col = (uint32_t)((int64_t)Ja * p.Db + ib);
                    low = Ja < (uint32_t)ia;
                    const size_t at = ia * p.a.nd + xa;
                    if (F32) {
                        hi = __ldg(p.a.d_hi + at);
                        lo = __ldg(p.a.d_lo + at);
                    } else {
                        vb = __double_as_longlong(__ldg(p.a.d_val + at));
                    }
                }
                if (F32)
                    keep = (__float_as_uint(hi) & 0x7FFFFFFFu) != 0u;  // splits are zero where |v| <= 1e-14
                else
                    keep = keep_bits(vb);
            }
            const uint32_t mask = __ballot_sync(0xffffffffu, keep);
            if (MODE == kCount) {
                nlow += __popc(__ballot_sync(0xffffffffu, keep && low));
            } else if (MODE == kFill64 || MODE == kFill32) {
                if (keep) {
                    const int64_t pos = base + running + __popc(mask & ((1u << lane) - 1u));
                    p.col[pos] = col;
                    if (MODE == kFill64) {
                        p.val64[pos] = __longlong_as_double(vb);
                    } else {
                        p.val32[pos] = hi;
                        p.val32lo[pos] = lo;
                    }
                }
            }
            running += __popc(mask);
        }
        if (MODE == kCount) {
            if (lane == 0) {
                p.row_count[r] = running;
                p.upper_off[r] = nlow;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// DOCI.
__global__ void k_unrank(int L, int n, int64_t D, uint64_t *strings) {
    __shared__ int64_t binom[64 * 33];  // C(p, m) for p < 64, m <= 32 (n <= 32 is enforced by the host)
    for (int i = threadIdx.x; i < 64 * 33; i += blockDim.x) {
        const int pp = i / 33, mm = i % 33;
        binom[i] = (pp <= L && mm <= n) ? d_binom(pp, mm) : 0;
    }
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
        // inverse of rank = sum_m C(p_m, m): pick the largest p with C(p, m) <= remaining
        uint64_t s = 0;
        int64_t rem = i;
        int p = L - 1;
        for (int m = n; m >= 1; --m) {
            while (p >= 0 && binom[p * 33 + m] > rem) --p;
            s |= (uint64_t)1 << p;
            rem -= binom[p * 33 + m];
            --p;
        }
        strings[i] = s;
    }
}

// DOCI diagonal: diagonal(up1, up1) (CIMethod.cpp:398-407, DOCI.cpp path :630).
__global__ void k_doci_diag(DociParams p, double *diag) {
    const size_t L1 = p.L, L2 = L1 * L1, L3 = L2 * L1;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < p.D; r += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t s = p.strings[r];
        int o[64];
        int n = 0;
        for (uint64_t t = s; t; t &= t - 1) o[n++] = __ffsll((long long)t) - 1;
        double d = 0;
        for (int a = 0; a < n; ++a) d += __ldg(p.h + o[a] * L1 + o[a]);
        for (int a = 0; a < n - 1; ++a)
            for (int b = a + 1; b < n; ++b)
                d += __ldg(p.eri + o[a] * L3 + o[a] * L2 + o[b] * L1 + o[b]) -
                     __ldg(p.eri + o[a] * L3 + o[b] * L2 + o[b] * L1 + o[a]);
        double tot = d;
        tot += d;
        double mix = 0;
        for (int a = 0; a < n; ++a)
            for (int b = 0; b < n; ++b) mix += __ldg(p.eri + o[a] * L3 + o[a] * L2 + o[b] * L1 + o[b]);
        tot += mix;
        diag[r] = tot;
    }
}

template <int MODE>
__global__ void __launch_bounds__(kDociThreads) k_doci_rows(DociParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int W = p.W;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    uint32_t *binom = reinterpret_cast<uint32_t *>(smem);  // [64][33]
    unsigned char *wbase = smem + 64 * 33 * sizeof(uint32_t);
    const size_t per_warp = (size_t)W * (sizeof(double) + sizeof(uint32_t) + sizeof(uint16_t));
    double *vals = reinterpret_cast<double *>(wbase + warp * ((per_warp + 15) & ~(size_t)15));
    uint32_t *keys = reinterpret_cast<uint32_t *>(vals + W);
    uint16_t *perm = reinterpret_cast<uint16_t *>(keys + W);
    // C(p, m) for p <= L, m <= n (n <= 32 is enforced by the host); every term of a
    // valid rank is below the dimension, which fits in 32 bits
    for (int i = tid; i < 64 * 33; i += blockDim.x) {
        const int nn = i / 33, kk = i % 33;
        binom[i] = (nn <= p.L && kk <= p.n) ? (uint32_t)d_binom(nn, kk) : 0u;
    }
    __syncthreads();
    const int nv = p.L - p.n;
    const size_t L1 = p.L, L2 = L1 * L1, L3 = L2 * L1;
    for (int64_t r = blockIdx.x * (int64_t)nwarps + warp; r < p.D; r += (int64_t)gridDim.x * nwarps) {
        const uint64_t s = p.strings[r];
        // generate all entries with their target rank
        for (int e = lane; e < W; e += 32) {
            uint32_t key;
            double v;
            if (e == 0) {
                key = (uint32_t)r;
                v = p.diag[r];
            } else {
                const int hh = e - 1, a = hh / nv, b = hh - a * nv;
                const int j = nth_set(s, a);
                const int k = nth_set(~s & p.fullmask, b);
                const uint64_t t = s ^ ((uint64_t)1 << j) ^ ((uint64_t)1 << k);
                uint32_t rk = 0;
                int m = 0;
                for (uint64_t u = t; u; u &= u - 1) {
                    ++m;
                    rk += binom[(__ffsll((long long)u) - 1) * 33 + m];
                }
                key = rk;
                // DOCI pair hop: two_diff_orbitals(up1,up2,up1,up2) = V(lo,lo,hi,hi) = (lo hi|lo hi)
                const int lo = j < k ? j : k, hi = j < k ? k : j;
                v = __ldg(p.eri + lo * L3 + hi * L2 + lo * L1 + hi);
            }
            keys[e] = key;
            vals[e] = v;
        }
        __syncwarp();
        if (MODE == kCount) {
            uint32_t cnt = 0, low = 0;
            for (int e = lane; e < W; e += 32) {
                const bool keep = keep_bits(__double_as_longlong(vals[e]));
                cnt += keep;
                low += keep && keys[e] < (uint32_t)r;
            }
            for (int o = 16; o > 0; o >>= 1) {
                cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
                low += __shfl_xor_sync(0xffffffffu, low, o);
            }
            if (lane == 0) {
                p.row_count[r] = cnt;
                p.upper_off[r] = low;
            }
            __syncwarp();
            continue;
        }
        // sorted position = number of smaller ranks (ranks are distinct)
        for (int e = lane; e < W; e += 32) {
            const uint32_t key = keys[e];
            int pos = 0;
            for (int f = 0; f < W; ++f) pos += keys[f] < key;
            perm[pos] = (uint16_t)e;
        }
        __syncwarp();
        const int64_t base = p.row_ptr[r];
        uint32_t running = 0;
        for (int k0 = 0; k0 < W; k0 += 32) {
            const int k = k0 + lane;
            double v = 0;
            uint32_t col = 0;
            if (k < W) {
                const int e = perm[k];
                v = vals[e];
                col = keys[e];
            }
            const bool keep = (k < W) && keep_bits(__double_as_longlong(v));
            const uint32_t mask = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const int64_t pos = base + running + __popc(mask & ((1u << lane) - 1u));
                p.col[pos] = col;
                if (MODE == kFill64) {
                    p.val64[pos] = v;
                } else {
                    const float hi = (float)v;
                    p.val32[pos] = hi;
                    p.val32lo[pos] = (float)(v - (double)hi);
                }
            }
            running += __popc(mask);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Upper-triangle extraction (the reference layout) from the full rows.
__global__ void k_upper_counts(int64_t dim, const int64_t *row_ptr, const uint32_t *upper_off, uint32_t *ucnt) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x)
        ucnt[r] = (uint32_t)(row_ptr[r + 1] - row_ptr[r]) - upper_off[r];
}

template <typename VT>
__global__ void k_extract_upper(int64_t dim, const int64_t *row_ptr, const uint32_t *upper_off, const uint32_t *col,
                                const VT *val, const int64_t *urow, uint32_t *ucol, double *uval) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = wid; r < dim; r += nw) {
        const int64_t s = row_ptr[r] + upper_off[r], e = row_ptr[r + 1], o = urow[r];
        for (int64_t k = s + lane; k < e; k += 32) {
            ucol[o + (k - s)] = col[k];
            uval[o + (k - s)] = (double)val[k];
        }
    }
}

// ---------------------------------------------------------------------------
// Host launchers.
static int grid_for(int64_t work, int threads, int per_sm = 8) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t g = (work + threads - 1) / threads;
    int64_t cap = (int64_t)sms * per_sm;
    return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

static size_t fci_base_smem(const FciParams &p) {
    const int W = p.b.nfull + p.a.ns * p.b.nsing + p.a.nd;
    size_t b = (size_t)p.a.nfull * 8 + ((size_t)p.a.nfull + 1) * 4 + (size_t)W * 2;
    return (b + 15) & ~(size_t)15;
}

// Integral slices of the alpha singles: nsa * L^2 entries of 8 bytes (FP64, or FP32 hi + lo).
static size_t fci_slice_smem(const FciParams &p) { return (size_t)p.a.ns * p.L * p.L * 8; }

size_t fci_smem_bytes(const FciParams &p) {
    const size_t b = fci_base_smem(p), sl = fci_slice_smem(p);
    return (b + sl <= kFciMaxSmem) ? b + sl : b;
}

void fci_launch(int mode, const FciParams &p0, cudaStream_t s) {
    FciParams p = p0;
    const size_t sm = fci_smem_bytes(p);
    p.staged = (sm == fci_base_smem(p) + fci_slice_smem(p)) ? 1 : 0;
    const int64_t nchunks = (p.Db + kFciRowsPerBlock - 1) / kFciRowsPerBlock;
    const int64_t blocks = p.a.D * nchunks;
    if (mode == kFill32 && (!p.eri_hi || !p.eri_lo))
        throw CudaError{cudaErrorInvalidValue, "FP32 integral tables missing"};
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_fci_rows<kCount>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFciMaxSmem);
        cudaFuncSetAttribute(k_fci_rows<kFill64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFciMaxSmem);
        cudaFuncSetAttribute(k_fci_rows<kFill32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFciMaxSmem);
        return true;
    }();
    (void)attr_set;
    switch (mode) {
        case kCount: k_fci_rows<kCount><<<(unsigned)blocks, kFciThreads, sm, s>>>(p); break;
        case kFill64: k_fci_rows<kFill64><<<(unsigned)blocks, kFciThreads, sm, s>>>(p); break;
        default: k_fci_rows<kFill32><<<(unsigned)blocks, kFciThreads, sm, s>>>(p); break;
    }
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void fci_singles_launch(const FciParams &p, double *sgl64, float *sgl_hi, float *sgl_lo, float *diag_hi,
                        float *diag_lo, cudaStream_t s) {
    const int64_t total = p.a.D * p.Db * (int64_t)(p.a.ns + p.b.ns);
    k_fci_singles<<<grid_for(std::max<int64_t>(total, 1), 256, 16), 256, 0, s>>>(p, sgl64, sgl_hi, sgl_lo, diag_hi,
                                                                                 diag_lo);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void fci_diag_launch(const FciParams &p, double *diag, cudaStream_t s) {
    k_fci_diag<<<grid_for(p.a.D * p.Db, 256), 256, 0, s>>>(p, diag);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

size_t doci_smem_bytes(int W, int warps) {
    const size_t per_warp = ((size_t)W * (sizeof(double) + sizeof(uint32_t) + sizeof(uint16_t)) + 15) & ~(size_t)15;
    return 64 * 33 * sizeof(uint32_t) + per_warp * warps;
}

void doci_strings_launch(int L, int n, int64_t D, uint64_t *strings, cudaStream_t s) {
    k_unrank<<<grid_for(D, 256), 256, 0, s>>>(L, n, D, strings);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void doci_diag_launch(const DociParams &p, double *diag, cudaStream_t s) {
    k_doci_diag<<<grid_for(p.D, 128), 128, 0, s>>>(p, diag);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void doci_launch(int mode, const DociParams &p, cudaStream_t s) {
    const int warps = kDociThreads / 32;
    const size_t sm = doci_smem_bytes(p.W, warps);
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_doci_rows<kCount>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_doci_rows<kFill64>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_doci_rows<kFill32>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        return true;
    }();
    (void)attr_set;
    const int blocks = grid_for(p.D * 32, kDociThreads, 16);
    switch (mode) {
        case kCount: k_doci_rows<kCount><<<blocks, kDociThreads, sm, s>>>(p); break;
        case kFill64: k_doci_rows<kFill64><<<blocks, kDociThreads, sm, s>>>(p); break;
        default: k_doci_rows<kFill32><<<blocks, kDociThreads, sm, s>>>(p); break;
    }
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void upper_counts_launch(int64_t dim, const int64_t *row_ptr, const uint32_t *upper_off, uint32_t *ucnt,
                         cudaStream_t s) {
    k_upper_counts<<<grid_for(dim, 256), 256, 0, s>>>(dim, row_ptr, upper_off, ucnt);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void extract_upper_launch(int64_t dim, const int64_t *row_ptr, const uint32_t *upper_off, const uint32_t *col,
                          const double *val64, const float *val32, const int64_t *urow, uint32_t *ucol, double *uval,
                          cudaStream_t s) {
    const int blocks = grid_for(dim * 32, 256, 16);
    if (val64)
        k_extract_upper<double><<<blocks, 256, 0, s>>>(dim, row_ptr, upper_off, col, val64, urow, ucol, uval);
    else
        k_extract_upper<float><<<blocks, 256, 0, s>>>(dim, row_ptr, upper_off, col, val32, urow, ucol, uval);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

// ---------------------------------------------------------------------------
// Device-wide exclusive scan of u32 counts into 64-bit offsets (row pointers).
namespace {
constexpr int kScanThreads = 512;
constexpr int kScanPerThread = 8;
constexpr int kScanTile = kScanThreads * kScanPerThread;

__device__ int64_t block_inclusive_scan(int64_t v, int64_t *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        sh[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v += sh[warp - 1];
    __syncthreads();
    return v;
}

__global__ void k_scan_tiles(const uint32_t *in, int64_t n, int64_t *tile_sums) {
    __shared__ int64_t sh[32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
    int64_t s = 0;
    for (int i = 0; i < kScanPerThread; ++i)
        if (base + i < n) s += in[base + i];
    s = block_inclusive_scan(s, sh);
    if (threadIdx.x == blockDim.x - 1) tile_sums[blockIdx.x] = s;
}

__global__ void k_scan_sums(int64_t *tile_sums, int64_t ntiles) {
    __shared__ int64_t sh[32];
    __shared__ int64_t total;
    int64_t carry = 0;
    for (int64_t b0 = 0; b0 < ntiles; b0 += blockDim.x) {
        const int64_t i = b0 + threadIdx.x;
        const int64_t v = i < ntiles ? tile_sums[i] : 0;
        const int64_t inc = block_inclusive_scan(v, sh);
        if (i < ntiles) tile_sums[i] = carry + inc - v;  // exclusive tile offsets
        if (threadIdx.x == blockDim.x - 1) total = inc;
        __syncthreads();
        carry += total;
        __syncthreads();
    }
}

__global__ void k_scan_apply(const uint32_t *in, int64_t n, const int64_t *tile_off, int64_t *out) {
    __shared__ int64_t sh[32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
    uint32_t v[kScanPerThread];
    int64_t s = 0;
    for (int i = 0; i < kScanPerThread; ++i) {
        v[i] = (base + i < n) ? in[base + i] : 0u;
        s += v[i];
    }
    int64_t run = block_inclusive_scan(s, sh) - s + tile_off[blockIdx.x];
    for (int i = 0; i < kScanPerThread; ++i) {
        run += v[i];
        if (base + i < n) out[base + i + 1] = run;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[0] = 0;
}
}  // namespace

void exclusive_scan_u32_async(const uint32_t *in, int64_t *out, int64_t n, DevBuf<int64_t> &sums, cudaStream_t s) {
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles == 0) {
        CIGPU_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), s));
        return;
    }
    sums.alloc(ntiles);
    k_scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, sums.p);
    k_scan_sums<<<1, 1024, 0, s>>>(sums.p, ntiles);
    k_scan_apply<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, sums.p, out);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(3);
}

void exclusive_scan_u32(const uint32_t *in, int64_t *out, int64_t n, cudaStream_t s) {
    DevBuf<int64_t> sums;
    exclusive_scan_u32_async(in, out, n, sums, s);
    // keep `sums` alive until the kernels finish
    CIGPU_CUDA(cudaStreamSynchronize(s));
}

int sm_count() {
    static const int sms = [] {  // thread-safe one-time init
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        return n;
    }();
    return sms;
}

}  // namespace cigpu
