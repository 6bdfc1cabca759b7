// Determinant-list CI: FCI_File and CI_Big (cigpu_build_dets), and the
// Permutator_File reader (cigpu_dets_read).
//
// The reference builds a CI matrix over an arbitrary list of determinants read
// from a text file (FCI_File::construct_CI_matrix, CIMethod.cpp:890-914): every
// pair (i, j >= i) of the list goes through get_ham_element (CIMethod.cpp:459-487),
// which classifies the pair by the popcounts of up1^up2 and down1^down2 and
// evaluates the Slater-Condon rule (diagonal, one_diff_orbital, two_diff_orbitals;
// CIMethod.cpp:329-457). CI_Big (CIMethod.cpp:591-609, 928-1144) keeps part of the
// matrix and recomputes the rest in every matvec.
//
// Here the list lives on the device as records of 2W 64-bit words (up string, then
// down string; W = 1 for L <= 64, W = 2 for L <= 128). One warp owns one row and
// streams the list through shared memory in tiles; each lane tests one column
// (popcount of the XORs, <= 2 excitations) and evaluates the element with the
// reference's summation order, so the values are bit-identical to the reference's.
// The full symmetric matrix is built row by row (every row scans the whole list;
// columns come out ascending, the kept set compacted with a warp ballot), so no
// transpose is needed and the upper triangle is the reference CRS. Storage:
//   CIGPU_DETS_CRS      the CRS (FP64, or FP32 hi/lo for the mixed method);
//   CIGPU_DETS_ONTHEFLY nothing but the list: every FP64 matvec rescans all pairs
//                       and applies the elements as it computes them (CI_Big with
//                       no stored part), y_i summed in a fixed order per row.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "crs.cuh"
#include "spmv.cuh"

namespace cigpu {

namespace {

constexpr int kDetWarps = 8;   // rows per block (one warp each)
constexpr int kDetTile = 256;  // determinants per shared-memory tile
enum DetMode : int { kDetCount = 0, kDetFill64 = 1, kDetFill32 = 2, kDetMatvec = 3 };

struct DetParams {
    int L, nup, ndown;
    int64_t n;
    // rows the pass visits (count / fill: the stored rows; matvec: all n) and the
    // stored block: count / fill take columns below `block` (n for a whole CRS); the
    // matvec takes the pairs outside the block (row i < block: columns >= block)
    int64_t nrows = 0, block = 0;
    const uint64_t *dets;  // [n][2W]
    const double *eri;     // chemist (pq|rs), L^4
    const double *h;       // L^2
    const double *diag;    // [n]
    // count pass
    uint32_t *row_count, *upper_off;
    // fill pass
    const int64_t *row_ptr;
    uint32_t *col;
    double *val64;
    float *val32, *val32lo;
};

__device__ __forceinline__ double Tm(const DetParams &p, int i, int j) { return p.h[i * p.L + j]; }
// physics <ij|kl> = chemist (ik|jl)
__device__ __forceinline__ double Vm(const DetParams &p, int i, int j, int k, int l) {
    const int64_t L = p.L;
    return p.eri[((i * L + k) * L + j) * L + l];
}

// Set bits of `up` in [min(o0,o1), max(o0,o1)) (get_nstacked, CIMethod.cpp:382-396).
template <int W>
__device__ __forceinline__ int nstacked(int o0, int o1, const uint64_t *up) {
    const int lo = min(o0, o1), hi = max(o0, o1);
    int n = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int b0 = max(lo - 64 * w, 0), b1 = min(hi - 64 * w, 64);
        if (b1 <= b0) continue;
        uint64_t m = b1 == 64 ? ~(uint64_t)0 : (((uint64_t)1 << b1) - 1);
        m &= ~(((uint64_t)1 << b0) - 1);
        n += __popcll(up[w] & m);
    }
    return n;
}

// Orbitals of s in ascending order (get_orbs); at most `cap` of them.
template <int W>
__device__ __forceinline__ int orbitals(const uint64_t *s, int *o, int cap) {
    int n = 0;
#pragma unroll
    for (int w = 0; w < W; ++w)
        for (uint64_t x = s[w]; x && n < cap; x &= x - 1) o[n++] = 64 * w + __ffsll((long long)x) - 1;
    return n;
}

// -e when odd, on the sign bit (exact, and off GB300's slow FP64 pipe)
__device__ __forceinline__ double negate_if(double e, int odd) {
    return __longlong_as_double(__double_as_longlong(e) ^ ((long long)odd << 63));
}

// |v| > 1e-14 (SparseMatrix_CRS::PushToRow's drop threshold) as an integer compare of
// the magnitude bits; the values are finite (the integrals are validated)
__device__ __forceinline__ bool keep_value(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull) > 0x3D06849B86A12B9Bull;
}

// Lowest set orbital of x (cleared from x); x is a register array (constant indices).
template <int W>
__device__ __forceinline__ int pop_lowest(uint64_t *x) {
    int o = -1;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        if (o < 0 && x[w]) {
            o = 64 * w + __ffsll((long long)x[w]) - 1;
            x[w] &= x[w] - 1;
        }
    }
    return o;
}

template <int W>
__device__ __forceinline__ bool has_bit(const uint64_t *s, int o) {
    return (s[o >> 6] >> (o & 63)) & 1;
}

// get_diag_cont_one_bitstring (CIMethod.cpp:329-342): sum of T, then of the pair terms
template <int W>
__device__ double diag_one(const DetParams &p, const uint64_t *s) {
    int o[128];
    const int n = orbitals<W>(s, o, 128);
    double sum = 0;
    for (int k = 0; k < n; ++k) sum += Tm(p, o[k], o[k]);
    for (int k = 0; k + 1 < n; ++k)
        for (int l = k + 1; l < n; ++l) sum += Vm(p, o[k], o[l], o[k], o[l]) - Vm(p, o[k], o[l], o[l], o[k]);
    return sum;
}

// CIMethod::diagonal (CIMethod.cpp:398-407): (up part + down part) + the up-down part
template <int W>
__device__ double diagonal(const DetParams &p, const uint64_t *up, const uint64_t *dn) {
    double tot = diag_one<W>(p, up);
    tot += diag_one<W>(p, dn);
    double mix = 0;
#pragma unroll
    for (int wu = 0; wu < W; ++wu)
        for (uint64_t xu = up[wu]; xu; xu &= xu - 1) {
            const int a = 64 * wu + __ffsll((long long)xu) - 1;
#pragma unroll
            for (int wd = 0; wd < W; ++wd)
                for (uint64_t xd = dn[wd]; xd; xd &= xd - 1) {
                    const int b = 64 * wd + __ffsll((long long)xd) - 1;
                    mix += Vm(p, a, b, a, b);
                }
        }
    tot += mix;
    return tot;
}

// one_diff_orbital (CIMethod.cpp:409-427); `other` is the opposite-spin string
template <int W>
__device__ __forceinline__ double one_diff(const DetParams &p, const uint64_t *s1, const uint64_t *s2, const uint64_t *other) {
    uint64_t x[W], c[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        x[w] = s1[w] ^ s2[w];
        c[w] = s1[w] & s2[w];
    }
    const int o0 = pop_lowest<W>(x), o1 = pop_lowest<W>(x);
    double e = Tm(p, o0, o1);
#pragma unroll
    for (int w = 0; w < W; ++w)
        for (uint64_t y = c[w]; y; y &= y - 1) {
            const int z = 64 * w + __ffsll((long long)y) - 1;
            e += Vm(p, o0, z, o1, z) - Vm(p, o0, z, z, o1);
        }
    const int diff = nstacked<W>(o0, o1, c);
#pragma unroll
    for (int w = 0; w < W; ++w)
        for (uint64_t y = other[w]; y; y &= y - 1) {
            const int z = 64 * w + __ffsll((long long)y) - 1;
            e += Vm(p, o0, z, o1, z);
        }
    return negate_if(e, diff & 1);
}

// arrange_order (CIMethod.cpp:353-380) for four ascending orbitals of which two are
// occupied in s1: (a0, a1) those of s1, (b0, b1) the others, each pair ascending.
// Written with register selects (no indexed local arrays).
template <int W>
__device__ __forceinline__ void arrange4(const int *o, const uint64_t *s1, int &a0, int &a1, int &b0, int &b1) {
    int na = 0, nb = 0;
    a0 = a1 = b0 = b1 = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (has_bit<W>(s1, o[k])) {
            if (na == 0) a0 = o[k]; else a1 = o[k];
            ++na;
        } else {
            if (nb == 0) b0 = o[k]; else b1 = o[k];
            ++nb;
        }
    }
}

// two_diff_orbitals(s1, s2) (CIMethod.cpp:429-442): same-spin double
template <int W>
__device__ __forceinline__ double two_diff_same(const DetParams &p, const uint64_t *s1, const uint64_t *s2) {
    uint64_t x[W], c[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        x[w] = s1[w] ^ s2[w];
        c[w] = s1[w] & s2[w];
    }
    int o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = pop_lowest<W>(x);
    int a0, a1, b0, b1;
    arrange4<W>(o, s1, a0, a1, b0, b1);
    const int diff = nstacked<W>(a0, a1, c) + nstacked<W>(b0, b1, c);
    double e = Vm(p, a0, a1, b0, b1) - Vm(p, a0, a1, b1, b0);
    return negate_if(e, diff & 1);
}

// two_diff_orbitals(u1, u2, d1, d2) (CIMethod.cpp:444-457): alpha-beta double
template <int W>
__device__ __forceinline__ double two_diff_ab(const DetParams &p, const uint64_t *u1, const uint64_t *u2, const uint64_t *d1,
                              const uint64_t *d2) {
    uint64_t xu[W], cu[W], xd[W], cd[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        xu[w] = u1[w] ^ u2[w];
        cu[w] = u1[w] & u2[w];
        xd[w] = d1[w] ^ d2[w];
        cd[w] = d1[w] & d2[w];
    }
    // arrange_order with two orbitals: the one occupied in the first string first
    int a0 = pop_lowest<W>(xu), a1 = pop_lowest<W>(xu);
    if (!has_bit<W>(u1, a0)) {
        const int t = a0;
        a0 = a1;
        a1 = t;
    }
    int b0 = pop_lowest<W>(xd), b1 = pop_lowest<W>(xd);
    if (!has_bit<W>(d1, b0)) {
        const int t = b0;
        b0 = b1;
        b1 = t;
    }
    const int diff = nstacked<W>(a0, a1, cu) + nstacked<W>(b0, b1, cd);
    double e = Vm(p, a0, b0, a1, b1);
    return negate_if(e, diff & 1);
}

// get_ham_element (CIMethod.cpp:459-487), the off-diagonal cases
template <int W>
__device__ __forceinline__ double element(const DetParams &p, const uint64_t *u1, const uint64_t *d1,
                                          const uint64_t *u2, const uint64_t *d2, int nu, int nd) {
    if (nd > 4 || nu > 4) return 0.0;
    if (nu == 4 && nd == 0) return two_diff_same<W>(p, u1, u2);
    if (nu == 2) {
        if (nd == 0) return one_diff<W>(p, u1, u2, d1);
        if (nd == 2) return two_diff_ab<W>(p, u1, u2, d1, d2);
        return 0.0;
    }
    if (nd == 4 && nu == 0) return two_diff_same<W>(p, d1, d2);
    if (nd == 2 && nu == 0) return one_diff<W>(p, d1, d2, u1);
    return 0.0;
}

template <int W>
__global__ void k_dets_diag(DetParams p, double *diag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t *d = p.dets + i * 2 * W;
        diag[i] = diagonal<W>(p, d, d + W);
    }
}

// RANGED: a stored block smaller than the list (CI_Big with a kept part), whose
// passes skip columns outside their range; the whole-list passes carry no test.
template <int W, int MODE, bool RANGED>
__global__ void __launch_bounds__(32 * kDetWarps) k_dets_rows(DetParams p, const double *__restrict__ x,
                                                              double *__restrict__ y) {
    __shared__ uint64_t tile[kDetTile * 2 * W];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    constexpr bool kStoring = MODE != kDetMatvec;
    for (int64_t r0 = (int64_t)blockIdx.x * kDetWarps; r0 < p.nrows; r0 += (int64_t)gridDim.x * kDetWarps) {
        const int64_t i = r0 + warp;
        const bool active = i < p.nrows;
        // this row's columns [cs, ce): a stored pass takes those of the block; the
        // matvec of a partly stored matrix takes those outside it
        const int64_t cs = (RANGED && !kStoring && i < p.block) ? p.block : 0, ce = kStoring ? p.block : p.n;
        // the warps' common start (rows of one pass below the block skip it together)
        const int64_t cs_all = (RANGED && !kStoring && r0 + kDetWarps <= p.block) ? p.block : 0;
        uint64_t ui[W], di[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            ui[w] = active ? p.dets[i * 2 * W + w] : 0;
            di[w] = active ? p.dets[i * 2 * W + W + w] : 0;
        }
        uint32_t cnt = 0, lower = 0;
        int64_t out = (MODE == kDetFill64 || MODE == kDetFill32) && active ? p.row_ptr[i] : 0;
        double acc = 0;
        const int64_t cend = kStoring ? p.block : p.n;  // the same for every row of the pass
        for (int64_t base = cs_all; base < cend; base += kDetTile) {
            const int tn = (int)(cend - base < kDetTile ? cend - base : kDetTile);
            __syncthreads();
            for (int t = threadIdx.x; t < tn * 2 * W; t += blockDim.x) tile[t] = p.dets[base * 2 * W + t];
            __syncthreads();
            if (!active) continue;
            for (int jj0 = 0; jj0 < tn; jj0 += 32) {
                const int jj = jj0 + lane;
                const int64_t j = base + jj;
                double v = 0;
                bool keep = false;
                if (jj < tn && (!RANGED || (j >= cs && j < ce))) {
                    const uint64_t *uj = tile + jj * 2 * W, *dj = uj + W;
                    int nu = 0, nd = 0;
#pragma unroll
                    for (int w = 0; w < W; ++w) {
                        nu += __popcll(ui[w] ^ uj[w]);
                        nd += __popcll(di[w] ^ dj[w]);
                    }
                    if (nu + nd <= 4) {
                        // the row itself, or a repeat of its determinant in the list, is the diagonal
                        v = (nu + nd == 0) ? p.diag[i] : element<W>(p, ui, di, uj, dj, nu, nd);
                        keep = keep_value(v);
                    }
                }
                if (MODE == kDetCount) {
                    cnt += keep;
                    lower += keep && j < i;
                } else if (MODE == kDetMatvec) {
                    if (keep) acc = fma(v, x[j], acc);
                } else {
                    const unsigned m = __ballot_sync(0xffffffffu, keep);
                    if (keep) {
                        const int64_t pos = out + __popc(m & below);
                        p.col[pos] = (uint32_t)j;
                        if (MODE == kDetFill64) {
                            p.val64[pos] = v;
                        } else {
                            split_fp32(v, p.val32[pos], p.val32lo[pos]);
                        }
                    }
                    out += __popc(m);
                }
            }
        }
        if (!active) continue;
        if (MODE == kDetCount) {
            for (int o = 16; o > 0; o >>= 1) {
                cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
                lower += __shfl_xor_sync(0xffffffffu, lower, o);
            }
            if (lane == 0) {
                p.row_count[i] = cnt;
                p.upper_off[i] = lower;
            }
        } else if (MODE == kDetMatvec) {
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            // rows of the stored block add to the stored block's product, already in y
            if (lane == 0) y[i] = ((RANGED && i < p.block) ? y[i] : 0.0) + acc;
        }
    }
}

__global__ void k_sum_u32(const uint32_t *a, int64_t n, unsigned long long *out) {
    unsigned long long s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += a[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);  // integer sum: exact in any order
}

int rows_grid(int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + kDetWarps - 1) / kDetWarps, (int64_t)sm_count() * 16));
}

template <int W, int MODE>
void launch_rows(const DetParams &p, const double *x, double *y, cudaStream_t s) {
    if (p.nrows == 0) return;
    // the matvec of a partly stored list, or the stored passes of a block smaller than it
    const bool ranged = MODE == kDetMatvec ? (p.block > 0 && p.block < p.n) : p.block < p.n;
    if (ranged)
        k_dets_rows<W, MODE, true><<<rows_grid(p.nrows), 32 * kDetWarps, 0, s>>>(p, x, y);
    else
        k_dets_rows<W, MODE, false><<<rows_grid(p.nrows), 32 * kDetWarps, 0, s>>>(p, x, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

template <int MODE>
void rows(const DetParams &p, int W, const double *x, double *y, cudaStream_t s) {
    if (W == 1)
        launch_rows<1, MODE>(p, x, y, s);
    else
        launch_rows<2, MODE>(p, x, y, s);
}

DetParams params_of(const cigpu_crs &c) {
    DetParams p{};
    p.L = c.L;
    p.nup = c.nup;
    p.ndown = c.ndown;
    p.n = c.dim;
    p.dets = c.dets.p;
    p.eri = c.ham->d_eri.p;
    p.h = c.ham->d_h.p;
    p.diag = c.diag.p;
    p.nrows = c.dim;
    p.block = c.onthefly ? c.det_block : c.dim;
    return p;
}

// one line of a determinant file: "<up bits>|<down bits>", most significant orbital first
bool parse_line(const std::string &line, int words, uint64_t *up, uint64_t *down, int *nbits) {
    const size_t bar = line.find('|');
    if (bar == std::string::npos) return false;
    auto parse = [&](const std::string &s, uint64_t *out) {
        for (int w = 0; w < words; ++w) out[w] = 0;
        int bit = 0;
        for (size_t k = s.size(); k-- > 0;) {
            const char ch = s[k];
            if (ch == '0' || ch == '1') {
                if (bit >= 64 * words) return -1;
                if (ch == '1') out[bit >> 6] |= (uint64_t)1 << (bit & 63);
                ++bit;
            } else if (ch != ' ' && ch != '\t' && ch != '\r') {
                return -1;
            }
        }
        return bit;
    };
    const int a = parse(line.substr(0, bar), up), b = parse(line.substr(bar + 1), down);
    if (a <= 0 || b <= 0) return false;
    *nbits = std::max(a, b);
    return true;
}

// ---------------------------------------------------------------------------
// RDMs of a list's state (DensFILE::construct_CI_one_dens / construct_CI_two_dens,
// CIDens.cpp:1468-1529): every pair i <= j contributes c_i c_j through the
// reference's fill rules (fill_density_matrix_one / fill_density_matrix,
// CIDens.cpp:676-896) into the symmetric (min, max) storage of CIDens. The sums are
// accumulated as 64-bit fixed-point integers (value * 2^60, rounded to nearest) with
// integer atomics: integer addition is associative, so the result does not depend on
// the order the warps reach an element (bit-identical runs), and two's-complement
// wrap-around keeps every final sum exact while it lies within +-8 (RDM elements lie
// within +-1). Each contribution is rounded by at most 2^-61.
struct RdmAcc {
    unsigned long long *one, *aa, *ab, *bb;
    int L, np;
    bool two;
};

__device__ __forceinline__ void acc_add(unsigned long long *at, double v) {
    atomicAdd(at, (unsigned long long)__double2ll_rn(v * 0x1p60));
}
__device__ __forceinline__ void rdm_add_one(const RdmAcc &R, int spin, int o1, int o2, double v) {
    const int a = min(o1, o2), b = max(o1, o2);
    acc_add(R.one + ((int64_t)spin * R.L + a) * R.L + b, v);
}
// add_two_rdm (CIDens.cpp:227-256)
__device__ __forceinline__ void rdm_add_two(const RdmAcc &R, int spin, int o1, int o2, int o3, int o4, double v) {
    const int L = R.L;
    if (spin == 1) {
        const int64_t A = (int64_t)o1 * L + o2, B = (int64_t)o3 * L + o4;
        acc_add(R.ab + min(A, B) * (int64_t)L * L + max(A, B), v);
        return;
    }
    if (o1 == o2 || o3 == o4) return;
    int odd = 0;
    if (o1 > o2) {
        const int t = o1;
        o1 = o2;
        o2 = t;
        odd ^= 1;
    }
    if (o3 > o4) {
        const int t = o3;
        o3 = o4;
        o4 = t;
        odd ^= 1;
    }
    const int64_t A = o1 * L + o2 - (o1 + 1) * (o1 + 2) / 2, B = o3 * L + o4 - (o3 + 1) * (o3 + 2) / 2;
    acc_add((spin == 0 ? R.aa : R.bb) + min(A, B) * R.np + max(A, B), negate_if(v, odd));
}

// fill_one_dense (CIDens.cpp:676-754) for strings b1 -> b2 differing in one orbital;
// `same` is the other spin's string. alpha: the moved electron is alpha.
template <int W>
__device__ void fill_single(const RdmAcc &R, const uint64_t *b1, const uint64_t *b2, const uint64_t *same, double contr,
                            bool alpha) {
    uint64_t x[W], c[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        x[w] = b1[w] ^ b2[w];
        c[w] = b1[w] & b2[w];
    }
    const int o0 = pop_lowest<W>(x), o1 = pop_lowest<W>(x);
    contr = negate_if(contr, nstacked<W>(o0, o1, c) & 1);
    rdm_add_one(R, alpha ? 0 : 1, o0, o1, contr);
    if (!R.two) return;
#pragma unroll
    for (int w = 0; w < W; ++w)
        for (uint64_t y = c[w]; y; y &= y - 1) {
            const int z = 64 * w + __ffsll((long long)y) - 1;
            rdm_add_two(R, alpha ? 0 : 2, o0, z, o1, z, contr);
        }
#pragma unroll
    for (int w = 0; w < W; ++w)
        for (uint64_t y = same[w]; y; y &= y - 1) {
            const int z = 64 * w + __ffsll((long long)y) - 1;
            if (alpha)
                rdm_add_two(R, 1, o0, z, o1, z, contr);
            else
                rdm_add_two(R, 1, z, o0, z, o1, contr);
        }
}

// fill_two_dense (CIDens.cpp:756-779): a same-spin double
template <int W>
__device__ void fill_double_same(const RdmAcc &R, const uint64_t *s1, const uint64_t *s2, double contr, int spin) {
    uint64_t x[W], c[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        x[w] = s1[w] ^ s2[w];
        c[w] = s1[w] & s2[w];
    }
    int o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = pop_lowest<W>(x);
    int a0, a1, b0, b1;
    arrange4<W>(o, s1, a0, a1, b0, b1);
    const int diff = nstacked<W>(a0, a1, c) + nstacked<W>(b0, b1, c);
    rdm_add_two(R, spin, a0, a1, b0, b1, negate_if(contr, diff & 1));
}

// fill_two_dense_upanddown (CIDens.cpp:781-806): an alpha-beta double
template <int W>
__device__ void fill_double_ab(const RdmAcc &R, const uint64_t *u1, const uint64_t *u2, const uint64_t *d1,
                               const uint64_t *d2, double contr) {
    uint64_t xu[W], cu[W], xd[W], cd[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        xu[w] = u1[w] ^ u2[w];
        cu[w] = u1[w] & u2[w];
        xd[w] = d1[w] ^ d2[w];
        cd[w] = d1[w] & d2[w];
    }
    int a0 = pop_lowest<W>(xu), a1 = pop_lowest<W>(xu);
    if (!has_bit<W>(u1, a0)) {
        const int t = a0;
        a0 = a1;
        a1 = t;
    }
    int b0 = pop_lowest<W>(xd), b1 = pop_lowest<W>(xd);
    if (!has_bit<W>(d1, b0)) {
        const int t = b0;
        b0 = b1;
        b1 = t;
    }
    const int diff = nstacked<W>(a0, a1, cu) + nstacked<W>(b0, b1, cd);
    rdm_add_two(R, 1, a0, b0, a1, b1, negate_if(contr, diff & 1));
}

// fill_diagonal (CIDens.cpp:808-853)
template <int W>
__device__ void fill_diag(const RdmAcc &R, const uint64_t *up, const uint64_t *dn, double contr) {
#pragma unroll
    for (int w = 0; w < W; ++w)
        for (uint64_t y = up[w]; y; y &= y - 1) rdm_add_one(R, 0, 64 * w + __ffsll((long long)y) - 1, 64 * w + __ffsll((long long)y) - 1, contr);
#pragma unroll
    for (int w = 0; w < W; ++w)
        for (uint64_t y = dn[w]; y; y &= y - 1) rdm_add_one(R, 1, 64 * w + __ffsll((long long)y) - 1, 64 * w + __ffsll((long long)y) - 1, contr);
    if (!R.two) return;
    for (int spin = 0; spin < 2; ++spin) {
        const uint64_t *s = spin == 0 ? up : dn;
#pragma unroll
        for (int w = 0; w < W; ++w)
            for (uint64_t y = s[w]; y; y &= y - 1) {
                const int i = 64 * w + __ffsll((long long)y) - 1;
                // partners j > i
#pragma unroll
                for (int w2 = 0; w2 < W; ++w2) {
                    uint64_t y2 = s[w2];
                    if (w2 == w) y2 &= y & (y - 1);  // bits above i in the same word
                    else if (w2 < w) y2 = 0;
                    for (; y2; y2 &= y2 - 1) {
                        const int j = 64 * w2 + __ffsll((long long)y2) - 1;
                        rdm_add_two(R, spin == 0 ? 0 : 2, i, j, i, j, contr);
                    }
                }
            }
    }
#pragma unroll
    for (int w = 0; w < W; ++w)
        for (uint64_t y = up[w]; y; y &= y - 1) {
            const int i = 64 * w + __ffsll((long long)y) - 1;
#pragma unroll
            for (int w2 = 0; w2 < W; ++w2)
                for (uint64_t y2 = dn[w2]; y2; y2 &= y2 - 1) {
                    const int j = 64 * w2 + __ffsll((long long)y2) - 1;
                    rdm_add_two(R, 1, i, j, i, j, contr);
                }
        }
}

template <int W>
__global__ void __launch_bounds__(32 * kDetWarps) k_dets_rdm(DetParams p, const double *__restrict__ c, RdmAcc R) {
    __shared__ uint64_t tile[kDetTile * 2 * W];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t r0 = (int64_t)blockIdx.x * kDetWarps; r0 < p.n; r0 += (int64_t)gridDim.x * kDetWarps) {
        const int64_t i = r0 + warp;
        const bool active = i < p.n;
        uint64_t ui[W], di[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            ui[w] = active ? p.dets[i * 2 * W + w] : 0;
            di[w] = active ? p.dets[i * 2 * W + W + w] : 0;
        }
        const double ci = active ? c[i] : 0.0;
        // columns j >= i: tiles from the one holding i
        for (int64_t base = (r0 / kDetTile) * kDetTile; base < p.n; base += kDetTile) {
            const int tn = (int)(p.n - base < kDetTile ? p.n - base : kDetTile);
            __syncthreads();
            for (int t = threadIdx.x; t < tn * 2 * W; t += blockDim.x) tile[t] = p.dets[base * 2 * W + t];
            __syncthreads();
            if (!active) continue;
            for (int jj = lane; jj < tn; jj += 32) {
                const int64_t j = base + jj;
                if (j < i) continue;
                const uint64_t *uj = tile + jj * 2 * W, *dj = uj + W;
                int nu = 0, nd = 0;
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    nu += __popcll(ui[w] ^ uj[w]);
                    nd += __popcll(di[w] ^ dj[w]);
                }
                if (nu + nd > 4) continue;
                const double contr = ci * c[j];
                // fill_density_matrix_one / fill_density_matrix (CIDens.cpp:855-896)
                if (nu == 0 && nd == 0) fill_diag<W>(R, ui, di, contr);
                else if (nu == 2 && nd == 0) fill_single<W>(R, ui, uj, di, contr, true);
                else if (nu == 0 && nd == 2) fill_single<W>(R, di, dj, ui, contr, false);
                else if (R.two && nu == 4 && nd == 0) fill_double_same<W>(R, ui, uj, contr, 0);
                else if (R.two && nu == 0 && nd == 4) fill_double_same<W>(R, di, dj, contr, 2);
                else if (R.two && nu == 2 && nd == 2) fill_double_ab<W>(R, ui, uj, di, dj, contr);
            }
        }
    }
}

// Expands the (min, max) fixed-point storage into the full symmetric output arrays.
__global__ void k_rdm_expand(RdmAcc R, double *rdm1, double *aa, double *ab, double *bb) {
    const int L = R.L, np = R.np;
    const int64_t L2 = (int64_t)L * L, n1 = 2 * L2, n2 = (int64_t)np * np, n3 = L2 * L2;
    const int64_t total = n1 + (R.two ? 2 * n2 + n3 : 0);
    auto val = [](unsigned long long q) { return (double)(long long)q * 0x1p-60; };
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        if (t < n1) {
            const int64_t s = t / L2, ij = t - s * L2;
            const int i = (int)(ij / L), j = (int)(ij - (int64_t)i * L);
            rdm1[t] = val(R.one[(s * L + min(i, j)) * L + max(i, j)]);
        } else if (t < n1 + 2 * n2) {
            const int64_t u = t - n1, which = u / n2, ij = u - which * n2;
            const int64_t i = ij / np, j = ij - i * np;
            const unsigned long long *X = which == 0 ? R.aa : R.bb;
            (which == 0 ? aa : bb)[ij] = val(X[min(i, j) * np + max(i, j)]);
        } else {
            const int64_t ij = t - n1 - 2 * n2, i = ij / L2, j = ij - i * L2;
            ab[ij] = val(R.ab[min(i, j) * L2 + max(i, j)]);
        }
    }
}

}  // namespace

void dets_rdm(cigpu_crs &c, const double *c_dev, double *rdm1, double *aa, double *ab, double *bb, cudaStream_t s) {
    const int L = c.L, np = L * (L - 1) / 2;
    const int64_t L2 = (int64_t)L * L, n1 = 2 * L2, n2 = (int64_t)np * np, n3 = L2 * L2;
    const bool two = aa && ab && bb;
    DevBuf<unsigned long long> acc(n1 + (two ? 2 * n2 + n3 : 0));
    CIGPU_CUDA(cudaMemsetAsync(acc.p, 0, acc.bytes(), s));
    RdmAcc R{acc.p, two ? acc.p + n1 : nullptr, two ? acc.p + n1 + 2 * n2 : nullptr, two ? acc.p + n1 + n2 : nullptr,
             L, np, two};
    DetParams p = params_of(c);
    if (c.det_words == 1)
        k_dets_rdm<1><<<rows_grid(c.dim), 32 * kDetWarps, 0, s>>>(p, c_dev, R);
    else
        k_dets_rdm<2><<<rows_grid(c.dim), 32 * kDetWarps, 0, s>>>(p, c_dev, R);
    CIGPU_CUDA(cudaGetLastError());
    DevBuf<double> out(n1 + (two ? 2 * n2 + n3 : 0));
    double *o1 = out.p, *oaa = two ? out.p + n1 : nullptr, *obb = two ? out.p + n1 + n2 : nullptr,
           *oab = two ? out.p + n1 + 2 * n2 : nullptr;
    const int64_t total = (int64_t)out.n;
    k_rdm_expand<<<(int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 8), 256, 0, s>>>(R, o1, oaa, oab, obb);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(2);
    if (rdm1) CIGPU_CUDA(cudaMemcpyAsync(rdm1, o1, sizeof(double) * n1, cudaMemcpyDeviceToHost, s));
    if (two) {
        CIGPU_CUDA(cudaMemcpyAsync(aa, oaa, sizeof(double) * n2, cudaMemcpyDeviceToHost, s));
        CIGPU_CUDA(cudaMemcpyAsync(bb, obb, sizeof(double) * n2, cudaMemcpyDeviceToHost, s));
        CIGPU_CUDA(cudaMemcpyAsync(ab, oab, sizeof(double) * n3, cudaMemcpyDeviceToHost, s));
    }
    CIGPU_CUDA(cudaStreamSynchronize(s));
}

void dets_mv64(cigpu_crs &c, const double *x, double *y, cudaStream_t s) {
    DetParams p = params_of(c);
    // the stored leading block first (rows and columns below det_block), then every
    // pair outside it recomputed (CI_Big::mvprod, CIMethod.cpp:943-984)
    if (c.det_block > 0) spmv_f64(c.det_block, c.nnz_full, c.row_ptr.p, c.col.p, c.val64.p, x, y, s);
    if (c.det_block < c.dim) rows<kDetMatvec>(p, c.det_words, x, y, s);  // nothing outside a whole-list block
}

}  // namespace cigpu

using namespace cigpu;

extern "C" {

int cigpu_dets_read(const char *path, int words, int64_t capacity, uint64_t *up, uint64_t *down, int64_t *ndet,
                    int *max_orbitals) {
    if (!path || !ndet || (words != 1 && words != 2) || capacity < 0) return CIGPU_EINVAL;
    std::ifstream f(path);
    if (!f.is_open()) return CIGPU_ENOTFOUND;
    std::string line;
    int64_t n = 0;
    int maxb = 0;
    uint64_t u[2], d[2];
    while (std::getline(f, line)) {
        if (line.find('#') != std::string::npos) continue;  // Permutator_File::read_file skips comment lines
        if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
        int nb = 0;
        if (!parse_line(line, words, u, d, &nb)) return CIGPU_EINVAL;
        maxb = std::max(maxb, nb);
        if (up && down && n < capacity) {
            for (int w = 0; w < words; ++w) {
                up[n * words + w] = u[w];
                down[n * words + w] = d[w];
            }
        }
        ++n;
    }
    *ndet = n;
    if (max_orbitals) *max_orbitals = maxb;
    return (up && down && n > capacity) ? CIGPU_ENOMEM : CIGPU_OK;
}

}  // extern "C"

namespace cigpu {
namespace {

// keep: the leading determinants whose block of the matrix is stored (all of them
// for CRS storage; 0 for CI_Big without a stored part)
int build_dets(cigpu_ham *ham, int64_t ndet, int words, const uint64_t *up, const uint64_t *down, int storage,
               int precision, int64_t keep, cigpu_stream stream, cigpu_crs **out) {
    if (!ham || !up || !down || !out) return CIGPU_EINVAL;
    *out = nullptr;
    if (ndet < 1 || ndet > (int64_t)UINT32_MAX || (words != 1 && words != 2)) return CIGPU_EINVAL;
    if (storage != CIGPU_DETS_CRS && storage != CIGPU_DETS_ONTHEFLY) return CIGPU_EINVAL;
    if (precision != CIGPU_FP64 && precision != CIGPU_MIXED) return CIGPU_EINVAL;
    if (storage == CIGPU_DETS_ONTHEFLY && precision != CIGPU_FP64) return CIGPU_ENOTSUP;
    if (keep < 0 || keep > ndet) return CIGPU_EINVAL;
    const int W = ham->L <= 64 ? 1 : 2;
    if (words < W) return CIGPU_EINVAL;
    // every determinant: nup / ndown electrons inside the L orbitals (the reference
    // takes the counts from the Hamiltonian and assumes them)
    std::vector<uint64_t> rec((size_t)ndet * 2 * W, 0);
    for (int64_t i = 0; i < ndet; ++i) {
        int cu = 0, cd = 0;
        for (int w = 0; w < words; ++w) {
            const uint64_t u = up[i * words + w], d = down[i * words + w];
            const int lo = 64 * w;
            const uint64_t valid = ham->L - lo >= 64 ? ~(uint64_t)0 : (ham->L - lo <= 0 ? 0 : (((uint64_t)1 << (ham->L - lo)) - 1));
            if ((u & ~valid) || (d & ~valid)) return CIGPU_EINVAL;
            cu += __builtin_popcountll(u);
            cd += __builtin_popcountll(d);
            if (w < W) {
                rec[(size_t)i * 2 * W + w] = u;
                rec[(size_t)i * 2 * W + W + w] = d;
            }
        }
        if (cu != ham->nup || cd != ham->ndown) return CIGPU_EINVAL;
    }
    CIGPU_TRY
    std::unique_ptr<cigpu_crs> c(new cigpu_crs);
    c->ham = ham;
    c->method = CIGPU_DETS;
    c->precision = precision;
    c->L = ham->L;
    c->nup = ham->nup;
    c->ndown = ham->ndown;
    c->dim = ndet;
    c->det_words = W;
    c->onthefly = storage == CIGPU_DETS_ONTHEFLY;
    c->det_block = c->onthefly ? keep : ndet;
    CIGPU_CUDA(cudaGetDevice(&c->device));
    if (stream) {
        c->stream = static_cast<cudaStream_t>(stream);
    } else {
        CIGPU_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    cudaStream_t s = c->stream;
    StreamScope scope(s);
    const auto t0 = std::chrono::steady_clock::now();
    c->dets.alloc(rec.size());
    CIGPU_CUDA(cudaMemcpyAsync(c->dets.p, rec.data(), rec.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    c->diag.alloc(ndet);
    DetParams p = params_of(*c);
    {
        const int g = (int)std::max<int64_t>(1, std::min<int64_t>((ndet + 255) / 256, (int64_t)sm_count() * 8));
        if (W == 1)
            k_dets_diag<1><<<g, 256, 0, s>>>(p, c->diag.p);
        else
            k_dets_diag<2><<<g, 256, 0, s>>>(p, c->diag.p);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
    }
    if (c->det_block > 0) {
        // the stored rows: the whole matrix (CRS storage) or the leading block of CI_Big
        const int64_t nb = c->det_block;
        p.nrows = nb;
        p.block = nb;
        DevBuf<uint32_t> count(nb);
        c->upper_off.alloc(nb);
        c->row_ptr.alloc(nb + 1);
        p.row_count = count.p;
        p.upper_off = c->upper_off.p;
        rows<kDetCount>(p, W, nullptr, nullptr, s);
        exclusive_scan_u32(count.p, c->row_ptr.p, nb, s);
        DevBuf<unsigned long long> lower(1);
        CIGPU_CUDA(cudaMemsetAsync(lower.p, 0, sizeof(unsigned long long), s));
        k_sum_u32<<<(int)std::min<int64_t>((nb + 255) / 256, 1024), 256, 0, s>>>(c->upper_off.p, nb, lower.p);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
        int64_t nnz = 0;
        unsigned long long nlow = 0;
        CIGPU_CUDA(cudaMemcpyAsync(&nnz, c->row_ptr.p + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        CIGPU_CUDA(cudaMemcpyAsync(&nlow, lower.p, sizeof(nlow), cudaMemcpyDeviceToHost, s));
        CIGPU_CUDA(cudaStreamSynchronize(s));
        c->nnz_full = nnz;
        c->nnz_upper = nnz - (int64_t)nlow;
        c->col.alloc(std::max<int64_t>(nnz, 1));
        p.row_ptr = c->row_ptr.p;
        p.col = c->col.p;
        if (precision == CIGPU_FP64) {
            c->val64.alloc(std::max<int64_t>(nnz, 1));
            p.val64 = c->val64.p;
            rows<kDetFill64>(p, W, nullptr, nullptr, s);
        } else {
            c->val32.alloc(std::max<int64_t>(nnz, 1));
            c->val32lo.alloc(std::max<int64_t>(nnz, 1));
            p.val32 = c->val32.p;
            p.val32lo = c->val32lo.p;
            rows<kDetFill32>(p, W, nullptr, nullptr, s);
        }
    }
    CIGPU_CUDA(cudaStreamSynchronize(s));
    c->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = c.release();
    return CIGPU_OK;
    CIGPU_CATCH
}

}  // namespace
}  // namespace cigpu

extern "C" {

int cigpu_build_dets(cigpu_ham *ham, int64_t ndet, int words, const uint64_t *up, const uint64_t *down, int storage,
                     int precision, cigpu_stream stream, cigpu_crs **out) {
    return build_dets(ham, ndet, words, up, down, storage, precision, storage == CIGPU_DETS_CRS ? ndet : 0, stream,
                      out);
}

int cigpu_build_dets_partial(cigpu_ham *ham, int64_t ndet, int words, const uint64_t *up, const uint64_t *down,
                             int64_t keep, cigpu_stream stream, cigpu_crs **out) {
    return build_dets(ham, ndet, words, up, down, CIGPU_DETS_ONTHEFLY, CIGPU_FP64, keep, stream, out);
}

}  // extern "C"
