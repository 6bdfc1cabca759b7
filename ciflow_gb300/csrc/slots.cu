// Values-only FCI layout of the mixed method ("slot tiles") and its matvec.
//
// Every FCI row has the same structural width W = (1 + ns_b + nd_b) + ns_a (1 + ns_b)
// + nd_a, and the meaning of each slot can be made the same for every row by
// ordering a row's slots by excitation kind rather than by column:
//   [alpha self]    beta self, beta singles xb = 0..ns_b-1, beta doubles xb = 0..nd_b-1
//   [alpha single xa, xa = 0..ns_a-1]    beta self, beta singles xb
//   [alpha double xa, xa = 0..nd_a-1]    beta self
// (xa, xb index a string's singles/doubles in the order of its string tables). The
// column of slot (alpha kind, xa, beta kind, xb) in row (Ia, Ib) is Ja * Db + Jb with
// Ja = Ia or the xa-th alpha single/double target of Ia and Jb = Ib or the xb-th beta
// single/double target of Ib, so no column index is stored: 4 bytes per element in
// FP32 instead of the 8 of an FP32 CRS, 8 instead of 12 for the FP64 product from
// the split values.
//
// Rows are grouped in tiles of kTileRows consecutive beta strings of one alpha
// string; a tile stores its values slot-major, val[(tile * W + k) * kTileRows + row],
// so a warp (32 rows) reads one slot of 32 rows with one coalesced 128-byte load and
// every lane of the warp executes the same slot kind. The x entries a slot reads all
// lie in the panel x[Ja * Db .. Ja * Db + Db) of one alpha string (L1-resident while
// the slot run lasts). Elements with |v| <= 1e-14 are stored as zero; padding rows
// of the last tile are zero and never written back.
//
// Replaces SparseMatrix_CRS_Sym::mvprod (SparseMatrix_CRS.cpp:700-723) for the FP32
// values of the mixed method; the build below produces the same element values as
// the CRS generator (build.cu), in slot order.
#include <algorithm>

#include "slots.cuh"
#include "spmv_formats.cuh"

namespace cigpu {

namespace {

constexpr int kSlotThreads = 256;  // 2 row halves x 4 slot quarters
constexpr int kSplits = 4;

// Walks slots [k0, k1) in homogeneous runs: v.run(kindA, xa, kindB, xb0, xb1, k)
// covers slots k .. k + (xb1 - xb0) - 1.
template <typename V>
__device__ __forceinline__ void walk_slots(const FciParams &p, int k0, int k1, V &v) {
    const int nsa = p.a.ns, nda = p.a.nd, nsb = p.b.ns, ndb = p.b.nd;
    const int WA = 1 + nsb + ndb, WS = 1 + nsb;
    const int kS = WA, kD = WA + nsa * WS;
    auto piece = [&](int kindA, int xa, int kindB, int xb_first, int k_first, int len) {
        const int a = max(k_first, k0), b = min(k_first + len, k1);
        if (a < b) v.run(kindA, xa, kindB, xb_first + (a - k_first), xb_first + (b - k_first), a);
    };
    if (k0 < WA) {
        piece(kSelf, 0, kSelf, 0, 0, 1);
        piece(kSelf, 0, kSingle, 0, 1, nsb);
        piece(kSelf, 0, kDouble, 0, 1 + nsb, ndb);
    }
    if (k1 > kS && k0 < kD) {
        const int x0 = max(0, (k0 - kS) / WS), x1 = min(nsa, (k1 - kS + WS - 1) / WS);
        for (int xa = x0; xa < x1; ++xa) {
            const int kb = kS + xa * WS;
            piece(kSingle, xa, kSelf, 0, kb, 1);
            piece(kSingle, xa, kSingle, 0, kb + 1, nsb);
        }
    }
    if (k1 > kD) {  // alpha doubles: one slot per xa, passed as one run over xa
        const int a = max(k0, kD), b = min(k1, kD + nda);
        if (a < b) v.run(kDouble, a - kD, kSelf, 0, b - a, a);
    }
}

// ---------------------------------------------------------------------------
// Matvec. Block = one tile; warp w: rows (w & 1) * 32 + lane, slot quarter w >> 1.
template <typename F>
struct MatvecRun {
    const FciParams &p;
    const F &f;
    const uint32_t *st;  // [nsb][kTileRows] beta single targets of the tile rows (shared)
    int64_t ia, ib, vbase;
    int rr;
    typename F::Acc acc;
    __device__ __forceinline__ void run(int kindA, int xa, int kindB, int xb0, int xb1, int k) {
        int64_t Ja = ia;
        if (kindA == kSingle) Ja = __ldg(p.a.s_target + ia * p.a.ns + xa);
        if (kindA == kDouble) {
            // alpha doubles: one slot per xa, beta self
            for (int xd = xb0; xd < xb1; ++xd, ++k) {
                const int64_t J = __ldg(p.a.d_target + ia * p.a.nd + xa + (xd - xb0));
                f.term1(vbase + (int64_t)k * kTileRows, J * p.Db + ib, acc);
            }
            return;
        }
        const int64_t pan = Ja * p.Db;  // x panel of alpha string Ja
        if (kindB == kSelf) {
            f.term1(vbase + (int64_t)k * kTileRows, pan + ib, acc);
        } else if (kindB == kSingle) {
#pragma unroll 4
            for (int xb = xb0; xb < xb1; ++xb, ++k)
                f.term1(vbase + (int64_t)k * kTileRows, pan + st[xb * kTileRows + rr], acc);
        } else {
            const uint32_t *dt = p.b.d_target + ib * p.b.nd;
#pragma unroll 4
            for (int xb = xb0; xb < xb1; ++xb, ++k)
                f.term1(vbase + (int64_t)k * kTileRows, pan + __ldg(dt + xb), acc);
        }
    }
};

template <typename F>
__global__ void __launch_bounds__(kSlotThreads) k_spmv_slots(const FciParams p, const F f,
                                                             typename F::X *__restrict__ y) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *st = reinterpret_cast<uint32_t *>(smem);  // [nsb][kTileRows]
    __shared__ typename F::Acc part[kSplits][kTileRows];
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    const int64_t ia = blockIdx.x / T, t = blockIdx.x - ia * T;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nsb = p.b.ns;
    for (int i = tid; i < nsb * kTileRows; i += blockDim.x) {
        const int xb = i / kTileRows, r = i - xb * kTileRows;
        const int64_t ib = t * kTileRows + r;
        st[i] = ib < p.Db ? __ldg(p.b.s_target + ib * nsb + xb) : 0u;
    }
    __syncthreads();
    const int rr = (warp & 1) * 32 + lane, ks = warp >> 1;
    const int64_t ib_raw = t * kTileRows + rr;
    const bool active = ib_raw < p.Db;
    const int W = fci_row_width(p);
    MatvecRun<F> v{p, f, st, ia, active ? ib_raw : p.Db - 1, (ia * T + t) * (int64_t)W * kTileRows + rr, rr, {}};
    walk_slots(p, (int)((int64_t)W * ks / kSplits), (int)((int64_t)W * (ks + 1) / kSplits), v);
    part[ks][rr] = v.acc;
    __syncthreads();
    if (ks == 0 && active) {
        typename F::Acc s = part[0][rr];
#pragma unroll
        for (int q = 1; q < kSplits; ++q) f.add(s, part[q][rr]);
        y[ia * p.Db + ib_raw] = f.result(s);
    }
}

// ---------------------------------------------------------------------------
// Build: the same element values as the CRS generator, as FP32 hi + lo splits
// (zero where |v| <= 1e-14), written in slot order.
struct FillRun {
    const FciParams &p;
    const float *slhi, *sllo;  // staged (ar ac|. .) slices of the alpha singles
    int64_t ia, ib, r, vbase;
    bool active;
    float *hi_out, *lo_out;
    __device__ __forceinline__ void put(int k, float h, float l) {
        const int64_t at = vbase + (int64_t)k * kTileRows;
        hi_out[at] = active ? h : 0.0f;
        lo_out[at] = active ? l : 0.0f;
    }
    __device__ __forceinline__ void run(int kindA, int xa, int kindB, int xb0, int xb1, int k) {
        const int L = p.L, L2 = L * L;
        const int nsr = p.a.ns + p.b.ns;
        if (kindA == kDouble) {
            for (int xd = xb0; xd < xb1; ++xd, ++k) {
                const size_t at = ia * p.a.nd + xa + (xd - xb0);
                put(k, __ldg(p.a.d_hi + at), __ldg(p.a.d_lo + at));
            }
            return;
        }
        if (kindB == kSelf) {
            if (kindA == kSelf) {
                put(k, p.diag_hi[r], p.diag_lo[r]);
            } else {
                const size_t at = (size_t)r * nsr + xa;  // alpha single (one_diff_orbital)
                put(k, __ldg(p.sgl_hi + at), __ldg(p.sgl_lo + at));
            }
            return;
        }
        if (kindA == kSelf) {
            if (kindB == kSingle) {
                for (int xb = xb0; xb < xb1; ++xb, ++k) {
                    const size_t at = (size_t)r * nsr + p.a.ns + xb;  // beta single
                    put(k, __ldg(p.sgl_hi + at), __ldg(p.sgl_lo + at));
                }
            } else {
                for (int xb = xb0; xb < xb1; ++xb, ++k) {
                    const size_t at = ib * p.b.nd + xb;  // beta-beta double
                    put(k, __ldg(p.b.d_hi + at), __ldg(p.b.d_lo + at));
                }
            }
            return;
        }
        // alpha-beta doubles (ar ac|br bc), sign from both phases (CIMethod.cpp:444-457);
        // the exact 8-fold symmetry of the stored integrals makes it row-independent
        const uint32_t infoA = __ldg(p.a.s_info + ia * p.a.ns + xa);
        const int ar = (infoA >> 12) & 63, ac = (infoA >> 18) & 63;
        for (int xb = xb0; xb < xb1; ++xb, ++k) {
            const uint32_t infoB = __ldg(p.b.s_info + ib * p.b.ns + xb);
            const int tt = ((infoB >> 12) & 63) * L + ((infoB >> 18) & 63);
            const uint32_t odd = ((infoA ^ infoB) >> 24) & 1;
            float h, l;
            if (p.staged) {
                h = slhi[xa * L2 + tt];
                l = sllo[xa * L2 + tt];
            } else {
                const size_t at = ((size_t)ar * L + ac) * L2 + tt;
                h = __ldg(p.eri_hi + at);
                l = __ldg(p.eri_lo + at);
            }
            put(k, __uint_as_float(__float_as_uint(h) ^ (odd << 31)), __uint_as_float(__float_as_uint(l) ^ (odd << 31)));
        }
    }
};

__global__ void __launch_bounds__(kSlotThreads) k_fill_slots(const FciParams p, float *__restrict__ hi,
                                                             float *__restrict__ lo) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int L2 = p.L * p.L, nsa = p.a.ns;
    float *slhi = reinterpret_cast<float *>(smem);
    float *sllo = slhi + (size_t)nsa * L2;
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    const int64_t ia = blockIdx.x / T, t = blockIdx.x - ia * T;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (p.staged) {
        for (int i = tid; i < nsa * L2; i += blockDim.x) {
            const int xa = i / L2, tt = i - xa * L2;
            const uint32_t info = __ldg(p.a.s_info + ia * nsa + xa);
            const int ar = (info >> 12) & 63, ac = (info >> 18) & 63;
            const size_t at = ((size_t)ar * p.L + ac) * L2 + tt;
            slhi[i] = __ldg(p.eri_hi + at);
            sllo[i] = __ldg(p.eri_lo + at);
        }
    }
    __syncthreads();
    const int rr = (warp & 1) * 32 + lane, ks = warp >> 1;
    const int64_t ib_raw = t * kTileRows + rr;
    const bool active = ib_raw < p.Db;
    const int64_t ib = active ? ib_raw : p.Db - 1;
    const int W = fci_row_width(p);
    FillRun v{p, slhi, sllo, ia, ib, ia * p.Db + ib, (ia * T + t) * (int64_t)W * kTileRows + rr, active, hi, lo};
    walk_slots(p, (int)((int64_t)W * ks / kSplits), (int)((int64_t)W * (ks + 1) / kSplits), v);
}

size_t matvec_smem(const FciParams &p) { return (size_t)p.b.ns * kTileRows * 4; }
size_t fill_smem(const FciParams &p) { return (size_t)p.a.ns * p.L * p.L * 8; }  // hi + lo slices

template <typename F>
void launch_slots(const FciParams &p, const F &f, typename F::X *y, cudaStream_t s) {
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_spmv_slots<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotsMaxSmem);
        return true;
    }();
    (void)attr_set;
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    k_spmv_slots<F><<<(unsigned)(p.a.D * T), kSlotThreads, matvec_smem(p), s>>>(p, f, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace

bool slots_supported(const FciParams &p) {
    return matvec_smem(p) <= kSlotsMaxSmem && p.a.D * ((p.Db + kTileRows - 1) / kTileRows) < (int64_t)INT32_MAX &&
           (int64_t)fci_row_width(p) < (int64_t)INT32_MAX / 2;
}

int64_t slots_count(const FciParams &p) {
    return p.a.D * ((p.Db + kTileRows - 1) / kTileRows) * kTileRows * (int64_t)fci_row_width(p);
}

void fill_slots_launch(const FciParams &p0, float *hi, float *lo, cudaStream_t s) {
    FciParams p = p0;
    const size_t sm = fill_smem(p);
    p.staged = sm <= kSlotsMaxSmem ? 1 : 0;
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_fill_slots, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotsMaxSmem);
        return true;
    }();
    (void)attr_set;
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    k_fill_slots<<<(unsigned)(p.a.D * T), kSlotThreads, p.staged ? sm : 0, s>>>(p, hi, lo);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void spmv_slots_f32(const FciParams &p, const float *val, const float *x, float *y, cudaStream_t s) {
    launch_slots(p, Plain<float>{val, x}, y, s);
}

void spmv_slots_hilo(const FciParams &p, const float *hi, const float *lo, const double *x, const float *x32,
                     double *y, cudaStream_t s) {
    launch_slots(p, HiLo{hi, lo, x, x32}, y, s);
}

}  // namespace cigpu
