// Values-only FCI layout of the mixed method ("slot tiles") and its matvec.
//
// Every FCI row has the same structural width W = (1 + ns_b + nd_b) + ns_a (1 + ns_b)
// + nd_a, and the meaning of each slot can be made the same for every row by
// ordering a row's slots by excitation kind rather than by column, in five
// segments, each padded with zero slots to a multiple of 4:
//   S0  alpha self, beta self                         (diagonal)
//   S1  alpha self, beta singles xb = 0..ns_b-1
//   S2  alpha self, beta doubles xb = 0..nd_b-1
//   S3  alpha singles xa = 0..ns_a-1, then alpha doubles, beta self
//   S4  alpha single xa x beta single xb, xa-major    (alpha-beta doubles)
// (xa, xb index a string's singles/doubles in the order of its string tables). The
// column of a slot in row (Ia, Ib) is Ja * Db + Jb with Ja = Ia or the xa-th alpha
// single/double target of Ia and Jb = Ib or the xb-th beta single/double target of
// Ib, so no column index is stored: 4 bytes per element in FP32 instead of the 8 of
// an FP32 CRS, 8 instead of 12 for the FP64 product from the split values.
//
// Rows are grouped in tiles of kTileRows consecutive beta strings of one alpha
// string. Within a tile the values are stored in quads of 4 consecutive slots per
// row, quad-major: val[((tile * Q + c) * kTileRows + row) * 4 + j] for slot 4c + j.
// A warp (32 rows) reads one quad of 32 rows with one fully coalesced 512-byte load,
// 16 bytes per lane; the 4 slots of a quad share their beta kind (the segments are
// quad-aligned), so a quad is one branch-free group of 4 gathers. The slot ->
// (Ja, xb) descriptors of the tile's alpha string sit in shared memory and are read
// as broadcasts; the x entries a slot reads lie in the panel x[Ja * Db, Ja * Db + Db).
// Elements with |v| <= 1e-14 and padding are stored as zero; padding rows of the
// last tile are zero and never written back.
//
// Replaces SparseMatrix_CRS_Sym::mvprod (SparseMatrix_CRS.cpp:700-723) for the FP32
// values of the mixed method. The fill below produces the same element values as
// the CRS generator (build.cu), in slot order, and counts each row's stored
// nonzeros and lower-triangle nonzeros on the way (the CRS row pointers of export).
#include <algorithm>
#include <stdexcept>
#include "slots.cuh"
#include "spmv_formats.cuh"

namespace cigpu {

namespace {

constexpr int kSlotThreads = 256;
constexpr int kPrefetchQuads = 4;  // quads (1 KB of FP32 values each) of a range prefetched to L2 at the start
constexpr int kRowWarps = kTileRows / 32;                // warps covering the tile's rows
constexpr int kSplits = kSlotThreads / 32 / kRowWarps;  // quad ranges per row

__host__ __device__ inline int pad4(int n) { return (n + 3) & ~3; }

// |v| > 1e-14 (the reference's drop threshold) on the bit pattern of v (integer pipe)
__device__ __forceinline__ bool above_drop(uint64_t u) { return (u & 0x7FFFFFFFFFFFFFFFull) > 0x3D06849B86A12B9Bull; }

// Segment starts S1..S4 and the padded width Wp.
struct SlotMap {
    int s1, s2, s3, s4, wp;
};
__host__ __device__ inline SlotMap slot_map(const FciParams &p) {
    SlotMap m;
    m.s1 = 4;
    m.s2 = m.s1 + pad4(p.b.ns);
    m.s3 = m.s2 + pad4(p.b.nd);
    m.s4 = m.s3 + pad4(p.a.ns + p.a.nd);
    m.wp = m.s4 + pad4(p.a.ns * p.b.ns);
    return m;
}

// Descriptor of slot k of alpha string ia: Ja | beta kind << 32 | xb << 34. Padding
// slots carry their segment's kind with Ja = ia, xb = 0 (a valid column, value 0).
__device__ __forceinline__ uint64_t slot_desc(const FciParams &p, const SlotMap &m, int64_t ia, int k) {
    const int nsa = p.a.ns, nsb = p.b.ns;
    uint64_t Ja = (uint64_t)ia, kindB = kSelf, xb = 0;
    if (k < m.s1) {
    } else if (k < m.s2) {
        kindB = kSingle;
        if (k - m.s1 < nsb) xb = k - m.s1;
    } else if (k < m.s3) {
        kindB = kDouble;
        if (k - m.s2 < p.b.nd) xb = k - m.s2;
    } else if (k < m.s4) {
        const int i = k - m.s3;
        if (i < nsa) Ja = __ldg(p.a.s_target + ia * nsa + i);
        else if (i < nsa + p.a.nd) Ja = __ldg(p.a.d_target + ia * p.a.nd + (i - nsa));
    } else {
        kindB = kSingle;
        const int i = k - m.s4;
        if (i < nsa * nsb) {
            const int xa = i / nsb;
            Ja = __ldg(p.a.s_target + ia * nsa + xa);
            xb = i - xa * nsb;
        }
    }
    return Ja | (kindB << 32) | (xb << 34);
}

// Shared memory: descriptors [Wp] (8 bytes), beta single targets [nsb][kTileRows].
__device__ __forceinline__ void stage_tile(const FciParams &p, const SlotMap &m, int64_t ia, int64_t t,
                                           uint64_t *desc, uint32_t *st) {
    for (int k = threadIdx.x; k < m.wp; k += blockDim.x) desc[k] = slot_desc(p, m, ia, k);
    const int nsb = p.b.ns;
    for (int i = threadIdx.x; i < nsb * kTileRows; i += blockDim.x) {
        const int xb = i / kTileRows, r = i - xb * kTileRows;
        const int64_t ib = t * kTileRows + r;
        st[i] = ib < p.Db ? __ldg(p.b.s_target + ib * nsb + xb) : 0u;
    }
}

// The matvec's staging from the precomputed tables (the tile's slot descriptors
// and beta single targets) with 16-byte loads: a few independent loads per thread
// where computing them took ~10 dependent table reads. The descriptors are staged
// in the matvec's own form: the low word is the x panel's start Ja * Db (the
// matrix dimension fits 32 bits), the high word the beta kind plus, shifted by 2,
// the offset of the beta target: xb * kTileRows into the staged single targets, or
// xb into the row's double targets. A column is then one 32-bit add.
__device__ __forceinline__ uint2 mv_desc(uint32_t lo, uint32_t hi, uint32_t Db) {
    const uint32_t kind = hi & 3u, xb = hi >> 2;
    return make_uint2(lo * Db, kind | ((kind == kSingle ? xb * kTileRows : xb) << 2));
}
__device__ __forceinline__ void stage_tile_tab(const FciParams &p, const SlotMap &m, int64_t ia, int64_t t,
                                               uint64_t *desc, uint32_t *st) {
    const uint4 *ds = reinterpret_cast<const uint4 *>(p.desc_tab + ia * m.wp);
    uint4 *dd = reinterpret_cast<uint4 *>(desc);
    const uint32_t Db = (uint32_t)p.Db;
    for (int i = threadIdx.x; i < m.wp / 2; i += blockDim.x) {
        const uint4 d = __ldg(ds + i);
        const uint2 a = mv_desc(d.x, d.y, Db), b = mv_desc(d.z, d.w, Db);
        dd[i] = make_uint4(a.x, a.y, b.x, b.y);
    }
    const int n4 = p.b.ns * kTileRows / 4;
    const uint4 *ss = reinterpret_cast<const uint4 *>(p.st_tab + t * p.b.ns * kTileRows);
    uint4 *sd = reinterpret_cast<uint4 *>(st);
    for (int i = threadIdx.x; i < n4; i += blockDim.x) sd[i] = __ldg(ss + i);
}

__global__ void k_slot_desc_table(const FciParams p, uint64_t *__restrict__ tab) {
    const SlotMap m = slot_map(p);
    const int64_t total = p.a.D * m.wp;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ia = i / m.wp;
        tab[i] = slot_desc(p, m, ia, (int)(i - ia * m.wp));
    }
}

__global__ void k_slot_st_table(const FciParams p, uint32_t *__restrict__ tab) {
    const int nsb = p.b.ns;
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows, per = (int64_t)nsb * kTileRows, total = T * per;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = i / per;
        const int rem = (int)(i - t * per), xb = rem / kTileRows, r = rem - xb * kTileRows;
        const int64_t ib = t * kTileRows + r;
        tab[i] = ib < p.Db ? __ldg(p.b.s_target + ib * nsb + xb) : 0u;
    }
}

// Blocks per SM the register budget is set for (measured at L=10..12): 6 for the
// FP32 matvec (40 registers once its staging reads the precomputed tables; 2.4%
// over 5 blocks at L=12, equal at L=11, 2% slower at L=10, and with 4 quads in
// flight 5% slower everywhere); the hi/lo variant runs 2% faster held to 4 blocks
// (64 registers).
template <typename F>
struct SlotOccupancy {
    static constexpr int kMinBlocks = 4;
};
template <>
struct SlotOccupancy<Plain<float>> {
    static constexpr int kMinBlocks = 6;
};

// 16-byte value loads in flight per lane: 3 for the FP32 matvec (2% over 2 at L=12;
// 4 spills at the 48-register budget), 2 for the hi/lo variant (two arrays per quad).
// Measured and dropped: a cp.async ring of 2-5 quads per lane in shared memory
// (3.0-3.6 TB/s, with or without an evict-first L2 policy) and two or three tiles
// of one alpha string per block sharing the staged descriptors (4.4 / 2.7 TB/s).
template <typename F>
struct SlotInFlight {
    static constexpr int kQuads = 2;
};
template <>
struct SlotInFlight<Plain<float>> {
    static constexpr int kQuads = 3;
};

// ---------------------------------------------------------------------------
// Matvec. Block = one tile; warp w: rows (w % kRowWarps) * 32 + lane, quad range w / kRowWarps.
// Measured and dropped: a tile split over a cluster of 2-4 blocks whose row sums
// meet through distributed shared memory (for matrices of few tiles, 1.33 waves
// at L=10): every block carries a fixed ~7-9 us (ramp, staging, drain), which
// costs more than the emptier last wave (L=10: 63 us at two blocks per tile
// against 66 us at one; L=11: 287 against 250 us).
template <typename F>
__global__ void __launch_bounds__(kSlotThreads, SlotOccupancy<F>::kMinBlocks) k_spmv_slots(const FciParams p, const F f,
                                                             typename F::X *__restrict__ y) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ typename F::Acc part[kSplits][kTileRows];
    const SlotMap m = slot_map(p);
    const int Q = m.wp >> 2;
    uint64_t *desc = reinterpret_cast<uint64_t *>(smem);
    uint32_t *st = reinterpret_cast<uint32_t *>(desc + m.wp);
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    const int64_t tile = blockIdx.x;
    const int64_t ia = tile / T, t = tile - ia * T;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rr = (warp % kRowWarps) * 32 + lane, ks = warp / kRowWarps;
    const int c0 = (int)((int64_t)Q * ks / kSplits), c1 = (int)((int64_t)Q * (ks + 1) / kSplits);
    const int64_t qbase = tile * (int64_t)Q;
    // the first values of each quad range head for L2 while the tables are staged
    if (lane == 0 && warp % kRowWarps == 0 && c1 > c0)
        f.prefetch((qbase + c0) * kTileRows * 4, (int64_t)min(c1 - c0, kPrefetchQuads) * kTileRows * 4);
    stage_tile_tab(p, m, ia, t, desc, st);
    __syncthreads();
    const int64_t ib_raw = t * kTileRows + rr;
    const bool active = ib_raw < p.Db;
    const int64_t ib = active ? ib_raw : p.Db - 1;
    const uint32_t ib32 = (uint32_t)ib;
    const uint32_t *dt = p.b.d_target + ib * p.b.nd;
    const uint32_t *stl = st + rr;  // this row's beta single targets, kTileRows apart
    constexpr int kQuadsInFlight = SlotInFlight<F>::kQuads;
    typename F::Acc acc{};
    typename F::Chunk v[kQuadsInFlight];
    // kQuadsInFlight quads in flight per lane; each quad has one beta kind (uniform branch)
    for (int c = c0; c < c1; c += kQuadsInFlight) {
#pragma unroll
        for (int u = 0; u < kQuadsInFlight; ++u) {
            if (c + u < c1)
                f.load4(((qbase + c + u) * kTileRows + rr) * 4, v[u]);
            else
                f.zero(v[u]);
        }
#pragma unroll
        for (int u = 0; u < kQuadsInFlight; ++u) {
            if (c + u < c1) {
                // the quad's four staged descriptors: (panel start, kind | target offset << 2)
                const uint4 *dq = reinterpret_cast<const uint4 *>(desc + 4 * (c + u));
                const uint32_t kind = reinterpret_cast<const uint32_t *>(dq)[1] & 3u;  // one kind per quad
                uint32_t col[4];
                if (kind == kSelf) {
                    const uint4 q0 = dq[0], q1 = dq[1];
                    col[0] = q0.x + ib32;
                    col[1] = q0.z + ib32;
                    col[2] = q1.x + ib32;
                    col[3] = q1.z + ib32;
                } else if (kind == kSingle) {
                    const uint4 q0 = dq[0], q1 = dq[1];
                    col[0] = q0.x + stl[q0.y >> 2];
                    col[1] = q0.z + stl[q0.w >> 2];
                    col[2] = q1.x + stl[q1.y >> 2];
                    col[3] = q1.z + stl[q1.w >> 2];
                } else {
                    const uint4 q0 = dq[0], q1 = dq[1];
                    col[0] = q0.x + __ldg(dt + (q0.y >> 2));
                    col[1] = q0.z + __ldg(dt + (q0.w >> 2));
                    col[2] = q1.x + __ldg(dt + (q1.y >> 2));
                    col[3] = q1.z + __ldg(dt + (q1.w >> 2));
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) f.term(v[u], j, (int64_t)col[j], acc);
            }
        }
    }
    part[ks][rr] = acc;
    __syncthreads();
    if (ks == 0 && active) {
        typename F::Acc s = part[0][rr];
#pragma unroll
        for (int q = 1; q < kSplits; ++q) f.add(s, part[q][rr]);
        y[ia * p.Db + ib_raw] = f.result(s);
    }
}

// ---------------------------------------------------------------------------
// FP64 matvec of compact tiles (p.fly): the quads of S0..S3 are stored
// (val[((tile * Qs + c) * kTileRows + row) * 4 + j], Qs = S4 / 4), and the alpha-single
// x beta-single block S4 -- 71% of the slots at L=12 6a6b -- is formed here from the
// staged integral slices: element (xa, xb) of row (Ia, Ib) is (ar ac|br bc) with the
// sign of both phases, zero where |v| <= 1e-14, the value the fill would store. The
// quad ranges, the order of the terms and the sums of the ranges are those of
// k_spmv_slots<Plain<double>>, so the product equals the full tiles' bit for bit.
// The values read from HBM drop from 8 Wp to 8 S4 bytes per row, but an S4 element
// costs a random 8-byte shared-memory gather of its integral and three more
// shared-memory reads besides the x gather both forms make, and the L1 / shared-
// memory data path, not the FP64 pipe, bounds the product: 3.81 against 2.71 ms at
// L=12 6a6b (0.65 of the FP64-pipe floor against 0.95). A memory saver, not a
// faster product.
// Shared memory: descriptors [Wp], beta single targets [nsb][kTileRows], beta pairs
// and parities [nsb][kTileRows], alpha parities [pad4(nsa)], alpha integral row
// offsets [pad4(nsa)], integral slices [nsa][L^2] (FP64).
__global__ void __launch_bounds__(kSlotThreads, 3) k_spmv_slots_fly(const FciParams p, const Plain<double> f,
                                                                    double *__restrict__ y) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double part[kSplits][kTileRows];
    const SlotMap m = slot_map(p);
    const int Q = m.wp >> 2, Qs = m.s4 >> 2;
    const int L2 = p.L * p.L, nsa = p.a.ns, nsb = p.b.ns;
    uint64_t *desc = reinterpret_cast<uint64_t *>(smem);
    uint32_t *st = reinterpret_cast<uint32_t *>(desc + m.wp);
    uint32_t *sbi = st + nsb * kTileRows;
    uint32_t *sai = sbi + nsb * kTileRows;
    uint32_t *roff = sai + pad4(nsa);
    double *sl64 = reinterpret_cast<double *>(roff + pad4(nsa));  // 16-byte aligned: every region is a multiple of 16 bytes
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    const int64_t tile = blockIdx.x;
    const int64_t ia = tile / T, t = tile - ia * T;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rr = (warp % kRowWarps) * 32 + lane, ks = warp / kRowWarps;
    const int c0 = (int)((int64_t)Q * ks / kSplits), c1 = (int)((int64_t)Q * (ks + 1) / kSplits);
    const int cs = min(c1, Qs);  // stored quads of this range end here
    const int64_t qbase = tile * (int64_t)Qs;
    if (lane == 0 && warp % kRowWarps == 0 && cs > c0)
        f.prefetch((qbase + c0) * kTileRows * 4, (int64_t)min(cs - c0, kPrefetchQuads) * kTileRows * 4);
    stage_tile_tab(p, m, ia, t, desc, st);
    // beta singles of the tile's rows: orbital pair br * L + bc | parity << 31 (read
    // in the table's order, row-major, and stored single-major)
    for (int i = threadIdx.x; i < nsb * kTileRows; i += blockDim.x) {
        const int r = i / nsb, xb = i - r * nsb;
        const int64_t ibr = t * kTileRows + r;
        uint32_t w = 0;
        if (ibr < p.Db) {
            const uint32_t info = __ldg(p.b.s_info + ibr * nsb + xb);
            w = (((info >> 12) & 63) * p.L + ((info >> 18) & 63)) | (((info >> 24) & 1u) << 31);
        }
        sbi[xb * kTileRows + r] = w;
    }
    for (int xa = threadIdx.x; xa < nsa; xa += blockDim.x) {
        const uint32_t info = __ldg(p.a.s_info + ia * nsa + xa);
        sai[xa] = ((info >> 24) & 1u) << 31;
        roff[xa] = (((info >> 12) & 63) * p.L + ((info >> 18) & 63)) * L2;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nsa * L2; i += blockDim.x) {
        const int xa = i / L2;
        sl64[i] = __ldg(p.eri + roff[xa] + (i - xa * L2));
    }
    __syncthreads();
    const int64_t ib_raw = t * kTileRows + rr;
    const bool active = ib_raw < p.Db;
    const int64_t ib = active ? ib_raw : p.Db - 1;
    const uint32_t ib32 = (uint32_t)ib;
    const uint32_t *dt = p.b.d_target + ib * p.b.nd;
    const uint32_t *stl = st + rr;  // this row's beta single targets, kTileRows apart
    constexpr int kQuadsInFlight = SlotInFlight<Plain<double>>::kQuads;
    Plain<double>::Acc acc{};
    Plain<double>::Chunk v[kQuadsInFlight];
    // stored quads: the loop of k_spmv_slots
    for (int c = c0; c < cs; c += kQuadsInFlight) {
#pragma unroll
        for (int u = 0; u < kQuadsInFlight; ++u) {
            if (c + u < cs)
                f.load4(((qbase + c + u) * kTileRows + rr) * 4, v[u]);
            else
                f.zero(v[u]);
        }
#pragma unroll
        for (int u = 0; u < kQuadsInFlight; ++u) {
            if (c + u < cs) {
                const uint4 *dq = reinterpret_cast<const uint4 *>(desc + 4 * (c + u));
                const uint32_t kind = reinterpret_cast<const uint32_t *>(dq)[1] & 3u;  // one kind per quad
                uint32_t col[4];
                const uint4 q0 = dq[0], q1 = dq[1];
                if (kind == kSelf) {
                    col[0] = q0.x + ib32;
                    col[1] = q0.z + ib32;
                    col[2] = q1.x + ib32;
                    col[3] = q1.z + ib32;
                } else if (kind == kSingle) {
                    col[0] = q0.x + stl[q0.y >> 2];
                    col[1] = q0.z + stl[q0.w >> 2];
                    col[2] = q1.x + stl[q1.y >> 2];
                    col[3] = q1.z + stl[q1.w >> 2];
                } else {
                    col[0] = q0.x + __ldg(dt + (q0.y >> 2));
                    col[1] = q0.z + __ldg(dt + (q0.w >> 2));
                    col[2] = q1.x + __ldg(dt + (q1.y >> 2));
                    col[3] = q1.z + __ldg(dt + (q1.w >> 2));
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) f.term(v[u], j, (int64_t)col[j], acc);
            }
        }
    }
    // S4 quads, formed: slot k = 4c + j is element i = k - S4 = xa * nsb + xb
    const int c4 = max(c0, Qs);
    if (c4 < c1) {
        const int npair = nsa * nsb;
        int i = 4 * c4 - m.s4;
        int xa = i / nsb, xb = i - xa * nsb;
        for (int c = c4; c < c1; ++c) {
            const uint4 *dq = reinterpret_cast<const uint4 *>(desc + 4 * c);  // kind single: Ja * Db, xb * kTileRows
            const uint4 q0 = dq[0], q1 = dq[1];
            const uint32_t col[4] = {q0.x + stl[q0.y >> 2], q0.z + stl[q0.w >> 2], q1.x + stl[q1.y >> 2],
                                     q1.z + stl[q1.w >> 2]};
            Plain<double>::Chunk e;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                uint64_t u = 0;  // padding slots hold zero
                if (i < npair) {
                    const uint32_t w = sbi[xb * kTileRows + rr];
                    const uint64_t odd = (uint64_t)((sai[xa] ^ w) >> 31);
                    u = (uint64_t)__double_as_longlong(sl64[xa * L2 + (int)(w & 0xFFFu)]) ^ (odd << 63);
                    if (!above_drop(u)) u = 0;
                    if (++xb == nsb) {
                        xb = 0;
                        ++xa;
                    }
                }
                ++i;
                e.v[j] = __longlong_as_double((long long)u);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) f.term(e, j, (int64_t)col[j], acc);
        }
    }
    part[ks][rr] = acc.s;
    __syncthreads();
    if (ks == 0 && active) {
        double sum = part[0][rr];
#pragma unroll
        for (int q = 1; q < kSplits; ++q) sum += part[q][rr];
        y[ia * p.Db + ib_raw] = sum;
    }
}

// ---------------------------------------------------------------------------
// Fill: the same element values as the CRS generator, as FP32 hi + lo splits (zero
// where |v| <= 1e-14; F64 = false) or as FP64 values (zero where |v| <= 1e-14;
// F64 = true, the plain method's tiles), with each row's nonzero count and
// lower-triangle count.
template <bool F64>
struct FillVals;
template <>
struct FillVals<false> {  // FP32 hi + lo
    float h[4] = {0, 0, 0, 0}, l[4] = {0, 0, 0, 0};
    __device__ __forceinline__ void from_split(int j, const float *hi, const float *lo, size_t at) {
        h[j] = __ldg(hi + at);
        l[j] = __ldg(lo + at);
    }
    __device__ __forceinline__ bool nonzero(int j) const { return (__float_as_uint(h[j]) & 0x7FFFFFFFu) != 0u; }
    __device__ __forceinline__ void clear(int j) { h[j] = l[j] = 0.0f; }
};
template <>
struct FillVals<true> {  // FP64, |v| <= 1e-14 stored as zero
    // the threshold test and the zero test on the bit patterns (integer pipe): FP64
    // compares, two per element, left the fill bound by GB300's FP64 pipe
    uint64_t b[4] = {0, 0, 0, 0};
    __device__ __forceinline__ void set(int j, double x) {
        const uint64_t u = (uint64_t)__double_as_longlong(x);
        b[j] = above_drop(u) ? u : 0ull;
    }
    __device__ __forceinline__ bool nonzero(int j) const { return b[j] != 0ull; }
    __device__ __forceinline__ void clear(int j) { b[j] = 0ull; }
    __device__ __forceinline__ double v(int j) const { return __longlong_as_double((long long)b[j]); }
};

template <bool F64>
__global__ void __launch_bounds__(kSlotThreads) k_fill_slots(const FciParams p, float *__restrict__ hi,
                                                             float *__restrict__ lo, double *__restrict__ v64,
                                                             uint32_t *__restrict__ count,
                                                             uint32_t *__restrict__ lower) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t cnt[kSplits][kTileRows], low[kSplits][kTileRows];
    const SlotMap m = slot_map(p);
    const int Q = m.wp >> 2;
    const int L2 = p.L * p.L, nsa = p.a.ns;
    uint64_t *desc = reinterpret_cast<uint64_t *>(smem);
    uint32_t *st = reinterpret_cast<uint32_t *>(desc + m.wp);
    // per (beta single, row): orbital pair tt = br * L + bc | parity << 31; per alpha
    // single: parity << 31 | (Ja < Ia) << 30 -- what an S4 element needs besides
    // its integral, read from shared memory instead of one dependent global load each
    uint32_t *sbi = st + p.b.ns * kTileRows;
    uint32_t *sai = sbi + p.b.ns * kTileRows;
    // alpha-single integral slices, nsa * L2 entries: FP32 (hi, lo) pairs (F64 = false,
    // one 8-byte shared load per element) or FP64 (true)
    float2 *slhl = reinterpret_cast<float2 *>(sai + pad4(nsa));  // 16-byte aligned: every region is a multiple of 16 bytes
    double *sl64 = reinterpret_cast<double *>(slhl);
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    const int64_t ia = blockIdx.x / T, t = blockIdx.x - ia * T;
    stage_tile(p, m, ia, t, desc, st);
    for (int i = threadIdx.x; i < p.b.ns * kTileRows; i += blockDim.x) {
        const int xb = i / kTileRows, r = i - xb * kTileRows;
        const int64_t ibr = t * kTileRows + r;
        uint32_t w = 0;
        if (ibr < p.Db) {
            const uint32_t info = __ldg(p.b.s_info + ibr * p.b.ns + xb);
            w = (((info >> 12) & 63) * p.L + ((info >> 18) & 63)) | (((info >> 24) & 1u) << 31);
        }
        sbi[i] = w;
    }
    for (int xa = threadIdx.x; xa < nsa; xa += blockDim.x) {
        const uint32_t info = __ldg(p.a.s_info + ia * nsa + xa);
        const uint32_t Ja = __ldg(p.a.s_target + ia * nsa + xa);
        sai[xa] = (((info >> 24) & 1u) << 31) | ((uint32_t)(Ja < (uint32_t)ia) << 30);
    }
    if (p.staged) {
        for (int i = threadIdx.x; i < nsa * L2; i += blockDim.x) {
            const int xa = i / L2, tt = i - xa * L2;
            const uint32_t info = __ldg(p.a.s_info + ia * nsa + xa);
            const int ar = (info >> 12) & 63, ac = (info >> 18) & 63;
            const size_t at = ((size_t)ar * p.L + ac) * L2 + tt;
            if constexpr (F64) {
                sl64[i] = __ldg(p.eri + at);
            } else {
                slhl[i] = make_float2(__ldg(p.eri_hi + at), __ldg(p.eri_lo + at));
            }
        }
    }
    __syncthreads();
    // Compact FP64 tiles (p.fly; the slices are not staged): the alpha-single x
    // beta-single block (S4) is not stored. Its element for alpha single xa and beta
    // pair tt has the magnitude of the integral (ar ac|tt), so a row's S4 nonzeros are
    // a sum over its beta singles of nz[tt] (alpha singles whose integral with tt
    // exceeds 1e-14) and its lower-triangle ones of nzl[tt] (those with Ja < Ia).
    uint32_t *nz = nullptr, *nzl = nullptr;
    if constexpr (F64) {
        if (p.fly) {
            nz = reinterpret_cast<uint32_t *>(sai + pad4(nsa));
            nzl = nz + L2;
            for (int tt = threadIdx.x; tt < L2; tt += blockDim.x) {
                uint32_t na = 0, nl = 0;
                for (int xa = 0; xa < nsa; ++xa) {
                    const uint32_t info = __ldg(p.a.s_info + ia * nsa + xa);
                    const size_t at = (((info >> 12) & 63) * (size_t)p.L + ((info >> 18) & 63)) * L2 + tt;
                    const bool keep = above_drop((uint64_t)__double_as_longlong(__ldg(p.eri + at)));
                    na += keep;
                    nl += keep && ((sai[xa] >> 30) & 1u);
                }
                nz[tt] = na;
                nzl[tt] = nl;
            }
            __syncthreads();
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rr = (warp % kRowWarps) * 32 + lane, ks = warp / kRowWarps;
    const int64_t ib_raw = t * kTileRows + rr;
    const bool active = ib_raw < p.Db;
    const int64_t ib = active ? ib_raw : p.Db - 1;
    const int64_t r = ia * p.Db + ib;
    const int c0 = (int)((int64_t)Q * ks / kSplits), c1 = (int)((int64_t)Q * (ks + 1) / kSplits);
    const bool fly = F64 && p.fly;
    const int Qs = fly ? m.s4 >> 2 : Q;  // stored quads per row
    const int cs = min(c1, Qs);
    const int64_t qbase = (ia * T + t) * (int64_t)Qs;
    const int nsb = p.b.ns, ndb = p.b.nd, nda = p.a.nd, nsr = nsa + nsb, L = p.L;
    uint32_t n_keep = 0, n_low = 0;
    // one quad at a time; a quad lies in one segment, so the branch is uniform
    for (int c = c0; c < cs; ++c) {
        const int k0 = 4 * c;
        FillVals<F64> q;
        bool lw[4] = {false, false, false, false};  // column below the diagonal
        if (k0 < m.s1) {  // S0: the diagonal
            if constexpr (F64) {
                q.set(0, p.diag[r]);
            } else {
                q.h[0] = p.diag_hi[r];
                q.l[0] = p.diag_lo[r];
            }
        } else if (k0 < m.s2) {  // S1: beta singles (one_diff_orbital), precomputed per row
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int xb = k0 - m.s1 + j;
                if (xb < nsb) {
                    const size_t at = (size_t)r * nsr + nsa + xb;
                    if constexpr (F64) q.set(j, __ldg(p.sgl64 + at));
                    else q.from_split(j, p.sgl_hi, p.sgl_lo, at);
                    lw[j] = st[xb * kTileRows + rr] < (uint32_t)ib;
                }
            }
        } else if (k0 < m.s3) {  // S2: beta-beta doubles
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int xb = k0 - m.s2 + j;
                if (xb < ndb) {
                    const size_t at = ib * ndb + xb;
                    if constexpr (F64) q.set(j, __ldg(p.b.d_val + at));
                    else q.from_split(j, p.b.d_hi, p.b.d_lo, at);
                    lw[j] = __ldg(p.b.d_target + at) < (uint32_t)ib;
                }
            }
        } else if (k0 < m.s4) {  // S3: alpha singles then alpha-alpha doubles, beta self
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int i = k0 - m.s3 + j;
                if (i < nsa) {
                    const size_t at = (size_t)r * nsr + i;
                    if constexpr (F64) q.set(j, __ldg(p.sgl64 + at));
                    else q.from_split(j, p.sgl_hi, p.sgl_lo, at);
                } else if (i < nsa + nda) {
                    const size_t at = ia * nda + (i - nsa);
                    if constexpr (F64) q.set(j, __ldg(p.a.d_val + at));
                    else q.from_split(j, p.a.d_hi, p.a.d_lo, at);
                }
                lw[j] = (uint32_t)desc[k0 + j] < (uint32_t)ia;
            }
        } else {  // S4: alpha-beta doubles (ar ac|br bc), sign from both phases (CIMethod.cpp:444-457)
            const int i0 = k0 - m.s4;
            int xa = nsb > 0 ? i0 / nsb : 0, xb = i0 - xa * nsb;
            uint32_t a = xa < nsa ? sai[xa] : 0u;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (i0 + j < nsa * nsb) {
                    const uint32_t w = sbi[xb * kTileRows + rr];
                    const int tt = (int)(w & 0xFFFu);
                    const uint32_t odd = (a ^ w) >> 31;
                    if constexpr (F64) {
                        double e;
                        if (p.staged) {
                            e = sl64[xa * L2 + tt];
                        } else {
                            const uint32_t infoA = __ldg(p.a.s_info + ia * nsa + xa);
                            const int ar = (infoA >> 12) & 63, ac = (infoA >> 18) & 63;
                            e = __ldg(p.eri + ((size_t)ar * L + ac) * L2 + tt);
                        }
                        q.set(j, __longlong_as_double(__double_as_longlong(e) ^ ((long long)odd << 63)));
                    } else {
                        float h, l;
                        if (p.staged) {
                            const float2 hl = slhl[xa * L2 + tt];
                            h = hl.x;
                            l = hl.y;
                        } else {
                            const uint32_t infoA = __ldg(p.a.s_info + ia * nsa + xa);
                            const int ar = (infoA >> 12) & 63, ac = (infoA >> 18) & 63;
                            const size_t at = ((size_t)ar * L + ac) * L2 + tt;
                            h = __ldg(p.eri_hi + at);
                            l = __ldg(p.eri_lo + at);
                        }
                        q.h[j] = __uint_as_float(__float_as_uint(h) ^ (odd << 31));
                        q.l[j] = __uint_as_float(__float_as_uint(l) ^ (odd << 31));
                    }
                    lw[j] = (a >> 30) & 1u;  // Ja < Ia: the column lies below the diagonal
                    if (++xb == nsb && j < 3) {
                        xb = 0;
                        ++xa;
                        a = xa < nsa ? sai[xa] : 0u;
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (!active) q.clear(j);
            const bool keep = q.nonzero(j);  // |v| > 1e-14
            n_keep += keep;
            n_low += keep && lw[j];
        }
        const int64_t at = ((qbase + c) * kTileRows + rr) * 4;
        if constexpr (F64) {
            double2 *d = reinterpret_cast<double2 *>(v64 + at);
            d[0] = make_double2(q.v(0), q.v(1));
            d[1] = make_double2(q.v(2), q.v(3));
        } else {
            *reinterpret_cast<float4 *>(hi + at) = make_float4(q.h[0], q.h[1], q.h[2], q.h[3]);
            *reinterpret_cast<float4 *>(lo + at) = make_float4(q.l[0], q.l[1], q.l[2], q.l[3]);
        }
    }
    if (fly && ks == kSplits - 1)
        for (int xb = 0; xb < nsb; ++xb) {
            const uint32_t tt = sbi[xb * kTileRows + rr] & 0xFFFu;
            n_keep += nz[tt];
            n_low += nzl[tt];
        }
    cnt[ks][rr] = n_keep;
    low[ks][rr] = n_low;
    __syncthreads();
    if (ks == 0 && active) {
        uint32_t a = 0, b = 0;
#pragma unroll
        for (int q = 0; q < kSplits; ++q) {
            a += cnt[q][rr];
            b += low[q][rr];
        }
        count[r] = a;
        lower[r] = b;
    }
}

size_t tile_smem(const FciParams &p) { return (size_t)slot_map(p).wp * 8 + (size_t)p.b.ns * kTileRows * 4; }
// the fill's staging: the tile tables, the beta singles' pairs / parities, the alpha flags
size_t fill_smem(const FciParams &p) {
    return tile_smem(p) + (size_t)p.b.ns * kTileRows * 4 + (size_t)pad4(p.a.ns) * 4;
}
size_t slice_smem(const FciParams &p) { return (size_t)p.a.ns * p.L * p.L * 8; }  // hi + lo slices
// compact FP64 tiles: the fill stages no slices but two histograms over the beta
// pairs; the matvec stages the slices and the alpha integral row offsets
size_t fly_smem(const FciParams &p) { return fill_smem(p) + (size_t)8 * p.L * p.L; }
size_t fly_mv_smem(const FciParams &p) { return fill_smem(p) + slice_smem(p) + (size_t)pad4(p.a.ns) * 4; }

template <typename F>
void launch_slots(const FciParams &p, const F &f0, typename F::X *y, cudaStream_t s) {
    F f = f0;
    f.nx = (uint64_t)(p.a.D * p.Db);
    f.err = check_word_device();
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_spmv_slots<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotsMaxSmem);
        return true;
    }();
    (void)attr_set;
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    k_spmv_slots<F><<<(unsigned)(p.a.D * T), kSlotThreads, tile_smem(p), s>>>(p, f, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace

bool slots_supported(const FciParams &p) {
    return p.a.D * p.Db < (int64_t)UINT32_MAX && fill_smem(p) <= kSlotsMaxSmem && (int64_t)p.L * p.L <= 4096 && p.a.D * ((p.Db + kTileRows - 1) / kTileRows) < (int64_t)INT32_MAX &&
           (int64_t)p.a.ns * p.b.ns < (int64_t)INT32_MAX / 8;
}

int64_t slots_count(const FciParams &p) {
    return p.a.D * ((p.Db + kTileRows - 1) / kTileRows) * kTileRows * (int64_t)slot_map(p).wp;
}

bool slots64_fly_fits(const FciParams &p) {
    return p.a.ns > 0 && p.b.ns > 0 && fly_smem(p) <= kSlotsMaxSmem && fly_mv_smem(p) <= kSlotsMaxSmem;
}

int64_t slots_stored(const FciParams &p) {
    if (!p.fly) return slots_count(p);
    return p.a.D * ((p.Db + kTileRows - 1) / kTileRows) * kTileRows * (int64_t)slot_map(p).s4;
}

void fill_slots_launch(const FciParams &p0, float *hi, float *lo, uint32_t *count, uint32_t *lower, cudaStream_t s) {
    FciParams p = p0;
    const size_t base = fill_smem(p), sl = slice_smem(p);
    p.staged = base + sl <= kSlotsMaxSmem ? 1 : 0;
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_fill_slots<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotsMaxSmem);
        return true;
    }();
    (void)attr_set;
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    k_fill_slots<false><<<(unsigned)(p.a.D * T), kSlotThreads, p.staged ? base + sl : base, s>>>(p, hi, lo, nullptr,
                                                                                                count, lower);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void fill_slots64_launch(const FciParams &p0, double *v64, uint32_t *count, uint32_t *lower, cudaStream_t s) {
    FciParams p = p0;
    const size_t base = fill_smem(p), sl = slice_smem(p);  // an FP64 slice takes the bytes of hi + lo
    p.staged = base + sl <= kSlotsMaxSmem ? 1 : 0;
    size_t smem = p.staged ? base + sl : base;
    if (p.fly) {  // no S4 elements to form: no slices, the two histograms in their place
        if (!slots64_fly_fits(p)) throw std::logic_error("compact FP64 slot tiles do not fit this space");
        p.staged = 0;
        smem = fly_smem(p);
    }
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_fill_slots<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotsMaxSmem);
        return true;
    }();
    (void)attr_set;
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    k_fill_slots<true><<<(unsigned)(p.a.D * T), kSlotThreads, smem, s>>>(p, nullptr, nullptr, v64, count, lower);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

int64_t slot_desc_count(const FciParams &p) { return p.a.D * (int64_t)slot_map(p).wp; }
int64_t slot_st_count(const FciParams &p) { return ((p.Db + kTileRows - 1) / kTileRows) * p.b.ns * kTileRows; }

void slot_tables_launch(const FciParams &p, uint64_t *desc, uint32_t *st, cudaStream_t s) {
    const int g = sm_count() * 8;
    k_slot_desc_table<<<g, 256, 0, s>>>(p, desc);
    if (slot_st_count(p) > 0) k_slot_st_table<<<g, 256, 0, s>>>(p, st);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(slot_st_count(p) > 0 ? 2 : 1);
}

void spmv_slots_f32(const FciParams &p, const float *val, const float *x, float *y, cudaStream_t s) {
    launch_slots(p, Plain<float>{val, x}, y, s);
}

void spmv_slots_hilo(const FciParams &p, const float *hi, const float *lo, const double *x, const float *x32,
                     double *y, cudaStream_t s) {
    launch_slots(p, HiLo{hi, lo, x, x32}, y, s);
}

void spmv_slots_f64(const FciParams &p, const double *val, const double *x, double *y, cudaStream_t s) {
    if (!p.fly) {
        launch_slots(p, Plain<double>{val, x}, y, s);
        return;
    }
    Plain<double> f{val, x};
    f.nx = (uint64_t)(p.a.D * p.Db);
    f.err = check_word_device();
    static const bool attr_set = [] {  // thread-safe one-time init; three blocks of ~76 KB per SM at L=12 6a6b
        cudaFuncSetAttribute(k_spmv_slots_fly, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotsMaxSmem);
        cudaFuncSetAttribute(k_spmv_slots_fly, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
        return true;
    }();
    (void)attr_set;
    const int64_t T = (p.Db + kTileRows - 1) / kTileRows;
    k_spmv_slots_fly<<<(unsigned)(p.a.D * T), kSlotThreads, fly_mv_smem(p), s>>>(p, f, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace cigpu
