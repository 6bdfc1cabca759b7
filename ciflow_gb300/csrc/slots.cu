// Values-only FCI matvec of the mixed method.
//
// The FCI Hamiltonian has the same structural row width W for every row
// (nfull_b + ns_a * nsing_b + nd_a), and the column of every slot follows from
// the alpha and beta string tables the build already uses (the generator order
// of build.cu). The mixed method therefore stores only the values, W per row at
// stride Wp (W rounded up to 4, zero-padded): 4 bytes per element for the FP32
// matvec instead of the 8 of an FP32 CRS (column + value), and 8 instead of 12
// for the FP64 product from the split values. Columns are regenerated on the fly:
//   * a block owns one alpha string Ia and kFciRowsPerBlock beta strings; it
//     turns the alpha neighbour list of Ia into a slot descriptor table in shared
//     memory (alpha target Ja, kind, position q in the beta run);
//   * a group of G lanes per row walks the row 4 slots at a time (16-byte value
//     loads, streamed); each slot's column is Ja * Db + Jb with Jb read from the
//     beta neighbour list of Ib (L1/L2-resident tables) or Jb = Ib;
//   * x is gathered through the read-only path; the sum order is fixed, so the
//     product is bit-reproducible run to run.
// Replaces SparseMatrix_CRS_Sym::mvprod (SparseMatrix_CRS.cpp:700-723) for the
// FP32 CRS values of the mixed method.
#include <algorithm>

#include "build.cuh"
#include "slots.cuh"
#include "spmv_formats.cuh"

namespace cigpu {

namespace {

constexpr int kSlotThreads = 256;
constexpr uint32_t kPad = 3;  // descriptor kind of a padding slot

// desc = Ja | kind << 32 | q << 34
template <typename F, int G>
__global__ void __launch_bounds__(kSlotThreads) k_spmv_slots(const FciParams p, const F f,
                                                             const typename F::X *__restrict__ x,
                                                             typename F::X *__restrict__ y) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nga = p.a.nfull;
    const int W = fci_row_width(p);
    const int Wp = (int)p.Wp;
    uint64_t *desc = reinterpret_cast<uint64_t *>(smem);    // [Wp]
    uint32_t *gstart = reinterpret_cast<uint32_t *>(desc + Wp);  // [nga + 1]

    const int64_t nchunks = (p.Db + kFciRowsPerBlock - 1) / kFciRowsPerBlock;
    const int64_t ia = blockIdx.x / nchunks;
    const int64_t chunk = blockIdx.x - ia * nchunks;
    const int tid = threadIdx.x;
    const uint64_t *nbA = p.a.nb_full + ia * nga;

    // run starts of the alpha groups (one warp, shuffle prefix sum)
    if (tid < 32) {
        const int lane = tid;
        uint32_t run = 0;
        for (int g0 = 0; g0 < nga; g0 += 32) {
            const int g = g0 + lane;
            uint32_t sz = 0;
            if (g < nga) {
                const uint32_t kind = (uint32_t)(__ldg(nbA + g) >> 32) & 3u;
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
    for (int g = tid; g < nga; g += blockDim.x) {
        const uint64_t ea = __ldg(nbA + g);
        const uint64_t head = (uint64_t)(uint32_t)ea | (((ea >> 32) & 3u) << 32);
        for (uint32_t k = gstart[g], q = 0; k < gstart[g + 1]; ++k, ++q) desc[k] = head | ((uint64_t)q << 34);
    }
    for (int k = W + tid; k < Wp; k += blockDim.x) desc[k] = (uint64_t)kPad << 32;
    __syncthreads();

    const int lane = tid & (G - 1);
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((tid & 31) & ~(G - 1)));
    const int nchunk4 = Wp >> 2;
    for (int rr = tid / G; rr < kFciRowsPerBlock; rr += kSlotThreads / G) {
        const int64_t ib = chunk * kFciRowsPerBlock + rr;
        if (ib >= p.Db) break;
        const int64_t r = ia * p.Db + ib;
        const uint64_t *nbF = p.b.nb_full + ib * p.b.nfull;
        const uint64_t *nbS = p.b.nb_sing + ib * p.b.nsing;
        const int64_t base = r * p.Wp;
        typename F::Acc acc;
        for (int c0 = 0; c0 < nchunk4; c0 += 2 * G) {
            typename F::Chunk v[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int c = c0 + u * G + lane;
                if (c < nchunk4)
                    f.load4(base + 4 * (int64_t)c, v[u]);
                else
                    f.zero(v[u]);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int c = c0 + u * G + lane;
                if (c < nchunk4) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const uint64_t d = desc[4 * c + j];
                        const uint32_t kind = (uint32_t)(d >> 32) & 3u;
                        if (kind == kPad) continue;
                        const uint32_t q = (uint32_t)(d >> 34);
                        const uint32_t Jb = kind == kSelf     ? (uint32_t)__ldg(nbF + q)
                                            : kind == kSingle ? (uint32_t)__ldg(nbS + q)
                                                              : (uint32_t)ib;
                        const int64_t col = (int64_t)(uint32_t)d * p.Db + Jb;
                        f.fma(v[u], j, __ldg(x + col), acc);
                    }
                }
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) f.reduce(acc, gmask, o);
        if (lane == 0) y[r] = f.result(acc);
    }
}

size_t slots_smem(const FciParams &p) {
    return (size_t)p.Wp * 8 + ((size_t)p.a.nfull + 1) * 4;
}

template <typename F>
void launch_slots(const FciParams &p, const F &f, const typename F::X *x, typename F::X *y, cudaStream_t s) {
    const size_t sm = slots_smem(p);
    static const bool attr_set = [] {  // thread-safe one-time init
        cudaFuncSetAttribute(k_spmv_slots<F, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotsMaxSmem);
        cudaFuncSetAttribute(k_spmv_slots<F, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlotsMaxSmem);
        return true;
    }();
    (void)attr_set;
    const int64_t nchunks = (p.Db + kFciRowsPerBlock - 1) / kFciRowsPerBlock;
    const unsigned blocks = (unsigned)(p.a.D * nchunks);
    if ((p.Wp >> 2) >= 48)
        k_spmv_slots<F, 32><<<blocks, kSlotThreads, sm, s>>>(p, f, x, y);
    else
        k_spmv_slots<F, 8><<<blocks, kSlotThreads, sm, s>>>(p, f, x, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace

bool slots_supported(const FciParams &p) { return slots_smem(p) <= kSlotsMaxSmem; }

int64_t slots_stride(const FciParams &p) { return ((int64_t)fci_row_width(p) + 3) & ~(int64_t)3; }

void spmv_slots_f32(const FciParams &p, const float *val, const float *x, float *y, cudaStream_t s) {
    launch_slots(p, Plain<float>{val}, x, y, s);
}

void spmv_slots_hilo(const FciParams &p, const float *hi, const float *lo, const double *x, double *y,
                     cudaStream_t s) {
    launch_slots(p, HiLo{hi, lo}, x, y, s);
}

}  // namespace cigpu
