// CRS matrix-vector product on the device.
//
// Replaces SparseMatrix_CRS_Sym::mvprod (SparseMatrix_CRS.cpp:700-723), the
// serial symmetric scatter over the upper triangle. The device keeps the full
// symmetric matrix, so y = H x is a plain row gather with no atomics and a
// fixed summation order (bit-reproducible run to run):
//   * a group of 8-32 lanes per row, rows dealt round-robin to a persistent grid;
//   * col/val are streamed once (ld.global.cs: they are not reused, so they
//     must not evict x from L2); x is gathered through the read-only path and
//     stays L2-resident (853,776 doubles = 6.8 MB for the L=12 FCI space);
//   * 16-byte vector loads for the aligned body of each row.
// FP64: double values, double x/y, double accumulation.
// FP32 (mixed method): float values, float x/y, float row accumulation.
// FP64 from the mixed method's split values: HiLo (spmv_formats.cuh).
#include "spmv.cuh"
#include "spmv_formats.cuh"

#include <algorithm>

namespace cigpu {

namespace {

// G lanes per row (32, 16 or 8 for shorter rows); each lane issues U 16-byte
// column loads and U value loads before its 4U gathers of x, so enough bytes are
// in flight to cover HBM latency (a single chunk per lane left the kernel
// latency-bound on the dependent gathers).
// Row filters: every row, or only rows of problems still active (batched solves:
// row_prob[r] is the row's problem, status[p] != 0 once it has finished).
struct AllRows {
    __device__ __forceinline__ bool skip(int64_t) const { return false; }
};
struct ActiveRows {
    const int *__restrict__ row_prob;
    const int *__restrict__ status;
    __device__ __forceinline__ bool skip(int64_t r) const { return status[row_prob[r]] != 0; }
};

template <typename F, int G, int U, typename M = AllRows>
__global__ void __launch_bounds__(kSpmvThreads) k_spmv_rows(int64_t n, const int64_t *__restrict__ row_ptr,
                                                            const uint32_t *__restrict__ col, const F f,
                                                            typename F::X *__restrict__ y, const M m = M{}) {
    const int lane = threadIdx.x & (G - 1);
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
    // a row's bounds are loaded one row ahead, and its unaligned ends (at most 3
    // elements each side, one per lane) with its first body chunks: short rows
    // (DOCI: 145 elements) were a chain of dependent loads, bounds -> head ->
    // body -> tail
    int64_t s = 0, e = 0;
    if (gid < n) {
        s = __ldg(row_ptr + gid);
        e = __ldg(row_ptr + gid + 1);
    }
    for (int64_t r = gid; r < n; r += ng) {
        const int64_t rn = r + ng;
        int64_t sn = 0, en = 0;
        if (rn < n) {
            sn = __ldg(row_ptr + rn);
            en = __ldg(row_ptr + rn + 1);
        }
        if (!m.skip(r) && CIGPU_CHECK(f.err, row_ok(s, e, n), kCheckRowBounds, r)) {  // the same for the row's lanes
            typename F::Acc acc{};
            const int64_t s4 = (s + 3) & ~(int64_t)3;
            const int64_t head_end = s4 < e ? s4 : e;
            const int64_t nb = (e > s4) ? ((e - s4) >> 2) : 0;
            const int64_t t0 = s4 + (nb << 2);
            const bool has_h = lane < 4 && s + lane < head_end;
            const bool has_t = lane < 4 && e > s4 && t0 + lane < e;
            uint32_t ch = 0, ct = 0;
            typename F::Chunk vh, vt;
            f.zero(vh);
            f.zero(vt);
            if (has_h) {
                ch = __ldcs(col + s + lane);
                f.load1(s + lane, vh);
            }
            if (has_t) {
                ct = __ldcs(col + t0 + lane);
                f.load1(t0 + lane, vt);
            }
            const uint4 *c4 = reinterpret_cast<const uint4 *>(col + s4);
            for (int64_t b0 = 0; b0 < nb; b0 += G * U) {
                uint4 c[U];
                typename F::Chunk v[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int64_t idx = b0 + u * G + lane;
                    if (idx < nb) {
                        c[u] = __ldcs(c4 + idx);
                        f.load4(s4 + (idx << 2), v[u]);
                    } else {
                        c[u] = make_uint4(0, 0, 0, 0);
                        f.zero(v[u]);
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (b0 + u * G + lane < nb) {
                        f.term(v[u], 0, c[u].x, acc);
                        f.term(v[u], 1, c[u].y, acc);
                        f.term(v[u], 2, c[u].z, acc);
                        f.term(v[u], 3, c[u].w, acc);
                    }
                }
            }
            if (has_h) f.term(vh, 0, ch, acc);
            if (has_t) f.term(vt, 0, ct, acc);
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) f.reduce(acc, gmask, o);
            if (lane == 0) y[r] = f.result(acc);
        }
        s = sn;
        e = en;
    }
}

}  // namespace

int spmv_grid() { return sm_count_spmv() * kSpmvBlocksPerSM; }

int sm_count_spmv() {
    static const int sms = [] {  // thread-safe one-time init
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        return n;
    }();
    return sms;
}

// lanes per row from the mean row length (in 4-element chunks: 32 lanes for FCI
// rows of hundreds, 8 for the DOCI rows of ~36); the grid covers
// the rows once (at most a full persistent grid), so a small matrix leaves SMs
// free for the kernels of concurrent solves on other streams.
template <typename F>
static void launch_rows(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const F &f0,
                        typename F::X *y, cudaStream_t s) {
    F f = f0;
    f.nx = (uint64_t)n;
    f.err = check_word_device();
    const double chunks = n > 0 ? (double)nnz / n / 4.0 : 0;
    const int G = chunks >= 48 ? 32 : 8;  // DOCI L=24 (36 chunks): 8 lanes 19% over 16
    const int64_t need = (n * G + kSpmvThreads - 1) / kSpmvThreads;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(spmv_grid(), need));
    if (G == 32)
        k_spmv_rows<F, 32, 4><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y);
    else if (G == 16)
        k_spmv_rows<F, 16, 4><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y);
    else  // five chunks per lane: one round covers a DOCI row's 36 (FP32 5% over four)
        k_spmv_rows<F, 8, 5><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void spmv_f64_shape(int64_t n, const int64_t *row_ptr, const uint32_t *col, const double *val, const double *x,
                    double *y, int lanes, int grid, cudaStream_t s, const int *row_prob, const int *status) {
    Plain<double> f{val, x};
    f.nx = (uint64_t)n;
    f.err = check_word_device();
    using P = Plain<double>;
    if (row_prob) {
        const ActiveRows m{row_prob, status};
        switch (lanes) {
            case 4: k_spmv_rows<P, 4, 4, ActiveRows><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y, m); break;
            case 8: k_spmv_rows<P, 8, 4, ActiveRows><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y, m); break;
            case 16: k_spmv_rows<P, 16, 4, ActiveRows><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y, m); break;
            default: k_spmv_rows<P, 32, 4, ActiveRows><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y, m); break;
        }
    } else {
        switch (lanes) {
            case 4: k_spmv_rows<P, 4, 4><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y); break;
            case 8: k_spmv_rows<P, 8, 4><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y); break;
            case 16: k_spmv_rows<P, 16, 4><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y); break;
            default: k_spmv_rows<P, 32, 4><<<grid, kSpmvThreads, 0, s>>>(n, row_ptr, col, f, y); break;
        }
    }
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void spmv_f64(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const double *val, const double *x,
              double *y, cudaStream_t s) {
    launch_rows(n, nnz, row_ptr, col, Plain<double>{val, x}, y, s);
}

void spmv_f32(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const float *val, const float *x,
              float *y, cudaStream_t s) {
    launch_rows(n, nnz, row_ptr, col, Plain<float>{val, x}, y, s);
}

void spmv_hilo(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const float *hi, const float *lo,
               const double *x, const float *x32, double *y, cudaStream_t s) {
    launch_rows(n, nnz, row_ptr, col, HiLo{hi, lo, x, x32}, y, s);
}

}  // namespace cigpu
