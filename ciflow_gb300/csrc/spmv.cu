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
#include "spmv.cuh"

namespace cigpu {

namespace {

template <typename T>
__device__ __forceinline__ T ld_stream(const T *p) {
    return __ldcs(p);
}

// Row body with 16-byte loads: 4 columns (uint4) and 4 values (2x double2 or float4).
template <typename VT>
struct Vec4;
template <>
struct Vec4<double> {
    __device__ __forceinline__ static void load(const double *p, double v[4]) {
        const double2 a = __ldcs(reinterpret_cast<const double2 *>(p));
        const double2 b = __ldcs(reinterpret_cast<const double2 *>(p) + 1);
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
};
template <>
struct Vec4<float> {
    __device__ __forceinline__ static void load(const float *p, float v[4]) {
        const float4 a = __ldcs(reinterpret_cast<const float4 *>(p));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
};

// G lanes per row (32, 16 or 8 for shorter rows); each lane issues U 16-byte
// column loads and U value loads before its 4U gathers of x, so enough bytes are
// in flight to cover HBM latency (a single chunk per lane left the kernel
// latency-bound on the dependent gathers).
template <typename VT, int G, int U>
__global__ void __launch_bounds__(kSpmvThreads) k_spmv_rows(int64_t n, const int64_t *__restrict__ row_ptr,
                                                            const uint32_t *__restrict__ col,
                                                            const VT *__restrict__ val, const VT *__restrict__ x,
                                                            VT *__restrict__ y) {
    const int lane = threadIdx.x & (G - 1);
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t r = gid; r < n; r += ng) {
        const int64_t s = row_ptr[r], e = row_ptr[r + 1];
        VT acc = 0;
        // scalar head up to a 16-byte boundary of both arrays (4 elements)
        const int64_t s4 = (s + 3) & ~(int64_t)3;
        const int64_t head_end = s4 < e ? s4 : e;
        if (s + lane < head_end) acc += __ldcs(val + s + lane) * __ldg(x + __ldcs(col + s + lane));
        const int64_t nb = (e > s4) ? ((e - s4) >> 2) : 0;
        const uint4 *c4 = reinterpret_cast<const uint4 *>(col + s4);
        const VT *v4 = val + s4;
        for (int64_t b0 = 0; b0 < nb; b0 += G * U) {
            uint4 c[U];
            VT v[U][4];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t idx = b0 + u * G + lane;
                if (idx < nb) {
                    c[u] = __ldcs(c4 + idx);
                    Vec4<VT>::load(v4 + (idx << 2), v[u]);
                } else {
                    c[u] = make_uint4(0, 0, 0, 0);
                    v[u][0] = v[u][1] = v[u][2] = v[u][3] = 0;
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (b0 + u * G + lane < nb) {
                    acc += v[u][0] * __ldg(x + c[u].x);
                    acc += v[u][1] * __ldg(x + c[u].y);
                    acc += v[u][2] * __ldg(x + c[u].z);
                    acc += v[u][3] * __ldg(x + c[u].w);
                }
            }
        }
        // scalar tail (< 4 elements)
        const int64_t t0 = s4 + (nb << 2);
        if (e > s4 && t0 + lane < e) acc += __ldcs(val + t0 + lane) * __ldg(x + __ldcs(col + t0 + lane));
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o);
        if (lane == 0) y[r] = acc;
    }
}

// FP64 product from split FP32 values: v = (double)hi + (double)lo.
__global__ void __launch_bounds__(kSpmvThreads) k_spmv_hilo(int64_t n, const int64_t *__restrict__ row_ptr,
                                                            const uint32_t *__restrict__ col,
                                                            const float *__restrict__ hi, const float *__restrict__ lo,
                                                            const double *__restrict__ x, double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = wid; r < n; r += nw) {
        const int64_t s = row_ptr[r], e = row_ptr[r + 1];
        double acc = 0;
        for (int64_t k = s + lane; k < e; k += 32) {
            const double v = (double)__ldcs(hi + k) + (double)__ldcs(lo + k);
            acc += v * __ldg(x + __ldcs(col + k));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) y[r] = acc;
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

// lanes per row from the mean row length (in 4-element chunks)
template <typename VT>
static void launch_rows(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const VT *val, const VT *x,
                        VT *y, cudaStream_t s) {
    const double chunks = n > 0 ? (double)nnz / n / 4.0 : 0;
    if (chunks >= 48)
        k_spmv_rows<VT, 32, 4><<<spmv_grid(), kSpmvThreads, 0, s>>>(n, row_ptr, col, val, x, y);
    else if (chunks >= 20)
        k_spmv_rows<VT, 16, 4><<<spmv_grid(), kSpmvThreads, 0, s>>>(n, row_ptr, col, val, x, y);
    else
        k_spmv_rows<VT, 8, 4><<<spmv_grid(), kSpmvThreads, 0, s>>>(n, row_ptr, col, val, x, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

void spmv_f64(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const double *val, const double *x,
              double *y, cudaStream_t s) {
    launch_rows<double>(n, nnz, row_ptr, col, val, x, y, s);
}

void spmv_f32(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const float *val, const float *x,
              float *y, cudaStream_t s) {
    launch_rows<float>(n, nnz, row_ptr, col, val, x, y, s);
}

void spmv_hilo(int64_t n, const int64_t *row_ptr, const uint32_t *col, const float *hi, const float *lo,
               const double *x, double *y, cudaStream_t s) {
    k_spmv_hilo<<<spmv_grid(), kSpmvThreads, 0, s>>>(n, row_ptr, col, hi, lo, x, y);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace cigpu
