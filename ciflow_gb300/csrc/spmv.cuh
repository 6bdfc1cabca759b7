// CRS matrix-vector product launchers.
#pragma once

#include "cigpu_internal.h"

namespace cigpu {

constexpr int kSpmvThreads = 256;
constexpr int kSpmvBlocksPerSM = 8;

int sm_count_spmv();
int spmv_grid();
void spmv_f64(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const double *val, const double *x, double *y,
              cudaStream_t s);
// FP64 CRS matvec with an explicit shape: `lanes` (4, 8, 16 or 32) lanes per row,
// `grid` blocks of kSpmvThreads (the batched solver's autotuner picks both). With
// row_prob non-null, row r is skipped when status[row_prob[r]] != 0 (finished
// problems of a batch; y keeps its old value there).
void spmv_f64_shape(int64_t n, const int64_t *row_ptr, const uint32_t *col, const double *val, const double *x,
                    double *y, int lanes, int grid, cudaStream_t s, const int *row_prob = nullptr,
                    const int *status = nullptr);
void spmv_f32(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const float *val, const float *x, float *y,
              cudaStream_t s);

// x32: FP32 copy of x (for the low parts)
void spmv_hilo(int64_t n, int64_t nnz, const int64_t *row_ptr, const uint32_t *col, const float *hi, const float *lo,
               const double *x, const float *x32, double *y, cudaStream_t s);

}  // namespace cigpu
