// Values-only FCI matvec of the mixed method (slots.cu).
#pragma once

#include "build.cuh"

namespace cigpu {

constexpr size_t kSlotsMaxSmem = 96 * 1024;  // slot descriptors of one row (8 bytes per slot)

// Whether the slot descriptors of a row fit in shared memory (W up to ~12,000).
bool slots_supported(const FciParams &p);
// Slot stride Wp: the row width rounded up to a multiple of 4.
int64_t slots_stride(const FciParams &p);
// y = H x from FP32 slot values, FP32 x/y and accumulation.
void spmv_slots_f32(const FciParams &p, const float *val, const float *x, float *y, cudaStream_t s);
// FP64 y = H x from the split slot values hi + lo.
void spmv_slots_hilo(const FciParams &p, const float *hi, const float *lo, const double *x, double *y,
                     cudaStream_t s);

}  // namespace cigpu
