// Values-only FCI layout ("slot tiles", slots.cu): FP32 hi + lo for the mixed
// method, FP64 for the plain one.
#pragma once

#include "build.cuh"

namespace cigpu {

constexpr int kTileRows = 64;                // beta strings per tile (rows of one alpha string; 128 measured slower at L=11, 12)
constexpr size_t kSlotsMaxSmem = 96 * 1024;  // per-block shared memory of the slot kernels

// Whether the layout applies (its shared-memory tables fit; indices fit 32 bits).
bool slots_supported(const FciParams &p);
// Stored values (FP32 each, hi and lo arrays): tiles x kTileRows x padded row width.
int64_t slots_count(const FciParams &p);
// Fills the FP32 hi/lo slot values (needs the row singles and FP32 tables in p) and
// each row's stored-nonzero count and lower-triangle count (count, lower: [dim]).
void fill_slots_launch(const FciParams &p, float *hi, float *lo, uint32_t *count, uint32_t *lower, cudaStream_t s);
// Compact FP64 tiles (p.fly = 1): the alpha-single x beta-single block of every row
// (71% of the slots at L=12 6a6b) is not stored but formed by the FP64 matvec from
// the integrals; the product equals the full tiles' bit for bit (and takes ~40%
// longer). Whether the kernels' shared-memory tables fit for this space:
bool slots64_fly_fits(const FciParams &p);
// Values the FP64 tiles store: slots_count(p), or fewer with p.fly.
int64_t slots_stored(const FciParams &p);
// Fills FP64 slot values (|v| <= 1e-14 stored as zero; needs the FP64 row singles
// in p) and the same row counts: the plain method's tiles (compact with p.fly).
void fill_slots64_launch(const FciParams &p, double *v64, uint32_t *count, uint32_t *lower, cudaStream_t s);
// Whether FP64 tiles pay off: the tiles' padding rows add at most a quarter.
inline bool slots64_pay(const FciParams &p) {
    return ((p.Db + kTileRows - 1) / kTileRows) * kTileRows * 4 <= 5 * p.Db;
}
// Sizes (elements) of the matvecs' staging tables: slot descriptors per alpha
// string (uint64) and beta single targets per tile (uint32).
int64_t slot_desc_count(const FciParams &p);
int64_t slot_st_count(const FciParams &p);
// Fills both tables (p needs the string tables); the matvecs stage a tile's
// descriptors and targets from them with 16-byte loads.
void slot_tables_launch(const FciParams &p, uint64_t *desc, uint32_t *st, cudaStream_t s);
// y = H x from FP32 slot values, FP32 x/y and accumulation.
void spmv_slots_f32(const FciParams &p, const float *val, const float *x, float *y, cudaStream_t s);
// FP64 y = H x from FP64 slot values (one DFMA per slot).
void spmv_slots_f64(const FciParams &p, const double *val, const double *x, double *y, cudaStream_t s);
// FP64 y = H x from the split slot values hi + lo; x32 is an FP32 copy of x.
void spmv_slots_hilo(const FciParams &p, const float *hi, const float *lo, const double *x, const float *x32,
                     double *y, cudaStream_t s);

}  // namespace cigpu
