// Value formats shared by the CRS matvec (spmv.cu) and the values-only FCI
// matvec (slots.cu).
#pragma once

#include "checked.cuh"
#include "cigpu_internal.h"

namespace cigpu {

// Value formats. A format holds the matrix values and x; it loads 4 values with
// 16-byte loads (load4) and accumulates value * x[col] for one of them (term), or
// loads one value and accumulates it (term1).
//   Plain<VT>: VT values, VT x/y, VT accumulation (FP64 method, FP32 matvec).
//   HiLo: FP64 product from split FP32 values v = hi + lo (|v - hi - lo| <= 2^-48 |v|):
//     hi * x accumulates in FP64 (one DFMA per element); lo * x is at most 2^-24 of
//     the term, so it accumulates in FP32 from an FP32 copy of x (x32), adding below
//     2^-48 relative error while keeping FP64 instructions to one per element
//     (GB300 issues FP64 at 1/64 of the FP32 rate).
// Starts an L2 prefetch of `bytes` (a multiple of 16) at the 16-byte aligned `p`: a
// bulk hint with nothing to wait for.
__device__ __forceinline__ void l2_prefetch_bulk(const void *p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

template <typename VT>
struct Plain {
    using X = VT;
    const VT *__restrict__ val;
    const VT *__restrict__ x;
    uint64_t nx = ~(uint64_t)0;           // length of x (checked build: columns are tested against it)
    unsigned long long *err = nullptr;    // checked build: the error word
    struct Acc {  // value-initialise (Acc a{}) to zero
        VT s;
    };
    struct Chunk {
        VT v[4];
    };
    __device__ __forceinline__ void load4(int64_t at, Chunk &c) const;
    // one value into slot 0 of a chunk (the unaligned ends of a CRS row)
    __device__ __forceinline__ void load1(int64_t at, Chunk &c) const { c.v[0] = __ldcs(val + at); }
    // L2 prefetch of the values [at, at + n) (at and n multiples of 16 bytes' worth)
    __device__ __forceinline__ void prefetch(int64_t at, int64_t n) const {
        l2_prefetch_bulk(val + at, (uint32_t)(n * sizeof(VT)));
    }
    __device__ __forceinline__ void zero(Chunk &c) const { c.v[0] = c.v[1] = c.v[2] = c.v[3] = 0; }
    __device__ __forceinline__ void term(const Chunk &c, int j, int64_t col, Acc &a) const {
        if (!CIGPU_CHECK(err, index_ok((uint64_t)col, nx), kCheckColumn, col)) return;
        a.s += c.v[j] * __ldg(x + col);
    }
    __device__ __forceinline__ void term1(int64_t at, int64_t col, Acc &a) const {
        if (!CIGPU_CHECK(err, index_ok((uint64_t)col, nx), kCheckColumn, col)) return;
        a.s += __ldcs(val + at) * __ldg(x + col);
    }
    __device__ __forceinline__ void reduce(Acc &a, unsigned mask, int o) const { a.s += __shfl_xor_sync(mask, a.s, o); }
    __device__ __forceinline__ void add(Acc &a, const Acc &b) const { a.s += b.s; }
    __device__ __forceinline__ X result(const Acc &a) const { return a.s; }
};
template <>
__device__ __forceinline__ void Plain<double>::load4(int64_t at, Chunk &c) const {
    const double2 a = __ldcs(reinterpret_cast<const double2 *>(val + at));
    const double2 b = __ldcs(reinterpret_cast<const double2 *>(val + at) + 1);
    c.v[0] = a.x; c.v[1] = a.y; c.v[2] = b.x; c.v[3] = b.y;
}
template <>
__device__ __forceinline__ void Plain<float>::load4(int64_t at, Chunk &c) const {
    const float4 a = __ldcs(reinterpret_cast<const float4 *>(val + at));
    c.v[0] = a.x; c.v[1] = a.y; c.v[2] = a.z; c.v[3] = a.w;
}

// Format conversions assembled from the IEEE-754 bit fields on the integer pipe
// (GB300 runs float<->double conversions on its FP64 pipe, 1/64 of the FP32 rate).
// float -> double, exact for zero and normal floats (the split values are 0 or
// normal: |v| > 1e-14); Inf/NaN keep their class.
__device__ __forceinline__ double f2d_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    const uint64_t ed = e == 0 ? 0 : (e == 0xFFu ? 0x7FFull : (uint64_t)e + 896u);
    const uint64_t m = e == 0 ? 0 : (uint64_t)(u & 0x7FFFFFu) << 29;
    return __longlong_as_double((long long)(sign | (ed << 52) | m));
}
// double -> float by truncation (relative error below 2^-23); magnitudes below
// 2^-126 flush to zero, above the float range become Inf.
__device__ __forceinline__ float d2f_trunc(double d) {
    const uint64_t u = (uint64_t)__double_as_longlong(d);
    const int e = (int)((u >> 52) & 0x7FF) - 896;
    const uint32_t sign = (uint32_t)(u >> 63) << 31;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((uint32_t)e << 23) | (uint32_t)((u >> 29) & 0x7FFFFFu));
}

struct HiLo {
    using X = double;
    const float *__restrict__ hi;
    const float *__restrict__ lo;
    const double *__restrict__ x;
    const float *__restrict__ x32;  // FP32 copy of x
    uint64_t nx = ~(uint64_t)0;           // length of x (checked build: columns are tested against it)
    unsigned long long *err = nullptr;    // checked build: the error word
    struct Acc {  // value-initialise (Acc a{}) to zero
        double d;
        float f;
    };
    struct Chunk {
        float4 h, l;
    };
    __device__ __forceinline__ void load4(int64_t at, Chunk &c) const {
        c.h = __ldcs(reinterpret_cast<const float4 *>(hi + at));
        c.l = __ldcs(reinterpret_cast<const float4 *>(lo + at));
    }
    __device__ __forceinline__ void load1(int64_t at, Chunk &c) const {
        c.h.x = __ldcs(hi + at);
        c.l.x = __ldcs(lo + at);
    }
    __device__ __forceinline__ void prefetch(int64_t at, int64_t n) const {
        l2_prefetch_bulk(hi + at, (uint32_t)(n * sizeof(float)));
        l2_prefetch_bulk(lo + at, (uint32_t)(n * sizeof(float)));
    }
    __device__ __forceinline__ void zero(Chunk &c) const { c.h = c.l = make_float4(0, 0, 0, 0); }
    __device__ __forceinline__ void term(const Chunk &c, int j, int64_t col, Acc &a) const {
        if (!CIGPU_CHECK(err, index_ok((uint64_t)col, nx), kCheckColumn, col)) return;
        const float h = j == 0 ? c.h.x : j == 1 ? c.h.y : j == 2 ? c.h.z : c.h.w;
        const float l = j == 0 ? c.l.x : j == 1 ? c.l.y : j == 2 ? c.l.z : c.l.w;
        a.d = ::fma(f2d_bits(h), __ldg(x + col), a.d);
        a.f = fmaf(l, __ldg(x32 + col), a.f);
    }
    __device__ __forceinline__ void term1(int64_t at, int64_t col, Acc &a) const {
        if (!CIGPU_CHECK(err, index_ok((uint64_t)col, nx), kCheckColumn, col)) return;
        a.d = ::fma(f2d_bits(__ldcs(hi + at)), __ldg(x + col), a.d);
        a.f = fmaf(__ldcs(lo + at), __ldg(x32 + col), a.f);
    }
    __device__ __forceinline__ void reduce(Acc &a, unsigned mask, int o) const {
        a.d += __shfl_xor_sync(mask, a.d, o);
        a.f += __shfl_xor_sync(mask, a.f, o);
    }
    __device__ __forceinline__ void add(Acc &a, const Acc &b) const {
        a.d += b.d;
        a.f += b.f;
    }
    __device__ __forceinline__ X result(const Acc &a) const { return a.d + f2d_bits(a.f); }
};

}  // namespace cigpu
