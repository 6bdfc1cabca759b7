// Bounds checks of the checked build (compiled with -DCIGPU_CHECKED into
// libcigpu_checked.so; the regular library compiles them out).
//
// The checked kernels test every index they derive from stored data or from a
// rank formula before the access it guards: matrix columns against the vector
// length, CRS row bounds against each other, DOCI hop ranks against the space,
// RDM pair and term indices against their tables. A failed check skips the access
// (the term counts as zero) and records the first violation in a device error
// word with atomicCAS: code << 56 | the offending index (its low 56 bits). No
// kernel traps or stops; the host reads the word through cigpu_check_word. The
// reference keeps the same checks in its matrix accessors (matrix.cpp:676-677,
// SparseMatrix_CRS.cpp:691-693), where a failure ends the program.
#pragma once

#include <cstdint>

namespace cigpu {

enum CheckCode : uint32_t {
    kCheckNone = 0,
    kCheckColumn = 1,     // a matvec column (CRS or generated) >= the vector length
    kCheckRowBounds = 2,  // CRS row pointers decreasing, or a row longer than the matrix is wide
    kCheckHopRank = 3,    // a generated DOCI pair-hop rank >= the space size
    kCheckRdmPair = 4,    // an RDM string-pair index >= the string count
    kCheckRdmTerm = 5,    // an RDM term index >= the pair-density count
    kCheckRdmExcit = 6,   // an RDM excitation's string index >= the string count
};

// The record of a violation: the code in the top byte, the index below it.
__host__ __device__ inline uint64_t check_record(uint32_t code, uint64_t index) {
    return ((uint64_t)code << 56) | (index & 0x00FFFFFFFFFFFFFFull);
}
__host__ __device__ inline uint32_t check_record_code(uint64_t word) { return (uint32_t)(word >> 56); }
__host__ __device__ inline uint64_t check_record_index(uint64_t word) { return word & 0x00FFFFFFFFFFFFFFull; }

// The predicate every check uses: an index is valid when it lies in [0, bound).
__host__ __device__ inline bool index_ok(uint64_t index, uint64_t bound) { return index < bound; }
// A CRS row [s, e) of a matrix n wide: s <= e and at most n entries.
__host__ __device__ inline bool row_ok(int64_t s, int64_t e, int64_t n) { return s >= 0 && s <= e && e - s <= n; }

#if defined(CIGPU_CHECKED) && defined(__CUDACC__)
// Keeps the first violation (later ones leave the word unchanged).
__device__ __forceinline__ void check_fail(unsigned long long *word, uint32_t code, uint64_t index) {
    if (word) atomicCAS(word, 0ull, (unsigned long long)check_record(code, index));
}
#define CIGPU_CHECKED_BUILD 1
// True when `cond` holds; otherwise records (code, index) in *word and is false.
#define CIGPU_CHECK(word, cond, code, index) \
    ((cond) ? true : (::cigpu::check_fail((word), (code), (uint64_t)(index)), false))
#else
#define CIGPU_CHECKED_BUILD 0
#define CIGPU_CHECK(word, cond, code, index) true
#endif

// Device address of the current device's error word (allocated on first use;
// nullptr in the regular build).
unsigned long long *check_word_device();

}  // namespace cigpu
