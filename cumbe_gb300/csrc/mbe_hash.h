// Canonical biclique hash shared by the host library and the kernels.
//
// A biclique (A, B) is given in file orientation: A = row-side ids,
// B = col-side ids.  The per-biclique hash depends only on the two SETS
// (element order never matters), so the enumeration kernels can sum
// per-element terms in any order instead of sorting every biclique:
//
//   e_row(a) = fmix64(a + 0x9E3779B97F4A7C15)
//   e_col(b) = fmix64(b + 0xD1B54A32D192ED03)
//   SA = sum e_row(a)  (mod 2^64),   SB = sum e_col(b)  (mod 2^64)
//   h(A,B)   = fmix64(SA ^ fmix64(SB + (|A| << 32 | |B|)))
//
// fmix64 is the splitmix64 output mixer (Steele, Lea, Flood 2014).
// The graph hash is the wrapping sum of h over all maximal bicliques.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define MBE_HD __host__ __device__ __forceinline__
#else
#define MBE_HD static inline
#endif

MBE_HD uint64_t mbe_fmix64(uint64_t z) {
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ULL;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return z;
}

MBE_HD uint64_t mbe_elem_row(uint32_t a) { return mbe_fmix64((uint64_t)a + 0x9E3779B97F4A7C15ULL); }
MBE_HD uint64_t mbe_elem_col(uint32_t b) { return mbe_fmix64((uint64_t)b + 0xD1B54A32D192ED03ULL); }

MBE_HD uint64_t mbe_pair_hash(uint64_t sum_rows, uint32_t n_rows, uint64_t sum_cols, uint32_t n_cols) {
    uint64_t sizes = ((uint64_t)n_rows << 32) | (uint64_t)n_cols;
    return mbe_fmix64(sum_rows ^ mbe_fmix64(sum_cols + sizes));
}
