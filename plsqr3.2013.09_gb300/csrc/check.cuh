// Bounds checks of the checked build (-DPLSQR_CHECK, `build(check=True)`):
// a failed check records its bit in the translation unit's check word and
// the kernel skips the access; plsqr_check_flags reads the words.  In the
// normal build every check is the constant true and compiles away.
#pragma once

#include <cuda_runtime.h>

namespace plsqr {

enum CheckBit : unsigned {
  kChkSlot = 1u,    // a unit slot (index or value) outside the layout
  kChkGather = 2u,  // a slab-local index outside the staged slab
  kChkLine = 4u,    // a line index outside the matrix, or a unit's line slot past 32
  kChkLane = 8u,    // a combiner lane outside the warp
  kChkFill = 16u,   // a fill or reorder address outside the layout
};

static __device__ unsigned int g_check_word;

__device__ __forceinline__ bool chk(bool ok, unsigned bit) {
#ifdef PLSQR_CHECK
  if (!ok) atomicOr(&g_check_word, bit);
  return ok;
#else
  (void)ok;
  (void)bit;
  return true;
#endif
}

// This translation unit's word (cleared after reading when reset).
static inline unsigned check_word(bool reset) {
  unsigned v = 0;
  if (cudaMemcpyFromSymbol(&v, g_check_word, sizeof v) != cudaSuccess) return ~0u;
  if (reset) {
    const unsigned z = 0;
    if (cudaMemcpyToSymbol(g_check_word, &z, sizeof z) != cudaSuccess) return ~0u;
  }
  return v;
}

}  // namespace plsqr
