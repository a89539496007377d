// Warp-level helpers shared by the sweep kernels (sdtw.cu, refdel.cu).
#pragma once

#include "dtwx_internal.h"

#define FULL_MASK 0xffffffffu

namespace dtwx {

// Work-queue ticket taken by lane 0 only, broadcast by the caller.
__device__ __forceinline__ int ticket_if(int32_t *counter, uint32_t pred) {
  int v;
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %2, 0;\n\tmov.u32 %0, 0;\n\t"
      "@p atom.global.add.u32 %0, [%1], 1;\n\t}"
      : "=r"(v)
      : "l"(counter), "r"(pred)
      : "memory");
  return v;
}

// 64-bit global min by the lanes whose pred is set, as predicated PTX.
__device__ __forceinline__ void red_min_if(unsigned long long *addr, unsigned long long v, uint32_t pred) {
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %2, 0;\n\t@p red.global.min.u64 [%0], %1;\n\t}" ::"l"(addr),
               "l"(v), "r"(pred)
               : "memory");
}

// Warp-wide lexicographic min of (value, column); column -1 (none) loses.
__device__ __forceinline__ void warp_argmin(float &v, int64_t &j) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    const float ov = __shfl_xor_sync(FULL_MASK, v, m);
    const int64_t oj = __shfl_xor_sync(FULL_MASK, j, m);
    if (ov < v || (ov == v && (uint64_t)oj < (uint64_t)j)) {
      v = ov;
      j = oj;
    }
  }
}

// Result key: orderable score in the high word, end column in the low word,
// so one 64-bit min keeps the lowest score and then the smallest column.
__device__ __forceinline__ unsigned long long make_key(float v, int64_t j) {
  return ((unsigned long long)float_to_ordered(v) << 32) | (unsigned long long)(uint32_t)j;
}

}  // namespace dtwx
