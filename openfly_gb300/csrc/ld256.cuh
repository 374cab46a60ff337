// ld256.cuh -- 256-bit read-only global loads (PTX ld.global.nc.v8.f32, sm_100 and later): a 32-byte
// record (a binary32 slot record, a merged spline record) in one load request instead of two.
#pragma once

#include <cuda_runtime.h>

namespace flygpu {

  // p must be 32-byte aligned and unchanged for the life of the calling kernel.
  __device__ __forceinline__ void ld256(void const* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
  }

}  // namespace flygpu
