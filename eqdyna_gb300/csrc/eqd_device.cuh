// Device-side helpers shared by the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "eqd_internal.h"

namespace eqd {

#define EQD_CUDA_OK(expr)                                   \
  do {                                                      \
    cudaError_t e_ = (expr);                                \
    if (e_ != cudaSuccess) return EQD_ERR_CUDA;             \
  } while (0)

// Constants of one element pass.
struct ElemConst {
  double dt;
  double rdampk;     // already multiplied by dt
  double rdampm;     // mass-proportional damping
  double gz;         // (1 - C_elastic) * grav * (roumax - (gamar + 1) rhow) / roumax
  double ccosphi, sinphi;
  double relax;      // exp(-dt / tv), Drucker-Prager visco-plastic relaxation
};

// Signs of the four hourglass base patterns used by the viscous form (src/hrglss.f90:60-63).
__device__ __forceinline__ double viscous_pattern(int m, int a) {
  // rows: (1,1,-1,-1,-1,-1,1,1) (1,-1,-1,1,-1,1,1,-1) (1,-1,1,-1,1,-1,1,-1) (1,-1,1,-1,-1,1,-1,1)
  const unsigned neg[4] = {0x3Cu, 0x96u, 0xAAu, 0x5Au};  // bit a set -> -1
  return ((neg[m] >> a) & 1u) ? -1.0 : 1.0;
}

// Warp-aggregated 64-bit counter increment.
__device__ __forceinline__ void warp_count_add(unsigned long long *ctr, unsigned v) {
  unsigned s = __reduce_add_sync(__activemask(), v);
  if ((threadIdx.x & 31) == (__ffs(__activemask()) - 1)) atomicAdd(ctr, (unsigned long long)s);
}

}  // namespace eqd
