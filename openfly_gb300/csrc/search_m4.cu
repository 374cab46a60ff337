// Batched search kernels: binary32 pairs / binary64 accumulation, 4 lanes per atom (both register variants).
#include "search_kernel.cuh"

FLYGPU_SEARCH_KERNELS(true, 4)
