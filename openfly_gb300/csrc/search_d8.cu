// Batched search kernels: binary64, 8 lanes per atom (both register variants).
#include "search_kernel.cuh"

FLYGPU_SEARCH_KERNELS(false, 8)
