// Batched search kernels: binary64, 1 lane per atom (both register variants).
#include "search_kernel.cuh"

FLYGPU_SEARCH_KERNELS(false, 1)
