// Kernel instantiations for line length 64 (row passes for ny = 64, column passes for nx = 64).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(64)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(64)
