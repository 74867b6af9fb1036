// Kernel instantiations for line length 32 (row passes for ny = 32, column passes for nx = 32).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(32)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(32)
