// Kernel instantiations for line length 128 (row passes for ny = 128, column passes for nx = 128).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(128)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(128)
