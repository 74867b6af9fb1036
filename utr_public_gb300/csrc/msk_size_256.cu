// Kernel instantiations for line length 256 (row passes for ny = 256, column passes for nx = 256).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(256)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(256)
