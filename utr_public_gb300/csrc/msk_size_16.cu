// Kernel instantiations for line length 16 (row passes for ny = 16, column passes for nx = 16).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(16)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(16)
