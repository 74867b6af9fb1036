// Kernel instantiations for line length 512 (row passes for ny = 512, column passes for nx = 512).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(512)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(512)
