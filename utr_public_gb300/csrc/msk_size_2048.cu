// Kernel instantiations for line length 2048 (row passes for ny = 2048, column passes for nx = 2048).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(2048)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(2048)
