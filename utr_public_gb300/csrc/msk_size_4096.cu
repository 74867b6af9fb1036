// Kernel instantiations for line length 4096 (row passes for ny = 4096, column passes for nx = 4096).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(4096)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(4096)
