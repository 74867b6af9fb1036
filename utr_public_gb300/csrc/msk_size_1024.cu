// Kernel instantiations for line length 1024 (row passes for ny = 1024, column passes for nx = 1024).
#include "msk_launch.cuh"
MSK_INSTANTIATE_SIZE(1024)
#include "utr_launch.cuh"
UTR_INSTANTIATE_SIZE(1024)
