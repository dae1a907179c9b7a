// zgpu_kernels2.cu -- instantiates the 2D kernels of zgpu_kernels.cuh.
#include "zgpu_kernels.cuh"

template struct zg::Launch<2>;
