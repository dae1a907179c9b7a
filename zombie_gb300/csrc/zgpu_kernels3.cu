// zgpu_kernels3.cu -- instantiates the 3D kernels of zgpu_kernels.cuh.
#include "zgpu_kernels.cuh"

template struct zg::Launch<3>;
