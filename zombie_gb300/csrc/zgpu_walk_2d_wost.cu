// zgpu_walk_2d_wost.cu -- instantiates the 2D Walk on Stars kernels.
#include "zgpu_kernels.cuh"

template struct zg::WalkLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>;
