// zgpu_walk_3d_wost.cu -- instantiates the 3D Walk on Stars kernels.
#include "zgpu_kernels.cuh"

template struct zg::WalkLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>;
