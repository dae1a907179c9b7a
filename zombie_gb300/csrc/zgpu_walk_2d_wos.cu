// zgpu_walk_2d_wos.cu -- instantiates the 2D Walk on Spheres kernels.
#include "zgpu_wave.cuh"

template struct zg::WalkLaunch<2, ZGPU_SOLVER_WALK_ON_SPHERES>;
template struct zg::WaveLaunch<2, ZGPU_SOLVER_WALK_ON_SPHERES>;
