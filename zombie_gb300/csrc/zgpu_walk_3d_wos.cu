// zgpu_walk_3d_wos.cu -- instantiates the 3D Walk on Spheres kernels.
#include "zgpu_wave.cuh"

template struct zg::WalkLaunch<3, ZGPU_SOLVER_WALK_ON_SPHERES>;
template struct zg::WaveLaunch<3, ZGPU_SOLVER_WALK_ON_SPHERES>;
