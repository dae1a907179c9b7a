// zgpu_walk_3d_wost.cu -- instantiates the 3D Walk on Stars kernels (persistent and wavefront).
#include "zgpu_wave.cuh"

template struct zg::WalkLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>;
template struct zg::WaveLaunch<3, ZGPU_SOLVER_WALK_ON_STARS>;
