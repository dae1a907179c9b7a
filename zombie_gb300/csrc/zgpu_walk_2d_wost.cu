// zgpu_walk_2d_wost.cu -- instantiates the 2D Walk on Stars kernels (persistent and wavefront).
#include "zgpu_wave.cuh"

template struct zg::WalkLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>;
template struct zg::WaveLaunch<2, ZGPU_SOLVER_WALK_ON_STARS>;
