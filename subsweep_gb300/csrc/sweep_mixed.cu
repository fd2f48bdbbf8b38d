// Mixed-precision kernels: FP32 transport (scaled photon rates, FP32 face weights,
// exact face classification), FP64 chemistry with the neutral fraction carried as
// its own state, FP64 level assignment.  FMA contraction allowed.
#define SWK_R float
#define SWK_CARRY true
#define SWK_OPS kOpsMixed
#define SWK_NAME "mixed"
#define SWK_PULL 1
#include "sweep_ops.cuh"
