// force_fp64.cu -- the plain FP64 force kernels.  Built with -fmad=false so
// every pair term is rounded operation by operation as in the reference.
#define COMDGB_FT_FLOAT 0
#define FT double
#include "force_launch.cuh"
