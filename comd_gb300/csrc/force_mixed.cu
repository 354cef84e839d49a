// force_mixed.cu -- the mixed-precision force kernels: FP32 pair terms on
// box-relative coordinates, Kahan-compensated FP32 per-atom sums.
#define COMDGB_FT_FLOAT 1
#define FT float
#include "force_launch.cuh"
