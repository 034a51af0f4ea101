// Optimized kernels: gaussian transfer function, f16 volume storage.
#define DVR_FAST_DEFINE
#include "dvr_fast_launch.cuh"
using namespace dvr;
DVR_INSTANTIATE_FAST(3, __half)
