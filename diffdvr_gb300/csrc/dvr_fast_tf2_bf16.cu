// Optimized kernels: linear transfer function, bf16 volume storage.
#define DVR_FAST_DEFINE
#include "dvr_fast_launch.cuh"
using namespace dvr;
DVR_INSTANTIATE_FAST(2, __nv_bfloat16)
