// Plain kernels for the gaussian transfer function.
#include "dvr_plain_launch.cuh"
using namespace dvr;
DVR_INSTANTIATE_PLAIN(3)
