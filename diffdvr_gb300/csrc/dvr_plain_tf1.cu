// Plain kernels for the texture transfer function.
#include "dvr_plain_launch.cuh"
using namespace dvr;
DVR_INSTANTIATE_PLAIN(1)
