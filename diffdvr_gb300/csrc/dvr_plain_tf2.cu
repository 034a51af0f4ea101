// Plain kernels for the linear transfer function.
#include "dvr_plain_launch.cuh"
using namespace dvr;
DVR_INSTANTIATE_PLAIN(2)
