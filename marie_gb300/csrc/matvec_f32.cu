// FP32 instantiation of the matvec passes.
#include "matvec_launch.cuh"
template struct marie::MatvecLaunch<float>;
