// FP64 instantiation of the matvec passes.
#include "matvec_impl.cuh"
template struct marie::MatvecLaunch<double>;
