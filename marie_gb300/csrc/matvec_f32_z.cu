// FP32 instantiation of the z pass (N and K operators, autotuner variants).
#include "matvec_impl.cuh"

namespace marie {
using V32 = MatvecLaunch<float>::V;
template cudaError_t MatvecLaunch<float>::zmul(V32*, long long, const V32*, int, const Dims&, const V32*, int,
                                               cudaStream_t, int, int, const ZTile*);
}  // namespace marie
