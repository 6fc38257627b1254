// FP64 instantiation of the z pass (N and K operators).
#include "matvec_impl.cuh"

namespace marie {
using V64 = MatvecLaunch<double>::V;
template cudaError_t MatvecLaunch<double>::zmul(V64*, long long, const V64*, int, const Dims&, const V64*, int,
                                                cudaStream_t, int, int, const ZTile*);
}  // namespace marie
