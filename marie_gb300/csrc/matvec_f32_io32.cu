// FP32 instantiation of the x/xy passes on FP32 vectors (the inner solves of
// mixed-precision refinement).
#include "matvec_impl.cuh"

namespace marie {
using V32 = MatvecLaunch<float>::V;
template cudaError_t MatvecLaunch<float>::xyfwd<float2>(const float2*, long long, const int*, Prologue, V32*,
                                                     long long, const Dims&, const V32*, const V32*, int, cudaStream_t,
                                                     int);
template cudaError_t MatvecLaunch<float>::yxinv<float2>(const V32*, long long, const float2*, long long, const int*,
                                                     Epilogue, float2*, long long, const Dims&, const V32*, const V32*,
                                                     int, cudaStream_t, int);
template cudaError_t MatvecLaunch<float>::xfwd<float2>(const float2*, long long, const int*, Prologue, V32*, long long,
                                                    const Dims&, const V32*, int, cudaStream_t);
template cudaError_t MatvecLaunch<float>::xinv<float2>(const V32*, long long, const float2*, long long, const int*,
                                                    Epilogue, float2*, long long, const Dims&, const V32*, int,
                                                    cudaStream_t);
}  // namespace marie
