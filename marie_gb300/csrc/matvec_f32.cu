// FP32 instantiation of the matvec passes other than the z pass, on FP64
// vectors (the z pass, with its schedule variants, is instantiated in
// matvec_f32_z.cu and the passes on FP32 vectors in matvec_f32_io32.cu, so
// the parts compile in parallel).
#include "matvec_impl.cuh"

namespace marie {
using V32 = MatvecLaunch<float>::V;
template bool MatvecLaunch<float>::fused(const Dims&);
template cudaError_t MatvecLaunch<float>::xyfwd<double2>(const double2*, long long, const int*, Prologue, V32*,
                                                     long long, const Dims&, const V32*, const V32*, int, cudaStream_t,
                                                     int);
template cudaError_t MatvecLaunch<float>::yxinv<double2>(const V32*, long long, const double2*, long long, const int*,
                                                     Epilogue, double2*, long long, const Dims&, const V32*, const V32*,
                                                     int, cudaStream_t, int);
template cudaError_t MatvecLaunch<float>::xfwd<double2>(const double2*, long long, const int*, Prologue, V32*, long long,
                                                    const Dims&, const V32*, int, cudaStream_t);
template cudaError_t MatvecLaunch<float>::xinv<double2>(const V32*, long long, const double2*, long long, const int*,
                                                    Epilogue, double2*, long long, const Dims&, const V32*, int,
                                                    cudaStream_t);
template cudaError_t MatvecLaunch<float>::cols(bool, int, const V32*, long long, long long, int, V32*, long long,
                                               long long, int, int, int, const V32*, int, cudaStream_t, const int*,
                                               int);
}  // namespace marie
