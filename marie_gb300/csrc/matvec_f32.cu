// FP32 instantiation of the matvec passes other than the z pass (the z pass,
// with its schedule variants, is instantiated in matvec_f32_z.cu so the two
// halves compile in parallel).
#include "matvec_impl.cuh"

namespace marie {
using V32 = MatvecLaunch<float>::V;
template bool MatvecLaunch<float>::fused(const Dims&);
template cudaError_t MatvecLaunch<float>::xyfwd(const double2*, long long, const int*, Prologue, V32*, long long,
                                                const Dims&, const V32*, const V32*, int, cudaStream_t, int);
template cudaError_t MatvecLaunch<float>::yxinv(const V32*, long long, const double2*, long long, const int*,
                                                Epilogue, double2*, long long, const Dims&, const V32*, const V32*,
                                                int, cudaStream_t, int);
template cudaError_t MatvecLaunch<float>::xfwd(const double2*, long long, const int*, Prologue, V32*, long long,
                                               const Dims&, const V32*, int, cudaStream_t);
template cudaError_t MatvecLaunch<float>::xinv(const V32*, long long, const double2*, long long, const int*, Epilogue,
                                               double2*, long long, const Dims&, const V32*, int, cudaStream_t);
template cudaError_t MatvecLaunch<float>::cols(bool, int, const V32*, long long, long long, int, V32*, long long,
                                               long long, int, int, int, const V32*, int, cudaStream_t, const int*,
                                               int);
}  // namespace marie
