// FP64 instantiation of the matvec passes other than the z pass (instantiated
// in matvec_f64_z.cu so the two halves compile in parallel).
#include "matvec_impl.cuh"

namespace marie {
using V64 = MatvecLaunch<double>::V;
template bool MatvecLaunch<double>::fused(const Dims&);
template cudaError_t MatvecLaunch<double>::xyfwd<double2>(const double2*, long long, const int*, Prologue, V64*,
                                                     long long, const Dims&, const V64*, const V64*, int, cudaStream_t,
                                                     int);
template cudaError_t MatvecLaunch<double>::yxinv<double2>(const V64*, long long, const double2*, long long, const int*,
                                                     Epilogue, double2*, long long, const Dims&, const V64*, const V64*,
                                                     int, cudaStream_t, int);
template cudaError_t MatvecLaunch<double>::xfwd<double2>(const double2*, long long, const int*, Prologue, V64*, long long,
                                                    const Dims&, const V64*, int, cudaStream_t);
template cudaError_t MatvecLaunch<double>::xinv<double2>(const V64*, long long, const double2*, long long, const int*,
                                                    Epilogue, double2*, long long, const Dims&, const V64*, int,
                                                    cudaStream_t);
template cudaError_t MatvecLaunch<double>::cols(bool, int, const V64*, long long, long long, int, V64*, long long,
                                                long long, int, int, int, const V64*, int, cudaStream_t, const int*,
                                                int);
}  // namespace marie
