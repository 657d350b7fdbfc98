// hc_hex_p1.cu -- order-1 instantiations of the hex apply kernel (own translation unit
// so that the orders compile in parallel).
#include "hc_hex_cplx.cuh"

namespace hc {
template cudaError_t hex_launch_p<double, 1>(const HexDev&, const double*, const double*, double*, double,
                                             double, bool, KrylovScalars*, double*, cudaStream_t, bool);
template cudaError_t hex_launch_p<float, 1>(const HexDev&, const float*, const float*, float*, float, float,
                                            bool, KrylovScalars*, double*, cudaStream_t, bool);
template cudaError_t hex_launch_cplx_p<double, 1>(const HexDev&, const double*, const double*, const double*,
                                                  double*, double*, double, double, bool, const int*, cudaStream_t);
template cudaError_t hex_launch_cplx_p<float, 1>(const HexDev&, const float*, const float*, const float*, float*,
                                                 float*, float, float, bool, const int*, cudaStream_t);
cudaError_t upload_tables_p1(const void* td, const void* tf) { return upload_tables_here(td, tf); }
}  // namespace hc
