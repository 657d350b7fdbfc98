// hc_hex_p3.cu -- order-3 instantiations of the hex apply kernel (own translation unit
// so that the orders compile in parallel).
#include "hc_hex_impl.cuh"

namespace hc {
template cudaError_t hex_launch_p<double, 3>(const HexDev&, const double*, const double*, double*, double,
                                             double, bool, KrylovScalars*, double*, cudaStream_t, bool);
template cudaError_t hex_launch_p<float, 3>(const HexDev&, const float*, const float*, float*, float, float,
                                            bool, KrylovScalars*, double*, cudaStream_t, bool);
template cudaError_t hex_launch_pair<double, 3>(const HexDev&, const double*, const double*, const double*,
                                                double*, double, double, cudaStream_t);
template cudaError_t hex_launch_pair<float, 3>(const HexDev&, const float*, const float*, const float*, float*,
                                               float, float, cudaStream_t);
cudaError_t upload_tables_p3(const void* td, const void* tf) { return upload_tables_here(td, tf); }
}  // namespace hc
