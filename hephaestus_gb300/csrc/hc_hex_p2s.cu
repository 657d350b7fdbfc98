// hc_hex_p2s.cu -- order-2 instantiations of the tiled hex kernels for the
// second brick shape (8 x 8 x 2; own translation unit so that it compiles in
// parallel with the first shape's in hc_hex_p2.cu).
#include "hc_hex_cplx.cuh"

namespace hc {
template cudaError_t hex_launch_ps<double, 2, 1>(const HexDev&, const double*, const double*, double*, double,
                                                 double, bool, KrylovScalars*, double*, cudaStream_t, bool);
template cudaError_t hex_launch_ps<float, 2, 1>(const HexDev&, const float*, const float*, float*, float, float,
                                                bool, KrylovScalars*, double*, cudaStream_t, bool);
template cudaError_t hex_launch_cplx_ps<double, 2, 1>(const HexDev&, const double*, const double*, const double*,
                                                      double*, double*, double, double, bool, const int*,
                                                      cudaStream_t);
template cudaError_t hex_launch_cplx_ps<float, 2, 1>(const HexDev&, const float*, const float*, const float*,
                                                     float*, float*, float, float, bool, const int*, cudaStream_t);
cudaError_t upload_tables_p2s(const void* td, const void* tf) { return upload_tables_here(td, tf); }
}  // namespace hc
