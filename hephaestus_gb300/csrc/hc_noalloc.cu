// hc_noalloc.cu -- hc_curl_static: B = curl A with host vectors and no device
// allocation during the call.
//
// hc_curl stages B in a device buffer it allocates per call.  This variant
// stages B in a fixed area of static device memory instead, so the call itself
// allocates nothing: the area is part of this library's device image, reserved
// when the runtime loads the library's device code on a device.
//  * size: HC_CURL_STATIC_MAX_RT_DOFS doubles (8 MiB); larger grids are
//    rejected with HC_EINVAL before any work is enqueued.
//  * set-up: the first call on each device looks the area up with
//    cudaGetSymbolAddress while that device is current and keeps the pointer
//    (one per device).  That lookup may load this library's device code on the
//    device, so the first call should come before any stream capture.
//  * zeroing: the area is cleared (cudaMemsetAsync) before each launch.  The
//    curl kernel writes every Raviart-Thomas dof, so the clear only keeps stale
//    values of an earlier, larger call from ever reaching B.
//  * concurrency: all callers on one device share the one area.  Calls that
//    overlap in time on the same device (two host threads, or two streams)
//    race on it and must be serialised by the caller.
#include <mutex>
#include <string>

#include "hc_internal.h"

namespace {

constexpr int kMaxDevices = 64;
static_assert(HC_CURL_STATIC_MAX_RT_DOFS == (1 << 20), "header and scratch size disagree");

// staging area of B (reference-element RT flux), one per device
static __device__ __align__(256) double g_curl_scratch[HC_CURL_STATIC_MAX_RT_DOFS];

std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Pointer of the staging area on the current device; nullptr on failure
// (reason in h->err).
double* scratch_on_current_device(hcop* h) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    h->err = std::string("hc_curl_static: cudaGetDevice: ") + cudaGetErrorString(e);
    return nullptr;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    h->err = "hc_curl_static: device ordinal beyond the supported 64 devices";
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_curl_scratch);
    if (e != cudaSuccess || !p) {
      h->err = std::string("hc_curl_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return nullptr;
    }
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  return g_scratch_ptr[dev];
}

}  // namespace

extern "C" hc_status hc_curl_static(hcop_t* h, const double* A, double* B) {
  if (!h || !A || !B) return HC_EINVAL;
  if (h->type != HC_HEX) {
    h->err = "hc_curl_static: structured hex grids only in this build";
    return HC_ENOTSUP;
  }
  int64_t o1, o2, nrt;
  hc::hex_rt_layout(h->hexdev(), &o1, &o2, &nrt);
  if (nrt > HC_CURL_STATIC_MAX_RT_DOFS) {
    h->err = "hc_curl_static: " + std::to_string(nrt) + " Raviart-Thomas dofs exceed the static scratch of " +
             std::to_string(HC_CURL_STATIC_MAX_RT_DOFS) + " doubles (8 MiB); use hc_curl";
    return HC_EINVAL;
  }
  double* dB = scratch_on_current_device(h);
  if (!dB) return HC_ECUDA;
  HC_CUDA_TRY(h, cudaMemcpyAsync(h->xbuf, A, h->ndof * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  HC_CUDA_TRY(h, cudaMemsetAsync(dB, 0, nrt * sizeof(double), h->stream));
  HC_CUDA_TRY(h, hc::hex_curl(h->hexdev(), h->xbuf, dB, h->stream));
  HC_CUDA_TRY(h, cudaMemcpyAsync(B, dB, nrt * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  HC_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return HC_OK;
}
