// hc_tune.cu -- launch autotuner of the tiled hex kernels: per problem (order,
// grid, axis-aligned or general parallelepipeds) it times each brick shape
// (16x4x2 and 8x8x2 elements) and CTA count per SM with CUDA events on the
// handle's stream and keeps the fastest.  Choices live in a process-wide
// table and, when the environment variable HC_TUNE_FILE names a file, in that
// file (one line per problem: p full nx ny nz shape per_sm us kind), so later
// processes start tuned: hc_create applies a stored entry for its key.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>

#include "hc_internal.h"
#include "hc_tune_table.h"

namespace hc {
namespace {

std::mutex g_mu;
std::map<TuneKey, TuneEntry> g_table;
bool g_loaded = false;

TuneKey key_of(const hcop* h) { return TuneKey{h->p, h->full ? 1 : 0, h->nx, h->ny, h->nz}; }

// entries of HC_TUNE_FILE (once per process)
void load_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const char* path = std::getenv("HC_TUNE_FILE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  tune_read(f, g_table);
  std::fclose(f);
}

void store_locked(const hcop* h, const TuneEntry& e, double us, int kind) {
  g_table[key_of(h)] = e;
  const char* path = std::getenv("HC_TUNE_FILE");
  if (path && *path) tune_append(path, key_of(h), e, us, kind);
}

}  // namespace

void tune_lookup(hcop* h) {
  if (h->type != HC_HEX || h->p > 2) return;
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  const auto it = g_table.find(key_of(h));
  if (it == g_table.end()) return;
  h->shape = it->second.shape;
  h->per_sm = it->second.per_sm;
}

}  // namespace hc

using namespace hc;

extern "C" {

hc_status hc_set_launch(hcop_t* h, int32_t shape, int32_t per_sm) {
  if (!h) return HC_EINVAL;
  if (h->type != HC_HEX) {
    h->err = "hc_set_launch: hex handles only";
    return HC_ENOTSUP;
  }
  if (shape < 0 || shape > 1 || (shape == 1 && h->p > 2) || per_sm < 0 || per_sm > 64) {
    h->err = "hc_set_launch: shape must be 0 or 1 (1 for orders 1-2), per_sm in 0..64";
    return HC_EINVAL;
  }
  h->shape = shape;
  h->per_sm = per_sm;
  return HC_OK;
}

hc_status hc_get_launch(const hcop_t* h, int32_t* shape, int32_t* per_sm) {
  if (!h || !shape || !per_sm) return HC_EINVAL;
  *shape = h->shape;
  *per_sm = h->per_sm;
  return HC_OK;
}

hc_status hc_autotune(hcop_t* h, int32_t kind, int32_t* shape, int32_t* per_sm, double* us_best,
                      double* us_default) {
  if (!h) return HC_EINVAL;
  if (h->type != HC_HEX || h->p > 2) {
    h->err = "hc_autotune: tiled kernels exist for hex handles of order 1-2";
    return HC_ENOTSUP;
  }
  if (kind != 0 && kind != 1) {
    h->err = "hc_autotune: kind must be 0 (real FP32 apply) or 1 (complex FP32 apply)";
    return HC_EINVAL;
  }
  const int64_t n = h->ndof;
  cudaStream_t s = h->stream;
  const int nv = kind ? 4 : 2;
  float* buf = nullptr;
  HC_CUDA_TRY(h, cudaMallocAsync((void**)&buf, (size_t)nv * n * sizeof(float), s));
  HC_CUDA_TRY(h, cudaMemsetAsync(buf, 0, (size_t)nv * n * sizeof(float), s));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const OpJ<float> op{h, h->facf};
  auto once = [&]() -> cudaError_t {
    if (kind == 0) {
      cudaError_t e = init_masked<float>(n, h->ess, buf, buf + n, s);
      return e != cudaSuccess ? e : op.apply(buf, buf + n, nullptr, nullptr, s);
    }
    return complex_apply<float>(h, 1.0, buf, buf + n, buf + 2 * n, buf + 3 * n, s);
  };
  const int old_shape = h->shape, old_per = h->per_sm;
  const int reps = 5;
  double best = 1e300, def = 0.0;
  TuneEntry pick{0, 0};
  cudaError_t err = cudaSuccess;
  for (int sh = 0; sh < 2 && err == cudaSuccess; ++sh) {
    for (int per = 0; per <= 4 && err == cudaSuccess; ++per) {
      h->shape = sh;
      h->per_sm = per;
      for (int w = 0; w < 2 && err == cudaSuccess; ++w) err = once();
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps && err == cudaSuccess; ++r) err = once();
      cudaEventRecord(e1, s);
      if (err == cudaSuccess) err = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
      const double us = 1e3 * ms / reps;
      if (sh == 0 && per == 0) def = us;
      if (us < best) {
        best = us;
        pick = TuneEntry{sh, per};
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, s);
  if (err != cudaSuccess) {
    h->shape = old_shape;
    h->per_sm = old_per;
    h->err = cudaGetErrorString(err);
    return HC_ECUDA;
  }
  h->shape = pick.shape;
  h->per_sm = pick.per_sm;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    store_locked(h, pick, best, kind);
  }
  if (shape) *shape = pick.shape;
  if (per_sm) *per_sm = pick.per_sm;
  if (us_best) *us_best = best;
  if (us_default) *us_default = def;
  return HC_OK;
}

}  // extern "C"
