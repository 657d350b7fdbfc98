// hc_hex_cplx.cuh -- fused apply of the frequency-domain operator
//
//   y_r = C_nu x_r - omega M_sigma x_i,     y_i = C_nu x_i + omega M_sigma x_r
//
// (masked: essential entries of x read as zero, essential rows of y skipped;
// y must hold (I-P)x beforehand) on planar real/imaginary vectors, in one
// launch: the element factors are staged once for both parts, each element
// evaluates two mass and two curl-curl contractions, and both outputs are
// flushed from shared memory.  Orders 1-2, brick-tiled persistent kernel
// (2 CTAs per SM: twice the staging of the real kernel).  A non-null `done`
// flag that reads 1 skips the launch (a converged COCG batch).
#pragma once
#include "hc_hex_impl.cuh"

namespace hc {

// out = C u_a + s M u_b for one element (fm carries s, fc carries the curl scale)
template <typename T, int P, bool FULL>
__device__ __forceinline__ void elem_cplx(const T* ua0, const T* ua1, const T* ua2, const T* ub0, const T* ub1,
                                          const T* ub2, const T (&fm)[6], const T (&fc)[6], bool has_mass,
                                          T* y0, T* y1, T* y2) {
  constexpr int C = P + 1, O = P;
  constexpr int NDC = O * C * C;
  constexpr int RTC = C * O * O;
  if (!has_mass) {
#pragma unroll
    for (int i = 0; i < NDC; ++i) y0[i] = y1[i] = y2[i] = T(0);
  } else {
    mass_block<T, P, 0, 0, false>(ub0, y0, fm[0]);
    mass_block<T, P, 1, 1, false>(ub1, y1, fm[3]);
    mass_block<T, P, 2, 2, false>(ub2, y2, fm[5]);
    if constexpr (FULL) {
      mass_block<T, P, 0, 1>(ub1, y0, fm[1]);
      mass_block<T, P, 0, 2>(ub2, y0, fm[2]);
      mass_block<T, P, 1, 0>(ub0, y1, fm[1]);
      mass_block<T, P, 1, 2>(ub2, y1, fm[4]);
      mass_block<T, P, 2, 0>(ub0, y2, fm[2]);
      mass_block<T, P, 2, 1>(ub1, y2, fm[4]);
    }
  }
  T r0[RTC], r1[RTC], r2[RTC];
  curl_nd<T, P>(ua0, ua1, ua2, r0, r1, r2);
  T g0[RTC], g1[RTC], g2[RTC];
  rt_block<T, P, 0, 0, false>(r0, g0, fc[0]);
  rt_block<T, P, 1, 1, false>(r1, g1, fc[3]);
  rt_block<T, P, 2, 2, false>(r2, g2, fc[5]);
  if constexpr (FULL) {
    rt_block<T, P, 0, 1>(r1, g0, fc[1]);
    rt_block<T, P, 0, 2>(r2, g0, fc[2]);
    rt_block<T, P, 1, 0>(r0, g1, fc[1]);
    rt_block<T, P, 1, 2>(r2, g1, fc[4]);
    rt_block<T, P, 2, 0>(r0, g2, fc[2]);
    rt_block<T, P, 2, 1>(r1, g2, fc[4]);
  }
  curl_nd_t<T, P>(g0, g1, g2, y0, y1, y2);
}

template <typename T, bool FULL>
__device__ __forceinline__ void load_factors(const T* sf, int stride, int t, T omega, T cscale, T (&fm)[6],
                                             T (&fmn)[6], T (&fc)[6]) {
  if constexpr (FULL) {
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      fm[k] = omega * sf[k * stride + t];
      fmn[k] = -fm[k];
      fc[k] = cscale * sf[(6 + k) * stride + t];
    }
  } else {
    constexpr int kd[3] = {0, 3, 5};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      fm[kd[q]] = omega * sf[q * stride + t];
      fmn[kd[q]] = -fm[kd[q]];
      fc[kd[q]] = cscale * sf[(3 + q) * stride + t];
    }
  }
}

template <typename T, int P, bool FULL, int BX, int BY, int BZ>
__global__ void __launch_bounds__(BX* BY* BZ, 2)
    hex_apply_tiled_cplx(HexDev d, const T* __restrict__ fac, const T* __restrict__ xr, const T* __restrict__ xi,
                         T* __restrict__ yr, T* __restrict__ yi, T omega, T cscale, int masked,
                         const int* __restrict__ done, int nbricks) {
  if (done && *done) return;
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int NT = BX * BY * BZ;
  constexpr int NF = FULL ? 12 : 6;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* base = reinterpret_cast<T*>(smem_raw);
  T* sxr[2] = {base, base + TL::total};
  T* sxi[2] = {base + 2 * TL::total, base + 3 * TL::total};
  T* syr = base + 4 * TL::total;
  T* syi = base + 5 * TL::total;
  T* sfb[2] = {base + 6 * TL::total, base + 6 * TL::total + NF * NT};
  const bool mk = masked != 0;
  const bool mask_needed = mk && (d.ess != nullptr || d.ess_bits != 0);
  const bool has_mass = omega != T(0);
  constexpr int C = P + 1, O = P;
  constexpr int NDC = O * C * C;
  const int lx = threadIdx.x % BX, ly = (threadIdx.x / BX) % BY, lz = threadIdx.x / (BX * BY);
  for (int r = threadIdx.x; r < 2 * TL::total; r += NT) syr[r] = T(0);  // syr and syi
  int b = blockIdx.x;
  auto prefetch_fac = [&](BrickGeom g, T* sf) {
    const int ex = g.X0 + lx, ey = g.Y0 + ly, ez = g.Z0 + lz;
    const bool in = ex < d.nx && ey < d.ny && ez < d.nz;
    const int64_t e = in ? ex + (int64_t)d.nx * (ey + (int64_t)d.ny * ez) : 0;
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      const int k = FULL ? q : (q < 3 ? (q == 0 ? 0 : (q == 1 ? 3 : 5)) : (q == 3 ? 6 : (q == 4 ? 9 : 11)));
      if constexpr (sizeof(T) == 4) cp_async4(sf + q * NT + threadIdx.x, fac + (int64_t)k * d.ne + e, in ? 4 : 0);
      else cp_async8(sf + q * NT + threadIdx.x, fac + (int64_t)k * d.ne + e, in ? 8 : 0);
    }
  };
  auto prefetch = [&](BrickGeom g, int buf) {
    prefetch_comp<T, P, BX, BY, BZ, 0>(d, xr, sxr[buf], g);
    prefetch_comp<T, P, BX, BY, BZ, 1>(d, xr, sxr[buf], g);
    prefetch_comp<T, P, BX, BY, BZ, 2>(d, xr, sxr[buf], g);
    prefetch_comp<T, P, BX, BY, BZ, 0>(d, xi, sxi[buf], g);
    prefetch_comp<T, P, BX, BY, BZ, 1>(d, xi, sxi[buf], g);
    prefetch_comp<T, P, BX, BY, BZ, 2>(d, xi, sxi[buf], g);
    prefetch_fac(g, sfb[buf]);
  };
  if (b < nbricks) prefetch(brick_of<BX, BY, BZ>(d, b), 0);
  cp_async_commit();
  for (int it = 0; b < nbricks; b += gridDim.x, ++it) {
    T* sr = sxr[it & 1];
    T* si = sxi[it & 1];
    const BrickGeom bg = brick_of<BX, BY, BZ>(d, b);
    const int bn = b + gridDim.x;
    if (bn < nbricks) prefetch(brick_of<BX, BY, BZ>(d, bn), (it + 1) & 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const bool full = bg.X0 + BX <= d.nx && bg.Y0 + BY <= d.ny && bg.Z0 + BZ <= d.nz;
    const bool touches = bg.X0 == 0 || bg.Y0 == 0 || bg.Z0 == 0 || bg.X0 + BX >= d.nx || bg.Y0 + BY >= d.ny ||
                         bg.Z0 + BZ >= d.nz;
    const bool fast = full && d.ess == nullptr;
    if (mask_needed && (d.ess != nullptr || touches)) {
      if (d.ess != nullptr) {
        mask_comp<T, P, BX, BY, BZ, 0>(d, sr, bg);
        mask_comp<T, P, BX, BY, BZ, 1>(d, sr, bg);
        mask_comp<T, P, BX, BY, BZ, 2>(d, sr, bg);
        mask_comp<T, P, BX, BY, BZ, 0>(d, si, bg);
        mask_comp<T, P, BX, BY, BZ, 1>(d, si, bg);
        mask_comp<T, P, BX, BY, BZ, 2>(d, si, bg);
      } else {
        zero_ess_planes<T, P, BX, BY, BZ>(d, sr, bg);
        zero_ess_planes<T, P, BX, BY, BZ>(d, si, bg);
      }
      __syncthreads();
    }
    const int ex = bg.X0 + lx, ey = bg.Y0 + ly, ez = bg.Z0 + lz;
    if (ex < d.nx && ey < d.ny && ez < d.nz) {
      T fm[6], fmn[6], fc[6];
      load_factors<T, FULL>(sfb[it & 1], NT, threadIdx.x, omega, cscale, fm, fmn, fc);
      T ur0[NDC], ur1[NDC], ur2[NDC], ui0[NDC], ui1[NDC], ui2[NDC];
      sgather<T, P, BX, BY, BZ, 0>(sr, lx, ly, lz, ur0);
      sgather<T, P, BX, BY, BZ, 1>(sr, lx, ly, lz, ur1);
      sgather<T, P, BX, BY, BZ, 2>(sr, lx, ly, lz, ur2);
      sgather<T, P, BX, BY, BZ, 0>(si, lx, ly, lz, ui0);
      sgather<T, P, BX, BY, BZ, 1>(si, lx, ly, lz, ui1);
      sgather<T, P, BX, BY, BZ, 2>(si, lx, ly, lz, ui2);
      T y0[NDC], y1[NDC], y2[NDC];
      elem_cplx<T, P, FULL>(ur0, ur1, ur2, ui0, ui1, ui2, fmn, fc, has_mass, y0, y1, y2);
      sscatter<T, P, BX, BY, BZ, 0>(syr, lx, ly, lz, y0);
      sscatter<T, P, BX, BY, BZ, 1>(syr, lx, ly, lz, y1);
      sscatter<T, P, BX, BY, BZ, 2>(syr, lx, ly, lz, y2);
      elem_cplx<T, P, FULL>(ui0, ui1, ui2, ur0, ur1, ur2, fm, fc, has_mass, y0, y1, y2);
      sscatter<T, P, BX, BY, BZ, 0>(syi, lx, ly, lz, y0);
      sscatter<T, P, BX, BY, BZ, 1>(syi, lx, ly, lz, y1);
      sscatter<T, P, BX, BY, BZ, 2>(syi, lx, ly, lz, y2);
    }
    __syncthreads();
    if (fast && mk && touches && d.ess_bits) {
      zero_ess_planes<T, P, BX, BY, BZ>(d, syr, bg);
      zero_ess_planes<T, P, BX, BY, BZ>(d, syi, bg);
      __syncthreads();
    }
    flush_comp<T, P, BX, BY, BZ, 0, true>(d, yr, syr, bg, mk, fast);
    flush_comp<T, P, BX, BY, BZ, 1, true>(d, yr, syr, bg, mk, fast);
    flush_comp<T, P, BX, BY, BZ, 2, true>(d, yr, syr, bg, mk, fast);
    flush_comp<T, P, BX, BY, BZ, 0, true>(d, yi, syi, bg, mk, fast);
    flush_comp<T, P, BX, BY, BZ, 1, true>(d, yi, syi, bg, mk, fast);
    flush_comp<T, P, BX, BY, BZ, 2, true>(d, yi, syi, bg, mk, fast);
  }
  cp_async_wait<0>();
}

// y_r/y_i must hold (I-P) x_r / (I-P) x_i (masked) or zero (unmasked) on entry.
template <typename T, int P, int S>
cudaError_t hex_launch_cplx_ps(const HexDev& d, const T* fac, const T* xr, const T* xi, T* yr, T* yi, T omega,
                               T cs, bool masked, const int* done, cudaStream_t s) {
  using B = BrickShapeS<P, S>;
  using TL = BrickTile<P, B::BX, B::BY, B::BZ>;
  constexpr int nt = B::BX * B::BY * B::BZ;
  const size_t sm = (6 * TL::total + 2 * (d.full ? 12 : 6) * nt) * sizeof(T);
  const int nbricks = brick_blocks<P, S>(d);
  static int occ_cache[2][2] = {{0, 0}, {0, 0}};
  const int nsm = device_sms();
  auto go = [&](auto kern, int f) {
    int& occ = occ_cache[f][sizeof(T) == 8];
    if (!occ) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, nt, sm);
      if (occ < 1) occ = 1;
    }
    const int per = d.per_sm > 0 ? std::min(d.per_sm, occ) : occ;
    const int grid = std::min(nbricks, per * nsm);
    kern<<<grid, nt, sm, s>>>(d, fac, xr, xi, yr, yi, omega, cs, masked, done, nbricks);
  };
  if (d.full) go(hex_apply_tiled_cplx<T, P, true, B::BX, B::BY, B::BZ>, 1);
  else go(hex_apply_tiled_cplx<T, P, false, B::BX, B::BY, B::BZ>, 0);
  return cudaGetLastError();
}
#define HC_EXTERN_CPLX_PS(T, P, S)                                                                             \
  extern template cudaError_t hex_launch_cplx_ps<T, P, S>(const HexDev&, const T*, const T*, const T*, T*, T*, \
                                                          T, T, bool, const int*, cudaStream_t);
HC_EXTERN_CPLX_PS(double, 1, 1)
HC_EXTERN_CPLX_PS(double, 2, 1)
HC_EXTERN_CPLX_PS(float, 1, 1)
HC_EXTERN_CPLX_PS(float, 2, 1)
#undef HC_EXTERN_CPLX_PS

template <typename T, int P>
cudaError_t hex_launch_cplx_p(const HexDev& d, const T* fac, const T* xr, const T* xi, T* yr, T* yi, T omega,
                              T cs, bool masked, const int* done, cudaStream_t s) {
  if constexpr (P <= 2) {
    if (d.shape == 1) return hex_launch_cplx_ps<T, P, 1>(d, fac, xr, xi, yr, yi, omega, cs, masked, done, s);
    return hex_launch_cplx_ps<T, P, 0>(d, fac, xr, xi, yr, yi, omega, cs, masked, done, s);
  } else {
    return cudaErrorInvalidValue;  // orders 1-2 only
  }
}

}  // namespace hc
