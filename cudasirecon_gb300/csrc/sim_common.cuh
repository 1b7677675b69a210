// Device-side structs and helpers shared by the reconstruction kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft.cuh"

namespace simrecon {

constexpr int kMaxDirs = 8;
constexpr int kMaxOrders = 8;
constexpr int kMaxPhases = 16;
constexpr int kMaxApo = 64;

// Rotationally averaged OTF tables: order o at otf[o], complex [nxotf][nzotf]
// (kr-major, kz fastest, kz in FFT order).
struct OTFView {
  const float2* otf[kMaxOrders];
  int nzotf;
  int nxotf;
  float dkrotf;
  float kzscale;
};

#ifdef __CUDACC__
// hardware square root (about 1 ulp): only for continuous quantities such as
// the OTF interpolation index, never for a decision
__device__ __forceinline__ float sqrt_approx(float x)
{
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Bilinear lookup in a rotationally averaged OTF (the interpolation of
// dev_otfinterpolate, gpuFunctionsImpl.cu:1677-1715).  Indices are clamped
// to the table so a lookup at the very edge of the support never reads past
// it (the reference reads one bin beyond there).
__device__ __forceinline__ float2 otf_lookup(const float2* __restrict__ otf, const OTFView& v, float kx, float ky,
                                             int kz)
{
  float krindex = sqrtf(kx * kx + ky * ky) / v.dkrotf;
  float kzindex = kz * v.kzscale;
  if (kzindex < 0) kzindex += v.nzotf;
  int ir = (int)floorf(krindex);
  int iz = (int)floorf(kzindex);
  float ar = krindex - ir;
  float az = kzindex - iz;
  int izp = (iz == v.nzotf - 1) ? 0 : iz + 1;
  int last = v.nxotf * v.nzotf - 1;
  int i00 = min(max(ir * v.nzotf + iz, 0), last);
  int i01 = min(max(ir * v.nzotf + izp, 0), last);
  int i10 = min(max((ir + 1) * v.nzotf + iz, 0), last);
  int i11 = min(max((ir + 1) * v.nzotf + izp, 0), last);
  float2 a = __ldg(otf + i00), b = __ldg(otf + i01), c = __ldg(otf + i10), d = __ldg(otf + i11);
  float2 r;
  r.x = (1 - ar) * (a.x * (1 - az) + b.x * az) + ar * (c.x * (1 - az) + d.x * az);
  r.y = (1 - ar) * (a.y * (1 - az) + b.y * az) + ar * (c.y * (1 - az) + d.y * az);
  return r;
}

// kz part of otf_lookup, shared by every lookup at one kz
struct OtfKz {
  int iz, izp;
  float az;
};
__device__ __forceinline__ OtfKz otf_kz(const OTFView& v, int kz)
{
  float kzindex = kz * v.kzscale;
  if (kzindex < 0) kzindex += v.nzotf;
  OtfKz r;
  r.iz = (int)floorf(kzindex);
  r.az = kzindex - r.iz;
  r.izp = (r.iz == v.nzotf - 1) ? 0 : r.iz + 1;
  return r;
}
// otf_lookup with the radius |k| already known and the kz part precomputed
// (same arithmetic: krindex = |k| / dkrotf)
__device__ __forceinline__ float2 otf_lookup_rk(const float2* __restrict__ otf, const OTFView& v, float kr,
                                               const OtfKz& z)
{
  float krindex = kr / v.dkrotf;
  int ir = (int)floorf(krindex);
  float ar = krindex - ir;
  int last = v.nxotf * v.nzotf - 1;
  int i00 = min(max(ir * v.nzotf + z.iz, 0), last);
  int i01 = min(max(ir * v.nzotf + z.izp, 0), last);
  int i10 = min(max((ir + 1) * v.nzotf + z.iz, 0), last);
  int i11 = min(max((ir + 1) * v.nzotf + z.izp, 0), last);
  float2 a = __ldg(otf + i00), b = __ldg(otf + i01), c = __ldg(otf + i10), d = __ldg(otf + i11);
  const float az = z.az;
  float2 r;
  r.x = (1 - ar) * (a.x * (1 - az) + b.x * az) + ar * (c.x * (1 - az) + d.x * az);
  r.y = (1 - ar) * (a.y * (1 - az) + b.y * az) + ar * (c.y * (1 - az) + d.y * az);
  return r;
}

// bilinear RA-OTF lookup at radius kr (otf_lookup's arithmetic with
// krindex = kr * (1/dkrotf))
// CLAMP = false only where the caller has shown that every lookup stays in
// the table (krindex + 1 < nxotf).
template <bool CLAMP = true>
__device__ __forceinline__ float2 otf_lookup_rr(const float2* __restrict__ otf, const OTFView& v, float krindex,
                                               const OtfKz& z)
{
  int ir = (int)floorf(krindex);
  float ar = krindex - ir;
  int i00 = ir * v.nzotf + z.iz, i01 = ir * v.nzotf + z.izp;
  int i10 = i00 + v.nzotf, i11 = i01 + v.nzotf;
  if (CLAMP) {
    const int last = v.nxotf * v.nzotf - 1;
    i00 = min(max(i00, 0), last);
    i01 = min(max(i01, 0), last);
    i10 = min(max(i10, 0), last);
    i11 = min(max(i11, 0), last);
  }
  float2 a = __ldg(otf + i00), b = __ldg(otf + i01), c = __ldg(otf + i10), d = __ldg(otf + i11);
  const float az = z.az;
  float2 r;
  r.x = (1 - ar) * (a.x * (1 - az) + b.x * az) + ar * (c.x * (1 - az) + d.x * az);
  r.y = (1 - ar) * (a.y * (1 - az) + b.y * az) + ar * (c.y * (1 - az) + d.y * az);
  return r;
}

__device__ __forceinline__ float cmag2(float2 a) { return a.x * a.x + a.y * a.y; }

// Block-wide sum of a double (all threads must call).  Result valid in thread 0.
__device__ __forceinline__ double block_sum_d(double v, double* scratch /* >= 32 */)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? scratch[threadIdx.x] : 0.0;
  if (wid == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

#endif  // __CUDACC__

}  // namespace simrecon
