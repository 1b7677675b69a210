// Wiener filtering and band assembly.
//
// k_filter applies the generalized Wiener filter of filterbands
// (gpuFunctionsImpl.cu:1222-1675) element by element.  The reference runs
// filterbands_kernel1 twice per order over the same half-spectrum arrays:
// the first pass treats stored column jin in [1, nx/2] as the kx = +jin
// pixel, the second treats column 0 (kx = 0) and columns jin in
// [1, nx/2-1] again, now as the conjugate pixel kx = -jin, ky = -y, kz = -z.
// Here one thread owns one stored element and applies both updates in the
// same order, so every element is read and written once.  Planes outside
// +-zdistcutoff are cleared (filterbands_kernel3).
//
// Assembly (assemblerealspacebands, gpuFunctionsImpl.cu:1741-1951) sums,
// over every direction d and order o, w * Re(IFFT3(zoom-pad(band_{d,o})) *
// exp(i phi_{d,o}(x, y))) with w = 1 for order 0 and 2 otherwise.  The ramp
// does not depend on z, so the z transform commutes with the sum:
//     out = Re( IFFTz( S ) ),  S = sum_{d,o} w ramp_{d,o} * IFFTxy(band_{d,o})
// k_asm_y (pruned, zero-padded y IFFT of every in-band kz plane),
// k_asm_x (zero-padded x IFFT, ramp, weighted sum over all (d, o) into S)
// and k_asm_z (one z IFFT of S, real part) write the zoomed output once.
#include <algorithm>
#include <cmath>
#include <vector>

#include "col_fft.cuh"
#include "kernels.h"
#include "reg_fft.cuh"
#include "thresholds.h"

namespace simrecon {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxElems = kFftElems;

__device__ __forceinline__ float dev_suppress(float x)
{
  float x6 = x * x * x;
  x6 *= x6;
  return 1.f / (1 + 20000 / (x6 + 20));  // float division: correctly rounded, like the double one rounded
}

// Per-launch constants derived on the host from FilterArgs (reciprocals and
// products the per-term arithmetic would otherwise recompute per element).
struct FilterK {
  float rnv[kMaxDirs * kMaxOrders];    // 1 / noisevar
  float kxo[kMaxDirs * kMaxOrders];    // order * k0x of each direction
  float kyo[kMaxDirs * kMaxOrders];
  float rdkrotf;                       // 1 / dkrotf
  float min_dkr, rmin_dkr, supp_r;     // suppression radius (1/um) and its unit
  float rrcut;                         // 1 / rdistcutoff
  // exact squared-radius forms of the reference's float-radius decisions
  // (sqrtf is correctly rounded and monotonic): sqrtf(r2) < rdistcutoff
  // <=> r2 < r2_in, sqrtf(r2) <= suppRadius <=> r2 <= r2_supp
  float r2_in, r2_supp;
  float rapo, rzapo;                   // 1 / apocutoff, 1 / zapocutoff
  // every direction's order-0 noise factor is the same (the reference's are
  // all 1): the order-0 Wiener denominator is then one sum for all directions
  int order0_shared;
};


// Wiener scale of pixel (x1f, y1f, z0) of band (dir, order): the body of
// filterbands_kernel1 (gpuFunctionsImpl.cu:1504-1592) without the final
// conjamp factor.  ND/NO: compile-time direction and order counts (0: use
// the runtime values).
// OTF value of order o at radial index krindex in the plane's kz: from the
// plane's radial table (TAB; its entries are the kz interpolation of the
// bilinear lookup, so the result is the same interpolation), else the
// bilinear lookup itself
template <bool CLAMP, bool TAB>
__device__ __forceinline__ float2 filter_otf(const FilterArgs& a, const float2* tabz, int o, float krindex,
                                             const OtfKz& kzi)
{
  if (TAB) {
    const float2* T = tabz + o * a.otf.nxotf;
    const int ir = (int)floorf(krindex);
    const float ar = krindex - ir;
    const float2 t0 = T[ir], t1 = T[ir + 1];
    return make_float2((1 - ar) * t0.x + ar * t1.x, (1 - ar) * t0.y + ar * t1.y);
  }
  return otf_lookup_rr<CLAMP>(a.otf.otf[o], a.otf, krindex, kzi);
}

// FL >= 0: the suppress (bit 0), dampen-order-0 (bit 1) and filter-overlaps
// (bit 2) switches fixed at compile time; FL < 0: read from the arguments.
// termw: |amp|^2 / noisevar of every (direction, order) (FitDev::termw, in
// registers on the compile-time paths); ampmag2: |amp|^2 of this band.
template <int ND, int NO, bool CLAMP, bool TAB, int FL>
__device__ __forceinline__ float2 filter_scale(const FilterArgs& a, const FilterK& k, const float* termw,
                                               float ampmag2, int dir, int order, int z0, float rdist1, float x1f,
                                               float y1f, const float2* tabz)
{
  const bool suppress = FL >= 0 ? (FL & 1) != 0 : a.suppress != 0;
  const bool dampen0 = FL >= 0 ? (FL & 2) != 0 : a.dampen0 != 0;
  const bool filteroverlaps = FL >= 0 ? (FL & 4) != 0 : a.filteroverlaps != 0;
  const int nd = ND ? ND : a.ndirs, no = NO ? NO : a.norders;
  const float xabs = x1f + k.kxo[dir * no + order], yabs = y1f + k.kyo[dir * no + order];
  const OtfKz kzi = otf_kz(a.otf, z0);
  // order-0 damping's axial part |z0 / zdc0|^3, the same for every term
  const float zf = fabsf(z0 / (float)a.zdc[0]);
  const float zf3 = zf * zf * zf;
  float2 otf1 = filter_otf<CLAMP, TAB>(a, tabz, order, rdist1 * k.rdkrotf, kzi);
  float weight = otf1.x * otf1.x + otf1.y * otf1.y;
  if (order != 0) weight *= ampmag2;
  float dampfact = k.rnv[dir * no + order];
  if (suppress && order != 0 && rdist1 <= k.supp_r)
    dampfact *= dev_suppress(rdist1 * k.rmin_dkr);
  else if (!dampen0 && suppress && order == 0 && rdist1 <= k.supp_r)
    dampfact *= dev_suppress(rdist1 * k.rmin_dkr);
  else if (dampen0 && order == 0) {
    const float rf = rdist1 * k.rrcut;
    dampfact *= rf * rf + zf3;
  }
  if (order == 0 && z0 == 0 && a.nokz0) dampfact = 0;
  weight *= dampfact;
  float sumweight = weight;
#pragma unroll
  for (int dir2 = 0; dir2 < nd; dir2++) {
#pragma unroll
    for (int order2 = -(no - 1); order2 < no; order2++) {
      if (dir2 == dir && order2 == order) continue;
      if (!filteroverlaps && !(order2 == 0 && order == 0)) continue;
      const int ao2 = order2 < 0 ? -order2 : order2;
      const float sx = order2 < 0 ? -k.kxo[dir2 * no + ao2] : k.kxo[dir2 * no + ao2];
      const float sy = order2 < 0 ? -k.kyo[dir2 * no + ao2] : k.kyo[dir2 * no + ao2];
      const float x2 = xabs - sx, y2 = yabs - sy;
      const float r2 = x2 * x2 + y2 * y2;
      if (r2 < k.r2_in) {  // rdist2 < rdistcutoff
        const float rdist2 = sqrt_approx(r2);
        const float2 otf2 = filter_otf<CLAMP, TAB>(a, tabz, ao2, rdist2 * k.rdkrotf, kzi);
        float w = (otf2.x * otf2.x + otf2.y * otf2.y) * termw[dir2 * no + ao2];
        if (suppress && order2 != 0 && r2 <= k.r2_supp)
          w *= dev_suppress(rdist2 * k.rmin_dkr);
        else if (!dampen0 && suppress && order2 == 0 && r2 <= k.r2_supp)
          w *= dev_suppress(rdist2 * k.rmin_dkr);
        else if (dampen0 && order2 == 0) {
          const float rf = rdist2 * k.rrcut;
          w *= rf * rf + zf3;
        }
        if (a.nokz0 && order2 == 0 && z0 == 0) w = 0.0f;
        sumweight += w;
      }
    }
  }
  sumweight += a.wiener2;
  const float f = dampfact / sumweight;
  float2 scale = make_float2(otf1.x * f, -otf1.y * f);
  if (a.apodizeoutput) {
    float rdistabs = sqrtf(xabs * xabs + yabs * yabs);
    float rho;
    float zdistabs = abs(z0);
    const float ra = rdistabs * k.rapo;
    if (a.zapocutoff > 0 && a.bessel) {  // gpuFunctionsImpl.cu:1572-1577
      const float rhox = xabs * k.rrcut, rhoy = yabs * k.rapo, rhoz = zdistabs * k.rzapo;
      rho = sqrtf(rhox * rhox + rhoy * rhoy + rhoz * rhoz);
    } else if (a.zapocutoff > 0) {
      const float rz = zdistabs * k.rzapo;
      rho = sqrtf(ra * ra + rz * rz);
    } else {
      rho = ra;
    }
    if (rho > 1.f) rho = 1.0f;
    float apofact = 1.f;
    if (a.apodizeoutput == 1) apofact = cosf(1.57079632679f * rho);
    else if (a.apodizeoutput == 2) apofact = 1.0f - rho;
    scale.x *= apofact;
    scale.y *= apofact;
  }
  return scale;
}

// split re/im into plus/minus, scale plus, recombine (gpuFunctionsImpl.cu:1617-1644)
__device__ __forceinline__ void apply_side(float2& re, float2& im, float2 scale, bool conj)
{
  if (conj) {
    re.y = -re.y;
    im.y = -im.y;
  }
  float2 plus = make_float2(re.x - im.y, re.y + im.x);
  float2 minus = make_float2(re.x + im.y, re.y - im.x);
  plus = cmul(plus, scale);
  re = make_float2(0.5f * (plus.x + minus.x), 0.5f * (plus.y + minus.y));
  im = make_float2(0.5f * (plus.y - minus.y), 0.5f * (-plus.x + minus.x));
  if (conj) {
    re.y = -re.y;
    im.y = -im.y;
  }
}

// TAB: the block (one kz plane) first builds, in shared memory, each order's
// OTF interpolated to this plane's kz (+z0) and to the conjugate pass's kz
// (-z0) along kr: [2][NO][nxotf]; only where no lookup can leave the table
template <int ND, int NO, bool CLAMP, bool TAB, int FL = -1>
__global__ void __launch_bounds__(kThreads) k_filter(const __grid_constant__ FilterArgs a, const __grid_constant__ FilterK k)
{
  extern __shared__ float2 tab[];
  const int nx = a.nx, ny = a.ny, nz = a.nz, nxh = nx / 2 + 1;
  const int order = blockIdx.z, iz = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int zdc = a.zdc[order];
  const bool inband = (iz <= zdc) || (iz >= nz - zdc);
  if (TAB) {
    static_assert(!TAB || NO > 0, "the table needs the order count at compile time");
    const int nxo = a.otf.nxotf, nzo = a.otf.nzotf;
    if (inband) {
      const int zp = iz <= zdc ? iz : iz - nz;
      for (int t = threadIdx.x; t < 2 * NO * nxo; t += blockDim.x) {
        const int pass = t / (NO * nxo), r = t - pass * NO * nxo, o = r / nxo, ir = r - o * nxo;
        const OtfKz kz = otf_kz(a.otf, pass ? -zp : zp);
        const float2 va = __ldg(a.otf.otf[o] + ir * nzo + kz.iz), vb = __ldg(a.otf.otf[o] + ir * nzo + kz.izp);
        const float az = kz.az;
        tab[t] = make_float2(va.x * (1 - az) + vb.x * az, va.y * (1 - az) + vb.y * az);
      }
    }
    __syncthreads();
  }
  if (e >= ny * nxh) return;
  const int iin = e / nxh, jin = e - iin * nxh;
  const size_t plane = (size_t)ny * nxh;
  float2* b1 = a.bands + (size_t)(order == 0 ? 0 : 2 * order - 1) * nz * plane;
  float2* b2 = order == 0 ? nullptr : a.bands + (size_t)(2 * order) * nz * plane;
  const size_t ind = (size_t)iz * plane + e;
  if (!inband) {  // filterbands_kernel3
    b1[ind] = make_float2(0.f, 0.f);
    if (b2) b2[ind] = make_float2(0.f, 0.f);
    return;
  }
  const int z0 = iz <= zdc ? iz : iz - nz;
  // the pixel this element is the non-conjugate copy of
  const int y1 = (iin < ny - ny / 2) ? iin : iin - ny;
  const int x1 = jin;
  float x1f = x1 * a.dkx, y1f = y1 * a.dky;
  float rdist1 = sqrtf(x1f * x1f + y1f * y1f);
  if (!(rdist1 <= a.rdistcutoff)) {
    b1[ind] = make_float2(0.f, 0.f);
    if (b2) b2[ind] = make_float2(0.f, 0.f);
    return;
  }
  const float ampmag2 = __ldg(a.fit->ampmag2 + a.dir * a.norders + order);
  const float2 amp = __ldg(a.fit->amp + a.dir * a.norders + order);
  const float2 conjamp = make_float2(amp.x, -amp.y);
  auto body = [&](const float* termw) {
    float2 s1 = filter_scale<ND, NO, CLAMP, TAB, FL>(a, k, termw, ampmag2, a.dir, order, z0, rdist1, x1f, y1f, tab);
    if (order == 0) {
      b1[ind] = cmul(b1[ind], s1);
      return;
    }
    float2 re = b1[ind], im = b2[ind];
    apply_side(re, im, cmul(s1, conjamp), false);
    if (jin >= 1 && jin <= nx / 2 - 1) {
      // second pass: the conjugate pixel (-jin, -y, -z0)
      const int y2 = (iin <= ny / 2) ? -iin : ny - iin;
      const int x2 = -jin;
      float x2f = x2 * a.dkx, y2f = y2 * a.dky;
      float rdist2 = sqrtf(x2f * x2f + y2f * y2f);
      float2 s2 = filter_scale<ND, NO, CLAMP, TAB, FL>(a, k, termw, ampmag2, a.dir, order, -z0, rdist2, x2f, y2f,
                                                       tab + (TAB ? NO * a.otf.nxotf : 0));
      apply_side(re, im, cmul(s2, conjamp), true);
    }
    b1[ind] = re;
    b2[ind] = im;
  };
  // the fitted amplitudes' weights: in registers on the compile-time paths
  if constexpr (ND > 0 && NO > 0) {
    float twr[ND * NO];
#pragma unroll
    for (int i = 0; i < ND * NO; ++i) twr[i] = __ldg(a.fit->termw + i);
    body(twr);
  } else {
    body(a.fit->termw);
  }
}

// One transformed plane: band (dir, order) at signed kz, summed into output
// plane zout.  dir < 0 marks the order-0 slot of a plane: the order-0 bands
// of all directions summed before the transforms (their phase ramps are all
// 1, so the sum commutes with the inverse FFTs).
struct Slot {
  int dir, order, kz, zout;
};

// zero-padded inverse FFT along y of the in-band plane kz of band (d, o);
// columns c = kx + nx/2 - 1, kx in [-nx/2+1, nx/2] (move_kernel ranges,
// gpuFunctionsImpl.cu:1853-1913)
template <int NF>
__global__ void __launch_bounds__(kThreads) k_asm_y(AssembleArgs a, const Slot* __restrict__ slots, FFTPlan plan, int W)
{
  extern __shared__ float2 sm[];
  const Slot sl = slots[blockIdx.y];
  const int nx = a.nx, ny = a.ny, nz = a.nz, nxh = nx / 2 + 1, Y = a.Y;
  const int c0 = blockIdx.x * W;
  const size_t plane = (size_t)ny * nxh;
  const int d0 = sl.dir < 0 ? 0 : sl.dir;
  const float2* br = a.bands + ((size_t)d0 * a.nphases + (sl.order == 0 ? 0 : 2 * sl.order - 1)) * nz * plane;
  const float2* bi = sl.order == 0 ? nullptr : a.bands + ((size_t)d0 * a.nphases + 2 * sl.order) * nz * plane;
  const size_t dstride = (size_t)a.nphases * nz * plane;  // next direction's band 0
  const int ylo = ny / 2 - 1;  // ky in [-ylo, ny/2]
  const int ld = W + 1;
  for (int t = threadIdx.x; t < Y * W; t += blockDim.x) {
    int yr = t / W, w = t - yr * W;
    int c = c0 + w;
    float2 v = make_float2(0.f, 0.f);
    int ky;
    bool valid = c < nx;
    if (yr <= ny / 2) ky = yr;
    else if (yr >= Y - ylo) ky = yr - Y;
    else valid = false;
    if (valid) {
      int x = c - (nx / 2 - 1), y = ky, z = sl.kz;
      bool conj = x < 0;
      if (conj) {
        x = -x;
        y = -y;
        z = -z;
      }
      if (y < 0) y += ny;
      if (z < 0) z += nz;
      size_t indin = (size_t)z * plane + (size_t)y * nxh + x;
      if (sl.order == 0) {
        v = br[indin];
        if (sl.dir < 0)
          for (int d = 1; d < a.ndirs; ++d) {
            float2 u = br[d * dstride + indin];
            v.x += u.x;
            v.y += u.y;
          }
        if (conj) v.y = -v.y;
      } else {
        float2 re = br[indin], im = bi[indin];
        if (conj) {
          re.y = -re.y;
          im.y = -im.y;
        }
        v = make_float2(re.x - im.y, re.y + im.x);
      }
    }
    sm[yr * ld + w] = v;
  }
  __syncthreads();
  const float2* res = fft_dispatch<NF, +1>(sm, sm + Y * ld, plan, W, 1, ld);
  float2* dst = a.T + (size_t)blockIdx.y * Y * nx;
  for (int t = threadIdx.x; t < Y * W; t += blockDim.x) {
    int yr = t / W, w = t - yr * W;
    if (c0 + w < nx) dst[(size_t)yr * nx + c0 + w] = res[yr * ld + w];
  }
}

// zero-padded inverse FFT along x of every slot of output plane zout, ramp,
// weighted sum -> S[zout][yr][:]
constexpr int kAccPerThread = 16;
template <int NF>
__global__ void __launch_bounds__(kThreads) k_asm_x(AssembleArgs a, const int* __restrict__ plane_slot0,
                                               const int* __restrict__ plane_nslot, const Slot* __restrict__ slots,
                                               const int* __restrict__ plane_zout, FFTPlan plan, int lines)
{
  extern __shared__ float2 sm[];
  const int nx = a.nx, X = a.X, Y = a.Y;
  const int pidx = blockIdx.y, yr = blockIdx.x;
  const int s0 = plane_slot0[pidx], ns = plane_nslot[pidx], zout = plane_zout[pidx];
  float2 acc[kAccPerThread];
#pragma unroll
  for (int k = 0; k < kAccPerThread; ++k) acc[k] = make_float2(0.f, 0.f);
  const int xlo = nx / 2 - 1;
  const int ldl = X + 1;
  for (int b0 = 0; b0 < ns; b0 += lines) {
    int nb = min(lines, ns - b0);
    __syncthreads();
    for (int t = threadIdx.x; t < lines * X; t += blockDim.x) {
      int l = t / X, xo = t - l * X;
      float2 v = make_float2(0.f, 0.f);
      if (l < nb) {
        int kx = xo <= nx / 2 ? xo : (xo >= X - xlo ? xo - X : 1 << 30);
        if (kx != (1 << 30)) {
          int c = kx + xlo;
          v = a.T[((size_t)(s0 + b0 + l) * Y + yr) * nx + c];
        }
      }
      sm[l * ldl + xo] = v;
    }
    __syncthreads();
    const float2* res = fft_dispatch<NF, +1>(sm, sm + lines * ldl, plan, lines, ldl, 1);
    for (int l = 0; l < nb; ++l) {
      const Slot sl = slots[s0 + b0 + l];
      if (sl.dir < 0) {  // summed order-0 slot: ramp 1, weight 1
#pragma unroll
        for (int k = 0; k < kAccPerThread; ++k) {
          int x = threadIdx.x + k * blockDim.x;
          if (x < X) {
            acc[k].x += res[l * ldl + x].x;
            acc[k].y += res[l * ldl + x].y;
          }
        }
        continue;
      }
      const int ro = sl.dir * a.norders + sl.order;
      const float w = sl.order == 0 ? 1.f : 2.f;
      float2 ey = a.ey[(size_t)ro * Y + yr];
      ey.x *= w;
      ey.y *= w;
#pragma unroll
      for (int k = 0; k < kAccPerThread; ++k) {
        int x = threadIdx.x + k * blockDim.x;
        if (x < X) {
          float2 e = cmul(a.ex[(size_t)ro * X + x], ey);
          float2 v = cmul(res[l * ldl + x], e);
          acc[k].x += v.x;
          acc[k].y += v.y;
        }
      }
    }
  }
  float2* dst = a.S + ((size_t)zout * Y + yr) * X;
#pragma unroll
  for (int k = 0; k < kAccPerThread; ++k) {
    int x = threadIdx.x + k * blockDim.x;
    if (x < X) dst[x] = acc[k];
  }
}

// Four-step variant of k_asm_y (col_fft.cuh) for zoomed column lengths with
// a column configuration: 8 output columns of one slot per CTA, band values
// loaded straight from HBM during the first stage.
// At most 128 registers (two CTAs per SM): left to its own heuristic the
// compiler has given this kernel 191 registers (one CTA per SM, 1.78 instead
// of 1.00 ms per 512^2 x 48 volume) after an unrelated change to its arguments.
template <int Y>
__global__ void __launch_bounds__(kThreads, 2) k_asm_y4(AssembleArgs a, const Slot* __restrict__ slots,
                                                    const float2* __restrict__ tw)
{
  constexpr int R1 = colfft_r1(Y), W = 8;
  extern __shared__ float2 sm[];  // ColFft<Y, R1, W>::kSmemElems
  const Slot sl = slots[blockIdx.y];
  const int nx = a.nx, ny = a.ny, nz = a.nz, nxh = nx / 2 + 1;
  const int c0 = blockIdx.x * W;
  const size_t plane = (size_t)ny * nxh;
  const int d0 = sl.dir < 0 ? 0 : sl.dir;
  const float2* br = a.bands + ((size_t)d0 * a.nphases + (sl.order == 0 ? 0 : 2 * sl.order - 1)) * nz * plane;
  const float2* bi = sl.order == 0 ? nullptr : a.bands + ((size_t)d0 * a.nphases + 2 * sl.order) * nz * plane;
  const size_t dstride = (size_t)a.nphases * nz * plane;
  const int ylo = ny / 2 - 1;  // ky in [-ylo, ny/2]
  colfft_stage1<Y, R1, W, +1>(sm, tw, [&](int yr, int w) {
    const int c = c0 + w;
    float2 v = make_float2(0.f, 0.f);
    int ky;
    bool valid = c < nx;
    if (yr <= ny / 2) ky = yr;
    else if (yr >= Y - ylo) ky = yr - Y;
    else valid = false;
    if (valid) {
      int x = c - (nx / 2 - 1), y = ky, z = sl.kz;
      const bool conj = x < 0;
      if (conj) {
        x = -x;
        y = -y;
        z = -z;
      }
      if (y < 0) y += ny;
      if (z < 0) z += nz;
      const size_t indin = (size_t)z * plane + (size_t)y * nxh + x;
      if (sl.order == 0) {
        v = br[indin];
        if (sl.dir < 0)
          for (int d = 1; d < a.ndirs; ++d) {
            float2 u = br[d * dstride + indin];
            v.x += u.x;
            v.y += u.y;
          }
        if (conj) v.y = -v.y;
      } else {
        float2 re = br[indin], im = bi[indin];
        if (conj) {
          re.y = -re.y;
          im.y = -im.y;
        }
        v = make_float2(re.x - im.y, re.y + im.x);
      }
    }
    return v;
  });
  float2* dst = a.T + (size_t)blockIdx.y * Y * nx + c0;
  colfft_stage2<Y, R1, W, +1>(sm, [&](int yr, int w, float2 v) {
    if (c0 + w < nx) dst[(size_t)yr * nx + w] = v;
  });
}

// k_asm_y4 with the Wiener filter fused into its band load (filterbands,
// gpuFunctionsImpl.cu:1222-1675, feeding move_kernel, 1853-1913): the bands
// are read unfiltered, once, and no filter pass writes them back.
//
// The reference's first filter pass scales only the plus part (re + i im) of
// a stored element and its second pass only the minus part (re - i im, the
// conjugate pixel), so the assembled value needs one scale per read: at the
// pixel (kx, ky', kz) for the plus part (kx >= 0) and for the conjugate part
// (kx < 0) alike, where ky' = ky except ky' = -ny/2 for the stored row ny/2
// (both filter passes index rows as y in [-ny/2, ny/2-1]).  Order 0 is
// filtered at its stored element's own pixel and conjugated for kx < 0, summed
// over the directions; with equal order-0 noise factors the directions share
// one Wiener denominator (each direction's own term equals the order-0 term of
// the other directions' sums), so it is evaluated once.  Pixels outside the lateral support are zero and not
// read; planes outside each order's zdistcutoff are never assembled.
//
// Phase A: the filtered band values of the CTA's 8 columns on the ny data
// rows, row-major in shared memory (a runtime loop: one copy of the filter
// code).  Stage 1 then reads its strided rows from there (the zero-padding
// rows read as zero; one barrier between the reads and the stage-1 stores into
// the same buffer), stage 2 as k_asm_y4.  The per-kz OTF radial tables of the
// filter (for kz and, for order 0, -kz) follow the transform buffer.
// Three CTAs per SM (at most 80 registers): the filter phase needs the warps
// more than the transform stages need registers (1.61 -> 1.31 ms per
// 512^2 x 48 volume against two CTAs per SM).
template <int Y, int NO, int FL>
__global__ void __launch_bounds__(kThreads, 3) k_asm_y4f(AssembleArgs a, const Slot* __restrict__ slots,
                                                     const float2* __restrict__ tw,
                                                     const __grid_constant__ FilterArgs fa,
                                                     const __grid_constant__ FilterK fk)
{
  constexpr int ND = 3;
  constexpr int R1 = colfft_r1(Y), W = 8;
  using CF = ColFft<Y, R1, W>;
  constexpr int R2 = CF::R2;
  static_assert(R2 * W <= kThreads, "one stage-1 item per thread");
  static_assert(Y * W <= CF::kSmemElems, "phase A fits the transform buffer");
  extern __shared__ float2 sm[];
  float2* tab = sm + CF::kSmemElems;  // [2][NO][nxotf]
  const Slot sl = slots[blockIdx.y];
  const int nx = a.nx, ny = a.ny, nz = a.nz, nxh = nx / 2 + 1;
  const int c0 = blockIdx.x * W;
  const size_t plane = (size_t)ny * nxh;
  const int order = sl.order;
  const int d0 = sl.dir < 0 ? 0 : sl.dir;
  const float2* br = a.bands + ((size_t)d0 * a.nphases + (order == 0 ? 0 : 2 * order - 1)) * nz * plane;
  const float2* bi = order == 0 ? nullptr : a.bands + ((size_t)d0 * a.nphases + 2 * order) * nz * plane;
  const size_t dstride = (size_t)a.nphases * nz * plane;  // next direction's band 0
  const int ylo = ny / 2 - 1;                              // ky in [-ylo, ny/2]
  {  // OTF of every order interpolated to kz (pass 0) and -kz (pass 1) along kr
    const int nxo = fa.otf.nxotf, nzo = fa.otf.nzotf;
    for (int t = threadIdx.x; t < 2 * NO * nxo; t += blockDim.x) {
      const int pass = t / (NO * nxo), r = t - pass * NO * nxo, o = r / nxo, ir = r - o * nxo;
      const OtfKz kz = otf_kz(fa.otf, pass ? -sl.kz : sl.kz);
      const float2 va = __ldg(fa.otf.otf[o] + ir * nzo + kz.iz), vb = __ldg(fa.otf.otf[o] + ir * nzo + kz.izp);
      tab[t] = make_float2(va.x * (1 - kz.az) + vb.x * kz.az, va.y * (1 - kz.az) + vb.y * kz.az);
    }
  }
  float termw[ND * NO];
#pragma unroll
  for (int i = 0; i < ND * NO; ++i) termw[i] = __ldg(fa.fit->termw + i);
  float ampmag2 = 0.f;
  float2 conjamp = make_float2(1.f, 0.f);
  if (order != 0) {
    ampmag2 = __ldg(fa.fit->ampmag2 + d0 * NO + order);
    const float2 am = __ldg(fa.fit->amp + d0 * NO + order);
    conjamp = make_float2(am.x, -am.y);
  }
  __syncthreads();
  // phase A over the ny data rows (ky in [-ylo, ny/2]); not unrolled (two
  // copies of the filter code in flight measured 46 % slower)
  for (int t = threadIdx.x; t < ny * W; t += blockDim.x) {
    const int r = t / W, w = t - r * W;
    const int yr = r <= ny / 2 ? r : r + (Y - ny);
    const int ky = r <= ny / 2 ? r : r - ny;
    const int c = c0 + w;
    float2 v = make_float2(0.f, 0.f);
    if (c < nx) {
      const int kx = c - (nx / 2 - 1);
      const int kyf = ky == ny / 2 ? -(ny / 2) : ky;
      const float x1f = kx * fa.dkx, y1f = kyf * fa.dky;
      const float rdist1 = sqrtf(x1f * x1f + y1f * y1f);
      if (rdist1 <= fa.rdistcutoff) {
        int x = kx, y = ky, z = sl.kz;
        const bool conj = x < 0;
        if (conj) {
          x = -x;
          y = -y;
          z = -z;
        }
        if (y < 0) y += ny;
        if (z < 0) z += nz;
        const size_t indin = (size_t)z * plane + (size_t)y * nxh + x;
        if (order == 0) {
          // each direction's order-0 band at the stored element's own pixel
          const float xs = conj ? -x1f : x1f;
          const float ys = conj ? (float)(-ky) * fa.dky : y1f;
          const int zs = conj ? -sl.kz : sl.kz;
          const float2* tz = tab + (conj ? NO * fa.otf.nxotf : 0);
          if (fk.order0_shared) {
            // one denominator for every direction: direction d's own term and
            // the (d, 0) term its sum skips are the same OTF value
            const float2 sc = filter_scale<ND, NO, false, true, FL>(fa, fk, termw, 0.f, 0, 0, zs, rdist1, xs, ys, tz);
            float2 b = br[indin];
#pragma unroll
            for (int d = 1; d < ND; ++d) {
              const float2 u = br[d * dstride + indin];
              b.x += u.x;
              b.y += u.y;
            }
            v = cmul(b, sc);
          } else {
#pragma unroll 1
            for (int d = 0; d < ND; ++d) {
              const float2 sc =
                  filter_scale<ND, NO, false, true, FL>(fa, fk, termw, 0.f, d, 0, zs, rdist1, xs, ys, tz);
              const float2 b = br[d * dstride + indin];
              v.x += b.x * sc.x - b.y * sc.y;
              v.y += b.x * sc.y + b.y * sc.x;
            }
          }
          if (conj) v.y = -v.y;
        } else {
          const float2 sc = filter_scale<ND, NO, false, true, FL>(fa, fk, termw, ampmag2, d0, order, sl.kz, rdist1,
                                                                   x1f, y1f, tab);
          float2 re = br[indin], im = bi[indin];
          if (conj) {
            re.y = -re.y;
            im.y = -im.y;
          }
          v = cmul(make_float2(re.x - im.y, re.y + im.x), cmul(sc, conjamp));
        }
      }
    }
    sm[yr * W + w] = v;
  }
  __syncthreads();
  // stage 1 from the row-major values (zero-padding rows read as zero)
  const int it = threadIdx.x;
  const bool has1 = it < R2 * W;
  const int cc = it % W, j = it / W;
  float2 v[R1];
#pragma unroll
  for (int e = 0; e < R1; ++e) {
    const int yr = j + R2 * e;
    const bool data = yr <= ny / 2 || yr >= Y - ylo;
    v[e] = has1 && data ? sm[yr * W + cc] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  if (has1) {
    reg_dft<R1, +1>(v);
#pragma unroll
    for (int k1 = 1; k1 < R1; ++k1) {
      float2 w = __ldg(tw + j * k1);
      w.y = -w.y;
      v[k1] = cmul(v[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) sm[k1 * CF::LD1 + j * W + cc] = v[k1];
  }
  __syncthreads();
  float2* dst = a.T + (size_t)blockIdx.y * Y * nx + c0;
  colfft_stage2<Y, R1, W, +1>(sm, [&](int yr, int w, float2 val) {
    if (c0 + w < nx) dst[(size_t)yr * nx + w] = val;
  });
}

// Warp-level variant of k_asm_x for the zoomed row lengths with a register
// path: each group of P lanes owns one output row yr of plane pidx and runs,
// for every slot of the plane, the zero-padded inverse FFT of the slot's T row
// in registers (one warp-private exchange, no CTA barrier), the phase ramp
// and the weighted sum; the row of S is written once.
template <int X>
struct XwLanes {
  static constexpr int P = X == 1024 ? 32 : (X == 512 || X == 256 ? 16 : 0);
};
constexpr int kXwWarps = 4;

template <int X>
constexpr size_t xw_smem_bytes()
{
  constexpr int P = XwLanes<X>::P, E = X / P, G = 32 / P;
  return ((size_t)kXwWarps * G * ((P + 1) * E + 1) + (size_t)kXwWarps * G * 2 * (X / 2)) * sizeof(float2);
}

// Two CTAs per SM: the 1024-point rows keep their 32 transform values and 32
// accumulators per lane without spilling (per 512^2 x 48 volume: 0.57 ms,
// against 0.66 ms at three CTAs per SM with spills)
template <int X>
__global__ void __launch_bounds__(kXwWarps * 32, 2) k_asm_xw(AssembleArgs a, const int* __restrict__ plane_slot0,
                                                          const int* __restrict__ plane_nslot,
                                                          const Slot* __restrict__ slots,
                                                          const int* __restrict__ plane_zout,
                                                          const float2* __restrict__ twr)
{
  constexpr int P = XwLanes<X>::P, E = X / P, G = 32 / P;
  constexpr int XB = (P + 1) * E + 1;
  constexpr int NXB = X / 2;  // band columns (T row length)
  // dynamic shared memory (xw_smem_bytes): the exchange buffers, then a
  // two-entry ring per group into which the T row of the next slot is
  // copied with cp.async while the current one is transformed
  extern __shared__ __align__(16) float2 xw_dyn[];
  float2* xs = xw_dyn;
  float2(*ring)[2][NXB] = reinterpret_cast<float2(*)[2][NXB]>(xw_dyn + kXwWarps * G * XB);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / P, p = lane - g * P;
  const int yr = (blockIdx.x * kXwWarps + warp) * G + g;
  const bool act = yr < a.Y;
  // output planes in the reverse of the order the y pass wrote their slots:
  // the last slots written are still in L2 when the first CTAs read them
  const int pidx = gridDim.y - 1 - blockIdx.y;
  const int s0 = plane_slot0[pidx], ns = plane_nslot[pidx], zout = plane_zout[pidx];
  const int nx = a.nx, Y = a.Y, xlo = nx / 2 - 1;
  float2* xb = xs + (warp * G + g) * XB;
  float2(*rg)[NXB] = ring[warp * G + g];
  // each lane copies 16-byte chunks (2 complex) of the nx-long row
  auto prefetch = [&](int si) {
    if (act && si < ns) {
      const float2* trow = a.T + ((size_t)(s0 + si) * Y + yr) * nx;
      for (int q = p; q < nx / 2; q += P) {
        const unsigned dst = (unsigned)__cvta_generic_to_shared(&rg[si & 1][2 * q]);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(trow + 2 * q) : "memory");
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  float2 acc[E];
#pragma unroll
  for (int i = 0; i < E; ++i) acc[i] = make_float2(0.f, 0.f);
  prefetch(0);
  for (int si = 0; si < ns; ++si) {  // same trip count for every lane of the warp
    const Slot sl = slots[s0 + si];
    prefetch(si + 1);
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this lane's copies of slot si landed
    __syncwarp();                                             // ... and every other lane's
    const float2* trow = rg[si & 1];
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int x = p + P * e;
      const bool in = act && (x <= nx / 2 || x >= X - xlo);
      v[e] = in ? trow[(x <= nx / 2 ? x : x - X) + xlo] : make_float2(0.f, 0.f);
    }
    __syncwarp();  // the ring entry is read before the next prefetch overwrites it
    reg_line<X, P, +1>(v, p, xb, twr, true);
    if (sl.dir < 0) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        acc[i].x += v[i].x;
        acc[i].y += v[i].y;
      }
    } else {
      const int ro = sl.dir * a.norders + sl.order;
      const float w = sl.order == 0 ? 1.f : 2.f;
      float2 ey = act ? __ldg(a.ey + (size_t)ro * Y + yr) : make_float2(0.f, 0.f);
      ey.x *= w;
      ey.y *= w;
      const float2* exr = a.ex + (size_t)ro * X;
#pragma unroll
      for (int m = 0; m < E / P; ++m)
#pragma unroll
        for (int k2 = 0; k2 < P; ++k2) {
          const int i = m * P + k2;
          const float2 e = cmul(__ldg(exr + p + P * m + E * k2), ey);
          const float2 t = cmul(v[i], e);
          acc[i].x += t.x;
          acc[i].y += t.y;
        }
    }
  }
  if (act) {
    float2* dst = a.S + ((size_t)zout * Y + yr) * X;
#pragma unroll
    for (int m = 0; m < E / P; ++m)
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) dst[p + P * m + E * k2] = acc[m * P + k2];
  }
}

// inverse FFT along z of S, real part -> out
template <int NF>
__global__ void __launch_bounds__(kThreads) k_asm_z(AssembleArgs a, const unsigned char* __restrict__ zactive,
                                                    FFTPlan plan, int W)
{
  extern __shared__ float2 sm[];
  const int X = a.X, Y = a.Y, Z = a.Z;
  const int yr = blockIdx.y, c0 = blockIdx.x * W;
  const int ld = W + 1;
  for (int t = threadIdx.x; t < Z * W; t += blockDim.x) {
    int z = t / W, w = t - z * W;
    sm[z * ld + w] = (zactive[z] && c0 + w < X) ? a.S[((size_t)z * Y + yr) * X + c0 + w] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2* res = fft_dispatch<NF, +1>(sm, sm + Z * ld, plan, W, 1, ld);
  for (int t = threadIdx.x; t < Z * W; t += blockDim.x) {
    int z = t / W, w = t - z * W;
    if (c0 + w < X) a.out[((size_t)z * Y + yr) * X + c0 + w] = res[z * ld + w].x;
  }
}

// Z = 1 (2D): the z transform is the identity, out = Re(S) (two elements per
// thread; X = 2 nx is even)
__global__ void __launch_bounds__(kThreads) k_asm_z1(const float4* __restrict__ S, float2* out, size_t npairs,
                                                     const unsigned char* __restrict__ zactive)
{
  const bool on = zactive[0] != 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npairs; i += (size_t)gridDim.x * blockDim.x) {
    const float4 v = on ? S[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    out[i] = make_float2(v.x, v.z);
  }
}

// Four-step variant of k_asm_z for Z = 16 * R1: 64 columns of one output row
// per CTA.  Stage 1: the thread for (column c, j < 16) loads the R1 planes
// z = j + 16 e of S (only the in-band ones; the rest are zero) and runs the
// inverse R1-point DFT times conj(W_Z^(j k1)); stage 2: the thread for
// (c, k1) runs the inverse 16-point DFT and stores the real part of planes
// k1 + R1 k2.
template <int R1>
__global__ void __launch_bounds__(kThreads) k_asm_z4(AssembleArgs a, const unsigned char* __restrict__ zactive,
                                                    const float2* __restrict__ tw)
{
  constexpr int R2 = 16, W = 64;
  constexpr int LD = R2 * W + 8;
  extern __shared__ float2 sm[];  // [R1][LD]
  const int X = a.X, Y = a.Y;
  const int yr = blockIdx.y, c0 = blockIdx.x * W;
  const int nc = min(W, X - c0);
  const size_t zstride = (size_t)Y * X;
  const float2* src = a.S + (size_t)yr * X + c0;
  for (int it = threadIdx.x; it < R2 * W; it += blockDim.x) {
    const int c = it % W, j = it / W;
    float2 v[R1];
#pragma unroll
    for (int e = 0; e < R1; ++e) {
      const int z = j + R2 * e;
      v[e] = (c < nc && zactive[z]) ? src[z * zstride + c] : make_float2(0.f, 0.f);
    }
    reg_dft<R1, +1>(v);
#pragma unroll
    for (int k1 = 1; k1 < R1; ++k1) {
      float2 w = __ldg(tw + j * k1);
      w.y = -w.y;
      v[k1] = cmul(v[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) sm[k1 * LD + j * W + c] = v[k1];
  }
  __syncthreads();
  float* dst = a.out + (size_t)yr * X + c0;
  for (int it = threadIdx.x; it < R1 * W; it += blockDim.x) {
    const int c = it % W, k1 = it / W;
    float2 u[R2];
#pragma unroll
    for (int jj = 0; jj < R2; ++jj) u[jj] = sm[k1 * LD + jj * W + c];
    reg_dft<R2, +1>(u);
    if (c < nc)
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) dst[(size_t)(k1 + R1 * k2) * zstride + c] = u[k2].x;
  }
}

__global__ void k_ramp(const __grid_constant__ K0List k0, int ndirs, int norders, int X, int Y, float dxyz, float fact,
                       float2* ex, float2* ey)
{
  int n = ndirs * norders * (X + Y);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int ro = t / (X + Y), r = t - ro * (X + Y);
    int d = ro / norders, o = ro - d * norders;
    float kx = k0.k[d].x * (float)o, ky = k0.k[d].y * (float)o;
    double ang;
    if (r < X) ang = (double)fact * M_PI * (double)(r - X / 2) * (double)kx * (double)dxyz;
    else ang = (double)fact * M_PI * (double)((r - X) - Y / 2) * (double)ky * (double)dxyz;
    double s, c;
    sincos(ang, &s, &c);
    float2 v = make_float2((float)c, (float)s);
    if (r < X) ex[(size_t)ro * X + r] = v;
    else ey[(size_t)ro * Y + (r - X)] = v;
  }
}

__global__ void k_fill(float* buf, size_t n, float v)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    buf[i] = v;
}

// Host form of an assembly's slot tables: the in-band planes of every
// (direction, order) band grouped by output plane (move_kernel ranges,
// gpuFunctionsImpl.cu:1853-1913), the order-0 bands of a plane in one summed
// slot.  The device copy is laid out as [slots][plane_slot0][plane_nslot]
// [plane_zout][zactive].
struct HostTables {
  std::vector<Slot> slots;
  std::vector<int> p0, pn, pzo;
  std::vector<unsigned char> zact;
  size_t bytes() const
  {
    return slots.size() * sizeof(Slot) + 3 * p0.size() * sizeof(int) + zact.size();
  }
};

HostTables build_tables(const AssembleArgs& a)
{
  HostTables t;
  const int nz = a.nz;
  std::vector<int> kzs;  // signed kz planes of the band grid (z in [-nz/2+1, nz/2])
  if (nz > 1)
    for (int z = -(nz / 2 - 1); z <= nz / 2; ++z) kzs.push_back(z);
  else
    kzs.push_back(0);
  t.zact.assign(a.Z, 0);
  for (int kz : kzs) {
    const int start = (int)t.slots.size();
    const int az = kz < 0 ? -kz : kz;
    const int zo = kz < 0 ? kz + a.Z : kz;
    if (az <= a.zdc[0]) t.slots.push_back(Slot{-1, 0, kz, zo});  // order 0 of all directions, summed
    for (int d = 0; d < a.ndirs; ++d)
      for (int o = 1; o < a.norders; ++o)
        if (az <= a.zdc[o]) t.slots.push_back(Slot{d, o, kz, zo});
    const int cnt = (int)t.slots.size() - start;
    if (cnt > 0) {
      t.p0.push_back(start);
      t.pn.push_back(cnt);
      t.pzo.push_back(zo);
      t.zact[zo] = 1;
    }
  }
  return t;
}

struct DevTables {
  Slot* slots;
  int *p0, *pn, *pz;
  unsigned char* zact;
};
DevTables dev_tables(const AssembleArgs& a, const HostTables& t)
{
  DevTables d;
  d.slots = (Slot*)a.tables;
  d.p0 = (int*)(d.slots + t.slots.size());
  d.pn = d.p0 + t.p0.size();
  d.pz = d.pn + t.p0.size();
  d.zact = (unsigned char*)(d.pz + t.p0.size());
  return d;
}

}  // namespace

namespace {
FilterK make_filter_k(const FilterArgs& a)
{
  FilterK k{};
  const int no = a.norders;
  for (int d = 0; d < a.ndirs; ++d)
    for (int o = 0; o < no; ++o) {
      const int i = d * no + o;
      k.rnv[i] = 1.f / a.noisevar[i];
      k.kxo[i] = o * a.k0[d].x;
      k.kyo[i] = o * a.k0[d].y;
    }
  k.rdkrotf = 1.f / a.otf.dkrotf;
  k.min_dkr = a.dkx < a.dky ? a.dkx : a.dky;
  k.rmin_dkr = 1.f / k.min_dkr;
  k.supp_r = a.supp_radius * k.min_dkr;
  k.rrcut = 1.f / a.rdistcutoff;
  k.r2_in = r2_below(a.rdistcutoff);
  k.r2_supp = r2_atmost(k.supp_r);
  k.rapo = 1.f / a.apocutoff;
  k.rzapo = a.zapocutoff > 0 ? 1.f / a.zapocutoff : 0.f;
  k.order0_shared = 1;
  for (int d = 1; d < a.ndirs; ++d)
    if (a.noisevar[d * no] != a.noisevar[0]) k.order0_shared = 0;
  return k;
}

// Every looked-up radius is <= rdistcutoff, so the table is never left when
// floor(rdistcutoff / dkrotf) + 3 <= nxotf (+ 3: a cross term's interpolation
// radius comes from an approximate square root and may pass rdistcutoff by
// an ulp) and no kz index, |kz| <= nz/2, leaves it along kz; otherwise the
// lookups clamp
bool filter_needs_clamp(const FilterArgs& a, const FilterK& k)
{
  return !(std::floor(a.rdistcutoff * k.rdkrotf) + 3 <= a.otf.nxotf) ||
         !(a.nz == 1 || (a.nz / 2) * (double)a.otf.kzscale + 1.0 < a.otf.nzotf);
}

// the switches fixed at compile time on the table path
int filter_flags(const FilterArgs& a)
{
  return (a.suppress ? 1 : 0) | (a.dampen0 ? 2 : 0) | (a.filteroverlaps ? 4 : 0);
}
}  // namespace

int launch_filter(const FilterArgs& a, cudaStream_t s, long long* launches)
{
  const int nxh = a.nx / 2 + 1;
  dim3 g((a.ny * nxh + kThreads - 1) / kThreads, a.nz, a.norders);
  const FilterK k = make_filter_k(a);
  const int no = a.norders;
  const bool clamp = filter_needs_clamp(a, k);
  KernelTimer* kt = kernel_timer();
  if (kt) kt->begin(s);
  // per-plane radial tables when the lookups stay inside the table and the
  // tables fit in 48 KB of shared memory
  const size_t tabb = 2 * (size_t)no * a.otf.nxotf * sizeof(float2);
  const bool tab = !clamp && tabb <= 48 * 1024;
  // the table path with the three switches fixed at compile time
  const int fl = filter_flags(a);
  auto tab_path = [&]<int NO>() {
    auto go = [&]<int FL>() { k_filter<3, NO, false, true, FL><<<g, kThreads, tabb, s>>>(a, k); };
    switch (fl) {
      case 0: go.template operator()<0>(); break;
      case 1: go.template operator()<1>(); break;
      case 2: go.template operator()<2>(); break;
      case 3: go.template operator()<3>(); break;
      case 4: go.template operator()<4>(); break;
      case 5: go.template operator()<5>(); break;
      case 6: go.template operator()<6>(); break;
      default: go.template operator()<7>(); break;
    }
  };
  if (a.ndirs == 3 && a.norders == 3 && tab) tab_path.template operator()<3>();
  else if (a.ndirs == 3 && a.norders == 3 && !clamp) k_filter<3, 3, false, false><<<g, kThreads, 0, s>>>(a, k);
  else if (a.ndirs == 3 && a.norders == 3) k_filter<3, 3, true, false><<<g, kThreads, 0, s>>>(a, k);
  else if (a.ndirs == 3 && a.norders == 2 && tab) tab_path.template operator()<2>();
  else if (a.ndirs == 3 && a.norders == 2 && !clamp) k_filter<3, 2, false, false><<<g, kThreads, 0, s>>>(a, k);
  else if (a.ndirs == 3 && a.norders == 2) k_filter<3, 2, true, false><<<g, kThreads, 0, s>>>(a, k);
  else k_filter<0, 0, true, false><<<g, kThreads, 0, s>>>(a, k);
  // every element of the 2*norders-1 bands of this direction is read (in
  // band) or only written (cleared)
  double planeb = (double)a.ny * nxh * sizeof(float2);
  double bytes = 0;
  for (int o = 0; o < a.norders; ++o) {
    int nb = o == 0 ? 1 : 2;
    int inb = std::min(a.nz, 2 * a.zdc[o] + 1);
    bytes += nb * planeb * (2.0 * inb + (a.nz - inb));
  }
  if (kt) kt->end("k_filter", s, bytes);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

int launch_ramp_tables(const K0List& k0, int ndirs, int norders, int X, int Y, float dxyz, float fact, float2* ex,
                       float2* ey, cudaStream_t s, long long* launches)
{
  if (ndirs < 1 || ndirs > kMaxDirs) return -1;
  int n = ndirs * norders * (X + Y);
  k_ramp<<<std::min(1024, (n + 255) / 256), 256, 0, s>>>(k0, ndirs, norders, X, Y, dxyz, fact, ex, ey);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

int launch_fill(float* buf, size_t n, float v, cudaStream_t s, long long* launches)
{
  k_fill<<<1216, 256, 0, s>>>(buf, n, v);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

// The slot tables live in their own small device buffer, written once per
// geometry: a launch makes no host-to-device copy, so it never waits behind
// another stream's large transfer on a copy engine and can be captured in a
// CUDA graph.
size_t assemble_tables_bytes(const AssembleArgs& a)
{
  // the largest table set of the geometry: every order in band on every plane
  AssembleArgs full = a;
  for (int o = 0; o < kMaxOrders; ++o) full.zdc[o] = a.nz;
  return (build_tables(full).bytes() + 255) / 256 * 256;
}

int assemble_tables_upload(const AssembleArgs& a)
{
  if (!a.tables) return -2;
  const HostTables t = build_tables(a);
  if (t.bytes() > assemble_tables_bytes(a)) return -2;
  const DevTables d = dev_tables(a, t);
  cudaError_t e = cudaSuccess;
  auto put = [&](void* dst, const void* src, size_t n) {
    if (n && e == cudaSuccess) e = cudaMemcpy(dst, src, n, cudaMemcpyHostToDevice);
  };
  put(d.slots, t.slots.data(), t.slots.size() * sizeof(Slot));
  put(d.p0, t.p0.data(), t.p0.size() * sizeof(int));
  put(d.pn, t.pn.data(), t.pn.size() * sizeof(int));
  put(d.pz, t.pzo.data(), t.pzo.size() * sizeof(int));
  put(d.zact, t.zact.data(), t.zact.size());
  return (int)e;
}

namespace {
constexpr size_t kFusedTabMax = 32 * 1024;  // OTF tables of the fused kernel (two CTAs per SM stay resident)

int assemble_impl(const AssembleArgs& a, const FilterArgs* filt, cudaStream_t s, long long* launches);
}  // namespace

bool assemble_filter_fusable(const AssembleArgs& a, const FilterArgs& f, bool one_otf)
{
  if (!one_otf || f.bessel || a.ndirs != 3 || f.ndirs != 3 || a.norders != f.norders) return false;
  if (f.norders != 2 && f.norders != 3) return false;
  if (!(a.Y == 1024 || a.Y == 512 || a.Y == 256) || a.nx != f.nx || a.ny != f.ny || a.nz != f.nz) return false;
  const FilterK k = make_filter_k(f);
  if (filter_needs_clamp(f, k)) return false;
  return 2 * (size_t)f.norders * f.otf.nxotf * sizeof(float2) <= kFusedTabMax;
}

int launch_assemble_filtered(const AssembleArgs& a, const FilterArgs& f, bool one_otf, cudaStream_t s,
                             long long* launches)
{
  if (!assemble_filter_fusable(a, f, one_otf)) return -10;
  return assemble_impl(a, &f, s, launches);
}

int launch_assemble(const AssembleArgs& a, cudaStream_t s, long long* launches)
{
  return assemble_impl(a, nullptr, s, launches);
}

namespace {
int assemble_impl(const AssembleArgs& a, const FilterArgs* filt, cudaStream_t s, long long* launches)
{
  FFTPlan py, px, pz;
  if (!get_fft_plan(a.Y, &py) || !get_fft_plan(a.X, &px) || !get_fft_plan(a.Z, &pz)) return -1;
  const int nx = a.nx;
  // slot tables: built on the host (a few hundred entries), their device copy
  // uploaded once per geometry by assemble_tables_upload
  if (!a.tables) return -2;
  const HostTables tabs = build_tables(a);
  const std::vector<Slot>& slots = tabs.slots;
  const std::vector<int>& p0 = tabs.p0;
  const std::vector<int>& pn = tabs.pn;
  const DevTables dt = dev_tables(a, tabs);
  Slot* d_slots = dt.slots;
  int* d_p0 = dt.p0;
  int* d_pn = dt.pn;
  int* d_pz = dt.pz;
  unsigned char* d_zact = dt.zact;
  const size_t per_slot = (size_t)a.Y * nx;  // complex elements of T per slot
  if (a.tcap < per_slot) return -2;
  const size_t tslots = a.tcap / per_slot;  // slots that fit in T at once
  // tile sizes
  int Wy = std::max(1, std::min(32, kMaxElems / a.Y));
  size_t smy = fft_stage_smem(a.Y, Wy, a.Y * (Wy + 1), kThreads);

  int xlines = std::max(1, kMaxElems / a.X);
  xlines = std::min(xlines, 16);
  size_t smx = fft_stage_smem(a.X, xlines, xlines * (a.X + 1), kThreads);

  if (a.X > kAccPerThread * kThreads) return -3;
  // process whole planes in groups whose slots fit in T
  size_t np = p0.size();
  size_t pi = 0;
  long long nl = 0;
  while (pi < np) {
    size_t pj = pi;
    int first = p0[pi];
    while (pj < np && (size_t)(p0[pj] + pn[pj] - first) <= tslots) ++pj;
    if (pj == pi) return -4;
    int nsl = p0[pj - 1] + pn[pj - 1] - first;
    // T holds slots [first, first + nsl); shift the slot pointer so that
    // blockIdx.y indexes T from 0
    AssembleArgs ay = a;
    KernelTimer* kt = kernel_timer();
    if (kt) kt->begin(s);
    if (filt) {
      const FilterK fk = make_filter_k(*filt);
      const int fl = filter_flags(*filt);
      const size_t tabb = 2 * (size_t)filt->norders * filt->otf.nxotf * sizeof(float2);
      auto go = [&]<int YN, int NO, int FL>() {
        const size_t bytes = ColFft<YN, colfft_r1(YN), 8>::kSmemElems * sizeof(float2) + tabb;
        allow_dynamic_smem((const void*)k_asm_y4f<YN, NO, FL>, bytes);
        k_asm_y4f<YN, NO, FL><<<dim3((nx + 7) / 8, nsl), kThreads, bytes, s>>>(ay, d_slots + first, py.tw, *filt, fk);
      };
      auto by_fl = [&]<int YN, int NO>() {
        switch (fl) {
          case 0: go.template operator()<YN, NO, 0>(); break;
          case 1: go.template operator()<YN, NO, 1>(); break;
          case 2: go.template operator()<YN, NO, 2>(); break;
          case 3: go.template operator()<YN, NO, 3>(); break;
          case 4: go.template operator()<YN, NO, 4>(); break;
          case 5: go.template operator()<YN, NO, 5>(); break;
          case 6: go.template operator()<YN, NO, 6>(); break;
          default: go.template operator()<YN, NO, 7>(); break;
        }
      };
      auto by_no = [&]<int YN>() {
        if (filt->norders == 3) by_fl.template operator()<YN, 3>();
        else by_fl.template operator()<YN, 2>();
      };
      if (a.Y == 1024) by_no.template operator()<1024>();
      else if (a.Y == 512) by_no.template operator()<512>();
      else by_no.template operator()<256>();
    } else if (colfft_r1(a.Y)) {
      auto go = [&]<int YN>() {
        const size_t bytes = ColFft<YN, colfft_r1(YN), 8>::kSmemElems * sizeof(float2);
        allow_dynamic_smem((const void*)k_asm_y4<YN>, bytes);
        k_asm_y4<YN><<<dim3((nx + 7) / 8, nsl), kThreads, bytes, s>>>(ay, d_slots + first, py.tw);
      };
      if (a.Y == 1024) go.template operator()<1024>();
      else if (a.Y == 512) go.template operator()<512>();
      else go.template operator()<256>();
    } else {
      dispatch_fft_len(kSiteAsmY, a.Y, [&]<int NF>() {
        allow_dynamic_smem((const void*)k_asm_y<NF>, smy);
        k_asm_y<NF><<<dim3((nx + Wy - 1) / Wy, nsl), kThreads, smy, s>>>(ay, d_slots + first, py, Wy);
      });
    }
    if (kt) {
      double rd = 0;
      for (int q = first; q < first + nsl; ++q)
        rd += (slots[q].dir < 0 ? a.ndirs : (slots[q].order == 0 ? 1 : 2)) * (double)a.ny * nx * 8;
      kt->end(filt ? "k_asm_y_filter" : "k_asm_y", s, rd + (double)nsl * per_slot * sizeof(float2));
    }
    // k_asm_x reads T[(slot - first)]: pass a shifted T base
    AssembleArgs ax = a;
    ax.T = a.T - (size_t)first * per_slot;
    if (kt) kt->begin(s);
    auto launch_xw = [&]<int XN>() {
      constexpr int G = 32 / XwLanes<XN>::P;
      const int rows_per_cta = kXwWarps * G;
      constexpr size_t bytes = xw_smem_bytes<XN>();
      allow_dynamic_smem((const void*)k_asm_xw<XN>, bytes);
      k_asm_xw<XN><<<dim3((a.Y + rows_per_cta - 1) / rows_per_cta, (unsigned)(pj - pi)), kXwWarps * 32, bytes,
                     s>>>(ax, d_p0 + pi, d_pn + pi, d_slots, d_pz + pi, px.twr);
    };
    // the warp kernel's prefetch ring holds X/2 = nx columns (zoom factor 2)
    if (a.X == 1024 && a.nx == 512) launch_xw.template operator()<1024>();
    else if (a.X == 512 && a.nx == 256) launch_xw.template operator()<512>();
    else if (a.X == 256 && a.nx == 128) launch_xw.template operator()<256>();
    else
      dispatch_fft_len(kSiteAsmX, a.X, [&]<int NF>() {
        allow_dynamic_smem((const void*)k_asm_x<NF>, smx);
        k_asm_x<NF><<<dim3(a.Y, (unsigned)(pj - pi)), kThreads, smx, s>>>(ax, d_p0 + pi, d_pn + pi, d_slots,
                                                                         d_pz + pi, px, xlines);
      });
    if (kt) kt->end("k_asm_x", s, (double)nsl * per_slot * sizeof(float2) + (double)(pj - pi) * a.X * a.Y * 8);
    nl += 2;
    pi = pj;
  }
  int Wz = std::max(1, std::min(32, kMaxElems / a.Z));
  size_t smz = fft_stage_smem(a.Z, Wz, a.Z * (Wz + 1), kThreads);
  KernelTimer* kt = kernel_timer();
  if (kt) kt->begin(s);
  const int zr1 = a.Z % 16 == 0 ? a.Z / 16 : 0;
  if (a.Z == 1 && ((size_t)a.X * a.Y) % 2 == 0) {
    const size_t npairs = (size_t)a.X * a.Y / 2;
    const unsigned nb = (unsigned)std::min<size_t>((npairs + kThreads - 1) / kThreads, 152 * 16);
    k_asm_z1<<<nb, kThreads, 0, s>>>((const float4*)a.S, (float2*)a.out, npairs, d_zact);
  } else if (zr1 == 2 || zr1 == 3 || zr1 == 4 || zr1 == 5 || zr1 == 6 || zr1 == 8) {
    auto go = [&]<int R1>() {
      const size_t bytes = (size_t)R1 * (16 * 64 + 8) * sizeof(float2);
      allow_dynamic_smem((const void*)k_asm_z4<R1>, bytes);
      k_asm_z4<R1><<<dim3((a.X + 63) / 64, a.Y), kThreads, bytes, s>>>(a, d_zact, pz.tw);
    };
    switch (zr1) {
      case 2: go.template operator()<2>(); break;
      case 3: go.template operator()<3>(); break;
      case 4: go.template operator()<4>(); break;
      case 5: go.template operator()<5>(); break;
      case 6: go.template operator()<6>(); break;
      default: go.template operator()<8>(); break;
    }
  } else {
    dispatch_fft_len(kSiteAsmZ, a.Z, [&]<int NF>() {
      allow_dynamic_smem((const void*)k_asm_z<NF>, smz);
      k_asm_z<NF><<<dim3((a.X + Wz - 1) / Wz, a.Y), kThreads, smz, s>>>(a, d_zact, pz, Wz);
    });
  }
  if (kt) kt->end("k_asm_z", s, (double)np * a.X * a.Y * 8 + (double)a.X * a.Y * a.Z * 4);
  nl += 1;
  if (launches) *launches += nl;
  return (int)cudaGetLastError();
}
}  // namespace

}  // namespace simrecon
