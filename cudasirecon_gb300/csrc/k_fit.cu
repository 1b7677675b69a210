// Pattern-vector (k0) and modulation-amplitude fitting kernels.
//
// The reference builds two full-complex "overlap" volumes per fit step
// (makeoverlaps, gpuFunctionsImpl.cu:497-872), inverse-3D-FFTs them, and then
// reduces sum_z conj(X) Y e^{i phi} for every candidate k0 (reductionKernel,
// gpuFunctionsImpl.cu:1150-1220) or sum_z X conj(Y) for the cross-correlation
// (aTimesConjBKernel, 391-414).  Both only need, per lateral pixel, the
// z-sum of conj(X) Y.  By Parseval along z that equals
//     nz * sum_kz conj(X~(kz)) Y~(kz),   X~ = 2D inverse FFT of plane kz,
// so the z transform is never performed: only the 2*zdc+1 non-zero kz
// planes are built and transformed in x and y, and their products are
// accumulated straight into a 2D map P(x, y).  Every candidate k0 of the
// search is then a 2D weighted sum over P.
//
//   k_ovl_build_x   build both overlaps (OTF-weighted band values) row by
//                   row and inverse-FFT along x
//   k_ovl_y_accum   inverse FFT along y, accumulate conj(X)Y, |X|^2, |Y|^2
//                   over a group of kz planes
//   k_p_reduce      sum the plane-group partial maps, finish |X|^2, |Y|^2
//   k_fft_rows/cols cross-correlation FFT of conj(P)
//   k_argmax_*      intensity peak with its neighbours
//   k_modamp_*      sum_xy P e^{i phi_c} for a batch of candidates
#include <algorithm>

#include "col_fft.cuh"
#include "kernels.h"
#include "reg_fft.cuh"
#include "thresholds.h"

namespace simrecon {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxElems = kFftElems;

// ---------------------------------------------------------------- overlaps
// the shift k0 * (order2 - order1): from the arguments, or from device memory
// (a k0 fitted on the device) times kfac
__device__ __forceinline__ float2 ovl_shift(const OverlapArgs& a)
{
  if (a.kdev == nullptr) return make_float2(a.kx, a.ky);
  const float2 k = *a.kdev;
  return make_float2(__fmul_rn(k.x, a.kfac), __fmul_rn(k.y, a.kfac));
}

// Element (j) of overlap `ov` on row (zb, i) before the x transform:
// makeOverlaps0Kernel (ov 0, gpuFunctionsImpl.cu:677-778) / makeOverlaps1Kernel
// (ov 1, 780-872): the order-1/order-2 band value times the partner OTF over
// sqrt(|OTF1|^2 + |OTF2|^2) inside both supports, merged re + i im.
// kzi = otf_kz(a.otf, zb - a.zdc), rdk = 1 / a.otf.dkrotf (per row / thread)
__device__ __forceinline__ float2 ovl_value(const OverlapArgs& a, float2 ks, int ov, int zb, int i, int j,
                                            const OtfKz& kzi, float rdk)
{
  const int nx = a.nx, ny = a.ny, nz = a.nz, nxh = nx / 2 + 1;
  const size_t bplane = (size_t)ny * nxh;
  int z0 = zb - a.zdc;
  if (z0 == 0 && a.nokz0) return make_float2(0.f, 0.f);
  float x1f = (float)j, y1f = (float)i;
  if (x1f > nx / 2) x1f -= nx;
  if (y1f > ny / 2) y1f -= ny;
  x1f *= a.dkx;
  y1f *= a.dky;
  const float r1sq = x1f * x1f + y1f * y1f;
  bool conj = j > nx / 2;
  int jin = conj ? nx - j : j;
  int iin = conj ? (ny - i) % ny : i;
  int zin = ((conj ? -z0 : z0) + nz) % nz;
  size_t indin = (size_t)zin * bplane + (size_t)iin * nxh + jin;
  // every decision below is the reference's float test on a square root,
  // made on the squared value (thresholds from launch_overlaps)
  if (ov == 0 && r1sq <= a.r2_le) {  // rdist1 <= cut
    float x12 = x1f - ks.x, y12 = y1f - ks.y;
    const float r12sq = x12 * x12 + y12 * y12;
    if (r12sq <= a.r2_le) {  // r12 <= cut
      float2 o1 = otf_lookup_rr(a.otf.otf[a.order1], a.otf, sqrtf(r1sq) * rdk, kzi);
      if (cmag2(o1) > a.m_le) {  // |OTF1| > otfcutoff
        float2 o12 = otf_lookup_rr(a.otf.otf[a.order2], a.otf, sqrtf(r12sq) * rdk, kzi);
        if (cmag2(o12) >= a.m_f) {  // |OTF12| * factor > otfcutoff
          const float rroot = 1.f / sqrtf(cmag2(o1) + cmag2(o12));
          float2 fact = make_float2(o12.x * rroot, o12.y * rroot);
          const float2* b1re = a.order1 == 0 ? a.bands : a.bands + (size_t)(2 * a.order1 - 1) * nz * bplane;
          float2 vre = b1re[indin];
          float2 vim = a.order1 == 0 ? make_float2(0.f, 0.f) : a.bands[(size_t)(2 * a.order1) * nz * bplane + indin];
          if (conj) {
            vre.y = -vre.y;
            vim.y = -vim.y;
          }
          vre = cmul(vre, fact);
          vim = cmul(vim, fact);
          return make_float2(vre.x - vim.y, vre.y + vim.x);
        }
      }
    }
  } else if (ov == 1 && r1sq < a.r2_lt) {  // rdist1 < cut
    float x21 = x1f + ks.x, y21 = y1f + ks.y;
    const float r21sq = x21 * x21 + y21 * y21;
    if (r21sq <= a.r2_le) {  // r21 <= cut
      float2 o2 = otf_lookup_rr(a.otf.otf[a.order2], a.otf, sqrtf(r1sq) * rdk, kzi);
      if (cmag2(o2) >= a.m_f) {  // |OTF2| * factor > otfcutoff
        float2 o21 = otf_lookup_rr(a.otf.otf[a.order1], a.otf, sqrtf(r21sq) * rdk, kzi);
        if (cmag2(o21) > a.m_le) {  // |OTF21| > otfcutoff
          const float rroot = 1.f / sqrtf(cmag2(o2) + cmag2(o21));
          float2 fact = make_float2(o21.x * rroot, o21.y * rroot);
          float2 vre = a.bands[(size_t)(2 * a.order2 - 1) * nz * bplane + indin];
          float2 vim = a.bands[(size_t)(2 * a.order2) * nz * bplane + indin];
          if (conj) {
            vre.y = -vre.y;
            vim.y = -vim.y;
          }
          vre = cmul(vre, fact);
          vim = cmul(vim, fact);
          return make_float2(vre.x - vim.y, vre.y + vim.x);
        }
      }
    }
  }
  return make_float2(0.f, 0.f);
}

template <int NF>
__global__ void __launch_bounds__(kThreads) k_ovl_build_x(OverlapArgs a, FFTPlan plan, int rows_per_cta, int ldl)
{
  extern __shared__ float2 sm[];
  const int nx = a.nx, ny = a.ny;
  const int nzb = 2 * a.zdc + 1;
  const int row0 = blockIdx.x * rows_per_cta;
  const int nrows = min(rows_per_cta, nzb * ny - row0);
  const float2 ks = ovl_shift(a);
  for (int t = threadIdx.x; t < 2 * rows_per_cta * nx; t += blockDim.x) {
    int l = t / nx, j = t - l * nx;
    int r = l >> 1, ov = l & 1;
    float2 val = make_float2(0.f, 0.f);
    if (r < nrows) {
      int row = row0 + r;
      int zb = row / ny, i = row - zb * ny;
      val = ovl_value(a, ks, ov, zb, i, j, otf_kz(a.otf, zb - a.zdc), 1.f / a.otf.dkrotf);
    }
    sm[l * ldl + j] = val;
  }
  __syncthreads();
  const float2* res = fft_dispatch<NF, +1>(sm, sm + 2 * rows_per_cta * ldl, plan, 2 * rows_per_cta, ldl, 1);
  const size_t vol = (size_t)nzb * ny * nx;
  for (int t = threadIdx.x; t < 2 * nrows * nx; t += blockDim.x) {
    int l = t / nx, j = t - l * nx;
    int r = l >> 1, ov = l & 1;
    a.ovl[(size_t)ov * vol + (size_t)(row0 + r) * nx + j] = res[l * ldl + j];
  }
}

// Warp-level variant for the row lengths with a register configuration:
// each warp owns 32/P consecutive overlap lines (line = 2 * row + ov), builds
// their elements into a warp-private buffer, and each group of P lanes runs
// its line's inverse x FFT in registers and stores it (no CTA barrier).
template <int N>
struct OvlLanes {
  static constexpr int P = N == 1024 ? 32 : (N == 512 || N == 256 ? 16 : 0);
};
constexpr int kOvlWarps = 4;

// Five CTAs per SM (at most 96 registers, no spills): the kernel is bound by
// its resident warps (per 512^2 x 48 volume: 0.64 ms with three CTAs, 0.55
// with four, 0.51 with five, 0.54 with six and spills)
template <int N>
__global__ void __launch_bounds__(kOvlWarps * 32, 5) k_ovl_build_xw(OverlapArgs a, const float2* __restrict__ twr)
{
  constexpr int P = OvlLanes<N>::P, E = N / P, G = 32 / P;
  constexpr int XB = (P + 1) * E + 1;
  constexpr int LB = N > XB ? N : XB;  // line buffer, reused as the exchange buffer
  __shared__ float2 lines[kOvlWarps][G][LB];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / P, p = lane - g * P;
  const int ny = a.ny, nzb = 2 * a.zdc + 1;
  const int nlines = 2 * nzb * ny;
  const int l0 = (blockIdx.x * kOvlWarps + warp) * G;
  // build the warp's G lines (all 32 lanes, consecutive j); the kz part of
  // the OTF lookups is the same along a line
  const float rdk = 1.f / a.otf.dkrotf;
  const float2 ks = ovl_shift(a);
#pragma unroll
  for (int gl = 0; gl < G; ++gl) {
    const int L = l0 + gl;
    if (L >= nlines) {
      for (int j = lane; j < N; j += 32) lines[warp][gl][j] = make_float2(0.f, 0.f);
      continue;
    }
    const int row = L >> 1, ov = L & 1;
    const int zb = row / ny, i = row - zb * ny;
    const OtfKz kzi = otf_kz(a.otf, zb - a.zdc);
    for (int j = lane; j < N; j += 32) lines[warp][gl][j] = ovl_value(a, ks, ov, zb, i, j, kzi, rdk);
  }
  __syncwarp();
  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) v[e] = lines[warp][g][p + P * e];
  __syncwarp();  // every lane has its values before the buffer becomes the exchange
  reg_line<N, P, +1>(v, p, lines[warp][g], twr, true);
  const int L = l0 + g;
  if (L < nlines) {
    const int row = L >> 1, ov = L & 1;
    float2* dst = a.ovl + (size_t)ov * nzb * ny * N + (size_t)row * N;
#pragma unroll
    for (int m = 0; m < E / P; ++m)
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) dst[p + P * m + E * k2] = v[m * P + k2];
  }
}

template <int NF>
__global__ void __launch_bounds__(kThreads) k_ovl_y_accum(OverlapArgs a, FFTPlan plan, int W, int planes_per_group,
                                                          int xoff)
{
  extern __shared__ float2 sm[];
  __shared__ double red[32];
  const int nx = a.nx, ny = a.ny;
  const int nzb = 2 * a.zdc + 1;
  const int c0 = blockIdx.x * W;
  const int zb0 = blockIdx.y * planes_per_group;
  const int zb1 = min(nzb, zb0 + planes_per_group);
  const int ld = 2 * W + 1;  // odd pitch: conflict-free strided lane reads
  float2* acc = sm + (size_t)xoff;  // [ny][W], after the two FFT buffers
  for (int t = threadIdx.x; t < ny * W; t += blockDim.x) acc[t] = make_float2(0.f, 0.f);
  double sx = 0.0, sy = 0.0;
  const size_t vol = (size_t)nzb * ny * nx;
  for (int zb = zb0; zb < zb1; ++zb) {
    __syncthreads();
    for (int t = threadIdx.x; t < ny * 2 * W; t += blockDim.x) {
      int y = t / (2 * W), q = t - y * 2 * W;
      int ov = q >= W, w = q - ov * W;
      sm[y * ld + q] =
          (c0 + w < nx) ? a.ovl[(size_t)ov * vol + ((size_t)zb * ny + y) * nx + c0 + w] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const float2* res = fft_dispatch<NF, +1>(sm, sm + ny * ld, plan, 2 * W, 1, ld);
    // this plane's |X|^2 and |Y|^2 in float (ny*W/blockDim terms per
    // thread), added to the double totals once per plane
    float px = 0.f, py = 0.f;
    for (int t = threadIdx.x; t < ny * W; t += blockDim.x) {
      int y = t / W, w = t - y * W;
      float2 X = res[y * ld + w], Y = res[y * ld + W + w];
      float2 p = acc[t];
      // conj(X) * Y, as reductionKernel's xsy (gpuFunctionsImpl.cu:1177-1178)
      p.x += X.x * Y.x + X.y * Y.y;
      p.y += X.x * Y.y - X.y * Y.x;
      acc[t] = p;
      px += cmag2(X);
      py += cmag2(Y);
    }
    sx += (double)px;
    sy += (double)py;
  }
  __syncthreads();
  float2* dst = a.ppart + (size_t)blockIdx.y * ny * nx;
  for (int t = threadIdx.x; t < ny * W; t += blockDim.x) {
    int y = t / W, w = t - y * W;
    if (c0 + w < nx) dst[(size_t)y * nx + c0 + w] = acc[t];
  }
  double tx = block_sum_d(sx, red);
  double ty = block_sum_d(sy, red);
  if (threadIdx.x == 0) {
    int cta = blockIdx.y * gridDim.x + blockIdx.x;
    a.sums[2 * cta] = tx;
    a.sums[2 * cta + 1] = ty;
  }
}

// Four-step variant (col_fft.cuh layout) of k_ovl_y_accum for ny in
// {256, 512}: per kz plane of the group, stage 1 transforms the 8 columns of
// both overlaps (half of the threads each, rows loaded straight from HBM),
// stage 2 gives each thread one (column, k1) of both, and conj(X)Y, |X|^2,
// |Y|^2 accumulate in registers over the planes.
template <int N, int R1>
__global__ void __launch_bounds__(kThreads, 2) k_ovl_y4(OverlapArgs a, const float2* __restrict__ tw,
                                                    int planes_per_group)
{
  using CF = ColFft<N, R1, 8>;
  constexpr int W = 8, R2 = CF::R2, LD1 = CF::LD1;
  static_assert(R2 * W * 2 == kThreads, "stage 1 gives half of the CTA to each overlap");
  static_assert(R1 * W <= kThreads, "one stage-2 item per thread");
  extern __shared__ float2 sm[];  // 2 * CF::kSmemElems
  __shared__ double red[32];
  const int nx = a.nx, ny = N;
  const int nzb = 2 * a.zdc + 1;
  const int c0 = blockIdx.x * W;
  const int nc = min(W, nx - c0);
  const int zb0 = blockIdx.y * planes_per_group;
  const int zb1 = min(nzb, zb0 + planes_per_group);
  const size_t vol = (size_t)nzb * ny * nx;
  // stage-1 item of this thread
  const int ov1 = threadIdx.x / (R2 * W), it1 = threadIdx.x - ov1 * (R2 * W);
  const int c1 = it1 % W, j1 = it1 / W;
  float2* buf1 = sm + ov1 * CF::kSmemElems;
  // stage-2 item
  const bool has2 = threadIdx.x < R1 * W;
  const int c2 = threadIdx.x % W, k1 = threadIdx.x / W;
  float2 acc[R2];
#pragma unroll
  for (int k2 = 0; k2 < R2; ++k2) acc[k2] = make_float2(0.f, 0.f);
  double sx = 0.0, sy = 0.0;
  for (int zb = zb0; zb < zb1; ++zb) {
    {
      const float2* src = a.ovl + (size_t)ov1 * vol + (size_t)zb * ny * nx + c0 + c1;
      float2 v[R1];
#pragma unroll
      for (int e = 0; e < R1; ++e) v[e] = c1 < nc ? src[(size_t)(j1 + R2 * e) * nx] : make_float2(0.f, 0.f);
      reg_dft<R1, +1>(v);
#pragma unroll
      for (int kk = 1; kk < R1; ++kk) {
        float2 w = __ldg(tw + j1 * kk);
        w.y = -w.y;
        v[kk] = cmul(v[kk], w);
      }
#pragma unroll
      for (int kk = 0; kk < R1; ++kk) buf1[kk * LD1 + j1 * W + c1] = v[kk];
    }
    __syncthreads();
    if (has2) {
      float2 X[R2], Y[R2];
#pragma unroll
      for (int j = 0; j < R2; ++j) {
        X[j] = sm[k1 * LD1 + j * W + c2];
        Y[j] = sm[CF::kSmemElems + k1 * LD1 + j * W + c2];
      }
      reg_dft<R2, +1>(X);
      reg_dft<R2, +1>(Y);
      float px = 0.f, py = 0.f;
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) {
        // conj(X) * Y, as reductionKernel's xsy (gpuFunctionsImpl.cu:1177-1178)
        acc[k2].x += X[k2].x * Y[k2].x + X[k2].y * Y[k2].y;
        acc[k2].y += X[k2].x * Y[k2].y - X[k2].y * Y[k2].x;
        px += cmag2(X[k2]);
        py += cmag2(Y[k2]);
      }
      if (c2 < nc) {  // columns past nx are zero padding, not data
        sx += (double)px;
        sy += (double)py;
      }
    }
    __syncthreads();
  }
  if (has2 && c2 < nc) {
    float2* dst = a.ppart + (size_t)blockIdx.y * ny * nx + c0 + c2;
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) dst[(size_t)(k1 + R1 * k2) * nx] = acc[k2];
  }
  double tx = block_sum_d(sx, red);
  double ty = block_sum_d(sy, red);
  if (threadIdx.x == 0) {
    int cta = blockIdx.y * gridDim.x + blockIdx.x;
    a.sums[2 * cta] = tx;
    a.sums[2 * cta + 1] = ty;
  }
}

// P = nz * sum_g Ppart[g];  sumxy = nz * sum of the CTA partial sums
__global__ void k_p_reduce(OverlapArgs a, int ngroups, int nctas)
{
  __shared__ double red[32];
  const size_t n = (size_t)a.nx * a.ny;
  const float fz = (float)a.nz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float2 s = a.ppart[i];
    for (int g = 1; g < ngroups; ++g) {
      float2 v = a.ppart[(size_t)g * n + i];
      s.x += v.x;
      s.y += v.y;
    }
    a.pmap[i] = make_float2(s.x * fz, s.y * fz);
  }
  if (blockIdx.x == 0) {
    double sx = 0.0, sy = 0.0;
    for (int i = threadIdx.x; i < nctas; i += blockDim.x) {
      sx += a.sums[2 * i];
      sy += a.sums[2 * i + 1];
    }
    sx = block_sum_d(sx, red);
    sy = block_sum_d(sy, red);
    if (threadIdx.x == 0) {
      a.sumxy[0] = sx * a.nz;
      a.sumxy[1] = sy * a.nz;
    }
  }
}

// ---------------------------------------------------------- generic FFTs
// rows of a [nrows][n] array; CONJ_IN conjugates the input on load
template <int DIR, bool CONJ_IN, int NF>
__global__ void __launch_bounds__(kThreads) k_fft_rows(const float2* in, float2* out, int n, int nrows, FFTPlan plan,
                                                       int nl)
{
  extern __shared__ float2 sm[];
  const int r0 = blockIdx.x * nl;
  const int nr = min(nl, nrows - r0);
  const int ldl = n + 1;
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    int l = t / n, i = t - l * n;
    float2 v = l < nr ? in[(size_t)r0 * n + t] : make_float2(0.f, 0.f);
    if (CONJ_IN) v.y = -v.y;
    sm[l * ldl + i] = v;
  }
  __syncthreads();
  const float2* res = fft_dispatch<NF, DIR>(sm, sm + nl * ldl, plan, nl, ldl, 1);
  for (int t = threadIdx.x; t < nr * n; t += blockDim.x) {
    int l = t / n, i = t - l * n;
    out[(size_t)r0 * n + t] = res[l * ldl + i];
  }
}

template <int DIR, int NF>
__global__ void __launch_bounds__(kThreads) k_fft_cols2(float2* data, int n, int ncol, FFTPlan plan, int W)
{
  extern __shared__ float2 sm[];
  const int c0 = blockIdx.x * W;
  const int ld = W + 1;
  for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
    int i = t / W, w = t - i * W;
    sm[i * ld + w] = (c0 + w < ncol) ? data[(size_t)i * ncol + c0 + w] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2* res = fft_dispatch<NF, DIR>(sm, sm + n * ld, plan, W, 1, ld);
  for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
    int i = t / W, w = t - i * W;
    if (c0 + w < ncol) data[(size_t)i * ncol + c0 + w] = res[i * ld + w];
  }
}

// ---------------------------------------------------------------- argmax
// first maximum in row-major order (findpeak, gpuFunctionsImpl.cu:443-457)
__device__ __forceinline__ void better(float& bv, int& bi, float v, int i)
{
  if (v > bv || (v == bv && i < bi)) {
    bv = v;
    bi = i;
  }
}

__global__ void k_argmax_partial(const float2* cc, int n, float* bval, int* bidx)
{
  float bv = -1e30f;
  int bi = 0x7fffffff;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float2 c = cc[i];
    better(bv, bi, c.x * c.x + c.y * c.y, i);
  }
  for (int o = 16; o > 0; o >>= 1) {
    float ov = __shfl_down_sync(0xffffffffu, bv, o);
    int oi = __shfl_down_sync(0xffffffffu, bi, o);
    better(bv, bi, ov, oi);
  }
  __shared__ float sv[32];
  __shared__ int si[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sv[wid] = bv;
    si[wid] = bi;
  }
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
    bv = lane < nw ? sv[lane] : -1e30f;
    bi = lane < nw ? si[lane] : 0x7fffffff;
    for (int o = 16; o > 0; o >>= 1) {
      float ov = __shfl_down_sync(0xffffffffu, bv, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o);
      better(bv, bi, ov, oi);
    }
    if (lane == 0) {
      bval[blockIdx.x] = bv;
      bidx[blockIdx.x] = bi;
    }
  }
}

__device__ __forceinline__ float inten(const float2* cc, int i)
{
  float2 c = cc[i];
  return c.x * c.x + c.y * c.y;
}

__global__ void k_argmax_final(const float2* cc, int nx, int ny, const float* bval, const int* bidx, int nb,
                               float* peak)
{
  float bv = -1e30f;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) better(bv, bi, bval[i], bidx[i]);
  for (int o = 16; o > 0; o >>= 1) {
    float ov = __shfl_down_sync(0xffffffffu, bv, o);
    int oi = __shfl_down_sync(0xffffffffu, bi, o);
    better(bv, bi, ov, oi);
  }
  __shared__ float sv[32];
  __shared__ int si[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sv[wid] = bv;
    si[wid] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int nw = blockDim.x >> 5;
    for (int w = 1; w < nw; ++w) better(sv[0], si[0], sv[w], si[w]);
    int idx = si[0];
    if (idx < 0 || idx >= nx * ny) idx = 0;  // all-NaN input: no maximum
    int ix = idx % nx, iy = idx / nx;
    peak[0] = (float)ix;
    peak[1] = (float)iy;
    peak[2] = inten(cc, iy * nx + (ix + nx - 1) % nx);
    peak[3] = inten(cc, idx);
    peak[4] = inten(cc, iy * nx + (ix + 1) % nx);
    peak[5] = inten(cc, ((iy + ny - 1) % ny) * nx + ix);
    peak[6] = inten(cc, ((iy + 1) % ny) * nx + ix);
  }
}

// ---------------------------------------------------- modamp candidates
constexpr int kCand = 8;  // candidates per pass (register accumulators)
static_assert(2 * kCand == 16, "k_modamp_partial reduces 16 values per thread");

// ex[c][x] = exp(i 2 pi (x - nx/2) kx_c dxy), ey[c][y] likewise
// kdev: one candidate, kdev[0] * kfac (a k0 fitted on the device)
__global__ void k_phase_tables(const __grid_constant__ CandList kc, int ncand, int nx, int ny, float dxy, float2* ex,
                               float2* ey, const float2* kdev, float kfac)
{
  int n = ncand * (nx + ny);
  float2 kd = make_float2(0.f, 0.f);
  if (kdev) kd = make_float2(__fmul_rn(kdev->x, kfac), __fmul_rn(kdev->y, kfac));
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int c = t / (nx + ny), r = t - c * (nx + ny);
    const float2 k = kdev ? kd : kc.k[c];
    double ang;
    if (r < nx) ang = 2.0 * M_PI * ((double)r - 0.5 * nx) * (double)k.x * (double)dxy;
    else ang = 2.0 * M_PI * ((double)(r - nx) - 0.5 * ny) * (double)k.y * (double)dxy;
    double s, co;
    sincos(ang, &s, &co);
    float2 v = make_float2((float)co, (float)s);
    if (r < nx) ex[(size_t)c * nx + r] = v;
    else ey[(size_t)c * ny + (r - nx)] = v;
  }
}

__global__ void __launch_bounds__(256) k_modamp_partial(const float2* __restrict__ P, int nx, int ny,
                                                         const float2* __restrict__ ex, const float2* __restrict__ ey,
                                                         int c0, int nc, double* partial, int ncand)
{
  // per-thread float sums, then one transposed pass over shared memory: 16
  // threads per value each add 16 threads' sums in double, then 16 of those
  __shared__ float sacc[256][2 * kCand + 1];
  __shared__ double sseg[16][2 * kCand];
  float2 acc[kCand];
#pragma unroll
  for (int c = 0; c < kCand; ++c) acc[c] = make_float2(0.f, 0.f);
  const int n = nx * ny;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int y = i / nx, x = i - y * nx;
    float2 p = P[i];
#pragma unroll
    for (int c = 0; c < kCand; ++c) {
      if (c < nc) {
        float2 e = cmul(__ldg(ex + (size_t)(c0 + c) * nx + x), __ldg(ey + (size_t)(c0 + c) * ny + y));
        float2 v = cmul(p, e);
        acc[c].x += v.x;
        acc[c].y += v.y;
      }
    }
  }
#pragma unroll
  for (int c = 0; c < kCand; ++c) {
    sacc[threadIdx.x][2 * c] = acc[c].x;
    sacc[threadIdx.x][2 * c + 1] = acc[c].y;
  }
  __syncthreads();
  const int v = threadIdx.x & 15, seg = threadIdx.x >> 4;
  double sum = 0.0;
#pragma unroll
  for (int i = 0; i < 16; ++i) sum += (double)sacc[seg * 16 + i][v];
  sseg[seg][v] = sum;
  __syncthreads();
  if (threadIdx.x < 2 * nc) {
    double tot = 0.0;
#pragma unroll
    for (int g = 0; g < 16; ++g) tot += sseg[g][threadIdx.x];
    partial[((size_t)blockIdx.x * ncand + c0 + (threadIdx.x >> 1)) * 2 + (threadIdx.x & 1)] = tot;
  }
}

__global__ void k_modamp_final(const double* partial, int nblocks, int ncand, double* out)
{
  __shared__ double red[32];
  int c = blockIdx.x;
  double re = 0.0, im = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    re += partial[((size_t)b * ncand + c) * 2];
    im += partial[((size_t)b * ncand + c) * 2 + 1];
  }
  re = block_sum_d(re, red);
  im = block_sum_d(im, red);
  if (threadIdx.x == 0) {
    out[2 * c] = re;
    out[2 * c + 1] = im;
  }
}

}  // namespace

int launch_overlaps(OverlapArgs& a, cudaStream_t s, long long* launches)
{
  a.r2_le = r2_atmost(a.rdistcutoff);
  a.r2_lt = r2_below(a.rdistcutoff);
  a.m_le = r2_atmost(a.otfcutoff);
  a.m_f = m_above_scaled_root(a.otfcutoff, a.order0_2_factor);
  FFTPlan px, py;
  if (!get_fft_plan(a.nx, &px) || !get_fft_plan(a.ny, &py)) return -1;
  const int nzb = 2 * a.zdc + 1;
  // 1) build + x inverse FFT
  const int ldl = a.nx + 1;
  int rows = std::max(1, kMaxElems / (2 * a.nx));
  rows = std::min(rows, nzb * a.ny);
  size_t sm1 = fft_stage_smem(a.nx, 2 * rows, 2 * rows * ldl, kThreads);
  int nb1 = (nzb * a.ny + rows - 1) / rows;

  KernelTimer* kt = kernel_timer();
  const double ovlb = 2.0 * nzb * a.ny * a.nx * sizeof(float2);
  const double bandplanes = (double)nzb * a.ny * (a.nx / 2 + 1) * sizeof(float2);
  if (kt) kt->begin(s);
  auto launch_w = [&]<int N>() {
    constexpr int G = 32 / OvlLanes<N>::P;
    const int nlines = 2 * nzb * a.ny;
    const int per_cta = kOvlWarps * G;
    k_ovl_build_xw<N><<<(nlines + per_cta - 1) / per_cta, kOvlWarps * 32, 0, s>>>(a, px.twr);
  };
  if (a.nx == 512) launch_w.template operator()<512>();
  else if (a.nx == 1024) launch_w.template operator()<1024>();
  else if (a.nx == 256) launch_w.template operator()<256>();
  else
    dispatch_fft_len(kSiteOvlX, a.nx, [&]<int NF>() {
      allow_dynamic_smem((const void*)k_ovl_build_x<NF>, sm1);
      k_ovl_build_x<NF><<<nb1, kThreads, sm1, s>>>(a, px, rows, ldl);
    });
  if (kt) kt->end("k_ovl_build_x", s, ovlb + (a.order1 == 0 ? 3 : 4) * bandplanes);
  // 2) y inverse FFT + accumulation over kz planes
  const int threads = kThreads;
  int W = std::max(1, std::min(16, kMaxElems / (2 * a.ny)));
  int tiles = (a.nx + W - 1) / W;
  int groups = std::max(1, std::min(nzb, (2 * 152 + tiles - 1) / tiles));
  int ppg = (nzb + groups - 1) / groups;
  groups = (nzb + ppg - 1) / ppg;
  const int tile = a.ny * (2 * W + 1);
  const size_t fsm = fft_stage_smem(a.ny, 2 * W, tile, threads);
  const int xoff = (int)(fsm / sizeof(float2));
  size_t sm2 = fsm + (size_t)a.ny * W * sizeof(float2);
  if (a.ny == 512 || a.ny == 256) {
    // 8 columns per CTA; plane groups so that the grid covers the GPU
    tiles = (a.nx + 7) / 8;
    groups = std::max(1, std::min(nzb, (4 * 152 + tiles - 1) / tiles));
    ppg = (nzb + groups - 1) / groups;
    groups = (nzb + ppg - 1) / ppg;
  }
  if (kt) kt->begin(s);
  auto go4 = [&]<int N, int R1>() {
    const size_t bytes = 2 * ColFft<N, R1, 8>::kSmemElems * sizeof(float2);
    allow_dynamic_smem((const void*)k_ovl_y4<N, R1>, bytes);
    k_ovl_y4<N, R1><<<dim3(tiles, groups), kThreads, bytes, s>>>(a, py.tw, ppg);
  };
  if (a.ny == 512) go4.template operator()<512, 32>();
  else if (a.ny == 256) go4.template operator()<256, 16>();
  else
    dispatch_fft_len(kSiteOvlY, a.ny, [&]<int NF>() {
      allow_dynamic_smem((const void*)k_ovl_y_accum<NF>, sm2);
      k_ovl_y_accum<NF><<<dim3(tiles, groups), threads, sm2, s>>>(a, py, W, ppg, xoff);
    });
  if (kt) kt->end("k_ovl_y_accum", s, ovlb + (double)groups * a.ny * a.nx * sizeof(float2));
  // 3) reduce plane groups
  k_p_reduce<<<std::min(1024, (a.nx * a.ny + 255) / 256), 256, 0, s>>>(a, groups, tiles * groups);
  if (launches) *launches += 3;
  return (int)cudaGetLastError();
}

int launch_crosscorr_peak(const float2* pmap, float2* cc, int nx, int ny, float* blockval, int* blockidx,
                          float* peak, cudaStream_t s, long long* launches)
{
  FFTPlan px, py;
  if (!get_fft_plan(nx, &px) || !get_fft_plan(ny, &py)) return -1;
  int nl = std::max(1, std::min(ny, kMaxElems / nx));
  size_t sm1 = fft_stage_smem(nx, nl, nl * (nx + 1), kThreads);
  KernelTimer* kt = kernel_timer();
  if (kt) kt->begin(s);
  dispatch_fft_len(kSiteCorrRows, nx, [&]<int NF>() {
    allow_dynamic_smem((const void*)k_fft_rows<-1, true, NF>, sm1);
    k_fft_rows<-1, true, NF><<<(ny + nl - 1) / nl, kThreads, sm1, s>>>(pmap, cc, nx, ny, px, nl);
  });
  int W = std::max(1, std::min(32, kMaxElems / ny));
  size_t sm2 = fft_stage_smem(ny, W, (W + 1) * ny, kThreads);
  dispatch_fft_len(kSiteCorrCols, ny, [&]<int NF>() {
    allow_dynamic_smem((const void*)k_fft_cols2<-1, NF>, sm2);
    k_fft_cols2<-1, NF><<<(nx + W - 1) / W, kThreads, sm2, s>>>(cc, ny, nx, py, W);
  });
  int nb = 256;
  k_argmax_partial<<<nb, 256, 0, s>>>(cc, nx * ny, blockval, blockidx);
  k_argmax_final<<<1, 256, 0, s>>>(cc, nx, ny, blockval, blockidx, nb, peak);
  // pmap in, cc out; cc in and out (columns); cc in (argmax)
  if (kt) kt->end("k_crosscorr", s, 5.0 * nx * ny * sizeof(float2));
  if (launches) *launches += 4;
  return (int)cudaGetLastError();
}

namespace {
__global__ void k_ovl_scatter(const float2* __restrict__ ovl, int nx, int ny, int nz, int zdc, float2* vol)
{
  const size_t plane = (size_t)nx * ny, n = 2 * (size_t)nz * plane;
  const int nzb = 2 * zdc + 1;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t ov = i / ((size_t)nz * plane), r = i - ov * nz * plane;
    const int z = (int)(r / plane);
    const size_t e = r - (size_t)z * plane;
    const int z0 = z <= nz / 2 ? z : z - nz;
    const int zb = z0 + zdc;
    vol[i] = (zb >= 0 && zb < nzb) ? ovl[(ov * nzb + zb) * plane + e] : make_float2(0.f, 0.f);
  }
}
}  // namespace

int launch_overlap_volumes(const OverlapArgs& a, float2* vol, cudaStream_t s)
{
  FFTPlan py, pz;
  if (!get_fft_plan(a.ny, &py) || !get_fft_plan(a.nz, &pz)) return -1;
  const size_t plane = (size_t)a.nx * a.ny;
  k_ovl_scatter<<<1216, 256, 0, s>>>(a.ovl, a.nx, a.ny, a.nz, a.zdc, vol);
  auto cols = [&](float2* data, int n, int ncol, const FFTPlan& p) {
    const int W = std::max(1, std::min(32, kMaxElems / n));
    const size_t sm = fft_stage_smem(n, W, (W + 1) * n, kThreads);
    allow_dynamic_smem((const void*)k_fft_cols2<+1, 0>, sm);
    k_fft_cols2<+1, 0><<<(ncol + W - 1) / W, kThreads, sm, s>>>(data, n, ncol, p, W);
  };
  for (int ov = 0; ov < 2; ++ov) {
    float2* v = vol + (size_t)ov * a.nz * plane;
    for (int z = 0; z < a.nz; ++z) cols(v + (size_t)z * plane, a.ny, a.nx, py);  // y
    if (a.nz > 1) cols(v, a.nz, (int)plane, pz);                                 // z
  }
  return (int)cudaGetLastError();
}

namespace {
__global__ void k_copy_out(const unsigned* __restrict__ s1, unsigned* d1, int n1, const unsigned* __restrict__ s2,
                           unsigned* d2, int n2)
{
  for (int i = threadIdx.x; i < n1; i += blockDim.x) d1[i] = s1[i];
  for (int i = threadIdx.x; i < n2; i += blockDim.x) d2[i] = s2[i];
}
}  // namespace

namespace {
// Float arithmetic as the host code does it (compiled without contraction
// into FMA): products and sums rounded separately, so device-finished
// amplitudes equal the host-computed ones bit for bit.
__device__ __forceinline__ float2 cmul_rn(float2 a, float2 b)
{
  return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                     __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float mag2_rn(float2 a) { return __fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)); }

// |amp|^2 and the filter's per-term weights (filterbands, gpuFunctionsImpl.cu:1341-1360)
__device__ void fit_derived(const FitFinishArgs& a, FitDev* out)
{
  for (int i = 0; i < a.ndirs * a.norders; ++i) {
    const int o = i % a.norders;
    const float m2 = mag2_rn(out->amp[i]);
    out->ampmag2[i] = m2;
    out->termw[i] = o == 0 ? a.rnv[i] : __fdiv_rn(m2, a.noisevar[i]);
  }
}

// findModulationVectorsAndPhasesForAllDirections without a k0 search
// (cudaSirecon.cpp:409-492): amp[o] = XStarY / sum|X|^2 of findrealspacemodamp
// (gpuFunctionsImpl.cu:1128-1130), then the 2D chaining, forcemodamp and the
// fitallphases = 0 phase rule, in that order.  One thread: at most 64 values.
__global__ void k_fit_finish(const double* __restrict__ slots, const __grid_constant__ FitFinishArgs a, FitDev* out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int no = a.norders;
  for (int d = 0; d < a.ndirs; ++d) {
    float2* amp = out->amp + d * no;
    amp[0] = make_float2(1.f, 0.f);
    for (int o = 1; o < no; ++o) {
      const double* sl = slots + (size_t)(d * no + o) * 4;
      const float sx = __double2float_rn(sl[2]);
      amp[o] = make_float2(__fdiv_rn(__double2float_rn(sl[0]), sx), __fdiv_rn(__double2float_rn(sl[1]), sx));
    }
    if (a.chain2d)
      for (int o = 2; o < no; ++o) amp[o] = cmul_rn(amp[o], amp[o - 1]);
    if (a.nforce > 0 && a.forceamp[0] > 0.f)
      for (int o = 1; o < no; ++o) {
        const float m = __fsqrt_rn(mag2_rn(amp[o]));
        const float want = o - 1 < a.nforce ? a.forceamp[o - 1] : 0.f;
        if (m < want) {
          const float f = __fdiv_rn(want, m);
          amp[o] = make_float2(__fmul_rn(amp[o].x, f), __fmul_rn(amp[o].y, f));
        }
      }
    if (!a.fitallphases && no > 1) {
      const float base = atan2f(amp[1].y, amp[1].x);
      for (int o = 2; o < no; ++o) {
        const float phi = __fmul_rn((float)o, base);
        amp[o] = cmul_rn(make_float2(__fsqrt_rn(mag2_rn(amp[o])), 0.f), make_float2(cosf(phi), sinf(phi)));
      }
    }
  }
  fit_derived(a, out);
}

__global__ void k_set_fit(const __grid_constant__ AmpList amps, const __grid_constant__ FitFinishArgs a, FitDev* out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i < a.ndirs * a.norders; ++i) out->amp[i] = amps.amp[i];
  fit_derived(a, out);
}
}  // namespace

int launch_fit_finish(const double* slots, const FitFinishArgs& a, FitDev* out, cudaStream_t s, long long* launches)
{
  if (a.ndirs < 1 || a.ndirs > kMaxDirs || a.norders < 1 || a.norders > kMaxOrders) return -1;
  k_fit_finish<<<1, 32, 0, s>>>(slots, a, out);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

int launch_set_fit(const AmpList& amps, const FitFinishArgs& a, FitDev* out, cudaStream_t s, long long* launches)
{
  if (a.ndirs < 1 || a.ndirs > kMaxDirs || a.norders < 1 || a.norders > kMaxOrders) return -1;
  k_set_fit<<<1, 32, 0, s>>>(amps, a, out);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

int launch_copy_out(const void* src1, void* dst1, size_t n1, const void* src2, void* dst2, size_t n2, cudaStream_t s,
                    long long* launches)
{
  k_copy_out<<<1, 128, 0, s>>>((const unsigned*)src1, (unsigned*)dst1, (int)n1, (const unsigned*)src2, (unsigned*)dst2,
                               (int)n2);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

static int modamp_impl(const float2* pmap, int nx, int ny, float dxy, const CandList& kcand, int ncand,
                       const float2* kdev, float kfac, float2* tables, double* partial, double* xstary, cudaStream_t s,
                       long long* launches)
{
  if (ncand < 1 || ncand > kMaxCand) return -1;
  float2* ex = tables;
  float2* ey = tables + (size_t)ncand * nx;
  KernelTimer* kt = kernel_timer();
  if (kt) kt->begin(s);
  // double sincos: spread over all SMs (FP64 throughput is per SM)
  k_phase_tables<<<(ncand * (nx + ny) + 63) / 64, 64, 0, s>>>(kcand, ncand, nx, ny, dxy, ex, ey, kdev, kfac);
  if (kt) kt->end("k_modamp_tables", s, (double)ncand * (nx + ny) * sizeof(float2));
  // about four elements per thread, at most kModampBlocks blocks
  const int nb = (int)std::min<long long>(kModampBlocks, std::max<long long>(1, ((long long)nx * ny + 1023) / 1024));
  if (kt) kt->begin(s);
  for (int c0 = 0; c0 < ncand; c0 += kCand) {
    int nc = std::min(kCand, ncand - c0);
    k_modamp_partial<<<nb, 256, 0, s>>>(pmap, nx, ny, ex, ey, c0, nc, partial, ncand);
    if (launches) *launches += 1;
  }
  if (kt) kt->end("k_modamp", s, (double)((ncand + kCand - 1) / kCand) * nx * ny * sizeof(float2));
  if (kt) kt->begin(s);
  k_modamp_final<<<ncand, 256, 0, s>>>(partial, nb, ncand, xstary);
  if (kt) kt->end("k_modamp_final", s, (double)nb * ncand * 2 * sizeof(double));
  if (launches) *launches += 2;
  return (int)cudaGetLastError();
}

int launch_modamp_candidates(const float2* pmap, int nx, int ny, float dxy, const CandList& kcand, int ncand,
                             float2* tables, double* partial, double* xstary, cudaStream_t s, long long* launches)
{
  return modamp_impl(pmap, nx, ny, dxy, kcand, ncand, nullptr, 0.f, tables, partial, xstary, s, launches);
}

int launch_modamp_device_k(const float2* pmap, int nx, int ny, float dxy, const float2* kdev, float kfac,
                           float2* tables, double* partial, double* xstary, cudaStream_t s, long long* launches)
{
  if (kdev == nullptr) return -1;
  return modamp_impl(pmap, nx, ny, dxy, CandList{}, 1, kdev, kfac, tables, partial, xstary, s, launches);
}

}  // namespace simrecon
