// makeotf on the GPU (the computation of src/otf/radialft.cpp).
//
// Pipeline, one stream, PSF resident in device memory:
//   k_mo_section    per section: camera-pixel fix, border background
//                   (radialft.cpp:228-237, 487-503), edge apodisation (695-720)
//   k_mo_argmax_*   bead centre: peak of the phase average + parabolas (507-614)
//   k_mo_separate   background subtraction (299-305) and band separation
//                   (440-485) into full-complex band volumes
//   k_mo_fft_*      3D forward FFT per band (339-348); y and z only over the
//                   kx >= 0 half the OTF keeps
//   k_mo_shift_comp shift of the bead to the origin (846-874) and bead-size
//                   compensation (784-841, 1155-1167), fused
//   k_mo_radial     radial average per (band, kz) over a precomputed table of
//                   the pixels of each kr bin (876-921): float sums in the
//                   reference's pixel order (deterministic)
//   k_mo_finish     one CTA: Hermitian symmetry (923-934), modify (1169-1186),
//                   cleanup (938-999), fixorigin (1188-1224), rescale
//                   (1226-1242), combine_reim (746-782), conj (411-415) and the
//                   output layout of outputdata (1073-1099)
// The float32 steps whose rounding decides something downstream (apodisation,
// the phase average and its argmax, the parabola fits, the separation, the
// shift phases and the bin index) use explicitly rounded operations so they
// follow the reference's (non-fused) float arithmetic.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kernels.h"
#include "makeotf.h"
#include "reg_fft.cuh"
#include "sim_common.cuh"

namespace simrecon {

namespace {

constexpr int kMoThreads = 256;
constexpr int kNapodize = 10;
constexpr int kBorder = 20;
constexpr int kMoMaxPhases = 9;

struct ApoFact {
  float f[kNapodize];
};

struct SepMatrix {
  float m[kMoMaxPhases * kMoMaxPhases];  // m[band * nph + phase]
};

// ------------------------------------------------------------------ sections
__global__ void __launch_bounds__(kMoThreads) k_mo_section(float* psf, float* bg, int nx, int ny, int use_const,
                                                           float bgconst, double border_count, ApoFact fact)
{
  __shared__ double red[32];
  __shared__ float s_bg;
  float* sec = psf + (size_t)blockIdx.x * nx * ny;
  if (threadIdx.x == 0) {
    // camera fix for old CCDs (radialft.cpp:229-230)
    float v = sec[(size_t)(ny - 1) * nx + nx - 1];
    if (v < 0) sec[(size_t)(ny - 1) * nx + nx - 1] = sec[(size_t)(ny - 1) * nx + nx - 2];
  }
  __syncthreads();
  if (use_const) {
    if (threadIdx.x == 0) s_bg = bgconst;
  } else {
    double s = 0.0;
    for (int t = threadIdx.x; t < nx * ny; t += blockDim.x) {
      int y = t / nx, x = t - y * nx;
      if (y < kBorder || y > ny - kBorder || x < kBorder || x > nx - kBorder) s += (double)sec[t];
    }
    s = block_sum_d(s, red);
    if (threadIdx.x == 0) s_bg = (float)(s / border_count);
  }
  __syncthreads();
  if (threadIdx.x == 0) bg[blockIdx.x] = s_bg;
  // apodize: columns (top/bottom rows) first, then rows (left/right columns)
  for (int k = threadIdx.x; k < nx; k += blockDim.x) {
    float d = __fdiv_rn(__fsub_rn(sec[(size_t)(ny - 1) * nx + k], sec[k]), 2.f);
    for (int l = 0; l < kNapodize; ++l) {
      float df = __fmul_rn(d, fact.f[l]);
      sec[(size_t)l * nx + k] = __fadd_rn(sec[(size_t)l * nx + k], df);
      sec[(size_t)(ny - 1 - l) * nx + k] = __fsub_rn(sec[(size_t)(ny - 1 - l) * nx + k], df);
    }
  }
  __syncthreads();
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    float* row = sec + (size_t)l * nx;
    float d = __fdiv_rn(__fsub_rn(row[nx - 1], row[0]), 2.f);
    for (int k = 0; k < kNapodize; ++k) {
      float df = __fmul_rn(d, fact.f[k]);
      row[k] = __fadd_rn(row[k], df);
      row[nx - 1 - k] = __fsub_rn(row[nx - 1 - k], df);
    }
  }
}

// ------------------------------------------------------------------- centre
// phase average of one voxel (float32, phases summed in order, then / nph)
__device__ __forceinline__ float mo_avg(const float* __restrict__ psf, int nph, size_t nxy, int z, size_t rem)
{
  float s = 0.f;
  for (int p = 0; p < nph; ++p) s = __fadd_rn(s, psf[((size_t)z * nph + p) * nxy + rem]);
  return __fdiv_rn(s, (float)nph);
}

// keep (v, i) if larger, or equal with a smaller index (first maximum)
__device__ __forceinline__ void mo_better(float& bv, long long& bi, float v, long long i)
{
  if (v > bv || (v == bv && i >= 0 && (bi < 0 || i < bi))) {
    bv = v;
    bi = i;
  }
}

__device__ __forceinline__ void mo_block_argmax(float& bv, long long& bi, float* sv, long long* si)
{
  for (int o = 16; o > 0; o >>= 1) {
    float ov = __shfl_down_sync(0xffffffffu, bv, o);
    long long oi = __shfl_down_sync(0xffffffffu, bi, o);
    mo_better(bv, bi, ov, oi);
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
    sv[wid] = bv;
    si[wid] = bi;
  }
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  bv = threadIdx.x < nw ? sv[threadIdx.x] : 0.f;
  bi = threadIdx.x < nw ? si[threadIdx.x] : -1;
  if (wid == 0)
    for (int o = 16; o > 0; o >>= 1) {
      float ov = __shfl_down_sync(0xffffffffu, bv, o);
      long long oi = __shfl_down_sync(0xffffffffu, bi, o);
      mo_better(bv, bi, ov, oi);
    }
}

// Only values > 0 count (the reference starts from maxval = 0 with a strict
// comparison), so the initial state is (0, none).
__global__ void __launch_bounds__(kMoThreads) k_mo_argmax_partial(const float* __restrict__ psf, int nx, int ny,
                                                                  int nz, int nph, float* bval, long long* bidx)
{
  __shared__ float sv[32];
  __shared__ long long si[32];
  const size_t nxy = (size_t)nx * ny, nv = nxy * nz;
  float bv = 0.f;
  long long bi = -1;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
    int z = (int)(v / nxy);
    float a = mo_avg(psf, nph, nxy, z, v - (size_t)z * nxy);
    if (a > bv) {
      bv = a;
      bi = (long long)v;
    }
  }
  mo_block_argmax(bv, bi, sv, si);
  if (threadIdx.x == 0) {
    bval[blockIdx.x] = bv;
    bidx[blockIdx.x] = bi;
  }
}

// radialft.cpp:672-690 (float32)
__device__ float mo_fitparabola(float a1, float a2, float a3)
{
  float slope = __fmul_rn(0.5f, __fsub_rn(a3, a1));
  float curve = __fsub_rn(__fadd_rn(a3, a1), __fmul_rn(2.f, a2));
  if (curve == 0.f) return 0.f;
  float peak = __fdiv_rn(-slope, curve);
  if (peak > 1.5f || peak < -1.5f) return 0.f;
  return peak;
}

// average at (z, y, x) of the reference's nxExtra-wide stack (zero padding)
__device__ float mo_avg_at(const float* __restrict__ psf, int nx, int ny, int nph, int z, int y, int x)
{
  if (x >= nx) return 0.f;
  return mo_avg(psf, nph, (size_t)nx * ny, z, (size_t)y * nx + x);
}

__global__ void k_mo_center(const float* __restrict__ psf, int nx, int ny, int nz, int nph, const float* bval,
                            const long long* bidx, int nparts, float* center)
{
  __shared__ float sv[32];
  __shared__ long long si[32];
  float bv = 0.f;
  long long bi = -1;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) mo_better(bv, bi, bval[i], bidx[i]);
  mo_block_argmax(bv, bi, sv, si);
  if (threadIdx.x == 0) {
    const int nxe = (nx % 2) ? nx + 1 : nx + 2;
    int maxk = 0, maxi = 0, maxj = 0;
    float maxval = 0.f;
    if (bi >= 0) {
      size_t nxy = (size_t)nx * ny;
      maxk = (int)(bi / nxy);
      size_t rem = bi - (size_t)maxk * nxy;
      maxi = (int)(rem / nx);
      maxj = (int)(rem - (size_t)maxi * nx);
      maxval = bv;
    }
    int im = maxi - 1 < 0 ? maxi - 1 + ny : maxi - 1, ip = maxi + 1 >= ny ? maxi + 1 - ny : maxi + 1;
    int jm = maxj - 1 < 0 ? maxj - 1 + nxe : maxj - 1, jp = maxj + 1 >= nxe ? maxj + 1 - nxe : maxj + 1;
    int km = maxk - 1 < 0 ? maxk - 1 + nz : maxk - 1, kp = maxk + 1 >= nz ? maxk + 1 - nz : maxk + 1;
    float zc = (float)maxk;
    if (nz > 1)
      zc = __fadd_rn((float)maxk, mo_fitparabola(mo_avg_at(psf, nx, ny, nph, km, maxi, maxj), maxval,
                                                 mo_avg_at(psf, nx, ny, nph, kp, maxi, maxj)));
    float yc = __fadd_rn((float)maxi, mo_fitparabola(mo_avg_at(psf, nx, ny, nph, maxk, im, maxj), maxval,
                                                     mo_avg_at(psf, nx, ny, nph, maxk, ip, maxj)));
    float xc = __fadd_rn((float)maxj, mo_fitparabola(mo_avg_at(psf, nx, ny, nph, maxk, maxi, jm), maxval,
                                                     mo_avg_at(psf, nx, ny, nph, maxk, maxi, jp)));
    center[0] = xc;
    center[1] = yc;
    center[2] = zc;
  }
}

// --------------------------------------------------------------- separation
__global__ void __launch_bounds__(kMoThreads) k_mo_separate(const float* __restrict__ psf,
                                                            const float* __restrict__ bg, int nx, int ny, int nz,
                                                            int nph, SepMatrix sm, float2* bands)
{
  const size_t nxy = (size_t)nx * ny, nv = nxy * nz;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
    int z = (int)(v / nxy);
    size_t rem = v - (size_t)z * nxy;
    float in[kMoMaxPhases];
#pragma unroll
    for (int j = 0; j < kMoMaxPhases; ++j)
      if (j < nph) in[j] = __fsub_rn(psf[((size_t)z * nph + j) * nxy + rem], bg[z * nph + j]);
    if (nph == 1) {
      bands[v] = make_float2(in[0], 0.f);
      continue;
    }
    for (int i = 0; i < nph; ++i) {
      float acc = 0.f;
#pragma unroll
      for (int j = 0; j < kMoMaxPhases; ++j)
        if (j < nph) acc = __fadd_rn(acc, __fmul_rn(in[j], sm.m[i * nph + j]));
      bands[(size_t)i * nv + v] = make_float2(acc, 0.f);
    }
  }
}

// ---------------------------------------------------------------------- FFT
// forward transform of nlines contiguous rows of length n (in place)
template <int NF>
__global__ void __launch_bounds__(kMoThreads) k_mo_fft_rows(float2* data, int n, int nlines, FFTPlan plan, int nl)
{
  extern __shared__ float2 sm[];
  const int r0 = blockIdx.x * nl;
  const int nr = min(nl, nlines - r0);
  const int ldl = n + 1;
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    int l = t / n, i = t - l * n;
    sm[l * ldl + i] = l < nr ? data[(size_t)r0 * n + t] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2* res = fft_dispatch<NF, -1>(sm, sm + nl * ldl, plan, nl, ldl, 1);
  for (int t = threadIdx.x; t < nr * n; t += blockDim.x) {
    int l = t / n, i = t - l * n;
    data[(size_t)r0 * n + t] = res[l * ldl + i];
  }
}

// forward transform of the columns c < ncols of length n at element stride
// es; blockIdx.y selects the outer index (base offset blockIdx.y * ostride)
template <int NF>
__global__ void __launch_bounds__(kMoThreads) k_mo_fft_cols(float2* data, int n, size_t es, int ncols,
                                                            size_t ostride, FFTPlan plan, int W)
{
  extern __shared__ float2 sm[];
  const int c0 = blockIdx.x * W;
  const int ld = W + 1;
  float2* base = data + (size_t)blockIdx.y * ostride;
  for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
    int i = t / W, w = t - i * W;
    sm[i * ld + w] = (c0 + w < ncols) ? base[(size_t)i * es + c0 + w] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2* res = fft_dispatch<NF, -1>(sm, sm + n * ld, plan, W, 1, ld);
  for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
    int i = t / W, w = t - i * W;
    if (c0 + w < ncols) base[(size_t)i * es + c0 + w] = res[i * ld + w];
  }
}

// ------------------------------------------------- shift + bead compensation
struct ShiftCompArgs {
  int nx, ny, nz, nph, norders, compensate;
  float dkx, dky, dkz;       // beadsize_compensate's float sampling
  float k0x[kMoMaxPhases];   // per order
  float k0y[kMoMaxPhases];
  float radius, limit;       // bead radius, sphere FT at the origin (float)
};

__global__ void __launch_bounds__(kMoThreads) k_mo_shift_comp(float2* bands, const float* center, ShiftCompArgs a)
{
  const int nxh = a.nx / 2 + 1;
  const int b = blockIdx.y;
  const int order = (b + 1) / 2;
  const size_t nh = (size_t)a.nz * a.ny * nxh;
  const float xc = center[0], yc = center[1], zc = center[2];
  // radialft.cpp:853-855: 2*M_PI*c/n in double, stored as float
  const float dphiz = (float)(2.0 * M_PI * (double)zc / a.nz);
  const float dphiy = (float)(2.0 * M_PI * (double)yc / a.ny);
  const float dphix = (float)(2.0 * M_PI * (double)xc / a.nx);
  float2* band = bands + (size_t)b * a.nz * a.ny * a.nx;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nh; t += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(t % nxh);
    size_t r = t / nxh;
    int y = (int)(r % a.ny), z = (int)(r / a.ny);
    int kz = z > a.nz / 2 ? z - a.nz : z;
    int ky = y > a.ny / 2 ? y - a.ny : y;
    float phi = __fadd_rn(__fadd_rn(__fmul_rn(dphiz, (float)kz), __fmul_rn(dphiy, (float)ky)),
                          __fmul_rn(dphix, (float)x));
    float c = cosf(phi), s = sinf(phi);
    size_t idx = ((size_t)z * a.ny + y) * a.nx + x;
    float2 v = band[idx];
    float2 w = make_float2(__fsub_rn(__fmul_rn(v.x, c), __fmul_rn(v.y, s)),
                           __fadd_rn(__fmul_rn(v.x, s), __fmul_rn(v.y, c)));
    if (a.compensate && !(order == 0 && t == 0)) {
      float fkz = __fmul_rn((float)kz, a.dkz);
      float fky = __fadd_rn(__fmul_rn((float)ky, a.dky), a.k0y[order]);
      float fkx = __fadd_rn(__fmul_rn((float)x, a.dkx), a.k0x[order]);
      float rho = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(fkz, fkz), __fmul_rn(fky, fky)), __fmul_rn(fkx, fkx)));
      double sph;
      if (rho > 0.f || rho < 0.f) {
        double xx = 2.0 * M_PI * (double)a.radius * (double)rho;
        sph = (double)a.radius / (M_PI * (double)rho * (double)rho) * (sin(xx) / xx - cos(xx));
      } else {
        sph = 4.0 * M_PI * pow((double)a.radius, 3.0) / 3.0;
      }
      float ratio = (float)(sph / (double)a.limit);
      w.x = __fdiv_rn(w.x, ratio);
      w.y = __fdiv_rn(w.y, ratio);
    }
    band[idx] = w;
  }
}

// ------------------------------------------------------------ radial average
// thread per (band, kz, bin): float sums over the bin's pixels in the
// reference's order (ky rows, then kx), then / count (radialft.cpp:893-921)
__global__ void __launch_bounds__(128) k_mo_radial(const float2* __restrict__ bands, const int* __restrict__ bin_start,
                                                   const int* __restrict__ bin_pix, int nbins, int nx, int ny, int nz,
                                                   float2* avg)
{
  const int bin = blockIdx.x * blockDim.x + threadIdx.x;
  const int kz = blockIdx.y, b = blockIdx.z;
  if (bin >= nbins) return;
  const int nxh = nx / 2 + 1;
  const float2* plane = bands + ((size_t)b * nz + kz) * ny * nx;
  const int s0 = bin_start[bin], s1 = bin_start[bin + 1];
  float re = 0.f, im = 0.f;
  for (int i = s0; i < s1; ++i) {
    int p = bin_pix[i];
    int y = p / nxh, x = p - y * nxh;
    float2 v = plane[(size_t)y * nx + x];
    re = __fadd_rn(re, v.x);
    im = __fadd_rn(im, v.y);
  }
  const int cnt = s1 - s0;
  float2 r = make_float2(re, im);
  if (cnt > 0) r = make_float2(__fdiv_rn(re, (float)cnt), __fdiv_rn(im, (float)cnt));
  avg[((size_t)b * nbins + bin) * nz + kz] = r;
}

// ---------------------------------------------------------------- finishing
struct FinishArgs {
  int nph, norders, nbins, nz, nx;
  int ifixz, ifixr;
  int cleanup, bessel;
  int leavekz[3];
  float cl_lamda, cl_na, cl_nimm, cl_cosalpha, cl_krmax, cl_dkr, cl_dkz;  // cleanup's float constants
  int fix_kx1, fix_kx2;
  int rescale, five_bands, conj, pishift;
};

__device__ __forceinline__ float2 c_mulf(float2 a, float f) { return make_float2(__fmul_rn(a.x, f), __fmul_rn(a.y, f)); }

__global__ void __launch_bounds__(1024) k_mo_finish(float2* avg, FinishArgs a, float* out, float* scal)
{
  __shared__ double red[32];
  __shared__ float s_scale;
  __shared__ double s_sums[64];
  const int nz = a.nz, nb = a.nbins;
  // Hermitian symmetry along kz per (band, bin)
  for (int t = threadIdx.x; t < a.nph * nb; t += blockDim.x) {
    float2* r = avg + (size_t)t * nz;
    r[0].y = 0.f;
    for (int kz = 1; kz <= nz / 2; ++kz) {
      float2 u = r[kz], w = r[nz - kz];
      float2 v = make_float2(__fdiv_rn(__fadd_rn(u.x, w.x), 2.f), __fdiv_rn(__fsub_rn(u.y, w.y), 2.f));
      r[kz] = v;
      r[nz - kz] = make_float2(v.x, -v.y);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) s_scale = 1.f;
  for (int p = 0; p < a.nph; ++p) {
    const int order = (p + 1) / 2;
    float2* o = avg + (size_t)p * nb * nz;
    __syncthreads();
    // modify (radialft.cpp:1169-1186)
    if (a.ifixz)
      for (int kz = threadIdx.x; kz < nz; kz += blockDim.x)
        if (kz != 0 || order > 0) o[kz] = o[nz + kz];
    __syncthreads();
    if (a.ifixr)
      for (int kx = a.ifixr + threadIdx.x; kx < nb; kx += blockDim.x) {
        float2 u = o[(size_t)kx * nz + 1], w = o[(size_t)kx * nz + nz - 1];
        o[(size_t)kx * nz] = make_float2(__fdiv_rn(__fadd_rn(u.x, w.x), 2.f), __fdiv_rn(__fadd_rn(u.y, w.y), 2.f));
      }
    __syncthreads();
    // cleanup (radialft.cpp:938-999, single objective)
    if (!a.bessel && a.cleanup)
      for (int ix = threadIdx.x; ix < nb; ix += blockDim.x) {
        float2* row = o + (size_t)ix * nz;
        float kr = __fmul_rn((float)ix, a.cl_dkr);
        if (kr <= a.cl_krmax) {
          float beta = asinf(__fdiv_rn(__fsub_rn(a.cl_na, __fmul_rn(kr, a.cl_lamda)), a.cl_nimm));
          float kzedge = __fmul_rn(__fdiv_rn(a.cl_nimm, a.cl_lamda), __fsub_rn(cosf(beta), a.cl_cosalpha));
          float q = __fdiv_rn(kzedge, a.cl_dkz);
          if (order == 0) {
            int kzstart = (int)rintf(__fadd_rn(q, 1.f));
            int kzend = nz - kzstart;
            for (int iz = max(kzstart, 0); iz <= kzend && iz < nz; ++iz) row[iz] = make_float2(0.f, 0.f);
          } else if (order == 1) {
            int jotf = (int)rint((double)q + 0.999);
            int kzend = a.leavekz[0] - jotf;
            for (int iz = 0; iz <= kzend && iz < nz; ++iz) {
              row[iz] = make_float2(0.f, 0.f);
              if (iz != 0) row[nz - iz] = make_float2(0.f, 0.f);
            }
            for (int iz = max(a.leavekz[1] + jotf + 1, 0); iz < nz / 2 + 1; ++iz) {
              row[iz] = make_float2(0.f, 0.f);
              row[(nz - iz) % nz] = make_float2(0.f, 0.f);
            }
          } else {
            int jotf = (int)rint((double)q + 0.999);
            for (int iz = max(a.leavekz[2] + jotf, 0); iz < nz / 2 + 1; ++iz) {
              row[iz] = make_float2(0.f, 0.f);
              row[(nz - iz) % nz] = make_float2(0.f, 0.f);
            }
          }
        } else {
          for (int iz = 0; iz < nz; ++iz) row[iz] = make_float2(0.f, 0.f);
        }
      }
    __syncthreads();
    // fixorigin on band 0 (radialft.cpp:1188-1224)
    if (p == 0 && a.fix_kx1 > 0) {
      for (int i = threadIdx.x; i <= a.fix_kx2; i += blockDim.x) {
        double s = 0.0;
        if (i == 0) s = o[0].x;
        else
          for (int j = 0; j < nz; ++j) s += o[(size_t)i * nz + j].x;
        s_sums[i] = s;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        const float meani = (float)(0.5 * (a.fix_kx1 + a.fix_kx2));
        const int numvals = a.fix_kx2 - a.fix_kx1 + 1;
        double totsum = 0, ysum = 0, sqsum = 0;
        for (int i = a.fix_kx1; i <= a.fix_kx2; ++i) {
          float d = __fsub_rn((float)i, meani);
          totsum += s_sums[i];
          ysum += s_sums[i] * (double)d;
          sqsum += (double)__fmul_rn(d, d);
        }
        const float slope = (float)(ysum / sqsum);
        const float av = (float)(totsum / numvals);
        for (int i = 0; i < a.fix_kx1; ++i) {
          float lineval = __fadd_rn(av, __fmul_rn(__fsub_rn((float)i, meani), slope));
          float2 v = o[(size_t)i * nz];
          v.x = (float)((double)v.x - (s_sums[i] - (double)lineval));
          o[(size_t)i * nz] = v;
        }
      }
      __syncthreads();
    }
    // rescale (radialft.cpp:1226-1242): factor from band 0 (or each band with -rescale)
    if (threadIdx.x == 0 && (order == 0 || a.rescale)) s_scale = __fdiv_rn(1.f, o[0].x);
    __syncthreads();
    const float sc = s_scale;
    for (int i = threadIdx.x; i < nb * nz; i += blockDim.x) o[i] = c_mulf(o[i], sc);
  }
  __syncthreads();
  if (threadIdx.x == 0) *scal = s_scale;
  // combine_reim (radialft.cpp:746-782)
  if (!a.five_bands && a.nph > 1) {
    for (int ord = 1; ord < a.norders; ++ord) {
      float2* re_b = avg + (size_t)(2 * ord - 1) * nb * nz;
      float2* im_b = avg + (size_t)(2 * ord) * nb * nz;
      const int n = (a.nx / 2 + 1) * nz;
      double sr = 0.0, si = 0.0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        sr += (double)hypotf(re_b[i].x, re_b[i].y);
        si += (double)hypotf(im_b[i].x, im_b[i].y);
      }
      sr = block_sum_d(sr, red);
      __syncthreads();
      si = block_sum_d(si, red);
      __shared__ float s_c, s_s;
      if (threadIdx.x == 0) {
        double phi = atan(si / sr);
        const size_t q = (size_t)(a.nx / 4) * nz;
        float r0 = re_b[q].x, i0 = im_b[q].x;
        if (r0 < 0 && i0 > 0) phi += M_PI;
        else if (r0 < 0 && i0 < 0) phi = M_PI - phi;
        else if (r0 > 0 && i0 > 0) phi = -phi;
        if (ord == 1 && a.pishift) phi = M_PI - phi;
        s_c = (float)cos(phi);
        s_s = (float)sin(-phi);
      }
      __syncthreads();
      const float c = s_c, s = s_s;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        float2 u = c_mulf(re_b[i], c), w = c_mulf(im_b[i], s);
        re_b[i] = make_float2(__fadd_rn(u.x, w.x), __fadd_rn(u.y, w.y));
        im_b[i] = make_float2(0.f, 0.f);
      }
      __syncthreads();
    }
  }
  __syncthreads();
  // output bands: all with -5bands, else 0 and the combined 2*o-1
  const int nout = a.five_bands ? a.nph : a.norders;
  for (int t = threadIdx.x; t < nout * nb * nz; t += blockDim.x) {
    int ob = t / (nb * nz), r = t - ob * (nb * nz);
    int src = (a.five_bands || ob == 0) ? ob : 2 * ob - 1;
    float2 v = avg[(size_t)src * nb * nz + r];
    if (a.conj) v.y = -v.y;
    out[2 * (size_t)t] = v.x;
    out[2 * (size_t)t + 1] = v.y;
  }
}

template <typename K>
void set_smem(K kernel, size_t bytes)
{
  allow_dynamic_smem((const void*)kernel, bytes);
}

bool mo_fail(std::string* err, const std::string& m)
{
  if (err) *err = m;
  return false;
}

bool parse_int(const char* s, int* v)
{
  if (!s || !*s) return false;
  char* end = nullptr;
  long x = std::strtol(s, &end, 10);
  if (*end) return false;
  *v = (int)x;
  return true;
}

bool parse_float(const char* s, float* v)
{
  if (!s || !*s) return false;
  char* end = nullptr;
  float x = std::strtof(s, &end);
  if (*end) return false;
  *v = x;
  return true;
}

// shared switch parser; positional arguments go to `pos` (nullptr: refused)
bool parse_common(int n, const char* const* a, MakeOtfOptions* o, std::vector<std::string>* pos, std::string* err)
{
  int i = 0;
  auto need = [&](int k) { return i + k < n; };
  while (i < n) {
    std::string s = a[i];
    bool ok = true;
    if (s == "-angle") ok = need(1) && parse_float(a[i + 1], &o->angle), i += 2;
    else if (s == "-ls") ok = need(1) && parse_float(a[i + 1], &o->ls), i += 2;
    else if (s == "-fixorigin")
      ok = need(2) && parse_int(a[i + 1], &o->fixorigin[0]) && parse_int(a[i + 2], &o->fixorigin[1]), i += 3;
    else if (s == "-leavekz")
      ok = need(3) && parse_int(a[i + 1], &o->leavekz[0]) && parse_int(a[i + 2], &o->leavekz[1]) &&
           parse_int(a[i + 3], &o->leavekz[2]),
      i += 4;
    else if (s == "-rescale") o->rescale = true, i += 1;
    else if (s == "-5bands") o->five_bands = true, i += 1;
    else if (s == "-conj") o->conj = true, i += 1;
    else if (s == "-nocompen") o->compensate = false, i += 1;
    else if (s == "-nphases") ok = need(1) && parse_int(a[i + 1], &o->nphases), i += 2;
    else if (s == "-beaddiam") ok = need(1) && parse_float(a[i + 1], &o->beaddiam), i += 2;
    else if (s == "-background") ok = need(1) && parse_float(a[i + 1], &o->background), i += 2;
    else if (s == "-na") ok = need(1) && parse_float(a[i + 1], &o->na), i += 2;
    else if (s == "-nimm") ok = need(1) && parse_float(a[i + 1], &o->nimm), i += 2;
    else if (s == "-ifixkz") ok = need(1) && parse_int(a[i + 1], &o->ifixz), i += 2;
    else if (s == "-ifixkr") ok = need(1) && parse_int(a[i + 1], &o->ifixr), i += 2;
    else if (s == "-wavelength") {
      int w = 0;
      ok = need(1) && parse_int(a[i + 1], &w) && w > 0;
      o->wavelength = (unsigned)w;
      i += 2;
    } else if (s == "-xyres") ok = need(1) && parse_float(a[i + 1], &o->dr), o->user_dr = true, i += 2;
    else if (s == "-zres") ok = need(1) && parse_float(a[i + 1], &o->dz), o->user_dz = true, i += 2;
    else if (s == "-bessel") o->bessel = true, i += 1;
    else if (s == "-PIshift") o->pishift = true, i += 1;
    else if (s == "-2lenses" || s == "-I2M" || s == "-gen_order0" || s == "-bgInExtHdr")
      return mo_fail(err, "makeotf switch " + s + " (two-objective / I2M / band-0 export / extended-header "
                                                  "background) is not supported");
    else if (s == "-help" || s == "-h")
      return mo_fail(err, "usage: makeotf psf otf [-nphases n] [-angle a] [-ls s] [-xyres dr] [-zres dz] "
                          "[-na NA] [-nimm n] [-wavelength nm] [-beaddiam d] [-background b] [-fixorigin k1 k2] "
                          "[-leavekz a b c] [-ifixkz n] [-ifixkr n] [-nocompen] [-5bands] [-rescale] [-conj] "
                          "[-bessel] [-PIshift]");
    else if (pos && s.size() && s[0] != '-' && pos->size() < 2) pos->push_back(s), i += 1;
    else
      return mo_fail(err, "invalid command line option " + s);
    if (!ok) return mo_fail(err, "invalid input for switch " + s);
  }
  if (o->nphases < 1 || o->nphases > kMoMaxPhases) return mo_fail(err, "nphases must be 1..9");
  return true;
}

}  // namespace

bool makeotf_parse(int argc, const char* const* argv, MakeOtfOptions* o, std::string* in, std::string* out,
                   std::string* err)
{
  std::vector<std::string> pos;
  if (!parse_common(argc - 1, argv + 1, o, &pos, err)) return false;
  if (pos.size() < 2) return mo_fail(err, "makeotf needs a PSF file and an output OTF file");
  *in = pos[0];
  *out = pos[1];
  return true;
}

bool makeotf_parse_switches(int n, const char* const* args, MakeOtfOptions* o, std::string* err)
{
  return parse_common(n, args, o, nullptr, err);
}

bool makeotf_run(const float* psf, int nx, int ny, int nsec, const MakeOtfOptions& o, OtfResult* res,
                 std::string* err, cudaStream_t s)
{
  const int nph = o.nphases;
  if (nph < 1 || nph > kMoMaxPhases) return mo_fail(err, "nphases must be 1..9");
  const int nz = nsec / nph;
  if (nz < 1) return mo_fail(err, "fewer sections than phases");
  if (nx < kBorder || ny < kBorder) return mo_fail(err, "PSF sections must be at least 20 x 20 pixels");
  if (nx > ny)
    return mo_fail(err, "PSF width larger than its height is not supported (makeotf's radial average is sized by "
                        "min(nx, ny) but filled up to nx/2)");
  const int norders = (nph + 1) / 2;
  const int nxh = nx / 2 + 1;
  const int nr = std::min(nx, ny);
  const int nbins = nr / 2 + 1;
  if (o.fixorigin[0] > 0 && (o.fixorigin[1] < o.fixorigin[0] || o.fixorigin[1] >= nbins || o.fixorigin[1] >= 64))
    return mo_fail(err, "-fixorigin needs kr1 <= kr2 < min(nx/2+1, 64)");
  if (o.ifixr < 0 || o.leavekz[0] < 0) return mo_fail(err, "invalid -ifixkr / -leavekz");
  FFTPlan px, py, pz;
  if (!get_fft_plan(nx, &px) || !get_fft_plan(ny, &py) || (nz > 1 && !get_fft_plan(nz, &pz)))
    return mo_fail(err, "PSF dimensions must factor into 2, 3, 5 and 7");

  // host-side constants with the reference's float arithmetic
  ApoFact fact;
  for (int l = 0; l < kNapodize; ++l)
    fact.f[l] = (float)(1.0 - std::sin((((float)l + 0.5) / kNapodize) * M_PI * 0.5));
  SepMatrix sepm{};
  {
    const double phi = 2 * M_PI / nph;
    for (int j = 0; j < nph; ++j) {
      sepm.m[0 * nph + j] = (float)(1.0 / nph);
      for (int ord = 1; ord < norders; ++ord) {
        sepm.m[(2 * ord - 1) * nph + j] = (float)(std::cos(j * ord * phi) / nph);
        sepm.m[(2 * ord) * nph + j] = (float)(std::sin(j * ord * phi) / nph);
      }
    }
  }
  double border_count = 0;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x)
      if (y < kBorder || y > ny - kBorder || x < kBorder || x > nx - kBorder) border_count += 1;
  // radial bins (radialft.cpp:889-913): rint of the float quotient
  std::vector<int> pix_bin((size_t)ny * nxh, -1), bin_start(nbins + 1, 0), bin_pix;
  {
    volatile float dkx = 1.f / (nx * o.dr), dky = 1.f / (ny * o.dr);
    volatile float maxk = .5f / o.dr, dkr = 1.f / (nr * o.dr);
    for (int iin = 0; iin < ny; ++iin) {
      int ky = iin > ny / 2 ? iin - ny : iin;
      volatile float kyf = ky * dky;
      for (int jin = 0; jin < nxh; ++jin) {
        volatile float kxf = jin * dkx;
        volatile float sx = kxf * kxf, sy = kyf * kyf;
        volatile float ss = sx + sy;
        float rd = std::sqrt((float)ss);
        if (rd < maxk) {
          volatile float q = rd / dkr;
          int b = (int)std::rint((float)q);
          if (b < 0 || b >= nbins) return mo_fail(err, "internal: radial bin out of range");
          pix_bin[(size_t)iin * nxh + jin] = b;
          bin_start[b + 1]++;
        }
      }
    }
    for (int b = 0; b < nbins; ++b) bin_start[b + 1] += bin_start[b];
    bin_pix.resize(bin_start[nbins]);
    std::vector<int> fill(bin_start.begin(), bin_start.end() - 1);
    for (size_t p = 0; p < pix_bin.size(); ++p)
      if (pix_bin[p] >= 0) bin_pix[fill[pix_bin[p]]++] = (int)p;
  }
  ShiftCompArgs sc{};
  sc.nx = nx, sc.ny = ny, sc.nz = nz, sc.nph = nph, sc.norders = norders, sc.compensate = o.compensate;
  sc.dkx = (float)(1. / (nx * o.dr));
  sc.dky = (float)(1. / (ny * o.dr));
  sc.dkz = (float)(1. / (nz * o.dz));
  {
    const float k0mag = 1 / o.ls;
    sc.radius = (float)(o.beaddiam * 0.5);
    sc.limit = (float)(4 * M_PI * sc.radius * sc.radius * sc.radius / 3);
    for (int ord = 0; ord < norders; ++ord) {
      volatile float frac = ((float)ord) / (norders - 1);  // 0/0 for one order, as the reference
      sc.k0x[ord] = frac * k0mag * std::cos(o.angle);
      sc.k0y[ord] = frac * k0mag * std::sin(o.angle);
    }
  }
  FinishArgs fa{};
  fa.nph = nph, fa.norders = norders, fa.nbins = nbins, fa.nz = nz, fa.nx = nx;
  fa.ifixz = o.ifixz, fa.ifixr = o.ifixr;
  fa.cleanup = o.leavekz[0] > 0, fa.bessel = o.bessel;
  for (int i = 0; i < 3; ++i) fa.leavekz[i] = o.leavekz[i];
  fa.cl_lamda = (float)(o.wavelength * 0.001);
  fa.cl_na = o.na;
  fa.cl_nimm = o.nimm;
  fa.cl_cosalpha = std::cos(std::asin(o.na / o.nimm));
  fa.cl_krmax = 2 * o.na / fa.cl_lamda;
  fa.cl_dkr = (float)(1. / (nr * o.dr));
  fa.cl_dkz = (float)(1. / (nz * o.dz));
  fa.fix_kx1 = o.fixorigin[0], fa.fix_kx2 = o.fixorigin[1];
  fa.rescale = o.rescale, fa.five_bands = o.five_bands, fa.conj = o.conj, fa.pishift = o.pishift;

  // device buffers
  const size_t nxy = (size_t)nx * ny, nvox = nxy * nz;
  const int nparts = 2 * 152;
  const int nout = o.five_bands ? nph : norders;
  struct Buf {
    void** p;
    size_t bytes;
  };
  float *d_psf = nullptr, *d_bg = nullptr, *d_center = nullptr, *d_bval = nullptr, *d_out = nullptr,
        *d_scal = nullptr;
  long long* d_bidx = nullptr;
  float2 *d_bands = nullptr, *d_avg = nullptr;
  int *d_bstart = nullptr, *d_bpix = nullptr;
  std::vector<Buf> bufs = {{(void**)&d_psf, (size_t)nsec * nxy * sizeof(float)},
                           {(void**)&d_bg, (size_t)nsec * sizeof(float)},
                           {(void**)&d_center, 4 * sizeof(float)},
                           {(void**)&d_bval, nparts * sizeof(float)},
                           {(void**)&d_bidx, nparts * sizeof(long long)},
                           {(void**)&d_bands, (size_t)nph * nvox * sizeof(float2)},
                           {(void**)&d_avg, (size_t)nph * nbins * nz * sizeof(float2)},
                           {(void**)&d_bstart, (nbins + 1) * sizeof(int)},
                           {(void**)&d_bpix, std::max<size_t>(1, bin_pix.size()) * sizeof(int)},
                           {(void**)&d_out, (size_t)nout * nbins * nz * 2 * sizeof(float)},
                           {(void**)&d_scal, sizeof(float)}};
  size_t total = 0;
  for (auto& b : bufs) total += (b.bytes + 255) & ~(size_t)255;
  char* arena = nullptr;
  cudaError_t e = cudaMalloc((void**)&arena, total);
  if (e != cudaSuccess) return mo_fail(err, std::string("device allocation failed: ") + cudaGetErrorString(e));
  size_t off = 0;
  for (auto& b : bufs) {
    *b.p = arena + off;
    off += (b.bytes + 255) & ~(size_t)255;
  }
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaMemcpyAsync(d_psf, psf, (size_t)nsec * nxy * sizeof(float), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_bstart, bin_start.data(), (nbins + 1) * sizeof(int), cudaMemcpyHostToDevice, s);
  if (!bin_pix.empty())
    cudaMemcpyAsync(d_bpix, bin_pix.data(), bin_pix.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaEventRecord(ev0, s);

  k_mo_section<<<nsec, kMoThreads, 0, s>>>(d_psf, d_bg, nx, ny, o.background >= 0, o.background, border_count,
                                           fact);
  k_mo_argmax_partial<<<nparts, kMoThreads, 0, s>>>(d_psf, nx, ny, nz, nph, d_bval, d_bidx);
  k_mo_center<<<1, kMoThreads, 0, s>>>(d_psf, nx, ny, nz, nph, d_bval, d_bidx, nparts, d_center);
  k_mo_separate<<<4 * 152, kMoThreads, 0, s>>>(d_psf, d_bg, nx, ny, nz, nph, sepm, d_bands);
  // 3D forward FFT of every band: x rows, then y and z over kx <= nx/2
  {
    const int rows = nph * nz * ny;
    int nl = std::max(1, std::min(rows, kFftElems / nx));
    size_t smr = fft_stage_smem(nx, nl, nl * (nx + 1), kMoThreads);
    dispatch_fft_len(kSiteMakeOtf, nx, [&]<int NF>() {
      set_smem(k_mo_fft_rows<NF>, smr);
      k_mo_fft_rows<NF><<<(rows + nl - 1) / nl, kMoThreads, smr, s>>>(d_bands, nx, rows, px, nl);
    });
    int Wy = std::max(1, std::min(32, kFftElems / ny));
    size_t smy = fft_stage_smem(ny, Wy, ny * (Wy + 1), kMoThreads);
    dispatch_fft_len(kSiteMakeOtf, ny, [&]<int NF>() {
      set_smem(k_mo_fft_cols<NF>, smy);
      k_mo_fft_cols<NF><<<dim3((nxh + Wy - 1) / Wy, nph * nz), kMoThreads, smy, s>>>(d_bands, ny, (size_t)nx, nxh,
                                                                                     nxy, py, Wy);
    });
    if (nz > 1) {
      int Wz = std::max(1, std::min(32, kFftElems / nz));
      size_t smz = fft_stage_smem(nz, Wz, nz * (Wz + 1), kMoThreads);
      dispatch_fft_len(kSiteMakeOtf, nz, [&]<int NF>() {
        set_smem(k_mo_fft_cols<NF>, smz);
        for (int b = 0; b < nph; ++b)
          k_mo_fft_cols<NF><<<dim3((nxh + Wz - 1) / Wz, ny), kMoThreads, smz, s>>>(d_bands + (size_t)b * nvox, nz,
                                                                                   nxy, nxh, (size_t)nx, pz, Wz);
      });
    }
  }
  k_mo_shift_comp<<<dim3(2 * 152, nph), kMoThreads, 0, s>>>(d_bands, d_center, sc);
  k_mo_radial<<<dim3((nbins + 127) / 128, nz, nph), 128, 0, s>>>(d_bands, d_bstart, d_bpix, nbins, nx, ny, nz,
                                                                 d_avg);
  k_mo_finish<<<1, 1024, 0, s>>>(d_avg, fa, d_out, d_scal);
  cudaEventRecord(ev1, s);
  e = cudaGetLastError();
  std::vector<float> center(4, 0.f);
  res->data.assign((size_t)nout * nbins * nz * 2, 0.f);
  if (e == cudaSuccess) e = cudaMemcpyAsync(center.data(), d_center, 3 * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(res->data.data(), d_out, res->data.size() * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  float ms = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  cudaFree(arena);
  if (e != cudaSuccess) return mo_fail(err, std::string("makeotf device error: ") + cudaGetErrorString(e));
  res->device_ms = ms;
  res->xc = center[0], res->yc = center[1], res->zc = center[2];
  res->dkr = (float)(1.f / (nx * o.dr));
  res->dkz = (float)(1.f / (nz * o.dz));
  if (nz > 1) {
    res->width = 2 * nz, res->height = nxh, res->depth = nout;
  } else {
    res->width = 2 * nxh, res->height = 1, res->depth = nout;
  }
  return true;
}

}  // namespace simrecon
