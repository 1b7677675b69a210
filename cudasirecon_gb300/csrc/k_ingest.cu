// Ingest stage: raw camera planes -> separated, z-transformed bands.
//
//   k_ingest_x   flat-field, edge apodization and the x half of the 2D R2C
//                FFT (two real rows packed in one complex line), per plane.
//   k_fft_cols   forward FFT along y of the half spectra (in place).
//   k_rescale    bleach-correction ratios from the plane sums (= DC terms).
//   k_separate   ratio * plane, band separation (nphases x nphases matrix)
//                and the forward FFT along z, in place, per (ky, kx tile).
//
// Reference stages replaced: load_and_flatfield (cudaSirecon.cpp:1715-1731),
// rescale (gpuFunctionsImpl.cu:110-195), apodize (gpuFunctionsImpl.cu:39-82),
// transformXYSlice (cudaSirecon.cpp:542-579), separate
// (gpuFunctionsImpl.cu:214-291) and the z FFT (cudaSirecon.cpp:238-257).
#include <algorithm>

#include "col_fft.cuh"
#include "kernels.h"
#include "reg_fft.cuh"

namespace simrecon {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxElems = kFftElems;  // complex elements per CTA and buffer

__device__ __forceinline__ int raw_section(int d, int p, int z, int nz, int ndirs, int nph, int fastSI)
{
  // loadImageData section order, cudaSirecon.cpp:1374-1382
  return fastSI ? (z * ndirs * nph + d * nph + p) : (d * nz * nph + z * nph + p);
}

template <typename T>
__device__ __forceinline__ float flat(const T* __restrict__ plane, const IngestArgs& a, int y, int x)
{
  float v = (float)plane[(size_t)y * a.nx + x];
  float bg = a.bg ? __ldg(a.bg + (size_t)y * a.nx + x) : a.bgconst;
  float sl = a.slope ? __ldg(a.slope + (size_t)y * a.nx + x) : 1.0f;
  return (v - bg - a.bgextra) * sl * a.inscale;
}

// flat() for a raw value already loaded
__device__ __forceinline__ float flat_v(float v, const IngestArgs& a, int y, int x)
{
  float bg = a.bg ? __ldg(a.bg + (size_t)y * a.nx + x) : a.bgconst;
  float sl = a.slope ? __ldg(a.slope + (size_t)y * a.nx + x) : 1.0f;
  return (v - bg - a.bgextra) * sl * a.inscale;
}

// VEC consecutive raw pixels of row y starting at x (x % VEC == 0), as floats
template <typename T, int VEC>
__device__ __forceinline__ void load_vec(const T* __restrict__ plane, int nx, int y, int x, float* out)
{
  const T* src = plane + (size_t)y * nx + x;
  if constexpr (sizeof(T) == 2 && VEC == 8) {
    uint4 u = __ldg((const uint4*)src);
    const unsigned short* h = (const unsigned short*)&u;
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = (float)h[i];
  } else if constexpr (sizeof(T) == 4 && VEC == 4) {
    float4 f = __ldg((const float4*)src);
    out[0] = f.x;
    out[1] = f.y;
    out[2] = f.z;
    out[3] = f.w;
  } else {
#pragma unroll
    for (int i = 0; i < VEC; ++i) out[i] = (float)src[i];
  }
}

// One CTA: `nl` complex lines = 2*nl rows [y0, y0 + 2 nl) of plane `pl`.
// Line l (rows y0+2l, y0+2l+1 as real / imaginary parts) sits at sm[l*ldl].
template <typename T, int VEC, int NF>
__global__ void __launch_bounds__(kThreads) k_ingest_x(IngestArgs a, FFTPlan plan, int nl, int ldl)
{
  extern __shared__ float2 sm[];
  __shared__ float diffr[2 * 256];
  const int nx = a.nx, ny = a.ny, nxh = nx / 2 + 1;
  const int pl = blockIdx.y;  // plane id = (d*nph + p)*nz + z
  const int z = pl % a.nz;
  const int dp = pl / a.nz;
  const int p = dp % a.nphases, d = dp / a.nphases;
  const int y0 = blockIdx.x * 2 * nl;
  const T* plane = (const T*)a.raw + (size_t)raw_section(d, p, z, a.nz, a.ndirs, a.nphases, a.fastSI) * nx * ny;
  float* smr = (float*)sm;  // row r at x -> smr[2*((r>>1)*ldl + x) + (r&1)]
  const int napo = a.napodize;
  const int nrows = 2 * nl;
  const int nchunk = nx / VEC;
  const bool plainbg = !a.bg && !a.slope;
  // 1) flat-field + top/bottom edge blend (apodize_x_kernel), VEC pixels per thread
  for (int t = threadIdx.x; t < nrows * nchunk; t += blockDim.x) {
    const int r = t / nchunk, x0 = (t - r * nchunk) * VEC;
    const int y = y0 + r;
    float v[VEC];
    if (y < ny) {
      if (plainbg) {
        load_vec<T, VEC>(plane, nx, y, x0, v);
#pragma unroll
        for (int i = 0; i < VEC; ++i) v[i] = (v[i] - a.bgconst - a.bgextra) * 1.0f * a.inscale;
      } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i) v[i] = flat(plane, a, y, x0 + i);
      }
      const bool top = y < napo, bot = (ny - 1 - y) < napo;
      if (top || bot) {
#pragma unroll
        for (int i = 0; i < VEC; ++i) {
          float diff = (flat(plane, a, ny - 1, x0 + i) - flat(plane, a, 0, x0 + i)) / 2.0f;
          if (top) v[i] += diff * a.apofact[y];
          if (bot) v[i] -= diff * a.apofact[ny - 1 - y];
        }
      }
    } else {
#pragma unroll
      for (int i = 0; i < VEC; ++i) v[i] = 0.f;
    }
    float* dst = smr + 2 * ((r >> 1) * ldl + x0) + (r & 1);
#pragma unroll
    for (int i = 0; i < VEC; ++i) dst[2 * i] = v[i];
  }
  __syncthreads();
  // 2) left/right edge blend (apodize_y_kernel) using the blended row ends
  if (napo > 0) {
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
      float e0 = smr[2 * ((r >> 1) * ldl + 0) + (r & 1)];
      float e1 = smr[2 * ((r >> 1) * ldl + nx - 1) + (r & 1)];
      diffr[r] = (e1 - e0) / 2.0f;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nrows * 2 * napo; t += blockDim.x) {
      int r = t / (2 * napo), q = t - r * 2 * napo;
      if (y0 + r >= ny) continue;
      int x = q < napo ? q : nx - 1 - (q - napo);
      int l = q < napo ? q : q - napo;
      float f = diffr[r] * a.apofact[l];
      float* e = &smr[2 * ((r >> 1) * ldl + x) + (r & 1)];
      if (q < napo) *e += f;
      else *e -= f;
    }
  }
  __syncthreads();
  // 3) forward FFT along x of the packed lines
  const float2* res = fft_dispatch<NF, -1>(sm, sm + nl * ldl, plan, nl, ldl, 1);
  // 4) split the two real transforms, keep kx in [0, nx/2]
  float2* dst = a.spec + (size_t)pl * ny * nxh;
  for (int t = threadIdx.x; t < nl * nxh; t += blockDim.x) {
    int l = t / nxh, k = t - l * nxh;
    float2 zk = res[l * ldl + k];
    float2 zn = res[l * ldl + (nx - k) % nx];
    float2 A = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
    float2 B = make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x));
    int y = y0 + 2 * l;
    if (y < ny) dst[(size_t)y * nxh + k] = A;
    if (y + 1 < ny) dst[(size_t)(y + 1) * nxh + k] = B;
  }
}

// Forward/inverse FFT along the middle axis of [nplanes][n][ncol], in place.
// Tile [n][W] with pitch W+1 (odd: conflict-free strided lane reads).
template <int DIR, int NF>
__global__ void __launch_bounds__(kThreads) k_fft_cols(float2* data, int n, int ncol, FFTPlan plan, int W)
{
  extern __shared__ float2 sm[];
  const int c0 = blockIdx.x * W;
  const int ld = W + 1;
  float2* base = data + (size_t)blockIdx.y * n * ncol;
  for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
    int i = t / W, w = t - i * W;
    sm[i * ld + w] = (c0 + w < ncol) ? base[(size_t)i * ncol + c0 + w] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2* res = fft_dispatch<NF, DIR>(sm, sm + n * ld, plan, W, 1, ld);
  for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
    int i = t / W, w = t - i * W;
    if (c0 + w < ncol) base[(size_t)i * ncol + c0 + w] = res[i * ld + w];
  }
}

// Warp-level variant of k_ingest_x for nx in {256, 512, 1024}: each group of
// P lanes owns row pairs (row 2l real, row 2l+1 imaginary), K of them in
// turn; the raw rows of the next pair are copied into a two-entry shared ring
// with cp.async while the current pair is processed.  Per pair the lanes
// read their pixels x = p + P e from the ring, apply the flat field and both
// edge blends in registers (row ends by warp shuffle), transform the line in
// registers and split the two real spectra through their exchange buffer.
// No CTA barrier.
template <int N>
struct IngestLanes {
  static constexpr int P = N == 1024 ? 32 : 16;
};
constexpr int kIngestWarps = 4;
// row pairs per lane group: one, so that a plane spreads over the most CTAs
// (per 512^2 x 48 x 15 volume: 0.56 ms with four pairs, 0.50 with two, 0.46
// with one)
constexpr int kIngestPairs = 1;

template <typename T, int N>
constexpr size_t ingest_xw_smem()
{
  constexpr int P = IngestLanes<N>::P, E = N / P, G = 32 / P;
  return (size_t)kIngestWarps * G * (((P + 1) * E + 1) * sizeof(float2) + 2 * 2 * N * sizeof(T));
}

template <typename T, int N>
__global__ void __launch_bounds__(kIngestWarps * 32, 3) k_ingest_xw(IngestArgs a, const float2* __restrict__ twr)
{
  constexpr int P = IngestLanes<N>::P, E = N / P, G = 32 / P;
  constexpr int XB = (P + 1) * E + 1;  // >= N: also holds the transformed line
  constexpr int RB = 2 * N * (int)sizeof(T);
  static_assert(XB >= N, "exchange buffer too small for the split");
  extern __shared__ __align__(16) unsigned char ig_dyn[];
  const int ny = a.ny, nxh = N / 2 + 1;
  const int pl = blockIdx.y;  // plane id = (d*nph + p)*nz + z
  const int z = pl % a.nz;
  const int dp = pl / a.nz;
  const int ph = dp % a.nphases, d = dp / a.nphases;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / P, p = lane - g * P;
  const int gi = warp * G + g;
  float2* xb = (float2*)ig_dyn + gi * XB;
  unsigned char* rg = ig_dyn + (size_t)kIngestWarps * G * XB * sizeof(float2) + (size_t)gi * 2 * RB;
  const T* plane = (const T*)a.raw + (size_t)raw_section(d, ph, z, a.nz, a.ndirs, a.nphases, a.fastSI) * N * ny;
  const int pairs = (ny + 1) / 2;
  const int lbase = (blockIdx.x * kIngestWarps + warp) * G * kIngestPairs + g;  // pair of turn it: lbase + G*it
  const int napo = a.napodize;
  const bool plainbg = !a.bg && !a.slope;
  auto prefetch = [&](int it) {
    const int l = lbase + G * it;
    if (it < kIngestPairs && l < pairs) {
      const int y = 2 * l;
      const int chunks = (y + 1 < ny ? 2 : 1) * N * (int)sizeof(T) / 16;
      const unsigned char* src = (const unsigned char*)(plane + (size_t)y * N);
      unsigned char* dst = rg + (it & 1) * RB;
      for (int q = p; q < chunks; q += P) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + 16 * q);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + 16 * q) : "memory");
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  prefetch(0);
  for (int it = 0; it < kIngestPairs; ++it) {  // same trip count in every lane
    prefetch(it + 1);
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    __syncwarp();
    const int l = lbase + G * it;
    const int y = 2 * l;
    const bool r0 = y < ny, r1 = y + 1 < ny;
    const T* rrow = (const T*)(rg + (it & 1) * RB);  // row y at [0, N), row y+1 at [N, 2N)
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int x = p + P * e;
      float re = 0.f, im = 0.f;
      if (plainbg) {
        if (r0) re = ((float)rrow[x] - a.bgconst - a.bgextra) * 1.0f * a.inscale;
        if (r1) im = ((float)rrow[N + x] - a.bgconst - a.bgextra) * 1.0f * a.inscale;
      } else {
        if (r0) re = flat_v((float)rrow[x], a, y, x);
        if (r1) im = flat_v((float)rrow[N + x], a, y + 1, x);
      }
      v[e] = make_float2(re, im);
    }
    __syncwarp();  // the ring entry is read before prefetch(it + 2) reuses it
    // top/bottom edge blend (apodize_x_kernel) with the unblended end rows
    const bool e0 = r0 && (y < napo || (ny - 1 - y) < napo);
    const bool e1 = r1 && (y + 1 < napo || (ny - 2 - y) < napo);
    if (e0 || e1) {
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int x = p + P * e;
        const float diff = (flat(plane, a, ny - 1, x) - flat(plane, a, 0, x)) / 2.0f;
        if (e0) {
          if (y < napo) v[e].x += diff * a.apofact[y];
          if ((ny - 1 - y) < napo) v[e].x -= diff * a.apofact[ny - 1 - y];
        }
        if (e1) {
          if (y + 1 < napo) v[e].y += diff * a.apofact[y + 1];
          if ((ny - 2 - y) < napo) v[e].y -= diff * a.apofact[ny - 2 - y];
        }
      }
    }
    // left/right edge blend (apodize_y_kernel) from the blended row ends
    if (napo > 0) {
      const int gb = g * P;
      const float2 first = make_float2(__shfl_sync(0xffffffffu, v[0].x, gb), __shfl_sync(0xffffffffu, v[0].y, gb));
      const float2 last = make_float2(__shfl_sync(0xffffffffu, v[E - 1].x, gb + P - 1),
                                      __shfl_sync(0xffffffffu, v[E - 1].y, gb + P - 1));
      const float dx = (last.x - first.x) / 2.0f, dy = (last.y - first.y) / 2.0f;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int x = p + P * e;
        if (x < napo) {
          v[e].x += dx * a.apofact[x];
          v[e].y += dy * a.apofact[x];
        } else if (x >= N - napo) {
          v[e].x -= dx * a.apofact[N - 1 - x];
          v[e].y -= dy * a.apofact[N - 1 - x];
        }
      }
    }
    reg_line<N, P, -1>(v, p, xb, twr, true);
    // split the two real transforms: X[k] and X[N-k] live in different lanes
#pragma unroll
    for (int m = 0; m < E / P; ++m)
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) xb[p + P * m + E * k2] = v[m * P + k2];
    __syncwarp();
    float2* dst = a.spec + (size_t)pl * ny * nxh;
    for (int k = p; k < nxh; k += P) {
      const float2 zk = xb[k], zn = xb[(N - k) % N];
      const float2 A = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
      const float2 B = make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x));
      if (r0) dst[(size_t)y * nxh + k] = A;
      if (r1) dst[(size_t)(y + 1) * nxh + k] = B;
    }
    // the next turn's reg_line rewrites xb only after the wait + __syncwarp
    // at its top, which every lane reaches after finishing these reads
  }
}

// Four-step variant (col_fft.cuh) for the lengths with a column
// configuration: 8 columns of one plane per CTA, loaded straight from HBM.
template <int N>
__global__ void __launch_bounds__(kThreads) k_fft_cols_4s(float2* data, int ncol, const float2* __restrict__ tw)
{
  constexpr int R1 = colfft_r1(N), W = 8;
  extern __shared__ float2 sm[];  // ColFft<N, R1, W>::kSmemElems
  const int c0 = blockIdx.x * W;
  // planes in the reverse of the order the x pass wrote them: the last ones
  // written are still in L2 when the first CTAs read them
  const int plane = gridDim.y - 1 - blockIdx.y;
  float2* base = data + (size_t)plane * N * ncol + c0;
  const int nc = min(W, ncol - c0);
  colfft_stage1<N, R1, W, -1>(sm, tw, [&](int row, int c) {
    return c < nc ? base[(size_t)row * ncol + c] : make_float2(0.f, 0.f);
  });
  colfft_stage2<N, R1, W, -1>(sm, [&](int row, int c, float2 v) {
    if (c < nc) base[(size_t)row * ncol + c] = v;
  });
}

// Bleach correction (rescale, gpuFunctionsImpl.cu:110-157): per (d, z) the
// nphases plane sums, ref = dir-0 phase-0 sum at z (or at z = 0 with
// equalizez; from time 0 with equalizet), ratio = ref / sum.
__global__ void k_rescale(const float2* __restrict__ spec, int ny, int nxh, int nz, int ndirs, int nph, int t,
                          int equalizez, int equalizet, double* sdp0, float* scale)
{
  const size_t plane = (size_t)ny * nxh;
  for (int z = threadIdx.x; z < nz; z += blockDim.x)
    if (!(equalizet && t != 0)) sdp0[z] = (double)spec[(size_t)z * plane].x;  // d = 0, p = 0
  __syncthreads();
  for (int i = threadIdx.x; i < ndirs * nph * nz; i += blockDim.x) {
    int z = i % nz;
    float sum = spec[(size_t)i * plane].x;
    float ref = (float)(equalizez ? sdp0[0] : sdp0[z]);
    scale[i] = ref / sum;
  }
}

// Separation + forward z FFT.  One CTA = (ky, W columns of kx) of one
// direction; shared tile [z][band][w].
template <int NF>
__global__ void __launch_bounds__(kThreads) k_separate(float2* spec, const float* __restrict__ scale,
                                                       const float* __restrict__ sepmat, int ny, int nxh, int nz,
                                                       int nph, FFTPlan plan, int W)
{
  extern __shared__ float2 sm[];
  __shared__ float M[kMaxPhases * kMaxPhases];
  const int ky = blockIdx.y, c0 = blockIdx.x * W, d = blockIdx.z;
  for (int i = threadIdx.x; i < nph * nph; i += blockDim.x) M[i] = sepmat[i];
  __syncthreads();
  const size_t plane = (size_t)ny * nxh;
  float2* dbase = spec + (size_t)d * nph * nz * plane + (size_t)ky * nxh + c0;
  const float* dscale = scale + d * nph * nz;
  const int ld = nph * W + 1;  // odd pitch
  for (int t = threadIdx.x; t < nz * W; t += blockDim.x) {
    int z = t / W, w = t - z * W;
    float2 in[kMaxPhases];
    bool ok = c0 + w < nxh;
    for (int p = 0; p < nph; ++p) {
      float s = dscale[p * nz + z];
      float2 v = ok ? dbase[((size_t)p * nz + z) * plane + w] : make_float2(0.f, 0.f);
      in[p] = make_float2(v.x * s, v.y * s);
    }
    for (int b = 0; b < nph; ++b) {
      float2 acc = make_float2(0.f, 0.f);
      for (int p = 0; p < nph; ++p) {
        float m = M[b * nph + p];
        acc.x += m * in[p].x;
        acc.y += m * in[p].y;
      }
      sm[z * ld + b * W + w] = acc;
    }
  }
  __syncthreads();
  const float2* res = sm;
  if (nz > 1) res = fft_dispatch<NF, -1>(sm, sm + nz * ld, plan, nph * W, 1, ld);
  const int lw = nph * W;
  for (int t = threadIdx.x; t < nz * lw; t += blockDim.x) {
    int z = t / lw, r = t - z * lw;
    int b = r / W, w = r - b * W;
    if (c0 + w < nxh) dbase[((size_t)b * nz + z) * plane + w] = res[z * ld + r];
  }
}

// 2D (nz = 1): separation alone (no z transform), one thread per element of
// one direction's plane, coalesced along kx; the same arithmetic as k_separate
template <int NPH>
__global__ void __launch_bounds__(kThreads) k_separate_z1(float2* spec, const float* __restrict__ scale,
                                                          const float* __restrict__ sepmat, size_t plane)
{
  __shared__ float M[NPH * NPH];
  for (int i = threadIdx.x; i < NPH * NPH; i += blockDim.x) M[i] = sepmat[i];
  __syncthreads();
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int d = blockIdx.y;
  if (e >= plane) return;
  float2* base = spec + (size_t)d * NPH * plane + e;
  float2 in[NPH];
#pragma unroll
  for (int p = 0; p < NPH; ++p) {
    const float s = scale[d * NPH + p];
    const float2 v = base[(size_t)p * plane];
    in[p] = make_float2(v.x * s, v.y * s);
  }
#pragma unroll
  for (int b = 0; b < NPH; ++b) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < NPH; ++p) {
      const float m = M[b * NPH + p];
      acc.x += m * in[p].x;
      acc.y += m * in[p].y;
    }
    base[(size_t)b * plane] = acc;
  }
}

}  // namespace

static size_t fft_smem(int n, int lines, int elems) { return fft_stage_smem(n, lines, elems, kThreads); }

int launch_ingest(const IngestArgs& a, cudaStream_t s, long long* launches)
{
  FFTPlan px, py;
  if (!get_fft_plan(a.nx, &px) || !get_fft_plan(a.ny, &py)) return -1;
  const int nxh = a.nx / 2 + 1;
  const int nplanes = a.ndirs * a.nphases * a.nz;
  const int ldl = a.nx + 1;
  int nl = std::max(1, std::min(kMaxElems / a.nx, 256));
  nl = std::min(nl, (a.ny + 1) / 2);
  size_t smx = fft_smem(a.nx, nl, nl * ldl);
  dim3 gx((a.ny + 2 * nl - 1) / (2 * nl), nplanes);
  KernelTimer* kt = kernel_timer();
  const double specb = (double)nplanes * a.ny * nxh * sizeof(float2);
  if (kt) kt->begin(s);
  auto go_w = [&]<int N>() {
    constexpr int G = 32 / IngestLanes<N>::P;
    const int pairs = (a.ny + 1) / 2;
    const int per_cta = kIngestWarps * G * kIngestPairs;
    dim3 gw((pairs + per_cta - 1) / per_cta, nplanes);
    if (a.raw_is_u16) {
      constexpr size_t bytes = ingest_xw_smem<uint16_t, N>();
      allow_dynamic_smem((const void*)k_ingest_xw<uint16_t, N>, bytes);
      k_ingest_xw<uint16_t, N><<<gw, kIngestWarps * 32, bytes, s>>>(a, px.twr);
    } else {
      constexpr size_t bytes = ingest_xw_smem<float, N>();
      allow_dynamic_smem((const void*)k_ingest_xw<float, N>, bytes);
      k_ingest_xw<float, N><<<gw, kIngestWarps * 32, bytes, s>>>(a, px.twr);
    }
  };
  if (a.nx == 512) go_w.template operator()<512>();
  else if (a.nx == 1024) go_w.template operator()<1024>();
  else if (a.nx == 256) go_w.template operator()<256>();
  else
  dispatch_fft_len(kSiteIngestX, a.nx, [&]<int NF>() {
    if (a.raw_is_u16) {
      if (a.nx % 8 == 0) {
        allow_dynamic_smem((const void*)k_ingest_x<uint16_t, 8, NF>, smx);
        k_ingest_x<uint16_t, 8, NF><<<gx, kThreads, smx, s>>>(a, px, nl, ldl);
      } else {
        allow_dynamic_smem((const void*)k_ingest_x<uint16_t, 1, 0>, smx);
        k_ingest_x<uint16_t, 1, 0><<<gx, kThreads, smx, s>>>(a, px, nl, ldl);
      }
    } else {
      if (a.nx % 4 == 0) {
        allow_dynamic_smem((const void*)k_ingest_x<float, 4, NF>, smx);
        k_ingest_x<float, 4, NF><<<gx, kThreads, smx, s>>>(a, px, nl, ldl);
      } else {
        allow_dynamic_smem((const void*)k_ingest_x<float, 1, 0>, smx);
        k_ingest_x<float, 1, 0><<<gx, kThreads, smx, s>>>(a, px, nl, ldl);
      }
    }
  });
  if (kt) kt->end("k_ingest_x", s, (double)nplanes * a.nx * a.ny * (a.raw_is_u16 ? 2 : 4) + specb);
  int W = std::max(1, std::min(32, kMaxElems / a.ny));
  size_t smy = fft_smem(a.ny, W, a.ny * (W + 1));
  dim3 gy((nxh + W - 1) / W, nplanes);
  if (kt) kt->begin(s);
  if (colfft_r1(a.ny)) {
    dim3 g4((nxh + 7) / 8, nplanes);
    auto go = [&]<int N>() {
      const size_t bytes = ColFft<N, colfft_r1(N), 8>::kSmemElems * sizeof(float2);
      allow_dynamic_smem((const void*)k_fft_cols_4s<N>, bytes);
      k_fft_cols_4s<N><<<g4, kThreads, bytes, s>>>(a.spec, nxh, py.tw);
    };
    if (a.ny == 512) go.template operator()<512>();
    else if (a.ny == 1024) go.template operator()<1024>();
    else go.template operator()<256>();
  } else {
    dispatch_fft_len(kSiteIngestY, a.ny, [&]<int NF>() {
      allow_dynamic_smem((const void*)k_fft_cols<-1, NF>, smy);
      k_fft_cols<-1, NF><<<gy, kThreads, smy, s>>>(a.spec, a.ny, nxh, py, W);
    });
  }
  if (kt) kt->end("k_fft_y", s, 2 * specb);
  if (launches) *launches += 2;
  return (int)cudaGetLastError();
}

// Four-step variant of k_separate for nz = 16 * R1 (R1 <= 8): 16 columns of
// one (direction, ky) row per CTA.  Stage 1: the thread for (column c,
// j < 16) loads the R1 planes z = j + 16 e of every phase straight from HBM,
// applies the bleach ratios and the separation matrix, and runs the R1-point
// DFT of each band times W_nz^(j k1); stage 2: the thread for (c, band, k1)
// runs the 16-point DFT over j and stores planes k1 + R1 k2 in place.
template <int R1, int NPH>
__global__ void __launch_bounds__(kThreads) k_separate4(float2* spec, const float* __restrict__ scale,
                                                       const float* __restrict__ sepmat, int ny, int nxh,
                                                       const float2* __restrict__ tw)
{
  constexpr int nph = NPH;
  constexpr int R2 = 16, W = 16, NZ = R1 * R2;
  constexpr int LD = R2 * W + 8;  // 2*LD = 16 mod 32 words
  extern __shared__ float2 sm[];   // [nph * R1][LD]
  __shared__ float M[kMaxPhases * kMaxPhases];
  const int ky = blockIdx.y, c0 = blockIdx.x * W, d = blockIdx.z;
  for (int i = threadIdx.x; i < nph * nph; i += blockDim.x) M[i] = sepmat[i];
  __syncthreads();
  const size_t plane = (size_t)ny * nxh;
  float2* dbase = spec + (size_t)d * nph * NZ * plane + (size_t)ky * nxh + c0;
  const float* dscale = scale + d * nph * NZ;
  const int nc = min(W, nxh - c0);
  {
    const int c = threadIdx.x % W, j = threadIdx.x / W;  // R2 * W == blockDim
    float2 in[NPH][R1];
#pragma unroll
    for (int e = 0; e < R1; ++e) {
      const int z = j + R2 * e;
#pragma unroll
      for (int p = 0; p < nph; ++p) {
        float sc = dscale[p * NZ + z];
        float2 v = c < nc ? dbase[((size_t)p * NZ + z) * plane + c] : make_float2(0.f, 0.f);
        in[p][e] = make_float2(v.x * sc, v.y * sc);
      }
    }
#pragma unroll
    for (int b = 0; b < nph; ++b) {
      float2 v[R1];
#pragma unroll
      for (int e = 0; e < R1; ++e) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int p = 0; p < nph; ++p) {
          float m = M[b * nph + p];
          acc.x += m * in[p][e].x;
          acc.y += m * in[p][e].y;
        }
        v[e] = acc;
      }
      reg_dft<R1, -1>(v);
#pragma unroll
      for (int k1 = 1; k1 < R1; ++k1) v[k1] = cmul(v[k1], __ldg(tw + j * k1));
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) sm[(b * R1 + k1) * LD + j * W + c] = v[k1];
    }
  }
  __syncthreads();
  for (int it = threadIdx.x; it < nph * R1 * W; it += blockDim.x) {
    const int c = it % W, r = it / W;  // r = b * R1 + k1
    const int b = r / R1, k1 = r - b * R1;
    float2 u[R2];
#pragma unroll
    for (int jj = 0; jj < R2; ++jj) u[jj] = sm[r * LD + jj * W + c];
    reg_dft<R2, -1>(u);
    if (c < nc)
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) dbase[((size_t)b * NZ + k1 + R1 * k2) * plane + c] = u[k2];
  }
}

namespace {
template <typename T>
__global__ void k_precondition(const __grid_constant__ PrecondArgs a)
{
  const size_t plane = (size_t)a.ny * a.nx, n = (size_t)a.nimg * plane;
  const T* raw = (const T*)a.raw;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(i / plane);
    const size_t r = i - (size_t)s * plane;
    const int y = (int)(r / a.nx), xo = (int)(r - (size_t)y * a.nx);
    const T* sec = raw + (size_t)s * a.ny * a.nx_raw;
    const float bgx = a.bgx ? a.bgx[s] : 0.f;
    // load_and_flatfield of raw pixel (yy, k)
    auto flat = [&](int yy, int k) {
      const size_t q = (size_t)yy * a.nx_raw + k;
      const float bg = a.bg ? a.bg[q] : a.bgconst;
      const float sl = a.slope ? a.slope[q] : 1.0f;
      return (((float)sec[q] - bg) - bgx) * sl * a.inscale;
    };
    float v = 0.f;
    if (a.deskew_factor == 0.f) {
      if (xo < a.nx_raw) v = flat(y, xo);
    } else {
      // z of this raw section (loadImageData's order, cudaSirecon.cpp:1374-1382)
      const int z = a.fastSI ? s / (a.ndirs * a.nphases) : (s / a.nphases) % a.nz;
      const float xin = (float)((double)xo - a.nx / 2. + a.extra_shift - (double)a.deskew_factor * (z - a.nz / 2.) +
                                a.nx_raw / 2.);
      if (xin >= 0 && xin < a.nx_raw) {
        const int i0 = (int)floorf(xin);
        const float off = xin - floorf(xin);
        // the reference reads the next pixel of the section buffer: the next
        // row's first one at the end of a row (zero past the last row)
        const float a1 = i0 + 1 < a.nx_raw ? flat(y, i0 + 1) : (y + 1 < a.ny ? flat(y + 1, 0) : 0.f);
        v = __fadd_rn(__fmul_rn(1.f - off, flat(y, i0)), __fmul_rn(off, a1));
      }
    }
    a.out[i] = v;
  }
}
}  // namespace

int launch_precondition(const PrecondArgs& a, cudaStream_t s, long long* launches)
{
  const size_t n = (size_t)a.nimg * a.ny * a.nx;
  const unsigned nb = (unsigned)std::min<size_t>((n + kThreads - 1) / kThreads, 152 * 16);
  KernelTimer* kt = kernel_timer();
  if (kt) kt->begin(s);
  if (a.raw_is_u16) k_precondition<uint16_t><<<nb, kThreads, 0, s>>>(a);
  else k_precondition<float><<<nb, kThreads, 0, s>>>(a);
  if (kt) kt->end("k_precondition", s, (double)a.nimg * a.ny * a.nx_raw * (a.raw_is_u16 ? 2 : 4) + 4.0 * n);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

int launch_rescale(const float2* spec, int nx, int ny, int nz, int ndirs, int nphases, int t, int equalizez,
                   int equalizet, double* sdp0, float* scale, cudaStream_t s, long long* launches)
{
  k_rescale<<<1, 256, 0, s>>>(spec, ny, nx / 2 + 1, nz, ndirs, nphases, t, equalizez, equalizet, sdp0, scale);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

int launch_separate(float2* spec, const float* scale, const float* sepmat, int nx, int ny, int nz, int ndirs,
                    int nphases, cudaStream_t s, long long* launches)
{
  FFTPlan pz;
  if (!get_fft_plan(nz, &pz)) return -1;
  if (nphases > kMaxPhases) return -1;
  const int nxh = nx / 2 + 1;
  int W = 32;
  while (W > 1 && (nphases * W + 1) * nz > kMaxElems) W >>= 1;
  size_t sm = fft_smem(nz, nphases * W, (nphases * W + 1) * nz);
  dim3 g((nxh + W - 1) / W, ny, ndirs);
  KernelTimer* kt = kernel_timer();
  if (kt) kt->begin(s);
  const int r1 = nz % 16 == 0 ? nz / 16 : 0;
  if (nz == 1 && (nphases == 3 || nphases == 5)) {
    const size_t plane = (size_t)ny * nxh;
    dim3 g1((unsigned)((plane + kThreads - 1) / kThreads), ndirs);
    if (nphases == 3) k_separate_z1<3><<<g1, kThreads, 0, s>>>(spec, scale, sepmat, plane);
    else k_separate_z1<5><<<g1, kThreads, 0, s>>>(spec, scale, sepmat, plane);
  } else if ((r1 == 2 || r1 == 3 || r1 == 4 || r1 == 5 || r1 == 6 || r1 == 8) && nphases == 5) {
    dim3 g4((nxh + 15) / 16, ny, ndirs);
    auto go = [&]<int R1>() {
      const size_t bytes = (size_t)nphases * R1 * (16 * 16 + 8) * sizeof(float2);
      allow_dynamic_smem((const void*)k_separate4<R1, 5>, bytes);
      k_separate4<R1, 5><<<g4, kThreads, bytes, s>>>(spec, scale, sepmat, ny, nxh, pz.tw);
    };
    switch (r1) {
      case 2: go.template operator()<2>(); break;
      case 3: go.template operator()<3>(); break;
      case 4: go.template operator()<4>(); break;
      case 5: go.template operator()<5>(); break;
      case 6: go.template operator()<6>(); break;
      default: go.template operator()<8>(); break;
    }
  } else {
    dispatch_fft_len(kSiteSeparateZ, nz, [&]<int NF>() {
      allow_dynamic_smem((const void*)k_separate<NF>, sm);
      k_separate<NF><<<g, kThreads, sm, s>>>(spec, scale, sepmat, ny, nxh, nz, nphases, pz, W);
    });
  }
  if (kt) kt->end("k_separate", s, 2.0 * ndirs * nphases * nz * (double)ny * nxh * sizeof(float2));
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

}  // namespace simrecon
