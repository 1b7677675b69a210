// Shared-memory Stockham FFT engine for sm_103a.
//
// One CTA transforms `nl` lines of length n held in shared memory, element
// (line l, index i) at sm[l*ldl + i*ldi].  Two layouts are used:
//   * "rows"    (ldi == 1): lines are contiguous rows (x transforms);
//   * "columns" (ldl == 1): lines are interleaved, W consecutive columns of a
//     strided axis staged as an [n][W] tile (y / z transforms), so that the
//     global loads and stores of a tile are 8*W-byte coalesced segments.
// The transform is an autosorting Stockham sequence of radix-2/3/4/5/7/8/16/32
// stages ping-ponging between two shared buffers of the same layout.  Twiddles come from a per-length
// table tw[k] = exp(-2 pi i k / n) computed in double precision on the host.
//
// Kernels built on this engine supply a Loader that fills the shared lines
// (fusing whatever element-wise work precedes the transform: flat-fielding,
// apodization, band separation, OTF weighting, zero padding ...) and a Storer
// that consumes them (fusing what follows: two-for-one real splits, phase
// ramps, accumulation, reductions ...).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace simrecon {

constexpr int kMaxStages = 16;

struct FFTPlan {
  int n;
  int nstages;
  int radix[kMaxStages];
  const float2* tw;   // device table of n twiddles exp(-2 pi i k/n)
  const float2* twr;  // register path (n with P lanes): twr[(k1-1)*P + p] = tw[p*k1], lane-major so a
                      // lane group reads consecutive entries; null when n has no register path
};

#ifdef __CUDACC__

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b)  // a * conj(b)
{
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i*DIR... : for the forward transform (DIR=-1) rot(a) = -i a, inverse (+1) = +i a
template <int DIR>
__device__ __forceinline__ float2 rot90(float2 a)
{
  return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

// ---------------------------------------------------------------- butterflies
template <int DIR>
__device__ __forceinline__ void dft2(float2* v)
{
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <int DIR>
__device__ __forceinline__ void dft3(float2* v)
{
  const float c = -0.5f;
  const float s = 0.86602540378443864676f * (DIR < 0 ? -1.f : 1.f);
  float2 t1 = cadd(v[1], v[2]);
  float2 t2 = csub(v[1], v[2]);
  float2 m = make_float2(v[0].x + c * t1.x, v[0].y + c * t1.y);
  float2 r = make_float2(-s * t2.y, s * t2.x);  // i*s*t2
  v[0] = cadd(v[0], t1);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}

template <int DIR>
__device__ __forceinline__ void dft4(float2* v)
{
  float2 a0 = cadd(v[0], v[2]);
  float2 a1 = csub(v[0], v[2]);
  float2 a2 = cadd(v[1], v[3]);
  float2 a3 = rot90<DIR>(csub(v[1], v[3]));
  v[0] = cadd(a0, a2);
  v[2] = csub(a0, a2);
  v[1] = cadd(a1, a3);
  v[3] = csub(a1, a3);
}

template <int DIR>
__device__ __forceinline__ void dft5(float2* v)
{
  const float c1 = 0.30901699437494742410f;   // cos(2pi/5)
  const float c2 = -0.80901699437494742410f;  // cos(4pi/5)
  const float sg = DIR < 0 ? -1.f : 1.f;
  const float s1 = 0.95105651629515357212f * sg;  // sin(2pi/5)
  const float s2 = 0.58778525229247312917f * sg;  // sin(4pi/5)
  float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  float2 t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  float2 a1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
  float2 a2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
  // b = i*(s1*t3 + s2*t4), d = i*(s2*t3 - s1*t4)
  float2 b1 = make_float2(-(s1 * t3.y + s2 * t4.y), s1 * t3.x + s2 * t4.x);
  float2 b2 = make_float2(-(s2 * t3.y - s1 * t4.y), s2 * t3.x - s1 * t4.x);
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = cadd(a1, b1);
  v[4] = csub(a1, b1);
  v[2] = cadd(a2, b2);
  v[3] = csub(a2, b2);
}

template <int DIR>
__device__ __forceinline__ void dft7(float2* v)
{
  const float c1 = 0.62348980185873353053f, c2 = -0.22252093395631440429f, c3 = -0.90096886790241912624f;
  const float sg = DIR < 0 ? -1.f : 1.f;
  const float s1 = 0.78183148246802980871f * sg, s2 = 0.97492791218182360702f * sg,
              s3 = 0.43388373911755812048f * sg;
  float2 p1 = cadd(v[1], v[6]), m1 = csub(v[1], v[6]);
  float2 p2 = cadd(v[2], v[5]), m2 = csub(v[2], v[5]);
  float2 p3 = cadd(v[3], v[4]), m3 = csub(v[3], v[4]);
  float2 x0 = v[0];
  float2 a1 = make_float2(x0.x + c1 * p1.x + c2 * p2.x + c3 * p3.x, x0.y + c1 * p1.y + c2 * p2.y + c3 * p3.y);
  float2 a2 = make_float2(x0.x + c2 * p1.x + c3 * p2.x + c1 * p3.x, x0.y + c2 * p1.y + c3 * p2.y + c1 * p3.y);
  float2 a3 = make_float2(x0.x + c3 * p1.x + c1 * p2.x + c2 * p3.x, x0.y + c3 * p1.y + c1 * p2.y + c2 * p3.y);
  float bx1 = s1 * m1.x + s2 * m2.x + s3 * m3.x, by1 = s1 * m1.y + s2 * m2.y + s3 * m3.y;
  float bx2 = s2 * m1.x - s3 * m2.x - s1 * m3.x, by2 = s2 * m1.y - s3 * m2.y - s1 * m3.y;
  float bx3 = s3 * m1.x - s1 * m2.x + s2 * m3.x, by3 = s3 * m1.y - s1 * m2.y + s2 * m3.y;
  v[0] = make_float2(x0.x + p1.x + p2.x + p3.x, x0.y + p1.y + p2.y + p3.y);
  v[1] = make_float2(a1.x - by1, a1.y + bx1);
  v[6] = make_float2(a1.x + by1, a1.y - bx1);
  v[2] = make_float2(a2.x - by2, a2.y + bx2);
  v[5] = make_float2(a2.x + by2, a2.y - bx2);
  v[3] = make_float2(a3.x - by3, a3.y + bx3);
  v[4] = make_float2(a3.x + by3, a3.y - bx3);
}

template <int DIR>
__device__ __forceinline__ void dft8(float2* v)
{
  const float h = 0.70710678118654752440f;
  // radix-2 first level
  float2 a[8];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    a[i] = cadd(v[i], v[i + 4]);
    a[i + 4] = csub(v[i], v[i + 4]);
  }
  // twiddles W8^k on the odd half: k=1: (h, DIR*h) ; k=2: DIR*i ; k=3: (-h, DIR*h)
  a[5] = cmul(a[5], make_float2(h, DIR < 0 ? -h : h));
  a[6] = rot90<DIR>(a[6]);
  a[7] = cmul(a[7], make_float2(-h, DIR < 0 ? -h : h));
  float2 e[4] = {a[0], a[1], a[2], a[3]};
  float2 o[4] = {a[4], a[5], a[6], a[7]};
  dft4<DIR>(e);
  dft4<DIR>(o);
  v[0] = e[0];
  v[2] = e[1];
  v[4] = e[2];
  v[6] = e[3];
  v[1] = o[0];
  v[3] = o[1];
  v[5] = o[2];
  v[7] = o[3];
}

// exp(DIR * 2 pi i m / 32) for a compile-time m
__device__ __forceinline__ float2 w32c(int m, int dir)
{
  constexpr float c[32] = {1.000000000e+00f, 9.807852804e-01f, 9.238795325e-01f, 8.314696123e-01f, 7.071067812e-01f, 5.555702330e-01f, 3.826834324e-01f, 1.950903220e-01f, 6.123233996e-17f, -1.950903220e-01f, -3.826834324e-01f, -5.555702330e-01f, -7.071067812e-01f, -8.314696123e-01f, -9.238795325e-01f, -9.807852804e-01f, -1.000000000e+00f, -9.807852804e-01f, -9.238795325e-01f, -8.314696123e-01f, -7.071067812e-01f, -5.555702330e-01f, -3.826834324e-01f, -1.950903220e-01f, -1.836970199e-16f, 1.950903220e-01f, 3.826834324e-01f, 5.555702330e-01f, 7.071067812e-01f, 8.314696123e-01f, 9.238795325e-01f, 9.807852804e-01f};
  constexpr float s[32] = {0.000000000e+00f, 1.950903220e-01f, 3.826834324e-01f, 5.555702330e-01f, 7.071067812e-01f, 8.314696123e-01f, 9.238795325e-01f, 9.807852804e-01f, 1.000000000e+00f, 9.807852804e-01f, 9.238795325e-01f, 8.314696123e-01f, 7.071067812e-01f, 5.555702330e-01f, 3.826834324e-01f, 1.950903220e-01f, 1.224646799e-16f, -1.950903220e-01f, -3.826834324e-01f, -5.555702330e-01f, -7.071067812e-01f, -8.314696123e-01f, -9.238795325e-01f, -9.807852804e-01f, -1.000000000e+00f, -9.807852804e-01f, -9.238795325e-01f, -8.314696123e-01f, -7.071067812e-01f, -5.555702330e-01f, -3.826834324e-01f, -1.950903220e-01f};
  return make_float2(c[m & 31], dir < 0 ? -s[m & 31] : s[m & 31]);
}

// radix 16 = 4 x 4: inner DFT4 over x[i + 4j], twiddle W16^(i k1), outer DFT4 over i
template <int DIR>
__device__ __forceinline__ void dft16(float2* v)
{
  float2 a[16];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float2 t[4] = {v[i], v[i + 4], v[i + 8], v[i + 12]};
    dft4<DIR>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) a[i * 4 + k1] = (i * k1 == 0) ? t[k1] : cmul(t[k1], w32c(2 * i * k1, DIR));
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 u[4] = {a[k1], a[4 + k1], a[8 + k1], a[12 + k1]};
    dft4<DIR>(u);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = u[k2];
  }
}

// radix 32 = 4 x 8: inner DFT8 over x[i + 4j], twiddle W32^(i k1), outer DFT4 over i
template <int DIR>
__device__ __forceinline__ void dft32(float2* v)
{
  float2 a[32];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float2 t[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) t[j] = v[i + 4 * j];
    dft8<DIR>(t);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) a[i * 8 + k1] = (i * k1 == 0) ? t[k1] : cmul(t[k1], w32c(i * k1, DIR));
  }
#pragma unroll
  for (int k1 = 0; k1 < 8; ++k1) {
    float2 u[4] = {a[k1], a[8 + k1], a[16 + k1], a[24 + k1]};
    dft4<DIR>(u);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 8 * k2] = u[k2];
  }
}

template <int R, int DIR>
__device__ __forceinline__ void dftR(float2* v)
{
  if (R == 2) dft2<DIR>(v);
  else if (R == 3) dft3<DIR>(v);
  else if (R == 4) dft4<DIR>(v);
  else if (R == 5) dft5<DIR>(v);
  else if (R == 7) dft7<DIR>(v);
  else if (R == 8) dft8<DIR>(v);
  else if (R == 16) dft16<DIR>(v);
  else if (R == 32) dft32<DIR>(v);
}

// q = t / d for t, d < 2^16 with m = floor((2^32 - 1) / d) + 1 (exact in that range)
__device__ __forceinline__ unsigned magic_of(unsigned d) { return d == 1 ? 0u : 0xFFFFFFFFu / d + 1u; }
__device__ __forceinline__ unsigned fdiv(unsigned t, unsigned d, unsigned m) { return d == 1 ? t : __umulhi(t, m); }

// One Stockham stage of radix R over nl lines, reading `src` and writing
// `dst` (ping-pong shared buffers of identical layout), then a barrier.
// Index arithmetic uses multiply-high division (all indices < 2^16).
template <int R, int DIR>
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ src, float2* __restrict__ dst, int n,
                                               int nl, int ldl, int ldi, int Ns, const float2* __restrict__ tw)
{
  const unsigned m = n / R;  // butterflies per line
  const unsigned total = m * nl;
  const int twstep = n / (Ns * R);
  const bool rows = (ldi == 1);
  const unsigned mm = magic_of(m), mnl = magic_of(nl), mns = magic_of(Ns);
  for (unsigned t = threadIdx.x; t < total; t += blockDim.x) {
    unsigned l, j;
    if (rows) {
      l = fdiv(t, m, mm);
      j = t - l * m;
    } else {
      j = fdiv(t, nl, mnl);
      l = t - j * nl;
    }
    float2 v[R];
    const float2* s = src + l * ldl;
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[(j + r * m) * ldi];
    const unsigned jq = fdiv(j, Ns, mns);
    const unsigned k = j - jq * Ns;
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = __ldg(tw + r * k * twstep);
        if (DIR > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    dftR<R, DIR>(v);
    float2* d = dst + l * ldl + (jq * Ns * R + k) * ldi;
#pragma unroll
    for (int r = 0; r < R; ++r) d[r * Ns * ldi] = v[r];
  }
  __syncthreads();
}

// Transform of nl lines held in shared buffer `a` (same layout scratch in
// `b`).  Requires the whole CTA and a barrier after the lines were filled.
// Returns the buffer that holds the result (a or b).  Unnormalised:
// DIR = -1 forward e^{-i}, +1 inverse e^{+i}.
template <int DIR>
__device__ float2* fft_lines(float2* a, float2* b, const FFTPlan& p, int nl, int ldl, int ldi)
{
  int Ns = 1;
  float2* src = a;
  float2* dst = b;
  for (int s = 0; s < p.nstages; ++s) {
    int R = p.radix[s];
    switch (R) {
      case 2: stockham_stage<2, DIR>(src, dst, p.n, nl, ldl, ldi, Ns, p.tw); break;
      case 3: stockham_stage<3, DIR>(src, dst, p.n, nl, ldl, ldi, Ns, p.tw); break;
      case 4: stockham_stage<4, DIR>(src, dst, p.n, nl, ldl, ldi, Ns, p.tw); break;
      case 5: stockham_stage<5, DIR>(src, dst, p.n, nl, ldl, ldi, Ns, p.tw); break;
      case 7: stockham_stage<7, DIR>(src, dst, p.n, nl, ldl, ldi, Ns, p.tw); break;
      case 8: stockham_stage<8, DIR>(src, dst, p.n, nl, ldl, ldi, Ns, p.tw); break;
      case 16: stockham_stage<16, DIR>(src, dst, p.n, nl, ldl, ldi, Ns, p.tw); break;
      default: stockham_stage<32, DIR>(src, dst, p.n, nl, ldl, ldi, Ns, p.tw); break;
    }
    Ns *= R;
    float2* t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// Complex elements a CTA of kFftThreads threads stages per transform.
constexpr int kFftThreads = 256;
constexpr int kFftElems = 4096;

#endif  // __CUDACC__

}  // namespace simrecon
