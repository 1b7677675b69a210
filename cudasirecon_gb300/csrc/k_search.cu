// The pattern-vector search on the device: findk0's peak refinement and
// fitk0andmodamps' line searches (gpuFunctionsImpl.cu:306-372, 874-1044)
// without a host round trip.
//
// k_findk0_finish   the cross-correlation peak's parabola fits and the
//                   wrap-around choice -> k0 (one thread)
// k_k0_search       one thread-block cluster per direction (all directions in
//                   one launch, side by side on the GPU): the angle and
//                   magnitude line searches with their parabola fits and the
//                   final modulation amplitude.  The cluster's eight CTAs
//                   evaluate batches of candidate k0s over the overlap map P
//                   (each CTA one tile of P, its partial sums written into
//                   the leader CTA's shared memory); one thread of the
//                   leader runs the sequential search between batches.
//
// The search visits the same float32 angles and magnitudes as the reference
// (float-accumulated steps from the start value) and makes its decisions
// and parabola fits with separately rounded float operations, as the
// reference's host code does.  The candidate values themselves come from the
// device's cosf/sinf/atan2f, which may differ from a host libm in the last
// bit, and the phase factors from float sincospi of an exactly reduced
// argument (the host-driven evaluation uses double sincos), so the fitted k0
// matches the host-driven search to a few 1e-5 pixel, not bit for bit.
#include <cooperative_groups.h>

#include "kernels.h"

namespace cg = cooperative_groups;

namespace simrecon {

namespace {

// fitparabola, gpuFunctionsImpl.cu:479-495
__device__ float fitparabola_rn(float a1, float a2, float a3)
{
  const float slope = __fmul_rn(0.5f, __fsub_rn(a3, a1));
  const float curve = __fsub_rn(__fadd_rn(a3, a1), __fmul_rn(2.f, a2));
  if (curve == 0.f) return 0.f;
  const float peak = __fdiv_rn(-slope, curve);
  if (peak > 1.5f || peak < -1.5f) return 0.f;
  return peak;
}

// fitxyparabola, gpuFunctionsImpl.cu:1022-1044
__device__ float fitxyparabola_rn(float x1, float y1, float x2, float y2, float x3, float y3)
{
  if (x1 == x2 || x2 == x3 || x3 == x1) return 0.f;
  const float xbar1 = __fmul_rn(0.5f, __fadd_rn(x1, x2));
  const float xbar2 = __fmul_rn(0.5f, __fadd_rn(x2, x3));
  const float slope1 = __fdiv_rn(__fsub_rn(y2, y1), __fsub_rn(x2, x1));
  const float slope2 = __fdiv_rn(__fsub_rn(y3, y2), __fsub_rn(x3, x2));
  const float curve = __fdiv_rn(__fsub_rn(slope2, slope1), __fsub_rn(xbar2, xbar1));
  if (curve == 0.f) return 0.f;
  return __fsub_rn(xbar2, __fdiv_rn(slope2, curve));
}

__device__ __forceinline__ float2 polar_rn(float mag, float angle)
{
  return make_float2(__fmul_rn(mag, cosf(angle)), __fmul_rn(mag, sinf(angle)));
}

// findk0's tail (gpuFunctionsImpl.cu:345-371): peak = {ix, iy, a1x, a2, a3x,
// a1y, a3y}; k0 = the parabola-refined peak, moved by a period towards the
// guess, over fitorder2.  k1 = k0 through (|k0|, atan2) and back: the vector
// the search's first getmodamp rebuilds the overlaps at.
__global__ void k_findk0_finish(const float* __restrict__ pk, float2 guess, int nx, int ny, float dkx, float dky,
                                int fitorder2, float2* k0out, float2* k1out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int xcent = (int)pk[0], ycent = (int)pk[1];
  float peakx = __fadd_rn(fitparabola_rn(pk[2], pk[3], pk[4]), (float)xcent);
  float peaky = __fadd_rn(fitparabola_rn(pk[5], pk[3], pk[6]), (float)ycent);
  if (__fdiv_rn(guess.x, dkx) < __fsub_rn(peakx, (float)(nx / 2))) peakx = __fsub_rn(peakx, (float)nx);
  if (__fdiv_rn(guess.x, dkx) > __fadd_rn(peakx, (float)(nx / 2))) peakx = __fadd_rn(peakx, (float)nx);
  if (__fdiv_rn(guess.y, dky) < __fsub_rn(peaky, (float)(ny / 2))) peaky = __fsub_rn(peaky, (float)ny);
  if (__fdiv_rn(guess.y, dky) > __fadd_rn(peaky, (float)(ny / 2))) peaky = __fadd_rn(peaky, (float)ny);
  const float2 k0 = make_float2(__fmul_rn(peakx, __fdiv_rn(dkx, (float)fitorder2)),
                                __fmul_rn(peaky, __fdiv_rn(dky, (float)fitorder2)));
  *k0out = k0;
  const float mag = __fsqrt_rn(__fadd_rn(__fmul_rn(k0.x, k0.x), __fmul_rn(k0.y, k0.y)));
  *k1out = polar_rn(mag, atan2f(k0.y, k0.x));
}

constexpr int kSC = 8;        // CTAs per cluster: one direction's search
constexpr int kST = 512;      // threads per CTA
constexpr int kSW = kST / 32;
constexpr int kSB = 32;       // candidates per batch at most
constexpr int kSL = 1024;     // line cache: steps -kSL..kSL from the start value
constexpr int kSLine0 = 12;   // first batch of a line: the start and 12 steps each way
constexpr int kSLineK = 16;   // later batches: 16 steps further along the climb
// every batch but the two line starts and the final evaluation extends a
// climb by kSLineK steps, so this bounds the batches of a search
constexpr int kSMaxBatches = 2 * (2 * kSL / kSLineK + 2) + 4;

enum : int { kPhaseAngle = 0, kPhaseMag = 1, kPhaseFinal = 2, kPhaseDone = 3 };

struct SearchLine {
  float val[2 * kSL + 1];  // |modamp|^2 at step j (index j + kSL)
  float pos[2 * kSL + 1];  // the angle or magnitude at step j
  unsigned char have[2 * kSL + 1];
};

struct __align__(16) SearchCtl {
  int nbatch;                // candidates of the current batch; 0: finished
  int vary_angle;            // 1: pos[] are angles at magnitude `fixed`; 0: magnitudes at angle `fixed`
  float fixed;
  int pad;
  float pos[kSB];            // the batch's positions along its line
  int j[kSB];                // their line steps
  float2 kc[kSB];            // candidate vectors k1 * fitorder2
  double red[kSC][kSB][2];   // every CTA's partial XStarY (leader only)
  double res[kSB][2];        // the batch's XStarY (leader only)
};

struct ClimbResult {
  int need;   // 1: step `j` is not evaluated yet
  int j;
  float fit;  // fitxyparabola of the last three points
  float x1, amp1;
};

// One line search of fitk0andmodamps (gpuFunctionsImpl.cu:902-942 for the
// angle, 944-985 for the magnitude), replayed from the line's cached values;
// x1 / amp1 carry over from the previous line as in the reference (declared
// once, not reset between the two searches).
__device__ ClimbResult run_climb(const SearchLine& L, float x1, float amp1)
{
  ClimbResult r{0, 0, 0.f, x1, amp1};
  auto has = [&](int j) { return j >= -kSL && j <= kSL && L.have[j + kSL]; };
  if (!has(0)) return ClimbResult{1, 0, 0.f, x1, amp1};
  if (!has(1)) return ClimbResult{1, 1, 0.f, x1, amp1};
  float x2 = L.pos[kSL], amp2 = L.val[kSL];
  float x3 = L.pos[kSL + 1], amp3 = L.val[kSL + 1];
  int steps = 0;
  if (amp3 > amp2) {
    int j = 1;
    while (amp3 > amp2 && steps < kMaxClimbSteps) {
      amp1 = amp2;
      x1 = x2;
      amp2 = amp3;
      x2 = x3;
      ++j;
      ++steps;
      if (!has(j)) return ClimbResult{1, j, 0.f, x1, amp1};
      x3 = L.pos[j + kSL];
      amp3 = L.val[j + kSL];
    }
  } else {
    float a = amp3;
    amp3 = amp2;
    amp2 = a;
    a = x3;
    x3 = x2;
    x2 = a;
    int j = 0;
    while (amp3 > amp2 && steps < kMaxClimbSteps) {
      amp1 = amp2;
      x1 = x2;
      amp2 = amp3;
      x2 = x3;
      --j;
      ++steps;
      if (!has(j)) return ClimbResult{1, j, 0.f, x1, amp1};
      x3 = L.pos[j + kSL];
      amp3 = L.val[j + kSL];
    }
  }
  r.fit = fitxyparabola_rn(x1, amp1, x2, amp2, x3, amp3);
  r.x1 = x1;
  r.amp1 = amp1;
  return r;
}

// Leader state, held by thread 0 of CTA 0 across batches
struct Controller {
  int phase;
  int status;
  int ncand;           // candidates evaluated
  float k0mag, k0angle, delta_angle, delta_mag;
  float afit, mfit;    // fitted angle, magnitude
  float x1, amp1;      // carried between the lines
  float sx;            // sum |X|^2 as float
};

// position of step j from its neighbour towards the start (float-accumulated
// like the reference's angle += deltaangle)
__device__ void set_pos(SearchLine& L, int j, float base, float delta)
{
  if (j == 0) L.pos[kSL] = base;
  else if (j > 0) L.pos[j + kSL] = __fadd_rn(L.pos[j - 1 + kSL], delta);
  else L.pos[j + kSL] = __fsub_rn(L.pos[j + 1 + kSL], delta);
}

// queue steps j, j+s, ... (or the start batch) of the current line; the
// candidate vectors are formed by the leader's threads in parallel
__device__ void request_line(const Controller& c, SearchLine& L, SearchCtl& ctl, int j)
{
  const bool ang = c.phase == kPhaseAngle;
  const float base = ang ? c.k0angle : c.k0mag;
  const float delta = ang ? c.delta_angle : c.delta_mag;
  int n = 0;
  auto add = [&](int jj) {
    if (jj < -kSL || jj > kSL || L.have[jj + kSL]) return;
    set_pos(L, jj, base, delta);
    ctl.pos[n] = L.pos[jj + kSL];
    ctl.j[n] = jj;
    ++n;
  };
  if (j == 0 || j == 1) {
    add(0);
    for (int i = 1; i <= kSLine0; ++i) add(i);
    for (int i = 1; i <= kSLine0; ++i) add(-i);
  } else {
    const int s = j > 0 ? 1 : -1;
    for (int i = 0; i < kSLineK; ++i) add(j + s * i);
  }
  ctl.vary_angle = ang;
  ctl.fixed = ang ? c.k0mag : c.afit;
  ctl.nbatch = n;
}

// Consume the finished batch, advance the search, queue the next batch (or
// none).  Runs on one thread; lines[0] is the angle line, lines[1] the
// magnitude line.
__device__ void control(Controller& c, SearchLine* lines, SearchCtl& ctl, const K0SearchArgs& a, int dir)
{
  const int nb = ctl.nbatch;
  if (c.phase == kPhaseFinal && nb > 0) {
    // getmodamp at the fitted (angle, magnitude): the amplitude of fitorder2
    double* slot = a.slot[dir];
    slot[0] = ctl.res[0][0];
    slot[1] = ctl.res[0][1];
    slot[2] = a.sumxy[dir][0];
    slot[3] = a.sumxy[dir][1];
    *a.k0fit[dir] = polar_rn(c.mfit, c.afit);
    c.phase = kPhaseDone;
    ctl.nbatch = 0;
    return;
  }
  if (nb > 0) {
    SearchLine& L = lines[c.phase == kPhaseAngle ? 0 : 1];
    for (int i = 0; i < nb; ++i) {
      const float mx = __fdiv_rn(__double2float_rn(ctl.res[i][0]), c.sx);
      const float my = __fdiv_rn(__double2float_rn(ctl.res[i][1]), c.sx);
      L.val[ctl.j[i] + kSL] = __fadd_rn(__fmul_rn(mx, mx), __fmul_rn(my, my));
      L.have[ctl.j[i] + kSL] = 1;
    }
  }
  ctl.nbatch = 0;
  while (c.phase == kPhaseAngle || c.phase == kPhaseMag) {
    SearchLine& L = lines[c.phase == kPhaseAngle ? 0 : 1];
    const ClimbResult r = run_climb(L, c.x1, c.amp1);
    if (r.need) {
      if (r.j < -kSL || r.j > kSL) {  // beyond the line cache: the host search takes over
        c.status = 1;
        c.phase = kPhaseDone;
        return;
      }
      request_line(c, L, ctl, r.j);
      return;
    }
    c.x1 = r.x1;
    c.amp1 = r.amp1;
    if (c.phase == kPhaseAngle) {
      c.afit = r.fit;
      c.phase = kPhaseMag;
      continue;
    }
    c.mfit = r.fit;
    c.phase = kPhaseFinal;
    ctl.pos[0] = c.mfit;
    ctl.j[0] = 0;
    ctl.vary_angle = 0;
    ctl.fixed = c.afit;
    ctl.nbatch = 1;
  }
}

// Phase factor e^{i 2 pi m k dxy} for m = x - n/2 (an integer or a half
// integer, exact in float): m * (k dxy) split into a float product, its exact
// rounding error (fmaf) and the low part of k dxy, reduced to [-1/2, 1/2]
// turns before sincospif -- a phase error of a few 1e-7 rad at any m.
__device__ __forceinline__ float2 phase_factor(int x, int n, float hi, float lo)
{
  const float fm = 0.5f * (float)(2 * x - n);
  const float p = fm * hi;
  const float e = fmaf(fm, hi, -p);
  const float t = fmaf(fm, lo, e);
  const float r = (p - rintf(p)) + t;
  float s, c;
  sincospif(2.f * r, &s, &c);
  return make_float2(c, s);
}

// XStarY partial sums of CC candidates over this CTA's tile: per row the x
// sum with the x phase factors, times the row's y factor; two rows per pass
// share the x factors.  acc: per-thread sums.
template <int CC>
__device__ __forceinline__ void tile_sums(const float2* __restrict__ pmap, int nx, const float2* ex, const float2* ey,
                                          int tw, int th, int x0, int y0, int warp, int lane, float2 (&acc)[CC])
{
#pragma unroll
  for (int k = 0; k < CC; ++k) acc[k] = make_float2(0.f, 0.f);
  const int y1 = y0 + th, x1 = x0 + tw;
  for (int y = y0 + 2 * warp; y < y1; y += 2 * kSW) {
    const bool two = y + 1 < y1;
    float2 r0[CC], r1[CC];
#pragma unroll
    for (int k = 0; k < CC; ++k) r0[k] = r1[k] = make_float2(0.f, 0.f);
    for (int x = x0 + lane; x < x1; x += 32) {
      const float2 p0 = __ldg(pmap + (size_t)y * nx + x);
      const float2 p1 = two ? __ldg(pmap + (size_t)(y + 1) * nx + x) : make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < CC; ++k) {
        const float2 e = ex[k * tw + (x - x0)];
        r0[k].x = fmaf(p0.x, e.x, fmaf(-p0.y, e.y, r0[k].x));
        r0[k].y = fmaf(p0.x, e.y, fmaf(p0.y, e.x, r0[k].y));
        r1[k].x = fmaf(p1.x, e.x, fmaf(-p1.y, e.y, r1[k].x));
        r1[k].y = fmaf(p1.x, e.y, fmaf(p1.y, e.x, r1[k].y));
      }
    }
#pragma unroll
    for (int k = 0; k < CC; ++k) {
      const float2 e0 = ey[k * th + (y - y0)];
      acc[k].x += r0[k].x * e0.x - r0[k].y * e0.y;
      acc[k].y += r0[k].x * e0.y + r0[k].y * e0.x;
      if (two) {
        const float2 e1 = ey[k * th + (y + 1 - y0)];
        acc[k].x += r1[k].x * e1.x - r1[k].y * e1.y;
        acc[k].y += r1[k].x * e1.y + r1[k].y * e1.x;
      }
    }
  }
}

// the CTA's sums of CC candidates in double (warps by shuffles, then the
// warps in order) into the leader's partial-sum table at candidate c0
template <int CC>
__device__ __forceinline__ void tile_reduce(const float2 (&acc)[CC], double (*wsum)[2 * 16], SearchCtl* lead,
                                            int rank, int c0, int tid, int warp, int lane)
{
#pragma unroll
  for (int k = 0; k < CC; ++k) {
    double sr = acc[k].x, si = acc[k].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
      wsum[warp][2 * k] = sr;
      wsum[warp][2 * k + 1] = si;
    }
  }
  __syncthreads();
  if (tid < 2 * CC) {
    double s = 0.0;
    for (int w = 0; w < kSW; ++w) s += wsum[w][tid];
    lead->red[rank][c0 + (tid >> 1)][tid & 1] = s;
  }
}

template <int CC>
__device__ void chunk(const float2* __restrict__ pmap, int nx, const float2* ex, const float2* ey, int tw, int th,
                      int x0, int y0, double (*wsum)[2 * 16], SearchCtl* lead, int rank, int c0)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float2 acc[CC];
  tile_sums<CC>(pmap, nx, ex, ey, tw, th, x0, y0, warp, lane, acc);
  tile_reduce<CC>(acc, wsum, lead, rank, c0, tid, warp, lane);
}

// C: the most candidates one pass holds (phase tables in shared memory)
template <int C>
__global__ void __cluster_dims__(kSC, 1, 1) __launch_bounds__(kST, 1) k_k0_search(const __grid_constant__ K0SearchArgs a)
{
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const int dir = blockIdx.x / kSC;  // one cluster per direction
  const float2* __restrict__ pmap = a.pmap[dir];
  __shared__ SearchCtl ctl;
  __shared__ SearchLine lines[2];
  __shared__ double wsum[kSW][2 * 16];
  __shared__ float2 kloc[kSB];
  __shared__ float2 khl[kSB][2];  // k dxy of each candidate and axis as hi + lo floats
  __shared__ int nloc;
  extern __shared__ float2 tab[];
  SearchCtl* lead = cluster.map_shared_rank(&ctl, 0);
  const int tid = threadIdx.x;
  const int nx = a.nx, ny = a.ny;
  // tile of P: 2 column halves x 4 row quarters
  const int tx = rank & 1, ty = rank >> 1;
  const int x0 = tx * nx / 2, x1 = (tx + 1) * nx / 2;
  const int y0 = ty * ny / 4, y1 = (ty + 1) * ny / 4;
  const int tw = x1 - x0, th = y1 - y0;

  Controller c{};
  if (rank == 0) {
    for (int i = tid; i < 2 * kSL + 1; i += kST) lines[0].have[i] = lines[1].have[i] = 0;
    if (tid == 0) {
      const float2 k0 = *a.k0find[dir];
      c.phase = kPhaseAngle;
      c.k0mag = __fsqrt_rn(__fadd_rn(__fmul_rn(k0.x, k0.x), __fmul_rn(k0.y, k0.y)));
      c.k0angle = atan2f(k0.y, k0.x);
      c.delta_angle = a.delta_angle;
      c.delta_mag = a.delta_mag;
      c.sx = __double2float_rn(a.sumxy[dir][0]);
      ctl.nbatch = 0;
    }
  }
  const float fac = (float)a.fitorder2;
  int it = 0;
  for (; it < kSMaxBatches; ++it) {
    if (rank == 0) {
      __syncthreads();  // the previous batch's sums are in ctl.res; the line caches are clear
      if (tid == 0) {
        control(c, lines, ctl, a, dir);
        c.ncand += ctl.nbatch;
      }
      __syncthreads();
      // the candidate vectors (getmodamp: k1 = mag (cosf, sinf)(angle), times fitorder2 - fitorder1)
      if (tid < ctl.nbatch) {
        const float2 k1 = ctl.vary_angle ? polar_rn(ctl.fixed, ctl.pos[tid]) : polar_rn(ctl.pos[tid], ctl.fixed);
        ctl.kc[tid] = make_float2(__fmul_rn(k1.x, fac), __fmul_rn(k1.y, fac));
      }
    }
    cluster.sync();  // the batch (or the end) is visible to every CTA
    if (tid == 0) nloc = lead->nbatch;
    if (tid < kSB) kloc[tid] = lead->kc[tid];
    __syncthreads();
    const int nb = nloc;
    if (nb == 0) break;
    if (tid < 2 * nb) {  // the double products once per candidate and axis (FP64 is slow on this GPU)
      const float2 kk = kloc[tid >> 1];
      const double kd = (double)((tid & 1) ? kk.y : kk.x) * (double)a.dxy;
      const float hi = (float)kd;
      khl[tid >> 1][tid & 1] = make_float2(hi, (float)(kd - (double)hi));
    }
    __syncthreads();
    for (int c0 = 0; c0 < nb;) {
      const int rem = nb - c0;
      const int cc = rem >= 16 && C >= 16 ? 16 : rem >= 8 && C >= 8 ? 8 : rem >= 4 ? 4 : rem >= 2 ? 2 : 1;
      float2* ex = tab;                    // [cc][tw]
      float2* ey = tab + (size_t)cc * tw;  // [cc][th]
      for (int e = tid; e < cc * (tw + th); e += kST) {
        const int k = e / (tw + th), r = e - k * (tw + th);
        const bool isx = r < tw;
        const float2 hl = khl[c0 + k][isx ? 0 : 1];
        if (isx) ex[k * tw + r] = phase_factor(x0 + r, nx, hl.x, hl.y);
        else ey[k * th + (r - tw)] = phase_factor(y0 + (r - tw), ny, hl.x, hl.y);
      }
      __syncthreads();
      if (cc == 16) chunk<16>(pmap, nx, ex, ey, tw, th, x0, y0, wsum, lead, rank, c0);
      else if (cc == 8) chunk<8>(pmap, nx, ex, ey, tw, th, x0, y0, wsum, lead, rank, c0);
      else if (cc == 4) chunk<4>(pmap, nx, ex, ey, tw, th, x0, y0, wsum, lead, rank, c0);
      else if (cc == 2) chunk<2>(pmap, nx, ex, ey, tw, th, x0, y0, wsum, lead, rank, c0);
      else chunk<1>(pmap, nx, ex, ey, tw, th, x0, y0, wsum, lead, rank, c0);
      __syncthreads();  // tables and wsum are reused by the next chunk
      c0 += cc;
    }
    cluster.sync();  // every CTA's partial sums are in the leader
    if (rank == 0 && tid < 2 * nb) {
      double s = 0.0;
      for (int r = 0; r < kSC; ++r) s += ctl.red[r][tid >> 1][tid & 1];
      ctl.res[tid >> 1][tid & 1] = s;
    }
  }
  // no CTA leaves while another may still read the leader's shared memory
  cluster.sync();
  if (rank == 0 && tid == 0) {
    if (c.phase != kPhaseDone && c.status == 0) c.status = 2;  // batch limit reached
    atomicAdd(a.info, c.ncand);
    if (c.status) atomicOr(a.info + 1, c.status);
  }
}

}  // namespace

int launch_findk0_finish(const float* peak, float2 guess, int nx, int ny, float dkx, float dky, int fitorder2,
                         float2* k0out, float2* k1out, cudaStream_t s, long long* launches)
{
  k_findk0_finish<<<1, 32, 0, s>>>(peak, guess, nx, ny, dkx, dky, fitorder2, k0out, k1out);
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

// candidates per chunk: the phase tables of a tile (C x (tw + th) complex)
// within 160 KB of shared memory
static int search_chunk(int nx, int ny)
{
  const size_t per = ((size_t)(nx + 1) / 2 + (size_t)(ny + 3) / 4) * sizeof(float2);
  for (int c : {16, 8, 4})
    if (c * per <= 160 * 1024) return c;
  return 0;
}

// Up to 1024^2 maps (a tile of at most 512 x 256 per CTA).  Larger maps
// take the host-driven search, whose candidate batches run on every SM: one
// cluster per direction would spend milliseconds per batch on a 1024 x 512
// tile.
bool k0_search_supported(int nx, int ny)
{
  return nx >= 64 && ny >= 8 && (long long)nx * ny <= 1024LL * 1024 && search_chunk(nx, ny) > 0;
}

int launch_k0_search(const K0SearchArgs& a, cudaStream_t s, long long* launches)
{
  const int C = search_chunk(a.nx, a.ny);
  if (C == 0 || a.nx < 64 || a.ny < 8 || a.ndirs < 1 || a.ndirs > kMaxDirs) return -1;
  const size_t tw = (size_t)(a.nx + 1) / 2, th = (size_t)(a.ny + 3) / 4;
  const size_t smem = (size_t)C * (tw + th) * sizeof(float2);
  auto go = [&](auto kern) {
    // raised only (under a lock): handles of other shapes launch concurrently
    allow_dynamic_smem((const void*)kern, smem);
    kern<<<kSC * a.ndirs, kST, smem, s>>>(a);
  };
  KernelTimer* kt = kernel_timer();
  if (kt) kt->begin(s);
  if (C == 16) go(k_k0_search<16>);
  else if (C == 8) go(k_k0_search<8>);
  else go(k_k0_search<4>);
  if (kt) kt->end("k_k0_search", s, (double)a.ndirs * a.nx * a.ny * sizeof(float2));
  if (launches) *launches += 1;
  return (int)cudaGetLastError();
}

}  // namespace simrecon
