// Four-step transform of W adjacent columns of length N = R1 * R2, for the
// y transforms of row-major planes.
//
// Stage 1: the thread for (column c, j < R2) loads x[j + R2*e] (e < R1) of its
// column straight from global memory -- adjacent threads read adjacent
// columns, so every load instruction reads whole row segments -- runs an
// in-register DFT of R1 points, multiplies by W_N^(j*k1) and stores the R1
// results to shared memory.  After one CTA barrier, stage 2: the thread for
// (c, k1 < R1) reads the R2 values over j, runs an in-register DFT of R2
// points and hands X[k1 + R1*k2] (k2 < R2) to the caller's store.
//
//   X[k1 + R1 k2] = sum_j W_N^(j k1) W_R2^(j k2) sum_e x[j + R2 e] W_R1^(e k1)
//
// Shared layout: element (k1, j, c) at k1*LD1 + j*W + c with LD1 = R2*W + 8,
// so 2*LD1 is 16 mod 32 words: the stage-1 stores of a warp are contiguous
// and the stage-2 reads of each half-warp hit distinct banks.
#pragma once
#include "reg_fft.cuh"

namespace simrecon {

#ifdef __CUDACC__

template <int N, int R1, int W>
struct ColFft {
  static constexpr int R2 = N / R1;
  static constexpr int LD1 = R2 * W + 8;
  static constexpr int kSmemElems = R1 * LD1;  // float2 elements of shared memory
  static_assert(N % R1 == 0, "R1 must divide N");
  static_assert(W == 8, "the bank-conflict-free layout assumes 8 columns per CTA");
};

// Stage 1 for every (c, j) item of the CTA; load(row, c) -> float2 (0 outside
// the data).  tw: table of N twiddles exp(-2 pi i k / N).  Ends with a CTA
// barrier.
template <int N, int R1, int W, int DIR, class Load>
__device__ __forceinline__ void colfft_stage1(float2* sm, const float2* __restrict__ tw, Load&& load)
{
  using C = ColFft<N, R1, W>;
  constexpr int R2 = C::R2;
  for (int it = threadIdx.x; it < R2 * W; it += blockDim.x) {
    const int c = it % W, j = it / W;
    float2 v[R1];
#pragma unroll
    for (int e = 0; e < R1; ++e) v[e] = load(j + R2 * e, c);
    reg_dft<R1, DIR>(v);
#pragma unroll
    for (int k1 = 1; k1 < R1; ++k1) {
      float2 w = __ldg(tw + j * k1);
      if (DIR > 0) w.y = -w.y;
      v[k1] = cmul(v[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) sm[k1 * C::LD1 + j * W + c] = v[k1];
  }
  __syncthreads();
}

// Stage 2 for every (c, k1) item; store(row, c, value) for row = k1 + R1*k2.
template <int N, int R1, int W, int DIR, class Store>
__device__ __forceinline__ void colfft_stage2(const float2* sm, Store&& store)
{
  using C = ColFft<N, R1, W>;
  constexpr int R2 = C::R2;
  for (int it = threadIdx.x; it < R1 * W; it += blockDim.x) {
    const int c = it % W, k1 = it / W;
    float2 u[R2];
#pragma unroll
    for (int j = 0; j < R2; ++j) u[j] = sm[k1 * C::LD1 + j * W + c];
    reg_dft<R2, DIR>(u);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) store(k1 + R1 * k2, c, u[k2]);
  }
}

#endif  // __CUDACC__

// Column-transform configuration per length: R1 (0: none)
__host__ __device__ constexpr int colfft_r1(int n) { return n == 1024 ? 32 : n == 512 ? 16 : n == 256 ? 16 : 0; }

}  // namespace simrecon
