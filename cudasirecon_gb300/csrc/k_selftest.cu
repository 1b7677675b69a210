// FFT-engine self test: transforms `nl` lines of length n through the same
// shared-memory Stockham path the reconstruction kernels use, in either the
// rows or the columns layout, so tests can compare it with a reference FFT.
#include <algorithm>

#include "kernels.h"

namespace simrecon {

namespace {
template <int DIR>
__global__ void k_fft_selftest(float2* data, int n, int nl, int columns, FFTPlan plan)
{
  extern __shared__ float2 sm[];
  float2* base = data + (size_t)blockIdx.x * nl * n;
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    int l = t / n, i = t - l * n;
    sm[columns ? i * nl + l : t] = base[t];
  }
  __syncthreads();
  const float2* res = columns ? fft_lines<DIR>(sm, sm + nl * n, plan, nl, 1, nl)
                              : fft_lines<DIR>(sm, sm + nl * n, plan, nl, n, 1);
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    int l = t / n, i = t - l * n;
    base[t] = res[columns ? i * nl + l : t];
  }
}
}  // namespace

int launch_fft_selftest(float2* data, int n, int nlines, int inverse, int columns, cudaStream_t s)
{
  FFTPlan p;
  if (!get_fft_plan(n, &p)) return -1;
  int nl = std::max(1, std::min(nlines, kFftElems / n));
  while (nlines % nl) --nl;
  size_t sm = (size_t)2 * nl * n * sizeof(float2);
  if (inverse) {
    cudaFuncSetAttribute(k_fft_selftest<+1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_selftest<+1><<<nlines / nl, kFftThreads, sm, s>>>(data, n, nl, columns, p);
  } else {
    cudaFuncSetAttribute(k_fft_selftest<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_fft_selftest<-1><<<nlines / nl, kFftThreads, sm, s>>>(data, n, nl, columns, p);
  }
  return (int)cudaGetLastError();
}

}  // namespace simrecon

