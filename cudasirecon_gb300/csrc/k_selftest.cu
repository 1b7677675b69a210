// FFT-engine self test: transforms `nl` lines of length n through the same
// shared-memory Stockham path the reconstruction kernels use, in either the
// rows or the columns layout, so tests can compare it with a reference FFT.
#include <algorithm>
#include <mutex>

#include "cudasirecon.h"
#include "kernels.h"
#include "reg_fft.cuh"

namespace simrecon {

namespace {
template <int DIR, int NF>
__global__ void k_fft_selftest(float2* data, int n, int nl, int columns, FFTPlan plan)
{
  extern __shared__ float2 sm[];
  float2* base = data + (size_t)blockIdx.x * nl * n;
  const int ldc = nl + 1, ldr = n + 1;  // odd pitches, as the reconstruction kernels use
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    int l = t / n, i = t - l * n;
    sm[columns ? i * ldc + l : l * ldr + i] = base[t];
  }
  __syncthreads();
  const int elems = columns ? n * ldc : nl * ldr;
  const float2* res = columns ? fft_dispatch<NF, DIR>(sm, sm + elems, plan, nl, 1, ldc)
                              : fft_dispatch<NF, DIR>(sm, sm + elems, plan, nl, ldr, 1);
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    int l = t / n, i = t - l * n;
    base[t] = res[columns ? i * ldc + l : l * ldr + i];
  }
}
size_t selftest_smem(int n, int nl, int columns)
{
  int elems = columns ? n * (nl + 1) : nl * (n + 1);
  return fft_stage_smem(n, nl, elems, kFftThreads);
}
}  // namespace

int launch_fft_selftest(float2* data, int n, int nlines, int inverse, int columns, cudaStream_t s)
{
  FFTPlan p;
  if (!get_fft_plan(n, &p)) return -1;
  int nl = std::max(1, std::min(nlines, kFftElems / (n + 1)));
  while (nlines % nl) --nl;
  size_t sm = selftest_smem(n, nl, columns);
  dispatch_fft_len(kSiteSelfTest, n, [&]<int NF>() {
    if (inverse) {
      allow_dynamic_smem((const void*)k_fft_selftest<+1, NF>, sm);
      k_fft_selftest<+1, NF><<<nlines / nl, kFftThreads, sm, s>>>(data, n, nl, columns, p);
    } else {
      allow_dynamic_smem((const void*)k_fft_selftest<-1, NF>, sm);
      k_fft_selftest<-1, NF><<<nlines / nl, kFftThreads, sm, s>>>(data, n, nl, columns, p);
    }
  });
  return (int)cudaGetLastError();
}

}  // namespace simrecon

// ---------------------------------------------------------------------------
// Allocation-free FFT entry point (SRX_fftLinesNoAlloc).
//
// Some callers of this library cannot call cudaMalloc: real-time acquisition
// loops in microscope control software, where an allocation's implicit device
// synchronisation would stall the camera pipeline, and plug-in hosts (for
// example a JVM image-analysis application driving this library over JNI)
// that own the device and forbid allocations outside their own memory pool.
// For them this entry point transforms lines with the same kernel as
// SRX_fftSelfTest but keeps its device staging buffer and its twiddle table in
// the file-scope array below instead of allocating them.
//
// Limits and contract:
//  * a synchronous host-to-host call: the input is copied from host memory,
//    transformed and copied back with blocking copies and launches on the
//    calling thread's default stream; the call returns when the result is in
//    `out`;
//  * at most kNoAllocMaxElems complex values (4 Mi floats, 16 MiB of
//    staging) per call and line lengths up to kNoAllocMaxN; in the column
//    layout a line must also fit the per-CTA shared-memory limit (lengths up
//    to 7264 with GB300's 227 KB).  Larger requests are rejected with an
//    error; nothing is transformed and `out` is not written;
//  * the array lives in every GPU that loads this library, for the life of
//    the process, whether or not the entry point is used;
//  * all calls share the array: calls whose work overlaps on the GPU (from
//    different host threads, or on a device where another call has not
//    finished) race and corrupt each other's results.  Each call finishes
//    its device work before returning, so calls made one after another from
//    one thread are safe.  The twiddle table is rewritten on every call and
//    the staging area is fully overwritten by the call's input, so no state
//    carries over from the previous call;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture begins.
// ---------------------------------------------------------------------------

namespace simrecon {
namespace {

constexpr size_t kNoAllocMaxElems = (size_t)1 << 21;  // complex values per call
constexpr int kNoAllocMaxN = 8192;                    // longest line

// [0, kNoAllocMaxN): twiddles; [kNoAllocMaxN, 2 kNoAllocMaxN): the same
// twiddles in the register path's lane-major order; then the staging area
static __device__ __align__(256) float2 g_noalloc_scratch[2 * kNoAllocMaxN + kNoAllocMaxElems];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
float2* g_noalloc_addr[kMaxDevices] = {nullptr};

// one-time (per device) lookup of the array's device address
cudaError_t noalloc_scratch(int dev, float2** out)
{
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = (float2*)p;
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

// tw[k] = exp(-2 pi i k / n), computed in double precision on the device;
// with P register-path lanes (P > 0) also twr[(k1-1)*P + q] = tw[q*k1 mod n]
// for k1 < n/P (FFTPlan::twr), each entry from the same formula as tw
__device__ __forceinline__ float2 noalloc_twiddle(int k, int n)
{
  double s, c;
  sincospi(-2.0 * (double)k / (double)n, &s, &c);
  return make_float2((float)c, (float)s);
}
__global__ void k_noalloc_twiddles(float2* tw, float2* twr, int n, int P)
{
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    tw[k] = noalloc_twiddle(k, n);
    if (P > 0 && k < n - P) {
      const int k1 = k / P + 1, q = k % P;
      twr[k] = noalloc_twiddle((int)(((long long)q * k1) % n), n);
    }
  }
}

thread_local char t_noalloc_err[256];

int noalloc_fail(const char* msg, cudaError_t e = cudaSuccess)
{
  if (e != cudaSuccess) snprintf(t_noalloc_err, sizeof(t_noalloc_err), "%s: %s", msg, cudaGetErrorString(e));
  else snprintf(t_noalloc_err, sizeof(t_noalloc_err), "%s", msg);
  return -1;
}

}  // namespace

}  // namespace simrecon

extern "C" int SRX_fftLinesNoAlloc(const float* in, float* out, int n, int nlines, int inverse, int columns)
{
  using namespace simrecon;
  t_noalloc_err[0] = '\0';
  if (!in || !out || n < 1 || nlines < 1) return noalloc_fail("SRX_fftLinesNoAlloc: invalid arguments");
  if (n > kNoAllocMaxN || (size_t)n * (size_t)nlines > kNoAllocMaxElems)
    return noalloc_fail("SRX_fftLinesNoAlloc: request exceeds the 2 Mi complex-value (16 MiB) staging limit or "
                        "the 8192-point line limit");
  FFTPlan p{};
  p.n = n;
  if (!fft_radix_plan(n, p.radix, &p.nstages))
    return noalloc_fail("SRX_fftLinesNoAlloc: line length must factor into 2, 3, 5 and 7");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail("SRX_fftLinesNoAlloc: cudaGetDevice", e);
  float2* base = nullptr;
  e = noalloc_scratch(dev, &base);
  if (e != cudaSuccess) return noalloc_fail("SRX_fftLinesNoAlloc: cudaGetSymbolAddress", e);
  float2* tw = base;
  float2* twr = base + kNoAllocMaxN;
  float2* data = base + 2 * kNoAllocMaxN;
  const int P = reg_fft_lanes(n);
  p.tw = tw;
  p.twr = P ? twr : nullptr;
  const size_t bytes = (size_t)n * nlines * sizeof(float2);
  int nl = std::max(1, std::min(nlines, kFftElems / (n + 1)));
  while (nlines % nl) --nl;
  size_t sm = selftest_smem(n, nl, columns);
  int smem_max = 0;
  e = cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return noalloc_fail("SRX_fftLinesNoAlloc: cudaDeviceGetAttribute", e);
  if (sm > (size_t)smem_max)
    return noalloc_fail("SRX_fftLinesNoAlloc: line too long for the column layout (the per-CTA shared-memory "
                        "limit is exceeded); use the row layout");
  k_noalloc_twiddles<<<(n + 255) / 256, 256>>>(tw, twr, n, P);
  e = cudaMemcpy(data, in, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return noalloc_fail("SRX_fftLinesNoAlloc: input copy", e);
  dispatch_fft_len(kSiteSelfTest, n, [&]<int NF>() {
    if (inverse) {
      allow_dynamic_smem((const void*)k_fft_selftest<+1, NF>, sm);
      k_fft_selftest<+1, NF><<<nlines / nl, kFftThreads, sm>>>(data, n, nl, columns, p);
    } else {
      allow_dynamic_smem((const void*)k_fft_selftest<-1, NF>, sm);
      k_fft_selftest<-1, NF><<<nlines / nl, kFftThreads, sm>>>(data, n, nl, columns, p);
    }
  });
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail("SRX_fftLinesNoAlloc: launch", e);
  e = cudaMemcpy(out, data, bytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return noalloc_fail("SRX_fftLinesNoAlloc: output copy", e);
  return 0;
}

extern "C" const char* SRX_fftLinesNoAllocError(void) { return simrecon::t_noalloc_err; }
