// FFT plans: radix sequences and double-precision twiddle tables, cached per
// (device, length).  The tables are allocated once per length and live until
// process exit.
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "kernels.h"
#include "reg_fft.cuh"

namespace simrecon {

namespace {
std::mutex g_mu;
std::map<std::pair<int, int>, FFTPlan> g_plans;

bool factor(int n, std::vector<int>& radix)
{
  radix.clear();
  if (n < 1) return false;
  int m = n;
  int p2 = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++p2;
  }
  // powers of two in as few stages as possible: radix 32 / 16 / 8 / 4 / 2
  // (e.g. 1024 = 32*32, 512 = 32*16, 256 = 16*16, 128 = 16*8, 64 = 8*8)
  static const int plan2[14][3] = {{0, 0, 0},  {2, 0, 0},   {4, 0, 0},   {8, 0, 0},   {16, 0, 0},
                                   {32, 0, 0}, {8, 8, 0},   {16, 8, 0},  {16, 16, 0}, {32, 16, 0},
                                   {32, 32, 0}, {16, 16, 8}, {16, 16, 16}, {32, 16, 16}};
  if (p2 > 13) return false;
  for (int i = 0; i < 3; ++i)
    if (plan2[p2][i]) radix.push_back(plan2[p2][i]);
  for (int r : {3, 5, 7})
    while (m % r == 0) {
      m /= r;
      radix.push_back(r);
    }
  if (m != 1) return false;
  if ((int)radix.size() > kMaxStages) return false;
  return true;
}
}  // namespace

namespace {
thread_local KernelTimer* t_timer = nullptr;
}
void set_kernel_timer(KernelTimer* t) { t_timer = t; }
KernelTimer* kernel_timer() { return t_timer; }

// The radix sequence of get_fft_plan, written into a caller array without
// any allocation (used by the allocation-free FFT entry point).
bool fft_radix_plan(int n, int* radix, int* nstages)
{
  if (n < 1) return false;
  int m = n, p2 = 0, ns = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++p2;
  }
  static const int plan2[14][3] = {{0, 0, 0},  {2, 0, 0},   {4, 0, 0},   {8, 0, 0},   {16, 0, 0},
                                   {32, 0, 0}, {8, 8, 0},   {16, 8, 0},  {16, 16, 0}, {32, 16, 0},
                                   {32, 32, 0}, {16, 16, 8}, {16, 16, 16}, {32, 16, 16}};
  if (p2 > 13) return false;
  for (int i = 0; i < 3; ++i)
    if (plan2[p2][i]) radix[ns++] = plan2[p2][i];
  for (int r : {3, 5, 7})
    while (m % r == 0) {
      if (ns >= kMaxStages) return false;
      m /= r;
      radix[ns++] = r;
    }
  if (m != 1) return false;
  *nstages = ns;
  return true;
}

bool reg_fft_site_enabled(FftSite site, int n)
{
  // Built-in choice, from timing both paths in every kernel on GB300 at
  // 256^2 x 32 and 512^2 x 48: the register path wins for all lengths up to
  // 256 and, at any length, in the ingest rows and the short z lines; the
  // 512- and 1024-point transforms of the overlap, correlation and assembly
  // kernels are faster with the Stockham stages (the register path's 130-255
  // registers per thread leave one CTA per SM there).
  static const int forced = [] {
    const char* e = std::getenv("SIMRECON_FFT_REGISTER_SITES");
    return e ? (int)(std::strtoul(e, nullptr, 16) | (1u << kSiteSelfTest)) : -1;
  }();
  if (forced >= 0) return (forced >> (int)site) & 1;
  switch (site) {
    case kSiteIngestX:
    case kSiteSeparateZ:
    case kSiteAsmZ:
    case kSiteSelfTest:
      return true;
    default:
      return n <= 256;
  }
}

void allow_dynamic_smem(const void* func, size_t bytes)
{
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> cur;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  size_t& have = cur[{dev, func}];
  if (bytes > have) {
    if (cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess)
      have = bytes;
  }
}

bool fft_length_ok(int n)
{
  std::vector<int> r;
  return factor(n, r);
}

bool get_fft_plan(int n, FFTPlan* plan)
{
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_plans.find({dev, n});
  if (it != g_plans.end()) {
    *plan = it->second;
    return true;
  }
  std::vector<int> radix;
  if (!factor(n, radix)) return false;
  FFTPlan p{};
  p.n = n;
  p.nstages = (int)radix.size();
  for (int i = 0; i < p.nstages; ++i) p.radix[i] = radix[i];
  std::vector<float2> tw(2 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    double a = -2.0 * M_PI * (double)k / (double)n;
    tw[k] = make_float2((float)cos(a), (float)sin(a));
  }
  const int P = reg_fft_lanes(n);
  if (P) {
    const int E = n / P;
    for (int k1 = 1; k1 < E; ++k1)
      for (int q = 0; q < P; ++q) tw[n + (size_t)(k1 - 1) * P + q] = tw[((size_t)q * k1) % n];
  }
  float2* d = nullptr;
  if (cudaMalloc(&d, sizeof(float2) * 2 * n) != cudaSuccess) return false;
  if (cudaMemcpy(d, tw.data(), sizeof(float2) * 2 * n, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return false;
  }
  p.tw = d;
  p.twr = P ? d + n : nullptr;
  g_plans[{dev, n}] = p;
  *plan = p;
  return true;
}

}  // namespace simrecon
