// FFT plans: radix sequences and double-precision twiddle tables, cached per
// (device, length).  The tables are allocated once per length and live until
// process exit.
#include <sys/stat.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
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

// ------------------------------------------------------------- site choices
// Which FFT path a call site uses for a length the register path supports:
//  1. a choice forced on the calling thread (the tuner's trial runs),
//  2. the SIMRECON_FFT_REGISTER_SITES hex mask (a manual override),
//  3. the tuned table: choices measured by SRX_tuneFFT on this GPU model and
//     kept in a plan-cache file (SIMRECON_FFT_PLAN_CACHE, else
//     $XDG_CACHE_HOME or ~/.cache /cudasirecon_gb300/fft_plans.tsv), one line
//     per choice: GPU name, site, length, path, and both measured times,
//  4. the built-in default.
namespace {
const char* const kSiteNames[kNumFftSites] = {"ingest_x", "ingest_y", "separate_z", "overlap_x", "overlap_y",
                                              "crosscorr_rows", "crosscorr_cols", "assemble_y", "assemble_x",
                                              "assemble_z", "makeotf", "selftest"};
thread_local int t_force_site = -1, t_force_reg = 0;
thread_local std::set<std::pair<int, int>>* t_seen = nullptr;

struct Tuned {
  bool loaded = false;
  // (gpu name, site, n) -> register path?
  std::map<std::tuple<std::string, int, int>, std::pair<bool, std::pair<double, double>>> table;
};
std::mutex g_tuned_mu;
Tuned g_tuned;
std::map<int, std::string> g_dev_names;

std::string cache_path()
{
  if (const char* e = std::getenv("SIMRECON_FFT_PLAN_CACHE")) return e;
  std::string base;
  if (const char* x = std::getenv("XDG_CACHE_HOME")) base = x;
  else if (const char* h = std::getenv("HOME")) base = std::string(h) + "/.cache";
  else base = "/tmp";
  return base + "/cudasirecon_gb300/fft_plans.tsv";
}

std::string device_name()
{
  int dev = 0;
  cudaGetDevice(&dev);
  auto it = g_dev_names.find(dev);
  if (it != g_dev_names.end()) return it->second;
  cudaDeviceProp prop{};
  std::string name = cudaGetDeviceProperties(&prop, dev) == cudaSuccess ? prop.name : "unknown";
  for (char& c : name)
    if (c == '\t' || c == '\n') c = ' ';
  g_dev_names[dev] = name;
  return name;
}

int site_index(const std::string& name)
{
  for (int i = 0; i < kNumFftSites; ++i)
    if (name == kSiteNames[i]) return i;
  return -1;
}

// caller holds g_tuned_mu
void load_tuned()
{
  if (g_tuned.loaded) return;
  g_tuned.loaded = true;
  std::ifstream f(cache_path());
  std::string line;
  while (std::getline(f, line)) {
    std::vector<std::string> col;
    size_t a = 0;
    for (size_t b; (b = line.find('\t', a)) != std::string::npos; a = b + 1) col.push_back(line.substr(a, b - a));
    col.push_back(line.substr(a));
    if (col.size() < 6) continue;
    const int site = site_index(col[1]);
    const int n = std::atoi(col[2].c_str());
    if (site < 0 || n <= 0 || (col[3] != "register" && col[3] != "stockham")) continue;
    g_tuned.table[{col[0], site, n}] = {col[3] == "register", {std::atof(col[4].c_str()), std::atof(col[5].c_str())}};
  }
}

// caller holds g_tuned_mu; the whole table is rewritten through a temporary
// file and a rename, so a concurrent reader sees the old or the new file
bool save_tuned(std::string* err)
{
  const std::string path = cache_path();
  const size_t slash = path.find_last_of('/');
  if (slash != std::string::npos) {
    std::string dir = path.substr(0, slash), cur;
    for (size_t i = 0; i <= dir.size(); ++i)
      if (i == dir.size() || dir[i] == '/') {
        cur = dir.substr(0, i);
        if (!cur.empty()) mkdir(cur.c_str(), 0755);
      }
  }
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  {
    std::ofstream f(tmp, std::ios::trunc);
    if (!f) {
      *err = "cannot write the FFT plan cache " + tmp;
      return false;
    }
    for (auto& [k, v] : g_tuned.table)
      f << std::get<0>(k) << '\t' << kSiteNames[std::get<1>(k)] << '\t' << std::get<2>(k) << '\t'
        << (v.first ? "register" : "stockham") << '\t' << v.second.first << '\t' << v.second.second << '\n';
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) {
    *err = "cannot replace the FFT plan cache " + path;
    return false;
  }
  return true;
}

bool builtin_choice(FftSite site, int n)
{
  // Built-in choice, from timing both paths in every kernel on GB300 at
  // 256^2 x 32 and 512^2 x 48: the register path wins for all lengths up to
  // 256 and, at any length, in the ingest rows and the short z lines; the
  // 512- and 1024-point transforms of the overlap, correlation and assembly
  // kernels are faster with the Stockham stages (the register path's 130-255
  // registers per thread leave one CTA per SM there).
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
}  // namespace

bool reg_fft_site_enabled(FftSite site, int n)
{
  if (t_seen) t_seen->insert({(int)site, n});
  if (t_force_site == (int)site) return t_force_reg != 0;
  static const int forced = [] {
    const char* e = std::getenv("SIMRECON_FFT_REGISTER_SITES");
    return e ? (int)(std::strtoul(e, nullptr, 16) | (1u << kSiteSelfTest)) : -1;
  }();
  if (forced >= 0) return (forced >> (int)site) & 1;
  if (site != kSiteSelfTest && reg_fft_lanes(n)) {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    load_tuned();
    auto it = g_tuned.table.find({device_name(), (int)site, n});
    if (it != g_tuned.table.end()) return it->second.first;
  }
  return builtin_choice(site, n);
}

void fft_site_force(int site, bool reg) { t_force_site = site, t_force_reg = reg; }
void fft_site_unforce() { t_force_site = -1; }
void fft_sites_track(std::set<std::pair<int, int>>* seen) { t_seen = seen; }
const char* fft_site_name(int site) { return site >= 0 && site < kNumFftSites ? kSiteNames[site] : "?"; }

bool fft_plan_record(int site, int n, bool reg, double ms_reg, double ms_stockham, std::string* err)
{
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  load_tuned();
  g_tuned.table[{device_name(), site, n}] = {reg, {ms_reg, ms_stockham}};
  return save_tuned(err);
}

// 1 register path, 0 Stockham stages; *source: "forced", "environment",
// "tuned", "built-in" or "stockham-only" (no register path for n)
int fft_plan_choice(int site, int n, const char** source)
{
  const char* src = "built-in";
  int r;
  if (site < 0 || site >= kNumFftSites) return -1;
  if (!reg_fft_lanes(n)) {
    src = "stockham-only";
    r = 0;
  } else if (t_force_site == site) {
    src = "forced";
    r = t_force_reg;
  } else if (std::getenv("SIMRECON_FFT_REGISTER_SITES")) {
    src = "environment";
    r = reg_fft_site_enabled((FftSite)site, n);
  } else {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    load_tuned();
    auto it = g_tuned.table.find({device_name(), site, n});
    if (it != g_tuned.table.end()) {
      src = "tuned";
      r = it->second.first;
    } else {
      r = builtin_choice((FftSite)site, n);
    }
  }
  if (source) *source = src;
  return r;
}

std::string fft_plan_cache_path() { return cache_path(); }

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
