// extern "C" SR_* entry points (src/cudaSirecon/interface.cpp:10-71 of the
// reference) plus the additions declared in include/cudasirecon.h.  No C++
// exception crosses this boundary and nothing here calls exit(): failures are
// recorded as a thread-local message for SR_getLastError.
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "cudasirecon.h"
#include "makeotf.h"
#include "reconstructor.h"
#include "server.h"

namespace simrecon {
int makeotf_main(int argc, const char* const* argv, std::string* err);
}

namespace {
thread_local std::string g_last_error;

template <typename F>
bool guarded(F&& f)
{
  try {
    f();
    return true;
  } catch (const std::exception& e) {
    g_last_error = e.what();
  } catch (...) {
    g_last_error = "unknown error";
  }
  return false;
}

bool need(SIM_Reconstructor* sr)
{
  if (!sr) {
    g_last_error = "null SIM_Reconstructor handle";
    return false;
  }
  return true;
}

ReconParams g_dummy_params;
ImageParams g_dummy_image;
}  // namespace

extern "C" {

SIM_Reconstructor* SR_new_from_shape(int nx, int ny, int nImages, const char* configFileName)
{
  SIM_Reconstructor* r = nullptr;
  guarded([&] {
    std::string err;
    r = SIM_Reconstructor::from_shape(nx, ny, nImages, configFileName ? configFileName : "", &err);
    if (!r) g_last_error = err;
  });
  return r;
}

void SR_setRaw(SIM_Reconstructor* sr, const float* raw_data, int nx, int ny, int nz)
{
  if (need(sr)) guarded([&] { sr->set_raw_float(raw_data, nx, ny, nz); });
}

void SR_setRawU16(SIM_Reconstructor* sr, const uint16_t* raw_data, int nx, int ny, int nz)
{
  if (need(sr)) guarded([&] { sr->set_raw_u16(raw_data, nx, ny, nz); });
}

void SR_loadAndRescaleImage(SIM_Reconstructor* sr, int it, int iw)
{
  if (need(sr)) guarded([&] { sr->load_and_rescale(it, iw); });
}

void SR_setCurTimeIdx(SIM_Reconstructor* sr, int it)
{
  if (need(sr)) guarded([&] { sr->set_cur_time(it); });
}

void SR_processOneVolume(SIM_Reconstructor* sr)
{
  if (need(sr)) guarded([&] { sr->process_one_volume(); });
}

void SR_getResult(SIM_Reconstructor* sr, float* result)
{
  if (need(sr)) guarded([&] { sr->get_result(result); });
}

ReconParams& SR_getReconParams(SIM_Reconstructor* sr)
{
  if (!need(sr)) return g_dummy_params;
  return sr->opt.p;
}

ImageParams& SR_getImageParams(SIM_Reconstructor* sr)
{
  if (!need(sr)) return g_dummy_image;
  return sr->opt.ip;
}

SIM_Reconstructor* SR_new_from_argv(int argc, char** argv)
{
  SIM_Reconstructor* r = nullptr;
  guarded([&] {
    std::string err;
    r = SIM_Reconstructor::from_argv(argc, argv, &err);
    if (!r) g_last_error = err;
  });
  return r;
}

void SR_setFile(SIM_Reconstructor* sr, int it, int iw)
{
  if (need(sr)) guarded([&] { sr->set_file(it, iw); });
}

void SR_writeResult(SIM_Reconstructor* sr, int it, int iw)
{
  if (need(sr)) guarded([&] { sr->write_result(it, iw); });
}

void SR_closeFiles(SIM_Reconstructor* sr)
{
  if (need(sr)) guarded([&] { sr->close_files(); });
}

void SR_delete(SIM_Reconstructor* sr)
{
  guarded([&] { delete sr; });
}

const char* SR_getLastError(void) { return g_last_error.c_str(); }

void SR_clearError(void) { g_last_error.clear(); }

int SR_getNTimes(SIM_Reconstructor* sr) { return need(sr) ? sr->ntimes() : 0; }

void SRX_getFit(SIM_Reconstructor* sr, float* k0, float* amps)
{
  if (need(sr)) guarded([&] { sr->get_fit(k0, amps); });
}

int SRX_prepare(SIM_Reconstructor* sr)
{
  int rc = -1;
  if (need(sr)) guarded([&] { rc = sr->prepare(); });
  return rc;
}

int SRX_getBand(SIM_Reconstructor* sr, int dir, int b, float* out)
{
  int rc = -1;
  if (need(sr)) guarded([&] { rc = sr->get_band(dir, b, out); });
  return rc;
}

int SRX_benchDevice(SIM_Reconstructor* sr, int steps, double* total_ms)
{
  int rc = -1;
  if (need(sr))
    guarded([&] {
      double t = sr->bench_device(steps);
      if (total_ms) *total_ms = t;
      rc = 0;
    });
  return rc;
}

void SRX_setProfiling(SIM_Reconstructor* sr, int on)
{
  if (need(sr)) sr->set_profiling(on != 0);
}

int SRX_getProfile(SIM_Reconstructor* sr, char* json, int maxlen)
{
  int rc = -1;
  if (need(sr))
    guarded([&] {
      std::string s = sr->profile_json();
      if (json && maxlen > 0) {
        strncpy(json, s.c_str(), maxlen - 1);
        json[maxlen - 1] = '\0';
      }
      rc = (int)s.size();
    });
  return rc;
}

void SRX_resetProfile(SIM_Reconstructor* sr)
{
  if (need(sr)) guarded([&] { sr->reset_profile(); });
}

void SRX_fitCounts(SIM_Reconstructor* sr, long long* out3)
{
  if (need(sr) && out3) sr->fit_counts(out3);
}

int SRX_tuneFFT(SIM_Reconstructor* sr, int reps, char* json, int maxlen)
{
  if (!need(sr)) return -1;
  int rc = -1;
  guarded([&] {
    const std::string j = sr->tune_fft(reps);
    if (json && maxlen > 0) {
      std::strncpy(json, j.c_str(), (size_t)maxlen - 1);
      json[maxlen - 1] = '\0';
    }
    rc = (int)j.size();
  });
  return rc;
}

int SRX_fftPlanChoice(int site, int n, char* source, int maxlen)
{
  const char* src = "";
  const int r = simrecon::fft_plan_choice(site, n, &src);
  if (source && maxlen > 0) {
    std::strncpy(source, src, (size_t)maxlen - 1);
    source[maxlen - 1] = '\0';
  }
  return r;
}

int SRX_lastProcessResult(SIM_Reconstructor* sr) { return need(sr) ? sr->last_process_result() : -1; }

void SRX_setFilterFusion(SIM_Reconstructor* sr, int on)
{
  if (need(sr)) sr->set_filter_fusion(on != 0);
}

void SRX_setDeviceK0Search(SIM_Reconstructor* sr, int on)
{
  if (need(sr)) sr->set_device_search(on != 0);
}

long long SRX_kernelLaunches(SIM_Reconstructor* sr) { return need(sr) ? sr->launches() : -1; }

int SRX_fftSelfTest(float* data, int n, int nlines, int inverse, int columns)
{
  int rc = -1;
  guarded([&] {
    size_t bytes = (size_t)n * nlines * 2 * sizeof(float);
    float2* d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) throw std::runtime_error("cudaMalloc failed");
    cudaMemcpy(d, data, bytes, cudaMemcpyHostToDevice);
    rc = simrecon::launch_fft_selftest(d, n, nlines, inverse, columns, 0);
    cudaMemcpy(data, d, bytes, cudaMemcpyDeviceToHost);
    cudaError_t e = cudaDeviceSynchronize();
    cudaFree(d);
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
  });
  return rc;
}

int SRX_processSeries(SIM_Reconstructor* sr, const void* const* raws, int raw_is_u16, float* const* outs, int n,
                      int t0)
{
  int rc = -1;
  if (need(sr))
    guarded([&] {
      sr->process_series(raws, raw_is_u16 != 0, outs, n, t0);
      rc = 0;
    });
  return rc;
}

int SRX_makeOTF(const float* psf, int nx, int ny, int nsections, int nargs, const char* const* args, float* out,
                size_t out_floats, int* dims)
{
  int rc = -1;
  guarded([&] {
    simrecon::MakeOtfOptions o;
    std::string err;
    if (!psf || nx <= 0 || ny <= 0 || nsections <= 0 || nargs < 0 || (nargs > 0 && !args)) {
      g_last_error = "SRX_makeOTF: invalid arguments";
      return;
    }
    if (!simrecon::makeotf_parse_switches(nargs, args, &o, &err)) {
      g_last_error = err;
      return;
    }
    simrecon::OtfResult r;
    if (!simrecon::makeotf_run(psf, nx, ny, nsections, o, &r, &err)) {
      g_last_error = err;
      return;
    }
    if (dims) {
      dims[0] = r.width;
      dims[1] = r.height;
      dims[2] = r.depth;
    }
    if (out) {
      if (out_floats < r.data.size()) {
        g_last_error = "SRX_makeOTF: output buffer too small (" + std::to_string(r.data.size()) + " floats needed)";
        return;
      }
      std::memcpy(out, r.data.data(), r.data.size() * sizeof(float));
    }
    rc = 0;
  });
  return rc;
}

int SRX_makeotfMain(int argc, char** argv)
{
  int rc = -1;
  guarded([&] {
    std::string err;
    rc = simrecon::makeotf_main(argc, argv, &err);
    if (rc != 0) g_last_error = err;
  });
  return rc;
}

SRX_Server* SRX_serverCreate(int workers, size_t hbm_budget_bytes)
{
  SRX_Server* s = nullptr;
  guarded([&] { s = (SRX_Server*)new simrecon::ReconServer(workers, hbm_budget_bytes); });
  return s;
}

int SRX_serverAddConfig(SRX_Server* s, const char* config_path)
{
  int id = -1;
  if (!s || !config_path) {
    g_last_error = "SRX_serverAddConfig: invalid arguments";
    return -1;
  }
  guarded([&] { id = ((simrecon::ReconServer*)s)->add_config(config_path); });
  return id;
}

long long SRX_serverSubmit(SRX_Server* s, int config, int nx, int ny, int nimages, const void* raw, int raw_is_u16,
                           float* out)
{
  long long t = -1;
  if (!s) {
    g_last_error = "SRX_serverSubmit: null server";
    return -1;
  }
  guarded([&] {
    std::string err;
    t = ((simrecon::ReconServer*)s)->submit(config, nx, ny, nimages, raw, raw_is_u16 != 0, out, &err);
    if (t < 0) g_last_error = err;
  });
  return t;
}

int SRX_serverWait(SRX_Server* s, long long ticket, double* latency_ms)
{
  int rc = -1;
  if (!s) {
    g_last_error = "SRX_serverWait: null server";
    return -1;
  }
  guarded([&] {
    std::string err;
    rc = ((simrecon::ReconServer*)s)->wait(ticket, latency_ms, &err);
    if (rc != 0) g_last_error = err;
  });
  return rc;
}

int SRX_serverReserve(SRX_Server* s, int config, int nx, int ny, int nimages, int count)
{
  int n = -1;
  if (!s) {
    g_last_error = "SRX_serverReserve: null server";
    return -1;
  }
  guarded([&] {
    std::string err;
    n = ((simrecon::ReconServer*)s)->reserve(config, nx, ny, nimages, count, &err);
    if (n < count) g_last_error = err;
  });
  return n;
}

int SRX_serverRunBatch(SRX_Server* s, const SRX_BatchItem* items, int n)
{
  if (!s || n < 0 || (n > 0 && !items)) {
    g_last_error = "SRX_serverRunBatch: invalid arguments";
    return -1;
  }
  int rc = -1;
  guarded([&] {
    std::vector<simrecon::ReconServer::BatchItem> v((size_t)n);
    for (int i = 0; i < n; ++i)
      v[i] = {items[i].config, items[i].nx, items[i].ny, items[i].nimages, items[i].raw, items[i].raw_is_u16 != 0,
              items[i].out};
    std::string err;
    rc = ((simrecon::ReconServer*)s)->run_batch(v, &err);
    if (rc != 0) g_last_error = err;
  });
  return rc;
}

int SRX_serverSetK0Reuse(SRX_Server* s, int config, int on)
{
  if (!s) {
    g_last_error = "SRX_serverSetK0Reuse: null server";
    return -1;
  }
  int rc = -1;
  guarded([&] {
    std::string err;
    rc = ((simrecon::ReconServer*)s)->set_k0_reuse(config, on != 0, &err);
    if (rc != 0) g_last_error = err;
  });
  return rc;
}

int SRX_serverRecordedK0(SRX_Server* s, int config, float* k0, int ndirs)
{
  if (!s || !k0) return 0;
  std::vector<float> v;
  if (!((simrecon::ReconServer*)s)->recorded_k0(config, &v)) return 0;
  for (int i = 0; i < 2 * ndirs && i < (int)v.size(); ++i) k0[i] = v[i];
  return 1;
}

void SRX_serverCounters(SRX_Server* s, long long* created, long long* evicted)
{
  if (s) ((simrecon::ReconServer*)s)->counters(created, evicted);
}

int SRX_batchPlan(const SRX_BatchItem* items, int n, int workers, int* chunk_of_item)
{
  if (n < 0 || (n > 0 && (!items || !chunk_of_item))) {
    g_last_error = "SRX_batchPlan: invalid arguments";
    return -1;
  }
  int nchunks = -1;
  guarded([&] {
    std::vector<simrecon::ReconServer::BatchItem> v((size_t)n);
    for (int i = 0; i < n; ++i)
      v[i] = {items[i].config, items[i].nx, items[i].ny, items[i].nimages, items[i].raw, items[i].raw_is_u16 != 0,
              items[i].out};
    const auto plan = simrecon::plan_batch(v, workers < 1 ? 1 : (size_t)workers);
    for (size_t c = 0; c < plan.size(); ++c)
      for (size_t i : plan[c]) chunk_of_item[i] = (int)c;
    nchunks = (int)plan.size();
  });
  return nchunks;
}

size_t SRX_serverDeviceBytes(SRX_Server* s) { return s ? ((simrecon::ReconServer*)s)->device_bytes_in_use() : 0; }

size_t SRX_serverDeviceBytesHeld(SRX_Server* s) { return s ? ((simrecon::ReconServer*)s)->device_bytes_held() : 0; }

void SRX_serverMemory(SRX_Server* s, size_t* reserved, size_t* held)
{
  size_t r = 0, h = 0;
  if (s) ((simrecon::ReconServer*)s)->memory_snapshot(&r, &h);
  if (reserved) *reserved = r;
  if (held) *held = h;
}

size_t SRX_serverPlannedBytes(SRX_Server* s, int config, int nx, int ny, int nimages)
{
  if (!s) {
    g_last_error = "SRX_serverPlannedBytes: null server";
    return 0;
  }
  size_t b = 0;
  std::string e;
  if (!((simrecon::ReconServer*)s)->planned_bytes(config, nx, ny, nimages, &b, &e)) {
    g_last_error = e;
    return 0;
  }
  return b;
}

long long SRX_serverAdmissionWaits(SRX_Server* s)
{
  long long w = 0;
  if (s) ((simrecon::ReconServer*)s)->counters(nullptr, nullptr, &w);
  return w;
}

void SRX_serverDestroy(SRX_Server* s)
{
  guarded([&] { delete (simrecon::ReconServer*)s; });
}

int SRX_pinHost(void* ptr, size_t bytes)
{
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) {
    g_last_error = std::string("cudaHostRegister: ") + cudaGetErrorString(e);
    return (int)e;
  }
  return 0;
}

void* SRX_hostAlloc(size_t bytes)
{
  void* p = nullptr;
  cudaError_t e = cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    g_last_error = std::string("cudaHostAlloc: ") + cudaGetErrorString(e);
    return nullptr;
  }
  return p;
}

void SRX_hostFree(void* ptr)
{
  if (ptr) cudaFreeHost(ptr);
}

int SRX_deviceMemInfo(size_t* free_bytes, size_t* total_bytes)
{
  if (!free_bytes || !total_bytes) {
    g_last_error = "SRX_deviceMemInfo: null argument";
    return -1;
  }
  cudaError_t e = cudaMemGetInfo(free_bytes, total_bytes);
  if (e != cudaSuccess) {
    g_last_error = std::string("SRX_deviceMemInfo: ") + cudaGetErrorString(e);
    return -1;
  }
  return 0;
}

int SRX_unpinHost(void* ptr)
{
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) {
    g_last_error = std::string("cudaHostUnregister: ") + cudaGetErrorString(e);
    return (int)e;
  }
  return 0;
}

}  // extern "C"
