// SIM_Reconstructor: the object behind the SR_* C ABI (the reference's
// class of the same name, src/cudaSirecon/SIM_reconstructor.hpp:19-158),
// rebuilt around device-resident buffers, one CUDA stream per handle and the
// fused kernels of this library.
#pragma once
#include <cuda_runtime.h>

#include <complex>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "image_io.h"
#include "kernels.h"
#include "params.h"

struct float2v {
  float x, y;
};

class SIM_Reconstructor {
 public:
  // construction paths (interface.cpp:13-17, 54-57)
  static SIM_Reconstructor* from_shape(int nx, int ny, int nimages, const std::string& config, std::string* err);
  static SIM_Reconstructor* from_argv(int argc, char** argv, std::string* err);
  // device bytes a from_shape handle of this shape and configuration can
  // hold (arena, time-series buffers, calibration), found without allocating
  static bool plan_bytes(int nx, int ny, int nimages, const std::string& config, size_t* bytes, std::string* err);
  ~SIM_Reconstructor();

  void set_raw_float(const float* raw, int nx, int ny, int nz);
  void set_raw_u16(const uint16_t* raw, int nx, int ny, int nz);
  void load_and_rescale(int it, int iw);
  void set_cur_time(int it) { opt.ip.curTimeIdx = (unsigned short)it; }
  // sync = false leaves the volume's work queued on the handle's stream
  int process_one_volume(bool sync = true);
  void get_result(float* out);
  // n volumes: per volume i the same as setRaw(raws[i]) ->
  // loadAndRescaleImage(t0+i) -> setCurTimeIdx(t0+i) -> processOneVolume ->
  // getResult(outs[i]), with the upload of volume i+1 and the download of
  // volume i-1 overlapped with the computation of volume i (double-buffered
  // device raw/output buffers, separate copy streams; page-locked host
  // buffers make the copies asynchronous).  standalone: every volume is
  // processed as time 0 instead (its own k0 search), the plain per-request
  // flow, with the same overlap.
  void process_series(const void* const* raws, bool u16, float* const* outs, int n, int t0,
                      bool standalone = false);
  void set_file(int it, int iw);
  void write_result(int it, int iw);
  void close_files();
  // what the last process_one_volume returned: 1 reconstructed, 0 stopped
  // after the debug dumps (the reference's driver then writes no result)
  int last_process_result() const { return last_result_; }
  int ntimes() const { return opt.ip.ntimes; }
  void set_ntimes(int n) { opt.ip.ntimes = (short)n; }
  // the k0 of every direction as if time point 0 had fitted it (k0[2 d], k0[2 d + 1])
  void set_fitted_k0(const float* k0);

  // introspection / performance
  void get_fit(float* k0, float* amps);
  int prepare();  // separate bands without fitting (for stage checks)
  int get_band(int dir, int b, float* out);
  double bench_device(int steps);
  void set_profiling(bool on) { profiling_ = on; }
  // Wiener filter inside the assembly's band load where supported (default),
  // or always as its own pass; both give the same volume within float rounding
  void set_filter_fusion(bool on) { filter_fusion_ = on; }
  // k0 search on the device (default) or host-driven with batched candidate
  // evaluations; both visit the same float32 angles and magnitudes
  void set_device_search(bool on) { device_search_ = on; }
  // time both FFT paths at every site and length this handle's volume uses
  // (best of `reps`), record the faster in the plan cache; returns JSON
  std::string tune_fft(int reps);
  std::string profile_json();
  void reset_profile();
  long long launches() const { return launches_; }
  // executed overlap builds (makeoverlaps), reductions over an overlap pair
  // (modamp evaluations and the cross-correlation) and k0 searches since
  // creation: the n_mo / n_red of the algorithmic-bytes model
  void fit_counts(long long* out3) const
  {
    for (int i = 0; i < 3; ++i) out3[i] = fit_counts_[i];
  }
  size_t out_elems() const { return (size_t)X_ * Y_ * Z_; }
  size_t device_bytes() const  // device memory the handle holds
  {
    return arena_bytes_ + series_bytes_ + (d_bgslope_ ? 2 * (size_t)nx_ * ny_ * sizeof(float) : 0);
  }

  simrecon::Options opt;  // ReconParams + ImageParams live here (references handed out)

 private:
  SIM_Reconstructor() = default;
  bool init_shape(int nx, int ny, int nimages, const std::string& config, std::string* err);
  bool setup(int nx, int ny, int nimages, int nwaves, const simrecon::Stack* otf, std::string* err);
  bool load_otf_tiff(const std::string& path, simrecon::Stack* out, std::string* err);
  bool load_corr(std::string* err);
  void stage_raw(const void* raw, bool u16);
  void ingest();
  void separate();
  void fit_all();
  void fit_direction(int d);
  bool fit_without_search() const;
  void fit_on_device();
  bool device_search_possible() const;
  bool fit_search_on_device();
  simrecon::FitFinishArgs fit_finish_args() const;
  int upload_amps();
  void sync_amps() const;
  void filter_and_assemble();
  void filter_zdc(int* zdc) const;
  simrecon::AssembleArgs asm_geometry() const;
  size_t asm_table_bytes() const;
  bool asm_tables_current(const simrecon::AssembleArgs& aa) const;
  void prepare_asm_tables();
  bool capture_volume(int b, void* raw, float* out, int t, cudaEvent_t raw_free);
  // debug dumps (saveprefiltered / savealignedraw / saveoverlaps)
  bool debug_requested() const;
  bool open_debug_files(std::string* err);
  int debug_volume();
  void debug_write_bands(int d);
  void debug_dump_overlaps(bool search_branch);
  void close_debug_files();
  void drop_graphs();
  static void check(cudaError_t e, const char* what);
  void check_launch(int rc, const char* what);

  // fitting helpers (gpuFunctionsImpl.cu:306-1148 semantics)
  // kdev: the shift from device memory (times kfac); pmap / sumxy: outputs
  // other than the handle's single overlap map
  void build_overlaps(int d, int o1, int o2, float k0x, float k0y, const float2* kdev = nullptr, float kfac = 0.f,
                      float2* pmap = nullptr, double* sumxy = nullptr, int lane = 0);
  // fit lanes (the overlap pairs of the fit built side by side on their own
  // streams)
  static constexpr int kFitLanes = 3;  // six lanes measured 1 % faster for twice the buffers
  size_t ovl_lane_elems() const;
  size_t ppart_lane_elems() const;
  size_t sums_lane_elems() const;
  size_t tables_lane_elems() const;
  size_t partial_lane_elems() const;
  float2* lane_pmap(int l) const;
  float2* lane_tables(int l) const;
  double* lane_partial(int l) const;
  double* lane_xstary(int l) const;
  cudaStream_t lane_stream(int l) const;
  int lanes_begin();
  void lanes_end(int nl);
  int overlap_zdc_bessel(int order2, float k0x, float k0y) const;
  // evaluate XStarY for candidate (angle, mag) pairs on the current overlaps
  void eval_candidates(int o1, int o2, const std::vector<std::pair<float, float>>& cands);
  float getmodamp(int d, float angle, float mag, int o1, int o2, int redo, float2v* modamp);
  void findk0(int d);
  void fitk0andmodamps(int d);
  float2v findrealspacemodamp(int d, int o1, int o2, float k0x, float k0y, int redo);
  void prefetch_line(int o1, int o2, bool angle_axis, float fixed, float start, float step, int count, int dir);

  // geometry
  int nx_ = 0, ny_ = 0, nz_ = 0, nxh_ = 0, nimg_ = 0, norders_ = 0, nph_ = 0, ndirs_ = 0;
  int nx_raw_ = 0;             // width of the raw planes (nx_ after deskew / cropXY)
  float deskew_factor_ = 0.f;  // loadImageData's deskewFactor (0: no deskew)
  bool precondition_ = false;  // deskew, crop or per-section backgrounds: a pass before ingest
  float* d_pre_ = nullptr;     // the preconditioned planes [nimg][ny][nx]
  float* d_bgx_ = nullptr;     // per-section extra background [nimg] (bBgInExtHdr)
  std::vector<float> bgx_host_;
  float* pre_own_ = nullptr;  // their allocation when not in the arena
  void ensure_precondition_buffers();
  int X_ = 0, Y_ = 0, Z_ = 0;
  int ndirs_otf_ = 1;
  int zdc_ovl_ = 0;  // makeoverlaps zdistcutoff
  bool otf_dk_from_header_ = false;  // MRC OTF: dkr / dkz taken from its header
  cudaStream_t stream_ = nullptr;
  int fit_lanes_ = 1;  // set at setup: min(ndirs * (norders - 1), kFitLanes)
  cudaStream_t fit_stream_[kFitLanes] = {};
  cudaEvent_t fit_join_[kFitLanes] = {};
  cudaEvent_t fit_fork_ = nullptr;
  int device_ = 0;
  bool filter_fusion_ = true;
  bool device_search_ = true;
  bool dry_run_ = false;      // setup computes planned_bytes_ and allocates nothing
  size_t planned_bytes_ = 0;

  // device arena
  char* arena_ = nullptr;
  size_t arena_bytes_ = 0;
  size_t series_bytes_ = 0;  // process_series' second raw and output buffers
  void* d_raw_ = nullptr;
  float2* d_spec_ = nullptr;
  float* d_scale_ = nullptr;
  double* d_sdp0_ = nullptr;
  float* d_bgslope_ = nullptr;  // usecorr: per-pixel background then slope, [2][ny][nx]
  float* d_sepmat_ = nullptr;
  float* d_apofact_ = nullptr;
  float2* d_otf_ = nullptr;
  float2* d_ovl_ = nullptr;
  float2* d_ppart_ = nullptr;
  double* d_sums_ = nullptr;
  float2* d_pmap_ = nullptr;
  double* d_sumxy_ = nullptr;
  float2* d_cc_ = nullptr;
  float* d_bval_ = nullptr;
  int* d_bidx_ = nullptr;
  float* d_peak_ = nullptr;
  float2* d_tables_ = nullptr;
  double* d_partial_ = nullptr;
  double* d_xstary_ = nullptr;
  simrecon::FitDev* d_fit_ = nullptr;  // amplitudes + filter weights of the last fit
  double* d_fitslots_ = nullptr;       // [ndirs * norders][4]: XStarY re, im, sum |X|^2 per order
  float2* d_kst_ = nullptr;            // device search, per direction: findk0's k0, k1, the fitted k0
  int* d_sinfo_ = nullptr;             // device search: candidates evaluated, status
  float2* d_pmapd_ = nullptr;          // device search: each direction's overlap map [ndirs][ny][nx]
  double* d_sumxyd_ = nullptr;         // and its sum |X|^2, sum |Y|^2 [ndirs][2]
  void* d_asmtab_ = nullptr;           // assembly slot tables
  bool asm_tables_valid_ = false;
  int asm_tables_zdc_[simrecon::kMaxOrders] = {0};
  float2* d_ex_ = nullptr;
  float2* d_ey_ = nullptr;
  float2* d_T_ = nullptr;
  size_t tcap_ = 0;
  float2* d_S_ = nullptr;
  float* d_out_ = nullptr;
  float* d_flush_ = nullptr;
  size_t flush_n_ = 0;
  // second raw and output buffers, copy streams and events of process_series
  // (allocated on first use)
  void* d_raw_alt_ = nullptr;
  float* d_out_alt_ = nullptr;   // the output buffer not holding the last result
  float* d_out_extra_ = nullptr;  // the allocation behind the second output buffer
  cudaStream_t h2d_stream_ = nullptr, d2h_stream_ = nullptr;
  cudaEvent_t ev_raw_ready_[2] = {nullptr, nullptr}, ev_raw_free_[2] = {nullptr, nullptr};
  cudaEvent_t ev_out_ready_[2] = {nullptr, nullptr}, ev_out_free_[2] = {nullptr, nullptr};
  // small page-locked host buffer for results of the fit, mapped into the
  // device's address space (dh_pinned_) so that kernels write the results
  double* h_pinned_ = nullptr;
  double* dh_pinned_ = nullptr;

  // host-side state (ReconData equivalents)
  std::vector<float> sepmat_;
  std::vector<float> noisevar_;
  std::vector<float2v> k0_, k0_time0_, k0guess_;
  // amp_ is the host copy of the device fit results; after a fit on the
  // device it is refreshed on demand (sync_amps)
  mutable std::vector<std::vector<float2v>> amp_;
  mutable bool amps_on_device_only_ = false;
  // per raw/output buffer pair of process_series: the captured volume
  struct VolumeGraph {
    cudaGraphExec_t exec = nullptr;
    void* raw = nullptr;
    float* out = nullptr;
    bool t_nonzero = false, u16 = false;
    long long launches = 0;
    long long fit_counts[3] = {0, 0, 0};
  };
  VolumeGraph graphs_[2];
  bool raw_u16_ = false;
  bool raw_staged_ = false;  // d_raw_ holds a stack staged by setRaw/setFile
  bool have_raw_ = false;
  bool rescaled_ = false;
  // overlap state for the candidate evaluator
  int cur_o1_ = -1, cur_o2_ = -1;
  double sumx_ = 0, sumy_ = 0;
  std::map<std::pair<uint32_t, uint32_t>, float2v> cache_;
  std::vector<std::complex<double>> xstary_;

  // files
  std::vector<std::string> tiff_files_;
  simrecon::MrcFile mrc_in_;
  std::string out_path_;
  std::ofstream mrc_out_;
  simrecon::MrcHeader out_hdr_{};
  char in_label0_[80] = {0};  // the input file's first label (closeFiles appends it)
  struct DebugFile {
    std::ofstream f;
    simrecon::MrcHeader h{};
    bool open = false;
  };
  DebugFile dbg_sep_, dbg_aligned_, dbg_ovl_;
  simrecon::OverlapArgs last_ovl_{};  // the arguments of the last overlap build
  int last_result_ = 1;
  std::vector<float> host_raw_;
  std::vector<std::string> argv_;

  // profiling: stage events and, per kernel, events + algorithmic bytes
  bool profiling_ = false;
  struct Pending {
    std::string stage;
    cudaEvent_t a, b;
    long long launches;
    double bytes;
    bool kernel;
  };
  std::vector<Pending> pending_;
  std::map<std::string, std::pair<double, long long>> prof_;
  struct KStat {
    double ms = 0;
    long long launches = 0;
    double bytes = 0;
  };
  std::map<std::string, KStat> kprof_;
  struct KTimer : simrecon::KernelTimer {
    SIM_Reconstructor* r = nullptr;
    cudaEvent_t cur = nullptr;
    void begin(cudaStream_t s) override;
    void end(const char* kernel, cudaStream_t s, double alg_bytes) override;
  } ktimer_;
  struct TimerScope {
    simrecon::KernelTimer* prev;
    explicit TimerScope(SIM_Reconstructor* r);
    ~TimerScope();
  };
  long long launches_ = 0;
  long long fit_counts_[3] = {0, 0, 0};
  void stage_begin(const char* name, cudaEvent_t* a, long long* l0);
  void stage_end(const char* name, cudaEvent_t a, long long l0);
};
