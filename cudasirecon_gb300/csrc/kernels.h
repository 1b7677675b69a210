// Host-side launchers of the reconstruction kernels.  Every launcher takes
// plain device pointers, sizes and a stream; none allocates.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <set>
#include <string>
#include <utility>

#include "sim_common.cuh"

namespace simrecon {

// blocks of the modamp candidate reduction at most (four per SM); its
// partial-sum buffer holds kModampBlocks x candidates x 2 doubles
constexpr int kModampBlocks = 608;

// ------------------------------------------------------------ kernel timing
// When a timer is installed on the calling thread, every launcher brackets
// its launches with begin()/end() on the launch stream and reports the
// algorithmic bytes of that launch (ideal single-pass reads + writes).
struct KernelTimer {
  virtual ~KernelTimer() {}
  virtual void begin(cudaStream_t s) = 0;
  virtual void end(const char* kernel, cudaStream_t s, double alg_bytes) = 0;
};
void set_kernel_timer(KernelTimer* t);
KernelTimer* kernel_timer();

// ----------------------------------------------------------------- FFT plans
// Returns a plan (radix sequence + device twiddles) for length n; cached per
// (device, n).  n must factor into 2, 3, 5, 7.  Returns false if it cannot.
bool get_fft_plan(int n, FFTPlan* plan);
bool fft_length_ok(int n);
// radix sequence of length n into radix[kMaxStages] (no allocation)
bool fft_radix_plan(int n, int* radix, int* nstages);

// FFT path choice per call site and length (register path or Stockham
// stages).  The tuner forces a choice on the calling thread, tracks which
// (site, length) pairs a run queries, and records measured choices in the
// on-disk plan cache that every process reads.
void fft_site_force(int site, bool reg);
void fft_site_unforce();
void fft_sites_track(std::set<std::pair<int, int>>* seen);  // nullptr stops tracking
const char* fft_site_name(int site);
bool fft_plan_record(int site, int n, bool reg, double ms_reg, double ms_stockham, std::string* err);
int fft_plan_choice(int site, int n, const char** source);
std::string fft_plan_cache_path();

// -------------------------------------------------------------------- ingest
struct IngestArgs {
  const void* raw;       // [nimg][ny][nx] uint16 or float
  int raw_is_u16;
  int nx, ny, nz, ndirs, nphases;
  int fastSI;
  const float* bg;       // [ny][nx] or null (then bgconst)
  const float* slope;    // [ny][nx] or null (then 1)
  float bgconst;
  float bgextra;
  float inscale;
  int napodize;
  const float* apofact;  // device [napodize]
  float2* spec;          // [ndirs*nphases*nz][ny][nx/2+1]
};
// flat-field + apodize + 2D R2C FFT of every raw plane into spec
// Allow `func` to be launched with `bytes` of dynamic shared memory.  The
// limit is per kernel and device and is only ever raised: host threads that
// launch the same kernel with different sizes (handles of different shapes
// used concurrently) must not lower it between another thread's set and its
// launch.
void allow_dynamic_smem(const void* func, size_t bytes);

int launch_ingest(const IngestArgs& a, cudaStream_t s, long long* launches);

// The load steps before the transforms when the raw planes are not taken as
// they are: load_and_flatfield (cudaSirecon.cpp:1715-1731) with a per-section
// extra background, then deskewOneSection (1733-1760): a shift along x that
// grows with z (linear interpolation), or, without deskew, the first nx
// columns.  out = [nimg][ny][nx] float in raw section order, ready for
// launch_ingest with no background, unit slope and unit scale.
struct PrecondArgs {
  const void* raw;  // [nimg][ny][nx_raw] uint16 or float
  int raw_is_u16;
  int nx_raw, ny, nx, nz, ndirs, nphases, fastSI, nimg;
  const float* bg;     // [ny][nx_raw] or null (then bgconst)
  const float* slope;  // [ny][nx_raw] or null (then 1)
  float bgconst;
  const float* bgx;    // [nimg] extra background per raw section
  float inscale;
  float deskew_factor;  // 0: no deskew
  int extra_shift;
  float* out;
};
int launch_precondition(const PrecondArgs& a, cudaStream_t s, long long* launches);

// Bleach-correction ratios from the plane sums (DC terms of spec):
// scale[d][p][z] (float); sdp0 [nz] (double) persists across time points.
int launch_rescale(const float2* spec, int nx, int ny, int nz, int ndirs, int nphases, int t, int equalizez,
                   int equalizet, double* sdp0, float* scale, cudaStream_t s, long long* launches);

// Separation (band_i = sum_j M[i][j] * scale[p][z] * spec_j) + forward z FFT,
// in place, all directions.
int launch_separate(float2* spec, const float* scale, const float* sepmat /* device [nb][nph] */, int nx, int ny,
                    int nz, int ndirs, int nphases, cudaStream_t s, long long* launches);

// ----------------------------------------------------------------- fitting
struct OverlapArgs {
  const float2* bands;  // bands of one direction: [nph][nz][ny][nxh]
  int nx, ny, nz;
  int order1, order2;
  float kx, ky;         // k0 * (order2 - order1), 1/um
  const float2* kdev;   // if set: k0 from device memory, times kfac (kx, ky unused)
  float kfac;
  float dkx, dky;
  float rdistcutoff, otfcutoff, order0_2_factor;
  // exact squared forms of makeoverlaps' float decisions (set by
  // launch_overlaps): sqrtf(r2) <= rdistcutoff <=> r2 <= r2_le,
  // sqrtf(r2) < rdistcutoff <=> r2 < r2_lt, sqrtf(m) > otfcutoff <=> m > m_le,
  // sqrtf(m) * order0_2_factor > otfcutoff <=> m >= m_f
  float r2_le, r2_lt, m_le, m_f;
  int zdc;              // planes -zdc..zdc are built
  int nokz0;
  OTFView otf;
  float2* ovl;          // [2][2*zdc+1][ny][nx]   (x-inverse-transformed rows)
  float2* ppart;        // [ngroups][ny][nx]
  double* sums;         // [2 * nctas] partial |X|^2, |Y|^2
  float2* pmap;         // [ny][nx] result: nz * sum_kz conj(X~) Y~
  double* sumxy;        // [2] result: sum |X|^2, sum |Y|^2 (real-space, like the reference)
};
int launch_overlaps(OverlapArgs& a, cudaStream_t s, long long* launches);

// The two overlaps of the last launch_overlaps as full real-space volumes,
// [2][nz][ny][nx] complex (the reference's overlap0/overlap1 after
// makeoverlaps' inverse 3D FFT): the x-transformed rows of the built kz
// planes scattered into every kz plane (zero outside +-zdc), then inverse
// FFTs along y and z.  For the debug dump only; vol is the caller's.
int launch_overlap_volumes(const OverlapArgs& a, float2* vol, cudaStream_t s);

// crosscorr = FFT2(conj(pmap)); intensity argmax with the two-neighbour
// values along x and y (wrap-around) written to peak[0..6]:
// {ix, iy, a1x, a2, a3x, a1y, a3y}
int launch_crosscorr_peak(const float2* pmap, float2* cc, int nx, int ny, float* blockval, int* blockidx,
                          float* peak, cudaStream_t s, long long* launches);

// Copies n1 and n2 4-byte words with one small kernel: from device memory to
// (mapped, page-locked) host memory, so that results of a few bytes reach the
// host without queueing on the copy engines behind other streams' large
// transfers, or from device to device memory.
int launch_copy_out(const void* src1, void* dst1, size_t n1, const void* src2, void* dst2, size_t n2, cudaStream_t s,
                    long long* launches);

// Candidate pattern vectors of one modamp pass, passed by value as a kernel
// argument (no host-to-device copy): k[c] = k0_c * (order2 - order1), 1/um.
constexpr int kMaxCand = 64;
struct CandList {
  float2 k[kMaxCand];
};
// XStarY[c] = sum_xy pmap(x,y) exp(i 2pi ((x - nx/2) kx_c + (y - ny/2) ky_c) dxy), c < ncand
int launch_modamp_candidates(const float2* pmap, int nx, int ny, float dxy, const CandList& kcand, int ncand,
                             float2* tables, double* partial, double* xstary, cudaStream_t s, long long* launches);
// one candidate read from device memory: kdev[0] * kfac
int launch_modamp_device_k(const float2* pmap, int nx, int ny, float dxy, const float2* kdev, float kfac,
                           float2* tables, double* partial, double* xstary, cudaStream_t s, long long* launches);

// The pattern-vector search on the device (k_search.cu).
// Upper bound on each line search's climb (the reference's loops have none):
// 4096 steps is 4 rad of angle or 400 frequency pixels of magnitude.
constexpr int kMaxClimbSteps = 4096;
// findk0's peak refinement: peak = {ix, iy, a1x, a2, a3x, a1y, a3y} ->
// k0out; k1out = k0 through (|k0|, atan2) and back (where the search's first
// amplitude evaluation rebuilds the overlaps)
int launch_findk0_finish(const float* peak, float2 guess, int nx, int ny, float dkx, float dky, int fitorder2,
                         float2* k0out, float2* k1out, cudaStream_t s, long long* launches);
struct K0SearchArgs {
  // per direction:
  const float2* pmap[kMaxDirs];    // [ny][nx] overlap map of orders (0, fitorder2), built at k1
  const double* sumxy[kMaxDirs];   // [2] sum |X|^2, sum |Y|^2 of that build
  const float2* k0find[kMaxDirs];  // findk0's k0 (the lines start at its angle and magnitude)
  float2* k0fit[kMaxDirs];         // out: the fitted k0
  double* slot[kMaxDirs];          // out: XStarY re, im, sum |X|^2, sum |Y|^2 at the fitted k0
  int* info;                       // [0] += candidates evaluated; [1] |= 1 line cache exceeded, 2 batch limit
  int ndirs, nx, ny, fitorder2;
  float dxy, delta_angle, delta_mag;
};
// whether the search's phase tables fit a CTA's shared memory at this size
bool k0_search_supported(int nx, int ny);
// one thread-block cluster (8 CTAs) per direction, all directions at once:
// both line searches, their parabola fits and the amplitude at the fitted k0
// (fitk0andmodamps, gpuFunctionsImpl.cu:874-1020)
int launch_k0_search(const K0SearchArgs& a, cudaStream_t s, long long* launches);

// Modulation amplitudes of the last fit and the Wiener-filter weights derived
// from them, in device memory: the filter reads them there, so a volume whose
// fit needs no host decision runs without a host round trip.  Index d *
// norders + o.
struct FitDev {
  float2 amp[kMaxDirs * kMaxOrders];
  float ampmag2[kMaxDirs * kMaxOrders];  // |amp|^2
  float termw[kMaxDirs * kMaxOrders];    // |amp|^2 / noisevar; order 0: 1 / noisevar
};
struct FitFinishArgs {
  int ndirs, norders;
  int chain2d;       // nz == 1: amp[o] *= amp[o - 1] for o >= 2 (cudaSirecon.cpp:450-452)
  int nforce;        // forcemodamp values (cudaSirecon.cpp:453-464); 0: none
  float forceamp[kMaxOrders];
  int fitallphases;  // 0: orders >= 2 take order * phase of order 1 (cudaSirecon.cpp:465-482)
  float noisevar[kMaxDirs * kMaxOrders];
  float rnv[kMaxDirs * kMaxOrders];  // 1 / noisevar
};
// The no-search branch of the modamp fit (findrealspacemodamp at the known k0
// for every direction and order, cudaSirecon.cpp:409-492) finished on the
// device: slots[(d * norders + o) * 4 + {0, 1, 2}] = XStarY re, im and
// sum |X|^2 of order o (o >= 1) -> FitDev.
int launch_fit_finish(const double* slots, const FitFinishArgs& a, FitDev* out, cudaStream_t s, long long* launches);
// Host-fitted amplitudes (after a k0 search) -> FitDev, through the kernel's
// arguments.
struct AmpList {
  float2 amp[kMaxDirs * kMaxOrders];
};
int launch_set_fit(const AmpList& amps, const FitFinishArgs& a, FitDev* out, cudaStream_t s, long long* launches);

// ---------------------------------------------------------------- assembly
struct FilterArgs {
  float2* bands;         // bands of direction dir [nph][nz][ny][nxh]
  int dir, ndirs, norders, nx, ny, nz;
  float dkx, dky, rdistcutoff, apocutoff, zapocutoff, wiener2;
  int zdc[kMaxOrders];
  float2 k0[kMaxDirs];
  float noisevar[kMaxDirs * kMaxOrders];
  const FitDev* fit;     // modulation amplitudes and term weights (device)
  int suppress, supp_radius, dampen0, nokz0, filteroverlaps, apodizeoutput, bessel;
  OTFView otf;
};
int launch_filter(const FilterArgs& a, cudaStream_t s, long long* launches);

// Pattern vectors of every direction, by value (1/um)
struct K0List {
  float2 k[kMaxDirs];
};

struct AssembleArgs {
  const float2* bands;  // all directions [ndirs][nph][nz][ny][nxh]
  int ndirs, norders, nphases, nx, ny, nz;
  int X, Y, Z;          // zoomed output grid
  int zdc[kMaxOrders];  // in-band planes of each order after filtering
  const float2* ex;     // [ndirs*norders][X] phase-ramp factors along x
  const float2* ey;     // [ndirs*norders][Y]
  float2* T;            // scratch: [maxslots][Y][nx]
  size_t tcap;          // capacity of T in complex elements
  float2* S;            // [Z][Y][X]
  float* out;           // [Z][Y][X]
  void* tables;         // device slot tables (assemble_tables_bytes), uploaded by assemble_tables_upload
};
// The slot tables of an assembly (which band planes are summed into which
// output plane) depend only on the shape and the in-band plane counts; they
// are uploaded once and reused by every launch_assemble of that geometry.
size_t assemble_tables_bytes(const AssembleArgs& a);
// Writes the tables of `a` into a.tables (synchronous copy; call outside the
// timed/captured work, again whenever zdc changes).
int assemble_tables_upload(const AssembleArgs& a);
int launch_assemble(const AssembleArgs& a, cudaStream_t s, long long* launches);
// Filter and assembly in one pass: the Wiener filter of every direction
// applied in the assembly's band load (the bands are left unfiltered in
// memory).  Available for 3 directions, 2 or 3 orders, one OTF for all
// directions, zoomed y lengths 256/512/1024 and OTF lookups that stay inside
// the table; returns -10 (nothing launched) otherwise.
bool assemble_filter_fusable(const AssembleArgs& a, const FilterArgs& f, bool one_otf);
int launch_assemble_filtered(const AssembleArgs& a, const FilterArgs& f, bool one_otf, cudaStream_t s,
                             long long* launches);

// Phase-ramp tables for assembly: ex[d*no+o][j] = exp(i fact pi (j - X/2) o k0x_d dxyz),
// ey likewise along y (computed in double precision).
int launch_ramp_tables(const K0List& k0, int ndirs, int norders, int X, int Y, float dxyz, float fact, float2* ex,
                       float2* ey, cudaStream_t s, long long* launches);

// FFT-engine self test on `nlines` lines of length n (in place, device memory)
int launch_fft_selftest(float2* data, int n, int nlines, int inverse, int columns, cudaStream_t s);

// L2 flush helper for timing
int launch_fill(float* buf, size_t n, float v, cudaStream_t s, long long* launches);

}  // namespace simrecon
