/*
 * cudasirecon_gb300 -- C ABI of libcudasirecon.so (drop-in for the SR_* entry
 * points of scopetools/cudasirecon, src/cudaSirecon/interface.cpp).
 *
 * The twelve SR_* functions keep the reference's names, argument meaning and
 * call order; each declaration below cites the reference entry point it
 * replaces.  ReconParams and ImageParams keep the reference's member order
 * and types (src/cudaSirecon/cudaSireconImpl.h:104-195) because
 * SR_getReconParams / SR_getImageParams hand out references into the object
 * and callers read and write those structs in place.
 *
 * Additions (no reference counterpart): SR_delete, SR_getLastError,
 * SR_clearError, SR_setRawU16, the SRX_* performance/introspection calls.
 *
 * Errors never cross the ABI as C++ exceptions and the library never calls
 * exit(): a failing call records a message readable with SR_getLastError()
 * (thread-local) and, for constructors, returns NULL.
 *
 * Threading: one SIM_Reconstructor may be used by one host thread at a time;
 * distinct handles are independent (each owns its CUDA stream and device
 * memory) and may be used concurrently from different threads.
 */
#ifndef CUDASIRECON_GB300_H
#define CUDASIRECON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#include <string>
#include <vector>

/* Overall image reconstruction parameters (cudaSireconImpl.h:104-178). */
struct ReconParams {
  float k0startangle, linespacing;
  float na, nimm;
  int ndirs, nphases, norders_output;
  int norders;
  float* phaseSteps;
  bool bTwolens;
  bool bFastSIM;
  bool bBessel;
  float BesselNA;
  float BesselLambdaEx;
  float deskewAngle;
  int extraShift;
  bool bNoRecon;
  unsigned cropXYto;
  bool bWriteTitle;
  float otfcutoff;
  float zoomfact;
  int z_zoom;
  int nzPadTo;
  float explodefact;
  bool bFilteroverlaps;
  int recalcarrays;
  int napodize;
  int bSearchforvector;
  int bUseTime0k0;
  int apodizeoutput;
  float apoGamma;
  int bSuppress_singularities;
  int suppression_radius;
  bool bDampenOrder0;
  int bFitallphases;
  int do_rescale;
  bool equalizez;
  bool equalizet;
  bool bNoKz0;
  float wiener, wienerInr;
  std::vector<float> forceamp;
  std::vector<float> k0angles;
  int nxotf, nyotf, nzotf;
  float dzPSF;
  float dkzotf, dkrotf;
  bool bRadAvgOTF;
  bool bOneOTFperAngle;
  int bFixdrift;
  float drift_filter_fact;
  float constbkgd;
  int bBgInExtHdr;
  int bUsecorr;
  std::string corrfiles;
  float readoutNoiseVar;
  float electrons_per_bit;
  int bMakemodel;
  int bSaveSeparated;
  std::string fileSeparated;
  int bSaveAlignedRaw;
  std::string fileRawAligned;
  int bSaveOverlaps;
  std::string fileOverlaps;
  bool bTIFF;
  std::string ifiles;
  std::string ofiles;
  std::string otffiles;
};

/* Image geometry (cudaSireconImpl.h:179-195). */
struct ImageParams {
  int nx;
  int nx_raw;
  int ny;
  int nz;
  int nz0;
  short nwaves;
  short wave[5];
  short ntimes;
  unsigned short curTimeIdx;
  float dxy;
  float dz;
  float dz_raw;
  float inscale;
};

class SIM_Reconstructor;
extern "C" {
#define SR_PARAMS_REF(T) T&
#else
typedef struct SIM_Reconstructor SIM_Reconstructor;
typedef struct ReconParams ReconParams;
typedef struct ImageParams ImageParams;
#define SR_PARAMS_REF(T) T*
#endif

/* --- the reference's twelve entry points --------------------------------- */

/* interface.cpp:13-17.  nImages = ndirs*nphases*nz raw planes; the config
 * file uses the reference's key=value option names and must name the OTF
 * TIFF with otf-file=.  Returns NULL on error (see SR_getLastError). */
SIM_Reconstructor* SR_new_from_shape(int nx, int ny, int nImages, const char* configFileName);

/* interface.cpp:19-25.  raw_data is [nz][ny][nx] float (nz = total planes),
 * sections in the reference's order (Angle->Z->Phase, or Z->Angle->Phase
 * with fastSI). */
void SR_setRaw(SIM_Reconstructor* sr, const float* raw_data, int nx, int ny, int nz);

/* interface.cpp:26-29: bleach correction of the loaded volume. */
void SR_loadAndRescaleImage(SIM_Reconstructor* sr, int it, int iw);

/* interface.cpp:30-33 */
void SR_setCurTimeIdx(SIM_Reconstructor* sr, int it);

/* interface.cpp:34-37: k0 / modamp fit, Wiener filter and band assembly. */
void SR_processOneVolume(SIM_Reconstructor* sr);

/* interface.cpp:38-41: result is (zoom*nx)*(zoom*ny)*(zzoom*nz) floats. */
void SR_getResult(SIM_Reconstructor* sr, float* result);

/* interface.cpp:42-45 / 47-50: references into the object. */
SR_PARAMS_REF(ReconParams) SR_getReconParams(SIM_Reconstructor* sr);
SR_PARAMS_REF(ImageParams) SR_getImageParams(SIM_Reconstructor* sr);

/* interface.cpp:54-57: construct from a cudasirecon command line
 * (input output otf [--options] [-c config]). */
SIM_Reconstructor* SR_new_from_argv(int argc, char** argv);

/* interface.cpp:59-62: read time point it of the input file(s). */
void SR_setFile(SIM_Reconstructor* sr, int it, int iw);

/* interface.cpp:63-66: write the result of time point it. */
void SR_writeResult(SIM_Reconstructor* sr, int it, int iw);

/* interface.cpp:67-70 */
void SR_closeFiles(SIM_Reconstructor* sr);

/* --- additions (no counterpart in the reference) -------------------------- */

/* Destroy a handle and release its device memory (the reference leaks). */
void SR_delete(SIM_Reconstructor* sr);

/* Last error of the calling thread ("" if none); SR_clearError resets it. */
const char* SR_getLastError(void);
void SR_clearError(void);

/* Integer camera readout: raw_data is [nz][ny][nx] uint16.  Same result as
 * SR_setRaw of the same values converted to float. */
void SR_setRawU16(SIM_Reconstructor* sr, const uint16_t* raw_data, int nx, int ny, int nz);

/* Number of time points of a file-backed reconstructor (getNTimes). */
int SR_getNTimes(SIM_Reconstructor* sr);

/* Fitted pattern vectors (1/um, [ndirs][2]) and modulation amplitudes
 * ([ndirs][norders] complex as float pairs) of the last processed volume. */
void SRX_getFit(SIM_Reconstructor* sr, float* k0, float* amps);

/* Copy the separated (before processOneVolume's filter) or current bands of
 * direction dir, band b, as complex [nz][ny][nx/2+1] (float pairs).
 * Stage 0 = after separation (SRX_prepare), 1 = current device contents. */
int SRX_prepare(SIM_Reconstructor* sr);
int SRX_getBand(SIM_Reconstructor* sr, int dir, int b, float* out);

/* Device-resident timing: run the full device pipeline (ingest of the staged
 * raw planes, bleach correction, fit, filter, assembly) `steps` times from
 * the raw data already in device memory, flushing L2 between steps, and
 * return the summed device time in ms (CUDA events on the handle's stream). */
int SRX_benchDevice(SIM_Reconstructor* sr, int steps, double* total_ms);

/* Per-stage profiling: when enabled, every stage is bracketed by CUDA events
 * on the handle's stream.  SRX_getProfile writes a JSON object
 * {"stage": {"ms": t, "launches": n}, ...} accumulated since the last reset. */
void SRX_setProfiling(SIM_Reconstructor* sr, int on);
int SRX_getProfile(SIM_Reconstructor* sr, char* json, int maxlen);
void SRX_resetProfile(SIM_Reconstructor* sr);

/* No counterpart in the reference.  Fit work executed since the handle was
 * created: out3[0] overlap builds (the reference's makeoverlaps), out3[1]
 * reductions over an overlap pair (modamp evaluations, the k0
 * cross-correlation), out3[2] k0 searches (findk0 + fitk0andmodamps). */
void SRX_fitCounts(SIM_Reconstructor* sr, long long* out3);

/* No counterpart in the reference.  FFT plan autotuning.  The library's FFT
 * call sites (site ids: 0 ingest x, 1 ingest y, 2 separation z, 3 overlap x,
 * 4 overlap y, 5/6 cross-correlation rows/columns, 7/8/9 assembly y/x/z,
 * 10 makeotf) run a length either with the register path (lengths 32, 48,
 * 64, 96, 128, 256, 512, 1024) or with the shared-memory Stockham stages.
 * SRX_tuneFFT runs the handle's staged raw stack (SR_setRaw first) once per
 * choice and repeat for every site and length its volume uses, times the
 * site's kernel with CUDA events, and records the faster choice in the plan
 * cache file (SIMRECON_FFT_PLAN_CACHE, else ~/.cache/cudasirecon_gb300/
 * fft_plans.tsv; one line per GPU model, site and length) that every process
 * then uses.  It leaves the handle's fit state as after processing that stack
 * at time point 0.  Returns the length of the JSON report written to json
 * (truncated to maxlen), or -1 (SR_getLastError).
 * SRX_fftPlanChoice: 1 register path, 0 Stockham, -1 bad site, with the
 * choice's source ("tuned", "built-in", "environment", "stockham-only"). */
int SRX_tuneFFT(SIM_Reconstructor* sr, int reps, char* json, int maxlen);
int SRX_fftPlanChoice(int site, int n, char* source, int maxlen);

/* No counterpart in the reference.  What the last SR_processOneVolume
 * returned in the reference's terms: 1 reconstructed, 0 stopped after the
 * debug dumps (saveprefiltered / savealignedraw / saveoverlaps), when the
 * reference's driver writes no result for that time point. */
int SRX_lastProcessResult(SIM_Reconstructor* sr);

/* Wiener filter placement (default on): inside the band load of the
 * assembly's y transform where supported (3 directions, one OTF, zoomed y
 * 256/512/1024), else -- or with on = 0 -- as its own in-place pass over the
 * bands, as the reference's filterbands does.  Both give the same volume
 * within float rounding.  After SR_processOneVolume the band contents
 * (SRX_getBand) are unspecified. */
void SRX_setFilterFusion(SIM_Reconstructor* sr, int on);

/* k0 search placement (default on): on the device -- findk0's peak
 * refinement and fitk0andmodamps' angle and magnitude line searches run as
 * kernels (one thread-block cluster per direction), with one host
 * synchronisation per volume instead of one per candidate batch -- or, with
 * on = 0, driven from the host.  Both visit the same float32 angles and
 * magnitudes (cudaSirecon.cpp:296-408, gpuFunctionsImpl.cu:306-372,
 * 874-1044); the fitted k0 agree within float rounding of the start angle.
 * Bessel mode, the overlap debug dump, later time points of a series
 * (which may fall back to time 0's k0) and images larger than 1024 x 1024
 * (whose candidate batches are better spread over the whole GPU) use the
 * host-driven search. */
void SRX_setDeviceK0Search(SIM_Reconstructor* sr, int on);

/* Number of this library's kernels launched since the handle was created. */
long long SRX_kernelLaunches(SIM_Reconstructor* sr);

/* Page-lock (pin) / unpin a caller's host buffer so that SR_setRaw* and
 * SR_getResult copies run at full host-link bandwidth.  Return 0 on success. */
int SRX_pinHost(void* ptr, size_t bytes);
/* Test hook: transform `nlines` complex lines of length n (interleaved
 * float pairs, in place) with the library's FFT engine; inverse != 0 for
 * e^{+i}; columns != 0 stages the lines interleaved (strided-axis layout).
 * Unnormalised, like cuFFT.  Returns 0 on success. */
int SRX_fftSelfTest(float* data, int n, int nlines, int inverse, int columns);

/* No counterpart in the reference.  The same line transform for callers
 * that must not allocate device memory (real-time acquisition loops, where an
 * allocation's implicit synchronisation stalls the camera pipeline, and
 * plug-in hosts that own the device's memory): `in` and `out` are host arrays
 * of nlines x n complex values; the device staging buffer and twiddle table
 * live in a fixed 16 MiB file-scope device array, so no cudaMalloc/cudaFree
 * is made.  A synchronous host-to-host call (blocking copies and launches on
 * the default stream).  At most 2 Mi complex values per call and n <= 8192
 * (in the column layout n <= 7264, the per-CTA shared-memory limit); larger
 * requests return -1 without running and leave `out` unwritten.  Calls share
 * the array: calls that overlap on the GPU race.  The first call on a device
 * looks up the array's address; make it before any stream capture.  Returns
 * 0 on success; SRX_fftLinesNoAllocError() describes a failure. */
int SRX_fftLinesNoAlloc(const float* in, float* out, int n, int nlines, int inverse, int columns);
const char* SRX_fftLinesNoAllocError(void);
int SRX_unpinHost(void* ptr);

/* No counterpart in the reference.  Page-locked host memory allocated by the
 * CUDA runtime (cudaHostAlloc), for raw stacks and results: on GB300 (Grace,
 * NVLink-C2C) copies from it run at the link's full rate in both directions
 * at once, about 35 % faster than from ordinary memory page-locked with
 * SRX_pinHost.  NULL on failure (SR_getLastError); free with SRX_hostFree. */
void* SRX_hostAlloc(size_t bytes);
void SRX_hostFree(void* ptr);

/* No counterpart in the reference.  Free and total device memory of the
 * current device (cudaMemGetInfo); returns 0 on success. */
int SRX_deviceMemInfo(size_t* free_bytes, size_t* total_bytes);

/* No counterpart in the reference.  Reconstruct n volumes of a time series:
 * for volume i the same as SR_setRaw(raws[i]) (SR_setRawU16 when
 * raw_is_u16), SR_loadAndRescaleImage(t0+i, 0), SR_setCurTimeIdx(t0+i),
 * SR_processOneVolume, SR_getResult(outs[i]) -- the results are identical --
 * but the upload of volume i+1 and the download of volume i-1 run on their
 * own streams while volume i is computed.  raws[i] and outs[i] are host
 * buffers of the SR_setRaw / SR_getResult sizes; page-lock them
 * (SRX_pinHost) for the copies to overlap.  Entries may repeat, except that
 * an output buffer must not be reused within two consecutive volumes.
 * Returns 0 on success, -1 on error (SR_getLastError). */
int SRX_processSeries(SIM_Reconstructor* sr, const void* const* raws, int raw_is_u16, float* const* outs, int n,
                      int t0);

/* No counterpart in the reference.  A request server for many volumes of
 * different shapes and acquisition configurations: worker threads run the
 * SR_* flow on pooled handles (one per configuration, shape and worker, each
 * with its own CUDA stream), so requests overlap on the GPU; the handles are
 * admitted within hbm_budget_bytes of device memory (idle ones evicted least
 * recently used first, else the request waits for a busy one to finish).  A configuration is a reference-style config file
 * that names its OTF (otf-file=).  Each request is one volume in the
 * SR_setRaw layout, processed as a time-0 volume (k0 fitted), its result
 * written in the SR_getResult layout; raw and out stay the caller's and must
 * remain valid until SRX_serverWait returns for the ticket.  Submit returns a
 * ticket (or -1); Wait blocks until that request is done, returns 0 or -1
 * (SR_getLastError) and gives the latency from submission to the result in
 * host memory.  Destroy finishes the queued requests first. */
typedef struct SRX_Server SRX_Server;
SRX_Server* SRX_serverCreate(int workers, size_t hbm_budget_bytes);
int SRX_serverAddConfig(SRX_Server* s, const char* config_path);
long long SRX_serverSubmit(SRX_Server* s, int config, int nx, int ny, int nimages, const void* raw, int raw_is_u16,
                           float* out);
int SRX_serverWait(SRX_Server* s, long long ticket, double* latency_ms);
/* Create `count` handles for one shape ahead of its requests (a handle is
 * created otherwise by the first request that finds none idle, which then
 * pays for the device allocation).  Returns how many were created. */
int SRX_serverReserve(SRX_Server* s, int config, int nx, int ny, int nimages, int count);
/* A batch of standalone acquisitions of uneven shapes and configurations (2D
 * and 3D mixed), each processed exactly like a submitted request.  Items are
 * grouped by (config, shape); each group runs in chunks on pooled handles, a
 * chunk's volumes back to back with the upload of the next and the download
 * of the previous overlapped with the computation, and chunks of different
 * shapes run concurrently on the workers' streams, largest first.  Blocks
 * until every item is done.  Returns 0, or -1 (SR_getLastError: the first
 * failing item's error; the other items are still processed). */
typedef struct SRX_BatchItem {
  int config;          /* SRX_serverAddConfig id */
  int nx, ny, nimages; /* the SR_new_from_shape shape */
  const void* raw;     /* [nimages][ny][nx], uint16 when raw_is_u16 else float */
  int raw_is_u16;
  float* out;          /* the SR_getResult layout */
} SRX_BatchItem;
int SRX_serverRunBatch(SRX_Server* s, const SRX_BatchItem* items, int n);
/* The schedule SRX_serverRunBatch would use for these items with `workers`
 * workers, without running it (no GPU needed): chunk_of_item[i] = the chunk
 * (in execution order) of item i; returns the number of chunks, or -1. */
int SRX_batchPlan(const SRX_BatchItem* items, int n, int workers, int* chunk_of_item);
/* Device bytes reserved against the budget by the pooled handles: a handle's
 * bytes are planned from its shape and configuration before it is created
 * (every buffer it can come to hold) and a request waits until they fit, so
 * this never exceeds hbm_budget_bytes.  DeviceBytesHeld: what the handles
 * actually hold now (at most the reserved bytes). */
size_t SRX_serverDeviceBytes(SRX_Server* s);
size_t SRX_serverDeviceBytesHeld(SRX_Server* s);
/* Both figures taken together (a consistent pair: held <= reserved). */
void SRX_serverMemory(SRX_Server* s, size_t* reserved, size_t* held);
/* The bytes admission reserves for a handle of this configuration and shape
 * (planned without allocating); 0 on error (SR_getLastError). */
size_t SRX_serverPlannedBytes(SRX_Server* s, int config, int nx, int ny, int nimages);
/* k0 kept per acquisition configuration (off by default).  With it on, the
 * first submitted request of the configuration to finish searches k0 as
 * usual and the server records it; every later submitted request of that
 * configuration, of any shape, is processed like a later time point of a
 * series with time-0 k0 reuse (cudaSirecon.cpp:296-301: k0 kept, modamps
 * fitted) -- the same as SR_setRaw -> SR_loadAndRescaleImage(0) ->
 * SR_setCurTimeIdx(1) -> SR_processOneVolume on a handle whose time point 0
 * fitted that k0.  Turning it on clears the record.  Batches
 * (SRX_serverRunBatch) always search.  RecordedK0 copies 2 floats per
 * direction (k0x, k0y in 1/um) and returns 1, or returns 0 if none yet. */
int SRX_serverSetK0Reuse(SRX_Server* s, int config, int on);
int SRX_serverRecordedK0(SRX_Server* s, int config, float* k0, int ndirs);
/* Handles created, and handles deleted to stay within the budget, so far. */
void SRX_serverCounters(SRX_Server* s, long long* created, long long* evicted);
/* How often a request waited for busy handles to release device memory. */
long long SRX_serverAdmissionWaits(SRX_Server* s);
void SRX_serverDestroy(SRX_Server* s);

/* makeotf.  The reference's makeotf is a program, not a library call
 * (src/otf/radialft.cpp:82-434); these replace it:
 *
 * SRX_makeotfMain: the program itself, with the reference's command line
 * (radialft.cpp:1381-1553: `makeotf psf otf [switches]`, TIFF or MRC/DV in,
 * the same format out).  Returns 0 on success, else -1 with the message in
 * SR_getLastError().
 *
 * SRX_makeOTF: the same computation on a PSF stack in host memory, float
 * [nsections][ny][nx] with the phase fastest (section = z*nphases + phase).
 * `args` are makeotf's switches without file names (e.g. "-angle", "-0.8",
 * "-ls", "0.2035", "-xyres", "0.08", "-zres", "0.125").  The result is the
 * float array the program writes to its OTF TIFF, [dims[2]][dims[1]][dims[0]]
 * with dims = {width = 2*nz, height = nx/2+1, depth = number of bands}
 * (width 2*(nx/2+1), height 1 for a 2D PSF).  out may be NULL to query dims;
 * out_floats is its capacity.  Returns 0 on success, -1 on error. */
int SRX_makeotfMain(int argc, char** argv);
int SRX_makeOTF(const float* psf, int nx, int ny, int nsections, int nargs, const char* const* args, float* out,
                size_t out_floats, int* dims);

#ifdef __cplusplus
}
#endif
#undef SR_PARAMS_REF

#endif /* CUDASIRECON_GB300_H */
