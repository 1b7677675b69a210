// Reference harness: drives the reference's OWN GPU functions and kernels
// (src/cudaSirecon/gpuFunctionsImpl.cu, compiled unmodified from the staged
// reference sources) through a restatement of the host orchestration of
// src/cudaSirecon/cudaSirecon.cpp, which cannot be compiled here (it needs
// Boost.program_options/filesystem, libtiff and Priism IVE).
//
// TEST INFRASTRUCTURE ONLY.  It is the results-parity target for the GPU
// product (golden fixtures are generated by running it on a GB300) and the
// "reference CUDA build" arm of bench.py.  The product never links it.
//
// Every function below restates one piece of cudaSirecon.cpp and cites the
// lines it follows.  Parameters are filled from a key=value text with the
// reference's boost::program_options defaults (cudaSirecon.cpp:913-1070 over
// SetDefaultParams cudaSirecon.cpp:16-72).

#include "cudaSireconImpl.h"
#include "gpuFunctions.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sstream>
#include <vector>
#include <map>

// Symbols that gpuFunctionsImpl.cu takes from cudaSirecon.cpp (cudaSirecon.cpp:726-745).
float get_phase(cuFloatComplex b) { return atan2(b.y, b.x); }
float cmag(cuFloatComplex a) { return (sqrt(a.x * a.x + a.y * a.y)); }
cuFloatComplex cmul(cuFloatComplex a, cuFloatComplex b)
{
  cuFloatComplex r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

// allocateOTFs, allocateImageBuffers and allocSepMatrixAndNoiseVarFactors
// live in cudaSirecon.cpp (101-136, 719-723); restated here.
void allocateOTFs(ReconParams* pParams, int sizeOTF, std::vector<std::vector<GPUBuffer> >& otfs)
{
  otfs.clear();
  unsigned short nDirsOTF = pParams->bOneOTFperAngle ? pParams->ndirs : 1;
  otfs.resize(nDirsOTF);
  for (int dir = 0; dir < nDirsOTF; dir++)
    for (int i = 0; i < pParams->norders; ++i) {
      GPUBuffer buff;
      buff.resize(sizeOTF * sizeof(cuFloatComplex));
      otfs[dir].push_back(buff);
    }
}

void allocateImageBuffers(const ReconParams& params, const ImageParams& imgParams, ReconData* data)
{
  data->savedBands.clear();
  data->savedBands.reserve(params.ndirs);
  for (int i = 0; i < params.ndirs; ++i) {
    data->savedBands.push_back(std::vector<GPUBuffer>());
    data->savedBands[i].reserve(params.nphases);
    for (int j = 0; j < params.nphases; ++j)
      data->savedBands[i].push_back(
          GPUBuffer((imgParams.nx / 2 + 1) * imgParams.ny * imgParams.nz0 * sizeof(cuFloatComplex), 0));
  }
  for (int i = 0; i < params.ndirs; ++i)
    for (int j = 0; j < params.nphases; ++j) data->savedBands[i][j].setToZero();
}

void allocSepMatrixAndNoiseVarFactors(const ReconParams& params, ReconData* reconData)
{
  reconData->sepMatrix.resize(params.nphases * (params.norders * 2 - 1));
  reconData->noiseVarFactors.resize(params.ndirs * params.norders, 1.0f);
}

namespace {

struct Harness {
  ReconParams p;
  ImageParams ip;
  ReconData d;
  DriftParams drift;
  int zoffset = 0;
  std::vector<float> raw;   // [nImages][ny][nx] as given to setRaw
  int nImages = 0;
  // executed fit work (for the measurement's algorithmic-bytes model): each
  // findrealspacemodamp with redo builds the overlaps once and reduces them
  // once; a k0 search (findk0 + fitk0andmodamps) runs an unobserved number
  // of both inside the reference's own functions and is only counted
  long long n_overlap_builds = 0, n_reductions = 0, n_searches = 0;
  // the overlap pair right after findk0, per direction (the reference's
  // saveoverlaps dump point), when capturing is on
  bool capture_overlaps = false;
  std::vector<std::vector<float>> captured;  // [dir][2 * nx * ny * nz0 * 2 floats]
  std::vector<float> section_bg;  // per raw section of a time point (bBgInExtHdr)
};

// SetDefaultParams, cudaSirecon.cpp:16-72, then the program_options defaults
// of cudaSirecon.cpp:913-1009 (those win because notify() writes them).
void set_defaults(ReconParams* pp, ImageParams* ip)
{
  ReconParams& p = *pp;
  p.k0startangle = 1.648f;   // po angle0
  p.linespacing = 0.172f;    // po ls
  p.na = 1.2f;               // po na
  p.nimm = 1.33f;            // po nimm
  p.ndirs = 3;
  p.nphases = 5;
  p.phaseSteps = 0;
  p.norders_output = 0;
  p.bTwolens = false;
  p.bFastSIM = false;
  p.bBessel = false;
  p.BesselNA = 0.144f;
  p.BesselLambdaEx = 0.488f;
  p.deskewAngle = 0.f;
  p.extraShift = 0;
  p.bNoRecon = false;
  p.cropXYto = 0;
  p.bWriteTitle = false;
  p.otfcutoff = 0.006f;
  p.zoomfact = 2.f;
  p.z_zoom = 1;
  p.nzPadTo = 0;
  p.explodefact = 1.f;
  p.bFilteroverlaps = 1;
  p.recalcarrays = 1;
  p.napodize = 10;
  p.forceamp.assign(1, 0.f);
  p.bSearchforvector = 1;
  p.bUseTime0k0 = 1;
  p.apodizeoutput = 2;       // gammaApo always present (cudaSirecon.cpp:1040-1045)
  p.apoGamma = 1.f;
  p.bSuppress_singularities = 1;
  p.suppression_radius = 10;
  p.bDampenOrder0 = false;
  p.bFitallphases = 1;
  p.do_rescale = 1;
  p.equalizez = false;
  p.equalizet = false;
  p.bNoKz0 = false;
  p.wiener = 0.01f;
  p.bRadAvgOTF = false;
  p.bOneOTFperAngle = false;
  p.dzPSF = 0.15f;
  p.bFixdrift = 0;
  p.drift_filter_fact = 0.f;
  p.constbkgd = 0.f;
  p.bBgInExtHdr = 0;
  p.bUsecorr = 0;
  p.electrons_per_bit = 0.6528f;
  p.readoutNoiseVar = 32.42f;
  p.bMakemodel = 0;
  p.bSaveSeparated = 0;
  p.bSaveAlignedRaw = 0;
  p.bSaveOverlaps = 0;
  p.bTIFF = true;
  ip->dxy = 0.1f;
  ip->dz = 0.2f;
  ip->wave[0] = 530;
  ip->ntimes = 1;
  ip->curTimeIdx = 0;
}

bool parse_bool(const std::string& v)
{
  return v == "1" || v == "true" || v == "yes" || v == "on" || v.empty();
}

// The config-file keys of setupProgramOptions (cudaSirecon.cpp:913-1009) that
// the recon path reads.  Values are stored exactly as boost::program_options
// stores them (e.g. k0searchAll -> bUseTime0k0, norescale -> do_rescale).
void apply_config(Harness* h, const char* text)
{
  ReconParams& p = h->p;
  ImageParams& ip = h->ip;
  std::istringstream in(text ? text : "");
  std::string line;
  while (std::getline(in, line)) {
    size_t hash = line.find('#');
    if (hash != std::string::npos) line = line.substr(0, hash);
    size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    auto trim = [](std::string s) {
      size_t a = s.find_first_not_of(" \t\r\n");
      size_t b = s.find_last_not_of(" \t\r\n");
      return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    };
    std::string k = trim(line.substr(0, eq));
    std::string v = trim(line.substr(eq + 1));
    float f = (float)atof(v.c_str());
    int i = atoi(v.c_str());
    if (k == "ndirs") p.ndirs = i;
    else if (k == "nphases") p.nphases = i;
    else if (k == "nordersout") p.norders_output = i;
    else if (k == "angle0") p.k0startangle = f;
    else if (k == "ls") p.linespacing = f;
    else if (k == "na") p.na = f;
    else if (k == "nimm") p.nimm = f;
    else if (k == "wiener") p.wiener = f;
    else if (k == "otfcutoff") p.otfcutoff = f;
    else if (k == "zoomfact") p.zoomfact = f;
    else if (k == "zzoom") p.z_zoom = i;
    else if (k == "background") p.constbkgd = f;
    else if (k == "forcemodamp") {
      p.forceamp.clear();
      std::istringstream vs(v);
      float x;
      while (vs >> x) p.forceamp.push_back(x);
    }
    else if (k == "k0angles") {
      p.k0angles.clear();
      std::istringstream vs(v);
      std::string tok;
      while (std::getline(vs, tok, ',')) if (!tok.empty()) p.k0angles.push_back(strtod(tok.c_str(), NULL));
    }
    else if (k == "otfRA") p.bRadAvgOTF = parse_bool(v);
    else if (k == "otfPerAngle") p.bOneOTFperAngle = parse_bool(v);
    else if (k == "fastSI") p.bFastSIM = parse_bool(v);
    else if (k == "k0searchAll") p.bUseTime0k0 = i;
    else if (k == "norescale") p.do_rescale = i;
    else if (k == "equalizez") p.equalizez = parse_bool(v);
    else if (k == "equalizet") p.equalizet = parse_bool(v);
    else if (k == "dampenOrder0") p.bDampenOrder0 = parse_bool(v);
    else if (k == "nosuppress") p.bSuppress_singularities = i;
    else if (k == "nokz0") p.bNoKz0 = parse_bool(v);
    else if (k == "gammaApo") p.apoGamma = f;
    else if (k == "explodefact") p.explodefact = f;
    else if (k == "nofilterovlps") p.bFilteroverlaps = parse_bool(v);
    else if (k == "bessel") p.bBessel = parse_bool(v);
    else if (k == "besselExWave") p.BesselLambdaEx = f;
    else if (k == "besselNA") p.BesselNA = f;
    else if (k == "deskew") p.deskewAngle = f;
    else if (k == "deskewshift") p.extraShift = i;
    else if (k == "noRecon") p.bNoRecon = parse_bool(v);
    else if (k == "cropXY") p.cropXYto = (unsigned)i;
    else if (k == "bgInExtHdr") p.bBgInExtHdr = i;
    else if (k == "xyres") ip.dxy = f;
    else if (k == "zres") ip.dz = f;
    else if (k == "zresPSF") p.dzPSF = f;
    else if (k == "wavelength") ip.wave[0] = (short)i;
  }
}

// notGoodDimension / findOptimalDimension, cudaSirecon.cpp:76-97
bool not_good_dimension(unsigned num)
{
  if (num == 2 || num == 3 || num == 5 || num == 7) return false;
  else if (num % 2 == 0) return not_good_dimension(num / 2);
  else if (num % 3 == 0) return not_good_dimension(num / 3);
  else if (num % 5 == 0) return not_good_dimension(num / 5);
  else if (num % 7 == 0) return not_good_dimension(num / 7);
  else return true;
}

unsigned find_optimal_dimension(unsigned inSize, int step = -1)
{
  unsigned outSize = inSize;
  while (not_good_dimension(outSize)) outSize += step;
  return outSize;
}

// makematrix default branch, cudaSirecon.cpp:591-617 (the LAPACK branch is
// unreachable: phaseSteps is never set).
void makematrix_default(int nphases, int norders, float* sepMatrix)
{
  float phi = 2.0 * M_PI / nphases;
  for (int j = 0; j < nphases; ++j) {
    sepMatrix[0 * nphases + j] = 1.0;
    for (int order = 1; order < norders; ++order) {
      sepMatrix[(2 * order - 1) * nphases + j] = cos(j * order * phi);
      sepMatrix[2 * order * nphases + j] = sin(j * order * phi);
    }
  }
}

// setup() + setup_common(), cudaSirecon.cpp:1104-1115 and 1139-1261, with the
// TIFF branch of determine_otf_dimensions (1446-1482) and loadOTFs (1532-1569)
// reading the OTF from memory (pages of [height][width] floats).
void setup(Harness* h, int nx, int ny, int nImages, const float* otf, int otf_w, int otf_h, int otf_d)
{
  ReconParams& p = h->p;
  ImageParams& ip = h->ip;
  ReconData& d = h->d;
  ip.nx = nx;
  ip.nx_raw = nx;
  ip.ny = ny;
  ip.nwaves = 1;
  ip.nz = nImages / (ip.nwaves * p.nphases * p.ndirs);
  h->nImages = nImages;
  ip.nz0 = ip.nz;
  h->zoffset = 0;
  ip.dz_raw = 0;
  // setup_common's deskew and crop, cudaSirecon.cpp:1153-1170
  if (fabs(p.deskewAngle) > 0.) {
    if (p.deskewAngle < 0) p.deskewAngle += 180.;
    ip.nx = find_optimal_dimension(ip.nx_raw + ip.nz0 * fabs(cos(p.deskewAngle * M_PI / 180.)) * ip.dz / ip.dxy);
    ip.dz_raw = ip.dz;
    ip.dz *= fabs(sin(p.deskewAngle * M_PI / 180.));
  } else {
    ip.nx = ip.nx_raw;
    ip.dz_raw = 0;
  }
  if (p.cropXYto > 0 && p.cropXYto < (unsigned)ip.nx) ip.nx = p.cropXYto;

  p.norders = (p.norders_output != 0) ? p.norders_output : p.nphases / 2 + 1;

  // determine_otf_dimensions, TIFF branch (cudaSirecon.cpp:1446-1482)
  int nxotf_f = otf_w / 2, nyotf_f = otf_h, nzotf_f = otf_d;
  if (ip.nz == 1) {
    p.nxotf = nxotf_f;
    p.nyotf = p.bRadAvgOTF ? 1 : nyotf_f;
    p.nzotf = 1;
    p.dkrotf = 1 / (ip.dxy * (nxotf_f - 1) * 2);
    p.dkzotf = 1;
  } else if (p.bRadAvgOTF) {
    p.nzotf = nxotf_f;
    p.nxotf = nyotf_f;
    p.nyotf = 1;
    p.dkzotf = 1 / (p.dzPSF * p.nzotf);
    p.dkrotf = 1 / (ip.dxy * (p.nxotf - 1) * 2);
  } else {
    p.nzotf = nzotf_f / p.norders;
    p.nxotf = nxotf_f;
    p.nyotf = nyotf_f;
    p.dkzotf = 1 / (p.dzPSF * p.nzotf);
    p.dkrotf = 1 / (ip.dxy * p.nxotf);
  }
  d.sizeOTF = (size_t)p.nzotf * p.nxotf * p.nyotf;
  allocateOTFs(&p, d.sizeOTF, d.otf);
  // loadOTFs, TIFF branch (cudaSirecon.cpp:1540-1569)
  int nDirsOTF = p.bOneOTFperAngle ? p.ndirs : 1;
  size_t page = (size_t)otf_w * otf_h;
  for (int dir = 0; dir < nDirsOTF; dir++) {
    for (int i = 0; i < p.norders; i++) {
      if (ip.nz == 1 || p.bRadAvgOTF) {
        if (otf_d > i + dir * p.norders) {
          cudaMemcpy(d.otf[dir][i].getPtr(), otf + page * i, d.sizeOTF * sizeof(cuFloatComplex), cudaMemcpyHostToDevice);
        } else {
          cudaMemcpy(d.otf[dir][i].getPtr(), d.otf[0][0].getPtr(), d.otf[0][0].getSize(), cudaMemcpyDeviceToDevice);
        }
      } else {
        cudaMemcpy(d.otf[dir][i].getPtr(), otf + page * i * p.nzotf, d.sizeOTF * sizeof(cuFloatComplex), cudaMemcpyHostToDevice);
      }
    }
  }

  allocSepMatrixAndNoiseVarFactors(p, &d);
  makematrix_default(p.nphases, p.norders, &d.sepMatrix[0]);
  allocateImageBuffers(p, ip, &d);

  ip.inscale = 1.0 / (ip.nx * ip.ny * ip.nz0 * p.zoomfact * p.zoomfact * p.z_zoom * p.ndirs);
  d.k0 = std::vector<vector>(p.ndirs);
  d.k0_time0 = std::vector<vector>(p.ndirs);
  d.k0guess = std::vector<vector>(p.ndirs);
  float delta_angle = M_PI / p.ndirs;
  float k0magguess = 1.0 / p.linespacing;
  if (ip.nz > 1) {
    int nordersIn = p.nphases / 2 + 1;
    k0magguess /= nordersIn - 1;
  }
  for (int i = 0; i < p.ndirs; ++i) {
    float k0angleguess;
    if (p.k0angles.size() < (size_t)p.ndirs)
      k0angleguess = p.k0startangle + i * delta_angle;
    else
      k0angleguess = p.k0angles[i];
    d.k0guess[i].x = k0magguess * cos(k0angleguess);
    d.k0guess[i].y = k0magguess * sin(k0angleguess);
  }
  d.sum_dir0_phase0 = std::vector<double>(ip.nz * ip.nwaves);
  d.amp = std::vector<std::vector<cuFloatComplex> >(p.ndirs, std::vector<cuFloatComplex>(p.norders));
  for (int i = 0; i < p.ndirs; ++i) {
    d.amp[i][0].x = 1.0f;
    d.amp[i][0].y = 0.0f;
  }
  // bgAndSlope, constant-background branch (cudaSirecon.cpp:139-161)
  // sized for the raw planes: load_and_flatfield indexes them with the raw
  // width (constant values, so the reference's nx-sized arrays read the same)
  const int nbg = std::max(ip.nx, ip.nx_raw) * ip.ny;
  d.background.resize(sizeof(float) * nbg);
  d.slope.resize(sizeof(float) * nbg);
  for (int i = 0; i < nbg; i++) {
    ((float*)d.background.getPtr())[i] = p.constbkgd;
    ((float*)d.slope.getPtr())[i] = 1.0;
  }
  d.backgroundExtra = 0;
}

// loadImageData (cudaSirecon.cpp:1354-1435) with load_and_flatfield
// (1715-1731) and deskewOneSection (1733-1760): one synchronous
// host->device copy per plane, like the reference, which builds with OpenMP
// (src/CMakeLists.txt:55-64) and runs deskewOneSection's column loop on every
// host thread.  The per-section extra
// background of the bBgInExtHdr branch (1386-1393) comes from
// refh_set_section_backgrounds (the reference reads the MRC extended header).
void load_image_data(Harness* h)
{
  ReconParams& p = h->p;
  ImageParams& ip = h->ip;
  ReconData& d = h->d;
  const int nx_raw = ip.nx_raw, nx = ip.nx, ny = ip.ny;
  const int xdim = (nx / 2 + 1) * 2;
  float deskewFactor = 0;
  if (fabs(p.deskewAngle) > 0.0) deskewFactor = cos(p.deskewAngle * M_PI / 180.) * ip.dz_raw / ip.dxy;
  std::vector<float> section((size_t)nx_raw * ny + 1, 0.f);  // + 1: the reference's in[indin + 1] at the end
  std::vector<float> ext((size_t)xdim * ny);
  const float* bg = (const float*)d.background.getPtr();
  const float* sl = (const float*)d.slope.getPtr();
  for (int direction = 0; direction < p.ndirs; ++direction) {
    for (int z = 0; z < ip.nz; ++z) {
      int zsec = p.bFastSIM ? (z * p.ndirs * p.nphases + direction * p.nphases)
                            : (direction * ip.nz * p.nphases + z * p.nphases);
      for (int phase = 0; phase < p.nphases; ++phase) {
        if (p.bBgInExtHdr) d.backgroundExtra = zsec < (int)h->section_bg.size() ? h->section_bg[zsec] : 0.f;
        const float* buffer = h->raw.data() + (size_t)zsec * nx_raw * ny;
        for (int l = 0; l < ny; l++)
          for (int k = 0; k < nx_raw; k++)
            section[l * nx_raw + k] =
                (buffer[l * nx_raw + k] - bg[l * nx_raw + k] - d.backgroundExtra) * sl[l * nx_raw + k] * ip.inscale;
        // the reference's loop is an OpenMP parallel for over xout
#pragma omp parallel for
        for (int xout = 0; xout < xdim; xout++) {
          float xin = xout;
          if (fabs(deskewFactor) > 0)
            xin = xout - nx / 2. + p.extraShift - deskewFactor * (z - ip.nz / 2.) + nx_raw / 2.;
          for (int y = 0; y < ny; y++) {
            unsigned indout = y * xdim + xout;
            if (xin >= 0 && xin < nx_raw) {
              unsigned indin = y * nx_raw + (unsigned int)floor(xin);
              float offset = xin - floor(xin);
              ext[indout] = (1 - offset) * section[indin] + offset * section[indin + 1];
            } else {
              ext[indout] = 0.;
            }
          }
        }
        cudaMemcpy((char*)d.savedBands[direction][phase].getPtr() +
                       (size_t)(z + h->zoffset) * xdim * ny * sizeof(float),
                   ext.data(), (size_t)xdim * ny * sizeof(float), cudaMemcpyHostToDevice);
        ++zsec;
      }
    }
  }
}

// transformXYSlice, cudaSirecon.cpp:542-579.
void transform_xy(Harness* h)
{
  ImageParams& ip = h->ip;
  cufftHandle plan;
  int fftN[2] = {ip.ny, ip.nx};
  int inembed[2] = {ip.nx * ip.ny, (ip.nx / 2 + 1) * 2};
  int idist = (ip.nx / 2 + 1) * 2 * ip.ny;
  int onembed[2] = {ip.nx * ip.ny, ip.nx / 2 + 1};
  int odist = (ip.nx / 2 + 1) * ip.ny;
  cufftPlanMany(&plan, 2, fftN, inembed, 1, idist, onembed, 1, odist, CUFFT_R2C, ip.nz);
  for (int dir = 0; dir < h->p.ndirs; ++dir)
    for (int ph = 0; ph < h->p.nphases; ++ph)
      cufftExecR2C(plan, (float*)h->d.savedBands[dir][ph].getPtr(), (cuFloatComplex*)h->d.savedBands[dir][ph].getPtr());
  cufftDestroy(plan);
}

// The per-direction separation + z-FFT of
// findModulationVectorsAndPhasesForAllDirections (cudaSirecon.cpp:194-257),
// preceded by apodizationDriver (496-518) and transformXYSlice.
void stage_separate(Harness* h)
{
  ReconParams& p = h->p;
  ImageParams& ip = h->ip;
  ReconData& d = h->d;
  for (int direction = 0; direction < p.ndirs; ++direction)
    for (int z = 0; z < ip.nz; ++z)
      for (int phase = 0; phase < p.nphases; ++phase)
        if (p.napodize > 0)
          apodize(p.napodize, ip.nx, ip.ny, &(d.savedBands[direction][phase]),
                  (z + h->zoffset) * (ip.nx / 2 + 1) * 2 * ip.ny);
  transform_xy(h);
  for (int direction = 0; direction < p.ndirs; ++direction) {
    std::vector<GPUBuffer>* bands = &(d.savedBands[direction]);
    separate(ip.nx, ip.ny, ip.nz, direction, p.nphases, p.norders, bands, &d.sepMatrix[0]);
    if (ip.nz > 1) {
      cufftHandle plan1D;
      int fftN[1] = {ip.nz0};
      int stride = (ip.nx / 2 + 1) * ip.ny;
      cufftPlanMany(&plan1D, 1, fftN, fftN, stride, 1, fftN, stride, 1, CUFFT_C2C, (ip.nx / 2 + 1) * ip.ny);
      for (int i = 0; i < p.nphases; ++i)
        cufftExecC2C(plan1D, (cuFloatComplex*)(*bands)[i].getPtr(), (cuFloatComplex*)(*bands)[i].getPtr(), CUFFT_FORWARD);
      cufftDestroy(plan1D);
    }
  }
}

// The k0 / modamp part of findModulationVectorsAndPhasesForAllDirections,
// cudaSirecon.cpp:296-493.
void stage_fit(Harness* h)
{
  ReconParams* params = &h->p;
  ImageParams& ip = h->ip;
  ReconData* data = &h->d;
  float dkx = 1. / (ip.dxy * ip.nx);
  float dky = 1. / (ip.dxy * ip.ny);
  float k0magguess = 1.0 / params->linespacing;
  for (int direction = 0; direction < params->ndirs; ++direction) {
    std::vector<GPUBuffer>* bands = &(data->savedBands[direction]);
    if (!(ip.ntimes > 1 && ip.curTimeIdx > 0 && params->bUseTime0k0)) {
      data->k0[direction] = data->k0guess[direction];
    }
    cuFloatComplex amp_inv, amp_combo;
    int dir_ = params->bOneOTFperAngle ? direction : 0;
    if (params->bSearchforvector && !(ip.ntimes > 1 && ip.curTimeIdx > 0 && params->bUseTime0k0)) {
      ++h->n_searches;
      findk0(bands, &data->overlap0, &data->overlap1, ip.nx, ip.ny, ip.nz0, params->norders,
             &(data->k0[direction]), ip.dxy, ip.dz, &(data->otf[dir_]), ip.wave[0], params);
      if (h->capture_overlaps) {
        const size_t n = data->overlap0.getSize();
        std::vector<float> c(2 * n / sizeof(float));
        cudaMemcpy(c.data(), data->overlap0.getPtr(), n, cudaMemcpyDeviceToHost);
        cudaMemcpy(c.data() + n / sizeof(float), data->overlap1.getPtr(), n, cudaMemcpyDeviceToHost);
        if (h->captured.size() < (size_t)params->ndirs) h->captured.resize(params->ndirs);
        h->captured[direction] = std::move(c);
      }
      params->recalcarrays = 1;
      fitk0andmodamps(bands, &data->overlap0, &data->overlap1, ip.nx, ip.ny, ip.nz0, params->norders,
                      &(data->k0[direction]), ip.dxy, ip.dz, &(data->otf[dir_]), ip.wave[0],
                      &data->amp[direction][0], params);
      if (ip.curTimeIdx == 0) data->k0_time0[direction] = data->k0[direction];
      vector deltak0;
      deltak0.x = data->k0[direction].x - data->k0guess[direction].x;
      deltak0.y = data->k0[direction].y - data->k0guess[direction].y;
      float dist = sqrt(deltak0.x * deltak0.x + deltak0.y * deltak0.y);
      (void)k0magguess;
      if (ip.ntimes > 1 && ip.curTimeIdx > 0 && dist > 2 * K0_WARNING_THRESH) {
        data->k0[direction] = data->k0_time0[direction];
        for (int order = 1; order < params->norders; ++order) {
          h->n_overlap_builds++, h->n_reductions++;
          if (ip.nz0 > 1)
            findrealspacemodamp(bands, &data->overlap0, &data->overlap1, ip.nx, ip.ny, ip.nz0, 0, order,
                                data->k0[direction], ip.dxy, ip.dz, &(data->otf[dir_]), ip.wave[0],
                                &data->amp[direction][order], &amp_inv, &amp_combo, 1, params);
          else
            findrealspacemodamp(bands, &data->overlap0, &data->overlap1, ip.nx, ip.ny, ip.nz0, order - 1, order,
                                data->k0[direction], ip.dxy, ip.dz, &(data->otf[dir_]), ip.wave[0],
                                &data->amp[direction][order], &amp_inv, &amp_combo, 1, params);
        }
      }
    } else {
      for (int order = 1; order < params->norders; ++order) {
        h->n_overlap_builds++, h->n_reductions++;
        findrealspacemodamp(bands, &data->overlap0, &data->overlap1, ip.nx, ip.ny, ip.nz0, 0, order,
                            data->k0[direction], ip.dxy, ip.dz, &(data->otf[dir_]), ip.wave[0],
                            &data->amp[direction][order], &amp_inv, &amp_combo, 1, params);
      }
    }
    if (ip.nz == 1)
      for (int order = 2; order < params->norders; ++order)
        data->amp[direction][order] = cmul(data->amp[direction][order], data->amp[direction][order - 1]);
    if (params->forceamp[0] > 0.0) {
      for (int order = 1; order < params->norders; ++order) {
        float a = cmag(data->amp[direction][order]);
        if (a < params->forceamp[order - 1]) {
          float ampfact = params->forceamp[order - 1] / a;
          data->amp[direction][order].x *= ampfact;
          data->amp[direction][order].y *= ampfact;
        }
      }
    }
    if (!params->bFitallphases) {
      float base_phase = get_phase(data->amp[direction][1]);
      for (int order = 2; order < params->norders; ++order) {
        cuFloatComplex amplitude, expiphi;
        amplitude.x = cmag(data->amp[direction][order]);
        amplitude.y = 0;
        float phi = order * base_phase;
        expiphi.x = cos(phi);
        expiphi.y = sin(phi);
        data->amp[direction][order] = cmul(amplitude, expiphi);
      }
    }
  }
}

// processOneVolume, cudaSirecon.cpp:1264-1321, split into stages so that the
// separated bands can be captured between them.
void stage_assemble(Harness* h)
{
  ReconParams& p = h->p;
  ImageParams& ip = h->ip;
  ReconData& d = h->d;
  d.overlap0.resize(0);
  d.overlap1.resize(0);
  size_t nbig = (size_t)(p.zoomfact * ip.nx) * (size_t)(p.zoomfact * ip.ny) * (size_t)(p.z_zoom * ip.nz0);
  d.bigbuffer.resize(nbig * sizeof(cuFloatComplex));
  d.bigbuffer.setToZero();
  d.outbuffer.resize(nbig * sizeof(float));
  d.outbuffer.setToZero();
  for (int direction = 0; direction < p.ndirs; ++direction) {
    int dir_ = p.bOneOTFperAngle ? direction : 0;
    filterbands(direction, &d.savedBands[direction], d.k0, p.ndirs, p.norders, d.otf[dir_], ip.dxy, ip.dz,
                d.amp, d.noiseVarFactors, ip.nx, ip.ny, ip.nz0, ip.wave[0], &p);
    assemblerealspacebands(direction, &d.outbuffer, &d.bigbuffer, &d.savedBands[direction], p.ndirs, p.norders,
                           d.k0, ip.nx, ip.ny, ip.nz0, ip.dxy, p.zoomfact, p.z_zoom, p.explodefact);
  }
}

void begin_volume(Harness* h)
{
  ReconData& d = h->d;
  ImageParams& ip = h->ip;
  d.bigbuffer.resize(0);
  d.outbuffer.resize(0);
  d.overlap0.resize((size_t)ip.nx * ip.ny * ip.nz * sizeof(cuFloatComplex));
  d.overlap0.setToZero();
  d.overlap1.resize((size_t)ip.nx * ip.ny * ip.nz * sizeof(cuFloatComplex));
  d.overlap1.setToZero();
}

}  // namespace

extern "C" {

void* refh_new(int nx, int ny, int nImages, const char* config_text, const float* otf, int otf_w, int otf_h,
               int otf_d)
{
  Harness* h = new Harness();
  set_defaults(&h->p, &h->ip);
  apply_config(h, config_text);
  setup(h, nx, ny, nImages, otf, otf_w, otf_h, otf_d);
  return h;
}

void refh_delete(void* hv) { delete (Harness*)hv; }

void refh_set_ntimes(void* hv, int ntimes) { ((Harness*)hv)->ip.ntimes = (short)ntimes; }
void refh_set_cur_time(void* hv, int it) { ((Harness*)hv)->ip.curTimeIdx = (unsigned short)it; }

// SR_setRaw -> setRaw -> loadImageData
void refh_set_raw(void* hv, const float* raw)
{
  Harness* h = (Harness*)hv;
  size_t n = (size_t)h->nImages * h->ip.nx_raw * h->ip.ny;
  h->raw.assign(raw, raw + n);
  load_image_data(h);
}

void refh_set_section_backgrounds(void* hv, const float* v, int n)
{
  ((Harness*)hv)->section_bg.assign(v, v + n);
}

int refh_nx(void* hv) { return ((Harness*)hv)->ip.nx; }

// SR_loadAndRescaleImage -> rescaleDriver (cudaSirecon.cpp:520-540)
void refh_load_and_rescale(void* hv, int it)
{
  Harness* h = (Harness*)hv;
  if (h->p.bBessel && h->p.bNoRecon) return;  // cudaSirecon.cpp:1325
  for (int direction = 0; direction < h->p.ndirs; ++direction)
    for (int z = 0; z < h->ip.nz; ++z)
      if (h->p.do_rescale)
        rescale(h->ip.nx, h->ip.ny, h->ip.nz, z, h->zoffset, direction, 0, it, h->p.nphases,
                &h->d.savedBands[direction], h->p.equalizez, h->p.equalizet, &h->d.sum_dir0_phase0[0]);
}

void refh_stage_separate(void* hv)
{
  begin_volume((Harness*)hv);
  stage_separate((Harness*)hv);
  cudaDeviceSynchronize();
}
void refh_stage_fit(void* hv)
{
  stage_fit((Harness*)hv);
  cudaDeviceSynchronize();
}
void refh_stage_assemble(void* hv)
{
  stage_assemble((Harness*)hv);
  cudaDeviceSynchronize();
}

// SR_processOneVolume
int refh_process(void* hv)
{
  Harness* h = (Harness*)hv;
  begin_volume(h);
  stage_separate(h);
  stage_fit(h);
  stage_assemble(h);
  return 1;
}

// SR_getResult (cudaSirecon.cpp:1620-1634)
void refh_get_result(void* hv, float* out)
{
  Harness* h = (Harness*)hv;
  cudaMemcpy(out, h->d.outbuffer.getPtr(), h->d.outbuffer.getSize(), cudaMemcpyDeviceToHost);
}

// band b (0..nphases-1) of direction dir, half-complex [nz0][ny][nx/2+1]
void refh_get_band(void* hv, int dir, int b, float* out)
{
  Harness* h = (Harness*)hv;
  size_t n = (size_t)(h->ip.nx / 2 + 1) * h->ip.ny * h->ip.nz0 * sizeof(cuFloatComplex);
  cudaMemcpy(out, h->d.savedBands[dir][b].getPtr(), n, cudaMemcpyDeviceToHost);
}

// k0 (1/um) as [ndirs][2]; amp as [ndirs][norders][2]
void refh_get_fit(void* hv, float* k0, float* amp)
{
  Harness* h = (Harness*)hv;
  for (int d = 0; d < h->p.ndirs; ++d) {
    k0[2 * d] = h->d.k0[d].x;
    k0[2 * d + 1] = h->d.k0[d].y;
    for (int o = 0; o < h->p.norders; ++o) {
      amp[(d * h->p.norders + o) * 2] = h->d.amp[d][o].x;
      amp[(d * h->p.norders + o) * 2 + 1] = h->d.amp[d][o].y;
    }
  }
}

// k0guess as [ndirs][2]
void refh_get_k0guess(void* hv, float* k0)
{
  Harness* h = (Harness*)hv;
  for (int d = 0; d < h->p.ndirs; ++d) {
    k0[2 * d] = h->d.k0guess[d].x;
    k0[2 * d + 1] = h->d.k0guess[d].y;
  }
}

// capture the overlap pair after each direction's findk0 (on != 0); then
// refh_get_captured(dir) copies [overlap0 | overlap1] (complex, nz0 x ny x nx
// each) and returns its float count, or 0 if none was captured
void refh_capture_overlaps(void* hv, int on) { ((Harness*)hv)->capture_overlaps = on != 0; }

long long refh_get_captured(void* hv, int dir, float* out)
{
  Harness* h = (Harness*)hv;
  if (dir < 0 || (size_t)dir >= h->captured.size() || h->captured[dir].empty()) return 0;
  if (out) memcpy(out, h->captured[dir].data(), h->captured[dir].size() * sizeof(float));
  return (long long)h->captured[dir].size();
}

// executed overlap builds, reductions and k0 searches since creation
void refh_fit_counts(void* hv, long long* out3)
{
  Harness* h = (Harness*)hv;
  out3[0] = h->n_overlap_builds;
  out3[1] = h->n_reductions;
  out3[2] = h->n_searches;
}

int refh_norders(void* hv) { return ((Harness*)hv)->p.norders; }
int refh_nz(void* hv) { return ((Harness*)hv)->ip.nz; }

}  // extern "C"
