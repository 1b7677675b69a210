// Host orchestration of the reconstruction (the reference's
// SIM_Reconstructor, cudaSirecon.cpp:792-1713, and the host halves of
// gpuFunctionsImpl.cu).  All device work is issued on the handle's own
// stream; the host only steers the k0 / modamp search, reading back a few
// scalars per search step.
#include "reconstructor.h"
#include "reg_fft.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <dirent.h>
#include <regex>
#include <set>
#include <sstream>
#include <stdexcept>
#include <sys/stat.h>

using namespace simrecon;

namespace {

constexpr float kK0WarningThresh = 0.05f;  // cudaSireconImpl.h:55

uint32_t fbits(float f)
{
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// notGoodDimension / findOptimalDimension (cudaSirecon.cpp:76-97): the
// largest size <= n that factors into 2, 3, 5 and 7
bool not_good_dimension(unsigned num)
{
  if (num == 2 || num == 3 || num == 5 || num == 7) return false;
  if (num % 2 == 0) return not_good_dimension(num / 2);
  if (num % 3 == 0) return not_good_dimension(num / 3);
  if (num % 5 == 0) return not_good_dimension(num / 5);
  if (num % 7 == 0) return not_good_dimension(num / 7);
  return true;
}
unsigned find_optimal_dimension(unsigned n)
{
  while (n > 1 && not_good_dimension(n)) --n;
  return n;
}

float2v cmulh(float2v a, float2v b) { return float2v{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
float cmagh(float2v a) { return sqrt(a.x * a.x + a.y * a.y); }

// fitparabola, gpuFunctionsImpl.cu:479-495
float fitparabola(float a1, float a2, float a3)
{
  float slope = 0.5 * (a3 - a1);
  float curve = (a3 + a1) - 2 * a2;
  if (curve == 0) return 0.0;
  float peak = -slope / curve;
  if (peak > 1.5 || peak < -1.5) return 0.0;
  return peak;
}

// fitxyparabola, gpuFunctionsImpl.cu:1022-1044
float fitxyparabola(float x1, float y1, float x2, float y2, float x3, float y3)
{
  if (x1 == x2 || x2 == x3 || x3 == x1) return 0.0;
  float xbar1 = 0.5 * (x1 + x2);
  float xbar2 = 0.5 * (x2 + x3);
  float slope1 = (y2 - y1) / (x2 - x1);
  float slope2 = (y3 - y2) / (x3 - x2);
  float curve = (slope2 - slope1) / (xbar2 - xbar1);
  if (curve == 0) return 0.0;
  return xbar2 - slope2 / curve;
}

bool is_directory(const std::string& p)
{
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

// gatherMatchingFiles (boostfs.cpp:9-56): regular files of the folder whose
// full path matches ".*<pattern>" (".*<pattern>.*\.[tT][iI][fF]" unless the
// pattern already names a .tif), sorted
std::vector<std::string> gather_matching(const std::string& dir, std::string pattern)
{
  std::vector<std::string> out;
  if (pattern.rfind(".tif") == std::string::npos && pattern.rfind(".TIF") == std::string::npos)
    pattern.append(".*\\.[tT][iI][fF]");
  pattern.insert(0, ".*");
  std::regex filt;
  try {
    filt = std::regex(pattern);
  } catch (...) {
    return out;
  }
  DIR* dp = opendir(dir.c_str());
  if (!dp) return out;
  while (struct dirent* e = readdir(dp)) {
    std::string name = e->d_name;
    if (name == "." || name == "..") continue;
    std::string full = dir + (dir.empty() || dir.back() == '/' ? "" : "/") + name;
    struct stat st;
    if (stat(full.c_str(), &st) != 0 || !S_ISREG(st.st_mode)) continue;
    if (std::regex_match(full, filt)) out.push_back(full);
  }
  closedir(dp);
  std::sort(out.begin(), out.end());
  if (!out.empty()) mkdir((dir + "/GPUsirecon").c_str(), 0755);
  return out;
}

// makeOutputFilePath (boostfs.cpp:59-72)
std::string output_path_for(const std::string& input, const std::string& insert)
{
  std::string base = input.substr(input.find_last_of('/') + 1);
  std::string dir = input.substr(0, input.find_last_of('/') + 1);
  size_t pos = base.find_last_of(".tif");
  if (pos != std::string::npos && pos >= 3) base.insert(pos - 3, insert);
  return dir + "GPUsirecon/" + base;
}

}  // namespace

// ------------------------------------------------------------ construction
void SIM_Reconstructor::check(cudaError_t e, const char* what)
{
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void SIM_Reconstructor::check_launch(int rc, const char* what)
{
  if (rc != 0) {
    if (rc > 0) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString((cudaError_t)rc));
    throw std::runtime_error(std::string(what) + ": unsupported size (code " + std::to_string(rc) + ")");
  }
}

bool SIM_Reconstructor::load_otf_tiff(const std::string& path, Stack* out, std::string* err)
{
  return tiff_read(path, out, err);
}

bool SIM_Reconstructor::init_shape(int nx, int ny, int nimages, const std::string& config, std::string* err)
{
  set_defaults(&opt);
  // the config file is parsed if it can be opened (cudaSirecon.cpp:884-890)
  if (!apply_config_file(&opt, config, false, err)) return false;
  if (opt.p.otffiles.empty()) {
    *err = "the option '--otf-file' is required but missing";
    return false;
  }
  Stack otf;
  if (!load_otf_tiff(opt.p.otffiles, &otf, err)) return false;
  opt.p.bTIFF = true;  // cudaSirecon.cpp:901
  return setup(nx, ny, nimages, 1, &otf, err);
}

SIM_Reconstructor* SIM_Reconstructor::from_shape(int nx, int ny, int nimages, const std::string& config,
                                                 std::string* err)
{
  SIM_Reconstructor* r = new SIM_Reconstructor();
  if (!r->init_shape(nx, ny, nimages, config, err)) {
    delete r;
    return nullptr;
  }
  return r;
}

bool SIM_Reconstructor::plan_bytes(int nx, int ny, int nimages, const std::string& config, size_t* bytes,
                                   std::string* err)
{
  SIM_Reconstructor r;
  r.dry_run_ = true;
  if (!r.init_shape(nx, ny, nimages, config, err)) return false;
  *bytes = r.planned_bytes_;
  return true;
}

SIM_Reconstructor* SIM_Reconstructor::from_argv(int argc, char** argv, std::string* err)
{
  SIM_Reconstructor* r = new SIM_Reconstructor();
  set_defaults(&r->opt);
  for (int i = 0; i < argc; ++i) r->argv_.push_back(argv[i] ? argv[i] : "");
  if (!parse_command_line(&r->opt, argc, argv, err)) {
    delete r;
    return nullptr;
  }
  if (r->opt.help || argc <= 1) {
    *err = "help requested\n" + usage_text();
    delete r;
    return nullptr;
  }
  if (r->opt.version) {
    *err = "version requested";
    delete r;
    return nullptr;
  }
  ReconParams& p = r->opt.p;
  ImageParams& ip = r->opt.ip;
  if (p.ifiles.empty() || p.ofiles.empty()) {
    *err = "Calling openFiles() but no input or output files were specified";
    delete r;
    return nullptr;
  }
  // TIFF mode when the input is a folder with files matching the pattern
  if (is_directory(p.ifiles)) {
    r->tiff_files_ = gather_matching(p.ifiles, p.ofiles);
    p.bTIFF = !r->tiff_files_.empty();
  }
  Stack otf;
  int nx = 0, ny = 0, nimg = 0, nwaves = 1;
  if (p.bTIFF) {
    ip.ntimes = (short)r->tiff_files_.size();
    int depth;
    if (!tiff_info(r->tiff_files_[0], &nx, &ny, &depth, err)) {
      delete r;
      return nullptr;
    }
    nimg = depth;
    if (!tiff_read(p.otffiles, &otf, err)) {
      delete r;
      return nullptr;
    }
  } else {
    // MRC / DV input (loadHeader, mrc.h:18-45)
    if (!mrc_open(p.ifiles, &r->mrc_in_, err)) {
      delete r;
      return nullptr;
    }
    const MrcHeader& h = r->mrc_in_.hdr;
    nx = h.nx;
    ny = h.ny;
    nwaves = std::max<int>(1, h.num_waves);
    int ntimes = std::max<int>(1, h.num_times);
    nimg = h.nz / ntimes;  // sections per time point (all waves)
    ip.ntimes = (short)ntimes;
    ip.wave[0] = h.iwav1;
    ip.wave[1] = h.iwav2;
    ip.wave[2] = h.iwav3;
    ip.wave[3] = h.iwav4;
    ip.wave[4] = h.iwav5;
    ip.dxy = h.ylen;
    ip.dz = h.zlen;
    // the OTF: MRC (complex) or TIFF
    MrcFile of;
    std::string e2;
    if (mrc_open(p.otffiles, &of, &e2)) {
      std::vector<float> all;
      if (!mrc_read_all(of, &all, err)) {
        delete r;
        return nullptr;
      }
      // determine_otf_dimensions, MRC branch (cudaSirecon.cpp:1484-1523):
      // complex sections of nx (kz) by ny (kr); stored like the TIFF layout
      otf.width = 2 * of.hdr.nx;
      otf.height = of.hdr.ny;
      otf.depth = of.hdr.nz;
      otf.data = all;
      // dkz / dkr come from the header
      p.dkzotf = of.hdr.xlen;
      p.dkrotf = of.hdr.ylen;
      if (nimg / (nwaves * p.nphases * p.ndirs) == 1) p.dkrotf = of.hdr.xlen;
      r->otf_dk_from_header_ = true;
    } else if (!tiff_read(p.otffiles, &otf, err)) {
      delete r;
      return nullptr;
    }
  }
  if (!r->setup(nx, ny, nimg, nwaves, &otf, err)) {
    delete r;
    return nullptr;
  }
  if (!p.bTIFF) {
    // output header (setOutputHeader, mrc.h:47-60)
    MrcHeader h = r->mrc_in_.hdr;
    h.mode = 2;
    h.nz = ip.nz * ip.nwaves * ip.ntimes * p.z_zoom;
    h.nx = (int)(ip.nx * p.zoomfact);
    h.ny = (int)(h.ny * p.zoomfact);
    h.xlen /= p.zoomfact;
    h.ylen /= p.zoomfact;
    h.zlen /= p.z_zoom;
    h.next = 0;
    r->out_hdr_ = h;
    memcpy(r->in_label0_, r->mrc_in_.hdr.label[0], 80);
    r->out_path_ = p.ofiles;
    r->mrc_out_.open(p.ofiles, std::ios::binary | std::ios::trunc);
    if (!r->mrc_out_) {
      *err = "File " + p.ofiles + " can not be created.";
      delete r;
      return nullptr;
    }
    r->mrc_out_.write((const char*)&r->out_hdr_, sizeof(MrcHeader));
    if (!r->open_debug_files(err)) {
      delete r;
      return nullptr;
    }
  }
  return r;
}

// setup() + setup_common(), cudaSirecon.cpp:1104-1261
bool SIM_Reconstructor::setup(int nx, int ny, int nimages, int nwaves, const Stack* otf, std::string* err)
{
  ReconParams& p = opt.p;
  ImageParams& ip = opt.ip;
  ip.nx = nx;
  ip.nx_raw = nx;
  ip.ny = ny;
  ip.nwaves = (short)nwaves;
  ip.nz = nimages / (nwaves * p.nphases * p.ndirs);
  ip.nz0 = ip.nz;
  ip.dz_raw = 0;
  if (ip.nz < 1 || nimages != ip.nz * nwaves * p.nphases * p.ndirs) {
    *err = "number of images (" + std::to_string(nimages) + ") is not a multiple of ndirs*nphases";
    return false;
  }
  if (p.bTwolens) {  // makeoverlaps / filterbands stop there (gpuFunctionsImpl.cu:540-543)
    *err = "Sorry, this program doesn't handel 2-objective mode data";
    return false;
  }
  if (p.nzPadTo) {
    *err = "nzPadTo is not supported by this build";
    return false;
  }
  // setup_common's deskew and crop (cudaSirecon.cpp:1153-1170): the width
  // reconstructed becomes a good FFT size covering the sheared planes, dz
  // the distance between them; cropXY keeps the first cropXYto columns
  if (fabs(p.deskewAngle) > 0.) {
    if (p.deskewAngle < 0) p.deskewAngle += 180.;
    ip.nx = (int)find_optimal_dimension(
        (unsigned)(ip.nx_raw + ip.nz0 * fabs(cos(p.deskewAngle * M_PI / 180.)) * ip.dz / ip.dxy));
    ip.dz_raw = ip.dz;
    ip.dz *= fabs(sin(p.deskewAngle * M_PI / 180.));
  }
  if (p.cropXYto > 0 && p.cropXYto < (unsigned)ip.nx) ip.nx = (int)p.cropXYto;
  nx = ip.nx;
  nx_raw_ = ip.nx_raw;
  deskew_factor_ = 0.f;
  if (fabs(p.deskewAngle) > 0.0) deskew_factor_ = cos(p.deskewAngle * M_PI / 180.) * ip.dz_raw / ip.dxy;
  // deskew or crop change the planes' geometry; per-section backgrounds
  // (bBgInExtHdr, also settable later through ReconParams) use the same pass
  precondition_ = deskew_factor_ != 0.f || ip.nx != ip.nx_raw;
  p.norders = p.norders_output != 0 ? p.norders_output : p.nphases / 2 + 1;
  if (2 * p.norders - 1 != p.nphases) {
    *err = "nphases must equal 2*norders-1 (the band separation swaps nphases bands)";
    return false;
  }
  if (p.ndirs > kMaxDirs || p.norders > kMaxOrders || p.nphases > kMaxPhases) {
    *err = "too many directions / orders / phases";
    return false;
  }
  if (!p.bRadAvgOTF) {
    *err = "only rotationally averaged OTFs (otfRA) are supported: the reference's GPU OTF lookup returns 0 "
           "for other OTFs (gpuFunctionsImpl.cu:1677-1715)";
    return false;
  }
  nx_ = nx;
  ny_ = ny;
  nz_ = ip.nz;
  nxh_ = nx / 2 + 1;
  nimg_ = nimages;
  nph_ = p.nphases;
  ndirs_ = p.ndirs;
  norders_ = p.norders;
  X_ = (int)lrint(p.zoomfact * nx);
  Y_ = (int)lrint(p.zoomfact * ny);
  Z_ = p.z_zoom * nz_;
  if (X_ < nx || Y_ < ny || Z_ < nz_) {
    *err = "zoom factors below 1 are not supported";
    return false;
  }
  for (int n : {nx, ny, nz_, X_, Y_, Z_})
    if (!fft_length_ok(n) || n > 8192) {
      *err = "image size " + std::to_string(n) + " does not factor into 2, 3, 5 and 7 (or exceeds 8192)";
      return false;
    }
  if (p.napodize > ny / 2 || p.napodize > nx / 2 || p.napodize > kMaxApo) {
    *err = "napodize too large for the image";
    return false;
  }
  // determine_otf_dimensions (cudaSirecon.cpp:1446-1523), RA OTF
  const int w2 = otf->width / 2;
  if (nz_ == 1) {
    p.nxotf = w2;
    p.nyotf = 1;
    p.nzotf = 1;
    if (!otf_dk_from_header_) p.dkrotf = 1 / (ip.dxy * (w2 - 1) * 2);
    p.dkzotf = 1;
  } else {
    p.nzotf = w2;
    p.nxotf = otf->height;
    p.nyotf = 1;
    if (!otf_dk_from_header_) {
      p.dkzotf = 1 / (p.dzPSF * p.nzotf);
      p.dkrotf = 1 / (ip.dxy * (p.nxotf - 1) * 2);
    }
  }
  ndirs_otf_ = p.bOneOTFperAngle ? p.ndirs : 1;
  const size_t otf_size = (size_t)p.nxotf * p.nzotf;
  const size_t page = (size_t)otf->width * otf->height;
  std::vector<float2v> hotf((size_t)ndirs_otf_ * norders_ * otf_size);
  // loadOTFs: section i of the file is order i; missing ones copy otf[0][0]
  for (int d = 0; d < ndirs_otf_; ++d)
    for (int o = 0; o < norders_; ++o) {
      int sec = o + d * norders_;
      const float* src = (otf->depth > sec) ? otf->data.data() + page * sec : otf->data.data();
      if (otf_size * 2 > page) {
        *err = "OTF file smaller than its declared size";
        return false;
      }
      memcpy(&hotf[((size_t)d * norders_ + o) * otf_size], src, otf_size * sizeof(float2v));
    }

  // makematrix, default branch (cudaSirecon.cpp:606-617)
  sepmat_.assign((size_t)nph_ * nph_, 0.f);
  float phi = 2.0 * M_PI / nph_;
  for (int j = 0; j < nph_; ++j) {
    sepmat_[0 * nph_ + j] = 1.0;
    for (int order = 1; order < norders_; ++order) {
      sepmat_[(2 * order - 1) * nph_ + j] = cos(j * order * phi);
      sepmat_[2 * order * nph_ + j] = sin(j * order * phi);
    }
  }
  noisevar_.assign((size_t)ndirs_ * norders_, 1.0f);

  // inscale and k0guess (cudaSirecon.cpp:1231-1252)
  ip.inscale = 1.0 / (ip.nx * ip.ny * ip.nz0 * p.zoomfact * p.zoomfact * p.z_zoom * p.ndirs);
  k0_.assign(ndirs_, float2v{0, 0});
  k0_time0_.assign(ndirs_, float2v{0, 0});
  k0guess_.assign(ndirs_, float2v{0, 0});
  float delta_angle = M_PI / p.ndirs;
  float k0magguess = 1.0 / p.linespacing;
  if (ip.nz > 1) {
    int nordersIn = p.nphases / 2 + 1;
    k0magguess /= nordersIn - 1;
  }
  for (int i = 0; i < p.ndirs; ++i) {
    float k0angleguess;
    if (p.k0angles.size() < (size_t)p.ndirs) k0angleguess = p.k0startangle + i * delta_angle;
    else k0angleguess = p.k0angles[i];
    k0guess_[i].x = k0magguess * cos(k0angleguess);
    k0guess_[i].y = k0magguess * sin(k0angleguess);
  }
  amp_.assign(ndirs_, std::vector<float2v>(norders_, float2v{0, 0}));
  for (int i = 0; i < ndirs_; ++i) amp_[i][0] = float2v{1.0f, 0.0f};

  // makeoverlaps zdistcutoff (gpuFunctionsImpl.cu:529-548) bounds the overlap planes
  {
    float dkz = 1.0f / (nz_ * ip.dz);
    float lambdaem = (ip.wave[0] / p.nimm) / 1.0e3;
    float alpha = asinf(p.na / p.nimm);
    float zd = (int)ceil(((1.0 - cosf(alpha)) / lambdaem) / dkz);
    if (zd > nz_ / 2) zd = ((nz_ / 2 - 1) > 0) ? (nz_ / 2 - 1) : 0;
    // Bessel mode: the cutoff depends on k0 and the order (overlap_zdc_bessel):
    // buffers for the largest one
    if (p.bBessel) zd = ((nz_ / 2 - 1) > 0) ? (nz_ / 2 - 1) : 0;
    zdc_ovl_ = (int)zd;
  }

  // device arena
  const size_t nrawxy = (size_t)nx_raw_ * ny_;
  const size_t nspec = (size_t)ndirs_ * nph_ * nz_ * ny_ * nxh_;
  const int nzb = 2 * zdc_ovl_ + 1;
  const size_t nxy = (size_t)nx_ * ny_;
  fit_lanes_ = std::max(1, std::min(ndirs_ * std::max(1, norders_ - 1), (int)kFitLanes));
  // assembly scratch: every slot of the volume (at most nz planes of
  // 1 + ndirs*(norders-1) slots) when that fits in 2 GiB, else as many as do
  // (at least one plane's worth); the slots are processed in plane groups
  const size_t per_slot = (size_t)Y_ * nx_;
  const size_t all_slots = (size_t)nz_ * (1 + (size_t)ndirs_ * (norders_ - 1));
  size_t want_slots = std::max<size_t>(1 + (size_t)ndirs_ * (norders_ - 1),
                                       std::min<size_t>(all_slots, (size_t)(2ull << 30) / (per_slot * sizeof(float2))));
  tcap_ = want_slots * per_slot + 65536;
  struct Req {
    void** ptr;
    size_t bytes;
  };
  std::vector<Req> reqs = {
      {&d_raw_, (size_t)nimg_ * nrawxy * sizeof(float)},
      {(void**)&d_pre_, precondition_ ? (size_t)nimg_ * nxy * sizeof(float) : 0},
      {(void**)&d_bgx_, precondition_ ? (size_t)nimg_ * sizeof(float) : 0},
      {(void**)&d_spec_, nspec * sizeof(float2)},
      {(void**)&d_scale_, (size_t)ndirs_ * nph_ * nz_ * sizeof(float)},
      {(void**)&d_sdp0_, (size_t)nz_ * sizeof(double)},
      {(void**)&d_sepmat_, sepmat_.size() * sizeof(float)},
      {(void**)&d_apofact_, (size_t)kMaxApo * sizeof(float)},
      {(void**)&d_otf_, hotf.size() * sizeof(float2)},
      // the fit's working buffers, one set per fit lane (directions fitted side by side)
      {(void**)&d_ovl_, fit_lanes_ * ovl_lane_elems() * sizeof(float2)},
      {(void**)&d_ppart_, fit_lanes_ * ppart_lane_elems() * sizeof(float2)},
      {(void**)&d_sums_, fit_lanes_ * sums_lane_elems() * sizeof(double)},
      {(void**)&d_pmap_, fit_lanes_ * nxy * sizeof(float2)},
      {(void**)&d_sumxy_, fit_lanes_ * 2 * sizeof(double)},
      {(void**)&d_cc_, fit_lanes_ * nxy * sizeof(float2)},
      {(void**)&d_bval_, fit_lanes_ * 256 * sizeof(float)},
      {(void**)&d_bidx_, fit_lanes_ * 256 * sizeof(int)},
      {(void**)&d_peak_, fit_lanes_ * 8 * sizeof(float)},
      {(void**)&d_tables_, fit_lanes_ * tables_lane_elems() * sizeof(float2)},
      {(void**)&d_partial_, fit_lanes_ * partial_lane_elems() * sizeof(double)},
      {(void**)&d_xstary_, fit_lanes_ * (size_t)kMaxCand * 2 * sizeof(double)},
      {(void**)&d_fit_, sizeof(FitDev)},
      {(void**)&d_fitslots_, (size_t)kMaxDirs * kMaxOrders * 4 * sizeof(double)},
      {(void**)&d_kst_, (size_t)kMaxDirs * 3 * sizeof(float2)},
      {(void**)&d_pmapd_, (size_t)ndirs_ * nxy * sizeof(float2)},
      {(void**)&d_sumxyd_, (size_t)ndirs_ * 2 * sizeof(double)},
      {(void**)&d_sinfo_, 2 * sizeof(int)},
      {(void**)&d_asmtab_, asm_table_bytes()},
      {(void**)&d_ex_, (size_t)ndirs_ * norders_ * X_ * sizeof(float2)},
      {(void**)&d_ey_, (size_t)ndirs_ * norders_ * Y_ * sizeof(float2)},
      {(void**)&d_T_, tcap_ * sizeof(float2)},
      {(void**)&d_S_, (size_t)X_ * Y_ * Z_ * sizeof(float2)},
      {(void**)&d_out_, (size_t)X_ * Y_ * Z_ * sizeof(float)},
  };
  size_t total = 0;
  for (auto& r : reqs) total += align_up(r.bytes, 256);
  if (dry_run_) {
    // every buffer the handle can hold: the arena, process_series' second raw
    // and output buffers, the flat-field calibration
    planned_bytes_ = total + (size_t)nimg_ * nrawxy * sizeof(float) + (size_t)X_ * Y_ * Z_ * sizeof(float) +
                     (p.bUsecorr ? 2 * nrawxy * sizeof(float) : 0);
    return true;
  }
  check(cudaGetDevice(&device_), "cudaGetDevice");
  check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  for (int l = 1; l < fit_lanes_; ++l) {
    check(cudaStreamCreateWithFlags(&fit_stream_[l], cudaStreamNonBlocking), "cudaStreamCreate");
    check(cudaEventCreateWithFlags(&fit_join_[l], cudaEventDisableTiming), "cudaEventCreate");
  }
  check(cudaEventCreateWithFlags(&fit_fork_, cudaEventDisableTiming), "cudaEventCreate");
  cudaError_t e = cudaMalloc((void**)&arena_, total);
  if (e != cudaSuccess) {
    *err = std::string("device allocation of ") + std::to_string(total >> 20) + " MiB failed: " +
           cudaGetErrorString(e);
    return false;
  }
  arena_bytes_ = total;
  size_t off = 0;
  for (auto& r : reqs) {
    *r.ptr = r.bytes ? arena_ + off : nullptr;
    off += align_up(r.bytes, 256);
  }
  check(cudaHostAlloc((void**)&h_pinned_, 4096, cudaHostAllocMapped), "cudaHostAlloc");
  check(cudaHostGetDevicePointer((void**)&dh_pinned_, h_pinned_, 0), "cudaHostGetDevicePointer");
  std::vector<float> fact(kMaxApo, 0.f);
  for (int l = 0; l < p.napodize; ++l) fact[l] = 1.0 - sinf((l + 0.5) / (float)p.napodize * M_PI * 0.5);
  check(cudaMemcpy(d_apofact_, fact.data(), kMaxApo * sizeof(float), cudaMemcpyHostToDevice), "upload");
  check(cudaMemcpy(d_sepmat_, sepmat_.data(), sepmat_.size() * sizeof(float), cudaMemcpyHostToDevice), "upload");
  check(cudaMemcpy(d_otf_, hotf.data(), hotf.size() * sizeof(float2), cudaMemcpyHostToDevice), "upload");
  check(cudaMemset(d_sdp0_, 0, (size_t)nz_ * sizeof(double)), "memset");
  check(cudaMemset(d_spec_, 0, nspec * sizeof(float2)), "memset");
  check(cudaMemset(d_fitslots_, 0, (size_t)kMaxDirs * kMaxOrders * 4 * sizeof(double)), "memset");
  if (precondition_) check(cudaMemset(d_bgx_, 0, (size_t)nimg_ * sizeof(float)), "memset");
  if (p.bBgInExtHdr) ensure_precondition_buffers();
  check_launch(upload_amps(), "fit init");
  check(cudaStreamSynchronize(stream_), "fit init");
  if (p.bUsecorr && !load_corr(err)) return false;
  return true;
}

SIM_Reconstructor::~SIM_Reconstructor()
{
  drop_graphs();
  for (auto& pd : pending_) {
    cudaEventDestroy(pd.a);
    cudaEventDestroy(pd.b);
  }
  if (stream_) cudaStreamSynchronize(stream_);
  if (h2d_stream_) cudaStreamSynchronize(h2d_stream_);
  if (d2h_stream_) cudaStreamSynchronize(d2h_stream_);
  for (int b = 0; b < 2; ++b)
    for (cudaEvent_t e : {ev_raw_ready_[b], ev_raw_free_[b], ev_out_ready_[b], ev_out_free_[b]})
      if (e) cudaEventDestroy(e);
  if (h2d_stream_) cudaStreamDestroy(h2d_stream_);
  if (d2h_stream_) cudaStreamDestroy(d2h_stream_);
  if (d_raw_alt_) cudaFree(d_raw_alt_);
  if (d_out_extra_) cudaFree(d_out_extra_);
  if (arena_) cudaFree(arena_);
  if (d_flush_) cudaFree(d_flush_);
  if (d_bgslope_) cudaFree(d_bgslope_);
  if (pre_own_) cudaFree(pre_own_);
  if (h_pinned_) cudaFreeHost(h_pinned_);
  for (int l = 1; l < kFitLanes; ++l) {
    if (fit_stream_[l]) cudaStreamDestroy(fit_stream_[l]);
    if (fit_join_[l]) cudaEventDestroy(fit_join_[l]);
  }
  if (fit_fork_) cudaEventDestroy(fit_fork_);
  if (stream_) cudaStreamDestroy(stream_);
}

// ---------------------------------------------------------------- profiling
void SIM_Reconstructor::stage_begin(const char* name, cudaEvent_t* a, long long* l0)
{
  (void)name;
  *l0 = launches_;
  if (!profiling_) return;
  cudaEventCreate(a);
  cudaEventRecord(*a, stream_);
}

void SIM_Reconstructor::stage_end(const char* name, cudaEvent_t a, long long l0)
{
  if (!profiling_) return;
  cudaEvent_t b;
  cudaEventCreate(&b);
  cudaEventRecord(b, stream_);
  pending_.push_back(Pending{name, a, b, launches_ - l0, 0.0, false});
}

void SIM_Reconstructor::KTimer::begin(cudaStream_t s)
{
  cudaEventCreate(&cur);
  cudaEventRecord(cur, s);
}

void SIM_Reconstructor::KTimer::end(const char* kernel, cudaStream_t s, double alg_bytes)
{
  cudaEvent_t b;
  cudaEventCreate(&b);
  cudaEventRecord(b, s);
  r->pending_.push_back(Pending{kernel, cur, b, 1, alg_bytes, true});
}

SIM_Reconstructor::TimerScope::TimerScope(SIM_Reconstructor* r) : prev(kernel_timer())
{
  r->ktimer_.r = r;
  set_kernel_timer(r->profiling_ ? &r->ktimer_ : nullptr);
}

SIM_Reconstructor::TimerScope::~TimerScope() { set_kernel_timer(prev); }

std::string SIM_Reconstructor::profile_json()
{
  cudaStreamSynchronize(stream_);
  for (auto& pd : pending_) {
    float ms = 0;
    cudaEventElapsedTime(&ms, pd.a, pd.b);
    if (pd.kernel) {
      auto& e = kprof_[pd.stage];
      e.ms += ms;
      e.launches += pd.launches;
      e.bytes += pd.bytes;
    } else {
      auto& e = prof_[pd.stage];
      e.first += ms;
      e.second += pd.launches;
    }
    cudaEventDestroy(pd.a);
    cudaEventDestroy(pd.b);
  }
  pending_.clear();
  std::ostringstream s;
  s.precision(9);
  s << "{\"stages\": {";
  bool first = true;
  for (auto& kv : prof_) {
    if (!first) s << ", ";
    first = false;
    s << "\"" << kv.first << "\": {\"ms\": " << kv.second.first << ", \"launches\": " << kv.second.second << "}";
  }
  s << "}, \"kernels\": {";
  first = true;
  for (auto& kv : kprof_) {
    if (!first) s << ", ";
    first = false;
    s << "\"" << kv.first << "\": {\"ms\": " << kv.second.ms << ", \"launches\": " << kv.second.launches
      << ", \"alg_bytes\": " << kv.second.bytes << "}";
  }
  s << "}}";
  return s.str();
}

void SIM_Reconstructor::reset_profile()
{
  profile_json();
  prof_.clear();
  kprof_.clear();
}

// -------------------------------------------------------------- ingestion
void SIM_Reconstructor::stage_raw(const void* raw, bool u16)
{
  const size_t n = (size_t)nimg_ * nx_raw_ * ny_;
  raw_u16_ = u16;
  check(cudaMemcpyAsync(d_raw_, raw, n * (u16 ? 2 : 4), cudaMemcpyHostToDevice, stream_), "raw upload");
  have_raw_ = true;
  raw_staged_ = true;
  ingest();
  // setRaw copies the caller's stack (interface.cpp:19-25): return once the
  // upload and the ingest kernels are done with it
  check(cudaStreamSynchronize(stream_), "ingest");
}

void SIM_Reconstructor::ingest()
{
  TimerScope ts(this);
  cudaEvent_t a;
  long long l0;
  stage_begin("ingest", &a, &l0);
  IngestArgs ia{};
  ia.raw = d_raw_;
  ia.raw_is_u16 = raw_u16_;
  ia.nx = nx_;
  ia.ny = ny_;
  ia.nz = nz_;
  ia.ndirs = ndirs_;
  ia.nphases = nph_;
  ia.fastSI = opt.p.bFastSIM;
  ia.bg = d_bgslope_;
  ia.slope = d_bgslope_ ? d_bgslope_ + (size_t)nx_ * ny_ : nullptr;
  ia.bgconst = opt.p.constbkgd;
  ia.bgextra = 0.f;
  ia.inscale = opt.ip.inscale;
  ia.napodize = opt.p.napodize;
  ia.apofact = d_apofact_;
  ia.spec = d_spec_;
  if (precondition_ || opt.p.bBgInExtHdr) {
    ensure_precondition_buffers();
    // flat field with the per-section backgrounds, then deskew or crop, into
    // d_pre_; the transforms then take those planes as they are
    PrecondArgs pa{};
    pa.raw = d_raw_;
    pa.raw_is_u16 = raw_u16_;
    pa.nx_raw = nx_raw_;
    pa.ny = ny_;
    pa.nx = nx_;
    pa.nz = nz_;
    pa.ndirs = ndirs_;
    pa.nphases = nph_;
    pa.fastSI = opt.p.bFastSIM;
    pa.nimg = nimg_;
    pa.bg = d_bgslope_;
    pa.slope = d_bgslope_ ? d_bgslope_ + (size_t)nx_raw_ * ny_ : nullptr;
    pa.bgconst = opt.p.constbkgd;
    pa.bgx = d_bgx_;
    pa.inscale = opt.ip.inscale;
    pa.deskew_factor = deskew_factor_;
    pa.extra_shift = opt.p.extraShift;
    pa.out = d_pre_;
    check_launch(launch_precondition(pa, stream_, &launches_), "deskew / crop");
    ia.raw = d_pre_;
    ia.raw_is_u16 = 0;
    ia.bg = nullptr;
    ia.slope = nullptr;
    ia.bgconst = 0.f;
    ia.inscale = 1.f;
  }
  check_launch(launch_ingest(ia, stream_, &launches_), "ingest");
  // processOneVolume without loadAndRescaleImage uses unit ratios
  check_launch(launch_fill(d_scale_, (size_t)ndirs_ * nph_ * nz_, 1.0f, stream_, &launches_), "scale init");
  stage_end("ingest", a, l0);
  rescaled_ = false;
}

void SIM_Reconstructor::set_raw_float(const float* raw, int nx, int ny, int nz)
{
  if (nx != nx_raw_ || ny != ny_ || nz != nimg_)
    throw std::runtime_error("setRaw: shape does not match the reconstructor");
  stage_raw(raw, false);
}

void SIM_Reconstructor::set_raw_u16(const uint16_t* raw, int nx, int ny, int nz)
{
  if (nx != nx_raw_ || ny != ny_ || nz != nimg_)
    throw std::runtime_error("setRaw: shape does not match the reconstructor");
  stage_raw(raw, true);
}

// loadAndRescaleImage -> rescaleDriver (cudaSirecon.cpp:520-540, 1323-1329)
void SIM_Reconstructor::load_and_rescale(int it, int iw)
{
  TimerScope ts(this);
  (void)iw;
  if (!have_raw_) throw std::runtime_error("loadAndRescaleImage before setRaw/setFile");
  if (opt.p.bBessel && opt.p.bNoRecon) return;  // cudaSirecon.cpp:1325
  if (!opt.p.do_rescale) return;
  cudaEvent_t a;
  long long l0;
  stage_begin("rescale", &a, &l0);
  check_launch(launch_rescale(d_spec_, nx_, ny_, nz_, ndirs_, nph_, it, opt.p.equalizez, opt.p.equalizet, d_sdp0_,
                              d_scale_, stream_, &launches_),
               "rescale");
  stage_end("rescale", a, l0);
  rescaled_ = true;
}

void SIM_Reconstructor::separate()
{
  TimerScope ts(this);
  cudaEvent_t a;
  long long l0;
  stage_begin("separate", &a, &l0);
  check_launch(launch_separate(d_spec_, d_scale_, d_sepmat_, nx_, ny_, nz_, ndirs_, nph_, stream_, &launches_),
               "separate");
  stage_end("separate", a, l0);
}

// ------------------------------------------------------------------ fitting
void SIM_Reconstructor::build_overlaps(int d, int o1, int o2, float k0x, float k0y, const float2* kdev, float kfac,
                                       float2* pmap, double* sumxy, int lane)
{
  cudaStream_t s = lane_stream(lane);
  const ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  OverlapArgs a{};
  a.bands = d_spec_ + (size_t)d * nph_ * nz_ * ny_ * nxh_;
  a.nx = nx_;
  a.ny = ny_;
  a.nz = nz_;
  a.order1 = o1;
  a.order2 = o2;
  // makeoverlaps scalars, gpuFunctionsImpl.cu:497-555 (float arithmetic)
  float order0_2_factor = 1.0f;
  if (nz_ > 1) {
    order0_2_factor = 5.0f;
    if (p.bBessel) order0_2_factor = 4.0f;
  }
  float dxy = ip.dxy;
  float dkx = 1.0f / (nx_ * dxy);
  float dky = 1.0f / (ny_ * dxy);
  float dkz = ip.dz > 0.0f ? 1.0f / (nz_ * ip.dz) : p.dkzotf;
  float kzscale = dkz / p.dkzotf;
  float rdistcutoff = p.na * 2.0 / (ip.wave[0] * 0.001);
  if (rdistcutoff > 1. / (2. * dxy)) rdistcutoff = 1. / (2. * dxy);
  a.kx = k0x * (o2 - o1);
  a.ky = k0y * (o2 - o1);
  a.kdev = kdev;  // a k0 fitted on the device (not in Bessel mode, whose zdc depends on |k0|)
  a.kfac = kfac;
  a.dkx = dkx;
  a.dky = dky;
  a.rdistcutoff = rdistcutoff;
  a.otfcutoff = p.bBessel ? 0.01f : p.otfcutoff;
  a.order0_2_factor = order0_2_factor;
  a.zdc = p.bBessel ? overlap_zdc_bessel(o2, k0x, k0y) : zdc_ovl_;
  a.nokz0 = effective_nokz0(opt);
  const int dir_ = p.bOneOTFperAngle ? d : 0;
  for (int o = 0; o < norders_; ++o)
    a.otf.otf[o] = d_otf_ + ((size_t)dir_ * norders_ + o) * p.nxotf * p.nzotf;
  a.otf.nzotf = p.nzotf;
  a.otf.nxotf = p.nxotf;
  a.otf.dkrotf = p.dkrotf;
  a.otf.kzscale = kzscale;
  a.ovl = d_ovl_ + lane * ovl_lane_elems();
  a.ppart = d_ppart_ + lane * ppart_lane_elems();
  a.sums = d_sums_ + lane * sums_lane_elems();
  a.pmap = pmap ? pmap : lane_pmap(lane);
  a.sumxy = sumxy ? sumxy : d_sumxy_ + 2 * lane;
  check_launch(launch_overlaps(a, s, &launches_), "makeoverlaps");
  ++fit_counts_[0];
  last_ovl_ = a;
  cur_o1_ = o1;
  cur_o2_ = o2;
  cache_.clear();
  sumx_ = sumy_ = -1;
}

// makeoverlaps' zdistcutoff in Bessel mode (gpuFunctionsImpl.cu:533-548): it
// depends on the pattern's magnitude and the order built; clamped like the
// widefield one to nz/2 - 1 (never more than the overlap buffers hold)
int SIM_Reconstructor::overlap_zdc_bessel(int order2, float k0x, float k0y) const
{
  const ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  float dkz = ip.dz > 0.0f ? 1.0f / (nz_ * ip.dz) : p.dkzotf;
  float k0mag = sqrt(k0x * k0x + k0y * k0y);
  float lambdaem = (ip.wave[0] / p.nimm) / 1.0e3;
  float alpha = asinf(p.na / p.nimm);
  float kzExMax = 2.0 * p.BesselNA / p.BesselLambdaEx;
  float halfangle = acosf(k0mag * order2 / (p.norders - 1) / kzExMax);
  float zd = ceil((kzExMax * sinf(halfangle) + (1.0 - cosf(alpha)) / lambdaem) / dkz);
  const int zmax = (nz_ / 2 - 1) > 0 ? (nz_ / 2 - 1) : 0;
  if (!(zd <= nz_ / 2)) zd = zmax;  // also a NaN half angle
  return std::min((int)zd, zdc_ovl_);
}

// XStarY for a batch of (angle, mag) candidates, cached as modamp1 = XStarY/sumX
void SIM_Reconstructor::eval_candidates(int o1, int o2, const std::vector<std::pair<float, float>>& cands)
{
  std::vector<std::pair<float, float>> todo;
  for (auto& c : cands)
    if (!cache_.count({fbits(c.first), fbits(c.second)})) todo.push_back(c);
  for (size_t b0 = 0; b0 < todo.size(); b0 += kMaxCand) {
    size_t nc = std::min<size_t>(kMaxCand, todo.size() - b0);
    CandList kc{};
    for (size_t i = 0; i < nc; ++i) {
      float angle = todo[b0 + i].first, mag = todo[b0 + i].second;
      // getmodamp: k1 = klength*(cosf, sinf)(kangle); findrealspacemodamp: k1*(order2-order1)
      float k1x = mag * cosf(angle), k1y = mag * sinf(angle);
      kc.k[i] = make_float2(k1x * (o2 - o1), k1y * (o2 - o1));
    }
    check_launch(launch_modamp_candidates(d_pmap_, nx_, ny_, opt.ip.dxy, kc, (int)nc, d_tables_, d_partial_,
                                          d_xstary_, stream_, &launches_),
                 "modamp");
    fit_counts_[1] += (long long)nc;
    check_launch(launch_copy_out(d_xstary_, dh_pinned_, nc * 4, d_sumxy_, dh_pinned_ + 2 * kMaxCand, 4, stream_,
                                 &launches_),
                 "d2h");
    check(cudaStreamSynchronize(stream_), "modamp");
    sumx_ = h_pinned_[2 * kMaxCand];
    sumy_ = h_pinned_[2 * kMaxCand + 1];
    float sx = (float)sumx_;
    for (size_t i = 0; i < nc; ++i) {
      float xr = (float)h_pinned_[2 * i], xi = (float)h_pinned_[2 * i + 1];
      cache_[{fbits(todo[b0 + i].first), fbits(todo[b0 + i].second)}] = float2v{xr / sx, xi / sx};
    }
  }
}

// getmodamp (gpuFunctionsImpl.cu:1046-1072); redo rebuilds the overlaps at k1
float SIM_Reconstructor::getmodamp(int d, float angle, float mag, int o1, int o2, int redo, float2v* modamp)
{
  if (redo || o1 != cur_o1_ || o2 != cur_o2_) {
    float k1x = mag * cosf(angle), k1y = mag * sinf(angle);
    build_overlaps(d, o1, o2, k1x, k1y);
  }
  auto key = std::make_pair(fbits(angle), fbits(mag));
  if (!cache_.count(key)) eval_candidates(o1, o2, {{angle, mag}});
  float2v m = cache_[key];
  if (modamp) *modamp = m;
  return m.x * m.x + m.y * m.y;
}

// queue `count` candidates along the search line (float-accumulated steps,
// exactly the values the sequential search would visit)
void SIM_Reconstructor::prefetch_line(int o1, int o2, bool angle_axis, float fixed, float start, float step,
                                      int count, int dir)
{
  std::vector<std::pair<float, float>> c;
  float x = start;
  for (int i = 0; i < count; ++i) {
    x = dir > 0 ? x + step : x - step;
    c.push_back(angle_axis ? std::make_pair(x, fixed) : std::make_pair(fixed, x));
  }
  eval_candidates(o1, o2, c);
}

// findrealspacemodamp (gpuFunctionsImpl.cu:1074-1148): modamp1 at k0
float2v SIM_Reconstructor::findrealspacemodamp(int d, int o1, int o2, float k0x, float k0y, int redo)
{
  if (redo || o1 != cur_o1_ || o2 != cur_o2_) build_overlaps(d, o1, o2, k0x, k0y);
  // the candidate kernel takes (angle, mag) pairs; pass k0 through an exact
  // (angle, mag) key by evaluating directly
  CandList kc{};
  kc.k[0] = make_float2(k0x * (o2 - o1), k0y * (o2 - o1));
  check_launch(launch_modamp_candidates(d_pmap_, nx_, ny_, opt.ip.dxy, kc, 1, d_tables_, d_partial_, d_xstary_,
                                        stream_, &launches_),
               "modamp");
  ++fit_counts_[1];
  check_launch(launch_copy_out(d_xstary_, dh_pinned_, 4, d_sumxy_, dh_pinned_ + 2, 4, stream_, &launches_), "d2h");
  check(cudaStreamSynchronize(stream_), "modamp");
  float sx = (float)h_pinned_[2];
  return float2v{(float)h_pinned_[0] / sx, (float)h_pinned_[1] / sx};
}

// findk0 (gpuFunctionsImpl.cu:306-372)
void SIM_Reconstructor::findk0(int d)
{
  const int fitorder2 = nz_ > 1 && !opt.p.bBessel ? 2 : 1;
  float2v k0 = k0_[d];
  build_overlaps(d, 0, fitorder2, k0.x, k0.y);
  check_launch(launch_crosscorr_peak(d_pmap_, d_cc_, nx_, ny_, d_bval_, d_bidx_, d_peak_, stream_, &launches_),
               "crosscorr");
  ++fit_counts_[1];  // the cross-correlation reads the overlap pair once, like a modamp reduction
  float* pk = (float*)(h_pinned_ + 256);
  check_launch(launch_copy_out(d_peak_, dh_pinned_ + 256, 7, nullptr, nullptr, 0, stream_, &launches_), "d2h");
  check(cudaStreamSynchronize(stream_), "findk0");
  int xcent = (int)pk[0], ycent = (int)pk[1];
  float peakx = fitparabola(pk[2], pk[3], pk[4]) + xcent;
  float peaky = fitparabola(pk[5], pk[3], pk[6]) + ycent;
  float dxy = opt.ip.dxy;
  float dkx = 1 / (nx_ * dxy);
  float dky = 1 / (ny_ * dxy);
  if (k0.x / dkx < peakx - nx_ / 2) peakx -= nx_;
  if (k0.x / dkx > peakx + nx_ / 2) peakx += nx_;
  if (k0.y / dky < peaky - ny_ / 2) peaky -= ny_;
  if (k0.y / dky > peaky + ny_ / 2) peaky += ny_;
  k0_[d].x = peakx * (dkx / fitorder2);
  k0_[d].y = peaky * (dky / fitorder2);
}

// fitk0andmodamps (gpuFunctionsImpl.cu:874-1020).  The search visits the same
// float-accumulated angles and magnitudes as the reference; their modamps are
// evaluated in batches on the device and the sequential logic reads them
// from a cache.
void SIM_Reconstructor::fitk0andmodamps(int d)
{
  ReconParams& p = opt.p;
  const int fitorder1 = 0;
  const int fitorder2 = nz_ > 1 && !opt.p.bBessel ? 2 : 1;
  float2v* k0 = &k0_[d];
  float k0mag = sqrt(k0->x * k0->x + k0->y * k0->y);
  float k0angle = atan2(k0->y, k0->x);
  int redoarrays = (p.recalcarrays >= 1);
  float x2 = k0angle;
  float2v modamp;
  float amp2 = getmodamp(d, k0angle, k0mag, fitorder1, fitorder2, redoarrays, &modamp);
  redoarrays = (p.recalcarrays >= 3);
  float deltaangle = 0.001;
  float deltamag = 0.1 / (std::max(nx_, ny_) * opt.ip.dxy);
  const int K = 12;
  // each climb stops after kMaxClimbSteps (the reference's loops have no
  // bound; it only ends a climb whose amplitude never peaks)
  // both directions of the angle search in one batch
  prefetch_line(fitorder1, fitorder2, true, k0mag, k0angle, deltaangle, K, +1);
  prefetch_line(fitorder1, fitorder2, true, k0mag, k0angle, deltaangle, K, -1);
  float angle = k0angle + deltaangle;
  float x3 = angle;
  float amp3 = getmodamp(d, angle, k0mag, fitorder1, fitorder2, redoarrays, &modamp);
  float amp1 = 0, x1 = 0.0, a;
  int steps = 0;
  if (amp3 > amp2) {
    while (amp3 > amp2 && steps < kMaxClimbSteps) {
      amp1 = amp2;
      x1 = x2;
      amp2 = amp3;
      x2 = x3;
      angle += deltaangle;
      x3 = angle;
      if (++steps % K == K - 1) prefetch_line(fitorder1, fitorder2, true, k0mag, angle, deltaangle, K, +1);
      amp3 = getmodamp(d, angle, k0mag, fitorder1, fitorder2, redoarrays, &modamp);
    }
  } else {
    angle = k0angle;
    a = amp3;
    amp3 = amp2;
    amp2 = a;
    a = x3;
    x3 = x2;
    x2 = a;
    while (amp3 > amp2 && steps < kMaxClimbSteps) {
      amp1 = amp2;
      x1 = x2;
      amp2 = amp3;
      x2 = x3;
      angle -= deltaangle;
      x3 = angle;
      if (++steps % K == K - 1) prefetch_line(fitorder1, fitorder2, true, k0mag, angle, deltaangle, K, -1);
      amp3 = getmodamp(d, angle, k0mag, fitorder1, fitorder2, redoarrays, &modamp);
    }
  }
  angle = fitxyparabola(x1, amp1, x2, amp2, x3, amp3);

  x2 = k0mag;
  // magnitude search at the fitted angle
  std::vector<std::pair<float, float>> first = {{angle, k0mag}};
  eval_candidates(fitorder1, fitorder2, first);
  prefetch_line(fitorder1, fitorder2, false, angle, k0mag, deltamag, K, +1);
  prefetch_line(fitorder1, fitorder2, false, angle, k0mag, deltamag, K, -1);
  amp2 = getmodamp(d, angle, k0mag, fitorder1, fitorder2, redoarrays, &modamp);
  float mag = k0mag + deltamag;
  x3 = mag;
  amp3 = getmodamp(d, angle, mag, fitorder1, fitorder2, redoarrays, &modamp);
  steps = 0;
  if (amp3 > amp2) {
    while (amp3 > amp2 && steps < kMaxClimbSteps) {
      amp1 = amp2;
      x1 = x2;
      amp2 = amp3;
      x2 = x3;
      mag += deltamag;
      x3 = mag;
      if (++steps % K == K - 1) prefetch_line(fitorder1, fitorder2, false, angle, mag, deltamag, K, +1);
      amp3 = getmodamp(d, angle, mag, fitorder1, fitorder2, redoarrays, &modamp);
    }
  } else {
    mag = k0mag;
    a = amp3;
    amp3 = amp2;
    amp2 = a;
    a = x3;
    x3 = x2;
    x2 = a;
    while (amp3 > amp2 && steps < kMaxClimbSteps) {
      amp1 = amp2;
      x1 = x2;
      amp2 = amp3;
      x2 = x3;
      mag -= deltamag;
      x3 = mag;
      if (++steps % K == K - 1) prefetch_line(fitorder1, fitorder2, false, angle, mag, deltamag, K, -1);
      amp3 = getmodamp(d, angle, mag, fitorder1, fitorder2, redoarrays, &modamp);
    }
  }
  mag = fitxyparabola(x1, amp1, x2, amp2, x3, amp3);

  redoarrays = (p.recalcarrays >= 2);
  getmodamp(d, angle, mag, fitorder1, fitorder2, redoarrays, &modamp);
  k0->x = mag * cosf(angle);
  k0->y = mag * sinf(angle);
  amp_[d][fitorder2] = modamp;
  redoarrays = 1;
  if (nz_ == 1) {
    for (int order = 2; order < norders_; ++order) {
      getmodamp(d, angle, mag, order - 1, order, redoarrays, &modamp);
      amp_[d][order] = modamp;
    }
  } else {
    for (int order = 1; order < norders_; ++order) {
      if (order != fitorder2) {
        getmodamp(d, angle, mag, 0, order, redoarrays, &modamp);
        amp_[d][order] = modamp;
      }
    }
  }
}

// findModulationVectorsAndPhasesForAllDirections, k0 / modamp part with a
// k0 search (cudaSirecon.cpp:296-408, 450-492)
void SIM_Reconstructor::fit_direction(int direction)
{
  ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  k0_[direction] = k0guess_[direction];
  cur_o1_ = cur_o2_ = -1;  // overlaps belong to another direction
  ++fit_counts_[2];
  findk0(direction);
  p.recalcarrays = 1;
  fitk0andmodamps(direction);
  if (ip.curTimeIdx == 0) k0_time0_[direction] = k0_[direction];
  float dx = k0_[direction].x - k0guess_[direction].x, dy = k0_[direction].y - k0guess_[direction].y;
  float dist = sqrt(dx * dx + dy * dy);
  if (ip.ntimes > 1 && ip.curTimeIdx > 0 && dist > 2 * kK0WarningThresh) {
    k0_[direction] = k0_time0_[direction];
    for (int order = 1; order < norders_; ++order) {
      int o1 = nz_ > 1 ? 0 : order - 1;
      amp_[direction][order] = findrealspacemodamp(direction, o1, order, k0_[direction].x, k0_[direction].y, 1);
    }
  }
  if (ip.nz == 1)
    for (int order = 2; order < norders_; ++order)
      amp_[direction][order] = cmulh(amp_[direction][order], amp_[direction][order - 1]);
  if (p.forceamp.size() > 0 && p.forceamp[0] > 0.0) {
    for (int order = 1; order < norders_; ++order) {
      float a = cmagh(amp_[direction][order]);
      float want = (size_t)(order - 1) < p.forceamp.size() ? p.forceamp[order - 1] : 0.f;
      if (a < want) {
        float ampfact = want / a;
        amp_[direction][order].x *= ampfact;
        amp_[direction][order].y *= ampfact;
      }
    }
  }
  if (!p.bFitallphases) {
    float base_phase = atan2(amp_[direction][1].y, amp_[direction][1].x);
    for (int order = 2; order < norders_; ++order) {
      float2v amplitude{cmagh(amp_[direction][order]), 0};
      float phi = order * base_phase;
      float2v expiphi{cosf(phi), sinf(phi)};
      amp_[direction][order] = cmulh(amplitude, expiphi);
    }
  }
}

// Whether this volume's fit makes no host decision: k0 known (reused from
// time 0 or no search), only the modamps are evaluated
bool SIM_Reconstructor::fit_without_search() const
{
  const ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  const bool reuse = ip.ntimes > 1 && ip.curTimeIdx > 0 && p.bUseTime0k0;
  return reuse || !p.bSearchforvector;
}

void SIM_Reconstructor::fit_all()
{
  TimerScope ts(this);
  cudaEvent_t a;
  long long l0;
  stage_begin("fit", &a, &l0);
  if (fit_without_search()) {
    fit_on_device();
  } else if (!device_search_possible() || !fit_search_on_device()) {
    for (int d = 0; d < ndirs_; ++d) fit_direction(d);
    check_launch(upload_amps(), "fit results");
  }
  stage_end("fit", a, l0);
}

// The k0 search runs on the device unless a host decision is part of it:
// Bessel mode (the overlaps' kz range depends on |k0|), a later time point
// that may fall back to time 0's k0, the overlap debug dump after findk0.
bool SIM_Reconstructor::device_search_possible() const
{
  const ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  if (!device_search_ || p.bBessel || debug_requested()) return false;
  if (ip.ntimes > 1 && ip.curTimeIdx > 0) return false;
  return k0_search_supported(nx_, ny_);
}

// findModulationVectorsAndPhasesForAllDirections with a k0 search
// (cudaSirecon.cpp:296-408, 450-492) on the device: per direction findk0
// (overlaps at the guess, cross-correlation peak, parabola refinement), the
// overlaps rebuilt at the refined k0, the cluster search of fitk0andmodamps,
// then the other orders' amplitudes at the fitted k0; the amplitudes are
// finished like the no-search branch's.  One synchronisation at the end
// brings the fitted k0 to the host (the filter's set-up needs it).  Returns
// false, having changed nothing the host search depends on, when a climb
// left the device's line cache; the host search then runs instead.
bool SIM_Reconstructor::fit_search_on_device()
{
  ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  const int fo2 = nz_ > 1 ? 2 : 1;
  const float dxy = ip.dxy;
  const float dkx = 1 / (nx_ * dxy), dky = 1 / (ny_ * dxy);
  check(cudaMemsetAsync(d_sinfo_, 0, 2 * sizeof(int), stream_), "fit");
  long long builds = 0, reductions = 0;
  K0SearchArgs sa{};
  const size_t nxy = (size_t)nx_ * ny_;
  // each direction's findk0 and first overlap rebuild on its fit lane
  const int nl0 = lanes_begin();
  for (int d = 0; d < ndirs_; ++d) {
    k0_[d] = k0guess_[d];
    float2* kfind = d_kst_ + 3 * d;
    float2* k1 = kfind + 1;
    const int lane = d % nl0;
    cudaStream_t ls = lane_stream(lane);
    float* peak = d_peak_ + 8 * lane;
    build_overlaps(d, 0, fo2, k0guess_[d].x, k0guess_[d].y, nullptr, 0.f, nullptr, nullptr, lane);
    check_launch(launch_crosscorr_peak(lane_pmap(lane), d_cc_ + lane * nxy, nx_, ny_, d_bval_ + 256 * lane,
                                       d_bidx_ + 256 * lane, peak, ls, &launches_),
                 "crosscorr");
    check_launch(launch_findk0_finish(peak, make_float2(k0guess_[d].x, k0guess_[d].y), nx_, ny_, dkx, dky, fo2,
                                      kfind, k1, ls, &launches_),
                 "findk0");
    // fitk0andmodamps' first getmodamp rebuilds the overlaps at k1; every
    // direction keeps its map for the searches, which run side by side
    build_overlaps(d, 0, fo2, 0.f, 0.f, k1, (float)fo2, d_pmapd_ + d * nxy, d_sumxyd_ + 2 * d, lane);
    sa.pmap[d] = d_pmapd_ + d * nxy;
    sa.sumxy[d] = d_sumxyd_ + 2 * d;
    sa.k0find[d] = kfind;
    sa.k0fit[d] = kfind + 2;
    sa.slot[d] = d_fitslots_ + (size_t)(d * norders_ + fo2) * 4;
    builds += 2;
    reductions += 1;  // the cross-correlation
  }
  lanes_end(nl0);
  sa.info = d_sinfo_;
  sa.ndirs = ndirs_;
  sa.nx = nx_;
  sa.ny = ny_;
  sa.fitorder2 = fo2;
  sa.dxy = dxy;
  sa.delta_angle = 0.001f;
  sa.delta_mag = 0.1 / (std::max(nx_, ny_) * dxy);
  check_launch(launch_k0_search(sa, stream_, &launches_), "k0 search");
  const int nl = lanes_begin();
  for (int d = 0; d < ndirs_; ++d) {
    float2* kfit = d_kst_ + 3 * d + 2;
    // the other orders at the fitted k0 (overlaps rebuilt each time)
    for (int order = 1; order < norders_; ++order) {
      const int o1 = nz_ == 1 ? order - 1 : 0;
      if (nz_ == 1 ? order < 2 : order == fo2) continue;
      const int lane = (d * (norders_ - 1) + order - 1) % nl;
      cudaStream_t ls = lane_stream(lane);
      build_overlaps(d, o1, order, 0.f, 0.f, kfit, (float)(order - o1), nullptr, nullptr, lane);
      check_launch(launch_modamp_device_k(lane_pmap(lane), nx_, ny_, dxy, kfit, (float)(order - o1),
                                          lane_tables(lane), lane_partial(lane), lane_xstary(lane), ls, &launches_),
                   "modamp");
      double* slot = d_fitslots_ + (size_t)(d * norders_ + order) * 4;
      check_launch(launch_copy_out(lane_xstary(lane), slot, 4, d_sumxy_ + 2 * lane, slot + 2, 4, ls, &launches_),
                   "modamp");
      ++builds;
      ++reductions;
    }
  }
  lanes_end(nl);
  check_launch(launch_fit_finish(d_fitslots_, fit_finish_args(), d_fit_, stream_, &launches_), "fit results");
  // the fitted k0s and the search's counters through mapped host memory
  double* base = dh_pinned_ + 320;
  check_launch(launch_copy_out(d_kst_, base, (size_t)ndirs_ * 6, d_sinfo_, base + 32, 2, stream_, &launches_),
               "fit results");
  check(cudaStreamSynchronize(stream_), "k0 search");
  const float* kst = (const float*)(h_pinned_ + 320);
  const int* info = (const int*)(h_pinned_ + 352);
  fit_counts_[0] += builds;
  fit_counts_[1] += reductions + info[0];
  fit_counts_[2] += ndirs_;
  cur_o1_ = cur_o2_ = -1;
  cache_.clear();
  if (info[1] != 0) return false;  // a climb left the line cache: the host search runs
  for (int d = 0; d < ndirs_; ++d) {
    k0_[d] = float2v{kst[6 * d + 4], kst[6 * d + 5]};
    if (ip.curTimeIdx == 0) k0_time0_[d] = k0_[d];
  }
  p.recalcarrays = 1;  // fit_direction's setting, kept for callers that read it
  amps_on_device_only_ = true;
  return true;
}

FitFinishArgs SIM_Reconstructor::fit_finish_args() const
{
  const ReconParams& p = opt.p;
  FitFinishArgs fa{};
  fa.ndirs = ndirs_;
  fa.norders = norders_;
  fa.chain2d = opt.ip.nz == 1;
  fa.nforce = (int)std::min<size_t>(p.forceamp.size(), kMaxOrders);
  for (int i = 0; i < fa.nforce; ++i) fa.forceamp[i] = p.forceamp[i];
  fa.fitallphases = p.bFitallphases;
  for (int i = 0; i < ndirs_ * norders_; ++i) {
    fa.noisevar[i] = noisevar_[i];
    fa.rnv[i] = 1.f / noisevar_[i];
  }
  return fa;
}

// the host's amplitudes (after a k0 search) into the device fit results
int SIM_Reconstructor::upload_amps()
{
  AmpList al{};
  for (int d = 0; d < ndirs_; ++d)
    for (int o = 0; o < norders_; ++o) al.amp[d * norders_ + o] = make_float2(amp_[d][o].x, amp_[d][o].y);
  amps_on_device_only_ = false;
  return launch_set_fit(al, fit_finish_args(), d_fit_, stream_, &launches_);
}

// The no-search branch (cudaSirecon.cpp:409-449 and the amplitude rules
// after it): findrealspacemodamp(d, 0, order, k0) for every direction and
// order, each XStarY / sum|X|^2 kept in device memory, the amplitudes
// finished on the device.  No copy and no synchronisation: the host learns
// the amplitudes only when asked (get_fit).
void SIM_Reconstructor::fit_on_device()
{
  const ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  const bool reuse = ip.ntimes > 1 && ip.curTimeIdx > 0 && p.bUseTime0k0;
  // the (direction, order) overlap pairs are independent: each runs on its
  // own fit lane (stream and working buffers), joined before the amplitudes
  // are finished
  const int nl = lanes_begin();
  for (int d = 0; d < ndirs_; ++d) {
    if (!reuse) k0_[d] = k0guess_[d];
    const float2v k = k0_[d];
    for (int order = 1; order < norders_; ++order) {
      const int lane = (d * (norders_ - 1) + order - 1) % nl;
      build_overlaps(d, 0, order, k.x, k.y, nullptr, 0.f, nullptr, nullptr, lane);
      CandList kc{};
      kc.k[0] = make_float2(k.x * order, k.y * order);
      check_launch(launch_modamp_candidates(lane_pmap(lane), nx_, ny_, ip.dxy, kc, 1, lane_tables(lane),
                                            lane_partial(lane), lane_xstary(lane), lane_stream(lane), &launches_),
                   "modamp");
      ++fit_counts_[1];
      double* slot = d_fitslots_ + (size_t)(d * norders_ + order) * 4;
      check_launch(launch_copy_out(lane_xstary(lane), slot, 4, d_sumxy_ + 2 * lane, slot + 2, 2, lane_stream(lane),
                                   &launches_),
                   "modamp");
    }
  }
  lanes_end(nl);
  check_launch(launch_fit_finish(d_fitslots_, fit_finish_args(), d_fit_, stream_, &launches_), "modamp");
  cur_o1_ = cur_o2_ = -1;
  amps_on_device_only_ = true;
}

// Fit lanes: per-lane working buffers of the overlap builds and amplitude
// evaluations, and the lane's stream (lane 0: the handle's stream)
size_t SIM_Reconstructor::ovl_lane_elems() const { return 2 * (size_t)(2 * zdc_ovl_ + 1) * nx_ * ny_; }
size_t SIM_Reconstructor::ppart_lane_elems() const { return (size_t)(2 * zdc_ovl_ + 1) * nx_ * ny_; }
size_t SIM_Reconstructor::sums_lane_elems() const { return 2 * (size_t)(nx_ + 1) * (2 * zdc_ovl_ + 1); }
size_t SIM_Reconstructor::tables_lane_elems() const { return (size_t)kMaxCand * (nx_ + ny_); }
size_t SIM_Reconstructor::partial_lane_elems() const { return (size_t)kModampBlocks * kMaxCand * 2; }
float2* SIM_Reconstructor::lane_pmap(int l) const { return d_pmap_ + (size_t)l * nx_ * ny_; }
float2* SIM_Reconstructor::lane_tables(int l) const { return d_tables_ + l * tables_lane_elems(); }
double* SIM_Reconstructor::lane_partial(int l) const { return d_partial_ + l * partial_lane_elems(); }
double* SIM_Reconstructor::lane_xstary(int l) const { return d_xstary_ + (size_t)l * kMaxCand * 2; }
cudaStream_t SIM_Reconstructor::lane_stream(int l) const { return l == 0 ? stream_ : fit_stream_[l]; }

// fork the fit lanes off the handle's stream; returns how many are used (one
// while profiling, so that every kernel's CUDA-event time is its own)
int SIM_Reconstructor::lanes_begin()
{
  const int nl = profiling_ ? 1 : fit_lanes_;
  if (nl > 1) {
    check(cudaEventRecord(fit_fork_, stream_), "fit fork");
    for (int l = 1; l < nl; ++l) check(cudaStreamWaitEvent(fit_stream_[l], fit_fork_, 0), "fit fork");
  }
  return nl;
}

void SIM_Reconstructor::lanes_end(int nl)
{
  for (int l = 1; l < nl; ++l) {
    check(cudaEventRecord(fit_join_[l], fit_stream_[l]), "fit join");
    check(cudaStreamWaitEvent(stream_, fit_join_[l], 0), "fit join");
  }
}

// the device's amplitudes into amp_ (waits for the stream)
void SIM_Reconstructor::sync_amps() const
{
  if (!amps_on_device_only_) return;
  FitDev f;
  check(cudaStreamSynchronize(stream_), "fit results");
  check(cudaMemcpy(&f, d_fit_, sizeof(FitDev), cudaMemcpyDeviceToHost), "fit results");
  for (int d = 0; d < ndirs_; ++d)
    for (int o = 0; o < norders_; ++o) amp_[d][o] = float2v{f.amp[d * norders_ + o].x, f.amp[d * norders_ + o].y};
  amps_on_device_only_ = false;
}

// ------------------------------------------------------ filter + assembly
// zdistcutoff of every order after filtering (filterbands,
// gpuFunctionsImpl.cu:1253-1289): the kz planes each band keeps
void SIM_Reconstructor::filter_zdc(int* zdc) const
{
  const ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  float dkz = ip.dz > 0 ? (1 / (nz_ * ip.dz)) : p.dkzotf;
  float lambdaem = (ip.wave[0] / p.nimm) / 1000.0;
  float lambdaexc = 0.88 * lambdaem;
  float alpha = asinf(p.na / p.nimm);
  for (int o = 0; o < kMaxOrders; ++o) zdc[o] = 0;
  if (p.bBessel) {  // gpuFunctionsImpl.cu:1260-1271
    float k0mag = sqrt(k0_[0].x * k0_[0].x + k0_[0].y * k0_[0].y);
    float kzExMax = 2 * p.BesselNA / p.BesselLambdaEx;
    zdc[0] = (int)rint((kzExMax + (1 - cosf(alpha)) / lambdaem) / dkz);
    for (int order = 1; order < norders_; order++) {
      float halfangle = acosf(k0mag * order / (norders_ - 1) / kzExMax);
      float zd = ceil((kzExMax * sinf(halfangle) + (1.0 - cosf(alpha)) / lambdaem) / dkz);
      zdc[order] = zd == zd ? (int)zd : nz_;  // a NaN half angle: clamped below
    }
  } else {
    zdc[0] = (int)ceil(((1 - cosf(alpha)) / lambdaem) / dkz);
    zdc[norders_ - 1] = 1.3 * zdc[0];
    if (norders_ >= 3)
      for (int order = 1; order < norders_ - 1; order++) zdc[order] = (1 + lambdaem / lambdaexc) * zdc[0];
  }
  for (int order = 0; order < norders_; order++)
    if (zdc[order] >= nz_ / 2) zdc[order] = ((nz_ / 2 - 1) > 0 ? (nz_ / 2 - 1) : 0);
}

// the geometry part of the assembly arguments (no buffers but the tables)
AssembleArgs SIM_Reconstructor::asm_geometry() const
{
  AssembleArgs aa{};
  aa.ndirs = ndirs_;
  aa.norders = norders_;
  aa.nphases = nph_;
  aa.nx = nx_;
  aa.ny = ny_;
  aa.nz = nz_;
  aa.X = X_;
  aa.Y = Y_;
  aa.Z = Z_;
  aa.tables = d_asmtab_;
  return aa;
}

size_t SIM_Reconstructor::asm_table_bytes() const { return assemble_tables_bytes(asm_geometry()); }

bool SIM_Reconstructor::asm_tables_current(const AssembleArgs& aa) const
{
  return asm_tables_valid_ && std::equal(aa.zdc, aa.zdc + kMaxOrders, asm_tables_zdc_);
}

// Upload the assembly's slot tables when the in-band planes changed (the
// first volume, or options changed through SR_getReconParams).  Synchronous:
// called before a volume's launches, never inside a captured graph.
void SIM_Reconstructor::prepare_asm_tables()
{
  AssembleArgs aa = asm_geometry();
  filter_zdc(aa.zdc);
  if (asm_tables_current(aa)) return;
  check(cudaStreamSynchronize(stream_), "assembly tables");
  check_launch(assemble_tables_upload(aa), "assembly tables");
  std::copy(aa.zdc, aa.zdc + kMaxOrders, asm_tables_zdc_);
  asm_tables_valid_ = true;
}

void SIM_Reconstructor::filter_and_assemble()
{
  TimerScope ts(this);
  const ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  cudaEvent_t ev;
  long long l0;
  stage_begin("filter", &ev, &l0);
  // filterbands scalars (gpuFunctionsImpl.cu:1222-1298), float arithmetic
  FilterArgs fa{};
  fa.ndirs = ndirs_;
  fa.norders = norders_;
  fa.nx = nx_;
  fa.ny = ny_;
  fa.nz = nz_;
  float dxy = ip.dxy;
  float dkz = ip.dz > 0 ? (1 / (nz_ * ip.dz)) : p.dkzotf;
  float kzscale = dkz / p.dkzotf;
  float k0mag = sqrt(k0_[0].x * k0_[0].x + k0_[0].y * k0_[0].y);
  float lambdaem = (ip.wave[0] / p.nimm) / 1000.0;
  float lambdaexc = 0.88 * lambdaem;
  float alpha = asinf(p.na / p.nimm);
  float rdistcutoff = (p.na * 2 / (ip.wave[0] / 1000.0));
  if (rdistcutoff > 1. / (2. * dxy)) rdistcutoff = 1. / (2. * dxy);
  int zdc[kMaxOrders] = {0};
  filter_zdc(zdc);
  (void)alpha;
  (void)lambdaexc;
  float apocutoff = rdistcutoff + k0mag * (norders_ - 1);
  float zapocutoff = p.bBessel ? zdc[0] : (norders_ > 1 ? zdc[1] : 0);
  fa.dkx = 1. / (nx_ * dxy);
  fa.dky = 1. / (ny_ * dxy);
  fa.rdistcutoff = rdistcutoff;
  fa.apocutoff = apocutoff;
  fa.zapocutoff = zapocutoff;
  fa.wiener2 = p.wiener * p.wiener;
  for (int o = 0; o < norders_; ++o) fa.zdc[o] = zdc[o];
  for (int d = 0; d < ndirs_; ++d) {
    fa.k0[d] = make_float2(k0_[d].x, k0_[d].y);
    for (int o = 0; o < norders_; ++o) fa.noisevar[d * norders_ + o] = noisevar_[d * norders_ + o];
  }
  fa.fit = d_fit_;
  fa.suppress = p.bSuppress_singularities;
  fa.supp_radius = p.suppression_radius;
  fa.dampen0 = p.bDampenOrder0;
  fa.nokz0 = effective_nokz0(opt);
  fa.filteroverlaps = p.bFilteroverlaps;
  fa.apodizeoutput = p.apodizeoutput;
  fa.bessel = p.bBessel;
  fa.otf.nzotf = p.nzotf;
  fa.otf.nxotf = p.nxotf;
  fa.otf.dkrotf = p.dkrotf;
  fa.otf.kzscale = kzscale;
  for (int o = 0; o < norders_; ++o) fa.otf.otf[o] = d_otf_ + (size_t)o * p.nxotf * p.nzotf;
  const bool one_otf = !p.bOneOTFperAngle || ndirs_otf_ == 1;

  AssembleArgs aa{};
  aa.bands = d_spec_;
  aa.ndirs = ndirs_;
  aa.norders = norders_;
  aa.nphases = nph_;
  aa.nx = nx_;
  aa.ny = ny_;
  aa.nz = nz_;
  aa.X = X_;
  aa.Y = Y_;
  aa.Z = Z_;
  for (int o = 0; o < norders_; ++o) aa.zdc[o] = zdc[o];
  aa.ex = d_ex_;
  aa.ey = d_ey_;
  aa.T = d_T_;
  aa.tcap = tcap_;
  aa.S = d_S_;
  aa.out = d_out_;
  aa.tables = d_asmtab_;
  if (!asm_tables_current(aa)) throw std::runtime_error("assembly tables not prepared for this geometry");
  // the filter runs inside the assembly's band load where it can; else as
  // its own in-place pass per direction (filterbands_kernel1 x 2 + kernel3)
  const bool fused = filter_fusion_ && assemble_filter_fusable(aa, fa, one_otf);
  if (!fused)
    for (int d = 0; d < ndirs_; ++d) {
      const int dir_ = p.bOneOTFperAngle ? d : 0;
      for (int o = 0; o < norders_; ++o)
        fa.otf.otf[o] = d_otf_ + ((size_t)dir_ * norders_ + o) * p.nxotf * p.nzotf;
      fa.dir = d;
      fa.bands = d_spec_ + (size_t)d * nph_ * nz_ * ny_ * nxh_;
      check_launch(launch_filter(fa, stream_, &launches_), "filterbands");
    }
  stage_end("filter", ev, l0);

  stage_begin("assemble", &ev, &l0);
  K0List k0l{};
  for (int d = 0; d < ndirs_; ++d) k0l.k[d] = make_float2(k0_[d].x, k0_[d].y);
  float fact = p.explodefact / 0.5;
  check_launch(launch_ramp_tables(k0l, ndirs_, norders_, X_, Y_, dxy / p.zoomfact, fact, d_ex_, d_ey_, stream_,
                                  &launches_),
               "ramp");
  if (fused) check_launch(launch_assemble_filtered(aa, fa, one_otf, stream_, &launches_), "filter + assemble");
  else check_launch(launch_assemble(aa, stream_, &launches_), "assemble");
  stage_end("assemble", ev, l0);
}

// processOneVolume (cudaSirecon.cpp:1264-1321)
int SIM_Reconstructor::process_one_volume(bool sync)
{
  if (!have_raw_) throw std::runtime_error("processOneVolume before setRaw/setFile");
  if (debug_requested()) {  // dumps, then no reconstruction (cudaSirecon.cpp:1264-1321)
    separate();
    last_result_ = debug_volume();
    have_raw_ = false;
    return last_result_;
  }
  last_result_ = 1;
  separate();
  fit_all();
  prepare_asm_tables();  // after the fit: in Bessel mode the in-band planes depend on k0
  filter_and_assemble();
  if (sync) check(cudaStreamSynchronize(stream_), "processOneVolume");
  have_raw_ = false;  // the bands are consumed (filtered in place)
  return 1;
}

int SIM_Reconstructor::prepare()
{
  if (!have_raw_) throw std::runtime_error("prepare before setRaw");
  separate();
  check(cudaStreamSynchronize(stream_), "prepare");
  have_raw_ = false;
  return 0;
}

int SIM_Reconstructor::get_band(int dir, int b, float* out)
{
  if (dir < 0 || dir >= ndirs_ || b < 0 || b >= nph_) throw std::runtime_error("getBand: index out of range");
  const size_t n = (size_t)nz_ * ny_ * nxh_;
  check(cudaMemcpyAsync(out, d_spec_ + ((size_t)dir * nph_ + b) * n, n * sizeof(float2), cudaMemcpyDeviceToHost,
                        stream_),
        "getBand");
  check(cudaStreamSynchronize(stream_), "getBand");
  return 0;
}

// bgAndSlope / getbg_and_slope (cudaSirecon.cpp:139-192): with usecorr the
// per-pixel background and slope come from the two first sections of an MRC
// calibration file of the data's nx x ny; ingest applies
// (raw - background) * slope * inscale instead of the constant background
bool SIM_Reconstructor::load_corr(std::string* err)
{
  const std::string& path = opt.p.corrfiles;
  MrcFile f;
  std::string e;
  if (!mrc_open(path, &f, &e)) {
    *err = "File " + path + " does not exist";
    return false;
  }
  if (f.hdr.nx != nx_raw_ || f.hdr.ny != ny_ || f.hdr.nz < 2) {
    *err = "calibration file " + path + " has different dimension than data file";
    return false;
  }
  std::vector<float> bg, sl;
  if (!mrc_read_section(f, 0, &bg, err) || !mrc_read_section(f, 1, &sl, err)) return false;
  const size_t n = (size_t)nx_raw_ * ny_;
  if (bg.size() != n || sl.size() != n) {
    *err = "calibration file " + path + ": sections are not real nx x ny images";
    return false;
  }
  if (!d_bgslope_) check(cudaMalloc((void**)&d_bgslope_, 2 * n * sizeof(float)), "calibration buffer");
  check(cudaMemcpy(d_bgslope_, bg.data(), n * sizeof(float), cudaMemcpyHostToDevice), "calibration upload");
  check(cudaMemcpy(d_bgslope_ + n, sl.data(), n * sizeof(float), cudaMemcpyHostToDevice), "calibration upload");
  return true;
}

void SIM_Reconstructor::set_fitted_k0(const float* k0)
{
  for (int d = 0; d < ndirs_; ++d) {
    k0_[d] = float2v{k0[2 * d], k0[2 * d + 1]};
    k0_time0_[d] = k0_[d];
  }
}

void SIM_Reconstructor::get_fit(float* k0, float* amps)
{
  if (amps) sync_amps();
  for (int d = 0; d < ndirs_; ++d) {
    if (k0) {
      k0[2 * d] = k0_[d].x;
      k0[2 * d + 1] = k0_[d].y;
    }
    if (amps)
      for (int o = 0; o < norders_; ++o) {
        amps[2 * (d * norders_ + o)] = amp_[d][o].x;
        amps[2 * (d * norders_ + o) + 1] = amp_[d][o].y;
      }
  }
}

// A volume whose fit makes no host decision (k0 reused from time 0, or no
// search) is one fixed sequence of launches: ingest, bleach correction,
// separation, modamp evaluation and device-side amplitude finish, filter and
// assembly.  It is captured once per raw/output buffer pair as a CUDA graph
// and replayed, with the "raw buffer free" event recorded inside the graph
// right after ingest.
bool SIM_Reconstructor::capture_volume(int b, void* raw, float* out, int t, cudaEvent_t raw_free)
{
  VolumeGraph& g = graphs_[b];
  const bool tnz = t != 0;
  if (g.exec && g.raw == raw && g.out == out && g.t_nonzero == tnz && g.u16 == raw_u16_) return true;
  if (g.exec) {
    cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
  }
  prepare_asm_tables();  // synchronous upload, outside the capture
  d_raw_ = raw;
  d_out_ = out;
  const long long l0 = launches_;
  long long fc0[3];
  std::copy(fit_counts_, fit_counts_ + 3, fc0);
  check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed), "graph capture");
  cudaGraph_t graph = nullptr;
  try {
    have_raw_ = true;
    ingest();
    check(cudaEventRecordWithFlags(raw_free, stream_, cudaEventRecordExternal), "graph event");
    load_and_rescale(t, 0);
    set_cur_time(t);
    separate();
    fit_all();
    filter_and_assemble();
  } catch (...) {
    cudaStreamEndCapture(stream_, &graph);
    if (graph) cudaGraphDestroy(graph);
    launches_ = l0;
    std::copy(fc0, fc0 + 3, fit_counts_);
    throw;
  }
  check(cudaStreamEndCapture(stream_, &graph), "graph capture");
  cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  check(e, "graph instantiate");
  g.launches = launches_ - l0;
  launches_ = l0;
  for (int i = 0; i < 3; ++i) {
    g.fit_counts[i] = fit_counts_[i] - fc0[i];
    fit_counts_[i] = fc0[i];
  }
  g.raw = raw;
  g.out = out;
  g.t_nonzero = tnz;
  g.u16 = raw_u16_;
  return true;
}

void SIM_Reconstructor::drop_graphs()
{
  for (VolumeGraph& g : graphs_) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = VolumeGraph{};
  }
}

void SIM_Reconstructor::process_series(const void* const* raws, bool u16, float* const* outs, int n, int t0,
                                       bool standalone)
{
  if (n <= 0) return;
  if (!raws || !outs) throw std::runtime_error("processSeries: null buffer list");
  const size_t raw_bytes = (size_t)nimg_ * nx_raw_ * ny_ * (u16 ? 2 : 4);
  const size_t out_bytes = out_elems() * sizeof(float);
  if (!d_raw_alt_) {
    check(cudaMalloc(&d_raw_alt_, (size_t)nimg_ * nx_raw_ * ny_ * sizeof(float)), "series raw buffer");
    check(cudaMalloc((void**)&d_out_extra_, out_bytes), "series output buffer");
    series_bytes_ = (size_t)nimg_ * nx_raw_ * ny_ * sizeof(float) + out_bytes;
    d_out_alt_ = d_out_extra_;
    check(cudaStreamCreateWithFlags(&h2d_stream_, cudaStreamNonBlocking), "series stream");
    check(cudaStreamCreateWithFlags(&d2h_stream_, cudaStreamNonBlocking), "series stream");
    for (int b = 0; b < 2; ++b)
      for (cudaEvent_t* e : {&ev_raw_ready_[b], &ev_raw_free_[b], &ev_out_ready_[b], &ev_out_free_[b]})
        check(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "series event");
  }
  void* raw_buf[2] = {d_raw_, d_raw_alt_};
  float* out_buf[2] = {d_out_, d_out_alt_};
  for (int b = 0; b < 2; ++b) {  // both buffers start free
    check(cudaEventRecord(ev_raw_free_[b], stream_), "series event");
    check(cudaEventRecord(ev_out_free_[b], stream_), "series event");
  }
  auto upload = [&](int i) {
    const int b = i & 1;
    check(cudaStreamWaitEvent(h2d_stream_, ev_raw_free_[b], 0), "series wait");
    check(cudaMemcpyAsync(raw_buf[b], raws[i], raw_bytes, cudaMemcpyHostToDevice, h2d_stream_), "series upload");
    check(cudaEventRecord(ev_raw_ready_[b], h2d_stream_), "series event");
  };
  upload(0);
  if (n > 1) upload(1);
  raw_u16_ = u16;
  // graphs are captured per call: options changed between calls through
  // SR_getReconParams take effect on the next call
  drop_graphs();
  try {
    for (int i = 0; i < n; ++i) {
      const int b = i & 1;
      const int t = standalone ? 0 : t0 + i;
      check(cudaStreamWaitEvent(stream_, ev_raw_ready_[b], 0), "series wait");
      check(cudaStreamWaitEvent(stream_, ev_out_free_[b], 0), "series wait");
      set_cur_time(t);
      // the t > 0 volumes of a series with k0 reuse, or every volume without
      // a k0 search; the rescale step differs between t = 0 and t > 0 only
      const bool graph_ok = !profiling_ && fit_without_search();
      if (graph_ok) {
        capture_volume(b, raw_buf[b], out_buf[b], t, ev_raw_free_[b]);
        check(cudaGraphLaunch(graphs_[b].exec, stream_), "graph launch");
        launches_ += graphs_[b].launches;
        for (int c = 0; c < 3; ++c) fit_counts_[c] += graphs_[b].fit_counts[c];
        amps_on_device_only_ = true;
        have_raw_ = false;
        rescaled_ = true;
      } else {
        d_raw_ = raw_buf[b];
        d_out_ = out_buf[b];
        have_raw_ = true;
        ingest();
        check(cudaEventRecord(ev_raw_free_[b], stream_), "series event");
        load_and_rescale(t, 0);
        set_cur_time(t);
        process_one_volume(false);
      }
      if (i + 2 < n) upload(i + 2);
      check(cudaEventRecord(ev_out_ready_[b], stream_), "series event");
      check(cudaStreamWaitEvent(d2h_stream_, ev_out_ready_[b], 0), "series wait");
      check(cudaMemcpyAsync(outs[i], out_buf[b], out_bytes, cudaMemcpyDeviceToHost, d2h_stream_), "series download");
      check(cudaEventRecord(ev_out_free_[b], d2h_stream_), "series event");
    }
  } catch (...) {
    cudaStreamSynchronize(stream_);
    cudaStreamSynchronize(h2d_stream_);
    cudaStreamSynchronize(d2h_stream_);
    drop_graphs();
    d_raw_ = raw_buf[0];
    d_out_ = out_buf[0];
    d_out_alt_ = out_buf[1];
    throw;
  }
  check(cudaStreamSynchronize(stream_), "series compute");
  check(cudaStreamSynchronize(h2d_stream_), "series upload");
  check(cudaStreamSynchronize(d2h_stream_), "series download");
  drop_graphs();
  // getResult after the series returns the last volume; keep the arena's raw
  // buffer as the one setRaw uses
  d_raw_ = raw_buf[0];
  d_out_ = out_buf[(n - 1) & 1];
  d_out_alt_ = out_buf[((n - 1) & 1) ^ 1];
}

// getResult (cudaSirecon.cpp:1620-1634)
void SIM_Reconstructor::get_result(float* out)
{
  check(cudaMemcpyAsync(out, d_out_, out_elems() * sizeof(float), cudaMemcpyDeviceToHost, stream_), "getResult");
  check(cudaStreamSynchronize(stream_), "getResult");
}

double SIM_Reconstructor::bench_device(int steps)
{
  if (!d_flush_) {
    flush_n_ = (size_t)64 << 20;  // 256 MiB of floats: twice the L2
    check(cudaMalloc(&d_flush_, flush_n_ * sizeof(float)), "flush buffer");
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double total = 0;
  for (int s = 0; s < steps; ++s) {
    check_launch(launch_fill(d_flush_, flush_n_, (float)s, stream_, nullptr), "flush");
    cudaEventRecord(a, stream_);
    have_raw_ = true;
    ingest();
    load_and_rescale(opt.ip.curTimeIdx, 0);
    process_one_volume();
    cudaEventRecord(b, stream_);
    check(cudaEventSynchronize(b), "bench");
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    total += ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  have_raw_ = true;
  return total;
}

// The preconditioning buffers when the geometry did not need them at setup
// (bBgInExtHdr alone): allocated on first use, zero backgrounds
void SIM_Reconstructor::ensure_precondition_buffers()
{
  if (d_pre_ && d_bgx_) return;
  const size_t npre = (size_t)nimg_ * nx_ * ny_;
  check(cudaMalloc((void**)&pre_own_, npre * sizeof(float) + (size_t)nimg_ * sizeof(float) + 256),
        "preconditioning buffers");
  d_pre_ = pre_own_;
  d_bgx_ = pre_own_ + npre;
  check(cudaMemset(d_bgx_, 0, (size_t)nimg_ * sizeof(float)), "memset");
  series_bytes_ += npre * sizeof(float) + (size_t)nimg_ * sizeof(float);
}

// ------------------------------------------------------------ debug dumps
namespace {
// IMWrHdr(..., title, ntflag = 1, ...) restated: the title becomes a new
// 80-byte label after the others (the oldest dropped when all ten are used)
void append_label(MrcHeader& h, const char* title, size_t len)
{
  if (h.nlab < 0) h.nlab = 0;
  if (h.nlab >= 10) {
    memmove(h.label[0], h.label[1], 9 * 80);
    h.nlab = 9;
  }
  memset(h.label[h.nlab], 0, 80);
  memcpy(h.label[h.nlab], title, std::min<size_t>(len, 80));
  h.nlab++;
}
}  // namespace

bool SIM_Reconstructor::debug_requested() const
{
  return opt.p.bSaveSeparated || opt.p.bSaveAlignedRaw || opt.p.bSaveOverlaps;
}

// The intermediate files of setup_common (cudaSirecon.cpp:1179-1210): MRC
// mode only, headers copied from the input file's
bool SIM_Reconstructor::open_debug_files(std::string* err)
{
  const ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  auto open = [&](DebugFile& d, const std::string& path, const MrcHeader& h) {
    d.h = h;
    d.f.open(path, std::ios::binary | std::ios::trunc);
    if (!d.f) {
      *err = "File " + path + " can not be created.";
      return false;
    }
    d.f.write((const char*)&d.h, sizeof(MrcHeader));
    d.open = true;
    return true;
  };
  const MrcHeader& in = mrc_in_.hdr;
  if (p.bSaveAlignedRaw) {
    MrcHeader h = in;
    h.mode = 2;
    h.nx = ip.nx;
    h.next = 0;
    if (!open(dbg_aligned_, p.fileRawAligned, h)) return false;
  }
  if (p.bSaveSeparated) {
    MrcHeader h = in;
    h.nx = ip.nx / 2 + 1;  // separated half-spectrum bands
    h.mode = 4;            // complex
    h.next = 0;
    if (!open(dbg_sep_, p.fileSeparated, h)) return false;
  }
  if (p.bSaveOverlaps) {
    MrcHeader h = in;
    h.nz = ip.nz * 2 * p.ndirs * ip.ntimes * ip.nwaves;
    h.nx = ip.nx;
    h.num_waves = 2;    // overlap 0 and 1 as waves 0 and 1
    h.interleaved = 1;  // WZT sequence
    h.mode = 4;         // full-complex overlaps in real space
    h.next = 0;
    if (!open(dbg_ovl_, p.fileOverlaps, h)) return false;
  }
  return true;
}

// the separated bands of direction d, each kz plane a (nx/2+1) x ny complex
// section (cudaSirecon.cpp:275-284)
void SIM_Reconstructor::debug_write_bands(int d)
{
  const size_t plane = (size_t)ny_ * nxh_;
  std::vector<float2> buf((size_t)nph_ * nz_ * plane);
  check(cudaMemcpy(buf.data(), d_spec_ + (size_t)d * nph_ * nz_ * plane, buf.size() * sizeof(float2),
                   cudaMemcpyDeviceToHost),
        "saveprefiltered");
  dbg_sep_.f.write((const char*)buf.data(), buf.size() * sizeof(float2));
}

// The last overlap pair in real space (cudaSirecon.cpp:330-354 after findk0;
// 433-445 in the no-search branch, whose sections start every nx*ny floats
// of the complex buffers -- the reference's pointer arithmetic -- and so
// overlap by half a section)
void SIM_Reconstructor::debug_dump_overlaps(bool search_branch)
{
  const ReconParams& p = opt.p;
  const size_t plane = (size_t)nx_ * ny_, vol = (size_t)nz_ * plane;
  float2* d = nullptr;
  check(cudaMalloc((void**)&d, 2 * vol * sizeof(float2)), "saveoverlaps buffer");
  std::vector<float2> h(2 * vol);
  cudaError_t e = (cudaError_t)launch_overlap_volumes(last_ovl_, d, stream_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  if (e == cudaSuccess) e = cudaMemcpy(h.data(), d, h.size() * sizeof(float2), cudaMemcpyDeviceToHost);
  cudaFree(d);
  check(e, "saveoverlaps");
  if (p.bTIFF) {  // [overlap0 planes, overlap1 planes], each plane 2 nx floats wide
    std::string err;
    if (search_branch && !tiff_write_float(p.fileOverlaps, (const float*)h.data(), 2 * nx_, ny_, 2 * nz_, &err))
      throw std::runtime_error(err);
    return;
  }
  if (!dbg_ovl_.open) return;
  const float* f0 = (const float*)h.data();
  const float* f1 = (const float*)(h.data() + vol);
  for (int z = 0; z < nz_; ++z) {
    const size_t off = search_branch ? 2 * z * plane : z * plane;  // in floats
    dbg_ovl_.f.write((const char*)(f0 + off), 2 * plane * sizeof(float));
    dbg_ovl_.f.write((const char*)(f1 + off), 2 * plane * sizeof(float));
  }
}

// saveIntermediateDataForDebugging (mrc.h:76-97): titles, min/max/mean and close
void SIM_Reconstructor::close_debug_files()
{
  auto fin = [&](DebugFile& d, const char* title, float amin, float amax, float amean) {
    if (!d.open) return;
    append_label(d.h, title, strlen(title));
    d.h.amin = amin;
    d.h.amax = amax;
    d.h.amean = amean;
    d.f.seekp(0);
    d.f.write((const char*)&d.h, sizeof(MrcHeader));
    d.f.close();
    d.open = false;
  };
  fin(dbg_sep_, "separated bands of all directions", 0, 1, 0);
  fin(dbg_aligned_, "drift-corrected raw images", dbg_aligned_.h.amin, dbg_aligned_.h.amax, dbg_aligned_.h.amean);
  fin(dbg_ovl_, "overlaps in real space", 0, 1, 0);
}

// findModulationVectorsAndPhasesForAllDirections with its debug dumps
// (cudaSirecon.cpp:194-494), then the stop of processOneVolume: returns 0
int SIM_Reconstructor::debug_volume()
{
  ReconParams& p = opt.p;
  const ImageParams& ip = opt.ip;
  const bool reuse = ip.ntimes > 1 && ip.curTimeIdx > 0 && p.bUseTime0k0;
  for (int d = 0; d < ndirs_; ++d) {
    if (p.bSaveSeparated) {
      if (p.bTIFF) {
        std::printf("No unmixed raw images were saved in TIFF mode\n");
      } else {
        if (dbg_sep_.open) debug_write_bands(d);
        continue;  // no k0 search or modamp fit for this direction
      }
    }
    cur_o1_ = cur_o2_ = -1;
    if (p.bSearchforvector && !reuse) {
      k0_[d] = k0guess_[d];
      findk0(d);
      if (p.bSaveOverlaps) debug_dump_overlaps(true);
      p.recalcarrays = 1;
      fitk0andmodamps(d);
      if (ip.curTimeIdx == 0) k0_time0_[d] = k0_[d];
    } else {
      if (!reuse) k0_[d] = k0guess_[d];
      for (int order = 1; order < norders_; ++order) {
        amp_[d][order] = findrealspacemodamp(d, 0, order, k0_[d].x, k0_[d].y, 1);
        if (order == 1 && p.bSaveOverlaps) {
          if (p.bTIFF) std::printf("No overlaps were saved in TIFF mode\n");
          else debug_dump_overlaps(false);
        }
      }
    }
  }
  amps_on_device_only_ = false;
  close_debug_files();
  return 0;
}

// ------------------------------------------------------------- FFT tuning
// The kernel (as reported to the per-kernel timer) that runs each FFT site
static const char* site_kernel(int site)
{
  switch (site) {
    case kSiteIngestX: return "k_ingest_x";
    case kSiteIngestY: return "k_fft_y";
    case kSiteSeparateZ: return "k_separate";
    case kSiteOvlX: return "k_ovl_build_x";
    case kSiteOvlY: return "k_ovl_y_accum";
    case kSiteCorrRows:
    case kSiteCorrCols: return "k_crosscorr";
    case kSiteAsmY: return "k_asm_y";
    case kSiteAsmX: return "k_asm_x";
    case kSiteAsmZ: return "k_asm_z";
    default: return nullptr;
  }
}

// Measure, for every (FFT site, length) a volume of this handle queries and
// the register path supports, the site's kernel time with the register path
// and with the Stockham stages, on the staged raw stack (each run restarts
// from it), and record the faster choice in the plan cache.  The volume runs
// as time point 0 (k0 search) so that the search's transforms are included.
std::string SIM_Reconstructor::tune_fft(int reps)
{
  if (!raw_staged_) throw std::runtime_error("tuneFFT: no raw stack staged (SR_setRaw first)");
  const unsigned short t_saved = opt.ip.curTimeIdx;
  const bool prof_saved = profiling_;
  std::set<std::pair<int, int>> seen;
  std::ostringstream out;
  out.precision(6);
  out << "{\"cache\": \"" << fft_plan_cache_path() << "\", \"sites\": [";
  try {
    set_cur_time(0);
    profiling_ = false;
    fft_sites_track(&seen);
    bench_device(1);
    fft_sites_track(nullptr);
    bool first = true;
    for (auto [site, n] : seen) {
      const char* kname = site_kernel(site);
      if (!kname || !reg_fft_lanes(n)) continue;
      double best[2] = {1e30, 1e30};  // [stockham, register]
      for (int rep = 0; rep < std::max(1, reps); ++rep)
        for (int reg = 1; reg >= 0; --reg) {
          fft_site_force(site, reg != 0);
          profiling_ = true;
          reset_profile();
          bench_device(1);
          profile_json();
          profiling_ = false;
          fft_site_unforce();
          auto it = kprof_.find(kname);
          if (it != kprof_.end()) best[reg] = std::min(best[reg], it->second.ms);
        }
      const bool reg = best[1] <= best[0];
      std::string err;
      if (!fft_plan_record(site, n, reg, best[1], best[0], &err)) throw std::runtime_error(err);
      out << (first ? "" : ", ") << "{\"site\": \"" << fft_site_name(site) << "\", \"n\": " << n
          << ", \"kernel\": \"" << kname << "\", \"register_ms\": " << best[1] << ", \"stockham_ms\": " << best[0]
          << ", \"choice\": \"" << (reg ? "register" : "stockham") << "\"}";
      first = false;
    }
  } catch (...) {
    fft_sites_track(nullptr);
    fft_site_unforce();
    profiling_ = prof_saved;
    set_cur_time(t_saved);
    throw;
  }
  out << "]}";
  reset_profile();
  profiling_ = prof_saved;
  set_cur_time(t_saved);
  return out.str();
}

// ------------------------------------------------------------------ files
// setFile (cudaSirecon.cpp:1337-1352)
void SIM_Reconstructor::set_file(int it, int iw)
{
  std::string err;
  if (opt.p.bTIFF) {
    if (it < 0 || (size_t)it >= tiff_files_.size()) throw std::runtime_error("setFile: time index out of range");
    Stack s;
    if (!tiff_read(tiff_files_[it], &s, &err)) throw std::runtime_error(err);
    if (s.width != nx_raw_ || s.height != ny_ || s.depth != nimg_)
      throw std::runtime_error("setFile: TIFF size differs from the first file");
    stage_raw(s.data.data(), false);
  } else {
    // sections of time point it (single wave): nimg consecutive sections
    std::vector<float> all((size_t)nimg_ * nx_raw_ * ny_), sec;
    for (int s = 0; s < nimg_; ++s) {
      int idx = it * nimg_ * opt.ip.nwaves + iw * nimg_ + s;
      if (!mrc_read_section(mrc_in_, idx, &sec, &err)) throw std::runtime_error(err);
      memcpy(&all[(size_t)s * nx_raw_ * ny_], sec.data(), (size_t)nx_raw_ * ny_ * sizeof(float));
    }
    if (opt.p.bBgInExtHdr) {
      ensure_precondition_buffers();
      // loadImageData (cudaSirecon.cpp:1386-1393): each section's extra
      // background is the third float of its extended-header record
      // (IMRtExHdrZWT: nint ints, then nreal floats per section)
      const MrcHeader& h = mrc_in_.hdr;
      const size_t rec = (size_t)(h.nint + h.nreal) * 4;
      bgx_host_.assign(nimg_, 0.f);
      for (int s = 0; s < nimg_; ++s) {
        const size_t idx = (size_t)it * nimg_ * opt.ip.nwaves + (size_t)iw * nimg_ + s;
        const size_t off = idx * rec + (size_t)h.nint * 4 + 8;
        if (h.nreal >= 3 && off + 4 <= mrc_in_.ext.size()) {
          uint32_t u;
          memcpy(&u, mrc_in_.ext.data() + off, 4);
          if (mrc_in_.swapped) u = __builtin_bswap32(u);
          memcpy(&bgx_host_[s], &u, 4);
        }
      }
      check(cudaMemcpy(d_bgx_, bgx_host_.data(), (size_t)nimg_ * sizeof(float), cudaMemcpyHostToDevice),
            "section backgrounds");
    }
    stage_raw(all.data(), false);
  }
}

// writeResult (cudaSirecon.cpp:1636-1699)
void SIM_Reconstructor::write_result(int it, int iw)
{
  std::vector<float> out(out_elems());
  get_result(out.data());
  std::string err;
  if (opt.p.bTIFF) {
    std::string path = output_path_for(tiff_files_[it], "_proc");
    if (!tiff_write_float(path, out.data(), X_, Y_, Z_, &err)) throw std::runtime_error(err);
  } else {
    if (!mrc_out_) throw std::runtime_error("output file is not open");
    float maxval = -FLT_MAX, minval = FLT_MAX;
    const size_t plane = (size_t)X_ * Y_;
    for (int z = 0; z < Z_; ++z) {
      const float* ptr = out.data() + z * plane;
      mrc_out_.write((const char*)ptr, plane * sizeof(float));
      if (it == 0)
        for (size_t j = 0; j < plane; ++j) {
          // the reference's min/max update (cudaSirecon.cpp:1676-1680)
          if (ptr[j] > maxval) maxval = ptr[j];
          else if (ptr[j] < minval) minval = ptr[j];
        }
    }
    if (it == 0 && iw == 0) {
      out_hdr_.amin = minval;
      out_hdr_.amax = maxval;
    }
  }
}

// closeFiles (cudaSirecon.cpp:1702-1713) -> saveCommandLineToHeader
// (mrc.h:62-74).  The two IM-library calls it makes are restated from the
// Priism IM library's documented behaviour (the library is not part of the
// reference tree):
//  * IMAlLab(stream, titles, strlen(titles)/80 + 1) with bWriteTitle: the
//    header's labels become that many 80-byte records cut from `titles`, the
//    arguments after the three positional ones, each followed by a space, in
//    a 1000-byte buffer.  The bytes the reference copies past the string's
//    terminator are its uninitialised stack; they are written as zeros here.
//  * IMWrHdr(stream, header.label, 1, amin, amax, amean): the title argument
//    is the first label of the header the program keeps (the input file's
//    first label, m_in_out_header); ntflag = 1 appends it to the labels,
//    dropping the oldest when all ten are in use; amin/amax are the values of
//    writeResult's scan of time point 0 and amean the input's.
void SIM_Reconstructor::close_files()
{
  if (opt.p.bTIFF || !mrc_out_.is_open()) return;
  if (opt.p.bWriteTitle) {
    char titles[1000];
    memset(titles, 0, sizeof(titles));
    size_t len = 0;
    for (size_t i = 3; i < argv_.size(); ++i)
      for (const std::string& piece : {argv_[i], std::string(" ")})
        for (char c : piece)
          if (len + 1 < sizeof(titles)) titles[len++] = c;
    int nl = (int)(len / 80) + 1;
    if (nl > 10) nl = 10;
    memset(out_hdr_.label, 0, sizeof(out_hdr_.label));
    for (int l = 0; l < nl; ++l) memcpy(out_hdr_.label[l], titles + 80 * l, 80);
    out_hdr_.nlab = nl;
  }
  char title[80];
  memcpy(title, in_label0_, 80);
  if (out_hdr_.nlab < 0) out_hdr_.nlab = 0;
  if (out_hdr_.nlab >= 10) {
    memmove(out_hdr_.label[0], out_hdr_.label[1], 9 * 80);
    out_hdr_.nlab = 9;
  }
  memcpy(out_hdr_.label[out_hdr_.nlab], title, 80);
  out_hdr_.nlab++;
  mrc_out_.seekp(0);
  mrc_out_.write((const char*)&out_hdr_, sizeof(MrcHeader));
  mrc_out_.close();
}
