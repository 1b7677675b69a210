// makeotf on the GPU: bead PSF stack -> rotationally averaged SIM OTF, the
// computation of the reference's program src/otf/radialft.cpp (main 82-434
// and its helpers), with the same switches and output layout.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace simrecon {

// Switches of radialft.cpp:commandline (1381-1553); defaults from main
// (82-108).  The two-objective and I2M modes are not supported.
struct MakeOtfOptions {
  int nphases = 5;
  float angle = 1.57f;      // -angle
  float ls = 0.2f;          // -ls
  float dr = 0.106f;        // -xyres (TIFF input; MRC takes the header's ylen)
  float dz = 0.1f;          // -zres  (TIFF input; MRC takes the header's zlen)
  float beaddiam = 0.12f;   // -beaddiam
  float na = 1.4f;          // -na
  float nimm = 1.515f;      // -nimm
  unsigned wavelength = 525;  // -wavelength (nm)
  float background = -1.f;  // -background (< 0: estimate from a 20-pixel border)
  int fixorigin[2] = {0, 0};  // -fixorigin kr1 kr2 (kr1 > 0 enables)
  int leavekz[3] = {0, 0, 0};  // -leavekz (first > 0 enables cleanup)
  int ifixz = 1;            // -ifixkz
  int ifixr = 0;            // -ifixkr
  bool rescale = false;     // -rescale
  bool five_bands = false;  // -5bands
  bool conj = false;        // -conj
  bool compensate = true;   // -nocompen clears it
  bool pishift = false;     // -PIshift
  bool bessel = false;      // -bessel
  bool user_dr = false, user_dz = false;  // -xyres / -zres given
};

// Parses the reference command line (program name first; the first two
// non-switch arguments are the PSF and OTF files, like the reference).
// Returns false with a message for an invalid or unsupported switch.
bool makeotf_parse(int argc, const char* const* argv, MakeOtfOptions* o, std::string* in, std::string* out,
                   std::string* err);
// Same for switches only (no program name, no file names).
bool makeotf_parse_switches(int n, const char* const* args, MakeOtfOptions* o, std::string* err);

struct OtfResult {
  // the OTF file's float array [depth][height][width]: width = 2*nz (complex
  // kz along a row), height = nx/2+1, depth = norders (2*norders-1 with
  // -5bands); for nz == 1: width 2*(nx/2+1), height 1
  std::vector<float> data;
  int width = 0, height = 0, depth = 0;
  float xc = 0, yc = 0, zc = 0;  // bead centre found (pixels)
  float dkr = 0, dkz = 0;        // OTF sampling (1/um)
  double device_ms = 0;          // device time of the computation
};

// psf: float [nsections][ny][nx], section = z * nphases + phase.
bool makeotf_run(const float* psf, int nx, int ny, int nsections, const MakeOtfOptions& o, OtfResult* r,
                 std::string* err, cudaStream_t s = 0);

}  // namespace simrecon
