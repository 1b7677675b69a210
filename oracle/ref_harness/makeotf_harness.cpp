// Harness that runs the reference's makeotf program (src/otf/radialft.cpp,
// compiled unmodified with its `main` renamed to radialft_reference_main) in
// this process, for the tests and the golden-fixture generator only.
//
// radialft.cpp needs two libraries this machine does not have:
//  * FFTW3f (radialft.cpp:30, 339-348): the four calls it makes are declared
//    by the fftw3.h shim that oracle/build_ref.py writes and are implemented
//    below over a double-precision DFT (the same unnormalised forward
//    transform, e^{-2 pi i k n / N}, with FFTW's in-place r2c layout: rows
//    padded to 2*(nx/2+1) floats, output [nz][ny][nx/2+1] complex);
//  * libtiff (radialft.cpp:124-130, 1100, 1116): the CImg.h shim undefines
//    cimg_use_tiff, declares TIFFOpen/TIFFClose/TIFFSet*Handler (defined
//    below: TIFFOpen returns a non-null token when the file can be opened)
//    and routes CImg's save_tiff to save_cimg.  PSF stacks are therefore
//    handed over, and OTFs come back, in CImg's own ".cimg" raw format,
//    which CImg reads and writes without any library.
// Everything else -- every helper and the whole of main -- is the
// reference's own code.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fftw3.h"
#include "tiffio_stub.h"

int radialft_reference_main(int argc, char** argv);

struct fftwf_plan_s {
  int nz, ny, nx;
};

extern "C" {

void fftwf_plan_with_nthreads(int) {}

fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float*, fftwf_complex*, unsigned)
{
  return new fftwf_plan_s{n0, n1, n2};
}

void fftwf_destroy_plan(fftwf_plan p) { delete p; }

}  // extern "C"

namespace {

// in place DFT of `n` complex doubles at stride `st` (O(n^2), exact twiddle
// indices reduced mod n)
void dft_line(double* re, double* im, int n, size_t st, std::vector<double>& c, std::vector<double>& s,
              std::vector<double>& tr, std::vector<double>& ti)
{
  if ((int)c.size() != n) {
    c.resize(n);
    s.resize(n);
    for (int k = 0; k < n; ++k) {
      c[k] = std::cos(2.0 * M_PI * k / n);
      s[k] = -std::sin(2.0 * M_PI * k / n);
    }
  }
  tr.assign(n, 0.0);
  ti.assign(n, 0.0);
  for (int k = 0; k < n; ++k) {
    double ar = 0.0, ai = 0.0;
    for (int j = 0; j < n; ++j) {
      const int m = (int)(((long long)j * k) % n);
      const double xr = re[j * st], xi = im[j * st];
      ar += xr * c[m] - xi * s[m];
      ai += xr * s[m] + xi * c[m];
    }
    tr[k] = ar;
    ti[k] = ai;
  }
  for (int k = 0; k < n; ++k) {
    re[k * st] = tr[k];
    im[k * st] = ti[k];
  }
}

}  // namespace

extern "C" void fftwf_execute_dft_r2c(fftwf_plan p, float* in, fftwf_complex* out)
{
  const int nz = p->nz, ny = p->ny, nx = p->nx, nxh = nx / 2 + 1, pitch = 2 * nxh;
  const size_t vol = (size_t)nz * ny * nx;
  std::vector<double> re(vol), im(vol, 0.0);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) re[((size_t)z * ny + y) * nx + x] = in[((size_t)z * ny + y) * pitch + x];
  std::vector<double> c, s, tr, ti;
  for (size_t l = 0; l < (size_t)nz * ny; ++l) dft_line(&re[l * nx], &im[l * nx], nx, 1, c, s, tr, ti);
  c.clear();
  for (int z = 0; z < nz; ++z)
    for (int x = 0; x < nx; ++x) {
      size_t o = (size_t)z * ny * nx + x;
      dft_line(&re[o], &im[o], ny, nx, c, s, tr, ti);
    }
  c.clear();
  for (size_t o = 0; o < (size_t)ny * nx; ++o) dft_line(&re[o], &im[o], nz, (size_t)ny * nx, c, s, tr, ti);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nxh; ++x) {
        size_t i = ((size_t)z * ny + y) * nx + x;
        size_t o = ((size_t)z * ny + y) * nxh + x;
        out[o][0] = (float)re[i];
        out[o][1] = (float)im[i];
      }
}

// libtiff entry points radialft.cpp's main calls directly
extern "C" {
TIFFErrorHandler TIFFSetWarningHandler(TIFFErrorHandler) { return nullptr; }
TIFFErrorHandler TIFFSetErrorHandler(TIFFErrorHandler) { return nullptr; }
TIFF* TIFFOpen(const char* name, const char*)
{
  FILE* f = std::fopen(name, "rb");
  if (!f) return nullptr;
  std::fclose(f);
  static int token;
  return (TIFF*)&token;
}
void TIFFClose(TIFF*) {}

// Runs the reference program with the given command line; returns its exit
// status, or -2 when it threw.
int mo_ref_main(int argc, char** argv)
{
  try {
    return radialft_reference_main(argc, argv);
  } catch (...) {
    return -2;
  }
}
}
