// File-level makeotf driver: the flow of radialft.cpp main (82-434) around
// the GPU computation -- read the PSF (TIFF, else MRC/DV), run, write the
// OTF in the file format of the input:
//  * TIFF: float pages [depth][height][width] exactly as outputdata
//    (radialft.cpp:1073-1100) writes them, plus the "_OnlyForViewing" TIFF of
//    sqrt(|OTF|) (1102-1119);
//  * MRC: complex sections with nx = nz, ny = nx/2+1, nz = bands,
//    xlen = dkz, ylen = dkr (radialft.cpp:1124-1150).
// For MRC input dr, dz and the wavelength come from the header (172-177) and
// no background is subtracted: the reference fills its background array only
// for TIFF input or from the extended header (232-246), which is not
// supported here.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "image_io.h"
#include "makeotf.h"

namespace simrecon {

int makeotf_main(int argc, const char* const* argv, std::string* err)
{
  MakeOtfOptions o;
  std::string in, out;
  if (!makeotf_parse(argc, argv, &o, &in, &out, err)) return -1;
  Stack st;
  bool tiff = false;
  MrcFile mf;
  std::vector<float> data;
  int nx = 0, ny = 0, nsec = 0;
  std::string e1;
  int w, h, d;
  if (tiff_info(in, &w, &h, &d, &e1)) {
    if (!tiff_read(in, &st, err)) return -1;
    tiff = true;
    nx = st.width, ny = st.height, nsec = st.depth;
  } else {
    if (!mrc_open(in, &mf, err)) {
      *err = "cannot read PSF " + in + " as TIFF (" + e1 + ") or MRC (" + *err + ")";
      return -1;
    }
    if (!mrc_read_all(mf, &data, err)) return -1;
    nx = mf.hdr.nx, ny = mf.hdr.ny, nsec = mf.hdr.nz;
    o.dr = mf.hdr.ylen;
    o.dz = mf.hdr.zlen;
    o.wavelength = (unsigned)mf.hdr.iwav1;
    o.background = 0.f;
  }
  const float* psf = tiff ? st.data.data() : data.data();
  std::printf("nx=%d, ny=%d, nz=%d, dr=%f, dz=%f, wavelength=%u\n", nx, ny, nsec / o.nphases, o.dr, o.dz,
              o.wavelength);
  OtfResult r;
  if (!makeotf_run(psf, nx, ny, nsec, o, &r, err)) return -1;
  std::printf("Center of mass is (%.3f, %.3f, %.3f)\n", r.xc, r.yc, r.zc);
  if (tiff) {
    if (!tiff_write_float(out, r.data.data(), r.width, r.height, r.depth, err)) return -1;
    size_t pos = out.rfind(".tif");
    if (pos == std::string::npos) pos = out.rfind(".TIF");
    if (pos == std::string::npos) {
      *err = "output OTF name must contain .tif (the viewing copy is named from it)";
      return -1;
    }
    std::vector<float> amps((size_t)(r.width / 2) * r.height * r.depth);
    for (size_t i = 0; i < amps.size(); ++i)
      amps[i] = std::sqrt(std::hypot(r.data[2 * i], r.data[2 * i + 1]));
    std::string vname = out;
    vname.insert(pos, "_OnlyForViewing");
    if (!tiff_write_float(vname, amps.data(), r.width / 2, r.height, r.depth, err)) return -1;
  } else {
    MrcHeader hdr = mf.hdr;
    hdr.xlen = r.dkz;
    hdr.ylen = r.dkr;
    hdr.zlen = 0;
    hdr.amin = 0;
    hdr.amax = 1;
    // header nx = nz, ny = nx/2+1 (for nz == 1 that is 1 x (nx/2+1))
    const int mnx = r.height == 1 ? 1 : r.width / 2, mny = r.height == 1 ? r.width / 2 : r.height;
    hdr.mx = mnx, hdr.my = mny, hdr.mz = r.depth;
    if (!mrc_write(out, hdr, std::vector<char>(), r.data.data(), mnx, mny, r.depth, 4, err)) return -1;
  }
  return 0;
}

}  // namespace simrecon
