// Minimal image file I/O for the reconstruction boundary: baseline
// uncompressed multi-page TIFF (8/16/32-bit integer and 32-bit float
// samples, strips, either byte order) and MRC/DV (Priism) stacks.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace simrecon {

struct Stack {
  int width = 0, height = 0, depth = 0;  // depth = number of pages / sections
  std::vector<float> data;               // [depth][height][width]
};

// TIFF
bool tiff_read(const std::string& path, Stack* out, std::string* err);
bool tiff_info(const std::string& path, int* width, int* height, int* depth, std::string* err);
bool tiff_write_float(const std::string& path, const float* data, int width, int height, int depth,
                      std::string* err);

// MRC / DV header (1024 bytes, Priism layout)
struct MrcHeader {
  int32_t nx, ny, nz, mode;
  int32_t nxst, nyst, nzst;
  int32_t mx, my, mz;
  float xlen, ylen, zlen;
  float alpha, beta, gamma;
  int32_t mapc, mapr, maps;
  float amin, amax, amean;
  int32_t ispg, next;
  int16_t dvid, nblank;
  int32_t ntst;
  char extra[24];
  int16_t nint, nreal, nres, nzfact;
  float min2, max2, min3, max3, min4, max4;
  int16_t type, lensnum, n1, n2, v1, v2;
  float min5, max5;
  int16_t num_times, interleaved;
  float tilt_x, tilt_y, tilt_z;
  int16_t num_waves, iwav1, iwav2, iwav3, iwav4, iwav5;
  float zorig, xorig, yorig;
  int32_t nlab;
  char label[10][80];
};
static_assert(sizeof(MrcHeader) == 1024, "MRC header must be 1024 bytes");

struct MrcFile {
  std::string path;
  MrcHeader hdr;
  bool swapped = false;
  std::vector<char> ext;  // extended header bytes
};

bool mrc_open(const std::string& path, MrcFile* f, std::string* err);
// read section `sec` (0-based) as float; complex modes give interleaved pairs
bool mrc_read_section(const MrcFile& f, int sec, std::vector<float>* out, std::string* err);
bool mrc_read_all(const MrcFile& f, std::vector<float>* out, std::string* err);
// write a float32 stack with the given header (mode and sizes are set here)
bool mrc_write(const std::string& path, const MrcHeader& hdr, const std::vector<char>& ext, const float* data,
               int nx, int ny, int nz, int mode, std::string* err);

}  // namespace simrecon
