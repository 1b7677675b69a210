// Baseline TIFF and MRC/DV readers and writers (see image_io.h).
#include "image_io.h"

#include <cstdio>
#include <cstring>
#include <fstream>

namespace simrecon {

namespace {

template <typename T>
T bswap(T v)
{
  T r;
  const unsigned char* s = (const unsigned char*)&v;
  unsigned char* d = (unsigned char*)&r;
  for (size_t i = 0; i < sizeof(T); ++i) d[i] = s[sizeof(T) - 1 - i];
  return r;
}

bool read_file(const std::string& path, std::vector<unsigned char>* buf, std::string* err)
{
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    if (err) *err = "cannot open " + path;
    return false;
  }
  f.seekg(0, std::ios::end);
  size_t n = (size_t)f.tellg();
  f.seekg(0);
  buf->resize(n);
  if (n) f.read((char*)buf->data(), n);
  if (!f) {
    if (err) *err = "cannot read " + path;
    return false;
  }
  return true;
}

struct TiffReader {
  const std::vector<unsigned char>& b;
  bool be;
  explicit TiffReader(const std::vector<unsigned char>& buf) : b(buf), be(false) {}
  bool ok(size_t off, size_t n) const { return off + n <= b.size(); }
  uint16_t u16(size_t off) const
  {
    uint16_t v;
    memcpy(&v, &b[off], 2);
    return be ? bswap(v) : v;
  }
  uint32_t u32(size_t off) const
  {
    uint32_t v;
    memcpy(&v, &b[off], 4);
    return be ? bswap(v) : v;
  }
};

struct Ifd {
  uint32_t width = 0, height = 0, bps = 8, fmt = 1, spp = 1, compression = 1, rows_per_strip = 0xffffffffu;
  std::vector<uint32_t> offsets, counts;
  uint32_t next = 0;
};

bool parse_ifd(const TiffReader& r, uint32_t off, Ifd* ifd, std::string* err)
{
  if (!r.ok(off, 2)) {
    if (err) *err = "truncated TIFF directory";
    return false;
  }
  uint16_t n = r.u16(off);
  if (!r.ok(off + 2, 12u * n + 4)) {
    if (err) *err = "truncated TIFF directory";
    return false;
  }
  for (uint16_t i = 0; i < n; ++i) {
    size_t e = off + 2 + 12u * i;
    uint16_t tag = r.u16(e), type = r.u16(e + 2);
    uint32_t count = r.u32(e + 4);
    size_t tsz = (type == 3) ? 2 : (type == 4 ? 4 : (type == 1 ? 1 : 4));
    size_t voff = (tsz * count <= 4) ? e + 8 : r.u32(e + 8);
    auto val = [&](uint32_t k) -> uint32_t {
      size_t p = voff + k * tsz;
      if (!r.ok(p, tsz)) return 0;
      return type == 3 ? r.u16(p) : (type == 1 ? r.b[p] : r.u32(p));
    };
    switch (tag) {
      case 256: ifd->width = val(0); break;
      case 257: ifd->height = val(0); break;
      case 258: ifd->bps = val(0); break;
      case 259: ifd->compression = val(0); break;
      case 273:
        ifd->offsets.resize(count);
        for (uint32_t k = 0; k < count; ++k) ifd->offsets[k] = val(k);
        break;
      case 277: ifd->spp = val(0); break;
      case 278: ifd->rows_per_strip = val(0); break;
      case 279:
        ifd->counts.resize(count);
        for (uint32_t k = 0; k < count; ++k) ifd->counts[k] = val(k);
        break;
      case 339: ifd->fmt = val(0); break;
      default: break;
    }
  }
  ifd->next = r.u32(off + 2 + 12u * n);
  return true;
}

bool tiff_dirs(const std::vector<unsigned char>& buf, std::vector<Ifd>* dirs, bool* be, std::string* err)
{
  if (buf.size() < 8) {
    if (err) *err = "not a TIFF file";
    return false;
  }
  TiffReader r(buf);
  if (buf[0] == 'I' && buf[1] == 'I') r.be = false;
  else if (buf[0] == 'M' && buf[1] == 'M') r.be = true;
  else {
    if (err) *err = "not a TIFF file";
    return false;
  }
  if (r.u16(2) != 42) {
    if (err) *err = "unsupported TIFF variant";
    return false;
  }
  uint32_t off = r.u32(4);
  int guard = 0;
  while (off != 0 && guard++ < 1000000) {
    Ifd d;
    if (!parse_ifd(r, off, &d, err)) return false;
    dirs->push_back(d);
    off = d.next;
  }
  *be = r.be;
  return true;
}

}  // namespace

bool tiff_info(const std::string& path, int* width, int* height, int* depth, std::string* err)
{
  std::vector<unsigned char> buf;
  if (!read_file(path, &buf, err)) return false;
  std::vector<Ifd> dirs;
  bool be;
  if (!tiff_dirs(buf, &dirs, &be, err)) return false;
  if (dirs.empty()) {
    if (err) *err = "TIFF without images";
    return false;
  }
  *width = dirs[0].width;
  *height = dirs[0].height;
  *depth = (int)dirs.size();
  return true;
}

bool tiff_read(const std::string& path, Stack* out, std::string* err)
{
  std::vector<unsigned char> buf;
  if (!read_file(path, &buf, err)) return false;
  std::vector<Ifd> dirs;
  bool be;
  if (!tiff_dirs(buf, &dirs, &be, err)) return false;
  if (dirs.empty()) {
    if (err) *err = "TIFF without images";
    return false;
  }
  TiffReader r(buf);
  r.be = be;
  out->width = dirs[0].width;
  out->height = dirs[0].height;
  out->depth = (int)dirs.size();
  const size_t plane = (size_t)out->width * out->height;
  out->data.assign(plane * out->depth, 0.f);
  for (size_t p = 0; p < dirs.size(); ++p) {
    const Ifd& d = dirs[p];
    if (d.width != (uint32_t)out->width || d.height != (uint32_t)out->height) {
      if (err) *err = "TIFF pages of different sizes";
      return false;
    }
    if (d.compression != 1 || d.spp != 1) {
      if (err) *err = "only uncompressed single-channel TIFF is supported";
      return false;
    }
    const int bytes = d.bps / 8;
    if (!(bytes == 1 || bytes == 2 || bytes == 4) || (d.fmt == 3 && bytes != 4)) {
      if (err) *err = "unsupported TIFF sample type";
      return false;
    }
    float* dst = out->data.data() + plane * p;
    size_t written = 0;
    for (size_t s = 0; s < d.offsets.size() && written < plane; ++s) {
      size_t off = d.offsets[s];
      size_t cnt = s < d.counts.size() ? d.counts[s] : (plane - written) * bytes;
      size_t n = std::min(cnt / bytes, plane - written);
      if (!r.ok(off, n * bytes)) {
        if (err) *err = "truncated TIFF strip";
        return false;
      }
      for (size_t i = 0; i < n; ++i) {
        size_t q = off + i * bytes;
        float v;
        if (bytes == 1) v = (d.fmt == 2) ? (float)(int8_t)buf[q] : (float)buf[q];
        else if (bytes == 2) {
          uint16_t u = r.u16(q);
          v = (d.fmt == 2) ? (float)(int16_t)u : (float)u;
        } else {
          uint32_t u = r.u32(q);
          if (d.fmt == 3) memcpy(&v, &u, 4);
          else if (d.fmt == 2) v = (float)(int32_t)u;
          else v = (float)u;
        }
        dst[written + i] = v;
      }
      written += n;
    }
    if (written < plane) {
      if (err) *err = "TIFF page shorter than its size";
      return false;
    }
  }
  return true;
}

bool tiff_write_float(const std::string& path, const float* data, int width, int height, int depth,
                      std::string* err)
{
  std::ofstream f(path, std::ios::binary);
  if (!f) {
    if (err) *err = "cannot create " + path;
    return false;
  }
  auto w16 = [&](uint16_t v) { f.write((const char*)&v, 2); };
  auto w32 = [&](uint32_t v) { f.write((const char*)&v, 4); };
  const uint32_t plane_bytes = (uint32_t)width * height * 4;
  const int ntags = 10;
  const uint32_t ifd_bytes = 2 + 12 * ntags + 4;
  f.write("II", 2);
  w16(42);
  w32(8);
  uint32_t pos = 8;
  for (int p = 0; p < depth; ++p) {
    uint32_t data_off = pos + ifd_bytes;
    uint32_t next = (p + 1 < depth) ? data_off + plane_bytes : 0;
    w16(ntags);
    auto tag = [&](uint16_t t, uint16_t type, uint32_t cnt, uint32_t v) {
      w16(t);
      w16(type);
      w32(cnt);
      if (type == 3) {
        w16((uint16_t)v);
        w16(0);
      } else {
        w32(v);
      }
    };
    tag(256, 4, 1, width);
    tag(257, 4, 1, height);
    tag(258, 3, 1, 32);
    tag(259, 3, 1, 1);
    tag(262, 3, 1, 1);
    tag(273, 4, 1, data_off);
    tag(277, 3, 1, 1);
    tag(278, 4, 1, height);
    tag(279, 4, 1, plane_bytes);
    tag(339, 3, 1, 3);
    w32(next);
    f.write((const char*)(data + (size_t)p * width * height), plane_bytes);
    pos = data_off + plane_bytes;
  }
  if (!f) {
    if (err) *err = "write failed: " + path;
    return false;
  }
  return true;
}

// ------------------------------------------------------------------- MRC
namespace {
void swap_header(MrcHeader* h)
{
  int32_t* i = (int32_t*)h;
  for (int k = 0; k < 24; ++k) i[k] = bswap(i[k]);  // nx .. next (24 words)
  h->dvid = bswap(h->dvid);
  h->nblank = bswap(h->nblank);
  h->ntst = bswap(h->ntst);
  int16_t* s = &h->nint;
  for (int k = 0; k < 4; ++k) s[k] = bswap(s[k]);
  float* f = &h->min2;
  for (int k = 0; k < 6; ++k) f[k] = bswap(f[k]);
  s = &h->type;
  for (int k = 0; k < 6; ++k) s[k] = bswap(s[k]);
  h->min5 = bswap(h->min5);
  h->max5 = bswap(h->max5);
  h->num_times = bswap(h->num_times);
  h->interleaved = bswap(h->interleaved);
  h->tilt_x = bswap(h->tilt_x);
  h->tilt_y = bswap(h->tilt_y);
  h->tilt_z = bswap(h->tilt_z);
  s = &h->num_waves;
  for (int k = 0; k < 6; ++k) s[k] = bswap(s[k]);
  h->zorig = bswap(h->zorig);
  h->xorig = bswap(h->xorig);
  h->yorig = bswap(h->yorig);
  h->nlab = bswap(h->nlab);
}

int mode_bytes(int mode)
{
  switch (mode) {
    case 0: return 1;
    case 1: return 2;
    case 2: return 4;
    case 3: return 4;   // complex int16
    case 4: return 8;   // complex float
    case 6: return 2;   // uint16
    default: return 0;
  }
}
}  // namespace

bool mrc_open(const std::string& path, MrcFile* f, std::string* err)
{
  std::ifstream in(path, std::ios::binary);
  if (!in) {
    if (err) *err = "cannot open " + path;
    return false;
  }
  in.read((char*)&f->hdr, sizeof(MrcHeader));
  if (!in) {
    if (err) *err = "truncated MRC header: " + path;
    return false;
  }
  f->path = path;
  f->swapped = false;
  // the DV magic 0xc0a0 (or a plausible mode) tells the byte order
  if ((uint16_t)f->hdr.dvid != 0xc0a0 && (f->hdr.mode < 0 || f->hdr.mode > 16)) {
    swap_header(&f->hdr);
    f->swapped = true;
  }
  if (mode_bytes(f->hdr.mode) == 0 || f->hdr.nx <= 0 || f->hdr.ny <= 0 || f->hdr.nz <= 0) {
    if (err) *err = "unsupported or corrupt MRC header: " + path;
    return false;
  }
  f->ext.assign(f->hdr.next > 0 ? f->hdr.next : 0, 0);
  if (!f->ext.empty()) in.read(f->ext.data(), f->ext.size());
  return (bool)in;
}

bool mrc_read_section(const MrcFile& f, int sec, std::vector<float>* out, std::string* err)
{
  const MrcHeader& h = f.hdr;
  const int mb = mode_bytes(h.mode);
  const bool cplx = (h.mode == 3 || h.mode == 4);
  const size_t n = (size_t)h.nx * h.ny;
  std::ifstream in(f.path, std::ios::binary);
  in.seekg(1024 + (std::streamoff)f.ext.size() + (std::streamoff)sec * n * mb);
  std::vector<char> raw(n * mb);
  in.read(raw.data(), raw.size());
  if (!in) {
    if (err) *err = "truncated MRC data: " + f.path;
    return false;
  }
  out->resize(n * (cplx ? 2 : 1));
  for (size_t i = 0; i < n; ++i) {
    const char* p = raw.data() + i * mb;
    switch (h.mode) {
      case 0: (*out)[i] = (float)(uint8_t)p[0]; break;
      case 1: {
        int16_t v;
        memcpy(&v, p, 2);
        (*out)[i] = (float)(f.swapped ? bswap(v) : v);
        break;
      }
      case 6: {
        uint16_t v;
        memcpy(&v, p, 2);
        (*out)[i] = (float)(f.swapped ? bswap(v) : v);
        break;
      }
      case 2: {
        float v;
        memcpy(&v, p, 4);
        (*out)[i] = f.swapped ? bswap(v) : v;
        break;
      }
      case 3: {
        int16_t a, b;
        memcpy(&a, p, 2);
        memcpy(&b, p + 2, 2);
        (*out)[2 * i] = (float)(f.swapped ? bswap(a) : a);
        (*out)[2 * i + 1] = (float)(f.swapped ? bswap(b) : b);
        break;
      }
      case 4: {
        float a, b;
        memcpy(&a, p, 4);
        memcpy(&b, p + 4, 4);
        (*out)[2 * i] = f.swapped ? bswap(a) : a;
        (*out)[2 * i + 1] = f.swapped ? bswap(b) : b;
        break;
      }
    }
  }
  return true;
}

bool mrc_read_all(const MrcFile& f, std::vector<float>* out, std::string* err)
{
  out->clear();
  std::vector<float> sec;
  for (int z = 0; z < f.hdr.nz; ++z) {
    if (!mrc_read_section(f, z, &sec, err)) return false;
    out->insert(out->end(), sec.begin(), sec.end());
  }
  return true;
}

bool mrc_write(const std::string& path, const MrcHeader& hdr_in, const std::vector<char>& ext, const float* data,
               int nx, int ny, int nz, int mode, std::string* err)
{
  MrcHeader h = hdr_in;
  h.nx = nx;
  h.ny = ny;
  h.nz = nz;
  h.mode = mode;
  h.next = (int32_t)ext.size();
  h.dvid = (int16_t)0xc0a0;
  std::ofstream o(path, std::ios::binary);
  if (!o) {
    if (err) *err = "cannot create " + path;
    return false;
  }
  o.write((const char*)&h, sizeof(h));
  if (!ext.empty()) o.write(ext.data(), ext.size());
  size_t n = (size_t)nx * ny * nz * (mode == 4 ? 2 : 1);
  o.write((const char*)data, n * sizeof(float));
  if (!o) {
    if (err) *err = "write failed: " + path;
    return false;
  }
  return true;
}

}  // namespace simrecon
