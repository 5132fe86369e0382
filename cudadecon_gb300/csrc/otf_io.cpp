// OTF file loading without libtiff or CImg.
//
// The reference reads the OTF with CImg (complexOTF.assign(OTF_file_name),
// src/RL-Biggs-Andrews.cpp:568), which dispatches on the file extension.
// radialft writes the radially averaged OTF as a single-page float32 TIFF of
// width 2*nz_otf and height nr, complex interleaved with kz fastest
// (src/radialft_interface.cpp:160-193).  This reader accepts
//   * baseline uncompressed TIFF (little or big endian, strips, one or more
//     pages = depth; 8/16/32-bit integer or 32/64-bit float samples), and
//   * CImg's own .cimg format (uncompressed; first image of the list),
// and returns the image in CImg order (x fastest, then y, then z).
#include "otf_io.h"

#include <stdio.h>
#include <string.h>
#include <strings.h>

#include <string>
#include <vector>

namespace cdx {

namespace {

struct Reader {
  std::vector<unsigned char> buf;
  bool big = false;
  bool ok(size_t off, size_t n) const { return off + n <= buf.size() && off + n >= off; }
  unsigned u16(size_t o) const {
    return big ? (unsigned)(buf[o] << 8 | buf[o + 1]) : (unsigned)(buf[o] | buf[o + 1] << 8);
  }
  unsigned u32(size_t o) const {
    return big ? ((unsigned)buf[o] << 24 | (unsigned)buf[o + 1] << 16 | (unsigned)buf[o + 2] << 8 |
                  (unsigned)buf[o + 3])
               : ((unsigned)buf[o] | (unsigned)buf[o + 1] << 8 | (unsigned)buf[o + 2] << 16 |
                  (unsigned)buf[o + 3] << 24);
  }
};

bool read_file(const char* path, std::vector<unsigned char>& out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  if (fseek(f, 0, SEEK_END) != 0) {
    fclose(f);
    return false;
  }
  long n = ftell(f);
  if (n < 0) {
    fclose(f);
    return false;
  }
  fseek(f, 0, SEEK_SET);
  out.resize((size_t)n);
  size_t got = n ? fread(out.data(), 1, (size_t)n, f) : 0;
  fclose(f);
  return got == (size_t)n;
}

// Decode one sample of the given type/bits at p (endian-aware).
float sample_value(const Reader& r, size_t p, int fmt, int bits) {
  if (fmt == 3) {
    if (bits == 32) {
      unsigned u = r.u32(p);
      float v;
      memcpy(&v, &u, 4);
      return v;
    }
    unsigned long long lo = r.u32(p), hi = r.u32(p + 4);
    unsigned long long u = r.big ? (lo << 32 | hi) : (hi << 32 | lo);
    double v;
    memcpy(&v, &u, 8);
    return (float)v;
  }
  if (bits == 8) return fmt == 2 ? (float)(signed char)r.buf[p] : (float)r.buf[p];
  if (bits == 16) {
    unsigned v = r.u16(p);
    return fmt == 2 ? (float)(short)(unsigned short)v : (float)v;
  }
  unsigned v = r.u32(p);
  return fmt == 2 ? (float)(int)v : (float)v;
}

bool load_tiff(const char* path, HostImage& img, std::string& err) {
  Reader r;
  if (!read_file(path, r.buf)) {
    err = "cannot read file";
    return false;
  }
  if (r.buf.size() < 8) {
    err = "file too short for TIFF";
    return false;
  }
  if (r.buf[0] == 'I' && r.buf[1] == 'I') r.big = false;
  else if (r.buf[0] == 'M' && r.buf[1] == 'M') r.big = true;
  else {
    err = "not a TIFF file";
    return false;
  }
  if (r.u16(2) != 42) {
    err = "unsupported TIFF variant (BigTIFF?)";
    return false;
  }
  size_t ifd = r.u32(4);
  std::vector<float> data;
  int W = -1, H = -1, D = 0;
  while (ifd) {
    if (!r.ok(ifd, 2)) {
      err = "bad IFD offset";
      return false;
    }
    const unsigned n = r.u16(ifd);
    if (!r.ok(ifd + 2, (size_t)n * 12 + 4)) {
      err = "truncated IFD";
      return false;
    }
    int w = 0, h = 0, bits = 8, comp = 1, spp = 1, fmt = 1, planar = 1;
    long rps = -1;
    std::vector<size_t> offs, cnts;
    for (unsigned e = 0; e < n; ++e) {
      const size_t t = ifd + 2 + (size_t)e * 12;
      const unsigned tag = r.u16(t), type = r.u16(t + 2), count = r.u32(t + 4);
      const unsigned tsize = (type == 3) ? 2 : (type == 4 ? 4 : (type == 1 ? 1 : 4));
      const size_t vpos = ((size_t)count * tsize <= 4) ? t + 8 : r.u32(t + 8);
      auto val = [&](unsigned i) -> unsigned long {
        if (type == 3) return r.u16(vpos + 2 * i);
        if (type == 1) return r.buf[vpos + i];
        return r.u32(vpos + 4 * i);
      };
      if (!r.ok(vpos, (size_t)count * tsize)) {
        err = "TIFF tag data out of range";
        return false;
      }
      switch (tag) {
        case 256: w = (int)val(0); break;
        case 257: h = (int)val(0); break;
        case 258: bits = (int)val(0); break;
        case 259: comp = (int)val(0); break;
        case 273: offs.resize(count); for (unsigned i = 0; i < count; ++i) offs[i] = val(i); break;
        case 277: spp = (int)val(0); break;
        case 278: rps = (long)val(0); break;
        case 279: cnts.resize(count); for (unsigned i = 0; i < count; ++i) cnts[i] = val(i); break;
        case 284: planar = (int)val(0); break;
        case 339: fmt = (int)val(0); break;
        case 322: case 323: case 324: case 325:
          err = "tiled TIFF is not supported";
          return false;
        default: break;
      }
    }
    (void)planar;
    (void)rps;
    if (comp != 1) {
      err = "compressed TIFF is not supported";
      return false;
    }
    if (spp != 1) {
      err = "TIFF with more than one sample per pixel is not supported";
      return false;
    }
    if (!(bits == 8 || bits == 16 || bits == 32 || (bits == 64 && fmt == 3))) {
      err = "unsupported TIFF sample size";
      return false;
    }
    if (w <= 0 || h <= 0 || offs.empty()) {
      err = "TIFF page without size or strips";
      return false;
    }
    if (W < 0) {
      W = w;
      H = h;
    } else if (w != W || h != H) {
      err = "TIFF pages of different sizes";
      return false;
    }
    const size_t bps = (size_t)bits / 8;
    const size_t page = (size_t)w * h;
    const size_t base = data.size();
    data.resize(base + page);
    size_t done = 0;
    for (size_t s = 0; s < offs.size() && done < page; ++s) {
      size_t nbytes = s < cnts.size() ? cnts[s] : (page - done) * bps;
      size_t nsamp = nbytes / bps;
      if (nsamp > page - done) nsamp = page - done;
      if (!r.ok(offs[s], nsamp * bps)) {
        err = "TIFF strip out of range";
        return false;
      }
      for (size_t i = 0; i < nsamp; ++i)
        data[base + done + i] = sample_value(r, offs[s] + i * bps, fmt, bits);
      done += nsamp;
    }
    if (done != page) {
      err = "TIFF strips hold fewer samples than the page";
      return false;
    }
    ++D;
    const size_t next = ifd + 2 + (size_t)n * 12;
    ifd = r.u32(next);
    if (D > 1 << 20) {
      err = "too many TIFF pages";
      return false;
    }
  }
  if (D == 0) {
    err = "TIFF without pages";
    return false;
  }
  img.w = W;
  img.h = H;
  img.d = D;
  img.data.swap(data);
  return true;
}

bool load_cimg(const char* path, HostImage& img, std::string& err) {
  Reader r;
  if (!read_file(path, r.buf)) {
    err = "cannot read file";
    return false;
  }
  size_t pos = 0;
  auto line = [&](std::string& s) -> bool {
    s.clear();
    while (pos < r.buf.size() && r.buf[pos] != '\n') s.push_back((char)r.buf[pos++]);
    if (pos >= r.buf.size()) return false;
    ++pos;
    return true;
  };
  std::string s;
  do {
    if (!line(s)) {
      err = "CImg header not found";
      return false;
    }
  } while (!s.empty() && s[0] == '#');
  unsigned N = 0;
  char type[256] = {0}, endian[256] = {0};
  if (sscanf(s.c_str(), "%u %255s %255s", &N, type, endian) < 2 || N == 0) {
    err = "CImg header not found";
    return false;
  }
  r.big = strncasecmp(endian, "big", 3) == 0;
  int bits = 32, fmt = 3;
  if (!strcasecmp(type, "float")) { bits = 32; fmt = 3; }
  else if (!strcasecmp(type, "double")) { bits = 64; fmt = 3; }
  else if (!strcasecmp(type, "unsigned_short") || !strcasecmp(type, "ushort")) { bits = 16; fmt = 1; }
  else if (!strcasecmp(type, "short")) { bits = 16; fmt = 2; }
  else if (!strcasecmp(type, "unsigned_char") || !strcasecmp(type, "uchar")) { bits = 8; fmt = 1; }
  else if (!strcasecmp(type, "char")) { bits = 8; fmt = 2; }
  else if (!strcasecmp(type, "unsigned_int") || !strcasecmp(type, "uint")) { bits = 32; fmt = 1; }
  else if (!strcasecmp(type, "int")) { bits = 32; fmt = 2; }
  else {
    err = std::string("unsupported CImg pixel type ") + type;
    return false;
  }
  if (!line(s)) {
    err = "CImg image size line missing";
    return false;
  }
  unsigned W = 0, H = 0, D = 0, C = 0;
  unsigned long csiz = 0;
  int got = sscanf(s.c_str(), "%u %u %u %u #%lu", &W, &H, &D, &C, &csiz);
  if (got < 4) {
    err = "invalid CImg image size";
    return false;
  }
  if (got == 5) {
    err = "compressed .cimg is not supported";
    return false;
  }
  const size_t n = (size_t)W * H * D * C;
  const size_t bps = (size_t)bits / 8;
  if (n == 0 || !r.ok(pos, n * bps)) {
    err = "CImg data truncated";
    return false;
  }
  img.w = (int)W;
  img.h = (int)H;
  img.d = (int)(D * C);
  img.data.resize(n);
  for (size_t i = 0; i < n; ++i) img.data[i] = sample_value(r, pos + i * bps, fmt, bits);
  return true;
}

bool ends_with(const std::string& s, const char* suf) {
  const size_t n = strlen(suf);
  return s.size() >= n && strcasecmp(s.c_str() + s.size() - n, suf) == 0;
}

}  // namespace

bool load_image_file(const char* path, HostImage& img, std::string& err) {
  if (!path) {
    err = "null file name";
    return false;
  }
  std::string p(path);
  if (ends_with(p, ".cimg")) return load_cimg(path, img, err);
  if (ends_with(p, ".tif") || ends_with(p, ".tiff")) return load_tiff(path, img, err);
  // no recognised extension: sniff the magic bytes
  std::vector<unsigned char> head;
  FILE* f = fopen(path, "rb");
  if (!f) {
    err = "cannot open file";
    return false;
  }
  unsigned char m[4] = {0, 0, 0, 0};
  size_t got = fread(m, 1, 4, f);
  fclose(f);
  if (got >= 2 && ((m[0] == 'I' && m[1] == 'I') || (m[0] == 'M' && m[1] == 'M')))
    return load_tiff(path, img, err);
  return load_cimg(path, img, err);
}


// Write img as a little-endian, uncompressed float32 TIFF: one page per z
// slice, each page one strip of width x height samples (the layout radialft
// writes through libtiff, src/radialft_interface.cpp:194).
bool save_float_tiff(const char* path, const HostImage& img, std::string& err) {
  if (img.w < 1 || img.h < 1 || img.d < 1 ||
      img.data.size() != (size_t)img.w * img.h * img.d) {
    err = "inconsistent image sizes";
    return false;
  }
  const size_t page = (size_t)img.w * img.h * sizeof(float);
  const unsigned kEntries = 10;
  const size_t ifd_size = 2 + kEntries * 12 + 4;
  std::vector<unsigned char> out;
  auto put16 = [&](size_t o, unsigned v) {
    out[o] = v & 255;
    out[o + 1] = (v >> 8) & 255;
  };
  auto put32 = [&](size_t o, unsigned long long v) {
    for (int b = 0; b < 4; ++b) out[o + b] = (v >> (8 * b)) & 255;
  };
  // header, then per page: IFD, then the samples
  size_t total = 8;
  for (int z = 0; z < img.d; ++z) total += ifd_size + page;
  if (total > 0xFFFFFFFFull) {
    err = "image too large for a classic TIFF";
    return false;
  }
  out.assign(total, 0);
  out[0] = 'I';
  out[1] = 'I';
  put16(2, 42);
  size_t pos = 8;
  put32(4, pos);
  for (int z = 0; z < img.d; ++z) {
    const size_t ifd = pos, data = ifd + ifd_size;
    const size_t next = (z + 1 < img.d) ? data + page : 0;
    put16(ifd, kEntries);
    size_t e = ifd + 2;
    auto entry = [&](unsigned tag, unsigned type, unsigned long long count, unsigned long long v) {
      put16(e, tag);
      put16(e + 2, type);
      put32(e + 4, count);
      if (type == 3 && count == 1) put16(e + 8, (unsigned)v);
      else put32(e + 8, v);
      e += 12;
    };
    entry(256, 4, 1, (unsigned)img.w);   // ImageWidth
    entry(257, 4, 1, (unsigned)img.h);   // ImageLength
    entry(258, 3, 1, 32);                // BitsPerSample
    entry(259, 3, 1, 1);                 // Compression: none
    entry(262, 3, 1, 1);                 // Photometric: min-is-black
    entry(273, 4, 1, data);              // StripOffsets
    entry(277, 3, 1, 1);                 // SamplesPerPixel
    entry(278, 4, 1, (unsigned)img.h);   // RowsPerStrip
    entry(279, 4, 1, page);              // StripByteCounts
    entry(339, 3, 1, 3);                 // SampleFormat: IEEE float
    put32(e, next);
    const float* src = img.data.data() + (size_t)z * img.w * img.h;
    for (size_t i = 0; i < (size_t)img.w * img.h; ++i) {
      unsigned u;
      memcpy(&u, src + i, 4);
      put32(data + 4 * i, u);
    }
    pos = data + page;
  }
  FILE* f = fopen(path, "wb");
  if (!f) {
    err = "cannot open output file";
    return false;
  }
  const bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
  if (fclose(f) != 0 || !ok) {
    err = "write failed";
    return false;
  }
  return true;
}

}  // namespace cdx
