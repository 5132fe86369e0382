// ORACLE — test infrastructure only: the libtiff calls of
// oracle/shim/tiffio.h.  A TIFF opened for writing collects its
// directories (width, height, bits per sample, strip bytes) in memory;
// cdx_tiff_captured() hands the last closed file's directories to the
// runner.  Reading is not supported (every read call fails).
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tiffio.h"

namespace {
struct Dir {
  uint32 width = 0, height = 0, bps = 32, spp = 1, rows = 0;
  std::vector<unsigned char> data;
};
}  // namespace

struct cdx_tiff {
  std::string name;
  std::vector<Dir> dirs;
  Dir cur;
};

static std::vector<Dir> g_last;

extern "C" {
TIFFErrorHandler TIFFSetWarningHandler(TIFFErrorHandler) { return nullptr; }
TIFFErrorHandler TIFFSetErrorHandler(TIFFErrorHandler) { return nullptr; }
TIFF* TIFFOpen(const char* name, const char* mode) {
  if (!mode || mode[0] != 'w') return nullptr;
  TIFF* t = new cdx_tiff;
  t->name = name ? name : "";
  return t;
}
void TIFFClose(TIFF* t) {
  if (!t) return;
  g_last = t->dirs;
  delete t;
}
const char* TIFFFileName(TIFF* t) { return t ? t->name.c_str() : ""; }
int TIFFSetField(TIFF* t, uint32 tag, ...) {
  va_list ap;
  va_start(ap, tag);
  switch (tag) {
    case TIFFTAG_IMAGEWIDTH: t->cur.width = va_arg(ap, unsigned); break;
    case TIFFTAG_IMAGELENGTH: t->cur.height = va_arg(ap, unsigned); break;
    case TIFFTAG_BITSPERSAMPLE: t->cur.bps = va_arg(ap, unsigned); break;
    case TIFFTAG_SAMPLESPERPIXEL: t->cur.spp = va_arg(ap, unsigned); break;
    case TIFFTAG_ROWSPERSTRIP: t->cur.rows = va_arg(ap, unsigned); break;
    default: break;
  }
  va_end(ap);
  return 1;
}
int TIFFGetField(TIFF*, uint32, ...) { return 0; }
int TIFFGetFieldDefaulted(TIFF*, uint32, ...) { return 0; }
int TIFFSetDirectory(TIFF*, uint16) { return 1; }
int TIFFReadDirectory(TIFF*) { return 0; }
int TIFFWriteDirectory(TIFF* t) {
  t->dirs.push_back(t->cur);
  t->cur = Dir{};
  return 1;
}
uint32 TIFFDefaultStripSize(TIFF* t, uint32 req) {
  return (req == 0 || req == (uint32)-1) ? t->cur.height : req;
}
tmsize_t TIFFStripSize(TIFF* t) {
  const uint32 rows = t->cur.rows ? t->cur.rows : t->cur.height;
  return (tmsize_t)t->cur.width * rows * t->cur.spp * (t->cur.bps / 8);
}
tmsize_t TIFFTileSize(TIFF*) { return 0; }
uint32 TIFFComputeStrip(TIFF* t, uint32 row, uint16) {
  return t->cur.rows ? row / t->cur.rows : 0;
}
tmsize_t TIFFWriteEncodedStrip(TIFF* t, uint32, void* buf, tmsize_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(buf);
  t->cur.data.insert(t->cur.data.end(), b, b + n);
  return n;
}
tmsize_t TIFFReadEncodedStrip(TIFF*, uint32, void*, tmsize_t) { return -1; }
tmsize_t TIFFReadTile(TIFF*, void*, uint32, uint32, uint32, uint16) { return -1; }
int TIFFIsTiled(TIFF*) { return 0; }
int TIFFReadRGBAImage(TIFF*, uint32, uint32, uint32*, int) { return 0; }
void* _TIFFmalloc(tmsize_t n) { return std::malloc((size_t)n); }
void _TIFFfree(void* p) { std::free(p); }

// The directories of the last TIFF closed after writing: their count, and
// for directory i (when out is not NULL) width, height and the float samples
// (32-bit samples only).  Returns the number of directories.
int cdx_tiff_captured(int i, int* width, int* height, float* out, long capacity) {
  if (i < 0 || i >= (int)g_last.size()) return (int)g_last.size();
  const Dir& d = g_last[i];
  *width = (int)d.width;
  *height = (int)d.height;
  if (out && d.bps == 32) {
    const long n = (long)d.data.size() / 4;
    std::memcpy(out, d.data.data(), sizeof(float) * (size_t)(n < capacity ? n : capacity));
  }
  return (int)g_last.size();
}
}
