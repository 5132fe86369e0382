/* ORACLE — test infrastructure only.
 *
 * A stand-in for libtiff's public header (libtiff is not in this image),
 * enough for CImg's TIFF code as compiled into the reference's
 * src/radialft_interface.cpp (makeOTF).  Writes are captured in memory
 * (oracle/shim/tiff_capture.cpp) instead of going to a file, so that the
 * runner in oracle/radialft_runner.cpp can hand makeOTF's output to the
 * tests; reads are not supported (inputs are given to makeOTF as .cimg).
 * Tag numbers and values are those of the TIFF 6.0 specification. */
#ifndef CDX_TIFF_SHIM_H
#define CDX_TIFF_SHIM_H

#include <stdarg.h>
#include <stdint.h>

typedef uint8_t uint8;
typedef uint16_t uint16;
typedef uint32_t uint32;
typedef int32_t int32;
typedef int64_t tmsize_t;
typedef tmsize_t tsize_t;
typedef uint32 tstrip_t;
typedef uint32 ttile_t;
typedef void* tdata_t;
typedef void* thandle_t;
typedef uint64_t toff_t;
typedef struct cdx_tiff TIFF;
typedef void (*TIFFErrorHandler)(const char*, const char*, va_list);

#define TIFFTAG_IMAGEWIDTH 256
#define TIFFTAG_IMAGELENGTH 257
#define TIFFTAG_BITSPERSAMPLE 258
#define TIFFTAG_COMPRESSION 259
#define TIFFTAG_PHOTOMETRIC 262
#define TIFFTAG_FILLORDER 266
#define TIFFTAG_IMAGEDESCRIPTION 270
#define TIFFTAG_ORIENTATION 274
#define TIFFTAG_SAMPLESPERPIXEL 277
#define TIFFTAG_ROWSPERSTRIP 278
#define TIFFTAG_XRESOLUTION 282
#define TIFFTAG_YRESOLUTION 283
#define TIFFTAG_PLANARCONFIG 284
#define TIFFTAG_RESOLUTIONUNIT 296
#define TIFFTAG_SOFTWARE 305
#define TIFFTAG_TILEWIDTH 322
#define TIFFTAG_TILELENGTH 323
#define TIFFTAG_SAMPLEFORMAT 339
#define COMPRESSION_NONE 1
#define COMPRESSION_LZW 5
#define COMPRESSION_JPEG 7
#define PHOTOMETRIC_MINISBLACK 1
#define PHOTOMETRIC_RGB 2
#define FILLORDER_MSB2LSB 1
#define ORIENTATION_TOPLEFT 1
#define PLANARCONFIG_CONTIG 1
#define RESUNIT_NONE 1
#define SAMPLEFORMAT_UINT 1
#define SAMPLEFORMAT_INT 2
#define SAMPLEFORMAT_IEEEFP 3

#define TIFFGetR(abgr) ((abgr) & 0xff)
#define TIFFGetG(abgr) (((abgr) >> 8) & 0xff)
#define TIFFGetB(abgr) (((abgr) >> 16) & 0xff)
#define TIFFGetA(abgr) (((abgr) >> 24) & 0xff)

#ifdef __cplusplus
extern "C" {
#endif
TIFFErrorHandler TIFFSetWarningHandler(TIFFErrorHandler);
TIFFErrorHandler TIFFSetErrorHandler(TIFFErrorHandler);
TIFF* TIFFOpen(const char*, const char*);
void TIFFClose(TIFF*);
const char* TIFFFileName(TIFF*);
int TIFFSetField(TIFF*, uint32, ...);
int TIFFGetField(TIFF*, uint32, ...);
int TIFFGetFieldDefaulted(TIFF*, uint32, ...);
int TIFFSetDirectory(TIFF*, uint16);
int TIFFReadDirectory(TIFF*);
int TIFFWriteDirectory(TIFF*);
uint32 TIFFDefaultStripSize(TIFF*, uint32);
tmsize_t TIFFStripSize(TIFF*);
tmsize_t TIFFTileSize(TIFF*);
uint32 TIFFComputeStrip(TIFF*, uint32, uint16);
tmsize_t TIFFWriteEncodedStrip(TIFF*, uint32, void*, tmsize_t);
tmsize_t TIFFReadEncodedStrip(TIFF*, uint32, void*, tmsize_t);
tmsize_t TIFFReadTile(TIFF*, void*, uint32, uint32, uint32, uint16);
int TIFFIsTiled(TIFF*);
int TIFFReadRGBAImage(TIFF*, uint32, uint32, uint32*, int);
void* _TIFFmalloc(tmsize_t);
void _TIFFfree(void*);
#ifdef __cplusplus
}
#endif

#endif
