// Registry of the compile-time specialised transform lengths.
//
// CDX_SPLAN_LIST gives each registered length and its radices (their
// product is the length; radices up to 32 points run in registers).  The
// per-axis lists say for which pass kernels a length is instantiated and
// with which tile: x passes with P row pairs per block (the same P as the
// generic x tiles), y passes with V rows, z passes with W columns.  Other
// lengths use the generic engine.
#pragma once

#include <vector>

#include "fft_static.cuh"
#include "static_plans_gen.cuh"

#define CDX_SPLAN_LIST(F) \
  F(32, 8, 4)             \
  F(64, 8, 8)             \
  F(100, 10, 10)          \
  F(128, 16, 8)           \
  F(256, 16, 16)          \
  F(512, 32, 16)          \
  F(756, 9, 12, 7)        \
  F(1024, 32, 32)         \
  F(1620, 15, 12, 9)      \
  CDX_GEN_SPLANS(F)

// Plans for the x ratio and x update passes where they differ from the
// length's registered plan: F(L, P, radices...).  1024 = 32*32 gives a row
// pair 32 threads of 32 values, and those two passes, which stage several
// row arrays per tile, then fit few warps per SM; 8*16*8 with two pairs per
// block holds 16 values per thread in a 256-thread block.
#define CDX_XR_PLANS(F) F(1024, 2, 8, 16, 8)

#define CDX_X_PLANS(F) F(128, 8) F(256, 8) F(512, 4) F(756, 2) F(1024, 4) F(1620, 2)
// y entries: F(L, rows per block, extra registers of the launch bounds,
// padding periods of the two stage layouts of a three-radix plan)
#define CDX_Y_PLANS(F) \
  F(128, 16, 0, 0, 0) F(256, 8, 0, 0, 0) F(512, 4, 0, 0, 0) F(1024, 4, 0, 0, 0) CDX_GEN_Y_PLANS(F)
#define CDX_Z_PLANS(F) F(32, 16) F(64, 16) F(100, 16) F(128, 16) F(256, 16)
// generated z plans (types SPZ<L>, twiddles FftLen::gzdev): F(L, columns
// per block, extra registers); instantiated for radially averaged OTFs only
#define CDX_Z_GEN_PLANS(F) CDX_GEN_Z_PLANS(F)

namespace cdx {

#define CDX_DEF_SPLAN(L, ...) using SP##L = SPlan<L, __VA_ARGS__>;
CDX_SPLAN_LIST(CDX_DEF_SPLAN)
#undef CDX_DEF_SPLAN

#define CDX_DEF_GXPLAN(L, ...) using SPX##L = SPlan<L, __VA_ARGS__>;
CDX_GEN_X_SPLANS(CDX_DEF_GXPLAN)
#undef CDX_DEF_GXPLAN

#define CDX_DEF_GZPLAN(L, ...) using SPZ##L = SPlan<L, __VA_ARGS__>;
CDX_GEN_Z_SPLANS(CDX_DEF_GZPLAN)
#undef CDX_DEF_GZPLAN

#define CDX_DEF_XRPLAN(L, P, ...) using SPR##L = SPlan<L, __VA_ARGS__>;
CDX_XR_PLANS(CDX_DEF_XRPLAN)
#undef CDX_DEF_XRPLAN

#define CDX_FIT_ROWS(L, V) \
  static_assert(splan_rows_fit<SP##L, V>(), "row tile too small for the static plan of length " #L);
CDX_X_PLANS(CDX_FIT_ROWS)
#undef CDX_FIT_ROWS
#define CDX_FIT_GX(L, P) \
  static_assert(splan_rows_fit<SPX##L, P>(), "row tile too small for the x plan of length " #L);
CDX_GEN_X_PAIRS(CDX_FIT_GX)
#undef CDX_FIT_GX
#define CDX_FIT_XR(L, P, ...) \
  static_assert(splan_rows_fit<SPR##L, P>(), "row tile too small for the x ratio plan of " #L);
CDX_XR_PLANS(CDX_FIT_XR)
#undef CDX_FIT_XR

// Radices of the registered plan for length L (false when L is not registered).
inline bool static_radices(int L, std::vector<int>& rad) {
  switch (L) {
#define CDX_RAD_CASE(LL, ...) \
  case LL:                    \
    rad = {__VA_ARGS__};      \
    return true;
    CDX_SPLAN_LIST(CDX_RAD_CASE)
#undef CDX_RAD_CASE
    default:
      return false;
  }
}

// Radices of the generated x-pass plan for length L (false when it has none).
inline bool gx_radices(int L, std::vector<int>& rad) {
  switch (L) {
#define CDX_GX_CASE(LL, ...) \
  case LL:                   \
    rad = {__VA_ARGS__};     \
    return true;
    CDX_GEN_X_SPLANS(CDX_GX_CASE)
#undef CDX_GX_CASE
    default:
      return false;
  }
}

// Row pairs per block of the generated x-pass plan for length L (false when
// it has none).
inline bool gx_pairs(int L, int& pairs) {
  switch (L) {
#define CDX_GXP_CASE(LL, PP) \
  case LL:                   \
    pairs = PP;              \
    return true;
    CDX_GEN_X_PAIRS(CDX_GXP_CASE)
#undef CDX_GXP_CASE
    default:
      return false;
  }
}

// Radices of the generated z-pass plan for length L (false when it has none).
inline bool gz_radices(int L, std::vector<int>& rad) {
  switch (L) {
#define CDX_GZ_CASE(LL, ...) \
  case LL:                   \
    rad = {__VA_ARGS__};     \
    return true;
    CDX_GEN_Z_SPLANS(CDX_GZ_CASE)
#undef CDX_GZ_CASE
    default:
      return false;
  }
}

// Radices and row pairs of the x ratio / x update plan for length L (false
// when those passes use the length's registered plan).
inline bool xr_radices(int L, std::vector<int>& rad, int& pairs) {
  switch (L) {
#define CDX_XR_CASE(LL, PP, ...) \
  case LL:                       \
    rad = {__VA_ARGS__};         \
    pairs = PP;                  \
    return true;
    CDX_XR_PLANS(CDX_XR_CASE)
#undef CDX_XR_CASE
    default:
      return false;
  }
}

}  // namespace cdx
