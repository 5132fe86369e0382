/*
 * ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load this file's library; the product
 * (cudadecon_gb300/lib/libcudaDecon.so) never does.
 *
 * Plain C restatement of the reference's geometry kernels, evaluated on the
 * CPU in the same floating-point order as the CUDA code the reference's
 * nvcc build produces (nvcc contracts a*b+c into fused multiply-adds by
 * default; the contractions are written out here with fma()/fmaf(), and the
 * file is compiled with -ffp-contract=off so the C compiler adds none):
 *
 *   oracle_deskew  <- deskew_kernel,  src/geometryTransform.cu:4-31
 *   oracle_rotate  <- rotate_kernel,  src/geometryTransform.cu:50-88
 *   oracle_camcor  <- camcor_kernel,  src/camcor.cu:80-108
 *
 * With contract == 0 every product is rounded separately (no fused
 * multiply-add), which is what a build with -fmad=false would compute.
 * camcor calls the C library's expf(), which may differ from CUDA's expf()
 * in the last bit; callers compare camcor with a tolerance of one count.
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>

void oracle_deskew(const float* in, int nx, int ny, int nz, float* out, int nxOut, int extraShift,
                   double deskewFactor, float padVal, int contract) {
  for (int zout = 0; zout < nz; ++zout)
    for (int yout = 0; yout < ny; ++yout)
      for (int xout = 0; xout < nxOut; ++xout) {
        /* (xout - nxOut/2. + extraShift) - deskewFactor*(zout - nz/2.) + nx/2. in double */
        const double a = ((double)(unsigned)xout - nxOut / 2.) + (double)extraShift;
        const double b = (double)(unsigned)zout - nz / 2.;
        const double t = contract ? fma(-deskewFactor, b, a) : a - deskewFactor * b;
        const float xin = (float)(t + nx / 2.);
        const size_t indout = ((size_t)zout * ny + yout) * nxOut + xout;
        if (xin >= 0 && xin < (float)(nx - 1)) {
          const float fl = floorf(xin);
          const size_t indin = ((size_t)zout * ny + yout) * nx + (unsigned)fl;
          const float off = xin - fl;
          const float w0 = 1.0f - off;
          out[indout] = contract ? fmaf(w0, in[indin], off * in[indin + 1])
                                 : w0 * in[indin] + off * in[indin + 1];
        } else {
          out[indout] = padVal;
        }
      }
}

/* coord_mode: how r0*zc + r1*xc is contracted (0: not at all, 1: fmaf(r0, zc, r1*xc),
 * 2: fmaf(r1, xc, r0*zc)); interp_mode likewise for each a*b + c*d of the
 * bilinear blend (0: none, 1: first product fused, 2: second product fused). */
void oracle_rotate_v(const float* in, int nx_in, int ny, int nz_in, float* out, int nx_out,
                     int nz_out, const float* rot, int coord_mode, int interp_mode) {
  const size_t nxy_in = (size_t)nx_in * ny, nxy_out = (size_t)nx_out * ny;
#define MAC2(a, b, c, d, mode) \
  ((mode) == 1 ? fmaf((a), (b), (c) * (d)) : (mode) == 2 ? fmaf((c), (d), (a) * (b)) : (a) * (b) + (c) * (d))
  for (int zout = 0; zout < nz_out; ++zout)
    for (int yout = 0; yout < ny; ++yout)
      for (int xout = 0; xout < nx_out; ++xout) {
        const float xc = (float)((double)(unsigned)xout - nx_out / 2.);
        const float zc = (float)((double)(unsigned)zout - nz_out / 2.);
        const float s0 = MAC2(rot[0], zc, rot[1], xc, coord_mode);
        const float s1 = MAC2(rot[2], zc, rot[3], xc, coord_mode);
        const float zin = (float)((double)s0 + nz_in / 2.);
        const float xin = (float)((double)s1 + nx_in / 2.);
        const size_t indout = (size_t)(nz_out - 1 - zout) * nxy_out + (size_t)yout * nx_out + xout;
        if (xin >= 0 && xin < (float)(nx_in - 1) && zin >= 0 && zin < (float)(nz_in - 1)) {
          const float fz = floorf(zin), fx = floorf(xin);
          const size_t i00 = (size_t)(unsigned)fz * nxy_in + (size_t)yout * nx_in + (unsigned)fx;
          const size_t i01 = i00 + 1, i10 = i00 + nxy_in, i11 = i10 + 1;
          const float xo = xin - fx, zo = zin - fz;
          const float wx = 1.0f - xo, wz = 1.0f - zo;
          const float a = MAC2(wx, in[i00], xo, in[i01], interp_mode);
          const float b = MAC2(wx, in[i10], xo, in[i11], interp_mode);
          out[indout] = MAC2(wz, a, zo, b, interp_mode);
        } else {
          out[indout] = 0.f;
        }
      }
#undef MAC2
}

/* The contraction the reference's nvcc build applies to rotate_kernel, as
 * pinned by tests/golden/golden_rotate.npz (reference kernel output). */
int g_rotate_coord_mode = 1, g_rotate_interp_mode = 1;

void oracle_rotate(const float* in, int nx_in, int ny, int nz_in, float* out, int nx_out,
                   int nz_out, const float* rot, int contract) {
  oracle_rotate_v(in, nx_in, ny, nz_in, out, nx_out, nz_out, rot,
                  contract ? g_rotate_coord_mode : 0, contract ? g_rotate_interp_mode : 0);
}

/* float -> unsigned short as the GPU converts it: round toward zero,
 * saturating to [0, 65535], NaN -> 0. */
static unsigned short f2u16_sat(float v) {
  if (!(v > 0.f)) return 0;
  if (v >= 65535.f) return 65535;
  return (unsigned short)v;
}

void oracle_camcor(const uint16_t* raw, int nx, int ny, int nz, const float* camparam,
                   uint16_t* out, int contract) {
  const size_t nxy = (size_t)nx * ny;
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const size_t pix = (size_t)y * nx + x;
        const float a = camparam[pix], b = camparam[nxy + pix], off = camparam[2 * nxy + pix];
        const unsigned v = raw[(size_t)z * nxy + pix];
        const int zp = z == 0 ? nz - 1 : z - 1;
        const unsigned vp = raw[(size_t)zp * nxy + pix];
        const float p = (float)vp - off;
        const float e = expf(-b * p);
        const float q = 1.0f - e;
        const float m = 0.9f * a;
        const float t1 = (float)(int)(unsigned short)v - off;
        const float r = contract ? fmaf(-m, q, t1) : t1 - m * q;
        out[(size_t)z * nxy + pix] = f2u16_sat(r);
      }
}
