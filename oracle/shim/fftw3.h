/* ORACLE — test infrastructure only.
 *
 * A stand-in for the three FFTW calls of the reference's makeOTF
 * (src/radialft_interface.cpp:144-151): an in-place 3D real-to-complex
 * transform with FFTW's layout (input rows padded to 2*(n2/2+1) floats,
 * output (n0, n1, n2/2+1) complex), unnormalised, forward sign -1.  FFTW is
 * not in this image; oracle/shim/fftw_shim.cpp computes the transform as
 * direct DFTs along each axis in double precision. */
#ifndef CDX_FFTW_SHIM_H
#define CDX_FFTW_SHIM_H

typedef float fftwf_complex[2];
typedef struct cdx_fftwf_plan* fftwf_plan;
#define FFTW_ESTIMATE (1U << 6)

#ifdef __cplusplus
extern "C" {
#endif
fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float* in, fftwf_complex* out,
                                 unsigned flags);
void fftwf_execute_dft_r2c(const fftwf_plan p, float* in, fftwf_complex* out);
void fftwf_destroy_plan(fftwf_plan p);
#ifdef __cplusplus
}
#endif

#endif
