// ORACLE — test infrastructure only: the FFTW calls of oracle/shim/fftw3.h
// as direct DFTs along each axis in double precision (exact twiddles
// cos/sin(2 pi ((j k) mod n) / n)), rounded once to float at the end.
#include <cmath>
#include <complex>
#include <vector>

#include "fftw3.h"

struct cdx_fftwf_plan {
  int n0, n1, n2;
};

extern "C" fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float*, fftwf_complex*,
                                            unsigned) {
  return new cdx_fftwf_plan{n0, n1, n2};
}

extern "C" void fftwf_destroy_plan(fftwf_plan p) { delete p; }

// In-place DFT of n complex values at stride s.
static void dft1(std::complex<double>* a, int n, long s, std::vector<std::complex<double>>& tmp,
                 const std::vector<std::complex<double>>& w) {
  tmp.assign(n, 0.0);
  for (int k = 0; k < n; ++k) {
    std::complex<double> acc = 0.0;
    for (int j = 0; j < n; ++j) acc += a[j * s] * w[(long)j * k % n];
    tmp[k] = acc;
  }
  for (int k = 0; k < n; ++k) a[k * s] = tmp[k];
}

static std::vector<std::complex<double>> roots(int n) {
  std::vector<std::complex<double>> w(n);
  const double two_pi = 6.283185307179586476925286766559;
  for (int m = 0; m < n; ++m) w[m] = std::polar(1.0, -two_pi * m / n);
  return w;
}

extern "C" void fftwf_execute_dft_r2c(const fftwf_plan p, float* in, fftwf_complex* out) {
  const int n0 = p->n0, n1 = p->n1, n2 = p->n2, h = n2 / 2 + 1, pad = 2 * h;
  std::vector<std::complex<double>> a((size_t)n0 * n1 * n2);
  for (int z = 0; z < n0; ++z)
    for (int y = 0; y < n1; ++y)
      for (int x = 0; x < n2; ++x)
        a[((size_t)z * n1 + y) * n2 + x] = in[((size_t)z * n1 + y) * pad + x];
  std::vector<std::complex<double>> tmp;
  const auto w2 = roots(n2), w1 = roots(n1), w0 = roots(n0);
  for (int z = 0; z < n0; ++z)
    for (int y = 0; y < n1; ++y) dft1(&a[((size_t)z * n1 + y) * n2], n2, 1, tmp, w2);
  for (int z = 0; z < n0; ++z)
    for (int x = 0; x < n2; ++x) dft1(&a[(size_t)z * n1 * n2 + x], n1, n2, tmp, w1);
  for (int y = 0; y < n1; ++y)
    for (int x = 0; x < n2; ++x) dft1(&a[(size_t)y * n2 + x], n0, (long)n1 * n2, tmp, w0);
  for (int z = 0; z < n0; ++z)
    for (int y = 0; y < n1; ++y)
      for (int k = 0; k < h; ++k) {
        const std::complex<double> v = a[((size_t)z * n1 + y) * n2 + k];
        out[((size_t)z * n1 + y) * h + k][0] = (float)v.real();
        out[((size_t)z * n1 + y) * h + k][1] = (float)v.imag();
      }
}
