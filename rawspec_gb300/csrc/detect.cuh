// detect.cuh -- detection of the two polarisations' spectra into the output
// products, accumulated in registers.
//
// Formulas follow the reference's cuFFT store callbacks:
//   total power (Npolout 1)  P  += |X0|^2 (+ |X1|^2)          rawspec_gpu.cu:153-161
//   full pol    (Npolout +4) XX += |X0|^2, YY += |X1|^2,
//                            re += Re(X0 X1*), im += Im(X0 X1*) rawspec_gpu.cu:223-267
//   Stokes      (Npolout -4) I  += |X0|^2 + |X1|^2, Q += |X0|^2 - |X1|^2,
//                            U  += Re(X0 X1*), V += Im(X0 X1*)  rawspec_gpu.cu:167-218
// with the imaginary cross term negated when the input is conjugated.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace rsg {

template <int POL>
struct PolOut {
  static constexpr int NP = (POL == POL_TP) ? 1 : 4;
};

template <int POL, int NV>
__device__ __forceinline__ void detect_acc(float (&a)[PolOut<POL>::NP], const float2 (&x)[NV],
                                           float im_sign) {
  if constexpr (POL == POL_TP) {
    float s = a[0];
    s = __fmaf_rn(x[0].x, x[0].x, s);
    s = __fmaf_rn(x[0].y, x[0].y, s);
    if constexpr (NV == 2) {
      s = __fmaf_rn(x[1].x, x[1].x, s);
      s = __fmaf_rn(x[1].y, x[1].y, s);
    }
    a[0] = s;
  } else {
    static_assert(NV == 2, "cross-pol products need two polarisations");
    const float p0 = __fmaf_rn(x[0].x, x[0].x, x[0].y * x[0].y);
    const float p1 = __fmaf_rn(x[1].x, x[1].x, x[1].y * x[1].y);
    const float re = __fmaf_rn(x[0].x, x[1].x, x[0].y * x[1].y);
    const float im = __fmaf_rn(x[0].y, x[1].x, -(x[0].x * x[1].y));
    if constexpr (POL == POL_FULL) {
      a[0] += p0;
      a[1] += p1;
    } else {
      a[0] += p0 + p1;
      a[1] += p0 - p1;
    }
    a[2] += re;
    a[3] = __fmaf_rn(im_sign, im, a[3]);
  }
}

// Position of forward-FFT bin k in the FFT-shifted output of an N-point
// transform in the requested direction: inverse transforms read bin -k, and
// the shift puts bin 0 at N/2 (rawspec_gpu.cu:1659-1691).
__device__ __forceinline__ int out_pos(int k, int N, int inverse) {
  const int kr = inverse ? ((N - k) & (N - 1)) : k;
  return (kr + (N >> 1)) & (N - 1);
}

}  // namespace rsg
