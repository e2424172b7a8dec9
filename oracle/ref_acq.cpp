// ref_acq.cpp -- the reference's acquisition post-processing, compiled for
// the host.
//
// TEST INFRASTRUCTURE ONLY.  This translation unit includes the reference's
// unmodified headers from its source tree (include path from the build
// recipe, oracle/Makefile): linear_regression (src/util/misc.cuh:41-59), the
// gradient functors (src/functors/gfunctors.cuh) and
// phaseAcquisition<FieldType>::calcADC / getSignal
// (src/acquisition/phaseAcquisition.cuh:46-77), with __device__/__host__
// defined empty and real = double.  It exports them as C functions so the
// tests can pin this repository's calcADC and linear_regression (the Python
// mirror and the C++ adapter) bit for bit.  Output: oracle/_ref/libaxxref_acq.so.
#include <cassert>
#include <cmath>
#include <cstdint>
#include <iostream>
#include <vector>

#include <cuda_runtime_api.h>

#define __device__
#define __host__
#define __global__
#define EPSILON 1e-14
#define GAMMA 267500.0
#define PI 3.1415926535897932384626433832795

namespace refacq {
typedef double real;
using std::vector;
#include "misc.cuh"
#include "vector3.cuh"
#include "gfunctors.cuh"
#include "phaseAcquisition.cuh"

template <class F>
void adc_points(std::vector<F> &fs, int n, int points, const double *mx, const double *my,
                double *adc, double *adcms, double *signal) {
  phaseAcquisition<F> a(n, 10, 1, 0);
  for (int i = 0; i < n; ++i) a.addMeasurement(fs[i]);
  for (int p = 0; p < points; ++p) {
    for (int i = 0; i < n; ++i) {
      a.getMx()[i] = mx[p * n + i];
      a.getMy()[i] = my[p * n + i];
    }
    a.calcADC();
    adc[p] = a.getADC();
    adcms[p] = a.getADCMeanSquare();
  }
  for (int i = 0; i < n; ++i) signal[i] = a.getSignal(i);
}
}  // namespace refacq

extern "C" {

double ref_linear_regression(const double *y, const double *x, int n) {
  std::vector<double> yy(y, y + n), xx(x, x + n);
  return refacq::linear_regression(yy, xx);
}

// kind 0: RectGrad(G[i], duration, spacing); kind 1: CosGFunc(G[i], duration,
// spacing, periods, x); kind 2: SinGFunc.  `points` sets of n sums (mx, my
// row-major); after each set, calcADC; adc/adcms receive the running values,
// signal the last set's getSignal(i).
int ref_calc_adc(int kind, int n, const double *G, double duration, double spacing, int periods,
                 int points, const double *mx, const double *my, double *adc, double *adcms,
                 double *signal) {
  using namespace refacq;
  Vector3 x(1.0, 0.0, 0.0);
  if (kind == 0) {
    std::vector<RectGrad> fs;
    for (int i = 0; i < n; ++i) fs.push_back(RectGrad(G[i], duration, spacing));
    adc_points(fs, n, points, mx, my, adc, adcms, signal);
  } else if (kind == 1) {
    std::vector<CosGFunc> fs;
    for (int i = 0; i < n; ++i) fs.push_back(CosGFunc(G[i], duration, spacing, periods, x));
    adc_points(fs, n, points, mx, my, adc, adcms, signal);
  } else if (kind == 2) {
    std::vector<SinGFunc> fs;
    for (int i = 0; i < n; ++i) fs.push_back(SinGFunc(G[i], duration, spacing, periods, x));
    adc_points(fs, n, points, mx, my, adc, adcms, signal);
  } else {
    return 1;
  }
  return 0;
}

}  // extern "C"
