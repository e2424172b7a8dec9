// adapter_adc.cpp -- the C++ adapter's post-processing without a GPU:
// linear_regression and phaseAcquisition<F>::calcADC / getSignal on given
// sums.  Reads from stdin: kind n points duration spacing periods, then n G
// values, then points*n mx and points*n my values; prints the running ADC and
// ADC mean square after each point, then the last point's signals (%.17g).
// TEST INFRASTRUCTURE.
#include <cstdio>
#include <vector>

#include "axx_acquisition.hpp"
using namespace axonexa;

template <class F>
int run(std::vector<F> fs, int n, int points, const std::vector<double> &mx,
        const std::vector<double> &my) {
  phaseAcquisition<F> a(n, 10, 1, 0);
  for (int i = 0; i < n; ++i) a.addMeasurement(fs[i]);
  for (int p = 0; p < points; ++p) {
    for (int i = 0; i < n; ++i) {
      a.getMx()[i] = mx[p * n + i];
      a.getMy()[i] = my[p * n + i];
    }
    a.calcADC();
    std::printf("%.17g %.17g\n", a.getADC(), a.getADCMeanSquare());
  }
  for (int i = 0; i < n; ++i) std::printf("%.17g\n", a.getSignal(i));
  return 0;
}

int main() {
  int kind, n, points, periods;
  double d, sp;
  if (std::scanf("%d %d %d %lf %lf %d", &kind, &n, &points, &d, &sp, &periods) != 6) return 2;
  std::vector<double> G(n), mx(points * n), my(points * n);
  for (auto &g : G)
    if (std::scanf("%lf", &g) != 1) return 2;
  for (auto &v : mx)
    if (std::scanf("%lf", &v) != 1) return 2;
  for (auto &v : my)
    if (std::scanf("%lf", &v) != 1) return 2;
  const Vector3 x(1.0, 0.0, 0.0);
  if (kind == 0) {
    std::vector<RectGrad> f;
    for (double g : G) f.push_back(RectGrad(g, d, sp));
    return run(f, n, points, mx, my);
  }
  if (kind == 1) {
    std::vector<CosGFunc> f;
    for (double g : G) f.push_back(CosGFunc(g, d, sp, periods, x));
    return run(f, n, points, mx, my);
  }
  std::vector<SinGFunc> f;
  for (double g : G) f.push_back(SinGFunc(g, d, sp, periods, x));
  return run(f, n, points, mx, my);
}
