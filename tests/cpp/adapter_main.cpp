// adapter_main.cpp -- drive.hpp's reference-style main against the C++
// adapter (include/axx_acquisition.hpp) over libaxx.so.  Prints the signals
// and the ADC, one value per line (%.17g).  Usage: adapter_main particles
// steps timestep seed.  TEST INFRASTRUCTURE.
#define SPECULAR_REFLECTION
#define USE_RELAXATION
#define GAMMA 267500.0

#include <cstdio>
#include <cstdlib>
#include <stdexcept>

#include "axx_acquisition.hpp"
using namespace axonexa;
#include "drive.hpp"

int main(int argc, char **argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s particles steps timestep seed\n", argv[0]);
    return 2;
  }
  std::vector<double> s;
  double adc = 0.0;
  try {
    drive_cylinder_lattice<phaseAcquisitionStream<RectGrad>, phaseAcquisition<RectGrad>, RectGrad,
                           Cylinder_XY, Lattice>(std::atoi(argv[1]), std::atoi(argv[2]),
                                                 std::atof(argv[3]), std::atoi(argv[4]), s, adc);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  for (double v : s) std::printf("%.17g\n", v);
  std::printf("%.17g\n", adc);
  return 0;
}
