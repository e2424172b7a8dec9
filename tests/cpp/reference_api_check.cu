// reference_api_check.cu -- compiles drive.hpp's reference-style main against
// the reference's own headers (compile only, never run): the same text that
// runs against include/axx_acquisition.hpp is a valid program of the
// reference's API.  The include list is that of the reference's
// examples/hexPhase.cu without the magnetisation headers (kernelMag.cuh does
// not compile with USE_RELAXATION: its T1/T2 are undeclared there).
// TEST INFRASTRUCTURE.
#define WARP_SIZE 32
#define USE_DOUBLE
#define SPECULAR_REFLECTION
#define USE_RELAXATION
#define GAMMA 267500.0
#define PI 3.1415926535897932384626433832795

#include <assert.h>
#include <cmath>
#include <cuda.h>
#include <curand_kernel.h>
#include <iomanip>
#include <iostream>
#include <time.h>
#include <vector>

typedef double real;
#define EPSILON 1e-14
using namespace std;

#include "CPUkernels.cuh"
#include "Sphere.cuh"
#include "boundaryCheck.cuh"
#include "compare.cuh"
#include "cudaVector.cu"
#include "cudaVector.cuh"
#include "cylinderXY.cuh"
#include "empty.cuh"
#include "gfunctors.cuh"
#include "kernelDEBUG.cuh"
#include "kernelLattice.cuh"
#include "kernelPhase.cuh"
#include "kernelSetup.cuh"
#include "kernelWC.cuh"
#include "lattice.cuh"
#include "misc.cuh"
#include "phaseAcquisition.cuh"
#include "phaseAcquisitionStream.cuh"
#include "pinnedVector.cu"
#include "pinnedVector.cuh"
#include "plane.cuh"
#include "simuParams.cuh"
#include "substrate.cuh"
#include "timer.cuh"
#include "vector3.cuh"

#include "drive.hpp"

// the instantiation the adapter's main runs, with the reference's classes
void reference_api_check(std::vector<double> &s, double &adc) {
  drive_cylinder_lattice<phaseAcquisitionStream<RectGrad>, phaseAcquisition<RectGrad>, RectGrad,
                         Cylinder_XY, Lattice>(1024, 100, 0.002, 7, s, adc);
}
