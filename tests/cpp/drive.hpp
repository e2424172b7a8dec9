// drive.hpp -- the body of a reference-style main, templated on the API's
// types so that one text compiles against the reference's own classes
// (src/acquisition/phaseAcquisitionStream.cuh, phaseAcquisition.cuh,
// src/substrate/lattice.cuh, src/primitives/cylinderXY.cuh,
// src/functors/gfunctors.cuh) and runs against include/axx_acquisition.hpp.
// The call sequence follows the reference's examples (examples/hexPhase.cu:
// phaseAcquisitionStream(particles), phaseAcquisition(NOM, steps, particles,
// seed), addMeasurement, addAcquisition, runAcquisitionLattice(num, basis,
// lattice, timestep, blocks, threads, numOfSM), getSignal, calcEveryADC,
// getADC).  TEST INFRASTRUCTURE.
#pragma once
#include <vector>

// One impermeable cylinder (r 5 um) in a 12 um periodic cell, D 2 um^2/ms,
// T2 80/60 ms; PGSE delta 10 / Delta 40 ms with NOM gradient strengths
// 0..175 mT/m along x; units mm, ms, T.
template <class Stream, class Acq, class PGSE, class Cyl, class Lat>
void drive_cylinder_lattice(int particles, int steps, double timestep, int seed,
                            std::vector<double> &signal, double &adc) {
  const int NOM = 8;
  Stream pas(particles);
  Acq pa(NOM, steps, particles, seed);
  for (int i = 0; i < NOM; i++) {
    PGSE pgse(i * 25e-6, 10.0, 30.0);
    pa.addMeasurement(pgse);
  }
  pas.addAcquisition(pa);
  const double cell = 0.012, radius = 0.005;
  Cyl cyls[1];
  Lat lattice(cell, cell, cell, 60.0, 0.0, 2e-6, 1);
  cyls[0] = Cyl(cell / 2.0, cell / 2.0, radius, 80.0, 0.0, 2e-6, 1, 0.0);
  const int threads = 128;
  const int blocks = particles / threads;
  pas.runAcquisitionLattice(0, cyls, lattice, timestep, blocks, threads, 1);
  signal.clear();
  for (int i = 0; i < NOM; i++) signal.push_back(pas.getAcquisition(0).getSignal(i));
  pas.calcEveryADC();
  adc = pas.getAcquisition(0).getADC();
}
