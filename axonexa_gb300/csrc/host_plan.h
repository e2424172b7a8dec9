// host_plan.h -- host-side planning of one walk: from the C-ABI records to
// the device tables of axx_walk.h.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "../../include/axx.h"
#include "axx_walk.h"

namespace axx {

constexpr double kGammaDefault = 267500.0;  // rad / (ms * T), examples/gammadist.cu:5
constexpr double kPi = 3.1415926535897932384626433832795;

// Unit waveform of a sequence: the x component of the reference functor's
// G(t) for G = 1 and gHat = (1, 0, 0).
double wave_unit(const axx_sequence &q, double t);
double bvalue(const axx_sequence &q, double gamma);
void gradient(const axx_sequence &q, double t, double out[3]);

struct Channel {
  int wave;     // waveform index
  float p[3];   // projection vector (FP32, as the kernel uses it)
};

struct SeqPlan {
  int W = 0;                      // distinct waveforms
  std::vector<int> seq_wave;      // per sequence
  std::vector<Channel> channels;  // K
  std::vector<double> coef;       // [M][K]
  std::vector<float> wave;        // [W][steps]
};

struct GeomPlan {
  int geom = AXX_GEOM_FREE;
  std::vector<float4> geo, aux;
  std::vector<uint32_t> cstart;
  std::vector<uint16_t> clist;
  int gx = 1, gy = 1, gz = 1;
  float inv_hx = 0.f, inv_hy = 0.f, inv_hz = 0.f;
  std::vector<float4> slot_tab;
  std::vector<int> slot_region;
  int ecs_slot = 0;
  float lmax = 0.f;
  float ann_h2x2 = 0.f;  // z-cylinder lattices: 2 h^2 of the annulus test
};

// Returns "" on success or an error message.
std::string plan_sequences(const axx_sequence *seqs, int nseq, int steps, double dt,
                           double gamma, SeqPlan &out);
// list_budget > 0: a lattice of z-cylinders (a 2-D grid) may take a finer
// grid, whose staged tables (instances, cell starts and lists) stay within
// list_budget bytes.
std::string plan_lattice(const axx_lattice *lat, const axx_basis *basis, int nbasis,
                         double dt, uint32_t flags, GeomPlan &out, size_t list_budget = 0);
std::string plan_single(const axx_basis *basis, double dt, GeomPlan &out, float &speed,
                        float &step);

}  // namespace axx
