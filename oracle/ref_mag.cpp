// ref_mag.cpp -- the reference's magnetisation walker, compiled for the host.
//
// TEST INFRASTRUCTURE ONLY.  This translation unit includes the reference's
// unmodified headers (include paths from oracle/Makefile) and runs its kernel
// updateWalkersMag (src/kernels/kernelMag.cuh:1-141) with the B-field
// functors (src/functors/bfunctors.cuh) and Bloch integrators
// (src/bloch/blochdiff.cuh) as a host function, one walker at a time, with
// the stand-ins of ref_shim.cpp (empty __device__, real = double, the
// Philox stream behind curandState, a hook after every boundaryNormal call).
// One build per compile-time switch set (SPECULAR_REFLECTION,
// RK4_NORELAXATION, ROTATE_MULTISTEP), each in its own namespace SHIM_NS and
// exporting ref_mag_<SHIM_NS>.  Output: part of oracle/_ref/libaxxref.so.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <vector>

#include <cuda_runtime_api.h>

#include "oracle.h"

#ifndef SHIM_NS
#error "define SHIM_NS"
#endif

struct curandState {
  uint64_t seed, sub;
  uint32_t word;
};
struct ShimDim3 {
  unsigned x, y, z;
};
extern thread_local ShimDim3 threadIdx, blockIdx, blockDim;
extern thread_local uint32_t shim_last_word;
uint32_t shim_stream_word(uint64_t seed, uint64_t walker, uint32_t k);

inline void curand_init(unsigned long long seed, unsigned long long sub, unsigned long long offset,
                        curandState *s) {
  s->seed = seed;
  s->sub = sub;
  s->word = 1u + (uint32_t)offset;
}
inline float curand_uniform(curandState *s) {
  const uint32_t x = shim_stream_word(s->seed, s->sub, s->word++);
  shim_last_word = s->word;
  return (float)(x >> 9) * 1.1920928955078125e-07f + 5.9604644775390625e-08f;
}
inline unsigned int curand(curandState *s) {
  const uint32_t x = shim_stream_word(s->seed, s->sub, s->word++);
  shim_last_word = s->word;
  return x;
}

#define __device__
#define __host__
#define __global__
#define EPSILON 1e-14
#define GAMMA 267500.0
#define PI 3.1415926535897932384626433832795
#define private public

namespace SHIM_NS {
typedef double real;
using std::max;
using std::min;
using std::vector;
#include "misc.cuh"
#include "vector3.cuh"
#include "compare.cuh"
#include "simuParams.cuh"
#include "cylinderXY.cuh"
#include "Sphere.cuh"
#include "boundaryCheck.cuh"
#include "bfunctors.cuh"
#include "blochdiff.cuh"
#include "kernelSetup.cuh"

thread_local long calls0 = 0;

template <class B>
struct Counted : B {
  bool intersect(const Vector3 &ri, const Vector3 &rf, real &v) const {
    ++calls0;
    return B::intersect(ri, rf, v);
  }
};

// Functor standing for any of the reference's B-field functors.
struct AnyField {
  int kind = 0;
  QSC_GRE gre;
  QSC_PGSE pgse;
  QSC_COS_GRE qcos;
  QSC_GRE_TRAP trap;
  SIN_GRE sing;
  COS_GRE cosg;
  RECT_GRE rect;
  UCN_lowfield ucn;
  Vector3 operator()(Vector3 r, real t) const {
    switch (kind) {
      case 0: return gre(r, t);
      case 1: return pgse(r, t);
      case 2: return qcos(r, t);
      case 3: return trap(r, t);
      case 4: return sing(r, t);
      case 5: return cosg(r, t);
      case 6: return rect(r, t);
      default: return ucn(r, t);
    }
  }
  real getStepTimeMin(real t) const {
    // QSC_PGSE declares it non-const
    return kind == 1 ? const_cast<QSC_PGSE &>(pgse).getStepTimeMin(t) : ucn.getStepTimeMin(t);
  }
};

AnyField make_field(const orc_field &f) {
  AnyField a;
  a.kind = f.kind;
  const Vector3 g(f.gx, f.gy, f.gz);
  switch (f.kind) {
    case 0: a.gre = QSC_GRE(f.B0, f.G, f.duration, f.spacing); break;
    case 1:
      a.pgse = QSC_PGSE(f.B0, f.G, f.duration, f.spacing, f.rf_duration, f.dtmin, f.dtmax, f.TE);
      break;
    case 2: a.qcos = QSC_COS_GRE(f.B0, f.G, f.duration, f.spacing, (real)f.num_periods); break;
    case 3: a.trap = QSC_GRE_TRAP(f.B0, f.G, f.duration, f.spacing, f.ramp); break;
    case 4: a.sing = SIN_GRE(f.B0, g, f.duration, f.spacing, f.period); break;
    case 5: a.cosg = COS_GRE(f.B0, g, f.duration, f.spacing, f.num_periods); break;
    case 6: a.rect = RECT_GRE(f.B0, g, f.duration, f.spacing); break;
    default: a.ucn = UCN_lowfield(f.B0, f.G, f.rf_duration, f.dtmin, f.dtmax); break;
  }
  return a;
}

struct Hook {
  orc_trace *tr = nullptr;
  int64_t w = 0;
  int steps = 0, i = 0;
  long last_calls = 0;
  const void *basis = nullptr;
  bool (*inside)(const void *basis, const Vector3 &r) = nullptr;
};
thread_local Hook hook;

inline void shim_after_single_move(Vector3 &r) {
  if (!hook.tr || hook.w >= hook.tr->ntrace) return;
  ++hook.i;
  const size_t o = (size_t)hook.w * (size_t)(hook.steps - 1) + (size_t)(hook.i - 1);
  hook.tr->pos[o * 3 + 0] = r.x;
  hook.tr->pos[o * 3 + 1] = r.y;
  hook.tr->pos[o * 3 + 2] = r.z;
  hook.tr->region[o] = hook.inside(hook.basis, r) ? 0 : -1;
  const long d = calls0 - hook.last_calls;
  hook.last_calls = calls0;
  hook.tr->hits[o] = d == 0 ? 0 : (int32_t)(d - 1);
  hook.tr->words[o] = (int32_t)shim_last_word;
}

#define boundaryNormal(a, b, c, d, e) \
  boundaryNormal(a, b, c, d, e);      \
  shim_after_single_move(b)
#include "kernelMag.cuh"
#undef boundaryNormal

template <class B>
bool inside_of(const void *basisp, const Vector3 &r) {
  return ((const Counted<B> *)basisp)->inside(r);
}

template <class B>
B make_basis(const orc_basis &q);
template <>
Cylinder_XY make_basis<Cylinder_XY>(const orc_basis &q) {
  return Cylinder_XY(q.cx, q.cy, q.radius, q.T2, q.T1, q.D, q.region, q.permeability, q.eps);
}
template <>
Sphere make_basis<Sphere>(const orc_basis &q) {
  return Sphere(q.cx, q.cy, q.cz, q.radius, q.T2, q.T1, q.D, q.region, q.permeability, q.eps);
}

template <class B>
int run(const orc_basis *pore, const orc_field *f, int nf, const orc_mag_params *p, double *sums,
        double *m_walk, orc_trace *tr) {
  const int N = (int)p->num_walkers;
  Counted<B> basis;
  static_cast<B &>(basis) = make_basis<B>(*pore);
  std::vector<AnyField> F(nf);
  for (int j = 0; j < nf; ++j) F[j] = make_field(f[j]);
  SimuParams par(N, p->steps, nf, p->timestep, (int)p->seed, p->m0[0], p->m0[1], p->m0[2]);
  std::vector<curandState> states(N);
  std::vector<real> mx((size_t)nf * N), my((size_t)nf * N), mz((size_t)nf * N);
  blockIdx.x = 0;
  blockDim.x = 1;
  for (int w = 0; w < N; ++w) {
    threadIdx.x = (unsigned)w;
    setup_kernel(states.data(), &par);
    hook = Hook();
    if (tr && w < tr->ntrace) {
      hook.tr = tr;
      hook.w = w;
      hook.steps = p->steps;
      hook.basis = &basis;
      hook.inside = inside_of<B>;
      hook.last_calls = calls0;
      curandState tmp = states[w];
      const Vector3 r0 = basis.unifRand(tmp);
      tr->init_pos[w * 3 + 0] = r0.x;
      tr->init_pos[w * 3 + 1] = r0.y;
      tr->init_pos[w * 3 + 2] = r0.z;
    }
    updateWalkersMag<AnyField, Counted<B>>(&par, &basis, F.data(), states.data(), mx.data(),
                                           my.data(), mz.data());
    hook = Hook();
  }
  // magAcquisitionStream::runAcquisition: per-field sums over the walkers
  for (int j = 0; j < nf; ++j) {
    double s[3] = {0, 0, 0};
    for (int w = 0; w < N; ++w) {
      const size_t o = (size_t)w + (size_t)j * N;
      s[0] += mx[o];
      s[1] += my[o];
      s[2] += mz[o];
      if (m_walk && tr && w < tr->ntrace) {
        double *m = m_walk + ((size_t)w * nf + j) * 3;
        m[0] = mx[o];
        m[1] = my[o];
        m[2] = mz[o];
      }
    }
    for (int k = 0; k < 3; ++k) sums[j * 3 + k] = s[k];
  }
  return 0;
}

}  // namespace SHIM_NS

#define SHIM_CAT2(a, b) a##b
#define SHIM_CAT(a, b) SHIM_CAT2(a, b)

extern "C" int SHIM_CAT(ref_mag_, SHIM_NS)(const orc_basis *pore, const orc_field *f, int nf,
                                           const orc_mag_params *p, double *sums, double *m_walk,
                                           orc_trace *trace) {
  if (!pore || !p || p->num_walkers < 1 || p->steps < 1 || nf < 1 || !f || !sums) return -1;
  if (pore->type == 1)
    return SHIM_NS::run<SHIM_NS::Sphere>(pore, f, nf, p, sums, m_walk, trace);
  return SHIM_NS::run<SHIM_NS::Cylinder_XY>(pore, f, nf, p, sums, m_walk, trace);
}
