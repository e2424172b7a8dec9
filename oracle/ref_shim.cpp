// ref_shim.cpp -- the reference's own walker, compiled for the host.
//
// TEST INFRASTRUCTURE ONLY.  This translation unit includes the reference's
// unmodified headers from its source tree (the include path is given by the
// build recipe, oracle/Makefile) and runs its kernels
// updateWalkersLatticePhase (src/kernels/kernelLattice.cuh:1-104) and
// updateWalkersPhase (src/kernels/kernelPhase.cuh:4-66) as plain host
// functions, one walker at a time, with:
//   * __device__/__host__/__global__ defined empty and real = double;
//   * curandState/curand_init/curand_uniform standing for the stream the GPU
//     path uses (Philox4x32-10, word k of walker tid under seed s, draws from
//     word 1 on), so both consume identical uniforms;
//   * a Basis wrapper that counts intersect() calls (boundary hits) and a
//     hook after every Lattice::correctBoundary / boundaryNormal call that
//     records the position, the first containing basis and the stream word.
// The reference's compile-time switches (SPECULAR_REFLECTION, USE_PERMEABLE,
// USE_RELAXATION) are set per build of this file; each build lives in its own
// namespace SHIM_NS and exports ref_walk_<SHIM_NS>.
//
// Nothing here is shipped or copied: the output is oracle/_ref/libaxxref.so,
// used only to pin the oracle and to make tests/golden fixtures.
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <thread>
#include <type_traits>
#include <vector>

#include <cuda_runtime_api.h>

#include "oracle.h"

#ifndef SHIM_NS
#error "define SHIM_NS"
#endif

// ---- stand-ins shared by every variant (defined once, weak) ----------------
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
using std::vector;
#include "misc.cuh"
#include "vector3.cuh"
#include "compare.cuh"
#include "simuParams.cuh"
#include "lattice.cuh"
#include "cylinderXY.cuh"
#include "Sphere.cuh"
#include "plane.cuh"
#include "boundaryCheck.cuh"
#include "gfunctors.cuh"
#include "kernelSetup.cuh"

thread_local long calls0 = 0;  // intersect() calls on basis 0

template <class B>
struct Counted : B {
  int idx = 0;
  bool intersect(const Vector3 &ri, const Vector3 &rf, real &v) const {
    if (idx == 0) ++calls0;
    return B::intersect(ri, rf, v);
  }
};

// Functor standing for any of the reference's gradient functors.
struct AnyG {
  int kind = 0;
  RectGrad rect;
  CosGFunc cosf;
  SinGFunc sinf;
  ApodCosGFunc apod;
  Vector3 operator()(real t) const {
    switch (kind) {
      case 0: return rect(t);
      case 1: return cosf(t);
      case 2: return sinf(t);
      default: return apod(t);
    }
  }
};

struct Hook {
  orc_trace *tr = nullptr;
  int64_t w = 0;
  int steps = 0;
  int i = 0;
  long last_calls = 0;
  bool lattice = true;
  const void *lat = nullptr;
  int (*first_inside)(const void *lat, const void *basis, const Vector3 &r) = nullptr;
  const void *basis = nullptr;
};
thread_local Hook hook;

inline void after_move(Vector3 &r, bool lattice) {
  if (!hook.tr || hook.w >= hook.tr->ntrace) return;
  ++hook.i;
  const size_t o = (size_t)hook.w * (size_t)(hook.steps - 1) + (size_t)(hook.i - 1);
  hook.tr->pos[o * 3 + 0] = r.x;
  hook.tr->pos[o * 3 + 1] = r.y;
  hook.tr->pos[o * 3 + 2] = r.z;
  hook.tr->region[o] = hook.first_inside(hook.lat, hook.basis, r);
  const long d = calls0 - hook.last_calls;
  hook.last_calls = calls0;
  hook.tr->hits[o] = d == 0 ? 0 : (int32_t)(lattice ? d / 2 - 1 : d - 1);
  hook.tr->words[o] = (int32_t)shim_last_word;
}
inline void shim_after_lattice_move(Vector3 &r) { after_move(r, true); }
inline void shim_after_single_move(Vector3 &r) { after_move(r, false); }

#define correctBoundary(v) \
  correctBoundary(v);      \
  shim_after_lattice_move(v)
#define boundaryNormal(a, b, c, d, e) \
  boundaryNormal(a, b, c, d, e);      \
  shim_after_single_move(b)
#include "kernelLattice.cuh"
#include "kernelPhase.cuh"
#undef correctBoundary
#undef boundaryNormal

template <class B>
int first_inside_lattice(const void *latp, const void *basisp, const Vector3 &r) {
  const Lattice *lat = (const Lattice *)latp;
  const Counted<B> *basis = (const Counted<B> *)basisp;
  Vector3 t = r;
  lat->lmod(t);
  for (int i = 0; i < lat->basisSize; ++i)
    if (basis[i].inside(t)) return i;
  return -1;
}

template <class B>
int first_inside_single(const void *, const void *basisp, const Vector3 &r) {
  const Counted<B> *basis = (const Counted<B> *)basisp;
  return basis[0].inside(r) ? 0 : -1;
}

// The reference's Plane (plane.cuh:1-40) has no inside(), which the
// Lattice's region, D and T2 lookups call on every basis, so no lattice walk
// over planes compiles as shipped.  A wall encloses nothing: inside() = false
// completes the class consistently with its getRegion 0, getT2 -1 and
// getD -1; everything else (intersect, getNormal, getPermeability) is the
// reference's own code.
struct PlaneBasis : Plane {
  PlaneBasis() {}
  explicit PlaneBasis(const Plane &p) : Plane(p) {}
  bool inside(const Vector3 &) const { return false; }
};

template <class B>
B make_basis(const orc_basis &q);
template <>
PlaneBasis make_basis<PlaneBasis>(const orc_basis &q) {
  return PlaneBasis(Plane(Vector3(q.cx, q.cy, q.cz), Vector3(q.nx, q.ny, q.nz)));
}
template <>
Cylinder_XY make_basis<Cylinder_XY>(const orc_basis &q) {
  Cylinder_XY c(q.cx, q.cy, q.radius, q.T2, q.T1, q.D, q.region, q.permeability, q.eps);
  c.permeability = q.permeability;  // the constructors leave it unset (cylinderXY.cuh:16-40)
  return c;
}
template <>
Sphere make_basis<Sphere>(const orc_basis &q) {
  return Sphere(q.cx, q.cy, q.cz, q.radius, q.T2, q.T1, q.D, q.region, q.permeability, q.eps);
}

AnyG make_g(const orc_sequence &s) {
  AnyG g;
  g.kind = s.kind;
  Vector3 gh(s.gx, s.gy, s.gz);
  switch (s.kind) {
    case 0:
      g.rect = RectGrad(s.G, s.duration, s.spacing);
      g.rect.g_hat = gh;
      break;
    case 1: g.cosf = CosGFunc(s.G, s.duration, s.spacing, s.num_periods, gh); break;
    case 2: g.sinf = SinGFunc(s.G, s.duration, s.spacing, s.num_periods, gh); break;
    default: g.apod = ApodCosGFunc(s.G, s.duration, s.spacing, s.num_periods, gh); break;
  }
  return g;
}

template <class B>
int run(const orc_lattice *latp, const orc_basis *bases, int nbasis, const orc_sequence *seqs,
        int nseq, const orc_params *p, int nthreads, double *sums, orc_trace *tr) {
  const bool single = latp == nullptr;
  const int N = (int)p->num_walkers;
  std::vector<Counted<B>> basis(std::max(nbasis, 1));
  for (int k = 0; k < nbasis; ++k) {
    static_cast<B &>(basis[k]) = make_basis<B>(bases[k]);
    basis[k].idx = k;
  }
  Lattice lat;
  if (!single) lat = Lattice(latp->a, latp->b, latp->c, latp->T2, latp->T1, latp->D, nbasis);
  std::vector<AnyG> G(std::max(nseq, 1));
  for (int j = 0; j < nseq; ++j) G[j] = make_g(seqs[j]);
  SimuParamsPhase par(N, p->steps, nseq, p->timestep, (int)p->seed, 0.0);
  std::vector<curandState> states(N);
  std::vector<real> phase((size_t)std::max(nseq, 1) * N, 0.0), t2((size_t)N, 0.0);
  if (nthreads < 1) nthreads = 1;
  auto work = [&](int t) {
    blockIdx.x = 0;
    blockDim.x = 1;
    for (int w = (int)((int64_t)N * t / nthreads); w < (int)((int64_t)N * (t + 1) / nthreads); ++w) {
      threadIdx.x = (unsigned)w;
      setup_kernel(states.data(), &par);
      hook = Hook();
      if (tr && w < tr->ntrace) {
        hook.tr = tr;
        hook.w = w;
        hook.steps = p->steps;
        hook.lattice = !single;
        hook.lat = &lat;
        hook.basis = basis.data();
        hook.first_inside = single ? first_inside_single<B> : first_inside_lattice<B>;
        hook.last_calls = calls0;
        curandState tmp = states[w];
        Vector3 r0;
        if constexpr (!std::is_same<B, PlaneBasis>::value) {
          if (single) r0 = basis[0].unifRand(tmp);
          else lat.initializeUniformly(r0, tmp);
        } else {
          lat.initializeUniformly(r0, tmp);
        }
        tr->init_pos[w * 3 + 0] = r0.x;
        tr->init_pos[w * 3 + 1] = r0.y;
        tr->init_pos[w * 3 + 2] = r0.z;
      }
      if constexpr (!std::is_same<B, PlaneBasis>::value) {
        if (single)
          updateWalkersPhase<AnyG, Counted<B>>(&par, basis.data(), G.data(), states.data(),
                                               phase.data());
        else
          updateWalkersLatticePhase<AnyG, Counted<B>>(&par, &lat, basis.data(), G.data(),
                                                      states.data(), t2.data(), phase.data());
      } else {
        updateWalkersLatticePhase<AnyG, Counted<B>>(&par, &lat, basis.data(), G.data(), states.data(),
                                                    t2.data(), phase.data());
      }
      hook = Hook();
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
  for (auto &x : th) x.join();
  // transformAndSum(TwoVectors) (cudaVector.cu:143-172) in walker order
  for (int j = 0; j < nseq; ++j) {
    double s[5] = {0, 0, 0, 0, 0};
    for (int w = 0; w < N; ++w) {
      const double ph = phase[(size_t)w + (size_t)j * N];
#if defined USE_RELAXATION
      const double xv = single ? cos(ph) : COS_EXP_BINARY<real>()(ph, t2[w]);
      const double yv = single ? sin(ph) : SIN_EXP_BINARY<real>()(ph, t2[w]);
#else
      const double xv = COS_UNARY<real>()(ph), yv = SIN_UNARY<real>()(ph);
#endif
      s[0] += xv;
      s[1] += yv;
      s[2] += xv * xv;
      s[3] += yv * yv;
      s[4] += xv * yv;
    }
    for (int k = 0; k < 5; ++k) sums[j * 5 + k] = s[k];
  }
  return 0;
}

}  // namespace SHIM_NS

#define SHIM_CAT2(a, b) a##b
#define SHIM_CAT(a, b) SHIM_CAT2(a, b)

extern "C" int SHIM_CAT(ref_walk_, SHIM_NS)(const orc_lattice *lat, const orc_basis *basis,
                                            int nbasis, const orc_sequence *seqs, int nseq,
                                            const orc_params *p, int nthreads, double *sums,
                                            orc_trace *trace) {
  if (!p || p->num_walkers < 1 || p->steps < 1) return -1;
  if (lat == nullptr && nbasis < 1) return -1;
  for (int j = 0; j < nseq; ++j)
    if (seqs[j].kind == 4) return -2;  // SWOGSEFunc::ampMod is NaN (gfunctors.cuh:281-283)
  int type = nbasis > 0 ? basis[0].type : 0;
  for (int k = 0; k < nbasis; ++k)
    if (basis[k].type != type) return -3;  // one Basis type per lattice in the reference
  if (type == 2) {
    if (lat == nullptr) return -1;  // a plane is no pore
    return SHIM_NS::run<SHIM_NS::PlaneBasis>(lat, basis, nbasis, seqs, nseq, p, nthreads, sums,
                                             trace);
  }
  if (type == 1)
    return SHIM_NS::run<SHIM_NS::Sphere>(lat, basis, nbasis, seqs, nseq, p, nthreads, sums, trace);
  return SHIM_NS::run<SHIM_NS::Cylinder_XY>(lat, basis, nbasis, seqs, nseq, p, nthreads, sums,
                                            trace);
}
