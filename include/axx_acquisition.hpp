/*
 * axx_acquisition.hpp -- header-only C++ adapter with axonexa's acquisition
 * API over the C ABI of axx.h.
 *
 * A program written against the reference's classes switches to the GB300
 * walker by replacing the reference's includes with this header and adding
 * `using namespace axonexa;`: the class names, constructors and the
 * simulate-and-read-signal calls are the reference's
 *
 *   phaseAcquisition<F>   (src/acquisition/phaseAcquisition.cuh:1-86):
 *       phaseAcquisition(numOfMeas, numOfSteps, numOfParticles, seed),
 *       addMeasurement, getGradientFunctors, getMx, getMy, getSignal,
 *       getNumOfMeas, getNumOfSteps, getSeed, calcADC, getADC,
 *       getADCMeanSquare, getPoints, getADCError;
 *   phaseAcquisitionStream<F>
 *       (src/acquisition/phaseAcquisitionStream.cuh:3-640):
 *       phaseAcquisitionStream(numOfParticles), addAcquisition,
 *       getAcquisition, runAcquisition (:37-39) -> axx_run_single,
 *       runAcquisitionLattice (:126-129) -> axx_run_lattice,
 *       runAcquisitionStream / runAcquisitionStreamLattice (:254-258,
 *       :425-429) -> one call per acquisition, changeSeeds, calcEveryADC,
 *       flushADC;
 *   Lattice (src/substrate/lattice.cuh:3-23), Cylinder_XY
 *   (src/primitives/cylinderXY.cuh:16-40), Sphere (Sphere.cuh:19-44), Plane
 *   (plane.cuh:9-14), Vector3 (src/util/vector3.cuh);
 *   RectGrad, CosGFunc, SinGFunc, ApodCosGFunc, SWOGSEFunc
 *   (src/functors/gfunctors.cuh) with getB / operator()(t) served by
 *   axx_bvalue / axx_gradient_eval;
 *   linear_regression (src/util/misc.cuh:41-59).
 *
 * The reference's compile-time switches are read where this header is
 * included, as the reference reads them: SPECULAR_REFLECTION (else simple
 * rejection), USE_RELAXATION, USE_PERMEABLE, USE_INITIALIZE_IN_REGION and
 * GAMMA (default 267500 rad/(ms T)).  The launch arguments (blocks, threads,
 * numOfSM, numOfDevices, plan) are accepted and ignored: the library sizes
 * its own grid and takes any number of particles.  Errors throw
 * std::runtime_error with the library's message (the reference asserts).
 * Each host thread drives device 0 through its own context unless
 * setDevice() picks another.
 */
#ifndef AXX_ACQUISITION_HPP_
#define AXX_ACQUISITION_HPP_

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "axx.h"

namespace axonexa {

typedef double real;

struct Vector3 {
  real x, y, z;
  Vector3() : x(0), y(0), z(0) {}
  Vector3(real x_, real y_, real z_) : x(x_), y(y_), z(z_) {}
  Vector3 operator+(const Vector3 &o) const { return Vector3(x + o.x, y + o.y, z + o.z); }
  Vector3 operator-(const Vector3 &o) const { return Vector3(x - o.x, y - o.y, z - o.z); }
  Vector3 operator*(real s) const { return Vector3(x * s, y * s, z * s); }
  real operator*(const Vector3 &o) const { return x * o.x + y * o.y + z * o.z; }
  real magnitude() const { return std::sqrt(x * x + y * y + z * z); }
};

namespace detail {

struct ThreadContext {
  axx_ctx *ctx = nullptr;
  int device = 0;
  ~ThreadContext() {
    if (ctx) axx_destroy(ctx);
  }
};

inline ThreadContext &thread_context() {
  static thread_local ThreadContext t;
  return t;
}

inline axx_ctx *context() {
  ThreadContext &t = thread_context();
  if (!t.ctx) {
    const axx_status s = axx_create(&t.ctx, t.device);
    if (s != AXX_OK) {
      t.ctx = nullptr;
      throw std::runtime_error(std::string("axx_create: ") + axx_status_string(s));
    }
  }
  return t.ctx;
}

inline void check(axx_status s, axx_ctx *ctx, const char *what) {
  if (s == AXX_OK) return;
  std::string msg = std::string(what) + ": " + axx_status_string(s);
  const char *e = ctx ? axx_last_error(ctx) : nullptr;
  if (e && *e) msg += std::string(" (") + e + ")";
  throw std::runtime_error(msg);
}

// gamma of the including program (its GAMMA macro), else the library default
inline double gamma_value() {
#ifdef GAMMA
  return (double)(GAMMA);
#else
  return 267500.0;
#endif
}

// the reference's compile-time switches as run flags
inline uint32_t run_flags() {
  uint32_t f = 0;
#ifndef SPECULAR_REFLECTION
  f |= AXX_FLAG_SIMPLE_REJECTION;
#endif
#ifdef USE_RELAXATION
  f |= AXX_FLAG_RELAXATION;
#endif
#ifdef USE_PERMEABLE
  f |= AXX_FLAG_PERMEABLE;
#endif
  return f;
}

inline void init_mode(int32_t &mode, int32_t &arg) {
#if defined USE_INITIALIZE_IN_REGION
#if USE_INITIALIZE_IN_REGION == 0
  mode = AXX_INIT_IN_REGION;
  arg = 0;
#else
  mode = AXX_INIT_IN_BASIS;
  arg = (USE_INITIALIZE_IN_REGION)-1;
#endif
#else
  mode = AXX_INIT_UNIFORM;
  arg = 0;
#endif
}

inline axx_sequence sequence(int32_t kind, int32_t periods, real G, real duration,
                             real spacing, const Vector3 &g) {
  axx_sequence q;
  q.kind = kind;
  q.num_periods = periods;
  q.G = G;
  q.duration = duration;
  q.spacing = spacing;
  q.gx = g.x;
  q.gy = g.y;
  q.gz = g.z;
  return q;
}

inline real bvalue(const axx_sequence &q) {
  double b = 0.0;
  check(axx_bvalue(&q, gamma_value(), &b), nullptr, "axx_bvalue");
  return b;
}

inline Vector3 gradient(const axx_sequence &q, real t) {
  double out[3] = {0.0, 0.0, 0.0};
  check(axx_gradient_eval(&q, &t, 1, out), nullptr, "axx_gradient_eval");
  return Vector3(out[0], out[1], out[2]);
}

inline axx_basis basis(int32_t type, int32_t region, real cx, real cy, real cz, real R, real D,
                       real T2, real T1, real kappa, real eps) {
  axx_basis b;
  b.type = type;
  b.region = region;
  b.cx = cx;
  b.cy = cy;
  b.cz = cz;
  b.radius = R;
  b.D = D;
  b.T2 = T2;
  b.T1 = T1;
  b.permeability = kappa;
  b.eps = eps;
  b.nx = b.ny = b.nz = 0.0;
  return b;
}

}  // namespace detail

// Selects the GPU the calling thread's acquisitions run on (default 0).
inline void setDevice(int device) {
  detail::ThreadContext &t = detail::thread_context();
  if (t.ctx && t.device != device) {
    axx_destroy(t.ctx);
    t.ctx = nullptr;
  }
  t.device = device;
}

// ---- substrate ------------------------------------------------------------

class Lattice {
 public:
  Lattice() : a_(0), b_(0), c_(0), T2_(0), T1_(0), D_(0), basisSize_(0) {}
  Lattice(real a, real b, real c, real T2, real T1, real D, int basisSize = 0)
      : a_(a), b_(b), c_(c), T2_(T2), T1_(T1), D_(D), basisSize_(basisSize) {}
  real getA() const { return a_; }
  real getB() const { return b_; }
  real getC() const { return c_; }
  int getBasisSize() const { return basisSize_; }
  axx_lattice record() const {
    axx_lattice l;
    l.a = a_;
    l.b = b_;
    l.c = c_;
    l.T2 = T2_;
    l.T1 = T1_;
    l.D = D_;
    return l;
  }

 private:
  real a_, b_, c_, T2_, T1_, D_;
  int basisSize_;
};

class Cylinder_XY {
 public:
  Cylinder_XY() : cx_(0), cy_(0), R_(0), T2_(0), T1_(0), D_(0), region_(0), kappa_(0), eps_(1e-14) {}
  Cylinder_XY(real centerX, real centerY, real radius, real T2, real T1, real D, int region,
              real permeability, real eps = 1e-14)
      : cx_(centerX), cy_(centerY), R_(radius), T2_(T2), T1_(T1), D_(D), region_(region),
        kappa_(permeability), eps_(eps) {}
  bool inside(const Vector3 &r) const {
    return (r.x - cx_) * (r.x - cx_) + (r.y - cy_) * (r.y - cy_) < R_ * R_;
  }
  real getRadius() const { return R_; }
  real getT2() const { return T2_; }
  real getT1() const { return T1_; }
  real getD() const { return D_; }
  real getPermeability() const { return kappa_; }
  int getRegion() const { return region_; }
  Vector3 getCenter() const { return Vector3(cx_, cy_, 0.0); }
  void setCenter(Vector3 v) {
    cx_ = v.x;
    cy_ = v.y;
  }
  void setRadius(real r) { R_ = r; }
  void setEPS(real e) { eps_ = e; }
  void setRegion(int r) { region_ = r; }
  axx_basis record() const {
    return detail::basis(AXX_PRIM_CYLINDER_Z, region_, cx_, cy_, 0.0, R_, D_, T2_, T1_, kappa_,
                         eps_);
  }

 private:
  real cx_, cy_, R_, T2_, T1_, D_;
  int region_;
  real kappa_, eps_;
};

class Sphere {
 public:
  Sphere() : cx_(0), cy_(0), cz_(0), R_(0), T2_(0), T1_(0), D_(0), region_(0), kappa_(0), eps_(1e-14) {}
  Sphere(real centerX, real centerY, real centerZ, real radius, real T2, real T1, real D,
         int region, real permeability, real eps = 1e-14)
      : cx_(centerX), cy_(centerY), cz_(centerZ), R_(radius), T2_(T2), T1_(T1), D_(D),
        region_(region), kappa_(permeability), eps_(eps) {}
  bool inside(const Vector3 &r) const {
    const Vector3 p = r - getCenter();
    return p * p < R_ * R_;
  }
  real getRadius() const { return R_; }
  real getT2() const { return T2_; }
  real getT1() const { return T1_; }
  real getD() const { return D_; }
  real getPermeability() const { return kappa_; }
  int getRegion() const { return region_; }
  Vector3 getCenter() const { return Vector3(cx_, cy_, cz_); }
  void setRadius(real r) { R_ = r; }
  void setRegion(int r) { region_ = r; }
  axx_basis record() const {
    return detail::basis(AXX_PRIM_SPHERE, region_, cx_, cy_, cz_, R_, D_, T2_, T1_, kappa_,
                         eps_);
  }

 private:
  real cx_, cy_, cz_, R_, T2_, T1_, D_;
  int region_;
  real kappa_, eps_;
};

// An impermeable wall through `center` with normal `normal` (lattices only).
class Plane {
 public:
  Plane() {}
  Plane(Vector3 center, Vector3 normal) : c_(center), n_(normal) {}
  Vector3 getNormal() const { return n_; }
  axx_basis record() const {
    axx_basis b = detail::basis(AXX_PRIM_PLANE, 0, c_.x, c_.y, c_.z, 0.0, 0.0, 0.0, 0.0, 0.0,
                                1e-14);
    b.nx = n_.x;
    b.ny = n_.y;
    b.nz = n_.z;
    return b;
  }

 private:
  Vector3 c_, n_;
};

// ---- gradient functors -----------------------------------------------------

class GradientFunctor {
 public:
  Vector3 operator()(real time) const { return detail::gradient(q_, time); }
  real getB() const { return detail::bvalue(q_); }
  real getG() const { return q_.G; }
  const axx_sequence &record() const { return q_; }

 protected:
  GradientFunctor() { q_ = detail::sequence(AXX_SEQ_PGSE, 0, 0.0, 1.0, 0.0, Vector3(1, 0, 0)); }
  axx_sequence q_;
};

class RectGrad : public GradientFunctor {
 public:
  RectGrad() {}
  // gradient strength, duration, spacing; along x
  RectGrad(real gstr, real gd, real gspac) {
    q_ = detail::sequence(AXX_SEQ_PGSE, 0, gstr, gd, gspac, Vector3(1.0, 0.0, 0.0));
  }
  // b-value, duration, spacing, direction: the strength solved from b
  RectGrad(real b, real gd, real gspac, const Vector3 &ghat) {
    const double g = detail::gamma_value();
    const real gstr = std::sqrt(b / (gd * gd * g * g * ((2.0 / 3.0) * gd + gspac)));
    q_ = detail::sequence(AXX_SEQ_PGSE, 0, gstr, gd, gspac, ghat);
    b_ = b;
    has_b_ = true;
  }
  real getB() const { return has_b_ ? b_ : GradientFunctor::getB(); }
  real getDiffusionTime() const { return q_.spacing + q_.duration; }
  real getTau() const { return q_.duration + q_.spacing * .5; }

 private:
  real b_ = 0.0;
  bool has_b_ = false;
};

class OscillatingGradient : public GradientFunctor {
 public:
  real getFreq() const {
    return q_.kind == AXX_SEQ_SQUARE ? (real)q_.num_periods / q_.duration
                                     : 1.0 / (q_.duration / (real)q_.num_periods);
  }

 protected:
  OscillatingGradient() {}
  OscillatingGradient(int32_t kind, real G, real gd, real gs, int N, const Vector3 &ghat) {
    q_ = detail::sequence(kind, N, G, gd, gs, ghat);
  }
};

class CosGFunc : public OscillatingGradient {
 public:
  CosGFunc() {}
  CosGFunc(real G, real gradientDuration, real gradientSpacing, int numOfPeriods,
           const Vector3 &gHat)
      : OscillatingGradient(AXX_SEQ_COS, G, gradientDuration, gradientSpacing, numOfPeriods,
                            gHat) {}
};

class SinGFunc : public OscillatingGradient {
 public:
  SinGFunc() {}
  SinGFunc(real G, real gradientDuration, real gradientSpacing, int numOfPeriods,
           const Vector3 &gHat)
      : OscillatingGradient(AXX_SEQ_SIN, G, gradientDuration, gradientSpacing, numOfPeriods,
                            gHat) {}
};

class ApodCosGFunc : public OscillatingGradient {
 public:
  ApodCosGFunc() {}
  ApodCosGFunc(real G, real gradientDuration, real gradientSpacing, int numOfPeriods,
               const Vector3 &gHat)
      : OscillatingGradient(AXX_SEQ_APODCOS, G, gradientDuration, gradientSpacing,
                            numOfPeriods, gHat) {}
};

// Square-wave OGSE with sign (-1)^floor(2 t nu): the reference's
// pow(-1., 2 t nu) is NaN for non-integer exponents (gfunctors.cuh:281-283).
class SWOGSEFunc : public OscillatingGradient {
 public:
  SWOGSEFunc() {}
  SWOGSEFunc(real G, real gradientDuration, real gradientSpacing, int numOfPeriods,
             const Vector3 &gHat)
      : OscillatingGradient(AXX_SEQ_SQUARE, G, gradientDuration, gradientSpacing,
                            numOfPeriods, gHat) {}
};

// ---- acquisitions ------------------------------------------------------------

// Least-squares slope of y against x (src/util/misc.cuh:41-59), the same
// sums in the same order.
inline double linear_regression(std::vector<real> y, std::vector<real> x) {
  if (y.size() != x.size()) throw std::runtime_error("linear_regression: y.size != x.size");
  double term1 = (double)y.size(), term2 = 0.0, term3 = 0.0, term4 = 0.0, term5 = 0.0;
  for (size_t i = 0; i < y.size(); i++) {
    term2 = term2 + (x[i] * y[i]);
    term3 = term3 + (x[i]);
    term4 = term4 + (y[i]);
    term5 = term5 + (x[i] * x[i]);
  }
  const double delta = term1 * term5 - term3 * term3;
  return (1 / delta) * (term1 * term2 - term3 * term4);
}

template <class FieldType>
class phaseAcquisition {
 public:
  phaseAcquisition(int numOfMeas, int numOfSteps, int numOfParticles, int seed)
      : numOfMeasurements_(numOfMeas), numOfSteps_(numOfSteps), lastAllocMeasurement_(0),
        seed_(seed), mx_(numOfMeas, 0.0), my_(numOfMeas, 0.0), gradientFunctors_(numOfMeas),
        T2factor_(numOfParticles, 1.0), ADC_(0.0), ADCmeansquare_(0.0), points_(0) {}
  phaseAcquisition()
      : numOfMeasurements_(0), numOfSteps_(0), lastAllocMeasurement_(0), seed_(0), ADC_(0.0),
        ADCmeansquare_(0.0), points_(0) {}

  void addMeasurement(const FieldType &field) {
    if (lastAllocMeasurement_ >= numOfMeasurements_)
      throw std::runtime_error("addMeasurement: more measurements than numOfMeas");
    gradientFunctors_[lastAllocMeasurement_++] = field;
  }
  std::vector<FieldType> &getGradientFunctors() { return gradientFunctors_; }
  std::vector<real> &getMx() { return mx_; }
  std::vector<real> &getMy() { return my_; }
  real getSignal(int i) { return std::sqrt(mx_[i] * mx_[i] + my_[i] * my_[i]); }
  int getNumOfMeas() { return numOfMeasurements_; }
  int getNumOfSteps() { return numOfSteps_; }
  int &getSeed() { return seed_; }

  // ln S against b over the measurements; the slope's negative is one ADC
  // point, averaged with the previous points (phaseAcquisition.cuh:54-77)
  void calcADC() {
    points_++;
    std::vector<real> lnsignal, bvalues;
    for (int i = 0; i < numOfMeasurements_; i++) {
      bvalues.push_back(gradientFunctors_[i].getB());
      lnsignal.push_back(std::log(std::sqrt(mx_[i] * mx_[i] + my_[i] * my_[i])));
    }
    if (points_ == 1) {
      ADC_ = -1.0 * linear_regression(lnsignal, bvalues);
      ADCmeansquare_ = ADC_ * ADC_;
    } else {
      const real t = -1.0 * linear_regression(lnsignal, bvalues);
      ADC_ = (ADC_ * (points_ - 1) + t) / (points_);
      ADCmeansquare_ = (ADCmeansquare_ * (points_ - 1) + t * t) / (points_);
    }
  }
  real &getADC() { return ADC_; }
  real &getADCMeanSquare() { return ADCmeansquare_; }
  int &getPoints() { return points_; }
  real getADCError() { return std::sqrt(ADCmeansquare_ - ADC_ * ADC_); }

  // the measurements as C-ABI records
  std::vector<axx_sequence> records() const {
    std::vector<axx_sequence> s;
    for (int i = 0; i < numOfMeasurements_; i++) s.push_back(gradientFunctors_[i].record());
    return s;
  }

 private:
  int numOfMeasurements_, numOfSteps_, lastAllocMeasurement_, seed_;
  std::vector<real> mx_, my_;
  std::vector<FieldType> gradientFunctors_;
  std::vector<real> T2factor_;
  real ADC_, ADCmeansquare_;
  int points_;
};

template <class FieldType>
class phaseAcquisitionStream {
 public:
  std::vector<phaseAcquisition<FieldType> > acqSet;

  explicit phaseAcquisitionStream(int num) : number_of_particles_(num), steps_max_(-1), meas_max_(-1) {}
  phaseAcquisitionStream() : number_of_particles_(0), steps_max_(-1), meas_max_(-1) {}

  void addAcquisition(phaseAcquisition<FieldType> acq) {
    acqSet.push_back(acq);
    if (acq.getNumOfSteps() > steps_max_) steps_max_ = acq.getNumOfSteps();
    if (acq.getNumOfMeas() > meas_max_) meas_max_ = acq.getNumOfMeas();
  }
  phaseAcquisition<FieldType> &getAcquisition(int num) { return acqSet[num]; }

  // One acquisition on a single pore (axx_run_single).
  template <class Basis>
  void runAcquisition(int num, Basis &basis, real timestep, int blocks = 0, int threads = 0,
                      int numOfSM = 0) {
    (void)blocks, (void)threads, (void)numOfSM;
    phaseAcquisition<FieldType> &a = acqSet[num];
    const std::vector<axx_sequence> S = a.records();
    const axx_basis B = basis.record();
    axx_run_params p = params(a, timestep);
    p.flags &= AXX_FLAG_SIMPLE_REJECTION;  // the single-pore walk has no T2 or kappa
    p.init_mode = AXX_INIT_UNIFORM;
    p.init_arg = 0;
    std::vector<double> mx(S.size()), my(S.size());
    axx_ctx *ctx = detail::context();
    detail::check(axx_run_single(ctx, &B, S.data(), (int)S.size(), &p, mx.data(), my.data(),
                                 nullptr),
                  ctx, "runAcquisition");
    a.getMx().assign(mx.begin(), mx.end());
    a.getMy().assign(my.begin(), my.end());
  }

  // One acquisition on a periodic lattice of lat.getBasisSize() bases
  // (axx_run_lattice).
  template <class Basis>
  void runAcquisitionLattice(int num, Basis *basis, Lattice &lat, real timestep, int blocks = 0,
                             int threads = 0, int numOfSM = 0) {
    (void)blocks, (void)threads, (void)numOfSM;
    phaseAcquisition<FieldType> &a = acqSet[num];
    const std::vector<axx_sequence> S = a.records();
    std::vector<axx_basis> B;
    for (int i = 0; i < lat.getBasisSize(); i++) B.push_back(basis[i].record());
    const axx_lattice L = lat.record();
    const axx_run_params p = params(a, timestep);
    std::vector<double> mx(S.size()), my(S.size());
    axx_ctx *ctx = detail::context();
    detail::check(axx_run_lattice(ctx, &L, B.empty() ? nullptr : B.data(), (int)B.size(),
                                  S.data(), (int)S.size(), &p, mx.data(), my.data(), nullptr),
                  ctx, "runAcquisitionLattice");
    a.getMx().assign(mx.begin(), mx.end());
    a.getMy().assign(my.begin(), my.end());
  }

  // Every acquisition of the set (the reference spreads them over devices
  // and streams; here they run one after another on the thread's device).
  template <class Basis>
  void runAcquisitionStream(Basis &basis, real timestep, int blocks, int threads,
                            int numOfDevices, std::vector<int> &plan,
                            std::vector<int> &numOfSMPerDevice) {
    (void)numOfDevices, (void)plan, (void)numOfSMPerDevice;
    for (int i = 0; i < (int)acqSet.size(); i++) runAcquisition(i, basis, timestep, blocks, threads, 0);
  }

  template <class Basis>
  void runAcquisitionStreamLattice(Basis *basis, Lattice &lat, real timestep, int blocks,
                                   int threads, int numOfDevices, std::vector<int> &plan,
                                   std::vector<int> &numOfSMPerDevice) {
    (void)numOfDevices, (void)plan, (void)numOfSMPerDevice;
    for (int i = 0; i < (int)acqSet.size(); i++)
      runAcquisitionLattice(i, basis, lat, timestep, blocks, threads, 0);
  }

  void changeSeeds(long int seed) {
    for (size_t i = 0; i < acqSet.size(); i++) acqSet[i].getSeed() = (int)(seed * (long)(i + 1));
  }
  void calcEveryADC() {
    for (size_t i = 0; i < acqSet.size(); i++) acqSet[i].calcADC();
  }
  void flushADC() {
    for (size_t i = 0; i < acqSet.size(); i++) {
      acqSet[i].getADC() = 0.0;
      acqSet[i].getADCMeanSquare() = 0.0;
      acqSet[i].getPoints() = 0;
    }
  }

 private:
  axx_run_params params(phaseAcquisition<FieldType> &a, real timestep) const {
    axx_run_params p;
    p.num_walkers = number_of_particles_;
    p.steps = a.getNumOfSteps();
    detail::init_mode(p.init_mode, p.init_arg);
    p.flags = detail::run_flags();
    p.seed = (uint64_t)a.getSeed();  // as curand_init receives the int seed
    p.timestep = timestep;
    p.gamma = detail::gamma_value();
    p.walker_offset = 0;
    return p;
  }

  int number_of_particles_, steps_max_, meas_max_;
};

}  // namespace axonexa

#endif  // AXX_ACQUISITION_HPP_
