/*
 * oracle.h -- CPU oracle of the axonexa random-walker phase path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it is linked or
 * loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
 * arm, and never by the product library (axonexa_gb300/libaxx.so).
 *
 * It restates the reference's walk in plain C++ (see oracle.cpp for the
 * file:line each function follows) in three modes:
 *   ORC_REF64    the reference's own algorithm and operation order in FP64:
 *                Lattice with two wrapped copies of every move, the expanded
 *                quadratic of Cylinder_XY/Sphere::intersect, acos-based step
 *                directions; pinned bit-for-bit against the reference's own
 *                headers compiled for the host (oracle/_ref) and the golden
 *                vectors in tests/golden/.
 *   ORC_KERN64   the GPU kernel's formulation (periodic ghost instances,
 *                centre-relative quadratic in the distance parameter, the
 *                polynomial direction) in FP64.
 *   ORC_KERN32   the same in FP32 with the kernel's exact operation sequence:
 *                a trajectory of the GPU kernel is reproduced bit for bit.
 * In every mode the phases are accumulated per sequence in FP64 exactly as
 * updateWalkersLatticePhase does (phase += GAMMA*(G(t).r_unbounded)*dt), and
 * the signal sums are FP64.
 *
 * The record layouts are the same plain structs as the product's C ABI, so a
 * test can hand the same bytes to both.
 */
#ifndef AXX_ORACLE_H_
#define AXX_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int32_t type, region;  /* type 0 cylinder along z, 1 sphere, 2 plane */
  double cx, cy, cz, radius, D, T2, T1, permeability, eps;
  double nx, ny, nz;     /* plane normal */
} orc_basis;

typedef struct {
  double a, b, c, T2, T1, D;
} orc_lattice;

typedef struct {
  int32_t kind, num_periods;
  double G, duration, spacing, gx, gy, gz;
} orc_sequence;

typedef struct {
  int64_t num_walkers;
  int32_t steps, init_mode, init_arg;
  uint32_t flags;
  uint64_t seed;
  double timestep, gamma;
  int64_t walker_offset;
} orc_params;

/* Trace of the first ntrace walkers: start position, then after every move
 * i = 1..steps-1 the wrapped position, the first containing basis (-1 if
 * none), the boundary hits of the move and the index of the next stream word. */
typedef struct {
  int32_t ntrace;
  double *init_pos;  /* [ntrace*3] */
  double *pos;       /* [ntrace*(steps-1)*3] */
  int32_t *region;   /* [ntrace*(steps-1)] */
  int32_t *hits;
  int32_t *words;
} orc_trace;

enum { ORC_REF64 = 0, ORC_KERN64 = 1, ORC_KERN32 = 2 };

/* Philox4x32-10 of one counter/key. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Words 0..n-1 of the stream of (seed, walker). */
void orc_stream_words(uint64_t seed, uint64_t walker, int n, uint32_t *out);
/* sin and cos of 2*pi*u by the kernel's FP32 polynomial (for host checks). */
void orc_sincos_2pi_f32(float u, float *s, float *c);

/* A closed triangle mesh as a single pore (GPU walker formulation, see
 * oracle.cpp): vertices[nvert][3], triangles[ntri][3]; mode ORC_KERN64 or
 * ORC_KERN32; sums as orc_walk; escaped = walkers outside the mesh after
 * their walk. */
int orc_mesh_walk(const double *vertices, int nvert, const int32_t *triangles, int ntri, double D,
                  const orc_sequence *seqs, int nseq, const orc_params *p, int mode, int nthreads,
                  double *sums, orc_trace *trace, int64_t *escaped);

/* Signal sums of a lattice walk (lat != NULL) or a single-pore walk
 * (lat == NULL, walkers start in basis[0]).  sums[5*j..5*j+4] =
 * (sum x, sum y, sum x^2, sum y^2, sum xy) for sequence j.  With flag 64
 * (compartment sums) on a lattice, rows nseq..2*nseq-1 hold the same sums
 * over the walkers that start inside a basis (sums has 10*nseq entries).
 * Walkers are split over nthreads host threads (partial sums combined in
 * thread order).
 * Returns 0, or a negative code for invalid input. */
int orc_walk(const orc_lattice *lat, const orc_basis *basis, int nbasis,
             const orc_sequence *seqs, int nseq, const orc_params *p, int mode, int nthreads,
             double *sums, orc_trace *trace, int64_t *cap_hits);

/* One move i of walker `walker` from the wrapped position r_in with the
 * stream positioned at word `word`: writes the wrapped end position, the
 * first containing basis there, the hits and the next word index. */
int orc_step(const orc_lattice *lat, const orc_basis *basis, int nbasis, const orc_params *p,
             int mode, int64_t walker, int i, const double r_in[3], int32_t word,
             double r_out[3], int32_t *region, int32_t *hits, int32_t *word_out);

/* b-value and gradient of a sequence, restating the reference functors. */
double orc_bvalue(const orc_sequence *q, double gamma);
void orc_gradient(const orc_sequence *q, double t, double out[3]);

/* Monte Carlo intracellular volume fraction (the algorithm of calcf /
 * kernelCalcf, src/util/calcf.cuh:1-38): point i draws words 1..3 of stream
 * (seed, i) as Lattice::initializeUniformly does and counts when the first
 * basis containing it has region > 0.  REF64: FP64 positions and the
 * reference lookup over the listed bases; KERN32: the kernel's FP32
 * positions and instance lookup.  *inside = the count. */
int orc_volume_fraction(const orc_lattice *lat, const orc_basis *basis, int nbasis,
                        int64_t points, uint64_t seed, int mode, int nthreads, int64_t *inside);

/* kernelWC (src/kernels/kernelWC.cuh:13-89) restated in FP64 (the reference
 * example builds it with real = double): per walker the xorshift uniforms,
 * Box-Muller displacements, rejection at the pore wall and the Kahan phase;
 * phase[n] (required) and sums of cosf/sinf of each phase (the reduction
 * evaluates cosf/sinf of the phase narrowed to float). */
int orc_wc(const orc_basis *pore, int64_t n, int steps, double timestep, double gamma,
           const uint32_t *rng_state, const double *start, const double *grad, double *phase,
           double *sum_cos, double *sum_sin);

/* ---- magnetisation (Bloch) path ------------------------------------------
 * The records have the layout of the product's axx_field / axx_mag_params.
 * Field kinds: 0 QSC_GRE, 1 QSC_PGSE, 2 QSC_COS_GRE, 3 QSC_GRE_TRAP,
 * 4 SIN_GRE, 5 COS_GRE, 6 RECT_GRE, 7 UCN_lowfield (src/functors/bfunctors.cuh).
 * Integrators: 0 rotation (the reference's default), 1 RK4 (RK4_NORELAXATION),
 * 2 multi-step rotation (ROTATE_MULTISTEP), 3 adaptive Dormand-Prince 5(4)
 * on a dyadic grid of sub-steps (the integrator DORP_NORELAXATION aims at;
 * no reference build exists: see mag_dorp in oracle.cpp). */
typedef struct {
  int32_t kind, num_periods;
  double B0, G, gx, gy, gz, duration, spacing, period, ramp, rf_duration, dtmin, dtmax, TE;
} orc_field;

typedef struct {
  int64_t num_walkers;
  int32_t steps, integrator;
  uint32_t flags; /* 4: simple rejection instead of specular reflection */
  uint32_t dorp_levels; /* integrator 3: halvings of the step allowed (0: 3) */
  uint64_t seed;
  double timestep, gamma, m0[3];
  int64_t walker_offset;
  double dorp_tol; /* integrator 3: error tolerance (0: 1e-6) */
} orc_mag_params;

/* B(r, t) of one field functor (FP64, the reference's expressions). */
void orc_bfield(const orc_field *f, double gamma, const double r[3], double t, double out[3]);

/* Magnetisation of one walker along a given trajectory: pos[0] is the start,
 * pos[i] the position after move i (i = 1..steps-1); m_out[3*j..] for field j.
 * The integrator and time points are updateWalkersMag's (kernelMag.cuh). */
void orc_mag_along(const orc_field *f, int nf, const orc_mag_params *p, const double *pos,
                   double *m_out);

/* updateWalkersMag restated in FP64 (reference order) for a single pore:
 * sums[3*j..3*j+2] = (sum Mx, sum My, sum Mz) of field j over the walkers;
 * m_walk (optional) = the first `trace->ntrace` walkers' final M
 * [ntrace][nf][3]; trace (optional) = their trajectories as orc_walk
 * records them.  Returns 0 or a negative code. */
int orc_mag_walk(const orc_basis *pore, const orc_field *f, int nf, const orc_mag_params *p,
                 int nthreads, double *sums, double *m_walk, orc_trace *trace);

#ifdef __cplusplus
}
#endif
#endif
