/*
 * axx.h -- C ABI of the GB300-native axonexa random-walker phase path.
 *
 * One process drives one GPU through an opaque context.  Every entry point
 * returns an axx_status; nothing aborts the process or traps on the device.
 * Inputs are plain structs of doubles and ints in the reference's own units
 * (lengths in mm, time in ms, gradients in T/mm, D in mm^2/ms, kappa in mm/ms,
 * gamma in rad/(ms*T)); any consistent unit set works as long as `gamma`
 * matches it.  Outputs are the reference's unnormalised sums
 *   mx[j] = sum_walkers cos(phase_j) * exp(-T2factor)
 *   my[j] = sum_walkers sin(phase_j) * exp(-T2factor)
 * in FP64, plus optional second moments for standard errors.
 *
 * Reference interfaces replaced (paths relative to the axonexa project root):
 *   axx_run_lattice  <- phaseAcquisitionStream<F>::runAcquisitionLattice
 *                       (src/acquisition/phaseAcquisitionStream.cuh:126-190),
 *                       whose device work is updateWalkersLatticePhase
 *                       (src/kernels/kernelLattice.cuh:1-104) followed by
 *                       cudaVector::transformAndSumTwoVectors
 *                       (src/util/cudaVector.cu:143-172).
 *   axx_run_single   <- phaseAcquisitionStream<F>::runAcquisition
 *                       (src/acquisition/phaseAcquisitionStream.cuh:37-88),
 *                       device work updateWalkersPhase
 *                       (src/kernels/kernelPhase.cuh:4-66).
 *   axx_run_batch    <- phaseAcquisitionStream<F>::runAcquisitionStreamLattice
 *                       (src/acquisition/phaseAcquisitionStream.cuh:425-613) and
 *                       runAcquisitionStream (:254-423): many acquisitions,
 *                       here in one persistent launch.
 *   axx_bvalue       <- RectGrad/CosGFunc/SinGFunc/ApodCosGFunc/SWOGSEFunc::getB
 *                       (src/functors/gfunctors.cuh:31-33, 89-91, 143-145,
 *                       196-199, 257-263).
 *   axx_gradient_eval<- the same functors' operator()(time)
 *                       (src/functors/gfunctors.cuh:36-54, 94-113, 148-167,
 *                       202-228, 265-283).
 *   axx_substrate_rps_gamma <- RPSLatticeInitializer<Basis>::gammaRadialDist +
 *                       uniformCenterDist + correctEdges
 *                       (src/substrate/RPSinitializer.h:76-186).
 *   axx_substrate_pack <- uniformCenterDist + correctEdges
 *                       (src/substrate/RPSinitializer.h:103-186) for given radii.
 *   axx_volume_fraction <- calcf + kernelCalcf (src/util/calcf.cuh:1-38).
 *   axx_run_wc       <- phaseAcquisitionStream<F>::runAcquisitionWC
 *                       (src/acquisition/phaseAcquisitionStream.cuh:193-252)
 *                       with kernelWC (src/kernels/kernelWC.cuh:13-89).
 *   axx_run_mag      <- magAcquisitionStream<F>::runAcquisition
 *                       (src/acquisition/magAcquisitionStream.cuh:37-90) with
 *                       the device work of updateWalkersMag
 *                       (src/kernels/kernelMag.cuh:1-141), the B-field
 *                       functors (src/functors/bfunctors.cuh) and the Bloch
 *                       updates (src/bloch/blochdiff.cuh:29-172).
 */
#ifndef AXX_H_
#define AXX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AXX_ABI_VERSION 1

typedef enum {
  AXX_OK = 0,
  AXX_ERR_INVALID_ARG = 1,     /* a size, pointer or parameter is out of range */
  AXX_ERR_CUDA = 2,            /* a CUDA runtime call failed (text in axx_last_error) */
  AXX_ERR_REFLECTION_CAP = 3,  /* some walker hit the per-step reflection cap;
                                  results are still written, the count is in stats */
  AXX_ERR_TIMEOUT = 4,         /* a bounded device wait ran out */
  AXX_ERR_NO_DEVICE = 5,       /* no CUDA device, or the library was built without one */
  AXX_ERR_OUT_OF_MEMORY = 6,
  AXX_ERR_ABORTED = 7,         /* axx_abort() was called while the run was in flight */
  AXX_ERR_UNSUPPORTED = 8,     /* a valid request this build does not implement */
  AXX_ERR_NUMERIC = 9          /* a non-finite input or result */
} axx_status;

typedef struct axx_ctx axx_ctx;
typedef struct axx_plan axx_plan;

/* ---- geometry ------------------------------------------------------------ */

enum { AXX_PRIM_CYLINDER_Z = 0, /* Cylinder_XY: infinite cylinder, axis along z */
       AXX_PRIM_SPHERE = 1,     /* Sphere */
       AXX_PRIM_PLANE = 2,      /* Plane: infinite impermeable wall (lattices only) */
       AXX_PRIM_CYLINDER = 3 }; /* Cylinder: infinite cylinder along (nx, ny, nz) */

/* One basis object (src/primitives/cylinderXY.cuh:1-40, Sphere.cuh:4-44,
 * plane.cuh:1-40, cylinder.cuh:1-199).  An AXX_PRIM_CYLINDER runs through
 * (cx, cy, cz) along the axis (nx, ny, nz): any axis for a single pore (the
 * walk runs in the cylinder's frame (ahat, bhat, chat) of cylinder.cuh:20-40
 * and traces come back in simulation coordinates); in a lattice all such
 * cylinders share one axis along a cell axis (x, y or z), and z-cylinders
 * (AXX_PRIM_CYLINDER_Z) may join them only when that axis is z.  A plane is the wall through (cx, cy, cz) with normal
 * (nx, ny, nz) (normalised by the library; Plane::getNormal returns it as
 * given and the reflection assumes unit length).  It has no inside: it never
 * contains a point (no region, D or T2 of its own), reflects every crossing
 * and transmits nothing (Plane::getPermeability is 0); radius, D, T2, T1 and
 * permeability are ignored for it. */
typedef struct {
  int32_t type;          /* AXX_PRIM_* */
  int32_t region;        /* value reported by the region lookup (Lattice::inRegion) */
  double cx, cy, cz;     /* centre (a point of a plane); cz is ignored for cylinders */
  double radius;
  double D;              /* diffusion coefficient inside */
  double T2;             /* transverse relaxation time inside */
  double T1;             /* carried for layout parity; unused on the phase path */
  double permeability;   /* kappa; transmission probability is 4*kappa/v */
  double eps;            /* minimum hit distance (cylEPS / sphereEPS; doub_equal's
                            1e-14 for a plane) */
  double nx, ny, nz;     /* plane normal, or AXX_PRIM_CYLINDER axis; ignored otherwise */
} axx_basis;

/* Periodic cell (src/substrate/lattice.cuh:3-23): a x b x c box with the
 * extracellular D, T2, T1. */
typedef struct {
  double a, b, c;
  double T2, T1, D;
} axx_lattice;

/* ---- gradient sequences (src/functors/gfunctors.cuh) --------------------- */

enum { AXX_SEQ_PGSE = 0,      /* RectGrad(G, duration, spacing) */
       AXX_SEQ_COS = 1,       /* CosGFunc */
       AXX_SEQ_SIN = 2,       /* SinGFunc */
       AXX_SEQ_APODCOS = 3,   /* ApodCosGFunc */
       AXX_SEQ_SQUARE = 4 };  /* SWOGSEFunc (square wave, sign (-1)^floor(2 t nu)) */

typedef struct {
  int32_t kind;          /* AXX_SEQ_* */
  int32_t num_periods;   /* OGSE periods per lobe; ignored for PGSE */
  double G;              /* gradient amplitude */
  double duration;       /* delta: lobe length */
  double spacing;        /* gap between lobes (Delta - delta) */
  double gx, gy, gz;     /* gradient direction (the reference's gHat) */
} axx_sequence;

/* ---- run parameters ------------------------------------------------------ */

enum {
  AXX_FLAG_RELAXATION = 1u << 0,        /* USE_RELAXATION: weight by exp(-sum dt/T2) */
  AXX_FLAG_PERMEABLE = 1u << 1,         /* USE_PERMEABLE: boundaryCheckPermeable */
  AXX_FLAG_SIMPLE_REJECTION = 1u << 2,  /* no SPECULAR_REFLECTION: reject moves that
                                           change region */
  AXX_FLAG_KEEP_INIT_QUIRK = 1u << 3,   /* single pore: the start position draws from a
                                           copy of the stream, as unifRand(curandState)
                                           by value does (Sphere.cuh:55); default on in
                                           axx_run_single unless AXX_FLAG_FIX_INIT_QUIRK */
  AXX_FLAG_FIX_INIT_QUIRK = 1u << 4,
  AXX_FLAG_LATTICE_PICKING = 1u << 5,   /* single pore, LATTICE_PICKING (kernelPhase.cuh:31-35):
                                           every move is +-stepLength along each axis, the
                                           signs from three stream words */
  AXX_FLAG_COMPARTMENTS = 1u << 6       /* lattice walks: also the sums over the walkers that
                                           start inside a basis (Lattice::inRegion != 0), in
                                           axx_stats.mx_in/my_in/walkers_in; the rest of the
                                           signal is the extracellular start compartment */
};

enum { AXX_INIT_UNIFORM = 0,     /* Lattice::initializeUniformly (lattice.cuh:31-37) */
       AXX_INIT_IN_REGION = 1,   /* Lattice::initializeInRegion(region = init_arg) */
       AXX_INIT_IN_BASIS = 2 };  /* basis[init_arg].randUnif (kernelLattice.cuh:29-34) */

typedef struct {
  int64_t num_walkers;   /* any N >= 1 (no multiple-of-block-size requirement) */
  int32_t steps;         /* SimuParamsPhase::steps: the walk makes steps-1 moves */
  int32_t init_mode;     /* AXX_INIT_* */
  int32_t init_arg;
  uint32_t flags;        /* AXX_FLAG_* */
  uint64_t seed;         /* Philox4x32-10 key; walker w uses stream (seed, w) */
  double timestep;
  double gamma;          /* gyromagnetic ratio; 0 selects 267500 rad/(ms*T) */
  int64_t walker_offset; /* first global walker id (sharding keeps streams fixed) */
} axx_run_params;

/* Optional per-sequence statistics.  Each array has nseq entries. */
typedef struct {
  double *sxx;           /* sum of x^2, x = cos(phase) exp(-T2factor) */
  double *syy;           /* sum of y^2 */
  double *sxy;           /* sum of x*y */
  int64_t reflection_cap_hits; /* walker-steps that hit the reflection cap */
  int64_t walker_steps;  /* moves simulated (num_walkers * (steps - 1)) */
  int64_t boundary_hits; /* reflections and transmissions over all moves */
  /* With AXX_FLAG_COMPARTMENTS (else left untouched): */
  double *mx_in;         /* nseq sums of x over the walkers starting inside a basis */
  double *my_in;         /* nseq sums of y over them */
  int64_t walkers_in;    /* how many walkers started inside a basis */
} axx_stats;

/* ---- context ------------------------------------------------------------- */

int axx_abi_version(void);
const char *axx_status_string(axx_status s);

/* Creates a context on `device` with its own stream.  One context per host
 * thread; contexts do not share state. */
axx_status axx_create(axx_ctx **out, int device);
axx_status axx_destroy(axx_ctx *ctx);
/* Text of the last error on this context (valid until the next call). */
const char *axx_last_error(const axx_ctx *ctx);
/* Device properties used for grid sizing. */
axx_status axx_device_info(axx_ctx *ctx, int *num_sms, int *cc_major, int *cc_minor,
                           size_t *global_mem_bytes);
/* Requests an in-flight run to stop at its next step boundary; the run then
 * returns AXX_ERR_ABORTED.  Safe to call from another host thread. */
axx_status axx_abort(axx_ctx *ctx);

/* ---- one-shot runs (host buffers in and out; synchronous) ---------------- */

/* Lattice walk: replaces runAcquisitionLattice.  basis may be NULL when
 * nbasis == 0 (free diffusion in the periodic box). */
axx_status axx_run_lattice(axx_ctx *ctx, const axx_lattice *lat, const axx_basis *basis,
                           int nbasis, const axx_sequence *seqs, int nseq,
                           const axx_run_params *params, double *mx, double *my,
                           axx_stats *stats);

/* Single-pore walk: replaces runAcquisition (walkers start inside basis[0],
 * phase uses the bounded position, no lattice, no relaxation). */
axx_status axx_run_single(axx_ctx *ctx, const axx_basis *basis, const axx_sequence *seqs,
                          int nseq, const axx_run_params *params, double *mx, double *my,
                          axx_stats *stats);

/* Lattice walk that allocates no GPU memory.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc when they run
 * a walk (a memory pool or budget that owns all device memory, a framework
 * that forbids allocation after start-up, a thread that must not trigger the
 * synchronisation cudaMalloc/cudaFree can cause).  Same inputs and outputs as
 * axx_run_lattice and the same kernels; every device-side buffer of the call
 * lives in one static array of AXX_NOALLOC_SCRATCH_BYTES that each GPU
 * loading the library holds until the process exits (with lazy module
 * loading it is committed when the module first loads on the device: at the
 * first call, or at any earlier use of the library's kernels).  A walk whose
 * tables and per-block partials do not fit even one block per SM is rejected
 * with AXX_ERR_INVALID_ARG; when the partials of the full grid do not fit,
 * the grid shrinks, and the results then equal axx_run_lattice's up to the
 * grouping of the per-block FP64 partial sums (rounding only).  The call is
 * synchronous: it returns after the results are on the host.  The array's
 * device address is looked up at the first call in each device context (and
 * again after a device reset), so make the first call before any stream
 * capture.  All calls on a device share the array: calls whose GPU work
 * overlaps race and must be serialised by the caller.  The context must have
 * been created beforehand (axx_create). */
#define AXX_NOALLOC_SCRATCH_BYTES (8u << 20)
axx_status axx_run_lattice_noalloc(axx_ctx *ctx, const axx_lattice *lat,
                                   const axx_basis *basis, int nbasis,
                                   const axx_sequence *seqs, int nseq,
                                   const axx_run_params *params, double *mx, double *my,
                                   axx_stats *stats);

/* ---- device-resident plans (inputs uploaded once, launched repeatedly) ---- */

axx_status axx_plan_lattice(axx_ctx *ctx, const axx_lattice *lat, const axx_basis *basis,
                            int nbasis, const axx_sequence *seqs, int nseq,
                            const axx_run_params *params, axx_plan **out);
axx_status axx_plan_single(axx_ctx *ctx, const axx_basis *basis, const axx_sequence *seqs,
                           int nseq, const axx_run_params *params, axx_plan **out);
/* Enqueues the walk and the signal reduction on the context stream; returns
 * without waiting. */
axx_status axx_plan_launch(axx_plan *plan);
/* Waits for the last launch and copies its results to host memory. */
axx_status axx_plan_read(axx_plan *plan, double *mx, double *my, axx_stats *stats);
/* Per-plan facts: channels = distinct (waveform, direction) phase
 * accumulators, instances = basis objects plus periodic ghosts,
 * kernel_launches = kernels one axx_plan_launch enqueues. */
axx_status axx_plan_info(const axx_plan *plan, int *channels, int *instances,
                         int *kernel_launches, int64_t *walker_steps);
/* Boundary candidates one move tests, averaged over the cell: the entries of
 * the grid-cell lists per cell (walkers are uniform in the cell), 1 for a
 * single pore, 0 for free diffusion.  The n_cand of the walk's op count;
 * the reference tests every basis each move (Lattice::intersectionCheck*,
 * src/substrate/lattice.cuh:184-246). */
axx_status axx_plan_candidates(const axx_plan *plan, double *per_move);
axx_status axx_plan_destroy(axx_plan *plan);

/* Bytes the walk entry points (plans and one-shot runs) copied host to
 * device (tables) and device to host (sums, counters) on this context since
 * it was created: what an end-to-end call moves across the host link.  The
 * reference copies the per-walker phases instead
 * (src/acquisition/phaseAcquisitionStream.cuh:139-189). */
axx_status axx_transfer_bytes(axx_ctx *ctx, int64_t *h2d_bytes, int64_t *d2h_bytes);

/* Timing on the context stream: record event `slot` (0..7), and read the
 * elapsed milliseconds between two recorded slots after a sync. */
axx_status axx_event_record(axx_ctx *ctx, int slot);
axx_status axx_event_elapsed(axx_ctx *ctx, int slot_a, int slot_b, float *ms);
axx_status axx_sync(axx_ctx *ctx);

/* Measured FP32 issue peak of this device: fused multiply-adds per second of
 * a register-resident FMA kernel on every SM (one FMA counts as one op, the
 * convention of the walker's roofline).  Diagnostics for roofline reports;
 * no reference counterpart. */
axx_status axx_fp32_fma_peak(axx_ctx *ctx, double *fma_per_s);

/* ---- batched acquisitions: many substrates in one persistent launch ------ */

/* One acquisition of a batch (one substrate, its sequences, its run). */
typedef struct {
  int32_t mode;                  /* 0: lattice walk, 1: single-pore walk */
  axx_lattice lattice;           /* lattice mode */
  const axx_basis *basis;        /* lattice bases, or the single pore in basis[0] */
  int32_t nbasis;
  const axx_sequence *seqs;      /* at most 64 per job */
  int32_t nseq;
  axx_run_params params;         /* walkers, steps, seed, timestep, flags */
} axx_job;

typedef struct {
  int32_t tile;          /* walkers per work item (multiple of 128); 0: autotuned */
  int32_t blocks_per_sm; /* resident blocks per SM; 0: the occupancy limit */
  int32_t use_graph;     /* 1: capture the launch in a CUDA graph and replay it */
} axx_batch_options;

typedef struct axx_batch axx_batch;

/* Plans a batch: uploads every job's tables once and cuts the jobs' walker
 * ranges into work items (longest first) that one persistent kernel takes
 * from a shared counter.  Replaces running the acquisitions one by one
 * (phaseAcquisitionStream::runAcquisitionStreamLattice / runAcquisitionStream,
 * src/acquisition/phaseAcquisitionStream.cuh:254-613).  Jobs may not use
 * AXX_FLAG_SIMPLE_REJECTION.  With tile == 0 the tile and blocks per SM come
 * from axx_autotune_batch's cache (or are tuned on first use). */
axx_status axx_batch_create(axx_ctx *ctx, const axx_job *jobs, int njobs,
                            const axx_batch_options *opt, axx_batch **out);
/* Enqueues one execution of the whole batch (graph replay or launches). */
axx_status axx_batch_launch(axx_batch *b);
/* Waits and writes the signals: mx/my hold sum(nseq) entries, job after job;
 * stats (optional) is an array of njobs records whose sxx/syy/sxy may be NULL. */
axx_status axx_batch_read(axx_batch *b, double *mx, double *my, axx_stats *stats);
axx_status axx_batch_info(const axx_batch *b, int *items, int *tile, int *blocks_per_sm,
                          int *kernel_launches, int64_t *walker_steps);
axx_status axx_batch_destroy(axx_batch *b);
/* One-shot batch: create, launch, read, destroy. */
axx_status axx_run_batch(axx_ctx *ctx, const axx_job *jobs, int njobs,
                         const axx_batch_options *opt, double *mx, double *my,
                         axx_stats *stats);
/* The project's autotuner: times candidate (tile, blocks per SM) pairs on a
 * shortened copy of the batch (steps capped at `probe_steps`), returns the
 * fastest in *best and its time in *best_ms, and records it in the tuning
 * cache (file named by AXX_AUTOTUNE_CACHE, default
 * $HOME/.cache/axonexa_gb300/autotune.tsv) under the device name and the
 * batch's shape. */
axx_status axx_autotune_batch(axx_ctx *ctx, const axx_job *jobs, int njobs, int probe_steps,
                              axx_batch_options *best, double *best_ms);

/* ---- learned surrogate: MLP in -> depth x width (SiLU) -> 1 -------------- */

/* No reference counterpart: the reference has no learned component.  A small
 * MLP maps substrate and sequence parameters to the signal; it is trained on
 * signals the walk above produces and runs on the tensor cores in BF16 with
 * FP32 accumulation.  Inputs are standardised by the caller. */
typedef struct axx_mlp axx_mlp;

axx_status axx_mlp_create(axx_ctx *ctx, int in_dim, int width, int depth, uint64_t seed,
                          axx_mlp **out);
axx_status axx_mlp_destroy(axx_mlp *m);
/* Number of parameters and FP32 copies of them (weights then biases per
 * layer, weights row-major [out][in]). */
axx_status axx_mlp_num_params(const axx_mlp *m, int64_t *n);
axx_status axx_mlp_get_params(axx_mlp *m, float *params);
axx_status axx_mlp_set_params(axx_mlp *m, const float *params);
/* Mean-squared-error gradients of one batch (host X[n][in_dim], y[n]); grads
 * has axx_mlp_num_params entries; *loss receives the batch loss. */
axx_status axx_mlp_gradients(axx_mlp *m, const float *X, const float *y, int n, float *grads,
                             float *loss);
/* Adam training on the device: `steps` updates with batches of `batch` rows
 * drawn (seeded) from the n training pairs; loss_out (optional, steps
 * entries) receives each batch loss. */
axx_status axx_mlp_train(axx_mlp *m, const float *X, const float *y, int n, int batch, int steps,
                         float lr, uint64_t seed, float *loss_out);
/* Predictions for host inputs (X[n][in_dim] -> y[n]) on the tensor cores.
 * The rows cross in up to four chunks whose copies overlap the kernel (the
 * overlap needs pinned host memory); the outputs equal
 * axx_mlp_predict_device's bit for bit.  The device copies of X and y are
 * kept with the network and grow to the largest n seen. */
axx_status axx_mlp_predict(axx_mlp *m, const float *X, int n, float *y);
/* Device-resident prediction for timing: X and y are device pointers. */
axx_status axx_mlp_predict_device(axx_mlp *m, const float *dX, int n, float *dy);
/* FLOPs of one forward row (2 per multiply-add). */
axx_status axx_mlp_flops_per_row(const axx_mlp *m, double *flops);

/* ---- sequences ----------------------------------------------------------- */

/* b-value of one sequence, as the reference functor's getB(). */
axx_status axx_bvalue(const axx_sequence *seq, double gamma, double *b);
/* Gradient vector of one sequence at `n` times, out[3*i..3*i+2]. */
axx_status axx_gradient_eval(const axx_sequence *seq, const double *t, int n, double *out);

/* ---- randomness ---------------------------------------------------------- */

/* The first n 32-bit words of walker `walker`'s stream for `seed`, computed
 * on the device (stream word k = Philox4x32-10(key = seed, counter =
 * (k/4, walker))[k % 4]; the walk uses words 1, 2, 3, ...). */
axx_status axx_philox_words(axx_ctx *ctx, uint64_t seed, uint64_t walker, int n,
                            uint32_t *out);

/* ---- parity instrumentation ---------------------------------------------- */

/* Runs the lattice walk for walkers [walker_offset, walker_offset+ntrace) and
 * records, after every move i = 1..steps-1: the wrapped position, the region
 * index (-1 = extracellular), the number of boundary hits of that move and
 * the number of random words consumed so far.  Layout: pos[(w*(steps-1)+i-1)*3+k],
 * region/hits/words[w*(steps-1)+i-1].  init_pos[w*3+k] is the start position. */
axx_status axx_trace_lattice(axx_ctx *ctx, const axx_lattice *lat, const axx_basis *basis,
                             int nbasis, const axx_run_params *params, int ntrace,
                             float *init_pos, float *pos, int32_t *region, int32_t *hits,
                             int32_t *words);
/* The same for the single-pore walk. */
axx_status axx_trace_single(axx_ctx *ctx, const axx_basis *basis,
                            const axx_run_params *params, int ntrace, float *init_pos,
                            float *pos, int32_t *region, int32_t *hits, int32_t *words);

/* ---- substrates (host) ---------------------------------------------------- */

/* Random sequential packing of `n` cylinders with gamma(shape, mean/shape)
 * radii in a periodic square cell whose side is chosen so the intracellular
 * area fraction is `fraction`; radii are truncated to [rmin, rmax].  Writes
 * the cell side to *side and up to max_out bases (originals first, then the
 * periodic images of the ones that cross the cell edge) to out, their count to
 * *nout and the achieved area fraction to *achieved.  D_in, T2_in and
 * permeability fill the basis records; region = index+1 as correctEdges sets.
 * Every pair of cylinders keeps a gap of 1 % of its radius sum. */
axx_status axx_substrate_rps_gamma(uint64_t seed, int n, double shape, double mean,
                                   double rmin, double rmax, double fraction,
                                   double D_in, double T2_in, double permeability,
                                   int max_out, axx_basis *out, int *nout, double *side,
                                   double *achieved);

/* One packing of axx_substrate_rps_gamma_gpu: n radii from gamma(shape,
 * mean/shape) truncated to (rmin, rmax); the cell side makes the cylinders'
 * area `fraction` of the cell; every cylinder gets D, T2 and permeability. */
typedef struct {
  double shape, mean;
  double rmin, rmax;
  double fraction;
  double D, T2, permeability;
} axx_pack_spec;

/* RPSLatticeInitializer (src/substrate/RPSinitializer.h:10-314) on the GPU,
 * npack packings of n cylinders at once (n <= 2048): gamma radii sampled on
 * the device (gammaRadialDist :76-101), random sequential addition largest
 * first with the periodic overlap test and a 1 % gap (uniformCenterDist
 * :103-129), pairwise overlap removal when addition jams, periodic images of
 * the cylinders that cross the cell edge (correctEdges :131-186).  Packing p's
 * bases (the n cylinders by ascending radius, region = index + 1, then the
 * images) go to out[p * max_out ...], their count to nout[p], the cell side
 * to side[p] and the area fraction to achieved[p].  The same algorithm as
 * axx_substrate_rps_gamma with the device's own draws: packings agree with
 * the host packer's in distribution. */
axx_status axx_substrate_rps_gamma_gpu(axx_ctx *ctx, uint64_t seed, int n, int npack,
                                       const axx_pack_spec *spec, int max_out, axx_basis *out,
                                       int *nout, double *side, double *achieved);

/* Monte Carlo intracellular volume fraction (calcf / kernelCalcf,
 * src/util/calcf.cuh:1-38): `points` uniform points in the cell (point i uses
 * words 1..3 of stream (seed, i), as a walker's start), counted when the first
 * basis containing them has region > 0.  Writes count / points and the count. */
axx_status axx_volume_fraction(axx_ctx *ctx, const axx_lattice *lat, const axx_basis *basis,
                               int nbasis, int64_t points, uint64_t seed, double *fraction,
                               int64_t *inside);

/* The WCDMC comparison walker (kernelWC, src/kernels/kernelWC.cuh:13-89, as
 * phaseAcquisitionStream::runAcquisitionWC drives it, :193-252): walkers in
 * one pore, per step Gaussian displacements of sigma = sqrt(2 D dt) per axis
 * from four uniforms of a per-walker 32-bit xorshift state (Box-Muller), a
 * move leaving the pore rejected, the Kahan-summed phase gamma dt sum_t
 * G[t] . r.  rng_state[n], start[n*3] and grad[steps*3] (T/mm) come from the
 * caller as the reference's driver makes them on the host; writes the phases
 * (optional, phase[n]) and sum_cos / sum_sin of the phases (FP64). */
axx_status axx_run_wc(axx_ctx *ctx, const axx_basis *pore, int64_t num_walkers, int32_t steps,
                      double timestep, double gamma, const uint32_t *rng_state,
                      const double *start, const double *grad, double *phase, double *sum_cos,
                      double *sum_sin);

/* ---- magnetisation (Bloch) walk of a single pore ------------------------- */

/* B-field functor kinds (src/functors/bfunctors.cuh). */
enum {
  AXX_FIELD_QSC_GRE = 0,      /* QSC_GRE(B0, G, duration, spacing) */
  AXX_FIELD_QSC_PGSE = 1,     /* QSC_PGSE(B0, G, duration, spacing, rf_duration,
                                 dtmin, dtmax, TE) */
  AXX_FIELD_QSC_COS_GRE = 2,  /* QSC_COS_GRE(B0, G, duration, spacing, num_periods) */
  AXX_FIELD_QSC_GRE_TRAP = 3, /* QSC_GRE_TRAP(B0, G, duration, spacing, ramp) */
  AXX_FIELD_SIN_GRE = 4,      /* SIN_GRE(B0, (gx,gy,gz), duration, spacing, period) */
  AXX_FIELD_COS_GRE = 5,      /* COS_GRE(B0, (gx,gy,gz), duration, spacing, num_periods) */
  AXX_FIELD_RECT_GRE = 6,     /* RECT_GRE(B0, (gx,gy,gz), duration, spacing) */
  AXX_FIELD_UCN_LOWFIELD = 7  /* UCN_lowfield(B0, G, rf_duration, dtmin, dtmax) */
};

/* One field functor; unused members are ignored.  B in T, G in T/mm,
 * times in ms (the reference's units). */
typedef struct {
  int32_t kind, num_periods;
  double B0, G, gx, gy, gz;
  double duration, spacing, period, ramp, rf_duration, dtmin, dtmax, TE;
} axx_field;

/* Integrators of updateWalkersMag's compile-time switches.  ROTATE: the
 * default exact rotation (updateMag_noT2_rotate).  RK4 (RK4_NORELAXATION):
 * fourth-order Runge-Kutta for the t = 0 update only -- the reference's step
 * loop has no RK4 branch and rotates.  ROTATE_MULTISTEP: rotations of the
 * functor's getStepTimeMin (QSC_PGSE and UCN_lowfield only).  DORP: adaptive
 * Dormand-Prince 5(4) over every step (the integrator DORP_NORELAXATION aims
 * at, updateMag_DORP, blochdiff.cuh:69-146, whose build does not compile):
 * sub-steps dt/2^k, k <= dorp_levels, halved while the embedded error
 * estimate exceeds dorp_tol (relative to 1 + |M|) and doubled when it falls
 * below 1/32 of it; the field is evaluated at the true stage times, so it
 * resolves fields that vary within a step.  For |gamma B| dt up to about 1
 * (low field); the rotations are exact at any field. */
enum { AXX_MAG_ROTATE = 0, AXX_MAG_RK4 = 1, AXX_MAG_ROTATE_MULTISTEP = 2, AXX_MAG_DORP = 3 };

typedef struct {
  int64_t num_walkers;
  int32_t steps;       /* time points 0..steps-1, steps-1 moves */
  int32_t integrator;  /* AXX_MAG_* */
  uint32_t flags;      /* AXX_FLAG_SIMPLE_REJECTION, AXX_FLAG_FIX_INIT_QUIRK */
  uint32_t dorp_levels; /* DORP: halvings of the step allowed, 0..8 (0: 3) */
  uint64_t seed;
  double timestep;     /* ms */
  double gamma;        /* rad/(ms T); the reference's GAMMA macro (0: 267500;
                          negative for helium-3, -203789, as its magLF examples) */
  double m0[3];        /* initial magnetisation (SimuParams mx/my/mz_initial) */
  int64_t walker_offset;
  double dorp_tol;     /* DORP: error tolerance (0: 1e-6) */
} axx_mag_params;

#define AXX_MAG_MAX_FIELDS 16

/* Walkers in one pore (Cylinder_XY or Sphere, as updateWalkersMag's
 * basis[0]); per field functor j the sums over walkers of the final
 * magnetisation: mx[j], my[j], mz[j] (FP64; magAcquisition::getMx/My/Mz).
 * 1 <= nfield <= AXX_MAG_MAX_FIELDS. */
axx_status axx_run_mag(axx_ctx *ctx, const axx_basis *pore, const axx_field *fields, int nfield,
                       const axx_mag_params *params, double *mx, double *my, double *mz);
/* The first ntrace walkers of the same walk: start position init_pos[3],
 * position after every move pos[(steps-1)*3], boundary hits and next stream
 * word per move, final magnetisation m_final[nfield*3] (all per walker). */
axx_status axx_trace_mag(axx_ctx *ctx, const axx_basis *pore, const axx_field *fields, int nfield,
                         const axx_mag_params *params, int ntrace, float *init_pos, float *pos,
                         int32_t *hits, int32_t *words, float *m_final);

/* ---- triangle-mesh pores -------------------------------------------------- */

/* A closed triangle mesh as a single pore (src/primitives/mesh.cuh:1-75 and
 * triangle.cuh:1-59, drafts that do not compile: "We assume no holes -> a
 * closed surface mesh").  Walkers start uniformly inside (rejection in the
 * bounding box with the mesh's vertical-ray parity test), move with speed
 * sqrt(6 D / dt) and reflect specularly off the nearest triangle hit
 * (Triangle::intersect: the plane of the triangle, then the barycentric
 * inside test, slightly widened so that shared edges leave no gap); the phase
 * uses the bounded position as the single-pore walk does. */
typedef struct {
  const double *vertices;    /* [nvert][3] */
  int32_t nvert;
  const int32_t *triangles;  /* [ntri][3] vertex indices, any orientation */
  int32_t ntri;
  double D;                  /* diffusion coefficient inside */
} axx_mesh;

/* One mesh-pore walk; params->flags must be 0 (specular reflection only),
 * init_mode is ignored.  escaped: walkers found outside the mesh after their
 * walk (a leak through the surface; 0 for a closed mesh), may be NULL. */
axx_status axx_run_mesh(axx_ctx *ctx, const axx_mesh *mesh, const axx_sequence *seqs, int nseq,
                        const axx_run_params *params, double *mx, double *my, axx_stats *stats,
                        int64_t *escaped);
/* The first ntrace walkers of the same walk: start init_pos[3], position
 * after every move pos[(steps-1)*3], triangle hits and next stream word per
 * move. */
axx_status axx_trace_mesh(axx_ctx *ctx, const axx_mesh *mesh, const axx_run_params *params,
                          int ntrace, float *init_pos, float *pos, int32_t *hits, int32_t *words,
                          int64_t *escaped);

/* The placement step of axx_substrate_rps_gamma for caller-chosen radii
 * (radii[n], any order; they are sorted ascending and region = index+1 in that
 * order).  Same cell, gap, image and output rules. */
axx_status axx_substrate_pack(uint64_t seed, int n, const double *radii, double fraction,
                              double D_in, double T2_in, double permeability, int max_out,
                              axx_basis *out, int *nout, double *side, double *achieved);

#ifdef __cplusplus
}
#endif

#endif /* AXX_H_ */
