/*
 * kb2pi.h -- C ABI of libkb2pi, a GB300 (sm_103a) implementation of the 2PI
 * Kadanoff-Baym time step of magdalenaeriksson/QFTdynamicsM.jl
 * src/TwoPIScalar (O(N) lambda phi^4 on an Ns^3 periodic lattice; LambdaLO,
 * LambdaNLO quantum = 3-loop sunset, LambdaNLO classical truncations).
 *
 * The entry points are what a Julia `TwoPIScalarGPU <: TwoPIScalarNumerics`
 * backend binds with `ccall`; each cites the reference function it replaces.
 * Plain C types only. Every call returns 0 on success or a negative KB_ERR_*
 * code; kb_last_error() gives the message. Calls on one handle must be
 * serialised (one CUDA stream per handle); distinct handles are independent.
 *
 * Time indices follow the reference: t counts from 1, the window after a step
 * t is [tmin, t] with tmin = max(1, t - M + 1) (expandSimData!,
 * src/TwoPIScalar/TwoPIScalar_SimDataStruct.jl:262-278).
 *
 * Momenta are stored per cubic orbit: the orbit of a lattice site is the set
 * reached by permuting and reflecting its coordinates. Orbits are numbered by
 * their sorted folded coordinates a <= b <= c (a_i = min(n_i, Ns - n_i)) as
 * c(c+1)(c+2)/6 + b(b+1)/2 + a. kb_get_orbits() returns the table.
 */
#ifndef KB2PI_H
#define KB2PI_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kb_handle kb_handle;

enum {
  KB_OK = 0,
  KB_ERR_PARAM = -1,   /* invalid parameter or call order */
  KB_ERR_OOM = -2,     /* device allocation failed */
  KB_ERR_CUDA = -3,    /* CUDA runtime error */
  KB_ERR_NAN = -4,     /* non-finite value detected in a measurement */
  KB_ERR_TIMEOUT = -5, /* a bounded device wait expired (kernel returned early) */
  KB_ERR_RANGE = -6,   /* time index outside the memory window (BoundsError) */
  KB_ERR_NODEV = -7    /* no CUDA device / library built without a device */
};

/* Perturbative expansion (src/TwoPIScalar/TwoPIScalar_Problemdefinition.jl:34-45):
 * LambdaLO, LambdaNLO (quantum), LambdaNLOclassical, NinverseLO, NinverseNLO.
 * KB_PEXP_NINV_NLO needs KB_PREC_FP64. */
enum { KB_PEXP_LO = 0, KB_PEXP_NLO_QUANTUM = 1, KB_PEXP_NLO_CLASSICAL = 2, KB_PEXP_NINV_LO = 3, KB_PEXP_NINV_NLO = 4 };
/* Precision: plain FP64 everywhere, or FP32 history/transforms/sunset with
 * FP64 leapfrog state, accumulation of the memory integrals, tadpole and
 * diagnostics. */
enum { KB_PREC_FP64 = 0, KB_PREC_MIXED = 1 };

/* One simulation; mirrors the fields of TwoPIScalarDiscretizationLattice
 * (TwoPIScalar_Discretization.jl:4-17) and Phi4 (…_ModelExpansionRenormalization.jl:5-9). */
typedef struct kb_params {
  int32_t Ns;        /* disc.Nx (even, 2..64) */
  int32_t sdim;      /* disc.sdim (3) */
  int32_t M;         /* NstepsinMemory (3 <= M <= 1024) */
  int32_t N;         /* model.ONgroup */
  int32_t pexp;      /* KB_PEXP_* */
  int32_t precision; /* KB_PREC_*; must be equal for all runs of one handle */
  int32_t device;    /* CUDA device ordinal */
  int32_t flags;     /* bits 0-15: extra ring slots kept beyond the memory
                      * window (kb_adjoint needs >= its ckpt_every); 0 otherwise */
  double dt;         /* disc.dt */
  double lambda;     /* model.Lambda */
  double mass2;      /* model.Mass2: m^2 used in the evolution (after Renormalize) */
  double mass;       /* disc.Mass: time unit of measurements */
} kb_params;

/* Scalars of MeasurementTwoPIScalar (TwoPIScalar_Measurement.jl:2-23) */
typedef struct kb_meas_scalars {
  double time, E, E_pot, E_kin, E_mem, M2;
} kb_meas_scalars;

/* Replaces getTwoPISimData + getTwoPIScalarTmpData
 * (TwoPIScalar_SimDataStruct.jl:669-721): allocates the device-resident
 * two-time history ring, self-energy ring and scratch for one run. */
int kb_create(const kb_params *p, kb_handle **out);
/* Batched form: nruns independent simulations that advance in lock-step
 * (same t) in one launch per kernel. Runs may differ in Ns, M, N, lambda,
 * mass2, pexp; dt and precision are per run too but precision must agree. */
int kb_create_batch(const kb_params *p, int32_t nruns, kb_handle **out);
/* Replaces the finalizer of the simulation data. */
void kb_destroy(kb_handle *h);
/* Message of the last failed call on this handle (or of kb_create). */
const char *kb_last_error(const kb_handle *h);

/* Number of cubic orbits S of run `run`, and their table: rep = sorted folded
 * coordinates (3 per orbit), k2 = lev2 = sum_i 4 sin^2(pi n_i / Ns), deg =
 * number of lattice sites (replaces FFTWhelper's getfftwhelper, used at
 * TwoPIScalar_Modelfile.jl:64). Any output pointer may be NULL. */
int kb_num_orbits(const kb_handle *h, int32_t run, int32_t *S);
int kb_get_orbits(const kb_handle *h, int32_t run, int32_t *rep, double *k2, int64_t *deg);
/* orbit index of every lattice site (column-major site order, Ns^3 entries) */
int kb_site_orbits(const kb_handle *h, int32_t run, int32_t *orbit_of_site);

/* Replaces initSimData! (TwoPIScalar_Initialization.jl:8-47): F(1,1), F(2,1),
 * F(2,2), rho(2,1) = dt from the occupation n (per orbit, without the 1/2)
 * and the initialisation mass; sets the window to [1,2]. */
int kb_init(kb_handle *h, int32_t run, const double *n_of_orbit, double init_mass);
/* Generic form: caller-computed F(1,1), F(2,1), F(2,2) per orbit, rho(2,1) =
 * dt (e.g. initSimData! for TwoPIScalarGauss, TwoPIScalar_Initialization.jl:95-112). */
int kb_init_rows(kb_handle *h, int32_t run, const double *F11, const double *F21, const double *F22);

/* Replaces evolve!(thesolution, tmpdata, t) (TwoPIScalar_Evolution.jl:924-981)
 * for every run of the handle; t must be the last evolved step + 1. Also
 * prepares the measurement of step t. */
int kb_step(kb_handle *h, int32_t t);
/* `count` steps t0, t0+1, ... from one captured CUDA graph; when
 * measure_every > 0 the scalars of steps with (t - 2) % measure_every == 0 are
 * stored run-major in out (nruns x ceil(count / measure_every) entries). */
int kb_steps(kb_handle *h, int32_t t0, int32_t count, int32_t measure_every, kb_meas_scalars *out,
             int32_t out_capacity);
/* Replaces expandSimData! alone (window advance without computing), as the
 * reference benchmark fills the window (TwoPIScalar_Bechmark.jl:64-69). */
int kb_expand(kb_handle *h);

/* Replaces measure!/createMeasurement (TwoPIScalar_Measurement.jl:31-99,223-228)
 * for the last evolved step t. Per-orbit arrays (S entries, NULL to skip):
 * F = F(t-1,t-1), ddF, n, omega, c. */
int kb_measure(kb_handle *h, int32_t run, int32_t t, kb_meas_scalars *s, double *F, double *ddF,
               double *n, double *omega, double *c);
/* Pipelined kb_measure for a time loop that issues step t+1 before it reads
 * step t (evolve!/measure! of G_Simulation.jl:11-30 with the measurement one
 * step behind): kb_measure_enqueue(h, run, t), right after kb_step(h, t), queues
 * a copy of step t's measurement into one of two pinned host slots (t mod 2)
 * and returns at once; kb_measure_take(h, run, t, ...) waits for that copy only
 * and fills the outputs of kb_measure. A slot holds one step: take step t
 * before enqueuing step t+2. Device error flags travel with the copy and fail
 * the take as kb_sync would; the enqueue clears them on the handle's stream right
 * after copying them, so an error raised by step t is reported once, by the take
 * of the first measurement enqueued after it. */
int kb_measure_enqueue(kb_handle *h, int32_t run, int32_t t);
int kb_measure_take(kb_handle *h, int32_t run, int32_t t, kb_meas_scalars *s, double *F, double *ddF,
                    double *n, double *omega, double *c);
/* Traces of createMeasurement at lattice site 1 (TwoPIScalar_Measurement.jl:89-96):
 * SigF/Sigr at (t-1, tp) for tp = t-1 down to tmin; Fonet/ronet = F/rho(tmin, tp)
 * for tp = tmin .. t-1. Each has t - tmin entries. */
int kb_get_traces(kb_handle *h, int32_t run, double *Fonet, double *ronet, double *SigF, double *Sigr);

/* Host view of the history (SymMatrix getindex, DefSimDataElements.jl:185-208):
 * which = 0 for F, 1 for rho (true antisymmetric value), a and b in the window. */
int kb_get(kb_handle *h, int32_t run, int32_t which, int32_t a, int32_t b, double *out);
/* Test hook: overwrite F/rho(a,b) for all orbits (SymMatrix setindex!). */
int kb_set(kb_handle *h, int32_t run, int32_t which, int32_t a, int32_t b, const double *in);
/* Replaces calcSelfEnergies! alone (TwoPIScalar_Evolution.jl:16-31):
 * Sigma(tmone, tp) for every tp in [tmin, tmone] of the current window. */
int kb_self_energies(kb_handle *h, int32_t tmone);
/* Sigma_F (which = 0) or Sigma_rho (which = 1) at (t-1, z) from the last step
 * or kb_self_energies (CyclVector getindex, DefSimDataElements.jl:129-132). */
int kb_get_sigma(kb_handle *h, int32_t run, int32_t which, int32_t z, double *out);
/* simdata.indices after the last step: [tmin, tmax] */
int kb_window(const kb_handle *h, int32_t run, int32_t *tmin, int32_t *tmax);

/* Device measurement stream: evolves t0 .. t0+count-1 like kb_steps, and every
 * step with (t - 2) % measure_every == 0 (measure! of the reference's drivers,
 * G_SimulationArgs.jl:96-101) appends its createMeasurement record
 * (TwoPIScalar_Measurement.jl:31-99) to a device buffer from inside the
 * captured step graph; the host reads all records once at the end. Record m of
 * run r: out[m * nruns + r] (scalars) and, if arrays is not NULL, the per-orbit
 * F, ddF, n, omega, c at arrays + m * sum_r 5 S_r + sum_{r' < r} 5 S_r'
 * (each S_r values). Fails with KB_ERR_PARAM if more than capacity steps are
 * measured; *n_recorded (if not NULL) receives the number recorded. */
int kb_steps_recorded(kb_handle *h, int32_t t0, int32_t count, int32_t measure_every, kb_meas_scalars *out,
                      double *arrays, int32_t capacity, int32_t *n_recorded);

/* Snapshot of the full state (history, self-energies, window) into a host
 * buffer and back; replaces the serialisation the reference could not do
 * ("Serialization broke because of pointers in simdata", G_SimulationArgs.jl:117).
 * Restore refuses (KB_ERR_PARAM, nothing copied) a buffer shorter than
 * kb_checkpoint_size, a damaged header, or a snapshot of a handle whose runs
 * differ in Ns, M, N, pexp, precision or ring slots. */
int kb_checkpoint_size(const kb_handle *h, size_t *bytes);
int kb_checkpoint_save(kb_handle *h, void *host_buf, size_t bytes);
int kb_checkpoint_restore(kb_handle *h, const void *host_buf, size_t bytes);

/* Wait for all work of the handle and report device-side errors (timeouts,
 * non-finite measurements). */
int kb_sync(kb_handle *h);

/* Profiling hooks (the reference times steps with BenchmarkTools,
 * src/TwoPIScalar/TwoPIScalar_Bechmark.jl:94-116; these time each kernel):
 * kb_get_stream returns the handle's cudaStream_t (as void*) so that callers
 * can record their own events on it. While profiling is enabled kb_step and
 * kb_steps record CUDA events around every kernel launch (kb_steps then
 * launches step by step instead of replaying its graph); kb_profile_read
 * synchronises and returns the summed milliseconds and launch counts of
 * [0] the sunset kernel and [1] the memory-integral kernel since the last
 * read, then resets them. */
int kb_get_stream(const kb_handle *h, void **stream);
int kb_profile(kb_handle *h, int32_t enable);
int kb_profile_read(kb_handle *h, double *ms, int64_t *launches);

/* Launch configuration of a handle's kernels. No counterpart in the reference
 * (it has no tunables). Every choice computes the same step; the memory-integral
 * variant only changes the order of the FP32 tile partial sums (KB_PREC_MIXED). */
typedef struct kb_tuning {
  int32_t memint_variant; /* KB_PREC_MIXED: 1 column/row consumer groups, 0 register-blocked consumers,
                           * 2 (default) as 1 with four more warps that run the leapfrog of whole
                           * chunks while the consumers stream; KB_PREC_FP64: 0 (one kernel) */
  int32_t sunset_grid;    /* CTAs of the persistent sunset kernel; 0 = one per SM */
  int32_t batch_order;    /* batched handles: 0 runs in order, 1 costliest runs first in both grids */
  int32_t sunset_variant; /* KB_PREC_MIXED: 0 1024 threads per CTA, 1 512 threads (two CTAs per SM where
                           * their shared memory fits), 2 tensor cores (tcgen05.mma kind::tf32 with
                           * TF32 head/tail operands, Ns <= 78); KB_PREC_FP64: 0 */
  int32_t memint_split;   /* 1: each chunk's triangle of history tiles is streamed by two CTAs (equal
                           * halves by column blocks), then a finishing kernel adds their sums and runs
                           * the leapfrog; 2: the chunks past the last whole wave of one CTA per SM
                           * only (the others as 0), each in 2..6 parts, as many as make the pieces
                           * fill the SMs best; 0 (default): one CTA per chunk, the same arithmetic
                           * whatever the handle's size. 1 and 2 need memint_variant 1 or 2 in
                           * KB_PREC_MIXED */
  int32_t memint_bulk;    /* 1: history tiles by plain bulk copies of whole rows instead of tensor-map
                           * boxes (the path taken when the CUDA driver has no tensor-map encoder); 0 */
  int32_t test_no_tiles;  /* test hook, 0 in use: 1 makes the memory-integral producer issue no tiles,
                           * so every consumer's bounded wait runs out (about 2 s) and the step ends
                           * with KB_ERR_TIMEOUT at the next kb_sync, the device still usable */
  int32_t memint_compensated; /* KB_PREC_MIXED with memint_variant 2: 1 = the FP32 partial sums of each
                               * history tile are compensated (Kahan: four FP32 operations per term
                               * instead of one fma) before they join the FP64 accumulators; 0
                               * (default) plain FP32 tile partials of at most 32 terms. Kept by
                               * kb_autotune, which then times memint_variant 2 only */
  int32_t batch_overlap;      /* batches of two or more runs (no 1/N expansion): 0 (default) one
                               * launch per kernel for all runs; n > 0 splits the runs into two
                               * groups of about equal memory-integral work and runs the second
                               * group's sunset on n SMs (as many CTAs as fit there), on a second
                               * stream, while the first group's memory integrals stream (on the
                               * other SMs with memint_persistent); the same arithmetic per run */
  int32_t memint_persistent;  /* 1: the memory-integral grid is persistent -- one CTA per SM takes
                               * chunk items (whole or split) from a device counter until none are
                               * left, keeping its TMEM, stage barriers and the run's tadpole sum
                               * across items (the same arithmetic per item); 0 (default): one CTA
                               * per item. 1 needs memint_variant 1 or 2 in KB_PREC_MIXED */
} kb_tuning;
int kb_get_tuning(const kb_handle *h, kb_tuning *out);
int kb_set_tuning(kb_handle *h, const kb_tuning *in);
/* Autotuner: times every candidate configuration (memory-integral variants,
 * whole or split;
 * sunset variants with grids of 1..4 CTAs per SM that fit; the chosen memory-integral
 * kernel as a persistent grid; both run orders of a batched handle) by re-running the last evolved
 * step t -- which reads rows < t and rewrites row t, so the state is unchanged
 * -- `trials` times each, keeps the fastest kernel configurations, re-runs step
 * t once with them and returns the choice and its time per step (ms) if the
 * pointers are not NULL. Needs t >= 3. */
int kb_autotune(kb_handle *h, int32_t trials, kb_tuning *chosen, double *ms_per_step);

/* Gradient of a late-time loss by the discrete adjoint of the step. No
 * counterpart in the reference (its ChainRulesCore rrule would wrap this):
 *   L = sum_k w_n[k] n(k, t_final) + w_E E(t_final)
 * over orbits k (kb_get_orbits order), with n and E as kb_measure reports them
 * at t_final, for the run that kb_init(h, 0, n_init, init_mass) starts and
 * kb_step evolves to t_final (>= 3). Returns dL/dlambda, dL/dm^2 (kb_params.mass2),
 * dL/dn_init[k] for every orbit (S values) and, if grad_init_mass is not NULL,
 * dL/d init_mass at fixed n_init (chain it through the gap equation when
 * init_mass is the gap mass), and L itself in *loss if loss is not NULL.
 * w_n may be NULL (energy only).
 * Checkpointing: the forward run keeps a device copy of the state every
 * ckpt_every steps; the reverse sweep recomputes each block of ckpt_every steps
 * from its copy and runs the block's adjoint steps backwards. The handle must
 * hold one run in KB_PREC_FP64, created with (kb_params.flags & 0xffff) >=
 * ckpt_every. Memory: two more history rings plus
 * ceil((t_final - 2) / ckpt_every) state copies. The handle's state is
 * consumed: afterwards it needs kb_init before the next kb_step. */
int kb_adjoint(kb_handle *h, const double *n_init, double init_mass, int32_t t_final, const double *w_n, double w_E,
               int32_t ckpt_every, double *grad_lambda, double *grad_mass2, double *grad_n, double *grad_init_mass,
               double *loss);

/* Self-energies of caller-owned rows, allocating nothing. No counterpart in
 * the reference: it is for callers that cannot call cudaMalloc -- a host
 * whose device memory is owned by its own pool (a CUDA.jl or PyTorch caching
 * allocator that must stay the only allocator of the process), or a loop that
 * must not let an allocation synchronise the device. Computes Sigma_F and
 * Sigma_rho (FP64, the KB_PREC_FP64 sunset of kb_step) for nrows rows given on
 * the device in orbit order (row i = F(t-1, t'_i) / rho(t-1, t'_i), S values
 * each, rho sign-corrected), on `stream` (a cudaStream_t, NULL for the legacy
 * default stream). The transform scratch is one fixed device array of
 * 160 x 5308 doubles (6.8 MB) compiled into the library, held on every GPU
 * that loads it until the process exits, so Ns is limited to 1 or an even
 * value in [2, 32]; larger Ns fails with KB_ERR_PARAM and a message in
 * kb_last_error(NULL). The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture. Every call shares the array, so calls whose
 * kernels overlap on the GPU (other streams, other host threads) race; issue
 * them on one stream. Nothing in the array needs to start at zero. The looked-up
 * address is kept for the life of the process: a cudaDeviceReset (or any other
 * teardown of the device's primary context) invalidates it, so do not call this
 * entry point on a device after resetting it. */
int kb_sunset_rows_noalloc(int32_t Ns, int32_t N, double lambda, int32_t pexp, int32_t nrows, const double *F_rows,
                           const double *rho_rows, double *sigF_rows, double *sigr_rows, void *stream);

#ifdef __cplusplus
}
#endif
#endif
