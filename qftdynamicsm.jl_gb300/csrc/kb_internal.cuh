// kb_internal.cuh -- device data layout shared by the kernels of libkb2pi.
//
// Layout in HBM of one run (S orbits padded to nchunks * KC, KC = 8):
//   hist_F, hist_r  [nchunks][Malloc/T][Malloc/T][T][T][KC]  storage type TS, tile-major
//       element (a, b) with a >= b (later time first) in the time tile of
//       slots (slot(a) / T, slot(b) / T), at tile row slot(a) mod T and tile
//       column (slot(b) mod T) ^ (slot(a) mod 4); slot(t) = t mod Malloc,
//       Malloc = M rounded up to the tile T. Each T x T x KC tile is contiguous
//       (one bulk copy), and the XOR swizzle of columns keeps both row-wise and
//       column-wise shared-memory reads conflict-free. rho holds the true value
//       rho(a, b) of the later-first pair.
//   st_F, st_r      [3][nchunks][Malloc][KC]  double: rows t, t-1, t-2 by t mod 3
//       (the leapfrog state; in KB_PREC_MIXED the only FP64 copy of F, rho)
//   sig_F, sig_r    [nchunks][Malloc][KC]     TS: Sigma(t-1, z) at slot(z)
//   tad             [2][nchunks]              double: sum_k deg_k F(t,t,k) per chunk,
//                                              by t mod 2
//   meas            [5][Spad]                 double: F(t-1,t-1), ddF, n, omega, c
//   epart           [nchunks][4]              double: E_kin, E_pot, E_mem partials
//   rowacc          [MEMINT_MAX_PARTS][nchunks][Malloc][KC]  double: row sums of the memory
//                                              integrals (buffers past the first in split mode)
//   colacc          [2][nchunks][Malloc][KC]  double: column sums (F, rho) of a split step
//   fin, fin_part, fin_prev, hcm2             partial sums and arrival counts of the
//                                              finishing kernel of a split step
//   sunset scratch  [grid][R1 + R2]           double: FP64 cosine-transform intermediates
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace kb {

constexpr int KC = 8;  // orbits per chunk (innermost dimension)
constexpr int MEMINT_MAX_PARTS = 6;  // parts a split chunk's triangle is streamed in (row-sum buffers)

// device error bits (per handle)
enum : int { DEVERR_TIMEOUT = 1, DEVERR_SMEM = 2, DEVERR_GEOM = 4, DEVERR_BOUNDS = 8 };
// sites of the bounds checks of KB_DEBUG builds, bits 8.. of the error word
enum : int {
  DCHK_SUN_ROW = 1 << 8,     // sunset: t' outside [tmin, t-1] or its slot outside the ring
  DCHK_SUN_SIGMA = 1 << 9,   // sunset: Sigma ring index outside [0, nchunks Malloc KC)
  DCHK_MI_TILE = 1 << 10,    // memory integrals: time tile or Sigma slot outside the ring
  DCHK_MI_ROW = 1 << 11,     // memory integrals: row / column outside the window
  DCHK_LF_WRITE = 1 << 12,   // leapfrog: history or state-row write outside the ring
  DCHK_FIN = 1 << 13         // finishing kernel of a split step: item outside the window
};

// KB_DEBUG builds check ring, tile and Sigma indices on the device: a failed
// check ORs DEVERR_BOUNDS and its site into the handle's error word (RunDev.err)
// and the caller skips the access. Nothing traps; release builds compile the
// checks away (KB_DCHECK is true).
#ifdef KB_DEBUG
#define KB_DCHECK(cond, errp, site) (::kb::dcheck((cond), (errp), (site)))
#else
#define KB_DCHECK(cond, errp, site) (true)
#endif

struct RunDev {
  int Ns, H, S, nchunks;
  int M, Malloc, pexp, T;
  double dt, dt2, dt3, mass2;
  double pref_ivol;   // Hartreeprefactor * ivol
  double ivol;
  double fac_r, fac_F;  // ivol^3 * coefficient of Sigma_rho, Sigma_F
  double mass;
  void *hist_F, *hist_r;
  double *st_F, *st_r;
  void *sig_F, *sig_r;
  const double *k2, *deg;   // [Spad]
  const double *Cm;         // [H][H] octant cosine matrix
  double *tad;              // [2][nchunks]
  double *meas;             // [5][Spad]
  double *epart;            // [nchunks][4]
  double *rowacc;           // [MEMINT_MAX_PARTS][nchunks][Malloc][KC] row sums of the memory integrals (one per part when split)
  double *colacc;           // [2][nchunks][Malloc][KC] column sums F, rho of a split step
  int cta_base_sun, cta_base_mi;  // first item of this run in the batched grids
  int sun_rows;                   // t' rows per sunset item (taken one after the other), 1 for FP64
  int pad1;
  // 1/N expansion at NLO (pexp 4), FP64: bubble rings (layout of hist_F) and the
  // momentum-space resummed kernels I_k, J_k of the window ([Malloc][Spad])
  double *pi_r, *pi_F, *Ik, *Jk;
  double lam;       // lambda
  double ninv_fac;  // -lambda / (3 N) * ivol^2
  // finishing kernel of a split step (memint_finish_kernel): FIN_TP t' per CTA
  int *fin;          // [nchunks] CTAs of the chunk done this step (0 between steps)
  int fin_nb;        // CTA slots per chunk: ceil(Malloc / FIN_TP)
  int pad2;
  double *fin_part;  // [nchunks][fin_nb][KC] per-CTA sums of acc_F(t) terms
  double *fin_prev;  // [nchunks][KC] acc_F(t-1)
  double *hcm2;      // [2] hartreecont and M^2(t-1) of the step
  // tensor maps (CUtensorMap, 64-byte aligned, device memory) of hist_F and hist_r
  // as [tiles][T rows][T KC]: [0], [1] a tile per box, [2], [3] its lower T/2 rows;
  // null when the CUDA driver has no encoder
  const void *tmap;
  int *err;  // the handle's device error word (timeouts; bounds checks of KB_DEBUG builds)
  // the sunset kernel's shared-memory tables for this run's lattice size, built once per
  // handle (shared by the runs of the same Ns); null: the kernel builds them itself
  const unsigned char *sun_img;
};

#ifdef KB_DEBUG
__device__ inline bool dcheck(bool ok, int *err, int site) {
  if (!ok && err) atomicOr(err, DEVERR_BOUNDS | site);
  return ok;
}
#endif

// perturbative expansions (kb2pi.h): 0 LambdaLO, 1 LambdaNLO, 2 LambdaNLOclassical,
// 3 NinverseLO, 4 NinverseNLO
__host__ __device__ inline bool pexp_lo(int pexp) { return pexp == 0 || pexp == 3; }
__host__ __device__ inline bool pexp_sunset(int pexp) { return pexp == 1 || pexp == 2; }

__host__ __device__ inline long long tet3(int c) { return (long long)c * (c + 1) * (c + 2) / 6; }
__host__ __device__ inline int tri2(int b) { return b * (b + 1) / 2; }
// orbit index of the sorted triple a <= b <= c
__host__ __device__ inline int orb3(int a, int b, int c) { return (int)(tet3(c) + tri2(b) + a); }

// element offset of history entry (a, b) of orbit j of chunk c (see the layout above)
__host__ __device__ inline size_t hist_off(int Malloc, int T, int c, int a, int b, int j) {
  const int sa = a % Malloc, sb = b % Malloc, nbA = Malloc / T;
  const int ra = sa % T, cb = sb % T;
  return ((((size_t)c * nbA + sa / T) * nbA + sb / T) * T + ra) * (size_t)T * KC + (size_t)((cb ^ (ra & 3)) * KC + j);
}

// Batched grids: sched[0, nruns) is the first item (CTA or row) of each
// position, increasing; sched[nruns, 2 nruns) the run at that position.
__device__ inline int run_at(const int *sched, int nruns, int item) {
  int lo = 0, hi = nruns - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sched[mid] <= item) lo = mid; else hi = mid - 1;
  }
  return sched[nruns + lo];
}

// host launchers (kb_sunset.cu, kb_memint.cu)
// queue: item counter (zeroed here before the launch) or null for a fixed item order
cudaError_t launch_sunset(bool fp64, int variant, const RunDev *d_runs, const int *d_base, int nruns,
                          int total_rows, int grid, const int *d_t, void *scratch, size_t scratch_stride, size_t smem,
                          int *queue, cudaStream_t st);
size_t sunset_smem_bytes(bool fp64, int H);
size_t sunset_image_bytes(bool fp64, int H);
cudaError_t launch_sunset_image(bool fp64, int H, const double *Cm, void *img, cudaStream_t st);
// tensor-core sunset of KB_PREC_MIXED (kb_sunset_tc.cu): sunset variant 2
size_t sunset_tc_smem_bytes(int H);  // dynamic shared memory; 0 when H is beyond the kernel
size_t sunset_tc_static_bytes();
cudaError_t configure_sunset_tc(size_t max_block_smem);  // the device's per-block maximum
cudaError_t launch_sunset_tc(const RunDev *d_runs, const int *d_base, int nruns, int total_rows, int grid,
                             const int *d_t, size_t smem, cudaStream_t st);
int sunset_rows_per_item(int H);  // FP32: t' rows per sunset item
size_t sunset_scratch_elems(int H);
int sunset_grid(bool fp64, int num_sms, int total_rows);
int sunset_max_ctas_per_sm(bool fp64, int variant, size_t smem);
cudaError_t configure_sunset(bool fp64, size_t smem);
int memint_split_parts(int nwhole, int nsplit, int sm_slots);
cudaError_t launch_memint(bool fp64, int variant, int split, int nwhole, const RunDev *d_runs, const int *d_base,
                          int nruns, int total_ctas, int fin_nb_max, int use_maps, const int *d_t, int *d_err,
                          int measure, size_t smem, int *queue, int grid_cap, cudaStream_t st);
constexpr int FIN_TP = 128;  // t' per CTA of the finishing kernel
size_t memint_smem_bytes(bool fp64, int Malloc, int variant);
cudaError_t configure_memint(bool fp64, size_t smem);
int memint_tile(bool fp64);
cudaError_t launch_measure_init(const RunDev *d_runs, int nruns, int t, cudaStream_t st);
// n, omega, c of a run's measured step from its F(t-1,t-1) and ddF (before they are read)
cudaError_t launch_meas_derive(const RunDev *d_runs, int run, int S, cudaStream_t st);
cudaError_t launch_set_t(int *d_t, int t, cudaStream_t st);
cudaError_t launch_record(const RunDev *d_runs, int nruns, const int *d_t, const int *d_ctl, double *rec,
                          const long long *d_off, long long block, cudaStream_t st);
cudaError_t launch_advance_t(int *d_t, cudaStream_t st);
// 1/N NLO self-energies (kb_sunset.cu), FP64: bubbles of row t-1, resummed
// kernels per chunk, then Sigma(t-1, .)
size_t ninv_smem_bytes(int H);
size_t ninv_volterra_smem_bytes(int Malloc);
cudaError_t configure_ninv(size_t smem);
cudaError_t launch_ninv(const RunDev *d_runs, const int *d_sched_sun, const int *d_sched_mi, int nruns,
                        int total_rows, int total_ctas, int grid, const int *d_t, void *scratch, size_t scratch_stride,
                        size_t smem_rows, size_t smem_volterra, cudaStream_t st);
// adjoint of the sunset (kb_sunset.cu), FP64 handles only
size_t sunset_adjoint_smem_bytes(int H);
cudaError_t launch_sunset_adjoint(const RunDev &R, int t, const double *sbar_r, const double *sbar_F, double *adjF,
                                  double *adjR, double *lam_part, void *scratch, size_t stride, int grid,
                                  double lambda, cudaStream_t st);

// reverse sweep of kb_adjoint (kb_adjoint.cu), FP64 single-run handles
struct AdjBuffers {
  double *adjF, *adjR;  // adjoint history, the layout of hist_F / hist_r
  double *xbr, *xbF;    // [Malloc][Spad]: adjoints of x_rho(z), x_F(z), then of Sigma(t-1, z)
  double *accF, *accR;  // [Malloc][Spad]: adjoints of acc_F(t'), acc_rho(t')
  double *omb;          // [Spad]: adjoint of omega^2 dt^2
  double *lamp;         // [Malloc]: dL/dlambda of each sunset row
  double *scal;         // [8]: 0 M^2(t-1), 1 hartreecont, 2 dL/dm^2, 3 dL/dlambda
};
struct SunsetLaunch {  // the handle's forward sunset launch
  const RunDev *runs;
  const int *base;
  int nruns, total_rows, grid;
  int *d_t;
  void *scratch;
  size_t stride, smem;
};
size_t adjoint_buffer_bytes(const RunDev &R);
void adjoint_carve(const RunDev &R, void *base, AdjBuffers *A);
cudaError_t launch_adjoint_seed(const RunDev &R, const AdjBuffers &A, int t_final, const double *d_wn, double w_E,
                                double dpref_ivol, cudaStream_t st);
// sigma_ready: Sigma(t-1, .) is already in the rings (restored from the forward
// step t), so the forward sunset is not run again
cudaError_t launch_adjoint_step(const RunDev &R, const AdjBuffers &A, int t, double emem_weight, double lambda,
                                double dpref_ivol, const SunsetLaunch &sl, int num_sms, bool sigma_ready,
                                cudaStream_t st);
cudaError_t launch_adjoint_init_grad(const RunDev &R, const AdjBuffers &A, const double *d_n0, double init_mass,
                                     double *d_out, cudaStream_t st);
// message returned by kb_last_error(NULL) (kb_api.cu)
void kb_set_global_error(const char *msg);

}  // namespace kb
