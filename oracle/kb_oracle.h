/*
 * kb_oracle.h -- CPU FP64 restatement of the 2PI Kadanoff-Baym step of
 * magdalenaeriksson/QFTdynamicsM.jl src/TwoPIScalar (LambdaLO / LambdaNLO
 * quantum / LambdaNLO classical truncations of O(N) lambda phi^4).
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity checker for the CUDA
 * path (libkb2pi). Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it. The product never links or calls it.
 *
 * Parity status: the reference is Julia and no Julia toolchain exists on the
 * build or GPU machines, so the oracle cannot be compared with outputs of the
 * reference itself ("parity unpinned" against the reference's own numbers).
 * It is pinned instead against:
 *   - numpy's pocketfft rfftn/irfftn for the sunset self-energy, which is the
 *     same unnormalised rfft/brfft convention the reference uses through FFTW
 *     (tests/test_oracle.py);
 *   - the closed-form lambda = 0 solution of the leapfrog recurrence;
 *   - the reference's own analytic conserved energy of the Gauss initial state
 *     (src/TwoPIScalar/TwoPIScalar_Initialization.jl:109);
 *   - agreement of its three engines with each other (full lattice, orbit
 *     reduced with full-lattice FFTs, orbit reduced with octant cosine
 *     transforms).
 *
 * Engines:
 *   ORC_ENGINE_FULL   : CPUfull semantics. Two-time history of full Ns^sdim
 *                       lattices in a SymMatrix ring with the reference's
 *                       mod1 slots and thesign bookkeeping
 *                       (src/DefSimDataElements.jl:169-230), sunset by 3D FFT
 *                       (src/TwoPIScalar/TwoPIScalar_Evolution.jl:25-31).
 *   ORC_ENGINE_ORBIT  : CPUred semantics. History holds one value per cubic
 *                       orbit; the sunset scatters to the full lattice, uses
 *                       the same FFTs and gathers back (Evolution.jl:91-105,
 *                       DefSimDataElements.jl:71-83).
 *   ORC_ENGINE_OCTANT : orbit history, sunset by separable cosine transforms on
 *                       the even octant (mathematically identical for
 *                       cubic-symmetric data; fast enough for larger tests).
 */
#ifndef KB_ORACLE_H
#define KB_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_ENGINE_FULL = 0, ORC_ENGINE_ORBIT = 1, ORC_ENGINE_OCTANT = 2 };
/* TwoPIScalar_Problemdefinition.jl:34-45 (LambdaLO, LambdaNLOquantum/classical, NinverseLO/NLO) */
enum { ORC_PEXP_LO = 0, ORC_PEXP_NLO_QUANTUM = 1, ORC_PEXP_NLO_CLASSICAL = 2, ORC_PEXP_NINV_LO = 3,
       ORC_PEXP_NINV_NLO = 4 };

typedef struct orc_params {
  int32_t Ns;        /* disc.Nx */
  int32_t sdim;      /* disc.sdim (1..3) */
  int32_t M;         /* NstepsinMemory (>= 3) */
  int32_t N;         /* model.ONgroup */
  int32_t pexp;      /* ORC_PEXP_* */
  int32_t engine;    /* ORC_ENGINE_* */
  int32_t nthreads;  /* workers for the t' loops (splitter chunks) */
  int32_t pad_;
  double dt;         /* disc.dt */
  double lambda;     /* model.Lambda */
  double mass2;      /* model.Mass2: the m^2 used in the evolution */
  double mass;       /* disc.Mass: sets the time unit of measurements */
} orc_params;

typedef struct orc_scalars {
  double time, E, E_pot, E_kin, E_mem, M2;
} orc_scalars;

void *orc_create(const orc_params *p);
void orc_destroy(void *h);
/* cubic orbits: rep = sorted folded coordinates (3 per orbit, unused axes 0) */
int orc_num_orbits(void *h);
int64_t orc_num_sites(void *h);
void orc_orbits(void *h, int32_t *rep, double *k2, int64_t *deg);
void orc_site_orbit(void *h, int32_t *orbit_of_site);

/* initSimData! (TwoPIScalar_Initialization.jl:8-47) with n per orbit */
int orc_init_occupation(void *h, const double *n_orbit, double init_mass);
/* initSimData! for TwoPIScalarGauss (TwoPIScalar_Initialization.jl:95-112) */
int orc_init_gauss(void *h, double xi, double eta, double sig);
/* evolve! (TwoPIScalar_Evolution.jl:924-981) for time t */
int orc_step(void *h, int32_t t);
/* expandSimData! alone (TwoPIScalar_SimDataStruct.jl:262-300) */
int orc_expand(void *h);
/* calcSelfEnergies! alone for tmone (TwoPIScalar_Evolution.jl:16-31) */
int orc_self_energies(void *h, int32_t tmone);
/* createMeasurement (TwoPIScalar_Measurement.jl:31-99); arrays have S entries
 * (per orbit); Fonet/ronet/sigF/sigr are the traces at lattice site 1 with
 * up to M entries each (any of them may be NULL). */
int orc_measure(void *h, int32_t t, orc_scalars *s, double *F, double *ddF,
                double *n, double *omega, double *c, double *Fonet,
                double *ronet, double *sigF, double *sigr);
/* true two-time values on orbits (site average over the orbit for ENGINE_FULL) */
int orc_get(void *h, int32_t which /*0 F, 1 rho*/, int32_t a, int32_t b, double *out);
int orc_set(void *h, int32_t which, int32_t a, int32_t b, const double *in);
int orc_get_sigma(void *h, int32_t which /*0 SigF, 1 Sigr*/, int32_t z, double *out);
/* full lattice values (ENGINE_FULL only), column-major site order */
int orc_get_lattice(void *h, int32_t which, int32_t a, int32_t b, double *out);
int orc_window(void *h, int32_t *tmin, int32_t *tmax);
double orc_hartree_mass2(void *h, int32_t a, int32_t b);
double orc_hartree_prefactor(void *h);
/* wall seconds of the last orc_step: self-energies, and the rest of evolve! */
void orc_step_times(void *h, double *t_sunset, double *t_rest);
/* getGapMass (TwoPIScalar_Initialization.jl:250-266): Newton from x0 */
double orc_gap_mass(void *h, const double *n_orbit, double x0);

/* standalone sunset on one pair of orbit rows (for kernel parity tests):
 * sig_r, sig_F = Sigma_rho, Sigma_F of (F, rho) (rho already sign corrected) */
int orc_sunset_rows(void *h, const double *F, const double *rho, double *sig_F,
                    double *sig_r);

/* Forward-mode derivatives through a templated restatement of the orbit/octant
 * engine with dual numbers (the stand-in for ForwardDiff through the Julia
 * reference): L = sum_o w_n[o] n(o, t_final) + w_E E(t_final) for the run
 * orc_init_occupation(n_init, init_mass) + orc_step(3..t_final), and
 * dL[0] = dL/dlambda, dL[1] = dL/dm^2, dL[2] = sum_o dL/dn_init[o] dn[o].
 * sdim = 3; single-threaded; w_n and dn may be NULL. */
int orc_dual_loss(const orc_params *p, const double *n_init, double init_mass, int32_t t_final,
                  const double *w_n, double w_E, const double *dn, double *L, double *dL);

#ifdef __cplusplus
}
#endif
#endif
