// kb_adjoint.cu -- reverse mode (adjoint) of the KB step, FP64 handles.
//
// Gradient of L = sum_k w_n(k) n(k, t_f) + w_E E(t_f) with respect to lambda,
// m^2 and the initial occupation n_init(k) per orbit, for a run started by
// initSimData! (TwoPIScalar_Initialization.jl:8-47) and evolved with evolve!
// (TwoPIScalar_Evolution.jl:924-981). The reference has no derivative code;
// this is the discrete adjoint of exactly the step the library runs, so the
// gradient is that of the discretised dynamics.
//
// All adjoints are orbit adjoints: derivatives with respect to the single value
// an orbit stores for all of its sites. Reverse step t, given the forward
// history of step t:
//   1. refill the FP64 state row t-1 from the history and recompute M^2(t-1)
//      and Sigma(t-1, .) with the forward sunset kernel;
//   2. diagonal and leapfrog (Evolution.jl:890-915, 969-974): push the adjoint
//      of row t to rows t-1, t-2, to omega^2 dt^2 and to the memory integrals;
//   3. tadpole (getHartreeMass2): omega^2 -> M^2 -> m^2, lambda, F(t-1,t-1);
//   4. memory integrals: adjoints of x_rho(z), x_F(z) (row and column sums of
//      the history weighted by the acc adjoints) and of every history pair;
//   5. sunset adjoint (kb_sunset.cu): Sigma(t-1, .) -> F(t-1, .), rho(t-1, .);
//   6. clear the adjoint of row t.
// The forward memory-integral weights are x(z) = w(z) Sigma(t-1, z) with
// w(tmin) = 1/2 and acc_F(t') = sum_z x_rho(z) F(z,t') + sum_{z<t'} x_F(z) rho(t',z),
// acc_rho(t') = sum_{z>t'} x_rho(z) rho(z,t'); F(t,t') = (2 - om) F(t-1,t')
// - F(t-2,t') - dt^3 acc_F(t'), likewise rho; rho(t,t-1) = dt, rho(t,t) = 0.
#include <algorithm>
#include <cmath>

#include "kb_internal.cuh"

namespace kb {
namespace {

__device__ __forceinline__ double hF(const RunDev &R, int c, int a, int b, int j) {
  return reinterpret_cast<const double *>(R.hist_F)[hist_off(R.Malloc, R.T, c, a, b, j)];
}
__device__ __forceinline__ double hR(const RunDev &R, int c, int a, int b, int j) {
  return reinterpret_cast<const double *>(R.hist_r)[hist_off(R.Malloc, R.T, c, a, b, j)];
}
__device__ __forceinline__ int win_min(const RunDev &R, int t) { return max(1, t - R.M + 1); }

// block-wide sum in a fixed order (blockDim.x a multiple of 32, at most 1024)
__device__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  return s;
}

// FP64 state row t-1 from the history (the forward state ring only holds the
// last three rows of the forward run); the sunset reads its rows from there
__global__ void adj_refill_kernel(RunDev R, int t) {
  const int tmin = win_min(R, t), a = t - 1;
  const int n = a - tmin + 1, Spad = R.nchunks * KC;
  const size_t rowstride = (size_t)R.Malloc * KC;
  const size_t st_row = (size_t)R.nchunks * rowstride;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * Spad; i += gridDim.x * blockDim.x) {
    const int b = tmin + i / Spad, k = i % Spad;
    const int c = k / KC, j = k % KC;
    const size_t so = (size_t)(a % 3) * st_row + (size_t)c * rowstride + (size_t)(b % R.Malloc) * KC + j;
    R.st_F[so] = hF(R, c, a, b, j);
    R.st_r[so] = hR(R, c, a, b, j);
  }
}

// M^2(t-1) = m^2 + pref ivol sum_k deg_k F(t-1,t-1,k); one block
__global__ void adj_scalars_kernel(RunDev R, int t, AdjBuffers A) {
  __shared__ double red[32];
  double s = 0.0;
  for (int k = threadIdx.x; k < R.S; k += blockDim.x) s += R.deg[k] * hF(R, k / KC, t - 1, t - 1, k % KC);
  const double hc = block_sum(s, red);
  if (threadIdx.x == 0) {
    A.scal[0] = hc * R.pref_ivol + R.mass2;
    A.scal[1] = hc;
  }
}

// loss seeds at t_f (createMeasurement, TwoPIScalar_Measurement.jl:38-64 with
// the same branches as the forward measurement); one block
__global__ void adj_seed_kernel(RunDev R, int tf, AdjBuffers A, const double *wn, double wE, double dpref_ivol) {
  __shared__ double red[32];
  double s = 0.0;
  for (int k = threadIdx.x; k < R.S; k += blockDim.x) s += R.deg[k] * hF(R, k / KC, tf - 1, tf - 1, k % KC);
  const double hc = block_sum(s, red);
  const double dt2 = R.dt2;
  for (int k = threadIdx.x; k < R.S; k += blockDim.x) {
    const int c = k / KC, j = k % KC;
    const double Ftt = hF(R, c, tf, tf, j), Ft1 = hF(R, c, tf, tf - 1, j), Fmm = hF(R, c, tf - 1, tf - 1, j);
    const double dg = R.deg[k];
    const double ddF = (Ftt - 2 * Ft1 + Fmm) / dt2;
    // E_kin = 1/2 sum deg ddF; E_pot = 1/2 sum deg (m^2 + k^2 + 1/2 pref ivol hc) F
    double b_ddF = wE * 0.5 * dg;
    double b_F = wE * 0.5 * dg * (R.mass2 + R.k2[k] + R.pref_ivol * hc);
    // n = c sqrt(ddF F) - 1/2, c = sqrt(1 - dt^2 omega^2 / 4), omega^2 = ddF / F
    if (wn && ddF * Fmm > 0) {
      const double om2 = (ddF / Fmm > 0) ? ddF / Fmm : 0.0;
      const double w = wn[k];
      if (0.25 * dt2 * om2 < 1) {
        const double q = ddF * Fmm - 0.25 * dt2 * ddF * ddF;  // (c sqrt(ddF F))^2
        const double sq = sqrt(q);
        b_ddF += w * (Fmm - 0.5 * dt2 * ddF) / (2 * sq);
        b_F += w * ddF / (2 * sq);
      } else {
        const double sq = sqrt(ddF * Fmm);
        b_ddF += w * Fmm / (2 * sq);
        b_F += w * ddF / (2 * sq);
      }
    }
    A.adjF[hist_off(R.Malloc, R.T, c, tf, tf, j)] += b_ddF / dt2;
    A.adjF[hist_off(R.Malloc, R.T, c, tf, tf - 1, j)] += -2 * b_ddF / dt2;
    A.adjF[hist_off(R.Malloc, R.T, c, tf - 1, tf - 1, j)] += b_ddF / dt2 + b_F;
  }
  if (threadIdx.x == 0) {
    A.scal[2] += wE * 0.5 * hc;                     // dE_pot/dm^2
    A.scal[3] += wE * 0.25 * dpref_ivol * hc * hc;  // dE_pot/dlambda
  }
}

// diagonal and off-diagonal leapfrog adjoints. One CTA per orbit chunk, a thread
// per (orbit j, t') with j fastest (rows of the history and of the adjoint rings
// are KC-contiguous per t'), t' in blocks of ADJ_TPB. Every thread first adds the
// diagonal's terms into its element (t, t') of the adjoint of row t, then pushes
// that element to rows t-1, t-2. The one element two t' reach, (t-1, t-2), is
// updated by the thread of t' = t-2 alone, with the adjoint of (t, t-1) formed
// the same way from the values read before any update. The omega adjoint of an
// orbit is reduced over t' in a fixed order.
constexpr int ADJ_TPB = 32;  // 256 threads = KC orbits x 32 t'
__global__ void __launch_bounds__(KC * ADJ_TPB) adj_step_kernel(RunDev R, int t, AdjBuffers A, double emem_weight) {
  __shared__ double red[ADJ_TPB][KC];
  const int c = blockIdx.x;
  const int j = (int)threadIdx.x % KC, l = (int)threadIdx.x / KC;
  const int k = c * KC + j;
  const bool kv = k < R.S;
  const int tmin = win_min(R, t);
  const int Ma = R.Malloc, T = R.T, Spad = R.nchunks * KC;
  const double dt3 = R.dt3;
  double *aF = A.adjF, *aR = A.adjR;
  auto off = [&](int a, int b) { return hist_off(Ma, T, c, a, b, j); };
  const bool nlo = pexp_sunset(R.pexp);
  const double *sgr = reinterpret_cast<const double *>(R.sig_r) + (size_t)c * Ma * KC + j;
  const double *sgF = reinterpret_cast<const double *>(R.sig_F) + (size_t)c * Ma * KC + j;
  double om = 0.0, Fbtt = 0.0, b1 = 0.0;
  if (kv) {
    om = (R.k2[k] + A.scal[0]) * R.dt2;
    Fbtt = aF[off(t, t)];
    b1 = aF[off(t, t - 1)];  // before any thread of this orbit adds to it
  }
  __syncthreads();
  // diagonal F(t,t) = (2 - om) F(t,t-1) - F(t,t-2) - dt^3 sum_z [x_rho(z) F(t,z) + x_F(z) rho(t,z)]
  const double accd = -dt3 * Fbtt;
  // the adjoint of (t, t-1) once the diagonal has added to it
  double Fb1 = b1 + (2.0 - om) * Fbtt;
  if (nlo) Fb1 += ((t - 1 == tmin) ? 0.5 : 1.0) * sgr[(size_t)((t - 1) % Ma) * KC] * accd;
  double ob_sum = 0.0;
  for (int tp0 = tmin; tp0 <= t - 1; tp0 += ADJ_TPB) {
    const int tp = tp0 + l;
    if (!kv || tp > t - 1) continue;
    double Fb;
    if (tp == t - 1) {
      Fb = Fb1;
    } else {
      double v = aF[off(t, tp)];
      if (tp == t - 2) v -= Fbtt;
      if (nlo) v += ((tp == tmin) ? 0.5 : 1.0) * sgr[(size_t)(tp % Ma) * KC] * accd;
      Fb = v;
    }
    if (nlo) {
      const double w = (tp == tmin) ? 0.5 : 1.0;
      const size_t zo = (size_t)(tp % Ma) * Spad + k;
      aR[off(t, tp)] += w * sgF[(size_t)(tp % Ma) * KC] * accd;  // rho(t, t-1) = dt: a constant, never read
      A.xbr[zo] = hF(R, c, t, tp, j) * accd;
      A.xbF[zo] = hR(R, c, t, tp, j) * accd;
    }
    aF[off(t, tp)] = Fb;
    // off-diagonal t' = tp
    const double Rb = (tp <= t - 2) ? aR[off(t, tp)] : 0.0;  // rho(t, t-1) = dt is not evolved
    double accbF = -dt3 * Fb;
    if (tp == t - 1) accbF += emem_weight * 0.25 * R.dt * R.deg[k];  // E_mem = dt/4 sum_k deg acc_F(t-1)
    const size_t to = (size_t)(tp % Ma) * Spad + k;
    A.accF[to] = accbF;
    A.accR[to] = -dt3 * Rb;
    if (tp <= t - 2) {
      double v = aF[off(t - 1, tp)] + (2.0 - om) * Fb;
      if (tp == t - 2) v -= Fb1;  // F(t-2, t-1) is the stored F(t-1, t-2)
      aF[off(t - 1, tp)] = v;
      aF[off(t - 2, tp)] -= Fb;
    } else {
      aF[off(t - 1, tp)] += (2.0 - om) * Fb;
    }
    double ob = hF(R, c, t - 1, tp, j) * Fb;
    if (tp <= t - 2) {
      aR[off(t - 1, tp)] += (2.0 - om) * Rb;
      if (tp <= t - 3) aR[off(t - 2, tp)] -= Rb;  // rho(t-2, t-2) = 0
      ob += hR(R, c, t - 1, tp, j) * Rb;
    }
    ob_sum += ob;
  }
  red[l][j] = ob_sum;
  __syncthreads();
  if (l == 0 && kv) {
    double omb = -hF(R, c, t, t - 1, j) * Fbtt;
    for (int q = 0; q < ADJ_TPB; ++q) omb -= red[q][j];
    A.omb[k] = omb;
  }
}

// omega^2 dt^2 = (k^2 + M^2) dt^2 with M^2 = m^2 + pref ivol sum_k deg_k F(t-1,t-1); one block
__global__ void adj_tadpole_kernel(RunDev R, int t, AdjBuffers A, double dpref_ivol) {
  __shared__ double red[32];
  double s = 0.0;
  for (int k = threadIdx.x; k < R.S; k += blockDim.x) s += A.omb[k];
  const double Mb2 = R.dt2 * block_sum(s, red);
  if (threadIdx.x == 0) {
    A.scal[2] += Mb2;                           // d/dm^2
    A.scal[3] += Mb2 * A.scal[1] * dpref_ivol;  // d/dlambda through the Hartree prefactor
  }
  for (int k = threadIdx.x; k < R.S; k += blockDim.x)
    A.adjF[hist_off(R.Malloc, R.T, k / KC, t - 1, t - 1, k % KC)] += Mb2 * R.pref_ivol * R.deg[k];
}

// adjoints of x_rho(z), x_F(z), turned into those of Sigma(t-1, z) = x / w(z):
// one CTA per (orbit chunk, z), a thread per (time in a tile, orbit) with the
// orbit fastest; row z is read along its tile rows (b <= z), column z down the
// rows a > z; each orbit's partial sums are added over the CTA in a fixed order
constexpr int ADJ_RED_MAX_T = 32;
__global__ void adj_memint_reduce_kernel(RunDev R, int t, AdjBuffers A) {
  __shared__ double red[2][ADJ_RED_MAX_T][KC];
  const int tmin = win_min(R, t);
  const int Spad = R.nchunks * KC, Ma = R.Malloc, T = R.T;
  const int c = (int)blockIdx.x % R.nchunks, z = tmin + (int)blockIdx.x / R.nchunks;
  const int j = (int)threadIdx.x % KC, bl = (int)threadIdx.x / KC;
  const int k = c * KC + j;
  double sr = 0.0, sF = 0.0;
  if (k < R.S) {
    for (int b0 = (tmin / T) * T; b0 <= z; b0 += T) {  // acc_F(b) <- x_rho(z) F(z, b); acc_rho(b) <- x_rho(z) rho(z, b), b < z
      const int b = b0 + bl;
      if (b < tmin || b > z) continue;
      const size_t bo = (size_t)(b % Ma) * Spad + k;
      sr += hF(R, c, z, b, j) * A.accF[bo];
      if (b < z) sr += hR(R, c, z, b, j) * A.accR[bo];
    }
    for (int a0 = ((z + 1) / T) * T; a0 <= t - 1; a0 += T) {  // acc_F(a) <- x_rho(z) F(a, z) + x_F(z) rho(a, z)
      const int a = a0 + bl;
      if (a <= z || a > t - 1) continue;
      const size_t ao = (size_t)(a % Ma) * Spad + k;
      sr += hF(R, c, a, z, j) * A.accF[ao];
      sF += hR(R, c, a, z, j) * A.accF[ao];
    }
  }
  red[0][bl][j] = sr;
  red[1][bl][j] = sF;
  __syncthreads();
  if (bl == 0 && k < R.S) {
    double tr = 0.0, tF = 0.0;
    for (int q = 0; q < T; ++q) {
      tr += red[0][q][j];
      tF += red[1][q][j];
    }
    const size_t zo = (size_t)(z % Ma) * Spad + k;
    const double w = (z == tmin) ? 0.5 : 1.0;
    A.xbr[zo] = w * (A.xbr[zo] + tr);
    A.xbF[zo] = w * (A.xbF[zo] + tF);
  }
}

// adjoints of the history pairs (a >= b) of the window: one CTA per (orbit chunk,
// row a), a thread per (column of a time tile, orbit) with the orbit fastest, so a
// tile's row segment (T columns x KC orbits) is one contiguous access; the CTA
// walks the tiles of the columns b <= a
__global__ void adj_memint_update_kernel(RunDev R, int t, AdjBuffers A) {
  const int tmin = win_min(R, t);
  const int Spad = R.nchunks * KC, Ma = R.Malloc, T = R.T;
  const int c = (int)blockIdx.x % R.nchunks, a = tmin + (int)blockIdx.x / R.nchunks;
  const int j = (int)threadIdx.x % KC, bl = (int)threadIdx.x / KC;
  const int k = c * KC + j;
  if (a > t - 1 || k >= R.S) return;
  const double *sg_r = reinterpret_cast<const double *>(R.sig_r);
  const double *sg_F = reinterpret_cast<const double *>(R.sig_F);
  const size_t cb = (size_t)c * Ma * KC + j;
  const double xra = ((a == tmin) ? 0.5 : 1.0) * sg_r[cb + (size_t)(a % Ma) * KC];
  const double aFa = A.accF[(size_t)(a % Ma) * Spad + k];
  for (int b0 = (tmin / T) * T; b0 <= a; b0 += T) {
    const int b = b0 + bl;
    if (b < tmin || b > a) continue;
    const double xrb = ((b == tmin) ? 0.5 : 1.0) * sg_r[cb + (size_t)(b % Ma) * KC];
    const double xFb = ((b == tmin) ? 0.5 : 1.0) * sg_F[cb + (size_t)(b % Ma) * KC];
    const double aFb = A.accF[(size_t)(b % Ma) * Spad + k];
    const double aRb = A.accR[(size_t)(b % Ma) * Spad + k];
    const size_t o = hist_off(Ma, T, c, a, b, j);
    if (a > b) {
      A.adjF[o] += xra * aFb + xrb * aFa;
      A.adjR[o] += xFb * aFa + xra * aRb;
    } else {
      A.adjF[o] += xra * aFb;
    }
  }
}

// sum of the sunset rows' dL/dlambda partials in a fixed order
__global__ void adj_lambda_rows_kernel(RunDev R, int t, AdjBuffers A) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int z = win_min(R, t); z <= t - 1; ++z) s += A.lamp[z % R.Malloc];
  A.scal[3] += s;
}

__global__ void adj_zero_row_kernel(RunDev R, int t, AdjBuffers A) {
  const int tmin = win_min(R, t);
  const int n = t - tmin + 1, Spad = R.nchunks * KC;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * Spad; i += gridDim.x * blockDim.x) {
    const int b = tmin + i / Spad, k = i % Spad;
    const size_t o = hist_off(R.Malloc, R.T, k / KC, t, b, k % KC);
    A.adjF[o] = 0.0;
    A.adjR[o] = 0.0;
  }
}

// initSimData! (Initialization.jl:38-41): F(1,1) = F(2,1) = (n + 1/2)/omega,
// F(2,2) = omega (n + 1/2) dt^2 + (n + 1/2)/omega, omega = sqrt(k^2 + Mass^2)
__global__ void adj_init_grad_kernel(RunDev R, AdjBuffers A, const double *n0, double init_mass, double *out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= R.S) return;
  const int c = k / KC, j = k % KC;
  const double a11 = A.adjF[hist_off(R.Malloc, R.T, c, 1, 1, j)];
  const double a21 = A.adjF[hist_off(R.Malloc, R.T, c, 2, 1, j)];
  const double a22 = A.adjF[hist_off(R.Malloc, R.T, c, 2, 2, j)];
  const double om = sqrt(R.k2[k] + init_mass * init_mass), dt2 = R.dt2;
  out[k] = (a11 + a21) / om + a22 * (om * dt2 + 1 / om);
  const double np = n0[k] + 0.5;
  out[R.S + k] = np * ((a11 + a21) * (-1 / (om * om)) + a22 * (dt2 - 1 / (om * om))) * (init_mass / om);
}

int grid_for(long long n, int threads, int cap) {
  return (int)std::max<long long>(1, std::min<long long>(cap, (n + threads - 1) / threads));
}

}  // namespace

size_t adjoint_buffer_bytes(const RunDev &R) {
  const size_t Spad = (size_t)R.nchunks * KC, Ma = (size_t)R.Malloc;
  const size_t hist = (size_t)R.nchunks * Ma * Ma * KC;
  return (2 * hist + 4 * Ma * Spad + Spad + Ma + 8) * sizeof(double);
}

void adjoint_carve(const RunDev &R, void *base, AdjBuffers *A) {
  const size_t Spad = (size_t)R.nchunks * KC, Ma = (size_t)R.Malloc;
  const size_t hist = (size_t)R.nchunks * Ma * Ma * KC;
  double *p = reinterpret_cast<double *>(base);
  A->adjF = p; p += hist;
  A->adjR = p; p += hist;
  A->xbr = p; p += Ma * Spad;
  A->xbF = p; p += Ma * Spad;
  A->accF = p; p += Ma * Spad;
  A->accR = p; p += Ma * Spad;
  A->omb = p; p += Spad;
  A->lamp = p; p += Ma;
  A->scal = p;
}

cudaError_t launch_adjoint_seed(const RunDev &R, const AdjBuffers &A, int t_final, const double *d_wn, double w_E,
                                double dpref_ivol, cudaStream_t st) {
  adj_seed_kernel<<<1, 256, 0, st>>>(R, t_final, A, d_wn, w_E, dpref_ivol);
  return cudaGetLastError();
}

cudaError_t launch_adjoint_step(const RunDev &R, const AdjBuffers &A, int t, double emem_weight, double lambda,
                                double dpref_ivol, const SunsetLaunch &sl, int num_sms, bool sigma_ready,
                                cudaStream_t st) {
  const int tmin = std::max(1, t - R.M + 1), n = t - tmin, Spad = R.nchunks * KC;
  const int cap = 64 * std::max(1, num_sms);
  cudaError_t e = launch_set_t(sl.d_t, t, st);
  if (e != cudaSuccess) return e;
  adj_refill_kernel<<<grid_for((long long)n * Spad, 256, cap), 256, 0, st>>>(R, t);
  adj_scalars_kernel<<<1, 256, 0, st>>>(R, t, A);
  const bool nlo = pexp_sunset(R.pexp);
  if (nlo && !sigma_ready) {
    e = launch_sunset(true, 0, sl.runs, sl.base, sl.nruns, sl.total_rows, sl.grid, sl.d_t, sl.scratch, sl.stride,
                      sl.smem, nullptr, st);
    if (e != cudaSuccess) return e;
  }
  adj_step_kernel<<<R.nchunks, KC * ADJ_TPB, 0, st>>>(R, t, A, emem_weight);
  adj_tadpole_kernel<<<1, 256, 0, st>>>(R, t, A, dpref_ivol);
  if (nlo) {
    adj_memint_reduce_kernel<<<n * R.nchunks, R.T * KC, 0, st>>>(R, t, A);
    adj_memint_update_kernel<<<n * R.nchunks, R.T * KC, 0, st>>>(R, t, A);
    e = launch_sunset_adjoint(R, t, A.xbr, A.xbF, A.adjF, A.adjR, A.lamp, sl.scratch, sl.stride,
                              std::max(1, std::min(sl.grid, n)), lambda, st);
    if (e != cudaSuccess) return e;
    adj_lambda_rows_kernel<<<1, 32, 0, st>>>(R, t, A);
  }
  adj_zero_row_kernel<<<grid_for((long long)(n + 1) * Spad, 256, cap), 256, 0, st>>>(R, t, A);
  return cudaGetLastError();
}

cudaError_t launch_adjoint_init_grad(const RunDev &R, const AdjBuffers &A, const double *d_n0, double init_mass,
                                     double *d_out, cudaStream_t st) {
  adj_init_grad_kernel<<<(R.S + 127) / 128, 128, 0, st>>>(R, A, d_n0, init_mass, d_out);
  return cudaGetLastError();
}

}  // namespace kb
