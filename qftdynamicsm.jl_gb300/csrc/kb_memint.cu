// kb_memint.cu -- memory integrals, leapfrog and diagonal of one KB step.
//
// Replaces the threaded t' loop of evolve! (src/TwoPIScalar/
// TwoPIScalar_Evolution.jl:950-974): getRHS_r!/getRHS_F! (:766-782, :846-854),
// evolve_r!/evolve_F! (:890-915), the diagonal F(t,t) (:969-974),
// setomega2values! with the tadpole mass getHartreeMass2(t-1,t-1)
// (:918-921, TwoPIScalar_Initialization.jl:207-229) and the per-orbit part of
// createMeasurement (TwoPIScalar_Measurement.jl:31-64, 135-197).
//
// With x_rho(z) = w(z) Sigma_rho(t-1,z), x_F(z) = w(z) Sigma_F(t-1,z),
// w(tmin) = 1/2 (trapezoid cut), w = 1 otherwise, the reference's sums are
//   R_F(t')   = -acc_F(t'),   acc_F(t') = sum_z x_rho(z) F(z,t') + sum_{z<t'} x_F(z) rho(t',z)
//   R_rho(t') = -acc_r(t'),   acc_r(t') = sum_{z>t'} x_rho(z) rho(z,t')
// over z in [tmin, t-1] (Sigma_rho(t-1,t-1) = 0 exactly, so the upper limits
// t-2 of the reference are included at no cost). Every stored pair (a > b) of
// the two-time triangle then feeds two rows at once:
//   F(a,b):   acc_F(b) += x_rho(a) F      acc_F(a) += x_rho(b) F
//   rho(a,b): acc_r(b) += x_rho(a) rho    acc_F(a) += x_F(b) rho
// and the diagonal pair F(a,a) feeds acc_F(a) once. One CTA owns KC = 8 orbits
// (a "chunk") and sweeps the whole triangle of its chunk exactly once, in
// T x T time tiles streamed from HBM by TMA bulk copies into a shared-memory
// ring: column sums stay in registers, row sums are reduced across threads
// into a shared accumulator. When a column block is complete its leapfrog
// runs at once, and after the last block the CTA computes the diagonal
// F(t,t), its tadpole partial sum and the measurement of its orbits. No data
// leaves the CTA except the new row, so the whole step needs no grid barrier.
#include <cstdio>

#include "kb_internal.cuh"

namespace kb {
namespace {

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + bulk asynchronous copy (TMA) global -> shared
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait: gives up after ~2 s of wall time (or 2^30 polls).
__device__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t it = 0; it < (1u << 30); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0 && globaltimer_ns() - t0 > 2000000000ull) return false;
  }
  return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <typename TS, int T_, int NST_>
struct Cfg {
  static constexpr int T = T_;
  static constexpr int NST = NST_;
  static constexpr int NT = T * KC;       // threads: one per (column b, orbit j)
  static constexpr int NW = NT / 32;
  static constexpr int LPJ = 32 / KC;     // columns per warp
  static constexpr int RPT = T / LPJ;     // rows per thread after the warp reduce-scatter
  static constexpr int TILE = T * T * KC; // elements of one field tile
  static constexpr int XROW = T * KC;
  static constexpr int STAGE = 2 * TILE + XROW;
  static constexpr uint32_t STAGE_BYTES = STAGE * sizeof(TS);
  static constexpr size_t RED_BYTES = ((size_t)NW * T * KC * sizeof(TS) + 15) / 16 * 16;
  static_assert((T * KC * sizeof(TS)) % 16 == 0, "bulk copies need 16-byte multiples");
  static_assert(T <= 32, "one tile row per lane of the issuing warp");
};

template <typename C>
__host__ __device__ constexpr size_t smem_fixed_bytes() {
  // stages + double-buffered row-reduction buffer + full/empty barriers + small scratch
  return (size_t)C::NST * C::STAGE_BYTES + 2 * C::RED_BYTES + 2 * C::NST * 8 + 128 * 8 + 16;
}

// Time tile iterator over the triangle: J = column block, I = row block >= J.
struct TileIt {
  int I, J, Jn;
  __device__ void next() {
    if (I < Jn) {
      ++I;
    } else {
      ++J;
      I = J;
    }
  }
};

// issued by the producer warp: the T row segments of the F and rho tiles and
// the Sigma_rho values of the tile's rows, all into one stage
template <typename TS, typename C>
__device__ __forceinline__ void issue_tile(int stage, int I, int J, const RunDev &R, int c, TS *stages,
                                           uint64_t *full) {
  const int lane = threadIdx.x & 31;
  uint64_t *bar = full + stage;
  if (lane == 0) mbar_expect_tx(bar, C::STAGE_BYTES);
  __syncwarp();
  TS *dst = stages + (size_t)stage * C::STAGE;
  const int sa0 = (I * C::T) % R.Malloc;  // Malloc is a multiple of T: rows stay contiguous
  const int sb0 = (J * C::T) % R.Malloc;
  const TS *hF = reinterpret_cast<const TS *>(R.hist_F);
  const TS *hR = reinterpret_cast<const TS *>(R.hist_r);
  if (lane < C::T) {
    const size_t off = (((size_t)c * R.Malloc + sa0 + lane) * R.Malloc + sb0) * KC;
    bulk_g2s(dst + lane * C::T * KC, hF + off, C::T * KC * sizeof(TS), bar);
    bulk_g2s(dst + C::TILE + lane * C::T * KC, hR + off, C::T * KC * sizeof(TS), bar);
  }
  if (lane == 0) {
    const TS *sg = reinterpret_cast<const TS *>(R.sig_r) + ((size_t)c * R.Malloc + sa0) * KC;
    bulk_g2s(dst + 2 * C::TILE, sg, C::XROW * sizeof(TS), bar);
  }
}

__device__ __forceinline__ void consumer_sync(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// Block = NT consumer threads (one per column b and orbit j of a tile) + one
// producer warp that streams tiles through an NST-deep ring of shared-memory
// stages guarded by full (TMA transaction count) and empty (consumer release)
// mbarriers. Consumers synchronise once per tile (named barrier 1) for the
// cross-thread row reduction; the producer never joins it.
template <typename TS, int T, int NST>
__global__ void __launch_bounds__(T *KC + 32)
memint_kernel(const RunDev *__restrict__ runs, const int *__restrict__ base, int nruns,
              const int *__restrict__ d_t, int *__restrict__ d_err, int measure) {
  using C = Cfg<TS, T, NST>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TS *stages = reinterpret_cast<TS *>(smem_raw);
  TS *redbuf = reinterpret_cast<TS *>(smem_raw + (size_t)NST * C::STAGE_BYTES);  // 2 x [NW][T][KC]
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + (size_t)NST * C::STAGE_BYTES + 2 * C::RED_BYTES);
  uint64_t *empty = full + NST;
  // misc: [0] hartreecont, [1] M^2, [2..2+KC) acc_F(t-1) per orbit, [10] abort flag,
  // [11] tiles issued, [12] consumer abort flag, [16..16+NW*KC) diagonal partials
  double *misc = reinterpret_cast<double *>(empty + NST);  // 128 doubles
  volatile int *abort_flag = reinterpret_cast<volatile int *>(misc + 10);
  volatile int *issued_count = reinterpret_cast<volatile int *>(misc + 11);
  // consumers leave the tile loop together: the flag is only written by
  // consumers before the named barrier and read by them after it
  volatile int *cabort = reinterpret_cast<volatile int *>(misc + 12);
  static_assert(16 + C::NW * KC <= 128, "misc scratch too small");

  const int r = find_run(base, nruns, blockIdx.x);
  const RunDev &R = runs[r];
  const int c = blockIdx.x - R.cta_base_mi;  // chunk
  const int tid = threadIdx.x;
  const bool producer = tid >= C::NT;
  const int j = tid % KC, bl = tid / KC;
  const int lane = tid & 31, warp = tid >> 5;
  const int t = *d_t;
  const int M = R.M, Ma = R.Malloc;
  const int tmin = max(1, t - M + 1);
  const size_t rowstride = (size_t)Ma * KC;              // one row of one chunk
  const size_t st_row = (size_t)R.nchunks * rowstride;   // one state row (all chunks)
  const int k = c * KC + j;                              // orbit of this thread
  // row sums of this chunk, [Malloc][KC]: entry (slot, j) is only ever touched
  // by consumer thread (slot mod T, j) -- row a is reduced by thread bl = a mod T
  // and column b = a is finalised by the same thread -- so it needs no
  // synchronisation; it lives in a global scratch slot that stays in L2.
  double *rowacc = R.rowacc + (size_t)c * rowstride;

  // --- tadpole mass M^2(t-1) from the per-chunk sums of F(t-1,t-1) (fixed order)
  if (warp == 0) {
    const double *tad = R.tad + (size_t)((t - 1) & 1) * R.nchunks;
    double s = 0.0;
    for (int q = lane; q < R.nchunks; q += 32) s += tad[q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      misc[0] = s;                          // hartreecont = sum_k deg_k F(t-1,t-1,k)
      misc[1] = s * R.pref_ivol + R.mass2;  // getHartreeMass2 order: (sum * (pref*ivol)) + Mass2
    }
  }
  if (tid < KC) misc[2 + tid] = 0.0;
  if (tid == 0) {
    *abort_flag = 0;
    *issued_count = 0;
    *cabort = 0;
    for (int q = 0; q < NST; ++q) {
      mbar_init(full + q, 1);
      mbar_init(empty + q, 1);
    }
    fence_proxy_async();
  }
  if (!producer)
    for (int q = tid; q < Ma * KC; q += C::NT) rowacc[q] = 0.0;  // entries owned by this thread
  __syncthreads();
  const double hc = misc[0], M2 = misc[1];

  const bool lo_only = (R.pexp == 0);
  const int J0 = tmin / T, Jn = (t - 1) / T;
  const int nb = Jn - J0 + 1;
  const int ntiles = lo_only ? 0 : nb * (nb + 1) / 2;

  if (producer) {
    // ---------------- producer warp: stream every tile of the triangle once
    TileIt it{J0, J0, Jn};
    for (int n = 0; n < ntiles; ++n, it.next()) {
      const int stage = n % NST;
      if (n >= NST && !mbar_wait_bounded(empty + stage, (uint32_t)(((n / NST) - 1) & 1))) {
        if (lane == 0) {
          *abort_flag = 1;
          atomicOr(d_err, DEVERR_TIMEOUT);
        }
        break;
      }
      if (*abort_flag) break;
      issue_tile<TS, C>(stage, it.I, it.J, R, c, stages, full);
      if (lane == 0) *issued_count = n + 1;
    }
    __syncwarp();
  } else {
    // ---------------- consumers
    const double dt3 = R.dt3;
    const double kk = (k < R.S) ? R.k2[k] : 0.0;
    const double om = (kk + M2) * R.dt2;  // setomega2values!: (kL2 + M^2) * dt^2
    const double *F1row = R.st_F + (size_t)((t - 1) % 3) * st_row + (size_t)c * rowstride;
    const double *F2row = R.st_F + (size_t)((t - 2) % 3) * st_row + (size_t)c * rowstride;
    const double *R1row = R.st_r + (size_t)((t - 1) % 3) * st_row + (size_t)c * rowstride;
    const double *R2row = R.st_r + (size_t)((t - 2) % 3) * st_row + (size_t)c * rowstride;
    double *FNrow = R.st_F + (size_t)(t % 3) * st_row + (size_t)c * rowstride;
    double *RNrow = R.st_r + (size_t)(t % 3) * st_row + (size_t)c * rowstride;
    TS *hFnew = reinterpret_cast<TS *>(R.hist_F) + ((size_t)c * Ma + (t % Ma)) * rowstride;
    TS *hRnew = reinterpret_cast<TS *>(R.hist_r) + ((size_t)c * Ma + (t % Ma)) * rowstride;
    const TS *sigr = reinterpret_cast<const TS *>(R.sig_r) + (size_t)c * rowstride;
    const TS *sigF = reinterpret_cast<const TS *>(R.sig_F) + (size_t)c * rowstride;

    double diag = 0.0;  // acc_F(t) for the diagonal, partial over this thread's columns
    double emem = 0.0;  // acc_F(t-1), kept by the thread of column t-1
    bool has_emem = false;
    bool aborted = false;
    int n = 0;  // tiles consumed

    for (int J = J0; J <= Jn && !aborted; ++J) {
      const int b = J * T + bl;
      const bool bvalid = (b >= tmin) && (b <= t - 1);
      const double wb = (b == tmin) ? 0.5 : 1.0;
      const double xbr_d = (bvalid && !lo_only) ? wb * (double)sigr[(size_t)(b % Ma) * KC + j] : 0.0;
      const double xbF_d = (bvalid && !lo_only) ? wb * (double)sigF[(size_t)(b % Ma) * KC + j] : 0.0;
      const TS xbr = (TS)xbr_d, xbF = (TS)xbF_d;
      double colF = 0.0, colR = 0.0;

      for (int I = lo_only ? Jn + 1 : J; I <= Jn; ++I, ++n) {
        const int stage = n % NST;
        if (!mbar_wait_bounded(full + stage, (uint32_t)((n / NST) & 1))) {
          *abort_flag = 1;  // stops the producer
          *cabort = 1;
          atomicOr(d_err, DEVERR_TIMEOUT);
        }
        const TS *tF = stages + (size_t)stage * C::STAGE;
        const TS *tR = tF + C::TILE;
        const TS *sx = tF + 2 * C::TILE;

        TS cF0 = 0, cF1 = 0, cR0 = 0, cR1 = 0;
        TS rp[T];
        const bool interior = (I > J) && (J * T >= tmin) && (I * T + T - 1 <= t - 1);
        if (interior) {
#pragma unroll
          for (int rr = 0; rr < T; rr += 2) {
            const TS xa0 = sx[rr * KC + j], xa1 = sx[(rr + 1) * KC + j];
            const TS f0 = tF[(rr * T + bl) * KC + j], f1 = tF[((rr + 1) * T + bl) * KC + j];
            const TS q0 = tR[(rr * T + bl) * KC + j], q1 = tR[((rr + 1) * T + bl) * KC + j];
            cF0 += xa0 * f0;
            cR0 += xa0 * q0;
            cF1 += xa1 * f1;
            cR1 += xa1 * q1;
            rp[rr] = xbr * f0 + xbF * q0;
            rp[rr + 1] = xbr * f1 + xbF * q1;
          }
        } else {
#pragma unroll
          for (int rr = 0; rr < T; ++rr) {
            const int a = I * T + rr;
            const bool av = (a >= tmin) && (a <= t - 1);
            const TS wa = (a == tmin) ? (TS)0.5 : (TS)1;
            const TS xa = av ? sx[rr * KC + j] * wa : (TS)0;
            const bool ok = av && bvalid && (b <= a);
            const TS f = ok ? tF[(rr * T + bl) * KC + j] : (TS)0;
            const TS q = ok ? tR[(rr * T + bl) * KC + j] : (TS)0;
            if (rr & 1) {
              cF1 += xa * f;
              cR1 += xa * q;
            } else {
              cF0 += xa * f;
              cR0 += xa * q;
            }
            rp[rr] = (ok && b < a) ? xbr * f + xbF * q : (TS)0;
          }
        }
        colF += (double)(cF0 + cF1);
        colR += (double)(cR0 + cR1);

        // reduce-scatter rp over the LPJ columns of this warp that share orbit j
        int row0 = 0;
#pragma unroll
        for (int o = 16, half = T / 2; o >= KC; o >>= 1, half >>= 1) {
          const bool hi = (lane & o) != 0;
#pragma unroll
          for (int i = 0; i < half; ++i) {
            const TS a0 = rp[i], a1 = rp[i + half];
            const TS send = hi ? a0 : a1;
            const TS keep = hi ? a1 : a0;
            rp[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
          }
          if (hi) row0 += half;
        }
        TS *red = redbuf + (size_t)(n & 1) * (C::RED_BYTES / sizeof(TS));
#pragma unroll
        for (int i = 0; i < C::RPT; ++i) red[((size_t)warp * T + row0 + i) * KC + j] = rp[i];
        consumer_sync(C::NT);  // every consumer is done with the stage and has written red
        if (tid == 0) mbar_arrive(empty + stage);
        {
          // thread (rr = bl, j): add the CTA-wide row sum of row a = I*T + bl
          const int a = I * T + bl;
          TS sum = 0;
#pragma unroll
          for (int w = 0; w < C::NW; ++w) sum += red[((size_t)w * T + bl) * KC + j];
          if (a >= tmin && a <= t - 1) rowacc[(size_t)(a % Ma) * KC + j] += (double)sum;
        }
        if (*cabort) {
          aborted = true;
          break;
        }
      }
      if (aborted) break;

      // leapfrog for t' = b (evolve_r!/evolve_F!, Evolution.jl:890-915); rowacc of
      // row b was last written by this same thread
      if (bvalid) {
        const int sb = b % Ma;
        const double accF = colF + rowacc[(size_t)sb * KC + j];
        const double accR = colR;
        const double F1 = F1row[(size_t)sb * KC + j];
        const double F2 = (b <= t - 2) ? F2row[(size_t)sb * KC + j] : F1row[(size_t)((t - 2) % Ma) * KC + j];
        const double Fn = (2.0 - om) * F1 - F2 - accF * dt3;
        double rn;
        if (b == t - 1) {
          rn = R.dt;  // phi-pi commutator rho(t, t-1) = dt
        } else {
          const double r1 = R1row[(size_t)sb * KC + j];
          const double r2 = R2row[(size_t)sb * KC + j];
          rn = (2.0 - om) * r1 - r2 - accR * dt3;
        }
        FNrow[(size_t)sb * KC + j] = Fn;
        RNrow[(size_t)sb * KC + j] = rn;
        hFnew[(size_t)sb * KC + j] = (TS)Fn;
        hRnew[(size_t)sb * KC + j] = (TS)rn;
        diag += xbr_d * Fn + xbF_d * rn;
        if (b == t - 1) {
          emem = accF;
          has_emem = true;
        }
      }
    }
    if (!aborted) {
      // partial sums of acc_F(t) over this warp's columns
      double v = diag;
#pragma unroll
      for (int o = 16; o >= KC; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane < KC) misc[16 + warp * KC + lane] = v;
      if (has_emem) misc[2 + j] = emem;
    }
  }
  __syncthreads();  // producer done issuing; consumers done with the triangle
  if (*abort_flag) {
    // drain copies still in flight into this CTA's shared memory, then leave
    if (tid == 0)
      for (int q = 0; q < *issued_count; ++q)
        (void)mbar_wait_bounded(full + (q % NST), (uint32_t)((q / NST) & 1));
    __syncthreads();
    return;
  }

  // --- diagonal F(t,t) (Evolution.jl:969-974)
  if (tid < KC) {
    const double *F1row = R.st_F + (size_t)((t - 1) % 3) * st_row + (size_t)c * rowstride;
    double *FNrow = R.st_F + (size_t)(t % 3) * st_row + (size_t)c * rowstride;
    double *RNrow = R.st_r + (size_t)(t % 3) * st_row + (size_t)c * rowstride;
    TS *hFnew = reinterpret_cast<TS *>(R.hist_F) + ((size_t)c * Ma + (t % Ma)) * rowstride;
    TS *hRnew = reinterpret_cast<TS *>(R.hist_r) + ((size_t)c * Ma + (t % Ma)) * rowstride;
    double accd = 0.0;
    for (int w = 0; w < C::NW; ++w) accd += misc[16 + w * KC + tid];
    const int jj = tid;
    const int kd = c * KC + jj;
    const double kd2 = (kd < R.S) ? R.k2[kd] : 0.0;
    const double omd = (kd2 + M2) * R.dt2;
    const double Ft1 = FNrow[(size_t)((t - 1) % Ma) * KC + jj];  // F(t, t-1)
    const double Ft2 = FNrow[(size_t)((t - 2) % Ma) * KC + jj];  // F(t, t-2)
    const double Ftt = (2.0 - omd) * Ft1 - Ft2 - accd * R.dt3;
    FNrow[(size_t)(t % Ma) * KC + jj] = Ftt;
    RNrow[(size_t)(t % Ma) * KC + jj] = 0.0;
    hFnew[(size_t)(t % Ma) * KC + jj] = (TS)Ftt;
    hRnew[(size_t)(t % Ma) * KC + jj] = (TS)0;
    const double dg = (kd < R.S) ? R.deg[kd] : 0.0;
    double tp = dg * Ftt;  // tadpole partial sum of this chunk for the next step
    // measurement (createMeasurement, Measurement.jl:38-64): F(t-1,t-1) from the state
    const double Fmm = F1row[(size_t)((t - 1) % Ma) * KC + jj];
    const double dt = R.dt, dt2 = R.dt2;
    const double ddF = (Ftt - 2 * Ft1 + Fmm) / dt2;
    const double omg = (ddF / Fmm > 0) ? sqrt(ddF / Fmm) : 0.0;
    const double cc = (0.25 * dt2 * (omg * omg) < 1) ? sqrt(1. - 0.25 * dt2 * (omg * omg)) : 1.0;
    const double nn = (ddF * Fmm > 0) ? (cc * sqrt(ddF * Fmm)) - 0.5 : 0.0;
    double ek = 0.5 * ddF * dg;
    double ep = 0.5 * (R.mass2 + kd2 + 0.5 * R.pref_ivol * hc) * Fmm * dg;
    double em = 0.25 * dt * dg * misc[2 + jj];
    if (kd < R.S && measure) {
      const int Sp = R.nchunks * KC;
      R.meas[0 * Sp + kd] = Fmm;
      R.meas[1 * Sp + kd] = ddF;
      R.meas[2 * Sp + kd] = nn;
      R.meas[3 * Sp + kd] = omg;
      R.meas[4 * Sp + kd] = cc;
    }
    // fixed-order reduction over the KC orbits (lanes 0..KC-1 of warp 0)
#pragma unroll
    for (int o = KC / 2; o > 0; o >>= 1) {
      tp += __shfl_xor_sync((1u << KC) - 1, tp, o);
      ek += __shfl_xor_sync((1u << KC) - 1, ek, o);
      ep += __shfl_xor_sync((1u << KC) - 1, ep, o);
      em += __shfl_xor_sync((1u << KC) - 1, em, o);
    }
    if (jj == 0) {
      R.tad[(size_t)(t & 1) * R.nchunks + c] = tp;
      if (measure) {
        R.epart[(size_t)c * 4 + 0] = ek;
        R.epart[(size_t)c * 4 + 1] = ep;
        R.epart[(size_t)c * 4 + 2] = em;
        R.epart[(size_t)c * 4 + 3] = M2;
      }
    }
  }
}

// t = 2 measurement after initSimData! (Measurement.jl:31-64 with E_mem = 0):
// one CTA per run, M^2 = getHartreeMass2(2,2) as the reference stores it.
__global__ void measure_init_kernel(const RunDev *__restrict__ runs, int nruns, int t) {
  const RunDev &R = runs[blockIdx.x];
  const size_t rowstride = (size_t)R.Malloc * KC;
  const size_t st_row = (size_t)R.nchunks * rowstride;
  const int Ma = R.Malloc;
  __shared__ double red[4][256];
  double s_tad = 0, s_hc = 0;
  for (int kd = threadIdx.x; kd < R.S; kd += blockDim.x) {
    const int c = kd / KC, jj = kd % KC;
    const double *Ft = R.st_F + (size_t)(t % 3) * st_row + c * rowstride;
    const double *Fm = R.st_F + (size_t)((t - 1) % 3) * st_row + c * rowstride;
    const double dg = R.deg[kd];
    s_tad += dg * Ft[(size_t)(t % Ma) * KC + jj];
    s_hc += dg * Fm[(size_t)((t - 1) % Ma) * KC + jj];
  }
  red[0][threadIdx.x] = s_tad;
  red[1][threadIdx.x] = s_hc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  const double M2 = red[0][0] * R.pref_ivol + R.mass2;
  const double hc = red[1][0];
  __syncthreads();
  double ek = 0, ep = 0;
  const int Sp = R.nchunks * KC;
  for (int kd = threadIdx.x; kd < R.S; kd += blockDim.x) {
    const int c = kd / KC, jj = kd % KC;
    const double *Ft = R.st_F + (size_t)(t % 3) * st_row + c * rowstride;
    const double *Fm = R.st_F + (size_t)((t - 1) % 3) * st_row + c * rowstride;
    const double Ftt = Ft[(size_t)(t % Ma) * KC + jj];
    const double Fmt = Ft[(size_t)((t - 1) % Ma) * KC + jj];
    const double Fmm = Fm[(size_t)((t - 1) % Ma) * KC + jj];
    const double dt2 = R.dt2;
    const double ddF = (Ftt - 2 * Fmt + Fmm) / dt2;
    const double omg = (ddF / Fmm > 0) ? sqrt(ddF / Fmm) : 0.0;
    const double cc = (0.25 * dt2 * (omg * omg) < 1) ? sqrt(1. - 0.25 * dt2 * (omg * omg)) : 1.0;
    const double nn = (ddF * Fmm > 0) ? (cc * sqrt(ddF * Fmm)) - 0.5 : 0.0;
    const double dg = R.deg[kd];
    R.meas[0 * Sp + kd] = Fmm;
    R.meas[1 * Sp + kd] = ddF;
    R.meas[2 * Sp + kd] = nn;
    R.meas[3 * Sp + kd] = omg;
    R.meas[4 * Sp + kd] = cc;
    ek += 0.5 * ddF * dg;
    ep += 0.5 * (R.mass2 + R.k2[kd] + 0.5 * R.pref_ivol * hc) * Fmm * dg;
  }
  red[0][threadIdx.x] = ek;
  red[1][threadIdx.x] = ep;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int c = 0; c < R.nchunks; ++c)
      for (int q = 0; q < 4; ++q) R.epart[(size_t)c * 4 + q] = 0.0;
    R.epart[0] = red[0][0];
    R.epart[1] = red[1][0];
    R.epart[3] = M2;
    // tadpole partial of F(2,2) for the first step, by chunk
  }
  for (int c = threadIdx.x; c < R.nchunks; c += blockDim.x) {
    double s = 0;
    const double *Ft = R.st_F + (size_t)(t % 3) * st_row + c * rowstride;
    for (int jj = 0; jj < KC; ++jj) {
      const int kd = c * KC + jj;
      if (kd < R.S) s += R.deg[kd] * Ft[(size_t)(t % Ma) * KC + jj];
    }
    R.tad[(size_t)(t & 1) * R.nchunks + c] = s;
  }
}

__global__ void set_t_kernel(int *d_t, int t) { *d_t = t; }
__global__ void advance_t_kernel(int *d_t) { *d_t += 1; }

using CfgF64 = Cfg<double, 16, 4>;
using CfgF32 = Cfg<float, 32, 3>;

}  // namespace

int memint_tile(bool fp64) { return fp64 ? CfgF64::T : CfgF32::T; }

size_t memint_smem_bytes(bool fp64, int Malloc) {
  (void)Malloc;
  return fp64 ? smem_fixed_bytes<CfgF64>() : smem_fixed_bytes<CfgF32>();
}

cudaError_t configure_memint(bool fp64, size_t smem) {
  if (fp64)
    return cudaFuncSetAttribute(memint_kernel<double, CfgF64::T, CfgF64::NST>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaFuncSetAttribute(memint_kernel<float, CfgF32::T, CfgF32::NST>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_memint(bool fp64, const RunDev *d_runs, const int *d_base, int nruns, int total_ctas,
                          const int *d_t, int *d_err, int measure, size_t smem, cudaStream_t st) {
  if (fp64)
    memint_kernel<double, CfgF64::T, CfgF64::NST>
        <<<total_ctas, CfgF64::NT + 32, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure);
  else
    memint_kernel<float, CfgF32::T, CfgF32::NST>
        <<<total_ctas, CfgF32::NT + 32, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure);
  return cudaGetLastError();
}

cudaError_t launch_measure_init(const RunDev *d_runs, int nruns, int t, cudaStream_t st) {
  measure_init_kernel<<<nruns, 256, 0, st>>>(d_runs, nruns, t);
  return cudaGetLastError();
}
cudaError_t launch_set_t(int *d_t, int t, cudaStream_t st) {
  set_t_kernel<<<1, 1, 0, st>>>(d_t, t);
  return cudaGetLastError();
}
cudaError_t launch_advance_t(int *d_t, cudaStream_t st) {
  advance_t_kernel<<<1, 1, 0, st>>>(d_t);
  return cudaGetLastError();
}

}  // namespace kb
