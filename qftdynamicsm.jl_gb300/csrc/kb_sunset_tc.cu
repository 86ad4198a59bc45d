// kb_sunset_tc.cu -- the sunset self-energy of the mixed-precision step on the
// fifth-generation tensor cores (tcgen05.mma, kind::tf32).
//
// Same transform as sunset_kernel (kb_sunset.cu; calcSelfEnergyattp!,
// src/TwoPIScalar/TwoPIScalar_Evolution.jl:25-31 quantum, :107-121 classical):
// each 3D cosine transform of a cubic-symmetric row is three axis passes, here
// written as matrix products D = A C^T with the H x H cosine matrix C (padded to
// N = NP columns, K = KP) as the B operand in shared memory and 128-row tiles of A
// in tensor memory (TMEM):
//   pass 1  A1[p][x]     = f(x, y_p, z_p)                 rows: pairs p = (y <= z)
//           D1[p][X]     = sum_x A1[p][x] C[X][x]
//   pass 2  A2[(X,z)][y] = D1[(min(y,z), max(y,z))][X]    rows: X H + z
//           D2[(X,z)][Y] = sum_y A2 C[Y][y]               (kept for Y >= X)
//   pass 3  A3[q][z]     = D2[(X_q, z)][Y_q]              rows: pairs q = (X <= Y)
//           out(X, Y, Z) = sum_z A3[q][z] C[Z][z]         for Z >= Y: one value per orbit
// Each pass output is read from TMEM by the warps (lane = row) and written to
// shared memory in the row-major form the next pass gathers its A rows from.
//
// Precision: every FP32 operand x is split into a TF32 head h = rna(x) and a
// TF32 tail l = rna(x - h), and each product runs as three MMAs,
//   A C ~ A_h C_h + A_l C_h + A_h C_l,
// accumulated in FP32 in TMEM (the dropped A_l C_l and the rounding of the tails
// are about 2^-21 of each product). The history, the rows and the pointwise
// products stay FP32, as in sunset_kernel.
//
// Layouts. B (C_h and C_l): K-major, no swizzle: the 8-row x 16-byte core matrix
// (g, kc) of rows 8g.., K elements 4kc.. at byte offset (g KCH + kc) 128, KCH = KP/4;
// the descriptor's leading offset (between K-adjacent core matrices) is 128 B and its
// stride offset (between 8-row groups) KCH 128 B. A: row r of a tile in TMEM lane r,
// K element k in column k (heads) and 40 + k (tails) of the tile's stage. D: row r in
// lane r, output column j in column 80 + j of the stage.
//
// Pipeline of a pass: three TMEM stages (A and D of one tile each, one mbarrier per
// stage); a tile's MMAs are issued once its A rows are built and it is read out two
// tiles later, so the MMA chains of up to three tiles overlap the building and reading.
// Every wait is bounded (~2 s); on expiry the CTA sets DEVERR_TIMEOUT and skips its
// remaining rows. One CTA per SM (about 212 KB of shared memory at Ns = 64), 512
// threads: warps w, w + 4, w + 8, w + 12 share TMEM lanes 32 (w mod 4).. and split
// the K (A build) and N (read-out) ranges of a tile between them.
#include <cstdio>

#include "kb_internal.cuh"

namespace kb {
namespace {

constexpr int TC_THREADS = 512;
constexpr int TC_NG = TC_THREADS / 128;     // thread groups sharing a TMEM lane
// TMEM: NSTG stages of (A: 40 heads + 40 tails, D: 48) = 128 columns each
constexpr int TC_NSTG = 3;
constexpr int TC_LAG = TC_NSTG - 1;         // a tile is read out TC_LAG tiles after it is issued
constexpr uint32_t TC_STAGE_COLS = 128, TC_D_OFF = 80;
constexpr uint32_t TC_TMEM_COLS = 512;      // power of two >= NSTG x 128
constexpr int TC_KMAX = 40;                 // H <= 40 (Ns <= 78)

__host__ __device__ inline int rup(int v, int m) { return (v + m - 1) / m * m; }

struct TcGeom {
  int H, P, S, KP, NP, KS, KCH, HH;
  __host__ __device__ explicit TcGeom(int H_) {
    H = H_;
    P = H * (H + 1) / 2;
    S = H * (H + 1) * (H + 2) / 6;
    KP = rup(H, 8);
    NP = rup(H, 16);
    KS = KP / 8;
    KCH = KP / 4;
    HH = H * H;
  }
};

// shared memory: B heads and tails, pair table, two orbit rows, two pass buffers
struct TcLayout {
  size_t bh, bl, pr, rowF, rowR, d1, d2, bytes;
};
__host__ __device__ inline TcLayout tc_layout(int H) {
  TcGeom g(H);
  TcLayout L;
  size_t o = 0;
  L.bh = o;
  o += (size_t)g.NP * g.KP * 4;
  L.bl = o;
  o += (size_t)g.NP * g.KP * 4;
  L.pr = o;
  o += (size_t)rup(g.P, 2) * 2;
  o = (o + 15) & ~(size_t)15;
  L.rowF = o;
  o += (size_t)rup(g.S, 4) * 4;
  L.rowR = o;
  o += (size_t)rup(g.S, 4) * 4;
  L.d1 = o;
  o += (size_t)g.P * g.H * 4;
  L.d2 = o;
  o += (size_t)g.P * g.H * 4;
  L.bytes = (o + 15) & ~(size_t)15;
  return L;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// orbit of the sorted triple a <= b <= c, and of (x, y, z) given y <= z
__device__ __forceinline__ int orb3s(int a, int b, int c) { return c * (c + 1) * (c + 2) / 6 + b * (b + 1) / 2 + a; }
__device__ __forceinline__ int orb_of(int x, int y, int z) {
  const int lo = min(x, y);
  const int mid = (x <= y) ? y : min(x, z);
  const int hi = max(x, z);
  return orb3s(lo, mid, hi);
}

// shared-memory matrix descriptor: K-major, no swizzle (version 1 for sm_100 and later)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor: D FP32, A and B TF32, both K-major, M x N
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_tf32(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
      "r"(a), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_st2(uint32_t ta, float a, float b) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};" ::"r"(ta), "r"(__float_as_uint(a)),
               "r"(__float_as_uint(b))
               : "memory");
}
__device__ __forceinline__ void tmem_ld4(uint32_t ta, float v[4]) {
  uint32_t w[4];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3])
      : "r"(ta)
      : "memory");
#pragma unroll
  for (int j = 0; j < 4; ++j) v[j] = __uint_as_float(w[j]);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// bounded wait for the phase of the given parity (~2 s)
__device__ bool mbar_wait_2s(uint64_t *bar, uint32_t parity) {
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t it = 0; it < (1u << 30); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((it & 255u) == 0 && globaltimer_ns() - t0 > 2000000000ull) return false;
  }
  return false;
}

struct TcCtx {
  TcGeom g{1};
  const float *bh, *bl;  // B heads / tails (canonical K-major layout)
  const uint16_t *pr;    // pair p -> (lo | hi << 8)
  float *d1, *d2;        // pass outputs, rows of H
  uint32_t tmem;         // TMEM base (lane 0, first column)
  uint64_t *bar;         // [TC_NSTG] MMA completion per stage
  uint32_t ph;           // bit s: parity of the next completion of stage s
  int *err;
  bool ok;
};

// One pass over nt tiles: build(m, acol) fills the A columns at TMEM column acol
// with tile m's rows (this thread: lane row, K group); readout(m, dcol) reads tile
// m's D columns. Tile m uses stage m mod NSTG; its MMAs are issued as soon as its
// A rows are in TMEM, and it is read out TC_LAG tiles later, so the MMAs of up to
// NSTG tiles are in flight while rows are built and read. Returns false (all
// threads) when a wait expired.
template <typename Build, typename Readout>
__device__ bool tc_pass(TcCtx &c, int nt, Build build, Readout readout) {
  const int tid = threadIdx.x;
  const TcGeom &g = c.g;
  constexpr uint32_t IDESC_N48 = tf32_idesc(128, 48), IDESC_N32 = tf32_idesc(128, 32), IDESC_N16 = tf32_idesc(128, 16);
  const uint32_t idesc = g.NP == 48 ? IDESC_N48 : (g.NP == 32 ? IDESC_N32 : IDESC_N16);
  const uint32_t lbo = 128u, sbo = (uint32_t)g.KCH * 128u;
  const uint32_t bh0 = smem_u32(c.bh), bl0 = smem_u32(c.bl);
  auto issue = [&](int st) {  // one thread: the 3 KS MMAs of the tile in stage st
    fence_after();
    const uint32_t a = c.tmem + (uint32_t)st * TC_STAGE_COLS, d = a + TC_D_OFF;
    for (int ks = 0; ks < g.KS; ++ks) {
      const uint64_t dh = smem_desc(bh0 + (uint32_t)ks * 256u, lbo, sbo);
      const uint64_t dl = smem_desc(bl0 + (uint32_t)ks * 256u, lbo, sbo);
      mma_tf32(d, a + 8u * ks, dh, idesc, ks > 0 ? 1u : 0u);  // heads x heads
      mma_tf32(d, a + 40u + 8u * ks, dh, idesc, 1u);          // tails x heads
      mma_tf32(d, a + 8u * ks, dl, idesc, 1u);                // heads x tails
    }
    mma_commit(c.bar + st);
  };
  // wait for the MMAs of tile j and read it out
  auto drain = [&](int j) -> bool {
    const int st = j % TC_NSTG;
    // warp-uniform: the read-out's tcgen05.ld is warp-collective
    const bool ok = __all_sync(0xffffffffu, mbar_wait_2s(c.bar + st, (c.ph >> st) & 1u));
    c.ph ^= 1u << st;
    fence_after();
    if (ok) readout(j, c.tmem + (uint32_t)st * TC_STAGE_COLS + TC_D_OFF);
    return ok;
  };
  bool ok = true;
  for (int m = 0; m < nt; ++m) {
    // stage m mod NSTG is free: tile m - NSTG was read out in iteration m - 1
    build(m, c.tmem + (uint32_t)(m % TC_NSTG) * TC_STAGE_COLS);
    st_wait();
    fence_before();
    ok = __syncthreads_and(ok);
    if (!ok) break;
    if (tid == 0) issue(m % TC_NSTG);
    if (m >= TC_LAG) ok = drain(m - TC_LAG);
  }
  for (int j = max(0, nt - TC_LAG); j < nt && ok; ++j) ok = drain(j);
  fence_before();
  ok = __syncthreads_and(ok);
  fence_after();
  if (!ok && tid == 0) atomicOr(c.err, DEVERR_TIMEOUT);
  return ok;
}

// the cosine transform of one orbit row src -> dst (dst may be src): three passes
__device__ bool tc_transform(TcCtx &c, const float *src, float *dst) {
  const TcGeom &g = c.g;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = (warp & 3) * 32 + lane;  // TMEM lane of this thread
  const uint32_t lanebits = (uint32_t)((warp & 3) * 32) << 16;
  const int kg = warp >> 2;                   // K / N group of this thread (TC_NG groups)
  const int kw = g.KP / TC_NG, k0 = kg * kw;  // K columns k0 .. k0 + kw - 1 (kw is even)
  const int nw = g.NP / TC_NG, n0 = kg * nw;  // N columns n0 .. n0 + nw - 1 (nw is a multiple of 4)
  const int H = g.H;
  // A rows: value(k) for k in [k0, k0 + kw), heads at acol + k, tails at acol + 40 + k
  auto put_row = [&](uint32_t acol, auto value) {
    for (int k = k0; k < k0 + kw; k += 2) {
      const float v0 = value(k), v1 = value(k + 1);
      const float h0 = tf32_rna(v0), h1 = tf32_rna(v1);
      tmem_st2(acol + lanebits + (uint32_t)k, h0, h1);
      tmem_st2(acol + lanebits + 40u + (uint32_t)k, tf32_rna(v0 - h0), tf32_rna(v1 - h1));
    }
  };
  auto get_row = [&](uint32_t dcol, auto store) {
    for (int j = n0; j < n0 + nw; j += 4) {
      float v[4];
      tmem_ld4(dcol + lanebits + (uint32_t)j, v);
#pragma unroll
      for (int u = 0; u < 4; ++u) store(j + u, v[u]);
    }
  };
  const int nt13 = (g.P + 127) / 128, nt2 = (g.HH + 127) / 128;
  // pass 1: rows p = (y <= z), K = x
  bool ok = tc_pass(
      c, nt13,
      [&](int m, uint32_t acol) {
        const int p = m * 128 + row;
        const bool valid = p < g.P;
        const int y = valid ? (c.pr[p] & 255) : 0, z = valid ? (c.pr[p] >> 8) : 0;
        put_row(acol, [&](int x) { return (valid && x < H) ? src[orb_of(x, y, z)] : 0.0f; });
      },
      [&](int m, uint32_t dcol) {
        const int p = m * 128 + row;
        get_row(dcol, [&](int X, float v) {
          if (p < g.P && X < H) c.d1[p * H + X] = v;
        });
      });
  if (!ok) return false;
  // pass 2: rows (X, z), K = y; keeps Y >= X as A3[(X,Y)][z]
  ok = tc_pass(
      c, nt2,
      [&](int m, uint32_t acol) {
        const int r = m * 128 + row;
        const bool valid = r < g.HH;
        const int X = valid ? r / H : 0, z = valid ? r - (r / H) * H : 0;
        put_row(acol, [&](int y) {
          if (!valid || y >= H) return 0.0f;
          const int lo = min(y, z), hi = max(y, z);
          return c.d1[(hi * (hi + 1) / 2 + lo) * H + X];
        });
      },
      [&](int m, uint32_t dcol) {
        const int r = m * 128 + row;
        const bool valid = r < g.HH;
        const int X = valid ? r / H : 0, z = valid ? r - (r / H) * H : 0;
        get_row(dcol, [&](int Y, float v) {
          if (valid && Y >= X && Y < H) c.d2[(Y * (Y + 1) / 2 + X) * H + z] = v;
        });
      });
  if (!ok) return false;
  // pass 3: rows q = (X <= Y), K = z; orbit outputs Z >= Y
  return tc_pass(
      c, nt13,
      [&](int m, uint32_t acol) {
        const int q = m * 128 + row;
        const bool valid = q < g.P;
        put_row(acol, [&](int z) { return (valid && z < H) ? c.d2[q * H + z] : 0.0f; });
      },
      [&](int m, uint32_t dcol) {
        const int q = m * 128 + row;
        const bool valid = q < g.P;
        const int X = valid ? (c.pr[q] & 255) : 0, Y = valid ? (c.pr[q] >> 8) : 0;
        get_row(dcol, [&](int Z, float v) {
          if (valid && Z >= Y && Z < H) dst[orb3s(X, Y, Z)] = v;
        });
      });
}

// Persistent grid over the t' rows of all runs (rows outside the window skipped),
// as sunset_kernel: Sigma(t-1, t') for t' in [tmin, t-1].
__global__ void __launch_bounds__(TC_THREADS, 1)
sunset_tc_kernel(const RunDev *__restrict__ runs, const int *__restrict__ base, int nruns, int total,
                 const int *__restrict__ d_t) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar[TC_NSTG];
  __shared__ uint32_t tmem_slot;
  const int t = *d_t;
  const int tid = threadIdx.x, warp = tid >> 5, nthr = blockDim.x;
  if (tid == 0) {
    for (int q = 0; q < TC_NSTG; ++q) mbar_init(bar + q, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  TcCtx c;
  c.tmem = tmem_slot;
  c.bar = bar;
  c.ph = 0;
  c.ok = true;
  c.err = nullptr;
  int cur_ns = -1;
  float *rowF = nullptr, *rowR = nullptr;
  for (int w = blockIdx.x; w < total && c.ok; w += gridDim.x) {
    const int r = run_at(base, nruns, w);
    const RunDev &R = runs[r];
    if (!pexp_sunset(R.pexp) || t < 3) continue;
    c.err = R.err;
    if (R.Ns != cur_ns) {  // tables of the lattice size, shared by the runs of the same Ns
      __syncthreads();
      cur_ns = R.Ns;
      const TcGeom g(R.H);
      const TcLayout L = tc_layout(g.H);
      float *bh = reinterpret_cast<float *>(smem_raw + L.bh), *bl = reinterpret_cast<float *>(smem_raw + L.bl);
      uint16_t *pr = reinterpret_cast<uint16_t *>(smem_raw + L.pr);
      // B[X][x] = C[X][x] (zero in the padding), heads and tails, canonical K-major layout
      for (int i = tid; i < g.NP * g.KP; i += nthr) {
        const int X = i / g.KP, x = i - X * g.KP;
        const double cv = (X < g.H && x < g.H) ? R.Cm[X * g.H + x] : 0.0;
        const float h = tf32_rna((float)cv);
        const float l = tf32_rna((float)(cv - (double)h));
        const int off = ((X >> 3) * g.KCH + (x >> 2)) * 32 + (X & 7) * 4 + (x & 3);
        bh[off] = h;
        bl[off] = l;
      }
      for (int z = tid; z < g.H; z += nthr)
        for (int y = 0; y <= z; ++y) pr[z * (z + 1) / 2 + y] = (uint16_t)(y | (z << 8));
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B is read by the tensor cores
      __syncthreads();
      c.g = g;
      c.bh = bh;
      c.bl = bl;
      c.pr = pr;
      c.d1 = reinterpret_cast<float *>(smem_raw + L.d1);
      c.d2 = reinterpret_cast<float *>(smem_raw + L.d2);
      rowF = reinterpret_cast<float *>(smem_raw + L.rowF);
      rowR = reinterpret_cast<float *>(smem_raw + L.rowR);
    }
    const int tmin = max(1, t - R.M + 1);
    const int S = c.g.S;
    const size_t rowstride = (size_t)R.Malloc * KC;
    const size_t cstride = (size_t)R.Malloc * R.Malloc * KC;
    auto gidx = [&](int o) { return (size_t)(o / KC) * rowstride + (o % KC); };
    for (int gi = 0; gi < R.sun_rows && c.ok; ++gi) {
      const int tp = tmin + (w - R.cta_base_sun) * R.sun_rows + gi;
      if (tp > t - 1) break;
      const int slot = tp % R.Malloc;
      // (uniform over the CTA: the skip passes no barrier another thread waits at)
      if (!KB_DCHECK(tp >= tmin && t - 1 - tp < R.M && slot >= 0 && S <= R.nchunks * KC, R.err, DCHK_SUN_ROW))
        continue;
      const size_t hbase = hist_off(R.Malloc, R.T, 0, t - 1, tp, 0);
      auto stage = [&](const void *hist, float *dst) {
        const float *h = reinterpret_cast<const float *>(hist) + hbase;
        for (int o = tid; o < S; o += nthr) dst[o] = h[(size_t)(o / KC) * cstride + (o % KC)];
      };
      stage(R.hist_F, rowF);
      stage(R.hist_r, rowR);
      __syncthreads();
      // the next row of this CTA goes to L2 while the transforms run
      {
        int w2 = w, g2 = gi + 1;
        if (g2 >= R.sun_rows) {
          w2 = w + gridDim.x;
          g2 = 0;
        }
        if (w2 < total) {
          const RunDev &Rn = runs[run_at(base, nruns, w2)];
          const int tp2 = max(1, t - Rn.M + 1) + (w2 - Rn.cta_base_sun) * Rn.sun_rows + g2;
          if (pexp_sunset(Rn.pexp) && tp2 <= t - 1) {
            const size_t b2 = hist_off(Rn.Malloc, Rn.T, 0, t - 1, tp2, 0) * sizeof(float);
            const size_t cs2 = (size_t)Rn.Malloc * Rn.Malloc * KC * sizeof(float);
            for (int q = tid; q < Rn.nchunks; q += nthr) {
              asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char *>(Rn.hist_F) + b2 + q * cs2));
              asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char *>(Rn.hist_r) + b2 + q * cs2));
            }
          }
        }
      }
      if (!(c.ok = tc_transform(c, rowF, rowF))) break;
      if (!(c.ok = tc_transform(c, rowR, rowR))) break;
      // pointwise sunset in position space (Evolution.jl:28-29, classical :114-115)
      const bool classical = (R.pexp == 2);
      for (int k = tid; k < S; k += nthr) {
        const float Fx = rowF[k], rx = rowR[k];
        const float F2 = Fx * Fx, r2 = rx * rx;
        rowR[k] = classical ? rx * F2 : rx * (F2 - (1.0f / 12.0f) * r2);
        rowF[k] = classical ? Fx * F2 : Fx * (F2 - 0.75f * r2);
      }
      __syncthreads();
      float *sigr = reinterpret_cast<float *>(R.sig_r) + (size_t)slot * KC;
      float *sigF = reinterpret_cast<float *>(R.sig_F) + (size_t)slot * KC;
      auto flush = [&](float *sig, const float *v, float f) {
        for (int o = tid; o < S; o += nthr)
          if (KB_DCHECK((size_t)slot * KC + gidx(o) < (size_t)R.nchunks * rowstride, R.err, DCHK_SUN_SIGMA))
            sig[gidx(o)] = f * v[o];
      };
      if (!(c.ok = tc_transform(c, rowR, rowR))) break;
      flush(sigr, rowR, (float)R.fac_r);
      if (!(c.ok = tc_transform(c, rowF, rowF))) break;
      flush(sigF, rowF, (float)R.fac_F);
      __syncthreads();
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_slot), "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

}  // namespace

// shared memory of sunset_tc_kernel for a run of H = Ns/2 + 1 (0 when H is beyond the kernel)
size_t sunset_tc_smem_bytes(int H) { return (H >= 1 && H <= TC_KMAX) ? tc_layout(H).bytes : 0; }

// static shared memory of the kernel (mbarriers, TMEM slot): the dynamic part may use
// the device's per-block maximum less this
size_t sunset_tc_static_bytes() {
  cudaFuncAttributes a{};
  if (cudaFuncGetAttributes(&a, sunset_tc_kernel) != cudaSuccess) {
    cudaGetLastError();
    return 1024;
  }
  return a.sharedSizeBytes;
}

cudaError_t configure_sunset_tc(size_t max_block_smem) {
  const size_t st = sunset_tc_static_bytes();
  if (max_block_smem <= st) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(sunset_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(max_block_smem - st));
}

cudaError_t launch_sunset_tc(const RunDev *d_runs, const int *d_base, int nruns, int total_rows, int grid,
                             const int *d_t, size_t smem, cudaStream_t st) {
  if (total_rows <= 0 || grid <= 0) return cudaSuccess;
  sunset_tc_kernel<<<grid, TC_THREADS, smem, st>>>(d_runs, d_base, nruns, total_rows, d_t);
  return cudaGetLastError();
}

}  // namespace kb
