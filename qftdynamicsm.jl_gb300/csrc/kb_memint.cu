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
// and the diagonal pair F(a,a) feeds acc_F(a) once. One CTA at a time owns KC = 8
// orbits (a "chunk") and sweeps the whole triangle of its chunk exactly once, in
// T x T time tiles streamed from HBM by TMA (tensor-map boxes, or bulk copies)
// into a shared-memory ring: column sums stay in registers, row sums collect
// in tensor memory (FP32 history) or a global scratch (FP64). When a column
// block is complete its leapfrog runs at once, and after the last block the
// CTA computes the diagonal F(t,t), its tadpole partial sum and the
// measurement of its orbits. No data leaves the CTA except the new row, so the
// whole step needs no grid barrier. In split mode a chunk's triangle is
// streamed in parts and memint_finish_kernel runs the leapfrog; the grid is
// one CTA per item, or persistent with the items taken from a queue
// (memint_kernel below).
#include <algorithm>
#include <cstdio>
#include <type_traits>

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
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(1000000u)  // suspend up to 1 ms per poll
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
// L2 prefetch of one box of a 3D tensor map (no shared memory, no barrier)
__device__ __forceinline__ void tma_prefetch_3d(const void *tmap, int x, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(tmap), "r"(x), "r"(y),
               "r"(z)
               : "memory");
}
// tiled TMA load of one box of a 3D tensor map (x innermost, in elements)
__device__ __forceinline__ void prefetch_l2g(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

__device__ __forceinline__ void tma_load_3d(void *dst, const void *tmap, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// Tensor memory (TMEM) for the FP64 row accumulators of memint_kernel: one lane
// per row-group thread, 2 x 32-bit columns per double. A warp reaches the 32
// lanes 32 (warp mod 4) ..; the row group is warps 4..7 and the column group
// warps 0..3, so the column-group thread with the same group index sits on the
// same lane and reads that row's sum for its leapfrog. Each load and store
// waits for itself (one asm block), so no register is read before it is valid.
// ---------------------------------------------------------------------------
constexpr uint32_t TMEM_COLS = 256;  // power of two in [32, 512]
__device__ __forceinline__ void tmem_alloc(uint32_t *slot) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(TMEM_COLS)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(TMEM_COLS) : "memory");
}
__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// OPT doubles of this thread's lane at columns ta .. ta + 2 OPT - 1 (warp-collective)
template <int OPT>
struct TmemRow;
template <>
struct TmemRow<2> {
  __device__ __forceinline__ static void ld(uint32_t ta, double v[2]) {
    uint32_t w0, w1, w2, w3;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(w0), "=r"(w1), "=r"(w2), "=r"(w3)
        : "r"(ta)
        : "memory");
    v[0] = __hiloint2double((int)w1, (int)w0);
    v[1] = __hiloint2double((int)w3, (int)w2);
  }
  __device__ __forceinline__ static void st(uint32_t ta, const double v[2]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};\n\t"
        "tcgen05.wait::st.sync.aligned;" ::"r"(ta),
        "r"(__double2loint(v[0])), "r"(__double2hiint(v[0])), "r"(__double2loint(v[1])), "r"(__double2hiint(v[1]))
        : "memory");
  }
};
template <>
struct TmemRow<1> {
  __device__ __forceinline__ static void ld(uint32_t ta, double v[1]) {
    uint32_t w0, w1;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(w0), "=r"(w1)
        : "r"(ta)
        : "memory");
    v[0] = __hiloint2double((int)w1, (int)w0);
  }
  __device__ __forceinline__ static void st(uint32_t ta, const double v[1]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};\n\t"
        "tcgen05.wait::st.sync.aligned;" ::"r"(ta),
        "r"(__double2loint(v[0])), "r"(__double2hiint(v[0]))
        : "memory");
  }
};

// sum over q = lane, lane + 32, ... < n in ascending q (the order of a plain
// loop), with eight loads in flight instead of one load per addition
__device__ __forceinline__ double tad_lane_sum(const double *tad, int n, int lane) {
  double s = 0.0;
  for (int q0 = lane; q0 < n; q0 += 8 * 32) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = (q0 + 32 * u < n) ? tad[q0 + 32 * u] : 0.0;
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (q0 + 32 * u < n) s += v[u];
  }
  return s;
}

// OPT adjacent orbits per consumer thread: two FP32 values move with one 8-byte
// shared-memory load and one packed fma.rn.f32x2; FP64 keeps one orbit per thread.
template <typename TS, int OPT>
struct Vec;
template <>
struct Vec<float, 2> {
  float2 v;
  __device__ __forceinline__ static Vec zero() { return Vec{make_float2(0.f, 0.f)}; }
  __device__ __forceinline__ static Vec ld(const float *p) { return Vec{*reinterpret_cast<const float2 *>(p)}; }
  __device__ __forceinline__ void fma(const Vec &a, const Vec &b) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;"
        : "=l"(d)
        : "l"(*reinterpret_cast<const unsigned long long *>(&a.v)),
          "l"(*reinterpret_cast<const unsigned long long *>(&b.v)),
          "l"(*reinterpret_cast<const unsigned long long *>(&v)));
    v = *reinterpret_cast<float2 *>(&d);
  }
  __device__ __forceinline__ void scale(float w) {
    v.x *= w;
    v.y *= w;
  }
  __device__ __forceinline__ double get(int i) const { return i == 0 ? (double)v.x : (double)v.y; }
  __device__ __forceinline__ void add(const Vec &o) {
    v.x += o.v.x;
    v.y += o.v.y;
  }
};
template <>
struct Vec<double, 1> {
  double v;
  __device__ __forceinline__ static Vec zero() { return Vec{0.0}; }
  __device__ __forceinline__ static Vec ld(const double *p) { return Vec{*p}; }
  __device__ __forceinline__ void fma(const Vec &a, const Vec &b) { v = fma_rn(a.v, b.v, v); }
  __device__ __forceinline__ static double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
  __device__ __forceinline__ void scale(double w) { v *= w; }
  __device__ __forceinline__ double get(int) const { return v; }
  __device__ __forceinline__ void add(const Vec &o) { v += o.v; }
};

// Compensated tile partial sums of the consumers (memint_kernel<..., COMP = true>).
// FP32 history: Kahan sums of packed pairs -- s is the running FP32 sum, m minus its
// compensation, so that each addition's rounding error is carried in m and s + m
// (formed in FP64) is the partial sum; four packed operations per term (fma, add,
// sub, sub) against one. FP64 history: plain FP64 sums.
template <typename TS, int OPT>
struct Acc;
template <>
struct Acc<float, 2> {
  unsigned long long s, m;
  __device__ __forceinline__ static Acc zero() { return Acc{0ull, 0ull}; }
  __device__ __forceinline__ static unsigned long long bits(const Vec<float, 2> &a) {
    return *reinterpret_cast<const unsigned long long *>(&a.v);
  }
  // one compensated step with the term y already formed
  __device__ __forceinline__ void step(unsigned long long y) {
    unsigned long long t, u;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(t) : "l"(s), "l"(y));
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(u) : "l"(t), "l"(s));
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(m) : "l"(y), "l"(u));
    s = t;
  }
  // s + m += a * b: the product and the previous compensation in one fma
  __device__ __forceinline__ void fma(const Vec<float, 2> &a, const Vec<float, 2> &b) {
    unsigned long long y;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(y) : "l"(bits(a)), "l"(bits(b)), "l"(m));
    step(y);
  }
  // s + m += o.s + o.m: both parts of o, one compensated step each
  __device__ __forceinline__ void add(const Acc &o) {
    unsigned long long y;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(y) : "l"(o.s), "l"(m));
    step(y);
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(y) : "l"(o.m), "l"(m));
    step(y);
  }
  __device__ __forceinline__ double get(int i) const {
    const float2 a = *reinterpret_cast<const float2 *>(&s), b = *reinterpret_cast<const float2 *>(&m);
    return i == 0 ? (double)a.x + (double)b.x : (double)a.y + (double)b.y;
  }
};
// plain FP32 (or FP64) tile partial sums: one fma per term
template <typename TS, int OPT>
struct PlainAcc {
  Vec<TS, OPT> a;
  __device__ __forceinline__ static PlainAcc zero() { return PlainAcc{Vec<TS, OPT>::zero()}; }
  __device__ __forceinline__ void fma(const Vec<TS, OPT> &x, const Vec<TS, OPT> &y) { a.fma(x, y); }
  __device__ __forceinline__ void add(const PlainAcc &o) { a.add(o.a); }
  __device__ __forceinline__ double get(int i) const { return a.get(i); }
};
template <>
struct Acc<double, 1> {
  Vec<double, 1> a;
  __device__ __forceinline__ static Acc zero() { return Acc{Vec<double, 1>::zero()}; }
  __device__ __forceinline__ void fma(const Vec<double, 1> &x, const Vec<double, 1> &y) { a.fma(x, y); }
  __device__ __forceinline__ void add(const Acc &o) { a.add(o.a); }
  __device__ __forceinline__ double get(int i) const { return a.get(i); }
};

template <typename TS, int T_, int NST_, int OPT_>
struct Cfg {
  static constexpr int T = T_;
  static constexpr int NST = NST_;
  static constexpr int OPT = OPT_;                          // orbits per consumer thread
  static constexpr int NJ = KC / OPT;                       // orbit groups per chunk
  static constexpr int NG = T * NJ;                         // threads per consumer group
  static constexpr int NT = 2 * NG;                         // column group + row group
  static constexpr int NW = NT / 32;                        // consumer warps
  static constexpr int RS = T * KC;                         // smem stride of one tile row (columns swizzled)
  static constexpr int TILE = T * RS;                       // elements of one field tile in smem
  static constexpr int XV = T * KC;                         // one x vector (T times x KC orbits)
  static constexpr int STAGE = 2 * TILE + 3 * XV;           // F, rho, x_rho(rows), x_rho(cols), x_F(cols)
  static constexpr uint32_t STAGE_BYTES = STAGE * sizeof(TS);
  static constexpr uint32_t TX_BYTES = (2 * T * T * KC + 3 * XV) * sizeof(TS);  // bytes the TMA delivers
  static_assert((T * KC * sizeof(TS)) % 16 == 0, "bulk copies need 16-byte multiples");
  static_assert((RS * sizeof(TS)) % 16 == 0, "tile rows must stay 16-byte aligned");
  static_assert(T <= 32, "one tile row per lane of the producer warp");
  static_assert(NG % 32 == 0, "whole warps per group");
};

// two copies of a run's parameters (memint_kernel: the current item's and the next
// one's) and two control words, after the small scratch
constexpr size_t RUNBUF_BYTES = (2 * sizeof(RunDev) + 2 * sizeof(int) + 15) & ~(size_t)15;
static_assert(sizeof(RunDev) % 8 == 0, "copied as 8-byte words");

template <typename C>
__host__ __device__ constexpr size_t smem_fixed_bytes() {
  // stages + full/empty barriers + small scratch + run parameters
  return (size_t)C::NST * C::STAGE_BYTES + 2 * C::NST * 8 + 128 * 8 + 16 + RUNBUF_BYTES;
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

// issued by the producer warp: the F and rho tiles (each one contiguous block in
// the tile-major history), Sigma_rho of the tile's rows and Sigma_rho, Sigma_F of
// its columns, all into one stage. The consumers only read rows a in
// [tmin, t-1], so a tile the window cuts is copied from its first to its last
// such row: one copy of contiguous whole rows (the newest row block is partly
// empty, the oldest diagonal tile starts at tmin). Cutting columns as well
// (one copy per row) saves another 7 % of the bytes at Ns = 64 but costs more
// time than it saves: the many small copies slow every CTA. The stage offsets
// are those of the whole tile, so the consumers index it unchanged.
// Box of tile (I, J) fetched through the tensor maps: the tile's size, from row
// r0 and column position x0 (in elements). Rows past t-1 (newest row block) or
// before tmin (oldest diagonal tile) and the columns before tmin (oldest column
// block, to the 4-column group of the XOR swizzle) fall outside the tile and are
// filled with zeros instead of read. The box lands at the start of the stage,
// so tile element (row, pos) sits at (row - r0) RS + pos - x0 there.
template <typename C>
__device__ __forceinline__ void tile_box(int I, int J, int tmin, int tlast, int &r0, int &x0) {
  constexpr int T = C::T;
  const int rlo = max(0, tmin - I * T), rhi = min(T - 1, tlast - I * T);
  r0 = (rhi < T - 1) ? rhi - (T - 1) : rlo;
  x0 = (J == tmin / T) ? ((tmin - J * T) & ~3) * KC : 0;
}

template <typename TS, typename C>
__device__ __forceinline__ void issue_tile(int stage, int I, int J, const RunDev &R, int c, TS *stages,
                                           uint64_t *full, int tmin, int tlast, bool use_tmap) {
  constexpr int T = C::T, TH = T / 2;
  const int lane = threadIdx.x & 31;
  uint64_t *bar = full + stage;
  TS *dst = stages + (size_t)stage * C::STAGE;
  const int sa0 = (I * C::T) % R.Malloc;  // Malloc is a multiple of T: rows stay contiguous
  const int sb0 = (J * C::T) % R.Malloc;
  const TS *hF = reinterpret_cast<const TS *>(R.hist_F);
  const TS *hR = reinterpret_cast<const TS *>(R.hist_r);
  // a diagonal tile inside the window is read only on and below its diagonal (column
  // sums take rows a >= b, row sums columns b < a): its upper-right quadrant (rows
  // < T/2, columns >= T/2) is not loaded -- the lower half as rows, the upper-left
  // quadrant as half rows; the stage keeps whatever that quadrant held
  int r0, x0;
  tile_box<C>(I, J, tmin, tlast, r0, x0);
  const bool quad = (I == J) && r0 == 0 && x0 == 0;
  const size_t off = hist_off(R.Malloc, T, c, sa0, sb0, 0);  // start of the tile
  if (lane == 0) {
    (void)KB_DCHECK(I >= J && J * T <= tlast && I * T <= tlast && (I + 1) * T - 1 >= tmin && c >= 0 &&
                        c < R.nchunks && (I - J) * T < R.M + T && R.Malloc % T == 0 && sa0 + T <= R.Malloc &&
                        sb0 + T <= R.Malloc && (!quad || (I * T >= tmin && I * T + T - 1 <= tlast)),
                    R.err, DCHK_MI_TILE);
    constexpr uint32_t QB = 2u * TH * (TH * KC) * (uint32_t)sizeof(TS);  // upper-left quadrants of F and rho
    constexpr uint32_t XB = 3u * C::XV * (uint32_t)sizeof(TS);           // the three x vectors
    if (use_tmap) {
      const int nb = R.Malloc / T;
      const int tile = (c * nb + sa0 / T) * nb + sb0 / T;
      const char *tm = reinterpret_cast<const char *>(R.tmap);
      if (quad) {  // maps 2, 3: boxes of the lower T/2 rows
        mbar_expect_tx(bar, 2u * TH * C::RS * (uint32_t)sizeof(TS) + QB + XB);
        tma_load_3d(dst + TH * C::RS, tm + 256, 0, TH, tile, bar);
        tma_load_3d(dst + C::TILE + TH * C::RS, tm + 384, 0, TH, tile, bar);
      } else {
        mbar_expect_tx(bar, 2 * C::TILE * (uint32_t)sizeof(TS) + XB);
        tma_load_3d(dst, tm, x0, r0, tile, bar);
        tma_load_3d(dst + C::TILE, tm + 128, x0, r0, tile, bar);
      }
    } else {
      constexpr uint32_t ROWB = (uint32_t)(C::RS * sizeof(TS));
      const int rlo = quad ? TH : max(0, tmin - I * T), rhi = min(T - 1, tlast - I * T);  // rows of the window
      const uint32_t n = (uint32_t)(rhi - rlo + 1) * ROWB;
      mbar_expect_tx(bar, 2 * n + (quad ? QB : 0u) + XB);
      const size_t e = (size_t)rlo * C::RS;
      bulk_g2s(dst + e, hF + off + e, n, bar);
      bulk_g2s(dst + C::TILE + e, hR + off + e, n, bar);
    }
    const TS *sr = reinterpret_cast<const TS *>(R.sig_r) + (size_t)c * R.Malloc * KC;
    const TS *sF = reinterpret_cast<const TS *>(R.sig_F) + (size_t)c * R.Malloc * KC;
    bulk_g2s(dst + 2 * C::TILE, sr + (size_t)sa0 * KC, C::XV * sizeof(TS), bar);
    bulk_g2s(dst + 2 * C::TILE + C::XV, sr + (size_t)sb0 * KC, C::XV * sizeof(TS), bar);
    bulk_g2s(dst + 2 * C::TILE + 2 * C::XV, sF + (size_t)sb0 * KC, C::XV * sizeof(TS), bar);
  }
  __syncwarp();  // the expected bytes are set before any half row lands
  if (quad && lane < 2 * TH) {  // one half row (columns < T/2 of row rr) per lane and field
    const int f = lane / TH, rr = lane % TH;
    const size_t e = (size_t)rr * C::RS;
    bulk_g2s(dst + f * C::TILE + e, (f ? hR : hF) + off + e, TH * KC * (uint32_t)sizeof(TS), bar);
  }
  __syncwarp();
}

__device__ __forceinline__ void consumer_sync(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// Per-orbit frequency, its lattice correction and particle number of the measurement
// (createMeasurement, Measurement.jl:38-64) from F(t-1,t-1) and its second time
// derivative ddF. Each product, quotient and root is rounded on its own (no fused
// multiply-adds), so the kernels that derive them -- at the measured step's read,
// in the recorded stream, at initialisation -- give the same bits.
__device__ __forceinline__ void meas_derived(double Fmm, double ddF, double dt2, double &omg, double &cc,
                                             double &nn) {
  const double q = __ddiv_rn(ddF, Fmm);
  omg = (q > 0) ? __dsqrt_rn(q) : 0.0;
  const double w = __dmul_rn(__dmul_rn(0.25, dt2), __dmul_rn(omg, omg));
  cc = (w < 1) ? __dsqrt_rn(__dsub_rn(1.0, w)) : 1.0;
  const double p = __dmul_rn(ddF, Fmm);
  nn = (p > 0) ? __dsub_rn(__dmul_rn(cc, __dsqrt_rn(p)), 0.5) : 0.0;
}

// Diagonal F(t,t) (Evolution.jl:969-974), its tadpole partial for the next
// step and the measurement of the chunk's orbits (createMeasurement,
// Measurement.jl:38-64: F(t-1,t-1) and ddF here, the rest by meas_derived where the
// measurement is read); threads 0..KC-1 of the CTA, one orbit each. misc holds
// hartreecont, acc_F(t-1) per orbit and the nwarps x KC partial sums of acc_F(t).
// pre (if not null): the orbits' k^2, degeneracy, F(t-1,t-1), F(t,t-1) and F(t,t-2),
// KC values each, gathered while the item was streamed; else they are loaded here.
// red (if not null): the orbit's tadpole and energy terms go to red[q KC + orbit]
// for memint_epilogue_sum, and the caller may spread the orbits over warps (the
// FP64 arithmetic then runs on several SM sub-partitions); else threads 0..KC-1 of
// one warp sum them with shuffles.
template <typename TS>
__device__ void memint_epilogue(const RunDev &R, int c, int t, int tid, const double *misc, int nwarps,
                                double M2, int measure, const double *pre = nullptr, double *red = nullptr) {
  const double hc = misc[0];
  const int Ma = R.Malloc, T = R.T;
  const size_t rowstride = (size_t)Ma * KC;
  const size_t st_row = (size_t)R.nchunks * rowstride;
  const double *F1row = R.st_F + (size_t)((t - 1) % 3) * st_row + (size_t)c * rowstride;
  double *FNrow = R.st_F + (size_t)(t % 3) * st_row + (size_t)c * rowstride;
  double *RNrow = R.st_r + (size_t)(t % 3) * st_row + (size_t)c * rowstride;
  const size_t hdo = hist_off(Ma, T, c, t, t, tid);
  double accd = 0.0;
  for (int w = 0; w < nwarps; ++w) accd += misc[16 + w * KC + tid];
  const int jj = tid;
  const int kd = c * KC + jj;
  // every load ahead of the first store (the stores below could alias them as far as
  // the compiler knows): one round trip instead of a chain of them
  const bool kin = kd < R.S;
  double kd2, dg, Ft1, Ft2, Fmm;
  if (pre) {
    kd2 = pre[jj];
    dg = pre[KC + jj];
    Fmm = pre[2 * KC + jj];
    Ft1 = pre[3 * KC + jj];
    Ft2 = pre[4 * KC + jj];
  } else {
    kd2 = kin ? R.k2[kd] : 0.0;
    dg = kin ? R.deg[kd] : 0.0;
    // F(t, t-1), F(t, t-2): written in this launch, possibly by another CTA of the chunk
    Ft1 = __ldcg(FNrow + (size_t)((t - 1) % Ma) * KC + jj);
    Ft2 = __ldcg(FNrow + (size_t)((t - 2) % Ma) * KC + jj);
    // measurement (createMeasurement, Measurement.jl:38-64): F(t-1,t-1) from the state
    Fmm = F1row[(size_t)((t - 1) % Ma) * KC + jj];
  }
  const double omd = (kd2 + M2) * R.dt2;
  const double Ftt = (2.0 - omd) * Ft1 - Ft2 - accd * R.dt3;
  FNrow[(size_t)(t % Ma) * KC + jj] = Ftt;
  RNrow[(size_t)(t % Ma) * KC + jj] = 0.0;
  reinterpret_cast<TS *>(R.hist_F)[hdo] = (TS)Ftt;
  reinterpret_cast<TS *>(R.hist_r)[hdo] = (TS)0;
  double tp = dg * Ftt;  // tadpole partial sum of this chunk for the next step
  const double dt = R.dt, dt2 = R.dt2;
  const double ddF = (Ftt - 2 * Ft1 + Fmm) / dt2;
  double ek = 0.5 * ddF * dg;
  double ep = 0.5 * (R.mass2 + kd2 + 0.5 * R.pref_ivol * hc) * Fmm * dg;
  double em = 0.25 * dt * dg * misc[2 + jj];
  if (kd < R.S && measure) {
    const int Sp = R.nchunks * KC;
    R.meas[0 * Sp + kd] = Fmm;
    R.meas[1 * Sp + kd] = ddF;
  }
  if (red) {
    red[jj] = tp;
    red[KC + jj] = ek;
    red[2 * KC + jj] = ep;
    red[3 * KC + jj] = em;
    return;
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

// sum q (0 tadpole, 1..3 kinetic, potential, memory energy) of memint_epilogue's
// per-orbit terms in red, added in the order lane 0 of its shuffle tree adds them
__device__ void memint_epilogue_sum(const RunDev &R, int c, int t, int q, const double *red, double M2,
                                    int measure) {
  static_assert(KC == 8, "the tree below is the one of eight lanes");
  const double *v = red + q * KC;
  const double s = ((v[0] + v[4]) + (v[2] + v[6])) + ((v[1] + v[5]) + (v[3] + v[7]));
  if (q == 0) {
    R.tad[(size_t)(t & 1) * R.nchunks + c] = s;
  } else if (measure) {
    R.epart[(size_t)c * 4 + q - 1] = s;
    if (q == 3) R.epart[(size_t)c * 4 + 3] = M2;
  }
}

// leapfrog of column b (t' = b) for orbits j0 .. j0+OPT-1 of chunk c
// (evolve_r!/evolve_F!, Evolution.jl:890-915) from the column sums colF, colR
// and the row sums rowb of row b; adds the column's acc_F(t) terms to diag and
// keeps acc_F(t-1) in emem (b = t-1); capt (if not null) gets F(t,t-1) at [j] and
// F(t,t-2) at [KC + j]
template <typename TS, int OPT>
__device__ __forceinline__ void leapfrog_column(const RunDev &R, int c, int t, int tmin, int b, int j0, double M2,
                                                bool lo_only, const double *colF, const double *colR,
                                                const double *rowb, double *diag, double *emem, bool &has_emem,
                                                double *capt = nullptr) {
  const int Ma = R.Malloc;
  const size_t rowstride = (size_t)Ma * KC, st_row = (size_t)R.nchunks * rowstride;
  const double dt3 = R.dt3;
  const int sb = b % Ma;
  const double wb = (b == tmin) ? 0.5 : 1.0;
  const TS *sigr = reinterpret_cast<const TS *>(R.sig_r) + (size_t)c * rowstride + (size_t)sb * KC;
  const TS *sigF = reinterpret_cast<const TS *>(R.sig_F) + (size_t)c * rowstride + (size_t)sb * KC;
  const size_t cs = (size_t)c * rowstride;
  const double *F1row = R.st_F + (size_t)((t - 1) % 3) * st_row + cs;
  const double *F2row = R.st_F + (size_t)((t - 2) % 3) * st_row + cs;
  const double *R1row = R.st_r + (size_t)((t - 1) % 3) * st_row + cs;
  const double *R2row = R.st_r + (size_t)((t - 2) % 3) * st_row + cs;
  double *FNrow = R.st_F + (size_t)(t % 3) * st_row + cs;
  double *RNrow = R.st_r + (size_t)(t % 3) * st_row + cs;
  TS *hF = reinterpret_cast<TS *>(R.hist_F);
  TS *hR = reinterpret_cast<TS *>(R.hist_r);
  if (!KB_DCHECK(b >= tmin && b <= t - 1 && t - b < R.M && c >= 0 && c < R.nchunks && j0 >= 0 && j0 + OPT <= KC,
                 R.err, DCHK_LF_WRITE))
    return;
  for (int o = 0; o < OPT; ++o) {
    const int j = j0 + o;
    const int k = c * KC + j;
    const double kk = (k < R.S) ? R.k2[k] : 0.0;
    const double om = (kk + M2) * R.dt2;  // setomega2values!: (kL2 + M^2) * dt^2
    const double xbr_d = lo_only ? 0.0 : wb * (double)sigr[j];
    const double xbF_d = lo_only ? 0.0 : wb * (double)sigF[j];
    const double accF = colF[o] + rowb[o];
    const double accR = colR[o];
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
    const size_t ho = hist_off(Ma, R.T, c, t, b, j);
    hF[ho] = (TS)Fn;
    hR[ho] = (TS)rn;
    diag[o] += xbr_d * Fn + xbF_d * rn;
    if (b == t - 1) emem[o] = accF;
    if (capt && b >= t - 2) capt[(t - 1 - b) * KC + j] = Fn;  // F(t,t-1), F(t,t-2) for the diagonal
  }
  if (b == t - 1) has_emem = true;
}

// wait of a leapfrog warp on a hand-off barrier: false when the consumers
// abort the chunk or after ~2 s
__device__ bool lf_wait(uint64_t *bar, uint32_t parity, volatile int *cabort) {
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t it = 0; it < (1u << 30); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*cabort) return false;
    if ((it & 255u) == 0 && globaltimer_ns() - t0 > 2000000000ull) return false;
  }
  return false;
}

// hand-off stage of the leapfrog warps: two buffers of (colF, colR) x OPT per
// column-group thread (128 threads x 2 orbits)
constexpr size_t LF_STAGE_BYTES = 2 * 128 * 2 * 2 * sizeof(double);
static_assert(LF_STAGE_BYTES <= 8 * 32 * KC * sizeof(double), "the stage fits where memint_blk_kernel keeps its column buffer");

// Split mode: the triangle of a chunk is cut between column blocks into k parts
// of (nearly) equal tile counts (block J of J0..Jn holds Jn - J + 1 tiles); part p
// takes blocks [split_bound(p), split_bound(p + 1)) and may be empty when the
// triangle has fewer blocks than parts. With k = 2 the cut is where the first
// half reaches half the tiles.
__host__ __device__ inline int split_bound(int J0, int Jn, int k, int p) {
  if (p <= 0) return J0;
  if (p >= k) return Jn + 1;
  const int nb = Jn - J0 + 1, total = nb * (nb + 1) / 2;
  int acc = 0;
  for (int J = J0; J <= Jn; ++J) {
    acc += Jn - J + 1;
    if (k * acc >= p * total) return J + 1;
  }
  return Jn + 1;
}

// Block = column group (NG threads: column b, orbits j) + row group (NG threads:
// row a, orbits j) + one producer warp. Both consumer groups read every tile
// from the shared-memory ring: the column group accumulates
//   acc_F(b) += x_rho(a) F(a,b),  acc_r(b) += x_rho(a) rho(a,b)   over rows a >= b,
// the row group
//   acc_F(a) += x_rho(b) F(a,b) + x_F(b) rho(a,b)                  over columns b < a,
// each in its own registers over the valid index range of the tile, so a tile
// needs no cross-thread reduction and no block barrier; every consumer warp
// releases the stage through the empty mbarrier. Once per column block both
// groups meet at a named barrier: the row sums of that block are complete and
// the column group runs its leapfrog.
// Items: with a null queue CTA v takes item v. With a queue the grid is
// persistent (one CTA per SM): every CTA takes items from the counter until none
// are left, keeping its TMEM allocation and its stage barriers -- whose phases
// run on across items -- and the tadpole sum of the run it last took.
// SPLIT: the first nwhole items are whole chunks as above; after them item
// nwhole + parts i + p streams part p of chunk nwhole + i's triangle, keeps its
// row sums in row buffer p and stores the column sums of its column blocks
// instead of running the leapfrog; memint_finish_kernel completes those chunks.
// Split chunks fill the partial last wave of a large grid (nwhole = whole waves,
// parts chosen so that the pieces fill the SMs) or double the CTAs of a small one
// (nwhole = 0, two parts).
// LFW (FP32 history): four more warps run the leapfrog of a whole chunk's column
// blocks. The column group hands each block's column sums over through a
// double-buffered shared-memory stage (lf_full / lf_empty mbarriers) and goes on
// streaming; leapfrog warp q reads the row sums from TMEM quadrant q, the lanes
// the column group's warp q reads, and takes over that warp's columns and
// orbits, so the arithmetic and its order are the column group's.
template <typename TS, int T, int NST, int OPT, bool SPLIT, bool LFW = false, bool COMP = false>
__global__ void __launch_bounds__(2 * T * (KC / OPT) + 32 + (LFW ? T * (KC / OPT) : 0), 1)
memint_kernel(const RunDev *__restrict__ runs, const int *__restrict__ base, int nruns,
              const int *__restrict__ d_t, int *__restrict__ d_err, int measure, int nwhole, int use_maps,
              int nitems, int *__restrict__ queue, int parts) {
  using C = Cfg<TS, T, NST, OPT>;
  using V = Vec<TS, OPT>;
  using A = typename std::conditional<COMP, Acc<TS, OPT>, PlainAcc<TS, OPT>>::type;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TS *stages = reinterpret_cast<TS *>(smem_raw);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + (size_t)NST * C::STAGE_BYTES);
  uint64_t *empty = full + NST;
  // misc: [0] hartreecont, [1] M^2, [2..2+KC) acc_F(t-1) per orbit, [10] abort flag,
  // [11] tiles issued, [12] consumer abort flag, [13] current item, [14] TMEM address,
  // [15] the next item when the producer took it early (else -1),
  // [16..16+(NG/32)*KC) diagonal partials, [48..48+5*KC) the diagonal's inputs (epi),
  // [88..88+4*KC) its per-orbit tadpole and energy terms
  double *misc = reinterpret_cast<double *>(empty + NST);  // 128 doubles
  volatile int *abort_flag = reinterpret_cast<volatile int *>(misc + 10);
  volatile int *issued_count = reinterpret_cast<volatile int *>(misc + 11);
  // consumers leave the tile loop together: the flag is only written by
  // consumers and they all meet at the named barrier after the tile loop
  volatile int *cabort = reinterpret_cast<volatile int *>(misc + 12);
  static_assert(16 + (C::NG / 32) * KC <= 48 && 48 + 5 * KC <= 88 && 88 + 4 * KC <= 120, "misc scratch too small");
  // inputs of memint_epilogue for a whole chunk: k^2, degeneracy and F(t-1,t-1) of its
  // orbits from the producer warp once it has issued the item's tiles, F(t,t-1) and
  // F(t,t-2) from the leapfrog of those columns
  double *epi = misc + 48;
  // the item's run parameters in shared memory (runbuf[rb]): the loop reads them all
  // through, and a global read that misses L1 under the stream costs a round trip to
  // L2. The producer copies the next item's into runbuf[rb ^ 1] once it has taken it;
  // runctl[0]: that run (-1: none), runctl[1]: the current item's run if copied so
  RunDev *runbuf = reinterpret_cast<RunDev *>(misc + 130);
  volatile int *runctl = reinterpret_cast<volatile int *>(runbuf + 2);
  int rb = 0;
  static_assert(C::NG == 128, "one TMEM lane per row-group thread, column group in warps 0..3");
  volatile uint32_t *tmem_slot = reinterpret_cast<volatile uint32_t *>(misc + 14);
  // LFW: [120..122) lf_full, [122..124) lf_empty mbarriers; the hand-off stage
  // (two buffers of colF, colR per column-group thread) after the fixed region
  uint64_t *lf_full = reinterpret_cast<uint64_t *>(misc + 120);
  uint64_t *lf_empty = lf_full + 2;
  double *lf_stage = reinterpret_cast<double *>(smem_raw + smem_fixed_bytes<C>());

  const int tid = threadIdx.x;
  const bool producer = tid >= C::NT && tid < C::NT + 32;
  const bool lfwarp = LFW && tid >= C::NT + 32;  // leapfrog warps
  const bool colgrp = tid < C::NG;
  const bool rowgrp = tid >= C::NG && tid < C::NT;
  const int gtid = colgrp ? tid : tid - C::NG;  // index inside the group
  const int jq = gtid % C::NJ, loc = gtid / C::NJ;  // orbit group; column (col group) or row (row group)
  const int j0 = jq * OPT;                          // first orbit of this thread in the chunk
  const int lane = tid & 31, warp = tid >> 5;
  const int t = *d_t;
  volatile int *item_slot = reinterpret_cast<volatile int *>(misc + 13);
  volatile int *next_slot = reinterpret_cast<volatile int *>(misc + 15);
  // row sums in TMEM (FP32 history): one allocation for every item of the CTA
  constexpr bool kTmem = sizeof(TS) == 4;
  if (kTmem && warp == 0) tmem_alloc(const_cast<uint32_t *>(tmem_slot));
  if (tid == 0) {
    for (int q = 0; q < NST; ++q) {
      mbar_init(full + q, 1);
      mbar_init(empty + q, C::NW);  // one arrival per consumer warp
    }
    if (LFW)
      for (int q = 0; q < 2; ++q) {
        mbar_init(lf_full + q, C::NG / 32);   // column-group warps
        mbar_init(lf_empty + q, C::NG / 32);  // leapfrog warps
      }
    *next_slot = -1;
    runctl[0] = -1;
    fence_proxy_async();
  }
  if (kTmem) tmem_fence_before();
  __syncthreads();
  if (kTmem) tmem_fence_after();
  const uint32_t tbase = kTmem ? *tmem_slot : 0u;
  const uint32_t tlane = ((uint32_t)(warp & 3) * 32u) << 16;  // this warp's TMEM lanes
  int nb = 0;      // tiles this CTA streamed before the current item (stage barrier phases)
  int lb = 0;      // column blocks it handed to the leapfrog warps before the current item
  int cur_r = -1;  // run whose tadpole sum misc[0..1] holds
  int pre_issued = 0;  // producer warp: tiles of the coming item it issued during the last one
  bool first = true;
  for (;;) {
  if (tid == 0) {
    const int pre = *next_slot;  // taken by the producer during the previous item
    *next_slot = -1;
    runctl[1] = pre >= 0 ? runctl[0] : -1;
    runctl[0] = -1;
    *item_slot = pre >= 0 ? pre : queue ? atomicAdd(queue, 1) : (first ? (int)blockIdx.x : nitems);
  }
  __syncthreads();
  const int vb = *item_slot;
  first = false;
  if (vb >= nitems) break;
  const bool split = SPLIT && vb >= nwhole;
  const int item = split ? nwhole + (vb - nwhole) / parts : vb;
  const int part = split ? (vb - nwhole) % parts : 0;
  int r = runctl[1];
  if (r >= 0) {
    rb ^= 1;  // copied by the producer during the previous item
  } else {
    r = run_at(base, nruns, item);
    if (warp == 0) {
      const uint64_t *src = reinterpret_cast<const uint64_t *>(runs + r);
      uint64_t *dst = reinterpret_cast<uint64_t *>(runbuf + rb);
      for (int w = lane; w < (int)(sizeof(RunDev) / 8); w += 32) dst[w] = src[w];
    }
    __syncthreads();
  }
  const RunDev &R = runbuf[rb];
  const int c = item - R.cta_base_mi;  // chunk
  const int M = R.M, Ma = R.Malloc;
  const int tmin = max(1, t - M + 1);
  const size_t rowstride = (size_t)Ma * KC;              // one row of one chunk
  // row sums of this chunk, [Malloc][KC]: entries (slot, j0..j0+OPT-1) are only
  // ever written by row-group thread (slot mod T, jq), so they need no atomics.
  // With FP32 history they live in TMEM (Malloc/T slots x OPT doubles per lane)
  // when they fit, else in a global scratch slot; a split CTA copies them there
  // at the end (one buffer per part) for memint_finish_kernel. The FP64 kernel,
  // bound by FP64 arithmetic, runs 1 % faster on the global scratch.
  double *rowacc = R.rowacc + (size_t)part * R.nchunks * rowstride + (size_t)c * rowstride;
  const bool use_tmem = kTmem && (Ma / T) * OPT * 2 <= (int)TMEM_COLS;
  const bool use_tmap = (use_maps & 1) && R.tmap != nullptr;
  const bool no_tiles = (use_maps & 2) != 0;  // test hook: nothing is issued, the consumers' waits run out

  // --- tadpole mass M^2(t-1) from the per-chunk sums of F(t-1,t-1) (fixed order), once per run
  if (r != cur_r && warp == 0) {
    const double *tad = R.tad + (size_t)((t - 1) & 1) * R.nchunks;
    double s = tad_lane_sum(tad, R.nchunks, lane);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      misc[0] = s;                          // hartreecont = sum_k deg_k F(t-1,t-1,k)
      misc[1] = s * R.pref_ivol + R.mass2;  // getHartreeMass2 order: (sum * (pref*ivol)) + Mass2
    }
  }
  cur_r = r;
  if (tid < KC) misc[2 + tid] = 0.0;
  if (tid == 0) {
    *abort_flag = 0;
    *issued_count = 0;
    *cabort = 0;
  }
  if (!use_tmem && rowgrp)
    for (int s = loc; s < Ma; s += T)  // the slots this thread owns
      for (int o = 0; o < OPT; ++o) rowacc[(size_t)s * KC + j0 + o] = 0.0;
  if (use_tmem) tmem_fence_before();
  __syncthreads();
  if (use_tmem) tmem_fence_after();
  const double M2 = misc[1];
  if (SPLIT && c == 0 && part == 0 && tid == 0) {  // for memint_finish_kernel
    R.hcm2[0] = misc[0];
    R.hcm2[1] = misc[1];
  }
  // TMEM column of the row sums of slot s (s mod T is the thread's loc)
  auto tcol = [&](int s) { return tbase + tlane + (uint32_t)((s / T) * OPT * 2); };
  if (use_tmem && rowgrp) {
    const double zero[OPT] = {};
    for (int s = 0; s < Ma; s += T) TmemRow<OPT>::st(tcol(s), zero);
  }
  // whole chunks of an LFW kernel leave their leapfrog to the leapfrog warps
  const bool lf_on = LFW && !split;

  const bool lo_only = pexp_lo(R.pexp);
  const int J0 = tmin / T, Jn = (t - 1) / T;
  // column blocks of this item: all of them, or one part of the triangle
  const int Jlo = split ? split_bound(J0, Jn, parts, part) : J0;
  const int Jhi = split ? split_bound(J0, Jn, parts, part + 1) - 1 : Jn;
  int ntiles = 0;
  if (!lo_only)
    for (int J = Jlo; J <= Jhi; ++J) ntiles += Jn - J + 1;

  if (producer) {
    // ---------------- producer warp: stream every tile of its column blocks once
    TileIt it{Jlo, Jlo, Jn};
    const int n0 = min(pre_issued, ntiles);  // already issued at the end of the previous item
    for (int q = 0; q < n0; ++q) it.next();
    pre_issued = 0;
    if (lane == 0) *issued_count = n0;
    for (int n = n0; n < ntiles; ++n, it.next()) {
      const int gn = nb + n;  // the CTA's tile count picks the stage and its phase
      const int stage = gn % NST;
      if (gn >= NST && !mbar_wait_bounded(empty + stage, (uint32_t)(((gn / NST) - 1) & 1))) {
        if (lane == 0) {
          *abort_flag = 1;
          atomicOr(d_err, DEVERR_TIMEOUT);
        }
        break;
      }
      if (*abort_flag || no_tiles) break;
      issue_tile<TS, C>(stage, it.I, it.J, R, c, stages, full, tmin, t - 1, use_tmap);
      if (lane == 0) *issued_count = n + 1;
    }
    // the diagonal's inputs that are not written in this step (the loads are in flight
    // while the tiles stream; the epilogue finds them in shared memory)
    if (!split && lane < KC) {
      const int kd = c * KC + lane;
      const bool kin = kd < R.S;
      const size_t st_row = (size_t)R.nchunks * rowstride;
      epi[lane] = kin ? R.k2[kd] : 0.0;
      epi[KC + lane] = kin ? R.deg[kd] : 0.0;
      epi[2 * KC + lane] = R.st_F[(size_t)((t - 1) % 3) * st_row + (size_t)c * rowstride + (size_t)((t - 1) % Ma) * KC + lane];
    }
    // with every tile of this item issued, take the next item now: its first tiles
    // go to L2 at once and into the stage ring as soon as this item's last tiles
    // release their stages, so that they load while the consumers finish this item
    if (queue && !no_tiles) {
      int nv = nitems;
      if (lane == 0 && !*abort_flag) {
        nv = atomicAdd(queue, 1);
        *next_slot = nv;
      }
      nv = __shfl_sync(0xffffffffu, nv, 0);
      if (nv < nitems) {
        const bool s2 = SPLIT && nv >= nwhole;
        const int it2 = s2 ? nwhole + (nv - nwhole) / parts : nv;
        const int p2 = s2 ? (nv - nwhole) % parts : 0;
        const int r2 = run_at(base, nruns, it2);
        const RunDev &R2 = runs[r2];
        {  // the next item's run parameters into the buffer the current item does not use
          const uint64_t *src = reinterpret_cast<const uint64_t *>(runs + r2);
          uint64_t *dst = reinterpret_cast<uint64_t *>(runbuf + (rb ^ 1));
          for (int w = lane; w < (int)(sizeof(RunDev) / 8); w += 32) dst[w] = src[w];
          __syncwarp();
          if (lane == 0) runctl[0] = r2;
        }
        const int c2 = it2 - R2.cta_base_mi;
        const int tmin2 = max(1, t - R2.M + 1), J02 = tmin2 / T, Jn2 = (t - 1) / T;
        const int Jlo2 = s2 ? split_bound(J02, Jn2, parts, p2) : J02;
        const int Jhi2 = s2 ? split_bound(J02, Jn2, parts, p2 + 1) - 1 : Jn2;
        int nt2 = 0;
        if (!pexp_lo(R2.pexp))
          for (int J = Jlo2; J <= Jhi2 && nt2 < NST; ++J) nt2 += Jn2 - J + 1;
        nt2 = min(nt2, NST);
        const bool tmap2 = (use_maps & 1) && R2.tmap != nullptr;
        if (tmap2 && lane == 0) {
          const int nbk = R2.Malloc / T;
          TileIt i2{Jlo2, Jlo2, Jn2};
          for (int q = 0; q < nt2; ++q, i2.next()) {
            const int tile = (c2 * nbk + ((i2.I * T) % R2.Malloc) / T) * nbk + ((i2.J * T) % R2.Malloc) / T;
            const char *tm = reinterpret_cast<const char *>(R2.tmap);
            tma_prefetch_3d(tm, 0, 0, tile);
            tma_prefetch_3d(tm + 128, 0, 0, tile);
          }
        }
        // the coming item's tiles continue this CTA's tile count: tile q of it is
        // tile ntiles + q of this item's count (the stage and phase it will be waited on)
        TileIt i2{Jlo2, Jlo2, Jn2};
        for (int q = 0; q < nt2; ++q, i2.next()) {
          const int gn = nb + ntiles + q;
          const int stage = gn % NST;
          const bool ok = gn < NST || mbar_wait_bounded(empty + stage, (uint32_t)(((gn / NST) - 1) & 1));
          if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) {
              *abort_flag = 1;
              atomicOr(d_err, DEVERR_TIMEOUT);
            }
            break;
          }
          if (__any_sync(0xffffffffu, *abort_flag != 0)) break;  // a consumer gave up: issue no more
          issue_tile<TS, C>(stage, i2.I, i2.J, R2, c2, stages, full, tmin2, t - 1, tmap2);
          pre_issued = q + 1;
          if (lane == 0) *issued_count = ntiles + q + 1;  // drained with this item's tiles on an abort
        }
      }
    }
    __syncwarp();
  } else if (lfwarp) {
    // ---------------- leapfrog warps (whole chunks of an LFW kernel)
    if (lf_on) {
      const int lq = warp & 3;         // TMEM quadrant of this warp
      const int lg = lq * 32 + lane;   // the column-group thread whose columns and orbits this lane takes
      const int lj0 = (lg % C::NJ) * OPT, lloc = lg / C::NJ;
      double diag[OPT], emem[OPT];
      for (int o = 0; o < OPT; ++o) diag[o] = emem[o] = 0.0;
      bool has_emem = false, ok = true;
      // the state and Sigma entries of this lane's column of the last block go to L2 one
      // block ahead: the step's stream has long evicted them, and that block's leapfrog,
      // which nothing overlaps, would otherwise wait on DRAM (an earlier block's runs
      // while tiles stream, and a prefetch a long column ahead would be evicted again)
      auto lf_prefetch = [&](int J) {
        const int b = J * T + lloc;
        if (J > Jhi || b < tmin || b > t - 1) return;
        const size_t str = (size_t)R.nchunks * rowstride, o = (size_t)c * rowstride + (size_t)(b % Ma) * KC + lj0;
        prefetch_l2g(R.st_F + (size_t)((t - 1) % 3) * str + o);
        prefetch_l2g(R.st_F + (size_t)((t - 2) % 3) * str + o);
        prefetch_l2g(R.st_r + (size_t)((t - 1) % 3) * str + o);
        prefetch_l2g(R.st_r + (size_t)((t - 2) % 3) * str + o);
        prefetch_l2g(reinterpret_cast<const TS *>(R.sig_r) + o);
        prefetch_l2g(reinterpret_cast<const TS *>(R.sig_F) + o);
      };
      if (Jlo == Jhi) lf_prefetch(Jlo);
      for (int J = Jlo; J <= Jhi; ++J) {
        if (J + 1 == Jhi) lf_prefetch(J + 1);
        const int slot = (lb + J - Jlo) & 1, use = (lb + J - Jlo) >> 1;
        ok = __all_sync(0xffffffffu, lf_wait(lf_full + slot, (uint32_t)(use & 1), cabort));
        if (!ok) break;
        if (use_tmem) tmem_fence_after();
        const double *stg = lf_stage + ((size_t)slot * C::NG + lg) * 2 * OPT;
        double colF[OPT], colR[OPT], rowb[OPT];
        for (int o = 0; o < OPT; ++o) {
          colF[o] = stg[o];
          colR[o] = stg[OPT + o];
        }
        if (use_tmem) TmemRow<OPT>::ld(tcol((J * T) % Ma), rowb);
        __syncwarp();
        if (lane == 0) mbar_arrive(lf_empty + slot);
        const int b = J * T + lloc;
        if (b >= tmin && b <= t - 1) {
          if (!use_tmem)
            for (int o = 0; o < OPT; ++o) rowb[o] = rowacc[(size_t)(b % Ma) * KC + lj0 + o];
          leapfrog_column<TS, OPT>(R, c, t, tmin, b, lj0, M2, lo_only, colF, colR, rowb, diag, emem, has_emem,
                                   epi + 3 * KC);
        }
      }
      if (ok) {
        // partial sums of acc_F(t) as the column group's warp lq would form them
        for (int o = 0; o < OPT; ++o) {
          double v = diag[o];
#pragma unroll
          for (int off = 16; off >= C::NJ; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
          if (lane < C::NJ) misc[16 + lq * KC + lj0 + o] = v;
          if (has_emem) misc[2 + lj0 + o] = emem[o];
        }
      } else if (lane == 0) {
        *abort_flag = 1;
        atomicOr(d_err, DEVERR_TIMEOUT);
      }
    }
  } else {
    // ---------------- consumers
    double diag[OPT];  // acc_F(t) for the diagonal, partial over this thread's columns
    double emem[OPT];  // acc_F(t-1), kept by the thread of column t-1
    for (int o = 0; o < OPT; ++o) diag[o] = emem[o] = 0.0;
    bool has_emem = false;
    bool aborted = false;
    int n = 0;  // tiles consumed
    // row group: accumulator of the row of the next tile, loaded one tile ahead
    double pre[OPT];
    for (int o = 0; o < OPT; ++o) pre[o] = 0.0;
    if (!colgrp) {
      const int a0 = Jlo * T + loc;
      if (a0 >= tmin && a0 <= t - 1)
        for (int o = 0; o < OPT; ++o) pre[o] = rowacc[(size_t)(a0 % Ma) * KC + j0 + o];
    }

    for (int J = Jlo; J <= Jhi && !aborted; ++J) {
      const int b = J * T + loc;  // column of a column-group thread
      const bool bvalid = colgrp && (b >= tmin) && (b <= t - 1);
      double colF[OPT], colR[OPT];
      for (int o = 0; o < OPT; ++o) colF[o] = colR[o] = 0.0;

      for (int I = lo_only ? Jn + 1 : J; I <= Jn; ++I, ++n) {
        const int gn = nb + n;
        const int stage = gn % NST;
        bool ok = !*cabort && mbar_wait_bounded(full + stage, (uint32_t)((gn / NST) & 1));
        ok = __all_sync(0xffffffffu, ok);  // warp-uniform decision
        if (!ok) {
          // a wait expired here or in another consumer: leave the tile loop; all
          // consumers meet at the named barrier that closes this column block
          *abort_flag = 1;  // stops the producer
          *cabort = 1;
          atomicOr(d_err, DEVERR_TIMEOUT);
          aborted = true;
          break;
        }
        const TS *sbase = stages + (size_t)stage * C::STAGE;
        int r0 = 0, x0 = 0;  // origin of the tensor-map box in the tile (see tile_box)
        if (use_tmap) tile_box<C>(I, J, tmin, t - 1, r0, x0);
        const TS *tF = sbase - ((ptrdiff_t)r0 * C::RS + x0);
        const TS *tR = tF + C::TILE;
        const TS *xr_row = sbase + 2 * C::TILE;
        const TS *xr_col = xr_row + C::XV;
        const TS *xF_col = xr_col + C::XV;
        if (colgrp) {
          // column sums over the valid rows a of the tile: a in [max(b, tmin), t-1]
          int lo = max(b, tmin) - I * T, hi = min(T - 1, t - 1 - I * T);
          if (!bvalid) hi = -1;
          lo = max(lo, 0);
          A cF0 = A::zero(), cF1 = A::zero(), cR0 = A::zero(), cR1 = A::zero();
          // column loc of row rr sits at swizzled position loc ^ (rr & 3)
          auto el = [&](int rr) { return rr * C::RS + (loc ^ (rr & 3)) * KC + j0; };
          const TS *xb = xr_row + j0;
          int rr = lo;
          if (rr <= hi && I * T + rr == tmin) {  // trapezoid half weight of z = tmin
            V x = V::ld(xb + rr * KC);
            x.scale((TS)0.5);
            cF0.fma(x, V::ld(tF + el(rr)));
            cR0.fma(x, V::ld(tR + el(rr)));
            ++rr;
          }
#pragma unroll 8  // 16 rows of loads in flight (8 measured 0.7 % faster than 4 at Ns = 64)
          for (; rr + 1 <= hi; rr += 2) {
            const V x0 = V::ld(xb + rr * KC), x1 = V::ld(xb + (rr + 1) * KC);
            const int e0 = el(rr), e1 = el(rr + 1);
            cF0.fma(x0, V::ld(tF + e0));
            cR0.fma(x0, V::ld(tR + e0));
            cF1.fma(x1, V::ld(tF + e1));
            cR1.fma(x1, V::ld(tR + e1));
          }
          if (rr <= hi) {
            const V x0 = V::ld(xb + rr * KC);
            cF0.fma(x0, V::ld(tF + el(rr)));
            cR0.fma(x0, V::ld(tR + el(rr)));
          }
          cF0.add(cF1);
          cR0.add(cR1);
          for (int o = 0; o < OPT; ++o) {
            colF[o] += cF0.get(o);
            colR[o] += cR0.get(o);
          }
          __syncwarp();
          if (lane == 0) mbar_arrive(empty + stage);
        } else {
          // row sums over the valid columns b of the tile: b in [tmin, a-1]; row a = I*T + loc
          const int a = I * T + loc;
          const bool av = (a >= tmin) && (a <= t - 1);
          (void)KB_DCHECK(!use_tmem || ((I * T) % Ma) / T * OPT * 2 + OPT * 2 <= (int)TMEM_COLS, R.err, DCHK_MI_ROW);
          double *racc = rowacc + (size_t)(a % Ma) * KC + j0;
          double prev[OPT];
          int an = -1;
          if (use_tmem) {
            TmemRow<OPT>::ld(tcol((I * T) % Ma), prev);  // the same column for the whole warp
          } else {
            // the accumulator of this row was loaded during the previous tile; load the
            // next tile's row now (tile order: (I+1, J), or (J+1, J+1) after the last row block)
            for (int o = 0; o < OPT; ++o) prev[o] = pre[o];
            an = (I < Jn ? (I + 1) : (J + 1)) * T + loc;
            if (an != a && an >= tmin && an <= t - 1)  // an == a: the value stored below is the next one
              for (int o = 0; o < OPT; ++o) pre[o] = rowacc[(size_t)(an % Ma) * KC + j0 + o];
          }
          int lo = max(0, tmin - J * T), hi = min(T - 1, a - 1 - J * T);
          if (!av) hi = -1;
          A s0 = A::zero(), s1 = A::zero();
          // column bb of row loc sits at swizzled position bb ^ (loc & 3)
          const int sw = loc & 3;
          const TS *fr = tF + loc * C::RS + j0;
          const TS *qr = tR + loc * C::RS + j0;
          const TS *xrc = xr_col + j0;
          const TS *xFc = xF_col + j0;
          int bb = lo;
          if (bb <= hi && J * T + bb == tmin) {  // trapezoid half weight of z = tmin
            V x = V::ld(xrc + bb * KC), y = V::ld(xFc + bb * KC);
            x.scale((TS)0.5);
            y.scale((TS)0.5);
            s0.fma(x, V::ld(fr + (bb ^ sw) * KC));
            s0.fma(y, V::ld(qr + (bb ^ sw) * KC));
            ++bb;
          }
#pragma unroll 8
          for (; bb + 1 <= hi; bb += 2) {
            const int e0 = (bb ^ sw) * KC, e1 = ((bb + 1) ^ sw) * KC;
            s0.fma(V::ld(xrc + bb * KC), V::ld(fr + e0));
            s0.fma(V::ld(xFc + bb * KC), V::ld(qr + e0));
            s1.fma(V::ld(xrc + (bb + 1) * KC), V::ld(fr + e1));
            s1.fma(V::ld(xFc + (bb + 1) * KC), V::ld(qr + e1));
          }
          if (bb <= hi) {
            s0.fma(V::ld(xrc + bb * KC), V::ld(fr + (bb ^ sw) * KC));
            s0.fma(V::ld(xFc + bb * KC), V::ld(qr + (bb ^ sw) * KC));
          }
          s0.add(s1);
          __syncwarp();
          if (lane == 0) mbar_arrive(empty + stage);
          if (use_tmem) {
            double nv[OPT];
            for (int o = 0; o < OPT; ++o) nv[o] = av ? prev[o] + s0.get(o) : prev[o];
            TmemRow<OPT>::st(tcol((I * T) % Ma), nv);
          } else if (av) {
            for (int o = 0; o < OPT; ++o) {
              const double v = prev[o] + s0.get(o);
              racc[o] = v;
              if (an == a) pre[o] = v;
            }
          }
        }
      }
      // both groups: the row sums of column block J are final after its diagonal tile
      if (use_tmem) tmem_fence_before();
      consumer_sync(C::NT);
      if (use_tmem) tmem_fence_after();
      if (*cabort) {
        aborted = true;
        break;
      }

      if (split) {  // column sums of this block, for memint_finish_kernel
        if (bvalid)
          for (int o = 0; o < OPT; ++o) {
            R.colacc[(size_t)c * rowstride + (size_t)(b % Ma) * KC + j0 + o] = colF[o];
            R.colacc[(size_t)(R.nchunks + c) * rowstride + (size_t)(b % Ma) * KC + j0 + o] = colR[o];
          }
        continue;
      }
      if (lf_on) {  // column sums of this block to the leapfrog warps
        if (colgrp) {
          const int slot = (lb + J - Jlo) & 1, use = (lb + J - Jlo) >> 1;
          // the buffer's previous block must have been read; a wait that runs out
          // aborts the chunk at the next tile wait of every consumer
          if (use > 0 && !mbar_wait_bounded(lf_empty + slot, (uint32_t)((use - 1) & 1))) {
            *abort_flag = 1;
            *cabort = 1;
            atomicOr(d_err, DEVERR_TIMEOUT);
            continue;
          }
          double *stg = lf_stage + ((size_t)slot * C::NG + gtid) * 2 * OPT;
          for (int o = 0; o < OPT; ++o) {
            stg[o] = colF[o];
            stg[OPT + o] = colR[o];
          }
          __syncwarp();
          if (lane == 0) mbar_arrive(lf_full + slot);
        }
        continue;
      }
      // leapfrog for t' = b; the row sums of row b come from the row-group thread
      // on this thread's TMEM lane
      double rowb[OPT];
      if (use_tmem) TmemRow<OPT>::ld(tcol((J * T) % Ma), rowb);
      if (bvalid) {
        if (!use_tmem)
          for (int o = 0; o < OPT; ++o) rowb[o] = rowacc[(size_t)(b % Ma) * KC + j0 + o];
        leapfrog_column<TS, OPT>(R, c, t, tmin, b, j0, M2, lo_only, colF, colR, rowb, diag, emem, has_emem,
                                 split ? nullptr : epi + 3 * KC);
      }
    }
    if (!split && !lf_on && !aborted && colgrp) {
      // partial sums of acc_F(t) over this warp's columns (lanes sharing jq)
      for (int o = 0; o < OPT; ++o) {
        double v = diag[o];
#pragma unroll
        for (int off = 16; off >= C::NJ; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane < C::NJ) misc[16 + warp * KC + j0 + o] = v;
        if (has_emem) misc[2 + j0 + o] = emem[o];
      }
    }
  }
  if (use_tmem) tmem_fence_before();
  __syncthreads();  // producer done issuing; consumers done with the triangle
  if (use_tmem) tmem_fence_after();
  const bool aborted_item = *abort_flag != 0;  // read by every thread between two barriers
  if (aborted_item) {
    // drain copies still in flight into this CTA's shared memory: only the last NST
    // issued tiles can be (the producer reuses a stage after its consumers release it),
    // and for those the stage barrier's latest phase is theirs; an older tile's phase
    // parity repeats on its stage, so waiting on it would run to the bound
    if (tid == 0)
      for (int q = max(0, *issued_count - NST); q < *issued_count; ++q)
        (void)mbar_wait_bounded(full + ((nb + q) % NST), (uint32_t)(((nb + q) / NST) & 1));
  } else {
    if (split && use_tmem && rowgrp)  // this part's row sums, for memint_finish_kernel
      for (int s = 0; s < Ma; s += T) {
        double v[OPT];
        TmemRow<OPT>::ld(tcol(s), v);
        for (int o = 0; o < OPT; ++o) rowacc[(size_t)(s + loc) * KC + j0 + o] = v[o];
      }
    if (!split) {
      // two orbits on each of warps 0..3, one warp per SM sub-partition
      if (warp < KC / 2 && lane < 2)
        memint_epilogue<TS>(R, c, t, 2 * warp + lane, misc, C::NG / 32, M2, measure, epi, misc + 88);
      __syncthreads();
      if (warp < 4 && lane == 0) memint_epilogue_sum(R, c, t, warp, misc + 88, M2, measure);
    }
  }
  nb += ntiles;
  if (lf_on) lb += Jhi - Jlo + 1;
  if (use_tmem) tmem_fence_before();
  __syncthreads();  // the item's TMEM reads and misc values are done with
  if (use_tmem) tmem_fence_after();
  // a wait that ran out leaves this CTA's stage barriers mid-phase: it takes no more
  // items (the others go on taking them; the error word reports the timeout)
  if (aborted_item) break;
  }  // items
  if (kTmem) {  // every path ends here: the allocating warp frees the TMEM
    tmem_fence_before();
    __syncthreads();
    if (warp == 0) {
      tmem_fence_after();
      tmem_dealloc(tbase);
    }
  }
}

// Second kernel of a split step: CTA (chunk, k) takes the FIN_TP t' from tmin +
// k FIN_TP on, FIN_IT (t', orbit) items per thread with all their loads issued
// before any arithmetic. It adds the column sums and the parts' row sums (in part order),
// runs the leapfrog (the same arithmetic as memint_kernel's) and stores its
// per-orbit sums of the acc_F(t) terms; the CTA of the chunk that arrives last
// adds those in CTA order and runs the diagonal and measurement (no CTA waits
// for another).
constexpr int FIN_THREADS = 256;
constexpr int FIN_IT = FIN_TP * KC / FIN_THREADS;
static_assert(FIN_IT * FIN_THREADS == FIN_TP * KC, "whole items per thread");

// FP32 history: four CTAs per SM (64 registers, about 120 bytes of spills), which
// overlaps more of the loads with the FP64 arithmetic than two CTAs per SM with
// 128 registers, or 512-thread CTAs with two items per thread, did when timed
template <typename TS>
__global__ void __launch_bounds__(FIN_THREADS, sizeof(TS) == 4 ? 4 : 2)
memint_finish_kernel(const RunDev *__restrict__ runs, const int *__restrict__ base, int nruns, int nb_max,
                     int nwhole, const int *__restrict__ d_t, int measure, int parts) {
  __shared__ double red[FIN_THREADS / 32][KC];
  __shared__ double misc[16 + KC];
  __shared__ int is_last;
  const int ci = nwhole + (int)blockIdx.x / nb_max, blk = (int)blockIdx.x % nb_max;
  const int r = run_at(base, nruns, ci);
  const RunDev &R = runs[r];
  const int c = ci - R.cta_base_mi;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t = *d_t;
  const int Ma = R.Malloc, T = R.T;
  const int tmin = max(1, t - R.M + 1);
  const int nq = (t - tmin) * KC;
  const int nact = (nq + FIN_TP * KC - 1) / (FIN_TP * KC);  // CTAs of this chunk with work (<= fin_nb)
  if (blk >= nact) return;
  const size_t rowstride = (size_t)Ma * KC, st_row = (size_t)R.nchunks * rowstride, cs = (size_t)c * rowstride;
  const size_t pbuf = (size_t)R.nchunks * rowstride;  // one row-sum buffer, and the rho column sums' offset
  const double M2 = R.hcm2[1];
  const bool lo_only = pexp_lo(R.pexp);
  const int j = tid % KC;  // FIN_THREADS is a multiple of KC: one orbit per thread
  const int k = c * KC + j;
  const double om = (((k < R.S) ? R.k2[k] : 0.0) + M2) * R.dt2;
  const double *F1 = R.st_F + (size_t)((t - 1) % 3) * st_row, *F2 = R.st_F + (size_t)((t - 2) % 3) * st_row;
  const double *R1 = R.st_r + (size_t)((t - 1) % 3) * st_row, *R2 = R.st_r + (size_t)((t - 2) % 3) * st_row;
  const TS *sr = reinterpret_cast<const TS *>(R.sig_r), *sf = reinterpret_cast<const TS *>(R.sig_F);
  // GB300 runs FP64 at about 1/64 of the FP32 rate and this kernel is bound by
  // it: the leapfrog is written as FMAs, and the acc_F(t) terms x * F(t,t') are
  // formed in the history's type from the values stored anyway (up to FIN_IT
  // terms per thread, as the memory integrals form theirs per tile) and summed
  // in FP64 from there on.
  const double c2 = 2.0 - om, dt3 = R.dt3;
  TS xr[FIN_IT], xf[FIN_IT];
  double aF[FIN_IT], aR[FIN_IT], f1[FIN_IT], f2[FIN_IT], r1[FIN_IT], r2[FIN_IT];
#pragma unroll
  for (int u = 0; u < FIN_IT; ++u) {
    const int q = blk * FIN_TP * KC + u * FIN_THREADS + tid;
    const int b = tmin + min(q, nq - 1) / KC;  // items past the window repeat the last one (not stored)
    const size_t e = cs + (size_t)(b % Ma) * KC + j;
    xr[u] = lo_only ? (TS)0 : sr[e];
    xf[u] = lo_only ? (TS)0 : sf[e];
    double rsum = R.rowacc[e] + R.rowacc[pbuf + e];
    for (int p = 2; p < parts; ++p) rsum += R.rowacc[(size_t)p * pbuf + e];
    aF[u] = R.colacc[e] + rsum;
    aR[u] = R.colacc[pbuf + e];
    f1[u] = F1[e];
    f2[u] = (b <= t - 2) ? F2[e] : F1[cs + (size_t)((t - 2) % Ma) * KC + j];
    r1[u] = R1[e];
    r2[u] = R2[e];
  }
  TS dp = (TS)0;
  bool wrote_shared = false;  // stores the last CTA reads: acc_F(t-1), F(t,t-1), F(t,t-2)
#pragma unroll
  for (int u = 0; u < FIN_IT; ++u) {
    const int q = blk * FIN_TP * KC + u * FIN_THREADS + tid;
    if (q >= nq) break;
    const int b = tmin + q / KC;
    if (!KB_DCHECK(b >= tmin && b <= t - 1 && t - b < R.M && c >= 0 && c < R.nchunks, R.err, DCHK_FIN)) break;
    const size_t e = cs + (size_t)(b % Ma) * KC + j;
    const double Fn = fma(c2, f1[u], -fma(aF[u], dt3, f2[u]));
    const double rn = (b == t - 1) ? R.dt : fma(c2, r1[u], -fma(aR[u], dt3, r2[u]));
    R.st_F[(size_t)(t % 3) * st_row + e] = Fn;
    R.st_r[(size_t)(t % 3) * st_row + e] = rn;
    const TS Fs = (TS)Fn, rs = (TS)rn;
    const size_t ho = hist_off(Ma, T, c, t, b, j);
    reinterpret_cast<TS *>(R.hist_F)[ho] = Fs;
    reinterpret_cast<TS *>(R.hist_r)[ho] = rs;
    const TS wb = (b == tmin) ? (TS)0.5 : (TS)1;
    dp += (wb * xr[u]) * Fs + (wb * xf[u]) * rs;
    if (b == t - 1) R.fin_prev[(size_t)c * KC + j] = aF[u];
    if (b >= t - 2) wrote_shared = true;
  }
  double d = (double)dp;
  // per-orbit sums over this CTA's t' in a fixed order: lanes l, l^8, l^16, l^24 share an orbit
  d += __shfl_xor_sync(0xffffffffu, d, 8);
  d += __shfl_xor_sync(0xffffffffu, d, 16);
  if (lane < KC) red[warp][lane] = d;
  __syncthreads();
  if (tid < KC) {
    double s = 0.0;
    for (int w = 0; w < FIN_THREADS / 32; ++w) s += red[w][tid];
    R.fin_part[((size_t)c * R.fin_nb + blk) * KC + tid] = s;
    wrote_shared = true;
  }
  // arrival: the stores the last CTA reads are published before the count moves
  if (wrote_shared) __threadfence();
  __syncthreads();
  if (tid == 0) {
    const int old = atomicAdd(R.fin + c, 1);
    is_last = (old == nact - 1);
    if (is_last) R.fin[c] = 0;  // all CTAs of the chunk are in: reset for the next step
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (tid < KC) {
    double s = 0.0;
    for (int k2 = 0; k2 < nact; ++k2) s += __ldcg(R.fin_part + ((size_t)c * R.fin_nb + k2) * KC + tid);
    misc[16 + tid] = s;
    misc[2 + tid] = __ldcg(R.fin_prev + (size_t)c * KC + tid);
  }
  if (tid == 0) misc[0] = R.hcm2[0];
  __syncthreads();
  if (tid < KC) memint_epilogue<TS>(R, c, t, tid, misc, 1, M2, measure);
}

// ---------------------------------------------------------------------------
// FP32 history, register-blocked consumers. Same pipeline, tile order, row
// accumulator and epilogue as memint_kernel, but every consumer thread owns a
// 4 x 4 block of (row, column) pairs of each tile for 2 adjacent orbits, so
// each F and rho element is read from shared memory once (memint_kernel reads
// it twice, once per consumer group; shared-memory wavefronts bound its CTA).
//   warp w        : tile rows 4w .. 4w+3
//   lane          : columns (lane >> 2) + 8k, k = 0..3; orbits 2 (lane & 3) + {0,1}
// A warp-wide 8-byte load covers 8 consecutive columns of one row (256
// contiguous bytes under the XOR swizzle, conflict-free). Row sums of a tile
// are reduce-scattered over the 8 column lanes (7 shuffles) so that every lane
// ends with one (row, orbit) sum, which it adds to its FP64 row accumulator.
// Column partials are summed in FP32 over at most 8 tiles (32 rows, as the
// per-tile partials of memint_kernel), then in FP64; at the end of a column
// block the 8 warps' column sums meet in shared memory and one thread per
// (column, orbit) runs the leapfrog.
// ---------------------------------------------------------------------------
constexpr int BLK_COLBUF_BYTES = 8 * 32 * KC * (int)sizeof(double);

template <int NST>
__global__ void __launch_bounds__(288)
memint_blk_kernel(const RunDev *__restrict__ runs, const int *__restrict__ base, int nruns,
                  const int *__restrict__ d_t, int *__restrict__ d_err, int measure) {
  using C = Cfg<float, 32, NST, 2>;
  using V = Vec<float, 2>;
  constexpr int T = 32, NT = 256;
  static_assert(C::NT == NT, "256 consumer threads");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float *stages = reinterpret_cast<float *>(smem_raw);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + (size_t)NST * C::STAGE_BYTES);
  uint64_t *empty = full + NST;
  // misc: [0] hartreecont, [1] M^2, [2..2+KC) acc_F(t-1) per orbit, [10] abort flag,
  // [11] tiles issued, [12] consumer abort flag, [16..16+8*KC) diagonal partials
  double *misc = reinterpret_cast<double *>(empty + NST);
  double *colbuf = misc + 128;  // [8 warps][32 columns][KC] column partials of one field
  volatile int *abort_flag = reinterpret_cast<volatile int *>(misc + 10);
  volatile int *issued_count = reinterpret_cast<volatile int *>(misc + 11);
  volatile int *cabort = reinterpret_cast<volatile int *>(misc + 12);

  const int r = run_at(base, nruns, blockIdx.x);
  const RunDev &R = runs[r];
  const int c = blockIdx.x - R.cta_base_mi;  // chunk
  const int tid = threadIdx.x;
  const bool producer = tid >= NT;
  const int lane = tid & 31, warp = tid >> 5;
  const int jq = lane & 3, c8 = lane >> 2;
  const int j0 = 2 * jq;
  // (row, orbit) owned after the reduce-scatter of the row sums
  const int own_rr = 4 * warp + 2 * ((lane >> 4) & 1) + ((lane >> 3) & 1);
  const int own_j = j0 + ((lane >> 2) & 1);
  const int t = *d_t;
  const int M = R.M, Ma = R.Malloc;
  const int tmin = max(1, t - M + 1);
  const size_t rowstride = (size_t)Ma * KC;
  const size_t st_row = (size_t)R.nchunks * rowstride;
  double *rowacc = R.rowacc + (size_t)c * rowstride;

  if (warp == 0) {
    const double *tad = R.tad + (size_t)((t - 1) & 1) * R.nchunks;
    double s = tad_lane_sum(tad, R.nchunks, lane);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      misc[0] = s;
      misc[1] = s * R.pref_ivol + R.mass2;
    }
  }
  if (tid < KC) misc[2 + tid] = 0.0;
  if (tid == 0) {
    *abort_flag = 0;
    *issued_count = 0;
    *cabort = 0;
    for (int q = 0; q < NST; ++q) {
      mbar_init(full + q, 1);
      mbar_init(empty + q, C::NW);
    }
    fence_proxy_async();
  }
  if (!producer)
    for (int s = own_rr; s < Ma; s += T) rowacc[(size_t)s * KC + own_j] = 0.0;
  __syncthreads();
  const double M2 = misc[1];

  const bool lo_only = pexp_lo(R.pexp);
  const int J0 = tmin / T, Jn = (t - 1) / T;
  const int nb = Jn - J0 + 1;
  const int ntiles = lo_only ? 0 : nb * (nb + 1) / 2;

  if (producer) {
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
      issue_tile<float, C>(stage, it.I, it.J, R, c, stages, full, tmin, t - 1, false);
      if (lane == 0) *issued_count = n + 1;
    }
    __syncwarp();
  } else {
    const double dt3 = R.dt3;
    double diag = 0.0, emem = 0.0;  // for (column loc, orbit jj) of the leapfrog thread
    bool has_emem = false, aborted = false;
    const int lf_loc = tid >> 3, lf_j = tid & 7;  // leapfrog thread: column, orbit
    int n = 0;
    double pre = 0.0;  // row accumulator of the owned row of the current tile
    {
      const int a0 = J0 * T + own_rr;
      if (a0 >= tmin && a0 <= t - 1) pre = rowacc[(size_t)(a0 % Ma) * KC + own_j];
    }
    for (int J = J0; J <= Jn && !aborted; ++J) {
      double colD[2][4][2];  // [F, rho][k][orbit]: FP64 column sums of this thread
      V colP[2][4];          // FP32 partials, flushed to colD every 8 tiles
      for (int k = 0; k < 4; ++k) {
        colP[0][k] = V::zero();
        colP[1][k] = V::zero();
        for (int o = 0; o < 2; ++o) colD[0][k][o] = colD[1][k][o] = 0.0;
      }
      int nin = 0;  // tiles of this column block consumed
      for (int I = lo_only ? Jn + 1 : J; I <= Jn; ++I, ++n, ++nin) {
        const int stage = n % NST;
        bool ok = !*cabort && mbar_wait_bounded(full + stage, (uint32_t)((n / NST) & 1));
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) {
          *abort_flag = 1;
          *cabort = 1;
          atomicOr(d_err, DEVERR_TIMEOUT);
          aborted = true;
          break;
        }
        const float *tF = stages + (size_t)stage * C::STAGE;
        const float *tR = tF + C::TILE;
        const float *xr_row = tF + 2 * C::TILE;
        const float *xr_col = xr_row + C::XV;
        const float *xF_col = xr_col + C::XV;
        // x of this thread's rows and columns; zero outside the window, half at tmin
        V xr[4], xc[4], xf[4];
        bool rv[4], cv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int a = I * T + 4 * warp + q;
          rv[q] = (a >= tmin) && (a <= t - 1);
          xr[q] = V::ld(xr_row + (4 * warp + q) * KC + j0);
          xr[q].scale(rv[q] ? (a == tmin ? 0.5f : 1.0f) : 0.0f);
          const int cc = c8 + 8 * q;
          const int b = J * T + cc;
          cv[q] = (b >= tmin) && (b <= t - 1);
          xc[q] = V::ld(xr_col + cc * KC + j0);
          xf[q] = V::ld(xF_col + cc * KC + j0);
          const float wb = cv[q] ? (b == tmin ? 0.5f : 1.0f) : 0.0f;
          xc[q].scale(wb);
          xf[q].scale(wb);
        }
        const bool interior = (I > J) && rv[0] && rv[1] && rv[2] && rv[3] && cv[0] && cv[1] && cv[2] && cv[3];
        const bool all_interior = __all_sync(0xffffffffu, interior);
        V rp[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) rp[q] = V::zero();
        if (all_interior) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int rr = 4 * warp + q;
            const float *fr = tF + rr * C::RS + j0;
            const float *qr = tR + rr * C::RS + j0;
            const int sw = rr & 3;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int e = ((c8 + 8 * k) ^ sw) * KC;
              const V f = V::ld(fr + e), g = V::ld(qr + e);
              colP[0][k].fma(xr[q], f);
              colP[1][k].fma(xr[q], g);
              rp[q].fma(xc[k], f);
              rp[q].fma(xf[k], g);
            }
          }
        } else {
          // edge tiles: rows/columns outside the window and, on the diagonal
          // tile, pairs above it (column sums take a >= b, row sums b < a)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int rr = 4 * warp + q;
            const float *fr = tF + rr * C::RS + j0;
            const float *qr = tR + rr * C::RS + j0;
            const int sw = rr & 3;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int cc = c8 + 8 * k;
              const int e = (cc ^ sw) * KC;
              V f = V::ld(fr + e), g = V::ld(qr + e);
              const bool in = rv[q] && cv[k];
              const bool vc = in && (I > J || rr >= cc);
              const bool vr = in && (I > J || rr > cc);
              const V zero = V::zero();
              const V fc = vc ? f : zero, gc = vc ? g : zero;
              const V fw = vr ? f : zero, gw = vr ? g : zero;
              colP[0][k].fma(xr[q], fc);
              colP[1][k].fma(xr[q], gc);
              rp[q].fma(xc[k], fw);
              rp[q].fma(xf[k], gw);
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + stage);
        // reduce-scatter the row sums over the 8 column lanes (lane bits 4, 3, 2)
        const bool b4 = (lane >> 4) & 1, b3 = (lane >> 3) & 1, b2 = (lane >> 2) & 1;
        float h[4];  // rows 2*b4 + {0,1}, orbits {0,1}
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const V mine = b4 ? rp[2 + i] : rp[i], theirs = b4 ? rp[i] : rp[2 + i];
          h[2 * i] = mine.v.x + __shfl_xor_sync(0xffffffffu, theirs.v.x, 16);
          h[2 * i + 1] = mine.v.y + __shfl_xor_sync(0xffffffffu, theirs.v.y, 16);
        }
        float g2[2];  // row 2*b4 + b3, orbits {0,1}
#pragma unroll
        for (int o = 0; o < 2; ++o) {
          const float mine = b3 ? h[2 + o] : h[o], theirs = b3 ? h[o] : h[2 + o];
          g2[o] = mine + __shfl_xor_sync(0xffffffffu, theirs, 8);
        }
        const float rsum = (b2 ? g2[1] : g2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? g2[0] : g2[1], 4);
        // this lane's (row, orbit) accumulator; the next tile's row is loaded one tile ahead
        {
          const int a = I * T + own_rr;
          const double prev = pre;
          const int an = (I < Jn ? (I + 1) : (J + 1)) * T + own_rr;
          if (an != a && an >= tmin && an <= t - 1) pre = rowacc[(size_t)(an % Ma) * KC + own_j];
          if (a >= tmin && a <= t - 1) {
            const double v = prev + (double)rsum;
            rowacc[(size_t)(a % Ma) * KC + own_j] = v;
            if (an == a) pre = v;
          }
        }
        if ((nin & 7) == 7)
#pragma unroll
          for (int f = 0; f < 2; ++f)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              colD[f][k][0] += (double)colP[f][k].v.x;
              colD[f][k][1] += (double)colP[f][k].v.y;
              colP[f][k] = V::zero();
            }
      }
      // all consumers: the row sums of column block J are complete
      consumer_sync(NT);
      if (*cabort) {
        aborted = true;
        break;
      }
      // column sums of the block: FP64 partials of the 8 warps meet in shared memory
      double accF = 0.0, accR = 0.0;
#pragma unroll
      for (int f = 0; f < 2; ++f) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          double *dst = colbuf + ((size_t)warp * 32 + (c8 + 8 * k)) * KC + j0;
          dst[0] = colD[f][k][0] + (double)colP[f][k].v.x;
          dst[1] = colD[f][k][1] + (double)colP[f][k].v.y;
        }
        consumer_sync(NT);
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) s += colbuf[((size_t)w * 32 + lf_loc) * KC + lf_j];
        if (f == 0) accF = s; else accR = s;
        consumer_sync(NT);
      }
      // leapfrog for t' = b (evolve_r!/evolve_F!, Evolution.jl:890-915)
      const int b = J * T + lf_loc;
      if (b >= tmin && b <= t - 1) {
        const int sb = b % Ma;
        const double wb = (b == tmin) ? 0.5 : 1.0;
        const float *sigr = reinterpret_cast<const float *>(R.sig_r) + (size_t)c * rowstride + (size_t)sb * KC;
        const float *sigF = reinterpret_cast<const float *>(R.sig_F) + (size_t)c * rowstride + (size_t)sb * KC;
        const size_t cs = (size_t)c * rowstride;
        const double *F1row = R.st_F + (size_t)((t - 1) % 3) * st_row + cs;
        const double *F2row = R.st_F + (size_t)((t - 2) % 3) * st_row + cs;
        const double *R1row = R.st_r + (size_t)((t - 1) % 3) * st_row + cs;
        const double *R2row = R.st_r + (size_t)((t - 2) % 3) * st_row + cs;
        double *FNrow = R.st_F + (size_t)(t % 3) * st_row + cs;
        double *RNrow = R.st_r + (size_t)(t % 3) * st_row + cs;
        const int j = lf_j;
        const int k = c * KC + j;
        const double kk = (k < R.S) ? R.k2[k] : 0.0;
        const double om = (kk + M2) * R.dt2;
        const double xbr_d = lo_only ? 0.0 : wb * (double)sigr[j];
        const double xbF_d = lo_only ? 0.0 : wb * (double)sigF[j];
        const double aF = accF + rowacc[(size_t)sb * KC + j];
        const double F1 = F1row[(size_t)sb * KC + j];
        const double F2 = (b <= t - 2) ? F2row[(size_t)sb * KC + j] : F1row[(size_t)((t - 2) % Ma) * KC + j];
        const double Fn = (2.0 - om) * F1 - F2 - aF * dt3;
        double rn;
        if (b == t - 1) {
          rn = R.dt;
        } else {
          const double r1 = R1row[(size_t)sb * KC + j];
          const double r2 = R2row[(size_t)sb * KC + j];
          rn = (2.0 - om) * r1 - r2 - accR * dt3;
        }
        FNrow[(size_t)sb * KC + j] = Fn;
        RNrow[(size_t)sb * KC + j] = rn;
        const size_t ho = hist_off(Ma, T, c, t, b, j);
        reinterpret_cast<float *>(R.hist_F)[ho] = (float)Fn;
        reinterpret_cast<float *>(R.hist_r)[ho] = (float)rn;
        diag += xbr_d * Fn + xbF_d * rn;
        if (b == t - 1) {
          emem = aF;
          has_emem = true;
        }
      }
    }
    if (!aborted) {
      // partial sums of acc_F(t) over this warp's columns, per orbit (lanes sharing lf_j)
      double v = diag;
      v += __shfl_xor_sync(0xffffffffu, v, 8);
      v += __shfl_xor_sync(0xffffffffu, v, 16);
      if (lane < KC) misc[16 + warp * KC + lane] = v;
      if (has_emem) misc[2 + lf_j] = emem;
    }
  }
  __syncthreads();
  if (*abort_flag) {
    if (tid == 0)  // the last NST issued tiles only, as in memint_kernel
      for (int q = max(0, *issued_count - NST); q < *issued_count; ++q)
        (void)mbar_wait_bounded(full + (q % NST), (uint32_t)((q / NST) & 1));
    __syncthreads();
    return;
  }
  if (tid < KC) memint_epilogue<float>(R, c, t, tid, misc, 8, M2, measure);
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
    double omg, cc, nn;
    meas_derived(Fmm, ddF, dt2, omg, cc, nn);
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

// Device measurement stream: after a step t with (t - 2) % every == 0, one
// block per run appends the createMeasurement record of that step -- the
// scalars (time, E, E_pot, E_kin, E_mem, M2, summed over chunks in order as
// kb_measure does on the host) and the per-orbit F, ddF, n, omega, c -- to a
// device buffer, so a captured multi-step graph needs no host round trip.
// ctl = {first measured t, every, capacity}; record m of run r starts at
// rec + m * block + off[r] and holds 6 + 5 S doubles.
__global__ void record_kernel(const RunDev *__restrict__ runs, const int *__restrict__ d_t,
                              const int *__restrict__ ctl, double *__restrict__ rec,
                              const long long *__restrict__ off, long long block) {
  const int t = *d_t;
  const int tf = ctl[0], every = ctl[1], cap = ctl[2];
  if (t < tf || (t - tf) % every != 0) return;
  const int m = (t - tf) / every;
  if (m >= cap) return;
  const RunDev &R = runs[blockIdx.x];
  double *out = rec + (long long)m * block + off[blockIdx.x];
  if (threadIdx.x == 0) {
    double ek = 0, ep = 0, em = 0;
    for (int c = 0; c < R.nchunks; ++c) {
      ek += R.epart[(size_t)c * 4 + 0];
      ep += R.epart[(size_t)c * 4 + 1];
      em += R.epart[(size_t)c * 4 + 2];
    }
    if (t == 2) em = 0.0;
    out[0] = (t - 1) * R.dt * R.mass;
    out[1] = ek + ep + em;
    out[2] = ep;
    out[3] = ek;
    out[4] = em;
    out[5] = R.epart[3];
  }
  const int Sp = R.nchunks * KC;
  for (int k = threadIdx.x; k < R.S; k += blockDim.x) {
    const double Fmm = R.meas[k], ddF = R.meas[(size_t)Sp + k];
    double omg, cc, nn;
    meas_derived(Fmm, ddF, R.dt2, omg, cc, nn);
    out[6 + k] = Fmm;
    out[6 + R.S + k] = ddF;
    out[6 + 2 * R.S + k] = nn;
    out[6 + 3 * R.S + k] = omg;
    out[6 + 4 * R.S + k] = cc;
  }
}

// n, omega and c of run `run`'s measured step (meas blocks 2, 3, 4) from its F(t-1,t-1)
// and ddF (blocks 0, 1)
__global__ void meas_derive_kernel(const RunDev *__restrict__ runs, int run) {
  const RunDev &R = runs[run];
  const int Sp = R.nchunks * KC;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R.S; k += gridDim.x * blockDim.x) {
    double omg, cc, nn;
    meas_derived(R.meas[k], R.meas[(size_t)Sp + k], R.dt2, omg, cc, nn);
    R.meas[(size_t)2 * Sp + k] = nn;
    R.meas[(size_t)3 * Sp + k] = omg;
    R.meas[(size_t)4 * Sp + k] = cc;
  }
}

__global__ void set_t_kernel(int *d_t, int t) { *d_t = t; }
__global__ void advance_t_kernel(int *d_t) { *d_t += 1; }

using CfgF64 = Cfg<double, 16, 4, 1>;
using CfgF32 = Cfg<float, 32, 3, 2>;

}  // namespace

int memint_tile(bool fp64) { return fp64 ? CfgF64::T : CfgF32::T; }

// FP32 variants: 1 = two consumer groups (memint_kernel, the default), 0 =
// register-blocked consumers (memint_blk_kernel: half the shared-memory
// wavefronts but more instructions per tile; slower on GB300 at Ns = 16..64,
// where both are latency-bound at about a third of the issue rate). Both stream
// the same tiles in the same order.
size_t memint_smem_bytes(bool fp64, int Malloc, int variant) {
  (void)Malloc;
  if (fp64) return smem_fixed_bytes<CfgF64>();
  return variant == 1                    ? smem_fixed_bytes<CfgF32>()
         : (variant == 2 || variant == 3) ? smem_fixed_bytes<CfgF32>() + LF_STAGE_BYTES
                                          : smem_fixed_bytes<CfgF32>() + BLK_COLBUF_BYTES;
}

cudaError_t configure_memint(bool fp64, size_t smem) {
  if (fp64) {
    cudaError_t e = cudaFuncSetAttribute(memint_kernel<double, CfgF64::T, CfgF64::NST, CfgF64::OPT, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(memint_kernel<double, CfgF64::T, CfgF64::NST, CfgF64::OPT, true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  cudaError_t e = cudaFuncSetAttribute(memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, false, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, true, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, false, true, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, true, true, true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(memint_blk_kernel<CfgF32::NST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem);
}

// parts of a split chunk: two, or for the chunks past the whole waves of a large
// grid (nwhole > 0) the k in [2, MEMINT_MAX_PARTS] whose nsplit k pieces fill the
// sm_slots CTA slots in the fewest piece lengths, ceil(nsplit k / sm_slots) / k
// (the smaller k on a tie): 59 chunks on 152 SMs take 5 parts, 0.4 of a chunk's
// stream for the last wave instead of 0.5
int memint_split_parts(int nwhole, int nsplit, int sm_slots) {
  if (nwhole <= 0 || nsplit <= 0 || sm_slots <= 0) return 2;
  int best = 2;
  double best_len = 1e30;
  for (int k = 2; k <= MEMINT_MAX_PARTS; ++k) {
    const double len = (double)((nsplit * k + sm_slots - 1) / sm_slots) / k;
    if (len < best_len - 1e-12) {
      best_len = len;
      best = k;
    }
  }
  return best;
}

// use_maps: bit 0 tensor-map boxes (else bulk copies), bit 1 the test hook that
// issues no tiles (memint_kernel only). queue: null, or a device counter that makes
// memint_kernel persistent on at most grid_cap CTAs (zeroed here before the launch).
cudaError_t launch_memint(bool fp64, int variant, int split, int nwhole, const RunDev *d_runs, const int *d_base,
                          int nruns, int total_ctas, int fin_nb_max, int use_maps, const int *d_t, int *d_err,
                          int measure, size_t smem, int *queue, int grid_cap, cudaStream_t st) {
  // split: the chunks from nwhole on are streamed in parts (memint_split_parts) and
  // completed by the finishing kernel
  const int nsplit = total_ctas - nwhole;
  const bool splitting = split && nsplit > 0;
  const int parts = splitting ? memint_split_parts(nwhole, nsplit, grid_cap) : 1;
  const int nitems = splitting ? nwhole + parts * nsplit : total_ctas;
  const bool persistent = queue != nullptr && grid_cap > 0 && (fp64 || variant != 0);
  const int grid = persistent ? std::min(nitems, grid_cap) : nitems;
  int *q = persistent ? queue : nullptr;
  if (persistent) {
    const cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
  }
  const int nw = splitting ? nwhole : total_ctas;
  constexpr int NTHR_LF = CfgF32::NT + 32 + CfgF32::NG;  // consumers, producer, leapfrog warps
  if (!fp64 && (variant == 2 || variant == 3)) {  // leapfrog warps for the whole chunks; 3: compensated sums
    if (splitting) {
      if (variant == 3)
        memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, true, true, true>
            <<<grid, NTHR_LF, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure, nw, use_maps, nitems, q, parts);
      else
        memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, true, true>
            <<<grid, NTHR_LF, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure, nw, use_maps, nitems, q, parts);
      memint_finish_kernel<float><<<nsplit * fin_nb_max, FIN_THREADS, 0, st>>>(d_runs, d_base, nruns, fin_nb_max,
                                                                               nwhole, d_t, measure, parts);
    } else if (variant == 3) {
      memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, false, true, true>
          <<<grid, NTHR_LF, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure, nw, use_maps, nitems, q, parts);
    } else {
      memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, false, true>
          <<<grid, NTHR_LF, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure, nw, use_maps, nitems, q, parts);
    }
    return cudaGetLastError();
  }
  if (splitting && (fp64 || variant == 1)) {
    if (fp64) {
      memint_kernel<double, CfgF64::T, CfgF64::NST, CfgF64::OPT, true>
          <<<grid, CfgF64::NT + 32, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure, nw, use_maps, nitems, q, parts);
      memint_finish_kernel<double><<<nsplit * fin_nb_max, FIN_THREADS, 0, st>>>(d_runs, d_base, nruns, fin_nb_max,
                                                                                nwhole, d_t, measure, parts);
    } else {
      memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, true>
          <<<grid, CfgF32::NT + 32, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure, nw, use_maps, nitems, q, parts);
      memint_finish_kernel<float><<<nsplit * fin_nb_max, FIN_THREADS, 0, st>>>(d_runs, d_base, nruns, fin_nb_max,
                                                                               nwhole, d_t, measure, parts);
    }
    return cudaGetLastError();
  }
  if (fp64)
    memint_kernel<double, CfgF64::T, CfgF64::NST, CfgF64::OPT, false>
        <<<grid, CfgF64::NT + 32, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure, nw, use_maps, nitems, q, parts);
  else if (variant == 1)
    memint_kernel<float, CfgF32::T, CfgF32::NST, CfgF32::OPT, false>
        <<<grid, CfgF32::NT + 32, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure, nw, use_maps, nitems, q, parts);
  else
    memint_blk_kernel<CfgF32::NST><<<total_ctas, 288, smem, st>>>(d_runs, d_base, nruns, d_t, d_err, measure);
  return cudaGetLastError();
}

cudaError_t launch_meas_derive(const RunDev *d_runs, int run, int S, cudaStream_t st) {
  meas_derive_kernel<<<(S + 255) / 256, 256, 0, st>>>(d_runs, run);
  return cudaGetLastError();
}

cudaError_t launch_measure_init(const RunDev *d_runs, int nruns, int t, cudaStream_t st) {
  measure_init_kernel<<<nruns, 256, 0, st>>>(d_runs, nruns, t);
  return cudaGetLastError();
}
cudaError_t launch_record(const RunDev *d_runs, int nruns, const int *d_t, const int *d_ctl, double *rec,
                          const long long *d_off, long long block, cudaStream_t st) {
  record_kernel<<<nruns, 256, 0, st>>>(d_runs, d_t, d_ctl, rec, d_off, block);
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
