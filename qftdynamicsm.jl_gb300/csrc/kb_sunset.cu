// kb_sunset.cu -- the 3-loop sunset self-energy of one KB step.
//
// Replaces calcSelfEnergies!/calcSelfEnergyattp! (src/TwoPIScalar/
// TwoPIScalar_Evolution.jl:16-31 quantum, :107-121 classical): for every t'
// of the window
//   Fx = Re rfft F(t-1,t'),  rx = Re rfft rho(t-1,t')
//   Sigma_rho(t') = ivol^3 (-lambda^2 (N+2)/(6 N^2))  brfft[rx (Fx^2 - rx^2/12)]
//   Sigma_F(t')   = ivol^3 (-lambda^2 (N+2)/(18 N^2)) brfft[Fx (Fx^2 - 3/4 rx^2)]
//
// F and rho are cubic-symmetric, so the 3D transforms reduce to cosine
// transforms on the even octant [0,H)^3 (H = Ns/2 + 1) with the matrix
// C[X][x] = m(x) cos(2 pi x X / Ns) (m = 1 at 0 and Ns/2, else 2) along each
// axis. Data stay on cubic orbits (S = C(H+2,3) values); the three axis
// passes keep the symmetry that survives them:
//   expand  E[x][p]   = f(x, y_p, z_p)                      p = (y <= z) pair
//   pass 1  B[X][p]   = sum_x C[X][x] E[x][p]                (symmetric in y,z)
//   pass 2  D[z][q]   = sum_y C[Y][y] B[X][(y,z)]            q = (X <= Y) pair
//   pass 3  P(X,Y,Z)  = sum_z C[Z][z] D[z][(X,Y)]            X <= Y <= Z: an orbit
// Each pass is a small dense GEMM; every thread computes a 4 x 4 register
// tile. Passes 1 and 3 are folded by the parity of the cosine matrix,
// C[X][h-x] = (-1)^X C[X][x] (h = Ns/2), so they contract over about half of
// x (z); pass 2 contracts over y, one index of the symmetric pair storage,
// and is not. At Ns = 64 a transform costs about 1.4 M multiply-adds (four per
// t') instead of the four 262144-point FFTs of the reference.
//
// Intermediates E/D and B live in two regions R1, R2 of about H*P values: in
// shared memory for FP32, in a per-CTA global scratch slot for FP64 (whose
// regions do not fit next to each other in 227 KB). The grid is persistent: its
// CTAs take the items (t' rows) of all runs of the batch from a device counter,
// so the same launch serves every step of a CUDA graph (rows outside the window
// are skipped).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/kb2pi.h"
#include "kb_internal.cuh"

namespace kb {
namespace {

constexpr int SUN_THREADS = 512;
constexpr int SUN_THREADS_F32 = 1024;

__host__ __device__ constexpr int rup4(int v) { return (v + 3) & ~3; }
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int sun_tri(int b) { return b * (b + 1) / 2; }
__host__ __device__ constexpr int sun_tet(int c) { return c * (c + 1) * (c + 2) / 6; }

// the two intermediate regions: R1 holds E then D (both [H][P4]), R2 holds B
// ([H][P4], pass 2 reads up to 3 entries past its last row); both also take rows
// of orbit values (S)
__host__ __device__ constexpr int sun_r1(int H) { return rup4(cmax(H * rup4(sun_tri(H)), sun_tet(H))); }
__host__ __device__ constexpr int sun_r2(int H) { return rup4(cmax(H * rup4(sun_tri(H)) + 4, sun_tet(H))); }

struct SunGeom {
  int H, H4, P, P4, S;
  int r1, r2;  // region sizes in elements
  // pass 1 folded by C[X][h-x] = (-1)^X C[X][x] (h = Ns/2 = H-1): npair pairs
  // x < h-x, a middle x = h/2 when h is even; ne even and no odd outputs X
  int npair, mid, ne, no, ne4, no4, cf;  // cf: elements of the two folded matrices
  int n2, n3;                            // work items of passes 2 and 3
  __host__ __device__ SunGeom(int H_) {
    H = H_;
    H4 = rup4(H);
    P = sun_tri(H);
    P4 = rup4(P);
    S = sun_tet(H);
    npair = H / 2;  // (h + 1) / 2
    mid = (H - 1) % 2 == 0;
    ne = npair + mid;
    no = H - ne;
    ne4 = rup4(ne);
    no4 = rup4(no);
    cf = rup4(ne * ne4 + no * no4);
    r1 = sun_r1(H);
    r2 = sun_r2(H);
    // pass 2: (H4/4 - X/4) Y blocks by H4/4 z blocks for every X
    const int nzb = H4 / 4, a = H >> 2, b = H & 3;
    n2 = nzb * (nzb * H - (2 * a * (a - 1) + a * b));
    // pass 3: items3(Y) for each block of four pairs whose first pair has row Y
    n3 = 0;
    for (int Y = 0; Y < H; ++Y) n3 += (((sun_tri(Y + 1) + 3) >> 2) - ((sun_tri(Y) + 3) >> 2)) * items3(Y);
  }
  // pass 3 items of a block of four pairs whose smallest Y is Ymin: blocks of four
  // even outputs Z = 2j >= Ymin, then blocks of four odd outputs Z = 2j+1 >= Ymin
  __host__ __device__ int items3(int Ymin) const { return (ne4 / 4 - ((Ymin + 1) / 2) / 4) + (no4 / 4 - (Ymin / 2) / 4); }
};

// shared memory of the tables of sun_transform without the expand table: cosine and
// folded matrices (compute type), the pair list, the work items of passes 2 and 3
__host__ __device__ inline size_t sun_tables_bytes(bool fp64, const SunGeom &g) {
  const size_t es = fp64 ? 8 : 4;
  const size_t b = ((size_t)g.H4 * g.H4 + g.cf) * es + (size_t)(g.P4 + g.n2 + g.n3) * sizeof(uint16_t);
  return (b + 15) & ~(size_t)15;
}

// shared memory of sunset_kernel: the tables, the expand table ([H][P4] orbit
// indices) when everything fits in the 227 KB a CTA may use, one orbit buffer and,
// FP32, the two pass regions (FP64 keeps them in a per-CTA global scratch slot)
constexpr size_t SUN_SMEM_HEAD = 16;  // sunset_kernel's item counter ahead of the layout
constexpr size_t SUN_SMEM_CAP = 232448 - SUN_SMEM_HEAD;
struct SunLayout {
  size_t etab, regions, bytes;
  bool has_etab;
};
__host__ __device__ inline SunLayout sun_layout(bool fp64, const SunGeom &g) {
  const size_t es = fp64 ? 8 : 4;
  SunLayout L;
  const size_t t0 = sun_tables_bytes(fp64, g);
  const size_t et = ((size_t)g.H * g.P4 * sizeof(uint16_t) + 15) & ~(size_t)15;
  const size_t rest = ((size_t)rup4(g.S) + (fp64 ? 0 : (size_t)g.r1 + g.r2)) * es;
  L.has_etab = t0 + et + rest <= SUN_SMEM_CAP;
  L.etab = t0;
  L.regions = t0 + (L.has_etab ? et : 0);
  L.bytes = L.regions + rest;
  return L;
}

__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
// 16-byte asynchronous copy global -> shared (L2 only), its group commit and the wait for
// all of this thread's groups
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// 4-wide vector load/store for float (float4) and double (2 x double2)
__device__ __forceinline__ void ld4(const float *p, float v[4]) {
  const float4 q = *reinterpret_cast<const float4 *>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void ld4(const double *p, double v[4]) {
  const double2 a = *reinterpret_cast<const double2 *>(p);
  const double2 b = *reinterpret_cast<const double2 *>(p + 2);
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void st4(float *p, const float v[4]) {
  *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double *p, const double v[4]) {
  *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
  *reinterpret_cast<double2 *>(p + 2) = make_double2(v[2], v[3]);
}

// orbit index of the sorted triple a <= b <= c
__device__ __forceinline__ int orb3s(int a, int b, int c) { return sun_tet(c) + sun_tri(b) + a; }

// orbit index of (x, y, z) given y <= z
__device__ __forceinline__ int orb_of(int x, int y, int z) {
  const int lo = min(x, y);
  const int mid = (x <= y) ? y : min(x, z);
  const int hi = max(x, z);
  return orb3s(lo, mid, hi);
}

template <typename TC>
struct SunCtx {
  const TC *CT;         // [H4][H4]: CT[x][X] = C[X][x], zero where x or X >= H; followed by CF:
                        // [ne][ne4] C[2j][k] (even X = 2j), then [no][no4] C[2j+1][k] (odd X)
  const uint16_t *pr;   // [P4]: pair p = tri(z) + y -> (y | z << 8)
  const uint16_t *it2;  // [n2]: pass 2 items (X | z block << 6 | Y block << 10)
  const uint16_t *it3;  // [n3]: pass 3 items (pair block | output block << 8)
  const uint16_t *etab; // [H][P4]: orbit of E[x][p] (0 in the padding), or null
  TC *R1, *R2, *bufF;
  SunGeom g;
};

// expand: E[x][p] = in(orbit of (x, y_p, z_p)) for x < H, p < P
template <typename TC, typename In>
__device__ void sun_expand(const SunCtx<TC> &c, TC *E, In in) {
  if (c.etab) {
    const int n = c.g.H * c.g.P4;
    for (int i = threadIdx.x; i < n; i += blockDim.x) E[i] = in(c.etab[i]);
    return;
  }
  const int n = c.g.H * c.g.P;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int x = i / c.g.P, p = i - x * c.g.P;
    const int y = c.pr[p] & 255, z = c.pr[p] >> 8;
    E[x * c.g.P4 + p] = in(orb_of(x, y, z));
  }
}

// folded cosine matrices of pass 1 at CF = CT + H4^2, from cm(X, x) = C[X][x]
template <typename TC, typename Cm>
__device__ void sun_build_cf(const SunGeom &g, TC *CF, Cm cm) {
  for (int i = threadIdx.x; i < g.ne * g.ne4; i += blockDim.x) {
    const int k = i / g.ne4, j = i - k * g.ne4;
    CF[i] = (j < g.ne) ? (TC)cm(2 * j, k) : (TC)0;
  }
  TC *CFo = CF + g.ne * g.ne4;
  for (int i = threadIdx.x; i < g.no * g.no4; i += blockDim.x) {
    const int k = i / g.no4, j = i - k * g.no4;
    CFo[i] = (j < g.no) ? (TC)cm(2 * j + 1, k) : (TC)0;
  }
}

// the tables of sun_transform for octant size g.H in shared memory at `base`
// (sun_tables_bytes), the expand table at `etab` unless null, the cosine matrix
// from cm(X, x) = C[X][x]; ends with a barrier. The regions and the orbit buffer of
// the returned context are left to the caller.
// the context of tables already at `base` (built there, or copied in from an image)
template <typename TC>
__device__ SunCtx<TC> sun_tables_ctx(const SunGeom &g, unsigned char *base, uint16_t *etab) {
  const TC *CT = reinterpret_cast<const TC *>(base);
  const uint16_t *pr = reinterpret_cast<const uint16_t *>(CT + g.H4 * g.H4 + g.cf);
  const uint16_t *it2 = pr + g.P4;
  return SunCtx<TC>{CT, pr, it2, it2 + g.n2, etab, nullptr, nullptr, nullptr, g};
}

template <typename TC, typename Cm>
__device__ SunCtx<TC> sun_build_tables(const SunGeom &g, unsigned char *base, uint16_t *etab, Cm cm) {
  TC *CT = reinterpret_cast<TC *>(base);
  uint16_t *pr = reinterpret_cast<uint16_t *>(CT + g.H4 * g.H4 + g.cf);
  uint16_t *it2 = pr + g.P4;
  uint16_t *it3 = it2 + g.n2;
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (int i = tid; i < g.H4 * g.H4; i += nthr) {
    const int x = i / g.H4, X = i - x * g.H4;
    CT[i] = (X < g.H && x < g.H) ? (TC)cm(X, x) : (TC)0;
  }
  sun_build_cf(g, CT + g.H4 * g.H4, cm);
  for (int z = tid; z < g.H; z += nthr)
    for (int y = 0; y <= z; ++y) pr[sun_tri(z) + y] = (uint16_t)(y | (z << 8));
  // pass 2: the items of X are its (z block, Y block) pairs, Y blocks from X/4 on,
  // neighbouring items in the same z block; they start after sum_{X'<X} (nzb - X'/4) nzb
  const int nzb = g.H4 / 4;
  for (int X = tid; X < g.H; X += nthr) {
    const int a = X >> 2, b = X & 3, nyb = nzb - a;
    const int off = nzb * (nzb * X - (2 * a * (a - 1) + a * b));
    for (int zb = 0; zb < nzb; ++zb)
      for (int yb = 0; yb < nyb; ++yb) it2[off + zb * nyb + yb] = (uint16_t)(X | (zb << 6) | (yb << 10));
  }
  // pass 3: the items3(Y) items of every block of four pairs whose first pair has
  // row Y; offsets by a scan over Y in warp 0 (lane = Y, 32 rows per round)
  if (tid < 32) {
    int off = 0;
    for (int Y0 = 0; Y0 < g.H; Y0 += 32) {
      const int Y = Y0 + tid;
      const int qa = (sun_tri(Y) + 3) >> 2, qe = (sun_tri(Y + 1) + 3) >> 2;
      const int n = Y < g.H ? g.items3(Y) : 0, cnt = Y < g.H ? (qe - qa) * n : 0;
      int inc = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (tid >= o) inc += v;
      }
      int w = off + inc - cnt;
      for (int qb = qa; qb < qe && Y < g.H; ++qb)
        for (int r = 0; r < n; ++r) it3[w++] = (uint16_t)(qb | (r << 8));
      off += __shfl_sync(0xffffffffu, inc, 31);
    }
  }
  if (etab) {
    __syncthreads();  // pr
    for (int i = tid; i < g.H * g.P4; i += nthr) {
      const int x = i / g.P4, p = i - x * g.P4;
      etab[i] = (p < g.P) ? (uint16_t)orb_of(x, pr[p] & 255, pr[p] >> 8) : (uint16_t)0;
    }
  }
  __syncthreads();
  return sun_tables_ctx<TC>(g, base, etab);
}

// copy of a table image (built by sun_image_kernel) into shared memory; ends with a barrier
__device__ __forceinline__ void sun_copy_image(const unsigned char *img, unsigned char *base, size_t bytes) {
  const uint4 *src = reinterpret_cast<const uint4 *>(img);
  uint4 *dst = reinterpret_cast<uint4 *>(base);
  for (size_t i = threadIdx.x; i < bytes / 16; i += blockDim.x) dst[i] = __ldg(src + i);
  __syncthreads();
}

// unroll of the pass loops (FP64 at 2: the 4 x 4 double tile fills the registers)
template <typename TC>
struct SunUnroll {
  static constexpr int value = sizeof(TC) == 4 ? 4 : 2;
};

template <typename TC>
__device__ __forceinline__ void fma4x4(TC acc[4][4], const TC a[4], const TC b[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
}

// pass 1: B[X][p] = sum_x C[X][x] E[x][p], folded: with C[X][h-x] = (-1)^X C[X][x]
// (h = H - 1), B[2j] = sum_{k<npair} C[2j][k] (E[k] + E[h-k]) (+ C[2j][h/2] E[h/2])
// and B[2j+1] = sum_{k<npair} C[2j+1][k] (E[k] - E[h-k]): half the multiply-adds
template <typename TC>
__device__ void sun_pass1(const SunCtx<TC> &c, const TC *E, TC *B) {
  const int P4 = c.g.P4, h = c.g.H - 1, npair = c.g.npair;
  const int npb = P4 / 4, nbe = c.g.ne4 / 4, nbo = c.g.no4 / 4;
  const TC *CF = c.CT + c.g.H4 * c.g.H4;
  for (int it = threadIdx.x; it < (nbe + nbo) * npb; it += blockDim.x) {
    const int jq = it / npb, pb = it - jq * npb;
    const int odd = jq >= nbe ? 1 : 0;
    const int j0 = 4 * (odd ? jq - nbe : jq), p0 = 4 * pb;
    const int stride = odd ? c.g.no4 : c.g.ne4;
    const TC *cf = CF + (odd ? c.g.ne * c.g.ne4 : 0) + j0;
    const TC sg = odd ? (TC)-1 : (TC)1;
    TC acc[4][4] = {};
#pragma unroll 2
    for (int k = 0; k < npair; ++k) {
      TC cv[4], ea[4], eb[4], ev[4];
      ld4(cf + k * stride, cv);
      ld4(E + k * P4 + p0, ea);
      ld4(E + (h - k) * P4 + p0, eb);
#pragma unroll
      for (int q = 0; q < 4; ++q) ev[q] = ea[q] + sg * eb[q];
      fma4x4(acc, cv, ev);
    }
    if (!odd && c.g.mid) {  // x = h/2: coefficient row npair of the even matrix
      TC cv[4], ev[4];
      ld4(cf + npair * stride, cv);
      ld4(E + (h / 2) * P4 + p0, ev);
      fma4x4(acc, cv, ev);
    }
    const int nrow = odd ? c.g.no : c.g.ne;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (j0 + i < nrow) st4(B + (2 * (j0 + i) + odd) * P4 + p0, acc[i]);
  }
}

// pass 2: D[z][tri(Y)+X] = sum_y CT[y][Y] B[X][(min(y,z), max(y,z))], Y >= X.
// B[X] holds the pairs (y <= z) at tri(z) + y. Every thread walks y in blocks
// of four and reads the 4 x 4 block of the symmetric B[X] at (y0.., z0..) as
// four rows of four packed entries: rows y0 + k at columns z0.. when y0 >= z0,
// rows z0 + k at columns y0.. (the transposed block) when y0 < z0; the block
// is then picked entry by entry, so all lanes run the same instructions
// whatever their z block. Rows past H - 1 are read as row H - 1 (their cosine
// rows are zero); the entries picked from outside the triangle only reach
// accumulators of z >= H, which are not stored.
template <typename TC>
__device__ void sun_pass2(const SunCtx<TC> &c, const TC *B, TC *D) {
  const int H = c.g.H, H4 = c.g.H4, P4 = c.g.P4;
  for (int it = threadIdx.x; it < c.g.n2; it += blockDim.x) {
    const int code = c.it2[it];  // neighbouring items share the z block
    const int X = code & 63, zb = (code >> 6) & 15, yb = code >> 10;
    const int Y0 = 4 * (X / 4) + 4 * yb, z0 = 4 * zb;
    const TC *Bx = B + X * P4;
    TC acc[4][4] = {};
    for (int y0 = 0; y0 < H4; y0 += 4) {
      TC cv[4][4];  // cv[i][a] = C[Y0 + a][y0 + i]
#pragma unroll
      for (int i = 0; i < 4; ++i) ld4(c.CT + (y0 + i) * H4 + Y0, cv[i]);
      const bool ge = y0 >= z0, gt = y0 > z0;
      const int rb = ge ? y0 : z0, cb = ge ? z0 : y0;
      TC L[4][4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const TC *row = Bx + sun_tri(min(rb + k, H - 1)) + cb;
#pragma unroll
        for (int m = 0; m < 4; ++m) L[k][m] = row[m];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (y0 + i >= H) break;  // the padded rows of the last block (same for all lanes)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // B(y0 + i, z0 + j): L[i][j] in the direct layout, L[j][i] in the transposed one
          const TC v = (i == j) ? L[i][i] : ((j < i ? ge : gt) ? L[i][j] : L[j][i]);
#pragma unroll
          for (int a = 0; a < 4; ++a) acc[a][j] += cv[i][a] * v;
        }
      }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int Y = Y0 + a;
      if (Y < X || Y >= H) continue;
      const int q = sun_tri(Y) + X;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (z0 + j < H) D[(z0 + j) * P4 + q] = acc[a][j];
    }
  }
}

// pass 3: out(orbit(X,Y,Z), sum_z C[Z][z] D[z][q]) for q = (X,Y), Z >= Y, folded
// as pass 1: even Z = 2j from D[k] + D[h-k] (and the middle row), odd Z = 2j+1
// from D[k] - D[h-k]; an item is four pairs by four outputs of one parity
template <typename TC, typename Out>
__device__ void sun_pass3(const SunCtx<TC> &c, const TC *D, Out out) {
  const int H = c.g.H, P = c.g.P, P4 = c.g.P4, h = H - 1, npair = c.g.npair;
  const TC *CF = c.CT + c.g.H4 * c.g.H4;
  for (int it = threadIdx.x; it < c.g.n3; it += blockDim.x) {
    const int code = c.it3[it];
    const int qb = code & 255, r = code >> 8;
    const int q0 = 4 * qb;
    const int Ymin = c.pr[min(q0, P - 1)] >> 8;
    const int jbe = ((Ymin + 1) / 2) / 4, ne_items = c.g.ne4 / 4 - jbe;
    const int odd = r >= ne_items ? 1 : 0;
    const int j0 = odd ? 4 * ((Ymin / 2) / 4 + (r - ne_items)) : 4 * (jbe + r);
    const int stride = odd ? c.g.no4 : c.g.ne4;
    const TC *cf = CF + (odd ? c.g.ne * c.g.ne4 : 0) + j0;
    const TC sg = odd ? (TC)-1 : (TC)1;
    TC acc[4][4] = {};
#pragma unroll 2
    for (int k = 0; k < npair; ++k) {
      TC cv[4], da[4], db[4], dv[4];
      ld4(cf + k * stride, cv);
      ld4(D + k * P4 + q0, da);
      ld4(D + (h - k) * P4 + q0, db);
#pragma unroll
      for (int i = 0; i < 4; ++i) dv[i] = da[i] + sg * db[i];
      fma4x4(acc, dv, cv);
    }
    if (!odd && c.g.mid) {  // z = h/2: coefficient row npair of the even matrix
      TC cv[4], dv[4];
      ld4(cf + npair * stride, cv);
      ld4(D + (h / 2) * P4 + q0, dv);
      fma4x4(acc, dv, cv);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int q = q0 + i;
      if (q >= P) continue;
      const int X = c.pr[q] & 255, Y = c.pr[q] >> 8;
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        const int Z = 2 * (j0 + jj) + odd;
        if (Z >= Y && Z < H) out(orb3s(X, Y, Z), acc[i][jj]);
      }
    }
  }
}

// after_expand() runs once the input has been read (every thread, behind a barrier),
// after_pass2() once R2 is free again (pass 3 reads R1 only)
template <typename TC, typename In, typename Out, typename A, typename B>
__device__ void sun_transform_hooked(const SunCtx<TC> &c, In in, Out out, A after_expand, B after_pass2) {
  sun_expand<TC>(c, c.R1, in);
  __syncthreads();
  after_expand();
  sun_pass1<TC>(c, c.R1, c.R2);
  __syncthreads();
  sun_pass2<TC>(c, c.R2, c.R1);
  __syncthreads();
  after_pass2();
  sun_pass3<TC>(c, c.R1, out);
  __syncthreads();
}

template <typename TC, typename In, typename Out>
__device__ void sun_transform(const SunCtx<TC> &c, In in, Out out) {
  sun_transform_hooked<TC>(c, in, out, [] {}, [] {});
}

// NTHR threads per CTA; MINB resident CTAs per SM the register budget allows.
// An item of a run is R.sun_rows consecutive t' rows (several for the small
// lattices of a batch, so that their per-item work -- finding the run, the L2

// NTHR threads per CTA; MINB resident CTAs per SM the register budget allows.
// An item of a run is R.sun_rows consecutive t' rows (several for the small
// lattices of a batch, so that their per-item work -- finding the run, the L2
// prefetch of the next row -- is spread over more rows), taken one after the other.
// Items: with a queue (a counter zeroed before the launch) every CTA takes the next
// item when it is done with one -- the items of a batch differ in cost, and runs are
// ordered costliest first -- and takes it early, so that its rows can go to L2 while
// the current item's inverse transforms run; without one CTA b takes b, b + grid, ...
template <typename TC, typename TS, bool SCRATCH, int NTHR, int MINB>
__global__ void __launch_bounds__(NTHR, MINB)
sunset_kernel(const RunDev *__restrict__ runs, const int *__restrict__ base, int nruns, int total,
              const int *__restrict__ d_t, TC *__restrict__ scratch, size_t scratch_stride, int *__restrict__ queue) {
  extern __shared__ __align__(16) unsigned char smem_dyn[];
  // the item counter's value in the first 16 bytes, the layout of sun_layout after them
  // (no static shared memory: the kernel may take the device's whole per-block maximum)
  volatile int &q_slot = *reinterpret_cast<int *>(smem_dyn);
  unsigned char *smem_raw = smem_dyn + SUN_SMEM_HEAD;
  const int t = *d_t;  // Sigma(t-1, t') for t' in [tmin, t-1]
  int cur_ns = -1;
  SunCtx<TC> c{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, SunGeom(1)};
  // the next item from the queue; every thread calls it (two barriers)
  auto take = [&]() {
    __syncthreads();  // the previous item number has been read by every thread
    if (threadIdx.x == 0) q_slot = atomicAdd(queue, 1);
    __syncthreads();
    return q_slot;
  };
  int nxt = -1;  // the next item if taken early (queue)
  // FP32 rows are staged with asynchronous copies: rho into R2 while F's pass 3 runs (R2
  // is free from then on), the next row's F into the orbit buffer while the current
  // row's inverse F transform runs (free once its expand has read it)
  constexpr bool ASYNC = !SCRATCH && sizeof(TS) == 4 && sizeof(TC) == 4;
  int pre_w = -1, pre_g = -1;  // the row whose F is on its way into the orbit buffer
  for (int w = queue ? take() : (int)blockIdx.x; w < total;
       w = queue ? (nxt >= 0 ? nxt : take()) : w + (int)gridDim.x) {
    nxt = -1;
    if (ASYNC) cp_async_wait_all();  // nothing of this thread's lands in shared memory later
    const int r = run_at(base, nruns, w);
    const RunDev &R = runs[r];
    if (!pexp_sunset(R.pexp) || t < 3) continue;
    if (R.Ns != cur_ns) {
      // tables of the lattice size (runs of the same Ns share them), then the
      // orbit buffer and the pass regions
      __syncthreads();
      cur_ns = R.Ns;
      const SunGeom g(R.H);
      const SunLayout L = sun_layout(sizeof(TC) == 8, g);
      uint16_t *etab = L.has_etab ? reinterpret_cast<uint16_t *>(smem_raw + L.etab) : nullptr;
      if (R.sun_img) {  // the handle's image of these tables
        sun_copy_image(R.sun_img, smem_raw, L.regions);
        c = sun_tables_ctx<TC>(g, smem_raw, etab);
      } else {
        c = sun_build_tables<TC>(g, smem_raw, etab, [&](int X, int x) { return R.Cm[X * g.H + x]; });
      }
      c.bufF = reinterpret_cast<TC *>(smem_raw + L.regions);
      if (SCRATCH) {
        c.R1 = scratch + (size_t)blockIdx.x * scratch_stride;
        c.R2 = c.R1 + g.r1;
      } else {
        c.R1 = c.bufF + rup4(g.S);
        c.R2 = c.R1 + g.r1;
      }
    }
    const int tmin = max(1, t - R.M + 1);
    const int S = c.g.S;
    const size_t rowstride = (size_t)R.Malloc * KC;
    auto gidx = [&](int o) { return (size_t)(o / KC) * rowstride + (o % KC); };
    const size_t cstride = (size_t)R.Malloc * R.Malloc * KC;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int nrow = SCRATCH ? 1 : R.sun_rows;
    for (int gi = 0; gi < nrow; ++gi) {
      const bool prestaged = ASYNC && pre_w == w && pre_g == gi;
      if (ASYNC) cp_async_wait_all();
      pre_w = pre_g = -1;
      const int tp = tmin + (w - R.cta_base_sun) * nrow + gi;
      if (tp > t - 1) break;  // rows of an item are consecutive: the rest are past the window too
      const int slot = tp % R.Malloc;
      // (uniform over the CTA: the skip passes no barrier another thread waits at)
      if (!KB_DCHECK(tp >= tmin && t - 1 - tp < R.M && slot >= 0 && S <= R.nchunks * KC, R.err, DCHK_SUN_ROW))
        continue;
      // row (t-1, t') of a history ring (the storage-type copy of the state row;
      // chunks are Malloc^2 KC apart) into shared memory, orbit layout
      const size_t hbase = hist_off(R.Malloc, R.T, 0, t - 1, tp, 0);
      auto stage = [&](const void *hist, TC *dst) {
        const TS *h = reinterpret_cast<const TS *>(hist) + hbase;
        constexpr int U = 4;
        for (int o0 = tid; o0 < S; o0 += U * nthr) {
          TS v[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int o = o0 + u * nthr;
            v[u] = (o < S) ? h[(size_t)(o / KC) * cstride + (o % KC)] : (TS)0;
          }
#pragma unroll
          for (int u = 0; u < U; ++u)
            if (o0 + u * nthr < S) dst[o0 + u * nthr] = (TC)v[u];
        }
        __syncthreads();
      };
      // the same with 16-byte asynchronous copies (FP32: half a chunk's 8 orbits each, the
      // padding orbits of the last chunk up to rup4(S) included); completes at a wait
      auto astage = [&](const void *hist, size_t hb, TC *dst, int nch, size_t cs) {
        const TS *h = reinterpret_cast<const TS *>(hist) + hb;
        const int lim = rup4(S);
        for (int q = tid; q < 2 * nch; q += nthr) {
          const int e0 = (q >> 1) * KC + (q & 1) * 4;
          if (e0 < lim) cp_async16(dst + e0, h + (size_t)(q >> 1) * cs + (q & 1) * 4);
        }
        cp_async_commit();
      };

      // forward transforms of F(t-1,t') -> bufF and rho(t-1,t') -> R2 (orbit layout);
      // each row is staged in the region the transform writes last, the rho row
      // fetched into L2 meanwhile
      for (int q = tid; q < R.nchunks; q += nthr)
        prefetch_l2(reinterpret_cast<const TS *>(R.hist_r) + hbase + q * cstride);
      if (prestaged)
        __syncthreads();  // every thread's copies have landed
      else
        stage(R.hist_F, c.bufF);
      sun_transform_hooked<TC>(
          c, [&](int o) { return c.bufF[o]; }, [&](int o, TC v) { c.bufF[o] = v; }, [] {},
          [&] {
            if (ASYNC) astage(R.hist_r, hbase, c.R2, R.nchunks, cstride);
          });
      if (ASYNC) {
        cp_async_wait_all();
        __syncthreads();
      } else {
        stage(R.hist_r, c.R2);
      }
      sun_transform<TC>(c, [&](int o) { return c.R2[o]; }, [&](int o, TC v) { c.R2[o] = v; });

      // pointwise sunset in position space (Evolution.jl:28-29, classical :114-115)
      const bool classical = (R.pexp == 2);
      for (int k = tid; k < S; k += nthr) {
        const TC Fx = c.bufF[k], rx = c.R2[k];
        const TC F2 = Fx * Fx, r2 = rx * rx;
        c.R2[k] = classical ? rx * F2 : rx * (F2 - (TC)(1 / 12.) * r2);
        c.bufF[k] = classical ? Fx * F2 : Fx * (F2 - (TC)0.75 * r2);
      }
      __syncthreads();

      // the next row of this CTA goes to L2 while the inverse transforms run; its F is
      // staged into the orbit buffer during the inverse F transform when it has this
      // lattice size (the same layout)
      const void *nhF = nullptr;
      size_t nhb = 0, ncs = 0;
      int nw = -1, ng = -1, nnch = 0;
      {
        int w2 = w, g2 = gi + 1;
        if (g2 >= nrow || tmin + (w - R.cta_base_sun) * nrow + g2 > t - 1) {  // the item's last row
          if (queue && nxt < 0) nxt = take();
          w2 = queue ? nxt : w + (int)gridDim.x;
          g2 = 0;
        }
        if (w2 >= 0 && w2 < total) {
          const RunDev &R2n = runs[run_at(base, nruns, w2)];
          const int ng2 = SCRATCH ? 1 : R2n.sun_rows;
          const int tp2 = max(1, t - R2n.M + 1) + (w2 - R2n.cta_base_sun) * ng2 + g2;
          if (pexp_sunset(R2n.pexp) && tp2 <= t - 1) {
            const size_t b2 = hist_off(R2n.Malloc, R2n.T, 0, t - 1, tp2, 0) * sizeof(TS);
            const size_t cs2 = (size_t)R2n.Malloc * R2n.Malloc * KC * sizeof(TS);
            for (int q = tid; q < R2n.nchunks; q += nthr) {
              prefetch_l2(reinterpret_cast<const char *>(R2n.hist_F) + b2 + q * cs2);
              prefetch_l2(reinterpret_cast<const char *>(R2n.hist_r) + b2 + q * cs2);
            }
            if (ASYNC && R2n.Ns == cur_ns) {
              nhF = R2n.hist_F;
              nhb = b2 / sizeof(TS);
              ncs = cs2 / sizeof(TS);
              nnch = R2n.nchunks;
              nw = w2;
              ng = g2;
            }
          }
        }
      }

      // inverse transforms: pass 3 leaves the orbit values in R2 (free once pass 2
      // has read B), then one coalesced sweep scales them into the Sigma rings
      // (ivol^3 * coefficient); the next writer of R2 is behind a barrier
      TS *sigr = reinterpret_cast<TS *>(R.sig_r) + (size_t)slot * KC;
      TS *sigF = reinterpret_cast<TS *>(R.sig_F) + (size_t)slot * KC;
      const TC fr = (TC)R.fac_r, fF = (TC)R.fac_F;
      auto flush = [&](TS *sig, TC f) {
        for (int o = tid; o < S; o += nthr)
          if (KB_DCHECK((size_t)slot * KC + gidx(o) < (size_t)R.nchunks * rowstride, R.err, DCHK_SUN_SIGMA))
            sig[gidx(o)] = (TS)(f * c.R2[o]);
      };
      const TC *gr = c.R2;
      // expand reads R2 into R1 before pass 1 overwrites R2
      sun_transform<TC>(c, [&](int o) { return gr[o]; }, [&](int o, TC v) { c.R2[o] = v; });
      flush(sigr, fr);
      const TC *gF = c.bufF;
      sun_transform_hooked<TC>(
          c, [&](int o) { return gF[o]; }, [&](int o, TC v) { c.R2[o] = v; },
          [&] {
            if (ASYNC && nw >= 0) {
              astage(nhF, nhb, c.bufF, nnch, ncs);
              pre_w = nw;
              pre_g = ng;
            }
          },
          [] {});
      flush(sigF, fF);
    }
  }
  if (ASYNC) cp_async_wait_all();  // no copy lands in this CTA's shared memory after it ends
}

}  // namespace

size_t sunset_smem_bytes(bool fp64, int H) { return SUN_SMEM_HEAD + sun_layout(fp64, SunGeom(H)).bytes; }

namespace {
// the tables of sunset_kernel for octant size H as the image of their shared memory
// ([0, regions) of sun_layout): one CTA builds them and writes them out
template <typename TC>
__global__ void __launch_bounds__(SUN_THREADS, 1) sun_image_kernel(int H, const double *__restrict__ Cm,
                                                                  unsigned char *__restrict__ img) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SunGeom g(H);
  const SunLayout L = sun_layout(sizeof(TC) == 8, g);
  (void)sun_build_tables<TC>(g, smem_raw, L.has_etab ? reinterpret_cast<uint16_t *>(smem_raw + L.etab) : nullptr,
                             [&](int X, int x) { return Cm[X * H + x]; });
  const uint4 *src = reinterpret_cast<const uint4 *>(smem_raw);
  uint4 *dst = reinterpret_cast<uint4 *>(img);
  for (size_t i = threadIdx.x; i < L.regions / 16; i += blockDim.x) dst[i] = src[i];
}
}  // namespace

size_t sunset_image_bytes(bool fp64, int H) { return sun_layout(fp64, SunGeom(H)).regions; }

cudaError_t launch_sunset_image(bool fp64, int H, const double *Cm, void *img, cudaStream_t st) {
  const size_t bytes = sunset_image_bytes(fp64, H);
  cudaError_t e = fp64 ? cudaFuncSetAttribute(sun_image_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)bytes)
                       : cudaFuncSetAttribute(sun_image_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)bytes);
  if (e != cudaSuccess) return e;
  if (fp64)
    sun_image_kernel<double><<<1, SUN_THREADS, bytes, st>>>(H, Cm, reinterpret_cast<unsigned char *>(img));
  else
    sun_image_kernel<float><<<1, SUN_THREADS, bytes, st>>>(H, Cm, reinterpret_cast<unsigned char *>(img));
  return cudaGetLastError();
}

// t' rows per sunset item of a run (FP32): up to 8 for the small lattices whose rows
// are short, as long as the work items of the largest pass of all the item's rows
// together stay within 5/4 of one round of the 512-thread kernel (Ns <= 20: 8,
// 24: 4, 32: 2, from 40 on: 1 -- longer rows would only coarsen the balance)
int sunset_rows_per_item(int H) {
  SunGeom g(H);
  const int p1 = (g.ne4 / 4 + g.no4 / 4) * (g.P4 / 4);
  const int items = p1 > g.n2 ? p1 : g.n2;
  for (int rows = 8; rows > 1; rows /= 2)
    if (items * rows <= SUN_THREADS + SUN_THREADS / 4) return rows;
  return 1;
}

size_t sunset_scratch_elems(int H) {
  SunGeom g(H);
  return (size_t)g.r1 + g.r2;
}

int sunset_grid(bool fp64, int num_sms, int total_rows) {
  (void)fp64;
  return total_rows < num_sms ? total_rows : num_sms;
}

// Kernel variants: FP64 (512 threads, global scratch); FP32 0: 1024 threads,
// 1 CTA per SM (the whole Ns = 64 octant in shared memory); FP32 1: 512 threads
// with registers for 2 CTAs per SM, which hide each other's barrier waits when
// the shared memory of two fits (Ns <= 48).
#define KB_SUNSET_F64 sunset_kernel<double, double, true, SUN_THREADS, 1>
#define KB_SUNSET_F32 sunset_kernel<float, float, false, SUN_THREADS_F32, 1>
#define KB_SUNSET_F32_HALF sunset_kernel<float, float, false, SUN_THREADS, 2>

int sunset_max_ctas_per_sm(bool fp64, int variant, size_t smem) {
  int n = 0;
  cudaError_t e = fp64 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, KB_SUNSET_F64, SUN_THREADS, smem)
                  : variant == 1
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, KB_SUNSET_F32_HALF, SUN_THREADS, smem)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, KB_SUNSET_F32, SUN_THREADS_F32, smem);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n < 1 ? 1 : n;
}

cudaError_t configure_sunset(bool fp64, size_t smem) {
  if (fp64) return cudaFuncSetAttribute(KB_SUNSET_F64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaError_t e = cudaFuncSetAttribute(KB_SUNSET_F32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(KB_SUNSET_F32_HALF, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_sunset(bool fp64, int variant, const RunDev *d_runs, const int *d_base, int nruns,
                          int total_rows, int grid, const int *d_t, void *scratch, size_t scratch_stride, size_t smem,
                          int *queue, cudaStream_t st) {
  if (total_rows <= 0 || grid <= 0) return cudaSuccess;
  if (queue) {  // a memset node in a captured step
    const cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
  }
  if (fp64)
    KB_SUNSET_F64<<<grid, SUN_THREADS, smem, st>>>(d_runs, d_base, nruns, total_rows, d_t,
                                                   reinterpret_cast<double *>(scratch), scratch_stride, queue);
  else if (variant == 1)
    KB_SUNSET_F32_HALF<<<grid, SUN_THREADS, smem, st>>>(d_runs, d_base, nruns, total_rows, d_t, nullptr, 0, queue);
  else
    KB_SUNSET_F32<<<grid, SUN_THREADS_F32, smem, st>>>(d_runs, d_base, nruns, total_rows, d_t, nullptr, 0, queue);
  return cudaGetLastError();
}

}  // namespace kb

// ---------------------------------------------------------------------------
// Allocation-free self-energies (kb_sunset_rows_noalloc)
//
// Same FP64 cosine-transform sunset as the persistent kernel above, for rows
// the caller passes in device memory, with the per-CTA transform scratch in a
// file-scope device array instead of a cudaMalloc'd buffer. The array holds
// NOALLOC_MAX_CTAS slots sized for the largest lattice accepted
// (Ns <= NOALLOC_MAX_NS): 160 x 5308 doubles = 6.8 MB, resident on every GPU
// that loads the library until the process exits.
// ---------------------------------------------------------------------------
namespace kb {
namespace {

constexpr int NOALLOC_MAX_NS = 32;
constexpr int NOALLOC_MAX_CTAS = 160;

constexpr size_t na_slot_elems(int H) {
  // the R1 + R2 regions of SunGeom for octant size H (pass intermediates)
  return (size_t)sun_r1(H) + (size_t)sun_r2(H);
}
constexpr size_t NOALLOC_SLOT_ELEMS = na_slot_elems(NOALLOC_MAX_NS / 2 + 1);

// Shared by every call on a device; contents persist between calls. Nothing in
// it needs to start at zero: each transform writes every element it reads.
__device__ __align__(256) double g_noalloc_scratch[NOALLOC_MAX_CTAS * NOALLOC_SLOT_ELEMS];

__global__ void __launch_bounds__(SUN_THREADS, 1)
sunset_rows_noalloc_kernel(int Ns, double fac_r, double fac_F, int classical, int nrows,
                           const double *__restrict__ F_rows, const double *__restrict__ r_rows,
                           double *__restrict__ sigF_rows, double *__restrict__ sigr_rows, double *scratch,
                           size_t stride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int H = Ns / 2 + 1;
  const SunGeom g(H);
  // cosine matrix of the even octant, C[X][x] = m(x) cos(2 pi x X / Ns)
  SunCtx<double> c = sun_build_tables<double>(g, smem_raw, nullptr, [&](int X, int x) {
    const double m = (x == 0 || 2 * x == Ns) ? 1.0 : 2.0;
    return m * cospi(2.0 * (double)((x * X) % Ns) / (double)Ns);
  });
  c.bufF = reinterpret_cast<double *>(smem_raw + sun_tables_bytes(true, g));
  c.R1 = scratch + (size_t)blockIdx.x * stride;
  c.R2 = c.R1 + g.r1;
  const int S = g.S;
  for (int row = blockIdx.x; row < nrows; row += gridDim.x) {
    const double *Fin = F_rows + (size_t)row * S;
    const double *rin = r_rows + (size_t)row * S;
    sun_transform<double>(c, [&](int o) { return Fin[o]; }, [&](int o, double v) { c.bufF[o] = v; });
    sun_transform<double>(c, [&](int o) { return rin[o]; }, [&](int o, double v) { c.R2[o] = v; });
    for (int k = threadIdx.x; k < S; k += blockDim.x) {
      const double Fx = c.bufF[k], rx = c.R2[k];
      const double F2 = Fx * Fx, r2 = rx * rx;
      c.R2[k] = classical ? rx * F2 : rx * (F2 - (1 / 12.) * r2);
      c.bufF[k] = classical ? Fx * F2 : Fx * (F2 - 0.75 * r2);
    }
    __syncthreads();
    double *outr = sigr_rows + (size_t)row * S;
    double *outF = sigF_rows + (size_t)row * S;
    const double *gr = c.R2;
    sun_transform<double>(c, [&](int o) { return gr[o]; }, [&](int o, double v) { outr[o] = fac_r * v; });
    const double *gF = c.bufF;
    sun_transform<double>(c, [&](int o) { return gF[o]; }, [&](int o, double v) { outF[o] = fac_F * v; });
  }
}

std::mutex g_noalloc_mu;
double *g_noalloc_ptr[64] = {};  // device address of g_noalloc_scratch, per device ordinal

}  // namespace
}  // namespace kb

extern "C" int kb_sunset_rows_noalloc(int32_t Ns, int32_t N, double lambda, int32_t pexp, int32_t nrows,
                                      const double *F_rows, const double *rho_rows, double *sigF_rows,
                                      double *sigr_rows, void *stream) {
  using namespace kb;
  char msg[256];
  if (!((Ns >= 2 && Ns <= NOALLOC_MAX_NS && Ns % 2 == 0) || Ns == 1)) {
    snprintf(msg, sizeof msg,
             "kb_sunset_rows_noalloc: Ns=%d is beyond the maximum of its fixed scratch (Ns must be 1 or even "
             "in [2,%d])",
             Ns, NOALLOC_MAX_NS);
    kb_set_global_error(msg);
    return KB_ERR_PARAM;
  }
  if (N < 1 || (pexp != KB_PEXP_NLO_QUANTUM && pexp != KB_PEXP_NLO_CLASSICAL) || nrows < 0 ||
      !std::isfinite(lambda)) {
    kb_set_global_error("kb_sunset_rows_noalloc: needs N >= 1, pexp = KB_PEXP_NLO_QUANTUM or "
                        "KB_PEXP_NLO_CLASSICAL, nrows >= 0 and a finite lambda");
    return KB_ERR_PARAM;
  }
  if (nrows == 0) return KB_OK;
  if (!F_rows || !rho_rows || !sigF_rows || !sigr_rows) {
    kb_set_global_error("kb_sunset_rows_noalloc: null row pointer");
    return KB_ERR_PARAM;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    kb_set_global_error("kb_sunset_rows_noalloc: no current CUDA device");
    return KB_ERR_NODEV;
  }
  double *scratch = nullptr;
  {
    // once per device, with that device current: device address of the array
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      cudaError_t e = cudaGetSymbolAddress((void **)&g_noalloc_ptr[dev], g_noalloc_scratch);
      if (e != cudaSuccess || !g_noalloc_ptr[dev]) {
        g_noalloc_ptr[dev] = nullptr;
        snprintf(msg, sizeof msg, "kb_sunset_rows_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        kb_set_global_error(msg);
        return KB_ERR_CUDA;
      }
    }
    scratch = g_noalloc_ptr[dev];
  }
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int H = Ns / 2 + 1;
  const size_t stride = na_slot_elems(H);
  int grid = nrows < NOALLOC_MAX_CTAS ? nrows : NOALLOC_MAX_CTAS;
  if (nsm > 0 && grid > nsm) grid = nsm;
  const double V = (double)Ns * Ns * Ns, iv = 1.0 / V, Nd = (double)N;
  const double fac_r = iv * iv * iv * (-(lambda * lambda) * (Nd + 2.0) / (6.0 * Nd * Nd));
  const double fac_F = iv * iv * iv * (-(lambda * lambda) * (Nd + 2.0) / (18.0 * Nd * Nd));
  const size_t smem = sun_tables_bytes(true, SunGeom(H)) + (size_t)rup4(sun_tet(H)) * sizeof(double);
  sunset_rows_noalloc_kernel<<<grid, SUN_THREADS, smem, (cudaStream_t)stream>>>(
      Ns, fac_r, fac_F, pexp == KB_PEXP_NLO_CLASSICAL ? 1 : 0, nrows, F_rows, rho_rows, sigF_rows, sigr_rows,
      scratch, stride);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, sizeof msg, "kb_sunset_rows_noalloc: launch failed: %s", cudaGetErrorString(e));
    kb_set_global_error(msg);
    return KB_ERR_CUDA;
  }
  return KB_OK;
}

// ---------------------------------------------------------------------------
// Adjoint of the sunset (reverse mode, FP64), used by kb_adjoint.
//
// Forward, per t' row z: Fx = A F, rx = A rho (A: orbit-level cosine transform),
// g_r = rx (Fx^2 - rx^2/12), g_F = Fx (Fx^2 - 3/4 rx^2),
// Sigma_rho = f_r A g_r, Sigma_F = f_F A g_F (classical: without the rx^2 terms).
// On the full lattice the transform is a symmetric matrix; on orbits its
// transpose is A^T = diag(deg) A diag(deg)^-1, so every adjoint transform
// divides by the orbit degeneracy, applies A and multiplies back.
// Given orbit adjoints Sbar_rho, Sbar_F of Sigma(t-1, z) (already weighted),
// this adds the adjoints of F(t-1, z), rho(t-1, z) into the adjoint history and
// writes the row's d L / d lambda partial (Sigma ~ lambda^2).
// ---------------------------------------------------------------------------
namespace kb {
namespace {

__global__ void __launch_bounds__(SUN_THREADS, 1)
sunset_adjoint_kernel(RunDev R, int t, const double *__restrict__ sbar_r, const double *__restrict__ sbar_F,
                      double *__restrict__ adjF, double *__restrict__ adjR, double *__restrict__ lam_part,
                      double *scratch, size_t stride, double lambda) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tmin = max(1, t - R.M + 1);
  const SunGeom g(R.H);
  double *bFx = reinterpret_cast<double *>(smem_raw + sun_tables_bytes(true, g));  // Fx, then adjoint of Fx / deg
  double *brx = bFx + rup4(g.S);      // rx, then adjoint of rx / deg
  double *bgr = brx + rup4(g.S);      // adjoint of g_r
  double *bgF = bgr + rup4(g.S);      // adjoint of g_F
  __shared__ double red[SUN_THREADS / 32];
  SunCtx<double> c = sun_build_tables<double>(g, smem_raw, nullptr, [&](int X, int x) { return R.Cm[X * g.H + x]; });
  c.R1 = scratch + (size_t)blockIdx.x * stride;
  c.R2 = c.R1 + g.r1;
  c.bufF = bFx;
  const int S = g.S, Spad = R.nchunks * KC;
  const bool classical = (R.pexp == 2);
  const size_t rowstride = (size_t)R.Malloc * KC;
  const int r3 = (t - 1) % 3;
  const double *deg = R.deg;
  const double *sigr = reinterpret_cast<const double *>(R.sig_r);
  const double *sigF = reinterpret_cast<const double *>(R.sig_F);
  auto gidx = [&](int o) { return (size_t)(o / KC) * rowstride + (o % KC); };
  for (int u = blockIdx.x; u < t - tmin; u += gridDim.x) {
    const int z = tmin + u;
    const int slot = z % R.Malloc;
    const double *stF = R.st_F + (size_t)r3 * R.nchunks * rowstride + (size_t)slot * KC;
    const double *stR = R.st_r + (size_t)r3 * R.nchunks * rowstride + (size_t)slot * KC;
    const double *sr = sbar_r + (size_t)slot * Spad;
    const double *sF = sbar_F + (size_t)slot * Spad;
    // Fx, rx of row t-1 (recomputed), and the adjoints of g_r, g_F
    sun_transform<double>(c, [&](int o) { return stF[gidx(o)]; }, [&](int o, double v) { bFx[o] = v; });
    sun_transform<double>(c, [&](int o) { return stR[gidx(o)]; }, [&](int o, double v) { brx[o] = v; });
    sun_transform<double>(c, [&](int o) { return sr[o] / deg[o]; },
                          [&](int o, double v) { bgr[o] = R.fac_r * v * deg[o]; });
    sun_transform<double>(c, [&](int o) { return sF[o] / deg[o]; },
                          [&](int o, double v) { bgF[o] = R.fac_F * v * deg[o]; });
    // pointwise Jacobian of (g_r, g_F) with respect to (Fx, rx); dL/dlambda partial
    double lam_acc = 0.0;
    for (int k = threadIdx.x; k < S; k += blockDim.x) {
      const double Fx = bFx[k], rx = brx[k], gr = bgr[k], gF = bgF[k];
      double dFx, drx;
      if (classical) {
        dFx = gr * 2 * rx * Fx + gF * 3 * Fx * Fx;
        drx = gr * Fx * Fx;
      } else {
        dFx = gr * 2 * rx * Fx + gF * (3 * Fx * Fx - 0.75 * rx * rx);
        drx = gr * (Fx * Fx - 0.25 * rx * rx) - gF * 1.5 * Fx * rx;
      }
      bFx[k] = dFx / deg[k];
      brx[k] = drx / deg[k];
      const size_t gi = gidx(k) + (size_t)slot * KC;
      lam_acc += sr[k] * sigr[gi] + sF[k] * sigF[gi];
    }
    for (int o = 16; o > 0; o >>= 1) lam_acc += __shfl_xor_sync(0xffffffffu, lam_acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lam_acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
      lam_part[slot] = (lambda != 0.0) ? 2.0 * s / lambda : 0.0;  // Sigma ~ lambda^2
    }
    // adjoints of F(t-1, z) and rho(t-1, z), added into the adjoint history
    const int T = R.T;
    sun_transform<double>(c, [&](int o) { return bFx[o]; }, [&](int o, double v) {
      adjF[hist_off(R.Malloc, T, o / KC, t - 1, z, o % KC)] += v * deg[o];
    });
    if (z < t - 1)
      sun_transform<double>(c, [&](int o) { return brx[o]; }, [&](int o, double v) {
        adjR[hist_off(R.Malloc, T, o / KC, t - 1, z, o % KC)] += v * deg[o];
      });
  }
}

}  // namespace

size_t sunset_adjoint_smem_bytes(int H) {
  return sun_tables_bytes(true, SunGeom(H)) + 4 * (size_t)rup4(sun_tet(H)) * sizeof(double);
}

cudaError_t launch_sunset_adjoint(const RunDev &R, int t, const double *sbar_r, const double *sbar_F, double *adjF,
                                  double *adjR, double *lam_part, void *scratch, size_t stride, int grid,
                                  double lambda, cudaStream_t st) {
  const size_t smem = sunset_adjoint_smem_bytes(R.H);
  cudaError_t e = cudaFuncSetAttribute(sunset_adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  sunset_adjoint_kernel<<<grid, SUN_THREADS, smem, st>>>(R, t, sbar_r, sbar_F, adjF, adjR, lam_part,
                                                         reinterpret_cast<double *>(scratch), stride, lambda);
  return cudaGetLastError();
}

}  // namespace kb

// ---------------------------------------------------------------------------
// 1/N expansion at NLO (calcSelfEnergies! for TwoPIScalarNinverseNLO,
// TwoPIScalar_Evolution.jl:144-758), FP64.
//
// The resummed kernels of the reference, I_rho^x (calcIrs!) and I_F^x
// (calcIFs!), are products and convolutions of x-space quantities; with the
// orbit cosine transform A (A A = V on orbits) they are diagonal in momentum.
// With the bubbles of every stored pair
//   Pr(a,b) = ivol^2 A[A F(a,b) . A rho(a,b)],   PF(a,b) = ivol^2 A[(A F)^2 - (A rho)^2 / 4]
// the momentum-space kernels I_k = A I_rho^x, J_k = A I_F^x of step t obey
//   I_k(t') = lam/3 Pr(t-1,t') - dt lam/3 sum_{z=t'+1}^{t-2} I_k(z) Pr(z,t'),      I_k(t-1) = 0
//   J_k(t') = lam/6 PF(t-1,t') - sum_{z=tmin}^{t-2} w_z lam/6 I_k(z) PF(z,t')
//                               + sum_{z=tmin}^{t'-1} w_z lam/3 J_k(z) Pr(z,t')
// (w_z = dt/2 at tmin, dt otherwise; Pr(z,t') = -Pr(t',z)), and the self-energies are
//   Sigma_rho = -lam/(3N) ivol^2 A[A F . A I_k + A rho . A J_k]
//   Sigma_F   = -lam/(3N) ivol^2 A[A F . A J_k - A rho . A I_k / 4]
// Three kernels per step: the bubbles of the new row t-1 (4 transforms per t',
// stored in two more rings with the history layout, so each pair's bubble is
// computed once), the two triangular Volterra solves per orbit chunk (one CTA
// per chunk, sequential in t', the sums over z split across 32 lanes), and the
// self-energies (6 transforms per t').
// ---------------------------------------------------------------------------
namespace kb {
namespace {

// shared memory: the tables of sun_transform, then NB orbit buffers
__host__ __device__ inline size_t ninv_rows_smem(int H, int NB) {
  return sun_tables_bytes(true, SunGeom(H)) + (size_t)NB * rup4(sun_tet(H)) * sizeof(double);
}

// MODE 0: bubbles of row t-1 (and of the pair (1,1) at t = 3); MODE 1: self-energies
template <int MODE>
__global__ void __launch_bounds__(SUN_THREADS, 1)
ninv_rows_kernel(const RunDev *__restrict__ runs, const int *__restrict__ sched, int nruns, int total,
                 const int *__restrict__ d_t, double *__restrict__ scratch, size_t stride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = *d_t;
  int cur_ns = -1;
  SunCtx<double> c{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, SunGeom(1)};
  double *buf[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int w = blockIdx.x; w < total; w += gridDim.x) {
    const int r = run_at(sched, nruns, w);
    const RunDev &R = runs[r];
    if (R.pexp != 4 || t < 3) continue;
    const int tmin = max(1, t - R.M + 1), tmone = t - 1;
    const int u = w - R.cta_base_sun;
    int a = tmone, tp = tmin + u;
    if (tp > tmone) {
      if (MODE == 0 && t == 3 && u == 2) {  // F(1,1) enters the first step's kernels
        a = 1;
        tp = 1;
      } else {
        continue;
      }
    }
    if (R.Ns != cur_ns) {
      __syncthreads();
      cur_ns = R.Ns;
      const SunGeom g(R.H);
      double *p = reinterpret_cast<double *>(smem_raw + sun_tables_bytes(true, g));
      for (int q = 0; q < (MODE == 0 ? 2 : 4); ++q) {
        buf[q] = p;
        p += rup4(g.S);
      }
      c = sun_build_tables<double>(g, smem_raw, nullptr, [&](int X, int x) { return R.Cm[X * g.H + x]; });
      c.R1 = scratch + (size_t)blockIdx.x * stride;
      c.R2 = c.R1 + g.r1;
      c.bufF = buf[0];
    }
    const int S = c.g.S, Spad = R.nchunks * KC;
    const size_t rowstride = (size_t)R.Malloc * KC;
    const int slot = tp % R.Malloc;
    const double *stF = R.st_F + (size_t)(a % 3) * R.nchunks * rowstride + (size_t)slot * KC;
    const double *stR = R.st_r + (size_t)(a % 3) * R.nchunks * rowstride + (size_t)slot * KC;
    auto gidx = [&](int o) { return (size_t)(o / KC) * rowstride + (o % KC); };
    double *Fx = buf[0], *rx = buf[1];
    sun_transform<double>(c, [&](int o) { return stF[gidx(o)]; }, [&](int o, double v) { Fx[o] = v; });
    sun_transform<double>(c, [&](int o) { return stR[gidx(o)]; }, [&](int o, double v) { rx[o] = v; });
    if (MODE == 0) {
      const double iv2 = R.ivol * R.ivol;
      const int T = R.T;
      sun_transform<double>(c, [&](int o) { return Fx[o] * rx[o]; },
                            [&](int o, double v) { R.pi_r[hist_off(R.Malloc, T, o / KC, a, tp, o % KC)] = iv2 * v; });
      sun_transform<double>(c, [&](int o) { return Fx[o] * Fx[o] - 0.25 * (rx[o] * rx[o]); },
                            [&](int o, double v) { R.pi_F[hist_off(R.Malloc, T, o / KC, a, tp, o % KC)] = iv2 * v; });
    } else {
      double *Ix = buf[2], *Jx = buf[3];
      const double *Ik = R.Ik + (size_t)slot * Spad, *Jk = R.Jk + (size_t)slot * Spad;
      sun_transform<double>(c, [&](int o) { return Ik[o]; }, [&](int o, double v) { Ix[o] = v; });
      sun_transform<double>(c, [&](int o) { return Jk[o]; }, [&](int o, double v) { Jx[o] = v; });
      double *sigr = reinterpret_cast<double *>(R.sig_r) + (size_t)slot * KC;
      double *sigF = reinterpret_cast<double *>(R.sig_F) + (size_t)slot * KC;
      const double fac = R.ninv_fac;
      sun_transform<double>(c, [&](int o) { return Fx[o] * Ix[o] + rx[o] * Jx[o]; },
                            [&](int o, double v) { sigr[gidx(o)] = fac * v; });
      sun_transform<double>(c, [&](int o) { return Fx[o] * Jx[o] - 0.25 * (rx[o] * Ix[o]); },
                            [&](int o, double v) { sigF[gidx(o)] = fac * v; });
    }
    (void)S;
  }
}

// One CTA per chunk of KC orbits solves both triangular systems of its orbits,
// blocked by the time tiles of the history layout (T times per block):
//   I_k, descending: for time block TB, the contributions of the solved blocks
//   above it (tiles (ZB, TB), ZB > TB) are summed by all threads -- thread
//   (group g, tile column tl, orbit j) -- with coalesced loads; then the
//   diagonal tile, staged in shared memory, is resolved t' by t' by KC threads.
//   J_k, ascending: the I_k term for every t' first (no dependence on J_k),
//   then the same blocked scheme for the J_k term over the blocks below.
constexpr int NV_T = 16;                  // the FP64 time tile
constexpr int NV_G = 8;                   // thread groups splitting the off-diagonal tiles
constexpr int NV_THREADS = NV_G * NV_T * KC;

// sum over the T rows zr in [0, nz) of tile (ZB, TB) at column tl, orbit j of
// v[z] * P(z, TB*T + tl): T independent loads (one tile row each, coalesced
// across the 4 columns x KC orbits of a warp), no branch for whole tiles
__device__ __forceinline__ double ninv_col_dot(const double *P, const double *v, size_t tile0, int Ma, int zbase,
                                               int tl, int j, int nz) {
  const double *vb = v + (size_t)(zbase % Ma) * KC + j;  // zbase is a block start: slots stay contiguous
  const double *pb = P + tile0 + j;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  if (nz == NV_T) {
#pragma unroll
    for (int zr = 0; zr < NV_T; zr += 4) {
      a0 += vb[zr * KC] * pb[(zr * NV_T + (tl ^ 0)) * KC];
      a1 += vb[(zr + 1) * KC] * pb[((zr + 1) * NV_T + (tl ^ 1)) * KC];
      a2 += vb[(zr + 2) * KC] * pb[((zr + 2) * NV_T + (tl ^ 2)) * KC];
      a3 += vb[(zr + 3) * KC] * pb[((zr + 3) * NV_T + (tl ^ 3)) * KC];
    }
  } else {
    for (int zr = 0; zr < nz; ++zr) a0 += vb[zr * KC] * pb[(zr * NV_T + (tl ^ (zr & 3))) * KC];
  }
  return (a0 + a1) + (a2 + a3);
}

// same along a tile row: sum over columns cl in [c0, c1) of v[z] * P(TB*T + row, zbase + cl)
__device__ __forceinline__ double ninv_row_dot(const double *P, const double *v, size_t tile0, int Ma, int zbase,
                                               int row, int j, int c0, int c1, const double *w) {
  const double *vb = v + (size_t)(zbase % Ma) * KC + j;
  const double *pb = P + tile0 + (size_t)row * NV_T * KC + j;
  const int sw = row & 3;
  double a0 = 0.0, a1 = 0.0;
  if (c0 == 0 && c1 == NV_T) {
#pragma unroll
    for (int cl = 0; cl < NV_T; cl += 2) {
      a0 += w[cl] * vb[cl * KC] * pb[(cl ^ sw) * KC];
      a1 += w[cl + 1] * vb[(cl + 1) * KC] * pb[((cl + 1) ^ sw) * KC];
    }
  } else {
    for (int cl = c0; cl < c1; ++cl) a0 += w[cl] * vb[cl * KC] * pb[(cl ^ sw) * KC];
  }
  return a0 + a1;
}

// One CTA per chunk of KC orbits solves both triangular systems of its orbits,
// blocked by the time tiles of the history layout:
//   I_k, descending in blocks: the contributions of the solved blocks above
//   (tiles (ZB, TB), ZB > TB) are column sums shared by two thread groups;
//   the diagonal tile, staged in shared memory, is resolved t' by t'.
//   J_k: its I_k term for every t' first (tile-wise, no dependence on J_k),
//   then ascending in blocks with the J_k term of the blocks below (row sums).
__global__ void __launch_bounds__(NV_THREADS, 1)
ninv_volterra_kernel(const RunDev *__restrict__ runs, const int *__restrict__ sched, int nruns,
                     const int *__restrict__ d_t) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int r = run_at(sched, nruns, blockIdx.x);
  const RunDev &R = runs[r];
  const int t = *d_t;
  if (R.pexp != 4 || t < 3 || R.T != NV_T) return;
  const int c = blockIdx.x - R.cta_base_mi;
  const int Ma = R.Malloc, Spad = R.nchunks * KC, nbA = Ma / NV_T;
  constexpr int T = NV_T;
  double *Iv = reinterpret_cast<double *>(smem_raw);  // [Ma][KC]
  double *Jv = Iv + (size_t)Ma * KC;                    // [Ma][KC]
  double *T1 = Jv + (size_t)Ma * KC;                    // [Ma][KC]: the I_k term of J_k
  double *red = T1 + (size_t)Ma * KC;                   // [NV_G][T][KC]
  double *tile = red + NV_G * T * KC;                   // [T][T][KC] diagonal tile
  double *prow = tile + T * T * KC;                     // [T][KC]: Pr or PF of (t-1, t') of the block
  double *wv = prow + T * KC;                           // [Ma]: trapezoid weights by slot
  const int tid = threadIdx.x, j = tid % KC, tl = (tid / KC) % T, g = tid / (KC * T);
  const int tmin = max(1, t - R.M + 1), tmone = t - 1;
  const double lam = R.lam, dt = R.dt;
  const double *PR = R.pi_r, *PF = R.pi_F;
  auto redsum = [&](int l, int jj) {  // the NV_G group sums of column l, fixed order
    double a = 0.0;
    for (int q = 0; q < NV_G; ++q) a += red[(q * T + l) * KC + jj];
    return a;
  };
  // start of tile (A, B) of this chunk (absolute time blocks)
  auto tile0 = [&](int A, int B) {
    return (((size_t)c * nbA + (size_t)((A * T) % Ma) / T) * nbA + (size_t)((B * T) % Ma) / T) * (size_t)T * T * KC;
  };
  const int J0 = tmin / T, Jn = tmone / T;
  for (int z = tid; z < Ma; z += NV_THREADS) wv[z] = 0.0;
  __syncthreads();
  for (int z = tmin + tid; z <= tmone; z += NV_THREADS) wv[z % Ma] = (z == tmin) ? 0.5 * dt : dt;
  if (tid < KC) Iv[(size_t)(tmone % Ma) * KC + j] = 0.0;
  __syncthreads();
  // ---- I_k(t') = lam/3 Pr(t-1,t') - dt lam/3 sum_{t' < z < t-1} I_k(z) Pr(z,t')
  for (int TB = Jn; TB >= J0; --TB) {
    double s = 0.0;
    for (int ZB = TB + 1 + g; ZB <= Jn; ZB += NV_G) {
      const int nz = min(T, tmone - ZB * T);  // rows z <= t-2 (I_k(t-1) = 0)
      if (nz > 0) s += ninv_col_dot(PR, Iv, tile0(ZB, TB), Ma, ZB * T, tl, j, nz);
    }
    red[(g * T + tl) * KC + j] = s;
    for (int q = tid; q < T * T * KC; q += NV_THREADS) {
      const int zr = q / (T * KC), cl = (q / KC) % T, jj = q % KC;
      tile[q] = PR[tile0(TB, TB) + (size_t)(zr * T + (cl ^ (zr & 3))) * KC + jj];
    }
    if (tid < T * KC) {  // Pr(t-1, t') of the block's columns
      const int l = tid / KC, p = TB * T + l;
      prow[tid] = (p >= tmin && p <= tmone) ? PR[hist_off(Ma, T, c, tmone, p, j)] : 0.0;
    }
    __syncthreads();
    if (tid < 4 * 32) {
      // the diagonal tile, t' by t': warp w resolves orbits 2w, 2w+1 with one lane per row zr
      const int lane = tid & 31, jj = 2 * (tid >> 5) + (lane >> 4), zr = lane & 15;
      const int zmax = min(T - 1, tmone - 1 - TB * T), sb = (TB * T) % Ma;
      for (int l = T - 1; l >= 0; --l) {
        const int p = TB * T + l;
        if (p < tmin || p > tmone - 1) continue;
        double v = (zr > l && zr <= zmax) ? Iv[(size_t)(sb + zr) * KC + jj] * tile[(zr * T + l) * KC + jj] : 0.0;
        for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (zr == 0) Iv[(size_t)(sb + l) * KC + jj] = lam / 3. * prow[l * KC + jj] - dt * lam / 3. * (redsum(l, jj) + v);
        __syncwarp();
      }
    }
    __syncthreads();
  }
  // ---- T1(t') = sum_{tmin <= z <= t-2} w_z I_k(z) PF(z, t') (PF symmetric): tile-wise,
  //      column sums for z >= t' (tiles (ZB, TB), ZB >= TB) and row sums for z < t'
  for (int TB = J0; TB <= Jn; ++TB) {
    double s = 0.0;
    const int p = TB * T + tl;
    if (p >= tmin && p <= tmone) {
      for (int ZB = TB + g; ZB <= Jn; ZB += NV_G) {
        // rows z = ZB*T + zr with z >= p, tmin <= z <= t-2, weighted
        const int zlo = max(ZB * T, max(p, tmin)), zhi = min(ZB * T + T - 1, tmone - 1);
        const size_t t0 = tile0(ZB, TB);
        const int sb = (ZB * T) % Ma;
        for (int z = zlo; z <= zhi; ++z) {
          const int zr = z - ZB * T;
          s += wv[sb + zr] * Iv[(size_t)(sb + zr) * KC + j] * PF[t0 + (size_t)(zr * T + (tl ^ (zr & 3))) * KC + j];
        }
      }
      for (int ZB = J0 + g; ZB <= TB; ZB += NV_G) {
        // columns z = ZB*T + cl with tmin <= z < p: row p of tile (TB, ZB)
        const int c0 = max(0, tmin - ZB * T), c1 = min(T, p - ZB * T);
        if (c1 > c0) s += ninv_row_dot(PF, Iv, tile0(TB, ZB), Ma, ZB * T, tl, j, c0, c1, wv + ((ZB * T) % Ma));
      }
    }
    red[(g * T + tl) * KC + j] = s;
    __syncthreads();
    if (g == 0 && p >= tmin && p <= tmone) T1[(size_t)(p % Ma) * KC + j] = redsum(tl, j);
    __syncthreads();
  }
  // ---- J_k(t') = lam/6 PF(t-1,t') - lam/6 T1(t') + lam/3 sum_{tmin <= z < t'} w_z J_k(z) Pr(z,t'),
  //      Pr(z,t') = -Pr(t',z) for z < t'
  for (int TB = J0; TB <= Jn; ++TB) {
    const int p = TB * T + tl;
    double s = 0.0;
    if (p >= tmin && p <= tmone)
      for (int ZB = J0 + g; ZB < TB; ZB += NV_G) {
        const int c0 = max(0, tmin - ZB * T);
        s -= ninv_row_dot(PR, Jv, tile0(TB, ZB), Ma, ZB * T, tl, j, c0, T, wv + ((ZB * T) % Ma));
      }
    red[(g * T + tl) * KC + j] = s;
    for (int q = tid; q < T * T * KC; q += NV_THREADS) {
      const int pr_ = q / (T * KC), cl = (q / KC) % T, jj = q % KC;
      tile[q] = PR[tile0(TB, TB) + (size_t)(pr_ * T + (cl ^ (pr_ & 3))) * KC + jj];
    }
    if (tid < T * KC) {
      const int l = tid / KC, pp = TB * T + l;
      prow[tid] = (pp >= tmin && pp <= tmone) ? PF[hist_off(Ma, T, c, tmone, pp, j)] : 0.0;
    }
    __syncthreads();
    if (tid < 4 * 32) {
      const int lane = tid & 31, jj = 2 * (tid >> 5) + (lane >> 4), zr = lane & 15;
      const int zmin = max(0, tmin - TB * T), sb = (TB * T) % Ma;
      for (int l = 0; l < T; ++l) {
        const int pp = TB * T + l;
        if (pp < tmin || pp > tmone) continue;
        double v = (zr < l && zr >= zmin)
                       ? -wv[sb + zr] * Jv[(size_t)(sb + zr) * KC + jj] * tile[(l * T + zr) * KC + jj]
                       : 0.0;
        for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (zr == 0)
          Jv[(size_t)(sb + l) * KC + jj] = lam / 6. * prow[l * KC + jj] -
                                           lam / 6. * T1[(size_t)(sb + l) * KC + jj] + lam / 3. * (redsum(l, jj) + v);
        __syncwarp();
      }
    }
    __syncthreads();
  }
  for (int q = tid; q < (tmone - tmin + 1) * KC; q += NV_THREADS) {
    const int tp = tmin + q / KC, jj = q % KC;
    const size_t o = (size_t)(tp % Ma) * Spad + (size_t)c * KC + jj;
    R.Ik[o] = Iv[(size_t)(tp % Ma) * KC + jj];
    R.Jk[o] = Jv[(size_t)(tp % Ma) * KC + jj];
  }
}

}  // namespace

size_t ninv_smem_bytes(int H) { return ninv_rows_smem(H, 4); }
size_t ninv_volterra_smem_bytes(int Malloc) {
  // I_k, J_k, their I_k term, block sums, one diagonal tile, a row of the block, weights
  return ((size_t)3 * Malloc * KC + NV_G * NV_T * KC + NV_T * NV_T * KC + NV_T * KC + Malloc) * sizeof(double);
}

cudaError_t configure_ninv(size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(ninv_rows_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(ninv_rows_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(ninv_volterra_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_ninv(const RunDev *d_runs, const int *d_sched_sun, const int *d_sched_mi, int nruns,
                        int total_rows, int total_ctas, int grid, const int *d_t, void *scratch, size_t scratch_stride,
                        size_t smem_rows, size_t smem_volterra, cudaStream_t st) {
  if (total_rows <= 0 || grid <= 0) return cudaSuccess;
  double *sc = reinterpret_cast<double *>(scratch);
  ninv_rows_kernel<0><<<grid, SUN_THREADS, smem_rows, st>>>(d_runs, d_sched_sun, nruns, total_rows, d_t, sc,
                                                             scratch_stride);
  ninv_volterra_kernel<<<total_ctas, NV_THREADS, smem_volterra, st>>>(d_runs, d_sched_mi, nruns, d_t);
  ninv_rows_kernel<1><<<grid, SUN_THREADS, smem_rows, st>>>(d_runs, d_sched_sun, nruns, total_rows, d_t, sc,
                                                             scratch_stride);
  return cudaGetLastError();
}

}  // namespace kb
