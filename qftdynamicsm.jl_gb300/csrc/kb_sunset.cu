// kb_sunset.cu -- the 3-loop sunset self-energy of one KB step.
//
// Replaces calcSelfEnergies!/calcSelfEnergyattp! (src/TwoPIScalar/
// TwoPIScalar_Evolution.jl:16-31 quantum, :107-121 classical): for every t'
// of the window
//   Fx = Re rfft F(t-1,t'),  rx = Re rfft rho(t-1,t')
//   Sigma_rho(t') = ivol^3 (-lambda^2 (N+2)/(6 N^2))  brfft[rx (Fx^2 - rx^2/12)]
//   Sigma_F(t')   = ivol^3 (-lambda^2 (N+2)/(18 N^2)) brfft[Fx (Fx^2 - 3/4 rx^2)]
//
// F and rho are cubic-symmetric, so both transforms reduce to cosine
// transforms on the even octant [0, H)^3 (H = Ns/2 + 1) with the matrix
// C[X][x] = m(x) cos(2 pi x X / Ns) (m = 1 at 0 and Ns/2, else 2), applied
// along the three axes. The data stay on cubic orbits (S = C(H+2,3) values):
// for a fixed first output coordinate X the three axis passes need only a
// slab of H(H+1)/2 + H^2 values, so a whole t' row is transformed in shared
// memory by one CTA without touching the full lattice:
//   pass 1  B_X(y,z)  = sum_x C[X][x] f(x,y,z)          y <= z  (symmetric in y,z)
//   pass 2  C_X(Y,z)  = sum_y C[Y][y] B_X(y,z)          Y >= X
//   pass 3  P(X,Y,Z)  = sum_z C[Z][z] C_X(Y,z)          X <= Y <= Z  (an orbit)
// 1.44 M multiply-adds per transform at Ns = 64 instead of 3.6 M on the octant
// and far fewer than the 4 full-lattice FFTs of the reference.
//
// One CTA per t' (grid = sum over runs of M); CTAs with t' outside the window
// return at once, so the same launch serves every step of a CUDA graph.
#include "kb_internal.cuh"

namespace kb {
namespace {

constexpr int SUN_THREADS = 256;

template <typename TC>
struct SunSmem {
  TC *Cm, *bufA, *bufB, *bufC, *Bx, *C2;
  uint16_t *pairs;
};

template <typename TC>
__device__ inline SunSmem<TC> sun_layout(unsigned char *raw, int H, int S) {
  SunSmem<TC> s;
  const int P = H * (H + 1) / 2;
  TC *p = reinterpret_cast<TC *>(raw);
  s.Cm = p;
  p += H * H;
  s.bufA = p;
  p += S;
  s.bufB = p;
  p += S;
  s.bufC = p;
  p += S;
  s.Bx = p;
  p += P;
  s.C2 = p;
  p += H * H;
  s.pairs = reinterpret_cast<uint16_t *>(p);
  return s;
}

// Cosine transform of a cubic-symmetric function given on orbits `in`;
// out(orbit, value) receives every orbit once. Ends with a barrier.
template <typename TC, typename Out>
__device__ void octant_transform3(const SunSmem<TC> &s, const TC *in, int H, Out out) {
  const int P = H * (H + 1) / 2;
  const TC *Cm = s.Cm;
  for (int X = 0; X < H; ++X) {
    const TC *cX = Cm + X * H;
    // pass 1: B_X(y,z) for y <= z; f(x,y,z) looked up on its sorted orbit
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
      const int y = s.pairs[p] & 255, z = s.pairs[p] >> 8;
      const int t3z = (int)tet3(z), t2y = tri2(y), t2z = tri2(z);
      TC acc = 0;
      int x = 0;
      for (; x <= y; ++x) acc += cX[x] * in[t3z + t2y + x];          // (x, y, z)
      for (; x <= z; ++x) acc += cX[x] * in[t3z + tri2(x) + y];      // (y, x, z)
      for (; x < H; ++x) acc += cX[x] * in[(int)tet3(x) + t2z + y];  // (y, z, x)
      s.Bx[p] = acc;
    }
    __syncthreads();
    // pass 2: C_X(Y,z) for Y >= X and all z
    const int n2 = (H - X) * H;
    for (int q = threadIdx.x; q < n2; q += blockDim.x) {
      const int Yo = q / H, z = q - Yo * H;
      const TC *cY = Cm + (X + Yo) * H;
      const int t2z = tri2(z);
      TC acc = 0;
      int y = 0;
      for (; y <= z; ++y) acc += cY[y] * s.Bx[t2z + y];
      for (; y < H; ++y) acc += cY[y] * s.Bx[tri2(y) + z];
      s.C2[Yo * H + z] = acc;
    }
    __syncthreads();
    // pass 3: P(X,Y,Z) for X <= Y <= Z
    const int h = H - X;
    const int n3 = h * (h + 1) / 2;
    for (int q = threadIdx.x; q < n3; q += blockDim.x) {
      const int Yo = s.pairs[q] & 255, Zo = s.pairs[q] >> 8;
      const TC *cZ = Cm + (X + Zo) * H;
      const TC *c2 = s.C2 + Yo * H;
      TC acc = 0;
      for (int z = 0; z < H; ++z) acc += cZ[z] * c2[z];
      out(orb3(X, X + Yo, X + Zo), acc);
    }
    // the next pass 1 writes Bx only, which pass 3 does not read
  }
  __syncthreads();
}

template <typename TC, typename TS>
__global__ void __launch_bounds__(SUN_THREADS)
sunset_kernel(const RunDev *__restrict__ runs, const int *__restrict__ base, int nruns,
              const int *__restrict__ d_t, int *__restrict__ d_err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int r = find_run(base, nruns, blockIdx.x);
  const RunDev &R = runs[r];
  const int t = *d_t;  // Sigma(t-1, t') for t' in [tmin, t-1]
  const int tmin = max(1, t - R.M + 1);
  const int tp = tmin + (int)(blockIdx.x - R.cta_base_sun);
  if (R.pexp == 0 || tp > t - 1 || t < 3) return;
  const int H = R.H, S = R.S;
  const int P = H * (H + 1) / 2;
  SunSmem<TC> s = sun_layout<TC>(smem_raw, H, S);

  for (int i = threadIdx.x; i < H * H; i += blockDim.x) s.Cm[i] = (TC)R.Cm[i];
  for (int z = threadIdx.x; z < H; z += blockDim.x)
    for (int y = 0; y <= z; ++y) s.pairs[tri2(z) + y] = (uint16_t)(y | (z << 8));
  (void)P;

  // row t-1 of the FP64 leapfrog state: F(t-1, t'), rho(t-1, t')
  const int r3 = (t - 1) % 3;
  const int slot = tp % R.Malloc;
  const size_t rowstride = (size_t)R.Malloc * KC;
  const double *stF = R.st_F + (size_t)r3 * R.nchunks * rowstride + (size_t)slot * KC;
  const double *stR = R.st_r + (size_t)r3 * R.nchunks * rowstride + (size_t)slot * KC;
  for (int k = threadIdx.x; k < S; k += blockDim.x)
    s.bufA[k] = (TC)stF[(size_t)(k / KC) * rowstride + (k % KC)];
  __syncthreads();
  octant_transform3<TC>(s, s.bufA, H, [&](int o, TC v) { s.bufB[o] = v; });  // Fx
  for (int k = threadIdx.x; k < S; k += blockDim.x)
    s.bufA[k] = (TC)stR[(size_t)(k / KC) * rowstride + (k % KC)];
  __syncthreads();
  octant_transform3<TC>(s, s.bufA, H, [&](int o, TC v) { s.bufC[o] = v; });  // rx

  // pointwise sunset in position space (Evolution.jl:28-29, classical :114-115)
  const bool classical = (R.pexp == 2);
  for (int k = threadIdx.x; k < S; k += blockDim.x) {
    const TC Fx = s.bufB[k], rx = s.bufC[k];
    const TC F2 = Fx * Fx, r2 = rx * rx;
    s.bufC[k] = classical ? rx * F2 : rx * (F2 - (TC)(1 / 12.) * r2);
    s.bufB[k] = classical ? Fx * F2 : Fx * (F2 - (TC)0.75 * r2);
  }
  __syncthreads();

  TS *sigr = reinterpret_cast<TS *>(R.sig_r) + (size_t)slot * KC;
  TS *sigF = reinterpret_cast<TS *>(R.sig_F) + (size_t)slot * KC;
  const double fr = R.fac_r, fF = R.fac_F;
  octant_transform3<TC>(s, s.bufC, H, [&](int o, TC v) {
    sigr[(size_t)(o / KC) * rowstride + (o % KC)] = (TS)(fr * (double)v);
  });
  octant_transform3<TC>(s, s.bufB, H, [&](int o, TC v) {
    sigF[(size_t)(o / KC) * rowstride + (o % KC)] = (TS)(fF * (double)v);
  });
  (void)d_err;
}

}  // namespace

size_t sunset_smem_bytes(bool fp64, int H) {
  const size_t S = (size_t)H * (H + 1) * (H + 2) / 6;
  const size_t P = (size_t)H * (H + 1) / 2;
  const size_t elems = 2 * (size_t)H * H + 3 * S + P;
  return elems * (fp64 ? sizeof(double) : sizeof(float)) + P * sizeof(uint16_t) + 16;
}

cudaError_t configure_sunset(bool fp64, size_t smem) {
  if (fp64)
    return cudaFuncSetAttribute(sunset_kernel<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
  return cudaFuncSetAttribute(sunset_kernel<float, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem);
}

cudaError_t launch_sunset(bool fp64, const RunDev *d_runs, const int *d_base, int nruns, int total_ctas,
                          const int *d_t, int *d_err, size_t smem, cudaStream_t st) {
  if (total_ctas <= 0) return cudaSuccess;
  if (fp64)
    sunset_kernel<double, double><<<total_ctas, SUN_THREADS, smem, st>>>(d_runs, d_base, nruns, d_t, d_err);
  else
    sunset_kernel<float, float><<<total_ctas, SUN_THREADS, smem, st>>>(d_runs, d_base, nruns, d_t, d_err);
  return cudaGetLastError();
}

}  // namespace kb
