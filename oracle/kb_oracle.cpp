// kb_oracle.cpp -- CPU FP64 restatement of the TwoPIScalar Kadanoff-Baym step.
//
// TEST INFRASTRUCTURE ONLY: the parity checker for libkb2pi. See kb_oracle.h
// for the parity status ("parity unpinned" against outputs of the Julia
// reference, which cannot run here) and for what pins it instead.
//
// Each function names the reference lines it restates (paths relative to the
// root of magdalenaeriksson/QFTdynamicsM.jl). Per-site operation order follows
// the Julia broadcasts so that the engines agree with the reference's
// arithmetic as closely as a different FFT allows.
#include "kb_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

typedef std::complex<double> cplx;

// ---------------------------------------------------------------------------
// Mixed-radix complex FFT (unnormalised, sign -1 forward / +1 backward), the
// convention of FFTW's rfft/brfft used at TwoPIScalar_SimDataStruct.jl:381-382.
// ---------------------------------------------------------------------------
struct FFTPlan {
  int n = 0;
  std::vector<int> factors;
  std::vector<cplx> tw;  // exp(-2 pi i j / n), j < n
  explicit FFTPlan(int n_ = 1) : n(n_) {
    int m = n;
    for (int p = 2; m > 1;) {
      if (m % p == 0) {
        factors.push_back(p);
        m /= p;
      } else {
        ++p;
      }
    }
    tw.resize(std::max(n, 1));
    for (int j = 0; j < n; ++j) {
      double a = -2.0 * M_PI * (double)j / (double)n;
      tw[j] = cplx(std::cos(a), std::sin(a));
    }
  }
  // w_len^(e) for the given sign, expressed through the length-n table
  inline cplx w(int len, long e, int sign) const {
    long j = ((e % len) + len) % len;
    cplx v = tw[(size_t)(j * (n / len))];
    return sign < 0 ? v : std::conj(v);
  }
  void rec(cplx *out, const cplx *in, int len, int stride, int sign, int fi,
           std::vector<cplx> &tmp) const {
    if (len == 1) {
      out[0] = in[0];
      return;
    }
    const int p = factors[fi];
    const int m = len / p;
    for (int r = 0; r < p; ++r) rec(out + r * m, in + r * stride, m, stride * p, sign, fi + 1, tmp);
    cplx *t = tmp.data() + (size_t)fi * 64;  // radix <= 64 per level scratch
    cplx small[64];
    for (int k = 0; k < m; ++k) {
      for (int r = 0; r < p; ++r) t[r] = out[r * m + k] * w(len, (long)r * k, sign);
      for (int q = 0; q < p; ++q) {
        cplx s = 0;
        for (int r = 0; r < p; ++r) s += t[r] * w(p, (long)r * q, sign);
        small[q] = s;
      }
      for (int q = 0; q < p; ++q) out[k + q * m] = small[q];
    }
  }
  // in-place transform of a strided line
  void run(cplx *data, int stride, int sign, std::vector<cplx> &buf_in,
           std::vector<cplx> &buf_out, std::vector<cplx> &tmp) const {
    if (n == 1) return;
    for (int i = 0; i < n; ++i) buf_in[i] = data[(size_t)i * stride];
    rec(buf_out.data(), buf_in.data(), n, 1, sign, 0, tmp);
    for (int i = 0; i < n; ++i) data[(size_t)i * stride] = buf_out[i];
  }
};

// ---------------------------------------------------------------------------
// Batched Stockham FFT (decimation in frequency, self-sorting), used for the
// real lattice transforms rfft / brfft of the sunset. Data are split into real
// and imaginary arrays x[i][l] (i < n the transform index, l < L independent
// lines side by side), so every butterfly runs over L contiguous values. One
// radix-r stage of length len = r m maps
//   y[q + s (r p + k)] = W_len^(p k) sum_j x[q + s (p + m j)] w_r^(j k),
// q < s (sub-transforms already split off), p < m, k < r; s grows by r per
// stage and the last stage leaves the natural frequency order.
// ---------------------------------------------------------------------------
struct BatchFFT {
  int n = 1;
  std::vector<int> radix;         // stage radices: 4s first, then 2, then odd primes
  std::vector<double> twr, twi;   // exp(-2 pi i j / n), j < n
  explicit BatchFFT(int n_ = 1) : n(n_) {
    int m = n;
    while (m % 4 == 0) { radix.push_back(4); m /= 4; }
    while (m % 2 == 0) { radix.push_back(2); m /= 2; }
    for (int p = 3; m > 1; p += 2)
      while (m % p == 0) { radix.push_back(p); m /= p; }
    twr.resize(n);
    twi.resize(n);
    for (int j = 0; j < n; ++j) {
      double a = -2.0 * M_PI * (double)j / (double)n;
      twr[j] = std::cos(a);
      twi[j] = std::sin(a);
    }
  }
  // Transforms (xr, xi) in place (sign -1 forward, +1 backward, unnormalised);
  // (wr, wi) are work arrays of n * L values each.
  void run(double *xr, double *xi, double *wr, double *wi, long L, int sign) const {
    if (n == 1) return;
    double *ar = xr, *ai = xi, *br = wr, *bi = wi;
    long s = 1;
    int len = n;
    const double sg = sign < 0 ? 1.0 : -1.0;  // conjugates the table for the backward transform
    for (int r : radix) {
      const int m = len / r;
      const int tstep = n / len;
      for (int p = 0; p < m; ++p) {
        double wkr[64], wki[64];
        for (int k = 0; k < r; ++k) {
          long e = ((long)p * k * tstep) % n;
          wkr[k] = twr[e];
          wki[k] = sg * twi[e];
        }
        for (long q = 0; q < s; ++q) {
          if (r == 2) {
            const double *a0r = ar + (q + s * p) * L, *a0i = ai + (q + s * p) * L;
            const double *a1r = ar + (q + s * (p + m)) * L, *a1i = ai + (q + s * (p + m)) * L;
            double *y0r = br + (q + s * (2 * p)) * L, *y0i = bi + (q + s * (2 * p)) * L;
            double *y1r = br + (q + s * (2 * p + 1)) * L, *y1i = bi + (q + s * (2 * p + 1)) * L;
            const double c = wkr[1], d = wki[1];
            for (long l = 0; l < L; ++l) {
              double ur = a0r[l] - a1r[l], ui = a0i[l] - a1i[l];
              y0r[l] = a0r[l] + a1r[l];
              y0i[l] = a0i[l] + a1i[l];
              y1r[l] = ur * c - ui * d;
              y1i[l] = ur * d + ui * c;
            }
          } else if (r == 4) {
            const double *a0r = ar + (q + s * p) * L, *a0i = ai + (q + s * p) * L;
            const double *a1r = ar + (q + s * (p + m)) * L, *a1i = ai + (q + s * (p + m)) * L;
            const double *a2r = ar + (q + s * (p + 2 * m)) * L, *a2i = ai + (q + s * (p + 2 * m)) * L;
            const double *a3r = ar + (q + s * (p + 3 * m)) * L, *a3i = ai + (q + s * (p + 3 * m)) * L;
            double *yr[4], *yi[4];
            for (int k = 0; k < 4; ++k) {
              yr[k] = br + (q + s * (4 * p + k)) * L;
              yi[k] = bi + (q + s * (4 * p + k)) * L;
            }
            // w_4 = exp(sign i pi / 2) = sign * i
            const double sgn = sign < 0 ? -1.0 : 1.0;
            for (long l = 0; l < L; ++l) {
              double s02r = a0r[l] + a2r[l], s02i = a0i[l] + a2i[l];
              double d02r = a0r[l] - a2r[l], d02i = a0i[l] - a2i[l];
              double s13r = a1r[l] + a3r[l], s13i = a1i[l] + a3i[l];
              double d13r = a1r[l] - a3r[l], d13i = a1i[l] - a3i[l];
              // w_4 * d13 = sgn * i * d13
              double wdr = -sgn * d13i, wdi = sgn * d13r;
              double c0r = s02r + s13r, c0i = s02i + s13i;
              double c1r = d02r + wdr, c1i = d02i + wdi;
              double c2r = s02r - s13r, c2i = s02i - s13i;
              double c3r = d02r - wdr, c3i = d02i - wdi;
              yr[0][l] = c0r;
              yi[0][l] = c0i;
              yr[1][l] = c1r * wkr[1] - c1i * wki[1];
              yi[1][l] = c1r * wki[1] + c1i * wkr[1];
              yr[2][l] = c2r * wkr[2] - c2i * wki[2];
              yi[2][l] = c2r * wki[2] + c2i * wkr[2];
              yr[3][l] = c3r * wkr[3] - c3i * wki[3];
              yi[3][l] = c3r * wki[3] + c3i * wkr[3];
            }
          } else {
            // generic radix: direct small DFT with w_r^(jk) = tw[(j k mod r) n / r]
            for (long l = 0; l < L; ++l) {
              double xr_[64], xi_[64];
              for (int j = 0; j < r; ++j) {
                xr_[j] = ar[(q + s * (p + (long)m * j)) * L + l];
                xi_[j] = ai[(q + s * (p + (long)m * j)) * L + l];
              }
              for (int k = 0; k < r; ++k) {
                double cr = 0.0, ci = 0.0;
                for (int j = 0; j < r; ++j) {
                  long e = ((long)(j * k) % r) * (n / r);
                  double vr = twr[e], vi = sg * twi[e];
                  cr += xr_[j] * vr - xi_[j] * vi;
                  ci += xr_[j] * vi + xi_[j] * vr;
                }
                br[(q + s * ((long)r * p + k)) * L + l] = cr * wkr[k] - ci * wki[k];
                bi[(q + s * ((long)r * p + k)) * L + l] = cr * wki[k] + ci * wkr[k];
              }
            }
          }
        }
      }
      std::swap(ar, br);
      std::swap(ai, bi);
      s *= r;
      len = m;
    }
    if (ar != xr) {
      std::memcpy(xr, ar, sizeof(double) * (size_t)n * L);
      std::memcpy(xi, ai, sizeof(double) * (size_t)n * L);
    }
  }
};

// FFTW's rfft / brfft of a real column-major lattice of sdim axes of length Ns
// (TwoPIScalar_SimDataStruct.jl:381-382): the half spectrum has H = Ns/2 + 1
// entries along the first axis, stored [k_sdim]...[k_1] with k_0 < H fastest.
// The first axis runs two real lines per complex transform; the other axes
// run batched over the contiguous planes.
struct RealFFT3 {
  int Ns = 1, sdim = 3, H = 1;
  long V = 1, nlines = 1, HV = 1;  // sites, lines along axis 0, half-spectrum size
  BatchFFT f;
  static const int B = 16;  // line pairs per batch of the first axis
  void setup(int Ns_, int sdim_) {
    Ns = Ns_;
    sdim = sdim_;
    H = Ns / 2 + 1;
    V = 1;
    for (int d = 0; d < sdim; ++d) V *= Ns;
    nlines = V / Ns;
    HV = (long)H * nlines;
    f = BatchFFT(Ns);
  }
  struct Work {
    std::vector<double> hr, hi, wr, wi, br, bi;
  };
  void alloc(Work &w) const {
    w.hr.resize(HV);
    w.hi.resize(HV);
    size_t big = std::max<size_t>((size_t)HV, (size_t)Ns * B);
    w.wr.resize(big);
    w.wi.resize(big);
    w.br.resize((size_t)Ns * B);
    w.bi.resize((size_t)Ns * B);
  }
  // axes 1.. of the half spectrum (in w.hr/hi), sign as for BatchFFT::run
  void outer_axes(Work &w, int sign) const {
    long inner = H;
    for (int d = 1; d < sdim; ++d) {
      const long block = inner * Ns;
      for (long o = 0; o < HV; o += block)
        f.run(w.hr.data() + o, w.hi.data() + o, w.wr.data(), w.wi.data(), inner, sign);
      inner = block;
    }
  }
  // out[k] = Re rfft(x)[k] on the half spectrum (HV values)
  void rfft_re(const double *x, double *out, Work &w) const {
    const int n = Ns;
    for (long l0 = 0; l0 < nlines; l0 += 2 * B) {
      const long nb = std::min<long>(B, (nlines - l0 + 1) / 2);
      for (int i = 0; i < n; ++i)
        for (long b = 0; b < nb; ++b) {
          long la = l0 + 2 * b, lb = la + 1;
          w.br[(size_t)i * nb + b] = x[la * n + i];
          w.bi[(size_t)i * nb + b] = lb < nlines ? x[lb * n + i] : 0.0;
        }
      f.run(w.br.data(), w.bi.data(), w.wr.data(), w.wi.data(), nb, -1);
      for (long b = 0; b < nb; ++b) {
        long la = l0 + 2 * b, lb = la + 1;
        for (int k = 0; k < H; ++k) {
          const int mk = (n - k) % n;
          double zr = w.br[(size_t)k * nb + b], zi = w.bi[(size_t)k * nb + b];
          double yr = w.br[(size_t)mk * nb + b], yi = w.bi[(size_t)mk * nb + b];
          w.hr[la * H + k] = 0.5 * (zr + yr);
          w.hi[la * H + k] = 0.5 * (zi - yi);
          if (lb < nlines) {
            w.hr[lb * H + k] = 0.5 * (zi + yi);
            w.hi[lb * H + k] = -0.5 * (zr - yr);
          }
        }
      }
    }
    outer_axes(w, -1);
    for (long q = 0; q < HV; ++q) out[q] = w.hr[q];
  }
  // x = brfft(g) of a real half spectrum g (HV values) into V reals
  void brfft(const double *g, double *x, Work &w) const {
    const int n = Ns;
    for (long q = 0; q < HV; ++q) {
      w.hr[q] = g[q];
      w.hi[q] = 0.0;
    }
    outer_axes(w, +1);
    for (long l0 = 0; l0 < nlines; l0 += 2 * B) {
      const long nb = std::min<long>(B, (nlines - l0 + 1) / 2);
      for (long b = 0; b < nb; ++b) {
        long la = l0 + 2 * b, lb = la + 1;
        for (int k = 0; k < n; ++k) {
          // Hermitian extension along the first axis; the imaginary parts at
          // k = 0 and at the Nyquist index do not enter a real result
          double pr, pi, qr = 0.0, qi = 0.0;
          const bool lower = k < H;
          const int kk = lower ? k : n - k;
          const bool selfconj = (kk == 0) || (2 * kk == n);
          pr = w.hr[la * H + kk];
          pi = selfconj ? 0.0 : (lower ? w.hi[la * H + kk] : -w.hi[la * H + kk]);
          if (lb < nlines) {
            qr = w.hr[lb * H + kk];
            qi = selfconj ? 0.0 : (lower ? w.hi[lb * H + kk] : -w.hi[lb * H + kk]);
          }
          w.br[(size_t)k * nb + b] = pr - qi;
          w.bi[(size_t)k * nb + b] = pi + qr;
        }
      }
      f.run(w.br.data(), w.bi.data(), w.wr.data(), w.wi.data(), nb, +1);
      for (int i = 0; i < n; ++i)
        for (long b = 0; b < nb; ++b) {
          long la = l0 + 2 * b, lb = la + 1;
          x[la * n + i] = w.br[(size_t)i * nb + b];
          if (lb < nlines) x[lb * n + i] = w.bi[(size_t)i * nb + b];
        }
    }
  }
};

struct FFTScratch {
  std::vector<cplx> a, b, tmp, lat, lat2;
  RealFFT3::Work rw;
  std::vector<double> h1, h2;          // half spectra of the sunset
  std::vector<double> g1, g2, g3, g4;  // lattice copies of orbit rows (ENGINE_ORBIT)
};

// ---------------------------------------------------------------------------
// Lattice and cubic orbits. Sites use Julia's column-major order
// (first coordinate fastest); momenta p_i = 2 pi n_i / Ns;
// lev2 = sum_i 4 sin^2(p_i / 2). An orbit is the set of sites reached by
// permutations and reflections of the coordinates; its label is the sorted
// folded coordinate triple (a <= b <= c, a_i = min(n_i, Ns - n_i)).
// FFTWhelper (Manifest.toml:352-358, not vendored) groups sites by lev2 value;
// the orbit is the exact symmetry class, and every CPUfull quantity the
// reference computes is independent of the grouping.
// ---------------------------------------------------------------------------
struct Orbits {
  int Ns = 1, sdim = 3, H = 1, S = 0;
  long V = 1;
  std::vector<int32_t> rep;      // 3 per orbit
  std::vector<double> k2;        // lev2 of the orbit
  std::vector<int64_t> deg;      // number of sites
  std::vector<int32_t> orbit_of_site;
  std::vector<long> rep_site;    // first site (column-major) of each orbit
  std::vector<long> site_start, site_list;  // sites of each orbit (CSR)

  static long tri_index(int sdim, int a, int b, int c) {
    if (sdim == 1) return c;
    if (sdim == 2) return (long)c * (c + 1) / 2 + b;
    return (long)c * (c + 1) * (c + 2) / 6 + (long)b * (b + 1) / 2 + a;
  }
  void build(int Ns_, int sdim_) {
    Ns = Ns_;
    sdim = sdim_;
    H = Ns / 2 + 1;
    V = 1;
    for (int d = 0; d < sdim; ++d) V *= Ns;
    long Smax = sdim == 1 ? H : (sdim == 2 ? (long)H * (H + 1) / 2 : (long)H * (H + 1) * (H + 2) / 6);
    S = (int)Smax;
    rep.assign((size_t)3 * S, 0);
    k2.assign(S, 0.0);
    deg.assign(S, 0);
    rep_site.assign(S, -1);
    orbit_of_site.assign(V, 0);
    for (long s = 0; s < V; ++s) {
      int n[3] = {0, 0, 0};
      long r = s;
      for (int d = 0; d < sdim; ++d) {
        n[d] = (int)(r % Ns);
        r /= Ns;
      }
      int f[3] = {0, 0, 0};
      for (int d = 0; d < sdim; ++d) f[d] = std::min(n[d], Ns - n[d]);
      // sort the active coordinates ascending; place them in the last slots
      int g[3] = {0, 0, 0};
      for (int d = 0; d < sdim; ++d) g[3 - sdim + d] = f[d];
      std::sort(g + 3 - sdim, g + 3);
      long o = tri_index(sdim, g[0], g[1], g[2]);
      orbit_of_site[s] = (int32_t)o;
      if (rep_site[o] < 0) {
        rep_site[o] = s;
        rep[3 * o + 0] = g[0];
        rep[3 * o + 1] = g[1];
        rep[3 * o + 2] = g[2];
        double kk = 0.0;
        for (int d = 0; d < sdim; ++d) {
          double sn = std::sin(M_PI * (double)g[3 - sdim + d] / (double)Ns);
          kk += 4.0 * sn * sn;
        }
        k2[o] = kk;
      }
      deg[o] += 1;
    }
    site_start.assign(S + 1, 0);
    for (int o = 0; o < S; ++o) site_start[o + 1] = site_start[o] + deg[o];
    site_list.assign(V, 0);
    std::vector<long> fill(site_start.begin(), site_start.end() - 1);
    for (long s = 0; s < V; ++s) site_list[fill[orbit_of_site[s]]++] = s;
  }
};

// Cosine matrix of the even octant: C[X][x] = m(x) cos(2 pi x X / Ns), with
// m(x) = 1 at x = 0 and at the Nyquist point, 2 elsewhere. For data that is
// even along an axis, the length-Ns DFT along it equals this H x H product.
static std::vector<double> octant_matrix(int Ns) {
  int H = Ns / 2 + 1;
  std::vector<double> C((size_t)H * H);
  for (int X = 0; X < H; ++X)
    for (int x = 0; x < H; ++x) {
      double m = (x == 0 || (Ns % 2 == 0 && 2 * x == Ns)) ? 1.0 : 2.0;
      C[(size_t)X * H + x] = m * std::cos(2.0 * M_PI * (double)((long)x * X % Ns) / (double)Ns);
    }
  return C;
}

// splitter (src/DefAbstractSimSetup.jl:7-10): xz = ceil.(range(0, n, length=k+1))
static std::vector<std::pair<int, int>> splitter(int idxmin, int n, int k) {
  std::vector<std::pair<int, int>> r;
  std::vector<long> xz(k + 1);
  for (int i = 0; i <= k; ++i) {
    double v = (k == 0) ? 0.0 : (double)n * (double)i / (double)k;
    xz[i] = (long)std::ceil(v - 1e-12 * std::max(1.0, std::fabs(v)));
  }
  for (int i = 0; i < k; ++i) r.push_back({(int)(xz[i] + idxmin), (int)(xz[i + 1] + idxmin - 1)});
  return r;
}

static void parallel_chunks(const std::vector<std::pair<int, int>> &ranges,
                            const std::function<void(int, int, int)> &body) {
  if (ranges.size() <= 1) {
    for (size_t c = 0; c < ranges.size(); ++c) body((int)c, ranges[c].first, ranges[c].second);
    return;
  }
  std::vector<std::thread> th;
  for (size_t c = 0; c < ranges.size(); ++c)
    th.emplace_back([&, c]() { body((int)c, ranges[c].first, ranges[c].second); });
  for (auto &t : th) t.join();
}

// ---------------------------------------------------------------------------
// The simulation state: SymMatrix F, r and CyclVector SigF, Sigr
// (src/DefSimDataElements.jl:88-230, TwoPIScalar_SimDataStruct.jl:63-89,204-247).
// ---------------------------------------------------------------------------
struct Oracle {
  orc_params p{};
  Orbits orb;
  int nv = 0;       // values per stored lattice (V or S)
  int M = 0;
  int tmin = 0, tmax = 0;  // simdata.indices
  std::vector<double> Fst, rst;      // M(M+1)/2 slots of nv values
  std::vector<double> SigF, Sigr;    // M slots of nv values
  std::vector<double> IrS, IFS;      // 1/N: M slots of I_rho, I_F (FULL: x-space lattice; else orbit momenta)
  std::vector<double> kL2, omega2;   // per stored value
  double hartreemass2 = 0.0;
  std::vector<double> Coct;          // octant cosine matrix
  std::vector<FFTPlan> plans;
  RealFFT3 rf;  // rfft / brfft of the sunset (FULL and ORBIT engines)
  std::vector<FFTScratch> scratch;
  std::vector<std::vector<double>> rhs;  // per chunk

  int mod1(int i) const { return ((i - 1) % M + M) % M + 1; }
  double thesign(int i, int j) const { return mod1(i) >= mod1(j) ? 1.0 : -1.0; }
  size_t pair_slot(int i, int j) const {
    int a = mod1(i) - 1, b = mod1(j) - 1;
    if (a < b) std::swap(a, b);
    return (size_t)a * (a + 1) / 2 + b;
  }
  void check(int i, int j) const {
    if (!(tmin <= i && i <= tmax) || !(tmin <= j && j <= tmax))
      throw std::out_of_range("Indices not in range!");
  }
  // raw slot values as stored (r carries the thesign of the slot order)
  double *Fp(int i, int j) {
    check(i, j);
    return Fst.data() + pair_slot(i, j) * nv;
  }
  double *rp(int i, int j) {
    check(i, j);
    return rst.data() + pair_slot(i, j) * nv;
  }
  double *sigFp(int z) {
    if (!(tmin <= z && z <= tmax)) throw std::out_of_range("Indices not in range!");
    return SigF.data() + (size_t)(mod1(z) - 1) * nv;
  }
  double *sigrp(int z) {
    if (!(tmin <= z && z <= tmax)) throw std::out_of_range("Indices not in range!");
    return Sigr.data() + (size_t)(mod1(z) - 1) * nv;
  }

  void setup(const orc_params &pp) {
    p = pp;
    if (p.sdim < 1 || p.sdim > 3 || p.Ns < 1 || p.M < 3 || p.N < 1 || p.pexp < 0 || p.pexp > ORC_PEXP_NINV_NLO)
      throw std::invalid_argument("bad parameters");
    if (p.nthreads < 1) p.nthreads = 1;
    orb.build(p.Ns, p.sdim);
    M = p.M;
    nv = (p.engine == ORC_ENGINE_FULL) ? (int)orb.V : orb.S;
    size_t npairs = (size_t)M * (M + 1) / 2;
    // createlattice returns ones (DefSimDataElements.jl:24-28)
    Fst.assign(npairs * nv, 1.0);
    rst.assign(npairs * nv, 1.0);
    SigF.assign((size_t)M * nv, 0.0);
    Sigr.assign((size_t)M * nv, 0.0);
    if (p.pexp == ORC_PEXP_NINV_NLO) {
      if (p.engine == ORC_ENGINE_ORBIT) throw std::invalid_argument("1/N NLO: FULL or OCTANT engine");
      if (p.sdim != 3) throw std::invalid_argument("1/N NLO: sdim 3");
      IrS.assign((size_t)M * nv, 0.0);
      IFS.assign((size_t)M * nv, 0.0);
    }
    kL2.assign(nv, 0.0);
    omega2.assign(nv, 0.0);
    // getTwoPISimData (TwoPIScalar_SimDataStruct.jl:669-687)
    for (int v = 0; v < nv; ++v) {
      int o = (p.engine == ORC_ENGINE_FULL) ? orb.orbit_of_site[v] : v;
      kL2[v] = orb.k2[o];
      omega2[v] = (orb.k2[o] + p.mass * p.mass) * (p.dt * p.dt);
    }
    Coct = octant_matrix(p.Ns);
    plans.clear();
    plans.emplace_back(p.Ns);
    rf.setup(p.Ns, p.sdim);
    scratch.resize(p.nthreads);
    for (auto &s : scratch) {
      if (p.engine != ORC_ENGINE_OCTANT) rf.alloc(s.rw);
      s.a.resize(p.Ns);
      s.b.resize(p.Ns);
      s.tmp.resize(64 * 64);
      s.lat.resize(orb.V);
      s.lat2.resize(orb.V);
    }
    rhs.assign(p.nthreads, std::vector<double>(nv));
  }

  // expandSimData! (TwoPIScalar_SimDataStruct.jl:262-278, DefSimDataElements.jl:141-165)
  void expand() {
    if (tmax + 1 > M) {
      tmin += 1;
      tmax += 1;
    } else {
      tmin = 1;
      tmax += 1;
    }
  }

  double hartree_prefactor() const {
    // Hartreeprefactor (TwoPIScalar_Initialization.jl:245-247): lambda/6 for the
    // 1/N expansion at LO, lambda (N+2)/(6N) otherwise
    if (p.pexp == ORC_PEXP_NINV_LO) return p.lambda * (1.0 / 6.0);
    return p.lambda * (double)(p.N + 2) / (double)(6 * p.N);
  }
  bool lo() const { return p.pexp == ORC_PEXP_LO || p.pexp == ORC_PEXP_NINV_LO; }
  double ivol() const { return 1.0 / (double)orb.V; }

  // getHartreeMass2 (TwoPIScalar_Initialization.jl:207-229)
  double hartree(int a, int b) {
    double h = 0.0;
    const double *F = Fp(a, b);
    if (p.engine == ORC_ENGINE_FULL) {
      // loop over shells and their sites: every site once
      for (int o = 0; o < orb.S; ++o)
        for (long q = orb.site_start[o]; q < orb.site_start[o + 1]; ++q) h += F[orb.site_list[q]];
    } else {
      for (int o = 0; o < orb.S; ++o) h += F[o] * (double)orb.deg[o];
    }
    h *= hartree_prefactor() * ivol();
    h += p.mass2;
    return h;
  }

  // --- 3D FFT on the full lattice, column-major --------------------------
  void fft_lattice(cplx *x, int sign, FFTScratch &sc) {
    const int Ns = p.Ns;
    const FFTPlan &pl = plans[0];
    long stride = 1;
    for (int d = 0; d < p.sdim; ++d) {
      long nlines = orb.V / Ns;
      for (long l = 0; l < nlines; ++l) {
        long lo = l % stride, hi = l / stride;
        long base = lo + hi * stride * Ns;
        pl.run(x + base, (int)stride, sign, sc.a, sc.b, sc.tmp);
      }
      stride *= Ns;
    }
  }
  // real(rfft(x)) followed by the Hermitian extension brfft applies to the
  // half spectrum: the values with first index above Ns/2 are those of -k.
  void real_half_spectrum(std::vector<cplx> &X) {
    const int Ns = p.Ns;
    for (long s = 0; s < orb.V; ++s) X[s] = cplx(X[s].real(), 0.0);
    for (long s = 0; s < orb.V; ++s) {
      int n[3] = {0, 0, 0};
      long r = s;
      for (int d = 0; d < p.sdim; ++d) {
        n[d] = (int)(r % Ns);
        r /= Ns;
      }
      if (n[0] <= Ns / 2) continue;
      long m = 0, mul = 1;
      for (int d = 0; d < p.sdim; ++d) {
        m += (long)((Ns - n[d]) % Ns) * mul;
        mul *= Ns;
      }
      X[s] = X[m];
    }
  }

  // One sunset on full lattices: Fin, rin (rin already times thesign).
  // calcSelfEnergyattp! CPUfull (TwoPIScalar_Evolution.jl:25-31): real parts of
  // the two rffts, pointwise products on the half spectrum, two brffts.
  void sunset_lattice(const double *Fin, const double *rin, double *sF, double *sr, FFTScratch &sc) {
    const long HV = rf.HV;
    sc.h1.resize(HV);
    sc.h2.resize(HV);
    rf.rfft_re(rin, sc.h1.data(), sc.rw);  // rx
    rf.rfft_re(Fin, sc.h2.data(), sc.rw);  // Fx
    const double iv = ivol();
    const double lam2 = p.lambda * p.lambda;
    const double N = (double)p.N;
    const double fr = iv * iv * iv * (-lam2 * (N + 2.0) / (6.0 * N * N));
    const double fF = iv * iv * iv * (-lam2 * (N + 2.0) / (18.0 * N * N));
    const bool classical = (p.pexp == ORC_PEXP_NLO_CLASSICAL);
    for (long s = 0; s < HV; ++s) {
      double rx = sc.h1[s], Fx = sc.h2[s];
      double gr = classical ? rx * (Fx * Fx) : rx * (Fx * Fx - (1 / 12.) * (rx * rx));
      double gF = classical ? Fx * (Fx * Fx) : Fx * (Fx * Fx - 0.75 * (rx * rx));
      sc.h1[s] = gr;
      sc.h2[s] = gF;
    }
    rf.brfft(sc.h1.data(), sr, sc.rw);
    rf.brfft(sc.h2.data(), sF, sc.rw);
    for (long s = 0; s < orb.V; ++s) {
      sr[s] *= fr;
      sF[s] *= fF;
    }
  }

  // Octant form of the same sunset on orbit rows (ENGINE_OCTANT).
  void octant_transform(std::vector<double> &a, std::vector<double> &tmp) {
    const int H = orb.H;
    long npt = 1;
    for (int d = 0; d < p.sdim; ++d) npt *= H;
    long stride = 1;
    for (int d = 0; d < p.sdim; ++d) {
      for (long q = 0; q < npt; ++q) {
        long xi = (q / stride) % H;
        long base = q - xi * stride;
        double s = 0.0;
        for (int x = 0; x < H; ++x) s += Coct[(size_t)xi * H + x] * a[base + (long)x * stride];
        tmp[q] = s;
      }
      std::swap(a, tmp);
      stride *= H;
    }
  }
  void sunset_octant(const double *Fin, const double *rin, double *sF, double *sr) {
    const int H = orb.H;
    long npt = 1;
    for (int d = 0; d < p.sdim; ++d) npt *= H;
    std::vector<double> fa(npt), ra(npt), tmp(npt);
    for (long q = 0; q < npt; ++q) {
      int g[3] = {0, 0, 0};
      long r = q;
      for (int d = 0; d < p.sdim; ++d) {
        g[3 - p.sdim + d] = (int)(r % H);
        r /= H;
      }
      std::sort(g + 3 - p.sdim, g + 3);
      long o = Orbits::tri_index(p.sdim, g[0], g[1], g[2]);
      fa[q] = Fin[o];
      ra[q] = rin[o];
    }
    octant_transform(fa, tmp);
    octant_transform(ra, tmp);
    const double iv = ivol();
    const double lam2 = p.lambda * p.lambda;
    const double N = (double)p.N;
    const double fr = iv * iv * iv * (-lam2 * (N + 2.0) / (6.0 * N * N));
    const double fF = iv * iv * iv * (-lam2 * (N + 2.0) / (18.0 * N * N));
    const bool classical = (p.pexp == ORC_PEXP_NLO_CLASSICAL);
    for (long q = 0; q < npt; ++q) {
      double rx = ra[q], Fx = fa[q];
      ra[q] = classical ? rx * (Fx * Fx) : rx * (Fx * Fx - (1 / 12.) * (rx * rx));
      fa[q] = classical ? Fx * (Fx * Fx) : Fx * (Fx * Fx - 0.75 * (rx * rx));
    }
    octant_transform(fa, tmp);
    octant_transform(ra, tmp);
    for (int o = 0; o < orb.S; ++o) {
      long q = 0, mul = 1;
      for (int d = 0; d < p.sdim; ++d) {
        q += (long)orb.rep[3 * o + 3 - p.sdim + d] * mul;
        mul *= H;
      }
      sr[o] = fr * ra[q];
      sF[o] = fF * fa[q];
    }
  }

  void sunset_rows(const double *F, const double *r, double *sF, double *sr, FFTScratch &sc) {
    if (p.engine == ORC_ENGINE_FULL) {
      sunset_lattice(F, r, sF, sr, sc);
    } else if (p.engine == ORC_ENGINE_ORBIT) {
      // copytolattice! -> FFT sunset -> copytoreducedlattice!
      // (TwoPIScalar_Evolution.jl:91-105, DefSimDataElements.jl:71-83)
      std::vector<double> &Fl = sc.g1, &rl = sc.g2, &sFl = sc.g3, &srl = sc.g4;
      Fl.resize(orb.V);
      rl.resize(orb.V);
      sFl.resize(orb.V);
      srl.resize(orb.V);
      for (long s = 0; s < orb.V; ++s) {
        Fl[s] = F[orb.orbit_of_site[s]];
        rl[s] = r[orb.orbit_of_site[s]];
      }
      sunset_lattice(Fl.data(), rl.data(), sFl.data(), srl.data(), sc);
      for (int o = 0; o < orb.S; ++o) {
        sF[o] = sFl[orb.rep_site[o]];
        sr[o] = srl[orb.rep_site[o]];
      }
    } else {
      sunset_octant(F, r, sF, sr);
    }
  }

  // ------------------------------------------------------------------------
  // 1/N expansion at NLO (TwoPIScalar_Evolution.jl:144-758)
  // ------------------------------------------------------------------------
  double *Irp(int z) { return IrS.data() + (size_t)(mod1(z) - 1) * nv; }
  double *IFp(int z) { return IFS.data() + (size_t)(mod1(z) - 1) * nv; }
  // rfft of a real even lattice, real part with the half-spectrum extension
  void Kf(const double *in, double *out, FFTScratch &sc) {
    std::vector<cplx> &X = sc.lat;
    for (long q = 0; q < orb.V; ++q) X[q] = cplx(in[q], 0.0);
    fft_lattice(X.data(), -1, sc);
    real_half_spectrum(X);
    for (long q = 0; q < orb.V; ++q) out[q] = X[q].real();
  }
  // brfft of a real half spectrum (stored extended on the full lattice)
  void Kb(const double *in, double *out, FFTScratch &sc) {
    std::vector<cplx> &X = sc.lat;
    for (long q = 0; q < orb.V; ++q) X[q] = cplx(in[q], 0.0);
    fft_lattice(X.data(), +1, sc);
    for (long q = 0; q < orb.V; ++q) out[q] = X[q].real();
  }
  // CPUfull: calcIrs! (:170-206), calcIFs! (:354-436), calcSelfEnergyattp! (:683-698)
  void ninv_full(int tmone) {
    FFTScratch &sc = scratch[0];
    const long V = orb.V;
    const double iv = ivol(), lam = p.lambda, dt = p.dt, N = (double)p.N;
    std::vector<double> Fx(V), rx(V), A(V), B(V), R2(V), R3(V), RHS(V), T(V);
    {  // calcIrs!
      double *I0 = Irp(tmone);
      for (long q = 0; q < V; ++q) I0[q] = 0.0;
      const double f1 = (lam / 3.) * iv * iv, f2 = dt * (lam / 3.) * iv, f3 = iv * iv;
      for (int tp = tmone - 1; tp >= tmin; --tp) {
        Kf(Fp(tmone, tp), Fx.data(), sc);
        Kf(rp(tmone, tp), rx.data(), sc);
        const double s = thesign(tmone, tp);
        double *I = Irp(tp);
        for (long q = 0; q < V; ++q) I[q] = s * f1 * Fx[q] * rx[q];
        for (long q = 0; q < V; ++q) RHS[q] = 0.0;
        for (int z = tp + 1; z <= tmone - 1; ++z) {
          Kf(Fp(z, tp), A.data(), sc);
          Kf(rp(z, tp), B.data(), sc);
          const double sz = thesign(z, tp);
          for (long q = 0; q < V; ++q) T[q] = A[q] * B[q];
          Kb(T.data(), R2.data(), sc);
          Kb(Irp(z), R3.data(), sc);
          for (long q = 0; q < V; ++q) RHS[q] -= f3 * sz * R2[q] * R3[q];
        }
        Kf(RHS.data(), T.data(), sc);
        for (long q = 0; q < V; ++q) I[q] += f2 * T[q];
      }
    }
    {  // calcIFs!
      const double f1 = lam / 6. * iv * iv, f2 = lam / 6. * dt, f3 = lam / 3. * dt;
      for (int tp = tmin; tp <= tmone; ++tp) {
        Kf(Fp(tmone, tp), Fx.data(), sc);
        Kf(rp(tmone, tp), rx.data(), sc);
        double *IF = IFp(tp);
        for (long q = 0; q < V; ++q) IF[q] = f1 * (Fx[q] * Fx[q] - 0.25 * rx[q] * rx[q]);
        for (long q = 0; q < V; ++q) RHS[q] = 0.0;
        for (int z = tmin + 1; z <= tp - 1; ++z) {  // first integral
          Kf(Fp(z, tp), A.data(), sc);
          Kf(rp(z, tp), B.data(), sc);
          for (long q = 0; q < V; ++q) {
            A[q] *= iv;
            B[q] *= iv;
          }
          Kb(Irp(z), R3.data(), sc);
          for (long q = 0; q < V; ++q) T[q] = A[q] * A[q] - 0.25 * B[q] * B[q];
          Kb(T.data(), R2.data(), sc);
          for (long q = 0; q < V; ++q) RHS[q] -= f2 * R3[q] * R2[q];  // nr 1
          for (long q = 0; q < V; ++q) T[q] = A[q] * B[q];
          const double sz = thesign(z, tp);
          Kb(T.data(), R3.data(), sc);
          Kb(IFp(z), R2.data(), sc);
          for (long q = 0; q < V; ++q) RHS[q] += f3 * sz * R2[q] * R3[q];  // nr 2
        }
        const int beginning = (tp == tmin) ? tmin + 1 : tp;
        for (int z = beginning; z <= tmone - 1; ++z) {  // second integral
          Kf(Fp(z, tp), A.data(), sc);
          Kf(rp(z, tp), B.data(), sc);
          for (long q = 0; q < V; ++q) {
            A[q] *= iv;
            B[q] *= iv;
          }
          for (long q = 0; q < V; ++q) T[q] = A[q] * A[q] - 0.25 * B[q] * B[q];
          Kb(T.data(), R3.data(), sc);
          Kb(Irp(z), R2.data(), sc);
          for (long q = 0; q < V; ++q) RHS[q] -= f2 * R2[q] * R3[q];
        }
        {  // border part
          Kf(Fp(tmin, tp), A.data(), sc);
          Kf(rp(tmin, tp), B.data(), sc);
          for (long q = 0; q < V; ++q) T[q] = A[q] * A[q] - 0.25 * B[q] * B[q];
          Kb(T.data(), R3.data(), sc);
          for (long q = 0; q < V; ++q) R3[q] *= iv * iv;
          Kb(Irp(tmin), R2.data(), sc);
          for (long q = 0; q < V; ++q) RHS[q] -= 0.5 * dt * lam / 6. * R2[q] * R3[q];
          if (tp > tmin) {
            const double sz = thesign(tmin, tp);
            for (long q = 0; q < V; ++q) T[q] = sz * A[q] * B[q];
            Kb(T.data(), R3.data(), sc);
            Kb(IFp(tmin), R2.data(), sc);
            for (long q = 0; q < V; ++q) RHS[q] += 0.5 * dt * lam / 3. * iv * iv * R2[q] * R3[q];
          }
        }
        Kf(RHS.data(), T.data(), sc);
        for (long q = 0; q < V; ++q) IF[q] += iv * T[q];
      }
    }
    // calcSelfEnergyattp! for every t' of the window
    const double fac = -lam / (3. * N) * iv;
    for (int tp = tmin; tp <= tmone; ++tp) {
      Kf(Fp(tmone, tp), Fx.data(), sc);
      Kf(rp(tmone, tp), rx.data(), sc);
      const double s = thesign(tmone, tp);
      for (long q = 0; q < V; ++q) rx[q] *= s;
      const double *I = Irp(tp), *IF = IFp(tp);
      for (long q = 0; q < V; ++q) T[q] = Fx[q] * I[q] + rx[q] * IF[q];
      Kb(T.data(), sigrp(tp), sc);
      for (long q = 0; q < V; ++q) sigrp(tp)[q] *= fac;
      for (long q = 0; q < V; ++q) T[q] = Fx[q] * IF[q] - 0.25 * rx[q] * I[q];
      Kb(T.data(), sigFp(tp), sc);
      for (long q = 0; q < V; ++q) sigFp(tp)[q] *= fac;
    }
  }
  // Orbit form: the resummed kernels are diagonal in momentum, so with the orbit
  // cosine transform A (A A = V) and the bubbles
  //   Pr(a,b) = ivol^2 A[A F(a,b) . A rho(a,b)],  PF(a,b) = ivol^2 A[(A F)^2 - (A rho)^2 / 4]
  // the momentum-space kernels I_k = A I_rho^x, J_k = A I_F^x obey
  //   I_k(t') = lam/3 Pr(t-1,t') - dt lam/3 sum_{z=t'+1}^{t-2} I_k(z) Pr(z,t')
  //   J_k(t') = lam/6 PF(t-1,t') - sum_{z=tmin}^{t-2} w_z lam/6 I_k(z) PF(z,t')
  //                             + sum_{z=tmin}^{t'-1} w_z lam/3 J_k(z) Pr(z,t')
  // (w = dt/2 at tmin, dt otherwise) and
  //   Sigma_rho = -lam/(3N) ivol^2 A[A F . A I_k + A rho . A J_k]
  //   Sigma_F   = -lam/(3N) ivol^2 A[A F . A J_k - A rho . A I_k / 4]
  void A_orbit(const double *in, double *out) {
    const int H = orb.H;
    const long npt = (long)H * H * H;
    std::vector<double> a(npt), tmp(npt);
    for (long q = 0; q < npt; ++q) {
      int g[3] = {(int)(q % H), (int)((q / H) % H), (int)(q / ((long)H * H))};
      std::sort(g, g + 3);
      a[q] = in[Orbits::tri_index(3, g[0], g[1], g[2])];
    }
    octant_transform(a, tmp);
    for (int o = 0; o < orb.S; ++o)
      out[o] = a[(long)orb.rep[3 * o] + (long)orb.rep[3 * o + 1] * H + (long)orb.rep[3 * o + 2] * H * H];
  }
  void bubbles(int a, int b, double *Pr, double *PF) {
    const int S = orb.S;
    const double iv = ivol();
    std::vector<double> Fx(S), rx(S), g(S), rt(S);
    const double s = thesign(a, b);
    for (int o = 0; o < S; ++o) rt[o] = rp(a, b)[o] * s;  // the true rho(a, b)
    A_orbit(Fp(a, b), Fx.data());
    A_orbit(rt.data(), rx.data());
    if (Pr) {
      for (int o = 0; o < S; ++o) g[o] = Fx[o] * rx[o];
      A_orbit(g.data(), Pr);
      for (int o = 0; o < S; ++o) Pr[o] *= iv * iv;
    }
    if (PF) {
      for (int o = 0; o < S; ++o) g[o] = Fx[o] * Fx[o] - 0.25 * rx[o] * rx[o];
      A_orbit(g.data(), PF);
      for (int o = 0; o < S; ++o) PF[o] *= iv * iv;
    }
  }
  void ninv_octant(int tmone) {
    const int S = orb.S;
    const double iv = ivol(), lam = p.lambda, dt = p.dt, N = (double)p.N;
    std::vector<double> Pr(S), PF(S), acc(S);
    for (int o = 0; o < S; ++o) Irp(tmone)[o] = 0.0;
    for (int tp = tmone - 1; tp >= tmin; --tp) {
      for (int o = 0; o < S; ++o) acc[o] = 0.0;
      for (int z = tp + 1; z <= tmone - 1; ++z) {
        bubbles(z, tp, Pr.data(), nullptr);
        for (int o = 0; o < S; ++o) acc[o] += Irp(z)[o] * Pr[o];
      }
      bubbles(tmone, tp, Pr.data(), nullptr);
      for (int o = 0; o < S; ++o) Irp(tp)[o] = lam / 3. * Pr[o] - dt * lam / 3. * acc[o];
    }
    for (int tp = tmin; tp <= tmone; ++tp) {
      std::vector<double> a1(S, 0.0), a2(S, 0.0);
      for (int z = tmin; z <= tmone - 1; ++z) {
        const double w = (z == tmin) ? 0.5 * dt : dt;
        bubbles(z, tp, nullptr, PF.data());
        for (int o = 0; o < S; ++o) a1[o] += w * Irp(z)[o] * PF[o];
      }
      for (int z = tmin; z <= tp - 1; ++z) {
        const double w = (z == tmin) ? 0.5 * dt : dt;
        bubbles(z, tp, Pr.data(), nullptr);
        for (int o = 0; o < S; ++o) a2[o] += w * IFp(z)[o] * Pr[o];
      }
      bubbles(tmone, tp, nullptr, PF.data());
      for (int o = 0; o < S; ++o) IFp(tp)[o] = lam / 6. * PF[o] - lam / 6. * a1[o] + lam / 3. * a2[o];
    }
    const double fac = -lam / (3. * N) * iv * iv;
    std::vector<double> Fx(S), rx(S), Ix(S), Jx(S), g(S), rt(S);
    for (int tp = tmin; tp <= tmone; ++tp) {
      const double s = thesign(tmone, tp);
      for (int o = 0; o < S; ++o) rt[o] = rp(tmone, tp)[o] * s;
      A_orbit(Fp(tmone, tp), Fx.data());
      A_orbit(rt.data(), rx.data());
      A_orbit(Irp(tp), Ix.data());
      A_orbit(IFp(tp), Jx.data());
      for (int o = 0; o < S; ++o) g[o] = Fx[o] * Ix[o] + rx[o] * Jx[o];
      A_orbit(g.data(), sigrp(tp));
      for (int o = 0; o < S; ++o) sigrp(tp)[o] *= fac;
      for (int o = 0; o < S; ++o) g[o] = Fx[o] * Jx[o] - 0.25 * rx[o] * Ix[o];
      A_orbit(g.data(), sigFp(tp));
      for (int o = 0; o < S; ++o) sigFp(tp)[o] *= fac;
    }
  }

  // calcSelfEnergyattp! (TwoPIScalar_Evolution.jl:25-31 / 91-105)
  void self_energy_at(int tmone, int tp, int ichunk) {
    std::vector<double> rs(nv);
    const double s = thesign(tmone, tp);
    const double *r = rp(tmone, tp);
    for (int v = 0; v < nv; ++v) rs[v] = r[v] * s;
    sunset_rows(Fp(tmone, tp), rs.data(), sigFp(tp), sigrp(tp), scratch[ichunk]);
  }

  // calcSelfEnergies! (TwoPIScalar_Evolution.jl:8-23)
  void self_energies(int tmone) {
    if (lo()) return;  // LO: no self-energy (:8-11)
    if (p.pexp == ORC_PEXP_NINV_NLO) {
      if (p.engine == ORC_ENGINE_FULL) ninv_full(tmone);
      else ninv_octant(tmone);
      return;
    }
    int n = (tmax - 1) - tmin + 1;
    auto ranges = splitter(tmin, n, p.nthreads);
    parallel_chunks(ranges, [&](int c, int lo, int hi) {
      for (int tp = lo; tp <= hi; ++tp) self_energy_at(tmone, tp, c);
    });
  }

  // getRHS_r! (TwoPIScalar_Evolution.jl:846-865); LO: zero (:842-844)
  void rhs_r(double *Mem, int t, int tp) {
    for (int v = 0; v < nv; ++v) Mem[v] = 0.0;
    if (lo()) return;
    for (int z = tp + 1; z <= t - 2; ++z) {
      const double *S = sigrp(z), *r = rp(z, tp);
      const double s = thesign(z, tp);
      for (int v = 0; v < nv; ++v) Mem[v] -= S[v] * r[v] * s;
    }
  }
  // getRHS_F! (TwoPIScalar_Evolution.jl:766-801); LO: zero (:763-765)
  void rhs_F(double *Mem, int t, int tp) {
    if (lo()) {
      for (int v = 0; v < nv; ++v) Mem[v] = 0.0;
      return;
    }
    const int tpmin = tmin;
    {
      const double *S = sigrp(tpmin), *F = Fp(tpmin, tp);
      for (int v = 0; v < nv; ++v) Mem[v] = S[v] * F[v];
      for (int v = 0; v < nv; ++v) Mem[v] *= -0.5;
    }
    for (int z = tpmin + 1; z <= t - 2; ++z) {
      const double *S = sigrp(z), *F = Fp(z, tp);
      for (int v = 0; v < nv; ++v) Mem[v] -= S[v] * F[v];
    }
    {
      const double *S = sigFp(tpmin), *r = rp(tpmin, tp);
      const double s = thesign(tpmin, tp);
      for (int v = 0; v < nv; ++v) Mem[v] += 0.5 * S[v] * r[v] * s;
    }
    for (int z = tpmin + 1; z <= tp - 1; ++z) {
      const double *S = sigFp(z), *r = rp(z, tp);
      const double s = thesign(z, tp);
      for (int v = 0; v < nv; ++v) Mem[v] += S[v] * r[v] * s;
    }
  }
  // evolve_r! (TwoPIScalar_Evolution.jl:890-905)
  void evolve_r(double *RHS, int t, int tp) {
    double *out = rp(t, tp);
    const double st = thesign(t, tp);
    if (tp == t - 1) {
      for (int v = 0; v < nv; ++v) out[v] = st * p.dt;
    } else if (tp == t) {
      for (int v = 0; v < nv; ++v) out[v] = 0.0;
    } else {
      const double dt3 = p.dt * p.dt * p.dt;
      for (int v = 0; v < nv; ++v) RHS[v] *= dt3;
      const double *r1 = rp(t - 1, tp), *r2 = rp(t - 2, tp);
      const double s1 = thesign(t - 1, tp), s2 = thesign(t - 2, tp);
      for (int v = 0; v < nv; ++v) out[v] = (2 - omega2[v]) * r1[v] * s1 - r2[v] * s2 + RHS[v];
      for (int v = 0; v < nv; ++v) out[v] *= st;
    }
  }
  // evolve_F! (TwoPIScalar_Evolution.jl:908-915)
  void evolve_F(double *RHS, int t, int tp) {
    const double dt3 = p.dt * p.dt * p.dt;
    for (int v = 0; v < nv; ++v) RHS[v] *= dt3;
    double *out = Fp(t, tp);
    const double *F1 = Fp(t - 1, tp), *F2 = Fp(t - 2, tp);
    for (int v = 0; v < nv; ++v) out[v] = (2 - omega2[v]) * F1[v] - F2[v] + RHS[v];
  }
  // setomega2values! (TwoPIScalar_Evolution.jl:918-921)
  void set_omega2() {
    for (int v = 0; v < nv; ++v) omega2[v] = kL2[v] + hartreemass2;
    for (int v = 0; v < nv; ++v) omega2[v] *= p.dt * p.dt;
  }

  // evolve! (TwoPIScalar_Evolution.jl:924-981)
  double last_t_sunset = 0.0, last_t_rest = 0.0;  // seconds of the last evolve!

  void evolve(int t) {
    auto c0 = std::chrono::steady_clock::now();
    expand();
    if (tmax != t) throw std::invalid_argument("evolve! must be called with t = lastEvolStep + 1");
    self_energies(t - 1);
    auto c1 = std::chrono::steady_clock::now();
    hartreemass2 = hartree(t - 1, t - 1);
    set_omega2();
    int n = (tmax - 1) - tmin + 1;
    auto ranges = splitter(tmin, n, p.nthreads);
    parallel_chunks(ranges, [&](int c, int lo, int hi) {
      double *R = rhs[c].data();
      for (int tp = lo; tp <= hi; ++tp) {
        rhs_r(R, t, tp);
        evolve_r(R, t, tp);
        rhs_F(R, t, tp);
        evolve_F(R, t, tp);
      }
    });
    double *R = rhs[0].data();
    evolve_r(R, t, t);
    rhs_F(R, t, t);
    evolve_F(R, t, t);
    auto c2 = std::chrono::steady_clock::now();
    last_t_sunset = std::chrono::duration<double>(c1 - c0).count();
    last_t_rest = std::chrono::duration<double>(c2 - c1).count();
  }

  // initSimData! (TwoPIScalar_Initialization.jl:8-47)
  void init_occupation(const double *n, double initmass) {
    expand();
    expand();
    for (int v = 0; v < nv; ++v) {
      int o = (p.engine == ORC_ENGINE_FULL) ? orb.orbit_of_site[v] : v;
      double omega = std::sqrt(orb.k2[o] + initmass * initmass);
      Fp(1, 1)[v] = (1 / omega) * (n[o] + 0.5);
      Fp(2, 1)[v] = (1 / omega) * (n[o] + 0.5);
      Fp(2, 2)[v] = (omega * (n[o] + 0.5) * (p.dt * p.dt) + (1 / omega) * (n[o] + 0.5));
      rp(1, 1)[v] = 0.0;
      rp(2, 1)[v] = p.dt * thesign(2, 1);
      rp(2, 2)[v] = 0.0;
    }
    hartreemass2 = hartree(2, 2);
  }
  // initSimData! for the Gauss state (TwoPIScalar_Initialization.jl:95-112)
  void init_gauss(double xi, double eta, double sig) {
    expand();
    expand();
    for (int v = 0; v < nv; ++v) {
      Fp(1, 1)[v] = xi * xi;
      Fp(2, 1)[v] = xi * eta * p.dt + Fp(1, 1)[v];
      Fp(2, 2)[v] = (eta * eta + sig * sig / (4 * xi * xi)) * (p.dt * p.dt) - Fp(1, 1)[v] + 2 * Fp(2, 1)[v];
      rp(1, 1)[v] = 0.0;
      rp(2, 1)[v] = p.dt * thesign(2, 1);
      rp(2, 2)[v] = 0.0;
    }
    hartreemass2 = hartree(2, 2);
  }

  int meas_idx(int o) const { return (p.engine == ORC_ENGINE_FULL) ? (int)orb.rep_site[o] : o; }

  // createMeasurement (TwoPIScalar_Measurement.jl:31-99, 135-197)
  void measure(int t, orc_scalars *sc, double *oF, double *oddF, double *on, double *oomega,
               double *oc, double *Fonet, double *ronet, double *osigF, double *osigr) {
    const double dt = p.dt;
    std::vector<double> ddF(orb.S), Fm(orb.S), om(orb.S), cc(orb.S), nn(orb.S);
    const double *Ftt = Fp(t, t), *Fmt = Fp(t - 1, t), *Fmm = Fp(t - 1, t - 1);
    for (int i = 0; i < orb.S; ++i) {
      int idx = meas_idx(i);
      ddF[i] = (Ftt[idx] - 2 * Fmt[idx] + Fmm[idx]) / (dt * dt);
      Fm[i] = Fmm[idx];
      om[i] = (ddF[i] / Fmm[idx] > 0) ? std::sqrt(ddF[i] / Fmm[idx]) : 0.0;
      cc[i] = (0.25 * (dt * dt) * (om[i] * om[i]) < 1) ? std::sqrt(1. - 0.25 * (dt * dt) * (om[i] * om[i])) : 1.0;
      nn[i] = (ddF[i] * Fmm[idx] > 0) ? (cc[i] * std::sqrt(ddF[i] * Fmm[idx])) - 0.5 : 0.0;
    }
    double E_kin = 0.0, E_pot = 0.0, E_mem = 0.0, hc = 0.0;
    for (int i = 0; i < orb.S; ++i) E_kin += 0.5 * ddF[i] * (double)orb.deg[i];
    for (int i = 0; i < orb.S; ++i) hc += Fm[i] * (double)orb.deg[i];
    for (int i = 0; i < orb.S; ++i)
      E_pot += 0.5 * (p.mass2 + orb.k2[i] + 0.5 * ivol() * hartree_prefactor() * hc) * Fm[i] * (double)orb.deg[i];
    if (t != 2) {
      const int tp0 = tmin;
      if (p.engine == ORC_ENGINE_FULL) {
        const double *S1 = sigrp(tp0), *F = Fp(tp0, t - 1), *S2 = sigFp(tp0), *r = rp(tp0, t - 1);
        const double s = thesign(tp0, t - 1);
        double acc = 0.0;
        for (int v = 0; v < nv; ++v) acc += S1[v] * F[v] - S2[v] * r[v] * s;
        E_mem = 0.5 * 0.25 * dt * acc;
        if (t > 3) {
          double tot = 0.0;
          for (int tp = tp0 + 1; tp <= t - 2; ++tp) {
            const double *A = sigrp(tp), *B = Fp(tp, t - 1), *C = sigFp(tp), *D = rp(tp, t - 1);
            const double st = thesign(tp, t - 1);
            double a = 0.0;
            for (int v = 0; v < nv; ++v) a += A[v] * B[v] - C[v] * D[v] * st;
            tot += a;
          }
          E_mem += 0.25 * dt * tot;
        }
      } else {
        const double *S1 = sigrp(tp0), *F = Fp(tp0, t - 1), *S2 = sigFp(tp0), *r = rp(tp0, t - 1);
        const double s = thesign(tp0, t - 1);
        for (int i = 0; i < orb.S; ++i)
          E_mem += 0.5 * 0.25 * dt * (double)orb.deg[i] * (S1[i] * F[i] - S2[i] * r[i] * s);
        if (t > 3) {
          for (int i = 0; i < orb.S; ++i)
            for (int tp = tp0 + 1; tp <= t - 2; ++tp) {
              const double st = thesign(tp, t - 1);
              E_mem += 0.25 * dt * (double)orb.deg[i] *
                       (sigrp(tp)[i] * Fp(tp, t - 1)[i] - sigFp(tp)[i] * rp(tp, t - 1)[i] * st);
            }
        }
      }
    }
    sc->time = (t - 1) * dt * p.mass;
    sc->M2 = hartreemass2;
    sc->E_kin = E_kin;
    sc->E_pot = E_pot;
    sc->E_mem = E_mem;
    sc->E = E_kin + E_pot + E_mem;
    for (int i = 0; i < orb.S; ++i) {
      if (oF) oF[i] = Fm[i];
      if (oddF) oddF[i] = ddF[i];
      if (on) on[i] = nn[i];
      if (oomega) oomega[i] = om[i];
      if (oc) oc[i] = cc[i];
    }
    // traces at site 1 (Measurement.jl:89-96)
    int k = 0;
    if (osigF || osigr)
      for (int tp = tmax - 1; tp >= tmin; --tp, ++k) {
        if (osigF) osigF[k] = sigFp(tp)[0];
        if (osigr) osigr[k] = sigrp(tp)[0];
      }
    k = 0;
    if (Fonet || ronet)
      for (int tp = tmin; tp <= tmax - 1; ++tp, ++k) {
        if (Fonet) Fonet[k] = Fp(tmin, tp)[0];
        if (ronet) ronet[k] = rp(tmin, tp)[0] * thesign(tmin, tp);
      }
  }

  // getGapMass (TwoPIScalar_Initialization.jl:250-266); Newton's method on
  // the gap equation with its analytic derivative.
  double gap_mass(const double *n, double x0) {
    auto g = [&](double x, double *dg) {
      double res = 0.0, dres = 0.0;
      for (int i = 0; i < orb.S; ++i) {
        double w2 = orb.k2[i] + x * x;
        res += (1 / std::sqrt(w2)) * (n[i] + 0.5) * (double)orb.deg[i];
        dres += -x / (w2 * std::sqrt(w2)) * (n[i] + 0.5) * (double)orb.deg[i];
      }
      *dg = dres * ivol() * hartree_prefactor() - 2 * x;
      return res * ivol() * hartree_prefactor() + p.mass2 - x * x;
    };
    double x = x0;
    for (int it = 0; it < 200; ++it) {
      double d;
      double f = g(x, &d);
      if (f == 0.0) break;
      double xn = x - f / d;
      if (std::fabs(xn - x) <= 4 * 2.220446049250313e-16 * std::fabs(xn)) {
        x = xn;
        break;
      }
      x = xn;
    }
    return x;
  }
};

// ---------------------------------------------------------------------------
// Forward-mode derivatives (the stand-in for ForwardDiff through the reference,
// which cannot run here): dual numbers carrying K directional derivatives
// through a templated restatement of the orbit/octant engine above -- the same
// ring (mod1 slots, thesign), the same evolve! order of operations, the same
// octant sunset and createMeasurement -- single-threaded, orbit values only.
// ---------------------------------------------------------------------------
template <int K>
struct Dual {
  double v = 0.0;
  double d[K] = {};
  Dual() = default;
  Dual(double x) : v(x) {}  // NOLINT: constants promote to duals
  friend Dual operator+(const Dual &a, const Dual &b) {
    Dual r(a.v + b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
  }
  friend Dual operator-(const Dual &a, const Dual &b) {
    Dual r(a.v - b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
  }
  friend Dual operator-(const Dual &a) {
    Dual r(-a.v);
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
  }
  friend Dual operator*(const Dual &a, const Dual &b) {
    Dual r(a.v * b.v);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
  }
  friend Dual operator/(const Dual &a, const Dual &b) {
    Dual r(a.v / b.v);
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
    return r;
  }
  Dual &operator+=(const Dual &b) { return *this = *this + b; }
  Dual &operator-=(const Dual &b) { return *this = *this - b; }
  Dual &operator*=(const Dual &b) { return *this = *this * b; }
};
template <int K>
Dual<K> dsqrt(const Dual<K> &a) {
  Dual<K> r(std::sqrt(a.v));
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] / (2.0 * r.v);
  return r;
}
inline double val(double x) { return x; }
template <int K>
double val(const Dual<K> &x) {
  return x.v;
}

template <class T>
struct DualEngine {
  orc_params p{};
  Orbits orb;
  int S = 0, M = 0, tmin = 0, tmax = 0;
  T lam, mass2;
  std::vector<std::vector<T>> Fst, rst, SigF, Sigr;
  std::vector<T> omega2;
  T hm2;
  std::vector<double> Coct;

  int mod1(int i) const { return ((i - 1) % M + M) % M + 1; }
  double thesign(int i, int j) const { return mod1(i) >= mod1(j) ? 1.0 : -1.0; }
  size_t slot(int i, int j) const {
    int a = mod1(i) - 1, b = mod1(j) - 1;
    if (a < b) std::swap(a, b);
    return (size_t)a * (a + 1) / 2 + b;
  }
  std::vector<T> &F(int i, int j) { return Fst[slot(i, j)]; }
  std::vector<T> &r(int i, int j) { return rst[slot(i, j)]; }
  std::vector<T> &sF(int z) { return SigF[mod1(z) - 1]; }
  std::vector<T> &sr(int z) { return Sigr[mod1(z) - 1]; }

  void setup(const orc_params &pp, T lam_, T mass2_) {
    p = pp;
    orb.build(p.Ns, 3);
    S = orb.S;
    M = p.M;
    lam = lam_;
    mass2 = mass2_;
    Fst.assign((size_t)M * (M + 1) / 2, std::vector<T>(S, T(1.0)));
    rst.assign((size_t)M * (M + 1) / 2, std::vector<T>(S, T(1.0)));
    SigF.assign(M, std::vector<T>(S, T(0.0)));
    Sigr.assign(M, std::vector<T>(S, T(0.0)));
    omega2.assign(S, T(0.0));
    Coct = octant_matrix(p.Ns);
  }
  void expand() {
    if (tmax + 1 > M) {
      tmin += 1;
      tmax += 1;
    } else {
      tmin = 1;
      tmax += 1;
    }
  }
  T pref() const { return lam * T((double)(p.N + 2) / (double)(6 * p.N)); }
  double ivol() const { return 1.0 / (double)orb.V; }
  T hartree(int a, int b) {
    T h(0.0);
    const std::vector<T> &f = F(a, b);
    for (int o = 0; o < S; ++o) h += f[o] * T((double)orb.deg[o]);
    return h * (pref() * T(ivol())) + mass2;
  }
  void octant(std::vector<T> &a, std::vector<T> &tmp) {
    const int H = orb.H;
    const long npt = (long)H * H * H;
    long stride = 1;
    for (int d = 0; d < 3; ++d) {
      for (long q = 0; q < npt; ++q) {
        const long xi = (q / stride) % H, base = q - xi * stride;
        T acc(0.0);
        for (int x = 0; x < H; ++x) acc += T(Coct[(size_t)xi * H + x]) * a[base + (long)x * stride];
        tmp[q] = acc;
      }
      std::swap(a, tmp);
      stride *= H;
    }
  }
  void sunset(const std::vector<T> &Fin, const std::vector<T> &rin, std::vector<T> &oF, std::vector<T> &orr) {
    const int H = orb.H;
    const long npt = (long)H * H * H;
    std::vector<T> fa(npt), ra(npt), tmp(npt);
    for (long q = 0; q < npt; ++q) {
      int g[3] = {(int)(q % H), (int)((q / H) % H), (int)(q / ((long)H * H))};
      std::sort(g, g + 3);
      const long o = Orbits::tri_index(3, g[0], g[1], g[2]);
      fa[q] = Fin[o];
      ra[q] = rin[o];
    }
    octant(fa, tmp);
    octant(ra, tmp);
    const double iv = ivol(), Nn = (double)p.N;
    const T lam2 = lam * lam;
    const T fr = T(iv * iv * iv) * (-lam2 * T((Nn + 2.0) / (6.0 * Nn * Nn)));
    const T fF = T(iv * iv * iv) * (-lam2 * T((Nn + 2.0) / (18.0 * Nn * Nn)));
    const bool classical = (p.pexp == ORC_PEXP_NLO_CLASSICAL);
    for (long q = 0; q < npt; ++q) {
      const T rx = ra[q], Fx = fa[q];
      ra[q] = classical ? rx * (Fx * Fx) : rx * (Fx * Fx - T(1 / 12.) * (rx * rx));
      fa[q] = classical ? Fx * (Fx * Fx) : Fx * (Fx * Fx - T(0.75) * (rx * rx));
    }
    octant(fa, tmp);
    octant(ra, tmp);
    for (int o = 0; o < S; ++o) {
      const long q = (long)orb.rep[3 * o] + (long)orb.rep[3 * o + 1] * H + (long)orb.rep[3 * o + 2] * H * H;
      orr[o] = fr * ra[q];
      oF[o] = fF * fa[q];
    }
  }
  void self_energies(int tmone) {
    if (p.pexp == ORC_PEXP_LO) return;
    std::vector<T> rs(S);
    for (int tp = tmin; tp <= tmax - 1; ++tp) {
      const double sg = thesign(tmone, tp);
      const std::vector<T> &rr = r(tmone, tp);
      for (int o = 0; o < S; ++o) rs[o] = rr[o] * T(sg);
      sunset(F(tmone, tp), rs, sF(tp), sr(tp));
    }
  }
  void rhs_r(std::vector<T> &Mem, int t, int tp) {
    for (auto &x : Mem) x = T(0.0);
    if (p.pexp == ORC_PEXP_LO) return;
    for (int z = tp + 1; z <= t - 2; ++z) {
      const double sg = thesign(z, tp);
      for (int o = 0; o < S; ++o) Mem[o] -= sr(z)[o] * r(z, tp)[o] * T(sg);
    }
  }
  void rhs_F(std::vector<T> &Mem, int t, int tp) {
    if (p.pexp == ORC_PEXP_LO) {
      for (auto &x : Mem) x = T(0.0);
      return;
    }
    for (int o = 0; o < S; ++o) Mem[o] = sr(tmin)[o] * F(tmin, tp)[o] * T(-0.5);
    for (int z = tmin + 1; z <= t - 2; ++z)
      for (int o = 0; o < S; ++o) Mem[o] -= sr(z)[o] * F(z, tp)[o];
    {
      const double sg = thesign(tmin, tp);
      for (int o = 0; o < S; ++o) Mem[o] += T(0.5) * sF(tmin)[o] * r(tmin, tp)[o] * T(sg);
    }
    for (int z = tmin + 1; z <= tp - 1; ++z) {
      const double sg = thesign(z, tp);
      for (int o = 0; o < S; ++o) Mem[o] += sF(z)[o] * r(z, tp)[o] * T(sg);
    }
  }
  void evolve_r(std::vector<T> &R, int t, int tp) {
    std::vector<T> &out = r(t, tp);
    const double st = thesign(t, tp);
    if (tp == t - 1) {
      for (auto &x : out) x = T(st * p.dt);
    } else if (tp == t) {
      for (auto &x : out) x = T(0.0);
    } else {
      const double dt3 = p.dt * p.dt * p.dt, s1 = thesign(t - 1, tp), s2 = thesign(t - 2, tp);
      for (int o = 0; o < S; ++o) {
        const T rhs = R[o] * T(dt3);
        out[o] = ((T(2.0) - omega2[o]) * r(t - 1, tp)[o] * T(s1) - r(t - 2, tp)[o] * T(s2) + rhs) * T(st);
      }
    }
  }
  void evolve_F(std::vector<T> &R, int t, int tp) {
    const double dt3 = p.dt * p.dt * p.dt;
    std::vector<T> &out = F(t, tp);
    for (int o = 0; o < S; ++o)
      out[o] = (T(2.0) - omega2[o]) * F(t - 1, tp)[o] - F(t - 2, tp)[o] + R[o] * T(dt3);
  }
  void evolve(int t) {
    expand();
    self_energies(t - 1);
    hm2 = hartree(t - 1, t - 1);
    for (int o = 0; o < S; ++o) omega2[o] = (T(orb.k2[o]) + hm2) * T(p.dt * p.dt);
    std::vector<T> R(S);
    for (int tp = tmin; tp <= tmax - 1; ++tp) {
      rhs_r(R, t, tp);
      evolve_r(R, t, tp);
      rhs_F(R, t, tp);
      evolve_F(R, t, tp);
    }
    evolve_r(R, t, t);
    rhs_F(R, t, t);
    evolve_F(R, t, t);
  }
  void init(const std::vector<T> &n, double initmass) {
    expand();
    expand();
    for (int o = 0; o < S; ++o) {
      const double om = std::sqrt(orb.k2[o] + initmass * initmass);
      F(1, 1)[o] = T(1 / om) * (n[o] + T(0.5));
      F(2, 1)[o] = T(1 / om) * (n[o] + T(0.5));
      F(2, 2)[o] = T(om) * (n[o] + T(0.5)) * T(p.dt * p.dt) + T(1 / om) * (n[o] + T(0.5));
      r(1, 1)[o] = T(0.0);
      r(2, 1)[o] = T(p.dt * thesign(2, 1));
      r(2, 2)[o] = T(0.0);
    }
    hm2 = hartree(2, 2);
  }
  // createMeasurement: L = sum_o w_n[o] n_o + w_E E at t
  T loss(int t, const double *w_n, double w_E) {
    const double dt = p.dt;
    T E_kin(0.0), E_pot(0.0), E_mem(0.0), hc(0.0), Lw(0.0);
    std::vector<T> ddF(S);
    for (int o = 0; o < S; ++o) {
      const T Fmm = F(t - 1, t - 1)[o];
      ddF[o] = (F(t, t)[o] - T(2.0) * F(t - 1, t)[o] + Fmm) / T(dt * dt);
      const T ow2 = ddF[o] / Fmm;
      const T om = val(ow2) > 0 ? dsqrt_any(ow2) : T(0.0);
      const T c = (0.25 * dt * dt * val(om * om) < 1) ? dsqrt_any(T(1.0) - T(0.25 * dt * dt) * (om * om)) : T(1.0);
      const T nn = (val(ddF[o] * Fmm) > 0) ? c * dsqrt_any(ddF[o] * Fmm) - T(0.5) : T(0.0);
      if (w_n) Lw += T(w_n[o]) * nn;
      E_kin += T(0.5) * ddF[o] * T((double)orb.deg[o]);
      hc += Fmm * T((double)orb.deg[o]);
    }
    for (int o = 0; o < S; ++o)
      E_pot += T(0.5) * (mass2 + T(orb.k2[o]) + T(0.5 * ivol()) * pref() * hc) * F(t - 1, t - 1)[o] *
               T((double)orb.deg[o]);
    if (t != 2) {
      const int tp0 = tmin;
      const double s = thesign(tp0, t - 1);
      for (int o = 0; o < S; ++o)
        E_mem += T(0.5 * 0.25 * dt * (double)orb.deg[o]) *
                 (sr(tp0)[o] * F(tp0, t - 1)[o] - sF(tp0)[o] * r(tp0, t - 1)[o] * T(s));
      for (int o = 0; o < S; ++o)
        for (int tp = tp0 + 1; tp <= t - 2; ++tp) {
          const double st = thesign(tp, t - 1);
          E_mem += T(0.25 * dt * (double)orb.deg[o]) * (sr(tp)[o] * F(tp, t - 1)[o] - sF(tp)[o] * r(tp, t - 1)[o] * T(st));
        }
    }
    return Lw + T(w_E) * (E_kin + E_pot + E_mem);
  }
  static T dsqrt_any(const T &x) {
    if constexpr (std::is_same<T, double>::value) return std::sqrt(x);
    else return dsqrt(x);
  }
};

template <class Fn>
int guarded(Fn f) {
  try {
    f();
    return 0;
  } catch (const std::out_of_range &) {
    return -6;
  } catch (const std::invalid_argument &) {
    return -1;
  } catch (...) {
    return -99;
  }
}

}  // namespace

extern "C" {

void *orc_create(const orc_params *p) {
  try {
    Oracle *o = new Oracle();
    o->setup(*p);
    return o;
  } catch (...) {
    return nullptr;
  }
}
void orc_destroy(void *h) { delete (Oracle *)h; }
int orc_num_orbits(void *h) { return ((Oracle *)h)->orb.S; }
int64_t orc_num_sites(void *h) { return ((Oracle *)h)->orb.V; }
void orc_orbits(void *h, int32_t *rep, double *k2, int64_t *deg) {
  Oracle *o = (Oracle *)h;
  for (int i = 0; i < o->orb.S; ++i) {
    if (rep)
      for (int d = 0; d < 3; ++d) rep[3 * i + d] = o->orb.rep[3 * i + d];
    if (k2) k2[i] = o->orb.k2[i];
    if (deg) deg[i] = o->orb.deg[i];
  }
}
void orc_site_orbit(void *h, int32_t *out) {
  Oracle *o = (Oracle *)h;
  std::memcpy(out, o->orb.orbit_of_site.data(), sizeof(int32_t) * o->orb.V);
}
int orc_init_occupation(void *h, const double *n, double m) {
  return guarded([&] { ((Oracle *)h)->init_occupation(n, m); });
}
int orc_init_gauss(void *h, double xi, double eta, double sig) {
  return guarded([&] { ((Oracle *)h)->init_gauss(xi, eta, sig); });
}
int orc_step(void *h, int32_t t) {
  return guarded([&] { ((Oracle *)h)->evolve(t); });
}
int orc_expand(void *h) {
  return guarded([&] { ((Oracle *)h)->expand(); });
}
int orc_self_energies(void *h, int32_t tmone) {
  return guarded([&] { ((Oracle *)h)->self_energies(tmone); });
}
int orc_measure(void *h, int32_t t, orc_scalars *s, double *F, double *ddF, double *n,
                double *omega, double *c, double *Fonet, double *ronet, double *sigF, double *sigr) {
  return guarded([&] { ((Oracle *)h)->measure(t, s, F, ddF, n, omega, c, Fonet, ronet, sigF, sigr); });
}
int orc_get(void *h, int32_t which, int32_t a, int32_t b, double *out) {
  Oracle *o = (Oracle *)h;
  return guarded([&] {
    const double *src = which == 0 ? o->Fp(a, b) : o->rp(a, b);
    double s = which == 0 ? 1.0 : o->thesign(a, b);
    for (int i = 0; i < o->orb.S; ++i) out[i] = src[o->meas_idx(i)] * s;
  });
}
int orc_set(void *h, int32_t which, int32_t a, int32_t b, const double *in) {
  Oracle *o = (Oracle *)h;
  return guarded([&] {
    double *dst = which == 0 ? o->Fp(a, b) : o->rp(a, b);
    double s = which == 0 ? 1.0 : o->thesign(a, b);
    for (int v = 0; v < o->nv; ++v) {
      int orb = (o->p.engine == ORC_ENGINE_FULL) ? o->orb.orbit_of_site[v] : v;
      dst[v] = in[orb] * s;
    }
  });
}
int orc_get_sigma(void *h, int32_t which, int32_t z, double *out) {
  Oracle *o = (Oracle *)h;
  return guarded([&] {
    const double *src = which == 0 ? o->sigFp(z) : o->sigrp(z);
    for (int i = 0; i < o->orb.S; ++i) out[i] = src[o->meas_idx(i)];
  });
}
int orc_get_lattice(void *h, int32_t which, int32_t a, int32_t b, double *out) {
  Oracle *o = (Oracle *)h;
  if (o->p.engine != ORC_ENGINE_FULL) return -1;
  return guarded([&] {
    const double *src = which == 0 ? o->Fp(a, b) : o->rp(a, b);
    double s = which == 0 ? 1.0 : o->thesign(a, b);
    for (long v = 0; v < o->orb.V; ++v) out[v] = src[v] * s;
  });
}
int orc_window(void *h, int32_t *tmin, int32_t *tmax) {
  Oracle *o = (Oracle *)h;
  *tmin = o->tmin;
  *tmax = o->tmax;
  return 0;
}
double orc_hartree_mass2(void *h, int32_t a, int32_t b) {
  double v = 0.0;
  guarded([&] { v = ((Oracle *)h)->hartree(a, b); });
  return v;
}
void orc_step_times(void *h, double *t_sunset, double *t_rest) {
  *t_sunset = ((Oracle *)h)->last_t_sunset;
  *t_rest = ((Oracle *)h)->last_t_rest;
}
double orc_hartree_prefactor(void *h) { return ((Oracle *)h)->hartree_prefactor(); }
double orc_gap_mass(void *h, const double *n, double x0) { return ((Oracle *)h)->gap_mass(n, x0); }
int orc_sunset_rows(void *h, const double *F, const double *rho, double *sig_F, double *sig_r) {
  Oracle *o = (Oracle *)h;
  return guarded([&] {
    if (o->p.engine == ORC_ENGINE_FULL) {
      std::vector<double> Fl(o->orb.V), rl(o->orb.V), a(o->orb.V), b(o->orb.V);
      for (long s = 0; s < o->orb.V; ++s) {
        Fl[s] = F[o->orb.orbit_of_site[s]];
        rl[s] = rho[o->orb.orbit_of_site[s]];
      }
      o->sunset_lattice(Fl.data(), rl.data(), a.data(), b.data(), o->scratch[0]);
      for (int i = 0; i < o->orb.S; ++i) {
        sig_F[i] = a[o->orb.rep_site[i]];
        sig_r[i] = b[o->orb.rep_site[i]];
      }
    } else {
      o->sunset_rows(F, rho, sig_F, sig_r, o->scratch[0]);
    }
  });
}

// Forward-mode loss derivatives (dual numbers, K = 3 directions: lambda,
// m^2 and the occupation direction dn)
int orc_dual_loss(const orc_params *p, const double *n_init, double init_mass, int32_t t_final, const double *w_n,
                  double w_E, const double *dn, double *L, double *dL) {
  return guarded([&] {
    using D = Dual<3>;
    if (p->sdim != 3 || t_final < 3 || p->pexp > ORC_PEXP_NLO_CLASSICAL)
      throw std::invalid_argument("sdim 3, t_final >= 3, lambda expansion");
    DualEngine<D> e;
    D lam(p->lambda), m2(p->mass2);
    lam.d[0] = 1.0;
    m2.d[1] = 1.0;
    e.setup(*p, lam, m2);
    std::vector<D> n(e.S);
    for (int o = 0; o < e.S; ++o) {
      n[o] = D(n_init[o]);
      n[o].d[2] = dn ? dn[o] : 0.0;
    }
    e.init(n, init_mass);
    for (int t = 3; t <= t_final; ++t) e.evolve(t);
    const D l = e.loss(t_final, w_n, w_E);
    *L = l.v;
    for (int k = 0; k < 3; ++k) dL[k] = l.d[k];
  });
}

}  // extern "C"
