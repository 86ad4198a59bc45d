// kb_api.cu -- host side of libkb2pi: the C ABI declared in include/kb2pi.h.
//
// Owns the device memory of one or more runs, orchestrates one KB step as
// two kernel launches (sunset, memory integral + leapfrog; a third, the
// finishing kernel, in split mode), captures multi-step sequences in a CUDA
// graph, and exposes host views of the history for the reference's
// measure!/getindex. No computation of the step happens on the
// host; without a CUDA device every entry point fails with KB_ERR_NODEV.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>  // header-only NVTX: ranges cost a branch unless a profiler is attached

#include <cuda.h>  // CUtensorMap and its enums (the encoder comes from the runtime's driver entry point)
#include <cudaTypedefs.h>

#include "../../include/kb2pi.h"
#include "kb_internal.cuh"

using kb::KC;
using kb::RunDev;

namespace {

struct Run {
  kb_params p{};
  int H = 0, S = 0, Spad = 0, nchunks = 0, Malloc = 0, T = 0;
  long V = 0;
  std::vector<int32_t> rep;   // 3 per orbit
  std::vector<double> k2, degd;
  std::vector<int64_t> deg;
  std::vector<double> Cm;
  size_t esz = 8;  // bytes per stored history element
  // device allocations
  void *hist_F = nullptr, *hist_r = nullptr, *sig_F = nullptr, *sig_r = nullptr;
  double *st_F = nullptr, *st_r = nullptr, *k2_d = nullptr, *deg_d = nullptr, *Cm_d = nullptr;
  double *tad = nullptr, *meas = nullptr, *epart = nullptr, *rowacc = nullptr, *colacc = nullptr;
  double *pi_r = nullptr, *pi_F = nullptr, *Ik = nullptr, *Jk = nullptr;  // 1/N NLO only
  int *fin = nullptr;  // finishing kernel of a split step
  double *fin_part = nullptr, *fin_prev = nullptr, *hcm2 = nullptr;
  void *tmap = nullptr;  // two CUtensorMap of the history rings
  size_t hist_elems = 0, st_elems = 0, sig_elems = 0;
  RunDev dev{};
};

}  // namespace

struct kb_handle {
  std::string err;
  int device = 0;
  cudaStream_t st = nullptr;
  bool fp64 = true;
  std::vector<Run> runs;
  RunDev *d_runs = nullptr;
  int *d_base_sun = nullptr, *d_base_mi = nullptr;
  int total_sun = 0, total_mi = 0;
  int fin_nb_max = 1;  // CTA slots per chunk of the finishing kernel (max over runs)
  // pipelined measurement (kb_measure_enqueue / kb_measure_take): two pinned
  // host slots holding meas [5][Spad], epart [nchunks][4] and the device error
  // flags of one measured step, by t mod 2
  struct MeasSlot {
    double *host = nullptr;
    size_t cap = 0;  // doubles
    int run = -1, t = -1;
    cudaEvent_t ev = nullptr;
  } mslot[2];
  int *d_t = nullptr, *d_err = nullptr;
  size_t smem_sun = 0, smem_mi = 0;
  size_t smem_sun_tc = 0;  // tensor-core sunset (sunset_variant 2); 0 where it does not apply
  int num_sms = 0, grid_sun = 0, grid_sun_max = 0;
  int memint_variant = 0;         // FP32 consumer layout of the memory-integral kernel
  int memint_compensated = 0;     // FP32 with variant 2: Kahan-compensated tile partial sums
  int memint_bulk = 0;            // 1: history tiles by bulk copies instead of tensor-map boxes
  int test_no_tiles = 0;          // test hook: the memint producer issues no tiles (waits run out)
  int memint_split = 0;           // 1: two half-triangle CTAs per chunk and a finishing kernel;
                                  // 2: the same for the chunks past the last whole wave only
  int memint_persistent = 0;      // 1: one memory-integral CTA per SM taking items from a queue
  std::vector<std::pair<int, void *>> sun_imgs;  // sunset table images by Ns (RunDev::sun_img)
  int *d_mi_queue = nullptr;      // [4] item counters: [0, 1] the persistent memory-integral grids,
                                  // [2, 3] the sunset grids (per group)
  int batch_order = 0;            // order of the runs' CTA ranges in the batched grids
  // concurrent halves of a batch (kb_tuning.batch_overlap > 0): the runs split into two
  // groups of about equal memory-integral work, each with its own schedule tables;
  // group 1's sunset (batch_overlap CTAs) runs on a second, higher-priority stream
  // beside group 0's memory integrals, then group 1's memory integrals follow there
  int batch_overlap = 0;
  int *d_grp_sun[2] = {nullptr, nullptr}, *d_grp_mi[2] = {nullptr, nullptr};
  int grp_n[2] = {0, 0}, grp_sun[2] = {0, 0}, grp_mi[2] = {0, 0};
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int sunset_variant = 0;         // FP32 sunset: 0 1024 threads per CTA, 1 512 threads (2 CTAs per SM),
                                  // 2 tensor cores (kb_sunset_tc.cu; one CTA per SM)
  void *sun_scratch = nullptr;    // FP64 cosine-transform intermediates, one slot per CTA
  size_t sun_scratch_stride = 0;  // elements per slot
  int t_cur = 0;      // last evolved (or initialised) step; window is [tmin(t_cur), t_cur]
  int inited_runs = 0;
  bool any_nlo = false;   // runs with the sunset (lambda expansion at NLO)
  bool any_ninv = false;  // runs of the 1/N expansion at NLO
  size_t smem_ninv = 0, smem_nv = 0;
  bool sigma_valid = false;
  cudaGraphExec_t graph = nullptr;
  int graph_measure = -1;
  // device measurement stream (kb_steps_recorded): step graph with the record
  // kernel, control block {first t, every, capacity}, per-run record offsets
  cudaGraphExec_t graph_rec = nullptr;
  int *d_rec_ctl = nullptr;
  long long *d_rec_off = nullptr;
  double *d_rec = nullptr;
  size_t rec_cap_doubles = 0;
  // profiling: event pairs around each kernel launch, summed on read
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;  // kernel id, (start, stop)
  size_t ev_next = 0;
  double prof_ms[2] = {0, 0};
  int64_t prof_n[2] = {0, 0};
};

namespace {

thread_local std::string g_create_err;

int fail(kb_handle *h, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  else g_create_err = buf;
  return code;
}

#define KB_CUDA(h, call)                                                                 \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail((h), KB_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));     \
  } while (0)

long tet3h(int c) { return (long)c * (c + 1) * (c + 2) / 6; }

// cubic orbits of the Ns^3 lattice (same numbering as the kernels)
void build_orbits(Run &R) {
  const int Ns = R.p.Ns, H = Ns / 2 + 1;
  R.H = H;
  R.S = (int)tet3h(H);
  R.V = (long)Ns * Ns * Ns;
  R.rep.assign((size_t)3 * R.S, 0);
  R.k2.assign(R.S, 0.0);
  R.deg.assign(R.S, 0);
  auto mult = [&](int x) { return (x == 0 || 2 * x == Ns) ? 1 : 2; };
  for (int c = 0; c < H; ++c)
    for (int b = 0; b <= c; ++b)
      for (int a = 0; a <= b; ++a) {
        const int o = kb::orb3(a, b, c);
        R.rep[3 * o] = a;
        R.rep[3 * o + 1] = b;
        R.rep[3 * o + 2] = c;
        double kk = 0.0;
        for (int v : {a, b, c}) {
          const double s = std::sin(M_PI * (double)v / (double)Ns);
          kk += 4.0 * s * s;
        }
        R.k2[o] = kk;
        const int nperm = (a == b && b == c) ? 1 : ((a == b || b == c) ? 3 : 6);
        R.deg[o] = (int64_t)nperm * mult(a) * mult(b) * mult(c);
      }
  R.nchunks = (R.S + KC - 1) / KC;
  R.Spad = R.nchunks * KC;
  R.degd.assign(R.Spad, 0.0);
  for (int o = 0; o < R.S; ++o) R.degd[o] = (double)R.deg[o];
  R.Cm.assign((size_t)H * H, 0.0);
  for (int X = 0; X < H; ++X)
    for (int x = 0; x < H; ++x)
      R.Cm[(size_t)X * H + x] = mult(x) * std::cos(2.0 * M_PI * (double)((long)x * X % Ns) / (double)Ns);
}

int validate(const kb_params &p, std::string &why) {
  char b[256];
  if (p.sdim != 3) { snprintf(b, sizeof b, "sdim=%d: only sdim=3 lattices are supported", p.sdim); why = b; return -1; }
  if ((p.Ns < 2 || p.Ns > 64 || (p.Ns % 2) != 0) && p.Ns != 1) { snprintf(b, sizeof b, "Ns=%d must be 1 or even in [2,64]", p.Ns); why = b; return -1; }
  if (p.M < 3 || p.M > 1024) { snprintf(b, sizeof b, "NstepsinMemory=%d must be in [3,1024]", p.M); why = b; return -1; }
  if (p.N < 1) { why = "ONgroup must be >= 1"; return -1; }
  if (p.flags < 0 || p.flags > 1024) { why = "flags: only bits 0-15 (extra ring slots, at most 1024) are defined"; return -1; }
  if (!(p.dt > 0.0) || !std::isfinite(p.dt)) { why = "dt must be positive"; return -1; }
  if (p.pexp < 0 || p.pexp > 4) { why = "pexp must be one of KB_PEXP_LO .. KB_PEXP_NINV_NLO"; return -1; }
  if (p.pexp == KB_PEXP_NINV_NLO && p.precision != KB_PREC_FP64) { why = "the 1/N expansion at NLO runs in KB_PREC_FP64"; return -1; }
  if (p.precision != KB_PREC_FP64 && p.precision != KB_PREC_MIXED) { why = "unknown precision"; return -1; }
  if (!std::isfinite(p.lambda) || !std::isfinite(p.mass2) || !std::isfinite(p.mass)) { why = "non-finite coupling or mass"; return -1; }
  return 0;
}

size_t slot_off(const Run &R, int a) { return (size_t)(a % R.Malloc); }

void free_run(Run &R) {
  void *ptrs[] = {R.hist_F, R.hist_r, R.sig_F, R.sig_r, R.st_F, R.st_r, R.k2_d, R.deg_d, R.Cm_d, R.tad, R.meas, R.epart,
                  R.rowacc, R.colacc, R.pi_r, R.pi_F, R.Ik, R.Jk, R.fin, R.fin_part, R.fin_prev, R.hcm2, R.tmap};
  for (void *q : ptrs)
    if (q) cudaFree(q);
}

int tmin_of(const Run &R, int t) { return std::max(1, t - R.p.M + 1); }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to
// the CUDA driver library); null when the CUDA driver does not provide it
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// Tensor maps of the two history rings as [tiles][T rows][T*KC] (tile-major
// layout: every T x T x KC tile is contiguous, rows RS apart): maps 0, 1 (F, rho)
// with one tile as the box, maps 2, 3 with the lower T/2 rows of a tile (diagonal
// tiles). Returns a device copy of the four maps, or null (the kernels then use
// plain bulk copies).
void *make_history_maps(const Run &R) {
  auto enc = tensor_map_encoder();
  if (!enc) return nullptr;
  alignas(64) CUtensorMap maps[4];
  const cuuint64_t inner = (cuuint64_t)R.T * KC;
  const cuuint64_t dims[3] = {inner, (cuuint64_t)R.T,
                              (cuuint64_t)R.nchunks * (R.Malloc / R.T) * (R.Malloc / R.T)};
  const cuuint64_t strides[2] = {inner * R.esz, inner * R.T * R.esz};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = R.esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  void *bases[2] = {R.hist_F, R.hist_r};
  for (int m = 0; m < 4; ++m) {
    const cuuint32_t box[3] = {(cuuint32_t)inner, (cuuint32_t)(m < 2 ? R.T : R.T / 2), 1};
    if (enc(&maps[m], dt, 3, bases[m & 1], dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
      return nullptr;
  }
  void *d = nullptr;
  if (cudaMalloc(&d, sizeof maps) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (cudaMemcpy(d, maps, sizeof maps, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d);
    return nullptr;
  }
  return d;
}

// host <-> device copies of one (a, b) element column: S values spread over
// chunks (KC contiguous per chunk)
template <typename TS>
void gather_host(const std::vector<TS> &chunked, int S, double *out) {
  for (int o = 0; o < S; ++o) out[o] = (double)chunked[o];
}

}  // namespace

void kb::kb_set_global_error(const char *msg) { g_create_err = msg; }

// Batched grids: run r owns a contiguous range of CTAs (memory integrals: one
// per chunk) and of persistent-loop items (sunset: one per row t'). The device
// schedule arrays hold [0, nruns) the first item of each position and
// [nruns, 2 nruns) the run at that position. order 0 keeps the runs in order;
// order 1 puts the costliest runs first (memory integrals ~ tiles per chunk,
// sunset ~ H^4 per row), so the longest CTAs start in the first wave and the
// cheap ones fill the tail.
static int apply_schedule(kb_handle *h, int order) {
  const int nr = (int)h->runs.size();
  std::vector<int> pos_mi(nr), pos_sun(nr);
  for (int r = 0; r < nr; ++r) pos_mi[r] = pos_sun[r] = r;
  if (order == 1) {
    auto cost_mi = [&](int r) {
      const double nb = std::ceil((double)h->runs[r].p.M / h->runs[r].T) + 1;
      return nb * (nb + 1) / 2;
    };
    auto cost_sun = [&](int r) { return std::pow((double)h->runs[r].H, 4); };
    std::stable_sort(pos_mi.begin(), pos_mi.end(), [&](int a, int b) { return cost_mi(a) > cost_mi(b); });
    std::stable_sort(pos_sun.begin(), pos_sun.end(), [&](int a, int b) { return cost_sun(a) > cost_sun(b); });
  }
  // group of every run: all in group 0, or (batch_overlap) each run, costliest memory
  // integrals first, to the group with less such work so far
  std::vector<int> grp(nr, 0);
  if (h->batch_overlap > 0) {
    auto cost_mi = [&](int r) {
      const double nb = std::ceil((double)h->runs[r].p.M / h->runs[r].T) + 1;
      return nb * (nb + 1) / 2 * h->runs[r].nchunks;
    };
    std::vector<int> by(nr);
    for (int r = 0; r < nr; ++r) by[r] = r;
    std::stable_sort(by.begin(), by.end(), [&](int a, int b) { return cost_mi(a) > cost_mi(b); });
    double load[2] = {0.0, 0.0};
    for (int r : by) {
      const int g = load[0] <= load[1] ? 0 : 1;
      grp[r] = g;
      load[g] += cost_mi(r);
    }
  }
  // one table pair per group; a run's CTA bases count from its group's first item
  std::vector<int> smi(2 * nr), ssun(2 * nr);
  std::vector<int> gsmi[2], gssun[2];
  for (int g = 0; g < (h->batch_overlap > 0 ? 2 : 1); ++g) {
    std::vector<int> qm, qs;
    for (int q = 0; q < nr; ++q) {
      if (grp[pos_mi[q]] == g) qm.push_back(pos_mi[q]);
      if (grp[pos_sun[q]] == g) qs.push_back(pos_sun[q]);
    }
    const int n = (int)qm.size();
    gsmi[g].assign(2 * n, 0);
    gssun[g].assign(2 * n, 0);
    int bm = 0, bs = 0;
    for (int q = 0; q < n; ++q) {
      Run &Rm = h->runs[qm[q]];
      gsmi[g][q] = bm;
      gsmi[g][n + q] = qm[q];
      Rm.dev.cta_base_mi = bm;
      bm += Rm.nchunks;
      Run &Rs = h->runs[qs[q]];
      gssun[g][q] = bs;
      gssun[g][n + q] = qs[q];
      Rs.dev.cta_base_sun = bs;
      bs += (Rs.p.M + Rs.dev.sun_rows - 1) / Rs.dev.sun_rows;
    }
    h->grp_n[g] = n;
    h->grp_mi[g] = bm;
    h->grp_sun[g] = bs;
  }
  if (h->batch_overlap > 0) {
    for (int g = 0; g < 2; ++g)
      if (cudaMemcpy(h->d_grp_mi[g], gsmi[g].data(), sizeof(int) * gsmi[g].size(), cudaMemcpyHostToDevice) !=
              cudaSuccess ||
          cudaMemcpy(h->d_grp_sun[g], gssun[g].data(), sizeof(int) * gssun[g].size(), cudaMemcpyHostToDevice) !=
              cudaSuccess)
        return KB_ERR_CUDA;
  } else {
    smi = gsmi[0];
    ssun = gssun[0];
  }
  std::vector<RunDev> devs(nr);
  for (int r = 0; r < nr; ++r) {
    h->runs[r].dev.err = h->d_err;
    devs[r] = h->runs[r].dev;
  }
  if (cudaMemcpy(h->d_runs, devs.data(), sizeof(RunDev) * nr, cudaMemcpyHostToDevice) != cudaSuccess)
    return KB_ERR_CUDA;
  if (h->batch_overlap == 0 &&
      (cudaMemcpy(h->d_base_mi, smi.data(), sizeof(int) * 2 * nr, cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(h->d_base_sun, ssun.data(), sizeof(int) * 2 * nr, cudaMemcpyHostToDevice) != cudaSuccess))
    return KB_ERR_CUDA;
  h->batch_order = order;
  return KB_OK;
}

// NVTX range over a scope: each step issued from the host (kb_step, every graph
// launch of kb_steps / kb_steps_recorded) is one named range in a timeline
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// switch the concurrent-group step on (value = CTAs of group 1's sunset) or off and
// upload the schedules for the given run order; the second stream (higher priority,
// so its sunset CTAs take the SMs group 0's memory-integral CTAs free) and its two
// events are created on first use
static int set_overlap(kb_handle *h, int value, int order) {
  if (value > 0 && !h->st2) {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&h->st2, cudaStreamNonBlocking, hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess)
      return fail(h, KB_ERR_CUDA, "second stream for batch_overlap: %s", cudaGetErrorString(cudaGetLastError()));
  }
  if (value != h->batch_overlap || order != h->batch_order) {
    h->batch_overlap = value;
    if (apply_schedule(h, order) != KB_OK) return fail(h, KB_ERR_CUDA, "upload of the run schedule failed");
  }
  return KB_OK;
}

// the memory-integral kernel of the handle's tuning (launch_memint: variant 3 is
// variant 2 with compensated tile sums)
static int memint_launch_variant(const kb_handle *h) {
  return (!h->fp64 && h->memint_variant == 2 && h->memint_compensated) ? 3 : h->memint_variant;
}

// message of a non-zero device error word
static int device_error(kb_handle *h, int e) {
  if (e & kb::DEVERR_TIMEOUT) return fail(h, KB_ERR_TIMEOUT, "a bounded device wait expired (kernel returned early)");
  if (e & kb::DEVERR_BOUNDS) {
    static const char *names[] = {"sunset row", "sunset Sigma index", "memory-integral tile",
                                  "memory-integral row/column", "leapfrog write", "finishing item"};
    char list[256] = "";
    for (int b = 0; b < 6; ++b)
      if (e & (kb::DCHK_SUN_ROW << b)) {
        strncat(list, list[0] ? ", " : "", sizeof list - strlen(list) - 1);
        strncat(list, names[b], sizeof list - strlen(list) - 1);
      }
    return fail(h, KB_ERR_RANGE, "device bounds check failed (KB_DEBUG build): %s", list);
  }
  return fail(h, KB_ERR_CUDA, "device error flags 0x%x", e);
}

// ------------------------------------------------------------------------
extern "C" {

const char *kb_last_error(const kb_handle *h) { return h ? h->err.c_str() : g_create_err.c_str(); }

int kb_create(const kb_params *p, kb_handle **out) { return kb_create_batch(p, 1, out); }

int kb_create_batch(const kb_params *p, int32_t nruns, kb_handle **out) {
  if (!out || !p || nruns < 1) return fail(nullptr, KB_ERR_PARAM, "kb_create: null argument or nruns < 1");
  *out = nullptr;
  for (int r = 0; r < nruns; ++r) {
    std::string why;
    if (validate(p[r], why)) return fail(nullptr, KB_ERR_PARAM, "run %d: %s", r, why.c_str());
    if (p[r].precision != p[0].precision) return fail(nullptr, KB_ERR_PARAM, "all runs of a handle need the same precision");
    if (p[r].device != p[0].device) return fail(nullptr, KB_ERR_PARAM, "all runs of a handle need the same device");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(nullptr, KB_ERR_NODEV, "no CUDA device available");
  }
  if (p[0].device < 0 || p[0].device >= ndev) return fail(nullptr, KB_ERR_PARAM, "device %d out of range", p[0].device);
  kb_handle *h = new kb_handle();
  h->device = p[0].device;
  h->fp64 = (p[0].precision == KB_PREC_FP64);
  h->memint_variant = h->fp64 ? 0 : 2;  // FP32: two consumer groups and leapfrog warps unless kb_set_tuning/kb_autotune choose
  if (cudaSetDevice(h->device) != cudaSuccess) { delete h; return fail(nullptr, KB_ERR_CUDA, "cudaSetDevice failed"); }
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return fail(nullptr, KB_ERR_CUDA, "cudaStreamCreate failed");
  }
  const int T = kb::memint_tile(h->fp64);
  h->runs.resize(nruns);
  size_t smem_sun = 0, smem_mi = 0;
  size_t smem_tc = 0;      // tensor-core sunset (FP32 handles whose lattices it takes), 0 = not available
  bool tc_ok = !h->fp64;
  int base_sun = 0, base_mi = 0;
  for (int r = 0; r < nruns; ++r) {
    Run &R = h->runs[r];
    R.p = p[r];
    build_orbits(R);
    R.T = T;
    R.Malloc = ((R.p.M + (R.p.flags & 0xffff) + T - 1) / T) * T;  // extra slots for kb_adjoint
    R.esz = h->fp64 ? 8 : 4;
    smem_sun = std::max(smem_sun, kb::sunset_smem_bytes(h->fp64, R.H));
    if (kb::pexp_sunset(R.p.pexp)) {
      const size_t b = kb::sunset_tc_smem_bytes(R.H);
      if (b == 0) tc_ok = false;
      smem_tc = std::max(smem_tc, b);
    }
    smem_mi = std::max({smem_mi, kb::memint_smem_bytes(h->fp64, R.Malloc, 0), kb::memint_smem_bytes(h->fp64, R.Malloc, 1),
                        kb::memint_smem_bytes(h->fp64, R.Malloc, 2)});
    base_sun += R.p.M;
    base_mi += R.nchunks;
    if (kb::pexp_sunset(R.p.pexp)) h->any_nlo = true;
    if (R.p.pexp == KB_PEXP_NINV_NLO) {
      h->any_ninv = true;
      h->smem_ninv = std::max(h->smem_ninv, kb::ninv_smem_bytes(R.H));
      h->smem_nv = std::max(h->smem_nv, kb::ninv_volterra_smem_bytes(R.Malloc));
    }
  }
  (void)base_sun;
  h->total_mi = base_mi;
  h->smem_sun = smem_sun;
  // sunset items: FP32 runs of small lattices put several t' rows in one item
  h->total_sun = 0;
  for (auto &R : h->runs) {
    R.dev.sun_rows = (h->fp64 || !kb::pexp_sunset(R.p.pexp)) ? 1 : kb::sunset_rows_per_item(R.H);
    h->total_sun += (R.p.M + R.dev.sun_rows - 1) / R.dev.sun_rows;
  }
  h->smem_mi = smem_mi;
  int maxsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  // the tensor-core kernel also has static shared memory (mbarriers, TMEM slot)
  h->smem_sun_tc = (tc_ok && smem_tc > 0 && smem_tc + kb::sunset_tc_static_bytes() <= (size_t)maxsm) ? smem_tc : 0;
  if ((int)smem_mi > maxsm || (int)smem_sun > maxsm || (int)h->smem_ninv > maxsm || (int)h->smem_nv > maxsm) {
    fail(nullptr, KB_ERR_PARAM, "shared memory need (%zu / %zu B) exceeds the device limit %d B", smem_sun, smem_mi, maxsm);
    kb_destroy(h);
    return KB_ERR_PARAM;
  }
  // allocations
  for (int r = 0; r < nruns; ++r) {
    Run &R = h->runs[r];
    R.hist_elems = (size_t)R.nchunks * R.Malloc * R.Malloc * KC;
    R.st_elems = (size_t)3 * R.nchunks * R.Malloc * KC;
    R.sig_elems = (size_t)R.nchunks * R.Malloc * KC;
    struct A { void **p; size_t bytes; } al[] = {
        {&R.hist_F, R.hist_elems * R.esz}, {&R.hist_r, R.hist_elems * R.esz},
        {&R.sig_F, R.sig_elems * R.esz},   {&R.sig_r, R.sig_elems * R.esz},
        {(void **)&R.st_F, R.st_elems * 8}, {(void **)&R.st_r, R.st_elems * 8},
        {(void **)&R.k2_d, (size_t)R.Spad * 8}, {(void **)&R.deg_d, (size_t)R.Spad * 8},
        {(void **)&R.Cm_d, (size_t)R.H * R.H * 8}, {(void **)&R.tad, (size_t)2 * R.nchunks * 8},
        {(void **)&R.meas, (size_t)5 * R.Spad * 8}, {(void **)&R.epart, (size_t)4 * R.nchunks * 8},
        {(void **)&R.rowacc, (size_t)kb::MEMINT_MAX_PARTS * R.nchunks * R.Malloc * KC * 8},
        {(void **)&R.colacc, (size_t)2 * R.nchunks * R.Malloc * KC * 8},
        {(void **)&R.fin, (size_t)R.nchunks * sizeof(int)},
        {(void **)&R.fin_part, (size_t)R.nchunks * ((R.Malloc + kb::FIN_TP - 1) / kb::FIN_TP) * KC * 8},
        {(void **)&R.fin_prev, (size_t)R.nchunks * KC * 8},
        {(void **)&R.hcm2, (size_t)2 * 8},
    };
    std::vector<A> all(std::begin(al), std::end(al));
    if (R.p.pexp == KB_PEXP_NINV_NLO) {  // bubble rings and the resummed kernels of the window
      all.push_back({(void **)&R.pi_r, R.hist_elems * 8});
      all.push_back({(void **)&R.pi_F, R.hist_elems * 8});
      all.push_back({(void **)&R.Ik, (size_t)R.Malloc * R.Spad * 8});
      all.push_back({(void **)&R.Jk, (size_t)R.Malloc * R.Spad * 8});
    }
    for (auto &a : all) {
      if (cudaMalloc(a.p, a.bytes) != cudaSuccess) {
        cudaGetLastError();
        fail(nullptr, KB_ERR_OOM, "cudaMalloc of %zu bytes failed (run %d)", a.bytes, r);
        kb_destroy(h);
        return KB_ERR_OOM;
      }
      cudaMemsetAsync(*a.p, 0, a.bytes, h->st);
    }
    std::vector<double> k2p(R.Spad, 0.0);
    std::copy(R.k2.begin(), R.k2.end(), k2p.begin());
    cudaMemcpyAsync(R.k2_d, k2p.data(), R.Spad * 8, cudaMemcpyHostToDevice, h->st);
    cudaMemcpyAsync(R.deg_d, R.degd.data(), R.Spad * 8, cudaMemcpyHostToDevice, h->st);
    cudaMemcpyAsync(R.Cm_d, R.Cm.data(), R.Cm.size() * 8, cudaMemcpyHostToDevice, h->st);
    cudaStreamSynchronize(h->st);  // host vectors above are temporaries
    RunDev &D = R.dev;
    // the sunset kernel's tables for this lattice size, built once and shared by the runs
    // of the same Ns (without an image the kernel builds them itself)
    D.sun_img = nullptr;
    if (kb::pexp_sunset(R.p.pexp)) {
      for (auto &im : h->sun_imgs)
        if (im.first == R.p.Ns) D.sun_img = static_cast<const unsigned char *>(im.second);
      if (!D.sun_img) {
        void *img = nullptr;
        if (cudaMalloc(&img, kb::sunset_image_bytes(h->fp64, R.H)) == cudaSuccess &&
            kb::launch_sunset_image(h->fp64, R.H, R.Cm_d, img, h->st) == cudaSuccess) {
          h->sun_imgs.push_back({R.p.Ns, img});
          D.sun_img = static_cast<const unsigned char *>(img);
        } else {
          cudaGetLastError();
          if (img) cudaFree(img);
        }
      }
    }
    D.Ns = R.p.Ns;
    D.H = R.H;
    D.S = R.S;
    D.nchunks = R.nchunks;
    D.M = R.p.M;
    D.Malloc = R.Malloc;
    D.pexp = R.p.pexp;
    D.T = T;
    D.dt = R.p.dt;
    D.dt2 = R.p.dt * R.p.dt;
    D.dt3 = R.p.dt * R.p.dt * R.p.dt;
    D.mass2 = R.p.mass2;
    const double ivol = 1.0 / (double)R.V;
    const double N = (double)R.p.N, lam = R.p.lambda;
    D.ivol = ivol;
    // Hartreeprefactor (TwoPIScalar_Initialization.jl:245-247): lambda/6 for NinverseLO
    D.pref_ivol = (R.p.pexp == KB_PEXP_NINV_LO ? lam * (1.0 / 6.0) : lam * (N + 2.0) / (6.0 * N)) * ivol;
    D.lam = lam;
    D.ninv_fac = -lam / (3.0 * N) * ivol * ivol;
    D.fac_r = ivol * ivol * ivol * (-(lam * lam) * (N + 2.0) / (6.0 * N * N));
    D.fac_F = ivol * ivol * ivol * (-(lam * lam) * (N + 2.0) / (18.0 * N * N));
    D.mass = R.p.mass;
    D.hist_F = R.hist_F;
    D.hist_r = R.hist_r;
    D.st_F = R.st_F;
    D.st_r = R.st_r;
    D.sig_F = R.sig_F;
    D.sig_r = R.sig_r;
    D.k2 = R.k2_d;
    D.deg = R.deg_d;
    D.Cm = R.Cm_d;
    D.tad = R.tad;
    D.meas = R.meas;
    D.epart = R.epart;
    D.rowacc = R.rowacc;
    D.colacc = R.colacc;
    D.fin = R.fin;
    D.fin_nb = (R.Malloc + kb::FIN_TP - 1) / kb::FIN_TP;
    D.fin_part = R.fin_part;
    D.fin_prev = R.fin_prev;
    D.hcm2 = R.hcm2;
    R.tmap = make_history_maps(R);
    D.tmap = R.tmap;
    h->fin_nb_max = std::max(h->fin_nb_max, D.fin_nb);
    D.pi_r = R.pi_r;
    D.pi_F = R.pi_F;
    D.Ik = R.Ik;
    D.Jk = R.Jk;
  }
  bool ok = cudaMalloc(&h->d_runs, sizeof(RunDev) * nruns) == cudaSuccess &&
            cudaMalloc(&h->d_base_sun, sizeof(int) * 2 * nruns) == cudaSuccess &&
            cudaMalloc(&h->d_base_mi, sizeof(int) * 2 * nruns) == cudaSuccess &&
            cudaMalloc(&h->d_grp_sun[0], sizeof(int) * 8 * nruns) == cudaSuccess &&
            cudaMalloc(&h->d_grp_mi[0], sizeof(int) * 8 * nruns) == cudaSuccess &&
            cudaMalloc(&h->d_t, sizeof(int)) == cudaSuccess && cudaMalloc(&h->d_err, sizeof(int)) == cudaSuccess &&
            cudaMalloc(&h->d_mi_queue, 4 * sizeof(int)) == cudaSuccess;
  if (ok) {  // the second group's tables follow the first's
    h->d_grp_sun[1] = h->d_grp_sun[0] + 4 * nruns;
    h->d_grp_mi[1] = h->d_grp_mi[0] + 4 * nruns;
  }
  if (!ok) {
    cudaGetLastError();
    fail(nullptr, KB_ERR_OOM, "cudaMalloc of the run table failed");
    kb_destroy(h);
    return KB_ERR_OOM;
  }
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  h->grid_sun = kb::sunset_grid(h->fp64, h->num_sms, h->total_sun);
  if (apply_schedule(h, 0) != KB_OK) {  // runs in order
    fail(nullptr, KB_ERR_CUDA, "upload of the run table failed");
    kb_destroy(h);
    return KB_ERR_CUDA;
  }
  cudaMemset(h->d_t, 0, sizeof(int));
  cudaMemset(h->d_err, 0, sizeof(int));
  // the attribute is per kernel, shared by all handles: allow the device maximum
  cudaError_t e1 = kb::configure_sunset(h->fp64, (size_t)maxsm);
  cudaError_t e2 = kb::configure_memint(h->fp64, (size_t)maxsm);
  if (e1 == cudaSuccess && !h->fp64) e1 = kb::configure_sunset_tc((size_t)maxsm);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    fail(nullptr, KB_ERR_CUDA, "kernel configuration failed: %s", cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    kb_destroy(h);
    return KB_ERR_CUDA;
  }
  // the largest sunset grid the tuner may pick: up to 4 resident CTAs per SM
  {
    int per_sm = kb::sunset_max_ctas_per_sm(h->fp64, 0, h->smem_sun);
    if (!h->fp64) per_sm = std::max(per_sm, kb::sunset_max_ctas_per_sm(false, 1, h->smem_sun));
    h->grid_sun_max = std::max(1, std::min(h->total_sun, h->num_sms * std::min(4, per_sm)));
  }
  if (h->any_ninv) {
    cudaError_t e3 = kb::configure_ninv((size_t)maxsm);
    if (e3 != cudaSuccess) {
      fail(nullptr, KB_ERR_CUDA, "kernel configuration failed: %s", cudaGetErrorString(e3));
      kb_destroy(h);
      return KB_ERR_CUDA;
    }
  }
  if (h->fp64 && (h->any_nlo || h->any_ninv)) {
    int Hmax = 1;
    for (auto &R : h->runs) Hmax = std::max(Hmax, R.H);
    h->sun_scratch_stride = kb::sunset_scratch_elems(Hmax);
    const size_t bytes = (size_t)h->grid_sun_max * h->sun_scratch_stride * sizeof(double);
    if (cudaMalloc(&h->sun_scratch, bytes) != cudaSuccess) {
      cudaGetLastError();
      fail(nullptr, KB_ERR_OOM, "cudaMalloc of %zu bytes of sunset scratch failed", bytes);
      kb_destroy(h);
      return KB_ERR_OOM;
    }
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    fail(nullptr, KB_ERR_CUDA, "device error during kb_create: %s", cudaGetErrorString(cudaGetLastError()));
    kb_destroy(h);
    return KB_ERR_CUDA;
  }
  *out = h;
  return KB_OK;
}

void kb_destroy(kb_handle *h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->graph_rec) cudaGraphExecDestroy(h->graph_rec);
  if (h->d_rec_ctl) cudaFree(h->d_rec_ctl);
  if (h->d_rec_off) cudaFree(h->d_rec_off);
  if (h->d_rec) cudaFree(h->d_rec);
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  for (auto &m : h->mslot) {
    if (m.ev) cudaEventDestroy(m.ev);
    if (m.host) cudaFreeHost(m.host);
  }
  for (auto &R : h->runs) free_run(R);
  for (auto &im : h->sun_imgs) cudaFree(im.second);
  void *ptrs[] = {h->d_runs, h->d_base_sun, h->d_base_mi, h->d_grp_sun[0], h->d_grp_mi[0], h->d_t, h->d_err, h->d_mi_queue,
                  h->sun_scratch};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->st2) cudaStreamDestroy(h->st2);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
}

int kb_num_orbits(const kb_handle *h, int32_t run, int32_t *S) {
  if (!h || run < 0 || run >= (int)h->runs.size() || !S) return KB_ERR_PARAM;
  *S = h->runs[run].S;
  return KB_OK;
}

int kb_get_orbits(const kb_handle *h, int32_t run, int32_t *rep, double *k2, int64_t *deg) {
  if (!h || run < 0 || run >= (int)h->runs.size()) return KB_ERR_PARAM;
  const Run &R = h->runs[run];
  if (rep) std::memcpy(rep, R.rep.data(), sizeof(int32_t) * 3 * R.S);
  if (k2) std::memcpy(k2, R.k2.data(), sizeof(double) * R.S);
  if (deg) std::memcpy(deg, R.deg.data(), sizeof(int64_t) * R.S);
  return KB_OK;
}

int kb_site_orbits(const kb_handle *h, int32_t run, int32_t *out) {
  if (!h || run < 0 || run >= (int)h->runs.size() || !out) return KB_ERR_PARAM;
  const Run &R = h->runs[run];
  const int Ns = R.p.Ns;
  for (long s = 0; s < R.V; ++s) {
    int n[3] = {(int)(s % Ns), (int)((s / Ns) % Ns), (int)(s / ((long)Ns * Ns))};
    int f[3];
    for (int d = 0; d < 3; ++d) f[d] = std::min(n[d], Ns - n[d]);
    std::sort(f, f + 3);
    out[s] = kb::orb3(f[0], f[1], f[2]);
  }
  return KB_OK;
}

// write one (a,b) element column (S values, double on the host) into the
// history (storage type) and, for the last three rows, into the FP64 state
static int put_pair(kb_handle *h, Run &R, int which, int a, int b, const double *vals, bool to_state) {
  // normalise to the later-first pair
  double sgn = 1.0;
  if (a < b) {
    std::swap(a, b);
    if (which == 1) sgn = -1.0;
  }
  const size_t pitch_hist = (size_t)R.Malloc * R.Malloc * KC;
  const size_t pitch_row = (size_t)R.Malloc * KC;
  std::vector<double> dv(R.Spad, 0.0);
  for (int o = 0; o < R.S; ++o) dv[o] = sgn * vals[o];
  if (a == b && which == 1)
    for (int o = 0; o < R.S; ++o) dv[o] = 0.0;  // rho(a,a) = 0 is structural
  std::vector<float> fv;
  const void *src = dv.data();
  if (R.esz == 4) {
    fv.resize(R.Spad);
    for (int o = 0; o < R.Spad; ++o) fv[o] = (float)dv[o];
    src = fv.data();
  }
  char *hist = (char *)(which == 0 ? R.hist_F : R.hist_r);
  char *dst = hist + kb::hist_off(R.Malloc, R.T, 0, a, b, 0) * R.esz;  // chunks are Malloc^2 * KC apart
  KB_CUDA(h, cudaMemcpy2DAsync(dst, pitch_hist * R.esz, src, KC * R.esz, KC * R.esz, R.nchunks,
                               cudaMemcpyHostToDevice, h->st));
  if (to_state) {
    double *stb = (which == 0 ? R.st_F : R.st_r) + (size_t)(a % 3) * R.nchunks * pitch_row + slot_off(R, b) * KC;
    KB_CUDA(h, cudaMemcpy2DAsync(stb, pitch_row * 8, dv.data(), KC * 8, KC * 8, R.nchunks,
                                 cudaMemcpyHostToDevice, h->st));
  }
  KB_CUDA(h, cudaStreamSynchronize(h->st));
  return KB_OK;
}

int kb_init_rows(kb_handle *h, int32_t run, const double *F11, const double *F21, const double *F22) {
  if (!h || run < 0 || run >= (int)h->runs.size() || !F11 || !F21 || !F22)
    return fail(h, KB_ERR_PARAM, "kb_init_rows: bad arguments");
  if (h->t_cur > 2) return fail(h, KB_ERR_PARAM, "kb_init: the simulation has already been evolved");
  cudaSetDevice(h->device);
  Run &R = h->runs[run];
  std::vector<double> zero(R.S, 0.0), dtv(R.S, R.p.dt);
  int rc;
  if ((rc = put_pair(h, R, 0, 1, 1, F11, true))) return rc;
  if ((rc = put_pair(h, R, 0, 2, 1, F21, true))) return rc;
  if ((rc = put_pair(h, R, 0, 2, 2, F22, true))) return rc;
  if ((rc = put_pair(h, R, 1, 1, 1, zero.data(), true))) return rc;
  if ((rc = put_pair(h, R, 1, 2, 1, dtv.data(), true))) return rc;
  if ((rc = put_pair(h, R, 1, 2, 2, zero.data(), true))) return rc;
  h->inited_runs |= 1;  // at least one run initialised
  h->t_cur = 2;
  h->sigma_valid = false;
  // measurement of t = 2 and the tadpole sums of F(2,2) for all runs
  KB_CUDA(h, kb::launch_measure_init(h->d_runs, (int)h->runs.size(), 2, h->st));
  KB_CUDA(h, cudaStreamSynchronize(h->st));
  return KB_OK;
}

int kb_init(kb_handle *h, int32_t run, const double *n, double init_mass) {
  if (!h || run < 0 || run >= (int)h->runs.size() || !n) return fail(h, KB_ERR_PARAM, "kb_init: bad arguments");
  const Run &R = h->runs[run];
  std::vector<double> F11(R.S), F21(R.S), F22(R.S);
  const double dt = R.p.dt;
  // initSimData! (TwoPIScalar_Initialization.jl:38-41)
  for (int o = 0; o < R.S; ++o) {
    const double omega = std::sqrt(R.k2[o] + init_mass * init_mass);
    F11[o] = 1 / omega * (n[o] + 0.5);
    F21[o] = 1 / omega * (n[o] + 0.5);
    F22[o] = omega * (n[o] + 0.5) * (dt * dt) + 1 / omega * (n[o] + 0.5);
  }
  return kb_init_rows(h, run, F11.data(), F21.data(), F22.data());
}

static cudaEvent_t next_event(kb_handle *h) {
  if (h->ev_next == h->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    h->ev_pool.push_back(e);
  }
  return h->ev_pool[h->ev_next++];
}

// Sigma(t-1, .) of every run: the sunset (lambda expansion) and/or the 1/N
// kernels; each kernel skips the runs of the other expansion.

// the sunset of the runs of one schedule table (all runs, or one group)
// (g: the group whose item counter the grid takes items from)
static int launch_sun(kb_handle *h, const int *base, int n, int total, int grid, cudaStream_t st, int g) {
  if (!h->any_nlo || total <= 0) return KB_OK;
  grid = std::max(1, std::min(grid, total));
  if (h->sunset_variant == 2)
    KB_CUDA(h, kb::launch_sunset_tc(h->d_runs, base, n, total, std::min(grid, h->num_sms), h->d_t, h->smem_sun_tc,
                                    st));
  else
    KB_CUDA(h, kb::launch_sunset(h->fp64, h->sunset_variant, h->d_runs, base, n, total, grid, h->d_t,
                                 h->sun_scratch, h->sun_scratch_stride, h->smem_sun, h->d_mi_queue + 2 + g, st));
  return KB_OK;
}
// the memory integrals of the runs of one schedule table (group g's queue when persistent)
// sms: the SMs the grid may take (a persistent grid has that many CTAs; fewer than the
// device's leaves the rest to a concurrent kernel); the whole waves are waves of sms CTAs
static int launch_mi(kb_handle *h, const int *base, int n, int total, int measure, cudaStream_t st, int g,
                     int sms) {
  const int nwhole = h->memint_split == 2 ? (total / sms) * sms : 0;
  KB_CUDA(h, kb::launch_memint(h->fp64, memint_launch_variant(h), h->memint_split, nwhole, h->d_runs, base, n, total,
                               h->fin_nb_max, !h->memint_bulk + 2 * h->test_no_tiles, h->d_t, h->d_err, measure,
                               h->smem_mi, h->memint_persistent ? h->d_mi_queue + g : nullptr, sms, st));
  return KB_OK;
}

static int launch_self_energies(kb_handle *h) {
  if (h->batch_overlap > 0) {  // both groups in turn (kb_self_energies, autotuning)
    for (int g = 0; g < 2; ++g) {
      const int rc = launch_sun(h, h->d_grp_sun[g], h->grp_n[g], h->grp_sun[g], h->grid_sun, h->st, g);
      if (rc) return rc;
    }
    return KB_OK;
  }
  if (h->any_nlo) {
    const int rc = launch_sun(h, h->d_base_sun, (int)h->runs.size(), h->total_sun, h->grid_sun, h->st, 0);
    if (rc) return rc;
  }
  if (h->any_ninv)
    KB_CUDA(h, kb::launch_ninv(h->d_runs, h->d_base_sun, h->d_base_mi, (int)h->runs.size(), h->total_sun, h->total_mi,
                               std::min(h->grid_sun, h->grid_sun_max), h->d_t, h->sun_scratch, h->sun_scratch_stride,
                               h->smem_ninv, h->smem_nv, h->st));
  return KB_OK;
}

// a step of a batch in two concurrent groups: group 0's sunset on the handle's
// stream; then group 0's memory integrals there while group 1's sunset (on
// batch_overlap CTAs) and memory integrals run on the second stream; joined at the end
static int launch_step_overlap(kb_handle *h, int measure, cudaEvent_t e0, cudaEvent_t e1, cudaEvent_t e2) {
  if (e0) KB_CUDA(h, cudaEventRecord(e0, h->st));
  int rc = launch_sun(h, h->d_grp_sun[0], h->grp_n[0], h->grp_sun[0], h->grid_sun, h->st, 0);
  if (rc) return rc;
  if (e1) KB_CUDA(h, cudaEventRecord(e1, h->st));
  KB_CUDA(h, cudaEventRecord(h->ev_fork, h->st));
  KB_CUDA(h, cudaStreamWaitEvent(h->st2, h->ev_fork, 0));
  // group 1's sunset on batch_overlap SMs (as many CTAs as fit there); a persistent grid
  // for group 0's memory integrals takes the other SMs
  const int occ = h->sunset_variant == 2 ? 1 : std::max(1, kb::sunset_max_ctas_per_sm(h->fp64, h->sunset_variant,
                                                                                        h->smem_sun));
  if ((rc = launch_sun(h, h->d_grp_sun[1], h->grp_n[1], h->grp_sun[1], h->batch_overlap * occ, h->st2, 1))) return rc;
  const int sms0 = h->memint_persistent ? std::max(1, h->num_sms - h->batch_overlap) : h->num_sms;
  if ((rc = launch_mi(h, h->d_grp_mi[0], h->grp_n[0], h->grp_mi[0], measure, h->st, 0, sms0))) return rc;
  if ((rc = launch_mi(h, h->d_grp_mi[1], h->grp_n[1], h->grp_mi[1], measure, h->st2, 1, h->num_sms))) return rc;
  KB_CUDA(h, cudaEventRecord(h->ev_join, h->st2));
  KB_CUDA(h, cudaStreamWaitEvent(h->st, h->ev_join, 0));
  if (e2) {
    KB_CUDA(h, cudaEventRecord(e2, h->st));
    h->ev_pending.push_back({0, {e0, e1}});  // group 0's sunset alone
    h->ev_pending.push_back({1, {e1, e2}});  // the rest of the step
  }
  return KB_OK;
}

static int launch_step(kb_handle *h, int measure) {
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  if (h->profiling) {
    e0 = next_event(h);
    e1 = next_event(h);
    e2 = next_event(h);
    if (!e0 || !e1 || !e2) return fail(h, KB_ERR_CUDA, "cudaEventCreate failed");
  }
  if (h->batch_overlap > 0) return launch_step_overlap(h, measure, e0, e1, e2);
  if (e0) KB_CUDA(h, cudaEventRecord(e0, h->st));
  {
    const int rc = launch_self_energies(h);
    if (rc) return rc;
  }
  if (h->profiling) {
    KB_CUDA(h, cudaEventRecord(e1, h->st));
    if (h->any_nlo || h->any_ninv) h->ev_pending.push_back({0, {e0, e1}});
  }
  {
    const int rc = launch_mi(h, h->d_base_mi, (int)h->runs.size(), h->total_mi, measure, h->st, 0, h->num_sms);
    if (rc) return rc;
  }
  if (h->profiling) {
    KB_CUDA(h, cudaEventRecord(e2, h->st));
    h->ev_pending.push_back({1, {e1, e2}});
  }
  return KB_OK;
}

// the graph of one step (its kernels, then t advanced on the device), captured once per
// tuning: kb_steps launches it per step, kb_step too unless per-kernel events are on
static int ensure_step_graph(kb_handle *h) {
  if (h->graph) return KB_OK;
  cudaGraph_t g;
  KB_CUDA(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  int rc = launch_step(h, 1);
  cudaError_t ea = (rc == 0) ? (cudaError_t)kb::launch_advance_t(h->d_t, h->st) : cudaSuccess;
  cudaError_t ec = cudaStreamEndCapture(h->st, &g);
  if (rc) return rc;
  if (ea != cudaSuccess || ec != cudaSuccess) return fail(h, KB_ERR_CUDA, "graph capture failed");
  cudaError_t ei = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) return fail(h, KB_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(ei));
  return KB_OK;
}

int kb_step(kb_handle *h, int32_t t) {
  if (!h) return KB_ERR_PARAM;
  if (h->t_cur < 2) return fail(h, KB_ERR_PARAM, "kb_step before kb_init");
  if (t != h->t_cur + 1) return fail(h, KB_ERR_PARAM, "kb_step(%d): expected t = %d (lastEvolStep + 1)", t, h->t_cur + 1);
  cudaSetDevice(h->device);
  NvtxRange range("kb_step");
  KB_CUDA(h, kb::launch_set_t(h->d_t, t, h->st));
  int rc = 0;
  if (h->profiling) {  // the step's own launches, between the profiling events
    rc = launch_step(h, 1);
  } else if (!(rc = ensure_step_graph(h))) {
    KB_CUDA(h, cudaGraphLaunch(h->graph, h->st));
  }
  if (rc) return rc;
  h->t_cur = t;
  h->sigma_valid = h->any_nlo || h->any_ninv;
  return KB_OK;
}

int kb_expand(kb_handle *h) {
  if (!h) return KB_ERR_PARAM;
  if (h->t_cur < 2) return fail(h, KB_ERR_PARAM, "kb_expand before kb_init");
  h->t_cur += 1;
  h->sigma_valid = false;
  return KB_OK;
}

// energies of step t from the per-chunk partials ep [nchunks][4]
static void scalars_from(const Run &R, int t, const double *ep, kb_meas_scalars *s) {
  double ek = 0, epo = 0, em = 0;
  for (int c = 0; c < R.nchunks; ++c) {
    ek += ep[(size_t)c * 4 + 0];
    epo += ep[(size_t)c * 4 + 1];
    em += ep[(size_t)c * 4 + 2];
  }
  s->time = (t - 1) * R.p.dt * R.p.mass;
  s->E_kin = ek;
  s->E_pot = epo;
  s->E_mem = (t == 2) ? 0.0 : em;
  s->E = s->E_kin + s->E_pot + s->E_mem;
  s->M2 = ep[3];
}

static int collect_scalars(kb_handle *h, int run, int t, kb_meas_scalars *s) {
  Run &R = h->runs[run];
  std::vector<double> ep((size_t)4 * R.nchunks);
  KB_CUDA(h, cudaMemcpyAsync(ep.data(), R.epart, ep.size() * 8, cudaMemcpyDeviceToHost, h->st));
  KB_CUDA(h, cudaStreamSynchronize(h->st));
  scalars_from(R, t, ep.data(), s);
  return KB_OK;
}

int kb_measure(kb_handle *h, int32_t run, int32_t t, kb_meas_scalars *s, double *F, double *ddF, double *n,
               double *omega, double *c) {
  if (!h || run < 0 || run >= (int)h->runs.size()) return KB_ERR_PARAM;
  if (t != h->t_cur || h->t_cur < 2) return fail(h, KB_ERR_PARAM, "kb_measure(%d): only the last evolved step %d can be measured", t, h->t_cur);
  cudaSetDevice(h->device);
  Run &R = h->runs[run];
  int rc = kb_sync(h);
  if (rc) return rc;
  double *outs[5] = {F, ddF, n, omega, c};
  if (n || omega || c) KB_CUDA(h, kb::launch_meas_derive(h->d_runs, run, R.S, h->st));
  for (int q = 0; q < 5; ++q)
    if (outs[q]) KB_CUDA(h, cudaMemcpyAsync(outs[q], R.meas + (size_t)q * R.Spad, R.S * 8, cudaMemcpyDeviceToHost, h->st));
  kb_meas_scalars tmp;
  rc = collect_scalars(h, run, t, s ? s : &tmp);
  if (rc) return rc;
  if (s && !std::isfinite(s->E)) return fail(h, KB_ERR_NAN, "non-finite energy at t=%d", t);
  return KB_OK;
}

int kb_measure_enqueue(kb_handle *h, int32_t run, int32_t t) {
  if (!h || run < 0 || run >= (int)h->runs.size()) return KB_ERR_PARAM;
  if (t != h->t_cur || h->t_cur < 2)
    return fail(h, KB_ERR_PARAM, "kb_measure_enqueue(%d): only the last evolved step %d can be measured", t, h->t_cur);
  cudaSetDevice(h->device);
  Run &R = h->runs[run];
  auto &m = h->mslot[t & 1];
  const size_t nm = (size_t)5 * R.Spad, ne = (size_t)4 * R.nchunks, need = nm + ne + 1;
  if (!m.ev) KB_CUDA(h, cudaEventCreateWithFlags(&m.ev, cudaEventDisableTiming));
  if (m.cap < need) {
    if (m.host) {
      KB_CUDA(h, cudaEventSynchronize(m.ev));  // a copy into the old buffer may be in flight
      cudaFreeHost(m.host);
      m.host = nullptr;
      m.cap = 0;
    }
    KB_CUDA(h, cudaHostAlloc((void **)&m.host, need * sizeof(double), cudaHostAllocDefault));
    m.cap = need;
  }
  // behind step t's kernels on the handle's stream; step t+1's run after them
  KB_CUDA(h, kb::launch_meas_derive(h->d_runs, run, R.S, h->st));
  KB_CUDA(h, cudaMemcpyAsync(m.host, R.meas, nm * 8, cudaMemcpyDeviceToHost, h->st));
  KB_CUDA(h, cudaMemcpyAsync(m.host + nm, R.epart, ne * 8, cudaMemcpyDeviceToHost, h->st));
  KB_CUDA(h, cudaMemcpyAsync(m.host + nm + ne, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  // the flags now travel with this measurement: clear them in stream order, so that
  // kernels of later steps set them afresh and each error is reported once (by take)
  KB_CUDA(h, cudaMemsetAsync(h->d_err, 0, sizeof(int), h->st));
  KB_CUDA(h, cudaEventRecord(m.ev, h->st));
  m.run = run;
  m.t = t;
  return KB_OK;
}

int kb_measure_take(kb_handle *h, int32_t run, int32_t t, kb_meas_scalars *s, double *F, double *ddF, double *n,
                    double *omega, double *c) {
  if (!h || run < 0 || run >= (int)h->runs.size()) return KB_ERR_PARAM;
  auto &m = h->mslot[t & 1];
  if (m.t != t || m.run != run)
    return fail(h, KB_ERR_PARAM, "kb_measure_take(%d): no measurement of step %d of run %d is queued", t, t, run);
  cudaSetDevice(h->device);
  KB_CUDA(h, cudaEventSynchronize(m.ev));
  m.t = -1;  // taken
  Run &R = h->runs[run];
  const size_t nm = (size_t)5 * R.Spad, ne = (size_t)4 * R.nchunks;
  int e = 0;
  std::memcpy(&e, m.host + nm + ne, sizeof(int));
  if (e) return device_error(h, e);  // flags cleared on the stream right after their copy (kb_measure_enqueue)
  double *outs[5] = {F, ddF, n, omega, c};
  for (int q = 0; q < 5; ++q)
    if (outs[q]) std::memcpy(outs[q], m.host + (size_t)q * R.Spad, (size_t)R.S * 8);
  kb_meas_scalars tmp;
  kb_meas_scalars *sp = s ? s : &tmp;
  scalars_from(R, t, m.host + nm, sp);
  if (!std::isfinite(sp->E)) return fail(h, KB_ERR_NAN, "non-finite energy at t=%d", t);
  return KB_OK;
}

static int fetch_pair(kb_handle *h, Run &R, int which, int a, int b, double *out) {
  double sgn = 1.0;
  if (a < b) {
    std::swap(a, b);
    if (which == 1) sgn = -1.0;
  }
  const size_t pitch_row = (size_t)R.Malloc * KC;
  std::vector<double> dv(R.Spad, 0.0);
  if (a >= h->t_cur - 2 && a <= h->t_cur) {
    const double *stb = (which == 0 ? R.st_F : R.st_r) + (size_t)(a % 3) * R.nchunks * pitch_row + slot_off(R, b) * KC;
    KB_CUDA(h, cudaMemcpy2DAsync(dv.data(), KC * 8, stb, pitch_row * 8, KC * 8, R.nchunks, cudaMemcpyDeviceToHost, h->st));
    KB_CUDA(h, cudaStreamSynchronize(h->st));
  } else {
    const size_t pitch_hist = (size_t)R.Malloc * R.Malloc * KC;
    const char *hist = (const char *)(which == 0 ? R.hist_F : R.hist_r);
    const char *src = hist + kb::hist_off(R.Malloc, R.T, 0, a, b, 0) * R.esz;  // chunks are Malloc^2 * KC apart
    if (R.esz == 8) {
      KB_CUDA(h, cudaMemcpy2DAsync(dv.data(), KC * 8, src, pitch_hist * 8, KC * 8, R.nchunks, cudaMemcpyDeviceToHost, h->st));
      KB_CUDA(h, cudaStreamSynchronize(h->st));
    } else {
      std::vector<float> fv(R.Spad);
      KB_CUDA(h, cudaMemcpy2DAsync(fv.data(), KC * 4, src, pitch_hist * 4, KC * 4, R.nchunks, cudaMemcpyDeviceToHost, h->st));
      KB_CUDA(h, cudaStreamSynchronize(h->st));
      for (int o = 0; o < R.Spad; ++o) dv[o] = fv[o];
    }
  }
  for (int o = 0; o < R.S; ++o) out[o] = sgn * dv[o];
  return KB_OK;
}

int kb_get(kb_handle *h, int32_t run, int32_t which, int32_t a, int32_t b, double *out) {
  if (!h || run < 0 || run >= (int)h->runs.size() || !out || (which != 0 && which != 1)) return KB_ERR_PARAM;
  Run &R = h->runs[run];
  const int tmin = tmin_of(R, h->t_cur);
  if (h->t_cur < 2 || a < tmin || a > h->t_cur || b < tmin || b > h->t_cur)
    return fail(h, KB_ERR_RANGE, "Indices not in range! (%d,%d) outside [%d,%d]", a, b, tmin, h->t_cur);
  cudaSetDevice(h->device);
  int rc = kb_sync(h);
  if (rc) return rc;
  return fetch_pair(h, R, which, a, b, out);
}

int kb_set(kb_handle *h, int32_t run, int32_t which, int32_t a, int32_t b, const double *in) {
  if (!h || run < 0 || run >= (int)h->runs.size() || !in || (which != 0 && which != 1)) return KB_ERR_PARAM;
  Run &R = h->runs[run];
  const int tmin = tmin_of(R, h->t_cur);
  if (h->t_cur < 2 || a < tmin || a > h->t_cur || b < tmin || b > h->t_cur)
    return fail(h, KB_ERR_RANGE, "Indices not in range! (%d,%d) outside [%d,%d]", a, b, tmin, h->t_cur);
  cudaSetDevice(h->device);
  int rc = kb_sync(h);
  if (rc) return rc;
  const int later = std::max(a, b);
  return put_pair(h, R, which, a, b, in, later >= h->t_cur - 2);
}

int kb_self_energies(kb_handle *h, int32_t tmone) {
  if (!h) return KB_ERR_PARAM;
  if (tmone != h->t_cur - 1 || h->t_cur < 3)
    return fail(h, KB_ERR_PARAM, "kb_self_energies(%d): tmone must be the current tmax - 1 = %d", tmone, h->t_cur - 1);
  cudaSetDevice(h->device);
  KB_CUDA(h, kb::launch_set_t(h->d_t, h->t_cur, h->st));
  {
    const int rc = launch_self_energies(h);
    if (rc) return rc;
  }
  h->sigma_valid = true;
  return kb_sync(h);
}

int kb_get_sigma(kb_handle *h, int32_t run, int32_t which, int32_t z, double *out) {
  if (!h || run < 0 || run >= (int)h->runs.size() || !out || (which != 0 && which != 1)) return KB_ERR_PARAM;
  Run &R = h->runs[run];
  const int tmin = tmin_of(R, h->t_cur);
  if (!h->sigma_valid) return fail(h, KB_ERR_PARAM, "no self-energies computed for the current window");
  if (z < tmin || z > h->t_cur - 1) return fail(h, KB_ERR_RANGE, "Indices not in range! z=%d outside [%d,%d]", z, tmin, h->t_cur - 1);
  cudaSetDevice(h->device);
  int rc = kb_sync(h);
  if (rc) return rc;
  const size_t pitch = (size_t)R.Malloc * KC;
  const char *base = (const char *)(which == 0 ? R.sig_F : R.sig_r) + slot_off(R, z) * KC * R.esz;
  std::vector<double> dv(R.Spad);
  if (R.esz == 8) {
    KB_CUDA(h, cudaMemcpy2DAsync(dv.data(), KC * 8, base, pitch * 8, KC * 8, R.nchunks, cudaMemcpyDeviceToHost, h->st));
  } else {
    std::vector<float> fv(R.Spad);
    KB_CUDA(h, cudaMemcpy2DAsync(fv.data(), KC * 4, base, pitch * 4, KC * 4, R.nchunks, cudaMemcpyDeviceToHost, h->st));
    KB_CUDA(h, cudaStreamSynchronize(h->st));
    for (int o = 0; o < R.Spad; ++o) dv[o] = fv[o];
  }
  KB_CUDA(h, cudaStreamSynchronize(h->st));
  for (int o = 0; o < R.S; ++o) out[o] = dv[o];
  return KB_OK;
}

int kb_window(const kb_handle *h, int32_t run, int32_t *tmin, int32_t *tmax) {
  if (!h || run < 0 || run >= (int)h->runs.size()) return KB_ERR_PARAM;
  if (tmin) *tmin = h->t_cur >= 1 ? tmin_of(h->runs[run], h->t_cur) : 0;
  if (tmax) *tmax = h->t_cur;
  return KB_OK;
}

int kb_get_traces(kb_handle *h, int32_t run, double *Fonet, double *ronet, double *SigF, double *Sigr) {
  if (!h || run < 0 || run >= (int)h->runs.size()) return KB_ERR_PARAM;
  Run &R = h->runs[run];
  const int t = h->t_cur, tmin = tmin_of(R, t);
  std::vector<double> v(R.S);
  for (int tp = tmin, q = 0; tp <= t - 1; ++tp, ++q) {
    int rc;
    if (Fonet) {
      if ((rc = kb_get(h, run, 0, tmin, tp, v.data()))) return rc;
      Fonet[q] = v[0];
    }
    if (ronet) {
      if ((rc = kb_get(h, run, 1, tmin, tp, v.data()))) return rc;
      ronet[q] = v[0];
    }
  }
  if ((SigF || Sigr) && kb::pexp_lo(R.p.pexp)) {  // LO: no self-energy, the traces are zero
    for (int tp = t - 1, q = 0; tp >= tmin; --tp, ++q) {
      if (SigF) SigF[q] = 0.0;
      if (Sigr) Sigr[q] = 0.0;
    }
  } else if (SigF || Sigr) {
    for (int tp = t - 1, q = 0; tp >= tmin; --tp, ++q) {
      int rc;
      if (SigF) {
        if ((rc = kb_get_sigma(h, run, 0, tp, v.data()))) return rc;
        SigF[q] = v[0];
      }
      if (Sigr) {
        if ((rc = kb_get_sigma(h, run, 1, tp, v.data()))) return rc;
        Sigr[q] = v[0];
      }
    }
  }
  return KB_OK;
}

int kb_steps(kb_handle *h, int32_t t0, int32_t count, int32_t measure_every, kb_meas_scalars *out,
             int32_t out_capacity) {
  if (!h || count < 0) return KB_ERR_PARAM;
  if (h->t_cur < 2) return fail(h, KB_ERR_PARAM, "kb_steps before kb_init");
  if (t0 != h->t_cur + 1) return fail(h, KB_ERR_PARAM, "kb_steps(t0=%d): expected t0 = %d", t0, h->t_cur + 1);
  if (count == 0) return KB_OK;
  cudaSetDevice(h->device);
  const int nr = (int)h->runs.size();
  // steps between measurements run from one captured graph
  if (int rc = ensure_step_graph(h)) return rc;
  KB_CUDA(h, kb::launch_set_t(h->d_t, t0, h->st));
  int nm = 0;
  for (int i = 0; i < count; ++i) {
    const int t = t0 + i;
    NvtxRange range("kb_steps: step");
    if (h->profiling) {
      int rc = launch_step(h, 1);
      if (rc) return rc;
      KB_CUDA(h, kb::launch_advance_t(h->d_t, h->st));
    } else {
      KB_CUDA(h, cudaGraphLaunch(h->graph, h->st));
    }
    h->t_cur = t;
    if (measure_every > 0 && (t - 2) % measure_every == 0 && out) {
      for (int r = 0; r < nr; ++r) {
        const int idx = r * ((count + measure_every - 1) / measure_every) + nm;
        if (idx < out_capacity) {
          int rc = collect_scalars(h, r, t, &out[idx]);
          if (rc) return rc;
        }
      }
      ++nm;
    }
  }
  h->sigma_valid = h->any_nlo || h->any_ninv;
  return kb_sync(h);
}

// Device measurement stream: count steps from a captured graph that also
// appends the measurement of every measured step to a device buffer; one
// copy to the host at the end (createMeasurement records, Measurement.jl:31-99).
int kb_steps_recorded(kb_handle *h, int32_t t0, int32_t count, int32_t measure_every, kb_meas_scalars *out,
                      double *arrays, int32_t capacity, int32_t *n_recorded) {
  if (!h || count < 0 || measure_every < 1 || capacity < 0) return KB_ERR_PARAM;
  if (h->t_cur < 2) return fail(h, KB_ERR_PARAM, "kb_steps_recorded before kb_init");
  if (t0 != h->t_cur + 1)
    return fail(h, KB_ERR_PARAM, "kb_steps_recorded(t0=%d): expected t0 = %d", t0, h->t_cur + 1);
  if (n_recorded) *n_recorded = 0;
  if (count == 0) return KB_OK;
  cudaSetDevice(h->device);
  const int nr = (int)h->runs.size();
  // measured steps: (t - 2) % measure_every == 0 (the reference's NstepsbetweenNmeas)
  const int rem = ((t0 - 2) % measure_every + measure_every) % measure_every;
  const int tf = t0 + (rem == 0 ? 0 : measure_every - rem);
  const int t_last = t0 + count - 1;
  const int nmeas = (tf <= t_last) ? (t_last - tf) / measure_every + 1 : 0;
  if (nmeas > capacity)
    return fail(h, KB_ERR_PARAM, "kb_steps_recorded: %d measurements, capacity %d", nmeas, capacity);
  std::vector<long long> off(nr);
  long long block = 0;
  for (int r = 0; r < nr; ++r) {
    off[r] = block;
    block += 6 + 5LL * h->runs[r].S;
  }
  const size_t need = (size_t)std::max(1, nmeas) * (size_t)block;
  if (!h->d_rec_ctl) {
    if (cudaMalloc(&h->d_rec_ctl, 4 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&h->d_rec_off, sizeof(long long) * nr) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, KB_ERR_OOM, "kb_steps_recorded: cudaMalloc of the control block failed");
    }
    KB_CUDA(h, cudaMemcpy(h->d_rec_off, off.data(), sizeof(long long) * nr, cudaMemcpyHostToDevice));
  }
  if (need > h->rec_cap_doubles) {
    if (h->graph_rec) {  // the graph holds the old buffer's address
      cudaGraphExecDestroy(h->graph_rec);
      h->graph_rec = nullptr;
    }
    KB_CUDA(h, cudaStreamSynchronize(h->st));
    if (h->d_rec) cudaFree(h->d_rec);
    h->d_rec = nullptr;
    h->rec_cap_doubles = 0;
    if (cudaMalloc(&h->d_rec, need * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, KB_ERR_OOM, "kb_steps_recorded: cudaMalloc of %zu record bytes failed", need * sizeof(double));
    }
    h->rec_cap_doubles = need;
  }
  const int ctl[4] = {tf, measure_every, nmeas, 0};
  KB_CUDA(h, cudaMemcpyAsync(h->d_rec_ctl, ctl, sizeof ctl, cudaMemcpyHostToDevice, h->st));
  if (!h->graph_rec) {
    cudaGraph_t g;
    const bool prof = h->profiling;  // no profiling events inside the graph
    h->profiling = false;
    KB_CUDA(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    int rc = launch_step(h, 1);
    h->profiling = prof;
    cudaError_t ea = cudaSuccess;
    if (rc == 0) ea = kb::launch_record(h->d_runs, nr, h->d_t, h->d_rec_ctl, h->d_rec, h->d_rec_off, block, h->st);
    if (rc == 0 && ea == cudaSuccess) ea = kb::launch_advance_t(h->d_t, h->st);
    cudaError_t ec = cudaStreamEndCapture(h->st, &g);
    if (rc) return rc;
    if (ea != cudaSuccess || ec != cudaSuccess) return fail(h, KB_ERR_CUDA, "graph capture failed");
    cudaError_t ei = cudaGraphInstantiate(&h->graph_rec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return fail(h, KB_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(ei));
  }
  KB_CUDA(h, kb::launch_set_t(h->d_t, t0, h->st));
  for (int i = 0; i < count; ++i) {
    NvtxRange range("kb_steps_recorded: step");
    KB_CUDA(h, cudaGraphLaunch(h->graph_rec, h->st));
  }
  h->t_cur = t_last;
  h->sigma_valid = h->any_nlo || h->any_ninv;
  std::vector<double> host((size_t)nmeas * block);
  if (nmeas > 0)
    KB_CUDA(h, cudaMemcpyAsync(host.data(), h->d_rec, host.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  int rc = kb_sync(h);
  if (rc) return rc;
  size_t aoff = 0;
  for (int m = 0; m < nmeas; ++m)
    for (int r = 0; r < nr; ++r) {
      const double *rec = host.data() + (size_t)m * block + off[r];
      if (out) {
        kb_meas_scalars &o = out[(size_t)m * nr + r];
        o.time = rec[0];
        o.E = rec[1];
        o.E_pot = rec[2];
        o.E_kin = rec[3];
        o.E_mem = rec[4];
        o.M2 = rec[5];
      }
      const size_t n5 = 5 * (size_t)h->runs[r].S;
      if (arrays) std::memcpy(arrays + aoff, rec + 6, n5 * sizeof(double));
      aoff += n5;
    }
  if (n_recorded) *n_recorded = nmeas;
  return KB_OK;
}

int kb_get_stream(const kb_handle *h, void **stream) {
  if (!h || !stream) return KB_ERR_PARAM;
  *stream = (void *)h->st;
  return KB_OK;
}

int kb_profile(kb_handle *h, int32_t enable) {
  if (!h) return KB_ERR_PARAM;
  h->profiling = enable != 0;
  return KB_OK;
}

int kb_profile_read(kb_handle *h, double *ms, int64_t *launches) {
  if (!h) return KB_ERR_PARAM;
  cudaSetDevice(h->device);
  KB_CUDA(h, cudaStreamSynchronize(h->st));
  for (auto &p : h->ev_pending) {
    float v = 0.f;
    KB_CUDA(h, cudaEventElapsedTime(&v, p.second.first, p.second.second));
    h->prof_ms[p.first] += v;
    h->prof_n[p.first] += 1;
  }
  h->ev_pending.clear();
  h->ev_next = 0;
  for (int q = 0; q < 2; ++q) {
    if (ms) ms[q] = h->prof_ms[q];
    if (launches) launches[q] = h->prof_n[q];
    h->prof_ms[q] = 0;
    h->prof_n[q] = 0;
  }
  return KB_OK;
}

int kb_sync(kb_handle *h) {
  if (!h) return KB_ERR_PARAM;
  cudaSetDevice(h->device);
  KB_CUDA(h, cudaStreamSynchronize(h->st));
  int e = 0;
  KB_CUDA(h, cudaMemcpy(&e, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    // cleared on the handle's stream (non-blocking, so not ordered with the legacy
    // stream): every later kernel of this handle runs after the clear
    KB_CUDA(h, cudaMemsetAsync(h->d_err, 0, sizeof(int), h->st));
    KB_CUDA(h, cudaStreamSynchronize(h->st));
    return device_error(h, e);
  }
  return KB_OK;
}

// checkpoint layout: header + per run (hist_F, hist_r, sig_F, sig_r, st_F, st_r, tad, meas, epart)
struct CkptHeader {
  uint64_t magic, bytes;
  int32_t nruns, t_cur, fp64, sigma_valid;
  uint64_t shape;  // hash of every run's Ns, M, N, pexp and ring slots (ckpt_shape)
};
// runs of equal storage size can differ in M (the ring is rounded up to the tile) or
// in N, pexp: the shape hash tells a checkpoint of another handle from this one's
static uint64_t ckpt_shape(const kb_handle *h) {
  uint64_t x = 1469598103934665603ull;  // FNV-1a over the fields
  auto mix = [&](int64_t v) {
    for (int b = 0; b < 8; ++b) {
      x ^= (uint64_t)((v >> (8 * b)) & 0xff);
      x *= 1099511628211ull;
    }
  };
  for (const Run &R : h->runs) {
    mix(R.p.Ns);
    mix(R.p.M);
    mix(R.p.N);
    mix(R.p.pexp);
    mix(R.p.flags & 0xffff);
    mix(R.Malloc);
  }
  return x;
}
static const uint64_t kCkptMagic = 0x6b623270692d636bull;

int kb_checkpoint_size(const kb_handle *h, size_t *bytes) {
  if (!h || !bytes) return KB_ERR_PARAM;
  size_t b = sizeof(CkptHeader);
  for (const Run &R : h->runs) {
    b += (2 * R.hist_elems + 2 * R.sig_elems) * R.esz + 2 * R.st_elems * 8 + (2 * R.nchunks + 5 * R.Spad + 4 * R.nchunks) * 8;
    if (R.pi_r) b += (2 * R.hist_elems + 2 * (size_t)R.Malloc * R.Spad) * 8;
  }
  *bytes = b;
  return KB_OK;
}

static int ckpt_copy(kb_handle *h, char *host, size_t bytes, bool save) {
  size_t need = 0;
  kb_checkpoint_size(h, &need);
  if (bytes < need) return fail(h, KB_ERR_PARAM, "checkpoint buffer of %zu bytes, need %zu", bytes, need);
  cudaSetDevice(h->device);
  int rc = kb_sync(h);
  if (rc) return rc;
  CkptHeader hd{kCkptMagic, need, (int32_t)h->runs.size(), h->t_cur, h->fp64 ? 1 : 0, h->sigma_valid ? 1 : 0,
                ckpt_shape(h)};
  if (save) {
    std::memcpy(host, &hd, sizeof hd);
  } else {
    CkptHeader in;
    std::memcpy(&in, host, sizeof in);
    if (in.magic != kCkptMagic || in.bytes != need || in.nruns != hd.nruns || in.fp64 != hd.fp64 ||
        in.shape != hd.shape)
      return fail(h, KB_ERR_PARAM, "checkpoint does not match this handle");
    hd = in;
  }
  size_t off = sizeof hd;
  for (Run &R : h->runs) {
    struct B { void *d; size_t n; } bufs[] = {
        {R.hist_F, R.hist_elems * R.esz}, {R.hist_r, R.hist_elems * R.esz}, {R.sig_F, R.sig_elems * R.esz},
        {R.sig_r, R.sig_elems * R.esz},   {R.st_F, R.st_elems * 8},         {R.st_r, R.st_elems * 8},
        {R.tad, (size_t)2 * R.nchunks * 8}, {R.meas, (size_t)5 * R.Spad * 8}, {R.epart, (size_t)4 * R.nchunks * 8},
    };
    std::vector<B> bl(std::begin(bufs), std::end(bufs));
    if (R.pi_r) {
      bl.push_back({R.pi_r, R.hist_elems * 8});
      bl.push_back({R.pi_F, R.hist_elems * 8});
      bl.push_back({R.Ik, (size_t)R.Malloc * R.Spad * 8});
      bl.push_back({R.Jk, (size_t)R.Malloc * R.Spad * 8});
    }
    for (auto &q : bl) {
      if (save) KB_CUDA(h, cudaMemcpyAsync(host + off, q.d, q.n, cudaMemcpyDeviceToHost, h->st));
      else KB_CUDA(h, cudaMemcpyAsync(q.d, host + off, q.n, cudaMemcpyHostToDevice, h->st));
      off += q.n;
    }
  }
  KB_CUDA(h, cudaStreamSynchronize(h->st));
  if (!save) {
    h->t_cur = hd.t_cur;
    h->sigma_valid = hd.sigma_valid != 0;
  }
  return KB_OK;
}

int kb_checkpoint_save(kb_handle *h, void *buf, size_t bytes) {
  if (!h || !buf) return KB_ERR_PARAM;
  return ckpt_copy(h, (char *)buf, bytes, true);
}
int kb_checkpoint_restore(kb_handle *h, const void *buf, size_t bytes) {
  if (!h || !buf) return KB_ERR_PARAM;
  return ckpt_copy(h, (char *)const_cast<void *>(buf), bytes, false);
}

// ---------------------------------------------------------------------------
// Tuning: launch configuration of the two step kernels, and an autotuner that
// times candidates by re-running the last step (idempotent: step t reads rows
// < t, the FP64 state rows t-1, t-2 and the tadpole sums of t-1, and rewrites
// row t, Sigma(t-1, .), the tadpole sums of t and the measurement).
int kb_get_tuning(const kb_handle *h, kb_tuning *out) {
  if (!h || !out) return KB_ERR_PARAM;
  *out = kb_tuning{};
  out->memint_variant = h->memint_variant;
  out->memint_compensated = h->memint_compensated;
  out->batch_overlap = h->batch_overlap;
  out->sunset_grid = h->grid_sun;
  out->batch_order = h->batch_order;
  out->sunset_variant = h->sunset_variant;
  out->memint_split = h->memint_split;
  out->memint_persistent = h->memint_persistent;
  out->memint_bulk = h->memint_bulk;
  out->test_no_tiles = h->test_no_tiles;
  return KB_OK;
}

int kb_set_tuning(kb_handle *h, const kb_tuning *in) {
  if (!h || !in) return KB_ERR_PARAM;
  if (in->memint_variant < 0 || in->memint_variant > 2 || (h->fp64 && in->memint_variant != 0))
    return fail(h, KB_ERR_PARAM, "memint_variant=%d: 0, 1 or 2, and 0 for KB_PREC_FP64", in->memint_variant);
  const int g = in->sunset_grid == 0 ? kb::sunset_grid(h->fp64, h->num_sms, h->total_sun) : in->sunset_grid;
  if (g < 1 || g > h->grid_sun_max)
    return fail(h, KB_ERR_PARAM, "sunset_grid=%d: at most %d CTAs fit on this device", in->sunset_grid,
                h->grid_sun_max);
  if (in->sunset_variant < 0 || in->sunset_variant > 2 || (h->fp64 && in->sunset_variant != 0))
    return fail(h, KB_ERR_PARAM, "sunset_variant=%d: 0, 1 or 2, and 0 for KB_PREC_FP64", in->sunset_variant);
  if (in->sunset_variant == 2 && h->smem_sun_tc == 0)
    return fail(h, KB_ERR_PARAM, "sunset_variant=2: the tensor-core sunset takes Ns <= 78 and needs its shared memory");
  if (in->sunset_grid != 0 &&
      in->sunset_grid > h->num_sms * kb::sunset_max_ctas_per_sm(h->fp64, in->sunset_variant, h->smem_sun) * 4)
    return fail(h, KB_ERR_PARAM, "sunset_grid=%d: too large for this variant", in->sunset_grid);
  if (in->memint_split < 0 || in->memint_split > 2 || (in->memint_split && !h->fp64 && in->memint_variant == 0))
    return fail(h, KB_ERR_PARAM, "memint_split=%d: 0, 1 or 2, and 1, 2 only with memint_variant 1 or 2 in KB_PREC_MIXED",
                in->memint_split);
  if (in->memint_persistent < 0 || in->memint_persistent > 1 ||
      (in->memint_persistent && !h->fp64 && in->memint_variant == 0))
    return fail(h, KB_ERR_PARAM,
                "memint_persistent=%d: 0 or 1, and 1 only with memint_variant 1 or 2 in KB_PREC_MIXED",
                in->memint_persistent);
  if (in->batch_order < 0 || in->batch_order > 1)
    return fail(h, KB_ERR_PARAM, "batch_order=%d: 0 (runs in order) or 1 (costliest first)", in->batch_order);
  if (in->memint_bulk < 0 || in->memint_bulk > 1)
    return fail(h, KB_ERR_PARAM, "memint_bulk=%d: 0 (tensor-map boxes) or 1 (bulk copies)", in->memint_bulk);
  if (in->test_no_tiles < 0 || in->test_no_tiles > 1)
    return fail(h, KB_ERR_PARAM, "test_no_tiles=%d: 0 or 1", in->test_no_tiles);
  if (in->memint_compensated < 0 || in->memint_compensated > 1 ||
      (in->memint_compensated && (h->fp64 || in->memint_variant != 2)))
    return fail(h, KB_ERR_PARAM, "memint_compensated=%d: 0 or 1, and 1 only with memint_variant 2 in KB_PREC_MIXED",
                in->memint_compensated);
  if (in->batch_overlap < 0 || in->batch_overlap >= h->num_sms ||
      (in->batch_overlap > 0 && (h->runs.size() < 2 || h->any_ninv)))
    return fail(h, KB_ERR_PARAM,
                "batch_overlap=%d: 0, or the CTAs (below the SM count %d) of the second group's sunset in a "
                "batch of two or more runs without the 1/N expansion",
                in->batch_overlap, h->num_sms);
  cudaSetDevice(h->device);
  int rc = kb_sync(h);
  if (rc) return rc;
  if ((rc = set_overlap(h, in->batch_overlap, in->batch_order))) return rc;
  h->memint_variant = in->memint_variant;
  h->memint_compensated = in->memint_compensated;
  h->memint_split = in->memint_split;
  h->memint_persistent = in->memint_persistent;
  h->memint_bulk = in->memint_bulk;
  h->test_no_tiles = in->test_no_tiles;
  h->sunset_variant = in->sunset_variant;
  h->grid_sun = g;
  if (h->graph) {  // captured with the old configuration
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  if (h->graph_rec) {
    cudaGraphExecDestroy(h->graph_rec);
    h->graph_rec = nullptr;
  }
  return KB_OK;
}

int kb_autotune(kb_handle *h, int32_t trials, kb_tuning *chosen, double *ms_per_step) {
  if (!h || trials < 1) return KB_ERR_PARAM;
  if (h->t_cur < 3) return fail(h, KB_ERR_PARAM, "kb_autotune needs an evolved step (t >= 3)");
  cudaSetDevice(h->device);
  int rc = kb_sync(h);
  if (rc) return rc;
  const int t = h->t_cur;
  // the kernel candidates are timed on the one-launch schedule; the concurrent-group
  // step of a batch is timed afterwards, on whole steps, with the chosen kernels
  if ((rc = set_overlap(h, 0, h->batch_order))) return rc;
  cudaEvent_t e[3];
  for (auto &x : e) KB_CUDA(h, cudaEventCreate(&x));
  auto time_cfg = [&](int variant, int split, int pers, int svar, int grid, float *ms_sun, float *ms_mi) -> int {
    h->memint_variant = variant;
    h->memint_split = split;
    h->memint_persistent = pers;
    h->sunset_variant = svar;
    h->grid_sun = grid;
    float best_s = 1e30f, best_m = 1e30f;
    for (int q = 0; q < trials; ++q) {
      KB_CUDA(h, kb::launch_set_t(h->d_t, t, h->st));
      KB_CUDA(h, cudaEventRecord(e[0], h->st));
      if ((rc = launch_self_energies(h))) return rc;
      KB_CUDA(h, cudaEventRecord(e[1], h->st));
      if ((rc = launch_mi(h, h->d_base_mi, (int)h->runs.size(), h->total_mi, 1, h->st, 0, h->num_sms))) return rc;
      KB_CUDA(h, cudaEventRecord(e[2], h->st));
      KB_CUDA(h, cudaEventSynchronize(e[2]));
      float a = 0, b = 0;
      KB_CUDA(h, cudaEventElapsedTime(&a, e[0], e[1]));
      KB_CUDA(h, cudaEventElapsedTime(&b, e[1], e[2]));
      best_s = std::min(best_s, a);
      best_m = std::min(best_m, b);
    }
    *ms_sun = best_s;
    *ms_mi = best_m;
    return KB_OK;
  };
  // sunset variants x grids of 1..4 resident CTAs per SM; memint (variant,
  // split): the whole or split two-group kernel, and for FP32 the
  // register-blocked one; run orders: batched handles only
  std::vector<std::pair<int, int>> sun_cands;  // (variant, grid)
  for (int sv = 0; sv < (h->fp64 ? 1 : 2); ++sv) {
    const int occ = std::min(4, kb::sunset_max_ctas_per_sm(h->fp64, sv, h->smem_sun));
    int last = -1;
    for (int k = 1; k <= occ; ++k) {
      const int g = std::min(h->total_sun, k * h->num_sms);
      if (g <= h->grid_sun_max && g != last) sun_cands.push_back({sv, g});
      last = g;
    }
  }
  if (!h->fp64 && h->smem_sun_tc) sun_cands.push_back({2, std::min(h->total_sun, h->num_sms)});  // tensor cores
  if (sun_cands.empty()) sun_cands.push_back({h->sunset_variant, h->grid_sun});
  const int norder = h->runs.size() > 1 ? 2 : 1;
  // the one-kernel FP64 or the two-group FP32 memint, whole chunks, first; compensated
  // tile sums exist for the leapfrog-warp kernel only, so with them it is the one timed
  const int v0 = h->fp64 ? 0 : (h->memint_compensated ? 2 : 1);
  std::vector<std::pair<int, int>> mi_cands = {{v0, 1}};  // (variant, split) after (v0, 0)
  if (h->total_mi > h->num_sms && h->total_mi % h->num_sms) mi_cands.push_back({v0, 2});
  if (!h->fp64 && !h->memint_compensated) {
    mi_cands.push_back({0, 0});
    // whole chunks with their leapfrog on the leapfrog warps: alone, or for the whole waves
    mi_cands.push_back({2, 0});
    if (h->total_mi > h->num_sms && h->total_mi % h->num_sms) mi_cands.push_back({2, 2});
  }
  int best_o = h->batch_order, best_v = v0, best_split = 0, best_pers = 0;
  std::pair<int, int> best_sc = sun_cands[0];
  float best_total = 1e30f, best_s_all = 0, best_m_all = 0;
  for (int o = 0; o < norder && !rc; ++o) {
    const int order = (norder == 1) ? h->batch_order : o;
    if (order != h->batch_order && apply_schedule(h, order) != KB_OK) {
      rc = fail(h, KB_ERR_CUDA, "upload of the run schedule failed");
      break;
    }
    std::pair<int, int> sc_o = sun_cands[0];
    int v_o = v0, sp_o = 0, pe_o = 0;
    float bs = 1e30f, bm = 1e30f;
    for (size_t q = 0; q < sun_cands.size(); ++q) {
      float ms_s, ms_m;
      if ((rc = time_cfg(v0, 0, 0, sun_cands[q].first, sun_cands[q].second, &ms_s, &ms_m))) break;
      if (ms_s < bs) { bs = ms_s; sc_o = sun_cands[q]; }
      if (q == 0) bm = ms_m;
    }
    for (size_t q = 0; q < mi_cands.size() && !rc; ++q) {
      float ms_s, ms_m;
      if ((rc = time_cfg(mi_cands[q].first, mi_cands[q].second, 0, sc_o.first, sc_o.second, &ms_s, &ms_m))) break;
      if (ms_m < bm) { bm = ms_m; v_o = mi_cands[q].first; sp_o = mi_cands[q].second; }
    }
    // the chosen memory-integral kernel once more as a persistent grid (one CTA per SM
    // taking items from a queue)
    if (!rc && (h->fp64 || v_o != 0)) {
      float ms_s, ms_m;
      if (!(rc = time_cfg(v_o, sp_o, 1, sc_o.first, sc_o.second, &ms_s, &ms_m)) && ms_m < bm) {
        bm = ms_m;
        pe_o = 1;
      }
    }
    if (!rc && bs + bm < best_total) {
      best_total = bs + bm;
      best_o = order;
      best_sc = sc_o;
      best_v = v_o;
      best_split = sp_o;
      best_pers = pe_o;
      best_s_all = bs;
      best_m_all = bm;
    }
  }
  if (rc) {
    for (auto &x : e) cudaEventDestroy(x);
    return rc;
  }
  if (best_o != h->batch_order && apply_schedule(h, best_o) != KB_OK)
    return fail(h, KB_ERR_CUDA, "upload of the run schedule failed");
  h->memint_variant = best_v;
  h->memint_split = best_split;
  h->memint_persistent = best_pers;
  h->sunset_variant = best_sc.first;
  h->grid_sun = best_sc.second;
  // batches: whole steps without and with the concurrent groups (second group's sunset
  // on a quarter, a third or half of the SMs)
  if (h->runs.size() >= 2 && !h->any_ninv) {
    int best_ov = 0;
    float best_step = 1e30f;
    const int cands[4] = {0, h->num_sms / 4, h->num_sms / 3, h->num_sms / 2};
    for (int ov : cands) {
      if (ov < 0 || (ov == 0 && best_step < 1e30f)) continue;
      if ((rc = set_overlap(h, ov, best_o))) break;
      // the step as kb_steps runs it, one launch of a captured graph: stream priorities do
      // not carry into a graph, so the two-stream step is timed the way it will run
      cudaGraph_t gr = nullptr;
      cudaGraphExec_t ge = nullptr;
      KB_CUDA(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
      rc = launch_step(h, 1);
      const cudaError_t ec = cudaStreamEndCapture(h->st, &gr);
      if (!rc && ec != cudaSuccess) rc = fail(h, KB_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
      if (!rc) {
        const cudaError_t ei = cudaGraphInstantiate(&ge, gr, 0);
        if (ei != cudaSuccess) rc = fail(h, KB_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(ei));
      }
      if (gr) cudaGraphDestroy(gr);
      float best = 1e30f;
      for (int q = 0; q < trials && !rc; ++q) {
        KB_CUDA(h, kb::launch_set_t(h->d_t, t, h->st));
        KB_CUDA(h, cudaEventRecord(e[0], h->st));
        KB_CUDA(h, cudaGraphLaunch(ge, h->st));
        KB_CUDA(h, cudaEventRecord(e[2], h->st));
        KB_CUDA(h, cudaEventSynchronize(e[2]));
        float a = 0;
        KB_CUDA(h, cudaEventElapsedTime(&a, e[0], e[2]));
        best = std::min(best, a);
      }
      if (ge) cudaGraphExecDestroy(ge);
      if (rc) break;
      // concurrent groups must win clearly: a repeated launch of one step flatters them
      // (64 uneven runs: 7.08 ms timed this way, 7.42 ms in consecutive steps)
      if (best < best_step * (ov ? 0.97f : 1.0f)) {
        best_step = best;
        best_ov = ov;
      }
    }
    if (!rc) rc = set_overlap(h, best_ov, best_o);
    if (!rc && best_step < 1e30f) {
      best_s_all = 0.0f;
      best_m_all = best_step;
    }
  }
  for (auto &x : e) cudaEventDestroy(x);
  if (rc) return rc;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  if (h->graph_rec) {
    cudaGraphExecDestroy(h->graph_rec);
    h->graph_rec = nullptr;
  }
  // step t once more with the chosen kernels, so the state is theirs
  KB_CUDA(h, kb::launch_set_t(h->d_t, t, h->st));
  if ((rc = launch_step(h, 1))) return rc;
  if ((rc = kb_sync(h))) return rc;
  if (chosen) kb_get_tuning(h, chosen);
  if (ms_per_step) *ms_per_step = (double)(best_s_all + best_m_all);
  return KB_OK;
}

// ---------------------------------------------------------------------------
// kb_adjoint: forward run with device state copies every ckpt_every steps,
// then blocks of ckpt_every steps recomputed from their copy and reversed
// (kernels in kb_adjoint.cu). The ring keeps ckpt_every slots beyond the window
// so that a recomputed block leaves the rows of its first reverse step intact.
int kb_adjoint(kb_handle *h, const double *n_init, double init_mass, int32_t t_final, const double *w_n, double w_E,
               int32_t ckpt_every, double *grad_lambda, double *grad_mass2, double *grad_n, double *grad_init_mass,
               double *loss) {
  if (!h) return KB_ERR_PARAM;
  if (!n_init || !grad_lambda || !grad_mass2 || !grad_n) return fail(h, KB_ERR_PARAM, "kb_adjoint: null argument");
  if (h->runs.size() != 1) return fail(h, KB_ERR_PARAM, "kb_adjoint: the handle must hold a single run");
  if (!h->fp64) return fail(h, KB_ERR_PARAM, "kb_adjoint: needs a KB_PREC_FP64 handle");
  if (h->runs[0].p.pexp > KB_PEXP_NLO_CLASSICAL)
    return fail(h, KB_ERR_PARAM, "kb_adjoint: the 1/N expansion has no adjoint (lambda expansion only)");
  if (t_final < 3) return fail(h, KB_ERR_PARAM, "kb_adjoint: t_final=%d must be >= 3", t_final);
  Run &R = h->runs[0];
  const int k = ckpt_every;
  if (k < 1 || R.Malloc - R.p.M < k)
    return fail(h, KB_ERR_PARAM,
                "kb_adjoint: ckpt_every=%d needs a handle created with kb_params.flags >= %d extra ring slots "
                "(this one keeps %d)", k, std::max(k, 1), R.Malloc - R.p.M);
  if (!std::isfinite(w_E)) return fail(h, KB_ERR_PARAM, "kb_adjoint: non-finite w_E");
  cudaSetDevice(h->device);
  int rc = kb_sync(h);
  if (rc) return rc;
  h->t_cur = 0;  // the state is consumed from here on
  h->sigma_valid = false;
  const RunDev &D = R.dev;
  const int nsnap = (t_final - 2 + k - 1) / k;  // state copies at t = 2, 2 + k, ... < t_final
  struct Part { void *d; size_t n; } parts[] = {
      {R.hist_F, R.hist_elems * 8}, {R.hist_r, R.hist_elems * 8}, {R.st_F, R.st_elems * 8},
      {R.st_r, R.st_elems * 8},     {R.tad, (size_t)2 * R.nchunks * 8},
  };
  size_t snap_bytes = 0;
  for (auto &q : parts) snap_bytes += (q.n + 255) / 256 * 256;
  const size_t adj_bytes = kb::adjoint_buffer_bytes(D);
  // Sigma(t-1, .) of the steps of one block, kept when the forward step computes
  // them (both rings, FP64), so that the reverse steps need not run the sunset again
  const bool nlo = kb::pexp_sunset(R.p.pexp);
  const size_t sig_bytes = R.sig_elems * R.esz;
  char *snaps = nullptr, *adj = nullptr, *sigs = nullptr;
  double *d_vec = nullptr;  // w_n [Spad], n_init [Spad], output [2][S]
  auto release = [&]() {
    cudaStreamSynchronize(h->st);
    if (snaps) cudaFree(snaps);
    if (adj) cudaFree(adj);
    if (sigs) cudaFree(sigs);
    if (d_vec) cudaFree(d_vec);
    cudaGetLastError();
  };
  if (cudaMalloc((void **)&snaps, snap_bytes * nsnap) != cudaSuccess ||
      cudaMalloc((void **)&adj, adj_bytes) != cudaSuccess ||
      (nlo && cudaMalloc((void **)&sigs, 2 * sig_bytes * k) != cudaSuccess) ||
      cudaMalloc((void **)&d_vec, (size_t)(2 * R.Spad + 2 * R.S) * 8) != cudaSuccess) {
    release();
    return fail(h, KB_ERR_OOM, "kb_adjoint: cudaMalloc of %zu + %zu + %zu bytes (state copies, adjoint, Sigma) failed",
                snap_bytes * nsnap, adj_bytes, nlo ? 2 * sig_bytes * k : (size_t)0);
  }
  auto copy_sigma = [&](int slot, bool save) -> int {  // slot: the step's place in its block
    char *s = sigs + (size_t)slot * 2 * sig_bytes;
    KB_CUDA(h, cudaMemcpyAsync(save ? s : R.sig_F, save ? R.sig_F : s, sig_bytes, cudaMemcpyDeviceToDevice, h->st));
    KB_CUDA(h, cudaMemcpyAsync(save ? s + sig_bytes : R.sig_r, save ? R.sig_r : s + sig_bytes, sig_bytes,
                               cudaMemcpyDeviceToDevice, h->st));
    return KB_OK;
  };
  auto copy_state = [&](int i, bool save) -> int {
    size_t off = 0;
    for (auto &q : parts) {
      char *dev = snaps + (size_t)i * snap_bytes + off;
      KB_CUDA(h, cudaMemcpyAsync(save ? dev : q.d, save ? q.d : dev, q.n, cudaMemcpyDeviceToDevice, h->st));
      off += (q.n + 255) / 256 * 256;
    }
    return KB_OK;
  };
  kb::AdjBuffers A{};
  kb::adjoint_carve(D, adj, &A);
  double *d_wn = d_vec, *d_n0 = d_vec + R.Spad, *d_out = d_vec + 2 * R.Spad;
  auto run = [&]() -> int {
    KB_CUDA(h, cudaMemsetAsync(adj, 0, adj_bytes, h->st));
    if (w_n) KB_CUDA(h, cudaMemcpyAsync(d_wn, w_n, R.S * 8, cudaMemcpyHostToDevice, h->st));
    KB_CUDA(h, cudaMemcpyAsync(d_n0, n_init, R.S * 8, cudaMemcpyHostToDevice, h->st));
    // forward, keeping the state copies
    int r = kb_init(h, 0, n_init, init_mass);
    if (r) return r;
    if ((r = copy_state(0, true))) return r;
    const int s0_last = 2 + (nsnap - 1) * k;  // the last block is reversed from this forward pass
    for (int t = 3; t <= t_final; ++t) {
      if ((r = kb_step(h, t))) return r;
      if ((t - 2) % k == 0 && t < t_final && (r = copy_state((t - 2) / k, true))) return r;
      if (nlo && t > s0_last && (r = copy_sigma(t - s0_last - 1, true))) return r;
    }
    if (loss) {  // L at t_final from the forward measurement
      kb_meas_scalars ms{};
      std::vector<double> nv(R.S);
      if ((r = kb_measure(h, 0, t_final, &ms, nullptr, nullptr, nv.data(), nullptr, nullptr))) return r;
      double L = w_E * ms.E;
      if (w_n)
        for (int q = 0; q < R.S; ++q) L += w_n[q] * nv[q];
      *loss = L;
    }
    const double N = (double)R.p.N;
    const double dpref_ivol = (N + 2.0) / (6.0 * N) * D.ivol;  // d(pref ivol)/dlambda
    KB_CUDA(h, kb::launch_adjoint_seed(D, A, t_final, w_n ? d_wn : nullptr, w_E, dpref_ivol, h->st));
    const kb::SunsetLaunch sl{h->d_runs, h->d_base_sun, 1, h->total_sun, h->grid_sun, h->d_t,
                              h->sun_scratch, h->sun_scratch_stride, h->smem_sun};
    for (int i = nsnap - 1; i >= 0; --i) {
      const int s0 = 2 + i * k, e = std::min(s0 + k, t_final);
      if (i != nsnap - 1) {  // recompute the block from its copy
        if ((r = copy_state(i, false))) return r;
        h->t_cur = s0;
        for (int t = s0 + 1; t <= e; ++t) {
          if ((r = kb_step(h, t))) return r;
          if (nlo && (r = copy_sigma(t - s0 - 1, true))) return r;
        }
      }
      for (int t = e; t > s0; --t) {
        if (nlo && (r = copy_sigma(t - s0 - 1, false))) return r;
        KB_CUDA(h, kb::launch_adjoint_step(D, A, t, t == t_final ? w_E : 0.0, R.p.lambda, dpref_ivol, sl,
                                           h->num_sms, nlo, h->st));
      }
    }
    KB_CUDA(h, kb::launch_adjoint_init_grad(D, A, d_n0, init_mass, d_out, h->st));
    double scal[8];
    std::vector<double> out((size_t)2 * R.S);
    KB_CUDA(h, cudaMemcpyAsync(scal, A.scal, sizeof scal, cudaMemcpyDeviceToHost, h->st));
    KB_CUDA(h, cudaMemcpyAsync(out.data(), d_out, out.size() * 8, cudaMemcpyDeviceToHost, h->st));
    if ((r = kb_sync(h))) return r;
    *grad_mass2 = scal[2];
    *grad_lambda = scal[3];
    std::copy(out.begin(), out.begin() + R.S, grad_n);
    if (grad_init_mass) {
      double gm = 0.0;
      for (int q = 0; q < R.S; ++q) gm += out[R.S + q];
      *grad_init_mass = gm;
    }
    if (!std::isfinite(*grad_lambda) || !std::isfinite(*grad_mass2))
      return fail(h, KB_ERR_NAN, "kb_adjoint: non-finite gradient");
    return KB_OK;
  };
  rc = run();
  release();
  h->t_cur = 0;
  h->sigma_valid = false;
  return rc;
}

}  // extern "C"
