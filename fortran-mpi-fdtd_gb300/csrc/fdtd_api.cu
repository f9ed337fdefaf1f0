// fdtd_api.cu -- the C ABI of include/fdtd_gb300.h: job set-up, device
// state, and the launch sequence of the time loop.
//
// The host side does what the reference does once before its time loop
// (material ranges, PML profiles, gold coefficients: all in FP64, with the
// reference's formulas and operation order) and then only launches kernels.
// There is no CPU compute path: without an sm_103 device every call that
// needs one fails with FDTD_ENODEV.
//
// Sections, in order: the job record and its device allocations (state
// buffers registered for checkpoints); PML coefficient tables; commit
// (material painting, dispersive coefficients and slots, PML, rows, the core
// and edge split, the uniformity bitmap, sampling tables, the tensor maps of
// the TMA-staged core, the block-shape tuner); stepping (the parts of a half
// step, their streams and programmatic dependencies, the DFT ring, CUDA-graph
// replay, the 1D line); packs of small 2D jobs; the C entry points, with the
// health checks and the checkpoint after the getters.
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fdtd_gb300.h"
#include "fdtd_internal.h"
#include "hostscan.h"

using namespace fdtd;

// an NVTX range over a host entry point: profilers (ncu --nvtx, nsys) can
// pick the engine's calls by name; without a profiler attached it costs a
// predictable branch
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

namespace {

thread_local std::string g_last_error;

int set_err(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return set_err(FDTD_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));  \
  } while (0)

// Mm/constants_mod.f90:3-7
struct Consts {
  double pi, ep0, mu0, c0, z0;
  Consts() {
    pi = 4.0 * std::atan(1.0);
    ep0 = 8.85418781762039e-12;
    mu0 = pi * 4e-7;
    c0 = 1.0 / std::sqrt(ep0 * mu0);
    z0 = std::sqrt(mu0 / ep0);
  }
};
const Consts K;

struct MatRec {
  int kind;  // MK_*
  double eps;
  fdtd_drude2cp gold;
  fdtd_graphene_desc gr;
  fdtd_lorentz_desc lz;
  fdtd_graphene_cp_desc gcp;
  double sigma;  // conductive dielectric: eps holds eps_inf
  fdtd_graphene_nk_desc gnk;
  fdtd_region region;
  std::vector<double> centers;
  std::vector<uint8_t> mask;
};

struct MonRec {
  fdtd_monitor_desc d;
  std::vector<double> omega;
  int ncomp;
  int comps[6];
  long long ncell;     // transformed samples per component (1 for a mean monitor)
  long long boxcells;  // cells of the box
};

struct ProbeRec {
  fdtd_probe_desc d;
  int ncomp;
  int comps[8];
  double *buf = nullptr;
  int cap = 0;
};

int comp_list(int mask, int *out, int maxn) {
  int n = 0;
  for (int c = 0; c < 8; ++c)
    if (mask & (1 << c)) {
      if (n >= maxn) return -1;
      out[n++] = c;
    }
  return n;
}

}  // namespace

struct fdtd_job {
  fdtd_grid_desc g{};
  int dim = 0;
  int nx = 1, ny = 1, nz = 1;
  long long ncell = 0;
  size_t esz = 8;
  std::vector<MatRec> mats;
  bool has_pml = false;
  fdtd_pml_desc pml{};
  bool has_tfsf = false;
  fdtd_tfsf1d_desc tfsf{};
  bool has_tfbox = false;        // 2D/3D total-field/scattered-field box
  fdtd_tfsf_desc tfbox{};
  int tb_face[3] = {0, 0, 0};
  void *d_tf_abc = nullptr;
  std::vector<fdtd_source_desc> srcs;
  std::vector<MonRec> mons;
  std::vector<ProbeRec> probes;
  bool committed = false;
  int device = 0;
  int num_sms = 152;
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  // the buffers a step changes (fields, split parts, slabs, dispersive
  // state, DFT sums and ring): what a checkpoint holds, in allocation order
  struct StateBuf {
    void *p;
    size_t bytes;
    int esz;  // element size: 4 float, 8 double
  };
  std::vector<StateBuf> state;
  uint64_t dev_bytes = 0;
  // device state
  void *F[8] = {};  // ex ey ez hx hy hz ex_inc hz_inc
  uint8_t *d_mat = nullptr;
  void *d_mc = nullptr, *d_ac = nullptr, *d_mca = nullptr, *d_mcs = nullptr;
  uint8_t *d_rowflag = nullptr;
  uint32_t *d_uni = nullptr;  // per x-vector: all ids id0 (see StepParams::uni)
  int uni_words = 0;
  int nade = 0, ade_stride = 0, ade_nf = 0, id0 = 0;
  std::vector<double> mca_host;
  std::vector<char> ac_host;  // AdeCoef<T> table, host copy
  int ade_kind = -1;          // the device kind of every dispersive material, or -1 (mixed)
  int *d_ade_cell = nullptr;
  uint8_t *d_ade_mat = nullptr;
  void *d_ade_state = nullptr;
  int slo[3] = {0, 0, 0}, shi[3] = {0, 0, 0};
  void *d_cf[4][3] = {};   // f1 f2 g1 g2 per axis (split PML)
  void *d_sp[12] = {};
  int slab_rows = 0, slab_on[2] = {0, 0}, slab_j0[2] = {0, 0};
  void *d_slab[2][12] = {};
  void *d_sc[2][12] = {};  // sf1x sf2x sg1x sg2x sf1y sf2y sg1y sg2y sf1z sf2z sg1z sg2z
  // 1D line slabs [line][side]
  void *d_lex[2][2] = {}, *d_lhz[2][2] = {}, *d_lc[2][2][4] = {};
  int ja = -1, jb = -1;
  // sampling
  std::vector<Monitor> mon_dev;
  long long stage_row = 0;
  void *d_stage = nullptr;
  long long stage_cap_rows = 0;
  int stage_fill = 0, stage_n0 = 1;
  // 2D/3D: the stage buffer holds two rings.  A replayed ring writes one half
  // while its graph folds the ring before it, from the other half, beside its
  // first steps; the last ring's fold runs when the replays end.
  int stage_half = 0;        // the half the current ring writes
  bool fold_pending = false; // a replayed ring whose fold has not run yet
  int pending_half = 0, pending_n0 = 0;
  int *d_half = nullptr, *d_gate = nullptr;  // the ring's half and the fold's gate, on the device
  cudaStream_t fold_stream = nullptr;
  cudaEvent_t ev_ffork = nullptr, ev_fjoin = nullptr;
  double *d_omega = nullptr, *d_acc_re = nullptr, *d_acc_im = nullptr;
  double *d_rot = nullptr;  // per frequency and ring slot: cos, sin of w s dt
  double *d_mean_part = nullptr;   // mean monitors: partial sums per block
  unsigned *d_mean_ctr = nullptr;  // mean monitors: blocks done per component
  long long acc_total = 0;
  bool gather_fused = true;
  int dft_blocks = 0;
  // 1D per-launch source values
  double *d_srcval = nullptr;
  long long srcval_cap = 0;
  // 2D/3D: amp*g(t) of every step, [(n-1)*nsrc + q], on the device
  std::vector<double> srctab;
  double *d_srctab = nullptr;
  long long srctab_steps = 0, srctab_cap_steps = 0;
  int nsrc_dev = 0;
  // CUDA graph of one ring of kStageSteps steps + its DFT fold
  int *d_base = nullptr;
  unsigned long long *d_count = nullptr;  // fdtd_check_finite
  // the TMA-staged 3D E core: tensor maps of Hx, Hy, Hz, and the flag its
  // bounded waits set when they give up
  TmaMaps tma{};
  bool tma_ok = false;
  // the fused step kernels (FP32): a second set of field buffers Fb (and of
  // the stored split-PML parts, spb, in 2D), the two sets taking turns as
  // step n and step n+1 (pp: the set that holds the current step inside
  // fdtd_step; 0, the canonical F, between calls), and in 3D the tensor maps
  // of each set's H arrays
  bool fused_ok = false;
  void *Fb[6] = {};
  void *spb[3] = {};
  int pp = 0;
  FusedMaps fmaps[2]{};
  int *d_err = nullptr;
  unsigned wait_limit = kWaitLimit;  // polls of a TMA core's mbarrier wait (fdtd_debug_wait_limit)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_kernels = 0;
  bool use_graph = true;
  int last_n = 0;
  // profiling
  bool prof = false;
  struct EvPair { cudaEvent_t a, b; int kind; };
  std::vector<EvPair> pending;
  std::vector<cudaEvent_t> ev_pool;
  long long kcount[FDTD_KERNEL_COUNT] = {};
  double kms[FDTD_KERNEL_COUNT] = {};
  long long launches = 0;
  cudaStream_t own_stream = nullptr;
  uint64_t h2d = 0, d2h = 0;
  // 2D work split (core box + edge unit list) and the streams that run the
  // parts of a half step as parallel branches of the job's stream
  int vec = 1, cv0 = 0, cw = 0, cy0 = 0, ncore = 0, nedge = 0;
  int ch = 0, cz0 = 0, cd = 0;  // 3D: core box rows and planes
  int tile_req = 0, tile = 1;    // core block shape: requested (0: tune) and used
  int *d_edge = nullptr;
  cudaStream_t side[2] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[2] = {};
  // programmatic events of the last two core kernels; prog_prev indexes
  // the one the next half step's side kernels may wait on (-1: none, after
  // any other kernel on the job's stream)
  cudaEvent_t ev_prog[2] = {};
  int prog_prev = -1;
  bool join_rec[2] = {false, false};
};

namespace {

// Job buffers come from the device's stream-ordered memory pool: freeing
// them (fdtd_destroy, buffer growth) queues behind the job's own work and
// does not synchronise the device, so jobs that come and go on a shared GPU
// do not stall the others.  The pool keeps freed memory for reuse.
void keep_pool_memory(int dev) {
  static std::once_flag once[64];
  if (dev < 0 || dev >= 64) return;
  std::call_once(once[dev], [dev] {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  });
}

// fdtd_debug_fail_alloc: the number of job allocations that still succeed
// before one fails (-1: none fails)
std::atomic<long long> g_fail_after{-1};

cudaError_t pool_alloc(fdtd_job *J, void **p, size_t bytes) {
  long long left = g_fail_after.load();
  while (left >= 0 && !g_fail_after.compare_exchange_weak(left, left - 1)) {}
  if (left == 0) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  keep_pool_memory(J->device);
  return cudaMallocAsync(p, bytes, J->stream);
}

void pool_free(fdtd_job *J, void *p) {
  if (p) cudaFreeAsync(p, J->stream);
}

int alloc_dev(fdtd_job *J, void **p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = pool_alloc(J, p, bytes);
  if (e != cudaSuccess) return set_err(FDTD_ENOMEM, "device allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
  J->allocs.push_back(*p);
  J->dev_bytes += bytes;
  e = cudaMemsetAsync(*p, 0, bytes, J->stream);
  if (e != cudaSuccess) return set_err(FDTD_ECUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
  // the buffer is ready only in the job stream's order: wait for it (and its
  // zeroing) before uploads on other streams or the host may touch it
  e = cudaStreamSynchronize(J->stream);
  if (e != cudaSuccess) return set_err(FDTD_ECUDA, "cudaStreamSynchronize: %s", cudaGetErrorString(e));
  return FDTD_OK;
}

// give back a buffer of alloc_dev before the job ends
void free_dev(fdtd_job *J, void *p, size_t bytes) {
  if (!p) return;
  for (size_t q = 0; q < J->allocs.size(); ++q)
    if (J->allocs[q] == p) {
      J->allocs.erase(J->allocs.begin() + (long)q);
      break;
    }
  pool_free(J, p);
  J->dev_bytes -= bytes;
}

// the device flag of bounded waits (after the stream has drained): a wait
// that gave up is reported once as FDTD_ECUDA
int kernel_flag(fdtd_job *J) {
  if (!J->d_err) return FDTD_OK;
  int h = 0;
  CK(cudaMemcpy(&h, J->d_err, sizeof h, cudaMemcpyDeviceToHost));
  if (!h) return FDTD_OK;
  CK(cudaMemset(J->d_err, 0, sizeof h));
  return set_err(FDTD_ECUDA, "a bounded wait in the TMA core kernel gave up");
}

// a zeroed buffer that the time steps change, of float or double elements
// (esz 0: the job's precision): registered for checkpoints and for
// fdtd_check_finite
int alloc_state(fdtd_job *J, void **p, size_t bytes, int esz = 0) {
  int rc = alloc_dev(J, p, bytes);
  if (rc) return rc;
  J->state.push_back({*p, bytes == 0 ? size_t(16) : bytes, esz ? esz : (int)J->esz});
  return FDTD_OK;
}

template <typename T>
int upload_vec(fdtd_job *J, void **dst, const std::vector<double> &v) {
  std::vector<T> t(v.begin(), v.end());
  int rc = alloc_dev(J, dst, t.size() * sizeof(T));
  if (rc) return rc;
  CK(cudaMemcpy(*dst, t.data(), t.size() * sizeof(T), cudaMemcpyHostToDevice));
  J->h2d += t.size() * sizeof(T);
  return FDTD_OK;
}

int check_device(int *dev) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return set_err(FDTD_ENODEV, "no CUDA device (%s); this library has no CPU path",
                   e != cudaSuccess ? cudaGetErrorString(e) : "count 0");
  int d = 0;
  CK(cudaGetDevice(&d));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, d));
  if (prop.major != 10 || prop.minor != 3)
    return set_err(FDTD_ENODEV, "device %d is sm_%d%d; the kernels are built for sm_103a only", d, prop.major,
                   prop.minor);
  *dev = d;
  return FDTD_OK;
}

bool inside(const fdtd_job *J, const MatRec &m, int i, int j, int k) {
  const fdtd_region &r = m.region;
  switch (r.kind) {
    case FDTD_REGION_BOX:
      return i >= r.lo[0] && i <= r.hi[0] && j >= r.lo[1] && j <= r.hi[1] && k >= r.lo[2] && k <= r.hi[2];
    case FDTD_REGION_SPHERES:
      for (int q = 0; q < r.count; ++q) {
        const double *c = m.centers.data() + 4 * q;
        double dx = i + 0.5 - c[0], dy = j + 0.5 - c[1];
        double d2 = dx * dx + dy * dy;
        if (J->dim == 3) {
          double dz = k + 0.5 - c[2];
          d2 += dz * dz;
        }
        if (d2 <= c[3] * c[3]) return true;
      }
      return false;
    case FDTD_REGION_MASK:
      return m.mask[(size_t)i + (size_t)J->nx * ((size_t)j + (size_t)J->ny * k)] != 0;
  }
  return false;
}

// bounding box of a region (to paint without a full-grid scan)
void region_bounds(const fdtd_job *J, const MatRec &m, int lo[3], int hi[3]) {
  const int n[3] = {J->nx, J->ny, J->nz};
  for (int a = 0; a < 3; ++a) { lo[a] = 0; hi[a] = n[a] - 1; }
  if (m.region.kind == FDTD_REGION_BOX) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::max(0, m.region.lo[a]);
      hi[a] = std::min(n[a] - 1, m.region.hi[a]);
    }
  } else if (m.region.kind == FDTD_REGION_SPHERES) {
    for (int a = 0; a < 3; ++a) { lo[a] = n[a]; hi[a] = -1; }
    for (int q = 0; q < m.region.count; ++q) {
      const double *c = m.centers.data() + 4 * q;
      for (int a = 0; a < 3; ++a) {
        if (a == 2 && J->dim < 3) { lo[2] = 0; hi[2] = n[2] - 1; continue; }
        lo[a] = std::min(lo[a], std::max(0, (int)std::floor(c[a] - c[3] - 1.0)));
        hi[a] = std::max(hi[a], std::min(n[a] - 1, (int)std::ceil(c[a] + c[3] + 1.0)));
      }
    }
  }
}

// exp(x + i y) - 1 without cancellation
std::complex<double> expm1c(double x, double y) {
  const double sh = std::sin(0.5 * y);
  return std::complex<double>(std::expm1(x) * std::cos(y) - 2.0 * sh * sh, std::exp(x) * std::sin(y));
}

// ---- PML coefficient tables (FP64, the reference's formulas) -----------
struct Prof {
  std::vector<double> f1, f2, g1, g2;
  void init(int n, double f2d, double g2d) {
    f1.assign(n, 1.0); f2.assign(n, f2d); g1.assign(n, 1.0); g2.assign(n, g2d);
  }
};

// low-side profile over 1-based positions 1..npml stored at index base+pos-1
// (init_varx1, M3/BERpmly_mod.f90:761-786, and the y low profile :674-692)
void prof_low(Prof &P, int base, int npml, double ep, double sigmam, double order, double dt, double ds) {
  const double z0 = std::sqrt(K.mu0 / K.ep0);
  for (int i = 1; i <= npml; ++i) {
    const int x = base + i - 1;
    double sE = ep * sigmam * std::pow(((double)(npml - i) + 0.5) / (double)npml, order);
    double aE = sE * dt / ep;
    P.f1[x] = std::exp(-aE);
    P.f2[x] = (1.0 - P.f1[x]) / (z0 * sE * ds);
    if (i < npml) {
      double sH = K.mu0 * sigmam * std::pow(((double)(npml - i)) / (double)npml, order);
      double aH = sH * dt / K.mu0;
      P.g1[x] = std::exp(-aH);
      P.g2[x] = z0 * (1.0 - P.g1[x]) / (sH * ds);
    }
  }
}

// high-side profile: first position stored at index base (ii counts down from npml)
// (init_varx2, M3/BERpmly_mod.f90:788-815, and the y high profile :695-714)
void prof_high(Prof &P, int base, int npml, double ep, double sigmam, double order, double dt, double ds) {
  const double z0 = std::sqrt(K.mu0 / K.ep0);
  int ii = npml;
  for (int q = 0; q < npml; ++q) {
    const int x = base + q;
    if (ii < npml) {
      double sE = ep * sigmam * std::pow(((double)(npml - ii)) / (double)npml, order);
      double aE = sE * dt / ep;
      P.f1[x] = std::exp(-aE);
      P.f2[x] = (1.0 - P.f1[x]) / (z0 * sE * ds);
    }
    double sH = K.mu0 * sigmam * std::pow(((double)(npml - ii) + 0.5) / (double)npml, order);
    double aH = sH * dt / K.mu0;
    P.g1[x] = std::exp(-aH);
    P.g2[x] = z0 * (1.0 - P.g1[x]) / (sH * ds);
    ii = ii - 1;
  }
}

template <typename T>
int upload_prof(fdtd_job *J, const Prof &P, void **f1, void **f2, void **g1, void **g2) {
  int rc;
  if ((rc = upload_vec<T>(J, f1, P.f1))) return rc;
  if ((rc = upload_vec<T>(J, f2, P.f2))) return rc;
  if ((rc = upload_vec<T>(J, g1, P.g1))) return rc;
  return upload_vec<T>(J, g2, P.g2);
}

// ---- commit ------------------------------------------------------------
// side streams and events that fork a half step's parts off the job's stream
int make_branches(fdtd_job *J) {
  for (int q = 0; q < 2; ++q) {
    CK(cudaStreamCreateWithFlags(&J->side[q], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&J->ev_join[q], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&J->ev_prog[q], cudaEventDisableTiming));
  }
  CK(cudaEventCreateWithFlags(&J->ev_fork, cudaEventDisableTiming));
  CK(cudaStreamCreateWithFlags(&J->fold_stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&J->ev_ffork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&J->ev_fjoin, cudaEventDisableTiming));
  return FDTD_OK;
}

// 2D work split.  Core units: whole V-cell vectors of the main range outside
// the split-PML shell, in rows without flags; they take only the interior
// Yee update.  Every other unit goes to a list for the edge kernel.
int split_2d(fdtd_job *J, const std::vector<uint8_t> &rf) {
  const int nx = J->nx, ny = J->ny;
  const int vw = J->esz == 4 ? 4 : 2;  // float4 / double2 rows when aligned
  const int V = J->vec = (nx % vw == 0) ? vw : 1;
  const int nvec = nx / V;
  if ((long long)nvec * ny > (long long)INT32_MAX)
    return set_err(FDTD_ERANGE, "2D grid of %d x %d cells is too large for 32-bit unit indices", nx, ny);
  const int xlo = std::max(J->g.main_lo[0], J->slo[0]), xhi = std::min(J->g.main_hi[0], J->shi[0]);
  const int ylo = std::max(J->g.main_lo[1], J->slo[1]), yhi = std::min(J->g.main_hi[1], J->shi[1]);
  const int cv0 = (xlo + V - 1) / V, cv1 = std::max(cv0, (xhi + 1) / V);  // whole vectors in [xlo, xhi]
  const int cy1 = std::max(ylo, yhi + 1);
  J->cv0 = cv0;
  J->cw = cv1 - cv0;
  J->cy0 = ylo;
  J->ch = cy1 - ylo;
  J->ncore = J->cw * J->ch;
  std::vector<int> edge;
  edge.reserve((size_t)nvec * ny - (size_t)J->ncore + (size_t)nvec * 8);
  for (int j = 0; j < ny; ++j) {
    const bool core_row = j >= ylo && j < cy1 && rf[j] == 0;
    for (int v = 0; v < nvec; ++v)
      if (!(core_row && v >= cv0 && v < cv1)) edge.push_back(j * nvec + v);
  }
  J->nedge = (int)edge.size();
  int rc;
  if (!edge.empty()) {
    if ((rc = alloc_dev(J, (void **)&J->d_edge, edge.size() * sizeof(int)))) return rc;
    CK(cudaMemcpy(J->d_edge, edge.data(), edge.size() * sizeof(int), cudaMemcpyHostToDevice));
    J->h2d += edge.size() * sizeof(int);
  }
  return make_branches(J);
}

// 3D work split.  Core units: whole V-cell x-vectors of the main range
// outside the split-PML shell, in (y, z) rows without a source.  Every other
// x-vector is listed for the edge blocks of the general launch.
int split_3d(fdtd_job *J, const std::vector<uint8_t> &rf) {
  const int nx = J->nx, ny = J->ny, nz = J->nz;
  const int vw = J->esz == 4 ? 4 : 2;
  const int V = J->vec = (nx % vw == 0) ? vw : 1;
  const int nvec = nx / V;
  if ((long long)nvec * ny * nz > (long long)INT32_MAX)
    return set_err(FDTD_ERANGE, "3D grid of %d x %d x %d cells is too large for 32-bit unit indices", nx, ny, nz);
  int lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = std::max(J->g.main_lo[a], J->slo[a]);
    hi[a] = std::min(J->g.main_hi[a], J->shi[a]);
  }
  const int cv0 = (lo[0] + V - 1) / V, cv1 = std::max(cv0, (hi[0] + 1) / V);
  J->cv0 = cv0;
  J->cw = cv1 - cv0;
  J->cy0 = lo[1];
  J->ch = std::max(0, hi[1] - lo[1] + 1);
  J->cz0 = lo[2];
  J->cd = std::max(0, hi[2] - lo[2] + 1);
  J->ncore = J->cw * J->ch * J->cd;
  std::vector<int> edge;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      const int row = k * ny + j;
      const bool core_row = j >= J->cy0 && j < J->cy0 + J->ch && k >= J->cz0 && k < J->cz0 + J->cd && rf[row] == 0;
      for (int v = 0; v < nvec; ++v)
        if (!(core_row && v >= cv0 && v < cv1)) edge.push_back(row * nvec + v);
    }
  J->nedge = (int)edge.size();
  int rc;
  if (!edge.empty()) {
    if ((rc = alloc_dev(J, (void **)&J->d_edge, edge.size() * sizeof(int)))) return rc;
    CK(cudaMemcpy(J->d_edge, edge.data(), edge.size() * sizeof(int), cudaMemcpyHostToDevice));
    J->h2d += edge.size() * sizeof(int);
  }
  return make_branches(J);
}

template <typename T>
int tune_tiles(fdtd_job *J);
int setup_tma(fdtd_job *J);
int setup_fused(fdtd_job *J);

void free_fused(fdtd_job *J);
// the tile (0-based) that selects the fused step kernel
int fused_tile(const fdtd_job *J) { return J->dim == 3 ? 8 : 3; }

// The TFSF box: faces, and the cells its face terms touch (the box widened by
// one cell across each face) inside the grid, the main range and the PML's
// interior, with no dispersive cell where an E term lands.
int check_tfbox(fdtd_job *J, const std::vector<uint8_t> &mat) {
  const int nx = J->nx, ny = J->ny, nz = J->nz;
  const int n3[3] = {nx, ny, nz};
  const int *lo = J->tfbox.lo, *hi = J->tfbox.hi;
  for (int a = 0; a < 3; ++a)
    J->tb_face[a] = a == 1 || (a < J->dim && !(J->g.periodic[a] && lo[a] == 0 && hi[a] == n3[a] - 1));
  if (J->dim == 2) J->tb_face[2] = 0;
  if (lo[1] < 1 || hi[1] > ny - 2 || hi[1] <= lo[1])
    return set_err(FDTD_ERANGE, "TFSF box rows %d..%d: need 1 <= lo < hi <= ny-2", lo[1], hi[1]);
  int wlo[3], whi[3];
  for (int a = 0; a < 3; ++a) {
    if (lo[a] < 0 || hi[a] >= n3[a] || lo[a] > hi[a]) return set_err(FDTD_ERANGE, "TFSF box out of grid on axis %d", a);
    if (J->tb_face[a] && hi[a] <= lo[a]) return set_err(FDTD_ERANGE, "TFSF box needs two cells across axis %d", a);
    wlo[a] = J->tb_face[a] ? lo[a] - 1 : lo[a];
    whi[a] = J->tb_face[a] ? hi[a] + 1 : hi[a];
    if (a >= J->dim) continue;
    if (wlo[a] < std::max(J->g.main_lo[a], J->slo[a]) || whi[a] > std::min(J->g.main_hi[a], J->shi[a]))
      return set_err(FDTD_ERANGE, "TFSF box faces on axis %d leave the main range or enter the PML", a);
  }
  if (J->slab_rows > 0 && (wlo[1] < J->slab_rows || whi[1] > ny - 1 - J->slab_rows))
    return set_err(FDTD_ERANGE, "TFSF box faces enter the PML slabs");
  auto disp = [&](int i, int j, int k) { return mat[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)] >= kAdeId; };
  const int k0 = J->dim == 3 ? lo[2] : 0, k1 = J->dim == 3 ? hi[2] : 0;
  for (int k = k0; k <= k1; ++k)
    for (int i = lo[0]; i <= hi[0]; ++i)
      if (disp(i, lo[1], k) || disp(i, hi[1], k)) return set_err(FDTD_EINVAL, "a dispersive cell lies on a TFSF face");
  if (J->tb_face[0])
    for (int k = k0; k <= k1; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        if (disp(lo[0], j, k) || disp(hi[0] + 1, j, k)) return set_err(FDTD_EINVAL, "a dispersive cell lies on a TFSF face");
  if (J->dim == 3 && J->tb_face[2])
    for (int j = lo[1]; j <= hi[1]; ++j)
      for (int i = lo[0]; i <= hi[0]; ++i)
        if (disp(i, j, lo[2]) || disp(i, j, hi[2] + 1)) return set_err(FDTD_EINVAL, "a dispersive cell lies on a TFSF face");
  for (auto &sr : J->srcs)
    if (sr.component == FDTD_E_INC && (sr.lo[1] < 0 || sr.hi[1] >= ny || sr.lo[1] > sr.hi[1]))
      return set_err(FDTD_ERANGE, "incident-line source rows out of the line");
  return FDTD_OK;
}

template <typename T>
int commit_impl(fdtd_job *J) {
  int rc;
  const int nx = J->nx, ny = J->ny, nz = J->nz;
  const long long N = J->ncell;
  const bool split = J->has_pml && J->pml.mode == FDTD_PML_SPLIT;
  const bool ref = J->has_pml && J->pml.mode == FDTD_PML_REFERENCE;
  // interior box of the split PML; the Yee update and materials run inside it
  if (split) {
    const int n[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
      int lo = J->pml.npml[a][0], hi = J->pml.npml[a][1];
      if (J->g.periodic[a] || n[a] == 1) lo = hi = 0;
      J->slo[a] = lo;
      J->shi[a] = n[a] - 1 - hi;
      J->g.main_lo[a] = J->slo[a];
      J->g.main_hi[a] = J->shi[a];
    }
  } else {
    for (int a = 0; a < 3; ++a) { J->slo[a] = 0; J->shi[a] = (a == 0 ? nx : a == 1 ? ny : nz) - 1; }
  }
  auto in_shell = [&](int i, int j, int k) {
    return split && (i < J->slo[0] || i > J->shi[0] || j < J->slo[1] || j > J->shi[1] || k < J->slo[2] || k > J->shi[2]);
  };
  // ---- fields ----
  const bool has[6] = {
      J->dim != 3 ? (J->g.layout == FDTD_LAYOUT_2D_TE || J->dim == 1) : true,
      J->dim == 3 || J->g.layout == FDTD_LAYOUT_2D_TE,
      J->dim == 3 || J->g.layout == FDTD_LAYOUT_2D_TM,
      J->dim == 3 || J->g.layout == FDTD_LAYOUT_2D_TM,
      J->dim == 3 || J->g.layout == FDTD_LAYOUT_2D_TM,
      J->dim == 3 || J->g.layout == FDTD_LAYOUT_2D_TE || J->dim == 1};
  for (int c = 0; c < 6; ++c)
    if (has[c] && (rc = alloc_state(J, &J->F[c], (size_t)N * sizeof(T)))) return rc;
  if (J->has_tfsf) {
    if ((rc = alloc_state(J, &J->F[6], (size_t)N * sizeof(T)))) return rc;
    if ((rc = alloc_state(J, &J->F[7], (size_t)N * sizeof(T)))) return rc;
  }
  if (J->has_tfbox) {
    if ((rc = alloc_state(J, &J->F[6], (size_t)ny * sizeof(T)))) return rc;
    if ((rc = alloc_state(J, &J->F[7], (size_t)ny * sizeof(T)))) return rc;
    if ((rc = alloc_state(J, &J->d_tf_abc, 4 * sizeof(T)))) return rc;
  }
  // ---- materials: device ids (constant dielectrics 1..127, dispersive
  // materials kAdeId..255), painted in call order ----
  std::vector<int> mid(J->mats.size());
  int ndiel = 0, nadem = 0;
  for (size_t m = 0; m < J->mats.size(); ++m) {
    const bool ade = is_ade_kind(J->mats[m].kind);
    mid[m] = ade ? kAdeId + nadem++ : 1 + ndiel++;
    if (ndiel >= kAdeId || nadem > 255 - kAdeId) return set_err(FDTD_ERANGE, "too many materials of one kind");
  }
  std::vector<uint8_t> mat((size_t)N, 0);
  for (size_t m = 0; m < J->mats.size(); ++m) {
    const MatRec &R = J->mats[m];
    if (R.region.kind == FDTD_REGION_SPHERES) {
      // a union of spheres: each sphere over its own bounding box, with the
      // distance test of inside()
      const int n3[3] = {nx, ny, nz};
      for (int q = 0; q < R.region.count; ++q) {
        const double *c = R.centers.data() + 4 * q;
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
          if (a == 2 && J->dim < 3) { lo[2] = 0; hi[2] = n3[2] - 1; continue; }
          lo[a] = std::max(0, (int)std::floor(c[a] - c[3] - 1.0));
          hi[a] = std::min(n3[a] - 1, (int)std::ceil(c[a] + c[3] + 1.0));
        }
        for (int k = lo[2]; k <= hi[2]; ++k)
          for (int j = lo[1]; j <= hi[1]; ++j)
            for (int i = lo[0]; i <= hi[0]; ++i) {
              const double dx = i + 0.5 - c[0], dy = j + 0.5 - c[1];
              double d2 = dx * dx + dy * dy;
              if (J->dim == 3) {
                const double dz = k + 0.5 - c[2];
                d2 += dz * dz;
              }
              if (d2 <= c[3] * c[3]) mat[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)] = (uint8_t)mid[m];
            }
      }
      continue;
    }
    int lo[3], hi[3];
    region_bounds(J, R, lo, hi);
    const bool is_box = R.region.kind == FDTD_REGION_BOX;  // every cell of its bounds: whole row runs
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j) {
        uint8_t *row = mat.data() + (size_t)nx * ((size_t)j + (size_t)ny * k);
        if (is_box) {
          if (hi[0] >= lo[0]) std::fill(row + lo[0], row + hi[0] + 1, (uint8_t)mid[m]);
          continue;
        }
        for (int i = lo[0]; i <= hi[0]; ++i)
          if (inside(J, R, i, j, k)) row[i] = (uint8_t)mid[m];
      }
  }
  std::vector<MatCoef<T>> mc(kMaxMat);
  std::vector<AdeCoef<T>> ac;
  for (auto &x : mc) { x.kind = MK_NONE; x.ade = -1; x.ca = T(0); x.cs = T(0); }
  const double Ku = J->g.ku, dt = J->g.dt;
  for (size_t m = 0; m < J->mats.size(); ++m) {
    const MatRec &R = J->mats[m];
    MatCoef<T> &c = mc[mid[m]];
    c.kind = R.kind;
    if (R.kind == MK_DIEL) {
      // gax = 1/constant_ep (M2/simpledielectric_mod.f90:176-186)
      const double gax = R.eps == 0.0 ? 0.0 : 1.0 / R.eps;
      c.ca = T(Ku * gax);
      c.cs = T(gax);
    } else if (R.kind == MK_GOLD) {
      // M2/gold_mod.f90:129-168 (setexp :160-168)
      typedef std::complex<double> cd;
      const fdtd_drude2cp &p = R.gold;
      cd gb[2], gc[2];
      for (int q = 0; q < 2; ++q) {
        cd expi = std::exp(cd(0.0, -p.phi[q]));
        gb[q] = std::exp(cd(-p.gamma[q] * dt, p.omega[q] * dt));
        gc[q] = cd(0.0, dt * 2.0 * p.amp[q] * p.omega[q]) * expi;
      }
      cd ga = cd(p.eps_inf, 0.0) - gc[0] - gc[1];
      cd w = 1.0 / ga;
      AdeCoef<T> a{};
      a.kind = MK_GOLD;
      a.normal = -1;
      a.ha = T(std::exp(-p.gamma_d * dt));
      a.hb = T((p.omega_d * p.omega_d) * dt / p.gamma_d);
      a.dha = T(-std::expm1(-p.gamma_d * dt));
      const cd d1 = expm1c(-p.gamma[0] * dt, p.omega[0] * dt), d2 = expm1c(-p.gamma[1] * dt, p.omega[1] * dt);
      a.dr[0] = T(d1.real()); a.di[0] = T(d1.imag());
      a.dr[1] = T(d2.real()); a.di[1] = T(d2.imag());
      (void)gb;
      a.gcr[0] = T(gc[0].real()); a.gci[0] = T(gc[0].imag());
      a.gcr[1] = T(gc[1].real()); a.gci[1] = T(gc[1].imag());
      a.wr = T(w.real()); a.wi = T(w.imag());
      c.ade = (int)ac.size();
      c.ca = T(Ku);
      c.cs = T(1);
      ac.push_back(a);
    } else if (R.kind == MK_CONDUCTIVE) {
      // SiL800 (3D/siL800_mod.f90:85-104): the gold update with no Drude
      // memory (ha = 0) and no critical points, E = (D - I)/ga, I += gb E
      const double gb = R.sigma * dt / K.ep0, ga = R.eps + gb;
      AdeCoef<T> a{};
      a.kind = MK_GOLD;
      a.normal = -1;
      a.ha = T(0);
      a.hb = T(gb);
      a.dha = T(1);
      a.wr = T(1.0 / ga);
      a.wi = T(0);
      c.kind = MK_GOLD;
      c.ade = (int)ac.size();
      c.ca = T(Ku);
      c.cs = T(1);
      ac.push_back(a);
    } else if (R.kind == MK_GRAPHENE_NK) {
      // graphene633 (1D/graphene633_mod.f90:48-105): the graphene update with
      // no Drude memory (ha = 0), ga = eps_inf + sigma dt/eps0, I += gb E,
      // Kerr chi3 alpha, Raman (1 - alpha) chi3 damped by gamma_nl
      const fdtd_graphene_nk_desc &p = R.gnk;
      const double sigma = std::sqrt(p.scale) * 4.0 * K.pi * p.n * p.k * K.c0 * K.ep0 / p.wavelength;
      const double eps_inf = p.scale * (p.n * p.n - p.k * p.k);
      const double gb = sigma * dt / K.ep0;
      AdeCoef<T> a{};
      a.kind = MK_GRAPHENE;
      a.normal = -1;
      a.ha = T(0);
      a.hb = T(gb);
      a.dha = T(1);
      a.ga = T(eps_inf + gb);
      a.kerr = T(p.alpha * p.chi3);
      double r0 = 0.0, c1 = 0.0, c2 = 0.0;
      if (p.chi3 != 0.0) {
        const double betaR = std::sqrt(p.w_nl * p.w_nl - p.gamma_nl * p.gamma_nl);
        const double omegaR = (p.w_nl * p.w_nl) / betaR;
        r0 = (1.0 - p.alpha) * p.chi3 * omegaR * dt * std::exp(-p.gamma_nl * dt) * std::sin(betaR * dt);
        const double sb = std::sin(0.5 * betaR * dt);
        c1 = 2.0 * (std::expm1(-p.gamma_nl * dt) * std::cos(betaR * dt) - 2.0 * sb * sb);
        c2 = -std::expm1(-2.0 * p.gamma_nl * dt);
      }
      a.r0 = T(r0);
      a.rv = T(1.0 - c2);
      a.rs = T(c1 + c2);
      c.kind = MK_GRAPHENE;
      c.ade = (int)ac.size();
      c.ca = T(Ku);
      c.cs = T(1);
      ac.push_back(a);
    } else if (R.kind == MK_GRAPHENE) {
      const fdtd_graphene_desc &p = R.gr;
      const double hbar = 6.62607015e-34 / (2.0 * K.pi), kb = 1.380649e-23, qe = 1.602176634e-19;
      const double kT = kb * p.temperature, ef = p.fermi_ev * qe;
      const double sigma_s0 = (2.0 * qe * qe * kT * p.tau / (K.pi * hbar * hbar)) * std::log(2.0 * std::cosh(ef / (2.0 * kT)));
      const double sigma0 = sigma_s0 / p.thickness;
      const double gam = 1.0 / p.tau;
      const double wNL = 2.0 * K.pi * p.raman_freq, dnuNL = 1.0 / p.raman_tau;
      const double alfaR = 0.5 * dnuNL, betaR = std::sqrt(wNL * wNL - alfaR * alfaR), omegaR = (wNL * wNL) / betaR;
      const double chi3n = p.chi3 * p.e_scale * p.e_scale;
      AdeCoef<T> a{};
      a.kind = MK_GRAPHENE;
      int normal = -1;
      const int n3[3] = {nx, ny, nz};
      for (int ax = 0; ax < 3; ++ax)
        if (R.region.lo[ax] == R.region.hi[ax] && n3[ax] > 1) { normal = ax; break; }
      a.normal = normal;
      a.ha = T(std::exp(-gam * dt));
      a.hb = T(sigma0 * dt / K.ep0);
      a.dha = T(-std::expm1(-gam * dt));
      a.ga = T(1.0);
      a.r0 = T(p.raman_frac * chi3n * omegaR * dt * std::exp(-alfaR * dt) * std::sin(betaR * dt));
      // r1 = 2 e^{-a} cos b, r2 = -e^{-2a}; c1 = r1 - 2, c2 = 1 + r2, without cancellation
      const double sb = std::sin(0.5 * betaR * dt);
      const double c1 = 2.0 * (std::expm1(-alfaR * dt) * std::cos(betaR * dt) - 2.0 * sb * sb);
      const double c2 = -std::expm1(-2.0 * alfaR * dt);
      a.rv = T(1.0 - c2);
      a.rs = T(c1 + c2);
      a.kerr = T((1.0 - p.raman_frac) * chi3n);
      c.ade = (int)ac.size();
      c.ca = T(Ku);
      c.cs = T(1);
      ac.push_back(a);
    } else if (R.kind == MK_GRAPHENE_CP) {
      // Graphene%initialize_GrapheneVars (3D/graphene_mod.f90:202-283,
      // 2D/graphene_mod.f90:163-236): the amplitudes and the Drude weight
      // scaled by s = Graphenewidth/ds (scaleParams), gb_p carried as gb_p - 1
      typedef std::complex<double> cd;
      const fdtd_graphene_cp_desc &p = R.gcp;
      const double sc = p.width / J->g.ds;
      AdeCoef<T> a{};
      a.kind = MK_GRAPHENE_CP;
      a.normal = p.normal_axis;
      a.ha = T(std::exp(-p.drude_gamma * dt));
      a.hb = T(sc * (p.drude_omega * p.drude_omega) * dt / p.drude_gamma);
      a.dha = T(-std::expm1(-p.drude_gamma * dt));
      cd ga = cd(p.eps_inf, 0.0);
      for (int q = 0; q < kMaxCp; ++q) {
        const cd d = expm1c(-p.gamma[q] * dt, p.omega[q] * dt);
        const cd gc = cd(0.0, dt * 2.0 * (sc * p.amp[q]) * p.omega[q]) * std::exp(cd(0.0, -p.phi[q]));
        ga -= gc;
        a.dr[q] = T(d.real()); a.di[q] = T(d.imag());
        a.gcr[q] = T(gc.real()); a.gci[q] = T(gc.imag());
      }
      a.gar = T(ga.real());
      a.gai = T(ga.imag());
      // Raman S_R(n) = r1 S_R(n-1) + r2 S_R(n-2) + r0 E^2 in velocity form:
      // V = rv V + rs S_R + r0 E^2, S_R += V, with rv = -r2 and rs = r1 - 1 + r2
      // from c1 = r1 - 2 and c2 = 1 + r2 computed without cancellation
      double r0 = 0.0, c1 = 0.0, c2 = 0.0;
      if (p.chi3 != 0.0) {
        const double wdt = p.w_nl * dt, gdt = p.gamma_nl * dt;
        if (p.raman_form == FDTD_RAMAN_CENTRAL) {  // 2D/graphene_mod.f90:210-212
          r0 = p.chi3 * (wdt * wdt) / (1.0 + gdt);
          c1 = -(wdt * wdt + 2.0 * gdt) / (1.0 + gdt);
          c2 = 2.0 * gdt / (1.0 + gdt);
        } else {  // 3D/graphene_mod.f90:216-218, 256-258
          const double alfaR = 0.5 * p.gamma_nl, betaR = std::sqrt(p.w_nl * p.w_nl - alfaR * alfaR);
          const double omegaR = (p.w_nl * p.w_nl) / betaR;
          r0 = p.chi3 * omegaR * dt * std::exp(-alfaR * dt) * std::sin(betaR * dt);
          const double sb = std::sin(0.5 * betaR * dt);
          c1 = 2.0 * (std::expm1(-alfaR * dt) * std::cos(betaR * dt) - 2.0 * sb * sb);
          c2 = -std::expm1(-2.0 * alfaR * dt);
        }
      }
      a.r0 = T(r0);
      a.rv = T(1.0 - c2);
      a.rs = T(c1 + c2);
      c.ade = (int)ac.size();
      c.ca = T(Ku);
      c.cs = T(1);
      ac.push_back(a);
    } else if (R.kind == MK_LORENTZ) {
      // Both reference codings reduce to one recursion in p = c0 P (JP) = S
      // (si_mod) and v = p(n) - p(n-1):
      //   JP (3D/goldLorentzJp_mod.f90:140-161): gamma1L = 1 - lv,
      //     gamma2L dt = ls, xi1 gamma2L dt = le;  c0 dt Jp = v
      //   S (3D/si_mod.f90:180-206): ga_l + gb_l = 1 - ls, -gb_l = 1 - lv,
      //     gc_l = le;  S(n) - S(n-1) = v
      // and E(n+1) = E(n) + (1/eps_inf) (Ku curl + source - sum_l v_l), the
      // E-form of update_EJp, since ds Ku sum_l Jp_l = sum_l v_l.
      const fdtd_lorentz_desc &p = R.lz;
      AdeCoef<T> a{};
      a.kind = MK_LORENTZ;
      a.normal = -1;
      if (p.sheet) {  // SLG_3LJp1nm: the thin axis is the normal (vacuum) component
        const int n3[3] = {nx, ny, nz};
        for (int ax = 0; ax < 3; ++ax)
          if (R.region.lo[ax] == R.region.hi[ax] && n3[ax] > 1) { a.normal = ax; break; }
      }
      a.nl = p.chi3 != 0.0;
      a.zx = p.ez_uses_x_current != 0;
      if (a.nl) {  // Kerr term of pole 0 (3D/graphene3LorentzJp1nm_mod.f90:74-77, 89-91)
        const double den = 1.0 + p.gamma_nl * dt;
        a.lk = T(((p.omega[0] * dt) * (p.omega[0] * dt) / (1.0 + p.gamma[0] * dt)) * p.chi3);
        a.lqv = T(2.0 * p.gamma_nl * dt / den);
        a.lqs = T((p.w_nl * dt) * (p.w_nl * dt) / den);
        a.escale = T(p.e_scale);
      }
      a.ga = T(1.0 / p.eps_inf);
      a.npoles = p.npoles;
      for (int l = 0; l < kMaxPoles; ++l) {
        if (l >= p.npoles) { a.lv[l] = a.ls[l] = a.le[l] = T(0); continue; }
        const double w = p.omega[l], nu = p.gamma[l], den = 1.0 + nu * dt;
        a.lv[l] = T(2.0 * nu * dt / den);
        a.ls[l] = T((w * dt) * (w * dt) / den);
        a.le[l] = T(p.delta_eps[l] * ((w * dt) * (w * dt) / den));
      }
      c.ade = (int)ac.size();
      c.ca = T(Ku);
      c.cs = T(1);
      ac.push_back(a);
    }
  }
  if (split && nadem > 0) {
    // the split-field update owns every shell cell, whatever is painted
    // there; a dispersive id would make the kernels leave the cell to an ADE
    // slot, and shell cells have none, so they keep no dispersive id
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j) {
        uint8_t *row = mat.data() + (size_t)nx * ((size_t)j + (size_t)ny * k);
        const bool whole = in_shell(J->slo[0], j, k);
        for (int i = 0; i < nx; ++i) {
          if (!whole && i == J->slo[0]) i = J->shi[0] + 1;
          if (i < nx && row[i] >= kAdeId) row[i] = 0;
        }
      }
  }
  if ((rc = alloc_dev(J, (void **)&J->d_mat, (size_t)N))) return rc;
  CK(cudaMemcpy(J->d_mat, mat.data(), (size_t)N, cudaMemcpyHostToDevice));
  J->h2d += (uint64_t)N;
  if ((rc = alloc_dev(J, &J->d_mc, sizeof(MatCoef<T>) * kMaxMat))) return rc;
  CK(cudaMemcpy(J->d_mc, mc.data(), sizeof(MatCoef<T>) * kMaxMat, cudaMemcpyHostToDevice));
  J->h2d += sizeof(MatCoef<T>) * kMaxMat + sizeof(AdeCoef<T>) * ac.size();
  {
    std::vector<double> ca(kMaxMat, 0.0), cs(kMaxMat, 0.0);
    for (int t = 0; t < kMaxMat; ++t)
      if (mc[t].kind == MK_DIEL) { ca[t] = (double)mc[t].ca; cs[t] = (double)mc[t].cs; }
    if ((rc = upload_vec<T>(J, &J->d_mca, ca))) return rc;
    J->mca_host = ca;
    if ((rc = upload_vec<T>(J, &J->d_mcs, cs))) return rc;
  }
  if ((rc = alloc_dev(J, &J->d_ac, sizeof(AdeCoef<T>) * std::max<size_t>(1, ac.size())))) return rc;
  if (!ac.empty()) CK(cudaMemcpy(J->d_ac, ac.data(), sizeof(AdeCoef<T>) * ac.size(), cudaMemcpyHostToDevice));
  J->ac_host.assign((const char *)ac.data(), (const char *)ac.data() + sizeof(AdeCoef<T>) * ac.size());
  J->ade_kind = ac.empty() ? -1 : ac[0].kind;  // the device update all the dispersive materials share, or -1
  for (const AdeCoef<T> &a : ac)
    if (a.kind != J->ade_kind) J->ade_kind = -1;
  // ---- ADE slots (dispersive cells) ----
  static_assert(kAdeId == 128, "the dispersive ids are the ids with the high bit set");
  std::vector<long long> disp;  // ids >= kAdeId are exactly the dispersive materials
  for_high_ids(mat.data(), N, [&](long long c) { disp.push_back(c); });
  std::vector<int> ade_cell;
  std::vector<uint8_t> ade_mat;
  ade_cell.reserve(disp.size());
  ade_mat.reserve(disp.size());
  for (const long long c : disp) {
    const uint8_t id = mat[(size_t)c];
    const int i = (int)(c % nx), j = (int)((c / nx) % ny), k = (int)(c / ((long long)nx * ny));
    if (in_shell(i, j, k)) continue;
    if (!(i >= J->g.main_lo[0] && i <= J->g.main_hi[0] && j >= J->g.main_lo[1] && j <= J->g.main_hi[1] &&
          k >= J->g.main_lo[2] && k <= J->g.main_hi[2]))
      return set_err(FDTD_EINVAL, "dispersive cell (%d,%d,%d) lies outside the Yee update range", i, j, k);
    ade_cell.push_back((int)c);
    ade_mat.push_back(id);
  }
  J->nade = (int)ade_cell.size();
  J->ade_stride = ((J->nade + 31) / 32) * 32;
  if ((rc = alloc_dev(J, (void **)&J->d_ade_cell, sizeof(int) * std::max(1, J->nade)))) return rc;
  if ((rc = alloc_dev(J, (void **)&J->d_ade_mat, std::max(1, J->nade)))) return rc;
  if (J->nade) {
    CK(cudaMemcpy(J->d_ade_cell, ade_cell.data(), sizeof(int) * J->nade, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J->d_ade_mat, ade_mat.data(), J->nade, cudaMemcpyHostToDevice));
    J->h2d += (uint64_t)J->nade * (sizeof(int) + 1);
  }
  J->ade_nf = 0;
  for (const MatRec &R : J->mats)
    J->ade_nf = std::max(J->ade_nf, ade_fields(R.kind, R.lz.npoles, R.lz.chi3 != 0.0, R.lz.ez_uses_x_current != 0));
  if ((rc = alloc_state(J, &J->d_ade_state, sizeof(T) * (size_t)std::max(1, J->ade_nf) * 3 * std::max(32, J->ade_stride))))
    return rc;
  {
    // most common constant-dielectric material: its Ku/eps is a kernel parameter
    static_assert(kMaxMat == 256, "one byte per material id");
    long long cnt[256];
    count_ids(mat.data(), N, cnt);
    int best = 0;
    for (int t = 1; t < kAdeId; ++t) if (cnt[t] > cnt[best]) best = t;
    J->id0 = best;
  }
  // ---- PML ----
  const double Kpml = dt * K.c0 / J->g.ds;  // dt*c0/ds (M3/BERpmly_mod.f90:506)
  if (split) {
    const fdtd_pml_desc &p = J->pml;
    const double ep = p.eps_lo * K.ep0, epr = ep / K.ep0;
    const int n[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
      Prof P;
      P.init(n[a], Kpml / epr, Kpml);
      int lo = p.npml[a][0], hi = p.npml[a][1];
      if (J->g.periodic[a] || n[a] == 1) lo = hi = 0;
      if (lo > 0) prof_low(P, 0, lo, ep, p.sigma_max, p.order, dt, J->g.ds);
      if (hi > 0) prof_high(P, n[a] - hi, hi, ep, p.sigma_max, p.order, dt, J->g.ds);
      if ((rc = upload_prof<T>(J, P, &J->d_cf[0][a], &J->d_cf[1][a], &J->d_cf[2][a], &J->d_cf[3][a]))) return rc;
    }
    const int nsp = J->dim == 3 ? 6 : 1;
    const bool two = sizeof(T) == 8;
    for (int q = 0; q < nsp; ++q) {
      if ((rc = alloc_state(J, &J->d_sp[q], (size_t)N * sizeof(T)))) return rc;
      if (two && (rc = alloc_state(J, &J->d_sp[6 + q], (size_t)N * sizeof(T)))) return rc;
    }
  }
  if (ref && J->dim >= 2) {
    const fdtd_pml_desc &p = J->pml;
    const int rows = p.npml[1][0];
    J->slab_rows = rows;
    if (rows > 0) {
      const double eps_side[2] = {p.eps_lo, p.eps_hi};
      for (int side = 0; side < 2; ++side) {
        J->slab_on[side] = 1;
        J->slab_j0[side] = side == 0 ? 0 : ny - rows;
        const double ep = eps_side[side] * K.ep0, epr = ep / K.ep0;
        // x (corner) profile
        Prof X; X.init(nx, Kpml / epr, Kpml);
        int nlo = p.npml[0][0], nhi = p.npml[0][1] > 0 ? p.npml[0][1] : p.npml[0][0];
        if (nlo > 0) {
          prof_low(X, 0, nlo, ep, p.sigma_max, p.order, dt, J->g.ds);
          prof_high(X, nx - nhi, nhi, ep, p.sigma_max, p.order, dt, J->g.ds);
        }
        Prof Y; Y.init(rows, Kpml / epr, Kpml);
        if (side == 0) prof_low(Y, 0, rows, ep, p.sigma_max, p.order, dt, J->g.ds);
        else prof_high(Y, 0, rows, ep, p.sigma_max, p.order, dt, J->g.ds);
        Prof Z; Z.init(nz, Kpml / epr, Kpml);
        int zlo = p.npml[2][0], zhi = p.npml[2][1] > 0 ? p.npml[2][1] : p.npml[2][0];
        if (J->dim == 3 && zlo > 0) {
          prof_low(Z, 0, zlo, ep, p.sigma_max, p.order, dt, J->g.ds);
          prof_high(Z, nz - zhi, zhi, ep, p.sigma_max, p.order, dt, J->g.ds);
        }
        void **sc = J->d_sc[side];
        if ((rc = upload_prof<T>(J, X, &sc[0], &sc[1], &sc[2], &sc[3]))) return rc;
        if ((rc = upload_prof<T>(J, Y, &sc[4], &sc[5], &sc[6], &sc[7]))) return rc;
        if ((rc = upload_prof<T>(J, Z, &sc[8], &sc[9], &sc[10], &sc[11]))) return rc;
        const int nf = J->dim == 3 ? 12 : 4;
        for (int q = 0; q < nf; ++q)
          if ((rc = alloc_state(J, &J->d_slab[side][q], (size_t)nx * rows * nz * sizeof(T)))) return rc;
      }
    }
  }
  if (ref && J->dim == 1) {
    const fdtd_pml_desc &p = J->pml;
    const int rows = p.npml[1][0];
    J->ja = rows - 1;
    J->jb = ny - rows;
    if (rows > 0) {
      for (int line = 0; line < (J->has_tfsf ? 2 : 1); ++line) {
        const double eps_side[2] = {line ? J->tfsf.eps_lo : p.eps_lo, line ? J->tfsf.eps_hi : p.eps_hi};
        for (int side = 0; side < 2; ++side) {
          J->slab_on[side] = 1;
          const double ep = eps_side[side] * K.ep0, epr = ep / K.ep0;
          Prof Y; Y.init(rows + 2, Kpml / epr, Kpml);
          if (side == 0) prof_low(Y, 1, rows, ep, p.sigma_max, p.order, dt, J->g.ds);
          else prof_high(Y, 1, rows, ep, p.sigma_max, p.order, dt, J->g.ds);
          void **lc = J->d_lc[line][side];
          if ((rc = upload_prof<T>(J, Y, &lc[0], &lc[1], &lc[2], &lc[3]))) return rc;
          if ((rc = alloc_state(J, &J->d_lex[line][side], (size_t)(rows + 2) * sizeof(T)))) return rc;
          if ((rc = alloc_state(J, &J->d_lhz[line][side], (size_t)(rows + 2) * sizeof(T)))) return rc;
        }
      }
    }
  }
  // ---- monitors ----
  long long base = 0, acc = 0;
  int foff = 0;
  std::vector<double> omega;
  bool touches_slab = false, has_mean = false;
  int mean_slots = 0;
  for (auto &M : J->mons) {
    Monitor m{};
    for (int a = 0; a < 3; ++a) { m.lo[a] = M.d.lo[a]; m.hi[a] = M.d.hi[a]; }
    m.ncomp = M.ncomp;
    for (int u = 0; u < M.ncomp; ++u) m.comps[u] = M.comps[u];
    m.ncell = (int)M.ncell;
    m.base = base;
    m.n_first = M.d.n_first;
    m.n_last = M.d.n_last;
    m.nfreq = M.d.nfreq;
    m.acc = acc;
    m.freq_off = foff;
    m.mean = M.d.reduce == FDTD_MONITOR_MEAN;
    m.boxcells = (int)M.boxcells;
    if (m.mean) {
      has_mean = true;
      // blocks of about 4096 cells: whole x-rows of the box
      const int wx = m.hi[0] - m.lo[0] + 1;
      const int rows = (m.hi[1] - m.lo[1] + 1) * (m.hi[2] - m.lo[2] + 1);
      m.mrows = std::max(1, 4096 / wx);
      m.mchunks = (rows + m.mrows - 1) / m.mrows;
      m.mpart = mean_slots;
      mean_slots += m.ncomp * m.mchunks;
    }
    base += (long long)M.ncomp * M.ncell;
    acc += (long long)M.ncomp * M.d.nfreq * M.ncell;
    foff += M.d.nfreq;
    omega.insert(omega.end(), M.omega.begin(), M.omega.end());
    J->mon_dev.push_back(m);
    if (ref && J->dim == 3 && J->slab_rows > 0 &&
        (m.lo[1] <= J->slab_rows - 1 || m.hi[1] >= ny - J->slab_rows))
      touches_slab = true;
  }
  for (auto &P : J->probes)
    if (ref && J->dim == 3 && J->slab_rows > 0 && (P.d.cell[1] <= J->slab_rows - 1 || P.d.cell[1] >= ny - J->slab_rows))
      touches_slab = true;
  if (mean_slots > 0) {
    if ((rc = alloc_dev(J, (void **)&J->d_mean_part, (size_t)mean_slots * sizeof(double)))) return rc;
    if ((rc = alloc_dev(J, (void **)&J->d_mean_ctr, (size_t)mean_slots * sizeof(unsigned)))) return rc;
  }
  if (J->has_tfbox && (rc = check_tfbox(J, mat))) return rc;
  // 2D samples fused into the H edge rows unless a monitor reduces its box
  // (the reduction runs in the stand-alone gather) or a TFSF box adds face
  // terms after the H kernels; 3D: stand-alone gather
  J->gather_fused = (J->dim == 2 && !has_mean && !J->has_tfbox) || (J->dim == 1 && !touches_slab);
  if (J->dim == 2) {
    std::vector<uint8_t> rf((size_t)ny, 0);
    for (auto &sr : J->srcs) {
      if (sr.component == FDTD_EX_INC) continue;
      for (int j = std::max(sr.lo[1], J->g.main_lo[1]); j <= std::min(sr.hi[1], J->g.main_hi[1]); ++j) rf[j] |= ROW_SRC;
    }
    for (auto &M : J->mons)
      if (M.d.reduce == FDTD_MONITOR_CELLS)
        for (int j = M.d.lo[1]; j <= M.d.hi[1]; ++j) rf[j] |= ROW_SAMPLE;
    for (auto &P : J->probes) rf[P.d.cell[1]] |= ROW_SAMPLE;
    if (ref && J->slab_rows > 0)
      for (int j = 0; j < ny; ++j)
        if (j < J->slab_rows || j >= ny - J->slab_rows) rf[j] |= ROW_SLAB;
    if ((rc = alloc_dev(J, (void **)&J->d_rowflag, (size_t)ny))) return rc;
    CK(cudaMemcpy(J->d_rowflag, rf.data(), (size_t)ny, cudaMemcpyHostToDevice));
    J->h2d += (uint64_t)ny;
    if ((rc = split_2d(J, rf))) return rc;
  } else if (J->dim == 3) {
    std::vector<uint8_t> rf((size_t)ny * nz, 0);
    for (auto &sr : J->srcs) {
      if (sr.component == FDTD_EX_INC) continue;
      for (int k = std::max(sr.lo[2], J->g.main_lo[2]); k <= std::min(sr.hi[2], J->g.main_hi[2]); ++k)
        for (int j = std::max(sr.lo[1], J->g.main_lo[1]); j <= std::min(sr.hi[1], J->g.main_hi[1]); ++j)
          rf[(size_t)k * ny + j] |= ROW_SRC;
    }
    if ((rc = alloc_dev(J, (void **)&J->d_rowflag, rf.size()))) return rc;
    CK(cudaMemcpy(J->d_rowflag, rf.data(), rf.size(), cudaMemcpyHostToDevice));
    J->h2d += rf.size();
    if ((rc = split_3d(J, rf))) return rc;
  }
  if (J->dim == 3) {
    // per x-vector of vec cells: 1 where every id is id0, so that the 3D E
    // cores (DRAM-bound) need not load the vector's ids; the 2D cores, which
    // run from L2, issue the id load with their field loads instead
    const int V = J->vec, nvec = nx / V, words = (nvec + 31) / 32;
    const long long rows = (long long)ny * nz;
    std::vector<uint32_t> bits((size_t)rows * words, 0u);
    const uint8_t id0 = (uint8_t)J->id0;
    for (long long r = 0; r < rows; ++r) {
      const uint8_t *row = mat.data() + (size_t)r * nx;
      uint32_t *wd = bits.data() + (size_t)r * words;
      for (int v = 0; v < nvec; ++v) {
        bool u = true;
        for (int q = 0; q < V; ++q) u = u && row[v * V + q] == id0;
        if (u) wd[v >> 5] |= 1u << (v & 31);
      }
    }
    if ((rc = alloc_dev(J, (void **)&J->d_uni, bits.size() * sizeof(uint32_t)))) return rc;
    CK(cudaMemcpy(J->d_uni, bits.data(), bits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    J->h2d += bits.size() * sizeof(uint32_t);
    J->uni_words = words;
  }
  J->stage_row = base;
  J->acc_total = acc;
  if (!omega.empty()) {
    if ((rc = alloc_dev(J, (void **)&J->d_omega, omega.size() * sizeof(double)))) return rc;
    CK(cudaMemcpy(J->d_omega, omega.data(), omega.size() * sizeof(double), cudaMemcpyHostToDevice));
    // e^{i w s dt} for the slots of a DFT ring
    std::vector<double> rot(omega.size() * 2 * kStageSteps);
    for (size_t f = 0; f < omega.size(); ++f)
      for (int sl = 0; sl < kStageSteps; ++sl) {
        const double ph = omega[f] * ((double)sl * J->g.dt);
        rot[(f * kStageSteps + sl) * 2] = std::cos(ph);
        rot[(f * kStageSteps + sl) * 2 + 1] = std::sin(ph);
      }
    if ((rc = alloc_dev(J, (void **)&J->d_rot, rot.size() * sizeof(double)))) return rc;
    CK(cudaMemcpy(J->d_rot, rot.data(), rot.size() * sizeof(double), cudaMemcpyHostToDevice));
    J->h2d += rot.size() * sizeof(double);
    J->h2d += omega.size() * sizeof(double);
  }
  if ((rc = alloc_state(J, (void **)&J->d_acc_re, (size_t)std::max(1LL, acc) * sizeof(double), 8))) return rc;
  if ((rc = alloc_state(J, (void **)&J->d_acc_im, (size_t)std::max(1LL, acc) * sizeof(double), 8))) return rc;
  J->stage_cap_rows = J->dim == 1 ? 4096 : kStageSteps;
  const long long stage_rows = J->dim == 1 ? J->stage_cap_rows : 2 * kStageSteps;  // 2D/3D: two rings
  if ((rc = alloc_state(J, &J->d_stage, (size_t)std::max(1LL, base) * stage_rows * sizeof(T)))) return rc;
  int blocks = 0;
  for (auto &m : J->mon_dev)
    blocks += ((m.ncomp * m.ncell + 255) / 256) * ((m.nfreq + 7) / 8);
  J->dft_blocks = blocks;
  CK(cudaStreamSynchronize(J->stream));
  if ((rc = setup_tma(J))) return rc;
  if ((rc = setup_fused(J))) return rc;
  if ((rc = tune_tiles<T>(J))) return rc;
  if (J->fused_ok && J->tile != fused_tile(J)) free_fused(J);  // the tuner kept a split shape
  if ((rc = kernel_flag(J))) return rc;
  J->committed = true;
  return FDTD_OK;
}

// ---- stepping ------------------------------------------------------------
double gauss_t(const fdtd_source_desc &s, double t) {
  // dexp(-0.5d0*((t-t0)/st)**2)*dsin(w0*t)   (2D/.../program.f90:337)
  const double a = (t - s.t0) / s.st;
  return std::exp(-0.5 * (a * a)) * std::sin(s.w0 * t);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)f;
  }();
  return fn;
}

// The TMA-staged E core (FP32, 4-cell vectors) needs every neighbour of the
// core box inside the grid: the box starts at least one cell in on each
// axis.  Its tensor maps cover the H arrays as nx x ny x nz floats with
// one-plane boxes of the kernel's tile: 128 cells along x (Hy, Hz: plus a
// 4-float halo), 8 rows (Hx, Hz: plus the row below).
int setup_tma(fdtd_job *J) {
  J->tma_ok = false;
  if (J->dim != 3 || J->esz != 4 || J->vec != 4 || J->ncore <= 0) return FDTD_OK;
  if (J->cv0 < 1 || J->cy0 < 1 || J->cz0 < 1) return FDTD_OK;
  if (getenv("FDTD_NO_TMA")) return FDTD_OK;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return FDTD_OK;
  const cuuint64_t dim[3] = {(cuuint64_t)J->nx, (cuuint64_t)J->ny, (cuuint64_t)J->nz};
  const cuuint64_t stride[2] = {(cuuint64_t)J->nx * 4, (cuuint64_t)J->nx * J->ny * 4};
  const cuuint32_t es[3] = {1, 1, 1};
  auto make = [&](CUtensorMap *m, void *base, cuuint32_t bx, cuuint32_t by) {
    const cuuint32_t box[3] = {bx, by, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dim, stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  if (!make(&J->tma.hx, J->F[3], 128, 9) || !make(&J->tma.hy, J->F[4], 132, 8) || !make(&J->tma.hz, J->F[5], 132, 9))
    return FDTD_OK;  // not offered
  // the H core reads the cells right of, above and beyond the core box: it
  // also needs the box to end at least one cell before the grid's far side
  J->tma.h_ok = 0;
  if ((J->cv0 + J->cw) * 4 <= J->nx - 1 && J->cy0 + J->ch <= J->ny - 1 && J->cz0 + J->cd <= J->nz - 1 &&
      make(&J->tma.ex, J->F[0], 128, 9) && make(&J->tma.ey, J->F[1], 132, 8) && make(&J->tma.ez, J->F[2], 132, 9))
    J->tma.h_ok = 1;
  int rc;
  if (!J->d_err && (rc = alloc_dev(J, (void **)&J->d_err, sizeof(int)))) return rc;
  J->tma_ok = true;
  return FDTD_OK;
}

// The second set of fields (and split parts) of a fused step kernel, with
// the accounting of its bytes
void free_fused(fdtd_job *J) {
  const size_t bytes = (size_t)J->ncell * 4;
  for (int c = 0; c < 6; ++c) { free_dev(J, J->Fb[c], bytes); J->Fb[c] = nullptr; }
  for (int q = 0; q < 3; ++q) { free_dev(J, J->spb[q], bytes); J->spb[q] = nullptr; }
  J->fused_ok = false;
}

// The fused 2D step kernel (TMz, FP32) handles every cell of the grid itself,
// dispersive cells aside: it needs 4-cell vectors, no periodic axis, no
// reference slabs, no TFSF box and no mean monitors (the samples are taken
// in the kernel).  Its second set of Ez, Hx, Hy (and Ezx) is allocated here,
// before the tuner times the kernel.
int setup_fused2(fdtd_job *J) {
  if (J->g.layout != FDTD_LAYOUT_2D_TM || J->esz != 4 || J->vec != 4 || J->g.periodic[0] || J->g.periodic[1] ||
      J->slab_rows > 0 || J->has_tfbox || !J->gather_fused)
    return FDTD_OK;
  int rc;
  const size_t bytes = (size_t)J->ncell * 4;
  for (int c = 2; c <= 4; ++c)
    if (!J->Fb[c] && (rc = alloc_dev(J, &J->Fb[c], bytes))) return rc;
  if (J->d_sp[0] && !J->spb[0] && (rc = alloc_dev(J, &J->spb[0], bytes))) return rc;
  J->fused_ok = true;
  return FDTD_OK;
}

// The fused 3D step kernel needs what the TMA cores need on both sides of the
// core box, and a grid without reference slabs or a TFSF box (their kernels
// update fields in place).  Its second set of field buffers is allocated
// here, before the tuner times the kernel; commit gives it back if the tuner
// keeps another shape.  Environment FDTD_NO_FUSED leaves the kernels out.
int setup_fused(fdtd_job *J) {
  J->fused_ok = false;
  if (getenv("FDTD_NO_FUSED") || J->ncore <= 0) return FDTD_OK;
  if (J->dim == 2) return setup_fused2(J);
  if (J->dim != 3 || !J->tma_ok || !J->tma.h_ok || J->slab_rows > 0 || J->has_tfbox) return FDTD_OK;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return FDTD_OK;
  int rc;
  const size_t bytes = (size_t)J->ncell * 4;
  for (int c = 0; c < 6; ++c)
    if (!J->Fb[c] && (rc = alloc_dev(J, &J->Fb[c], bytes))) return rc;
  const cuuint64_t dim[3] = {(cuuint64_t)J->nx, (cuuint64_t)J->ny, (cuuint64_t)J->nz};
  const cuuint64_t stride[2] = {(cuuint64_t)J->nx * 4, (cuuint64_t)J->nx * J->ny * 4};
  const cuuint32_t es[3] = {1, 1, 1};
  auto make = [&](CUtensorMap *m, void *base, cuuint32_t bx, cuuint32_t by) {
    const cuuint32_t box[3] = {bx, by, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dim, stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  for (int b = 0; b < 2; ++b) {
    void *const *F = b ? J->Fb : J->F;
    if (!make(&J->fmaps[b].hx, F[3], 128, 10) || !make(&J->fmaps[b].hy, F[4], 132, 9) ||
        !make(&J->fmaps[b].hz, F[5], 132, 10)) {
      free_fused(J);
      return FDTD_OK;  // not offered
    }
  }
  J->fused_ok = true;
  return FDTD_OK;
}

template <typename T>
void fill_common(fdtd_job *J, StepParams<T> &p) {
  memset(&p, 0, sizeof p);
  p.tma = J->tma_ok ? &J->tma : nullptr;
  p.err = J->d_err;
  p.wait_limit = J->wait_limit;
  p.uni = J->d_uni;
  p.uni_words = J->uni_words;
  p.layout = J->g.layout;
  p.nx = J->nx; p.ny = J->ny; p.nz = J->nz;
  for (int a = 0; a < 3; ++a) {
    p.per[a] = J->g.periodic[a];
    p.mlo[a] = J->g.main_lo[a];
    p.mhi[a] = J->g.main_hi[a];
    p.slo[a] = J->slo[a];
    p.shi[a] = J->shi[a];
  }
  p.ku = T(J->g.ku);
  p.ex = (T *)J->F[0]; p.ey = (T *)J->F[1]; p.ez = (T *)J->F[2];
  p.hx = (T *)J->F[3]; p.hy = (T *)J->F[4]; p.hz = (T *)J->F[5];
  p.exo = p.ex; p.eyo = p.ey; p.ezo = p.ez;  // in place unless a fused step sets a ping-pong pair
  p.hxo = p.hx; p.hyo = p.hy; p.hzo = p.hz;
  p.pp = 0;
  p.mat = J->d_mat;
  p.mc = (const MatCoef<T> *)J->d_mc;
  p.mca = (const T *)J->d_mca;
  p.mcs = (const T *)J->d_mcs;
  p.rowflag = J->d_rowflag;
  p.id0 = J->id0;
  p.ca0 = J->mca_host.empty() ? T(0) : T(J->mca_host[J->id0]);
  p.nade = J->nade;
  p.ade_cell = J->d_ade_cell;
  p.ade_mat = J->d_ade_mat;
  p.ac = (const AdeCoef<T> *)J->d_ac;
  for (size_t q = 0; q < J->ac_host.size() / sizeof(AdeCoef<T>) && q < (size_t)kAdeParam; ++q)
    memcpy(&p.acp[q], J->ac_host.data() + q * sizeof(AdeCoef<T>), sizeof(AdeCoef<T>));
  p.ade_kind = J->ade_kind;
  p.ade_state = (T *)J->d_ade_state;
  p.ade_stride = J->ade_stride;
  p.pml_mode = J->has_pml ? J->pml.mode : 0;
  for (int a = 0; a < 3; ++a) {
    p.cf1[a] = (const T *)J->d_cf[0][a]; p.cf2[a] = (const T *)J->d_cf[1][a];
    p.cg1[a] = (const T *)J->d_cf[2][a]; p.cg2[a] = (const T *)J->d_cf[3][a];
  }
  for (int q = 0; q < 12; ++q) p.sp[q] = (T *)J->d_sp[q];
  p.slab_rows = J->slab_rows;
  for (int s = 0; s < 2; ++s) {
    p.slab_on[s] = J->slab_on[s];
    p.slab_j0[s] = J->slab_j0[s];
    for (int q = 0; q < 12; ++q) p.slab[s][q] = (T *)J->d_slab[s][q];
    void *const *sc = J->d_sc[s];
    p.sf1x[s] = (const T *)sc[0]; p.sf2x[s] = (const T *)sc[1]; p.sg1x[s] = (const T *)sc[2]; p.sg2x[s] = (const T *)sc[3];
    p.sf1y[s] = (const T *)sc[4]; p.sf2y[s] = (const T *)sc[5]; p.sg1y[s] = (const T *)sc[6]; p.sg2y[s] = (const T *)sc[7];
    p.sf1z[s] = (const T *)sc[8]; p.sf2z[s] = (const T *)sc[9]; p.sg1z[s] = (const T *)sc[10]; p.sg2z[s] = (const T *)sc[11];
  }
  if (J->dim == 2) {
    p.vec = J->vec;
    p.cv0 = J->cv0;
    p.cw = J->cw;
    p.cy0 = J->cy0;
    p.ch = J->ch;
    p.ncore = J->ncore;
    p.tile = J->tile;
    p.nedge = J->nedge;
    p.edge_units = J->d_edge;
  } else {
    p.ntile_blocks = (J->nedge + 255) / 256;
    p.nedge = J->nedge;
    p.edge_units = J->d_edge;
    p.vec = J->vec;
    p.cv0 = J->cv0; p.cw = J->cw; p.cy0 = J->cy0; p.ch = J->ch; p.cz0 = J->cz0; p.cd = J->cd;
    p.ncore = J->ncore;
    p.tile = J->tile;
  }
  if (J->has_tfbox) {
    p.tf_on = 1;
    for (int a = 0; a < 3; ++a) {
      p.tf_lo[a] = J->tfbox.lo[a];
      p.tf_hi[a] = J->tfbox.hi[a];
      p.tf_face[a] = J->tb_face[a];
    }
    p.tf_cb = T(J->g.ku / J->tfbox.eps_line);
    p.tf_sign = T(J->g.layout == FDTD_LAYOUT_2D_TE ? 1.0 : -1.0);
    p.tf_e = (T *)J->F[6];
    p.tf_h = (T *)J->F[7];
    p.tf_abc = (T *)J->d_tf_abc;
  }
  p.nslab_blocks = (J->dim == 3 && J->slab_rows > 0) ? (2 * J->nx * J->slab_rows * J->nz + 255) / 256 : 0;
  p.nade_blocks = (J->nade + 255) / 256;
  p.nmon = (int)J->mon_dev.size();
  for (int q = 0; q < p.nmon; ++q) p.mon[q] = J->mon_dev[q];
  p.stage = (T *)J->d_stage + (size_t)J->stage_half * kStageSteps * J->stage_row;
  p.d_half = nullptr;
  p.stage_row = J->stage_row;
  p.mean_part = J->d_mean_part;
  p.mean_ctr = J->d_mean_ctr;
  p.nprobe = (int)J->probes.size();
  for (int q = 0; q < p.nprobe; ++q) {
    const ProbeRec &P = J->probes[q];
    Probe &d = p.probe[q];
    for (int a = 0; a < 3; ++a) d.cell[a] = P.d.cell[a];
    d.ncomp = P.ncomp;
    for (int u = 0; u < P.ncomp; ++u) d.comps[u] = P.comps[u];
    d.n_first = P.d.n_first;
    d.n_last = P.d.n_last;
    d.buf = P.buf;
    d.cap = P.cap;
  }
}

// Parameters of a step in a captured ring (graph) or an eager one: in a
// ring the step number and the stage half are read on the device, so that
// one graph serves every replay.
template <typename T>
void ring_params(fdtd_job *J, StepParams<T> &p, bool graph) {
  p.d_base = graph ? J->d_base : nullptr;
  if (graph) {
    p.stage = (T *)J->d_stage;
    p.d_half = J->d_half;
  }
}

// sources the 2D/3D kernels see: grid sources, and the incident line's when
// a TFSF box is present (their rows index the line)
bool src_on_device(const fdtd_job *J, const fdtd_source_desc &s) {
  return s.component != FDTD_EX_INC || J->has_tfbox;
}

template <typename T>
void set_sources(fdtd_job *J, StepParams<T> &p) {
  p.nsrc = 0;
  for (auto &s : J->srcs) {
    if (!src_on_device(J, s)) continue;
    Source &d = p.src[p.nsrc];
    d.comp = s.component;
    for (int a = 0; a < 3; ++a) {
      d.lo[a] = s.component == FDTD_E_INC ? s.lo[a] : std::max(s.lo[a], J->g.main_lo[a]);
      d.hi[a] = s.component == FDTD_E_INC ? s.hi[a] : std::min(s.hi[a], J->g.main_hi[a]);
    }
    d.amp = s.amp;
    ++p.nsrc;
  }
  p.srcval_tab = J->d_srctab;
}

void destroy_graph(fdtd_job *J) {
  if (J->graph_exec) cudaGraphExecDestroy(J->graph_exec);
  if (J->graph) cudaGraphDestroy(J->graph);
  J->graph_exec = nullptr;
  J->graph = nullptr;
}

// amp*g(t) for steps 1..n_max of the 2D/3D sources, kept on the device
int ensure_srctab(fdtd_job *J, int n_max) {
  int nsrc = 0;
  for (auto &s : J->srcs) if (src_on_device(J, s)) ++nsrc;
  J->nsrc_dev = nsrc;
  if (nsrc == 0 || n_max <= J->srctab_steps) return FDTD_OK;
  const long long old_steps = J->srctab_steps;
  // a larger device table first: if it cannot be had, nothing has changed
  double *nb = nullptr;
  long long cap = J->srctab_cap_steps;
  if (n_max > J->srctab_cap_steps) {
    cap = std::max<long long>(2 * J->srctab_cap_steps, std::max(n_max, 4096));
    cudaError_t e = pool_alloc(J, (void **)&nb, (size_t)cap * nsrc * sizeof(double));
    if (e != cudaSuccess) return set_err(FDTD_ENOMEM, "source table: %s", cudaGetErrorString(e));
  }
  for (long long n = old_steps + 1; n <= n_max; ++n) {
    const double t = (double)(n - 1) * J->g.dt;           // t=real(n-1,8)*dt
    for (auto &s : J->srcs)
      if (src_on_device(J, s)) J->srctab.push_back(gauss_t(s, t) * s.amp);
  }
  J->srctab_steps = n_max;
  if (nb) {
    CK(cudaStreamSynchronize(J->stream));
    if (J->d_srctab) { pool_free(J, J->d_srctab); J->dev_bytes -= (uint64_t)J->srctab_cap_steps * nsrc * sizeof(double); }
    J->d_srctab = nb;
    J->srctab_cap_steps = cap;
    J->dev_bytes += (uint64_t)cap * nsrc * sizeof(double);
    destroy_graph(J);  // the captured launches hold the old pointer
    CK(cudaMemcpy(J->d_srctab, J->srctab.data(), (size_t)n_max * nsrc * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    CK(cudaMemcpyAsync(J->d_srctab + (size_t)old_steps * nsrc, J->srctab.data() + (size_t)old_steps * nsrc,
                       (size_t)(n_max - old_steps) * nsrc * sizeof(double), cudaMemcpyHostToDevice, J->stream));
    CK(cudaStreamSynchronize(J->stream));  // the host vector may grow again
  }
  J->h2d += (uint64_t)(n_max - old_steps) * nsrc * sizeof(double);
  return FDTD_OK;
}

void ev_record(fdtd_job *J, int kind, bool begin) {
  if (!J->prof) return;
  cudaEvent_t e;
  if (J->ev_pool.empty()) cudaEventCreate(&e);
  else { e = J->ev_pool.back(); J->ev_pool.pop_back(); }
  cudaEventRecord(e, J->stream);
  if (begin) J->pending.push_back({e, nullptr, kind});
  else J->pending.back().b = e;
}

int ensure_probe_cap(fdtd_job *J, int n_max) {
  for (auto &P : J->probes) {
    long long need = (long long)std::min(P.d.n_last, n_max) - P.d.n_first + 1;
    if (need <= P.cap) continue;
    long long cap = std::max<long long>(need, 2LL * P.cap);
    cap = std::max<long long>(cap, 1024);
    double *nb = nullptr;
    cudaError_t e = pool_alloc(J, (void **)&nb, (size_t)cap * P.ncomp * sizeof(double));
    if (e != cudaSuccess) return set_err(FDTD_ENOMEM, "probe buffer: %s", cudaGetErrorString(e));
    CK(cudaMemsetAsync(nb, 0, (size_t)cap * P.ncomp * sizeof(double), J->stream));
    if (P.buf) {
      CK(cudaMemcpyAsync(nb, P.buf, (size_t)P.cap * P.ncomp * sizeof(double), cudaMemcpyDeviceToDevice, J->stream));
      CK(cudaStreamSynchronize(J->stream));
      pool_free(J, P.buf);
      J->dev_bytes -= (uint64_t)P.cap * P.ncomp * sizeof(double);
    }
    P.buf = nb;
    P.cap = (int)cap;
    J->dev_bytes += (uint64_t)cap * P.ncomp * sizeof(double);
    destroy_graph(J);  // the captured launches hold the old buffer
  }
  return FDTD_OK;
}

// The job's DFT fold parameters, without the ring's slots
void fold_params(const fdtd_job *J, DftParams &d) {
  d = DftParams{};
  d.nmon = (int)J->mon_dev.size();
  for (int q = 0; q < d.nmon; ++q) d.mon[q] = J->mon_dev[q];
  d.omega = J->d_omega;
  d.rot = (const double2 *)J->d_rot;
  d.acc_re = J->d_acc_re;
  d.acc_im = J->d_acc_im;
  d.dt = J->g.dt;
  d.stage_row = J->stage_row;
  d.total_work_blocks = J->dft_blocks;
}

// The fold of the last replayed ring, which no later replay has run
template <typename T>
int flush_fold(fdtd_job *J) {
  if (!J->fold_pending) return FDTD_OK;
  J->fold_pending = false;
  if (J->mon_dev.empty() || J->dft_blocks <= 0) return FDTD_OK;
  DftParams d;
  fold_params(J, d);
  d.nslots = kStageSteps;
  d.n0 = J->pending_n0;
  launch_dft<T>(d, (const T *)J->d_stage + (size_t)J->pending_half * kStageSteps * J->stage_row, J->stream);
  J->launches++;
  J->prog_prev = -1;
  CK(cudaGetLastError());
  return FDTD_OK;
}

template <typename T>
int dft_fold(fdtd_job *J) {
  if (J->stage_fill == 0) return FDTD_OK;
  if (!J->mon_dev.empty()) {
    DftParams d{};
    d.nmon = (int)J->mon_dev.size();
    for (int q = 0; q < d.nmon; ++q) d.mon[q] = J->mon_dev[q];
    d.omega = J->d_omega;
    d.rot = (const double2 *)J->d_rot;
    d.acc_re = J->d_acc_re;
    d.acc_im = J->d_acc_im;
    d.dt = J->g.dt;
    d.stage_row = J->stage_row;
    d.total_work_blocks = J->dft_blocks;
    // fold in rings of kStageSteps rows (the 1D stage holds many rings)
    for (int r0 = 0; r0 < J->stage_fill; r0 += kStageSteps) {
      d.nslots = std::min(kStageSteps, J->stage_fill - r0);
      d.n0 = J->stage_n0 + r0;
      ev_record(J, FDTD_KERNEL_DFT, true);
      launch_dft<T>(d, (const T *)J->d_stage + ((size_t)J->stage_half * kStageSteps + r0) * J->stage_row,
                    J->stream);
      ev_record(J, FDTD_KERNEL_DFT, false);
      J->launches++;
    }
    CK(cudaGetLastError());
  }
  J->stage_n0 += J->stage_fill;
  J->stage_fill = 0;
  J->prog_prev = -1;
  return FDTD_OK;
}

enum { ST_E = 1, ST_H = 2, ST_SAMPLE = 4 };

// The parts of one half step write disjoint cells and read only the other
// half's fields, so they run as parallel branches of the job's stream
// (forked and joined with events; a stream capture records them as parallel
// graph nodes).  2D: core, edge and ADE launches; 3D: core and the general
// launch (tiles with non-core cells, reference slabs, ADE cells).  Profiled
// runs launch them one after another so that each part's events time that
// part alone.
template <typename T>
int launch_part(const fdtd_job *J, const StepParams<T> &p, int part, bool e_half, cudaStream_t s,
                cudaEvent_t prog_event = nullptr) {
  if (J->dim == 2) return e_half ? launch_e2d<T>(p, part, s, prog_event) : launch_h2d<T>(p, part, s, prog_event);
  return e_half ? launch_e3d<T>(p, part, s, prog_event) : launch_h3d<T>(p, part, s, prog_event);
}

template <typename T>
int run_parts(fdtd_job *J, const StepParams<T> &p, const bool (&want)[3], bool e_half, bool graph) {
  static const int kind[3] = {-1, FDTD_KERNEL_EDGE, FDTD_KERNEL_ADE};
  const int general = J->dim == 2 ? p.nedge + (e_half ? p.nade : 0) : p.ntile_blocks + p.nslab_blocks + (e_half ? p.nade_blocks : 0);
  const int units[3] = {p.ncore, general, J->dim == 2 && e_half ? p.nade : 0};
  int use[3], nuse = 0;
  for (int q = 0; q < 3; ++q)
    if (want[q] && units[q] > 0) use[nuse++] = q;
  const bool par = !J->prof && nuse > 1;
  // The side kernels of this half step wait on the previous core
  // kernel's programmatic event rather than on its completion, so that they
  // are ready together with this half's core kernel (they wait for the
  // previous core kernel in their own pdl_wait), and fully on the side
  // streams' previous kernels; otherwise they fork off the job's stream.
  const bool chain = par && use[0] == K2D_CORE;
  const bool prog = chain && J->prog_prev >= 0;
  cudaStream_t st[3] = {J->stream, J->stream, J->stream};
  if (par) {
    if (!prog) CK(cudaEventRecord(J->ev_fork, J->stream));
    for (int b = 1; b < nuse; ++b) {
      st[b] = J->side[b - 1];
      if (prog) {
        CK(cudaStreamWaitEvent(st[b], J->ev_prog[J->prog_prev], 0));
        for (int c = 0; c < 2; ++c)
          if (c != b - 1 && J->join_rec[c]) CK(cudaStreamWaitEvent(st[b], J->ev_join[c], 0));
      } else {
        CK(cudaStreamWaitEvent(st[b], J->ev_fork, 0));
      }
    }
  }
  const int cur = J->prog_prev == 0 ? 1 : 0;
  for (int b = 0; b < nuse; ++b) {
    const int q = use[b];
    const int k = q == K2D_CORE ? (e_half ? FDTD_KERNEL_E : FDTD_KERNEL_H) : kind[q];
    if (!graph) ev_record(J, k, true);
    J->launches += launch_part<T>(J, p, q, e_half, st[b], chain && q == K2D_CORE ? J->ev_prog[cur] : nullptr);
    if (!graph) ev_record(J, k, false);
  }
  CK(cudaGetLastError());
  if (par) {
    for (int b = 1; b < nuse; ++b) {
      CK(cudaEventRecord(J->ev_join[b - 1], st[b]));
      J->join_rec[b - 1] = true;
      CK(cudaStreamWaitEvent(J->stream, J->ev_join[b - 1], 0));
    }
  }
  J->prog_prev = chain ? cur : -1;
  return FDTD_OK;
}

// Commit-time tuner of the core kernels' block shape.  Each candidate runs a
// few E and H core launches on the job's own grid, whose fields are still
// zero -- a core update of zero fields writes back the zeros it read -- and
// the fastest is kept.  The choice is cached per kind of grid (dimension,
// layout, precision, vector width, log2 of the core cells).
std::mutex g_tune_mu;
std::map<long long, int> g_tune;

template <typename T>
int tune_tiles(fdtd_job *J) {
  if (J->dim < 2 || J->ncore <= 0) return FDTD_OK;
  if (J->tile_req > 0) {
    J->tile = J->tile_req - 1;
    if ((J->tile == 6 && !J->tma_ok) || (J->tile == 7 && !(J->tma_ok && J->tma.h_ok)))
      return set_err(FDTD_EINVAL, "tiles 7 and 8 (the TMA cores) need FP32, 4-cell vectors and a core box inside the grid");
    if (J->dim == 3 && J->tile == 8 && !J->fused_ok)
      return set_err(FDTD_EINVAL, "tile 9 (the fused step kernel) needs FP32, 4-cell vectors, a core box inside the "
                                  "grid, and no reference slabs or TFSF box");
    if (J->dim == 2 && J->tile == 3 && !J->fused_ok)
      return set_err(FDTD_EINVAL, "2D tile 4 (the fused step kernel) needs TMz, FP32, nx a multiple of 4, no periodic "
                                  "axis, and no reference slabs, TFSF box or mean monitors");
    return FDTD_OK;
  }
  const char *off = getenv("FDTD_TUNE");
  if (off && off[0] == '0') {
    J->tile = 1;
    return FDTD_OK;
  }
  int lg = 0;
  for (long long c = J->ncore; c > 1; c >>= 1) ++lg;
  // which TMA-staged kernels the grid can take is part of the kind of grid
  const long long key = (((((long long)J->dim * 8 + J->g.layout) * 4 + J->g.precision) * 8 + J->vec) * 64 + lg) * 8 +
                        (J->fused_ok ? 4 : 0) + (J->tma_ok ? 2 : 0) + (J->tma_ok && J->tma.h_ok ? 1 : 0);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      J->tile = it->second;
      return FDTD_OK;
    }
  }
  StepParams<T> p;
  fill_common<T>(J, p);
  p.roles = ROLE_MAIN;
  cudaEvent_t a = nullptr, b = nullptr;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  float best = 3.0e38f;
  int choice = 1;
  // 3D: also the z-marching kernels and, where set up, the TMA-staged cores
  // and the fused step kernel (one launch in place of an E and an H core).
  // 2D: also the fused step kernel, against the E and H cores alone (in a
  // step the edge and dispersive-cell kernels run beside the cores, and
  // their work is a small part of a grid large enough for the fused kernel)
  const int nshapes = J->dim == 3 ? (J->fused_ok ? 9 : J->tma_ok ? (J->tma.h_ok ? 8 : 7) : 6) : J->fused_ok ? 4 : 3;
  auto cores = [&](int c) {
    if constexpr (sizeof(T) == 4) {
      if (c == fused_tile(J)) {
        StepParams<float> q = p;
        q.exo = (float *)J->Fb[0]; q.eyo = (float *)J->Fb[1]; q.ezo = (float *)J->Fb[2];
        q.hxo = (float *)J->Fb[3]; q.hyo = (float *)J->Fb[4]; q.hzo = (float *)J->Fb[5];
        q.spo[0] = (float *)J->spb[0];
        q.pp = 1;
        if (J->dim == 3) launch_step3d_fused(q, J->fmaps[0], J->stream);
        else launch_step2d_fused(q, J->stream);
        return;
      }
    }
    launch_part<T>(J, p, K2D_CORE, true, J->stream);
    launch_part<T>(J, p, K2D_CORE, false, J->stream);
  };
  for (int c = 0; c < nshapes; ++c) {
    p.tile = c;
    for (int w = 0; w < 2; ++w) cores(c);
    cudaEventRecord(a, J->stream);
    for (int r = 0; r < 5; ++r) cores(c);
    cudaEventRecord(b, J->stream);
    float ms = 0.f;
    if (cudaEventSynchronize(b) == cudaSuccess && cudaEventElapsedTime(&ms, a, b) == cudaSuccess && ms < best) {
      best = ms;
      choice = c;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CK(cudaGetLastError());
  J->tile = choice;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = choice;
  return FDTD_OK;
}

// the TFSF box's launch of a half step, after the half step's other kernels
template <typename T>
int tfsf_part(fdtd_job *J, const StepParams<T> &p, bool e_half, bool graph) {
  if (!graph) ev_record(J, FDTD_KERNEL_EDGE, true);
  J->launches += launch_tfsf<T>(p, e_half, J->stream);
  if (!graph) ev_record(J, FDTD_KERNEL_EDGE, false);
  J->prog_prev = -1;
  CK(cudaGetLastError());
  return FDTD_OK;
}

// 2D / 3D: one half step (or a role subset of it).  In graph mode the step
// number comes from the device-side ring base (d_base) plus the ring slot.
template <typename T>
int half_e(fdtd_job *J, int n, int roles, int slot = 0, bool graph = false) {
  StepParams<T> p;
  fill_common<T>(J, p);
  set_sources<T>(J, p);
  p.roles = roles;
  p.n = n;
  p.slot = slot;
  ring_params(J, p, graph);
  const bool parts[3] = {(roles & ROLE_MAIN) != 0, (roles & (ROLE_MAIN | ROLE_PML | ROLE_ADE)) != 0, false};
  int rc = run_parts<T>(J, p, parts, true, graph);
  if (!rc && J->has_tfbox && (roles & ROLE_MAIN)) rc = tfsf_part<T>(J, p, true, graph);
  return rc;
}

template <typename T>
int half_h(fdtd_job *J, int n, int roles, bool gather, int slot = -1, bool graph = false) {
  StepParams<T> p;
  fill_common<T>(J, p);
  p.roles = roles;
  p.n = n;
  p.gather = gather ? 1 : 0;
  p.slot = slot >= 0 ? slot : J->stage_fill;
  ring_params(J, p, graph);
  const bool parts[3] = {(roles & ROLE_MAIN) != 0, (roles & (ROLE_MAIN | ROLE_PML)) != 0, false};
  int rc = run_parts<T>(J, p, parts, false, graph);
  if (!rc && J->has_tfbox && (roles & ROLE_MAIN)) rc = tfsf_part<T>(J, p, false, graph);
  return rc;
}

template <typename T>
int sample_sep(fdtd_job *J, int n, int slot = -1, bool graph = false) {
  StepParams<T> p;
  fill_common<T>(J, p);
  p.n = n;
  p.slot = slot >= 0 ? slot : J->stage_fill;
  ring_params(J, p, graph);
  J->launches += launch_gather<T>(p, J->stream);
  J->prog_prev = -1;
  CK(cudaGetLastError());
  return FDTD_OK;
}

template <typename T>
int after_sample(fdtd_job *J, int n) {
  if (J->stage_fill == 0) J->stage_n0 = n;
  J->stage_fill++;
  J->last_n = n;
  if (J->stage_fill == kStageSteps) return dft_fold<T>(J);
  return FDTD_OK;
}

// A job steps through a fused step kernel when the tuner (or fdtd_set_tile)
// chose it.  The per-procedure entry points keep the split kernels.
bool fused_mode(const fdtd_job *J) { return J->fused_ok && J->tile == fused_tile(J); }

// One time step of the fused 2D path, from field set pp to the other: the
// dispersive cells' E (E^n and H^n of the current set, E^{n+1} into the
// other), then the fused kernel over the whole grid, which takes the samples
// of the new fields itself.  The fused kernel follows e2d_ade with a
// programmatic dependency and waits for it only at dispersive cells.
int fused_step2(fdtd_job *J, int n, int slot, bool graph) {
  const int from = J->pp, to = 1 - from;
  float *A[6] = {}, *B[6] = {};
  for (int c = 0; c < 6; ++c) {
    A[c] = (float *)(from ? J->Fb[c] : J->F[c]);
    B[c] = (float *)(to ? J->Fb[c] : J->F[c]);
  }
  StepParams<float> p;
  fill_common<float>(J, p);
  set_sources<float>(J, p);
  p.roles = ROLE_MAIN | ROLE_PML | ROLE_ADE;
  p.n = n;
  p.slot = slot;
  ring_params(J, p, graph);
  p.gather = 1;
  p.pp = 1;
  p.ez = A[2]; p.hx = A[3]; p.hy = A[4];
  p.ezo = B[2]; p.hxo = B[3]; p.hyo = B[4];
  p.sp[0] = (float *)(from ? J->spb[0] : J->d_sp[0]);
  p.spo[0] = (float *)(to ? J->spb[0] : J->d_sp[0]);
  if (!graph) ev_record(J, FDTD_KERNEL_ADE, true);
  J->launches += launch_e2d_ade_pdl<float>(p, J->stream);
  if (!graph) ev_record(J, FDTD_KERNEL_ADE, false);
  if (!graph) ev_record(J, FDTD_KERNEL_STEP, true);
  J->launches += launch_step2d_fused(p, J->stream);
  if (!graph) ev_record(J, FDTD_KERNEL_STEP, false);
  J->pp = to;
  J->prog_prev = -1;
  CK(cudaGetLastError());
  return FDTD_OK;
}

// One time step of the fused path, from field set pp to the other: the
// general E kernel (edge units and ADE cells; E^n and H^n of the current set,
// E^{n+1} into the other), the fused kernel over the core box, the general H
// kernel (E^{n+1} and H^{n+1} in the other set), then the samples of the new
// fields.  The four launches run in this order on the job's stream, each
// waiting for the one before in its programmatic dependency.
template <typename T>
int fused_step(fdtd_job *J, int n, int slot, bool graph) {
  if constexpr (sizeof(T) != 4) {
    (void)n; (void)slot; (void)graph;
    return set_err(FDTD_ESTATE, "the fused step kernel is FP32 only");
  } else {
    if (J->dim == 2) return fused_step2(J, n, slot, graph);
    const int from = J->pp, to = 1 - from;
    float *A[6], *B[6];
    for (int c = 0; c < 6; ++c) {
      A[c] = (float *)(from ? J->Fb[c] : J->F[c]);
      B[c] = (float *)(to ? J->Fb[c] : J->F[c]);
    }
    StepParams<float> p;
    fill_common<float>(J, p);
    set_sources<float>(J, p);
    p.roles = ROLE_MAIN | ROLE_PML | ROLE_ADE;
    p.n = n;
    p.slot = slot;
    ring_params(J, p, graph);
    p.pp = 1;
    p.ex = A[0]; p.ey = A[1]; p.ez = A[2]; p.hx = A[3]; p.hy = A[4]; p.hz = A[5];
    p.exo = B[0]; p.eyo = B[1]; p.ezo = B[2]; p.hxo = B[3]; p.hyo = B[4]; p.hzo = B[5];
    if (!graph) ev_record(J, FDTD_KERNEL_EDGE, true);
    J->launches += launch_e3d_general_pdl<float>(p, J->stream);
    if (!graph) ev_record(J, FDTD_KERNEL_EDGE, false);
    if (!graph) ev_record(J, FDTD_KERNEL_STEP, true);
    J->launches += launch_step3d_fused(p, J->fmaps[from], J->stream);
    if (!graph) ev_record(J, FDTD_KERNEL_STEP, false);
    p.ex = B[0]; p.ey = B[1]; p.ez = B[2];  // the H half reads E^{n+1}
    if (!graph) ev_record(J, FDTD_KERNEL_EDGE, true);
    J->launches += launch_h3d_general_pdl<float>(p, J->stream);
    if (!graph) ev_record(J, FDTD_KERNEL_EDGE, false);
    StepParams<float> g;  // samples of the new fields
    fill_common<float>(J, g);
    g.ex = g.exo = B[0]; g.ey = g.eyo = B[1]; g.ez = g.ezo = B[2];
    g.hx = g.hxo = B[3]; g.hy = g.hyo = B[4]; g.hz = g.hzo = B[5];
    g.n = n;
    g.slot = slot;
    ring_params(J, g, graph);
    J->launches += launch_gather<float>(g, J->stream);
    J->pp = to;
    J->prog_prev = -1;
    CK(cudaGetLastError());
    return FDTD_OK;
  }
}

// After an odd number of fused steps the current fields are in the second
// set: copy them to the canonical one, where every other entry point and the
// ring graph (which starts from it) expect them.
int fused_settle(fdtd_job *J) {
  if (!J->pp) return FDTD_OK;
  const size_t bytes = (size_t)J->ncell * 4;
  for (int c = 0; c < 6; ++c)
    if (J->Fb[c]) CK(cudaMemcpyAsync(J->F[c], J->Fb[c], bytes, cudaMemcpyDeviceToDevice, J->stream));
  for (int q = 0; q < 3; ++q)
    if (J->spb[q]) CK(cudaMemcpyAsync(J->d_sp[q], J->spb[q], bytes, cudaMemcpyDeviceToDevice, J->stream));
  J->pp = 0;
  J->prog_prev = -1;
  return FDTD_OK;
}

template <typename T>
int eager_step(fdtd_job *J, int n) {
  int rc;
  if (fused_mode(J)) {
    if ((rc = fused_step<T>(J, n, J->stage_fill, false))) return rc;
    return after_sample<T>(J, n);
  }
  if ((rc = half_e<T>(J, n, ROLE_MAIN | ROLE_PML | ROLE_ADE))) return rc;
  if ((rc = half_h<T>(J, n, ROLE_MAIN | ROLE_PML, J->gather_fused))) return rc;
  if (!J->gather_fused && (rc = sample_sep<T>(J, n))) return rc;
  return after_sample<T>(J, n);
}

// a replayed ring's step base, its half of the stage buffer and its fold's gate
__global__ void set_ring_kernel(int *base, int v, int *half, int h, int *gate, int g) {
  *base = v;
  *half = h;
  *gate = g;
}

// Capture one ring (kStageSteps steps and the DFT fold of the ring) as a CUDA
// graph; every replay reads its first step number from d_base.
template <typename T>
int ring_graph(fdtd_job *J) {
  int rc;
  if (J->graph_exec) return FDTD_OK;
  if (!J->d_base && (rc = alloc_dev(J, (void **)&J->d_base, sizeof(int)))) return rc;
  if (!J->d_half && (rc = alloc_dev(J, (void **)&J->d_half, sizeof(int)))) return rc;
  if (!J->d_gate && (rc = alloc_dev(J, (void **)&J->d_gate, sizeof(int)))) return rc;
  CK(cudaStreamSynchronize(J->stream));
  const long long launches0 = J->launches;
  J->prog_prev = -1;  // events recorded outside the capture cannot be waited on inside it
  CK(cudaStreamBeginCapture(J->stream, cudaStreamCaptureModeThreadLocal));
  int bad = FDTD_OK;
  // the fold of the ring before this one (the other half of the stage
  // buffer), on its own branch beside this ring's steps; its gate on the
  // device is 0 when no ring came before
  const bool fold = !J->mon_dev.empty() && J->dft_blocks > 0;
  if (fold) {
    bad = cudaEventRecord(J->ev_ffork, J->stream) != cudaSuccess ||
          cudaStreamWaitEvent(J->fold_stream, J->ev_ffork, 0) != cudaSuccess;
    if (!bad) {
      DftParams d;
      fold_params(J, d);
      d.nslots = kStageSteps;
      d.d_base = J->d_base;
      d.d_half = J->d_half;
      d.gate = J->d_gate;
      d.prev = 1;
      launch_dft<T>(d, (const T *)J->d_stage, J->fold_stream);
      J->launches++;
      bad = cudaEventRecord(J->ev_fjoin, J->fold_stream) != cudaSuccess;
    }
    if (bad) bad = set_err(FDTD_ECUDA, "fold branch of the ring graph");
  }
  // the fused path alternates the field sets over the ring's even number of
  // steps, so a replay starts and ends with the canonical set
  for (int s = 0; s < kStageSteps && !bad; ++s) {
    if (fused_mode(J)) {
      bad = fused_step<T>(J, 0, s, true);
      continue;
    }
    bad = half_e<T>(J, 0, ROLE_MAIN | ROLE_PML | ROLE_ADE, s, true);
    if (!bad) bad = half_h<T>(J, 0, ROLE_MAIN | ROLE_PML, J->gather_fused, s, true);
    if (!bad && !J->gather_fused) bad = sample_sep<T>(J, 0, s, true);
  }
  if (!bad && fold && cudaStreamWaitEvent(J->stream, J->ev_fjoin, 0) != cudaSuccess)
    bad = set_err(FDTD_ECUDA, "joining the fold branch");
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(J->stream, &g);
  J->prog_prev = -1;
  J->graph_kernels = (int)(J->launches - launches0);
  J->launches = launches0;
  if (bad) { if (g) cudaGraphDestroy(g); return bad; }
  if (e != cudaSuccess) return set_err(FDTD_ECUDA, "graph capture: %s", cudaGetErrorString(e));
  J->graph = g;
  e = cudaGraphInstantiate(&J->graph_exec, J->graph, 0);
  if (e != cudaSuccess) { destroy_graph(J); return set_err(FDTD_ECUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
  return FDTD_OK;
}

template <typename T>
int replay_ring(fdtd_job *J, int n0) {
  int rc = ring_graph<T>(J);
  if (rc) return rc;
  set_ring_kernel<<<1, 1, 0, J->stream>>>(J->d_base, n0, J->d_half, J->stage_half, J->d_gate, J->fold_pending ? 1 : 0);
  CK(cudaGetLastError());
  CK(cudaGraphLaunch(J->graph_exec, J->stream));
  // this ring's fold runs in the next replay's graph, or in flush_fold
  J->fold_pending = true;
  J->pending_half = J->stage_half;
  J->pending_n0 = n0;
  J->stage_half ^= 1;
  J->prog_prev = -1;
  J->launches += 1 + J->graph_kernels;
  J->stage_n0 = n0 + kStageSteps;
  J->last_n = n0 + kStageSteps - 1;
  return FDTD_OK;
}

// 1D: the persistent line kernel over a chunk of steps
template <typename T>
int line_run(fdtd_job *J, int n_first, int n_steps, int stages) {
  LineParams<T> p;
  memset(&p, 0, sizeof p);
  p.N = J->ny;
  p.mlo = J->g.main_lo[1];
  p.mhi = J->g.main_hi[1];
  p.ku = T(J->g.ku);
  p.ex = (T *)J->F[0];
  p.hz = (T *)J->F[5];
  p.exi = (T *)J->F[6];
  p.hzi = (T *)J->F[7];
  p.tfsf_bd = J->has_tfsf ? J->tfsf.boundary : -1;
  p.mat = J->d_mat;
  p.mc = (const MatCoef<T> *)J->d_mc;
  p.ac = (const AdeCoef<T> *)J->d_ac;
  p.nac = (int)(J->ac_host.size() / sizeof(AdeCoef<T>));
  p.nade = J->nade;
  p.ade_cell = J->d_ade_cell;
  p.ade_mat = J->d_ade_mat;
  p.ade_state = (T *)J->d_ade_state;
  p.ade_stride = J->ade_stride;
  p.ade_nf = J->ade_nf;
  p.ja = J->ja;
  p.jb = J->jb;
  for (int s = 0; s < 2; ++s) {
    p.slab_on[s] = J->slab_on[s];
    for (int line = 0; line < 2; ++line) {
      p.pex[line][s] = (T *)J->d_lex[line][s];
      p.phz[line][s] = (T *)J->d_lhz[line][s];
      p.f1[line][s] = (const T *)J->d_lc[line][s][0];
      p.f2[line][s] = (const T *)J->d_lc[line][s][1];
      p.g1[line][s] = (const T *)J->d_lc[line][s][2];
      p.g2[line][s] = (const T *)J->d_lc[line][s][3];
    }
  }
  // sources: values for every step of the chunk
  p.nsrc = 0;
  for (auto &s : J->srcs) {
    Source &d = p.src[p.nsrc];
    d.comp = s.component;
    for (int a = 0; a < 3; ++a) { d.lo[a] = s.lo[a]; d.hi[a] = s.hi[a]; }
    if (s.component != FDTD_EX_INC) {
      d.lo[1] = std::max(d.lo[1], J->g.main_lo[1]);
      d.hi[1] = std::min(d.hi[1], J->g.main_hi[1]);
    }
    d.amp = s.amp;
    ++p.nsrc;
  }
  if (p.nsrc) {
    std::vector<double> v((size_t)n_steps * p.nsrc);
    for (int st = 0; st < n_steps; ++st) {
      const double t = (double)(n_first + st - 1) * J->g.dt;
      int q = 0;
      for (auto &s : J->srcs) {
        const double g = gauss_t(s, t);
        v[(size_t)st * p.nsrc + q] = s.component == FDTD_EX_INC ? g : g * s.amp;
        ++q;
      }
    }
    if ((long long)v.size() > J->srcval_cap) {
      // the new buffer first: if it cannot be had, the old one stays
      const long long cap = std::max<long long>((long long)v.size(), 4096);
      double *nb = nullptr;
      cudaError_t e = pool_alloc(J, (void **)&nb, cap * sizeof(double));
      if (e != cudaSuccess) return set_err(FDTD_ENOMEM, "source values: %s", cudaGetErrorString(e));
      if (J->d_srcval) { pool_free(J, J->d_srcval); J->dev_bytes -= J->srcval_cap * sizeof(double); }
      J->d_srcval = nb;
      J->srcval_cap = cap;
      J->dev_bytes += cap * sizeof(double);
    }
    CK(cudaMemcpyAsync(J->d_srcval, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, J->stream));
    CK(cudaStreamSynchronize(J->stream));  // v is a temporary
  }
  p.srcval = J->d_srcval;
  p.nmon = (int)J->mon_dev.size();
  for (int q = 0; q < p.nmon; ++q) p.mon[q] = J->mon_dev[q];
  p.nprobe = (int)J->probes.size();
  for (int q = 0; q < p.nprobe; ++q) {
    const ProbeRec &P = J->probes[q];
    Probe &d = p.probe[q];
    for (int a = 0; a < 3; ++a) d.cell[a] = P.d.cell[a];
    d.ncomp = P.ncomp;
    for (int u = 0; u < P.ncomp; ++u) d.comps[u] = P.comps[u];
    d.n_first = P.d.n_first;
    d.n_last = P.d.n_last;
    d.buf = P.buf;
    d.cap = P.cap;
  }
  p.dt = J->g.dt;
  p.n_first = n_first;
  p.n_steps = n_steps;
  p.stages = stages;
  T *stage = (T *)J->d_stage + (size_t)J->stage_fill * J->stage_row;
  ev_record(J, FDTD_KERNEL_LINE1D, true);
  launch_line1d_stage<T>(p, stage, J->stage_row, J->stream);
  ev_record(J, FDTD_KERNEL_LINE1D, false);
  J->launches++;
  CK(cudaGetLastError());
  return FDTD_OK;
}

template <typename T>
int step_impl(fdtd_job *J, int n_first, int n_steps) {
  int rc;
  if ((rc = ensure_probe_cap(J, n_first + n_steps - 1))) return rc;
  if (J->dim == 1) {
    int n = n_first, left = n_steps;
    while (left > 0) {
      if (J->stage_fill == 0) J->stage_n0 = n;
      int chunk = (int)std::min<long long>(left, J->stage_cap_rows - J->stage_fill);
      if ((rc = line_run<T>(J, n, chunk, ST_E | ST_H | ST_SAMPLE))) return rc;
      J->stage_fill += chunk;
      n += chunk;
      left -= chunk;
      J->last_n = n - 1;
      if (J->stage_fill >= J->stage_cap_rows)
        if ((rc = dft_fold<T>(J))) return rc;
    }
    return FDTD_OK;
  }
  const int end = n_first + n_steps;
  if ((rc = ensure_srctab(J, end - 1))) return rc;
  int n = n_first;
  // finish a partly filled ring eagerly, replay whole rings from the graph,
  // run the tail eagerly (the per-launch events of fdtd_profile need eager)
  while (n < end && J->stage_fill != 0)
    if ((rc = eager_step<T>(J, n++))) return rc;
  if (J->use_graph && !J->prof && end - n >= kStageSteps) {
    if ((rc = fused_settle(J))) return rc;
    while (end - n >= kStageSteps) {
      if ((rc = replay_ring<T>(J, n))) return rc;
      n += kStageSteps;
    }
    if ((rc = flush_fold<T>(J))) return rc;
  }
  while (n < end)
    if ((rc = eager_step<T>(J, n++))) return rc;
  return fused_settle(J);
}

#define DISPATCH(J, call) ((J)->g.precision == FDTD_F32 ? call<float> : call<double>)

int check_job(fdtd_job *J, bool need_commit) {
  if (!J) return set_err(FDTD_EINVAL, "null job");
  if (need_commit && !J->committed) return set_err(FDTD_ESTATE, "job not committed");
  if (!need_commit && J->committed) return set_err(FDTD_ESTATE, "job already committed");
  return FDTD_OK;
}

}  // namespace

template <typename T>
static int proc_call(fdtd_job *J, int n, int what) {
  int rc = ensure_probe_cap(J, n);
  if (rc) return rc;
  if (J->dim >= 2 && (rc = ensure_srctab(J, n))) return rc;
  if (J->dim == 1) {
    if (what == 0) { if (J->stage_fill == 0) J->stage_n0 = n; return line_run<T>(J, n, 1, ST_E); }
    if (what == 2) return line_run<T>(J, n, 1, ST_H);
    if (what == 4) {
      if (J->stage_fill == 0) J->stage_n0 = n;
      if ((rc = line_run<T>(J, n, 1, ST_SAMPLE))) return rc;
      J->stage_fill++;
      J->last_n = n;
      if (J->stage_fill >= J->stage_cap_rows) return dft_fold<T>(J);
    }
    return FDTD_OK;
  }
  switch (what) {
    case 0: return half_e<T>(J, n, ROLE_MAIN | ROLE_ADE);
    case 1: return half_e<T>(J, n, ROLE_PML);
    case 2: return half_h<T>(J, n, ROLE_MAIN, false);
    case 3: return half_h<T>(J, n, ROLE_PML, false);
    case 4:
      if ((rc = sample_sep<T>(J, n))) return rc;
      return after_sample<T>(J, n);
  }
  return FDTD_OK;
}

// values of a component: the grid, or the ny cells of a TFSF box's line
static long long field_elems(const fdtd_job *J, int comp) {
  return (J->has_tfbox && comp >= FDTD_E_INC) ? (long long)J->ny : J->ncell;
}

template <typename T>
static int get_field_impl(fdtd_job *J, int comp, double *host) {
  if (comp < 0 || comp > 7 || !J->F[comp]) return set_err(FDTD_EINVAL, "component %d not in this layout", comp);
  const long long cnt = field_elems(J, comp);
  std::vector<T> tmp((size_t)cnt);
  CK(cudaMemcpyAsync(tmp.data(), J->F[comp], (size_t)cnt * sizeof(T), cudaMemcpyDeviceToHost, J->stream));
  CK(cudaStreamSynchronize(J->stream));
  for (long long c = 0; c < cnt; ++c) host[c] = (double)tmp[(size_t)c];
  J->d2h += (uint64_t)cnt * sizeof(T);
  return FDTD_OK;
}

template <typename T>
static int set_field_impl(fdtd_job *J, int comp, const double *host) {
  if (comp < 0 || comp > 7 || !J->F[comp]) return set_err(FDTD_EINVAL, "component %d not in this layout", comp);
  const long long cnt = field_elems(J, comp);
  std::vector<T> tmp(host, host + cnt);
  CK(cudaMemcpyAsync(J->F[comp], tmp.data(), (size_t)cnt * sizeof(T), cudaMemcpyHostToDevice, J->stream));
  CK(cudaStreamSynchronize(J->stream));
  J->h2d += (uint64_t)cnt * sizeof(T);
  return FDTD_OK;
}

// ---- packs of small 2D jobs ----------------------------------------------
// A pack advances several committed 2D jobs of one precision, layout and
// vector width together: each part of each half step is one launch over all
// the jobs' units (k2d.cu, *_pk kernels), each job's parameters coming from a
// device table with one copy per ring slot.  One ring of kStageSteps steps,
// with every job's DFT fold and the advance of every job's step base, is
// captured as a CUDA graph.  The kernels and their order per job are those of
// the job's own ring, so a job's results do not depend on its pack.
__global__ void pack_advance_kernel(int *n0, int njobs, int k) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < njobs) n0[q] += k;
}

struct fdtd::Pack {
  std::vector<fdtd_job *> jobs;
  int layout = 0, vec = 1;
  bool f64 = false;
  cudaStream_t stream = nullptr, side[2] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[2] = {};
  void *d_tab = nullptr;  // [2 halves][kStageSteps slots][jobs] StepParams
  int *d_n0 = nullptr;    // first step of each job's current ring
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int kernels_per_ring = 0;
};

namespace {

template <typename T>
int pack_capture(fdtd::Pack *P) {
  const int nj = (int)P->jobs.size();
  std::vector<StepParams<T>> tab((size_t)2 * kStageSteps * nj);
  for (int s = 0; s < kStageSteps; ++s)
    for (int q = 0; q < nj; ++q) {
      fdtd_job *J = P->jobs[q];
      StepParams<T> &e = tab[(size_t)s * nj + q];
      fill_common<T>(J, e);
      set_sources<T>(J, e);
      e.roles = ROLE_MAIN | ROLE_PML | ROLE_ADE;
      e.slot = s;
      e.d_base = P->d_n0 + q;
      StepParams<T> &h = tab[((size_t)kStageSteps + s) * nj + q];
      fill_common<T>(J, h);
      h.roles = ROLE_MAIN | ROLE_PML;
      h.gather = 1;
      h.slot = s;
      h.d_base = P->d_n0 + q;
    }
  CK(cudaMallocAsync(&P->d_tab, tab.size() * sizeof(StepParams<T>), P->stream));
  CK(cudaMemcpyAsync(P->d_tab, tab.data(), tab.size() * sizeof(StepParams<T>), cudaMemcpyHostToDevice, P->stream));
  CK(cudaStreamSynchronize(P->stream));
  // block ranges of each job in the five launches of a step
  PackLaunch<T> L[2][3];
  for (int h = 0; h < 2; ++h)
    for (int part = 0; part < 3; ++part) {
      PackLaunch<T> &a = L[h][part];
      memset(&a, 0, sizeof a);
      a.njobs = nj;
      int b = 0;
      for (int q = 0; q < nj; ++q) {
        const fdtd_job *J = P->jobs[q];
        const long long units = part == K2D_CORE ? J->ncore : part == K2D_EDGE ? J->nedge : (h == 0 ? J->nade : 0);
        a.bstart[q] = b;
        b += (int)((units + 255) / 256);
      }
      a.bstart[nj] = b;
    }
  const StepParams<T> *base = (const StepParams<T> *)P->d_tab;
  int kernels = 0;
  CK(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t bad = cudaSuccess;
  for (int s = 0; s < kStageSteps && bad == cudaSuccess; ++s)
    for (int h = 0; h < 2 && bad == cudaSuccess; ++h) {
      int use[3], nuse = 0;
      for (int part = 0; part < (h == 0 ? 3 : 2); ++part)
        if (L[h][part].bstart[nj] > 0) use[nuse++] = part;
      cudaStream_t st[3] = {P->stream, P->stream, P->stream};
      if (nuse > 1) {
        bad = cudaEventRecord(P->ev_fork, P->stream);
        for (int b = 1; b < nuse && bad == cudaSuccess; ++b) {
          st[b] = P->side[b - 1];
          bad = cudaStreamWaitEvent(st[b], P->ev_fork, 0);
        }
      }
      for (int b = 0; b < nuse && bad == cudaSuccess; ++b) {
        PackLaunch<T> a = L[h][use[b]];
        a.tab = base + ((size_t)h * kStageSteps + s) * nj;
        kernels += launch_pack2d<T>(a, P->layout, P->vec, h == 0, use[b], st[b]);
      }
      for (int b = 1; b < nuse && bad == cudaSuccess; ++b) {
        bad = cudaEventRecord(P->ev_join[b - 1], st[b]);
        if (bad == cudaSuccess) bad = cudaStreamWaitEvent(P->stream, P->ev_join[b - 1], 0);
      }
      if (bad == cudaSuccess) bad = cudaGetLastError();
    }
  for (int q = 0; q < nj && bad == cudaSuccess; ++q) {  // each job's DFT fold of the ring
    fdtd_job *J = P->jobs[q];
    if (J->mon_dev.empty() || J->dft_blocks <= 0) continue;
    DftParams d{};
    d.nmon = (int)J->mon_dev.size();
    for (int m = 0; m < d.nmon; ++m) d.mon[m] = J->mon_dev[m];
    d.omega = J->d_omega;
    d.rot = (const double2 *)J->d_rot;
    d.acc_re = J->d_acc_re;
    d.acc_im = J->d_acc_im;
    d.dt = J->g.dt;
    d.stage_row = J->stage_row;
    d.total_work_blocks = J->dft_blocks;
    d.nslots = kStageSteps;
    d.d_base = P->d_n0 + q;
    // the job's current half of its stage buffer, where its pack steps stage
    launch_dft<T>(d, (const T *)J->d_stage + (size_t)J->stage_half * kStageSteps * J->stage_row, P->stream);
    ++kernels;
    bad = cudaGetLastError();
  }
  if (bad == cudaSuccess) {
    pack_advance_kernel<<<(nj + 31) / 32, 32, 0, P->stream>>>(P->d_n0, nj, kStageSteps);
    ++kernels;
    bad = cudaGetLastError();
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(P->stream, &g);
  if (bad != cudaSuccess || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return set_err(FDTD_ECUDA, "pack graph capture: %s", cudaGetErrorString(bad != cudaSuccess ? bad : e));
  }
  P->graph = g;
  CK(cudaGraphInstantiate(&P->exec, P->graph, 0));
  P->kernels_per_ring = kernels;
  return FDTD_OK;
}

}  // namespace

long long fdtd::pack_key(const fdtd_job *J) {
  if (!J || !J->committed || J->dim != 2 || !J->gather_fused || J->prof || J->stage_fill != 0) return -1;
  return ((long long)J->g.precision * 16 + J->g.layout) * 16 + J->vec;
}

int fdtd::job_reserve(fdtd_job *J, int n_last) {
  if (!J || !J->committed) return set_err(FDTD_ESTATE, "job not committed");
  int rc = ensure_probe_cap(J, n_last);
  if (!rc && J->dim >= 2) rc = ensure_srctab(J, n_last);
  return rc;
}

void fdtd::pack_destroy(fdtd::Pack *P) {
  if (!P) return;
  if (P->stream) cudaStreamSynchronize(P->stream);
  if (P->exec) cudaGraphExecDestroy(P->exec);
  if (P->graph) cudaGraphDestroy(P->graph);
  if (P->d_tab) cudaFreeAsync(P->d_tab, P->stream);
  if (P->d_n0) cudaFreeAsync(P->d_n0, P->stream);
  for (int q = 0; q < 2; ++q) {
    if (P->side[q]) cudaStreamDestroy(P->side[q]);
    if (P->ev_join[q]) cudaEventDestroy(P->ev_join[q]);
  }
  if (P->ev_fork) cudaEventDestroy(P->ev_fork);
  if (P->stream) cudaStreamDestroy(P->stream);
  delete P;
}

int fdtd::pack_create(fdtd_job *const *jobs, int njobs, fdtd::Pack **out) {
  *out = nullptr;
  if (njobs < 1 || njobs > kMaxPack) return set_err(FDTD_EINVAL, "a pack holds 1..%d jobs", kMaxPack);
  const long long key = pack_key(jobs[0]);
  for (int q = 0; q < njobs; ++q)
    if (key < 0 || pack_key(jobs[q]) != key) return set_err(FDTD_EINVAL, "jobs of a pack must be 2D jobs of one kind");
  fdtd::Pack *P = new fdtd::Pack;
  P->jobs.assign(jobs, jobs + njobs);
  P->layout = jobs[0]->g.layout;
  P->vec = jobs[0]->vec;
  P->f64 = jobs[0]->g.precision == FDTD_F64;
  bool ok = cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&P->ev_fork, cudaEventDisableTiming) == cudaSuccess;
  for (int q = 0; q < 2 && ok; ++q)
    ok = cudaStreamCreateWithFlags(&P->side[q], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&P->ev_join[q], cudaEventDisableTiming) == cudaSuccess;
  std::vector<int> n0(njobs);
  for (int q = 0; q < njobs && ok; ++q) {
    ok = cudaStreamSynchronize(jobs[q]->stream) == cudaSuccess;  // the job's own work is done
    n0[q] = jobs[q]->last_n + 1;
  }
  if (ok) ok = cudaMallocAsync((void **)&P->d_n0, njobs * sizeof(int), P->stream) == cudaSuccess &&
               cudaMemcpyAsync(P->d_n0, n0.data(), njobs * sizeof(int), cudaMemcpyHostToDevice, P->stream) == cudaSuccess &&
               cudaStreamSynchronize(P->stream) == cudaSuccess;
  if (!ok) {
    pack_destroy(P);
    return set_err(FDTD_ECUDA, "pack set-up failed");
  }
  const int rc = P->f64 ? pack_capture<double>(P) : pack_capture<float>(P);
  if (rc) {
    pack_destroy(P);
    return rc;
  }
  *out = P;
  return FDTD_OK;
}

int fdtd::pack_run(fdtd::Pack *P, int rings, cudaEvent_t done) {
  for (int r = 0; r < rings; ++r) CK(cudaGraphLaunch(P->exec, P->stream));
  if (done) CK(cudaEventRecord(done, P->stream));
  const int nj = (int)P->jobs.size();
  for (fdtd_job *J : P->jobs) {  // the jobs' own step bookkeeping, as after their own rings
    J->last_n += rings * kStageSteps;
    J->stage_n0 = J->last_n + 1;
    J->launches += (long long)rings * ((P->kernels_per_ring + nj - 1) / nj);
  }
  return FDTD_OK;
}

// =========================================================================
extern "C" {

int fdtd_last_error(char *buf, size_t len) {
  if (buf && len) {
    snprintf(buf, len, "%s", g_last_error.c_str());
  }
  return FDTD_OK;
}

int fdtd_device_count(int32_t *count) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  int usable = 0;
  for (int d = 0; d < n; ++d) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, d) == cudaSuccess && prop.major == 10 && prop.minor == 3) ++usable;
  }
  if (count) *count = usable;
  return FDTD_OK;
}

int fdtd_create(const fdtd_grid_desc *g, fdtd_job **out) {
  if (!g || !out) return set_err(FDTD_EINVAL, "null argument");
  *out = nullptr;
  int dim;
  switch (g->layout) {
    case FDTD_LAYOUT_1D: dim = 1; break;
    case FDTD_LAYOUT_2D_TE: case FDTD_LAYOUT_2D_TM: dim = 2; break;
    case FDTD_LAYOUT_3D: dim = 3; break;
    default: return set_err(FDTD_EINVAL, "bad layout %d", g->layout);
  }
  if (g->precision != FDTD_F32 && g->precision != FDTD_F64) return set_err(FDTD_EINVAL, "bad precision");
  for (int a = 0; a < 3; ++a)
    if (g->n[a] < 1) return set_err(FDTD_EINVAL, "n[%d] < 1", a);
  if (dim == 1 && (g->n[0] != 1 || g->n[2] != 1)) return set_err(FDTD_EINVAL, "1D runs along y: n = (1, N, 1)");
  if (dim == 2 && g->n[2] != 1) return set_err(FDTD_EINVAL, "2D needs n[2] = 1");
  const long long N = (long long)g->n[0] * g->n[1] * g->n[2];
  if (N >= (1LL << 31)) return set_err(FDTD_ERANGE, "grid of %lld cells exceeds 2^31", N);
  if (g->dt <= 0 || g->ds <= 0) return set_err(FDTD_EINVAL, "dt and ds must be positive");
  int dev = 0, rc = check_device(&dev);
  if (rc) return rc;
  fdtd_job *J = new fdtd_job();
  J->g = *g;
  J->dim = dim;
  J->nx = g->n[0]; J->ny = g->n[1]; J->nz = g->n[2];
  J->ncell = N;
  J->esz = g->precision == FDTD_F32 ? 4 : 8;
  J->device = dev;
  cudaDeviceGetAttribute(&J->num_sms, cudaDevAttrMultiProcessorCount, dev);
  for (int a = 0; a < 3; ++a) {
    J->g.main_lo[a] = std::max(0, g->main_lo[a]);
    J->g.main_hi[a] = std::min(g->n[a] - 1, g->main_hi[a]);
  }
  if (cudaStreamCreateWithFlags(&J->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete J;
    return set_err(FDTD_ECUDA, "cudaStreamCreate failed");
  }
  J->own_stream = J->stream;
  const char *ng = getenv("FDTD_NO_GRAPH");
  J->use_graph = !(ng && ng[0] == '1');
  *out = J;
  return FDTD_OK;
}

int fdtd_destroy(fdtd_job *J) {
  if (!J) return FDTD_OK;
  if (J->stream) cudaStreamSynchronize(J->stream);
  J->stream = J->own_stream;  // the frees queue on the job's own stream
  for (void *p : J->allocs) pool_free(J, p);
  for (auto &P : J->probes) pool_free(J, P.buf);
  pool_free(J, J->d_srcval);
  pool_free(J, J->d_srctab);
  destroy_graph(J);
  for (auto &e : J->pending) { cudaEventDestroy(e.a); if (e.b) cudaEventDestroy(e.b); }
  for (auto e : J->ev_pool) cudaEventDestroy(e);
  for (int q = 0; q < 2; ++q) {
    if (J->side[q]) cudaStreamDestroy(J->side[q]);
    if (J->ev_join[q]) cudaEventDestroy(J->ev_join[q]);
    if (J->ev_prog[q]) cudaEventDestroy(J->ev_prog[q]);
  }
  if (J->ev_fork) cudaEventDestroy(J->ev_fork);
  if (J->fold_stream) cudaStreamDestroy(J->fold_stream);
  if (J->ev_ffork) cudaEventDestroy(J->ev_ffork);
  if (J->ev_fjoin) cudaEventDestroy(J->ev_fjoin);
  if (J->own_stream) cudaStreamDestroy(J->own_stream);
  delete J;
  return FDTD_OK;
}

static int add_mat(fdtd_job *J, const fdtd_region *r, MatRec &m, int32_t *id) {
  int rc = check_job(J, false);
  if (rc) return rc;
  if (!r) return set_err(FDTD_EINVAL, "null region");
  if (J->mats.size() >= (size_t)(kMaxMat - 1)) return set_err(FDTD_ERANGE, "too many materials");
  m.region = *r;
  if (r->kind == FDTD_REGION_SPHERES) {
    if (r->count < 0 || (r->count > 0 && !r->centers_radii)) return set_err(FDTD_EINVAL, "bad spheres");
    m.centers.assign(r->centers_radii, r->centers_radii + 4 * (size_t)r->count);
    m.region.centers_radii = nullptr;
  } else if (r->kind == FDTD_REGION_MASK) {
    if (!r->mask) return set_err(FDTD_EINVAL, "null mask");
    m.mask.assign(r->mask, r->mask + J->ncell);
    m.region.mask = nullptr;
  } else if (r->kind != FDTD_REGION_BOX) {
    return set_err(FDTD_EINVAL, "bad region kind %d", r->kind);
  }
  J->mats.push_back(m);
  if (id) *id = (int32_t)J->mats.size();
  return FDTD_OK;
}

int fdtd_add_dielectric(fdtd_job *J, const fdtd_region *r, double eps, int32_t *id) {
  MatRec m{};
  m.kind = MK_DIEL;
  m.eps = eps;
  return add_mat(J, r, m, id);
}

int fdtd_add_gold(fdtd_job *J, const fdtd_region *r, const fdtd_drude2cp *p, int32_t *id) {
  if (!p) return set_err(FDTD_EINVAL, "null gold parameters");
  if (p->gamma_d <= 0) return set_err(FDTD_EINVAL, "gamma_d must be positive");
  MatRec m{};
  m.kind = MK_GOLD;
  m.gold = *p;
  return add_mat(J, r, m, id);
}

int fdtd_add_graphene(fdtd_job *J, const fdtd_region *r, const fdtd_graphene_desc *p, int32_t *id) {
  if (!p || !r) return set_err(FDTD_EINVAL, "null argument");
  if (r->kind != FDTD_REGION_BOX) return set_err(FDTD_EINVAL, "graphene needs a one-cell-thick box");
  bool thin = false;
  for (int a = 0; a < 3; ++a) if (r->lo[a] == r->hi[a] && J && J->g.n[a] > 1) thin = true;
  if (!thin) return set_err(FDTD_EINVAL, "graphene box must be one cell thick");
  if (p->tau <= 0 || p->thickness <= 0 || p->raman_tau <= 0) return set_err(FDTD_EINVAL, "bad graphene parameters");
  MatRec m{};
  m.kind = MK_GRAPHENE;
  m.gr = *p;
  return add_mat(J, r, m, id);
}

int fdtd_add_graphene_nk(fdtd_job *J, const fdtd_region *r, const fdtd_graphene_nk_desc *p, int32_t *id) {
  if (!p) return set_err(FDTD_EINVAL, "null graphene parameters");
  if (!std::isfinite(p->n) || !std::isfinite(p->k) || !(p->wavelength > 0) || !(p->scale >= 0) ||
      !std::isfinite(p->chi3) || !std::isfinite(p->alpha))
    return set_err(FDTD_EINVAL, "graphene_nk needs finite n, k, chi3, alpha, wavelength > 0 and scale >= 0");
  if (p->chi3 != 0.0 && !(p->w_nl > p->gamma_nl && p->gamma_nl >= 0))
    return set_err(FDTD_EINVAL, "the Raman term needs w_nl > gamma_nl >= 0");
  MatRec m{};
  m.kind = MK_GRAPHENE_NK;
  m.gnk = *p;
  return add_mat(J, r, m, id);
}

int fdtd_add_conductive(fdtd_job *J, const fdtd_region *r, double eps_inf, double sigma, int32_t *id) {
  if (!std::isfinite(eps_inf) || !std::isfinite(sigma) || sigma < 0 || !(eps_inf + sigma > 0))
    return set_err(FDTD_EINVAL, "a conductive dielectric needs finite eps_inf, sigma >= 0 and eps_inf + sigma dt/eps0 > 0");
  MatRec m{};
  m.kind = MK_CONDUCTIVE;
  m.eps = eps_inf;
  m.sigma = sigma;
  return add_mat(J, r, m, id);
}

int fdtd_add_graphene_cp(fdtd_job *J, const fdtd_region *r, const fdtd_graphene_cp_desc *p, int32_t *id) {
  if (!p) return set_err(FDTD_EINVAL, "null graphene parameters");
  bool ok = std::isfinite(p->eps_inf) && std::isfinite(p->drude_omega) && p->drude_gamma > 0 && p->width > 0;
  for (int q = 0; q < 4; ++q)
    ok = ok && std::isfinite(p->amp[q]) && std::isfinite(p->phi[q]) && std::isfinite(p->omega[q]) && std::isfinite(p->gamma[q]);
  if (!ok) return set_err(FDTD_EINVAL, "graphene needs finite parameters, drude_gamma > 0 and width > 0");
  if (p->normal_axis < -1 || p->normal_axis > 2) return set_err(FDTD_EINVAL, "normal_axis %d outside -1..2", p->normal_axis);
  if (p->chi3 != 0.0) {
    if (p->raman_form != FDTD_RAMAN_EXACT && p->raman_form != FDTD_RAMAN_CENTRAL)
      return set_err(FDTD_EINVAL, "bad Raman form %d", p->raman_form);
    if (!std::isfinite(p->chi3) || !(p->gamma_nl >= 0) || !std::isfinite(p->w_nl))
      return set_err(FDTD_EINVAL, "bad Raman parameters");
    if (p->raman_form == FDTD_RAMAN_EXACT && !(p->w_nl > 0.5 * p->gamma_nl))
      return set_err(FDTD_EINVAL, "the exact Raman form needs w_nl > gamma_nl/2");
  }
  MatRec m{};
  m.kind = MK_GRAPHENE_CP;
  m.gcp = *p;
  return add_mat(J, r, m, id);
}

int fdtd_add_lorentz(fdtd_job *J, const fdtd_region *r, const fdtd_lorentz_desc *p, int32_t *id) {
  if (!p) return set_err(FDTD_EINVAL, "null Lorentz parameters");
  if (p->form != FDTD_LORENTZ_JP && p->form != FDTD_LORENTZ_S) return set_err(FDTD_EINVAL, "bad Lorentz form %d", p->form);
  if (p->npoles < 1 || p->npoles > FDTD_LORENTZ_MAX_POLES)
    return set_err(FDTD_EINVAL, "npoles %d outside 1..%d", p->npoles, FDTD_LORENTZ_MAX_POLES);
  if (!(p->eps_inf != 0.0) || !std::isfinite(p->eps_inf)) return set_err(FDTD_EINVAL, "eps_inf must be finite and nonzero");
  if (p->chi3 != 0.0 && p->form != FDTD_LORENTZ_JP) return set_err(FDTD_EINVAL, "the Kerr term needs the JP form");
  if (p->ez_uses_x_current && (p->form != FDTD_LORENTZ_JP || !J || J->g.layout != FDTD_LAYOUT_3D || !p->sheet ||
                                !r || r->lo[1] != r->hi[1]))
    return set_err(FDTD_EINVAL, "ez_uses_x_current needs the JP form and a sheet normal to y on a 3D grid");
  if (p->sheet) {
    if (!r || r->kind != FDTD_REGION_BOX) return set_err(FDTD_EINVAL, "a Lorentz sheet needs a one-cell-thick box");
    bool thin = false;
    for (int a = 0; a < 3; ++a) if (r->lo[a] == r->hi[a] && J && J->g.n[a] > 1) thin = true;
    if (!thin) return set_err(FDTD_EINVAL, "a Lorentz sheet must be one cell thick");
  }
  MatRec m{};
  m.kind = MK_LORENTZ;
  m.lz = *p;
  return add_mat(J, r, m, id);
}

int fdtd_add_pml(fdtd_job *J, const fdtd_pml_desc *p) {
  int rc = check_job(J, false);
  if (rc) return rc;
  if (!p) return set_err(FDTD_EINVAL, "null pml");
  if (p->mode != FDTD_PML_REFERENCE && p->mode != FDTD_PML_SPLIT) return set_err(FDTD_EINVAL, "bad pml mode");
  if (p->mode == FDTD_PML_SPLIT && J->dim == 1) return set_err(FDTD_EINVAL, "1D uses the reference PML");
  if (p->mode == FDTD_PML_REFERENCE && J->g.layout == FDTD_LAYOUT_2D_TM)
    return set_err(FDTD_EINVAL, "2D TM uses the split PML");
  const int n[3] = {J->nx, J->ny, J->nz};
  for (int a = 0; a < 3; ++a)
    for (int s = 0; s < 2; ++s)
      if (p->npml[a][s] < 0 || 2 * p->npml[a][s] >= n[a] + (n[a] == 1 ? 2 : 0))
        return set_err(FDTD_EINVAL, "npml[%d][%d] = %d does not fit the grid", a, s, p->npml[a][s]);
  if (p->mode == FDTD_PML_REFERENCE && p->npml[1][0] != p->npml[1][1])
    return set_err(FDTD_EINVAL, "reference PML: both y slabs have npmly cells");
  J->has_pml = true;
  J->pml = *p;
  return FDTD_OK;
}

int fdtd_add_tfsf_1d(fdtd_job *J, const fdtd_tfsf1d_desc *t) {
  int rc = check_job(J, false);
  if (rc) return rc;
  if (!t) return set_err(FDTD_EINVAL, "null tfsf");
  if (J->dim != 1) return set_err(FDTD_EINVAL, "TFSF line is 1D only");
  if (t->boundary < 1 || t->boundary >= J->ny) return set_err(FDTD_ERANGE, "TFSF boundary out of range");
  J->has_tfsf = true;
  J->tfsf = *t;
  return FDTD_OK;
}

int fdtd_add_tfsf(fdtd_job *J, const fdtd_tfsf_desc *t) {
  int rc = check_job(J, false);
  if (rc) return rc;
  if (!t) return set_err(FDTD_EINVAL, "null tfsf");
  if (J->dim < 2) return set_err(FDTD_EINVAL, "the TFSF box is 2D/3D; a 1D line uses fdtd_add_tfsf_1d");
  if (J->has_tfbox) return set_err(FDTD_ESTATE, "the job already has a TFSF box");
  if (!(t->eps_line > 0.0) || !std::isfinite(t->eps_line)) return set_err(FDTD_EINVAL, "eps_line must be positive");
  J->has_tfbox = true;
  J->tfbox = *t;
  if (J->dim == 2) J->tfbox.lo[2] = J->tfbox.hi[2] = 0;
  return FDTD_OK;
}

int fdtd_add_source(fdtd_job *J, const fdtd_source_desc *s, int32_t *id) {
  int rc = check_job(J, false);
  if (rc) return rc;
  if (!s) return set_err(FDTD_EINVAL, "null source");
  if (J->srcs.size() >= (size_t)kMaxSrc) return set_err(FDTD_ERANGE, "too many sources");
  if (!(s->component >= FDTD_EX && s->component <= FDTD_EZ) && s->component != FDTD_EX_INC)
    return set_err(FDTD_EINVAL, "source drives an E component");
  if (s->st == 0) return set_err(FDTD_EINVAL, "source width st = 0");
  J->srcs.push_back(*s);
  if (id) *id = (int32_t)J->srcs.size() - 1;
  return FDTD_OK;
}

int fdtd_add_monitor(fdtd_job *J, const fdtd_monitor_desc *m, int32_t *id) {
  int rc = check_job(J, false);
  if (rc) return rc;
  if (!m || (m->nfreq > 0 && !m->omega)) return set_err(FDTD_EINVAL, "null monitor");
  if (J->mons.size() >= (size_t)kMaxMon) return set_err(FDTD_ERANGE, "too many monitors");
  const int n[3] = {J->nx, J->ny, J->nz};
  for (int a = 0; a < 3; ++a)
    if (m->lo[a] < 0 || m->hi[a] >= n[a] || m->lo[a] > m->hi[a]) return set_err(FDTD_ERANGE, "monitor box out of grid");
  if (m->nfreq < 1) return set_err(FDTD_EINVAL, "monitor needs frequencies");
  MonRec R;
  R.d = *m;
  R.omega.assign(m->omega, m->omega + m->nfreq);
  R.d.omega = nullptr;
  R.ncomp = comp_list(m->comp_mask, R.comps, 6);
  if (R.ncomp <= 0) return set_err(FDTD_EINVAL, "monitor needs 1..6 components");
  for (int u = 0; u < R.ncomp; ++u)
    if ((R.comps[u] >= FDTD_EX_INC) != (J->dim == 1 && R.comps[u] >= FDTD_EX_INC) ||
        (R.comps[u] >= FDTD_EX_INC && !J->has_tfsf))
      return set_err(FDTD_EINVAL, "component %d not available", R.comps[u]);
  if (m->reduce != FDTD_MONITOR_CELLS && m->reduce != FDTD_MONITOR_MEAN)
    return set_err(FDTD_EINVAL, "monitor reduce must be FDTD_MONITOR_CELLS or FDTD_MONITOR_MEAN");
  if (m->reduce == FDTD_MONITOR_MEAN && J->dim == 1) return set_err(FDTD_EINVAL, "mean monitors need a 2D or 3D job");
  R.boxcells = (long long)(m->hi[0] - m->lo[0] + 1) * (m->hi[1] - m->lo[1] + 1) * (m->hi[2] - m->lo[2] + 1);
  R.ncell = m->reduce == FDTD_MONITOR_MEAN ? 1 : R.boxcells;
  J->mons.push_back(R);
  if (id) *id = (int32_t)J->mons.size() - 1;
  return FDTD_OK;
}

int fdtd_add_probe(fdtd_job *J, const fdtd_probe_desc *p, int32_t *id) {
  int rc = check_job(J, false);
  if (rc) return rc;
  if (!p) return set_err(FDTD_EINVAL, "null probe");
  if (J->probes.size() >= (size_t)kMaxProbe) return set_err(FDTD_ERANGE, "too many probes");
  const int n[3] = {J->nx, J->ny, J->nz};
  for (int a = 0; a < 3; ++a)
    if (p->cell[a] < 0 || p->cell[a] >= n[a]) return set_err(FDTD_ERANGE, "probe cell out of grid");
  ProbeRec R;
  R.d = *p;
  R.ncomp = comp_list(p->comp_mask, R.comps, 8);
  if (R.ncomp <= 0) return set_err(FDTD_EINVAL, "probe needs components");
  J->probes.push_back(R);
  if (id) *id = (int32_t)J->probes.size() - 1;
  return FDTD_OK;
}

int fdtd_commit(fdtd_job *J) {
  NvtxRange nvtx_("fdtd_commit");
  int rc = check_job(J, false);
  if (rc) return rc;
  if (J->dim == 1 && J->has_pml && J->pml.npml[1][0] < 1) return set_err(FDTD_EINVAL, "1D PML needs npmly >= 1");
  return DISPATCH(J, commit_impl)(J);
}

int fdtd_step(fdtd_job *J, int32_t n_first, int32_t n_steps) {
  NvtxRange nvtx_("fdtd_step");
  int rc = check_job(J, true);
  if (rc) return rc;
  if (n_steps < 0 || n_first < 1) return set_err(FDTD_EINVAL, "bad step range");
  if (n_steps == 0) return FDTD_OK;
  return DISPATCH(J, step_impl)(J, n_first, n_steps);
}

// ---- health checks ---------------------------------------------------------
int fdtd_check_finite(fdtd_job *J, int64_t *count) {
  NvtxRange nvtx_("fdtd_check_finite");
  int rc = check_job(J, true);
  if (rc) return rc;
  if (!count) return set_err(FDTD_EINVAL, "null count");
  if (!J->d_count && (rc = alloc_dev(J, (void **)&J->d_count, sizeof(unsigned long long)))) return rc;
  CK(cudaMemsetAsync(J->d_count, 0, sizeof(unsigned long long), J->stream));
  for (auto &s : J->state)
    if (launch_count_nonfinite(s.p, s.bytes, s.esz, J->d_count, J->num_sms, J->stream))
      return set_err(FDTD_ECUDA, "non-finite count launch failed");
  for (auto &P : J->probes)
    if (P.buf && launch_count_nonfinite(P.buf, (size_t)P.cap * P.ncomp * sizeof(double), 8, J->d_count, J->num_sms,
                                        J->stream))
      return set_err(FDTD_ECUDA, "non-finite count launch failed");
  J->launches += J->state.size() + J->probes.size();
  unsigned long long h = 0;
  CK(cudaMemcpyAsync(&h, J->d_count, sizeof h, cudaMemcpyDeviceToHost, J->stream));
  CK(cudaStreamSynchronize(J->stream));
  J->prog_prev = -1;
  *count = (int64_t)h;
  return FDTD_OK;
}

int fdtd_debug_wait_limit(fdtd_job *J, int32_t rounds) {
  if (!J) return set_err(FDTD_EINVAL, "null job");
  J->wait_limit = rounds < 0 ? kWaitLimit : (unsigned)rounds;
  destroy_graph(J);  // the captured launches hold the old limit
  return FDTD_OK;
}

int fdtd_debug_fail_alloc(int32_t after) {
  g_fail_after.store(after < 0 ? -1 : (long long)after);
  return FDTD_OK;
}

// ---- checkpoint ----------------------------------------------------------
// Layout: CkptHeader, then per state buffer its size (uint64), per probe its
// rows and components (int32 pairs), then the buffers' bytes in allocation
// order and the probes' rows.  The unfolded part of the DFT ring is part of
// the stage buffer (both halves), with stage_fill, stage_n0 and the half in
// use in the header, so a resumed job folds the same rings as the saved one
// would have.
struct CkptHeader {
  char magic[8];
  uint32_t version;
  int32_t layout, precision, n[3];
  uint32_t nbuf, nprobe;
  int32_t stage_fill, stage_n0, last_n, stage_half;  // stage_half: the ring in progress's half of the stage buffer
  uint64_t total;
};
constexpr char kCkptMagic[8] = {'F', 'D', 'T', 'D', 'C', 'K', 'P', 'T'};

static uint64_t ckpt_bytes(const fdtd_job *J) {
  uint64_t b = sizeof(CkptHeader) + J->state.size() * sizeof(uint64_t) + J->probes.size() * 2 * sizeof(int32_t);
  for (auto &s : J->state) b += s.bytes;
  for (auto &P : J->probes) b += (uint64_t)P.cap * P.ncomp * sizeof(double);
  return b;
}

int fdtd_state_bytes(const fdtd_job *J, uint64_t *bytes) {
  if (!J || !bytes) return set_err(FDTD_EINVAL, "null argument");
  if (!J->committed) return set_err(FDTD_ESTATE, "the job is not committed");
  *bytes = ckpt_bytes(J);
  return FDTD_OK;
}

int fdtd_save_state(fdtd_job *J, void *buf, uint64_t bytes) {
  NvtxRange nvtx_("fdtd_save_state");
  int rc = check_job(J, true);
  if (rc) return rc;
  if (!buf) return set_err(FDTD_EINVAL, "null buffer");
  const uint64_t need = ckpt_bytes(J);
  if (bytes < need) return set_err(FDTD_ERANGE, "checkpoint needs %llu bytes, got %llu", (unsigned long long)need,
                                   (unsigned long long)bytes);
  // the step boundary: everything queued has run; the ring is not folded
  CK(cudaStreamSynchronize(J->stream));
  CK(cudaGetLastError());
  char *o = (char *)buf;
  CkptHeader h{};
  memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.layout = J->g.layout;
  h.precision = J->g.precision;
  for (int a = 0; a < 3; ++a) h.n[a] = J->g.n[a];
  h.nbuf = (uint32_t)J->state.size();
  h.nprobe = (uint32_t)J->probes.size();
  h.stage_fill = J->stage_fill;
  h.stage_half = J->stage_half;
  h.stage_n0 = J->stage_n0;
  h.last_n = J->last_n;
  h.total = need;
  memcpy(o, &h, sizeof h);
  o += sizeof h;
  for (auto &s : J->state) {
    const uint64_t b = s.bytes;
    memcpy(o, &b, sizeof b);
    o += sizeof b;
  }
  for (auto &P : J->probes) {
    const int32_t rc2[2] = {P.cap, P.ncomp};
    memcpy(o, rc2, sizeof rc2);
    o += sizeof rc2;
  }
  for (auto &s : J->state) {
    CK(cudaMemcpy(o, s.p, s.bytes, cudaMemcpyDeviceToHost));
    o += s.bytes;
  }
  for (auto &P : J->probes) {
    const size_t b = (size_t)P.cap * P.ncomp * sizeof(double);
    if (b) CK(cudaMemcpy(o, P.buf, b, cudaMemcpyDeviceToHost));
    o += b;
  }
  J->d2h += need;
  return FDTD_OK;
}

int fdtd_load_state(fdtd_job *J, const void *buf, uint64_t bytes) {
  NvtxRange nvtx_("fdtd_load_state");
  int rc = check_job(J, true);
  if (rc) return rc;
  if (!buf || bytes < sizeof(CkptHeader)) return set_err(FDTD_EINVAL, "null or short checkpoint");
  const char *in = (const char *)buf;
  CkptHeader h;
  memcpy(&h, in, sizeof h);
  if (memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1) return set_err(FDTD_EINVAL, "not a checkpoint of this library");
  if (h.total != bytes) return set_err(FDTD_EINVAL, "checkpoint of %llu bytes given as %llu", (unsigned long long)h.total,
                                       (unsigned long long)bytes);
  bool same = h.layout == J->g.layout && h.precision == J->g.precision && h.nbuf == J->state.size() &&
              h.nprobe == J->probes.size();
  for (int a = 0; a < 3; ++a) same = same && h.n[a] == J->g.n[a];
  if (!same) return set_err(FDTD_EINVAL, "the checkpoint comes from a job of another layout, precision, size or set-up");
  // the size table and the probe records must lie inside the buffer before
  // they are read; the whole layout they describe must then fill it exactly
  const uint64_t tables = sizeof h + J->state.size() * sizeof(uint64_t) + J->probes.size() * 2 * sizeof(int32_t);
  if (bytes < tables) return set_err(FDTD_EINVAL, "checkpoint of %llu bytes is shorter than its tables",
                                     (unsigned long long)bytes);
  const char *sz = in + sizeof h;
  for (size_t q = 0; q < J->state.size(); ++q) {
    uint64_t b;
    memcpy(&b, sz + q * sizeof b, sizeof b);
    if (b != J->state[q].bytes) return set_err(FDTD_EINVAL, "checkpoint buffer %zu holds %llu bytes, the job %zu", q,
                                               (unsigned long long)b, J->state[q].bytes);
  }
  const char *pr = sz + J->state.size() * sizeof(uint64_t);
  int n_probe_max = 0;
  std::vector<int32_t> caps(J->probes.size());
  for (size_t q = 0; q < J->probes.size(); ++q) {
    int32_t rc2[2];
    memcpy(rc2, pr + q * sizeof rc2, sizeof rc2);
    if (rc2[1] != J->probes[q].ncomp || rc2[0] < 0) return set_err(FDTD_EINVAL, "checkpoint probe %zu does not match", q);
    caps[q] = rc2[0];
    if (rc2[0] > 0) n_probe_max = std::max(n_probe_max, J->probes[q].d.n_first + rc2[0] - 1);
  }
  uint64_t expect = tables;
  for (auto &st : J->state) expect += st.bytes;
  for (size_t q = 0; q < J->probes.size(); ++q) expect += (uint64_t)caps[q] * J->probes[q].ncomp * sizeof(double);
  if (expect != bytes) return set_err(FDTD_EINVAL, "checkpoint of %llu bytes, its tables describe %llu",
                                      (unsigned long long)bytes, (unsigned long long)expect);
  CK(cudaStreamSynchronize(J->stream));
  if (n_probe_max > 0 && (rc = ensure_probe_cap(J, n_probe_max))) return rc;
  const char *o = pr + J->probes.size() * 2 * sizeof(int32_t);
  for (auto &s : J->state) {
    CK(cudaMemcpy(s.p, o, s.bytes, cudaMemcpyHostToDevice));
    o += s.bytes;
  }
  for (size_t q = 0; q < J->probes.size(); ++q) {
    ProbeRec &P = J->probes[q];
    const size_t b = (size_t)caps[q] * P.ncomp * sizeof(double);
    if (P.buf && P.cap > 0) CK(cudaMemset(P.buf, 0, (size_t)P.cap * P.ncomp * sizeof(double)));
    if (b) CK(cudaMemcpy(P.buf, o, b, cudaMemcpyHostToDevice));
    o += b;
  }
  J->stage_fill = h.stage_fill;
  J->stage_half = h.stage_half & 1;
  J->fold_pending = false;
  J->stage_n0 = h.stage_n0;
  J->last_n = h.last_n;
  J->prog_prev = -1;
  J->h2d += bytes;
  return FDTD_OK;
}

int fdtd_update_DE(fdtd_job *J, int32_t n) {
  NvtxRange nvtx_("fdtd_update_DE");
  int rc = check_job(J, true);
  return rc ? rc : DISPATCH(J, proc_call)(J, n, 0);
}
int fdtd_pml_update_E(fdtd_job *J, int32_t n) {
  NvtxRange nvtx_("fdtd_pml_update_E");
  int rc = check_job(J, true);
  return rc ? rc : DISPATCH(J, proc_call)(J, n, 1);
}
int fdtd_interchange(fdtd_job *J, int32_t which) {
  int rc = check_job(J, true);
  if (rc) return rc;
  if (which != 0 && which != 1) return set_err(FDTD_EINVAL, "interchange: 0 = E, 1 = H");
  return FDTD_OK;  // one domain: the halo is the neighbouring cell
}
int fdtd_update_H(fdtd_job *J, int32_t n) {
  NvtxRange nvtx_("fdtd_update_H");
  int rc = check_job(J, true);
  return rc ? rc : DISPATCH(J, proc_call)(J, n, 2);
}
int fdtd_pml_update_H(fdtd_job *J, int32_t n) {
  NvtxRange nvtx_("fdtd_pml_update_H");
  int rc = check_job(J, true);
  return rc ? rc : DISPATCH(J, proc_call)(J, n, 3);
}
int fdtd_sample(fdtd_job *J, int32_t n) {
  NvtxRange nvtx_("fdtd_sample");
  int rc = check_job(J, true);
  return rc ? rc : DISPATCH(J, proc_call)(J, n, 4);
}

int fdtd_sync(fdtd_job *J) {
  NvtxRange nvtx_("fdtd_sync");
  int rc = check_job(J, true);
  if (rc) return rc;
  if ((rc = DISPATCH(J, dft_fold)(J))) return rc;
  CK(cudaStreamSynchronize(J->stream));
  CK(cudaGetLastError());
  return kernel_flag(J);
}

int fdtd_get_field(fdtd_job *J, int32_t comp, double *host) {
  NvtxRange nvtx_("fdtd_get_field");
  int rc = check_job(J, true);
  if (rc) return rc;
  if (!host) return set_err(FDTD_EINVAL, "null buffer");
  return DISPATCH(J, get_field_impl)(J, comp, host);
}

int fdtd_set_field(fdtd_job *J, int32_t comp, const double *host) {
  NvtxRange nvtx_("fdtd_set_field");
  int rc = check_job(J, true);
  if (rc) return rc;
  if (!host) return set_err(FDTD_EINVAL, "null buffer");
  return DISPATCH(J, set_field_impl)(J, comp, host);
}

int fdtd_get_monitor(fdtd_job *J, int32_t id, double *re, double *im) {
  NvtxRange nvtx_("fdtd_get_monitor");
  int rc = check_job(J, true);
  if (rc) return rc;
  if (id < 0 || id >= (int)J->mons.size()) return set_err(FDTD_ERANGE, "bad monitor id");
  if ((rc = fdtd_sync(J))) return rc;
  const Monitor &m = J->mon_dev[id];
  const size_t n = (size_t)m.ncomp * m.nfreq * m.ncell;
  if (re) CK(cudaMemcpy(re, J->d_acc_re + m.acc, n * sizeof(double), cudaMemcpyDeviceToHost));
  if (im) CK(cudaMemcpy(im, J->d_acc_im + m.acc, n * sizeof(double), cudaMemcpyDeviceToHost));
  J->d2h += (uint64_t)((re ? 1 : 0) + (im ? 1 : 0)) * n * sizeof(double);
  return FDTD_OK;
}

int fdtd_get_probe(fdtd_job *J, int32_t id, double *host, int32_t *count) {
  NvtxRange nvtx_("fdtd_get_probe");
  int rc = check_job(J, true);
  if (rc) return rc;
  if (id < 0 || id >= (int)J->probes.size()) return set_err(FDTD_ERANGE, "bad probe id");
  CK(cudaStreamSynchronize(J->stream));
  const ProbeRec &P = J->probes[id];
  long long cnt = (long long)std::min(P.d.n_last, J->last_n) - P.d.n_first + 1;
  cnt = std::max(0LL, std::min<long long>(cnt, P.cap));
  if (count) *count = (int32_t)cnt;
  if (host && cnt > 0) {
    CK(cudaMemcpy(host, P.buf, (size_t)cnt * P.ncomp * sizeof(double), cudaMemcpyDeviceToHost));
    J->d2h += (uint64_t)cnt * P.ncomp * sizeof(double);
  }
  return FDTD_OK;
}

int fdtd_device_bytes(const fdtd_job *J, uint64_t *bytes) {
  if (!J || !bytes) return set_err(FDTD_EINVAL, "null argument");
  *bytes = J->dev_bytes;
  return FDTD_OK;
}

int fdtd_estimate_bytes(const fdtd_job *J, uint64_t *bytes) {
  if (!J || !bytes) return set_err(FDTD_EINVAL, "null argument");
  if (J->committed) {
    *bytes = J->dev_bytes;
    return FDTD_OK;
  }
  const uint64_t N = (uint64_t)J->ncell, w = J->esz;
  const int nx = J->nx, ny = J->ny, nz = J->nz;
  uint64_t b = N * w * (J->dim == 3 ? 6 : J->dim == 2 ? 3 : 2) + N;  // fields, material ids
  // the fused 3D step kernel's second set of fields (commit may give it back)
  if (J->dim == 3 && w == 4 && J->nx % 4 == 0 && !J->has_tfbox &&
      !(J->has_pml && J->pml.mode == FDTD_PML_REFERENCE))
    b += 6 * N * w;
  // the fused 2D step kernel's: Ez, Hx, Hy and the stored PML part
  if (J->g.layout == FDTD_LAYOUT_2D_TM && w == 4 && J->nx % 4 == 0 && !J->has_tfbox &&
      !(J->has_pml && J->pml.mode == FDTD_PML_REFERENCE))
    b += 4 * N * w;
  if (J->has_tfsf) b += 2 * N * w;
  if (J->has_tfbox) b += 2ull * ny * w + 4 * w;
  // dispersive cells: each region's cells, bounded per sphere / box
  uint64_t nade = 0;
  for (auto &m : J->mats) {
    if (!is_ade_kind(m.kind)) continue;
    if (m.region.kind == FDTD_REGION_MASK) {
      for (uint8_t v : m.mask) nade += v != 0;
    } else if (m.region.kind == FDTD_REGION_SPHERES) {
      for (int q = 0; q < m.region.count; ++q) {
        const double d = 2.0 * m.centers[4 * q + 3] + 3.0;
        uint64_t c = 1;
        for (int a = 0; a < J->dim; ++a) c *= (uint64_t)d;
        nade += c;
      }
    } else {
      int lo[3], hi[3];
      region_bounds(J, m, lo, hi);
      uint64_t c = 1;
      for (int a = 0; a < 3; ++a) c *= (uint64_t)std::max(0, hi[a] - lo[a] + 1);
      nade += c;
    }
  }
  nade = std::min(nade, N);
  int nf = 0;
  for (auto &m : J->mats) nf = std::max(nf, ade_fields(m.kind, m.lz.npoles, m.lz.chi3 != 0.0, m.lz.ez_uses_x_current != 0));
  nf = std::max(nf, 1);
  b += nade * ((uint64_t)nf * 3 * w + 5) + 32ull * nf * 3 * w;
  if (J->has_pml && J->pml.mode == FDTD_PML_SPLIT) {
    b += (uint64_t)(J->dim == 3 ? 6 : 1) * (w == 8 ? 2 : 1) * N * w;
    b += 4ull * (nx + ny + nz) * w;
  } else if (J->has_pml && J->pml.mode == FDTD_PML_REFERENCE) {
    b += 2ull * 12 * (uint64_t)nx * (J->pml.npml[1][0] + 2) * nz * w + 24ull * (nx + ny + nz) * w;
  }
  if (J->dim == 2) {  // row flags and the edge unit list
    const uint64_t units = (uint64_t)nx * ny;
    const uint64_t frame = 2ull * ny * (J->pml.npml[0][0] + J->pml.npml[0][1] + 8) +
                           (uint64_t)nx * (J->pml.npml[1][0] + J->pml.npml[1][1] + 16);
    b += ny + 4 * std::min(units, frame);
  }
  for (auto &M : J->mons) {
    const uint64_t smp = (uint64_t)M.ncomp * M.ncell;
    b += smp * (J->dim == 1 ? 4096 : kStageSteps) * w + 2 * smp * M.d.nfreq * 8 + (uint64_t)M.d.nfreq * 8 +
         (uint64_t)M.d.nfreq * kStageSteps * 16;
    if (M.d.reduce == FDTD_MONITOR_MEAN)  // partial sums and counters: at most one block per x-row
      b += (uint64_t)M.ncomp * ((uint64_t)(M.d.hi[1] - M.d.lo[1] + 1) * (M.d.hi[2] - M.d.lo[2] + 1) + 1) * 12;
  }
  for (auto &P : J->probes) b += 1024ull * P.ncomp * 8;
  *bytes = b + (1ull << 20);  // coefficient tables, source table, step counter
  return FDTD_OK;
}

int fdtd_profile(fdtd_job *J, int32_t enable) {
  if (!J) return set_err(FDTD_EINVAL, "null job");
  J->prof = enable != 0;
  return FDTD_OK;
}

int fdtd_kernel_time(fdtd_job *J, int32_t kind, int64_t *launches, double *ms) {
  if (!J) return set_err(FDTD_EINVAL, "null job");
  if (kind < 0 || kind >= FDTD_KERNEL_COUNT) return set_err(FDTD_EINVAL, "bad kernel kind");
  CK(cudaStreamSynchronize(J->stream));
  for (auto &e : J->pending) {
    if (!e.b) continue;
    float t = 0.f;
    cudaEventElapsedTime(&t, e.a, e.b);
    J->kms[e.kind] += t;
    J->kcount[e.kind] += 1;
    J->ev_pool.push_back(e.a);
    J->ev_pool.push_back(e.b);
  }
  J->pending.clear();
  if (launches) *launches = J->kcount[kind];
  if (ms) *ms = J->kms[kind];
  return FDTD_OK;
}

int fdtd_set_tile(fdtd_job *J, int32_t tile) {
  int rc = check_job(J, false);
  if (rc) return rc;
  const int maxt = J->dim == 3 ? 9 : 4;
  if (tile < 0 || tile > maxt) return set_err(FDTD_EINVAL, "tile must be 0 (tune) or 1..%d", maxt);
  J->tile_req = tile;
  return FDTD_OK;
}

int fdtd_get_tile(const fdtd_job *J, int32_t *tile) {
  if (!J || !tile) return set_err(FDTD_EINVAL, "null argument");
  if (!J->committed) return set_err(FDTD_ESTATE, "job not committed");
  *tile = J->dim >= 2 && J->ncore > 0 ? J->tile + 1 : 0;
  return FDTD_OK;
}

int fdtd_kernel_cells(const fdtd_job *J, int32_t kind, int64_t *cells) {
  if (!J || !cells) return set_err(FDTD_EINVAL, "null argument");
  if (kind < 0 || kind >= FDTD_KERNEL_COUNT) return set_err(FDTD_EINVAL, "bad kernel kind");
  if (!J->committed) return set_err(FDTD_ESTATE, "job not committed");
  int64_t c = 0;
  if (kind == FDTD_KERNEL_E || kind == FDTD_KERNEL_H) c = J->dim >= 2 ? (int64_t)J->ncore * J->vec : 0;
  else if (kind == FDTD_KERNEL_STEP)
    c = !fused_mode(J) ? 0 : J->dim == 3 ? (int64_t)J->ncore * J->vec : (int64_t)J->ncell;
  else if (kind == FDTD_KERNEL_EDGE)
    c = J->dim >= 2 ? (int64_t)J->nedge * J->vec : 0;
  else if (kind == FDTD_KERNEL_ADE) c = J->dim == 2 ? J->nade : 0;
  else if (kind == FDTD_KERNEL_LINE1D) c = J->dim == 1 ? J->ncell : 0;
  else if (kind == FDTD_KERNEL_DFT) {
    for (auto &m : J->mon_dev) c += (int64_t)m.ncomp * m.ncell;
  }
  *cells = c;
  return FDTD_OK;
}

int fdtd_launch_count(const fdtd_job *J, int64_t *launches) {
  if (!J || !launches) return set_err(FDTD_EINVAL, "null argument");
  *launches = J->launches;
  return FDTD_OK;
}

int fdtd_set_stream(fdtd_job *J, void *cuda_stream) {
  if (!J) return set_err(FDTD_EINVAL, "null job");
  // finish what is queued on the old stream before switching
  CK(cudaStreamSynchronize(J->stream));
  J->stream = cuda_stream ? (cudaStream_t)cuda_stream : J->own_stream;
  return FDTD_OK;
}

int fdtd_transfer_bytes(const fdtd_job *J, uint64_t *h2d, uint64_t *d2h) {
  if (!J) return set_err(FDTD_EINVAL, "null job");
  if (h2d) *h2d = J->h2d;
  if (d2h) *d2h = J->d2h;
  return FDTD_OK;
}

}  // extern "C"

int fdtd::report_error(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
