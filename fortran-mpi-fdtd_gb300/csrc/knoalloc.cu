// knoalloc.cu -- the running DFT of one box of a field for callers that
// cannot allocate device memory.
//
// Some callers cannot call cudaMalloc while they run.  One kind takes all of
// its device memory from its own pool at start-up and forbids driver
// allocations, which synchronise the device and fragment the pool; another
// runs under a device-memory budget fixed before its time loop.
// fdtd_dft_sample_noalloc samples a box of such a caller's own field array at
// step n and folds the samples into the caller's own FP64 accumulators, like
// a monitor of a job (fdtd_add_monitor) does, without allocating anything.
//
// The samples of the current ring of kStageSteps steps are staged in
// g_noalloc_stage, a file-scope static device array of
// FDTD_NOALLOC_STAGE_BYTES on every device that runs it.  On the host the
// symbol is only a stand-in, so it is never handed to a kernel: the first
// call on each device, with that device current, looks up its device address
// with cudaGetSymbolAddress and caches it for later calls.  The same set-up
// loads the two gather kernels and the FP64 DFT fold (cudaFuncGetAttributes),
// which under lazy module loading would otherwise be loaded, and their code
// placed in device memory, at their first launch.
#include <cuda_runtime.h>

#include <mutex>

#include "fdtd_gb300.h"
#include "fdtd_internal.h"

static_assert(FDTD_NOALLOC_RING == fdtd::kStageSteps, "the stage ring is one DFT fold long");

namespace {

__device__ __align__(256) unsigned char g_noalloc_stage[FDTD_NOALLOC_STAGE_BYTES];

constexpr int kMaxDevices = 64;
double *g_stage_dev[kMaxDevices] = {};
int g_last_n[kMaxDevices] = {};  // step of the last sampled call per device (0: none)
std::mutex g_stage_mu;

// gather the box of the field (x fastest) into ring slot `slot`
template <typename F>
__global__ void noalloc_gather(const F *__restrict__ field, int nx, int ny, int lo0, int lo1, int lo2, int wx,
                               int wy, int ncell, double *stage, int slot) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell) return;
  const int i = lo0 + t % wx, j = lo1 + (t / wx) % wy, k = lo2 + t / (wx * wy);
  stage[(long long)slot * ncell + t] = (double)field[(long long)i + (long long)nx * (j + (long long)ny * k)];
}

int stage_address(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fdtd::report_error(FDTD_ENODEV, "cudaGetDevice failed");
  if (dev < 0 || dev >= kMaxDevices) return fdtd::report_error(FDTD_ENODEV, "device index out of range");
  std::lock_guard<std::mutex> lk(g_stage_mu);
  if (!g_stage_dev[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_stage);
    if (e != cudaSuccess || !p) return fdtd::report_error(FDTD_ECUDA, "cudaGetSymbolAddress of the stage ring failed");
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, noalloc_gather<float>) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, noalloc_gather<double>) != cudaSuccess || fdtd::preload_dft<double>() != 0)
      return fdtd::report_error(FDTD_ECUDA, "loading the allocation-free DFT kernels failed");
    g_stage_dev[dev] = (double *)p;
  }
  *out = g_stage_dev[dev];
  return FDTD_OK;
}

}  // namespace

extern "C" int fdtd_dft_sample_noalloc(const void *field, int32_t precision, int32_t nx, int32_t ny, int32_t nz,
                                       const int32_t lo[3], const int32_t hi[3], int32_t n, int32_t n_first,
                                       int32_t n_last, double dt, const double *omega, int32_t nfreq,
                                       double *acc_re, double *acc_im, int32_t flush, void *stream) {
  if (!field || !lo || !hi || !omega || !acc_re || !acc_im)
    return fdtd::report_error(FDTD_EINVAL, "fdtd_dft_sample_noalloc: null pointer");
  if (precision != FDTD_F32 && precision != FDTD_F64)
    return fdtd::report_error(FDTD_EINVAL, "fdtd_dft_sample_noalloc: precision must be FDTD_F32 or FDTD_F64");
  if (nx < 1 || ny < 1 || nz < 1 || nfreq < 1 || n < 1 || n_first < 1 || n_last < n_first || !(dt > 0.0))
    return fdtd::report_error(FDTD_EINVAL, "fdtd_dft_sample_noalloc: bad size, step window or dt");
  const int n3[3] = {nx, ny, nz};
  long long ncell = 1;
  for (int a = 0; a < 3; ++a) {
    if (lo[a] < 0 || hi[a] >= n3[a] || lo[a] > hi[a])
      return fdtd::report_error(FDTD_ERANGE, "fdtd_dft_sample_noalloc: box outside the field");
    // checked after every factor: each is below 2^31 and the product so far
    // at most the limit, so the product cannot overflow
    ncell *= hi[a] - lo[a] + 1;
    if (ncell > FDTD_NOALLOC_MAX_CELLS)
      return fdtd::report_error(FDTD_ERANGE, "fdtd_dft_sample_noalloc: box exceeds the stage ring's %d cells",
                                (int)FDTD_NOALLOC_MAX_CELLS);
  }
  if (n < n_first || n > n_last) return FDTD_OK;  // outside the window: nothing to sample
  double *stage = nullptr;
  int rc = stage_address(&stage);
  if (rc) return rc;
  int dev = 0;
  cudaGetDevice(&dev);  // succeeded in stage_address
  cudaStream_t s = (cudaStream_t)stream;
  const size_t row = (size_t)ncell * sizeof(double);
  // ring slot of step n: steps 1..32 fill slots 0..31, steps 33..64 again 0..31
  const int slot = (n - 1) % fdtd::kStageSteps;
  // A sequence that starts mid-ring (at n_first, or later when a run resumes
  // inside the window) folds the slots before its first step with the rest of
  // the ring, and the array still holds an earlier sequence's samples there:
  // those slots are cleared unless this call follows the previous one's step
  if (slot > 0 && (n == n_first || g_last_n[dev] != n - 1) && cudaMemsetAsync(stage, 0, row * slot, s) != cudaSuccess)
    return fdtd::report_error(FDTD_ECUDA, "fdtd_dft_sample_noalloc: clearing the stage ring failed");
  const int wx = hi[0] - lo[0] + 1, wy = hi[1] - lo[1] + 1;
  const int threads = 256, blocks = (int)((ncell + threads - 1) / threads);
  if (precision == FDTD_F64)
    noalloc_gather<double><<<blocks, threads, 0, s>>>((const double *)field, nx, ny, lo[0], lo[1], lo[2], wx, wy,
                                                      (int)ncell, stage, slot);
  else
    noalloc_gather<float><<<blocks, threads, 0, s>>>((const float *)field, nx, ny, lo[0], lo[1], lo[2], wx, wy,
                                                     (int)ncell, stage, slot);
  if (cudaGetLastError() != cudaSuccess)
    return fdtd::report_error(FDTD_ECUDA, "fdtd_dft_sample_noalloc: gather launch failed");
  g_last_n[dev] = n;
  if (slot == fdtd::kStageSteps - 1 || n == n_last || flush) {
    fdtd::DftParams d{};
    d.nmon = 1;
    fdtd::Monitor &m = d.mon[0];
    for (int a = 0; a < 3; ++a) {
      m.lo[a] = lo[a];
      m.hi[a] = hi[a];
    }
    m.ncomp = 1;
    m.ncell = (int)ncell;
    m.n_first = n_first;
    m.n_last = n_last;
    m.nfreq = nfreq;
    d.omega = omega;
    d.acc_re = acc_re;
    d.acc_im = acc_im;
    d.nslots = slot + 1;
    d.n0 = n - slot;
    d.dt = dt;
    d.stage_row = ncell;
    d.total_work_blocks = blocks * ((nfreq + 7) / 8);
    fdtd::launch_dft<double>(d, stage, (void *)s);
    if (cudaGetLastError() != cudaSuccess)
      return fdtd::report_error(FDTD_ECUDA, "fdtd_dft_sample_noalloc: DFT fold launch failed");
    // a fold before the end of the ring: the next fold covers these slots
    // again, so they must contribute nothing the second time
    if (slot < fdtd::kStageSteps - 1 && n < n_last && cudaMemsetAsync(stage, 0, row * (slot + 1), s) != cudaSuccess)
      return fdtd::report_error(FDTD_ECUDA, "fdtd_dft_sample_noalloc: clearing the stage ring failed");
  }
  return FDTD_OK;
}
