// kdft.cu -- running DFT of the monitored cells and the stand-alone gather.
//
// The reference accumulates, every step and for every monitored cell and
// frequency (2D/.../program.f90:383-391, 3D/.../program.f90:456-472):
//   re += cos(arg(m) t) F dt,  im += sin(arg(m) t) F dt,  t = (n-1) dt.
// Here the half-step kernels stage F for kStageSteps steps and this kernel
// folds the whole ring at once: each thread owns one (component, cell)
// sample, holds its kStageSteps values in registers, and for a chunk of
// frequencies adds sum_s cos(w t_s) F_s (and sin) into the FP64
// accumulators.  Phases are computed in FP64 (sincos of w*t, or the FP64
// rotation below); the products and the 32-term ring sum run in the job's
// precision; the accumulators are FP64.  In FP32 the fields themselves carry
// FP32 rounding, which bounds the spectra's precision: FP64 products measured
// the same FP32-vs-FP64 error on the 2D and 3D workloads while costing 135 us
// per fold of the 2D one (4.2 us a step) on the GPU's FP64 pipe.
// Slots outside a monitor's [n_first, n_last] get zero weight.  With the
// job's rotation table the phases of a ring come from one FP64 sincos per
// frequency, e^{i w t0}, times the table's e^{i w s dt}:
// cos(w (t0 + s dt)) = cos(w t0) cos(w s dt) - sin(w t0) sin(w s dt).
// Without it (the allocation-free entry point) each (frequency, slot) takes
// its own sincos.
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {

constexpr int kDftThreads = 256;
constexpr int kFreqChunk = 8;

template <typename T>
__global__ void __launch_bounds__(kDftThreads) dft_kernel(const __grid_constant__ DftParams d, const T *__restrict__ stage) {
  __shared__ T cw[kFreqChunk][kStageSteps];
  __shared__ T sw[kFreqChunk][kStageSteps];
  // locate (monitor, freq chunk, sample block) of this block
  int b = blockIdx.x, q = 0, sblocks = 0, fchunks = 0;
  for (q = 0; q < d.nmon; ++q) {
    const Monitor &m = d.mon[q];
    sblocks = (m.ncomp * m.ncell + kDftThreads - 1) / kDftThreads;
    fchunks = (m.nfreq + kFreqChunk - 1) / kFreqChunk;
    if (b < sblocks * fchunks) break;
    b -= sblocks * fchunks;
  }
  if (q >= d.nmon) return;
  if (d.gate && *d.gate == 0) return;  // a replay with no ring before it to fold
  const Monitor &m = d.mon[q];
  // skip the fold when no slot of it lies in the monitor's step window
  const int n0 = d.d_base ? *d.d_base - (d.prev ? kStageSteps : 0) : d.n0;
  if (d.d_half) stage += (long long)(d.prev ? 1 - *d.d_half : *d.d_half) * kStageSteps * d.stage_row;
  const int nlast = n0 + d.nslots - 1;
  if (nlast < m.n_first || n0 > m.n_last) return;
  const int fc = b / sblocks, sb = b % sblocks;
  const int f0 = fc * kFreqChunk;
  __shared__ double bc[kFreqChunk], bs[kFreqChunk];
  if (d.rot) {
    if (threadIdx.x < kFreqChunk) {
      double c = 1.0, sn = 0.0;
      if (f0 + (int)threadIdx.x < m.nfreq)
        sincos(d.omega[m.freq_off + f0 + threadIdx.x] * ((double)(n0 - 1) * d.dt), &sn, &c);
      bc[threadIdx.x] = c;
      bs[threadIdx.x] = sn;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < kFreqChunk * kStageSteps; t += kDftThreads) {
    const int f = t / kStageSteps, s = t % kStageSteps;
    double c = 0.0, sn = 0.0;
    const int n = n0 + s;
    if (f0 + f < m.nfreq && s < d.nslots && n >= m.n_first && n <= m.n_last) {
      if (d.rot) {
        const double2 r = d.rot[(long long)(m.freq_off + f0 + f) * kStageSteps + s];
        c = bc[f] * r.x - bs[f] * r.y;
        sn = bs[f] * r.x + bc[f] * r.y;
      } else {
        const double tt = (double)(n - 1) * d.dt;          // t=real(n-1,8)*dt
        sincos(d.omega[m.freq_off + f0 + f] * tt, &sn, &c);
      }
    }
    cw[f][s] = T(c);
    sw[f][s] = T(sn);
  }
  __syncthreads();
  const long long p = (long long)sb * kDftThreads + threadIdx.x;
  const long long nsamp = (long long)m.ncomp * m.ncell;
  if (p >= nsamp) return;
  T v[kStageSteps];
#pragma unroll
  for (int s = 0; s < kStageSteps; ++s) v[s] = s < d.nslots ? stage[(long long)s * d.stage_row + m.base + p] : T(0);
  const int u = (int)(p / m.ncell);
  const long long cell = p % m.ncell;
  const int nf = min(kFreqChunk, m.nfreq - f0);
  for (int f = 0; f < nf; ++f) {
    T sr = T(0), si = T(0);
#pragma unroll
    for (int s = 0; s < kStageSteps; ++s) {
      sr += cw[f][s] * v[s];
      si += sw[f][s] * v[s];
    }
    const long long a = m.acc + ((long long)u * m.nfreq + (f0 + f)) * m.ncell + cell;
    d.acc_re[a] += (double)sr * d.dt;
    d.acc_im[a] += (double)si * d.dt;
  }
}

template <typename T>
void launch_dft(const DftParams &d, const T *stage, void *stream) {
  if (d.total_work_blocks <= 0 || d.nslots <= 0) return;
  dft_kernel<T><<<d.total_work_blocks, kDftThreads, 0, (cudaStream_t)stream>>>(d, stage);
}

template void launch_dft<float>(const DftParams &, const float *, void *);
template void launch_dft<double>(const DftParams &, const double *, void *);

template <typename T>
int preload_dft() {
  cudaFuncAttributes fa;
  return cudaFuncGetAttributes(&fa, dft_kernel<T>) == cudaSuccess ? 0 : 1;
}
template int preload_dft<float>();
template int preload_dft<double>();

constexpr int kMeanThreads = 256;  // threads per block of the gather launch

// Stand-alone gather of the monitored cells and probes after the H update:
// one thread per monitored (component, cell) sample, plus one per probe.
template <typename T>
__device__ __forceinline__ void gather_cells(const StepParams<T> &p, long long t) {
  const int n = step_n(p);
  const T *F[6] = {p.ex, p.ey, p.ez, p.hx, p.hy, p.hz};
  for (int q = 0; q < p.nmon; ++q) {
    const Monitor &m = p.mon[q];
    const long long ns = (long long)m.ncomp * m.ncell;
    if (t < ns) {
      if (m.mean) return;  // the mean kernel writes these samples
      const int u = (int)(t / m.ncell);
      const long long c = t % m.ncell;
      const int wx = m.hi[0] - m.lo[0] + 1, wy = m.hi[1] - m.lo[1] + 1;
      const int i = m.lo[0] + (int)(c % wx);
      const int j = m.lo[1] + (int)((c / wx) % wy);
      const int k = m.lo[2] + (int)(c / ((long long)wx * wy));
      const long long cell = (long long)i + (long long)p.nx * (j + (long long)p.ny * k);
      const T *f = F[m.comps[u]];
      stage_ring(p)[(long long)p.slot * p.stage_row + m.base + t] = f ? f[cell] : T(0);
      return;
    }
    t -= ns;
  }
  if (t < p.nprobe) {
    const Probe &pr = p.probe[t];
    if (n < pr.n_first || n > pr.n_last) return;
    const long long st = n - pr.n_first;
    if (st >= pr.cap) return;
    const long long cell = (long long)pr.cell[0] + (long long)p.nx * (pr.cell[1] + (long long)p.ny * pr.cell[2]);
    for (int u = 0; u < pr.ncomp; ++u) {
      const T *f = F[pr.comps[u]];
      pr.buf[st * pr.ncomp + u] = f ? (double)f[cell] : 0.0;
    }
  }
}

// Mean monitors: the box is cut into blocks of m.mrows whole x-rows.  Each
// block sums its cells in FP64 -- each thread the cells threadIdx.x,
// threadIdx.x + 256, ... of its rows taken row after row (eight loads issued
// before they are added, in that order), then a warp-shuffle tree and the
// warps' sums in order -- into its partial-sum slot.  The last block of a
// component to finish (a per-component counter) adds the partial sums in
// block order, stages the mean as the component's one sample and resets the
// counter.  The result depends on neither which block finishes last nor
// timing.
template <typename T>
__device__ __forceinline__ void gather_mean(const StepParams<T> &p, int b) {
  __shared__ double part[kMeanThreads / 32];
  __shared__ int last;
  int q = 0;
  for (; q < p.nmon; ++q) {
    if (!p.mon[q].mean) continue;
    const int nb = p.mon[q].ncomp * p.mon[q].mchunks;
    if (b < nb) break;
    b -= nb;
  }
  if (q >= p.nmon) return;  // uniform over the block
  const Monitor &m = p.mon[q];
  const int u = b / m.mchunks, chunk = b % m.mchunks;
  const T *F[6] = {p.ex, p.ey, p.ez, p.hx, p.hy, p.hz};
  const T *f = F[m.comps[u]];
  const int wx = m.hi[0] - m.lo[0] + 1, wy = m.hi[1] - m.lo[1] + 1;
  const int rows = wy * (m.hi[2] - m.lo[2] + 1);
  const int r0 = chunk * m.mrows, r1 = min(rows, r0 + m.mrows);
  const int ne = (r1 - r0) * wx;  // the block's cells, row after row
  double sum = 0.0;
  if (f)
    for (int e0 = threadIdx.x; e0 < ne; e0 += 8 * kMeanThreads) {
      T v[8];  // eight loads in flight, then added in order
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) {
        const int e = e0 + q8 * kMeanThreads;
        v[q8] = T(0);
        if (e < ne) {
          const int r = r0 + e / wx, i = e % wx;
          const int j = m.lo[1] + r % wy, k = m.lo[2] + r / wy;
          v[q8] = f[(long long)(m.lo[0] + i) + (long long)p.nx * (j + (long long)p.ny * k)];
        }
      }
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) sum += (double)v[q8];
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = sum;
  __syncthreads();
  const int slot = m.mpart + u * m.mchunks;
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < kMeanThreads / 32; ++w) tot += part[w];
    p.mean_part[slot + chunk] = tot;
    __threadfence();
    last = atomicAdd(p.mean_ctr + slot, 1u) == (unsigned)(m.mchunks - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double tot = 0.0;
    for (int c = 0; c < m.mchunks; ++c) tot += __ldcg(p.mean_part + slot + c);
    stage_ring(p)[(long long)p.slot * p.stage_row + m.base + u] = T(tot / (double)m.boxcells);
    p.mean_ctr[slot] = 0u;
  }
}

// One launch for both: the first blocks stage monitored cells and probes,
// the rest reduce the mean monitors.  It follows the H half step with a
// programmatic dependency and releases the next kernel at once, so the next
// E half's launch overlaps it.
template <typename T>
__global__ void __launch_bounds__(kMeanThreads) gather_kernel(const __grid_constant__ StepParams<T> p, int cell_blocks) {
  pdl_wait();
  pdl_release();
  if ((int)blockIdx.x < cell_blocks) gather_cells<T>(p, (long long)blockIdx.x * kMeanThreads + threadIdx.x);
  else gather_mean<T>(p, (int)blockIdx.x - cell_blocks);
}

template <typename T>
int launch_gather(const StepParams<T> &p, void *stream) {
  long long total = p.nprobe;
  int nmean = 0;
  for (int q = 0; q < p.nmon; ++q) {
    total += (long long)p.mon[q].ncomp * p.mon[q].ncell;
    if (p.mon[q].mean) nmean += p.mon[q].ncomp * p.mon[q].mchunks;
  }
  const int cell_blocks = (int)((total + kMeanThreads - 1) / kMeanThreads);
  if (cell_blocks + nmean <= 0) return 0;
  launch_pdl2(gather_kernel<T>, cell_blocks + nmean, kMeanThreads, (cudaStream_t)stream, p, cell_blocks);
  return 1;
}

template int launch_gather<float>(const StepParams<float> &, void *);
template int launch_gather<double>(const StepParams<double> &, void *);

}  // namespace fdtd
