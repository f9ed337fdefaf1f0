// k1d.cu -- the 1D line (Ex, Hz along y) as one persistent thread block.
//
// A 1D job is a few thousand cells: one block of 1024 threads keeps the
// whole loop on the device and runs a chunk of steps per launch, with block
// barriers between the phases of a step (1D/.../program.f90:217-291):
//   E: dx += Ku (hz(j)-hz(j-1)); ex_inc likewise; source; incident PML;
//      TFSF correction dx(bd) -= Ku hz_inc(bd-1); materials; PML
//   H: hz += Ku (ex(j+1)-ex(j)); hz_inc likewise; both PMLs; TFSF
//      correction hz(bd-1) -= Ku ex_inc(bd)
// The PML slabs follow 1D/BERpmly_ExHz_mod.f90:51-159: slab arrays hold the
// PEC row, the npml slab cells and the coupling row (main value copied in,
// slab boundary value copied out).  Samples of every step go to a stage
// buffer that the DFT kernel folds afterwards.
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {

constexpr int kLineThreads = 1024;

template <typename T>
__device__ __forceinline__ void line_pml_e(const LineParams<T> &p, int line, int side, int tid) {
  // slab index q = r + 1: low side q=0 PEC, q=1..rows cells, q=rows+1 coupling
  //                       high side q=0 coupling, q=1..rows cells, q=rows+1 PEC
  const int rows = side == 0 ? p.ja + 1 : p.N - p.jb;
  T *Ex = p.pex[line][side];
  const T *Hz = p.phz[line][side];
  const T *f1 = p.f1[line][side], *f2 = p.f2[line][side];
  for (int q = 1 + tid; q <= rows; q += kLineThreads) Ex[q] = f1[q] * Ex[q] + f2[q] * (Hz[q] - Hz[q - 1]);
}

template <typename T>
__device__ __forceinline__ void line_pml_h(const LineParams<T> &p, int line, int side, int tid) {
  const int rows = side == 0 ? p.ja + 1 : p.N - p.jb;
  const T *Ex = p.pex[line][side];
  T *Hz = p.phz[line][side];
  const T *g1 = p.g1[line][side], *g2 = p.g2[line][side];
  for (int q = 1 + tid; q <= rows; q += kLineThreads) Hz[q] = g1[q] * Hz[q] + g2[q] * (Ex[q + 1] - Ex[q]);
}

template <typename T>
__device__ __forceinline__ T line_src(const LineParams<T> &p, int step, int comp, int j) {
  T s = T(0);
  for (int q = 0; q < p.nsrc; ++q)
    if (p.src[q].comp == comp && j >= p.src[q].lo[1] && j <= p.src[q].hi[1]) s += T(p.srcval[(long long)step * p.nsrc + q]);
  return s;
}

template <typename T>
__global__ void __launch_bounds__(kLineThreads, 1) line1d_kernel(const __grid_constant__ LineParams<T> p, T *stage,
                                                                 long long stage_row) {
  const int tid = threadIdx.x;
  const T ku = p.ku;
  T *ex = p.ex, *hz = p.hz, *exi = p.exi, *hzi = p.hzi;
  const int bd = p.tfsf_bd;
  for (int s = 0; s < p.n_steps; ++s) {
    const int n = p.n_first + s;
    if (p.stages & 1) {
      // ---- E half ----
      for (int j = p.mlo + tid; j <= p.mhi; j += kLineThreads) {
        const MatCoef<T> mc = p.mc[p.mat[j]];
        if (mc.kind == MK_DIEL) {
          const T curl = hz[j] - hz[j - 1];
          T sx = line_src(p, s, 0, j);
          if (exi && j == bd) sx -= ku * hzi[bd - 1];
          T e = ex[j] + mc.ca * curl;
          if (sx != T(0)) e += mc.cs * sx;
          ex[j] = e;
        }
        if (exi) {
          T v = exi[j] + ku * (hzi[j] - hzi[j - 1]);
          const T si = line_src(p, s, 6, j);
          if (si != T(0)) v = v + si;
          exi[j] = v;
        }
      }
      for (int q = tid; q < p.nade; q += kLineThreads) {
        const int j = p.ade_cell[q];
        const MatCoef<T> mc = p.mc[p.ade_mat[q]];
        T inc = ku * (hz[j] - hz[j - 1]) + line_src(p, s, 0, j);
        if (exi && j == bd) inc -= ku * hzi[bd - 1];
        ex[j] = ade_update_state<T>(p.ade_state, p.ade_stride, q, 0, p.ac[mc.ade], inc, ex[j]);
      }
      for (int side = 0; side < 2; ++side) {
        if (!p.slab_on[side]) continue;
        line_pml_e(p, 0, side, tid);
        if (exi) line_pml_e(p, 1, side, tid);
      }
      __syncthreads();
      if (tid < 4) {  // setboundaryEa / setboundaryEb for both lines
        const int line = tid >> 1, side = tid & 1;
        T *e = line ? exi : ex;
        if (e && p.slab_on[side]) {
          T *Ex = p.pex[line][side];
          const int rows = side == 0 ? p.ja + 1 : p.N - p.jb;
          if (side == 0) { Ex[rows + 1] = e[p.ja + 1]; e[p.ja] = Ex[rows]; }
          else { Ex[0] = e[p.jb - 1]; e[p.jb] = Ex[1]; }
        }
      }
      __syncthreads();
    }
    if (p.stages & 2) {
      // ---- H half ----
      for (int j = p.mlo + tid; j <= p.mhi; j += kLineThreads) {
        hz[j] = hz[j] + ku * (ex[j + 1] - ex[j]);
        if (hzi) hzi[j] = hzi[j] + ku * (exi[j + 1] - exi[j]);
      }
      for (int side = 0; side < 2; ++side) {
        if (!p.slab_on[side]) continue;
        if (hzi) line_pml_h(p, 1, side, tid);
        line_pml_h(p, 0, side, tid);
      }
      __syncthreads();
      if (tid < 4) {  // setboundaryHa / setboundaryHb
        const int line = tid >> 1, side = tid & 1;
        T *h = line ? hzi : hz;
        if (h && p.slab_on[side]) {
          T *Hz = p.phz[line][side];
          const int rows = side == 0 ? p.ja + 1 : p.N - p.jb;
          if (side == 0) { Hz[rows + 1] = h[p.ja + 1]; h[p.ja] = Hz[rows]; }
          else { Hz[0] = h[p.jb - 1]; h[p.jb] = Hz[1]; }
        }
      }
      __syncthreads();
      if (tid == 0 && exi && bd > 0) hz[bd - 1] = hz[bd - 1] - ku * exi[bd];
      __syncthreads();
    }
    if (p.stages & 4) {
      // ---- sampling: stage row s, probes ----
      const T *F[8] = {ex, nullptr, nullptr, nullptr, nullptr, hz, exi, hzi};
      long long t = tid;
      for (int q = 0; q < p.nmon; ++q) {
        const Monitor &m = p.mon[q];
        const long long ns = (long long)m.ncomp * m.ncell;
        for (long long x = t; x < ns; x += kLineThreads) {
          const int u = (int)(x / m.ncell);
          const int j = m.lo[1] + (int)(x % m.ncell);
          const T *f = F[m.comps[u]];
          stage[(long long)s * stage_row + m.base + x] = f ? f[j] : T(0);
        }
      }
      if (tid < p.nprobe) {
        const Probe &pr = p.probe[tid];
        if (n >= pr.n_first && n <= pr.n_last && n - pr.n_first < pr.cap) {
          double *out = pr.buf + (long long)(n - pr.n_first) * pr.ncomp;
          for (int u = 0; u < pr.ncomp; ++u) {
            const T *f = F[pr.comps[u]];
            out[u] = f ? (double)f[pr.cell[1]] : 0.0;
          }
        }
      }
      __syncthreads();
    }
  }
}

template <typename T>
void launch_line1d_impl(const LineParams<T> &p, T *stage, long long stage_row, void *stream) {
  line1d_kernel<T><<<1, kLineThreads, 0, (cudaStream_t)stream>>>(p, stage, stage_row);
}

template <typename T>
void launch_line1d_stage(const LineParams<T> &p, T *stage, long long stage_row, void *stream) {
  launch_line1d_impl<T>(p, stage, stage_row, stream);
}
template void launch_line1d_stage<float>(const LineParams<float> &, float *, long long, void *);
template void launch_line1d_stage<double>(const LineParams<double> &, double *, long long, void *);
}  // namespace fdtd
