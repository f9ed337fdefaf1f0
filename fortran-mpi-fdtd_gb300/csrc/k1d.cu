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
//
// A line of at least 512 cells runs instead on a thread-block cluster of
// kLineCluster CTAs (one per SM), each holding a segment in shared memory;
// the single-block kernel is kept for the lines the cluster cannot take.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>

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
        ex[j] = ade_update_state<T>(p.ade_state, p.ade_stride, q, 0, p.ac[mc.ade], p.ac + mc.ade, inc, ex[j]);
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

// ---- thread-block-cluster variant -----------------------------------------
// The line is split over a cluster of kLineCluster CTAs on as many SMs: CTA r
// owns cells [r W, (r+1) W) in its shared memory, and the one neighbour cell
// a segment needs across its ends (hz(j-1) for E, ex(j+1) for H, the TFSF
// cells) is read from the adjacent CTA's shared memory.  Two cluster
// barriers per step order the halves.  The low PML slab lives in CTA 0 and
// the high one in the last CTA.  The arithmetic of every cell is that of
// line1d_kernel.  Every thread of every CTA runs every barrier, and the last
// barrier of the last step comes after the last read of another CTA's
// shared memory, so no CTA leaves while its memory may still be read.
constexpr int kLineCluster = 8;
constexpr int kLineSrcAll = 8192;  // source values a launch keeps in shared memory

struct LineSmem {
  char *cur;
  __device__ __forceinline__ void *take(size_t bytes) {
    void *r = cur;
    cur += (bytes + 15) & ~size_t(15);
    return r;
  }
};

template <typename T>
__host__ __device__ __forceinline__ int slab_rows(const LineParams<T> &p, int side) {
  return side == 0 ? p.ja + 1 : p.N - p.jb;
}

template <typename T>
__global__ void __launch_bounds__(1024, 1) line1d_cluster_kernel(const __grid_constant__ LineParams<T> p, T *stage,
                                                                 long long stage_row, int W) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), last = kLineCluster - 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int N = p.N, c0 = rank * W, c1 = min(N, c0 + W);
  const T ku = p.ku;
  const int bd = p.tfsf_bd;
  const bool inc = p.exi != nullptr;
  extern __shared__ __align__(16) char smem[];
  LineSmem sm{smem};
  // the same layout in every CTA: a neighbour's copy sits at the same offset
  T *ex = (T *)sm.take(W * sizeof(T)), *hz = (T *)sm.take(W * sizeof(T));
  T *exi = inc ? (T *)sm.take(W * sizeof(T)) : nullptr, *hzi = inc ? (T *)sm.take(W * sizeof(T)) : nullptr;
  uint8_t *mat = (uint8_t *)sm.take(W);
  MatCoef<T> *mc = (MatCoef<T> *)sm.take(kMaxMat * sizeof(MatCoef<T>));
  AdeCoef<T> *ac = (AdeCoef<T> *)sm.take(p.nac * sizeof(AdeCoef<T>));
  int *ade_cell = (int *)sm.take(p.nade * sizeof(int));
  uint8_t *ade_mat = (uint8_t *)sm.take(p.nade);
  T *state = (T *)sm.take((size_t)p.ade_nf * 3 * p.ade_stride * sizeof(T));
  // the launch's source values: all of them when they fit, else this and
  // the next step's
  const bool all_src = (long long)p.n_steps * p.nsrc <= kLineSrcAll;
  double *sv = (double *)sm.take((all_src ? p.n_steps * p.nsrc : 2 * kMaxSrc) * sizeof(double));
  T *pex[2][2] = {}, *phz[2][2] = {}, *f1[2][2] = {}, *f2[2][2] = {}, *g1[2][2] = {}, *g2[2][2] = {};
#pragma unroll
  for (int l = 0; l < 2; ++l)
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      if (!p.slab_on[sd] || !p.pex[l][sd]) continue;
      const int len = slab_rows(p, sd) + 2;
      pex[l][sd] = (T *)sm.take(len * sizeof(T));
      phz[l][sd] = (T *)sm.take(len * sizeof(T));
      f1[l][sd] = (T *)sm.take(len * sizeof(T));
      f2[l][sd] = (T *)sm.take(len * sizeof(T));
      g1[l][sd] = (T *)sm.take(len * sizeof(T));
      g2[l][sd] = (T *)sm.take(len * sizeof(T));
    }
  // ---- copy in: the owned segment, the tables, the slabs ----
  for (int j = c0 + tid; j < c1; j += nth) {
    ex[j - c0] = p.ex[j];
    hz[j - c0] = p.hz[j];
    if (inc) {
      exi[j - c0] = p.exi[j];
      hzi[j - c0] = p.hzi[j];
    }
    mat[j - c0] = p.mat[j];
  }
  for (int q = tid; q < kMaxMat; q += nth) mc[q] = p.mc[q];
  for (int q = tid; q < p.nac; q += nth) ac[q] = p.ac[q];
  for (int q = tid; q < p.nade; q += nth) {
    ade_cell[q] = p.ade_cell[q];
    ade_mat[q] = p.ade_mat[q];
  }
  for (int q = tid; q < p.ade_nf * 3 * p.ade_stride; q += nth) state[q] = p.ade_state[q];
#pragma unroll
  for (int l = 0; l < 2; ++l)
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      if (!pex[l][sd]) continue;
      const int len = slab_rows(p, sd) + 2;
      for (int q = tid; q < len; q += nth) {
        pex[l][sd][q] = p.pex[l][sd][q];
        phz[l][sd][q] = p.phz[l][sd][q];
        f1[l][sd][q] = p.f1[l][sd][q];
        f2[l][sd][q] = p.f2[l][sd][q];
        g1[l][sd][q] = p.g1[l][sd][q];
        g2[l][sd][q] = p.g2[l][sd][q];
      }
    }
  if (all_src) {
    for (int q = tid; q < p.n_steps * p.nsrc; q += nth) sv[q] = p.srcval[q];
  } else if (tid < p.nsrc && p.n_steps > 0) {
    sv[tid] = p.srcval[tid];
  }
  // the neighbours' copies (same offsets in their shared memory)
  T *ex_r = rank < last ? cl.map_shared_rank(ex, rank + 1) : nullptr;
  T *exi_r = rank < last && inc ? cl.map_shared_rank(exi, rank + 1) : nullptr;
  T *hz_l = rank > 0 ? cl.map_shared_rank(hz, rank - 1) : nullptr;
  T *hzi_l = rank > 0 && inc ? cl.map_shared_rank(hzi, rank - 1) : nullptr;
  // cell j >= c0 - 1 of an H array, cell j <= c1 of an E array
  auto h_at = [&](const T *a, const T *a_l, int j) -> T { return j >= c0 ? a[j - c0] : a_l[W - 1]; };
  auto e_at = [&](const T *a, const T *a_r, int j) -> T { return j < c1 ? a[j - c0] : a_r[0]; };
  auto src = [&](int comp, int j, int s) -> T {
    T v = T(0);
    for (int q = 0; q < p.nsrc; ++q)
      if (p.src[q].comp == comp && j >= p.src[q].lo[1] && j <= p.src[q].hi[1])
        v += T(all_src ? sv[s * p.nsrc + q] : sv[(s & 1) * kMaxSrc + q]);
    return v;
  };
  // field of a component code on this segment (a select, not a table)
  auto fld = [&](int comp) -> const T * {
    return comp == FDTD_EX ? ex : comp == FDTD_HZ ? hz : comp == FDTD_EX_INC ? exi : comp == FDTD_HZ_INC ? hzi : nullptr;
  };
  cl.sync();
  const int jlo = max(p.mlo, c0), jhi = min(p.mhi, c1 - 1);
  for (int s = 0; s < p.n_steps; ++s) {
    const int n = p.n_first + s;
    if (p.stages & 1) {
      // ---- E half ----
      for (int j = jlo + tid; j <= jhi; j += nth) {
        const MatCoef<T> m = mc[mat[j - c0]];
        if (m.kind == MK_DIEL) {
          const T curl = hz[j - c0] - h_at(hz, hz_l, j - 1);
          T sx = src(0, j, s);
          if (inc && j == bd) sx -= ku * h_at(hzi, hzi_l, bd - 1);
          T e = ex[j - c0] + m.ca * curl;
          if (sx != T(0)) e += m.cs * sx;
          ex[j - c0] = e;
        }
        if (inc) {
          T w = exi[j - c0] + ku * (hzi[j - c0] - h_at(hzi, hzi_l, j - 1));
          const T si = src(6, j, s);
          if (si != T(0)) w = w + si;
          exi[j - c0] = w;
        }
      }
      for (int q = tid; q < p.nade; q += nth) {
        const int j = ade_cell[q];
        if (j < c0 || j >= c1) continue;
        const MatCoef<T> m = mc[ade_mat[q]];
        T d = ku * (hz[j - c0] - h_at(hz, hz_l, j - 1)) + src(0, j, s);
        if (inc && j == bd) d -= ku * h_at(hzi, hzi_l, bd - 1);
        ex[j - c0] = ade_update_state<T>(state, p.ade_stride, q, 0, ac[m.ade], ac + m.ade, d, ex[j - c0]);
      }
#pragma unroll
      for (int sd = 0; sd < 2; ++sd)
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          if (rank != (sd == 0 ? 0 : last) || !pex[l][sd]) continue;
          const int rows = slab_rows(p, sd);
          for (int q = 1 + tid; q <= rows; q += nth)
            pex[l][sd][q] = f1[l][sd][q] * pex[l][sd][q] + f2[l][sd][q] * (phz[l][sd][q] - phz[l][sd][q - 1]);
        }
      __syncthreads();
#pragma unroll
      for (int sd = 0; sd < 2; ++sd)
#pragma unroll
        for (int l = 0; l < 2; ++l) {  // setboundaryEa / setboundaryEb for both lines
          T *e = l ? exi : ex;
          if (tid != l * 2 + sd || !e || !pex[l][sd] || rank != (sd == 0 ? 0 : last)) continue;
          T *Ex = pex[l][sd];
          const int rows = slab_rows(p, sd);
          if (sd == 0) { Ex[rows + 1] = e[p.ja + 1 - c0]; e[p.ja - c0] = Ex[rows]; }
          else { Ex[0] = e[p.jb - 1 - c0]; e[p.jb - c0] = Ex[1]; }
        }
    }
    cl.sync();  // E of every segment done
    if (!all_src && tid < p.nsrc && s + 1 < p.n_steps)  // read in the next E, after the barriers below
      sv[((s + 1) & 1) * kMaxSrc + tid] = p.srcval[(long long)(s + 1) * p.nsrc + tid];
    if (p.stages & 2) {
      // ---- H half ----
      for (int j = jlo + tid; j <= jhi; j += nth) {
        hz[j - c0] = hz[j - c0] + ku * (e_at(ex, ex_r, j + 1) - ex[j - c0]);
        if (inc) hzi[j - c0] = hzi[j - c0] + ku * (e_at(exi, exi_r, j + 1) - exi[j - c0]);
      }
#pragma unroll
      for (int sd = 0; sd < 2; ++sd)
#pragma unroll
        for (int l = 1; l >= 0; --l) {
          if (rank != (sd == 0 ? 0 : last) || !phz[l][sd]) continue;
          const int rows = slab_rows(p, sd);
          for (int q = 1 + tid; q <= rows; q += nth)
            phz[l][sd][q] = g1[l][sd][q] * phz[l][sd][q] + g2[l][sd][q] * (pex[l][sd][q + 1] - pex[l][sd][q]);
        }
      __syncthreads();
#pragma unroll
      for (int sd = 0; sd < 2; ++sd)
#pragma unroll
        for (int l = 0; l < 2; ++l) {  // setboundaryHa / setboundaryHb
          T *h = l ? hzi : hz;
          if (tid != l * 2 + sd || !h || !phz[l][sd] || rank != (sd == 0 ? 0 : last)) continue;
          T *Hz = phz[l][sd];
          const int rows = slab_rows(p, sd);
          if (sd == 0) { Hz[rows + 1] = h[p.ja + 1 - c0]; h[p.ja - c0] = Hz[rows]; }
          else { Hz[0] = h[p.jb - 1 - c0]; h[p.jb - c0] = Hz[1]; }
        }
      if (inc) {
        __syncthreads();
        if (tid == 0 && bd > 0 && bd - 1 >= c0 && bd - 1 < c1)
          hz[bd - 1 - c0] = hz[bd - 1 - c0] - ku * e_at(exi, exi_r, bd);
      }
      __syncthreads();
    }
    if (p.stages & 4) {
      // ---- sampling of the owned cells: stage row s, probes ----
      for (int q = 0; q < p.nmon; ++q) {
        const Monitor &m = p.mon[q];
        const int ns = m.ncomp * m.ncell;
        for (int x = tid; x < ns; x += nth) {
          const int u = x / m.ncell, j = m.lo[1] + x % m.ncell;
          if (j < c0 || j >= c1) continue;
          const T *f = fld(m.comps[u]);
          stage[(long long)s * stage_row + m.base + x] = f ? f[j - c0] : T(0);
        }
      }
      if (tid < p.nprobe) {
        const Probe &pr = p.probe[tid];
        const int j = pr.cell[1];
        if (j >= c0 && j < c1 && n >= pr.n_first && n <= pr.n_last && n - pr.n_first < pr.cap) {
          double *out = pr.buf + (long long)(n - pr.n_first) * pr.ncomp;
          for (int u = 0; u < pr.ncomp; ++u) {
            const T *f = fld(pr.comps[u]);
            out[u] = f ? (double)f[j - c0] : 0.0;
          }
        }
      }
    }
    cl.sync();  // H and sampling of every segment done
  }
  // ---- copy out the owned state ----
  for (int j = c0 + tid; j < c1; j += nth) {
    p.ex[j] = ex[j - c0];
    p.hz[j] = hz[j - c0];
    if (inc) {
      p.exi[j] = exi[j - c0];
      p.hzi[j] = hzi[j - c0];
    }
  }
  for (int q = tid; q < p.nade; q += nth) {
    const int j = ade_cell[q];
    if (j < c0 || j >= c1) continue;
    for (int f = 0; f < p.ade_nf * 3; ++f)
      p.ade_state[(long long)f * p.ade_stride + q] = state[(long long)f * p.ade_stride + q];
  }
#pragma unroll
  for (int l = 0; l < 2; ++l)
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      if (!pex[l][sd] || rank != (sd == 0 ? 0 : last)) continue;
      const int len = slab_rows(p, sd) + 2;
      for (int q = tid; q < len; q += nth) {
        p.pex[l][sd][q] = pex[l][sd][q];
        p.phz[l][sd][q] = phz[l][sd][q];
      }
    }
}

// shared bytes per CTA of the cluster variant (same order as the kernel)
template <typename T>
size_t line_cluster_bytes(const LineParams<T> &p, int W) {
  auto r = [](size_t b) { return (b + 15) & ~size_t(15); };
  size_t b = (p.exi ? 4 : 2) * r(W * sizeof(T)) + r(W) + r(kMaxMat * sizeof(MatCoef<T>)) + r(p.nac * sizeof(AdeCoef<T>));
  b += r(p.nade * sizeof(int)) + r(p.nade) + r((size_t)p.ade_nf * 3 * p.ade_stride * sizeof(T));
  const bool all_src = (long long)p.n_steps * p.nsrc <= kLineSrcAll;
  b += r((all_src ? p.n_steps * p.nsrc : 2 * kMaxSrc) * sizeof(double));
  for (int l = 0; l < 2; ++l)
    for (int s = 0; s < 2; ++s)
      if (p.slab_on[s] && p.pex[l][s]) b += 6 * r((size_t)(slab_rows(p, s) + 2) * sizeof(T));
  return b;
}

// Whether the cluster variant can take the line: every segment non-empty,
// the main range and the TFSF cells away from the line's ends (their
// neighbours exist), and each slab's copy rows inside its end segment.
template <typename T>
bool line_cluster_fits(const LineParams<T> &p, int W, size_t bytes, size_t max_bytes) {
  if (p.N < 64 * kLineCluster || (long long)(kLineCluster - 1) * W >= p.N) return false;
  if (p.mlo < 1 || p.mhi > p.N - 2 || p.mlo > p.mhi) return false;
  if (p.exi && p.tfsf_bd >= 0 && (p.tfsf_bd < 1 || p.tfsf_bd > p.N - 2)) return false;
  if (p.slab_on[0] && p.ja + 1 >= W) return false;
  if (p.slab_on[1] && p.jb - 1 < (kLineCluster - 1) * W) return false;
  return p.nsrc <= kMaxSrc && bytes <= max_bytes;
}

template <typename T>
void launch_line1d_stage(const LineParams<T> &p, T *stage, long long stage_row, void *stream) {
  constexpr size_t kSmemMax = 200 * 1024;
  const int W = (p.N + kLineCluster - 1) / kLineCluster;
  const size_t bytes = line_cluster_bytes(p, W);
  if (line_cluster_fits(p, W, bytes, kSmemMax)) {
    static bool attr_set = false;  // once per process and precision
    if (!attr_set) {
      cudaFuncSetAttribute(line1d_cluster_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax);
      attr_set = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kLineCluster);
    cfg.blockDim = dim3(std::min(1024, (W + 31) / 32 * 32));
    cfg.dynamicSmemBytes = bytes;
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kLineCluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, line1d_cluster_kernel<T>, p, stage, stage_row, W) == cudaSuccess) return;
    cudaGetLastError();  // the single block takes it
  }
  line1d_kernel<T><<<1, kLineThreads, 0, (cudaStream_t)stream>>>(p, stage, stage_row);
}
template void launch_line1d_stage<float>(const LineParams<float> &, float *, long long, void *);
template void launch_line1d_stage<double>(const LineParams<double> &, double *, long long, void *);
}  // namespace fdtd
