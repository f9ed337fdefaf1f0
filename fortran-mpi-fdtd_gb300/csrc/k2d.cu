// k2d.cu -- 2D half-step kernels (TE: Ex, Ey, Hz; TM: Ez, Hx, Hy).
//
// One launch per half step; blockIdx selects the work:
//   grid-stride blocks : each thread takes (row, V-cell vector) units in
//                 turn (float4 / double2 when the row length allows); inputs
//                 come through the read-only path, the neighbour row and the
//                 neighbour cell at the vector edge from L1.  Main cells do the
//                 Yee update with the constant-dielectric material folded in
//                 (E += Ku/eps * curl: the reference's D update and E = D*gax,
//                 2D/.../myfdtd_2Dfunc.f90:16-44, 2D/simpledielectric_mod.f90:
//                 141-146); split-PML shell cells do the split update; rows of
//                 the reference y-slabs (2D/BERpmly_HzExEy_mod.f90) run the
//                 reference PML; monitored rows stage their samples.
//                 Sources, shells, slabs and samples are tested per row (warp
//                 uniform) before any per-cell test.
//   ADE blocks  : one thread per dispersive cell (gold Drude+2CP,
//                 2D/gold_mod.f90:47-75); tile threads never store E there.
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {

// store V values, skipping cells whose E belongs to an ADE thread
// (material ids >= kAdeId)
template <typename T, int V>
__device__ __forceinline__ void st_guard(T *a, const T (&v)[V], const uint8_t (&id)[V]) {
  bool any = false;
#pragma unroll
  for (int q = 0; q < V; ++q) any |= id[q] >= kAdeId;
  if (!any) {
    vst<T, V>(a, v);
  } else {
#pragma unroll
    for (int q = 0; q < V; ++q)
      if (id[q] < kAdeId) a[q] = v[q];
  }
}

// Ku/eps of a cell: the dominant material's coefficient is a parameter
template <typename T>
__device__ __forceinline__ T coef_ca(const StepParams<T> &p, uint8_t id) {
  return id == p.id0 ? p.ca0 : __ldg(p.mca + id);
}

template <typename T, int L, int V>
struct K2 {
  // ---- reference 2D slab, E part (2D/BERpmly_HzExEy_mod.f90:96-123, 144-178)
  static __device__ __forceinline__ void ref_slab_e(const StepParams<T> &p, int i, int j) {
    const int rows = p.slab_rows, nx = p.nx;
    int side = -1, r = 0;
    if (p.slab_on[0] && j < rows) { side = 0; r = j; }
    else if (p.slab_on[1] && j >= p.slab_j0[1]) { side = 1; r = j - p.slab_j0[1]; }
    if (side < 0) return;
    T *Ex = p.slab[side][0], *Ey = p.slab[side][1];
    const T *Hzx = p.slab[side][2], *Hzy = p.slab[side][3];
    const long long c = (long long)r * nx + i;
    T curlHzx_p = -Hzx[c] - Hzy[c];
    T curlHzx_m = i > 0 ? Hzx[c - 1] + Hzy[c - 1] : T(0);
    T curlHzy_p = Hzx[c] + Hzy[c];
    T curlHzy_m = r > 0 ? -Hzx[c - nx] - Hzy[c - nx] : T(0);
    if (side == 0 && r == rows - 1) curlHzy_p = p.hz[(long long)j * nx + i];
    if (side == 1 && r == 0) curlHzy_m = -p.hz[(long long)(j - 1) * nx + i];
    T ex = p.sf1y[side][r] * Ex[c] + p.sf2y[side][r] * (curlHzy_p + curlHzy_m);
    T ey = p.sf1x[side][i] * Ey[c] + p.sf2x[side][i] * (curlHzx_p + curlHzx_m);
    Ex[c] = ex;
    Ey[c] = ey;
    p.ex[(long long)j * nx + i] = ex;  // setboundayEya/b: Ex_ = this%Ex
  }

  // ---- reference 2D slab, H part (updateHs :125-140, setboundayHya/b :156-190);
  // returns true when it wrote main Hz
  static __device__ __forceinline__ bool ref_slab_h(const StepParams<T> &p, int i, int j, T *hz_out) {
    const int rows = p.slab_rows, nx = p.nx;
    int side = -1, r = 0;
    if (p.slab_on[0] && j < rows) { side = 0; r = j; }
    else if (p.slab_on[1] && j >= p.slab_j0[1]) { side = 1; r = j - p.slab_j0[1]; }
    if (side < 0) return false;
    const T *Ex = p.slab[side][0], *Ey = p.slab[side][1];
    T *Hzx = p.slab[side][2], *Hzy = p.slab[side][3];
    const long long c = (long long)r * nx + i;
    T exu = r + 1 < rows ? Ex[c + nx] : T(0);
    T eyr = i + 1 < nx ? Ey[c + 1] : T(0);
    T curlExy = exu - Ex[c];
    T curlEyx = -eyr + Ey[c];
    T hzy = p.sg1y[side][r] * Hzy[c] + p.sg2y[side][r] * curlExy;
    T hzx = p.sg1x[side][i] * Hzx[c] + p.sg2x[side][i] * curlEyx;
    Hzy[c] = hzy;
    Hzx[c] = hzx;
    if (side == 0 && r >= rows - 1) return false;  // copy-back rows 1..ja-1
    T hz = hzy + hzx;
    p.hz[(long long)j * nx + i] = hz;
    *hz_out = hz;
    return true;
  }

  // ---- E half step: one (row, V-cell vector) unit ------------------------
  static __device__ __forceinline__ void unit_e(const StepParams<T> &p, long long t, int n) {
    const int nvec = p.nx / V;
    const int j = (int)(t / nvec), i0 = (int)(t % nvec) * V;
    const int nx = p.nx, ny = p.ny;
    const long long c = (long long)j * nx + i0;
    const bool do_main = p.roles & ROLE_MAIN, do_pml = p.roles & ROLE_PML;
    const bool split = p.pml_mode == 2;
    const bool shell = split && (i0 < p.slo[0] || i0 + V - 1 > p.shi[0] || j < p.slo[1] || j > p.shi[1]);
    const bool main_y = j >= p.mlo[1] && j <= p.mhi[1];
    const bool main_x = i0 >= p.mlo[0] && i0 + V - 1 <= p.mhi[0];
    const int rf = __ldg(p.rowflag + j);
    const T *ydc = L == 3 ? p.hx : p.hz;  // component with the y derivative
    const T *xdc = L == 3 ? p.hy : p.hz;  // component with the x derivative
    T below[V], a0[V], a1[V], e0[V], e1[V];
    uint8_t id[V];
#pragma unroll
    for (int q = 0; q < V; ++q) below[q] = T(0);
    if (j > 0) vld_ro<T, V>(ydc + c - nx, below);
    else if (p.per[1]) vld_ro<T, V>(ydc + (long long)(ny - 1) * nx + i0, below);
    vld_ro<T, V>(xdc + c, a0);
    const T left = i0 > 0 ? __ldg(xdc + c - 1) : (p.per[0] ? __ldg(xdc + c + nx - 1) : T(0));
    vld_ids<V>(p.mat + c, id);
    if (L == 3) {
      vld_ro<T, V>(p.hx + c, a1);
      vld<T, V>(p.ez + c, e0);
      // TM: Ez += Ku/eps ((Hy(i)-Hy(i-1)) + (-Hx(j)+Hx(j-1)))
      T dxp[V], dyp[V];
#pragma unroll
      for (int q = 0; q < V; ++q) {
        dxp[q] = a0[q] - (q ? a0[q - 1] : left);  // curlhyx
        dyp[q] = -a1[q] + below[q];              // curlhxy
      }
      if (!shell && main_x && main_y && !(rf & ROW_SRC)) {
        if (do_main) {
          bool uni = true;
#pragma unroll
          for (int q = 0; q < V; ++q) uni &= id[q] == p.id0;
          if (uni) {
#pragma unroll
            for (int q = 0; q < V; ++q) e0[q] = e0[q] + p.ca0 * (dxp[q] + dyp[q]);
            vst<T, V>(p.ez + c, e0);
          } else {
#pragma unroll
            for (int q = 0; q < V; ++q) e0[q] = e0[q] + coef_ca(p, id[q]) * (dxp[q] + dyp[q]);
            st_guard<T, V>(p.ez + c, e0, id);
          }
        }
        return;
      }
      const bool shell_y = split && (j < p.slo[1] || j > p.shi[1]);
      bool wrote = false;
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const int i = i0 + q;
        if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
          if (do_pml) {
            // Ez = Ezx + Ezy (3D/BERpmly_mod.f90:151,153 with d/dz = 0)
            const long long cc = c + q;
            const T ezx = p.sp[0][cc];
            const T ezy = kTwoParts<T> ? p.sp[6][cc] : e0[q] - ezx;
            const T nezx = p.cf1[0][i] * ezx + p.cf2[0][i] * dxp[q];
            const T nezy = p.cf1[1][j] * ezy + p.cf2[1][j] * dyp[q];
            p.sp[0][cc] = nezx;
            if (kTwoParts<T>) p.sp[6][cc] = nezy;
            e0[q] = nezx + nezy;
            wrote = true;
          }
        } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
          e0[q] = e0[q] + coef_ca(p, id[q]) * (dxp[q] + dyp[q]);
          if (rf & ROW_SRC) {
            const T sv = src_sum<T>(p, n, 2, i, j, 0);
            if (sv != T(0)) e0[q] += __ldg(p.mcs + id[q]) * sv;
          }
          wrote = true;
        }
      }
      if (wrote) st_guard<T, V>(p.ez + c, e0, id);
    } else {
      vld<T, V>(p.ex + c, e0);
      vld<T, V>(p.ey + c, e1);
      // TE: Ex += Ku/eps (Hz(j)-Hz(j-1)), Ey -= Ku/eps (Hz(i)-Hz(i-1))
      T chx[V], chy[V], lft[V];
#pragma unroll
      for (int q = 0; q < V; ++q) {
        lft[q] = q ? a0[q - 1] : left;
        chx[q] = a0[q] - lft[q];    // curlhx
        chy[q] = a0[q] - below[q];  // curlhy
      }
      if (!shell && main_x && main_y && !(rf & (ROW_SRC | ROW_SLAB))) {
        if (do_main) {
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const T ca = coef_ca(p, id[q]);
            e0[q] = e0[q] + ca * chy[q];
            e1[q] = e1[q] - ca * chx[q];
          }
          st_guard<T, V>(p.ex + c, e0, id);
          st_guard<T, V>(p.ey + c, e1, id);
        }
        return;
      }
      const bool shell_y = split && (j < p.slo[1] || j > p.shi[1]);
      if (shell || (do_main && main_y)) {
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const int i = i0 + q;
          if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
            if (do_pml) {
              e0[q] = p.cf1[1][j] * e0[q] + p.cf2[1][j] * chy[q];
              e1[q] = p.cf1[0][i] * e1[q] + p.cf2[0][i] * (-a0[q] + lft[q]);
            }
          } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
            const T ca = coef_ca(p, id[q]);
            e0[q] = e0[q] + ca * chy[q];
            e1[q] = e1[q] - ca * chx[q];
            if (rf & ROW_SRC) {
              const T sx = src_sum<T>(p, n, 0, i, j, 0), sy = src_sum<T>(p, n, 1, i, j, 0);
              if (sx != T(0)) e0[q] += __ldg(p.mcs + id[q]) * sx;
              if (sy != T(0)) e1[q] += __ldg(p.mcs + id[q]) * sy;
            }
          }
        }
        st_guard<T, V>(p.ex + c, e0, id);
        st_guard<T, V>(p.ey + c, e1, id);
      }
      if (do_pml && (rf & ROW_SLAB)) {
#pragma unroll
        for (int q = 0; q < V; ++q) ref_slab_e(p, i0 + q, j);
      }
    }
  }

  // ---- H half step: one (row, V-cell vector) unit ------------------------
  static __device__ __forceinline__ void unit_h(const StepParams<T> &p, long long t, int n) {
    const int nvec = p.nx / V;
    const int j = (int)(t / nvec), i0 = (int)(t % nvec) * V;
    const int nx = p.nx, ny = p.ny;
    const long long c = (long long)j * nx + i0;
    const bool do_main = p.roles & ROLE_MAIN, do_pml = p.roles & ROLE_PML;
    const bool split = p.pml_mode == 2;
    const bool shell = split && (i0 < p.slo[0] || i0 + V - 1 > p.shi[0] || j < p.slo[1] || j > p.shi[1]);
    const bool main_y = j >= p.mlo[1] && j <= p.mhi[1];
    const bool main_x = i0 >= p.mlo[0] && i0 + V - 1 <= p.mhi[0];
    const int rf = __ldg(p.rowflag + j);
    const bool srow = p.gather && (rf & ROW_SAMPLE);
    const T *ydc = L == 3 ? p.ez : p.ex;  // E component with a y derivative
    const T *xdc = L == 3 ? p.ez : p.ey;  // E component with an x derivative
    T cur[V], up[V], xe[V], h0[V], h1[V];
#pragma unroll
    for (int q = 0; q < V; ++q) up[q] = T(0);
    vld_ro<T, V>(ydc + c, cur);
    if (j + 1 < ny) vld_ro<T, V>(ydc + c + nx, up);
    else if (p.per[1]) vld_ro<T, V>(ydc + i0, up);
    if (L == 3) {
#pragma unroll
      for (int q = 0; q < V; ++q) xe[q] = cur[q];
    } else {
      vld_ro<T, V>(p.ey + c, xe);
    }
    const T right = i0 + V < nx ? __ldg(xdc + c + V) : (p.per[0] ? __ldg(xdc + c + V - nx) : T(0));
    if (L == 3) {
      vld<T, V>(p.hx + c, h0);
      vld<T, V>(p.hy + c, h1);
      if (!shell && main_x && main_y && !srow) {
        if (do_main) {
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const T rgt = q < V - 1 ? cur[q + 1] : right;
            h0[q] = h0[q] + p.ku * (-up[q] + cur[q]);
            h1[q] = h1[q] + p.ku * (rgt - cur[q]);
          }
          vst<T, V>(p.hx + c, h0);
          vst<T, V>(p.hy + c, h1);
        }
        return;
      }
      const bool shell_y = split && (j < p.slo[1] || j > p.shi[1]);
      bool wrote = false;
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const int i = i0 + q;
        const T rgt = q < V - 1 ? cur[q + 1] : right;
        if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
          if (do_pml) {
            h0[q] = p.cg1[1][j] * h0[q] + p.cg2[1][j] * (-up[q] + cur[q]);
            h1[q] = p.cg1[0][i] * h1[q] + p.cg2[0][i] * (rgt - cur[q]);
            wrote = true;
          }
        } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
          h0[q] = h0[q] + p.ku * (-up[q] + cur[q]);
          h1[q] = h1[q] + p.ku * (rgt - cur[q]);
          wrote = true;
        }
      }
      if (wrote) { vst<T, V>(p.hx + c, h0); vst<T, V>(p.hy + c, h1); }
      if (srow) {
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const T vals[6] = {T(0), T(0), cur[q], h0[q], h1[q], T(0)};
          gather_cell<T>(p, n, i0 + q, j, 0, vals);
        }
      }
    } else {
      vld<T, V>(p.hz + c, h0);
      const bool slab = do_pml && (rf & ROW_SLAB);
      if (!shell && main_x && main_y && !srow && !slab) {
        if (do_main) {
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const T rgt = q < V - 1 ? xe[q + 1] : right;
            const T curlE = ((rgt - xe[q]) - up[q]) + cur[q];
            h0[q] = h0[q] - p.ku * curlE;
          }
          vst<T, V>(p.hz + c, h0);
        }
        return;
      }
      const bool shell_y = split && (j < p.slo[1] || j > p.shi[1]);
      bool wrote = false;
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const int i = i0 + q;
        const T rgt = q < V - 1 ? xe[q + 1] : right;
        if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
          if (do_pml) {
            const long long cc = c + q;
            T hzx = p.sp[0][cc];
            T hzy = kTwoParts<T> ? p.sp[6][cc] : h0[q] - hzx;
            hzy = p.cg1[1][j] * hzy + p.cg2[1][j] * (up[q] - cur[q]);
            hzx = p.cg1[0][i] * hzx + p.cg2[0][i] * (-rgt + xe[q]);
            p.sp[0][cc] = hzx;
            if (kTwoParts<T>) p.sp[6][cc] = hzy;
            h0[q] = hzy + hzx;
            wrote = true;
          }
        } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
          const T curlE = ((rgt - xe[q]) - up[q]) + cur[q];
          h0[q] = h0[q] - p.ku * curlE;
          wrote = true;
        }
      }
      if (wrote) vst<T, V>(p.hz + c, h0);
      if (slab) {
#pragma unroll
        for (int q = 0; q < V; ++q) {
          T v;
          if (ref_slab_h(p, i0 + q, j, &v)) h0[q] = v;
        }
      }
      if (srow) {
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const T vals[6] = {cur[q], xe[q], T(0), T(0), T(0), h0[q]};
          gather_cell<T>(p, n, i0 + q, j, 0, vals);
        }
      }
    }
  }
};

// ---- dispersive cells ------------------------------------------------------
template <typename T, int L>
__device__ __forceinline__ void ade_e2(const StepParams<T> &p, int s, int n) {
  const int cell = p.ade_cell[s];
  const int nx = p.nx, ny = p.ny;
  const int i = cell % nx, j = cell / nx;
  const AdeCoef<T> a = ade_coef(p, p.ade_mat[s]);
  if (L == 3) {
    T curl = (p.hy[cell] - ld_x(p.hy, i - 1, j, nx, p.per[0])) +
             (-p.hx[cell] + ld_y(p.hx, i, j - 1, nx, ny, p.per[1]));
    T inc = p.ku * curl + src_sum<T>(p, n, 2, i, j, 0);
    p.ez[cell] = ade_update<T>(p, a, s, 0, inc, p.ez[cell]);
  } else {
    T hzc = p.hz[cell];
    T curlhx = hzc - ld_x(p.hz, i - 1, j, nx, p.per[0]);
    T curlhy = hzc - ld_y(p.hz, i, j - 1, nx, ny, p.per[1]);
    T incx = p.ku * curlhy + src_sum<T>(p, n, 0, i, j, 0);
    T incy = -(p.ku * curlhx) + src_sum<T>(p, n, 1, i, j, 0);
    p.ex[cell] = ade_update<T>(p, a, s, 0, incx, p.ex[cell]);
    p.ey[cell] = ade_update<T>(p, a, s, 1, incy, p.ey[cell]);
  }
}

// Block layout of a launch: the ADE blocks first (their dependent loads start
// early), then the grid-stride blocks over (row, vector) units.
template <typename T, int L, int V>
__global__ void __launch_bounds__(256) e2d_kernel(const __grid_constant__ StepParams<T> p) {
  const int n = step_n(p);
  int b = blockIdx.x;
  if (b < p.nade_blocks) {
    if (p.roles & ROLE_ADE) {
      const int s = b * 256 + threadIdx.x;
      if (s < p.nade) ade_e2<T, L>(p, s, n);
    }
    return;
  }
  if (!(p.roles & (ROLE_MAIN | ROLE_PML))) return;
  b -= p.nade_blocks;
  const long long units = (long long)(p.nx / V) * p.ny;
  for (long long t = (long long)b * 256 + threadIdx.x; t < units; t += (long long)p.ntile_blocks * 256)
    K2<T, L, V>::unit_e(p, t, n);
}

template <typename T, int L, int V>
__global__ void __launch_bounds__(256) h2d_kernel(const __grid_constant__ StepParams<T> p) {
  const int n = step_n(p);
  const long long units = (long long)(p.nx / V) * p.ny;
  for (long long t = (long long)blockIdx.x * 256 + threadIdx.x; t < units; t += (long long)p.ntile_blocks * 256)
    K2<T, L, V>::unit_h(p, t, n);
}

// V: cells per thread along x; 4 (float) / 2 (double) when the row length
// allows aligned vector access, else 1
template <typename T, int L>
void launch_e2d_l(const StepParams<T> &p, int blocks, cudaStream_t s) {
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  if (p.vec == VW) e2d_kernel<T, L, VW><<<blocks, 256, 0, s>>>(p);
  else e2d_kernel<T, L, 1><<<blocks, 256, 0, s>>>(p);
}
template <typename T, int L>
void launch_h2d_l(const StepParams<T> &p, int blocks, cudaStream_t s) {
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  if (p.vec == VW) h2d_kernel<T, L, VW><<<blocks, 256, 0, s>>>(p);
  else h2d_kernel<T, L, 1><<<blocks, 256, 0, s>>>(p);
}

template <typename T>
void launch_e2d(const StepParams<T> &p, int blocks, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (p.layout == 3) launch_e2d_l<T, 3>(p, blocks, s);
  else launch_e2d_l<T, 2>(p, blocks, s);
}

template <typename T>
void launch_h2d(const StepParams<T> &p, int blocks, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (p.layout == 3) launch_h2d_l<T, 3>(p, blocks, s);
  else launch_h2d_l<T, 2>(p, blocks, s);
}

template void launch_e2d<float>(const StepParams<float> &, int, void *);
template void launch_e2d<double>(const StepParams<double> &, int, void *);
template void launch_h2d<float>(const StepParams<float> &, int, void *);
template void launch_h2d<double>(const StepParams<double> &, int, void *);

}  // namespace fdtd
