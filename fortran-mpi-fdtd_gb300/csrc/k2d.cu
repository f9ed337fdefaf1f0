// k2d.cu -- 2D half-step kernels (TE: Ex, Ey, Hz; TM: Ez, Hx, Hy).
//
// One launch per half step; blockIdx selects the work:
//   tile blocks : 32*V x 32 cells.  A warp owns a 32*V-cell row segment and
//                 walks 4 rows, each thread V consecutive cells (float4 /
//                 double2 loads when the row length allows).  The row's
//                 inputs are loaded up front through the read-only path; the
//                 x neighbour at a vector edge comes from a warp shuffle and
//                 the previous row's value from registers.  Main cells do the
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

constexpr int kRows = 4;  // rows per warp

template <typename T>
struct Smem {
  T ca[kMaxMat];
  T cs[kMaxMat];
  unsigned ade[kMaxMat / 32];
};

template <typename T>
__device__ __forceinline__ void load_smem(const StepParams<T> &p, Smem<T> &sm) {
  for (int t = threadIdx.x; t < kMaxMat; t += blockDim.x) {
    const MatCoef<T> mc = p.mc[t];
    sm.ca[t] = mc.kind == MK_DIEL ? mc.ca : T(0);
    sm.cs[t] = mc.kind == MK_DIEL ? mc.cs : T(0);
  }
  if (threadIdx.x < kMaxMat / 32) {
    unsigned m = 0;
    for (int b = 0; b < 32; ++b) {
      const int k = p.mc[threadIdx.x * 32 + b].kind;
      if (k == MK_GOLD || k == MK_GRAPHENE) m |= 1u << b;
    }
    sm.ade[threadIdx.x] = m;
  }
  __syncthreads();
}

template <typename T>
__device__ __forceinline__ bool is_ade(const Smem<T> &sm, uint8_t id) {
  return (sm.ade[id >> 5] >> (id & 31)) & 1u;
}

// store V values, skipping cells whose E belongs to an ADE thread
template <typename T, int V>
__device__ __forceinline__ void st_guard(T *a, const T (&v)[V], const uint8_t (&id)[V], const Smem<T> &sm) {
  bool any = false;
#pragma unroll
  for (int q = 0; q < V; ++q) any |= is_ade(sm, id[q]);
  if (!any) {
    vst<T, V>(a, v);
  } else {
#pragma unroll
    for (int q = 0; q < V; ++q)
      if (!is_ade(sm, id[q])) a[q] = v[q];
  }
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

  static __device__ __forceinline__ bool slab_row(const StepParams<T> &p, int j) {
    return p.pml_mode == 1 && ((p.slab_on[0] && j < p.slab_rows) || (p.slab_on[1] && j >= p.slab_j0[1]));
  }

  // ---- E half step ------------------------------------------------------
  static __device__ __forceinline__ void tile_e(const StepParams<T> &p, int bx, const Smem<T> &sm, int n) {
    const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int tx = bx % p.tiles_x, ty = bx / p.tiles_x;
    const int i0 = (tx * 32 + lane) * V;
    const int j0 = ty * (8 * kRows) + wy * kRows;
    const int nx = p.nx, ny = p.ny;
    if (j0 >= ny) return;  // whole warp
    const bool inx = i0 < nx;
    const bool do_main = p.roles & ROLE_MAIN, do_pml = p.roles & ROLE_PML;
    const bool shell_x = p.pml_mode == 2 && (i0 < p.slo[0] || i0 + V - 1 > p.shi[0]);
    const bool main_x = i0 >= p.mlo[0] && i0 + V - 1 <= p.mhi[0];
    // the y-derivative component one row below
    const T *ydc = L == 3 ? p.hx : p.hz;
    T prev[V];
#pragma unroll
    for (int q = 0; q < V; ++q) prev[q] = T(0);
    if (inx) {
      if (j0 > 0) vld_ro<T, V>(ydc + (long long)(j0 - 1) * nx + i0, prev);
      else if (p.per[1]) vld_ro<T, V>(ydc + (long long)(ny - 1) * nx + i0, prev);
    }
    for (int r = 0; r < kRows; ++r) {
      const int j = j0 + r;
      if (j >= ny) break;
      const long long c = (long long)j * nx + i0;
      const bool shell_y = p.pml_mode == 2 && (j < p.slo[1] || j > p.shi[1]);
      const bool main_y = j >= p.mlo[1] && j <= p.mhi[1];
      if (L == 3) {
        // TM: Ez += Ku/eps ((Hy(i)-Hy(i-1)) + (-Hx(j)+Hx(j-1)))
        T hy[V], hx[V];
#pragma unroll
        for (int q = 0; q < V; ++q) { hy[q] = T(0); hx[q] = T(0); }
        if (inx) { vld_ro<T, V>(p.hy + c, hy); vld_ro<T, V>(p.hx + c, hx); }
        T hyl = shfl_left(hy[V - 1], lane);
        if (lane == 0 && inx) hyl = ld_x(p.hy, i0 - 1, j, nx, p.per[0]);
        T dxp[V], dyp[V];
#pragma unroll
        for (int q = 0; q < V; ++q) {
          dxp[q] = hy[q] - (q ? hy[q - 1] : hyl);  // curlhyx
          dyp[q] = -hx[q] + prev[q];             // curlhxy
          prev[q] = hx[q];
        }
        if (!inx) continue;
        if (shell_x || shell_y) {
          // split-field shell cells (and the main cells of this vector)
          T ez[V];
          uint8_t id[V];
          vld<T, V>(p.ez + c, ez);
          vld_ids<V>(p.mat + c, id);
          bool wrote = false;
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const int i = i0 + q;
            if (i < p.slo[0] || i > p.shi[0] || shell_y) {
              if (do_pml) {
                const long long cc = c + q;
                const T ezx = p.sp[0][cc];
                const T ezy = kTwoParts<T> ? p.sp[6][cc] : ez[q] - ezx;
                const T nezx = p.cf1[0][i] * ezx + p.cf2[0][i] * dxp[q];
                const T nezy = p.cf1[1][j] * ezy + p.cf2[1][j] * dyp[q];
                p.sp[0][cc] = nezx;
                if (kTwoParts<T>) p.sp[6][cc] = nezy;
                ez[q] = nezx + nezy;
                wrote = true;
              }
            } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
              ez[q] = ez[q] + sm.ca[id[q]] * (dxp[q] + dyp[q]);
              if (p.nsrc) {
                const T s = src_sum<T>(p, n, 2, i, j, 0);
                if (s != T(0)) ez[q] += sm.cs[id[q]] * s;
              }
              wrote = true;
            }
          }
          if (wrote) st_guard<T, V>(p.ez + c, ez, id, sm);
        } else if (do_main && main_y) {
          T ez[V];
          uint8_t id[V];
          vld<T, V>(p.ez + c, ez);
          vld_ids<V>(p.mat + c, id);
          const bool srow = p.nsrc && src_row(p, 2, j, 0);
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const int i = i0 + q;
            if (main_x || (i >= p.mlo[0] && i <= p.mhi[0])) {
              ez[q] = ez[q] + sm.ca[id[q]] * (dxp[q] + dyp[q]);
              if (srow) {
                const T s = src_sum<T>(p, n, 2, i, j, 0);
                if (s != T(0)) ez[q] += sm.cs[id[q]] * s;
              }
            }
          }
          st_guard<T, V>(p.ez + c, ez, id, sm);
        }
      } else {
        // TE: Ex += Ku/eps (Hz(j)-Hz(j-1)), Ey -= Ku/eps (Hz(i)-Hz(i-1))
        T hz[V];
#pragma unroll
        for (int q = 0; q < V; ++q) hz[q] = T(0);
        if (inx) vld_ro<T, V>(p.hz + c, hz);
        T hzl = shfl_left(hz[V - 1], lane);
        if (lane == 0 && inx) hzl = ld_x(p.hz, i0 - 1, j, nx, p.per[0]);
        T chx[V], chy[V], left[V];
#pragma unroll
        for (int q = 0; q < V; ++q) {
          left[q] = q ? hz[q - 1] : hzl;
          chx[q] = hz[q] - left[q];              // curlhx
          chy[q] = hz[q] - prev[q];              // curlhy
          prev[q] = hz[q];
        }
        if (!inx) continue;
        const bool srow = p.nsrc && (src_row(p, 0, j, 0) || src_row(p, 1, j, 0));
        if (shell_x || shell_y || (do_main && main_y)) {
          T ex[V], ey[V];
          uint8_t id[V];
          vld<T, V>(p.ex + c, ex);
          vld<T, V>(p.ey + c, ey);
          vld_ids<V>(p.mat + c, id);
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const int i = i0 + q;
            if (p.pml_mode == 2 && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
              if (do_pml) {
                ex[q] = p.cf1[1][j] * ex[q] + p.cf2[1][j] * chy[q];
                ey[q] = p.cf1[0][i] * ey[q] + p.cf2[0][i] * (-hz[q] + left[q]);
              }
            } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
              const T ca = sm.ca[id[q]];
              ex[q] = ex[q] + ca * chy[q];
              ey[q] = ey[q] - ca * chx[q];
              if (srow) {
                const T sx = src_sum<T>(p, n, 0, i, j, 0), sy = src_sum<T>(p, n, 1, i, j, 0);
                if (sx != T(0)) ex[q] += sm.cs[id[q]] * sx;
                if (sy != T(0)) ey[q] += sm.cs[id[q]] * sy;
              }
            }
          }
          st_guard<T, V>(p.ex + c, ex, id, sm);
          st_guard<T, V>(p.ey + c, ey, id, sm);
        }
        if (do_pml && slab_row(p, j)) {
#pragma unroll
          for (int q = 0; q < V; ++q) ref_slab_e(p, i0 + q, j);
        }
      }
    }
  }

  // ---- H half step ------------------------------------------------------
  static __device__ __forceinline__ void tile_h(const StepParams<T> &p, int bx, int n) {
    const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int tx = bx % p.tiles_x, ty = bx / p.tiles_x;
    const int i0 = (tx * 32 + lane) * V;
    const int j0 = ty * (8 * kRows) + wy * kRows;
    const int nx = p.nx, ny = p.ny;
    if (j0 >= ny) return;
    const bool inx = i0 < nx;
    const bool do_main = p.roles & ROLE_MAIN, do_pml = p.roles & ROLE_PML;
    const bool shell_x = p.pml_mode == 2 && (i0 < p.slo[0] || i0 + V - 1 > p.shi[0]);
    const T *ydc = L == 3 ? p.ez : p.ex;   // E component with a y derivative
    T cur[V];
#pragma unroll
    for (int q = 0; q < V; ++q) cur[q] = T(0);
    if (inx) vld_ro<T, V>(ydc + (long long)j0 * nx + i0, cur);
    for (int r = 0; r < kRows; ++r) {
      const int j = j0 + r;
      if (j >= ny) break;
      const long long c = (long long)j * nx + i0;
      T up[V];
#pragma unroll
      for (int q = 0; q < V; ++q) up[q] = T(0);
      if (inx) {
        if (j + 1 < ny) vld_ro<T, V>(ydc + c + nx, up);
        else if (p.per[1]) vld_ro<T, V>(ydc + i0, up);
      }
      const bool shell_y = p.pml_mode == 2 && (j < p.slo[1] || j > p.shi[1]);
      const bool main_y = j >= p.mlo[1] && j <= p.mhi[1];
      const bool srow = p.gather && sample_row(p, j, 0);
      if (L == 3) {
        T ez[V];
#pragma unroll
        for (int q = 0; q < V; ++q) ez[q] = cur[q];
        T ezr = shfl_right(ez[0], lane);
        if ((lane == 31 || i0 + V >= nx) && inx) ezr = ld_x(p.ez, i0 + V, j, nx, p.per[0]);
#pragma unroll
        for (int q = 0; q < V; ++q) cur[q] = up[q];
        if (!inx) continue;
        if (shell_x || shell_y || (do_main && main_y) || srow) {
          T hx[V], hy[V];
          vld<T, V>(p.hx + c, hx);
          vld<T, V>(p.hy + c, hy);
          bool wrote = false;
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const int i = i0 + q;
            const T right = q < V - 1 ? ez[q + 1] : ezr;
            if (p.pml_mode == 2 && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
              if (do_pml) {
                hx[q] = p.cg1[1][j] * hx[q] + p.cg2[1][j] * (-up[q] + ez[q]);
                hy[q] = p.cg1[0][i] * hy[q] + p.cg2[0][i] * (right - ez[q]);
                wrote = true;
              }
            } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
              hx[q] = hx[q] + p.ku * (-up[q] + ez[q]);
              hy[q] = hy[q] + p.ku * (right - ez[q]);
              wrote = true;
            }
          }
          if (wrote) { vst<T, V>(p.hx + c, hx); vst<T, V>(p.hy + c, hy); }
          if (srow) {
#pragma unroll
            for (int q = 0; q < V; ++q) {
              const T vals[6] = {T(0), T(0), ez[q], hx[q], hy[q], T(0)};
              gather_cell<T>(p, n, i0 + q, j, 0, vals);
            }
          }
        }
      } else {
        T ex[V], ey[V];
#pragma unroll
        for (int q = 0; q < V; ++q) { ex[q] = cur[q]; ey[q] = T(0); }
        if (inx) vld_ro<T, V>(p.ey + c, ey);
        T eyr = shfl_right(ey[0], lane);
        if ((lane == 31 || i0 + V >= nx) && inx) eyr = ld_x(p.ey, i0 + V, j, nx, p.per[0]);
#pragma unroll
        for (int q = 0; q < V; ++q) cur[q] = up[q];
        if (!inx) continue;
        const bool slab = do_pml && slab_row(p, j);
        if (shell_x || shell_y || (do_main && main_y) || srow || slab) {
          T hz[V];
          vld<T, V>(p.hz + c, hz);
          bool wrote = false;
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const int i = i0 + q;
            const T right = q < V - 1 ? ey[q + 1] : eyr;
            if (p.pml_mode == 2 && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
              if (do_pml) {
                const long long cc = c + q;
                T hzx = p.sp[0][cc];
                T hzy = kTwoParts<T> ? p.sp[6][cc] : hz[q] - hzx;
                hzy = p.cg1[1][j] * hzy + p.cg2[1][j] * (up[q] - ex[q]);
                hzx = p.cg1[0][i] * hzx + p.cg2[0][i] * (-right + ey[q]);
                p.sp[0][cc] = hzx;
                if (kTwoParts<T>) p.sp[6][cc] = hzy;
                hz[q] = hzy + hzx;
                wrote = true;
              }
            } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
              const T curlE = ((right - ey[q]) - up[q]) + ex[q];
              hz[q] = hz[q] - p.ku * curlE;
              wrote = true;
            }
          }
          if (wrote) vst<T, V>(p.hz + c, hz);
          if (slab) {
#pragma unroll
            for (int q = 0; q < V; ++q) {
              T v;
              if (ref_slab_h(p, i0 + q, j, &v)) hz[q] = v;
            }
          }
          if (srow) {
#pragma unroll
            for (int q = 0; q < V; ++q) {
              const T vals[6] = {ex[q], ey[q], T(0), T(0), T(0), hz[q]};
              gather_cell<T>(p, n, i0 + q, j, 0, vals);
            }
          }
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
  const MatCoef<T> mc = p.mc[p.ade_mat[s]];
  const AdeCoef<T> &a = p.ac[mc.ade];
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

template <typename T, int L, int V>
__global__ void __launch_bounds__(256) e2d_kernel(const __grid_constant__ StepParams<T> p) {
  const int n = step_n(p);
  int b = blockIdx.x;
  if (b < p.ntile_blocks) {
    if (!(p.roles & (ROLE_MAIN | ROLE_PML))) return;
    __shared__ Smem<T> sm;
    load_smem(p, sm);
    K2<T, L, V>::tile_e(p, b, sm, n);
    return;
  }
  b -= p.ntile_blocks;
  if (p.roles & ROLE_ADE) {
    const int s = b * 256 + threadIdx.x;
    if (s < p.nade) ade_e2<T, L>(p, s, n);
  }
}

template <typename T, int L, int V>
__global__ void __launch_bounds__(256) h2d_kernel(const __grid_constant__ StepParams<T> p) {
  if ((int)blockIdx.x < p.ntile_blocks) K2<T, L, V>::tile_h(p, blockIdx.x, step_n(p));
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
