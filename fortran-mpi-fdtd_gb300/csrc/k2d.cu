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

  // ---- E half step ------------------------------------------------------
  static __device__ __forceinline__ void tile_e(const StepParams<T> &p, int bx, int n) {
    const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int tx = bx % p.tiles_x, ty = bx / p.tiles_x;
    const int i0 = (tx * 32 + lane) * V;
    const int j0 = ty * (8 * kRows) + wy * kRows;
    const int nx = p.nx, ny = p.ny;
    if (j0 >= ny) return;  // whole warp
    const bool inx = i0 < nx;
    const bool do_main = p.roles & ROLE_MAIN, do_pml = p.roles & ROLE_PML;
    const bool split = p.pml_mode == 2;
    const bool shell_x = split && (i0 < p.slo[0] || i0 + V - 1 > p.shi[0]);
    const bool main_x = i0 >= p.mlo[0] && i0 + V - 1 <= p.mhi[0];
    const int nr = min(kRows, ny - j0);
    // ---- prefetch the rows of this thread (and the row below) ----
    const T *ydc = L == 3 ? p.hx : p.hz;  // component with the y derivative
    T prev[V], a0[kRows][V], a1[kRows][V], e0[kRows][V], e1[kRows][V];
    uint8_t id[kRows][V];
    uint8_t rf[kRows];
#pragma unroll
    for (int q = 0; q < V; ++q) prev[q] = T(0);
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
#pragma unroll
      for (int q = 0; q < V; ++q) { a0[r][q] = a1[r][q] = e0[r][q] = e1[r][q] = T(0); id[r][q] = 0; }
      rf[r] = 0;
    }
    if (inx) {
      if (j0 > 0) vld_ro<T, V>(ydc + (long long)(j0 - 1) * nx + i0, prev);
      else if (p.per[1]) vld_ro<T, V>(ydc + (long long)(ny - 1) * nx + i0, prev);
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        if (r >= nr) break;
        const long long c = (long long)(j0 + r) * nx + i0;
        if (L == 3) {
          vld_ro<T, V>(p.hy + c, a0[r]);
          vld_ro<T, V>(p.hx + c, a1[r]);
          vld<T, V>(p.ez + c, e0[r]);
        } else {
          vld_ro<T, V>(p.hz + c, a0[r]);
          vld<T, V>(p.ex + c, e0[r]);
          vld<T, V>(p.ey + c, e1[r]);
        }
        vld_ids<V>(p.mat + c, id[r]);
        rf[r] = __ldg(p.rowflag + j0 + r);
      }
    }
    // x neighbour at the left edge of each vector
    T left[kRows];
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      left[r] = shfl_left(a0[r][V - 1], lane);
      if (lane == 0 && inx && r < nr) left[r] = ld_x(L == 3 ? p.hy : p.hz, i0 - 1, j0 + r, nx, p.per[0]);
    }
    if (!inx) return;
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      if (r >= nr) break;
      const int j = j0 + r;
      const long long c = (long long)j * nx + i0;
      const bool shell_y = split && (j < p.slo[1] || j > p.shi[1]);
      const bool main_y = j >= p.mlo[1] && j <= p.mhi[1];
      if (L == 3) {
        // TM: Ez += Ku/eps ((Hy(i)-Hy(i-1)) + (-Hx(j)+Hx(j-1)))
        T dxp[V], dyp[V];
#pragma unroll
        for (int q = 0; q < V; ++q) {
          dxp[q] = a0[r][q] - (q ? a0[r][q - 1] : left[r]);  // curlhyx
          dyp[q] = -a1[r][q] + prev[q];                      // curlhxy
          prev[q] = a1[r][q];
        }
        T (&ez)[V] = e0[r];
        if (!shell_x && !shell_y && main_x && main_y && !(rf[r] & ROW_SRC)) {
          if (do_main) {
#pragma unroll
            for (int q = 0; q < V; ++q) ez[q] = ez[q] + __ldg(p.mca + id[r][q]) * (dxp[q] + dyp[q]);
            st_guard<T, V>(p.ez + c, ez, id[r]);
          }
          continue;
        }
        bool wrote = false;
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const int i = i0 + q;
          if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
            if (do_pml) {
              // Ez = Ezx + Ezy (3D/BERpmly_mod.f90:151,153 with d/dz = 0)
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
            ez[q] = ez[q] + __ldg(p.mca + id[r][q]) * (dxp[q] + dyp[q]);
            if (rf[r] & ROW_SRC) {
              const T sv = src_sum<T>(p, n, 2, i, j, 0);
              if (sv != T(0)) ez[q] += __ldg(p.mcs + id[r][q]) * sv;
            }
            wrote = true;
          }
        }
        if (wrote) st_guard<T, V>(p.ez + c, ez, id[r]);
      } else {
        // TE: Ex += Ku/eps (Hz(j)-Hz(j-1)), Ey -= Ku/eps (Hz(i)-Hz(i-1))
        const T *hz = a0[r];
        T chx[V], chy[V], lft[V];
#pragma unroll
        for (int q = 0; q < V; ++q) {
          lft[q] = q ? hz[q - 1] : left[r];
          chx[q] = hz[q] - lft[q];   // curlhx
          chy[q] = hz[q] - prev[q];  // curlhy
          prev[q] = hz[q];
        }
        T (&ex)[V] = e0[r];
        T (&ey)[V] = e1[r];
        if (!shell_x && !shell_y && main_x && main_y && !(rf[r] & (ROW_SRC | ROW_SLAB))) {
          if (do_main) {
#pragma unroll
            for (int q = 0; q < V; ++q) {
              const T ca = __ldg(p.mca + id[r][q]);
              ex[q] = ex[q] + ca * chy[q];
              ey[q] = ey[q] - ca * chx[q];
            }
            st_guard<T, V>(p.ex + c, ex, id[r]);
            st_guard<T, V>(p.ey + c, ey, id[r]);
          }
          continue;
        }
        if (shell_x || shell_y || (do_main && main_y)) {
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const int i = i0 + q;
            if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
              if (do_pml) {
                ex[q] = p.cf1[1][j] * ex[q] + p.cf2[1][j] * chy[q];
                ey[q] = p.cf1[0][i] * ey[q] + p.cf2[0][i] * (-hz[q] + lft[q]);
              }
            } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
              const T ca = __ldg(p.mca + id[r][q]);
              ex[q] = ex[q] + ca * chy[q];
              ey[q] = ey[q] - ca * chx[q];
              if (rf[r] & ROW_SRC) {
                const T sx = src_sum<T>(p, n, 0, i, j, 0), sy = src_sum<T>(p, n, 1, i, j, 0);
                if (sx != T(0)) ex[q] += __ldg(p.mcs + id[r][q]) * sx;
                if (sy != T(0)) ey[q] += __ldg(p.mcs + id[r][q]) * sy;
              }
            }
          }
          st_guard<T, V>(p.ex + c, ex, id[r]);
          st_guard<T, V>(p.ey + c, ey, id[r]);
        }
        if (do_pml && (rf[r] & ROW_SLAB)) {
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
    const bool split = p.pml_mode == 2;
    const bool shell_x = split && (i0 < p.slo[0] || i0 + V - 1 > p.shi[0]);
    const bool main_x = i0 >= p.mlo[0] && i0 + V - 1 <= p.mhi[0];
    const int nr = min(kRows, ny - j0);
    const T *ydc = L == 3 ? p.ez : p.ex;  // E component with a y derivative
    // rows j0..j0+nr of ydc (one more above), the other E (TE: Ey) and H
    T ey_[kRows + 1][V], eo[kRows][V], h0[kRows][V], h1[kRows][V];
    uint8_t rf[kRows];
#pragma unroll
    for (int r = 0; r <= kRows; ++r)
#pragma unroll
      for (int q = 0; q < V; ++q) ey_[r][q] = T(0);
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
#pragma unroll
      for (int q = 0; q < V; ++q) eo[r][q] = h0[r][q] = h1[r][q] = T(0);
      rf[r] = 0;
    }
    if (inx) {
#pragma unroll
      for (int r = 0; r <= kRows; ++r) {
        if (r > nr) break;
        const int j = j0 + r;
        if (j < ny) vld_ro<T, V>(ydc + (long long)j * nx + i0, ey_[r]);
        else if (p.per[1]) vld_ro<T, V>(ydc + i0, ey_[r]);
      }
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        if (r >= nr) break;
        const long long c = (long long)(j0 + r) * nx + i0;
        if (L == 3) {
          vld<T, V>(p.hx + c, h0[r]);
          vld<T, V>(p.hy + c, h1[r]);
        } else {
          vld_ro<T, V>(p.ey + c, eo[r]);
          vld<T, V>(p.hz + c, h0[r]);
        }
        rf[r] = __ldg(p.rowflag + j0 + r);
      }
    }
    // x neighbour at the right edge of each vector (the x-derivative component)
    T right[kRows];
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      const T first = L == 3 ? ey_[r][0] : eo[r][0];
      right[r] = shfl_right(first, lane);
      if ((lane == 31 || i0 + V >= nx) && inx && r < nr) right[r] = ld_x(L == 3 ? p.ez : p.ey, i0 + V, j0 + r, nx, p.per[0]);
    }
    if (!inx) return;
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      if (r >= nr) break;
      const int j = j0 + r;
      const long long c = (long long)j * nx + i0;
      const bool shell_y = split && (j < p.slo[1] || j > p.shi[1]);
      const bool main_y = j >= p.mlo[1] && j <= p.mhi[1];
      const bool srow = p.gather && (rf[r] & ROW_SAMPLE);
      const T *cur = ey_[r], *up = ey_[r + 1];
      if (L == 3) {
        T (&hx)[V] = h0[r];
        T (&hy)[V] = h1[r];
        if (!shell_x && !shell_y && main_x && main_y && !srow) {
          if (do_main) {
#pragma unroll
            for (int q = 0; q < V; ++q) {
              const T rgt = q < V - 1 ? cur[q + 1] : right[r];
              hx[q] = hx[q] + p.ku * (-up[q] + cur[q]);
              hy[q] = hy[q] + p.ku * (rgt - cur[q]);
            }
            vst<T, V>(p.hx + c, hx);
            vst<T, V>(p.hy + c, hy);
          }
          continue;
        }
        bool wrote = false;
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const int i = i0 + q;
          const T rgt = q < V - 1 ? cur[q + 1] : right[r];
          if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
            if (do_pml) {
              hx[q] = p.cg1[1][j] * hx[q] + p.cg2[1][j] * (-up[q] + cur[q]);
              hy[q] = p.cg1[0][i] * hy[q] + p.cg2[0][i] * (rgt - cur[q]);
              wrote = true;
            }
          } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
            hx[q] = hx[q] + p.ku * (-up[q] + cur[q]);
            hy[q] = hy[q] + p.ku * (rgt - cur[q]);
            wrote = true;
          }
        }
        if (wrote) { vst<T, V>(p.hx + c, hx); vst<T, V>(p.hy + c, hy); }
        if (srow) {
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const T vals[6] = {T(0), T(0), cur[q], hx[q], hy[q], T(0)};
            gather_cell<T>(p, n, i0 + q, j, 0, vals);
          }
        }
      } else {
        T (&hz)[V] = h0[r];
        const T *ex = cur, *ey = eo[r];
        const bool slab = do_pml && (rf[r] & ROW_SLAB);
        if (!shell_x && !shell_y && main_x && main_y && !srow && !slab) {
          if (do_main) {
#pragma unroll
            for (int q = 0; q < V; ++q) {
              const T rgt = q < V - 1 ? ey[q + 1] : right[r];
              const T curlE = ((rgt - ey[q]) - up[q]) + ex[q];
              hz[q] = hz[q] - p.ku * curlE;
            }
            vst<T, V>(p.hz + c, hz);
          }
          continue;
        }
        bool wrote = false;
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const int i = i0 + q;
          const T rgt = q < V - 1 ? ey[q + 1] : right[r];
          if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
            if (do_pml) {
              const long long cc = c + q;
              T hzx = p.sp[0][cc];
              T hzy = kTwoParts<T> ? p.sp[6][cc] : hz[q] - hzx;
              hzy = p.cg1[1][j] * hzy + p.cg2[1][j] * (up[q] - ex[q]);
              hzx = p.cg1[0][i] * hzx + p.cg2[0][i] * (-rgt + ey[q]);
              p.sp[0][cc] = hzx;
              if (kTwoParts<T>) p.sp[6][cc] = hzy;
              hz[q] = hzy + hzx;
              wrote = true;
            }
          } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
            const T curlE = ((rgt - ey[q]) - up[q]) + ex[q];
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
    if (p.roles & (ROLE_MAIN | ROLE_PML)) K2<T, L, V>::tile_e(p, b, n);
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
