// k2d.cu -- 2D half-step kernels (TE: Ex, Ey, Hz; TM: Ez, Hx, Hy).
//
// The work unit is one row segment of V cells (float4 / double2 when the row
// length allows).  A half step is split over independent kernels that write
// disjoint cells, so the host runs them as parallel branches of its stream:
//   core : the units of the interior box -- main cells outside the PML shell
//          in rows without flags -- doing only the Yee update with the
//          constant-dielectric material folded in (E += Ku/eps * curl: the
//          reference's D update and E = D*gax, 2D/.../myfdtd_2Dfunc.f90:16-44,
//          2D/simpledielectric_mod.f90:141-146).  This is nearly all of the
//          grid, and leaving the rest out keeps its register count low.
//   edge : every other unit, from a list built at commit: split-PML shell
//          cells, the edges of the main range, source rows, monitored rows
//          (which stage their samples) and the rows of the reference y-slabs
//          (2D/BERpmly_HzExEy_mod.f90).
//   ADE  : one thread per dispersive cell (gold Drude+2CP,
//          2D/gold_mod.f90:47-75); core and edge threads never store E there.
//          Its blocks follow the edge units' in the E edge launch
//          (e2d_edge_ade); the fused 2D step launches them alone (e2d_ade).
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
      // general unit (PML shell, source row, edge of the main range): every
      // split part and profile value of the unit is loaded before any store,
      // so the unit costs one round of loads like an interior unit
      const bool shell_y = split && (j < p.slo[1] || j > p.shi[1]);
      const bool pml = do_pml && shell;
      T ezx[V], ezy[V], f1x[V], f2x[V], f1y = T(0), f2y = T(0);
      if (pml) {
        vld<T, V>(p.sp[0] + c, ezx);
        if (kTwoParts<T>) vld<T, V>(p.sp[6] + c, ezy);
        vld_ro<T, V>(p.cf1[0] + i0, f1x);
        vld_ro<T, V>(p.cf2[0] + i0, f2x);
        f1y = __ldg(p.cf1[1] + j);
        f2y = __ldg(p.cf2[1] + j);
      }
      bool wrote = false;
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const int i = i0 + q;
        if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
          if (do_pml) {
            // Ez = Ezx + Ezy (3D/BERpmly_mod.f90:151,153 with d/dz = 0)
            const T py = kTwoParts<T> ? ezy[q] : e0[q] - ezx[q];
            const T nezx = lin2(f1x[q], ezx[q], f2x[q], dxp[q]);
            const T nezy = lin2(f1y, py, f2y, dyp[q]);
            ezx[q] = nezx;
            ezy[q] = nezy;
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
      if (pml) {  // cells of the unit outside the shell store back what they read
        vst<T, V>(p.sp[0] + c, ezx);
        if (kTwoParts<T>) vst<T, V>(p.sp[6] + c, ezy);
      }
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
        T f1x[V], f2x[V], f1y = T(0), f2y = T(0);
        if (do_pml && shell) {  // profile values loaded before any store
          vld_ro<T, V>(p.cf1[0] + i0, f1x);
          vld_ro<T, V>(p.cf2[0] + i0, f2x);
          f1y = __ldg(p.cf1[1] + j);
          f2y = __ldg(p.cf2[1] + j);
        }
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const int i = i0 + q;
          if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
            if (do_pml) {
              e0[q] = f1y * e0[q] + f2y * chy[q];
              e1[q] = f1x[q] * e1[q] + f2x[q] * (-a0[q] + lft[q]);
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
      T g1x[V], g2x[V], g1y = T(0), g2y = T(0);
      if (do_pml && shell) {  // profile values loaded before any store
        vld_ro<T, V>(p.cg1[0] + i0, g1x);
        vld_ro<T, V>(p.cg2[0] + i0, g2x);
        g1y = __ldg(p.cg1[1] + j);
        g2y = __ldg(p.cg2[1] + j);
      }
      bool wrote = false;
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const int i = i0 + q;
        const T rgt = q < V - 1 ? cur[q + 1] : right;
        if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
          if (do_pml) {
            h0[q] = lin2(g1y, h0[q], g2y, -up[q] + cur[q]);
            h1[q] = lin2(g1x[q], h1[q], g2x[q], rgt - cur[q]);
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
      const bool pml = do_pml && shell;
      T hzx[V], hzy[V], g1x[V], g2x[V], g1y = T(0), g2y = T(0);
      if (pml) {  // split parts and profile values loaded before any store
        vld<T, V>(p.sp[0] + c, hzx);
        if (kTwoParts<T>) vld<T, V>(p.sp[6] + c, hzy);
        vld_ro<T, V>(p.cg1[0] + i0, g1x);
        vld_ro<T, V>(p.cg2[0] + i0, g2x);
        g1y = __ldg(p.cg1[1] + j);
        g2y = __ldg(p.cg2[1] + j);
      }
      bool wrote = false;
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const int i = i0 + q;
        const T rgt = q < V - 1 ? xe[q + 1] : right;
        if (split && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
          if (do_pml) {
            const T py = kTwoParts<T> ? hzy[q] : h0[q] - hzx[q];
            const T nhzy = g1y * py + g2y * (up[q] - cur[q]);
            const T nhzx = g1x[q] * hzx[q] + g2x[q] * (-rgt + xe[q]);
            hzx[q] = nhzx;
            hzy[q] = nhzy;
            h0[q] = nhzy + nhzx;
            wrote = true;
          }
        } else if (do_main && main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
          const T curlE = ((rgt - xe[q]) - up[q]) + cur[q];
          h0[q] = h0[q] - p.ku * curlE;
          wrote = true;
        }
      }
      if (wrote) vst<T, V>(p.hz + c, h0);
      if (pml) {  // cells of the unit outside the shell store back what they read
        vst<T, V>(p.sp[0] + c, hzx);
        if (kTwoParts<T>) vst<T, V>(p.sp[6] + c, hzy);
      }
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
// KIND: the kind of every dispersive material of the job when there is one
// (MatKind), else -1
template <typename T, int L, int KIND = -1>
__device__ __forceinline__ void ade_e2(const StepParams<T> &p, int s, int n) {
  const int cell = p.ade_cell[s];
  const int nx = p.nx, ny = p.ny;
  const int i = cell % nx, j = cell / nx;
  const AdeCoef<T> &a = ade_coef(p, p.ade_mat[s]);
  const AdeCoef<T> *am = p.ac + (p.ade_mat[s] - kAdeId);
  if (L == 3) {
    T curl = (p.hy[cell] - ld_x(p.hy, i - 1, j, nx, p.per[0])) +
             (-p.hx[cell] + ld_y(p.hx, i, j - 1, nx, ny, p.per[1]));
    T inc = p.ku * curl + src_sum<T>(p, n, 2, i, j, 0);
    p.ezo[cell] = ade_update<T, KIND>(p, a, am, s, 0, inc, p.ez[cell]);
  } else {
    T hzc = p.hz[cell];
    T curlhx = hzc - ld_x(p.hz, i - 1, j, nx, p.per[0]);
    T curlhy = hzc - ld_y(p.hz, i, j - 1, nx, ny, p.per[1]);
    T incx = p.ku * curlhy + src_sum<T>(p, n, 0, i, j, 0);
    T incy = -(p.ku * curlhx) + src_sum<T>(p, n, 1, i, j, 0);
    p.exo[cell] = ade_update<T, KIND>(p, a, am, s, 0, incx, p.ex[cell]);
    p.eyo[cell] = ade_update<T, KIND>(p, a, am, s, 1, incy, p.ey[cell]);
  }
}

// ---- core units: the Yee update of interior cells, nothing else ----------
template <typename T, int L, int V>
__device__ __forceinline__ void core_e(const StepParams<T> &p, int j, int i0) {
  const int nx = p.nx, ny = p.ny;
  const long long c = (long long)j * nx + i0;
  const T *ydc = L == 3 ? p.hx : p.hz;  // component with the y derivative
  const T *xdc = L == 3 ? p.hy : p.hz;  // component with the x derivative
  T below[V], a0[V], e0[V];
  uint8_t id[V];
#pragma unroll
  for (int q = 0; q < V; ++q) below[q] = T(0);
  if (j > 0) vld_ro<T, V>(ydc + c - nx, below);
  else if (p.per[1]) vld_ro<T, V>(ydc + (long long)(ny - 1) * nx + i0, below);
  vld_ro<T, V>(xdc + c, a0);
  const T left = i0 > 0 ? __ldg(xdc + c - 1) : (p.per[0] ? __ldg(xdc + c + nx - 1) : T(0));
  vld_ids<V>(p.mat + c, id);  // issued with the field loads: a bitmap test first costs a round trip here
  if (L == 3) {
    T a1[V];
    vld_ro<T, V>(p.hx + c, a1);
    vld<T, V>(p.ez + c, e0);
    if (__ldg(p.rowflag + j)) return;  // flagged rows belong to the edge kernel
    // TM: Ez += Ku/eps ((Hy(i)-Hy(i-1)) + (-Hx(j)+Hx(j-1)))
    T dxp[V], dyp[V];
    bool uni = true;
#pragma unroll
    for (int q = 0; q < V; ++q) {
      dxp[q] = a0[q] - (q ? a0[q - 1] : left);  // curlhyx
      dyp[q] = -a1[q] + below[q];              // curlhxy
      uni &= id[q] == p.id0;
    }
    if (uni) {
#pragma unroll
      for (int q = 0; q < V; ++q) e0[q] = e0[q] + p.ca0 * (dxp[q] + dyp[q]);
      vst<T, V>(p.ez + c, e0);
    } else {
#pragma unroll
      for (int q = 0; q < V; ++q) e0[q] = e0[q] + coef_ca(p, id[q]) * (dxp[q] + dyp[q]);
      st_guard<T, V>(p.ez + c, e0, id);
    }
  } else {
    T e1[V];
    vld<T, V>(p.ex + c, e0);
    vld<T, V>(p.ey + c, e1);
    if (__ldg(p.rowflag + j)) return;
    // TE: Ex += Ku/eps (Hz(j)-Hz(j-1)), Ey -= Ku/eps (Hz(i)-Hz(i-1))
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const T ca = coef_ca(p, id[q]);
      const T chx = a0[q] - (q ? a0[q - 1] : left);  // curlhx
      const T chy = a0[q] - below[q];                // curlhy
      e0[q] = e0[q] + ca * chy;
      e1[q] = e1[q] - ca * chx;
    }
    st_guard<T, V>(p.ex + c, e0, id);
    st_guard<T, V>(p.ey + c, e1, id);
  }
}

template <typename T, int L, int V>
__device__ __forceinline__ void core_h(const StepParams<T> &p, int j, int i0) {
  const int nx = p.nx, ny = p.ny;
  const long long c = (long long)j * nx + i0;
  const T *ydc = L == 3 ? p.ez : p.ex;  // E component with a y derivative
  const T *xdc = L == 3 ? p.ez : p.ey;  // E component with an x derivative
  T cur[V], up[V], h0[V];
#pragma unroll
  for (int q = 0; q < V; ++q) up[q] = T(0);
  vld_ro<T, V>(ydc + c, cur);
  if (j + 1 < ny) vld_ro<T, V>(ydc + c + nx, up);
  else if (p.per[1]) vld_ro<T, V>(ydc + i0, up);
  const T right = i0 + V < nx ? __ldg(xdc + c + V) : (p.per[0] ? __ldg(xdc + c + V - nx) : T(0));
  if (L == 3) {
    T h1[V];
    vld<T, V>(p.hx + c, h0);
    vld<T, V>(p.hy + c, h1);
    if (__ldg(p.rowflag + j)) return;
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const T rgt = q < V - 1 ? cur[q + 1] : right;
      h0[q] = h0[q] + p.ku * (-up[q] + cur[q]);
      h1[q] = h1[q] + p.ku * (rgt - cur[q]);
    }
    vst<T, V>(p.hx + c, h0);
    vst<T, V>(p.hy + c, h1);
  } else {
    T xe[V];
    vld_ro<T, V>(p.ey + c, xe);
    vld<T, V>(p.hz + c, h0);
    if (__ldg(p.rowflag + j)) return;
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const T rgt = q < V - 1 ? xe[q + 1] : right;
      const T curlE = ((rgt - xe[q]) - up[q]) + cur[q];
      h0[q] = h0[q] - p.ku * curlE;
    }
    vst<T, V>(p.hz + c, h0);
  }
}

// ---- kernels: one unit (or one dispersive cell) per thread -----------------
// core kernels: NT threads per block, one of the candidate shapes that the
// commit-time tuner times on the job's grid
template <typename T, int L, int V, int NT>
__global__ void __launch_bounds__(NT) e2d_core(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  pdl_release();
  const int t = blockIdx.x * NT + threadIdx.x;
  if (t >= p.ncore) return;
  core_e<T, L, V>(p, p.cy0 + t / p.cw, (p.cv0 + t % p.cw) * V);
}

template <typename T, int L, int V, int NT>
__global__ void __launch_bounds__(NT) h2d_core(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  pdl_release();
  const int t = blockIdx.x * NT + threadIdx.x;
  if (t >= p.ncore) return;
  core_h<T, L, V>(p, p.cy0 + t / p.cw, (p.cv0 + t % p.cw) * V);
}

// The core kernels follow the previous core kernel on the job's stream with
// a programmatic dependency, so their launch overlaps its drain (the edge and
// dispersive-cell kernels, which run beside them, launch plainly: releasing
// their successors early measured slower).
template <typename T, int L, int V, int NT>
void launch_core2(const StepParams<T> &p, bool e_half, cudaStream_t s, cudaEvent_t ev) {
  const int blocks = (p.ncore + NT - 1) / NT;
  if (e_half) launch_pdl(e2d_core<T, L, V, NT>, blocks, NT, s, p, ev);
  else launch_pdl(h2d_core<T, L, V, NT>, blocks, NT, s, p, ev);
}

// tile 0: 128 threads, 1: 256, 2: 512
template <typename T, int L, int V>
void launch_core2_tiled(const StepParams<T> &p, bool e_half, cudaStream_t s, cudaEvent_t ev) {
  if (p.tile == 0) launch_core2<T, L, V, 128>(p, e_half, s, ev);
  else if (p.tile == 2) launch_core2<T, L, V, 512>(p, e_half, s, ev);
  else launch_core2<T, L, V, 256>(p, e_half, s, ev);
}

// The edge and dispersive-cell kernels may be launched early, off the
// previous core kernel's programmatic event (run_parts): they wait for it
// here first (a no-op without such a dependency).
template <typename T, int L, int V>
__global__ void __launch_bounds__(256) e2d_edge(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  const int t = blockIdx.x * 256 + threadIdx.x;
  if (t >= p.nedge) return;
  K2<T, L, V>::unit_e(p, __ldg(p.edge_units + t), step_n(p));
}

template <typename T, int L, int V>
__global__ void __launch_bounds__(256) h2d_edge(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  const int t = blockIdx.x * 256 + threadIdx.x;
  if (t >= p.nedge) return;
  K2<T, L, V>::unit_h(p, __ldg(p.edge_units + t), step_n(p));
}

// The fused 2D step kernel follows this one with a programmatic dependency
// and waits for it only where it meets a dispersive cell: it may start once
// every block here has passed its own wait (and with it, the previous step).
template <typename T, int L, int KIND>
__global__ void __launch_bounds__(256) e2d_ade(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  pdl_release();
  const int s = blockIdx.x * 256 + threadIdx.x;
  if (s < p.nade) ade_e2<T, L, KIND>(p, s, step_n(p));
}

// the dispersive-cell kernel for the job's kinds: the gold update's own
// instance when every dispersive material runs it
template <typename T, int L>
void launch_ade(const StepParams<T> &p, int blocks, cudaStream_t s, bool pdl) {
  if (p.ade_kind == MK_GOLD) {
    if (pdl) launch_pdl(e2d_ade<T, L, MK_GOLD>, blocks, 256, s, p);
    else launch_side(e2d_ade<T, L, MK_GOLD>, blocks, 256, s, p);
  } else {
    if (pdl) launch_pdl(e2d_ade<T, L, -1>, blocks, 256, s, p);
    else launch_side(e2d_ade<T, L, -1>, blocks, 256, s, p);
  }
}

// The E half's side kernel when the job has dispersive cells: the edge
// units' blocks, then the dispersive cells' blocks, in one launch beside the
// core kernel (one branch of the step's graph instead of two)
template <typename T, int L, int V, int KIND>
__global__ void __launch_bounds__(256) e2d_edge_ade(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  const int eb = (p.nedge + 255) / 256;
  if ((int)blockIdx.x < eb) {
    const int t = blockIdx.x * 256 + threadIdx.x;
    if (t < p.nedge && (p.roles & (ROLE_MAIN | ROLE_PML))) K2<T, L, V>::unit_e(p, __ldg(p.edge_units + t), step_n(p));
    return;
  }
  const int s = ((int)blockIdx.x - eb) * 256 + threadIdx.x;
  if (s < p.nade && (p.roles & ROLE_ADE)) ade_e2<T, L, KIND>(p, s, step_n(p));
}

// V: cells per unit along x; 4 (float) / 2 (double) when the row length
// allows aligned vector access, else 1.  Returns the kernels launched (0/1).
// `ev`: the core kernel's programmatic event (see launch_pdl), or null; side
// kernels launch with the device's top priority
template <typename T, int L, int V>
int launch_e2d_v(const StepParams<T> &p, int part, cudaStream_t s, cudaEvent_t ev) {
  const int units = part == K2D_CORE ? p.ncore : part == K2D_EDGE ? p.nedge + p.nade : p.nade;
  if (units <= 0) return 0;
  const int blocks = (units + 255) / 256;
  if (part == K2D_CORE) launch_core2_tiled<T, L, V>(p, true, s, ev);
  else if (part == K2D_EDGE && p.nade > 0) {
    const int b2 = (p.nedge + 255) / 256 + (p.nade + 255) / 256;
    if (p.ade_kind == MK_GOLD) launch_side(e2d_edge_ade<T, L, V, MK_GOLD>, b2, 256, s, p);
    else launch_side(e2d_edge_ade<T, L, V, -1>, b2, 256, s, p);
  }
  else if (part == K2D_EDGE) launch_side(e2d_edge<T, L, V>, blocks, 256, s, p);
  else launch_ade<T, L>(p, blocks, s, false);
  return 1;
}
template <typename T, int L, int V>
int launch_h2d_v(const StepParams<T> &p, int part, cudaStream_t s, cudaEvent_t ev) {
  const int units = part == K2D_CORE ? p.ncore : part == K2D_EDGE ? p.nedge : 0;
  if (units <= 0) return 0;
  const int blocks = (units + 255) / 256;
  if (part == K2D_CORE) launch_core2_tiled<T, L, V>(p, false, s, ev);
  else launch_side(h2d_edge<T, L, V>, blocks, 256, s, p);
  return 1;
}

template <typename T>
int launch_e2d(const StepParams<T> &p, int part, void *stream, void *prog_event) {
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t ev = (cudaEvent_t)prog_event;
  if (p.layout == 3)
    return p.vec == VW ? launch_e2d_v<T, 3, VW>(p, part, s, ev) : launch_e2d_v<T, 3, 1>(p, part, s, ev);
  return p.vec == VW ? launch_e2d_v<T, 2, VW>(p, part, s, ev) : launch_e2d_v<T, 2, 1>(p, part, s, ev);
}

template <typename T>
int launch_e2d_ade_pdl(const StepParams<T> &p, void *stream) {
  if (p.nade <= 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (p.layout == 3) launch_ade<T, 3>(p, (p.nade + 255) / 256, s, true);
  else launch_ade<T, 2>(p, (p.nade + 255) / 256, s, true);
  return 1;
}

template <typename T>
int launch_h2d(const StepParams<T> &p, int part, void *stream, void *prog_event) {
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t ev = (cudaEvent_t)prog_event;
  if (p.layout == 3)
    return p.vec == VW ? launch_h2d_v<T, 3, VW>(p, part, s, ev) : launch_h2d_v<T, 3, 1>(p, part, s, ev);
  return p.vec == VW ? launch_h2d_v<T, 2, VW>(p, part, s, ev) : launch_h2d_v<T, 2, 1>(p, part, s, ev);
}

// ---- packs: one launch runs the same part of many jobs' half steps ---------
// Block b belongs to the job q with bstart[q] <= b < bstart[q+1]; the job's
// parameters come from the slot's table in device memory.
template <typename T>
__device__ __forceinline__ int pack_job(const PackLaunch<T> &a) {
  int q = 0;
  while (q + 1 < a.njobs && (int)blockIdx.x >= a.bstart[q + 1]) ++q;
  return q;
}

// The block's job parameters, copied once into shared memory: the kernels
// read many of them before their first field load, and from the table each
// would be a dependent global load.
template <typename T>
__device__ __forceinline__ const StepParams<T> &pack_params(const PackLaunch<T> &a, int q) {
  static_assert(sizeof(StepParams<T>) % 8 == 0, "StepParams is copied in 8-byte words");
  __shared__ unsigned long long sm[sizeof(StepParams<T>) / 8];
  const unsigned long long *src = reinterpret_cast<const unsigned long long *>(a.tab + q);
  for (int w = threadIdx.x; w < (int)(sizeof(StepParams<T>) / 8); w += blockDim.x) sm[w] = __ldg(src + w);
  __syncthreads();
  return *reinterpret_cast<const StepParams<T> *>(sm);
}

template <typename T, int L, int V>
__global__ void __launch_bounds__(256) e2d_core_pk(const __grid_constant__ PackLaunch<T> a) {
  const int q = pack_job(a);
  const StepParams<T> &p = pack_params(a, q);
  const int t = ((int)blockIdx.x - a.bstart[q]) * 256 + threadIdx.x;
  if (t >= p.ncore) return;
  core_e<T, L, V>(p, p.cy0 + t / p.cw, (p.cv0 + t % p.cw) * V);
}

template <typename T, int L, int V>
__global__ void __launch_bounds__(256) h2d_core_pk(const __grid_constant__ PackLaunch<T> a) {
  const int q = pack_job(a);
  const StepParams<T> &p = pack_params(a, q);
  const int t = ((int)blockIdx.x - a.bstart[q]) * 256 + threadIdx.x;
  if (t >= p.ncore) return;
  core_h<T, L, V>(p, p.cy0 + t / p.cw, (p.cv0 + t % p.cw) * V);
}

template <typename T, int L, int V>
__global__ void __launch_bounds__(256) e2d_edge_pk(const __grid_constant__ PackLaunch<T> a) {
  const int q = pack_job(a);
  const StepParams<T> &p = pack_params(a, q);
  const int t = ((int)blockIdx.x - a.bstart[q]) * 256 + threadIdx.x;
  if (t >= p.nedge) return;
  K2<T, L, V>::unit_e(p, __ldg(p.edge_units + t), step_n(p));
}

template <typename T, int L, int V>
__global__ void __launch_bounds__(256) h2d_edge_pk(const __grid_constant__ PackLaunch<T> a) {
  const int q = pack_job(a);
  const StepParams<T> &p = pack_params(a, q);
  const int t = ((int)blockIdx.x - a.bstart[q]) * 256 + threadIdx.x;
  if (t >= p.nedge) return;
  K2<T, L, V>::unit_h(p, __ldg(p.edge_units + t), step_n(p));
}

template <typename T, int L>
__global__ void __launch_bounds__(256) e2d_ade_pk(const __grid_constant__ PackLaunch<T> a) {
  const int q = pack_job(a);
  const StepParams<T> &p = pack_params(a, q);
  const int s = ((int)blockIdx.x - a.bstart[q]) * 256 + threadIdx.x;
  if (s < p.nade) ade_e2<T, L>(p, s, step_n(p));
}

template <typename T, int L, int V>
void launch_pack_v(const PackLaunch<T> &a, bool e_half, int part, cudaStream_t s) {
  const int blocks = a.bstart[a.njobs];
  if (e_half) {
    if (part == K2D_CORE) e2d_core_pk<T, L, V><<<blocks, 256, 0, s>>>(a);
    else if (part == K2D_EDGE) e2d_edge_pk<T, L, V><<<blocks, 256, 0, s>>>(a);
    else e2d_ade_pk<T, L><<<blocks, 256, 0, s>>>(a);
  } else {
    if (part == K2D_CORE) h2d_core_pk<T, L, V><<<blocks, 256, 0, s>>>(a);
    else h2d_edge_pk<T, L, V><<<blocks, 256, 0, s>>>(a);
  }
}

template <typename T>
int launch_pack2d(const PackLaunch<T> &a, int layout, int vec, bool e_half, int part, void *stream) {
  if (a.njobs <= 0 || a.bstart[a.njobs] <= 0) return 0;
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  cudaStream_t s = (cudaStream_t)stream;
  if (layout == 3) {
    if (vec == VW) launch_pack_v<T, 3, VW>(a, e_half, part, s);
    else launch_pack_v<T, 3, 1>(a, e_half, part, s);
  } else {
    if (vec == VW) launch_pack_v<T, 2, VW>(a, e_half, part, s);
    else launch_pack_v<T, 2, 1>(a, e_half, part, s);
  }
  return 1;
}

template int launch_pack2d<float>(const PackLaunch<float> &, int, int, bool, int, void *);
template int launch_pack2d<double>(const PackLaunch<double> &, int, int, bool, int, void *);

template int launch_e2d<float>(const StepParams<float> &, int, void *, void *);
template int launch_e2d<double>(const StepParams<double> &, int, void *, void *);
template int launch_h2d<float>(const StepParams<float> &, int, void *, void *);
template int launch_h2d<double>(const StepParams<double> &, int, void *, void *);
template int launch_e2d_ade_pdl<float>(const StepParams<float> &, void *);
template int launch_e2d_ade_pdl<double>(const StepParams<double> &, void *);

}  // namespace fdtd
