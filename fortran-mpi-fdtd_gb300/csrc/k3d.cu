// k3d.cu -- 3D half-step kernels (3D/.../include/myfdtd_func.f90:19-64).
//
// A half step is two independent launches that write disjoint cells, run by
// the host as parallel branches of its stream:
//   core    : the interior box -- main cells outside the PML shell, in
//             (y, z) rows without a source -- one x-vector of V cells per
//             thread, only the Yee update with the constant-dielectric
//             material folded in.  Nearly all of a large grid.
//   general : blockIdx selects the work:
//     edge blocks : one x-vector per thread from a list of the units outside
//                 the core box or in a source row: shell cells of the
//                 split-field PML do the split update, main cells the Yee
//                 update with their material and the sources.
//     slab blocks : the reference's y-slab PML (3D/BERpmly_mod.f90:72-306),
//                 one thread per slab cell and side, 12 split arrays, the
//                 coupling rows read straight from the main arrays.
//     ADE blocks  : one thread per dispersive cell (3D/gold_mod.f90:50-88).
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {


// Ku/eps of a cell: the dominant material's coefficient is a parameter
template <typename T>
__device__ __forceinline__ T coef_ca3(const StepParams<T> &p, uint8_t id) {
  return id == p.id0 ? p.ca0 : __ldg(p.mca + id);
}

template <typename T>
struct F3 {
  const StepParams<T> &p;
  __device__ F3(const StepParams<T> &pp) : p(pp) {}
  __device__ __forceinline__ long long ix(int i, int j, int k) const {
    return (long long)i + (long long)p.nx * (j + (long long)p.ny * k);
  }
  // boundary-aware loads along each axis
  __device__ __forceinline__ T lx(const T *a, int i, int j, int k) const {
    if (i < 0) { if (!p.per[0]) return T(0); i = p.nx - 1; }
    else if (i >= p.nx) { if (!p.per[0]) return T(0); i = 0; }
    return a[ix(i, j, k)];
  }
  __device__ __forceinline__ T ly(const T *a, int i, int j, int k) const {
    if (j < 0) { if (!p.per[1]) return T(0); j = p.ny - 1; }
    else if (j >= p.ny) { if (!p.per[1]) return T(0); j = 0; }
    return a[ix(i, j, k)];
  }
  __device__ __forceinline__ T lz(const T *a, int i, int j, int k) const {
    if (k < 0) { if (!p.per[2]) return T(0); k = p.nz - 1; }
    else if (k >= p.nz) { if (!p.per[2]) return T(0); k = 0; }
    return a[ix(i, j, k)];
  }
};

// a cell of the core box in a row without flags: updated by the core launch
// ---- core units: one x-vector of V interior cells per thread --------------
// Block: 32 vectors along x by RY rows along y (RY from the commit-time
// tuner), one z plane; blocks run x, y, then z, so the plane below (E) or
// above (H) was read moments earlier and its loads hit L2.
template <typename T, int V, int RY = 8>
struct Core3 {
  int j, k, i0;
  long long c;
  bool live;
  __device__ __forceinline__ Core3(const StepParams<T> &p) {
    const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int bx = (p.cw + 31) >> 5, by = (p.ch + RY - 1) / RY;
    const int b = blockIdx.x, tx = b % bx, t2 = b / bx, ty = t2 % by, tz = t2 / by;
    const int v = tx * 32 + lane, r = ty * RY + wy;
    live = v < p.cw && r < p.ch && tz < p.cd;
    j = p.cy0 + r;
    k = p.cz0 + tz;
    i0 = (p.cv0 + v) * V;
    c = ((long long)k * p.ny + j) * p.nx + i0;
  }
};

// neighbour vector one row (dy = +-1) or one plane (dz = +-1) away, wrapped
// on periodic axes and zero beyond open ones
template <typename T, int V>
__device__ __forceinline__ void nb_vec(const StepParams<T> &p, const T *a, long long c, int j, int k, int dy, int dz,
                                       T (&v)[V]) {
  const long long plane = (long long)p.nx * p.ny;
  long long d = 0;
  bool ok = true;
  if (dy) {
    const int jj = j + dy;
    if (jj >= 0 && jj < p.ny) d = (long long)dy * p.nx;
    else if (p.per[1]) d = (long long)(dy > 0 ? -(p.ny - 1) : (p.ny - 1)) * p.nx;
    else ok = false;
  } else {
    const int kk = k + dz;
    if (kk >= 0 && kk < p.nz) d = (long long)dz * plane;
    else if (p.per[2]) d = (long long)(dz > 0 ? -(p.nz - 1) : (p.nz - 1)) * plane;
    else ok = false;
  }
  if (ok) vld_ro<T, V>(a + c + d, v);
  else {
#pragma unroll
    for (int q = 0; q < V; ++q) v[q] = T(0);
  }
}

// cell next to the vector along x (dx = -1: left of its first cell, +1:
// right of its last), wrapped on a periodic axis, zero beyond an open one
template <typename T, int V>
__device__ __forceinline__ T nb_x(const StepParams<T> &p, const T *a, long long c, int i0, int dx) {
  if (dx < 0) return i0 > 0 ? __ldg(a + c - 1) : (p.per[0] ? __ldg(a + c + p.nx - 1) : T(0));
  return i0 + V < p.nx ? __ldg(a + c + V) : (p.per[0] ? __ldg(a + c + V - p.nx) : T(0));
}

// ---- edge units: x-vectors of V cells outside the core launch's box --------
// (split-PML shell, the edges of the main range, rows with a source).  Every
// value a unit needs is loaded before any store, then each cell takes the
// split update (shell), the Yee update with material and source (main), or
// is left alone.
template <typename T, int V>
struct Edge3 {
  int i0, j, k;
  long long c;
  __device__ __forceinline__ Edge3(const StepParams<T> &p, int unit) {
    const int nvec = p.nx / V;
    const int row = unit / nvec;
    i0 = (unit - row * nvec) * V;
    j = row % p.ny;
    k = row / p.ny;
    c = (long long)row * p.nx + i0;
  }
};

template <typename T, int V>
__device__ __forceinline__ void edge_e3(const StepParams<T> &p, int unit, int n) {
  const Edge3<T, V> u(p, unit);
  const long long c = u.c;
  const int i0 = u.i0, j = u.j, k = u.k;
  const bool do_main = p.roles & ROLE_MAIN, do_pml = p.roles & ROLE_PML;
  const bool split = p.pml_mode == 2;
  const bool shell_yz = split && (j < p.slo[1] || j > p.shi[1] || k < p.slo[2] || k > p.shi[2]);
  const bool pml = do_pml && split && (shell_yz || i0 < p.slo[0] || i0 + V - 1 > p.shi[0]);
  const bool main_yz = j >= p.mlo[1] && j <= p.mhi[1] && k >= p.mlo[2] && k <= p.mhi[2];
  T hx[V], hy[V], hz[V], hzd[V], hxd[V], hyb[V], hxb[V], ex[V], ey[V], ez[V];
  uint8_t id[V];
  vld_ro<T, V>(p.hx + c, hx);
  vld_ro<T, V>(p.hy + c, hy);
  vld_ro<T, V>(p.hz + c, hz);
  nb_vec<T, V>(p, p.hz, c, j, k, -1, 0, hzd);
  nb_vec<T, V>(p, p.hx, c, j, k, -1, 0, hxd);
  nb_vec<T, V>(p, p.hy, c, j, k, 0, -1, hyb);
  nb_vec<T, V>(p, p.hx, c, j, k, 0, -1, hxb);
  const T hzl = nb_x<T, V>(p, p.hz, c, i0, -1), hyl = nb_x<T, V>(p, p.hy, c, i0, -1);
  vld<T, V>(p.ex + c, ex);
  vld<T, V>(p.ey + c, ey);
  vld<T, V>(p.ez + c, ez);
  vld_ids<V>(p.mat + c, id);
  const int rf = __ldg(p.rowflag + (long long)k * p.ny + j);
  // split parts Exy Eyz Ezx (and, in FP64, Exz Eyx Ezy) and the profiles.
  // In FP32 a component is split only where one of its two curl axes is a
  // PML axis of the cell; with neither (Ez in a z-slab, say) both parts
  // would take f1 = 1 and the same f2, so the component takes the plain
  // update E += f2 * curl, and its stored part is neither read nor written.
  // FP64 keeps the split everywhere in the shell, as the reference does.
  bool anyx = false;
#pragma unroll
  for (int q = 0; q < V; ++q) anyx |= i0 + q < p.slo[0] || i0 + q > p.shi[0];
  const bool iny = j < p.slo[1] || j > p.shi[1], inz = k < p.slo[2] || k > p.shi[2];
  const bool need0 = kTwoParts<T> || iny || inz, need1 = kTwoParts<T> || inz || anyx,
             need2 = kTwoParts<T> || anyx || iny;
  T s0[V] = {}, s1[V] = {}, s2[V] = {}, s6[V], s7[V], s8[V], f1x[V], f2x[V];
  T f1y = T(0), f2y = T(0), f1z = T(0), f2z = T(0);
  if (pml) {
    if (need0) vld<T, V>(p.sp[0] + c, s0);
    if (need1) vld<T, V>(p.sp[1] + c, s1);
    if (need2) vld<T, V>(p.sp[2] + c, s2);
    if (kTwoParts<T>) {
      vld<T, V>(p.sp[6] + c, s6);
      vld<T, V>(p.sp[7] + c, s7);
      vld<T, V>(p.sp[8] + c, s8);
    }
    vld_ro<T, V>(p.cf1[0] + i0, f1x);
    vld_ro<T, V>(p.cf2[0] + i0, f2x);
    f1y = __ldg(p.cf1[1] + j); f2y = __ldg(p.cf2[1] + j);
    f1z = __ldg(p.cf1[2] + k); f2z = __ldg(p.cf2[2] + k);
  }
  bool wrote = false;
#pragma unroll
  for (int q = 0; q < V; ++q) {
    const int i = i0 + q;
    const T curlhzy = hz[q] - hzd[q], curlhyz = -hy[q] + hyb[q];
    const T curlhxz = hx[q] - hxb[q], curlhzx = -hz[q] + (q ? hz[q - 1] : hzl);
    const T curlhyx = hy[q] - (q ? hy[q - 1] : hyl), curlhxy = -hx[q] + hxd[q];
    if (split && (shell_yz || i < p.slo[0] || i > p.shi[0])) {
      if (do_pml) {  // 3D/BERpmly_mod.f90:117-159 on every face
        const bool inx = i < p.slo[0] || i > p.shi[0];
        const T exz = kTwoParts<T> ? s6[q] : ex[q] - s0[q];
        const T eyx = kTwoParts<T> ? s7[q] : ey[q] - s1[q];
        const T ezy = kTwoParts<T> ? s8[q] : ez[q] - s2[q];
        const T nexy = f1y * s0[q] + f2y * curlhzy;
        const T nexz = f1z * exz + f2z * curlhyz;
        const T neyz = f1z * s1[q] + f2z * curlhxz;
        const T neyx = f1x[q] * eyx + f2x[q] * curlhzx;
        const T nezx = f1x[q] * s2[q] + f2x[q] * curlhyx;
        const T nezy = f1y * ezy + f2y * curlhxy;
        s0[q] = nexy; s1[q] = neyz; s2[q] = nezx;
        s6[q] = nexz; s7[q] = neyx; s8[q] = nezy;
        if (kTwoParts<T> || iny || inz) ex[q] = nexy + nexz;
        else ex[q] = ex[q] + f2y * (curlhzy + curlhyz);
        if (kTwoParts<T> || inz || inx) ey[q] = neyz + neyx;
        else ey[q] = ey[q] + f2z * (curlhxz + curlhzx);
        if (kTwoParts<T> || inx || iny) ez[q] = nezx + nezy;
        else ez[q] = ez[q] + f2x[q] * (curlhyx + curlhxy);
        wrote = true;
      }
    } else if (do_main && main_yz && i >= p.mlo[0] && i <= p.mhi[0]) {
      const T ca = coef_ca3(p, id[q]);
      ex[q] = ex[q] + ca * (curlhzy + curlhyz);
      ey[q] = ey[q] + ca * (curlhxz + curlhzx);
      ez[q] = ez[q] + ca * (curlhyx + curlhxy);
      if (rf & ROW_SRC) {
        const T cs = __ldg(p.mcs + id[q]);
        const T sx = src_sum<T>(p, n, 0, i, j, k), sy = src_sum<T>(p, n, 1, i, j, k), sz = src_sum<T>(p, n, 2, i, j, k);
        if (sx != T(0)) ex[q] += cs * sx;
        if (sy != T(0)) ey[q] += cs * sy;
        if (sz != T(0)) ez[q] += cs * sz;
      }
      wrote = true;
    }
  }
  if (wrote || p.pp) {  // cells not updated store what they read; ADE cells are skipped
    st_guard3<T, V>(p.exo + c, ex, id);
    st_guard3<T, V>(p.eyo + c, ey, id);
    st_guard3<T, V>(p.ezo + c, ez, id);
  }
  if (pml) {
    if (need0) vst<T, V>(p.sp[0] + c, s0);
    if (need1) vst<T, V>(p.sp[1] + c, s1);
    if (need2) vst<T, V>(p.sp[2] + c, s2);
    if (kTwoParts<T>) {
      vst<T, V>(p.sp[6] + c, s6);
      vst<T, V>(p.sp[7] + c, s7);
      vst<T, V>(p.sp[8] + c, s8);
    }
  }
}

template <typename T, int V>
__device__ __forceinline__ void edge_h3(const StepParams<T> &p, int unit) {
  const Edge3<T, V> u(p, unit);
  const long long c = u.c;
  const int i0 = u.i0, j = u.j, k = u.k;
  const bool do_main = p.roles & ROLE_MAIN, do_pml = p.roles & ROLE_PML;
  const bool split = p.pml_mode == 2;
  const bool shell_yz = split && (j < p.slo[1] || j > p.shi[1] || k < p.slo[2] || k > p.shi[2]);
  const bool pml = do_pml && split && (shell_yz || i0 < p.slo[0] || i0 + V - 1 > p.shi[0]);
  const bool main_yz = j >= p.mlo[1] && j <= p.mhi[1] && k >= p.mlo[2] && k <= p.mhi[2];
  T ex[V], ey[V], ez[V], ezu[V], exu[V], exa[V], eya[V], hx[V], hy[V], hz[V];
  vld_ro<T, V>(p.ex + c, ex);
  vld_ro<T, V>(p.ey + c, ey);
  vld_ro<T, V>(p.ez + c, ez);
  nb_vec<T, V>(p, p.ez, c, j, k, 1, 0, ezu);
  nb_vec<T, V>(p, p.ex, c, j, k, 1, 0, exu);
  nb_vec<T, V>(p, p.ex, c, j, k, 0, 1, exa);
  nb_vec<T, V>(p, p.ey, c, j, k, 0, 1, eya);
  const T ezr = nb_x<T, V>(p, p.ez, c, i0, 1), eyr = nb_x<T, V>(p, p.ey, c, i0, 1);
  vld<T, V>(p.hx + c, hx);
  vld<T, V>(p.hy + c, hy);
  vld<T, V>(p.hz + c, hz);
  // split parts Hxy Hyz Hzx (and, in FP64, Hxz Hyx Hzy) and the profiles;
  // in FP32 only the components that need a split (as in edge_e3)
  bool anyx = false;
#pragma unroll
  for (int q = 0; q < V; ++q) anyx |= i0 + q < p.slo[0] || i0 + q > p.shi[0];
  const bool iny = j < p.slo[1] || j > p.shi[1], inz = k < p.slo[2] || k > p.shi[2];
  const bool need3 = kTwoParts<T> || iny || inz, need4 = kTwoParts<T> || inz || anyx,
             need5 = kTwoParts<T> || anyx || iny;
  T s3[V] = {}, s4[V] = {}, s5[V] = {}, s9[V], s10[V], s11[V], g1x[V], g2x[V];
  T g1y = T(0), g2y = T(0), g1z = T(0), g2z = T(0);
  if (pml) {
    if (need3) vld<T, V>(p.sp[3] + c, s3);
    if (need4) vld<T, V>(p.sp[4] + c, s4);
    if (need5) vld<T, V>(p.sp[5] + c, s5);
    if (kTwoParts<T>) {
      vld<T, V>(p.sp[9] + c, s9);
      vld<T, V>(p.sp[10] + c, s10);
      vld<T, V>(p.sp[11] + c, s11);
    }
    vld_ro<T, V>(p.cg1[0] + i0, g1x);
    vld_ro<T, V>(p.cg2[0] + i0, g2x);
    g1y = __ldg(p.cg1[1] + j); g2y = __ldg(p.cg2[1] + j);
    g1z = __ldg(p.cg1[2] + k); g2z = __ldg(p.cg2[2] + k);
  }
  bool wrote = false;
#pragma unroll
  for (int q = 0; q < V; ++q) {
    const int i = i0 + q;
    const T rz = q < V - 1 ? ez[q + 1] : ezr, ry = q < V - 1 ? ey[q + 1] : eyr;
    const T curleyz = eya[q] - ey[q], curlezy = -ezu[q] + ez[q];
    const T curlezx = rz - ez[q], curlexz = -exa[q] + ex[q];
    const T curlexy = exu[q] - ex[q], curleyx = -ry + ey[q];
    if (split && (shell_yz || i < p.slo[0] || i > p.shi[0])) {
      if (do_pml) {  // 3D/BERpmly_mod.f90:161-195 on every face
        const T hxz = kTwoParts<T> ? s9[q] : hx[q] - s3[q];
        const T hyx = kTwoParts<T> ? s10[q] : hy[q] - s4[q];
        const T hzy = kTwoParts<T> ? s11[q] : hz[q] - s5[q];
        const T nhxy = g1y * s3[q] + g2y * curlezy;
        const T nhxz = g1z * hxz + g2z * curleyz;
        const T nhyz = g1z * s4[q] + g2z * curlexz;
        const T nhyx = g1x[q] * hyx + g2x[q] * curlezx;
        const T nhzx = g1x[q] * s5[q] + g2x[q] * curleyx;
        const T nhzy = g1y * hzy + g2y * curlexy;
        s3[q] = nhxy; s4[q] = nhyz; s5[q] = nhzx;
        s9[q] = nhxz; s10[q] = nhyx; s11[q] = nhzy;
        const bool inx = i < p.slo[0] || i > p.shi[0];
        if (kTwoParts<T> || iny || inz) hx[q] = nhxy + nhxz;
        else hx[q] = hx[q] + g2y * (curleyz + curlezy);
        if (kTwoParts<T> || inz || inx) hy[q] = nhyz + nhyx;
        else hy[q] = hy[q] + g2z * (curlezx + curlexz);
        if (kTwoParts<T> || inx || iny) hz[q] = nhzx + nhzy;
        else hz[q] = hz[q] + g2x[q] * (curlexy + curleyx);
        wrote = true;
      }
    } else if (do_main && main_yz && i >= p.mlo[0] && i <= p.mhi[0]) {
      hx[q] = hx[q] + p.ku * (curleyz + curlezy);
      hy[q] = hy[q] + p.ku * (curlezx + curlexz);
      hz[q] = hz[q] + p.ku * (curlexy + curleyx);
      wrote = true;
    }
  }
  if (wrote || p.pp) {
    vst<T, V>(p.hxo + c, hx);
    vst<T, V>(p.hyo + c, hy);
    vst<T, V>(p.hzo + c, hz);
  }
  if (pml) {
    if (need3) vst<T, V>(p.sp[3] + c, s3);
    if (need4) vst<T, V>(p.sp[4] + c, s4);
    if (need5) vst<T, V>(p.sp[5] + c, s5);
    if (kTwoParts<T>) {
      vst<T, V>(p.sp[9] + c, s9);
      vst<T, V>(p.sp[10] + c, s10);
      vst<T, V>(p.sp[11] + c, s11);
    }
  }
}

// ---- the reference's y-slab PML (3D/BERpmly_mod.f90) ---------------------
// slab arrays: index (k*rows + r)*nx + i, split order
// 0 Exy 1 Exz 2 Eyz 3 Eyx 4 Ezx 5 Ezy 6 Hxy 7 Hxz 8 Hyz 9 Hyx 10 Hzx 11 Hzy
template <typename T>
__device__ __forceinline__ void slab_e3(const StepParams<T> &p, int t) {
  const int nx = p.nx, nz = p.nz, rows = p.slab_rows;
  const int per_side = nx * rows * nz;
  int side = t / per_side, q = t % per_side;
  if (side > 1 || !p.slab_on[side]) return;
  const int i = q % nx, r = (q / nx) % rows, k = q / (nx * rows);
  const int j = p.slab_j0[side] + r;
  T *const *s = p.slab[side];
  const long long c = ((long long)k * rows + r) * nx + i;
  auto at = [&](int a, int ii, int rr, int kk) -> T {
    if (ii < 0 || kk < 0) return T(0);
    return s[a][((long long)kk * rows + rr) * nx + ii];
  };
  // H splits at (i, r-1): low side r=0 -> zero; high side r=0 -> coupling row
  T hzx_jm, hzy_jm, hxy_jm, hxz_jm;
  if (r > 0) {
    hzx_jm = at(10, i, r - 1, k); hzy_jm = at(11, i, r - 1, k);
    hxy_jm = at(6, i, r - 1, k); hxz_jm = at(7, i, r - 1, k);
  } else if (side == 1) {
    const long long cm = (long long)i + (long long)nx * ((j - 1) + (long long)p.ny * k);
    hzx_jm = T(0); hzy_jm = p.hz[cm]; hxy_jm = p.hx[cm]; hxz_jm = T(0);
  } else {
    hzx_jm = hzy_jm = hxy_jm = hxz_jm = T(0);
  }
  const T curlHzy_p = s[10][c] + s[11][c];
  const T curlHzy_m = -hzx_jm - hzy_jm;
  const T curlHyz_p = -s[8][c] - s[9][c];
  const T curlHyz_m = at(8, i, r, k - 1) + at(9, i, r, k - 1);
  const T curlHxz_p = s[6][c] + s[7][c];
  const T curlHxz_m = -at(6, i, r, k - 1) - at(7, i, r, k - 1);
  const T curlHzx_p = -s[10][c] - s[11][c];
  const T curlHzx_m = at(10, i - 1, r, k) + at(11, i - 1, r, k);
  const T curlHyx_p = s[8][c] + s[9][c];
  const T curlHyx_m = -at(8, i - 1, r, k) - at(9, i - 1, r, k);
  const T curlHxy_p = -s[6][c] - s[7][c];
  const T curlHxy_m = hxy_jm + hxz_jm;
  const T f1x = p.sf1x[side][i], f2x = p.sf2x[side][i];
  const T f1y = p.sf1y[side][r], f2y = p.sf2y[side][r];
  const T f1z = p.sf1z[side][k], f2z = p.sf2z[side][k];
  s[3][c] = f1x * s[3][c] + f2x * (curlHzx_p + curlHzx_m);
  s[4][c] = f1x * s[4][c] + f2x * (curlHyx_p + curlHyx_m);
  const T exy = f1y * s[0][c] + f2y * (curlHzy_p + curlHzy_m);
  const T ezy = f1y * s[5][c] + f2y * (curlHxy_p + curlHxy_m);
  s[0][c] = exy;
  s[5][c] = ezy;
  s[1][c] = f1z * s[1][c] + f2z * (curlHyz_p + curlHyz_m);
  s[2][c] = f1z * s[2][c] + f2z * (curlHxz_p + curlHxz_m);
  // setboundayEya/b: Ex_(ja) = Exy(ja), Ez_(ja) = Ezy(ja) (jb on the high side)
  if ((side == 0 && r == rows - 1) || (side == 1 && r == 0)) {
    const long long cm = (long long)i + (long long)nx * (j + (long long)p.ny * k);
    p.ex[cm] = exy;
    p.ez[cm] = ezy;
  }
}

template <typename T>
__device__ __forceinline__ void slab_h3(const StepParams<T> &p, int t) {
  const int nx = p.nx, nz = p.nz, rows = p.slab_rows;
  const int per_side = nx * rows * nz;
  int side = t / per_side, q = t % per_side;
  if (side > 1 || !p.slab_on[side]) return;
  const int i = q % nx, r = (q / nx) % rows, k = q / (nx * rows);
  const int j = p.slab_j0[side] + r;
  T *const *s = p.slab[side];
  const long long c = ((long long)k * rows + r) * nx + i;
  auto at = [&](int a, int ii, int rr, int kk) -> T {
    if (ii >= nx || kk >= nz) return T(0);
    return s[a][((long long)kk * rows + rr) * nx + ii];
  };
  // E splits at (i, r+1): low side top row -> coupling row (main E at ja+1);
  // high side top row -> the PEC row (zero)
  T ezx_jp, ezy_jp, exy_jp, exz_jp;
  if (r + 1 < rows) {
    ezx_jp = at(4, i, r + 1, k); ezy_jp = at(5, i, r + 1, k);
    exy_jp = at(0, i, r + 1, k); exz_jp = at(1, i, r + 1, k);
  } else if (side == 0) {
    const long long cp = (long long)i + (long long)nx * ((j + 1) + (long long)p.ny * k);
    ezx_jp = T(0); ezy_jp = p.ez[cp]; exy_jp = p.ex[cp]; exz_jp = T(0);
  } else {
    ezx_jp = ezy_jp = exy_jp = exz_jp = T(0);
  }
  const T curlEzy_p = -ezx_jp - ezy_jp;
  const T curlEzy_m = s[4][c] + s[5][c];
  const T curlEyz_p = at(2, i, r, k + 1) + at(3, i, r, k + 1);
  const T curlEyz_m = -s[2][c] - s[3][c];
  const T curlExz_p = -at(0, i, r, k + 1) - at(1, i, r, k + 1);
  const T curlExz_m = s[0][c] + s[1][c];
  const T curlEzx_p = at(4, i + 1, r, k) + at(5, i + 1, r, k);
  const T curlEzx_m = -s[4][c] - s[5][c];
  const T curlEyx_p = -at(2, i + 1, r, k) - at(3, i + 1, r, k);
  const T curlEyx_m = s[2][c] + s[3][c];
  const T curlExy_p = exy_jp + exz_jp;
  const T curlExy_m = -s[0][c] - s[1][c];
  const T g1x = p.sg1x[side][i], g2x = p.sg2x[side][i];
  const T g1y = p.sg1y[side][r], g2y = p.sg2y[side][r];
  const T g1z = p.sg1z[side][k], g2z = p.sg2z[side][k];
  s[9][c] = g1x * s[9][c] + g2x * (curlEzx_m + curlEzx_p);
  s[10][c] = g1x * s[10][c] + g2x * (curlEyx_m + curlEyx_p);
  const T hxy = g1y * s[6][c] + g2y * (curlEzy_m + curlEzy_p);
  const T hzy = g1y * s[11][c] + g2y * (curlExy_m + curlExy_p);
  s[6][c] = hxy;
  s[11][c] = hzy;
  s[7][c] = g1z * s[7][c] + g2z * (curlEyz_m + curlEyz_p);
  s[8][c] = g1z * s[8][c] + g2z * (curlExz_m + curlExz_p);
  // setboundayHya/b: Hx_(ja) = Hxy(ja), Hz_(ja) = Hzy(ja) (jb on the high side)
  if ((side == 0 && r == rows - 1) || (side == 1 && r == 0)) {
    const long long cm = (long long)i + (long long)nx * (j + (long long)p.ny * k);
    p.hx[cm] = hxy;
    p.hz[cm] = hzy;
  }
}

template <typename T>
__device__ __forceinline__ void ade_e3(const StepParams<T> &p, int s, int n) {
  const int cell = p.ade_cell[s];
  const int nx = p.nx, ny = p.ny;
  const int i = cell % nx, j = (cell / nx) % ny, k = cell / (nx * ny);
  F3<T> f(p);
  const AdeCoef<T> &a = ade_coef(p, p.ade_mat[s]);
  const AdeCoef<T> *am = p.ac + (p.ade_mat[s] - kAdeId);
  const T hxc = p.hx[cell], hyc = p.hy[cell], hzc = p.hz[cell];
  const T curlhzy = hzc - f.ly(p.hz, i, j - 1, k), curlhyz = -hyc + f.lz(p.hy, i, j, k - 1);
  const T curlhxz = hxc - f.lz(p.hx, i, j, k - 1), curlhzx = -hzc + f.lx(p.hz, i - 1, j, k);
  const T curlhyx = hyc - f.lx(p.hy, i - 1, j, k), curlhxy = -hxc + f.ly(p.hx, i, j - 1, k);
  const T ix_ = p.ku * (curlhzy + curlhyz) + src_sum<T>(p, n, 0, i, j, k);
  const T iy_ = p.ku * (curlhxz + curlhzx) + src_sum<T>(p, n, 1, i, j, k);
  const T iz_ = p.ku * (curlhyx + curlhxy) + src_sum<T>(p, n, 2, i, j, k);
  p.exo[cell] = ade_update<T>(p, a, am, s, 0, ix_, p.ex[cell]);
  p.eyo[cell] = ade_update<T>(p, a, am, s, 1, iy_, p.ey[cell]);
  p.ezo[cell] = ade_update<T>(p, a, am, s, 2, iz_, p.ez[cell]);
}

// general launch: blockIdx selects edge units, reference slab cells, then
// dispersive cells.  It may be launched early, off the previous core kernel's
// programmatic event, and then waits for that kernel here first.
template <typename T, int V>
__global__ void __launch_bounds__(256, 3) e3d_kernel(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  const int n = step_n(p);
  int b = blockIdx.x;
  if (b < p.ntile_blocks) {
    const int t = b * 256 + threadIdx.x;
    if (t < p.nedge && (p.roles & (ROLE_MAIN | ROLE_PML))) edge_e3<T, V>(p, __ldg(p.edge_units + t), n);
    return;
  }
  b -= p.ntile_blocks;
  if (b < p.nslab_blocks) {
    if (p.roles & ROLE_PML) slab_e3<T>(p, b * 256 + threadIdx.x);
    return;
  }
  b -= p.nslab_blocks;
  if (p.roles & ROLE_ADE) {
    const int s = b * 256 + threadIdx.x;
    if (s < p.nade) ade_e3<T>(p, s, n);
  }
}

template <typename T, int V>
__global__ void __launch_bounds__(256, 3) h3d_kernel(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  int b = blockIdx.x;
  if (b < p.ntile_blocks) {
    const int t = b * 256 + threadIdx.x;
    if (t < p.nedge && (p.roles & (ROLE_MAIN | ROLE_PML))) edge_h3<T, V>(p, __ldg(p.edge_units + t));
    return;
  }
  b -= p.ntile_blocks;
  if (b < p.nslab_blocks && (p.roles & ROLE_PML)) slab_h3<T>(p, b * 256 + threadIdx.x);
}

template <typename T, int V, int RY>
__global__ void __launch_bounds__(32 * RY) e3d_core(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  pdl_release();
  const Core3<T, V, RY> u(p);
  if (!u.live) return;
  const long long c = u.c;
  T hx[V], hy[V], hz[V], hzd[V], hxd[V], hyb[V], hxb[V], ex[V], ey[V], ez[V];
  uint8_t id[V];
  vld_ro<T, V>(p.hx + c, hx);
  vld_ro<T, V>(p.hy + c, hy);
  vld_ro<T, V>(p.hz + c, hz);
  nb_vec<T, V>(p, p.hz, c, u.j, u.k, -1, 0, hzd);
  nb_vec<T, V>(p, p.hx, c, u.j, u.k, -1, 0, hxd);
  nb_vec<T, V>(p, p.hy, c, u.j, u.k, 0, -1, hyb);
  nb_vec<T, V>(p, p.hx, c, u.j, u.k, 0, -1, hxb);
  const T hzl = nb_x<T, V>(p, p.hz, c, u.i0, -1), hyl = nb_x<T, V>(p, p.hy, c, u.i0, -1);
  vld<T, V>(p.ex + c, ex);
  vld<T, V>(p.ey + c, ey);
  vld<T, V>(p.ez + c, ez);
  vec_ids<T, V>(p, (long long)u.k * p.ny + u.j, u.i0 / V, p.mat + c, id);
  if (__ldg(p.rowflag + (long long)u.k * p.ny + u.j)) return;  // source rows: general launch
  bool uni = true;
#pragma unroll
  for (int q = 0; q < V; ++q) uni &= id[q] == p.id0;
#pragma unroll
  for (int q = 0; q < V; ++q) {
    const T ca = uni ? p.ca0 : coef_ca3(p, id[q]);
    const T curlhzy = hz[q] - hzd[q], curlhyz = -hy[q] + hyb[q];
    const T curlhxz = hx[q] - hxb[q], curlhzx = -hz[q] + (q ? hz[q - 1] : hzl);
    const T curlhyx = hy[q] - (q ? hy[q - 1] : hyl), curlhxy = -hx[q] + hxd[q];
    ex[q] = ex[q] + ca * (curlhzy + curlhyz);
    ey[q] = ey[q] + ca * (curlhxz + curlhzx);
    ez[q] = ez[q] + ca * (curlhyx + curlhxy);
  }
  if (uni) {
    vst<T, V>(p.ex + c, ex);
    vst<T, V>(p.ey + c, ey);
    vst<T, V>(p.ez + c, ez);
  } else {  // dispersive cells belong to the ADE blocks
    st_guard3<T, V>(p.ex + c, ex, id);
    st_guard3<T, V>(p.ey + c, ey, id);
    st_guard3<T, V>(p.ez + c, ez, id);
  }
}

template <typename T, int V, int RY>
__global__ void __launch_bounds__(32 * RY) h3d_core(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  pdl_release();
  const Core3<T, V, RY> u(p);
  if (!u.live) return;
  const long long c = u.c;
  T ex[V], ey[V], ez[V], ezu[V], exu[V], exa[V], eya[V], hx[V], hy[V], hz[V];
  vld_ro<T, V>(p.ex + c, ex);
  vld_ro<T, V>(p.ey + c, ey);
  vld_ro<T, V>(p.ez + c, ez);
  nb_vec<T, V>(p, p.ez, c, u.j, u.k, 1, 0, ezu);
  nb_vec<T, V>(p, p.ex, c, u.j, u.k, 1, 0, exu);
  nb_vec<T, V>(p, p.ex, c, u.j, u.k, 0, 1, exa);
  nb_vec<T, V>(p, p.ey, c, u.j, u.k, 0, 1, eya);
  const T ezr = nb_x<T, V>(p, p.ez, c, u.i0, 1), eyr = nb_x<T, V>(p, p.ey, c, u.i0, 1);
  vld<T, V>(p.hx + c, hx);
  vld<T, V>(p.hy + c, hy);
  vld<T, V>(p.hz + c, hz);
  if (__ldg(p.rowflag + (long long)u.k * p.ny + u.j)) return;
#pragma unroll
  for (int q = 0; q < V; ++q) {
    const T rz = q < V - 1 ? ez[q + 1] : ezr, ry = q < V - 1 ? ey[q + 1] : eyr;
    const T curleyz = eya[q] - ey[q], curlezy = -ezu[q] + ez[q];
    const T curlezx = rz - ez[q], curlexz = -exa[q] + ex[q];
    const T curlexy = exu[q] - ex[q], curleyx = -ry + ey[q];
    hx[q] = hx[q] + p.ku * (curleyz + curlezy);
    hy[q] = hy[q] + p.ku * (curlezx + curlexz);
    hz[q] = hz[q] + p.ku * (curlexy + curleyx);
  }
  vst<T, V>(p.hx + c, hx);
  vst<T, V>(p.hy + c, hy);
  vst<T, V>(p.hz + c, hz);
}

// ---- z-marching core kernels: one thread owns an x-vector of one row and
// walks KZ planes upward.  The E half keeps Hx, Hy of the plane below from
// the previous plane's loads, the H half takes Ex, Ey of the plane above as
// the next plane's own values, so each cell reads two vectors fewer.  The
// arithmetic per cell is that of e3d_core / h3d_core, term for term.
template <typename T, int V, int RY, int KZ>
struct Core3z {
  int j, k0, k1, i0;
  bool live;
  __device__ __forceinline__ Core3z(const StepParams<T> &p) {
    const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int bx = (p.cw + 31) >> 5, by = (p.ch + RY - 1) / RY;
    const int b = blockIdx.x, tx = b % bx, t2 = b / bx, ty = t2 % by, tz = t2 / by;
    const int v = tx * 32 + lane, r = ty * RY + wy;
    k0 = p.cz0 + tz * KZ;
    k1 = min(p.cz0 + p.cd, k0 + KZ);
    live = v < p.cw && r < p.ch && k0 < k1;
    j = p.cy0 + r;
    i0 = (p.cv0 + v) * V;
  }
};

template <typename T, int V, int RY, int KZ>
__global__ void __launch_bounds__(32 * RY) e3d_corez(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  pdl_release();
  const Core3z<T, V, RY, KZ> u(p);
  if (!u.live) return;
  const long long plane = (long long)p.nx * p.ny;
  long long c = ((long long)u.k0 * p.ny + u.j) * p.nx + u.i0;
  T hyb[V], hxb[V];
  nb_vec<T, V>(p, p.hy, c, u.j, u.k0, 0, -1, hyb);
  nb_vec<T, V>(p, p.hx, c, u.j, u.k0, 0, -1, hxb);
  for (int k = u.k0; k < u.k1; ++k, c += plane) {
    T hx[V], hy[V], hz[V], hzd[V], hxd[V], ex[V], ey[V], ez[V];
    uint8_t id[V];
    vld_ro<T, V>(p.hx + c, hx);
    vld_ro<T, V>(p.hy + c, hy);
    vld_ro<T, V>(p.hz + c, hz);
    nb_vec<T, V>(p, p.hz, c, u.j, k, -1, 0, hzd);
    nb_vec<T, V>(p, p.hx, c, u.j, k, -1, 0, hxd);
    const T hzl = nb_x<T, V>(p, p.hz, c, u.i0, -1), hyl = nb_x<T, V>(p, p.hy, c, u.i0, -1);
    vld<T, V>(p.ex + c, ex);
    vld<T, V>(p.ey + c, ey);
    vld<T, V>(p.ez + c, ez);
    vec_ids<T, V>(p, (long long)k * p.ny + u.j, u.i0 / V, p.mat + c, id);
    if (!__ldg(p.rowflag + (long long)k * p.ny + u.j)) {  // source rows: general launch
      bool uni = true;
#pragma unroll
      for (int q = 0; q < V; ++q) uni &= id[q] == p.id0;
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const T ca = uni ? p.ca0 : coef_ca3(p, id[q]);
        const T curlhzy = hz[q] - hzd[q], curlhyz = -hy[q] + hyb[q];
        const T curlhxz = hx[q] - hxb[q], curlhzx = -hz[q] + (q ? hz[q - 1] : hzl);
        const T curlhyx = hy[q] - (q ? hy[q - 1] : hyl), curlhxy = -hx[q] + hxd[q];
        ex[q] = ex[q] + ca * (curlhzy + curlhyz);
        ey[q] = ey[q] + ca * (curlhxz + curlhzx);
        ez[q] = ez[q] + ca * (curlhyx + curlhxy);
      }
      if (uni) {
        vst<T, V>(p.ex + c, ex);
        vst<T, V>(p.ey + c, ey);
        vst<T, V>(p.ez + c, ez);
      } else {  // dispersive cells belong to the ADE blocks
        st_guard3<T, V>(p.ex + c, ex, id);
        st_guard3<T, V>(p.ey + c, ey, id);
        st_guard3<T, V>(p.ez + c, ez, id);
      }
    }
#pragma unroll
    for (int q = 0; q < V; ++q) {
      hyb[q] = hy[q];
      hxb[q] = hx[q];
    }
  }
}

template <typename T, int V, int RY, int KZ>
__global__ void __launch_bounds__(32 * RY) h3d_corez(const __grid_constant__ StepParams<T> p) {
  pdl_wait();
  pdl_release();
  const Core3z<T, V, RY, KZ> u(p);
  if (!u.live) return;
  const long long plane = (long long)p.nx * p.ny;
  long long c = ((long long)u.k0 * p.ny + u.j) * p.nx + u.i0;
  T ex[V], ey[V];
  vld_ro<T, V>(p.ex + c, ex);
  vld_ro<T, V>(p.ey + c, ey);
  for (int k = u.k0; k < u.k1; ++k, c += plane) {
    T ez[V], ezu[V], exu[V], exa[V], eya[V], hx[V], hy[V], hz[V];
    vld_ro<T, V>(p.ez + c, ez);
    nb_vec<T, V>(p, p.ez, c, u.j, k, 1, 0, ezu);
    nb_vec<T, V>(p, p.ex, c, u.j, k, 1, 0, exu);
    nb_vec<T, V>(p, p.ex, c, u.j, k, 0, 1, exa);
    nb_vec<T, V>(p, p.ey, c, u.j, k, 0, 1, eya);
    const T ezr = nb_x<T, V>(p, p.ez, c, u.i0, 1), eyr = nb_x<T, V>(p, p.ey, c, u.i0, 1);
    vld<T, V>(p.hx + c, hx);
    vld<T, V>(p.hy + c, hy);
    vld<T, V>(p.hz + c, hz);
    if (!__ldg(p.rowflag + (long long)k * p.ny + u.j)) {
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const T rz = q < V - 1 ? ez[q + 1] : ezr, ry = q < V - 1 ? ey[q + 1] : eyr;
        const T curleyz = eya[q] - ey[q], curlezy = -ezu[q] + ez[q];
        const T curlezx = rz - ez[q], curlexz = -exa[q] + ex[q];
        const T curlexy = exu[q] - ex[q], curleyx = -ry + ey[q];
        hx[q] = hx[q] + p.ku * (curleyz + curlezy);
        hy[q] = hy[q] + p.ku * (curlezx + curlexz);
        hz[q] = hz[q] + p.ku * (curlexy + curleyx);
      }
      vst<T, V>(p.hx + c, hx);
      vst<T, V>(p.hy + c, hy);
      vst<T, V>(p.hz + c, hz);
    }
#pragma unroll
    for (int q = 0; q < V; ++q) {
      ex[q] = exa[q];
      ey[q] = eya[q];
    }
  }
}

// ---- TMA-staged E core (FP32) ----------------------------------------------
// A block owns a tile of kTmaX cells along x by kTmaY rows and marches up to
// kTmaZ planes of the core box along z (more blocks than planes per block:
// a block's planes run one after another).  For every plane one thread issues
// three tiled bulk copies (cp.async.bulk.tensor) of the H planes into shared
// memory: Hx with the row below, Hy with the four cells to its left (a copy's
// x must start on a 16-byte boundary, so the halo is four floats wide, of
// which the kernel uses one), Hz with both.  The previous plane's Hx and Hy
// are still in shared memory for the z differences.  Three stages rotate:
// the plane below, this plane, and the next plane in flight.  E, the material
// ids and the stores are the threads' own vector accesses, as in e3d_core,
// whose arithmetic this kernel repeats term for term.  It runs only where the
// core box starts at least one cell inside the grid on every axis, so every
// neighbour it reads is a cell of the grid (no wrap, no zero fill).
constexpr int kTmaX = 128, kTmaY = 8, kTmaZ = 8;
constexpr int kTmaHx = (kTmaY + 1) * kTmaX;             // floats of one stage's Hx
constexpr int kTmaHy = kTmaY * (kTmaX + 4);
constexpr int kTmaHz = (kTmaY + 1) * (kTmaX + 4);
constexpr int kTmaHzPad = ((kTmaHz * 4 + 127) / 128) * 32;  // Hz rounded up to 128 bytes
constexpr int kTmaStage = kTmaHx + kTmaHy + kTmaHzPad;     // floats per stage
constexpr unsigned kTmaBytes = (unsigned)(kTmaHx + kTmaHy + kTmaHz) * 4u;  // bytes a stage receives
constexpr int kTmaSmem = 3 * kTmaStage * 4 + 128;           // dynamic shared bytes (+ alignment)
static_assert((kTmaHx * 4) % 128 == 0 && (kTmaHy * 4) % 128 == 0 && (kTmaStage * 4) % 128 == 0,
              "TMA destinations are 128-byte aligned");
__global__ void __launch_bounds__(32 * kTmaY) e3d_core_tma(const __grid_constant__ StepParams<float> p,
                                                           const __grid_constant__ TmaMaps m) {
  extern __shared__ unsigned char sm_raw[];
  __shared__ __align__(8) unsigned long long bar[3];
  pdl_wait();
  pdl_release();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int bx = (p.cw + 31) >> 5, by = (p.ch + kTmaY - 1) / kTmaY;
  const int tx = blockIdx.x % bx, t2 = blockIdx.x / bx, ty = t2 % by, tz = t2 / by;
  const int x0 = (p.cv0 + tx * 32) * 4, y0 = p.cy0 + ty * kTmaY;
  const int kz0 = p.cz0 + tz * kTmaZ, kz1 = min(kz0 + kTmaZ, p.cz0 + p.cd);
  const bool live = tx * 32 + lane < p.cw && ty * kTmaY + w < p.ch;
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(sm_raw);
  const uint32_t sbase = (raw + 127u) & ~127u;
  const float *gbase = (const float *)(sm_raw + (sbase - raw));
  const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(bar);
  if (threadIdx.x == 0) {
    for (int s = 0; s < 3; ++s) mbar_init(bar0 + 8 * s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // load number u (plane kz0 - 1 + u) goes to stage u % 3, whose (u / 3)-th
  // phase it completes
  auto issue = [&](int u) {
    const int s = u % 3, plane = kz0 - 1 + u;
    const uint32_t st = sbase + (uint32_t)(s * kTmaStage * 4), b = bar0 + 8 * s;
    mbar_expect_tx(b, kTmaBytes);
    tma_load_3d(st, &m.hx, x0, y0 - 1, plane, b);
    tma_load_3d(st + kTmaHx * 4, &m.hy, x0 - 4, y0, plane, b);
    tma_load_3d(st + (kTmaHx + kTmaHy) * 4, &m.hz, x0 - 4, y0 - 1, plane, b);
  };
  const int nload = kz1 - kz0 + 1;
  if (threadIdx.x == 0) {
    issue(0);
    if (nload > 1) issue(1);
  }
  int issued = nload > 1 ? 2 : 1, waited = 0;
  bool ok = __syncthreads_and(mbar_wait(bar0, 0, p.wait_limit));
  waited = ok ? 1 : 0;  // a first wait that gave up leaves load 0 to the drain below
  // this thread's E, material ids and row flag of the first plane; later
  // planes' are loaded before the barrier that ends the previous plane, so
  // their latency overlaps the wait for the H copies
  const int j = y0 + w, xr = 4 * lane;
  float ex[4] = {}, ey[4] = {}, ez[4] = {};
  uint8_t id[4] = {};
  bool skip = true;
  auto load_e = [&](int k) {
    skip = !live || __ldg(p.rowflag + (long long)k * p.ny + j);
    if (skip) return;
    const long long c = ((long long)k * p.ny + j) * p.nx + x0 + xr;
    vld<float, 4>(p.ex + c, ex);
    vld<float, 4>(p.ey + c, ey);
    vld<float, 4>(p.ez + c, ez);
    vec_ids<float, 4>(p, (long long)k * p.ny + j, (x0 + xr) / 4, p.mat + c, id);
  };
  load_e(kz0);
  for (int k = kz0; ok && k < kz1; ++k) {
    const int u = k - kz0 + 1;  // this plane's load number
    // the next plane goes into the stage the plane k - 2 held: every thread
    // finished reading it before the barrier that ended the last round
    if (threadIdx.x == 0 && u + 1 < nload) issue(u + 1);
    if (u + 1 < nload) issued = u + 2;
    ok = __syncthreads_and(mbar_wait(bar0 + 8 * (u % 3), (unsigned)(u / 3) & 1u, p.wait_limit));
    if (!ok) break;
    waited = u + 1;
    if (!skip) {
      const float *Hx = gbase + (u % 3) * kTmaStage, *Hy = Hx + kTmaHx, *Hz = Hy + kTmaHy;
      const float *Hxp = gbase + ((u + 2) % 3) * kTmaStage, *Hyp = Hxp + kTmaHx;
      const int yr = (kTmaX + 4) * w + 4 + xr, zr = (kTmaX + 4) * (w + 1) + 4 + xr;
      const float4 hx4 = *(const float4 *)(Hx + kTmaX * (w + 1) + xr);
      const float4 hxd4 = *(const float4 *)(Hx + kTmaX * w + xr);
      const float4 hxb4 = *(const float4 *)(Hxp + kTmaX * (w + 1) + xr);
      const float4 hy4 = *(const float4 *)(Hy + yr), hyb4 = *(const float4 *)(Hyp + yr);
      const float4 hz4 = *(const float4 *)(Hz + zr), hzd4 = *(const float4 *)(Hz + zr - (kTmaX + 4));
      const float hyl = Hy[yr - 1], hzl = Hz[zr - 1];
      const float hx[4] = {hx4.x, hx4.y, hx4.z, hx4.w}, hxd[4] = {hxd4.x, hxd4.y, hxd4.z, hxd4.w};
      const float hxb[4] = {hxb4.x, hxb4.y, hxb4.z, hxb4.w}, hy[4] = {hy4.x, hy4.y, hy4.z, hy4.w};
      const float hyb[4] = {hyb4.x, hyb4.y, hyb4.z, hyb4.w}, hz[4] = {hz4.x, hz4.y, hz4.z, hz4.w};
      const float hzd[4] = {hzd4.x, hzd4.y, hzd4.z, hzd4.w};
      const long long c = ((long long)k * p.ny + j) * p.nx + x0 + xr;
      bool uni = true;
#pragma unroll
      for (int q = 0; q < 4; ++q) uni &= id[q] == p.id0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float ca = uni ? p.ca0 : coef_ca3(p, id[q]);
        const float curlhzy = hz[q] - hzd[q], curlhyz = -hy[q] + hyb[q];
        const float curlhxz = hx[q] - hxb[q], curlhzx = -hz[q] + (q ? hz[q - 1] : hzl);
        const float curlhyx = hy[q] - (q ? hy[q - 1] : hyl), curlhxy = -hx[q] + hxd[q];
        ex[q] = ex[q] + ca * (curlhzy + curlhyz);
        ey[q] = ey[q] + ca * (curlhxz + curlhzx);
        ez[q] = ez[q] + ca * (curlhyx + curlhxy);
      }
      if (uni) {
        vst<float, 4>(p.ex + c, ex);
        vst<float, 4>(p.ey + c, ey);
        vst<float, 4>(p.ez + c, ez);
      } else {  // dispersive cells belong to the ADE blocks
        st_guard3<float, 4>(p.ex + c, ex, id);
        st_guard3<float, 4>(p.ey + c, ey, id);
        st_guard3<float, 4>(p.ez + c, ez, id);
      }
    }
    if (k + 1 < kz1) load_e(k + 1);
    __syncthreads();
  }
  if (!ok) {
    // a wait gave up: report it, and let the copies already issued land
    // (each wait bounded) before the block's shared memory goes away
    if (threadIdx.x == 0) atomicExch(p.err, 1);
    for (int u = waited; u < issued; ++u) mbar_wait(bar0 + 8 * (u % 3), (unsigned)(u / 3) & 1u);
  }
}

// The TMA-staged H core: the same tiles march up the core box, each plane's
// Ex (with the row above), Ey (with the cell to the right) and Ez (with both)
// copied into the 3-stage ring; the plane above is the next round's plane.
// The arithmetic is h3d_core's, term for term.  It runs only where the core
// box ends at least one cell before the far side of the grid on every axis.
__global__ void __launch_bounds__(32 * kTmaY) h3d_core_tma(const __grid_constant__ StepParams<float> p,
                                                           const __grid_constant__ TmaMaps m) {
  extern __shared__ unsigned char sm_raw[];
  __shared__ __align__(8) unsigned long long bar[3];
  pdl_wait();
  pdl_release();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int bx = (p.cw + 31) >> 5, by = (p.ch + kTmaY - 1) / kTmaY;
  const int tx = blockIdx.x % bx, t2 = blockIdx.x / bx, ty = t2 % by, tz = t2 / by;
  const int x0 = (p.cv0 + tx * 32) * 4, y0 = p.cy0 + ty * kTmaY;
  const int kz0 = p.cz0 + tz * kTmaZ, kz1 = min(kz0 + kTmaZ, p.cz0 + p.cd);
  const bool live = tx * 32 + lane < p.cw && ty * kTmaY + w < p.ch;
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(sm_raw);
  const uint32_t sbase = (raw + 127u) & ~127u;
  const float *gbase = (const float *)(sm_raw + (sbase - raw));
  const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(bar);
  if (threadIdx.x == 0) {
    for (int s = 0; s < 3; ++s) mbar_init(bar0 + 8 * s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // load number u is plane kz0 + u, in stage u % 3 (phase u / 3)
  auto issue = [&](int u) {
    const int s = u % 3, plane = kz0 + u;
    const uint32_t st = sbase + (uint32_t)(s * kTmaStage * 4), b = bar0 + 8 * s;
    mbar_expect_tx(b, kTmaBytes);
    tma_load_3d(st, &m.ex, x0, y0, plane, b);
    tma_load_3d(st + kTmaHx * 4, &m.ey, x0, y0, plane, b);
    tma_load_3d(st + (kTmaHx + kTmaHy) * 4, &m.ez, x0, y0, plane, b);
  };
  const int nload = kz1 - kz0 + 1;  // the planes kz0 .. kz1 (the last one only as the plane above)
  if (threadIdx.x == 0) {
    issue(0);
    issue(1);
  }
  int issued = 2, waited = 0;
  bool ok = __syncthreads_and(mbar_wait(bar0, 0, p.wait_limit));
  waited = ok ? 1 : 0;  // a first wait that gave up leaves load 0 to the drain below
  const int j = y0 + w, xr = 4 * lane;
  float hx[4] = {}, hy[4] = {}, hz[4] = {};
  bool skip = true;
  auto load_h = [&](int k) {
    skip = !live || __ldg(p.rowflag + (long long)k * p.ny + j);
    if (skip) return;
    const long long c = ((long long)k * p.ny + j) * p.nx + x0 + xr;
    vld<float, 4>(p.hx + c, hx);
    vld<float, 4>(p.hy + c, hy);
    vld<float, 4>(p.hz + c, hz);
  };
  load_h(kz0);
  for (int k = kz0; ok && k < kz1; ++k) {
    const int u = k - kz0;  // this plane's load number; u + 1 is the plane above
    if (threadIdx.x == 0 && u + 2 < nload) issue(u + 2);  // into the stage of plane k - 1
    if (u + 2 < nload) issued = u + 3;
    ok = __syncthreads_and(mbar_wait(bar0 + 8 * ((u + 1) % 3), (unsigned)((u + 1) / 3) & 1u, p.wait_limit));
    if (!ok) break;
    waited = u + 2;
    if (!skip) {
      const float *Ex = gbase + (u % 3) * kTmaStage, *Ey = Ex + kTmaHx, *Ez = Ey + kTmaHy;
      const float *Exa = gbase + ((u + 1) % 3) * kTmaStage, *Eya = Exa + kTmaHx;
      const int yr = (kTmaX + 4) * w + xr, zr = (kTmaX + 4) * w + xr;
      const float4 ex4 = *(const float4 *)(Ex + kTmaX * w + xr), exu4 = *(const float4 *)(Ex + kTmaX * (w + 1) + xr);
      const float4 exa4 = *(const float4 *)(Exa + kTmaX * w + xr);
      const float4 ey4 = *(const float4 *)(Ey + yr), eya4 = *(const float4 *)(Eya + yr);
      const float4 ez4 = *(const float4 *)(Ez + zr), ezu4 = *(const float4 *)(Ez + zr + (kTmaX + 4));
      const float eyr = Ey[yr + 4], ezr = Ez[zr + 4];
      const float ex[4] = {ex4.x, ex4.y, ex4.z, ex4.w}, exu[4] = {exu4.x, exu4.y, exu4.z, exu4.w};
      const float exa[4] = {exa4.x, exa4.y, exa4.z, exa4.w}, ey[4] = {ey4.x, ey4.y, ey4.z, ey4.w};
      const float eya[4] = {eya4.x, eya4.y, eya4.z, eya4.w}, ez[4] = {ez4.x, ez4.y, ez4.z, ez4.w};
      const float ezu[4] = {ezu4.x, ezu4.y, ezu4.z, ezu4.w};
      const long long c = ((long long)k * p.ny + j) * p.nx + x0 + xr;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float rz = q < 3 ? ez[q + 1] : ezr, ry = q < 3 ? ey[q + 1] : eyr;
        const float curleyz = eya[q] - ey[q], curlezy = -ezu[q] + ez[q];
        const float curlezx = rz - ez[q], curlexz = -exa[q] + ex[q];
        const float curlexy = exu[q] - ex[q], curleyx = -ry + ey[q];
        hx[q] = hx[q] + p.ku * (curleyz + curlezy);
        hy[q] = hy[q] + p.ku * (curlezx + curlexz);
        hz[q] = hz[q] + p.ku * (curlexy + curleyx);
      }
      vst<float, 4>(p.hx + c, hx);
      vst<float, 4>(p.hy + c, hy);
      vst<float, 4>(p.hz + c, hz);
    }
    if (k + 1 < kz1) load_h(k + 1);
    __syncthreads();
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(p.err, 1);
    for (int u = waited; u < issued; ++u) mbar_wait(bar0 + 8 * (u % 3), (unsigned)(u / 3) & 1u);
  }
}

constexpr int kCoreZ = 8;  // planes per thread of the z-marching kernels

template <typename T, int V, int RY>
void launch_core3z(const StepParams<T> &p, bool e_half, cudaStream_t s, cudaEvent_t ev) {
  const int blocks = ((p.cw + 31) / 32) * ((p.ch + RY - 1) / RY) * ((p.cd + kCoreZ - 1) / kCoreZ);
  if (e_half) launch_pdl(e3d_corez<T, V, RY, kCoreZ>, blocks, 32 * RY, s, p, ev);
  else launch_pdl(h3d_corez<T, V, RY, kCoreZ>, blocks, 32 * RY, s, p, ev);
}

template <typename T, int V, int RY>
void launch_core3(const StepParams<T> &p, bool e_half, cudaStream_t s, cudaEvent_t ev) {
  const int blocks = ((p.cw + 31) / 32) * ((p.ch + RY - 1) / RY) * p.cd;
  if (e_half) launch_pdl(e3d_core<T, V, RY>, blocks, 32 * RY, s, p, ev);
  else launch_pdl(h3d_core<T, V, RY>, blocks, 32 * RY, s, p, ev);
}

// the TMA-staged E core: one block per tile of kTmaX x kTmaY cells and
// kTmaZ planes, kTmaSmem bytes of dynamic shared memory
inline void launch_core3_tma(const StepParams<float> &p, bool e_half, cudaStream_t s, cudaEvent_t ev) {
  const int blocks = ((p.cw + 31) / 32) * ((p.ch + kTmaY - 1) / kTmaY) * ((p.cd + kTmaZ - 1) / kTmaZ);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(32 * kTmaY);
  cfg.dynamicSmemBytes = kTmaSmem;
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  int na = 1;
  if (ev) {
    at[1].id = cudaLaunchAttributeProgrammaticEvent;
    at[1].val.programmaticEvent.event = ev;
    at[1].val.programmaticEvent.flags = 0;
    at[1].val.programmaticEvent.triggerAtBlockStart = 1;
    na = 2;
  }
  cfg.attrs = at;
  cfg.numAttrs = na;
  cudaLaunchKernelEx(&cfg, e_half ? e3d_core_tma : h3d_core_tma, p, *p.tma);
}

// tile 0: 4 rows of 32 x-vectors, 1: 8 rows, 2: 16 rows, one plane per
// thread; tiles 3, 4, 5: the same shapes marching kCoreZ planes per thread;
// tile 6 (FP32 with 4-cell vectors, where the host set up the tensor maps):
// the TMA-staged E core, with tile 1's H core; tile 7: both TMA-staged cores
template <typename T, int V>
void launch_core3_v(const StepParams<T> &p, bool e_half, cudaStream_t s, cudaEvent_t ev) {
  if constexpr (sizeof(T) == 4 && V == 4) {
    if ((p.tile == 6 || p.tile == 7) && p.tma) {
      if (e_half || (p.tile == 7 && p.tma->h_ok)) launch_core3_tma(p, e_half, s, ev);
      else launch_core3<T, V, 8>(p, false, s, ev);
      return;
    }
  }
  switch (p.tile) {
    case 0: launch_core3<T, V, 4>(p, e_half, s, ev); break;
    case 2: launch_core3<T, V, 16>(p, e_half, s, ev); break;
    case 3: launch_core3z<T, V, 4>(p, e_half, s, ev); break;
    case 4: launch_core3z<T, V, 8>(p, e_half, s, ev); break;
    case 5: launch_core3z<T, V, 16>(p, e_half, s, ev); break;
    default: launch_core3<T, V, 8>(p, e_half, s, ev); break;
  }
}

template <typename T>
void launch_core3_tiled(const StepParams<T> &p, bool e_half, cudaStream_t s, cudaEvent_t ev) {
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  if (p.vec == VW) launch_core3_v<T, VW>(p, e_half, s, ev);
  else launch_core3_v<T, 1>(p, e_half, s, ev);
}

// `prog_event`: the core kernel's programmatic event (see launch_pdl), or
// null; the general kernel launches with the device's top priority
template <typename T>
int launch_e3d(const StepParams<T> &p, int part, void *stream, void *prog_event) {
  cudaStream_t s = (cudaStream_t)stream;
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  if (part == K2D_CORE) {
    if (p.ncore <= 0) return 0;
    launch_core3_tiled<T>(p, true, s, (cudaEvent_t)prog_event);
    return 1;
  }
  const int blocks = p.ntile_blocks + p.nslab_blocks + p.nade_blocks;
  if (blocks <= 0) return 0;
  if (p.vec == VW) launch_side(e3d_kernel<T, VW>, blocks, 256, s, p);
  else launch_side(e3d_kernel<T, 1>, blocks, 256, s, p);
  return 1;
}
template <typename T>
int launch_h3d(const StepParams<T> &p, int part, void *stream, void *prog_event) {
  cudaStream_t s = (cudaStream_t)stream;
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  if (part == K2D_CORE) {
    if (p.ncore <= 0) return 0;
    launch_core3_tiled<T>(p, false, s, (cudaEvent_t)prog_event);
    return 1;
  }
  const int blocks = p.ntile_blocks + p.nslab_blocks;
  if (blocks <= 0) return 0;
  if (p.vec == VW) launch_side(h3d_kernel<T, VW>, blocks, 256, s, p);
  else launch_side(h3d_kernel<T, 1>, blocks, 256, s, p);
  return 1;
}

template <typename T>
int launch_e3d_general_pdl(const StepParams<T> &p, void *stream) {
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  const int blocks = p.ntile_blocks + p.nslab_blocks + p.nade_blocks;
  if (blocks <= 0) return 0;
  if (p.vec == VW) launch_pdl(e3d_kernel<T, VW>, blocks, 256, (cudaStream_t)stream, p);
  else launch_pdl(e3d_kernel<T, 1>, blocks, 256, (cudaStream_t)stream, p);
  return 1;
}
template <typename T>
int launch_h3d_general_pdl(const StepParams<T> &p, void *stream) {
  constexpr int VW = sizeof(T) == 4 ? 4 : 2;
  const int blocks = p.ntile_blocks + p.nslab_blocks;
  if (blocks <= 0) return 0;
  if (p.vec == VW) launch_pdl(h3d_kernel<T, VW>, blocks, 256, (cudaStream_t)stream, p);
  else launch_pdl(h3d_kernel<T, 1>, blocks, 256, (cudaStream_t)stream, p);
  return 1;
}
template int launch_e3d_general_pdl<float>(const StepParams<float> &, void *);
template int launch_e3d_general_pdl<double>(const StepParams<double> &, void *);
template int launch_h3d_general_pdl<float>(const StepParams<float> &, void *);
template int launch_h3d_general_pdl<double>(const StepParams<double> &, void *);

template int launch_e3d<float>(const StepParams<float> &, int, void *, void *);
template int launch_e3d<double>(const StepParams<double> &, int, void *, void *);
template int launch_h3d<float>(const StepParams<float> &, int, void *, void *);
template int launch_h3d<double>(const StepParams<double> &, int, void *, void *);

}  // namespace fdtd
