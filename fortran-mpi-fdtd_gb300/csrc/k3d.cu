// k3d.cu -- 3D half-step kernels (3D/.../include/myfdtd_func.f90:19-64).
//
// One launch per half step; blockIdx selects the work:
//   tile blocks : 32 (x) x 8 (y) threads, each marching kKZ cells along z
//                 with the previous (E) or next (H) plane kept in registers;
//                 x neighbours by warp shuffle.  Main cells do the Yee
//                 update with the constant-dielectric material folded in;
//                 shell cells of the split-field PML do the split update.
//   slab blocks : the reference's y-slab PML (3D/BERpmly_mod.f90:72-306),
//                 one thread per slab cell and side, 12 split arrays, the
//                 coupling rows read straight from the main arrays.
//   ADE blocks  : one thread per dispersive cell (3D/gold_mod.f90:50-88).
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {

constexpr int kKZ = 16;

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

template <typename T>
__device__ __forceinline__ void tile_e3(const StepParams<T> &p, int b, int n) {
  const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
  const int tx = b % p.tiles_x, t2 = b / p.tiles_x;
  const int ty = t2 % p.tiles_y, tz = t2 / p.tiles_y;
  const int i = tx * 32 + lane, j = ty * 8 + wy, k0 = tz * kKZ;
  if (j >= p.ny || k0 >= p.nz) return;
  const bool inx = i < p.nx;
  F3<T> f(p);
  T hx_km = inx ? f.lz(p.hx, i, j, k0 - 1) : T(0);
  T hy_km = inx ? f.lz(p.hy, i, j, k0 - 1) : T(0);
  const int k1 = min(k0 + kKZ, p.nz);
  for (int k = k0; k < k1; ++k) {
    const long long c = f.ix(i, j, k);
    const T hxc = inx ? p.hx[c] : T(0);
    const T hyc = inx ? p.hy[c] : T(0);
    const T hzc = inx ? p.hz[c] : T(0);
    T hzl = shfl_left(hzc, lane), hyl = shfl_left(hyc, lane);
    if (lane == 0 && inx) { hzl = f.lx(p.hz, i - 1, j, k); hyl = f.lx(p.hy, i - 1, j, k); }
    const T hxkm = hx_km, hykm = hy_km;
    hx_km = hxc;
    hy_km = hyc;
    if (!inx) continue;
    const T hzd = f.ly(p.hz, i, j - 1, k), hxd = f.ly(p.hx, i, j - 1, k);
    const T curlhzy = hzc - hzd, curlhyz = -hyc + hykm;
    const T curlhxz = hxc - hxkm, curlhzx = -hzc + hzl;
    const T curlhyx = hyc - hyl, curlhxy = -hxc + hxd;
    if (p.pml_mode == 2 && in_shell3(p, i, j, k)) {
      if (p.roles & ROLE_PML) {
        const T f1x = p.cf1[0][i], f2x = p.cf2[0][i], f1y = p.cf1[1][j], f2y = p.cf2[1][j];
        const T f1z = p.cf1[2][k], f2z = p.cf2[2][k];
        T exy = p.sp[0][c], eyz = p.sp[1][c], ezx = p.sp[2][c];
        T exz, eyx, ezy;
        if (kTwoParts<T>) { exz = p.sp[6][c]; eyx = p.sp[7][c]; ezy = p.sp[8][c]; }
        else { exz = p.ex[c] - exy; eyx = p.ey[c] - eyz; ezy = p.ez[c] - ezx; }
        exy = f1y * exy + f2y * curlhzy;
        exz = f1z * exz + f2z * curlhyz;
        eyz = f1z * eyz + f2z * curlhxz;
        eyx = f1x * eyx + f2x * curlhzx;
        ezx = f1x * ezx + f2x * curlhyx;
        ezy = f1y * ezy + f2y * curlhxy;
        p.sp[0][c] = exy; p.sp[1][c] = eyz; p.sp[2][c] = ezx;
        if (kTwoParts<T>) { p.sp[6][c] = exz; p.sp[7][c] = eyx; p.sp[8][c] = ezy; }
        p.ex[c] = exy + exz; p.ey[c] = eyz + eyx; p.ez[c] = ezx + ezy;
      }
      continue;
    }
    if ((p.roles & ROLE_MAIN) && in_main3(p, i, j, k)) {
      const MatCoef<T> mc = p.mc[p.mat[c]];
      if (mc.kind == MK_DIEL) {
        T ex = p.ex[c] + mc.ca * (curlhzy + curlhyz);
        T ey = p.ey[c] + mc.ca * (curlhxz + curlhzx);
        T ez = p.ez[c] + mc.ca * (curlhyx + curlhxy);
        if (p.nsrc) {
          const T sx = src_sum<T>(p, n, 0, i, j, k), sy = src_sum<T>(p, n, 1, i, j, k), sz = src_sum<T>(p, n, 2, i, j, k);
          if (sx != T(0)) ex += mc.cs * sx;
          if (sy != T(0)) ey += mc.cs * sy;
          if (sz != T(0)) ez += mc.cs * sz;
        }
        p.ex[c] = ex; p.ey[c] = ey; p.ez[c] = ez;
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void tile_h3(const StepParams<T> &p, int b, int n) {
  const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
  const int tx = b % p.tiles_x, t2 = b / p.tiles_x;
  const int ty = t2 % p.tiles_y, tz = t2 / p.tiles_y;
  const int i = tx * 32 + lane, j = ty * 8 + wy, k0 = tz * kKZ;
  if (j >= p.ny || k0 >= p.nz) return;
  const bool inx = i < p.nx;
  F3<T> f(p);
  T exc = inx ? p.ex[f.ix(i, j, k0)] : T(0);
  T eyc = inx ? p.ey[f.ix(i, j, k0)] : T(0);
  const int k1 = min(k0 + kKZ, p.nz);
  for (int k = k0; k < k1; ++k) {
    const long long c = f.ix(i, j, k);
    const T ezc = inx ? p.ez[c] : T(0);
    T ezr = shfl_right(ezc, lane), eyr = shfl_right(eyc, lane);
    if ((lane == 31 || i + 1 >= p.nx) && inx) { ezr = f.lx(p.ez, i + 1, j, k); eyr = f.lx(p.ey, i + 1, j, k); }
    const T exkp = inx ? f.lz(p.ex, i, j, k + 1) : T(0);
    const T eykp = inx ? f.lz(p.ey, i, j, k + 1) : T(0);
    const T ex0 = exc, ey0 = eyc;
    exc = exkp;
    eyc = eykp;
    if (!inx) continue;
    const T ezu = f.ly(p.ez, i, j + 1, k), exu = f.ly(p.ex, i, j + 1, k);
    const T curleyz = eykp - ey0, curlezy = -ezu + ezc;
    const T curlezx = ezr - ezc, curlexz = -exkp + ex0;
    const T curlexy = exu - ex0, curleyx = -eyr + ey0;
    T hx, hy, hz;
    bool wrote = false;
    if (p.pml_mode == 2 && in_shell3(p, i, j, k)) {
      if (p.roles & ROLE_PML) {
        const T g1x = p.cg1[0][i], g2x = p.cg2[0][i], g1y = p.cg1[1][j], g2y = p.cg2[1][j];
        const T g1z = p.cg1[2][k], g2z = p.cg2[2][k];
        T hxy = p.sp[3][c], hyz = p.sp[4][c], hzx = p.sp[5][c];
        T hxz, hyx, hzy;
        if (kTwoParts<T>) { hxz = p.sp[9][c]; hyx = p.sp[10][c]; hzy = p.sp[11][c]; }
        else { hxz = p.hx[c] - hxy; hyx = p.hy[c] - hyz; hzy = p.hz[c] - hzx; }
        hxy = g1y * hxy + g2y * curlezy;
        hxz = g1z * hxz + g2z * curleyz;
        hyz = g1z * hyz + g2z * curlexz;
        hyx = g1x * hyx + g2x * curlezx;
        hzx = g1x * hzx + g2x * curleyx;
        hzy = g1y * hzy + g2y * curlexy;
        p.sp[3][c] = hxy; p.sp[4][c] = hyz; p.sp[5][c] = hzx;
        if (kTwoParts<T>) { p.sp[9][c] = hxz; p.sp[10][c] = hyx; p.sp[11][c] = hzy; }
        hx = hxy + hxz; hy = hyz + hyx; hz = hzx + hzy;
        p.hx[c] = hx; p.hy[c] = hy; p.hz[c] = hz;
        wrote = true;
      }
    } else if ((p.roles & ROLE_MAIN) && in_main3(p, i, j, k)) {
      hx = p.hx[c] + p.ku * (curleyz + curlezy);
      hy = p.hy[c] + p.ku * (curlezx + curlexz);
      hz = p.hz[c] + p.ku * (curlexy + curleyx);
      p.hx[c] = hx; p.hy[c] = hy; p.hz[c] = hz;
      wrote = true;
    }
    if (p.gather) {
      if (!wrote) { hx = p.hx[c]; hy = p.hy[c]; hz = p.hz[c]; }
      const T vals[6] = {ex0, ey0, ezc, hx, hy, hz};
      gather_cell<T>(p, n, i, j, k, vals);
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
  const AdeCoef<T> a = ade_coef(p, p.ade_mat[s]);
  const T hxc = p.hx[cell], hyc = p.hy[cell], hzc = p.hz[cell];
  const T curlhzy = hzc - f.ly(p.hz, i, j - 1, k), curlhyz = -hyc + f.lz(p.hy, i, j, k - 1);
  const T curlhxz = hxc - f.lz(p.hx, i, j, k - 1), curlhzx = -hzc + f.lx(p.hz, i - 1, j, k);
  const T curlhyx = hyc - f.lx(p.hy, i - 1, j, k), curlhxy = -hxc + f.ly(p.hx, i, j - 1, k);
  const T ix_ = p.ku * (curlhzy + curlhyz) + src_sum<T>(p, n, 0, i, j, k);
  const T iy_ = p.ku * (curlhxz + curlhzx) + src_sum<T>(p, n, 1, i, j, k);
  const T iz_ = p.ku * (curlhyx + curlhxy) + src_sum<T>(p, n, 2, i, j, k);
  p.ex[cell] = ade_update<T>(p, a, s, 0, ix_, p.ex[cell]);
  p.ey[cell] = ade_update<T>(p, a, s, 1, iy_, p.ey[cell]);
  p.ez[cell] = ade_update<T>(p, a, s, 2, iz_, p.ez[cell]);
}

template <typename T>
__global__ void __launch_bounds__(256) e3d_kernel(const __grid_constant__ StepParams<T> p) {
  const int n = step_n(p);
  int b = blockIdx.x;
  if (b < p.ntile_blocks) {
    if (p.roles & (ROLE_MAIN | ROLE_PML)) tile_e3<T>(p, b, n);
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

template <typename T>
__global__ void __launch_bounds__(256) h3d_kernel(const __grid_constant__ StepParams<T> p) {
  const int n = step_n(p);
  int b = blockIdx.x;
  if (b < p.ntile_blocks) {
    if (p.roles & (ROLE_MAIN | ROLE_PML)) tile_h3<T>(p, b, n);
    return;
  }
  b -= p.ntile_blocks;
  if (b < p.nslab_blocks && (p.roles & ROLE_PML)) slab_h3<T>(p, b * 256 + threadIdx.x);
}

template <typename T>
void launch_e3d(const StepParams<T> &p, int blocks, void *stream) {
  e3d_kernel<T><<<blocks, 256, 0, (cudaStream_t)stream>>>(p);
}
template <typename T>
void launch_h3d(const StepParams<T> &p, int blocks, void *stream) {
  h3d_kernel<T><<<blocks, 256, 0, (cudaStream_t)stream>>>(p);
}

template void launch_e3d<float>(const StepParams<float> &, int, void *);
template void launch_e3d<double>(const StepParams<double> &, int, void *);
template void launch_h3d<float>(const StepParams<float> &, int, void *);
template void launch_h3d<double>(const StepParams<double> &, int, void *);

}  // namespace fdtd
