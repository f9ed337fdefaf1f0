// k2d.cu -- 2D half-step kernels (TE: Ex, Ey, Hz; TM: Ez, Hx, Hy).
//
// One launch per half step does three kinds of work, selected by blockIdx:
//   tile blocks  : 32 x 32 cells, a warp per 32-cell row segment, 4 rows per
//                  thread; the Yee update + constant-dielectric material
//                  (E += Ku/eps * curl, the reference's D update and E=D*gax
//                  folded), the split-field PML shell, the reference y-slab
//                  PML (2D/BERpmly_HzExEy_mod.f90) and the fused DFT/probe
//                  sampling.
//   ADE blocks   : one thread per dispersive cell (gold Drude+2CP,
//                  2D/gold_mod.f90:47-75), D kept as Q = D - I.
// x neighbours come from warp shuffles; rows are walked with the previous
// row's value kept in a register.
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {

template <typename T, int L>
struct K2 {
  // ---- E half step ------------------------------------------------------
  static __device__ __forceinline__ void tile_e(const StepParams<T> &p, int bx) {
    const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int tx = bx % p.tiles_x, ty = bx / p.tiles_x;
    const int i = tx * 32 + lane;
    const int j0 = ty * 32 + wy * 4;
    const int nx = p.nx, ny = p.ny;
    const bool inx = i < nx;
    if (j0 >= ny) return;  // whole warp
    // value of the component below the first row (j0-1)
    T prev = 0;
    if (L == 3) prev = inx ? ld_y(p.hx, i, j0 - 1, nx, ny, p.per[1]) : T(0);
    else prev = inx ? ld_y(p.hz, i, j0 - 1, nx, ny, p.per[1]) : T(0);
    for (int r = 0; r < 4; ++r) {
      const int j = j0 + r;
      if (j >= ny) break;
      const long long c = (long long)j * nx + i;
      if (L == 3) {
        // TM: Ez += Ku/eps * ((Hy(i)-Hy(i-1)) + (-Hx(j)+Hx(j-1)))
        T hyc = inx ? p.hy[c] : T(0);
        T hyl = shfl_left(hyc, lane);
        if (lane == 0 && inx) hyl = ld_x(p.hy, i - 1, j, nx, p.per[0]);
        T hxc = inx ? p.hx[c] : T(0);
        const T dxpart = hyc - hyl;          // curlhyx
        const T dypart = -hxc + prev;        // curlhxy
        const T curl = dxpart + dypart;
        prev = hxc;
        if (!inx) continue;
        const bool shell = p.pml_mode == 2 && in_shell2(p, i, j);
        if (shell) {
          if (p.roles & ROLE_PML) {
            // Ez = Ezx + Ezy, Ezx stored (3D/BERpmly_mod.f90:151,153 with d/dz = 0)
            const T ezx = p.sp[0][c];
            const T ezy = kTwoParts<T> ? p.sp[6][c] : p.ez[c] - ezx;
            const T nezx = p.cf1[0][i] * ezx + p.cf2[0][i] * dxpart;
            const T nezy = p.cf1[1][j] * ezy + p.cf2[1][j] * dypart;
            p.sp[0][c] = nezx;
            if (kTwoParts<T>) p.sp[6][c] = nezy;
            p.ez[c] = nezx + nezy;
          }
        } else if ((p.roles & ROLE_MAIN) && in_main2(p, i, j)) {
          const uint8_t id = p.mat[c];
          const MatCoef<T> mc = p.mc[id];
          if (mc.kind == MK_DIEL) {
            T e = p.ez[c] + mc.ca * curl;
            T s = src_sum<T>(p, 2, i, j, 0);
            if (s != T(0)) e += mc.cs * s;
            p.ez[c] = e;
          }
        }
      } else {
        // TE: Ex += Ku/eps*(Hz(j)-Hz(j-1)), Ey -= Ku/eps*(Hz(i)-Hz(i-1))
        T hzc = inx ? p.hz[c] : T(0);
        T hzl = shfl_left(hzc, lane);
        if (lane == 0 && inx) hzl = ld_x(p.hz, i - 1, j, nx, p.per[0]);
        T hzd = prev;
        prev = hzc;
        if (!inx) continue;
        const T curlhx = hzc - hzl;
        const T curlhy = hzc - hzd;
        if (p.pml_mode == 2 && in_shell2(p, i, j)) {
          if (p.roles & ROLE_PML) {
            p.ex[c] = p.cf1[1][j] * p.ex[c] + p.cf2[1][j] * curlhy;
            p.ey[c] = p.cf1[0][i] * p.ey[c] + p.cf2[0][i] * (-hzc + hzl);
          }
          continue;
        }
        if ((p.roles & ROLE_MAIN) && in_main2(p, i, j)) {
          const uint8_t id = p.mat[c];
          const MatCoef<T> mc = p.mc[id];
          if (mc.kind == MK_DIEL) {
            T ex = p.ex[c] + mc.ca * curlhy;
            T ey = p.ey[c] - mc.ca * curlhx;
            if (p.nsrc) {
              T sx = src_sum<T>(p, 0, i, j, 0), sy = src_sum<T>(p, 1, i, j, 0);
              if (sx != T(0)) ex += mc.cs * sx;
              if (sy != T(0)) ey += mc.cs * sy;
            }
            p.ex[c] = ex;
            p.ey[c] = ey;
          }
        }
        if (p.pml_mode == 1 && (p.roles & ROLE_PML)) ref_slab_e(p, i, j);
      }
    }
  }

  // reference 2D slab, E part (2D/BERpmly_HzExEy_mod.f90:96-123, 144-178)
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

  // ---- H half step ------------------------------------------------------
  static __device__ __forceinline__ void tile_h(const StepParams<T> &p, int bx) {
    const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int tx = bx % p.tiles_x, ty = bx / p.tiles_x;
    const int i = tx * 32 + lane;
    const int j0 = ty * 32 + wy * 4;
    const int nx = p.nx, ny = p.ny;
    const bool inx = i < nx;
    if (j0 >= ny) return;
    // E component with a y derivative, row j0
    T cur = 0;
    if (L == 3) cur = inx ? p.ez[(long long)j0 * nx + i] : T(0);
    else cur = inx ? p.ex[(long long)j0 * nx + i] : T(0);
    for (int r = 0; r < 4; ++r) {
      const int j = j0 + r;
      if (j >= ny) break;
      const long long c = (long long)j * nx + i;
      T up = inx ? ld_y(L == 3 ? p.ez : p.ex, i, j + 1, nx, ny, p.per[1]) : T(0);
      if (L == 3) {
        T ezc = cur;
        T ezr = shfl_right(ezc, lane);
        if ((lane == 31 || i + 1 >= nx) && inx) ezr = ld_x(p.ez, i + 1, j, nx, p.per[0]);
        cur = up;
        if (!inx) continue;
        T hx, hy;
        bool wrote = false;
        if (p.pml_mode == 2 && in_shell2(p, i, j)) {
          if (p.roles & ROLE_PML) {
            hx = p.cg1[1][j] * p.hx[c] + p.cg2[1][j] * (-up + ezc);
            hy = p.cg1[0][i] * p.hy[c] + p.cg2[0][i] * (ezr - ezc);
            p.hx[c] = hx;
            p.hy[c] = hy;
            wrote = true;
          }
        } else if ((p.roles & ROLE_MAIN) && in_main2(p, i, j)) {
          hx = p.hx[c] + p.ku * (-up + ezc);
          hy = p.hy[c] + p.ku * (ezr - ezc);
          p.hx[c] = hx;
          p.hy[c] = hy;
          wrote = true;
        }
        if (p.gather) {
          if (!wrote) { hx = p.hx[c]; hy = p.hy[c]; }
          T vals[6] = {T(0), T(0), ezc, hx, hy, T(0)};
          gather_cell<T>(p, i, j, 0, vals);
        }
      } else {
        T exc = cur;
        T eyc = inx ? p.ey[c] : T(0);
        T eyr = shfl_right(eyc, lane);
        if ((lane == 31 || i + 1 >= nx) && inx) eyr = ld_x(p.ey, i + 1, j, nx, p.per[0]);
        cur = up;
        if (!inx) continue;
        T hz = 0;
        bool wrote = false;
        if (p.pml_mode == 2 && in_shell2(p, i, j)) {
          if (p.roles & ROLE_PML) {
            T hzx = p.sp[0][c];
            T hzy = kTwoParts<T> ? p.sp[6][c] : p.hz[c] - hzx;
            hzy = p.cg1[1][j] * hzy + p.cg2[1][j] * (up - exc);
            hzx = p.cg1[0][i] * hzx + p.cg2[0][i] * (-eyr + eyc);
            p.sp[0][c] = hzx;
            if (kTwoParts<T>) p.sp[6][c] = hzy;
            hz = hzy + hzx;
            p.hz[c] = hz;
            wrote = true;
          }
        } else {
          if ((p.roles & ROLE_MAIN) && in_main2(p, i, j)) {
            T curlE = ((eyr - eyc) - up) + exc;
            hz = p.hz[c] - p.ku * curlE;
            p.hz[c] = hz;
            wrote = true;
          }
          if (p.pml_mode == 1 && (p.roles & ROLE_PML)) {
            T v;
            if (ref_slab_h(p, i, j, &v)) { hz = v; wrote = true; }
          }
        }
        if (p.gather) {
          if (!wrote) hz = p.hz[c];
          T vals[6] = {exc, eyc, T(0), T(0), T(0), hz};
          gather_cell<T>(p, i, j, 0, vals);
        }
      }
    }
  }

  // reference 2D slab, H part (updateHs :125-140, setboundayHya/b :156-190);
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

  // ---- dispersive cells ---------------------------------------------------
  static __device__ __forceinline__ void ade_e(const StepParams<T> &p, int s) {
    const int cell = p.ade_cell[s];
    const int nx = p.nx, ny = p.ny;
    const int i = cell % nx, j = cell / nx;
    const MatCoef<T> mc = p.mc[p.ade_mat[s]];
    const AdeCoef<T> &a = p.ac[mc.ade];
    if (L == 3) {
      T curl = (p.hy[cell] - ld_x(p.hy, i - 1, j, nx, p.per[0])) +
               (-p.hx[cell] + ld_y(p.hx, i, j - 1, nx, ny, p.per[1]));
      T inc = p.ku * curl + src_sum<T>(p, 2, i, j, 0);
      p.ez[cell] = ade_update<T>(p, a, s, 0, inc, p.ez[cell]);
    } else {
      T hzc = p.hz[cell];
      T curlhx = hzc - ld_x(p.hz, i - 1, j, nx, p.per[0]);
      T curlhy = hzc - ld_y(p.hz, i, j - 1, nx, ny, p.per[1]);
      T incx = p.ku * curlhy + src_sum<T>(p, 0, i, j, 0);
      T incy = -(p.ku * curlhx) + src_sum<T>(p, 1, i, j, 0);
      p.ex[cell] = ade_update<T>(p, a, s, 0, incx, p.ex[cell]);
      p.ey[cell] = ade_update<T>(p, a, s, 1, incy, p.ey[cell]);
    }
  }
};

template <typename T, int L>
__global__ void __launch_bounds__(256) e2d_kernel(const __grid_constant__ StepParams<T> p) {
  int b = blockIdx.x;
  if (b < p.ntile_blocks) {
    if (p.roles & (ROLE_MAIN | ROLE_PML)) K2<T, L>::tile_e(p, b);
    return;
  }
  b -= p.ntile_blocks;
  if (p.roles & ROLE_ADE) {
    int s = b * 256 + threadIdx.x;
    if (s < p.nade) K2<T, L>::ade_e(p, s);
  }
}

template <typename T, int L>
__global__ void __launch_bounds__(256) h2d_kernel(const __grid_constant__ StepParams<T> p) {
  if ((int)blockIdx.x < p.ntile_blocks) K2<T, L>::tile_h(p, blockIdx.x);
}

template <typename T>
void launch_e2d(const StepParams<T> &p, int blocks, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (p.layout == 3) e2d_kernel<T, 3><<<blocks, 256, 0, s>>>(p);
  else e2d_kernel<T, 2><<<blocks, 256, 0, s>>>(p);
}

template <typename T>
void launch_h2d(const StepParams<T> &p, int blocks, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (p.layout == 3) h2d_kernel<T, 3><<<blocks, 256, 0, s>>>(p);
  else h2d_kernel<T, 2><<<blocks, 256, 0, s>>>(p);
}

template void launch_e2d<float>(const StepParams<float> &, int, void *);
template void launch_e2d<double>(const StepParams<double> &, int, void *);
template void launch_h2d<float>(const StepParams<float> &, int, void *);
template void launch_h2d<double>(const StepParams<double> &, int, void *);

}  // namespace fdtd
