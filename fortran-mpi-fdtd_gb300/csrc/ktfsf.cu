// ktfsf.cu -- total-field/scattered-field box of a 2D/3D job: a plane wave
// along +y, carried by an auxiliary line, enters through the faces of a box.
//
// One launch per half step, after the half step's other kernels:
//   block 0      the incident line.  E half: e(j) += cb s (h(j) - h(j-1)),
//                j = 1..ny-2, then the line's sources, then the two-step
//                absorbing ends e(0) = e(1) two steps ago, e(ny-1) = e(ny-2)
//                two steps ago (3D/.../include/myTFSF_incEzHx_3Dfunc.f90:
//                90-113).  H half: h(j) += Ku s (e(j+1) - e(j)), j = 0..ny-2
//                (:80-88).  s = -1 for Ez/Hx (3D, 2D TM), +1 for Ex/Hz (TE).
//   blocks 1..   the face terms: each update whose stencil crosses a face
//                gets the incident value of the neighbour on the other side
//                (consistCond_dz/dy/hx/hy, :117-221; for TE the same terms
//                of the TE grid's Ex, Ey and Hz updates).  An E term is a D
//                increment, so it enters E with the cell's 1/eps.
// Block 0 writes only the line component of its half; the face blocks read
// only the other one, so the blocks of a launch never race.  Host-side
// checks at commit keep every face cell inside the grid, in the main range,
// outside the PML and off dispersive cells; the box spans at least two rows.
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {

constexpr int kTfsfThreads = 256;

template <typename T>
struct TfsfFaces {
  // numbers of face cells: set A (faces normal to y), set B (faces normal
  // to x or z), for the E and the H half
  static __host__ __device__ void counts(const StepParams<T> &p, bool e_half, long long &na, long long &nb) {
    const long long wx = p.tf_hi[0] - p.tf_lo[0] + 1, wy = p.tf_hi[1] - p.tf_lo[1] + 1;
    const long long wz = p.layout == FDTD_LAYOUT_3D ? p.tf_hi[2] - p.tf_lo[2] + 1 : 1;
    const bool te = p.layout == FDTD_LAYOUT_2D_TE;
    if (te) {
      na = 2 * wx;
      nb = e_half && p.tf_face[0] ? 2 * (wy - 1) : 0;
    } else {
      na = 2 * wx * wz;
      if (e_half) nb = p.layout == FDTD_LAYOUT_3D && p.tf_face[2] ? 2 * wx * (wy - 1) : 0;
      else nb = p.tf_face[0] ? 2 * wy * wz : 0;
    }
  }
};

template <typename T>
__device__ __forceinline__ long long cidx(const StepParams<T> &p, int i, int j, int k) {
  return (long long)i + (long long)p.nx * ((long long)j + (long long)p.ny * k);
}

// E += (1/eps) * d on a non-dispersive cell
template <typename T>
__device__ __forceinline__ void add_e(const StepParams<T> &p, T *f, long long c, T d) {
  f[c] += p.mcs[p.mat[c]] * d;
}

template <typename T>
__global__ void __launch_bounds__(kTfsfThreads) tfsf_kernel(const __grid_constant__ StepParams<T> p, int e_half) {
  const T ku = p.ku;
  T *le = p.tf_e, *lh = p.tf_h;
  const int ny = p.ny;
  if (blockIdx.x == 0) {
    if (e_half) {
      for (int j = 1 + threadIdx.x; j <= ny - 2; j += blockDim.x) le[j] += p.tf_cb * (p.tf_sign * (lh[j] - lh[j - 1]));
      __syncthreads();
      if (threadIdx.x == 0) {
        const int n = step_n(p);
        for (int q = 0; q < p.nsrc; ++q) {
          const Source &s = p.src[q];
          if (s.comp != FDTD_E_INC) continue;
          const T g = T(p.srcval_tab[(long long)(n - 1) * p.nsrc + q]);
          for (int j = s.lo[1]; j <= s.hi[1]; ++j) le[j] += g;
        }
        T *abc = p.tf_abc;
        le[0] = abc[1];
        abc[1] = abc[0];
        abc[0] = le[1];
        le[ny - 1] = abc[3];
        abc[3] = abc[2];
        abc[2] = le[ny - 2];
      }
    } else {
      for (int j = threadIdx.x; j <= ny - 2; j += blockDim.x) lh[j] += ku * (p.tf_sign * (le[j + 1] - le[j]));
    }
    return;
  }
  long long na, nb;
  TfsfFaces<T>::counts(p, e_half != 0, na, nb);
  long long u = (long long)(blockIdx.x - 1) * blockDim.x + threadIdx.x;
  const int lo0 = p.tf_lo[0], hi0 = p.tf_hi[0], lo1 = p.tf_lo[1], hi1 = p.tf_hi[1];
  const int lo2 = p.layout == FDTD_LAYOUT_3D ? p.tf_lo[2] : 0, hi2 = p.layout == FDTD_LAYOUT_3D ? p.tf_hi[2] : 0;
  const int wx = hi0 - lo0 + 1, wy = hi1 - lo1 + 1, wz = hi2 - lo2 + 1;
  const bool te = p.layout == FDTD_LAYOUT_2D_TE;
  if (u < na) {  // faces normal to y
    const long long half = na / 2;
    const int side = u >= half;
    const long long r = side ? u - half : u;
    const int i = lo0 + (int)(r % wx), k = lo2 + (int)(r / wx);
    if (e_half) {
      const int j = side ? hi1 : lo1;
      if (te) add_e(p, p.ex, cidx(p, i, j, k), side ? ku * lh[hi1] : -(ku * lh[lo1 - 1]));
      else add_e(p, p.ez, cidx(p, i, j, k), side ? -(ku * lh[hi1]) : ku * lh[lo1 - 1]);
    } else {
      const int j = side ? hi1 : lo1 - 1;
      const long long c = cidx(p, i, j, k);
      if (te) p.hz[c] += side ? ku * le[hi1] : -(ku * le[lo1]);
      else p.hx[c] += side ? -(ku * le[hi1]) : ku * le[lo1];
    }
    return;
  }
  u -= na;
  if (u >= nb) return;
  const long long half = nb / 2;
  const int side = u >= half;
  const long long r = side ? u - half : u;
  if (e_half) {
    if (te) {  // Ey at the x faces, rows lo1..hi1-1
      const int j = lo1 + (int)r, i = side ? hi0 + 1 : lo0;
      add_e(p, p.ey, cidx(p, i, j, 0), side ? -(ku * lh[j]) : ku * lh[j]);
    } else {   // 3D: Ey at the z faces, rows lo1..hi1-1
      const int i = lo0 + (int)(r % wx), j = lo1 + (int)(r / wx), k = side ? hi2 + 1 : lo2;
      add_e(p, p.ey, cidx(p, i, j, k), side ? ku * lh[j] : -(ku * lh[j]));
    }
  } else {     // Hy at the x faces
    const int j = lo1 + (int)(r % wy), k = lo2 + (int)(r / wy), i = side ? hi0 : lo0 - 1;
    p.hy[cidx(p, i, j, k)] += side ? ku * le[j] : -(ku * le[j]);
  }
  (void)wz;
}

template <typename T>
int launch_tfsf(const StepParams<T> &p, bool e_half, void *stream) {
  long long na, nb;
  TfsfFaces<T>::counts(p, e_half, na, nb);
  const long long blocks = 1 + (na + nb + kTfsfThreads - 1) / kTfsfThreads;
  tfsf_kernel<T><<<(unsigned)blocks, kTfsfThreads, 0, (cudaStream_t)stream>>>(p, e_half ? 1 : 0);
  return 1;
}

template int launch_tfsf<float>(const StepParams<float> &, bool, void *);
template int launch_tfsf<double>(const StepParams<double> &, bool, void *);

}  // namespace fdtd
