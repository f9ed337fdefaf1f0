// k2f.cu -- the fused 2D step kernel (TMz, FP32): one pass over the grid that
// takes Ez, Hx and Hy from step n to n+1 (2D/.../include/myfdtd_2Dfunc.f90:
// 16-44, updateD then updateH), so that each field is read once and stored
// once per step instead of once per half step.
//
// A warp owns a strip of 31 x-vectors (124 cells) and marches kGRows rows of
// it upward.  At row j it computes Ez^{n+1} of row j+1 (one row ahead) and
// then H^{n+1} of row j, whose curl needs Ez^{n+1} of the row above and of the
// cell to the right.  Lane 31 computes Ez^{n+1} of the first vector of the
// next strip, for the cell to the right of lane 30's last cell (passed by a
// shuffle); the row above a warp's last row is computed the same way.  Those
// values belong to other warps, which compute them as well: the fields of
// step n are read from one set of buffers and those of step n+1 stored to the
// other (a ping-pong pair), so no warp can meet a value that another has
// already advanced, and every warp is independent of the others.
//
// Every cell is handled here: the split-field PML shell (its stored part Ezx
// ping-ponged too), the edges of the main range, source rows and sampled rows
// (monitor stage and probes).  Dispersive cells get their Ez^{n+1} from the
// output buffer, where e2d_ade -- launched just before this kernel, with a
// programmatic dependency -- stored it; a warp waits for that kernel only when
// it meets such a cell, so the two run side by side.  The arithmetic of every
// cell is that of the split kernels (core_e, core_h, K2::unit_e, K2::unit_h),
// term for term, so the results equal theirs bit for bit.
//
// It runs on grids without periodic axes, reference slabs, a TFSF box or mean
// monitors, with nx a multiple of 4.
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {

constexpr int kGOwn = 31;     // x-vectors a warp stores (lane 31: the neighbour's first)
constexpr int kGRows = 8;     // rows a warp marches
constexpr int kGWarps = 4;    // warps of a block: consecutive row groups of one strip
constexpr int kGThreads = 32 * kGWarps;
constexpr int kGAhead = 3;    // rows in flight beyond the row whose Ez^{n+1} is formed
constexpr int kGSlots = kGAhead + 1;
constexpr unsigned kFull = 0xffffffffu;

// A warp's rows travel through a ring of shared-memory slots, filled by
// asynchronous copies (cp.async) kGAhead rows ahead of their use, so that a
// warp keeps several rows of loads in flight without holding them in
// registers.  Each thread copies, and later reads, only its own vector.
struct RowSlot {
  float4 ez[32], hx[32], hy[32], ezx[32];
  unsigned id[32];
  float hyl, pad[3];
};
struct WarpRing {
  RowSlot s[kGSlots];
  float4 below[32];  // Hx of the row below the warp's first row
};

__device__ __forceinline__ void cp16(void *dst, const void *src, bool in) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(__cvta_generic_to_global(src)),
               "r"(in ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp4(void *dst, const void *src, bool in) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(__cvta_generic_to_global(src)),
               "r"(in ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// every group but the newest kGAhead - 1 has landed
__device__ __forceinline__ void cp_wait_ahead() { asm volatile("cp.async.wait_group %0;" ::"n"(kGAhead - 1) : "memory"); }

// one row of a thread's x-vector at step n, as loaded
struct Row2 {
  float ez[4], hx[4], hy[4];
  float ezx[4];   // the stored PML part Ezx (shell vectors)
  float hyl;      // lane 0: Hy of the cell left of the vector
  unsigned id;    // material ids, byte q for cell q
  int rf;         // row flags
  bool in;        // the vector lies in the grid
  bool shell;     // some cell of the vector lies in the split-PML shell
};

__device__ __forceinline__ int id_of(unsigned ids, int q) { return (ids >> (8 * q)) & 0xffu; }

__device__ __forceinline__ bool row_in(const StepParams<float> &p, int j, int i0) { return j < p.ny && i0 < p.nx; }
__device__ __forceinline__ bool vec_shell(const StepParams<float> &p, int j, int i0) {
  return p.pml_mode == 2 && (i0 < p.slo[0] || i0 + 3 > p.shi[0] || j < p.slo[1] || j > p.shi[1]);
}

// queue the copies of row j of the thread's vector into a ring slot (zeros
// for a vector outside the grid)
__device__ __forceinline__ void issue_row(const StepParams<float> &p, RowSlot &sl, int j, int i0, int lane) {
  const bool in = row_in(p, j, i0);
  const long long c = in ? (long long)j * p.nx + i0 : 0;
  cp16(&sl.ez[lane], p.ez + c, in);
  cp16(&sl.hx[lane], p.hx + c, in);
  cp16(&sl.hy[lane], p.hy + c, in);
  cp4(&sl.id[lane], p.mat + c, in);
  const bool sh = in && vec_shell(p, j, i0);
  if (p.pml_mode == 2) cp16(&sl.ezx[lane], sh ? p.sp[0] + c : p.ez, sh);
  if (lane == 0) cp4(&sl.hyl, in && i0 > 0 ? p.hy + c - 1 : p.hy, in && i0 > 0);
}

// row j of the thread's vector from its ring slot, once its copies landed
__device__ __forceinline__ void read_row(const StepParams<float> &p, const RowSlot &sl, int j, int i0, int lane,
                                         Row2 &r) {
  const float4 ez = sl.ez[lane], hx = sl.hx[lane], hy = sl.hy[lane];
  r.ez[0] = ez.x; r.ez[1] = ez.y; r.ez[2] = ez.z; r.ez[3] = ez.w;
  r.hx[0] = hx.x; r.hx[1] = hx.y; r.hx[2] = hx.z; r.hx[3] = hx.w;
  r.hy[0] = hy.x; r.hy[1] = hy.y; r.hy[2] = hy.z; r.hy[3] = hy.w;
  r.in = row_in(p, j, i0);
  r.shell = r.in && vec_shell(p, j, i0);
  if (r.shell) {
    const float4 x = sl.ezx[lane];
    r.ezx[0] = x.x; r.ezx[1] = x.y; r.ezx[2] = x.z; r.ezx[3] = x.w;
  } else {
    r.ezx[0] = r.ezx[1] = r.ezx[2] = r.ezx[3] = 0.f;
  }
  r.id = sl.id[lane];
  r.hyl = lane == 0 ? sl.hyl : 0.f;
  r.rf = r.in ? __ldg(p.rowflag + j) : 0;
}

// e plus the cell's source terms
__device__ __forceinline__ float src_add(const StepParams<float> &p, int n, int i, int j, int id, float e) {
  const float sv = src_sum<float>(p, n, 2, i, j, 0);
  if (sv != 0.f) e += __ldg(p.mcs + id) * sv;
  return e;
}

// Ez^{n+1} of row j of the vector (e), and the new stored part Ezx of a shell
// vector (ezx; the part as read for cells outside the shell).  below: Hx^n of
// row j-1.  Every lane of the warp calls it (it shuffles).
__device__ __forceinline__ void ez_new(const StepParams<float> &p, const Row2 &r, const float (&below)[4], int j,
                                       int i0, int lane, int n, float (&e)[4], float (&ezx)[4]) {
  float hl = __shfl_up_sync(kFull, r.hy[3], 1);
  if (lane == 0) hl = r.hyl;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    e[q] = r.ez[q];
    ezx[q] = r.ezx[q];
  }
  bool ade = false;
  if (r.in) {
    // TM: Ez += Ku/eps ((Hy(i)-Hy(i-1)) + (-Hx(j)+Hx(j-1)))
    float dxp[4], dyp[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      dxp[q] = r.hy[q] - (q ? r.hy[q - 1] : hl);  // curlhyx
      dyp[q] = -r.hx[q] + below[q];               // curlhxy
      ade |= id_of(r.id, q) >= kAdeId;
    }
    const bool main_y = j >= p.mlo[1] && j <= p.mhi[1];
    const bool main_x = i0 >= p.mlo[0] && i0 + 3 <= p.mhi[0];
    if (!r.shell && main_x && main_y && !(r.rf & ROW_SRC)) {
      const unsigned id0x4 = (unsigned)p.id0 * 0x01010101u;
      if (r.id == id0x4) {
#pragma unroll
        for (int q = 0; q < 4; ++q) e[q] = e[q] + p.ca0 * (dxp[q] + dyp[q]);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int id = id_of(r.id, q);
          const float ca = id == p.id0 ? p.ca0 : __ldg(p.mca + id);
          e[q] = e[q] + ca * (dxp[q] + dyp[q]);
        }
      }
    } else {
      // the general cell (split-PML shell, source row, edge of the main range)
      const bool shell_y = j < p.slo[1] || j > p.shi[1];
      float f1x[4] = {}, f2x[4] = {}, f1y = 0.f, f2y = 0.f;
      if (r.shell) {
        vld_ro<float, 4>(p.cf1[0] + i0, f1x);
        vld_ro<float, 4>(p.cf2[0] + i0, f2x);
        f1y = __ldg(p.cf1[1] + j);
        f2y = __ldg(p.cf2[1] + j);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = i0 + q;
        if (r.shell && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
          // Ez = Ezx + Ezy (3D/BERpmly_mod.f90:151,153 with d/dz = 0)
          const float py = e[q] - ezx[q];
          const float nezx = lin2(f1x[q], ezx[q], f2x[q], dxp[q]);
          const float nezy = lin2(f1y, py, f2y, dyp[q]);
          ezx[q] = nezx;
          e[q] = nezx + nezy;
        } else if (main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
          const int id = id_of(r.id, q);
          const float ca = id == p.id0 ? p.ca0 : __ldg(p.mca + id);
          e[q] = e[q] + ca * (dxp[q] + dyp[q]);
          if (r.rf & ROW_SRC) e[q] = src_add(p, n, i, j, id, e[q]);
        }
      }
    }
  }
  // dispersive cells: the value e2d_ade stored, once that kernel is complete
  if (__any_sync(kFull, ade)) {
    pdl_wait();
    if (ade) {
      const float *eo = p.ezo + (long long)j * p.nx + i0;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (id_of(r.id, q) >= kAdeId) e[q] = eo[q];
    }
  }
}

// the samples of a vector of a sampled row
__device__ __forceinline__ void gather_row4(const StepParams<float> &p, int n, int i0, int j, float4 ez, float4 hx,
                                         float4 hy) {
  const float e[4] = {ez.x, ez.y, ez.z, ez.w}, a[4] = {hx.x, hx.y, hx.z, hx.w}, b[4] = {hy.x, hy.y, hy.z, hy.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float vals[6] = {0.f, 0.f, e[q], a[q], b[q], 0.f};
    gather_cell<float>(p, n, i0 + q, j, 0, vals);
  }
}

// H^{n+1} of row j from the row's step-n values (r), Ez^{n+1} of the row (ec)
// and of the row above (en), and the stores of the row's new values (with the
// stored PML part xc) and its samples.  Every lane calls it (it shuffles);
// own: the lane stores its vector.
__device__ __forceinline__ void h_row(const StepParams<float> &p, const Row2 &r, const float (&ec)[4],
                                      const float (&en)[4], const float (&xc)[4], int j, int i0, bool own, int n) {
  const float rgt = __shfl_down_sync(kFull, ec[0], 1);
  if (!own) return;
  // Hx -= Ku (Ez(j+1)-Ez(j)), Hy += Ku (Ez(i+1)-Ez(i))
  float hx[4], hy[4];
  const bool main_y = j >= p.mlo[1] && j <= p.mhi[1];
  const bool main_x = i0 >= p.mlo[0] && i0 + 3 <= p.mhi[0];
  if (!r.shell && main_x && main_y) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float rt = q < 3 ? ec[q + 1] : rgt;
      hx[q] = r.hx[q] + p.ku * (-en[q] + ec[q]);
      hy[q] = r.hy[q] + p.ku * (rt - ec[q]);
    }
  } else {
    const bool shell_y = j < p.slo[1] || j > p.shi[1];
    float g1x[4] = {}, g2x[4] = {}, g1y = 0.f, g2y = 0.f;
    if (r.shell) {
      vld_ro<float, 4>(p.cg1[0] + i0, g1x);
      vld_ro<float, 4>(p.cg2[0] + i0, g2x);
      g1y = __ldg(p.cg1[1] + j);
      g2y = __ldg(p.cg2[1] + j);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = i0 + q;
      const float rt = q < 3 ? ec[q + 1] : rgt;
      hx[q] = r.hx[q];
      hy[q] = r.hy[q];
      if (r.shell && (i < p.slo[0] || i > p.shi[0] || shell_y)) {
        hx[q] = lin2(g1y, hx[q], g2y, -en[q] + ec[q]);
        hy[q] = lin2(g1x[q], hy[q], g2x[q], rt - ec[q]);
      } else if (main_y && i >= p.mlo[0] && i <= p.mhi[0]) {
        hx[q] = hx[q] + p.ku * (-en[q] + ec[q]);
        hy[q] = hy[q] + p.ku * (rt - ec[q]);
      }
    }
  }
  const long long c = (long long)j * p.nx + i0;
  // Ez of dispersive cells is e2d_ade's to store
  bool ade = false;
#pragma unroll
  for (int q = 0; q < 4; ++q) ade |= id_of(r.id, q) >= kAdeId;
  if (!ade) {
    vst<float, 4>(p.ezo + c, ec);
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (id_of(r.id, q) < kAdeId) p.ezo[c + q] = ec[q];
  }
  vst<float, 4>(p.hxo + c, hx);
  vst<float, 4>(p.hyo + c, hy);
  if (r.shell) vst<float, 4>(p.spo[0] + c, xc);
  if (p.gather && (r.rf & ROW_SAMPLE))
    gather_row4(p, n, i0, j, make_float4(ec[0], ec[1], ec[2], ec[3]), make_float4(hx[0], hx[1], hx[2], hx[3]),
                make_float4(hy[0], hy[1], hy[2], hy[3]));
}

__global__ void __launch_bounds__(kGThreads) step2d_fused(const __grid_constant__ StepParams<float> p) {
  // with no dispersive cells the kernel before this one is the previous step;
  // otherwise it is e2d_ade, which let this kernel start only after its own
  // wait for the previous step
  if (p.nade == 0) pdl_wait();
  pdl_release();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nvec = p.nx >> 2, nstrip = (nvec + kGOwn - 1) / kGOwn;
  const int strip = blockIdx.x % nstrip, grp = blockIdx.x / nstrip;
  const int j0 = (grp * kGWarps + w) * kGRows;
  const int i0 = (strip * kGOwn + lane) * 4;
  const bool own_x = lane < kGOwn && i0 < p.nx;
  const int n = step_n(p);
  __shared__ __align__(16) WarpRing rings[kGWarps];
  WarpRing &rg = rings[w];
  if (j0 < p.ny) {
    const int jend = min(j0 + kGRows, p.ny);  // rows j0..jend-1 are stored; row jend is the row above
    // copy group g holds row j0 + g (group 0 also the row below j0); every
    // round commits one group, empty past row jend, so that the count of
    // groups in flight is the same in every round
    cp16(&rg.below[lane], j0 > 0 && i0 < p.nx ? p.hx + (long long)(j0 - 1) * p.nx + i0 : p.hx, j0 > 0 && i0 < p.nx);
#pragma unroll
    for (int g = 0; g < kGAhead; ++g) {
      if (j0 + g <= jend) issue_row(p, rg.s[g], j0 + g, i0, lane);
      cp_commit();
    }
    cp_wait_ahead();
    Row2 cur, nxt;
    read_row(p, rg.s[0], j0, i0, lane, cur);
    float below[4];
    {
      const float4 b = rg.below[lane];
      below[0] = b.x; below[1] = b.y; below[2] = b.z; below[3] = b.w;
    }
    float ec[4], xc[4];
    ez_new(p, cur, below, j0, i0, lane, n, ec, xc);
#pragma unroll 1
    for (int t = 0; j0 + t < jend; ++t) {
      const int j = j0 + t;
      if (j + kGAhead <= jend) issue_row(p, rg.s[(t + kGAhead) % kGSlots], j + kGAhead, i0, lane);
      cp_commit();
      cp_wait_ahead();  // rows up to j + 1 have landed
      read_row(p, rg.s[(t + 1) % kGSlots], j + 1, i0, lane, nxt);
      float en[4], xn[4];
      ez_new(p, nxt, cur.hx, j + 1, i0, lane, n, en, xn);
      h_row(p, cur, ec, en, xc, j, i0, own_x, n);
      cur = nxt;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        ec[q] = en[q];
        xc[q] = xn[q];
      }
    }
  }
  // no copy may still be in flight into shared memory when the block exits
  asm volatile("cp.async.wait_all;" ::: "memory");
  // complete only after e2d_ade: the kernels after this one wait for this one
  pdl_wait();
}

int launch_step2d_fused(const StepParams<float> &p, void *stream) {
  const int nvec = p.nx / 4, nstrip = (nvec + kGOwn - 1) / kGOwn;
  const int ngrp = (p.ny + kGRows * kGWarps - 1) / (kGRows * kGWarps);
  launch_pdl(step2d_fused, nstrip * ngrp, kGThreads, (cudaStream_t)stream, p);
  return 1;
}

}  // namespace fdtd
