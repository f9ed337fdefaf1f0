// k3f.cu -- the fused 3D step kernel (FP32): one pass over the core box that
// takes E and H from step n to n+1 (3D/.../include/myfdtd_func.f90:19-64,
// updateD then updateH), so that each field is read once and written once
// per step instead of once per half step.
//
// A block owns a tile of 31 x-vectors (124 cells) by 8 rows and marches up to
// kFZ planes of the core box along z.  At plane k it computes E^{n+1}(k) on
// the tile widened by one vector to the right and one row above (lane 31 and
// warp 8 of the 9 warps), then H^{n+1}(k-1) on the tile, whose curl needs
// E^{n+1} one cell right, one row above and one plane above.  The widened
// E^{n+1} belongs to the neighbouring tiles, which compute the same values
// themselves; so every tile is independent of the others.  That works
// because the step reads the fields of step n from one buffer and stores
// those of step n+1 to the other (a ping-pong pair): no tile can see a
// neighbour's new values where it needs the old ones.
//
// The H planes of step n come by tiled bulk copies (TMA) into a 3-stage
// shared-memory ring, as in e3d_core_tma: Hx with the row below, Hy with a
// 4-float halo to the left, Hz with both, over the widened tile.  E^n and the
// material ids are the threads' own vector loads, one plane ahead.  E^{n+1}
// of the plane goes to shared memory (Ex, Ez: the row above for the warp
// below) and stays in registers (the plane below for the next plane's H);
// the cell to the right comes from the next lane by a shuffle.
//
// Cells the kernel does not update itself -- dispersive (ADE) cells, rows
// with a source, and the widened cells that lie outside the core box -- get
// their E^{n+1} from the output buffer, where the general E kernel, launched
// before this one, stored it.  H of rows with a source is left to the general
// H kernel, launched after.  The arithmetic of every cell is that of
// e3d_core and h3d_core, term for term, so the results equal the split
// kernels' bit for bit.
//
// It runs where the core box lies at least one cell inside the grid on every
// side (every neighbour a cell of the grid, no wrap) and the grid has no
// reference slabs and no TFSF box.
#include <cuda_runtime.h>

#include "fdtd_internal.h"
#include "kcommon.cuh"

namespace fdtd {

constexpr int kFOwn = 31;                 // owned x-vectors of a tile (lane 31: the widened vector)
constexpr int kFY = 8;                    // owned rows (warps 0..7; warp 8: the widened row)
constexpr int kFW = kFY + 1;
constexpr int kFThreads = 32 * kFW;
constexpr int kFZ = 32;                   // planes per block
constexpr int kFRow = 128, kFRowH = 132;  // floats per smem row: Hx (no halo) / Hy, Hz (4-float halo)
constexpr int kFHx = (kFY + 2) * kFRow;                 // Hx box 128 x 10
constexpr int kFHyBox = (kFY + 1) * kFRowH;             // Hy box 132 x 9
constexpr int kFHzBox = (kFY + 2) * kFRowH;             // Hz box 132 x 10
constexpr int kFHy = ((kFHyBox + 31) / 32) * 32;        // padded to 128 bytes
constexpr int kFHz = ((kFHzBox + 31) / 32) * 32;
constexpr int kFStage = kFHx + kFHy + kFHz;             // floats per stage
constexpr unsigned kFBytes = (unsigned)(kFHx + kFHyBox + kFHzBox) * 4u;  // bytes a stage receives
constexpr int kFXe = 2 * 2 * kFW * kFRow;               // E^{n+1} Ex, Ez rows: [plane parity][comp][row][x]
constexpr int kFSmem = (3 * kFStage + kFXe) * 4 + 128;  // dynamic shared bytes (+ alignment)
static_assert((kFHx * 4) % 128 == 0 && (kFHy * 4) % 128 == 0 && (kFStage * 4) % 128 == 0,
              "TMA destinations are 128-byte aligned");

__global__ void __launch_bounds__(kFThreads, 3) step3d_fused(const __grid_constant__ StepParams<float> p,
                                                          const __grid_constant__ FusedMaps m) {
  extern __shared__ unsigned char sm_raw[];
  __shared__ __align__(8) unsigned long long bar[3];
  pdl_wait();
  pdl_release();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int bx = (p.cw + kFOwn - 1) / kFOwn, by = (p.ch + kFY - 1) / kFY;
  const int tx = blockIdx.x % bx, t2 = blockIdx.x / bx, ty = t2 % by, tz = t2 / by;
  const int v = tx * kFOwn + lane, r = ty * kFY + w;  // vector and row of this thread, relative to the core box
  const int x0 = (p.cv0 + tx * kFOwn) * 4, y0 = p.cy0 + ty * kFY;
  const int kend = p.cz0 + p.cd;
  const int kz0 = p.cz0 + tz * kFZ, kz1 = min(kz0 + kFZ, kend);  // H planes kz0..kz1-1, E planes kz0..kz1
  // part: the thread's vector is needed (the owned tile, widened by a vector
  // and a row, within one past the core box); own: it is stored
  const bool part = v <= p.cw && r <= p.ch;
  const bool own = lane < kFOwn && w < kFY && v < p.cw && r < p.ch;
  const int j = y0 + w, xr = 4 * lane, i0 = x0 + xr;
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(sm_raw);
  const uint32_t sbase = (raw + 127u) & ~127u;
  float *gbase = (float *)(sm_raw + (sbase - raw));
  float *xe = gbase + 3 * kFStage;
  const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(bar);
  if (threadIdx.x == 0) {
    for (int s = 0; s < 3; ++s) mbar_init(bar0 + 8 * s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // load number u is plane kz0 - 1 + u, in stage u % 3, whose (u / 3)-th phase it completes
  auto issue = [&](int u) {
    const int s = u % 3, plane = kz0 - 1 + u;
    const uint32_t st = sbase + (uint32_t)(s * kFStage * 4), b = bar0 + 8 * s;
    mbar_expect_tx(b, kFBytes);
    tma_load_3d(st, &m.hx, x0, y0 - 1, plane, b);
    tma_load_3d(st + kFHx * 4, &m.hy, x0 - 4, y0, plane, b);
    tma_load_3d(st + (kFHx + kFHy) * 4, &m.hz, x0 - 4, y0 - 1, plane, b);
  };
  const int nload = kz1 - kz0 + 2;  // planes kz0-1 .. kz1
  if (threadIdx.x == 0) {
    issue(0);
    issue(1);
  }
  int issued = 2, waited = 0;
  bool ok = __syncthreads_and(mbar_wait(bar0, 0, p.wait_limit));
  waited = ok ? 1 : 0;
  // the inputs of plane k: E^n of a core vector, or E^{n+1} (from the output
  // buffer) of a vector the kernel does not update; loaded one plane ahead
  float ea[3][4] = {}, ep[3][4] = {};
  uint8_t id[4] = {};
  bool core = false, core_prev = false;
  auto load_e = [&](int k) {
    core = false;
    if (!part) return;
    const long long row = (long long)k * p.ny + j;
    const long long c = row * p.nx + i0;
    core = v < p.cw && r < p.ch && k < kend && !__ldg(p.rowflag + row);
    vld<float, 4>((core ? p.ex : p.exo) + c, ea[0]);
    vld<float, 4>((core ? p.ey : p.eyo) + c, ea[1]);
    vld<float, 4>((core ? p.ez : p.ezo) + c, ea[2]);
    if (core) vec_ids<float, 4>(p, row, i0 / 4, p.mat + c, id);
  };
  load_e(kz0);
  for (int k = kz0; ok && k <= kz1; ++k) {
    const int u = k - kz0 + 1;  // load number of plane k
    ok = __syncthreads_and(mbar_wait(bar0 + 8 * (u % 3), (unsigned)(u / 3) & 1u, p.wait_limit));
    if (!ok) break;
    waited = u + 1;
    // the next plane goes into the stage the plane k - 2 held, which the last
    // round read: every thread has passed the barrier above, so every thread
    // is done with it (and with the E rows the last round read, which this
    // round's rows of the other parity overwrite next round)
    if (threadIdx.x == 0 && u + 1 < nload) issue(u + 1);
    if (u + 1 < nload) issued = u + 2;
    const float *Hx = gbase + (u % 3) * kFStage, *Hy = Hx + kFHx, *Hz = Hy + kFHy;
    const float *Hxp = gbase + ((u + 2) % 3) * kFStage, *Hyp = Hxp + kFHx, *Hzp = Hyp + kFHy;
    // ---- E^{n+1} of plane k (e3d_core's arithmetic) ----
    float ne[3][4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int q = 0; q < 4; ++q) ne[c][q] = ea[c][q];
    if (core) {
      const int yr = kFRowH * w + 4 + xr, zr = kFRowH * (w + 1) + 4 + xr;
      const float4 hx4 = *(const float4 *)(Hx + kFRow * (w + 1) + xr);
      const float4 hxd4 = *(const float4 *)(Hx + kFRow * w + xr);
      const float4 hxb4 = *(const float4 *)(Hxp + kFRow * (w + 1) + xr);
      const float4 hy4 = *(const float4 *)(Hy + yr), hyb4 = *(const float4 *)(Hyp + yr);
      const float4 hz4 = *(const float4 *)(Hz + zr), hzd4 = *(const float4 *)(Hz + zr - kFRowH);
      const float hyl = Hy[yr - 1], hzl = Hz[zr - 1];
      const float hx[4] = {hx4.x, hx4.y, hx4.z, hx4.w}, hxd[4] = {hxd4.x, hxd4.y, hxd4.z, hxd4.w};
      const float hxb[4] = {hxb4.x, hxb4.y, hxb4.z, hxb4.w}, hy[4] = {hy4.x, hy4.y, hy4.z, hy4.w};
      const float hyb[4] = {hyb4.x, hyb4.y, hyb4.z, hyb4.w}, hz[4] = {hz4.x, hz4.y, hz4.z, hz4.w};
      const float hzd[4] = {hzd4.x, hzd4.y, hzd4.z, hzd4.w};
      bool uni = true;
#pragma unroll
      for (int q = 0; q < 4; ++q) uni &= id[q] == p.id0;
      const long long c = ((long long)k * p.ny + j) * p.nx + i0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float ca = uni ? p.ca0 : (id[q] == p.id0 ? p.ca0 : __ldg(p.mca + id[q]));
        const float curlhzy = hz[q] - hzd[q], curlhyz = -hy[q] + hyb[q];
        const float curlhxz = hx[q] - hxb[q], curlhzx = -hz[q] + (q ? hz[q - 1] : hzl);
        const float curlhyx = hy[q] - (q ? hy[q - 1] : hyl), curlhxy = -hx[q] + hxd[q];
        ne[0][q] = ea[0][q] + ca * (curlhzy + curlhyz);
        ne[1][q] = ea[1][q] + ca * (curlhxz + curlhzx);
        ne[2][q] = ea[2][q] + ca * (curlhyx + curlhxy);
        if (!uni && id[q] >= kAdeId) {  // a dispersive cell: the general kernel's value
          ne[0][q] = p.exo[c + q];
          ne[1][q] = p.eyo[c + q];
          ne[2][q] = p.ezo[c + q];
        }
      }
      if (own && k < kz1) {
        if (uni) {
          vst<float, 4>(p.exo + c, ne[0]);
          vst<float, 4>(p.eyo + c, ne[1]);
          vst<float, 4>(p.ezo + c, ne[2]);
        } else {
          st_guard3<float, 4>(p.exo + c, ne[0], id);
          st_guard3<float, 4>(p.eyo + c, ne[1], id);
          st_guard3<float, 4>(p.ezo + c, ne[2], id);
        }
      }
    }
    if (part) {  // Ex and Ez of this row for the warp below
      float *xr0 = xe + ((k & 1) * 2 + 0) * kFW * kFRow + w * kFRow + xr;
      float *xr2 = xe + ((k & 1) * 2 + 1) * kFW * kFRow + w * kFRow + xr;
      *(float4 *)xr0 = make_float4(ne[0][0], ne[0][1], ne[0][2], ne[0][3]);
      *(float4 *)xr2 = make_float4(ne[2][0], ne[2][1], ne[2][2], ne[2][3]);
    }
    // ---- H^{n+1} of plane k-1 (h3d_core's arithmetic) ----
    if (k > kz0) {
      // the cell right of the vector: the next lane's first cell
      const float eyr = __shfl_down_sync(0xffffffffu, ep[1][0], 1);
      const float ezr = __shfl_down_sync(0xffffffffu, ep[2][0], 1);
      if (own && core_prev) {
        const float *exu = xe + (((k - 1) & 1) * 2 + 0) * kFW * kFRow + (w + 1) * kFRow + xr;
        const float *ezu = xe + (((k - 1) & 1) * 2 + 1) * kFW * kFRow + (w + 1) * kFRow + xr;
        const float4 exu4 = *(const float4 *)exu, ezu4 = *(const float4 *)ezu;
        const float4 hx4 = *(const float4 *)(Hxp + kFRow * (w + 1) + xr);
        const float4 hy4 = *(const float4 *)(Hyp + kFRowH * w + 4 + xr);
        const float4 hz4 = *(const float4 *)(Hzp + kFRowH * (w + 1) + 4 + xr);
        const float exv[4] = {exu4.x, exu4.y, exu4.z, exu4.w}, ezv[4] = {ezu4.x, ezu4.y, ezu4.z, ezu4.w};
        float hx[4] = {hx4.x, hx4.y, hx4.z, hx4.w}, hy[4] = {hy4.x, hy4.y, hy4.z, hy4.w};
        float hz[4] = {hz4.x, hz4.y, hz4.z, hz4.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float rz = q < 3 ? ep[2][q + 1] : ezr, ry = q < 3 ? ep[1][q + 1] : eyr;
          const float curleyz = ne[1][q] - ep[1][q], curlezy = -ezv[q] + ep[2][q];
          const float curlezx = rz - ep[2][q], curlexz = -ne[0][q] + ep[0][q];
          const float curlexy = exv[q] - ep[0][q], curleyx = -ry + ep[1][q];
          hx[q] = hx[q] + p.ku * (curleyz + curlezy);
          hy[q] = hy[q] + p.ku * (curlezx + curlexz);
          hz[q] = hz[q] + p.ku * (curlexy + curleyx);
        }
        const long long c = ((long long)(k - 1) * p.ny + j) * p.nx + i0;
        vst<float, 4>(p.hxo + c, hx);
        vst<float, 4>(p.hyo + c, hy);
        vst<float, 4>(p.hzo + c, hz);
      }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int q = 0; q < 4; ++q) ep[c][q] = ne[c][q];
    core_prev = core;
    if (k + 1 <= kz1) load_e(k + 1);
  }
  if (!ok) {
    // a wait gave up: report it, and let the copies already issued land
    // (each wait bounded) before the block's shared memory goes away
    if (threadIdx.x == 0) atomicExch(p.err, 1);
    for (int u = waited; u < issued; ++u) mbar_wait(bar0 + 8 * (u % 3), (unsigned)(u / 3) & 1u);
  }
}

void step3d_fused_shape(const StepParams<float> &p, int *blocks, int *smem) {
  *blocks = ((p.cw + kFOwn - 1) / kFOwn) * ((p.ch + kFY - 1) / kFY) * ((p.cd + kFZ - 1) / kFZ);
  *smem = kFSmem;
}

int launch_step3d_fused(const StepParams<float> &p, const FusedMaps &m, void *stream) {
  static bool attr = [] {
    return cudaFuncSetAttribute(step3d_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, kFSmem) == cudaSuccess;
  }();
  (void)attr;
  int blocks = 0, smem = 0;
  step3d_fused_shape(p, &blocks, &smem);
  if (blocks <= 0) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kFThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = (cudaStream_t)stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, step3d_fused, p, m);
  return 1;
}

}  // namespace fdtd
