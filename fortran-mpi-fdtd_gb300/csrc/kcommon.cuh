// kcommon.cuh -- device helpers shared by the 2D and 3D half-step kernels.
#pragma once
#include <cuda_runtime.h>

#include "fdtd_internal.h"

namespace fdtd {

// The FP64 plain path keeps both parts of every split PML field (as the
// reference does); FP32 stores one part and takes the other as total - part.
template <typename T>
constexpr bool kTwoParts = sizeof(T) == 8;

// ---- programmatic dependent launch ----------------------------------------
// A kernel launched with programmatic stream serialisation may be scheduled
// while the kernel before it on its stream drains.  pdl_wait blocks until
// that kernel has completed and its writes are visible (with no such
// dependency it returns at once); pdl_release lets the next kernel on the
// stream be scheduled, which then waits in its own pdl_wait.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// a*b + c*d with one fixed rounding: a*b fused into the add, c*d rounded
// first.  Left to the compiler, the contraction of a sum of two products may
// fuse either one, and differently in different kernels; the split-field PML
// updates use this form wherever two kernels compute the same cell, so that
// their results agree bit for bit.
__device__ __forceinline__ float lin2(float a, float b, float c, float d) { return __fmaf_rn(a, b, __fmul_rn(c, d)); }
__device__ __forceinline__ double lin2(double a, double b, double c, double d) {
  return __fma_rn(a, b, __dmul_rn(c, d));
}

// launch a step kernel with a programmatic dependency on the kernel before it
// on the stream (the kernel starts with pdl_wait).  With `ev`, the launch also
// records ev as a programmatic event that fires once every block has started:
// kernels on other streams that wait on it may launch early and then wait in
// their own pdl_wait for this kernel's completion.
template <typename K, typename P>
inline void launch_pdl(K kernel, int blocks, int threads, cudaStream_t s, const P &p, cudaEvent_t ev = nullptr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(threads);
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
  cudaLaunchKernelEx(&cfg, kernel, p);
}

// launch_pdl for a kernel of two parameters
template <typename K, typename P, typename Q>
inline void launch_pdl2(K kernel, int blocks, int threads, cudaStream_t s, const P &p, const Q &q) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(threads);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, p, q);
}

// launch a small kernel that runs beside a large one with the device's
// highest scheduling priority, so that its blocks are dispatched ahead of the
// large kernel's pending blocks
inline int side_priority() {
  static int prio = [] {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return 0;
    return greatest;
  }();
  return prio;
}

template <typename K, typename P>
inline void launch_side(K kernel, int blocks, int threads, cudaStream_t s, const P &p) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(threads);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = side_priority();
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, p);
}

// ---- vector access of V consecutive cells along x ------------------------
template <typename T, int V> struct VecOf;
template <> struct VecOf<float, 1> { typedef float t; };
template <> struct VecOf<float, 2> { typedef float2 t; };
template <> struct VecOf<float, 4> { typedef float4 t; };
template <> struct VecOf<double, 1> { typedef double t; };
template <> struct VecOf<double, 2> { typedef double2 t; };
template <int V> struct ByteVec;
template <> struct ByteVec<1> { typedef unsigned char t; };
template <> struct ByteVec<2> { typedef uchar2 t; };
template <> struct ByteVec<4> { typedef uchar4 t; };

template <typename T, int V>
__device__ __forceinline__ void vld_ro(const T *a, T (&v)[V]) {  // read-only path
  typedef typename VecOf<T, V>::t VT;
  const VT x = __ldg(reinterpret_cast<const VT *>(a));
  const T *e = reinterpret_cast<const T *>(&x);
#pragma unroll
  for (int q = 0; q < V; ++q) v[q] = e[q];
}
template <typename T, int V>
__device__ __forceinline__ void vld(const T *a, T (&v)[V]) {
  typedef typename VecOf<T, V>::t VT;
  const VT x = *reinterpret_cast<const VT *>(a);
  const T *e = reinterpret_cast<const T *>(&x);
#pragma unroll
  for (int q = 0; q < V; ++q) v[q] = e[q];
}
template <typename T, int V>
__device__ __forceinline__ void vst(T *a, const T (&v)[V]) {
  typedef typename VecOf<T, V>::t VT;
  VT x;
  T *e = reinterpret_cast<T *>(&x);
#pragma unroll
  for (int q = 0; q < V; ++q) e[q] = v[q];
  *reinterpret_cast<VT *>(a) = x;
}
template <int V>
__device__ __forceinline__ void vld_ids(const uint8_t *a, uint8_t (&v)[V]) {
  typedef typename ByteVec<V>::t BT;
  const BT x = __ldg(reinterpret_cast<const BT *>(a));
  const uint8_t *e = reinterpret_cast<const uint8_t *>(&x);
#pragma unroll
  for (int q = 0; q < V; ++q) v[q] = e[q];
}

// Neighbour loads across a face of the domain: wrapped when the axis is
// periodic (the reference's interchange_E/H with PBC), zero otherwise (the
// halo cells the reference never writes).
template <typename T>
__device__ __forceinline__ T ld_x(const T *a, int i, int j, int nx, int per) {
  if (i < 0) return per ? a[(long long)j * nx + (nx - 1)] : T(0);
  if (i >= nx) return per ? a[(long long)j * nx] : T(0);
  return a[(long long)j * nx + i];
}
template <typename T>
__device__ __forceinline__ T ld_y(const T *a, int i, int j, int nx, int ny, int per) {
  if (j < 0) return per ? a[(long long)(ny - 1) * nx + i] : T(0);
  if (j >= ny) return per ? a[i] : T(0);
  return a[(long long)j * nx + i];
}

template <typename T>
__device__ __forceinline__ T shfl_left(T v, int lane) {
  return __shfl_up_sync(0xffffffffu, v, 1);
}
template <typename T>
__device__ __forceinline__ T shfl_right(T v, int lane) {
  return __shfl_down_sync(0xffffffffu, v, 1);
}

template <typename T>
__device__ __forceinline__ bool in_shell2(const StepParams<T> &p, int i, int j) {
  return i < p.slo[0] || i > p.shi[0] || j < p.slo[1] || j > p.shi[1];
}
template <typename T>
__device__ __forceinline__ bool in_shell3(const StepParams<T> &p, int i, int j, int k) {
  return i < p.slo[0] || i > p.shi[0] || j < p.slo[1] || j > p.shi[1] || k < p.slo[2] || k > p.shi[2];
}
template <typename T>
__device__ __forceinline__ bool in_main2(const StepParams<T> &p, int i, int j) {
  return i >= p.mlo[0] && i <= p.mhi[0] && j >= p.mlo[1] && j <= p.mhi[1];
}
template <typename T>
__device__ __forceinline__ bool in_main3(const StepParams<T> &p, int i, int j, int k) {
  return i >= p.mlo[0] && i <= p.mhi[0] && j >= p.mlo[1] && j <= p.mhi[1] && k >= p.mlo[2] && k <= p.mhi[2];
}

// Step number of this launch: a kernel parameter for eager launches, the
// device-side ring base + slot when the step is replayed from a CUDA graph.
template <typename T>
__device__ __forceinline__ int step_n(const StepParams<T> &p) {
  return p.d_base ? *p.d_base + p.slot : p.n;
}

// Sum of this step's soft-source values driving component `comp` at a cell
// (3D/.../program.f90:396-406: D += gauss_t*n_air on the source plane).
template <typename T>
__device__ __forceinline__ T src_sum(const StepParams<T> &p, int n, int comp, int i, int j, int k) {
  T s = T(0);
  for (int q = 0; q < p.nsrc; ++q) {
    const Source &sr = p.src[q];
    if (sr.comp == comp && i >= sr.lo[0] && i <= sr.hi[0] && j >= sr.lo[1] && j <= sr.hi[1] &&
        k >= sr.lo[2] && k <= sr.hi[2])
      s += T(p.srcval_tab[(long long)(n - 1) * p.nsrc + q]);
  }
  return s;
}

// Does any source drive component `comp` on row j (plane k)?
template <typename T>
__device__ __forceinline__ bool src_row(const StepParams<T> &p, int comp, int j, int k) {
  for (int q = 0; q < p.nsrc; ++q) {
    const Source &sr = p.src[q];
    if (sr.comp == comp && j >= sr.lo[1] && j <= sr.hi[1] && k >= sr.lo[2] && k <= sr.hi[2]) return true;
  }
  return false;
}

// Does any monitor or probe sample row j (plane k)?
template <typename T>
__device__ __forceinline__ bool sample_row(const StepParams<T> &p, int j, int k) {
  for (int q = 0; q < p.nmon; ++q)
    if (j >= p.mon[q].lo[1] && j <= p.mon[q].hi[1] && k >= p.mon[q].lo[2] && k <= p.mon[q].hi[2]) return true;
  for (int q = 0; q < p.nprobe; ++q)
    if (j == p.probe[q].cell[1] && k == p.probe[q].cell[2]) return true;
  return false;
}

// One E component of a dispersive cell.  `inc` is this step's D increment
// (Ku*curl + source).  Gold (2D/gold_mod.f90:57-71, 3D/gold_mod.f90:61-82):
//   E = Re[(D - I + ha S + gb1 g1 + gb2 g2) / ga];  I += hb E;
//   S = ha S + hb E;  g_p = gb_p g_p + gc_p E
// with Q = D - I kept instead of D and I (Q += inc - hb E) and the
// recursions in delta form (S += hb E - (1-ha) S, g += (gb-1) g + gc E).
// Graphene sheet (1D/graphene633_mod.f90:33-41, 3D/graphene_mod.f90:70-76):
//   E = (Q + ha S + 2 kerr E^3) / (ga + S_R + 3 kerr E^2) with the Raman
//   recursion S_R(n) = r1 S_R(n-1) + r2 S_R(n-2) + r0 E^2 in velocity form.
// Lorentz poles (3D/goldLorentzJp_mod.f90:60-86, 3D/si_mod.f90:55-60):
//   E += ga (inc - sum_l v_l);  v_l += -lv v_l + (le E - ls p_l);  p_l += v_l
// On a Lorentz-Jp sheet (3D/graphene3LorentzJp1nm_mod.f90:42-100) the normal
// component is vacuum, and the Kerr term adds lk Q E to pole 0's drive with
//   g += -lqv g + lqs ((escale E)^2 - Q);  Q += g.
// The components of a cell are updated in order x, y, z by one thread.
// KIND >= 0: every cell of the launch has that kind, known at compile time,
// so the state loads of its update need not wait for the kind's test.
template <typename T, int KIND = -1>
__device__ __forceinline__ T ade_update_state(T *st, int stride, int slot, int comp, const AdeCoef<T> &a,
                                               const AdeCoef<T> *am, T inc, T eold) {
  const int kind = KIND >= 0 ? KIND : a.kind;
  T *q_ = st + (0 * 3 + comp) * (long long)stride + slot;
  T *s_ = st + (1 * 3 + comp) * (long long)stride + slot;
  T *f2 = st + (2 * 3 + comp) * (long long)stride + slot;
  T *f3 = st + (3 * 3 + comp) * (long long)stride + slot;
  if (kind == MK_LORENTZ) {
    if (comp == a.normal) return eold + inc;  // sheet: the normal component is vacuum
    T pl[kMaxPoles], vl[kMaxPoles];
    T sv = T(0);
#pragma unroll
    for (int l = 0; l < kMaxPoles; ++l) {
      if (l < a.npoles) {
        pl[l] = st[(2 * l * 3 + comp) * (long long)stride + slot];
        vl[l] = st[((2 * l + 1) * 3 + comp) * (long long)stride + slot];
        sv += vl[l];
      }
    }
    const int nlf = 2 * a.npoles;  // the Kerr term's Q and g follow the poles
    if (a.zx) {
      // SLG_LJp's Ez line subtracts the x current of the previous step
      // (3D/grapheneLorentzJp_mod.f90:68): the x update leaves its sum in
      // field nlf+2 (component slot 0) for the z update of the same cell
      T *xs = st + ((nlf + 2) * 3) * (long long)stride + slot;
      if (comp == 0) *xs = sv;
      else if (comp == 2) sv = *xs;
    }
    const T e = eold + a.ga * (inc - sv);
    T *qk = st + (nlf * 3 + comp) * (long long)stride + slot, *gk = st + ((nlf + 1) * 3 + comp) * (long long)stride + slot;
    const T qv = a.nl ? *qk : T(0);
#pragma unroll
    for (int l = 0; l < kMaxPoles; ++l) {
      if (l < a.npoles) {
        T drive = a.le[l] * e;
        if (l == 0 && a.nl) drive = drive + a.lk * (qv * e);
        const T nv = vl[l] + ((drive - a.ls[l] * pl[l]) - a.lv[l] * vl[l]);
        st[((2 * l + 1) * 3 + comp) * (long long)stride + slot] = nv;
        st[(2 * l * 3 + comp) * (long long)stride + slot] = pl[l] + nv;
      }
    }
    if (a.nl) {
      const T es = a.escale * e;
      const T g = *gk;
      const T ng = g + (a.lqs * (es * es - qv) - a.lqv * g);
      *gk = ng;
      *qk = qv + ng;
    }
    return e;
  }
  T Q = *q_ + inc;
  T S = *s_;
  if (kind == MK_GOLD) {
    T *f4 = st + (4 * 3 + comp) * (long long)stride + slot;
    T *f5 = st + (5 * 3 + comp) * (long long)stride + slot;
    const T g1r = *f2, g1i = *f3, g2r = *f4, g2i = *f5;
    // gb*g = g + (gb-1)*g
    const T p1r = g1r + (a.dr[0] * g1r - a.di[0] * g1i), p1i = g1i + (a.dr[0] * g1i + a.di[0] * g1r);
    const T p2r = g2r + (a.dr[1] * g2r - a.di[1] * g2i), p2i = g2i + (a.dr[1] * g2i + a.di[1] * g2r);
    const T nre = ((Q + a.ha * S) + p1r) + p2r;
    const T nim = p1i + p2i;
    const T e = nre * a.wr - nim * a.wi;
    *q_ = Q - a.hb * e;
    *s_ = S + (a.hb * e - a.dha * S);
    *f2 = p1r + a.gcr[0] * e;
    *f3 = p1i + a.gci[0] * e;
    *f4 = p2r + a.gcr[1] * e;
    *f5 = p2i + a.gci[1] * e;
    return e;
  }
  if (kind == MK_GRAPHENE_CP) {
    // the reference's Graphene: Re[(Q + ha S + sum_p gb_p g_p) / (ga + S_R)].
    // Its coefficients are read through am, not the caller's copy a: a copy
    // of every kind's fields would stay in registers across the components.
    if (comp == a.normal) return eold + inc;  // the normal component is vacuum (E = D)
    const long long cs = 3 * (long long)stride;
    T *g0 = st + (2 * 3 + comp) * (long long)stride + slot;  // g_p: fields 2+2p (re), 3+2p (im)
    const T ha = am->ha, hb = am->hb, dha = am->dha;
    T nre = Q + ha * S, nim = T(0);
#pragma unroll 1  // unrolled, the loads of all four points would stay live together
    for (int q = 0; q < kMaxCp; ++q) {
      const T gr = g0[2 * q * cs], gi = g0[(2 * q + 1) * cs];
      const T dr = am->dr[q], di = am->di[q];
      nre = nre + (gr + (dr * gr - di * gi));
      nim = nim + (gi + (dr * gi + di * gr));
    }
    T *srp = st + (10 * 3 + comp) * (long long)stride + slot, *vp = st + (11 * 3 + comp) * (long long)stride + slot;
    const T sr = *srp, v = *vp;
    const T gai = am->gai, dre = am->gar + sr;
    const T e = (nre * dre + nim * gai) / (dre * dre + gai * gai);
    const T nv = am->rv * v + am->rs * sr + am->r0 * (e * e);
    *vp = nv;
    *srp = sr + nv;
    *q_ = Q - hb * e;
    *s_ = S + (hb * e - dha * S);
    // g_p = gb_p g_p + gc_p E, with gb_p g_p recomputed from the state (the
    // same operations as above, so the same values) rather than kept live
#pragma unroll 1
    for (int q = 0; q < kMaxCp; ++q) {
      const T gr = g0[2 * q * cs], gi = g0[(2 * q + 1) * cs];
      const T dr = am->dr[q], di = am->di[q];
      g0[2 * q * cs] = (gr + (dr * gr - di * gi)) + am->gcr[q] * e;
      g0[(2 * q + 1) * cs] = (gi + (dr * gi + di * gr)) + am->gci[q] * e;
    }
    return e;
  }
  // graphene
  if (comp == a.normal) {  // out-of-plane component: vacuum, E = D
    *q_ = Q;
    return eold + inc;
  }
  const T sr = *f2, v = *f3;
  const T num = (Q + a.ha * S) + T(2) * a.kerr * (eold * eold * eold);
  const T den = (a.ga + sr) + T(3) * a.kerr * (eold * eold);
  const T e = num / den;
  const T nv = a.rv * v + a.rs * sr + a.r0 * (e * e);
  *f3 = nv;
  *f2 = sr + nv;
  *q_ = Q - a.hb * e;
  *s_ = S + (a.hb * e - a.dha * S);
  return e;
}

// store V values, skipping cells whose E belongs to an ADE thread
template <typename T, int V>
__device__ __forceinline__ void st_guard3(T *a, const T (&v)[V], const uint8_t (&id)[V]) {
#pragma unroll
  for (int q = 0; q < V; ++q)
    if (id[q] < kAdeId) a[q] = v[q];
}

// the ids of the x-vector v of a row: id0 throughout when the uniformity
// bitmap says so, else loaded
template <typename T, int V>
__device__ __forceinline__ void vec_ids(const StepParams<T> &p, long long row, int v, const uint8_t *mat,
                                        uint8_t (&id)[V]) {
  if (p.uni && ((__ldg(p.uni + row * p.uni_words + (v >> 5)) >> (v & 31)) & 1u)) {
#pragma unroll
    for (int q = 0; q < V; ++q) id[q] = (uint8_t)p.id0;
  } else {
    vld_ids<V>(mat, id);
  }
}

// ---- mbarrier and tiled bulk copies (TMA) ------------------------------------

__device__ __forceinline__ void mbar_init(uint32_t bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// bounded wait for the phase of the given parity to complete: at most
// `limit` polls, then false
__device__ __forceinline__ bool mbar_wait(uint32_t bar, unsigned parity, unsigned limit = kWaitLimit) {
  for (unsigned it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// coefficients of a dispersive material id (>= kAdeId)
template <typename T>
__device__ __forceinline__ const AdeCoef<T> &ade_coef(const StepParams<T> &p, int id) {
  // a reference, not a copy: a copy would load every field of both candidate
  // sets (the kernel parameter's and the table's) before the kind is known;
  // read through the reference, each update loads only the fields it uses
  const int ai = id - kAdeId;
  return ai < kAdeParam ? p.acp[ai] : p.ac[ai];
}

// a: the coefficients by value; am: the same set in the job's table
template <typename T, int KIND = -1>
__device__ __forceinline__ T ade_update(const StepParams<T> &p, const AdeCoef<T> &a, const AdeCoef<T> *am, int slot,
                                         int comp, T inc, T eold) {
  return ade_update_state<T, KIND>(p.ade_state, p.ade_stride, slot, comp, a, am, inc, eold);
}

// vals[c] for a component number known only at run time, by constant-index
// selects: an indexed read would put the caller's array in local memory
template <typename T>
__device__ __forceinline__ T pick6(const T *vals, int c) {
  T r = vals[0];
#pragma unroll
  for (int q = 1; q < 6; ++q)
    if (c == q) r = vals[q];
  return r;
}

// Slot 0 of the stage ring this step's samples go to: a graph replay finds
// its ring's half of the two-ring stage buffer on the device.
template <typename T>
__device__ __forceinline__ T *stage_ring(const StepParams<T> &p) {
  return p.d_half ? p.stage + (long long)(*p.d_half) * kStageSteps * p.stage_row : p.stage;
}

// Fused sampling: write the monitored components of cell (i,j,k) into this
// step's stage row, and probe samples.  vals[c] = value of component c.
template <typename T>
__device__ __forceinline__ void gather_cell(const StepParams<T> &p, int n, int i, int j, int k, const T *vals) {
  for (int q = 0; q < p.nmon; ++q) {
    const Monitor &m = p.mon[q];
    if (i < m.lo[0] || i > m.hi[0] || j < m.lo[1] || j > m.hi[1] || k < m.lo[2] || k > m.hi[2]) continue;
    const int wx = m.hi[0] - m.lo[0] + 1, wy = m.hi[1] - m.lo[1] + 1;
    const long long idx = (long long)(i - m.lo[0]) + (long long)wx * ((j - m.lo[1]) + (long long)wy * (k - m.lo[2]));
    T *row = stage_ring(p) + (long long)p.slot * p.stage_row + m.base;
    for (int u = 0; u < m.ncomp; ++u) row[(long long)u * m.ncell + idx] = pick6(vals, m.comps[u]);
  }
  for (int q = 0; q < p.nprobe; ++q) {
    const Probe &pr = p.probe[q];
    if (i != pr.cell[0] || j != pr.cell[1] || k != pr.cell[2]) continue;
    if (n < pr.n_first || n > pr.n_last) continue;
    const long long st = n - pr.n_first;
    if (st >= pr.cap) continue;
    double *out = pr.buf + st * pr.ncomp;
    for (int u = 0; u < pr.ncomp; ++u) out[u] = (double)pick6(vals, pr.comps[u]);
  }
}

}  // namespace fdtd
