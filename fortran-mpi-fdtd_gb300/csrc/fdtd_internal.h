// fdtd_internal.h -- device-side parameter blocks shared by the kernels and
// the host job manager (fdtd_api.cu).  Not part of the public ABI.
//
// Data layout in HBM (per job, T = float or double):
//   * main fields: one array per component, nx*ny*nz values, x fastest, no
//     halo cells: neighbours across a periodic face are read by index wrap,
//     across a non-periodic face they are zero.  The MPI slabs of the
//     reference are one array, so interchange_E/H need no copies.
//   * material id map: one byte per cell (0 = no material).
//   * dispersive (ADE) cells: a compact slot list (cell index, material id)
//     with structure-of-arrays state per slot and component.
//   * PML: reference y-slabs (split arrays over npml rows only) or, for the
//     split-field PML on any faces, one stored sub-field per split component
//     (the other part is the total minus the stored part) over the full grid
//     (only shell cells are touched).
//   * DFT: samples of the monitored cells are staged per step in a ring of
//     kStageSteps slots and folded into FP64 accumulators once per ring.
#pragma once
#include <cuda.h>  // CUtensorMap (the maps are encoded through the runtime's driver entry point)
#include <cuda_runtime.h>

#include <cstdint>

#include "fdtd_gb300.h"

namespace fdtd {

// tensor maps of one buffer's H arrays for the fused 3D step kernel: one-plane
// boxes of Hx 128 x 10 rows from (x0, y0-1), Hy 132 x 9 from (x0-4, y0), Hz
// 132 x 10 from (x0-4, y0-1)
struct FusedMaps {
  CUtensorMap hx, hy, hz;
};

// tensor maps of the 3D H arrays (FP32) for the TMA-staged E core: boxes of
// one plane, Hx 128 x 9 rows from (x0, y0-1), Hy 132 x 8 from (x0-4, y0),
// Hz 132 x 9 from (x0-4, y0-1)
struct TmaMaps {
  CUtensorMap hx, hy, hz;
  // the H core's E planes: Ex 128 x 9 rows from (x0, y0), Ey 132 x 8 and Ez
  // 132 x 9 from (x0, y0) (the cell to the right, the row above); h_ok when set
  CUtensorMap ex, ey, ez;
  int h_ok;
};

constexpr int kMaxMat = 256;
constexpr int kMaxSrc = 8;
constexpr int kMaxMon = 16;
constexpr int kMaxProbe = 16;
constexpr int kStageSteps = 32;  // DFT staging ring length (steps per fold)
constexpr unsigned kWaitLimit = 1u << 22;  // default try_wait rounds before an mbarrier wait gives up

// MK_CONDUCTIVE and MK_GRAPHENE_NK exist on the host only: their cells run
// the gold and the graphene update
enum MatKind : int { MK_NONE = 0, MK_DIEL = 1, MK_GOLD = 2, MK_GRAPHENE = 3, MK_LORENTZ = 4, MK_GRAPHENE_CP = 5,
                     MK_CONDUCTIVE = 6, MK_GRAPHENE_NK = 7 };
constexpr int kMaxPoles = FDTD_LORENTZ_MAX_POLES;
constexpr int kMaxCp = 4;  // critical points of the reference's graphene
__host__ __device__ constexpr bool is_ade_kind(int k) {
  return k == MK_GOLD || k == MK_GRAPHENE || k == MK_LORENTZ || k == MK_GRAPHENE_CP || k == MK_CONDUCTIVE ||
         k == MK_GRAPHENE_NK;
}

// per material id, in the job's precision
template <typename T>
struct MatCoef {
  int kind;
  int ade;      // index into the ADE coefficient table (gold/graphene), -1 otherwise
  T ca;         // Ku * (1/eps): E += ca * curl
  T cs;         // 1/eps: E += cs * source
};

// Drude + 2 critical points (and the graphene Drude + Raman/Kerr variant)
// The recursions are carried in delta form, with the small deltas computed
// once in FP64 on the host: a decay factor ha = exp(-g dt) ~ 1 - 3.6e-4
// rounded to FP32 would perturb its decay rate 1 - ha by ~1e-4.
template <typename T>
struct AdeCoef {
  int kind;
  int normal;              // graphene sheet normal axis (in-plane comps updated)
  T ha, hb, dha;           // Drude: S += hb*E - dha*S (dha = 1-ha), Q -= hb*E
  T dr[kMaxCp], di[kMaxCp];   // CP p: g += (gb-1)*g + gc*E, d = gb-1
  T gcr[kMaxCp], gci[kMaxCp]; // CP drive (gold: p < 2)
  T wr, wi;                // gold: 1/ga (E = Re(num * (wr + i wi)))
  T gar, gai;              // 4-CP graphene: ga, E = Re(num / (ga + S_R))
  T r0, rv, rs, kerr, ga;  // graphene Raman in velocity form: V = rv*V + rs*SR + r0*E^2,
                           // SR += V (rv = 1-(1+r2), rs = (r1-2)+(1+r2)); Kerr; eps
                           // (Lorentz: ga = 1/eps_inf)
  int npoles;              // Lorentz: per pole l, with p = c0 P and v = p(n)-p(n-1):
  T lv[kMaxPoles];         //   v += -lv v + (le E - ls p);  p += v
  T ls[kMaxPoles];         //   lv = 2 nu dt/(1+nu dt), ls = (w dt)^2/(1+nu dt),
  T le[kMaxPoles];         //   le = deps ls
  int zx;                  // Lorentz: Ez takes the x current (SLG_LJp)
  int nl;                  // Lorentz sheet with a Kerr term on pole 0:
  T lk;                    //   drive of pole 0 += lk Q E, lk = ls[0] chi3
  T lqv, lqs, escale;      //   g += -lqv g + lqs ((escale E)^2 - Q);  Q += g
};

struct Source {
  int comp;                // 0..2 (E component) or 6 (1D incident line)
  int lo[3], hi[3];
  double amp;
};

struct Monitor {
  int lo[3], hi[3];
  int ncomp, comps[6];
  int ncell;
  long long base;          // first index of this monitor in the stage row
  int n_first, n_last;
  int nfreq;
  long long acc;           // offset of this monitor's accumulators
  int freq_off;            // offset into the omega table
  int mean;                // 1: one sample per component, the box mean
  int boxcells;            // cells of the box
  int mrows;               // mean: x-rows of the box summed per block
  int mchunks;             // mean: blocks per component (ceil(rows / mrows))
  int mpart;               // mean: first partial-sum slot (and counter) of
                           // this monitor's components, mchunks per component
};

struct Probe {
  int cell[3];
  int ncomp, comps[8];
  int n_first, n_last;
  double *buf;             // device buffer: [step - n_first][comp]
  int cap;                 // steps of capacity
};

// Everything a step kernel needs, passed by value.
template <typename T>
struct StepParams {
  // geometry
  int layout;              // FDTD_LAYOUT_*
  int nx, ny, nz;
  int per[3];
  int mlo[3], mhi[3];      // main (Yee) range
  T ku;
  // fields (E/H components; null when the layout lacks them)
  T *ex, *ey, *ez, *hx, *hy, *hz;
  // where the 3D edge, ADE and fused kernels store what they update: the same
  // arrays (in place), or with pp the other buffer of a ping-pong pair, in
  // which case every cell a kernel owns is stored, updated or not.  E half:
  // E^n read from ex.., E^{n+1} stored to exo..; H half: ex.. hold E^{n+1},
  // H^n read from hx.., H^{n+1} stored to hxo..
  T *exo, *eyo, *ezo, *hxo, *hyo, *hzo;
  int pp;
  const uint8_t *mat;      // material id per cell: 0 none, 1..127 constant
                           // dielectric, 128..255 dispersive (ADE slots)
  const MatCoef<T> *mc;
  const T *mca, *mcs;      // per id: Ku/eps and 1/eps (0 for none and ADE ids)
  int id0;                 // most common material id of the main cells and
  T ca0;                   //   its Ku/eps (no table lookup for it)
  const uint8_t *rowflag;  // per x-row, ROW_* bits: 2D [j], 3D [k*ny + j]
  const uint32_t *uni;     // 3D, per x-vector of vec cells: bit v of word [row*uni_words + v/32] is 1
  int uni_words;           //   when every cell of the vector has id id0 (its ids need no load)
  // ADE slots
  int nade;
  const int *ade_cell;     // linear cell index
  const uint8_t *ade_mat;  // material id
  const AdeCoef<T> *ac;
  AdeCoef<T> acp[4];       // the first dispersive materials' coefficients
  int ade_kind;            // the device kind (MatKind) of every dispersive material, or -1
  T *ade_state;            // [field][comp][slot], see AdeState
  int ade_stride;          // = padded nade
  // sources: boxes, and amp*g(t) of every step in a device table
  int nsrc;
  Source src[kMaxSrc];
  const double *srcval_tab;  // [(n-1)*nsrc + q]
  // PML
  int pml_mode;            // 0 none, 1 reference slabs, 2 split
  // split-field PML on any faces: shell = outside [slo, shi]
  int slo[3], shi[3];
  const T *cf1[3], *cf2[3], *cg1[3], *cg2[3];   // per-axis tables (len n[a])
  T *sp[12];               // stored sub-fields (3D: Exy Eyz Ezx Hxy Hyz Hzx;
                           // 2D TM: Ezx; 2D TE: Hzx).  FP64 also stores the
                           // other parts in sp[6+q] (Exz Eyx Ezy Hxz Hyx Hzy /
                           // Ezy / Hzy); FP32 takes them as total - part.
  T *spo[3];               // the fused 2D step: where sp[0..2] of step n+1 go
                           // (the other buffer of a ping-pong pair)
  // reference y-slabs (2D: Ex Ey Hzx Hzy; 3D: 12 split arrays) per side
  int slab_on[2];
  int slab_j0[2];          // first 0-based row of the slab
  int slab_rows;           // npmly
  T *slab[2][12];
  const T *sf1x[2], *sf2x[2], *sg1x[2], *sg2x[2];  // per side, len nx
  const T *sf1y[2], *sf2y[2], *sg1y[2], *sg2y[2];  // per side, len rows
  const T *sf1z[2], *sf2z[2], *sg1z[2], *sg2z[2];  // per side, len nz
  // work split of one launch
  int roles;               // ROLE_* bits
  int ntile_blocks;        // edge blocks of the general launch (3D)
  int nslab_blocks, nade_blocks;
  // 2D work split: core units are vectors [cv0, cv0+cw) of rows cy0.. (ncore
  // units in all); every other unit (j*nx/V + vector) is listed in edge_units
  int cv0, cw, cy0, ncore;
  int nedge;
  const int *edge_units;
  // 3D: the core box is vectors [cv0, cv0+cw) x rows [cy0, cy0+ch) x planes
  // [cz0, cz0+cd); edge_units are then x-vectors (k*ny + j)*nx/V + vector
  int ch, cz0, cd;
  int tile;                // block shape of the core kernels (tuned; 3D 6: the TMA-staged E core)
  const struct TmaMaps *tma;  // host copy of the H planes' tensor maps, for the launcher (or null)
  int *err;                // device flag: a bounded wait of a kernel gave up (nonzero)
  unsigned wait_limit;     // polls of an mbarrier before a main-loop wait gives up
  // sampling fused into the H kernel
  int gather;              // 1: tile threads write the stage row / probes
  int nmon;
  Monitor mon[kMaxMon];
  T *stage;                // [slot][sample]
  long long stage_row;     // samples per step
  int slot;                // ring slot of this step
  int nprobe;
  Probe probe[kMaxProbe];
  int n;                   // step number (eager launches)
  const int *d_base;       // graph replays: step number of ring slot 0 on the
                           // device; then n = *d_base + slot
  const int *d_half;       // graph replays: which half of the two-ring stage
                           // buffer this ring writes, on the device (null: stage
                           // already points at the ring's half)
  int vec;                 // cells per thread along x in the 2D tile path
  double *mean_part;       // mean monitors: FP64 partial sums per block
  unsigned *mean_ctr;      // mean monitors: blocks done per component
  // 2D/3D total-field/scattered-field box (plane wave along +y)
  int tf_on;
  int tf_lo[3], tf_hi[3];  // total-field box, inclusive cells
  int tf_face[3];          // 1: the box has the two faces normal to the axis
  T tf_cb, tf_sign;        // line E coefficient Ku/eps_line; +1 Ex/Hz, -1 Ez/Hx
  T *tf_e, *tf_h;          // incident line E and H (ny values)
  T *tf_abc;               // two-step absorbing ends: low m1 m2, high m1 m2
};

// per-row flags of the 2D tile path (precomputed from the job's set-up)
enum RowFlag : int { ROW_SRC = 1, ROW_SAMPLE = 2, ROW_SLAB = 4 };
constexpr int kAdeId = 128;  // material ids >= kAdeId are dispersive;
                             // id - kAdeId indexes the ADE coefficient table
constexpr int kAdeParam = 4; // ADE coefficient sets passed as kernel parameters

enum Role : int {
  ROLE_MAIN = 1,  // Yee update + materials on main cells
  ROLE_PML = 2,   // PML (slabs or shell)
  ROLE_ADE = 4,   // dispersive slots
};

// ADE state layout: state[(f*3 + comp)*stride + slot] with fields
// 0:Q (=D-I)  1:S  2:g1r 3:g1i 4:g2r 5:g2i  (graphene: 2:S_R 3:V = S_R(n)-S_R(n-1);
// Lorentz: 2l: p_l, 2l+1: v_l for pole l < npoles; with a Kerr term
// 2P: Q, 2P+1: g = Q(n)-Q(n-1); with zx, 2P+2 (component 0) holds the x
// current sum for the z update; 4-CP graphene: 2+2p, 3+2p:
// g_p for p < 4, 10: S_R, 11: V).  A job allocates the fields its materials
// use (ade_fields), at most kAdeFields.
constexpr int kAdeFields = 12;
constexpr int ade_fields(int kind, int npoles, int nl, int zx) {
  return kind == MK_GOLD || kind == MK_CONDUCTIVE ? 6
       : kind == MK_GRAPHENE || kind == MK_GRAPHENE_NK ? 4
       : kind == MK_GRAPHENE_CP ? 12
       : kind == MK_LORENTZ ? (zx ? 2 * npoles + 3 : nl ? 2 * npoles + 2 : 2 * npoles)
       : 0;
}

// launchers (defined in k2d.cu / k3d.cu / k1d.cu / kdft.cu)
// 2D half steps: the parts of one half step are independent launches
enum K2dPart { K2D_CORE = 0, K2D_EDGE = 1, K2D_ADE = 2 };
// prog_event: the core kernel records it as a programmatic event (or null)
template <typename T> int launch_e2d(const StepParams<T> &p, int part, void *stream, void *prog_event = nullptr);

// the dispersive cells' E update with a programmatic dependency on the kernel
// before it (the first launch of a fused 2D step); returns the kernels launched
template <typename T> int launch_e2d_ade_pdl(const StepParams<T> &p, void *stream);
// the fused 2D step kernel (k2f.cu, TMz, FP32): E^{n+1} and H^{n+1} of every
// cell in one pass, reading ez, hx, hy, sp[0] and storing to ezo, hxo, hyo,
// spo[0]; returns the kernels launched
int launch_step2d_fused(const StepParams<float> &p, void *stream);

// packs of 2D jobs: one launch runs one part of every job's half step
constexpr int kMaxPack = 32;
template <typename T>
struct PackLaunch {
  const StepParams<T> *tab;  // one StepParams per job (this ring slot)
  int njobs;
  int bstart[kMaxPack + 1];  // first block of each job; bstart[njobs] = blocks
};
template <typename T>
int launch_pack2d(const PackLaunch<T> &a, int layout, int vec, bool e_half, int part, void *stream);
template <typename T> int launch_h2d(const StepParams<T> &p, int part, void *stream, void *prog_event = nullptr);
template <typename T> int launch_e3d(const StepParams<T> &p, int part, void *stream, void *prog_event = nullptr);
template <typename T> int launch_h3d(const StepParams<T> &p, int part, void *stream, void *prog_event = nullptr);
// the 3D general kernels (edge units, slabs, ADE cells) on the job's stream
// with a programmatic dependency, for the serial order of a fused step
template <typename T> int launch_e3d_general_pdl(const StepParams<T> &p, void *stream);
template <typename T> int launch_h3d_general_pdl(const StepParams<T> &p, void *stream);
// the fused 3D step kernel (k3f.cu): E^{n+1} and H^{n+1} of the core box in
// one pass, reading buffer ex.. (maps m) and storing to exo.. (ping-pong)
int launch_step3d_fused(const StepParams<float> &p, const FusedMaps &m, void *stream);
// blocks and dynamic shared memory of one launch
void step3d_fused_shape(const StepParams<float> &p, int *blocks, int *smem);

// separate gather (per-procedure API, or monitors inside reference slabs)
// returns the kernels launched
template <typename T> int launch_gather(const StepParams<T> &p, void *stream);
// total-field/scattered-field box: incident line and face terms of a half step
// kcheck.cu: count the non-finite float (esz 4) or double (esz 8) values of a buffer
int launch_count_nonfinite(const void *p, size_t bytes, int esz, unsigned long long *out, int num_sms, void *stream);
template <typename T> int launch_tfsf(const StepParams<T> &p, bool e_half, void *stream);

// DFT fold: acc += sum over valid ring slots of e^{i w t} * sample * dt
struct DftParams {
  int nmon;
  Monitor mon[kMaxMon];
  const double *omega;     // all monitors' frequencies
  const double2 *rot;      // per frequency, e^{i w s dt} for s < kStageSteps;
                           // null: one sincos per (frequency, slot)
  double *acc_re, *acc_im; // FP64 accumulators
  int nslots;              // valid slots in this fold (0..kStageSteps)
  int n0;                  // step number of slot 0 (eager launches)
  const int *d_base;       // graph replays: slot-0 step number on the device
  const int *d_half;       // graph replays: the ring's half of the stage buffer
                           // on the device (null: stage points at the ring)
  int prev;                // graph replays: fold the ring before this one (the
                           // other half, slot 0 at *d_base - kStageSteps)
  const int *gate;         // graph replays: 0 on the device: nothing to fold
  double dt;
  long long stage_row;
  int total_work_blocks;
};
template <typename T> void launch_dft(const DftParams &d, const T *stage, void *stream);
// load the DFT fold kernel on the current device now (cudaFuncGetAttributes)
// rather than at its first launch; 0 on success
template <typename T> int preload_dft();

// 1D line: persistent single-block kernel running many steps
template <typename T>
struct LineParams {
  int N;                   // cells
  int mlo, mhi;            // main range
  T ku;
  T *ex, *hz, *dx;         // main line (dx only used for ADE cells)
  T *exi, *hzi;            // incident line (TFSF) or null
  int tfsf_bd;             // 0-based TFSF boundary cell (-1 none)
  const uint8_t *mat;
  const MatCoef<T> *mc;
  const AdeCoef<T> *ac;
  int nac;                 // entries of ac
  int nade;
  const int *ade_cell;
  const uint8_t *ade_mat;
  T *ade_state;
  int ade_stride;
  int ade_nf;              // state fields per component in use
  // reference PML, per side and line (0 main, 1 incident)
  int slab_on[2];
  int ja, jb;              // 0-based: low slab rows [0, ja], high [jb, N-1]
  T *pex[2][2], *phz[2][2];      // [line][side] slab arrays incl. coupling row
  const T *f1[2][2], *f2[2][2], *g1[2][2], *g2[2][2];
  // sources: values for every step of the launch
  int nsrc;
  Source src[kMaxSrc];
  const double *srcval;    // [step][src]
  // sampling
  int nmon;
  Monitor mon[kMaxMon];
  const double *omega;
  double *acc_re, *acc_im;
  int nprobe;
  Probe probe[kMaxProbe];
  double dt;
  int n_first, n_steps;
  int stages;              // bit0: E half, bit1: H half, bit2: sample
};
template <typename T> void launch_line1d_stage(const LineParams<T> &p, T *stage, long long stage_row, void *stream);

// Records a message for fdtd_last_error and returns `code`.
int report_error(int code, const char *fmt, ...);

// Packs of 2D jobs advanced by shared launches (fdtd_api.cu).  pack_key is
// -1 for a job that cannot join a pack (not a committed 2D job at a ring
// boundary) and otherwise equal for jobs that can share one.  job_reserve
// sizes a job's source table and probe buffers for steps up to n_last, as a
// pack bakes their addresses into its tables.  pack_run queues `rings`
// rings of every member on the pack's stream and records `done` after them.
struct Pack;
long long pack_key(const fdtd_job *J);
int job_reserve(fdtd_job *J, int n_last);
int pack_create(fdtd_job *const *jobs, int njobs, Pack **out);
int pack_run(Pack *P, int rings, cudaEvent_t done);
void pack_destroy(Pack *P);

}  // namespace fdtd
