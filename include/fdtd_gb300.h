/*
 * fdtd_gb300.h -- C ABI of the GB300 (sm_103a) FDTD time-step engine.
 *
 * The engine replaces the body of the reference's time loop
 * (FDTDsimulations/3D/air-AuAntennasSiO2-Si/program.f90:382-607,
 *  FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate/program.f90:320-471,
 *  FDTDsimulations/1D/TFSF-air_SLG_SiO2_Sidisp/program.f90:217-308):
 * the Yee curls (updateD/updateH), the material D->E updates
 * (ConstantDielectric, Gold Drude+2CP ADE, graphene sheet), the split-field
 * PML (pmly%updateE / pmly%updateH), the halo exchanges (interchange_E/H,
 * which become in-memory neighbours of one domain), the soft source and the
 * running DFT monitors.
 *
 * Conventions
 *  - Every function returns an int status: FDTD_OK (0) or an FDTD_E* code.
 *    fdtd_last_error() copies a message describing the last failure of the
 *    calling thread.
 *  - Device memory belongs to the job handle; the caller only passes host
 *    pointers.  Calls are asynchronous on the job's CUDA stream; getters and
 *    fdtd_sync() wait for it and report deferred device errors.
 *  - One host thread may use a job at a time; different jobs may be driven
 *    from different threads.
 *  - Cell indices are 0-based: reference index i maps to i-1.  Arrays passed
 *    in or out are x-fastest (Fortran column-major, like the reference's).
 *  - Time step numbers n are 1-based like the reference's `do n=1,Nt`; the
 *    field time inside step n is t = (n-1)*dt.
 *  - There is no CPU fallback: without a usable GB300 the calls that need
 *    the device return FDTD_ENODEV.
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
  FDTD_OK = 0,
  FDTD_EINVAL = 1,  /* bad argument or descriptor                       */
  FDTD_ENOMEM = 2,  /* device or host allocation failed                 */
  FDTD_ECUDA = 3,   /* a CUDA call or kernel failed                     */
  FDTD_ESTATE = 4,  /* call not valid in the job's current state        */
  FDTD_ERANGE = 5,  /* index or size out of range                       */
  FDTD_ENODEV = 6   /* no usable sm_103a device                         */
};

/* ---- grid layouts ------------------------------------------------------ */
enum {
  FDTD_LAYOUT_1D = 1,    /* Ex, Hz along y: 1D/.../program.f90:42-45          */
  FDTD_LAYOUT_2D_TE = 2, /* Ex, Ey, Hz in x-y: 2D/.../program.f90:68         */
  FDTD_LAYOUT_2D_TM = 3, /* Ez, Hx, Hy in x-y: the 3D equations with d/dz=0 */
  FDTD_LAYOUT_3D = 4     /* Ex..Hz: 3D/.../program.f90:77                   */
};

enum { FDTD_F32 = 1, FDTD_F64 = 2 };

/* Field components.  The *_INC codes address the auxiliary incident line of
 * a total-field/scattered-field set-up: the 1D line (1D/.../program.f90:45)
 * or the line of a 2D/3D box (fdtd_add_tfsf), whose E and H are FDTD_E_INC
 * and FDTD_H_INC. */
enum {
  FDTD_EX = 0, FDTD_EY = 1, FDTD_EZ = 2,
  FDTD_HX = 3, FDTD_HY = 4, FDTD_HZ = 5,
  FDTD_EX_INC = 6, FDTD_HZ_INC = 7,
  FDTD_E_INC = 6, FDTD_H_INC = 7
};

typedef struct fdtd_grid_desc {
  int32_t layout;       /* FDTD_LAYOUT_*                                    */
  int32_t precision;    /* FDTD_F32 or FDTD_F64 storage and arithmetic      */
  int32_t n[3];         /* cells along x, y, z (1 for unused axes)          */
  int32_t periodic[3];  /* 1 = periodic wrap on that axis (PBC_x, PBC_z)    */
  int32_t main_lo[3];   /* inclusive range of the Yee update (locI*range,   */
  int32_t main_hi[3];   /*   3D/.../include/mympi_func.f90:137-214)         */
  double ku;            /* Courant factor of the curls (Ku)                 */
  double dt;            /* time step [s]                                    */
  double ds;            /* cell size [m]                                    */
} fdtd_grid_desc;

/* ---- geometry of materials ------------------------------------------- */
enum {
  FDTD_REGION_BOX = 0,     /* axis-aligned box (the reference's xinit..zend) */
  FDTD_REGION_SPHERES = 1, /* union of spheres (3D) or cylinders (2D)        */
  FDTD_REGION_MASK = 2     /* explicit per-cell mask                          */
};

typedef struct fdtd_region {
  int32_t kind;
  int32_t lo[3], hi[3];          /* BOX: inclusive cell range              */
  int32_t count;                 /* SPHERES: number of (cx,cy,cz,r) rows   */
  const double *centers_radii;   /* SPHERES: cell (i,j,k) is inside when
                                    (i+.5-cx)^2+(j+.5-cy)^2[+(k+.5-cz)^2]
                                    <= r^2 (z term absent in 2D)           */
  const uint8_t *mask;           /* MASK: n[0]*n[1]*n[2] bytes, x fastest  */
} fdtd_region;

/* Drude + two critical points (2D/gold_mod.f90:25-31, 3D/gold_mod.f90:28-34).
 * Angular frequencies and dampings in rad/s. */
typedef struct fdtd_drude2cp {
  double eps_inf;
  double omega_d, gamma_d;
  double amp[2], phi[2], omega[2], gamma[2];
} fdtd_drude2cp;

/* Graphene sheet: intraband Drude surface conductivity from the Fermi level
 * and relaxation time, plus a Kerr + Raman-delayed third-order response
 * (1D/graphene633_mod.f90:26-44, 3D/graphene_mod.f90:202-262).  The sheet is
 * one cell thick; its in-plane E components get the update. */
typedef struct fdtd_graphene_desc {
  double fermi_ev;      /* E_F [eV]                                        */
  double tau;           /* relaxation time [s]                             */
  double temperature;   /* [K]                                             */
  double chi3;          /* third-order susceptibility [m^2/V^2]            */
  double raman_frac;    /* fraction of chi3 that is Raman-delayed          */
  double raman_freq;    /* Raman line centre [Hz]                          */
  double raman_tau;     /* Raman damping time [s]                          */
  double thickness;     /* physical sheet thickness [m] (surface -> bulk)  */
  double e_scale;       /* V/m per normalised field unit (for chi3 E^2)    */
} fdtd_graphene_desc;

/* Lorentz poles (up to FDTD_LORENTZ_MAX_POLES), in either of the reference's
 * two codings of the same discrete recursion:
 *   FDTD_LORENTZ_JP  the polarisation-current form of gold_LJp, si_LJp,
 *                    Ti_LJp and filmgold_LJp (3D/goldLorentzJp_mod.f90:37-91,
 *                    3D/siLorentzJp_mod.f90:41-96, 3D/titaniumJp_mod.f90:37-91,
 *                    2D/siLorentzJp_mod.f90:40-80):
 *                      E += Ku/eps_inf (curl H - ds sum_l Jp_l)
 *                      Jp_l = g1 Jp_l + g2 (xi_l E/c0 - P_l);  P_l += dt Jp_l
 *                    g1 = (1 - nu dt)/(1 + nu dt), g2 = w0^2 dt/(1 + nu dt)
 *   FDTD_LORENTZ_S   the second-order form of Si (3D/si_mod.f90:46-82,
 *                    1D/si_mod.f90:38-53), D-form with E = (D - sum_l S_l)/eps_inf
 *                    (eps_inf = 1 in the reference):
 *                      S_l(n) = ga S_l(n-1) + gb S_l(n-2) + gc E(n)
 *                    ga = (2 - (w dt)^2)/(1 + nu dt), gb = (nu dt - 1)/(1 + nu dt),
 *                    gc = deps (w dt)^2/(1 + nu dt)
 * delta_eps is xi1 / dep, omega is w0l / wp and gamma is dnu0l / dnup, all
 * angular [rad/s].  Signs are taken as given (the reference's fits have
 * negative w0 and nu for some poles).
 *
 * sheet = 1 makes it the Lorentz-Jp graphene sheet of SLG_3LJp1nm
 * (3D/graphene3LorentzJp1nm_mod.f90:42-100, 2D/graphene3LorentzJp1nm_mod.f90:
 * 42-80): the region is a one-cell-thick box, its in-plane components take
 * the Jp update and its normal component the vacuum one (E += Ku curl H).
 * chi3 != 0 adds the delayed Kerr term of its first pole (JP form):
 * P0_1 = (xi1 + chi3 Q) E/c0, with
 *   G = g1NL G + g2NL ((e_scale E)^2 - Q);  Q += dt G,
 * g1NL, g2NL built from w_nl and gamma_nl like g1, g2 (xi3, wNL, dnuNL, and
 * z0 for e_scale, in the reference).  The 4-pole SLG_LJp
 * (3D/grapheneLorentzJp_mod.f90:42-100) is the same sheet, except that its
 * Ez line subtracts JpxT, the x current of the previous step, where the
 * 3-pole module subtracts JpzT (:68); ez_uses_x_current = 1 reproduces that
 * (JP form, 3D grids, a sheet normal to y as in the reference: Ex and Ez
 * in-plane). */
enum { FDTD_LORENTZ_JP = 0, FDTD_LORENTZ_S = 1 };
#define FDTD_LORENTZ_MAX_POLES 4
typedef struct fdtd_lorentz_desc {
  int32_t form;          /* FDTD_LORENTZ_JP or FDTD_LORENTZ_S            */
  int32_t npoles;        /* 1..FDTD_LORENTZ_MAX_POLES                    */
  double eps_inf;
  double delta_eps[FDTD_LORENTZ_MAX_POLES];
  double omega[FDTD_LORENTZ_MAX_POLES];
  double gamma[FDTD_LORENTZ_MAX_POLES];
  int32_t sheet;         /* 1: one-cell-thick sheet, in-plane update only */
  int32_t ez_uses_x_current; /* 1: Ez takes JpxT (SLG_LJp)                */
  double chi3;           /* xi3 [m^2/V^2]; 0: linear                      */
  double w_nl, gamma_nl; /* wNL, dnuNL [rad/s]                            */
  double e_scale;        /* V/m per normalised field unit (z0)            */
} fdtd_lorentz_desc;

/* The reference's own graphene, Graphene: Drude plus four critical points,
 * scaled from the physical layer width to the cell, with a Raman-delayed
 * third-order term in the denominator (3D/graphene_mod.f90:59-105, 202-283;
 * 2D/graphene_mod.f90:56-92, 163-236; 1D/graphene_mod.f90:52-71, 126-183):
 *   E = Re[(D - I + ha S + sum_p gb_p g_p) / (gax + S_R)]
 *   S_R(n) = r1 S_R(n-1) + r2 S_R(n-2) + r0 E(n)^2
 *   I += hb E;  S = ha S + hb E;  g_p = gb_p g_p + gc_p E
 * with s = width/ds, ha = exp(-drude_gamma dt), hb = s drude_omega^2 dt /
 * drude_gamma, gb_p = exp((-gamma_p + i omega_p) dt),
 * gc_p = 2 i dt (s amp_p) omega_p exp(-i phi_p), gax = eps_inf - sum_p gc_p.
 *   FDTD_RAMAN_EXACT    r0 = chi3 wR dt e^{-aR dt} sin(bR dt), r1 = 2 e^{-aR dt}
 *                       cos(bR dt), r2 = -e^{-2 aR dt}; aR = gamma_nl/2,
 *                       bR = sqrt(w_nl^2 - aR^2), wR = w_nl^2/bR (3D module)
 *   FDTD_RAMAN_CENTRAL  r0 = chi3 (w_nl dt)^2/(1 + gamma_nl dt), r1 = (2 -
 *                       (w_nl dt)^2)/(1 + gamma_nl dt), r2 = -(1 - gamma_nl dt)/
 *                       (1 + gamma_nl dt) (2D module)
 * chi3 = 0 drops the Raman term (the 1D module).  chi3 multiplies the
 * normalised E^2 of the update, as xi3 does in the reference.  The component
 * along normal_axis is vacuum (E = D): the 2D module sets Ey = Dy, and the 3D
 * one updates Ex and Ez only, so normal_axis = 1 (y) is the reference's
 * sheet; -1 updates every component. */
/* The reference's 1D graphene at 633 nm, graphene633 (1D/graphene633_mod.f90:
 * 26-105): a conductive layer from its refractive index n + ik at one
 * wavelength, with the linearised Kerr term of an instantaneous fraction
 * alpha of chi3 and a Raman-delayed rest:
 *   E = (D - I + 2 chi3 alpha E^3) / (ga + S_R + 3 chi3 alpha E^2),  I += gb E
 *   S_R(n) = r1 S_R(n-1) + r2 S_R(n-2) + r0 E(n)^2
 * where E on the right is the previous step's; sigma = sqrt(s) 4 pi n k c0
 * eps0 / wavelength, eps_inf = s (n^2 - k^2), ga = eps_inf + sigma dt/eps0,
 * gb = sigma dt/eps0 (s = scale), and r0 = (1 - alpha) chi3 wR dt
 * e^{-gamma_nl dt} sin(bR dt), r1 = 2 e^{-gamma_nl dt} cos(bR dt),
 * r2 = -e^{-2 gamma_nl dt}, bR = sqrt(w_nl^2 - gamma_nl^2), wR = w_nl^2/bR
 * (this module damps with gamma_nl where the 3D Graphene takes gamma_nl/2).
 * Every E component of the layout takes the update. */
typedef struct fdtd_graphene_nk_desc {
  double n, k;              /* refractive index of the layer (the module's 2.731108, 1.357) */
  double wavelength;        /* [m] (633e-9)                                    */
  double scale;             /* scaleFactor                                     */
  double chi3, alpha;       /* xi3 and its instantaneous fraction              */
  double w_nl, gamma_nl;    /* wNL [rad/s], dnuNL [1/s]                         */
} fdtd_graphene_nk_desc;

enum { FDTD_RAMAN_EXACT = 0, FDTD_RAMAN_CENTRAL = 1 };
typedef struct fdtd_graphene_cp_desc {
  double eps_inf;                 /* graphene_epinf                          */
  double drude_omega;             /* graphene_wD [rad/s]                     */
  double drude_gamma;             /* graphene_dnur [1/s]                     */
  double amp[4], phi[4];          /* ap, phip                                */
  double omega[4], gamma[4];      /* omp, rp [rad/s]                         */
  double width;                   /* Graphenewidth [m]                       */
  double chi3;                    /* xi3; 0: no Raman term                   */
  double w_nl, gamma_nl;          /* wNL [rad/s], dnuNL [1/s]                */
  int32_t raman_form;             /* FDTD_RAMAN_EXACT or FDTD_RAMAN_CENTRAL  */
  int32_t normal_axis;            /* 0, 1, 2, or -1 for none                 */
} fdtd_graphene_cp_desc;

/* ---- PML ---------------------------------------------------------------- */
enum {
  FDTD_PML_REFERENCE = 1, /* the reference's y-slab split-field PML with its
                             copy-in/copy-out coupling: 1D/BERpmly_ExHz_mod,
                             2D/BERpmly_HzExEy_mod, 3D/BERpmly_mod            */
  FDTD_PML_SPLIT = 2      /* split-field PML on any set of faces; the same
                             graded profiles applied per axis                 */
};

typedef struct fdtd_pml_desc {
  int32_t mode;
  int32_t npml[3][2];  /* thickness per axis, [low, high] side.  REFERENCE:
                          npml[1][*] = slab thickness (npmly); npml[0][0] and
                          npml[2][0] = corner profile widths (npmlx, npmlz)  */
  double eps_lo;       /* relative permittivity of the low-y (REFERENCE) or
                          of every (SPLIT) PML medium (eplow/ep0)           */
  double eps_hi;       /* relative permittivity of the high-y slab          */
  double sigma_max;    /* sigmam [S/m] (3D/.../program.f90:102)            */
  double order;        /* grading order (3 in the reference)               */
} fdtd_pml_desc;

/* ---- sources, monitors, probes ------------------------------------------ */
/* Soft source added to D over a box of cells after the curl update
 * (3D/.../program.f90:396-406):  g(t) = exp(-0.5((t-t0)/st)^2) sin(w0 t). */
typedef struct fdtd_source_desc {
  int32_t component;    /* FDTD_EX..FDTD_EZ, or FDTD_EX_INC (1D TFSF line) */
  int32_t lo[3], hi[3]; /* inclusive cell box                              */
  double amp;           /* scale (n_air in 3D/.../program.f90:403)         */
  double t0, st, w0;
} fdtd_source_desc;

/* Running DFT over a box of cells (3D/.../program.f90:441-540):
 *   re += cos(omega_m t) F dt,  im += sin(omega_m t) F dt,  t = (n-1) dt
 * sampled after the H update of step n, for n_first <= n <= n_last. */
typedef struct fdtd_monitor_desc {
  int32_t lo[3], hi[3];  /* inclusive cell box (plane, line or point)      */
  int32_t comp_mask;     /* bit c = transform component c (FDTD_EX..)      */
  int32_t n_first, n_last;
  int32_t nfreq;
  const double *omega;   /* nfreq angular frequencies (arg(m))             */
  int32_t reduce;        /* FDTD_MONITOR_CELLS: every cell of the box;
                            FDTD_MONITOR_MEAN (2D/3D): the box mean of each
                            component, one value per component and
                            frequency (the DFT of a plane-averaged field)  */
} fdtd_monitor_desc;
enum { FDTD_MONITOR_CELLS = 0, FDTD_MONITOR_MEAN = 1 };

/* Per-step samples at one cell (the r*infld/rfld/tfld time series,
 * 2D/.../program.f90:376-419). */
typedef struct fdtd_probe_desc {
  int32_t cell[3];
  int32_t comp_mask;
  int32_t n_first, n_last;
} fdtd_probe_desc;

/* 1D total-field/scattered-field boundary (1D/.../program.f90:221-262). */
typedef struct fdtd_tfsf1d_desc {
  int32_t boundary;     /* TFSF_bd, 0-based                                */
  double eps_lo, eps_hi;/* relative permittivities of the incident line's PML */
} fdtd_tfsf1d_desc;

typedef struct fdtd_job fdtd_job;

/* ---- lifetime ---------------------------------------------------------- */
/* Replaces the program's static field arrays and my_mpi_init/set_index
 * (3D/.../program.f90:77, include/mympi_func.f90:86-214). */
int fdtd_create(const fdtd_grid_desc *grid, fdtd_job **out);
int fdtd_destroy(fdtd_job *job);
int fdtd_last_error(char *buf, size_t len);
/* Number of sm_103a devices the library can use (0 without a GPU). */
int fdtd_device_count(int32_t *count);

/* ---- set-up (host side, before fdtd_commit) ------------------------------ */
/* mat%initialize_material (2D/simpledielectric_mod.f90:150-187,
 * 3D/simpledielectric_mod.f90:52-103).  Materials paint cells in call order;
 * a later material overrides an earlier one on shared cells, as the
 * reference's call order of update_E does (3D/.../program.f90:411-414). */
int fdtd_add_dielectric(fdtd_job *job, const fdtd_region *region, double eps_r,
                        int32_t *material_id);
/* Gold%initialize_material (2D/gold_mod.f90:77-168, 3D/gold_mod.f90:90-195). */
int fdtd_add_gold(fdtd_job *job, const fdtd_region *region,
                  const fdtd_drude2cp *params, int32_t *material_id);
/* Graphene sheet (3D/graphene_mod.f90:59-269, 1D/graphene633_mod.f90:26-105). */
int fdtd_add_graphene(fdtd_job *job, const fdtd_region *region,
                      const fdtd_graphene_desc *params, int32_t *material_id);
/* gold_LJp / si_LJp / Ti_LJp / filmgold_LJp%initialize_material and
 * Si%initialize_material (3D/goldLorentzJp_mod.f90:93-161,
 * 3D/si_mod.f90:84-206).  Every E component of the layout gets the update. */
int fdtd_add_lorentz(fdtd_job *job, const fdtd_region *region,
                     const fdtd_lorentz_desc *params, int32_t *material_id);
/* SiL800%initialize_material (3D/siL800_mod.f90:53-104): a conductive
 * dielectric, E = (D - I)/ga, I += gb E, ga = eps_inf + sigma dt/eps0,
 * gb = sigma dt/eps0 (sigma in S/m), on every E component.  The reference's
 * update_E_inSi writes its Ey pair twice and never Ez (:42-46); the intended
 * update of all three components is built. */
int fdtd_add_conductive(fdtd_job *job, const fdtd_region *region, double eps_inf,
                        double sigma, int32_t *material_id);
/* graphene633%initialize_material (1D/graphene633_mod.f90:48-105). */
int fdtd_add_graphene_nk(fdtd_job *job, const fdtd_region *region,
                         const fdtd_graphene_nk_desc *params, int32_t *material_id);
/* Graphene%initialize_material (3D/graphene_mod.f90:107-283,
 * 2D/graphene_mod.f90:94-236, 1D/graphene_mod.f90:73-183). */
int fdtd_add_graphene_cp(fdtd_job *job, const fdtd_region *region,
                         const fdtd_graphene_cp_desc *params, int32_t *material_id);
/* pmly%initialize (3D/BERpmly_mod.f90:485-508, 2D/BERpmly_HzExEy_mod.f90:229-247,
 * 1D/BERpmly_ExHz_mod.f90:163-175). */
int fdtd_add_pml(fdtd_job *job, const fdtd_pml_desc *pml);
int fdtd_add_tfsf_1d(fdtd_job *job, const fdtd_tfsf1d_desc *tfsf);
/* Total-field/scattered-field box for a plane wave along +y (2D and 3D).
 * The incident wave runs on an auxiliary line along y (cells 0..ny-1),
 * driven by FDTD_E_INC sources at row lo[1] of their box, with the two-step
 * absorbing ends of a Ku = 0.5 line (exact in vacuum at Ku = 0.5).  Each face
 * of the box adds the incident term to the updates that cross it, as
 * consistCond_dy/dz/hx/hy do for Ez/Hx incidence
 * (3D/.../include/myTFSF_incEzHx_3Dfunc.f90:80-221): 3D and 2D TM carry Ez/Hx,
 * 2D TE carries Ex/Hz.  The total field holds Ez (Ex in TE) at cells lo..hi;
 * a periodic axis that the box spans end to end has no faces.  Face cells
 * must be non-dispersive main cells outside the PML.  FDTD_E_INC/FDTD_H_INC
 * address the line in fdtd_get_field (ny values). */
typedef struct fdtd_tfsf_desc {
  int32_t lo[3], hi[3];  /* total-field box, inclusive cells               */
  double eps_line;       /* relative permittivity of the incident line     */
} fdtd_tfsf_desc;
int fdtd_add_tfsf(fdtd_job *job, const fdtd_tfsf_desc *tfsf);
int fdtd_add_source(fdtd_job *job, const fdtd_source_desc *src, int32_t *id);
int fdtd_add_monitor(fdtd_job *job, const fdtd_monitor_desc *mon, int32_t *id);
int fdtd_add_probe(fdtd_job *job, const fdtd_probe_desc *probe, int32_t *id);
/* Builds the per-cell material map and coefficient tables and allocates and
 * uploads all device state.  No set-up call is accepted afterwards. */
int fdtd_commit(fdtd_job *job);

/* ---- the time loop ------------------------------------------------------ */
/* Whole steps n_first .. n_first+n_steps-1, fused (the do-n loop body). */
int fdtd_step(fdtd_job *job, int32_t n_first, int32_t n_steps);

/* The loop body one procedure group at a time, for a host loop written like
 * the reference's:
 *   fdtd_update_DE   = updateD + source + every mat%update_E
 *                      (3D/.../program.f90:389-414)
 *   fdtd_pml_update_E = pmly%updateE   (3D/.../program.f90:419)
 *   fdtd_interchange  = interchange_E / interchange_H (:423, :437); the
 *                      halo is an in-memory neighbour, so this only checks
 *                      the call order
 *   fdtd_update_H    = updateH         (3D/.../program.f90:427-429)
 *   fdtd_pml_update_H = pmly%updateH   (3D/.../program.f90:433)
 *   fdtd_sample      = the DFT accumulation and per-step writes (:441-540)
 */
int fdtd_update_DE(fdtd_job *job, int32_t n);
int fdtd_pml_update_E(fdtd_job *job, int32_t n);
int fdtd_interchange(fdtd_job *job, int32_t which /* 0 = E, 1 = H */);
int fdtd_update_H(fdtd_job *job, int32_t n);
int fdtd_pml_update_H(fdtd_job *job, int32_t n);
int fdtd_sample(fdtd_job *job, int32_t n);

/* Checkpoint and resume.  fdtd_save_state writes the job's evolving state at
 * a step boundary into one host buffer of fdtd_state_bytes bytes: the field
 * arrays (with an incident line), the split-PML parts and reference slabs,
 * the dispersive state, the DFT sums with the not yet folded part of the
 * sample ring, and the probe records.  fdtd_load_state puts it into a job
 * committed from the same description; the job then continues bit for bit
 * as the saved one would have, from the step after the last one that ran.
 * The reference keeps no checkpoints. */
int fdtd_state_bytes(const fdtd_job *job, uint64_t *bytes);
int fdtd_save_state(fdtd_job *job, void *buf, uint64_t bytes);
int fdtd_load_state(fdtd_job *job, const void *buf, uint64_t bytes);

/* Health.  fdtd_check_finite counts the NaN and infinite values in the same
 * buffers a checkpoint holds (one reduction pass over them, on the job's
 * stream; a caller checks every so many steps).  The reference checks
 * nothing.
 * fdtd_debug_fail_alloc makes the device allocation that follows `after`
 * further successful ones fail as an out-of-memory would, for any job of the
 * process (-1 switches it off): it lets a caller exercise its recovery from
 * FDTD_ENOMEM at every allocation of set-up and stepping. */
int fdtd_check_finite(fdtd_job *job, int64_t *count);
int fdtd_debug_fail_alloc(int32_t after);
/* fdtd_debug_wait_limit sets how many polls the TMA-staged 3D kernels (the
 * core kernels of tiles 7 and 8, and the fused step kernel of tile 9) make of
 * a copy's mbarrier before they give up on it (rounds < 0: the
 * default, 2^22).  With 0 every wait of the main loop gives up at once: the
 * kernel sets the job's error flag, lets the copies it issued land, and
 * returns, and the next fdtd_sync reports FDTD_ECUDA (once).  It lets a
 * caller exercise that path without a copy that never completes.  No
 * counterpart in the reference, which has no device code. */
int fdtd_debug_wait_limit(fdtd_job *job, int32_t rounds);

/* ---- results ------------------------------------------------------------- */
int fdtd_sync(fdtd_job *job);
/* n[0]*n[1]*n[2] values of one component, x fastest. */
int fdtd_get_field(fdtd_job *job, int32_t comp, double *host);
int fdtd_set_field(fdtd_job *job, int32_t comp, const double *host);
/* DFT sums: for each transformed component (ascending component code), for
 * each frequency, for each cell of the box (x fastest; one value for a
 * FDTD_MONITOR_MEAN monitor): re[], im[]. */
int fdtd_get_monitor(fdtd_job *job, int32_t id, double *re, double *im);
/* Samples of steps n_first..min(n_last, last stepped n): for each step the
 * selected components in ascending code order.  *count = steps returned. */
int fdtd_get_probe(fdtd_job *job, int32_t id, double *host, int32_t *count);
/* Bytes of device memory the job holds (HBM admission). */
int fdtd_device_bytes(const fdtd_job *job, uint64_t *bytes);
/* Before fdtd_commit: an upper bound of the bytes the job will hold once
 * committed (after commit: the bytes it holds), for admission by footprint. */
int fdtd_estimate_bytes(const fdtd_job *job, uint64_t *bytes);

/* ---- measurement --------------------------------------------------------- */
/* When enabled, every launch of the job's kernels is bracketed by CUDA events
 * on the job's stream; fdtd_kernel_time returns the number of launches and
 * the summed device time of kernel class `kind` since the last reset. */
/* FDTD_KERNEL_E / _H: the 3D half-step kernels, and in 2D the interior
 * (core) kernels; FDTD_KERNEL_EDGE: the 2D kernels for PML cells, the edges
 * of the main range and rows with sources, monitors or reference slabs (in
 * 3D with the fused step kernel: the general E and H kernels);
 * FDTD_KERNEL_ADE: the 2D dispersive-cell kernel of the fused step (the
 * split 2D step appends the dispersive cells' blocks to its E edge kernel,
 * timed as FDTD_KERNEL_EDGE); FDTD_KERNEL_STEP: the
 * fused step kernels (3D: E and H of the core box in one launch; 2D: E and
 * H of the whole grid, dispersive cells aside, in one launch). */
enum { FDTD_KERNEL_E = 0, FDTD_KERNEL_H = 1, FDTD_KERNEL_DFT = 2, FDTD_KERNEL_LINE1D = 3,
       FDTD_KERNEL_EDGE = 4, FDTD_KERNEL_ADE = 5, FDTD_KERNEL_STEP = 6, FDTD_KERNEL_COUNT = 7 };
int fdtd_profile(fdtd_job *job, int32_t enable);
int fdtd_kernel_time(fdtd_job *job, int32_t kind, int64_t *launches, double *ms);
/* Block shape of the interior (core) kernels.  Before fdtd_commit, tile 0
 * (the default) lets commit time the candidates on the job's own grid and
 * keep the fastest (cached per kind of grid; environment FDTD_TUNE=0 skips
 * the timing); 1..3 pins a candidate: 2D 128 / 256 / 512 threads per block
 * (2D 4: the fused step kernel, which takes Ez, Hx and Hy of every cell
 * from step n to n+1 in one pass over two sets of field buffers used in
 * turn, for TMz FP32 jobs with nx a multiple of 4, no periodic axis and no
 * reference slabs, TFSF box or mean monitors; the job then holds a second
 * copy of its fields and of the stored PML part),
 * 3D 4 / 8 / 16 rows of 32 x-vectors, one plane per thread; 3D also 4..6:
 * the same shapes with each thread walking 8 planes and keeping the
 * neighbour plane in registers.  FP32 with 4-cell vectors, where the core
 * box lies at least one cell inside the grid, adds 3D 7: the TMA-staged E
 * core (tiled bulk copies into shared memory), and 8: both TMA-staged cores;
 * where the core box also ends at least one cell before the grid's far sides
 * and the grid has no reference slabs or TFSF box, 9: the fused step kernel,
 * which takes E and H of the core box from step n to n+1 in one pass over
 * two sets of field buffers used in turn (the job then holds a second copy
 * of its six field arrays); pinning one elsewhere fails at commit with
 * FDTD_EINVAL.  Results do not depend on the shape.  Environment FDTD_NO_TMA
 * leaves the TMA-staged kernels out, FDTD_NO_FUSED the fused ones.
 * fdtd_get_tile returns the shape in use (0: the job has no core kernels). */
int fdtd_set_tile(fdtd_job *job, int32_t tile);
int fdtd_get_tile(const fdtd_job *job, int32_t *tile);
/* Cells one launch of kernel class `kind` updates (FDTD_KERNEL_DFT: monitored
 * samples per fold), for the algorithmic bytes of a roofline. */
int fdtd_kernel_cells(const fdtd_job *job, int32_t kind, int64_t *cells);
/* Launches of this library's kernels since the job was created. */
int fdtd_launch_count(const fdtd_job *job, int64_t *launches);
/* Run the job's work on a caller-owned cudaStream_t (NULL: the job's own
 * stream), so a host program can order it with its other GPU work. */
int fdtd_set_stream(fdtd_job *job, void *cuda_stream);
/* Host->device and device->host bytes moved by set-up, getters and setters
 * since the job was created. */
int fdtd_transfer_bytes(const fdtd_job *job, uint64_t *h2d, uint64_t *d2h);

/* ---- serving: continuous batching of jobs on one GPU ---------------------
 * No counterpart in the reference, which runs one simulation per MPI job.
 * A server owns the jobs submitted to it (built with the fdtd_add_* calls,
 * not committed) and advances every admitted job on its own stream in chunks
 * of chunk_steps steps, so the kernels of different jobs overlap on the GPU.
 * Jobs are admitted in submission order when fewer than max_active are
 * running and their fdtd_estimate_bytes fits in what hbm_budget has left
 * (0: 90% of the device's free memory at creation); a job that can never fit
 * fails with FDTD_ENOMEM.  Small 2D jobs of one precision and layout are
 * packed: each part of a half step is one launch over all of them.  A finished job keeps its memory until
 * fdtd_server_release.  Each job runs steps 1..n_steps, with the same
 * kernels in the same order as fdtd_step(job, 1, n_steps) on its own, so its
 * results do not depend on the other jobs. */
typedef struct fdtd_server fdtd_server;
typedef struct {
  uint64_t hbm_budget;  /* device bytes the admitted jobs may hold (0: 90% of free) */
  int32_t max_active;   /* jobs advanced at once */
  int32_t chunk_steps;  /* steps per scheduling turn (rounded up to whole 32-step rings) */
  int32_t pack_cells;   /* 2D jobs of at most this many cells share launches (0: 2^20; < 0: never) */
} fdtd_server_desc;
typedef struct {
  int32_t queued, active;
  int64_t finished;
  uint64_t held_bytes, held_bytes_max, budget_bytes;
  int64_t packed_rings;  /* 32-step rings run by packs (one per pack and ring) */
  int64_t pack_builds;   /* packs set up (each change of a pack's members) */
  double pack_build_s;   /* host seconds spent setting packs up */
} fdtd_server_status;
enum { FDTD_REQ_QUEUED = 0, FDTD_REQ_RUNNING = 1, FDTD_REQ_DONE = 2, FDTD_REQ_FAILED = 3 };
int fdtd_server_create(const fdtd_server_desc *desc, fdtd_server **server);
/* Takes ownership of `job` (uncommitted) on success. */
int fdtd_server_submit(fdtd_server *server, fdtd_job *job, int32_t n_steps, int64_t *ticket);
/* Waits until the job is done or failed, or timeout_ms passes (< 0: no
 * limit); *state is its FDTD_REQ_* state. */
int fdtd_server_wait(fdtd_server *server, int64_t ticket, int32_t timeout_ms, int32_t *state);
/* The finished job, for fdtd_get_monitor / fdtd_get_probe / fdtd_get_field;
 * valid until fdtd_server_release. */
int fdtd_server_job(fdtd_server *server, int64_t ticket, fdtd_job **job);
/* Host times in seconds since the server was created (-1: not yet). */
int fdtd_server_times(fdtd_server *server, int64_t ticket, double *t_submit, double *t_admit, double *t_done);
/* Destroys a finished job and returns its memory to the budget. */
int fdtd_server_release(fdtd_server *server, int64_t ticket);
int fdtd_server_stats(fdtd_server *server, fdtd_server_status *stats);
/* Stops admitting, lets the chunks in flight end and destroys every job. */
int fdtd_server_destroy(fdtd_server *server);

/* ---- allocation-free DFT of a caller-owned field ------------------------ *
 * No counterpart in the reference: its DFT sums live inside program.f90's
 * time loop (2D/.../program.f90:383-391, 3D/.../program.f90:441-540).  This
 * entry point serves host codes that keep their own device fields and cannot
 * let a library allocate device memory while they run: a code that takes
 * every device byte from its own pool at start-up (a driver allocation would
 * synchronise the device and fragment that pool), or one that runs under a
 * device-memory budget fixed before its time loop starts.
 *
 * Call it once per step n, after the H update, with the device field array
 * `field` (nx*ny*nz values of `precision`, x fastest) and the box lo..hi
 * (0-based, inclusive).  Steps n_first..n_last are sampled; the sums
 *   acc_re[f*ncell + c] += sum_n cos(omega[f] (n-1) dt) F_n(c) dt,
 *   acc_im[f*ncell + c] += sum_n sin(omega[f] (n-1) dt) F_n(c) dt
 * are folded into the caller's device accumulators (FP64, zeroed by the
 * caller) every FDTD_NOALLOC_RING steps, at n == n_last, and when `flush` is
 * non-zero.  Calls for n outside the window return at once.  `omega`,
 * `acc_re` and `acc_im` are device pointers; work is queued on `stream`
 * (a cudaStream_t, NULL for the legacy default stream).
 *
 * It allocates nothing: the samples of the current ring are staged in a
 * static device array of FDTD_NOALLOC_STAGE_BYTES that the library holds on
 * every device for the life of the process, so a box may hold at most
 * FDTD_NOALLOC_MAX_CELLS cells (a 512 x 512 plane); a larger box fails with
 * FDTD_ERANGE.  The first call on each device does the set-up, with the
 * device current: it looks up that array's device address
 * (cudaGetSymbolAddress) and loads the kernels it launches, so that no later
 * call makes the driver load code; make that first call before any stream
 * capture.  The array is shared by all calls on a device and keeps the last
 * call's samples, so one sequence of steps may run at a time per device:
 * calls that overlap on the GPU (two boxes at once, or two host threads or
 * streams) race on it.  A sequence may start at any step of the window
 * (a run resumed mid-window, say): the ring slots before its first step are
 * cleared whenever a call does not follow the previous call's step. */
#define FDTD_NOALLOC_RING 32
#define FDTD_NOALLOC_MAX_CELLS 262144
#define FDTD_NOALLOC_STAGE_BYTES (FDTD_NOALLOC_MAX_CELLS * FDTD_NOALLOC_RING * 8)
int fdtd_dft_sample_noalloc(const void *field, int32_t precision, int32_t nx, int32_t ny, int32_t nz,
                            const int32_t lo[3], const int32_t hi[3], int32_t n, int32_t n_first,
                            int32_t n_last, double dt, const double *omega, int32_t nfreq,
                            double *acc_re, double *acc_im, int32_t flush, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FDTD_GB300_H */
