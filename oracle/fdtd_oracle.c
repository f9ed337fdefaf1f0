/*
 * fdtd_oracle.c -- TEST INFRASTRUCTURE ONLY (see fdtd_oracle.h).
 *
 * An FP64, single-domain, line-by-line restatement of the reference's time
 * loop.  Reference paths below are relative to the reference checkout:
 *   P1 = FDTDsimulations/1D/TFSF-air_SLG_SiO2_Sidisp
 *   P2 = FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate
 *   P3 = FDTDsimulations/3D/air-AuAntennasSiO2-Si
 *   M1, M2, M3, Mm = modules/src/{1D,2D,3D,misc}
 *
 * Arrays use the reference's own 1-based indexing with one halo cell on each
 * side of every used axis (real*8 (0:N_x+1,0:N_y+1,0:N_z+1), P3/program.f90:77);
 * the MPI ranks' slabs along y are one array, so the y exchange of
 * interchange_E/H is the identity and only the periodic wraps remain.
 *
 * Compile with -ffp-contract=off: the operations are evaluated in the order
 * the Fortran expressions give, without fused multiply-adds.
 */
#include "fdtd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants: Mm/constants_mod.f90:3-7 -------------------------------- */
static double K_PI, K_EP0, K_MU0, K_C0, K_Z0;
static void init_constants(void) {
  K_PI = 4.0 * atan(1.0);
  K_EP0 = 8.85418781762039e-12;
  K_MU0 = K_PI * 4e-7;
  K_C0 = 1.0 / sqrt(K_EP0 * K_MU0);
  K_Z0 = sqrt(K_MU0 / K_EP0);
}

static char g_err[512];
const char *ora_error(void) { return g_err; }
#define FAIL(...) do { snprintf(g_err, sizeof g_err, __VA_ARGS__); return -1; } while (0)

typedef struct { double re, im; } cplx;
static cplx cmul(cplx a, cplx b) { cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static cplx cadd(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }
static cplx csub(cplx a, cplx b) { cplx r = {a.re - b.re, a.im - b.im}; return r; }
static cplx cscale(cplx a, double s) { cplx r = {a.re * s, a.im * s}; return r; }
static cplx cexp_(cplx z) { double e = exp(z.re); cplx r = {e * cos(z.im), e * sin(z.im)}; return r; }
/* Real part of a/b with range reduction (Smith), the Fortran complex division. */
static double cdiv_re(cplx a, cplx b) {
  if (fabs(b.re) >= fabs(b.im)) {
    double r = b.im / b.re, den = b.re + b.im * r;
    return (a.re + a.im * r) / den;
  } else {
    double r = b.re / b.im, den = b.re * r + b.im;
    return (a.re * r + a.im) / den;
  }
}

/* ---- job ------------------------------------------------------------------ */
enum { MAT_DIEL = 1, MAT_GOLD = 2, MAT_GRAPHENE = 3, MAT_LORENTZ_JP = 4, MAT_LORENTZ_S = 5, MAT_GRAPHENE_CP = 6 };
#define NPOLE FDTD_LORENTZ_MAX_POLES
#define MAXMAT 250

typedef struct {
  int kind;
  double gax;                          /* ConstantDielectric: 1/eps     */
  double ha, hb; cplx gb[2], gc[2], ga;/* Gold: M2/gold_mod.f90:147-157 */
  /* graphene sheet */
  double g_ha, g_hb, g_ga, r0, r1, r2, kerr; int normal;
  int64_t ncell; int64_t *cells;       /* cells whose final id is this   */
  double *I[3], *S[3];                 /* Drude running sums per comp    */
  cplx *g1[3], *g2[3];                 /* critical-point terms           */
  double *SR[3], *SRm1[3], *SRm2[3];   /* graphene Raman recursion       */
  /* Lorentz poles: JP form (M3/goldLorentzJp_mod.f90:14-18) and S form
     (M3/si_mod.f90:14-26) */
  int npoles; double l_ga;             /* 1/epinf                        */
  double g1L[NPOLE], g2L[NPOLE], xi[NPOLE];       /* gamma1L, gamma2L, xi1 */
  double sa[NPOLE], sb[NPOLE], sc[NPOLE];         /* ga_l, gb_l, gc_l      */
  double *P[3][NPOLE], *Jp[3][NPOLE], *JpT[3];    /* JP state              */
  double *Sm1[3][NPOLE], *Sm2[3][NPOLE];          /* S state: S(n-1), S(n-2) */
  int l_sheet, l_normal;                          /* SLG_3LJp1nm sheet      */
  int l_zx;                                       /* SLG_LJp: Ez takes JpxT */
  double chi3, g1N, g2N, escale;                  /* xi3, Kerr recursion, z0 */
  double *Qk[3], *Gk[3];                          /* Q, G per component      */
  /* the reference's Graphene (M3/graphene_mod.f90:8-44): Drude, 4 critical
     points, Raman; I, S and the Raman arrays are shared with the above */
  cplx cgb[4], cgc[4], cgax; double c_ha, c_hb; int c_normal;
  double c_r0, c_r1, c_r2;
  cplx *cg[3][4];
  fdtd_region region;                  /* painted at commit              */
  double *centers;                     /* owned copy for SPHERES         */
  uint8_t *mask;                       /* owned copy for MASK            */
} omat;

typedef struct {
  fdtd_source_desc d;
} osrc;

typedef struct {
  fdtd_monitor_desc d;
  int ncomp, comps[8], nfreq; int64_t ncell;
  double *omega;
  double *re, *im; /* [comp][freq][cell] */
} omon;

typedef struct {
  fdtd_probe_desc d;
  int ncomp, comps[8];
  int count;
  double *buf; int cap;
} oprobe;

/* PML slab of the reference (one pmly object on a first/last rank). */
typedef struct {
  int on, side;          /* side 0: low (ycord==0), 1: high (ycord==lastY) */
  int j0, j1;            /* allocated global rows (with the halo rows)     */
  int ja, jb;            /* yBDlow (low) / yBDhigh (high), global          */
  /* split fields, slab-local rows j-j0, full x/z with halos */
  double *f[12];
  /* coefficient arrays over the slab rows (1..N interior index space) */
  double *f1x, *f2x, *f1y, *f2y, *f1z, *f2z, *g1x, *g2x, *g1y, *g2y, *g1z, *g2z;
} oslab;

/* split-field names for the slab storage (3D uses all, 2D uses 0..3) */
enum { S_EXY, S_EXZ, S_EYZ, S_EYX, S_EZX, S_EZY, S_HXY, S_HXZ, S_HYZ, S_HYX, S_HZX, S_HZY };
enum { S2_EX = 0, S2_EY = 1, S2_HZX = 2, S2_HZY = 3 };

struct ora_job {
  fdtd_grid_desc g;
  int dim;                       /* 1, 2, 3 */
  int nx, ny, nz;                /* interior cells */
  int px, py, pz;                /* padded sizes */
  int64_t ntot;
  double *F[9];                  /* ex ey ez hx hy hz dx dy dz, padded */
  uint8_t *matid;                /* padded */
  int nmat; omat mat[MAXMAT + 1];
  int nsrc; osrc src[64];
  int nmon; omon mon[64];
  int nprobe; oprobe probe[64];
  int pml_mode; fdtd_pml_desc pml;
  oslab slab[2];
  /* SPLIT PML: per-axis coefficient tables (0-based cell index) */
  double *cf1[3], *cf2[3], *cg1[3], *cg2[3];
  double *sp[12];                /* split fields, padded full size     */
  int shell_lo[3], shell_hi[3];  /* interior box (0-based inclusive)   */
  /* 1D total-field/scattered-field incident line */
  int tfsf; fdtd_tfsf1d_desc tf;
  double *exi, *hzi;             /* padded 0..N+1                     */
  oslab islab[2];
  /* 2D/3D total-field/scattered-field box: incident line along y */
  int tfbox; fdtd_tfsf_desc tb;
  int tb_face[3];                /* 1: the box has faces normal to axis */
  double *le, *lh;               /* incident line E and H, 0..ny-1      */
  double labc[4];                /* two-step absorbing ends: low m1 m2, high m1 m2 */
  int committed;
  int last_n;
  int nth;
};

static int in_shell(const struct ora_job *J, int i0, int j0, int k0);
#define IX(J, i, j, k) ((int64_t)(i) + (int64_t)(J)->px * ((int64_t)(j) + (int64_t)(J)->py * (int64_t)(k)))

enum { EX = 0, EY, EZ, HX, HY, HZ, DX, DY, DZ };

ora_job *ora_create(const fdtd_grid_desc *grid) {
  init_constants();
  ora_job *J = (ora_job *)calloc(1, sizeof(ora_job));
  if (!J) return NULL;
  J->g = *grid;
  switch (grid->layout) {
    case FDTD_LAYOUT_1D: J->dim = 1; break;
    case FDTD_LAYOUT_2D_TE: case FDTD_LAYOUT_2D_TM: J->dim = 2; break;
    case FDTD_LAYOUT_3D: J->dim = 3; break;
    default: free(J); snprintf(g_err, sizeof g_err, "bad layout"); return NULL;
  }
  J->nx = grid->n[0]; J->ny = grid->n[1]; J->nz = grid->n[2];
  if (J->dim == 1) { J->nx = 1; J->nz = 1; }
  if (J->dim == 2) J->nz = 1;
  /* 1D arrays are (0:N+1) along y; x and z are single cells without halos */
  J->px = (J->dim >= 2) ? J->nx + 2 : 1;
  J->py = J->ny + 2;
  J->pz = (J->dim == 3) ? J->nz + 2 : 1;
  J->ntot = (int64_t)J->px * J->py * J->pz;
  for (int c = 0; c < 9; c++) {
    J->F[c] = (double *)calloc((size_t)J->ntot, sizeof(double));
    if (!J->F[c]) { snprintf(g_err, sizeof g_err, "oom"); return NULL; }
  }
  J->matid = (uint8_t *)calloc((size_t)J->ntot, 1);
  J->last_n = 0;
  return J;
}

static void free_slab(oslab *s) {
  for (int q = 0; q < 12; q++) free(s->f[q]);
  free(s->f1x); free(s->f2x); free(s->f1y); free(s->f2y); free(s->f1z); free(s->f2z);
  free(s->g1x); free(s->g2x); free(s->g1y); free(s->g2y); free(s->g1z); free(s->g2z);
}

void ora_destroy(ora_job *J) {
  if (!J) return;
  for (int c = 0; c < 9; c++) free(J->F[c]);
  free(J->matid);
  for (int m = 1; m <= J->nmat; m++) {
    omat *M = &J->mat[m];
    free(M->cells); free(M->centers); free(M->mask);
    for (int c = 0; c < 3; c++) { free(M->I[c]); free(M->S[c]); free(M->g1[c]); free(M->g2[c]);
      for (int q = 0; q < 4; q++) free(M->cg[c][q]);
      free(M->SR[c]); free(M->SRm1[c]); free(M->SRm2[c]); free(M->JpT[c]); free(M->Qk[c]); free(M->Gk[c]);
      for (int l = 0; l < NPOLE; l++) { free(M->P[c][l]); free(M->Jp[c][l]); free(M->Sm1[c][l]); free(M->Sm2[c][l]); } }
  }
  for (int q = 0; q < J->nmon; q++) { free(J->mon[q].omega); free(J->mon[q].re); free(J->mon[q].im); }
  for (int q = 0; q < J->nprobe; q++) free(J->probe[q].buf);
  free_slab(&J->slab[0]); free_slab(&J->slab[1]);
  free_slab(&J->islab[0]); free_slab(&J->islab[1]);
  for (int a = 0; a < 3; a++) { free(J->cf1[a]); free(J->cf2[a]); free(J->cg1[a]); free(J->cg2[a]); }
  for (int q = 0; q < 12; q++) free(J->sp[q]);
  free(J->exi); free(J->hzi);
  free(J->le); free(J->lh);
  free(J);
}

/* ---- materials ------------------------------------------------------------ */
static int add_material(ora_job *J, const fdtd_region *r, omat **out) {
  if (J->committed) FAIL("job already committed");
  if (J->nmat >= MAXMAT) FAIL("too many materials");
  omat *M = &J->mat[++J->nmat];
  memset(M, 0, sizeof *M);
  M->region = *r;
  if (r->kind == FDTD_REGION_SPHERES) {
    M->centers = (double *)malloc(sizeof(double) * 4 * (size_t)(r->count > 0 ? r->count : 1));
    memcpy(M->centers, r->centers_radii, sizeof(double) * 4 * (size_t)r->count);
    M->region.centers_radii = M->centers;
  } else if (r->kind == FDTD_REGION_MASK) {
    int64_t n = (int64_t)J->g.n[0] * J->g.n[1] * J->g.n[2];
    M->mask = (uint8_t *)malloc((size_t)n);
    memcpy(M->mask, r->mask, (size_t)n);
    M->region.mask = M->mask;
  } else if (r->kind != FDTD_REGION_BOX) {
    FAIL("bad region kind");
  }
  *out = M;
  return J->nmat;
}

/* ConstantDielectric: gax = 1/constant_ep (M2/simpledielectric_mod.f90:170-187) */
int ora_add_dielectric(ora_job *J, const fdtd_region *r, double eps) {
  omat *M; int id = add_material(J, r, &M); if (id < 0) return id;
  M->kind = MAT_DIEL;
  M->gax = (eps == 0.0) ? 0.0 : 1.0 / eps;
  return id;
}

/* Gold coefficients: M2/gold_mod.f90:129-168 (setexp :160-168) */
int ora_add_gold(ora_job *J, const fdtd_region *r, const fdtd_drude2cp *p) {
  omat *M; int id = add_material(J, r, &M); if (id < 0) return id;
  M->kind = MAT_GOLD;
  double dt = J->g.dt;
  cplx unoi = {0.0, 1.0};
  cplx expi[2], expg[2];
  for (int q = 0; q < 2; q++) {
    cplx a = {-unoi.re * p->phi[q], -unoi.im * p->phi[q]};      /* -unoi*phip */
    expi[q] = cexp_(a);
    cplx b = {(-p->gamma[q]) * dt, p->omega[q] * dt};            /* (-rp+unoi*omp)*dt */
    expg[q] = cexp_(b);
  }
  M->ha = exp(-p->gamma_d * dt);
  M->hb = (p->omega_d * p->omega_d) * dt / p->gamma_d;
  for (int q = 0; q < 2; q++) {
    M->gb[q] = expg[q];
    /* dt*2.d0*unoi*ap*omp*expi, evaluated left to right */
    cplx t = cscale(unoi, dt * 2.0);
    t = cscale(t, p->amp[q]);
    t = cscale(t, p->omega[q]);
    M->gc[q] = cmul(t, expi[q]);
  }
  cplx ga = {p->eps_inf, 0.0};
  ga = csub(ga, M->gc[0]);
  ga = csub(ga, M->gc[1]);
  M->ga = ga;
  return id;
}

/* SiL800 (M3/siL800_mod.f90:28-104): E = (D - I)/ga, I += gb E with
 * ga = ep_inf + sigma dt/ep0, gb = sigma dt/ep0.  It is the gold update with
 * ha = 0 and no critical points (gb_p = gc_p = 0), which leaves
 * E = (D - I + 0 S + 0 + 0)/ga and I += hb E.  The reference writes its Ey
 * pair twice and never Ez (:42-46); every component is updated here. */
int ora_add_conductive(ora_job *J, const fdtd_region *r, double eps_inf, double sigma) {
  omat *M; int id = add_material(J, r, &M); if (id < 0) return id;
  M->kind = MAT_GOLD;
  double dt = J->g.dt;
  M->ha = 0.0;
  M->hb = sigma * dt / K_EP0;
  cplx zero = {0.0, 0.0}, ga = {eps_inf + sigma * dt / K_EP0, 0.0};
  for (int q = 0; q < 2; q++) { M->gb[q] = zero; M->gc[q] = zero; }
  M->ga = ga;
  return id;
}

/* graphene633 (M1/graphene633_mod.f90:26-105), literally: the graphene
 * update below with no Drude memory (g_ha = 0), g_ga = ep_inf + sigma dt/ep0,
 * g_hb = sigma dt/ep0, kerr = xi3 alpha, and the module's Raman coefficients
 * (:101-103), damped by dnuNL itself; every component takes it. */
int ora_add_graphene_nk(ora_job *J, const fdtd_region *r, const fdtd_graphene_nk_desc *p) {
  if (!(p->wavelength > 0) || !(p->scale >= 0)) FAIL("graphene_nk needs wavelength > 0 and scale >= 0");
  omat *M; int id = add_material(J, r, &M); if (id < 0) return id;
  M->kind = MAT_GRAPHENE;
  M->normal = -1;
  double dt = J->g.dt;
  double sigma = sqrt(p->scale) * 4.0 * K_PI * p->n * p->k * K_C0 * K_EP0 / p->wavelength;
  double ep_inf = p->scale * ((p->n * p->n) - (p->k * p->k));
  M->g_ha = 0.0;
  M->g_hb = sigma * dt / K_EP0;
  M->g_ga = ep_inf + sigma * dt / K_EP0;
  M->kerr = p->chi3 * p->alpha;
  if (p->chi3 != 0.0) {
    double betaR = sqrt((p->w_nl * p->w_nl) - (p->gamma_nl * p->gamma_nl));
    double omegaR = (p->w_nl * p->w_nl) / betaR;
    M->r0 = (1.0 - p->alpha) * p->chi3 * omegaR * dt * exp(-p->gamma_nl * dt) * sin(betaR * dt);
    M->r1 = 2.0 * exp(-p->gamma_nl * dt) * cos(betaR * dt);
    M->r2 = -exp(-2.0 * p->gamma_nl * dt);
  }
  return id;
}

/* Graphene sheet: intraband Drude surface conductivity as an ADE of the
 * Drude form of the gold model (M3/gold_mod.f90:50-88 with no critical
 * points), the Raman recursion of M3/graphene_mod.f90:202-262 in the
 * denominator and the linearised Kerr term of M1/graphene633_mod.f90:33-35. */
int ora_add_graphene(ora_job *J, const fdtd_region *r, const fdtd_graphene_desc *p) {
  if (r->kind != FDTD_REGION_BOX) FAIL("graphene needs a one-cell-thick box");
  int normal = -1;
  for (int a = 0; a < 3; a++)
    if (r->lo[a] == r->hi[a] && J->g.n[a] > 1) { normal = a; break; }
  if (normal < 0) FAIL("graphene box must be one cell thick");
  omat *M; int id = add_material(J, r, &M); if (id < 0) return id;
  M->kind = MAT_GRAPHENE;
  M->normal = normal;
  const double hbar = 6.62607015e-34 / (2.0 * K_PI), kb = 1.380649e-23, qe = 1.602176634e-19;
  double kT = kb * p->temperature, ef = p->fermi_ev * qe;
  double sigma_s0 = (2.0 * qe * qe * kT * p->tau / (K_PI * hbar * hbar)) * log(2.0 * cosh(ef / (2.0 * kT)));
  double sigma0 = sigma_s0 / p->thickness;      /* bulk conductivity of the sheet cell */
  double gam = 1.0 / p->tau, dt = J->g.dt;
  M->g_ha = exp(-gam * dt);
  M->g_hb = sigma0 * dt / K_EP0;                /* = wp^2 dt / gamma */
  M->g_ga = 1.0;
  double wNL = 2.0 * K_PI * p->raman_freq, dnuNL = 1.0 / p->raman_tau;
  double alfaR = 0.5 * dnuNL;
  double betaR = sqrt(wNL * wNL - alfaR * alfaR);
  double omegaR = (wNL * wNL) / betaR;
  double chi3n = p->chi3 * p->e_scale * p->e_scale;
  M->r0 = p->raman_frac * chi3n * omegaR * dt * exp(-alfaR * dt) * sin(betaR * dt);
  M->r1 = 2.0 * exp(-alfaR * dt) * cos(betaR * dt);
  M->r2 = -exp(-2.0 * alfaR * dt);
  M->kerr = (1.0 - p->raman_frac) * chi3n;
  return id;
}

/* The reference's Graphene%initialize_GrapheneVars (M3/graphene_mod.f90:202-283,
 * M2/graphene_mod.f90:163-236, M1/graphene_mod.f90:126-183), with setexp and
 * scaleParams applied first: scaled_ap = (Graphenewidth/ds) ap, scaled_wD =
 * sqrt(Graphenewidth/ds) wD.  The Raman coefficients follow the 3D module
 * (exact) or the 2D one (central); chi3 = 0 leaves them zero, as the 1D
 * module has no Raman term. */
int ora_add_graphene_cp(ora_job *J, const fdtd_region *r, const fdtd_graphene_cp_desc *p) {
  if (!(p->drude_gamma > 0) || !(p->width > 0)) FAIL("graphene needs drude_gamma > 0 and width > 0");
  if (p->normal_axis < -1 || p->normal_axis > 2) FAIL("bad normal_axis");
  omat *M; int id = add_material(J, r, &M); if (id < 0) return id;
  M->kind = MAT_GRAPHENE_CP;
  M->c_normal = p->normal_axis;
  double dt = J->g.dt;
  cplx unoi = {0.0, 1.0};
  double scaleFact = p->width / J->g.ds;
  double scaled_wD = sqrt(scaleFact) * p->drude_omega;
  M->c_ha = exp(-p->drude_gamma * dt);
  M->c_hb = (scaled_wD * scaled_wD) * dt / p->drude_gamma;
  cplx gax = {p->eps_inf, 0.0};
  for (int q = 0; q < 4; q++) {
    cplx a = {-unoi.re * p->phi[q], -unoi.im * p->phi[q]};      /* -unoi*phip */
    cplx expi = cexp_(a);
    cplx b = {(-p->gamma[q]) * dt, p->omega[q] * dt};            /* (-rp+unoi*omp)*dt */
    M->cgb[q] = cexp_(b);
    /* dt*2.d0*unoi*scaled_ap*omp*expi, evaluated left to right */
    cplx t = cscale(unoi, dt * 2.0);
    t = cscale(t, scaleFact * p->amp[q]);
    t = cscale(t, p->omega[q]);
    M->cgc[q] = cmul(t, expi);
    gax = csub(gax, M->cgc[q]);
  }
  M->cgax = gax;
  if (p->chi3 != 0.0) {
    double xi3 = p->chi3, wNL = p->w_nl, dnuNL = p->gamma_nl;
    if (p->raman_form == FDTD_RAMAN_CENTRAL) {
      M->c_r0 = xi3 * ((wNL * dt) * (wNL * dt)) / (1.0 + dnuNL * dt);
      M->c_r1 = (2.0 - (wNL * dt) * (wNL * dt)) / (1.0 + dnuNL * dt);
      M->c_r2 = -(1.0 - dnuNL * dt) / (1.0 + dnuNL * dt);
    } else {
      double alfaR = 0.5 * dnuNL;
      double betaR = sqrt((wNL * wNL) - (alfaR * alfaR));
      double omegaR = (wNL * wNL) / betaR;
      M->c_r0 = xi3 * omegaR * dt * exp(-alfaR * dt) * sin(betaR * dt);
      M->c_r1 = 2.0 * exp(-alfaR * dt) * cos(betaR * dt);
      M->c_r2 = -exp(-2.0 * alfaR * dt);
    }
  }
  return id;
}

/* Lorentz poles.  JP: gamma1L = (1-dnu dt)/(1+dnu dt), gamma2L = w0^2 dt/(1+dnu dt),
 * ga = 1/epinf (M3/goldLorentzJp_mod.f90:140-161).  S: ga_l = (2-(dt wp)^2)/(1+dt dnup),
 * gb_l = (dt dnup-1)/(1+dt dnup), gc_l = dep (wp dt)^2/(1+dt dnup) (M3/si_mod.f90:180-206). */
int ora_add_lorentz(ora_job *J, const fdtd_region *r, const fdtd_lorentz_desc *p) {
  if (p->npoles < 1 || p->npoles > NPOLE) FAIL("npoles must be 1..%d", NPOLE);
  if (p->form != FDTD_LORENTZ_JP && p->form != FDTD_LORENTZ_S) FAIL("bad Lorentz form");
  if (!(p->eps_inf != 0.0)) FAIL("eps_inf must be nonzero");
  int normal = -1;
  if (p->sheet) {
    if (r->kind != FDTD_REGION_BOX) FAIL("a Lorentz sheet needs a one-cell-thick box");
    for (int a = 0; a < 3; a++)
      if (r->lo[a] == r->hi[a] && J->g.n[a] > 1) { normal = a; break; }
    if (normal < 0) FAIL("a Lorentz sheet must be one cell thick");
  }
  if (p->chi3 != 0.0 && p->form != FDTD_LORENTZ_JP) FAIL("the Kerr term needs the JP form");
  if (p->ez_uses_x_current && (p->form != FDTD_LORENTZ_JP || J->dim != 3 || !p->sheet || r->lo[1] != r->hi[1]))
    FAIL("ez_uses_x_current needs the JP form and a sheet normal to y in 3D");
  omat *M; int id = add_material(J, r, &M); if (id < 0) return id;
  M->kind = p->form == FDTD_LORENTZ_JP ? MAT_LORENTZ_JP : MAT_LORENTZ_S;
  M->npoles = p->npoles;
  M->l_ga = 1.0 / p->eps_inf;
  double dt = J->g.dt;
  /* SLG_3LJp1nm: (1-dnuNL dt)/(1+dnuNL dt), wNL^2 dt/(1+dnuNL dt) (M3/graphene3LorentzJp1nm_mod.f90:89-91) */
  M->l_sheet = p->sheet != 0; M->l_normal = normal; M->l_zx = p->ez_uses_x_current != 0;
  M->chi3 = p->chi3; M->escale = p->e_scale;
  M->g1N = (1.0 - p->gamma_nl * dt) / (1.0 + p->gamma_nl * dt);
  M->g2N = (p->w_nl * p->w_nl) * dt / (1.0 + p->gamma_nl * dt);
  for (int l = 0; l < p->npoles; l++) {
    double w = p->omega[l], nu = p->gamma[l];
    M->xi[l] = p->delta_eps[l];
    M->g1L[l] = (1.0 - nu * dt) / (1.0 + nu * dt);
    M->g2L[l] = (w * w) * dt / (1.0 + nu * dt);
    M->sa[l] = (2.0 - (dt * w) * (dt * w)) / (1.0 + dt * nu);
    M->sb[l] = (dt * nu - 1.0) / (1.0 + dt * nu);
    M->sc[l] = (p->delta_eps[l] * ((w * dt) * (w * dt))) / (1.0 + dt * nu);
  }
  return id;
}

static int inside_region(const ora_job *J, const fdtd_region *r, int i, int j, int k) {
  /* i, j, k are 0-based cell indices */
  switch (r->kind) {
    case FDTD_REGION_BOX:
      return i >= r->lo[0] && i <= r->hi[0] && j >= r->lo[1] && j <= r->hi[1] && k >= r->lo[2] && k <= r->hi[2];
    case FDTD_REGION_SPHERES:
      for (int q = 0; q < r->count; q++) {
        const double *c = r->centers_radii + 4 * q;
        double ddx = i + 0.5 - c[0], ddy = j + 0.5 - c[1];
        double d2 = ddx * ddx + ddy * ddy;
        if (J->dim == 3) { double ddz = k + 0.5 - c[2]; d2 += ddz * ddz; }
        if (d2 <= c[3] * c[3]) return 1;
      }
      return 0;
    case FDTD_REGION_MASK:
      return r->mask[(int64_t)i + (int64_t)J->g.n[0] * ((int64_t)j + (int64_t)J->g.n[1] * k)] != 0;
  }
  return 0;
}

/* interior 0-based (i,j,k) -> padded linear index */
static int64_t cell_ix(const ora_job *J, int i, int j, int k) {
  if (J->dim == 1) return (int64_t)(j + 1);
  if (J->dim == 2) return IX(J, i + 1, j + 1, 0);
  return IX(J, i + 1, j + 1, k + 1);
}

/* ---- PML ------------------------------------------------------------------ */
int ora_add_pml(ora_job *J, const fdtd_pml_desc *p) {
  if (J->committed) FAIL("job already committed");
  if (p->mode != FDTD_PML_REFERENCE && p->mode != FDTD_PML_SPLIT) FAIL("bad pml mode");
  if (p->mode == FDTD_PML_SPLIT && J->dim == 1) FAIL("1D uses the reference PML");
  if (p->mode == FDTD_PML_REFERENCE && J->g.layout == FDTD_LAYOUT_2D_TM) FAIL("2D TM uses the split PML");
  J->pml_mode = p->mode;
  J->pml = *p;
  return 0;
}

int ora_add_tfsf_1d(ora_job *J, const fdtd_tfsf1d_desc *t) {
  if (J->dim != 1) FAIL("TFSF line is 1D only");
  J->tfsf = 1; J->tf = *t;
  return 0;
}

int ora_add_source(ora_job *J, const fdtd_source_desc *s) {
  if (J->nsrc >= 64) FAIL("too many sources");
  J->src[J->nsrc].d = *s;
  return J->nsrc++;
}

static int comp_list(int mask, int *comps) {
  int n = 0;
  for (int c = 0; c < 8; c++) if (mask & (1 << c)) comps[n++] = c;
  return n;
}

int ora_add_monitor(ora_job *J, const fdtd_monitor_desc *m) {
  if (J->nmon >= 64) FAIL("too many monitors");
  omon *M = &J->mon[J->nmon];
  memset(M, 0, sizeof *M);
  M->d = *m;
  M->ncomp = comp_list(m->comp_mask, M->comps);
  M->nfreq = m->nfreq;
  M->omega = (double *)malloc(sizeof(double) * (size_t)m->nfreq);
  memcpy(M->omega, m->omega, sizeof(double) * (size_t)m->nfreq);
  M->d.omega = M->omega;
  if (m->reduce != FDTD_MONITOR_CELLS && m->reduce != FDTD_MONITOR_MEAN) FAIL("bad monitor reduce mode");
  M->ncell = m->reduce == FDTD_MONITOR_MEAN
                 ? 1
                 : (int64_t)(m->hi[0] - m->lo[0] + 1) * (m->hi[1] - m->lo[1] + 1) * (m->hi[2] - m->lo[2] + 1);
  size_t n = (size_t)M->ncomp * M->nfreq * M->ncell;
  M->re = (double *)calloc(n, sizeof(double));
  M->im = (double *)calloc(n, sizeof(double));
  return J->nmon++;
}

int ora_add_probe(ora_job *J, const fdtd_probe_desc *p) {
  if (J->nprobe >= 64) FAIL("too many probes");
  oprobe *P = &J->probe[J->nprobe];
  memset(P, 0, sizeof *P);
  P->d = *p;
  P->ncomp = comp_list(p->comp_mask, P->comps);
  return J->nprobe++;
}

/* Reference PML slab coefficients and fields.
 * 2D: M2/BERpmly_HzExEy_mod.f90:229-425; 3D: M3/BERpmly_mod.f90:485-874;
 * 1D: M1/BERpmly_ExHz_mod.f90:163-254.  The arrays cover the slab rows only
 * (the reference allocates the whole rank but touches only these rows). */
static double *zalloc(int64_t n) { return (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

static void init_ref_slab(ora_job *J, oslab *S, int side, double eplow_r, double ephigh_r, int npmly) {
  const fdtd_pml_desc *p = &J->pml;
  int dim = J->dim, nx = J->nx, nz = J->nz, Ny = J->ny;
  double dt = J->g.dt, ds = J->g.ds, sigmam = p->sigma_max, order = p->order;
  double eplow = eplow_r * K_EP0, ephigh = ephigh_r * K_EP0;   /* air_ep*ep0 (P3/program.f90:205) */
  double ep = side == 0 ? eplow : ephigh;
  double Ku = dt * K_C0 / ds;                                   /* dt*c0/ds (M3/BERpmly_mod.f90:506) */
  double epr = ep / K_EP0;                                       /* eplow/ep0 */
  double z0 = sqrt(K_MU0 / K_EP0);
  memset(S, 0, sizeof *S);
  S->on = 1; S->side = side;
  S->ja = npmly;                    /* yBDlow = npmly           */
  S->jb = Ny - npmly + 1;           /* yBDhigh = N_y-npmly+1    */
  if (side == 0) { S->j0 = 0; S->j1 = S->ja + 1; }
  else { S->j0 = S->jb - 1; S->j1 = Ny + 1; }
  int rows = S->j1 - S->j0 + 1;
  int64_t plane = (int64_t)J->px * rows * J->pz;
  int nf = dim == 3 ? 12 : (dim == 2 ? 4 : 2);
  for (int q = 0; q < nf; q++) S->f[q] = zalloc(plane);
  /* coefficient arrays over (i, row, k) with the 1-based interior index */
  int64_t cn = (int64_t)J->px * rows * J->pz;
  double **arr[12] = {&S->f1x, &S->f2x, &S->f1y, &S->f2y, &S->f1z, &S->f2z,
                      &S->g1x, &S->g2x, &S->g1y, &S->g2y, &S->g1z, &S->g2z};
  for (int q = 0; q < 12; q++) *arr[q] = zalloc(cn);
#define CI(i, j, k) ((int64_t)(i) + (int64_t)J->px * ((int64_t)((j) - S->j0) + (int64_t)rows * (int64_t)(k)))
  int kl = dim == 3 ? 1 : 0, kh = dim == 3 ? nz : 0;
  int il = dim >= 2 ? 1 : 0, ih = dim >= 2 ? nx : 0;
  /* allocate_vars defaults: f1=1, f2=Ku/epr, g1=1, g2=Ku */
  for (int k = kl; k <= kh; k++)
    for (int j = S->j0; j <= S->j1; j++)
      for (int i = il; i <= ih; i++) {
        int64_t c = CI(i, j, k);
        S->f1x[c] = 1.0; S->f1y[c] = 1.0; S->f1z[c] = 1.0;
        S->f2x[c] = Ku / epr; S->f2y[c] = Ku / epr; S->f2z[c] = Ku / epr;
        S->g1x[c] = 1.0; S->g1y[c] = 1.0; S->g1z[c] = 1.0;
        S->g2x[c] = Ku; S->g2y[c] = Ku; S->g2z[c] = Ku;
      }
  int yi = side == 0 ? 1 : S->jb, yf = side == 0 ? npmly : Ny;
  /* x profiles in the slab corners: init_varx1 / init_varx2 */
  int npmlx_lo = p->npml[0][0], npmlx_hi = p->npml[0][1] > 0 ? p->npml[0][1] : p->npml[0][0];
  if (dim >= 2 && npmlx_lo > 0) {
    int npmlx = npmlx_lo;
    for (int k = kl; k <= kh; k++)
      for (int j = yi; j <= yf; j++)
        for (int i = 1; i <= npmlx; i++) {
          int64_t c = CI(i, j, k);
          double sE = ep * sigmam * pow(((double)(npmlx - i) + 0.5) / (double)npmlx, order);
          double aE = sE * dt / ep;
          S->f1x[c] = exp(-aE);
          S->f2x[c] = (1.0 - S->f1x[c]) / (z0 * sE * ds);
          if (i < npmlx) {
            double sH = K_MU0 * sigmam * pow(((double)(npmlx - i)) / (double)npmlx, order);
            double aH = sH * dt / K_MU0;
            S->g1x[c] = exp(-aH);
            S->g2x[c] = z0 * (1.0 - S->g1x[c]) / (sH * ds);
          }
        }
    npmlx = npmlx_hi;
    int xBDhigh = nx - npmlx + 1;
    for (int k = kl; k <= kh; k++)
      for (int j = yi; j <= yf; j++) {
        int ii = npmlx;
        for (int i = xBDhigh; i <= nx; i++) {
          int64_t c = CI(i, j, k);
          if (ii < npmlx) {
            double sE = ep * sigmam * pow(((double)(npmlx - ii)) / (double)npmlx, order);
            double aE = sE * dt / ep;
            S->f1x[c] = exp(-aE);
            S->f2x[c] = (1.0 - S->f1x[c]) / (z0 * sE * ds);
          }
          double sH = K_MU0 * sigmam * pow(((double)(npmlx - ii) + 0.5) / (double)npmlx, order);
          double aH = sH * dt / K_MU0;
          S->g1x[c] = exp(-aH);
          S->g2x[c] = z0 * (1.0 - S->g1x[c]) / (sH * ds);
          ii = ii - 1;
        }
      }
  }
  /* y profile: M3/BERpmly_mod.f90:674-714 */
  for (int k = kl; k <= kh; k++)
    for (int i = il; i <= ih; i++) {
      if (side == 0) {
        for (int j = 1; j <= npmly; j++) {
          int64_t c = CI(i, j, k);
          double sE = eplow * sigmam * pow(((double)(npmly - j) + 0.5) / (double)npmly, order);
          double aE = sE * dt / eplow;
          S->f1y[c] = exp(-aE);
          S->f2y[c] = (1.0 - S->f1y[c]) / (z0 * sE * ds);
          if (j < npmly) {
            double sH = K_MU0 * sigmam * pow(((double)(npmly - j)) / (double)npmly, order);
            double aH = sH * dt / K_MU0;
            S->g1y[c] = exp(-aH);
            S->g2y[c] = z0 * (1.0 - S->g1y[c]) / (sH * ds);
          }
        }
      } else {
        int jj = npmly;
        for (int j = S->jb; j <= Ny; j++) {
          int64_t c = CI(i, j, k);
          if (jj < npmly) {
            double sE = ephigh * sigmam * pow(((double)(npmly - jj)) / (double)npmly, order);
            double aE = sE * dt / ephigh;
            S->f1y[c] = exp(-aE);
            S->f2y[c] = (1.0 - S->f1y[c]) / (z0 * sE * ds);
          }
          double sH = K_MU0 * sigmam * pow(((double)(npmly - jj) + 0.5) / (double)npmly, order);
          double aH = sH * dt / K_MU0;
          S->g1y[c] = exp(-aH);
          S->g2y[c] = z0 * (1.0 - S->g1y[c]) / (sH * ds);
          jj = jj - 1;
        }
      }
    }
  /* z profiles in the slab: init_varz1 / init_varz2 (3D only) */
  int npmlz_lo = p->npml[2][0], npmlz_hi = p->npml[2][1] > 0 ? p->npml[2][1] : p->npml[2][0];
  if (dim == 3 && npmlz_lo > 0) {
    int npmlz = npmlz_lo;
    for (int k = 1; k <= npmlz; k++)
      for (int j = yi; j <= yf; j++)
        for (int i = 1; i <= nx; i++) {
          int64_t c = CI(i, j, k);
          double sE = ep * sigmam * pow(((double)(npmlz - k) + 0.5) / (double)npmlz, order);
          double aE = sE * dt / ep;
          S->f1z[c] = exp(-aE);
          S->f2z[c] = (1.0 - S->f1z[c]) / (z0 * sE * ds);
          if (k < npmlz) {
            double sH = K_MU0 * sigmam * pow(((double)(npmlz - k)) / (double)npmlz, order);
            double aH = sH * dt / K_MU0;
            S->g1z[c] = exp(-aH);
            S->g2z[c] = z0 * (1.0 - S->g1z[c]) / (sH * ds);
          }
        }
    npmlz = npmlz_hi;
    int zBDhigh = nz - npmlz + 1;
    for (int i = 1; i <= nx; i++)
      for (int j = yi; j <= yf; j++) {
        int kk = npmlz;
        for (int k = zBDhigh; k <= nz; k++) {
          int64_t c = CI(i, j, k);
          if (kk < npmlz) {
            double sE = ep * sigmam * pow(((double)(npmlz - kk)) / (double)npmlz, order);
            double aE = sE * dt / ep;
            S->f1z[c] = exp(-aE);
            S->f2z[c] = (1.0 - S->f1z[c]) / (z0 * sE * ds);
          }
          double sH = K_MU0 * sigmam * pow(((double)(npmlz - kk) + 0.5) / (double)npmlz, order);
          double aH = sH * dt / K_MU0;
          S->g1z[c] = exp(-aH);
          S->g2z[c] = z0 * (1.0 - S->g1z[c]) / (sH * ds);
          kk = kk - 1;
        }
      }
  }
#undef CI
}

/* SPLIT PML: the reference's graded profiles (M3/BERpmly_mod.f90:674-714 for
 * y, :761-874 for x and z) applied independently on every axis that has a
 * layer.  Tables are 0-based over the axis; cells outside every layer keep
 * f1=1, f2=Ku/eps, g1=1, g2=Ku. */
static void init_split_tables(ora_job *J) {
  const fdtd_pml_desc *p = &J->pml;
  double dt = J->g.dt, ds = J->g.ds, sigmam = p->sigma_max, order = p->order;
  double ep = p->eps_lo * K_EP0;
  double Ku = dt * K_C0 / ds, epr = ep / K_EP0, z0 = sqrt(K_MU0 / K_EP0);
  for (int a = 0; a < 3; a++) {
    int N = J->g.n[a];
    J->cf1[a] = zalloc(N); J->cf2[a] = zalloc(N); J->cg1[a] = zalloc(N); J->cg2[a] = zalloc(N);
    for (int x = 0; x < N; x++) { J->cf1[a][x] = 1.0; J->cf2[a][x] = Ku / epr; J->cg1[a][x] = 1.0; J->cg2[a][x] = Ku; }
    int lo = p->npml[a][0], hi = p->npml[a][1];
    if (J->g.periodic[a]) lo = hi = 0;
    for (int i1 = 1; i1 <= lo; i1++) {          /* 1-based, low side */
      int x = i1 - 1;
      double sE = ep * sigmam * pow(((double)(lo - i1) + 0.5) / (double)lo, order);
      double aE = sE * dt / ep;
      J->cf1[a][x] = exp(-aE);
      J->cf2[a][x] = (1.0 - J->cf1[a][x]) / (z0 * sE * ds);
      if (i1 < lo) {
        double sH = K_MU0 * sigmam * pow(((double)(lo - i1)) / (double)lo, order);
        double aH = sH * dt / K_MU0;
        J->cg1[a][x] = exp(-aH);
        J->cg2[a][x] = z0 * (1.0 - J->cg1[a][x]) / (sH * ds);
      }
    }
    if (hi > 0) {
      int ii = hi;
      for (int i1 = N - hi + 1; i1 <= N; i1++) {
        int x = i1 - 1;
        if (ii < hi) {
          double sE = ep * sigmam * pow(((double)(hi - ii)) / (double)hi, order);
          double aE = sE * dt / ep;
          J->cf1[a][x] = exp(-aE);
          J->cf2[a][x] = (1.0 - J->cf1[a][x]) / (z0 * sE * ds);
        }
        double sH = K_MU0 * sigmam * pow(((double)(hi - ii) + 0.5) / (double)hi, order);
        double aH = sH * dt / K_MU0;
        J->cg1[a][x] = exp(-aH);
        J->cg2[a][x] = z0 * (1.0 - J->cg1[a][x]) / (sH * ds);
        ii = ii - 1;
      }
    }
    J->shell_lo[a] = lo;
    J->shell_hi[a] = N - 1 - hi;
  }
}

int ora_commit(ora_job *J) {
  if (J->committed) FAIL("already committed");
  int nx = J->nx, ny = J->ny, nz = J->nz;
  int split = J->pml_mode == FDTD_PML_SPLIT;
  if (split) {
    /* the Yee update and the materials run on the interior box; the shell
       cells belong to the PML */
    init_split_tables(J);
    for (int a = 0; a < 3; a++) {
      J->g.main_lo[a] = J->shell_lo[a];
      J->g.main_hi[a] = J->shell_hi[a];
    }
    if (J->dim == 2) { J->g.main_lo[2] = 0; J->g.main_hi[2] = 0; }
  }
  /* paint materials in call order */
  for (int m = 1; m <= J->nmat; m++) {
    const fdtd_region *r = &J->mat[m].region;
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
          if (inside_region(J, r, i, j, k)) J->matid[cell_ix(J, i, j, k)] = (uint8_t)m;
  }
  for (int m = 1; m <= J->nmat; m++) {
    omat *M = &J->mat[m];
    int64_t cnt = 0;
    for (int k = 0; k < nz; k++) for (int j = 0; j < ny; j++) for (int i = 0; i < nx; i++)
      if (J->matid[cell_ix(J, i, j, k)] == m && !(split && in_shell(J, i, j, k))) cnt++;
    M->ncell = cnt;
    M->cells = (int64_t *)malloc(sizeof(int64_t) * (size_t)(cnt > 0 ? cnt : 1));
    cnt = 0;
    /* the reference loops i-outer (M2/gold_mod.f90:55-56); each cell is independent */
    for (int k = 0; k < nz; k++) for (int j = 0; j < ny; j++) for (int i = 0; i < nx; i++)
      if (J->matid[cell_ix(J, i, j, k)] == m && !(split && in_shell(J, i, j, k)))
        M->cells[cnt++] = cell_ix(J, i, j, k);
    if (M->kind == MAT_GOLD || M->kind == MAT_GRAPHENE || M->kind == MAT_GRAPHENE_CP) {
      for (int c = 0; c < 3; c++) {
        if (M->kind == MAT_GRAPHENE_CP)
          for (int q = 0; q < 4; q++) M->cg[c][q] = (cplx *)calloc((size_t)(cnt > 0 ? cnt : 1), sizeof(cplx));
        M->I[c] = zalloc(cnt); M->S[c] = zalloc(cnt);
        M->g1[c] = (cplx *)calloc((size_t)(cnt > 0 ? cnt : 1), sizeof(cplx));
        M->g2[c] = (cplx *)calloc((size_t)(cnt > 0 ? cnt : 1), sizeof(cplx));
        M->SR[c] = zalloc(cnt); M->SRm1[c] = zalloc(cnt); M->SRm2[c] = zalloc(cnt);
      }
    } else if (M->kind == MAT_LORENTZ_JP || M->kind == MAT_LORENTZ_S) {
      for (int c = 0; c < 3; c++) {
        M->JpT[c] = zalloc(cnt); M->Qk[c] = zalloc(cnt); M->Gk[c] = zalloc(cnt);
        for (int l = 0; l < M->npoles; l++) {
          M->P[c][l] = zalloc(cnt); M->Jp[c][l] = zalloc(cnt);
          M->Sm1[c][l] = zalloc(cnt); M->Sm2[c][l] = zalloc(cnt);
        }
      }
    }
  }
  if (J->pml_mode == FDTD_PML_REFERENCE) {
    int npmly = J->pml.npml[1][0];
    if (npmly > 0) {
      init_ref_slab(J, &J->slab[0], 0, J->pml.eps_lo, J->pml.eps_hi, npmly);
      init_ref_slab(J, &J->slab[1], 1, J->pml.eps_lo, J->pml.eps_hi, npmly);
    }
  } else if (J->pml_mode == FDTD_PML_SPLIT) {
    int nsplit = J->dim == 3 ? 12 : 2;
    for (int q = 0; q < nsplit; q++) J->sp[q] = zalloc(J->ntot);
  }
  if (J->tfbox) {
    const int n3[3] = {nx, ny, nz};
    for (int a = 0; a < 3; a++)
      J->tb_face[a] = (a == 1) || (a < J->dim && !(J->g.periodic[a] && J->tb.lo[a] == 0 && J->tb.hi[a] == n3[a] - 1));
    const int *lo = J->tb.lo, *hi = J->tb.hi;
    if (lo[1] < 1 || hi[1] > ny - 2 || hi[1] <= lo[1]) FAIL("TFSF box rows must satisfy 1 <= lo < hi <= ny-2");
    for (int a = 0; a < 3; a += 2)
      if (J->tb_face[a] && (lo[a] < 1 || hi[a] > n3[a] - 2 || hi[a] <= lo[a]))
        FAIL("TFSF box faces on axis %d must lie inside the grid", a);
    J->le = zalloc(ny); J->lh = zalloc(ny);
  }
  if (J->tfsf) {
    J->exi = zalloc(J->ntot); J->hzi = zalloc(J->ntot);
    if (J->pml_mode == FDTD_PML_REFERENCE && J->pml.npml[1][0] > 0) {
      /* mypmly_inc%initialize(air_ep*ep0, air_ep*ep0, ...) (P1/program.f90:134) */
      init_ref_slab(J, &J->islab[0], 0, J->tf.eps_lo, J->tf.eps_hi, J->pml.npml[1][0]);
      init_ref_slab(J, &J->islab[1], 1, J->tf.eps_lo, J->tf.eps_hi, J->pml.npml[1][0]);
    }
  }
  J->committed = 1;
  return 0;
}

static double gauss_t(const fdtd_source_desc *s, double t);

/* ---- 2D/3D total-field/scattered-field box --------------------------------- */
/* The incident plane wave runs along +y on its own line, E at rows j and H
 * between j and j+1, with the main grid's differences: Ez/Hx for 3D and 2D TM
 * (update_ezincz / update_hxincy, P3/include/myTFSF_incEzHx_3Dfunc.f90:80-99),
 * Ex/Hz for 2D TE (the TE grid's own updateD/updateH,
 * P2/include/myfdtd_2Dfunc.f90:16-44).  Its ends are the two-step absorbing
 * boundary of ezincy_boundaryCond (P3/include/myTFSF_incEzHx_3Dfunc.f90:101-113). */
int ora_add_tfsf(ora_job *J, const fdtd_tfsf_desc *t) {
  if (J->committed) FAIL("job already committed");
  if (J->dim < 2) FAIL("the TFSF box is 2D/3D; 1D uses ora_add_tfsf_1d");
  if (!(t->eps_line > 0.0)) FAIL("eps_line must be positive");
  J->tfbox = 1; J->tb = *t;
  return 0;
}

/* sign of the line's differences: +1 for Ex/Hz (TE), -1 for Ez/Hx */
static double tb_sign(const ora_job *J) { return J->g.layout == FDTD_LAYOUT_2D_TE ? 1.0 : -1.0; }

static void tfbox_line_E(ora_job *J, int n) {
  const int ny = J->ny;
  const double cb = J->g.ku / J->tb.eps_line, sg = tb_sign(J);
  double *e = J->le, *h = J->lh;
  for (int j = 1; j <= ny - 2; j++) e[j] = e[j] + cb * (sg * (h[j] - h[j - 1]));
  const double t = (double)(n - 1) * J->g.dt;
  for (int q = 0; q < J->nsrc; q++) {
    const fdtd_source_desc *d = &J->src[q].d;
    if (d->component != FDTD_E_INC) continue;
    const double g = gauss_t(d, t) * d->amp;
    for (int j = d->lo[1]; j <= d->hi[1]; j++) e[j] = e[j] + g;
  }
  e[0] = J->labc[1]; J->labc[1] = J->labc[0]; J->labc[0] = e[1];
  e[ny - 1] = J->labc[3]; J->labc[3] = J->labc[2]; J->labc[2] = e[ny - 2];
}

static void tfbox_line_H(ora_job *J) {
  const int ny = J->ny;
  const double Ku = J->g.ku, sg = tb_sign(J);
  double *e = J->le, *h = J->lh;
  for (int j = 0; j <= ny - 2; j++) h[j] = h[j] + Ku * (sg * (e[j + 1] - e[j]));
}

/* the incident terms of the D updates that cross a face (consistCond_dz /
   consistCond_dy, P3/include/myTFSF_incEzHx_3Dfunc.f90:117-170; TE: Ex at the
   y faces and Ey at the x faces) */
static void tfbox_faces_D(ora_job *J) {
  const int *lo = J->tb.lo, *hi = J->tb.hi;
  const double Ku = J->g.ku;
  const double *h = J->lh;
  const int k0 = J->dim == 3 ? lo[2] : 0, k1 = J->dim == 3 ? hi[2] : 0;
  if (J->g.layout == FDTD_LAYOUT_2D_TE) {
    double *dx = J->F[DX], *dy = J->F[DY];
    for (int i = lo[0]; i <= hi[0]; i++) {
      int64_t a = cell_ix(J, i, lo[1], 0), b = cell_ix(J, i, hi[1], 0);
      dx[a] = dx[a] - Ku * h[lo[1] - 1];
      dx[b] = dx[b] + Ku * h[hi[1]];
    }
    if (J->tb_face[0])
      for (int j = lo[1]; j <= hi[1] - 1; j++) {
        int64_t a = cell_ix(J, lo[0], j, 0), b = cell_ix(J, hi[0] + 1, j, 0);
        dy[a] = dy[a] + Ku * h[j];
        dy[b] = dy[b] - Ku * h[j];
      }
    return;
  }
  double *dy = J->F[DY], *dz = J->F[DZ];
  for (int k = k0; k <= k1; k++)
    for (int i = lo[0]; i <= hi[0]; i++) {
      int64_t a = cell_ix(J, i, lo[1], k), b = cell_ix(J, i, hi[1], k);
      dz[a] = dz[a] + Ku * h[lo[1] - 1];
      dz[b] = dz[b] - Ku * h[hi[1]];
    }
  if (J->dim == 3 && J->tb_face[2])
    for (int j = lo[1]; j <= hi[1] - 1; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        int64_t a = cell_ix(J, i, j, lo[2]), b = cell_ix(J, i, j, hi[2] + 1);
        dy[a] = dy[a] - Ku * h[j];
        dy[b] = dy[b] + Ku * h[j];
      }
}

/* the incident terms of the H updates that cross a face (consistCond_hx /
   consistCond_hy, P3/include/myTFSF_incEzHx_3Dfunc.f90:172-221; TE: Hz at the
   y faces) */
static void tfbox_faces_H(ora_job *J) {
  const int *lo = J->tb.lo, *hi = J->tb.hi;
  const double Ku = J->g.ku;
  const double *e = J->le;
  const int k0 = J->dim == 3 ? lo[2] : 0, k1 = J->dim == 3 ? hi[2] : 0;
  if (J->g.layout == FDTD_LAYOUT_2D_TE) {
    double *hz = J->F[HZ];
    for (int i = lo[0]; i <= hi[0]; i++) {
      int64_t a = cell_ix(J, i, lo[1] - 1, 0), b = cell_ix(J, i, hi[1], 0);
      hz[a] = hz[a] - Ku * e[lo[1]];
      hz[b] = hz[b] + Ku * e[hi[1]];
    }
    return;
  }
  double *hx = J->F[HX], *hy = J->F[HY];
  for (int k = k0; k <= k1; k++)
    for (int i = lo[0]; i <= hi[0]; i++) {
      int64_t a = cell_ix(J, i, lo[1] - 1, k), b = cell_ix(J, i, hi[1], k);
      hx[a] = hx[a] + Ku * e[lo[1]];
      hx[b] = hx[b] - Ku * e[hi[1]];
    }
  if (J->tb_face[0])
    for (int k = k0; k <= k1; k++)
      for (int j = lo[1]; j <= hi[1]; j++) {
        int64_t a = cell_ix(J, lo[0] - 1, j, k), b = cell_ix(J, hi[0], j, k);
        hy[a] = hy[a] - Ku * e[j];
        hy[b] = hy[b] + Ku * e[j];
      }
}

/* ---- helpers for the loop ------------------------------------------------- */
static double gauss_t(const fdtd_source_desc *s, double t) {
  /* dexp(-0.5d0*((t-t0)/st)**2)*dsin(w0*t)  (P2/program.f90:337) */
  double a = (t - s->t0) / s->st;
  return exp(-0.5 * (a * a)) * sin(s->w0 * t);
}

static int in_main(const ora_job *J, int i0, int j0, int k0) {
  const fdtd_grid_desc *g = &J->g;
  return i0 >= g->main_lo[0] && i0 <= g->main_hi[0] && j0 >= g->main_lo[1] && j0 <= g->main_hi[1] &&
         k0 >= g->main_lo[2] && k0 <= g->main_hi[2];
}

/* ---- materials: update_E -------------------------------------------------- */
/* curl H of E component a at padded cell c, as the E-form update_EJp writes
   it (M3/goldLorentzJp_mod.f90:53-58, M2/siLorentzJp_mod.f90:54-55); the 1D
   line is the 2D TE Ex row along y */
static double curl_at(const ora_job *J, int a, int64_t c) {
  const double *hx = J->F[HX], *hy = J->F[HY], *hz = J->F[HZ];
  const int64_t sy = J->px, sz = (int64_t)J->px * J->py;
  if (J->g.layout == FDTD_LAYOUT_3D) {
    if (a == 0) return (hz[c] - hz[c - sy]) + (-hy[c] + hy[c - sz]);
    if (a == 1) return (hx[c] - hx[c - sz]) + (-hz[c] + hz[c - 1]);
    return (hy[c] - hy[c - 1]) + (-hx[c] + hx[c - sy]);
  }
  if (J->g.layout == FDTD_LAYOUT_2D_TM) return (hy[c] - hy[c - 1]) + (-hx[c] + hx[c - sy]);
  if (a == 0) return hz[c] - hz[c - sy];
  return -hz[c] + hz[c - 1];
}

/* what updateD adds to D at cell c beside Ku*curl: the soft sources and the
   1D TFSF correction (P1/program.f90:229-235) */
static double d_extra_at(const ora_job *J, int n, int a, int64_t c) {
  const int64_t ii = c % J->px, jj = (c / J->px) % J->py, kk = c / ((int64_t)J->px * J->py);
  const int i = J->dim >= 2 ? (int)ii - 1 : 0, j = (int)jj - 1, k = J->dim == 3 ? (int)kk - 1 : 0;
  const double t = (double)(n - 1) * J->g.dt;
  double s = 0.0;
  for (int q = 0; q < J->nsrc; q++) {
    const fdtd_source_desc *d = &J->src[q].d;
    if (d->component != a) continue;
    if (i < d->lo[0] || i > d->hi[0] || j < d->lo[1] || j > d->hi[1] || k < d->lo[2] || k > d->hi[2]) continue;
    s += gauss_t(d, t) * d->amp;
  }
  if (J->tfsf && J->dim == 1 && c == J->tf.boundary + 1) s -= J->g.ku * J->hzi[c - 1];
  return s;
}

static void materials_update_E(ora_job *J, int n) {
  double *E[3] = {J->F[EX], J->F[EY], J->F[EZ]};
  double *D[3] = {J->F[DX], J->F[DY], J->F[DZ]};
  int ncomp_list[3], nc = 0;
  if (J->g.layout == FDTD_LAYOUT_2D_TE) { ncomp_list[0] = 0; ncomp_list[1] = 1; nc = 2; }
  else if (J->g.layout == FDTD_LAYOUT_2D_TM) { ncomp_list[0] = 2; nc = 1; }
  else if (J->g.layout == FDTD_LAYOUT_1D) { ncomp_list[0] = 0; nc = 1; }
  else { ncomp_list[0] = 0; ncomp_list[1] = 1; ncomp_list[2] = 2; nc = 3; }
  for (int m = 1; m <= J->nmat; m++) {
    omat *M = &J->mat[m];
    if (M->kind == MAT_DIEL) {
      /* E = D*gax (M2/simpledielectric_mod.f90:141-146) */
#pragma omp parallel for num_threads(J->nth) schedule(static) if (J->nth > 1)
      for (int64_t q = 0; q < M->ncell; q++) {
        int64_t c = M->cells[q];
        for (int u = 0; u < nc; u++) { int a = ncomp_list[u]; E[a][c] = D[a][c] * M->gax; }
      }
    } else if (M->kind == MAT_GOLD) {
      /* M2/gold_mod.f90:57-71, M3/gold_mod.f90:61-82 */
#pragma omp parallel for num_threads(J->nth) schedule(static) if (J->nth > 1)
      for (int64_t q = 0; q < M->ncell; q++) {
        int64_t c = M->cells[q];
        for (int u = 0; u < nc; u++) {
          int a = ncomp_list[u];
          double r = (D[a][c] - M->I[a][q]) + M->ha * M->S[a][q];
          cplx num = {r, 0.0};
          num = cadd(num, cmul(M->gb[0], M->g1[a][q]));
          num = cadd(num, cmul(M->gb[1], M->g2[a][q]));
          double e = cdiv_re(num, M->ga);
          E[a][c] = e;
          M->I[a][q] = M->I[a][q] + M->hb * e;
          M->S[a][q] = M->ha * M->S[a][q] + M->hb * e;
          M->g1[a][q] = cadd(cmul(M->gb[0], M->g1[a][q]), cscale(M->gc[0], e));
          M->g2[a][q] = cadd(cmul(M->gb[1], M->g2[a][q]), cscale(M->gc[1], e));
        }
      }
    } else if (M->kind == MAT_GRAPHENE) {
      for (int64_t q = 0; q < M->ncell; q++) {
        int64_t c = M->cells[q];
        for (int u = 0; u < nc; u++) {
          int a = ncomp_list[u];
          if (a == M->normal) { E[a][c] = D[a][c]; continue; }   /* out-of-plane: vacuum */
          double eo = E[a][c];
          /* E = (D - I + ha*S + 2 kerr E^3)/(ga + S_R + 3 kerr E^2) (M1/graphene633_mod.f90:33-35) */
          double num = (D[a][c] - M->I[a][q]) + M->g_ha * M->S[a][q] + 2.0 * M->kerr * (eo * eo * eo);
          double den = (M->g_ga + M->SR[a][q]) + 3.0 * M->kerr * (eo * eo);
          double e = num / den;
          E[a][c] = e;
          /* S_R(n) = r1 S_R(n-1) + r2 S_R(n-2) + r0 E^2 (M3/graphene_mod.f90:73-76) */
          double sr = M->r1 * M->SRm1[a][q] + M->r2 * M->SRm2[a][q] + M->r0 * (e * e);
          M->SR[a][q] = sr; M->SRm2[a][q] = M->SRm1[a][q]; M->SRm1[a][q] = sr;
          M->I[a][q] = M->I[a][q] + M->g_hb * e;
          M->S[a][q] = M->g_ha * M->S[a][q] + M->g_hb * e;
        }
      }
    } else if (M->kind == MAT_GRAPHENE_CP) {
      /* E = (D - I + ha S + gb1 g1 + .. + gb4 g4)/(gax + S_R), real part;
         S_R = r1 S_R(n-1) + r2 S_R(n-2) + r0 E^2; I += hb E; S = ha S + hb E;
         g_p = gb_p g_p + gc_p E (M3/graphene_mod.f90:70-100, M2/graphene_mod.f90:70-88,
         M1/graphene_mod.f90:59-68).  The normal component: Ey = Dy
         (M2/graphene_mod.f90:68; the 3D module leaves Ey to the material
         updated before it, vacuum for a sheet in air). */
      for (int64_t q = 0; q < M->ncell; q++) {
        int64_t c = M->cells[q];
        for (int u = 0; u < nc; u++) {
          int a = ncomp_list[u];
          if (a == M->c_normal) { E[a][c] = D[a][c]; continue; }
          double r = (D[a][c] - M->I[a][q]) + M->c_ha * M->S[a][q];
          cplx num = {r, 0.0};
          for (int p = 0; p < 4; p++) num = cadd(num, cmul(M->cgb[p], M->cg[a][p][q]));
          cplx den = M->cgax; den.re = den.re + M->SR[a][q];
          double e = cdiv_re(num, den);
          E[a][c] = e;
          double sr = M->c_r1 * M->SRm1[a][q] + M->c_r2 * M->SRm2[a][q] + M->c_r0 * (e * e);
          M->SR[a][q] = sr; M->SRm2[a][q] = M->SRm1[a][q]; M->SRm1[a][q] = sr;
          M->I[a][q] = M->I[a][q] + M->c_hb * e;
          M->S[a][q] = M->c_ha * M->S[a][q] + M->c_hb * e;
          for (int p = 0; p < 4; p++) M->cg[a][p][q] = cadd(cmul(M->cgb[p], M->cg[a][p][q]), cscale(M->cgc[p], e));
        }
      }
    } else if (M->kind == MAT_LORENTZ_JP) {
      /* E += Ku ga (curl - ds JpT); JpT = sum_l Jp_l with
         Jp_l = gamma1L Jp_l + gamma2L (xi_l E/c0 - P_l), P_l += dt Jp_l
         (M3/goldLorentzJp_mod.f90:60-86, M2/siLorentzJp_mod.f90:57-77) */
      /* the sheet's normal component: Ey += Ku (curlhxz + curlhzx), vacuum
         (M3/graphene3LorentzJp1nm_mod.f90:66, M2/...:60); the Kerr term of
         pole 1 (:74-77) and its G, Q recursion (:89-95) */
      /* SLG_LJp's Ez line subtracts JpxT (M3/grapheneLorentzJp_mod.f90:68):
         the x sum of the previous step, as all E lines of a cell run before
         its Jp updates (:62-70) */
      const double Ku = J->g.ku, ds = J->g.ds, dt = J->g.dt;
      for (int64_t q = 0; q < M->ncell; q++) {
        int64_t c = M->cells[q];
        const double jpx_old = M->JpT[0][q];
        for (int u = 0; u < nc; u++) {
          int a = ncomp_list[u];
          if (M->l_sheet && a == M->l_normal) {
            E[a][c] = E[a][c] + Ku * curl_at(J, a, c) + d_extra_at(J, n, a, c);
            continue;
          }
          const double jt_e = (M->l_zx && a == 2) ? jpx_old : M->JpT[a][q];
          double e = E[a][c] + Ku * M->l_ga * (curl_at(J, a, c) - ds * jt_e);
          e = e + M->l_ga * d_extra_at(J, n, a, c);
          E[a][c] = e;
          double jt = 0.0;
          for (int l = 0; l < M->npoles; l++) {
            double p0 = M->xi[l] * e / K_C0;
            if (l == 0 && M->chi3 != 0.0) p0 = p0 + M->chi3 * M->Qk[a][q] * e / K_C0;
            double jp = M->g1L[l] * M->Jp[a][l][q] + M->g2L[l] * (p0 - M->P[a][l][q]);
            M->Jp[a][l][q] = jp;
            M->P[a][l][q] = M->P[a][l][q] + dt * jp;
            jt = jt + jp;
          }
          M->JpT[a][q] = jt;
          if (M->chi3 != 0.0) {
            const double ez = M->escale * e;
            M->Gk[a][q] = M->g1N * M->Gk[a][q] + M->g2N * ((ez * ez) - M->Qk[a][q]);
            M->Qk[a][q] = M->Qk[a][q] + dt * M->Gk[a][q];
          }
        }
      }
    } else if (M->kind == MAT_LORENTZ_S) {
      /* E = D - S_1 - S_2 - S_3; S_l(n) = ga_l S_l(n-1) + gb_l S_l(n-2) + gc_l E
         (M3/si_mod.f90:55-60, M1/si_mod.f90:43-48); E is scaled by 1/eps_inf,
         which is 1 in the reference */
      for (int64_t q = 0; q < M->ncell; q++) {
        int64_t c = M->cells[q];
        for (int u = 0; u < nc; u++) {
          int a = ncomp_list[u];
          double e = D[a][c];
          for (int l = 0; l < M->npoles; l++) e = e - M->Sm1[a][l][q];
          e = e * M->l_ga;
          E[a][c] = e;
          for (int l = 0; l < M->npoles; l++) {
            double sn = M->sa[l] * M->Sm1[a][l][q] + M->sb[l] * M->Sm2[a][l][q] + M->sc[l] * e;
            M->Sm2[a][l][q] = M->Sm1[a][l][q];
            M->Sm1[a][l][q] = sn;
          }
        }
      }
    }
  }
}

/* ---- sources --------------------------------------------------------------- */
static void apply_sources(ora_job *J, int n, int incident) {
  double t = (double)(n - 1) * J->g.dt;           /* t=real(n-1,8)*dt */
  for (int q = 0; q < J->nsrc; q++) {
    const fdtd_source_desc *s = &J->src[q].d;
    int inc = s->component == FDTD_EX_INC;
    if (inc != incident) continue;
    double g = gauss_t(s, t);
    double *D;
    if (inc) D = J->exi;
    else D = J->F[DX + s->component];
    for (int k = s->lo[2]; k <= s->hi[2]; k++)
      for (int j = s->lo[1]; j <= s->hi[1]; j++)
        for (int i = s->lo[0]; i <= s->hi[0]; i++) {
          if (!inc && !in_main(J, i, j, k)) continue;   /* D is only updated on main cells */
          int64_t c = cell_ix(J, i, j, k);
          if (inc) D[c] = D[c] + g;                  /* ex_inc=ex_inc+gauss_t (P1/program.f90:229) */
          else D[c] = D[c] + g * s->amp;             /* Dx=Dx+gauss_t*n_air (P3/program.f90:403) */
        }
  }
}

/* ---- 2D TE (Hz, Ex, Ey): P2 ------------------------------------------------ */
static void te2d_updateD(ora_job *J) {
  /* P2/include/myfdtd_2Dfunc.f90:16-30 */
  double *hz = J->F[HZ], *dx = J->F[DX], *dy = J->F[DY];
  double Ku = J->g.ku;
  /* the reference loops i-outer; every cell is independent, so the
     cache-friendly order gives the same values */
#pragma omp parallel for num_threads(J->nth) schedule(static) if (J->nth > 1)
  for (int j = J->g.main_lo[1] + 1; j <= J->g.main_hi[1] + 1; j++)
    for (int i = J->g.main_lo[0] + 1; i <= J->g.main_hi[0] + 1; i++) {
      double curlhx = hz[IX(J, i, j, 0)] - hz[IX(J, i - 1, j, 0)];
      double curlhy = hz[IX(J, i, j, 0)] - hz[IX(J, i, j - 1, 0)];
      dx[IX(J, i, j, 0)] = dx[IX(J, i, j, 0)] + Ku * curlhy;
      dy[IX(J, i, j, 0)] = dy[IX(J, i, j, 0)] - Ku * curlhx;
    }
}

static void te2d_updateH(ora_job *J) {
  /* P2/include/myfdtd_2Dfunc.f90:34-44 */
  double *hz = J->F[HZ], *ex = J->F[EX], *ey = J->F[EY];
  double Ku = J->g.ku;
#pragma omp parallel for num_threads(J->nth) schedule(static) if (J->nth > 1)
  for (int j = J->g.main_lo[1] + 1; j <= J->g.main_hi[1] + 1; j++)
    for (int i = J->g.main_lo[0] + 1; i <= J->g.main_hi[0] + 1; i++) {
      double curlE = ey[IX(J, i + 1, j, 0)] - ey[IX(J, i, j, 0)] - ex[IX(J, i, j + 1, 0)] + ex[IX(J, i, j, 0)];
      hz[IX(J, i, j, 0)] = hz[IX(J, i, j, 0)] - Ku * curlE;
    }
}

/* slab-local index: 1-based (i, j) with i in 0..N_x+1 */
#define SX(S, i, j, k) ((int64_t)(i) + (int64_t)J->px * ((int64_t)((j) - (S)->j0) + (int64_t)((S)->j1 - (S)->j0 + 1) * (int64_t)(k)))

static void te2d_pml_E(ora_job *J) {
  /* M2/BERpmly_HzExEy_mod.f90:58-74, updateEs :96-123, setboundayEya/b :144-178, setPecE :193-207 */
  double *HzM = J->F[HZ], *ExM = J->F[EX];
  int nx = J->nx;
  for (int s = 0; s < 2; s++) {
    oslab *S = &J->slab[s];
    if (!S->on) continue;
    double *Ex = S->f[S2_EX], *Ey = S->f[S2_EY], *Hzx = S->f[S2_HZX], *Hzy = S->f[S2_HZY];
    int yi = s == 0 ? 1 : S->jb, yf = s == 0 ? S->ja : J->ny;
    int ja = S->ja, jb = S->jb;
    for (int j = yi; j <= yf; j++)
      for (int i = 1; i <= nx; i++) {
        double curlHzx_p = -Hzx[SX(S, i, j, 0)] - Hzy[SX(S, i, j, 0)];
        double curlHzx_m = Hzx[SX(S, i - 1, j, 0)] + Hzy[SX(S, i - 1, j, 0)];
        double curlHzy_p = Hzx[SX(S, i, j, 0)] + Hzy[SX(S, i, j, 0)];
        double curlHzy_m = (j - 1 >= S->j0) ? -Hzx[SX(S, i, j - 1, 0)] - Hzy[SX(S, i, j - 1, 0)] : 0.0;
        if (s == 0 && j == ja) curlHzy_p = HzM[IX(J, i, j, 0)];
        if (s == 1 && j == jb) curlHzy_m = -HzM[IX(J, i, j - 1, 0)];
        int64_t c = SX(S, i, j, 0);
        Ex[c] = S->f1y[c] * Ex[c] + S->f2y[c] * (curlHzy_p + curlHzy_m);
        Ey[c] = S->f1x[c] * Ey[c] + S->f2x[c] * (curlHzx_p + curlHzx_m);
      }
    /* copy-back Ex over j=1..ja (low) or jb..N_y (high), i=0..N_x+1 */
    for (int j = yi; j <= yf; j++)
      for (int i = 0; i <= nx + 1; i++) ExM[IX(J, i, j, 0)] = Ex[SX(S, i, j, 0)];
    /* PEC rows */
    int jp = s == 0 ? 0 : J->ny + 1;
    for (int i = 0; i <= nx + 1; i++) Ex[SX(S, i, jp, 0)] = 0.0;
  }
}

static void te2d_pml_H(ora_job *J) {
  /* M2/BERpmly_HzExEy_mod.f90:76-92, updateHs :125-140, setboundayHya/b :156-190, setPecH :209-225 */
  double *HzM = J->F[HZ];
  int nx = J->nx;
  for (int s = 0; s < 2; s++) {
    oslab *S = &J->slab[s];
    if (!S->on) continue;
    double *Ex = S->f[S2_EX], *Ey = S->f[S2_EY], *Hzx = S->f[S2_HZX], *Hzy = S->f[S2_HZY];
    int yi = s == 0 ? 1 : S->jb, yf = s == 0 ? S->ja : J->ny;
    for (int j = yi; j <= yf; j++)
      for (int i = 1; i <= nx; i++) {
        int64_t c = SX(S, i, j, 0);
        double curlExy = Ex[SX(S, i, j + 1, 0)] - Ex[c];
        double curlEyx = -Ey[SX(S, i + 1, j, 0)] + Ey[c];
        Hzy[c] = S->g1y[c] * Hzy[c] + S->g2y[c] * curlExy;
        Hzx[c] = S->g1x[c] * Hzx[c] + S->g2x[c] * curlEyx;
      }
    int cl = s == 0 ? 1 : S->jb, ch = s == 0 ? S->ja - 1 : J->ny;
    for (int j = cl; j <= ch; j++)
      for (int i = 0; i <= nx + 1; i++) HzM[IX(J, i, j, 0)] = Hzy[SX(S, i, j, 0)] + Hzx[SX(S, i, j, 0)];
    int jp = s == 0 ? 0 : J->ny + 1;
    for (int i = 0; i <= nx + 1; i++) { Hzx[SX(S, i, jp, 0)] = 0.0; Hzy[SX(S, i, jp, 0)] = 0.0; }
  }
}

/* interchange_E / interchange_H of P2/include/mympi_2Dfunc.f90:141-272:
 * the y messages connect the stitched slabs (identity here); the x wraps
 * are copies when PBC_x. */
static void wrap_x_both(ora_job *J, double *f, int pz) {
  int nx = J->nx;
  for (int k = 0; k < pz; k++)
    for (int j = 0; j < J->py; j++) {
      f[IX(J, nx + 1, j, k)] = f[IX(J, 1, j, k)];
      f[IX(J, 0, j, k)] = f[IX(J, nx, j, k)];
    }
}
static void wrap_x_low(ora_job *J, double *f) {
  for (int k = 0; k < J->pz; k++)
    for (int j = 0; j < J->py; j++) f[IX(J, 0, j, k)] = f[IX(J, J->nx, j, k)];
}
static void wrap_x_high(ora_job *J, double *f) {
  for (int k = 0; k < J->pz; k++)
    for (int j = 0; j < J->py; j++) f[IX(J, J->nx + 1, j, k)] = f[IX(J, 1, j, k)];
}
static void wrap_y_both(ora_job *J, double *f) {
  int ny = J->ny;
  for (int k = 0; k < J->pz; k++)
    for (int i = 0; i < J->px; i++) {
      f[IX(J, i, ny + 1, k)] = f[IX(J, i, 1, k)];
      f[IX(J, i, 0, k)] = f[IX(J, i, ny, k)];
    }
}
static void wrap_y_low(ora_job *J, double *f) {
  for (int k = 0; k < J->pz; k++)
    for (int i = 0; i < J->px; i++) f[IX(J, i, 0, k)] = f[IX(J, i, J->ny, k)];
}
static void wrap_z_both(ora_job *J, double *f) {
  int nz = J->nz;
  for (int j = 0; j < J->py; j++)
    for (int i = 0; i < J->px; i++) {
      f[IX(J, i, j, nz + 1)] = f[IX(J, i, j, 1)];
      f[IX(J, i, j, 0)] = f[IX(J, i, j, nz)];
    }
}
static void wrap_z_low(ora_job *J, double *f) {
  for (int j = 0; j < J->py; j++)
    for (int i = 0; i < J->px; i++) f[IX(J, i, j, 0)] = f[IX(J, i, j, J->nz)];
}

/* ---- 2D TM (Ez, Hx, Hy): the 3D curls of P3/include/myfdtd_func.f90 with d/dz = 0 */
static void tm2d_updateD(ora_job *J) {
  double *hx = J->F[HX], *hy = J->F[HY], *dz = J->F[DZ];
  double Ku = J->g.ku;
#pragma omp parallel for num_threads(J->nth) schedule(static) if (J->nth > 1)
  for (int j = J->g.main_lo[1] + 1; j <= J->g.main_hi[1] + 1; j++)
    for (int i = J->g.main_lo[0] + 1; i <= J->g.main_hi[0] + 1; i++) {
      double curlhyx = hy[IX(J, i, j, 0)] - hy[IX(J, i - 1, j, 0)];
      double curlhxy = -hx[IX(J, i, j, 0)] + hx[IX(J, i, j - 1, 0)];
      dz[IX(J, i, j, 0)] = dz[IX(J, i, j, 0)] + Ku * (curlhyx + curlhxy);
    }
}
static void tm2d_updateH(ora_job *J) {
  double *hx = J->F[HX], *hy = J->F[HY], *ez = J->F[EZ];
  double Ku = J->g.ku;
#pragma omp parallel for num_threads(J->nth) schedule(static) if (J->nth > 1)
  for (int j = J->g.main_lo[1] + 1; j <= J->g.main_hi[1] + 1; j++)
    for (int i = J->g.main_lo[0] + 1; i <= J->g.main_hi[0] + 1; i++) {
      double curlezy = -ez[IX(J, i, j + 1, 0)] + ez[IX(J, i, j, 0)];
      double curlezx = ez[IX(J, i + 1, j, 0)] - ez[IX(J, i, j, 0)];
      hx[IX(J, i, j, 0)] = hx[IX(J, i, j, 0)] + Ku * curlezy;
      hy[IX(J, i, j, 0)] = hy[IX(J, i, j, 0)] + Ku * curlezx;
    }
}

/* ---- SPLIT PML on any faces (2D TE, 2D TM, 3D) ------------------------------
 * Berenger split of M3/BERpmly_mod.f90:117-195 applied in every shell cell
 * (cells outside the interior box), reading the total fields of the
 * neighbours; the total (sum of the two parts) is written to the main array. */
static int in_shell(const ora_job *J, int i0, int j0, int k0) {
  return i0 < J->shell_lo[0] || i0 > J->shell_hi[0] || j0 < J->shell_lo[1] || j0 > J->shell_hi[1] ||
         (J->dim == 3 && (k0 < J->shell_lo[2] || k0 > J->shell_hi[2]));
}

static void split_E(ora_job *J) {
  double *ex = J->F[EX], *ey = J->F[EY], *ez = J->F[EZ], *hx = J->F[HX], *hy = J->F[HY], *hz = J->F[HZ];
  int L = J->g.layout;
  for (int k0 = 0; k0 < J->nz; k0++)
  #pragma omp parallel for num_threads(J->nth) schedule(static) if (J->nth > 1)
    for (int j0 = 0; j0 < J->ny; j0++)
      for (int i0 = 0; i0 < J->nx; i0++) {
        if (!in_shell(J, i0, j0, k0)) continue;
        int i = i0 + 1, j = j0 + 1, k = J->dim == 3 ? k0 + 1 : 0;
        int64_t c = IX(J, i, j, k);
        double f1x = J->cf1[0][i0], f2x = J->cf2[0][i0], f1y = J->cf1[1][j0], f2y = J->cf2[1][j0];
        if (L == FDTD_LAYOUT_2D_TM) {
          double *Ezx = J->sp[0], *Ezy = J->sp[1];
          Ezx[c] = f1x * Ezx[c] + f2x * (hy[c] - hy[IX(J, i - 1, j, k)]);
          Ezy[c] = f1y * Ezy[c] + f2y * (-hx[c] + hx[IX(J, i, j - 1, k)]);
          ez[c] = Ezx[c] + Ezy[c];
        } else if (L == FDTD_LAYOUT_2D_TE) {
          ex[c] = f1y * ex[c] + f2y * (hz[c] - hz[IX(J, i, j - 1, k)]);
          ey[c] = f1x * ey[c] + f2x * (-hz[c] + hz[IX(J, i - 1, j, k)]);
        } else {
          double f1z = J->cf1[2][k0], f2z = J->cf2[2][k0];
          double **s = J->sp;
          s[S_EXY][c] = f1y * s[S_EXY][c] + f2y * (hz[c] - hz[IX(J, i, j - 1, k)]);
          s[S_EXZ][c] = f1z * s[S_EXZ][c] + f2z * (-hy[c] + hy[IX(J, i, j, k - 1)]);
          s[S_EYZ][c] = f1z * s[S_EYZ][c] + f2z * (hx[c] - hx[IX(J, i, j, k - 1)]);
          s[S_EYX][c] = f1x * s[S_EYX][c] + f2x * (-hz[c] + hz[IX(J, i - 1, j, k)]);
          s[S_EZX][c] = f1x * s[S_EZX][c] + f2x * (hy[c] - hy[IX(J, i - 1, j, k)]);
          s[S_EZY][c] = f1y * s[S_EZY][c] + f2y * (-hx[c] + hx[IX(J, i, j - 1, k)]);
          ex[c] = s[S_EXY][c] + s[S_EXZ][c];
          ey[c] = s[S_EYZ][c] + s[S_EYX][c];
          ez[c] = s[S_EZX][c] + s[S_EZY][c];
        }
      }
}

static void split_H(ora_job *J) {
  double *ex = J->F[EX], *ey = J->F[EY], *ez = J->F[EZ], *hx = J->F[HX], *hy = J->F[HY], *hz = J->F[HZ];
  int L = J->g.layout;
  for (int k0 = 0; k0 < J->nz; k0++)
  #pragma omp parallel for num_threads(J->nth) schedule(static) if (J->nth > 1)
    for (int j0 = 0; j0 < J->ny; j0++)
      for (int i0 = 0; i0 < J->nx; i0++) {
        if (!in_shell(J, i0, j0, k0)) continue;
        int i = i0 + 1, j = j0 + 1, k = J->dim == 3 ? k0 + 1 : 0;
        int64_t c = IX(J, i, j, k);
        double g1x = J->cg1[0][i0], g2x = J->cg2[0][i0], g1y = J->cg1[1][j0], g2y = J->cg2[1][j0];
        if (L == FDTD_LAYOUT_2D_TM) {
          hx[c] = g1y * hx[c] + g2y * (-ez[IX(J, i, j + 1, k)] + ez[c]);
          hy[c] = g1x * hy[c] + g2x * (ez[IX(J, i + 1, j, k)] - ez[c]);
        } else if (L == FDTD_LAYOUT_2D_TE) {
          double *Hzx = J->sp[0], *Hzy = J->sp[1];
          Hzy[c] = g1y * Hzy[c] + g2y * (ex[IX(J, i, j + 1, k)] - ex[c]);
          Hzx[c] = g1x * Hzx[c] + g2x * (-ey[IX(J, i + 1, j, k)] + ey[c]);
          hz[c] = Hzy[c] + Hzx[c];
        } else {
          double g1z = J->cg1[2][k0], g2z = J->cg2[2][k0];
          double **s = J->sp;
          s[S_HXY][c] = g1y * s[S_HXY][c] + g2y * (-ez[IX(J, i, j + 1, k)] + ez[c]);
          s[S_HXZ][c] = g1z * s[S_HXZ][c] + g2z * (ey[IX(J, i, j, k + 1)] - ey[c]);
          s[S_HYZ][c] = g1z * s[S_HYZ][c] + g2z * (-ex[IX(J, i, j, k + 1)] + ex[c]);
          s[S_HYX][c] = g1x * s[S_HYX][c] + g2x * (ez[IX(J, i + 1, j, k)] - ez[c]);
          s[S_HZX][c] = g1x * s[S_HZX][c] + g2x * (-ey[IX(J, i + 1, j, k)] + ey[c]);
          s[S_HZY][c] = g1y * s[S_HZY][c] + g2y * (ex[IX(J, i, j + 1, k)] - ex[c]);
          hx[c] = s[S_HXY][c] + s[S_HXZ][c];
          hy[c] = s[S_HYZ][c] + s[S_HYX][c];
          hz[c] = s[S_HZX][c] + s[S_HZY][c];
        }
      }
}

/* ---- 3D: P3 ----------------------------------------------------------------- */
static void d3_updateD(ora_job *J, int nth) {
  /* P3/include/myfdtd_func.f90:19-41 */
  double *hx = J->F[HX], *hy = J->F[HY], *hz = J->F[HZ], *dx = J->F[DX], *dy = J->F[DY], *dz = J->F[DZ];
  double Ku = J->g.ku;
  int k0 = J->g.main_lo[2] + 1, k1 = J->g.main_hi[2] + 1;
  (void)nth;
#pragma omp parallel for num_threads(nth) schedule(static) if (nth > 1)
  for (int k = k0; k <= k1; k++)
    for (int j = J->g.main_lo[1] + 1; j <= J->g.main_hi[1] + 1; j++)
      for (int i = J->g.main_lo[0] + 1; i <= J->g.main_hi[0] + 1; i++) {
        int64_t c = IX(J, i, j, k);
        double curlhzy = hz[c] - hz[IX(J, i, j - 1, k)];
        double curlhyz = -hy[c] + hy[IX(J, i, j, k - 1)];
        double curlhxz = hx[c] - hx[IX(J, i, j, k - 1)];
        double curlhzx = -hz[c] + hz[IX(J, i - 1, j, k)];
        double curlhyx = hy[c] - hy[IX(J, i - 1, j, k)];
        double curlhxy = -hx[c] + hx[IX(J, i, j - 1, k)];
        dx[c] = dx[c] + Ku * (curlhzy + curlhyz);
        dy[c] = dy[c] + Ku * (curlhxz + curlhzx);
        dz[c] = dz[c] + Ku * (curlhyx + curlhxy);
      }
}

static void d3_updateH(ora_job *J, int nth) {
  /* P3/include/myfdtd_func.f90:45-64 */
  double *hx = J->F[HX], *hy = J->F[HY], *hz = J->F[HZ], *ex = J->F[EX], *ey = J->F[EY], *ez = J->F[EZ];
  double Ku = J->g.ku;
  int k0 = J->g.main_lo[2] + 1, k1 = J->g.main_hi[2] + 1;
  (void)nth;
#pragma omp parallel for num_threads(nth) schedule(static) if (nth > 1)
  for (int k = k0; k <= k1; k++)
    for (int j = J->g.main_lo[1] + 1; j <= J->g.main_hi[1] + 1; j++)
      for (int i = J->g.main_lo[0] + 1; i <= J->g.main_hi[0] + 1; i++) {
        int64_t c = IX(J, i, j, k);
        double curleyz = ey[IX(J, i, j, k + 1)] - ey[c];
        double curlezy = -ez[IX(J, i, j + 1, k)] + ez[c];
        double curlezx = ez[IX(J, i + 1, j, k)] - ez[c];
        double curlexz = -ex[IX(J, i, j, k + 1)] + ex[c];
        double curlexy = ex[IX(J, i, j + 1, k)] - ex[c];
        double curleyx = -ey[IX(J, i + 1, j, k)] + ey[c];
        hx[c] = hx[c] + Ku * (curleyz + curlezy);
        hy[c] = hy[c] + Ku * (curlezx + curlexz);
        hz[c] = hz[c] + Ku * (curlexy + curleyx);
      }
}

/* reference 3D PML: M3/BERpmly_mod.f90:72-306 */
static void d3_pml_E(ora_job *J) {
  double *ExM = J->F[EX], *EzM = J->F[EZ];
  int nx = J->nx, nz = J->nz;
  for (int s = 0; s < 2; s++) {
    oslab *S = &J->slab[s];
    if (!S->on) continue;
    double **f = S->f;
    int yi = s == 0 ? 1 : S->jb, yf = s == 0 ? S->ja : J->ny;
    for (int k = 1; k <= nz; k++)
      for (int j = yi; j <= yf; j++)
        for (int i = 1; i <= nx; i++) {
          int64_t c = SX(S, i, j, k), cjm = SX(S, i, j - 1, k), ckm = SX(S, i, j, k - 1), cim = SX(S, i - 1, j, k);
          double curlHzy_p = f[S_HZX][c] + f[S_HZY][c];
          double curlHzy_m = -f[S_HZX][cjm] - f[S_HZY][cjm];
          double curlHyz_p = -f[S_HYZ][c] - f[S_HYX][c];
          double curlHyz_m = f[S_HYZ][ckm] + f[S_HYX][ckm];
          double curlHxz_p = f[S_HXY][c] + f[S_HXZ][c];
          double curlHxz_m = -f[S_HXY][ckm] - f[S_HXZ][ckm];
          double curlHzx_p = -f[S_HZX][c] - f[S_HZY][c];
          double curlHzx_m = f[S_HZX][cim] + f[S_HZY][cim];
          double curlHyx_p = f[S_HYZ][c] + f[S_HYX][c];
          double curlHyx_m = -f[S_HYZ][cim] - f[S_HYX][cim];
          double curlHxy_p = -f[S_HXY][c] - f[S_HXZ][c];
          double curlHxy_m = f[S_HXY][cjm] + f[S_HXZ][cjm];
          f[S_EYX][c] = S->f1x[c] * f[S_EYX][c] + S->f2x[c] * (curlHzx_p + curlHzx_m);
          f[S_EZX][c] = S->f1x[c] * f[S_EZX][c] + S->f2x[c] * (curlHyx_p + curlHyx_m);
          f[S_EXY][c] = S->f1y[c] * f[S_EXY][c] + S->f2y[c] * (curlHzy_p + curlHzy_m);
          f[S_EZY][c] = S->f1y[c] * f[S_EZY][c] + S->f2y[c] * (curlHxy_p + curlHxy_m);
          f[S_EXZ][c] = S->f1z[c] * f[S_EXZ][c] + S->f2z[c] * (curlHyz_p + curlHyz_m);
          f[S_EYZ][c] = S->f1z[c] * f[S_EYZ][c] + S->f2z[c] * (curlHxz_p + curlHxz_m);
        }
    /* setboundayEya / setboundayEyb */
    int jc = s == 0 ? S->ja + 1 : S->jb - 1, jw = s == 0 ? S->ja : S->jb;
    for (int k = 1; k <= nz; k++)
      for (int i = 1; i <= nx; i++) {
        f[S_EXY][SX(S, i, jc, k)] = ExM[IX(J, i, jc, k)];
        ExM[IX(J, i, jw, k)] = f[S_EXY][SX(S, i, jw, k)];
        f[S_EZY][SX(S, i, jc, k)] = EzM[IX(J, i, jc, k)];
        EzM[IX(J, i, jw, k)] = f[S_EZY][SX(S, i, jw, k)];
      }
  }
}

static void d3_pml_H(ora_job *J) {
  double *HxM = J->F[HX], *HzM = J->F[HZ];
  int nx = J->nx, nz = J->nz;
  for (int s = 0; s < 2; s++) {
    oslab *S = &J->slab[s];
    if (!S->on) continue;
    double **f = S->f;
    int yi = s == 0 ? 1 : S->jb, yf = s == 0 ? S->ja : J->ny;
    for (int k = 1; k <= nz; k++)
      for (int j = yi; j <= yf; j++)
        for (int i = 1; i <= nx; i++) {
          int64_t c = SX(S, i, j, k), cjp = SX(S, i, j + 1, k), ckp = SX(S, i, j, k + 1), cip = SX(S, i + 1, j, k);
          double curlEzy_p = -f[S_EZX][cjp] - f[S_EZY][cjp];
          double curlEzy_m = f[S_EZX][c] + f[S_EZY][c];
          double curlEyz_p = f[S_EYZ][ckp] + f[S_EYX][ckp];
          double curlEyz_m = -f[S_EYZ][c] - f[S_EYX][c];
          double curlExz_p = -f[S_EXY][ckp] - f[S_EXZ][ckp];
          double curlExz_m = f[S_EXY][c] + f[S_EXZ][c];
          double curlEzx_p = f[S_EZX][cip] + f[S_EZY][cip];
          double curlEzx_m = -f[S_EZX][c] - f[S_EZY][c];
          double curlEyx_p = -f[S_EYZ][cip] - f[S_EYX][cip];
          double curlEyx_m = f[S_EYZ][c] + f[S_EYX][c];
          double curlExy_p = f[S_EXY][cjp] + f[S_EXZ][cjp];
          double curlExy_m = -f[S_EXY][c] - f[S_EXZ][c];
          f[S_HYX][c] = S->g1x[c] * f[S_HYX][c] + S->g2x[c] * (curlEzx_m + curlEzx_p);
          f[S_HZX][c] = S->g1x[c] * f[S_HZX][c] + S->g2x[c] * (curlEyx_m + curlEyx_p);
          f[S_HXY][c] = S->g1y[c] * f[S_HXY][c] + S->g2y[c] * (curlEzy_m + curlEzy_p);
          f[S_HZY][c] = S->g1y[c] * f[S_HZY][c] + S->g2y[c] * (curlExy_m + curlExy_p);
          f[S_HXZ][c] = S->g1z[c] * f[S_HXZ][c] + S->g2z[c] * (curlEyz_m + curlEyz_p);
          f[S_HYZ][c] = S->g1z[c] * f[S_HYZ][c] + S->g2z[c] * (curlExz_m + curlExz_p);
        }
    int jc = s == 0 ? S->ja + 1 : S->jb - 1, jw = s == 0 ? S->ja : S->jb;
    for (int k = 1; k <= nz; k++)
      for (int i = 1; i <= nx; i++) {
        f[S_HXY][SX(S, i, jc, k)] = HxM[IX(J, i, jc, k)];
        HxM[IX(J, i, jw, k)] = f[S_HXY][SX(S, i, jw, k)];
        f[S_HZY][SX(S, i, jc, k)] = HzM[IX(J, i, jc, k)];
        HzM[IX(J, i, jw, k)] = f[S_HZY][SX(S, i, jw, k)];
      }
  }
}

/* ---- 1D: P1 ------------------------------------------------------------------ */
/* 1D PML (M1/BERpmly_ExHz_mod.f90:51-159); slab arrays use f[0]=Ex, f[1]=Hz,
 * indexed by the global 1-based j with the slab's j0 offset. */
static void d1_pml_E(ora_job *J, oslab *sl, double *Ex_) {
  for (int s = 0; s < 2; s++) {
    oslab *S = &sl[s];
    if (!S->on) continue;
    double *Ex = S->f[0], *Hz = S->f[1];
    int yi = s == 0 ? 1 : S->jb, yf = s == 0 ? S->ja : J->ny;
    for (int j = yi; j <= yf; j++) {
      int64_t c = j - S->j0;
      double curlH = Hz[c] - Hz[c - 1];
      Ex[c] = S->f1y[c] * Ex[c] + S->f2y[c] * curlH;
    }
    if (s == 0) { Ex[S->ja + 1 - S->j0] = Ex_[S->ja + 1]; Ex_[S->ja] = Ex[S->ja - S->j0]; }
    else { Ex[S->jb - 1 - S->j0] = Ex_[S->jb - 1]; Ex_[S->jb] = Ex[S->jb - S->j0]; }
  }
}
static void d1_pml_H(ora_job *J, oslab *sl, double *Hz_) {
  for (int s = 0; s < 2; s++) {
    oslab *S = &sl[s];
    if (!S->on) continue;
    double *Ex = S->f[0], *Hz = S->f[1];
    int yi = s == 0 ? 1 : S->jb, yf = s == 0 ? S->ja : J->ny;
    for (int j = yi; j <= yf; j++) {
      int64_t c = j - S->j0;
      double curlE = Ex[c + 1] - Ex[c];
      Hz[c] = S->g1y[c] * Hz[c] + S->g2y[c] * curlE;
    }
    if (s == 0) { Hz[S->ja + 1 - S->j0] = Hz_[S->ja + 1]; Hz_[S->ja] = Hz[S->ja - S->j0]; }
    else { Hz[S->jb - 1 - S->j0] = Hz_[S->jb - 1]; Hz_[S->jb] = Hz[S->jb - S->j0]; }
  }
}

static void d1_step(ora_job *J, int n) {
  /* P1/program.f90:217-291 */
  double *ex = J->F[EX], *hz = J->F[HZ], *dx = J->F[DX];
  double Ku = J->g.ku;
  int j0 = J->g.main_lo[1] + 1, j1 = J->g.main_hi[1] + 1;
  for (int j = j0; j <= j1; j++) {
    dx[j] = dx[j] + Ku * (hz[j] - hz[j - 1]);
    if (J->tfsf) J->exi[j] = J->exi[j] + Ku * (J->hzi[j] - J->hzi[j - 1]);
  }
  apply_sources(J, n, 1);
  apply_sources(J, n, 0);
  if (J->tfsf) {
    d1_pml_E(J, J->islab, J->exi);
    int bd = J->tf.boundary + 1;
    dx[bd] = dx[bd] - Ku * J->hzi[bd - 1];
  }
  materials_update_E(J, n);
  d1_pml_E(J, J->slab, ex);
  for (int j = j0; j <= j1; j++) {
    hz[j] = hz[j] + Ku * (ex[j + 1] - ex[j]);
    if (J->tfsf) J->hzi[j] = J->hzi[j] + Ku * (J->exi[j + 1] - J->exi[j]);
  }
  if (J->tfsf) d1_pml_H(J, J->islab, J->hzi);
  d1_pml_H(J, J->slab, hz);
  if (J->tfsf) {
    int bd = J->tf.boundary + 1;
    hz[bd - 1] = hz[bd - 1] - Ku * J->exi[bd];
  }
}

/* ---- sampling: probes and DFT (P2/program.f90:373-433, P3/program.f90:441-540) */
static double *comp_ptr(ora_job *J, int comp) {
  if (comp <= FDTD_HZ) return J->F[comp];
  if (comp == FDTD_EX_INC) return J->exi;
  if (comp == FDTD_HZ_INC) return J->hzi;
  return NULL;
}

static void sample(ora_job *J, int n, int nth) {
  double t = (double)(n - 1) * J->g.dt;
  double dt = J->g.dt;
  (void)nth;
  for (int q = 0; q < J->nprobe; q++) {
    oprobe *P = &J->probe[q];
    if (n < P->d.n_first || n > P->d.n_last) continue;
    if (P->count + 1 > P->cap) {
      P->cap = P->cap ? 2 * P->cap : 1024;
      P->buf = (double *)realloc(P->buf, sizeof(double) * (size_t)P->cap * P->ncomp);
    }
    int64_t c = cell_ix(J, P->d.cell[0], P->d.cell[1], P->d.cell[2]);
    for (int u = 0; u < P->ncomp; u++) P->buf[(size_t)P->count * P->ncomp + u] = comp_ptr(J, P->comps[u])[c];
    P->count++;
  }
  for (int q = 0; q < J->nmon; q++) {
    omon *M = &J->mon[q];
    if (n < M->d.n_first || n > M->d.n_last) continue;
    const int *lo = M->d.lo, *hi = M->d.hi;
    int wx = hi[0] - lo[0] + 1, wy = hi[1] - lo[1] + 1;
    if (M->d.reduce == FDTD_MONITOR_MEAN) {
      /* the DFT of the box mean of each component (the plane-averaged
         transmitted field of a laterally uniform problem) */
      const int64_t cnt = (int64_t)wx * wy * (hi[2] - lo[2] + 1);
      for (int u = 0; u < M->ncomp; u++) {
        const double *F = comp_ptr(J, M->comps[u]);
        double sum = 0.0;
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) sum += F[cell_ix(J, i, j, k)];
        const double f = sum / (double)cnt;
        for (int m = 0; m < M->nfreq; m++) {
          const double cs = cos(M->omega[m] * t), sn = sin(M->omega[m] * t);
          double *re = M->re + (size_t)u * M->nfreq + m, *im = M->im + (size_t)u * M->nfreq + m;
          *re = *re + cs * f * dt;
          *im = *im + sn * f * dt;
        }
      }
      continue;
    }
#pragma omp parallel for num_threads(nth) schedule(static) if (nth > 1)
    for (int m = 0; m < M->nfreq; m++) {
      /* dcos(arg(m)*t) is the same for every cell of the plane */
      double cs = cos(M->omega[m] * t), sn = sin(M->omega[m] * t);
      for (int u = 0; u < M->ncomp; u++) {
        double *F = comp_ptr(J, M->comps[u]);
        double *re = M->re + ((size_t)u * M->nfreq + m) * M->ncell;
        double *im = M->im + ((size_t)u * M->nfreq + m) * M->ncell;
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) {
              int64_t p = (int64_t)(i - lo[0]) + (int64_t)wx * ((j - lo[1]) + (int64_t)wy * (k - lo[2]));
              double f = F[cell_ix(J, i, j, k)];
              re[p] = re[p] + cs * f * dt;
              im[p] = im[p] + sn * f * dt;
            }
      }
    }
  }
}

/* ---- the loop body --------------------------------------------------------------- */
int ora_step(ora_job *J, int n_first, int n_steps, int nth) {
  if (!J->committed) FAIL("commit first");
  J->nth = nth > 1 ? nth : 1;
  int L = J->g.layout;
  for (int n = n_first; n < n_first + n_steps; n++) {
    if (L == FDTD_LAYOUT_1D) {
      d1_step(J, n);
    } else if (L == FDTD_LAYOUT_2D_TE) {
      te2d_updateD(J);
      apply_sources(J, n, 0);
      if (J->tfbox) { tfbox_line_E(J, n); tfbox_faces_D(J); }
      materials_update_E(J, n);
      if (J->pml_mode == FDTD_PML_REFERENCE) te2d_pml_E(J);
      if (J->pml_mode == FDTD_PML_SPLIT) split_E(J);
      /* interchange_E: Ey x-wrap (Ex y-exchange is the identity) */
      if (J->g.periodic[0]) wrap_x_both(J, J->F[EY], 1);
      if (J->g.periodic[1]) wrap_y_both(J, J->F[EX]);
      te2d_updateH(J);
      if (J->pml_mode == FDTD_PML_REFERENCE) te2d_pml_H(J);
      if (J->pml_mode == FDTD_PML_SPLIT) split_H(J);
      if (J->tfbox) { tfbox_line_H(J); tfbox_faces_H(J); }
      /* interchange_H: Hz x-wrap */
      if (J->g.periodic[0]) wrap_x_both(J, J->F[HZ], 1);
      if (J->g.periodic[1]) wrap_y_both(J, J->F[HZ]);
    } else if (L == FDTD_LAYOUT_2D_TM) {
      tm2d_updateD(J);
      apply_sources(J, n, 0);
      if (J->tfbox) { tfbox_line_E(J, n); tfbox_faces_D(J); }
      materials_update_E(J, n);
      if (J->pml_mode == FDTD_PML_SPLIT) split_E(J);
      if (J->g.periodic[0]) wrap_x_high(J, J->F[EZ]);
      if (J->g.periodic[1]) wrap_y_both(J, J->F[EZ]);
      tm2d_updateH(J);
      if (J->pml_mode == FDTD_PML_SPLIT) split_H(J);
      if (J->tfbox) { tfbox_line_H(J); tfbox_faces_H(J); }
      if (J->g.periodic[0]) wrap_x_low(J, J->F[HY]);
      if (J->g.periodic[1]) wrap_y_low(J, J->F[HX]);
    } else {
      d3_updateD(J, nth);
      apply_sources(J, n, 0);
      if (J->tfbox) { tfbox_line_E(J, n); tfbox_faces_D(J); }
      materials_update_E(J, n);
      if (J->pml_mode == FDTD_PML_REFERENCE) d3_pml_E(J);
      if (J->pml_mode == FDTD_PML_SPLIT) split_E(J);
      /* interchange_E (P3/include/mympi_func.f90:241-518) */
      if (J->g.periodic[0]) { wrap_x_both(J, J->F[EY], J->pz); wrap_x_both(J, J->F[EZ], J->pz); }
      if (J->g.periodic[1]) { wrap_y_both(J, J->F[EX]); wrap_y_both(J, J->F[EZ]); }
      if (J->g.periodic[2]) { wrap_z_both(J, J->F[EX]); wrap_z_both(J, J->F[EY]); }
      d3_updateH(J, nth);
      if (J->pml_mode == FDTD_PML_REFERENCE) d3_pml_H(J);
      if (J->pml_mode == FDTD_PML_SPLIT) split_H(J);
      if (J->tfbox) { tfbox_line_H(J); tfbox_faces_H(J); }
      /* interchange_H (P3/include/mympi_func.f90:522-690) */
      if (J->g.periodic[0]) { wrap_x_low(J, J->F[HY]); wrap_x_low(J, J->F[HZ]); }
      if (J->g.periodic[1]) { wrap_y_low(J, J->F[HX]); wrap_y_low(J, J->F[HZ]); }
      if (J->g.periodic[2]) { wrap_z_low(J, J->F[HX]); wrap_z_low(J, J->F[HY]); }
    }
    sample(J, n, nth);
    J->last_n = n;
  }
  return 0;
}

/* ---- access ------------------------------------------------------------------ */
static int field_index(ora_job *J, int comp) {
  if (comp < 0 || comp > FDTD_HZ_INC) return -1;
  return comp;
}

int ora_get_field(ora_job *J, int comp, double *host) {
  if (field_index(J, comp) < 0) FAIL("bad component");
  if (J->tfbox && comp >= FDTD_E_INC) {  /* the box's incident line: ny values */
    memcpy(host, comp == FDTD_E_INC ? J->le : J->lh, sizeof(double) * (size_t)J->ny);
    return 0;
  }
  double *F = comp_ptr(J, comp);
  if (!F) FAIL("component not present");
  int64_t q = 0;
  for (int k = 0; k < J->nz; k++)
    for (int j = 0; j < J->ny; j++)
      for (int i = 0; i < J->nx; i++) host[q++] = F[cell_ix(J, i, j, k)];
  return 0;
}

int ora_set_field(ora_job *J, int comp, const double *host) {
  if (field_index(J, comp) < 0) FAIL("bad component");
  double *F = comp_ptr(J, comp);
  if (!F) FAIL("component not present");
  int64_t q = 0;
  for (int k = 0; k < J->nz; k++)
    for (int j = 0; j < J->ny; j++)
      for (int i = 0; i < J->nx; i++) F[cell_ix(J, i, j, k)] = host[q++];
  return 0;
}

int ora_monitor_size(ora_job *J, int id, int *ncomp, int *nfreq, int *ncell) {
  if (id < 0 || id >= J->nmon) FAIL("bad monitor id");
  *ncomp = J->mon[id].ncomp; *nfreq = J->mon[id].nfreq; *ncell = (int)J->mon[id].ncell;
  return 0;
}

int ora_get_monitor(ora_job *J, int id, double *re, double *im) {
  if (id < 0 || id >= J->nmon) FAIL("bad monitor id");
  omon *M = &J->mon[id];
  size_t n = (size_t)M->ncomp * M->nfreq * M->ncell;
  memcpy(re, M->re, n * sizeof(double));
  memcpy(im, M->im, n * sizeof(double));
  return 0;
}

int ora_get_probe(ora_job *J, int id, double *host, int *count) {
  if (id < 0 || id >= J->nprobe) FAIL("bad probe id");
  oprobe *P = &J->probe[id];
  if (host) memcpy(host, P->buf, sizeof(double) * (size_t)P->count * P->ncomp);
  *count = P->count;
  return 0;
}
