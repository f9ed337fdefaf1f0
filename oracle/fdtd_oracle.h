/*
 * fdtd_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 CPU restatement of the reference's FDTD time-loop body, used by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as
 * the checker.  The product (the CUDA library) never links or calls it.
 *
 * It follows the reference line by line on one domain (the MPI ranks'
 * slabs stitched into one array with explicit one-cell halos), with the
 * descriptor structs of include/fdtd_gb300.h as input so that the same job
 * description drives the oracle and the library.
 *
 * Parity pin: the 2D path reproduces the reference's shipped 2D outputs
 * (FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate/{transforms,
 * timesLiney,timesGnuplotmap}); see tests/test_oracle_golden.py.
 */
#ifndef FDTD_ORACLE_H
#define FDTD_ORACLE_H
#include "fdtd_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_job ora_job;

ora_job *ora_create(const fdtd_grid_desc *grid);
void ora_destroy(ora_job *job);
const char *ora_error(void);
int ora_add_dielectric(ora_job *job, const fdtd_region *region, double eps_r);
int ora_add_gold(ora_job *job, const fdtd_region *region, const fdtd_drude2cp *p);
int ora_add_graphene(ora_job *job, const fdtd_region *region, const fdtd_graphene_desc *p);
int ora_add_lorentz(ora_job *job, const fdtd_region *region, const fdtd_lorentz_desc *p);
int ora_add_graphene_cp(ora_job *job, const fdtd_region *region, const fdtd_graphene_cp_desc *p);
int ora_add_conductive(ora_job *job, const fdtd_region *region, double eps_inf, double sigma);
int ora_add_graphene_nk(ora_job *job, const fdtd_region *region, const fdtd_graphene_nk_desc *p);
int ora_add_pml(ora_job *job, const fdtd_pml_desc *pml);
int ora_add_tfsf_1d(ora_job *job, const fdtd_tfsf1d_desc *tfsf);
int ora_add_tfsf(ora_job *job, const fdtd_tfsf_desc *tfsf);
int ora_add_source(ora_job *job, const fdtd_source_desc *src);
int ora_add_monitor(ora_job *job, const fdtd_monitor_desc *mon);
int ora_add_probe(ora_job *job, const fdtd_probe_desc *probe);
int ora_commit(ora_job *job);
/* steps n_first .. n_first+n_steps-1; nthreads <= 1 runs serially */
int ora_step(ora_job *job, int n_first, int n_steps, int nthreads);
int ora_get_field(ora_job *job, int comp, double *host);
int ora_set_field(ora_job *job, int comp, const double *host);
int ora_get_monitor(ora_job *job, int id, double *re, double *im);
int ora_monitor_size(ora_job *job, int id, int *ncomp, int *nfreq, int *ncell);
int ora_get_probe(ora_job *job, int id, double *host, int *count);

#ifdef __cplusplus
}
#endif
#endif
