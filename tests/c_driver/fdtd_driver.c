/* A C user of the engine: builds a 2D TMz job through the C ABI alone
 * (dielectric background, a gold cylinder, split-field PML, a soft line
 * source, a line DFT monitor and a point probe), steps it and prints what it
 * read back, so that a test can compare it with the same job built through
 * the Python binding.
 *
 *   fdtd_driver <precision 1|2> <steps>
 *
 * Output: "ENODEV" when there is no usable device, else one line of
 * "key value" pairs (%.17g). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "fdtd_gb300.h"

#define CHECK(call)                                               \
  do {                                                            \
    int rc_ = (call);                                             \
    if (rc_ != FDTD_OK) {                                         \
      char msg[512];                                              \
      fdtd_last_error(msg, sizeof msg);                           \
      fprintf(stderr, "%s: %d %s\n", #call, rc_, msg);            \
      return 1;                                                   \
    }                                                             \
  } while (0)

int main(int argc, char **argv) {
  const int prec = argc > 1 ? atoi(argv[1]) : FDTD_F64;
  const int steps = argc > 2 ? atoi(argv[2]) : 300;
  const int n = 96, npml = 10;
  const double pi = 4.0 * atan(1.0), ep0 = 8.85418781762039e-12, mu0 = pi * 4e-7;
  const double c0 = 1.0 / sqrt(ep0 * mu0), ds = 1e-9, ku = 0.5, dt = ku * ds / c0;

  fdtd_grid_desc g = {FDTD_LAYOUT_2D_TM, prec, {n, n, 1}, {0, 0, 0}, {0, 0, 0}, {n - 1, n - 1, 0}, ku, dt, ds};
  fdtd_job *job = NULL;
  int rc = fdtd_create(&g, &job);
  if (rc == FDTD_ENODEV) {
    printf("ENODEV\n");
    return 0;
  }
  CHECK(rc);
  int32_t id;
  fdtd_region all = {FDTD_REGION_BOX, {0, 0, 0}, {n - 1, n - 1, 0}, 0, NULL, NULL};
  CHECK(fdtd_add_dielectric(job, &all, 1.0, &id));
  const double cyl[4] = {48.0, 52.0, 0.0, 8.0};
  fdtd_region rod = {FDTD_REGION_SPHERES, {0, 0, 0}, {0, 0, 0}, 1, cyl, NULL};
  const fdtd_drude2cp gold = {1.1431, 1.3202e16, 1.0805e14, {0.26698, 3.0834}, {-1.2371, -1.0968},
                              {3.8711e15, 4.1684e15}, {4.4642e14, 2.4555e15}};
  CHECK(fdtd_add_gold(job, &rod, &gold, &id));
  /* graded profile: sigma_max = (m + 1) c0 ln(1/R0) / (2 npml ds) with m = 3, R0 = e^-16 */
  fdtd_pml_desc pml = {FDTD_PML_SPLIT, {{npml, npml}, {npml, npml}, {0, 0}}, 1.0, 1.0,
                       4.0 * c0 * 16.0 / (2.0 * npml * ds), 3.0};
  CHECK(fdtd_add_pml(job, &pml));
  const double f0 = c0 / 600e-9, st = 1.0 / f0;
  fdtd_source_desc src = {FDTD_EZ, {npml, 20, 0}, {n - 1 - npml, 20, 0}, 1.0, 4.0 * st, st, 2.0 * pi * f0};
  CHECK(fdtd_add_source(job, &src, &id));
  double omega[8];
  for (int m = 0; m < 8; ++m) omega[m] = 2.0 * pi * c0 / (400e-9 + 50e-9 * m);
  fdtd_monitor_desc mon = {{npml, 70, 0}, {n - 1 - npml, 70, 0}, 1 << FDTD_EZ, 1, 1 << 30, 8, omega,
                           FDTD_MONITOR_CELLS};
  int32_t mid;
  CHECK(fdtd_add_monitor(job, &mon, &mid));
  fdtd_probe_desc pr = {{48, 70, 0}, 1 << FDTD_EZ, 1, 1 << 30};
  int32_t pid;
  CHECK(fdtd_add_probe(job, &pr, &pid));
  CHECK(fdtd_commit(job));
  CHECK(fdtd_step(job, 1, steps));

  double *ez = malloc(sizeof(double) * n * n);
  CHECK(fdtd_get_field(job, FDTD_EZ, ez));
  double ez2 = 0.0;
  for (int c = 0; c < n * n; ++c) ez2 += ez[c] * ez[c];
  const int ncell = n - 2 * npml;
  double *re = malloc(sizeof(double) * 8 * ncell), *im = malloc(sizeof(double) * 8 * ncell);
  CHECK(fdtd_get_monitor(job, mid, re, im));
  double sre = 0.0, sim = 0.0;
  for (int q = 0; q < 8 * ncell; ++q) {
    sre += re[q];
    sim += im[q];
  }
  int32_t cnt = 0;
  CHECK(fdtd_get_probe(job, pid, NULL, &cnt));
  double *pv = malloc(sizeof(double) * (cnt > 0 ? cnt : 1));
  CHECK(fdtd_get_probe(job, pid, pv, &cnt));
  printf("ez2 %.17g re %.17g im %.17g probe_count %d probe_last %.17g\n", ez2, sre, sim, cnt, pv[cnt - 1]);
  free(ez);
  free(re);
  free(im);
  free(pv);
  CHECK(fdtd_destroy(job));
  return 0;
}
