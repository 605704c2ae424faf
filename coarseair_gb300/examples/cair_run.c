/*
 * cair_run: a C caller of the trajectory library through include/cair_gpu.h only -- the shape of the
 * driver a C or Fortran host (RunTrajectories.F90:277) puts around Integrator%Integrate.
 *
 *   cair_run <N3_UMN.dat> <levels.txt> <out_dir> <ntraj per level> <ttra [K]> <seed>
 *
 * N3_UMN.dat: the 276 N3 UMN coefficients, one per line ('#' comments).
 * levels.txt: one level per line: vqn jqn eint egam rmin rmax vmin vmax tau ri ro.
 * Runs N2 + N (masses 14.0067 amu, b = 7 sqrt(U) bohr, Dinit 15 bohr, rmax 16 bohr) for every level as
 * one work item with stream seed + 2 k, writes out_dir/trajectories.out and _HNotCons.out, and prints
 * one summary line.  Exit status 0 on success; library errors are printed with cair_last_error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cair_gpu.h"

#define AMU_TO_AU 1822.888486209

static int fail(cair_handle* h, int rc, const char* what) {
  fprintf(stderr, "cair_run: %s failed (%d): %s\n", what, rc, h ? cair_last_error(h) : "");
  return 1;
}

int main(int argc, char** argv) {
  if (argc != 7) {
    fprintf(stderr, "usage: cair_run <N3_UMN.dat> <levels.txt> <out_dir> <ntraj> <ttra> <seed>\n");
    return 2;
  }
  const int64_t ntraj = atoll(argv[4]);
  const double ttra = atof(argv[5]);
  const int64_t seed = atoll(argv[6]);
  /* surface coefficients */
  double coef[276];
  int nc = 0;
  char line[512];
  FILE* f = fopen(argv[1], "r");
  if (!f) return fprintf(stderr, "cair_run: cannot open %s\n", argv[1]), 1;
  while (nc < 276 && fgets(line, sizeof line, f))
    if (line[0] != '#' && sscanf(line, "%lf", &coef[nc]) == 1) ++nc;
  fclose(f);
  if (nc != 276) return fprintf(stderr, "cair_run: %s holds %d coefficients, not 276\n", argv[1], nc), 1;
  /* levels */
  cair_level lv[1024];
  int nl = 0;
  f = fopen(argv[2], "r");
  if (!f) return fprintf(stderr, "cair_run: cannot open %s\n", argv[2]), 1;
  while (nl < 1024 && fgets(line, sizeof line, f)) {
    cair_level L;
    if (sscanf(line, "%d %d %lf %lf %lf %lf %lf %lf %lf %lf %lf", &L.vqn, &L.jqn, &L.eint, &L.egam, &L.rmin, &L.rmax,
               &L.vmin, &L.vmax, &L.tau, &L.ri, &L.ro) == 11)
      lv[nl++] = L;
  }
  fclose(f);
  if (nl == 0) return fprintf(stderr, "cair_run: no levels in %s\n", argv[2]), 1;
  /* system: N2 + N on the N3 UMN surface with the reference's integrator settings */
  cair_system_desc sys;
  memset(&sys, 0, sizeof sys);
  sys.abi_version = CAIR_ABI_VERSION;
  sys.natoms = 3;
  sys.npes = 1;
  sys.diat_model = CAIR_DIAT_N2_UMN_FORN4;
  for (int i = 0; i < 3; ++i) sys.mass[i] = 14.0067 * AMU_TO_AU;
  sys.pes[0].model = CAIR_PES_N3_UMN;
  sys.pes[0].ncoef = 276;
  sys.pes[0].coef = coef;
  sys.pes[0].a = 1.0; sys.pes[0].ab = 1.5; sys.pes[0].ra = 1.098; sys.pes[0].rb = 1.098;
  sys.pes[0].totdiss = 457.4;
  sys.dt0 = 5.0; sys.eps = 1.0e-8; sys.relax = 0.5; sys.rmax = 16.0; sys.tmax = 4.0e5; sys.ham_abs_tol = 1.0e-5;
  sys.nsteps = 3; sys.inc_step = 1; sys.ncall = 10; sys.nquad = 50;
  sys.rsmal = 1.0; sys.rcent = 30.0; sys.rfact = 0.0; sys.tthresau = 1.0e-100;
  cair_handle* h = NULL;
  int rc = cair_create(&h, &sys);
  if (rc) return fail(h, rc, "cair_create");
  /* one state-specific run per level */
  cair_work_item* items = calloc((size_t)nl, sizeof *items);
  for (int k = 0; k < nl; ++k) {
    items[k].ilevel = k;
    items[k].ipes = 0;
    items[k].first = (int64_t)k * ntraj;
    items[k].ntraj = ntraj;
    items[k].seed = seed + 2 * k;
    items[k].ttra = ttra;
    items[k].bmax = 7.0;
    items[k].dinit = 15.0;
  }
  const int64_t ntot = ntraj * nl;
  cair_traj_result* rows = calloc((size_t)ntot, sizeof *rows);
  rc = cair_run_queue(h, nl, lv, nl, items, ntot, 1000000, rows);
  if (rc) return fail(h, rc, "cair_run_queue");
  int64_t counts[2] = {0, 0};
  rc = cair_write_trajectories(argv[3], rows, ntot, 0, 1, sys.ham_abs_tol, counts);
  if (rc) return fail(h, rc, "cair_write_trajectories");
  int64_t att[5];
  cair_last_counters(h, att);
  printf("cair_run: %lld trajectories, %lld in trajectories.out, %lld in trajectories_HNotCons.out, %lld attempts\n",
         (long long)ntot, (long long)counts[0], (long long)counts[1], (long long)att[0]);
  free(rows);
  free(items);
  cair_destroy(h);
  return 0;
}
