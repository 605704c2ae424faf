/*
 * CPU oracle -- TEST INFRASTRUCTURE ONLY: final-state statistics, cross sections and rate
 * coefficients of one state-specific run, restated from app/TrajectoriesStats/Statistics_Class.F90
 * (Histogram assignment, NCond conditions, no identical diatoms) and the Boltzmann mean velocity of
 * src/Collision/Collision_Class.F90:576-595.
 *
 * Input rows are the trajectories.csv columns: bMax, bSampled, Qini(NCond), Qfin(NCond).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* IdentifyInitialStates (Statistics_Class.F90:591-680) for one row: transforms qini/qfin in place
 * and returns the initial-state code. */
static long long identify(int ncond, const int* iskip, const int* pres, long long qnmax, double* qini, double* qfin,
                          int* err) {
  long long ifact = 1, isum = 0;
  int ipair_ini = (int)((qini[ncond - 1] - 0.49) / 16);
  int ipair_fin = (int)((qfin[ncond - 1] - 0.49) / 16);
  for (int c = 0; c < ncond; ++c) {
    qini[c] = qini[c] - 0.5;
    long long ini = (long long)lround(qini[c]);
    if (ini >= qnmax) *err = 1;
    double fin_raw = qfin[c];
    qfin[c] = qfin[c] - 0.5;
    if (pres[c] && ipair_ini == ipair_fin) {
      if (ini % 2 == 1) {   /* Fortran mod: sign of the dividend */
        qfin[c] = qfin[c] - 1.0;
        if (lround(qfin[c] * 0.5) < 0 && fin_raw > 0.0) qfin[c] = qfin[c] + 2.0;
      }
      qfin[c] = qfin[c] * 0.5;
    }
    ini = ini + 2;
    if (iskip[c] != 0) isum = isum + ini * ifact;
    else isum = isum + 2 * ifact;
    ifact = ifact * qnmax;
  }
  return isum;
}

/* Final-state code of one row (AddFinState, Statistics_Class.F90:935-1282, Histogram branch:
 * every weight is one and the Main_Loop makes a single pass). */
static long long fin_code(int ncond, const int* iskip, long long qnmax, const double* qfin) {
  long long isum = 0, ifact = 1;
  for (int c = 0; c < ncond; ++c) {
    long long iquse = (long long)lround(qfin[c]);
    iquse = iquse * iskip[c];
    if (iquse + 2 > qnmax) iquse = 0;
    if (iskip[c] != 0 || c == ncond - 1) isum = isum + (iquse + 2) * ifact;
    ifact = ifact * qnmax;
  }
  return isum;
}

/* One run (all rows share the initial state, as in a state-specific run).  Writes up to `cap`
 * final states: code, decoded FinCondVec (ncond ints each), count, Cross, CrossSD [bohr^2].
 * Returns the number of final states, or -1 on an out-of-range quantum number. */
int orc_statistics(int nrows, int ncond, const int* iskip, const int* pres, int qnmax_, const double* bmax,
                   const double* bsamp, const double* qini_in, const double* qfin_in, int cap, long long* codes,
                   int* fincond, int* inistate, long long* counts, double* cross, double* cross_sd) {
  const long long qnmax = qnmax_;
  double* qi = (double*)malloc(sizeof(double) * (size_t)nrows * ncond);
  double* qf = (double*)malloc(sizeof(double) * (size_t)nrows * ncond);
  memcpy(qi, qini_in, sizeof(double) * (size_t)nrows * ncond);
  memcpy(qf, qfin_in, sizeof(double) * (size_t)nrows * ncond);
  int err = 0;
  long long code0 = 0;
  for (int k = 0; k < nrows; ++k) {
    long long c = identify(ncond, iskip, pres, qnmax, qi + (size_t)k * ncond, qf + (size_t)k * ncond, &err);
    if (k == 0) code0 = c;
  }
  if (err) { free(qi); free(qf); return -1; }
  /* SetRings (511-586): distinct bMax within 1e-3, sorted, ring areas */
  double rb[64];
  int nr = 0;
  for (int k = 0; k < nrows; ++k) {
    int dup = 0;
    for (int r = 0; r < nr; ++r)
      if (fabs(bmax[k] - rb[r]) < 1.0e-3) dup = 1;
    if (!dup && nr < 64) rb[nr++] = bmax[k];
  }
  for (int i = 1; i < nr; ++i)
    for (int j = i; j > 0 && rb[j - 1] > rb[j]; --j) { double t = rb[j]; rb[j] = rb[j - 1]; rb[j - 1] = t; }
  double area[64], prev = 0.0;
  for (int r = 0; r < nr; ++r) {
    double t = M_PI * rb[r] * rb[r];
    area[r] = t - prev;
    prev = t;
  }
  if (nr == 1 && area[0] == 0.0) area[0] = 1.0;
  /* IniState from the first code (ProcessStatistics, 782-929) */
  long long ifacts = 1;
  for (int c = 0; c < ncond; ++c) ifacts *= qnmax;
  {
    long long isum = code0, ifact = ifacts;
    for (int c = ncond - 1; c >= 0; --c) {
      ifact /= qnmax;
      long long t = isum / ifact;
      inistate[c] = (int)(t - 2);
      isum -= t * ifact;
    }
  }
  /* AddFinState over every row */
  long long perb[64] = {0};
  int nfs = 0;
  double* w = (double*)calloc((size_t)cap * 64, sizeof(double));
  for (int k = 0; k < nrows; ++k) {
    int ring = 0;
    if (nr > 1)
      for (int r = 0; r < nr - 1; ++r)
        if (!(bsamp[k] > rb[r + 1] || bsamp[k] <= rb[r])) { ring = r + 1; break; }
    perb[ring] += 1;
    long long code = fin_code(ncond, iskip, qnmax, qf + (size_t)k * ncond);
    int s;
    for (s = 0; s < nfs; ++s)
      if (codes[s] == code) break;
    if (s == nfs) {
      if (nfs == cap) { free(qi); free(qf); free(w); return -2; }
      codes[nfs] = code;
      counts[nfs] = 0;
      ++nfs;
    }
    counts[s] += 1;
    w[(size_t)s * 64 + ring] += 1.0;
  }
  /* WriteFinStateProbabilities (1288-1440) */
  int ini_arr = inistate[ncond - 1] / 16;
  for (int s = 0; s < nfs; ++s) {
    double cr = 0.0, sd = 0.0;
    for (int r = 0; r < nr; ++r) {
      double fw = w[(size_t)s * 64 + r] / (double)(perb[r] > 1 ? perb[r] : 1);
      cr = cr + area[r] * fw;
      sd = sd + fw * (1.0 - fw) * area[r] * area[r] / (double)(perb[r] > 1 ? perb[r] : 1);
    }
    cross[s] = cr;
    cross_sd[s] = sqrt(sd);
    long long isum = codes[s], ifact = ifacts;
    int fin_arr = 0;
    for (int c = ncond - 1; c >= 0; --c) {
      ifact /= qnmax;
      long long fc = isum / ifact;
      if (c == ncond - 1) fin_arr = (int)((fc - 2) / 16);
      isum -= fc * ifact;
      fc -= 2;
      if (pres[c] && ini_arr == fin_arr) {
        fc = fc * 2;
        if (inistate[c] % 2 != 0) fc = fc + 1;
      }
      fincond[s * ncond + c] = (int)fc;
    }
  }
  free(qi);
  free(qf);
  free(w);
  return nfs;
}

/* Boltzmann mean relative speed in cm^3/s per bohr^2 (Collision_Class.F90:576-595):
 * Va = 2/sqrt(pi) sqrt(2 T k/mu), times the atomic unit of time^-1 and bohr^3 in cm^3. */
double orc_mean_velocity(double ttra, double xmu) {
  const double kelvin_to_hartree = 1.0 / 3.1577513e5;   /* One / Hartree_To_Kelvin (Parameters_Module.F90:64-65) */
  double vp = sqrt(2.0 * ttra * kelvin_to_hartree / xmu);
  double va = 2.0 / sqrt(M_PI) * vp;
  return va * 4.134137e16 * (0.5291771e-8 * 0.5291771e-8 * 0.5291771e-8);
}
