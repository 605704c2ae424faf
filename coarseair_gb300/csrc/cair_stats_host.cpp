// Host half of the final-state statistics (app/TrajectoriesStats/Statistics_Class.F90): SetRings
// (511-586) per run before the device counting pass, ProcessStatistics' IniState (782-929) and
// WriteFinStateProbabilities (1288-1440) after it, and the rate of Process_Class.F90:122-209 with
// the Boltzmann mean velocity of Collision_Class.F90:576-595.  No CUDA.
#include "cair_stats_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace cair {

std::string stats_runs(int32_t nitems, const cair_work_item* items, const int32_t* item_run, StatsRuns& out) {
  out = StatsRuns{};
  out.run_of.resize(nitems);
  for (int i = 0; i < nitems; ++i) {
    out.run_of[i] = item_run ? item_run[i] : i;
    if (out.run_of[i] < 0 || out.run_of[i] >= nitems) return "cair_statistics: run out of range";
    out.nruns = std::max(out.nruns, out.run_of[i] + 1);
  }
  out.ttra.assign(out.nruns, -1.0);
  for (int i = 0; i < nitems; ++i) {
    double& t = out.ttra[out.run_of[i]];
    if (t < 0.0) t = items[i].ttra;
    else if (std::fabs(t - items[i].ttra) > 1e-12 * t) return "cair_statistics: items of one run differ in temperature";
  }
  return "";
}

std::string stats_rings(const cair_stats_params& P, int32_t nitems, const cair_work_item* items,
                        const unsigned long long* item_rows, const long long* item_ini, StatsRuns& runs) {
  const int32_t nruns = runs.nruns;
  runs.ring_b.assign((size_t)nruns * kStatsMaxRings, 0.0);
  runs.nring.assign(nruns, 0);
  runs.ini.assign(nruns, std::numeric_limits<long long>::max());
  for (int i = 0; i < nitems; ++i) {
    if (item_rows[i] == 0) continue;
    const int r = runs.run_of[i];
    runs.ini[r] = std::min(runs.ini[r], item_ini[i]);
    double* e = runs.ring_b.data() + (size_t)r * kStatsMaxRings;
    const double b = std::fabs(items[i].bmax);
    bool dup = false;
    for (int q = 0; q < runs.nring[r]; ++q) dup = dup || std::fabs(b - e[q]) < 1.0e-3;
    if (dup) continue;
    if (runs.nring[r] == kStatsMaxRings) return "cair_statistics: more than 64 rings in a run";
    e[runs.nring[r]++] = b;
  }
  runs.R = 1;
  for (int r = 0; r < nruns; ++r) {
    std::sort(runs.ring_b.begin() + (size_t)r * kStatsMaxRings,
              runs.ring_b.begin() + (size_t)r * kStatsMaxRings + runs.nring[r]);
    runs.R = std::max(runs.R, runs.nring[r]);
  }
  // codes lie within +-70 qn_max^ncond; with the run and ring folded in they must fit a signed 64-bit key
  double span = 70.0 * (double)nruns * (double)runs.R;
  for (int q = 0; q < P.ncond; ++q) span *= (double)P.qn_max;
  if (span >= 4.6e18) return "cair_statistics: qn_max^ncond x runs x rings too large";
  return "";
}

std::vector<StatsEntry> stats_decode(const StatsRuns& runs, int64_t n, const unsigned long long* keys,
                                     const unsigned long long* counts) {
  const long long R = runs.R, nruns = runs.nruns;
  // a possibly negative code: decode with floor division
  auto floordiv = [](long long a, long long b) { return a / b - ((a % b != 0) && ((a < 0) != (b < 0))); };
  std::vector<StatsEntry> ent((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    const long long ks = (long long)keys[i];
    const long long rest = floordiv(ks, R);
    ent[i].ring = (int)(ks - rest * R);
    ent[i].code = floordiv(rest, nruns);
    ent[i].run = (int)(rest - ent[i].code * nruns);
    ent[i].count = counts[i];
  }
  return ent;
}

std::string stats_finish(const cair_stats_params& P, const StatsRuns& runs, int64_t n, const unsigned long long* keys,
                         const unsigned long long* counts, const unsigned long long* ring_rows, cair_final_state* out,
                         int64_t cap, int64_t* nout) {
  return stats_finish_entries(P, runs, stats_decode(runs, n, keys, counts), ring_rows, out, cap, nout);
}

std::string stats_finish_entries(const cair_stats_params& P, const StatsRuns& runs, std::vector<StatsEntry> ent,
                                 const unsigned long long* ring_rows, cair_final_state* out, int64_t cap,
                                 int64_t* nout) {
  const int nc = P.ncond;
  std::sort(ent.begin(), ent.end(), [](const StatsEntry& a, const StatsEntry& b) {
    return a.run != b.run ? a.run < b.run : (a.code != b.code ? a.code < b.code : a.ring < b.ring);
  });
  const long long qn = P.qn_max;
  long long ifacts = 1;
  for (int q = 0; q < nc; ++q) ifacts *= qn;
  const double pi = std::acos(-1.0), k_to_h = 1.0 / 3.1577513e5, bohr_cm = 0.5291771e-8;
  int64_t lines = 0;
  for (size_t i = 0; i < ent.size();) {
    size_t j = i;
    while (j < ent.size() && ent[j].run == ent[i].run && ent[j].code == ent[i].code) ++j;
    ++lines;
    i = j;
  }
  if (lines > cap) return "cair_statistics: cap too small, " + std::to_string(lines) + " final states";
  int64_t o = 0;
  for (size_t i = 0; i < ent.size();) {
    size_t j = i;
    while (j < ent.size() && ent[j].run == ent[i].run && ent[j].code == ent[i].code) ++j;
    const int run = ent[i].run;
    const long long code = ent[i].code;
    const int nr = runs.nring[run];
    const unsigned long long* perb = ring_rows + (size_t)run * kStatsMaxRings;
    cair_final_state& F = out[o++];
    std::memset(&F, 0, sizeof F);
    F.run = run;
    F.nrings = nr;
    for (size_t a = i; a < j; ++a) F.count += (int64_t)ent[a].count;
    for (int q = 0; q < nr; ++q) F.nrows += (int64_t)perb[q];
    // IniState from the run's initial-state code (ProcessStatistics, 782-929)
    long long isum = runs.ini[run], ifact = ifacts;
    for (int cnd = nc - 1; cnd >= 0; --cnd) {
      ifact /= qn;
      const long long t = isum / ifact;
      F.ini[cnd] = (int)(t - 2);
      isum -= t * ifact;
    }
    // ring areas, then Cross and CrossSD summed over the rings
    const double* e = runs.ring_b.data() + (size_t)run * kStatsMaxRings;
    double cr = 0.0, sd = 0.0, prev = 0.0;
    for (int q = 0; q < nr; ++q) {
      const double t = pi * e[q] * e[q];
      double area = t - prev;
      prev = t;
      if (nr == 1 && area == 0.0) area = 1.0;
      unsigned long long w = 0;
      for (size_t a = i; a < j; ++a)
        if (ent[a].ring == q) w += ent[a].count;
      const double pb = (double)std::max<unsigned long long>(perb[q], 1ull);
      const double fw = (double)w / pb;
      cr = cr + area * fw;
      sd = sd + fw * (1.0 - fw) * area * area / pb;
    }
    F.cross = cr;
    F.cross_sd = std::sqrt(sd);
    // FinCondVec from the code, with even/oddness restored where the arrangement is kept
    const int ini_arr = F.ini[nc - 1] / 16;
    isum = code;
    ifact = ifacts;
    int fin_arr = 0;
    for (int cnd = nc - 1; cnd >= 0; --cnd) {
      ifact /= qn;
      long long fc = isum / ifact;
      if (cnd == nc - 1) fin_arr = (int)((fc - 2) / 16);
      isum -= fc * ifact;
      fc -= 2;
      if (P.pres_even_odd[cnd] && ini_arr == fin_arr) {
        fc = fc * 2;
        if (F.ini[cnd] % 2 != 0) fc = fc + 1;
      }
      F.fin[cnd] = (int)fc;
    }
    const double vp = std::sqrt(2.0 * runs.ttra[run] * k_to_h / P.xmu);
    const double vel = 2.0 / std::sqrt(pi) * vp * 4.134137e16 * (bohr_cm * bohr_cm * bohr_cm);
    F.rate = F.cross * vel;
    F.rate_sd = F.cross_sd * vel;
    i = j;
  }
  *nout = o;
  return "";
}

}  // namespace cair

// Internal entry points (not part of include/cair_gpu.h): the host half alone, for tests that count
// the keys themselves.  Both return 0 or CAIR_EINVAL with the message copied into err.
namespace {
int report(const std::string& e, char* err, int errcap) {
  if (e.empty()) return 0;
  if (err && errcap > 0) {
    std::strncpy(err, e.c_str(), (size_t)errcap - 1);
    err[errcap - 1] = 0;
  }
  return CAIR_EINVAL;
}
}  // namespace

extern "C" int cair_internal_stats_rings(const cair_stats_params* P, int32_t nitems, const cair_work_item* items,
                                         const int32_t* item_run, const unsigned long long* item_rows,
                                         const long long* item_ini, double* ring_b, int32_t* nring, int32_t* R,
                                         int32_t* nruns, char* err, int errcap) {
  cair::StatsRuns runs;
  std::string e = cair::stats_runs(nitems, items, item_run, runs);
  if (e.empty()) e = cair::stats_rings(*P, nitems, items, item_rows, item_ini, runs);
  if (!e.empty()) return report(e, err, errcap);
  std::memcpy(ring_b, runs.ring_b.data(), runs.ring_b.size() * sizeof(double));
  std::memcpy(nring, runs.nring.data(), runs.nring.size() * sizeof(int32_t));
  *R = runs.R;
  *nruns = runs.nruns;
  return 0;
}

extern "C" int cair_internal_stats_finish(const cair_stats_params* P, int32_t nitems, const cair_work_item* items,
                                          const int32_t* item_run, const unsigned long long* item_rows,
                                          const long long* item_ini, int64_t n, const unsigned long long* keys,
                                          const unsigned long long* counts, const unsigned long long* ring_rows,
                                          cair_final_state* out, int64_t cap, int64_t* nout, char* err, int errcap) {
  cair::StatsRuns runs;
  std::string e = cair::stats_runs(nitems, items, item_run, runs);
  if (e.empty()) e = cair::stats_rings(*P, nitems, items, item_rows, item_ini, runs);
  if (e.empty()) e = cair::stats_finish(*P, runs, n, keys, counts, ring_rows, out, cap, nout);
  return report(e, err, errcap);
}

extern "C" int cair_statistics_finish(int32_t nitems, const cair_work_item* items, const int32_t* item_run,
                                      const uint64_t* item_rows, const int64_t* item_ini,
                                      const cair_stats_params* params, int64_t n, const cair_stats_count* counts,
                                      const uint64_t* ring_rows, cair_final_state* out, int64_t cap, int64_t* nout,
                                      char* msg, int32_t msg_cap) {
  if (nitems < 1 || !items || !item_rows || !item_ini || !params || n < 0 || (n > 0 && !counts) || !ring_rows ||
      cap < 0 || (cap > 0 && !out) || !nout)
    return report("cair_statistics_finish: bad argument", msg, msg_cap);
  if (params->ncond != 3 && params->ncond != 5) return report("cair_statistics_finish: ncond must be 3 or 5", msg, msg_cap);
  cair::StatsRuns runs;
  std::string e = cair::stats_runs(nitems, items, item_run, runs);
  if (e.empty())
    e = cair::stats_rings(*params, nitems, items, (const unsigned long long*)item_rows, (const long long*)item_ini,
                          runs);
  if (!e.empty()) return report(e, msg, msg_cap);
  std::vector<cair::StatsEntry> ent((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    const cair_stats_count& c = counts[i];
    if (c.run < 0 || c.run >= runs.nruns || c.ring < 0 || c.ring >= runs.nring[c.run] || c.count < 0)
      return report("cair_statistics_finish: a count outside the runs and rings of the totals", msg, msg_cap);
    ent[i] = cair::StatsEntry{(long long)c.code, c.run, c.ring, (unsigned long long)c.count};
  }
  *nout = 0;
  e = cair::stats_finish_entries(*params, runs, std::move(ent), (const unsigned long long*)ring_rows, out, cap, nout);
  return report(e, msg, msg_cap);
}
