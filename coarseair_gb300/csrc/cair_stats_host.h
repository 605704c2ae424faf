// Host half of the final-state statistics (no CUDA): the impact-parameter rings of every run
// before the counting pass, and the statistics lines from the counted (run, final state, ring)
// table after it.  cair_statistics_dev calls these between and after its two device passes; the
// extern "C" wrappers let the CPU tests drive them with keys they count themselves.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cair_gpu.h"

namespace cair {

constexpr int kStatsMaxRings = 64;  // impact-parameter rings per run

struct StatsRuns {
  int32_t nruns = 0;
  int32_t R = 1;                      // largest ring count of a run (the key's ring radix)
  std::vector<int32_t> run_of;        // run of each item
  std::vector<double> ttra;           // temperature of each run
  std::vector<double> ring_b;         // ascending ring bounds, kStatsMaxRings per run
  std::vector<int32_t> nring;         // rings of each run
  std::vector<long long> ini;         // smallest initial-state code of each run
};

// Runs from item_run (NULL: every item its own run) and the items' temperatures; "" or an error.
std::string stats_runs(int32_t nitems, const cair_work_item* items, const int32_t* item_run, StatsRuns& out);
// SetRings per run from the items with counted rows (item_rows > 0): the distinct |bmax| within
// 1e-3, ascending; IniState code = the smallest of the run's items'; then the key's ring radix R
// and the range check of the key.  "" or an error.
std::string stats_rings(const cair_stats_params& P, int32_t nitems, const cair_work_item* items,
                        const unsigned long long* item_rows, const long long* item_ini, StatsRuns& runs);
// One counted (run, final-state code, ring) entry of the table.
struct StatsEntry {
  long long code;
  int run, ring;
  unsigned long long count;
};

// The table's keys decoded: key = (code x nruns + run) x R + ring, the code possibly negative.
std::vector<StatsEntry> stats_decode(const StatsRuns& runs, int64_t n, const unsigned long long* keys,
                                     const unsigned long long* counts);
// WriteFinStateProbabilities over decoded entries (any order; entries with equal run, code and ring
// must already be summed); lines sorted by run then code.  "" or an error (cap too small).
std::string stats_finish_entries(const cair_stats_params& P, const StatsRuns& runs, std::vector<StatsEntry> ent,
                                 const unsigned long long* ring_rows, cair_final_state* out, int64_t cap,
                                 int64_t* nout);
// WriteFinStateProbabilities over the counted entries: key = (code x nruns + run) x R + ring,
// ring_rows = TrajsPerb of each (run, ring); lines sorted by run then code.  "" or an error
// (cap too small).
std::string stats_finish(const cair_stats_params& P, const StatsRuns& runs, int64_t n, const unsigned long long* keys,
                         const unsigned long long* counts, const unsigned long long* ring_rows, cair_final_state* out,
                         int64_t cap, int64_t* nout);

}  // namespace cair
