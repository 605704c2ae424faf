// trajectories.out / trajectories_HNotCons.out / trajectories.bin writers (host code).
//
// Rows follow Integrator_Class.F90:884-920, format (I10, A, I5, 2(A, ES11.5), *(A, ES14.8)) with
// iTraj = IdxOverall, iPES 1-based, bmax, b_i, then the initial and the final conditions: J, v,
// arrangement for one initial molecule, J1, v1, J2, v2, arrangement for two (NInitMolecules, with
// the header line of Integrator_Class.F90:183-189 for each).  Fortran's formatted output is
// reproduced field by field: a value wider than its field prints as asterisks (so a negative
// number in ES14.8 is fourteen '*'), a three-digit exponent drops the 'E', NaN and Infinity are
// right-justified words.  The binary file is the stream that Statistics_Class.F90:283-314 writes
// and ReadInputsUnformatted (346-506) reads: NTraj, then per row Idx, iPES, bMax, bSampled,
// Qini(NCond), Qfin(NCond) as 8-byte integers and reals.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cair_gpu.h"

namespace {

void put_int(std::string& s, long long v, int w) {
  char b[32];
  int n = std::snprintf(b, sizeof b, "%lld", v);
  if (n > w) s.append((size_t)w, '*');
  else s.append((size_t)(w - n), ' ').append(b, (size_t)n);
}

// Fortran ESw.d: one nonzero digit, d decimals, exponent E+dd (or +ddd without the E)
void put_es(std::string& s, double x, int w, int d) {
  char b[64];
  int n;
  if (std::isnan(x)) n = std::snprintf(b, sizeof b, "NaN");
  else if (std::isinf(x)) n = std::snprintf(b, sizeof b, x > 0 ? (w >= 8 ? "Infinity" : "Inf") : (w >= 9 ? "-Infinity" : "-Inf"));
  else {
    n = std::snprintf(b, sizeof b, "%.*E", d, x);
    char* e = std::strchr(b, 'E');
    if (e) {
      int ex = std::atoi(e + 1);
      if (ex > 99 || ex < -99) {  // three exponent digits: drop the E
        std::memmove(e, e + 1, std::strlen(e + 1) + 1);
        n -= 1;
      }
    }
  }
  if (n > w) s.append((size_t)w, '*');
  else s.append((size_t)(w - n), ' ').append(b, (size_t)n);
}

// The NCond initial then the NCond final conditions of a row (3 or 5 per side).
int conditions(const cair_traj_result& r, int nmol, double* q) {
  if (nmol == 1) {
    const double v[6] = {r.j_i, r.v_i, r.arr_i, r.j_f, r.v_f, r.arr_f};
    std::memcpy(q, v, sizeof v);
    return 3;
  }
  const double v[10] = {r.j_i, r.v_i, r.j2_i, r.v2_i, r.arr_i, r.j_f, r.v_f, r.j2_f, r.v2_f, r.arr_f};
  std::memcpy(q, v, sizeof v);
  return 5;
}

void format_row(std::string& s, const cair_traj_result& r, int64_t idx_offset, int nmol) {
  put_int(s, idx_offset + r.idx, 10);
  s += ',';
  put_int(s, (long long)r.ipes + 1, 5);
  s += ',';
  put_es(s, r.bmax, 11, 5);
  s += ',';
  put_es(s, r.b, 11, 5);
  double q[10];
  const int nc = conditions(r, nmol, q);
  for (int c = 0; c < 2 * nc; ++c) {
    s += ',';
    put_es(s, q[c], 14, 8);
  }
  s += '\n';
}

const char* kHeader1 =
    "#    iTraj, iPES,       bmax,        b_i,           j_i,           v_i,         arr_i,           j_f,"
    "           v_f,         arr_f\n";
const char* kHeader2 =
    "#    iTraj, iPES,       bmax,        b_i,          j1_i,          v1_i,          j2_i,          v2_i,"
    "         arr_i,          j1_f,          v1_f,          j2_f,          v2_f,         arr_f\n";

const char* header(int nmol) { return nmol == 1 ? kHeader1 : kHeader2; }

bool conserved(const cair_traj_result& r, double tol) {
  return r.status == CAIR_TRAJ_DONE && std::fabs(r.dH) <= tol;
}

// Runs work(0..nt-1), work(0) on the calling thread and the others on their own threads (inline
// when a thread cannot be started), and returns when all are done.
template <class F>
void run_parallel(int nt, F&& work) {
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) {
    try {
      th.emplace_back(work, t);
    } catch (...) {
      work(t);
    }
  }
  work(0);
  for (std::thread& x : th) x.join();
}

}  // namespace

extern "C" {

int cair_format_rows(const cair_traj_result* rows, int64_t n, int64_t idx_offset, int32_t nmol, int32_t with_header,
                     char* buf, int64_t cap, int64_t* len) {
  if (n < 0 || (n > 0 && !rows) || !len || cap < 0 || (cap > 0 && !buf) || (nmol != 1 && nmol != 2))
    return CAIR_EINVAL;
  std::string s;
  if (with_header) s += header(nmol);
  for (int64_t k = 0; k < n; ++k) format_row(s, rows[k], idx_offset, nmol);
  *len = (int64_t)s.size();
  if ((int64_t)s.size() > cap) return CAIR_EINVAL;
  std::memcpy(buf, s.data(), s.size());
  return 0;
}

int cair_write_trajectories(const char* dir, const cair_traj_result* rows, int64_t n, int64_t idx_offset, int32_t nmol,
                            double ham_abs_tol, int64_t* counts) {
  if (!dir || n < 0 || (n > 0 && !rows) || (nmol != 1 && nmol != 2)) return CAIR_EINVAL;
  const std::string d(dir);
  FILE* f[2] = {std::fopen((d + "/trajectories.out").c_str(), "w"),
                std::fopen((d + "/trajectories_HNotCons.out").c_str(), "w")};
  if (!f[0] || !f[1]) {
    for (FILE* x : f)
      if (x) std::fclose(x);
    return CAIR_EINVAL;
  }
  // Rows are formatted in batches of nt chunks, the chunks on their own threads, and written chunk
  // by chunk in row order, so the files are the same as a sequential write's.
  const int64_t chunk = 16384;
  const int nt = (int)std::max<int64_t>(1, std::min<int64_t>({16, (int64_t)std::thread::hardware_concurrency(),
                                                               (n + chunk - 1) / chunk}));
  std::vector<std::string> part[2] = {std::vector<std::string>(nt), std::vector<std::string>(nt)};
  std::vector<int64_t> cnt(2 * (size_t)nt, 0);
  bool ok = std::fputs(header(nmol), f[0]) >= 0 && std::fputs(header(nmol), f[1]) >= 0;
  for (int64_t base = 0; base < n && ok; base += chunk * nt) {
    run_parallel(nt, [&](int t) {
      part[0][t].clear();
      part[1][t].clear();
      const int64_t lo = base + chunk * t, hi = std::min(n, lo + chunk);
      for (int64_t k = lo; k < hi; ++k) {
        const int which = conserved(rows[k], ham_abs_tol) ? 0 : 1;
        format_row(part[which][t], rows[k], idx_offset, nmol);
        ++cnt[2 * (size_t)t + which];
      }
    });
    for (int t = 0; t < nt; ++t)
      for (int i = 0; i < 2; ++i)
        ok = ok && std::fwrite(part[i][t].data(), 1, part[i][t].size(), f[i]) == part[i][t].size();
  }
  int64_t c[2] = {0, 0};
  for (int t = 0; t < nt; ++t) {
    c[0] += cnt[2 * (size_t)t];
    c[1] += cnt[2 * (size_t)t + 1];
  }
  for (int i = 0; i < 2; ++i) ok = (std::fclose(f[i]) == 0) && ok;
  if (counts) {
    counts[0] = c[0];
    counts[1] = c[1];
  }
  return ok ? 0 : CAIR_EINVAL;
}

int cair_write_trajectories_bin(const char* path, const cair_traj_result* rows, int64_t n, int64_t idx_offset,
                                int32_t nmol, double ham_abs_tol) {
  if (!path || n < 0 || (n > 0 && !rows) || (nmol != 1 && nmol != 2)) return CAIR_EINVAL;
  FILE* f = std::fopen(path, "wb");
  if (!f) return CAIR_EINVAL;
  int64_t nt = 0;
  for (int64_t k = 0; k < n; ++k) nt += conserved(rows[k], ham_abs_tol) ? 1 : 0;
  bool ok = std::fwrite(&nt, 8, 1, f) == 1;
  for (int64_t k = 0; k < n && ok; ++k) {
    const cair_traj_result& r = rows[k];
    if (!conserved(r, ham_abs_tol)) continue;
    const int64_t ii[2] = {idx_offset + r.idx, (int64_t)r.ipes + 1};
    double dd[12] = {r.bmax, r.b};
    const size_t nd = 2 + 2 * (size_t)conditions(r, nmol, dd + 2);
    ok = std::fwrite(ii, 8, 2, f) == 2 && std::fwrite(dd, 8, nd, f) == nd;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? 0 : CAIR_EINVAL;
}

// MergeTrajectories (scripts/executing/ComputeRates.sh:406-472), for each source directory that
// holds a trajectories.out: while <out>/trajectories.csv does not exist, the source's
// trajectories.out and trajectories_HNotCons.out are copied whole over <out>/trajectories.csv and
// <out>/trajectories_HNotCons.out; after that they are appended without their header line.  Then
// NConvTraj.dat = lines of trajectories.csv - 1.
int cair_merge_trajectories(int32_t nsrc, const char* const* src_dirs, const char* out_dir, int64_t* ntraj) {
  if (nsrc < 0 || (nsrc > 0 && !src_dirs) || !out_dir) return CAIR_EINVAL;
  const std::string out(out_dir);
  const std::string csv = out + "/trajectories.csv", hnc = out + "/trajectories_HNotCons.out";
  auto exists = [](const std::string& p) {
    FILE* f = std::fopen(p.c_str(), "rb");
    if (f) std::fclose(f);
    return f != nullptr;
  };
  // the first source is copied whole over dst (the script's `cat >`); later ones are appended
  // without their first line (`tail -n+2 >>`)
  auto append = [](const std::string& src, const std::string& dst, bool skip_header) {
    FILE* in = std::fopen(src.c_str(), "rb");
    if (!in) return false;
    FILE* o = std::fopen(dst.c_str(), skip_header ? "ab" : "wb");
    if (!o) {
      std::fclose(in);
      return false;
    }
    bool ok = true, at_body = !skip_header;
    char buf[1 << 16];
    size_t n;
    while (ok && (n = std::fread(buf, 1, sizeof buf, in)) > 0) {
      size_t from = 0;
      if (!at_body) {
        const char* nl = (const char*)std::memchr(buf, '\n', n);
        if (!nl) continue;
        from = (size_t)(nl - buf) + 1;
        at_body = true;
      }
      ok = std::fwrite(buf + from, 1, n - from, o) == n - from;
    }
    ok = !std::ferror(in) && ok;
    std::fclose(in);
    return (std::fclose(o) == 0) && ok;
  };
  bool ok = true;
  for (int32_t i = 0; i < nsrc && ok; ++i) {
    if (!src_dirs[i]) return CAIR_EINVAL;
    const std::string d(src_dirs[i]);
    if (!exists(d + "/trajectories.out")) continue;
    const bool first = !exists(csv);
    ok = append(d + "/trajectories.out", csv, !first);
    if (ok && exists(d + "/trajectories_HNotCons.out")) ok = append(d + "/trajectories_HNotCons.out", hnc, !first);
  }
  if (!ok) return CAIR_EINVAL;
  int64_t lines = 0;
  if (FILE* f = std::fopen(csv.c_str(), "rb")) {
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0)
      for (size_t k = 0; k < n; ++k) lines += buf[k] == '\n';
    std::fclose(f);
  }
  const int64_t nt = lines > 0 ? lines - 1 : 0;
  FILE* f = std::fopen((out + "/NConvTraj.dat").c_str(), "w");
  if (!f) return CAIR_EINVAL;
  ok = std::fprintf(f, "%lld\n", (long long)nt) > 0;
  ok = (std::fclose(f) == 0) && ok;
  if (ntraj) *ntraj = nt;
  return ok ? 0 : CAIR_EINVAL;
}

}  // extern "C"
