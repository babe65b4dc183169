// adams_schedule.cpp -- coefficients and the per-level schedule of
// AdamsBashforth with local time stepping (see adams.hpp).
#include "adams.hpp"

#include <algorithm>
#include <cmath>

#include "host_setup.hpp"

namespace dgsw {
namespace {

// Adams-Bashforth weights for constant steps, oldest point first: the
// standard table (AdamsCoefficients.cpp:20-47 lists the same rationals).
const double kAbNum[kAbMaxOrder][kAbMaxOrder] = {
    {1},
    {-1, 3},
    {5, -16, 23},
    {-9, 37, -59, 55},
    {251, -1274, 2616, -2774, 1901},
    {-475, 2877, -7298, 9982, -7923, 4277},
    {19087, -134472, 407139, -688256, 705549, -447288, 198721},
    {-36799, 295767, -1041723, 2102243, -2664477, 2183877, -1152169, 434241}};
const double kAbDen[kAbMaxOrder] = {1, 2, 12, 24, 720, 1440, 60480, 120960};

// Exact times: ticks, slab / ticks_per_slab each.  As the reference's
// TimeDelta::value (Time.cpp:116-118) a difference of d ticks is
// slab * (d / ticks_per_slab).
struct Ticks {
  double slab;
  int64_t S;
  double span(int64_t d) const { return slab * ((double)d / (double)S); }
  // Time::compute_value (Time.cpp:96-99) on the slab holding t
  double at(int64_t t) const {
    const int64_t m = t >= 0 ? t / S : -((S - 1 - t) / S);
    const int64_t r = t - m * S;
    return ((double)(S - r) / (double)S) * (slab * (double)m) +
           ((double)r / (double)S) * (slab * (double)(m + 1));
  }
};

// integral over [a, b] of each Lagrange polynomial on the nodes x, by a
// Gauss-Legendre rule exact for their degree
void lagrange_integrals(const std::vector<double>& x, double a, double b, double* out) {
  const int n = (int)x.size();
  GaussTables gq;
  lg_spectral(std::max(2, n / 2 + 1), &gq);
  const double half = 0.5 * (b - a), mid = 0.5 * (a + b);
  for (int j = 0; j < n; ++j) {
    double acc = 0.0;
    for (int q = 0; q < gq.n; ++q) {
      const double t = mid + half * gq.x[q];
      double l = 1.0;
      for (int m = 0; m < n; ++m)
        if (m != j) l *= (t - x[m]) / (x[j] - x[m]);
      acc += gq.w[q] * l;
    }
    out[j] = half * acc;
  }
}

bool same_id(const AbId& a, const AbId& b) { return a.slab == b.slab && a.tick == b.tick; }
bool id_less(const AbId& a, const AbId& b) {
  return a.slab < b.slab || (a.slab == b.slab && a.tick < b.tick);
}

// the `order` history entries ending at the last one before time `end`
// (find_relevant_ids, AdamsLts.cpp:178-210)
int relevant(const std::vector<AbId>& h, int64_t end, int order) {
  int stop = (int)h.size();
  while (stop > 0 && h[stop - 1].tick >= end) --stop;
  return stop >= order ? stop - order : -1;
}

}  // namespace

bool adams_step_coefficients(int n, const int64_t* t, int64_t start, int64_t end, double slab,
                             int64_t ticks_per_slab, double* out) {
  if (n < 0 || n > kAbMaxOrder || ticks_per_slab < 1 || (n > 0 && (!t || !out))) return false;
  if (n == 0) return true;
  const Ticks T{slab, ticks_per_slab};
  bool uniform = true;
  for (int i = 1; i < n; ++i) uniform = uniform && t[i] - t[i - 1] == end - start;
  if (uniform && t[n - 1] == start) {
    const double h = T.span(end - start);
    for (int i = 0; i < n; ++i) out[i] = (kAbNum[n - 1][i] / kAbDen[n - 1]) * h;
    return true;
  }
  // control times relative to the first one, accumulated step by step
  std::vector<double> x(n, 0.0);
  for (int i = 1; i < n; ++i) x[i] = x[i - 1] + T.span(t[i] - t[i - 1]);
  lagrange_integrals(x, x[n - 1] + T.span(start - t[n - 1]), x[n - 1] + T.span(end - t[n - 1]),
                     out);
  return true;
}

int adams_lts_terms(const std::vector<AbId>& local, const std::vector<AbId>& remote, int64_t start,
                    int64_t end, int lo, int ro, int so, double slab, int64_t S,
                    std::vector<AbTerm>* out) {
  out->clear();
  if (start == end) return 0;
  if (lo < 1 || ro < 1 || so < 1 || lo > kAbMaxOrder || ro > kAbMaxOrder || so > kAbMaxOrder)
    return -1;
  const Ticks T{slab, S};
  std::vector<AbTerm> terms;
  int64_t sub_end = end;
  for (;;) {
    const int lf = relevant(local, sub_end, lo), rf = relevant(remote, sub_end, ro);
    if (lf < 0 || rf < 0) return -1;
    if (terms.empty() && lo == ro && lo == so) {
      // both sides stepped together: the global-stepping weights
      // (lts_coefficients_for_gts, AdamsLts.cpp:288-299)
      bool gts = true;
      for (int i = 0; i < lo && gts; ++i) gts = same_id(local[lf + i], remote[rf + i]);
      if (gts) {
        int64_t tk[kAbMaxOrder];
        double c[kAbMaxOrder];
        for (int i = 0; i < lo; ++i) tk[i] = local[lf + i].tick;
        adams_step_coefficients(lo, tk, start, end, slab, S, c);
        for (int i = 0; i < lo; ++i) out->push_back({lf + i, rf + i, c[i]});
        return 0;
      }
    }
    // the small steps: the union of both sides' step times, newest so of
    // them (merge_to_small_steps, AdamsLts.cpp:212-272)
    int64_t small[kAbMaxOrder];
    int a = lo - 1, b = ro - 1;
    for (int o = so - 1; o >= 0; --o) {
      const int64_t ta = a >= 0 ? local[lf + a].tick : INT64_MIN;
      const int64_t tb = b >= 0 ? remote[rf + b].tick : INT64_MIN;
      if (a < 0 && b < 0) return -1;
      small[o] = std::max(ta, tb);
      if (a >= 0 && ta == small[o]) --a;
      if (b >= 0 && tb == small[o]) --b;
    }
    const int64_t cur = small[so - 1];
    if (cur < start) return -2;
    double sc[kAbMaxOrder];
    adams_step_coefficients(so, small, cur, sub_end, slab, S, sc);
    // each small-step time's value on either side: its own record when the
    // side has one there, else the side's interpolant (AdamsLts.cpp:274-299)
    auto weights = [&](const std::vector<AbId>& h, int first, int n, int64_t t, double* w) {
      for (int i = 0; i < n; ++i)
        if (h[first + i].tick == t) {
          for (int k = 0; k < n; ++k) w[k] = k == i ? 1.0 : 0.0;
          return;
        }
      const double x = T.at(t);
      for (int i = 0; i < n; ++i) {
        const double xi = T.at(h[first + i].tick);
        double r = 1.0;
        for (int m = 0; m < n; ++m)
          if (m != i) {
            const double xm = T.at(h[first + m].tick);
            r *= (xm - x) / (xm - xi);
          }
        w[i] = r;
      }
    };
    for (int s = 0; s < so; ++s) {
      double wl[kAbMaxOrder], wr[kAbMaxOrder];
      weights(local, lf, lo, small[s], wl);
      weights(remote, rf, ro, small[s], wr);
      for (int i = 0; i < lo; ++i)
        for (int k = 0; k < ro; ++k)
          if (wl[i] != 0.0 && wr[k] != 0.0) terms.push_back({lf + i, rf + k, sc[s] * wl[i] * wr[k]});
    }
    if (cur == start) break;
    sub_end = cur;
  }
  // one term per (local id, remote id), summed in ascending order
  std::sort(terms.begin(), terms.end(), [&](const AbTerm& x, const AbTerm& y) {
    if (x.local != y.local) return id_less(local[x.local], local[y.local]);
    if (x.remote != y.remote) return id_less(remote[x.remote], remote[y.remote]);
    return x.coef < y.coef;
  });
  for (const AbTerm& t : terms) {
    if (!out->empty() && out->back().local == t.local && out->back().remote == t.remote)
      out->back().coef += t.coef;
    else
      out->push_back(t);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// The schedule.  Per level it keeps what the reference keeps per element
// (AdamsBashforth.cpp:131-330, SelfStartActions.hpp:136-482,
// ComputeTimeDerivative.hpp:642-645, ApplyBoundaryCorrections.hpp:990-1011,
// CleanHistory.hpp:63-130): a step records dt u and the face data at its
// start, and at its end the volume update and the boundary delta are applied
// and the histories cleaned.  One device launch handles one tick position:
// the levels whose step ends there finish it and record the next.

bool AdamsSchedule::init(int order, const bool adj[kAbMaxLevels][kAbMaxLevels],
                         const int64_t count[kAbMaxLevels], std::string* err) {
  if (order < 1 || order > kAbMaxOrder) {
    *err = "Adams-Bashforth order must be in [1, 8]";
    return false;
  }
  order_ = order;
  L_ = -1;
  for (int l = 0; l < kAbMaxLevels; ++l) {
    count_[l] = count[l];
    lv_[l].present = count[l] > 0;
    if (count[l] > 0) L_ = l;
    for (int m = 0; m < kAbMaxLevels; ++m) adj_[l][m] = adj[l][m];
  }
  if (L_ < 0) {
    *err = "no elements";
    return false;
  }
  // a slab is order * 2^L ticks: the start-up steps are one tick
  // (SelfStartActions.hpp:196-216 divides the first step by the number of
  // values to generate plus one), the first real steps slab / 2^L for every
  // level, and from the first slab boundary after which no start-up value is
  // left in any history each level steps slab / 2^level.
  S_ = (int64_t)order << L_;
  first_step_ = S_ >> L_;
  const int64_t switch_slabs = ((int64_t)order - 1 + ((int64_t)1 << L_) - 1) >> L_;
  switch_tick_ = switch_slabs * S_;
  // dry run over the start-up, the switch and a few periodic slabs: the
  // largest ring slot any level needs
  dry_ = true;
  ring_slots_ = 127;
  max_slot_ = -1;
  slab_ = 1.0;
  restart();
  std::vector<AbLaunch> scratch;
  for (int64_t s = 0; s < switch_slabs + 3; ++s)
    if (!slab(&scratch, err)) return false;
  ring_slots_ = max_slot_ + 1;
  dry_ = false;
  restart();
  return true;
}

void AdamsSchedule::restart() {
  for (Level& l : lv_) {
    l.vol.clear();
    l.loc.clear();
    for (auto& r : l.rem) r.clear();
    l.start = l.end = 0;
    l.pending = false;
  }
  next_slab_ = 0;
  started_ = false;
}

bool AdamsSchedule::live(int l, int slot) const {
  for (const Rec& r : lv_[l].vol)
    if (r.slot == slot) return true;
  for (const Rec& r : lv_[l].loc)
    if (r.slot == slot) return true;
  for (int x = 0; x < kAbMaxLevels; ++x)
    for (const Rec& r : lv_[x].rem[l])
      if (r.slot == slot) return true;
  return false;
}

int AdamsSchedule::alloc_slot(int l, const std::vector<int>& busy, std::string* err) {
  for (int s = 0; s < ring_slots_; ++s) {
    if (std::find(busy.begin(), busy.end(), s) != busy.end() || live(l, s)) continue;
    max_slot_ = std::max(max_slot_, s);
    return s;
  }
  *err = "history ring exhausted";
  return -1;
}

void AdamsSchedule::clean(int l) {
  Level& v = lv_[l];
  const size_t ov = (size_t)v.vol.back().order;
  while (v.vol.size() >= ov) v.vol.erase(v.vol.begin());
  const size_t ob = (size_t)v.loc.back().order;
  while (v.loc.size() >= ob) v.loc.erase(v.loc.begin());
  for (auto& r : v.rem)
    while (r.size() > ob) r.erase(r.begin());
}

bool AdamsSchedule::position(AbId id, const bool* finish, bool reset, int rec_order,
                             bool unused_record, std::vector<AbLaunch>* out, std::string* err) {
  AbLaunch launch;
  std::vector<int> busy[kAbMaxLevels];
  int job_of[kAbMaxLevels];
  int64_t first = 0;
  for (int l = 0; l < kAbMaxLevels; ++l) {
    job_of[l] = -1;
    const int64_t begin = first;
    first += count_[l];
    if (!lv_[l].present || !finish[l]) continue;
    AbLevelJob& job = launch.job[launch.n_jobs];
    job_of[l] = launch.n_jobs++;
    job.level = l;
    job.begin = (int32_t)begin;
    job.count = (int32_t)count_[l];
    Level& v = lv_[l];
    if (!v.pending) continue;
    job.update = 1;
    // volume: AdamsBashforth::update_u over the last `order` records
    const int ov = v.vol.back().order;
    if ((int)v.vol.size() != ov) {
      *err = "volume history does not hold the integration order's records";
      return false;
    }
    int64_t tk[kAbMaxOrder];
    for (int i = 0; i < ov; ++i) tk[i] = v.vol[i].id.tick;
    adams_step_coefficients(ov, tk, v.start, id.tick, slab_, S_, job.vol_c);
    job.n_vol = (int8_t)ov;
    for (int i = 0; i < ov; ++i) {
      job.vol_slot[i] = (int8_t)v.vol[i].slot;
      busy[l].push_back(v.vol[i].slot);
    }
    // boundary: add_boundary_delta per neighbour level
    const int ob = v.loc.back().order;
    std::vector<AbId> lid;
    for (const Rec& r : v.loc) lid.push_back(r.id);
    for (int m = 0; m < kAbMaxLevels; ++m) {
      if (!adj_[l][m]) continue;
      std::vector<AbId> rid;
      for (const Rec& r : v.rem[m]) rid.push_back(r.id);
      std::vector<AbTerm> terms;
      if (adams_lts_terms(lid, rid, v.start, id.tick, ob, ob, ob, slab_, S_, &terms)) {
        *err = "a boundary history lacks the data of the step";
        return false;
      }
      AbFaceTable& f = job.face[m];
      std::vector<double> a(v.loc.size(), 0.0), b(v.rem[m].size(), 0.0);
      std::vector<bool> ua(v.loc.size(), false), ub(v.rem[m].size(), false);
      for (const AbTerm& t : terms) {
        a[t.local] += t.coef;
        b[t.remote] += t.coef;
        ua[t.local] = ub[t.remote] = true;
      }
      for (size_t i = 0; i < a.size(); ++i)
        if (ua[i]) {
          if (f.n_loc >= kAbMaxOrder) {
            *err = "too many local terms";
            return false;
          }
          f.loc_slot[f.n_loc] = (int8_t)v.loc[i].slot;
          f.loc_c[f.n_loc++] = a[i];
          busy[l].push_back(v.loc[i].slot);
        }
      for (size_t i = 0; i < b.size(); ++i)
        if (ub[i]) {
          if (f.n_rem >= kAbMaxRemote) {
            *err = "too many remote terms";
            return false;
          }
          f.rem_slot[f.n_rem] = (int8_t)v.rem[m][i].slot;
          f.rem_c[f.n_rem++] = b[i];
          busy[m].push_back(v.rem[m][i].slot);
        }
    }
    v.pending = false;
  }
  // clean after every level's reads (CleanHistory follows the delta)
  for (int l = 0; l < kAbMaxLevels; ++l)
    if (job_of[l] >= 0 && launch.job[job_of[l]].update) clean(l);
  // records of the new state
  for (int l = 0; l < kAbMaxLevels; ++l) {
    if (job_of[l] < 0) continue;
    AbLevelJob& job = launch.job[job_of[l]];
    job.reset = reset ? 1 : 0;
    const int slot = alloc_slot(l, busy[l], err);
    if (slot < 0) return false;
    job.rec_slot = (int8_t)slot;
    const Rec rec{id, rec_order, slot};
    lv_[l].vol.push_back(rec);
    lv_[l].loc.push_back(rec);
    for (int x = 0; x < kAbMaxLevels; ++x)
      if (lv_[x].present && adj_[x][l]) lv_[x].rem[l].push_back(rec);
  }
  for (int l = 0; l < kAbMaxLevels; ++l) {
    if (job_of[l] < 0) continue;
    if (unused_record) {
      clean(l);  // SelfStart::step_unused: no update, histories cleaned
    } else {
      lv_[l].pending = true;
      lv_[l].start = id.tick;
    }
  }
  if (!dry_) out->push_back(launch);
  return true;
}

bool AdamsSchedule::run_startup(std::vector<AbLaunch>* out, std::string* err) {
  bool all[kAbMaxLevels];
  for (int l = 0; l < kAbMaxLevels; ++l) all[l] = lv_[l].present;
  const int k = order_;
  // self-start: for o = 1 .. k-1 (slab number o - k), restore the initial
  // values, take o one-tick steps at order o and record one unused value
  // at tick o with order o + 1
  for (int o = 1; o < k; ++o) {
    const int64_t sn = o - k;
    for (int j = 0; j <= o; ++j) {
      if (!position(AbId{sn, j}, all, j == 0 && o > 1, j < o ? o : o + 1, j == o, out, err))
        return false;
      for (int l = 0; l < kAbMaxLevels; ++l) lv_[l].end = j + 1;
    }
  }
  if (!position(AbId{0, 0}, all, k > 1, k, false, out, err)) return false;
  for (int l = 0; l < kAbMaxLevels; ++l) lv_[l].end = step_at(l, 0);
  started_ = true;
  return true;
}

bool AdamsSchedule::slab(std::vector<AbLaunch>* out, std::string* err) {
  out->clear();
  if (!started_ && !run_startup(out, err)) return false;
  const int64_t t0 = next_slab_ * S_, t1 = t0 + S_;
  for (int64_t P = t0 + 1; P <= t1; ++P) {
    bool fin[kAbMaxLevels];
    bool any = false;
    for (int l = 0; l < kAbMaxLevels; ++l) {
      fin[l] = lv_[l].present && lv_[l].end == P;
      any = any || fin[l];
    }
    if (!any) continue;
    if (!position(AbId{P / S_, P}, fin, false, order_, false, out, err)) return false;
    for (int l = 0; l < kAbMaxLevels; ++l)
      if (fin[l]) lv_[l].end = P + step_at(l, P);
  }
  ++next_slab_;
  return true;
}

}  // namespace dgsw
