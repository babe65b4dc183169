// adams_oracle.cpp -- CPU FP64 restatement of SpECTRE's Adams-Bashforth time
// stepper with local time stepping (test infrastructure only; part of the
// oracle library, never linked by the product).
//
// Follows (file:line relative to the SpECTRE source tree):
//   constant AB coefficients     src/Time/TimeSteppers/AdamsCoefficients.cpp:20-47
//   variable_coefficients        src/Time/TimeSteppers/AdamsCoefficients.cpp:73-117
//   coefficients (dispatcher)    src/Time/TimeSteppers/AdamsCoefficients.hpp:29-67
//   find_relevant_ids            src/Time/TimeSteppers/AdamsLts.cpp:178-210
//   merge_to_small_steps         src/Time/TimeSteppers/AdamsLts.cpp:212-272 (explicit)
//   interpolation_coefficients   src/Time/TimeSteppers/AdamsLts.cpp:274-299
//   lts_coefficients(_for_gts)   src/Time/TimeSteppers/AdamsLts.cpp:301-415
//   AB update / clean / boundary src/Time/TimeSteppers/AdamsBashforth.cpp:131-330
//   self-start procedure         src/Time/Actions/SelfStartActions.hpp:136-482,
//                                src/Time/SelfStart.cpp:9-17
//   LTS DG step                  src/Evolution/DiscontinuousGalerkin/Actions/
//                                ComputeTimeDerivative.hpp:642-645,776-840 (record +
//                                volume update), ApplyBoundaryCorrections.hpp:
//                                816-1011 (coupling, add_boundary_delta,
//                                add_slice_to_data), src/Time/TakeStep.hpp:36-61,
//                                src/Time/Actions/CleanHistory.hpp:63-130
//
// Times are exact: an integer tick count, a slab being ticks_per_slab ticks,
// converted to double the way the reference's Time/TimeDelta do
// (src/Time/Time.cpp:96-118: slab duration times the reduced fraction).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <vector>

#include "adams_oracle.hpp"
#include "dgsw_oracle.h"

namespace {

constexpr int kMaxOrder = 8;

// Adams-Bashforth coefficients for constant steps, oldest first, as exact
// rationals over a common denominator (the standard table; equal to the
// reference's values, AdamsCoefficients.cpp:20-47).
const double kAbNum[kMaxOrder][kMaxOrder] = {
    {1},
    {-1, 3},
    {5, -16, 23},
    {-9, 37, -59, 55},
    {251, -1274, 2616, -2774, 1901},
    {-475, 2877, -7298, 9982, -7923, 4277},
    {19087, -134472, 407139, -688256, 705549, -447288, 198721},
    {-36799, 295767, -1041723, 2102243, -2664477, 2183877, -1152169, 434241}};
const double kAbDen[kMaxOrder] = {1, 2, 12, 24, 720, 1440, 60480, 120960};

struct Clock {
  double slab;     // slab duration
  int64_t ticks;   // ticks per slab
  double t0;       // initial time
  double delta(int64_t d) const { return slab * ((double)d / (double)ticks); }
  double value(int64_t t) const {
    // Time::compute_value on the slab containing t
    const int64_t m = t >= 0 ? t / ticks : -((-t + ticks - 1) / ticks);
    const int64_t r = t - m * ticks;
    const double start = t0 + slab * (double)m, end = t0 + slab * (double)(m + 1);
    return ((double)(ticks - r) / (double)ticks) * start + ((double)r / (double)ticks) * end;
  }
};

std::vector<double> variable_coefficients(std::vector<double> ct, double start, double end) {
  for (double& t : ct) t -= start;
  const size_t order = ct.size();
  std::vector<double> out;
  for (size_t j = 0; j < order; ++j) {
    // Lagrange polynomial l_j in monomial form, built one factor at a time
    std::vector<double> poly(order, 0.0);
    poly[0] = 1.0;
    for (size_t m = 0; m < order; ++m) {
      if (m == j) continue;
      const double denom = 1.0 / (ct[j] - ct[m]);
      for (size_t i = m < j ? m + 1 : m; i > 0; --i) poly[i] = (poly[i - 1] - poly[i] * ct[m]) * denom;
      poly[0] *= -ct[m] * denom;
    }
    // integral from 0 (the step start) to end - start, Horner from the top
    for (size_t m = 0; m < order; ++m) poly[m] /= (double)(m + 1);
    const double x = end - start;
    double acc = 0.0;
    for (size_t m = order; m-- > 0;) acc = acc * x + poly[m];
    out.push_back(x * acc);
  }
  return out;
}

std::vector<double> coefficients(const std::vector<int64_t>& times, int64_t start, int64_t end,
                                 const Clock& clk) {
  if (times.empty()) return {};
  const double step = clk.delta(end - start);
  bool constant = true;
  std::vector<double> ct{0.0};
  int64_t prev = times[0];
  for (size_t i = 1; i < times.size(); ++i) {
    ct.push_back(ct.back() + clk.delta(times[i] - prev));
    if (times[i] - prev != end - start) constant = false;
    prev = times[i];
  }
  if (constant && start == prev) {
    const size_t k = times.size();
    std::vector<double> out(k);
    for (size_t i = 0; i < k; ++i) out[i] = (kAbNum[k - 1][i] / kAbDen[k - 1]) * step;
    return out;
  }
  return variable_coefficients(ct, ct.back() + clk.delta(start - prev),
                               ct.back() + clk.delta(end - prev));
}

struct Id {
  int64_t slab;
  int64_t tick;
  bool operator<(const Id& o) const { return slab < o.slab || (slab == o.slab && tick < o.tick); }
  bool operator==(const Id& o) const { return slab == o.slab && tick == o.tick; }
};

struct Term {
  int32_t local, remote;  // indices into the local / remote histories
  double coef;
};

int find_relevant(const std::vector<Id>& ids, int64_t end, int order, int* first) {
  int used_end = (int)ids.size();
  while (used_end > 0) {
    if (ids[used_end - 1].tick < end) break;
    --used_end;
  }
  if (used_end < order) return -1;  // "Insufficient past data"
  *first = used_end - order;
  return 0;
}

std::vector<double> interpolation_coefficients(const std::vector<int64_t>& ct, int64_t t,
                                               const Clock& clk) {
  std::vector<double> out(ct.size(), 0.0);
  for (size_t i = 0; i < ct.size(); ++i)
    if (ct[i] == t) {
      out[i] = 1.0;
      return out;
    }
  const double x = clk.value(t);
  for (size_t i = 0; i < ct.size(); ++i) {
    const double xi = clk.value(ct[i]);
    double r = 1.0;
    for (size_t m = 0; m < ct.size(); ++m) {
      if (m == i) continue;
      const double xm = clk.value(ct[m]);
      r *= (xm - x) / (xm - xi);
    }
    out[i] = r;
  }
  return out;
}

// lts_coefficients for explicit schemes of orders lo (local side), ro
// (remote side) and so (small steps); AdamsBashforth::add_boundary_delta_impl
// (AdamsBashforth.cpp:264-281) uses one order for all three.
int lts_coefficients(const std::vector<Id>& local, const std::vector<Id>& remote, int64_t start,
                     int64_t end, int lo, int ro, int so, const Clock& clk,
                     std::vector<Term>* out) {
  out->clear();
  if (start == end) return 0;
  std::vector<Term> terms;
  int64_t small_end = end;
  for (;;) {
    int lf, rf;
    if (find_relevant(local, small_end, lo, &lf) || find_relevant(remote, small_end, ro, &rf))
      return -1;
    bool same = terms.empty() && lo == ro && lo == so;
    for (int i = 0; same && i < lo; ++i) same = local[lf + i] == remote[rf + i];
    if (same) {
      std::vector<int64_t> t(lo);
      for (int i = 0; i < lo; ++i) t[i] = local[lf + i].tick;
      const std::vector<double> c = coefficients(t, start, end, clk);
      for (int i = 0; i < lo; ++i) out->push_back({lf + i, rf + i, c[i]});
      return 0;
    }
    std::vector<int64_t> lt(lo), rt(ro);
    for (int i = 0; i < lo; ++i) lt[i] = local[lf + i].tick;
    for (int i = 0; i < ro; ++i) rt[i] = remote[rf + i].tick;
    // merge_to_small_steps: newest first, the later of the two sides each time
    std::vector<int64_t> small(so);
    int li = lo - 1, ri = ro - 1;
    for (int o = so - 1; o >= 0; --o) {
      if (li < 0 && ri < 0) return -1;  // "Ran out of data"
      if (li < 0) {
        small[o] = rt[ri--];
      } else if (ri < 0) {
        small[o] = lt[li--];
      } else {
        const int64_t m = std::max(lt[li], rt[ri]);
        small[o] = m;
        if (lt[li] == m) --li;
        if (rt[ri] == m) --ri;
      }
    }
    const int64_t current = small[so - 1];
    if (current < start) return -2;
    const std::vector<double> sc = coefficients(small, current, small_end, clk);
    for (int s = 0; s < so; ++s) {
      const std::vector<double> lic = interpolation_coefficients(lt, small[s], clk);
      const std::vector<double> ric = interpolation_coefficients(rt, small[s], clk);
      for (int a = 0; a < lo; ++a) {
        if (lic[a] == 0.0) continue;
        for (int b = 0; b < ro; ++b) {
          if (ric[b] == 0.0) continue;
          terms.push_back({lf + a, rf + b, sc[s] * lic[a] * ric[b]});
        }
      }
    }
    if (current == start) break;
    small_end = current;
  }
  // sort by (local id, remote id, value) and combine duplicates in order
  std::sort(terms.begin(), terms.end(), [&](const Term& x, const Term& y) {
    if (!(local[x.local] == local[y.local])) return local[x.local] < local[y.local];
    if (!(remote[x.remote] == remote[y.remote])) return remote[x.remote] < remote[y.remote];
    return x.coef < y.coef;
  });
  for (const Term& t : terms) {
    if (!out->empty() && local[out->back().local] == local[t.local] &&
        remote[out->back().remote] == remote[t.remote])
      out->back().coef += t.coef;
    else
      out->push_back(t);
  }
  return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// The evolution.  Every element keeps the reference's three histories: the
// volume history of dt u (no internal mortar terms), and per internal mortar
// the local and remote boundary histories of packaged face data
// (dg_package_data).  A step records dt u and the face data, updates u with
// the volume part at once, adds the boundary delta when the step ends, then
// cleans the histories.
namespace orc_adams {
namespace {

constexpr int kVarsA = 5;

struct LocalEntry {
  Id id;
  int order;
  std::vector<double> pkg, mag;
};
struct RemoteEntry {
  Id id;
  std::vector<double> pkg;
};
struct VolEntry {
  Id id;
  int order;
  std::vector<double> dt;
};
struct Mortar {
  std::deque<LocalEntry> local;
  std::deque<RemoteEntry> remote;
};
struct Elem {
  std::deque<VolEntry> vol;
  Mortar mortar[6];
  int64_t start = 0, end = 0;
};

int64_t face_volume_index(int n, int d, int slice, int a, int b) {
  switch (d) {
    case 0: return slice + (int64_t)n * (a + (int64_t)n * b);
    case 1: return a + (int64_t)n * (slice + (int64_t)n * b);
    default: return a + (int64_t)n * (b + (int64_t)n * slice);
  }
}

struct Run {
  System& sys;
  std::vector<Elem> el;
  Clock clk;
  explicit Run(System& s) : sys(s), el(s.E) {}

  // ComputeTimeDerivative for the listed elements: dt u into the volume
  // history, face packages into the own local and the neighbours' remote
  // boundary histories
  void record(const double* u, const std::vector<int64_t>& who, Id id, int order) {
    std::vector<double> dudt((size_t)sys.total_values());
    sys.volume_rhs(u, dudt.data());
    for (int64_t e : who) {
      const int64_t o = sys.offset_of(e), per = (int64_t)kVarsA * sys.n_of(e) * sys.n_of(e) * sys.n_of(e);
      el[e].vol.push_back({id, order, std::vector<double>(dudt.begin() + o, dudt.begin() + o + per)});
      for (int dir = 0; dir < 6; ++dir) {
        const int64_t nb = sys.neighbor(e, dir);
        if (nb < 0) continue;
        LocalEntry le{id, order, {}, {}};
        sys.package(u, e, dir, &le.pkg, &le.mag);
        el[e].mortar[dir].local.push_back(std::move(le));
        const int bd = sys.back_dir(e, dir);
        RemoteEntry re{id, {}};
        sys.exterior_package(u, nb, bd, &re.pkg);
        el[nb].mortar[bd].remote.push_back(std::move(re));
      }
    }
  }

  // AdamsBashforth::update_u_impl with the element's volume history
  int volume_update(double* u, int64_t e, int64_t start, int64_t end) const {
    const std::deque<VolEntry>& h = el[e].vol;
    const int order = h.back().order;
    if ((int)h.size() != order) return -3;
    std::vector<int64_t> t;
    for (const VolEntry& v : h) t.push_back(v.id.tick);
    const std::vector<double> c = coefficients(t, start, end, clk);
    double* ue = u + sys.offset_of(e);
    const int64_t per = (int64_t)h.back().dt.size();
    for (int j = 0; j < order; ++j)
      for (int64_t p = 0; p < per; ++p) ue[p] += c[j] * h[j].dt[p];
    return 0;
  }

  // AdamsBashforth::add_boundary_delta_impl on every internal mortar, the
  // coupling being dg_boundary_terms lifted onto the GLL face; then
  // add_slice_to_data
  int boundary_delta(double* u, int64_t e, int64_t start, int64_t end) const {
    const int n = sys.n_of(e), nf = n * n;
    const int64_t np = (int64_t)nf * n;
    double* ue = u + sys.offset_of(e);
    const double slice_factor = -0.5 * (double)(n * (n - 1));
    for (int dir = 0; dir < 6; ++dir) {
      if (sys.neighbor(e, dir) < 0) continue;
      const Mortar& m = el[e].mortar[dir];
      std::vector<Id> lid, rid;
      for (const LocalEntry& x : m.local) lid.push_back(x.id);
      for (const RemoteEntry& x : m.remote) rid.push_back(x.id);
      std::vector<Term> terms;
      const int ord = m.local.back().order;
      const int rc = lts_coefficients(lid, rid, start, end, ord, ord, ord, clk, &terms);
      if (rc) return rc;
      std::vector<double> lifted((size_t)kVarsA * nf, 0.0), bc((size_t)kVarsA * nf);
      std::vector<double> bc_m;
      for (const Term& t : terms) {
        const LocalEntry& L = m.local[t.local];
        const int nm = sys.mortar_n(e, dir);
        bc_m.assign((size_t)kVarsA * nm * nm, 0.0);
        sys.boundary_terms(L.pkg, m.remote[t.remote].pkg, bc_m.data());
        sys.mortar_to_face(e, dir, bc_m.data(), bc.data());
        for (int v = 0; v < kVarsA; ++v)
          for (int f = 0; f < nf; ++f)
            lifted[(size_t)v * nf + f] += t.coef * (bc[(size_t)v * nf + f] * (slice_factor * L.mag[f]));
      }
      const int d = dir / 2, slice = (dir % 2) ? n - 1 : 0;
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const int64_t vi = face_volume_index(n, d, slice, a, b);
          for (int v = 0; v < kVarsA; ++v) ue[v * np + vi] += lifted[(size_t)v * nf + a + n * b];
        }
    }
    return 0;
  }

  // AdamsBashforth::clean_history_impl and clean_boundary_history_impl
  void clean(int64_t e) {
    std::deque<VolEntry>& h = el[e].vol;
    const size_t order = (size_t)h.back().order;
    while (h.size() >= order) h.pop_front();
    for (int dir = 0; dir < 6; ++dir) {
      Mortar& m = el[e].mortar[dir];
      if (m.local.empty()) continue;
      const size_t ob = (size_t)m.local.back().order;
      while (m.local.size() >= ob) m.local.pop_front();
      while (m.remote.size() > ob) m.remote.pop_front();
    }
  }
};

// Flat scalar wave on conforming periodic bricks of uniform extent n
struct FlatSystem : System {
  int n_inst;
  const OrcBrick* br;
  double gamma2;
  int threads;
  std::vector<int32_t> elem_n, nbr, inst;
  std::vector<double> invjac;  // 3 per element

  int64_t neighbor(int64_t e, int dir) const override { return nbr[6 * e + dir]; }
  int back_dir(int64_t, int dir) const override { return dir ^ 1; }
  void volume_rhs(const double* u, double* dudt) override {
    orc_volume_rhs(n_inst, br, elem_n.data(), gamma2, u, dudt, threads);
  }
  void package(const double* u, int64_t e, int dir, std::vector<double>* pkg,
               std::vector<double>* mag) const override {
    const int d = dir / 2, nf = n * n;
    const bool upper = dir % 2;
    const int slice = upper ? n - 1 : 0;
    const double* ue = u + e * kVarsA * np;
    std::vector<double> psi(nf), pi(nf), phi(3 * nf), g2(nf, gamma2), nrm(3 * nf, 0.0);
    mag->assign(nf, invjac[3 * e + d]);
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        const int f = a + n * b;
        const int64_t v = face_volume_index(n, d, slice, a, b);
        psi[f] = ue[v];
        pi[f] = ue[np + v];
        for (int i = 0; i < 3; ++i) phi[i * nf + f] = ue[(2 + i) * np + v];
        nrm[d * nf + f] = upper ? 1.0 : -1.0;
      }
    pkg->assign((size_t)16 * nf, 0.0);
    double ms;
    orc_package(nf, psi.data(), pi.data(), phi.data(), g2.data(), nrm.data(), nullptr, pkg->data(),
                &ms);
  }
  void exterior_package(const double* u, int64_t e, int dir,
                        std::vector<double>* pkg) const override {
    std::vector<double> mag;
    package(u, nbr[6 * e + dir], dir ^ 1, pkg, &mag);  // aligned bricks: same point order
  }
  void boundary_terms(const std::vector<double>& pi, const std::vector<double>& pe,
                      double* out) const override {
    orc_boundary_terms(n * n, pi.data(), pe.data(), out);
  }
};

// M (rows x cols, row-major) applied along both axes of nfields face blocks
// of cols^2 values: out[f][ip + rows bp] = sum M[ip][i] M[bp][b] in[f][i + cols b]
void face_matrix(int rows, int cols, const double* M, int nfields, const double* in, double* out) {
  std::vector<double> tmp((size_t)rows * cols);
  for (int f = 0; f < nfields; ++f) {
    const double* src = in + (size_t)f * cols * cols;
    double* dst = out + (size_t)f * rows * rows;
    for (int b = 0; b < cols; ++b)
      for (int ip = 0; ip < rows; ++ip) {
        double s = 0.0;
        for (int i = 0; i < cols; ++i) s += M[ip * cols + i] * src[i + cols * b];
        tmp[ip + (size_t)rows * b] = s;
      }
    for (int bp = 0; bp < rows; ++bp)
      for (int ip = 0; ip < rows; ++ip) {
        double s = 0.0;
        for (int b = 0; b < cols; ++b) s += M[bp * cols + b] * tmp[ip + (size_t)rows * b];
        dst[ip + (size_t)rows * bp] = s;
      }
  }
}

// Flat scalar wave on conforming periodic bricks whose elements have their own
// LGL extents (p-nonconforming faces).  The mortar of a face has the larger of
// the two extents (mortar_mesh, MortarHelpers.cpp:21-47); each side's package
// is interpolated onto it where it is finer than the face
// (projection_matrix_parent_to_child, Projection.cpp:310-330), and the
// corrections come back by Legendre truncation (projection_matrix_child_to_
// parent, Projection.cpp:97-130), as ApplyBoundaryCorrections.hpp:880-937
// does for every (local, remote) record pair.
struct MixedFlatSystem : System {
  int n_inst = 0;
  const OrcBrick* br = nullptr;
  double gamma2 = 0.0;
  int threads = 0;
  std::vector<int32_t> elem_n, nbr, inst;
  std::vector<int64_t> off;     // n_elem + 1 block offsets
  std::vector<double> invjac;  // 3 per element

  int n_of(int64_t e) const override { return elem_n[e]; }
  int64_t offset_of(int64_t e) const override { return off[e]; }
  int64_t total_values() const override { return off[E]; }
  int64_t neighbor(int64_t e, int dir) const override { return nbr[6 * e + dir]; }
  int back_dir(int64_t, int dir) const override { return dir ^ 1; }
  void volume_rhs(const double* u, double* dudt) override {
    orc_volume_rhs(n_inst, br, elem_n.data(), gamma2, u, dudt, threads);
  }
  int mortar_n(int64_t e, int dir) const override {
    return std::max(elem_n[e], elem_n[nbr[6 * e + dir]]);
  }
  // dg_package_data on e's own face points
  void face_package(const double* u, int64_t e, int dir, std::vector<double>* pkg,
                    std::vector<double>* mag) const {
    const int ne = elem_n[e], d = dir / 2, nf = ne * ne;
    const int64_t np_e = (int64_t)nf * ne;
    const bool upper = dir % 2;
    const int slice = upper ? ne - 1 : 0;
    const double* ue = u + off[e];
    std::vector<double> psi(nf), pi(nf), phi(3 * nf), g2(nf, gamma2), nrm(3 * nf, 0.0);
    mag->assign(nf, invjac[3 * e + d]);
    for (int b = 0; b < ne; ++b)
      for (int a = 0; a < ne; ++a) {
        const int f = a + ne * b;
        const int64_t v = face_volume_index(ne, d, slice, a, b);
        psi[f] = ue[v];
        pi[f] = ue[np_e + v];
        for (int i = 0; i < 3; ++i) phi[i * nf + f] = ue[(2 + i) * np_e + v];
        nrm[d * nf + f] = upper ? 1.0 : -1.0;
      }
    pkg->assign((size_t)16 * nf, 0.0);
    double ms;
    orc_package(nf, psi.data(), pi.data(), phi.data(), g2.data(), nrm.data(), nullptr, pkg->data(),
                &ms);
  }
  // a face package of extent nf_n onto the mortar of extent nm
  static void to_mortar(int nf_n, int nm, const std::vector<double>& f, std::vector<double>* out) {
    if (nm == nf_n) {
      *out = f;
      return;
    }
    std::vector<double> P((size_t)nm * nf_n);
    orc_proj_face_to_mortar(nf_n, nm, P.data());
    out->assign((size_t)16 * nm * nm, 0.0);
    face_matrix(nm, nf_n, P.data(), 16, f.data(), out->data());
  }
  void package(const double* u, int64_t e, int dir, std::vector<double>* pkg,
               std::vector<double>* mag) const override {
    std::vector<double> f;
    face_package(u, e, dir, &f, mag);
    to_mortar(elem_n[e], mortar_n(e, dir), f, pkg);
  }
  void exterior_package(const double* u, int64_t e, int dir,
                        std::vector<double>* pkg) const override {
    // aligned bricks: the neighbour's face points run in e's order
    const int64_t nb = nbr[6 * e + dir];
    std::vector<double> f, mag;
    face_package(u, nb, dir ^ 1, &f, &mag);
    to_mortar(elem_n[nb], mortar_n(e, dir), f, pkg);
  }
  void boundary_terms(const std::vector<double>& pi, const std::vector<double>& pe,
                      double* out) const override {
    orc_boundary_terms((int)(pi.size() / 16), pi.data(), pe.data(), out);
  }
  void mortar_to_face(int64_t e, int dir, const double* on_mortar, double* on_face) const override {
    const int ne = elem_n[e], nm = mortar_n(e, dir);
    if (nm == ne) {
      std::copy(on_mortar, on_mortar + (size_t)kVarsA * ne * ne, on_face);
      return;
    }
    std::vector<double> R((size_t)ne * nm);
    orc_proj_mortar_to_face(ne, nm, R.data());
    face_matrix(ne, nm, R.data(), kVarsA, on_mortar, on_face);
  }
};

}  // namespace

int lts_evolve(System& sys, int order, const int32_t* levels, double slab, int n_slabs, double* u) {
  if (order < 1 || order > kMaxOrder || !(slab > 0.0) || n_slabs < 0 || !u) return -1;
  Run R(sys);
  int L = 0;
  for (int64_t e = 0; e < sys.E; ++e) {
    const int l = levels ? levels[e] : 0;
    if (l < 0 || l > 6) return -1;
    L = std::max(L, l);
  }
  // ticks: a slab of order * 2^L ticks; the first real steps are
  // slab / 2^L = order ticks, the self-start steps one tick
  // (SelfStartActions.hpp:196-216: initial step / (values_needed + 1))
  const int64_t S = (int64_t)order << L;
  const int64_t first_step = S >> L;
  // levels keep the first step until the slab boundary after which no
  // self-start value is left in any history; there they take slab / 2^level
  const int64_t switch_tick = (((int64_t)order - 1 + ((int64_t)1 << L) - 1) >> L) * S;
  auto step_of = [&](int64_t e, int64_t t) -> int64_t {
    return t < switch_tick ? first_step : (S >> (levels ? levels[e] : 0));
  };
  R.clk = Clock{slab, S, 0.0};
  const int64_t total = sys.total_values();
  std::vector<double> u0(u, u + total);
  std::vector<int64_t> all(sys.E);
  for (int64_t e = 0; e < sys.E; ++e) all[e] = e;
  int rc = 0;
  // self-start (SelfStartActions.hpp:471-482): for each order o < k, reset to
  // the initial values, take o steps of one tick at order o from the slab
  // start, and record one more (unused) value at tick o with order o + 1
  for (int o = 1; o < order; ++o) {
    const int64_t sn = -(int64_t)(order - o);
    for (int j = 0; j <= o; ++j) {
      if (j >= 1)
        for (int64_t e : all) {
          if ((rc = R.boundary_delta(u, e, j - 1, j))) return rc;
          R.clean(e);
          sys.filter_element(u, e);
        }
      if (j == 0) std::copy(u0.begin(), u0.end(), u);
      R.record(u, all, Id{sn, j}, j < o ? o : o + 1);
      for (int64_t e : all) {
        if (j < o) {
          if ((rc = R.volume_update(u, e, j, j + 1))) return rc;
        } else {
          R.clean(e);  // the step is unused (SelfStart::step_unused)
        }
      }
    }
  }
  if (order > 1) std::copy(u0.begin(), u0.end(), u);
  R.record(u, all, Id{0, 0}, order);
  for (int64_t e : all) {
    R.el[e].start = 0;
    R.el[e].end = step_of(e, 0);
    if ((rc = R.volume_update(u, e, 0, R.el[e].end))) return rc;
  }
  const int64_t final_tick = (int64_t)n_slabs * S;
  for (int64_t P = 1; P <= final_tick; ++P) {
    std::vector<int64_t> fin;
    for (int64_t e : all)
      if (R.el[e].end == P) fin.push_back(e);
    if (fin.empty()) continue;
    for (int64_t e : fin) {
      if ((rc = R.boundary_delta(u, e, R.el[e].start, P))) return rc;
      R.clean(e);
      sys.filter_element(u, e);
    }
    if (P == final_tick) break;
    R.record(u, fin, Id{P / S, P}, order);
    for (int64_t e : fin) {
      R.el[e].start = P;
      R.el[e].end = P + step_of(e, P);
      if ((rc = R.volume_update(u, e, P, R.el[e].end))) return rc;
    }
  }
  return 0;
}

}  // namespace orc_adams

extern "C" {


int orc_variable_coefficients(int n, const double* control_times, double step_start,
                              double step_end, double* out) {
  if (n < 0 || n > kMaxOrder || (n > 0 && (!control_times || !out))) return -1;
  const std::vector<double> c =
      variable_coefficients(std::vector<double>(control_times, control_times + n), step_start,
                            step_end);
  std::copy(c.begin(), c.end(), out);
  return 0;
}

int orc_adams_coefficients(int n, const int64_t* control_ticks, int64_t step_start,
                           int64_t step_end, double slab, int64_t ticks_per_slab, double* out) {
  if (n < 0 || n > kMaxOrder || ticks_per_slab < 1 || (n > 0 && (!control_ticks || !out)))
    return -1;
  const Clock clk{slab, ticks_per_slab, 0.0};
  const std::vector<double> c =
      coefficients(std::vector<int64_t>(control_ticks, control_ticks + n), step_start, step_end,
                   clk);
  std::copy(c.begin(), c.end(), out);
  return 0;
}

int orc_lts_coefficients(int n_local, const int64_t* local_slab, const int64_t* local_tick,
                         int n_remote, const int64_t* remote_slab, const int64_t* remote_tick,
                         int64_t step_start, int64_t step_end, double slab, int64_t ticks_per_slab,
                         int local_order, int remote_order, int small_order, int max_out,
                         int32_t* out_local, int32_t* out_remote, double* out_coef) {
  for (int o : {local_order, remote_order, small_order})
    if (o < 1 || o > kMaxOrder) return -1;
  if (n_local < 0 || n_remote < 0 || ticks_per_slab < 1 || max_out < 0) return -1;
  std::vector<Id> l(n_local), r(n_remote);
  for (int i = 0; i < n_local; ++i) l[i] = {local_slab[i], local_tick[i]};
  for (int i = 0; i < n_remote; ++i) r[i] = {remote_slab[i], remote_tick[i]};
  std::vector<Term> terms;
  const int rc = lts_coefficients(l, r, step_start, step_end, local_order, remote_order,
                                  small_order, Clock{slab, ticks_per_slab, 0.0}, &terms);
  if (rc) return -2;
  if ((int)terms.size() > max_out) return -3;
  for (size_t i = 0; i < terms.size(); ++i) {
    out_local[i] = terms[i].local;
    out_remote[i] = terms[i].remote;
    out_coef[i] = terms[i].coef;
  }
  return (int)terms.size();
}

int orc_evolve_adams(int n_inst, const OrcBrick* br, int n, double gamma2, int order,
                     const int32_t* levels, double slab, int n_slabs, double* u, int n_threads) {
  if (n_inst < 1 || !br || n < 2 || n > 20) return -1;
  orc_adams::FlatSystem sys;
  sys.n_inst = n_inst;
  sys.br = br;
  sys.n = n;
  sys.E = orc_num_elements(n_inst, br);
  sys.np = (int64_t)n * n * n;
  sys.gamma2 = gamma2;
  sys.threads = n_threads;
  sys.elem_n.assign(sys.E, n);
  sys.nbr.resize(6 * sys.E);
  sys.inst.resize(sys.E);
  std::vector<uint64_t> ids(sys.E);
  std::vector<int32_t> ijk(3 * sys.E);
  const int mrc = orc_index_maps(n_inst, br, ids.data(), sys.nbr.data(), ijk.data(), sys.inst.data());
  if (mrc != 0 && mrc != -2) return -1;
  sys.invjac.resize(3 * sys.E);
  for (int64_t e = 0; e < sys.E; ++e)
    for (int d = 0; d < 3; ++d) {
      const OrcBrick& b = br[sys.inst[e]];
      sys.invjac[3 * e + d] = 2.0 / ((b.hi[d] - b.lo[d]) / b.n[d]);
    }
  return orc_adams::lts_evolve(sys, order, levels, slab, n_slabs, u);
}

int orc_evolve_adams_extents(int n_inst, const OrcBrick* br, const int32_t* elem_n, double gamma2,
                             int order, const int32_t* levels, double slab, int n_slabs, double* u,
                             int n_threads) {
  if (n_inst < 1 || !br || !elem_n) return -1;
  orc_adams::MixedFlatSystem sys;
  sys.n_inst = n_inst;
  sys.br = br;
  sys.E = orc_num_elements(n_inst, br);
  sys.gamma2 = gamma2;
  sys.threads = n_threads;
  sys.elem_n.assign(elem_n, elem_n + sys.E);
  sys.off.assign(sys.E + 1, 0);
  for (int64_t e = 0; e < sys.E; ++e) {
    const int ne = sys.elem_n[e];
    if (ne < 2 || ne > 20) return -1;
    sys.off[e + 1] = sys.off[e] + (int64_t)5 * ne * ne * ne;
  }
  sys.n = sys.elem_n[0];
  sys.np = (int64_t)sys.n * sys.n * sys.n;
  sys.nbr.resize(6 * sys.E);
  sys.inst.resize(sys.E);
  std::vector<uint64_t> ids(sys.E);
  std::vector<int32_t> ijk(3 * sys.E);
  const int mrc = orc_index_maps(n_inst, br, ids.data(), sys.nbr.data(), ijk.data(), sys.inst.data());
  if (mrc != 0 && mrc != -2) return -1;
  sys.invjac.resize(3 * sys.E);
  for (int64_t e = 0; e < sys.E; ++e)
    for (int d = 0; d < 3; ++d) {
      const OrcBrick& b = br[sys.inst[e]];
      sys.invjac[3 * e + d] = 2.0 / ((b.hi[d] - b.lo[d]) / b.n[d]);
    }
  return orc_adams::lts_evolve(sys, order, levels, slab, n_slabs, u);
}

}  // extern "C"
