// refined_setup.cpp -- host-side maps of a periodic block lattice whose
// blocks carry different refinement levels (h-nonconforming 2:1 faces), and
// the half-interval mortar projections.
//
// Elements are numbered block by block (blocks x fastest), then x-outer /
// z-inner segments inside a block (InitialElementIds.cpp:45-96).  A face
// between blocks of levels L and L+1 joins one coarse element to four fine
// ones: the coarse side has four mortars, each a LowerHalf / UpperHalf in the
// two transverse dimensions, and each fine side one Full mortar
// (mortar_size, MortarHelpers.cpp:49-75).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "host_setup.hpp"

namespace dgsw {
namespace {
// P_k(x) by the three-term recurrence
double legendre_p(int k, double x) {
  double a = 1.0, b = x;
  if (k == 0) return a;
  for (int m = 2; m <= k; ++m) {
    const double c = ((2.0 * m - 1.0) * x * b - (m - 1.0) * a) / m;
    a = b;
    b = c;
  }
  return b;
}
}  // namespace

bool half_projections(int n, int upper, double* P, double* R) {
  if (n < 2 || n > kMaxN) return false;
  double x[kMaxN], w[kMaxN];
  lgl_nodes_weights(n, x, w);
  const double shift = upper ? 1.0 : -1.0;
  if (P) {
    // parent -> child: interpolation to the half (Projection.cpp:341-372)
    double t[kMaxN];
    for (int i = 0; i < n; ++i) t[i] = 0.5 * (x[i] + shift);
    lgl_interp_matrix(n, n, t, P);
  }
  if (R) {
    // child -> parent: the parent's Legendre coefficients of the
    // half-supported child polynomial, c_k = (2k+1)/4 int P_k(x(xi)) g(xi) dxi
    // (the integral Projection.cpp:140-220 evaluates in closed form), here by
    // an n+1 point Gauss rule, exact for the degree 2n-2 integrands.  The
    // child's modal coefficients come from the discrete Legendre norms of the
    // LGL rule (V^-1 = diag(1/g) V^T W, exact on LGL nodes).
    GaussTables gq;
    lg_spectral(n + 1, &gq);
    double V[kMaxN * kMaxN], Vinv[kMaxN * kMaxN], S[kMaxN * kMaxN];
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k) V[i * n + k] = legendre_p(k, x[i]);
    for (int k = 0; k < n; ++k) {
      double g = 0.0;
      for (int i = 0; i < n; ++i) g += w[i] * V[i * n + k] * V[i * n + k];
      for (int j = 0; j < n; ++j) Vinv[k * n + j] = V[j * n + k] * w[j] / g;
    }
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j) {
        double acc = 0.0;
        for (int q = 0; q <= n; ++q)
          acc += gq.w[q] * legendre_p(k, 0.5 * (gq.x[q] + shift)) * legendre_p(j, gq.x[q]);
        S[k * n + j] = (2.0 * k + 1.0) * 0.25 * acc;
      }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double acc = 0.0;
        for (int k = 0; k < n; ++k) {
          double sv = 0.0;
          for (int l = 0; l < n; ++l) sv += S[k * n + l] * Vinv[l * n + j];
          acc += V[i * n + k] * sv;
        }
        R[i * n + j] = acc;
      }
  }
  return true;
}

bool build_refined_domain(const DgswConfig& cfg, Domain* dom, RefinedMaps* rm,
                          std::string* err) {
  const DgswRefinedBrick* b = cfg.refined;
  if (!b || !b->levels) {
    *err = "refined lattice without levels";
    return false;
  }
  if (cfg.system != DGSW_SYSTEM_SCALAR_WAVE_3D || cfg.quadrature != DGSW_QUADRATURE_GAUSS_LOBATTO ||
      cfg.precision != DGSW_PRECISION_FP64 || cfg.points_per_element ||
      cfg.boundary_correction != DGSW_CORRECTION_UPWIND_PENALTY ||
      cfg.time_stepper != DGSW_STEPPER_RK3_HESTHAVEN_SSP) {
    *err = "refined lattices: flat system, Gauss-Lobatto, one extent, FP64, UpwindPenalty, SSP-RK3";
    return false;
  }
  const int n = cfg.uniform_points;
  if (n < kMinN || n > kMaxN || !std::isfinite(cfg.gamma2)) {
    *err = "points per dimension must be in [2, 12] and gamma2 finite";
    return false;
  }
  const int bx = b->blocks[0], by = b->blocks[1], bz = b->blocks[2];
  if (bx < 1 || by < 1 || bz < 1 || (int64_t)bx * by * bz > 255) {
    *err = "need 1 to 255 blocks";
    return false;
  }
  for (int d = 0; d < 3; ++d)
    if (!(b->upper[d] > b->lower[d]) || !std::isfinite(b->upper[d]) || !std::isfinite(b->lower[d])) {
      *err = "lattice bounds must satisfy lower < upper";
      return false;
    }
  const int nb = bx * by * bz;
  std::vector<int64_t> first(nb + 1, 0);
  for (int k = 0; k < nb; ++k) {
    const int L = b->levels[k];
    if (L < 0 || L > 6) {
      *err = "block levels must be in [0, 6]";
      return false;
    }
    first[k + 1] = first[k] + ((int64_t)1 << (3 * L));
  }
  const int64_t E = first[nb];
  const int64_t np = (int64_t)n * n * n;
  dom->bricks.clear();
  dom->layout.clear();
  dom->n_elem = E;
  dom->elem_n.assign(E, n);
  dom->uniform = true;
  dom->max_n = n;
  dom->block_ids_fit = true;
  dom->offset.resize(E + 1);
  for (int64_t e = 0; e <= E; ++e) dom->offset[e] = e * kVars * np;
  dom->n_points = E * np;
  dom->instance.assign(E, 0);
  dom->lower.resize(3 * E);
  dom->width.resize(3 * E);
  dom->element_id.resize(E);
  dom->neighbor.assign(6 * E, 0);
  rm->level.resize(E);
  rm->slots.assign(24 * E, -1);
  rm->sizes.assign(48 * E, 0);
  rm->face_index.assign(6 * E, -1);
  rm->faces.clear();
  std::vector<int> seg(3 * E), blk(E);
  auto block_of = [&](const int q[3]) { return q[0] + bx * (q[1] + by * q[2]); };
  auto elem_of = [&](int k, const int s[3]) {
    const int L = b->levels[k];
    return first[k] + (((int64_t)s[0] << (2 * L)) | ((int64_t)s[1] << L) | s[2]);
  };
  for (int k = 0; k < nb; ++k) {
    const int L = b->levels[k];
    const int q[3] = {k % bx, (k / bx) % by, k / (bx * by)};
    for (int64_t wi = 0; wi < ((int64_t)1 << (3 * L)); ++wi) {
      const int64_t e = first[k] + wi;
      int* s = &seg[3 * e];
      s[2] = (int)(wi & ((1 << L) - 1));
      s[1] = (int)((wi >> L) & ((1 << L) - 1));
      s[0] = (int)(wi >> (2 * L));
      blk[e] = k;
      rm->level[e] = L;
      const int cnt[3] = {bx, by, bz};
      for (int d = 0; d < 3; ++d) {
        const double W = (b->upper[d] - b->lower[d]) / cnt[d];
        dom->width[3 * e + d] = W / (1 << L);
        dom->lower[3 * e + d] = b->lower[d] + W * q[d] + dom->width[3 * e + d] * s[d];
      }
      dom->element_id[e] = (uint64_t)k | ((uint64_t)s[0] << 16) | ((uint64_t)L << 28) |
                           ((uint64_t)s[1] << 32) | ((uint64_t)L << 44) |
                           ((uint64_t)s[2] << 48) | ((uint64_t)L << 60);
    }
  }
  const int cnt[3] = {bx, by, bz};
  for (int64_t e = 0; e < E; ++e) {
    const int* s = &seg[3 * e];
    const int L = rm->level[e];
    const int k = blk[e];
    const int q[3] = {k % bx, (k / bx) % by, k / (bx * by)};
    for (int dir = 0; dir < 6; ++dir) {
      const int d = dir >> 1;
      const bool up = dir & 1;
      const int t0 = d == 0 ? 1 : 0, t1 = d == 2 ? 1 : 2;  // transverse, ascending
      int32_t* slot = &rm->slots[(6 * e + dir) * 4];
      int32_t* size = &rm->sizes[(6 * e + dir) * 8];
      const int last = (1 << L) - 1;
      if ((up && s[d] < last) || (!up && s[d] > 0)) {
        int sg[3] = {s[0], s[1], s[2]};
        sg[d] += up ? 1 : -1;
        slot[0] = (int32_t)elem_of(k, sg);
        dom->neighbor[6 * e + dir] = slot[0];
        continue;
      }
      int q2[3] = {q[0], q[1], q[2]};
      q2[d] = (q2[d] + (up ? 1 : cnt[d] - 1)) % cnt[d];
      const int k2 = block_of(q2);
      const int L2 = b->levels[k2];
      int sg[3] = {0, 0, 0};
      sg[d] = up ? 0 : (1 << L2) - 1;
      if (L2 == L) {
        sg[t0] = s[t0];
        sg[t1] = s[t1];
        slot[0] = (int32_t)elem_of(k2, sg);
      } else if (L2 == L + 1) {
        RefinedFace f{};
        f.element = (int32_t)e;
        f.dir = dir;
        f.coarse = 1;
        for (int c = 0; c < 4; ++c) {
          sg[t0] = 2 * s[t0] + (c & 1);
          sg[t1] = 2 * s[t1] + (c >> 1);
          slot[c] = (int32_t)elem_of(k2, sg);
          size[2 * c] = 1 + (c & 1);
          size[2 * c + 1] = 1 + (c >> 1);
          f.nb[c] = slot[c];
        }
        rm->face_index[6 * e + dir] = (int32_t)rm->faces.size();
        rm->faces.push_back(f);
      } else if (L2 == L - 1) {
        sg[t0] = s[t0] >> 1;
        sg[t1] = s[t1] >> 1;
        slot[0] = (int32_t)elem_of(k2, sg);
        RefinedFace f{};
        f.element = (int32_t)e;
        f.dir = dir;
        f.coarse = 0;
        f.nb[0] = slot[0];
        f.nb[1] = f.nb[2] = f.nb[3] = -1;
        f.child[0] = s[t0] & 1;
        f.child[1] = s[t1] & 1;
        rm->face_index[6 * e + dir] = (int32_t)rm->faces.size();
        rm->faces.push_back(f);
      } else {
        *err = "neighbouring blocks differ by more than one refinement level";
        return false;
      }
      dom->neighbor[6 * e + dir] = slot[0];
    }
  }
  return true;
}

}  // namespace dgsw
