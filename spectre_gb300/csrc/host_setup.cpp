// host_setup.cpp -- host-side spectral tables and domain index maps.
#include "host_setup.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace dgsw {
namespace {

// Legendre P_p(x) and P_{p+1}(x), P_{p-1}(x) by the three-term recurrence.
void legendre_triple(int p, double x, double* pm1, double* pp, double* pp1) {
  double a = 1.0, b = x;  // P_0, P_1
  if (p == 0) {
    *pm1 = 0.0;
    *pp = 1.0;
    *pp1 = x;
    return;
  }
  for (int k = 2; k <= p + 1; ++k) {
    const double c = ((2.0 * k - 1.0) * x * b - (k - 1.0) * a) / k;
    a = b;
    b = c;
  }
  // after the loop: a = P_p, b = P_{p+1}; recover P_{p-1} from the recurrence
  *pp = a;
  *pp1 = b;
  // (p+1) P_{p+1} = (2p+1) x P_p - p P_{p-1}
  *pm1 = ((2.0 * p + 1.0) * x * a - (p + 1.0) * b) / p;
}

double legendre(int k, double x) {
  if (k == 0) return 1.0;
  double a = 1.0, b = x;
  for (int j = 2; j <= k; ++j) {
    const double c = ((2.0 * j - 1.0) * x * b - (j - 1.0) * a) / j;
    a = b;
    b = c;
  }
  return b;
}

void split_count(int n, int* blocks, int* level) {
  int L = 0;
  while (n > 0 && (n & 1) == 0) {
    n >>= 1;
    ++L;
  }
  *blocks = n;
  *level = L;
}

}  // namespace

bool lgl_nodes_weights(int n, double* x, double* w) {
  if (n < 2 || n > 20 || !x || !w) return false;
  const int p = n - 1;
  x[0] = -1.0;
  x[p] = 1.0;
  w[0] = w[p] = 2.0 / (p * (p + 1.0));
  for (int j = 1; j <= p / 2; ++j) {
    // interior roots of q = P_{p+1} - P_{p-1}, symmetric about 0
    double r = -std::cos(M_PI * j / p);  // Chebyshev-Gauss-Lobatto guess
    if (2 * j == p) r = 0.0;
    for (int it = 0; it < 100; ++it) {
      double pm1, pp, pp1;
      legendre_triple(p, r, &pm1, &pp, &pp1);
      const double q = pp1 - pm1;
      const double dq = (2.0 * p + 1.0) * pp;
      const double dr = q / dq;
      r -= dr;
      if (std::abs(dr) <= 1e-17) break;
    }
    if (2 * j == p) r = 0.0;
    double pm1, pp, pp1;
    legendre_triple(p, r, &pm1, &pp, &pp1);
    x[j] = r;
    x[p - j] = -r;
    w[j] = w[p - j] = 2.0 / (p * (p + 1.0) * pp * pp);
  }
  return true;
}

static bool barycentric(int n, const double* x, double* bw) {
  for (int j = 0; j < n; ++j) {
    double prod = 1.0;
    for (int k = 0; k < n; ++k)
      if (k != j) prod *= x[j] - x[k];
    bw[j] = 1.0 / prod;
  }
  return true;
}

bool lgl_diff_matrix(int n, double* D) {
  double x[20], w[20], bw[20];
  if (!D || !lgl_nodes_weights(n, x, w)) return false;
  barycentric(n, x, bw);
  for (int i = 0; i < n; ++i) {
    double diag = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      D[i * n + j] = bw[j] / (bw[i] * (x[i] - x[j]));
      diag -= D[i * n + j];
    }
    D[i * n + i] = diag;
  }
  return true;
}

bool lgl_interp_matrix(int n, int m, const double* t, double* M) {
  double x[20], w[20], bw[20];
  if (!M || m < 0 || (m > 0 && !t) || !lgl_nodes_weights(n, x, w)) return false;
  barycentric(n, x, bw);
  const double eps = 100.0 * 2.220446049250313e-16;
  for (int k = 0; k < m; ++k) {
    int hit = -1;
    for (int j = 0; j < n; ++j) {
      const double scale = std::max(std::max(std::abs(t[k]), std::abs(x[j])), 1.0);
      if (std::abs(t[k] - x[j]) <= eps * scale) hit = j;
    }
    if (hit >= 0) {
      for (int j = 0; j < n; ++j) M[k * n + j] = (j == hit) ? 1.0 : 0.0;
      continue;
    }
    double sum = 0.0;
    for (int j = 0; j < n; ++j) {
      M[k * n + j] = bw[j] / (t[k] - x[j]);
      sum += M[k * n + j];
    }
    for (int j = 0; j < n; ++j) M[k * n + j] /= sum;
  }
  return true;
}

bool lgl_mortar_projections(int ne, int nm, double* to_mortar, double* from_mortar) {
  if (ne < 2 || nm < ne || nm > 20) return false;
  double xm[20], wm[20], xe[20], we[20];
  lgl_nodes_weights(nm, xm, wm);
  lgl_nodes_weights(ne, xe, we);
  if (to_mortar && !lgl_interp_matrix(ne, nm, xm, to_mortar)) return false;
  if (from_mortar) {
    // Modal coefficients on the mortar by LGL discrete orthogonality:
    //   c_k = sum_j w_j P_k(x_j) u_j / g_k,  g_k = 2/(2k+1) for k < nm-1 and
    //   g_{nm-1} = 2/(nm-1) (the LGL rule's norm of the top mode), which is
    // the exact inverse of the mortar Vandermonde matrix.  Keeping the
    // first ne modes and evaluating at the face points gives the L2
    // restriction.
    for (int i = 0; i < ne; ++i)
      for (int j = 0; j < nm; ++j) {
        double s = 0.0;
        for (int k = 0; k < ne; ++k) {
          const double g = (k < nm - 1) ? 2.0 / (2.0 * k + 1.0) : 2.0 / (nm - 1.0);
          s += legendre(k, xe[i]) * (wm[j] * legendre(k, xm[j]) / g);
        }
        from_mortar[i * nm + j] = s;
      }
  }
  return true;
}

static bool eo_from_matrix(int n, const double* D, EoTable* t) {
  std::memset(t, 0, sizeof(*t));
  const int h = n / 2, H = (n + 1) / 2;
  for (int i = 0; i < H; ++i) {
    for (int j = 0; j < h; ++j) {
      t->A[i][j] = 0.5 * (D[i * n + j] + D[i * n + (n - 1 - j)]);
      t->B[i][j] = 0.5 * (D[i * n + j] - D[i * n + (n - 1 - j)]);
    }
    t->M[i] = (n % 2) ? D[i * n + h] : 0.0;
  }
  if (n % 2) {
    // middle row: exactly antisymmetric, so its even part vanishes
    for (int j = 0; j < h; ++j) t->A[h][j] = 0.0;
    t->M[h] = 0.0;
  }
  return true;
}

bool lg_spectral(int n, GaussTables* g) {
  if (n < 2 || n > 20 || !g) return false;
  g->n = n;
  // nodes: roots of P_n by Newton from the Chebyshev-Gauss guess, weights
  // 2 / ((1 - x^2) P_n'(x)^2) (Legendre.cpp:106-149, Kopriva algorithm 23)
  for (int j = 0; j < (n + 1) / 2; ++j) {
    double r = -std::cos((2.0 * j + 1.0) * M_PI / (2.0 * n));
    if (2 * j + 1 == n) r = 0.0;
    double dP = 0.0;
    for (int it = 0; it < 100; ++it) {
      double pm1, p, pp1;
      legendre_triple(n - 1, r, &pm1, &p, &pp1);  // P_{n-2}, P_{n-1}, P_n
      dP = n * (r * pp1 - p) / (r * r - 1.0);
      const double dr = pp1 / dP;
      r -= dr;
      if (std::abs(dr) <= 1e-17) break;
    }
    if (2 * j + 1 == n) r = 0.0;
    double pm1, p, pp1;
    legendre_triple(n - 1, r, &pm1, &p, &pp1);
    dP = n * (r * pp1 - p) / (r * r - 1.0);
    g->x[j] = r;
    g->x[n - 1 - j] = -r;
    g->w[j] = g->w[n - 1 - j] = 2.0 / ((1.0 - r * r) * dP * dP);
  }
  double bw[20];
  barycentric(n, g->x, bw);
  for (int i = 0; i < n; ++i) {
    double diag = 0.0;
    for (int j = 0; j < n; ++j)
      if (j != i) {
        g->D[i * n + j] = bw[j] / (bw[i] * (g->x[i] - g->x[j]));
        diag -= g->D[i * n + j];
      }
    g->D[i * n + i] = diag;
  }
  for (int side = 0; side < 2; ++side) {
    const double t = side ? 1.0 : -1.0;
    double* row = side ? g->hi : g->lo;
    double sum = 0.0;
    for (int j = 0; j < n; ++j) {
      row[j] = bw[j] / (t - g->x[j]);
      sum += row[j];
    }
    for (int j = 0; j < n; ++j) row[j] /= sum;
  }
  for (int j = 0; j < n; ++j) {
    g->lift_lo[j] = g->lo[j] / g->w[j];
    g->lift_hi[j] = g->hi[j] / g->w[j];
  }
  return true;
}

bool lg_eo_table(int n, EoTable* t) {
  GaussTables g;
  if (n < kMinN || n > kMaxN || !lg_spectral(n, &g)) return false;
  return eo_from_matrix(n, g.D, t);
}

bool lgl_exponential_filter(int n, double alpha, int half_power, double* F) {
  if (n < 2 || n > 20 || !F || half_power < 0 || !std::isfinite(alpha)) return false;
  double x[20], w[20];
  lgl_nodes_weights(n, x, w);
  // nodal -> modal through the discrete Legendre norms of the LGL rule:
  // V^T W V = diag(g) exactly (P_{n-1}^2 is the only product above the rule's
  // degree, and it sits on the diagonal), so V^-1 = diag(1/g) V^T W
  double V[20 * 20], g[20], d[20];
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) V[i * n + k] = legendre(k, x[i]);
  const double order = n - 1.0;
  for (int k = 0; k < n; ++k) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += w[i] * V[i * n + k] * V[i * n + k];
    g[k] = s;
    d[k] = std::exp(-alpha * std::pow(k / order, 2.0 * half_power));
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += V[i * n + k] * (d[k] / g[k]) * V[j * n + k];
      F[i * n + j] = s * w[j];
    }
  return true;
}

bool lgl_eo_table(int n, EoTable* t) {
  if (n < kMinN || n > kMaxN || !t) return false;
  double D[kMaxN * kMaxN];
  lgl_diff_matrix(n, D);
  return eo_from_matrix(n, D, t);
}

bool lgl_eo_table_transposed(int n, EoTable* t) {
  if (n < kMinN || n > kMaxN || !t) return false;
  double D[kMaxN * kMaxN], Dt[kMaxN * kMaxN];
  lgl_diff_matrix(n, D);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Dt[i * n + j] = D[j * n + i];
  return eo_from_matrix(n, Dt, t);
}

bool sample_weights(const Domain& dom, int n, int n_samples, const double* xyz,
                    int64_t* elem_off, double* weights) {
  if (dom.bricks.size() != 1 || !dom.uniform) return false;
  const DgswBrick& b = dom.bricks[0];
  const BrickLayout& L = dom.layout[0];
  const int64_t per_block = (int64_t)1 << (L.level[0] + L.level[1] + L.level[2]);
  for (int s = 0; s < n_samples; ++s) {
    int q[3];
    double xi[3];
    for (int d = 0; d < 3; ++d) {
      const double x = xyz[3 * s + d];
      if (!(x >= b.lower[d] && x <= b.upper[d])) return false;
      const double h = (b.upper[d] - b.lower[d]) / b.elements[d];
      int k = (int)std::floor((x - b.lower[d]) / h);
      if (k >= b.elements[d]) k = b.elements[d] - 1;
      if (k < 0) k = 0;
      q[d] = k;
      xi[d] = 2.0 * (x - (b.lower[d] + h * k)) / h - 1.0;
    }
    int64_t blk[3], seg[3];
    for (int d = 0; d < 3; ++d) {
      blk[d] = q[d] >> L.level[d];
      seg[d] = q[d] & ((1 << L.level[d]) - 1);
    }
    const int64_t bid = blk[0] + L.blocks[0] * (blk[1] + (int64_t)L.blocks[1] * blk[2]);
    const int64_t e = bid * per_block + ((seg[0] << (L.level[1] + L.level[2])) |
                                        (seg[1] << L.level[2]) | seg[2]);
    elem_off[s] = dom.offset[e];
    for (int d = 0; d < 3; ++d)
      if (!lgl_interp_matrix(n, 1, &xi[d], weights + (size_t)s * 3 * n + d * n)) return false;
  }
  return true;
}

bool build_domain(const DgswConfig& cfg, Domain* dom, std::string* err) {
  if (cfg.system != DGSW_SYSTEM_SCALAR_WAVE_3D) {
    *err = "unsupported system";
    return false;
  }
  if (cfg.boundary_correction != DGSW_CORRECTION_UPWIND_PENALTY) {
    *err = "unsupported boundary correction";
    return false;
  }
  if (cfg.time_stepper != DGSW_STEPPER_RK3_HESTHAVEN_SSP &&
      cfg.time_stepper != DGSW_STEPPER_ADAMS_BASHFORTH) {
    *err = "unsupported time stepper";
    return false;
  }
  if (cfg.precision != DGSW_PRECISION_FP64 && cfg.precision != DGSW_PRECISION_MIXED &&
      cfg.precision != DGSW_PRECISION_DOUBLE_FLOAT) {
    *err = "unknown precision";
    return false;
  }
  if (cfg.n_instances < 1 || !cfg.bricks) {
    *err = "need at least one brick";
    return false;
  }
  if (!std::isfinite(cfg.gamma2)) {
    *err = "gamma2 must be finite";
    return false;
  }
  dom->bricks.assign(cfg.bricks, cfg.bricks + cfg.n_instances);
  dom->layout.resize(cfg.n_instances);
  int64_t total = 0;
  for (int i = 0; i < cfg.n_instances; ++i) {
    const DgswBrick& b = dom->bricks[i];
    for (int d = 0; d < 3; ++d) {
      if (b.elements[d] < 1 || b.elements[d] > 4096) {
        *err = "elements per axis must be in [1, 4096]";
        return false;
      }
      if (!(b.upper[d] > b.lower[d]) || !std::isfinite(b.lower[d]) || !std::isfinite(b.upper[d])) {
        *err = "brick bounds must satisfy lower < upper";
        return false;
      }
      split_count(b.elements[d], &dom->layout[i].blocks[d], &dom->layout[i].level[d]);
      if (dom->layout[i].level[d] > 12) {
        *err = "refinement level above 12";
        return false;
      }
    }
    dom->layout[i].first = total;
    dom->layout[i].count = (int64_t)b.elements[0] * b.elements[1] * b.elements[2];
    total += dom->layout[i].count;
  }
  if (total > (int64_t)1 << 30) {
    *err = "too many elements";
    return false;
  }
  const int64_t E = total;
  dom->n_elem = E;
  dom->elem_n.resize(E);
  if (cfg.points_per_element) {
    for (int64_t e = 0; e < E; ++e) dom->elem_n[e] = cfg.points_per_element[e];
  } else {
    for (int64_t e = 0; e < E; ++e) dom->elem_n[e] = cfg.uniform_points;
  }
  dom->max_n = 0;
  dom->uniform = true;
  for (int64_t e = 0; e < E; ++e) {
    const int n = dom->elem_n[e];
    if (n < kMinN || n > kMaxN) {
      *err = "points per dimension must be in [2, 12]";
      return false;
    }
    dom->max_n = std::max(dom->max_n, n);
    if (n != dom->elem_n[0]) dom->uniform = false;
  }
  dom->offset.resize(E + 1);
  dom->offset[0] = 0;
  dom->n_points = 0;
  for (int64_t e = 0; e < E; ++e) {
    const int64_t np = (int64_t)dom->elem_n[e] * dom->elem_n[e] * dom->elem_n[e];
    dom->offset[e + 1] = dom->offset[e] + kVars * np;
    dom->n_points += np;
  }
  dom->neighbor.resize(6 * E);
  dom->instance.resize(E);
  dom->lower.resize(3 * E);
  dom->width.resize(3 * E);
  dom->element_id.resize(E);
  dom->block_ids_fit = true;
  for (int i = 0; i < cfg.n_instances; ++i) {
    const BrickLayout& L = dom->layout[i];
    const DgswBrick& b = dom->bricks[i];
    const int64_t per_block = (int64_t)1 << (L.level[0] + L.level[1] + L.level[2]);
    // element index of lattice point q (blocks x fastest, then x-outer /
    // z-inner segments inside a block: InitialElementIds.cpp:50-66)
    auto index_of = [&](const int q[3]) {
      int64_t blk[3], seg[3];
      for (int d = 0; d < 3; ++d) {
        blk[d] = q[d] >> L.level[d];
        seg[d] = q[d] & ((1 << L.level[d]) - 1);
      }
      const int64_t bid = blk[0] + L.blocks[0] * (blk[1] + (int64_t)L.blocks[1] * blk[2]);
      return L.first + bid * per_block + ((seg[0] << (L.level[1] + L.level[2])) | (seg[1] << L.level[2]) | seg[2]);
    };
    for (int64_t l = 0; l < L.count; ++l) {
      const int64_t e = L.first + l;
      const int64_t bid = l / per_block;
      const int64_t within = l % per_block;
      int seg[3], blk[3], q[3];
      seg[2] = (int)(within & ((1 << L.level[2]) - 1));
      seg[1] = (int)((within >> L.level[2]) & ((1 << L.level[1]) - 1));
      seg[0] = (int)(within >> (L.level[1] + L.level[2]));
      blk[0] = (int)(bid % L.blocks[0]);
      blk[1] = (int)((bid / L.blocks[0]) % L.blocks[1]);
      blk[2] = (int)(bid / ((int64_t)L.blocks[0] * L.blocks[1]));
      for (int d = 0; d < 3; ++d) q[d] = (blk[d] << L.level[d]) + seg[d];
      if (bid > 255) dom->block_ids_fit = false;
      dom->element_id[e] = (uint64_t)(bid & 0xff) | ((uint64_t)seg[0] << 16) |
                           ((uint64_t)L.level[0] << 28) | ((uint64_t)seg[1] << 32) |
                           ((uint64_t)L.level[1] << 44) | ((uint64_t)seg[2] << 48) |
                           ((uint64_t)L.level[2] << 60);
      dom->instance[e] = i;
      for (int d = 0; d < 3; ++d) {
        const double h = (b.upper[d] - b.lower[d]) / b.elements[d];
        dom->width[3 * e + d] = h;
        dom->lower[3 * e + d] = b.lower[d] + h * q[d];
      }
      for (int dir = 0; dir < 6; ++dir) {
        const int d = dir >> 1;
        int r[3] = {q[0], q[1], q[2]};
        const int n = b.elements[d];
        r[d] = (dir & 1) ? (r[d] + 1 == n ? 0 : r[d] + 1) : (r[d] == 0 ? n - 1 : r[d] - 1);
        dom->neighbor[6 * e + dir] = (int32_t)index_of(r);
      }
    }
  }
  return true;
}

}  // namespace dgsw
