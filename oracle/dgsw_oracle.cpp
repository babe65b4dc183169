// dgsw_oracle.cpp -- CPU FP64 restatement of the reference DG scalar-wave step.
//
// Test infrastructure: the checker for the CUDA path, never part of it.
// Each function names the reference file:line it restates (paths relative to
// the SpECTRE source tree).  Compiled with -ffp-contract=off so that every
// product and sum is rounded separately, as in the reference's scalar code.
#include "adams_oracle.hpp"
#include "dgsw_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kMaxN = 20;  // Spectral::maximum_number_of_points<Legendre>
constexpr int kVars = 5;   // Psi, Pi, Phi_x, Phi_y, Phi_z
constexpr int kPkg = 16;   // UpwindPenalty packaged doubles per face point

// EvaluateQandL, Legendre.cpp:160-184 (Kopriva algorithm 24 with errata).
void eval_q_and_l(int poly_degree, double x, double* q, double* L) {
  double lm2 = 1.0, lm1 = x, ln = 0.0;
  for (int k = 2; k <= poly_degree; ++k) {
    ln = ((2. * k - 1.) * x * lm1 - (k - 1.) * lm2) / k;
    lm2 = lm1;
    lm1 = ln;
  }
  const int k = poly_degree + 1;
  const double lnp1 = ((2. * k - 1.) * x * ln - (k - 1.) * lm2) / k;
  *q = lnp1 - lm2;
  *L = ln;
}

// Root of q on a sign-changing bracket.  The reference uses TOMS748 with a
// relative tolerance of 6e-16 (Legendre.cpp:218-226); plain bisection to
// adjacent doubles lands on the same root of the computed q.
double lgl_root(int poly_degree, double a, double b) {
  double qa, qb, L;
  eval_q_and_l(poly_degree, a, &qa, &L);
  eval_q_and_l(poly_degree, b, &qb, &L);
  if (qa == 0.0) return a;
  if (qb == 0.0) return b;
  for (int it = 0; it < 200; ++it) {
    const double m = 0.5 * (a + b);
    if (m <= std::min(a, b) || m >= std::max(a, b)) break;
    double qm;
    eval_q_and_l(poly_degree, m, &qm, &L);
    if (qm == 0.0) return m;
    if ((qm < 0) == (qa < 0)) {
      a = m;
      qa = qm;
    } else {
      b = m;
    }
  }
  return 0.5 * (a + b);
}

// compute_basis_function_value_impl for Legendre: P_k(x) by recurrence.
double legendre_p(int k, double x) {
  if (k == 0) return 1.0;
  double pm2 = 1.0, pm1 = x;
  for (int j = 2; j <= k; ++j) {
    const double p = ((2. * j - 1.) * x * pm1 - (j - 1.) * pm2) / j;
    pm2 = pm1;
    pm1 = p;
  }
  return pm1;
}

// Utilities/EqualWithinRoundoff.hpp: |a-b| <= eps*max(|a|,|b|,scale),
// eps = 100 * machine epsilon, scale = 1.
bool equal_within_roundoff(double a, double b) {
  const double eps = std::numeric_limits<double>::epsilon() * 100.0;
  return std::abs(a - b) <=
         eps * std::max(std::max(std::abs(a), std::abs(b)), 1.0);
}

struct Spectral1d {
  int n = 0;
  double x[kMaxN], w[kMaxN], bw[kMaxN];
  double D[kMaxN * kMaxN];
};

const Spectral1d& spectral(int n) {
  static Spectral1d table[kMaxN + 1];
  static bool init = [] {
    for (int m = 2; m <= kMaxN; ++m) {
      Spectral1d& s = table[m];
      s.n = m;
      orc_lgl(m, s.x, s.w);
      orc_barycentric_weights(m, s.bw);
      orc_diff_matrix(m, s.D);
    }
    return true;
  }();
  (void)init;
  return table[n];
}

// Decomposition of an element count into b blocks of refinement L (b odd).
void split_count(int n, int* blocks, int* level) {
  int L = 0;
  while ((n % 2) == 0) {
    n /= 2;
    ++L;
  }
  *blocks = n;
  *level = L;
}

struct InstLayout {
  int b[3], L[3];
  int64_t base;   // first global element index
  int64_t count;  // elements in this instance
};

std::vector<InstLayout> layouts(int n_inst, const OrcBrick* br) {
  std::vector<InstLayout> out(n_inst);
  int64_t base = 0;
  for (int i = 0; i < n_inst; ++i) {
    for (int d = 0; d < 3; ++d) split_count(br[i].n[d], &out[i].b[d], &out[i].L[d]);
    out[i].base = base;
    out[i].count = (int64_t)br[i].n[0] * br[i].n[1] * br[i].n[2];
    base += out[i].count;
  }
  return out;
}

// Global element index of lattice point (ix, iy, iz) of an instance:
// blocks x fastest (DomainHelpers.cpp:1187-1201), then elements of a block in
// x-outer / z-inner order (InitialElementIds.cpp:50-66).
int64_t element_index(const InstLayout& lay, const int ijk[3]) {
  int blk[3], seg[3];
  for (int d = 0; d < 3; ++d) {
    blk[d] = ijk[d] >> lay.L[d];
    seg[d] = ijk[d] & ((1 << lay.L[d]) - 1);
  }
  const int64_t block_id = blk[0] + (int64_t)lay.b[0] * (blk[1] + (int64_t)lay.b[1] * blk[2]);
  const int64_t per_block = (int64_t)1 << (lay.L[0] + lay.L[1] + lay.L[2]);
  const int64_t within =
      ((int64_t)seg[0] << (lay.L[1] + lay.L[2])) + ((int64_t)seg[1] << lay.L[2]) + seg[2];
  return lay.base + block_id * per_block + within;
}

void element_lattice(const InstLayout& lay, int64_t local, int ijk[3], int* block_id,
                     int seg[3]) {
  const int64_t per_block = (int64_t)1 << (lay.L[0] + lay.L[1] + lay.L[2]);
  const int64_t bid = local / per_block;
  int64_t within = local % per_block;
  seg[2] = (int)(within & ((1 << lay.L[2]) - 1));
  within >>= lay.L[2];
  seg[1] = (int)(within & ((1 << lay.L[1]) - 1));
  within >>= lay.L[1];
  seg[0] = (int)within;
  int blk[3];
  blk[0] = (int)(bid % lay.b[0]);
  blk[1] = (int)((bid / lay.b[0]) % lay.b[1]);
  blk[2] = (int)(bid / ((int64_t)lay.b[0] * lay.b[1]));
  for (int d = 0; d < 3; ++d) ijk[d] = (blk[d] << lay.L[d]) + seg[d];
  *block_id = (int)bid;
}

struct ElemGeom {
  int inst;
  int ijk[3];
  double lo[3];     // lower corner
  double h[3];      // widths
  double invjac[3]; // d xi^d / d x^d (diagonal; off-diagonal entries are 0)
};

struct Mesh {
  int n_inst;
  const OrcBrick* br;
  std::vector<InstLayout> lay;
  std::vector<ElemGeom> geom;
  std::vector<int32_t> nbr;  // 6 per element
  std::vector<int64_t> off;
  const int32_t* elem_n;
  int64_t n_elem;
};

void build_mesh(Mesh* m, int n_inst, const OrcBrick* br, const int32_t* elem_n) {
  m->n_inst = n_inst;
  m->br = br;
  m->lay = layouts(n_inst, br);
  m->n_elem = orc_num_elements(n_inst, br);
  m->elem_n = elem_n;
  m->geom.resize(m->n_elem);
  m->nbr.resize(6 * m->n_elem);
  m->off.resize(m->n_elem + 1);
  orc_offsets(m->n_elem, elem_n, m->off.data());
  for (int i = 0; i < n_inst; ++i) {
    const InstLayout& lay = m->lay[i];
    for (int64_t l = 0; l < lay.count; ++l) {
      int ijk[3], bid, seg[3];
      element_lattice(lay, l, ijk, &bid, seg);
      const int64_t e = lay.base + l;
      ElemGeom& g = m->geom[e];
      g.inst = i;
      for (int d = 0; d < 3; ++d) {
        g.ijk[d] = ijk[d];
        g.h[d] = (br[i].hi[d] - br[i].lo[d]) / br[i].n[d];
        g.lo[d] = br[i].lo[d] + g.h[d] * ijk[d];
        g.invjac[d] = 2.0 / g.h[d];
      }
      for (int dir = 0; dir < 6; ++dir) {
        const int d = dir / 2;
        int q[3] = {ijk[0], ijk[1], ijk[2]};
        q[d] = (dir % 2) ? (q[d] + 1) % br[i].n[d] : (q[d] + br[i].n[d] - 1) % br[i].n[d];
        m->nbr[6 * e + dir] = (int32_t)element_index(lay, q);
      }
    }
  }
}

// Face slice of a volume field: ProjectToBoundary.hpp:114-146 for GLL (the
// face is a slice of volume points).  Face point index = a + n*b over the two
// remaining dimensions in ascending order.
inline int64_t volume_index(int n, int d, int slice, int a, int b) {
  switch (d) {
    case 0: return slice + (int64_t)n * (a + (int64_t)n * b);
    case 1: return a + (int64_t)n * (slice + (int64_t)n * b);
    default: return a + (int64_t)n * (b + (int64_t)n * slice);
  }
}

// apply_matrices on a 2D face: out(i', j') = sum_i sum_j M(i',i) M(j',j) in(i,j),
// first index fastest; M is rows x cols row-major.
void apply_face_matrix(int rows, int cols, const double* M, int nfields,
                       const double* in, double* out) {
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

// Package one face of element e in direction dir: InternalMortarDataImpl.hpp
// :177-221 (normal = sign * inverse-Jacobian row, normalised as in
// NormalCovectorAndMagnitude.hpp:84-98) then UpwindPenalty::dg_package_data.
void package_face(const Mesh& m, const double* u, double gamma2, int64_t e, int dir,
                  double* pkg, double* magnitude) {
  const int n = m.elem_n[e];
  const int64_t np = (int64_t)n * n * n;
  const int d = dir / 2;
  const bool upper = dir % 2;
  const int slice = upper ? n - 1 : 0;
  const int nf = n * n;
  const double* ue = u + m.off[e];
  std::vector<double> psi(nf), pi(nf), phi(3 * nf), g2(nf, gamma2), nrm(3 * nf);
  const double sign = upper ? 1.0 : -1.0;
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < n; ++a) {
      const int f = a + n * b;
      const int64_t v = volume_index(n, d, slice, a, b);
      psi[f] = ue[v];
      pi[f] = ue[np + v];
      for (int i = 0; i < 3; ++i) phi[i * nf + f] = ue[(2 + i) * np + v];
      double un[3];
      for (int i = 0; i < 3; ++i) un[i] = sign * (i == d ? m.geom[e].invjac[d] : 0.0);
      const double mag = std::sqrt(un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
      const double inv = 1.0 / mag;
      for (int i = 0; i < 3; ++i) nrm[i * nf + f] = un[i] * inv;
      magnitude[f] = mag;
    }
  double ms;
  orc_package(nf, psi.data(), pi.data(), phi.data(), g2.data(), nrm.data(), nullptr, pkg, &ms);
}

void volume_terms(const Mesh& m, const double* u, double gamma2, int64_t e, double* dt,
                  const double* Dmat = nullptr) {
  const int n = m.elem_n[e];
  const int64_t np = (int64_t)n * n * n;
  const double* Dm = Dmat ? Dmat : spectral(n).D;
  const double* ue = u + m.off[e];
  // logical derivatives of all 5 vars (PartialDerivatives.tpp:315-363)
  std::vector<double> dl((size_t)3 * kVars * np);
  for (int v = 0; v < kVars; ++v) {
    const double* f = ue + v * np;
    for (int a = 0; a < 3; ++a) {
      double* out = dl.data() + ((size_t)a * kVars + v) * np;
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) {
            const int idx[3] = {i, j, k};
            double s = 0.0;
            for (int q = 0; q < n; ++q) {
              int id2[3] = {i, j, k};
              id2[a] = q;
              s += Dm[idx[a] * n + q] * f[id2[0] + n * (id2[1] + n * id2[2])];
            }
            out[i + n * (j + n * k)] = s;
          }
    }
  }
  // du_i = sum_a invjac(a, i) * d_a u, a = 0 first (PartialDerivatives.tpp:82-105)
  const ElemGeom& g = m.geom[e];
  auto ij = [&](int a, int i) { return a == i ? g.invjac[a] : 0.0; };
  std::vector<double> du((size_t)3 * kVars * np);  // [v][i][pt]
  for (int v = 0; v < kVars; ++v)
    for (int i = 0; i < 3; ++i) {
      double* out = du.data() + ((size_t)v * 3 + i) * np;
      const double* l0 = dl.data() + ((size_t)0 * kVars + v) * np;
      const double* l1 = dl.data() + ((size_t)1 * kVars + v) * np;
      const double* l2 = dl.data() + ((size_t)2 * kVars + v) * np;
      for (int64_t p = 0; p < np; ++p) {
        double s = ij(0, i) * l0[p];
        s += ij(1, i) * l1[p];
        s += ij(2, i) * l2[p];
        out[p] = s;
      }
    }
  // ScalarWave::TimeDerivative<3>::apply, TimeDerivative.cpp:37-44
  const double* pi = ue + np;
  for (int64_t p = 0; p < np; ++p) {
    auto dpsi = [&](int i) { return du[((size_t)0 * 3 + i) * np + p]; };
    auto dpi = [&](int i) { return du[((size_t)1 * 3 + i) * np + p]; };
    auto dphi = [&](int i, int j) { return du[((size_t)(2 + j) * 3 + i) * np + p]; };
    dt[p] = -pi[p];
    double s = -dphi(0, 0);
    s -= dphi(1, 1);
    s -= dphi(2, 2);
    dt[np + p] = s;
    for (int dd = 0; dd < 3; ++dd)
      dt[(2 + dd) * np + p] = -dpi(dd) + gamma2 * (dpsi(dd) - ue[(2 + dd) * np + p]);
  }
}

// ApplyBoundaryCorrections.hpp:723-1050 for GLL global time stepping: per
// mortar, dg_boundary_terms, project from mortar if needed, lift_flux, then
// add_slice_to_data.
void boundary_terms(const Mesh& m, const double* u, double gamma2, int64_t e, double* dt) {
  const int n = m.elem_n[e];
  const int64_t np = (int64_t)n * n * n;
  for (int dir = 0; dir < 6; ++dir) {
    const int d = dir / 2;
    const bool upper = dir % 2;
    const int64_t nb = m.nbr[6 * e + dir];
    const int nn = m.elem_n[nb];
    const int nm = std::max(n, nn);  // mortar_mesh, MortarHelpers.cpp:41
    std::vector<double> pkg_i((size_t)kPkg * n * n), pkg_e((size_t)kPkg * nn * nn);
    std::vector<double> mag_i(n * n), mag_e(nn * nn);
    package_face(m, u, gamma2, e, dir, pkg_i.data(), mag_i.data());
    package_face(m, u, gamma2, nb, dir ^ 1, pkg_e.data(), mag_e.data());
    std::vector<double> mi((size_t)kPkg * nm * nm), me((size_t)kPkg * nm * nm);
    if (nm != n) {
      std::vector<double> P((size_t)nm * n);
      orc_proj_face_to_mortar(n, nm, P.data());
      apply_face_matrix(nm, n, P.data(), kPkg, pkg_i.data(), mi.data());
    } else {
      mi = pkg_i;
    }
    if (nm != nn) {
      std::vector<double> P((size_t)nm * nn);
      orc_proj_face_to_mortar(nn, nm, P.data());
      apply_face_matrix(nm, nn, P.data(), kPkg, pkg_e.data(), me.data());
    } else {
      me = pkg_e;
    }
    std::vector<double> bc_m((size_t)kVars * nm * nm), bc((size_t)kVars * n * n);
    orc_boundary_terms(nm * nm, mi.data(), me.data(), bc_m.data());
    if (nm != n) {
      std::vector<double> P((size_t)n * nm);
      orc_proj_mortar_to_face(n, nm, P.data());
      apply_face_matrix(n, nm, P.data(), kVars, bc_m.data(), bc.data());
    } else {
      bc = bc_m;
    }
    // lift_flux, LiftFlux.hpp:57-61
    const int nf = n * n;
    const double slice_factor = -0.5 * static_cast<double>(n * (n - 1));
    const int slice = upper ? n - 1 : 0;
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        const int f = a + n * b;
        const int64_t vi = volume_index(n, d, slice, a, b);
        const double fac = slice_factor * mag_i[f];
        for (int v = 0; v < kVars; ++v) dt[v * np + vi] += bc[(size_t)v * nf + f] * fac;
      }
  }
}

}  // namespace

extern "C" {

int orc_lgl(int n, double* x, double* w) {
  // Legendre.cpp:186-239 (Kopriva algorithm 25)
  if (n < 2 || n > kMaxN || !x || !w) return -1;
  const int p = n - 1;
  if (p == 1) {
    x[0] = -1.;
    x[1] = 1.;
    w[0] = w[1] = 1.;
    return 0;
  }
  x[0] = -1.;
  x[p] = 1.;
  w[0] = w[p] = 2. / (p * (p + 1.));
  for (int j = 1; j < (p + 1) / 2; ++j) {
    const double a = -std::cos((j - 0.25) * M_PI / p - 0.375 / (p * M_PI * (j - 0.25)));
    const double b = -std::cos((j + 0.75) * M_PI / p - 0.375 / (p * M_PI * (j + 0.75)));
    const double r = lgl_root(p, a, b);
    double q, L;
    eval_q_and_l(p, r, &q, &L);
    x[j] = r;
    x[p - j] = -r;
    w[j] = w[p - j] = 2. / (p * (p + 1.) * (L * L));
  }
  if (p % 2 == 0) {
    double q, L;
    eval_q_and_l(p, 0., &q, &L);
    x[p / 2] = 0.;
    w[p / 2] = 2. / (p * (p + 1.) * (L * L));
  }
  return 0;
}

int orc_barycentric_weights(int n, double* bw) {
  // Spectral.cpp:84-101 (Kopriva algorithm 30)
  if (n < 2 || n > kMaxN || !bw) return -1;
  double x[kMaxN], w[kMaxN];
  orc_lgl(n, x, w);
  for (int j = 0; j < n; ++j) bw[j] = 1.;
  for (int j = 1; j < n; ++j)
    for (int k = 0; k < j; ++k) {
      bw[k] *= x[k] - x[j];
      bw[j] *= x[j] - x[k];
    }
  for (int j = 0; j < n; ++j) bw[j] = 1. / bw[j];
  return 0;
}

int orc_diff_matrix(int n, double* D) {
  // Spectral.cpp:431-444 (Kopriva algorithm 37, negative-sum diagonal)
  if (n < 2 || n > kMaxN || !D) return -1;
  double x[kMaxN], w[kMaxN], bw[kMaxN];
  orc_lgl(n, x, w);
  orc_barycentric_weights(n, bw);
  for (int i = 0; i < n; ++i) {
    double diag = 0.0;
    for (int j = 0; j < n; ++j) {
      if (i != j) {
        D[i * n + j] = bw[j] / (bw[i] * (x[i] - x[j]));
        diag -= D[i * n + j];
      }
    }
    D[i * n + i] = diag;
  }
  return 0;
}

int orc_vandermonde(int n, double* V) {
  // ModalToNodalMatrixGenerator, Spectral.cpp:499-516
  if (n < 2 || n > kMaxN || !V) return -1;
  double x[kMaxN], w[kMaxN];
  orc_lgl(n, x, w);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) V[i * n + k] = legendre_p(k, x[i]);
  return 0;
}

int orc_inv_vandermonde(int n, double* Vinv) {
  // NodalToModalMatrixGenerator, Spectral.cpp:518-523: numerical inverse
  // (LU with partial pivoting, as LAPACK's getrf/getri behind blaze::inv).
  if (n < 2 || n > kMaxN || !Vinv) return -1;
  double A[kMaxN * kMaxN];
  orc_vandermonde(n, A);
  double B[kMaxN * kMaxN];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) B[i * n + j] = (i == j) ? 1.0 : 0.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::abs(A[r * n + c]) > std::abs(A[piv * n + c])) piv = r;
    if (piv != c)
      for (int j = 0; j < n; ++j) {
        std::swap(A[c * n + j], A[piv * n + j]);
        std::swap(B[c * n + j], B[piv * n + j]);
      }
    const double inv = 1.0 / A[c * n + c];
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = A[r * n + c] * inv;
      if (f == 0.0) continue;
      for (int j = 0; j < n; ++j) {
        A[r * n + j] -= f * A[c * n + j];
        B[r * n + j] -= f * B[c * n + j];
      }
    }
  }
  for (int r = 0; r < n; ++r) {
    const double inv = 1.0 / A[r * n + r];
    for (int j = 0; j < n; ++j) Vinv[r * n + j] = B[r * n + j] * inv;
  }
  return 0;
}

int orc_interp_matrix(int n, int m, const double* t, double* M) {
  // Spectral.cpp:625-670 (Kopriva algorithm 32)
  if (n < 2 || n > kMaxN || m < 0 || !M || (m > 0 && !t)) return -1;
  const Spectral1d& s = spectral(n);
  for (int k = 0; k < m; ++k) {
    bool match = false;
    for (int j = 0; j < n; ++j) {
      M[k * n + j] = 0.0;
      if (equal_within_roundoff(t[k], s.x[j])) {
        M[k * n + j] = 1.0;
        match = true;
      }
    }
    if (!match) {
      double sum = 0.0;
      for (int j = 0; j < n; ++j) {
        M[k * n + j] = s.bw[j] / (t[k] - s.x[j]);
        sum += M[k * n + j];
      }
      for (int j = 0; j < n; ++j) M[k * n + j] /= sum;
    }
  }
  return 0;
}

int orc_proj_face_to_mortar(int ne, int nm, double* P) {
  // projection_matrix_parent_to_child, ChildSize::Full: interpolation of the
  // element's face polynomial to the mortar points (Projection.cpp:310-330)
  if (ne < 2 || nm < ne || nm > kMaxN || !P) return -1;
  const Spectral1d& sm = spectral(nm);
  return orc_interp_matrix(ne, nm, sm.x, P);
}

int orc_proj_mortar_to_face(int ne, int nm, double* P) {
  // projection_matrix_child_to_parent, ChildSize::Full, not massive:
  // truncation of the mortar's Legendre modes (Projection.cpp:97-130)
  if (ne < 2 || nm < ne || nm > kMaxN || !P) return -1;
  double Ve[kMaxN * kMaxN], Vm_inv[kMaxN * kMaxN];
  orc_vandermonde(ne, Ve);
  orc_inv_vandermonde(nm, Vm_inv);
  for (int i = 0; i < ne; ++i)
    for (int j = 0; j < nm; ++j) {
      double s = 0.;
      for (int k = 0; k < ne; ++k) s += Ve[i * ne + k] * Vm_inv[k * nm + j];
      P[i * nm + j] = s;
    }
  return 0;
}

int64_t orc_num_elements(int n_inst, const OrcBrick* br) {
  int64_t c = 0;
  for (int i = 0; i < n_inst; ++i) c += (int64_t)br[i].n[0] * br[i].n[1] * br[i].n[2];
  return c;
}

int orc_index_maps(int n_inst, const OrcBrick* br, uint64_t* elem_id, int32_t* nbr,
                   int32_t* ijk_out, int32_t* inst) {
  if (n_inst < 1 || !br) return -1;
  for (int i = 0; i < n_inst; ++i)
    for (int d = 0; d < 3; ++d)
      if (br[i].n[d] < 1) return -1;
  std::vector<InstLayout> lay = layouts(n_inst, br);
  int rc = 0;
  for (int i = 0; i < n_inst; ++i) {
    for (int64_t l = 0; l < lay[i].count; ++l) {
      int ijk[3], bid, seg[3];
      element_lattice(lay[i], l, ijk, &bid, seg);
      const int64_t e = lay[i].base + l;
      if (bid >= 256) rc = -2;  // not representable in the 8 block-id bits
      if (elem_id) {
        // ElementId.hpp:138-147 bit fields, least significant first
        uint64_t id = (uint64_t)(bid & 0xff);
        id |= (uint64_t)0 << 8;   // grid index
        id |= (uint64_t)0 << 12;  // direction
        id |= (uint64_t)seg[0] << 16;
        id |= (uint64_t)lay[i].L[0] << 28;
        id |= (uint64_t)seg[1] << 32;
        id |= (uint64_t)lay[i].L[1] << 44;
        id |= (uint64_t)seg[2] << 48;
        id |= (uint64_t)lay[i].L[2] << 60;
        elem_id[e] = id;
      }
      if (ijk_out)
        for (int d = 0; d < 3; ++d) ijk_out[3 * e + d] = ijk[d];
      if (inst) inst[e] = i;
      if (nbr)
        for (int dir = 0; dir < 6; ++dir) {
          const int d = dir / 2;
          int q[3] = {ijk[0], ijk[1], ijk[2]};
          q[d] = (dir % 2) ? (q[d] + 1) % br[i].n[d] : (q[d] + br[i].n[d] - 1) % br[i].n[d];
          nbr[6 * e + dir] = (int32_t)element_index(lay[i], q);
        }
    }
  }
  return rc;
}

int orc_offsets(int64_t n_elem, const int32_t* elem_n, int64_t* off) {
  if (n_elem < 0 || !elem_n || !off) return -1;
  off[0] = 0;
  for (int64_t e = 0; e < n_elem; ++e) {
    const int64_t n = elem_n[e];
    off[e + 1] = off[e] + kVars * n * n * n;
  }
  return 0;
}

int orc_coords(int n_inst, const OrcBrick* br, const int32_t* elem_n, double* xyz) {
  if (n_inst < 1 || !br || !elem_n || !xyz) return -1;
  Mesh m;
  build_mesh(&m, n_inst, br, elem_n);
  int64_t pos = 0;
  for (int64_t e = 0; e < m.n_elem; ++e) {
    const int n = elem_n[e];
    const int64_t np = (int64_t)n * n * n;
    const Spectral1d& s = spectral(n);
    const ElemGeom& g = m.geom[e];
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int64_t p = i + n * (j + (int64_t)n * k);
          const int id[3] = {i, j, k};
          for (int d = 0; d < 3; ++d)
            xyz[pos + d * np + p] = g.lo[d] + (s.x[id[d]] + 1.0) * (0.5 * g.h[d]);
        }
    pos += 3 * np;
  }
  return 0;
}

int orc_initial_data(int n_inst, const OrcBrick* br, const int32_t* elem_n, int kind,
                     const double* params, double t, double* u) {
  if (n_inst < 1 || !br || !elem_n || !params || !u) return -1;
  Mesh m;
  build_mesh(&m, n_inst, br, elem_n);
  for (int64_t e = 0; e < m.n_elem; ++e) {
    const int n = elem_n[e];
    const int64_t np = (int64_t)n * n * n;
    const Spectral1d& s = spectral(n);
    const ElemGeom& g = m.geom[e];
    double* ue = u + m.off[e];
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int64_t p = i + n * (j + (int64_t)n * k);
          const int id[3] = {i, j, k};
          double x[3];
          for (int d = 0; d < 3; ++d) x[d] = g.lo[d] + (s.x[id[d]] + 1.0) * (0.5 * g.h[d]);
          if (kind == 0) {
            // PlaneWave.cpp:56-80: psi = f(k.x - omega t), Pi = -dpsi/dt
            const double* kv = params;
            const double omega = std::sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
            const double ph = kv[0] * x[0] + kv[1] * x[1] + kv[2] * x[2] - omega * t;
            ue[p] = std::sin(ph);
            ue[np + p] = omega * std::cos(ph);
            for (int d = 0; d < 3; ++d) ue[(2 + d) * np + p] = kv[d] * std::cos(ph);
          } else if (kind == 1) {
            const double* q = params + 5 * g.inst;
            const double A = q[0], w = q[1];
            double r2 = 0.0, dx[3];
            for (int d = 0; d < 3; ++d) {
              dx[d] = x[d] - q[2 + d];
              r2 += dx[d] * dx[d];
            }
            const double psi = A * std::exp(-r2 / (w * w));
            ue[p] = psi;
            ue[np + p] = 0.0;
            for (int d = 0; d < 3; ++d) ue[(2 + d) * np + p] = -2.0 * dx[d] / (w * w) * psi;
          } else {
            return -1;
          }
        }
  }
  return 0;
}

int orc_package(int npts, const double* psi, const double* pi, const double* phi,
                const double* gamma2, const double* normal, const double* ndotv,
                double* pkg, double* max_speed) {
  // UpwindPenalty<3>::dg_package_data, UpwindPenalty.cpp:35-108
  if (npts < 0 || !psi || !pi || !phi || !gamma2 || !normal || !pkg) return -1;
  const int n = npts;
  double* v_psi = pkg;
  double* v_zero = pkg + n;
  double* v_plus = pkg + 4 * n;
  double* v_minus = pkg + 5 * n;
  double* n_v_plus = pkg + 6 * n;
  double* n_v_minus = pkg + 9 * n;
  double* g2_v_psi = pkg + 12 * n;
  double* speeds = pkg + 13 * n;
  double mx = -std::numeric_limits<double>::infinity();
  for (int p = 0; p < n; ++p) {
    double c0, c1, c2;
    if (ndotv) {
      c0 = -ndotv[p];
      c1 = 1.0 - ndotv[p];
      c2 = -1.0 - ndotv[p];
    } else {
      c0 = 0.0;
      c1 = 1.0;
      c2 = -1.0;
    }
    speeds[p] = c0;
    speeds[n + p] = c1;
    speeds[2 * n + p] = c2;
    const double g2psi = gamma2[p] * psi[p];
    // dot_product(normal, phi): n_0 phi_0 + n_1 phi_1 + n_2 phi_2
    double ndp = normal[p] * phi[p];
    ndp += normal[n + p] * phi[n + p];
    ndp += normal[2 * n + p] * phi[2 * n + p];
    for (int i = 0; i < 3; ++i)
      v_zero[i * n + p] = c0 * (phi[i * n + p] - normal[i * n + p] * ndp);
    v_plus[p] = c1 * (pi[p] + ndp - g2psi);
    v_minus[p] = c2 * (pi[p] - ndp - g2psi);
    for (int i = 0; i < 3; ++i) {
      n_v_plus[i * n + p] = v_plus[p] * normal[i * n + p];
      n_v_minus[i * n + p] = v_minus[p] * normal[i * n + p];
    }
    v_psi[p] = c0 * psi[p];
    g2_v_psi[p] = g2psi * c0;
    mx = std::max(mx, std::max(c0, std::max(c1, c2)));
  }
  if (max_speed) *max_speed = mx;
  return 0;
}

int orc_boundary_terms(int npts, const double* pi_, const double* pe, double* out) {
  // UpwindPenalty<3>::dg_boundary_terms, UpwindPenalty.cpp:110-205, with
  // step_function(x) = x >= 0 ? 1 : 0 (Utilities/Math.hpp:70-74)
  if (npts < 0 || !pi_ || !pe || !out) return -1;
  const int n = npts;
  auto step = [](double x) { return x >= 0.0 ? 1.0 : 0.0; };
  for (int p = 0; p < n; ++p) {
    const double* si = pi_ + 13 * n;
    const double* se = pe + 13 * n;
    const double wpsi_i = step(-si[p]);
    const double wpsi_e = -step(se[p]);
    const double wzero_i = step(-si[p]);
    const double wzero_e = -step(se[p]);
    const double wplus_i = step(-si[n + p]);
    const double wplus_e = -step(se[n + p]);
    const double wminus_i = step(-si[2 * n + p]);
    const double wminus_e = -step(se[2 * n + p]);
    out[p] = wpsi_e * pe[p] - wpsi_i * pi_[p];
    out[n + p] = 0.5 * (wplus_e * pe[4 * n + p] + wminus_e * pe[5 * n + p]) +
                 wpsi_e * pe[12 * n + p] -
                 0.5 * (wplus_i * pi_[4 * n + p] + wminus_i * pi_[5 * n + p]) -
                 wpsi_i * pi_[12 * n + p];
    for (int d = 0; d < 3; ++d)
      out[(2 + d) * n + p] =
          0.5 * (wplus_e * pe[(6 + d) * n + p] - wminus_e * pe[(9 + d) * n + p]) +
          wzero_e * pe[(1 + d) * n + p] -
          0.5 * (wplus_i * pi_[(6 + d) * n + p] - wminus_i * pi_[(9 + d) * n + p]) -
          wzero_i * pi_[(1 + d) * n + p];
  }
  return 0;
}

int orc_volume_rhs(int n_inst, const OrcBrick* br, const int32_t* elem_n, double gamma2,
                   const double* u, double* dudt, int n_threads) {
  if (n_inst < 1 || !br || !elem_n || !u || !dudt) return -1;
  Mesh m;
  build_mesh(&m, n_inst, br, elem_n);
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t e = 0; e < m.n_elem; ++e) volume_terms(m, u, gamma2, e, dudt + m.off[e]);
  (void)n_threads;
  return 0;
}

int orc_rhs(int n_inst, const OrcBrick* br, const int32_t* elem_n, double gamma2,
            const double* u, double* dudt, int n_threads) {
  if (n_inst < 1 || !br || !elem_n || !u || !dudt) return -1;
  for (int i = 0; i < n_inst; ++i)
    for (int d = 0; d < 3; ++d)
      if (br[i].n[d] < 1) return -1;
  Mesh m;
  build_mesh(&m, n_inst, br, elem_n);
  for (int64_t e = 0; e < m.n_elem; ++e)
    if (elem_n[e] < 2 || elem_n[e] > kMaxN) return -1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t e = 0; e < m.n_elem; ++e) {
    volume_terms(m, u, gamma2, e, dudt + m.off[e]);
    boundary_terms(m, u, gamma2, e, dudt + m.off[e]);
  }
  (void)n_threads;
  return 0;
}

int orc_rk3_substep(int64_t n, int k, double dt, const double* u0, const double* ucur,
                    const double* du, double* un) {
  // Rk3HesthavenSsp::update_u_impl, Rk3HesthavenSsp.cpp:63-80
  if (n < 0 || k < 0 || k > 2 || !u0 || !ucur || !du || !un) return -1;
  for (int64_t i = 0; i < n; ++i) {
    if (k == 0) {
      un[i] = ucur[i] + dt * du[i];
    } else if (k == 1) {
      un[i] = 0.25 * (3.0 * u0[i] + ucur[i] + dt * du[i]);
    } else {
      un[i] = (1.0 / 3.0) * (u0[i] + 2.0 * ucur[i] + 2.0 * dt * du[i]);
    }
  }
  return 0;
}

int orc_evolve(int n_inst, const OrcBrick* br, const int32_t* elem_n, double gamma2,
               double dt, int n_steps, double* u, int n_threads) {
  if (n_inst < 1 || !br || !elem_n || !u || n_steps < 0) return -1;
  const int64_t n_elem = orc_num_elements(n_inst, br);
  std::vector<int64_t> off(n_elem + 1);
  orc_offsets(n_elem, elem_n, off.data());
  const int64_t n = off[n_elem];
  std::vector<double> u0(n), u1(n), du(n);
  for (int s = 0; s < n_steps; ++s) {
    std::memcpy(u0.data(), u, n * sizeof(double));
    int rc = orc_rhs(n_inst, br, elem_n, gamma2, u0.data(), du.data(), n_threads);
    if (rc) return rc;
    orc_rk3_substep(n, 0, dt, u0.data(), u0.data(), du.data(), u1.data());
    orc_rhs(n_inst, br, elem_n, gamma2, u1.data(), du.data(), n_threads);
    orc_rk3_substep(n, 1, dt, u0.data(), u1.data(), du.data(), u);
    std::memcpy(u1.data(), u, n * sizeof(double));
    orc_rhs(n_inst, br, elem_n, gamma2, u1.data(), du.data(), n_threads);
    orc_rk3_substep(n, 2, dt, u0.data(), u1.data(), du.data(), u);
  }
  return 0;
}

}  // extern "C"

// ===================== CurvedScalarWave (configuration 5) =====================
extern "C" {

int orc_ks_background(int npts, double M, const double* xyz, double* bg) {
  // Schwarzschild in Kerr-Schild coordinates (spin 0, centre 0): the closed
  // forms of Test_KerrSchild.cpp:55-232.
  if (npts < 0 || !xyz || !bg) return -1;
  const int n = npts;
  for (int p = 0; p < n; ++p) {
    const double x[3] = {xyz[p], xyz[n + p], xyz[2 * n + p]};
    const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    const double r = std::sqrt(r2);
    const double lapse = 1.0 / std::sqrt(1.0 + 2.0 * M / r);
    const double l2 = lapse * lapse;
    bg[p] = lapse;
    for (int i = 0; i < 3; ++i) bg[(1 + i) * n + p] = 2.0 * M * x[i] / r2 * l2;
    for (int i = 0; i < 3; ++i) bg[(4 + i) * n + p] = M * x[i] / (r2 * r) * l2 * lapse;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        // d_i shift^j
        double v = (i == j) ? 2.0 * M / r2 * l2 : 0.0;
        v -= 4.0 * M * x[i] * x[j] / (r2 * r2) * l2 * (1.0 - M / r * l2);
        bg[(7 + 3 * i + j) * n + p] = v;
      }
    const int pairs[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    for (int q = 0; q < 6; ++q) {
      const int i = pairs[q][0], j = pairs[q][1];
      bg[(16 + q) * n + p] = (i == j ? 1.0 : 0.0) - 2.0 * M * x[i] * x[j] / (r2 * (r + 2.0 * M));
    }
    const double f = M * (8.0 * M + 3.0 * r) / ((2.0 * M + r) * (2.0 * M + r) * r2);
    for (int i = 0; i < 3; ++i) bg[(22 + i) * n + p] = f * x[i];
    bg[25 * n + p] = 2.0 * M * (3.0 * M + r) * std::pow((2.0 * M + r) * r, -1.5);
  }
  return 0;
}

static inline double inv_metric(const double* bg, int n, int p, int i, int j) {
  static const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  return bg[(16 + idx[i][j]) * n + p];
}

int orc_csw_time_derivative(int npts, const double* d_psi, const double* d_pi,
                            const double* d_phi, const double* pi, const double* phi,
                            const double* bg, double gamma1, double gamma2, double* dt) {
  // CurvedScalarWave::TimeDerivative<3>::apply, TimeDerivative.cpp:47-68
  if (npts < 0 || !d_psi || !d_pi || !d_phi || !pi || !phi || !bg || !dt) return -1;
  const int n = npts;
  for (int p = 0; p < n; ++p) {
    const double lapse = bg[p];
    const double* shift = bg + n;  // shift^i at (1+i)*n + p
    auto sh = [&](int i) { return shift[i * n + p]; };
    auto dl = [&](int i) { return bg[(4 + i) * n + p]; };
    auto ds = [&](int i, int j) { return bg[(7 + 3 * i + j) * n + p]; };
    auto gam = [&](int i) { return bg[(22 + i) * n + p]; };
    const double K = bg[25 * n + p];
    auto dps = [&](int i) { return d_psi[i * n + p]; };
    auto dpi = [&](int i) { return d_pi[i * n + p]; };
    auto dph = [&](int i, int j) { return d_phi[(3 * i + j) * n + p]; };
    auto ph = [&](int i) { return phi[i * n + p]; };
    double s = -lapse * pi[p];
    for (int i = 0; i < 3; ++i) s += sh(i) * dps(i);
    for (int j = 0; j < 3; ++j) s += gamma1 * sh(j) * (dps(j) - ph(j));
    dt[p] = s;
    s = lapse * pi[p] * K;
    for (int i = 0; i < 3; ++i) s += sh(i) * dpi(i);
    for (int i = 0; i < 3; ++i) s += lapse * gam(i) * ph(i);
    for (int i = 0; i < 3; ++i) s += gamma1 * gamma2 * sh(i) * (dps(i) - ph(i));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) s -= lapse * inv_metric(bg, n, p, i, j) * dph(i, j);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) s -= inv_metric(bg, n, p, i, j) * ph(i) * dl(j);
    dt[n + p] = s;
    for (int i = 0; i < 3; ++i) {
      double v = -lapse * dpi(i);
      for (int j = 0; j < 3; ++j) v += sh(j) * dph(j, i);
      v += gamma2 * lapse * (dps(i) - ph(i));
      v -= pi[p] * dl(i);
      for (int j = 0; j < 3; ++j) v += ph(j) * ds(i, j);
      dt[(2 + i) * n + p] = v;
    }
  }
  return 0;
}

int orc_csw_package(int npts, const double* psi, const double* pi, const double* phi,
                    const double* lapse, const double* shift, const double* gamma1,
                    const double* gamma2, const double* nrm, const double* nvec,
                    const double* ndotv, double* pkg, double* max_speed) {
  // CurvedScalarWave UpwindPenalty::dg_package_data, UpwindPenalty.cpp:35-75,
  // with characteristic_fields / characteristic_speeds, Characteristics.cpp
  if (npts < 0 || !psi || !pi || !phi || !lapse || !shift || !gamma1 || !gamma2 || !nrm ||
      !nvec || !pkg)
    return -1;
  const int n = npts;
  double mx = -std::numeric_limits<double>::infinity();
  for (int p = 0; p < n; ++p) {
    double ndp = 0.0;  // n^i Phi_i
    for (int i = 0; i < 3; ++i) ndp += nvec[i * n + p] * phi[i * n + p];
    pkg[p] = psi[p];
    for (int i = 0; i < 3; ++i) pkg[(1 + i) * n + p] = phi[i * n + p] - nrm[i * n + p] * ndp;
    pkg[4 * n + p] = pi[p] + ndp - gamma2[p] * psi[p];
    pkg[5 * n + p] = pi[p] - ndp - gamma2[p] * psi[p];
    pkg[6 * n + p] = gamma2[p];
    for (int i = 0; i < 3; ++i) pkg[(7 + i) * n + p] = nrm[i * n + p];
    double bn = 0.0;  // shift^i n_i
    for (int i = 0; i < 3; ++i) bn += shift[i * n + p] * nrm[i * n + p];
    double c0 = -(1.0 + gamma1[p]) * bn, c1 = -bn, c2 = -bn + lapse[p], c3 = -bn - lapse[p];
    if (ndotv) {
      c0 -= ndotv[p];
      c1 -= ndotv[p];
      c2 -= ndotv[p];
      c3 -= ndotv[p];
    }
    pkg[10 * n + p] = c0;
    pkg[11 * n + p] = c1;
    pkg[12 * n + p] = c2;
    pkg[13 * n + p] = c3;
    mx = std::max(mx, std::max(c0, std::max(c1, c2)));
  }
  if (max_speed) *max_speed = mx;
  return 0;
}

int orc_csw_boundary_terms(int npts, const double* pi_, const double* pe, double* out) {
  // CurvedScalarWave UpwindPenalty::dg_boundary_terms, UpwindPenalty.cpp:77-127
  if (npts < 0 || !pi_ || !pe || !out) return -1;
  const int n = npts;
  auto step = [](double x) { return x >= 0.0 ? 1.0 : 0.0; };
  for (int p = 0; p < n; ++p) {
    const double* si = pi_ + 10 * n;
    const double* se = pe + 10 * n;
    const double psi_bc = -step(se[p]) * se[p] * pe[p] - step(-si[p]) * si[p] * pi_[p];
    const double t1 = -step(se[2 * n + p]) * se[2 * n + p] * pe[4 * n + p] -
                      step(-si[3 * n + p]) * si[3 * n + p] * pi_[5 * n + p];
    const double t2 = step(-si[2 * n + p]) * si[2 * n + p] * pi_[4 * n + p] +
                      step(se[3 * n + p]) * se[3 * n + p] * pe[5 * n + p];
    out[p] = psi_bc;
    out[n + p] = 0.5 * (t1 - t2) + pi_[6 * n + p] * psi_bc;
    const double t1b = -0.5 * (t1 + t2);
    for (int i = 0; i < 3; ++i)
      out[(2 + i) * n + p] = t1b * pi_[(7 + i) * n + p] -
                             step(se[n + p]) * se[n + p] * pe[(1 + i) * n + p] -
                             step(-si[n + p]) * si[n + p] * pi_[(1 + i) * n + p];
  }
  return 0;
}

int orc_csw_cpsr(int npts, const double* psi, const double* pi, const double* phi,
                 const double* lapse, const double* shift, const double* gamma1,
                 const double* gamma2, const double* nrm, const double* nvec,
                 const double* xyz, const double* d_psi, const double* d_pi,
                 const double* d_phi, const double* dt_psi, const double* dt_pi,
                 const double* dt_phi, double* out) {
  // ConstraintPreservingSphericalRadiation::dg_time_derivative,
  // ConstraintPreservingSphericalRadiation.cpp:40-156 (static mesh)
  if (npts < 0 || !psi || !pi || !phi || !lapse || !shift || !gamma1 || !gamma2 || !nrm ||
      !nvec || !xyz || !d_psi || !d_pi || !d_phi || !dt_psi || !dt_pi || !dt_phi || !out)
    return -1;
  (void)d_pi;
  const int n = npts;
  for (int p = 0; p < n; ++p) {
    const double r = std::sqrt(xyz[p] * xyz[p] + xyz[n + p] * xyz[n + p] +
                               xyz[2 * n + p] * xyz[2 * n + p]);
    const double inv_r = 1.0 / r;
    double bn = 0.0;
    for (int i = 0; i < 3; ++i) bn += shift[i * n + p] * nrm[i * n + p];
    const double c0 = -(1.0 + gamma1[p]) * bn, c1 = -bn;
    double dpsi_c = nvec[p] * (d_psi[p] - phi[p]);
    for (int i = 1; i < 3; ++i) dpsi_c += nvec[i * n + p] * (d_psi[i * n + p] - phi[i * n + p]);
    dpsi_c *= std::min(0.0, c0);
    out[p] = dpsi_c;
    for (int i = 0; i < 3; ++i) {
      double v = nvec[p] * (d_phi[(3 * 0 + i) * n + p] - d_phi[(3 * i + 0) * n + p]);
      for (int j = 1; j < 3; ++j)
        v += nvec[j * n + p] * (d_phi[(3 * j + i) * n + p] - d_phi[(3 * i + j) * n + p]);
      out[(2 + i) * n + p] = v * std::min(0.0, c1);
    }
    double dpi_c = (2.0 * inv_r * psi[p] + 4.0 * dt_psi[p]) * inv_r;
    for (int i = 0; i < 3; ++i) {
      dpi_c += nvec[i * n + p] * (2.0 * dt_phi[i * n + p] + 4.0 * inv_r * phi[i * n + p]) +
               shift[i * n + p] * dt_phi[i * n + p];
      for (int j = 0; j < 3; ++j)
        dpi_c += nvec[i * n + p] * nvec[j * n + p] * d_phi[(3 * i + j) * n + p];
    }
    dpi_c /= lapse[p];
    dpi_c += gamma2[p] * dpsi_c - dt_pi[p];
    out[n + p] = dpi_c;
  }
  return 0;
}

}  // extern "C"

// ======================= Legendre-Gauss quadrature =======================
namespace {

// P_n(x) and P_n'(x) by the three-term recurrence (Kopriva algorithm 22)
void legendre_and_derivative(int n, double x, double* L, double* dL) {
  double lm2 = 1.0, lm1 = x, dm2 = 0.0, dm1 = 1.0;
  if (n == 0) {
    *L = 1.0;
    *dL = 0.0;
    return;
  }
  for (int k = 2; k <= n; ++k) {
    const double l = ((2.0 * k - 1.0) * x * lm1 - (k - 1.0) * lm2) / k;
    const double d = dm2 + (2.0 * k - 1.0) * lm1;
    lm2 = lm1;
    lm1 = l;
    dm2 = dm1;
    dm1 = d;
  }
  *L = lm1;
  *dL = dm1;
}

// root of P_n on a sign-changing bracket, bisected to adjacent doubles (the
// reference runs TOMS748 to 6e-16 on the same brackets, Legendre.cpp:128-134)
double lg_root(int n, double a, double b) {
  double fa, fb, d;
  legendre_and_derivative(n, a, &fa, &d);
  legendre_and_derivative(n, b, &fb, &d);
  if (fa == 0.0) return a;
  if (fb == 0.0) return b;
  for (int it = 0; it < 200; ++it) {
    const double m = 0.5 * (a + b);
    if (m <= std::min(a, b) || m >= std::max(a, b)) break;
    double fm;
    legendre_and_derivative(n, m, &fm, &d);
    if (fm == 0.0) return m;
    if ((fm < 0) == (fa < 0)) {
      a = m;
      fa = fm;
    } else {
      b = m;
    }
  }
  return 0.5 * (a + b);
}

struct Gauss1d {
  int n = 0;
  double x[kMaxN], w[kMaxN], bw[kMaxN];
  double D[kMaxN * kMaxN];
  double lo[kMaxN], hi[kMaxN];            // interpolation to xi = -1, +1
  double lift_lo[kMaxN], lift_hi[kMaxN];  // boundary_lifting_term
};

const Gauss1d& gauss(int n) {
  static Gauss1d table[kMaxN + 1];
  static bool init = [] {
    for (int m = 2; m <= kMaxN; ++m) {
      Gauss1d& g = table[m];
      g.n = m;
      orc_lg(m, g.x, g.w);
      for (int j = 0; j < m; ++j) g.bw[j] = 1.0;
      for (int j = 1; j < m; ++j)
        for (int k = 0; k < j; ++k) {
          g.bw[k] *= g.x[k] - g.x[j];
          g.bw[j] *= g.x[j] - g.x[k];
        }
      for (int j = 0; j < m; ++j) g.bw[j] = 1.0 / g.bw[j];
      for (int i = 0; i < m; ++i) {
        double diag = 0.0;
        for (int j = 0; j < m; ++j)
          if (i != j) {
            g.D[i * m + j] = g.bw[j] / (g.bw[i] * (g.x[i] - g.x[j]));
            diag -= g.D[i * m + j];
          }
        g.D[i * m + i] = diag;
      }
      // barycentric interpolation to the end points (no node sits there)
      for (int side = 0; side < 2; ++side) {
        const double t = side ? 1.0 : -1.0;
        double* row = side ? g.hi : g.lo;
        double sum = 0.0;
        for (int j = 0; j < m; ++j) {
          row[j] = g.bw[j] / (t - g.x[j]);
          sum += row[j];
        }
        for (int j = 0; j < m; ++j) row[j] /= sum;
      }
      for (int j = 0; j < m; ++j) {
        g.lift_lo[j] = g.lo[j] / g.w[j];
        g.lift_hi[j] = g.hi[j] / g.w[j];
      }
    }
    return true;
  }();
  (void)init;
  return table[n];
}

}  // namespace

extern "C" {

int orc_lg(int n, double* x, double* w) {
  // compute_collocation_points_and_weights<Legendre, Gauss>, Legendre.cpp:106-149
  // (Kopriva algorithm 23): roots of P_n, w = 2 / ((1 - x^2) P_n'(x)^2)
  if (n < 2 || n > kMaxN || !x || !w) return -1;
  const int p = n - 1;  // polynomial degree
  if (p == 1) {
    x[0] = -std::sqrt(1.0 / 3.0);
    x[1] = -x[0];
    w[0] = w[1] = 1.0;
    return 0;
  }
  for (int j = 0; j <= (p + 1) / 2 - 1; ++j) {
    const double r = lg_root(n, -std::cos((2.0 * j) * M_PI / (2.0 * p + 2.0)),
                             -std::cos((2.0 * j + 2.0) * M_PI / (2.0 * p + 2.0)));
    double L, dL;
    legendre_and_derivative(n, r, &L, &dL);
    x[j] = r;
    x[p - j] = -r;
    w[j] = w[p - j] = 2.0 / (1.0 - r * r) / (dL * dL);
  }
  if (p % 2 == 0) {
    double L, dL;
    legendre_and_derivative(n, 0.0, &L, &dL);
    x[p / 2] = 0.0;
    w[p / 2] = 2.0 / (dL * dL);
  }
  return 0;
}

int orc_lg_diff_matrix(int n, double* D) {
  // differentiation_matrix<Legendre, Gauss>: the barycentric formula of
  // Spectral.cpp:431-444 on the Gauss nodes
  if (n < 2 || n > kMaxN || !D) return -1;
  std::memcpy(D, gauss(n).D, sizeof(double) * n * n);
  return 0;
}

int orc_lg_boundary(int n, double* lo, double* hi, double* lift_lo, double* lift_hi) {
  // boundary_interpolation_matrices and boundary_lifting_term,
  // Spectral.cpp:676-790
  if (n < 2 || n > kMaxN) return -1;
  const Gauss1d& g = gauss(n);
  for (int j = 0; j < n; ++j) {
    if (lo) lo[j] = g.lo[j];
    if (hi) hi[j] = g.hi[j];
    if (lift_lo) lift_lo[j] = g.lift_lo[j];
    if (lift_hi) lift_hi[j] = g.lift_hi[j];
  }
  return 0;
}

}  // extern "C"

// Gauss-point boundary corrections of element e (uniform extent n):
// ApplyBoundaryCorrections.hpp:938-987 with lift_boundary_terms_gauss_points,
// LiftFromBoundary.cpp:20-140.  Each side interpolates its own volume data to
// the shared face (boundary_interpolation_matrices); on an affine element
// det(inverse Jacobian) x det(Jacobian on the face) = 1, so
//   dt(line point i) -= |n| lift_i(side) correction(face point).
namespace {
void boundary_terms_gauss(const Mesh& m, const double* u, double gamma2, int64_t e,
                          double* dt) {
  const int n = m.elem_n[e];
  const int64_t np = (int64_t)n * n * n;
  const int nf = n * n;
  const Gauss1d& g = gauss(n);
  for (int dir = 0; dir < 6; ++dir) {
    const int d = dir / 2;
    const bool upper = dir % 2;
    const int64_t nb = m.nbr[6 * e + dir];
    auto face_package = [&](int64_t el, bool up, double sign, double* pkg, double* mag) {
      const double* ue = u + m.off[el];
      const double* I = up ? g.hi : g.lo;
      std::vector<double> psi(nf), pi(nf), phi(3 * nf), g2(nf, gamma2), nrm(3 * nf, 0.0);
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const int f = a + n * b;
          double acc[kVars] = {0, 0, 0, 0, 0};
          for (int i = 0; i < n; ++i) {
            const int64_t vi = volume_index(n, d, i, a, b);
            for (int v = 0; v < kVars; ++v) acc[v] += I[i] * ue[v * np + vi];
          }
          psi[f] = acc[0];
          pi[f] = acc[1];
          for (int c = 0; c < 3; ++c) phi[c * nf + f] = acc[2 + c];
          nrm[d * nf + f] = sign;  // sign * invjac / |invjac|
          mag[f] = m.geom[el].invjac[d];
        }
      double ms;
      orc_package(nf, psi.data(), pi.data(), phi.data(), g2.data(), nrm.data(), nullptr, pkg,
                  &ms);
    };
    std::vector<double> pi_((size_t)kPkg * nf), pe((size_t)kPkg * nf), mi(nf), me(nf);
    face_package(e, upper, upper ? 1.0 : -1.0, pi_.data(), mi.data());
    face_package(nb, !upper, upper ? -1.0 : 1.0, pe.data(), me.data());
    std::vector<double> bc((size_t)kVars * nf);
    orc_boundary_terms(nf, pi_.data(), pe.data(), bc.data());
    const double* lift = upper ? g.lift_hi : g.lift_lo;
    for (int b = 0; b < n; ++b)
      for (int a = 0; a < n; ++a) {
        const int f = a + n * b;
        for (int i = 0; i < n; ++i) {
          const int64_t vi = volume_index(n, d, i, a, b);
          const double fac = mi[f] * lift[i];
          for (int v = 0; v < kVars; ++v) dt[v * np + vi] -= fac * bc[(size_t)v * nf + f];
        }
      }
  }
}
}  // namespace

extern "C" {

int orc_coords_gauss(int n_inst, const OrcBrick* br, int n, double* xyz) {
  if (n_inst < 1 || !br || n < 2 || n > kMaxN || !xyz) return -1;
  const int64_t E = orc_num_elements(n_inst, br);
  std::vector<int32_t> en(E, n);
  Mesh m;
  build_mesh(&m, n_inst, br, en.data());
  const Gauss1d& g = gauss(n);
  const int64_t np = (int64_t)n * n * n;
  for (int64_t e = 0; e < E; ++e)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int64_t p = i + n * (j + (int64_t)n * k);
          const int id[3] = {i, j, k};
          for (int c = 0; c < 3; ++c)
            xyz[e * 3 * np + c * np + p] =
                m.geom[e].lo[c] + (g.x[id[c]] + 1.0) * (0.5 * m.geom[e].h[c]);
        }
  return 0;
}

int orc_rhs_gauss(int n_inst, const OrcBrick* br, int n, double gamma2, const double* u,
                  double* dudt, int n_threads) {
  if (n_inst < 1 || !br || n < 2 || n > kMaxN || !u || !dudt) return -1;
  const int64_t E = orc_num_elements(n_inst, br);
  std::vector<int32_t> en(E, n);
  Mesh m;
  build_mesh(&m, n_inst, br, en.data());
  const Gauss1d& g = gauss(n);
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t e = 0; e < E; ++e) {
    volume_terms(m, u, gamma2, e, dudt + m.off[e], g.D);
    boundary_terms_gauss(m, u, gamma2, e, dudt + m.off[e]);
  }
  (void)n_threads;
  return 0;
}

int orc_evolve_gauss(int n_inst, const OrcBrick* br, int n, double gamma2, double dt,
                     int n_steps, double* u, int n_threads) {
  if (n_inst < 1 || !br || n < 2 || n > kMaxN || !u || n_steps < 0) return -1;
  const int64_t size = orc_num_elements(n_inst, br) * 5 * (int64_t)n * n * n;
  std::vector<double> u0(size), u1(size), du(size);
  for (int st = 0; st < n_steps; ++st) {
    std::memcpy(u0.data(), u, size * sizeof(double));
    orc_rhs_gauss(n_inst, br, n, gamma2, u0.data(), du.data(), n_threads);
    orc_rk3_substep(size, 0, dt, u0.data(), u0.data(), du.data(), u1.data());
    orc_rhs_gauss(n_inst, br, n, gamma2, u1.data(), du.data(), n_threads);
    orc_rk3_substep(size, 1, dt, u0.data(), u1.data(), du.data(), u);
    std::memcpy(u1.data(), u, size * sizeof(double));
    orc_rhs_gauss(n_inst, br, n, gamma2, u1.data(), du.data(), n_threads);
    orc_rk3_substep(size, 2, dt, u0.data(), u1.data(), du.data(), u);
  }
  return 0;
}

}  // extern "C"

// ======================= h-nonconforming refined bricks =======================
namespace {

struct RElem {
  int block, level, seg[3];
  double lo[3], h[3];
};

struct RMesh {
  int n = 0;
  std::vector<RElem> el;
  std::vector<int32_t> nbr;    // 4 per face
  std::vector<int32_t> msize;  // 2 per slot
  std::vector<uint64_t> ids;
};

// ChildSize codes: 0 Full, 1 LowerHalf, 2 UpperHalf
int build_refined(const OrcRefinedBrick& b, RMesh* m) {
  const int nb = b.blocks[0] * b.blocks[1] * b.blocks[2];
  std::vector<int64_t> first(nb + 1, 0);
  for (int k = 0; k < nb; ++k) {
    const int L = b.level[k];
    if (L < 0 || L > 8) return -1;
    first[k + 1] = first[k] + ((int64_t)1 << (3 * L));
  }
  const int64_t E = first[nb];
  m->el.resize(E);
  m->ids.resize(E);
  auto block_xyz = [&](int k, int q[3]) {
    q[0] = k % b.blocks[0];
    q[1] = (k / b.blocks[0]) % b.blocks[1];
    q[2] = k / (b.blocks[0] * b.blocks[1]);
  };
  auto block_of = [&](const int q[3]) { return q[0] + b.blocks[0] * (q[1] + b.blocks[1] * q[2]); };
  auto elem_of = [&](int k, const int seg[3]) {
    const int L = b.level[k];
    return first[k] + (((int64_t)seg[0] << (2 * L)) | ((int64_t)seg[1] << L) | seg[2]);
  };
  for (int k = 0; k < nb; ++k) {
    const int L = b.level[k];
    int q[3];
    block_xyz(k, q);
    for (int64_t w = 0; w < ((int64_t)1 << (3 * L)); ++w) {
      RElem& r = m->el[first[k] + w];
      r.block = k;
      r.level = L;
      r.seg[2] = (int)(w & ((1 << L) - 1));
      r.seg[1] = (int)((w >> L) & ((1 << L) - 1));
      r.seg[0] = (int)(w >> (2 * L));
      for (int d = 0; d < 3; ++d) {
        const double W = (b.hi[d] - b.lo[d]) / b.blocks[d];
        r.h[d] = W / (1 << L);
        r.lo[d] = b.lo[d] + W * q[d] + r.h[d] * r.seg[d];
      }
      m->ids[first[k] + w] = (uint64_t)(k & 0xff) | ((uint64_t)r.seg[0] << 16) |
                             ((uint64_t)L << 28) | ((uint64_t)r.seg[1] << 32) |
                             ((uint64_t)L << 44) | ((uint64_t)r.seg[2] << 48) |
                             ((uint64_t)L << 60);
    }
  }
  m->nbr.assign(E * 24, -1);
  m->msize.assign(E * 48, 0);
  for (int64_t e = 0; e < E; ++e) {
    const RElem& r = m->el[e];
    const int L = r.level;
    for (int dir = 0; dir < 6; ++dir) {
      const int d = dir / 2;
      const bool up = dir % 2;
      int32_t* nbr = &m->nbr[(6 * e + dir) * 4];
      int32_t* ms = &m->msize[(6 * e + dir) * 8];
      const int t0 = d == 0 ? 1 : 0, t1 = d == 2 ? 1 : 2;  // transverse dims, ascending
      const int last = (1 << L) - 1;
      if ((up && r.seg[d] < last) || (!up && r.seg[d] > 0)) {
        int sg[3] = {r.seg[0], r.seg[1], r.seg[2]};
        sg[d] += up ? 1 : -1;
        nbr[0] = (int32_t)elem_of(r.block, sg);
        continue;
      }
      int q[3];
      block_xyz(r.block, q);
      q[d] = (q[d] + (up ? 1 : b.blocks[d] - 1)) % b.blocks[d];
      const int k2 = block_of(q);
      const int L2 = b.level[k2];
      if (L2 == L) {
        int sg[3] = {r.seg[0], r.seg[1], r.seg[2]};
        sg[d] = up ? 0 : last;
        nbr[0] = (int32_t)elem_of(k2, sg);
      } else if (L2 == L + 1) {
        for (int c = 0; c < 4; ++c) {
          int sg[3] = {0, 0, 0};
          sg[d] = up ? 0 : (1 << L2) - 1;
          sg[t0] = 2 * r.seg[t0] + (c & 1);
          sg[t1] = 2 * r.seg[t1] + (c >> 1);
          nbr[c] = (int32_t)elem_of(k2, sg);
          ms[2 * c] = 1 + (c & 1);
          ms[2 * c + 1] = 1 + (c >> 1);
        }
      } else if (L2 == L - 1) {
        int sg[3] = {0, 0, 0};
        sg[d] = up ? 0 : (1 << L2) - 1;
        sg[t0] = r.seg[t0] >> 1;
        sg[t1] = r.seg[t1] >> 1;
        nbr[0] = (int32_t)elem_of(k2, sg);
      } else {
        return -2;
      }
    }
  }
  return 0;
}

// Legendre-Gauss nodes/weights of a high-order rule for exact projections
void gauss_rule(int m, double* x, double* w) { orc_lg(m, x, w); }

}  // namespace

extern "C" {

int orc_proj_half(int n, int upper, double* P, double* R) {
  // parent -> child: interpolation to x = (xi -+ 1) / 2 (Projection.cpp:341-372);
  // child -> parent: L2 projection of the half-supported child polynomial
  // onto the parent's Legendre modes, c_k = (2k+1)/4 int P_k(x(xi)) f(xi) dxi,
  // the integral of Projection.cpp:140-220 evaluated with a Gauss rule exact
  // for its degree
  if (n < 2 || n > kMaxN) return -1;
  const Spectral1d& sp = spectral(n);
  const double shift = upper ? 1.0 : -1.0;
  if (P) {
    double t[kMaxN];
    for (int i = 0; i < n; ++i) t[i] = 0.5 * (sp.x[i] + shift);
    orc_interp_matrix(n, n, t, P);
  }
  if (R) {
    double V[kMaxN * kMaxN], Vi[kMaxN * kMaxN];
    orc_vandermonde(n, V);
    orc_inv_vandermonde(n, Vi);
    const int m = n + 1;  // degree 2n - 2 integrands
    double gx[kMaxN + 1], gw[kMaxN + 1];
    gauss_rule(m, gx, gw);
    double S[kMaxN * kMaxN];  // S[k][j]
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j) {
        double acc = 0.0;
        for (int q = 0; q < m; ++q)
          acc += gw[q] * legendre_p(k, 0.5 * (gx[q] + shift)) * legendre_p(j, gx[q]);
        S[k * n + j] = (2.0 * k + 1.0) / 4.0 * acc;
      }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double acc = 0.0;
        for (int k = 0; k < n; ++k) {
          double vs = 0.0;
          for (int l = 0; l < n; ++l) vs += S[k * n + l] * Vi[l * n + j];
          acc += V[i * n + k] * vs;
        }
        R[i * n + j] = acc;
      }
  }
  return 0;
}

int64_t orc_refined_num_elements(const OrcRefinedBrick* b) {
  if (!b || !b->level) return -1;
  int64_t c = 0;
  for (int k = 0; k < b->blocks[0] * b->blocks[1] * b->blocks[2]; ++k)
    c += (int64_t)1 << (3 * b->level[k]);
  return c;
}

int orc_refined_index_maps(const OrcRefinedBrick* b, uint64_t* ids, int32_t* nbr,
                           int32_t* msize) {
  if (!b || !b->level) return -1;
  RMesh m;
  const int rc = build_refined(*b, &m);
  if (rc) return rc;
  if (ids) std::memcpy(ids, m.ids.data(), m.ids.size() * sizeof(uint64_t));
  if (nbr) std::memcpy(nbr, m.nbr.data(), m.nbr.size() * sizeof(int32_t));
  if (msize) std::memcpy(msize, m.msize.data(), m.msize.size() * sizeof(int32_t));
  return 0;
}

int orc_refined_coords(const OrcRefinedBrick* b, int n, double* xyz) {
  if (!b || !b->level || n < 2 || n > kMaxN || !xyz) return -1;
  RMesh m;
  if (build_refined(*b, &m)) return -1;
  const Spectral1d& sp = spectral(n);
  const int64_t np = (int64_t)n * n * n;
  for (size_t e = 0; e < m.el.size(); ++e)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int id[3] = {i, j, k};
          for (int c = 0; c < 3; ++c)
            xyz[e * 3 * np + c * np + i + n * (j + (int64_t)n * k)] =
                m.el[e].lo[c] + (sp.x[id[c]] + 1.0) * 0.5 * m.el[e].h[c];
        }
  return 0;
}

}  // extern "C"

namespace {

// out(a', b') = sum_a sum_b M0(a', a) M1(b', b) in(a, b), a fastest; a null
// matrix is the identity
void apply_face_2d(int n, const double* M0, const double* M1, int nfields, const double* in,
                   double* out) {
  std::vector<double> tmp((size_t)n * n);
  for (int f = 0; f < nfields; ++f) {
    const double* src = in + (size_t)f * n * n;
    double* dst = out + (size_t)f * n * n;
    for (int b = 0; b < n; ++b)
      for (int ap = 0; ap < n; ++ap) {
        double acc = 0.0;
        if (M0)
          for (int a = 0; a < n; ++a) acc += M0[ap * n + a] * src[a + n * b];
        else
          acc = src[ap + n * b];
        tmp[ap + n * b] = acc;
      }
    for (int bp = 0; bp < n; ++bp)
      for (int ap = 0; ap < n; ++ap) {
        double acc = 0.0;
        if (M1)
          for (int b = 0; b < n; ++b) acc += M1[bp * n + b] * tmp[ap + n * b];
        else
          acc = tmp[ap + n * bp];
        dst[ap + n * bp] = acc;
      }
  }
}

void make_mesh_view(const RMesh& rm, int n, const OrcRefinedBrick& b, Mesh* m,
                    std::vector<int32_t>* elem_n) {
  const int64_t E = (int64_t)rm.el.size();
  elem_n->assign(E, n);
  m->n_inst = 1;
  m->br = nullptr;
  m->n_elem = E;
  m->elem_n = elem_n->data();
  m->geom.resize(E);
  m->off.resize(E + 1);
  orc_offsets(E, elem_n->data(), m->off.data());
  for (int64_t e = 0; e < E; ++e) {
    ElemGeom& g = m->geom[e];
    g.inst = 0;
    for (int d = 0; d < 3; ++d) {
      g.ijk[d] = rm.el[e].seg[d];
      g.lo[d] = rm.el[e].lo[d];
      g.h[d] = rm.el[e].h[d];
      g.invjac[d] = 2.0 / g.h[d];
    }
  }
  (void)b;
}

// ApplyBoundaryCorrections.hpp:723-1050 with h-nonconforming mortars: per
// mortar, both packages projected face -> mortar (identity where the mortar
// is the face), dg_boundary_terms, mortar -> face (identity, or the
// half-interval restriction), lift_flux on the GLL face.
void boundary_terms_refined(const Mesh& m, const RMesh& rm, const double* u, double gamma2,
                            int64_t e, double* dt) {
  const int n = m.elem_n[e];
  const int64_t np = (int64_t)n * n * n;
  const int nf = n * n;
  double P[2][kMaxN * kMaxN], R[2][kMaxN * kMaxN];
  orc_proj_half(n, 0, P[0], R[0]);
  orc_proj_half(n, 1, P[1], R[1]);
  for (int dir = 0; dir < 6; ++dir) {
    const int d = dir / 2;
    const bool upper = dir % 2;
    const int t0 = d == 0 ? 1 : 0, t1 = d == 2 ? 1 : 2;
    std::vector<double> pki((size_t)kPkg * nf), mag(nf), pke((size_t)kPkg * nf), mage(nf);
    package_face(m, u, gamma2, e, dir, pki.data(), mag.data());
    std::vector<double> bc_face((size_t)kVars * nf, 0.0);
    for (int k = 0; k < 4; ++k) {
      const int32_t nb = rm.nbr[(6 * e + dir) * 4 + k];
      if (nb < 0) continue;
      const int32_t* ms = &rm.msize[((6 * e + dir) * 4 + k) * 2];
      package_face(m, u, gamma2, nb, dir ^ 1, pke.data(), mage.data());
      // mortar_size(neighbour, self): halves where this element is the
      // neighbour's child (the neighbour is one level coarser)
      int mse[2] = {0, 0};
      if (rm.el[nb].level == rm.el[e].level - 1) {
        mse[0] = 1 + (rm.el[e].seg[t0] & 1);
        mse[1] = 1 + (rm.el[e].seg[t1] & 1);
      }
      std::vector<double> mi((size_t)kPkg * nf), me((size_t)kPkg * nf);
      apply_face_2d(n, ms[0] ? P[ms[0] - 1] : nullptr, ms[1] ? P[ms[1] - 1] : nullptr, kPkg,
                    pki.data(), mi.data());
      apply_face_2d(n, mse[0] ? P[mse[0] - 1] : nullptr, mse[1] ? P[mse[1] - 1] : nullptr,
                    kPkg, pke.data(), me.data());
      std::vector<double> bcm((size_t)kVars * nf), bcf((size_t)kVars * nf);
      orc_boundary_terms(nf, mi.data(), me.data(), bcm.data());
      apply_face_2d(n, ms[0] ? R[ms[0] - 1] : nullptr, ms[1] ? R[ms[1] - 1] : nullptr, kVars,
                    bcm.data(), bcf.data());
      // lift this mortar's correction (LiftFlux.hpp:57-61)
      const double slice_factor = -0.5 * static_cast<double>(n * (n - 1));
      const int slice = upper ? n - 1 : 0;
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) {
          const int f = a + n * b;
          const int64_t vi = volume_index(n, d, slice, a, b);
          const double fac = slice_factor * mag[f];
          for (int v = 0; v < kVars; ++v) dt[v * np + vi] += bcf[(size_t)v * nf + f] * fac;
        }
    }
  }
}

}  // namespace

extern "C" {

int orc_refined_rhs(const OrcRefinedBrick* b, int n, double gamma2, const double* u,
                    double* dudt, int n_threads) {
  if (!b || !b->level || n < 2 || n > kMaxN || !u || !dudt) return -1;
  RMesh rm;
  if (build_refined(*b, &rm)) return -2;
  Mesh m;
  std::vector<int32_t> en;
  make_mesh_view(rm, n, *b, &m, &en);
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t e = 0; e < m.n_elem; ++e) {
    volume_terms(m, u, gamma2, e, dudt + m.off[e]);
    boundary_terms_refined(m, rm, u, gamma2, e, dudt + m.off[e]);
  }
  (void)n_threads;
  return 0;
}

int orc_refined_evolve(const OrcRefinedBrick* b, int n, double gamma2, double dt, int n_steps,
                       double* u, int n_threads) {
  const int64_t E = orc_refined_num_elements(b);
  if (E < 0 || n < 2 || n > kMaxN || !u || n_steps < 0) return -1;
  const int64_t size = E * 5 * (int64_t)n * n * n;
  std::vector<double> u0(size), u1(size), du(size);
  for (int st = 0; st < n_steps; ++st) {
    std::memcpy(u0.data(), u, size * sizeof(double));
    int rc = orc_refined_rhs(b, n, gamma2, u0.data(), du.data(), n_threads);
    if (rc) return rc;
    orc_rk3_substep(size, 0, dt, u0.data(), u0.data(), du.data(), u1.data());
    orc_refined_rhs(b, n, gamma2, u1.data(), du.data(), n_threads);
    orc_rk3_substep(size, 1, dt, u0.data(), u1.data(), du.data(), u);
    std::memcpy(u1.data(), u, size * sizeof(double));
    orc_refined_rhs(b, n, gamma2, u1.data(), du.data(), n_threads);
    orc_rk3_substep(size, 2, dt, u0.data(), u1.data(), du.data(), u);
  }
  return 0;
}

}  // extern "C"

// ======================= exponential filter =======================
extern "C" {

int orc_exponential_filter(int n, double alpha, int half_power, double* F) {
  // exponential_filter, Filtering.cpp:18-31: modal_to_nodal * diag * nodal_to_modal
  if (n < 2 || n > kMaxN || !F || half_power < 0) return -1;
  double V[kMaxN * kMaxN], Vi[kMaxN * kMaxN];
  orc_vandermonde(n, V);
  orc_inv_vandermonde(n, Vi);
  const double order = n - 1.0;
  double d[kMaxN];
  for (int k = 0; k < n; ++k) d[k] = std::exp(-alpha * std::pow(k / order, 2.0 * half_power));
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double acc = 0.0;
      for (int k = 0; k < n; ++k) acc += V[i * n + k] * d[k] * Vi[k * n + j];
      F[i * n + j] = acc;
    }
  return 0;
}

int orc_filter_elements(int64_t n_elem, const int32_t* elem_n, double alpha, int half_power,
                        double* u) {
  // dg::Actions::Filter, FilterAction.hpp:109-180: apply_matrices with the
  // filter matrix of each dimension on every evolved variable
  if (n_elem < 0 || !elem_n || !u) return -1;
  std::vector<int64_t> off(n_elem + 1, 0);
  for (int64_t e = 0; e < n_elem; ++e) {
    const int64_t n = elem_n[e];
    if (n < 2 || n > kMaxN) return -1;
    off[e + 1] = off[e] + 5 * n * n * n;
  }
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < n_elem; ++e) {
    const int n = elem_n[e];
    const int64_t np = (int64_t)n * n * n;
    double F[kMaxN * kMaxN];
    orc_exponential_filter(n, alpha, half_power, F);
    std::vector<double> tmp(np);
    for (int v = 0; v < 5; ++v) {
      double* f = u + off[e] + v * np;
      for (int d = 0; d < 3; ++d) {
        for (int k = 0; k < n; ++k)
          for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
              const int idx[3] = {i, j, k};
              double acc = 0.0;
              for (int q = 0; q < n; ++q) {
                int id2[3] = {i, j, k};
                id2[d] = q;
                acc += F[idx[d] * n + q] * f[id2[0] + n * (id2[1] + (int64_t)n * id2[2])];
              }
              tmp[i + n * (j + (int64_t)n * k)] = acc;
            }
        std::memcpy(f, tmp.data(), np * sizeof(double));
      }
    }
  }
  return 0;
}

}  // extern "C"

// ======================= ObserveNorms =======================
extern "C" {

// norms over elements of one extent n, det_jac: one value per point
int orc_shell_observe_norms_impl(int64_t n_elem, int n, const double* det_jac, const double* u,
                                 const double* subtract, double* out) {
  if (n_elem < 0 || n < 2 || n > kMaxN || !det_jac || !u || !out) return -1;
  const Spectral1d& sp = spectral(n);
  const int64_t np = (int64_t)n * n * n;
  double mx[5], mn[5], sq[5], isq[5], iv[5], vol = 0.0;
  for (int v = 0; v < 5; ++v) {
    mx[v] = -std::numeric_limits<double>::infinity();
    mn[v] = std::numeric_limits<double>::infinity();
    sq[v] = isq[v] = iv[v] = 0.0;
  }
  for (int64_t e = 0; e < n_elem; ++e)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int64_t p = i + n * (j + (int64_t)n * k);
          const double w = sp.w[i] * sp.w[j] * sp.w[k] * det_jac[e * np + p];
          vol += w;
          for (int v = 0; v < 5; ++v) {
            double x = u[e * 5 * np + v * np + p];
            if (subtract) x -= subtract[e * 5 * np + v * np + p];
            mx[v] = std::max(mx[v], x);
            mn[v] = std::min(mn[v], x);
            sq[v] += x * x;
            isq[v] += w * x * x;
            iv[v] += w * x;
          }
        }
  const double pts = (double)(n_elem * np);
  for (int v = 0; v < 5; ++v) {
    out[5 * v + 0] = mx[v];
    out[5 * v + 1] = mn[v];
    out[5 * v + 2] = std::sqrt(sq[v] / pts);
    out[5 * v + 3] = std::sqrt(isq[v] / vol);
    out[5 * v + 4] = iv[v];
  }
  out[25] = pts;
  out[26] = vol;
  return 0;
}

int orc_observe_norms(int n_inst, const OrcBrick* br, const int32_t* elem_n, const double* u,
                      const double* subtract, double* out) {
  if (n_inst < 1 || !br || !elem_n || !u || !out) return -1;
  Mesh m;
  build_mesh(&m, n_inst, br, elem_n);
  double mx[5], mn[5], sq[5], isq[5], iv[5], vol = 0.0, pts = 0.0;
  for (int v = 0; v < 5; ++v) {
    mx[v] = -std::numeric_limits<double>::infinity();
    mn[v] = std::numeric_limits<double>::infinity();
    sq[v] = isq[v] = iv[v] = 0.0;
  }
  int64_t pos = 0;
  for (int64_t e = 0; e < m.n_elem; ++e) {
    const int n = elem_n[e];
    const int64_t np = (int64_t)n * n * n;
    const Spectral1d& sp = spectral(n);
    const ElemGeom& g = m.geom[e];
    const double dj = 0.125 * g.h[0] * g.h[1] * g.h[2];
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int64_t p = i + n * (j + (int64_t)n * k);
          const double w = sp.w[i] * sp.w[j] * sp.w[k] * dj;
          vol += w;
          for (int v = 0; v < 5; ++v) {
            double x = u[pos + v * np + p];
            if (subtract) x -= subtract[pos + v * np + p];
            mx[v] = std::max(mx[v], x);
            mn[v] = std::min(mn[v], x);
            sq[v] += x * x;
            isq[v] += w * x * x;
            iv[v] += w * x;
          }
        }
    pts += (double)np;
    pos += 5 * np;
  }
  for (int v = 0; v < 5; ++v) {
    out[5 * v + 0] = mx[v];
    out[5 * v + 1] = mn[v];
    out[5 * v + 2] = std::sqrt(sq[v] / pts);
    out[5 * v + 3] = std::sqrt(isq[v] / vol);
    out[5 * v + 4] = iv[v];
  }
  out[25] = pts;
  out[26] = vol;
  return 0;
}

}  // extern "C"

// ======================= spherical shell (configuration 5) =======================
namespace {

// global[i] = sign[b][i] * wedge_frame[perm[b][i]]: discrete_rotation of the
// six orientations of DomainHelpers.cpp:553-578 (+z, -z, +y, -y, +x, -x)
const int kShellPerm[6][3] = {{0, 1, 2}, {0, 1, 2}, {0, 2, 1}, {0, 2, 1}, {2, 0, 1}, {2, 0, 1}};
const double kShellSign[6][3] = {{1, 1, 1}, {1, -1, -1}, {1, 1, -1},
                                 {1, -1, 1}, {1, 1, 1},  {-1, -1, 1}};

struct ShellLayout {
  int per_axis[3];  // elements per block along xi, eta, zeta
  int L[3];
  int64_t per_block;
};

ShellLayout shell_layout(const OrcShell& s) {
  ShellLayout l;
  l.L[0] = l.L[1] = s.ref_ang;
  l.L[2] = s.ref_rad;
  for (int d = 0; d < 3; ++d) l.per_axis[d] = 1 << l.L[d];
  l.per_block = (int64_t)l.per_axis[0] * l.per_axis[1] * l.per_axis[2];
  return l;
}

// block and segments of element e (x-outer, z-inner inside a block)
void shell_element(const ShellLayout& l, int64_t e, int* block, int seg[3]) {
  *block = (int)(e / l.per_block);
  int64_t w = e % l.per_block;
  seg[2] = (int)(w % l.per_axis[2]);
  w /= l.per_axis[2];
  seg[1] = (int)(w % l.per_axis[1]);
  seg[0] = (int)(w / l.per_axis[1]);
}

// Wedge<3> (Wedge.cpp:476-536) composed with the element map: coordinates
// and the Jacobian dx^i/dxi_e^a (jac[3*i + a]) at element logical xi_e.
void shell_map(const OrcShell& s, const ShellLayout& l, int block, const int seg[3],
               const double xe[3], double x[3], double jac[9]) {
  double xb[3], scale[3];
  for (int d = 0; d < 3; ++d) {
    scale[d] = 1.0 / l.per_axis[d];
    xb[d] = -1.0 + (2.0 * seg[d] + 1.0 + xe[d]) * scale[d];
  }
  const double a = std::tan(M_PI_4 * xb[0]), b = std::tan(M_PI_4 * xb[1]);
  const double rho2 = 1.0 + a * a + b * b, rho = std::sqrt(rho2), rho3 = rho2 * rho;
  const double z0 = 0.5 * std::log(s.r_outer * s.r_inner);
  const double k = 0.5 * std::log(s.r_outer / s.r_inner);
  const double r = std::exp(z0 + k * xb[2]);
  const double wf[3] = {r * a / rho, r * b / rho, r / rho};
  const double da = M_PI_4 * (1.0 + a * a), db = M_PI_4 * (1.0 + b * b);
  const double dxi[3] = {r * da * (1.0 + b * b) / rho3, -r * da * a * b / rho3, -r * da * a / rho3};
  const double deta[3] = {-r * db * a * b / rho3, r * db * (1.0 + a * a) / rho3, -r * db * b / rho3};
  const double dzeta[3] = {k * wf[0], k * wf[1], k * wf[2]};
  for (int i = 0; i < 3; ++i) {
    const int p = kShellPerm[block][i];
    const double sg = kShellSign[block][i];
    x[i] = sg * wf[p];
    jac[3 * i + 0] = sg * dxi[p] * scale[0];
    jac[3 * i + 1] = sg * deta[p] * scale[1];
    jac[3 * i + 2] = sg * dzeta[p] * scale[2];
  }
}

void invert3(const double m[9], double out[9]) {
  const double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8],
               c02 = m[3] * m[7] - m[4] * m[6];
  const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
  const double id = 1.0 / det;
  out[0] = c00 * id;
  out[1] = (m[2] * m[7] - m[1] * m[8]) * id;
  out[2] = (m[1] * m[5] - m[2] * m[4]) * id;
  out[3] = c01 * id;
  out[4] = (m[0] * m[8] - m[2] * m[6]) * id;
  out[5] = (m[2] * m[3] - m[0] * m[5]) * id;
  out[6] = c02 * id;
  out[7] = (m[1] * m[6] - m[0] * m[7]) * id;
  out[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}

// face-point coordinates of element e, direction dir (points a + n*b)
void shell_face_points(const OrcShell& s, const ShellLayout& l, int64_t e, int dir,
                       std::vector<double>* pts) {
  const int n = s.n;
  const Spectral1d& sp = spectral(n);
  int block, seg[3];
  shell_element(l, e, &block, seg);
  const int d = dir / 2;
  const double side = (dir % 2) ? 1.0 : -1.0;
  pts->resize(3 * n * n);
  for (int bb = 0; bb < n; ++bb)
    for (int aa = 0; aa < n; ++aa) {
      double xe[3];
      int fi[2] = {aa, bb}, c = 0;
      for (int q = 0; q < 3; ++q) xe[q] = (q == d) ? side : sp.x[fi[c++]];
      double x[3], jac[9];
      shell_map(s, l, block, seg, xe, x, jac);
      for (int q = 0; q < 3; ++q) (*pts)[3 * (aa + n * bb) + q] = x[q];
    }
}

struct ShellMesh {
  OrcShell s;
  ShellLayout l;
  int64_t E;
  std::vector<double> xyz, ij;     // per element 3*NP, 9*NP
  std::vector<int32_t> nbr, perm;  // 6 per element, 6*N^2 per element
};

void build_shell(const OrcShell& s, ShellMesh* m) {
  m->s = s;
  m->l = shell_layout(s);
  m->E = 6 * m->l.per_block;
  const int n = s.n;
  const int64_t np = (int64_t)n * n * n;
  const Spectral1d& sp = spectral(n);
  m->xyz.assign(3 * np * m->E, 0.0);
  m->ij.assign(9 * np * m->E, 0.0);
  for (int64_t e = 0; e < m->E; ++e) {
    int block, seg[3];
    shell_element(m->l, e, &block, seg);
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int64_t p = i + n * (j + (int64_t)n * k);
          const double xe[3] = {sp.x[i], sp.x[j], sp.x[k]};
          double x[3], jac[9], inv[9];
          shell_map(s, m->l, block, seg, xe, x, jac);
          invert3(jac, inv);  // inv[3*a + i] = d xi^a / d x^i
          for (int q = 0; q < 3; ++q) m->xyz[e * 3 * np + q * np + p] = x[q];
          for (int q = 0; q < 9; ++q) m->ij[e * 9 * np + q * np + p] = inv[q];
        }
  }
  // connectivity: inside a block by segments; across blocks by face centres
  m->nbr.assign(6 * m->E, 0);
  m->perm.assign(6 * (size_t)n * n * m->E, 0);
  std::vector<double> centre(18 * m->E);
  for (int64_t e = 0; e < m->E; ++e) {
    int block, seg[3];
    shell_element(m->l, e, &block, seg);
    for (int dir = 0; dir < 6; ++dir) {
      const int d = dir / 2;
      double xe[3] = {0, 0, 0};
      xe[d] = (dir % 2) ? 1.0 : -1.0;
      double x[3], jac[9];
      shell_map(s, m->l, block, seg, xe, x, jac);
      for (int q = 0; q < 3; ++q) centre[18 * e + 3 * dir + q] = x[q];
    }
  }
  const double tol = 1e-9 * s.r_outer;
  for (int64_t e = 0; e < m->E; ++e) {
    int block, seg[3];
    shell_element(m->l, e, &block, seg);
    for (int dir = 0; dir < 6; ++dir) {
      const int d = dir / 2;
      const bool upper = dir % 2;
      int64_t nb = -1;
      int ndir = -1;
      if (d == 2 && !upper && seg[2] == 0) {
        m->nbr[6 * e + dir] = -1;
        continue;
      }
      if (d == 2 && upper && seg[2] == m->l.per_axis[2] - 1) {
        m->nbr[6 * e + dir] = -2;
        continue;
      }
      const double* c = &centre[18 * e + 3 * dir];
      for (int64_t f = 0; f < m->E && nb < 0; ++f) {
        if (f == e) continue;
        for (int fd = 0; fd < 6; ++fd) {
          const double* cf = &centre[18 * f + 3 * fd];
          if (std::abs(cf[0] - c[0]) < tol && std::abs(cf[1] - c[1]) < tol &&
              std::abs(cf[2] - c[2]) < tol) {
            nb = f;
            ndir = fd;
            break;
          }
        }
      }
      m->nbr[6 * e + dir] = (int32_t)nb;
      std::vector<double> mine, theirs;
      shell_face_points(s, m->l, e, dir, &mine);
      shell_face_points(s, m->l, nb, ndir, &theirs);
      for (int q = 0; q < n * n; ++q) {
        int hit = -1;
        for (int r = 0; r < n * n; ++r) {
          if (std::abs(mine[3 * q] - theirs[3 * r]) < tol &&
              std::abs(mine[3 * q + 1] - theirs[3 * r + 1]) < tol &&
              std::abs(mine[3 * q + 2] - theirs[3 * r + 2]) < tol) {
            hit = r;
            break;
          }
        }
        m->perm[(6 * e + dir) * (size_t)n * n + q] = hit;
      }
    }
  }
}

// the face direction of neighbour nb that touches element e
int shell_back_dir(const ShellMesh& m, int64_t e, int64_t nb) {
  for (int fd = 0; fd < 6; ++fd)
    if (m.nbr[6 * nb + fd] == e) return fd;
  return -1;
}

// curved normal on a face point: unnormalised n_i = sign * invjac(d, i),
// NormalCovectorAndMagnitude.hpp:57-84 with the inverse spatial metric
void curved_normal(const double* ij9, double sign, const double* gi6, double nco[3],
                   double nvec[3], double* mag) {
  static const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  double un[3];
  for (int i = 0; i < 3; ++i) un[i] = sign * ij9[i];
  double v[3];
  for (int i = 0; i < 3; ++i) {
    v[i] = gi6[idx[i][0]] * un[0];
    for (int j = 1; j < 3; ++j) v[i] += gi6[idx[i][j]] * un[j];
  }
  double m2 = v[0] * un[0] + v[1] * un[1] + v[2] * un[2];
  *mag = std::sqrt(m2);
  const double inv = 1.0 / *mag;
  for (int i = 0; i < 3; ++i) {
    nco[i] = un[i] * inv;
    nvec[i] = v[i] * inv;
  }
}

int shell_rhs_impl(const ShellMesh& m, const double* u, double* dudt, bool mortars = true) {
  const OrcShell& s = m.s;
  const int n = s.n;
  const int64_t np = (int64_t)n * n * n;
  const int nf = n * n;
  const Spectral1d& sp = spectral(n);
  int excision_violation = 0;
#pragma omp parallel for schedule(dynamic, 2) reduction(| : excision_violation)
  for (int64_t e = 0; e < m.E; ++e) {
    const double* ue = u + e * 5 * np;
    double* dt = dudt + e * 5 * np;
    const double* X = &m.xyz[e * 3 * np];
    const double* IJ = &m.ij[e * 9 * np];
    std::vector<double> dl(15 * np), du(15 * np), bg(26 * np);
    // logical derivatives (PartialDerivatives.tpp:315-363)
    for (int v = 0; v < 5; ++v)
      for (int a = 0; a < 3; ++a)
        for (int k = 0; k < n; ++k)
          for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
              const int idx[3] = {i, j, k};
              double acc = 0.0;
              for (int q = 0; q < n; ++q) {
                int id2[3] = {i, j, k};
                id2[a] = q;
                acc += sp.D[idx[a] * n + q] * ue[v * np + id2[0] + n * (id2[1] + n * id2[2])];
              }
              dl[(3 * v + a) * np + i + n * (j + (int64_t)n * k)] = acc;
            }
    // partial derivatives: du[(3v+i)] = sum_a invjac(a,i) d_a u_v, a = 0 first
    for (int v = 0; v < 5; ++v)
      for (int i = 0; i < 3; ++i)
        for (int64_t p = 0; p < np; ++p) {
          double acc = IJ[(3 * 0 + i) * np + p] * dl[(3 * v + 0) * np + p];
          acc += IJ[(3 * 1 + i) * np + p] * dl[(3 * v + 1) * np + p];
          acc += IJ[(3 * 2 + i) * np + p] * dl[(3 * v + 2) * np + p];
          du[(3 * v + i) * np + p] = acc;
        }
    orc_ks_background((int)np, s.mass, X, bg.data());
    // d_phi(i, j) = d_i Phi_j = du[(3*(2+j)+i)]
    std::vector<double> dphi(9 * np);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int64_t p = 0; p < np; ++p) dphi[(3 * i + j) * np + p] = du[(3 * (2 + j) + i) * np + p];
    orc_csw_time_derivative((int)np, du.data(), du.data() + 3 * np, dphi.data(), ue + np,
                            ue + 2 * np, bg.data(), s.gamma1, s.gamma2, dt);
    // external faces first (they use the volume time derivative), then mortars
    for (int pass = 0; pass < 2; ++pass)
      for (int dir = 0; dir < 6; ++dir) {
        const int64_t nb = m.nbr[6 * e + dir];
        if ((pass == 0) != (nb < 0)) continue;
        if (nb >= 0 && !mortars) continue;
        const int d = dir / 2;
        const bool upper = dir % 2;
        const int slice = upper ? n - 1 : 0;
        const double sign = upper ? 1.0 : -1.0;
        for (int bb = 0; bb < n; ++bb)
          for (int aa = 0; aa < n; ++aa) {
            const int q = aa + n * bb;
            const int64_t vp = volume_index(n, d, slice, aa, bb);
            double ij9[3], gi6[6], nco[3], nvec[3], mag;
            for (int i = 0; i < 3; ++i) ij9[i] = IJ[(3 * d + i) * np + vp];
            for (int t = 0; t < 6; ++t) gi6[t] = bg[(16 + t) * np + vp];
            curved_normal(ij9, sign, gi6, nco, nvec, &mag);
            const double lapse = bg[vp];
            double shift[3];
            for (int i = 0; i < 3; ++i) shift[i] = bg[(1 + i) * np + vp];
            const double g1 = s.gamma1, g2 = s.gamma2;
            const double psi = ue[vp], pi = ue[np + vp];
            double phi[3];
            for (int i = 0; i < 3; ++i) phi[i] = ue[(2 + i) * np + vp];
            if (nb == -1) {
              // DemandOutgoingCharSpeeds (DemandOutgoingCharSpeeds.cpp:40-77)
              double bn = shift[0] * nco[0] + shift[1] * nco[1] + shift[2] * nco[2];
              const double sp4[4] = {-(1.0 + g1) * bn, -bn, -bn + lapse, -bn - lapse};
              for (double c : sp4)
                if (c < 0.0) excision_violation = 1;
              continue;
            }
            if (nb == -2) {
              // ConstraintPreservingSphericalRadiation::dg_time_derivative
              double dps[3], dpi[3], dph[9], dtphi[3], xyz3[3], out[5];
              for (int i = 0; i < 3; ++i) {
                dps[i] = du[(3 * 0 + i) * np + vp];
                dpi[i] = du[(3 * 1 + i) * np + vp];
                dtphi[i] = dt[(2 + i) * np + vp];
                xyz3[i] = X[i * np + vp];
              }
              for (int t = 0; t < 9; ++t) dph[t] = dphi[t * np + vp];
              double dtpsi = dt[vp], dtpi = dt[np + vp];
              orc_csw_cpsr(1, &psi, &pi, phi, &lapse, shift, &g1, &g2, nco, nvec, xyz3, dps, dpi,
                           dph, &dtpsi, &dtpi, dtphi, out);
              for (int v = 0; v < 5; ++v) dt[v * np + vp] += out[v];
              continue;
            }
            // interior mortar: UpwindPenalty on both sides, lift_flux
            double pk_i[14], pk_e[14], ms;
            orc_csw_package(1, &psi, &pi, phi, &lapse, shift, &g1, &g2, nco, nvec, nullptr, pk_i,
                            &ms);
            const int nd = shell_back_dir(m, e, nb);
            const int nd_d = nd / 2;
            const int nq = m.perm[(6 * e + dir) * (size_t)nf + q];
            const int na = nq % n, nbq = nq / n;
            const int nslice = (nd % 2) ? n - 1 : 0;
            const int64_t nvp = volume_index(n, nd_d, nslice, na, nbq);
            const double* un = u + nb * 5 * np;
            const double* IJn = &m.ij[nb * 9 * np];
            double nX[3];
            for (int i = 0; i < 3; ++i) nX[i] = m.xyz[nb * 3 * np + i * np + nvp];
            double nbg[26];
            orc_ks_background(1, s.mass, nX, nbg);
            double nij9[3], ngi6[6], nnco[3], nnvec[3], nmag;
            for (int i = 0; i < 3; ++i) nij9[i] = IJn[(3 * nd_d + i) * np + nvp];
            for (int t = 0; t < 6; ++t) ngi6[t] = nbg[16 + t];
            curved_normal(nij9, (nd % 2) ? 1.0 : -1.0, ngi6, nnco, nnvec, &nmag);
            const double npsi = un[nvp], npi = un[np + nvp];
            double nphi[3], nshift[3];
            for (int i = 0; i < 3; ++i) {
              nphi[i] = un[(2 + i) * np + nvp];
              nshift[i] = nbg[1 + i];
            }
            orc_csw_package(1, &npsi, &npi, nphi, &nbg[0], nshift, &g1, &g2, nnco, nnvec, nullptr,
                            pk_e, &ms);
            double bc[5];
            orc_csw_boundary_terms(1, pk_i, pk_e, bc);
            const double fac = -0.5 * static_cast<double>(n * (n - 1)) * mag;
            for (int v = 0; v < 5; ++v) dt[v * np + vp] += bc[v] * fac;
          }
      }
  }
  return excision_violation;
}

// The curved shell as a system of the Adams-Bashforth / LTS oracle: volume
// terms with the radiation condition on the outer sphere (a time-derivative
// condition, part of dt u), packaged data with each side's own normal and
// background, and the curved UpwindPenalty boundary terms.
struct ShellSystem : orc_adams::System {
  ShellMesh m;
  bool filter = false;  // the exponential filter after every step
  double filter_alpha = 0.0;
  int filter_half_power = 0;
  void filter_element(double* u, int64_t e) const override {
    if (!filter) return;
    const int32_t ne = n;
    orc_filter_elements(1, &ne, filter_alpha, filter_half_power, u + e * 5 * np);
  }
  int64_t neighbor(int64_t e, int dir) const override { return m.nbr[6 * e + dir]; }
  int back_dir(int64_t e, int dir) const override {
    return shell_back_dir(m, e, m.nbr[6 * e + dir]);
  }
  void volume_rhs(const double* u, double* dudt) override { shell_rhs_impl(m, u, dudt, false); }
  // package of face point vp of element e on its face dir (14 values)
  void point_package(const double* u, int64_t e, int dir, int64_t vp, double* pk,
                     double* mag) const {
    const OrcShell& s = m.s;
    const int d = dir / 2;
    const double* ue = u + e * 5 * np;
    const double* IJ = &m.ij[e * 9 * np];
    double X[3], bg[26];
    for (int i = 0; i < 3; ++i) X[i] = m.xyz[e * 3 * np + i * np + vp];
    orc_ks_background(1, s.mass, X, bg);
    double ij9[3], gi6[6], nco[3], nvec[3];
    for (int i = 0; i < 3; ++i) ij9[i] = IJ[(3 * d + i) * np + vp];
    for (int t = 0; t < 6; ++t) gi6[t] = bg[16 + t];
    curved_normal(ij9, (dir % 2) ? 1.0 : -1.0, gi6, nco, nvec, mag);
    const double psi = ue[vp], pi = ue[np + vp];
    double phi[3], shift[3];
    for (int i = 0; i < 3; ++i) {
      phi[i] = ue[(2 + i) * np + vp];
      shift[i] = bg[1 + i];
    }
    const double g1 = s.gamma1, g2 = s.gamma2;
    double ms;
    orc_csw_package(1, &psi, &pi, phi, &bg[0], shift, &g1, &g2, nco, nvec, nullptr, pk, &ms);
  }
  void package(const double* u, int64_t e, int dir, std::vector<double>* pkg,
               std::vector<double>* mag) const override {
    const int nf = n * n, d = dir / 2, slice = (dir % 2) ? n - 1 : 0;
    pkg->assign((size_t)14 * nf, 0.0);
    mag->assign(nf, 0.0);
    for (int bb = 0; bb < n; ++bb)
      for (int aa = 0; aa < n; ++aa) {
        const int q = aa + n * bb;
        point_package(u, e, dir, volume_index(n, d, slice, aa, bb), &(*pkg)[14 * q], &(*mag)[q]);
      }
  }
  void exterior_package(const double* u, int64_t e, int dir,
                        std::vector<double>* pkg) const override {
    const int nf = n * n;
    const int64_t nb = m.nbr[6 * e + dir];
    const int nd = shell_back_dir(m, e, nb);
    const int nslice = (nd % 2) ? n - 1 : 0;
    pkg->assign((size_t)14 * nf, 0.0);
    for (int q = 0; q < nf; ++q) {
      const int nq = m.perm[(6 * e + dir) * (size_t)nf + q];
      double mag;
      point_package(u, nb, nd, volume_index(n, nd / 2, nslice, nq % n, nq / n), &(*pkg)[14 * q],
                    &mag);
    }
  }
  void boundary_terms(const std::vector<double>& pi, const std::vector<double>& pe,
                      double* out) const override {
    const int nf = n * n;
    for (int q = 0; q < nf; ++q) {
      double bc[5];
      orc_csw_boundary_terms(1, &pi[14 * q], &pe[14 * q], bc);
      for (int v = 0; v < 5; ++v) out[(size_t)v * nf + q] = bc[v];
    }
  }
};

}  // namespace

extern "C" {

int64_t orc_shell_num_elements(const OrcShell* s) {
  if (!s) return -1;
  return 6 * shell_layout(*s).per_block;
}

static int check_shell(const OrcShell* s) {
  if (!s || s->n < 2 || s->n > kMaxN || s->ref_ang < 0 || s->ref_rad < 0 || s->ref_ang > 6 ||
      s->ref_rad > 6 || !(s->r_outer > s->r_inner) || !(s->r_inner > 0))
    return -1;
  return 0;
}

int orc_shell_geometry(const OrcShell* s, double* xyz, double* inv_jac) {
  if (check_shell(s) || !xyz || !inv_jac) return -1;
  ShellMesh m;
  build_shell(*s, &m);
  std::memcpy(xyz, m.xyz.data(), m.xyz.size() * sizeof(double));
  std::memcpy(inv_jac, m.ij.data(), m.ij.size() * sizeof(double));
  return 0;
}

int orc_shell_connectivity(const OrcShell* s, int32_t* nbr, int32_t* perm, uint64_t* ids) {
  if (check_shell(s)) return -1;
  ShellMesh m;
  build_shell(*s, &m);
  if (nbr) std::memcpy(nbr, m.nbr.data(), m.nbr.size() * sizeof(int32_t));
  if (perm) std::memcpy(perm, m.perm.data(), m.perm.size() * sizeof(int32_t));
  if (ids)
    for (int64_t e = 0; e < m.E; ++e) {
      int block, seg[3];
      shell_element(m.l, e, &block, seg);
      ids[e] = (uint64_t)block | ((uint64_t)seg[0] << 16) | ((uint64_t)m.l.L[0] << 28) |
               ((uint64_t)seg[1] << 32) | ((uint64_t)m.l.L[1] << 44) |
               ((uint64_t)seg[2] << 48) | ((uint64_t)m.l.L[2] << 60);
    }
  return 0;
}

int orc_shell_initial_data(const OrcShell* s, double r0, double w, double* u) {
  if (check_shell(s) || !u) return -1;
  ShellMesh m;
  build_shell(*s, &m);
  const int64_t np = (int64_t)s->n * s->n * s->n;
  for (int64_t e = 0; e < m.E; ++e)
    for (int64_t p = 0; p < np; ++p) {
      double x[3];
      for (int i = 0; i < 3; ++i) x[i] = m.xyz[e * 3 * np + i * np + p];
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      const double psi = std::exp(-(r - r0) * (r - r0) / (w * w));
      double* ue = u + e * 5 * np;
      ue[p] = psi;
      ue[np + p] = 0.0;
      for (int i = 0; i < 3; ++i) ue[(2 + i) * np + p] = -2.0 * (r - r0) / (w * w) * psi * x[i] / r;
    }
  return 0;
}

int orc_shell_rhs(const OrcShell* s, const double* u, double* dudt, int n_threads) {
  if (check_shell(s) || !u || !dudt) return -1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  (void)n_threads;
  ShellMesh m;
  build_shell(*s, &m);
  return shell_rhs_impl(m, u, dudt);
}

int orc_shell_evolve_adams(const OrcShell* s, int order, const int32_t* levels, double slab,
                           int n_slabs, double* u, int n_threads) {
  if (check_shell(s) || !u) return -1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  (void)n_threads;
  ShellSystem sys;
  build_shell(*s, &sys.m);
  sys.E = sys.m.E;
  sys.n = s->n;
  sys.np = (int64_t)s->n * s->n * s->n;
  return orc_adams::lts_evolve(sys, order, levels, slab, n_slabs, u);
}

int orc_shell_evolve_adams_filtered(const OrcShell* s, int order, const int32_t* levels,
                                    double slab, int n_slabs, double alpha, int half_power,
                                    double* u, int n_threads) {
  if (check_shell(s) || !u || !(alpha >= 0.0) || half_power < 0) return -1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  (void)n_threads;
  ShellSystem sys;
  build_shell(*s, &sys.m);
  sys.E = sys.m.E;
  sys.n = s->n;
  sys.np = (int64_t)s->n * s->n * s->n;
  sys.filter = true;
  sys.filter_alpha = alpha;
  sys.filter_half_power = half_power;
  return orc_adams::lts_evolve(sys, order, levels, slab, n_slabs, u);
}

int orc_shell_observe_norms(const OrcShell* s, const double* u, double* out) {
  if (check_shell(s) || !u || !out) return -1;
  ShellMesh m;
  build_shell(*s, &m);
  const int64_t np = (int64_t)s->n * s->n * s->n;
  std::vector<double> dj(m.E * np);
  for (int64_t e = 0; e < m.E; ++e)
    for (int64_t p = 0; p < np; ++p) {
      double inv[9];
      for (int c = 0; c < 9; ++c) inv[c] = m.ij[e * 9 * np + c * np + p];
      const double det = inv[0] * (inv[4] * inv[8] - inv[5] * inv[7]) -
                         inv[1] * (inv[3] * inv[8] - inv[5] * inv[6]) +
                         inv[2] * (inv[3] * inv[7] - inv[4] * inv[6]);
      dj[e * np + p] = 1.0 / det;
    }
  return orc_shell_observe_norms_impl(m.E, s->n, dj.data(), u, nullptr, out);
}

int orc_shell_evolve(const OrcShell* s, double dt, int n_steps, double* u, int n_threads) {
  if (check_shell(s) || !u || n_steps < 0) return -1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  (void)n_threads;
  ShellMesh m;
  build_shell(*s, &m);
  const int64_t n = m.E * 5 * (int64_t)s->n * s->n * s->n;
  std::vector<double> u0(n), u1(n), du(n);
  int rc = 0;
  for (int st = 0; st < n_steps; ++st) {
    std::memcpy(u0.data(), u, n * sizeof(double));
    rc |= shell_rhs_impl(m, u0.data(), du.data());
    orc_rk3_substep(n, 0, dt, u0.data(), u0.data(), du.data(), u1.data());
    rc |= shell_rhs_impl(m, u1.data(), du.data());
    orc_rk3_substep(n, 1, dt, u0.data(), u1.data(), du.data(), u);
    std::memcpy(u1.data(), u, n * sizeof(double));
    rc |= shell_rhs_impl(m, u1.data(), du.data());
    orc_rk3_substep(n, 2, dt, u0.data(), u1.data(), du.data(), u);
  }
  return rc;
}


// The 1D matrix (dst x src) of amr::projectors::ProjectVariables along one
// dimension (ParallelAlgorithms/Amr/Projectors/Variables.hpp:25-99):
// child 0 is p_projection_matrices (Projection.cpp:401-421: identity, the
// parent-to-child interpolation when the target is at least as fine, else
// the child-to-parent modal truncation); child 1 / 2 is
// projection_matrix_parent_to_child LowerHalf / UpperHalf
// (Projection.cpp:291-372), interpolation to 0.5 (x -/+ 1), target at least
// as fine as the source.
int orc_amr_matrix(int src, int dst, int child, double* M) {
  if (src < 2 || dst < 2 || src > kMaxN || dst > kMaxN || child < 0 || child > 2 || !M)
    return -1;
  if (child == 0) {
    if (src == dst) {
      for (int i = 0; i < dst; ++i)
        for (int j = 0; j < src; ++j) M[i * src + j] = i == j ? 1.0 : 0.0;
      return 0;
    }
    return dst > src ? orc_proj_face_to_mortar(src, dst, M) : orc_proj_mortar_to_face(dst, src, M);
  }
  if (dst < src) return -1;
  const Spectral1d& sd = spectral(dst);
  std::vector<double> t(dst);
  for (int i = 0; i < dst; ++i) t[i] = 0.5 * (sd.x[i] + (child == 2 ? 1.0 : -1.0));
  return orc_interp_matrix(src, dst, t.data(), M);
}

// Target block k = the source block src[k] with the three 1D matrices
// applied as apply_matrices does (x fastest), n_vars components per block.
int orc_amr_project(int n_vars, int64_t n_out, const int32_t* src, const int32_t* src_ext,
                    const int32_t* dst_ext, const int8_t* child, const double* in,
                    const int64_t* in_off, double* out, const int64_t* out_off) {
  for (int64_t k = 0; k < n_out; ++k) {
    const int* se = src_ext + 3 * k;
    const int* de = dst_ext + 3 * k;
    std::vector<double> Mx(de[0] * se[0]), My(de[1] * se[1]), Mz(de[2] * se[2]);
    if (orc_amr_matrix(se[0], de[0], child[3 * k], Mx.data()) ||
        orc_amr_matrix(se[1], de[1], child[3 * k + 1], My.data()) ||
        orc_amr_matrix(se[2], de[2], child[3 * k + 2], Mz.data()))
      return -1;
    const int64_t s_np = (int64_t)se[0] * se[1] * se[2], d_np = (int64_t)de[0] * de[1] * de[2];
    for (int v = 0; v < n_vars; ++v) {
      const double* u = in + in_off[src[k]] + v * s_np;
      double* w = out + out_off[k] + v * d_np;
      for (int c = 0; c < de[2]; ++c)
        for (int b = 0; b < de[1]; ++b)
          for (int a = 0; a < de[0]; ++a) {
            double acc = 0.0;
            for (int r = 0; r < se[2]; ++r)
              for (int q = 0; q < se[1]; ++q)
                for (int p = 0; p < se[0]; ++p)
                  acc += Mz[c * se[2] + r] * My[b * se[1] + q] * Mx[a * se[0] + p] *
                         u[p + se[0] * (q + se[1] * r)];
            w[a + de[0] * (b + de[1] * c)] = acc;
          }
    }
  }
  return 0;
}

}  // extern "C"
