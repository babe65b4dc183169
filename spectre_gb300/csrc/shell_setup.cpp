// shell_setup.cpp -- host-side geometry and connectivity of the six-wedge
// spherical shell used by the CurvedScalarWave evolution.
//
// The shell is SpECTRE's Sphere domain without its interior cube
// (Domain/Creators/Sphere.cpp): six Wedge<3> blocks, equiangular, sphericity
// 1 at both radii, ordered +z, -z, +y, -y, +x, -x with the orientations of
// orientations_for_sphere_wrappings (Domain/DomainHelpers.cpp:553-578).
// Each block carries the same initial refinement, elements are numbered as
// initial_element_ids does (InitialElementIds.cpp:45-96: blocks in order,
// then xi-outer / zeta-inner segments), and every element's map is the
// affine segment map composed with the wedge (ElementMap).  All of this runs
// once per handle in FP64 on the CPU.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "host_setup.hpp"

namespace dgsw {
namespace {

// Block b's inertial coordinate i is kSign[b][i] * (wedge-frame coordinate
// kAxis[b][i]): discrete_rotation (Domain/Structure/OrientationMap.cpp:219-234)
// of the six sphere-wrapping orientations.
constexpr int kAxis[6][3] = {{0, 1, 2}, {0, 1, 2}, {0, 2, 1}, {0, 2, 1}, {2, 0, 1}, {2, 0, 1}};
constexpr double kSign[6][3] = {{1, 1, 1},  {1, -1, -1}, {1, 1, -1},
                                {1, -1, 1}, {1, 1, 1},   {-1, -1, 1}};

struct ShellMap {
  double r_lo, r_hi;
  bool log_radial;
  int level[3];
  int per_axis[3];
  int64_t per_block;
};

void element_segments(const ShellMap& m, int64_t e, int* block, int seg[3]) {
  *block = (int)(e / m.per_block);
  const int64_t w = e % m.per_block;
  seg[2] = (int)(w & (m.per_axis[2] - 1));
  seg[1] = (int)((w >> m.level[2]) & (m.per_axis[1] - 1));
  seg[0] = (int)(w >> (m.level[1] + m.level[2]));
}

// Inertial coordinates and Jacobian dx^i / dxi^a (jac[3i + a]) at the element
// logical point xe.  Wedge<3>::operator() and jacobian (Wedge.cpp:476-536,
// 677-790) for the centred, fully spherical, equiangular case:
//   a = tan(pi/4 xi), b = tan(pi/4 eta), rho = sqrt(1 + a^2 + b^2),
//   x_wedge = r(zeta) (a, b, 1) / rho,
//   r = z0 + k zeta (linear) or exp(z0 + k zeta) (logarithmic).
void map_point(const ShellMap& m, int block, const int seg[3], const double xe[3], double x[3],
               double jac[9]) {
  double xb[3], scale[3];
  for (int d = 0; d < 3; ++d) {
    scale[d] = 1.0 / m.per_axis[d];
    xb[d] = -1.0 + (2.0 * seg[d] + 1.0 + xe[d]) * scale[d];
  }
  const double q = 0.78539816339744830962;  // pi / 4
  const double a = std::tan(q * xb[0]), b = std::tan(q * xb[1]);
  const double rho2 = 1.0 + a * a + b * b;
  const double rho = std::sqrt(rho2);
  const double rho3 = rho2 * rho;
  double r, dr;
  if (m.log_radial) {
    const double z0 = 0.5 * std::log(m.r_hi * m.r_lo), k = 0.5 * std::log(m.r_hi / m.r_lo);
    r = std::exp(z0 + k * xb[2]);
    dr = k * r;
  } else {
    const double z0 = 0.5 * (m.r_hi + m.r_lo), k = 0.5 * (m.r_hi - m.r_lo);
    r = z0 + k * xb[2];
    dr = k;
  }
  const double wf[3] = {r * a / rho, r * b / rho, r / rho};
  const double da = q * (1.0 + a * a), db = q * (1.0 + b * b);
  // columns of the wedge-frame Jacobian
  const double c_xi[3] = {r * da * (1.0 + b * b) / rho3, -r * da * a * b / rho3,
                          -r * da * a / rho3};
  const double c_eta[3] = {-r * db * a * b / rho3, r * db * (1.0 + a * a) / rho3,
                           -r * db * b / rho3};
  const double c_zeta[3] = {dr * a / rho, dr * b / rho, dr / rho};
  for (int i = 0; i < 3; ++i) {
    const int p = kAxis[block][i];
    const double s = kSign[block][i];
    x[i] = s * wf[p];
    jac[3 * i + 0] = s * c_xi[p] * scale[0];
    jac[3 * i + 1] = s * c_eta[p] * scale[1];
    jac[3 * i + 2] = s * c_zeta[p] * scale[2];
  }
}

// inv[3a + i] = d xi^a / d x^i of jac[3i + a] (cofactors over the determinant)
void invert(const double m[9], double inv[9]) {
  const double c00 = m[4] * m[8] - m[5] * m[7];
  const double c01 = m[5] * m[6] - m[3] * m[8];
  const double c02 = m[3] * m[7] - m[4] * m[6];
  const double rdet = 1.0 / (m[0] * c00 + m[1] * c01 + m[2] * c02);
  inv[0] = c00 * rdet;
  inv[1] = (m[2] * m[7] - m[1] * m[8]) * rdet;
  inv[2] = (m[1] * m[5] - m[2] * m[4]) * rdet;
  inv[3] = c01 * rdet;
  inv[4] = (m[0] * m[8] - m[2] * m[6]) * rdet;
  inv[5] = (m[2] * m[3] - m[0] * m[5]) * rdet;
  inv[6] = c02 * rdet;
  inv[7] = (m[1] * m[6] - m[0] * m[7]) * rdet;
  inv[8] = (m[0] * m[4] - m[1] * m[3]) * rdet;
}

// Logical coordinates of face point (fa, fb) of face dir: the face's normal
// axis is at -1 or +1, the two others take LGL nodes in ascending axis order.
void face_point(const double* nodes, int dir, int fa, int fb, double xe[3]) {
  const int d = dir >> 1;
  int c = 0;
  const int f[2] = {fa, fb};
  for (int a = 0; a < 3; ++a) xe[a] = (a == d) ? ((dir & 1) ? 1.0 : -1.0) : nodes[f[c++]];
}

struct CellKey {
  int64_t k[3];
  bool operator==(const CellKey& o) const {
    return k[0] == o.k[0] && k[1] == o.k[1] && k[2] == o.k[2];
  }
};
struct CellHash {
  size_t operator()(const CellKey& c) const {
    uint64_t h = 1469598103934665603ull;
    for (int i = 0; i < 3; ++i) h = (h ^ (uint64_t)c.k[i]) * 1099511628211ull;
    return (size_t)h;
  }
};

}  // namespace

bool build_shell_domain(const DgswConfig& cfg, Domain* dom, ShellGeometry* geo,
                        std::string* err) {
  const DgswShell* sh = cfg.shell;
  if (!sh) {
    *err = "the curved system needs a shell description";
    return false;
  }
  if (cfg.boundary_correction != DGSW_CORRECTION_UPWIND_PENALTY ||
      (cfg.time_stepper != DGSW_STEPPER_RK3_HESTHAVEN_SSP &&
       cfg.time_stepper != DGSW_STEPPER_ADAMS_BASHFORTH)) {
    *err = "unsupported boundary correction or time stepper";
    return false;
  }
  if (cfg.precision != DGSW_PRECISION_FP64 && cfg.precision != DGSW_PRECISION_MIXED) {
    *err = "unknown precision";
    return false;
  }
  if (cfg.n_instances != 1 || cfg.points_per_element) {
    *err = "the shell is one evolution with one extent per element";
    return false;
  }
  if (!(sh->inner_radius > 0.0) || !(sh->outer_radius > sh->inner_radius) ||
      !std::isfinite(sh->outer_radius)) {
    *err = "shell radii must satisfy 0 < inner < outer";
    return false;
  }
  if (sh->refinement_angular < 0 || sh->refinement_angular > 8 || sh->refinement_radial < 0 ||
      sh->refinement_radial > 10) {
    *err = "shell refinement out of range";
    return false;
  }
  if (sh->radial_distribution != DGSW_RADIAL_LINEAR &&
      sh->radial_distribution != DGSW_RADIAL_LOGARITHMIC) {
    *err = "unknown radial distribution";
    return false;
  }
  if (!(sh->mass > 0.0) || !std::isfinite(sh->mass) || !std::isfinite(sh->gamma1) ||
      !std::isfinite(cfg.gamma2)) {
    *err = "mass must be positive and the damping parameters finite";
    return false;
  }
  const int n = cfg.uniform_points;
  if (n < kMinN || n > kMaxN) {
    *err = "points per dimension must be in [2, 12]";
    return false;
  }
  ShellMap m;
  m.r_lo = sh->inner_radius;
  m.r_hi = sh->outer_radius;
  m.log_radial = sh->radial_distribution == DGSW_RADIAL_LOGARITHMIC;
  m.level[0] = m.level[1] = sh->refinement_angular;
  m.level[2] = sh->refinement_radial;
  for (int d = 0; d < 3; ++d) m.per_axis[d] = 1 << m.level[d];
  m.per_block = (int64_t)m.per_axis[0] * m.per_axis[1] * m.per_axis[2];
  const int64_t E = 6 * m.per_block;
  const int64_t np = (int64_t)n * n * n;
  const int nf = n * n;
  if (E * kVars * np >= ((int64_t)1 << 31)) {
    *err = "shell too large for 32-bit point indices";
    return false;
  }

  dom->bricks.clear();
  dom->layout.clear();
  dom->n_elem = E;
  dom->elem_n.assign(E, n);
  dom->uniform = true;
  dom->max_n = n;
  dom->offset.resize(E + 1);
  for (int64_t e = 0; e <= E; ++e) dom->offset[e] = e * kVars * np;
  dom->n_points = E * np;
  dom->instance.assign(E, 0);
  dom->lower.assign(3 * E, 0.0);
  dom->width.assign(3 * E, 0.0);
  dom->element_id.resize(E);
  dom->neighbor.assign(6 * E, -1);
  dom->block_ids_fit = true;

  double nodes[kMaxN], w[kMaxN];
  lgl_nodes_weights(n, nodes, w);
  geo->n = n;
  geo->xyz.resize(3 * np * E);
  geo->inv_jac.resize(9 * np * E);
  geo->face_perm.assign(6 * nf * E, -1);
  geo->back_dir.assign(6 * E, -1);
  for (int64_t e = 0; e < E; ++e) {
    int block, seg[3];
    element_segments(m, e, &block, seg);
    dom->element_id[e] = (uint64_t)block | ((uint64_t)seg[0] << 16) |
                         ((uint64_t)m.level[0] << 28) | ((uint64_t)seg[1] << 32) |
                         ((uint64_t)m.level[1] << 44) | ((uint64_t)seg[2] << 48) |
                         ((uint64_t)m.level[2] << 60);
    double* X = &geo->xyz[e * 3 * np];
    double* IJ = &geo->inv_jac[e * 9 * np];
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int64_t p = i + n * (j + (int64_t)n * k);
          const double xe[3] = {nodes[i], nodes[j], nodes[k]};
          double x[3], jac[9], inv[9];
          map_point(m, block, seg, xe, x, jac);
          invert(jac, inv);
          for (int c = 0; c < 3; ++c) X[c * np + p] = x[c];
          for (int c = 0; c < 9; ++c) IJ[c * np + p] = inv[c];
        }
  }

  // Neighbours: the zeta faces of the first / last radial segment lie on the
  // inner / outer sphere; every other face is matched to the face of another
  // element with the same centre (a spatial hash of face centres), and its
  // points to the neighbour's by one of the eight symmetries of the square.
  const double cell = 1e-7 * m.r_hi;
  const double tol = 1e-9 * m.r_hi;
  std::vector<double> centre(18 * E);
  std::unordered_map<CellKey, std::vector<int64_t>, CellHash> grid;
  grid.reserve(6 * E);
  for (int64_t e = 0; e < E; ++e) {
    int block, seg[3];
    element_segments(m, e, &block, seg);
    for (int dir = 0; dir < 6; ++dir) {
      double xe[3] = {0.0, 0.0, 0.0}, jac[9];
      xe[dir >> 1] = (dir & 1) ? 1.0 : -1.0;
      double* c = &centre[18 * e + 3 * dir];
      map_point(m, block, seg, xe, c, jac);
      CellKey key{{(int64_t)std::floor(c[0] / cell), (int64_t)std::floor(c[1] / cell),
                   (int64_t)std::floor(c[2] / cell)}};
      grid[key].push_back(6 * e + dir);
    }
  }
  std::vector<double> mine(3 * nf), theirs(3 * nf);
  auto face_coords = [&](int64_t el, int dir, std::vector<double>* out) {
    int block, seg[3];
    element_segments(m, el, &block, seg);
    for (int fb = 0; fb < n; ++fb)
      for (int fa = 0; fa < n; ++fa) {
        double xe[3], x[3], jac[9];
        face_point(nodes, dir, fa, fb, xe);
        map_point(m, block, seg, xe, x, jac);
        for (int c = 0; c < 3; ++c) (*out)[3 * (fa + n * fb) + c] = x[c];
      }
  };
  for (int64_t e = 0; e < E; ++e) {
    int block, seg[3];
    element_segments(m, e, &block, seg);
    for (int dir = 0; dir < 6; ++dir) {
      if (dir == 4 && seg[2] == 0) {
        dom->neighbor[6 * e + dir] = -1;
        continue;
      }
      if (dir == 5 && seg[2] == m.per_axis[2] - 1) {
        dom->neighbor[6 * e + dir] = -2;
        continue;
      }
      const double* c = &centre[18 * e + 3 * dir];
      const int64_t base[3] = {(int64_t)std::floor(c[0] / cell), (int64_t)std::floor(c[1] / cell),
                               (int64_t)std::floor(c[2] / cell)};
      int64_t found = -1;
      for (int dz = -1; dz <= 1 && found < 0; ++dz)
        for (int dy = -1; dy <= 1 && found < 0; ++dy)
          for (int dx = -1; dx <= 1 && found < 0; ++dx) {
            auto it = grid.find(CellKey{{base[0] + dx, base[1] + dy, base[2] + dz}});
            if (it == grid.end()) continue;
            for (int64_t f : it->second) {
              if (f / 6 == e) continue;
              const double* o = &centre[3 * f];
              if (std::abs(o[0] - c[0]) < tol && std::abs(o[1] - c[1]) < tol &&
                  std::abs(o[2] - c[2]) < tol) {
                found = f;
                break;
              }
            }
          }
      if (found < 0) {
        *err = "shell connectivity: unmatched face";
        return false;
      }
      const int64_t nb = found / 6;
      const int ndir = (int)(found % 6);
      dom->neighbor[6 * e + dir] = (int32_t)nb;
      geo->back_dir[6 * e + dir] = ndir;
      face_coords(e, dir, &mine);
      face_coords(nb, ndir, &theirs);
      int32_t* perm = &geo->face_perm[(6 * e + dir) * nf];
      bool matched = false;
      for (int sym = 0; sym < 8 && !matched; ++sym) {
        const bool swap = sym & 4, flip_a = sym & 1, flip_b = sym & 2;
        matched = true;
        for (int fb = 0; fb < n && matched; ++fb)
          for (int fa = 0; fa < n; ++fa) {
            int ta = swap ? fb : fa, tb = swap ? fa : fb;
            if (flip_a) ta = n - 1 - ta;
            if (flip_b) tb = n - 1 - tb;
            const int q = fa + n * fb, t = ta + n * tb;
            if (std::abs(mine[3 * q] - theirs[3 * t]) > tol ||
                std::abs(mine[3 * q + 1] - theirs[3 * t + 1]) > tol ||
                std::abs(mine[3 * q + 2] - theirs[3 * t + 2]) > tol) {
              matched = false;
              break;
            }
            perm[q] = t;
          }
      }
      if (!matched) {
        *err = "shell connectivity: face points do not match";
        return false;
      }
    }
  }
  return true;
}

}  // namespace dgsw
