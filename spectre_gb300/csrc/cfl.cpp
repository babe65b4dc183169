// cfl.cpp -- StepChoosers::Cfl for every element of a configuration
// (Time/StepChoosers/Cfl.hpp:55-67):
//   step = safety * stable_step * minimum_grid_spacing / (speed * 3)
// with
//  - stable_step of the time stepper: Rk3HesthavenSsp::stable_step
//    (Rk3HesthavenSsp.cpp:23-26) or AdamsBashforth::stable_step
//    (AdamsBashforth.cpp:66-82);
//  - the element's minimum grid spacing: the smallest distance between a
//    point and its neighbours one index away in any dimension
//    (Domain/MinimumGridSpacing.cpp), in inertial coordinates;
//  - the largest characteristic speed: 1 for ScalarWave
//    (ScalarWave/Characteristics.hpp:222-231); for CurvedScalarWave the
//    element's maximum of max(|1 + gamma1| |beta|, |beta| + alpha)
//    (CurvedScalarWave/Characteristics.cpp:202-212), with the Kerr-Schild
//    (spin 0) lapse alpha = (1 + 2H)^-1/2, H = M / r, and |beta| = 2 H alpha.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "adams.hpp"
#include "host_setup.hpp"

namespace dgsw {

double time_stepper_stable_step(const DgswConfig& cfg) {
  if (cfg.time_stepper == DGSW_STEPPER_ADAMS_BASHFORTH) {
    const int k = cfg.stepper_order ? cfg.stepper_order : 3;
    if (k == 1) return 1.0;
    // the constant-step weights, oldest first, folded with alternating signs
    int64_t t[kAbMaxOrder];
    double c[kAbMaxOrder];
    for (int i = 0; i < k; ++i) t[i] = i;
    adams_step_coefficients(k, t, k - 1, k, 1.0, 1, c);
    double inv = 0.0;
    for (int i = 0; i < k; ++i) inv = c[i] - inv;
    return 1.0 / inv;
  }
  const double r = std::cbrt(4.0 + std::sqrt(17.0));
  return 0.5 * (1.0 + r - 1.0 / r);
}

bool cfl_steps(const DgswConfig& cfg, const Domain& dom, const ShellGeometry* geo, double safety,
               std::vector<double>* steps, std::string* err) {
  if (!(safety > 0.0) || !std::isfinite(safety)) {
    *err = "the safety factor must be positive";
    return false;
  }
  const double stable = time_stepper_stable_step(cfg);
  const int64_t E = dom.n_elem;
  steps->assign(E, 0.0);
  const bool gauss = cfg.quadrature == DGSW_QUADRATURE_GAUSS;
  if (cfg.system == DGSW_SYSTEM_CURVED_SCALAR_WAVE_3D) {
    if (!geo || geo->xyz.empty()) {
      *err = "the shell geometry is missing";
      return false;
    }
    const int n = geo->n;
    const int64_t np = (int64_t)n * n * n;
    const double M = cfg.shell->mass, g1 = cfg.shell->gamma1;
    for (int64_t e = 0; e < E; ++e) {
      const double* X = &geo->xyz[e * 3 * np];
      auto at = [&](int i, int j, int k, int c) { return X[c * np + i + n * (j + (int64_t)n * k)]; };
      double spacing = INFINITY, speed = 0.0;
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) {
            // offsets in {-1, 0, 1}^3 up to the centre: the others are the
            // opposites, found from the other point
            for (int o = 0; o < 13; ++o) {
              const int di = o % 3 - 1, dj = (o / 3) % 3 - 1, dk = o / 9 - 1;
              const int i2 = i + di, j2 = j + dj, k2 = k + dk;
              if (i2 < 0 || i2 >= n || j2 < 0 || j2 >= n || k2 < 0 || k2 >= n) continue;
              double d2 = 0.0;
              for (int c = 0; c < 3; ++c) {
                const double dx = at(i2, j2, k2, c) - at(i, j, k, c);
                d2 += dx * dx;
              }
              spacing = std::min(spacing, std::sqrt(d2));
            }
            const double r = std::sqrt(at(i, j, k, 0) * at(i, j, k, 0) +
                                        at(i, j, k, 1) * at(i, j, k, 1) +
                                        at(i, j, k, 2) * at(i, j, k, 2));
            const double H = M / r;
            const double alpha = 1.0 / std::sqrt(1.0 + 2.0 * H);
            const double beta = 2.0 * H * alpha;
            speed = std::max(speed, std::max(std::abs(1.0 + g1) * beta, beta + alpha));
          }
      (*steps)[e] = safety * stable * spacing / (speed * 3.0);
    }
    return true;
  }
  // affine elements: the closest points are neighbours along an axis, at
  // the smallest node gap (the ends of the interval) scaled by width / 2
  double gap[kMaxN + 1] = {};
  for (int n = kMinN; n <= kMaxN; ++n) {
    double x[kMaxN], w[kMaxN];
    if (gauss) {
      GaussTables g;
      lg_spectral(n, &g);
      for (int i = 0; i < n; ++i) x[i] = g.x[i];
    } else {
      lgl_nodes_weights(n, x, w);
    }
    double m = INFINITY;
    for (int i = 0; i + 1 < n; ++i) m = std::min(m, x[i + 1] - x[i]);
    gap[n] = m;
  }
  for (int64_t e = 0; e < E; ++e) {
    const int n = dom.elem_n[e];
    double spacing = INFINITY;
    for (int d = 0; d < 3; ++d) spacing = std::min(spacing, 0.5 * dom.width[3 * e + d] * gap[n]);
    (*steps)[e] = safety * stable * spacing / 3.0;  // largest speed 1
  }
  return true;
}

}  // namespace dgsw
