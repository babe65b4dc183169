// adams_oracle.hpp -- the system interface of the Adams-Bashforth / local
// time-stepping oracle (test infrastructure only).  The time stepping
// (adams_oracle.cpp) is written once against this interface; the flat brick
// of one extent and of per-element extents (adams_oracle.cpp) and the curved
// shell (dgsw_oracle.cpp) implement it.
#pragma once

#include <cstdint>
#include <vector>

namespace orc_adams {

struct System {
  int64_t E = 0;   // elements
  int n = 0;       // GLL points per dimension (one extent)
  int64_t np = 0;  // points per element (one extent)
  virtual ~System() = default;
  // extent of element e, the offset of its 5 n^3 block in the state, and the
  // state's length (one extent unless overridden)
  virtual int n_of(int64_t) const { return n; }
  virtual int64_t offset_of(int64_t e) const { return e * 5 * np; }
  virtual int64_t total_values() const { return E * 5 * np; }
  // neighbour across face dir of element e; < 0 for an external face
  virtual int64_t neighbor(int64_t e, int dir) const = 0;
  // the neighbour's face that touches e
  virtual int back_dir(int64_t e, int dir) const = 0;
  // every element's volume time derivative with the external boundary
  // conditions of time-derivative type, no internal mortar terms
  // (ComputeTimeDerivative in local time stepping)
  virtual void volume_rhs(const double* u, double* dudt) = 0;
  // dg_package_data of e's face dir on the mortar (projected onto it where
  // the mortar is finer than the face; mortar points in e's face order), and
  // the normal magnitudes on the face
  virtual void package(const double* u, int64_t e, int dir, std::vector<double>* pkg,
                       std::vector<double>* magnitude) const = 0;
  // the neighbour's own packaged data of the face it shares with e's face
  // dir, on the same mortar in e's face-point order (the mortar data it sends)
  virtual void exterior_package(const double* u, int64_t e, int dir,
                                std::vector<double>* pkg) const = 0;
  // dg_boundary_terms of interior and exterior mortar packages: 5 values per
  // mortar point, component-major
  virtual void boundary_terms(const std::vector<double>& pkg_int,
                              const std::vector<double>& pkg_ext, double* out) const = 0;
  // extent of the mortar of e's face dir (the face's own unless overridden)
  virtual int mortar_n(int64_t e, int dir) const {
    (void)dir;
    return n_of(e);
  }
  // dg::Actions::Filter on element e after each of its steps (the curved
  // executable's step actions end with it; none unless overridden)
  virtual void filter_element(double* u, int64_t e) const {
    (void)u;
    (void)e;
  }
  // project_from_mortar of the 5 corrections onto e's face dir (a copy where
  // the mortar is the face)
  virtual void mortar_to_face(int64_t e, int dir, const double* on_mortar, double* on_face) const {
    (void)dir;
    const int ne = n_of(e);
    for (int64_t i = 0; i < (int64_t)5 * ne * ne; ++i) on_face[i] = on_mortar[i];
  }
};

// Self-start and n_slabs slabs of AdamsBashforth(order) with local time
// stepping; element e steps slab / 2^levels[e] after the start-up (levels
// may be NULL).  Returns 0, or < 0 on bad input or missing history data.
int lts_evolve(System& sys, int order, const int32_t* levels, double slab, int n_slabs, double* u);

}  // namespace orc_adams
