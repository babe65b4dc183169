// adams.hpp -- Adams-Bashforth time stepping with local time stepping (LTS):
// the host-side schedule that turns the reference's per-element histories
// into per-level coefficient tables for the fused device kernel
// (adams_step.cu).
//
// Elements carry a step level l: after the start-up they step slab / 2^l.
// Every element of one level steps at the same times, so the histories of the
// reference (volume history of dt u, and per mortar the local and remote
// boundary histories; TimeSteppers/History.hpp, BoundaryHistory.hpp) have the
// same time ids for all of a level's elements.  The schedule therefore keeps
// one volume / local history per level and one remote history per pair of
// adjacent levels, holding only (time id, integration order, ring slot): the
// data sit in device rings indexed by the slot.
//
// The coupling of the flat UpwindPenalty is linear in the local and the
// remote face data, so the reference's sum over (local id, remote id) pairs,
// sum_{l,r} c_lr C(L_l, R_r) (AdamsLts.cpp:150-156), equals
// C(sum_l a_l L_l, sum_r b_r R_r) with the marginals a_l = sum_r c_lr and
// b_r = sum_l c_lr; the tables carry those marginals.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dgsw {

constexpr int kAbMaxOrder = 8;    // AdamsBashforth::maximum_order
constexpr int kAbMaxLevels = 4;   // step ratios up to 8 between elements
constexpr int kAbMaxRemote = 16;  // remote terms of one face: order + ratio - 1

// Coefficients of one step of AdamsBashforth over the control times (ticks),
// adams_coefficients::coefficients (AdamsCoefficients.hpp:29-67).  A tick is
// slab / ticks_per_slab.  Returns false on bad input.
bool adams_step_coefficients(int n, const int64_t* ticks, int64_t start, int64_t end, double slab,
                             int64_t ticks_per_slab, double* out);

// A time id: TimeStepId without substeps (slab number, then time in ticks).
struct AbId {
  int64_t slab = 0;
  int64_t tick = 0;
};
struct AbTerm {
  int32_t local, remote;  // indices into the given histories
  double coef;
};
// adams_lts::lts_coefficients for explicit schemes of orders lo (local), ro
// (remote) and so (small steps) (AdamsLts.cpp:301-415).  Returns 0, or < 0
// when a history lacks the data the step needs.
int adams_lts_terms(const std::vector<AbId>& local, const std::vector<AbId>& remote, int64_t start,
                    int64_t end, int lo, int ro, int so, double slab, int64_t ticks_per_slab,
                    std::vector<AbTerm>* out);

// Coupling of one (own level, neighbour level) face for one step: marginal
// weights of the own face records and of the neighbour's.
struct AbFaceTable {
  int8_t n_loc = 0, n_rem = 0;
  int8_t loc_slot[kAbMaxOrder] = {};
  int8_t rem_slot[kAbMaxRemote] = {};
  double loc_c[kAbMaxOrder] = {};
  double rem_c[kAbMaxRemote] = {};
};

// The work of one level in one launch: finish its step (volume update plus
// boundary delta), optionally restore the initial values (self-start), then
// record dt u and the face data of the new state into ring slot rec_slot.
struct AbLevelJob {
  int32_t level = 0;
  int32_t begin = 0, count = 0;  // range of the level in the level-sorted element list
  int8_t update = 0, reset = 0, n_vol = 0, rec_slot = -1;
  int8_t vol_slot[kAbMaxOrder] = {};
  double vol_c[kAbMaxOrder] = {};
  AbFaceTable face[kAbMaxLevels];  // by the neighbour's level
};

struct AbLaunch {
  int32_t n_jobs = 0;
  AbLevelJob job[kAbMaxLevels];
};

class AdamsSchedule {
 public:
  // order: 1..8; adj[l][m]: some element of level l has a face neighbour of
  // level m; count[l]: elements of level l (levels 0..kAbMaxLevels-1).
  bool init(int order, const bool adj[kAbMaxLevels][kAbMaxLevels],
            const int64_t count[kAbMaxLevels], std::string* err);
  // Launches of the next slab (the first call also runs the self-start).
  bool slab(std::vector<AbLaunch>* out, std::string* err);
  // Forget the histories: the next slab() self-starts again.
  void restart();
  bool started() const { return started_; }
  int ring_slots() const { return ring_slots_; }
  int64_t ticks_per_slab() const { return S_; }
  // element steps per slab after the start-up, by level
  int64_t steps_per_slab(int level) const { return S_ / step_after_switch(level); }
  void set_slab(double slab) { slab_ = slab; }

 private:
  struct Rec {
    AbId id;
    int order;
    int slot;
  };
  struct Level {
    bool present = false;
    std::vector<Rec> vol, loc;
    std::vector<Rec> rem[kAbMaxLevels];  // records of level m seen from this level
    int64_t start = 0, end = 0;
    bool pending = false;  // a used step awaits its update
  };
  int64_t step_after_switch(int l) const { return S_ >> l; }
  int64_t step_at(int l, int64_t t) const { return t < switch_tick_ ? first_step_ : S_ >> l; }
  bool position(AbId id, const bool* finish, bool reset, int rec_order, bool unused_record,
                std::vector<AbLaunch>* out, std::string* err);
  void clean(int l);
  int alloc_slot(int l, const std::vector<int>& busy, std::string* err);
  bool live(int l, int slot) const;
  bool run_startup(std::vector<AbLaunch>* out, std::string* err);

  int order_ = 0;
  int L_ = 0;  // finest level present
  bool adj_[kAbMaxLevels][kAbMaxLevels] = {};
  int64_t count_[kAbMaxLevels] = {};
  int64_t S_ = 1, first_step_ = 1, switch_tick_ = 0;
  double slab_ = 1.0;
  Level lv_[kAbMaxLevels];
  int64_t next_slab_ = 0;
  bool started_ = false;
  int ring_slots_ = 0;   // ring size fixed by the dry run
  int max_slot_ = -1;    // largest slot index handed out
  bool dry_ = false;
};

}  // namespace dgsw
