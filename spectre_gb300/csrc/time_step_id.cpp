// time_step_id.cpp -- the time bookkeeping of a step: TimeStepId and the time
// steppers' next_time_id, with exact slab fractions.
//
// A time is a position in a slab [start, end] given as a reduced fraction
// f = num/den of the slab, with value (1 - f) start + f end (Time.cpp:96-98;
// Rational::value() is num/den in double, Rational.cpp:41-43, and fractions
// are kept reduced with a positive denominator and must fit 32 bits,
// Rational.cpp:18-32).  A TimeStepId (TimeStepId.hpp:26-70) holds the slab
// number, the time at the start of its step, the substep, the step size as a
// slab fraction (only the sign of time's direction at substep 0) and the
// substep's time:
//  - next_step (TimeStepId.cpp:65-69): the start of the next step, at
//    step_time + step_size;
//  - next_substep (TimeStepId.cpp:71-81): substep + 1 at time
//    (1 - r) t0 + r (t0 + dt) for the substep's fraction r of the step;
//  - canonicalize (TimeStepId.cpp:83-97): a step start at the end of its
//    slab (start, when time runs backwards) moves into the next slab
//    (Slab::advance / retreat, Slab.cpp:31-33: same duration) and the slab
//    number goes up by one.
// Rk3HesthavenSsp::next_time_id (Rk3HesthavenSsp.cpp:36-48): substep 0 -> 1 at
// fraction 1, 1 -> 2 at fraction 1/2, 2 -> the next step.  AdamsBashforth has
// one substep per step: next_time_id is next_step (AdamsBashforth.cpp:
// 86-90).  The reference ERRORs or ASSERTs where this returns false with a
// message.
#include <cstdint>
#include <string>

#include "host_setup.hpp"

namespace dgsw {
namespace {

int64_t gcd64(int64_t a, int64_t b) {
  if (a < 0) a = -a;
  if (b < 0) b = -b;
  while (b != 0) {
    const int64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

struct Frac {
  int64_t num = 0, den = 1;
};

bool reduce(int64_t num, int64_t den, Frac* out, std::string* err) {
  if (den == 0) {
    *err = "division by zero in a slab fraction";
    return false;
  }
  const int64_t g = gcd64(num, den);
  if (g != 0) {
    num /= g;
    den /= g;
  }
  if (den < 0) {
    num = -num;
    den = -den;
  }
  if (num != (int32_t)num || den != (int32_t)den) {
    *err = "slab fraction overflows 32 bits";
    return false;
  }
  out->num = num;
  out->den = den;
  return true;
}

bool add(const Frac& a, const Frac& b, Frac* out, std::string* err) {
  return reduce(a.num * b.den + a.den * b.num, a.den * b.den, out, err);
}

double frac_value(const Frac& f) { return (double)f.num / (double)f.den; }

// (1 - f) start + f end, each product rounded on its own (no fused
// multiply-add, which the compiler could otherwise form on FMA hardware)
double time_value(double start, double end, const Frac& f) {
  Frac one_minus;
  std::string unused;
  reduce(f.den - f.num, f.den, &one_minus, &unused);
  volatile double a = frac_value(one_minus) * start;
  volatile double b = frac_value(f) * end;
  return a + b;
}

void set_time(DgswTimeStepId* id, const Frac& f) {
  id->step_num = (int32_t)f.num;
  id->step_den = (int32_t)f.den;
}

// canonicalize (TimeStepId.cpp:83-97)
bool canonicalize(DgswTimeStepId* id, std::string* err) {
  const bool forward = id->size_num > 0;
  const bool at_end = id->step_num == id->step_den;
  const bool at_start = id->step_num == 0;
  if (forward ? at_end : at_start) {
    if (id->substep != 0) {
      *err = "time needs to be advanced, but the step already started";
      return false;
    }
    const double dur = id->slab_end - id->slab_start;
    if (forward) {
      id->slab_start = id->slab_end;
      id->slab_end = id->slab_end + dur;
      id->step_num = 0;
      id->step_den = 1;
    } else {
      id->slab_end = id->slab_start;
      id->slab_start = id->slab_start - dur;
      id->step_num = 1;
      id->step_den = 1;
    }
    ++id->slab_number;
  }
  return true;
}

bool check_id(const DgswTimeStepId& id, std::string* err) {
  if (id.step_den <= 0 || id.step_num < 0 || id.step_num > id.step_den || id.size_den <= 0 ||
      id.size_num == 0 || !(id.slab_end > id.slab_start) || id.substep < 0) {
    *err = "bad time step id";
    return false;
  }
  if (id.substep == 0 && id.size_den != 1) {
    *err = "a time step id at substep 0 carries only the direction of time (+-1/1)";
    return false;
  }
  return true;
}

// step_time + step_size as a slab fraction, range-checked (Time::operator+=)
bool step_end(const DgswTimeStepId& id, const Frac& size, Frac* out, std::string* err) {
  Frac t;
  t.num = id.step_num;
  t.den = id.step_den;
  if (!add(t, size, out, err)) return false;
  if (out->num < 0 || out->num > out->den) {
    *err = "the step leaves its slab";
    return false;
  }
  return true;
}

}  // namespace

bool make_time_step_id(int forward, int64_t slab_number, double slab_start, double slab_end,
                       int32_t num, int32_t den, DgswTimeStepId* out, std::string* err) {
  Frac f;
  if (!reduce(num, den, &f, err)) return false;
  if (f.num < 0 || f.num > f.den || !(slab_end > slab_start)) {
    *err = "the time must lie in its slab";
    return false;
  }
  DgswTimeStepId id{};
  id.slab_number = slab_number;
  id.slab_start = slab_start;
  id.slab_end = slab_end;
  set_time(&id, f);
  id.substep = 0;
  id.size_num = forward ? 1 : -1;
  id.size_den = 1;
  id.substep_time = time_value(slab_start, slab_end, f);
  if (!canonicalize(&id, err)) return false;
  *out = id;
  return true;
}

bool substep_fraction(int time_stepper, int substep, double* fraction, std::string* err) {
  if (time_stepper == DGSW_STEPPER_RK3_HESTHAVEN_SSP) {
    static const double kFrac[3] = {0.0, 1.0, 0.5};
    if (substep < 0 || substep > 2) {
      *err = "Rk3HesthavenSsp has substeps 0, 1, 2";
      return false;
    }
    *fraction = kFrac[substep];
    return true;
  }
  if (time_stepper == DGSW_STEPPER_ADAMS_BASHFORTH) {
    if (substep != 0) {
      *err = "AdamsBashforth has one substep";
      return false;
    }
    *fraction = 0.0;
    return true;
  }
  *err = "unknown time stepper";
  return false;
}

bool next_time_id(int time_stepper, const DgswTimeStepId& cur, int32_t size_num, int32_t size_den,
                  DgswTimeStepId* next, std::string* err) {
  if (!check_id(cur, err)) return false;
  Frac size;
  if (!reduce(size_num, size_den, &size, err)) return false;
  if (size.num == 0 || (size.num > 0) != (cur.size_num > 0)) {
    *err = "the step size must be nonzero and point in the direction of time";
    return false;
  }
  if (cur.substep != 0 && (size.num != cur.size_num || size.den != cur.size_den)) {
    *err = "step size inconsistent with the step in progress";
    return false;
  }
  int n_sub = 0;
  if (time_stepper == DGSW_STEPPER_RK3_HESTHAVEN_SSP)
    n_sub = 3;
  else if (time_stepper == DGSW_STEPPER_ADAMS_BASHFORTH)
    n_sub = 1;
  else {
    *err = "unknown time stepper";
    return false;
  }
  if (cur.substep >= n_sub) {
    *err = "bad substep for this time stepper";
    return false;
  }
  Frac end;
  if (!step_end(cur, size, &end, err)) return false;
  DgswTimeStepId id = cur;
  if (cur.substep == n_sub - 1) {
    // next_step: the start of the next step
    set_time(&id, end);
    id.substep = 0;
    id.size_num = size.num > 0 ? 1 : -1;
    id.size_den = 1;
    id.substep_time = time_value(id.slab_start, id.slab_end, end);
    if (!canonicalize(&id, err)) return false;
  } else {
    // next_substep at the fraction of the following substep
    const double r = time_stepper == DGSW_STEPPER_RK3_HESTHAVEN_SSP
                         ? (cur.substep == 0 ? 1.0 : 0.5)
                         : 0.0;
    Frac t0;
    t0.num = cur.step_num;
    t0.den = cur.step_den;
    volatile double a = (1.0 - r) * time_value(cur.slab_start, cur.slab_end, t0);
    volatile double b = r * time_value(cur.slab_start, cur.slab_end, end);
    id.substep = cur.substep + 1;
    id.size_num = (int32_t)size.num;
    id.size_den = (int32_t)size.den;
    id.substep_time = a + b;
  }
  *next = id;
  return true;
}

}  // namespace dgsw
