// hostemu.cpp -- host build of the kernel's dynamics phases (dynamics.cuh).
//
// Runs phase A for the four legs, sums their contributions in the order the device quad
// does ((leg0 + leg1) + (leg2 + leg3)), phase B once, phase C for the four legs. Used by
// the tests to check the kernel's equations against the FP64 oracle on the CPU, and to
// count FP operations of one substep (each operation once: the device repeats phase B on
// the four lanes of a rollout, which is not counted). The same driver runs the legs by
// the articulated-body algorithm of the oracle (aba_reference.h): its count is the
// algorithmic per-substep figure, and its results must equal the condensed phases'.
#include <cmath>
#include <cstring>

#include "aba_reference.h"
#include "model.h"

namespace spi {

// Counting scalar: +, -, *, / and sqrt / tanh / sin / cos count one operation each;
// comparisons, selects, negation, min / max / abs count none.
struct Cf {
  double v;
  static long long n;
  Cf() : v(0) {}
  Cf(double x) : v(x) {}
  Cf(float x) : v(x) {}
  Cf(int x) : v(x) {}
};
long long Cf::n = 0;
inline Cf operator+(Cf a, Cf b) { ++Cf::n; return Cf(a.v + b.v); }
inline Cf operator-(Cf a, Cf b) { ++Cf::n; return Cf(a.v - b.v); }
inline Cf operator*(Cf a, Cf b) { ++Cf::n; return Cf(a.v * b.v); }
inline Cf operator/(Cf a, Cf b) { ++Cf::n; return Cf(a.v / b.v); }
inline Cf operator-(Cf a) { return Cf(-a.v); }
inline Cf& operator+=(Cf& a, Cf b) { a = a + b; return a; }
inline Cf& operator-=(Cf& a, Cf b) { a = a - b; return a; }
inline bool operator>(Cf a, Cf b) { return a.v > b.v; }
inline bool operator<=(Cf a, Cf b) { return a.v <= b.v; }
inline bool operator<(Cf a, Cf b) { return a.v < b.v; }
inline Cf m_sqrt(Cf x) { ++Cf::n; return Cf(std::sqrt(x.v)); }
inline Cf m_tanh(Cf x) { ++Cf::n; return Cf(std::tanh(x.v)); }
inline void m_sincos(Cf x, Cf* s, Cf* c) { Cf::n += 2; *s = Cf(std::sin(x.v)); *c = Cf(std::cos(x.v)); }
inline Cf m_fabs(Cf x) { return Cf(std::fabs(x.v)); }
inline Cf m_fmax(Cf a, Cf b) { return Cf(std::fmax(a.v, b.v)); }
inline Cf m_fmin(Cf a, Cf b) { return Cf(std::fmin(a.v, b.v)); }

template <class T> static void add_out(LegOut<T>& a, const LegOut<T>& b) {
  add_to(a.I, b.I);
  a.p.w = a.p.w + b.p.w;
  a.p.v = a.p.v + b.p.v;
}

// ABA = false: the kernel's condensed legs, act = the twelve joint targets (joint_target);
// true: the oracle's articulated-body algorithm, act = the twelve actions.
template <bool ABA, class T>
static void substep(const DevModel& M, BaseState<T>& B, LegState<T> L[4], const BaseParams<T>& bp,
                    const LegParams<T> lp[4], const T act[12]) {
  LegWork<T> W[4];
  aba::AbaWork<T> Wa[4];
  SV<T> a0;
  if (ABA) {
    LegOut<T> o[4];
    for (int leg = 0; leg < 4; ++leg) o[leg] = aba::phase_a_aba(M, leg, B, L[leg], lp[leg], act + 3 * leg, Wa[leg]);
    add_out(o[0], o[1]);
    add_out(o[2], o[3]);
    add_out(o[0], o[2]);
    a0 = phase_b(M, bp, o[0], B);
  } else {
    // as the lane-per-rollout kernel: the legs summed onto the base body's own terms in order
    LegOut<T> sum = base_terms(bp, B);
    const bool corners = corners_may_touch(M, B);
    for (int leg = 0; leg < 4; ++leg) phase_a_into(M, leg, B, L[leg], lp[leg], act + 3 * leg, W[leg], sum, corners);
    a0 = base_solve(M, sum.I, sum.p, B);
  }
  for (int leg = 0; leg < 4; ++leg) {
    if (ABA) aba::phase_c_aba(M, leg, a0, Wa[leg], L[leg]);
    else phase_c(M, leg, a0, W[leg], L[leg]);
  }
}

template <class T>
static void load_rollout(const DevModel& M, const double* x, const double* th, BaseState<T>& B,
                         LegState<T> L[4], BaseParams<T>& bp, LegParams<T> lp[4]) {
  T s13[13], t[SPI_THETA_DIM];
  for (int i = 0; i < 13; ++i) s13[i] = T(x[i]);
  for (int i = 0; i < SPI_THETA_DIM; ++i) t[i] = T(th[i]);
  base_from_world(B, s13);
  for (int leg = 0; leg < 4; ++leg) {
    for (int k = 0; k < 3; ++k) {
      L[leg].q[k] = T(x[13 + 3 * leg + k]);
      L[leg].qd[k] = T(x[25 + 3 * leg + k]);
    }
    lp[leg] = leg_params<T>(t, leg);
  }
  bp = base_params<T>(M, t);
}

}  // namespace spi

using namespace spi;

template <bool ABA, class T>
static int hostemu_rollout(const spi_robot* robot, const double* init, const double* actions,
                           const double* theta, int nb, int H, double* trace) {
  DevModel M;
  const char* why = "";
  int rc = build_dev_model(*robot, &M, &why);
  if (rc) return rc;
  for (int b = 0; b < nb; ++b) {
    BaseState<T> B;
    LegState<T> L[4];
    BaseParams<T> bp;
    LegParams<T> lp[4];
    load_rollout(M, init + (size_t)b * SPI_STATE_DIM, theta + (size_t)b * SPI_THETA_DIM, B, L, bp, lp);
    for (int h = 0; h < H; ++h) {
      const double* a = actions + ((size_t)b * H + h) * 12;
      T act[12];
      for (int j = 0; j < 12; ++j) act[j] = ABA ? T(a[j]) : joint_target(M, j % 3, j / 3, T(a[j]));
      for (int s = 0; s < M.decimation; ++s) substep<ABA>(M, B, L, bp, lp, act);
      double* out = trace + ((size_t)b * H + h) * SPI_STATE_DIM;
      T s13[13];
      base_to_world(B, s13);
      for (int i = 0; i < 13; ++i) out[i] = s13[i];
      for (int leg = 0; leg < 4; ++leg)
        for (int k = 0; k < 3; ++k) {
          out[13 + 3 * leg + k] = L[leg].q[k];
          out[25 + 3 * leg + k] = L[leg].qd[k];
        }
    }
  }
  return SPI_OK;
}

template <bool ABA>
static int count_ops(const spi_robot* robot, const double* state, const double* theta, const double* act12,
                     long long* per_substep, long long* per_rollout_setup) {
  DevModel M;
  const char* why = "";
  int rc = build_dev_model(*robot, &M, &why);
  if (rc) return rc;
  BaseState<Cf> B;
  LegState<Cf> L[4];
  BaseParams<Cf> bp;
  LegParams<Cf> lp[4];
  Cf::n = 0;
  load_rollout(M, state, theta, B, L, bp, lp);
  if (per_rollout_setup) *per_rollout_setup = Cf::n;
  // the joint targets are formed once per control step, outside the substep counted here
  Cf act[12];
  for (int j = 0; j < 12; ++j) act[j] = ABA ? Cf(act12[j]) : joint_target(M, j % 3, j / 3, Cf(act12[j]));
  Cf::n = 0;
  substep<ABA>(M, B, L, bp, lp, act);
  if (per_substep) *per_substep = Cf::n;
  return SPI_OK;
}

extern "C" {

// Rollouts through the kernel's phases on the host: init [B][37], actions [B][H][12],
// theta [B][13] -> trace [B][H][37]; FP64, and FP32 (the device's arithmetic type).
int spi_hostemu_rollout(const spi_robot* robot, const double* init, const double* actions,
                        const double* theta, int nb, int H, double* trace) {
  return hostemu_rollout<false, double>(robot, init, actions, theta, nb, H, trace);
}
int spi_hostemu_rollout_f32(const spi_robot* robot, const double* init, const double* actions,
                            const double* theta, int nb, int H, double* trace) {
  return hostemu_rollout<false, float>(robot, init, actions, theta, nb, H, trace);
}
// The same rollouts with the legs by the articulated-body algorithm (FP64).
int spi_hostemu_rollout_aba(const spi_robot* robot, const double* init, const double* actions,
                            const double* theta, int nb, int H, double* trace) {
  return hostemu_rollout<true, double>(robot, init, actions, theta, nb, H, trace);
}

// FP operations the kernel executes in one physics substep (whole rollout, phase B counted
// once) and in the per-rollout setup (theta -> base inertia, world -> body velocity).
int spi_hostemu_count_ops(const spi_robot* robot, const double* state, const double* theta,
                          const double* act12, long long* per_substep, long long* per_rollout_setup) {
  return count_ops<false>(robot, state, theta, act12, per_substep, per_rollout_setup);
}
// The same for the oracle's formulation (legs by the articulated-body algorithm): the
// algorithmic count.
int spi_hostemu_count_ops_aba(const spi_robot* robot, const double* state, const double* theta,
                              const double* act12, long long* per_substep, long long* per_rollout_setup) {
  return count_ops<true>(robot, state, theta, act12, per_substep, per_rollout_setup);
}

// Algorithmic FP operations of one substep per phase: [A (all four legs), B (base), C (all legs)].
int spi_hostemu_count_phases(const spi_robot* robot, const double* state, const double* theta,
                             const double* act12, long long* out3) {
  DevModel M;
  const char* why = "";
  int rc = build_dev_model(*robot, &M, &why);
  if (rc) return rc;
  BaseState<Cf> B;
  LegState<Cf> L[4];
  BaseParams<Cf> bp;
  LegParams<Cf> lp[4];
  load_rollout(M, state, theta, B, L, bp, lp);
  Cf act[12];
  for (int j = 0; j < 12; ++j) act[j] = joint_target(M, j % 3, j / 3, Cf(act12[j]));
  LegWork<Cf> W[4];
  Cf::n = 0;
  LegOut<Cf> sum = base_terms(bp, B);
  const bool corners = corners_may_touch(M, B);
  for (int leg = 0; leg < 4; ++leg) phase_a_into(M, leg, B, L[leg], lp[leg], act + 3 * leg, W[leg], sum, corners);
  out3[0] = Cf::n;
  Cf::n = 0;
  SV<Cf> a0 = base_solve(M, sum.I, sum.p, B);
  out3[1] = Cf::n;
  Cf::n = 0;
  for (int leg = 0; leg < 4; ++leg) phase_c(M, leg, a0, W[leg], L[leg]);
  out3[2] = Cf::n;
  return SPI_OK;
}

}  // extern "C"
