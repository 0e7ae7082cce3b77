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

#include <vector>

#include "aba_reference.h"
#include "adjoint.cuh"
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

// Counting dual number: value and one tangent, each operation as the device's forward-mode
// scalar (dual.cuh) evaluates it, every + - * / sqrt tanh sin cos counted once.
struct Cd {
  Cf v, d;
  Cd() {}
  Cd(double x) : v(x), d(0.0) {}
  Cd(float x) : v(x), d(0.0) {}
  Cd(int x) : v(x), d(0.0) {}
  Cd(Cf a, Cf b) : v(a), d(b) {}
};
inline Cd operator+(Cd a, Cd b) { return Cd(a.v + b.v, a.d + b.d); }
inline Cd operator-(Cd a, Cd b) { return Cd(a.v - b.v, a.d - b.d); }
inline Cd operator*(Cd a, Cd b) { return Cd(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Cd operator/(Cd a, Cd b) {
  const Cf q = a.v / b.v;
  return Cd(q, (a.d - q * b.d) / b.v);
}
inline Cd operator-(Cd a) { return Cd(-a.v, -a.d); }
inline Cd& operator+=(Cd& a, Cd b) { a = a + b; return a; }
inline Cd& operator-=(Cd& a, Cd b) { a = a - b; return a; }
inline bool operator>(Cd a, Cd b) { return a.v > b.v; }
inline bool operator<=(Cd a, Cd b) { return a.v <= b.v; }
inline bool operator<(Cd a, Cd b) { return a.v < b.v; }
inline Cd m_sqrt(Cd x) {
  const Cf r = m_sqrt(x.v);
  return Cd(r, r.v > 0 ? x.d * Cf(0.5) / r : Cf(0.0));
}
inline Cd m_tanh(Cd x) {
  const Cf t = m_tanh(x.v);
  return Cd(t, x.d * (Cf(1.0) - t * t));
}
inline void m_sincos(Cd x, Cd* s, Cd* c) {
  Cf sv, cv;
  m_sincos(x.v, &sv, &cv);
  *s = Cd(sv, cv * x.d);
  *c = Cd(cv, -sv * x.d);
}
inline Cd m_fabs(Cd x) { return x.v.v >= 0 ? x : Cd(-x.v, -x.d); }
inline Cd m_fmax(Cd a, Cd b) { return a.v.v >= b.v.v ? a : b; }
inline Cd m_fmin(Cd a, Cd b) { return a.v.v <= b.v.v ? a : b; }

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

// The adjoint of one substep (adjoint.cuh), legs in a loop: lam / lq / lqd hold the adjoint of
// the state after the substep on entry and of the state before it (B0, L0) on exit; the theta
// adjoint accumulates into gth.
template <class T>
static void substep_vjp(const DevModel& M, const BaseState<T>& B0, const LegState<T> L0[4], const BaseParams<T>& bp,
                        const LegParams<T> lp[4], const T* th, const T tgt[12], adj::BaseAdj<T>& lam, T lq[4][3],
                        T lqd[4][3], T* gth) {
  adj::SolveWork<T> W[4];
  LegOut<T> sum = base_terms(bp, B0);
  const bool corners = corners_may_touch(M, B0);
  for (int leg = 0; leg < 4; ++leg) phase_a_into(M, leg, B0, L0[leg], lp[leg], tgt + 3 * leg, W[leg], sum, corners);
  const Art<T> IA = sum.I;
  BaseState<T> B1 = B0;
  const SV<T> a0 = base_solve(M, sum.I, sum.p, B1);
  T qdd[4][3];
  for (int leg = 0; leg < 4; ++leg) adj::leg_qdd(W[leg], a0, qdd[leg]);
  // integrator backwards
  adj::BaseAdj<T> lam0;
  SV<T> a0b;
  M3<T> R0b = adj::zm3<T>();
  adj::base_integrate_bar(M, B0, B1, lam, lam0, a0b, R0b);
  T qb0[4][3], qdb0[4][3], qddb[4][3];
  for (int leg = 0; leg < 4; ++leg) adj::leg_integrate_bar(M, lq[leg], lqd[leg], qb0[leg], qdb0[leg], qddb[leg]);
  // mu = M'^-1 (a0b; qddb)
  T z[4][3];
  SV<T> rhs = a0b;
  for (int leg = 0; leg < 4; ++leg) rhs = adj::sub_sv(rhs, adj::leg_solve_down(W[leg], qddb[leg], z[leg]));
  const SV<T> mub = adj::art_solve(IA, rhs);
  T mu[4][3];
  for (int leg = 0; leg < 4; ++leg) adj::leg_solve_up(W[leg], z[leg], mub, mu[leg]);
  // residual backwards with the seed mu
  adj::BaseBar<T> bb = adj::zero_base_bar<T>();
  for (int leg = 0; leg < 4; ++leg) {
    adj::LegTape<T> t;
    T r[3];
    SV<T> fb;
    adj::leg_residual<kMotorRuntime>(M, leg, B0, L0[leg], lp[leg], tgt + 3 * leg, a0, qdd[leg], t, r, fb);
    T qb[3] = {T(0), T(0), T(0)}, qdb[3] = {T(0), T(0), T(0)};
    adj::LegParamBar<T> pb = {T(0), T(0), T(0), T(0)};
    adj::leg_residual_bar<kMotorRuntime>(M, leg, B0, L0[leg], lp[leg], tgt + 3 * leg, a0, qdd[leg], t, mu[leg], mub,
                                         bb, qb, qdb, pb);
    if (corners)
      for (int j = 0; j < 2; ++j) adj::corner_residual_bar(M, B0, lc_corner<T>(M.legc[leg], j), a0, mub, bb);
    for (int k = 0; k < 3; ++k) {
      lq[leg][k] = qb0[leg][k] - qb[k];
      lqd[leg][k] = qdb0[leg][k] - qdb[k];
    }
    const int g = leg >= 2 ? 9 : 5;
    gth[g] -= pb.kps; gth[g + 1] -= pb.fc; gth[g + 2] -= pb.arm; gth[g + 3] -= pb.ts;
  }
  T mb = T(0);
  V3<T> hb = adj::z3<T>();
  S3<T> Iob;
  Iob.xx = Iob.yy = Iob.zz = Iob.xy = Iob.xz = Iob.yz = T(0);
  adj::base_residual_bar(bp, B0, a0, mub, bb, mb, hb, Iob);
  T gb[5] = {T(0), T(0), T(0), T(0), T(0)};
  adj::base_params_bar(M, th, mb, hb, Iob, gb);
  for (int i = 0; i < 5; ++i) gth[i] -= gb[i];
  lam0.p.z -= bb.pz;
  lam0.nu = adj::sub_sv(lam0.nu, bb.nu);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R0b.m[i][j] -= bb.R.m[i][j];
  adj::quat_to_R_bar(B0.qx, B0.qy, B0.qz, B0.qw, R0b, lam0.qx, lam0.qy, lam0.qz, lam0.qw);
  lam = lam0;
}

// Squared-error (mode 1, per-component weights qw [37]) or reference L2 (mode 0: 10 |dp| +
// 5 |dquat| + |dq|) cost of a final world-frame state, and its adjoint.
template <class T> static T final_cost(const T* s, const double* tgt, const double* qw, int mode, T* sb) {
  T d[SPI_STATE_DIM];
  for (int i = 0; i < SPI_STATE_DIM; ++i) { d[i] = s[i] - T(tgt[i]); sb[i] = T(0); }
  if (mode == 1) {
    T c = T(0);
    for (int i = 0; i < SPI_STATE_DIM; ++i) { c += T(qw[i]) * d[i] * d[i]; sb[i] = T(2) * T(qw[i]) * d[i]; }
    return c;
  }
  const int lo[3] = {0, 3, 13}, hi[3] = {3, 7, 25};
  const double coef[3] = {10.0, 5.0, 1.0};
  T c = T(0);
  for (int b = 0; b < 3; ++b) {
    T n2 = T(0);
    for (int i = lo[b]; i < hi[b]; ++i) n2 += d[i] * d[i];
    const T n = std::sqrt(n2);
    c += T(coef[b]) * n;
    if (n > T(0))
      for (int i = lo[b]; i < hi[b]; ++i) sb[i] = T(coef[b]) * d[i] / n;
  }
  return c;
}

}  // namespace spi

using namespace spi;

// Cost of each rollout's final state and its gradient in theta by the adjoint (all substep
// states kept: the host has the memory; the device kernel recomputes from checkpoints).
template <class T>
static int hostemu_grad(const spi_robot* robot, const double* init, const double* actions, const double* theta,
                        const double* target, const double* qw, int mode, int nb, int H, double* cost,
                        double* grad) {
  DevModel M;
  const char* why = "";
  int rc = build_dev_model(*robot, &M, &why);
  if (rc) return rc;
  const int dec = M.decimation;
  for (int b = 0; b < nb; ++b) {
    BaseState<T> B;
    LegState<T> L[4];
    BaseParams<T> bp;
    LegParams<T> lp[4];
    load_rollout(M, init + (size_t)b * SPI_STATE_DIM, theta + (size_t)b * SPI_THETA_DIM, B, L, bp, lp);
    T th[SPI_THETA_DIM];
    for (int i = 0; i < SPI_THETA_DIM; ++i) th[i] = T(theta[(size_t)b * SPI_THETA_DIM + i]);
    std::vector<BaseState<T>> Bs;
    std::vector<LegState<T>> Ls;
    std::vector<T> tgts((size_t)H * 12);
    for (int h = 0; h < H; ++h) {
      const double* a = actions + ((size_t)b * H + h) * 12;
      T* tg = &tgts[(size_t)h * 12];
      for (int j = 0; j < 12; ++j) tg[j] = joint_target(M, j % 3, j / 3, T(a[j]));
      for (int s = 0; s < dec; ++s) {
        Bs.push_back(B);
        for (int leg = 0; leg < 4; ++leg) Ls.push_back(L[leg]);
        substep<false>(M, B, L, bp, lp, tg);
      }
    }
    T s[SPI_STATE_DIM], sb[SPI_STATE_DIM];
    base_to_world(B, s);
    for (int leg = 0; leg < 4; ++leg)
      for (int k = 0; k < 3; ++k) {
        s[13 + 3 * leg + k] = L[leg].q[k];
        s[25 + 3 * leg + k] = L[leg].qd[k];
      }
    cost[b] = (double)final_cost(s, target + (size_t)b * SPI_STATE_DIM, qw, mode, sb);
    adj::BaseAdj<T> lam = adj::base_to_world_bar(B, sb);
    T lq[4][3], lqd[4][3], gth[SPI_THETA_DIM];
    for (int leg = 0; leg < 4; ++leg)
      for (int k = 0; k < 3; ++k) {
        lq[leg][k] = sb[13 + 3 * leg + k];
        lqd[leg][k] = sb[25 + 3 * leg + k];
      }
    for (int i = 0; i < SPI_THETA_DIM; ++i) gth[i] = T(0);
    for (int j = H * dec - 1; j >= 0; --j)
      substep_vjp(M, Bs[j], &Ls[(size_t)j * 4], bp, lp, th, &tgts[(size_t)(j / dec) * 12], lam, lq, lqd, gth);
    for (int i = 0; i < SPI_THETA_DIM; ++i) grad[(size_t)b * SPI_THETA_DIM + i] = (double)gth[i];
  }
  return SPI_OK;
}

// The residual r(x, theta, a) at the accelerations the forward substep computes: [4][3] joint
// residuals and the base's 6 (near zero up to rounding when the residual is the forward's model).
static int hostemu_residual(const spi_robot* robot, const double* state, const double* theta, const double* act12,
                            double* out18) {
  DevModel M;
  const char* why = "";
  int rc = build_dev_model(*robot, &M, &why);
  if (rc) return rc;
  BaseState<double> B;
  LegState<double> L[4];
  BaseParams<double> bp;
  LegParams<double> lp[4];
  load_rollout(M, state, theta, B, L, bp, lp);
  double tgt[12];
  for (int j = 0; j < 12; ++j) tgt[j] = joint_target(M, j % 3, j / 3, act12[j]);
  adj::SolveWork<double> W[4];
  LegOut<double> sum = base_terms(bp, B);
  const bool corners = corners_may_touch(M, B);
  for (int leg = 0; leg < 4; ++leg) phase_a_into(M, leg, B, L[leg], lp[leg], tgt + 3 * leg, W[leg], sum, corners);
  BaseState<double> B1 = B;
  const SV<double> a0 = base_solve(M, sum.I, sum.p, B1);
  SV<double> rb = rigid_mul(bp.m, bp.h, bp.Io, a0);
  adj::add_sv(rb, crf(B.nu, rigid_mul(bp.m, bp.h, bp.Io, B.nu)));
  for (int leg = 0; leg < 4; ++leg) {
    double qdd[3], r[3];
    adj::leg_qdd(W[leg], a0, qdd);
    adj::LegTape<double> t;
    SV<double> fb;
    adj::leg_residual<kMotorRuntime>(M, leg, B, L[leg], lp[leg], tgt + 3 * leg, a0, qdd, t, r, fb);
    adj::add_sv(rb, fb);
    for (int k = 0; k < 3; ++k) out18[3 * leg + k] = r[k];
    for (int j = 0; j < 2; ++j) {   // corners: P(mc, rc) a0 - (rc x Fb; Fb)
      const V3<double> rc = lc_corner<double>(M.legc[leg], j);
      const V3<double> vc = cross_acc(B.nu.w, rc, B.nu.v);
      const double zc = B.p.z + B.R.m[2][0] * rc.x + B.R.m[2][1] * rc.y + B.R.m[2][2] * rc.z;
      double mc;
      const V3<double> Fw = contact_force_local(M, 0.0, zc, mul(B.R, vc), v3(0.0, 0.0, 1.0), &mc);
      const V3<double> Fb = mulT(B.R, Fw);
      RI<double> Pu;
      Pu.m = 1.0; Pu.h = rc;
      Pu.I.xx = rc.y * rc.y + rc.z * rc.z; Pu.I.yy = rc.x * rc.x + rc.z * rc.z; Pu.I.zz = rc.x * rc.x + rc.y * rc.y;
      Pu.I.xy = -rc.x * rc.y; Pu.I.xz = -rc.x * rc.z; Pu.I.yz = -rc.y * rc.z;
      adj::add_sv(rb, mc * ri_mul(Pu, a0));
      rb.w = rb.w - cross(rc, Fb);
      rb.v = rb.v - Fb;
    }
  }
  out18[12] = rb.w.x; out18[13] = rb.w.y; out18[14] = rb.w.z;
  out18[15] = rb.v.x; out18[16] = rb.v.y; out18[17] = rb.v.z;
  return SPI_OK;
}

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

// Cost and d cost / d theta by the hand-written adjoint, FP64: init [B][37], actions [B][H][12],
// theta [B][13], target [B][37], qw [37] (mode 1) -> cost [B], grad [B][13].
int spi_hostemu_grad(const spi_robot* robot, const double* init, const double* actions, const double* theta,
                     const double* target, const double* qw, int mode, int nb, int H, double* cost, double* grad) {
  return hostemu_grad<double>(robot, init, actions, theta, target, qw, mode, nb, H, cost, grad);
}
// The equations-of-motion residual at the forward substep's accelerations (see hostemu_residual).
int spi_hostemu_residual(const spi_robot* robot, const double* state, const double* theta, const double* act12,
                         double* out18) {
  return hostemu_residual(robot, state, theta, act12, out18);
}

// FP operations of one substep on the forward-mode dual scalar (value + one tangent), phase B
// counted once: the work of one sensitivity direction per substep.
int spi_hostemu_count_ops_dual(const spi_robot* robot, const double* state, const double* theta,
                               const double* act12, long long* per_substep) {
  DevModel M;
  const char* why = "";
  int rc = build_dev_model(*robot, &M, &why);
  if (rc) return rc;
  BaseState<Cd> B;
  LegState<Cd> L[4];
  BaseParams<Cd> bp;
  LegParams<Cd> lp[4];
  load_rollout(M, state, theta, B, L, bp, lp);
  Cd act[12];
  for (int j = 0; j < 12; ++j) act[j] = joint_target(M, j % 3, j / 3, Cd(act12[j]));
  Cf::n = 0;
  substep<false>(M, B, L, bp, lp, act);
  *per_substep = Cf::n;
  return SPI_OK;
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
