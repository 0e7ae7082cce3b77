// adjoint.cuh -- hand-written reverse sweep (adjoint) of one physics substep.
//
// A substep maps the state x = (base position p, quaternion, base spatial velocity nu, joint
// angles q, joint velocities qd) to x' through the accelerations a = (a0, qdd) that solve the
// equations of motion r(x, theta, a) = 0, where
//   r(x, theta, a) = M'(x, theta) a + b(x, theta) - tau(x, theta)
// is the recursive Newton-Euler residual of the same model the forward kernel condenses (leg
// bodies, the base, the contacts' implicit point masses, armature, motor torques; accelerations
// in the gravity-shifted frame), and then integrates (semi-implicit Euler, quaternion
// renormalised). Given the adjoint lambda' of x', the reverse sweep
//   1. recomputes the forward substep from x (phase A / B of dynamics.cuh), keeping the leg
//      factorisation (L, D^-1, K') and the base articulated inertia,
//   2. runs the integrator backwards: lambda_x (direct) and lambda_a,
//   3. solves mu = M'^-1 lambda_a with that factorisation (M' is symmetric),
//   4. runs the residual forward (keeping its intermediates) and backwards with the seed mu:
//      lambda_x -= (dr/dx)^T mu,  lambda_theta -= (dr/dtheta)^T mu
// (a = FD(x) with r(x, a) = 0 gives da/dx = -M'^-1 dr/dx). Every reverse helper below is the
// transpose of the forward helper of the same name in dynamics.cuh, written out by hand; the
// non-smooth operations take the derivative of the branch the forward selected (clip, max,
// contact on / off, stick / slip), as the forward-mode scalar does.
//
// Templated on the scalar type: the device kernel (adjoint.cu) runs it in FP32 with one lane
// per leg; the host emulation (hostemu.cpp) runs it in FP64 with the legs in a loop, which is
// how the tests check it against finite differences.
#pragma once

#include "dynamics.cuh"

namespace spi {
namespace adj {

template <class T> SPI_INL V3<T> z3() { return v3(T(0), T(0), T(0)); }
template <class T> SPI_INL SV<T> zsv() { SV<T> r; r.w = z3<T>(); r.v = z3<T>(); return r; }
template <class T> SPI_INL T sdot(const SV<T>& a, const SV<T>& b) { return dot(a.w, b.w) + dot(a.v, b.v); }
template <class T> SPI_INL void add_sv(SV<T>& a, const SV<T>& b) { a.w = a.w + b.w; a.v = a.v + b.v; }
template <class T> SPI_INL SV<T> sub_sv(const SV<T>& a, const SV<T>& b) {
  SV<T> r; r.w = a.w - b.w; r.v = a.v - b.v; return r;
}

// ---------------------------------------------------------------------------
// transposes of the spatial helpers
// ---------------------------------------------------------------------------
// o = rot<AX>(c, s, u): ub += R^T ob, and the angle terms.
template <int AX, class T> SPI_INL void rot_bar(T c, T s, V3<T> u, V3<T> ob, V3<T>& ub, T& cb, T& sb) {
  ub = ub + rotT<AX>(c, s, ob);
  if (AX == 0) { cb += ob.y * u.y + ob.z * u.z; sb += ob.z * u.y - ob.y * u.z; }
  else { cb += ob.x * u.x + ob.z * u.z; sb += ob.x * u.z - ob.z * u.x; }
}
// o = rotT<AX>(c, s, u)
template <int AX, class T> SPI_INL void rotT_bar(T c, T s, V3<T> u, V3<T> ob, V3<T>& ub, T& cb, T& sb) {
  ub = ub + rot<AX>(c, s, ob);
  if (AX == 0) { cb += ob.y * u.y + ob.z * u.z; sb += ob.y * u.z - ob.z * u.y; }
  else { cb += ob.x * u.x + ob.z * u.z; sb += ob.z * u.x - ob.x * u.z; }
}
// o = motion_to_child<AX>(m, c, s, r): o.w = R^T m.w, o.v = R^T (m.v - r x m.w)
template <int AX, class T>
SPI_INL void motion_to_child_bar(const SV<T>& m, T c, T s, V3<T> r, const SV<T>& ob, SV<T>& mb, T& cb, T& sb) {
  const V3<T> u = m.v - cross(r, m.w);
  V3<T> ub = z3<T>();
  rotT_bar<AX>(c, s, u, ob.v, ub, cb, sb);
  rotT_bar<AX>(c, s, m.w, ob.w, mb.w, cb, sb);
  mb.v = mb.v + ub;
  mb.w = mb.w + cross(r, ub);
}
// o = force_to_parent<AX>(f, c, s, r): o.v = R f.v, o.w = R f.w + r x o.v
template <int AX, class T>
SPI_INL void force_to_parent_bar(const SV<T>& f, T c, T s, V3<T> r, const SV<T>& ob, SV<T>& fb, T& cb, T& sb) {
  const V3<T> ovb = ob.v - cross(r, ob.w);
  rot_bar<AX>(c, s, f.w, ob.w, fb.w, cb, sb);
  rot_bar<AX>(c, s, f.v, ovb, fb.v, cb, sb);
}
// o = crf(v, f)
template <class T> SPI_INL void crf_bar(const SV<T>& v, const SV<T>& f, const SV<T>& ob, SV<T>& vb, SV<T>& fb) {
  vb.w = vb.w + cross(f.w, ob.w) + cross(f.v, ob.v);
  vb.v = vb.v + cross(f.v, ob.w);
  fb.w = fb.w + cross(ob.w, v.w);
  fb.v = fb.v + cross(ob.w, v.v) + cross(ob.v, v.w);
}
// o = vel_product<AX>(v, qd)
template <int AX, class T> SPI_INL void vel_product_bar(const SV<T>& v, T qd, const SV<T>& ob, SV<T>& vb, T& qdb) {
  if (AX == 0) {   // (0, w.z qd, -w.y qd; 0, v.z qd, -v.y qd)
    vb.w.z += ob.w.y * qd; vb.w.y -= ob.w.z * qd;
    vb.v.z += ob.v.y * qd; vb.v.y -= ob.v.z * qd;
    qdb += ob.w.y * v.w.z - ob.w.z * v.w.y + ob.v.y * v.v.z - ob.v.z * v.v.y;
  } else {         // (-w.z qd, 0, w.x qd; -v.z qd, 0, v.x qd)
    vb.w.z -= ob.w.x * qd; vb.w.x += ob.w.z * qd;
    vb.v.z -= ob.v.x * qd; vb.v.x += ob.v.z * qd;
    qdb += ob.w.z * v.w.x - ob.w.x * v.w.z + ob.v.z * v.v.x - ob.v.x * v.v.z;
  }
}
// Parameters of o = rigid_mul(m, h, Io, v): mb, hb, Iob (the input v's adjoint is rigid_mul(m, h,
// Io, ob) by symmetry of the spatial inertia).
template <class T>
SPI_INL void rigid_mul_params_bar(const SV<T>& v, const SV<T>& ob, T& mb, V3<T>& hb, S3<T>& Iob) {
  mb += dot(ob.v, v.v);
  hb = hb + cross(v.v, ob.w) + cross(ob.v, v.w);
  Iob.xx += ob.w.x * v.w.x; Iob.yy += ob.w.y * v.w.y; Iob.zz += ob.w.z * v.w.z;
  Iob.xy += ob.w.x * v.w.y + ob.w.y * v.w.x;
  Iob.xz += ob.w.x * v.w.z + ob.w.z * v.w.x;
  Iob.yz += ob.w.y * v.w.z + ob.w.z * v.w.y;
}
// R = quat_to_R(x, y, z, w): the quaternion's adjoint from R's (row-major Rb).
template <class T> SPI_INL void quat_to_R_bar(T x, T y, T z, T w, const M3<T>& Rb, T& xb, T& yb, T& zb, T& wb) {
  const T b01 = Rb.m[0][1], b02 = Rb.m[0][2], b10 = Rb.m[1][0], b12 = Rb.m[1][2], b20 = Rb.m[2][0], b21 = Rb.m[2][1];
  const T d0 = Rb.m[0][0], d1 = Rb.m[1][1], d2 = Rb.m[2][2];
  xb += T(2) * (y * (b01 + b10) + z * (b02 + b20) + w * (b21 - b12)) - T(4) * x * (d1 + d2);
  yb += T(2) * (x * (b01 + b10) + z * (b12 + b21) + w * (b02 - b20)) - T(4) * y * (d0 + d2);
  zb += T(2) * (x * (b02 + b20) + y * (b12 + b21) + w * (b10 - b01)) - T(4) * z * (d0 + d1);
  wb += T(2) * (x * (b21 - b12) + y * (b02 - b20) + z * (b10 - b01));
}
template <class T> SPI_INL void outer_add(M3<T>& A, V3<T> a, V3<T> b) {   // A += a b^T
  A.m[0][0] += a.x * b.x; A.m[0][1] += a.x * b.y; A.m[0][2] += a.x * b.z;
  A.m[1][0] += a.y * b.x; A.m[1][1] += a.y * b.y; A.m[1][2] += a.y * b.z;
  A.m[2][0] += a.z * b.x; A.m[2][1] += a.z * b.y; A.m[2][2] += a.z * b.z;
}
template <class T> SPI_INL M3<T> zm3() {
  M3<T> A;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A.m[i][j] = T(0);
  return A;
}

// Penalty contact (contact_force_local of dynamics.cuh; with n = e_z it is also contact_force
// plus the caller's mimp g): the adjoints of z, v and n from those of F and mimp.
template <class T>
SPI_INL void contact_local_bar(const DevModel& M, T radius, T z, V3<T> v, V3<T> n, V3<T> Fb, T mb, T& zb,
                               V3<T>& vb, V3<T>& nb) {
  const T vz = dot(n, v);
  const V3<T> vt = v3(v.x - vz * n.x, v.y - vz * n.y, v.z - vz * n.z);
  const T pen = radius - z;
  const T sarg = pen * T(M.ramp_inv);
  const T s = m_clamp(sarg, T(0), T(1));
  const T fnarg = T(M.k) * pen - T(M.c) * s * vz;
  const T fn = m_fmax(T(0), fnarg);
  const T vtn = m_sqrt(dot(vt, vt));
  const T lim = T(M.mu) * fn;
  const bool stick = T(M.ct) * vtn <= lim;
  const T scale = stick ? T(M.ct) : lim / vtn;
  const T dmds = m_mul2_c(T(1), M.dt, M.imp_c, M.dt_imp_c);
  const T mimp = s * dmds;
  const T fz = fn + mimp * T(M.g);
  // F = fz n - scale vt
  const T fzb = dot(Fb, n);
  nb = nb + fz * Fb;
  V3<T> vtb = (-scale) * Fb;
  const T scaleb = -dot(Fb, vt);
  T fnb = fzb;
  const T mimpb = mb + fzb * T(M.g);
  if (!stick) {
    const T limb = scaleb / vtn;
    fnb += T(M.mu) * limb;
    const T vtnb = -scaleb * lim / (vtn * vtn);
    vtb = vtb + (vtnb / vtn) * vt;
  }
  T penb = T(0), sb = mimpb * dmds, vzb = T(0);
  if (fnarg > T(0)) {
    penb += T(M.k) * fnb;
    sb += -T(M.c) * vz * fnb;
    vzb += -T(M.c) * s * fnb;
  }
  if (sarg > T(0) && sarg < T(1)) penb += sb * T(M.ramp_inv);
  zb += -penb;
  vb = vb + vtb;
  vzb += -dot(vtb, n);
  nb = nb + (-vz) * vtb;
  nb = nb + vzb * v;
  vb = vb + vzb * n;
}

// Motor torque (motor_torque_at of dynamics.cuh) of joint k: adjoints of q, qd and of the leg's
// Kp scale, friction and torque-limit scale from the torque's.
template <int MS, class T>
SPI_INL void motor_torque_bar(const DevModel& M, const LegParams<T>& P, int k, int leg, T target, T q, T qd,
                              T taub, T& qb, T& qdb, T& kpsb, T& fcb, T& tsb) {
  const F4* lc = M.legc[leg];
  const T Kp = T(M.kp[k][leg]);
  const T kp = P.kp_of(M, k, leg);
  const T e = target - q;
  const T kdk = m_mul2_c(T(1), M.kd_scale, M.kd[k][leg], lc[k].w);
  const T tau0 = kp * e - m_mul2_c(qd, M.kd_scale, M.kd[k][leg], lc[k].w);
  const T lim0 = P.lim_of(M, k, leg);
  const bool spd = MS == kMotorSpeedLimit || M.torque_speed;
  T sp = T(1), u = T(1);
  if (spd) {
    u = T(1) - m_div_c(m_fabs(qd), M.vlim[k][leg], lc[5 + 3 * k].z);
    sp = m_fmax(T(0), u);
  }
  const T lim = spd ? lim0 * sp : lim0;
  const T tau1 = m_clamp(tau0, -lim, lim);
  // tau = g(tau1) - fc tanh(qd / w)
  const T tf = m_tanh_div(qd, M.fric_vel, M.fric_k2);
  fcb += -taub * tf;
  qdb += -taub * P.fc * (T(1) - tf * tf) / T(M.fric_vel);
  T t1b = taub;
  if (MS == kMotorRuntime) {
    const T tau2 = tau1 * T(M.gain[k]);
    if (M.tanh_a[k] > 0.0f) {
      const T th = m_tanh(tau2 / T(M.tanh_a[k]));
      t1b = t1b * (T(1) - th * th);
    }
    t1b = t1b * T(M.gain[k]);
  }
  T t0b = T(0), limb = T(0);
  if (tau0 > lim) limb += t1b;
  else if (tau0 < -lim) limb -= t1b;
  else t0b = t1b;
  T lim0b = limb;
  if (spd) {
    lim0b = limb * sp;
    if (u > T(0)) {
      const T ub = limb * lim0;   // d lim / d sp
      const T sgn = qd > T(0) ? T(1) : (qd < T(0) ? T(-1) : T(0));
      qdb += -ub * sgn * m_div_c(T(1), M.vlim[k][leg], lc[5 + 3 * k].z);
    }
  }
  tsb += lim0b * T(M.tlim[k][leg]);
  kpsb += t0b * Kp * e;
  qb += -t0b * kp;
  qdb += -t0b * kdk;
}

// ---------------------------------------------------------------------------
// the residual of one leg (recursive Newton-Euler with the contact's point mass at the foot)
// ---------------------------------------------------------------------------
template <class T> struct LegTape {
  T c[3], s[3];
  SV<T> v0, v1, v2, h0, h1, h2;      // body velocities and I v (the calf's without the point mass)
  SV<T> al0, al1, al2;               // body accelerations (gravity-shifted frame)
  SV<T> f0, f1, f2;                  // body forces, the children's carried in
  V3<T> g0, g1, g2, g3;              // world vertical in the base, hip, thigh, calf frames
  T zf, mimp;
  V3<T> vf, Fc;                      // foot velocity and contact force (calf frame)
};

// r[k]: joint k's residual f_k . S_k + arm qdd_k - tau_k; fb: the leg's force on the base
// (X_0^T f_0). tgt: the three joint targets (joint_target of the actions).
template <int MS, class T>
SPI_INL void leg_residual(const DevModel& M, int leg, const BaseState<T>& B, const LegState<T>& L,
                          const LegParams<T>& P, const T tgt[3], const SV<T>& a0, const T qdd[3], LegTape<T>& t,
                          T r[3], SV<T>& fb) {
  const F4* lc = M.legc[leg];
  const V3<T> r0 = lc_org<T>(lc, 0), r1 = lc_org<T>(lc, 1), r2 = lc_org<T>(lc, 2);
  const V3<T> rf = v3(T(0), T(0), T(M.foot[2]));
  T tau[3];
  for (int k = 0; k < 3; ++k) {
    tau[k] = motor_torque_at<MS>(M, P, k, leg, tgt[k], L.q[k], L.qd[k]);
    m_sincos(L.q[k], &t.s[k], &t.c[k]);
  }
  t.v0 = motion_to_child<0>(B.nu, t.c[0], t.s[0], r0); t.v0.w.x = t.v0.w.x + L.qd[0];
  t.v1 = motion_to_child<1>(t.v0, t.c[1], t.s[1], r1); t.v1.w.y = t.v1.w.y + L.qd[1];
  t.v2 = motion_to_child<1>(t.v1, t.c[2], t.s[2], r2); t.v2.w.y = t.v2.w.y + L.qd[2];
  const SV<T> cb0 = vel_product<0>(t.v0, L.qd[0]), cb1 = vel_product<1>(t.v1, L.qd[1]),
              cb2 = vel_product<1>(t.v2, L.qd[2]);
  t.g0 = row(B.R, 2);
  t.g1 = rotT<0>(t.c[0], t.s[0], t.g0);
  t.g2 = rotT<1>(t.c[1], t.s[1], t.g1);
  t.g3 = rotT<1>(t.c[2], t.s[2], t.g2);
  t.zf = B.p.z + dot(t.g0, r0) + dot(t.g1, r1) + dot(t.g2, r2) + dot(t.g3, rf);
  t.vf = t.v2.v + cross(t.v2.w, rf);
  t.Fc = contact_force_local(M, T(M.foot_r), t.zf, t.vf, t.g3, &t.mimp);
  t.al0 = motion_to_child<0>(a0, t.c[0], t.s[0], r0); t.al0.w.x = t.al0.w.x + qdd[0]; add_sv(t.al0, cb0);
  t.al1 = motion_to_child<1>(t.al0, t.c[1], t.s[1], r1); t.al1.w.y = t.al1.w.y + qdd[1]; add_sv(t.al1, cb1);
  t.al2 = motion_to_child<1>(t.al1, t.c[2], t.s[2], r2); t.al2.w.y = t.al2.w.y + qdd[2]; add_sv(t.al2, cb2);
  const RI<T> Ihp = lc_ri<T>(lc, 0), Ith = lc_ri<T>(lc, 1), Ical = lc_ri<T>(lc, 2);
  t.h0 = ri_mul(Ihp, t.v0);
  t.h1 = ri_mul(Ith, t.v1);
  t.h2 = ri_mul(Ical, t.v2);
  RI<T> Rc2 = Ical;
  {
    const T hz = t.mimp * rf.z;
    Rc2.m = Rc2.m + t.mimp;
    Rc2.h.z = Rc2.h.z + hz;
    Rc2.I.xx = Rc2.I.xx + hz * rf.z;
    Rc2.I.yy = Rc2.I.yy + hz * rf.z;
  }
  t.f2 = ri_mul(Rc2, t.al2);
  add_sv(t.f2, crf(t.v2, t.h2));
  t.f2.w = t.f2.w - cross(rf, t.Fc);
  t.f2.v = t.f2.v - t.Fc;
  t.f1 = ri_mul(Ith, t.al1);
  add_sv(t.f1, crf(t.v1, t.h1));
  add_sv(t.f1, force_to_parent<1>(t.f2, t.c[2], t.s[2], r2));
  t.f0 = ri_mul(Ihp, t.al0);
  add_sv(t.f0, crf(t.v0, t.h0));
  add_sv(t.f0, force_to_parent<1>(t.f1, t.c[1], t.s[1], r1));
  r[0] = t.f0.w.x + P.arm * qdd[0] - tau[0];
  r[1] = t.f1.w.y + P.arm * qdd[1] - tau[1];
  r[2] = t.f2.w.y + P.arm * qdd[2] - tau[2];
  fb = force_to_parent<0>(t.f0, t.c[0], t.s[0], r0);
}

// Adjoints the residual's reverse hands to the base state.
template <class T> struct BaseBar {
  T pz;            // base height
  M3<T> R;         // rotation matrix (row-major)
  SV<T> nu;        // base spatial velocity
};
template <class T> SPI_INL BaseBar<T> zero_base_bar() {
  BaseBar<T> b; b.pz = T(0); b.R = zm3<T>(); b.nu = zsv<T>(); return b;
}
// Adjoints of the leg's motor terms (theta slots of its leg group).
template <class T> struct LegParamBar { T kps, fc, arm, ts; };

// Reverse of leg_residual for the seed mu . r + mub . fb: accumulates into the base adjoints
// bb, the leg's joint adjoints qb / qdb and its motor-term adjoints pb.
template <int MS, class T>
SPI_INL void leg_residual_bar(const DevModel& M, int leg, const BaseState<T>& B, const LegState<T>& L,
                              const LegParams<T>& P, const T tgt[3], const SV<T>& a0, const T qdd[3],
                              const LegTape<T>& t, const T mu[3], const SV<T>& mub, BaseBar<T>& bb, T qb[3],
                              T qdb[3], LegParamBar<T>& pb) {
  const F4* lc = M.legc[leg];
  const V3<T> r0 = lc_org<T>(lc, 0), r1 = lc_org<T>(lc, 1), r2 = lc_org<T>(lc, 2);
  const V3<T> rf = v3(T(0), T(0), T(M.foot[2]));
  const RI<T> Ihp = lc_ri<T>(lc, 0), Ith = lc_ri<T>(lc, 1), Ical = lc_ri<T>(lc, 2);
  T cb[3] = {T(0), T(0), T(0)}, sb[3] = {T(0), T(0), T(0)};
  SV<T> f0b = zsv<T>(), f1b = zsv<T>(), f2b = zsv<T>();
  // fb = X0^T f0; r_k = f_k . S_k + arm qdd_k - tau_k
  force_to_parent_bar<0>(t.f0, t.c[0], t.s[0], r0, mub, f0b, cb[0], sb[0]);
  f0b.w.x += mu[0];
  f1b.w.y += mu[1];
  f2b.w.y += mu[2];
  pb.arm += mu[0] * qdd[0] + mu[1] * qdd[1] + mu[2] * qdd[2];
  // f0 = Ihp al0 + crf(v0, h0) + X1^T f1
  SV<T> al0b = ri_mul(Ihp, f0b), v0b = zsv<T>(), h0b = zsv<T>();
  crf_bar(t.v0, t.h0, f0b, v0b, h0b);
  add_sv(v0b, ri_mul(Ihp, h0b));
  force_to_parent_bar<1>(t.f1, t.c[1], t.s[1], r1, f0b, f1b, cb[1], sb[1]);
  // f1 = Ith al1 + crf(v1, h1) + X2^T f2
  SV<T> al1b = ri_mul(Ith, f1b), v1b = zsv<T>(), h1b = zsv<T>();
  crf_bar(t.v1, t.h1, f1b, v1b, h1b);
  add_sv(v1b, ri_mul(Ith, h1b));
  force_to_parent_bar<1>(t.f2, t.c[2], t.s[2], r2, f1b, f2b, cb[2], sb[2]);
  // f2 = (Ical + mimp point(rf)) al2 + crf(v2, h2) - (rf x Fc; Fc)
  RI<T> Rc2 = Ical;
  {
    const T hz = t.mimp * rf.z;
    Rc2.m = Rc2.m + t.mimp;
    Rc2.h.z = Rc2.h.z + hz;
    Rc2.I.xx = Rc2.I.xx + hz * rf.z;
    Rc2.I.yy = Rc2.I.yy + hz * rf.z;
  }
  SV<T> al2b = ri_mul(Rc2, f2b), v2b = zsv<T>(), h2b = zsv<T>();
  T mimpb;
  {
    RI<T> Pu;   // unit point mass at the foot
    Pu.m = T(1); Pu.h = rf;
    Pu.I.xx = rf.z * rf.z; Pu.I.yy = rf.z * rf.z; Pu.I.zz = T(0); Pu.I.xy = T(0); Pu.I.xz = T(0); Pu.I.yz = T(0);
    mimpb = sdot(f2b, ri_mul(Pu, t.al2));
  }
  crf_bar(t.v2, t.h2, f2b, v2b, h2b);
  add_sv(v2b, ri_mul(Ical, h2b));
  const V3<T> Fcb = cross(rf, f2b.w) - f2b.v;
  // accelerations: al_k = X_k al_{k-1} + S_k qdd_k + cb_k (al_{-1} = a0, fixed)
  SV<T> cb2b = al2b, cb1b, cb0b;
  motion_to_child_bar<1>(t.al1, t.c[2], t.s[2], r2, al2b, al1b, cb[2], sb[2]);
  cb1b = al1b;
  motion_to_child_bar<1>(t.al0, t.c[1], t.s[1], r1, al1b, al0b, cb[1], sb[1]);
  cb0b = al0b;
  {
    SV<T> a0b = zsv<T>();
    motion_to_child_bar<0>(a0, t.c[0], t.s[0], r0, al0b, a0b, cb[0], sb[0]);
  }
  // foot contact
  T zfb = T(0);
  V3<T> vfb = z3<T>(), g3b = z3<T>();
  contact_local_bar(M, T(M.foot_r), t.zf, t.vf, t.g3, Fcb, mimpb, zfb, vfb, g3b);
  bb.pz += zfb;
  V3<T> g0b = zfb * r0, g1b = zfb * r1, g2b = zfb * r2;
  g3b = g3b + zfb * rf;
  v2b.v = v2b.v + vfb;
  v2b.w = v2b.w + cross(rf, vfb);
  rotT_bar<1>(t.c[2], t.s[2], t.g2, g3b, g2b, cb[2], sb[2]);
  rotT_bar<1>(t.c[1], t.s[1], t.g1, g2b, g1b, cb[1], sb[1]);
  rotT_bar<0>(t.c[0], t.s[0], t.g0, g1b, g0b, cb[0], sb[0]);
  bb.R.m[2][0] += g0b.x; bb.R.m[2][1] += g0b.y; bb.R.m[2][2] += g0b.z;
  // velocity products, then velocities
  vel_product_bar<1>(t.v2, L.qd[2], cb2b, v2b, qdb[2]);
  vel_product_bar<1>(t.v1, L.qd[1], cb1b, v1b, qdb[1]);
  vel_product_bar<0>(t.v0, L.qd[0], cb0b, v0b, qdb[0]);
  qdb[2] += v2b.w.y;
  motion_to_child_bar<1>(t.v1, t.c[2], t.s[2], r2, v2b, v1b, cb[2], sb[2]);
  qdb[1] += v1b.w.y;
  motion_to_child_bar<1>(t.v0, t.c[1], t.s[1], r1, v1b, v0b, cb[1], sb[1]);
  qdb[0] += v0b.w.x;
  motion_to_child_bar<0>(B.nu, t.c[0], t.s[0], r0, v0b, bb.nu, cb[0], sb[0]);
  // motor torques (r_k has -tau_k) and the joint angles' sine / cosine
  for (int k = 0; k < 3; ++k) {
    motor_torque_bar<MS>(M, P, k, leg, tgt[k], L.q[k], L.qd[k], -mu[k], qb[k], qdb[k], pb.kps, pb.fc, pb.ts);
    qb[k] += t.c[k] * sb[k] - t.s[k] * cb[k];
  }
}

// One base-box corner (rc in base coordinates): residual term P(mc, rc) a0 - (rc x Fb; Fb) and its
// reverse for the seed mub.
template <class T>
SPI_INL void corner_residual_bar(const DevModel& M, const BaseState<T>& B, V3<T> rc, const SV<T>& a0,
                                 const SV<T>& mub, BaseBar<T>& bb) {
  const V3<T> vc = cross_acc(B.nu.w, rc, B.nu.v);
  const V3<T> vw = mul(B.R, vc);
  const T zc = B.p.z + B.R.m[2][0] * rc.x + B.R.m[2][1] * rc.y + B.R.m[2][2] * rc.z;
  const V3<T> ez = v3(T(0), T(0), T(1));
  T mc;
  const V3<T> Fw = contact_force_local(M, T(0), zc, vw, ez, &mc);
  RI<T> Pu;   // unit point mass at rc
  Pu.m = T(1); Pu.h = rc;
  Pu.I.xx = rc.y * rc.y + rc.z * rc.z; Pu.I.yy = rc.x * rc.x + rc.z * rc.z; Pu.I.zz = rc.x * rc.x + rc.y * rc.y;
  Pu.I.xy = -rc.x * rc.y; Pu.I.xz = -rc.x * rc.z; Pu.I.yz = -rc.y * rc.z;
  const T mcb = sdot(mub, ri_mul(Pu, a0));
  const V3<T> Fbb = cross(rc, mub.w) - mub.v;
  const V3<T> Fwb = mul(B.R, Fbb);                 // Fb = R^T Fw
  outer_add(bb.R, Fw, Fbb);
  T zcb = T(0);
  V3<T> vwb = z3<T>(), nb = z3<T>();
  contact_local_bar(M, T(0), zc, vw, ez, Fwb, mcb, zcb, vwb, nb);
  bb.pz += zcb;
  bb.R.m[2][0] += zcb * rc.x; bb.R.m[2][1] += zcb * rc.y; bb.R.m[2][2] += zcb * rc.z;
  const V3<T> vcb = mulT(B.R, vwb);
  outer_add(bb.R, vwb, vc);
  bb.nu.v = bb.nu.v + vcb;
  bb.nu.w = bb.nu.w + cross(rc, vcb);
}

// The base body's own residual terms I_b a0 + crf(nu, I_b nu) and their reverse for mub:
// adjoints of nu (into bb) and of the base inertia (mb, hb, Iob).
template <class T>
SPI_INL void base_residual_bar(const BaseParams<T>& bp, const BaseState<T>& B, const SV<T>& a0, const SV<T>& mub,
                               BaseBar<T>& bb, T& mb, V3<T>& hb, S3<T>& Iob) {
  rigid_mul_params_bar(a0, mub, mb, hb, Iob);
  const SV<T> h = rigid_mul(bp.m, bp.h, bp.Io, B.nu);
  SV<T> hbar = zsv<T>();
  crf_bar(B.nu, h, mub, bb.nu, hbar);
  add_sv(bb.nu, rigid_mul(bp.m, bp.h, bp.Io, hbar));
  rigid_mul_params_bar(B.nu, hbar, mb, hb, Iob);
}

// theta slots 0..4 from the base inertia's adjoints (base_params of dynamics.cuh).
template <class T>
SPI_INL void base_params_bar(const DevModel& M, const T* th, T mb, V3<T> hb, const S3<T>& Iob, T* gth) {
  const T m = th[0];
  const V3<T> c = v3(T(M.base_com[0]) + th[1], T(M.base_com[1]) + th[2], T(M.base_com[2]) + th[3]);
  const T f = M.inertia_follows_mass ? m / T(M.base_m0) : T(1);
  T m_b = mb + dot(hb, c);
  V3<T> c_b = m * hb;
  m_b += Iob.xx * (c.y * c.y + c.z * c.z) + Iob.yy * (c.x * c.x + c.z * c.z) + Iob.zz * (c.x * c.x + c.y * c.y)
       - Iob.xy * c.x * c.y - Iob.xz * c.x * c.z - Iob.yz * c.y * c.z;
  c_b.x += m * (T(2) * c.x * (Iob.yy + Iob.zz) - Iob.xy * c.y - Iob.xz * c.z);
  c_b.y += m * (T(2) * c.y * (Iob.xx + Iob.zz) - Iob.xy * c.x - Iob.yz * c.z);
  c_b.z += m * (T(2) * c.z * (Iob.xx + Iob.yy) - Iob.xz * c.x - Iob.yz * c.y);
  const T fb = Iob.xx * T(M.base_Ic[0]) * th[4] + Iob.yy * T(M.base_Ic[1]) * th[4] + Iob.zz * T(M.base_Ic[2]) * th[4]
             + Iob.xy * T(M.base_Ic[3]) + Iob.xz * T(M.base_Ic[4]) + Iob.yz * T(M.base_Ic[5]);
  if (M.inertia_follows_mass) m_b += fb / T(M.base_m0);
  gth[0] += m_b;
  gth[1] += c_b.x; gth[2] += c_b.y; gth[3] += c_b.z;
  gth[4] += f * (Iob.xx * T(M.base_Ic[0]) + Iob.yy * T(M.base_Ic[1]) + Iob.zz * T(M.base_Ic[2]));
}

// ---------------------------------------------------------------------------
// the leg factorisation phase A produces, and the solve with it
// ---------------------------------------------------------------------------
template <class T> struct SolveWork {
  SV<T> Kp[3];
  T y[3], i[3];
  T l10, l20, l21;
  SPI_INL void put_col(int k, const SV<T>& v, T yk, T lk) {
    Kp[k] = v;
    y[k] = yk;
    if (k == 0) l10 = lk; else if (k == 1) l20 = lk; else l21 = lk;
  }
  SPI_INL void put_diag(T a, T b, T c) { i[0] = a; i[1] = b; i[2] = c; }
};
// The leg's joint accelerations for the base acceleration a0 (phase C of dynamics.cuh).
template <class T> SPI_INL void leg_qdd(const SolveWork<T>& W, const SV<T>& a0, T qdd[3]) {
  T w[3];
  for (int k = 0; k < 3; ++k) w[k] = W.y[k] - sdot(W.Kp[k], a0);
  qdd[2] = w[2];
  qdd[1] = w[1] - W.l21 * qdd[2];
  qdd[0] = w[0] - W.l10 * qdd[1] - W.l20 * qdd[2];
}
// First half of M'^-1 for one leg: z = L^-1 lam, and K D^-1 z's contribution (sum_k K'_k z_k)
// to the base right-hand side.
template <class T> SPI_INL SV<T> leg_solve_down(const SolveWork<T>& W, const T lam[3], T z[3]) {
  z[0] = lam[0];
  z[1] = lam[1] - W.l10 * z[0];
  z[2] = lam[2] - W.l20 * z[0] - W.l21 * z[1];
  SV<T> s = z[0] * W.Kp[0];
  add_sv(s, z[1] * W.Kp[1]);
  add_sv(s, z[2] * W.Kp[2]);
  return s;
}
// Second half: mu_leg = L^-T (D^-1 z - K'^T mu_base).
template <class T> SPI_INL void leg_solve_up(const SolveWork<T>& W, const T z[3], const SV<T>& mub, T mu[3]) {
  T w[3];
  for (int k = 0; k < 3; ++k) w[k] = W.i[k] * z[k] - sdot(W.Kp[k], mub);
  mu[2] = w[2];
  mu[1] = w[1] - W.l21 * mu[2];
  mu[0] = w[0] - W.l10 * mu[1] - W.l20 * mu[2];
}
// Solve IA x = b for the symmetric positive definite 6x6 articulated inertia, (w; v) order.
template <class T> SPI_INL SV<T> art_solve(const Art<T>& IA, const SV<T>& b) {
  T Mx[6][6];
  Mx[0][0] = IA.A.xx; Mx[1][1] = IA.A.yy; Mx[2][2] = IA.A.zz;
  Mx[1][0] = IA.A.xy; Mx[2][0] = IA.A.xz; Mx[2][1] = IA.A.yz;
  Mx[3][3] = IA.C.xx; Mx[4][4] = IA.C.yy; Mx[5][5] = IA.C.zz;
  Mx[4][3] = IA.C.xy; Mx[5][3] = IA.C.xz; Mx[5][4] = IA.C.yz;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Mx[3 + j][i] = IA.B.m[i][j];
  T x[6] = {b.w.x, b.w.y, b.w.z, b.v.x, b.v.y, b.v.z};
  T invL[6];
  for (int j = 0; j < 6; ++j) {
    T d = Mx[j][j];
    for (int k = 0; k < j; ++k) d = d - Mx[j][k] * Mx[j][k];
    const T inv = T(1) / m_sqrt(d);
    invL[j] = inv;
    for (int i = j + 1; i < 6; ++i) {
      T a = Mx[i][j];
      for (int k = 0; k < j; ++k) a = a - Mx[i][k] * Mx[j][k];
      Mx[i][j] = a * inv;
    }
  }
  for (int i = 0; i < 6; ++i) {
    T a = x[i];
    for (int k = 0; k < i; ++k) a = a - Mx[i][k] * x[k];
    x[i] = a * invL[i];
  }
  for (int i = 5; i >= 0; --i) {
    T a = x[i];
    for (int k = i + 1; k < 6; ++k) a = a - Mx[k][i] * x[k];
    x[i] = a * invL[i];
  }
  SV<T> r;
  r.w = v3(x[0], x[1], x[2]);
  r.v = v3(x[3], x[4], x[5]);
  return r;
}

// ---------------------------------------------------------------------------
// the integrator (base_solve / phase_c of dynamics.cuh) backwards
// ---------------------------------------------------------------------------
// Adjoint of the base state (R is a function of the quaternion and carries no adjoint of its own).
template <class T> struct BaseAdj {
  V3<T> p;
  T qx, qy, qz, qw;
  SV<T> nu;
};
template <class T> SPI_INL BaseAdj<T> zero_base_adj() {
  BaseAdj<T> a; a.p = z3<T>(); a.qx = a.qy = a.qz = a.qw = T(0); a.nu = zsv<T>(); return a;
}

// B0: the state before the substep, B1: after it. Given lam1 (adjoint after), returns the direct
// part of the adjoint before (lam0) and the base acceleration's adjoint a0b; R0b receives the
// adjoint of B0.R (gravity term), which the caller maps to the quaternion with the residual's.
template <class T>
SPI_INL void base_integrate_bar(const DevModel& M, const BaseState<T>& B0, const BaseState<T>& B1,
                                const BaseAdj<T>& lam1, BaseAdj<T>& lam0, SV<T>& a0b, M3<T>& R0b) {
  const T dt = T(M.dt), g = T(M.g), hx = T(0.5) * dt;
  // p1 = p0 + dt R1 nu1.v
  lam0.p = lam1.p;
  M3<T> R1b = zm3<T>();
  outer_add(R1b, dt * lam1.p, B1.nu.v);
  SV<T> nu1b = lam1.nu;
  nu1b.v = nu1b.v + dt * mulT(B1.R, lam1.p);
  T q1b[4] = {lam1.qx, lam1.qy, lam1.qz, lam1.qw};
  quat_to_R_bar(B1.qx, B1.qy, B1.qz, B1.qw, R1b, q1b[0], q1b[1], q1b[2], q1b[3]);
  // q1 = n / |n|, n = q0 + hx Omega(w1) q0
  const V3<T> w = B1.nu.w;
  const T nx = B0.qx + hx * (B0.qw * w.x + (B0.qy * w.z - B0.qz * w.y));
  const T ny = B0.qy + hx * (B0.qw * w.y + (B0.qz * w.x - B0.qx * w.z));
  const T nz = B0.qz + hx * (B0.qw * w.z + (B0.qx * w.y - B0.qy * w.x));
  const T nw = B0.qw - hx * (B0.qx * w.x + B0.qy * w.y + B0.qz * w.z);
  const T inv = T(1) / m_sqrt(nx * nx + ny * ny + nz * nz + nw * nw);
  const T ux = nx * inv, uy = ny * inv, uz = nz * inv, uw = nw * inv;
  const T pr = ux * q1b[0] + uy * q1b[1] + uz * q1b[2] + uw * q1b[3];
  const T nbx = (q1b[0] - ux * pr) * inv, nby = (q1b[1] - uy * pr) * inv, nbz = (q1b[2] - uz * pr) * inv,
          nbw = (q1b[3] - uw * pr) * inv;
  lam0.qx = nbx + hx * (-nbw * w.x + nbz * w.y - nby * w.z);
  lam0.qy = nby + hx * (-nbw * w.y + nbx * w.z - nbz * w.x);
  lam0.qz = nbz + hx * (-nbw * w.z + nby * w.x - nbx * w.y);
  lam0.qw = nbw + hx * (nbx * w.x + nby * w.y + nbz * w.z);
  nu1b.w.x += hx * (nbx * B0.qw + nby * B0.qz - nbz * B0.qy - nbw * B0.qx);
  nu1b.w.y += hx * (-nbx * B0.qz + nby * B0.qw + nbz * B0.qx - nbw * B0.qy);
  nu1b.w.z += hx * (nbx * B0.qy - nby * B0.qx + nbz * B0.qw - nbw * B0.qz);
  // nu1.w = nu0.w + dt a0.w;  nu1.v = nu0.v + dt (a0.v - g R0 row 2)
  lam0.nu = nu1b;
  a0b.w = dt * nu1b.w;
  a0b.v = dt * nu1b.v;
  R0b.m[2][0] += -dt * g * nu1b.v.x;
  R0b.m[2][1] += -dt * g * nu1b.v.y;
  R0b.m[2][2] += -dt * g * nu1b.v.z;
}
// Leg joints: qd1 = qd0 + dt qdd, q1 = q0 + dt qd1.
template <class T>
SPI_INL void leg_integrate_bar(const DevModel& M, const T qb1[3], const T qdb1[3], T qb0[3], T qdb0[3], T qddb[3]) {
  const T dt = T(M.dt);
  for (int k = 0; k < 3; ++k) {
    const T qdt = qdb1[k] + dt * qb1[k];
    qb0[k] = qb1[k];
    qdb0[k] = qdt;
    qddb[k] = dt * qdt;
  }
}

// ---------------------------------------------------------------------------
// the final-state cost's adjoint (base_to_world backwards)
// ---------------------------------------------------------------------------
// s13 = (p, quaternion, R nu.v, R nu.w): the base adjoint from the world-frame one.
template <class T> SPI_INL BaseAdj<T> base_to_world_bar(const BaseState<T>& B, const T* s13b) {
  BaseAdj<T> a;
  a.p = v3(s13b[0], s13b[1], s13b[2]);
  a.qx = s13b[3]; a.qy = s13b[4]; a.qz = s13b[5]; a.qw = s13b[6];
  const V3<T> vb = v3(s13b[7], s13b[8], s13b[9]), wb = v3(s13b[10], s13b[11], s13b[12]);
  a.nu.v = mulT(B.R, vb);
  a.nu.w = mulT(B.R, wb);
  M3<T> Rb = zm3<T>();
  outer_add(Rb, vb, B.nu.v);
  outer_add(Rb, wb, B.nu.w);
  quat_to_R_bar(B.qx, B.qy, B.qz, B.qw, Rb, a.qx, a.qy, a.qz, a.qw);
  return a;
}

}  // namespace adj
}  // namespace spi
