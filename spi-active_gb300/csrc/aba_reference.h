// aba_reference.h -- the legs' dynamics by Featherstone's articulated-body algorithm (host only).
//
// The FP64 oracle computes the floating-base dynamics with the ABA; the kernel condenses each
// leg through its 3x3 joint-space inertia instead (dynamics.cuh, phase_a / phase_c), which is
// the same mathematics in fewer operations. This header restates the ABA backward / forward
// pass of one leg with the kernel's types so that the host emulation can
//   * check the condensed phases against the ABA phases (equal to FP64 rounding), and
//   * count the ABA's FP operations: the algorithmic count of the oracle's equations, fixed
//     as the roofline's per-substep figure.
#pragma once

#include "dynamics.cuh"

namespace spi {
namespace aba {

template <class T> struct AbaWork {                                 // phase A -> phase C
  SV<T> U[3], cb[3];
  T invD[3], u[3], c[3], s[3];
  // phase A hands its results over through these (a kernel may store them elsewhere, e.g.
  // straight to shared memory, with a type that has the same three members)
  SPI_INL void put_cs(int k, T cc, T ss) { c[k] = cc; s[k] = ss; }
  SPI_INL void put_cb(int k, const SV<T>& v) { cb[k] = v; }
  SPI_INL void put_U(int k, const SV<T>& Uk, T invDk, T uk) { U[k] = Uk; invD[k] = invDk; u[k] = uk; }
};

// R B R^T for general B.
template <int AX, class T> SPI_INL M3<T> rot_gen(T c, T s, const M3<T>& B) {
  // rows of R B, then columns of (R B) R^T
  V3<T> r0 = row(B, 0), r1 = row(B, 1), r2 = row(B, 2);
  V3<T> q0, q1, q2;
  if (AX == 1) { q0 = c * r0 + s * r2; q1 = r1; q2 = (-s) * r0 + c * r2; }
  else { q0 = r0; q1 = c * r1 - s * r2; q2 = s * r1 + c * r2; }
  M3<T> o;
  V3<T> t0 = rot<AX>(c, s, q0), t1 = rot<AX>(c, s, q1), t2 = rot<AX>(c, s, q2);
  o.m[0][0] = t0.x; o.m[0][1] = t0.y; o.m[0][2] = t0.z;
  o.m[1][0] = t1.x; o.m[1][1] = t1.y; o.m[1][2] = t1.z;
  o.m[2][0] = t2.x; o.m[2][1] = t2.y; o.m[2][2] = t2.z;
  return o;
}

// X^T I X for the joint transform X = plucker(R^T, r): rotate by the active joint rotation,
// then shift by the joint origin r (child origin in parent coordinates):
//   A' = A1 + P + P^T - [r]C1[r],  B' = B1 + [r]C1,  C' = C1,  P = [r] B1^T.
template <int AX, int RM = 7, class T> SPI_INL Art<T> art_to_parent(const Art<T>& I, T c, T s, V3<T> r) {
  Art<T> o;
  S3<T> A1 = rot_sym<AX>(c, s, I.A);
  M3<T> B1 = rot_gen<AX>(c, s, I.B);
  S3<T> C1 = rot_sym<AX>(c, s, I.C);
  if (RM == 4) {   // r = (0, 0, z)
    const T z = r.z, zz = r.z * r.z;
    o.A.xx = A1.xx - T(2) * z * B1.m[0][1] + zz * C1.yy;
    o.A.yy = A1.yy + T(2) * z * B1.m[1][0] + zz * C1.xx;
    o.A.zz = A1.zz;
    o.A.xy = A1.xy + z * (B1.m[0][0] - B1.m[1][1]) - zz * C1.xy;
    o.A.xz = A1.xz - z * B1.m[2][1];
    o.A.yz = A1.yz + z * B1.m[2][0];
    o.B.m[0][0] = B1.m[0][0] - z * C1.xy; o.B.m[0][1] = B1.m[0][1] - z * C1.yy; o.B.m[0][2] = B1.m[0][2] - z * C1.yz;
    o.B.m[1][0] = B1.m[1][0] + z * C1.xx; o.B.m[1][1] = B1.m[1][1] + z * C1.xy; o.B.m[1][2] = B1.m[1][2] + z * C1.xz;
    o.B.m[2][0] = B1.m[2][0]; o.B.m[2][1] = B1.m[2][1]; o.B.m[2][2] = B1.m[2][2];
    o.C = C1;
    return o;
  }
  if (RM == 2) {   // r = (0, y, 0)
    const T y = r.y, yy = r.y * r.y;
    o.A.xx = A1.xx + T(2) * y * B1.m[0][2] + yy * C1.zz;
    o.A.yy = A1.yy;
    o.A.zz = A1.zz - T(2) * y * B1.m[2][0] + yy * C1.xx;
    o.A.xy = A1.xy + y * B1.m[1][2];
    o.A.xz = A1.xz + y * (B1.m[2][2] - B1.m[0][0]) - yy * C1.xz;
    o.A.yz = A1.yz - y * B1.m[1][0];
    o.B.m[0][0] = B1.m[0][0] + y * C1.xz; o.B.m[0][1] = B1.m[0][1] + y * C1.yz; o.B.m[0][2] = B1.m[0][2] + y * C1.zz;
    o.B.m[1][0] = B1.m[1][0]; o.B.m[1][1] = B1.m[1][1]; o.B.m[1][2] = B1.m[1][2];
    o.B.m[2][0] = B1.m[2][0] - y * C1.xx; o.B.m[2][1] = B1.m[2][1] - y * C1.xy; o.B.m[2][2] = B1.m[2][2] - y * C1.xz;
    o.C = C1;
    return o;
  }
  // P = skew(r) B1^T: column j = r x (row j of B1)
  V3<T> p0 = cross(r, row(B1, 0)), p1 = cross(r, row(B1, 1)), p2 = cross(r, row(B1, 2));
  // Q = skew(r) C1: column j = r x (column j of C1);  skew(r) C1 skew(r): column j = r x (C1 (r x e_j))
  V3<T> cq0 = cross(r, col(C1, 0)), cq1 = cross(r, col(C1, 1)), cq2 = cross(r, col(C1, 2));
  V3<T> e0 = v3(T(0), r.z, -r.y), e1 = v3(-r.z, T(0), r.x), e2 = v3(r.y, -r.x, T(0));  // r x e_j
  V3<T> k0 = cross(r, mul(C1, e0)), k1 = cross(r, mul(C1, e1)), k2 = cross(r, mul(C1, e2));
  // A' = A1 + P + P^T - skew(r) C1 skew(r)
  o.A.xx = A1.xx + T(2) * p0.x - k0.x;
  o.A.yy = A1.yy + T(2) * p1.y - k1.y;
  o.A.zz = A1.zz + T(2) * p2.z - k2.z;
  o.A.xy = A1.xy + p1.x + p0.y - k1.x;
  o.A.xz = A1.xz + p2.x + p0.z - k2.x;
  o.A.yz = A1.yz + p2.y + p1.z - k2.y;
  // B' = B1 + skew(r) C1
  o.B.m[0][0] = B1.m[0][0] + cq0.x; o.B.m[0][1] = B1.m[0][1] + cq1.x; o.B.m[0][2] = B1.m[0][2] + cq2.x;
  o.B.m[1][0] = B1.m[1][0] + cq0.y; o.B.m[1][1] = B1.m[1][1] + cq1.y; o.B.m[1][2] = B1.m[1][2] + cq2.y;
  o.B.m[2][0] = B1.m[2][0] + cq0.z; o.B.m[2][1] = B1.m[2][1] + cq1.z; o.B.m[2][2] = B1.m[2][2] + cq2.z;
  o.C = C1;
  return o;
}
template <class T> SPI_INL Art<T> leg_rigid(const DevModel& M, int k, int leg) {
  S3<T> Io;
  Io.xx = T(M.I[k][0][leg]); Io.yy = T(M.I[k][1][leg]); Io.zz = T(M.I[k][2][leg]);
  Io.xy = T(M.I[k][3][leg]); Io.xz = T(M.I[k][4][leg]); Io.yz = T(M.I[k][5][leg]);
  return rigid(T(M.m[k][leg]), v3(T(M.h[k][0][leg]), T(M.h[k][1][leg]), T(M.h[k][2][leg])), Io);
}
template <class T> SPI_INL SV<T> leg_bias(const DevModel& M, int k, int leg, const SV<T>& v) {
  S3<T> Io;
  Io.xx = T(M.I[k][0][leg]); Io.yy = T(M.I[k][1][leg]); Io.zz = T(M.I[k][2][leg]);
  Io.xy = T(M.I[k][3][leg]); Io.xz = T(M.I[k][4][leg]); Io.yz = T(M.I[k][5][leg]);
  V3<T> h = v3(T(M.h[k][0][leg]), T(M.h[k][1][leg]), T(M.h[k][2][leg]));
  return crf(v, rigid_mul(T(M.m[k][leg]), h, Io, v));
}

// One ABA backward step of joint k (axis AX): project out the joint, move to the parent.
template <int AX, int RM, class T, class WK>
SPI_INL void aba_back(Art<T>& IA, SV<T>& pA, const SV<T>& cb, T tau, T arm, T c, T s, V3<T> r, WK& W, int k,
                      Art<T>* Iout, SV<T>* pout) {
  SV<T> U;
  U.w = col(IA.A, AX);
  U.v = row(IA.B, AX);
  T D = (AX == 0 ? IA.A.xx : IA.A.yy) + arm;
  T invD = T(1) / D;
  T u = tau - (AX == 0 ? pA.w.x : pA.w.y);
  // Ia = IA - U U^T / D
  Art<T> Ia = IA;
  V3<T> Uw = invD * U.w, Uv = invD * U.v;
  Ia.A.xx -= Uw.x * U.w.x; Ia.A.yy -= Uw.y * U.w.y; Ia.A.zz -= Uw.z * U.w.z;
  Ia.A.xy -= Uw.x * U.w.y; Ia.A.xz -= Uw.x * U.w.z; Ia.A.yz -= Uw.y * U.w.z;
  Ia.B.m[0][0] -= Uw.x * U.v.x; Ia.B.m[0][1] -= Uw.x * U.v.y; Ia.B.m[0][2] -= Uw.x * U.v.z;
  Ia.B.m[1][0] -= Uw.y * U.v.x; Ia.B.m[1][1] -= Uw.y * U.v.y; Ia.B.m[1][2] -= Uw.y * U.v.z;
  Ia.B.m[2][0] -= Uw.z * U.v.x; Ia.B.m[2][1] -= Uw.z * U.v.y; Ia.B.m[2][2] -= Uw.z * U.v.z;
  Ia.C.xx -= Uv.x * U.v.x; Ia.C.yy -= Uv.y * U.v.y; Ia.C.zz -= Uv.z * U.v.z;
  Ia.C.xy -= Uv.x * U.v.y; Ia.C.xz -= Uv.x * U.v.z; Ia.C.yz -= Uv.y * U.v.z;
  // pa = pA + Ia c + U u / D
  SV<T> pa = mul(Ia, cb);
  T uD = u * invD;
  pa.w = pA.w + pa.w + uD * U.w;
  pa.v = pA.v + pa.v + uD * U.v;
  W.put_U(k, U, invD, u);
  *Iout = art_to_parent<AX, RM>(Ia, c, s, r);
  *pout = force_to_parent<AX, RM>(pa, c, s, r);
}

template <class T, class WK>
SPI_INL LegOut<T> phase_a_aba(const DevModel& M, int leg, const BaseState<T>& B, const LegState<T>& L,
                          const LegParams<T>& P, const T act[3], WK& W) {
  T tau[3], C[3], S[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    tau[k] = motor_torque(M, P, k, leg, act[k], L.q[k], L.qd[k]);
    m_sincos(L.q[k], &S[k], &C[k]);
    W.put_cs(k, C[k], S[k]);
  }
  V3<T> r0 = leg_org<T>(M, 0, leg), r1 = leg_org<T>(M, 1, leg), r2 = leg_org<T>(M, 2, leg);
  // body velocities (body coordinates) and velocity-product accelerations
  SV<T> v0 = motion_to_child<0>(B.nu, C[0], S[0], r0); v0.w.x = v0.w.x + L.qd[0];
  SV<T> v1 = motion_to_child<1, 2>(v0, C[1], S[1], r1);   v1.w.y = v1.w.y + L.qd[1];
  SV<T> v2 = motion_to_child<1, 4>(v1, C[2], S[2], r2);   v2.w.y = v2.w.y + L.qd[2];
  const SV<T> cb0 = vel_product<0>(v0, L.qd[0]), cb1 = vel_product<1>(v1, L.qd[1]),
              cb2 = vel_product<1>(v2, L.qd[2]);
  W.put_cb(0, cb0); W.put_cb(1, cb1); W.put_cb(2, cb2);
  // foot: position and velocity, calf -> thigh -> hip -> base -> world
  V3<T> fc = v3(T(M.foot[0]), T(M.foot[1]), T(M.foot[2]));
  V3<T> vf = v2.v + cross(v2.w, fc);
  V3<T> pf = rot<1>(C[2], S[2], fc) + r2;
  vf = rot<1>(C[2], S[2], vf);
  pf = rot<1>(C[1], S[1], pf) + r1;
  vf = rot<1>(C[1], S[1], vf);
  pf = rot<0>(C[0], S[0], pf) + r0;
  vf = rot<0>(C[0], S[0], vf);
  T mimp;
  V3<T> F = contact_force(M, T(M.foot_r), B.p.z + dot(row(B.R, 2), pf), mul(B.R, vf), &mimp);
  // the implicit point mass acts on the true acceleration while the ABA runs in the
  // gravity-shifted frame: its share of the shift enters as a force mimp*g upwards
  F.z = F.z + mimp * T(M.g);
  V3<T> Fc = mulT(B.R, F);
  Fc = rotT<0>(C[0], S[0], Fc);
  Fc = rotT<1>(C[1], S[1], Fc);
  Fc = rotT<1>(C[2], S[2], Fc);
  // ABA backward pass: calf -> thigh -> hip -> base
  Art<T> IA = leg_rigid<T>(M, 2, leg);
  add_point_mass(IA, mimp, fc);
  SV<T> pA = leg_bias(M, 2, leg, v2);
  pA.w = pA.w - cross(fc, Fc);
  pA.v = pA.v - Fc;
  Art<T> Ip; SV<T> pp;
  aba_back<1, 4>(IA, pA, cb2, tau[2], P.arm, C[2], S[2], r2, W, 2, &Ip, &pp);
  IA = leg_rigid<T>(M, 1, leg); add_to(IA, Ip);
  pA = leg_bias(M, 1, leg, v1); pA.w = pA.w + pp.w; pA.v = pA.v + pp.v;
  aba_back<1, 2>(IA, pA, cb1, tau[1], P.arm, C[1], S[1], r1, W, 1, &Ip, &pp);
  IA = leg_rigid<T>(M, 0, leg); add_to(IA, Ip);
  pA = leg_bias(M, 0, leg, v0); pA.w = pA.w + pp.w; pA.v = pA.v + pp.v;
  LegOut<T> out;
  aba_back<0, 7>(IA, pA, cb0, tau[0], P.arm, C[0], S[0], r0, W, 0, &out.I, &out.p);
  // two of the eight base-box corners; a corner can only reach the ground when the base origin
  // is lower than the box's half-diagonal, so a warp whose rollouts are all higher skips them
  // (a corner off the ground adds exactly zero force and zero implicit mass)
  if (M.base_contact && warp_any(B.p.z < T(M.corner_reach))) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const float* cc = M.corner[2 * leg + j];
      V3<T> rc = v3(T(cc[0]), T(cc[1]), T(cc[2]));
      V3<T> vc = B.nu.v + cross(B.nu.w, rc);
      T mc;
      V3<T> Fw = contact_force(M, T(0), B.p.z + dot(row(B.R, 2), rc), mul(B.R, vc), &mc);
      Fw.z = Fw.z + mc * T(M.g);
      V3<T> Fb = mulT(B.R, Fw);
      out.p.w = out.p.w - cross(rc, Fb);
      out.p.v = out.p.v - Fb;
      add_point_mass(out.I, mc, rc);
    }
  }
  return out;
}

template <class T>
SPI_INL void phase_c_aba(const DevModel& M, int leg, const SV<T>& a0, const AbaWork<T>& W, LegState<T>& L) {
  T qdd[3];
  SV<T> a = motion_to_child<0>(a0, W.c[0], W.s[0], leg_org<T>(M, 0, leg));
  a.w = a.w + W.cb[0].w; a.v = a.v + W.cb[0].v;
  qdd[0] = (W.u[0] - dot(W.U[0].w, a.w) - dot(W.U[0].v, a.v)) * W.invD[0];
  a.w.x = a.w.x + qdd[0];
  a = motion_to_child<1, 2>(a, W.c[1], W.s[1], leg_org<T>(M, 1, leg));
  a.w = a.w + W.cb[1].w; a.v = a.v + W.cb[1].v;
  qdd[1] = (W.u[1] - dot(W.U[1].w, a.w) - dot(W.U[1].v, a.v)) * W.invD[1];
  a.w.y = a.w.y + qdd[1];
  a = motion_to_child<1, 4>(a, W.c[2], W.s[2], leg_org<T>(M, 2, leg));
  a.w = a.w + W.cb[2].w; a.v = a.v + W.cb[2].v;
  qdd[2] = (W.u[2] - dot(W.U[2].w, a.w) - dot(W.U[2].v, a.v)) * W.invD[2];
  T dt = T(M.dt);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    L.qd[k] = L.qd[k] + dt * qdd[k];
    L.q[k] = L.q[k] + dt * L.qd[k];
  }
}

}  // namespace aba
}  // namespace spi
