// dynamics.cuh -- one physics substep of the Go2 floating-base model, split per leg.
//
// Templated on the scalar type T so the same source builds (a) the sm_103a rollout
// kernel (T = float, one lane per leg, four lanes per rollout) and (b) a host
// emulation (T = double, or a flop-counting scalar) that runs the phases in sequence.
//
// Phases of a substep (leg l = 0..3, FL FR RL RR):
//   A  per leg : motor torques, leg kinematics, foot + 2 base-corner contacts, and the leg
//               condensed onto the base through its 3x3 joint-space inertia (composite
//               inertias, joint force columns, L D L^T, bias pass) -> the leg's articulated
//               inertia and bias force expressed at the base (LegOut, 27 values), the same
//               quantities as the backward pass of Featherstone's ABA
//   (sum of the four LegOut: warp shuffles on the device, a loop on the host)
//   B  base    : base articulated inertia + bias, 6x6 Cholesky solve for the base
//               acceleration, semi-implicit Euler step of the floating base
//   C  per leg : joint accelerations from the base acceleration (3x3 triangular solve) and
//               joint integration
//
// Equations (Featherstone spatial algebra, motion = (w; v), force = (n; f)):
//   PD law  tau = kp_s*Kp*(action_scale*clip(a) + q0 - q) - kd_s*Kd*qd, clipped to
//           +-ts*tau_lim*(1 - |qd|/qd_max)+ -- spigym/envs/legged_base_task/
//           legged_robot_base.py:185-187, 542-560 (hip action x hip_scale: go2_omni.py:437)
//   motor   per-type gain and a*tanh(tau/a) -- spigym/envs/sysid/active_sysid_openloop.py:365-400
//   joint   friction -Fc*tanh(qd/w_f); armature added to the joint-space inertia diagonal
//   contact fn = max(0, k*pen - c*s*vz) if pen > 0, s = min(1, pen/ramp) (damping fades in over
//           the first `ramp` of penetration, so the force is continuous at touchdown);
//           ft = -min(ct, mu*fn/|vt|)*vt. Contact damping is linearly implicit: an active
//           contact adds a point mass dt*max(c, ct)*s at the contact point to its body's
//           inertia (exact for linear damping, stable at any dt)
//   base    nu += dt*a;  q <- normalise(q + dt/2 q(x)w_b);  p += dt*R(q)*v_b
#pragma once

#include "spi_engine.h"

#if defined(__CUDACC__)
#define SPI_HD __host__ __device__
#define SPI_INL __host__ __device__ __forceinline__
#else
#define SPI_HD
#define SPI_INL inline
#include <cmath>
#endif

namespace spi {

// ---------------------------------------------------------------------------
// scalar helpers (overloaded for float / double; the flop counter adds its own)
// ---------------------------------------------------------------------------
SPI_INL float m_sqrt(float x) { return sqrtf(x); }
SPI_INL double m_sqrt(double x) { return sqrt(x); }
// Device FP32: tanh(x) = 1 - 2/(2^{x k} + 1) with k = 2 log2(e), from one MUFU base-2
// exponential and one MUFU reciprocal (absolute error ~1e-7). Large |x| needs no clamp: the
// exponential saturates to +inf or 0 and the expression to +1 or -1; NaN propagates.
constexpr float kTwoLog2e = 2.88539008177792681f;
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float tanh_from_k(float xk) { return 1.0f - __fdividef(2.0f, ex2_approx(xk) + 1.0f); }
#endif
SPI_INL float m_tanh(float x) {
#if defined(__CUDA_ARCH__)
  return tanh_from_k(x * kTwoLog2e);
#else
  return tanhf(x);
#endif
}
SPI_INL double m_tanh(double x) { return tanh(x); }
// tanh(x / d) given k2 = 2 log2(e) / d and x / d given dinv = 1 / d (model constants): the FP32
// forms multiply by the precomputed constant, every other scalar type divides.
SPI_INL float m_tanh_div(float x, float d, float k2) {
#if defined(__CUDA_ARCH__)
  (void)d;
  return tanh_from_k(x * k2);
#else
  (void)k2;
  return tanhf(x / d);
#endif
}
template <class T> SPI_INL T m_tanh_div(T x, float d, float k2) { (void)k2; return m_tanh(x / T(d)); }
SPI_INL float m_div_c(float x, float d, float dinv) { (void)d; return x * dinv; }
template <class T> SPI_INL T m_div_c(T x, float d, float dinv) { (void)dinv; return x / T(d); }
// a b x given ab = fl(a b) (a model constant): FP32 multiplies once, to the same result as
// (a b) x; every other scalar type forms a b in its own precision.
SPI_INL float m_mul2_c(float x, float a, float b, float ab) { (void)a; (void)b; return ab * x; }
template <class T> SPI_INL T m_mul2_c(T x, float a, float b, float ab) { (void)ab; return T(a) * T(b) * x; }
// Device FP32: the MUFU sine / cosine. Joint angles stay within a few radians (the PD targets
// lie within action_clip * action_scale of the default pose), where their absolute error is
// ~2^-21 for |x| <= pi and ~2^-20.5 out to many periods, so no range reduction is applied.
SPI_INL void m_sincos(float x, float* s, float* c) {
#if defined(__CUDA_ARCH__)
  __sincosf(x, s, c);
#else
  *s = sinf(x); *c = cosf(x);
#endif
}
SPI_INL void m_sincos(double x, double* s, double* c) { *s = sin(x); *c = cos(x); }
SPI_INL float m_fabs(float x) { return fabsf(x); }
SPI_INL double m_fabs(double x) { return fabs(x); }
SPI_INL float m_fmax(float a, float b) { return fmaxf(a, b); }
SPI_INL double m_fmax(double a, double b) { return fmax(a, b); }
SPI_INL float m_fmin(float a, float b) { return fminf(a, b); }
SPI_INL double m_fmin(double a, double b) { return fmin(a, b); }
template <class T> SPI_INL T m_sel(bool c, T a, T b) { return c ? a : b; }
// True if the predicate holds on any lane of the warp (the host emulation runs one lane).
SPI_INL bool warp_any(bool p) {
#if defined(__CUDA_ARCH__)
  return __any_sync(0xffffffffu, p);
#else
  return p;
#endif
}
template <class T> SPI_INL T m_clamp(T x, T lo, T hi) { return m_fmin(m_fmax(x, lo), hi); }

// ---------------------------------------------------------------------------
// small vector / matrix types
// ---------------------------------------------------------------------------
template <class T> struct V3 { T x, y, z; };
template <class T> struct S3 { T xx, yy, zz, xy, xz, yz; };   // symmetric 3x3
template <class T> struct M3 { T m[3][3]; };                  // general 3x3, row-major
template <class T> struct SV { V3<T> w, v; };                 // spatial vector
template <class T> struct Art { S3<T> A; M3<T> B; S3<T> C; };  // [[A, B], [B^T, C]]

template <class T> SPI_INL V3<T> v3(T x, T y, T z) { V3<T> r; r.x = x; r.y = y; r.z = z; return r; }
template <class T> SPI_INL V3<T> operator+(V3<T> a, V3<T> b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> SPI_INL V3<T> operator-(V3<T> a, V3<T> b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> SPI_INL V3<T> operator*(T s, V3<T> a) { return v3(s * a.x, s * a.y, s * a.z); }
template <class T> SPI_INL T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> SPI_INL V3<T> cross(V3<T> a, V3<T> b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T> SPI_INL V3<T> mul(const S3<T>& S, V3<T> u) {
  return v3(S.xx * u.x + S.xy * u.y + S.xz * u.z,
            S.xy * u.x + S.yy * u.y + S.yz * u.z,
            S.xz * u.x + S.yz * u.y + S.zz * u.z);
}
template <class T> SPI_INL V3<T> mul(const M3<T>& M, V3<T> u) {
  return v3(M.m[0][0] * u.x + M.m[0][1] * u.y + M.m[0][2] * u.z,
            M.m[1][0] * u.x + M.m[1][1] * u.y + M.m[1][2] * u.z,
            M.m[2][0] * u.x + M.m[2][1] * u.y + M.m[2][2] * u.z);
}
template <class T> SPI_INL V3<T> mulT(const M3<T>& M, V3<T> u) {
  return v3(M.m[0][0] * u.x + M.m[1][0] * u.y + M.m[2][0] * u.z,
            M.m[0][1] * u.x + M.m[1][1] * u.y + M.m[2][1] * u.z,
            M.m[0][2] * u.x + M.m[1][2] * u.y + M.m[2][2] * u.z);
}
template <class T> SPI_INL V3<T> row(const M3<T>& M, int i) { return v3(M.m[i][0], M.m[i][1], M.m[i][2]); }
template <class T> SPI_INL V3<T> col(const S3<T>& S, int j) {
  return j == 0 ? v3(S.xx, S.xy, S.xz) : (j == 1 ? v3(S.xy, S.yy, S.yz) : v3(S.xz, S.yz, S.zz));
}

// Active rotation by angle (c, s) about the x (AX = 0) or y (AX = 1) axis, and its transpose.
template <int AX, class T> SPI_INL V3<T> rot(T c, T s, V3<T> u) {
  if (AX == 0) return v3(u.x, c * u.y - s * u.z, s * u.y + c * u.z);
  return v3(c * u.x + s * u.z, u.y, -s * u.x + c * u.z);
}
template <int AX, class T> SPI_INL V3<T> rotT(T c, T s, V3<T> u) {
  if (AX == 0) return v3(u.x, c * u.y + s * u.z, -s * u.y + c * u.z);
  return v3(c * u.x - s * u.z, u.y, s * u.x + c * u.z);
}
// R M R^T for symmetric M and the active plane rotation R about AX.
template <int AX, class T> SPI_INL S3<T> rot_sym(T c, T s, const S3<T>& M) {
  S3<T> r;
  if (AX == 1) {  // plane (x, z): x' = c x + s z, z' = -s x + c z
    T cc = c * c, ss = s * s, cs = c * s;
    r.xx = cc * M.xx + T(2) * cs * M.xz + ss * M.zz;
    r.zz = ss * M.xx - T(2) * cs * M.xz + cc * M.zz;
    r.xz = cs * (M.zz - M.xx) + (cc - ss) * M.xz;
    r.xy = c * M.xy + s * M.yz;
    r.yz = -s * M.xy + c * M.yz;
    r.yy = M.yy;
  } else {        // plane (y, z): y' = c y - s z, z' = s y + c z
    T cc = c * c, ss = s * s, cs = c * s;
    r.yy = cc * M.yy - T(2) * cs * M.yz + ss * M.zz;
    r.zz = ss * M.yy + T(2) * cs * M.yz + cc * M.zz;
    r.yz = cs * (M.yy - M.zz) + (cc - ss) * M.yz;
    r.xy = c * M.xy - s * M.xz;
    r.xz = s * M.xy + c * M.xz;
    r.xx = M.xx;
  }
  return r;
}
// I * v for an articulated inertia.
template <class T> SPI_INL SV<T> mul(const Art<T>& I, const SV<T>& m) {
  SV<T> r;
  r.w = mul(I.A, m.w) + mul(I.B, m.v);
  r.v = mulT(I.B, m.w) + mul(I.C, m.v);
  return r;
}
// v x* f (force cross product).
template <class T> SPI_INL SV<T> crf(const SV<T>& v, const SV<T>& f) {
  SV<T> r;
  const V3<T> a = cross(v.w, f.w);
  r.w = v3(a.x + v.v.y * f.v.z - v.v.z * f.v.y, a.y + v.v.z * f.v.x - v.v.x * f.v.z,
           a.z + v.v.x * f.v.y - v.v.y * f.v.x);
  r.v = cross(v.w, f.v);
  return r;
}
// Rigid-body spatial inertia from mass, first moment h = m c and rotational inertia about the origin.
template <class T> SPI_INL Art<T> rigid(T m, V3<T> h, const S3<T>& Io) {
  Art<T> I;
  I.A = Io;
  I.B.m[0][0] = T(0); I.B.m[0][1] = -h.z; I.B.m[0][2] = h.y;
  I.B.m[1][0] = h.z;  I.B.m[1][1] = T(0); I.B.m[1][2] = -h.x;
  I.B.m[2][0] = -h.y; I.B.m[2][1] = h.x;  I.B.m[2][2] = T(0);
  I.C.xx = m; I.C.yy = m; I.C.zz = m; I.C.xy = T(0); I.C.xz = T(0); I.C.yz = T(0);
  return I;
}
// Rigid-body I*v without forming the 6x6.
template <class T> SPI_INL SV<T> rigid_mul(T m, V3<T> h, const S3<T>& Io, const SV<T>& v) {
  SV<T> r;   // (Io w + h x v; m v - h x w), each sum one chain of fused multiply-adds
  const V3<T> iw = mul(Io, v.w);
  r.w = v3(iw.x + h.y * v.v.z - h.z * v.v.y, iw.y + h.z * v.v.x - h.x * v.v.z, iw.z + h.x * v.v.y - h.y * v.v.x);
  r.v = v3(m * v.v.x + v.w.y * h.z - v.w.z * h.y, m * v.v.y + v.w.z * h.x - v.w.x * h.z,
           m * v.v.z + v.w.x * h.y - v.w.y * h.x);
  return r;
}
// Accumulating forms: acc + (product sums), written with the accumulator innermost so that
// every product fuses into a multiply-add (no separate multiply and final add).
template <class T> SPI_INL V3<T> mul_acc(const S3<T>& S, V3<T> u, V3<T> acc) {
  return v3(acc.x + S.xx * u.x + S.xy * u.y + S.xz * u.z,
            acc.y + S.xy * u.x + S.yy * u.y + S.yz * u.z,
            acc.z + S.xz * u.x + S.yz * u.y + S.zz * u.z);
}
template <class T> SPI_INL V3<T> cross_acc(V3<T> a, V3<T> b, V3<T> acc) {   // acc + a x b
  return v3(acc.x + a.y * b.z - a.z * b.y, acc.y + a.z * b.x - a.x * b.z, acc.z + a.x * b.y - a.y * b.x);
}
template <class T> SPI_INL SV<T> crf_acc(const SV<T>& v, const SV<T>& f, const SV<T>& acc) {   // acc + v x* f
  SV<T> r;
  r.w = cross_acc(v.v, f.v, cross_acc(v.w, f.w, acc.w));
  r.v = cross_acc(v.w, f.v, acc.v);
  return r;
}
template <class T> SPI_INL SV<T> rigid_mul_acc(T m, V3<T> h, const S3<T>& Io, const SV<T>& v, const SV<T>& acc) {
  SV<T> r;   // acc + I v
  r.w = cross_acc(h, v.v, mul_acc(Io, v.w, acc.w));
  r.v = cross_acc(v.w, h, v3(acc.v.x + m * v.v.x, acc.v.y + m * v.v.y, acc.v.z + m * v.v.z));
  return r;
}
template <class T> SPI_INL void add_to(Art<T>& a, const Art<T>& b) {
  a.A.xx += b.A.xx; a.A.yy += b.A.yy; a.A.zz += b.A.zz; a.A.xy += b.A.xy; a.A.xz += b.A.xz; a.A.yz += b.A.yz;
  a.C.xx += b.C.xx; a.C.yy += b.C.yy; a.C.zz += b.C.zz; a.C.xy += b.C.xy; a.C.xz += b.C.xz; a.C.yz += b.C.yz;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) a.B.m[i][j] += b.B.m[i][j];
}
// Rigid-body inertia as mass, first moment h = m c and rotational inertia about the body
// origin (10 numbers; sums of rigid bodies stay rigid, so composite inertias use it too).
template <class T> struct RI { T m; V3<T> h; S3<T> I; };
template <class T> SPI_INL SV<T> ri_mul(const RI<T>& a, const SV<T>& v) { return rigid_mul(a.m, a.h, a.I, v); }
template <class T> SPI_INL SV<T> ri_mul_acc(const RI<T>& a, const SV<T>& v, const SV<T>& acc) {
  return rigid_mul_acc(a.m, a.h, a.I, v, acc);
}
// I S for the revolute joint axis AX of the body's own frame: (I e_AX; e_AX x h).
template <int AX, class T> SPI_INL SV<T> ri_col(const RI<T>& a) {
  SV<T> f;
  f.w = col(a.I, AX);
  f.v = AX == 0 ? v3(T(0), -a.h.z, a.h.y) : v3(a.h.z, T(0), -a.h.x);
  return f;
}
// Articulated-inertia form [[I, [h]x], [[h]x^T, m 1]].
template <class T> SPI_INL Art<T> ri_art(const RI<T>& a) { return rigid(a.m, a.h, a.I); }

// Joint-origin sparsity. RM = 2: origin on the y axis (thigh joints), RM = 4: on the z axis
// (calf joints), RM = 3: in the x-y plane (hip joints), RM = 7: general. The model builder
// checks the pattern.
constexpr int kHipRM = 3;
// u - r x w, with the known-zero terms of r x w not subtracted.
template <int RM, class T> SPI_INL V3<T> sub_rcross(V3<T> u, V3<T> r, V3<T> w) {
  if (RM == 2) return v3(u.x - r.y * w.z, u.y, u.z + r.y * w.x);
  if (RM == 4) return v3(u.x + r.z * w.y, u.y - r.z * w.x, u.z);
  if (RM == 3) return v3(u.x - r.y * w.z, u.y + r.x * w.z, u.z - r.x * w.y + r.y * w.x);
  return v3(u.x - r.y * w.z + r.z * w.y, u.y - r.z * w.x + r.x * w.z, u.z - r.x * w.y + r.y * w.x);
}
template <int RM, class T> SPI_INL V3<T> add_rcross(V3<T> u, V3<T> r, V3<T> w) {
  if (RM == 2) return v3(u.x + r.y * w.z, u.y, u.z - r.y * w.x);
  if (RM == 4) return v3(u.x - r.z * w.y, u.y + r.z * w.x, u.z);
  if (RM == 3) return v3(u.x + r.y * w.z, u.y - r.x * w.z, u.z + r.x * w.y - r.y * w.x);
  return v3(u.x + r.y * w.z - r.z * w.y, u.y + r.z * w.x - r.x * w.z, u.z + r.x * w.y - r.y * w.x);
}
// acc + R u for the active rotation about AX.
template <int AX, class T> SPI_INL V3<T> rot_acc(T c, T s, V3<T> u, V3<T> acc) {
  if (AX == 0) return v3(acc.x + u.x, acc.y + c * u.y - s * u.z, acc.z + s * u.y + c * u.z);
  return v3(acc.x + c * u.x + s * u.z, acc.y + u.y, acc.z - s * u.x + c * u.z);
}
template <int AX, class T> SPI_INL V3<T> rotT_acc(T c, T s, V3<T> u, V3<T> acc) {
  if (AX == 0) return v3(acc.x + u.x, acc.y + c * u.y + s * u.z, acc.z - s * u.y + c * u.z);
  return v3(acc.x + c * u.x - s * u.z, acc.y + u.y, acc.z + s * u.x + c * u.z);
}
// X^T f: child force to parent coordinates.
template <int AX, int RM = 7, class T> SPI_INL SV<T> force_to_parent(const SV<T>& f, T c, T s, V3<T> r) {
  SV<T> o;
  o.v = rot<AX>(c, s, f.v);
  o.w = add_rcross<RM>(rot<AX>(c, s, f.w), r, o.v);
  return o;
}
// acc + X^T f.
template <int AX, int RM = 7, class T>
SPI_INL SV<T> force_to_parent_acc(const SV<T>& f, T c, T s, V3<T> r, const SV<T>& acc) {
  SV<T> o;
  const V3<T> fv = rot<AX>(c, s, f.v);
  o.v = acc.v + fv;
  o.w = add_rcross<RM>(rot_acc<AX>(c, s, f.w, acc.w), r, fv);
  return o;
}
// X m: parent motion to child coordinates.
template <int AX, int RM = 7, class T> SPI_INL SV<T> motion_to_child(const SV<T>& m, T c, T s, V3<T> r) {
  SV<T> o;
  o.w = rotT<AX>(c, s, m.w);
  o.v = rotT<AX>(c, s, sub_rcross<RM>(m.v, r, m.w));
  return o;
}

// base + R M R^T for symmetric M and the active plane rotation R about AX (rot_sym with the
// parent's own inertia as accumulator).
template <int AX, class T> SPI_INL S3<T> rot_sym_acc(T c, T s, const S3<T>& M, const S3<T>& base) {
  S3<T> r;
  const T cc = c * c, ss = s * s, cs = c * s, cs2 = T(2) * cs;
  if (AX == 1) {
    r.xx = base.xx + cc * M.xx + cs2 * M.xz + ss * M.zz;
    r.zz = base.zz + ss * M.xx - cs2 * M.xz + cc * M.zz;
    r.xz = base.xz + cs * (M.zz - M.xx) + (cc - ss) * M.xz;
    r.xy = base.xy + c * M.xy + s * M.yz;
    r.yz = base.yz - s * M.xy + c * M.yz;
    r.yy = base.yy + M.yy;
  } else {
    r.yy = base.yy + cc * M.yy - cs2 * M.yz + ss * M.zz;
    r.zz = base.zz + ss * M.yy + cs2 * M.yz + cc * M.zz;
    r.yz = base.yz + cs * (M.yy - M.zz) + (cc - ss) * M.yz;
    r.xy = base.xy + c * M.xy - s * M.xz;
    r.xz = base.xz + s * M.xy + c * M.xz;
    r.xx = base.xx + M.xx;
  }
  return r;
}
// base + X^T I X: ri_to_parent with the parent body's own inertia as accumulator.
template <int AX, int RM, class T> SPI_INL RI<T> ri_to_parent_acc(const RI<T>& c, T cs, T sn, V3<T> r, const RI<T>& base) {
  RI<T> o;
  o.m = base.m + c.m;
  const S3<T> I1 = rot_sym_acc<AX>(cs, sn, c.I, base.I);
  const V3<T> a = rot<AX>(cs, sn, c.h);
  if (RM == 4) {   // r = (0, 0, z)
    const T z = r.z, mz = c.m * z;
    const T t = T(2) * a.z + mz;
    o.h = v3(base.h.x + a.x, base.h.y + a.y, base.h.z + a.z + mz);
    o.I.xx = I1.xx + z * t; o.I.yy = I1.yy + z * t; o.I.zz = I1.zz;
    o.I.xy = I1.xy; o.I.xz = I1.xz - a.x * z; o.I.yz = I1.yz - a.y * z;
    return o;
  }
  if (RM == 2) {   // r = (0, y, 0)
    const T y = r.y, my = c.m * y;
    const T t = T(2) * a.y + my;
    o.h = v3(base.h.x + a.x, base.h.y + a.y + my, base.h.z + a.z);
    o.I.xx = I1.xx + y * t; o.I.yy = I1.yy; o.I.zz = I1.zz + y * t;
    o.I.xy = I1.xy - a.x * y; o.I.xz = I1.xz; o.I.yz = I1.yz - a.z * y;
    return o;
  }
  const V3<T> mr = c.m * r;
  o.h = base.h + a + mr;
  const T ax = a.x * r.x, ay = a.y * r.y, az = a.z * r.z;
  o.I.xx = I1.xx + T(2) * (ay + az) + mr.y * r.y + mr.z * r.z;
  o.I.yy = I1.yy + T(2) * (ax + az) + mr.x * r.x + mr.z * r.z;
  o.I.zz = I1.zz + T(2) * (ax + ay) + mr.x * r.x + mr.y * r.y;
  o.I.xy = I1.xy - (a.x * r.y + a.y * r.x) - mr.x * r.y;
  o.I.xz = I1.xz - (a.x * r.z + a.z * r.x) - mr.x * r.z;
  o.I.yz = I1.yz - (a.y * r.z + a.z * r.y) - mr.y * r.z;
  return o;
}

// X^T I X for a rigid inertia: the child's inertia in parent coordinates, child frame rotated
// by the active joint rotation R about AX and placed at r. With a = R h:
//   h' = a + m r,  I' = R I R^T + 2 (a.r) 1 - a r^T - r a^T + m (|r|^2 1 - r r^T).
template <int AX, int RM, class T> SPI_INL RI<T> ri_to_parent(const RI<T>& c, T cs, T sn, V3<T> r) {
  RI<T> o;
  o.m = c.m;
  const S3<T> I1 = rot_sym<AX>(cs, sn, c.I);
  const V3<T> a = rot<AX>(cs, sn, c.h);
  if (RM == 4) {   // r = (0, 0, z)
    const T z = r.z, mz = c.m * z;
    const T t = z * (T(2) * a.z + mz);
    o.h = v3(a.x, a.y, a.z + mz);
    o.I.xx = I1.xx + t; o.I.yy = I1.yy + t; o.I.zz = I1.zz;
    o.I.xy = I1.xy; o.I.xz = I1.xz - a.x * z; o.I.yz = I1.yz - a.y * z;
    return o;
  }
  if (RM == 2) {   // r = (0, y, 0)
    const T y = r.y, my = c.m * y;
    const T t = y * (T(2) * a.y + my);
    o.h = v3(a.x, a.y + my, a.z);
    o.I.xx = I1.xx + t; o.I.yy = I1.yy; o.I.zz = I1.zz + t;
    o.I.xy = I1.xy - a.x * y; o.I.xz = I1.xz; o.I.yz = I1.yz - a.z * y;
    return o;
  }
  // with h' = a + m r and u = a + h' = 2 a + m r: I'.xx = I1.xx + u.y r.y + u.z r.z (and cyclic),
  // I'.xy = I1.xy - h'.x r.y - a.y r.x (and the like), two multiply-adds an entry
  if (RM == 3) {   // r = (x, y, 0)
    o.h = v3(a.x + c.m * r.x, a.y + c.m * r.y, a.z);
    const T ux = a.x + o.h.x, uy = a.y + o.h.y;
    o.I.xx = I1.xx + uy * r.y;
    o.I.yy = I1.yy + ux * r.x;
    o.I.zz = I1.zz + ux * r.x + uy * r.y;
    o.I.xy = I1.xy - o.h.x * r.y - a.y * r.x;
    o.I.xz = I1.xz - a.z * r.x;
    o.I.yz = I1.yz - a.z * r.y;
    return o;
  }
  o.h = v3(a.x + c.m * r.x, a.y + c.m * r.y, a.z + c.m * r.z);
  const V3<T> u = a + o.h;
  o.I.xx = I1.xx + u.y * r.y + u.z * r.z;
  o.I.yy = I1.yy + u.x * r.x + u.z * r.z;
  o.I.zz = I1.zz + u.x * r.x + u.y * r.y;
  o.I.xy = I1.xy - o.h.x * r.y - a.y * r.x;
  o.I.xz = I1.xz - o.h.x * r.z - a.z * r.x;
  o.I.yz = I1.yz - o.h.y * r.z - a.z * r.y;
  return o;
}

// acc += ri_art(ri_to_parent<AX, RM>(c, cs, sn, r)) for a joint origin r in the x-y plane
// (RM = 3) or general (RM = 7): the rotated inertia accumulates straight onto acc's
// rotational block.
template <int AX, int RM, class T> SPI_INL void ri_to_parent_art_acc(const RI<T>& c, T cs, T sn, V3<T> r, Art<T>& acc) {
  static_assert(RM == 3 || RM == 7, "ri_to_parent_art_acc: origin pattern");
  const S3<T> I1 = rot_sym_acc<AX>(cs, sn, c.I, acc.A);
  const V3<T> a = rot<AX>(cs, sn, c.h);
  V3<T> h;
  if (RM == 3) {
    h = v3(a.x + c.m * r.x, a.y + c.m * r.y, a.z);
    const T ux = a.x + h.x, uy = a.y + h.y;
    acc.A.xx = I1.xx + uy * r.y;
    acc.A.yy = I1.yy + ux * r.x;
    acc.A.zz = I1.zz + ux * r.x + uy * r.y;
    acc.A.xy = I1.xy - h.x * r.y - a.y * r.x;
    acc.A.xz = I1.xz - a.z * r.x;
    acc.A.yz = I1.yz - a.z * r.y;
  } else {
    h = v3(a.x + c.m * r.x, a.y + c.m * r.y, a.z + c.m * r.z);
    const V3<T> u = a + h;
    acc.A.xx = I1.xx + u.y * r.y + u.z * r.z;
    acc.A.yy = I1.yy + u.x * r.x + u.z * r.z;
    acc.A.zz = I1.zz + u.x * r.x + u.y * r.y;
    acc.A.xy = I1.xy - h.x * r.y - a.y * r.x;
    acc.A.xz = I1.xz - h.x * r.z - a.z * r.x;
    acc.A.yz = I1.yz - h.y * r.z - a.z * r.y;
  }
  acc.B.m[0][1] -= h.z; acc.B.m[0][2] += h.y;
  acc.B.m[1][0] += h.z; acc.B.m[1][2] -= h.x;
  acc.B.m[2][0] -= h.y; acc.B.m[2][1] += h.x;
  acc.C.xx += c.m; acc.C.yy += c.m; acc.C.zz += c.m;
}

// ---------------------------------------------------------------------------
// model constants as the kernel sees them (built on the host from spi_robot)
// ---------------------------------------------------------------------------
struct alignas(16) F4 { float x, y, z, w; };
constexpr int kLegSlots = 14;

struct DevModel {
  // The per-leg constants phase A reads, leg-major, four to a 16-byte slot, so that one leg's
  // are contiguous (one 128-bit load per slot) and the four legs' copies of a slot sit 56
  // words apart (distinct shared-memory banks when lanes of one quad read the four legs):
  //   0..2   joint k: origin x, y, z, kd_scale kd (float product)
  //   3..11  body b at 3 + 3 b: (m, h x, h y, h z), (Ixx, Iyy, Izz, Ixy), (Ixz, Iyz, 1 / vlim_b, 0)
  //          (1 / vlim is 0 without the torque-speed limit)
  //   12, 13 the leg's two base-box corners: (c0 x, c0 y, c0 z, c1 x), (c1 y, c1 z, 0, 0)
  F4 legc[4][kLegSlots];
  // per leg body k (0 hip, 1 thigh, 2 calf), component, leg: [k][c][leg] (the same constants
  // as the source arrays of legc, for the host-side formulations)
  float org[3][3][4];
  float m[3][4];
  float h[3][3][4];
  float I[3][6][4];   // xx yy zz xy xz yz about the body origin
  float kp[3][4], kd[3][4], q0[3][4], tlim[3][4], vlim[3][4];
  float corner[8][3];
  float foot[3];
  float gain[3], tanh_a[3];
  float base_com[3], base_Ic[6];
  float base_m0, fixed_m, fixed_h[3], fixed_I[6];
  float foot_r, k, c, ct, mu, ramp_inv, imp_c;
  float corner_reach;   // largest distance of a base-box corner from the base origin
  float kd_scale, act_scale, act_clip, hip_scale, fric_vel;
  float fric_k2;          // 2 log2(e) / fric_vel
  float dt_imp_c;         // dt imp_c (float product)
  float dt, g;
  int decimation, torque_speed, base_contact, inertia_follows_mass;
};

// ---------------------------------------------------------------------------
// rollout state
// ---------------------------------------------------------------------------
template <class T> struct BaseState {
  V3<T> p;          // base origin, world
  T qx, qy, qz, qw; // orientation xyzw
  SV<T> nu;         // base spatial velocity, base coordinates
  M3<T> R;          // R(q): base -> world
};
template <class T> struct LegState { T q[3], qd[3]; };
template <class T> struct BaseParams { T m; V3<T> h; S3<T> Io; };   // base rigid inertia (+ fixed links)
template <class T> struct LegParams {                                // leg group's motor terms
  T kps, fc, arm, ts;
  // joint k's stiffness kps kp and torque limit ts tlim
  SPI_INL T kp_of(const DevModel& M, int k, int leg) const { return kps * T(M.kp[k][leg]); }
  SPI_INL T lim_of(const DevModel& M, int k, int leg) const { return ts * T(M.tlim[k][leg]); }
};
// One leg's motor terms with the per-joint products formed once (theta is fixed over a
// rollout): the same members as LegParams, for phase A's per-leg loop.
template <class T> struct LegGains {
  T kpk[3], lim[3], fc, arm;
  SPI_INL T kp_of(const DevModel&, int k, int) const { return kpk[k]; }
  SPI_INL T lim_of(const DevModel&, int k, int) const { return lim[k]; }
};
template <class T> SPI_INL LegGains<T> leg_gains(const DevModel& M, const LegParams<T>& P, int leg) {
  LegGains<T> g;
  for (int k = 0; k < 3; ++k) {
    g.kpk[k] = P.kp_of(M, k, leg);
    g.lim[k] = P.lim_of(M, k, leg);
  }
  g.fc = P.fc;
  g.arm = P.arm;
  return g;
}
template <class T> struct LegOut { Art<T> I; SV<T> p; };            // leg contribution at the base
// Phase A -> phase C. The leg's joint-space inertia factors as M = L D L^T (L unit lower
// triangular: l10, l20, l21), the coupling to the base as K = F L^-T (F = the joints' spatial
// force columns in base coordinates), so that qdd = L^-T (y - K'^T a0) with K' = K D^-1 and
// y = D^-1 L^-1 (tau - C).
template <class T> struct LegWork {
  SV<T> Kp[3];
  T y[3];
  T l10, l20, l21;
  // phase A hands its results over through this, one joint column at a time: K'_k, y_k and
  // the k-th factor entry (l10, l20, l21 in that order). A kernel may store them elsewhere,
  // e.g. straight to shared memory, with a type that has the same member.
  SPI_INL void put_col(int k, const SV<T>& v, T yk, T lk) {
    Kp[k] = v;
    y[k] = yk;
    if (k == 0) l10 = lk; else if (k == 1) l20 = lk; else l21 = lk;
  }
};

// Work records that also want the inverse pivots of M = L D L^T (D^-1 = diag(i0, i1, i2)) define
// put_diag; phase A hands them over only to those (overload resolution on the int / long tag).
template <class WK, class T>
SPI_INL auto put_diag_if(WK& w, T i0, T i1, T i2, int) -> decltype(w.put_diag(i0, i1, i2), void()) {
  w.put_diag(i0, i1, i2);
}
template <class WK, class T> SPI_INL void put_diag_if(WK&, T, T, T, long) {}

template <class T> SPI_INL M3<T> quat_to_R(T x, T y, T z, T w) {
  M3<T> R;
  R.m[0][0] = T(1) - T(2) * (y * y + z * z); R.m[0][1] = T(2) * (x * y - z * w); R.m[0][2] = T(2) * (x * z + y * w);
  R.m[1][0] = T(2) * (x * y + z * w); R.m[1][1] = T(1) - T(2) * (x * x + z * z); R.m[1][2] = T(2) * (y * z - x * w);
  R.m[2][0] = T(2) * (x * z - y * w); R.m[2][1] = T(2) * (y * z + x * w); R.m[2][2] = T(1) - T(2) * (x * x + y * y);
  return R;
}

// theta -> base rigid inertia (base + collapsed fixed links) and leg motor terms.
template <class T> SPI_INL BaseParams<T> base_params(const DevModel& M, const T* th) {
  T m = th[0];
  V3<T> c = v3(T(M.base_com[0]) + th[1], T(M.base_com[1]) + th[2], T(M.base_com[2]) + th[3]);
  T f = M.inertia_follows_mass ? m / T(M.base_m0) : T(1);
  S3<T> Ic;
  Ic.xx = f * T(M.base_Ic[0]) * th[4]; Ic.yy = f * T(M.base_Ic[1]) * th[4]; Ic.zz = f * T(M.base_Ic[2]) * th[4];
  Ic.xy = f * T(M.base_Ic[3]); Ic.xz = f * T(M.base_Ic[4]); Ic.yz = f * T(M.base_Ic[5]);
  T cc = dot(c, c);
  BaseParams<T> b;
  b.m = m + T(M.fixed_m);
  b.h = v3(m * c.x + T(M.fixed_h[0]), m * c.y + T(M.fixed_h[1]), m * c.z + T(M.fixed_h[2]));
  b.Io.xx = Ic.xx + m * (cc - c.x * c.x) + T(M.fixed_I[0]);
  b.Io.yy = Ic.yy + m * (cc - c.y * c.y) + T(M.fixed_I[1]);
  b.Io.zz = Ic.zz + m * (cc - c.z * c.z) + T(M.fixed_I[2]);
  b.Io.xy = Ic.xy - m * c.x * c.y + T(M.fixed_I[3]);
  b.Io.xz = Ic.xz - m * c.x * c.z + T(M.fixed_I[4]);
  b.Io.yz = Ic.yz - m * c.y * c.z + T(M.fixed_I[5]);
  return b;
}
template <class T> SPI_INL LegParams<T> leg_params(const T* th, int leg) {
  const bool rear = leg >= 2;   // selects, not a runtime index: keeps th in registers
  LegParams<T> p;
  p.kps = m_sel(rear, th[9], th[5]);
  p.fc = m_sel(rear, th[10], th[6]);
  p.arm = m_sel(rear, th[11], th[7]);
  p.ts = m_sel(rear, th[12], th[8]);
  return p;
}

// Penalty contact force (world) on a point at height z with world velocity v; *mimp receives
// the implicit-damping point mass of the contact (0 without contact).
template <class T> SPI_INL V3<T> contact_force(const DevModel& M, T radius, T z, V3<T> v, T* mimp) {
  T pen = radius - z;
  T s = m_clamp(pen * T(M.ramp_inv), T(0), T(1));
  // (for pen <= 0 the ramp s is 0 and k pen <= 0, so the max is 0: no contact, no select)
  T fn = m_fmax(T(0), T(M.k) * pen - T(M.c) * s * v.z);
  T vtn = m_sqrt(v.x * v.x + v.y * v.y);
  T lim = T(M.mu) * fn;
  T scale = m_sel(T(M.ct) * vtn <= lim, T(M.ct), lim / vtn);
  *mimp = m_mul2_c(s, M.dt, M.imp_c, M.dt_imp_c);
  return v3(-scale * v.x, -scale * v.y, fn);
}

// contact_force evaluated in the frame of the contact point's body: n is the world vertical
// there (unit), v the point's velocity there. The tangential velocity is v - (n.v) n, whose norm
// is the world-horizontal speed; returns the force in that frame with the implicit point mass's
// share of the gravity shift (mimp g along n) included.
template <class T> SPI_INL V3<T> contact_force_local(const DevModel& M, T radius, T z, V3<T> v, V3<T> n, T* mimp) {
  const T vz = dot(n, v);
  const V3<T> vt = v3(v.x - vz * n.x, v.y - vz * n.y, v.z - vz * n.z);
  T pen = radius - z;
  T s = m_clamp(pen * T(M.ramp_inv), T(0), T(1));
  T fn = m_fmax(T(0), T(M.k) * pen - T(M.c) * s * vz);
  T vtn = m_sqrt(dot(vt, vt));
  T lim = T(M.mu) * fn;
  T scale = m_sel(T(M.ct) * vtn <= lim, T(M.ct), lim / vtn);
  *mimp = m_mul2_c(s, M.dt, M.imp_c, M.dt_imp_c);
  const T fz = fn + *mimp * T(M.g);
  return v3(fz * n.x - scale * vt.x, fz * n.y - scale * vt.y, fz * n.z - scale * vt.z);
}

// Spatial inertia of a point mass m at r added to I.
template <class T> SPI_INL void add_point_mass(Art<T>& I, T m, V3<T> r) {
  const V3<T> h = m * r;
  I.A.xx += h.y * r.y + h.z * r.z; I.A.yy += h.x * r.x + h.z * r.z; I.A.zz += h.x * r.x + h.y * r.y;
  I.A.xy -= h.x * r.y; I.A.xz -= h.x * r.z; I.A.yz -= h.y * r.z;
  I.B.m[0][1] -= h.z; I.B.m[0][2] += h.y;
  I.B.m[1][0] += h.z; I.B.m[1][2] -= h.x;
  I.B.m[2][0] -= h.y; I.B.m[2][1] += h.x;
  I.C.xx += m; I.C.yy += m; I.C.zz += m;
}

// Joint k's position target for an action (constant over a control step's substeps).
template <class T> SPI_INL T joint_target(const DevModel& M, int k, int leg, T action) {
  T a = m_clamp(action, T(-M.act_clip), T(M.act_clip)) * T(M.act_scale);
  if (k == 0) a = a * T(M.hip_scale);
  return a + T(M.q0[k][leg]);
}
// Motor torque of joint k towards its position target.
// Motor-model shape known at compile time. kMotorRuntime: the model's flags are read at run time;
// kMotorSpeedLimit: torque-speed limit on, unit gains, no tanh saturation (motor_shape_of
// picks it for such a model; the results are the same, the flags' tests and the unit-gain
// multiplies are left out).
constexpr int kMotorRuntime = 0;
constexpr int kMotorSpeedLimit = 1;
inline int motor_shape_of(const DevModel& M) {
  for (int k = 0; k < 3; ++k)
    if (M.gain[k] != 1.0f || M.tanh_a[k] > 0.0f) return kMotorRuntime;
  return M.torque_speed ? kMotorSpeedLimit : kMotorRuntime;
}

template <int MS = kMotorRuntime, class T, class PT>
SPI_INL T motor_torque_at(const DevModel& M, const PT& P, int k, int leg, T target, T q, T qd) {
  const F4* lc = M.legc[leg];
  T tau = P.kp_of(M, k, leg) * (target - q) - m_mul2_c(qd, M.kd_scale, M.kd[k][leg], lc[k].w);
  T lim = P.lim_of(M, k, leg);
  if (MS == kMotorSpeedLimit || M.torque_speed)
    lim = lim * m_fmax(T(0), T(1) - m_div_c(m_fabs(qd), M.vlim[k][leg], lc[5 + 3 * k].z));
  tau = m_clamp(tau, -lim, lim);
  if (MS == kMotorRuntime) {
    tau = tau * T(M.gain[k]);
    if (M.tanh_a[k] > 0.0f) tau = T(M.tanh_a[k]) * m_tanh(tau / T(M.tanh_a[k]));
  }
  return tau - P.fc * m_tanh_div(qd, M.fric_vel, M.fric_k2);
}
template <class T> SPI_INL T motor_torque(const DevModel& M, const LegParams<T>& P, int k, int leg,
                                          T action, T q, T qd) {
  return motor_torque_at(M, P, k, leg, joint_target(M, k, leg, action), q, qd);
}

template <class T> SPI_INL V3<T> leg_org(const DevModel& M, int k, int leg) {
  return v3(T(M.org[k][0][leg]), T(M.org[k][1][leg]), T(M.org[k][2][leg]));
}

// The same constants from a leg's packed slots (DevModel::legc).
template <class T> SPI_INL V3<T> lc_org(const F4* c, int k) { return v3(T(c[k].x), T(c[k].y), T(c[k].z)); }
template <class T> SPI_INL RI<T> lc_ri(const F4* c, int b) {
  const F4 a = c[3 + 3 * b], d = c[4 + 3 * b], e = c[5 + 3 * b];
  RI<T> r;
  r.m = T(a.x);
  r.h = v3(T(a.y), T(a.z), T(a.w));
  r.I.xx = T(d.x); r.I.yy = T(d.y); r.I.zz = T(d.z); r.I.xy = T(d.w); r.I.xz = T(e.x); r.I.yz = T(e.y);
  return r;
}
template <class T> SPI_INL V3<T> lc_corner(const F4* c, int j) {
  return j == 0 ? v3(T(c[12].x), T(c[12].y), T(c[12].z)) : v3(T(c[12].w), T(c[13].x), T(c[13].y));
}

// c = v x (S qd) for a revolute joint about axis AX.
template <int AX, class T> SPI_INL SV<T> vel_product(const SV<T>& v, T qd) {
  SV<T> c;
  if (AX == 0) { c.w = v3(T(0), v.w.z * qd, -v.w.y * qd); c.v = v3(T(0), v.v.z * qd, -v.v.y * qd); }
  else { c.w = v3(-v.w.z * qd, T(0), v.w.x * qd); c.v = v3(-v.v.z * qd, T(0), v.v.x * qd); }
  return c;
}
template <class T> SPI_INL SV<T> operator+(const SV<T>& a, const SV<T>& b) {
  SV<T> r; r.w = a.w + b.w; r.v = a.v + b.v; return r;
}
template <class T> SPI_INL SV<T> operator*(T s, const SV<T>& a) {
  SV<T> r; r.w = s * a.w; r.v = s * a.v; return r;
}
// K - s J, componentwise.
template <class T> SPI_INL SV<T> sub_scaled(const SV<T>& K, T s, const SV<T>& J) {
  SV<T> r; r.w = K.w - s * J.w; r.v = K.v - s * J.v; return r;
}
// I -= a b^T for a symmetric rank-one a b^T (only the 21 stored entries).
template <class T> SPI_INL void art_sub_outer(Art<T>& I, const SV<T>& a, const SV<T>& b) {
  I.A.xx -= a.w.x * b.w.x; I.A.yy -= a.w.y * b.w.y; I.A.zz -= a.w.z * b.w.z;
  I.A.xy -= a.w.x * b.w.y; I.A.xz -= a.w.x * b.w.z; I.A.yz -= a.w.y * b.w.z;
  I.B.m[0][0] -= a.w.x * b.v.x; I.B.m[0][1] -= a.w.x * b.v.y; I.B.m[0][2] -= a.w.x * b.v.z;
  I.B.m[1][0] -= a.w.y * b.v.x; I.B.m[1][1] -= a.w.y * b.v.y; I.B.m[1][2] -= a.w.y * b.v.z;
  I.B.m[2][0] -= a.w.z * b.v.x; I.B.m[2][1] -= a.w.z * b.v.y; I.B.m[2][2] -= a.w.z * b.v.z;
  I.C.xx -= a.v.x * b.v.x; I.C.yy -= a.v.y * b.v.y; I.C.zz -= a.v.z * b.v.z;
  I.C.xy -= a.v.x * b.v.y; I.C.xz -= a.v.x * b.v.z; I.C.yz -= a.v.y * b.v.z;
}

// Sparse forms of the above for operands with structural zeros. IEEE rules keep a product
// with a literal 0.0f (it is NaN for an infinite factor), so these write only the terms that
// are not structurally zero; for finite operands each equals its dense counterpart.
//
// acc + X m across a thigh joint (axis y, origin on y) for m = vel_product<0>(...) (m.w.x =
// m.v.x = 0) and acc = vel_product<1>(...) (acc.w.y = acc.v.y = 0).
template <class T> SPI_INL SV<T> thigh_accel(const SV<T>& m, T c, T s, V3<T> r, const SV<T>& acc) {
  SV<T> o;
  o.w = v3(acc.w.x - s * m.w.z, m.w.y, acc.w.z + c * m.w.z);
  const T t = -(r.y * m.w.z);
  o.v = v3(acc.v.x + c * t - s * m.v.z, m.v.y, acc.v.z + s * t + c * m.v.z);
  return o;
}
// acc + X m across a joint about y (origin sparsity RM) for acc = vel_product<1>(...).
template <int RM, class T> SPI_INL SV<T> motion_to_child_acc_y0(const SV<T>& m, T c, T s, V3<T> r, const SV<T>& acc) {
  SV<T> o;
  o.w = v3(acc.w.x + c * m.w.x - s * m.w.z, m.w.y, acc.w.z + s * m.w.x + c * m.w.z);
  const V3<T> u = sub_rcross<RM>(m.v, r, m.w);
  o.v = v3(acc.v.x + c * u.x - s * u.z, u.y, acc.v.z + s * u.x + c * u.z);
  return o;
}
// acc + I m for m = vel_product<0>(...) (m.w.x = m.v.x = 0).
template <class T> SPI_INL SV<T> ri_mul_acc_x0(const RI<T>& I, const SV<T>& m, const SV<T>& acc) {
  const T a = m.w.y, b = m.w.z, c = m.v.y, d = m.v.z;
  const V3<T> h = I.h;
  SV<T> r;
  r.w = v3(acc.w.x + I.I.xy * a + I.I.xz * b + h.y * d - h.z * c,
           acc.w.y + I.I.yy * a + I.I.yz * b - h.x * d,
           acc.w.z + I.I.yz * a + I.I.zz * b + h.x * c);
  r.v = v3(acc.v.x + a * h.z - b * h.y, acc.v.y + I.m * c + b * h.x, acc.v.z + I.m * d - a * h.x);
  return r;
}
// X^T f across a joint about y (origin sparsity RM = 2 or 4) for a joint force column
// f = ri_col<1>(...) or one already carried across such a joint (f.v.y = 0, and so is the
// result's).
template <int RM, class T> SPI_INL SV<T> col_to_parent_y(const SV<T>& f, T c, T s, V3<T> r) {
  SV<T> o;
  o.v = v3(c * f.v.x + s * f.v.z, T(0), c * f.v.z - s * f.v.x);
  const V3<T> u = rot<1>(c, s, f.w);
  if (RM == 4) o.w = v3(u.x, u.y + r.z * o.v.x, u.z);
  else o.w = v3(u.x + r.y * o.v.z, u.y, u.z - r.y * o.v.x);
  return o;
}
// X^T f across the hip joint (axis x, origin in the x-y plane) for f.v.y = 0.
template <class T> SPI_INL SV<T> hip_col_to_base_vy0(const SV<T>& f, T c, T s, V3<T> r) {
  SV<T> o;
  o.v = v3(f.v.x, -(s * f.v.z), c * f.v.z);
  o.w = add_rcross<kHipRM>(rot<0>(c, s, f.w), r, o.v);
  return o;
}
// X^T f across the hip joint for the hip's own column f = ri_col<0>(...) (f.v.x = 0, and so
// is the result's).
template <class T> SPI_INL SV<T> hip_col_to_base_vx0(const SV<T>& f, T c, T s, V3<T> r) {
  SV<T> o;
  o.v = v3(T(0), c * f.v.y - s * f.v.z, s * f.v.y + c * f.v.z);
  const V3<T> u = rot<0>(c, s, f.w);
  o.w = v3(u.x + r.y * o.v.z, u.y - r.x * o.v.z, u.z + r.x * o.v.y);
  return o;
}
// K - s J (as sub_scaled) for J.v.x = 0.
template <class T> SPI_INL SV<T> sub_scaled_vx0(const SV<T>& K, T s, const SV<T>& J) {
  SV<T> r;
  r.w = K.w - s * J.w;
  r.v = v3(K.v.x, K.v.y - s * J.v.y, K.v.z - s * J.v.z);
  return r;
}
// I -= a b^T (as art_sub_outer) for a.v.x = b.v.x = 0.
template <class T> SPI_INL void art_sub_outer_vx0(Art<T>& I, const SV<T>& a, const SV<T>& b) {
  I.A.xx -= a.w.x * b.w.x; I.A.yy -= a.w.y * b.w.y; I.A.zz -= a.w.z * b.w.z;
  I.A.xy -= a.w.x * b.w.y; I.A.xz -= a.w.x * b.w.z; I.A.yz -= a.w.y * b.w.z;
  I.B.m[0][1] -= a.w.x * b.v.y; I.B.m[0][2] -= a.w.x * b.v.z;
  I.B.m[1][1] -= a.w.y * b.v.y; I.B.m[1][2] -= a.w.y * b.v.z;
  I.B.m[2][1] -= a.w.z * b.v.y; I.B.m[2][2] -= a.w.z * b.v.z;
  I.C.yy -= a.v.y * b.v.y; I.C.zz -= a.v.z * b.v.z; I.C.yz -= a.v.y * b.v.z;
}

// ---------------------------------------------------------------------------
// Phase A: everything of one leg (and two base corners) up to its base contribution.
//
// The leg is condensed onto the base through its joint-space equations. With the base
// acceleration a0 (gravity-shifted frame) as input, the leg obeys
//   M qdd + F^T a0 + C = tau,    force on the base = I_c a0 + F qdd + p_c,
// where I_c is the leg's composite rigid inertia at the base, F_k = I_k^c S_k the spatial force
// column of joint k (composite inertia of the bodies below joint k times its axis), M the
// 3x3 joint-space inertia plus armature, and (p_c, C) the bias force and joint bias torques of
// a recursive Newton-Euler pass with a0 = 0, qdd = 0 (velocity products, the foot contact,
// body velocity terms). Eliminating qdd gives the leg's articulated inertia and bias at the
// base, I_c - F M^-1 F^T and p_c + F M^-1 (tau - C) -- the quantities Featherstone's ABA
// backward pass produces, from fewer operations for a three-joint chain.
// ---------------------------------------------------------------------------
// Whether phase A evaluates the base-box corners: a corner can only reach the ground when the
// base origin is lower than the box's half-diagonal, so a warp whose rollouts are all higher
// skips them. One vote per warp and base state, shared by the four legs.
template <class T> SPI_INL bool corners_may_touch(const DevModel& M, const BaseState<T>& B) {
  return M.base_contact && warp_any(B.p.z < T(M.corner_reach));
}

// ACC = false: out receives the leg's contribution; ACC = true: the contribution is added to out
// (the running sum over legs, which may start from the base body's own terms).
// TGT = false: act holds the leg's three actions; TGT = true: their joint targets (joint_target).
// PT: LegParams, or LegGains.
template <bool ACC, bool TGT, int MS, class T, class WK, class PT>
SPI_INL void phase_a_core(const DevModel& M, int leg, const BaseState<T>& B, const LegState<T>& L,
                          const PT& P, const T act[3], WK& W, LegOut<T>& out, bool corners) {
  T tau[3], C[3], S[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    tau[k] = motor_torque_at<MS>(M, P, k, leg, TGT ? act[k] : joint_target(M, k, leg, act[k]), L.q[k], L.qd[k]);
    m_sincos(L.q[k], &S[k], &C[k]);
  }
  const F4* lc = M.legc[leg];
  V3<T> r0 = lc_org<T>(lc, 0), r1 = lc_org<T>(lc, 1), r2 = lc_org<T>(lc, 2);
  // body velocities (body coordinates) and velocity-product accelerations
  SV<T> v0 = motion_to_child<0, kHipRM>(B.nu, C[0], S[0], r0); v0.w.x = v0.w.x + L.qd[0];
  SV<T> v1 = motion_to_child<1, 2>(v0, C[1], S[1], r1);   v1.w.y = v1.w.y + L.qd[1];
  SV<T> v2 = motion_to_child<1, 4>(v1, C[2], S[2], r2);   v2.w.y = v2.w.y + L.qd[2];
  const SV<T> cb0 = vel_product<0>(v0, L.qd[0]), cb1 = vel_product<1>(v1, L.qd[1]),
              cb2 = vel_product<1>(v2, L.qd[2]);
  // foot contact, evaluated in the calf frame: the world vertical brought down the chain (g_k in
  // body k's parent frame), the foot height from it and the joint origins, the foot velocity
  // from the calf's. The implicit point mass acts on the true acceleration while the dynamics
  // run in the gravity-shifted frame: its share of the shift enters as a force mimp g upwards.
  // (the foot lies on the calf's z axis, fc = (0, 0, fz): the model builder checks it)
  const T fz = T(M.foot[2]);
  const V3<T> g0 = row(B.R, 2);
  const V3<T> g1 = rotT<0>(C[0], S[0], g0);
  const V3<T> g2 = rotT<1>(C[1], S[1], g1);
  const V3<T> g3 = rotT<1>(C[2], S[2], g2);
  const T zf = B.p.z + g0.x * r0.x + g0.y * r0.y + g1.y * r1.y + g2.z * r2.z + g3.z * fz;
  T mimp;
  const V3<T> Fc = contact_force_local(M, T(M.foot_r), zf, v3(v2.v.x + v2.w.y * fz, v2.v.y - v2.w.x * fz, v2.v.z),
                                       g3, &mimp);
  // composite inertias: calf (+ the contact's implicit point mass at the foot) -> thigh -> hip
  const RI<T> Ical = lc_ri<T>(lc, 2);
  RI<T> Rc2 = Ical;
  {   // ri_add_point(Rc2, mimp, (0, 0, fz))
    const T hz = mimp * fz, q = hz * fz;
    Rc2.m = Rc2.m + mimp;
    Rc2.h.z = Rc2.h.z + hz;
    Rc2.I.xx = Rc2.I.xx + q;
    Rc2.I.yy = Rc2.I.yy + q;
  }
  const RI<T> Rc1 = ri_to_parent_acc<1, 4>(Rc2, C[2], S[2], r2, lc_ri<T>(lc, 1));
  const RI<T> Rc0 = ri_to_parent_acc<1, 2>(Rc1, C[1], S[1], r1, lc_ri<T>(lc, 0));
  // bias pass (a0 = 0, qdd = 0): accelerations are the accumulated velocity products; the
  // implicit point mass takes part in the inertial force, not in the velocity term
  const SV<T> ab1 = thigh_accel(cb0, C[1], S[1], r1, cb1);
  const SV<T> ab2 = motion_to_child_acc_y0<4>(ab1, C[2], S[2], r2, cb2);
  SV<T> f2 = ri_mul_acc(Rc2, ab2, crf(v2, ri_mul(Ical, v2)));
  f2.w = v3(f2.w.x + Fc.y * fz, f2.w.y - Fc.x * fz, f2.w.z);   // + Fc x (0, 0, fz)
  f2.v = f2.v - Fc;
  SV<T> f1;
  {
    const RI<T> Ith = lc_ri<T>(lc, 1);
    f1 = ri_mul_acc(Ith, ab1, crf_acc(v1, ri_mul(Ith, v1), force_to_parent<1, 4>(f2, C[2], S[2], r2)));
  }
  SV<T> f0;
  {
    const RI<T> Ihp = lc_ri<T>(lc, 0);
    f0 = ri_mul_acc_x0(Ihp, cb0, crf_acc(v0, ri_mul(Ihp, v0), force_to_parent<1, 2>(f1, C[1], S[1], r1)));
  }
  const SV<T> pc = ACC ? force_to_parent_acc<0, kHipRM>(f0, C[0], S[0], r0, out.p)
                       : force_to_parent<0, kHipRM>(f0, C[0], S[0], r0);
  // joint force columns F_k = I_k^c S_k in base coordinates, and the joint-space inertia
  const SV<T> F2t = col_to_parent_y<4>(ri_col<1>(Rc2), C[2], S[2], r2);
  const SV<T> F2h = col_to_parent_y<2>(F2t, C[1], S[1], r1);
  const SV<T> F1h = col_to_parent_y<2>(ri_col<1>(Rc1), C[1], S[1], r1);
  const SV<T> F0h = ri_col<0>(Rc0);
  const T M00 = Rc0.I.xx + P.arm, M11 = Rc1.I.yy + P.arm, M22 = Rc2.I.yy + P.arm;
  const T M01 = F1h.w.x, M02 = F2h.w.x, M12 = F2t.w.y;
  // M = L D L^T
  const T i0 = T(1) / M00;
  const T l10 = M01 * i0, l20 = M02 * i0;
  const T i1 = T(1) / (M11 - l10 * M01);
  const T e12 = M12 - l20 * M01;
  const T l21 = e12 * i1;
  const T i2 = T(1) / (M22 - l20 * M02 - l21 * e12);
  put_diag_if(W, i0, i1, i2, 0);
  // K = F L^-T (base coordinates), K' = K D^-1, y = D^-1 L^-1 (tau - C)
  // (F0h.v.x = 0 and F1h.v.y = F2h.v.y = 0 by construction, so K0.v.x = 0)
  const SV<T> K0 = hip_col_to_base_vx0(F0h, C[0], S[0], r0);
  const SV<T> K1 = sub_scaled_vx0(hip_col_to_base_vy0(F1h, C[0], S[0], r0), l10, K0);
  const SV<T> K2 = sub_scaled(sub_scaled_vx0(hip_col_to_base_vy0(F2h, C[0], S[0], r0), l20, K0), l21, K1);
  SV<T> Kp0;
  Kp0.w = i0 * K0.w;
  Kp0.v = v3(T(0), i0 * K0.v.y, i0 * K0.v.z);
  const SV<T> Kp1 = i1 * K1, Kp2 = i2 * K2;
  const T z0 = tau[0] - f0.w.x;
  const T z1 = (tau[1] - f1.w.y) - l10 * z0;
  const T z2 = (tau[2] - f2.w.y) - l20 * z0 - l21 * z1;
  const T y0 = z0 * i0, y1 = z1 * i1, y2 = z2 * i2;
  W.put_col(0, Kp0, y0, l10);
  W.put_col(1, Kp1, y1, l20);
  W.put_col(2, Kp2, y2, l21);
  // the leg at the base: articulated inertia I_c - K D^-1 K^T, bias p_c + K y
  if (ACC) ri_to_parent_art_acc<0, kHipRM>(Rc0, C[0], S[0], r0, out.I);
  else out.I = ri_art(ri_to_parent<0, kHipRM>(Rc0, C[0], S[0], r0));
  art_sub_outer_vx0(out.I, Kp0, K0);
  art_sub_outer(out.I, Kp1, K1);
  art_sub_outer(out.I, Kp2, K2);
  out.p.w = v3(pc.w.x + y2 * K2.w.x + y1 * K1.w.x + y0 * K0.w.x, pc.w.y + y2 * K2.w.y + y1 * K1.w.y + y0 * K0.w.y,
               pc.w.z + y2 * K2.w.z + y1 * K1.w.z + y0 * K0.w.z);
  out.p.v = v3(pc.v.x + y2 * K2.v.x + y1 * K1.v.x, pc.v.y + y2 * K2.v.y + y1 * K1.v.y + y0 * K0.v.y,
               pc.v.z + y2 * K2.v.z + y1 * K1.v.z + y0 * K0.v.z);
  // two of the eight base-box corners, when corners_may_touch (a corner off the ground adds
  // exactly zero force and zero implicit mass)
  if (corners) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const V3<T> rc = lc_corner<T>(lc, j);
      V3<T> vc = cross_acc(B.nu.w, rc, B.nu.v);
      T mc;
      V3<T> Fw = contact_force(M, T(0), B.p.z + B.R.m[2][0] * rc.x + B.R.m[2][1] * rc.y + B.R.m[2][2] * rc.z,
                               mul(B.R, vc), &mc);
      Fw.z = Fw.z + mc * T(M.g);
      V3<T> Fb = mulT(B.R, Fw);
      out.p.w = cross_acc(Fb, rc, out.p.w);
      out.p.v = out.p.v - Fb;
      add_point_mass(out.I, mc, rc);
    }
  }
}

template <class T, class WK>
SPI_INL LegOut<T> phase_a(const DevModel& M, int leg, const BaseState<T>& B, const LegState<T>& L,
                          const LegParams<T>& P, const T act[3], WK& W) {
  LegOut<T> out;
  phase_a_core<false, false, kMotorRuntime>(M, leg, B, L, P, act, W, out, corners_may_touch(M, B));
  return out;
}
// Phase A adding the leg's contribution to acc, from the leg's joint targets tgt (joint_target
// of its three actions, formed once per control step); corners: corners_may_touch(M, B).
// MS: the motor shape (motor_shape_of the model, or kMotorRuntime).
template <int MS = kMotorRuntime, class T, class WK, class PT>
SPI_INL void phase_a_into(const DevModel& M, int leg, const BaseState<T>& B, const LegState<T>& L,
                          const PT& P, const T tgt[3], WK& W, LegOut<T>& acc, bool corners) {
  phase_a_core<true, true, MS>(M, leg, B, L, P, tgt, W, acc, corners);
}

// ---------------------------------------------------------------------------
// Phase B: base solve and base integration. `sum` is the sum of the four LegOut.
// Returns the base acceleration with gravity removed (the frame the legs' forward pass uses).
// ---------------------------------------------------------------------------
template <class T>
SPI_INL SV<T> base_solve(const DevModel& M, const Art<T>& IA, const SV<T>& pA, BaseState<T>& B);

template <class T>
SPI_INL SV<T> phase_b(const DevModel& M, const BaseParams<T>& bp, const LegOut<T>& sum, BaseState<T>& B) {
  Art<T> IA = rigid(bp.m, bp.h, bp.Io);
  add_to(IA, sum.I);
  return base_solve(M, IA, crf_acc(B.nu, rigid_mul(bp.m, bp.h, bp.Io, B.nu), sum.p), B);
}

// The base body's own terms, the start of a running sum over legs (phase_a_into) that
// base_solve then takes as the total articulated inertia and bias force.
template <class T> SPI_INL LegOut<T> base_terms(const BaseParams<T>& bp, const BaseState<T>& B) {
  LegOut<T> o;
  o.I = rigid(bp.m, bp.h, bp.Io);
  o.p = crf(B.nu, rigid_mul(bp.m, bp.h, bp.Io, B.nu));
  return o;
}

// Base solve and base integration from the total articulated inertia IA and bias force pA at
// the base. Returns the base acceleration with gravity removed.
template <class T>
SPI_INL SV<T> base_solve(const DevModel& M, const Art<T>& IA, const SV<T>& pA, BaseState<T>& B) {
  // 6x6 symmetric matrix in (w; v) order, Cholesky L L^T, solve IA a = -pA
  T Mx[6][6];
  Mx[0][0] = IA.A.xx; Mx[1][1] = IA.A.yy; Mx[2][2] = IA.A.zz;
  Mx[1][0] = IA.A.xy; Mx[2][0] = IA.A.xz; Mx[2][1] = IA.A.yz;
  Mx[3][3] = IA.C.xx; Mx[4][4] = IA.C.yy; Mx[5][5] = IA.C.zz;
  Mx[4][3] = IA.C.xy; Mx[5][3] = IA.C.xz; Mx[5][4] = IA.C.yz;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Mx[3 + j][i] = IA.B.m[i][j];   // lower block = B^T
  T rhs[6] = {-pA.w.x, -pA.w.y, -pA.w.z, -pA.v.x, -pA.v.y, -pA.v.z};
  T invL[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    T d = Mx[j][j];
#pragma unroll
    for (int k = 0; k < j; ++k) d = d - Mx[j][k] * Mx[j][k];
    T inv = T(1) / m_sqrt(d);
    invL[j] = inv;
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      T a = Mx[i][j];
#pragma unroll
      for (int k = 0; k < j; ++k) a = a - Mx[i][k] * Mx[j][k];
      Mx[i][j] = a * inv;
    }
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    T a = rhs[i];
#pragma unroll
    for (int k = 0; k < i; ++k) a = a - Mx[i][k] * rhs[k];
    rhs[i] = a * invL[i];
  }
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    T a = rhs[i];
#pragma unroll
    for (int k = i + 1; k < 6; ++k) a = a - Mx[k][i] * rhs[k];
    rhs[i] = a * invL[i];
  }
  SV<T> a0;
  a0.w = v3(rhs[0], rhs[1], rhs[2]);
  a0.v = v3(rhs[3], rhs[4], rhs[5]);
  // integrate: true acceleration adds gravity expressed in base coordinates
  T dt = T(M.dt), g = T(M.g);
  B.nu.w = B.nu.w + dt * a0.w;
  B.nu.v = B.nu.v + dt * (a0.v - g * row(B.R, 2));
  T hx = T(0.5) * dt;
  V3<T> w = B.nu.w;
  T nx = B.qx + hx * (B.qw * w.x + (B.qy * w.z - B.qz * w.y));
  T ny = B.qy + hx * (B.qw * w.y + (B.qz * w.x - B.qx * w.z));
  T nz = B.qz + hx * (B.qw * w.z + (B.qx * w.y - B.qy * w.x));
  T nw = B.qw - hx * (B.qx * w.x + B.qy * w.y + B.qz * w.z);
  T inv = T(1) / m_sqrt(nx * nx + ny * ny + nz * nz + nw * nw);
  B.qx = nx * inv; B.qy = ny * inv; B.qz = nz * inv; B.qw = nw * inv;
  B.R = quat_to_R(B.qx, B.qy, B.qz, B.qw);
  B.p = B.p + dt * mul(B.R, B.nu.v);
  return a0;
}

// ---------------------------------------------------------------------------
// Phase C: joint accelerations of one leg from the base acceleration, then joint integration:
// qdd = L^-T (y - K'^T a0).
// ---------------------------------------------------------------------------
template <class T, class WK>
SPI_INL void phase_c(const DevModel& M, int leg, const SV<T>& a0, const WK& W, LegState<T>& L) {
  (void)leg;
  T w[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const SV<T>& q = W.Kp[k];
    // K'_0.v.x is 0 by construction (the hip's own force column has no x force)
    const T vx = k == 0 ? W.y[k] : W.y[k] - q.v.x * a0.v.x;
    w[k] = vx - q.w.x * a0.w.x - q.w.y * a0.w.y - q.w.z * a0.w.z - q.v.y * a0.v.y - q.v.z * a0.v.z;
  }
  const T w0 = w[0], w1 = w[1], w2 = w[2];
  T qdd[3];
  qdd[2] = w2;
  qdd[1] = w1 - W.l21 * qdd[2];
  qdd[0] = w0 - W.l10 * qdd[1] - W.l20 * qdd[2];
  T dt = T(M.dt);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    L.qd[k] = L.qd[k] + dt * qdd[k];
    L.q[k] = L.q[k] + dt * L.qd[k];
  }
}

// Window start: world-frame root state -> body-frame velocity.
template <class T> SPI_INL void base_from_world(BaseState<T>& B, const T* s13) {
  B.p = v3(s13[0], s13[1], s13[2]);
  B.qx = s13[3]; B.qy = s13[4]; B.qz = s13[5]; B.qw = s13[6];
  B.R = quat_to_R(B.qx, B.qy, B.qz, B.qw);
  B.nu.v = mulT(B.R, v3(s13[7], s13[8], s13[9]));
  B.nu.w = mulT(B.R, v3(s13[10], s13[11], s13[12]));
}
template <class T> SPI_INL void base_to_world(const BaseState<T>& B, T* s13) {
  s13[0] = B.p.x; s13[1] = B.p.y; s13[2] = B.p.z;
  s13[3] = B.qx; s13[4] = B.qy; s13[5] = B.qz; s13[6] = B.qw;
  V3<T> v = mul(B.R, B.nu.v), w = mul(B.R, B.nu.w);
  s13[7] = v.x; s13[8] = v.y; s13[9] = v.z;
  s13[10] = w.x; s13[11] = w.y; s13[12] = w.z;
}

}  // namespace spi
