// dual.cuh -- forward-mode (tangent-linear) scalar for the rollout dynamics.
//
// Df carries a value and one directional derivative. Instantiating the templated phases of
// dynamics.cuh with T = Df propagates d(state)/d(theta_k) through exactly the same
// arithmetic as the primal kernel: each rollout lane quad follows one parameter direction.
// Non-smooth operations take the derivative of the branch they select (clip, max, min,
// contact on/off, stick/slip), the usual convention for penalty contact.
#pragma once

#include "dynamics.cuh"

namespace spi {

struct Df {
  float v, d;
  SPI_INL Df() : v(0.f), d(0.f) {}
  SPI_INL Df(float x) : v(x), d(0.f) {}
  SPI_INL Df(double x) : v((float)x), d(0.f) {}
  SPI_INL Df(int x) : v((float)x), d(0.f) {}
  SPI_INL Df(float x, float dx) : v(x), d(dx) {}
};

SPI_INL Df operator+(Df a, Df b) { return Df(a.v + b.v, a.d + b.d); }
SPI_INL Df operator-(Df a, Df b) { return Df(a.v - b.v, a.d - b.d); }
SPI_INL Df operator*(Df a, Df b) { return Df(a.v * b.v, a.d * b.v + a.v * b.d); }
SPI_INL Df operator/(Df a, Df b) {
  const float q = a.v / b.v;
  return Df(q, (a.d - q * b.d) / b.v);
}
SPI_INL Df operator-(Df a) { return Df(-a.v, -a.d); }
SPI_INL Df& operator+=(Df& a, Df b) { a = a + b; return a; }
SPI_INL Df& operator-=(Df& a, Df b) { a = a - b; return a; }
SPI_INL bool operator>(Df a, Df b) { return a.v > b.v; }
SPI_INL bool operator<=(Df a, Df b) { return a.v <= b.v; }
SPI_INL bool operator<(Df a, Df b) { return a.v < b.v; }

SPI_INL Df m_sqrt(Df x) {
  const float r = m_sqrt(x.v);
  return Df(r, r > 0.f ? x.d * 0.5f / r : 0.f);
}
SPI_INL Df m_tanh(Df x) {
  const float t = m_tanh(x.v);
  return Df(t, x.d * (1.f - t * t));
}
SPI_INL void m_sincos(Df x, Df* s, Df* c) {
  float sv, cv;
  m_sincos(x.v, &sv, &cv);
  *s = Df(sv, cv * x.d);
  *c = Df(cv, -sv * x.d);
}
SPI_INL Df m_fabs(Df x) { return x.v >= 0.f ? x : Df(-x.v, -x.d); }
SPI_INL Df m_fmax(Df a, Df b) { return a.v >= b.v ? a : b; }
SPI_INL Df m_fmin(Df a, Df b) { return a.v <= b.v ? a : b; }

}  // namespace spi
