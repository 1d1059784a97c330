// Exchange-correlation energy densities, differentiated by forward-mode duals.
//
// LDA pieces follow hqc/tools/excor.py:3-126 (Slater exchange; VWN, HL71,
// BH72, GL77 correlation).  The reference takes v = d(rho*eps)/d rho with
// jax.grad per grid point (hqc/pbc/solver.py:672-678); here the same
// derivative comes from a two-component dual number, which is exact to
// rounding.  GGA-PBE (Perdew-Burke-Ernzerhof 1996 on PW92 correlation) has no
// counterpart in the reference.
#pragma once
#include <cuda_runtime.h>

namespace hqcgb {

template <typename T>
struct Dual2 {
  T v, a, b;  // value, d/d rho, d/d sigma
  __host__ __device__ Dual2() : v(0), a(0), b(0) {}
  __host__ __device__ Dual2(T x) : v(x), a(0), b(0) {}
  __host__ __device__ Dual2(T x, T da, T db) : v(x), a(da), b(db) {}
};

#define HQ_DOP __host__ __device__ inline
template <typename T> HQ_DOP Dual2<T> operator+(Dual2<T> x, Dual2<T> y) { return {x.v + y.v, x.a + y.a, x.b + y.b}; }
template <typename T> HQ_DOP Dual2<T> operator-(Dual2<T> x, Dual2<T> y) { return {x.v - y.v, x.a - y.a, x.b - y.b}; }
template <typename T> HQ_DOP Dual2<T> operator-(Dual2<T> x) { return {-x.v, -x.a, -x.b}; }
template <typename T> HQ_DOP Dual2<T> operator*(Dual2<T> x, Dual2<T> y) {
  return {x.v * y.v, x.a * y.v + x.v * y.a, x.b * y.v + x.v * y.b};
}
template <typename T> HQ_DOP Dual2<T> operator/(Dual2<T> x, Dual2<T> y) {
  T inv = T(1) / y.v;
  T q = x.v * inv;
  return {q, (x.a - q * y.a) * inv, (x.b - q * y.b) * inv};
}
template <typename T> HQ_DOP Dual2<T> operator+(Dual2<T> x, T c) { return {x.v + c, x.a, x.b}; }
template <typename T> HQ_DOP Dual2<T> operator+(T c, Dual2<T> x) { return {x.v + c, x.a, x.b}; }
template <typename T> HQ_DOP Dual2<T> operator-(Dual2<T> x, T c) { return {x.v - c, x.a, x.b}; }
template <typename T> HQ_DOP Dual2<T> operator-(T c, Dual2<T> x) { return {c - x.v, -x.a, -x.b}; }
template <typename T> HQ_DOP Dual2<T> operator*(Dual2<T> x, T c) { return {x.v * c, x.a * c, x.b * c}; }
template <typename T> HQ_DOP Dual2<T> operator*(T c, Dual2<T> x) { return {x.v * c, x.a * c, x.b * c}; }
template <typename T> HQ_DOP Dual2<T> operator/(Dual2<T> x, T c) { return {x.v / c, x.a / c, x.b / c}; }
template <typename T> HQ_DOP Dual2<T> operator/(T c, Dual2<T> y) { return Dual2<T>(c) / y; }

HQ_DOP double d_log(double x) { return log(x); }
HQ_DOP float d_log(float x) { return logf(x); }
HQ_DOP double d_exp(double x) { return exp(x); }
HQ_DOP float d_exp(float x) { return expf(x); }
HQ_DOP double d_sqrt(double x) { return sqrt(x); }
HQ_DOP float d_sqrt(float x) { return sqrtf(x); }
HQ_DOP double d_cbrt(double x) { return cbrt(x); }
HQ_DOP float d_cbrt(float x) { return cbrtf(x); }
HQ_DOP double d_atan(double x) { return atan(x); }
HQ_DOP float d_atan(float x) { return atanf(x); }

template <typename T> HQ_DOP Dual2<T> dlog(Dual2<T> x) { T i = T(1) / x.v; return {d_log(x.v), x.a * i, x.b * i}; }
template <typename T> HQ_DOP Dual2<T> dexp(Dual2<T> x) { T e = d_exp(x.v); return {e, x.a * e, x.b * e}; }
template <typename T> HQ_DOP Dual2<T> dsqrt(Dual2<T> x) { T s = d_sqrt(x.v); T h = T(0.5) / s; return {s, x.a * h, x.b * h}; }
template <typename T> HQ_DOP Dual2<T> dcbrt(Dual2<T> x) {
  T c = d_cbrt(x.v);
  T h = T(1) / (T(3) * c * c);
  return {c, x.a * h, x.b * h};
}
template <typename T> HQ_DOP Dual2<T> datan(Dual2<T> x) { T h = T(1) / (T(1) + x.v * x.v); return {d_atan(x.v), x.a * h, x.b * h}; }

// ---------------------------------------------------------------------------
template <typename T>
HQ_DOP Dual2<T> eps_x_lda(Dual2<T> rho) {
  // -3/4 (3/pi)^(1/3) rho^(1/3)      (excor.py:8-12)
  const T c = T(-0.75) * T(0.98474502184269651);  // (3/pi)^(1/3)
  return c * dcbrt(rho);
}

template <typename T>
HQ_DOP Dual2<T> eps_vwn(Dual2<T> rho) {
  // excor.py:37-49, 76-85
  const T A = T(0.0621814), y0 = T(-0.10498), b = T(3.72744), c = T(12.93532);
  const T Yy0 = y0 * y0 + b * y0 + c;
  const T Q = d_sqrt(T(4) * c - b * b);
  const T c0 = A / T(2);
  const T c1 = c0 * T(2) * b / Q;
  const T c2 = c0 * b * y0 / Yy0;
  const T c3 = c2 * T(2) * (b + T(2) * y0) / Q;
  const T c4 = c1 - c3;
  const T ws = T(0.62035049089940013);  // (3/(4 pi))^(1/3)
  Dual2<T> rs = ws / dcbrt(rho);
  Dual2<T> y = dsqrt(rs);
  Dual2<T> Yy = y * y + b * y + c;
  Dual2<T> at = datan(Q / (T(2) * y + b));
  Dual2<T> ym = y - y0;
  return c0 * dlog(y * y / Yy) + c4 * at - c2 * dlog(ym * ym / Yy);
}

template <typename T>
HQ_DOP Dual2<T> eps_hl_family(Dual2<T> rho, T Acoef, T Ccoef) {
  // excor.py:87-112
  const T ws = T(0.62035049089940013);
  Dual2<T> rs = ws / dcbrt(rho);
  Dual2<T> x = rs / Acoef;
  Dual2<T> x3 = x * x * x;
  return T(-0.5) * Ccoef * ((T(1) + x3) * dlog(T(1) + T(1) / x) + x / T(2) - x * x - T(1) / T(3));
}

template <typename T>
HQ_DOP Dual2<T> eps_c_pw92(Dual2<T> rs) {
  const T A = T(0.0310907), a1 = T(0.21370), b1 = T(7.5957), b2 = T(3.5876), b3 = T(1.6382),
          b4 = T(0.49294);
  Dual2<T> srs = dsqrt(rs);
  Dual2<T> q = T(2) * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  return T(-2) * A * (T(1) + a1 * rs) * dlog(T(1) + T(1) / q);
}

// PBE energy per volume e(rho, sigma), sigma = |grad rho|^2.
template <typename T>
HQ_DOP Dual2<T> e_pbe(Dual2<T> rho, Dual2<T> sigma) {
  const T kappa = T(0.804), beta = T(0.06672455060314922);
  const T mu = T(0.21951497276451704);          // beta pi^2 / 3
  const T gam = T(0.031090690869654900);        // (1 - ln 2)/pi^2
  const T pi = T(3.14159265358979324);
  Dual2<T> kf = dcbrt(T(3) * pi * pi * rho);
  Dual2<T> exu = T(-3) / (T(4) * pi) * kf;
  Dual2<T> s2 = sigma / (T(4) * kf * kf * rho * rho);
  Dual2<T> Fx = T(1) + kappa - kappa / (T(1) + mu * s2 / kappa);
  Dual2<T> rs = dcbrt(T(3) / (T(4) * pi * rho));
  Dual2<T> ec = eps_c_pw92(rs);
  Dual2<T> ks2 = T(4) * kf / pi;
  Dual2<T> t2 = sigma / (T(4) * ks2 * rho * rho);
  Dual2<T> Acoef = (beta / gam) / (dexp(-ec / gam) - T(1));
  Dual2<T> At2 = Acoef * t2;
  Dual2<T> H = gam * dlog(T(1) + (beta / gam) * t2 * (T(1) + At2) / (T(1) + At2 + At2 * At2));
  return rho * (exu * Fx + ec + H);
}

// Energy per volume and its partials (v_rho, v_sigma) for one grid point.
template <typename T>
__device__ inline void xc_point(int kind, T rho, T sigma, T &e, T &vrho, T &vsig) {
  if (kind == HQCGB_XC_PBE) {
    if (!(rho > T(1e-14))) { e = vrho = vsig = T(0); return; }
    Dual2<T> r(rho, T(1), T(0)), s(sigma, T(0), T(1));
    Dual2<T> out = e_pbe(r, s);
    e = out.v; vrho = out.a; vsig = out.b;
    return;
  }
  Dual2<T> r(rho, T(1), T(0));
  Dual2<T> eps = eps_x_lda(r);
  if (kind == HQCGB_XC_LDA_VWN) eps = eps + eps_vwn(r);
  else if (kind == HQCGB_XC_LDA_HL) eps = eps + eps_hl_family(r, T(21), T(0.045));
  else if (kind == HQCGB_XC_LDA_BH) eps = eps + eps_hl_family(r, T(30), T(0.0504));
  else if (kind == HQCGB_XC_LDA_GL) eps = eps + eps_hl_family(r, T(11.4), T(0.0666));
  Dual2<T> out = r * eps;
  e = out.v; vrho = out.a; vsig = T(0);
}

}  // namespace hqcgb
