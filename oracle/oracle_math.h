/*
 * oracle_math.h -- scalar arithmetic of the CPU oracle (test infrastructure).
 *
 * This is the oracle's own restatement of the reference's scalar helpers; the GPU
 * library has an independent copy (pgdg_p2_gb300/csrc/pgdg_math.cuh) and the
 * tests check the two against each other and against glibc.
 *
 * Build with -ffp-contract=off: every expression below is meant to be evaluated
 * in the written order with one rounding per operation.
 */
#ifndef PGDG_ORACLE_MATH_H
#define PGDG_ORACLE_MATH_H

#include <cmath>
#include <cstdint>

namespace oracle {

constexpr double PI_REF = 3.1415926;   /* glbparam.h:36 */
constexpr double CELL_RATIO = 3.2;     /* glbparam.h:31 */
constexpr double CUT_OFF = 2.;         /* glbparam.h:32 */

/* powern (glbfunc.h:28-40): repeated multiplication starting from 1 */
inline double powern(double a, int n) {
  double r = 1;
  for (int i = 0; i < n; i++) r *= a;
  return r;
}

/* Deterministic natural log to ~1e-17 relative, from frexp and the atanh series.
 * Only used to form the tiny correction x^(-eps) below, so its accuracy is ample. */
inline double det_log(double x) {
  int e;
  double m = std::frexp(x, &e);          /* x = m 2^e, m in [0.5,1) */
  if (m < 0.70710678118654752) { m = m * 2.0; e -= 1; }
  double t = (m - 1.0) / (m + 1.0);
  double t2 = t * t;
  double s = 0.0;
  for (int k = 23; k >= 3; k -= 2) s = (s + 1.0 / k) * t2;
  s = (s + 1.0) * t;
  return 2.0 * s + e * 0.69314718055994531;
}

/* The double nearest to x^(1/d) as the reference computes it with
 * pow(vol, 1./DIM) (mpm.cpp:1089,1399; particle.cpp:643; particle_flow.cpp:473).
 * For d == 2 the exponent 1./2 is exact, so this is sqrt(x).
 * For d == 3 the exponent is the double 1/3 - 1/(3*2^54); the result is
 * cbrt(x) * x^(-1/(3*2^54)), refined in double-double so that the final
 * rounding is (almost always) correct. */
inline double root_d(double x, int d) {
  if (d == 2) return std::sqrt(x);
  if (!(x > 0.0) || std::isinf(x)) return std::pow(x, 1.0 / 3.0);
  double y0 = std::cbrt(x);
  /* y0^3 in double-double */
  double p = y0 * y0;
  double pl = std::fma(y0, y0, -p);
  double q = p * y0;
  double ql = std::fma(p, y0, -q);
  ql = ql + pl * y0;
  double r = (q - x) + ql;                 /* q - x is exact (Sterbenz) */
  double delta = r / (3.0 * p);            /* Newton correction */
  /* y1 = y0 - delta (double-double); apply x^(-eps), eps = 1/(3*2^54) */
  double lx = det_log(x);
  double eps_l = lx * 1.8503717077085943e-17;   /* eps * ln x */
  double corr = y0 * eps_l;
  double small = (-delta) - corr;
  return y0 + small;
}

/* Wendland C4 kernel (particle.cpp:131-149, _WINDLAND_C4_) */
inline double kernel_w(double dist, double h, int d) {
  double C = (d == 2) ? 1.0 / PI_REF / powern(h, 2) * 7. / 4.
                      : 1.0 / PI_REF / powern(h, 3) * 21. / 16.;
  double s = dist / h;
  double val = 0.0;
  if (s < 2) val = C * powern((1. - 0.5 * s), 4) * (1. + 2. * s);
  return val;
}

/* dW/dr / r (particle.cpp:297-315) */
inline double kernel_dw(double dist, double h, int d) {
  double C = (d == 2) ? 1.0 / PI_REF / powern(h, 2) * 7. / 4.
                      : 1.0 / PI_REF / powern(h, 3) * 21. / 16.;
  double s = dist / h;
  double val = 0.0;
  if (s < 2) val = -5. * C * powern((1. - 0.5 * s), 3) * s / h / dist;
  return val;
}

/* EOS (mpm.cpp:859-876) */
inline double eos_p(double ee, double g, double pinf) { return ee * (g - 1) - g * pinf; }
inline double eos_rhoe(double p, double g, double pinf) { return (p + g * pinf) / (g - 1); }

inline double amax1(double a, double b) { return a >= b ? a : b; }
inline double amin1(double a, double b) { return a <= b ? a : b; }

/* Hugoniot helpers (glbfunc.h:314-337) */
inline double rhols_cal(double rhol, double pl, double ps, double g, double pinf) {
  double vn = (g + 1) * ps + (g - 1) * pl + 2 * g * pinf;
  double vd = (g - 1) * ps + (g + 1) * pl + 2 * g * pinf;
  return rhol * vn / vd;
}
inline double wl_cal(double rhol, double pl, double ps, double g, double pinf) {
  return std::sqrt(0.5 * rhol * ((g + 1.0) * ps + (g - 1.0) * pl + 2.0 * g * pinf));
}
inline double jaco_cal(double W, double pl, double rhol, double ps, double g, double pinf) {
  (void)pinf;
  return 1. / W - (ps - pl) / (W * W) * rhol * (g + 1) / 4. / W;
}

/* MGFM two-shock Newton solve.  variant 0: mpm.cpp:882-926; variant 1:
 * Triple_point_2phase/mpm.cpp:1373-1416.  Returns (rho*_L, p*, u*) and the
 * iteration count.  seed_p > 0 overrides the initial p* (surrogate seed). */
inline void mgfm(double ul, double ur, double pl, double pr, double rhol, double rhor,
                 double gl, double pinfl, double gr, double pinfr, int variant,
                 double seed_p, double out[3], int* iters) {
  double pstar;
  if (variant == 0) {
    pl = amax1(pl, 1e-10);
    pr = amax1(pr, 1e-10);
    rhol = amax1(rhol, 1e-10);
    rhor = amax1(rhor, 1e-10);
    pstar = amax1(pl, pr);
  } else {
    if (pl < 0) pl = 0;
    if (pr < 0) pr = 0;
    pstar = (pl + pr) * 0.5;
  }
  if (seed_p > 0) pstar = seed_p;
  double tol = amax1(1e-8, 1e-3 * std::fabs(ul - ur));
  double f1 = 1.;
  double rhols = 0, usl = 0, Wl = 0, Wr = 0;
  int nn = 0;
  do {
    Wl = wl_cal(rhol, pl, pstar, gl, pinfl);
    Wr = wl_cal(rhor, pr, pstar, gr, pinfr);
    if (variant == 0) usl = ul - (pstar - pl) / Wl;
    rhols = rhols_cal(rhol, pl, pstar, gl, pinfl);
    f1 = ul - ur - (pstar - pl) / Wl - (pstar - pr) / Wr;
    double jac = -jaco_cal(Wl, pl, rhol, pstar, gl, pinfl) - jaco_cal(Wr, pr, rhor, pstar, gr, pinfr);
    double dp = -f1 / jac;
    if (std::fabs(dp) > 0.6 * pstar) dp = std::copysign(0.6 * pstar, dp);
    pstar += dp;
    pstar = amax1(pstar, 1e-8);
    nn++;
  } while (std::fabs(f1) > tol && nn < 50);
  if (variant != 0) usl = ul - (pstar - pl) / Wl;
  out[0] = rhols;
  out[1] = pstar;
  out[2] = usl;
  if (iters) *iters = nn;
}

}  // namespace oracle
#endif
