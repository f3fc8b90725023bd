/* Stand-in for GSL integration (oracle build only).
 *
 * gsl_integration_qag is replaced by adaptive 20-point Gauss-Legendre
 * quadrature: an interval is accepted when its 20-point value and the sum of
 * its two halves' agree to 1e-14 relative (or 1e-300 absolute), else both
 * halves are refined, to a depth of 40.  The nodes and weights come from
 * Newton's iteration on the Legendre polynomial P_20.  For the smooth band
 * shapes the chain set-up integrates (constant, Lorentzian, piecewise linear)
 * this is accurate to rounding, as GSL's QAG is for them; it reports success
 * and the refinement estimate as the error.  gsl_integration_qawc (Cauchy
 * principal values, diagnostic only) still returns 0. */
#ifndef ORACLE_SHIM_GSL_INTEGRATION_H
#define ORACLE_SHIM_GSL_INTEGRATION_H
#include <math.h>
#include <stddef.h>
#include "gsl_errno.h"
typedef struct { double (*function)(double x, void* params); void* params; } gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
static inline gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n) {
  static gsl_integration_workspace w; w.limit = n; return &w; }
static inline void gsl_integration_workspace_free(gsl_integration_workspace* w) { (void)w; }

static inline void oracle_shim_gl20(double* x, double* w) {
  const int n = 20;
  const double pi = 3.141592653589793238462643383279502884197169;
  for (int i = 0; i < n / 2; ++i) {
    double z = cos(pi * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) { double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k; p0 = p1; p1 = p2; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-17) break;
    }
    x[i] = -z; x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

static inline double oracle_shim_gl_panel(const gsl_function* f, double a, double b, const double* x,
                                          const double* w) {
  double c = 0.5 * (a + b), h = 0.5 * (b - a), s = 0.0;
  for (int i = 0; i < 20; ++i) s += w[i] * (*f->function)(c + h * x[i], f->params);
  return s * h;
}

static inline double oracle_shim_adapt(const gsl_function* f, double a, double b, double whole, int depth,
                                       const double* x, const double* w, double* err) {
  double m = 0.5 * (a + b);
  double l = oracle_shim_gl_panel(f, a, m, x, w), r = oracle_shim_gl_panel(f, m, b, x, w);
  double d = fabs(l + r - whole);
  if (depth >= 40 || d <= 1e-14 * fabs(l + r) || d <= 1e-300) { *err += d; return l + r; }
  return oracle_shim_adapt(f, a, m, l, depth + 1, x, w, err) + oracle_shim_adapt(f, m, b, r, depth + 1, x, w, err);
}

static inline int gsl_integration_qag(const gsl_function* f, double a, double b, double epsabs,
    double epsrel, size_t limit, int key, gsl_integration_workspace* ws, double* result, double* abserr) {
  (void)epsabs;(void)epsrel;(void)limit;(void)key;(void)ws;
  static double x[20], w[20];
  static int ready = 0;
  if (!ready) { oracle_shim_gl20(x, w); ready = 1; }
  double err = 0.0;
  *result = (a == b) ? 0.0 : oracle_shim_adapt(f, a, b, oracle_shim_gl_panel(f, a, b, x, w), 0, x, w, &err);
  *abserr = err;
  return 0; }
static inline int gsl_integration_qawc(gsl_function* f, double a, double b, double c, double epsabs,
    double epsrel, size_t limit, gsl_integration_workspace* w, double* result, double* abserr) {
  (void)f;(void)a;(void)b;(void)c;(void)epsabs;(void)epsrel;(void)limit;(void)w;
  *result = 0.0; *abserr = 0.0; return 0; }
#endif
