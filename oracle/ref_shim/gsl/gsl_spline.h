/* Minimal stand-in for GSL linear interpolation (oracle build only). */
#ifndef ORACLE_SHIM_GSL_SPLINE_H
#define ORACLE_SHIM_GSL_SPLINE_H
#include <stddef.h>
typedef struct { int kind; } gsl_interp_type;
static const gsl_interp_type oracle_shim_linear = {1};
#define gsl_interp_linear (&oracle_shim_linear)
typedef struct { size_t cache; } gsl_interp_accel;
typedef struct { const double* x; const double* y; size_t n; } gsl_interp;
static inline gsl_interp_accel* gsl_interp_accel_alloc(void) { return new gsl_interp_accel(); }
static inline void gsl_interp_accel_free(gsl_interp_accel* a) { delete a; }
static inline gsl_interp* gsl_interp_alloc(const gsl_interp_type* t, size_t n) {
  (void)t; gsl_interp* p = new gsl_interp(); p->n = n; return p; }
static inline void gsl_interp_free(gsl_interp* p) { delete p; }
static inline int gsl_interp_init(gsl_interp* p, const double* x, const double* y, size_t n) {
  p->x = x; p->y = y; p->n = n; return 0; }
static inline double gsl_interp_eval(const gsl_interp* p, const double* x, const double* y,
                                     double xi, gsl_interp_accel* a) {
  (void)a; size_t n = p->n;
  if (n == 0) return 0.0;
  if (xi <= x[0]) return y[0];
  if (xi >= x[n - 1]) return y[n - 1];
  size_t lo = 0, hi = n - 1;
  while (hi - lo > 1) { size_t mid = (lo + hi) / 2; if (x[mid] > xi) hi = mid; else lo = mid; }
  double t = (xi - x[lo]) / (x[hi] - x[lo]);
  return y[lo] + t * (y[hi] - y[lo]);
}
#endif
