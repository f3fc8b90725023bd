/* Minimal stand-in for GSL integration (oracle build only).  The reference
 * only integrates for diagnostic norms and non-flat band set-up, neither of
 * which is on the NRG iteration path; the routines return 0 with result 0. */
#ifndef ORACLE_SHIM_GSL_INTEGRATION_H
#define ORACLE_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
#include "gsl_errno.h"
typedef struct { double (*function)(double x, void* params); void* params; } gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
static inline gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n) {
  static gsl_integration_workspace w; w.limit = n; return &w; }
static inline void gsl_integration_workspace_free(gsl_integration_workspace* w) { (void)w; }
static inline int gsl_integration_qag(const gsl_function* f, double a, double b, double epsabs,
    double epsrel, size_t limit, int key, gsl_integration_workspace* w, double* result, double* abserr) {
  (void)f;(void)a;(void)b;(void)epsabs;(void)epsrel;(void)limit;(void)key;(void)w;
  *result = 0.0; *abserr = 0.0; return 0; }
static inline int gsl_integration_qawc(gsl_function* f, double a, double b, double c, double epsabs,
    double epsrel, size_t limit, gsl_integration_workspace* w, double* result, double* abserr) {
  (void)f;(void)a;(void)b;(void)c;(void)epsabs;(void)epsrel;(void)limit;(void)w;
  *result = 0.0; *abserr = 0.0; return 0; }
#endif
