/* Minimal stand-in for GSL complex arithmetic (oracle build only). */
#ifndef ORACLE_SHIM_GSL_COMPLEX_MATH_H
#define ORACLE_SHIM_GSL_COMPLEX_MATH_H
#include "gsl_complex.h"
static inline gsl_complex gsl_complex_rect(double x, double y) { gsl_complex z; z.dat[0]=x; z.dat[1]=y; return z; }
static inline gsl_complex gsl_complex_add(gsl_complex a, gsl_complex b) { return gsl_complex_rect(a.dat[0]+b.dat[0], a.dat[1]+b.dat[1]); }
static inline gsl_complex gsl_complex_add_real(gsl_complex a, double x) { return gsl_complex_rect(a.dat[0]+x, a.dat[1]); }
static inline gsl_complex gsl_complex_mul(gsl_complex a, gsl_complex b) {
  return gsl_complex_rect(a.dat[0]*b.dat[0]-a.dat[1]*b.dat[1], a.dat[0]*b.dat[1]+a.dat[1]*b.dat[0]); }
static inline gsl_complex gsl_complex_mul_real(gsl_complex a, double x) { return gsl_complex_rect(a.dat[0]*x, a.dat[1]*x); }
static inline gsl_complex gsl_complex_mul_imag(gsl_complex a, double y) { return gsl_complex_rect(-a.dat[1]*y, a.dat[0]*y); }
static inline double gsl_complex_abs2(gsl_complex a) { return a.dat[0]*a.dat[0]+a.dat[1]*a.dat[1]; }
static inline gsl_complex gsl_complex_inverse(gsl_complex a) { double s = 1.0/gsl_complex_abs2(a); return gsl_complex_rect(a.dat[0]*s, -a.dat[1]*s); }
static inline gsl_complex gsl_complex_div(gsl_complex a, gsl_complex b) { return gsl_complex_mul(a, gsl_complex_inverse(b)); }
#endif
