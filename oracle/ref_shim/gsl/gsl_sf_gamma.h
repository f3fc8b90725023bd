/* Minimal stand-in for the GSL special-function header, used only to compile
 * the reference TwoChNRG sources as a test oracle.  gsl_sf_fact(n) is n!
 * rounded once to double (the integer product is exact in 128 bits up to 33!),
 * which is what a table of correctly rounded factorials holds. */
#ifndef ORACLE_SHIM_GSL_SF_GAMMA_H
#define ORACLE_SHIM_GSL_SF_GAMMA_H
static inline double gsl_sf_fact(unsigned int n) {
  if (n > 33) { double f = 1.0; for (unsigned int k = 2; k <= n; ++k) f *= (double)k; return f; }
  unsigned __int128 p = 1;
  for (unsigned int k = 2; k <= n; ++k) p *= k;
  return (double)p;
}
static inline double gsl_sf_gamma(double x) { return __builtin_tgamma(x); }
#endif
