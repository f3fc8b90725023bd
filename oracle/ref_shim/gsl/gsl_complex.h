/* Minimal stand-in for GSL complex numbers (oracle build only). */
#ifndef ORACLE_SHIM_GSL_COMPLEX_H
#define ORACLE_SHIM_GSL_COMPLEX_H
typedef struct { double dat[2]; } gsl_complex;
#define GSL_REAL(z) ((z).dat[0])
#define GSL_IMAG(z) ((z).dat[1])
#define GSL_SET_COMPLEX(zp, x, y) do { (zp)->dat[0] = (x); (zp)->dat[1] = (y); } while (0)
#endif
