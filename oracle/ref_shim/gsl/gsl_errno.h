/* Minimal stand-in for GSL error handling (oracle build only). */
#ifndef ORACLE_SHIM_GSL_ERRNO_H
#define ORACLE_SHIM_GSL_ERRNO_H
#define GSL_SUCCESS 0
#define GSL_EROUND 18
typedef void gsl_error_handler_t(const char*, const char*, int, int);
static inline gsl_error_handler_t* gsl_set_error_handler_off(void) { return 0; }
static inline gsl_error_handler_t* gsl_set_error_handler(gsl_error_handler_t* h) { (void)h; return 0; }
#endif
