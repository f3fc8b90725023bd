/* C interface of the CPU oracle (test infrastructure only; see nrg_oracle.cpp). */
#ifndef NRG_ORACLE_H
#define NRG_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_MODEL_1CHQS 0  /* one-channel Anderson, (Q,S) basis  */
#define ORACLE_MODEL_1CHQSZ 1 /* one-channel Anderson, (Q,Sz) basis */
#define ORACLE_MODEL_2CHQS 2  /* two-channel Anderson, (Q,S) basis  */
#define ORACLE_MODEL_1CHQ 3   /* one-channel Anderson, (Q) basis    */
#define ORACLE_MODEL_1CHS 4   /* one-channel Anderson, superconducting leads, (S) basis */
#define ORACLE_MODEL_1CHSZ 5  /* the same in the (Sz) basis with a field B (gamma2_or_B) */

typedef struct {
  int model;          /* ORACLE_MODEL_* */
  int nsites;         /* Wilson iterations N = 0 .. nsites-1 */
  int ncutoff;        /* kept multiplets (states in Q,Sz) */
  double lambda, U, ed, gamma1;
  double gamma2_or_B; /* Gamma2 for 2chQS, magnetic field B for 1chQSz */
  double degen_eps;   /* SetDegen tolerance, <=0 -> 1e-18 */
  int nthreads;       /* host threads over blocks / block pairs */
  int capture_iter;   /* iteration whose DiagHN inputs/H are kept, -1 none */
  int dm;             /* keep DM-NRG shells (UpdateBefCut = 1, c_d); 1chQS and 2chQS */
  int chain;          /* the free Wilson chain of calcdens = 3 (H_0 = first site, iterations 1..nsites-1) */
  double delta_sc;    /* gap of the superconducting leads (1chS, 1chSz) */
  const double* chain_chi; /* a Wilson chain other than the flat band's: chi_N, */
  const double* chain_en;  /* e_N for N < chain_len (0: the flat band's) */
  int chain_len;
  int chain_alambda;       /* sqrt(A_Lambda) on the impurity coupling */
} oracle_config;

/* DM-NRG parameters (DM_NRG command line, DM_NRG_CommandLineRead.cpp). */
typedef struct {
  double temp;        /* temperature in units of the half-bandwidth (> 0), or 0 for DM_NRG's choice */
  double betabar;     /* -b, default 0.727 */
  double bbroad;      /* -e, log-Gaussian width */
  double twindow;     /* -w, default 2 */
  double broadtemp;   /* -B, default 0.8 */
  double site_dim;    /* states per Wilson site in the FDM weights (4 in DM_NRG.cpp) */
  int nw;             /* -n, frequencies per shell for the default grid */
  int mtemp;          /* -M: T = D_Mtemp/betabar when Mtemp < nsites-1; -1 otherwise */
} oracle_dm_params;

int oracle_load_lapack(const char* path);
const char* oracle_last_error(void);
void oracle_blas_threads(int n);
double oracle_cgordan(double j1, double m1, double j2, double m2, double j, double m);
int oracle_diag_block(int n, const double* packed, double* w, double* Z);
void* oracle_run(const oracle_config* cfg);
void oracle_free(void* h);
/* Named arrays of the capture iteration (NULL and *len = -1 if absent). */
const double* oracle_cap_d(void* h, int n, const char* name, int* len);
const int* oracle_cap_i(void* h, int n, const char* name, int* len);
const double* oracle_dm_d(void* h, int N, const char* name, int* len);
const int* oracle_dm_i(void* h, int N, const char* name, int* len);
int oracle_dm_spectral(void* h, const oracle_dm_params* prm, const double* omegas, int nomega, double* omega_out,
                       double* a_out, int cap, double* rho_trace);

#ifdef __cplusplus
}
#endif
#endif
