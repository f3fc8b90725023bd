/*
 * twochnrg_gb300.h — C ABI of the GB300-native TwoChNRG iterative-
 * diagonalization engine.
 *
 * The engine replaces the hot path of the TwoChNRG NRG_main loop
 * (src/Main/NRG_main.cpp:282-427): block-Hamiltonian assembly and block
 * diagonalization (CNRGmatrix::DiagHN, src/DiagHN.cpp:6-119 and
 * src/NRGmatrixClass.cpp:566-696), truncation (CNRGarray::SetKept,
 * src/NRGarrayClass.cpp:461-491, and CutStates, src/CutStates.cpp:10-95),
 * operator rotation (UpdateMatrices, src/UpdateMatrices.cpp:272-568) and the
 * per-iteration observables (CalcSuscep/CalcEntropy, src/CalcThermo.cpp:16-121;
 * CalcOpAvg, src/CalcOpAvg.cpp:13-84).
 *
 * Data cross this boundary as plain host arrays laid out like the
 * reference's containers (include/NRGclasses.hpp:47-759):
 *   - blocks:      QNumbers[nblocks*nqn], BlockBegEnd[2*nblocks] (inclusive)
 *   - states:      dEn[nstates], iType[nstates], StCameFrom[nstates]
 *   - eigenvectors: dEigVec, per block a row-major (rows x cols) matrix whose
 *                  row k is eigenvector k
 *   - operators:   MatBlockMap[2*npairs], MatBlockBegEnd[2*npairs], MatEl
 *                  (dense row-major block per pair, block-pair order as the
 *                  reference produces it: ibl major, jbl minor).
 * Every call returns an nrg_status.  Nothing calls exit(); no call falls back
 * to the CPU: without a usable sm_103 device, nrg_create() fails with
 * NRG_ERR_CUDA.  Output arrays are owned by the context and stay valid until
 * the next call on the same context.  One context drives one CUDA stream;
 * distinct contexts may be used from distinct host threads.
 */
#ifndef TWOCHNRG_GB300_H
#define TWOCHNRG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  NRG_OK = 0,
  NRG_ERR_ARG = 1,          /* bad argument / unsupported model            */
  NRG_ERR_CUDA = 2,         /* CUDA runtime error or no usable device      */
  NRG_ERR_NOMEM = 3,        /* device or host allocation failed            */
  NRG_ERR_NOT_CONVERGED = 4,/* eigensolver iteration limit reached         */
  NRG_ERR_SIZE = 5,         /* a block exceeds the compiled size limits    */
  NRG_ERR_SYNC = 6,         /* block structures out of sync (ChkSync)      */
  NRG_ERR_TIMEOUT = 7,      /* a bounded device-side wait gave up          */
  NRG_ERR_STATE = 8         /* call order violated (e.g. no sweep loaded)  */
} nrg_status;

/* Model families (CNRGCodeHandler::ModelSwitch, src/CodeHandler_ModelSwitch.cpp). */
typedef enum {
  NRG_MODEL_1CH_QS = 0,  /* one-channel Anderson, |Q S> basis   (SymNo 0, ModelNo 0) */
  NRG_MODEL_1CH_QSZ = 1, /* one-channel Anderson, |Q Sz> basis  (SymNo 2, ModelNo 0) */
  NRG_MODEL_2CH_QS = 2,  /* two-channel Anderson, |Q S> basis   (SymNo 1)            */
  NRG_MODEL_1CH_Q = 3,   /* one-channel Anderson, |Q> basis     (SymNo 3, ModelNo 0);
                            whole sweeps only.  Blocks are reported as (Q, 0); the
                            averaged operators are S_z and S_z^2; the reference takes
                            only the entropy for this symmetry, and the T chi slot of
                            nrg_iteration.thermo is 0 */
  NRG_MODEL_1CH_S = 4,   /* one-channel Anderson with superconducting leads, |S> basis
                            (SymNo 7, ModelNo 0); whole sweeps only.  Blocks are reported
                            as (0, S); nrg_iteration.params[2] is the Delta_N of that
                            iteration; no free-chain run */
  NRG_MODEL_1CH_SZ = 5   /* the same with a Zeeman field, |Sz> basis (SymNo 8, ModelNo 0);
                            blocks (0, Sz); averaged operators n_d, S_z, S_z^2 (the
                            reference names them Ndot, NdSq, SdSq) */
} nrg_model;

/* Arithmetic of the dense steps. */
typedef enum {
  NRG_PREC_FP64 = 0,     /* plain FP64 everywhere */
  NRG_PREC_MIXED = 1     /* the largest blocks' Householder reduction (from 4200 states on;
                            NRG_MIXED_N overrides) blocked by panels of 32 columns, its
                            trailing rank-64 updates as split-BF16 products on the tensor
                            cores (6 slices, FP32 accumulation, FP64 recombination; error of
                            order 2^-36 of the operands' magnitudes); everything else FP64 */
} nrg_precision;

typedef struct nrg_ctx nrg_ctx;

/* Sweep parameters: the input_nrg.dat quantities NRG_main reads
 * (CNRGCodeHandler::ReadParams, src/NRGcodehandlerClass.cpp:104-149). */
typedef struct {
  int model;          /* nrg_model */
  int nsites;         /* Wilson iterations N = 0 .. nsites-1 */
  int ncutoff;        /* Ncutoff: kept multiplets (Q,S) or states (Q,Sz) */
  double lambda;      /* Lambda */
  double U, ed;       /* impurity interaction and level */
  double gamma1;      /* hybridization Gamma (channel 1) */
  double gamma2_or_B; /* Gamma2 for NRG_MODEL_2CH_QS, field B for NRG_MODEL_1CH_QSZ and
                         NRG_MODEL_1CH_SZ */
  double degen_eps;   /* CNRGarray::MyEPS (-E flag); <= 0 selects 1e-18 */
  int precision;      /* nrg_precision */
  double delta_sc;    /* gap of the superconducting leads, NRG_MODEL_1CH_S / NRG_MODEL_1CH_SZ
                         (input_nrg.dat model parameter 4, NRG_main.cpp:220-227); else ignored */
} nrg_sweep_config;

/* Per-iteration results of a sweep (what NRG_main prints / writes). */
typedef struct {
  int nblocks;             /* blocks of H_N */
  const double* qnumbers;  /* [nblocks*2] (Q,S) or (Q,Sz) */
  const int* block_size;   /* [nblocks] */
  int nstates;
  const double* en;        /* [nstates] rescaled energies after SetE0zero/SetDegen */
  double emin;             /* ground energy subtracted by SetE0zero */
  double ecut;             /* CNRGarray::Ecut(Ncutoff) */
  int nkept;               /* states with E <= Ecut */
  int nkept_blocks;
  const int* kept_block_size; /* [nkept_blocks] block sizes of AeigCut */
  const double* thermo;    /* [4*4]: (betabar_n, T_M, T chi (CalcSuscep), S (CalcEntropy)) */
  int nops;
  const double* opavg;     /* [nops] CalcOpAvg of the averaged operators at betabar */
  const double* params;    /* [4] ParamsHN used: Lambda, chi_1, chi_2 (0 if 1ch; Delta_N for
                              NRG_MODEL_1CH_S), eN */
  double wall_ms;          /* host wall time of the iteration (table building, copies, kernels) */
  double device_ms;        /* CUDA-event span of the iteration on the engine stream */
} nrg_iteration;

/* Phase timing of the last sweep (device time from CUDA events). */
typedef struct {
  double total_ms;        /* host wall time of nrg_sweep_run                   */
  double assemble_ms;     /* H_N assembly kernels                               */
  double tridiag_ms;      /* Householder tridiagonalization                     */
  double tridiag_eig_ms;  /* eigenvalues of the tridiagonals (bisection, sort)  */
  double backtransform_ms;/* eigenvector back-transformation                    */
  double cut_ms;          /* SetE0zero/SetDegen/Ecut/CutStates + observables    */
  double update_ms;       /* operator rotation (UpdateMatrices)                 */
  double tridiag_flops;   /* algorithmic FP64 flops of the tridiagonalization   */
  double update_flops;    /* algorithmic flops of the rotation GEMMs            */
  double backtransform_flops;
  int64_t kernel_launches;/* kernels launched by the sweep                      */
  int64_t tridiag_launches;
  double device_ms;       /* CUDA-event span of the sweep on the engine stream  */
  int64_t h2d_bytes;      /* host-to-device bytes copied by the sweep           */
  int64_t d2h_bytes;      /* device-to-host bytes copied by the sweep           */
  double dm_backprop_ms;  /* nrg_dm_backprop: rotations + partial traces        */
  double dm_spectral_ms;  /* nrg_lehmann: pair weights + Lehmann sums           */
  double lehmann_ms;      /* nrg_lehmann: the Lehmann-sum kernels alone         */
  int64_t lehmann_pairs;  /* Lehmann pairs whose term can be nonzero, all shells */
  int64_t lehmann_evals;  /* those pairs x the frequencies of their shell window */
  double vectors_ms;      /* inverse iteration + reorthogonalization            */
} nrg_timing;

/* ---- context ---------------------------------------------------------- */
nrg_status nrg_create(int device, nrg_ctx** out);
void nrg_destroy(nrg_ctx* ctx);
const char* nrg_last_error(const nrg_ctx* ctx);
const char* nrg_status_string(nrg_status s);
/* Number of kernels this library has launched on the context so far. */
int64_t nrg_kernel_count(const nrg_ctx* ctx);

/* ---- whole sweep (NRG_main main loop, src/Main/NRG_main.cpp:282-427) ----
 * Runs the Wilson chain from the impurity H_{-1} through nsites iterations
 * with all state (kept eigenvectors, operator blocks) resident in HBM. */
nrg_status nrg_sweep_run(nrg_ctx* ctx, const nrg_sweep_config* cfg);
int nrg_sweep_num_iterations(const nrg_ctx* ctx);
nrg_status nrg_sweep_iteration(const nrg_ctx* ctx, int n, nrg_iteration* out);
nrg_status nrg_sweep_opavg_initial(const nrg_ctx* ctx, int* nops, const double** vals);
nrg_status nrg_sweep_timing(const nrg_ctx* ctx, nrg_timing* out);

/* ---- batched independent sweeps ----------------------------------------
 * The reference's only batching is one process per parameter point
 * (src/Scripts/RunNRGcluster.perl:18-122).  nrg_sweep_batch runs `ninst`
 * independent sweeps on one GPU with `nworkers` host threads, each owning
 * its own context and CUDA stream, so the instances' launches overlap on the
 * device.  Per instance i and iteration n (n < cfgs[i].nsites, row stride
 * `max_sites`) it writes
 *   thermo[(i*max_sites + n)*16 .. +16]  as nrg_iteration.thermo,
 *   opavg [(i*max_sites + n)*4  .. +4]   CalcOpAvg values (unused slots 0),
 *   nkept [i*max_sites + n]              states with E <= Ecut.
 * *seconds receives the wall time of the whole batch.  Eight workers
 * measured best on a GB300 with 16 host cores; the workers' small blocks use
 * the cluster Householder kernel's two-CTAs-per-SM form. */
nrg_status nrg_sweep_batch(int device, int ninst, const nrg_sweep_config* cfgs, int nworkers, int max_sites,
                           double* thermo, double* opavg, int* nkept, double* seconds);

/* Measured FP64 FMA throughput of the device (TFLOP/s), from a register-only
 * DFMA loop over all SMs: the roofline denominator of the FP64 kernels. */
nrg_status nrg_fp64_peak(nrg_ctx* ctx, double* tflops);

/* FP64-accurate product on the tcgen05 tensor cores, the building block of
 * the mixed-precision form: C (m x n) += alpha * A (m x k) * B (n x k)^T, all
 * row-major FP64 DEVICE pointers with leading dimensions lda, ldb, ldc.  Each
 * row of A and B is cut into `slices` BF16 fixed-point slices of 8 bits under
 * a power-of-two row scale; the slice products accumulate in FP32 in tensor
 * memory, without rounding for the three leading levels, and are summed in
 * FP64.  The error is of order 2^-35 sqrt(k/64) |A_i| |B_j| per element with
 * slices = 5 and 2^-36 with 6 (|A_i|: largest magnitude in row i).  The
 * reference's dense products it stands for are the cblas_dgemm calls of
 * UpdateMatrices (src/UpdateMatrices.cpp:481-494) and the Householder
 * trailing updates inside dspev (src/NRGmatrixClass.cpp:645).  k <= 256,
 * 1 <= slices <= 6; returns after the product is complete. */
nrg_status nrg_gemm_f64_tensor(nrg_ctx* ctx, int m, int n, int k, double alpha, const double* A, int64_t lda,
                               const double* B, int64_t ldb, double* C, int64_t ldc, int slices);

/* ---- derivatives: a forward / backward pair ------------------------------
 * The reference has no derivative code; its CalcOpAvg averages of the
 * operators dH/dp (n_d for eps_d, (n_d^2 - n_d)/2 for U, -S_z for B;
 * src/CalcOpAvg.cpp:13-84, CodeHandler_ModelSwitch.cpp:748-780) are the
 * Hellmann-Feynman values these derivatives meet for the ground-state energy.
 *
 * nrg_grad_forward runs the sweep of cfg (NRG_MODEL_1CH_QS or
 * NRG_MODEL_1CH_QSZ, FP64) and, at its kept-state set, the derivatives of
 * every iteration's reported values with respect to p = (eps_d, U, Gamma1,
 * B) (B is cfg->gamma2_or_B).  They come from tangents carried through each
 * step on the device: the assembly of dH_N from the previous tangents, the
 * eigenvalue and kept-eigenvector derivatives from first-order perturbation
 * theory with every eigenvector of the block (no coupling between levels
 * closer than 1e-10 of the block's scale: inside a degenerate multiplet the
 * eigenvectors are not determined and do not couple), the operator rotation
 * differentiated, and the thermodynamic and average sums differentiated.
 * Forward tangents carry the four directions beside the primal iteration by
 * iteration, so no eigenvectors are stored between iterations (nothing to
 * checkpoint).  The iterations stay readable with nrg_sweep_iteration. */
typedef struct {
  int nsites;              /* iterations */
  int nparams;             /* 4: eps_d, U, Gamma1, B */
  int nops;                /* averaged operators, as nrg_iteration.opavg */
  const double* d_thermo;  /* [(n*nparams + k)*16 + v]: d thermo[v] of iteration n / d p_k */
  const double* d_opavg;   /* [(n*nparams + k)*nops + o] */
  const double* d_emin;    /* [n*nparams + k]: d emin (the raw lowest level) / d p_k */
  const double* egs;       /* [n] absolute ground-state energy sum_{M<=n} D_M emin_M */
  const double* d_egs;     /* [n*nparams + k] */
} nrg_grad;
nrg_status nrg_grad_forward(nrg_ctx* ctx, const nrg_sweep_config* cfg, nrg_grad* out);

/* Vector-Jacobian product of the last nrg_grad_forward: grad[k] =
 * sum over iterations n of g_thermo[n*16+v] d thermo[v]/dp_k + g_opavg[n*nops+o]
 * d opavg[o]/dp_k + g_egs[n] d egs/dp_k; any of the three weight arrays may
 * be NULL.  NRG_ERR_STATE without a preceding forward. */
nrg_status nrg_grad_backward(nrg_ctx* ctx, const double* g_thermo, const double* g_opavg, const double* g_egs,
                             double* grad);

/* Arithmetic (nrg_precision) of the drop-in calls nrg_diag_blocks and
 * nrg_diag_hn on this context; a sweep sets it from its configuration. */
nrg_status nrg_set_precision(nrg_ctx* ctx, int precision);

/* ---- drop-in replacements --------------------------------------------- */

/* CNRGmatrix::DiagBlock replacement for a batch of blocks
 * (src/NRGmatrixClass.cpp:566-696, dspev_ at :645).  Block b (size
 * sizes[b]) is given as the reference hands it to dspev: its upper triangle
 * packed row by row (element (i,j), j >= i, at i*n - i*(i-1)/2 + (j-i),
 * ij2rUpTr src/ij2r.cpp:63-68), blocks concatenated.  On return eigvals
 * holds each block's eigenvalues in ascending order (concatenated) and
 * eigvecs each block's n x n eigenvector matrix, row k = eigenvector k
 * (concatenated), exactly the dEn / dEigVec layout DiagBlock appends.
 * All blocks are diagonalized in one batched launch series. */
nrg_status nrg_diag_blocks(nrg_ctx* ctx, int nblocks, const int* sizes, const double* packed_upper,
                           double* eigvals, double* eigvecs);

/* ---- per-step drop-ins for the NRG_main call sites ----------------------
 * Block structure of a CNRGarray (include/NRGclasses.hpp:47-200).  All
 * models here carry two quantum numbers per block: (Q,S) for the |Q S>
 * models, (Q,Sz) for NRG_MODEL_1CH_QSZ.  States are numbered from 0 and the
 * blocks tile them in order. */
typedef struct {
  int nblocks;
  int nqn;                       /* must be 2 */
  const double* qnumbers;        /* [nblocks*nqn] QNumbers */
  const int* block_beg_end;      /* [2*nblocks] BlockBegEnd: first, last state (inclusive) */
} nrg_blocks;

/* CNRGbasisarray as BuildBasis leaves it (src/BuildBasis.cpp:8-432). */
typedef struct {
  nrg_blocks blocks;
  const int* itype;              /* [nstates] iType: single-site state type */
  const int* st_came_from;       /* [nstates] StCameFrom: state of the previous AeigCut */
  const double* en;              /* [nstates] dEn: energy of that previous kept state */
} nrg_basis;

/* One real operator, CNRGmatrix (include/NRGclasses.hpp:365-434): dense
 * row-major (size_i x size_j) blocks for the listed block pairs, in the block
 * structure the operator is synced with. */
typedef struct {
  int nmatblocks;
  const int* mat_block_map;      /* [2*nmatblocks] MatBlockMap: (iblock, jblock) */
  const int* mat_block_beg_end;  /* [2*nmatblocks] MatBlockBegEnd: first, last index in mat_el */
  const double* mat_el;          /* MatEl */
} nrg_matrix;

/* AeigCut as CutStates leaves it (src/CutStates.cpp:10-95, CNRGbasisarray). */
typedef struct {
  nrg_blocks blocks;               /* kept blocks; BlockBegEnd over the kept states */
  const int* block_beg_end_bc;     /* [2*nblocks] BlockBegEndBC: the block's state range before the cut */
  const int* block_beg_end_eigvec; /* [2*nblocks] BlockBegEndEigVec: range of its rows in eigvec */
  const int* st_came_from;         /* [nstates] StCameFrom: state of the uncut array */
  const double* en;                /* [nstates] dEn */
  const unsigned char* kept;       /* [nstates] Kept */
  const double* eigvec;            /* dEigVec: per block, kept rows x n_BC, row-major */
} nrg_eigcut;

/* Result of nrg_cut_states; all arrays are owned by the context. */
typedef struct {
  const double* en;              /* [nstates] Aeig.dEn after SetKept (SetDegen applied) */
  const unsigned char* kept;     /* [nstates] Aeig.Kept */
  int nkept;                     /* states with E <= Ecut */
  double ecut;                   /* CNRGarray::Ecut(Ncutoff) */
  nrg_eigcut cut;                /* AeigCut (cut.eigvec NULL when no eigvec was given) */
} nrg_cut_result;

/* Operators, in this order, that nrg_diag_hn and nrg_update_ops take and
 * return (the NRGMats of CNRGCodeHandler::ModelSwitch,
 * src/CodeHandler_ModelSwitch.cpp:136-157, 748-780):
 *   NRG_MODEL_1CH_QS : f_N, n_d, n_d^2, S_d^2
 *   NRG_MODEL_1CH_QSZ: f_N,up, f_N,dn, n_d, S_z
 *   NRG_MODEL_2CH_QS : f_N,ch1, f_N,ch2, n_d, n_d^2, S_d^2
 * The f operators (the first one, or two) enter H_N; n_d, n_d^2, S_d^2 and S_z
 * are the impurity operators CalcOpAvg averages. */

/* CNRGmatrix::DiagHN (src/DiagHN.cpp:6-119, declared include/NRGclasses.hpp:642-646),
 * including its closing SetE0zero (DiagHN.cpp:116, src/NRGarrayClass.cpp:234-241);
 * called by NRG_main at src/Main/NRG_main.cpp:313.
 *   params_hn  ParamsHN as NRG_main builds it (NRG_main.cpp:264-276):
 *              Lambda, chi_1 [, chi_2], e_N, Delta_SC; nparams >= nchannels + 2,
 *              Delta_SC (if given) must be 0
 *   old_kept   block structure of the previous AeigCut (the operators' sync)
 *   ops        the model's operators (order above) in that structure; the
 *              f operators are read
 *   abasis     the basis BuildBasis made from old_kept; a basis that does not
 *              match BuildBasis's layout returns NRG_ERR_SYNC
 * Outputs (caller-owned): en[nstates] each block's eigenvalues ascending,
 * E_min subtracted; eigvec, per block its n x n eigenvector matrix (row k =
 * eigenvector k), blocks concatenated (sum of n_b^2); *emin the subtracted
 * ground energy.  H_N is assembled and diagonalized on the device. */
nrg_status nrg_diag_hn(nrg_ctx* ctx, int model, const double* params_hn, int nparams, const nrg_blocks* old_kept,
                       int nops, const nrg_matrix* ops, const nrg_basis* abasis, double* en, double* eigvec,
                       double* emin);

/* CNRGarray::SetKept (src/NRGarrayClass.cpp:461-491: SetDegen and Ecut)
 * then CutStates (src/CutStates.cpp:10-95) on Aeig as DiagHN leaves it.
 *   aeig, en    block structure and dEn of Aeig (E_min-shifted: min(en) == 0,
 *               else NRG_ERR_ARG)
 *   eigvec      Aeig.dEigVec (per block n x n, row = eigenvector) or NULL
 *   ncutoff     Ncutoff; degen_eps MyEPS (<= 0 selects 1e-18)
 * Kept flags, Nkept, BlockBegEnd, BlockBegEndBC, BlockBegEndEigVec and
 * StCameFrom equal the reference's; `out` points into context storage. */
nrg_status nrg_cut_states(nrg_ctx* ctx, const nrg_blocks* aeig, const double* en, const double* eigvec,
                          int ncutoff, double degen_eps, nrg_cut_result* out);

/* UpdateMatrices (src/UpdateMatrices.cpp:272-568) for all of the model's
 * operators: O_new(i,j) = Z_i F Z_j^T for every pair of kept blocks allowed
 * by CheckForMatEl, F from the single-site rules (times the old operator for
 * the impurity operators).
 *   old_kept  block structure the old operators are synced with
 *   abasis    the basis BuildBasis made from old_kept (NRG_ERR_SYNC otherwise)
 *   acut      AeigCut of this iteration (blocks, eigvec, block_beg_end_eigvec
 *             are read; kept blocks are matched to abasis blocks by their
 *             quantum numbers, FindMatchBlock src/FindMatchBlock.cpp:5-24)
 *   old_ops   [nops] the model's operators (order above), nops = the model's count
 * new_ops[o] receives MatBlockMap/MatBlockBegEnd/MatEl in the reference's
 * block-pair order (iblock major, jblock minor), pointing into context
 * storage. */
nrg_status nrg_update_ops(nrg_ctx* ctx, int model, const nrg_blocks* old_kept, const nrg_basis* abasis,
                          const nrg_eigcut* acut, int nops, const nrg_matrix* old_ops, nrg_matrix* new_ops);

/* ---- DM-NRG spectral function (src/DM_NRG/DM_NRG.cpp) --------------------
 * Parameters of DM_NRG's command line (DM_NRG_CommandLineRead.cpp). */
typedef struct {
  double temp;        /* T in units of the half-bandwidth; <= 0: DM_NRG's own
                         choice, D_{nsites+199}/betabar (or see mtemp) */
  int mtemp;          /* -M: T = D_Mtemp/betabar when 0 <= mtemp < nsites-1 (else -1) */
  double betabar;     /* -b, 0.727 */
  double bbroad;      /* -e, log-Gaussian width b */
  double twindow;     /* -w, 2: |E_j - E_i| < twindow T/D_N uses the Gaussian */
  double broadtemp;   /* -B, 0.8: width of that Gaussian */
  double site_dim;    /* states per Wilson site in the FDM weights (4, DM_NRG.cpp:292; 16 for two channels) */
  int nw;             /* -n, frequencies per shell of the default grid */
} nrg_dm_params;

/* NRG_main with the spectral density of the impurity d operator switched on
 * (input_nrg.dat calc_density = 1, UpdateBefCut = 1; NRG_main.cpp:334-396):
 * the sweep of nrg_sweep_run, but the operators f_N and c_d are rotated into
 * every shell's full eigenbasis, and each shell's energies, Kept flags,
 * eigenvectors, basis and c_d stay on the device (what SaveArrays writes,
 * NRGcodehandlerClass.cpp:887-932).  NRG_MODEL_1CH_QS, and NRG_MODEL_2CH_QS
 * (operators f_N1, f_N2 and c_d; the reference has no two-channel c_d rule
 * and its DM_NRG is one-channel only, so the two-channel shells take the
 * one-channel recoupling of c_d across the 16-state site and site_dim = 16
 * in nrg_dm_params; they cannot be written as .bin snapshots). */
nrg_status nrg_sweep_run_dm(nrg_ctx* ctx, const nrg_sweep_config* cfg);
int nrg_dm_num_shells(const nrg_ctx* ctx);

/* The FDM density-matrix backward sweep of DM_NRG (DM_NRG.cpp:195-383):
 * partition sums, DM_NRG_SetRhoNmax (DM_NRG_SetRhoNmax.cpp:9-126), then shell
 * by shell RotateMatrix (RotateMatrix.cpp:17-99) and DM_NRG_CalcRhoN_withSU2
 * (DM_NRG_CalcRhoN.cpp:252-449).  rho_trace (optional, [nshells]) receives
 * sum_b (2S_b+1) Tr rho_N(b) per shell. */
nrg_status nrg_dm_backprop(nrg_ctx* ctx, const nrg_dm_params* prm, double* rho_trace);

/* The c_d spectral function after nrg_dm_backprop (same parameters):
 * CalcSpecDM_NRG (SpecFuncClass.cpp:1827-1883) over FDM_SpecDens_M_STL
 * (SpecFunc_allSTL.cpp:1253-2358) and, for the last shell, CalcSpecCosti_T_N
 * (SpecFuncClass.cpp:417-650).  With omegas != NULL the nomega given
 * frequencies are used; with omegas == NULL the grid of CalcSpec_ManyOmegas
 * (SpecFuncClass.cpp:2238-2341, prm->nw points per shell), which must fit in
 * nomega.  Writes Omega_Rhow: omega_rhow[k] = omega_k and
 * omega_rhow[nomega + k] = A(omega_k) for k < *nout. */
nrg_status nrg_lehmann(nrg_ctx* ctx, const nrg_dm_params* prm, int nomega, const double* omegas, double* omega_rhow,
                       int* nout);

/* ---- derivatives of A(omega) ---------------------------------------------
 * The reference has no derivative code (see nrg_grad_forward).
 * nrg_grad_forward_dm runs the sweep of nrg_sweep_run_dm (NRG_MODEL_1CH_QS,
 * FP64) with the tangent pass of nrg_grad_forward (out as there).  Each
 * shell keeps, per parameter p = (eps_d, U, Gamma1, B), the tangents of its
 * energies, of every eigenvector (all states, as the DM-NRG rotations and
 * c_d use them all; no coupling inside a degenerate level) and of c_d.
 * nrg_dm_backprop on those shells also carries the four tangents of the
 * density matrices: d rho~ = Z^T (d rho Z + rho dZ) + dZ^T rho Z, the same
 * partial trace, and the Boltzmann weights differentiated with d ln ZTot.
 * nrg_lehmann_grad then returns what nrg_lehmann returns and d_rhow[k *
 * nomega + j] = d A(omega_j) / d p_k (k < 4; d_rhow holds 4 * nomega), from
 * d(rho A) = d rho A + rho dA, d(A rho) = dA rho + A d rho, the records'
 * weight and energy tangents and the broadening kernels differentiated.
 * These are the derivatives at the forward sweep's kept-state set and at the
 * undisplaced parameters' choice between the log-Gaussian and the Gaussian
 * kernel for every pair.  B does not enter the |Q S> model: its row is 0.
 * nrg_lehmann_grad_backward: grad[k] = sum_j g_rhow[j] d A(omega_j) / d p_k
 * over the *nout frequencies of the last nrg_lehmann_grad. */
nrg_status nrg_grad_forward_dm(nrg_ctx* ctx, const nrg_sweep_config* cfg, nrg_grad* out);
nrg_status nrg_lehmann_grad(nrg_ctx* ctx, const nrg_dm_params* prm, int nomega, const double* omegas,
                            double* omega_rhow, double* d_rhow, int* nout);
nrg_status nrg_lehmann_grad_backward(nrg_ctx* ctx, const double* g_rhow, double* grad);

/* ---- model plug-in -----------------------------------------------------
 * A model supplied by the caller, without rebuilding the engine: the
 * reference's per-model function pointers of CNRGmatrix (CalcHNMatEl,
 * CalcMatEl, CheckForMatEl; include/NRGclasses.hpp:612-634, assigned per
 * model in src/CodeHandler_ModelSwitch.cpp:131-640), its SetSingleSite and
 * its H_{-1} set-up, as tables and callbacks.  The engine calls the
 * callbacks on the host while it builds each iteration's tables (once per
 * distinct argument set; results are cached for the sweep) and assembles
 * H_N and updates the operators on the device from those tables.
 *
 * H_N element between new states i (site type t_i, from old state a_i) and j
 * (t_j, a_j), i < j, with O_o the old operators entering H_N and
 * c(o, dir) = hn_coef(user, S, t_i, t_j, channel, sigma, dir) for the block's
 * second quantum number S (the rule is taken for (t_i, t_j) and read as
 * O(a_i, a_j), dir 0, or -- when that element is below 1e-20 in magnitude --
 * as O(a_j, a_i), dir 1, as the reference's HN rules do):
 *   NRG_HN_ONE_OP      (chi_1 O_0) c(0)                         one operator
 *   NRG_HN_SPIN_SUM    (sum_{s=0,1} c(s) O_s) chi_1             O_0, O_1 (channel 0, sigma s)
 *   NRG_HN_CHANNEL_SUM sum_{ch=0,1} [(chi_ch O_ch) c(ch,0) + (chi_ch O_ch) c(ch,1)]
 * with IEEE products and sums in that order (the reference's evaluation
 * orders of OneChQS_HN_MatEl, OneChQSz_HN_MatEl and TwoChQS_HN_MatEl).  The
 * diagonal is sqrt(Lambda) E_old(a_i), plus e_N (Q_site(t_i) + 1) with
 * `onsite`.
 *
 * Operators (the first hn_ops -- 1 for NRG_HN_ONE_OP, else 2 -- enter H_N):
 *   NRG_OP_SITE           acts on the new site (f_N): F(i, j) = op_factor(user,
 *                         o, S_i, S_j, t_i, t_j) between states of the same old state
 *   NRG_OP_IMPURITY       an old operator recoupled across the site (c_d):
 *                         F(i, j) = op_factor(...) O_old(a_i, a_j)
 *   NRG_OP_IMPURITY_DIAG  an old operator times the site identity (n_d, S_z):
 *                         F(i, j) = [t_i == t_j] O_old(a_i, a_j); op_factor is not called
 * and the new O(i, j) blocks are kept only for block pairs with
 * op_check(user, o, qn_i, qn_j) != 0 (qn: the two quantum numbers of each
 * kept block).  op_avg[o] = 1 reports <O_o> per iteration (CalcOpAvg).
 *
 * Site basis: site_nblocks blocks of site_bsize states with site_nqn
 * quantum numbers: (Q, S, S_z) with total_spin (SU(2) multiplets; BuildBasis
 * couples S_old and S_site by the triangle rule), else (Q, S_z) added.
 * Types t are the site states in block order.
 *
 * H_{-1}: start_nblocks kept blocks (Q, S or S_z), their sizes and levels
 * (in units of Lambda (1 + 1/Lambda)/2, as the reference's *_SetAnderson_Hm1
 * leave them), and per operator start_npairs[o] block pairs
 * (start_pairs: bi, bj per pair, all operators concatenated) with their
 * dense row-major blocks concatenated in start_el.
 *
 * nrg_sweep_run_model runs the sweep of nrg_sweep_run with this model
 * (cfg->model is ignored; gamma1 and, with two channels, gamma2_or_B give
 * chi_{-1}); results through nrg_sweep_iteration.  The superconducting-lead
 * pairing term, DM-NRG shells, the free chain and derivatives are available
 * for the built-in models only.  A callback returning a non-finite value, a
 * malformed description or a basis with no states returns NRG_ERR_ARG. */
typedef double (*nrg_hn_coef_fn)(void* user, double s_block, int ti, int tj, int channel, int sigma, int dir);
typedef double (*nrg_op_factor_fn)(void* user, int op, double s_i, double s_j, int ti, int tj);
typedef int (*nrg_op_check_fn)(void* user, int op, const double* qn_i, const double* qn_j);

enum { NRG_HN_ONE_OP = 0, NRG_HN_SPIN_SUM = 1, NRG_HN_CHANNEL_SUM = 2 };
enum { NRG_OP_SITE = 0, NRG_OP_IMPURITY = 1, NRG_OP_IMPURITY_DIAG = 2 };

typedef struct {
  int total_spin;
  int site_nqn;              /* 3 with total_spin (Q, S, S_z), else 2 (Q, S_z) */
  int site_nblocks;
  const double* site_qn;     /* [site_nblocks * site_nqn] */
  const int* site_bsize;     /* [site_nblocks] */
  int hn_form;               /* NRG_HN_* */
  int onsite;                /* 1: the diagonal adds e_N (Q_site + 1) */
  nrg_hn_coef_fn hn_coef;
  int nops;                  /* 1 .. 8 */
  const int* op_class;       /* [nops] NRG_OP_* */
  const int* op_avg;         /* [nops] 1: <O> reported */
  nrg_op_factor_fn op_factor;
  nrg_op_check_fn op_check;
  int start_nblocks;
  const double* start_qn;    /* [2 * start_nblocks] */
  const int* start_bsize;    /* [start_nblocks] */
  const double* start_en;    /* [sum of start_bsize] */
  const int* start_npairs;   /* [nops] */
  const int* start_pairs;    /* [2 * sum of start_npairs] */
  const double* start_el;    /* the pairs' blocks */
  void* user;                /* passed to every callback */
} nrg_model_desc;

nrg_status nrg_sweep_run_model(nrg_ctx* ctx, const nrg_sweep_config* cfg, const nrg_model_desc* model);

/* nrg_diag_hn and nrg_update_ops (below) for a described model: the per-call-
 * site drop-ins of DiagHN and UpdateMatrices, where the reference calls
 * CalcHNMatEl, CalcMatEl and CheckForMatEl.  params_hn as for nrg_diag_hn
 * (one chi per channel of the description); ops / old_ops hold the
 * description's operators in its order (the first hn_ops enter H_N). */
nrg_status nrg_diag_hn_model(nrg_ctx* ctx, const nrg_model_desc* model, const double* params_hn, int nparams,
                             const nrg_blocks* old_kept, int nops, const nrg_matrix* ops, const nrg_basis* abasis,
                             double* en, double* eigvec, double* emin);
nrg_status nrg_update_ops_model(nrg_ctx* ctx, const nrg_model_desc* model, const nrg_blocks* old_kept,
                                const nrg_basis* abasis, const nrg_eigcut* acut, int nops, const nrg_matrix* old_ops,
                                nrg_matrix* new_ops);

/* The tables the device assembly and operator update read, built on the host
 * (no device needed) for a built-in model (desc NULL, model = nrg_model) or
 * a described one (desc non-NULL, model ignored):
 *   nrg_model_hn_table  coefficient table of a block of second quantum
 *                       number s_block: entry ((ti ntypes + tj) nchan nsigma +
 *                       channel nsigma + sigma) 2 + dir; *n receives its length
 *                       (ntypes^2 nchan nsigma 2), written when cap >= *n
 *   nrg_model_op_factor site factor of operator op (F between site types ti,
 *                       tj in blocks of spin s_i, s_j); 1/0 for n_d-like operators
 *   nrg_model_op_check  CheckForMatEl of operator op between kept blocks of
 *                       quantum numbers qn_i, qn_j (two each); *out 0 or 1 */
nrg_status nrg_model_hn_table(int model, const nrg_model_desc* desc, double s_block, double* coef, int cap, int* n);
nrg_status nrg_model_op_factor(int model, const nrg_model_desc* desc, int op, double s_i, double s_j, int ti, int tj,
                               double* out);
nrg_status nrg_model_op_check(int model, const nrg_model_desc* desc, int op, const double* qn_i,
                              const double* qn_j, int* out);

/* Clebsch-Gordan coefficient <j1 m1; j2 m2 | j m> (the reference's CGordan,
 * src/CGordan.cpp:34-120), for plug-in rules; 0 outside the triangle. */
double nrg_clebsch(double j1, double m1, double j2, double m2, double j, double m);

/* ---- thermodynamics with the free-chain subtraction --------------------
 * The reference computes the impurity T chi and S in two NRG_main runs
 * (calcdens = 3, then 2): the free Wilson chain first, written to
 * SuscepChain*.dat / EntropyChain*.dat, then the impurity sweep, which reads
 * those files back (CNRGthermo::ReadNChainValue, NRGthermoClass.cpp:66-103)
 * and writes T, value, chain value, value - chain
 * (CNRGthermo::SaveNValue, NRGthermoClass.cpp:109-150).
 *
 * nrg_sweep_run_chain: the calcdens = 3 sweep (ModelNo 3,
 * CodeHandler_ModelSwitch.cpp:377-420, 667-720, 940-1000).  H_0 is the first
 * Wilson site alone (iteration 0, thermodynamics at D_0 as NRG_main.cpp:242-255
 * takes them); iterations 1 .. nsites-1 add one site each.  U, ed, gamma1 and
 * gamma2_or_B are ignored (ZeroParams).  For NRG_MODEL_1CH_Q, which has no
 * chain case in ModelSwitch, NRG_main.cpp:215-218 runs the Anderson model with
 * every parameter zeroed instead: a decoupled impurity beside the chain,
 * iterations 0 .. nsites-1, its ln 4 of entropy subtracted by nrg_thermo_run
 * (dImpValue, CodeHandler_ModelSwitch.cpp:1191).  Results through
 * nrg_sweep_iteration. */
nrg_status nrg_sweep_run_chain(nrg_ctx* ctx, const nrg_sweep_config* cfg);

typedef struct {
  int nvalues;                 /* 4*nsites: value k = 4N + nc - 1, N the iteration, nc = 1..4 */
  const double* temp;          /* [nvalues] T_M = D_N / betabar_nc (both sweeps agree bit for bit) */
  const double* suscep;        /* T chi (CalcSuscep) of the impurity sweep */
  const double* suscep_chain;  /* T chi of the free chain */
  const double* suscep_imp;    /* suscep - suscep_chain */
  const double* entropy;       /* S (CalcEntropy) of the impurity sweep */
  const double* entropy_chain;
  const double* entropy_imp;
  int chain_reused;            /* 1: the chain values came from an earlier call */
  double chain_ms, imp_ms, total_ms; /* host wall times of the chain sweep, the impurity sweep, the call */
} nrg_thermo;

/* Both sweeps for one parameter set: the chain sweep runs on a second
 * context (own stream, own host thread) beside the impurity sweep on `ctx`.
 * With reuse_chain != 0 and the chain parameters (model, nsites, ncutoff,
 * lambda, degen_eps, precision) equal to the last call's, the stored chain
 * values are used instead, as the reference reuses its chain files.  The
 * impurity sweep's iterations stay readable with nrg_sweep_iteration.
 * Returns NRG_ERR_SYNC if the two sweeps' temperatures differ. */
nrg_status nrg_thermo_run(nrg_ctx* ctx, const nrg_sweep_config* cfg, int reuse_chain, nrg_thermo* out);

/* One thermodynamics file in the layout of CNRGthermo::SaveNValue: per line
 * T value chain value-chain, each "%.20e" (ofstream precision 20,
 * scientific).  chain == NULL writes a chain file (third column 0).  Needs
 * no device. */
nrg_status nrg_write_thermo(const char* path, int nvalues, const double* temp, const double* value,
                            const double* chain);

/* ---- Wilson chains of non-flat bands ------------------------------------
 * The sweep's chain is Wilson's analytic one for the flat band
 * (CNRGchain::SetChainWilson, NRGchainClass.cpp:132-155) unless the caller
 * sets another: hoppings chi[N] (CNRGchain::GetChin(N), the hopping from site
 * N to N+1) and on-site energies en[N] (GetEn(N)), N = 0 .. n-1, in the
 * rescaled units NRG_main uses.  Iteration N then uses chi[N-1] (the
 * impurity coupling at N = 0) and e_N = en[N]; the free-chain run starts
 * from chi[0].  apply_alambda = 0 leaves the impurity coupling without the
 * sqrt(A_Lambda) factor, as NRG_main does for the Campo-Oliveira scheme
 * (NRG_main.cpp:204-207).  n = 0 restores the Wilson chain.  A sweep needs
 * n >= nsites.  The two-channel model uses chi for both channels and has no
 * e_N term (TwoChQS_HN_MatEl). */
nrg_status nrg_set_chain(nrg_ctx* ctx, int n, const double* chi, const double* en, int apply_alambda);

/* Band types of CNRGCodeHandler::SetChain (NRGcodehandlerClass.cpp:202-400)
 * with their hybridization functions (HybFuncDefs.cpp). */
enum {
  NRG_BAND_CONST = 0,      /* -b Const: Gamma(w) = params[0] (1 without params) */
  NRG_BAND_LORENTZIAN = 1, /* -b SideDot: the six lanc.in values; Gamma(w) =
                              params[4]^2 params[2] / ((w - params[1])^2 + params[2]^2) */
  NRG_BAND_TABLE = 2       /* -b FromFile: (omega, Gamma(omega)) pairs, ascending
                              omega, linear in between (HybFunc_FromFile) */
};
typedef struct {
  int kind;                /* NRG_BAND_* */
  int nparams;
  const double* params;
  double lambda;
  double z;                /* z-trick twist (1: none) */
  int disc_scheme;         /* 0 usual, 1 Campo-Oliveira (not for NRG_BAND_LORENTZIAN) */
  double band_offset;      /* the band is [-(1+offset), 1-offset] (ChemPot) */
} nrg_band;

/* The chain of a band by the reference's Lanczos procedure
 * (CNRGchain::SetChainLanczos, NRGchainClass.cpp:234-520, with CalcF2 and
 * CalcFabmEabm): chi[0..nsites), en[0..nsites) and Fsq = int Gamma / Gamma_ref.
 * The discretization keeps ceil(nsites/2) intervals per side, so the last
 * coefficients carry its truncation; NRG_main asks for max(Nsitesmax, 100)
 * sites (NRGcodehandlerClass.cpp:219).  Host code, no device. */
nrg_status nrg_chain_lanczos(const nrg_band* band, int nsites, double* chi, double* en, double* fsq);

/* ---- .bin snapshots in the reference's layout ---------------------------
 * One DM-NRG shell as NRG_main saves it with UpdateBefCut = 1
 * (CNRGCodeHandler::SaveArrays, NRGcodehandlerClass.cpp:887-932). */
typedef struct {
  int nshell;                    /* N */
  nrg_basis basis;               /* Abasis_N: blocks, iType, StCameFrom, dEn (old energies) */
  nrg_blocks blocks;             /* Acut_N: the blocks of all states of H_N */
  const double* en;              /* [nstates] dEn (SetE0zero, SetDegen) */
  const unsigned char* kept;     /* [nstates] Kept */
  const double* eigvec;          /* dEigVec: per block n x n, row = eigenvector */
  nrg_matrix cd;                 /* c_d between all states of H_N */
} nrg_dm_shell;

/* Writes Abasis_<name>_N<n>.bin, Acut_<name>_N<n>.bin and Mat0_<name>_N<n>.bin
 * into `dir` in the byte layout of CNRGbasisarray::SaveBin / CNRGmatrix::SaveBin
 * (NRGarrayClass.cpp:780-868, 1947-2003; NRGmatrixClass.cpp:957-1015), for the
 * one-channel |Q S> model; needs no device. */
nrg_status nrg_write_dm_shell(const char* dir, const char* name, const nrg_dm_shell* s);

/* ThisCodePars.dat as CNRGCodeHandler::SaveGenPars writes it
 * (NRGcodehandlerClass.cpp): what DM_NRG reads before the shells. */
nrg_status nrg_write_code_pars(const char* dir, double lambda, int nsites, const char* name);

/* The shells of the last nrg_sweep_run_dm written with nrg_write_dm_shell,
 * plus ThisCodePars.dat: the reference's DM_NRG can then run on them. */
nrg_status nrg_dm_save_bin(nrg_ctx* ctx, const char* dir, const char* name);

/* The inverse of nrg_dm_save_bin: shells 0 .. nshells-1 (nshells <= 0: the
 * Nsitesmax of ThisCodePars.dat) of a one-channel |Q S> NRG_main run saved
 * with the spectral density switched on (calcdens = 1), read from dir in the
 * reference's layout -- what DM_NRG reads (DM_NRG.cpp:163-298;
 * CNRGarray::ReadBinInStream NRGarrayClass.cpp:886-958,
 * CNRGbasisarray::ReadBin :2005-2078, CNRGmatrix::ReadBin
 * NRGmatrixClass.cpp:1016-1082) -- into the context's DM-NRG state, so that
 * nrg_dm_backprop and nrg_lehmann run on them.  Each shell's basis must be
 * what BuildBasis makes of the previous shell's kept states (else
 * NRG_ERR_SYNC); Lambda comes from ThisCodePars.dat. */
nrg_status nrg_dm_load_bin(nrg_ctx* ctx, const char* dir, const char* name, int nshells);

/* Largest block nrg_diag_block_noalloc accepts. */
#define NRG_NOALLOC_MAX_N 256

/* Eigenvalues and eigenvectors of ONE symmetric block with no device memory
 * allocated by the call.  This entry point has no counterpart in the
 * reference; it exists for callers that cannot allocate device memory when
 * they need the solve (all memory carved out at start-up, or an allocation's
 * implicit device synchronisation not acceptable on their code path).
 *   n        block size, 1 <= n <= NRG_NOALLOC_MAX_N (larger: NRG_ERR_SIZE)
 *   a        device pointer, the full symmetric n x n matrix, row-major (read only)
 *   eigvals  device pointer, n ascending eigenvalues (written)
 *   eigvecs  device pointer, n x n row-major, row k = eigenvector k (written)
 *   stream   cudaStream_t to run on (NULL = default stream); the call returns
 *            after the stream has reached the end of the solve
 * The solver's scratch is one fixed array of about 3.7 MB in device memory,
 * kept by every GPU that loads it until the process exits.  Each call looks
 * up the array's device address on the current device; call on the device
 * you want to use.  CUDA loads the module that holds the array lazily, at its
 * first use on a device, and that load can allocate device memory and
 * synchronise: make one warm-up call per device before carving out device
 * memory, or run the process with CUDA_MODULE_LOADING=EAGER.  All calls share
 * the array: calls that overlap on the GPU (other host threads, other
 * streams) race and must not be issued. */
nrg_status nrg_diag_block_noalloc(int n, const double* a, double* eigvals, double* eigvecs, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TWOCHNRG_GB300_H */
