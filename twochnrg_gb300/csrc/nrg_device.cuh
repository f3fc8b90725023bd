// Device-side declarations shared by the GB300 NRG kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nrg {

// Largest opt-in dynamic shared memory per block of the current device.
// Kernels get this one value as their MaxDynamicSharedMemorySize attribute
// (never a per-launch size), so concurrent host threads cannot lower the
// limit between another thread's attribute call and its launch.
inline int max_dyn_smem() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

// Error flags a kernel can raise without trapping; the host reads the word
// after the launch series and turns it into an nrg_status.
enum DeviceFlag : int {
  DEV_OK = 0,
  DEV_SIZE = 1,           // a block exceeded a compiled / shared-memory limit
  DEV_NOT_CONVERGED = 2,  // inverse iteration did not converge
  DEV_BAD_INPUT = 4,      // NaN / Inf met in an input
  DEV_DEGEN_OVERFLOW = 8, // too many near-zero levels for the SetDegen pass
  DEV_TIMEOUT = 16        // a bounded wait on an mbarrier gave up
};

// ---------------------------------------------------------------- tensor-core products
// C[i][j] += alpha * sum_k A[i][k] B[j][k] (FP64 in and out) on the tcgen05
// tensor cores from split-BF16 slices (k_ozaki.cu); error of order 2^-36
// |A_i| |B_j| with S = 6.  work: oz_work_bytes(m, n, K, S) bytes of device
// scratch.  a_swap / b_swap read the operand's column (k + K/2) mod K.
constexpr int kOzMaxK = 256;
constexpr int kOzMaxSlices = 6;
struct OzGemm {
  double* C;
  int64_t ldc;
  int m, n, K, S;
  double alpha;
  const double* A;
  int64_t lda;
  const double* B;
  int64_t ldb;
  bool a_swap, b_swap;
  void* work;
  int* flag;
  int max_ctas;  // 0: one CTA per SM
};
size_t oz_work_bytes(int m, int n, int K, int S);

// One panel of the blocked Householder reduction of a large block (k_panel.cu):
// steps j in [k0, k1) against the matrix as it was at the panel's start,
// writing [V W] (n x 2nb, zeroed by the caller beforehand) for the trailing
// product H[k1:, k1:] -= [V W] [W V]^T; with `last` (k1 == n - 2) also the
// closing 2 x 2 block.
struct PanelArgs {
  double* H;      // the block, n x n row-major
  int n, k0, k1, nb;
  int last;
  double* d;      // at the block's state offset
  double* e;
  double* tau;
  double* VW;     // n x 2nb
  double* col;    // 2n scratch
  double* part;   // grid x (2nb + 2) scratch
  double* ybuf;   // 2 scratch
};
size_t panel_smem_bytes(int n, int k0, int nb, int grid);
cudaError_t launch_panel(const PanelArgs& a, int grid, cudaStream_t s);
int panel_max_grid();
size_t oz_smem_bytes(int S);
cudaError_t oz_gemm(const OzGemm& p, cudaStream_t s);

// ---------------------------------------------------------------- assembly
// One H_N block (dense n x n row-major at hoff) per new (Q,S)/(Q,Sz) sector.
struct AssembleArgs {
  int nblocks;
  const int* bsize;          // [nblocks]
  const int* bstate;         // [nblocks] first global state of the block
  const int64_t* hoff;       // [nblocks] offset of the block in H
  const int* seg_nseg;       // [nblocks] segments in the block
  // per global state
  const int* st_seg;         // local segment index
  const int* st_a;           // old state inside the old block
  const int* st_type;        // site type
  const double* st_eold;     // energy of the old state it came from
  // per (block, p, q, old operator): old-operator block for the pair of old
  // blocks of segments p and q, forward (p,q) and backward (q,p)
  const int64_t* pair_base;  // [nblocks] offset of the block's pair table
  const int64_t* pair_fwd;   // element offset or -1
  const int* pair_fwd_ld;    // columns of the forward block
  const int64_t* pair_bwd;
  const int* pair_bwd_ld;
  // coefficient tables (see nrg_model.h HNTables)
  const double* coef;        // [nblocks * per_block]
  int ntypes, nchan, nsigma;
  int nops_h;                // old operators entering H_N (pair-table stride)
  int model;                 // element arithmetic: ModelKind of the rule it follows
  int onsite;                // the diagonal adds e_N (site charge + 1)
  const double* const* ops;  // [nops_h] old operator element arrays
  double sqrt_lambda, eN;
  double chi[2];
  const double* site_q;      // [ntypes] site charge Q~ of each type
  double* H;
  // superconducting-lead |S> model (model 4): old state of every state, the
  // pairing table and the hopping's h.c. switch per type pair, Delta_N
  const int* st_old;
  const double* sc_pair;     // [ntypes^2]
  const int* hc_switch;      // [ntypes^2]; model 5: [2 * ntypes^2], spin up first
  double delta;
};
void launch_assemble(const AssembleArgs& a, int64_t total_rows, const int* row_block,
                     const int* row_index, cudaStream_t s);

// ---------------------------------------------------------------- eigensolver
struct TridiagArgs {
  int nblocks;
  const int* order;      // processing order (largest first)
  const int* bsize;
  const int64_t* hoff;   // matrix offsets; on exit row j holds v_j in cols j+1..n-1
  const int* soff;       // state offsets for d/e/tau
  double* H;
  double* d;
  double* e;
  double* tau;
  int* queue;            // work counter (reset to 0 before launch)
  int* flag;
  int maxn;
};
// threads: 512 (one CTA per SM) or 256 (two per SM, for concurrent contexts).
cudaError_t launch_tridiag(const TridiagArgs& a, int cluster, int nclusters, cudaStream_t s, int threads = 512);
size_t tridiag_smem_bytes(int maxn, int cluster, int threads = 512);
int tridiag_max_clusters(int cluster, int maxn, int threads = 512);
// Whole-GPU cooperative variant for the largest blocks (processed in turn).
int tridiag_grid_size(int maxn);
// work: tridiag_grid_work(maxn, grid) doubles of device memory.
size_t tridiag_grid_work(int maxn, int grid);
cudaError_t launch_tridiag_grid(const TridiagArgs& a, const int* big, int nbig, double* work, int grid,
                                cudaStream_t s);

struct TdEigArgs {
  int nblocks;
  const int* bsize;
  const int* soff;       // state offset of each block
  const double* d;
  const double* e;
  double* ev;            // [nstates] ascending per block
  int nstates;
  int* flag;
  int maxn;              // largest block (sizes the sort's shared memory)
  float* fde;            // scratch [2*nstates]: FP32 copies of d and e for the FP32 bracket
  double* e2;            // scratch [nstates]: e^2
  unsigned char* split;  // scratch [nstates]: e_i negligible (the pieces' ends)
  int mixed_n;           // blocks of at least this many states were reduced in mixed
                         // precision (their levels carry its ~2^-36 error); <= 0: none
};
void launch_bisect(const TdEigArgs& a, const int* state_block, cudaStream_t s);

struct InvIterArgs {
  int nblocks;
  const int* bsize;
  const int* soff;
  const double* d;
  const double* e;
  const double* ev;       // eigenvalues of T
  const int* nvec;        // [nblocks] eigenvectors wanted (lowest ones)
  const int64_t* yoff;    // [nblocks] offset of the block's Y (n x nvec, row-major)
  double* Y;              // eigenvectors of T: Y[yoff + i*nvec + k]
  double* scratch;        // 5 interleaved n x nvec arrays per block at 5*yoff
  const int* cl_block;    // per cluster of close eigenvalues: block
  const int* cl_first;    // first eigenvalue index in block
  const int* cl_count;    // eigenvalues in the cluster
  int nclusters;
  int* flag;
};
void launch_inviter(const InvIterArgs& a, const int* vec_block, const int* vec_index, int nvecs,
                    cudaStream_t s);

struct BackArgs {
  const int* bsize;
  const int64_t* hoff;    // Householder vectors in rows of H
  const double* H_const;
  const int* soff;        // tau offsets
  const double* tau;
  const int* nvec;
  const int64_t* yoff;
  const double* Y;        // eigenvectors of T (n x nvec, interleaved)
  double* Z;              // row k = eigenvector k (nvec x n) at zoff
  double* Zt;             // transposed (n x nvec) at zoff, may be null
  const int64_t* zoff;
  int maxn;
};
cudaError_t launch_backtransform(const BackArgs& a, const int* cta_block, const int* cta_first, int nctas,
                                 cudaStream_t s);
size_t backtransform_smem_bytes(int maxn);
int backtransform_warps(int maxn);  // eigenvectors per CTA

// ---------------------------------------------------------------- cut
struct CutArgs {
  int nstates;
  const double* ev;      // raw eigenvalues (left untouched)
  double* en;            // out: shifted + SetDegen-merged energies
  int ncutoff;
  double eps;            // SetDegen tolerance
  double* out_scalars;   // [0]=emin [1]=ecut [2]=nkept
  int* flag;
};
void launch_cut(const CutArgs& a, cudaStream_t s);

struct BlockStatsArgs {   // per block: kept count (leading run <= ecut) or 0 if removed
  int nblocks;
  const int* bsize;
  const int* soff;
  const double* en;
  const double* scalars;  // ecut in [1]
  int* kept;
};
void launch_block_stats(const BlockStatsArgs& a, cudaStream_t s);

struct ThermoArgs {
  const double* bq;       // [nblocks*2] block quantum numbers
  const double* en;
  int totalS;
  double beta[4];
  double* out;            // [4*3]: per beta  Z, sum SzSq e^{-bE}, sum deg E e^{-bE}
};
void launch_thermo(const ThermoArgs& a, const int* state_block, int n, double* partial, cudaStream_t s);

// ---------------------------------------------------------------- update
struct GatherTerm {       // T[dst rows] += coef * M . Zt[src rows]
  int job;                // rotation job
  int dst_base, dst_stride, rows;   // rows of T (local to the job's T)
  int src_base, src_stride, srows;  // rows of Zt_J (local to block J)
  int mode;               // 0: identity (srows == rows); 1: old block (rows x srows)
  double coef;
  int64_t old_off;        // element offset of the old block (mode 1)
  int old_ld;             // its row stride (columns of the stored old block)
  int op;                 // old operator index (mode 1)
};
struct RotJob {           // O (ki x kj) = Z_I (ki x nI) . T (nI x kj)
  int ki, kj, nI;
  int ldz, ldo;           // row strides of Zt_J and of O (>= kj: a leading part of each)
  int64_t z_off;          // Z_I (row-major ki x nI)
  int64_t zt_off;         // Zt_J (row-major nJ x ldz)
  int64_t t_off;          // T scratch (nI x kj)
  int64_t o_off;          // output in the new operator's element array
  int op;                 // operator index
};
struct UpdateArgs {
  const GatherTerm* terms;
  const int* group_first; // terms grouped by destination rows
  const int* group_count;
  int ngroups;
  const RotJob* jobs;
  const double* Z;
  const double* Zt;
  double* T;
  const double* const* old_ops;
  double* const* new_ops;
  const int* tile_job;    // GEMM tiles: job
  const int* tile_mn;     // GEMM tiles: (mtile << 16) | ntile
  int ntiles;
  // impurity-operator terms (mode 1) as GEMM tiles; the terms of one group
  // share their destination rows and are summed inside one tile
  const GatherTerm* terms1;
  const int* group1_first;
  const int* group1_count;
  const int* tile1_group;
  const int* tile1_mn;
  int ntiles1;
};
void launch_update(const UpdateArgs& a, cudaStream_t s);

struct OpDiagArgs {       // Boltzmann sums of diagonal elements over kept states
  int nblocks;
  const int* ksize;       // kept states per block
  const int* kld;         // row stride of the block's diagonal operator block (NULL: ksize)
  const int* koff;        // kept state offsets
  const double* ken;      // kept energies
  const double* bq;
  int totalS;
  double beta;
  int nops;
  const double* const* ops;
  const int64_t* diag_off; // [nops*nblocks] element offset of diagonal block, -1 if none
  double* out;            // [nops+1]: sums, last = Z
};
void launch_opdiag(const OpDiagArgs& a, const int* kstate_block, int nk, double* partial, cudaStream_t s);
int reduce_partial_count();

// ---------------------------------------------------------------- tangents (k_tangent.cu)
struct TanEigArgs {      // per block: dlambda = diag(dH~), C = dH~_kl / (lambda_l - lambda_k)
  const int* bsize;
  const int* soff;
  const int64_t* hoff;   // dH~ per block, n x n at hoff
  const double* dHt;
  const double* ev;      // levels, ascending per block
  const int* nkeep;      // kept eigenvectors per block (columns of C)
  const int64_t* coff;   // C per block, n x nkeep row-major
  double* C;
  double* dlam;          // per state
  double degen_tol;      // relative gap below which two levels do not couple
};
void launch_tan_eig(const TanEigArgs& a, int nblocks, cudaStream_t s);
void launch_tan_shift(const double* dlam, int nstates, int gs, double* dE_all, const int* kept_state, int nkept,
                      double* dE_kept, cudaStream_t s);
void launch_tan_gather(const double* dE_kept_old, const int* stcf, int n, double* out, cudaStream_t s);
void launch_tan_axpy3(const double* a, const double* b, const double* c, double scale, int64_t n, double* out,
                      cudaStream_t s);
void launch_tan_scale(const double* a, double scale, int64_t n, double* out, cudaStream_t s);
struct TanSumArgs {      // weighted sums of the thermodynamics and operator-average tangents
  static constexpr int kMaxOut = 24;  // 12 thermo sums, 2 per operator (<= 5), the last: sum deg w dE (kept)
  int nstates;
  const int* state_block;
  const double* bq;      // block quantum numbers (Q, S or Sz)
  const double* en;      // shifted energies
  const double* dE;      // their tangents
  int totalS;
  double beta[4];
  int nkept, nkblocks;
  const int* kstate_block;
  const int* koff;
  const int* kld;        // row stride of each kept block's diagonal operator block
  const double* kbq;
  const double* ken;
  const double* dEk;
  double betabar;
  int nops;
  const double* const* ops;   // averaged operators (primal) and their tangents
  const double* const* dops;
  const int64_t* diag_off;    // [nops * nkblocks]
};
size_t tan_partial_doubles();
void launch_tan_sums(const TanSumArgs& a, double* partial, double* out, cudaStream_t s);

// ---------------------------------------------------------------- DM-NRG
struct GemmJob {          // C (m x n) = op(A) (m x k) . B (k x n), row-major, FP64
  int m, n, k;
  int transA;             // 0: A stored m x k; 1: A stored k x m and used transposed
  const double* A;
  int lda;
  const double* B;
  int ldb;
  double* C;
  int ldc;
  int accum;              // 1: C += op(A) . B (after the launches that write C before)
};
// One 64x64 tile of C per CTA: tile t belongs to job tile_job[t] at
// (tile_mn[t] >> 16, tile_mn[t] & 0xffff).
void launch_gemm_jobs(const GemmJob* jobs, const int* tile_job, const int* tile_mn, int ntiles, cudaStream_t s);

struct DmTraceTerm {      // rho_N(i,j) += cg * rot[(base + i*stride) * nb + base + j*stride]
  int64_t rot_off;        // the child block of the rotated rho_{N+1} (dense nb x nb)
  int nb, base, stride;
  int count;              // i, j < count (kept states of the parent block in this segment)
  double cg;
};
struct DmTraceArgs {      // DM_NRG_CalcRhoN_withSU2 for all blocks of shell N
  const int* bsize;
  const int* soff;        // first state of each block
  const int64_t* roff;    // each block's dense n x n matrix in rho
  const int* nkept;       // kept states of each block (a prefix)
  const int* term_first;
  const int* term_count;
  const DmTraceTerm* terms;
  const double* rot;
  const double* en;
  const unsigned char* kept;
  double beta;            // FDM diagonal of discarded states: exp(-beta E) / zdisc
  double zdisc;
  double* rho;
  // Tangent form (dE != NULL): rot is the rotated tangent, and a discarded
  // state's diagonal is d[exp(-beta E) / zdisc] = exp(-beta E) / zdisc
  // (-beta dE - dlogz), dlogz = d ln zdisc.
  const double* dE;
  double dlogz;
};
void launch_dm_trace(const DmTraceArgs& a, int nblocks, cudaStream_t s);

struct DmPair {           // one block pair (b1, b2) of c_d
  int n1, n2;
  int s1, s2;             // first states of the blocks
  int64_t a_off;          // c_d block (n1 x n2) in cd
  int64_t p_off;          // rho1 . A and A . rho2 (each n1 x n2) in scratch
  double cg;              // sum_Sz CG^2 of the spectral sum
  int skip;               // both blocks without kept or without discarded states
  int r1, r2;             // rho1 . A is zero beyond row r1, A . rho2 beyond column r2
};
// The Lehmann pairs of one shell as records of the broadened-delta sum.
// A pair (i, j) of a c_d block pair has dE = E_j - E_i and the FDM weights
// W+ (omega >= 0) and W- (omega < 0).  Only pairs whose term can be nonzero
// are kept, in four lists: 0 (omega >= 0, log-Gaussian: W+ != 0, dE > 0),
// 1 (omega >= 0, Gaussian: W+ != 0, |dE| < twindow T/D_N), 2 and 3 the same
// for omega < 0 with W- and dE < 0.  Every list holds (key, w) with the
// term w exp(-(t - key)^2): log-Gaussian key = ln|dE| / b, w = W / (b |dE|
// sqrt(pi)), t = ln|omega/D_N| / b - b/4; Gaussian key = dE / bt, w = W /
// (bt sqrt(pi)), t = (omega/D_N) / bt (LogGaussDelta / GaussDelta,
// BroadDelta.cpp:96-133).  The dropped pairs contribute exactly 0.
constexpr int kPairChunk = 1024;  // pairs per CTA of the record passes
struct DmChunk { int pair, start; };
struct DmRecArgs {
  const DmPair* pairs;
  const DmChunk* chunks;
  int nchunks;
  const double* cd;
  const double* P1;
  const double* P2;
  const double* en;
  const unsigned char* kept;
  int last;               // last shell: CalcSpecCosti_T_N weights
  double beta_last, inv_z_last;
  double gauss_below;     // twindow * T / D_N
  double inv_b, inv_bt, log_scale, gauss_scale;  // 1/b, 1/bt, 1/(b sqrt pi), 1/(bt sqrt pi)
  int* counts;            // [nchunks][4]
  int64_t* offsets;       // [nchunks][4], exclusive per list
  int64_t* totals;        // [4]
  double* key[4];
  double* w[4];
  // Tangents along ntan (0 or 4) parameter directions, written by the
  // scatter pass beside each record: d(rho A) and d(A rho) of direction p at
  // dP1 / dP2 + p * pstride (the layout of P1 / P2), c_d's tangent dcd[p],
  // the energies' tangents at dE + p * nstates, d ln Z of the last shell.
  // Record q of list L gets tw[L][p * totals[L] + q] = d w and
  // tg[L][p * totals[L] + q] = 2 w d key, so that the term's tangent is
  // (d w + 2 w d key x) exp(-x^2), x = t - key.
  int ntan;
  const double* dP1;
  const double* dP2;
  int64_t pstride;
  const double* dcd[4];
  const double* dE;
  int nstates;
  double dlogz_last[4];
  double* tw[4];
  double* tg[4];
};
void launch_dm_records(const DmRecArgs& a, int pass, cudaStream_t s);  // pass 0 count + scan, 1 scatter

// One (shell, sign, branch) list of records and the frequencies whose
// window holds the shell.
constexpr int kRecChunk = 8192;   // records per CTA of the Lehmann kernel
constexpr int kOmegaTile = 64;    // frequencies per CTA
struct LehList {
  const double* key;
  const double* w;
  int64_t nrec;
  int shell, gauss;
  int nomega, omega_first;  // frequencies: omega_idx[omega_first .. +nomega)
  double* part;             // partial sums [chunk][nomega]
  const double* g;          // tangent lists: 2 w d key per record (w holds d w)
};
// delta != 0: the tile's frequencies are evenly spaced in t by delta (a
// log-spaced grid on a log-Gaussian list), and exp(-(t - key)^2) along the
// 16 frequencies of a warp follows from two exponentials by the recurrence
// g_{q+1} = g_q r_q, r_{q+1} = r_q exp(-2 delta^2).
struct LehItem { int list, chunk, tile; double delta; };
struct LehmannArgs {      // A(omega) = sum_N sum_records w exp(-(t - key)^2) / D_N
  const LehList* lists;
  const LehItem* items;
  int nitems;
  const int* omega_idx;
  const double* omega;
  const double* log_omega;  // ln|omega|
  const double* dn;         // D_N
  const double* log_dn;     // ln D_N
  double inv_b, b_quarter, inv_bt;
  int nomega;
  const int* win_first;     // first shell of each frequency's window
  const int* win_count;     // shells in the window (<= window)
  int window;
  const int* fold_list;     // [nomega][window][2]: list of (shell, branch) or -1
  const int* fold_pos;      // the frequency's position in that list
  double* out;              // [nomega]
};
void launch_lehmann(const LehmannArgs& a, cudaStream_t s);       // the items (one shell's lists)
// The same items over tangent lists: sum (d w + g x) exp(-x^2), x = t - key.
void launch_lehmann_tangent(const LehmannArgs& a, cudaStream_t s);
void launch_lehmann_fold(const LehmannArgs& a, cudaStream_t s);  // every list -> out

}  // namespace nrg
