// Host driver of the GB300 NRG engine and the C ABI (include/twochnrg_gb300.h).
//
// nrg_sweep_run follows the iteration order of NRG_main
// (src/Main/NRG_main.cpp:282-427): BuildBasis -> DiagHN -> SetKept ->
// CalcThermo -> CutStates -> UpdateMatrices -> CalcStuff -> next chi_N.
// The host does the block bookkeeping (a few hundred blocks) and builds the
// small tables the kernels read; everything per state and per matrix element
// runs on the device, and the kept eigenvectors and operator blocks stay in
// HBM from one iteration to the next.  Two host synchronisations per
// iteration remain: after the cut (the kept counts shape the next launches)
// and after the operator averages.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/twochnrg_gb300.h"
#include "nrg_device.cuh"
#include "nrg_model.h"

namespace nrg {

// ------------------------------------------------------------------ errors
struct NrgError : std::runtime_error {
  nrg_status st;
  NrgError(nrg_status s, const std::string& m) : std::runtime_error(m), st(s) {}
};

#define CU(x)                                                                                   \
  do {                                                                                          \
    cudaError_t _e = (x);                                                                       \
    if (_e != cudaSuccess)                                                                      \
      throw NrgError(_e == cudaErrorMemoryAllocation ? NRG_ERR_NOMEM : NRG_ERR_CUDA,            \
                     std::string(#x) + ": " + cudaGetErrorString(_e));                          \
  } while (0)

// ------------------------------------------------------------------ device buffers
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  ~DevBuf() { if (p) cudaFree(p); }
  // Grows by at least half the current capacity, so that a sweep whose
  // sizes creep up reallocates rarely (cudaFree synchronises the device).
  void ensure(size_t bytes) {
    if (bytes <= cap) return;
    const size_t want = std::max(bytes, cap + cap / 2);
    if (p) { CU(cudaFree(p)); p = nullptr; cap = 0; }
    CU(cudaMalloc(&p, want));
    cap = want;
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

// Packs host arrays into one staging buffer and one device buffer so a table
// set costs a single host-to-device copy.
struct Packer {
  std::vector<char> host;
  struct Item { size_t off; };
  size_t add(const void* src, size_t bytes) {
    size_t off = (host.size() + 255) & ~size_t(255);
    host.resize(off + bytes);
    if (bytes) std::memcpy(host.data() + off, src, bytes);
    return off;
  }
  template <class T> size_t add(const std::vector<T>& v) { return add(v.data(), v.size() * sizeof(T)); }
};

// Block pairs of an operator and where each dense row-major block starts.
struct OpMeta {
  std::vector<int> bi, bj;
  std::vector<int64_t> off;
  int64_t size = 0;
  int find(int i, int j) const {
    for (size_t k = 0; k < bi.size(); ++k) if (bi[k] == i && bj[k] == j) return (int)k;
    return -1;
  }
};

struct DmTan { static constexpr int NP = 4; };  // parameter directions of the DM-NRG tangents

// One Wilson shell as the DM-NRG backward sweep needs it (what NRG_main
// saves with UpdateBefCut = 1: Abasis_N, the uncut eigen-array Acut_N and
// c_d in it), kept on the device between the forward and backward sweeps.
struct DmShell {
  std::vector<int> bsize, boff;        // blocks of H_N (all states)
  std::vector<double> qn;              // (Q,S) per block
  std::vector<double> en;              // energies after SetE0zero / SetDegen
  std::vector<unsigned char> kept;     // Kept (E <= Ecut)
  std::vector<int> kept_src;           // block of each kept block (AeigCut -> Aeig)
  Basis basis;                         // Abasis_N (segments over shell N-1's kept blocks)
  OpMeta cd;                           // c_d blocks in this shell's full basis
  std::vector<int64_t> zoff;           // each block's n x n eigenvector matrix in Z
  int64_t zsize = 0;
  DevBuf Z, cdel;                      // eigenvectors (row = eigenvector) and c_d elements
  DevBuf rho;                          // reduced density matrix, dense blocks laid out like Z
  std::vector<int> rrows;              // per block: rho is zero beyond its leading rrows x rrows part
  DevBuf lpart;                        // Lehmann partial sums of this shell's record lists
  int64_t nrec[4] = {0, 0, 0, 0};
  // Tangents along the four parameters (eps_d, U, Gamma, B) of
  // nrg_grad_forward_dm; ntan = 0 without them.
  int ntan = 0;
  std::vector<double> den;             // [p * nstates + i]: d en
  DevBuf dZ[4], dcd[4], drho[4];       // d Z (rows, the layout of Z), d c_d, d rho (the layout of rho)
  DevBuf ltpart;                       // tangent Lehmann partial sums, [p][the layout of lpart]
};

struct IterResult {
  std::vector<double> params, qn, en, thermo, opavg;
  std::vector<int> bsize, kept_bsize;
  double emin = 0, ecut = 0;
  int nkept = 0;
  double wall_ms = 0, device_ms = 0;  // host wall time and CUDA-event span of the iteration
};

}  // namespace nrg

namespace nrg { namespace { struct TangentState; } }

struct nrg_ctx {
  int device = 0;
  // derivatives of the last nrg_grad_forward: the tangent pass's state and
  // the absolute ground-state energy per iteration with its tangents
  nrg::TangentState* tan = nullptr;
  std::vector<double> grad_egs, grad_degs, grad_demin;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t launches = 0;
  int num_sms = 0;
  // sweep results
  std::vector<nrg::IterResult> iters;
  std::vector<double> opavg_m1;
  nrg_timing timing{};
  // device buffers
  nrg::DevBuf meta, vmeta, H, d, e, tau, ev, en, flag, scal, Y, scratch, Z, Zt, T, partial, red, gpart, fde, e2, spl;
  nrg::DevBuf ops_a[6], ops_b[6], opptr;
  nrg::DevBuf dmcnt, dmrec, dmtab;     // Lehmann record counts / offsets, records, frequency tables
  nrg::DevBuf dmtmeta;                 // work items of the tangent Lehmann sums
  nrg::DevBuf ozw;                     // split-BF16 slices and row scales of the tensor-core products
  cudaEvent_t ev_a[8];
  // concurrent whole-GPU tridiagonalizations: side streams, fork/join events,
  // per-stream scratch and the block lists
  static constexpr int kMaxSplit = 8;
  cudaStream_t aux[kMaxSplit] = {};
  cudaEvent_t fork = nullptr, join[kMaxSplit] = {};
  nrg::DevBuf gpart_k[kMaxSplit], gbig;
  // mixed precision: per concurrent grid the blocked reduction's [V W], column
  // and share scratch, and the tensor-core product's slices
  nrg::DevBuf pvw[kMaxSplit], pcol[kMaxSplit], ppart[kMaxSplit], ozk[kMaxSplit];
  int precision = NRG_PREC_FP64;
  // drop-in outputs (host, valid until the next call on the context)
  std::vector<double> out_en, out_qn, out_cut_en, out_vec, out_el;
  std::vector<unsigned char> out_kept, out_cut_kept;
  std::vector<int> out_bbe, out_bbe_bc, out_bbe_eig, out_stcf, out_map, out_mbe;
  // DM-NRG shells of the last nrg_sweep_run_dm, and the density matrices
  double dm_lambda = 0.0;
  int dm_model = 0;  // ModelKind of the shells
  bool shared_gpu = false;  // a batch worker: other contexts run beside this one
  cudaEvent_t bsync = nullptr;  // blocking-sync event of stream_wait
  std::vector<std::unique_ptr<nrg::DmShell>> dm;
  bool dm_rho_valid = false;
  bool dm_drho_valid = false;          // the density matrices' tangents are built too
  nrg::DevBuf dmtan;                   // scratch of the tangent rotations and rho.A products
  std::vector<double> dm_drhow;        // [p][omega]: d A / d p of the last nrg_lehmann_grad
  double dm_temp = 0.0;                // temperature the density matrices were built for
  std::vector<double> dm_hm1_en;       // H_{-1} energies (what shell 0's basis came from)
  // thermodynamics with the free-chain subtraction (nrg_thermo_run): the
  // chain sweep runs on a second context beside the impurity sweep, and its
  // values are kept for later calls with the same chain parameters (the
  // reference keeps them in its chain files)
  nrg_ctx* chain_ctx = nullptr;
  bool chain_valid = false;
  nrg_sweep_config chain_cfg{};
  std::vector<double> chain_thermo;    // 16 per iteration, as nrg_iteration.thermo
  std::vector<double> th_temp, th_sus, th_sus_chain, th_sus_imp, th_ent, th_ent_chain, th_ent_imp;
  double th_chain_ms = 0.0, th_imp_ms = 0.0, th_total_ms = 0.0;
  int th_chain_reused = 0;
  // the Wilson chain set with nrg_set_chain (empty: the flat band's)
  std::vector<double> chain_chi, chain_en;
  bool chain_alambda = true;
};

namespace nrg {

namespace {

const double kPi = 3.141592653589793238462643383279502884197169;

// Chain hoppings of CNRGchain::SetChainWilson (NRGchainClass.cpp:132-155).
double chin(double lambda, int N) {
  double d0 = 1.0 - std::pow(lambda, -((double)N + 1.0));
  double d1 = std::sqrt(1.0 - std::pow(lambda, -(2.0 * (double)N + 1.0)));
  double d2 = std::sqrt(1.0 - std::pow(lambda, -(2.0 * (double)N + 3.0)));
  return d0 / (d1 * d2);
}

// chi_{-1} of NRG_main.cpp:194-207 with the sqrt(A_Lambda) factor (left out
// for the Campo-Oliveira discretization, :204-207).
double chi_m1(double lambda, double gamma, bool alambda = true) {
  double HLF = 0.5 * (1.0 + 1.0 / lambda);
  double c = std::sqrt(2.0 * gamma / kPi) / (std::sqrt(lambda) * HLF);
  return alambda ? c * std::sqrt(0.5 * std::log(lambda) * (lambda + 1) / (lambda - 1)) : c;
}

struct Timer {
  nrg_ctx* c;
  std::vector<std::pair<double*, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  explicit Timer(nrg_ctx* ctx) : c(ctx) {}
  ~Timer() { for (auto e : pool) cudaEventDestroy(e); }
  cudaEvent_t get() {
    if (used == pool.size()) { cudaEvent_t e; CU(cudaEventCreate(&e)); pool.push_back(e); }
    return pool[used++];
  }
  cudaEvent_t start() { cudaEvent_t e = get(); CU(cudaEventRecord(e, c->stream)); return e; }
  void stop(cudaEvent_t s, double* acc) {
    cudaEvent_t e = get();
    CU(cudaEventRecord(e, c->stream));
    pending.push_back({acc, {s, e}});
  }
  void collect() {  // stream must be synchronised
    for (auto& p : pending) {
      float ms = 0.f;
      CU(cudaEventElapsedTime(&ms, p.second.first, p.second.second));
      *p.first += ms;
    }
    pending.clear();
    used = 0;
  }
};

// Stream-ordered copies that also count the bytes crossing the host boundary.
void h2d(nrg_ctx* c, void* dst, const void* src, size_t bytes) {
  if (!bytes) return;
  CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
  c->timing.h2d_bytes += (int64_t)bytes;
}
void d2h(nrg_ctx* c, void* dst, const void* src, size_t bytes) {
  if (!bytes) return;
  CU(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
  c->timing.d2h_bytes += (int64_t)bytes;
}

// Waits for the context's stream.  A batch worker (shared_gpu) sleeps in the
// wait (an event with cudaEventBlockingSync) instead of spinning, so that
// many workers do not take the host cores from each other's table
// building; a context alone on the GPU spins, for the shortest wake-up.
void stream_wait(nrg_ctx* c) {
  if (!c->shared_gpu) {
    CU(cudaStreamSynchronize(c->stream));
    return;
  }
  if (!c->bsync) CU(cudaEventCreateWithFlags(&c->bsync, cudaEventBlockingSync | cudaEventDisableTiming));
  CU(cudaEventRecord(c->bsync, c->stream));
  CU(cudaEventSynchronize(c->bsync));
}

void check_flag(nrg_ctx* c) {
  int f = 0;
  CU(cudaMemcpy(&f, c->flag.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (f & DEV_SIZE) throw NrgError(NRG_ERR_SIZE, "a block exceeds the eigensolver size limit");
  if (f & DEV_DEGEN_OVERFLOW) throw NrgError(NRG_ERR_SIZE, "too many near-degenerate levels for SetDegen");
  if (f & DEV_BAD_INPUT) throw NrgError(NRG_ERR_ARG, "non-finite value met in an eigenvalue solve");
  if (f & DEV_NOT_CONVERGED) throw NrgError(NRG_ERR_NOT_CONVERGED, "inverse iteration did not converge");
  if (f & DEV_TIMEOUT) throw NrgError(NRG_ERR_TIMEOUT, "a tensor-core kernel's bounded wait gave up");
}

// ------------------------------------------------------------------ eigensolve
// Tridiagonalize all blocks, eigenvalues of all, eigenvectors of the first
// nvec[b] of each block (Z: nvec x n row-major, Zt: n x nvec), all on device.
struct EigPlan {
  std::vector<int> bsize, soff, nvec;
  std::vector<int64_t> hoff, yoff;
  int nstates = 0, maxn = 0;
  int64_t hsize = 0, ysize = 0;
};

void plan_blocks(EigPlan& P, const std::vector<int>& bsize) {
  P.bsize = bsize;
  P.soff.assign(bsize.size(), 0);
  P.hoff.assign(bsize.size(), 0);
  int s = 0;
  int64_t h = 0;
  P.maxn = 0;
  for (size_t b = 0; b < bsize.size(); ++b) {
    P.soff[b] = s; P.hoff[b] = h;
    s += bsize[b];
    h += (int64_t)bsize[b] * bsize[b];
    P.maxn = std::max(P.maxn, bsize[b]);
  }
  P.nstates = s;
  P.hsize = h;
}

// Cluster size of the small-block tridiagonalization.  A context that shares
// the GPU with others (the workers of nrg_sweep_batch) uses 4 CTAs: large
// clusters need whole free GPCs and serialize against the other contexts'
// kernels, and a block's Householder steps wait on one barrier each however
// many SMs share them (256 batched solves, 16 workers: 40.2 s with clusters
// of 16 and 8, 35.0 s with 8, 28.9 s with 4, 36.2 s with 2).
int choose_cluster(int maxn, bool shared_gpu) {
  const char* s = std::getenv("NRG_CLUSTER");
  if (s) return std::atoi(s);
  if (shared_gpu) return 4;
  return maxn >= 256 ? 16 : 8;
}

// Threads per CTA of the cluster kernel: 256 (two CTAs per SM) for the
// workers of nrg_sweep_batch, whose small latency-bound blocks gain from more
// of them in flight, else 512.
int cluster_threads(bool shared_gpu) {
  const char* s = std::getenv("NRG_CLUSTER_THREADS");
  if (s) return std::atoi(s) == 256 ? 256 : 512;
  return shared_gpu ? 256 : 512;
}

// Blocks at least this large are tridiagonalized by a cooperative grid of
// many SMs (one block after the other per grid); smaller ones by one
// thread-block cluster each.
int big_block_threshold() {
  const char* s = std::getenv("NRG_BIG_N");
  return s ? std::atoi(s) : 1800;
}

// The large blocks are dealt (by n^3, largest first) to this many concurrent
// cooperative grids, each with an equal share of the SMs: part of every
// Householder step is latency (a grid barrier, block reductions, the L2 round
// trips of the Householder vector and y), so independent blocks on fewer SMs
// each overlap those latencies.  Four grids of 38 SMs with blocks from 1800
// states on measured fastest on the two-channel workload (1 to 8 grids and
// thresholds 1500 to 3200 tried), and again with the lower-triangle kernels:
// iterations 3-7 at 3000 kept took 4.83 s, against 4.89 / 4.90 s for
// thresholds 1400 / 2400, 5.34 / 5.36 / 5.74 s for 3 / 5 / 6 grids.
// Mixed precision: blocks at least this large take the blocked reduction
// with the tensor-core trailing product (the other large blocks the FP64
// whole-grid kernel, the small ones the cluster kernel).
int mixed_block_threshold() {
  const char* s = std::getenv("NRG_MIXED_N");
  // With the lower-triangle FP64 grid kernel the blocked path pays off only
  // for the largest blocks: per full-size iteration of the two-channel sweep
  // at 3000 kept, thresholds 2600 / 3000 / 3400 / 3800 / 4200 gave 1.42 /
  // 1.33 / 1.38 / 1.21 / 1.06 s against 1.04 s for FP64.
  return s ? std::atoi(s) : 4200;
}

int grid_split(int nbig) {
  const char* s = std::getenv("NRG_GRID_SPLIT");
  int k = s ? std::atoi(s) : 4;
  k = std::max(1, std::min(k, nrg_ctx::kMaxSplit));
  return std::min(k, nbig);
}

// Cooperative grids of different contexts (the chain sweep beside the
// impurity sweep, batch workers) never run at the same time: the grids of one
// context together ask for one CTA per SM, and two contexts' grids, each
// partly resident and waiting at grid.sync for the rest, could wait on each
// other.  A context holds this lock from the launch of its grids until they
// have finished; the launches of other contexts' non-cooperative kernels are
// not held up.
std::mutex g_coop_mu;

// Panel width of the blocked reduction (mixed precision): the trailing
// product has K = 2 nb.
constexpr int kPanelNb = 32;
constexpr int kOzSlices = 6;

// Mixed precision: the large blocks of `blocks` tridiagonalized one after
// the other on stream `s` by the blocked reduction, each panel of kPanelNb
// columns on a cooperative grid of G CTAs (k_panel.cu) followed by the
// trailing rank-2 kPanelNb update H[k1:, k1:] -= [V W] [W V]^T as an
// FP64-accurate split-BF16 product on the tensor cores (k_ozaki.cu), limited
// to G CTAs so that concurrent grids share the GPU evenly.
void blocked_reduction(nrg_ctx* c, const EigPlan& P, const std::vector<int>& blocks, int slot, int G,
                       cudaStream_t s) {
  const int nb = kPanelNb, ld = 2 * kPanelNb;
  int maxn = 3;
  for (int b : blocks) maxn = std::max(maxn, P.bsize[b]);
  // sized for the next multiple of 1024 states: the largest block creeps up
  // over a sweep, and a reallocation synchronises the device
  const size_t nres = ((size_t)maxn + 1023) / 1024 * 1024;
  c->pvw[slot].ensure(sizeof(double) * nres * ld);
  c->pcol[slot].ensure(sizeof(double) * (2 * nres + 2 + (size_t)G * (ld + 2)));
  c->ozk[slot].ensure(oz_work_bytes((int)nres, (int)nres, ld, kOzSlices));
  double* VW = c->pvw[slot].as<double>();
  double* col = c->pcol[slot].as<double>();
  double* ybuf = col + 2 * (size_t)maxn;
  double* part = ybuf + 2;
  for (int b : blocks) {
    const int n = P.bsize[b];
    double* H = c->H.as<double>() + P.hoff[b];
    const int so = P.soff[b];
    if (n < 3) throw NrgError(NRG_ERR_SIZE, "blocked reduction needs n >= 3");
    if (panel_smem_bytes(n, 0, nb, G) > (size_t)max_dyn_smem())
      throw NrgError(NRG_ERR_SIZE, "blocked reduction: block too large for shared memory");
    for (int k0 = 0; k0 < n - 2; k0 += nb) {
      const int k1 = std::min(k0 + nb, n - 2);
      const bool last = k1 == n - 2;
      CU(cudaMemsetAsync(VW, 0, sizeof(double) * (size_t)n * ld, s));
      PanelArgs pa{};
      pa.H = H; pa.n = n; pa.k0 = k0; pa.k1 = k1; pa.nb = nb; pa.last = last ? 1 : 0;
      pa.d = c->d.as<double>() + so; pa.e = c->e.as<double>() + so; pa.tau = c->tau.as<double>() + so;
      pa.VW = VW; pa.col = col; pa.part = part; pa.ybuf = ybuf;
      CU(launch_panel(pa, G, s));
      c->launches++; c->timing.tridiag_launches++;
      if (last) break;
      OzGemm g{};
      g.C = H + (size_t)k1 * n + k1; g.ldc = n; g.m = n - k1; g.n = n - k1; g.K = ld; g.S = kOzSlices;
      g.alpha = -1.0; g.A = VW + (size_t)k1 * ld; g.lda = ld; g.B = g.A; g.ldb = ld; g.b_swap = true;
      g.work = c->ozk[slot].p; g.flag = c->flag.as<int>(); g.max_ctas = G;
      CU(oz_gemm(g, s));
      c->launches += 3;
    }
  }
}

// Deals blocks (largest cost first) to K bins: longest-processing-time
// greedy, then single moves and pairwise swaps out of the most loaded bin
// while they lower its load (a few passes; the bins' order within is kept
// largest first).
std::vector<std::vector<int>> deal_by_cost(const std::vector<int>& blocks, const std::vector<double>& cost, int K) {
  std::vector<std::vector<int>> bins(K);
  std::vector<double> load(K, 0.0);
  std::vector<int> idx(blocks.size());
  for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  std::vector<int> where(blocks.size());
  for (int i : idx) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    where[i] = k;
    load[k] += cost[i];
  }
  for (int pass = 0; pass < 8; ++pass) {
    const int hk = (int)(std::max_element(load.begin(), load.end()) - load.begin());
    double best = load[hk];
    int bi = -1, bj = -1, bk = -1;  // move i to bk, or swap i and j
    for (size_t i = 0; i < blocks.size(); ++i) {
      if (where[i] != hk) continue;
      for (int k = 0; k < K; ++k) {
        if (k == hk) continue;
        const double m = std::max(load[hk] - cost[i], load[k] + cost[i]);
        if (m < best - 1e-9 * best) { best = m; bi = (int)i; bj = -1; bk = k; }
        for (size_t j = 0; j < blocks.size(); ++j) {
          if (where[j] != k || cost[j] >= cost[i]) continue;
          const double d = cost[i] - cost[j];
          const double sw = std::max(load[hk] - d, load[k] + d);
          if (sw < best - 1e-9 * best) { best = sw; bi = (int)i; bj = (int)j; bk = k; }
        }
      }
    }
    if (bi < 0) break;
    if (bj < 0) {
      load[hk] -= cost[bi]; load[bk] += cost[bi]; where[bi] = bk;
    } else {
      const double d = cost[bi] - cost[bj];
      load[hk] -= d; load[bk] += d; where[bi] = bk; where[bj] = hk;
    }
  }
  for (int i : idx) bins[where[i]].push_back(blocks[i]);
  return bins;
}

// `order`: all blocks, largest first (host copy `order_h`); the big blocks
// form its prefix.
void run_tridiag_and_bisect(nrg_ctx* c, Timer& tm, const EigPlan& P, const std::vector<int>& order_h,
                            const int* d_order, const int* d_bsize, const int64_t* d_hoff, const int* d_soff,
                            const int* d_state_block) {
  const int nb = (int)P.bsize.size();
  const bool mixed = c->precision == NRG_PREC_MIXED;
  const int thr = big_block_threshold();
  int nbig = 0;
  while (nbig < nb && P.bsize[order_h[nbig]] >= thr) ++nbig;
  CU(cudaMemsetAsync(c->red.p, 0, sizeof(int), c->stream));
  TridiagArgs ta{};
  ta.nblocks = nb; ta.order = d_order; ta.bsize = d_bsize; ta.hoff = d_hoff; ta.soff = d_soff;
  ta.H = c->H.as<double>(); ta.d = c->d.as<double>(); ta.e = c->e.as<double>(); ta.tau = c->tau.as<double>();
  ta.queue = c->red.as<int>(); ta.flag = c->flag.as<int>(); ta.maxn = std::max(P.maxn, 2);
  const int K = nbig > 0 ? grid_split(nbig) : 0;
  std::vector<std::vector<int>> bins(std::max(K, 1));
  size_t o_bins[nrg_ctx::kMaxSplit] = {};
  if (K > 1) {  // deal the large blocks by cost and upload the lists before the fork
    // the lower-triangle grid kernel: 2/3 n^3 FMA plus ~21 us of barriers and
    // vector work per column (2.8e6 FMA of a quarter of the GPU)
    std::vector<int> big(order_h.begin(), order_h.begin() + nbig);
    std::vector<double> cst(nbig);
    for (int q = 0; q < nbig; ++q) {
      const double n = (double)P.bsize[big[q]];
      cst[q] = 2.0 * n * n * n / 3.0 + 2.8e6 * n;
    }
    bins = deal_by_cost(big, cst, K);
    Packer pk;
    for (int k = 0; k < K; ++k) o_bins[k] = pk.add(bins[k]);
    c->gbig.ensure(pk.host.size() + 256);
    h2d(c, c->gbig.p, pk.host.data(), pk.host.size());
  }
  std::unique_lock<std::mutex> coop(g_coop_mu, std::defer_lock);
  if (K >= 1) {
    coop.lock();
    for (int k = 0; k < K; ++k)
      if (!c->join[k]) CU(cudaEventCreateWithFlags(&c->join[k], cudaEventDisableTiming));
  }
  cudaEvent_t t0 = tm.start();
  if (mixed && K >= 1) {
    // Mixed precision: blocks from the mixed threshold on take the blocked
    // reduction (FP64 panels + tensor-core trailing products); the other
    // large blocks the FP64 whole-grid kernel, on the same stream before them.
    const int G = panel_max_grid();
    const int Gfp = tridiag_grid_size(ta.maxn);
    if (G <= 0 || Gfp <= 0) throw NrgError(NRG_ERR_SIZE, "blocked tridiagonalization does not fit");
    const int mthr = mixed_block_threshold();
    // Deal the large blocks to the K streams by their cost on the path they
    // take (greedy, largest first): per column, the FP64 kernel does two
    // FMAs per trailing element of the lower triangle and pays ~21 us of
    // barriers and vector work, the blocked panel one FMA per element of the
    // full trailing matrix and ~50 us; in FMA units of a quarter of the GPU
    // (about 1.3e11 FMA/s), 2.8e6 and 6.6e6 per column.
    auto cost = [&](int n) {
      const double n3 = (double)n * n * n;
      return n >= mthr ? n3 / 3.0 + 6.6e6 * n : 2.0 * n3 / 3.0 + 2.8e6 * n;
    };
    {
      std::vector<int> big(order_h.begin(), order_h.begin() + nbig);
      std::vector<double> cst(nbig);
      for (int q = 0; q < nbig; ++q) cst[q] = cost(P.bsize[big[q]]);
      bins = deal_by_cost(big, cst, K);
    }
    if (!c->fork) CU(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
    CU(cudaEventRecord(c->fork, c->stream));
    Packer pk;
    std::vector<std::vector<int>> fp(K), bl(K);
    size_t o_fp[nrg_ctx::kMaxSplit] = {};
    for (int k = 0; k < K; ++k) {
      for (int b : bins[k]) (P.bsize[b] >= mthr ? bl[k] : fp[k]).push_back(b);
      o_fp[k] = pk.add(fp[k]);
    }
    c->gbig.ensure(pk.host.size() + 256);
    h2d(c, c->gbig.p, pk.host.data(), pk.host.size());
    for (int k = 0; k < K; ++k) {
      cudaStream_t sk = c->stream;
      if (K > 1) {
        if (!c->aux[k]) CU(cudaStreamCreateWithFlags(&c->aux[k], cudaStreamNonBlocking));
        sk = c->aux[k];
        CU(cudaStreamWaitEvent(sk, c->fork, 0));
      }
      if (!fp[k].empty()) {
        c->gpart_k[k].ensure(sizeof(double) * tridiag_grid_work(ta.maxn, Gfp / K));
        CU(launch_tridiag_grid(ta, (const int*)(c->gbig.as<char>() + o_fp[k]), (int)fp[k].size(),
                               c->gpart_k[k].as<double>(), Gfp / K, sk));
        c->launches++; c->timing.tridiag_launches++;
      }
      if (!bl[k].empty()) blocked_reduction(c, P, bl[k], k, G / K, sk);
      CU(cudaEventRecord(c->join[k], sk));
    }
  } else if (K == 1) {
    const int G = tridiag_grid_size(ta.maxn);
    if (G <= 0) throw NrgError(NRG_ERR_SIZE, "whole-GPU tridiagonalization does not fit");
    c->gpart.ensure(sizeof(double) * tridiag_grid_work(ta.maxn, G));
    CU(launch_tridiag_grid(ta, d_order, nbig, c->gpart.as<double>(), G, c->stream));
    CU(cudaEventRecord(c->join[0], c->stream));
    c->launches++; c->timing.tridiag_launches++;
  } else if (K > 1) {
    const int G = tridiag_grid_size(ta.maxn);
    if (G <= 0) throw NrgError(NRG_ERR_SIZE, "whole-GPU tridiagonalization does not fit");
    const int Gk = G / K;
    if (!c->fork) CU(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
    CU(cudaEventRecord(c->fork, c->stream));
    for (int k = 0; k < K; ++k) {
      if (!c->aux[k]) CU(cudaStreamCreateWithFlags(&c->aux[k], cudaStreamNonBlocking));
      c->gpart_k[k].ensure(sizeof(double) * tridiag_grid_work(ta.maxn, Gk));
      CU(cudaStreamWaitEvent(c->aux[k], c->fork, 0));
      CU(launch_tridiag_grid(ta, (const int*)(c->gbig.as<char>() + o_bins[k]), (int)bins[k].size(),
                             c->gpart_k[k].as<double>(), Gk, c->aux[k]));
      CU(cudaEventRecord(c->join[k], c->aux[k]));
      c->launches++; c->timing.tridiag_launches++;
    }
  }
  if (nbig < nb) {
    int maxs = P.bsize[order_h[nbig]];
    TridiagArgs ts = ta;
    ts.order = d_order + nbig;
    ts.nblocks = nb - nbig;
    ts.maxn = std::max(maxs, 2);
    int cluster = choose_cluster(maxs, c->shared_gpu);
    int threads = cluster_threads(c->shared_gpu);
    int ncl = tridiag_max_clusters(cluster, ts.maxn, threads);
    if (ncl <= 0) { cluster = 8; threads = 512; ncl = tridiag_max_clusters(cluster, ts.maxn, threads); }
    if (ncl <= 0) throw NrgError(NRG_ERR_SIZE, "tridiagonalization does not fit on the device");
    ncl = std::min(ncl, nb - nbig);
    CU(launch_tridiag(ts, cluster, ncl, c->stream, threads));
    c->launches++; c->timing.tridiag_launches++;
  }
  for (int k = 0; K > 1 && k < K; ++k) CU(cudaStreamWaitEvent(c->stream, c->join[k], 0));
  if (coop.owns_lock()) {
    for (int k = 0; k < K; ++k) CU(cudaEventSynchronize(c->join[k]));
    coop.unlock();
  }
  tm.stop(t0, &c->timing.tridiag_ms);
  double fl = 0.0;
  for (int n : P.bsize) fl += 4.0 / 3.0 * (double)n * n * n;
  c->timing.tridiag_flops += fl;
  TdEigArgs ea{};
  ea.nblocks = nb; ea.bsize = d_bsize; ea.soff = d_soff; ea.d = c->d.as<double>(); ea.e = c->e.as<double>();
  ea.ev = c->ev.as<double>(); ea.nstates = P.nstates; ea.flag = c->flag.as<int>(); ea.maxn = std::max(P.maxn, 1);
  c->fde.ensure(sizeof(float) * 2 * std::max(P.nstates, 1));
  ea.fde = c->fde.as<float>();
  c->e2.ensure(sizeof(double) * std::max(P.nstates, 1));
  ea.e2 = c->e2.as<double>();
  c->spl.ensure(std::max(P.nstates, 1));
  ea.split = c->spl.as<unsigned char>();
  ea.mixed_n = mixed ? std::max(thr, mixed_block_threshold()) : 0;
  cudaEvent_t t1 = tm.start();
  launch_bisect(ea, d_state_block, c->stream);
  c->launches += 3;  // FP32 copies, levels, ordering
  tm.stop(t1, &c->timing.tridiag_eig_ms);
}

// Eigenvectors for the lowest nvec[b] levels of every block (host has the
// eigenvalues `ev` to form clusters).
void run_vectors(nrg_ctx* c, Timer& tm, EigPlan& P, const std::vector<double>& ev_host, const int* d_bsize,
                 const int64_t* d_hoff, const int* d_soff) {
  const int nb = (int)P.bsize.size();
  P.yoff.assign(nb, 0);
  int64_t y = 0;
  for (int b = 0; b < nb; ++b) { P.yoff[b] = y; y += (int64_t)P.bsize[b] * P.nvec[b]; }
  P.ysize = y;
  if (y == 0) return;
  std::vector<int> vb, vi, cb, cf, cn, ctab, ctaf;
  const int bw = backtransform_warps(std::max(P.maxn, 1));
  for (int b = 0; b < nb; ++b) {
    const int n = P.bsize[b], k = P.nvec[b];
    if (k == 0) continue;
    double onenrm = 0.0;
    for (int i = 0; i < n; ++i) onenrm = std::max(onenrm, std::fabs(ev_host[P.soff[b] + i]));
    const double ortol = 1e-4 * std::max(onenrm, 1e-300);
    int start = 0;
    for (int x = 0; x < k; ++x) {
      vb.push_back(b); vi.push_back(x);
      if (x > 0 && ev_host[P.soff[b] + x] - ev_host[P.soff[b] + x - 1] > ortol) {
        cb.push_back(b); cf.push_back(start); cn.push_back(x - start); start = x;
      }
    }
    cb.push_back(b); cf.push_back(start); cn.push_back(k - start);
    for (int x = 0; x < k; x += bw) { ctab.push_back(b); ctaf.push_back(x); }
  }
  Packer pk;
  size_t o_nvec = pk.add(P.nvec), o_yoff = pk.add(P.yoff), o_vb = pk.add(vb), o_vi = pk.add(vi), o_cb = pk.add(cb),
         o_cf = pk.add(cf), o_cn = pk.add(cn), o_tb = pk.add(ctab), o_tf = pk.add(ctaf);
  DevBuf& mb = c->vmeta;
  mb.ensure(pk.host.size() + 256);
  h2d(c, mb.p, pk.host.data(), pk.host.size());
  char* base = mb.as<char>();
  c->Y.ensure(sizeof(double) * y);
  c->scratch.ensure(sizeof(double) * 5 * y);
  c->Z.ensure(sizeof(double) * y);
  c->Zt.ensure(sizeof(double) * y);
  InvIterArgs ia{};
  ia.nblocks = nb; ia.bsize = d_bsize; ia.soff = d_soff; ia.d = c->d.as<double>(); ia.e = c->e.as<double>();
  ia.ev = c->ev.as<double>(); ia.nvec = (const int*)(base + o_nvec); ia.yoff = (const int64_t*)(base + o_yoff);
  ia.Y = c->Y.as<double>(); ia.scratch = c->scratch.as<double>();
  ia.cl_block = (const int*)(base + o_cb); ia.cl_first = (const int*)(base + o_cf); ia.cl_count = (const int*)(base + o_cn);
  ia.nclusters = (int)cb.size(); ia.flag = c->flag.as<int>();
  cudaEvent_t t0 = tm.start();
  launch_inviter(ia, (const int*)(base + o_vb), (const int*)(base + o_vi), (int)vb.size(), c->stream);
  c->launches += 2;
  tm.stop(t0, &c->timing.vectors_ms);
  BackArgs ba{};
  ba.bsize = d_bsize; ba.hoff = d_hoff; ba.H_const = c->H.as<double>(); ba.soff = d_soff; ba.tau = c->tau.as<double>();
  ba.nvec = ia.nvec; ba.yoff = ia.yoff; ba.Y = c->Y.as<double>(); ba.Z = c->Z.as<double>(); ba.Zt = c->Zt.as<double>();
  ba.zoff = ia.yoff; ba.maxn = std::max(P.maxn, 1);
  cudaEvent_t t1 = tm.start();
  CU(launch_backtransform(ba, (const int*)(base + o_tb), (const int*)(base + o_tf), (int)ctab.size(), c->stream));
  c->launches++;
  tm.stop(t1, &c->timing.backtransform_ms);
  double fl = 0.0;
  for (int b = 0; b < nb; ++b) fl += 2.0 * (double)P.bsize[b] * P.bsize[b] * P.nvec[b];
  c->timing.backtransform_flops += fl;
}

// ------------------------------------------------------------------ sweep state

struct Kept {
  BlockArray blk;        // kept blocks: QNs, kept sizes, offsets
  std::vector<int> src;  // index of the block in the previous iteration's basis
};

struct Sweep {
  nrg_ctx* c;
  ModelSpec m;
  nrg_sweep_config cfg;
  Kept kept;
  std::vector<OpMeta> ops;
  int cur = 0;           // which of ops_a / ops_b holds the current operators
  DevBuf* opbuf(int which, int o) { return which == 0 ? &c->ops_a[o] : &c->ops_b[o]; }
};

double opavg_host(const BlockArray& a, const std::vector<double>& en, const std::vector<double>& diag, bool totalS,
                  double beta) {
  // CalcOpAvg (CalcOpAvg.cpp:13-84) on a one-state-per-block array.
  double s = 0, Z = 0;
  for (int b = 0; b < a.nblocks(); ++b) {
    double deg = totalS ? 2.0 * a.q(b, 1) + 1.0 : 1.0;
    for (int i = a.offset[b]; i < a.offset[b] + a.size[b]; ++i) {
      double w = std::exp(-beta * en[i]);
      s += deg * diag[i] * w; Z += deg * w;
    }
  }
  if (!(std::fabs(Z) < 1.e-20)) s = s / Z;
  return s;
}

// CalcSuscep / CalcEntropy (CalcThermo.cpp:16-121) at the four betabar_nc of
// CNRGCodeHandler::CalcThermo (NRGcodehandlerClass.cpp:627-677) for a small
// host array (the free-chain H_0): (betabar_nc, D/betabar_nc, T chi, S) x 4,
// the layout the thermo kernel's results are reported in.
std::vector<double> thermo_host(const BlockArray& a, const std::vector<double>& en, bool totalS, double lambda,
                                double DN, double betabar) {
  std::vector<double> out;
  for (int nc = 1; nc <= 4; ++nc) {
    const double beta = betabar * std::pow(lambda, (nc - 4) / (2.0 * 4));
    double Z = 0, s1 = 0, sE = 0;
    for (int b = 0; b < a.nblocks(); ++b) {
      const double S = a.q(b, 1);
      const double deg = totalS ? 2.0 * S + 1.0 : 1.0;
      const double szsq = totalS ? (1.0 / 12.0) * deg * (deg * deg - 1.0) : S * S;
      for (int i = a.offset[b]; i < a.offset[b] + a.size[b]; ++i) {
        const double w = std::exp(-beta * en[i]);
        Z += deg * w; s1 += szsq * w; sE += deg * en[i] * w;
      }
    }
    out.push_back(beta);
    out.push_back(DN / beta);
    out.push_back(s1 / Z);
    out.push_back(beta * (sE / Z) + std::log(Z));
  }
  return out;
}

// Device tables of one DiagHN assembly, uploaded to c->meta.
struct AsmTables {
  EigPlan P;
  std::vector<int> order;  // blocks, largest first
  size_t o_bsize = 0, o_soff = 0, o_hoff = 0, o_order = 0, o_sb = 0, o_ri = 0, o_bq = 0;
  AssembleArgs aa{};
};

// Builds and uploads everything the assembly kernel reads for basis B:
// per-state rows (segment, old state, site type, E_old), per block the
// (old block pair, operator) -> operator block offsets, the coefficient
// tables, and sizes H/d/e/tau/ev/en for the blocks.  `oldops` describe the
// operators (device pointers `hops`) in the block structure whose block
// sizes are `old_size`; opblock maps a block of the previous kept array to
// that structure's block (NULL: the operators live in the kept array itself).
// Kept states are the leading states of their block, so a state's row is the
// same in both.
AsmTables prepare_assembly(nrg_ctx* c, const ModelSpec& m, const Basis& B, const HNTables& tabs,
                           const std::vector<double>& st_eold, const std::vector<OpMeta>& oldops,
                           const std::vector<int>& old_size, int nops_h, const std::vector<const double*>& hops,
                           double lambda, const double chi[2], double eN,
                           const std::vector<int>* opblock = nullptr, double delta = 0.0) {
  auto ob = [&](int k) { return opblock ? (*opblock)[k] : k; };
  AsmTables T;
  EigPlan& P = T.P;
  const int nb = B.blk.nblocks();
  plan_blocks(P, B.blk.size);
  T.order.resize(nb);
  for (int b = 0; b < nb; ++b) T.order[b] = b;
  std::stable_sort(T.order.begin(), T.order.end(), [&](int x, int y) { return P.bsize[x] > P.bsize[y]; });
  std::vector<int> state_block(P.nstates), row_index(P.nstates), st_seg(P.nstates), st_a(P.nstates),
      st_type(P.nstates);
  for (int b = 0; b < nb; ++b)
    for (int i = 0; i < P.bsize[b]; ++i) {
      int g = P.soff[b] + i;
      state_block[g] = b; row_index[g] = i;
      st_seg[g] = B.seg_of[g]; st_a[g] = B.a_of[g]; st_type[g] = B.itype[g];
    }
  std::vector<int> nseg(nb);
  std::vector<int64_t> pair_base(nb), pair_fwd, pair_bwd;
  std::vector<int> pair_fwd_ld, pair_bwd_ld;
  for (int b = 0; b < nb; ++b) {
    const auto& sg = B.seg[b];
    nseg[b] = (int)sg.size();
    pair_base[b] = (int64_t)pair_fwd.size();
    for (size_t p = 0; p < sg.size(); ++p)
      for (size_t q = 0; q < sg.size(); ++q)
        for (int o = 0; o < nops_h; ++o) {
          const OpMeta& om = oldops[o];
          int kf = om.find(ob(sg[p].old_block), ob(sg[q].old_block));
          int kb = om.find(ob(sg[q].old_block), ob(sg[p].old_block));
          pair_fwd.push_back(kf >= 0 ? om.off[kf] : -1);
          pair_fwd_ld.push_back(kf >= 0 ? old_size[om.bj[kf]] : 0);
          pair_bwd.push_back(kb >= 0 ? om.off[kb] : -1);
          pair_bwd_ld.push_back(kb >= 0 ? old_size[om.bj[kb]] : 0);
        }
  }
  std::vector<double> site_q(m.site.nstates);
  for (int t = 0; t < m.site.nstates; ++t) site_q[t] = m.site.blk.q(m.site.block_of_state(t), 0);
  // |S> model: the e_N term counts the site's electrons, {0, 2, 1, 1}
  // (OneChS_HNsc_MatEl's auxN); pairing and h.c.-switch tables
  const int NT = m.site.nstates;
  std::vector<double> sc_pair(NT * NT, 0.0);
  std::vector<int> hc_sw(2 * NT * NT, 0), st_old(P.nstates, 0);
  if (m.kind == MODEL_1CHS || m.kind == MODEL_1CHSZ) {
    site_q = {-1.0, 1.0, 0.0, 0.0};
    for (int a = 0; a < NT; ++a)
      for (int b2 = 0; b2 < NT; ++b2) {
        sc_pair[a * NT + b2] = sc_pair_1chS(a, b2);
        if (m.kind == MODEL_1CHS) {
          hc_sw[a * NT + b2] = hc_switch_1chS(a, b2) ? 1 : 0;
        } else {  // per spin: sigma = +1 first, as the old operators f_up, f_dn
          hc_sw[a * NT + b2] = hc_switch_1chSz(1, a, b2) ? 1 : 0;
          hc_sw[NT * NT + a * NT + b2] = hc_switch_1chSz(-1, a, b2) ? 1 : 0;
        }
      }
    for (int g = 0; g < P.nstates; ++g) st_old[g] = B.stcf[g];
  }
  Packer pk;
  T.o_bsize = pk.add(P.bsize); T.o_soff = pk.add(P.soff); T.o_hoff = pk.add(P.hoff); T.o_order = pk.add(T.order);
  T.o_sb = pk.add(state_block); T.o_ri = pk.add(row_index);
  size_t o_seg = pk.add(st_seg), o_a = pk.add(st_a), o_type = pk.add(st_type), o_eold = pk.add(st_eold),
         o_nseg = pk.add(nseg), o_pb = pk.add(pair_base), o_pf = pk.add(pair_fwd), o_pfl = pk.add(pair_fwd_ld),
         o_pbw = pk.add(pair_bwd), o_pbl = pk.add(pair_bwd_ld), o_coef = pk.add(tabs.coef), o_sq = pk.add(site_q),
         o_scp = pk.add(sc_pair), o_hcs = pk.add(hc_sw), o_sto = pk.add(st_old);
  T.o_bq = pk.add(B.blk.qn);
  c->meta.ensure(pk.host.size() + 256);
  h2d(c, c->meta.p, pk.host.data(), pk.host.size());
  char* mb = c->meta.as<char>();
  c->H.ensure(sizeof(double) * std::max<int64_t>(P.hsize, 1));
  c->d.ensure(sizeof(double) * P.nstates); c->e.ensure(sizeof(double) * P.nstates);
  c->tau.ensure(sizeof(double) * P.nstates); c->ev.ensure(sizeof(double) * P.nstates);
  c->en.ensure(sizeof(double) * P.nstates);
  c->red.ensure(sizeof(int) * (nb + 8));
  c->opptr.ensure(sizeof(double*) * 32);
  std::vector<const double*> ptrs(hops);
  ptrs.resize(8, nullptr);
  h2d(c, c->opptr.p, ptrs.data(), sizeof(double*) * ptrs.size());
  AssembleArgs& aa = T.aa;
  aa.nblocks = nb; aa.bsize = (const int*)(mb + T.o_bsize); aa.bstate = (const int*)(mb + T.o_soff);
  aa.hoff = (const int64_t*)(mb + T.o_hoff); aa.seg_nseg = (const int*)(mb + o_nseg);
  aa.st_seg = (const int*)(mb + o_seg); aa.st_a = (const int*)(mb + o_a); aa.st_type = (const int*)(mb + o_type);
  aa.st_eold = (const double*)(mb + o_eold); aa.pair_base = (const int64_t*)(mb + o_pb);
  aa.pair_fwd = (const int64_t*)(mb + o_pf); aa.pair_fwd_ld = (const int*)(mb + o_pfl);
  aa.pair_bwd = (const int64_t*)(mb + o_pbw); aa.pair_bwd_ld = (const int*)(mb + o_pbl);
  aa.coef = (const double*)(mb + o_coef); aa.ntypes = tabs.ntypes; aa.nchan = tabs.nchan; aa.nsigma = tabs.nsigma;
  aa.nops_h = nops_h; aa.model = m.hn_form; aa.onsite = m.onsite ? 1 : 0; aa.ops = (const double* const*)c->opptr.p;
  aa.sqrt_lambda = std::sqrt(lambda); aa.eN = eN; aa.chi[0] = chi[0]; aa.chi[1] = chi[1];
  aa.site_q = (const double*)(mb + o_sq); aa.H = c->H.as<double>();
  aa.sc_pair = (const double*)(mb + o_scp); aa.hc_switch = (const int*)(mb + o_hcs);
  aa.st_old = (const int*)(mb + o_sto); aa.delta = delta;
  return T;
}

// UpdateMatrices for all operators: the host lists, per kept block pair
// (i, j) allowed by CheckForMatEl, one rotation job Z_i F Z_j^T and the terms
// of F (site factor x identity, or old operator block x identity), packed in
// `up`.  The caller adds the operator pointer tables (o_old, o_new) and any
// tables of its own to `up` before launch_update_plan.
struct UpdatePlan {
  std::vector<OpMeta> newops;
  std::vector<RotJob> jobs;
  std::vector<GatherTerm> terms, terms1;
  std::vector<int> g1first, g1count, t1group, t1mn, gfirst, gcount, tjob, tmn;
  int64_t tsize = 0;
  Packer up;
  size_t o_t1 = 0, o_g1f = 0, o_g1c = 0, o_t1g = 0, o_t1m = 0, o_terms = 0, o_gf = 0, o_gc = 0, o_jobs = 0,
         o_tj = 0, o_tm = 0;
  size_t o_old = 0, o_new = 0;
  char* ub = nullptr;  // device copy of `up` once launched
};

// kept: the new kept structure (K.src = block of B each kept block came
// from); yoff/bsize: where each B block's kept eigenvector rows sit in c->Z
// (kept x n, row-major) and c->Zt (n x kept).  opblock maps a block of the
// previous kept array (a segment's old_block) to the block the old operators
// are stored by (NULL: the same block).
//
// kept_rows (DM-NRG shells, K = every state): per block of B its kept
// states.  Operators other than c_d are then computed on the kept states only
// (the next iteration reads nothing else), in the full layout.
void plan_update(UpdatePlan& U, const ModelSpec& m, const Basis& B, const EigPlan& P, const Kept& K,
                 const std::vector<OpMeta>& oldops, const std::vector<int>* opblock = nullptr,
                 const std::vector<int>* opsize = nullptr, const std::vector<int>* kept_rows = nullptr) {
  auto ob = [&](int k) { return opblock ? (*opblock)[k] : k; };
  const int nops = (int)m.op_kind.size();
  U.newops.assign(nops, OpMeta());
  const int nk = K.blk.nblocks();
  for (int o = 0; o < nops; ++o) {
    OpMeta& no = U.newops[o];
    for (int i = 0; i < nk; ++i)
      for (int j = 0; j < nk; ++j) {
        if (!op_check(m, m.op_check[o], K.blk, i, j)) continue;
        const int bI = K.src[i], bJ = K.src[j];
        const bool cd_like = m.op_kind[o] == OP_CD_QS || m.op_kind[o] == OP_CD_2CH || m.op_kind[o] >= OP_PLUGIN_IMP;
        const bool kept_only = kept_rows && !cd_like;
        RotJob J{};
        J.ki = K.blk.size[i]; J.kj = K.blk.size[j]; J.nI = P.bsize[bI];
        J.ldz = J.kj; J.ldo = J.kj;
        J.z_off = P.yoff[bI]; J.zt_off = P.yoff[bJ]; J.t_off = U.tsize; J.o_off = no.size; J.op = o;
        no.bi.push_back(i); no.bj.push_back(j); no.off.push_back(no.size);
        no.size += (int64_t)J.ki * J.kj;
        if (kept_only) { J.ki = (*kept_rows)[bI]; J.kj = (*kept_rows)[bJ]; }
        U.tsize += (int64_t)J.nI * J.kj;
        const int jid = (int)U.jobs.size();
        U.jobs.push_back(J);
        const double SI = B.blk.q(bI, 1), SJ = B.blk.q(bJ, 1);
        const auto& segI = B.seg[bI];
        const auto& segJ = B.seg[bJ];
        for (const Segment& p : segI)
          for (int u = 0; u < p.nsite; ++u) {
            const int tu_ = m.site.blk.offset[p.site_block] + u;
            const int first = (int)U.terms.size();
            const int first1 = (int)U.terms1.size();
            for (const Segment& q : segJ)
              for (int v = 0; v < q.nsite; ++v) {
                const int tv = m.site.blk.offset[q.site_block] + v;
                GatherTerm G{};
                G.job = jid; G.dst_base = p.offset + u; G.dst_stride = p.nsite; G.rows = p.count;
                G.src_base = q.offset + v; G.src_stride = q.nsite; G.srows = q.count;
                if (m.op_kind[o] == OP_IMPONLY || cd_like) {
                  double g = 1.0;
                  if (m.op_kind[o] == OP_IMPONLY) {
                    if (tu_ != tv) continue;
                  } else {
                    g = op_site_factor(m, m.op_kind[o], SI, SJ, tu_, tv);
                    if (g == 0.0) continue;
                  }
                  const OpMeta& om = oldops[o];
                  int kx = om.find(ob(p.old_block), ob(q.old_block));
                  if (kx < 0) continue;
                  G.mode = 1; G.coef = g; G.old_off = om.off[kx]; G.op = o;
                  G.old_ld = opsize ? (*opsize)[ob(q.old_block)] : q.count;
                } else {
                  if (p.old_block != q.old_block) continue;
                  double g = op_site_factor(m, m.op_kind[o], SI, SJ, tu_, tv);
                  if (g == 0.0) continue;
                  G.mode = 0; G.coef = g;
                }
                if (G.mode == 1) {  // old block x Zt rows: tiled GEMM over the row group's terms
                  U.terms1.push_back(G);
                  continue;
                }
                U.terms.push_back(G);
              }
            if ((int)U.terms.size() > first) { U.gfirst.push_back(first); U.gcount.push_back((int)U.terms.size() - first); }
            if ((int)U.terms1.size() > first1) {
              const int gid = (int)U.g1first.size();
              U.g1first.push_back(first1); U.g1count.push_back((int)U.terms1.size() - first1);
              for (int mt = 0; mt * 64 < p.count; ++mt)
                for (int nt = 0; nt * 64 < J.kj; ++nt) { U.t1group.push_back(gid); U.t1mn.push_back((mt << 16) | nt); }
            }
          }
        for (int mt = 0; mt * 64 < J.ki; ++mt)
          for (int nt = 0; nt * 64 < J.kj; ++nt) { U.tjob.push_back(jid); U.tmn.push_back((mt << 16) | nt); }
      }
  }
  U.o_t1 = U.up.add(U.terms1); U.o_g1f = U.up.add(U.g1first); U.o_g1c = U.up.add(U.g1count);
  U.o_t1g = U.up.add(U.t1group); U.o_t1m = U.up.add(U.t1mn);
  U.o_terms = U.up.add(U.terms); U.o_gf = U.up.add(U.gfirst); U.o_gc = U.up.add(U.gcount);
  U.o_jobs = U.up.add(U.jobs); U.o_tj = U.up.add(U.tjob); U.o_tm = U.up.add(U.tmn);
}

// Substitutions for a run of an update plan with other inputs (the tangent
// pass): eigenvector rows Z and columns Zt, device tables of old and new
// operator pointers, and whether the site-operator (identity-on-old) terms
// take part.
struct UpdateInputs {
  const double* Z = nullptr;
  const double* Zt = nullptr;
  const double* const* old_tab = nullptr;
  double* const* new_tab = nullptr;
  bool site_terms = true;
};

void launch_update_plan(nrg_ctx* c, Timer& tm, UpdatePlan& U, const UpdateInputs* sub = nullptr) {
  cudaEvent_t tu = tm.start();
  const size_t tbytes = sizeof(double) * std::max<int64_t>(U.tsize, 1);
  if (!sub) {
    c->T.ensure(tbytes + U.up.host.size() + 512);
    U.ub = c->T.as<char>() + ((tbytes + 255) & ~size_t(255));
    h2d(c, U.ub, U.up.host.data(), U.up.host.size());
  }
  CU(cudaMemsetAsync(c->T.p, 0, tbytes, c->stream));
  char* ub = U.ub;
  UpdateArgs ua{};
  ua.terms = (const GatherTerm*)(ub + U.o_terms); ua.group_first = (const int*)(ub + U.o_gf);
  ua.group_count = (const int*)(ub + U.o_gc); ua.ngroups = (int)U.gfirst.size(); ua.jobs = (const RotJob*)(ub + U.o_jobs);
  ua.Z = c->Z.as<double>(); ua.Zt = c->Zt.as<double>(); ua.T = c->T.as<double>();
  ua.old_ops = (const double* const*)(ub + U.o_old); ua.new_ops = (double* const*)(ub + U.o_new);
  if (sub) {
    ua.Z = sub->Z; ua.Zt = sub->Zt; ua.old_ops = sub->old_tab; ua.new_ops = sub->new_tab;
    if (!sub->site_terms) ua.ngroups = 0;
  }
  ua.tile_job = (const int*)(ub + U.o_tj); ua.tile_mn = (const int*)(ub + U.o_tm); ua.ntiles = (int)U.tjob.size();
  ua.terms1 = (const GatherTerm*)(ub + U.o_t1); ua.group1_first = (const int*)(ub + U.o_g1f);
  ua.group1_count = (const int*)(ub + U.o_g1c); ua.tile1_group = (const int*)(ub + U.o_t1g);
  ua.tile1_mn = (const int*)(ub + U.o_t1m); ua.ntiles1 = (int)U.t1group.size();
  launch_update(ua, c->stream);
  if (ua.ntiles1 > 0) c->launches++;
  c->launches += 2;
  for (const RotJob& J : U.jobs) c->timing.update_flops += 2.0 * J.ki * (double)J.nI * J.kj;
  tm.stop(tu, &c->timing.update_ms);
}

// Grouped FP64 GEMM jobs (gemm_jobs_kernel): one 64 x 64 tile per CTA.
struct GemmPlan {
  std::vector<GemmJob> jobs;
  std::vector<int> tjob, tmn;
  void add(const GemmJob& J) {
    const int id = (int)jobs.size();
    jobs.push_back(J);
    for (int mt = 0; mt * 64 < J.m; ++mt)
      for (int nt = 0; nt * 64 < J.n; ++nt) { tjob.push_back(id); tmn.push_back((mt << 16) | nt); }
  }
};

void run_gemm_plan(nrg_ctx* c, const GemmPlan& G) {
  if (G.jobs.empty()) return;
  Packer pk;
  size_t oj = pk.add(G.jobs), ot = pk.add(G.tjob), om = pk.add(G.tmn);
  c->vmeta.ensure(pk.host.size() + 256);
  h2d(c, c->vmeta.p, pk.host.data(), pk.host.size());
  char* b = c->vmeta.as<char>();
  launch_gemm_jobs((const GemmJob*)(b + oj), (const int*)(b + ot), (const int*)(b + om), (int)G.tjob.size(), c->stream);
  c->launches++;
}

// The tangent pass of nrg_grad_forward: for each of the four parameters
// (eps_d, U, Gamma, B) the tangents of the kept energies and of the
// operators, carried from iteration to iteration beside the primal sweep
// (ping-pong buffers like the primal operators), the scratch of the
// eigen-derivatives, and the per-iteration results.
struct TangentState {
  static constexpr int NP = 4;
  double params[NP] = {0, 0, 0, 0};     // eps_d, U, Gamma, B of the sweep
  DevBuf dEk[NP][2], dops[NP][2][6];
  DevBuf deold, dH, T1, dHt, C, dZ, dZt, dlam, dEall, tmp[3][6], gscaled[6], tabs, part, out;
  // per iteration n and parameter k (index n * NP + k): tangents of the
  // thermodynamic values (the 16 of nrg_iteration.thermo), of the operator
  // averages, and of the raw lowest level (lambda_min, before SetE0zero)
  std::vector<double> dthermo, dopavg, dlmin;
  int nops = 0;
};

// dm: NRG_main with the spectral density switched on (calcdens = 1,
// UpdateBefCut = 1; CodeHandler_ModelSwitch.cpp:162-176, NRG_main.cpp:334-396):
// the operators are f_N and c_d, they are rotated into the full (uncut)
// eigenbasis of every shell, and each shell's eigen-array, eigenvectors and
// c_d stay on the device for the DM-NRG backward sweep.
//
// chain: the free Wilson chain of calcdens = 3 (NRGcodehandlerClass.cpp:85-91
// switches to ModelNo 3; CodeHandler_ModelSwitch.cpp:377-420, 667-720,
// 940-1000): H_0 is the first site alone (Nsites0 = 1), its thermodynamics
// are taken before the loop at D_0 (NRG_main.cpp:242-255), and iteration N =
// 1 .. nsites-1 adds site N with hopping chi_{N-1}.  Only f_N is carried.
//
// ext: a caller-described model (nrg_sweep_run_model); cfg->model is then
// ignored.
void sweep_run(nrg_ctx* c, const nrg_sweep_config* cfg, bool dm = false, bool chain = false,
               TangentState* tan = nullptr, const nrg_model_desc* ext = nullptr) {
  using clock = std::chrono::steady_clock;
  auto t_begin = clock::now();
  if (ext && (dm || chain || tan))
    throw NrgError(NRG_ERR_ARG, "DM-NRG shells, the free chain and derivatives are built for the built-in models");
  if (!ext && (cfg->model < 0 || cfg->model > 5)) throw NrgError(NRG_ERR_ARG, "unknown model");
  if (chain && (cfg->model == NRG_MODEL_1CH_S || cfg->model == NRG_MODEL_1CH_SZ))
    throw NrgError(NRG_ERR_ARG, "the reference has no free-chain run for the superconducting-lead models");
  if (dm && cfg->model != NRG_MODEL_1CH_QS && cfg->model != NRG_MODEL_2CH_QS)
    throw NrgError(NRG_ERR_ARG, "DM-NRG shells are available for the |Q S> models (one and two channels)");
  if (cfg->nsites < 1 || cfg->ncutoff < 4 || !(cfg->lambda > 1.0)) throw NrgError(NRG_ERR_ARG, "bad sweep parameters");
  if (cfg->precision != NRG_PREC_FP64 && cfg->precision != NRG_PREC_MIXED)
    throw NrgError(NRG_ERR_ARG, "unsupported precision");
  c->precision = cfg->precision;
  c->iters.clear();
  c->opavg_m1.clear();
  std::memset(&c->timing, 0, sizeof(c->timing));
  const int64_t launches0 = c->launches;
  Sweep S;
  S.c = c;
  if (ext) {
    try {
      S.m = make_plugin_model(*ext);
    } catch (const std::invalid_argument& e) {
      throw NrgError(NRG_ERR_ARG, e.what());
    }
  } else {
    S.m = make_model((ModelKind)cfg->model);
  }
  S.cfg = *cfg;
  if (chain) {
    const int nf = (S.m.kind == MODEL_1CHQS || S.m.kind == MODEL_1CHS) ? 1 : 2;
    S.m.op_kind.resize(nf); S.m.op_check.resize(nf); S.m.op_name.resize(nf); S.m.op_avg.resize(nf);
  }
  if (dm && S.m.kind == MODEL_1CHQS) {
    S.m.op_kind = {OP_F_QS, OP_CD_QS};
    S.m.op_check = {CHK_QS_CD, CHK_QS_CD};
    S.m.op_name = {"fN", "cdot1"};
    S.m.op_avg = {0, 0};
  } else if (dm) {
    // Two channels: f_N of both channels (they enter H_N) and c_d.
    S.m.op_kind = {OP_F1_2CH, OP_F2_2CH, OP_CD_2CH};
    S.m.op_check = {CHK_2CH_CD, CHK_2CH_CD, CHK_2CH_CD};
    S.m.op_name = {"fNch1", "fNch2", "cdot1"};
    S.m.op_avg = {0, 0, 0};
  }
  if (dm) {
    c->dm.clear();
    c->dm_rho_valid = false;
    c->dm_drho_valid = false;
    c->dm_lambda = cfg->lambda;
    c->dm_model = S.m.kind;
  }
  const ModelSpec& m = S.m;
  const double eps = cfg->degen_eps > 0 ? cfg->degen_eps : 1.0e-18;
  const double lambda = cfg->lambda;
  const double HLF = 0.5 * (1.0 + 1.0 / lambda);
  const double betabar = 0.727;
  const int nops = (int)m.op_kind.size();
  const int nops_h = m.nops_h;  // old operators entering H_N
  Timer tm(c);
  cudaEvent_t span0, span1;
  CU(cudaEventCreate(&span0));
  CU(cudaEventCreate(&span1));
  struct EvGuard { cudaEvent_t a, b; ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); } } evg{span0, span1};
  CU(cudaEventRecord(span0, c->stream));
  c->flag.ensure(sizeof(int) * 4);
  CU(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
  c->scal.ensure(sizeof(double) * 32);
  c->partial.ensure(sizeof(double) * 64 * 16);
  c->opptr.ensure(sizeof(double*) * 32);

  // H_{-1} (the initial CutStates keeps everything: Ncutoff >= 4 states).
  // calcdens = 3 for the |Q> symmetry: NRG_main.cpp:215-218 turns the chain
  // run back into the Anderson model with every parameter zeroed (U = ed =
  // Gamma = 0): a decoupled four-state impurity beside the chain from site 0
  // on (Nsites0 = 0); its ln 4 is CNRGthermo::dImpValue.
  const bool chain_q = chain && m.kind == MODEL_1CHQ;
  StartState st;
  try {
    st = ext ? make_plugin_start(m)
         : chain && !chain_q ? make_chain_start(m, lambda)
                             : make_start(m, lambda, chain ? 0.0 : cfg->U, chain ? 0.0 : cfg->ed,
                                          chain ? 0.0 : cfg->gamma2_or_B);
  } catch (const std::invalid_argument& e) {
    throw NrgError(NRG_ERR_ARG, e.what());
  }
  if (chain_q) st.ops.resize(nops);
  if (dm) {
    // c_d at H_{-1} is a copy of f (Main_SetH0.cpp:1958-1961); f_ch1 = f_ch2 = d.
    if (m.kind == MODEL_1CHQS) st.ops = {st.ops[0], st.ops[0]};
    else st.ops = {st.ops[0], st.ops[1], st.ops[0]};
    c->dm_hm1_en = st.en;
  }
  S.kept.blk = st.blk;
  // Operators are stored by the blocks of `opsize`; opblock maps a kept
  // block to that structure (empty: the kept array itself).
  std::vector<int> opsize = st.blk.size, opblock;
  std::vector<double> kept_en = st.en;
  for (int o = 0; o < nops; ++o) {
    OpMeta om;
    om.bi = st.ops[o].bi; om.bj = st.ops[o].bj; om.off = st.ops[o].off; om.size = (int64_t)st.ops[o].el.size();
    S.ops.push_back(om);
    DevBuf* b = S.opbuf(0, o);
    b->ensure(sizeof(double) * std::max<int64_t>(om.size, 1));
    h2d(c, b->p, st.ops[o].el.data(), sizeof(double) * om.size);
    if (m.op_avg[o]) {
      std::vector<double> diag(st.en.size(), 0.0);
      for (size_t k = 0; k < st.ops[o].bi.size(); ++k) {
        const int b = st.ops[o].bi[k], n = st.blk.size[b];
        if (b != st.ops[o].bj[k]) continue;
        for (int x = 0; x < n; ++x) diag[st.blk.offset[b] + x] = st.ops[o].el[st.ops[o].off[k] + (int64_t)x * n + x];
      }
      c->opavg_m1.push_back(opavg_host(st.blk, st.en, diag, m.totalS, betabar));
    }
  }

  // Tangents at H_{-1}: its levels are linear in eps_d, U and B (no shift is
  // applied to them), its operators do not depend on the parameters, and
  // Gamma enters through chi_{-1} at iteration 0.
  const bool fullvec = dm || tan;
  if (tan) {
    if (chain || (m.kind != MODEL_1CHQS && m.kind != MODEL_1CHQSZ) || (dm && m.kind != MODEL_1CHQS))
      throw NrgError(NRG_ERR_ARG,
                     "derivatives are built for the one-channel |Q S> and |Q Sz> Anderson sweeps "
                     "(with DM-NRG shells: |Q S>)");
    const StartState s0 = make_start(m, lambda, 0.0, 0.0, 0.0);
    const StartState sd[3] = {make_start(m, lambda, 0.0, 1.0, 0.0), make_start(m, lambda, 1.0, 0.0, 0.0),
                              make_start(m, lambda, 0.0, 0.0, 1.0)};
    tan->params[0] = cfg->ed; tan->params[1] = cfg->U; tan->params[2] = cfg->gamma1; tan->params[3] = cfg->gamma2_or_B;
    tan->dthermo.clear(); tan->dopavg.clear(); tan->dlmin.clear();
    for (int p = 0; p < TangentState::NP; ++p) {
      std::vector<double> de(st.en.size(), 0.0);
      if (p != 2)
        for (size_t k = 0; k < de.size(); ++k) de[k] = sd[p == 3 ? 2 : p].en[k] - s0.en[k];
      tan->dEk[p][0].ensure(sizeof(double) * std::max<size_t>(de.size(), 1));
      h2d(c, tan->dEk[p][0].p, de.data(), sizeof(double) * de.size());
      for (int o = 0; o < nops; ++o) {
        tan->dops[p][0][o].ensure(sizeof(double) * std::max<int64_t>(S.ops[o].size, 1));
        CU(cudaMemsetAsync(tan->dops[p][0][o].p, 0, sizeof(double) * std::max<int64_t>(S.ops[o].size, 1), c->stream));
      }
    }
  }
  int tcur = 0;  // which tangent ping-pong buffer holds the current tangents

  // The chain: Wilson's (SetChainWilson: e_N = 0) or the caller's
  // (nrg_set_chain); iteration N uses hop(N-1) (chi_{-1} at N = 0) and
  // e_N = onsite(N) (NRG_main.cpp:198, 402-413).
  const bool custom = !c->chain_chi.empty();
  if (custom && (int)c->chain_chi.size() < cfg->nsites)
    throw NrgError(NRG_ERR_ARG, "the chain set with nrg_set_chain is shorter than nsites");
  auto hop = [&](int n) { return custom ? c->chain_chi[n] : chin(lambda, n); };
  auto onsite = [&](int n) { return custom ? c->chain_en[n] : 0.0; };
  const bool alam = !custom || c->chain_alambda;
  double chi[2] = {chi_m1(lambda, chain ? 0.0 : cfg->gamma1, alam), 0.0};
  if (m.nchan == 2) chi[1] = chi_m1(lambda, chain ? 0.0 : cfg->gamma2_or_B, alam);
  double eN = onsite(0);
  int N0 = 0;
  if (chain && !chain_q) {
    // chi_m1 = chiN(0) for every channel; H_0 is recorded as iteration 0 with
    // the thermodynamics CalcThermo takes before the loop, at
    // D = HLF Lambda^(-(Nsites0-2)/2) = D_0.
    chi[0] = hop(0);
    chi[1] = m.nchan == 2 ? hop(0) : 0.0;
    IterResult R;
    R.params = {lambda, chi[0], chi[1], eN};
    R.qn = st.blk.qn; R.bsize = st.blk.size; R.kept_bsize = st.blk.size;
    R.en = st.en; R.nkept = st.blk.nstates();
    R.thermo = thermo_host(st.blk, st.en, m.totalS, lambda, HLF * std::pow(lambda, 0.5), betabar);
    c->iters.push_back(std::move(R));
    N0 = 1;
  }

  // |S> model with superconducting leads: Delta_SC enters H_N unscaled at
  // N = 0 and as ScaleFactor(N-1) * Delta_SC = Lambda^((N-1)/2) / HLF *
  // Delta_SC after that (NRG_main.cpp:220-227, 276, 414-419).
  const bool sc = m.kind == MODEL_1CHS || m.kind == MODEL_1CHSZ;
  cudaEvent_t it0, it1;
  CU(cudaEventCreate(&it0));
  CU(cudaEventCreateWithFlags(&it1, c->shared_gpu ? cudaEventBlockingSync : cudaEventDefault));
  EvGuard itg{it0, it1};
  for (int N = N0; N < cfg->nsites; ++N) {
    const auto t_iter = clock::now();
    CU(cudaEventRecord(it0, c->stream));
    IterResult R;
    eN = onsite(N);
    const double delta = !sc ? 0.0 : (N == 0 ? cfg->delta_sc
                                             : std::pow(lambda, 0.5 * (double)(N - 1)) / HLF * cfg->delta_sc);
    R.params = {lambda, chi[0], sc ? delta : chi[1], eN};
    const double DN = HLF * std::pow(lambda, (-(N - 1) / 2.0));
    // ---------------- BuildBasis + tables (host)
    Basis B;
    build_basis(m, S.kept.blk, B);
    HNTables tabs;
    build_hn_tables(m, B, tabs);
    const int nb = B.blk.nblocks();
    std::vector<double> st_eold(B.stcf.size());
    for (size_t g = 0; g < B.stcf.size(); ++g) st_eold[g] = kept_en[B.stcf[g]];
    std::vector<const double*> hops(8, nullptr);
    for (int o = 0; o < nops; ++o) hops[o] = S.opbuf(S.cur, o)->as<double>();
    AsmTables AT = prepare_assembly(c, m, B, tabs, st_eold, S.ops, opsize, nops_h, hops, lambda, chi, eN,
                                    opblock.empty() ? nullptr : &opblock, delta);
    EigPlan& P = AT.P;
    std::vector<int>& order = AT.order;
    char* mb = c->meta.as<char>();
    const size_t o_order = AT.o_order, o_bsize = AT.o_bsize, o_hoff = AT.o_hoff, o_soff = AT.o_soff,
                 o_sb = AT.o_sb, o_bq = AT.o_bq;
    AssembleArgs& aa = AT.aa;
    cudaEvent_t ta = tm.start();
    launch_assemble(aa, P.nstates, (const int*)(mb + o_sb), (const int*)(mb + AT.o_ri), c->stream);
    c->launches++;
    tm.stop(ta, &c->timing.assemble_ms);
    // ---------------- tridiagonalization + eigenvalues
    run_tridiag_and_bisect(c, tm, P, order, (const int*)(mb + o_order), (const int*)(mb + o_bsize),
                           (const int64_t*)(mb + o_hoff), (const int*)(mb + o_soff), (const int*)(mb + o_sb));
    // ---------------- SetE0zero / SetDegen / Ecut / Kept / CutStates bookkeeping
    cudaEvent_t tc = tm.start();
    CutArgs ca{};
    ca.nstates = P.nstates; ca.ev = c->ev.as<double>(); ca.en = c->en.as<double>(); ca.ncutoff = cfg->ncutoff; ca.eps = eps;
    ca.out_scalars = c->scal.as<double>(); ca.flag = c->flag.as<int>();
    launch_cut(ca, c->stream);
    std::vector<int> keptb(nb);
    BlockStatsArgs bs{};
    bs.nblocks = nb; bs.bsize = aa.bsize; bs.soff = aa.bstate; bs.en = c->en.as<double>(); bs.scalars = ca.out_scalars;
    bs.kept = c->red.as<int>() + 4;
    launch_block_stats(bs, c->stream);
    ThermoArgs th{};
    std::vector<double> betas(4);
    for (int nc = 1; nc <= 4; ++nc) betas[nc - 1] = betabar * std::pow(lambda, (nc - 4) / (2.0 * 4));
    th.bq = (const double*)(mb + o_bq); th.en = c->en.as<double>(); th.totalS = m.totalS ? 1 : 0;
    for (int t = 0; t < 4; ++t) th.beta[t] = betas[t];
    th.out = c->scal.as<double>() + 8;
    launch_thermo(th, (const int*)(mb + o_sb), P.nstates, c->partial.as<double>(), c->stream);
    c->launches += 4;
    std::vector<double> scal(20);
    R.en.resize(P.nstates);
    d2h(c, scal.data(), c->scal.p, sizeof(double) * 20);
    d2h(c, keptb.data(), bs.kept, sizeof(int) * nb);
    d2h(c, R.en.data(), c->en.p, sizeof(double) * P.nstates);
    tm.stop(tc, &c->timing.cut_ms);
    stream_wait(c);
    check_flag(c);
    R.emin = scal[0]; R.ecut = scal[1]; R.nkept = (int)scal[2];
    R.qn = B.blk.qn; R.bsize = P.bsize;
    for (int t = 0; t < 4; ++t) {
      const double Z = scal[8 + 3 * t], s1 = scal[8 + 3 * t + 1], sE = scal[8 + 3 * t + 2];
      R.thermo.push_back(betas[t]);
      R.thermo.push_back(DN / betas[t]);
      R.thermo.push_back((s1 - 0.0 * s1) / Z);
      R.thermo.push_back(betas[t] * (sE / Z) + std::log(Z));
    }
    // ---------------- new kept array (CutStates)
    Kept K;
    K.blk.nqn = 2;
    std::vector<double> new_kept_en;
    for (int b = 0; b < nb; ++b) {
      if (keptb[b] <= 0) continue;
      K.blk.push(&B.blk.qn[2 * b], keptb[b]);
      K.src.push_back(b);
      for (int x = 0; x < keptb[b]; ++x) new_kept_en.push_back(R.en[P.soff[b] + x]);
    }
    for (int x : K.blk.size) R.kept_bsize.push_back(x);
    // ---------------- kept eigenvectors
    P.nvec.assign(nb, 0);
    for (int b = 0; b < nb; ++b) P.nvec[b] = fullvec ? P.bsize[b] : keptb[b];
    // eigenvalues for clustering: shifted energies have the same gaps
    run_vectors(c, tm, P, R.en, aa.bsize, aa.hoff, aa.bstate);
    // ---------------- UpdateMatrices
    UpdatePlan U;
    Kept Kfull;  // UpdateBefCut (and the tangent pass): the layout of every state of H_N
    if (fullvec) {
      Kfull.blk = B.blk;
      for (int b = 0; b < nb; ++b) Kfull.src.push_back(b);
    }
    plan_update(U, m, B, P, fullvec ? Kfull : K, S.ops, opblock.empty() ? nullptr : &opblock, &opsize,
                fullvec ? &keptb : nullptr);
    std::vector<OpMeta>& newops = U.newops;
    const int nk = K.blk.nblocks();
    int nxt = 1 - S.cur;
    std::vector<double*> newptr(8, nullptr), oldptr(8, nullptr);
    for (int o = 0; o < nops; ++o) {
      DevBuf* b = S.opbuf(nxt, o);
      b->ensure(sizeof(double) * std::max<int64_t>(newops[o].size, 1));
      newptr[o] = b->as<double>();
      oldptr[o] = S.opbuf(S.cur, o)->as<double>();
      if (fullvec && m.op_kind[o] != OP_CD_QS && m.op_kind[o] != OP_CD_2CH)  // only the kept part is computed
        CU(cudaMemsetAsync(newptr[o], 0, sizeof(double) * newops[o].size, c->stream));
    }
    Packer& up = U.up;
    U.o_old = up.add(oldptr); U.o_new = up.add(newptr);
    size_t o_ken = up.add(new_kept_en);
    // kept-state tables for the operator averages
    std::vector<int> kstate_block, ksz = K.blk.size, koff = K.blk.offset;
    for (int i = 0; i < nk; ++i) for (int x = 0; x < K.blk.size[i]; ++x) kstate_block.push_back(i);
    std::vector<int64_t> diag_off;
    std::vector<int> avg_ops;
    for (int o = 0; o < nops; ++o) if (m.op_avg[o]) avg_ops.push_back(o);
    std::vector<const double*> avgptr;
    for (int o : avg_ops) {
      avgptr.push_back(newptr[o]);
      for (int i = 0; i < nk; ++i) {  // full layout: the kept block's own block of H_N
        const int bi = fullvec ? K.src[i] : i;
        const int k = newops[o].find(bi, bi);
        diag_off.push_back(k >= 0 ? newops[o].off[k] : -1);
      }
    }
    std::vector<int> kld(nk);  // row stride of each kept block's diagonal operator block
    for (int i = 0; i < nk; ++i) kld[i] = fullvec ? P.bsize[K.src[i]] : K.blk.size[i];
    size_t o_ksb = up.add(kstate_block), o_ksz = up.add(ksz), o_koff = up.add(koff), o_doff = up.add(diag_off),
           o_avp = up.add(avgptr), o_kq = up.add(K.blk.qn), o_kld = up.add(kld);
    launch_update_plan(c, tm, U);
    char* ub = U.ub;
    // ---------------- CalcStuff: operator averages over the kept states
    cudaEvent_t to = tm.start();
    OpDiagArgs od{};
    od.nblocks = nk; od.ksize = (const int*)(ub + o_ksz); od.koff = (const int*)(ub + o_koff);
    od.kld = (const int*)(ub + o_kld);
    od.ken = (const double*)(ub + o_ken); od.bq = (const double*)(ub + o_kq); od.totalS = m.totalS ? 1 : 0;
    od.beta = betabar; od.nops = (int)avg_ops.size(); od.ops = (const double* const*)(ub + o_avp);
    od.diag_off = (const int64_t*)(ub + o_doff); od.out = c->scal.as<double>() + 24;
    launch_opdiag(od, (const int*)(ub + o_ksb), (int)kstate_block.size(), c->partial.as<double>(), c->stream);
    c->launches += 2;
    std::vector<double> avg(8);
    d2h(c, avg.data(), c->scal.as<double>() + 24, sizeof(double) * 8);
    tm.stop(to, &c->timing.cut_ms);
    stream_wait(c);
    check_flag(c);
    tm.collect();
    const double Zk = avg[avg_ops.size()];
    for (size_t k = 0; k < avg_ops.size(); ++k) {
      double s = avg[k];
      if (!(std::fabs(Zk) < 1.e-20)) s = s / Zk;
      R.opavg.push_back(s);
    }
    // ---------------- tangents of this iteration (nrg_grad_forward)
    std::unique_ptr<DmShell> shp;
    if (dm) shp = std::make_unique<DmShell>();
    if (tan) {
      TangentState& TS = *tan;
      const int NP = TangentState::NP;
      TS.nops = (int)avg_ops.size();
      // host tables: kept states, coupling-matrix offsets, pointer tables
      std::vector<int> kept_state;
      for (int i = 0; i < nk; ++i)
        for (int x = 0; x < K.blk.size[i]; ++x) kept_state.push_back(P.soff[K.src[i]] + x);
      // Eigenvector tangents: of the kept states; of every state when the
      // shell is kept for DM-NRG (its rotations and c_d use them all).
      const std::vector<int>& ccols = dm ? P.bsize : keptb;
      std::vector<int64_t> coff(nb);
      int64_t csz = 0;
      for (int b = 0; b < nb; ++b) { coff[b] = csz; csz += (int64_t)P.bsize[b] * ccols[b]; }
      int gs = 0;
      for (int g = 1; g < P.nstates; ++g) if (R.en[g] < R.en[gs]) gs = g;
      const int nkept = (int)kept_state.size();
      TS.deold.ensure(sizeof(double) * std::max(P.nstates, 1));
      for (DevBuf* b : {&TS.dH, &TS.T1, &TS.dHt}) b->ensure(sizeof(double) * std::max<int64_t>(P.hsize, 1));
      TS.C.ensure(sizeof(double) * std::max<int64_t>(csz, 1));
      TS.dZ.ensure(sizeof(double) * std::max<int64_t>(P.ysize, 1));
      TS.dZt.ensure(sizeof(double) * std::max<int64_t>(P.ysize, 1));
      TS.dlam.ensure(sizeof(double) * std::max(P.nstates, 1));
      TS.dEall.ensure(sizeof(double) * std::max(P.nstates, 1));
      for (int r = 0; r < 3; ++r)
        for (int o = 0; o < nops; ++o) TS.tmp[r][o].ensure(sizeof(double) * std::max<int64_t>(newops[o].size, 1));
      for (int p = 0; p < NP; ++p) {
        TS.dEk[p][1 - tcur].ensure(sizeof(double) * std::max(nkept, 1));
        for (int o = 0; o < nops; ++o)
          TS.dops[p][1 - tcur][o].ensure(sizeof(double) * std::max<int64_t>(newops[o].size, 1));
      }
      // iteration 0, Gamma: chi_{-1} is proportional to sqrt(Gamma), so the
      // coupling's tangent is the primal coupling over 2 Gamma
      const bool gamma_term = N == 0 && !(std::fabs(cfg->gamma1) == 0.0);
      if (gamma_term)
        for (int o = 0; o < nops_h; ++o) {
          TS.gscaled[o].ensure(sizeof(double) * std::max<int64_t>(S.ops[o].size, 1));
          launch_tan_scale(S.opbuf(S.cur, o)->as<double>(), 0.5 / cfg->gamma1, S.ops[o].size,
                           TS.gscaled[o].as<double>(), c->stream);
        }
      // pointer tables: per parameter the tangent old operators (8) and new
      // ones (8), then the three rotation outputs (8 each), the Gamma-scaled
      // couplings (8), and per parameter the averaged operators' tangents (8)
      std::vector<const double*> ptrs;
      for (int p = 0; p < NP; ++p) {
        for (int o = 0; o < 8; ++o) ptrs.push_back(o < nops ? TS.dops[p][tcur][o].as<double>() : nullptr);
        for (int o = 0; o < 8; ++o) ptrs.push_back(o < nops ? TS.dops[p][1 - tcur][o].as<double>() : nullptr);
      }
      for (int r = 0; r < 3; ++r)
        for (int o = 0; o < 8; ++o) ptrs.push_back(o < nops ? TS.tmp[r][o].as<double>() : nullptr);
      for (int o = 0; o < 8; ++o) ptrs.push_back(gamma_term && o < nops_h ? TS.gscaled[o].as<double>() : nullptr);
      for (int p = 0; p < NP; ++p)
        for (int k = 0; k < 8; ++k)
          ptrs.push_back(k < (int)avg_ops.size() ? TS.dops[p][1 - tcur][avg_ops[k]].as<double>() : nullptr);
      Packer tp;
      const size_t o_ptr = tp.add(ptrs), o_kst = tp.add(kept_state), o_coff = tp.add(coff), o_nkeep = tp.add(ccols),
                   o_stcf = tp.add(B.stcf);
      TS.tabs.ensure(tp.host.size() + 256);
      h2d(c, TS.tabs.p, tp.host.data(), tp.host.size());
      char* tb = TS.tabs.as<char>();
      const double* const* dptr = (const double* const*)(tb + o_ptr);
      auto tab_old = [&](int p) { return dptr + 16 * p; };
      auto tab_tmp = [&](int r) { return dptr + 16 * NP + 8 * r; };
      const double* const* tab_gamma = dptr + 16 * NP + 24;
      auto tab_avg = [&](int p) { return dptr + 16 * NP + 32 + 8 * p; };
      // the eigen-derivative GEMMs of every block (the same for all parameters)
      GemmPlan G1, G2, G3, G4;
      for (int b = 0; b < nb; ++b) {
        const int n = P.bsize[b], kb = ccols[b];
        const int64_t h = P.hoff[b], y = P.yoff[b];
        double* Zb = c->Z.as<double>() + y;
        double* Ztb = c->Zt.as<double>() + y;
        G1.add(GemmJob{n, n, n, 0, TS.dH.as<double>() + h, n, Ztb, n, TS.T1.as<double>() + h, n});
        G2.add(GemmJob{n, n, n, 0, Zb, n, TS.T1.as<double>() + h, n, TS.dHt.as<double>() + h, n});
        if (kb == 0) continue;
        G3.add(GemmJob{n, kb, n, 0, Ztb, n, TS.C.as<double>() + coff[b], kb, TS.dZt.as<double>() + y, n});
        G4.add(GemmJob{kb, n, n, 1, TS.C.as<double>() + coff[b], kb, Zb, n, TS.dZ.as<double>() + y, n});
      }
      TS.part.ensure(sizeof(double) * tan_partial_doubles());
      TS.out.ensure(sizeof(double) * TanSumArgs::kMaxOut * NP + 64);
      std::vector<double> sums((size_t)TanSumArgs::kMaxOut * NP), dl(NP);
      if (dm) {
        shp->ntan = NP;
        shp->den.assign((size_t)NP * P.nstates, 0.0);
      }
      for (int p = 0; p < NP; ++p) {
        // dH_N: the assembly on the tangents of the old energies and operators
        launch_tan_gather(TS.dEk[p][tcur].as<double>(), (const int*)(tb + o_stcf), P.nstates, TS.deold.as<double>(),
                          c->stream);
        AssembleArgs a2 = aa;
        a2.H = TS.dH.as<double>(); a2.st_eold = TS.deold.as<double>(); a2.eN = 0.0;
        a2.ops = (gamma_term && p == 2) ? tab_gamma : tab_old(p);
        launch_assemble(a2, P.nstates, (const int*)(mb + o_sb), (const int*)(mb + AT.o_ri), c->stream);
        run_gemm_plan(c, G1);
        run_gemm_plan(c, G2);
        TanEigArgs te{};
        te.bsize = aa.bsize; te.soff = aa.bstate; te.hoff = aa.hoff; te.dHt = TS.dHt.as<double>();
        te.ev = c->ev.as<double>(); te.nkeep = (const int*)(tb + o_nkeep); te.coff = (const int64_t*)(tb + o_coff);
        te.C = TS.C.as<double>(); te.dlam = TS.dlam.as<double>(); te.degen_tol = 1e-10;
        launch_tan_eig(te, nb, c->stream);
        run_gemm_plan(c, G3);
        run_gemm_plan(c, G4);
        launch_tan_shift(TS.dlam.as<double>(), P.nstates, gs, TS.dEall.as<double>(), (const int*)(tb + o_kst), nkept,
                         TS.dEk[p][1 - tcur].as<double>(), c->stream);
        if (dm) {  // the shell's tangents: every eigenvector's and every energy's
          shp->dZ[p].ensure(sizeof(double) * std::max<int64_t>(P.ysize, 1));
          CU(cudaMemcpyAsync(shp->dZ[p].p, TS.dZ.p, sizeof(double) * P.ysize, cudaMemcpyDeviceToDevice, c->stream));
          d2h(c, shp->den.data() + (size_t)p * P.nstates, TS.dEall.p, sizeof(double) * P.nstates);
        }
        // dO_new = dZ_I F Z_J^T + Z_I F dZ_J^T + Z_I dF Z_J^T
        for (int r = 0; r < 3; ++r)
          for (int o = 0; o < nops; ++o)
            CU(cudaMemsetAsync(TS.tmp[r][o].p, 0, sizeof(double) * newops[o].size, c->stream));
        const double* const* old_primal = (const double* const*)(ub + U.o_old);
        UpdateInputs u1{TS.dZ.as<double>(), c->Zt.as<double>(), old_primal, (double* const*)tab_tmp(0), true};
        UpdateInputs u2{c->Z.as<double>(), TS.dZt.as<double>(), old_primal, (double* const*)tab_tmp(1), true};
        UpdateInputs u3{c->Z.as<double>(), c->Zt.as<double>(), tab_old(p), (double* const*)tab_tmp(2), false};
        launch_update_plan(c, tm, U, &u1);
        launch_update_plan(c, tm, U, &u2);
        launch_update_plan(c, tm, U, &u3);
        for (int o = 0; o < nops; ++o)
          launch_tan_axpy3(TS.tmp[0][o].as<double>(), TS.tmp[1][o].as<double>(), TS.tmp[2][o].as<double>(), 1.0,
                           newops[o].size, TS.dops[p][1 - tcur][o].as<double>(), c->stream);
        if (dm) {
          const int64_t ncd = newops[nops_h].size;
          shp->dcd[p].ensure(sizeof(double) * std::max<int64_t>(ncd, 1));
          CU(cudaMemcpyAsync(shp->dcd[p].p, TS.dops[p][1 - tcur][nops_h].p, sizeof(double) * ncd,
                             cudaMemcpyDeviceToDevice, c->stream));
        }
        // weighted sums of the thermodynamics and operator-average tangents
        TanSumArgs ts{};
        ts.nstates = P.nstates; ts.state_block = (const int*)(mb + o_sb); ts.bq = (const double*)(mb + o_bq);
        ts.en = c->en.as<double>(); ts.dE = TS.dEall.as<double>(); ts.totalS = m.totalS ? 1 : 0;
        for (int t = 0; t < 4; ++t) ts.beta[t] = betas[t];
        ts.nkept = nkept; ts.nkblocks = nk; ts.kstate_block = (const int*)(ub + o_ksb); ts.koff = (const int*)(ub + o_koff);
        ts.kld = (const int*)(ub + o_kld); ts.kbq = (const double*)(ub + o_kq); ts.ken = (const double*)(ub + o_ken);
        ts.dEk = TS.dEk[p][1 - tcur].as<double>(); ts.betabar = betabar; ts.nops = (int)avg_ops.size();
        ts.ops = (const double* const*)(ub + o_avp); ts.dops = tab_avg(p); ts.diag_off = (const int64_t*)(ub + o_doff);
        launch_tan_sums(ts, TS.part.as<double>(), TS.out.as<double>() + (size_t)p * TanSumArgs::kMaxOut, c->stream);
        d2h(c, &dl[p], TS.dlam.as<double>() + gs, sizeof(double));
        c->launches += 14;
      }
      d2h(c, sums.data(), TS.out.p, sizeof(double) * sums.size());
      CU(cudaStreamSynchronize(c->stream));
      check_flag(c);
      tm.collect();
      // derivatives of the reported values from the sums (CalcSuscep,
      // CalcEntropy and CalcOpAvg differentiated: d e^{-beta E} = -beta e^{-beta E} dE)
      for (int p = 0; p < NP; ++p) {
        const double* q = sums.data() + (size_t)p * TanSumArgs::kMaxOut;
        for (int t = 0; t < 4; ++t) {
          const double Z = scal[8 + 3 * t], s1 = scal[8 + 3 * t + 1], sE = scal[8 + 3 * t + 2], b = betas[t];
          const double dZ = -b * q[3 * t], ds1 = -b * q[3 * t + 1], dsE = q[3 * t] - b * q[3 * t + 2];
          TS.dthermo.push_back(0.0);                                         // beta
          TS.dthermo.push_back(0.0);                                         // T
          TS.dthermo.push_back(ds1 / Z - s1 * dZ / (Z * Z));                 // T chi
          TS.dthermo.push_back(b * (dsE / Z - sE * dZ / (Z * Z)) + dZ / Z);  // S
        }
        const double Zk = avg[avg_ops.size()];
        const double dZk = -betabar * q[TanSumArgs::kMaxOut - 1];
        for (size_t k = 0; k < avg_ops.size(); ++k) {
          const double SO = avg[k], dSO = q[12 + 2 * k] - betabar * q[12 + 2 * k + 1];
          TS.dopavg.push_back(std::fabs(Zk) < 1.e-20 ? 0.0 : dSO / Zk - SO * dZk / (Zk * Zk));
        }
        TS.dlmin.push_back(dl[p]);
      }
      tcur = 1 - tcur;
    }
    // ---------------- DM-NRG shell (SaveArrays, NRGcodehandlerClass.cpp:887-932)
    if (dm) {
      std::unique_ptr<DmShell> sh = std::move(shp);
      sh->bsize = P.bsize; sh->boff = P.soff; sh->qn = B.blk.qn; sh->en = R.en;
      sh->kept.resize(P.nstates);
      for (int g = 0; g < P.nstates; ++g) sh->kept[g] = R.en[g] <= R.ecut ? 1 : 0;
      sh->kept_src = K.src;
      sh->cd = newops[nops_h];
      sh->zoff = P.yoff; sh->zsize = P.ysize;
      sh->Z.ensure(sizeof(double) * std::max<int64_t>(P.ysize, 1));
      CU(cudaMemcpyAsync(sh->Z.p, c->Z.p, sizeof(double) * P.ysize, cudaMemcpyDeviceToDevice, c->stream));
      sh->cdel.ensure(sizeof(double) * std::max<int64_t>(newops[nops_h].size, 1));
      CU(cudaMemcpyAsync(sh->cdel.p, newptr[nops_h], sizeof(double) * newops[nops_h].size, cudaMemcpyDeviceToDevice,
                         c->stream));
      sh->basis = std::move(B);
      c->dm.push_back(std::move(sh));
      opsize = P.bsize;
      opblock = K.src;
    } else if (tan) {  // operators stay in the full layout (kept part computed)
      opsize = P.bsize;
      opblock = K.src;
    } else {
      opsize = K.blk.size;
    }
    // ---------------- next iteration
    S.kept = K;
    kept_en = new_kept_en;
    S.ops = newops;
    S.cur = nxt;
    for (int ich = 0; ich < m.nchan; ++ich) chi[ich] = hop(N);
    CU(cudaEventRecord(it1, c->stream));
    CU(cudaEventSynchronize(it1));
    float it_ms = 0.f;
    CU(cudaEventElapsedTime(&it_ms, it0, it1));
    R.device_ms = it_ms;
    R.wall_ms = std::chrono::duration<double, std::milli>(clock::now() - t_iter).count();
    c->iters.push_back(std::move(R));
  }
  CU(cudaEventRecord(span1, c->stream));
  CU(cudaEventSynchronize(span1));
  float span_ms = 0.f;
  CU(cudaEventElapsedTime(&span_ms, span0, span1));
  c->timing.device_ms = span_ms;
  c->timing.kernel_launches = c->launches - launches0;
  c->timing.total_ms = std::chrono::duration<double, std::milli>(clock::now() - t_begin).count();
}

// nrg_grad_forward: the sweep with the tangent pass, then the absolute
// ground-state energy sum_{M<=N} D_M E_min,M (H_N is built from energies
// already shifted by the earlier E_min and rescaled, so the shifts add up in
// absolute units) and its tangents.
//
// dm: the sweep keeps the DM-NRG shells (nrg_sweep_run_dm) with their
// tangents (nrg_grad_forward_dm).
void grad_forward_impl(nrg_ctx* c, const nrg_sweep_config* cfg, bool dm = false) {
  if (!c->tan) c->tan = new TangentState();
  c->dm_drhow.clear();
  sweep_run(c, cfg, dm, false, c->tan);
  const int NP = TangentState::NP;
  const int ni = (int)c->iters.size();
  const double lambda = cfg->lambda, HLF = 0.5 * (1.0 + 1.0 / lambda);
  c->grad_egs.assign(ni, 0.0);
  c->grad_degs.assign((size_t)ni * NP, 0.0);
  c->grad_demin = c->tan->dlmin;
  double e = 0.0;
  std::vector<double> de(NP, 0.0);
  for (int n = 0; n < ni; ++n) {
    const double DN = HLF * std::pow(lambda, (-(n - 1) / 2.0));
    e += DN * c->iters[n].emin;
    c->grad_egs[n] = e;
    for (int k = 0; k < NP; ++k) {
      de[k] += DN * c->tan->dlmin[(size_t)n * NP + k];
      c->grad_degs[(size_t)n * NP + k] = de[k];
    }
  }
}

// ------------------------------------------------------------------ DM-NRG
// CalcDN (CalcDN.cpp) with z = 1: the energy scale of shell N.
double calc_dn(double L, int N) {
  const double hlf = L > 0.0 ? 0.5 * (1.0 + (1.0 / L)) : 1.0;
  return hlf * std::pow(L, (-(N - 1) / 2.0) - 1.0 + 1.0);
}

struct DmResolved {
  double temp, tempbar0, betabar, bbroad, twindow, broadtemp, site_dim;
};

// The temperature logic of DM_NRG.cpp:100-121: Mtemp < Nsitesmax-1 puts T at
// D_Mtemp/betabar (and SetRhoNmax gets T/D_Mtemp); otherwise T is
// D_{Nsitesmax+199}/betabar, or the caller's positive temp, and SetRhoNmax
// gets T/D_{Nsitesmax-1}.
DmResolved dm_resolve(const nrg_dm_params* p, double L, int nsites) {
  if (!p) throw NrgError(NRG_ERR_ARG, "DM-NRG parameters are NULL");
  if (!(p->betabar > 0.0) || !(p->bbroad > 0.0) || !(p->broadtemp > 0.0) || !(p->site_dim > 0.0) ||
      p->twindow < 0.0)
    throw NrgError(NRG_ERR_ARG, "betabar, bbroad, broadtemp and site_dim must be positive");
  DmResolved r{0, 0, p->betabar, p->bbroad, p->twindow, p->broadtemp, p->site_dim};
  if (p->mtemp >= 0 && p->mtemp < nsites - 1) {
    const double DM = calc_dn(L, p->mtemp);
    r.temp = DM / p->betabar;
    r.tempbar0 = r.temp / DM;
  } else {
    r.temp = p->temp > 0.0 ? p->temp : calc_dn(L, nsites + 199) / p->betabar;
    r.tempbar0 = r.temp / calc_dn(L, nsites - 1);
  }
  return r;
}

// (2S+1)-weighted Boltzmann sums over all / discarded states of a shell
// (PartitionFunc / PartitionFuncDisc, NRGarrayClass.cpp:997-1060).
double dm_partition(const DmShell& s, double beta, bool disc_only) {
  double sum = 0.0;
  for (size_t b = 0; b < s.bsize.size(); ++b) {
    const double Si = s.qn[2 * b + 1];
    for (int i = s.boff[b]; i < s.boff[b] + s.bsize[b]; ++i)
      if (!disc_only || !s.kept[i]) sum += (2.0 * Si + 1.0) * std::exp(-beta * s.en[i]);
  }
  return sum;
}


// The tangent of dm_partition along parameter k of the shells' tangents.
double dm_partition_tangent(const DmShell& s, double beta, bool disc_only, int k) {
  const double* dE = s.den.data() + (size_t)k * s.en.size();
  double sum = 0.0;
  for (size_t b = 0; b < s.bsize.size(); ++b) {
    const double Si = s.qn[2 * b + 1];
    for (int i = s.boff[b]; i < s.boff[b] + s.bsize[b]; ++i)
      if (!disc_only || !s.kept[i]) sum += (2.0 * Si + 1.0) * (-beta * dE[i]) * std::exp(-beta * s.en[i]);
  }
  return sum;
}

// DM_NRG_SetRhoNmax + (RotateMatrix, DM_NRG_CalcRhoN_withSU2) per shell, FDM.
void dm_backprop_impl(nrg_ctx* c, const nrg_dm_params* prm, double* rho_trace) {
  if (c->dm.empty()) throw NrgError(NRG_ERR_STATE, "no DM-NRG shells: run nrg_sweep_run_dm first");
  const int nsh = (int)c->dm.size(), Nmax = nsh - 1;
  const double L = c->dm_lambda;
  const DmResolved p = dm_resolve(prm, L, nsh);
  Timer tm(c);
  cudaEvent_t t0 = tm.start();
  // Partition sums (DM_NRG.cpp:201-257).
  double TempBar = p.temp / calc_dn(L, Nmax - 1);
  double ZTot = dm_partition(*c->dm[Nmax], 1.0 / TempBar, false);
  for (int N = Nmax - 1; N >= 0; --N) {
    TempBar = p.temp / calc_dn(L, N - 1);
    ZTot += dm_partition(*c->dm[N], 1.0 / TempBar, true) * std::pow(p.site_dim, Nmax - N);
  }
  // Tangents (shells of nrg_grad_forward_dm): d ln ZTot per parameter, with
  // d exp(-beta E) = -beta dE exp(-beta E).
  bool tg = true;
  for (const auto& sp : c->dm) tg = tg && sp->ntan == DmTan::NP;
  double dlogz[DmTan::NP] = {0.0, 0.0, 0.0, 0.0};
  if (tg) {
    for (int k = 0; k < DmTan::NP; ++k) {
      TempBar = p.temp / calc_dn(L, Nmax - 1);
      double dz = dm_partition_tangent(*c->dm[Nmax], 1.0 / TempBar, false, k);
      for (int N = Nmax - 1; N >= 0; --N) {
        TempBar = p.temp / calc_dn(L, N - 1);
        dz += dm_partition_tangent(*c->dm[N], 1.0 / TempBar, true, k) * std::pow(p.site_dim, Nmax - N);
      }
      dlogz[k] = dz / ZTot;
    }
  }
  {  // SetRhoNmax (DM_NRG_SetRhoNmax.cpp:9-126): diagonal Boltzmann weights.
    DmShell& s = *c->dm[Nmax];
    const double beta = std::fabs(p.tempbar0) < 1.e-20 ? 1.0e10 : 1.0 / p.tempbar0;
    std::vector<double> R((size_t)std::max<int64_t>(s.zsize, 1), 0.0);
    for (size_t b = 0; b < s.bsize.size(); ++b) {
      const int n = s.bsize[b];
      for (int i = 0; i < n; ++i) R[s.zoff[b] + (int64_t)i * n + i] = std::exp(-beta * s.en[s.boff[b] + i]) / ZTot;
    }
    s.rho.ensure(sizeof(double) * R.size());
    h2d(c, s.rho.p, R.data(), sizeof(double) * s.zsize);
    s.rrows.assign(s.bsize.size(), 0);
    for (size_t b = 0; b < s.bsize.size(); ++b) {
      const int n = s.bsize[b];
      for (int i = 0; i < n; ++i)
        if (R[s.zoff[b] + (int64_t)i * n + i] != 0.0) s.rrows[b] = i + 1;
    }
    for (int k = 0; tg && k < DmTan::NP; ++k) {  // d rho = rho (-beta dE - d ln ZTot)
      std::vector<double> dR((size_t)std::max<int64_t>(s.zsize, 1), 0.0);
      const double* dE = s.den.data() + (size_t)k * s.en.size();
      for (size_t b = 0; b < s.bsize.size(); ++b) {
        const int n = s.bsize[b];
        for (int i = 0; i < n; ++i) {
          const int64_t q = s.zoff[b] + (int64_t)i * n + i;
          dR[q] = R[q] * (-beta * dE[s.boff[b] + i] - dlogz[k]);
        }
      }
      s.drho[k].ensure(sizeof(double) * dR.size());
      h2d(c, s.drho[k].p, dR.data(), sizeof(double) * s.zsize);
    }
  }
  for (int N = Nmax - 1; N >= 0; --N) {
    DmShell& sN = *c->dm[N];
    DmShell& s1 = *c->dm[N + 1];
    // RotateMatrix: rho~_b = Z_b^T (rho_b Z_b), Z_b rows = eigenvectors.
    const size_t zs = sizeof(double) * std::max<int64_t>(s1.zsize, 1);
    c->T.ensure(2 * zs + 512);
    double* Tm = c->T.as<double>();
    double* rot = (double*)((char*)c->T.p + ((zs + 255) & ~size_t(255)));
    GemmPlan g1, g2;
    // rho_b is zero beyond its leading r x r part (kept x kept, then the
    // discarded states whose Boltzmann weight is not 0), so T = rho Z has r
    // nonzero rows and Z^T T sums over r of them: the same terms in the
    // same order as the full products.
    for (size_t b = 0; b < s1.bsize.size(); ++b) {
      const int n = s1.bsize[b], r = s1.rrows[b];
      const double* Z = s1.Z.as<double>() + s1.zoff[b];
      g1.add(GemmJob{r, n, r, 0, s1.rho.as<double>() + s1.zoff[b], n, Z, n, Tm + s1.zoff[b], n});
      g2.add(GemmJob{n, n, r, 1, Z, n, Tm + s1.zoff[b], n, rot + s1.zoff[b], n});
    }
    run_gemm_plan(c, g1);
    run_gemm_plan(c, g2);
    // Tangents: d rho~ = Z^T (d rho Z + rho dZ) + dZ^T (rho Z), per parameter.
    const size_t zsa = (zs + 255) & ~size_t(255);
    double* U0 = nullptr;
    if (tg) {
      c->dmtan.ensure(2 * DmTan::NP * zsa);
      U0 = c->dmtan.as<double>();
      auto Uk = [&](int k) { return (double*)((char*)U0 + k * zsa); };
      auto Rk = [&](int k) { return (double*)((char*)U0 + (DmTan::NP + k) * zsa); };
      GemmPlan h[4];
      for (int k = 0; k < DmTan::NP; ++k)
        for (size_t b = 0; b < s1.bsize.size(); ++b) {
          const int n = s1.bsize[b], r = s1.rrows[b];
          const int64_t o = s1.zoff[b];
          const double* Z = s1.Z.as<double>() + o;
          const double* dZ = s1.dZ[k].as<double>() + o;
          h[0].add(GemmJob{r, n, r, 0, s1.drho[k].as<double>() + o, n, Z, n, Uk(k) + o, n});
          h[1].add(GemmJob{r, n, r, 0, s1.rho.as<double>() + o, n, dZ, n, Uk(k) + o, n, 1});
          h[2].add(GemmJob{n, n, r, 1, Z, n, Uk(k) + o, n, Rk(k) + o, n});
          h[3].add(GemmJob{n, n, r, 1, dZ, n, Tm + o, n, Rk(k) + o, n, 1});
        }
      for (int q = 0; q < 4; ++q) run_gemm_plan(c, h[q]);
    }
    // Partial trace over the child states (DM_NRG_SetChildSt, SetChildSameType).
    const Basis& B1 = s1.basis;
    const int nbN = (int)sN.bsize.size();
    const ModelSpec ms = make_model((ModelKind)c->dm_model);
    std::vector<std::vector<DmTraceTerm>> per(nbN);
    for (int nb1 = 0; nb1 < B1.blk.nblocks(); ++nb1) {
      const double Si = B1.blk.q(nb1, 1);
      for (const Segment& sg : B1.seg[nb1]) {
        const int fb = sN.kept_src[sg.old_block];
        const double Sold = sN.qn[2 * fb + 1];
        for (int u = 0; u < sg.nsite; ++u) {
          // S of the site state.
          const int t = ms.site.blk.offset[sg.site_block] + u;
          const double St = ms.site.blk.q(ms.site.block_of_state(t), 1);
          double cgf = 0.0;
          for (double Sz = -Si; Sz <= Si; Sz += 1.0) {
            const double x = clebsch(Sold, Sold, St, Sz - Sold, Si, Sz);
            cgf += x * x;
          }
          per[fb].push_back(DmTraceTerm{s1.zoff[nb1], s1.bsize[nb1], sg.offset + u, sg.nsite, sg.count, cgf});
        }
      }
    }
    std::vector<DmTraceTerm> terms;
    std::vector<int> tfirst(nbN), tcount(nbN), nkept(nbN, 0);
    for (int b = 0; b < nbN; ++b) {
      tfirst[b] = (int)terms.size();
      tcount[b] = (int)per[b].size();
      terms.insert(terms.end(), per[b].begin(), per[b].end());
      while (nkept[b] < sN.bsize[b] && sN.kept[sN.boff[b] + nkept[b]]) nkept[b]++;
    }
    Packer pk;
    size_t o_bs = pk.add(sN.bsize), o_so = pk.add(sN.boff), o_ro = pk.add(sN.zoff), o_nk = pk.add(nkept),
           o_tf = pk.add(tfirst), o_tc = pk.add(tcount), o_t = pk.add(terms), o_en = pk.add(sN.en),
           o_kp = pk.add(sN.kept), o_den = tg ? pk.add(sN.den) : 0;
    c->meta.ensure(pk.host.size() + 256);
    h2d(c, c->meta.p, pk.host.data(), pk.host.size());
    char* mb = c->meta.as<char>();
    sN.rho.ensure(sizeof(double) * std::max<int64_t>(sN.zsize, 1));
    TempBar = p.temp / calc_dn(L, N - 1);
    DmTraceArgs ta{};
    ta.bsize = (const int*)(mb + o_bs); ta.soff = (const int*)(mb + o_so); ta.roff = (const int64_t*)(mb + o_ro);
    ta.nkept = (const int*)(mb + o_nk); ta.term_first = (const int*)(mb + o_tf); ta.term_count = (const int*)(mb + o_tc);
    ta.terms = (const DmTraceTerm*)(mb + o_t); ta.rot = rot; ta.en = (const double*)(mb + o_en);
    ta.kept = (const unsigned char*)(mb + o_kp); ta.beta = 1 / TempBar;
    ta.zdisc = ZTot / std::pow(p.site_dim, Nmax - N); ta.rho = sN.rho.as<double>();
    // Nonzero rows of rho_N: the kept states, then the discarded ones whose
    // exp(-beta E) may not underflow (beta E <= 800; exp gives 0 beyond
    // 745.2), a prefix of each block as the energies ascend.
    sN.rrows.assign(nbN, 0);
    for (int b = 0; b < nbN; ++b) {
      int r = nkept[b];
      if (ta.zdisc != 0.0)
        for (int i = nkept[b]; i < sN.bsize[b]; ++i)
          if (ta.beta * sN.en[sN.boff[b] + i] <= 800.0) r = i + 1;
      sN.rrows[b] = r;
    }
    launch_dm_trace(ta, nbN, c->stream);
    c->launches++;
    for (int k = 0; tg && k < DmTan::NP; ++k) {
      DmTraceArgs tt = ta;
      tt.rot = (const double*)((char*)U0 + (DmTan::NP + k) * zsa);
      tt.dE = (const double*)(mb + o_den) + (size_t)k * sN.en.size();
      tt.dlogz = dlogz[k];
      sN.drho[k].ensure(sizeof(double) * std::max<int64_t>(sN.zsize, 1));
      tt.rho = sN.drho[k].as<double>();
      launch_dm_trace(tt, nbN, c->stream);
      c->launches++;
    }
    CU(cudaStreamSynchronize(c->stream));  // meta and T are reused by the next shell
  }
  tm.stop(t0, &c->timing.dm_backprop_ms);
  CU(cudaStreamSynchronize(c->stream));
  check_flag(c);
  tm.collect();
  c->dm_rho_valid = true;
  c->dm_drho_valid = tg;
  c->dm_temp = p.temp;
  if (rho_trace) {
    for (int N = 0; N < nsh; ++N) {
      const DmShell& s = *c->dm[N];
      std::vector<double> R((size_t)std::max<int64_t>(s.zsize, 1));
      d2h(c, R.data(), s.rho.p, sizeof(double) * s.zsize);
      CU(cudaStreamSynchronize(c->stream));
      double t = 0.0;
      for (size_t b = 0; b < s.bsize.size(); ++b) {
        const int n = s.bsize[b];
        for (int i = 0; i < n; ++i) t += (2.0 * s.qn[2 * b + 1] + 1.0) * R[s.zoff[b] + (int64_t)i * n + i];
      }
      rho_trace[N] = t;
    }
  }
}

// CalcSpec_ManyOmegas's frequency grid (SpecFuncClass.cpp:2238-2341), FDM:
// nw points per shell from shell 2 to the last-but-one, negative side first.
std::vector<double> dm_grid(double L, int nsh, int nw) {
  const double factorWN = std::pow(L, 1.25);
  const int Nmax = nsh - 1, N0 = 2;
  std::vector<double> om;
  for (int N = N0; N <= Nmax; ++N) {
    const double WN = factorWN * calc_dn(L, N);
    for (int i = 0; i < nw; ++i) om.push_back(-(std::pow(L, -((double)i / (2.0 * nw))) * WN));
  }
  for (int N = Nmax; N >= N0; --N) {
    const double WN = factorWN * calc_dn(L, N);
    for (int i = nw - 1; i >= 0; --i) om.push_back(std::pow(L, -((double)i / (2.0 * nw))) * WN);
  }
  return om;
}

// CalcSpecDM_NRG (SpecFuncClass.cpp:1827-1883) with FDM_SpecDens_M_STL /
// CalcSpecCosti_T_N for every shell of the window, for all frequencies.
//
// d_rhow != NULL (nrg_lehmann_grad): the same sums differentiated along the
// four parameter directions of the shells' tangents, d_rhow[k * nomega + j].
// Per shell: d(rho A) = d rho A + rho dA and d(A rho) = dA rho + A d rho
// (grouped GEMMs), the records' tangents beside the records, and the
// Lehmann kernel over them.
void lehmann_impl(nrg_ctx* c, const nrg_dm_params* prm, int nomega, const double* omegas, double* omega_rhow,
                  int* nout, double* d_rhow = nullptr) {
  if (!c->dm_rho_valid) throw NrgError(NRG_ERR_STATE, "no density matrices: run nrg_dm_backprop first");
  const bool tg = d_rhow != nullptr;
  constexpr int NP = DmTan::NP;
  if (tg && !c->dm_drho_valid)
    throw NrgError(NRG_ERR_STATE, "no density-matrix tangents: run nrg_grad_forward_dm, then nrg_dm_backprop");
  if (!omega_rhow || !nout || nomega < 0) throw NrgError(NRG_ERR_ARG, "bad output arguments");
  const int nsh = (int)c->dm.size(), Nmax = nsh - 1;
  const double L = c->dm_lambda, hlf = 0.5 * (1.0 + (1.0 / L));
  const DmResolved p = dm_resolve(prm, L, nsh);
  if (p.temp != c->dm_temp) throw NrgError(NRG_ERR_STATE, "temperature differs from the one of nrg_dm_backprop");
  std::vector<double> om;
  if (omegas) om.assign(omegas, omegas + nomega);
  else {
    if (prm->nw < 1) throw NrgError(NRG_ERR_ARG, "nw must be positive");
    om = dm_grid(L, nsh, prm->nw);
    if ((int)om.size() > nomega) throw NrgError(NRG_ERR_SIZE, "omega_rhow holds fewer frequencies than the grid");
  }
  const int nw_ = (int)om.size();
  Timer tm(c);
  cudaEvent_t t0 = tm.start();
  const double sqrt_pi = 1.7724538509055160273;
  const double beta_last = std::fabs(p.temp) < 1.e-20 ? 1.0e10 : p.betabar;
  // Windows of shells per frequency (CalcNfromOmega, SpecFuncClass.cpp:41-49)
  // and, per shell and sign, the frequencies whose window holds the shell.
  const int window = 22;
  std::vector<int> wfirst(nw_), wcount(nw_);
  for (int k = 0; k < nw_; ++k) {
    int iaux = (int)(2.0 * std::log(2.0 * std::fabs(om[k]) / hlf) / std::log(L));
    iaux = 1 - iaux;
    if (iaux < 0) iaux = 0;
    const int N0 = iaux - 8 > 0 ? iaux - 8 : 0;
    const int N1 = iaux + 14 < nsh ? iaux + 14 : nsh;
    wfirst[k] = N0;
    wcount[k] = std::max(0, N1 - N0);
  }
  std::vector<std::vector<int>> oms(2 * (size_t)nsh);  // [shell][sign]: frequency indices, ascending
  for (int k = 0; k < nw_; ++k)
    for (int sl = 0; sl < wcount[k]; ++sl) oms[2 * (size_t)(wfirst[k] + sl) + (om[k] >= 0.0 ? 0 : 1)].push_back(k);
  std::vector<double> dn(nsh), ldn(nsh), lom(nw_);
  for (int N = 0; N < nsh; ++N) { dn[N] = calc_dn(L, N); ldn[N] = std::log(dn[N]); }
  for (int k = 0; k < nw_; ++k) lom[k] = std::log(std::fabs(om[k]));
  Packer tab;
  const size_t o_om = tab.add(om), o_lo = tab.add(lom), o_dn = tab.add(dn), o_ld = tab.add(ldn), o_wf = tab.add(wfirst),
               o_wc = tab.add(wcount);
  c->dmtab.ensure(tab.host.size() + 256);
  h2d(c, c->dmtab.p, tab.host.data(), tab.host.size());
  char* tb = c->dmtab.as<char>();
  LehmannArgs la{};
  la.omega = (const double*)(tb + o_om); la.log_omega = (const double*)(tb + o_lo);
  la.dn = (const double*)(tb + o_dn); la.log_dn = (const double*)(tb + o_ld);
  la.inv_b = 1.0 / p.bbroad; la.b_quarter = p.bbroad / 4.0; la.inv_bt = 1.0 / p.broadtemp;
  la.nomega = nw_; la.win_first = (const int*)(tb + o_wf); la.win_count = (const int*)(tb + o_wc); la.window = window;
  // Shell by shell: the Lehmann records (FDM_SpecDens_M_STL / CalcSpecCosti_T_N
  // weights; only the pairs whose term can be nonzero), then their sums
  // against every frequency whose window holds the shell, one partial sum
  // per record chunk and frequency.  Only one shell's records exist at a time.
  std::vector<LehList> lists;                      // every shell's lists (for the fold)
  std::vector<LehList> tlists[NP];                 // their tangent lists (parts only are read by the fold)
  std::vector<int> list_of(4 * (size_t)nsh, -1);  // [shell][list L]
  int64_t evals = 0, nrec_all = 0;
  for (int N = 0; N < nsh; ++N) {
    DmShell& s = *c->dm[N];
    const bool last = N == Nmax;
    for (int Lk = 0; Lk < 4; ++Lk) s.nrec[Lk] = 0;
    std::vector<DmPair> pairs;
    std::vector<DmChunk> chunks;
    GemmPlan g;
    int64_t poff = 0;
    std::vector<int> nk(s.bsize.size(), 0), nd(s.bsize.size(), 0);
    for (size_t b = 0; b < s.bsize.size(); ++b)
      for (int i = 0; i < s.bsize[b]; ++i) (s.kept[s.boff[b] + i] ? nk[b] : nd[b])++;
    int64_t pbytes = 0;
    for (size_t k = 0; k < s.cd.bi.size(); ++k) pbytes += (int64_t)s.bsize[s.cd.bi[k]] * s.bsize[s.cd.bj[k]];
    c->Y.ensure(sizeof(double) * std::max<int64_t>(2 * pbytes, 1));
    double* P1 = c->Y.as<double>();
    double* P2 = P1 + pbytes;
    // tangents: d(rho A) of parameter k at X1 + k pbytes, d(A rho) at X2 + k pbytes
    double *X1 = nullptr, *X2 = nullptr;
    GemmPlan gt0, gt1;
    if (tg) {
      c->dmtan.ensure(sizeof(double) * std::max<int64_t>(2 * NP * pbytes, 1));
      X1 = c->dmtan.as<double>();
      X2 = X1 + NP * pbytes;
    }
    for (size_t k = 0; k < s.cd.bi.size(); ++k) {
      const int b1 = s.cd.bi[k], b2 = s.cd.bj[k];
      DmPair P{};
      P.n1 = s.bsize[b1]; P.n2 = s.bsize[b2]; P.s1 = s.boff[b1]; P.s2 = s.boff[b2];
      P.a_off = s.cd.off[k]; P.p_off = poff;
      const double S1 = s.qn[2 * b1 + 1], S2 = s.qn[2 * b2 + 1];
      double cgf = 0.0;
      for (double Sz1 = -S1; Sz1 <= S1; Sz1 += 1.0) {
        const double x = clebsch(S1, Sz1, 0.5, 0.5, S2, Sz1 + 0.5);
        cgf += x * x;
      }
      P.cg = cgf;
      P.skip = ((nk[b1] == 0 && nk[b2] == 0) || (nd[b1] == 0 && nd[b2] == 0)) ? 1 : 0;
      P.r1 = s.rrows[b1]; P.r2 = s.rrows[b2];
      if (!last && !P.skip) {
        // rho A has r1 nonzero rows, A rho r2 nonzero columns (the rest is
        // never read).
        const double* Acd = s.cdel.as<double>() + P.a_off;
        const double* rho1 = s.rho.as<double>() + s.zoff[b1];
        const double* rho2 = s.rho.as<double>() + s.zoff[b2];
        g.add(GemmJob{P.r1, P.n2, P.r1, 0, rho1, P.n1, Acd, P.n2, P1 + poff, P.n2});
        g.add(GemmJob{P.n1, P.r2, P.r2, 0, Acd, P.n2, rho2, P.n2, P2 + poff, P.n2});
        for (int k = 0; tg && k < NP; ++k) {
          const double* dA = s.dcd[k].as<double>() + P.a_off;
          const double* drho1 = s.drho[k].as<double>() + s.zoff[b1];
          const double* drho2 = s.drho[k].as<double>() + s.zoff[b2];
          double* x1 = X1 + k * pbytes + poff;
          double* x2 = X2 + k * pbytes + poff;
          gt0.add(GemmJob{P.r1, P.n2, P.r1, 0, drho1, P.n1, Acd, P.n2, x1, P.n2});
          gt1.add(GemmJob{P.r1, P.n2, P.r1, 0, rho1, P.n1, dA, P.n2, x1, P.n2, 1});
          gt0.add(GemmJob{P.n1, P.r2, P.r2, 0, dA, P.n2, rho2, P.n2, x2, P.n2});
          gt1.add(GemmJob{P.n1, P.r2, P.r2, 0, Acd, P.n2, drho2, P.n2, x2, P.n2, 1});
        }
      }
      if ((int64_t)P.n1 * P.n2 > (int64_t)INT32_MAX) throw NrgError(NRG_ERR_SIZE, "c_d block pair too large");
      if (last || !P.skip)
        for (int64_t st = 0; st < (int64_t)P.n1 * P.n2; st += kPairChunk)
          chunks.push_back(DmChunk{(int)pairs.size(), (int)st});
      pairs.push_back(P);
      poff += (int64_t)P.n1 * P.n2;
    }
    if (chunks.empty()) continue;
    run_gemm_plan(c, g);
    run_gemm_plan(c, gt0);
    run_gemm_plan(c, gt1);
    Packer pk;
    size_t o_p = pk.add(pairs), o_c = pk.add(chunks), o_en = pk.add(s.en), o_kp = pk.add(s.kept),
           o_den = tg ? pk.add(s.den) : 0;
    c->meta.ensure(pk.host.size() + 256);
    h2d(c, c->meta.p, pk.host.data(), pk.host.size());
    char* mb = c->meta.as<char>();
    const int nch = (int)chunks.size();
    c->dmcnt.ensure(sizeof(int64_t) * (8 * (size_t)nch + 8));
    DmRecArgs a{};
    a.pairs = (const DmPair*)(mb + o_p); a.chunks = (const DmChunk*)(mb + o_c); a.nchunks = nch;
    a.cd = s.cdel.as<double>(); a.P1 = P1; a.P2 = P2;
    a.en = (const double*)(mb + o_en); a.kept = (const unsigned char*)(mb + o_kp);
    a.last = last ? 1 : 0;
    a.beta_last = beta_last;
    if (last) {
      double z = 0.0;
      for (size_t b = 0; b < s.bsize.size(); ++b)
        for (int i = s.boff[b]; i < s.boff[b] + s.bsize[b]; ++i)
          z += (2.0 * s.qn[2 * b + 1] + 1.0) * std::exp(-beta_last * s.en[i]);
      a.inv_z_last = 1.0 / z;
      for (int k = 0; tg && k < NP; ++k) a.dlogz_last[k] = dm_partition_tangent(s, beta_last, false, k) / z;
    }
    if (tg) {
      a.ntan = NP;
      a.dP1 = X1; a.dP2 = X2; a.pstride = pbytes;
      for (int k = 0; k < NP; ++k) a.dcd[k] = s.dcd[k].as<double>();
      a.dE = (const double*)(mb + o_den);
      a.nstates = (int)s.en.size();
    }
    a.gauss_below = p.twindow * (p.temp / dn[N]);
    a.inv_b = 1.0 / p.bbroad; a.inv_bt = 1.0 / p.broadtemp;
    a.log_scale = 1.0 / (p.bbroad * sqrt_pi); a.gauss_scale = 1.0 / (p.broadtemp * sqrt_pi);
    a.offsets = c->dmcnt.as<int64_t>();
    a.totals = a.offsets + 4 * (size_t)nch;
    a.counts = (int*)(a.totals + 8);
    launch_dm_records(a, 0, c->stream);
    c->launches += 2;
    int64_t tot[4];
    d2h(c, tot, a.totals, sizeof(tot));
    CU(cudaStreamSynchronize(c->stream));
    int64_t nrec = 0;
    for (int Lk = 0; Lk < 4; ++Lk) nrec += tot[Lk];
    const int per_rec = tg ? 2 + 2 * NP : 2;  // key, w (and per parameter d w, 2 w d key)
    c->dmrec.ensure(sizeof(double) * std::max<int64_t>(per_rec * nrec, 1));
    double* r = c->dmrec.as<double>();
    for (int Lk = 0; Lk < 4; ++Lk) {
      s.nrec[Lk] = tot[Lk];
      a.key[Lk] = r;
      a.w[Lk] = r + tot[Lk];
      if (tg) {
        a.tw[Lk] = r + 2 * tot[Lk];
        a.tg[Lk] = r + (2 + NP) * tot[Lk];
      }
      r += per_rec * tot[Lk];
    }
    launch_dm_records(a, 1, c->stream);
    c->launches++;
    // This shell's lists, their frequencies and work items.
    std::vector<LehList> sl;
    std::vector<int> sl_kind;
    std::vector<int64_t> sl_off;
    std::vector<LehItem> items;
    std::vector<int> omega_idx;
    int64_t part = 0;
    for (int Lk = 0; Lk < 4; ++Lk) {
      const std::vector<int>& ks = oms[2 * (size_t)N + (Lk < 2 ? 0 : 1)];
      nrec_all += s.nrec[Lk];
      if (s.nrec[Lk] == 0 || ks.empty()) continue;
      LehList li{};
      li.key = a.key[Lk]; li.w = a.w[Lk]; li.nrec = s.nrec[Lk]; li.shell = N; li.gauss = Lk & 1;
      li.nomega = (int)ks.size(); li.omega_first = (int)omega_idx.size();
      omega_idx.insert(omega_idx.end(), ks.begin(), ks.end());
      const int64_t nchk = (li.nrec + kRecChunk - 1) / kRecChunk;
      const int ntile = (li.nomega + kOmegaTile - 1) / kOmegaTile;
      part += nchk * li.nomega;
      evals += li.nrec * li.nomega;
      // Tiles of a log-Gaussian list whose frequencies are evenly spaced in
      // ln|omega| (to 1e-12 of the step; the step at most 0.1 b, so that 16
      // steps move the Gaussian's argument by at most 1.6) take the
      // recurrence.
      std::vector<double> tile_delta(ntile, 0.0);
      if (!li.gauss)
        for (int tl = 0; tl < ntile; ++tl) {
          const int j0 = tl * kOmegaTile, j1 = std::min(li.nomega, j0 + kOmegaTile);
          if (j1 - j0 < 2) continue;
          const double d = (lom[ks[j1 - 1]] - lom[ks[j0]]) / (j1 - 1 - j0);
          bool even = std::isfinite(d) && d != 0.0 && std::fabs(d) <= 0.1 * p.bbroad;
          for (int j = j0; even && j + 1 < j1; ++j)
            even = std::fabs((lom[ks[j + 1]] - lom[ks[j]]) - d) <= 1e-12 * std::fabs(d);
          if (even) tile_delta[tl] = d / p.bbroad;
        }
      for (int64_t ch = 0; ch < nchk; ++ch)
        for (int tl = 0; tl < ntile; ++tl) items.push_back(LehItem{(int)sl.size(), (int)ch, tl, tile_delta[tl]});
      sl.push_back(li);
      sl_kind.push_back(Lk);
      sl_off.push_back(part - nchk * li.nomega);
    }
    if (items.size() > (size_t)INT32_MAX) throw NrgError(NRG_ERR_SIZE, "too many Lehmann work items");
    s.lpart.ensure(sizeof(double) * std::max<int64_t>(part, 1));
    if (tg) s.ltpart.ensure(sizeof(double) * std::max<int64_t>(NP * part, 1));
    std::vector<LehList> stl;  // this shell's tangent lists, parameter major
    for (int k = 0; tg && k < NP; ++k)
      for (size_t q = 0; q < sl.size(); ++q) {
        LehList t = sl[q];
        const int Lk = sl_kind[q];
        t.w = a.tw[Lk] + k * tot[Lk];
        t.g = a.tg[Lk] + k * tot[Lk];
        t.part = s.ltpart.as<double>() + k * part + sl_off[q];
        stl.push_back(t);
        tlists[k].push_back(t);
      }
    for (size_t q = 0; q < sl.size(); ++q) {
      sl[q].part = s.lpart.as<double>() + sl_off[q];
      list_of[4 * (size_t)N + sl_kind[q]] = (int)lists.size();
      lists.push_back(sl[q]);
    }
    if (!items.empty()) {
      Packer pl;
      const size_t o_li = pl.add(sl), o_it = pl.add(items), o_oi = pl.add(omega_idx);
      c->vmeta.ensure(pl.host.size() + 256);
      h2d(c, c->vmeta.p, pl.host.data(), pl.host.size());
      char* vb = c->vmeta.as<char>();
      la.lists = (const LehList*)(vb + o_li); la.items = (const LehItem*)(vb + o_it); la.nitems = (int)items.size();
      la.omega_idx = (const int*)(vb + o_oi);
      cudaEvent_t t1 = tm.start();
      launch_lehmann(la, c->stream);
      c->launches++;
      tm.stop(t1, &c->timing.lehmann_ms);
      if (tg) {  // the same items over the tangent lists of every parameter
        std::vector<LehItem> titems;
        for (int k = 0; k < NP; ++k)
          for (LehItem it : items) {
            it.list += k * (int)sl.size();
            titems.push_back(it);
          }
        if (titems.size() > (size_t)INT32_MAX) throw NrgError(NRG_ERR_SIZE, "too many Lehmann work items");
        Packer pt;
        const size_t o_tl = pt.add(stl), o_ti = pt.add(titems), o_to = pt.add(omega_idx);
        c->dmtmeta.ensure(pt.host.size() + 256);
        h2d(c, c->dmtmeta.p, pt.host.data(), pt.host.size());
        char* tb2 = c->dmtmeta.as<char>();
        LehmannArgs lt = la;
        lt.lists = (const LehList*)(tb2 + o_tl); lt.items = (const LehItem*)(tb2 + o_ti);
        lt.nitems = (int)titems.size(); lt.omega_idx = (const int*)(tb2 + o_to);
        launch_lehmann_tangent(lt, c->stream);
        c->launches++;
      }
    }
    CU(cudaStreamSynchronize(c->stream));  // meta, vmeta, dmrec and Y are reused by the next shell
  }
  // A(omega): every frequency's window shells in order.
  std::vector<int> fold_list((size_t)nw_ * window * 2, -1), fold_pos((size_t)nw_ * window * 2, 0);
  for (int k = 0; k < nw_; ++k)
    for (int sl2 = 0; sl2 < wcount[k]; ++sl2) {
      const int N = wfirst[k] + sl2, sg = om[k] >= 0.0 ? 0 : 1;
      const std::vector<int>& ks = oms[2 * (size_t)N + sg];
      const int pos = (int)(std::lower_bound(ks.begin(), ks.end(), k) - ks.begin());
      for (int gsn = 0; gsn < 2; ++gsn) {
        const size_t fi = ((size_t)k * window + sl2) * 2 + gsn;
        fold_list[fi] = list_of[4 * (size_t)N + 2 * sg + gsn];
        fold_pos[fi] = pos;
      }
    }
  Packer pf;
  const size_t o_li = pf.add(lists), o_fl = pf.add(fold_list), o_fp = pf.add(fold_pos);
  size_t o_tli[NP] = {0, 0, 0, 0};
  for (int k = 0; tg && k < NP; ++k) o_tli[k] = pf.add(tlists[k]);
  c->meta.ensure(pf.host.size() + 256);
  h2d(c, c->meta.p, pf.host.data(), pf.host.size());
  char* fb = c->meta.as<char>();
  const int nout_sets = tg ? 1 + NP : 1;
  c->dmrec.ensure(sizeof(double) * std::max(nout_sets * nw_, 1));
  la.lists = (const LehList*)(fb + o_li); la.items = nullptr; la.nitems = 0;
  la.fold_list = (const int*)(fb + o_fl); la.fold_pos = (const int*)(fb + o_fp);
  la.out = c->dmrec.as<double>();
  cudaEvent_t t2 = tm.start();
  launch_lehmann_fold(la, c->stream);
  c->launches++;
  for (int k = 0; tg && k < NP; ++k) {  // the tangent lists have the primal lists' order
    LehmannArgs lf = la;
    lf.lists = (const LehList*)(fb + o_tli[k]);
    lf.out = c->dmrec.as<double>() + (size_t)(1 + k) * nw_;
    launch_lehmann_fold(lf, c->stream);
    c->launches++;
  }
  tm.stop(t2, &c->timing.lehmann_ms);
  std::vector<double> A((size_t)nout_sets * nw_);
  d2h(c, A.data(), la.out, sizeof(double) * nout_sets * nw_);
  tm.stop(t0, &c->timing.dm_spectral_ms);
  CU(cudaStreamSynchronize(c->stream));
  check_flag(c);
  tm.collect();
  c->timing.lehmann_pairs = nrec_all;
  c->timing.lehmann_evals = evals;
  for (int k = 0; k < nw_; ++k) { omega_rhow[k] = om[k]; omega_rhow[nomega + k] = A[k]; }
  if (tg) {
    c->dm_drhow.assign((size_t)NP * nw_, 0.0);
    for (int k = 0; k < NP; ++k)
      for (int j = 0; j < nw_; ++j) {
        d_rhow[(size_t)k * nomega + j] = A[(size_t)(1 + k) * nw_ + j];
        c->dm_drhow[(size_t)k * nw_ + j] = A[(size_t)(1 + k) * nw_ + j];
      }
  }
  *nout = nw_;
}

// The DM-NRG shells as the reference's .bin snapshots.  Abasis_N's
// StCameFrom numbers the states of the uncut array of shell N-1 (UpdateBefCut,
// BuildBasis.cpp:386-391): a state that came from state a of kept block k came
// from state a of that kept block's uncut block.
void dm_save_bin_impl(nrg_ctx* c, const char* dir, const char* name) {
  if (c->dm.empty()) throw NrgError(NRG_ERR_STATE, "no DM-NRG shells: run nrg_sweep_run_dm first");
  if (!dir || !name) throw NrgError(NRG_ERR_ARG, "directory or name is NULL");
  if (c->dm_model != MODEL_1CHQS)
    throw NrgError(NRG_ERR_ARG, "the reference's DM_NRG reads one-channel |Q S> shells only (DM_NRG.cpp:292)");
  for (size_t N = 0; N < c->dm.size(); ++N) {
    const DmShell& s = *c->dm[N];
    const Basis& B = s.basis;
    const int ns = B.blk.nstates();
    std::vector<int> bbbe, stcf(ns), bbe;
    std::vector<double> ben(ns);
    for (int b = 0; b < B.blk.nblocks(); ++b) {
      bbbe.push_back(B.blk.offset[b]);
      bbbe.push_back(B.blk.offset[b] + B.blk.size[b] - 1);
      for (int i = 0; i < B.blk.size[b]; ++i) {
        const int g = B.blk.offset[b] + i;
        const Segment& sg = B.seg[b][B.seg_of[g]];
        int full;
        double e;
        if (N == 0) {
          full = B.stcf[g];
          e = c->dm_hm1_en[full];
        } else {
          const DmShell& p = *c->dm[N - 1];
          full = p.boff[p.kept_src[sg.old_block]] + B.a_of[g];
          e = p.en[full];
        }
        stcf[g] = full;
        ben[g] = e;
      }
    }
    for (size_t b = 0; b < s.bsize.size(); ++b) {
      bbe.push_back(s.boff[b]);
      bbe.push_back(s.boff[b] + s.bsize[b] - 1);
    }
    std::vector<double> Z((size_t)std::max<int64_t>(s.zsize, 1)), el((size_t)std::max<int64_t>(s.cd.size, 1));
    d2h(c, Z.data(), s.Z.p, sizeof(double) * s.zsize);
    d2h(c, el.data(), s.cdel.p, sizeof(double) * s.cd.size);
    CU(cudaStreamSynchronize(c->stream));
    std::vector<int> map, mbe;
    for (size_t k = 0; k < s.cd.bi.size(); ++k) {
      map.push_back(s.cd.bi[k]);
      map.push_back(s.cd.bj[k]);
      const int64_t len = (int64_t)s.bsize[s.cd.bi[k]] * s.bsize[s.cd.bj[k]];
      mbe.push_back((int)s.cd.off[k]);
      mbe.push_back((int)(s.cd.off[k] + len - 1));
    }
    nrg_dm_shell v{};
    v.nshell = (int)N;
    v.basis.blocks = nrg_blocks{B.blk.nblocks(), 2, B.blk.qn.data(), bbbe.data()};
    v.basis.itype = B.itype.data();
    v.basis.st_came_from = stcf.data();
    v.basis.en = ben.data();
    v.blocks = nrg_blocks{(int)s.bsize.size(), 2, s.qn.data(), bbe.data()};
    v.en = s.en.data();
    v.kept = s.kept.data();
    v.eigvec = Z.data();
    v.cd = nrg_matrix{(int)s.cd.bi.size(), map.data(), mbe.data(), el.data()};
    const nrg_status st = nrg_write_dm_shell(dir, name, &v);
    if (st != NRG_OK) throw NrgError(st, std::string("cannot write the shell files into ") + dir);
  }
  const nrg_status st = nrg_write_code_pars(dir, c->dm_lambda, (int)c->dm.size(), name);
  if (st != NRG_OK) throw NrgError(st, std::string("cannot write ThisCodePars.dat into ") + dir);
}

// The DM-NRG shells from .bin snapshots in the reference's layout, as
// DM_NRG reads them (DM_NRG.cpp:163-298 with CNRGarray::ReadBinInStream,
// NRGarrayClass.cpp:886-958; CNRGbasisarray::ReadBin, :2005-2078;
// CNRGmatrix::ReadBin, NRGmatrixClass.cpp:1016-1082): Lambda from
// ThisCodePars.dat, then per shell N Abasis_N, Acut_N and Mat0_N (c_d).  The
// device needs each shell's BuildBasis segments, which the files do not
// hold: they are rebuilt from the previous shell's kept blocks (H_{-1}'s for
// shell 0) and the rebuilt basis must equal the file's -- sectors, block
// sizes, iType and StCameFrom -- or the call returns NRG_ERR_SYNC.
void dm_load_bin_impl(nrg_ctx* c, const char* dir, const char* name, int nshells) {
  if (!dir || !name) throw NrgError(NRG_ERR_ARG, "directory or name is NULL");
  double lambda = 0.0;
  int nsites0 = 0, nmax = 0;
  {
    std::ifstream pars(std::string(dir) + "/ThisCodePars.dat");
    if (!(pars >> lambda >> nsites0 >> nmax)) throw NrgError(NRG_ERR_ARG, std::string("cannot read ") + dir +
                                                                      "/ThisCodePars.dat");
  }
  if (!(lambda > 1.0)) throw NrgError(NRG_ERR_ARG, "ThisCodePars.dat: Lambda must exceed 1");
  if (nshells <= 0) nshells = nmax;
  if (nshells <= 0) throw NrgError(NRG_ERR_ARG, "no shells to load");
  ModelSpec m = make_model(MODEL_1CHQS);
  StartState st = make_start(m, lambda, 0.0, 0.0, 0.0);
  // the device words the backward sweep and the spectral function use (a
  // fresh context has run no sweep that would have made them)
  c->flag.ensure(sizeof(int) * 4);
  CU(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
  c->scal.ensure(sizeof(double) * 32);
  c->partial.ensure(sizeof(double) * 64 * 16);
  c->opptr.ensure(sizeof(double*) * 32);
  c->dm.clear();
  c->dm_rho_valid = false;
  c->dm_drho_valid = false;
  c->dm_lambda = lambda;
  c->dm_model = MODEL_1CHQS;
  c->dm_hm1_en.assign(st.en.size(), 0.0);
  BlockArray prev = st.blk;                        // the kept array shell N was built from
  std::vector<int> prev_full_off = st.blk.offset;  // where each kept block starts in the previous full array
  for (int N = 0; N < nshells; ++N) {
    BinShellFile fb, fa, fm;
    std::string err;
    if (!read_bin_file(bin_path(dir, "Abasis", name, N), 1, fb, err) ||
        !read_bin_file(bin_path(dir, "Acut", name, N), 1, fa, err) ||
        !read_bin_file(bin_path(dir, "Mat0", name, N), 2, fm, err))
      throw NrgError(NRG_ERR_ARG, err);
    if (fb.nqn != 2 || fa.nqn != 2 || fm.nqn != 2 || fb.nshell != N || fa.nshell != N)
      throw NrgError(NRG_ERR_ARG, "snapshot of shell " + std::to_string(N) + " is not a one-channel |Q S> shell N");
    Basis B;
    build_basis(m, prev, B);
    const int nb = B.blk.nblocks(), ns = B.blk.nstates();
    bool same = (int)fb.qn.size() == 2 * nb && (int)fb.itype.size() == ns && (int)fb.stcf.size() == ns &&
                (int)fb.en.size() == ns;
    for (int b = 0; same && b < nb; ++b)
      same = fb.qn[2 * b] == B.blk.q(b, 0) && fb.qn[2 * b + 1] == B.blk.q(b, 1) &&
             fb.bbe[2 * b] == B.blk.offset[b] && fb.bbe[2 * b + 1] == B.blk.offset[b] + B.blk.size[b] - 1;
    for (int b = 0; same && b < nb; ++b)
      for (int i = 0; same && i < B.blk.size[b]; ++i) {
        const int g = B.blk.offset[b] + i;
        const Segment& sg = B.seg[b][B.seg_of[g]];
        same = fb.itype[g] == B.itype[g] && fb.stcf[g] == prev_full_off[sg.old_block] + B.a_of[g];
      }
    if (!same)
      throw NrgError(NRG_ERR_SYNC, "Abasis of shell " + std::to_string(N) +
                                       " is not what BuildBasis makes of the previous shell's kept states");
    if (N == 0)
      for (int g = 0; g < ns; ++g) c->dm_hm1_en[fb.stcf[g]] = fb.en[g];
    // Acut_N: the blocks of H_N, energies, Kept, all eigenvectors
    if (fa.qn != fb.qn || fa.bbe != fb.bbe || (int)fa.en.size() != ns || (int)fa.kept.size() != ns)
      throw NrgError(NRG_ERR_SYNC, "Acut of shell " + std::to_string(N) + " does not match its Abasis");
    auto sh = std::make_unique<DmShell>();
    sh->bsize = B.blk.size; sh->boff = B.blk.offset; sh->qn = B.blk.qn;
    sh->en = fa.en; sh->kept = fa.kept;
    int64_t z = 0;
    for (int b = 0; b < nb; ++b) {
      const int n = B.blk.size[b];
      if ((int)fa.bbe_eig.size() != 2 * nb || fa.bbe_eig[2 * b] != z || fa.bbe_eig[2 * b + 1] != z + (int64_t)n * n - 1)
        throw NrgError(NRG_ERR_SYNC, "eigenvector layout of shell " + std::to_string(N) + " is not n x n per block");
      sh->zoff.push_back(z);
      z += (int64_t)n * n;
    }
    if ((int64_t)fa.evec.size() != z) throw NrgError(NRG_ERR_SYNC, "eigenvector count of shell " + std::to_string(N));
    sh->zsize = z;
    // kept blocks (Kept is a prefix of each block: CutStates keeps the levels up to E_cut)
    BlockArray kept;
    kept.nqn = 2;
    std::vector<int> kept_full_off;
    for (int b = 0; b < nb; ++b) {
      int k = 0;
      while (k < B.blk.size[b] && fa.kept[B.blk.offset[b] + k]) ++k;
      for (int x = k; x < B.blk.size[b]; ++x)
        if (fa.kept[B.blk.offset[b] + x]) throw NrgError(NRG_ERR_SYNC, "Kept is not a prefix of its block");
      if (k == 0) continue;
      kept.push(&B.blk.qn[2 * b], k);
      sh->kept_src.push_back(b);
      kept_full_off.push_back(B.blk.offset[b]);
    }
    // c_d: MatBlockMap / MatBlockBegEnd over the blocks of H_N
    const int nmb = (int)fm.map.size() / 2;
    if ((int)fm.mbe.size() != 2 * nmb || fm.qn != fa.qn || fm.bbe != fa.bbe)
      throw NrgError(NRG_ERR_SYNC, "Mat0 of shell " + std::to_string(N) + " is not synced with Acut");
    int64_t nel = 0;
    for (int k = 0; k < nmb; ++k) {
      const int bi = fm.map[2 * k], bj = fm.map[2 * k + 1];
      if (bi < 0 || bi >= nb || bj < 0 || bj >= nb ||
          fm.mbe[2 * k + 1] - fm.mbe[2 * k] + 1 != B.blk.size[bi] * B.blk.size[bj])
        throw NrgError(NRG_ERR_SYNC, "c_d block table of shell " + std::to_string(N));
      sh->cd.bi.push_back(bi); sh->cd.bj.push_back(bj); sh->cd.off.push_back(fm.mbe[2 * k]);
      nel = std::max<int64_t>(nel, (int64_t)fm.mbe[2 * k + 1] + 1);
    }
    if ((int64_t)fm.mat_el.size() < nel) throw NrgError(NRG_ERR_SYNC, "c_d elements of shell " + std::to_string(N));
    sh->cd.size = nel;
    sh->Z.ensure(sizeof(double) * std::max<int64_t>(z, 1));
    h2d(c, sh->Z.p, fa.evec.data(), sizeof(double) * z);
    sh->cdel.ensure(sizeof(double) * std::max<int64_t>(nel, 1));
    h2d(c, sh->cdel.p, fm.mat_el.data(), sizeof(double) * nel);
    CU(cudaStreamSynchronize(c->stream));
    sh->basis = std::move(B);
    c->dm.push_back(std::move(sh));
    prev = kept;
    prev_full_off = kept_full_off;
  }
}

// DiagBlock for a batch of blocks given in the reference's packed upper
// storage: same device pipeline as the sweep, all eigenvectors kept.
// ------------------------------------------------------------ thermodynamics
// calcdens = 3 then 2 (NRGthermoClass.cpp:10-150, NRGcodehandlerClass.cpp:
// 627-677): the free chain's T chi and S at the same temperatures T_M = D_N /
// betabar_nc as the impurity sweep, and the impurity contribution as the
// difference.  Value k (= 4 N + nc - 1) of the impurity sweep is paired with
// value k of the chain, which is what CNRGthermo::ReadNChainValue does with
// line k of the chain file.  The chain's own CNRGthermo::dImpValue is never
// set by ModelSwitch for ModelNo 3 and reads as 0 there; it is 0 here.
bool same_chain(const nrg_sweep_config& a, const nrg_sweep_config& b) {
  return a.model == b.model && a.nsites == b.nsites && a.ncutoff == b.ncutoff && a.lambda == b.lambda &&
         a.degen_eps == b.degen_eps && a.precision == b.precision;
}

void thermo_run_impl(nrg_ctx* c, const nrg_sweep_config* cfg, int reuse_chain) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  const bool reuse = reuse_chain != 0 && c->chain_valid && same_chain(c->chain_cfg, *cfg);
  double chain_ms = 0.0, imp_ms = 0.0;
  if (!reuse) {
    c->chain_valid = false;
    if (!c->chain_ctx) {
      const nrg_status st = nrg_create(c->device, &c->chain_ctx);
      if (st != NRG_OK) throw NrgError(st, "cannot create the free-chain context");
    }
    c->chain_ctx->chain_chi = c->chain_chi;
    c->chain_ctx->chain_en = c->chain_en;
    c->chain_ctx->chain_alambda = c->chain_alambda;
    nrg_ctx* cc = c->chain_ctx;
    nrg_status cst = NRG_OK;
    std::string cerr;
    // The chain sweep on its own stream and host thread: the two sweeps'
    // launches overlap on the device.
    std::thread th([&]() {
      const auto a = clock::now();
      try {
        CU(cudaSetDevice(cc->device));
        sweep_run(cc, cfg, false, true);
      } catch (const NrgError& e) {
        cst = e.st; cerr = e.what();
      } catch (const std::exception& e) {
        cst = NRG_ERR_ARG; cerr = e.what();
      }
      chain_ms = std::chrono::duration<double, std::milli>(clock::now() - a).count();
    });
    try {
      const auto a = clock::now();
      sweep_run(c, cfg);
      imp_ms = std::chrono::duration<double, std::milli>(clock::now() - a).count();
    } catch (...) {
      th.join();
      throw;
    }
    th.join();
    if (cst != NRG_OK) throw NrgError(cst, "free-chain sweep: " + cerr);
    c->chain_thermo.clear();
    for (const IterResult& R : cc->iters) c->chain_thermo.insert(c->chain_thermo.end(), R.thermo.begin(), R.thermo.end());
    // CNRGthermo::AddValue (NRGthermoClass.cpp:17-18) subtracts dImpValue in
    // the chain run: 2 ln 2 for the |Q> entropy (CodeHandler_ModelSwitch.cpp:
    // 1187-1191, the decoupled impurity); never set, and 0, for the others.
    if (cfg->model == NRG_MODEL_1CH_Q)
      for (size_t k = 3; k < c->chain_thermo.size(); k += 4) c->chain_thermo[k] -= 2.0 * std::log(2.0);
    c->chain_cfg = *cfg;
    c->chain_valid = true;
  } else {
    const auto a = clock::now();
    sweep_run(c, cfg);
    imp_ms = std::chrono::duration<double, std::milli>(clock::now() - a).count();
  }
  const int nv = 4 * (int)c->iters.size();
  if ((int)c->chain_thermo.size() != 4 * nv) throw NrgError(NRG_ERR_SYNC, "chain and impurity sweeps differ in length");
  for (auto* v : {&c->th_temp, &c->th_sus, &c->th_sus_chain, &c->th_sus_imp, &c->th_ent, &c->th_ent_chain,
                  &c->th_ent_imp})
    v->assign(nv, 0.0);
  for (int k = 0; k < nv; ++k) {
    const double* imp = c->iters[k / 4].thermo.data() + 4 * (k % 4);
    const double* ch = c->chain_thermo.data() + 4 * k;
    if (imp[1] != ch[1]) throw NrgError(NRG_ERR_SYNC, "chain and impurity temperatures differ");
    c->th_temp[k] = imp[1];
    c->th_sus[k] = imp[2]; c->th_sus_chain[k] = ch[2]; c->th_sus_imp[k] = imp[2] - ch[2];
    c->th_ent[k] = imp[3]; c->th_ent_chain[k] = ch[3]; c->th_ent_imp[k] = imp[3] - ch[3];
  }
  c->th_chain_reused = reuse ? 1 : 0;
  c->th_chain_ms = chain_ms;
  c->th_imp_ms = imp_ms;
  c->th_total_ms = std::chrono::duration<double, std::milli>(clock::now() - t0).count();
}

void diag_blocks_impl(nrg_ctx* c, int nb, const int* sizes, const double* packed, double* evals, double* evecs) {
  if (nb <= 0 || !sizes || !packed || !evals || !evecs) throw NrgError(NRG_ERR_ARG, "bad arguments");
  std::vector<int> bs(sizes, sizes + nb);
  for (int n : bs) if (n <= 0) throw NrgError(NRG_ERR_ARG, "block size must be positive");
  std::memset(&c->timing, 0, sizeof(c->timing));
  Timer tm(c);
  EigPlan P;
  plan_blocks(P, bs);
  std::vector<double> Hh((size_t)P.hsize);
  size_t pos = 0;
  for (int b = 0; b < nb; ++b) {
    const int n = bs[b];
    double* h = Hh.data() + P.hoff[b];
    for (int i = 0; i < n; ++i)
      for (int j = i; j < n; ++j) { const double v = packed[pos++]; h[(size_t)i * n + j] = v; h[(size_t)j * n + i] = v; }
  }
  std::vector<int> order(nb), state_block(P.nstates);
  for (int b = 0; b < nb; ++b) order[b] = b;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return bs[x] > bs[y]; });
  for (int b = 0; b < nb; ++b) for (int i = 0; i < bs[b]; ++i) state_block[P.soff[b] + i] = b;
  Packer pk;
  size_t o_bsize = pk.add(P.bsize), o_soff = pk.add(P.soff), o_hoff = pk.add(P.hoff), o_order = pk.add(order),
         o_sb = pk.add(state_block);
  c->meta.ensure(pk.host.size() + 256);
  c->H.ensure(sizeof(double) * (size_t)P.hsize);
  c->d.ensure(sizeof(double) * P.nstates); c->e.ensure(sizeof(double) * P.nstates);
  c->tau.ensure(sizeof(double) * P.nstates); c->ev.ensure(sizeof(double) * P.nstates);
  c->red.ensure(sizeof(int) * 8);
  c->flag.ensure(sizeof(int) * 4);
  CU(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
  h2d(c, c->meta.p, pk.host.data(), pk.host.size());
  h2d(c, c->H.p, Hh.data(), sizeof(double) * (size_t)P.hsize);
  char* mb = c->meta.as<char>();
  run_tridiag_and_bisect(c, tm, P, order, (const int*)(mb + o_order), (const int*)(mb + o_bsize),
                         (const int64_t*)(mb + o_hoff), (const int*)(mb + o_soff), (const int*)(mb + o_sb));
  std::vector<double> ev(P.nstates);
  d2h(c, ev.data(), c->ev.p, sizeof(double) * P.nstates);
  CU(cudaStreamSynchronize(c->stream));
  check_flag(c);
  P.nvec = bs;
  run_vectors(c, tm, P, ev, (const int*)(mb + o_bsize), (const int64_t*)(mb + o_hoff), (const int*)(mb + o_soff));
  d2h(c, evecs, c->Z.p, sizeof(double) * (size_t)P.ysize);
  CU(cudaStreamSynchronize(c->stream));
  check_flag(c);
  tm.collect();
  std::memcpy(evals, ev.data(), sizeof(double) * P.nstates);
}

// ------------------------------------------------------------------ per-step drop-ins
// Reference containers crossing the ABI are checked and turned into the
// engine's block structures here.
BlockArray blocks_from_abi(const nrg_blocks* b, const char* what) {
  if (!b || b->nblocks < 0 || (b->nblocks > 0 && (!b->qnumbers || !b->block_beg_end)))
    throw NrgError(NRG_ERR_ARG, std::string(what) + ": missing block structure");
  if (b->nqn != 2) throw NrgError(NRG_ERR_ARG, std::string(what) + ": expected 2 quantum numbers per block");
  BlockArray a;
  a.nqn = 2;
  int next = 0;
  for (int k = 0; k < b->nblocks; ++k) {
    const int beg = b->block_beg_end[2 * k], end = b->block_beg_end[2 * k + 1];
    if (beg != next || end < beg)
      throw NrgError(NRG_ERR_ARG, std::string(what) + ": BlockBegEnd must tile the states in order");
    a.push(&b->qnumbers[2 * k], end - beg + 1);
    next = end + 1;
  }
  return a;
}

// A built-in model of the per-call-site drop-ins, or a caller's description.
ModelSpec model_from_abi(int model, const nrg_model_desc* desc = nullptr) {
  if (desc) {
    try {
      return make_plugin_model(*desc);
    } catch (const std::invalid_argument& e) {
      throw NrgError(NRG_ERR_ARG, e.what());
    }
  }
  if (model < 0 || model > 2) throw NrgError(NRG_ERR_ARG, "unknown model");
  return make_model((ModelKind)model);
}

// BuildBasis of `kept` must reproduce the caller's basis: the assembly and
// rotation tables are derived from that layout (BuildBasis.cpp:292-403).
void check_basis(const Basis& B, const nrg_basis* ab) {
  if (!ab) throw NrgError(NRG_ERR_ARG, "abasis is NULL");
  const nrg_blocks& bb = ab->blocks;
  if (bb.nqn != 2 || bb.nblocks != B.blk.nblocks())
    throw NrgError(NRG_ERR_SYNC, "abasis blocks differ from BuildBasis of the kept array");
  for (int k = 0; k < bb.nblocks; ++k) {
    if (bb.qnumbers[2 * k] != B.blk.qn[2 * k] || bb.qnumbers[2 * k + 1] != B.blk.qn[2 * k + 1] ||
        bb.block_beg_end[2 * k] != B.blk.offset[k] || bb.block_beg_end[2 * k + 1] != B.blk.offset[k] + B.blk.size[k] - 1)
      throw NrgError(NRG_ERR_SYNC, "abasis blocks differ from BuildBasis of the kept array");
  }
  const int ns = B.blk.nstates();
  if (ns > 0 && (!ab->itype || !ab->st_came_from || !ab->en)) throw NrgError(NRG_ERR_ARG, "abasis arrays missing");
  for (int g = 0; g < ns; ++g)
    if (ab->itype[g] != B.itype[g] || ab->st_came_from[g] != B.stcf[g])
      throw NrgError(NRG_ERR_SYNC, "abasis iType/StCameFrom differ from BuildBasis of the kept array");
}

// A reference operator in the engine's storage (same row-major blocks):
// pair list, offsets and element count, after range checks.
OpMeta op_from_abi(const nrg_matrix& M, const BlockArray& blk, int64_t* nel) {
  OpMeta om;
  if (M.nmatblocks < 0 || (M.nmatblocks > 0 && (!M.mat_block_map || !M.mat_block_beg_end || !M.mat_el)))
    throw NrgError(NRG_ERR_ARG, "operator arrays missing");
  int64_t top = 0;
  for (int k = 0; k < M.nmatblocks; ++k) {
    const int i = M.mat_block_map[2 * k], j = M.mat_block_map[2 * k + 1];
    const int beg = M.mat_block_beg_end[2 * k], end = M.mat_block_beg_end[2 * k + 1];
    if (i < 0 || j < 0 || i >= blk.nblocks() || j >= blk.nblocks())
      throw NrgError(NRG_ERR_SYNC, "MatBlockMap names a block outside the kept structure");
    if (beg < 0 || (int64_t)end - beg + 1 != (int64_t)blk.size[i] * blk.size[j])
      throw NrgError(NRG_ERR_SYNC, "MatBlockBegEnd does not match the block sizes");
    om.bi.push_back(i); om.bj.push_back(j); om.off.push_back(beg);
    top = std::max<int64_t>(top, (int64_t)end + 1);
  }
  om.size = top;
  *nel = top;
  return om;
}

// DiagHN + SetE0zero for a caller-given basis (all eigenvectors).
void diag_hn_impl(nrg_ctx* c, int model, const double* params, int nparams, const nrg_blocks* old_kept, int nops,
                  const nrg_matrix* ops, const nrg_basis* abasis, double* en_out, double* evec_out, double* emin_out,
                  const nrg_model_desc* desc = nullptr) {
  const ModelSpec m = model_from_abi(model, desc);
  if (!params || nparams < m.nchan + 2) throw NrgError(NRG_ERR_ARG, "ParamsHN needs Lambda, chi per channel and e_N");
  if (nparams > m.nchan + 2 && params[m.nchan + 2] != 0.0)
    throw NrgError(NRG_ERR_ARG, "superconducting leads (Delta_SC != 0) are not supported");
  if (!(params[0] > 1.0)) throw NrgError(NRG_ERR_ARG, "Lambda must exceed 1");
  const int nops_h = m.nops_h;
  if (nops < nops_h || !ops) throw NrgError(NRG_ERR_ARG, "the model's f operators are required");
  if (!en_out || !evec_out) throw NrgError(NRG_ERR_ARG, "output arrays are NULL");
  std::memset(&c->timing, 0, sizeof(c->timing));
  const BlockArray K = blocks_from_abi(old_kept, "old_kept");
  Basis B;
  build_basis(m, K, B);
  check_basis(B, abasis);
  if (B.blk.nblocks() == 0) throw NrgError(NRG_ERR_ARG, "empty basis");
  HNTables tabs;
  build_hn_tables(m, B, tabs);
  std::vector<OpMeta> oldops(nops_h);
  std::vector<const double*> hops(8, nullptr);
  for (int o = 0; o < nops_h; ++o) {
    int64_t nel = 0;
    oldops[o] = op_from_abi(ops[o], K, &nel);
    c->ops_a[o].ensure(sizeof(double) * std::max<int64_t>(nel, 1));
    h2d(c, c->ops_a[o].p, ops[o].mat_el, sizeof(double) * nel);
    hops[o] = c->ops_a[o].as<double>();
  }
  const int ns = B.blk.nstates();
  std::vector<double> st_eold(abasis->en, abasis->en + ns);
  const double chi[2] = {params[1], m.nchan == 2 ? params[2] : 0.0};
  const double eN = params[1 + m.nchan];
  Timer tm(c);
  c->flag.ensure(sizeof(int) * 4);
  CU(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
  AsmTables AT = prepare_assembly(c, m, B, tabs, st_eold, oldops, K.size, nops_h, hops, params[0], chi, eN);
  EigPlan& P = AT.P;
  char* mb = c->meta.as<char>();
  cudaEvent_t ta = tm.start();
  launch_assemble(AT.aa, P.nstates, (const int*)(mb + AT.o_sb), (const int*)(mb + AT.o_ri), c->stream);
  c->launches++;
  tm.stop(ta, &c->timing.assemble_ms);
  run_tridiag_and_bisect(c, tm, P, AT.order, (const int*)(mb + AT.o_order), (const int*)(mb + AT.o_bsize),
                         (const int64_t*)(mb + AT.o_hoff), (const int*)(mb + AT.o_soff), (const int*)(mb + AT.o_sb));
  std::vector<double> ev(P.nstates);
  d2h(c, ev.data(), c->ev.p, sizeof(double) * P.nstates);
  CU(cudaStreamSynchronize(c->stream));
  check_flag(c);
  P.nvec = P.bsize;
  run_vectors(c, tm, P, ev, AT.aa.bsize, AT.aa.hoff, AT.aa.bstate);
  d2h(c, evec_out, c->Z.p, sizeof(double) * (size_t)P.ysize);
  CU(cudaStreamSynchronize(c->stream));
  check_flag(c);
  tm.collect();
  // SetE0zero (NRGarrayClass.cpp:234-241).
  const double emin = *std::min_element(ev.begin(), ev.end());
  for (int g = 0; g < P.nstates; ++g) en_out[g] = ev[g] - emin;
  if (emin_out) *emin_out = emin;
}

// SetKept + CutStates on the device cut kernels; the AeigCut bookkeeping is
// the host loop of CutStates.cpp:10-95 over the per-block kept counts.
void cut_states_impl(nrg_ctx* c, const nrg_blocks* aeig, const double* en, const double* evec, int ncutoff,
                     double eps, nrg_cut_result* out) {
  if (!en || !out) throw NrgError(NRG_ERR_ARG, "en/out is NULL");
  if (ncutoff < 1) throw NrgError(NRG_ERR_ARG, "Ncutoff must be positive");
  const BlockArray A = blocks_from_abi(aeig, "aeig");
  const int nb = A.nblocks(), ns = A.nstates();
  if (ns == 0) throw NrgError(NRG_ERR_ARG, "no states");
  double mn = en[0];
  for (int g = 1; g < ns; ++g) mn = std::min(mn, en[g]);
  if (mn != 0.0) throw NrgError(NRG_ERR_ARG, "energies must be E_min-shifted (SetE0zero) as DiagHN leaves them");
  std::memset(&c->timing, 0, sizeof(c->timing));
  Timer tm(c);
  EigPlan P;
  plan_blocks(P, A.size);
  std::vector<int> state_block(ns);
  for (int b = 0; b < nb; ++b) for (int i = 0; i < P.bsize[b]; ++i) state_block[P.soff[b] + i] = b;
  Packer pk;
  size_t o_bsize = pk.add(P.bsize), o_soff = pk.add(P.soff);
  c->meta.ensure(pk.host.size() + 256);
  c->ev.ensure(sizeof(double) * ns); c->en.ensure(sizeof(double) * ns);
  c->red.ensure(sizeof(int) * (nb + 8));
  c->scal.ensure(sizeof(double) * 32);
  c->flag.ensure(sizeof(int) * 4);
  CU(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
  h2d(c, c->meta.p, pk.host.data(), pk.host.size());
  h2d(c, c->ev.p, en, sizeof(double) * ns);
  char* mb = c->meta.as<char>();
  cudaEvent_t tc = tm.start();
  CutArgs ca{};
  ca.nstates = ns; ca.ev = c->ev.as<double>(); ca.en = c->en.as<double>(); ca.ncutoff = ncutoff; ca.eps = eps;
  ca.out_scalars = c->scal.as<double>(); ca.flag = c->flag.as<int>();
  launch_cut(ca, c->stream);
  BlockStatsArgs bs{};
  bs.nblocks = nb; bs.bsize = (const int*)(mb + o_bsize); bs.soff = (const int*)(mb + o_soff);
  bs.en = c->en.as<double>(); bs.scalars = ca.out_scalars; bs.kept = c->red.as<int>() + 4;
  launch_block_stats(bs, c->stream);
  c->launches += 2;
  std::vector<double> scal(4);
  std::vector<int> keptb(nb);
  c->out_en.resize(ns);
  d2h(c, scal.data(), c->scal.p, sizeof(double) * 4);
  d2h(c, keptb.data(), bs.kept, sizeof(int) * nb);
  d2h(c, c->out_en.data(), c->en.p, sizeof(double) * ns);
  tm.stop(tc, &c->timing.cut_ms);
  CU(cudaStreamSynchronize(c->stream));
  check_flag(c);
  tm.collect();
  const double ecut = scal[1];
  c->out_kept.assign(ns, 0);
  int nkept = 0;
  for (int g = 0; g < ns; ++g) if (c->out_en[g] <= ecut) { c->out_kept[g] = 1; ++nkept; }
  c->out_qn.clear(); c->out_bbe.clear(); c->out_bbe_bc.clear(); c->out_bbe_eig.clear(); c->out_stcf.clear();
  c->out_cut_en.clear(); c->out_cut_kept.clear(); c->out_vec.clear();
  int ist = 0;
  int64_t eig = 0, eoff = 0;
  for (int b = 0; b < nb; ++b) {
    const int n = P.bsize[b], k = keptb[b], b0 = P.soff[b];
    if (k > 0) {
      c->out_qn.push_back(A.q(b, 0)); c->out_qn.push_back(A.q(b, 1));
      c->out_bbe.push_back(ist); c->out_bbe.push_back(ist + k - 1);
      c->out_bbe_bc.push_back(b0); c->out_bbe_bc.push_back(b0 + n - 1);
      c->out_bbe_eig.push_back((int)eig); c->out_bbe_eig.push_back((int)(eig + (int64_t)k * n - 1));
      for (int i = 0; i < k; ++i) {
        c->out_stcf.push_back(b0 + i);
        c->out_cut_en.push_back(c->out_en[b0 + i]);
        c->out_cut_kept.push_back(c->out_kept[b0 + i]);
      }
      if (evec) c->out_vec.insert(c->out_vec.end(), evec + eoff, evec + eoff + (int64_t)k * n);
      eig += (int64_t)k * n;
      ist += k;
    }
    eoff += (int64_t)n * n;
  }
  out->en = c->out_en.data();
  out->kept = c->out_kept.data();
  out->nkept = nkept;
  out->ecut = ecut;
  nrg_eigcut& cut = out->cut;
  cut.blocks.nblocks = (int)c->out_bbe.size() / 2;
  cut.blocks.nqn = 2;
  cut.blocks.qnumbers = c->out_qn.data();
  cut.blocks.block_beg_end = c->out_bbe.data();
  cut.block_beg_end_bc = c->out_bbe_bc.data();
  cut.block_beg_end_eigvec = c->out_bbe_eig.data();
  cut.st_came_from = c->out_stcf.data();
  cut.en = c->out_cut_en.data();
  cut.kept = c->out_cut_kept.data();
  cut.eigvec = evec ? c->out_vec.data() : nullptr;
}

// UpdateMatrices for a caller-given AeigCut (kept rows of the eigenvectors
// uploaded as Z and Z^T) and old operators.
void update_ops_impl(nrg_ctx* c, int model, const nrg_blocks* old_kept, const nrg_basis* abasis, const nrg_eigcut* acut,
                     int nops, const nrg_matrix* old_ops, nrg_matrix* new_ops, const nrg_model_desc* desc = nullptr) {
  const ModelSpec m = model_from_abi(model, desc);
  if (nops != (int)m.op_kind.size() || !old_ops || !new_ops)
    throw NrgError(NRG_ERR_ARG, "nops must equal the model's operator count");
  if (!acut) throw NrgError(NRG_ERR_ARG, "acut is NULL");
  std::memset(&c->timing, 0, sizeof(c->timing));
  const BlockArray Kold = blocks_from_abi(old_kept, "old_kept");
  Basis B;
  build_basis(m, Kold, B);
  check_basis(B, abasis);
  Kept K;
  K.blk = blocks_from_abi(&acut->blocks, "acut");
  const int nk = K.blk.nblocks(), nb = B.blk.nblocks();
  if (nk > 0 && (!acut->eigvec || !acut->block_beg_end_eigvec)) throw NrgError(NRG_ERR_ARG, "acut eigvec missing");
  EigPlan P;
  plan_blocks(P, B.blk.size);
  P.nvec.assign(nb, 0);
  for (int i = 0; i < nk; ++i) {
    const int b = B.blk.find(&K.blk.qn[2 * i]);  // FindMatchBlock (FindMatchBlock.cpp:5-24)
    if (b < 0) throw NrgError(NRG_ERR_SYNC, "a kept block has no match in abasis");
    if (K.blk.size[i] > P.bsize[b]) throw NrgError(NRG_ERR_SYNC, "kept block larger than its basis block");
    if (P.nvec[b] != 0) throw NrgError(NRG_ERR_SYNC, "two kept blocks match one basis block");
    const int64_t len = (int64_t)acut->block_beg_end_eigvec[2 * i + 1] - acut->block_beg_end_eigvec[2 * i] + 1;
    if (acut->block_beg_end_eigvec[2 * i] < 0 || len != (int64_t)K.blk.size[i] * P.bsize[b])
      throw NrgError(NRG_ERR_SYNC, "BlockBegEndEigVec does not match kept x basis block size");
    K.src.push_back(b);
    P.nvec[b] = K.blk.size[i];
  }
  P.yoff.assign(nb, 0);
  int64_t y = 0;
  for (int b = 0; b < nb; ++b) { P.yoff[b] = y; y += (int64_t)P.bsize[b] * P.nvec[b]; }
  P.ysize = y;
  std::vector<double> Zh((size_t)std::max<int64_t>(y, 1)), Zth((size_t)std::max<int64_t>(y, 1));
  for (int i = 0; i < nk; ++i) {
    const int b = K.src[i], n = P.bsize[b], k = K.blk.size[i];
    const double* src = acut->eigvec + acut->block_beg_end_eigvec[2 * i];
    double* z = Zh.data() + P.yoff[b];
    double* zt = Zth.data() + P.yoff[b];
    std::memcpy(z, src, sizeof(double) * (size_t)k * n);
    for (int r = 0; r < k; ++r)
      for (int col = 0; col < n; ++col) zt[(size_t)col * k + r] = src[(size_t)r * n + col];
  }
  Timer tm(c);
  c->flag.ensure(sizeof(int) * 4);
  CU(cudaMemsetAsync(c->flag.p, 0, sizeof(int), c->stream));
  c->Z.ensure(sizeof(double) * std::max<int64_t>(y, 1));
  c->Zt.ensure(sizeof(double) * std::max<int64_t>(y, 1));
  h2d(c, c->Z.p, Zh.data(), sizeof(double) * y);
  h2d(c, c->Zt.p, Zth.data(), sizeof(double) * y);
  std::vector<OpMeta> oldops(nops);
  std::vector<double*> oldptr(8, nullptr), newptr(8, nullptr);
  for (int o = 0; o < nops; ++o) {
    int64_t nel = 0;
    oldops[o] = op_from_abi(old_ops[o], Kold, &nel);
    c->ops_a[o].ensure(sizeof(double) * std::max<int64_t>(nel, 1));
    h2d(c, c->ops_a[o].p, old_ops[o].mat_el, sizeof(double) * nel);
    oldptr[o] = c->ops_a[o].as<double>();
  }
  UpdatePlan U;
  plan_update(U, m, B, P, K, oldops);
  int64_t total = 0;
  std::vector<int64_t> obase(nops);
  for (int o = 0; o < nops; ++o) {
    c->ops_b[o].ensure(sizeof(double) * std::max<int64_t>(U.newops[o].size, 1));
    newptr[o] = c->ops_b[o].as<double>();
    obase[o] = total;
    total += U.newops[o].size;
  }
  U.o_old = U.up.add(oldptr);
  U.o_new = U.up.add(newptr);
  launch_update_plan(c, tm, U);
  c->out_el.resize((size_t)std::max<int64_t>(total, 1));
  for (int o = 0; o < nops; ++o)
    d2h(c, c->out_el.data() + obase[o], newptr[o], sizeof(double) * U.newops[o].size);
  CU(cudaStreamSynchronize(c->stream));
  check_flag(c);
  tm.collect();
  c->out_map.clear(); c->out_mbe.clear();
  std::vector<size_t> mbase(nops);
  for (int o = 0; o < nops; ++o) {
    const OpMeta& no = U.newops[o];
    mbase[o] = c->out_map.size();
    for (size_t k = 0; k < no.bi.size(); ++k) {
      const int64_t len = (int64_t)K.blk.size[no.bi[k]] * K.blk.size[no.bj[k]];
      if (no.off[k] + len > INT32_MAX) throw NrgError(NRG_ERR_SIZE, "operator exceeds MatBlockBegEnd's int range");
      c->out_map.push_back(no.bi[k]); c->out_map.push_back(no.bj[k]);
      c->out_mbe.push_back((int)no.off[k]); c->out_mbe.push_back((int)(no.off[k] + len - 1));
    }
  }
  for (int o = 0; o < nops; ++o) {
    new_ops[o].nmatblocks = (int)U.newops[o].bi.size();
    new_ops[o].mat_block_map = c->out_map.data() + mbase[o];
    new_ops[o].mat_block_beg_end = c->out_mbe.data() + mbase[o];
    new_ops[o].mat_el = c->out_el.data() + obase[o];
  }
}

// Register-only DFMA loop: eight independent chains per thread.
__global__ void fp64_peak_kernel(double* out, int iters, double seed) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + k + threadIdx.x * 1e-3;
  const double m = 0.999999999, s = 1e-9;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, s);
  }
  double t = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) t += a[k];
  if (t == 12345.678) out[0] = t;  // keeps the loop alive
}

double fp64_peak(nrg_ctx* c) {
  c->scal.ensure(sizeof(double) * 32);
  const int threads = 256, blocks = c->num_sms * 8, iters = 1 << 14;
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  fp64_peak_kernel<<<blocks, threads, 0, c->stream>>>(c->scal.as<double>(), 256, 1.0);  // warm-up
  CU(cudaEventRecord(a, c->stream));
  fp64_peak_kernel<<<blocks, threads, 0, c->stream>>>(c->scal.as<double>(), iters, 1.0);
  CU(cudaEventRecord(b, c->stream));
  CU(cudaEventSynchronize(b));
  c->launches += 2;
  float ms = 0.f;
  CU(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  const double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace
}  // namespace nrg

// ================================================================== C ABI
using namespace nrg;

#define GUARD(ctx, body)                                   \
  try {                                                    \
    body;                                                  \
  } catch (const NrgError& ex) {                           \
    if (ctx) (ctx)->err = ex.what();                       \
    return ex.st;                                          \
  } catch (const std::exception& ex) {                     \
    if (ctx) (ctx)->err = ex.what();                       \
    return NRG_ERR_ARG;                                    \
  }

static std::mutex g_batch_mu;
static std::string g_batch_err;

extern "C" {

const char* nrg_status_string(nrg_status s) {
  switch (s) {
    case NRG_OK: return "ok";
    case NRG_ERR_ARG: return "bad argument";
    case NRG_ERR_CUDA: return "CUDA error";
    case NRG_ERR_NOMEM: return "out of memory";
    case NRG_ERR_NOT_CONVERGED: return "not converged";
    case NRG_ERR_SIZE: return "size limit exceeded";
    case NRG_ERR_SYNC: return "block structures out of sync";
    case NRG_ERR_TIMEOUT: return "device wait timed out";
    case NRG_ERR_STATE: return "bad call order";
  }
  return "unknown";
}

nrg_status nrg_create(int device, nrg_ctx** out) {
  if (!out) return NRG_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return NRG_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return NRG_ERR_CUDA;
  if (prop.major < 10) return NRG_ERR_CUDA;  // built for sm_103a only
  if (cudaSetDevice(device) != cudaSuccess) return NRG_ERR_CUDA;
  nrg_ctx* c = new nrg_ctx();
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; return NRG_ERR_CUDA; }
  *out = c;
  return NRG_OK;
}

void nrg_destroy(nrg_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (int k = 0; k < nrg_ctx::kMaxSplit; ++k) {
    if (ctx->aux[k]) { cudaStreamSynchronize(ctx->aux[k]); cudaStreamDestroy(ctx->aux[k]); }
    if (ctx->join[k]) cudaEventDestroy(ctx->join[k]);
  }
  if (ctx->fork) cudaEventDestroy(ctx->fork);
  if (ctx->bsync) cudaEventDestroy(ctx->bsync);
  cudaStreamDestroy(ctx->stream);
  delete ctx->tan;
  ctx->tan = nullptr;
  nrg_ctx* chain = ctx->chain_ctx;
  delete ctx;
  nrg_destroy(chain);
}

const char* nrg_last_error(const nrg_ctx* ctx) {
  if (ctx) return ctx->err.c_str();
  std::lock_guard<std::mutex> lock(g_batch_mu);  // without a context: the last nrg_sweep_batch error
  return g_batch_err.c_str();
}

int64_t nrg_kernel_count(const nrg_ctx* ctx) { return ctx ? ctx->launches : 0; }

nrg_status nrg_sweep_run(nrg_ctx* ctx, const nrg_sweep_config* cfg) {
  if (!ctx || !cfg) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    sweep_run(ctx, cfg);
  });
  return NRG_OK;
}

nrg_status nrg_sweep_run_model(nrg_ctx* ctx, const nrg_sweep_config* cfg, const nrg_model_desc* model) {
  if (!ctx || !cfg || !model) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    sweep_run(ctx, cfg, false, false, nullptr, model);
  });
  return NRG_OK;
}

namespace {
nrg::ModelSpec host_model(int model, const nrg_model_desc* desc) {
  if (desc) return nrg::make_plugin_model(*desc);
  if (model < 0 || model > 5) throw std::invalid_argument("unknown model");
  return nrg::make_model((nrg::ModelKind)model);
}
}  // namespace

nrg_status nrg_model_hn_table(int model, const nrg_model_desc* desc, double s_block, double* coef, int cap, int* n) {
  if (!n) return NRG_ERR_ARG;
  try {
    const nrg::ModelSpec m = host_model(model, desc);
    nrg::Basis B;
    B.blk.nqn = 2;
    const double q[2] = {0.0, s_block};
    B.blk.push(q, 1);
    nrg::HNTables t;
    nrg::build_hn_tables(m, B, t);
    *n = (int)t.coef.size();
    if (coef && cap >= *n) std::copy(t.coef.begin(), t.coef.end(), coef);
  } catch (const std::exception&) {
    return NRG_ERR_ARG;
  }
  return NRG_OK;
}

nrg_status nrg_model_op_factor(int model, const nrg_model_desc* desc, int op, double s_i, double s_j, int ti, int tj,
                               double* out) {
  if (!out) return NRG_ERR_ARG;
  try {
    const nrg::ModelSpec m = host_model(model, desc);
    if (op < 0 || op >= (int)m.op_kind.size() || ti < 0 || tj < 0 || ti >= m.site.nstates || tj >= m.site.nstates)
      return NRG_ERR_ARG;
    const int k = m.op_kind[op];
    *out = k == nrg::OP_IMPONLY ? (ti == tj ? 1.0 : 0.0) : nrg::op_site_factor(m, k, s_i, s_j, ti, tj);
  } catch (const std::exception&) {
    return NRG_ERR_ARG;
  }
  return NRG_OK;
}

nrg_status nrg_model_op_check(int model, const nrg_model_desc* desc, int op, const double* qn_i, const double* qn_j,
                              int* out) {
  if (!out || !qn_i || !qn_j) return NRG_ERR_ARG;
  try {
    const nrg::ModelSpec m = host_model(model, desc);
    if (op < 0 || op >= (int)m.op_check.size()) return NRG_ERR_ARG;
    nrg::BlockArray a;
    a.nqn = 2;
    a.push(qn_i, 1);
    a.push(qn_j, 1);
    const bool same = qn_i[0] == qn_j[0] && qn_i[1] == qn_j[1];  // one kept block: Diag_check holds
    *out = nrg::op_check(m, m.op_check[op], a, 0, same ? 0 : 1) ? 1 : 0;
  } catch (const std::exception&) {
    return NRG_ERR_ARG;
  }
  return NRG_OK;
}

double nrg_clebsch(double j1, double m1, double j2, double m2, double j, double m) {
  return nrg::clebsch(j1, m1, j2, m2, j, m);
}

int nrg_sweep_num_iterations(const nrg_ctx* ctx) { return ctx ? (int)ctx->iters.size() : 0; }

nrg_status nrg_sweep_iteration(const nrg_ctx* ctx, int n, nrg_iteration* out) {
  if (!ctx || !out || n < 0 || n >= (int)ctx->iters.size()) return NRG_ERR_ARG;
  const IterResult& R = ctx->iters[n];
  out->nblocks = (int)R.bsize.size();
  out->qnumbers = R.qn.data();
  out->block_size = R.bsize.data();
  out->nstates = (int)R.en.size();
  out->en = R.en.data();
  out->emin = R.emin;
  out->ecut = R.ecut;
  out->nkept = R.nkept;
  out->nkept_blocks = (int)R.kept_bsize.size();
  out->kept_block_size = R.kept_bsize.data();
  out->thermo = R.thermo.data();
  out->nops = (int)R.opavg.size();
  out->opavg = R.opavg.data();
  out->params = R.params.data();
  out->wall_ms = R.wall_ms;
  out->device_ms = R.device_ms;
  return NRG_OK;
}

nrg_status nrg_sweep_opavg_initial(const nrg_ctx* ctx, int* nops, const double** vals) {
  if (!ctx || !nops || !vals) return NRG_ERR_ARG;
  *nops = (int)ctx->opavg_m1.size();
  *vals = ctx->opavg_m1.data();
  return NRG_OK;
}

nrg_status nrg_sweep_timing(const nrg_ctx* ctx, nrg_timing* out) {
  if (!ctx || !out) return NRG_ERR_ARG;
  *out = ctx->timing;
  return NRG_OK;
}

namespace {
nrg_status grad_forward_abi(nrg_ctx* ctx, const nrg_sweep_config* cfg, nrg_grad* out, bool dm) {
  if (!ctx || !cfg || !out) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    grad_forward_impl(ctx, cfg, dm);
  });
  const nrg::TangentState& T = *ctx->tan;
  out->nsites = (int)ctx->iters.size();
  out->nparams = nrg::TangentState::NP;
  out->nops = T.nops;
  out->d_thermo = T.dthermo.data();
  out->d_opavg = T.dopavg.data();
  out->d_emin = ctx->grad_demin.data();
  out->egs = ctx->grad_egs.data();
  out->d_egs = ctx->grad_degs.data();
  return NRG_OK;
}
}  // namespace

nrg_status nrg_grad_forward(nrg_ctx* ctx, const nrg_sweep_config* cfg, nrg_grad* out) {
  return grad_forward_abi(ctx, cfg, out, false);
}

nrg_status nrg_grad_forward_dm(nrg_ctx* ctx, const nrg_sweep_config* cfg, nrg_grad* out) {
  if (cfg && cfg->model != NRG_MODEL_1CH_QS) {
    if (ctx) ctx->err = "nrg_grad_forward_dm: DM-NRG tangents are built for NRG_MODEL_1CH_QS";
    return NRG_ERR_ARG;
  }
  return grad_forward_abi(ctx, cfg, out, true);
}

nrg_status nrg_lehmann_grad_backward(nrg_ctx* ctx, const double* g_rhow, double* grad) {
  if (!ctx || !g_rhow || !grad) return NRG_ERR_ARG;
  if (ctx->dm_drhow.empty()) {
    ctx->err = "nrg_lehmann_grad_backward needs a preceding nrg_lehmann_grad on the context";
    return NRG_ERR_STATE;
  }
  const int NP = nrg::DmTan::NP;
  const size_t nw = ctx->dm_drhow.size() / NP;
  for (int k = 0; k < NP; ++k) {
    double g = 0.0;
    for (size_t j = 0; j < nw; ++j) g += g_rhow[j] * ctx->dm_drhow[(size_t)k * nw + j];
    grad[k] = g;
  }
  return NRG_OK;
}

nrg_status nrg_grad_backward(nrg_ctx* ctx, const double* g_thermo, const double* g_opavg, const double* g_egs,
                             double* grad) {
  if (!ctx || !grad) return NRG_ERR_ARG;
  if (!ctx->tan || ctx->grad_egs.size() != ctx->iters.size()) {
    ctx->err = "nrg_grad_backward needs a preceding nrg_grad_forward on the context";
    return NRG_ERR_STATE;
  }
  const nrg::TangentState& T = *ctx->tan;
  const int NP = nrg::TangentState::NP, ni = (int)ctx->iters.size(), no = T.nops;
  for (int k = 0; k < NP; ++k) {
    double g = 0.0;
    for (int n = 0; n < ni; ++n) {
      const size_t r = (size_t)n * NP + k;
      if (g_thermo)
        for (int v = 0; v < 16; ++v) g += g_thermo[(size_t)n * 16 + v] * T.dthermo[r * 16 + v];
      if (g_opavg)
        for (int o = 0; o < no; ++o) g += g_opavg[(size_t)n * no + o] * T.dopavg[r * no + o];
      if (g_egs) g += g_egs[n] * ctx->grad_degs[r];
    }
    grad[k] = g;
  }
  return NRG_OK;
}

nrg_status nrg_set_precision(nrg_ctx* ctx, int precision) {
  if (!ctx || (precision != NRG_PREC_FP64 && precision != NRG_PREC_MIXED)) return NRG_ERR_ARG;
  ctx->precision = precision;
  return NRG_OK;
}

nrg_status nrg_gemm_f64_tensor(nrg_ctx* ctx, int m, int n, int k, double alpha, const double* A, int64_t lda,
                               const double* B, int64_t ldb, double* C, int64_t ldc, int slices) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  if (m < 0 || n < 0 || k < 0 || k > nrg::kOzMaxK || slices < 1 || slices > nrg::kOzMaxSlices) return NRG_ERR_ARG;
  if ((m > 0 && (!A || lda < k)) || (n > 0 && (!B || ldb < k)) || (m > 0 && n > 0 && (!C || ldc < n)))
    return NRG_ERR_ARG;
  if (m == 0 || n == 0 || k == 0) return NRG_OK;
  GUARD(ctx, {
    using namespace nrg;
    CU(cudaSetDevice(ctx->device));
    ctx->flag.ensure(sizeof(int) * 4);
    CU(cudaMemsetAsync(ctx->flag.p, 0, sizeof(int), ctx->stream));
    ctx->ozw.ensure(oz_work_bytes(m, n, k, slices));
    OzGemm g{};
    g.C = C; g.ldc = ldc; g.m = m; g.n = n; g.K = k; g.S = slices; g.alpha = alpha;
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.work = ctx->ozw.p; g.flag = ctx->flag.as<int>();
    CU(oz_gemm(g, ctx->stream));
    ctx->launches += 3;
    CU(cudaStreamSynchronize(ctx->stream));
    check_flag(ctx);
  });
  return NRG_OK;
}

nrg_status nrg_diag_blocks(nrg_ctx* ctx, int nblocks, const int* sizes, const double* packed_upper,
                           double* eigvals, double* eigvecs) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    diag_blocks_impl(ctx, nblocks, sizes, packed_upper, eigvals, eigvecs);
  });
  return NRG_OK;
}

nrg_status nrg_diag_hn(nrg_ctx* ctx, int model, const double* params_hn, int nparams, const nrg_blocks* old_kept,
                       int nops, const nrg_matrix* ops, const nrg_basis* abasis, double* en, double* eigvec,
                       double* emin) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    diag_hn_impl(ctx, model, params_hn, nparams, old_kept, nops, ops, abasis, en, eigvec, emin);
  });
  return NRG_OK;
}

nrg_status nrg_cut_states(nrg_ctx* ctx, const nrg_blocks* aeig, const double* en, const double* eigvec,
                          int ncutoff, double degen_eps, nrg_cut_result* out) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    cut_states_impl(ctx, aeig, en, eigvec, ncutoff, degen_eps > 0 ? degen_eps : 1.0e-18, out);
  });
  return NRG_OK;
}

nrg_status nrg_update_ops(nrg_ctx* ctx, int model, const nrg_blocks* old_kept, const nrg_basis* abasis,
                          const nrg_eigcut* acut, int nops, const nrg_matrix* old_ops, nrg_matrix* new_ops) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    update_ops_impl(ctx, model, old_kept, abasis, acut, nops, old_ops, new_ops);
  });
  return NRG_OK;
}

nrg_status nrg_diag_hn_model(nrg_ctx* ctx, const nrg_model_desc* model, const double* params_hn, int nparams,
                             const nrg_blocks* old_kept, int nops, const nrg_matrix* ops, const nrg_basis* abasis,
                             double* en, double* eigvec, double* emin) {
  if (!ctx || !model) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    diag_hn_impl(ctx, -1, params_hn, nparams, old_kept, nops, ops, abasis, en, eigvec, emin, model);
  });
  return NRG_OK;
}

nrg_status nrg_update_ops_model(nrg_ctx* ctx, const nrg_model_desc* model, const nrg_blocks* old_kept,
                                const nrg_basis* abasis, const nrg_eigcut* acut, int nops, const nrg_matrix* old_ops,
                                nrg_matrix* new_ops) {
  if (!ctx || !model) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    update_ops_impl(ctx, -1, old_kept, abasis, acut, nops, old_ops, new_ops, model);
  });
  return NRG_OK;
}

nrg_status nrg_sweep_run_dm(nrg_ctx* ctx, const nrg_sweep_config* cfg) {
  if (!ctx || !cfg) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    sweep_run(ctx, cfg, true);
  });
  return NRG_OK;
}

nrg_status nrg_set_chain(nrg_ctx* ctx, int n, const double* chi, const double* en, int apply_alambda) {
  if (!ctx || n < 0 || (n > 0 && (!chi || !en))) return NRG_ERR_ARG;
  ctx->chain_chi.assign(chi, chi + n);
  ctx->chain_en.assign(en, en + n);
  ctx->chain_alambda = apply_alambda != 0;
  ctx->chain_valid = false;  // stored free-chain values were for the previous chain
  if (ctx->chain_ctx) nrg_set_chain(ctx->chain_ctx, n, chi, en, apply_alambda);
  return NRG_OK;
}

nrg_status nrg_sweep_run_chain(nrg_ctx* ctx, const nrg_sweep_config* cfg) {
  if (!ctx || !cfg) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    sweep_run(ctx, cfg, false, true);
  });
  return NRG_OK;
}

nrg_status nrg_thermo_run(nrg_ctx* ctx, const nrg_sweep_config* cfg, int reuse_chain, nrg_thermo* out) {
  if (!ctx || !cfg || !out) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    thermo_run_impl(ctx, cfg, reuse_chain);
  });
  out->nvalues = (int)ctx->th_temp.size();
  out->temp = ctx->th_temp.data();
  out->suscep = ctx->th_sus.data();
  out->suscep_chain = ctx->th_sus_chain.data();
  out->suscep_imp = ctx->th_sus_imp.data();
  out->entropy = ctx->th_ent.data();
  out->entropy_chain = ctx->th_ent_chain.data();
  out->entropy_imp = ctx->th_ent_imp.data();
  out->chain_reused = ctx->th_chain_reused;
  out->chain_ms = ctx->th_chain_ms;
  out->imp_ms = ctx->th_imp_ms;
  out->total_ms = ctx->th_total_ms;
  return NRG_OK;
}

int nrg_dm_num_shells(const nrg_ctx* ctx) { return ctx ? (int)ctx->dm.size() : 0; }

nrg_status nrg_dm_backprop(nrg_ctx* ctx, const nrg_dm_params* prm, double* rho_trace) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    std::memset(&ctx->timing, 0, sizeof(ctx->timing));
    dm_backprop_impl(ctx, prm, rho_trace);
  });
  return NRG_OK;
}

nrg_status nrg_lehmann(nrg_ctx* ctx, const nrg_dm_params* prm, int nomega, const double* omegas, double* omega_rhow,
                       int* nout) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    std::memset(&ctx->timing, 0, sizeof(ctx->timing));
    lehmann_impl(ctx, prm, nomega, omegas, omega_rhow, nout);
  });
  return NRG_OK;
}

nrg_status nrg_lehmann_grad(nrg_ctx* ctx, const nrg_dm_params* prm, int nomega, const double* omegas,
                            double* omega_rhow, double* d_rhow, int* nout) {
  if (!ctx || !d_rhow) return NRG_ERR_ARG;
  ctx->err.clear();
  ctx->dm_drhow.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    std::memset(&ctx->timing, 0, sizeof(ctx->timing));
    lehmann_impl(ctx, prm, nomega, omegas, omega_rhow, nout, d_rhow);
  });
  return NRG_OK;
}

nrg_status nrg_dm_load_bin(nrg_ctx* ctx, const char* dir, const char* name, int nshells) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    dm_load_bin_impl(ctx, dir, name, nshells);
  });
  return NRG_OK;
}

nrg_status nrg_dm_save_bin(nrg_ctx* ctx, const char* dir, const char* name) {
  if (!ctx) return NRG_ERR_ARG;
  ctx->err.clear();
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    dm_save_bin_impl(ctx, dir, name);
  });
  return NRG_OK;
}

nrg_status nrg_sweep_batch(int device, int ninst, const nrg_sweep_config* cfgs, int nworkers, int max_sites,
                           double* thermo, double* opavg, int* nkept, double* seconds) {
  if (ninst < 0 || !cfgs || nworkers < 1 || max_sites < 1 || !thermo || !opavg || !nkept) return NRG_ERR_ARG;
  for (int i = 0; i < ninst; ++i)
    if (cfgs[i].nsites > max_sites) return NRG_ERR_ARG;
  auto t0 = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> lock(g_batch_mu);
    g_batch_err.clear();
  }
  // Largest instances first (kept count x iterations x site size): the
  // workers' device buffers reach their final size on their first instance,
  // so later instances do not reallocate (cudaFree waits for the whole
  // device, every worker's kernels included), and the last instances to
  // finish are short ones.
  std::vector<int> order(ninst);
  for (int i = 0; i < ninst; ++i) order[i] = i;
  auto cost = [&](int i) {
    const double site = cfgs[i].model == NRG_MODEL_2CH_QS ? 16.0 : 4.0;
    return (double)cfgs[i].ncutoff * site * cfgs[i].nsites;
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost(a) > cost(b); });
  std::atomic<int> next(0);
  std::atomic<int> status(NRG_OK);
  std::vector<std::thread> th;
  const int nw = std::min(nworkers, std::max(ninst, 1));
  for (int w = 0; w < nw; ++w) {
    th.emplace_back([&]() {
      nrg_ctx* c = nullptr;
      nrg_status st = nrg_create(device, &c);
      if (st != NRG_OK) {
        status.store(st);
        std::lock_guard<std::mutex> lock(g_batch_mu);
        if (g_batch_err.empty()) g_batch_err = "nrg_create failed in a batch worker";
        return;
      }
      c->shared_gpu = nw > 1;
      for (int k; (k = next.fetch_add(1)) < ninst;) {
        const int i = order[k];
        st = nrg_sweep_run(c, &cfgs[i]);
        if (st != NRG_OK) {
          status.store(st);
          std::lock_guard<std::mutex> lock(g_batch_mu);
          if (g_batch_err.empty()) g_batch_err = "instance " + std::to_string(i) + ": " + c->err;
          break;
        }
        for (int n = 0; n < (int)c->iters.size(); ++n) {
          const IterResult& R = c->iters[n];
          const size_t row = (size_t)i * max_sites + n;
          std::copy(R.thermo.begin(), R.thermo.end(), thermo + row * 16);
          for (int k = 0; k < 4; ++k) opavg[row * 4 + k] = k < (int)R.opavg.size() ? R.opavg[k] : 0.0;
          nkept[row] = R.nkept;
        }
      }
      nrg_destroy(c);
    });
  }
  for (auto& t : th) t.join();
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return (nrg_status)status.load();
}

nrg_status nrg_fp64_peak(nrg_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return NRG_ERR_ARG;
  GUARD(ctx, {
    CU(cudaSetDevice(ctx->device));
    *tflops = fp64_peak(ctx);
  });
  return NRG_OK;
}

}  // extern "C"
