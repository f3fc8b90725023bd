// Truncation and per-iteration observables on the device.
//
// cut_kernel restates, for the whole spectrum of one iteration:
//   CNRGarray::SetE0zero  (NRGarrayClass.cpp:234-241)  subtract the global minimum,
//   CNRGarray::SetDegen   (NRGarrayClass.cpp:244-268)  pairwise merge of levels
//                                                       closer than MyEPS,
//   CNRGarray::Ecut       (NRGarrayClass.cpp:661-691)  Ncutoff-th level widened
//                                                       over the 1% window,
//   CNRGarray::SetKept    (NRGarrayClass.cpp:461-491)  Kept = E <= Ecut.
// The Ncutoff-th level is found by an 8-pass radix select on the IEEE bit
// patterns (non-negative doubles order like their bits).  Because the sorted
// walk of the reference's window stops at the first level whose relative
// distance to E_sorted[Ncut-1] reaches 1%, and that distance is monotone in
// the level, the widened Ecut is the largest level within the window, which
// one max-reduction finds.  SetDegen can only move a level that has a
// different neighbour closer than MyEPS; such levels are below MyEPS*2^53, so
// the reference's O(n^2) loop runs exactly, in index order, on that set only.
//
// block_stats_kernel restates the block bookkeeping of CutStates
// (CutStates.cpp:38-90): a block whose lowest level is above Ecut is removed,
// every other block keeps its leading run of levels <= Ecut
// (GetBlockEcutPos, NRGarrayClass.cpp:439-457).
//
// thermo_kernel / opdiag_kernel: Boltzmann sums of CalcSuscep, CalcEntropy
// (CalcThermo.cpp:16-121) and CalcOpAvg (CalcOpAvg.cpp:13-84), reduced in a
// fixed order (per-CTA partials, then one ordered pass).
#include <cfloat>

#include "nrg_device.cuh"

namespace nrg {

namespace {

constexpr int kCutThreads = 1024;
constexpr int kDegenMax = 2048;

__device__ double block_reduce_min(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmin(m, red[w]);
    red[32] = m;
  }
  __syncthreads();
  return red[32];
}

__device__ double block_reduce_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    red[32] = m;
  }
  __syncthreads();
  return red[32];
}

__global__ void __launch_bounds__(kCutThreads) cut_kernel(CutArgs A) {
  __shared__ double red[40];
  __shared__ unsigned int hist[256];
  __shared__ int cand_idx[kDegenMax];
  __shared__ double cand_val[kDegenMax];
  __shared__ int ncand;
  __shared__ unsigned long long prefix_s;
  __shared__ int kk_s;
  const int n = A.nstates;
  double* en = A.en;
  // SetE0zero
  double m = DBL_MAX;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmin(m, A.ev[i]);
  const double emin = block_reduce_min(m, red);
  for (int i = threadIdx.x; i < n; i += blockDim.x) en[i] = A.ev[i] - emin;
  if (threadIdx.x == 0) ncand = 0;
  __syncthreads();
  // SetDegen on the levels that can have a distinct neighbour within eps.
  const double lim = A.eps * 9007199254740992.0;  // eps * 2^53
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (en[i] < lim) {
      const int p = atomicAdd(&ncand, 1);
      if (p < kDegenMax) cand_idx[p] = i;
    }
  }
  __syncthreads();
  if (ncand > kDegenMax) {
    if (threadIdx.x == 0) atomicOr(A.flag, DEV_DEGEN_OVERFLOW);
  } else if (threadIdx.x == 0 && ncand > 1) {
    const int c = ncand;
    // index order, as the reference's double loop runs
    for (int a = 1; a < c; ++a) {
      int x = cand_idx[a], b = a - 1;
      while (b >= 0 && cand_idx[b] > x) { cand_idx[b + 1] = cand_idx[b]; --b; }
      cand_idx[b + 1] = x;
    }
    for (int a = 0; a < c; ++a) cand_val[a] = en[cand_idx[a]];
    for (int a = 0; a < c; ++a)
      for (int b = a + 1; b < c; ++b)
        if (fabs(cand_val[b] - cand_val[a]) < A.eps) {
          if (cand_val[b] > cand_val[a]) cand_val[b] = cand_val[a]; else cand_val[a] = cand_val[b];
        }
    for (int a = 0; a < c; ++a) en[cand_idx[a]] = cand_val[a];
  }
  __syncthreads();
  // Ecut
  double ecut;
  if ((long long)A.ncutoff >= (long long)n - 1) {
    double mx = -DBL_MAX;
    for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, en[i]);
    ecut = block_reduce_max(mx, red);
  } else {
    // radix select of the (Ncut-1)-th smallest level (0-based)
    if (threadIdx.x == 0) { prefix_s = 0ull; kk_s = A.ncutoff - 1; }
    __syncthreads();
    for (int pass = 7; pass >= 0; --pass) {
      for (int h = threadIdx.x; h < 256; h += blockDim.x) hist[h] = 0u;
      __syncthreads();
      const unsigned long long prefix = prefix_s;
      const int shift = pass * 8;
      const unsigned long long hmask = (pass == 7) ? 0ull : (~0ull << (shift + 8));
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const unsigned long long key = (unsigned long long)__double_as_longlong(en[i]);
        if ((key & hmask) == (prefix & hmask)) atomicAdd(&hist[(key >> shift) & 0xffull], 1u);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        int k = kk_s;
        unsigned int acc = 0;
        int digit = 0;
        for (; digit < 256; ++digit) {
          if (acc + hist[digit] > (unsigned)k) break;
          acc += hist[digit];
        }
        kk_s = k - (int)acc;
        prefix_s = prefix | ((unsigned long long)digit << shift);
      }
      __syncthreads();
    }
    const double aux = __longlong_as_double((long long)prefix_s);
    double mx = aux;
    if (aux > 0.0) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double x = en[i];
        if (x >= aux && fabs((x - aux) / aux) < 0.01) mx = fmax(mx, x);
      }
    }
    ecut = block_reduce_max(mx, red);
  }
  int cnt = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) cnt += en[i] <= ecut ? 1 : 0;
  __shared__ int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  atomicAdd(&total, cnt);
  __syncthreads();
  if (threadIdx.x == 0) {
    A.out_scalars[0] = emin;
    A.out_scalars[1] = ecut;
    A.out_scalars[2] = (double)total;
  }
}

__global__ void block_stats_kernel(BlockStatsArgs A) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= A.nblocks) return;
  const double ecut = A.scalars[1];
  const double* e = A.en + A.soff[b];
  const int n = A.bsize[b];
  double mn = DBL_MAX;
  for (int i = 0; i < n; ++i) mn = fmin(mn, e[i]);
  int k = 0;
  if (!(mn > ecut)) {
    while (k < n && e[k] <= ecut) ++k;
  }
  A.kept[b] = k;
}

constexpr int kRedThreads = 256;

// Per-CTA partials of the thermodynamic sums; a second launch folds them.
__global__ void __launch_bounds__(kRedThreads) thermo_partial_kernel(ThermoArgs A, const int* state_block, int n,
                                                                     double* partial) {
  __shared__ double sh[kRedThreads / 32][12];
  double acc[12];
  for (int t = 0; t < 12; ++t) acc[t] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int b = state_block[i];
    const double S = A.bq[2 * b + 1];
    double deg, szsq;
    if (A.totalS) {
      deg = 2.0 * S + 1.0;
      szsq = (1.0 / 12.0) * deg * (deg * deg - 1.0);
    } else {
      deg = 1.0;
      szsq = S * S;
    }
    const double E = A.en[i];
    for (int t = 0; t < 4; ++t) {
      const double w = exp(-A.beta[t] * E);
      acc[3 * t + 0] += deg * w;
      acc[3 * t + 1] += szsq * w;
      acc[3 * t + 2] += deg * E * w;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t = 0; t < 12; ++t) {
    double v = acc[t];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][t] = v;
  }
  __syncthreads();
  if (threadIdx.x < 12) {
    double s = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) s += sh[w][threadIdx.x];
    partial[blockIdx.x * 12 + threadIdx.x] = s;
  }
}

__global__ void fold_kernel(const double* partial, int nparts, int width, double* out) {
  const int t = threadIdx.x;
  if (t >= width) return;
  double s = 0.0;
  for (int p = 0; p < nparts; ++p) s += partial[p * width + t];
  out[t] = s;
}

__global__ void __launch_bounds__(kRedThreads) opdiag_partial_kernel(OpDiagArgs A, const int* kstate_block, int nk,
                                                                     double* partial) {
  __shared__ double sh[kRedThreads / 32][9];
  double acc[9];
  const int W = A.nops + 1;
  for (int t = 0; t < 9; ++t) acc[t] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nk; i += gridDim.x * blockDim.x) {
    const int b = kstate_block[i];
    const int x = i - A.koff[b];
    const int kb = A.kld ? A.kld[b] : A.ksize[b];
    const double deg = A.totalS ? 2.0 * A.bq[2 * b + 1] + 1.0 : 1.0;
    const double w = exp(-A.beta * A.ken[i]);
    for (int o = 0; o < A.nops; ++o) {
      const int64_t off = A.diag_off[o * A.nblocks + b];
      const double el = off >= 0 ? A.ops[o][off + (int64_t)x * kb + x] : 0.0;
      acc[o] += deg * el * w;
    }
    acc[A.nops] += deg * w;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t = 0; t < W; ++t) {
    double v = acc[t];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][t] = v;
  }
  __syncthreads();
  if (threadIdx.x < W) {
    double s = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) s += sh[w][threadIdx.x];
    partial[blockIdx.x * W + threadIdx.x] = s;
  }
}

}  // namespace

void launch_cut(const CutArgs& a, cudaStream_t s) { cut_kernel<<<1, kCutThreads, 0, s>>>(a); }

void launch_block_stats(const BlockStatsArgs& a, cudaStream_t s) {
  if (a.nblocks > 0) block_stats_kernel<<<(a.nblocks + 63) / 64, 64, 0, s>>>(a);
}

constexpr int kRedBlocks = 64;

void launch_thermo(const ThermoArgs& a, const int* state_block, int n, double* partial, cudaStream_t s) {
  thermo_partial_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(a, state_block, n, partial);
  fold_kernel<<<1, 32, 0, s>>>(partial, kRedBlocks, 12, a.out);
}

void launch_opdiag(const OpDiagArgs& a, const int* kstate_block, int nk, double* partial, cudaStream_t s) {
  opdiag_partial_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(a, kstate_block, nk, partial);
  fold_kernel<<<1, 32, 0, s>>>(partial, kRedBlocks, a.nops + 1, a.out);
}

int reduce_partial_count() { return kRedBlocks; }

}  // namespace nrg
