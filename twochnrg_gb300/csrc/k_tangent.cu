// Tangents of the NRG sweep with respect to the model parameters (the
// derivative pass behind nrg_grad_forward / nrg_grad_backward).
//
// The reference has no derivative code; its Hellmann-Feynman averages
// (CalcOpAvg of n_d, n_d^2 and S_z, CalcOpAvg.cpp:13-84, set up in
// CodeHandler_ModelSwitch.cpp:748-780) are what these derivatives are checked
// against, besides finite differences.  At a fixed kept-state set the sweep is
// a smooth map parameters -> observables, and one tangent direction dp is
// carried through every step:
//
//   dH_N            the assembly kernel on (dE_old, dO_old) (H_N is linear in them)
//   dH~ = Z^T dH Z  two grouped GEMMs with every eigenvector of the block
//   dlambda_k       = dH~_kk
//   dz_l            = sum_k z_k dH~_kl / (lambda_l - lambda_k)     (kept l)
//                     with no coupling inside a degenerate level (|gap| below
//                     a tolerance), where the eigenvectors are not determined
//   dO_new          = dZ_I F Z_J^T + Z_I F dZ_J^T + Z_I dF Z_J^T   (the update plan, three times)
//   d<O>, dTchi     weighted sums below
//
// This file holds the small kernels of that pass; the GEMMs and the
// rotation reuse the sweep's own kernels.
#include <algorithm>

#include "nrg_device.cuh"

namespace nrg {

namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 304;  // two CTAs per SM for the reductions

// One CTA per block: dlambda and the coupling matrix C (n x kept, row-major)
// of the block's kept eigenvectors.
__global__ void __launch_bounds__(kThreads) tan_eig_kernel(TanEigArgs A) {
  const int b = blockIdx.x;
  const int n = A.bsize[b], k = A.nkeep[b];
  const double* D = A.dHt + A.hoff[b];
  const double* lam = A.ev + A.soff[b];
  double lmax = 0.0;
  for (int i = 0; i < n; ++i) lmax = fmax(lmax, fabs(lam[i]));
  const double tol = A.degen_tol * fmax(1.0, lmax);
  for (int x = threadIdx.x; x < n; x += blockDim.x) A.dlam[A.soff[b] + x] = D[(int64_t)x * n + x];
  double* C = A.C + A.coff[b];
  for (int idx = threadIdx.x; idx < n * k; idx += blockDim.x) {
    const int r = idx / k, l = idx - r * k;
    const double gap = lam[l] - lam[r];
    C[idx] = (r == l || fabs(gap) <= tol) ? 0.0 : D[(int64_t)r * n + l] / gap;
  }
}

// dE of every state (shifted: dlambda - dlambda of the ground state) into
// dE_all, and the kept states' dE in the kept order into dE_kept.
__global__ void tan_shift_kernel(const double* dlam, int nstates, int gs, double* dE_all, const int* kept_state,
                                 int nkept, double* dE_kept) {
  const double g = dlam[gs];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nstates; i += gridDim.x * blockDim.x)
    dE_all[i] = dlam[i] - g;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nkept; i += gridDim.x * blockDim.x)
    dE_kept[i] = dlam[kept_state[i]] - g;
}

// Per new-basis state g, the tangent of the old energy it came from.
__global__ void tan_gather_kernel(const double* dE_kept_old, const int* stcf, int n, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = dE_kept_old[stcf[i]];
}

__global__ void tan_axpy3_kernel(const double* a, const double* b, const double* c, double s, int64_t n, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = s * (a[i] + b[i] + c[i]);
}

__global__ void tan_scale_kernel(const double* a, double s, int64_t n, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = s * a[i];
}

// Partial sums over states, in a fixed order per CTA (deterministic):
// per temperature t: sum deg w dE, sum SzSq w dE, sum deg E w dE, with w = e^{-beta_t E};
// then per averaged operator o over the kept states at betabar:
// sum deg w dO_ii, sum deg w O_ii dE, and sum deg w dE.
__global__ void __launch_bounds__(kThreads) tan_sums_kernel(TanSumArgs A, double* partial) {
  constexpr int W = TanSumArgs::kMaxOut;
  double acc[W];
  for (int t = 0; t < W; ++t) acc[t] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.nstates; i += gridDim.x * blockDim.x) {
    const int b = A.state_block[i];
    const double S = A.bq[2 * b + 1];
    const double deg = A.totalS ? 2.0 * S + 1.0 : 1.0;
    const double szsq = A.totalS ? (1.0 / 12.0) * deg * (deg * deg - 1.0) : S * S;
    const double E = A.en[i], dE = A.dE[i];
    for (int t = 0; t < 4; ++t) {
      const double w = exp(-A.beta[t] * E);
      acc[3 * t] += deg * w * dE;
      acc[3 * t + 1] += szsq * w * dE;
      acc[3 * t + 2] += deg * E * w * dE;
    }
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.nkept; i += gridDim.x * blockDim.x) {
    const int kb = A.kstate_block[i];
    const int x = i - A.koff[kb];
    const double deg = A.totalS ? 2.0 * A.kbq[2 * kb + 1] + 1.0 : 1.0;
    const double E = A.ken[i], dE = A.dEk[i];
    const double w = deg * exp(-A.betabar * E);
    for (int o = 0; o < A.nops; ++o) {
      const int64_t off = A.diag_off[o * A.nkblocks + kb];
      const int64_t e = off >= 0 ? off + (int64_t)x * A.kld[kb] + x : -1;
      const double O = e >= 0 ? A.ops[o][e] : 0.0, dO = e >= 0 ? A.dops[o][e] : 0.0;
      acc[12 + 2 * o] += w * dO;
      acc[12 + 2 * o + 1] += w * O * dE;
    }
    acc[W - 1] += w * dE;
  }
  __shared__ double sh[kThreads / 32][W];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t = 0; t < W; ++t) {
    double v = acc[t];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][t] = v;
  }
  __syncthreads();
  if (threadIdx.x < W) {
    double v = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) v += sh[w][threadIdx.x];
    partial[(size_t)blockIdx.x * W + threadIdx.x] = v;
  }
}

__global__ void tan_fold_kernel(const double* partial, int nparts, double* out) {
  constexpr int W = TanSumArgs::kMaxOut;
  const int t = threadIdx.x;
  if (t >= W) return;
  double v = 0.0;
  for (int p = 0; p < nparts; ++p) v += partial[(size_t)p * W + t];
  out[t] = v;
}

int grid_for(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 1184); }

}  // namespace

void launch_tan_eig(const TanEigArgs& a, int nblocks, cudaStream_t s) {
  if (nblocks > 0) tan_eig_kernel<<<nblocks, kThreads, 0, s>>>(a);
}
void launch_tan_shift(const double* dlam, int nstates, int gs, double* dE_all, const int* kept_state, int nkept,
                      double* dE_kept, cudaStream_t s) {
  tan_shift_kernel<<<grid_for(std::max(nstates, nkept)), 256, 0, s>>>(dlam, nstates, gs, dE_all, kept_state, nkept,
                                                                       dE_kept);
}
void launch_tan_gather(const double* dE_kept_old, const int* stcf, int n, double* out, cudaStream_t s) {
  if (n > 0) tan_gather_kernel<<<grid_for(n), 256, 0, s>>>(dE_kept_old, stcf, n, out);
}
void launch_tan_axpy3(const double* a, const double* b, const double* c, double scale, int64_t n, double* out,
                      cudaStream_t s) {
  if (n > 0) tan_axpy3_kernel<<<grid_for(n), 256, 0, s>>>(a, b, c, scale, n, out);
}
void launch_tan_scale(const double* a, double scale, int64_t n, double* out, cudaStream_t s) {
  if (n > 0) tan_scale_kernel<<<grid_for(n), 256, 0, s>>>(a, scale, n, out);
}
size_t tan_partial_doubles() { return (size_t)kBlocks * TanSumArgs::kMaxOut; }
void launch_tan_sums(const TanSumArgs& a, double* partial, double* out, cudaStream_t s) {
  tan_sums_kernel<<<kBlocks, kThreads, 0, s>>>(a, partial);
  tan_fold_kernel<<<1, 32, 0, s>>>(partial, kBlocks, out);
}

}  // namespace nrg
