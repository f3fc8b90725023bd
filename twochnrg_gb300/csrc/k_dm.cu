// DM-NRG on the device: density-matrix backward sweep and Lehmann sums.
//
// The reference DM_NRG (src/DM_NRG/DM_NRG.cpp) rotates rho_{N+1} back into
// the product basis with two uBLAS products per block (RotateMatrix,
// RotateMatrix.cpp:17-99), traces out the last site element by element over
// child-state lists (DM_NRG_CalcRhoN_withSU2, DM_NRG_CalcRhoN.cpp:252-449),
// and for every frequency redoes two dgemm per block pair and kept/discarded
// split (FDM_SpecDens_M_STL, SpecFunc_allSTL.cpp:1253-2358).  Here the
// rotations and the rho.A / A.rho products are one grouped FP64 GEMM launch
// per shell, the partial trace is a gather over per-block term lists, and the
// frequency dependence is isolated: every shell becomes a list of
// (E_j - E_i, weight) pairs once, and the Lehmann kernel streams those pairs
// for every frequency, with the log-Gaussian / Gaussian kernels of
// BroadDelta.cpp evaluated on the fly.
#include "nrg_device.cuh"

namespace nrg {

namespace {

constexpr int TM = 64, TN = 64, TK = 16;

__global__ void __launch_bounds__(256) gemm_jobs_kernel(const GemmJob* jobs, const int* tile_job, const int* tile_mn) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN];
  const GemmJob J = jobs[tile_job[blockIdx.x]];
  const int mn = tile_mn[blockIdx.x];
  const int m0 = (mn >> 16) * TM, n0 = (mn & 0xffff) * TN;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < J.k; k0 += TK) {
    for (int idx = threadIdx.x; idx < TM * TK; idx += 256) {
      const int r = idx / TK, c = idx - r * TK;
      const int gr = m0 + r, gc = k0 + c;
      double v = 0.0;
      if (gr < J.m && gc < J.k) v = J.transA ? J.A[(int64_t)gc * J.lda + gr] : J.A[(int64_t)gr * J.lda + gc];
      As[c][r] = v;
    }
    for (int idx = threadIdx.x; idx < TK * TN; idx += 256) {
      const int r = idx / TN, c = idx - r * TN;
      const int gr = k0 + r, gc = n0 + c;
      Bs[r][c] = (gr < J.k && gc < J.n) ? J.B[(int64_t)gr * J.ldb + gc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + ty + 16 * i;
    if (r >= J.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tx + 16 * j;
      if (c < J.n) J.C[(int64_t)r * J.ldc + c] = acc[i][j];
    }
  }
}

// One CTA per block of shell N.  Kept x kept elements are the SU(2)-weighted
// sums over the block's child terms, evaluated for i <= j and mirrored (the
// reference fills the upper triangle); a discarded state's diagonal is its
// FDM Boltzmann weight; everything else is zero.
__global__ void __launch_bounds__(256) dm_trace_kernel(DmTraceArgs A) {
  const int b = blockIdx.x;
  const int n = A.bsize[b], k = A.nkept[b], s0 = A.soff[b];
  const int t0 = A.term_first[b], nt = A.term_count[b];
  double* R = A.rho + A.roff[b];
  for (int64_t idx = threadIdx.x; idx < (int64_t)n * n; idx += blockDim.x) {
    const int i = (int)(idx / n), j = (int)(idx - (int64_t)i * n);
    const int ii = i < j ? i : j, jj = i < j ? j : i;
    double v = 0.0;
    if (jj < k) {
      for (int t = t0; t < t0 + nt; ++t) {
        const DmTraceTerm T = A.terms[t];
        if (jj < T.count)
          v += T.cg * A.rot[T.rot_off + (int64_t)(T.base + ii * T.stride) * T.nb + T.base + jj * T.stride];
      }
    }
    if (i == j && !A.kept[s0 + i] && A.zdisc != 0.0) v = exp(-A.beta * A.en[s0 + i]) / A.zdisc;
    R[idx] = v;
  }
}

// One CTA per block pair of c_d: the (E_j - E_i, weight) pairs.
__global__ void __launch_bounds__(256) dm_pairs_kernel(DmPairArgs A) {
  const DmPair P = A.pairs[blockIdx.x];
  const int64_t n = (int64_t)P.n1 * P.n2;
  for (int64_t idx = threadIdx.x; idx < n; idx += blockDim.x) {
    const int a = (int)(idx / P.n2), b = (int)(idx - (int64_t)a * P.n2);
    const double m = A.cd[P.a_off + idx];
    const double E1 = A.en[P.s1 + a], E2 = A.en[P.s2 + b];
    double wp = 0.0, wn = 0.0;
    if (A.last) {
      const double sum12 = m * exp(-A.beta_last * E1) + exp(-A.beta_last * E2) * m;
      wp = wn = P.cg * (sum12 * m) * A.inv_z_last;
    } else if (!P.skip) {
      const double w = P.cg * ((A.P1[P.p_off + idx] + A.P2[P.p_off + idx]) * m);
      if (!A.kept[P.s2 + b]) wp = w;
      if (!A.kept[P.s1 + a]) wn = w;
    }
    A.dE[P.out_off + idx] = E2 - E1;
    A.Wp[P.out_off + idx] = wp;
    A.Wn[P.out_off + idx] = wn;
  }
}

// LogGaussDelta (BroadDelta.cpp:116-133), replaced by GaussDelta
// (BroadDelta.cpp:96-106) inside the thermal window, as MijxBDeltaEij does.
__device__ __forceinline__ double broad_delta(double om, double dE, double b, double tw, double bt, double tempdn) {
  const double sqrt_pi = 1.7724538509055160273;
  if (fabs(dE) < tw * tempdn) {
    const double a1 = (om - dE) / bt;
    return (1.0 / (bt * sqrt_pi)) * exp(-a1 * a1);
  }
  const double Ep = dE == 0.0 ? 1.0e-100 : dE;
  if (om * Ep < 0.0) return 0.0;
  const double a0 = 1.0 / (b * fabs(Ep) * sqrt_pi);
  const double a1 = log(fabs(om / Ep)) / b;
  const double x = a1 - b / 4.0;
  return a0 * exp(-x * x);
}

// grid (frequency, shell slot of its window): one shell's pairs per CTA.
__global__ void __launch_bounds__(256) lehmann_kernel(LehmannArgs A) {
  __shared__ double red[8];
  const int k = blockIdx.x, s = blockIdx.y;
  double acc = 0.0;
  int N = -1;
  if (s < A.win_count[k]) {
    N = A.win_first[k] + s;
    const double dn = A.dn[N];
    const double om = A.omega[k] / dn;
    const double tempdn = A.tempdn[N];
    const double* W = om >= 0.0 ? A.Wp : A.Wn;
    for (int64_t p = A.shell_off[N] + threadIdx.x; p < A.shell_off[N + 1]; p += blockDim.x) {
      const double w = W[p];
      if (w != 0.0) acc += w * broad_delta(om, A.dE[p], A.b, A.twindow, A.broadtemp, tempdn);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    A.partial[(int64_t)k * A.window + s] = N >= 0 ? t / A.dn[N] : 0.0;
  }
}

__global__ void lehmann_fold_kernel(LehmannArgs A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.nomega) return;
  double t = 0.0;
  for (int s = 0; s < A.window; ++s) t += A.partial[(int64_t)k * A.window + s];
  A.out[k] = t;
}

}  // namespace

void launch_gemm_jobs(const GemmJob* jobs, const int* tile_job, const int* tile_mn, int ntiles, cudaStream_t s) {
  if (ntiles > 0) gemm_jobs_kernel<<<ntiles, 256, 0, s>>>(jobs, tile_job, tile_mn);
}

void launch_dm_trace(const DmTraceArgs& a, int nblocks, cudaStream_t s) {
  if (nblocks > 0) dm_trace_kernel<<<nblocks, 256, 0, s>>>(a);
}

void launch_dm_pairs(const DmPairArgs& a, int npairs_blocks, cudaStream_t s) {
  if (npairs_blocks > 0) dm_pairs_kernel<<<npairs_blocks, 256, 0, s>>>(a);
}

void launch_lehmann(const LehmannArgs& a, cudaStream_t s) {
  if (a.nomega <= 0) return;
  lehmann_kernel<<<dim3(a.nomega, a.window), 256, 0, s>>>(a);
  lehmann_fold_kernel<<<(a.nomega + 127) / 128, 128, 0, s>>>(a);
}

}  // namespace nrg
