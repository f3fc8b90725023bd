// Operator rotation into the new kept basis (FP64).
//
// Replaces the per-pair element loop and the two cblas_dgemm calls of
// UpdateMatrices (UpdateMatrices.cpp:333-560): O_new(i,j) = Z_i . F(i,j) . Z_j^T.
// F is never formed: it is a sum of site-structured terms (an f-type operator
// acts on the new site only, so F couples states that came from the same old
// state; an impurity operator acts on the old part only, so F is the old
// operator block between states of the same site type).  gather_kernel
// builds T = F . Z_j^T row group by row group from those terms (no atomics:
// each CTA owns one destination row group), then gemm_kernel forms
// O = Z_i . T for every (operator, block pair) job of the iteration in one
// grouped launch.
#include "nrg_device.cuh"

namespace nrg {

namespace {

__global__ void __launch_bounds__(256) gather_kernel(UpdateArgs A) {
  const int g = blockIdx.x;
  const int t0 = A.group_first[g], nt = A.group_count[g];
  for (int t = t0; t < t0 + nt; ++t) {
    const GatherTerm G = A.terms[t];
    const RotJob J = A.jobs[G.job];
    const int kj = J.kj;
    double* T = A.T + J.t_off;
    const double* Zt = A.Zt + J.zt_off;
    if (G.mode == 0) {
      for (int idx = threadIdx.x; idx < G.rows * kj; idx += blockDim.x) {
        const int a = idx / kj, c = idx - a * kj;
        double* dst = T + (int64_t)(G.dst_base + a * G.dst_stride) * kj + c;
        *dst = fma(G.coef, Zt[(int64_t)(G.src_base + a * G.src_stride) * J.ldz + c], *dst);
      }
    } else {
      const double* M = A.old_ops[G.op] + G.old_off;
      for (int idx = threadIdx.x; idx < G.rows * kj; idx += blockDim.x) {
        const int a = idx / kj, c = idx - a * kj;
        double acc = 0.0;
        const double* Ma = M + (int64_t)a * G.old_ld;
        for (int bb = 0; bb < G.srows; ++bb)
          acc = fma(Ma[bb], Zt[(int64_t)(G.src_base + bb * G.src_stride) * J.ldz + c], acc);
        double* dst = T + (int64_t)(G.dst_base + a * G.dst_stride) * kj + c;
        *dst = fma(G.coef, acc, *dst);
      }
    }
    __syncthreads();
  }
}

constexpr int TM = 64, TN = 64, TK = 16;

// C (m x n) = A (m x k) . B (k x n), all row-major, one 64x64 tile per CTA,
// 256 threads with 4x4 outputs each.
__global__ void __launch_bounds__(256) gemm_kernel(UpdateArgs A) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN];
  const int job = A.tile_job[blockIdx.x];
  const int mn = A.tile_mn[blockIdx.x];
  const RotJob J = A.jobs[job];
  const int m0 = (mn >> 16) * TM, n0 = (mn & 0xffff) * TN;
  const int M = J.ki, N = J.kj, K = J.nI;
  const double* Am = A.Z + J.z_off;   // ki x nI
  const double* Bm = A.T + J.t_off;   // nI x kj
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < K; k0 += TK) {
    for (int idx = threadIdx.x; idx < TM * TK; idx += 256) {
      const int r = idx / TK, c = idx - r * TK;
      const int gr = m0 + r, gc = k0 + c;
      As[c][r] = (gr < M && gc < K) ? Am[(int64_t)gr * K + gc] : 0.0;
    }
    for (int idx = threadIdx.x; idx < TK * TN; idx += 256) {
      const int r = idx / TN, c = idx - r * TN;
      const int gr = k0 + r, gc = n0 + c;
      Bs[r][c] = (gr < K && gc < N) ? Bm[(int64_t)gr * N + gc] : 0.0;
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
  double* O = A.new_ops[J.op] + J.o_off;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + ty + 16 * i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tx + 16 * j;
      if (c < N) O[(int64_t)r * J.ldo + c] = acc[i][j];
    }
  }
}

// Impurity-operator terms (old block x rows of Zt) as 64x64 GEMM tiles:
// T[dst(a)] += sum_terms coef * sum_b M[a][b] Zt[src(b)].  The terms of one
// group share their destination rows (one row group of one job) and are
// summed inside the tile, so tiles of different groups never overlap.
__global__ void __launch_bounds__(256) imp_gemm_kernel(UpdateArgs A) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN];
  const int grp = A.tile1_group[blockIdx.x];
  const int t0 = A.group1_first[grp], nt = A.group1_count[grp];
  const int mn = A.tile1_mn[blockIdx.x];
  const GatherTerm G0 = A.terms1[t0];
  const RotJob J = A.jobs[G0.job];
  const int m0 = (mn >> 16) * TM, n0 = (mn & 0xffff) * TN;
  const int M = G0.rows, N = J.kj;
  const double* Zt = A.Zt + J.zt_off;
  double* T = A.T + J.t_off;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int t = t0; t < t0 + nt; ++t) {
    const GatherTerm G = A.terms1[t];
    const int K = G.srows;
    const double* Am = A.old_ops[G.op] + G.old_off;  // rows x srows, row stride old_ld
    for (int k0 = 0; k0 < K; k0 += TK) {
      for (int idx = threadIdx.x; idx < TM * TK; idx += 256) {
        const int r = idx / TK, c = idx - r * TK;
        const int gr = m0 + r, gc = k0 + c;
        As[c][r] = (gr < M && gc < K) ? G.coef * Am[(int64_t)gr * G.old_ld + gc] : 0.0;
      }
      for (int idx = threadIdx.x; idx < TK * TN; idx += 256) {
        const int r = idx / TN, c = idx - r * TN;
        const int gr = k0 + r, gc = n0 + c;
        Bs[r][c] = (gr < K && gc < N) ? Zt[(int64_t)(G.src_base + gr * G.src_stride) * J.ldz + gc] : 0.0;
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
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + ty + 16 * i;
    if (r >= M) continue;
    double* Trow = T + (int64_t)(G0.dst_base + r * G0.dst_stride) * N;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tx + 16 * j;
      if (c < N) Trow[c] += acc[i][j];
    }
  }
}

}  // namespace

void launch_update(const UpdateArgs& a, cudaStream_t s) {
  if (a.ngroups > 0) gather_kernel<<<a.ngroups, 256, 0, s>>>(a);
  if (a.ntiles1 > 0) imp_gemm_kernel<<<a.ntiles1, 256, 0, s>>>(a);
  if (a.ntiles > 0) gemm_kernel<<<a.ntiles, 256, 0, s>>>(a);
}

}  // namespace nrg
