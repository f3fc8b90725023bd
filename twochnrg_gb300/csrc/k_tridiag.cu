// Batched Householder tridiagonalization of all H_N blocks of one iteration
// in a single persistent launch (FP64).
//
// This is the first half of the reference's per-block LAPACK dspev call
// (CNRGmatrix::DiagBlock, NRGmatrixClass.cpp:638-656), re-designed for the
// GB300: one thread-block CLUSTER owns one H_N block at a time and pulls the
// next block (largest first) from a global work counter.  The CTAs of the
// cluster split the trailing matrix by rows; per Householder step they make
// one pass over their rows that applies the previous step's rank-2 update and
// accumulates their share of the symmetric product A v in shared memory; the
// shares are summed through distributed shared memory after one hardware
// cluster barrier.  The matrix lives in HBM/L2 (full storage, both
// triangles kept symmetric); each step touches every trailing element once.
//
// Outputs: d (diagonal), e (sub-diagonal), tau (reflector scalars) at the
// block's state offset, and the Householder vector v_j (v_j[j+1] = 1) in row j
// of the block's matrix, columns j+1..n-1, for the back-transformation.
//
// There are no spin waits: the only synchronisation is barrier.cluster, which
// every CTA of a cluster reaches the same number of times.
#include <cooperative_groups.h>

#include "nrg_device.cuh"

namespace cg = cooperative_groups;

namespace nrg {

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;

// Deterministic block-wide sum (same tree in every CTA of the cluster): a
// shuffle tree per warp, then one over the warp sums (FP64 latency is long,
// so no serial chains).
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = lane < kWarps ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) red[kWarps] = t;
  }
  __syncthreads();
  return red[kWarps];
}

__global__ void __launch_bounds__(kThreads, 1) tridiag_kernel(TridiagArgs A) {
  extern __shared__ double sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int CL = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const int maxn = A.maxn;
  double* V0 = sm;
  double* V1 = sm + maxn;
  double* W = sm + 2 * maxn;
  double* Y0 = sm + 3 * maxn;
  double* Y1 = sm + 4 * maxn;
  double* red = sm + 5 * maxn;  // kWarps + 1 doubles
  int* sblk = (int*)(red + kWarps + 2);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (;;) {
    if (rank == 0 && tid == 0) *sblk = atomicAdd(A.queue, 1);
    cl.sync();
    const int qi = *cl.map_shared_rank(sblk, 0);
    cl.sync();
    if (qi >= A.nblocks) break;
    const int b = A.order[qi];
    const int n = A.bsize[b];
    double* H = A.H + A.hoff[b];
    const int so = A.soff[b];
    if (n > maxn) {
      if (rank == 0 && tid == 0) atomicOr(A.flag, DEV_SIZE);
      continue;
    }
    if (n == 1) {
      if (rank == 0 && tid == 0) { A.d[so] = H[0]; A.e[so] = 0.0; A.tau[so] = 0.0; }
      continue;
    }
    double* vnew = V0;
    double* vold = V1;
    bool have_old = false;
    for (int j = 0; j + 2 < n; ++j) {
      // Phase 1: row j of A^(j) (pending rank-2 update applied) -> x.
      double s = 0.0;
      for (int c = j + tid; c < n; c += kThreads) {
        double a = __ldcg(H + (int64_t)j * n + c);
        if (have_old) a = fma(-vold[j], W[c], fma(-W[j], vold[c], a));
        vnew[c] = a;
        if (c >= j + 2) s = fma(a, a, s);
      }
      if (have_old && rank == 0)
        for (int c = j + tid; c < n; c += kThreads) H[(int64_t)(j - 1) * n + c] = vold[c];
      s = block_sum(s, red);
      const double dj = vnew[j], alpha = vnew[j + 1];
      double tau, beta, scal;
      if (s == 0.0) {
        tau = 0.0; beta = alpha; scal = 0.0;
      } else {
        beta = -copysign(sqrt(fma(alpha, alpha, s)), alpha);
        tau = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      __syncthreads();
      for (int c = j + 1 + tid; c < n; c += kThreads) vnew[c] = (c == j + 1) ? 1.0 : vnew[c] * scal;
      if (rank == 0 && tid == 0) { A.d[so + j] = dj; A.e[so + j] = beta; A.tau[so + j] = tau; }
      __syncthreads();

      // Phase 2: this CTA's rows of the trailing block: apply the pending
      // update, store, and accumulate column sums of A^(j) v_j.
      const int m = n - j - 1;
      const int rows_per = (m + CL - 1) / CL;
      const int r0 = j + 1 + rank * rows_per;
      const int r1 = min(n, r0 + rows_per);
      double* yp = (j & 1) ? Y1 : Y0;
      const int nchunks = (m + 63) / 64;
      for (int chk = warp; chk < nchunks; chk += kWarps) {
        const int c0 = j + 1 + chk * 64 + lane;
        const int c1 = c0 + 32;
        const bool ok0 = c0 < n, ok1 = c1 < n;
        double vo0 = 0.0, wo0 = 0.0, vo1 = 0.0, wo1 = 0.0;
        if (have_old) {
          if (ok0) { vo0 = vold[c0]; wo0 = W[c0]; }
          if (ok1) { vo1 = vold[c1]; wo1 = W[c1]; }
        }
        double acc0 = 0.0, acc1 = 0.0;
        int r = r0;
        for (; r + 1 < r1; r += 2) {  // two rows in flight
          const double* Ha = H + (int64_t)r * n;
          const double* Hb = Ha + n;
          double a0 = ok0 ? __ldcg(Ha + c0) : 0.0, a1 = ok1 ? __ldcg(Ha + c1) : 0.0;
          double b0 = ok0 ? __ldcg(Hb + c0) : 0.0, b1 = ok1 ? __ldcg(Hb + c1) : 0.0;
          if (have_old) {
            const double vra = vold[r], wra = W[r], vrb = vold[r + 1], wrb = W[r + 1];
            a0 = fma(-vra, wo0, fma(-wra, vo0, a0)); a1 = fma(-vra, wo1, fma(-wra, vo1, a1));
            b0 = fma(-vrb, wo0, fma(-wrb, vo0, b0)); b1 = fma(-vrb, wo1, fma(-wrb, vo1, b1));
            if (ok0) { __stcg((double*)Ha + c0, a0); __stcg((double*)Hb + c0, b0); }
            if (ok1) { __stcg((double*)Ha + c1, a1); __stcg((double*)Hb + c1, b1); }
          }
          const double va = vnew[r], vb = vnew[r + 1];
          acc0 = fma(a0, va, acc0); acc1 = fma(a1, va, acc1);
          acc0 = fma(b0, vb, acc0); acc1 = fma(b1, vb, acc1);
        }
        if (r < r1) {
          const double* Ha = H + (int64_t)r * n;
          double a0 = ok0 ? __ldcg(Ha + c0) : 0.0, a1 = ok1 ? __ldcg(Ha + c1) : 0.0;
          if (have_old) {
            const double vra = vold[r], wra = W[r];
            a0 = fma(-vra, wo0, fma(-wra, vo0, a0)); a1 = fma(-vra, wo1, fma(-wra, vo1, a1));
            if (ok0) __stcg((double*)Ha + c0, a0);
            if (ok1) __stcg((double*)Ha + c1, a1);
          }
          const double va = vnew[r];
          acc0 = fma(a0, va, acc0); acc1 = fma(a1, va, acc1);
        }
        if (ok0) yp[c0] = acc0;
        if (ok1) yp[c1] = acc1;
      }
      cl.sync();

      // Phase 3: p = tau * A v (sum of the CTAs' shares), w = p - (tau/2)(p.v) v.
      {
        const double* rem[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) rem[q] = q < CL ? cl.map_shared_rank(yp, q) : yp;
        for (int c = j + 1 + tid; c < n; c += kThreads) {
          double sh[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) sh[q] = q < CL ? rem[q][c] : 0.0;  // all loads in flight
          double p = 0.0;
#pragma unroll
          for (int q = 0; q < 16; ++q) p += sh[q];
          W[c] = tau * p;
        }
      }
      __syncthreads();
      double dt = 0.0;
      for (int c = j + 1 + tid; c < n; c += kThreads) dt = fma(W[c], vnew[c], dt);
      dt = block_sum(dt, red);
      const double h = 0.5 * tau * dt;
      for (int c = j + 1 + tid; c < n; c += kThreads) W[c] = fma(-h, vnew[c], W[c]);
      __syncthreads();
      double* t = vnew; vnew = vold; vold = t;
      have_old = true;
    }
    // Last 2x2 block with the pending update, and the last reflector.
    if (rank == 0) {
      if (have_old)
        for (int c = n - 2 + tid; c < n; c += kThreads) H[(int64_t)(n - 3) * n + c] = vold[c];
      if (tid == 0) {
        const int j = n - 2;
        double a00 = H[(int64_t)j * n + j], a10 = H[(int64_t)(j + 1) * n + j], a11 = H[(int64_t)(j + 1) * n + j + 1];
        if (have_old) {
          a00 = fma(-vold[j], W[j], fma(-W[j], vold[j], a00));
          a10 = fma(-vold[j + 1], W[j], fma(-W[j + 1], vold[j], a10));
          a11 = fma(-vold[j + 1], W[j + 1], fma(-W[j + 1], vold[j + 1], a11));
        }
        A.d[so + j] = a00; A.e[so + j] = a10; A.tau[so + j] = 0.0;
        A.d[so + j + 1] = a11; A.e[so + j + 1] = 0.0; A.tau[so + j + 1] = 0.0;
      }
    }
  }
}

// Whole-GPU variant for the largest blocks: every CTA of a cooperative grid
// works on the same block and owns a contiguous range of its rows.  Per
// Householder step each CTA applies the pending rank-2 update to its rows and
// forms their complete entries of y = tau A v (the rows hold both triangles),
// writes them and its share of y.v to global memory, and after ONE grid
// barrier every CTA reads y and the shares and forms w.  y and the shares are
// double-buffered by step parity: a CTA that runs ahead into the next step
// writes the other buffer, and cannot run two steps ahead past the barrier.
// Same outputs as tridiag_kernel.
constexpr int kSeg = 4;  // column segments per row: warps work on (row, segment) items

__global__ void __launch_bounds__(kThreads, 1) tridiag_grid_kernel(TridiagArgs A, const int* big, int nbig,
                                                                  double* work) {
  extern __shared__ double sm[];
  cg::grid_group grid = cg::this_grid();
  const int G = (int)gridDim.x;
  const int rank = (int)blockIdx.x;
  const int maxn = A.maxn;
  double* V0 = sm;
  double* V1 = sm + maxn;
  double* W = sm + 2 * maxn;
  double* rowp = sm + 3 * maxn;  // (row, segment) partial sums, up to 2 maxn
  double* red = sm + 5 * maxn;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int qb = 0; qb < nbig; ++qb) {
    const int b = big[qb];
    const int n = A.bsize[b];
    double* H = A.H + A.hoff[b];
    const int so = A.soff[b];
    if (n > maxn) {
      if (rank == 0 && tid == 0) atomicOr(A.flag, DEV_SIZE);
      continue;
    }
    double* vnew = V0;
    double* vold = V1;
    bool have_old = false;
    int par = 0;
    for (int j = 0; j + 2 < n; ++j) {
      for (int c = j + tid; c < n; c += kThreads) {
        double a = __ldcg(H + (int64_t)j * n + c);
        if (have_old) a = fma(-vold[j], W[c], fma(-W[j], vold[c], a));
        vnew[c] = a;
      }
      if (have_old && rank == 0)
        for (int c = j + tid; c < n; c += kThreads) H[(int64_t)(j - 1) * n + c] = vold[c];
      __syncthreads();
      double s = 0.0;
      for (int c = j + 2 + tid; c < n; c += kThreads) s = fma(vnew[c], vnew[c], s);
      s = block_sum(s, red);
      const double dj = vnew[j], alpha = vnew[j + 1];
      double tau, beta, scal;
      if (s == 0.0) {
        tau = 0.0; beta = alpha; scal = 0.0;
      } else {
        beta = -copysign(sqrt(fma(alpha, alpha, s)), alpha);
        tau = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      __syncthreads();
      for (int c = j + 1 + tid; c < n; c += kThreads) vnew[c] = (c == j + 1) ? 1.0 : vnew[c] * scal;
      if (rank == 0 && tid == 0) { A.d[so + j] = dj; A.e[so + j] = beta; A.tau[so + j] = tau; }
      __syncthreads();
      const int m = n - j - 1;
      const int rows_per = (m + G - 1) / G;
      const int r0 = j + 1 + rank * rows_per;
      const int nr = max(0, min(n, r0 + rows_per) - r0);
      int S = kSeg;
      while (S > 1 && rows_per * S > 2 * maxn) S >>= 1;
      const int seglen = (((m + S - 1) / S) + 31) & ~31;
      for (int it = warp; it < nr * S; it += kWarps) {
        const int rr = it / S, sg = it - rr * S;
        const int r = r0 + rr;
        const int cb = j + 1 + sg * seglen, ce = min(n, cb + seglen);
        double* Hr = H + (int64_t)r * n;
        double acc = 0.0;
        if (have_old) {
          const double vr = vold[r], wr = W[r];
          for (int c = cb + lane; c < ce; c += 32) {
            double a = __ldcg(Hr + c);
            a = fma(-vr, W[c], fma(-wr, vold[c], a));
            __stcg(Hr + c, a);
            acc = fma(a, vnew[c], acc);
          }
        } else {
          for (int c = cb + lane; c < ce; c += 32) acc = fma(__ldcg(Hr + c), vnew[c], acc);
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) rowp[rr * S + sg] = acc;
      }
      __syncthreads();
      double* yb = work + (int64_t)par * maxn;
      double* db = work + 2 * (int64_t)maxn + par * G;
      double dpart = 0.0;
      for (int rr = tid; rr < nr; rr += kThreads) {
        double y = 0.0;
        for (int sg = 0; sg < S; ++sg) y += rowp[rr * S + sg];
        y *= tau;
        __stcg(yb + r0 + rr, y);
        dpart = fma(y, vnew[r0 + rr], dpart);
      }
      dpart = block_sum(dpart, red);
      if (tid == 0) __stcg(db + rank, dpart);
      grid.sync();
      double dt = 0.0;
      if (tid < 32) {
        for (int q = lane; q < G; q += 32) dt += __ldcg(db + q);
        for (int o = 16; o > 0; o >>= 1) dt += __shfl_xor_sync(0xffffffffu, dt, o);
        if (lane == 0) red[kWarps + 1] = dt;
      }
      __syncthreads();
      dt = red[kWarps + 1];
      const double h = 0.5 * tau * dt;
      for (int c = j + 1 + tid; c < n; c += kThreads) W[c] = fma(-h, vnew[c], __ldcg(yb + c));
      __syncthreads();
      double* t = vnew; vnew = vold; vold = t;
      have_old = true;
      par ^= 1;
    }
    if (rank == 0) {
      if (have_old)
        for (int c = n - 2 + tid; c < n; c += kThreads) H[(int64_t)(n - 3) * n + c] = vold[c];
      if (tid == 0) {
        const int j = n - 2;
        double a00 = H[(int64_t)j * n + j], a10 = H[(int64_t)(j + 1) * n + j], a11 = H[(int64_t)(j + 1) * n + j + 1];
        if (have_old) {
          a00 = fma(-vold[j], W[j], fma(-W[j], vold[j], a00));
          a10 = fma(-vold[j + 1], W[j], fma(-W[j + 1], vold[j], a10));
          a11 = fma(-vold[j + 1], W[j + 1], fma(-W[j + 1], vold[j + 1], a11));
        }
        A.d[so + j] = a00; A.e[so + j] = a10; A.tau[so + j] = 0.0;
        A.d[so + j + 1] = a11; A.e[so + j + 1] = 0.0; A.tau[so + j + 1] = 0.0;
      }
    }
    grid.sync();  // the next block's phase 1 must not race the last writes
  }
}

}  // namespace

int tridiag_grid_size(int maxn) {
  size_t smem = sizeof(double) * (5 * (size_t)maxn + kWarps + 4) + 16;
  if (cudaFuncSetAttribute(tridiag_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()) !=
      cudaSuccess)
    return 0;
  int per_sm = 0, dev = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tridiag_grid_kernel, kThreads, smem) != cudaSuccess)
    return 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return per_sm >= 1 ? sms : 0;  // one CTA per SM
}

size_t tridiag_grid_work(int maxn, int grid) { return 2 * (size_t)maxn + 2 * (size_t)grid + 64; }

cudaError_t launch_tridiag_grid(const TridiagArgs& a, const int* big, int nbig, double* work, int grid,
                                cudaStream_t s) {
  size_t smem = sizeof(double) * (5 * (size_t)a.maxn + kWarps + 4) + 16;
  cudaError_t err =
      cudaFuncSetAttribute(tridiag_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem());
  if (err != cudaSuccess) return err;
  TridiagArgs aa = a;
  void* args[] = {(void*)&aa, (void*)&big, (void*)&nbig, (void*)&work};
  return cudaLaunchCooperativeKernel((const void*)tridiag_grid_kernel, dim3(grid), dim3(kThreads), args, smem, s);
}

size_t tridiag_smem_bytes(int maxn) {
  return sizeof(double) * (5 * (size_t)maxn + kWarps + 4) + 16;
}

cudaError_t launch_tridiag(const TridiagArgs& a, int cluster, int nclusters, cudaStream_t s) {
  size_t smem = tridiag_smem_bytes(a.maxn);
  cudaError_t err = cudaFuncSetAttribute(tridiag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem());
  if (err != cudaSuccess) return err;
  if (cluster > 8) {
    err = cudaFuncSetAttribute(tridiag_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (err != cudaSuccess) return err;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(cluster * nclusters), 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, tridiag_kernel, a);
}

int tridiag_max_clusters(int cluster, int maxn) {
  size_t smem = tridiag_smem_bytes(maxn);
  if (cudaFuncSetAttribute(tridiag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()) != cudaSuccess)
    return 0;
  if (cluster > 8) cudaFuncSetAttribute(tridiag_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cluster, 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nc = 0;
  if (cudaOccupancyMaxActiveClusters(&nc, tridiag_kernel, &cfg) != cudaSuccess) return 0;
  return nc;
}

}  // namespace nrg
