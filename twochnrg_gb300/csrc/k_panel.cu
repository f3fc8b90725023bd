// Blocked Householder tridiagonalization of one large H_N block: the panel
// part, for the mixed-precision form.
//
// This is dspev's reduction (CNRGmatrix::DiagBlock, NRGmatrixClass.cpp:
// 638-656) reorganised the way LAPACK's blocked dsytrd/dlatrd does it, so
// that the trailing update becomes one rank-2nb product per panel that runs
// on the tensor cores (k_ozaki.cu), instead of a rank-2 update per column on
// the FP64 pipe.  Within a panel of nb columns the trailing matrix is left as
// it was at the panel's start; column j's Householder vector v and
// w = tau A v - (tau^2/2)(v^T A v) v are formed against that stale matrix and
// corrected with the panel's earlier vectors:
//
//   A_now = H - V W^T - W V^T          (V, W: the panel's v's and w's so far)
//   a_j   = H[j][:] - V W[j]^T - W V[j]^T
//   y     = H v - V (W^T v) - W (V^T v)
//
// so every column costs one FP64 pass over the trailing rows (y = H v, one
// FMA per element) instead of three.  After the panel the caller applies
// H -= [V W] [W V]^T to the trailing block.
//
// One cooperative grid works on the block; CTA c owns a fixed range of rows
// of [k0, n) for the panel and keeps their V and W rows in shared memory
// (written through to the [V W] array that the trailing product reads).  Per
// column there are two grid barriers: after the column pieces and norm shares
// (every CTA then forms v in full), and after the shares of V^T v, W^T v and
// y.v (every CTA then forms its rows of w, and the next column's W entry).
// No spin waits; the grid barrier is CUDA's cooperative one, reached the same
// number of times by every CTA.
//
// Outputs as tridiag_kernel: d, e, tau of the panel's columns, v_j in row j
// of the block (columns j+1..n-1), and, after the last panel, the closing
// 2 x 2 block.
#include <cooperative_groups.h>

#include "nrg_device.cuh"

namespace cg = cooperative_groups;

namespace nrg {

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;

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

struct SmemLayout {
  int rows_per, nseg;
  size_t v, vw, y, rowp, cur, nxt, pq, red, total;  // offsets in doubles
};

__host__ __device__ inline SmemLayout smem_layout(int n, int k0, int nb, int G) {
  SmemLayout L;
  const int m = n - k0;
  L.rows_per = (m + G - 1) / G;
  L.nseg = 2;
  L.v = 0;
  L.vw = L.v + (size_t)n;
  L.y = L.vw + (size_t)L.rows_per * (2 * nb + 1);
  L.rowp = L.y + (size_t)L.rows_per;
  L.cur = L.rowp + (size_t)L.rows_per * L.nseg * 33;
  L.nxt = L.cur + 2 * (size_t)nb;
  L.pq = L.nxt + 2 * (size_t)nb;
  L.red = L.pq + 2 * (size_t)nb + 2;
  L.total = L.red + kWarps + 8;
  return L;
}

__global__ void __launch_bounds__(kThreads, 1) panel_kernel(PanelArgs A) {
  extern __shared__ double sm[];
  cg::grid_group grid = cg::this_grid();
  const int G = (int)gridDim.x, rank = (int)blockIdx.x;
  const int n = A.n, nb = A.nb, ld = 2 * nb, lds = ld + 1, k0 = A.k0;
  const SmemLayout L = smem_layout(n, k0, nb, G);
  double* v = sm + L.v;        // v_j over [j+1, n)
  double* vw = sm + L.vw;      // own rows' [V W], rows_per x 2nb (row stride 2nb + 1: no bank conflicts)
  double* yl = sm + L.y;       // own rows' y
  double* rowp = sm + L.rowp;  // (row, segment) lane partial sums of H v, 33 apart
  double* cur = sm + L.cur;    // row j of [V W] for the column correction
  double* nxt = sm + L.nxt;    // row j+1 of [V W], formed during step j
  double* pq = sm + L.pq;      // W^T v (l < i), V^T v (nb + l), v^T y (2nb)
  double* red = sm + L.red;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = k0 + rank * L.rows_per;
  const int r1 = min(n, r0 + L.rows_per);
  double* H = A.H;
  // [V W] rows of this panel start at zero
  for (int x = tid; x < L.rows_per * lds; x += kThreads) vw[x] = 0.0;
  for (int x = tid; x < 2 * nb; x += kThreads) cur[x] = 0.0;
  __syncthreads();
  double* part = A.part;  // [G][2nb + 2]
  for (int j = k0; j < A.k1; ++j) {
    const int i = j - k0;
    const int par = i & 1;
    double* col = A.col + (size_t)par * n;
    // cur: row j of [V W], entries l < i (the last one formed by every CTA
    // at step j-1, in what was nxt then)
    // Phase 1: own pieces of column j of the corrected matrix, and norm shares.
    double s = 0.0;
    for (int r = max(r0, j) + tid; r < r1; r += kThreads) {
      double a = __ldcg(H + (size_t)j * n + r);
      const double* vr = vw + (size_t)(r - r0) * lds;
      for (int l = 0; l < i; ++l) a = fma(-vr[l], cur[nb + l], fma(-vr[nb + l], cur[l], a));
      __stcg(col + r, a);
      if (r >= j + 2) s = fma(a, a, s);
    }
    s = block_sum(s, red);
    if (tid == 0) __stcg(part + (size_t)rank * (ld + 2) + ld + 1, s);
    grid.sync();  // (A)
    // Phase 2: the Householder vector of column j, in full in every CTA.  The
    // column pieces and the norm shares are fetched in one round trip.
    for (int c = j + tid; c < n; c += kThreads) v[c] = __ldcg(col + c);
    if (tid == 0) {
      double t = 0.0;
      for (int q0 = 0; q0 < G; q0 += 8) {
        double sh[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) sh[u] = q0 + u < G ? __ldcg(part + (size_t)(q0 + u) * (ld + 2) + ld + 1) : 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) t += sh[u];
      }
      red[kWarps + 1] = t;
    }
    __syncthreads();
    const double nrm2 = red[kWarps + 1];
    const double dj = v[j], alpha = v[j + 1];
    double tau, beta, scal;
    if (nrm2 == 0.0) {
      tau = 0.0; beta = alpha; scal = 0.0;
    } else {
      beta = -copysign(sqrt(fma(alpha, alpha, nrm2)), alpha);
      tau = (beta - alpha) / beta;
      scal = 1.0 / (alpha - beta);
    }
    __syncthreads();
    for (int c = j + 1 + tid; c < n; c += kThreads) v[c] = (c == j + 1) ? 1.0 : v[c] * scal;
    if (rank == 0 && tid == 0) { A.d[j] = dj; A.e[j] = beta; A.tau[j] = tau; }
    __syncthreads();
    // v_j into row j of the block (no CTA reads row j again), own share of
    // the columns; V(r, i) for own rows.
    for (int c = max(r0, j + 1) + tid; c < r1; c += kThreads) {
      H[(size_t)j * n + c] = v[c];
      vw[(size_t)(c - r0) * lds + i] = v[c];
      A.VW[(size_t)c * ld + i] = v[c];
    }
    // y = H v over the own rows r >= j+1 (stale matrix, one FMA per element)
    const int ra = max(r0, j + 1);
    const int nr = max(0, r1 - ra);
    const int m = n - j - 1;
    const int S = L.nseg;
    const int seglen = (((m + S - 1) / S) + 31) & ~31;
    for (int it = warp; it < nr * S; it += kWarps) {
      const int rr = it / S, sg = it - rr * S;
      const int r = ra + rr;
      const int cb = j + 1 + sg * seglen, ce = min(n, cb + seglen);
      const double* Hr = H + (size_t)r * n;
      // eight independent loads in flight per lane: the row streams from L2
      // or HBM and the FP64 pipe, not the load latency, must set the pace
      double acc0 = 0.0, acc1 = 0.0;
      for (int c = cb + lane; c < ce; c += 8 * 32) {
        double h[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) h[u] = c + 32 * u < ce ? __ldcg(Hr + c + 32 * u) : 0.0;
#pragma unroll
        for (int u = 0; u < 8; u += 2) {
          acc0 = fma(h[u], c + 32 * u < ce ? v[c + 32 * u] : 0.0, acc0);
          acc1 = fma(h[u + 1], c + 32 * (u + 1) < ce ? v[c + 32 * (u + 1)] : 0.0, acc1);
        }
      }
      // lane partials to shared memory: one thread per row adds them (32
      // additions per item instead of a warp-wide shuffle tree's 160)
      rowp[(size_t)(rr * S + sg) * 33 + lane] = acc0 + acc1;
    }
    __syncthreads();
    double yv = 0.0;
    for (int rr = tid; rr < nr; rr += kThreads) {
      double y = 0.0;
      for (int sg = 0; sg < S; ++sg) {
        const double* pr = rowp + (size_t)(rr * S + sg) * 33;
        double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
#pragma unroll
        for (int q = 0; q < 32; q += 4) { t0 += pr[q]; t1 += pr[q + 1]; t2 += pr[q + 2]; t3 += pr[q + 3]; }
        y += (t0 + t1) + (t2 + t3);
      }
      yl[ra - r0 + rr] = y;
      yv = fma(y, v[ra + rr], yv);
      if (ra + rr == j + 1) __stcg(A.ybuf + par, y);
    }
    yv = block_sum(yv, red);
    // shares of W^T v and V^T v over the own rows (l < i): warp per column
    for (int x = warp; x < 2 * i; x += kWarps) {
      const int l = x < i ? nb + x : x - i;  // W columns first, then V
      double t = 0.0;
      for (int rr = lane; rr < nr; rr += 32) t = fma(vw[(size_t)(ra - r0 + rr) * lds + l], v[ra + rr], t);
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (lane == 0) __stcg(part + (size_t)rank * (ld + 2) + (x < i ? x : nb + (x - i)), t);
    }
    if (tid == 0) __stcg(part + (size_t)rank * (ld + 2) + ld, yv);
    grid.sync();  // (B)
    // Phase 3: sums of the shares, own rows of w, and row j+1's new W entry;
    // the shares, row j+1 of [V W] (entries l < i, from the owners' earlier
    // writes) and y(j+1) are fetched in one round trip.
    for (int x = tid; x < 2 * nb; x += kThreads) {
      const int l = x < nb ? x : x - nb;
      nxt[x] = l < i ? __ldcg(A.VW + (size_t)(j + 1) * ld + x) : 0.0;
    }
    if (tid == kThreads - 1) red[kWarps + 2] = __ldcg(A.ybuf + par);
    // a thread per value (2i + 1 of them) adds the G shares, loaded eight at a time
    for (int xx = tid; xx < 2 * i + 1; xx += kThreads) {
      const int x = xx == 2 * i ? ld : (xx < i ? xx : nb + (xx - i));
      double t = 0.0;
      for (int q0 = 0; q0 < G; q0 += 8) {
        double sh[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) sh[u] = q0 + u < G ? __ldcg(part + (size_t)(q0 + u) * (ld + 2) + x) : 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) t += sh[u];
      }
      pq[x] = t;
    }
    __syncthreads();
    if (warp == 0) {  // v^T (A_now v) = y.v - 2 (W^T v).(V^T v), formed once
      double t = 0.0;
      for (int l = lane; l < i; l += 32) t = fma(pq[l], pq[nb + l], t);
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (lane == 0) red[kWarps + 3] = pq[ld] - 2.0 * t;
    }
    __syncthreads();
    const double yvt = red[kWarps + 3];
    const double h = 0.5 * tau * tau * yvt;
    for (int rr = tid; rr < nr; rr += kThreads) {
      const int r = ra + rr;
      double* vr = vw + (size_t)(r - r0) * lds;
      double y = yl[r - r0];
      for (int l = 0; l < i; ++l) y = fma(-vr[l], pq[l], fma(-vr[nb + l], pq[nb + l], y));
      const double w = fma(tau, y, -h * v[r]);
      vr[nb + i] = w;
      A.VW[(size_t)r * ld + nb + i] = w;
    }
    if (warp == 0) {
      double t = 0.0;
      for (int l = lane; l < i; l += 32) t = fma(-nxt[l], pq[l], fma(-nxt[nb + l], pq[nb + l], t));
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (lane == 0) {
        nxt[i] = 1.0;
        nxt[nb + i] = fma(tau, red[kWarps + 2] + t, -h);
      }
    }
    __syncthreads();
    double* sw = cur; cur = nxt; nxt = sw;
  }
  if (A.last) {
    // closing 2 x 2 block with the whole panel's correction
    grid.sync();
    if (rank == 0 && tid == 0) {
      const int j = n - 2, w = A.k1 - k0;
      const double* V0 = A.VW + (size_t)j * ld;
      const double* V1 = A.VW + (size_t)(j + 1) * ld;
      double a00 = __ldcg(H + (size_t)j * n + j), a10 = __ldcg(H + (size_t)(j + 1) * n + j),
             a11 = __ldcg(H + (size_t)(j + 1) * n + j + 1);
      for (int l = 0; l < w; ++l) {
        const double v0 = __ldcg(V0 + l), w0 = __ldcg(V0 + nb + l), v1 = __ldcg(V1 + l), w1 = __ldcg(V1 + nb + l);
        a00 = fma(-v0, w0, fma(-w0, v0, a00));
        a10 = fma(-v1, w0, fma(-w1, v0, a10));
        a11 = fma(-v1, w1, fma(-w1, v1, a11));
      }
      A.d[j] = a00; A.e[j] = a10; A.tau[j] = 0.0;
      A.d[j + 1] = a11; A.e[j + 1] = 0.0; A.tau[j + 1] = 0.0;
    }
  }
}

}  // namespace

size_t panel_smem_bytes(int n, int k0, int nb, int grid) {
  return sizeof(double) * smem_layout(n, k0, nb, grid).total + 16;
}

cudaError_t launch_panel(const PanelArgs& a, int grid, cudaStream_t s) {
  const size_t smem = panel_smem_bytes(a.n, a.k0, a.nb, grid);
  if (smem > (size_t)max_dyn_smem()) return cudaErrorInvalidValue;
  cudaError_t err = cudaFuncSetAttribute(panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem());
  if (err != cudaSuccess) return err;
  PanelArgs aa = a;
  void* args[] = {(void*)&aa};
  return cudaLaunchCooperativeKernel((const void*)panel_kernel, dim3(grid), dim3(kThreads), args, smem, s);
}

int panel_max_grid() {
  int per_sm = 0, dev = 0, sms = 0;
  if (cudaFuncSetAttribute(panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, panel_kernel, kThreads, 100 * 1024) != cudaSuccess)
    return 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return per_sm >= 1 ? sms : 0;
}

}  // namespace nrg
