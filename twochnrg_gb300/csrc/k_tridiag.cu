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
// works on the same block.  It touches the LOWER triangle only, so each
// Householder step costs 4 FMA per stored element (2 for the pending rank-2
// update, 1 for each of the two products a_rc v_c and a_rc v_r of y = A v):
// 2/3 n^3 FMA per block, the algorithmic count, against n^3 for a full-storage
// update (2 FMA per element of both triangles plus one for the row product).
//
// Per step j (trailing rows j+1..n-1, m of them):
//  * The rows form tiles of kRowTile rows, dealt to the CTAs in the order
//    g, 2G-1-g, 2G+g, 4G-1-g, ... so that every CTA gets short and long rows
//    alike (equal work, and no CTA holds a tall narrow triangle whose first
//    strip would be a long chain of dependent loads for one warp).  A row
//    tile is cut into strips of 32 columns; strip s belongs to the same warp
//    of the CTA in every row tile (a snake over the warps), so the column
//    sums of y (lane = column, accumulated over the tile's rows in
//    registers, then into the CTA's column array) need no synchronisation
//    inside the CTA.  The row sums go through a per-warp shared tile read
//    transposed (lane = row), so they also accumulate by FMA.
//  * Each CTA publishes its column sums (G x m) and its warps' row sums (one
//    value per warp and row of its tiles); grid barrier 1.
//  * Columns are dealt evenly to the CTAs, which add the shares in a fixed
//    order (the warps' row sums, then the CTAs' column sums) into
//    y = tau A v and their part of y.v; grid barrier 2; every CTA forms w.
//  * Column j+1 of the updated matrix is captured during the sweep (the
//    element in column j+1 of each row), double-buffered by step parity: it
//    is row j+1 of the next step.
// The upper triangle is free storage: row j receives v_j (v_j[j+1] = 1) in
// columns j+1..n-1 for the back-transformation, as in tridiag_kernel.
// Every sum has a fixed order, so all CTAs hold bitwise identical vectors
// and the result does not depend on timing.
constexpr int kRowTile = 8;
constexpr int kTileLd = 33;  // padded row of a warp's transpose tile
constexpr int kTileDoubles = (kRowTile + 1) * kTileLd;  // + one row for v of the strip's columns

__host__ __device__ constexpr size_t grid_smem_doubles(int maxn) {
  return 4 * (size_t)maxn + (size_t)kWarps * kTileDoubles + kWarps + 4;
}
__host__ __device__ constexpr size_t grid_smem_bytes(int maxn) { return sizeof(double) * grid_smem_doubles(maxn); }

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
  double* CA = sm + 3 * maxn;  // this CTA's column sums, indexed by column
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double* tl = sm + 4 * (size_t)maxn + (size_t)warp * kTileDoubles;
  double* red = sm + 4 * (size_t)maxn + (size_t)kWarps * kTileDoubles;
  double* part = work;                              // G x maxn column sums
  double* rpart = work + (size_t)G * maxn;          // kWarps x maxn row sums
  double* colb = rpart + (size_t)kWarps * maxn;     // 2 x maxn captured column
  double* ybuf = colb + 2 * (size_t)maxn;           // maxn
  double* dpart = ybuf + maxn;                      // G
  for (int qb = 0; qb < nbig; ++qb) {
    const int b = big[qb];
    const int n = A.bsize[b];
    double* H = A.H + A.hoff[b];
    const int so = A.soff[b];
    if (n > maxn || n < 2) {
      if (rank == 0 && tid == 0) {
        if (n > maxn) atomicOr(A.flag, DEV_SIZE);
        else if (n == 1) { A.d[so] = H[0]; A.e[so] = 0.0; A.tau[so] = 0.0; }
      }
      continue;
    }
    double* vnew = V0;
    double* vold = V1;
    bool have_old = false;
    for (int j = 0; j + 2 < n; ++j) {
      const int m = n - j - 1;
      // Row j of A^(j): row 0 of the input, later the column captured in the
      // previous sweep; the pending update applied.  Also the row
      // boundaries and the cleared column sums of this step.
      const double* src = j == 0 ? H : colb + (size_t)((j - 1) & 1) * maxn;
      double s = 0.0;
      for (int c = j + tid; c < n; c += kThreads) {
        double a = __ldcg(src + c);
        if (have_old) a = fma(-vold[j], W[c], fma(-W[j], vold[c], a));
        vnew[c] = a;
        if (c >= j + 2) s = fma(a, a, s);
      }
      if (have_old && rank == 0)
        for (int c = j + tid; c < n; c += kThreads) H[(int64_t)(j - 1) * n + c] = vold[c];
      s = block_sum(s, red);  // synchronises: vnew visible
      for (int c = j + 1 + tid; c < n; c += kThreads) CA[c] = 0.0;
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

      // The sweep over this CTA's rows: tiles of kRowTile rows x 32 columns.
      double* cnext = colb + (size_t)(j & 1) * maxn;
      const int ntiles = (m + kRowTile - 1) / kRowTile;
      for (int q = 0;; ++q) {
        // row tiles dealt g, 2G-1-g, 2G+g, 4G-1-g, ...: short and long rows alike
        const int tt = (q >> 1) * 2 * G + ((q & 1) ? 2 * G - 1 - rank : rank);
        if (tt >= ntiles) {
          if ((q >> 1) * 2 * G >= ntiles) break;
          continue;
        }
        const int t0 = j + 1 + tt * kRowTile, t1 = min(n, t0 + kRowTile);
        const int ns = (t1 - 1 - j + 31) >> 5;  // strips covering columns j+1 .. t1-1
        double P = 0.0;  // lane: row t0 + (lane % kRowTile), columns of its lane group
        // strip st belongs to warp st % 32 < 16 ? st % 32 : 31 - st % 32 in every
        // row tile (a snake over the warps: the strips' heights fall to the right)
        for (int k = 0; k < 2 * ns; ++k) {
          const int st = (k >> 1) * 32 + ((k & 1) ? 31 - warp : warp);
          if (st >= ns) {
            if ((k >> 1) * 32 >= ns) break;
            continue;
          }
          const int c = j + 1 + st * 32 + lane;
          const bool okc = c < t1;
          double vc = 0.0, wc = 0.0, vn = 0.0;
          if (okc) {
            vn = vnew[c];
            if (have_old) { vc = vold[c]; wc = W[c]; }
          }
          double a[kRowTile];
#pragma unroll
          for (int rr = 0; rr < kRowTile; ++rr) {
            const int r = t0 + rr;
            a[rr] = (okc && r < t1 && c <= r) ? __ldcg(H + (int64_t)r * n + c) : 0.0;
          }
          double acc = 0.0;
#pragma unroll
          for (int rr = 0; rr < kRowTile; ++rr) {
            const int r = t0 + rr;
            const bool ok = okc && r < t1 && c <= r;
            double x = a[rr];
            if (ok) {
              if (have_old) {
                x = fma(-vold[r], wc, fma(-W[r], vc, x));
                __stcg(H + (int64_t)r * n + c, x);
              }
              if (c == j + 1) __stcg(cnext + r, x);
              if (c < r) acc = fma(x, vnew[r], acc);
            }
            tl[rr * kTileLd + lane] = ok ? x : 0.0;
          }
          tl[kRowTile * kTileLd + lane] = vn;
          if (okc) CA[c] += acc;
          __syncwarp();
          {
            // lane: row rr of the tile, columns q*kGroup .. q*kGroup+kGroup-1 of
            // the strip (32 / kRowTile lane groups share the 32 columns)
            constexpr int kGroup = 32 / (32 / kRowTile);
            const int rr = lane % kRowTile, q = lane / kRowTile;
            const double* trow = tl + rr * kTileLd + q * kGroup;
            const double* tv = tl + kRowTile * kTileLd + q * kGroup;
#pragma unroll
            for (int k = 0; k < kGroup; ++k) P = fma(trow[k], tv[k], P);
          }
          __syncwarp();
        }
#pragma unroll
        for (int o = kRowTile; o < 32; o <<= 1) P += __shfl_xor_sync(0xffffffffu, P, o);
        if (lane < kRowTile && t0 + lane < t1) __stcg(rpart + (size_t)warp * maxn + t0 + lane, P);
      }
      __syncthreads();
      for (int c = j + 1 + tid; c < n; c += kThreads) __stcg(part + (size_t)rank * maxn + c, CA[c]);
      grid.sync();

      // y = tau A v over this CTA's even share of the columns, in a fixed order.
      const int chunk = (m + G - 1) / G;
      const int q0 = j + 1 + rank * chunk, q1 = min(n, q0 + chunk);
      // Eight threads per column, each over every eighth share, so that the
      // loads of a column are in flight together; then a shuffle tree.
      double dp = 0.0;
      for (int cb = q0; cb < q1; cb += kThreads / 8) {
        const int c = cb + (tid >> 3), sub = tid & 7;
        double y = 0.0;
        if (c < q1) {
          // all of a thread's loads issued before the first add (8 per round)
          double v[8];
#pragma unroll
          for (int k = 0; k < kWarps / 8; ++k) v[k] = __ldcg(rpart + (size_t)(sub + 8 * k) * maxn + c);
#pragma unroll
          for (int k = 0; k < kWarps / 8; ++k) y += v[k];
          for (int g0 = sub; g0 < G; g0 += 64) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const int g = g0 + 8 * k;
              v[k] = g < G ? __ldcg(part + (size_t)g * maxn + c) : 0.0;
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) y += v[k];
          }
        }
        y += __shfl_xor_sync(0xffffffffu, y, 1);
        y += __shfl_xor_sync(0xffffffffu, y, 2);
        y += __shfl_xor_sync(0xffffffffu, y, 4);
        if (c < q1 && sub == 0) {
          y *= tau;
          __stcg(ybuf + c, y);
          dp = fma(y, vnew[c], dp);
        }
      }
      dp = block_sum(dp, red);
      if (tid == 0) __stcg(dpart + rank, dp);
      grid.sync();
      if (tid < 32) {
        double dt = 0.0;
        for (int q = lane; q < G; q += 32) dt += __ldcg(dpart + q);
        for (int o = 16; o > 0; o >>= 1) dt += __shfl_xor_sync(0xffffffffu, dt, o);
        if (lane == 0) red[kWarps + 1] = dt;
      }
      __syncthreads();
      const double h = 0.5 * tau * red[kWarps + 1];
      for (int c = j + 1 + tid; c < n; c += kThreads) W[c] = fma(-h, vnew[c], __ldcg(ybuf + c));
      __syncthreads();
      double* t = vnew; vnew = vold; vold = t;
      have_old = true;
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
    grid.sync();  // the next block's first reads must not race the last writes
  }
}

}  // namespace

int tridiag_grid_size(int maxn) {
  const size_t smem = grid_smem_bytes(maxn);
  if (smem > (size_t)max_dyn_smem()) return 0;
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

size_t tridiag_grid_work(int maxn, int grid) {
  return ((size_t)grid + kWarps + 4) * (size_t)maxn + (size_t)grid + 64;
}

cudaError_t launch_tridiag_grid(const TridiagArgs& a, const int* big, int nbig, double* work, int grid,
                                cudaStream_t s) {
  const size_t smem = grid_smem_bytes(a.maxn);
  if (smem > (size_t)max_dyn_smem() || grid < 1) return cudaErrorInvalidValue;
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
