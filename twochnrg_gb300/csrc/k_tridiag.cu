// Batched Householder tridiagonalization of all H_N blocks of one iteration
// (FP64).
//
// This is the first half of the reference's per-block LAPACK dspev call
// (CNRGmatrix::DiagBlock, NRGmatrixClass.cpp:638-656), re-designed for the
// GB300.  Both kernels work on the LOWER triangle of each block only: per
// Householder step a stored element a_rc (c <= r) takes the pending rank-2
// update (2 FMA), is written back, and contributes to y = A v twice, a_rc v_c
// to row r and a_rc v_r to column c (2 FMA) -- 2/3 n^3 FMA per block, the
// algorithmic count (a full-storage update does n^3).  The shared sweep is
// lower_sweep below; the kernels differ in who cooperates on a block:
//   tridiag_kernel       one thread-block CLUSTER per block (blocks pulled
//                        largest first from a work counter); the CTAs' shares
//                        of y are summed through distributed shared memory
//                        after one hardware cluster barrier per step;
//   tridiag_grid_kernel  every CTA of a cooperative grid on the same block
//                        (the largest blocks), two grid barriers per step.
//
// Outputs: d (diagonal), e (sub-diagonal), tau (reflector scalars) at the
// block's state offset, and the Householder vector v_j (v_j[j+1] = 1) in row j
// of the block's matrix, columns j+1..n-1 (the upper triangle, free storage),
// for the back-transformation.
//
// There are no spin waits: the only synchronisation is barrier.cluster and
// the cooperative grid barrier, which every CTA reaches the same number of
// times.
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
template <int NW = kWarps>
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = lane < NW ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) red[NW] = t;
  }
  __syncthreads();
  return red[NW];
}

constexpr int kRowTile = 8;
constexpr int kTileLd = 33;  // padded row of a warp's transpose tile
constexpr int kTileDoubles = (kRowTile + 1) * kTileLd;  // + one row for v of the strip's columns

__host__ __device__ constexpr size_t grid_smem_doubles(int maxn) {
  return 4 * (size_t)maxn + (size_t)kWarps * kTileDoubles + kWarps + 4;
}
__host__ __device__ constexpr size_t grid_smem_bytes(int maxn) { return sizeof(double) * grid_smem_doubles(maxn); }

// One Householder step's sweep over the trailing lower triangle of part
// `rank` of `parts` (the CTAs of a grid or of a cluster): rows j+1..n-1 in
// tiles of kRowTile rows dealt rank, 2 parts-1-rank, 2 parts+rank, ...; strips
// of 32 columns snaked over the NW warps (strip s to the same warp in every
// tile).  Each stored element a_rc (c <= r) gets the pending rank-2 update
// (vold, W; have_old), is written back, adds a_rc v_r to the column sum CA[c]
// (c < r; the CTA's own array, one warp per column) and a_rc v_c to the row
// sum of r.  Per row tile, row_sink(k, t0, t1, P) receives the warp's row
// sums (lane l < kRowTile: row t0 + l; k counts this part's tiles) and
// capture(r, x) the updated element of column j+1 of every row.
template <int NW, class RowSink, class Capture>
__device__ __forceinline__ void lower_sweep(double* H, int n, int j, int parts, int rank, bool have_old,
                                            const double* vnew, const double* vold, const double* W, double* CA,
                                            double* tl, RowSink row_sink, Capture capture) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m = n - j - 1;
  const int ntiles = (m + kRowTile - 1) / kRowTile;
  int k_own = 0;
  for (int q = 0;; ++q) {
    // row tiles dealt g, 2G-1-g, 2G+g, 4G-1-g, ...: short and long rows alike
    const int tt = (q >> 1) * 2 * parts + ((q & 1) ? 2 * parts - 1 - rank : rank);
    if (tt >= ntiles) {
      if ((q >> 1) * 2 * parts >= ntiles) break;
      continue;
    }
    const int t0 = j + 1 + tt * kRowTile, t1 = min(n, t0 + kRowTile);
    const int ns = (t1 - 1 - j + 31) >> 5;  // strips covering columns j+1 .. t1-1
    double P = 0.0;  // lane: row t0 + (lane % kRowTile), columns of its lane group
    // strip st belongs to warp st % 2NW < NW ? st % 2NW : 2NW-1 - st % 2NW in
    // every row tile (a snake over the NW warps: the strips' heights fall to
    // the right)
    for (int ks = 0; ks < 2 * ns; ++ks) {
      const int st = (ks >> 1) * 2 * NW + ((ks & 1) ? 2 * NW - 1 - warp : warp);
      if (st >= ns) {
        if ((ks >> 1) * 2 * NW >= ns) break;
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
          if (c == j + 1) capture(r, x);
          if (c < r) acc = fma(x, vnew[r], acc);
        }
        tl[rr * kTileLd + lane] = ok ? x : 0.0;
      }
      tl[kRowTile * kTileLd + lane] = vn;
      if (okc) CA[c] += acc;
      __syncwarp();
      {
        // lane: row rr of the tile, columns g*kGroup .. g*kGroup+kGroup-1 of
        // the strip (32 / kRowTile lane groups share the 32 columns)
        constexpr int kGroup = 32 / (32 / kRowTile);
        const int rr = lane % kRowTile, g = lane / kRowTile;
        const double* trow = tl + rr * kTileLd + g * kGroup;
        const double* tv = tl + kRowTile * kTileLd + g * kGroup;
#pragma unroll
        for (int x = 0; x < kGroup; ++x) P = fma(trow[x], tv[x], P);
      }
      __syncwarp();
    }
#pragma unroll
    for (int o = kRowTile; o < 32; o <<= 1) P += __shfl_xor_sync(0xffffffffu, P, o);
    row_sink(k_own, t0, t1, P);
    ++k_own;
  }
}

// Rows of the trailing matrix a CTA of a cluster of `cluster` CTAs can own
// (row tiles dealt as in lower_sweep), for its row-sum buffer.
__host__ __device__ constexpr int cluster_own_rows(int maxn, int cluster) {
  return kRowTile * (((maxn + kRowTile - 1) / kRowTile + cluster - 1) / cluster + 1);
}

// NT threads per CTA: 512 (one CTA per SM) when the sweep has the GPU to
// itself, 256 (two per SM) for concurrent batch workers, whose small blocks
// are latency-bound: twice as many blocks in flight.
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) tridiag_kernel(TridiagArgs A) {
  constexpr int NW = NT / 32;
  extern __shared__ double sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int CL = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const int maxn = A.maxn;
  const int own_max = cluster_own_rows(maxn, CL);
  double* V0 = sm;
  double* V1 = sm + maxn;
  double* W = sm + 2 * maxn;
  double* Y0 = sm + 3 * maxn;
  double* Y1 = sm + 4 * maxn;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double* tl = sm + 5 * (size_t)maxn + (size_t)warp * kTileDoubles;
  double* rowp = sm + 5 * (size_t)maxn + (size_t)NW * kTileDoubles;  // NW x own_max
  double* red = rowp + (size_t)NW * own_max;  // NW + 2 doubles
  int* sblk = (int*)(red + NW + 2);

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
      // Phase 1: row j of A^(j) -> vnew.  Row 0 is the input's; row j > 0
      // holds column j as the previous sweep captured it (updated through
      // step j-2) in its upper part; the pending update is applied here.
      double s = 0.0;
      for (int c = j + tid; c < n; c += NT) {
        double a = __ldcg(H + (int64_t)j * n + c);
        if (have_old) a = fma(-vold[j], W[c], fma(-W[j], vold[c], a));
        vnew[c] = a;
        if (c >= j + 2) s = fma(a, a, s);
      }
      s = block_sum<NW>(s, red);
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
      // v_{j-1} into row j-1 (its upper part was last read at step j-1)
      if (have_old && rank == 0)
        for (int c = j + tid; c < n; c += NT) H[(int64_t)(j - 1) * n + c] = vold[c];
      double* yp = (j & 1) ? Y1 : Y0;
      for (int c = j + 1 + tid; c < n; c += NT) {
        vnew[c] = (c == j + 1) ? 1.0 : vnew[c] * scal;
        yp[c] = 0.0;
      }
      if (rank == 0 && tid == 0) { A.d[so + j] = dj; A.e[so + j] = beta; A.tau[so + j] = tau; }
      __syncthreads();

      // Phase 2: this CTA's row tiles of the trailing lower triangle: the
      // pending update, column sums of y into its share yp, row sums per
      // warp; column j+1 captured into the upper part of row j+1.
      lower_sweep<NW>(H, n, j, CL, rank, have_old, vnew, vold, W, yp, tl,
                  [&](int k, int, int, double P) {
                    if (lane < kRowTile) rowp[(size_t)warp * own_max + k * kRowTile + lane] = P;
                  },
                  [&](int r, double x) { __stcg(H + (int64_t)(j + 1) * n + r, x); });
      __syncthreads();
      {
        // the warps' row sums of the CTA's own rows into its share
        const int m = n - j - 1;
        const int ntiles = (m + kRowTile - 1) / kRowTile;
        for (int idx = tid; idx < own_max; idx += NT) {
          const int k = idx / kRowTile, rr = idx - k * kRowTile;
          const int tt = (k >> 1) * 2 * CL + ((k & 1) ? 2 * CL - 1 - rank : rank);
          const int r = j + 1 + tt * kRowTile + rr;
          if (tt >= ntiles || r >= n) continue;
          double v = 0.0;
          for (int w = 0; w < NW; ++w) v += rowp[(size_t)w * own_max + idx];
          yp[r] += v;
        }
      }
      cl.sync();

      // Phase 3: p = tau * A v (sum of the CTAs' shares), w = p - (tau/2)(p.v) v.
      {
        const double* rem[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) rem[q] = q < CL ? cl.map_shared_rank(yp, q) : yp;
        for (int c = j + 1 + tid; c < n; c += NT) {
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
      for (int c = j + 1 + tid; c < n; c += NT) dt = fma(W[c], vnew[c], dt);
      dt = block_sum<NW>(dt, red);
      const double h = 0.5 * tau * dt;
      for (int c = j + 1 + tid; c < n; c += NT) W[c] = fma(-h, vnew[c], W[c]);
      __syncthreads();
      double* t = vnew; vnew = vold; vold = t;
      have_old = true;
    }
    // Last 2x2 block (lower triangle) with the pending update, and the last reflector.
    if (rank == 0) {
      if (have_old)
        for (int c = n - 2 + tid; c < n; c += NT) H[(int64_t)(n - 3) * n + c] = vold[c];
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

      // The sweep over this CTA's row tiles; row sums to rpart, column j+1 to colb.
      double* cnext = colb + (size_t)(j & 1) * maxn;
      lower_sweep<kWarps>(H, n, j, G, rank, have_old, vnew, vold, W, CA, tl,
                  [&](int, int t0, int t1, double P) {
                    if (lane < kRowTile && t0 + lane < t1) __stcg(rpart + (size_t)warp * maxn + t0 + lane, P);
                  },
                  [&](int r, double x) { __stcg(cnext + r, x); });
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

size_t tridiag_smem_bytes(int maxn, int cluster, int threads) {
  const size_t nw = (size_t)threads / 32;
  return sizeof(double) * (5 * (size_t)maxn + nw * kTileDoubles + nw * cluster_own_rows(maxn, cluster) + nw + 2) + 16;
}

namespace {
const void* cluster_kernel(int threads) {
  return threads == 256 ? (const void*)tridiag_kernel<256> : (const void*)tridiag_kernel<512>;
}

cudaLaunchConfig_t cluster_config(int cluster, int nclusters, int threads, size_t smem, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(cluster * nclusters), 1, 1);
  cfg.blockDim = dim3((unsigned)threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

cudaError_t cluster_attributes(int cluster, int threads) {
  const void* k = cluster_kernel(threads);
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem());
  if (err == cudaSuccess && cluster > 8) err = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return err;
}
}  // namespace

cudaError_t launch_tridiag(const TridiagArgs& a, int cluster, int nclusters, cudaStream_t s, int threads) {
  if (threads != 256 && threads != 512) return cudaErrorInvalidValue;
  const size_t smem = tridiag_smem_bytes(a.maxn, cluster, threads);
  if (smem > (size_t)max_dyn_smem()) return cudaErrorInvalidValue;
  cudaError_t err = cluster_attributes(cluster, threads);
  if (err != cudaSuccess) return err;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config(cluster, nclusters, threads, smem, attr);
  cfg.stream = s;
  if (threads == 256) return cudaLaunchKernelEx(&cfg, tridiag_kernel<256>, a);
  return cudaLaunchKernelEx(&cfg, tridiag_kernel<512>, a);
}

int tridiag_max_clusters(int cluster, int maxn, int threads) {
  if (threads != 256 && threads != 512) return 0;
  const size_t smem = tridiag_smem_bytes(maxn, cluster, threads);
  if (smem > (size_t)max_dyn_smem()) return 0;
  if (cluster_attributes(cluster, threads) != cudaSuccess) return 0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config(cluster, 1, threads, smem, attr);
  int nc = 0;
  if (cudaOccupancyMaxActiveClusters(&nc, cluster_kernel(threads), &cfg) != cudaSuccess) return 0;
  return nc;
}

}  // namespace nrg
