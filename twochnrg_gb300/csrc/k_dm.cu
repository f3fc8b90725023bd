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
// frequency dependence is isolated: every shell becomes lists of
// (E_j - E_i, weight) records once, keeping only the pairs whose term can be
// nonzero, and the Lehmann kernel stages each chunk of records in shared
// memory and sums it against a tile of frequencies, with the log-Gaussian /
// Gaussian kernels of BroadDelta.cpp evaluated on the fly.
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
      if (c < J.n) {
        double* o = J.C + (int64_t)r * J.ldc + c;
        *o = J.accum ? *o + acc[i][j] : acc[i][j];
      }
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
    if (i == j && !A.kept[s0 + i] && A.zdisc != 0.0) {
      const double e = exp(-A.beta * A.en[s0 + i]) / A.zdisc;
      v = A.dE ? e * (-A.beta * A.dE[s0 + i] - A.dlogz) : e;
    }
    R[idx] = v;
  }
}

// The weights of pair idx of a c_d block pair: FDM_SpecDens_M_STL's
// (rho A + A rho) A with the kept / discarded split, or on the last shell
// CalcSpecCosti_T_N's Boltzmann weights.  Explicitly rounded (no FMA
// contraction), so that the counting and the scattering pass, which both
// call it, classify every pair alike.
__device__ __forceinline__ void pair_value(const DmRecArgs& A, const DmPair& P, int64_t idx, double& dE,
                                           double& wp, double& wn) {
  const int a = (int)(idx / P.n2), b = (int)(idx - (int64_t)a * P.n2);
  const double m = A.cd[P.a_off + idx];
  const double E1 = A.en[P.s1 + a], E2 = A.en[P.s2 + b];
  wp = 0.0; wn = 0.0;
  if (A.last) {
    const double sum12 = __dadd_rn(__dmul_rn(m, exp(-A.beta_last * E1)), __dmul_rn(exp(-A.beta_last * E2), m));
    wp = wn = __dmul_rn(__dmul_rn(P.cg, __dmul_rn(sum12, m)), A.inv_z_last);
  } else if (!P.skip) {
    const double p1 = a < P.r1 ? A.P1[P.p_off + idx] : 0.0, p2 = b < P.r2 ? A.P2[P.p_off + idx] : 0.0;
    const double w = __dmul_rn(P.cg, __dmul_rn(__dadd_rn(p1, p2), m));
    if (!A.kept[P.s2 + b]) wp = w;
    if (!A.kept[P.s1 + a]) wn = w;
  }
  dE = E2 - E1;
}

// pair_value differentiated along direction p: d(E_j - E_i) and the
// tangents of W+ and W- (the same kept / discarded split).
__device__ __forceinline__ void pair_tangent(const DmRecArgs& A, const DmPair& P, int64_t idx, int p, double& ddE,
                                             double& dwp, double& dwn) {
  const int a = (int)(idx / P.n2), b = (int)(idx - (int64_t)a * P.n2);
  const double m = A.cd[P.a_off + idx], dm = A.dcd[p][P.a_off + idx];
  const double* dE = A.dE + (int64_t)p * A.nstates;
  const double dE1 = dE[P.s1 + a], dE2 = dE[P.s2 + b];
  dwp = 0.0; dwn = 0.0;
  if (A.last) {
    const double e1 = exp(-A.beta_last * A.en[P.s1 + a]), e2 = exp(-A.beta_last * A.en[P.s2 + b]);
    const double s12 = (e1 + e2) * m;
    const double ds12 = (e1 + e2) * dm - A.beta_last * (e1 * dE1 + e2 * dE2) * m;
    const double w = P.cg * s12 * m * A.inv_z_last;
    dwp = dwn = P.cg * (ds12 * m + s12 * dm) * A.inv_z_last - w * A.dlogz_last[p];
  } else if (!P.skip) {
    const int64_t q = (int64_t)p * A.pstride + P.p_off + idx;
    const double p1 = a < P.r1 ? A.P1[P.p_off + idx] : 0.0, p2 = b < P.r2 ? A.P2[P.p_off + idx] : 0.0;
    const double dp1 = a < P.r1 ? A.dP1[q] : 0.0, dp2 = b < P.r2 ? A.dP2[q] : 0.0;
    const double dw = P.cg * ((dp1 + dp2) * m + (p1 + p2) * dm);
    if (!A.kept[P.s2 + b]) dwp = dw;
    if (!A.kept[P.s1 + a]) dwn = dw;
  }
  ddE = dE2 - dE1;
}

// Bit L set: the pair's term is in list L (see DmRecArgs).
__device__ __forceinline__ unsigned pair_lists(const DmRecArgs& A, double dE, double wp, double wn) {
  const bool gauss = fabs(dE) < A.gauss_below;
  const double Ep = dE == 0.0 ? 1.0e-100 : dE;
  unsigned f = 0u;
  if (wp != 0.0) f |= gauss ? 2u : (Ep > 0.0 ? 1u : 0u);
  if (wn != 0.0) f |= gauss ? 8u : (Ep < 0.0 ? 4u : 0u);
  return f;
}

// pass 0: per chunk of kPairChunk pairs, how many go to each list.
__global__ void __launch_bounds__(256) dm_count_kernel(DmRecArgs A) {
  __shared__ int cnt[4];
  const DmChunk C = A.chunks[blockIdx.x];
  const DmPair P = A.pairs[C.pair];
  const int64_t n = (int64_t)P.n1 * P.n2;
  if (threadIdx.x < 4) cnt[threadIdx.x] = 0;
  __syncthreads();
  int local[4] = {0, 0, 0, 0};
  for (int i = threadIdx.x; i < kPairChunk; i += blockDim.x) {
    const int64_t idx = (int64_t)C.start + i;
    if (idx >= n) break;
    double dE, wp, wn;
    pair_value(A, P, idx, dE, wp, wn);
    const unsigned f = pair_lists(A, dE, wp, wn);
    for (int L = 0; L < 4; ++L) local[L] += (f >> L) & 1u;
  }
  for (int L = 0; L < 4; ++L) {
    int v = local[L];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&cnt[L], v);
  }
  __syncthreads();
  if (threadIdx.x < 4) A.counts[(int64_t)blockIdx.x * 4 + threadIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of the chunk counts of every list (one CTA of 1024).
__global__ void __launch_bounds__(1024) dm_scan_kernel(DmRecArgs A) {
  __shared__ int64_t part[1024];
  const int T = blockDim.x, t = threadIdx.x;
  const int per = (A.nchunks + T - 1) / T;
  const int c0 = min(t * per, A.nchunks), c1 = min(c0 + per, A.nchunks);
  for (int L = 0; L < 4; ++L) {
    int64_t sum = 0;
    for (int c = c0; c < c1; ++c) sum += A.counts[(int64_t)c * 4 + L];
    part[t] = sum;
    __syncthreads();
    for (int o = 1; o < T; o <<= 1) {  // inclusive Hillis-Steele scan
      const int64_t v = t >= o ? part[t - o] : 0;
      __syncthreads();
      part[t] += v;
      __syncthreads();
    }
    int64_t run = part[t] - sum;
    for (int c = c0; c < c1; ++c) {
      A.offsets[(int64_t)c * 4 + L] = run;
      run += A.counts[(int64_t)c * 4 + L];
    }
    if (t == T - 1) A.totals[L] = part[t];
    __syncthreads();
  }
}

// pass 1: the records, in pair order within every list (TAN: and their
// tangents).
template <bool TAN>
__global__ void __launch_bounds__(256) dm_scatter_kernel(DmRecArgs A) {
  constexpr int NW = 8;
  __shared__ int wtot[4][NW];
  const DmChunk C = A.chunks[blockIdx.x];
  const DmPair P = A.pairs[C.pair];
  const int64_t n = (int64_t)P.n1 * P.n2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t run[4];
  for (int L = 0; L < 4; ++L) run[L] = A.offsets[(int64_t)blockIdx.x * 4 + L];
  for (int r = 0; r < kPairChunk; r += 256) {
    const int64_t idx = (int64_t)C.start + r + threadIdx.x;
    const bool in = (r + (int)threadIdx.x) < kPairChunk && idx < n;
    double dE = 0.0, wp = 0.0, wn = 0.0;
    if (in) pair_value(A, P, idx, dE, wp, wn);
    const unsigned f = in ? pair_lists(A, dE, wp, wn) : 0u;
    double tdd[4] = {0.0, 0.0, 0.0, 0.0}, twp[4] = {0.0, 0.0, 0.0, 0.0}, twn[4] = {0.0, 0.0, 0.0, 0.0};
    if (TAN) {
#pragma unroll
      for (int p = 0; p < 4; ++p)
        if (f && p < A.ntan) pair_tangent(A, P, idx, p, tdd[p], twp[p], twn[p]);
    }
    unsigned mask[4];
    for (int L = 0; L < 4; ++L) {
      mask[L] = __ballot_sync(0xffffffffu, (f >> L) & 1u);
      if (lane == 0) wtot[L][warp] = __popc(mask[L]);
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    for (int L = 0; L < 4; ++L) {
      int before = 0, all = 0;
      for (int w2 = 0; w2 < NW; ++w2) { before += w2 < warp ? wtot[L][w2] : 0; all += wtot[L][w2]; }
      const int64_t pos = run[L] + before + __popc(mask[L] & lt);
      if (((f >> L) & 1u) && pos < A.totals[L]) {
        const double W = L < 2 ? wp : wn;
        if (L == 0 || L == 2) {
          const double aE = fabs(dE == 0.0 ? 1.0e-100 : dE);
          A.key[L][pos] = log(aE) * A.inv_b;
          A.w[L][pos] = W * A.log_scale / aE;
        } else {
          A.key[L][pos] = dE * A.inv_bt;
          A.w[L][pos] = W * A.gauss_scale;
        }
        // tangents: log-Gaussian w = W c / |dE|, key = ln|dE| / b;
        // Gaussian w = W c, key = dE / bt
        const int64_t T = A.totals[L];
#pragma unroll
        for (int p = 0; p < (TAN ? 4 : 0); ++p) {
          if (p >= A.ntan) break;
          const double dW = L < 2 ? twp[p] : twn[p];
          double tw, tg;
          if (L == 0 || L == 2) {
            const double aE = fabs(dE == 0.0 ? 1.0e-100 : dE);
            const double daE = (dE < 0.0 ? -1.0 : 1.0) * tdd[p];
            const double w = W * A.log_scale / aE;
            tw = dW * A.log_scale / aE - w * daE / aE;
            tg = 2.0 * w * (daE / aE) * A.inv_b;
          } else {
            tw = dW * A.gauss_scale;
            tg = 2.0 * (W * A.gauss_scale) * tdd[p] * A.inv_bt;
          }
          A.tw[L][p * T + pos] = tw;
          A.tg[L][p * T + pos] = tg;
        }
      }
      run[L] += all;
    }
    __syncthreads();
  }
}

// One CTA per (list, chunk of kRecChunk records, tile of kOmegaTile
// frequencies): the records are staged in shared memory once; warp w sums
// the records of its half (w / 4) against the 16 frequencies of its quarter
// of the tile (w % 4), held in registers, and the halves are added in
// shared memory in a fixed order.
__global__ void __launch_bounds__(256) lehmann_kernel(LehmannArgs A) {
  constexpr int kStage = 2048, kPerWarp = 16, kGroups = kOmegaTile / kPerWarp, kSplit = 8 / kGroups;
  __shared__ double sk[kStage], sw[kStage], st[kOmegaTile], sred[8][kPerWarp];
  const LehItem it = A.items[blockIdx.x];
  const LehList L = A.lists[it.list];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = warp % kGroups, part = warp / kGroups;
  const int jt = it.tile * kOmegaTile;
  const double ldn = A.log_dn[L.shell], dn = A.dn[L.shell];
  if (threadIdx.x < kOmegaTile) {
    const int j = jt + threadIdx.x;
    double t = 0.0;
    if (j < L.nomega) {
      const int k = A.omega_idx[L.omega_first + j];
      t = L.gauss ? (A.omega[k] / dn) * A.inv_bt : (A.log_omega[k] - ldn) * A.inv_b - A.b_quarter;
    }
    st[threadIdx.x] = t;
  }
  const int j0 = jt + grp * kPerWarp;
  const bool active = j0 < L.nomega;
  double acc[kPerWarp];
#pragma unroll
  for (int q = 0; q < kPerWarp; ++q) acc[q] = 0.0;
  const int64_t r0 = (int64_t)it.chunk * kRecChunk;
  const int64_t r1 = min(r0 + (int64_t)kRecChunk, L.nrec);
  for (int64_t base = r0; base < r1; base += kStage) {
    const int n = (int)min((int64_t)kStage, r1 - base);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) { sk[i] = L.key[base + i]; sw[i] = L.w[base + i]; }
    __syncthreads();
    if (!active) continue;
    const double* tq = st + grp * kPerWarp;
    if (it.delta != 0.0) {
      const double d = it.delta, c = exp(-2.0 * d * d), t0 = tq[0];
      for (int i = part * 32 + lane; i < n; i += 32 * kSplit) {
        const double ww = sw[i], x0 = t0 - sk[i];
        double g = exp(-x0 * x0), r = exp(-d * (2.0 * x0 + d));
        acc[0] += ww * g;
#pragma unroll
        for (int q = 1; q < kPerWarp; ++q) {
          g *= r;
          r *= c;
          acc[q] += ww * g;
        }
      }
    } else {
      // Eight frequencies per pass over the records (register pressure).
#pragma unroll
      for (int qb = 0; qb < kPerWarp; qb += 8) {
        double a8[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int i = part * 32 + lane; i < n; i += 32 * kSplit) {
          const double kk = sk[i], ww = sw[i];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const double x = tq[qb + q] - kk;
            a8[q] += ww * exp(-x * x);
          }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[qb + q] += a8[q];
      }
    }
  }
  // Warp sums: lane q < kPerWarp ends with frequency q's.
  double mine = 0.0;
#pragma unroll
  for (int q = 0; q < kPerWarp; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == q) mine = v;
  }
  if (lane < kPerWarp) sred[warp][lane] = mine;
  __syncthreads();
  if (part == 0 && active && lane < kPerWarp) {
    double v = 0.0;
    for (int p = 0; p < kSplit; ++p) v += sred[grp + p * kGroups][lane];
    const int j = j0 + lane;
    if (j < L.nomega) L.part[(int64_t)it.chunk * L.nomega + j] = v;
  }
}

// lehmann_kernel over the tangent of every record: the term's tangent is
// (d w + g x) exp(-x^2), x = t - key, with g = 2 w d key.
__global__ void __launch_bounds__(256) lehmann_tangent_kernel(LehmannArgs A) {
  constexpr int kStage = 1024, kPerWarp = 16, kGroups = kOmegaTile / kPerWarp, kSplit = 8 / kGroups;
  __shared__ double sk[kStage], sw[kStage], sg[kStage], st[kOmegaTile], sred[8][kPerWarp];
  const LehItem it = A.items[blockIdx.x];
  const LehList L = A.lists[it.list];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = warp % kGroups, part = warp / kGroups;
  const int jt = it.tile * kOmegaTile;
  const double ldn = A.log_dn[L.shell], dn = A.dn[L.shell];
  if (threadIdx.x < kOmegaTile) {
    const int j = jt + threadIdx.x;
    double t = 0.0;
    if (j < L.nomega) {
      const int k = A.omega_idx[L.omega_first + j];
      t = L.gauss ? (A.omega[k] / dn) * A.inv_bt : (A.log_omega[k] - ldn) * A.inv_b - A.b_quarter;
    }
    st[threadIdx.x] = t;
  }
  const int j0 = jt + grp * kPerWarp;
  const bool active = j0 < L.nomega;
  double acc[kPerWarp];
#pragma unroll
  for (int q = 0; q < kPerWarp; ++q) acc[q] = 0.0;
  const int64_t r0 = (int64_t)it.chunk * kRecChunk;
  const int64_t r1 = min(r0 + (int64_t)kRecChunk, L.nrec);
  for (int64_t base = r0; base < r1; base += kStage) {
    const int n = (int)min((int64_t)kStage, r1 - base);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      sk[i] = L.key[base + i];
      sw[i] = L.w[base + i];
      sg[i] = L.g[base + i];
    }
    __syncthreads();
    if (!active) continue;
    const double* tq = st + grp * kPerWarp;
    if (it.delta != 0.0) {
      const double d = it.delta, c = exp(-2.0 * d * d), t0 = tq[0];
      for (int i = part * 32 + lane; i < n; i += 32 * kSplit) {
        const double ww = sw[i], gg = sg[i];
        double x = t0 - sk[i];
        double g = exp(-x * x), r = exp(-d * (2.0 * x + d));
        acc[0] += (ww + gg * x) * g;
#pragma unroll
        for (int q = 1; q < kPerWarp; ++q) {
          g *= r;
          r *= c;
          x += d;
          acc[q] += (ww + gg * x) * g;
        }
      }
    } else {
#pragma unroll
      for (int qb = 0; qb < kPerWarp; qb += 8) {
        double a8[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int i = part * 32 + lane; i < n; i += 32 * kSplit) {
          const double kk = sk[i], ww = sw[i], gg = sg[i];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const double x = tq[qb + q] - kk;
            a8[q] += (ww + gg * x) * exp(-x * x);
          }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[qb + q] += a8[q];
      }
    }
  }
  double mine = 0.0;
#pragma unroll
  for (int q = 0; q < kPerWarp; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == q) mine = v;
  }
  if (lane < kPerWarp) sred[warp][lane] = mine;
  __syncthreads();
  if (part == 0 && active && lane < kPerWarp) {
    double v = 0.0;
    for (int p = 0; p < kSplit; ++p) v += sred[grp + p * kGroups][lane];
    const int j = j0 + lane;
    if (j < L.nomega) L.part[(int64_t)it.chunk * L.nomega + j] = v;
  }
}

// A(omega_k): the shells of its window in order, each shell's chunks in
// order, divided by D_N (CalcSpecDM_NRG, SpecFuncClass.cpp:1827-1883).
__global__ void lehmann_fold_kernel(LehmannArgs A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.nomega) return;
  double tot = 0.0;
  for (int s = 0; s < A.win_count[k]; ++s) {
    const int N = A.win_first[k] + s;
    double sh = 0.0;
    for (int g = 0; g < 2; ++g) {
      const int64_t fi = ((int64_t)k * A.window + s) * 2 + g;
      const int li = A.fold_list[fi];
      if (li < 0) continue;
      const LehList L = A.lists[li];
      const int pos = A.fold_pos[fi];
      const int64_t nch = (L.nrec + kRecChunk - 1) / kRecChunk;
      for (int64_t c = 0; c < nch; ++c) sh += L.part[c * L.nomega + pos];
    }
    tot += sh / A.dn[N];
  }
  A.out[k] = tot;
}

}  // namespace

void launch_gemm_jobs(const GemmJob* jobs, const int* tile_job, const int* tile_mn, int ntiles, cudaStream_t s) {
  if (ntiles > 0) gemm_jobs_kernel<<<ntiles, 256, 0, s>>>(jobs, tile_job, tile_mn);
}

void launch_dm_trace(const DmTraceArgs& a, int nblocks, cudaStream_t s) {
  if (nblocks > 0) dm_trace_kernel<<<nblocks, 256, 0, s>>>(a);
}

void launch_dm_records(const DmRecArgs& a, int pass, cudaStream_t s) {
  if (a.nchunks <= 0) return;
  if (pass == 0) {
    dm_count_kernel<<<a.nchunks, 256, 0, s>>>(a);
    dm_scan_kernel<<<1, 1024, 0, s>>>(a);
  } else {
    if (a.ntan > 0) dm_scatter_kernel<true><<<a.nchunks, 256, 0, s>>>(a);
    else dm_scatter_kernel<false><<<a.nchunks, 256, 0, s>>>(a);
  }
}

void launch_lehmann(const LehmannArgs& a, cudaStream_t s) {
  if (a.nitems > 0) lehmann_kernel<<<a.nitems, 256, 0, s>>>(a);
}

void launch_lehmann_tangent(const LehmannArgs& a, cudaStream_t s) {
  if (a.nitems > 0) lehmann_tangent_kernel<<<a.nitems, 256, 0, s>>>(a);
}

void launch_lehmann_fold(const LehmannArgs& a, cudaStream_t s) {
  if (a.nomega > 0) lehmann_fold_kernel<<<(a.nomega + 127) / 128, 128, 0, s>>>(a);
}

}  // namespace nrg
