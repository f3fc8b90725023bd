// Eigenpairs of the tridiagonal matrices left by the tridiagonalization, and
// the back-transformation to eigenvectors of the H_N blocks (FP64).
//
// Together with k_tridiag.cu this replaces the per-block dspev call of
// CNRGmatrix::DiagBlock (NRGmatrixClass.cpp:566-696).  Eigenvalues come from
// Sturm-count bisection (one thread per eigenvalue, all blocks in one grid);
// eigenvectors are only formed for the states that survive the cut (the
// reference keeps only those rows of dEigVec, CutStates.cpp:10-95 and
// RemoveStatesFromBlock NRGarrayClass.cpp:1467-1548): inverse iteration per
// wanted eigenvalue (one thread per vector), a modified Gram-Schmidt pass over
// clusters of close eigenvalues, then the Householder reflectors are applied
// in reverse order with one warp per eigenvector.
#include <cfloat>

#include "nrg_device.cuh"

namespace nrg {

namespace {

constexpr double kEps = 2.220446049250313e-16;

// e2: the squared off-diagonal, formed once per call (a square in every
// pass of every level would cost an FP64 multiply per step).
__device__ __forceinline__ int sturm_count(const double* d, const double* e2, int n, double x, double pivmin) {
  int cnt = 0;
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0.0) cnt++;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e2[i - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) cnt++;
  }
  return cnt;
}

// FP32 Sturm count over FP32 copies of d and e, made once per call (a
// double-to-float conversion in the pass itself would run on the FP64 pipe).
__device__ __forceinline__ int sturm_count_f32(const float* d, const float* e, int n, float x, float pivmin) {
  int cnt = 0;
  float q = d[0] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  if (q < 0.0f) cnt++;
  for (int i = 1; i < n; ++i) {
    const float ei = e[i - 1];
    q = (d[i] - x) - __fdividef(ei * ei, q);
    if (fabsf(q) < pivmin) q = -pivmin;
    if (q < 0.0f) cnt++;
  }
  return cnt;
}

// One FP64 pass: Sturm count of T - x and, from the pivot recurrence q_i
// and its first two derivatives, S1 = sum q_i'/q_i = f'/f and
// S2 = sum (q_i''/q_i - (q_i'/q_i)^2) = (log f)'' of f(x) = det(T - x).
__device__ __forceinline__ int sturm_sums(const double* d, const double* e2v, int n, double x, double pivmin,
                                          double* S1, double* S2) {
  int cnt = 0;
  double q = d[0] - x, dq = -1.0, ddq = 0.0;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0.0) cnt++;
  double r = 1.0 / q;
  double u = dq * r;
  double s1 = u, s2 = -u * u;
  for (int i = 1; i < n; ++i) {
    const double e2 = e2v[i - 1];
    const double qn = (d[i] - x) - e2 * r;
    const double e2rr = e2 * r * r;
    const double ddqn = e2rr * fma(-2.0 * dq * dq, r, ddq);
    dq = fma(e2rr, dq, -1.0);
    ddq = ddqn;
    q = fabs(qn) < pivmin ? -pivmin : qn;
    if (q < 0.0) cnt++;
    r = 1.0 / q;
    u = dq * r;
    s1 += u;
    s2 = fma(ddq, r, fma(-u, u, s2));
  }
  *S1 = s1;
  *S2 = s2;
  return cnt;
}

// Step towards the wanted level from a local two-level model
// f ~ C (x-a)(x-b): 1/(x-a) + 1/(x-b) = S1 and 1/(x-a)^2 + 1/(x-b)^2 = -S2
// (Laguerre's step for degree 2).  `above` tells on which side of x the
// level lies and `rank` how many levels of that side come first (both from
// the Sturm count at x).  A level with a close partner (the channel doublets
// of the two-channel model) is then reached in a few steps, where Newton on f
// converges only linearly; without a real two-level fit the Newton step on
// f/f' (S1/S2) is taken.
__device__ __forceinline__ double pair_step(double S1, double S2, bool above, int rank) {
  const double disc = -2.0 * S2 - S1 * S1;
  if (disc >= 0.0) {
    const double sq = sqrt(disc);
    const double t1 = 0.5 * (S1 + sq), t2 = 0.5 * (S1 - sq);
    const double d1 = t1 != 0.0 ? -1.0 / t1 : 0.0, d2 = t2 != 0.0 ? -1.0 / t2 : 0.0;
    const bool ok1 = t1 != 0.0 && ((d1 > 0.0) == above), ok2 = t2 != 0.0 && ((d2 > 0.0) == above);
    if (ok1 && ok2) {
      const double nearer = fabs(d1) <= fabs(d2) ? d1 : d2, farther = fabs(d1) <= fabs(d2) ? d2 : d1;
      return rank == 0 ? nearer : farther;
    }
    if (ok1) return d1;
    if (ok2) return d2;
  }
  return S1 / S2;
}

// e_i is negligible next to its diagonal neighbours (the splitting test of
// LAPACK's tridiagonal solvers): the block then falls apart into unreduced
// pieces whose eigenvalues are simple.
__device__ __forceinline__ bool split_at(const double* d, const double* e, int i) {
  const double ei = e[i];
  return ei * ei <= (kEps * kEps) * fabs(d[i] * d[i + 1]) || ei == 0.0;
}

// One thread per diagonal position k of each tridiagonal block: the piece
// (unreduced sub-block) containing position k is found, and thread k
// computes that piece's (k - start)-th eigenvalue.  Over all threads this is
// every eigenvalue of the block exactly once; sort_levels orders them.  On a
// piece the levels are simple, so after an FP32 Sturm bisection to about
// 1e-6 of the piece's spectral radius, safeguarded FP64 steps from a local
// two-level model (pair_step) converge in a few passes also next to a
// near-degenerate partner (a bisection step whenever the model step leaves
// the bracket); every FP64 pass also tightens the bracket with its Sturm
// count.  Dropping the negligible e_i moves the levels by at
// most one ulp of the neighbouring diagonal.
__global__ void bisect_kernel(TdEigArgs A, const int* state_block) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.nstates) return;
  const int b = state_block[g];
  const int nb = A.bsize[b];
  const int so = A.soff[b];
  const int pos = g - so;
  const double* db = A.d + so;
  const double* eb = A.e + so;
  int s0 = pos, s1 = pos;
  const unsigned char* spl = A.split + so;  // split_at for every position, formed once per call
  while (s0 > 0 && !spl[s0 - 1]) --s0;
  while (s1 < nb - 1 && !spl[s1]) ++s1;
  const int n = s1 - s0 + 1;
  const int k = pos - s0;
  const double* d = db + s0;
  const double* e = eb + s0;
  const float* fd32 = A.fde + so + s0;
  const float* fe32 = A.fde + A.nstates + so + s0;
  const double* e2 = A.e2 + so + s0;
  if (n == 1) {
    if (!isfinite(d[0])) atomicOr(A.flag, DEV_BAD_INPUT);
    A.ev[g] = d[0];
    return;
  }
  // Gershgorin bounds in FP32, widened past their rounding: they only seed
  // the bracket.
  float fgl = FLT_MAX, fgu = -FLT_MAX, femax = 0.0f;
  for (int i = 0; i < n; ++i) {
    const float fe0 = i > 0 ? fabsf(fe32[i - 1]) : 0.0f, fe1 = i + 1 < n ? fabsf(fe32[i]) : 0.0f;
    const float fd = fd32[i];
    fgl = fminf(fgl, fd - (fe0 + fe1));
    fgu = fmaxf(fgu, fd + (fe0 + fe1));
    femax = fmaxf(femax, fe1);
  }
  const double tnorm = fmax(fabs((double)fgl), fabs((double)fgu));
  const double emax2 = (double)femax * (double)femax;
  const double pivmin = DBL_MIN * fmax(1.0, emax2);
  double lo = (double)fgl - 1e-6 * tnorm - 2.0 * kEps * tnorm * n - 2.0 * pivmin;
  double hi = (double)fgu + 1e-6 * tnorm + 2.0 * kEps * tnorm * n + 2.0 * pivmin;
  const double atol = 1e-3 * kEps * fmax(tnorm, DBL_MIN);
  int clo = -1, chi = -1;  // Sturm counts at lo / hi once checked in FP64
  double x0 = 0.5 * (lo + hi);
  // FP32 bracket
  if (tnorm > 1e-30 && tnorm < 1e30) {
    float flo = (float)lo, fhi = (float)hi;
    const float fpiv = 1e-30f;
    for (int it = 0; it < 40 && (fhi - flo) > 1e-6f * (float)tnorm; ++it) {
      const float mid = 0.5f * (flo + fhi);
      if (sturm_count_f32(fd32, fe32, n, mid, fpiv) > k) fhi = mid; else flo = mid;
    }
    x0 = 0.5 * ((double)flo + (double)fhi);  // within 1e-6 tnorm of the level: the first step lands
    const double margin = 1e-5 * tnorm;
    const double tlo = (double)flo - margin, thi = (double)fhi + margin;
    if (tlo > lo) {
      const int c = sturm_count(d, e2, n, tlo, pivmin);
      if (c <= k) { lo = tlo; clo = c; }
    }
    if (thi < hi) {
      const int c = sturm_count(d, e2, n, thi, pivmin);
      if (c > k) { hi = thi; chi = c; }
    }
  }
  // The bracket holds the k-th level alone: Newton kept inside it can only
  // converge to that level.
  const bool unique = clo == k && chi == k + 1;
  // Stop at a few ulps of the spectral radius: below that the Sturm counts
  // are at the round-off of the recurrence.
  const double floor_w = fmax(8.0 * kEps * tnorm, atol);
  double x = (x0 > lo && x0 < hi) ? x0 : 0.5 * (lo + hi);
  double v = x;
  bool newton = true, done = false;
  for (int it = 0; it < 200 && !done; ++it) {
    if (hi - lo <= fmax(2.0 * kEps * fmax(fabs(lo), fabs(hi)), floor_w)) break;
    if (it >= 16) newton = false;  // a model step that has not converged by now: bisect
    if (!newton) {
      // plain bisection needs the count alone (about half the FP64 work of a
      // pass with the derivative sums)
      const int c = sturm_count(d, e2, n, x, pivmin);
      if (c > k) hi = x; else lo = x;
      x = 0.5 * (lo + hi);
      v = x;
      continue;
    }
    double S1, S2;
    const int c = sturm_sums(d, e2, n, x, pivmin, &S1, &S2);
    if (c > k) hi = x; else lo = x;
    const bool above = c <= k;
    const double step = pair_step(S1, S2, above, above ? k - c : c - 1 - k);
    double xn = 0.5 * (lo + hi);
    if (isfinite(step)) {
      // round-off floor of the recurrence: a few ulps of the spectral radius
      const double small = 4.0 * kEps * fabs(x) + 16.0 * kEps * tnorm;
      if (fabs(step) <= small) {
        // converged: accept only if the k-th level is within reach of x + step;
        // the count at x already settles the side x is on
        // A group of levels split only by round-off (the two-channel
        // spectrum's channel partners and free-chain combinations) is accepted
        // as resolved at 64 ulps of the spectral radius, about the accuracy
        // LAPACK's solvers give such a group; for a block reduced in mixed
        // precision, whose reduction leaves the levels about 2^-36 of the
        // block's scale apart from H's, at 2^-40 of the spectral radius.
        const double gtol = (A.mixed_n > 0 && nb >= A.mixed_n) ? 0x1p-40 : 64.0 * kEps;
        const double xc = x + step, del = fmax(2.0 * fabs(step) + small, gtol * tnorm);
        bool ok;
        // The bracket holding the k-th level alone settles it, provided x is
        // near a root (|f'/f| large): a small step also comes out at a
        // stationary point of f between two levels (S1 = 0), which the
        // bracket can hold too; there the Sturm counts decide.
        if (unique && xc >= lo && xc <= hi && fabs(S1) * small >= 1.0) ok = true;
        else if (above && step >= 0.0) ok = sturm_count(d, e2, n, xc + del, pivmin) > k;
        else if (!above && step <= 0.0) ok = sturm_count(d, e2, n, xc - del, pivmin) <= k;
        else ok = sturm_count(d, e2, n, xc - del, pivmin) <= k && sturm_count(d, e2, n, xc + del, pivmin) > k;
        if (ok) {
          v = xc;
          done = true;
          break;
        }
        newton = false;
      } else if (x + step > lo && x + step < hi) {
        xn = x + step;
      }
    }
    x = xn;
    v = x;
  }
  if (!done) v = 0.5 * (lo + hi);  // the bracket always holds the k-th level
  if (!isfinite(v)) atomicOr(A.flag, DEV_BAD_INPUT);
  A.ev[g] = v;
}

// Levels come out piece by piece (and two close levels of one piece can come
// out an ulp out of order); CutStates reads a block's levels as ascending
// (its first level above E_cut ends the block).  Each block is sorted in
// shared memory with a bitonic network, one CTA per block, padded with +inf
// to a power of two.
__global__ void sort_levels_kernel(TdEigArgs A, int pmax) {
  extern __shared__ double sv[];
  const int b = blockIdx.x;
  const int n = A.bsize[b];
  double* v = A.ev + A.soff[b];
  int P = 1;
  while (P < n) P <<= 1;
  if (P > pmax) return;  // launched only when every block fits
  for (int i = threadIdx.x; i < P; i += blockDim.x) sv[i] = i < n ? v[i] : DBL_MAX;
  for (int size = 2; size <= P; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      for (int i = threadIdx.x; i < (P >> 1); i += blockDim.x) {
        const int lo = 2 * i - (i & (stride - 1));
        const int hi = lo + stride;
        const bool asc = (lo & size) == 0;
        const double x = sv[lo], y = sv[hi];
        if ((x > y) == asc) { sv[lo] = y; sv[hi] = x; }
      }
    }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) v[i] = sv[i];
}

// Fallback for blocks too large for the shared-memory sort: odd-even
// transposition passes in global memory, one CTA per block, stopping after
// two passes without a swap; n + 1 passes always suffice.
__global__ void order_levels_kernel(TdEigArgs A) {
  const int b = blockIdx.x;
  const int n = A.bsize[b];
  double* v = A.ev + A.soff[b];
  int quiet = 0;
  for (int pass = 0; pass <= n && quiet < 2; ++pass) {
    int swapped = 0;
    for (int i = 2 * threadIdx.x + (pass & 1); i + 1 < n; i += 2 * blockDim.x) {
      const double x = v[i], y = v[i + 1];
      if (y < x) { v[i] = y; v[i + 1] = x; swapped = 1; }
    }
    quiet = __syncthreads_or(swapped) ? 0 : quiet + 1;
  }
}

// Deterministic pseudo-random start vector component in (-1, 1).
__device__ __forceinline__ double start_component(int k, int i) {
  uint64_t z = ((uint64_t)(uint32_t)k << 32) ^ (uint64_t)(uint32_t)i ^ 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
}

// One thread per wanted eigenvector.  Scratch per block: five interleaved
// n x nv arrays (l, 1/u1, u2, u3, pivot flag); Y is interleaved n x nv.
__global__ void inviter_kernel(InvIterArgs A, const int* vec_block, const int* vec_index, int nvecs) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nvecs) return;
  const int b = vec_block[g];
  const int k = vec_index[g];
  const int n = A.bsize[b];
  const int so = A.soff[b];
  const int nv = A.nvec[b];
  const double* d = A.d + so;
  const double* e = A.e + so;
  const double* ev = A.ev + so;
  double* Y = A.Y + A.yoff[b];
  double* L = A.scratch + 5 * A.yoff[b];
  double* IU1 = L + (int64_t)n * nv;
  double* U2 = IU1 + (int64_t)n * nv;
  double* U3 = U2 + (int64_t)n * nv;
  double* PV = U3 + (int64_t)n * nv;
#define AT(arr, i) arr[(int64_t)(i) * nv + k]
  double onenrm = 0.0;
  for (int i = 0; i < n; ++i)
    onenrm = fmax(onenrm, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0));
  if (onenrm == 0.0) {
    // T = 0 (a block of exactly degenerate zero levels, e.g. a decoupled
    // impurity beside an empty chain): every unit vector is an eigenvector,
    // and the identity is what the reference's dspev returns for it.
    for (int i = 0; i < n; ++i) AT(Y, i) = (i == k) ? 1.0 : 0.0;
    return;
  }
  // Shift: separate numerically equal eigenvalues as LAPACK dstein does.
  double sigma = ev[k];
  {
    int run = 0;
    for (int kk = k - 1; kk >= 0 && ev[k] - ev[kk] < 10.0 * kEps * fmax(fabs(ev[k]), onenrm * 1e-3); --kk) run++;
    sigma += run * 10.0 * kEps * fmax(fabs(ev[k]), onenrm * 1e-3);
  }
  if (n == 1) { AT(Y, 0) = 1.0; return; }
  // LU with partial pivoting of T - sigma I (rows i, i+1 may swap).
  const double tiny = kEps * onenrm;
  double u1 = d[0] - sigma, u2 = e[0];
  for (int i = 0; i + 1 < n; ++i) {
    const double c = e[i];                  // sub-diagonal below row i
    const double an = d[i + 1] - sigma;     // next diagonal
    const double bn = (i + 2 < n) ? e[i + 1] : 0.0;
    double l, nu1, nu2, r1, r2, r3;
    if (fabs(c) > fabs(u1)) {               // swap rows i and i+1
      l = u1 / c;
      r1 = c; r2 = an; r3 = bn;
      nu1 = u2 - l * an; nu2 = -l * bn;
      AT(PV, i) = 1.0;
    } else {
      if (fabs(u1) < tiny) u1 = copysign(tiny, u1);
      l = c / u1;
      r1 = u1; r2 = u2; r3 = 0.0;
      nu1 = an - l * u2; nu2 = bn;
      AT(PV, i) = 0.0;
    }
    if (fabs(r1) < tiny) r1 = copysign(tiny, r1);
    AT(L, i) = l; AT(IU1, i) = 1.0 / r1; AT(U2, i) = r2; AT(U3, i) = r3;
    u1 = nu1; u2 = nu2;
  }
  if (fabs(u1) < tiny) u1 = copysign(tiny, u1);
  AT(IU1, n - 1) = 1.0 / u1; AT(U2, n - 1) = 0.0; AT(U3, n - 1) = 0.0; AT(L, n - 1) = 0.0; AT(PV, n - 1) = 0.0;
  const double last = fabs(u1);
  for (int i = 0; i < n; ++i) AT(Y, i) = start_component(k, i);
  const double dtpcrt = sqrt(0.1 / n);
  int extra = 0;
  bool conv = false;
  for (int it = 0; it < 8; ++it) {
    double asum = 0.0;
    for (int i = 0; i < n; ++i) asum += fabs(AT(Y, i));
    const double scl = n * onenrm * fmax(kEps, last) / fmax(asum, DBL_MIN);
    // forward: P and L, in place
    double xi = AT(Y, 0) * scl;
    for (int i = 0; i + 1 < n; ++i) {
      double xn = AT(Y, i + 1) * scl;
      if (AT(PV, i) != 0.0) { const double t = xi; xi = xn; xn = t - AT(L, i) * xn; }
      else xn = xn - AT(L, i) * xi;
      AT(Y, i) = xi;
      xi = xn;
    }
    AT(Y, n - 1) = xi;
    // backward: U
    double x2 = 0.0, x1 = 0.0;
    double nrmmax = 0.0;
    for (int i = n - 1; i >= 0; --i) {
      const double x = (AT(Y, i) - AT(U2, i) * x1 - AT(U3, i) * x2) * AT(IU1, i);
      AT(Y, i) = x;
      x2 = x1; x1 = x;
      nrmmax = fmax(nrmmax, fabs(x));
    }
    // normalise to max 1 to keep the next scaling in range
    const double inv = 1.0 / fmax(nrmmax, DBL_MIN);
    for (int i = 0; i < n; ++i) AT(Y, i) *= inv;
    if (nrmmax >= dtpcrt) { conv = true; if (++extra >= 2) break; }
  }
  if (!conv) atomicOr(A.flag, DEV_NOT_CONVERGED);
  double s2 = 0.0, big = 0.0;
  int jmax = 0;
  for (int i = 0; i < n; ++i) {
    const double x = AT(Y, i);
    s2 += x * x;
    if (fabs(x) > big) { big = fabs(x); jmax = i; }
  }
  double nrm = 1.0 / sqrt(s2);
  if (AT(Y, jmax) < 0.0) nrm = -nrm;
  for (int i = 0; i < n; ++i) AT(Y, i) *= nrm;
#undef AT
}

// Modified Gram-Schmidt over each cluster of close eigenvalues (one warp per
// cluster, vectors in ascending order, two passes).
__global__ void mgs_kernel(InvIterArgs A) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= A.nclusters) return;
  const int b = A.cl_block[warp], k0 = A.cl_first[warp], cnt = A.cl_count[warp];
  if (cnt < 2) return;
  const int n = A.bsize[b], nv = A.nvec[b];
  double* Y = A.Y + A.yoff[b];
  for (int kk = 1; kk < cnt; ++kk) {
    const int k = k0 + kk;
    for (int pass = 0; pass < 2; ++pass) {
      for (int jj = 0; jj < kk; ++jj) {
        const int j = k0 + jj;
        double dot = 0.0;
        for (int i = lane; i < n; i += 32) dot = fma(Y[(int64_t)i * nv + j], Y[(int64_t)i * nv + k], dot);
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        for (int i = lane; i < n; i += 32) Y[(int64_t)i * nv + k] = fma(-dot, Y[(int64_t)i * nv + j], Y[(int64_t)i * nv + k]);
      }
      double s2 = 0.0;
      for (int i = lane; i < n; i += 32) { const double x = Y[(int64_t)i * nv + k]; s2 = fma(x, x, s2); }
      for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      const double inv = 1.0 / sqrt(s2);
      for (int i = lane; i < n; i += 32) Y[(int64_t)i * nv + k] *= inv;
    }
  }
}

constexpr int kBackWarps = 8;

// Apply H_0 H_1 ... H_{n-3} to the eigenvectors of T.  One CTA takes up to
// eight eigenvectors of one block; each reflector is staged once in shared
// memory for all of them.
__global__ void __launch_bounds__(kBackWarps * 32) backtransform_kernel(BackArgs A, const int* cta_block,
                                                                       const int* cta_first) {
  extern __shared__ double sm[];
  const int b = cta_block[blockIdx.x];
  const int k0 = cta_first[blockIdx.x];
  const int n = A.bsize[b];
  const int nv = A.nvec[b];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = k0 + warp;
  const bool active = k < nv;
  double* vbuf = sm;                       // n
  double* y = sm + A.maxn * (1 + warp);    // n per warp
  const double* Yb = A.Y + A.yoff[b];
  if (active)
    for (int i = lane; i < n; i += 32) y[i] = Yb[(int64_t)i * nv + k];
  const double* H = A.H_const;
  const double* tau = A.tau + A.soff[b];
  for (int j = n - 3; j >= 0; --j) {
    __syncthreads();
    const double* vrow = H + A.hoff[b] + (int64_t)j * n;
    for (int c = j + 1 + threadIdx.x; c < n; c += blockDim.x) vbuf[c] = vrow[c];
    __syncthreads();
    const double t = tau[j];
    if (!active || t == 0.0) continue;
    double dot = 0.0;
    for (int c = j + 1 + lane; c < n; c += 32) dot = fma(vbuf[c], y[c], dot);
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
    const double s = t * dot;
    for (int c = j + 1 + lane; c < n; c += 32) y[c] = fma(-s, vbuf[c], y[c]);
  }
  if (!active) return;
  double* Zb = A.Z + A.zoff[b] + (int64_t)k * n;
  for (int i = lane; i < n; i += 32) Zb[i] = y[i];
  if (A.Zt) {
    double* Ztb = A.Zt + A.zoff[b];
    for (int i = lane; i < n; i += 32) Ztb[(int64_t)i * nv + k] = y[i];
  }
}

}  // namespace

// FP32 copies of d and e for the FP32 bracket, e^2 for the FP64 passes, and
// the splitting test at every position (the last state of a block has e = 0).
__global__ void prep_levels_kernel(const double* d, const double* e, float* out, double* e2, unsigned char* spl,
                                   int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    out[i] = (float)d[i];
    out[n + i] = (float)e[i];
    e2[i] = e[i] * e[i];
    spl[i] = (i + 1 < n) ? (split_at(d, e, i) ? 1 : 0) : 1;
  }
}

void launch_bisect(const TdEigArgs& a, const int* state_block, cudaStream_t s) {
  if (a.nstates <= 0) return;
  prep_levels_kernel<<<(a.nstates + 255) / 256 < 1024 ? (a.nstates + 255) / 256 : 1024, 256, 0, s>>>(
      a.d, a.e, a.fde, a.e2, a.split, a.nstates);
  // One warp per CTA: the long-running threads of the largest blocks then
  // spread over all SMs instead of crowding a few.
  bisect_kernel<<<(a.nstates + 31) / 32, 32, 0, s>>>(a, state_block);
  int P = 1;
  while (P < a.maxn) P <<= 1;
  const size_t smem = sizeof(double) * (size_t)P;
  if (smem <= (size_t)max_dyn_smem() &&
      cudaFuncSetAttribute(sort_levels_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem()) ==
          cudaSuccess) {
    sort_levels_kernel<<<a.nblocks, 512, smem, s>>>(a, P);
  } else {
    order_levels_kernel<<<a.nblocks, 256, 0, s>>>(a);
  }
}

void launch_inviter(const InvIterArgs& a, const int* vec_block, const int* vec_index, int nvecs, cudaStream_t s) {
  if (nvecs > 0) inviter_kernel<<<(nvecs + 63) / 64, 64, 0, s>>>(a, vec_block, vec_index, nvecs);
  if (a.nclusters > 0) mgs_kernel<<<(a.nclusters * 32 + 127) / 128, 128, 0, s>>>(a);
}

int backtransform_warps(int maxn) {
  int w = (int)((220 * 1024) / (sizeof(double) * (size_t)maxn)) - 1;
  return w < 1 ? 1 : (w > kBackWarps ? kBackWarps : w);
}
size_t backtransform_smem_bytes(int maxn) { return sizeof(double) * (size_t)maxn * (1 + backtransform_warps(maxn)); }

cudaError_t launch_backtransform(const BackArgs& a, const int* cta_block, const int* cta_first, int nctas,
                                 cudaStream_t s) {
  if (nctas <= 0) return cudaSuccess;
  size_t smem = backtransform_smem_bytes(a.maxn);
  cudaError_t err = cudaFuncSetAttribute(backtransform_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem());
  if (err != cudaSuccess) return err;
  backtransform_kernel<<<nctas, backtransform_warps(a.maxn) * 32, smem, s>>>(a, cta_block, cta_first);
  return cudaGetLastError();
}

}  // namespace nrg
