// H_N block assembly on the device.
//
// Replaces the element loop of CNRGmatrix::DiagHN (DiagHN.cpp:45-76) and the
// per-element rules OneChQS_HN_MatEl (OpMatRules.cpp:1410-1535),
// OneChQSz_HN_MatEl (OpMatRules.cpp:431-537) and TwoChQS_HN_MatEl
// (TwoChQS_OpMatRules.cpp:794-986).  Every element is a product of an old
// operator element (read from the device-resident operator blocks of the
// previous iteration) and a site coefficient that depends only on the block
// spin and the two site types; the coefficients come from host tables built
// with the reference's loop order, and the products/sums below use explicit
// round-to-nearest intrinsics in the reference's evaluation order, so every
// element equals the reference's bit for bit.  Both triangles are written;
// element (r,c) is evaluated as the reference evaluates (min, max).
#include "nrg_device.cuh"

namespace nrg {

namespace {

__device__ __forceinline__ double old_element(const double* op, int64_t off, int ld, int row, int col) {
  return off >= 0 ? op[off + (int64_t)row * ld + col] : 0.0;
}

__global__ void __launch_bounds__(256) assemble_kernel(AssembleArgs A, const int* row_block, const int* row_index) {
  const int64_t row = blockIdx.x;
  const int b = row_block[row];
  const int r = row_index[row];
  const int n = A.bsize[b];
  const int s0 = A.bstate[b];
  const int nseg = A.seg_nseg[b];
  const int NO = A.nchan * A.nsigma;  // old operators entering H_N
  const int NT = A.ntypes;
  const size_t PB = (size_t)NT * NT * NO * 2;
  const double* coef = A.coef + PB * b;
  double* Hrow = A.H + A.hoff[b] + (int64_t)r * n;
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    const int i = min(r, c), j = max(r, c);  // the reference evaluates ist <= jst
    const int gi = s0 + i, gj = s0 + j;
    double v;
    if (i == j) {
      v = __dmul_rn(A.sqrt_lambda, A.st_eold[gi]);
      if (A.onsite) v = __dadd_rn(v, __dmul_rn(A.eN, __dadd_rn(A.site_q[A.st_type[gi]], 1.0)));
    } else {
      const int p = A.st_seg[gi], q = A.st_seg[gj];
      const int ai = A.st_a[gi], aj = A.st_a[gj];
      const int ti = A.st_type[gi], tj = A.st_type[gj];
      const int64_t pt = A.pair_base[b] + ((int64_t)p * nseg + q) * A.nops_h;
      const double* cij = coef + ((size_t)ti * NT + tj) * NO * 2;
      if (A.model == 5) {
        if (A.st_old[gi] == A.st_old[gj]) {
          v = __dsub_rn(__dsub_rn(0.0, __dmul_rn(A.delta, A.sc_pair[ti * NT + tj])),
                        __dmul_rn(A.delta, A.sc_pair[tj * NT + ti]));
        } else {
          // OneChSz_HNsc_MatEl: sum over sigma of FermiSign*OldEl*fd, then
          // times chi_N (sign and table folded into cij, exact)
          double acc = 0.0;
          for (int o = 0; o < 2; ++o) {
            double old = old_element(A.ops[o], A.pair_fwd[pt + o], A.pair_fwd_ld[pt + o], ai, aj);
            int dir = 0;
            if (fabs(old) < 1.e-20 || A.hc_switch[o * NT * NT + ti * NT + tj]) {
              old = old_element(A.ops[o], A.pair_bwd[pt + o], A.pair_bwd_ld[pt + o], aj, ai);
              dir = 1;
            }
            acc = __dadd_rn(acc, __dmul_rn(cij[o * 2 + dir], old));
          }
          v = __dmul_rn(acc, A.chi[0]);
        }
      } else if (A.model == 4) {
        if (A.st_old[gi] == A.st_old[gj]) {
          // OneChS_HNsc_MatEl: the lead's pairing term on the new site
          v = __dsub_rn(__dsub_rn(0.0, __dmul_rn(A.delta, A.sc_pair[ti * NT + tj])),
                        __dmul_rn(A.delta, A.sc_pair[tj * NT + ti]));
        } else {
          double old = old_element(A.ops[0], A.pair_fwd[pt], A.pair_fwd_ld[pt], ai, aj);
          int dir = 0;
          if (fabs(old) < 1.e-20 || A.hc_switch[ti * NT + tj]) {
            old = old_element(A.ops[0], A.pair_bwd[pt], A.pair_bwd_ld[pt], aj, ai);
            dir = 1;
          }
          v = __dmul_rn(__dmul_rn(A.chi[0], old), cij[dir]);
        }
      } else if (A.model == 0) {
        // ((chi_N*OldEl)*CoefMatEl)*FermiSign, FermiSign folded into the table.
        double old = old_element(A.ops[0], A.pair_fwd[pt], A.pair_fwd_ld[pt], ai, aj);
        int dir = 0;
        if (fabs(old) < 1.e-20) { old = old_element(A.ops[0], A.pair_bwd[pt], A.pair_bwd_ld[pt], aj, ai); dir = 1; }
        v = __dmul_rn(__dmul_rn(A.chi[0], old), cij[dir]);
      } else if (A.model == 1) {
        // sum over sigma of FermiSign*OldEl*fd, then times chi_N.
        double acc = 0.0;
        for (int o = 0; o < 2; ++o) {
          double old = old_element(A.ops[o], A.pair_fwd[pt + o], A.pair_fwd_ld[pt + o], ai, aj);
          int dir = 0;
          if (fabs(old) < 1.e-20) { old = old_element(A.ops[o], A.pair_bwd[pt + o], A.pair_bwd_ld[pt + o], aj, ai); dir = 1; }
          acc = __dadd_rn(acc, __dmul_rn(cij[o * 2 + dir], old));
        }
        v = __dmul_rn(acc, A.chi[0]);
      } else {
        // sum over channels and sigma of (chi_ch*OldEl_ch)*FullMatEl.
        double acc = 0.0;
        for (int ch = 0; ch < 2; ++ch) {
          double old = old_element(A.ops[ch], A.pair_fwd[pt + ch], A.pair_fwd_ld[pt + ch], ai, aj);
          int dir = 0;
          if (fabs(old) < 1.e-20) { old = old_element(A.ops[ch], A.pair_bwd[pt + ch], A.pair_bwd_ld[pt + ch], aj, ai); dir = 1; }
          const double x = __dmul_rn(A.chi[ch], old);
          acc = __dadd_rn(acc, __dmul_rn(x, cij[(ch * 2 + 0) * 2 + dir]));
          acc = __dadd_rn(acc, __dmul_rn(x, cij[(ch * 2 + 1) * 2 + dir]));
        }
        v = acc;
      }
    }
    Hrow[c] = v;
  }
}

}  // namespace

void launch_assemble(const AssembleArgs& a, int64_t total_rows, const int* row_block, const int* row_index,
                     cudaStream_t s) {
  if (total_rows <= 0) return;
  assemble_kernel<<<(unsigned)total_rows, 256, 0, s>>>(a, row_block, row_index);
}

}  // namespace nrg
