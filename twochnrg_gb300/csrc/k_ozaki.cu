// FP64-accurate rank-k products on the tcgen05 tensor cores.
//
//   C[i][j] += alpha * sum_k A[i][k] * B[j][k]      (i < m, j < n, k < K <= 256)
//
// A and B are FP64.  Each row is scaled by a power of two so that its largest
// magnitude is at most 1, and the scaled row is cut into S fixed-point slices
// of 8 bits: x / 2^e = 2^-7 sum_t c_t 2^-8t with integers |c_t| <= 128.  A
// slice is stored in BF16 as c_t 2^-8t, which BF16 holds exactly (8
// significant bits).  The product of slices s and t is then a sum of terms
// c_s d_t 2^-8(s+t): the tensor core forms it in FP32 without rounding as long
// as the sum stays below 2^24 units of its last place (products <= 2^14).
// Four TMEM accumulators collect the slice pairs of level s + t = 0, 1, 2
// (exact for K <= 256: at level 2, 3 pairs x 256 x 2^14 x 2^-16 < 2^24 x
// 2^-16) and 3 <= s + t < S together (its magnitude is below 2^-2 of the
// leading level's unit, so FP32 rounds it at about 2^-25 of that unit); the
// epilogue joins them without FP64 arithmetic -- the first three are exact
// integers in units of 1, 2^-8 and 2^-16, the fourth is rounded to units of
// 2^-24 (below its own FP32 rounding), and the four are combined in one int64
// -- then makes one conversion to FP64, applies the column's power-of-two
// scale in the exponent field and the row's scale and alpha in the single
// FMA into C: two FP64 operations per element, where the FP64 pipe is the
// scarce resource of this GPU.  With
// S = 6 (21 BF16 products per element pair) the dropped levels (below
// 2^-48) and the rounding of the fourth accumulator (about 2^-39 per
// addition) leave an error of order 2^-36 sqrt(K/64) |A_i| |B_j|; with S = 5,
// 2^-35.  The NRG trailing updates use S = 6.
//
// The MMA is tcgen05.mma kind::f16 (BF16 x BF16 -> FP32), M = N = 128, K = 16
// per instruction, one CTA (cta_group::1), issued by one thread; operand
// tiles (128 rows x 64 BF16 = 128 bytes, 128-byte swizzle) are staged in
// shared memory by TMA (cp.async.bulk.tensor) against an mbarrier, and the
// accumulators live in tensor memory (4 x 128 = all 512 columns) and are read
// back with tcgen05.ld by the four epilogue warps (warp w owns lanes 32w..).
//
// Every wait on an mbarrier is bounded: on expiry the kernel raises
// DEV_TIMEOUT in the flag word, waits (bounded) for its own copies, frees its
// tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "nrg_device.cuh"

namespace nrg {

namespace {

constexpr int kTile = 128;           // output tile rows and columns
constexpr int kChunk = 64;           // BF16 per swizzled operand row (128 bytes)
constexpr int kSliceBytes = kTile * kChunk * 2;  // one operand slice tile: 16 KB
constexpr uint32_t kTmemCols = 512;  // four 128-column FP32 accumulators

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait for the phase of the given parity (about a second at most).
__device__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < (1 << 24); ++it) {
    if (mbar_try(bar, parity)) return true;
    if (it > 64) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile with 128-byte
// swizzle: rows of 128 bytes, 8-row atoms 1024 bytes apart (stride byte
// offset), one atom along K (leading byte offset unused), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// BF16 (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTile >> 3) << 17) |
                            ((uint32_t)(kTile >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// One warp per row: the row's power-of-two scale 2^ex (ex stored) and its S slices.  Rows at
// or past `rows` (padding up to the slab height) and columns at or past K
// (padding to whole 64-column chunks) are written as zeros.  swap_halves
// reads column (k + K/2) mod K instead of k: [W V] from a stored [V W].
__global__ void oz_split_kernel(const double* __restrict__ X, int64_t ldx, int rows, int K, int kpad, int slab,
                                int S, int swap_halves, __nv_bfloat16* __restrict__ out,
                                int* __restrict__ scale_exp) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= slab) return;
  const int r = warp;
  double mx = 0.0;
  if (r < rows)
    for (int k = lane; k < K; k += 32) mx = fmax(mx, fabs(X[(int64_t)r * ldx + k]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  int ex = 0;
  if (mx > 0.0) frexp(mx, &ex);  // mx = f 2^ex, f in [0.5, 1): |x| / 2^ex <= 1
  if (lane == 0 && r < rows) scale_exp[r] = mx > 0.0 ? ex : 0;
  const int half = K / 2;
  for (int k = lane; k < kpad; k += 32) {
    double x = 0.0;
    if (r < rows && k < K) {
      const int src = swap_halves ? (k < half ? k + half : k - half) : k;
      x = X[(int64_t)r * ldx + src];
    }
    double v = mx > 0.0 ? ldexp(x, 7 - ex) : 0.0;  // |v| <= 128, exact
    for (int t = 0; t < S; ++t) {
      const double c = rint(v);                   // integer, |c| <= 128
      out[((int64_t)t * slab + r) * kpad + k] = __double2bfloat16(ldexp(c, -8 * t));
      v = (v - c) * 256.0;                        // exact: |v - c| <= 1/2
    }
  }
}

struct OzArgs {
  double* C;
  int64_t ldc;
  int m, n;
  int kchunks;       // K / 64, rounded up
  int S;             // slices per operand
  int slab_a, slab_b;  // rows per slice slab of the A and B slice arrays
  double alpha;
  const int* ea;     // row scale exponents of A and B (row i scaled by 2^ea[i])
  const int* eb;
  int tiles_n;
  int ntiles;
  int* flag;
};

__global__ void __launch_bounds__(128, 1) oz_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmB, OzArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int S = g.S;
  uint8_t* sA = smem;
  uint8_t* sB = smem + (size_t)S * kSliceBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + (size_t)S * kSliceBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2);
  volatile int* sfail = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t bar_load = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[1]);

  if (tid == 0) {
    mbar_init(bar_load, 1);
    mbar_init(bar_mma, 1);
    *sfail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;
  uint32_t ph_load = 0, ph_mma = 0;
  bool failed = false;

  for (int tile = blockIdx.x; tile < g.ntiles && !failed; tile += gridDim.x) {
    const int ti = tile / g.tiles_n, tj = tile - ti * g.tiles_n;
    bool acc_used[4] = {false, false, false, false};
    for (int kc = 0; kc < g.kchunks; ++kc) {
      if (tid == 0) {
        mbar_expect_tx(bar_load, (uint32_t)(2 * S * kSliceBytes));
        for (int s = 0; s < S; ++s)
          tma_load_2d(smem_u32(sA + (size_t)s * kSliceBytes), &tmA, kc * kChunk, s * g.slab_a + ti * kTile, bar_load);
        for (int t = 0; t < S; ++t)
          tma_load_2d(smem_u32(sB + (size_t)t * kSliceBytes), &tmB, kc * kChunk, t * g.slab_b + tj * kTile, bar_load);
        if (!mbar_wait(bar_load, ph_load)) {
          *sfail = 1;
          mbar_wait(bar_load, ph_load);  // second bounded wait for the copies in flight
        } else {
          fence_after();
          for (int s = 0; s < S; ++s)
            for (int t = 0; s + t < S; ++t) {
              const int a = s + t < 3 ? s + t : 3;
              const uint32_t d = tmem + (uint32_t)(a * kTile);
#pragma unroll
              for (int kk = 0; kk < kChunk / 16; ++kk) {
                const uint64_t ad = sw128_desc(smem_u32(sA + (size_t)s * kSliceBytes + kk * 32));
                const uint64_t bd = sw128_desc(smem_u32(sB + (size_t)t * kSliceBytes + kk * 32));
                mma_bf16(d, ad, bd, acc_used[a] ? 1u : 0u);
                acc_used[a] = true;
              }
            }
          mma_commit(bar_mma);
        }
      }
      ph_load ^= 1;
      __syncthreads();
      if (*sfail) { failed = true; break; }
      if (!mbar_wait(bar_mma, ph_mma)) *sfail = 1;
      ph_mma ^= 1;
      __syncthreads();
      if (*sfail) { failed = true; break; }
    }
    if (failed) break;
    fence_after();
    // Epilogue: thread (warp w, lane l) owns row 32w + l of the tile.
    const int row = ti * kTile + warp * 32 + lane;
    const bool row_ok = row < g.m;
    // alpha 2^(ea - 14 - 24): the slices' 2^-7 per operand and the 2^-24 unit of the joined sum
    const double ra = row_ok ? g.alpha * ldexp(1.0, g.ea[row] - 38) : 0.0;
    double* crow = g.C + (int64_t)(row_ok ? row : 0) * g.ldc;
    for (int c0 = 0; c0 < kTile; c0 += 16) {
      float a0[16], a1[16], a2[16], a3[16];
      const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      tmem_ld16(base, a0);
      tmem_ld16(base + kTile, a1);
      tmem_ld16(base + 2 * kTile, a2);
      tmem_ld16(base + 3 * kTile, a3);
      if (!row_ok) continue;
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int col = tj * kTile + c0 + q;
        if (col < g.n) {
          // levels 0, 1, 2 exact in units of 1, 2^-8, 2^-16; level 3 and up to 2^-24
          long long T = (long long)__float2int_rn(a0[q]);
          T = (T << 8) + __float2int_rn(a1[q] * 256.0f);
          T = (T << 8) + __float2int_rn(a2[q] * 65536.0f);
          T = (T << 8) + __float2int_rn(a3[q] * 16777216.0f);  // |T| < 2^47: exact in FP64
          double v = (double)T;
          const int ec = g.eb[col];
          const long long bits = __double_as_longlong(v);
          const int ne = (int)((bits >> 52) & 0x7FF) + ec;
          if (T == 0) v = 0.0;
          else if (ne > 0 && ne < 2047) v = __longlong_as_double(bits + ((long long)ec << 52));
          else v = ldexp(v, ec);
          crow[col] = fma(ra, v, crow[col]);
        }
      }
    }
    fence_before();
    __syncthreads();
    fence_after();
  }
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  if (tid == 0 && *sfail) atomicOr(g.flag, DEV_TIMEOUT);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2D map over a slice array [S * slab rows][kpad BF16], boxes of 128 rows x 64.
bool make_map(CUtensorMap* m, const void* base, int S, int slab, int kpad) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)S * (cuuint64_t)slab};
  cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
  cuuint32_t box[2] = {(cuuint32_t)kChunk, (cuuint32_t)kTile};
  cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int round_up(int x, int q) { return (x + q - 1) / q * q; }

}  // namespace

size_t oz_smem_bytes(int S) { return 1024 + 2 * (size_t)S * kSliceBytes + 64; }

size_t oz_work_bytes(int m, int n, int K, int S) {
  const int kpad = round_up(std::max(K, 1), kChunk);
  const size_t slab_a = (size_t)round_up(std::max(m, 1), kTile), slab_b = (size_t)round_up(std::max(n, 1), kTile);
  const size_t sl = (size_t)S * (slab_a + slab_b) * kpad * 2;
  return ((sl + 255) & ~size_t(255)) + 8 * (slab_a + slab_b) + 256;
}

cudaError_t oz_gemm(const OzGemm& p, cudaStream_t s) {
  if (p.m <= 0 || p.n <= 0 || p.K <= 0) return cudaSuccess;
  if (p.K > kOzMaxK || p.S < 1 || p.S > kOzMaxSlices) return cudaErrorInvalidValue;
  const int kpad = round_up(p.K, kChunk);
  const int slab_a = round_up(p.m, kTile), slab_b = round_up(p.n, kTile);
  uint8_t* w = static_cast<uint8_t*>(p.work);
  __nv_bfloat16* sla = reinterpret_cast<__nv_bfloat16*>(w);
  __nv_bfloat16* slb = sla + (size_t)p.S * slab_a * kpad;
  size_t sl_bytes = (size_t)p.S * ((size_t)slab_a + slab_b) * kpad * 2;
  sl_bytes = (sl_bytes + 255) & ~size_t(255);
  int* sca = reinterpret_cast<int*>(w + sl_bytes);
  int* scb = sca + slab_a;
  // Slices of both operands (one warp per row).
  {
    const int rows_a = slab_a, rows_b = slab_b;
    oz_split_kernel<<<(rows_a * 32 + 255) / 256, 256, 0, s>>>(p.A, p.lda, p.m, p.K, kpad, slab_a, p.S,
                                                             p.a_swap ? 1 : 0, sla, sca);
    oz_split_kernel<<<(rows_b * 32 + 255) / 256, 256, 0, s>>>(p.B, p.ldb, p.n, p.K, kpad, slab_b, p.S,
                                                             p.b_swap ? 1 : 0, slb, scb);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  CUtensorMap ma, mb;
  if (!make_map(&ma, sla, p.S, slab_a, kpad) || !make_map(&mb, slb, p.S, slab_b, kpad))
    return cudaErrorInvalidValue;
  OzArgs g{};
  g.C = p.C; g.ldc = p.ldc; g.m = p.m; g.n = p.n; g.kchunks = kpad / kChunk; g.S = p.S;
  g.slab_a = slab_a; g.slab_b = slab_b; g.alpha = p.alpha; g.ea = sca; g.eb = scb;
  g.tiles_n = slab_b / kTile;
  g.ntiles = (slab_a / kTile) * g.tiles_n;
  g.flag = p.flag;
  const size_t smem = oz_smem_bytes(p.S);
  cudaError_t e = cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn_smem());
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = std::min(g.ntiles, p.max_ctas > 0 ? p.max_ctas : sms);
  oz_gemm_kernel<<<grid, 128, smem, s>>>(ma, mb, g);
  return cudaGetLastError();
}

}  // namespace nrg
