// Block diagonalization that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the point where they need a block
// diagonalized: an application that carves all device memory out once at
// start-up and forbids allocation afterwards, a host that runs the solve from
// a code path where an implicit device synchronisation (which cudaMalloc and
// cudaFree can cause) is not acceptable, or a plug-in whose memory is owned by
// a framework allocator.  nrg_diag_block_noalloc serves them: the caller passes
// device pointers for the input matrix and the outputs, and every scratch
// array of the eigensolver (the tridiagonalization workspace, the inverse-
// iteration factors, the launch tables and the error word) lives in one
// file-scope __device__ array of fixed size, held by every GPU that loads this
// file's module until the process exits.
//
// CUDA loads modules lazily by default: the module holding the array (and the
// eigensolver kernels') is loaded on a device at its first use there, which
// can allocate device memory and synchronise.  A caller that must never see
// that makes one warm-up call per device before it carves out its memory, or
// runs the process with CUDA_MODULE_LOADING=EAGER.
//
// The kernels are the ones nrg_diag_blocks runs (k_tridiag.cu, k_tdeig.cu);
// only the tables they read are generated on the device instead of uploaded.
#include <cuda_runtime.h>

#include "../../include/twochnrg_gb300.h"
#include "nrg_device.cuh"

namespace nrg {
namespace {

constexpr int kN = NRG_NOALLOC_MAX_N;
// doubles: A copy, Y, five LU arrays, d/e/tau/ev, FP32 copies of d and e
// (2 kN floats), e^2, the split flags (kN bytes), then an integer area
constexpr size_t kOffA = 0;
constexpr size_t kOffY = (size_t)kN * kN;
constexpr size_t kOffLU = 2 * (size_t)kN * kN;
constexpr size_t kOffVec = 7 * (size_t)kN * kN;
constexpr size_t kOffInt = kOffVec + 6 * (size_t)kN + (size_t)kN / 8 + 1;
constexpr size_t kIntWords = 16 + 8 * (size_t)kN;  // in 4-byte words
constexpr size_t kScratchDoubles = kOffInt + (kIntWords + 1) / 2 + 8;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct Layout {
  double *A, *Y, *LU, *d, *e, *tau, *ev;
  float* fde;
  double* e2;
  unsigned char* split;
  int *queue, *flag, *bsize, *soff, *order, *nvec;
  int64_t *hoff, *yoff;
  int *state_block, *vec_block, *vec_index, *cl_block, *cl_first, *cl_count, *cta_block, *cta_first;
};

Layout layout(double* base) {
  Layout L;
  L.A = base + kOffA; L.Y = base + kOffY; L.LU = base + kOffLU;
  L.d = base + kOffVec; L.e = L.d + kN; L.tau = L.e + kN; L.ev = L.tau + kN;
  L.fde = reinterpret_cast<float*>(L.ev + kN);
  L.e2 = L.ev + 2 * kN;
  L.split = reinterpret_cast<unsigned char*>(L.e2 + kN);
  int* ip = reinterpret_cast<int*>(base + kOffInt);
  L.queue = ip; L.flag = ip + 1; L.bsize = ip + 2; L.soff = ip + 3; L.order = ip + 4; L.nvec = ip + 5;
  L.hoff = reinterpret_cast<int64_t*>(ip + 8); L.yoff = L.hoff + 1;
  int* t = ip + 16;
  L.state_block = t; L.vec_block = t + kN; L.vec_index = t + 2 * kN; L.cl_block = t + 3 * kN;
  L.cl_first = t + 4 * kN; L.cl_count = t + 5 * kN; L.cta_block = t + 6 * kN; L.cta_first = t + 7 * kN;
  return L;
}

// Copies the input, writes the one-block tables and clears the words that
// must start at zero (the array keeps the previous call's contents).
__global__ void setup_kernel(Layout L, int n, const double* a, int bw) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = tid; i < n * n; i += gridDim.x * blockDim.x) L.A[i] = a[i];
  for (int i = tid; i < n; i += gridDim.x * blockDim.x) {
    L.state_block[i] = 0; L.vec_block[i] = 0; L.vec_index[i] = i;
    L.cta_block[i] = 0; L.cta_first[i] = i * bw;
  }
  if (tid == 0) {
    *L.queue = 0; *L.flag = 0; *L.bsize = n; *L.soff = 0; *L.order = 0; *L.nvec = n;
    *L.hoff = 0; *L.yoff = 0;
  }
}

// Clusters of close eigenvalues (gap below 1e-4 of the largest magnitude), as
// the host forms them for nrg_diag_blocks; unused entries get count 0.
__global__ void cluster_kernel(Layout L, int n) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double mx = 0.0;
  for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(L.ev[i]));
  const double ortol = 1e-4 * fmax(mx, 1e-300);
  int nc = 0, start = 0;
  for (int x = 1; x < n; ++x)
    if (L.ev[x] - L.ev[x - 1] > ortol) {
      L.cl_block[nc] = 0; L.cl_first[nc] = start; L.cl_count[nc] = x - start; ++nc; start = x;
    }
  L.cl_block[nc] = 0; L.cl_first[nc] = start; L.cl_count[nc] = n - start; ++nc;
  for (int c = nc; c < n; ++c) { L.cl_block[c] = 0; L.cl_first[c] = 0; L.cl_count[c] = 0; }
}

}  // namespace
}  // namespace nrg

extern "C" nrg_status nrg_diag_block_noalloc(int n, const double* a, double* eigvals, double* eigvecs,
                                             void* stream) {
  using namespace nrg;
  if (n < 1 || !a || !eigvals || !eigvecs) return NRG_ERR_ARG;
  if (n > NRG_NOALLOC_MAX_N) return NRG_ERR_SIZE;
  // The array's device address on the current device, looked up on every
  // call: a cached address would go stale if the module were reloaded (a
  // device reset, another context), and the lookup allocates nothing once
  // the module is loaded.
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return NRG_ERR_CUDA;
  double* base = static_cast<double*>(p);
  if (tridiag_max_clusters(8, n < 2 ? 2 : n) <= 0) return NRG_ERR_SIZE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const Layout L = layout(base);
  const int bw = backtransform_warps(n);
  setup_kernel<<<8, 256, 0, s>>>(L, n, a, bw);
  if (cudaGetLastError() != cudaSuccess) return NRG_ERR_CUDA;
  TridiagArgs ta{};
  ta.nblocks = 1; ta.order = L.order; ta.bsize = L.bsize; ta.hoff = L.hoff; ta.soff = L.soff;
  ta.H = L.A; ta.d = L.d; ta.e = L.e; ta.tau = L.tau; ta.queue = L.queue; ta.flag = L.flag;
  ta.maxn = n < 2 ? 2 : n;
  if (launch_tridiag(ta, 8, 1, s) != cudaSuccess) return NRG_ERR_CUDA;
  TdEigArgs ea{};
  ea.nblocks = 1; ea.bsize = L.bsize; ea.soff = L.soff; ea.d = L.d; ea.e = L.e; ea.ev = L.ev; ea.nstates = n;
  ea.flag = L.flag; ea.maxn = n; ea.fde = L.fde; ea.e2 = L.e2; ea.split = L.split;
  launch_bisect(ea, L.state_block, s);
  if (cudaGetLastError() != cudaSuccess) return NRG_ERR_CUDA;
  cluster_kernel<<<1, 32, 0, s>>>(L, n);
  if (cudaGetLastError() != cudaSuccess) return NRG_ERR_CUDA;
  InvIterArgs ia{};
  ia.nblocks = 1; ia.bsize = L.bsize; ia.soff = L.soff; ia.d = L.d; ia.e = L.e; ia.ev = L.ev; ia.nvec = L.nvec;
  ia.yoff = L.yoff; ia.Y = L.Y; ia.scratch = L.LU; ia.cl_block = L.cl_block; ia.cl_first = L.cl_first;
  ia.cl_count = L.cl_count; ia.nclusters = n; ia.flag = L.flag;
  launch_inviter(ia, L.vec_block, L.vec_index, n, s);
  if (cudaGetLastError() != cudaSuccess) return NRG_ERR_CUDA;
  BackArgs ba{};
  ba.bsize = L.bsize; ba.hoff = L.hoff; ba.H_const = L.A; ba.soff = L.soff; ba.tau = L.tau; ba.nvec = L.nvec;
  ba.yoff = L.yoff; ba.Y = L.Y; ba.Z = eigvecs; ba.Zt = nullptr; ba.zoff = L.yoff; ba.maxn = n;
  if (launch_backtransform(ba, L.cta_block, L.cta_first, (n + bw - 1) / bw, s) != cudaSuccess) return NRG_ERR_CUDA;
  if (cudaMemcpyAsync(eigvals, L.ev, sizeof(double) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return NRG_ERR_CUDA;
  int flag = 0;
  if (cudaMemcpyAsync(&flag, L.flag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return NRG_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return NRG_ERR_CUDA;
  if (flag & DEV_SIZE) return NRG_ERR_SIZE;
  if (flag & DEV_BAD_INPUT) return NRG_ERR_ARG;
  if (flag & DEV_NOT_CONVERGED) return NRG_ERR_NOT_CONVERGED;
  return NRG_OK;
}
