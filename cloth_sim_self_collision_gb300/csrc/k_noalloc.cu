// k_noalloc.cu -- Solve_CG for callers that cannot allocate device memory.
//
// Some callers of this library own every byte of device memory themselves: a
// physics or render engine with its own pool allocator, or a real-time frame
// loop that must never enter the CUDA allocator.  They cannot let the library
// call cudaMalloc for the Krylov work vectors.  cs_solve_cg_noalloc runs the
// reference's Solve_CG (matrix_square_sparse.cpp:338-406) on a 3x3 block
// matrix the caller passes in device memory, with its work vectors (r, p, Ap)
// and results in one file-scope device array of fixed size.  That array exists
// on every GPU that loads the library, for the life of the process.
//
// Limits and rules:
// * at most CS_NOALLOC_MAX_VERTICES block rows (larger systems are rejected
//   with CS_ERR_CAPACITY before anything runs);
// * the array's device address is looked up once per device, on the first
//   call made with that device current; make that first call before any stream
//   capture;
// * every call copies the convergence ratio and iteration count to the host
//   and waits for its stream before returning;
// * every call shares the one array, so calls that overlap on the GPU (on
//   different streams or devices' contexts racing on the same device) corrupt
//   each other: serialise them;
// * nothing carries over between calls: the kernel clears what must start at
//   zero (the solution and the product vector) on entry.
#include <mutex>

#include "../../include/clothgpu.h"

namespace {

constexpr int kMaxRows = CS_NOALLOC_MAX_VERTICES;
constexpr int kThreads = 1024;

struct NoAllocScratch {
  double r[3 * kMaxRows];
  double p[3 * kMaxRows];
  double ap[3 * kMaxRows];
  double conv;
  int iter;
  int pad;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

__device__ double cta_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

__device__ double cta_dot(const double* a, const double* b, int n, double* sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += a[i] * b[i];
  return cta_sum(s, sh);
}

// one CTA runs the whole solve (x = 0 start, the loop from 1 like the reference,
// the reported ratio from the previous residual)
__global__ void __launch_bounds__(kThreads) k_cg_noalloc(const int* row_ptr, const int* col_idx, const double* vcrs,
                                                          const double* vdia, const double* b, double* x, int np,
                                                          double tol, int maxit, NoAllocScratch* S) {
  __shared__ double sh[40];
  const int n = 3 * np;
  double *r = S->r, *p = S->p, *ap = S->ap;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    x[i] = 0.0;
    r[i] = b[i];
    p[i] = b[i];
    ap[i] = 0.0;
  }
  __syncthreads();
  double sq = cta_dot(r, r, n, sh);
  if (sq < 1.0e-30) {
    if (threadIdx.x == 0) {
      S->conv = 0.0;
      S->iter = 0;
    }
    return;
  }
  const double inv0 = 1.0 / sq;
  double conv = tol;
  int iter = maxit;
  for (int it = 1; it < maxit; it++) {
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      double y0 = ap[3 * i + 0] * 0.0, y1 = ap[3 * i + 1] * 0.0, y2 = ap[3 * i + 2] * 0.0;
      for (int s = row_ptr[i]; s < row_ptr[i + 1]; s++) {
        const int j = col_idx[s];
        const double* a = vcrs + 9 * (size_t)s;
        y0 += a[0] * p[3 * j] + a[1] * p[3 * j + 1] + a[2] * p[3 * j + 2];
        y1 += a[3] * p[3 * j] + a[4] * p[3 * j + 1] + a[5] * p[3 * j + 2];
        y2 += a[6] * p[3 * j] + a[7] * p[3 * j + 1] + a[8] * p[3 * j + 2];
      }
      const double* a = vdia + 9 * (size_t)i;
      y0 += a[0] * p[3 * i] + a[1] * p[3 * i + 1] + a[2] * p[3 * i + 2];
      y1 += a[3] * p[3 * i] + a[4] * p[3 * i + 1] + a[5] * p[3 * i + 2];
      y2 += a[6] * p[3 * i] + a[7] * p[3 * i + 1] + a[8] * p[3 * i + 2];
      ap[3 * i + 0] = y0;
      ap[3 * i + 1] = y1;
      ap[3 * i + 2] = y2;
    }
    __syncthreads();
    const double alpha = sq / cta_dot(p, ap, n, sh);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      x[i] += alpha * p[i];
      r[i] += (-alpha) * ap[i];
    }
    __syncthreads();
    const double sqn = cta_dot(r, r, n, sh);
    if (sqn * inv0 < tol * tol) {
      conv = sqrt(sq * inv0);
      iter = it;
      break;
    }
    const double beta = sqn / sq;
    sq = sqn;
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = r[i] + beta * p[i];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    S->conv = conv;
    S->iter = iter;
  }
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
NoAllocScratch* g_addr[kMaxDevices] = {};

}  // namespace

extern "C" int cs_solve_cg_noalloc(const int* row_ptr, const int* col_idx, const double* vcrs, const double* vdia,
                                   const double* b, double* x, int np, double tol, int maxit, double* conv,
                                   int* iter, void* stream) {
  if (!row_ptr || !col_idx || !vcrs || !vdia || !b || !x || np <= 0 || maxit < 0) return CS_ERR_ARG;
  if (np > kMaxRows) return CS_ERR_CAPACITY;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CS_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return CS_ERR_ARG;
  NoAllocScratch* S = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
      // the host-side name of the array is not a device address: look it up
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return CS_ERR_CUDA;
      g_addr[dev] = (NoAllocScratch*)p;
    }
    S = g_addr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  k_cg_noalloc<<<1, kThreads, 0, s>>>(row_ptr, col_idx, vcrs, vdia, b, x, np, tol, maxit, S);
  if (cudaGetLastError() != cudaSuccess) return CS_ERR_CUDA;
  double c = 0.0;
  int it = 0;
  if (cudaMemcpyAsync(&c, &S->conv, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&it, &S->iter, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return CS_ERR_CUDA;
  if (conv) *conv = c;
  if (iter) *iter = it;
  return CS_OK;
}
