// k_mixed.cu -- mixed-precision solve of the implicit system: FP64 iterative
// refinement around an FP32 block-Jacobi preconditioned CG.
//
// The system A dx = b is assembled in FP64 exactly as the reference does; its
// FP32 copy lives in warp slices (SELL-32: the 32 rows of a slice are a warp's
// lanes, block entries stored entry-major, so every value and column load is
// one coalesced 128-byte line).  Each refinement cycle solves A32 d = r32 to a
// relative residual eta in FP32 (FP32 arithmetic and accumulation), adds d to
// dx in FP64 and recomputes r = b - A dx with the FP64 matrix.  Cycles stop at
// the reference's criterion |r|^2 / |b|^2 < tol^2 (Solve_CG / Solve_PCG,
// matrix_square_sparse.cpp:338-406, ilu_sparse.cpp:628-709).
#include "kernels.h"

namespace cs {
namespace {

constexpr int kSliceThreads = 128;  // 4 slices (warps) per block
constexpr int kChunk = 256;         // rows per FP64 chunk (matches the CG chunks)

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum of one field of the per-slice partials of a cloth, by a whole warp in a fixed order
__device__ __forceinline__ double cloth_total(const Arena& A, int inst, int field) {
  double s = 0.0;
  for (int k = A.slice_lo[inst] + (threadIdx.x & 31); k < A.slice_hi[inst]; k += 32) s += A.part32[3 * k + field];
  return warp_sum_d(s);
}

// The last warp of a cloth to finish (ticket counter) sums the cloth's slice
// partials [f0, f0 + nf) in slice order into st.red: one pass, deterministic.
__device__ void finish_cloth(const Arena& A, int inst, int lane, int f0, int nf) {
  int last = 0;
  if (lane == 0) {
    __threadfence();
    const int n = A.slice_hi[inst] - A.slice_lo[inst];
    last = (atomicAdd(&A.red_cnt[inst], 1) == n - 1);
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return;
  __threadfence();
  for (int f = f0; f < f0 + nf; f++) {
    double s = 0.0;
    for (int k = A.slice_lo[inst] + lane; k < A.slice_hi[inst]; k += 32) s += __ldcg(&A.part32[3 * k + f]);
    s = warp_sum_d(s);
    if (lane == 0) A.st[inst].red[f] = s;
  }
  if (lane == 0) A.red_cnt[inst] = 0;
}

__device__ __forceinline__ void apply_dinv(const float* D, const float r[3], float z[3]) {
  z[0] = D[0] * r[0] + D[1] * r[1] + D[2] * r[2];
  z[1] = D[3] * r[0] + D[4] * r[1] + D[5] * r[2];
  z[2] = D[6] * r[0] + D[7] * r[1] + D[8] * r[2];
}

struct SliceCtx {
  int slice, lane, inst, row;
  bool valid;
};

// warp-uniform slice lookup; false when the slice's cloth sits this phase out
__device__ __forceinline__ bool slice_ctx(const Arena& A, SliceCtx& c, bool need_inner) {
  c.slice = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  c.lane = threadIdx.x & 31;
  if (c.slice >= A.nslice) return false;
  c.inst = A.slice_inst[c.slice];
  if (!A.active[c.inst] || A.st[c.inst].done) return false;
  if (need_inner && A.st[c.inst].idone) return false;
  c.row = A.slice_row0[c.slice] + c.lane;
  c.valid = c.row < A.voff[c.inst + 1];
  return true;
}

// r32 = r (FP64 residual), d = 0, z = D^-1 r, p = z; slice partials of r.z and r.r
__global__ void __launch_bounds__(kSliceThreads) k_mx_inner_init(Arena A) {
  SliceCtx c;
  if (!slice_ctx(A, c, false)) return;
  float rz = 0.f, rr = 0.f;
  if (c.valid) {
    float r[3], z[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      r[k] = (float)A.r[3 * c.row + k];
      A.r32[3 * c.row + k] = r[k];
      A.d32[3 * c.row + k] = 0.f;
    }
    apply_dinv(A.dinv32 + 9 * (size_t)c.row, r, z);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      A.z32[3 * c.row + k] = z[k];
      A.p32[3 * c.row + k] = z[k];
      rz += r[k] * z[k];
      rr += r[k] * r[k];
    }
  }
  rz = warp_sum_f(rz);
  rr = warp_sum_f(rr);
  if (c.lane == 0) {
    A.part32[3 * c.slice + 1] = rz;
    A.part32[3 * c.slice + 2] = rr;
  }
}

__global__ void k_mx_inner_start(Arena A) {
  const int inst = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (inst >= A.ni || !A.active[inst] || A.st[inst].done) return;
  const double rz = cloth_total(A, inst, 1), rr = cloth_total(A, inst, 2);
  if ((threadIdx.x & 31) == 0) {
    InstState& S = A.st[inst];
    S.rz[1] = rz;  // iteration 1 reads parity 1
    S.rr_in0 = rr;
    S.idone = (rr <= 0.0) ? 1 : 0;
    S.inner_iters = 0;
  }
}

// q = A32 p (one warp per slice, one lane per row); slice partial of p.q
__global__ void __launch_bounds__(kSliceThreads) k_mx_spmv(Arena A) {
  SliceCtx c;
  if (!slice_ctx(A, c, true)) return;
  const int w = A.slice_w[c.slice];
  const float* V = A.val32 + A.slice_voff[c.slice] + c.lane;
  const int* Cc = A.col32 + A.slice_coff[c.slice] + c.lane;
  float y0 = 0.f, y1 = 0.f, y2 = 0.f;
  for (int j = 0; j < w; j++) {
    const int col = Cc[32 * j];
    const float x0 = A.p32[3 * col + 0], x1 = A.p32[3 * col + 1], x2 = A.p32[3 * col + 2];
    const float* v = V + 288 * j;
    y0 = fmaf(v[0], x0, fmaf(v[32], x1, fmaf(v[64], x2, y0)));
    y1 = fmaf(v[96], x0, fmaf(v[128], x1, fmaf(v[160], x2, y1)));
    y2 = fmaf(v[192], x0, fmaf(v[224], x1, fmaf(v[256], x2, y2)));
  }
  float pq = 0.f;
  if (c.valid) {
    A.q32[3 * c.row + 0] = y0;
    A.q32[3 * c.row + 1] = y1;
    A.q32[3 * c.row + 2] = y2;
    pq = A.p32[3 * c.row + 0] * y0 + A.p32[3 * c.row + 1] * y1 + A.p32[3 * c.row + 2] * y2;
  }
  pq = warp_sum_f(pq);
  if (c.lane == 0) {
    A.part32[3 * c.slice + 0] = pq;
    if (A.count_bytes) atomicAdd(&A.bytes_acc[0], (unsigned long long)A.slice_bytes[c.slice]);
  }
  finish_cloth(A, c.inst, c.lane, 0, 1);
}

// alpha = r.z / p.q; d += alpha p; r -= alpha q; z = D^-1 r; partials of r.z, r.r
__global__ void __launch_bounds__(kSliceThreads) k_mx_update(Arena A, int it) {
  SliceCtx c;
  if (!slice_ctx(A, c, true)) return;
  const double pq = A.st[c.inst].red[0];
  const float alpha = (float)(A.st[c.inst].rz[it & 1] / pq);
  float rz = 0.f, rr = 0.f;
  if (c.valid) {
    float r[3], z[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int i = 3 * c.row + k;
      A.d32[i] = fmaf(alpha, A.p32[i], A.d32[i]);
      r[k] = fmaf(-alpha, A.q32[i], A.r32[i]);
      A.r32[i] = r[k];
    }
    apply_dinv(A.dinv32 + 9 * (size_t)c.row, r, z);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      A.z32[3 * c.row + k] = z[k];
      rz += r[k] * z[k];
      rr += r[k] * r[k];
    }
  }
  rz = warp_sum_f(rz);
  rr = warp_sum_f(rr);
  if (c.lane == 0) {
    A.part32[3 * c.slice + 1] = rz;
    A.part32[3 * c.slice + 2] = rr;
  }
  finish_cloth(A, c.inst, c.lane, 1, 2);
}

// inner convergence (|r|^2 <= eta^2 |r0|^2 or the cap), beta, p = z + beta p
__global__ void __launch_bounds__(kSliceThreads) k_mx_direction(Arena A, int it, float eta, int cap) {
  SliceCtx c;
  if (!slice_ctx(A, c, true)) return;
  InstState& S = A.st[c.inst];
  const double rzn = S.red[1], rrn = S.red[2];
  const bool first = (c.slice == A.slice_lo[c.inst]) && c.lane == 0;
  if (rrn <= (double)eta * (double)eta * S.rr_in0 || it >= cap) {
    if (first) {
      S.idone = 1;
      S.inner_iters = it;
    }
    return;
  }
  const float beta = (float)(rzn / S.rz[it & 1]);
  if (c.valid) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int i = 3 * c.row + k;
      A.p32[i] = fmaf(beta, A.p32[i], A.z32[i]);
    }
  }
  if (first) {
    S.rz[(it + 1) & 1] = rzn;
    S.inner_iters = it;
  }
}

// ---- FP64 outer refinement --------------------------------------------------------
__device__ __forceinline__ int chunk_row(const Arena& A, int c, int inst) {
  return A.voff[inst] + (c - A.chunk_lo[inst]) * kChunk + threadIdx.x;
}

__device__ double block_sum_d(double v, double* sh) {
  v = warp_sum_d(v);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    t = warp_sum_d(t);
  }
  return t;  // valid in thread 0
}

// dx = 0, r = b; chunk partials of b.b
__global__ void __launch_bounds__(kChunk) k_mx_outer_init(Arena A) {
  __shared__ double sh[33];
  const int c = blockIdx.x;
  const int inst = A.chunk_inst[c];
  if (!A.active[inst]) return;
  const int row = chunk_row(A, c, inst);
  double s = 0.0;
  if (row < A.voff[inst + 1]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double bk = A.b[3 * row + k];
      A.dx[3 * row + k] = 0.0;
      A.r[3 * row + k] = bk;
      s += bk * bk;
    }
  }
  s = block_sum_d(s, sh);
  if (threadIdx.x == 0) A.part[c] = s;
}

__global__ void k_mx_outer_start(Arena A) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= A.ni || !A.active[inst]) return;
  double s0 = 0.0;
  for (int c = A.chunk_lo[inst]; c < A.chunk_hi[inst]; c++) s0 += A.part[c];
  InstState& S = A.st[inst];
  S.cycles = 0;
  S.total_iters = 0;
  S.idone = 0;
  if (s0 < 1.0e-30) {
    S.done = 1;
    S.solver_conv = 0.0;
    S.solver_iterations = 0;
  } else {
    S.done = 0;
    S.inv0 = 1.0 / s0;
  }
}

// warm start: dx = dt v (the increment of the previous velocity); the stopping
// criterion stays relative to |b|, the reference's initial residual
__global__ void k_mx_warm(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * A.nv) return;
  const int inst = A.vinst[i / 3];
  if (!A.active[inst] || A.st[inst].done) return;
  A.dx[i] = A.bc[i / 3] ? 0.0 : A.prm[inst].dt * A.v[i];
}

// dx += d (FP64)
__global__ void k_mx_correct(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * A.nv) return;
  const int inst = A.vinst[i / 3];
  if (!A.active[inst] || A.st[inst].done) return;
  A.dx[i] += (double)A.d32[i];
}

// r = b - A dx with the FP64 matrix; chunk partials of r.r
__global__ void __launch_bounds__(kChunk) k_mx_residual(Arena A) {
  __shared__ double sh[33];
  const int c = blockIdx.x;
  const int inst = A.chunk_inst[c];
  if (!A.active[inst] || A.st[inst].done) return;
  const int i = chunk_row(A, c, inst);
  double s = 0.0;
  if (i < A.voff[inst + 1]) {
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
    const double* x = A.dx;
    for (int k = A.row_ptr[i]; k < A.row_ptr[i + 1]; k++) {
      const int j = A.col_idx[k];
      const double* a = A.vcrs + 9 * (size_t)k;
      const double x0 = x[3 * j + 0], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
      y0 += a[0] * x0 + a[1] * x1 + a[2] * x2;
      y1 += a[3] * x0 + a[4] * x1 + a[5] * x2;
      y2 += a[6] * x0 + a[7] * x1 + a[8] * x2;
    }
    const double* a = A.vdia + 9 * (size_t)i;
    const double x0 = x[3 * i + 0], x1 = x[3 * i + 1], x2 = x[3 * i + 2];
    y0 += a[0] * x0 + a[1] * x1 + a[2] * x2;
    y1 += a[3] * x0 + a[4] * x1 + a[5] * x2;
    y2 += a[6] * x0 + a[7] * x1 + a[8] * x2;
    const double r0 = A.b[3 * i + 0] - y0, r1 = A.b[3 * i + 1] - y1, r2 = A.b[3 * i + 2] - y2;
    A.r[3 * i + 0] = r0;
    A.r[3 * i + 1] = r1;
    A.r[3 * i + 2] = r2;
    s = r0 * r0 + r1 * r1 + r2 * r2;
  }
  s = block_sum_d(s, sh);
  if (threadIdx.x == 0) A.part[A.nchunk + c] = s;
}

// the reference's criterion on the FP64 residual; cycles capped at maxcycles
__global__ void k_mx_check(Arena A, double tol_in, int maxcycles) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= A.ni || !A.active[inst] || A.st[inst].done) return;
  const DevParams& P = A.prm[inst];
  const double tol = tol_in >= 0 ? tol_in : P.tol;
  double sq = 0.0;
  for (int c = A.chunk_lo[inst]; c < A.chunk_hi[inst]; c++) sq += A.part[A.nchunk + c];
  InstState& S = A.st[inst];
  S.total_iters += S.inner_iters;
  S.cycles += 1;
  S.solver_conv = sqrt(sq * S.inv0);
  S.solver_iterations = S.total_iters;
  // stop one decade below the reference's tolerance: the result then stays
  // within the reference's own truncation error of the exact solution
  if (sq * S.inv0 < 0.01 * tol * tol || S.cycles >= maxcycles) S.done = 1;
}

}  // namespace

void launch_mx_outer_init(const Arena& A, cudaStream_t s) {
  k_mx_outer_init<<<A.nchunk, kChunk, 0, s>>>(A);
  k_mx_outer_start<<<(A.ni + 127) / 128, 128, 0, s>>>(A);
  g_launches += 2;
}

void launch_mx_warm_start(const Arena& A, cudaStream_t s) {
  k_mx_warm<<<(3 * A.nv + 255) / 256, 256, 0, s>>>(A);
  prof_begin(PK_MX_RESIDUAL, s);
  k_mx_residual<<<A.nchunk, kChunk, 0, s>>>(A);
  prof_end(PK_MX_RESIDUAL, s);
  g_launches += 2;
}

void launch_mx_inner_init(const Arena& A, cudaStream_t s) {
  const int blocks = (A.nslice * 32 + kSliceThreads - 1) / kSliceThreads;
  k_mx_inner_init<<<blocks, kSliceThreads, 0, s>>>(A);
  k_mx_inner_start<<<(A.ni * 32 + 127) / 128, 128, 0, s>>>(A);
  g_launches += 2;
}

void launch_mx_inner_iteration(const Arena& A, int it, float eta, int cap, cudaStream_t s) {
  const int blocks = (A.nslice * 32 + kSliceThreads - 1) / kSliceThreads;
  prof_begin(PK_MX_SPMV, s);
  k_mx_spmv<<<blocks, kSliceThreads, 0, s>>>(A);
  prof_end(PK_MX_SPMV, s);
  prof_begin(PK_MX_UPDATE, s);
  k_mx_update<<<blocks, kSliceThreads, 0, s>>>(A, it);
  prof_end(PK_MX_UPDATE, s);
  prof_begin(PK_MX_DIRECTION, s);
  k_mx_direction<<<blocks, kSliceThreads, 0, s>>>(A, it, eta, cap);
  prof_end(PK_MX_DIRECTION, s);
  g_launches += 3;
}

void launch_mx_refine(const Arena& A, double tol, int maxcycles, cudaStream_t s) {
  k_mx_correct<<<(3 * A.nv + 255) / 256, 256, 0, s>>>(A);
  prof_begin(PK_MX_RESIDUAL, s);
  k_mx_residual<<<A.nchunk, kChunk, 0, s>>>(A);
  prof_end(PK_MX_RESIDUAL, s);
  k_mx_check<<<(A.ni + 127) / 128, 128, 0, s>>>(A, tol, maxcycles);
  g_launches += 3;
}

}  // namespace cs
