// k_mixed.cu -- mixed-precision solve of the implicit system: FP64 iterative
// refinement around an FP32 CG (block-Jacobi or unpreconditioned, per cloth).
//
// The system A dx = b is assembled in FP64 exactly as the reference does; its
// FP32 copy lives in warp slices (SELL-32: the 32 rows of a slice are a warp's
// lanes, block entries stored entry-major, so every value and column load is
// one coalesced 128-byte line).  Each refinement cycle solves A32 d = r32 to a
// relative residual eta in FP32 (FP32 arithmetic and accumulation), adds d to
// dx in FP64 and recomputes r = b - A dx with the FP64 matrix.  Cycles stop at
// a decade below the reference's criterion |r|^2 / |b|^2 < tol^2 (Solve_CG /
// Solve_PCG, matrix_square_sparse.cpp:338-406, ilu_sparse.cpp:628-709).
#include <algorithm>

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

// Preconditioner choice per cloth and frame: block-Jacobi when the diagonal's
// entries spread by more than kJacobiSpread (obstacle contact terms), else none
// (CG as the reference's Solve_CG).  Without contact the right-hand side of a
// falling sheet is close to a rigid translation, an eigenvector of M/dt^2 + K,
// which unpreconditioned CG resolves in a few iterations and the boundary-varying
// Jacobi scaling does not; with contact terms block-Jacobi converges faster.
// Block-Jacobi is applied as a symmetric scaling: with D_i = L_i L_i^T (Cholesky
// of the diagonal block) and S = blockdiag(L_i^-1), CG on S A S^T y = S r,
// d = S^T y is block-Jacobi PCG, and the inner loop carries no preconditioner.
constexpr float kJacobiSpread = 10.0f;

// y = L^-1 x, with L^-1 lower triangular (row-major 3x3)
__device__ __forceinline__ void apply_l(const float* S, const float x[3], float y[3]) {
  y[0] = S[0] * x[0];
  y[1] = S[3] * x[0] + S[4] * x[1];
  y[2] = S[6] * x[0] + S[7] * x[1] + S[8] * x[2];
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

// FP32 matrix of the cloths that use block-Jacobi: each block A_ij becomes
// L_i^-1 A_ij L_j^-T (once per frame, after the preconditioner choice)
__global__ void __launch_bounds__(kSliceThreads) k_mx_scale(Arena A) {
  SliceCtx c;
  if (!slice_ctx(A, c, false) || !A.st[c.inst].bjac || !c.valid) return;
  const int w = A.slice_w[c.slice];
  float* V = A.val32 + A.slice_voff[c.slice] + c.lane;
  const int* Cc = A.col32 + A.slice_coff[c.slice] + c.lane;
  float Si[9];
#pragma unroll
  for (int k = 0; k < 9; k++) Si[k] = A.linv32[9 * (size_t)c.row + k];
  for (int j = 0; j < w; j++) {
    const int col = Cc[32 * j];
    float Sj[9], B[9], T[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
      Sj[k] = A.linv32[9 * (size_t)col + k];
      B[k] = V[288 * j + 32 * k];
    }
    // T = B L_j^-T: T[a][b] = sum_c B[a][c] Sj[b][c]
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) T[3 * a + b] = B[3 * a + 0] * Sj[3 * b + 0] + B[3 * a + 1] * Sj[3 * b + 1] +
                                                 B[3 * a + 2] * Sj[3 * b + 2];
    // L_i^-1 T
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++)
        V[288 * j + 32 * (3 * a + b)] = Si[3 * a + 0] * T[b] + Si[3 * a + 1] * T[3 + b] + Si[3 * a + 2] * T[6 + b];
  }
}

// r32 = S r (scaled cloths) or r, from the FP64 residual; d = 0, z = p = r32;
// slice partials of r.r (fields 1 and 2: r.z equals r.r without a preconditioner)
// The FP32 vectors of the inner solve (r, w, s, p, d, z, q) keep a vertex's
// x, y, z and a pad in 16 bytes: one aligned load or store per vertex.
constexpr int kV = 4;
__device__ __forceinline__ float4 ld_v4(const float* a, int v) {
  return *reinterpret_cast<const float4*>(a + kV * (size_t)v);
}
__device__ __forceinline__ void st_v4(float* a, int v, const float x[3]) {
  *reinterpret_cast<float4*>(a + kV * (size_t)v) = make_float4(x[0], x[1], x[2], 0.f);
}

__global__ void __launch_bounds__(kSliceThreads) k_mx_inner_init(Arena A) {
  SliceCtx c;
  if (!slice_ctx(A, c, false)) return;
  float rr = 0.f;
  if (c.valid) {
    float r[3];
    if (A.st[c.inst].bjac) {
      const float* S = A.linv32 + 9 * (size_t)c.row;
      const double r0 = A.r[3 * c.row], r1 = A.r[3 * c.row + 1], r2 = A.r[3 * c.row + 2];
      r[0] = (float)((double)S[0] * r0);
      r[1] = (float)((double)S[3] * r0 + (double)S[4] * r1);
      r[2] = (float)((double)S[6] * r0 + (double)S[7] * r1 + (double)S[8] * r2);
    } else {
#pragma unroll
      for (int k = 0; k < 3; k++) r[k] = (float)A.r[3 * c.row + k];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      A.r32[kV * c.row + k] = r[k];
      A.d32[kV * c.row + k] = 0.f;
      A.z32[kV * c.row + k] = r[k];
      A.p32[kV * c.row + k] = r[k];
      rr += r[k] * r[k];
    }
  }
  rr = warp_sum_f(rr);
  if (c.lane == 0) {
    A.part32[3 * c.slice + 1] = rr;
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
    const float x0 = A.p32[kV * col + 0], x1 = A.p32[kV * col + 1], x2 = A.p32[kV * col + 2];
    const float* v = V + 288 * j;
    y0 = fmaf(v[0], x0, fmaf(v[32], x1, fmaf(v[64], x2, y0)));
    y1 = fmaf(v[96], x0, fmaf(v[128], x1, fmaf(v[160], x2, y1)));
    y2 = fmaf(v[192], x0, fmaf(v[224], x1, fmaf(v[256], x2, y2)));
  }
  float pq = 0.f;
  if (c.valid) {
    A.q32[kV * c.row + 0] = y0;
    A.q32[kV * c.row + 1] = y1;
    A.q32[kV * c.row + 2] = y2;
    pq = A.p32[kV * c.row + 0] * y0 + A.p32[kV * c.row + 1] * y1 + A.p32[kV * c.row + 2] * y2;
  }
  pq = warp_sum_f(pq);
  if (c.lane == 0) {
    A.part32[3 * c.slice + 0] = pq;
    if (A.count_bytes) atomicAdd(&A.bytes_acc[0], (unsigned long long)A.slice_bytes[c.slice]);
  }
  finish_cloth(A, c.inst, c.lane, 0, 1);
}

// alpha = r.z / p.q; d += alpha p; r -= alpha q; z = r; partials of r.z, r.r
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
      const int i = kV * c.row + k;
      A.d32[i] = fmaf(alpha, A.p32[i], A.d32[i]);
      r[k] = fmaf(-alpha, A.q32[i], A.r32[i]);
      A.r32[i] = r[k];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      z[k] = r[k];
      A.z32[kV * c.row + k] = z[k];
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

// The inner tolerance of cloth inst: eta, or eta_big for cloths of more than
// kBigClothRows rows.  A large stiff sheet needs many inner iterations per
// refinement cycle, and each cycle restarts its Krylov space: measured on the
// serving scenes (up to 1e5 vertices), 1e-4 there raised the throughput by
// 14 %, while on the batch of sheets up to 6561 vertices 1e-4 everywhere was
// 1 % slower than 1e-3.  The choice depends only on the cloth itself.
constexpr int kBigClothRows = 16384;
__device__ __forceinline__ float inner_eta(const Arena& A, int inst, float eta) {
  return A.voff[inst + 1] - A.voff[inst] > kBigClothRows ? fminf(eta, A.mx_eta_big) : eta;
}

// inner convergence (|r|^2 <= eta^2 |r0|^2 or the cap), beta, p = z + beta p
__global__ void __launch_bounds__(kSliceThreads) k_mx_direction(Arena A, int it, float eta, int cap) {
  SliceCtx c;
  if (!slice_ctx(A, c, true)) return;
  InstState& S = A.st[c.inst];
  const double rzn = S.red[1], rrn = S.red[2];
  const bool first = (c.slice == A.slice_lo[c.inst]) && c.lane == 0;
  const double e = inner_eta(A, c.inst, eta);
  if (rrn <= e * e * S.rr_in0 || it >= cap) {
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
      const int i = kV * c.row + k;
      A.p32[i] = fmaf(beta, A.p32[i], A.z32[i]);
    }
  }
  if (first) {
    S.rz[(it + 1) & 1] = rzn;
    S.inner_iters = it;
  }
}

// ---- persistent inner solve ---------------------------------------------------------
// One cooperative launch runs every inner CG iteration of a refinement cycle for
// all cloths, in the single-reduction form of CG (Chronopoulos and Gear, 1989:
// "s-step iterative methods for symmetric linear systems", J. Comput. Appl.
// Math. 25): with w = A r and s = A p carried by recurrence, both inner
// products of an iteration are taken together, so an iteration is one phase
// and one grid barrier.  Iteration i (alpha_i, beta_i from the previous one):
//   s_i = w_i + beta_i s_{i-1},  p_i = r_i + beta_i p_{i-1},  d += alpha_i p_i,
//   r_{i+1} = r_i - alpha_i s_i,  w_{i+1} = A r_{i+1},
//   gamma_{i+1} = r_{i+1}.r_{i+1},  delta_{i+1} = w_{i+1}.r_{i+1},
//   beta_{i+1} = gamma_{i+1} / gamma_i,
//   alpha_{i+1} = gamma_{i+1} / (delta_{i+1} - beta_{i+1} gamma_{i+1} / alpha_i).
// The SpMV needs r_{i+1} at the neighbour rows, which other blocks update in the
// same phase: it recomputes them from r_i, w_i and s_{i-1} with the same fused
// operations the owning row uses, so both agree bit for bit.  r, w and s are
// double-buffered by parity; p and d are read only by their own row.
// Block-Jacobi cloths run on the scaled matrix, so no preconditioner appears.
// Totals: the block whose slices complete a cloth (a per-cloth ticket counted in
// slices) sums the cloth's partials in slice order with a block of fixed size,
// so results depend neither on the launch shape nor on the other cloths; it
// decides convergence (|r|^2 <= eta^2 |r0|^2, or the cap) or stores alpha and
// beta.  A converged cloth sets istop and decrements the count of cloths still
// iterating; all blocks read that count after the barrier that ends the
// iteration, so they leave the loop together.
// Work split: the slices of the cloths still iterating, in arena order, are cut
// into one contiguous range per block, re-cut whenever a cloth stops, so blocks
// do not idle on converged cloths (arenas of more than kRebalanceMax cloths
// keep the static cut over all slices and skip converged cloths).
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
constexpr int kRebalanceMax = 2048;        // cloths whose slice prefix fits in shared memory

// Grid-wide barrier on A.grid_bar with a bounded wait.  Returns false when the
// wait ran out here or in another block (the flag A.grid_bar[2] is then set and
// every block leaves the kernel at its next barrier).
__device__ bool grid_sync(const Arena& A) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* bar = A.grid_bar;
    __threadfence();
    const unsigned gen = bar[1];
    // with the test hook set, block 0 does not arrive and every wait runs out
    const bool hold = A.bar_hold != 0 && blockIdx.x == 0;
    if (!hold && atomicAdd(&A.grid_bar[0], 1u) == gridDim.x - 1) {
      atomicExch(&A.grid_bar[0], 0u);
      __threadfence();
      atomicAdd(&A.grid_bar[1], 1u);
    } else {
      // poll with a pause of A.bar_sleep_ns between reads; give up (flag the
      // error for every block) after A.bar_timeout_ns of the device's clock
      const unsigned long long t0 = global_ns();
      const unsigned long long limit = (unsigned long long)A.bar_timeout_ns;
      const unsigned ns = (unsigned)A.bar_sleep_ns;
      while (bar[1] == gen && bar[2] == 0u) {
        if (global_ns() - t0 > limit) {
          atomicExch(&A.grid_bar[2], 1u);
          break;
        }
        if (ns) __nanosleep(ns);
      }
    }
    __threadfence();
    s_ok = bar[2] == 0u;
  }
  __syncthreads();
  return s_ok != 0;
}

// Totals over the slices of cloth inst of nf partial fields starting at f0, as
// fixed-order block sums (every thread gets them in tot[]).
template <int kPersistThreads>
__device__ void cloth_totals(const Arena& A, int inst, int f0, int nf, double* sh, double* tot) {
  constexpr int kPersistWarps = kPersistThreads / 32;
  const int lo = A.slice_lo[inst], hi = A.slice_hi[inst];
  for (int f = 0; f < nf; f++) {
    double v = 0.0;
    for (int k = lo + threadIdx.x; k < hi; k += kPersistThreads) v += __ldcg(&A.part32[3 * k + f0 + f]);
    v = warp_sum_d(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kPersistWarps; w++) t += sh[w];
    tot[f] = t;
  }
}

// After a block's n slices of cloth inst have written their partials: true in
// the block whose slices complete the cloth (it then resets the ticket).
__device__ bool last_portion(const Arena& A, int inst, int n, int* s_flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const int total = A.slice_hi[inst] - A.slice_lo[inst];
    const int old = atomicAdd(&A.red_cnt[inst], n);
    const int last = old + n == total;
    if (last) {
      A.red_cnt[inst] = 0;
      __threadfence();
    }
    *s_flag = last;
  }
  __syncthreads();
  return *s_flag != 0;
}

__device__ __forceinline__ bool iterating(const Arena& A, int inst) {
  return A.active[inst] && !A.st[inst].done && !A.st[inst].istop;
}

// This block's share of the slices of the cloths still iterating: cloths
// [c0, c1], clipped to [a0, a1) in the prefix s_pref (compact cut) or to the
// slices [a0, a1) themselves (static cut).
struct PersistRange {
  int a0, a1, c0, c1;
};

template <int kPersistThreads>
__device__ void compact_range(const Arena& A, int* s_pref, int* s_wsum, PersistRange& R) {
  constexpr int kPersistWarps = kPersistThreads / 32;
  const int ni = A.ni;
  const int per = (ni + kPersistThreads - 1) / kPersistThreads;
  const int b0 = min(ni, threadIdx.x * per), b1 = min(ni, b0 + per);
  int sum = 0;
  for (int c = b0; c < b1; c++) sum += iterating(A, c) ? A.slice_hi[c] - A.slice_lo[c] : 0;
  // exclusive block scan of the thread sums
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  __syncthreads();
  if (lane == 31) s_wsum[warp] = inc;
  __syncthreads();
  int off = inc - sum;
  for (int w = 0; w < warp; w++) off += s_wsum[w];
  for (int c = b0; c < b1; c++) {
    s_pref[c] = off;
    off += iterating(A, c) ? A.slice_hi[c] - A.slice_lo[c] : 0;
  }
  if (threadIdx.x == kPersistThreads - 1) s_pref[ni] = off;
  __syncthreads();
  (void)kPersistWarps;
  const long long total = s_pref[ni];
  R.a0 = (int)(total * blockIdx.x / gridDim.x);
  R.a1 = (int)(total * (blockIdx.x + 1) / gridDim.x);
  // the largest c with s_pref[c] <= x
  auto find = [&](int x) {
    int lo = 0, hi = ni - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_pref[mid] <= x) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  };
  if (R.a0 < R.a1) {
    R.c0 = find(R.a0);
    R.c1 = find(R.a1 - 1);
  } else {
    R.c0 = 0;
    R.c1 = -1;
  }
}

// slices [lo, hi) of cloth inst in this block's range; false when empty
__device__ __forceinline__ bool portion(const Arena& A, const PersistRange& R, bool compact, const int* s_pref,
                                        int inst, int& lo, int& hi) {
  if (compact) {
    const int p0 = s_pref[inst];
    lo = A.slice_lo[inst] + (max(R.a0, p0) - p0);
    hi = A.slice_lo[inst] + (min(R.a1, s_pref[inst + 1]) - p0);
  } else {
    if (!iterating(A, inst)) return false;
    lo = max(R.a0, A.slice_lo[inst]);
    hi = min(R.a1, A.slice_hi[inst]);
  }
  return lo < hi;
}

// kMinBlocks: the blocks per SM the build keeps room for (256 threads and 6
// blocks: 40 registers a thread, a few spills; 4 blocks: 64 registers, none);
// the launch picks the build for the blocks per SM it runs
template <int kPersistThreads, int kMinBlocks = 1536 / kPersistThreads>
__global__ void __launch_bounds__(kPersistThreads, kMinBlocks)
    k_mx_persist(Arena A, float eta, int cap, int exit_slices, int resume) {
  constexpr int kPersistWarps = kPersistThreads / 32;
  __shared__ double sh[kPersistWarps];
  __shared__ int s_wsum[kPersistWarps];
  __shared__ int s_flag, s_left;
  __shared__ int s_pref[kRebalanceMax + 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool compact = A.ni <= kRebalanceMax;
  PersistRange R;
  {
    const long long S = A.nslice;
    R.a0 = (int)(S * blockIdx.x / gridDim.x);
    R.a1 = (int)(S * (blockIdx.x + 1) / gridDim.x);
    R.c0 = R.a0 < R.a1 ? A.slice_inst[R.a0] : 0;
    R.c1 = R.a0 < R.a1 ? A.slice_inst[R.a1 - 1] : -1;
  }
  if (threadIdx.x == 0) s_left = ((volatile unsigned*)A.grid_bar)[3];
  __syncthreads();
  unsigned cut_at = 0xffffffffu;  // cloths iterating when the range was cut
  // a resumed launch continues after the last iteration the first one ran
  const int it0 = resume ? (int)((volatile unsigned*)A.grid_bar)[4] + 1 : 1;
  for (int it = it0; it <= cap; it++) {
    const unsigned left = (unsigned)s_left;
    if (left == 0u) break;
    if (compact && left != cut_at) {
      compact_range<kPersistThreads>(A, s_pref, s_wsum, R);
      cut_at = left;
    }
    // fewer slices left than exit_slices: every block leaves here (they all
    // read the same cut), and a launch with fewer blocks, whose grid barriers
    // cost less, resumes at this iteration
    if (exit_slices > 0 && compact && s_pref[A.ni] < exit_slices) {
      if (blockIdx.x == 0 && threadIdx.x == 0) A.grid_bar[4] = (unsigned)(it - 1);
      break;
    }
    // iteration 1 reads r_1, w_1 from r32, w32 (the start kernels) and no s, p
    const bool odd = (it & 1) != 0;
    const float* Rc = odd ? A.r32 : A.r32b;
    const float* Wc = odd ? A.w32 : A.w32b;
    const float* Sp = odd ? A.s32b : A.s32;
    float* Rn = odd ? A.r32b : A.r32;
    float* Wn = odd ? A.w32b : A.w32;
    float* Sn = odd ? A.s32 : A.s32b;
    const bool first = it == 1;
    for (int inst = R.c0; inst <= R.c1; inst++) {
      int lo, hi;
      if (!portion(A, R, compact, s_pref, inst, lo, hi)) continue;
      const InstState& St = A.st[inst];
      const float alpha = St.alpha32;
      const float beta = first ? 0.f : St.beta32;
      for (int sl = lo + warp; sl < hi; sl += kPersistWarps) {
        const int row = A.slice_row0[sl] + lane;
        const int w = A.slice_w[sl];
        const float* V = A.val32 + A.slice_voff[sl] + lane;
        const int* Cc = A.col32 + A.slice_coff[sl] + lane;
        float y0 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll 2
        for (int j = 0; j < w; j++) {
          // the matrix streams (read once per iteration, evict first), so that
          // the gathered vectors keep their place in L2
          const int col = __ldcs(Cc + 32 * j);
          // r, w and s of the neighbour, one 16-byte load each
          const float4 rc = ld_v4(Rc, col), wc = ld_v4(Wc, col);
          const float4 sp = first ? make_float4(0.f, 0.f, 0.f, 0.f) : ld_v4(Sp, col);
          const float sk[3] = {first ? wc.x : fmaf(beta, sp.x, wc.x), first ? wc.y : fmaf(beta, sp.y, wc.y),
                               first ? wc.z : fmaf(beta, sp.z, wc.z)};
          const float x[3] = {fmaf(-alpha, sk[0], rc.x), fmaf(-alpha, sk[1], rc.y), fmaf(-alpha, sk[2], rc.z)};
          const float* v = V + 288 * j;
          y0 = fmaf(__ldcs(v), x[0], fmaf(__ldcs(v + 32), x[1], fmaf(__ldcs(v + 64), x[2], y0)));
          y1 = fmaf(__ldcs(v + 96), x[0], fmaf(__ldcs(v + 128), x[1], fmaf(__ldcs(v + 160), x[2], y1)));
          y2 = fmaf(__ldcs(v + 192), x[0], fmaf(__ldcs(v + 224), x[1], fmaf(__ldcs(v + 256), x[2], y2)));
        }
        float gam = 0.f, del = 0.f;
        if (row < A.voff[inst + 1]) {
          const float y[3] = {y0, y1, y2};
          const float4 rc = ld_v4(Rc, row), wc = ld_v4(Wc, row);
          const float4 sp = first ? make_float4(0.f, 0.f, 0.f, 0.f) : ld_v4(Sp, row);
          const float4 pp = first ? make_float4(0.f, 0.f, 0.f, 0.f) : ld_v4(A.p32, row);
          const float4 dd = ld_v4(A.d32, row);
          const float R_[3] = {rc.x, rc.y, rc.z}, W_[3] = {wc.x, wc.y, wc.z}, S_[3] = {sp.x, sp.y, sp.z};
          const float P_[3] = {pp.x, pp.y, pp.z}, D_[3] = {dd.x, dd.y, dd.z};
          float sn[3], pn[3], dn[3], rn[3];
#pragma unroll
          for (int k = 0; k < 3; k++) {
            sn[k] = first ? W_[k] : fmaf(beta, S_[k], W_[k]);
            pn[k] = first ? R_[k] : fmaf(beta, P_[k], R_[k]);
            rn[k] = fmaf(-alpha, sn[k], R_[k]);
            dn[k] = fmaf(alpha, pn[k], D_[k]);
            gam += rn[k] * rn[k];
            del += y[k] * rn[k];
          }
          st_v4(Sn, row, sn);
          st_v4(A.p32, row, pn);
          st_v4(A.d32, row, dn);
          st_v4(Rn, row, rn);
          st_v4(Wn, row, y);
        }
        gam = warp_sum_f(gam);
        del = warp_sum_f(del);
        if (lane == 0) {
          A.part32[3 * sl + 0] = gam;
          A.part32[3 * sl + 1] = del;
          if (A.count_bytes) atomicAdd(&A.bytes_acc[6], (unsigned long long)A.slice_pbytes[sl]);
        }
      }
      if (last_portion(A, inst, hi - lo, &s_flag)) {
        double tot[2];
        cloth_totals<kPersistThreads>(A, inst, 0, 2, sh, tot);
        if (threadIdx.x == 0) {
          InstState& Sw = A.st[inst];
          Sw.inner_iters = it;
          const double gam = tot[0], del = tot[1];
          const double beta_n = gam / Sw.gam;
          const double den = del - beta_n * gam / Sw.alf;
          const double e = inner_eta(A, inst, eta);
          if (gam <= e * e * Sw.rr_in0 || it >= cap || !(den > 0.0)) {
            Sw.istop = 1;
            Sw.idone = 1;
            Sw.red[2] = gam;
            atomicSub(&A.grid_bar[3], 1u);
          } else {
            Sw.alf = gam / den;
            Sw.gam = gam;
            Sw.alpha32 = (float)Sw.alf;
            Sw.beta32 = (float)beta_n;
          }
        }
      }
    }
    if (!grid_sync(A)) return;
    if (threadIdx.x == 0) s_left = ((volatile unsigned*)A.grid_bar)[3];
    __syncthreads();
  }
}

// start of the persistent inner solve: w_1 = A r_1 over the slices (r_1 = r32
// from k_mx_inner_init), with the slice partials of gamma = r.r and delta = w.r
__global__ void __launch_bounds__(kSliceThreads) k_mx_pw0(Arena A) {
  SliceCtx c;
  if (!slice_ctx(A, c, false)) return;
  const int w = A.slice_w[c.slice];
  const float* V = A.val32 + A.slice_voff[c.slice] + c.lane;
  const int* Cc = A.col32 + A.slice_coff[c.slice] + c.lane;
  float y0 = 0.f, y1 = 0.f, y2 = 0.f;
  for (int j = 0; j < w; j++) {
    const int col = Cc[32 * j];
    const float x0 = A.r32[kV * col + 0], x1 = A.r32[kV * col + 1], x2 = A.r32[kV * col + 2];
    const float* v = V + 288 * j;
    y0 = fmaf(v[0], x0, fmaf(v[32], x1, fmaf(v[64], x2, y0)));
    y1 = fmaf(v[96], x0, fmaf(v[128], x1, fmaf(v[160], x2, y1)));
    y2 = fmaf(v[192], x0, fmaf(v[224], x1, fmaf(v[256], x2, y2)));
  }
  float gam = 0.f, del = 0.f;
  if (c.valid) {
    const float y[3] = {y0, y1, y2};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float r = A.r32[kV * c.row + k];
      A.w32[kV * c.row + k] = y[k];
      gam += r * r;
      del += y[k] * r;
    }
  }
  gam = warp_sum_f(gam);
  del = warp_sum_f(del);
  if (c.lane == 0) {
    A.part32[3 * c.slice + 0] = gam;
    A.part32[3 * c.slice + 1] = del;
    if (A.count_bytes) atomicAdd(&A.bytes_acc[0], (unsigned long long)A.slice_bytes[c.slice]);
  }
}

// per-cloth totals of the start: gamma_1, alpha_1 = gamma_1 / delta_1, and the
// count of cloths that iterate
__global__ void k_mx_pstart(Arena A) {
  const int inst = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (inst >= A.ni || !A.active[inst] || A.st[inst].done) return;
  const double gam = cloth_total(A, inst, 0), del = cloth_total(A, inst, 1);
  if ((threadIdx.x & 31) == 0) {
    InstState& S = A.st[inst];
    S.rr_in0 = gam;
    S.gam = gam;
    S.alf = del > 0.0 ? gam / del : 0.0;
    S.alpha32 = (float)S.alf;
    S.beta32 = 0.f;
    S.idone = (gam <= 0.0 || !(del > 0.0)) ? 1 : 0;
    S.istop = S.idone;
    S.inner_iters = 0;
    if (!S.idone) atomicAdd(&A.grid_bar[3], 1u);
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
  {
    const float lo = __uint_as_float(A.dg_range[2 * inst]), hi = __uint_as_float(A.dg_range[2 * inst + 1]);
    S.bjac = hi > kJacobiSpread * lo;
  }
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

// dx += S^T d (scaled cloths) or d, in FP64
__global__ void k_mx_correct(Arena A) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  const int inst = A.vinst[v];
  if (!A.active[inst] || A.st[inst].done) return;
  const double d0 = A.d32[kV * v], d1 = A.d32[kV * v + 1], d2 = A.d32[kV * v + 2];
  if (A.st[inst].bjac) {
    const float* S = A.linv32 + 9 * (size_t)v;
    A.dx[3 * v + 0] += (double)S[0] * d0 + (double)S[3] * d1 + (double)S[6] * d2;
    A.dx[3 * v + 1] += (double)S[4] * d1 + (double)S[7] * d2;
    A.dx[3 * v + 2] += (double)S[8] * d2;
  } else {
    A.dx[3 * v + 0] += d0;
    A.dx[3 * v + 1] += d1;
    A.dx[3 * v + 2] += d2;
  }
}

// r = b - A dx with the FP64 matrix, one thread per row; chunk partials of r.r.
// GB300 issues FP64 at 2 lanes per clock per SM, so this product is bound by
// the FP64 pipe, not by HBM: the row's in-order sum must stay on one lane (a
// row split over lanes pays the sequential adds on every lane of the group).
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
  k_mx_scale<<<(A.nslice * 32 + kSliceThreads - 1) / kSliceThreads, kSliceThreads, 0, s>>>(A);
  g_launches += 3;
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

template <int T>
static void persist_launch(const Arena& A, float eta, int cap, int blocks_per_sm, int tail_slices, cudaStream_t s) {
  int dev = 0, sms = 0, occ = 0;
  launch_check(cudaGetDevice(&dev), "cudaGetDevice");
  launch_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
  // at 4 blocks of 256 threads per SM or fewer, the build with 64 registers
  const void* kern = (const void*)k_mx_persist<T>;
  if constexpr (T == 256) {
    if (blocks_per_sm > 0 && blocks_per_sm <= 4) kern = (const void*)k_mx_persist<T, 4>;
  }
  launch_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, T, 0),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
  if (blocks_per_sm > 0) occ = std::min(occ, blocks_per_sm);
  // at least one slice per warp
  const int grid = std::max(1, std::min((A.nslice + T / 32 - 1) / (T / 32), sms * std::max(occ, 1)));
  // the tail launch: one warp for each of at most tail_slices slices
  const bool tail = tail_slices > 0 && A.ni <= kRebalanceMax;
  const int grid2 = std::max(1, std::min(grid, (tail_slices + T / 32 - 1) / (T / 32)));
  int exit1 = tail && grid2 < grid ? tail_slices : 0, resume = 0;
  void* args[] = {(void*)&A, (void*)&eta, (void*)&cap, (void*)&exit1, (void*)&resume};
  prof_begin(PK_MX_PERSIST, s);
  launch_check(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(T), args, 0, s),
               "cudaLaunchCooperativeKernel");
  prof_end(PK_MX_PERSIST, s);
  g_launches += 1;
  if (exit1 > 0) {
    int exit2 = 0, resume2 = 1;
    void* args2[] = {(void*)&A, (void*)&eta, (void*)&cap, (void*)&exit2, (void*)&resume2};
    prof_begin(PK_MX_PERSIST, s);
    launch_check(cudaLaunchCooperativeKernel(kern, dim3(grid2), dim3(T), args2, 0, s),
                 "cudaLaunchCooperativeKernel");
    prof_end(PK_MX_PERSIST, s);
    g_launches += 1;
  }
}

void launch_mx_inner_persistent(const Arena& A, float eta, int cap, int blocks_per_sm, int threads, int tail_slices,
                                cudaStream_t s) {
  launch_check(cudaMemsetAsync(A.grid_bar, 0, 8 * sizeof(unsigned int), s), "cudaMemsetAsync");
  launch_check(cudaMemsetAsync(A.red_cnt, 0, sizeof(int) * (size_t)std::max(A.ni, 1), s), "cudaMemsetAsync");
  const int blocks = (A.nslice * 32 + kSliceThreads - 1) / kSliceThreads;
  k_mx_inner_init<<<blocks, kSliceThreads, 0, s>>>(A);
  k_mx_pw0<<<blocks, kSliceThreads, 0, s>>>(A);
  k_mx_pstart<<<(A.ni * 32 + 127) / 128, 128, 0, s>>>(A);
  g_launches += 3;
  if (threads == 1024)
    persist_launch<1024>(A, eta, cap, blocks_per_sm, tail_slices, s);
  else if (threads == 512)
    persist_launch<512>(A, eta, cap, blocks_per_sm, tail_slices, s);
  else
    persist_launch<256>(A, eta, cap, blocks_per_sm, tail_slices, s);
}

void launch_mx_refine(const Arena& A, double tol, int maxcycles, cudaStream_t s) {
  k_mx_correct<<<(A.nv + 255) / 256, 256, 0, s>>>(A);
  prof_begin(PK_MX_RESIDUAL, s);
  k_mx_residual<<<A.nchunk, kChunk, 0, s>>>(A);
  prof_end(PK_MX_RESIDUAL, s);
  k_mx_check<<<(A.ni + 127) / 128, 128, 0, s>>>(A, tol, maxcycles);
  g_launches += 3;
}

}  // namespace cs
