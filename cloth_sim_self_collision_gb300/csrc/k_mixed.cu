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

__device__ __forceinline__ void precondition(const Arena& A, int bjac, int row, const float r[3], float z[3]);

// Preconditioner choice per cloth and frame: block-Jacobi when the diagonal's
// entries spread by more than kJacobiSpread (obstacle contact terms), else none
// (CG as the reference's Solve_CG).  Without contact the right-hand side of a
// falling sheet is close to a rigid translation, an eigenvector of M/dt^2 + K,
// which unpreconditioned CG resolves in a few iterations and the boundary-varying
// Jacobi scaling does not; with contact terms block-Jacobi converges faster.
constexpr float kJacobiSpread = 10.0f;

__device__ __forceinline__ void apply_dinv(const float* D, const float r[3], float z[3]) {
  z[0] = D[0] * r[0] + D[1] * r[1] + D[2] * r[2];
  z[1] = D[3] * r[0] + D[4] * r[1] + D[5] * r[2];
  z[2] = D[6] * r[0] + D[7] * r[1] + D[8] * r[2];
}

__device__ __forceinline__ void precondition(const Arena& A, int bjac, int row, const float r[3], float z[3]) {
  if (bjac) {
    apply_dinv(A.dinv32 + 9 * (size_t)row, r, z);
  } else {
    z[0] = r[0];
    z[1] = r[1];
    z[2] = r[2];
  }
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
    precondition(A, A.st[c.inst].bjac, c.row, r, z);
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
    precondition(A, A.st[c.inst].bjac, c.row, r, z);
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

// ---- persistent inner solve ---------------------------------------------------------
// One cooperative launch runs every inner CG iteration of a refinement cycle for
// all cloths.  Per iteration, two phases separated by grid barriers:
//   A: p = z + beta p_prev is built on the fly (for the rows a slice reads and
//      for its own rows, which it stores), q = A32 p, and the slice partials
//      of p.q; the last block to finish a cloth's slices sums its partials and
//      stores alpha = r.z / p.q.
//   B: d += alpha p, r -= alpha q, z = D^-1 r, and the slice partials of r.z
//      and r.r; the last block to finish a cloth's slices sums them and decides
//      convergence (|r|^2 <= eta^2 |r0|^2, or the cap) or stores beta.
// "Last block" is a per-cloth ticket counted in slices, so each total is
// summed once, in slice order by a block of fixed size: results depend neither
// on the launch shape nor on the other cloths.  A converged cloth sets istop and
// decrements the count of cloths still iterating; all blocks read that count
// after the barrier that ends phase B (nothing changes it before the next
// phase B), so they leave the loop together.
// Work split: the slices of the cloths still iterating, in arena order, are cut
// into one contiguous range per block, re-cut whenever a cloth stops, so blocks
// do not idle on converged cloths (arenas of more than kRebalanceMax cloths
// keep the static cut over all slices and skip converged cloths).  The
// direction buffers alternate between iterations.
constexpr unsigned kSpinLimit = 1u << 22;  // ~1 s of polling at the least
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
    if (atomicAdd(&A.grid_bar[0], 1u) == gridDim.x - 1) {
      atomicExch(&A.grid_bar[0], 0u);
      __threadfence();
      atomicAdd(&A.grid_bar[1], 1u);
    } else {
      unsigned n = 0;
      while (bar[1] == gen && bar[2] == 0u) {
        if (++n > kSpinLimit) {
          atomicExch(&A.grid_bar[2], 1u);
          break;
        }
        __nanosleep(256);
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

template <int kPersistThreads>
__global__ void __launch_bounds__(kPersistThreads, 1536 / kPersistThreads) k_mx_persist(Arena A, float eta, int cap) {
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
  for (int it = 1; it <= cap; it++) {
    const unsigned left = (unsigned)s_left;
    if (left == 0u) break;
    if (compact && left != cut_at) {
      compact_range<kPersistThreads>(A, s_pref, s_wsum, R);
      cut_at = left;
    }
    const float* Pold = (it & 1) ? A.p32 : A.p32b;
    float* Pnew = (it & 1) ? A.p32b : A.p32;
    // ---- phase A: direction, SpMV, p.q
    for (int inst = R.c0; inst <= R.c1; inst++) {
      int lo, hi;
      if (!portion(A, R, compact, s_pref, inst, lo, hi)) continue;
      const InstState& St = A.st[inst];
      const float beta = it > 1 ? St.beta32 : 0.f;
      const int bjac = St.bjac;
      for (int sl = lo + warp; sl < hi; sl += kPersistWarps) {
        const int row = A.slice_row0[sl] + lane;
        const int w = A.slice_w[sl];
        const float* V = A.val32 + A.slice_voff[sl] + lane;
        const int* Cc = A.col32 + A.slice_coff[sl] + lane;
        float y0 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll 2
        for (int j = 0; j < w; j++) {
          const int col = Cc[32 * j];
          const float x0 = fmaf(beta, Pold[3 * col + 0], A.z32[3 * col + 0]);
          const float x1 = fmaf(beta, Pold[3 * col + 1], A.z32[3 * col + 1]);
          const float x2 = fmaf(beta, Pold[3 * col + 2], A.z32[3 * col + 2]);
          const float* v = V + 288 * j;
          y0 = fmaf(v[0], x0, fmaf(v[32], x1, fmaf(v[64], x2, y0)));
          y1 = fmaf(v[96], x0, fmaf(v[128], x1, fmaf(v[160], x2, y1)));
          y2 = fmaf(v[192], x0, fmaf(v[224], x1, fmaf(v[256], x2, y2)));
        }
        float pq = 0.f;
        if (row < A.voff[inst + 1]) {
          float p[3];
#pragma unroll
          for (int k = 0; k < 3; k++) {
            p[k] = fmaf(beta, Pold[3 * row + k], A.z32[3 * row + k]);
            Pnew[3 * row + k] = p[k];
          }
          A.q32[3 * row + 0] = y0;
          A.q32[3 * row + 1] = y1;
          A.q32[3 * row + 2] = y2;
          pq = p[0] * y0 + p[1] * y1 + p[2] * y2;
        }
        pq = warp_sum_f(pq);
        if (lane == 0) {
          A.part32[3 * sl + 0] = pq;
          if (A.count_bytes) {  // without the preconditioner no D^-1 is read (36 B a row)
            const int rows = min(32, A.voff[inst + 1] - A.slice_row0[sl]);
            atomicAdd(&A.bytes_acc[6], (unsigned long long)(A.slice_pbytes[sl] - (bjac ? 0 : 36LL * rows)));
          }
        }
      }
      if (last_portion(A, inst, hi - lo, &s_flag)) {
        double tot[1];
        cloth_totals<kPersistThreads>(A, inst, 0, 1, sh, tot);
        if (threadIdx.x == 0) A.st[inst].alpha32 = (float)(A.st[inst].rzh[it & 1] / tot[0]);
      }
    }
    if (!grid_sync(A)) return;
    // ---- phase B: update, r.z and r.r, convergence or beta
    for (int inst = R.c0; inst <= R.c1; inst++) {
      int lo, hi;
      if (!portion(A, R, compact, s_pref, inst, lo, hi)) continue;
      InstState& St = A.st[inst];
      const float alpha = St.alpha32;
      const int bjac = St.bjac;
      for (int sl = lo + warp; sl < hi; sl += kPersistWarps) {
        const int row = A.slice_row0[sl] + lane;
        float rz = 0.f, rr = 0.f;
        if (row < A.voff[inst + 1]) {
          float r[3], z[3];
#pragma unroll
          for (int k = 0; k < 3; k++) {
            const int i = 3 * row + k;
            A.d32[i] = fmaf(alpha, Pnew[i], A.d32[i]);
            r[k] = fmaf(-alpha, A.q32[i], A.r32[i]);
            A.r32[i] = r[k];
          }
          precondition(A, bjac, row, r, z);
#pragma unroll
          for (int k = 0; k < 3; k++) {
            A.z32[3 * row + k] = z[k];
            rz += r[k] * z[k];
            rr += r[k] * r[k];
          }
        }
        rz = warp_sum_f(rz);
        rr = warp_sum_f(rr);
        if (lane == 0) {
          A.part32[3 * sl + 1] = rz;
          A.part32[3 * sl + 2] = rr;
        }
      }
      if (last_portion(A, inst, hi - lo, &s_flag)) {
        double tot[2];
        cloth_totals<kPersistThreads>(A, inst, 1, 2, sh, tot);
        if (threadIdx.x == 0) {
          St.inner_iters = it;
          if (tot[1] <= (double)eta * (double)eta * St.rr_in0 || it >= cap) {
            St.istop = 1;
            St.idone = 1;
            St.red[1] = tot[0];
            St.red[2] = tot[1];
            atomicSub(&A.grid_bar[3], 1u);
          } else {
            St.beta32 = (float)(tot[0] / St.rzh[it & 1]);
            St.rzh[(it + 1) & 1] = tot[0];
          }
        }
      }
    }
    if (!grid_sync(A)) return;
    if (threadIdx.x == 0) s_left = ((volatile unsigned*)A.grid_bar)[3];
    __syncthreads();
  }
}

// inner-solve start for the persistent kernel: totals of r.z and r.r per cloth
// and the count of cloths that iterate
__global__ void k_mx_pstart(Arena A) {
  const int inst = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (inst >= A.ni || !A.active[inst] || A.st[inst].done) return;
  const double rz = cloth_total(A, inst, 1), rr = cloth_total(A, inst, 2);
  if ((threadIdx.x & 31) == 0) {
    InstState& S = A.st[inst];
    S.rzh[1] = rz;  // iteration 1 reads parity 1
    S.rr_in0 = rr;
    S.idone = (rr <= 0.0) ? 1 : 0;
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

template <int T>
static void persist_launch(const Arena& A, float eta, int cap, int blocks_per_sm, cudaStream_t s) {
  int dev = 0, sms = 0, occ = 0;
  launch_check(cudaGetDevice(&dev), "cudaGetDevice");
  launch_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
  launch_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mx_persist<T>, T, 0),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
  if (blocks_per_sm > 0) occ = std::min(occ, blocks_per_sm);
  // at least one slice per warp
  const int grid = std::max(1, std::min((A.nslice + T / 32 - 1) / (T / 32), sms * std::max(occ, 1)));
  void* args[] = {(void*)&A, (void*)&eta, (void*)&cap};
  prof_begin(PK_MX_PERSIST, s);
  launch_check(cudaLaunchCooperativeKernel((const void*)k_mx_persist<T>, dim3(grid), dim3(T), args, 0, s),
               "cudaLaunchCooperativeKernel");
  prof_end(PK_MX_PERSIST, s);
  g_launches += 1;
}

void launch_mx_inner_persistent(const Arena& A, float eta, int cap, int blocks_per_sm, int threads,
                                cudaStream_t s) {
  launch_check(cudaMemsetAsync(A.grid_bar, 0, 4 * sizeof(unsigned int), s), "cudaMemsetAsync");
  launch_check(cudaMemsetAsync(A.red_cnt, 0, sizeof(int) * (size_t)std::max(A.ni, 1), s), "cudaMemsetAsync");
  const int blocks = (A.nslice * 32 + kSliceThreads - 1) / kSliceThreads;
  k_mx_inner_init<<<blocks, kSliceThreads, 0, s>>>(A);
  k_mx_pstart<<<(A.ni * 32 + 127) / 128, 128, 0, s>>>(A);
  g_launches += 2;
  if (threads == 1024)
    persist_launch<1024>(A, eta, cap, blocks_per_sm, s);
  else if (threads == 512)
    persist_launch<512>(A, eta, cap, blocks_per_sm, s);
  else
    persist_launch<256>(A, eta, cap, blocks_per_sm, s);
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
