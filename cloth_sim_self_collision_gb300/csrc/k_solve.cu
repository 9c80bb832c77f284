// k_solve.cu -- linear solvers of the implicit step.
//
// * Block ILU(0) + PCG (CPreconditionerILU / Solve_PCG, ilu_sparse.cpp:352-709):
//   one CTA per cloth runs the factorisation and the whole PCG loop.  Rows are
//   processed in dependency levels of the natural-order factorisation (and of
//   the forward / backward sweeps), separated by __syncthreads, so every row
//   is computed with exactly the reference's operation order; only the inner
//   products are tree-summed (deterministically).
// * CG (Solve_CG, matrix_square_sparse.cpp:338-406): three grid-wide kernels
//   per iteration over the rows of all active cloths; per-cloth reductions go
//   through per-chunk partials summed in a fixed order.
#include <float.h>

#include "kernels.h"

namespace cs {
namespace {

constexpr int kSolveThreads = 512;
constexpr int kChunk = 256;  // rows per CG chunk (one CTA)

__device__ __forceinline__ double det33(const double* a) {
  return +a[0] * a[4] * a[8] + a[3] * a[7] * a[2] + a[6] * a[1] * a[5] - a[0] * a[7] * a[5] -
         a[6] * a[4] * a[2] - a[3] * a[1] * a[8];
}

// CalcInvMat3 (ilu_sparse.cpp:76-97): cofactor inverse into out from t
__device__ __forceinline__ void inv33(double* out, const double* t) {
  const double r = 1.0 / det33(t);
  out[0] = r * (t[4] * t[8] - t[5] * t[7]);
  out[1] = r * (t[2] * t[7] - t[1] * t[8]);
  out[2] = r * (t[1] * t[5] - t[2] * t[4]);
  out[3] = r * (t[5] * t[6] - t[3] * t[8]);
  out[4] = r * (t[0] * t[8] - t[2] * t[6]);
  out[5] = r * (t[2] * t[3] - t[0] * t[5]);
  out[6] = r * (t[3] * t[7] - t[4] * t[6]);
  out[7] = r * (t[1] * t[6] - t[0] * t[7]);
  out[8] = r * (t[0] * t[4] - t[1] * t[3]);
}

// Deterministic block-wide sum: fixed xor-shuffle tree per warp, then the
// warp totals in warp order.  All threads receive the result.
__device__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

// <a, b> over dofs [lo, hi) of a cloth, by one CTA: a deterministic tree sum,
// or with `serial` one running sum in dof order like the reference's
// InnerProduct (matrix_square_sparse.cpp:313-325)
__device__ double cta_dot(const double* a, const double* b, int lo, int hi, double* sh, bool serial) {
  if (serial) {
    __syncthreads();
    if (threadIdx.x == 0) {
      double r = 0.0;
      for (int i = lo; i < hi; i++) r += a[i] * b[i];
      sh[33] = r;
    }
    __syncthreads();
    return sh[33];
  }
  double s = 0.0;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) s += a[i] * b[i];
  return block_sum(s, sh);
}

__device__ __forceinline__ double serial_dot(const double* a, const double* b, int lo, int hi) {
  double r = 0.0;
  for (int i = lo; i < hi; i++) r += a[i] * b[i];
  return r;
}

// y_i = 0 * y_i + sum_j A_ij x_j for row i (MatVec(1, x, 0, y), matrix_square_sparse.cpp:218-242)
__device__ __forceinline__ void spmv_row(const Arena& A, int i, const double* x, double* y) {
  double y0 = y[3 * i + 0] * 0.0, y1 = y[3 * i + 1] * 0.0, y2 = y[3 * i + 2] * 0.0;
  for (int s = A.row_ptr[i]; s < A.row_ptr[i + 1]; s++) {
    const int j = A.col_idx[s];
    const double* a = A.vcrs + 9 * (size_t)s;
    const double x0 = x[3 * j + 0], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
    y0 += 1.0 * (a[0] * x0 + a[1] * x1 + a[2] * x2);
    y1 += 1.0 * (a[3] * x0 + a[4] * x1 + a[5] * x2);
    y2 += 1.0 * (a[6] * x0 + a[7] * x1 + a[8] * x2);
  }
  const double* a = A.vdia + 9 * (size_t)i;
  const double x0 = x[3 * i + 0], x1 = x[3 * i + 1], x2 = x[3 * i + 2];
  y0 += 1.0 * (a[0] * x0 + a[1] * x1 + a[2] * x2);
  y1 += 1.0 * (a[3] * x0 + a[4] * x1 + a[5] * x2);
  y2 += 1.0 * (a[6] * x0 + a[7] * x1 + a[8] * x2);
  y[3 * i + 0] = y0;
  y[3 * i + 1] = y1;
  y[3 * i + 2] = y2;
}

// one row of DoILUDecomp (3x3 branch, ilu_sparse.cpp:507-569).  stop_here:
// the row at which the reference gives up (updates only).  Returns 1 when the
// pivot is singular.
__device__ int factor_row(const Arena& A, int i, bool stop_here) {
  double* D = A.fdia + 9 * (size_t)i;
  for (int o = A.fac_ptr[i]; o < A.fac_ptr[i + 1]; o++) {
    const int s = A.fac_ops[3 * o + 0], ks = A.fac_ops[3 * o + 1], tg = A.fac_ops[3 * o + 2];
    const double* lik = A.fcrs + 9 * (size_t)s;
    const double* ukj = A.fcrs + 9 * (size_t)ks;
    double* dst = (tg < 0) ? D : A.fcrs + 9 * (size_t)tg;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      dst[r * 3 + 0] -= lik[r * 3 + 0] * ukj[0] + lik[r * 3 + 1] * ukj[3] + lik[r * 3 + 2] * ukj[6];
      dst[r * 3 + 1] -= lik[r * 3 + 0] * ukj[1] + lik[r * 3 + 1] * ukj[4] + lik[r * 3 + 2] * ukj[7];
      dst[r * 3 + 2] -= lik[r * 3 + 0] * ukj[2] + lik[r * 3 + 1] * ukj[5] + lik[r * 3 + 2] * ukj[8];
    }
  }
  int singular = 0;
  double t[9];
#pragma unroll
  for (int k = 0; k < 9; k++) t[k] = D[k];
  if (fabs(det33(t)) > 1.0e-30) {
    if (!stop_here) inv33(D, t);
  } else {
    singular = 1;
  }
  if (stop_here) return singular;
  for (int s = A.dia_split[i]; s < A.row_ptr[i + 1]; s++) {  // U <- D^-1 U
    double* u = A.fcrs + 9 * (size_t)s;
    double w[9];
#pragma unroll
    for (int k = 0; k < 9; k++) w[k] = u[k];
#pragma unroll
    for (int r = 0; r < 3; r++) {
      u[r * 3 + 0] = D[r * 3 + 0] * w[0] + D[r * 3 + 1] * w[3] + D[r * 3 + 2] * w[6];
      u[r * 3 + 1] = D[r * 3 + 0] * w[1] + D[r * 3 + 1] * w[4] + D[r * 3 + 2] * w[7];
      u[r * 3 + 2] = D[r * 3 + 0] * w[2] + D[r * 3 + 1] * w[5] + D[r * 3 + 2] * w[8];
    }
  }
  return singular;
}

__device__ void copy_matrix(const Arena& A, int v0, int v1) {
  for (int k = 9 * v0 + threadIdx.x; k < 9 * v1; k += blockDim.x) A.fdia[k] = A.vdia[k];
  const int s0 = A.row_ptr[v0], s1 = A.row_ptr[v1];
  for (int k = 9 * s0 + threadIdx.x; k < 9 * s1; k += blockDim.x) A.fcrs[k] = A.vcrs[k];
  __syncthreads();
}

// Rows with more blocks than this are factorised by one thread (factor_row);
// grid rows have at most 13.
constexpr int kRowSlots = 24;

// One row of DoILUDecomp by a warp, the row's blocks staged in shared memory
// (sm: 9 * (1 + kRowSlots) doubles: D, then the row's slots).  Lanes 0-8 own one
// entry (r, c) of the 3x3 blocks and apply the updates in the reference's
// order, entry by entry exactly as factor_row does; the warp syncs between
// updates because a later update may read a block an earlier one wrote.
// Returns 1 when the pivot is singular (all lanes).
__device__ int factor_row_warp(const Arena& A, int i, bool stop_here, double* sm) {
  const int lane = threadIdx.x & 31;
  const int r0 = A.row_ptr[i], r1 = A.row_ptr[i + 1], n = r1 - r0;
  for (int k = lane; k < 9 * (n + 1); k += 32) sm[k] = k < 9 ? A.fdia[9 * (size_t)i + k] : A.fcrs[9 * (size_t)r0 + k - 9];
  __syncwarp();
  const int r = lane / 3, c = lane % 3;
  for (int o = A.fac_ptr[i]; o < A.fac_ptr[i + 1]; o++) {
    const int s = A.fac_ops[3 * o + 0], ks = A.fac_ops[3 * o + 1], tg = A.fac_ops[3 * o + 2];
    if (lane < 9) {
      const double* lik = sm + 9 * (1 + s - r0);
      const double* ukj = A.fcrs + 9 * (size_t)ks;
      double* dst = (tg < 0) ? sm : sm + 9 * (1 + tg - r0);
      dst[r * 3 + c] -= lik[r * 3 + 0] * ukj[c] + lik[r * 3 + 1] * ukj[3 + c] + lik[r * 3 + 2] * ukj[6 + c];
    }
    __syncwarp();
  }
  double t[9];
#pragma unroll
  for (int k = 0; k < 9; k++) t[k] = sm[k];
  __syncwarp();
  const double det = det33(t);
  const int singular = fabs(det) > 1.0e-30 ? 0 : 1;
  if (!singular && !stop_here && lane < 9) {
    // CalcInvMat3 (ilu_sparse.cpp:76-97) as inv33: entry `lane` of the cofactor inverse
    double inv[9];
    inv33(inv, t);
    double val = inv[0];
#pragma unroll
    for (int q = 1; q < 9; q++)
      if (lane == q) val = inv[q];
    sm[lane] = val;
  }
  __syncwarp();
  if (!stop_here) {
    // U <- D^-1 U, three blocks at a time (lanes 9g .. 9g + 8 for block g)
    const int ds = A.dia_split[i];
    const int g = lane / 9, e = lane % 9, er = e / 3, ec = e % 3;
    for (int s0 = ds; s0 < r1; s0 += 3) {
      const int s = s0 + g;
      double val = 0.0;
      const bool mine = g < 3 && s < r1;
      if (mine) {
        const double* w = sm + 9 * (1 + s - r0);
        val = sm[er * 3 + 0] * w[ec] + sm[er * 3 + 1] * w[3 + ec] + sm[er * 3 + 2] * w[6 + ec];
      }
      __syncwarp();
      if (mine) sm[9 * (1 + s - r0) + e] = val;
      __syncwarp();
    }
  }
  for (int k = lane; k < 9 * (n + 1); k += 32) {
    if (k < 9)
      A.fdia[9 * (size_t)i + k] = sm[k];
    else
      A.fcrs[9 * (size_t)r0 + k - 9] = sm[k];
  }
  __syncwarp();
  return singular;
}

// Factorises rows by level, one warp per row; rows after `limit` are left as
// copied and row `limit` gets its updates only, as when the reference stops
// after more than ten singular pivots (ilu_sparse.cpp:541-551).
__device__ void factor_levels(const Arena& A, int inst, int limit) {
  __shared__ double sm_rows[kSolveThreads / 32][9 * (1 + kRowSlots)];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int l0 = A.lev_off[inst], l1 = A.lev_off[inst + 1];
  for (int l = l0; l < l1; l++) {
    for (int k = A.lev_ptr[l] + warp; k < A.lev_ptr[l + 1]; k += nw) {
      const int i = A.lev_rows[k];
      if (i > limit) continue;
      if (A.row_ptr[i + 1] - A.row_ptr[i] <= kRowSlots) {
        const int sg = factor_row_warp(A, i, i == limit, sm_rows[warp]);
        if (lane == 0) A.sing[i] = sg;
      } else if (lane == 0) {
        A.sing[i] = factor_row(A, i, i == limit);
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kSolveThreads) k_ilu_factor(Arena A, const int* list, int masked) {
  __shared__ double sh[40];
  __shared__ int limit;
  const int inst = list[blockIdx.x];
  if (masked && !A.active[inst]) return;
  const int v0 = A.voff[inst], v1 = A.voff[inst + 1];
  copy_matrix(A, v0, v1);
  factor_levels(A, inst, INT_MAX);
  double cnt = 0;
  for (int i = v0 + threadIdx.x; i < v1; i += blockDim.x) cnt += A.sing[i];
  const int nsing = (int)block_sum(cnt, sh);
  if (nsing > 10) {
    if (threadIdx.x == 0) {
      int seen = 0;
      limit = v1;
      for (int i = v0; i < v1; i++)
        if (A.sing[i] && ++seen == 11) {
          limit = i;
          break;
        }
    }
    __syncthreads();
    copy_matrix(A, v0, v1);
    factor_levels(A, inst, limit);
  }
  if (threadIdx.x == 0) A.st[inst].ilu_singular = nsing > 10 ? 11 : nsing;
}

// t -= sum over the slots [s0, s1) of B_s z_col(s), in slot order, by a warp:
// lane j forms slot j's three row products (B[r][0] y0 + B[r][1] y1 + B[r][2] y2,
// the reference's grouping), then every lane subtracts them in slot order
__device__ __forceinline__ void row_sweep_sub(const Arena& A, const double* z, int s0, int s1, double t[3]) {
  const int lane = threadIdx.x & 31;
  for (int base = s0; base < s1; base += 32) {
    const int s = base + lane;
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    if (s < s1) {
      const int j = A.col_idx[s];
      const double* b9 = A.fcrs + 9 * (size_t)s;
      const double y0 = z[3 * j + 0], y1 = z[3 * j + 1], y2 = z[3 * j + 2];
      d0 = b9[0] * y0 + b9[1] * y1 + b9[2] * y2;
      d1 = b9[3] * y0 + b9[4] * y1 + b9[5] * y2;
      d2 = b9[6] * y0 + b9[7] * y1 + b9[8] * y2;
    }
    const int m = min(32, s1 - base);
    for (int q = 0; q < m; q++) {
      t[0] -= __shfl_sync(0xffffffffu, d0, q);
      t[1] -= __shfl_sync(0xffffffffu, d1, q);
      t[2] -= __shfl_sync(0xffffffffu, d2, q);
    }
  }
}

// z <- (LU)^-1 z in place: forward sweep by levels, then backward sweep by
// levels (ilu_sparse.cpp:185-215, 295-324), one warp per row
__device__ void ilu_apply(const Arena& A, int inst, double* z) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int l = A.lev_off[inst]; l < A.lev_off[inst + 1]; l++) {
    for (int k = A.lev_ptr[l] + warp; k < A.lev_ptr[l + 1]; k += nw) {
      const int i = A.lev_rows[k];
      double t[3] = {z[3 * i + 0], z[3 * i + 1], z[3 * i + 2]};
      row_sweep_sub(A, z, A.row_ptr[i], A.dia_split[i], t);
      if (lane == 0) {
        const double* d = A.fdia + 9 * (size_t)i;
        z[3 * i + 0] = d[0] * t[0] + d[1] * t[1] + d[2] * t[2];
        z[3 * i + 1] = d[3] * t[0] + d[4] * t[1] + d[5] * t[2];
        z[3 * i + 2] = d[6] * t[0] + d[7] * t[1] + d[8] * t[2];
      }
    }
    __syncthreads();
  }
  for (int l = A.blev_off[inst]; l < A.blev_off[inst + 1]; l++) {
    for (int k = A.blev_ptr[l] + warp; k < A.blev_ptr[l + 1]; k += nw) {
      const int i = A.blev_rows[k];
      double t[3] = {z[3 * i + 0], z[3 * i + 1], z[3 * i + 2]};
      row_sweep_sub(A, z, A.dia_split[i], A.row_ptr[i + 1], t);
      if (lane == 0) {
        z[3 * i + 0] = t[0];
        z[3 * i + 1] = t[1];
        z[3 * i + 2] = t[2];
      }
    }
    __syncthreads();
  }
}

// Solve_PCG (ilu_sparse.cpp:628-709) from dx = 0 with r = b
__global__ void __launch_bounds__(kSolveThreads) k_pcg(Arena A, const int* list, double tol_in, int maxit_in,
                                                       int masked) {
  __shared__ double sh[40];
  const int inst = list[blockIdx.x];
  if (masked && !A.active[inst]) return;
  const DevParams& P = A.prm[inst];
  const double tol = tol_in >= 0 ? tol_in : P.tol;
  const int maxit = maxit_in >= 0 ? maxit_in : P.maxit;
  const bool serial = (P.flags & 1) != 0;
  const int v0 = A.voff[inst], v1 = A.voff[inst + 1];
  const int d0 = 3 * v0, d1 = 3 * v1;
  double *x = A.dx, *r = A.r, *p = A.p, *z = A.z;
  for (int i = d0 + threadIdx.x; i < d1; i += blockDim.x) {
    x[i] = 0.0;
    r[i] = A.b[i];
  }
  __syncthreads();
  const double s0 = cta_dot(r, r, d0, d1, sh, serial);
  if (s0 < 1.0e-30) {
    if (threadIdx.x == 0) {
      A.st[inst].solver_conv = 0.0;
      A.st[inst].solver_iterations = 0;
    }
    return;
  }
  const double inv0 = 1.0 / s0;
  for (int i = d0 + threadIdx.x; i < d1; i += blockDim.x) z[i] = r[i];
  __syncthreads();
  ilu_apply(A, inst, z);
  for (int i = d0 + threadIdx.x; i < d1; i += blockDim.x) p[i] = z[i];
  __syncthreads();
  double rPr = cta_dot(r, z, d0, d1, sh, serial);
  for (int it = 0; it < maxit; it++) {
    for (int i = v0 + threadIdx.x; i < v1; i += blockDim.x) spmv_row(A, i, p, z);  // Ap in z
    __syncthreads();
    const double pAp = cta_dot(p, z, d0, d1, sh, serial);
    const double alpha = rPr / pAp;
    for (int i = d0 + threadIdx.x; i < d1; i += blockDim.x) {
      r[i] += -alpha * z[i];
      x[i] += +alpha * p[i];
    }
    __syncthreads();
    const double sq = cta_dot(r, r, d0, d1, sh, serial);
    if (sq * inv0 < tol * tol) {
      if (threadIdx.x == 0) {
        A.st[inst].solver_conv = sqrt(sq * inv0);
        A.st[inst].solver_iterations = it;
      }
      return;
    }
    for (int i = d0 + threadIdx.x; i < d1; i += blockDim.x) z[i] = r[i];
    __syncthreads();
    ilu_apply(A, inst, z);
    const double rPr1 = cta_dot(r, z, d0, d1, sh, serial);
    const double beta = rPr1 / rPr;
    rPr = rPr1;
    for (int i = d0 + threadIdx.x; i < d1; i += blockDim.x) p[i] = z[i] + beta * p[i];
    __syncthreads();
  }
  const double sq = cta_dot(r, r, d0, d1, sh, serial);
  if (threadIdx.x == 0) {
    A.st[inst].solver_conv = sqrt(sq * inv0);
    A.st[inst].solver_iterations = maxit;
  }
}

// ---- CG over all active cloths ---------------------------------------------
__device__ __forceinline__ double chunk_total(const double* part, int c0, int c1) {
  double s = 0.0;
  for (int c = c0; c < c1; c++) s += part[c];
  return s;
}

__global__ void __launch_bounds__(kChunk) k_cg_init(Arena A, double tol_in, int maxit_in) {
  __shared__ double sh[40];
  const int c = blockIdx.x;
  const int inst = A.chunk_inst[c];
  if (!A.active[inst]) return;
  const int row = A.voff[inst] + (c - A.chunk_lo[inst]) * kChunk + threadIdx.x;
  double s = 0.0;
  if (row < A.voff[inst + 1]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double bk = A.b[3 * row + k];
      A.dx[3 * row + k] = 0.0;
      A.r[3 * row + k] = bk;
      A.p[3 * row + k] = bk;
      A.z[3 * row + k] = 0.0;
      s += bk * bk;
    }
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) A.part[c] = s;
  (void)tol_in;
  (void)maxit_in;
}

// per cloth: r.r of the start, the early exit of a tiny right-hand side
__global__ void k_cg_start(Arena A, double tol_in, int maxit_in) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= A.ni || !A.active[inst]) return;
  const DevParams& P = A.prm[inst];
  const double tol = tol_in >= 0 ? tol_in : P.tol;
  const int maxit = maxit_in >= 0 ? maxit_in : P.maxit;
  const double s0 = (P.flags & 1) ? serial_dot(A.b, A.b, 3 * A.voff[inst], 3 * A.voff[inst + 1])
                                   : chunk_total(A.part, A.chunk_lo[inst], A.chunk_hi[inst]);
  InstState& S = A.st[inst];
  S.sq[1] = s0;  // iteration 1 reads parity 1
  S.solver_iterations = maxit;
  S.solver_conv = tol;
  if (s0 < 1.0e-30) {
    S.done = 1;
    S.solver_conv = 0.0;
    S.solver_iterations = 0;
  } else {
    S.done = maxit <= 1 ? 1 : 0;
    S.inv0 = 1.0 / s0;
  }
}

// Ap = A p and the chunk partials of p.Ap, one thread per row (FP64-pipe bound
// on GB300; the row's in-order sum stays on one lane)
__global__ void __launch_bounds__(kChunk) k_cg_spmv(Arena A) {
  __shared__ double sh[40];
  const int c = blockIdx.x;
  const int inst = A.chunk_inst[c];
  if (!A.active[inst] || A.st[inst].done) return;
  const int row = A.voff[inst] + (c - A.chunk_lo[inst]) * kChunk + threadIdx.x;
  double s = 0.0;
  if (row < A.voff[inst + 1]) {
    spmv_row(A, row, A.p, A.z);
    s = A.p[3 * row + 0] * A.z[3 * row + 0] + A.p[3 * row + 1] * A.z[3 * row + 1] +
        A.p[3 * row + 2] * A.z[3 * row + 2];
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) {
    A.part[c] = s;
    if (A.count_bytes) atomicAdd(&A.bytes_acc[1], (unsigned long long)A.chunk_bytes[c]);
  }
}

// the iteration number: the launch's, or (it < 0, a graph frame) the device counter
__device__ __forceinline__ int cg_iter(const Arena& A, int it) { return it >= 0 ? it : A.ctl->cycle; }

// alpha = r.r / p.Ap; x += alpha p; r -= alpha Ap; chunk partials of r.r
__global__ void __launch_bounds__(kChunk) k_cg_update(Arena A, int it_in) {
  __shared__ double sh[40];
  const int it = cg_iter(A, it_in);
  const int c = blockIdx.x;
  const int inst = A.chunk_inst[c];
  if (!A.active[inst] || A.st[inst].done) return;
  const double pAp = (A.prm[inst].flags & 1) ? A.st[inst].dot[0] : chunk_total(A.part, A.chunk_lo[inst], A.chunk_hi[inst]);
  const double alpha = A.st[inst].sq[it & 1] / pAp;
  const int row = A.voff[inst] + (c - A.chunk_lo[inst]) * kChunk + threadIdx.x;
  double s = 0.0;
  if (row < A.voff[inst + 1]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int i = 3 * row + k;
      A.dx[i] += alpha * A.p[i];
      const double rk = A.r[i] + (-alpha) * A.z[i];
      A.r[i] = rk;
      s += rk * rk;
    }
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) A.part[A.nchunk + c] = s;
}

// convergence test, beta and p = r + beta p
__global__ void __launch_bounds__(kChunk) k_cg_direction(Arena A, int it_in, double tol_in, int maxit_in) {
  const int it = cg_iter(A, it_in);
  const int c = blockIdx.x;
  const int inst = A.chunk_inst[c];
  if (!A.active[inst] || A.st[inst].done) return;
  const DevParams& P = A.prm[inst];
  const double tol = tol_in >= 0 ? tol_in : P.tol;
  InstState& S = A.st[inst];
  const double sq = S.sq[it & 1];
  const double sqn = (P.flags & 1) ? S.dot[1] : chunk_total(A.part + A.nchunk, A.chunk_lo[inst], A.chunk_hi[inst]);
  const bool first = (c == A.chunk_lo[inst]);
  if (sqn * S.inv0 < tol * tol) {
    if (first && threadIdx.x == 0) {
      S.solver_conv = sqrt(sq * S.inv0);
      S.solver_iterations = it;
      S.done = 1;
    }
    return;
  }
  const double beta = sqn / sq;
  const int row = A.voff[inst] + (c - A.chunk_lo[inst]) * kChunk + threadIdx.x;
  if (row < A.voff[inst + 1]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int i = 3 * row + k;
      A.p[i] = A.r[i] + beta * A.p[i];
    }
  }
  if (first && threadIdx.x == 0) {
    S.sq[(it + 1) & 1] = sqn;
    if (it + 1 >= (maxit_in >= 0 ? maxit_in : P.maxit)) S.done = 1;  // iteration cap reached
  }
}

// serial inner products of the cloths that ask for them (one thread per cloth):
// which = 0: p.Ap into dot[0]; which = 1: r.r into dot[1]
__global__ void k_cg_serial_dot(Arena A, int which) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= A.ni || !A.active[inst] || A.st[inst].done || !(A.prm[inst].flags & 1)) return;
  const int lo = 3 * A.voff[inst], hi = 3 * A.voff[inst + 1];
  if (which == 0)
    A.st[inst].dot[0] = serial_dot(A.p, A.z, lo, hi);
  else
    A.st[inst].dot[1] = serial_dot(A.r, A.r, lo, hi);
}

__global__ void k_spmv_all(Arena A, const double* x, double* y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.nv) return;
  spmv_row(A, i, x, y);
}

// y = beta y + alpha A x over rows [v0, v1), in the operation order of
// MatVec's 3x3 branch (matrix_square_sparse.cpp:218-242)
__global__ void k_matvec_rows(Arena A, int v0, int v1, double alpha, const double* x, double beta, double* y) {
  const int i = v0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v1) return;
  double y0 = y[3 * i + 0] * beta, y1 = y[3 * i + 1] * beta, y2 = y[3 * i + 2] * beta;
  for (int s = A.row_ptr[i]; s < A.row_ptr[i + 1]; s++) {
    const int j = A.col_idx[s];
    const double* a = A.vcrs + 9 * (size_t)s;
    const double x0 = x[3 * j + 0], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
    y0 += alpha * (a[0] * x0 + a[1] * x1 + a[2] * x2);
    y1 += alpha * (a[3] * x0 + a[4] * x1 + a[5] * x2);
    y2 += alpha * (a[6] * x0 + a[7] * x1 + a[8] * x2);
  }
  const double* a = A.vdia + 9 * (size_t)i;
  const double x0 = x[3 * i + 0], x1 = x[3 * i + 1], x2 = x[3 * i + 2];
  y0 += alpha * (a[0] * x0 + a[1] * x1 + a[2] * x2);
  y1 += alpha * (a[3] * x0 + a[4] * x1 + a[5] * x2);
  y2 += alpha * (a[6] * x0 + a[7] * x1 + a[8] * x2);
  y[3 * i + 0] = y0;
  y[3 * i + 1] = y1;
  y[3 * i + 2] = y2;
}

// CPreconditionerILU::Solve (ilu_sparse.h:23-26): z <- (LU)^-1 z for one cloth
__global__ void __launch_bounds__(kSolveThreads) k_ilu_solve(Arena A, int inst, double* z) { ilu_apply(A, inst, z); }

}  // namespace

void launch_ilu_factor(const Arena& A, const int* list, int n, cudaStream_t s, bool masked) {
  if (n <= 0) return;
  prof_begin(PK_ILU_FACTOR, s);
  k_ilu_factor<<<n, kSolveThreads, 0, s>>>(A, list, masked ? 1 : 0);
  prof_end(PK_ILU_FACTOR, s);
  g_launches++;
}

void launch_pcg(const Arena& A, const int* list, int n, double tol, int maxit, cudaStream_t s, bool masked) {
  if (n <= 0) return;
  prof_begin(PK_PCG, s);
  k_pcg<<<n, kSolveThreads, 0, s>>>(A, list, tol, maxit, masked ? 1 : 0);
  prof_end(PK_PCG, s);
  g_launches++;
}

void launch_cg_init(const Arena& A, double tol, int maxit, cudaStream_t s) {
  k_cg_init<<<A.nchunk, kChunk, 0, s>>>(A, tol, maxit);
  k_cg_start<<<(A.ni + 127) / 128, 128, 0, s>>>(A, tol, maxit);
  g_launches += 2;
}

void launch_cg_iteration(const Arena& A, int it, double tol, int maxit, bool serial, cudaStream_t s) {
  prof_begin(PK_CG_SPMV, s);
  k_cg_spmv<<<A.nchunk, kChunk, 0, s>>>(A);
  prof_end(PK_CG_SPMV, s);
  if (serial) {
    k_cg_serial_dot<<<(A.ni + 127) / 128, 128, 0, s>>>(A, 0);
    g_launches++;
  }
  prof_begin(PK_CG_UPDATE, s);
  k_cg_update<<<A.nchunk, kChunk, 0, s>>>(A, it);
  prof_end(PK_CG_UPDATE, s);
  if (serial) {
    k_cg_serial_dot<<<(A.ni + 127) / 128, 128, 0, s>>>(A, 1);
    g_launches++;
  }
  prof_begin(PK_CG_DIRECTION, s);
  k_cg_direction<<<A.nchunk, kChunk, 0, s>>>(A, it, tol, maxit);
  prof_end(PK_CG_DIRECTION, s);
  g_launches += 3;
}

void launch_spmv(const Arena& A, const double* x, double* y, cudaStream_t s) {
  k_spmv_all<<<(A.nv + 127) / 128, 128, 0, s>>>(A, x, y);
  g_launches++;
}

void launch_matvec(const Arena& A, int v0, int v1, double alpha, const double* x, double beta, double* y,
                   cudaStream_t s) {
  if (v1 <= v0) return;
  k_matvec_rows<<<(v1 - v0 + 127) / 128, 128, 0, s>>>(A, v0, v1, alpha, x, beta, y);
  g_launches++;
}

void launch_ilu_solve(const Arena& A, int inst, double* z, cudaStream_t s) {
  k_ilu_solve<<<1, kSolveThreads, 0, s>>>(A, inst, z);
  g_launches++;
}

}  // namespace cs
