// k_assemble.cu -- element kernels and deterministic assembly of the implicit
// system (solve_internal_sparse.h:19-183, 276-313; matrix_square_sparse.cpp:88-302).
//
// Assembly without float atomics: each triangle writes its nine 3x3 Hessian
// blocks and its gradient rows to element buffers; each matrix slot then sums
// its contributions from a precomputed source list in the reference's merge
// order (triangles ascending, then bending stencils ascending, then the
// obstacle term on the diagonal), so the FP64 sums round exactly like the
// reference's sequential Mearge.  Bending Hessians are constant (K K^T s I3):
// the stencil entries are rebuilt from the rest-shape factors on the fly.
#include "element.cuh"
#include "kernels.h"

namespace cs {

std::atomic<long long> g_launches{0};

namespace {

constexpr int kThreads = 128;

inline int blocks_for(long long n, int t = kThreads) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ void load3(const double* a, int v, double* out) {
  out[0] = a[3 * v + 0];
  out[1] = a[3 * v + 1];
  out[2] = a[3 * v + 2];
}

template <int A, int B>
__device__ __forceinline__ void store_block(const CstState<double>& st, double* dst) {
  double blk[9];
  cst_hessian_block<double, A, B>(st, blk);
#pragma unroll
  for (int k = 0; k < 9; k++) dst[(A * 3 + B) * 9 + k] = blk[k];
}

__global__ void k_quad_factors(Arena A) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= A.nq) return;
  const DevParams& P = A.prm[A.qinst[q]];
  double C[12];
#pragma unroll
  for (int a = 0; a < 4; a++) load3(A.X0, A.quad[4 * q + a], C + 3 * a);
  double K[4], s;
  bend_factors<double>(C, P.stiff_bend, K, s);
#pragma unroll
  for (int a = 0; a < 4; a++) A.qK[4 * q + a] = K[a];
  A.qscale[q] = s;
}

// per triangle: CST gradient rows (and Hessian blocks) at the current positions
__global__ void k_tri_elements(Arena A, int hess, int masked) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nt) return;
  const int inst = A.tinst[t];
  if (masked && !A.active[inst]) return;
  const DevParams& P = A.prm[inst];
  double C[9], c[9];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const int v = A.tri[3 * t + a];
    load3(A.X0, v, C + 3 * a);
    load3(A.x, v, c + 3 * a);
  }
  CstState<double> st;
  cst_state<double>(C, c, P.lambda, P.myu, st);
  double g[9];
  cst_gradient<double>(st, g);
#pragma unroll
  for (int k = 0; k < 9; k++) A.tri_grad[9 * (size_t)t + k] = g[k];
  if (!hess) return;
  double* dst = A.tri_blk + 81 * (size_t)t;
  store_block<0, 0>(st, dst);
  store_block<0, 1>(st, dst);
  store_block<0, 2>(st, dst);
  store_block<1, 0>(st, dst);
  store_block<1, 1>(st, dst);
  store_block<1, 2>(st, dst);
  store_block<2, 0>(st, dst);
  store_block<2, 1>(st, dst);
  store_block<2, 2>(st, dst);
}

// per bending stencil: gradient H c
__global__ void k_quad_grad(Arena A, int masked) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= A.nq) return;
  if (masked && !A.active[A.qinst[q]]) return;
  double c[12], K[4], g[12];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    load3(A.x, A.quad[4 * q + a], c + 3 * a);
    K[a] = A.qK[4 * q + a];
  }
  bend_gradient<double>(K, A.qscale[q], c, g);
#pragma unroll
  for (int k = 0; k < 12; k++) A.quad_grad[12 * (size_t)q + k] = g[k];
}

// per matrix slot (off-diagonal blocks, then diagonal blocks): ordered sum of
// its element contributions, then the obstacle term, mass / dt^2 and the
// boundary conditions (SetBoundaryCondition, matrix_square_sparse.cpp:272-302)
__global__ void k_slot_reduce(Arena A) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= A.nb + A.nv) return;
  double acc[9];
#pragma unroll
  for (int k = 0; k < 9; k++) acc[k] = 0.0;
  // A slot's list holds its triangle blocks, then its stencil blocks (all
  // triangles are merged before the stencils), so two loops keep warps uniform.
  const int e_end = A.slot_ptr[s + 1];
  int e = A.slot_ptr[s];
  for (; e < e_end; e++) {
    const int code = A.slot_src[e];
    if (code < 0) break;
    const double* blk = A.tri_blk + 9 * (size_t)code;
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] += blk[k];
  }
  for (; e < e_end; e++) {
    const int c = -A.slot_src[e] - 1;
    const int q = c >> 4, a = (c >> 2) & 3, b = c & 3;
    const double h = A.qK[4 * q + a] * A.qK[4 * q + b] * A.qscale[q];
    acc[0] += h;
    acc[4] += h;
    acc[8] += h;
    // the stencil block's off-diagonal entries are +0.0; x + (+0.0) is x
    // except that -0.0 becomes +0.0, done here on the bits
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if (k % 4 == 0) continue;
      const unsigned long long u = (unsigned long long)__double_as_longlong(acc[k]);
      if (u == 0x8000000000000000ull) acc[k] = 0.0;
    }
  }
  if (s < A.nb) {
    const int row = A.blk_row[s], col = A.col_idx[s];
    const bool fixed = A.bc[row] != 0 || A.bc[col] != 0;
#pragma unroll
    for (int k = 0; k < 9; k++) A.vcrs[9 * (size_t)s + k] = fixed ? 0.0 : acc[k];
    if (A.mixed) {
      float* dst = A.val32 + A.sell_pos[s];
#pragma unroll
      for (int k = 0; k < 9; k++) dst[32 * k] = fixed ? 0.f : (float)acc[k];
    }
    return;
  }
  const int v = s - A.nb;
  const DevParams& P = A.prm[A.vinst[v]];
  {
    double p[3], W, dW[3], ddW[9];
    load3(A.x, v, p);
    contact_energy<double>(P.obstacle_kind, P.obs_center, P.obs_radius, P.stiff_contact, P.contact_clearance, p,
                           W, dW, ddW);
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] += ddW[k];
  }
  const double m = P.mass_point / (P.dt * P.dt);
  acc[0] += m;
  acc[4] += m;
  acc[8] += m;
  const bool fixed = A.bc[v] != 0;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    acc[k] = fixed ? ((k % 4 == 0) ? 1.0 : 0.0) : acc[k];
    A.vdia[9 * (size_t)v + k] = acc[k];
  }
  if (A.mixed) {
    float* dst = A.val32 + A.sell_pos[s];
#pragma unroll
    for (int k = 0; k < 9; k++) dst[32 * k] = (float)acc[k];
    if (!fixed) {  // the cloth's range of diagonal entries (positive floats order as their bits)
      const float lo = (float)fmin(fabs(acc[0]), fmin(fabs(acc[4]), fabs(acc[8])));
      const float hi = (float)fmax(fabs(acc[0]), fmax(fabs(acc[4]), fabs(acc[8])));
      const int inst = A.vinst[v];
      atomicMin(&A.dg_range[2 * inst], __float_as_uint(lo));
      atomicMax(&A.dg_range[2 * inst + 1], __float_as_uint(hi));
    }
    // block-Jacobi scaling: L^-1 for the Cholesky factor D = L L^T of the
    // diagonal block (lower triangle of D), identity unless D is positive definite
    float* S = A.linv32 + 9 * (size_t)v;
    const double l00 = sqrt(acc[0]);
    const double l10 = acc[3] / l00, l20 = acc[6] / l00;
    const double t11 = acc[4] - l10 * l10;
    const double l11 = sqrt(t11);
    const double l21 = (acc[7] - l20 * l10) / l11;
    const double t22 = acc[8] - l20 * l20 - l21 * l21;
    const double l22 = sqrt(t22);
    if (acc[0] > 0.0 && t11 > 0.0 && t22 > 0.0 && isfinite(l22) && isfinite(l21)) {
      const double m00 = 1.0 / l00, m11 = 1.0 / l11, m22 = 1.0 / l22;
      const double m10 = -l10 * m00 * m11;
      const double m21 = -l21 * m11 * m22;
      const double m20 = -(l20 * m00 + l21 * m10) * m22;
      S[0] = (float)m00;
      S[1] = 0.f;
      S[2] = 0.f;
      S[3] = (float)m10;
      S[4] = (float)m11;
      S[5] = 0.f;
      S[6] = (float)m20;
      S[7] = (float)m21;
      S[8] = (float)m22;
    } else {
#pragma unroll
      for (int k = 0; k < 9; k++) S[k] = (k % 4 == 0) ? 1.f : 0.f;
    }
  }
}

__global__ void k_dg_reset_hi(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.ni) A.dg_range[2 * i + 1] = 0u;
}

// ordered gradient sum of vertex v: triangles, stencils (then caller's terms)
__device__ __forceinline__ void vertex_gradient(const Arena& A, int v, double g[3]) {
  g[0] = g[1] = g[2] = 0.0;
  for (int e = A.grad_ptr[v]; e < A.grad_ptr[v + 1]; e++) {
    const int code = A.grad_src[e];
    const double* src = (code >= 0) ? A.tri_grad + 3 * (size_t)code : A.quad_grad + 3 * (size_t)(-code - 1);
    g[0] += src[0];
    g[1] += src[1];
    g[2] += src[2];
  }
}

// right-hand side -grad W + m v / dt (solve_internal_sparse.h:299-313)
__global__ void k_rhs(Arena A) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  const DevParams& P = A.prm[A.vinst[v]];
  double g[3];
  vertex_gradient(A, v, g);
  {
    double p[3], W, dW[3], ddW[9];
    load3(A.x, v, p);
    contact_energy<double>(P.obstacle_kind, P.obs_center, P.obs_radius, P.stiff_contact, P.contact_clearance, p,
                           W, dW, ddW);
    g[0] += dW[0];
    g[1] += dW[1];
    g[2] += dW[2];
  }
  const bool fixed = A.bc[v] != 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    g[k] -= P.mass_point * P.gravity[k];
    const double bk = -g[k] + P.mass_point * A.v[3 * v + k] / P.dt;
    A.b[3 * v + k] = fixed ? 0.0 : bk;
  }
}

// UpdateIntermidiateVelocity (solve_internal_sparse.h:329-369) on active cloths
__global__ void k_update_velocity(Arena A) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  const int inst = A.vinst[v];
  if (!A.active[inst]) return;
  const DevParams& P = A.prm[inst];
  double g[3];
  vertex_gradient(A, v, g);
  const double f = -(0.5 * P.dt / P.mass_point);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    g[k] -= P.mass_point * P.gravity[k];
    double u = A.bc[v] ? 0.0 : A.v[3 * v + k];
    u += f * g[k];
    A.v[3 * v + k] = u;
  }
}

// MakeNormal (self_contact_sparse/main.cpp:183-211): per vertex, the unit
// normals (UnitNormalAreaTri3D, utility.h:58-73) of its triangles added in
// triangle order (the vertex's gradient sources list them ascending), then the
// sum scaled by 1 / sqrt(|sum|^2): the reference's operations, in its order.
__global__ void k_vertex_normals(Arena A, const double* xs, double* out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv || !A.active[A.vinst[v]]) return;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int e = A.grad_ptr[v]; e < A.grad_ptr[v + 1]; e++) {
    const int code = A.grad_src[e];
    if (code < 0) continue;  // a bending stencil
    const int t = code / 3;
    const double* a = xs + 3 * A.tri[3 * t];
    const double* b = xs + 3 * A.tri[3 * t + 1];
    const double* c = xs + 3 * A.tri[3 * t + 2];
    double n0 = (b[1] - a[1]) * (c[2] - a[2]) - (c[1] - a[1]) * (b[2] - a[2]);
    double n1 = (b[2] - a[2]) * (c[0] - a[0]) - (c[2] - a[2]) * (b[0] - a[0]);
    double n2 = (b[0] - a[0]) * (c[1] - a[1]) - (c[0] - a[0]) * (b[1] - a[1]);
    const double area = sqrt(n0 * n0 + n1 * n1 + n2 * n2) * 0.5;
    const double inv = 0.5 / area;
    n0 *= inv;
    n1 *= inv;
    n2 *= inv;
    s0 += n0;
    s1 += n1;
    s2 += n2;
  }
  const double sq = s0 * s0 + s1 * s1 + s2 * s2;
  const double inv = 1.0 / sqrt(sq);
  out[3 * v + 0] = s0 * inv;
  out[3 * v + 1] = s1 * inv;
  out[3 * v + 2] = s2 * inv;
}

// x += dx, v = dx / dt; a speed above kMaxSpeed (or not a number) marks the
// cloth as blown up
__global__ void k_finish_implicit(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * A.nv) return;
  const int inst = A.vinst[i / 3];
  if (!A.active[inst]) return;
  const double d = A.dx[i];
  A.x[i] += d;
  const double v = d / A.prm[inst].dt;
  A.v[i] = v;
  if (!(fabs(v) <= kMaxSpeed)) A.st[inst].diverged = 1;
}

__global__ void k_reintegrate(Arena A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * A.nv) return;
  const int inst = A.vinst[i / 3];
  if (!A.active[inst]) return;
  A.x[i] = A.x1[i] + A.v[i] * A.prm[inst].dt;
}

__global__ void k_batch_cst(int n, const double* C, const double* c, double lambda, double myu, double* W,
                            double* dW, double* ddW) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double Ce[9], ce[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    Ce[k] = C[9 * (size_t)e + k];
    ce[k] = c[9 * (size_t)e + k];
  }
  CstState<double> st;
  cst_state<double>(Ce, ce, lambda, myu, st);
  W[e] = st.W;
  double g[9];
  cst_gradient<double>(st, g);
#pragma unroll
  for (int k = 0; k < 9; k++) dW[9 * (size_t)e + k] = g[k];
  double* dst = ddW + 81 * (size_t)e;
  // element layout [a][b][i][j] is block (a, b) row-major
  store_block<0, 0>(st, dst);
  store_block<0, 1>(st, dst);
  store_block<0, 2>(st, dst);
  store_block<1, 0>(st, dst);
  store_block<1, 1>(st, dst);
  store_block<1, 2>(st, dst);
  store_block<2, 0>(st, dst);
  store_block<2, 1>(st, dst);
  store_block<2, 2>(st, dst);
}

__global__ void k_batch_bend(int n, const double* C, const double* c, double stiff, double* W, double* dW,
                             double* ddW) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double Ce[12], ce[12], K[4], s, g[12];
#pragma unroll
  for (int k = 0; k < 12; k++) {
    Ce[k] = C[12 * (size_t)e + k];
    ce[k] = c[12 * (size_t)e + k];
  }
  bend_factors<double>(Ce, stiff, K, s);
  bend_gradient<double>(K, s, ce, g);
  double w = 0;  // energy accumulated like the reference (cloth_internal_physics.h:235)
  for (int a = 0; a < 4; a++)
    for (int k = 0; k < 3; k++) w += g[a * 3 + k] * ce[a * 3 + k];
  W[e] = w;
  for (int k = 0; k < 12; k++) dW[12 * (size_t)e + k] = g[k];
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) {
      const double h = K[a] * K[b] * s;
      for (int k = 0; k < 9; k++) ddW[144 * (size_t)e + (a * 4 + b) * 9 + k] = (k % 4 == 0) ? h : 0.0;
    }
}

__global__ void k_batch_contact(int n, const double* c, DevParams P, double* W, double* dW, double* ddW) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double p[3] = {c[3 * e], c[3 * e + 1], c[3 * e + 2]};
  contact_energy<double>(P.obstacle_kind, P.obs_center, P.obs_radius, P.stiff_contact, P.contact_clearance, p,
                         W[e], dW + 3 * e, ddW + 9 * e);
}

}  // namespace

void launch_quad_factors(const Arena& A, cudaStream_t s) {
  if (A.nq == 0) return;
  k_quad_factors<<<blocks_for(A.nq), kThreads, 0, s>>>(A);
  g_launches++;
}

void launch_elements(const Arena& A, bool hess, bool masked, cudaStream_t s) {
  prof_begin(PK_TRI_ELEMENTS, s);
  k_tri_elements<<<blocks_for(A.nt), kThreads, 0, s>>>(A, hess ? 1 : 0, masked ? 1 : 0);
  prof_end(PK_TRI_ELEMENTS, s);
  g_launches++;
  if (A.nq) {
    k_quad_grad<<<blocks_for(A.nq), kThreads, 0, s>>>(A, masked ? 1 : 0);
    g_launches++;
  }
}

void launch_slot_reduce(const Arena& A, cudaStream_t s) {
  if (A.mixed) {
    // smallest entry starts at a large positive float (0x7f7f7f7f), largest at 0
    cudaMemsetAsync(A.dg_range, 0x7f, 2 * sizeof(unsigned) * (size_t)A.ni, s);
    k_dg_reset_hi<<<blocks_for(A.ni), kThreads, 0, s>>>(A);
    g_launches++;
  }
  prof_begin(PK_SLOT_REDUCE, s);
  k_slot_reduce<<<blocks_for(A.nb + A.nv), kThreads, 0, s>>>(A);
  prof_end(PK_SLOT_REDUCE, s);
  g_launches++;
}

void launch_rhs(const Arena& A, cudaStream_t s) {
  prof_begin(PK_RHS, s);
  k_rhs<<<blocks_for(A.nv), kThreads, 0, s>>>(A);
  prof_end(PK_RHS, s);
  g_launches++;
}

void launch_update_velocity(const Arena& A, cudaStream_t s) {
  k_update_velocity<<<blocks_for(A.nv), kThreads, 0, s>>>(A);
  g_launches++;
}

void launch_finish_implicit(const Arena& A, cudaStream_t s) {
  k_finish_implicit<<<blocks_for(3LL * A.nv), kThreads, 0, s>>>(A);
  g_launches++;
}

void launch_vertex_normals(const Arena& A, const double* xs, double* out, cudaStream_t s) {
  k_vertex_normals<<<blocks_for(A.nv), kThreads, 0, s>>>(A, xs, out);
  g_launches++;
}

void launch_reintegrate(const Arena& A, cudaStream_t s) {
  k_reintegrate<<<blocks_for(3LL * A.nv), kThreads, 0, s>>>(A);
  g_launches++;
}

void launch_element_batch_cst(int n, const double* C, const double* c, double lambda, double myu, double* W,
                              double* dW, double* ddW, cudaStream_t s) {
  k_batch_cst<<<blocks_for(n), kThreads, 0, s>>>(n, C, c, lambda, myu, W, dW, ddW);
  g_launches++;
}

void launch_element_batch_bend(int n, const double* C, const double* c, double stiff, double* W, double* dW,
                               double* ddW, cudaStream_t s) {
  k_batch_bend<<<blocks_for(n), kThreads, 0, s>>>(n, C, c, stiff, W, dW, ddW);
  g_launches++;
}

void launch_element_batch_contact(int n, const double* c, const DevParams* prm, double* W, double* dW,
                                  double* ddW, cudaStream_t s) {
  k_batch_contact<<<blocks_for(n), kThreads, 0, s>>>(n, c, *prm, W, dW, ddW);
  g_launches++;
}

}  // namespace cs
