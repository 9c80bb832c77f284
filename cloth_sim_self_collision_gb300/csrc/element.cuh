// element.cuh -- per-element energy, gradient and Hessian of the cloth
// (cloth_internal_physics.h of the reference), templated on the arithmetic type.
// In double precision with -fmad=false they round exactly like the reference.
#pragma once
#include "geom.cuh"

namespace cs {

// 2x2 symmetric stress (xx, yy, xy) clamped to its positive semi-definite part
// (MakePositiveDefinite_Sim22, cloth_internal_physics.h:15-67).
template <typename T>
CS_HD void psd_clamp_sym22(const T s[3], T out[3]) {
  const T b = (s[0] + s[1]) * T(0.5);
  const T d = (s[0] - s[1]) * (s[0] - s[1]) * T(0.25) + s[2] * s[2];
  const T e = sqrt(d);
  if (b - e > T(1.0e-20)) {
    out[0] = s[0];
    out[1] = s[1];
    out[2] = s[2];
    return;
  }
  if (b + e < 0) {
    out[0] = out[1] = out[2] = 0;
    return;
  }
  const T l = b + e;
  const T a0 = s[0] - l, a1 = s[2];
  const T c0 = s[2], c1 = s[1] - l;
  const T sq0 = a0 * a0 + a1 * a1;
  const T sq1 = c0 * c0 + c1 * c1;
  T u0, u1;
  if (sq0 > sq1) {
    if (sq0 < T(1.0e-20)) {
      out[0] = out[1] = out[2] = 0;
      return;
    }
    const T inv = T(1) / sqrt(sq0);
    u0 = a0 * inv;
    u1 = a1 * inv;
  } else {
    if (sq1 < T(1.0e-20)) {
      out[0] = out[1] = out[2] = 0;
      return;
    }
    const T inv = T(1) / sqrt(sq1);
    u0 = c0 * inv;
    u1 = c1 * inv;
  }
  out[0] = l * u0 * u0;
  out[1] = l * u1 * u1;
  out[2] = l * u0 * u1;
}

// Per-triangle quantities of the St.Venant-Kirchhoff CST shared by its
// gradient and all nine Hessian blocks (WdWddW_CST, cloth_internal_physics.h:70-134).
template <typename T>
struct CstState {
  T area;
  T d[2][3];   // deformed edge vectors
  T Cm[3][3];  // constitutive matrix in the triangle's chart
  T S[3];      // 2nd Piola-Kirchhoff stress (xx, yy, xy)
  T Sp[3];     // its positive part
  T W;
};

template <typename T>
CS_HD void cst_state(const T C[9], const T c[9], T lambda, T myu, CstState<T>& st) {
  T D0[3], D1[3], N[3], G0[3], G1[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    D0[k] = C[3 + k] - C[k];
    D1[k] = C[6 + k] - C[k];
  }
  // UnitNormalAreaTri3D (utility.h:58-73)
  N[0] = (C[4] - C[1]) * (C[8] - C[2]) - (C[7] - C[1]) * (C[5] - C[2]);
  N[1] = (C[5] - C[2]) * (C[6] - C[0]) - (C[8] - C[2]) * (C[3] - C[0]);
  N[2] = (C[3] - C[0]) * (C[7] - C[1]) - (C[6] - C[0]) * (C[4] - C[1]);
  const T area = sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]) * T(0.5);
  {
    const T inv = T(0.5) / area;
    N[0] *= inv;
    N[1] *= inv;
    N[2] *= inv;
  }
  // Cross3D (utility.h:22-26)
  G0[0] = D1[1] * N[2] - N[1] * D1[2];
  G0[1] = D1[2] * N[0] - N[2] * D1[0];
  G0[2] = D1[0] * N[1] - N[0] * D1[1];
  {
    const T s = T(1) / (G0[0] * D0[0] + G0[1] * D0[1] + G0[2] * D0[2]);
    G0[0] *= s;
    G0[1] *= s;
    G0[2] *= s;
  }
  G1[0] = N[1] * D0[2] - D0[1] * N[2];
  G1[1] = N[2] * D0[0] - D0[2] * N[0];
  G1[2] = N[0] * D0[1] - D0[0] * N[1];
  {
    const T s = T(1) / (G1[0] * D1[0] + G1[1] * D1[1] + G1[2] * D1[2]);
    G1[0] *= s;
    G1[1] *= s;
    G1[2] *= s;
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    st.d[0][k] = c[3 + k] - c[k];
    st.d[1][k] = c[6 + k] - c[k];
  }
  const T(&d)[2][3] = st.d;
  const T E0 = T(0.5) * ((d[0][0] * d[0][0] + d[0][1] * d[0][1] + d[0][2] * d[0][2]) -
                         (D0[0] * D0[0] + D0[1] * D0[1] + D0[2] * D0[2]));
  const T E1 = T(0.5) * ((d[1][0] * d[1][0] + d[1][1] * d[1][1] + d[1][2] * d[1][2]) -
                         (D1[0] * D1[0] + D1[1] * D1[1] + D1[2] * D1[2]));
  const T E2 = T(1.0) * ((d[0][0] * d[1][0] + d[0][1] * d[1][1] + d[0][2] * d[1][2]) -
                         (D0[0] * D1[0] + D0[1] * D1[1] + D0[2] * D1[2]));
  const T g0 = G0[0] * G0[0] + G0[1] * G0[1] + G0[2] * G0[2];
  const T g1 = G1[0] * G1[0] + G1[1] * G1[1] + G1[2] * G1[2];
  const T g2 = G1[0] * G0[0] + G1[1] * G0[1] + G1[2] * G0[2];
  st.Cm[0][0] = lambda * g0 * g0 + 2 * myu * (g0 * g0);
  st.Cm[0][1] = lambda * g0 * g1 + 2 * myu * (g2 * g2);
  st.Cm[0][2] = lambda * g0 * g2 + 2 * myu * (g0 * g2);
  st.Cm[1][0] = lambda * g1 * g0 + 2 * myu * (g2 * g2);
  st.Cm[1][1] = lambda * g1 * g1 + 2 * myu * (g1 * g1);
  st.Cm[1][2] = lambda * g1 * g2 + 2 * myu * (g2 * g1);
  st.Cm[2][0] = lambda * g2 * g0 + 2 * myu * (g0 * g2);
  st.Cm[2][1] = lambda * g2 * g1 + 2 * myu * (g2 * g1);
  st.Cm[2][2] = lambda * g2 * g2 + 1 * myu * (g0 * g1 + g2 * g2);
#pragma unroll
  for (int i = 0; i < 3; i++) st.S[i] = st.Cm[i][0] * E0 + st.Cm[i][1] * E1 + st.Cm[i][2] * E2;
  st.W = T(0.5) * area * (E0 * st.S[0] + E1 * st.S[1] + E2 * st.S[2]);
  st.area = area;
  psd_clamp_sym22(st.S, st.Sp);
}

// gradient rows of the CST (cloth_internal_physics.h:118-128).  The chart
// gradients of the three shape functions are (-1,-1), (1,0), (0,1); the sums
// below are the reference's four terms with those factors applied exactly.
template <typename T>
CS_HD void cst_gradient(const CstState<T>& st, T dW[9]) {
  const T(&d)[2][3] = st.d;
  const T* S = st.S;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const T a = S[0] * d[0][k], b = S[2] * d[0][k], c = S[2] * d[1][k], e = S[1] * d[1][k];
    // vertex 0: (-a) + (-b) + (-c) + (-e)
    dW[0 * 3 + k] = st.area * (((-a) + (-b)) + (-c) + (-e));
    // vertex 1: a + 0*b + c + 0*e
    dW[1 * 3 + k] = st.area * (((a + b * T(0)) + c) + e * T(0));
    // vertex 2: 0*a + b + 0*c + e
    dW[2 * 3 + k] = st.area * (((a * T(0) + b) + c * T(0)) + e);
  }
}

// chart gradient components of the linear triangle (cloth_internal_physics.h:98)
__host__ __device__ constexpr int dn(int vertex, int axis) {
  return vertex == 0 ? -1 : ((vertex == 1) == (axis == 0) ? 1 : 0);
}

// One 3x3 Hessian block (a, b) of the CST (cloth_internal_physics.h:136-174):
// the 16 material products of the reference in its order (terms whose chart
// factor is 0 contribute an exact zero and are skipped), times the area, plus
// the geometric stiffness on the diagonal.
template <typename T, int A, int B>
CS_HD void cst_hessian_block(const CstState<T>& st, T out[9]) {
  const T(&d)[2][3] = st.d;
  const T(&Cm)[3][3] = st.Cm;
  // {edge a, chart index of N_A, C row, C col, edge b, chart index of N_B}
  constexpr int terms[16][6] = {{0, 0, 0, 0, 0, 0}, {0, 0, 0, 1, 1, 1}, {0, 0, 0, 2, 0, 1}, {0, 0, 0, 2, 1, 0},
                                {1, 1, 1, 0, 0, 0}, {1, 1, 1, 1, 1, 1}, {1, 1, 1, 2, 0, 1}, {1, 1, 1, 2, 1, 0},
                                {0, 1, 2, 0, 0, 0}, {0, 1, 2, 1, 1, 1}, {0, 1, 2, 2, 0, 1}, {0, 1, 2, 2, 1, 0},
                                {1, 0, 2, 0, 0, 0}, {1, 0, 2, 1, 1, 1}, {1, 0, 2, 2, 0, 1}, {1, 0, 2, 2, 1, 0}};
#pragma unroll
  for (int i = 0; i < 3; i++) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
      T acc = 0;
#pragma unroll
      for (int t = 0; t < 16; t++) {
        const int sa = dn(A, terms[t][1]), sb = dn(B, terms[t][5]);
        if (sa == 0 || sb == 0) continue;
        // ((d_a * sa) * C) * d_b * sb with sa, sb = +-1: an exact sign flip
        const T m = (d[terms[t][0]][i] * Cm[terms[t][2]][terms[t][3]]) * d[terms[t][4]][j];
        acc += (sa * sb > 0) ? m : -m;
      }
      out[i * 3 + j] = acc * st.area;
    }
  }
  // geometric term, area * (Sp0 N_A0 N_B0 + Sp2 N_A0 N_B1 + Sp2 N_A1 N_B0 + Sp1 N_A1 N_B1)
  T g = 0;
  {
    const T* Sp = st.Sp;
    const T t0 = Sp[0] * T(dn(A, 0)) * T(dn(B, 0));
    const T t1 = Sp[2] * T(dn(A, 0)) * T(dn(B, 1));
    const T t2 = Sp[2] * T(dn(A, 1)) * T(dn(B, 0));
    const T t3 = Sp[1] * T(dn(A, 1)) * T(dn(B, 1));
    g = st.area * (((t0 + t1) + t2) + t3);
  }
  out[0] += g;
  out[4] += g;
  out[8] += g;
}

template <typename T>
CS_HD void cst_hessian_block_rt(const CstState<T>& st, int a, int b, T out[9]) {
  switch (a * 3 + b) {
    case 0: cst_hessian_block<T, 0, 0>(st, out); break;
    case 1: cst_hessian_block<T, 0, 1>(st, out); break;
    case 2: cst_hessian_block<T, 0, 2>(st, out); break;
    case 3: cst_hessian_block<T, 1, 0>(st, out); break;
    case 4: cst_hessian_block<T, 1, 1>(st, out); break;
    case 5: cst_hessian_block<T, 1, 2>(st, out); break;
    case 6: cst_hessian_block<T, 2, 0>(st, out); break;
    case 7: cst_hessian_block<T, 2, 1>(st, out); break;
    default: cst_hessian_block<T, 2, 2>(st, out); break;
  }
}

// Rest-shape factors of a bending stencil (WdWddW_Bend, cloth_internal_physics.h:187-212):
// cotangent weights K[4] and scale = stiff / ((A0 + A1) L0^2).  The Hessian is
// K_a K_b scale I3 and does not depend on the deformed shape.
template <typename T>
CS_HD void bend_factors(const T C[12], T stiff, T K[4], T& scale) {
  const T *C0 = C, *C1 = C + 3, *C2 = C + 6, *C3 = C + 9;
  auto tri_area = [](const T* a, const T* b, const T* c) {
    const T n0 = (b[1] - a[1]) * (c[2] - a[2]) - (c[1] - a[1]) * (b[2] - a[2]);
    const T n1 = (b[2] - a[2]) * (c[0] - a[0]) - (c[2] - a[2]) * (b[0] - a[0]);
    const T n2 = (b[0] - a[0]) * (c[1] - a[1]) - (c[0] - a[0]) * (b[1] - a[1]);
    return sqrt(n0 * n0 + n1 * n1 + n2 * n2) * T(0.5);
  };
  const T A0 = tri_area(C0, C2, C3);
  const T A1 = tri_area(C1, C3, C2);
  const T L0 = sqrt((C3[0] - C2[0]) * (C3[0] - C2[0]) + (C3[1] - C2[1]) * (C3[1] - C2[1]) +
                    (C3[2] - C2[2]) * (C3[2] - C2[2]));
  const T H0 = A0 * T(2.0) / L0;
  const T H1 = A1 * T(2.0) / L0;
  T e23[3], e02[3], e03[3], e12[3], e13[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    e23[k] = C3[k] - C2[k];
    e02[k] = C2[k] - C0[k];
    e03[k] = C3[k] - C0[k];
    e12[k] = C2[k] - C1[k];
    e13[k] = C3[k] - C1[k];
  }
  auto d3 = [](const T* a, const T* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  const T cot023 = -d3(e02, e23) / H0;
  const T cot032 = +d3(e03, e23) / H0;
  const T cot123 = -d3(e12, e23) / H1;
  const T cot132 = +d3(e13, e23) / H1;
  scale = stiff / ((A0 + A1) * L0 * L0);
  K[0] = -cot023 - cot032;
  K[1] = -cot123 - cot132;
  K[2] = cot032 + cot132;
  K[3] = cot023 + cot123;
}

// Bending gradient H c (cloth_internal_physics.h:226-237): for component k of
// vertex a, the reference sums (K_a K_b s) c_b[k] over b in order, with exact
// zeros from the off-diagonal entries of each 3x3 block.
template <typename T>
CS_HD void bend_gradient(const T K[4], T scale, const T c[12], T dW[12]) {
#pragma unroll
  for (int a = 0; a < 4; a++) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      T g = 0;
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const T h = K[a] * K[b] * scale;
#pragma unroll
        for (int j = 0; j < 3; j++) g += (j == k ? h : T(0)) * c[b * 3 + j];
      }
      dW[a * 3 + k] = g;
    }
  }
}

// Obstacle penetration depth and normal at p (replaces the reference's
// penetrationDepth callbacks, self_contact_sparse/main.cpp:110-133).
// kind: 0 none, 1 plane z = c[2], 2 solid sphere, 3 inside-out sphere.
template <typename T>
CS_HD bool obstacle_depth(int kind, const T c[3], T radius, const T p[3], T& pd, T n[3]) {
  if (kind == 1) {
    n[0] = 0.0;
    n[1] = 0.0;
    n[2] = 1.0;
    pd = c[2] - p[2];
    return true;
  }
  if (kind == 2 || kind == 3) {
    n[0] = p[0] - c[0];
    n[1] = p[1] - c[1];
    n[2] = p[2] - c[2];
    const T len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] /= len;
    n[1] /= len;
    n[2] /= len;
    pd = radius - len;
    if (kind == 3) {
      n[0] *= -1;
      n[1] *= -1;
      n[2] *= -1;
      pd *= -1;
    }
    return true;
  }
  return false;
}

// Penalty contact with the obstacle (WdWddW_Contact, cloth_internal_physics.h:243-280).
template <typename T>
CS_HD void contact_energy(int kind, const T oc[3], T radius, T stiff, T clearance, const T p[3], T& W, T dW[3],
                          T ddW[9]) {
  T pd, n[3];
  if (!obstacle_depth(kind, oc, radius, p, pd, n)) pd = T(-1.0e30);
  pd += clearance;
  if (pd < 0) {
    W = 0;
    dW[0] = dW[1] = dW[2] = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) ddW[i] = 0;
    return;
  }
  W = T(0.5) * stiff * pd * pd;
#pragma unroll
  for (int i = 0; i < 3; i++) dW[i] = -stiff * pd * n[i];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) ddW[i * 3 + j] = stiff * n[i] * n[j];
}

}  // namespace cs
