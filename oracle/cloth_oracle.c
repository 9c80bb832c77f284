/*
 * cloth_oracle.c -- TEST INFRASTRUCTURE ONLY (see cloth_oracle.h).
 *
 * Plain-C FP64 restatement of the reference's self_contact_sparse step.  The
 * arithmetic of every floating-point expression keeps the reference's operand
 * order and association (C evaluates left to right), so that with IEEE double
 * and no FMA contraction the results agree bit for bit with the reference
 * compiled from its own sources (oracle/ref_driver.cpp).  Data structures are
 * this file's own: flat arrays, a sorted-merge contact set in place of
 * std::set, a per-vertex zone table in place of std::vector<std::set<int>>.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cloth_oracle.h"

/* ======================================================================== */
/* 3-vectors (vector3d.h:33-297, utility.h:15-73)                            */
/* ======================================================================== */
typedef struct {
  double x, y, z;
} vec3;

static vec3 mk(double x, double y, double z) {
  vec3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
static vec3 at(const double *a, int i) { return mk(a[i * 3 + 0], a[i * 3 + 1], a[i * 3 + 2]); }
static vec3 add(vec3 a, vec3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static vec3 sub(vec3 a, vec3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
/* scalar * vector multiplies each component (vector3d.h:143-148) */
static vec3 scl(double s, vec3 a) { return mk(a.x * s, a.y * s, a.z * s); }
static double dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static vec3 cross(vec3 a, vec3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static double len3(vec3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
/* SetNormalizedVector multiplies by the reciprocal length (vector3d.h:96-102) */
static vec3 normalized(vec3 a) {
  const double inv = 1.0 / len3(a);
  return mk(a.x * inv, a.y * inv, a.z * inv);
}
/* operator/= skips tiny divisors (vector3d.h:63-67) */
static vec3 div_guarded(vec3 a, double d) {
  if (fabs(d) < 1.e-16) return a;
  return mk(a.x / d, a.y / d, a.z / d);
}
/* ScalarTripleProduct, vector3d.h:216-218 */
static double stp(vec3 a, vec3 b, vec3 c) {
  return a.x * (b.y * c.z - b.z * c.y) + a.y * (b.z * c.x - b.x * c.z) + a.z * (b.x * c.y - b.y * c.x);
}
/* Height of v4 over the plane of v1 v2 v3, vector3d.h:254-267 */
static double height4(vec3 v1, vec3 v2, vec3 v3, vec3 v4) {
  double nx = (v2.y - v1.y) * (v3.z - v1.z) - (v2.z - v1.z) * (v3.y - v1.y);
  double ny = (v2.z - v1.z) * (v3.x - v1.x) - (v2.x - v1.x) * (v3.z - v1.z);
  double nz = (v2.x - v1.x) * (v3.y - v1.y) - (v2.y - v1.y) * (v3.x - v1.x);
  const double inv = 1.0 / sqrt(nx * nx + ny * ny + nz * nz);
  nx *= inv;
  ny *= inv;
  nz *= inv;
  return (v4.x - v1.x) * nx + (v4.y - v1.y) * ny + (v4.z - v1.z) * nz;
}
/* closest point of segment s-e to p, vector3d.h:282-295 */
static vec3 closest_on_segment(vec3 p, vec3 s, vec3 e) {
  const vec3 d = sub(e, s);
  const double a = dot(d, d);
  const double b = dot(d, sub(s, p));
  double t = -b / a;
  if (t < 0) t = 0;
  if (t > 1) t = 1;
  return add(s, scl(t, d));
}

/* array forms, utility.h:15-73 */
static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void cross3(double *r, const double *u, const double *v) {
  r[0] = u[1] * v[2] - v[1] * u[2];
  r[1] = u[2] * v[0] - v[2] * u[0];
  r[2] = u[0] * v[1] - v[0] * u[1];
}
static double dist3(const double *a, const double *b) {
  const double t = (b[0] - a[0]) * (b[0] - a[0]) + (b[1] - a[1]) * (b[1] - a[1]) + (b[2] - a[2]) * (b[2] - a[2]);
  return sqrt(t);
}
static void tri_normal_raw(double *n, const double *a, const double *b, const double *c) {
  n[0] = (b[1] - a[1]) * (c[2] - a[2]) - (c[1] - a[1]) * (b[2] - a[2]);
  n[1] = (b[2] - a[2]) * (c[0] - a[0]) - (c[2] - a[2]) * (b[0] - a[0]);
  n[2] = (b[0] - a[0]) * (c[1] - a[1]) - (c[0] - a[0]) * (b[1] - a[1]);
}
static double tri_area3(const double *a, const double *b, const double *c) {
  double n[3];
  tri_normal_raw(n, a, b, c);
  return sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) * 0.5;
}
static void unit_normal_area3(double *n, double *area, const double *a, const double *b, const double *c) {
  tri_normal_raw(n, a, b, c);
  *area = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) * 0.5;
  const double inv = 0.5 / *area;
  n[0] *= inv;
  n[1] *= inv;
  n[2] *= inv;
}

/* ======================================================================== */
/* axis-aligned boxes (aabb.h:16-148): 6 bounds + a non-empty flag           */
/* ======================================================================== */
typedef struct {
  double lo[3], hi[3];
  int full;
} box3;

static void box_clear(box3 *b) {
  memset(b, 0, sizeof(*b));
}
/* AddPoint(x,y,z,eps), aabb.h:102-122 */
static void box_add_point(box3 *b, vec3 p, double eps) {
  const double q[3] = {p.x, p.y, p.z};
  int k;
  if (eps <= 0) return;
  if (b->full) {
    for (k = 0; k < 3; k++) {
      b->lo[k] = (b->lo[k] < q[k] - eps) ? b->lo[k] : q[k] - eps;
      b->hi[k] = (b->hi[k] > q[k] + eps) ? b->hi[k] : q[k] + eps;
    }
  } else {
    b->full = 1;
    for (k = 0; k < 3; k++) {
      b->lo[k] = q[k] - eps;
      b->hi[k] = q[k] + eps;
    }
  }
}
/* operator+=(box), aabb.h:55-72 */
static void box_merge(box3 *b, const box3 *o) {
  int k;
  if (!o->full) return;
  if (!b->full) {
    *b = *o;
    return;
  }
  for (k = 0; k < 3; k++) {
    b->hi[k] = (b->hi[k] > o->hi[k]) ? b->hi[k] : o->hi[k];
    b->lo[k] = (b->lo[k] < o->lo[k]) ? b->lo[k] : o->lo[k];
  }
}
/* IsIntersect, aabb.h:73-84 (closed intervals) */
static int box_overlap(const box3 *a, const box3 *b) {
  int k;
  if (!a->full || !b->full) return 0;
  for (k = 0; k < 3; k++) {
    if (a->hi[k] < b->lo[k]) return 0;
    if (a->lo[k] > b->hi[k]) return 0;
  }
  return 1;
}
/* IsInside, aabb.h:137-144 */
static int box_inside(const box3 *b, vec3 p) {
  if (!b->full) return 0;
  return p.x >= b->lo[0] && p.x <= b->hi[0] && p.y >= b->lo[1] && p.y <= b->hi[1] && p.z >= b->lo[2] &&
         p.z <= b->hi[2];
}

/* ======================================================================== */
/* element energies (cloth_internal_physics.h)                               */
/* ======================================================================== */

/* 2x2 symmetric stress (xx, yy, xy) clamped to its non-negative part,
 * MakePositiveDefinite_Sim22, cloth_internal_physics.h:15-67 */
static void psd_clamp_sym22(const double s[3], double out[3]) {
  const double b = (s[0] + s[1]) * 0.5;
  const double d = (s[0] - s[1]) * (s[0] - s[1]) * 0.25 + s[2] * s[2];
  const double e = sqrt(d);
  double l, u0, u1, sq0, sq1;
  if (b - e > 1.0e-20) {
    out[0] = s[0];
    out[1] = s[1];
    out[2] = s[2];
    return;
  }
  if (b + e < 0) {
    out[0] = out[1] = out[2] = 0;
    return;
  }
  l = b + e;
  {
    double a0 = s[0] - l, a1 = s[2]; /* first row of (S - l I) */
    double c0 = s[2], c1 = s[1] - l; /* second row            */
    sq0 = a0 * a0 + a1 * a1;
    sq1 = c0 * c0 + c1 * c1;
    if (sq0 > sq1) {
      if (sq0 < 1.0e-20) {
        out[0] = out[1] = out[2] = 0;
        return;
      }
      const double inv = 1.0 / sqrt(sq0);
      u0 = a0 * inv;
      u1 = a1 * inv;
    } else {
      if (sq1 < 1.0e-20) {
        out[0] = out[1] = out[2] = 0;
        return;
      }
      const double inv = 1.0 / sqrt(sq1);
      u0 = c0 * inv;
      u1 = c1 * inv;
    }
  }
  out[0] = l * u0 * u0;
  out[1] = l * u1 * u1;
  out[2] = l * u0 * u1;
}

/* shape-function gradients of the linear triangle in its (r0, r1) chart */
static const double kDN[3][2] = {{-1.0, -1.0}, {+1.0, +0.0}, {+0.0, +1.0}};

/* The 16 material-stiffness products of one Hessian entry, in the order the
 * reference sums them (cloth_internal_physics.h:146-161): each row is
 * {edge a, chart index of N_i, C row, C col, edge b, chart index of N_j}. */
static const int kCstTerms[16][6] = {
    {0, 0, 0, 0, 0, 0}, {0, 0, 0, 1, 1, 1}, {0, 0, 0, 2, 0, 1}, {0, 0, 0, 2, 1, 0},
    {1, 1, 1, 0, 0, 0}, {1, 1, 1, 1, 1, 1}, {1, 1, 1, 2, 0, 1}, {1, 1, 1, 2, 1, 0},
    {0, 1, 2, 0, 0, 0}, {0, 1, 2, 1, 1, 1}, {0, 1, 2, 2, 0, 1}, {0, 1, 2, 2, 1, 0},
    {1, 0, 2, 0, 0, 0}, {1, 0, 2, 1, 1, 1}, {1, 0, 2, 2, 0, 1}, {1, 0, 2, 2, 1, 0}};

/* St.Venant-Kirchhoff constant-strain triangle: energy, gradient (3x3) and
 * Hessian (3x3 blocks of 3x3), WdWddW_CST, cloth_internal_physics.h:70-176.
 * C, c: rest / current vertex positions, row-major [vertex][xyz]. */
void co_wdwddw_cst(const double C[9], const double c[9], double lambda, double myu, double *W,
                   double dW[9], double ddW[81]) {
  double D0[3], D1[3], Nrm[3], area, G0[3], G1[3], d[2][3];
  int k, i, j, a, b;
  for (k = 0; k < 3; k++) {
    D0[k] = C[3 + k] - C[k];
    D1[k] = C[6 + k] - C[k];
  }
  unit_normal_area3(Nrm, &area, C, C + 3, C + 6);
  cross3(G0, D1, Nrm);
  {
    const double s = 1.0 / dot3(G0, D0);
    G0[0] *= s;
    G0[1] *= s;
    G0[2] *= s;
  }
  cross3(G1, Nrm, D0);
  {
    const double s = 1.0 / dot3(G1, D1);
    G1[0] *= s;
    G1[1] *= s;
    G1[2] *= s;
  }
  for (k = 0; k < 3; k++) {
    d[0][k] = c[3 + k] - c[k];
    d[1][k] = c[6 + k] - c[k];
  }
  /* Green strain in engineering notation (xx, yy, 2xy) */
  const double E[3] = {0.5 * (dot3(d[0], d[0]) - dot3(D0, D0)), 0.5 * (dot3(d[1], d[1]) - dot3(D1, D1)),
                       1.0 * (dot3(d[0], d[1]) - dot3(D0, D1))};
  const double g0 = dot3(G0, G0), g1 = dot3(G1, G1), g2 = dot3(G1, G0);
  const double Cm[3][3] = {
      {lambda * g0 * g0 + 2 * myu * (g0 * g0), lambda * g0 * g1 + 2 * myu * (g2 * g2),
       lambda * g0 * g2 + 2 * myu * (g0 * g2)},
      {lambda * g1 * g0 + 2 * myu * (g2 * g2), lambda * g1 * g1 + 2 * myu * (g1 * g1),
       lambda * g1 * g2 + 2 * myu * (g2 * g1)},
      {lambda * g2 * g0 + 2 * myu * (g0 * g2), lambda * g2 * g1 + 2 * myu * (g2 * g1),
       lambda * g2 * g2 + 1 * myu * (g0 * g1 + g2 * g2)}};
  double S[3], Sp[3];
  for (i = 0; i < 3; i++) S[i] = Cm[i][0] * E[0] + Cm[i][1] * E[1] + Cm[i][2] * E[2];
  *W = 0.5 * area * (E[0] * S[0] + E[1] * S[1] + E[2] * S[2]);
  for (a = 0; a < 3; a++)
    for (k = 0; k < 3; k++)
      dW[a * 3 + k] = area * (+S[0] * d[0][k] * kDN[a][0] + S[2] * d[0][k] * kDN[a][1] +
                              S[2] * d[1][k] * kDN[a][0] + S[1] * d[1][k] * kDN[a][1]);
  psd_clamp_sym22(S, Sp);
  for (a = 0; a < 3; a++) {
    for (b = 0; b < 3; b++) {
      for (i = 0; i < 3; i++) {
        for (j = 0; j < 3; j++) {
          double acc = 0;
          int t;
          for (t = 0; t < 16; t++) {
            const int *q = kCstTerms[t];
            acc += d[q[0]][i] * kDN[a][q[1]] * Cm[q[2]][q[3]] * d[q[4]][j] * kDN[b][q[5]];
          }
          ddW[((a * 3 + b) * 3 + i) * 3 + j] = acc * area;
        }
      }
      const double geo = area * (+Sp[0] * kDN[a][0] * kDN[b][0] + Sp[2] * kDN[a][0] * kDN[b][1] +
                                 Sp[2] * kDN[a][1] * kDN[b][0] + Sp[1] * kDN[a][1] * kDN[b][1]);
      for (i = 0; i < 3; i++) ddW[((a * 3 + b) * 3 + i) * 3 + i] += geo;
    }
  }
}

/* Rest-shape factors of a bending stencil: the four cotangent weights K and
 * the scale stiff/((A0+A1) L0^2), WdWddW_Bend, cloth_internal_physics.h:187-212. */
static void bend_factors(const double C[12], double stiff, double K[4], double *scale) {
  const double *C0 = C, *C1 = C + 3, *C2 = C + 6, *C3 = C + 9;
  const double A0 = tri_area3(C0, C2, C3);
  const double A1 = tri_area3(C1, C3, C2);
  const double L0 = dist3(C2, C3);
  const double H0 = A0 * 2.0 / L0;
  const double H1 = A1 * 2.0 / L0;
  double e23[3], e02[3], e03[3], e12[3], e13[3];
  int k;
  for (k = 0; k < 3; k++) {
    e23[k] = C3[k] - C2[k];
    e02[k] = C2[k] - C0[k];
    e03[k] = C3[k] - C0[k];
    e12[k] = C2[k] - C1[k];
    e13[k] = C3[k] - C1[k];
  }
  const double cot023 = -dot3(e02, e23) / H0;
  const double cot032 = +dot3(e03, e23) / H0;
  const double cot123 = -dot3(e12, e23) / H1;
  const double cot132 = +dot3(e13, e23) / H1;
  *scale = stiff / ((A0 + A1) * L0 * L0);
  K[0] = -cot023 - cot032;
  K[1] = -cot123 - cot132;
  K[2] = cot032 + cot132;
  K[3] = cot023 + cot123;
}

/* Dihedral bending: constant Hessian (K K^T scale) x I3, gradient H c,
 * WdWddW_Bend, cloth_internal_physics.h:180-238.  W accumulates like the
 * reference (the caller clears it). */
void co_wdwddw_bend(const double C[12], const double c[12], double stiff, double *W, double dW[12],
                    double ddW[144]) {
  double K[4], s;
  int a, b, i, j;
  bend_factors(C, stiff, K, &s);
  memset(ddW, 0, sizeof(double) * 144);
  for (a = 0; a < 4; a++)
    for (b = 0; b < 4; b++) {
      const double h = K[a] * K[b] * s;
      for (i = 0; i < 3; i++) ddW[((a * 4 + b) * 3 + i) * 3 + i] = h;
    }
  for (a = 0; a < 4; a++)
    for (i = 0; i < 3; i++) {
      double g = 0;
      for (b = 0; b < 4; b++)
        for (j = 0; j < 3; j++) g += ddW[((a * 4 + b) * 3 + i) * 3 + j] * c[b * 3 + j];
      dW[a * 3 + i] = g;
      *W += g * c[a * 3 + i];
    }
}

/* Penetration depth and outward normal of the obstacle at p; restates the
 * callbacks of self_contact_sparse/main.cpp:110-133 (plane, inside-out sphere)
 * plus a solid sphere.  Returns 0 when there is no obstacle. */
static int obstacle_depth(const co_params *prm, const double *p, double *pd, double n[3]) {
  const double *c = prm->obs_center;
  double len;
  switch (prm->obstacle_kind) {
    case CO_OBSTACLE_PLANE_Z:
      n[0] = 0.0;
      n[1] = 0.0;
      n[2] = 1.0;
      *pd = c[2] - p[2];
      return 1;
    case CO_OBSTACLE_SPHERE_SOLID:
    case CO_OBSTACLE_SPHERE_HOLLOW:
      n[0] = p[0] - c[0];
      n[1] = p[1] - c[1];
      n[2] = p[2] - c[2];
      len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      n[0] /= len;
      n[1] /= len;
      n[2] /= len;
      *pd = prm->obs_radius - len;
      if (prm->obstacle_kind == CO_OBSTACLE_SPHERE_HOLLOW) {
        n[0] *= -1;
        n[1] *= -1;
        n[2] *= -1;
        *pd *= -1;
      }
      return 1;
    default:
      return 0;
  }
}

/* Penalty contact with the obstacle, WdWddW_Contact, cloth_internal_physics.h:243-280 */
void co_wdwddw_contact(const double c[3], const co_params *prm, double *W, double dW[3], double ddW[9]) {
  double pd, n[3];
  const double k = prm->stiff_contact;
  int i, j;
  if (!obstacle_depth(prm, c, &pd, n)) pd = -1.0e300;
  pd += prm->contact_clearance;
  if (pd < 0) {
    *W = 0;
    for (i = 0; i < 3; i++) dW[i] = 0;
    for (i = 0; i < 9; i++) ddW[i] = 0;
    return;
  }
  *W = 0.5 * k * pd * pd;
  for (i = 0; i < 3; i++) dW[i] = -k * pd * n[i];
  for (i = 0; i < 3; i++)
    for (j = 0; j < 3; j++) ddW[i * 3 + j] = k * n[i] * n[j];
}

/* ======================================================================== */
/* the cloth object                                                          */
/* ======================================================================== */
typedef struct {
  int *mem; /* member vertices, ascending */
  int n, cap;
} zone_t;

struct co_cloth {
  co_params prm;
  int np, nt, nq, nb;
  double *X0;
  int *bc, *tri, *quad;
  /* 3x3 block CSR pattern with the diagonal held apart
   * (matrix_square_sparse.h:14-48) */
  int *row_ptr, *col_idx;
  double *vdia, *vcrs, *rhs;
  /* ILU(0) factor on the same pattern (ilu_sparse.h:16-34) */
  int *dia_split;
  double *fdia, *fcrs;
  int ilu_singular;
  /* BVH (bvh_aabb.h:18-23) */
  int nnode;
  int *node; /* 3 per node: parent, child0, child1 (child1 == -1 at a leaf) */
  box3 *bb;
  /* vertex 1-ring over triangles, CJaggedArray::SetEdgeOfElem order */
  int *ring_ptr, *ring;
  /* rigid impact zones */
  zone_t *zones;
  int nzone, zcap;
  int *zone_of;
  /* scratch */
  double *tmp0, *tmp1, *tmp2, *tmp3;
  /* contact log of the last co_resolve: one entry per detection */
  int log_on, log_n, log_cap;
  int *log_kind, *log_count;
  unsigned long long *log_digest;
};

static void *xmalloc(size_t n) {
  void *p = malloc(n ? n : 1);
  if (!p) abort();
  return p;
}
static void *xcalloc(size_t n, size_t s) {
  void *p = calloc(n ? n : 1, s ? s : 1);
  if (!p) abort();
  return p;
}

/* vertex -> incident elements in ascending element order,
 * CJaggedArray::SetNodeToElem, jagged_array.h:96-126 */
static void node_to_elem(int nnode, int nelem, int nnoel, const int *elem, int **ptr_out, int **arr_out) {
  int *ptr = (int *)xcalloc((size_t)nnode + 1, sizeof(int));
  int *arr, *fill, e, k;
  for (e = 0; e < nelem; e++)
    for (k = 0; k < nnoel; k++) ptr[elem[e * nnoel + k] + 1]++;
  for (k = 0; k < nnode; k++) ptr[k + 1] += ptr[k];
  arr = (int *)xmalloc(sizeof(int) * (size_t)ptr[nnode]);
  fill = (int *)xmalloc(sizeof(int) * (size_t)nnode);
  memcpy(fill, ptr, sizeof(int) * (size_t)nnode);
  for (e = 0; e < nelem; e++)
    for (k = 0; k < nnoel; k++) arr[fill[elem[e * nnoel + k]]++] = e;
  free(fill);
  *ptr_out = ptr;
  *arr_out = arr;
}

/* vertex adjacency through elements, self excluded, in discovery order,
 * CJaggedArray::SetEdgeOfElem(is_dia=false), jagged_array.h:158-207 */
static void elem_adjacency(int nnode, int nelem, int nnoel, const int *elem, int **ptr_out, int **arr_out) {
  int *eptr, *earr, *mark, *ptr, *arr, v, pass;
  node_to_elem(nnode, nelem, nnoel, elem, &eptr, &earr);
  mark = (int *)xmalloc(sizeof(int) * (size_t)nnode);
  ptr = (int *)xcalloc((size_t)nnode + 1, sizeof(int));
  arr = NULL;
  for (pass = 0; pass < 2; pass++) {
    int n = 0;
    for (v = 0; v < nnode; v++) mark[v] = -1;
    for (v = 0; v < nnode; v++) {
      int i, k;
      mark[v] = v;
      if (pass == 1) n = ptr[v];
      for (i = eptr[v]; i < eptr[v + 1]; i++) {
        const int e = earr[i];
        for (k = 0; k < nnoel; k++) {
          const int w = elem[e * nnoel + k];
          if (mark[w] != v) {
            mark[w] = v;
            if (pass == 0)
              ptr[v + 1]++;
            else
              arr[n++] = w;
          }
        }
      }
    }
    if (pass == 0) {
      for (v = 0; v < nnode; v++) ptr[v + 1] += ptr[v];
      arr = (int *)xmalloc(sizeof(int) * (size_t)ptr[nnode]);
    }
  }
  free(mark);
  free(eptr);
  free(earr);
  *ptr_out = ptr;
  *arr_out = arr;
}

static int cmp_int(const void *a, const void *b) {
  const int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

static void bvh_build(co_cloth *h);

co_cloth *co_create(int np, const double *X0, const int *bc, int nt, const int *tri, int nq, const int *quad,
                    const co_params *prm) {
  co_cloth *h = (co_cloth *)xcalloc(1, sizeof(co_cloth));
  int v;
  h->prm = *prm;
  h->np = np;
  h->nt = nt;
  h->nq = nq;
  h->X0 = (double *)xmalloc(sizeof(double) * 3 * (size_t)np);
  memcpy(h->X0, X0, sizeof(double) * 3 * (size_t)np);
  h->bc = (int *)xmalloc(sizeof(int) * (size_t)np);
  memcpy(h->bc, bc, sizeof(int) * (size_t)np);
  h->tri = (int *)xmalloc(sizeof(int) * 3 * (size_t)nt);
  memcpy(h->tri, tri, sizeof(int) * 3 * (size_t)nt);
  h->quad = (int *)xmalloc(sizeof(int) * 4 * (size_t)nq);
  memcpy(h->quad, quad, sizeof(int) * 4 * (size_t)nq);
  /* matrix pattern: bending-stencil adjacency, rows sorted
   * (self_contact_sparse/main.cpp:578-581) */
  elem_adjacency(np, nq, 4, quad, &h->row_ptr, &h->col_idx);
  for (v = 0; v < np; v++)
    qsort(h->col_idx + h->row_ptr[v], (size_t)(h->row_ptr[v + 1] - h->row_ptr[v]), sizeof(int), cmp_int);
  h->nb = h->row_ptr[np];
  h->vdia = (double *)xcalloc(9 * (size_t)np, sizeof(double));
  h->vcrs = (double *)xcalloc(9 * (size_t)h->nb, sizeof(double));
  h->rhs = (double *)xcalloc(3 * (size_t)np, sizeof(double));
  h->fdia = (double *)xcalloc(9 * (size_t)np, sizeof(double));
  h->fcrs = (double *)xcalloc(9 * (size_t)h->nb, sizeof(double));
  /* first strictly-upper entry of each row, Initialize_ILU0, ilu_sparse.cpp:114-134 */
  h->dia_split = (int *)xmalloc(sizeof(int) * (size_t)np);
  for (v = 0; v < np; v++) {
    int k;
    h->dia_split[v] = h->row_ptr[v + 1];
    for (k = h->row_ptr[v]; k < h->row_ptr[v + 1]; k++)
      if (h->col_idx[k] > v) {
        h->dia_split[v] = k;
        break;
      }
  }
  elem_adjacency(np, nt, 3, tri, &h->ring_ptr, &h->ring);
  bvh_build(h);
  h->bb = (box3 *)xcalloc((size_t)h->nnode, sizeof(box3));
  h->zone_of = (int *)xmalloc(sizeof(int) * (size_t)np);
  for (v = 0; v < np; v++) h->zone_of[v] = -1;
  h->tmp0 = (double *)xcalloc(3 * (size_t)np, sizeof(double));
  h->tmp1 = (double *)xcalloc(3 * (size_t)np, sizeof(double));
  h->tmp2 = (double *)xcalloc(3 * (size_t)np, sizeof(double));
  h->tmp3 = (double *)xcalloc(3 * (size_t)np, sizeof(double));
  return h;
}

void co_riz_reset(co_cloth *h) {
  int i;
  for (i = 0; i < h->nzone; i++) free(h->zones[i].mem);
  free(h->zones);
  h->zones = NULL;
  h->nzone = h->zcap = 0;
  for (i = 0; i < h->np; i++) h->zone_of[i] = -1;
}

void co_destroy(co_cloth *h) {
  if (!h) return;
  co_riz_reset(h);
  free(h->X0);
  free(h->bc);
  free(h->tri);
  free(h->quad);
  free(h->row_ptr);
  free(h->col_idx);
  free(h->vdia);
  free(h->vcrs);
  free(h->rhs);
  free(h->fdia);
  free(h->fcrs);
  free(h->dia_split);
  free(h->node);
  free(h->bb);
  free(h->ring_ptr);
  free(h->ring);
  free(h->zone_of);
  free(h->tmp0);
  free(h->tmp1);
  free(h->tmp2);
  free(h->tmp3);
  free(h->log_kind);
  free(h->log_count);
  free(h->log_digest);
  free(h);
}

void co_set_params(co_cloth *h, const co_params *prm) { h->prm = *prm; }
int co_num_blocks(const co_cloth *h) { return h->nb; }
void co_pattern(const co_cloth *h, int *row_ptr, int *col_idx) {
  memcpy(row_ptr, h->row_ptr, sizeof(int) * ((size_t)h->np + 1));
  memcpy(col_idx, h->col_idx, sizeof(int) * (size_t)h->nb);
}
int co_num_nodes(const co_cloth *h) { return h->nnode; }
void co_bvh_nodes(const co_cloth *h, int *nodes) { memcpy(nodes, h->node, sizeof(int) * 3 * (size_t)h->nnode); }
int co_num_edges(const co_cloth *h) { return h->ring_ptr[h->np]; }
void co_edges(const co_cloth *h, int *index, int *array) {
  memcpy(index, h->ring_ptr, sizeof(int) * ((size_t)h->np + 1));
  memcpy(array, h->ring, sizeof(int) * (size_t)h->ring_ptr[h->np]);
}

/* ======================================================================== */
/* assembly (solve_internal_sparse.h:19-183, matrix_square_sparse.cpp:88-302) */
/* ======================================================================== */

/* slot of column j in row i of the pattern, or -1 */
static int find_slot(const co_cloth *h, int i, int j) {
  int lo = h->row_ptr[i], hi = h->row_ptr[i + 1] - 1;
  while (lo <= hi) {
    const int m = (lo + hi) >> 1;
    if (h->col_idx[m] == j) return m;
    if (h->col_idx[m] < j)
      lo = m + 1;
    else
      hi = m - 1;
  }
  return -1;
}

/* Adds an n x n element matrix of 3x3 blocks; off-pattern blocks are dropped
 * like CMatrixSquareSparse::Mearge, matrix_square_sparse.cpp:88-138. */
static void scatter_blocks(co_cloth *h, int n, const int *vid, const double *emat) {
  int a, b, k;
  for (a = 0; a < n; a++) {
    const int i = vid[a];
    for (b = 0; b < n; b++) {
      const double *blk = emat + (a * n + b) * 9;
      double *dst;
      if (a == b) {
        dst = h->vdia + (size_t)i * 9;
      } else {
        const int s = find_slot(h, i, vid[b]);
        if (s < 0) continue;
        dst = h->vcrs + (size_t)s * 9;
      }
      for (k = 0; k < 9; k++) dst[k] += blk[k];
    }
  }
}

static void gather(const double *x, const int *vid, int n, double *out) {
  int a, k;
  for (a = 0; a < n; a++)
    for (k = 0; k < 3; k++) out[a * 3 + k] = x[vid[a] * 3 + k];
}

/* cloth internal forces: gradient into g (accumulated), Hessian into the matrix
 * when with_hessian (AddWdWddW_Cloth :19-76 / AddWdW_Cloth :81-132) */
static void add_cloth_terms(co_cloth *h, const double *x, double *g, int with_hessian) {
  int e, a, k;
  double C[12], c[12], W, dW[12], ddW[144];
  for (e = 0; e < h->nt; e++) {
    const int *vid = h->tri + e * 3;
    gather(h->X0, vid, 3, C);
    gather(x, vid, 3, c);
    co_wdwddw_cst(C, c, h->prm.lambda, h->prm.myu, &W, dW, ddW);
    for (a = 0; a < 3; a++)
      for (k = 0; k < 3; k++) g[vid[a] * 3 + k] += dW[a * 3 + k];
    if (with_hessian) scatter_blocks(h, 3, vid, ddW);
  }
  for (e = 0; e < h->nq; e++) {
    const int *vid = h->quad + e * 4;
    gather(h->X0, vid, 4, C);
    gather(x, vid, 4, c);
    W = 0;
    co_wdwddw_bend(C, c, h->prm.stiff_bend, &W, dW, ddW);
    for (a = 0; a < 4; a++)
      for (k = 0; k < 3; k++) g[vid[a] * 3 + k] += dW[a * 3 + k];
    if (with_hessian) scatter_blocks(h, 4, vid, ddW);
  }
}

/* AddWdW_Gravity, solve_internal_sparse.h:165-183 */
static void add_gravity(const co_cloth *h, double *g) {
  int v;
  for (v = 0; v < h->np; v++) {
    g[v * 3 + 0] -= h->prm.mass_point * h->prm.gravity[0];
    g[v * 3 + 1] -= h->prm.mass_point * h->prm.gravity[1];
    g[v * 3 + 2] -= h->prm.mass_point * h->prm.gravity[2];
  }
}

/* Linear system of one backward-Euler Newton step, the assembly half of
 * StepTime_InternalDynamicsILU, solve_internal_sparse.h:276-313. */
void co_assemble(co_cloth *h, const double *x, const double *v, double *vdia, double *vcrs, double *b) {
  const co_params *q = &h->prm;
  const int np = h->np, nd = 3 * np;
  int i, k;
  memset(h->vdia, 0, sizeof(double) * 9 * (size_t)np);
  memset(h->vcrs, 0, sizeof(double) * 9 * (size_t)h->nb);
  memset(h->rhs, 0, sizeof(double) * (size_t)nd);
  add_cloth_terms(h, x, h->rhs, 1);
  for (i = 0; i < np; i++) { /* AddWdWddW_Contact :137-161 */
    double W, dW[3], ddW[9];
    co_wdwddw_contact(x + i * 3, q, &W, dW, ddW);
    for (k = 0; k < 3; k++) h->rhs[i * 3 + k] += dW[k];
    scatter_blocks(h, 1, &i, ddW);
  }
  add_gravity(h, h->rhs);
  for (i = 0; i < nd; i++) h->rhs[i] = -h->rhs[i] + q->mass_point * v[i] / q->dt;
  for (i = 0; i < np; i++) {
    h->vdia[i * 9 + 0] += q->mass_point / (q->dt * q->dt);
    h->vdia[i * 9 + 4] += q->mass_point / (q->dt * q->dt);
    h->vdia[i * 9 + 8] += q->mass_point / (q->dt * q->dt);
  }
  /* SetBoundaryCondition, matrix_square_sparse.cpp:272-302 */
  for (i = 0; i < np; i++) {
    if (h->bc[i] == 0) continue;
    for (k = 0; k < 9; k++) h->vdia[i * 9 + k] = (k % 4 == 0) ? 1.0 : 0.0;
    for (k = h->row_ptr[i] * 9; k < h->row_ptr[i + 1] * 9; k++) h->vcrs[k] = 0.0;
  }
  for (i = 0; i < h->nb; i++) {
    if (h->bc[h->col_idx[i]] == 0) continue;
    for (k = 0; k < 9; k++) h->vcrs[i * 9 + k] = 0.0;
  }
  for (i = 0; i < np; i++)
    if (h->bc[i]) h->rhs[i * 3 + 0] = h->rhs[i * 3 + 1] = h->rhs[i * 3 + 2] = 0;
  if (vdia) memcpy(vdia, h->vdia, sizeof(double) * 9 * (size_t)np);
  if (vcrs) memcpy(vcrs, h->vcrs, sizeof(double) * 9 * (size_t)h->nb);
  if (b) memcpy(b, h->rhs, sizeof(double) * (size_t)nd);
}

/* ======================================================================== */
/* block ILU(0) and Krylov solvers (ilu_sparse.cpp, matrix_square_sparse.cpp) */
/* ======================================================================== */

/* determinant of a row-major 3x3 in the reference's term order (ilu_sparse.cpp:78-80) */
static double det33(const double *a) {
  return +a[0] * a[4] * a[8] + a[3] * a[7] * a[2] + a[6] * a[1] * a[5] - a[0] * a[7] * a[5] -
         a[6] * a[4] * a[2] - a[3] * a[1] * a[8];
}
/* cofactor inverse, CalcInvMat3 (ilu_sparse.cpp:76-97, self_collision_cloth.cpp:278-296) */
static void inv33(double *out, const double *t) {
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

/* Block ILU(0) in natural row order, SetValueILU + DoILUDecomp (3x3 branch),
 * ilu_sparse.cpp:352-384, 387-395, 507-569.  Like the reference it stops after
 * more than 10 singular pivots, leaving later rows unfactorised. */
int co_ilu(co_cloth *h, double *fdia, double *fcrs) {
  const int np = h->np;
  double *D = h->fdia, *U = h->fcrs;
  int *col_slot = (int *)xmalloc(sizeof(int) * (size_t)np);
  int i, nsing = 0;
  memcpy(D, h->vdia, sizeof(double) * 9 * (size_t)np);
  memcpy(U, h->vcrs, sizeof(double) * 9 * (size_t)h->nb);
  for (i = 0; i < np; i++) col_slot[i] = -1;
  for (i = 0; i < np; i++) {
    int s, ks, r;
    for (s = h->row_ptr[i]; s < h->row_ptr[i + 1]; s++) col_slot[h->col_idx[s]] = s;
    for (s = h->row_ptr[i]; s < h->dia_split[i]; s++) { /* L part of row i */
      const int kk = h->col_idx[s];
      const double *lik = U + (size_t)s * 9;
      for (ks = h->dia_split[kk]; ks < h->row_ptr[kk + 1]; ks++) { /* U part of row k */
        const int j = h->col_idx[ks];
        const double *ukj = U + (size_t)ks * 9;
        double *dst;
        if (j != i) {
          const int t = col_slot[j];
          if (t == -1) continue;
          dst = U + (size_t)t * 9;
        } else {
          dst = D + (size_t)i * 9;
        }
        for (r = 0; r < 3; r++) {
          dst[r * 3 + 0] -= lik[r * 3 + 0] * ukj[0] + lik[r * 3 + 1] * ukj[3] + lik[r * 3 + 2] * ukj[6];
          dst[r * 3 + 1] -= lik[r * 3 + 0] * ukj[1] + lik[r * 3 + 1] * ukj[4] + lik[r * 3 + 2] * ukj[7];
          dst[r * 3 + 2] -= lik[r * 3 + 0] * ukj[2] + lik[r * 3 + 1] * ukj[5] + lik[r * 3 + 2] * ukj[8];
        }
      }
    }
    {
      double *dii = D + (size_t)i * 9;
      if (fabs(det33(dii)) > 1.0e-30) {
        double t[9];
        memcpy(t, dii, sizeof(t));
        inv33(dii, t);
      } else {
        nsing++;
        if (nsing > 10) break;
      }
    }
    for (s = h->dia_split[i]; s < h->row_ptr[i + 1]; s++) { /* U <- D^-1 U */
      double *uij = U + (size_t)s * 9, t[9];
      const double *dii = D + (size_t)i * 9;
      memcpy(t, uij, sizeof(t));
      for (r = 0; r < 3; r++) {
        uij[r * 3 + 0] = dii[r * 3 + 0] * t[0] + dii[r * 3 + 1] * t[3] + dii[r * 3 + 2] * t[6];
        uij[r * 3 + 1] = dii[r * 3 + 0] * t[1] + dii[r * 3 + 1] * t[4] + dii[r * 3 + 2] * t[7];
        uij[r * 3 + 2] = dii[r * 3 + 0] * t[2] + dii[r * 3 + 1] * t[5] + dii[r * 3 + 2] * t[8];
      }
    }
    for (s = h->row_ptr[i]; s < h->row_ptr[i + 1]; s++) col_slot[h->col_idx[s]] = -1;
  }
  free(col_slot);
  h->ilu_singular = nsing;
  if (fdia) memcpy(fdia, D, sizeof(double) * 9 * (size_t)np);
  if (fcrs) memcpy(fcrs, U, sizeof(double) * 9 * (size_t)h->nb);
  return nsing;
}

/* Applies (LU)^-1 in place: forward then backward substitution,
 * ilu_sparse.cpp:185-215, 295-324. */
static void ilu_apply(const co_cloth *h, double *z) {
  int i, s, r;
  for (i = 0; i < h->np; i++) {
    double t[3] = {z[i * 3 + 0], z[i * 3 + 1], z[i * 3 + 2]};
    const double *d = h->fdia + (size_t)i * 9;
    for (s = h->row_ptr[i]; s < h->dia_split[i]; s++) {
      const int j = h->col_idx[s];
      const double *l = h->fcrs + (size_t)s * 9;
      const double y0 = z[j * 3 + 0], y1 = z[j * 3 + 1], y2 = z[j * 3 + 2];
      for (r = 0; r < 3; r++) t[r] -= l[r * 3 + 0] * y0 + l[r * 3 + 1] * y1 + l[r * 3 + 2] * y2;
    }
    for (r = 0; r < 3; r++) z[i * 3 + r] = d[r * 3 + 0] * t[0] + d[r * 3 + 1] * t[1] + d[r * 3 + 2] * t[2];
  }
  for (i = h->np - 1; i >= 0; i--) {
    double t[3] = {z[i * 3 + 0], z[i * 3 + 1], z[i * 3 + 2]};
    for (s = h->dia_split[i]; s < h->row_ptr[i + 1]; s++) {
      const int j = h->col_idx[s];
      const double *u = h->fcrs + (size_t)s * 9;
      const double y0 = z[j * 3 + 0], y1 = z[j * 3 + 1], y2 = z[j * 3 + 2];
      for (r = 0; r < 3; r++) t[r] -= u[r * 3 + 0] * y0 + u[r * 3 + 1] * y1 + u[r * 3 + 2] * y2;
    }
    for (r = 0; r < 3; r++) z[i * 3 + r] = t[r];
  }
}

/* y = A x with y scaled by zero first, MatVec(1, x, 0, y), matrix_square_sparse.cpp:218-242 */
static void spmv(const co_cloth *h, const double *x, double *y) {
  int i, s, r;
  for (i = 0; i < h->np; i++) {
    double *yi = y + i * 3;
    for (r = 0; r < 3; r++) yi[r] *= 0.0;
    for (s = h->row_ptr[i]; s < h->row_ptr[i + 1]; s++) {
      const int j = h->col_idx[s];
      const double *a = h->vcrs + (size_t)s * 9;
      for (r = 0; r < 3; r++)
        yi[r] += 1.0 * (a[r * 3 + 0] * x[j * 3 + 0] + a[r * 3 + 1] * x[j * 3 + 1] + a[r * 3 + 2] * x[j * 3 + 2]);
    }
    {
      const double *a = h->vdia + (size_t)i * 9;
      for (r = 0; r < 3; r++)
        yi[r] += 1.0 * (a[r * 3 + 0] * x[i * 3 + 0] + a[r * 3 + 1] * x[i * 3 + 1] + a[r * 3 + 2] * x[i * 3 + 2]);
    }
  }
}

/* InnerProduct, matrix_square_sparse.cpp:313-325: one running sum in index order */
static double vdot(const double *a, const double *b, int n) {
  double r = 0.0;
  int i;
  for (i = 0; i < n; i++) r += a[i] * b[i];
  return r;
}
/* AXPY, matrix_square_sparse.cpp:327-336 */
static void vaxpy(double a, const double *x, double *y, int n) {
  int i;
  for (i = 0; i < n; i++) y[i] += a * x[i];
}

/* ILU(0)-preconditioned CG from x = 0, Solve_PCG, ilu_sparse.cpp:628-709.
 * r is overwritten with the final residual. */
static void pcg_solve(co_cloth *h, double *r, double *x, double tol, int maxit, double *conv, int *iter) {
  const int n = 3 * h->np;
  double *Pr = h->tmp1, *p = h->tmp2;
  double inv0, rPr;
  int it, i;
  for (i = 0; i < n; i++) x[i] = 0;
  {
    const double s0 = vdot(r, r, n);
    if (s0 < 1.0e-30) {
      *conv = 0.0;
      *iter = 0;
      return;
    }
    inv0 = 1.0 / s0;
  }
  memcpy(Pr, r, sizeof(double) * (size_t)n);
  ilu_apply(h, Pr);
  memcpy(p, Pr, sizeof(double) * (size_t)n);
  rPr = vdot(r, Pr, n);
  for (it = 0; it < maxit; it++) {
    {
      double *Ap = Pr; /* the reference reuses the preconditioned vector's storage */
      spmv(h, p, Ap);
      const double pAp = vdot(p, Ap, n);
      const double alpha = rPr / pAp;
      vaxpy(-alpha, Ap, r, n);
      vaxpy(+alpha, p, x, n);
    }
    {
      const double sq = vdot(r, r, n);
      if (sq * inv0 < tol * tol) {
        *conv = sqrt(sq * inv0);
        *iter = it;
        return;
      }
    }
    {
      memcpy(Pr, r, sizeof(double) * (size_t)n);
      ilu_apply(h, Pr);
      const double rPr1 = vdot(r, Pr, n);
      const double beta = rPr1 / rPr;
      rPr = rPr1;
      for (i = 0; i < n; i++) p[i] = Pr[i] + beta * p[i];
    }
  }
  *conv = sqrt(vdot(r, r, n) * inv0);
  *iter = maxit;
}

/* Plain CG from x = 0, Solve_CG, matrix_square_sparse.cpp:338-406.  Note the
 * loop starts at 1 and the reported ratio uses the previous residual. */
static void cg_solve(co_cloth *h, double *r, double *x, double tol, int maxit, double *conv, int *iter) {
  const int n = 3 * h->np;
  double *Ap = h->tmp1, *p = h->tmp2;
  double sq, inv0;
  int it, i;
  for (i = 0; i < n; i++) x[i] = 0;
  sq = vdot(r, r, n);
  if (sq < 1.0e-30) {
    *conv = 0.0;
    *iter = 0;
    return;
  }
  inv0 = 1.0 / sq;
  memcpy(p, r, sizeof(double) * (size_t)n);
  *iter = maxit;
  *conv = tol;
  for (it = 1; it < maxit; it++) {
    spmv(h, p, Ap);
    const double pAp = vdot(p, Ap, n);
    const double alpha = sq / pAp;
    vaxpy(alpha, p, x, n);
    vaxpy(-alpha, Ap, r, n);
    const double sq_new = vdot(r, r, n);
    if (sq_new * inv0 < tol * tol) {
      *conv = sqrt(sq * inv0);
      *iter = it;
      return;
    }
    const double beta = sq_new / sq;
    sq = sq_new;
    for (i = 0; i < n; i++) p[i] = r[i] + beta * p[i];
  }
}

void co_pcg(co_cloth *h, const double *b, double tol, int maxit, double *x, double *conv, int *iter) {
  memcpy(h->tmp0, b, sizeof(double) * 3 * (size_t)h->np);
  pcg_solve(h, h->tmp0, x, tol, maxit, conv, iter);
}

void co_cg(co_cloth *h, const double *b, double tol, int maxit, double *x, double *conv, int *iter) {
  memcpy(h->tmp0, b, sizeof(double) * 3 * (size_t)h->np);
  cg_solve(h, h->tmp0, x, tol, maxit, conv, iter);
}

/* the residual r_vec that the last co_cg / co_pcg left behind */
void co_last_residual(const co_cloth *h, double *r) { memcpy(r, h->tmp0, sizeof(double) * 3 * (size_t)h->np); }

/* CPreconditionerILU::Solve (ilu_sparse.h:23-26) with the last co_ilu factor */
void co_ilu_solve(const co_cloth *h, double *vec) { ilu_apply(h, vec); }

/* MatVec(alpha, x, beta, y) on the last assembled matrix, 3x3 branch of
 * matrix_square_sparse.cpp:218-242 */
void co_matvec(const co_cloth *h, double alpha, const double *x, double beta, double *y) {
  int i, s, r;
  for (i = 0; i < h->np; i++) {
    double *yi = y + i * 3;
    for (r = 0; r < 3; r++) yi[r] *= beta;
    for (s = h->row_ptr[i]; s < h->row_ptr[i + 1]; s++) {
      const int j = h->col_idx[s];
      const double *a = h->vcrs + (size_t)s * 9;
      for (r = 0; r < 3; r++)
        yi[r] += alpha * (a[r * 3 + 0] * x[j * 3 + 0] + a[r * 3 + 1] * x[j * 3 + 1] + a[r * 3 + 2] * x[j * 3 + 2]);
    }
    {
      const double *a = h->vdia + (size_t)i * 9;
      for (r = 0; r < 3; r++)
        yi[r] += alpha * (a[r * 3 + 0] * x[i * 3 + 0] + a[r * 3 + 1] * x[i * 3 + 1] + a[r * 3 + 2] * x[i * 3 + 2]);
    }
  }
}

/* One Newton step of backward Euler, StepTime_InternalDynamicsILU
 * (solve_internal_sparse.h:255-326) or StepTime_InternalDynamics (:185-253)
 * with the tolerance and cap from the parameters. */
void co_implicit(co_cloth *h, double *x, double *v, co_stats *st) {
  const int n = 3 * h->np;
  double conv = 0;
  int iter = 0, i;
  double *dx = h->tmp3;
  co_assemble(h, x, v, NULL, NULL, NULL);
  memcpy(h->tmp0, h->rhs, sizeof(double) * (size_t)n);
  if (h->prm.solver_kind == CO_SOLVER_CG) {
    cg_solve(h, h->tmp0, dx, h->prm.tol, h->prm.maxit, &conv, &iter);
  } else {
    co_ilu(h, NULL, NULL);
    if (st) st->ilu_singular = h->ilu_singular;
    pcg_solve(h, h->tmp0, dx, h->prm.tol, h->prm.maxit, &conv, &iter);
  }
  for (i = 0; i < n; i++) x[i] += dx[i];
  for (i = 0; i < n; i++) v[i] = dx[i] / h->prm.dt;
  if (st) {
    st->solver_iterations = iter;
    st->solver_conv = conv;
  }
}

/* ======================================================================== */
/* BVH topology (bvh_aabb.cpp:109-313)                                       */
/* ======================================================================== */

static vec3 tri_centroid(const co_cloth *h, int t) {
  const int *v = h->tri + t * 3;
  const double *X = h->X0;
  return mk((X[v[0] * 3 + 0] + X[v[1] * 3 + 0] + X[v[2] * 3 + 0]) / 3.0,
            (X[v[0] * 3 + 1] + X[v[1] * 3 + 1] + X[v[2] * 3 + 1]) / 3.0,
            (X[v[0] * 3 + 2] + X[v[1] * 3 + 2] + X[v[2] * 3 + 2]) / 3.0);
}

typedef struct {
  co_cloth *h;
  int *owner;    /* triangle -> node currently holding it */
  int *across;   /* triangle -> neighbour across each edge, -1 on the border */
  int *stack;
  int cap;
} bvh_builder;

static int node_new(bvh_builder *B, int parent) {
  co_cloth *h = B->h;
  if (h->nnode == B->cap) {
    B->cap = B->cap ? 2 * B->cap : 64;
    h->node = (int *)realloc(h->node, sizeof(int) * 3 * (size_t)B->cap);
    if (!h->node) abort();
  }
  h->node[h->nnode * 3 + 0] = parent;
  h->node[h->nnode * 3 + 1] = -1;
  h->node[h->nnode * 3 + 2] = -1;
  return h->nnode++;
}

/* Finds a seed triangle on the positive side of the plane through org normal
 * to dir (flipping dir toward it), as in DevideTriAryConnex :185-192. */
static int pick_seed(const co_cloth *h, const int *list, int n, vec3 org, vec3 *dir) {
  int i;
  for (i = 0; i < n; i++) {
    const vec3 g = tri_centroid(h, list[i]);
    if (fabs(dot(sub(g, org), *dir)) < 1.0e-10) continue;
    if (dot(sub(g, org), *dir) < 0) *dir = scl(-1.0, *dir);
    return list[i];
  }
  return -1;
}

/* Splits the triangles of node `self` in two connected halves, recursively,
 * DevideTriAryConnex, bvh_aabb.cpp:156-290. */
static void bvh_split(bvh_builder *B, int self, const int *list, int n) {
  co_cloth *h = B->h;
  box3 bb;
  vec3 dir = mk(0, 0, 0), org;
  int i, seed, c0, c1, n0 = 0, n1 = 0, sp = 0;
  int *l0, *l1;
  box_clear(&bb);
  for (i = 0; i < n; i++) box_add_point(&bb, tri_centroid(h, list[i]), 1.0e-10);
  {
    const double lx = bb.hi[0] - bb.lo[0], ly = bb.hi[1] - bb.lo[1], lz = bb.hi[2] - bb.lo[2];
    if (lx > ly && lx > lz) dir = mk(1, 0, 0);
    if (ly > lz && ly > lx) dir = mk(0, 1, 0);
    if (lz > lx && lz > ly) dir = mk(0, 0, 1);
  }
  org = mk((bb.lo[0] + bb.hi[0]) * 0.5, (bb.lo[1] + bb.hi[1]) * 0.5, (bb.lo[2] + bb.hi[2]) * 0.5);
  seed = pick_seed(h, list, n, org, &dir);
  if (seed == -1) { /* no unique longest axis: principal axis by power iteration */
    double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    int r, c, it;
    org = mk(0, 0, 0);
    for (i = 0; i < n; i++) org = add(org, tri_centroid(h, list[i]));
    org = div_guarded(org, (double)n);
    for (i = 0; i < n; i++) {
      const vec3 g = sub(tri_centroid(h, list[i]), org);
      const double gv[3] = {g.x, g.y, g.z};
      for (r = 0; r < 3; r++)
        for (c = 0; c < 3; c++) M[r][c] += gv[r] * gv[c];
    }
    {
      double d[3] = {1, 1, 1};
      for (it = 0; it < 10; it++) {
        const double t[3] = {M[0][0] * d[0] + M[0][1] * d[1] + M[0][2] * d[2],
                             M[1][0] * d[0] + M[1][1] * d[1] + M[1][2] * d[2],
                             M[2][0] * d[0] + M[2][1] * d[1] + M[2][2] * d[2]};
        const double len = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        d[0] = t[0] / len;
        d[1] = t[1] / len;
        d[2] = t[2] / len;
      }
      dir = mk(d[0], d[1], d[2]);
    }
    seed = pick_seed(h, list, n, org, &dir);
    if (seed == -1) seed = list[0]; /* all centroids on the plane: not met on sheets */
  }
  c0 = node_new(B, self);
  c1 = node_new(B, self);
  h->node[self * 3 + 1] = c0;
  h->node[self * 3 + 2] = c1;
  l0 = (int *)xmalloc(sizeof(int) * (size_t)n);
  l1 = (int *)xmalloc(sizeof(int) * (size_t)n);
  /* flood fill over edge neighbours on the positive side, LIFO order */
  B->owner[seed] = c0;
  l0[n0++] = seed;
  B->stack[sp++] = seed;
  while (sp > 0) {
    const int t = B->stack[--sp];
    int e;
    for (e = 0; e < 3; e++) {
      const int u = B->across[t * 3 + e];
      if (u == -1) continue;
      if (B->owner[u] != self) continue;
      if (dot(sub(tri_centroid(h, u), org), dir) < 0) continue;
      B->stack[sp++] = u;
      B->owner[u] = c0;
      l0[n0++] = u;
    }
  }
  for (i = 0; i < n; i++) {
    const int t = list[i];
    if (B->owner[t] == c0) continue;
    B->owner[t] = c1;
    l1[n1++] = t;
  }
  if (n0 == 1) {
    h->node[c0 * 3 + 1] = l0[0];
    h->node[c0 * 3 + 2] = -1;
  } else {
    bvh_split(B, c0, l0, n0);
  }
  free(l0);
  if (n1 == 1) {
    h->node[c1 * 3 + 1] = l1[0];
    h->node[c1 * 3 + 2] = -1;
  } else {
    bvh_split(B, c1, l1, n1);
  }
  free(l1);
}

/* MakeBVHTopology_TopDown with MakeTriSurTri, bvh_aabb.cpp:109-138, 294-313 */
static void bvh_build(co_cloth *h) {
  static const int kEdge[3][2] = {{1, 2}, {2, 0}, {0, 1}};
  bvh_builder B;
  int *eptr, *earr, t, e, i, *list;
  memset(&B, 0, sizeof(B));
  B.h = h;
  B.across = (int *)xmalloc(sizeof(int) * 3 * (size_t)h->nt);
  node_to_elem(h->np, h->nt, 3, h->tri, &eptr, &earr);
  for (t = 0; t < h->nt; t++) {
    for (e = 0; e < 3; e++) {
      const int a = h->tri[t * 3 + kEdge[e][0]], b = h->tri[t * 3 + kEdge[e][1]];
      int found = -1;
      B.across[t * 3 + e] = -1;
      for (i = eptr[a]; i < eptr[a + 1] && found < 0; i++) {
        const int u = earr[i];
        int f;
        if (u == t) continue;
        for (f = 0; f < 3; f++)
          if (a == h->tri[u * 3 + kEdge[f][1]] && b == h->tri[u * 3 + kEdge[f][0]]) {
            found = u;
            break;
          }
      }
      B.across[t * 3 + e] = found;
    }
  }
  free(eptr);
  free(earr);
  B.owner = (int *)xcalloc((size_t)h->nt, sizeof(int));
  B.stack = (int *)xmalloc(sizeof(int) * ((size_t)h->nt + 1));
  list = (int *)xmalloc(sizeof(int) * (size_t)h->nt);
  for (t = 0; t < h->nt; t++) list[t] = t;
  h->nnode = 0;
  node_new(&B, -1);
  if (h->nt == 1) {
    h->node[1] = 0;
    h->node[2] = -1;
  } else {
    bvh_split(&B, 0, list, h->nt);
  }
  free(list);
  free(B.owner);
  free(B.stack);
  free(B.across);
}

/* ======================================================================== */
/* box refit (bvh_aabb.cpp:23-106)                                           */
/* ======================================================================== */

/* children are created after their parent, so a reverse sweep is bottom-up */
static void refit(co_cloth *h, const double *x, const double *v, double dt, double eps, int swept) {
  int n;
  for (n = h->nnode - 1; n >= 0; n--) {
    box3 *b = h->bb + n;
    const int c0 = h->node[n * 3 + 1], c1 = h->node[n * 3 + 2];
    if (c1 == -1) {
      const int *tv = h->tri + c0 * 3;
      int k;
      box_clear(b);
      for (k = 0; k < 3; k++) box_add_point(b, at(x, tv[k]), eps);
      if (swept)
        for (k = 0; k < 3; k++) {
          const int p = tv[k];
          box_add_point(b, mk(x[p * 3 + 0] + dt * v[p * 3 + 0], x[p * 3 + 1] + dt * v[p * 3 + 1],
                              x[p * 3 + 2] + dt * v[p * 3 + 2]),
                        eps);
        }
    } else {
      *b = h->bb[c0];
      box_merge(b, h->bb + c1);
    }
  }
}

static void export_boxes(const co_cloth *h, double *out) {
  int n, k;
  for (n = 0; n < h->nnode; n++) {
    for (k = 0; k < 3; k++) {
      out[n * 7 + 2 * k] = h->bb[n].lo[k];
      out[n * 7 + 2 * k + 1] = h->bb[n].hi[k];
    }
    out[n * 7 + 6] = h->bb[n].full ? 1.0 : 0.0;
  }
}

/* BuildBoundingBoxChild_Prx: leaf = triangle inflated by delta/2 */
void co_refit_prx(co_cloth *h, const double *x, double delta, double *boxes) {
  refit(h, x, NULL, 0, delta * 0.5, 0);
  if (boxes) export_boxes(h, boxes);
}

/* BuildBoundingBoxChild_CCD: leaf = triangle swept over dt, inflated by 1e-10 */
void co_refit_ccd(co_cloth *h, const double *x, const double *v, double dt, double *boxes) {
  refit(h, x, v, dt, 1.0e-10, 1);
  if (boxes) export_boxes(h, boxes);
}

/* ======================================================================== */
/* narrow phase (bvh_aabb.cpp:320-793)                                       */
/* ======================================================================== */

/* barycentric weights of the projection of p3 on the plane p0 p1 p2 and the
 * distance to it, DistanceFaceVertex :321-340 */
static double dist_face_vertex(vec3 p0, vec3 p1, vec3 p2, vec3 p3, double *w0, double *w1) {
  const vec3 v20 = sub(p0, p2), v21 = sub(p1, p2);
  const double t0 = dot(v20, v20), t1 = dot(v21, v21), t2 = dot(v20, v21);
  const double t3 = dot(v20, sub(p3, p2)), t4 = dot(v21, sub(p3, p2));
  const double det = t0 * t1 - t2 * t2;
  const double invdet = 1.0 / det;
  *w0 = (+t1 * t3 - t2 * t4) * invdet;
  *w1 = (-t2 * t3 + t0 * t4) * invdet;
  const double w2 = 1 - *w0 - *w1;
  const vec3 pw = add(add(scl(*w0, p0), scl(*w1, p1)), scl(w2, p2));
  return len3(sub(pw, p3));
}

/* closest points of the lines through two edges, DistanceEdgeEdge :343-384 */
static double dist_edge_edge(vec3 p0, vec3 p1, vec3 q0, vec3 q1, double *rp, double *rq) {
  const vec3 vp = sub(p1, p0), vq = sub(q1, q0);
  if (len3(cross(vp, vq)) < 1.0e-10) { /* parallel edges */
    const vec3 pq0 = sub(p0, q0);
    const vec3 nvp = normalized(vp);
    const vec3 vert = sub(pq0, scl(dot(pq0, nvp), nvp));
    const double dist = len3(vert);
    const double lp0 = dot(p0, nvp), lp1 = dot(p1, nvp), lq0 = dot(q0, nvp), lq1 = dot(q1, nvp);
    const double pmin = (lp0 < lp1) ? lp0 : lp1, pmax = (lp0 > lp1) ? lp0 : lp1;
    const double qmin = (lq0 < lq1) ? lq0 : lq1, qmax = (lq0 > lq1) ? lq0 : lq1;
    double lm;
    if (pmax < qmin)
      lm = (pmax + qmin) * 0.5;
    else if (qmax < pmin)
      lm = (qmax + pmin) * 0.5;
    else if (pmax < qmax)
      lm = (pmax + qmin) * 0.5;
    else
      lm = (qmax + pmin) * 0.5;
    *rp = (lm - lp0) / (lp1 - lp0);
    *rq = (lm - lq0) / (lq1 - lq0);
    return dist;
  }
  {
    const double t0 = dot(vp, vp), t1 = dot(vq, vq), t2 = dot(vp, vq);
    const double t3 = dot(vp, sub(q0, p0)), t4 = dot(vq, sub(q0, p0));
    const double det = t0 * t1 - t2 * t2;
    const double invdet = 1.0 / det;
    *rp = (+t1 * t3 - t2 * t4) * invdet;
    *rq = (+t2 * t3 - t0 * t4) * invdet;
    const vec3 pc = add(p0, scl(*rp, vp)), qc = add(q0, scl(*rq, vq));
    return len3(sub(pc, qc));
  }
}

/* IsContact_FV_Proximity :392-412; `bb` is the box the reference passes */
static int fv_proximity(int i0, int i1, int i2, int i3, vec3 p0, vec3 p1, vec3 p2, vec3 p3, const box3 *bb,
                        double delta) {
  double w0, w1, w2, dist;
  if (i3 == i0 || i3 == i1 || i3 == i2) return 0;
  if (!box_inside(bb, p3)) return 0;
  if (fabs(height4(p0, p1, p2, p3)) > delta) return 0;
  dist = dist_face_vertex(p0, p1, p2, p3, &w0, &w1);
  w2 = 1 - w0 - w1;
  if (dist > delta) return 0;
  if (w0 < 0 || w0 > 1) return 0;
  if (w1 < 0 || w1 > 1) return 0;
  if (w2 < 0 || w2 > 1) return 0;
  return 1;
}

/* IsContact_EE_Proximity :415-438 */
static int ee_proximity(int i0, int i1, int j0, int j1, vec3 p0, vec3 p1, vec3 q0, vec3 q1, double delta) {
  double rp, rq, dist;
  if (i0 == j0 || i0 == j1 || i1 == j0 || i1 == j1) return 0;
  if (q0.x + delta < p0.x && q0.x + delta < p1.x && q1.x + delta < p0.x && q1.x + delta < p1.x) return 0;
  if (q0.x - delta > p0.x && q0.x - delta > p1.x && q1.x - delta > p0.x && q1.x - delta > p1.x) return 0;
  if (q0.y + delta < p0.y && q0.y + delta < p1.y && q1.y + delta < p0.y && q1.y + delta < p1.y) return 0;
  if (q0.y - delta > p0.y && q0.y - delta > p1.y && q1.y - delta > p0.y && q1.y - delta > p1.y) return 0;
  if (q0.z + delta < p0.z && q0.z + delta < p1.z && q1.z + delta < p0.z && q1.z + delta < p1.z) return 0;
  if (q0.z - delta > p0.z && q0.z - delta > p1.z && q1.z - delta > p0.z && q1.z - delta > p1.z) return 0;
  dist = dist_edge_edge(p0, p1, q0, q1, &rp, &rq);
  if (dist > delta) return 0;
  if (rp < 0 || rp > 1 || rq < 0 || rq > 1) return 0;
  {
    const vec3 pm = add(scl(1 - rp, p0), scl(rp, p1));
    const vec3 qm = add(scl(1 - rq, q0), scl(rq, q1));
    if (len3(sub(pm, qm)) > delta) return 0;
  }
  return 1;
}

/* EvaluateCubic :563-568 */
static double cubic(double r, double k0, double k1, double k2, double k3) {
  return k0 + k1 * r + k2 * r * r + k3 * r * r * r;
}

/* FindRootCubic + BisectRangeCubicRoot :571-595: 14 halvings; the sign
 * reference stays the value at the initial left end. */
static double bisect_cubic(double r0, double r1, double v0, double k0, double k1, double k2, double k3) {
  int n;
  for (n = 14; n > 0; n--) {
    const double r2 = 0.5 * (r0 + r1);
    const double v2 = cubic(r2, k0, k1, k2, k3);
    if (v0 * v2 < 0)
      r1 = r2;
    else
      r0 = r2;
  }
  return 0.5 * (r0 + r1);
}

/* First time in [0,1] at which the four linearly moving points are coplanar,
 * or -1, FindCoplanerInterp :598-662. */
static double coplanar_time(vec3 s0, vec3 s1, vec3 s2, vec3 s3, vec3 e0, vec3 e1, vec3 e2, vec3 e3) {
  const vec3 x1 = sub(s1, s0), x2 = sub(s2, s0), x3 = sub(s3, s0);
  const vec3 v1 = sub(sub(e1, e0), x1), v2 = sub(sub(e2, e0), x2), v3 = sub(sub(e3, e0), x3);
  const double k0 = stp(x3, x1, x2);
  const double k1 = stp(v3, x1, x2) + stp(x3, v1, x2) + stp(x3, x1, v2);
  const double k2 = stp(v3, v1, x2) + stp(v3, x1, v2) + stp(x3, v1, v2);
  const double k3 = stp(v3, v1, v2);
  const double r0 = -0.0, r1 = +1.0;
  const double f0 = cubic(r0, k0, k1, k2, k3), f1 = cubic(r1, k0, k1, k2, k3);
  const double det = k2 * k2 - 3 * k1 * k3;
  if (fabs(k3) < 1.0e-10 && fabs(k2) > 1.0e-10) { /* quadratic */
    const double r2 = -k1 / (2 * k2);
    const double f2 = cubic(r2, k0, k1, k2, k3);
    if (r2 > 0 && r2 < 1) {
      if (f0 * f2 < 0) return bisect_cubic(r0, r2, f0, k0, k1, k2, k3);
      if (f2 * f1 < 0) return bisect_cubic(r2, r1, f2, k0, k1, k2, k3);
    }
  }
  if (det > 0 && fabs(k3) > 1.0e-10) { /* cubic with two extrema */
    const double r3 = (-k2 - sqrt(det)) / (3 * k3);
    const double f3 = cubic(r3, k0, k1, k2, k3);
    if (r3 > 0 && r3 < 1) {
      if (f0 * f3 < 0) return bisect_cubic(r0, r3, f0, k0, k1, k2, k3);
      if (f3 * f1 < 0) return bisect_cubic(r3, r1, f3, k0, k1, k2, k3);
    }
    const double r4 = (-k2 + sqrt(det)) / (3 * k3);
    const double f4 = cubic(r4, k0, k1, k2, k3);
    if (r3 > 0 && r3 < 1 && r4 > 0 && r4 < 1) {
      if (f3 * f4 < 0) return bisect_cubic(r3, r4, f3, k0, k1, k2, k3);
    }
    if (r4 > 0 && r4 < 1) {
      if (f0 * f4 < 0) return bisect_cubic(r0, r4, f0, k0, k1, k2, k3);
      if (f4 * f1 < 0) return bisect_cubic(r4, r1, f4, k0, k1, k2, k3);
    }
  }
  if (f0 * f1 > 0) return -1;
  return bisect_cubic(r0, r1, f0, k0, k1, k2, k3);
}

static vec3 lerp(double t, vec3 a, vec3 b) { return add(scl(1 - t, a), scl(t, b)); }

/* IsContact_FV_CCD :666-719 */
static int fv_ccd(int i0, int i1, int i2, int i3, vec3 p0, vec3 p1, vec3 p2, vec3 p3, vec3 q0, vec3 q1, vec3 q2,
                  vec3 q3, const box3 *bb) {
  const double eps = 1.0e-10;
  box3 bp;
  double r0, r1, dist, t, w0, w1, w2;
  if (i3 == i0 || i3 == i1 || i3 == i2) return 0;
  box_clear(&bp);
  box_add_point(&bp, p3, eps);
  box_add_point(&bp, q3, eps);
  if (!box_overlap(bb, &bp)) return 0;
  {
    const vec3 n = cross(sub(p1, p0), sub(p2, p0));
    const double t0 = dot(sub(p0, p3), n), t1 = dot(sub(q0, q3), n), t2 = dot(sub(q1, q3), n),
                 t3 = dot(sub(q2, q3), n);
    if (t0 * t1 > 0 && t0 * t2 > 0 && t0 * t3 > 0) return 0;
  }
  dist = dist_face_vertex(p0, p1, p2, p3, &r0, &r1);
  {
    const double vn0 = len3(sub(p0, q0)), vn1 = len3(sub(p1, q1)), vn2 = len3(sub(p2, q2)),
                 vn3 = len3(sub(p3, q3));
    double vnt = (vn0 > vn1) ? vn0 : vn1;
    vnt = (vn2 > vnt) ? vn2 : vnt;
    const double max_app = vnt + vn3;
    const double r2 = 1 - r0 - r1;
    if (dist > max_app) return 0;
    if (r0 < 0 || r0 > 1 || r1 < 0 || r1 > 1 || r2 < 0 || r2 > 1) {
      const double d01 = len3(sub(closest_on_segment(p3, p0, p1), p3));
      const double d12 = len3(sub(closest_on_segment(p3, p1, p2), p3));
      const double d20 = len3(sub(closest_on_segment(p3, p2, p0), p3));
      if (d01 > max_app && d12 > max_app && d20 > max_app) return 0;
    }
  }
  t = coplanar_time(p0, p1, p2, p3, q0, q1, q2, q3);
  if (t < 0 || t > 1) return 0;
  dist_face_vertex(lerp(t, p0, q0), lerp(t, p1, q1), lerp(t, p2, q2), lerp(t, p3, q3), &w0, &w1);
  w2 = 1 - w0 - w1;
  if (w0 < 0 || w0 > 1) return 0;
  if (w1 < 0 || w1 > 1) return 0;
  if (w2 < 0 || w2 > 1) return 0;
  return 1;
}

/* IsContact_EE_CCD :723-793 */
static int ee_ccd(int i0, int i1, int j0, int j1, vec3 p0s, vec3 p1s, vec3 q0s, vec3 q1s, vec3 p0e, vec3 p1e,
                  vec3 q0e, vec3 q1e) {
  const double eps = 1.0e-10;
  box3 bq, bp;
  double t, w0, w1, dist;
  if (i0 == j0 || i0 == j1 || i1 == j0 || i1 == j1) return 0;
  box_clear(&bq);
  box_add_point(&bq, q0s, eps);
  box_add_point(&bq, q1s, eps);
  box_add_point(&bq, q0e, eps);
  box_add_point(&bq, q1e, eps);
  box_clear(&bp);
  box_add_point(&bp, p0s, eps);
  box_add_point(&bp, p1s, eps);
  box_add_point(&bp, p0e, eps);
  box_add_point(&bp, p1e, eps);
  if (!box_overlap(&bp, &bq)) return 0;
  t = coplanar_time(p0s, p1s, q0s, q1s, p0e, p1e, q0e, q1e);
  if (t < 0 || t > 1) return 0;
  dist = dist_edge_edge(lerp(t, p0s, p0e), lerp(t, p1s, p1e), lerp(t, q0s, q0e), lerp(t, q1s, q1e), &w0, &w1);
  if (w0 < 0 || w0 > 1) return 0;
  if (w1 < 0 || w1 > 1) return 0;
  if (dist > 1.0e-2) return 0;
  return 1;
}

/* ======================================================================== */
/* contact sets (bvh_aabb.h:65-106, bvh_aabb.cpp:441-557, 797-923)           */
/* ======================================================================== */

typedef struct {
  int k[4];
  int fv;
  int seq; /* insertion order */
} celem;

typedef struct {
  celem *a;
  int n, cap;
} cset;

/* canonical key of a contact element, CContactElement ctor, bvh_aabb.h:68-93:
 * face-vertex: face sorted ascending, then the vertex; edge-edge: smallest index
 * first with its edge partner, then the other edge sorted. */
static void cset_push(cset *s, int fv, int j0, int j1, int j2, int j3) {
  celem e;
  if (s->n == s->cap) {
    s->cap = s->cap ? 2 * s->cap : 256;
    s->a = (celem *)realloc(s->a, sizeof(celem) * (size_t)s->cap);
    if (!s->a) abort();
  }
  e.fv = fv;
  if (fv) {
    int a = j0, b = j1, c = j2, t;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
    e.k[0] = a; e.k[1] = b; e.k[2] = c; e.k[3] = j3;
  } else {
    int m0, m1, o0, o1;
    const int lo01 = j0 < j1 ? j0 : j1, lo23 = j2 < j3 ? j2 : j3;
    if (lo01 < lo23) {
      m0 = lo01; m1 = (j0 < j1) ? j1 : j0; o0 = j2; o1 = j3;
    } else {
      m0 = lo23; m1 = (j2 < j3) ? j3 : j2; o0 = j0; o1 = j1;
    }
    e.k[0] = m0; e.k[1] = m1;
    e.k[2] = o0 < o1 ? o0 : o1; e.k[3] = o0 < o1 ? o1 : o0;
  }
  e.seq = s->n;
  s->a[s->n++] = e;
}

static int celem_cmp(const void *pa, const void *pb) {
  const celem *a = (const celem *)pa, *b = (const celem *)pb;
  int i;
  for (i = 0; i < 4; i++)
    if (a->k[i] != b->k[i]) return a->k[i] < b->k[i] ? -1 : 1;
  return (a->seq > b->seq) - (a->seq < b->seq);
}

/* std::set semantics: ordered by the 4 indices only, the first insertion of a
 * key is kept (is_fv is not part of the key). */
static int cset_finish(cset *s, int *out, int cap) {
  int i, n = 0;
  qsort(s->a, (size_t)s->n, sizeof(celem), celem_cmp);
  for (i = 0; i < s->n; i++) {
    if (n > 0 && i > 0 && memcmp(s->a[i].k, s->a[i - 1].k, sizeof(int) * 4) == 0) continue;
    if (out && n < cap) {
      out[n * 5 + 0] = s->a[i].fv;
      out[n * 5 + 1] = s->a[i].k[0];
      out[n * 5 + 2] = s->a[i].k[1];
      out[n * 5 + 3] = s->a[i].k[2];
      out[n * 5 + 4] = s->a[i].k[3];
    }
    n++;
  }
  return n;
}

typedef struct {
  co_cloth *h;
  const double *x, *v;
  double dt, delta;
  int ccd;
  cset *out;
} walk_ctx;

/* the 9 edge pairs tested per triangle pair: (edge of a) x (edge of b) */
static const int kEE[9][4] = {{0, 1, 0, 1}, {0, 1, 1, 2}, {0, 1, 2, 0}, {1, 2, 0, 1}, {1, 2, 1, 2},
                              {1, 2, 2, 0}, {2, 0, 0, 1}, {2, 0, 1, 2}, {2, 0, 2, 0}};

/* The 15 elementary tests of one leaf pair (na holds triangle a, nb holds b) in
 * the reference's order, bvh_aabb.cpp:473-536 (proximity) and 836-901 (CCD). */
static void leaf_pair(walk_ctx *W, int na, int nb) {
  co_cloth *h = W->h;
  const int ta = h->node[na * 3 + 1], tb = h->node[nb * 3 + 1];
  const int *ia = h->tri + ta * 3, *ib = h->tri + tb * 3;
  vec3 P[3], Q[3], Pe[3], Qe[3];
  int k;
  for (k = 0; k < 3; k++) {
    P[k] = at(W->x, ia[k]);
    Q[k] = at(W->x, ib[k]);
  }
  if (!W->ccd) {
    const box3 *ba = h->bb + ta, *bbx = h->bb + tb; /* triangle index used as a node index */
    for (k = 0; k < 3; k++)
      if (fv_proximity(ia[0], ia[1], ia[2], ib[k], P[0], P[1], P[2], Q[k], ba, W->delta))
        cset_push(W->out, 1, ia[0], ia[1], ia[2], ib[k]);
    for (k = 0; k < 3; k++)
      if (fv_proximity(ib[0], ib[1], ib[2], ia[k], Q[0], Q[1], Q[2], P[k], bbx, W->delta))
        cset_push(W->out, 1, ib[0], ib[1], ib[2], ia[k]);
    for (k = 0; k < 9; k++) {
      const int *e = kEE[k];
      if (ee_proximity(ia[e[0]], ia[e[1]], ib[e[2]], ib[e[3]], P[e[0]], P[e[1]], Q[e[2]], Q[e[3]], W->delta))
        cset_push(W->out, 0, ia[e[0]], ia[e[1]], ib[e[2]], ib[e[3]]);
    }
  } else {
    const double dt = W->dt;
    const double *x = W->x, *v = W->v;
    for (k = 0; k < 3; k++) {
      int p = ia[k], q = ib[k];
      Pe[k] = mk(x[p * 3 + 0] + dt * v[p * 3 + 0], x[p * 3 + 1] + dt * v[p * 3 + 1], x[p * 3 + 2] + dt * v[p * 3 + 2]);
      Qe[k] = mk(x[q * 3 + 0] + dt * v[q * 3 + 0], x[q * 3 + 1] + dt * v[q * 3 + 1], x[q * 3 + 2] + dt * v[q * 3 + 2]);
    }
    for (k = 0; k < 3; k++)
      if (fv_ccd(ia[0], ia[1], ia[2], ib[k], P[0], P[1], P[2], Q[k], Pe[0], Pe[1], Pe[2], Qe[k], h->bb + na))
        cset_push(W->out, 1, ia[0], ia[1], ia[2], ib[k]);
    for (k = 0; k < 3; k++)
      if (fv_ccd(ib[0], ib[1], ib[2], ia[k], Q[0], Q[1], Q[2], P[k], Qe[0], Qe[1], Qe[2], Pe[k], h->bb + nb))
        cset_push(W->out, 1, ib[0], ib[1], ib[2], ia[k]);
    for (k = 0; k < 9; k++) {
      const int *e = kEE[k];
      if (ee_ccd(ia[e[0]], ia[e[1]], ib[e[2]], ib[e[3]], P[e[0]], P[e[1]], Q[e[2]], Q[e[3]], Pe[e[0]], Pe[e[1]],
                 Qe[e[2]], Qe[e[3]]))
        cset_push(W->out, 0, ia[e[0]], ia[e[1]], ib[e[2]], ib[e[3]]);
    }
  }
}

/* simultaneous descent of two subtrees, GetContactElement_* (pair) :441-472, :797-835 */
static void walk_pair(walk_ctx *W, int a, int b) {
  const int *N = W->h->node;
  if (!box_overlap(W->h->bb + a, W->h->bb + b)) return;
  {
    const int a0 = N[a * 3 + 1], a1 = N[a * 3 + 2], b0 = N[b * 3 + 1], b1 = N[b * 3 + 2];
    const int la = (a1 == -1), lb = (b1 == -1);
    if (!la && !lb) {
      walk_pair(W, a0, b0);
      walk_pair(W, a1, b0);
      walk_pair(W, a0, b1);
      walk_pair(W, a1, b1);
    } else if (!la && lb) {
      walk_pair(W, a0, b);
      walk_pair(W, a1, b);
    } else if (la && !lb) {
      walk_pair(W, a, b0);
      walk_pair(W, a, b1);
    } else {
      leaf_pair(W, a, b);
    }
  }
}

/* self pairs within a subtree, GetContactElement_* (self) :540-557, :904-923 */
static void walk_self(walk_ctx *W, int n) {
  const int c0 = W->h->node[n * 3 + 1], c1 = W->h->node[n * 3 + 2];
  if (c1 == -1) return;
  walk_pair(W, c0, c1);
  walk_self(W, c0);
  walk_self(W, c1);
}

static int collect(co_cloth *h, const double *x, const double *v, double dt, double delta, int ccd, int *out, int cap) {
  cset s;
  walk_ctx W;
  int n;
  memset(&s, 0, sizeof(s));
  W.h = h;
  W.x = x;
  W.v = v;
  W.dt = dt;
  W.delta = delta;
  W.ccd = ccd;
  W.out = &s;
  walk_self(&W, 0);
  n = cset_finish(&s, out, cap);
  free(s.a);
  return n;
}

/* DistanceFaceVertex / DistanceEdgeEdge / FindCoplanerInterp
 * (bvh_aabb.cpp:321-384, 598-662) on 12 doubles of points */
double co_distance_fv(const double *p, double *w) {
  return dist_face_vertex(at(p, 0), at(p, 1), at(p, 2), at(p, 3), w, w + 1);
}
double co_distance_ee(const double *p, double *r) {
  return dist_edge_edge(at(p, 0), at(p, 1), at(p, 2), at(p, 3), r, r + 1);
}
double co_coplanar_time(const double *s, const double *e) {
  return coplanar_time(at(s, 0), at(s, 1), at(s, 2), at(s, 3), at(e, 0), at(e, 1), at(e, 2), at(e, 3));
}

void co_fv_ccd_batch(int n, const double *p, const double *box, int *out) {
  box3 bb;
  int i, k;
  for (k = 0; k < 3; k++) {
    bb.lo[k] = box[k];
    bb.hi[k] = box[3 + k];
  }
  bb.full = 1;
  for (i = 0; i < n; i++) {
    const double *a = p + 24 * (size_t)i;
    out[i] = fv_ccd(0, 1, 2, 3, at(a, 0), at(a, 1), at(a, 2), at(a, 3), at(a, 4), at(a, 5), at(a, 6), at(a, 7), &bb);
  }
}
void co_ee_ccd_batch(int n, const double *p, int *out) {
  int i;
  for (i = 0; i < n; i++) {
    const double *a = p + 24 * (size_t)i;
    out[i] = ee_ccd(0, 1, 2, 3, at(a, 0), at(a, 1), at(a, 2), at(a, 3), at(a, 4), at(a, 5), at(a, 6), at(a, 7));
  }
}

int co_contacts_prx(co_cloth *h, const double *x, double delta, int *out, int cap) {
  co_refit_prx(h, x, delta, NULL);
  return collect(h, x, NULL, 0, delta, 0, out, cap);
}

int co_contacts_ccd(co_cloth *h, const double *x, const double *v, double dt, double delta, int *out, int cap) {
  co_refit_ccd(h, x, v, dt, NULL);
  return collect(h, x, v, dt, delta, 1, out, cap);
}

/* ======================================================================== */
/* impulses (self_collision_cloth.cpp:20-212)                                */
/* ======================================================================== */

static void add_vel(double *v, int i, vec3 d) {
  v[i * 3 + 0] += d.x;
  v[i * 3 + 1] += d.y;
  v[i * 3 + 2] += d.z;
}

/* Sequential impulses over the contacts in set order,
 * SelfCollisionImpulse_Proximity (ccd = 0) / SelfCollisionImpulse_CCD (ccd = 1). */
static void impulses(co_cloth *h, const double *x, double *v, const int *ce, int nce, int ccd) {
  const co_params *q = &h->prm;
  const double delta = q->contact_clearance, stiff = q->stiff_contact, dt = q->dt, mass = q->mass_point;
  int c;
  for (c = 0; c < nce; c++) {
    const int *e = ce + c * 5;
    const int i0 = e[1], i1 = e[2], i2 = e[3], i3 = e[4];
    const vec3 p0 = at(x, i0), p1 = at(x, i1), p2 = at(x, i2), p3 = at(x, i3);
    const vec3 v0 = at(v, i0), v1 = at(v, i1), v2 = at(v, i2), v3 = at(v, i3);
    double t = 0;
    if (ccd) {
      t = coplanar_time(p0, p1, p2, p3, add(p0, v0), add(p1, v1), add(p2, v2), add(p3, v3));
      if (t < 0 || t > 1) continue;
    }
    if (e[0]) { /* face (i0 i1 i2) - vertex i3 */
      double w0, w1, w2, dist, rel_v, imp_mod;
      vec3 pc, nrm;
      if (ccd)
        dist = dist_face_vertex(add(p0, scl(t, v0)), add(p1, scl(t, v1)), add(p2, scl(t, v2)), add(p3, scl(t, v3)),
                                &w0, &w1);
      else
        dist = dist_face_vertex(p0, p1, p2, p3, &w0, &w1);
      if (w0 < 0 || w0 > 1) continue;
      if (w1 < 0 || w1 > 1) continue;
      if (dist > delta) continue;
      w2 = 1.0 - w0 - w1;
      pc = add(add(scl(w0, p0), scl(w1, p1)), scl(w2, p2));
      nrm = normalized(sub(p3, pc));
      rel_v = dot(sub(sub(sub(v3, scl(w0, v0)), scl(w1, v1)), scl(w2, v2)), nrm);
      if (!ccd) {
        const double depth = delta - dot(sub(p3, pc), nrm);
        if (rel_v > 0.1 * depth / dt) continue;
        const double imp_el = dt * stiff * depth;
        const double imp_ie = mass * (0.1 * depth / dt - rel_v);
        const double imp_min = (imp_el < imp_ie) ? imp_el : imp_ie;
        imp_mod = 2 * imp_min / (1 + w0 * w0 + w1 * w1 + w2 * w2);
        imp_mod /= mass;
        imp_mod *= 0.25;
      } else {
        if (rel_v > 0.1 * delta / dt) continue;
        const double imp = mass * (0.1 * delta / dt - rel_v);
        imp_mod = 2 * imp / (1.0 + w0 * w0 + w1 * w1 + w2 * w2);
        imp_mod /= mass;
        imp_mod *= 0.1;
      }
      {
        const vec3 m = mk(-nrm.x, -nrm.y, -nrm.z);
        add_vel(v, i0, mk(m.x * imp_mod * w0, m.y * imp_mod * w0, m.z * imp_mod * w0));
        add_vel(v, i1, mk(m.x * imp_mod * w1, m.y * imp_mod * w1, m.z * imp_mod * w1));
        add_vel(v, i2, mk(m.x * imp_mod * w2, m.y * imp_mod * w2, m.z * imp_mod * w2));
        add_vel(v, i3, mk(nrm.x * imp_mod, nrm.y * imp_mod, nrm.z * imp_mod));
      }
    } else { /* edge (i0 i1) - edge (i2 i3) */
      double w01, w23, dist, rel_v, imp_mod;
      vec3 c01, c23, nrm;
      if (ccd)
        dist = dist_edge_edge(add(p0, scl(t, v0)), add(p1, scl(t, v1)), add(p2, scl(t, v2)), add(p3, scl(t, v3)), &w01,
                              &w23);
      else
        dist = dist_edge_edge(p0, p1, p2, p3, &w01, &w23);
      if (w01 < 0 || w01 > 1) continue;
      if (w23 < 0 || w23 > 1) continue;
      if (dist > delta) continue;
      c01 = add(scl(1 - w01, p0), scl(w01, p1));
      c23 = add(scl(1 - w23, p2), scl(w23, p3));
      nrm = normalized(sub(c23, c01));
      rel_v = dot(sub(sub(add(scl(1 - w23, v2), scl(w23, v3)), scl(1 - w01, v0)), scl(w01, v1)), nrm);
      {
        const double wsum = w01 * w01 + (1 - w01) * (1 - w01) + w23 * w23 + (1 - w23) * (1 - w23);
        if (!ccd) {
          const double depth = delta - len3(sub(c23, c01));
          if (rel_v > 0.1 * depth / dt) continue;
          const double imp_el = dt * stiff * depth;
          const double imp_ie = mass * (0.1 * depth / dt - rel_v);
          const double imp_min = (imp_el < imp_ie) ? imp_el : imp_ie;
          imp_mod = 2 * imp_min / wsum;
          imp_mod /= mass;
          imp_mod *= 0.25;
        } else {
          if (rel_v > 0.1 * delta / dt) continue;
          const double imp = mass * (0.1 * delta / dt - rel_v);
          imp_mod = 2 * imp / wsum;
          imp_mod /= mass;
          imp_mod *= 0.1;
        }
      }
      {
        const vec3 m = mk(-nrm.x, -nrm.y, -nrm.z);
        add_vel(v, i0, mk(m.x * imp_mod * (1 - w01), m.y * imp_mod * (1 - w01), m.z * imp_mod * (1 - w01)));
        add_vel(v, i1, mk(m.x * imp_mod * w01, m.y * imp_mod * w01, m.z * imp_mod * w01));
        add_vel(v, i2, mk(nrm.x * imp_mod * (1 - w23), nrm.y * imp_mod * (1 - w23), nrm.z * imp_mod * (1 - w23)));
        add_vel(v, i3, mk(nrm.x * imp_mod * w23, nrm.y * imp_mod * w23, nrm.z * imp_mod * w23));
      }
    }
  }
}

void co_impulse_prx(co_cloth *h, const double *x, double *v, const int *ce, int n) { impulses(h, x, v, ce, n, 0); }
void co_impulse_ccd(co_cloth *h, const double *x, double *v, const int *ce, int n) { impulses(h, x, v, ce, n, 1); }

/* ======================================================================== */
/* rigid impact zones (self_collision_cloth.cpp:220-348)                     */
/* ======================================================================== */

static void zone_insert(zone_t *z, int v) {
  int lo = 0, hi = z->n;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (z->mem[m] < v)
      lo = m + 1;
    else
      hi = m;
  }
  if (lo < z->n && z->mem[lo] == v) return;
  if (z->n == z->cap) {
    z->cap = z->cap ? 2 * z->cap : 8;
    z->mem = (int *)realloc(z->mem, sizeof(int) * (size_t)z->cap);
    if (!z->mem) abort();
  }
  memmove(z->mem + lo + 1, z->mem + lo, sizeof(int) * (size_t)(z->n - lo));
  z->mem[lo] = v;
  z->n++;
}

static void zones_reindex(co_cloth *h) {
  int z, i;
  for (i = 0; i < h->np; i++) h->zone_of[i] = -1;
  for (z = 0; z < h->nzone; z++)
    for (i = 0; i < h->zones[z].n; i++) h->zone_of[h->zones[z].mem[i]] = z;
}

/* MakeRigidImpactZone :220-274: each contact joins every zone holding one of
 * its vertices or a 1-ring neighbour of one; touching several merges them
 * (untouched zones keep their order, the merged zone goes last). */
void co_riz_add(co_cloth *h, const int *ce, int nce) {
  int c, k, j, z;
  int *hit = (int *)xcalloc((size_t)h->nzone + (size_t)nce + 1, sizeof(int));
  for (c = 0; c < nce; c++) {
    const int *n = ce + c * 5 + 1;
    int nhit = 0, first = -1;
    for (z = 0; z < h->nzone; z++) hit[z] = 0;
    for (k = 0; k < 4; k++) {
      const int v = n[k];
      if (h->zone_of[v] >= 0) hit[h->zone_of[v]] = 1;
      for (j = h->ring_ptr[v]; j < h->ring_ptr[v + 1]; j++) {
        const int w = h->ring[j];
        if (h->zone_of[w] >= 0) hit[h->zone_of[w]] = 1;
      }
    }
    for (z = 0; z < h->nzone; z++)
      if (hit[z]) {
        nhit++;
        if (first < 0) first = z;
      }
    if (nhit == 0) {
      if (h->nzone == h->zcap) {
        h->zcap = h->zcap ? 2 * h->zcap : 8;
        h->zones = (zone_t *)realloc(h->zones, sizeof(zone_t) * (size_t)h->zcap);
        if (!h->zones) abort();
      }
      memset(h->zones + h->nzone, 0, sizeof(zone_t));
      for (k = 0; k < 4; k++) {
        zone_insert(h->zones + h->nzone, n[k]);
        h->zone_of[n[k]] = h->nzone;
      }
      h->nzone++;
    } else if (nhit == 1) {
      for (k = 0; k < 4; k++) {
        zone_insert(h->zones + first, n[k]);
        h->zone_of[n[k]] = first;
      }
    } else {
      zone_t merged;
      int nz = 0, i;
      memset(&merged, 0, sizeof(merged));
      for (z = 0; z < h->nzone; z++) {
        if (hit[z]) {
          for (i = 0; i < h->zones[z].n; i++) zone_insert(&merged, h->zones[z].mem[i]);
          free(h->zones[z].mem);
        } else {
          h->zones[nz++] = h->zones[z];
        }
      }
      for (k = 0; k < 4; k++) zone_insert(&merged, n[k]);
      h->zones[nz++] = merged;
      h->nzone = nz;
      zones_reindex(h);
    }
    hit = (int *)realloc(hit, sizeof(int) * ((size_t)h->nzone + (size_t)nce + 1));
  }
  free(hit);
}

int co_riz_zones(const co_cloth *h, int *zone_of_vertex) {
  memcpy(zone_of_vertex, h->zone_of, sizeof(int) * (size_t)h->np);
  return h->nzone;
}

/* Rigid-body velocity of each zone from the pre-zone velocities v0,
 * ApplyRigidImpactZone :298-348 (its "inertia" diagonal uses |v|^2). */
void co_riz_apply(co_cloth *h, const double *x, double *v, const double *v0) {
  int z, i;
  for (z = 0; z < h->nzone; z++) {
    const zone_t *Z = h->zones + z;
    vec3 gc = mk(0, 0, 0), av = mk(0, 0, 0), L = mk(0, 0, 0), omg;
    double I[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, Iinv[9];
    for (i = 0; i < Z->n; i++) {
      gc = add(gc, at(x, Z->mem[i]));
      av = add(av, at(v0, Z->mem[i]));
    }
    gc = div_guarded(gc, (double)Z->n);
    av = div_guarded(av, (double)Z->n);
    for (i = 0; i < Z->n; i++) {
      const vec3 p = at(x, Z->mem[i]), u = at(v0, Z->mem[i]);
      const vec3 q = sub(p, gc);
      const double uu = dot(u, u);
      L = add(L, cross(sub(p, gc), sub(u, av)));
      I[0] += uu - q.x * q.x;
      I[1] += -q.x * q.y;
      I[2] += -q.x * q.z;
      I[3] += -q.y * q.x;
      I[4] += uu - q.y * q.y;
      I[5] += -q.y * q.z;
      I[6] += -q.z * q.x;
      I[7] += -q.z * q.y;
      I[8] += uu - q.z * q.z;
    }
    inv33(Iinv, I);
    omg = mk(Iinv[0] * L.x + Iinv[1] * L.y + Iinv[2] * L.z, Iinv[3] * L.x + Iinv[4] * L.y + Iinv[5] * L.z,
             Iinv[6] * L.x + Iinv[7] * L.y + Iinv[8] * L.z);
    for (i = 0; i < Z->n; i++) {
      const int m = Z->mem[i];
      const vec3 r = cross(sub(at(x, m), gc), omg);
      v[m * 3 + 0] = av.x + (-r.x);
      v[m * 3 + 1] = av.y + (-r.y);
      v[m * 3 + 2] = av.z + (-r.z);
    }
  }
}

/* ======================================================================== */
/* contact resolution and the frame (self_collision_cloth.cpp:355-456,        */
/* solve_internal_sparse.h:329-369, self_contact_sparse/main.cpp:213-263)     */
/* ======================================================================== */

static int *grow_ce(int *buf, int *cap, int need) {
  if (need <= *cap) return buf;
  while (*cap < need) *cap = *cap ? 2 * *cap : 1024;
  buf = (int *)realloc(buf, sizeof(int) * 5 * (size_t)*cap);
  if (!buf) abort();
  return buf;
}

/* FNV-1a over the 32-bit words of an ordered contact list (5 words a contact) */
unsigned long long co_contact_digest(const int *ce, int n) {
  unsigned long long d = 14695981039346656037ULL;
  long long i;
  for (i = 0; i < 5LL * n; i++) {
    d ^= (unsigned long long)(unsigned int)ce[i];
    d *= 1099511628211ULL;
  }
  return d;
}

static void log_detection(co_cloth *h, int ccd, const int *ce, int n) {
  if (!h->log_on) return;
  if (h->log_n == h->log_cap) {
    h->log_cap = h->log_cap ? 2 * h->log_cap : 16;
    h->log_kind = (int *)realloc(h->log_kind, sizeof(int) * (size_t)h->log_cap);
    h->log_count = (int *)realloc(h->log_count, sizeof(int) * (size_t)h->log_cap);
    h->log_digest = (unsigned long long *)realloc(h->log_digest, sizeof(unsigned long long) * (size_t)h->log_cap);
    if (!h->log_kind || !h->log_count || !h->log_digest) abort();
  }
  h->log_kind[h->log_n] = ccd;
  h->log_count[h->log_n] = n;
  h->log_digest[h->log_n] = co_contact_digest(ce, n);
  h->log_n++;
}

void co_contact_log(co_cloth *h, int enable) {
  h->log_on = enable != 0;
  h->log_n = 0;
}

int co_contact_log_read(const co_cloth *h, int *kind, int *count, unsigned long long *digest, int cap) {
  int i;
  for (i = 0; i < h->log_n && i < cap; i++) {
    kind[i] = h->log_kind[i];
    count[i] = h->log_count[i];
    digest[i] = h->log_digest[i];
  }
  return h->log_n;
}

static int contacts_alloc(co_cloth *h, const double *x, const double *v, int ccd, int **buf, int *cap) {
  const co_params *q = &h->prm;
  int n;
  if (ccd) {
    co_refit_ccd(h, x, v, q->dt, NULL);
    n = collect(h, x, v, q->dt, q->contact_clearance, 1, *buf, *cap);
  } else {
    co_refit_prx(h, x, q->contact_clearance, NULL);
    n = collect(h, x, NULL, 0, q->contact_clearance, 0, *buf, *cap);
  }
  if (n > *cap) {
    *buf = grow_ce(*buf, cap, n);
    n = collect(h, x, v, q->dt, q->contact_clearance, ccd, *buf, *cap);
  }
  log_detection(h, ccd, *buf, n);
  return n;
}

/* GetIntermidiateVelocityContactResolved: proximity impulses, up to 5 CCD
 * impulse passes, then up to 100 rigid-impact-zone passes. */
void co_resolve(co_cloth *h, const double *x1, double *v, co_stats *st) {
  int cap = 0, n, it, i;
  int *ce = NULL;
  co_stats s;
  memset(&s, 0, sizeof(s));
  h->log_n = 0;
  if (st) {
    s.solver_iterations = st->solver_iterations;
    s.solver_conv = st->solver_conv;
    s.ilu_singular = st->ilu_singular;
  }
  ce = grow_ce(ce, &cap, 1024);
  n = contacts_alloc(h, x1, NULL, 0, &ce, &cap);
  s.n_prx = n;
  s.impulse_applied = n > 0;
  co_impulse_prx(h, x1, v, ce, n);
  for (it = 0; it < 5; it++) {
    n = contacts_alloc(h, x1, v, 1, &ce, &cap);
    s.n_ccd[it] = n;
    s.n_ccd_passes = it + 1;
    if (n == 0) goto done;
    s.impulse_applied = 1;
    co_impulse_ccd(h, x1, v, ce, n);
  }
  {
    double *v0 = (double *)xmalloc(sizeof(double) * 3 * (size_t)h->np);
    memcpy(v0, v, sizeof(double) * 3 * (size_t)h->np);
    co_riz_reset(h);
    for (it = 0; it < 100; it++) {
      n = contacts_alloc(h, x1, v, 1, &ce, &cap);
      s.n_riz_passes++;
      s.n_riz_last = n;
      s.n_riz_total += n;
      s.riz_nodes = 0;
      for (i = 0; i < h->nzone; i++) s.riz_nodes += h->zones[i].n;
      if (n == 0) break;
      co_riz_add(h, ce, n);
      co_riz_apply(h, x1, v, v0);
    }
    free(v0);
  }
done:
  free(ce);
  if (st) *st = s;
}

/* MakeNormal, self_contact_sparse/main.cpp:183-211: every triangle's unit
 * normal (UnitNormalAreaTri3D) added to its three vertices in triangle order,
 * then each sum scaled by 1 / sqrt(|sum|^2) */
void co_vertex_normals(const co_cloth *h, const double *x, double *nrm) {
  int t, i;
  for (i = 0; i < 3 * h->np; i++) nrm[i] = 0.0;
  for (t = 0; t < h->nt; t++) {
    const int *f = h->tri + 3 * t;
    double n[3], area;
    int k;
    unit_normal_area3(n, &area, x + 3 * f[0], x + 3 * f[1], x + 3 * f[2]);
    for (k = 0; k < 3; k++) {
      nrm[3 * f[k] + 0] += n[0];
      nrm[3 * f[k] + 1] += n[1];
      nrm[3 * f[k] + 2] += n[2];
    }
  }
  for (i = 0; i < h->np; i++) {
    double *m = nrm + 3 * i;
    const double sq = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
    const double inv = 1.0 / sqrt(sq);
    m[0] *= inv;
    m[1] *= inv;
    m[2] *= inv;
  }
}

/* UpdateIntermidiateVelocity, solve_internal_sparse.h:329-369 */
void co_update_velocity(co_cloth *h, const double *x, double *v) {
  const co_params *q = &h->prm;
  double *g = h->tmp0;
  int i;
  memset(g, 0, sizeof(double) * 3 * (size_t)h->np);
  add_cloth_terms(h, x, g, 0);
  add_gravity(h, g);
  for (i = 0; i < h->np; i++)
    if (h->bc[i]) v[i * 3 + 0] = v[i * 3 + 1] = v[i * 3 + 2] = 0;
  for (i = 0; i < 3 * h->np; i++) v[i] += -(0.5 * q->dt / q->mass_point) * g[i];
}

/* StepTime, self_contact_sparse/main.cpp:213-263 (normals are render-only) */
void co_step(co_cloth *h, double *x, double *v, co_stats *st) {
  const int n = 3 * h->np;
  double *x1 = (double *)xmalloc(sizeof(double) * (size_t)n);
  co_stats s;
  int i;
  memset(&s, 0, sizeof(s));
  memcpy(x1, x, sizeof(double) * (size_t)n);
  co_implicit(h, x, v, &s);
  co_resolve(h, x1, v, &s);
  if (s.impulse_applied) {
    for (i = 0; i < n; i++) x[i] = x1[i] + v[i] * h->prm.dt;
    co_update_velocity(h, x, v);
  }
  free(x1);
  if (st) *st = s;
}
