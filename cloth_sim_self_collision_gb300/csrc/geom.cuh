// geom.cuh -- device geometry of the cloth step.
//
// Every floating-point expression keeps the operand order and association of
// the reference (vector3d.h, utility.h, aabb.h, bvh_aabb.cpp,
// cloth_internal_physics.h, self_collision_cloth.cpp).  The library is built
// with -fmad=false, so in double precision these functions round exactly like
// the reference's IEEE double code.  The templates also instantiate in float
// for the mixed-precision bulk path.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#define CS_HD __host__ __device__ __forceinline__

namespace cs {

template <typename T>
struct V3 {
  T x, y, z;
};

template <typename T>
CS_HD V3<T> mk(T x, T y, T z) {
  V3<T> r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
template <typename T>
CS_HD V3<T> ld3(const T* a, int i) {
  return mk<T>(a[3 * i + 0], a[3 * i + 1], a[3 * i + 2]);
}
template <typename T>
CS_HD V3<T> operator+(V3<T> a, V3<T> b) {
  return mk<T>(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <typename T>
CS_HD V3<T> operator-(V3<T> a, V3<T> b) {
  return mk<T>(a.x - b.x, a.y - b.y, a.z - b.z);
}
// scalar * vector scales each component (vector3d.h:143-148)
template <typename T>
CS_HD V3<T> operator*(T s, V3<T> a) {
  return mk<T>(a.x * s, a.y * s, a.z * s);
}
template <typename T>
CS_HD T dot(V3<T> a, V3<T> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
CS_HD V3<T> cross(V3<T> a, V3<T> b) {
  return mk<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename T>
CS_HD T length(V3<T> a) {
  return sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
}
// SetNormalizedVector: multiply by the reciprocal length (vector3d.h:96-102)
template <typename T>
CS_HD V3<T> normalized(V3<T> a) {
  const T inv = T(1) / length(a);
  return mk<T>(a.x * inv, a.y * inv, a.z * inv);
}
// operator/= ignores divisors below 1e-16 (vector3d.h:63-67)
template <typename T>
CS_HD V3<T> div_guarded(V3<T> a, T d) {
  if (fabs(d) < T(1.e-16)) return a;
  return mk<T>(a.x / d, a.y / d, a.z / d);
}
// ScalarTripleProduct (vector3d.h:216-218)
template <typename T>
CS_HD T stp(V3<T> a, V3<T> b, V3<T> c) {
  return a.x * (b.y * c.z - b.z * c.y) + a.y * (b.z * c.x - b.x * c.z) + a.z * (b.x * c.y - b.y * c.x);
}
// Height of v4 over the plane of v1 v2 v3 (vector3d.h:254-267)
template <typename T>
CS_HD T height4(V3<T> v1, V3<T> v2, V3<T> v3, V3<T> v4) {
  T nx = (v2.y - v1.y) * (v3.z - v1.z) - (v2.z - v1.z) * (v3.y - v1.y);
  T ny = (v2.z - v1.z) * (v3.x - v1.x) - (v2.x - v1.x) * (v3.z - v1.z);
  T nz = (v2.x - v1.x) * (v3.y - v1.y) - (v2.y - v1.y) * (v3.x - v1.x);
  const T inv = T(1) / sqrt(nx * nx + ny * ny + nz * nz);
  nx *= inv;
  ny *= inv;
  nz *= inv;
  return (v4.x - v1.x) * nx + (v4.y - v1.y) * ny + (v4.z - v1.z) * nz;
}
// closest point of segment s-e to p (vector3d.h:282-295)
template <typename T>
CS_HD V3<T> closest_on_segment(V3<T> p, V3<T> s, V3<T> e) {
  const V3<T> d = e - s;
  const T a = dot(d, d);
  const T b = dot(d, s - p);
  T t = -b / a;
  if (t < 0) t = 0;
  if (t > 1) t = 1;
  return s + t * d;
}
template <typename T>
CS_HD V3<T> lerp(T t, V3<T> a, V3<T> b) {
  return (T(1) - t) * a + t * b;
}

// ---------------------------------------------------------------------------
// boxes (aabb.h:16-148)
// ---------------------------------------------------------------------------
struct Box {
  double lo[3], hi[3];
  int full;
};

CS_HD void box_clear(Box& b) {
  b.lo[0] = b.lo[1] = b.lo[2] = 0;
  b.hi[0] = b.hi[1] = b.hi[2] = 0;
  b.full = 0;
}
// AddPoint(x, y, z, eps), aabb.h:102-122
CS_HD void box_add(Box& b, V3<double> p, double eps) {
  const double q[3] = {p.x, p.y, p.z};
  if (eps <= 0) return;
  if (b.full) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      b.lo[k] = (b.lo[k] < q[k] - eps) ? b.lo[k] : q[k] - eps;
      b.hi[k] = (b.hi[k] > q[k] + eps) ? b.hi[k] : q[k] + eps;
    }
  } else {
    b.full = 1;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      b.lo[k] = q[k] - eps;
      b.hi[k] = q[k] + eps;
    }
  }
}
// operator+=(box), aabb.h:55-72
CS_HD void box_merge(Box& b, const Box& o) {
  if (!o.full) return;
  if (!b.full) {
    b = o;
    return;
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    b.hi[k] = (b.hi[k] > o.hi[k]) ? b.hi[k] : o.hi[k];
    b.lo[k] = (b.lo[k] < o.lo[k]) ? b.lo[k] : o.lo[k];
  }
}
// IsIntersect, aabb.h:73-84 (closed intervals)
CS_HD bool box_overlap(const Box& a, const Box& b) {
  if (!a.full || !b.full) return false;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if (a.hi[k] < b.lo[k]) return false;
    if (a.lo[k] > b.hi[k]) return false;
  }
  return true;
}
// IsInside, aabb.h:137-144
CS_HD bool box_inside(const Box& b, V3<double> p) {
  if (!b.full) return false;
  return p.x >= b.lo[0] && p.x <= b.hi[0] && p.y >= b.lo[1] && p.y <= b.hi[1] && p.z >= b.lo[2] &&
         p.z <= b.hi[2];
}

// ---------------------------------------------------------------------------
// distances and the coplanarity time (bvh_aabb.cpp:321-384, 563-662)
// ---------------------------------------------------------------------------
// barycentric weights of p3 projected on plane p0 p1 p2, and the distance
template <typename T>
CS_HD T dist_face_vertex(V3<T> p0, V3<T> p1, V3<T> p2, V3<T> p3, T& w0, T& w1) {
  const V3<T> v20 = p0 - p2, v21 = p1 - p2;
  const T t0 = dot(v20, v20), t1 = dot(v21, v21), t2 = dot(v20, v21);
  const T t3 = dot(v20, p3 - p2), t4 = dot(v21, p3 - p2);
  const T det = t0 * t1 - t2 * t2;
  const T invdet = T(1) / det;
  w0 = (+t1 * t3 - t2 * t4) * invdet;
  w1 = (-t2 * t3 + t0 * t4) * invdet;
  const T w2 = 1 - w0 - w1;
  const V3<T> pw = w0 * p0 + w1 * p1 + w2 * p2;
  return length(pw - p3);
}

// closest points of the lines of two edges, with the parallel-edge branch
template <typename T>
CS_HD T dist_edge_edge(V3<T> p0, V3<T> p1, V3<T> q0, V3<T> q1, T& rp, T& rq) {
  const V3<T> vp = p1 - p0, vq = q1 - q0;
  if (length(cross(vp, vq)) < T(1.0e-10)) {
    const V3<T> pq0 = p0 - q0;
    const V3<T> nvp = normalized(vp);
    const V3<T> vert = pq0 - dot(pq0, nvp) * nvp;
    const T dist = length(vert);
    const T lp0 = dot(p0, nvp), lp1 = dot(p1, nvp), lq0 = dot(q0, nvp), lq1 = dot(q1, nvp);
    const T pmin = (lp0 < lp1) ? lp0 : lp1, pmax = (lp0 > lp1) ? lp0 : lp1;
    const T qmin = (lq0 < lq1) ? lq0 : lq1, qmax = (lq0 > lq1) ? lq0 : lq1;
    T lm;
    if (pmax < qmin)
      lm = (pmax + qmin) * T(0.5);
    else if (qmax < pmin)
      lm = (qmax + pmin) * T(0.5);
    else if (pmax < qmax)
      lm = (pmax + qmin) * T(0.5);
    else
      lm = (qmax + pmin) * T(0.5);
    rp = (lm - lp0) / (lp1 - lp0);
    rq = (lm - lq0) / (lq1 - lq0);
    return dist;
  }
  const T t0 = dot(vp, vp), t1 = dot(vq, vq), t2 = dot(vp, vq);
  const T t3 = dot(vp, q0 - p0), t4 = dot(vq, q0 - p0);
  const T det = t0 * t1 - t2 * t2;
  const T invdet = T(1) / det;
  rp = (+t1 * t3 - t2 * t4) * invdet;
  rq = (+t2 * t3 - t0 * t4) * invdet;
  const V3<T> pc = p0 + rp * vp, qc = q0 + rq * vq;
  return length(pc - qc);
}

CS_HD double cubic(double r, double k0, double k1, double k2, double k3) {
  return k0 + k1 * r + k2 * r * r + k3 * r * r * r;
}
// FindRootCubic + BisectRangeCubicRoot (bvh_aabb.cpp:571-595): 14 halvings
// with the sign reference fixed at the initial left end.
CS_HD double bisect_cubic(double r0, double r1, double v0, double k0, double k1, double k2, double k3) {
  for (int n = 14; n > 0; n--) {
    const double r2 = 0.5 * (r0 + r1);
    const double v2 = cubic(r2, k0, k1, k2, k3);
    if (v0 * v2 < 0)
      r1 = r2;
    else
      r0 = r2;
  }
  return 0.5 * (r0 + r1);
}
// First coplanarity time in [0,1] of four points moving s -> e, or -1
// (FindCoplanerInterp, bvh_aabb.cpp:598-662).  Always FP64.
CS_HD double coplanar_time(V3<double> s0, V3<double> s1, V3<double> s2, V3<double> s3, V3<double> e0,
                           V3<double> e1, V3<double> e2, V3<double> e3) {
  const V3<double> x1 = s1 - s0, x2 = s2 - s0, x3 = s3 - s0;
  const V3<double> v1 = (e1 - e0) - x1, v2 = (e2 - e0) - x2, v3 = (e3 - e0) - x3;
  const double k0 = stp(x3, x1, x2);
  const double k1 = stp(v3, x1, x2) + stp(x3, v1, x2) + stp(x3, x1, v2);
  const double k2 = stp(v3, v1, x2) + stp(v3, x1, v2) + stp(x3, v1, v2);
  const double k3 = stp(v3, v1, v2);
  const double r0 = -0.0, r1 = +1.0;
  const double f0 = cubic(r0, k0, k1, k2, k3), f1 = cubic(r1, k0, k1, k2, k3);
  const double det = k2 * k2 - 3 * k1 * k3;
  if (fabs(k3) < 1.0e-10 && fabs(k2) > 1.0e-10) {
    const double r2 = -k1 / (2 * k2);
    const double f2 = cubic(r2, k0, k1, k2, k3);
    if (r2 > 0 && r2 < 1) {
      if (f0 * f2 < 0) return bisect_cubic(r0, r2, f0, k0, k1, k2, k3);
      if (f2 * f1 < 0) return bisect_cubic(r2, r1, f2, k0, k1, k2, k3);
    }
  }
  if (det > 0 && fabs(k3) > 1.0e-10) {
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

// Closest points of segments a0 a1 and b0 b1 (FP32, clamped): the vector from
// the point on a to the point on b.  Only a direction for the hull certificate
// of the continuous-collision tests (cert.cuh).
CS_HD void seg_seg_dir32(const float a0[3], const float a1[3], const float b0[3],
                                              const float b1[3], float d[3]) {
  float u[3], v[3], w[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    u[k] = a1[k] - a0[k];
    v[k] = b1[k] - b0[k];
    w[k] = a0[k] - b0[k];
  }
  const float A = u[0] * u[0] + u[1] * u[1] + u[2] * u[2], B = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
  const float C = v[0] * v[0] + v[1] * v[1] + v[2] * v[2], D = u[0] * w[0] + u[1] * w[1] + u[2] * w[2];
  const float E = v[0] * w[0] + v[1] * w[1] + v[2] * w[2];
  const float den = A * C - B * B;
  float sa = (den > 1e-12f * A * C) ? (B * E - C * D) / den : 0.f;
  sa = fminf(fmaxf(sa, 0.f), 1.f);
  float sb = C > 0.f ? (B * sa + E) / C : 0.f;
  if (sb < 0.f) {
    sb = 0.f;
    sa = A > 0.f ? fminf(fmaxf(-D / A, 0.f), 1.f) : 0.f;
  } else if (sb > 1.f) {
    sb = 1.f;
    sa = A > 0.f ? fminf(fmaxf((B - D) / A, 0.f), 1.f) : 0.f;
  }
#pragma unroll
  for (int k = 0; k < 3; k++) d[k] = (b0[k] + sb * v[k]) - (a0[k] + sa * u[k]);
}

// ---------------------------------------------------------------------------
// elementary contact tests (bvh_aabb.cpp:392-438, 666-793)
// ---------------------------------------------------------------------------
CS_HD bool fv_proximity(int i0, int i1, int i2, int i3, V3<double> p0, V3<double> p1, V3<double> p2,
                        V3<double> p3, const Box& bb, double delta) {
  if (i3 == i0 || i3 == i1 || i3 == i2) return false;
  if (!box_inside(bb, p3)) return false;
  if (fabs(height4(p0, p1, p2, p3)) > delta) return false;
  double w0, w1;
  const double dist = dist_face_vertex(p0, p1, p2, p3, w0, w1);
  const double w2 = 1 - w0 - w1;
  if (dist > delta) return false;
  if (w0 < 0 || w0 > 1) return false;
  if (w1 < 0 || w1 > 1) return false;
  if (w2 < 0 || w2 > 1) return false;
  return true;
}

CS_HD bool ee_proximity(int i0, int i1, int j0, int j1, V3<double> p0, V3<double> p1, V3<double> q0,
                        V3<double> q1, double delta) {
  if (i0 == j0 || i0 == j1 || i1 == j0 || i1 == j1) return false;
  if (q0.x + delta < p0.x && q0.x + delta < p1.x && q1.x + delta < p0.x && q1.x + delta < p1.x) return false;
  if (q0.x - delta > p0.x && q0.x - delta > p1.x && q1.x - delta > p0.x && q1.x - delta > p1.x) return false;
  if (q0.y + delta < p0.y && q0.y + delta < p1.y && q1.y + delta < p0.y && q1.y + delta < p1.y) return false;
  if (q0.y - delta > p0.y && q0.y - delta > p1.y && q1.y - delta > p0.y && q1.y - delta > p1.y) return false;
  if (q0.z + delta < p0.z && q0.z + delta < p1.z && q1.z + delta < p0.z && q1.z + delta < p1.z) return false;
  if (q0.z - delta > p0.z && q0.z - delta > p1.z && q1.z - delta > p0.z && q1.z - delta > p1.z) return false;
  double rp, rq;
  const double dist = dist_edge_edge(p0, p1, q0, q1, rp, rq);
  if (dist > delta) return false;
  if (rp < 0 || rp > 1 || rq < 0 || rq > 1) return false;
  const V3<double> pm = (1 - rp) * p0 + rp * p1;
  const V3<double> qm = (1 - rq) * q0 + rq * q1;
  if (length(pm - qm) > delta) return false;
  return true;
}

// Conservative FP32 rejection for ee_proximity (edges p = p0 p1, q = q0 q1),
// from vp = p1 - p0, vq = q1 - q0, w = q0 - p0 in FP32 whose components are
// within E of the exact differences.  Returns true only when the FP64 test
// certainly rejects the pair.  The FP64 test accepts only with rp, rq in [0, 1] and |pm - qm| <=
// delta for the points pm, qm at those ratios, which lie on the segments: so
// any axis along which the two segments are more than delta apart rejects (the
// edge directions vp and vq, and the common normal vp x vq), in either branch
// of dist_edge_edge.  When its non-parallel branch is certain
// (|vp x vq|^2 = det > 1e-20), closest-point ratios certainly outside [0, 1]
// reject as well.  Every FP32 quantity carries an error bound (coordinates
// within one ulp of the FP64 position, then each product and sum rounded
// separately); decisions need twice that bound as margin, which also covers
// the rounding of the FP64 evaluation.
__device__ __forceinline__ bool ee_reject_core(const float* vp, const float* vq, const float* w, float E,
                                               float delta_hi) {
  const float u = 5.9604645e-8f;  // 2^-24
  // t = a . b with its error bound
  auto dot_err = [&](const float* a, const float* b, float& t, float& e) {
    float s = 0.f, l1a = 0.f, l1b = 0.f, sab = 0.f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float m = a[k] * b[k];
      s = s + m;
      l1a += fabsf(a[k]);
      l1b += fabsf(b[k]);
      sab += fabsf(m);
    }
    t = s;
    e = 1.001f * (E * (l1a + l1b) + 3.0f * E * E + 3.1f * u * sab);
  };
  float t0, t1, t2, t3, t4, e0, e1, e2, e3, e4;
  dot_err(vp, vp, t0, e0);
  dot_err(vq, vq, t1, e1);
  dot_err(vp, vq, t2, e2);
  dot_err(vp, w, t3, e3);
  dot_err(vq, w, t4, e4);
  const float A0 = fabsf(t0) + e0, A1 = fabsf(t1) + e1, A2 = fabsf(t2) + e2, A3 = fabsf(t3) + e3,
              A4 = fabsf(t4) + e4;
  const float d2 = delta_hi * delta_hi * 1.00001f;
  // axis vp: p spans [0, t0] (relative to a0), q spans its two ends t3, t3 + t2
  {
    const float q1 = t3 + t2, lo = fminf(t3, q1), hi = fmaxf(t3, q1);
    const float g = fmaxf(lo - t0, -hi), eg = 1.001f * (e0 + e2 + 2.0f * e3 + u * (fabsf(q1) + A0 + A3));
    const float gl = g - 2.0f * eg;
    if (gl > 0.f && gl * gl > d2 * (t0 + 2.0f * e0)) return true;
  }
  // axis vq: q spans [0, t1] (relative to b0), p spans its two ends -t4, t2 - t4
  {
    const float p1 = t2 - t4, lo = fminf(-t4, p1), hi = fmaxf(-t4, p1);
    const float g = fmaxf(lo - t1, -hi), eg = 1.001f * (e1 + e2 + 2.0f * e4 + u * (fabsf(p1) + A1 + A4));
    const float gl = g - 2.0f * eg;
    if (gl > 0.f && gl * gl > d2 * (t1 + 2.0f * e1)) return true;
  }
  // The reference's ratios are rp = (t1 t3 - t2 t4) / det, rq = (t2 t3 - t0 t4) / det
  // with det = t0 t1 - t2^2.  By the Binet-Cauchy identity these equal
  // n.(w x vq) / |n|^2 and n.(w x vp) / |n|^2 with n = vp x vq, which stay well
  // conditioned for nearly parallel edges, where t0 t1 - t2^2 cancels.
  float n[3], en[3], mp[3], emp[3], mq[3], emq[3];
  auto cross_err = [&](const float* a, const float* b, float* c, float* ec) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int i = (k + 1) % 3, j = (k + 2) % 3;
      c[k] = a[i] * b[j] - a[j] * b[i];
      ec[k] = 1.001f * (E * (fabsf(a[i]) + fabsf(b[j]) + fabsf(a[j]) + fabsf(b[i])) + 2.0f * E * E +
                        2.1f * u * (fabsf(a[i] * b[j]) + fabsf(a[j] * b[i])));
    }
  };
  auto dot3_err = [&](const float* a, const float* ea, const float* b, const float* eb, float& t, float& e) {
    float s = 0.f, r = 0.f, m = 0.f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      s = s + a[k] * b[k];
      r += (fabsf(a[k]) + ea[k]) * eb[k] + fabsf(b[k]) * ea[k];
      m += fabsf(a[k] * b[k]);
    }
    t = s;
    e = 1.001f * (r + 3.1f * u * m);
  };
  cross_err(vp, vq, n, en);
  cross_err(w, vq, mp, emp);
  cross_err(w, vp, mq, emq);
  float det, edet, np, enp, nq, enq;
  dot3_err(n, en, n, en, det, edet);
  dot3_err(n, en, mp, emp, np, enp);
  dot3_err(n, en, mq, emq, nq, enq);
  // the reference evaluates the t-formulas in FP64: their rounding (inputs, the
  // five dot products, products and differences) stays below these bounds
  const float e64 = 2.0e-15f;
  const float fdet = e64 * (A0 * A1 + A2 * A2), fnp = e64 * (A1 * A3 + A2 * A4), fnq = e64 * (A2 * A3 + A0 * A4);
  if (!(det - 2.0f * edet - fdet > 0.f)) return false;
  const float dhi = (det + 2.0f * edet + fdet) * 1.000001f;
  // certainly the non-parallel branch of dist_edge_edge (|vp x vq| > 1e-10): ratios
  if (det - 2.0f * edet - fdet > 2.0e-20f) {
    if (np + 2.0f * enp + fnp < 0.f || np - 2.0f * enp - fnp > dhi) return true;  // rp < 0 or rp > 1
    if (nq + 2.0f * enq + fnq < 0.f || nq - 2.0f * enq - fnq > dhi) return true;  // rq < 0 or rq > 1
  }
  // axis n = vp x vq (|n|^2 = det): both segments project to single points
  float s = 0.f, es = 0.f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s = s + w[k] * n[k];
    es += (fabsf(w[k]) + E) * en[k] + E * fabsf(n[k]) + 3.1f * u * fabsf(w[k] * n[k]);
  }
  es *= 1.001f;
  const float sl = fabsf(s) - 2.0f * es;
  return sl > 0.f && sl * sl > d2 * dhi;
}

// The filter on the FP32 vertex bounds (lo[3], hi[3] around each FP64 position,
// so every coordinate is within one ulp of it): absolute errors of 2^-23 |x|.
__device__ __forceinline__ bool ee_prx_reject32(const float* a0, const float* a1, const float* b0, const float* b1,
                                                float delta_hi) {
  const float u = 5.9604645e-8f;  // 2^-24
  float X = 0.f;
#pragma unroll
  for (int k = 0; k < 6; k++)
    X = fmaxf(X, fmaxf(fmaxf(fabsf(a0[k]), fabsf(a1[k])), fmaxf(fabsf(b0[k]), fabsf(b1[k]))));
  float vp[3], vq[3], w[3], D = 0.f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    vp[k] = a1[k] - a0[k];
    vq[k] = b1[k] - b0[k];
    w[k] = b0[k] - a0[k];
    D = fmaxf(D, fmaxf(fabsf(vp[k]), fmaxf(fabsf(vq[k]), fabsf(w[k]))));
  }
  // two coordinates within an ulp each (ulp <= 2^-23 |x|), plus the subtraction
  return ee_reject_core(vp, vq, w, 1.001f * (4.0f * u * X + u * D), delta_hi);
}

// The filter on differences taken in FP64 and rounded to FP32: relative errors
// of 2^-24 (plus the FP64 subtraction's), which resolves nearly parallel edges
// whose angle the absolute FP32 coordinates cannot.
__device__ __forceinline__ bool ee_prx_reject_rel(V3<double> p0, V3<double> p1, V3<double> q0, V3<double> q1,
                                                  float delta_hi) {
  const float vp[3] = {(float)(p1.x - p0.x), (float)(p1.y - p0.y), (float)(p1.z - p0.z)};
  const float vq[3] = {(float)(q1.x - q0.x), (float)(q1.y - q0.y), (float)(q1.z - q0.z)};
  const float w[3] = {(float)(q0.x - p0.x), (float)(q0.y - p0.y), (float)(q0.z - p0.z)};
  float D = 0.f;
#pragma unroll
  for (int k = 0; k < 3; k++) D = fmaxf(D, fmaxf(fabsf(vp[k]), fmaxf(fabsf(vq[k]), fabsf(w[k]))));
  return ee_reject_core(vp, vq, w, 1.001f * (5.9604645e-8f + 2.0e-16f) * D, delta_hi);
}

CS_HD bool fv_ccd(int i0, int i1, int i2, int i3, V3<double> p0, V3<double> p1, V3<double> p2, V3<double> p3,
                  V3<double> q0, V3<double> q1, V3<double> q2, V3<double> q3, const Box& bb) {
  const double eps = 1.0e-10;
  if (i3 == i0 || i3 == i1 || i3 == i2) return false;
  Box bp;
  box_clear(bp);
  box_add(bp, p3, eps);
  box_add(bp, q3, eps);
  if (!box_overlap(bb, bp)) return false;
  {
    const V3<double> n = cross(p1 - p0, p2 - p0);
    const double t0 = dot(p0 - p3, n), t1 = dot(q0 - q3, n), t2 = dot(q1 - q3, n), t3 = dot(q2 - q3, n);
    if (t0 * t1 > 0 && t0 * t2 > 0 && t0 * t3 > 0) return false;
  }
  double r0, r1;
  const double dist = dist_face_vertex(p0, p1, p2, p3, r0, r1);
  {
    const double vn0 = length(p0 - q0), vn1 = length(p1 - q1), vn2 = length(p2 - q2), vn3 = length(p3 - q3);
    double vnt = (vn0 > vn1) ? vn0 : vn1;
    vnt = (vn2 > vnt) ? vn2 : vnt;
    const double max_app = vnt + vn3;
    const double r2 = 1 - r0 - r1;
    if (dist > max_app) return false;
    if (r0 < 0 || r0 > 1 || r1 < 0 || r1 > 1 || r2 < 0 || r2 > 1) {
      const double d01 = length(closest_on_segment(p3, p0, p1) - p3);
      const double d12 = length(closest_on_segment(p3, p1, p2) - p3);
      const double d20 = length(closest_on_segment(p3, p2, p0) - p3);
      if (d01 > max_app && d12 > max_app && d20 > max_app) return false;
    }
  }
  const double t = coplanar_time(p0, p1, p2, p3, q0, q1, q2, q3);
  if (t < 0 || t > 1) return false;
  double w0, w1;
  dist_face_vertex(lerp(t, p0, q0), lerp(t, p1, q1), lerp(t, p2, q2), lerp(t, p3, q3), w0, w1);
  const double w2 = 1 - w0 - w1;
  if (w0 < 0 || w0 > 1) return false;
  if (w1 < 0 || w1 > 1) return false;
  if (w2 < 0 || w2 > 1) return false;
  return true;
}

CS_HD bool ee_ccd(int i0, int i1, int j0, int j1, V3<double> p0s, V3<double> p1s, V3<double> q0s,
                  V3<double> q1s, V3<double> p0e, V3<double> p1e, V3<double> q0e, V3<double> q1e) {
  const double eps = 1.0e-10;
  if (i0 == j0 || i0 == j1 || i1 == j0 || i1 == j1) return false;
  Box bq, bp;
  box_clear(bq);
  box_add(bq, q0s, eps);
  box_add(bq, q1s, eps);
  box_add(bq, q0e, eps);
  box_add(bq, q1e, eps);
  box_clear(bp);
  box_add(bp, p0s, eps);
  box_add(bp, p1s, eps);
  box_add(bp, p0e, eps);
  box_add(bp, p1e, eps);
  if (!box_overlap(bp, bq)) return false;
  const double t = coplanar_time(p0s, p1s, q0s, q1s, p0e, p1e, q0e, q1e);
  if (t < 0 || t > 1) return false;
  double w0, w1;
  const double dist = dist_edge_edge(lerp(t, p0s, p0e), lerp(t, p1s, p1e), lerp(t, q0s, q0e), lerp(t, q1s, q1e),
                                     w0, w1);
  if (w0 < 0 || w0 > 1) return false;
  if (w1 < 0 || w1 > 1) return false;
  if (dist > 1.0e-2) return false;
  return true;
}

}  // namespace cs
