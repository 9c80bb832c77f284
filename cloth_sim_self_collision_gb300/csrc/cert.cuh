// cert.cuh -- FP32 certificates, over pieces of a frame's motion, that the
// reference's FP64 continuous-collision tests reject.
//
// IsContact_FV_CCD and IsContact_EE_CCD (bvh_aabb.cpp:666-793) find the first
// coplanarity time t of the four moving points (FindCoplanerInterp) and then
// test closest-point ratios (and, edge-edge, a distance of 1e-2) at t.  The
// certificates below bound those ratios and that distance over whole
// sub-intervals of [0, 1], so they reject a test without knowing t:
//
// the coplanarity cubic's roots are localised to the pieces (eighths, halved
// down to 1/32 where needed) on which its Bernstein coefficients do not keep
// one sign; the reference's bisection returns a t within 2^-15 of a sign change
// of its FP64 cubic, so only those pieces, widened by 2^-14, can hold t; on
// each:
// * face-vertex: one barycentric ratio of the vertex's projection stays
//   outside [0, 1];
// * edge-edge: one ratio stays outside [0, 1], or the lines stay more than
//   1e-2 apart, or the segments' hulls are separated by more than 1e-2 along
//   one axis.
//
// Arithmetic: every quantity is an FP32 value with a bound on its distance from
// the exact value (R32), rounding to nearest, with the bound of a product or
// sum taking the operands' bounds and 2^-24 of the result (widened by 1.001 for
// the rounding of the bound's own few operations).  The inputs are the FP64
// differences FindCoplanerInterp forms; the reference's own FP64 rounding at t
// (interpolation, inner products, the division) is covered by a margin of 1e-6
// of the fourth power of the configuration's size S: its error is of order
// 1e-15 S^4 in the same units.  All functions run on the host too, so the CPU
// checks evaluate the same bounds.
#pragma once
#include <math.h>

#include "geom.cuh"

namespace cs {

struct R32 {
  float m, r;  // value, and a bound on |exact - m|
};
struct RV {
  R32 x, y, z;
};

constexpr float kU24 = 5.9604645e-8f;  // 2^-24, the unit roundoff of FP32

// lower and upper bounds of an R32 (the subtraction rounded outward)
CS_HD float lo32(R32 a) {
#ifdef __CUDA_ARCH__
  return __fsub_rd(a.m, a.r);
#else
  return nextafterf(a.m - a.r, -INFINITY);
#endif
}
CS_HD float hi32(R32 a) {
#ifdef __CUDA_ARCH__
  return __fadd_ru(a.m, a.r);
#else
  return nextafterf(a.m + a.r, INFINITY);
#endif
}

CS_HD R32 rc(float m, float r) {
  R32 a;
  a.m = m;
  a.r = r;
  return a;
}
CS_HD R32 operator+(R32 a, R32 b) {
  R32 c;
  c.m = a.m + b.m;
  c.r = 1.001f * (a.r + b.r + kU24 * fabsf(c.m));
  return c;
}
CS_HD R32 operator-(R32 a, R32 b) {
  R32 c;
  c.m = a.m - b.m;
  c.r = 1.001f * (a.r + b.r + kU24 * fabsf(c.m));
  return c;
}
CS_HD R32 operator-(R32 a) { return rc(-a.m, a.r); }
CS_HD R32 operator*(R32 a, R32 b) {
  R32 c;
  c.m = a.m * b.m;
  c.r = 1.001f * (fabsf(a.m) * b.r + fabsf(b.m) * a.r + a.r * b.r + kU24 * fabsf(c.m)) + 1e-37f;
  return c;
}
// exact float s times a
CS_HD R32 operator*(float s, R32 a) {
  R32 c;
  c.m = s * a.m;
  c.r = 1.001f * (fabsf(s) * a.r + kU24 * fabsf(c.m)) + 1e-37f;
  return c;
}

CS_HD RV operator+(const RV& a, const RV& b) {
  RV c;
  c.x = a.x + b.x;
  c.y = a.y + b.y;
  c.z = a.z + b.z;
  return c;
}
CS_HD RV operator-(const RV& a, const RV& b) {
  RV c;
  c.x = a.x - b.x;
  c.y = a.y - b.y;
  c.z = a.z - b.z;
  return c;
}
CS_HD RV rcross(const RV& a, const RV& b) {
  RV c;
  c.x = a.y * b.z - a.z * b.y;
  c.y = a.z * b.x - a.x * b.z;
  c.z = a.x * b.y - a.y * b.x;
  return c;
}
CS_HD R32 rdot(const RV& a, const RV& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
// an upper bound of |a| (the 1-norm of the component bounds)
CS_HD float rlen_hi(const RV& a) {
  return 1.0001f * ((fabsf(a.x.m) + a.x.r) + (fabsf(a.y.m) + a.y.r) + (fabsf(a.z.m) + a.z.r));
}
// a lower bound of |a|^2 (the box around a kept away from the origin)
CS_HD float rlen2_lo(const RV& a) {
  const float x = fmaxf(0.f, fabsf(a.x.m) - a.x.r), y = fmaxf(0.f, fabsf(a.y.m) - a.y.r),
              z = fmaxf(0.f, fabsf(a.z.m) - a.z.r);
  return 0.9999f * (x * x + y * y + z * z);
}

// x + t d for every t in [tm - hh, tm + hh] (tm, hh exact): the value at tm,
// with the bound widened by hh |d|
CS_HD R32 rpiece(R32 x, R32 d, float tm, float hh) {
  R32 c;
  const float td = tm * d.m;
  c.m = x.m + td;
  c.r = 1.001f * (x.r + fabsf(tm) * d.r + hh * (fabsf(d.m) + d.r) + kU24 * (fabsf(td) + fabsf(c.m))) + 1e-37f;
  return c;
}
CS_HD RV rvpiece(const RV& x, const RV& d, float tm, float hh) {
  RV c;
  c.x = rpiece(x.x, d.x, tm, hh);
  c.y = rpiece(x.y, d.y, tm, hh);
  c.z = rpiece(x.z, d.z, tm, hh);
  return c;
}

// A point's start position p and its displacement d = e - p over the frame
// (e its end position, d formed in FP64), each coordinate as FP32 hi + lo
// parts (hi the FP64 value rounded, lo the remainder rounded; hi + lo is within
// 2^-48 of the value): 12 floats, three float4 in memory.
struct PS {
  float ph[3], pl[3], dh[3], dl[3];
};

// b - a of two hi/lo values: the parts subtracted apart, then added; the bound
// takes each rounding and the splits' own error
CS_HD R32 hl_diff(float ah, float al, float bh, float bl) {
  const float dh = bh - ah, dl = bl - al;
  R32 c;
  c.m = dh + dl;
  c.r = 1.001f * (kU24 * (fabsf(dh) + fabsf(dl) + fabsf(c.m)) + 4e-15f * (fabsf(ah) + fabsf(bh))) + 1e-37f;
  return c;
}
// x = p_b - p_a and v = d_b - d_a: the differences FindCoplanerInterp forms
// (x = p_b - p_a, v = (e_b - e_a) - x, in FP64), enclosed: v's bound adds the
// FP64 roundings that separate the reference's v from d_b - d_a (its own two
// subtractions and those of d), 4e-16 of the magnitudes involved
CS_HD void hl_xv1(const PS& a, const PS& b, int k, R32& x, R32& v) {
  x = hl_diff(a.ph[k], a.pl[k], b.ph[k], b.pl[k]);
  v = hl_diff(a.dh[k], a.dl[k], b.dh[k], b.dl[k]);
  v.r = 1.001f * (v.r + 4e-16f * (fabsf(x.m) + fabsf(v.m) + fabsf(a.dh[k]) + fabsf(b.dh[k]))) + 1e-37f;
}
CS_HD void hl_xv(const PS& a, const PS& b, RV& x, RV& v) {
  hl_xv1(a, b, 0, x.x, v.x);
  hl_xv1(a, b, 1, x.y, v.y);
  hl_xv1(a, b, 2, x.z, v.z);
}

// a ratio N / D of the reference (D > 0) certainly outside [0, 1], with margin M
CS_HD bool ratio_out(R32 N, R32 D, float M) { return hi32(N) < -M || lo32(N - D) > M; }

// (S + 1e-6)^4 from above, S an upper bound of the configuration's size
CS_HD float size4(float S) {
  const float s = S + 1e-6f;
  return 1.0001f * (s * s) * (s * s);
}

// --- face-vertex ----------------------------------------------------------
// x_i = p_i - p0 at the start and v_i their changes over the frame (i = 1, 2,
// 3; p3 the vertex), as FindCoplanerInterp forms them.  True when on the piece
// [tm - hh, tm + hh] one barycentric ratio of DistanceFaceVertex (w0, w1, or
// w2 = 1 - w0 - w1, bvh_aabb.cpp:304-326 and :710-716) stays outside [0, 1].
// With X_i the piece's x_i + t v_i: n = X1 x X2 is the face normal (v20 x v21),
// and the three ratios are ((X3 - X2) x (X1 - X2)).n, (X3 x X2).n and
// (X1 x X3).n over |n|^2 (they sum to 1).
CS_HD bool fv_piece_reject32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2, const RV& v3,
                             float tm, float hh) {
  const RV X1 = rvpiece(x1, v1, tm, hh), X2 = rvpiece(x2, v2, tm, hh), X3 = rvpiece(x3, v3, tm, hh);
  const RV n = rcross(X1, X2);
  const R32 n2 = rdot(n, n);
  const float S4 = size4(rlen_hi(X1) + rlen_hi(X2) + rlen_hi(X3));
  // the reference divides by its own |n|^2: keep it far from its rounding
  if (!(lo32(n2) > 1e-12f * S4)) return false;
  const float M = 1e-6f * S4;
  if (ratio_out(rdot(rcross(X1, X3), n), n2, M)) return true;  // w2
  if (ratio_out(rdot(rcross(X3, X2), n), n2, M)) return true;  // w1
  return ratio_out(rdot(rcross(X3 - X2, X1 - X2), n), n2, M);  // w0
}

// --- edge-edge ------------------------------------------------------------
// x1 = p1 - p0, x2 = q0 - p0, x3 = q1 - p0 at the start and v_i their changes,
// as FindCoplanerInterp forms them for IsContact_EE_CCD.  True when on the
// piece the test's ratios or distance at any t there reject
// (DistanceEdgeEdge, bvh_aabb.cpp:343-384, and :782-791).  With the piece's
// vp = X1, W = X2 (q0 - p0) and vq = X3 - X2, n = vp x vq:
// * ratios: rp = ((W x vq).n) / |n|^2 and rq = ((W x vp).n) / |n|^2
//   (Lagrange's identity on the reference's t0..t4), valid where the
//   reference takes its non-parallel branch (|n| above 1e-10);
// * line distance: whatever branch it takes, the distance it measures is
//   between a point of each line (its closest points, or q0 and its foot on
//   line p), so at least the lines' distance |W.n| / |n|;
// * hull separation: with both ratios in [0, 1] its points lie on the
//   segments (non-parallel branch), or its line distance undercuts the
//   segments' distance by at most 1e-10 over an edge's length (parallel
//   branch), so the segments' convex hulls over the piece being more than
//   1e-2 + 1e-6 apart along one axis, with both edges at least 1e-3 m long
//   throughout, rejects as well.
CS_HD bool ee_hull_far32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2, const RV& v3,
                         float tm, float hh);
CS_HD bool ee_piece_reject32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2, const RV& v3,
                             float tm, float hh) {
  const RV vp = rvpiece(x1, v1, tm, hh), W = rvpiece(x2, v2, tm, hh), Q1 = rvpiece(x3, v3, tm, hh);
  const RV vq = Q1 - W;
  const float S4 = size4(rlen_hi(vp) + rlen_hi(vq) + rlen_hi(W));
  const RV n = rcross(vp, vq);
  const R32 n2 = rdot(n, n);
  if (lo32(n2) > 1e-12f * S4) {
    if (lo32(n2) > 1.0001e-20f) {
      const float M = 1e-6f * S4;
      if (ratio_out(rdot(rcross(W, vq), n), n2, M)) return true;
      if (ratio_out(rdot(rcross(W, vp), n), n2, M)) return true;
    }
    const R32 wn = rdot(W, n);
    const float a = fmaxf(0.f, fmaxf(lo32(wn), -hi32(wn)));
    const float need = 1e-2f + 1e-7f;
    if (0.9999f * (a * a) > 1.0001f * (need * need) * hi32(n2)) return true;
  }
  return ee_hull_far32(x1, x2, x3, v1, v2, v3, tm, hh);
}

// The hull certificate of ee_piece_reject32 on its own (the piece [tm - hh,
// tm + hh]; the whole motion for tm = hh = 1/2).
CS_HD bool ee_hull_far32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2, const RV& v3,
                         float tm, float hh) {
  const RV vp = rvpiece(x1, v1, tm, hh), W = rvpiece(x2, v2, tm, hh), Q1 = rvpiece(x3, v3, tm, hh);
  const RV vq = Q1 - W;
  if (!(rlen2_lo(vp) > 1.0001e-6f) || !(rlen2_lo(vq) > 1.0001e-6f)) return false;
  float d[3];
  {
    const float a0[3] = {0.f, 0.f, 0.f}, a1[3] = {vp.x.m, vp.y.m, vp.z.m};
    const float b0[3] = {W.x.m, W.y.m, W.z.m}, b1[3] = {Q1.x.m, Q1.y.m, Q1.z.m};
    seg_seg_dir32(a0, a1, b0, b1, d);
  }
  const float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  if (!(dd > 0.f) || !isfinite(dd)) return false;
  RV dv;  // any axis will do: d is taken as exact
  dv.x = rc(d[0], 0.f);
  dv.y = rc(d[1], 0.f);
  dv.z = rc(d[2], 0.f);
  const R32 pp = rdot(vp, dv), pw = rdot(W, dv), pq1 = rdot(Q1, dv);
  const float pmax = fmaxf(0.f, hi32(pp)), pmin = fminf(0.f, lo32(pp));
  const float qmax = fmaxf(hi32(pw), hi32(pq1)), qmin = fminf(lo32(pw), lo32(pq1));
  const float dlen = 1.0001f * sqrtf(dd);
  const float need = 1.0001f * (1.0e-2f + 1.0e-6f) * dlen;
  const float gap = fmaxf(0.9999f * (qmin - pmax), 0.9999f * (pmin - qmax));
  return gap > need;
}

// True when t cannot lie in [a, a + h] (a, h exact), or the test rejects at
// every t there: the cubic k keeps one sign on the piece beyond the reference's
// FP64 evaluation error F (its Bernstein coefficients), so its bisection ends
// elsewhere, unless the piece ends at 1 and k0 may vanish; otherwise the
// piece, widened by 2^-14 on each side, passes the face-vertex or edge-edge
// certificate.
// The cubic k keeps one sign on [a, a + h] (a, h exact) beyond F: its
// Bernstein coefficients there do.
CS_HD bool cubic_one_sign(const R32 k[4], float F, float a, float h) {
  const R32 third = rc(0.33333334f, 1.0e-8f), two_thirds = rc(0.6666667f, 3.0e-8f);
  const R32 K0 = k[0] + a * (k[1] + a * (k[2] + a * k[3]));
  const R32 K1 = h * (k[1] + a * (2.f * k[2] + (3.f * a) * k[3]));
  const R32 K2 = (h * h) * (k[2] + (3.f * a) * k[3]);
  const R32 K3 = (h * h * h) * k[3];
  const R32 B1 = K0 + third * K1, B2 = (K0 + two_thirds * K1) + third * K2, B3 = ((K0 + K1) + K2) + K3;
  const bool pos = lo32(K0) > F && lo32(B1) > F && lo32(B2) > F && lo32(B3) > F;
  const bool neg = hi32(K0) < -F && hi32(B1) < -F && hi32(B2) < -F && hi32(B3) < -F;
  return pos || neg;
}

template <bool kFV>
CS_HD bool piece_clear(const R32 k[4], float F, bool k0_zero, float a, float h, const RV& x1, const RV& x2,
                       const RV& x3, const RV& v1, const RV& v2, const RV& v3) {
  if (cubic_one_sign(k, F, a, h) && !(k0_zero && a + h == 1.f)) return true;
  const float eps = 6.1035156e-5f;  // 2^-14
  const float ta = fmaxf(0.f, a - eps), tb = fminf(1.f, a + h + eps);
  const float tm = 0.5f * (ta + tb), hh = 0.5f * (tb - ta);
  return kFV ? fv_piece_reject32(x1, x2, x3, v1, v2, v3, tm, hh) : ee_piece_reject32(x1, x2, x3, v1, v2, v3, tm, hh);
}

// The coplanarity cubic k0 + k1 t + k2 t^2 + k3 t^3 of FindCoplanerInterp
// (triple products a . (b x c) of x_i and v_i), with F, a bound on the
// reference's FP64 rounding of its coefficients and of each evaluation: below
// 4e-15 of the magnitude of the terms, F allows 1e-14.  k0_zero: the FP64 k0
// may be exactly 0, which sends the bisection to t = 1 - 2^-15.
struct Cubic32 {
  R32 k[4];
  float F;
  bool k0_zero;
};
CS_HD Cubic32 coplanar_cubic32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2,
                               const RV& v3) {
  Cubic32 c;
  float mk = 0.f;
  const RV* X[3] = {&x1, &x2, &x3};
  const RV* V[3] = {&v1, &v2, &v3};
  // stp(c3, c1, c2) with each c_i = x_i (bit clear) or v_i (bit set); the
  // bits set count the power of t
  R32 acc[4] = {rc(0.f, 0.f), rc(0.f, 0.f), rc(0.f, 0.f), rc(0.f, 0.f)};
#pragma unroll
  for (int s = 0; s < 8; s++) {
    const RV& c1 = (s & 1) ? *V[0] : *X[0];
    const RV& c2 = (s & 2) ? *V[1] : *X[1];
    const RV& c3 = (s & 4) ? *V[2] : *X[2];
    const R32 t = rdot(c3, rcross(c1, c2));
    const int deg = (s & 1) + ((s >> 1) & 1) + ((s >> 2) & 1);
    acc[deg] = acc[deg] + t;
    mk += fabsf(t.m) + t.r +
          (fabsf(c3.x.m) + c3.x.r) * ((fabsf(c1.y.m) + c1.y.r) * (fabsf(c2.z.m) + c2.z.r) +
                                      (fabsf(c1.z.m) + c1.z.r) * (fabsf(c2.y.m) + c2.y.r)) +
          (fabsf(c3.y.m) + c3.y.r) * ((fabsf(c1.z.m) + c1.z.r) * (fabsf(c2.x.m) + c2.x.r) +
                                      (fabsf(c1.x.m) + c1.x.r) * (fabsf(c2.z.m) + c2.z.r)) +
          (fabsf(c3.z.m) + c3.z.r) * ((fabsf(c1.x.m) + c1.x.r) * (fabsf(c2.y.m) + c2.y.r) +
                                      (fabsf(c1.y.m) + c1.y.r) * (fabsf(c2.x.m) + c2.x.r));
  }
#pragma unroll
  for (int d = 0; d < 4; d++) c.k[d] = acc[d];
  c.F = 1.0e-14f * mk + 1e-30f;
  c.k0_zero = !(lo32(c.k[0]) > c.F || hi32(c.k[0]) < -c.F);
  return c;
}

// The test (face-vertex when kFV, else edge-edge) rejects at whatever t
// FindCoplanerInterp returns, piece by piece: pieces of 1/8, halved down to
// 1/32 where a piece that may hold t fails.  Each eighth is a tree of 7 nodes
// in preorder (0: the eighth; 1, 4: its halves; 2, 3 and 5, 6: their halves),
// a node tested only if its parent failed, and a failing leaf ends the
// certificate (one call site, so the piece certificate is compiled once).
template <bool kFV>
CS_HD bool ccd_pieces32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2, const RV& v3,
                        const Cubic32& c) {
#pragma unroll 1
  for (int j = 0; j < 8; j++) {
    unsigned need = 1u;
#pragma unroll 1
    for (int n = 0; n < 7; n++) {
      if (!((need >> n) & 1u)) continue;
      const float off = n == 3 ? 0.03125f : (n == 4 || n == 5) ? 0.0625f : n == 6 ? 0.09375f : 0.f;
      const float h = n == 0 ? 0.125f : (n == 1 || n == 4) ? 0.0625f : 0.03125f;
      if (piece_clear<kFV>(c.k, c.F, c.k0_zero, 0.125f * (float)j + off, h, x1, x2, x3, v1, v2, v3)) continue;
      if (n == 0)
        need |= (1u << 1) | (1u << 4);
      else if (n == 1)
        need |= (1u << 2) | (1u << 3);
      else if (n == 4)
        need |= (1u << 5) | (1u << 6);
      else
        return false;
    }
  }
  return true;
}

// x_i, v_i of the face-vertex test (face p0 p1 p2, vertex p3) and of the
// edge-edge test (edges p0 p1 and q0 q1) from the points' hi/lo parts
CS_HD void ccd_xv(const PS& s0, const PS& s1, const PS& s2, const PS& s3, RV& x1, RV& x2, RV& x3, RV& v1, RV& v2,
                  RV& v3) {
  hl_xv(s0, s1, x1, v1);
  hl_xv(s0, s2, x2, v2);
  hl_xv(s0, s3, x3, v3);
}

// IsContact_FV_CCD certainly rejects over the whole motion: the vertex stays
// on one side of the start face plane (the test's sign block,
// bvh_aabb.cpp:683-690: the four heights (p0 - p3).n, (q0 - q3).n,
// (q1 - q3).n, (q2 - q3).n with n = x1 x2, each beyond twice its bound, which
// also covers the reference's FP64 rounding, and 1e-30, so that its products
// keep their signs), or the four points are never coplanar in [0, 1].
CS_HD bool fv_ccd_whole32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2, const RV& v3) {
  {
    const RV n = rcross(x1, x2);
    const RV e3 = x3 + v3;  // q3 - q0
    const R32 h[4] = {-rdot(x3, n), -rdot(e3, n), rdot((x1 + v1) - e3, n), rdot((x2 + v2) - e3, n)};
    bool pos = true, neg = true;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const R32 w = rc(h[i].m, 2.f * h[i].r);
      pos = pos && lo32(w) > 1e-30f;
      neg = neg && hi32(w) < -1e-30f;
    }
    if (pos || neg) return true;
  }
  const Cubic32 c = coplanar_cubic32(x1, x2, x3, v1, v2, v3);
  return !c.k0_zero && cubic_one_sign(c.k, c.F, 0.f, 1.f);
}

// IsContact_EE_CCD certainly rejects over the whole motion: no coplanarity in
// [0, 1], or the edges more than 1e-2 apart throughout.
CS_HD bool ee_ccd_whole32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2, const RV& v3) {
  const Cubic32 c = coplanar_cubic32(x1, x2, x3, v1, v2, v3);
  if (!c.k0_zero && cubic_one_sign(c.k, c.F, 0.f, 1.f)) return true;
  return ee_hull_far32(x1, x2, x3, v1, v2, v3, 0.5f, 0.5f);
}

// The piece stage on its own (after the whole-motion stage kept the test):
// at any coplanarity time the vertex projects outside the face (face-vertex),
// or a ratio is out of range or the edges are apart (edge-edge).
template <bool kFV>
CS_HD bool ccd_pieces_stage32(const RV& x1, const RV& x2, const RV& x3, const RV& v1, const RV& v2, const RV& v3) {
  return ccd_pieces32<kFV>(x1, x2, x3, v1, v2, v3, coplanar_cubic32(x1, x2, x3, v1, v2, v3));
}

// Both stages: true when IsContact_FV_CCD (the face p0 p1 p2 and the vertex p3
// moving to their end points) or IsContact_EE_CCD (the edges p0 p1 and q0 q1)
// certainly rejects, from enclosures of the differences FindCoplanerInterp
// forms (x_i = p_i - p0, v_i = (q_i - q0) - x_i).
CS_HD bool fv_ccd_cert32(const PS& s0, const PS& s1, const PS& s2, const PS& s3) {
  RV x1, x2, x3, v1, v2, v3;
  ccd_xv(s0, s1, s2, s3, x1, x2, x3, v1, v2, v3);
  return fv_ccd_whole32(x1, x2, x3, v1, v2, v3) || ccd_pieces_stage32<true>(x1, x2, x3, v1, v2, v3);
}
CS_HD bool ee_ccd_cert32(const PS& p0, const PS& p1, const PS& q0, const PS& q1) {
  RV x1, x2, x3, v1, v2, v3;
  ccd_xv(p0, p1, q0, q1, x1, x2, x3, v1, v2, v3);
  return ee_ccd_whole32(x1, x2, x3, v1, v2, v3) || ccd_pieces_stage32<false>(x1, x2, x3, v1, v2, v3);
}

}  // namespace cs
