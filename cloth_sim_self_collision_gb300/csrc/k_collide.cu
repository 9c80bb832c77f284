// k_collide.cu -- self-collision on the device (bvh_aabb.cpp,
// self_collision_cloth.cpp), all FP64 with the reference's rounding.
//
// * refit: one thread per leaf; parents are merged by the second child to
//   arrive (atomic counter per node), bottom-up in one launch.
// * broad phase: one thread per triangle walks its cloth's BVH without a stack
//   (depth-first preorder with skip links) and keeps the leaves to its right in
//   leaf order, which is exactly the set and orientation of leaf pairs the
//   reference's recursive descent visits.  Pairs are appended with
//   warp-aggregated atomics.
// * narrow phase: one thread per leaf pair runs the reference's 15 elementary
//   tests and appends canonical contact elements.
// * contact set: two stable radix sorts give the std::set order; a key seen
//   more than once keeps the element the reference inserts first (decided by
//   the reference's traversal order when face-vertex and edge-edge collide).
// * impulses: contacts of a cloth are split into levels so that no two
//   contacts of a level share a vertex and every contact follows all earlier
//   contacts it shares a vertex with; levels run in order, which reproduces
//   the reference's sequential Gauss-Seidel sweep exactly.
// * impact zones: union-find over contact vertices and mesh edges, then one
//   thread per zone sums its members in ascending order.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cooperative_groups.h>

#include "cert.cuh"
#include "kernels.h"

namespace cs {
namespace {

constexpr int kT = 128;
inline int nblk(long long n, int t = kT) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ Box load_box(const Box* b, int n) {
  // boxes written by other threads in this launch: read around L1
  Box r;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    r.lo[k] = __ldcg(&b[n].lo[k]);
    r.hi[k] = __ldcg(&b[n].hi[k]);
  }
  r.full = __ldcg(&b[n].full);
  return r;
}

// outward-rounded FP32 copy of an FP64 box (contains it); empty -> never overlaps
__device__ __forceinline__ void store_box32(float* dst, const Box& b) {
  if (!b.full) {
    dst[0] = dst[1] = dst[2] = __int_as_float(0x7f800000);
    dst[3] = dst[4] = dst[5] = -__int_as_float(0x7f800000);
    return;
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    dst[k] = __double2float_rd(b.lo[k]);
    dst[3 + k] = __double2float_ru(b.hi[k]);
  }
}

__device__ __forceinline__ bool overlap32(const float* a, const float* b) {
  return !(a[3] < b[0] || a[0] > b[3] || a[4] < b[1] || a[1] > b[4] || a[5] < b[2] || a[2] > b[5]);
}

__device__ __forceinline__ V3<double> end_pos(const double* x, const double* v, int i, double dt) {
  return mk<double>(x[3 * i + 0] + dt * v[3 * i + 0], x[3 * i + 1] + dt * v[3 * i + 1], x[3 * i + 2] + dt * v[3 * i + 2]);
}

// The start positions and the displacements e - x (e = end_pos, FP64) of the
// active cloths' vertices as FP32 hi/lo parts, for the certificates of a
// continuous-collision detection
__global__ void k_ccd_split(Arena A, const double* xs, const double* vs) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  const int inst = A.vinst[v];
  if (!A.active[inst]) return;
  const V3<double> p = ld3(xs, v), e = end_pos(xs, vs, v, A.prm[inst].dt);
  const double pv[3] = {p.x, p.y, p.z}, dv[3] = {e.x - p.x, e.y - p.y, e.z - p.z};
  float f[12];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    f[c] = (float)pv[c];
    f[3 + c] = (float)(pv[c] - (double)f[c]);
    f[6 + c] = (float)dv[c];
    f[9 + c] = (float)(dv[c] - (double)f[6 + c]);
  }
  float4* o = A.ccd32 + 3 * (size_t)v;
  o[0] = make_float4(f[0], f[1], f[2], f[3]);
  o[1] = make_float4(f[4], f[5], f[6], f[7]);
  o[2] = make_float4(f[8], f[9], f[10], f[11]);
}

__device__ __forceinline__ PS ld_ps(const Arena& A, int v) {
  const float4* q = A.ccd32 + 3 * (size_t)v;
  const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
  PS s;
  s.ph[0] = a.x, s.ph[1] = a.y, s.ph[2] = a.z;
  s.pl[0] = a.w, s.pl[1] = b.x, s.pl[2] = b.y;
  s.dh[0] = b.z, s.dh[1] = b.w, s.dh[2] = c.x;
  s.dl[0] = c.y, s.dl[1] = c.z, s.dl[2] = c.w;
  return s;
}

// BuildBoundingBoxChild_Prx / _CCD (bvh_aabb.cpp:23-106)
__global__ void k_refit(Arena A, int ccd, const double* xs, const double* vs, double delta_override) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nt) return;
  const int inst = A.tinst[t];
  if (!A.active[inst]) return;
  const DevParams& P = A.prm[inst];
  Box b;
  box_clear(b);
  const double delta = delta_override >= 0 ? delta_override : P.contact_clearance;
  const double eps = ccd ? 1.0e-10 : delta * 0.5;
  int vid[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    vid[a] = A.tri[3 * t + a];
    box_add(b, ld3(xs, vid[a]), eps);
  }
  if (ccd) {
#pragma unroll
    for (int a = 0; a < 3; a++) box_add(b, end_pos(xs, vs, vid[a], P.dt), eps);
  }
  int n = A.tri_leaf[t];
  A.box[n] = b;
  store_box32(A.box32 + 6 * (size_t)n, b);
  for (;;) {
    __threadfence();
    const int par = A.node[3 * n + 0];
    if (par < 0) break;
    if (atomicAdd(&A.refit_cnt[par], 1) == 0) break;  // the sibling finishes the parent
    Box m = load_box(A.box, A.node[3 * par + 1]);
    box_merge(m, load_box(A.box, A.node[3 * par + 2]));
    A.box[par] = m;
    store_box32(A.box32 + 6 * (size_t)par, m);
    n = par;
  }
}

// per vertex FP32 bounds for the prefilters: the point (proximity) or its swept
// box [min(p-eps, q-eps), max(p+eps, q+eps)], q = p + dt v, eps = 1e-10, with the
// FP64 rounding of the reference's AddPoint (CCD), rounded outward
__global__ void k_vertex_bounds(Arena A, int ccd, const double* xs, const double* vs) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  const int inst = A.vinst[v];
  if (!A.active[inst]) return;
  float* dst = A.vb32 + 6 * (size_t)v;
  if (!ccd) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double p = xs[3 * v + k];
      dst[k] = __double2float_rd(p);
      dst[3 + k] = __double2float_ru(p);
    }
    return;
  }
  const double dt = A.prm[inst].dt, eps = 1.0e-10;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double p = xs[3 * v + k];
    const double q = p + dt * vs[3 * v + k];
    const double lo = (p - eps < q - eps) ? p - eps : q - eps;
    const double hi = (p + eps > q + eps) ? p + eps : q + eps;
    dst[k] = __double2float_rd(lo);
    dst[3 + k] = __double2float_ru(hi);
  }
}

// Reserves one slot per active lane with one atomic per warp.  The counter may
// pass INT_MAX (and wrap) when a buffer overflows badly: callers compare the
// slot as unsigned against their capacity, so a wrapped slot is never written.
__device__ __forceinline__ int warp_append(int* counter) {
  const unsigned m = __activemask();
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(m, base, leader);
  return base + __popc(m & ((1u << lane) - 1u));
}

// broad phase: leaf pairs with overlapping boxes (GetContactElement_* recursion,
// bvh_aabb.cpp:441-557 / 797-923).  A triangle that overlaps more than
// kMaxPairsPerTriangle leaves to its right marks its cloth as blown up (the
// reference would go on with a quadratic contact set); the cloth's pairs are
// then dropped by the narrow phase and the host stops stepping it.
// Nodes are culled with the outward-rounded FP32 boxes (a miss there is a
// miss in FP64; a node's box holds its children's), and each leaf pair is
// accepted by the FP64 boxes, so the pairs are exactly the reference's.
__device__ __forceinline__ void load_box32(const float* src, float* b) {
  const float2* p = reinterpret_cast<const float2*>(src);
#pragma unroll
  for (int h = 0; h < 3; h++) {
    const float2 v = p[h];
    b[2 * h] = v.x;
    b[2 * h + 1] = v.y;
  }
}

// Leaf pairs a thread of the broad phase found, appended to C.pairs in batches
// of 8 (one atomic per batch; the pair order does not matter, the contact set
// being sorted by key afterwards).  A count past the capacity sets the overflow
// flag, and the host regrows the buffer from the count.
struct PairBuf {
  int2 p[8];
  int n;
};
__device__ __forceinline__ void pairbuf_flush(const ContactBufs& C, PairBuf& b) {
  if (b.n == 0) return;
  const int slot = atomicAdd(&C.counters[0], b.n);
  for (int i = 0; i < b.n; i++) {
    if ((unsigned)(slot + i) < (unsigned)C.pair_cap)
      C.pairs[slot + i] = b.p[i];
    else
      C.counters[3] = 1;
  }
  b.n = 0;
}
__device__ __forceinline__ void pairbuf_add(const ContactBufs& C, PairBuf& b, int2 pr) {
  b.p[b.n++] = pr;
  if (b.n == 8) pairbuf_flush(C, b);
}

__device__ __forceinline__ void traverse_tri(const Arena& A, const ContactBufs& C, int t) {
  const int inst = A.tinst[t];
  if (!A.active[inst] || A.st[inst].diverged) return;
  const int la = A.tri_leaf[t];
  const int oa = A.leaf_lo[la];
  const Box ba = A.box[la];
  float ba32[6];
  load_box32(A.box32 + 6 * (size_t)la, ba32);
  int k = A.preoff[inst];
  const int end = A.preoff[inst + 1];
  int found = 0;
  PairBuf buf;
  buf.n = 0;
  while (k < end) {
    const int n = A.pre[k];
    float nb32[6];
    load_box32(A.box32 + 6 * (size_t)n, nb32);
    if (A.leaf_hi[n] <= oa || !overlap32(ba32, nb32)) {
      k = A.skip[k];
      continue;
    }
    if (A.node[3 * n + 2] == -1) {
      if (!box_overlap(ba, A.box[n])) {
        k = A.skip[k];
        continue;
      }
      if (++found > kMaxPairsPerTriangle) {
        A.st[inst].diverged = 1;
        pairbuf_flush(C, buf);
        return;
      }
      pairbuf_add(C, buf, make_int2(la, n));
      k = A.skip[k];
    } else {
      k++;
    }
  }
  pairbuf_flush(C, buf);
}

__global__ void k_traverse(Arena A, ContactBufs C) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < A.nt) traverse_tri(A, C, t);
}

// every overlapping leaf pair with a dirty triangle, oriented by leaf order; a
// pair of two dirty triangles is emitted by its left one
// (overlaps on both sides are walked here: the blow-up limit is doubled)
__device__ __forceinline__ void traverse_dirty_tri(const Arena& A, const ContactBufs& C, int t) {
  if (!A.tdirty[t]) return;
  const int inst = A.tinst[t];
  if (!A.active[inst] || A.st[inst].diverged) return;
  const int la = A.tri_leaf[t];
  const int oa = A.leaf_lo[la];
  const Box ba = A.box[la];
  float ba32[6];
  load_box32(A.box32 + 6 * (size_t)la, ba32);
  int k = A.preoff[inst];
  const int end = A.preoff[inst + 1];
  int found = 0;
  PairBuf buf;
  buf.n = 0;
  while (k < end) {
    const int n = A.pre[k];
    float nb32[6];
    load_box32(A.box32 + 6 * (size_t)n, nb32);
    if (!overlap32(ba32, nb32)) {
      k = A.skip[k];
      continue;
    }
    if (A.node[3 * n + 2] == -1) {
      if (!box_overlap(ba, A.box[n])) {
        k = A.skip[k];
        continue;
      }
      if (++found > 2 * kMaxPairsPerTriangle) {
        A.st[inst].diverged = 1;
        pairbuf_flush(C, buf);
        return;
      }
      const int ob = A.leaf_lo[n];
      const bool other_dirty = A.tdirty[A.node[3 * n + 1]] != 0;
      if (n != la && (!other_dirty || oa < ob)) pairbuf_add(C, buf, (oa < ob) ? make_int2(la, n) : make_int2(n, la));
      k = A.skip[k];
    } else {
      k++;
    }
  }
  pairbuf_flush(C, buf);
}

__global__ void k_traverse_dirty(Arena A, ContactBufs C) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < A.nt) traverse_dirty_tri(A, C, t);
}

// candidates of the previous detection whose pair has no dirty triangle
__global__ void k_keep_clean(Arena A, ContactBufs C, int ncand, int* nkeep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncand) return;
  const Cand c = C.cand[i];
  const int ta = A.node[3 * c.na + 1], tb = A.node[3 * c.nb + 1];
  if (A.tdirty[ta] || A.tdirty[tb] || !A.active[A.tinst[ta]]) return;
  C.cand_sorted[atomicAdd(nkeep, 1)] = c;
}

__global__ void k_mark_contacts(Arena A, ContactBufs C, int nce) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nce) return;
  const int* e = C.ce + 5 * c;
  if (!A.active[A.vinst[e[1]]]) return;
#pragma unroll
  for (int k = 1; k <= 4; k++) A.vdirty[e[k]] = 1;
}

__global__ void k_mark_zones(Arena A) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  if (A.active[A.vinst[v]] && A.inzone[v]) A.vdirty[v] = 1;
}

__global__ void k_mark_tris(Arena A) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nt) return;
  A.tdirty[t] = A.vdirty[A.tri[3 * t]] | A.vdirty[A.tri[3 * t + 1]] | A.vdirty[A.tri[3 * t + 2]];
}

// canonical key (CContactElement constructor, bvh_aabb.h:68-93)
__device__ __forceinline__ void canonical(int fv, int j0, int j1, int j2, int j3, int k[4]) {
  if (fv) {
    int a = j0, b = j1, c = j2, t;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
    k[0] = a; k[1] = b; k[2] = c; k[3] = j3;
  } else {
    const int lo01 = j0 < j1 ? j0 : j1, lo23 = j2 < j3 ? j2 : j3;
    int o0, o1;
    if (lo01 < lo23) {
      k[0] = lo01; k[1] = (j0 < j1) ? j1 : j0; o0 = j2; o1 = j3;
    } else {
      k[0] = lo23; k[1] = (j2 < j3) ? j3 : j2; o0 = j0; o1 = j1;
    }
    k[2] = o0 < o1 ? o0 : o1;
    k[3] = o0 < o1 ? o1 : o0;
  }
}

__device__ __forceinline__ void emit(const ContactBufs& C, int fv, int j0, int j1, int j2, int j3, int na, int nb,
                                     int test) {
  const int slot = warp_append(&C.counters[1]);
  if ((unsigned)slot >= (unsigned)C.cand_cap) {
    C.counters[3] = 1;
    return;
  }
  Cand c;
  canonical(fv, j0, j1, j2, j3, c.k);
  c.fv = fv;
  c.na = na;
  c.nb = nb;
  c.test = test;
  C.cand[slot] = c;
}

// the 9 edge pairs of a triangle pair, in the reference's order
__constant__ int kEE[9][4] = {{0, 1, 0, 1}, {0, 1, 1, 2}, {0, 1, 2, 0}, {1, 2, 0, 1}, {1, 2, 1, 2},
                              {1, 2, 2, 0}, {2, 0, 0, 1}, {2, 0, 1, 2}, {2, 0, 2, 0}};

__device__ __forceinline__ void count_fp64_test(const Arena& A, int slot) {
  if (!A.count_bytes) return;
  const unsigned m = __activemask();
  if ((threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(&A.bytes_acc[slot], (unsigned long long)__popc(m));
}

// Narrow phase (bvh_aabb.cpp:473-536 proximity, 836-901 CCD) in two passes.
// Pass 1: one thread per leaf pair runs the FP32 prefilters of the pair's 15
// elementary tests (0-2: face a vs the vertices of b; 3-5: face b vs the
// vertices of a; 6-14: the 9 edge pairs).  The prefilters reject only what the
// FP64 tests reject; the survivors are queued (face-vertex and edge-edge tests
// apart).  Pass 2: the FP64 tests run on
// the packed queues, one kind per kernel, so their warps stay full.  The
// candidates' order does not matter (they are sorted afterwards).
// Pass 1 for leaf pair pid: the tests that survive the FP32 prefilters, as
// bit masks (face-vertex tests 0-5, edge-edge tests 6-14 as bits 0-8)
__device__ __forceinline__ void narrow_filter_pair(const Arena& A, const ContactBufs& C, int ccd,
                                                   double delta_override, int pid, unsigned& fvm,
                                                   unsigned& eem) {
  // the 9 edge pairs of a triangle pair (kEE), as compile-time indices
  constexpr int kE[9][4] = {{0, 1, 0, 1}, {0, 1, 1, 2}, {0, 1, 2, 0}, {1, 2, 0, 1}, {1, 2, 1, 2},
                            {1, 2, 2, 0}, {2, 0, 0, 1}, {2, 0, 1, 2}, {2, 0, 2, 0}};
  const int2 pr = C.pairs[pid];
  const int na = pr.x, nb = pr.y;
  const int ta = A.node[3 * na + 1], tb = A.node[3 * nb + 1];
  const int inst = A.tinst[ta];
  if (A.st[inst].diverged) return;
  const double delta = delta_override >= 0 ? delta_override : A.prm[inst].contact_clearance;
  const float du = __double2float_ru(delta);
  int va[3], vb[3];
  // the FP32 bounds (lo[3], hi[3]) of the six vertices, read once
  float ba[3][6], bb[3][6];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    va[m] = A.tri[3 * ta + m];
    vb[m] = A.tri[3 * tb + m];
    const float2* pa = reinterpret_cast<const float2*>(A.vb32 + 6 * (size_t)va[m]);
    const float2* pb = reinterpret_cast<const float2*>(A.vb32 + 6 * (size_t)vb[m]);
#pragma unroll
    for (int h = 0; h < 3; h++) {
      const float2 x = pa[h], y = pb[h];
      ba[m][2 * h] = x.x;
      ba[m][2 * h + 1] = x.y;
      bb[m][2 * h] = y.x;
      bb[m][2 * h + 1] = y.y;
    }
  }
  // face-vertex: the vertex inside the face's box (the reference's aBB quirk for
  // proximity: the node whose index is the triangle's index within its cloth)
  {
    float fa[6], fb[6];
    const int bna = ccd ? na : A.noff[inst] + (ta - A.toff[inst]);
    const int bnb = ccd ? nb : A.noff[inst] + (tb - A.toff[inst]);
    const float2* qa = reinterpret_cast<const float2*>(A.box32 + 6 * (size_t)bna);
    const float2* qb = reinterpret_cast<const float2*>(A.box32 + 6 * (size_t)bnb);
#pragma unroll
    for (int h = 0; h < 3; h++) {
      const float2 x = qa[h], y = qb[h];
      fa[2 * h] = x.x;
      fa[2 * h + 1] = x.y;
      fb[2 * h] = y.x;
      fb[2 * h + 1] = y.y;
    }
#pragma unroll
    for (int test = 0; test < 6; test++) {
      const bool on_a = test < 3;
      const int k = on_a ? test : test - 3;
      const int q = on_a ? vb[k] : va[k];
      const int* f = on_a ? va : vb;
      if (q == f[0] || q == f[1] || q == f[2]) continue;
      if (!overlap32(on_a ? fa : fb, on_a ? bb[k] : ba[k])) continue;
      fvm |= 1u << test;
    }
  }
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const int i0 = va[kE[k][0]], i1 = va[kE[k][1]];
    const int j0 = vb[kE[k][2]], j1 = vb[kE[k][3]];
    if (i0 == j0 || i0 == j1 || i1 == j0 || i1 == j1) continue;
    // for CCD the edges' swept boxes must overlap; for proximity the reference's
    // six slab tests (bvh_aabb.cpp:420-425) are bounded with directed rounding,
    // then the closest-point / distance filter
    const float *a0 = ba[kE[k][0]], *a1 = ba[kE[k][1]], *b0 = bb[kE[k][2]], *b1 = bb[kE[k][3]];
    bool keep = true;
    if (ccd) {
      float ea[6], eb[6];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        ea[c] = fminf(a0[c], a1[c]);
        ea[3 + c] = fmaxf(a0[3 + c], a1[3 + c]);
        eb[c] = fminf(b0[c], b1[c]);
        eb[3 + c] = fmaxf(b0[3 + c], b1[3 + c]);
      }
      keep = overlap32(ea, eb);
    } else {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float plo = fminf(a0[c], a1[c]), phi = fmaxf(a0[3 + c], a1[3 + c]);
        const float qlo = fminf(b0[c], b1[c]), qhi = fmaxf(b0[3 + c], b1[3 + c]);
        if (__fadd_ru(qhi, du) < plo || __fsub_rd(qlo, du) > phi) keep = false;
      }
      if (keep && ee_prx_reject32(a0, a1, b0, b1, du)) keep = false;
    }
    if (keep) eem |= 1u << k;
  }
}

// The survivors of a warp's 32 leaf pairs into the two test queues: one atomic
// per queue and warp (a scan of the lanes' counts gives each lane its slots).
// Every lane of the warp calls it; the queue order does not matter (the
// contact set is sorted by key afterwards).
__device__ __forceinline__ void enqueue_masks(const ContactBufs& C, int pid, unsigned fvm, unsigned eem) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int nf = __popc(fvm), ne = __popc(eem);
  int sf = nf, se = ne;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int yf = __shfl_up_sync(full, sf, o), ye = __shfl_up_sync(full, se, o);
    if (lane >= o) {
      sf += yf;
      se += ye;
    }
  }
  const int tf = __shfl_sync(full, sf, 31), te = __shfl_sync(full, se, 31);
  int bf = 0, be = 0;
  if (lane == 0) {
    if (tf) bf = atomicAdd(&C.counters[6], tf);
    if (te) be = atomicAdd(&C.counters[7], te);
  }
  bf = __shfl_sync(full, bf, 0);
  be = __shfl_sync(full, be, 0);
  int of = bf + sf - nf, oe = be + se - ne;
  while (fvm) {
    const int t = __ffs(fvm) - 1;
    fvm &= fvm - 1;
    if ((unsigned)of < (unsigned)C.q_cap[0])
      C.queue[0][of] = make_int2(pid, t);
    else
      C.counters[3] = 1;
    of++;
  }
  while (eem) {
    const int t = __ffs(eem) - 1;
    eem &= eem - 1;
    if ((unsigned)oe < (unsigned)C.q_cap[1])
      C.queue[1][oe] = make_int2(pid, 6 + t);
    else
      C.counters[3] = 1;
    oe++;
  }
}

__global__ void __launch_bounds__(kT) k_narrow_filter(Arena A, ContactBufs C, int ccd, double delta_override,
                                                      int npairs) {
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned fvm = 0, eem = 0;
  if (pid < npairs) narrow_filter_pair(A, C, ccd, delta_override, pid, fvm, eem);
  enqueue_masks(C, pid, fvm, eem);
}

// the same over the pair count the broad phase left on the device (grid-stride,
// the loop uniform over each block so that whole warps enqueue together)
__global__ void __launch_bounds__(kT) k_narrow_filter_dev(Arena A, ContactBufs C, int ccd, double delta_override) {
  const int n = min(__ldcg(&C.counters[0]), C.pair_cap);
  for (int b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
    const int pid = b + threadIdx.x;
    unsigned fvm = 0, eem = 0;
    if (pid < n) narrow_filter_pair(A, C, ccd, delta_override, pid, fvm, eem);
    enqueue_masks(C, pid, fvm, eem);
  }
}

// pass 2, face-vertex tests (grid-stride over their queue)
__device__ __forceinline__ void narrow_fv_body(const Arena& A, const ContactBufs& C, int ccd, const double* xs,
                                               const double* vs, double delta_override) {
  const int n = min(__ldcg(&C.counters[6]), C.q_cap[0]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 it = C.queue[0][i];
    const int2 pr = C.pairs[it.x];
    const int na = pr.x, nb = pr.y, test = it.y;
    const int ta = A.node[3 * na + 1], tb = A.node[3 * nb + 1];
    const int inst = A.tinst[ta];
    const DevParams& P = A.prm[inst];
    const double delta = delta_override >= 0 ? delta_override : P.contact_clearance;
    const bool fa = test < 3;
    const int tf = fa ? ta : tb, tv = fa ? tb : ta, k = fa ? test : test - 3;
    const int f0 = A.tri[3 * tf], f1 = A.tri[3 * tf + 1], f2 = A.tri[3 * tf + 2], q = A.tri[3 * tv + k];
    const V3<double> p0 = ld3(xs, f0), p1 = ld3(xs, f1), p2 = ld3(xs, f2), p3 = ld3(xs, q);
    if (!ccd) {
      count_fp64_test(A, 2);
      // the reference passes aBB[triangle index]: the box of the node whose
      // index equals the triangle's index within its cloth
      const Box bb = A.box[A.noff[inst] + (tf - A.toff[inst])];
      if (fv_proximity(f0, f1, f2, q, p0, p1, p2, p3, bb, delta)) emit(C, 1, f0, f1, f2, q, na, nb, test);
    } else {
      // FP32 certificates that the FP64 test rejects (cert.cuh): the vertex
      // stays on one side of the start face plane (the test's sign block), the
      // four points are never coplanar in [0, 1] (FindCoplanerInterp returns
      // -1), or at any coplanarity time the vertex projects outside the face;
      // from enclosures of the FP64 differences the FP64 test itself forms
      // (the whole-motion stage here, the piece stage on the packed survivors
      // in k_narrow_fv_pieces, so each stage's warps stay full)
      RV x1, x2, x3, v1, v2, v3;
      ccd_xv(ld_ps(A, f0), ld_ps(A, f1), ld_ps(A, f2), ld_ps(A, q), x1, x2, x3, v1, v2, v3);
      if (fv_ccd_whole32(x1, x2, x3, v1, v2, v3)) continue;
      C.queue64[0][warp_append(&C.counters[10])] = it;
    }
  }
}

// The piece stage of the certificates on the tests the whole-motion stage
// kept (queue64[kind], counters[10 + kind]); the tests it cannot reject go to
// the FP64 test, packed into queue[kind] (free again after pass 2),
// counters[12 + kind].
template <bool kFV>
__device__ __forceinline__ void narrow_pieces_body(const Arena& A, const ContactBufs& C) {
  constexpr int kind = kFV ? 0 : 1;
  const int n = __ldcg(&C.counters[10 + kind]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 it = C.queue64[kind][i];
    const int2 pr = C.pairs[it.x];
    const int ta = A.node[3 * pr.x + 1], tb = A.node[3 * pr.y + 1];
    int a, b, c, d;
    if (kFV) {
      const bool fa = it.y < 3;
      const int tf = fa ? ta : tb, tv = fa ? tb : ta, k = fa ? it.y : it.y - 3;
      a = A.tri[3 * tf], b = A.tri[3 * tf + 1], c = A.tri[3 * tf + 2], d = A.tri[3 * tv + k];
    } else {
      const int k = it.y - 6;
      a = A.tri[3 * ta + kEE[k][0]], b = A.tri[3 * ta + kEE[k][1]];
      c = A.tri[3 * tb + kEE[k][2]], d = A.tri[3 * tb + kEE[k][3]];
    }
    RV x1, x2, x3, v1, v2, v3;
    ccd_xv(ld_ps(A, a), ld_ps(A, b), ld_ps(A, c), ld_ps(A, d), x1, x2, x3, v1, v2, v3);
    if (ccd_pieces_stage32<kFV>(x1, x2, x3, v1, v2, v3)) continue;
    C.queue[kind][warp_append(&C.counters[12 + kind])] = it;
  }
}

// the face-vertex continuous-collision tests the certificates left (FP64)
__device__ __forceinline__ void narrow_fv64_body(const Arena& A, const ContactBufs& C, const double* xs,
                                                 const double* vs) {
  const int n = __ldcg(&C.counters[12]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 it = C.queue[0][i];
    const int2 pr = C.pairs[it.x];
    const int na = pr.x, nb = pr.y, test = it.y;
    const int ta = A.node[3 * na + 1], tb = A.node[3 * nb + 1];
    const DevParams& P = A.prm[A.tinst[ta]];
    const bool fa = test < 3;
    const int tf = fa ? ta : tb, tv = fa ? tb : ta, k = fa ? test : test - 3;
    const int f0 = A.tri[3 * tf], f1 = A.tri[3 * tf + 1], f2 = A.tri[3 * tf + 2], q = A.tri[3 * tv + k];
    const V3<double> p0 = ld3(xs, f0), p1 = ld3(xs, f1), p2 = ld3(xs, f2), p3 = ld3(xs, q);
    const V3<double> q0 = end_pos(xs, vs, f0, P.dt), q1 = end_pos(xs, vs, f1, P.dt);
    const V3<double> q2 = end_pos(xs, vs, f2, P.dt), q3 = end_pos(xs, vs, q, P.dt);
    count_fp64_test(A, 4);
    const Box bb = A.box[fa ? na : nb];
    if (fv_ccd(f0, f1, f2, q, p0, p1, p2, p3, q0, q1, q2, q3, bb)) emit(C, 1, f0, f1, f2, q, na, nb, test);
  }
}

// the face-vertex pass as compiled freely (about 164 registers) and capped at
// 128 registers for 4 blocks per SM (more warps in flight, a few spills):
// the autotuner picks one per arena (Arena::narrow_regs)
__global__ void k_narrow_fv(Arena A, ContactBufs C, int ccd, const double* xs, const double* vs,
                            double delta_override) {
  narrow_fv_body(A, C, ccd, xs, vs, delta_override);
}
__global__ void __launch_bounds__(kT, 4) k_narrow_fv_b4(Arena A, ContactBufs C, int ccd, const double* xs,
                                                        const double* vs, double delta_override) {
  narrow_fv_body(A, C, ccd, xs, vs, delta_override);
}

// pass 2, edge-edge tests (grid-stride over their queue)
__device__ __forceinline__ void narrow_ee_body(const Arena& A, const ContactBufs& C, int ccd, const double* xs,
                                               const double* vs, double delta_override) {
  const int n = min(__ldcg(&C.counters[7]), C.q_cap[1]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 it = C.queue[1][i];
    const int2 pr = C.pairs[it.x];
    const int na = pr.x, nb = pr.y, test = it.y;
    const int ta = A.node[3 * na + 1], tb = A.node[3 * nb + 1];
    const int inst = A.tinst[ta];
    const DevParams& P = A.prm[inst];
    const double delta = delta_override >= 0 ? delta_override : P.contact_clearance;
    const int k = test - 6;
    const int i0 = A.tri[3 * ta + kEE[k][0]], i1 = A.tri[3 * ta + kEE[k][1]];
    const int j0 = A.tri[3 * tb + kEE[k][2]], j1 = A.tri[3 * tb + kEE[k][3]];
    const V3<double> p0 = ld3(xs, i0), p1 = ld3(xs, i1), q0 = ld3(xs, j0), q1 = ld3(xs, j1);
    if (!ccd) {
      // second filter stage on FP64 differences (nearly parallel edges)
      if (ee_prx_reject_rel(p0, p1, q0, q1, __double2float_ru(delta))) continue;
      count_fp64_test(A, 3);
      if (ee_proximity(i0, i1, j0, j1, p0, p1, q0, q1, delta)) emit(C, 0, i0, i1, j0, j1, na, nb, test);
    } else {
      // FP32 certificates that the FP64 test rejects (cert.cuh): no coplanarity
      // in [0, 1], the edges more than the test's 1e-2 apart over the whole
      // motion, or at any coplanarity time a ratio out of range or the edges
      // apart; from enclosures of the vectors coplanar_time forms
      // (the whole-motion stage here, the piece stage on the packed survivors
      // in k_narrow_ee_pieces)
      RV x1, x2, x3, v1, v2, v3;
      ccd_xv(ld_ps(A, i0), ld_ps(A, i1), ld_ps(A, j0), ld_ps(A, j1), x1, x2, x3, v1, v2, v3);
      if (ee_ccd_whole32(x1, x2, x3, v1, v2, v3)) continue;
      C.queue64[1][warp_append(&C.counters[11])] = it;
    }
  }
}

// the edge-edge continuous-collision tests the certificates left (FP64)
__device__ __forceinline__ void narrow_ee64_body(const Arena& A, const ContactBufs& C, const double* xs,
                                                 const double* vs) {
  const int n = __ldcg(&C.counters[13]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 it = C.queue[1][i];
    const int2 pr = C.pairs[it.x];
    const int na = pr.x, nb = pr.y, test = it.y;
    const int ta = A.node[3 * na + 1], tb = A.node[3 * nb + 1];
    const DevParams& P = A.prm[A.tinst[ta]];
    const int k = test - 6;
    const int i0 = A.tri[3 * ta + kEE[k][0]], i1 = A.tri[3 * ta + kEE[k][1]];
    const int j0 = A.tri[3 * tb + kEE[k][2]], j1 = A.tri[3 * tb + kEE[k][3]];
    const V3<double> p0 = ld3(xs, i0), p1 = ld3(xs, i1), q0 = ld3(xs, j0), q1 = ld3(xs, j1);
    const V3<double> p0e = end_pos(xs, vs, i0, P.dt), p1e = end_pos(xs, vs, i1, P.dt);
    const V3<double> q0e = end_pos(xs, vs, j0, P.dt), q1e = end_pos(xs, vs, j1, P.dt);
    count_fp64_test(A, 5);
    if (ee_ccd(i0, i1, j0, j1, p0, p1, q0, q1, p0e, p1e, q0e, q1e)) emit(C, 0, i0, i1, j0, j1, na, nb, test);
  }
}

__global__ void k_narrow_ee(Arena A, ContactBufs C, int ccd, const double* xs, const double* vs,
                            double delta_override) {
  narrow_ee_body(A, C, ccd, xs, vs, delta_override);
}
__global__ void __launch_bounds__(kT, 4) k_narrow_ee_b4(Arena A, ContactBufs C, int ccd, const double* xs,
                                                        const double* vs, double delta_override) {
  narrow_ee_body(A, C, ccd, xs, vs, delta_override);
}
__global__ void k_narrow_fv_pieces(Arena A, ContactBufs C) { narrow_pieces_body<true>(A, C); }
__global__ void k_narrow_ee_pieces(Arena A, ContactBufs C) { narrow_pieces_body<false>(A, C); }
__global__ void k_narrow_fv64(Arena A, ContactBufs C, const double* xs, const double* vs) {
  narrow_fv64_body(A, C, xs, vs);
}
__global__ void __launch_bounds__(kT, 4) k_narrow_fv64_b4(Arena A, ContactBufs C, const double* xs,
                                                          const double* vs) {
  narrow_fv64_body(A, C, xs, vs);
}
__global__ void k_narrow_ee64(Arena A, ContactBufs C, const double* xs, const double* vs) {
  narrow_ee64_body(A, C, xs, vs);
}
__global__ void __launch_bounds__(kT, 4) k_narrow_ee64_b4(Arena A, ContactBufs C, const double* xs,
                                                          const double* vs) {
  narrow_ee64_body(A, C, xs, vs);
}

// The passes after the FP32 prefilter, in the arena's register variant:
// face-vertex and edge-edge tests (proximity: the FP64 tests; continuous
// collision: the FP32 certificates, then the FP64 tests they leave, packed)
void narrow_fp64_passes(const Arena& A, const ContactBufs& C, int ccd, const double* xs, const double* vs,
                        double delta_override, int grid, cudaStream_t s) {
  const bool b4 = A.narrow_regs == 128;
  if (ccd) {
    k_ccd_split<<<nblk(A.nv), kT, 0, s>>>(A, xs, vs);
    g_launches++;
  }
  prof_begin(PK_NARROW_FV, s);
  if (b4)
    k_narrow_fv_b4<<<grid, kT, 0, s>>>(A, C, ccd, xs, vs, delta_override);
  else
    k_narrow_fv<<<grid, kT, 0, s>>>(A, C, ccd, xs, vs, delta_override);
  prof_end(PK_NARROW_FV, s);
  prof_begin(PK_NARROW_EE, s);
  if (b4)
    k_narrow_ee_b4<<<grid, kT, 0, s>>>(A, C, ccd, xs, vs, delta_override);
  else
    k_narrow_ee<<<grid, kT, 0, s>>>(A, C, ccd, xs, vs, delta_override);
  prof_end(PK_NARROW_EE, s);
  if (!ccd) return;
  prof_begin(PK_NARROW_FV, s);
  k_narrow_fv_pieces<<<grid, kT, 0, s>>>(A, C);
  prof_end(PK_NARROW_FV, s);
  prof_begin(PK_NARROW_EE, s);
  k_narrow_ee_pieces<<<grid, kT, 0, s>>>(A, C);
  prof_end(PK_NARROW_EE, s);
  g_launches += 2;
  prof_begin(PK_NARROW_CCD64, s);
  if (b4) {
    k_narrow_fv64_b4<<<grid, kT, 0, s>>>(A, C, xs, vs);
    k_narrow_ee64_b4<<<grid, kT, 0, s>>>(A, C, xs, vs);
  } else {
    k_narrow_fv64<<<grid, kT, 0, s>>>(A, C, xs, vs);
    k_narrow_ee64<<<grid, kT, 0, s>>>(A, C, xs, vs);
  }
  prof_end(PK_NARROW_CCD64, s);
  g_launches += 2;
}

__device__ __forceinline__ unsigned long long key_hi(const Cand& c) {
  return ((unsigned long long)(unsigned)c.k[0] << 32) | (unsigned)c.k[1];
}
__device__ __forceinline__ unsigned long long key_lo(const Cand& c) {
  return ((unsigned long long)(unsigned)c.k[2] << 32) | (unsigned)c.k[3];
}

__global__ void k_keys_lo(ContactBufs C, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  C.key_a[i] = key_lo(C.cand[i]);
  C.idx_a[i] = i;
}

__global__ void k_keys_hi(ContactBufs C, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  C.key_a[i] = key_hi(C.cand[C.idx_b[i]]);
}

__global__ void k_gather_cand(ContactBufs C, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  C.cand_sorted[i] = C.cand[C.idx_a[i]];
}

__device__ __forceinline__ bool same_key(const Cand& a, const Cand& b) {
  return a.k[0] == b.k[0] && a.k[1] == b.k[1] && a.k[2] == b.k[2] && a.k[3] == b.k[3];
}

constexpr int kMaxDepth = 128;

// child choices (0 / 1) from below `top` down to `leaf`, top-down; returns the count
__device__ int path_bits(const Arena& A, int top, int leaf, unsigned char* bits) {
  int n = 0;
  int cur = leaf;
  while (cur != top && n < kMaxDepth) {
    const int par = A.node[3 * cur];
    bits[n++] = (A.node[3 * par + 2] == cur) ? 1 : 0;
    cur = par;
  }
  for (int i = 0; i < n / 2; i++) {
    const unsigned char t = bits[i];
    bits[i] = bits[n - 1 - i];
    bits[n - 1 - i] = t;
  }
  return n;
}

__device__ int lca(const Arena& A, int a, int b) {
  while (A.depth[a] > A.depth[b]) a = A.node[3 * a];
  while (A.depth[b] > A.depth[a]) b = A.node[3 * b];
  while (a != b) {
    a = A.node[3 * a];
    b = A.node[3 * b];
  }
  return a;
}

// True when the reference's recursive traversal reaches candidate x before y.
// Pairs are visited grouped by their lowest common ancestor in depth-first
// preorder (walk_self: pair(child0, child1), then each subtree); within one
// ancestor the simultaneous descent of walk_pair orders children as
// (0,0), (1,0), (0,1), (1,1) while both sides are internal, then by the side
// still internal; within a leaf pair, by test index.
__device__ bool visited_before(const Arena& A, const Cand& x, const Cand& y) {
  const int lx = lca(A, x.na, x.nb), ly = lca(A, y.na, y.nb);
  if (lx != ly) return A.prepos[lx] < A.prepos[ly];
  if (x.na == y.na && x.nb == y.nb) return x.test < y.test;
  const int c0 = A.node[3 * lx + 1], c1 = A.node[3 * lx + 2];
  unsigned char xa[kMaxDepth], xb[kMaxDepth], ya[kMaxDepth], yb[kMaxDepth];
  const int mxa = path_bits(A, c0, x.na, xa), mxb = path_bits(A, c1, x.nb, xb);
  const int mya = path_bits(A, c0, y.na, ya), myb = path_bits(A, c1, y.nb, yb);
  for (int k = 0;; k++) {
    const bool xi = k < mxa || k < mxb, yi = k < mya || k < myb;
    if (!xi || !yi) return xi < yi;  // unreachable for distinct pairs
    const int dx = (k < mxa && k < mxb) ? xa[k] + 2 * xb[k] : (k < mxa ? xa[k] : xb[k]);
    const int dy = (k < mya && k < myb) ? ya[k] + 2 * yb[k] : (k < mya ? ya[k] : yb[k]);
    if (dx != dy) return dx < dy;
  }
}

// run heads of the sorted candidates and the element std::set keeps for each key
__global__ void k_dedupe(Arena A, ContactBufs C, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Cand ci = C.cand_sorted[i];
  const bool head = (i == 0) || !same_key(C.cand_sorted[i - 1], ci);
  C.idx_b[i] = head ? 1 : 0;
  if (!head) return;
  int j = i + 1;
  bool mixed = false;
  while (j < n && same_key(C.cand_sorted[j], ci)) {
    mixed |= (C.cand_sorted[j].fv != ci.fv);
    j++;
  }
  int win = i;
  if (mixed)
    for (int k = i + 1; k < j; k++)
      if (visited_before(A, C.cand_sorted[k], C.cand_sorted[win])) win = k;
  C.level[i] = C.cand_sorted[win].fv;
}

__global__ void k_compact(Arena A, ContactBufs C, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pos = C.idx_a[i];
  if (i == n - 1) C.counters[2] = pos + C.idx_b[i];
  if (!C.idx_b[i]) return;
  const Cand c = C.cand_sorted[i];
  C.ce[5 * pos + 0] = C.level[i];
  C.ce[5 * pos + 1] = c.k[0];
  C.ce[5 * pos + 2] = c.k[1];
  C.ce[5 * pos + 3] = c.k[2];
  C.ce[5 * pos + 4] = c.k[3];
}

// per-cloth segments of the contact list (contacts of one cloth are contiguous
// because vertex ids of a cloth are contiguous and lists are sorted)
__global__ void k_segments(Arena A, ContactBufs C) {
  const int n = C.counters[2];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int inst = A.vinst[C.ce[5 * e + 1]];
  if (e == 0 || A.vinst[C.ce[5 * (e - 1) + 1]] != inst) C.ce_inst_lo[inst] = e;
  if (e == n - 1 || A.vinst[C.ce[5 * (e + 1) + 1]] != inst) C.ce_inst_hi[inst] = e + 1;
}

__global__ void k_counts(Arena A, ContactBufs C) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= A.ni) return;
  A.st[inst].n_contacts = A.active[inst] ? C.ce_inst_hi[inst] - C.ce_inst_lo[inst] : 0;
  A.st[inst].riz_nodes = 0;
}

// ---- impulses (self_collision_cloth.cpp:20-212) ------------------------------
// levels of the sequential sweep, one thread per cloth
__global__ void k_token_next(Arena A) { A.ctl->token++; }

// Impulse levels of each cloth's contacts, one warp per cloth.  The
// Gauss-Seidel sweep of SelfCollisionImpulse_* (self_collision_cloth.cpp:20-212)
// is sequential in set order; a contact's level is one more than the highest
// level among the earlier contacts that share a vertex with it (0 if none), so
// the contacts of a level share no vertex and each follows every earlier
// contact it depends on: applying the levels in turn reproduces the sweep.
// The warp takes the contacts 32 at a time in set order: a lane's in-chunk
// predecessor for each of its 4 vertices is the last earlier lane touching it
// (found with shuffles); a vertex without one takes the level its last
// toucher before the chunk left in vmark (stamped with this detection's
// token); the in-chunk levels then settle in at most 32 rounds, and for each
// vertex the chunk's last toucher writes its level back.  The contacts are
// then grouped by level (counts, a prefix sum, a scatter; the order within a
// level does not matter, its contacts being independent).
__global__ void k_impulse_levels(Arena A, ContactBufs C, int ccd) {
  const int inst = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (inst >= A.ni) return;  // the whole warp
  const int token = A.ctl->token;
  if (lane == 0) A.st[inst].nlev = 0;
  if (!A.active[inst]) return;
  const int lo = C.ce_inst_lo[inst], hi = C.ce_inst_hi[inst];
  if (lo >= hi) return;
  const unsigned full = 0xffffffffu;
  int nlev = 0;
  for (int base = lo; base < hi; base += 32) {
    const int c = base + lane;
    const bool valid = c < hi;
    // a proximity contact that the positions alone reject changes no velocity:
    // it depends on nothing and nothing depends on it (level 0)
    const bool live = valid && (ccd || C.imp_pre[9 * (size_t)c + 8] != 0.0);
    int vv[4];
#pragma unroll
    for (int k = 0; k < 4; k++) vv[k] = live ? C.ce[5 * c + 1 + k] : -1 - 4 * lane - k;  // no match
    int pred[4] = {-1, -1, -1, -1};
    bool last[4] = {true, true, true, true};
    for (int j = 0; j < 32; j++) {
      const int u0 = __shfl_sync(full, vv[0], j), u1 = __shfl_sync(full, vv[1], j);
      const int u2 = __shfl_sync(full, vv[2], j), u3 = __shfl_sync(full, vv[3], j);
      if (j == lane) continue;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (vv[k] == u0 || vv[k] == u1 || vv[k] == u2 || vv[k] == u3) {
          if (j < lane)
            pred[k] = j;
          else
            last[k] = false;
        }
      }
    }
    int ext = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (live && pred[k] < 0) {
        const int v = vv[k];
        if (C.vstamp[v] == token) ext = max(ext, C.vmark[v] + 1);
      }
    }
    int l = ext;
    for (int round = 0; round < 32; round++) {
      int m = ext;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int lp = __shfl_sync(full, l, pred[k] < 0 ? lane : pred[k]);
        if (pred[k] >= 0) m = max(m, lp + 1);
      }
      const bool changed = m != l;
      l = m;
      if (!__any_sync(full, changed)) break;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (live && last[k]) {
        C.vmark[vv[k]] = l;
        C.vstamp[vv[k]] = token;
      }
    }
    if (valid) C.level[c] = l;
    int top = valid ? l + 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) top = max(top, __shfl_xor_sync(full, top, o));
    nlev = max(nlev, top);
    __syncwarp();  // the marks are read by the next chunk's lanes
  }
  // group by level: counts at off[l + 1], prefix sums (off[l] = first of level
  // l), a scatter that advances off[l] to the end of level l, and a shift back
  int* off = C.lev_cnt + lo + inst;  // nlev + 1 counters, disjoint per cloth
  for (int l = lane; l <= nlev; l += 32) off[l] = 0;
  __syncwarp();
  for (int c = lo + lane; c < hi; c += 32) atomicAdd(&off[C.level[c] + 1], 1);
  __syncwarp();
  int carry = 0;
  for (int b0 = 0; b0 <= nlev; b0 += 32) {
    const int l = b0 + lane;
    int x = l <= nlev ? off[l] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(full, x, o);
      if (lane >= o) x += y;
    }
    x += carry;
    if (l <= nlev) off[l] = x;
    carry = __shfl_sync(full, x, 31);
  }
  __syncwarp();
  for (int c = lo + lane; c < hi; c += 32) C.order[lo + atomicAdd(&off[C.level[c]], 1)] = c;
  __syncwarp();
  for (int b0 = ((nlev + 31) / 32) * 32; b0 >= 0; b0 -= 32) {
    const int l = b0 + lane;
    const int x = (l >= 1 && l <= nlev) ? off[l - 1] : 0;
    __syncwarp();
    if (l >= 1 && l <= nlev) off[l] = x;
    __syncwarp();
  }
  if (lane == 0) {
    off[0] = 0;
    A.st[inst].nlev = nlev;
  }
}

__device__ __forceinline__ void add_v(double* v, int i, double a, double b, double c) {
  v[3 * i + 0] += a;
  v[3 * i + 1] += b;
  v[3 * i + 2] += c;
}

// Position-only terms of one proximity impulse (SelfCollisionImpulse_Proximity,
// self_collision_cloth.cpp:20-112), computed for every contact in parallel
// before the sweep, in q: the barycentric weights (w0 w1 w2, or w01 w23), the
// normal, the threshold 0.1 depth / dt, the elastic impulse dt stiff depth and
// the weight denominator.  A contact that the positions alone reject (weights
// outside [0, 1], distance above the clearance) gets a zero denominator: it
// changes no velocity and leaves the sweep's dependency chain.
__device__ void prox_prep(const DevParams& P, const int* e, const double* x, double* q) {
  const double delta = P.contact_clearance, stiff = P.stiff_contact, dt = P.dt;
  const int i0 = e[1], i1 = e[2], i2 = e[3], i3 = e[4];
  const V3<double> p0 = ld3(x, i0), p1 = ld3(x, i1), p2 = ld3(x, i2), p3 = ld3(x, i3);
  q[8] = 0.0;
  if (e[0]) {  // face (i0 i1 i2) - vertex i3
    double w0, w1;
    const double dist = dist_face_vertex(p0, p1, p2, p3, w0, w1);
    if (w0 < 0 || w0 > 1) return;
    if (w1 < 0 || w1 > 1) return;
    if (dist > delta) return;
    const double w2 = 1.0 - w0 - w1;
    const V3<double> pc = w0 * p0 + w1 * p1 + w2 * p2;
    const V3<double> nrm = normalized(p3 - pc);
    const double depth = delta - dot(p3 - pc, nrm);
    q[0] = w0;
    q[1] = w1;
    q[2] = w2;
    q[3] = nrm.x;
    q[4] = nrm.y;
    q[5] = nrm.z;
    q[6] = 0.1 * depth / dt;
    q[7] = dt * stiff * depth;
    q[8] = 1 + w0 * w0 + w1 * w1 + w2 * w2;
  } else {  // edge (i0 i1) - edge (i2 i3)
    double w01, w23;
    const double dist = dist_edge_edge(p0, p1, p2, p3, w01, w23);
    if (w01 < 0 || w01 > 1) return;
    if (w23 < 0 || w23 > 1) return;
    if (dist > delta) return;
    const V3<double> c01 = (1 - w01) * p0 + w01 * p1;
    const V3<double> c23 = (1 - w23) * p2 + w23 * p3;
    const V3<double> nrm = normalized(c23 - c01);
    const double depth = delta - length(c23 - c01);
    q[0] = w01;
    q[1] = w23;
    q[2] = 0.0;
    q[3] = nrm.x;
    q[4] = nrm.y;
    q[5] = nrm.z;
    q[6] = 0.1 * depth / dt;
    q[7] = dt * stiff * depth;
    q[8] = w01 * w01 + (1 - w01) * (1 - w01) + w23 * w23 + (1 - w23) * (1 - w23);
  }
}

// the velocity part of one proximity impulse, from the terms of prox_prep
__device__ void impulse_prx(const DevParams& P, const int* e, const double* q, double* v) {
  const double den = q[8];
  if (den == 0.0) return;
  const double mass = P.mass_point;
  const int i0 = e[1], i1 = e[2], i2 = e[3], i3 = e[4];
  const V3<double> v0 = ld3((const double*)v, i0), v1 = ld3((const double*)v, i1), v2 = ld3((const double*)v, i2),
                   v3 = ld3((const double*)v, i3);
  const V3<double> nrm = mk<double>(q[3], q[4], q[5]);
  const double thr = q[6], imp_el = q[7];
  if (e[0]) {  // face (i0 i1 i2) - vertex i3
    const double w0 = q[0], w1 = q[1], w2 = q[2];
    const double rel_v = dot(v3 - w0 * v0 - w1 * v1 - w2 * v2, nrm);
    if (rel_v > thr) return;
    const double imp_ie = mass * (thr - rel_v);
    const double imp_min = (imp_el < imp_ie) ? imp_el : imp_ie;
    double imp_mod = 2 * imp_min / den;
    imp_mod /= mass;
    imp_mod *= 0.25;
    const double mx = -nrm.x, my = -nrm.y, mz = -nrm.z;
    add_v(v, i0, mx * imp_mod * w0, my * imp_mod * w0, mz * imp_mod * w0);
    add_v(v, i1, mx * imp_mod * w1, my * imp_mod * w1, mz * imp_mod * w1);
    add_v(v, i2, mx * imp_mod * w2, my * imp_mod * w2, mz * imp_mod * w2);
    add_v(v, i3, nrm.x * imp_mod, nrm.y * imp_mod, nrm.z * imp_mod);
  } else {  // edge (i0 i1) - edge (i2 i3)
    const double w01 = q[0], w23 = q[1];
    const double rel_v = dot((1 - w23) * v2 + w23 * v3 - (1 - w01) * v0 - w01 * v1, nrm);
    if (rel_v > thr) return;
    const double imp_ie = mass * (thr - rel_v);
    const double imp_min = (imp_el < imp_ie) ? imp_el : imp_ie;
    double imp_mod = 2 * imp_min / den;
    imp_mod /= mass;
    imp_mod *= 0.25;
    const double mx = -nrm.x, my = -nrm.y, mz = -nrm.z;
    add_v(v, i0, mx * imp_mod * (1 - w01), my * imp_mod * (1 - w01), mz * imp_mod * (1 - w01));
    add_v(v, i1, mx * imp_mod * w01, my * imp_mod * w01, mz * imp_mod * w01);
    add_v(v, i2, nrm.x * imp_mod * (1 - w23), nrm.y * imp_mod * (1 - w23), nrm.z * imp_mod * (1 - w23));
    add_v(v, i3, nrm.x * imp_mod * w23, nrm.y * imp_mod * w23, nrm.z * imp_mod * w23);
  }
}

// one contact of the CCD sweep (SelfCollisionImpulse_CCD, self_collision_cloth.cpp:116-212)
__device__ void impulse_ccd(const DevParams& P, const int* e, const double* x, double* v) {
  const double delta = P.contact_clearance, dt = P.dt, mass = P.mass_point;
  const int i0 = e[1], i1 = e[2], i2 = e[3], i3 = e[4];
  const V3<double> p0 = ld3(x, i0), p1 = ld3(x, i1), p2 = ld3(x, i2), p3 = ld3(x, i3);
  const V3<double> v0 = ld3((const double*)v, i0), v1 = ld3((const double*)v, i1), v2 = ld3((const double*)v, i2),
                   v3 = ld3((const double*)v, i3);
  const double t = coplanar_time(p0, p1, p2, p3, p0 + v0, p1 + v1, p2 + v2, p3 + v3);
  if (t < 0 || t > 1) return;
  if (e[0]) {  // face (i0 i1 i2) - vertex i3
    double w0, w1;
    const double dist = dist_face_vertex(p0 + t * v0, p1 + t * v1, p2 + t * v2, p3 + t * v3, w0, w1);
    if (w0 < 0 || w0 > 1) return;
    if (w1 < 0 || w1 > 1) return;
    if (dist > delta) return;
    const double w2 = 1.0 - w0 - w1;
    const V3<double> pc = w0 * p0 + w1 * p1 + w2 * p2;
    const V3<double> nrm = normalized(p3 - pc);
    const double rel_v = dot(v3 - w0 * v0 - w1 * v1 - w2 * v2, nrm);
    if (rel_v > 0.1 * delta / dt) return;
    const double imp = mass * (0.1 * delta / dt - rel_v);
    double imp_mod = 2 * imp / (1.0 + w0 * w0 + w1 * w1 + w2 * w2);
    imp_mod /= mass;
    imp_mod *= 0.1;
    const double mx = -nrm.x, my = -nrm.y, mz = -nrm.z;
    add_v(v, i0, mx * imp_mod * w0, my * imp_mod * w0, mz * imp_mod * w0);
    add_v(v, i1, mx * imp_mod * w1, my * imp_mod * w1, mz * imp_mod * w1);
    add_v(v, i2, mx * imp_mod * w2, my * imp_mod * w2, mz * imp_mod * w2);
    add_v(v, i3, nrm.x * imp_mod, nrm.y * imp_mod, nrm.z * imp_mod);
  } else {  // edge (i0 i1) - edge (i2 i3)
    double w01, w23;
    const double dist = dist_edge_edge(p0 + t * v0, p1 + t * v1, p2 + t * v2, p3 + t * v3, w01, w23);
    if (w01 < 0 || w01 > 1) return;
    if (w23 < 0 || w23 > 1) return;
    if (dist > delta) return;
    const V3<double> c01 = (1 - w01) * p0 + w01 * p1;
    const V3<double> c23 = (1 - w23) * p2 + w23 * p3;
    const V3<double> nrm = normalized(c23 - c01);
    const double rel_v = dot((1 - w23) * v2 + w23 * v3 - (1 - w01) * v0 - w01 * v1, nrm);
    const double wsum = w01 * w01 + (1 - w01) * (1 - w01) + w23 * w23 + (1 - w23) * (1 - w23);
    if (rel_v > 0.1 * delta / dt) return;
    const double imp = mass * (0.1 * delta / dt - rel_v);
    double imp_mod = 2 * imp / wsum;
    imp_mod /= mass;
    imp_mod *= 0.1;
    const double mx = -nrm.x, my = -nrm.y, mz = -nrm.z;
    add_v(v, i0, mx * imp_mod * (1 - w01), my * imp_mod * (1 - w01), mz * imp_mod * (1 - w01));
    add_v(v, i1, mx * imp_mod * w01, my * imp_mod * w01, mz * imp_mod * w01);
    add_v(v, i2, nrm.x * imp_mod * (1 - w23), nrm.y * imp_mod * (1 - w23), nrm.z * imp_mod * (1 - w23));
    add_v(v, i3, nrm.x * imp_mod * w23, nrm.y * imp_mod * w23, nrm.z * imp_mod * w23);
  }
}

// contact c of the sweep
__device__ __forceinline__ void impulse_at(const DevParams& P, const ContactBufs& C, int c, const double* xs,
                                           double* vs, int ccd) {
  if (ccd)
    impulse_ccd(P, C.ce + 5 * c, xs, vs);
  else
    impulse_prx(P, C.ce + 5 * c, C.imp_pre + 9 * (size_t)c, vs);
}

// prox_prep for every contact of the list, C.counters[2] of them
__global__ void k_impulse_prep(Arena A, ContactBufs C, const double* xs) {
  const int n = C.counters[2];
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const int* e = C.ce + 5 * c;
    prox_prep(A.prm[A.vinst[e[1]]], e, xs, C.imp_pre + 9 * (size_t)c);
  }
}

// one CTA per cloth applies its levels in order
// The same sweep by a cluster of blocks per cloth (cloth = cluster index): a
// level's contacts spread over the cluster's SMs, whose FP64 pipes then work
// together, and the levels are separated by cluster barriers.
__global__ void k_impulse_apply_cluster(Arena A, ContactBufs C, int ccd, const double* xs, double* vs) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), size = (int)cl.num_blocks();
  const int inst = blockIdx.x / size;
  if (inst >= A.ni || !A.active[inst]) return;  // the whole cluster
  const int nlev = A.st[inst].nlev;
  if (nlev == 0) return;
  const int lo = C.ce_inst_lo[inst];
  const int* off = C.lev_cnt + lo + inst;
  const DevParams& P = A.prm[inst];
  const int stride = size * blockDim.x;
  for (int l = 0; l < nlev; l++) {
    for (int j = off[l] + rank * blockDim.x + threadIdx.x; j < off[l + 1]; j += stride)
      impulse_at(P, C, C.order[lo + j], xs, vs, ccd);
    cl.sync();
  }
}

__global__ void k_impulse_apply(Arena A, ContactBufs C, int ccd, const double* xs, double* vs) {
  const int inst = blockIdx.x;
  if (!A.active[inst]) return;
  const int nlev = A.st[inst].nlev;
  if (nlev == 0) return;
  const int lo = C.ce_inst_lo[inst];
  const int* off = C.lev_cnt + lo + inst;
  const DevParams& P = A.prm[inst];
  for (int l = 0; l < nlev; l++) {
    for (int j = off[l] + threadIdx.x; j < off[l + 1]; j += blockDim.x)
      impulse_at(P, C, C.order[lo + j], xs, vs, ccd);
    __syncthreads();
  }
}

// ---- rigid impact zones (self_collision_cloth.cpp:220-348) --------------------
__device__ int uf_find(int* uf, int x) {
  volatile int* u = uf;
  int p = u[x];
  while (p != x) {
    x = p;
    p = u[x];
  }
  return x;
}

// link the larger root under the smaller; parents only decrease, so every
// find terminates, and each failed exchange means another thread made progress
__device__ void uf_union(int* uf, int a, int b) {
  for (;;) {
    a = uf_find(uf, a);
    b = uf_find(uf, b);
    if (a == b) return;
    if (a > b) {
      const int t = a;
      a = b;
      b = t;
    }
    if (atomicCAS(&uf[b], b, a) == b) return;
  }
}

__global__ void k_riz_reset(Arena A) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv || !A.active[A.vinst[v]]) return;
  A.uf[v] = v;
  A.inzone[v] = 0;
}

__global__ void k_riz_count(Arena A) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  const int inst = A.vinst[v];
  if (A.active[inst] && A.inzone[v]) atomicAdd(&A.st[inst].riz_nodes, 1);
}

__global__ void k_riz_contacts(Arena A, ContactBufs C, int nce) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nce) return;
  const int* e = C.ce + 5 * c;
  if (!A.active[A.vinst[e[1]]]) return;
#pragma unroll
  for (int k = 1; k <= 4; k++) A.inzone[e[k]] = 1;
  uf_union(A.uf, e[1], e[2]);
  uf_union(A.uf, e[1], e[3]);
  uf_union(A.uf, e[1], e[4]);
}

// a contact joins every zone holding one of its vertices or a 1-ring
// neighbour of one: mesh edges between zone vertices merge their zones
__global__ void k_riz_edges(Arena A) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= A.ne) return;
  const int u = A.edge_uv[2 * e], w = A.edge_uv[2 * e + 1];
  if (!A.active[A.vinst[u]]) return;
  if (A.inzone[u] && A.inzone[w]) uf_union(A.uf, u, w);
}

__global__ void k_riz_collect(Arena A, ContactBufs C, int* count) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  if (!A.active[A.vinst[v]] || !A.inzone[v]) return;
  const int root = uf_find(A.uf, v);
  const int pos = atomicAdd(count, 1);
  C.zkey[pos] = ((unsigned long long)(unsigned)root << 32) | (unsigned)v;
}

// per zone: centroid, mean velocity, angular momentum and the reference's
// "inertia" (diagonal |v|^2 - q_i^2), all summed over members in ascending order
__device__ __forceinline__ void riz_stats_one(const Arena& A, const ContactBufs& C, int i, int n, const double* xs,
                                              const double* v0s) {
  const unsigned long long* z = C.zkey2;
  const unsigned root = (unsigned)(z[i] >> 32);
  if (i > 0 && (unsigned)(z[i - 1] >> 32) == root) return;
  int j = i;
  V3<double> gc = mk(0.0, 0.0, 0.0), av = mk(0.0, 0.0, 0.0);
  while (j < n && (unsigned)(z[j] >> 32) == root) {
    const int m = (int)(unsigned)(z[j] & 0xffffffffull);
    gc = gc + ld3(xs, m);
    av = av + ld3(v0s, m);
    j++;
  }
  const double cnt = (double)(j - i);
  gc = div_guarded(gc, cnt);
  av = div_guarded(av, cnt);
  V3<double> L = mk(0.0, 0.0, 0.0);
  double I[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = i; k < j; k++) {
    const int m = (int)(unsigned)(z[k] & 0xffffffffull);
    const V3<double> p = ld3(xs, m), u = ld3(v0s, m);
    const V3<double> q = p - gc;
    const double uu = dot(u, u);
    L = L + cross(p - gc, u - av);
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
  // CalcInvMat3 of self_collision_cloth.cpp:278-296
  const double det = +I[0] * I[4] * I[8] + I[3] * I[7] * I[2] + I[6] * I[1] * I[5] - I[0] * I[7] * I[5] -
                     I[6] * I[4] * I[2] - I[3] * I[1] * I[8];
  const double r = 1.0 / det;
  double Iv[9];
  Iv[0] = r * (I[4] * I[8] - I[5] * I[7]);
  Iv[1] = r * (I[2] * I[7] - I[1] * I[8]);
  Iv[2] = r * (I[1] * I[5] - I[2] * I[4]);
  Iv[3] = r * (I[5] * I[6] - I[3] * I[8]);
  Iv[4] = r * (I[0] * I[8] - I[2] * I[6]);
  Iv[5] = r * (I[2] * I[3] - I[0] * I[5]);
  Iv[6] = r * (I[3] * I[7] - I[4] * I[6]);
  Iv[7] = r * (I[1] * I[6] - I[0] * I[7]);
  Iv[8] = r * (I[0] * I[4] - I[1] * I[3]);
  double* rec = C.zrec + 9 * (size_t)root;
  rec[0] = gc.x;
  rec[1] = gc.y;
  rec[2] = gc.z;
  rec[3] = av.x;
  rec[4] = av.y;
  rec[5] = av.z;
  rec[6] = Iv[0] * L.x + Iv[1] * L.y + Iv[2] * L.z;
  rec[7] = Iv[3] * L.x + Iv[4] * L.y + Iv[5] * L.z;
  rec[8] = Iv[6] * L.x + Iv[7] * L.y + Iv[8] * L.z;
}

__global__ void k_riz_stats(Arena A, ContactBufs C, int n, const double* xs, const double* v0s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) riz_stats_one(A, C, i, n, xs, v0s);
}

__device__ __forceinline__ void riz_velocity_one(const ContactBufs& C, int i, const double* xs, double* vs) {
  const unsigned root = (unsigned)(C.zkey2[i] >> 32);
  const int m = (int)(unsigned)(C.zkey2[i] & 0xffffffffull);
  const double* rec = C.zrec + 9 * (size_t)root;
  const V3<double> gc = mk(rec[0], rec[1], rec[2]), omg = mk(rec[6], rec[7], rec[8]);
  const V3<double> rot = cross(ld3(xs, m) - gc, omg);
  vs[3 * m + 0] = rec[3] + (-rot.x);
  vs[3 * m + 1] = rec[4] + (-rot.y);
  vs[3 * m + 2] = rec[5] + (-rot.z);
}

__global__ void k_riz_velocity(ContactBufs C, int n, const double* xs, double* vs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) riz_velocity_one(C, i, xs, vs);
}

__global__ void k_riz_labels(Arena A, int* zone_of) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  zone_of[v] = (A.active[A.vinst[v]] && A.inzone[v]) ? uf_find(A.uf, v) : -1;
}

}  // namespace

// ---- launchers ----------------------------------------------------------------
void launch_refit(const Arena& A, int ccd, const double* xs, const double* vs, double delta_override,
                  cudaStream_t s) {
  k_vertex_bounds<<<nblk(A.nv), kT, 0, s>>>(A, ccd, xs, vs);
  g_launches++;
  cudaMemsetAsync(A.refit_cnt, 0, sizeof(int) * (size_t)A.nn, s);
  prof_begin(PK_REFIT, s);
  k_refit<<<nblk(A.nt), kT, 0, s>>>(A, ccd, xs, vs, delta_override);
  prof_end(PK_REFIT, s);
  g_launches++;
}

void launch_traverse(const Arena& A, const ContactBufs& C, cudaStream_t s) {
  prof_begin(PK_TRAVERSE, s);
  k_traverse<<<nblk(A.nt), kT, 0, s>>>(A, C);
  prof_end(PK_TRAVERSE, s);
  g_launches++;
}

void launch_traverse_dirty(const Arena& A, const ContactBufs& C, cudaStream_t s) {
  prof_begin(PK_TRAVERSE, s);
  k_traverse_dirty<<<nblk(A.nt), kT, 0, s>>>(A, C);
  prof_end(PK_TRAVERSE, s);
  g_launches++;
}

void launch_keep_clean_candidates(const Arena& A, ContactBufs& C, int ncand, cudaStream_t s) {
  int* nkeep = C.counters + 5;
  cudaMemsetAsync(nkeep, 0, sizeof(int), s);
  if (ncand > 0) {
    k_keep_clean<<<nblk(ncand), kT, 0, s>>>(A, C, ncand, nkeep);
    g_launches++;
  }
  int h = 0;
  cudaMemcpyAsync(&h, nkeep, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  if (h > 0) cudaMemcpyAsync(C.cand, C.cand_sorted, sizeof(Cand) * (size_t)h, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(C.counters + 1, nkeep, sizeof(int), cudaMemcpyDeviceToDevice, s);
}

void launch_mark_dirty(const Arena& A, const ContactBufs& C, int nce, bool zones, cudaStream_t s) {
  cudaMemsetAsync(A.vdirty, 0, sizeof(int) * (size_t)A.nv, s);
  if (zones) {
    k_mark_zones<<<nblk(A.nv), kT, 0, s>>>(A);
  } else if (nce > 0) {
    k_mark_contacts<<<nblk(nce), kT, 0, s>>>(A, C, nce);
  }
  k_mark_tris<<<nblk(A.nt), kT, 0, s>>>(A);
  g_launches += 2;
}

void launch_narrow(const Arena& A, const ContactBufs& C, int ccd, const double* xs, const double* vs,
                   double delta_override, int npairs, cudaStream_t s) {
  if (npairs <= 0) return;
  static int grid2 = 0;
  if (grid2 == 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid2 = 8 * (sms > 0 ? sms : 1);
  }
  prof_begin(PK_NARROW, s);
  cudaMemsetAsync(C.counters + 6, 0, 8 * sizeof(int), s);  // queue counts [6, 7], [10, 13]
  prof_begin(PK_NARROW_FILTER, s);
  k_narrow_filter<<<nblk(npairs), kT, 0, s>>>(A, C, ccd, delta_override, npairs);
  prof_end(PK_NARROW_FILTER, s);
  narrow_fp64_passes(A, C, ccd, xs, vs, delta_override, grid2, s);
  prof_end(PK_NARROW, s);
  g_launches += 3;
}

size_t cub_sort_bytes(int n) {
  size_t b1 = 0, b2 = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b1, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                  (int*)nullptr, (int*)nullptr, n);
  cub::DeviceScan::ExclusiveSum(nullptr, b2, (int*)nullptr, (int*)nullptr, n);
  return b1 > b2 ? b1 : b2;
}

void cub_sort_pairs(void* tmp, size_t bytes, const unsigned long long* kin, unsigned long long* kout, const int* vin,
                    int* vout, int n, cudaStream_t s) {
  cub::DeviceRadixSort::SortPairs(tmp, bytes, kin, kout, vin, vout, n, 0, 64, s);
  g_launches += 4;
}

void cub_sort_keys(void* tmp, size_t bytes, const unsigned long long* kin, unsigned long long* kout, int n,
                   cudaStream_t s) {
  cub::DeviceRadixSort::SortKeys(tmp, bytes, kin, kout, n, 0, 64, s);
  g_launches += 4;
}

void cub_exclusive_sum(void* tmp, size_t bytes, const int* in, int* out, int n, cudaStream_t s) {
  cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, n, s);
  g_launches += 2;
}

void sort_dedupe(const Arena& A, ContactBufs& C, int n, cudaStream_t s) {
  cudaMemsetAsync(C.ce_inst_lo, 0, sizeof(int) * (size_t)A.ni, s);
  cudaMemsetAsync(C.ce_inst_hi, 0, sizeof(int) * (size_t)A.ni, s);
  if (n <= 0) {
    cudaMemsetAsync(C.counters + 2, 0, sizeof(int), s);
    k_counts<<<nblk(A.ni), kT, 0, s>>>(A, C);
    g_launches++;
    return;
  }
  // lexicographic (k0, k1, k2, k3): stable sort by the low pair, then the high pair
  prof_begin(PK_SORT, s);
  k_keys_lo<<<nblk(n), kT, 0, s>>>(C, n);
  cub_sort_pairs(C.cub_tmp, C.cub_bytes, C.key_a, C.key_b, C.idx_a, C.idx_b, n, s);
  k_keys_hi<<<nblk(n), kT, 0, s>>>(C, n);
  cub_sort_pairs(C.cub_tmp, C.cub_bytes, C.key_a, C.key_b, C.idx_b, C.idx_a, n, s);
  k_gather_cand<<<nblk(n), kT, 0, s>>>(C, n);
  k_dedupe<<<nblk(n), kT, 0, s>>>(A, C, n);
  cub_exclusive_sum(C.cub_tmp, C.cub_bytes, C.idx_b, C.idx_a, n, s);
  k_compact<<<nblk(n), kT, 0, s>>>(A, C, n);
  k_segments<<<nblk(n), kT, 0, s>>>(A, C);
  k_counts<<<nblk(A.ni), kT, 0, s>>>(A, C);
  prof_end(PK_SORT, s);
  g_launches += 7;
}

void launch_impulses(const Arena& A, const ContactBufs& C, int ccd, const double* xs, double* vs, cudaStream_t s) {
  prof_begin(PK_IMPULSE, s);
  if (!ccd) {
    static int grid = 0;
    if (grid == 0) {
      int dev = 0, sms = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      grid = 4 * (sms > 0 ? sms : 1);
    }
    k_impulse_prep<<<grid, 128, 0, s>>>(A, C, xs);
    g_launches++;
  }
  k_token_next<<<1, 1, 0, s>>>(A);
  k_impulse_levels<<<nblk(A.ni * 32, 128), 128, 0, s>>>(A, C, ccd);
  if (A.impulse_cluster > 1) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(A.ni * A.impulse_cluster));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)A.impulse_cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    launch_check(cudaLaunchKernelEx(&cfg, k_impulse_apply_cluster, A, C, ccd, xs, vs), "cudaLaunchKernelEx");
  } else {
    k_impulse_apply<<<A.ni, 256, 0, s>>>(A, C, ccd, xs, vs);
  }
  prof_end(PK_IMPULSE, s);
  g_launches += 3;
}

namespace {
__device__ __forceinline__ V3<double> pt(const double* a, int k) { return V3<double>{a[3 * k], a[3 * k + 1], a[3 * k + 2]}; }

// DistanceFaceVertex (bvh_aabb.cpp:321-340) per item: face p0 p1 p2, vertex p3
__global__ void k_distance_fv(int n, const double* pts, double* dist, double* w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* a = pts + 12 * (size_t)i;
  double w0, w1;
  dist[i] = dist_face_vertex(pt(a, 0), pt(a, 1), pt(a, 2), pt(a, 3), w0, w1);
  w[2 * i] = w0;
  w[2 * i + 1] = w1;
}

// DistanceEdgeEdge (bvh_aabb.cpp:343-384) per item: edges p0 p1 and q0 q1
__global__ void k_distance_ee(int n, const double* pts, double* dist, double* ratio) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* a = pts + 12 * (size_t)i;
  double rp, rq;
  dist[i] = dist_edge_edge(pt(a, 0), pt(a, 1), pt(a, 2), pt(a, 3), rp, rq);
  ratio[2 * i] = rp;
  ratio[2 * i + 1] = rq;
}

// FindCoplanerInterp (bvh_aabb.cpp:598-662) per item: start and end points
__global__ void k_coplanar_time(int n, const double* s0, const double* e0, double* t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* a = s0 + 12 * (size_t)i;
  const double* b = e0 + 12 * (size_t)i;
  t[i] = coplanar_time(pt(a, 0), pt(a, 1), pt(a, 2), pt(a, 3), pt(b, 0), pt(b, 1), pt(b, 2), pt(b, 3));
}
}  // namespace

void launch_distance_fv(int n, const double* pts, double* dist, double* w, cudaStream_t s) {
  k_distance_fv<<<nblk(n), kT, 0, s>>>(n, pts, dist, w);
  g_launches++;
}

void launch_distance_ee(int n, const double* pts, double* dist, double* ratio, cudaStream_t s) {
  k_distance_ee<<<nblk(n), kT, 0, s>>>(n, pts, dist, ratio);
  g_launches++;
}

void launch_coplanar_time(int n, const double* s0, const double* e0, double* t, cudaStream_t s) {
  k_coplanar_time<<<nblk(n), kT, 0, s>>>(n, s0, e0, t);
  g_launches++;
}

void launch_riz_reset(const Arena& A, cudaStream_t s) {
  k_riz_reset<<<nblk(A.nv), kT, 0, s>>>(A);
  g_launches++;
}

void launch_riz_add(const Arena& A, const ContactBufs& C, int nce, cudaStream_t s) {
  if (nce > 0) {
    k_riz_contacts<<<nblk(nce), kT, 0, s>>>(A, C, nce);
    g_launches++;
  }
  if (A.ne > 0) {
    k_riz_edges<<<nblk(A.ne), kT, 0, s>>>(A);
    g_launches++;
  }
}

// rigid velocities of all zones of the active cloths; returns nothing, uses
// C.counters[4] as the member count
int riz_apply(const Arena& A, ContactBufs& C, const double* xs, double* vs, const double* v0s, cudaStream_t s) {
  int* cnt = C.counters + 4;
  cudaMemsetAsync(cnt, 0, sizeof(int), s);
  k_riz_collect<<<nblk(A.nv), kT, 0, s>>>(A, C, cnt);
  g_launches++;
  int n = 0;
  cudaMemcpyAsync(&n, cnt, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  if (n == 0) return 0;
  cub_sort_keys(C.cub_tmp, C.cub_bytes, C.zkey, C.zkey2, n, s);
  k_riz_stats<<<nblk(n), kT, 0, s>>>(A, C, n, xs, v0s);
  k_riz_velocity<<<nblk(n), kT, 0, s>>>(C, n, xs, vs);
  g_launches += 2;
  return n;
}

int riz_count_zones(const Arena& A, ContactBufs& C, int* zone_of, cudaStream_t s) {
  k_riz_labels<<<nblk(A.nv), kT, 0, s>>>(A, zone_of);
  g_launches++;
  (void)C;
  return 0;
}

void launch_riz_count(const Arena& A, cudaStream_t s) {
  k_riz_count<<<nblk(A.nv), kT, 0, s>>>(A);
  g_launches++;
}

// ---- graph frames: the pipeline with every count read on the device ---------------
// A frame captured in a CUDA graph cannot size launches from counts the host
// reads back.  These launchers use fixed grids and read the counts from device
// memory; the candidate and zone sorts run at fixed, padded sizes (pad keys sort
// last).  A count above a fixed capacity sets A.ctl->overflow, and the host then
// re-runs the frame on the host-driven path, which grows the buffers.
namespace {

constexpr int kDevGrid = 1216;  // 8 blocks of kT threads per SM of a GB300, unless the arena sets one
inline int dev_grid(const Arena& A) { return A.dev_grid > 0 ? A.dev_grid : kDevGrid; }

// gates of the kernels a loop body runs only on its first or later passes
__device__ __forceinline__ bool gate_open(const FrameCtl* c, int g) {
  switch (g) {
    case kGateCcdFirst: return c->ccd_pass == 0;
    case kGateCcdLater: return c->ccd_pass > 0;
    case kGateRizFirst: return c->riz_pass == 0;
    case kGateRizLater: return c->riz_pass > 0;
    default: return true;
  }
}

__global__ void k_traverse_gated(Arena A, ContactBufs C, int gate) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < A.nt && gate_open(A.ctl, gate)) traverse_tri(A, C, t);
}

__global__ void k_traverse_dirty_gated(Arena A, ContactBufs C, int gate) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < A.nt && gate_open(A.ctl, gate)) traverse_dirty_tri(A, C, t);
}

// candidates of the previous detection without a dirty triangle (count from the device)
__global__ void k_keep_clean_dev(Arena A, ContactBufs C, int gate) {
  if (!gate_open(A.ctl, gate)) return;
  const int n = min(A.ctl->last_ncand, C.cand_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const Cand c = C.cand[i];
    const int ta = A.node[3 * c.na + 1], tb = A.node[3 * c.nb + 1];
    if (A.tdirty[ta] || A.tdirty[tb] || !A.active[A.tinst[ta]]) continue;
    C.cand_sorted[atomicAdd(&C.counters[5], 1)] = c;
  }
}

// the kept candidates to the front of C.cand; the candidate count starts there
__global__ void k_kept_to_front(ContactBufs C) {
  const int n = __ldcg(&C.counters[5]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) C.cand[i] = C.cand_sorted[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) C.counters[1] = n;
}

__global__ void k_mark_contacts_dev(Arena A, ContactBufs C, int gate) {
  if (!gate_open(A.ctl, gate)) return;
  const int n = A.ctl->last_nce;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const int* e = C.ce + 5 * c;
    if (!A.active[A.vinst[e[1]]]) continue;
#pragma unroll
    for (int k = 1; k <= 4; k++) A.vdirty[e[k]] = 1;
  }
}

__global__ void k_mark_zones_gated(Arena A, int gate) {
  if (!gate_open(A.ctl, gate)) return;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= A.nv) return;
  if (A.active[A.vinst[v]] && A.inzone[v]) A.vdirty[v] = 1;
}

// padded sort of the candidates: n = candidate count (C.counters[8])
__global__ void k_sort_prep(Arena A, ContactBufs C, int S) {
  const int n = C.counters[1];
  const bool over = n > S || n > C.cand_cap;
  C.counters[8] = over ? 0 : n;
  C.counters[2] = 0;
  if (over) A.ctl->overflow |= kOverflowSort;
}

__global__ void k_keys_lo_pad(ContactBufs C, int S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S) return;
  C.key_a[i] = i < C.counters[8] ? key_lo(C.cand[i]) : ~0ull;
  C.idx_a[i] = i;
}

__global__ void k_keys_hi_pad(ContactBufs C, int S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S) return;
  C.key_a[i] = i < C.counters[8] ? key_hi(C.cand[C.idx_b[i]]) : ~0ull;
}

__global__ void k_gather_dev(ContactBufs C, int S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < S && i < C.counters[8]) C.cand_sorted[i] = C.cand[C.idx_a[i]];
}

__global__ void k_dedupe_dev(Arena A, ContactBufs C, int S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S) return;
  const int n = C.counters[8];
  if (i >= n) {
    C.idx_b[i] = 0;
    return;
  }
  const Cand ci = C.cand_sorted[i];
  const bool head = (i == 0) || !same_key(C.cand_sorted[i - 1], ci);
  C.idx_b[i] = head ? 1 : 0;
  if (!head) return;
  int j = i + 1;
  bool mixed = false;
  while (j < n && same_key(C.cand_sorted[j], ci)) {
    mixed |= (C.cand_sorted[j].fv != ci.fv);
    j++;
  }
  int win = i;
  if (mixed)
    for (int k = i + 1; k < j; k++)
      if (visited_before(A, C.cand_sorted[k], C.cand_sorted[win])) win = k;
  C.level[i] = C.cand_sorted[win].fv;
}

__global__ void k_compact_dev(ContactBufs C, int S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = C.counters[8];
  if (i >= S || i >= n) return;
  const int pos = C.idx_a[i];
  if (i == n - 1) C.counters[2] = pos + C.idx_b[i];
  if (!C.idx_b[i]) return;
  const Cand c = C.cand_sorted[i];
  C.ce[5 * pos + 0] = C.level[i];
  C.ce[5 * pos + 1] = c.k[0];
  C.ce[5 * pos + 2] = c.k[1];
  C.ce[5 * pos + 3] = c.k[2];
  C.ce[5 * pos + 4] = c.k[3];
}

// end of a detection: what the next incremental detection starts from, and the
// overflow flag of the broad and narrow phases
__global__ void k_detect_done(Arena A, ContactBufs C) {
  FrameCtl* c = A.ctl;
  if (C.counters[3]) c->overflow |= kOverflowBuffers;
  c->last_ncand = C.counters[8];
  c->last_nce = C.counters[2];
}

__global__ void k_riz_contacts_dev(Arena A, ContactBufs C) {
  const int n = A.ctl->last_nce;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const int* e = C.ce + 5 * c;
    if (!A.active[A.vinst[e[1]]]) continue;
#pragma unroll
    for (int k = 1; k <= 4; k++) A.inzone[e[k]] = 1;
    uf_union(A.uf, e[1], e[2]);
    uf_union(A.uf, e[1], e[3]);
    uf_union(A.uf, e[1], e[4]);
  }
}

// padded sort of the zone members: n = member count (C.counters[9])
__global__ void k_zone_prep(Arena A, ContactBufs C, int S) {
  const int n = C.counters[4];
  const bool over = n > S;
  if (over) A.ctl->overflow |= kOverflowZone;
  C.counters[9] = over ? 0 : n;
}

__global__ void k_zone_pad(ContactBufs C, int S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < S && i >= C.counters[9]) C.zkey[i] = ~0ull;
}

__global__ void k_riz_stats_dev(Arena A, ContactBufs C, int S, const double* xs, const double* v0s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < S && i < C.counters[9]) riz_stats_one(A, C, i, C.counters[9], xs, v0s);
}

__global__ void k_riz_velocity_dev(ContactBufs C, int S, const double* xs, double* vs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < S && i < C.counters[9]) riz_velocity_one(C, i, xs, vs);
}

}  // namespace

void launch_narrow_dev(const Arena& A, const ContactBufs& C, int ccd, const double* xs, const double* vs,
                       cudaStream_t s) {
  launch_check(cudaMemsetAsync(C.counters + 6, 0, 8 * sizeof(int), s), "cudaMemsetAsync");
  k_narrow_filter_dev<<<dev_grid(A), kT, 0, s>>>(A, C, ccd, -1.0);
  narrow_fp64_passes(A, C, ccd, xs, vs, -1.0, dev_grid(A), s);
  g_launches += 3;
}

void sort_dedupe_dev(const Arena& A, ContactBufs& C, int S, cudaStream_t s) {
  launch_check(cudaMemsetAsync(C.ce_inst_lo, 0, sizeof(int) * (size_t)A.ni, s), "cudaMemsetAsync");
  launch_check(cudaMemsetAsync(C.ce_inst_hi, 0, sizeof(int) * (size_t)A.ni, s), "cudaMemsetAsync");
  k_sort_prep<<<1, 1, 0, s>>>(A, C, S);
  k_keys_lo_pad<<<nblk(S), kT, 0, s>>>(C, S);
  cub_sort_pairs(C.cub_tmp, C.cub_bytes, C.key_a, C.key_b, C.idx_a, C.idx_b, S, s);
  k_keys_hi_pad<<<nblk(S), kT, 0, s>>>(C, S);
  cub_sort_pairs(C.cub_tmp, C.cub_bytes, C.key_a, C.key_b, C.idx_b, C.idx_a, S, s);
  k_gather_dev<<<nblk(S), kT, 0, s>>>(C, S);
  k_dedupe_dev<<<nblk(S), kT, 0, s>>>(A, C, S);
  cub_exclusive_sum(C.cub_tmp, C.cub_bytes, C.idx_b, C.idx_a, S, s);
  k_compact_dev<<<nblk(S), kT, 0, s>>>(C, S);
  k_segments<<<nblk(S), kT, 0, s>>>(A, C);
  k_counts<<<nblk(A.ni), kT, 0, s>>>(A, C);
  k_detect_done<<<1, 1, 0, s>>>(A, C);
  g_launches += 10;
}

void detect_dev(const Arena& A, ContactBufs& C, int ccd, int gate_full, int gate_incr, int S, const double* xs,
                const double* vs, cudaStream_t s) {
  launch_refit(A, ccd, xs, vs, -1.0, s);
  launch_check(cudaMemsetAsync(C.counters, 0, 4 * sizeof(int), s), "cudaMemsetAsync");
  launch_check(cudaMemsetAsync(C.counters + 5, 0, sizeof(int), s), "cudaMemsetAsync");
  if (gate_incr >= 0) {
    k_keep_clean_dev<<<dev_grid(A), kT, 0, s>>>(A, C, gate_incr);
    k_kept_to_front<<<dev_grid(A), kT, 0, s>>>(C);
    k_traverse_dirty_gated<<<nblk(A.nt), kT, 0, s>>>(A, C, gate_incr);
    g_launches += 3;
  }
  if (gate_full >= 0) {
    k_traverse_gated<<<nblk(A.nt), kT, 0, s>>>(A, C, gate_full);
    g_launches++;
  }
  launch_narrow_dev(A, C, ccd, xs, vs, s);
  sort_dedupe_dev(A, C, S, s);
}

void mark_dirty_dev(const Arena& A, const ContactBufs& C, int gate_contacts, int gate_zones, cudaStream_t s) {
  launch_check(cudaMemsetAsync(A.vdirty, 0, sizeof(int) * (size_t)A.nv, s), "cudaMemsetAsync");
  if (gate_zones >= 0) {
    k_mark_zones_gated<<<nblk(A.nv), kT, 0, s>>>(A, gate_zones);
    g_launches++;
  }
  k_mark_contacts_dev<<<dev_grid(A), kT, 0, s>>>(A, C, gate_contacts);
  k_mark_tris<<<nblk(A.nt), kT, 0, s>>>(A);
  g_launches += 2;
}

void riz_add_dev(const Arena& A, const ContactBufs& C, cudaStream_t s) {
  k_riz_contacts_dev<<<dev_grid(A), kT, 0, s>>>(A, C);
  g_launches++;
  if (A.ne > 0) {
    k_riz_edges<<<nblk(A.ne), kT, 0, s>>>(A);
    g_launches++;
  }
}

void riz_apply_dev(const Arena& A, ContactBufs& C, int S, const double* xs, double* vs, const double* v0s,
                   cudaStream_t s) {
  int* cnt = C.counters + 4;
  launch_check(cudaMemsetAsync(cnt, 0, sizeof(int), s), "cudaMemsetAsync");
  k_riz_collect<<<nblk(A.nv), kT, 0, s>>>(A, C, cnt);
  k_zone_prep<<<1, 1, 0, s>>>(A, C, S);
  k_zone_pad<<<nblk(S), kT, 0, s>>>(C, S);
  cub_sort_keys(C.cub_tmp, C.cub_bytes, C.zkey, C.zkey2, S, s);
  k_riz_stats_dev<<<nblk(S), kT, 0, s>>>(A, C, S, xs, v0s);
  k_riz_velocity_dev<<<nblk(S), kT, 0, s>>>(C, S, xs, vs);
  g_launches += 5;
}

}  // namespace cs
