// arena.h -- device arena shared by all kernels: every cloth of a context is
// packed into one set of arrays with global vertex / triangle / stencil /
// block / node indices (a block-diagonal system of independent cloths).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "geom.cuh"

namespace cs {

// same layout as cs_params (include/clothgpu.h)
struct DevParams {
  double dt, lambda, myu, stiff_bend;
  double gravity[3];
  double mass_point, stiff_contact, contact_clearance;
  double obs_center[3];
  double obs_radius, tol;
  int obstacle_kind, solver_kind, maxit, flags;
};

// contact element as produced by the narrow phase
struct Cand {
  int k[4];     // canonical key (global vertex ids)
  int fv;       // 1 face-vertex, 0 edge-edge
  int na, nb;   // leaf nodes of the pair, na on the child-0 side of their common ancestor
  int test;     // index of the elementary test within the pair (0..14)
};

// per-cloth control block kept on the device
struct InstState {
  int nlev;          // impulse levels of the current contact list
  int n_contacts;    // contacts of the last detection
  int impulse_applied;
  int riz_nodes;
  int solver_iterations;
  int ilu_singular;
  int done;          // solver converged
  int diverged;      // a triangle's broad phase exceeded kMaxPairsPerTriangle: the cloth stops
  double solver_conv;
  double sq[2];      // CG: r.r of the previous / current iteration (by parity)
  double inv0;
  double rpr;        // PCG: r.Pr
  double dot[2];     // CG with serial inner products: p.Ap, r.r of this iteration
  // mixed precision: inner FP32 solve state
  double rz[2];      // r.z of the previous / current inner iteration (by parity)
  double rr_in0;     // r.r at the start of the inner solve
  int idone;         // inner solve finished
  int inner_iters;   // inner iterations of the current inner solve
  int total_iters;   // inner iterations summed over refinement cycles
  int cycles;        // refinement cycles
  double red[3];     // per-cloth totals of the slice partials: p.q, r.z, r.r
  // persistent inner solve (single-reduction CG): gamma = r.r of the current
  // iteration and alpha (FP64 copies for the recurrence); istop is set at the
  // end of an iteration when the cloth converges (no block reads it before the
  // barrier that follows); alpha and beta as the cloth's last block left them
  double gam, alf;
  int istop;
  int bjac;          // the inner solve runs on the block-Jacobi-scaled matrix
  float alpha32, beta32;
  // frame control on the device (a frame captured in a CUDA graph): the cloth
  // takes part in this frame (want), is still in the contact loop of
  // GetIntermidiateVelocityContactResolved (phase), got an impulse (applied);
  // and the frame's contact counters (cs_stats)
  int want, phase, applied;
  int st_prx, st_ccd[5], st_ccd_passes, st_riz_passes, st_riz_last, st_riz_total, st_riz_nodes;
};

// Device-side state of a frame captured in a CUDA graph.  The loops of
// GetIntermidiateVelocityContactResolved (self_collision_cloth.cpp:398-455:
// up to 5 CCD passes, up to 100 impact-zone passes) and of the solvers run as
// conditional graph nodes whose conditions kernels set from these counters.
// reasons a graph frame is re-run host-driven (FrameCtl::overflow bits)
constexpr int kOverflowSort = 1;     // candidates beyond the padded sort size
constexpr int kOverflowZone = 2;     // impact-zone members beyond the padded sort size
constexpr int kOverflowBuffers = 4;  // leaf pairs, test queues or candidates beyond their buffers
constexpr int kOverflowSolver = 8;   // refinement cycles beyond the graph's cap, or a barrier gave up

struct FrameCtl {
  int ccd_pass;     // CCD passes run in this frame
  int riz_pass;     // impact-zone passes run
  int cycle;        // refinement cycles (mixed) / CG iterations (FP64)
  int overflow;     // a fixed size was outgrown (the host re-runs the frame): bits kOverflow*
  int last_ncand;   // candidates of the last detection (kept for the incremental one)
  int last_nce;     // contacts of the last detection
  int token;        // stamp of the impulse level schedule (host and graph frames share it)
  int pad;
};

struct Arena {
  int ni = 0, nv = 0, nt = 0, nq = 0, nb = 0, nn = 0, ne = 0, nchunk = 0;
  // per cloth
  int* active = nullptr;  // takes part in the current pass
  int *voff = nullptr, *toff = nullptr, *qoff = nullptr, *boff = nullptr, *noff = nullptr;
  int *chunk_lo = nullptr, *chunk_hi = nullptr;  // row chunks of each cloth for the CG reductions
  DevParams* prm = nullptr;
  InstState* st = nullptr;
  // vertices
  double *x = nullptr, *v = nullptr, *x1 = nullptr, *X0 = nullptr, *v0 = nullptr;
  int *bc = nullptr, *vinst = nullptr;
  // elements
  int *tri = nullptr, *tinst = nullptr, *quad = nullptr, *qinst = nullptr;
  double *qK = nullptr, *qscale = nullptr;
  double *tri_blk = nullptr, *tri_grad = nullptr, *quad_grad = nullptr;
  // matrix (3x3 blocks, row-major), global rows
  int *row_ptr = nullptr, *col_idx = nullptr, *dia_split = nullptr, *blk_row = nullptr;
  int *slot_ptr = nullptr, *slot_src = nullptr, *grad_ptr = nullptr, *grad_src = nullptr;
  double *vdia = nullptr, *vcrs = nullptr, *fdia = nullptr, *fcrs = nullptr;
  // solver vectors (3 per vertex)
  double *b = nullptr, *r = nullptr, *p = nullptr, *z = nullptr, *dx = nullptr;
  double *part = nullptr;  // per-chunk partial sums
  int* chunk_inst = nullptr;
  // ILU(0) schedule: per cloth offsets into level tables
  int *lev_off = nullptr, *lev_ptr = nullptr, *lev_rows = nullptr;
  int *blev_off = nullptr, *blev_ptr = nullptr, *blev_rows = nullptr;
  int *fac_ptr = nullptr, *fac_ops = nullptr, *sing = nullptr;
  // BVH (global node ids; a leaf's child0 is a global triangle id)
  int *node = nullptr, *pre = nullptr, *skip = nullptr, *leaf_lo = nullptr, *leaf_hi = nullptr;
  int *depth = nullptr, *prepos = nullptr, *tri_leaf = nullptr, *refit_cnt = nullptr, *preoff = nullptr;
  Box* box = nullptr;
  // FP32 copies rounded outward (they contain the FP64 boxes): 6 floats per node
  // (lo xyz, hi xyz; an empty box is lo = +inf, hi = -inf) and per vertex (the
  // point, or its swept box for CCD), for conservative prefilters
  float* box32 = nullptr;
  float* vb32 = nullptr;
  // impact zones
  int *edge_uv = nullptr, *uf = nullptr, *inzone = nullptr;
  // incremental CCD re-detection: vertices / triangles whose velocity changed
  // since the last detection
  int *vdirty = nullptr, *tdirty = nullptr;
  // per vertex, for the continuous-collision certificates of a detection: the
  // start position and the displacement over the frame as FP32 hi/lo parts
  // (cert.cuh PS, three float4)
  float4* ccd32 = nullptr;
  // mixed precision: FP32 copy of the matrix in warp slices (SELL-32: 32 rows per
  // slice, blocks of a slice stored entry-major so every load is 32 consecutive
  // floats), block-Jacobi inverse, FP32 work vectors
  int nslice = 0;
  int *slice_inst = nullptr, *slice_row0 = nullptr, *slice_w = nullptr, *slice_lo = nullptr, *slice_hi = nullptr;
  long long* slice_voff = nullptr;  // float offset of the slice's values
  long long* slice_coff = nullptr;  // int offset of the slice's column indices
  long long* sell_pos = nullptr;    // per slot (off-diagonal then diagonal): value offset of entry 0
  float* val32 = nullptr;
  int* col32 = nullptr;
  // block-Jacobi scaling: L^-1 of the Cholesky factor of each diagonal block
  // (lower triangular, 9 per vertex; identity where the block is not positive
  // definite).  Cloths that use it have their FP32 matrix scaled once per frame
  // to S A S^T (S = blockdiag(L^-1)), on which CG is block-Jacobi PCG.
  float* linv32 = nullptr;
  float *r32 = nullptr, *d32 = nullptr, *p32 = nullptr, *q32 = nullptr, *z32 = nullptr;
  // single-reduction CG of the persistent solve: residual, A * residual and
  // A * direction, each double-buffered by iteration parity
  float *r32b = nullptr, *w32 = nullptr, *w32b = nullptr, *s32 = nullptr, *s32b = nullptr;
  double* part32 = nullptr;         // 3 per slice: inner-product partials
  int* red_cnt = nullptr;           // per cloth: slices that have written their partials
  // algorithmic bytes of one SpMV over a slice / chunk (real blocks, column
  // indices, x once, y once) and their running totals while profiling
  long long* slice_bytes = nullptr;
  long long* chunk_bytes = nullptr;
  unsigned long long* bytes_acc = nullptr;  // [0] FP32 SpMV, [1] FP64 SpMV, [2..5] narrow-phase
                                            // tests reaching FP64: FV prx, EE prx, FV ccd, EE ccd
  int count_bytes = 0;
  int mixed = 0;                    // mixed-precision arrays present
  // persistent inner solve: per-slice algorithmic bytes of one iteration and
  // the grid barrier state
  long long* slice_pbytes = nullptr;
  // per cloth: smallest and largest diagonal entry of the assembled matrix (as
  // the bits of positive floats) for the choice of preconditioner
  unsigned* dg_range = nullptr;
  unsigned int* grid_bar = nullptr; // [0] arrivals, [1] generation, [2] gave up, [3] cloths still iterating,
                                    // [4] last iteration of a launch that left for the tail launch
  FrameCtl* ctl = nullptr;          // frame control on the device
  int dev_grid = 0;                 // blocks of the grid-stride narrow-phase kernels of a graph frame
  int narrow_regs = 0;              // 128: FP64 narrow-phase kernels capped at 128 registers
  int bar_sleep_ns = 256;           // pause between polls of a waiting grid barrier
  int impulse_cluster = 1;          // blocks (one cluster) sweeping a cloth's impulse levels
  float mx_eta_big = 1.0e-4f;       // FP32 inner tolerance of large cloths (mixed solve)
  long long bar_timeout_ns = 2000000000;  // a waiting grid barrier gives up after this long
  int bar_hold = 0;                 // test hook: block 0 never arrives at the grid barrier
};

// scratch for the contact pipeline (grown on demand)
struct ContactBufs {
  int pair_cap = 0, cand_cap = 0, ce_cap = 0;
  int2* pairs = nullptr;
  // elementary tests that passed the FP32 prefilters, waiting for their FP64
  // test, as (pair index, test index): face-vertex [0] and edge-edge [1]
  int q_cap[2] = {0, 0};
  int2* queue[2] = {nullptr, nullptr};
  // continuous-collision tests the certificates' whole-motion stage kept for
  // their piece stage (face-vertex, edge-edge; counts in counters[10, 11]);
  // the tests the piece stage leaves to the FP64 test go back into queue[]
  // (counts in counters[12, 13])
  int2* queue64[2] = {nullptr, nullptr};
  Cand* cand = nullptr;
  Cand* cand_sorted = nullptr;
  unsigned long long *key_a = nullptr, *key_b = nullptr;
  int *idx_a = nullptr, *idx_b = nullptr;
  int* ce = nullptr;          // 5 ints per contact, sorted, deduplicated
  int* ce_inst_lo = nullptr;  // per cloth segment of ce
  int* ce_inst_hi = nullptr;
  int* counters = nullptr;    // [0] pairs, [1] candidates, [2] contacts, [3] overflow flag,
                              // [4] zone members, [5] kept candidates, [6] / [7] face-vertex /
                              // edge-edge tests queued, [8] / [9] sorted candidates / zone
                              // members of a graph frame, [10] / [11] CCD tests kept for the
                              // certificates' piece stage, [12] / [13] CCD tests left to FP64
  int* level = nullptr;       // impulse level per contact
  int* order = nullptr;       // contacts grouped by level
  double* imp_pre = nullptr;  // per contact: position-only terms of the proximity impulse (9)
  int* lev_cnt = nullptr;     // per cloth: level count (then offsets)
  int* vmark = nullptr;       // per vertex: last level touching it (stamped)
  int* vstamp = nullptr;
  int* zone_list = nullptr;   // in-zone vertices
  unsigned long long* zkey = nullptr;
  unsigned long long* zkey2 = nullptr;
  double* zrec = nullptr;     // per vertex: zone record at its root (gc, av, omega)
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0;
};

}  // namespace cs
