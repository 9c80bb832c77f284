// kernels.h -- host launchers of the device kernels (one translation unit each
// for assembly, solvers and collision).
#pragma once
#include <atomic>
#include <stdexcept>
#include <string>

#include "arena.h"
#include "prof.h"

namespace cs {

// Leaf pairs one triangle's broad-phase walk may emit before its cloth is taken
// as blown up.  Normal frames stay far below: a few tens per triangle, a few
// hundred in deep folds or with fast incoherent motion.  A blown-up cloth is
// normally caught first by its speed (kMaxSpeed); this limit bounds the pair
// buffers when it is not.
constexpr int kMaxPairsPerTriangle = 4096;
// A velocity component above this (m/s) after the implicit step also marks the
// cloth as blown up (no cloth frame of the reference's scenes comes near it).
constexpr double kMaxSpeed = 1.0e3;

// a failed CUDA call (the C ABI reports it as CS_ERR_CUDA, or CS_ERR_OOM)
struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};
inline void launch_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// launches issued by this process (all contexts), for launch accounting
extern std::atomic<long long> g_launches;

// --- assembly (k_assemble.cu) ---------------------------------------------
void launch_quad_factors(const Arena& A, cudaStream_t s);
// element gradients (and Hessian blocks when hess) at positions A.x; masked:
// only cloths with A.active set
void launch_elements(const Arena& A, bool hess, bool masked, cudaStream_t s);
void launch_slot_reduce(const Arena& A, cudaStream_t s);
void launch_rhs(const Arena& A, cudaStream_t s);
void launch_update_velocity(const Arena& A, cudaStream_t s);  // masked
void launch_finish_implicit(const Arena& A, cudaStream_t s);  // x += dx, v = dx/dt
// MakeNormal for the active cloths at positions xs into out (3 per vertex)
void launch_vertex_normals(const Arena& A, const double* xs, double* out, cudaStream_t s);
void launch_reintegrate(const Arena& A, cudaStream_t s);      // masked: x = x1 + v dt
void launch_element_batch_cst(int n, const double* C, const double* c, double lambda, double myu, double* W,
                              double* dW, double* ddW, cudaStream_t s);
void launch_element_batch_bend(int n, const double* C, const double* c, double stiff, double* W, double* dW,
                               double* ddW, cudaStream_t s);
void launch_element_batch_contact(int n, const double* c, const DevParams* prm, double* W, double* dW,
                                  double* ddW, cudaStream_t s);

// --- solvers (k_solve.cu) --------------------------------------------------
// block ILU(0) of the ILU cloths in list (device array of cloth ids); masked:
// only those with A.active set
void launch_ilu_factor(const Arena& A, const int* list, int n, cudaStream_t s, bool masked = false);
// PCG on A.b -> A.dx for the cloths in list (tol / maxit < 0: take the cloth's)
void launch_pcg(const Arena& A, const int* list, int n, double tol, int maxit, cudaStream_t s, bool masked = false);
// CG building blocks on all cloths with A.active set
void launch_cg_init(const Arena& A, double tol, int maxit, cudaStream_t s);
// it < 0: the iteration number is A.ctl->cycle (a graph frame)
void launch_cg_iteration(const Arena& A, int it, double tol, int maxit, bool serial, cudaStream_t s);
void launch_spmv(const Arena& A, const double* x, double* y, cudaStream_t s);
// y = beta y + alpha A x over the rows [v0, v1) (MatVec's operation order)
void launch_matvec(const Arena& A, int v0, int v1, double alpha, const double* x, double beta, double* y,
                   cudaStream_t s);
// (LU)^-1 z in place with the last ILU(0) factor of cloth slot inst
void launch_ilu_solve(const Arena& A, int inst, double* z, cudaStream_t s);

// --- mixed precision (k_mixed.cu) ----------------------------------------------
void launch_mx_outer_init(const Arena& A, cudaStream_t s);
void launch_mx_inner_init(const Arena& A, cudaStream_t s);
// dx = dt v and r = b - A dx (FP64) for the active, unconverged cloths
void launch_mx_warm_start(const Arena& A, cudaStream_t s);
void launch_mx_inner_iteration(const Arena& A, int it, float eta, int cap, cudaStream_t s);
// the whole inner FP32 CG of one refinement cycle (up to cap iterations) in one
// cooperative launch; blocks_per_sm <= 0 picks the occupancy limit
// threads per block: 256, 512 or 1024; tail_slices > 0: once fewer slices
// than that are still iterating, a second launch with one warp per slice
// finishes the solve (0: one launch)
void launch_mx_inner_persistent(const Arena& A, float eta, int cap, int blocks_per_sm, int threads, int tail_slices,
                                cudaStream_t s);
void launch_mx_refine(const Arena& A, double tol, int maxcycles, cudaStream_t s);

// --- collision (k_collide.cu) ------------------------------------------------
// refit boxes of the active cloths from positions xs (and velocities vs when ccd)
void launch_refit(const Arena& A, int ccd, const double* xs, const double* vs, double delta_override,
                  cudaStream_t s);
void launch_traverse(const Arena& A, const ContactBufs& C, cudaStream_t s);
// incremental CCD detection: keeps the candidates of pairs whose six vertices
// kept their velocity (moved to the front of C.cand, count in C.counters[1]) and
// lists every overlapping leaf pair with a dirty triangle
void launch_keep_clean_candidates(const Arena& A, ContactBufs& C, int ncand, cudaStream_t s);
void launch_traverse_dirty(const Arena& A, const ContactBufs& C, cudaStream_t s);
// dirty marks: the vertices of the current contact list (after impulses) or the
// zone vertices (after an impact-zone pass); then per triangle
void launch_mark_dirty(const Arena& A, const ContactBufs& C, int nce, bool zones, cudaStream_t s);
void launch_narrow(const Arena& A, const ContactBufs& C, int ccd, const double* xs, const double* vs,
                   double delta_override, int npairs, cudaStream_t s);
// sort + deduplicate ncand candidates into C.ce; returns via C.counters[2]
void sort_dedupe(const Arena& A, ContactBufs& C, int ncand, cudaStream_t s);
// impulse sweep of the active cloths' contact lists (level stamps from A.ctl->token)
void launch_impulses(const Arena& A, const ContactBufs& C, int ccd, const double* xs, double* vs, cudaStream_t s);
void launch_riz_reset(const Arena& A, cudaStream_t s);
// counts the in-zone vertices of each active cloth into st.riz_nodes
void launch_riz_count(const Arena& A, cudaStream_t s);
void launch_riz_add(const Arena& A, const ContactBufs& C, int nce, cudaStream_t s);
// zone rigid velocities: v of zone members from snapshot v0 at positions xs
// returns the number of zone members
int riz_apply(const Arena& A, ContactBufs& C, const double* xs, double* vs, const double* v0s, cudaStream_t s);
int riz_count_zones(const Arena& A, ContactBufs& C, int* zone_of_vertex_dev, cudaStream_t s);

// geometry on batches (bvh_aabb.cpp:321-384, 598-662), 12 doubles of points per item
void launch_distance_fv(int n, const double* pts, double* dist, double* w, cudaStream_t s);
void launch_distance_ee(int n, const double* pts, double* dist, double* ratio, cudaStream_t s);
void launch_coplanar_time(int n, const double* s0, const double* e0, double* t, cudaStream_t s);

// ---- graph frames (k_collide.cu): counts read on the device, fixed launch sizes ----
// gates: 0 always, 1 / 2 first / later CCD pass, 3 / 4 first / later impact-zone pass;
// a negative gate leaves the kernel out
enum GraphGate { kGateAlways = 0, kGateCcdFirst = 1, kGateCcdLater = 2, kGateRizFirst = 3, kGateRizLater = 4 };
void launch_narrow_dev(const Arena& A, const ContactBufs& C, int ccd, const double* xs, const double* vs,
                       cudaStream_t s);
// sorts and deduplicates C.counters[1] candidates at the padded size S
void sort_dedupe_dev(const Arena& A, ContactBufs& C, int S, cudaStream_t s);
// a detection: refit, incremental part (keep clean candidates, dirty traversal)
// under gate_incr, full traversal under gate_full, narrow phase, sort
void detect_dev(const Arena& A, ContactBufs& C, int ccd, int gate_full, int gate_incr, int S, const double* xs,
                const double* vs, cudaStream_t s);
void mark_dirty_dev(const Arena& A, const ContactBufs& C, int gate_contacts, int gate_zones, cudaStream_t s);
void riz_add_dev(const Arena& A, const ContactBufs& C, cudaStream_t s);
void riz_apply_dev(const Arena& A, ContactBufs& C, int S, const double* xs, double* vs, const double* v0s,
                   cudaStream_t s);

size_t cub_sort_bytes(int n);
void cub_sort_pairs(void* tmp, size_t bytes, const unsigned long long* kin, unsigned long long* kout,
                    const int* vin, int* vout, int n, cudaStream_t s);
void cub_sort_keys(void* tmp, size_t bytes, const unsigned long long* kin, unsigned long long* kout, int n,
                   cudaStream_t s);
size_t cub_scan_bytes(int n);
void cub_exclusive_sum(void* tmp, size_t bytes, const int* in, int* out, int n, cudaStream_t s);

}  // namespace cs
