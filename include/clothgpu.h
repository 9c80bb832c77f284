/*
 * clothgpu.h -- C ABI of the GB300 (sm_103a) implementation of the
 * self_contact_sparse cloth step (implicit-Euler FEM cloth with
 * self-collision), from the reference nobuyuki83/cloth_sim_self_collision.
 *
 * Plain C: opaque context handle, plain pointers and sizes, int status codes.
 * Host arrays use the reference's layouts: positions / velocities as 3 doubles
 * per vertex (std::vector<double> aXYZ / aUVW), triangles as 3 ints, bending
 * stencils as 4 ints (aTri / aQuad), 3x3 blocks row-major.
 *
 * One context owns one CUDA device, one stream and a device arena holding any
 * number of cloth instances ("cloths").  A cloth's topology is built once when
 * it is added; its state (x, v) stays resident on the device between steps.
 *
 * Each entry point names the reference interface it replaces (file:line in the
 * reference repository).
 */
#ifndef CLOTHGPU_H
#define CLOTHGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define CS_OK 0
#define CS_ERR_ARG 1          /* bad argument (null pointer, bad id, size)         */
#define CS_ERR_CUDA 2         /* a CUDA call failed; see cs_last_error              */
#define CS_ERR_NO_DEVICE 3    /* no usable GPU                                       */
#define CS_ERR_OOM 4          /* device allocation failed                            */
#define CS_ERR_CAPACITY 5     /* a caller-supplied output buffer is too small        */
#define CS_ERR_TIMEOUT 6      /* a bounded device wait gave up                        */
#define CS_ERR_DIVERGED 7     /* a cloth blew up (a speed above 1000 m/s after its implicit
                                 step, or more than 4096 overlapping leaf pairs for one
                                 triangle); it is no longer stepped                    */

/* precision of the implicit solve */
#define CS_PREC_FP64 0        /* plain: FP64 throughout, bit-exact with the reference */
#define CS_PREC_MIXED 1       /* FP64 elements and assembly; FP32 SpMV/CG inside FP64
                                 iterative refinement; collision in FP64               */

/* obstacle kinds (replace the penetrationDepth callback,
 * self_contact_sparse/main.cpp:110-133) */
#define CS_OBSTACLE_NONE 0
#define CS_OBSTACLE_PLANE_Z 1      /* pd = obs_center[2] - z, n = (0,0,1)              */
#define CS_OBSTACLE_SPHERE_SOLID 2 /* pd = r - |p-c|, n = (p-c)/|p-c|                   */
#define CS_OBSTACLE_SPHERE_HOLLOW 3 /* the reference demo's inside-out sphere          */

/* linear solver of the implicit step */
#define CS_SOLVER_ILU_PCG 0   /* Solve_PCG with block ILU(0), ilu_sparse.cpp:628     */
#define CS_SOLVER_CG 1        /* Solve_CG, matrix_square_sparse.cpp:338              */

/* cs_params.flags */
#define CS_FLAG_EXACT_DOTS 1  /* Krylov inner products as one running sum in dof order, like the
                                 reference's InnerProduct (matrix_square_sparse.cpp:313): the FP64
                                 path then reproduces the reference bit for bit, at the cost of a
                                 serial sum per inner product.  Off: deterministic tree sums. */

/* Parameters of one cloth: the arguments of StepTime_InternalDynamicsILU
 * (solve_internal_sparse.h:255-275) and GetIntermidiateVelocityContactResolved
 * (self_collision_cloth.h:21-34), plus the solver tolerance and cap that the
 * reference hard-codes (solve_internal_sparse.h:318-319). */
typedef struct {
  double dt;
  double lambda;
  double myu;
  double stiff_bend;
  double gravity[3];
  double mass_point;
  double stiff_contact;
  double contact_clearance;
  double obs_center[3];
  double obs_radius;
  double tol;
  int obstacle_kind;
  int solver_kind;
  int maxit;
  int flags; /* CS_FLAG_* */
} cs_params;

/* Per-frame counters of one cloth (the reference prints these,
 * solve_internal_sparse.h:321, self_collision_cloth.cpp:386-450). */
typedef struct {
  int solver_iterations;
  int n_prx;
  int n_ccd_passes;
  int n_ccd[5];
  int n_riz_passes;
  int n_riz_last;
  int n_riz_total;
  int riz_nodes;
  int impulse_applied;
  int ilu_singular;
  double solver_conv;
  int diverged;             /* 1 once the cloth blew up (see CS_ERR_DIVERGED)          */
} cs_stats;

typedef struct cs_ctx cs_ctx;

/* ---- host-only topology (no device needed) --------------------------------- */
/* MakeBVHTopology_TopDown (bvh_aabb.cpp:294-313): nodes[3 nnode] = parent,
 * child0, child1 (CNodeBVH, bvh_aabb.h:18-23); node 0 is the root.  *nnode is
 * always set; CS_ERR_CAPACITY when 3 * nnode > cap. */
int cs_build_bvh(int np, const double *X, int nt, const int *tri, int *nodes, int cap, int *nnode);
/* Block pattern of the implicit matrix from the bending stencils, rows sorted
 * (CJaggedArray::SetEdgeOfElem + Sort + SetPattern, self_contact_sparse/main.cpp:578-581):
 * row_ptr[np+1], col_idx[nb]; CS_ERR_CAPACITY when nb > cap. */
int cs_build_pattern(int np, int nq, const int *quad, int *row_ptr, int *col_idx, int cap, int *nb);

/* ---- context --------------------------------------------------------------- */
int cs_create(int device, int precision, cs_ctx **out);
void cs_destroy(cs_ctx *ctx);
const char *cs_last_error(const cs_ctx *ctx);
int cs_set_precision(cs_ctx *ctx, int precision);
int cs_synchronize(cs_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for recording events around calls. */
void *cs_stream(const cs_ctx *ctx);

/* ---- cloths ---------------------------------------------------------------- */
/* Adds a cloth: builds its topology on the host (matrix pattern as in
 * self_contact_sparse/main.cpp:578-581, BVH as MakeBVHTopology_TopDown
 * bvh_aabb.cpp:294, 1-ring as CJaggedArray::SetEdgeOfElem jagged_array.h:158)
 * and uploads it.  State starts at x = X0, v = 0. */
int cs_add_cloth(cs_ctx *ctx, int np, const double *X0, const int *bc, int nt, const int *tri, int nq,
                 const int *quad, const cs_params *prm, int *id_out);
int cs_remove_cloth(cs_ctx *ctx, int id);
int cs_num_cloths(const cs_ctx *ctx);
int cs_set_params(cs_ctx *ctx, int id, const cs_params *prm);
int cs_set_state(cs_ctx *ctx, int id, const double *x, const double *v);
int cs_get_state(cs_ctx *ctx, int id, double *x, double *v);
int cs_get_stats(cs_ctx *ctx, int id, cs_stats *st);

/* ---- whole frames -------------------------------------------------------------
 * StepTime, self_contact_sparse/main.cpp:213-263: implicit step, contact
 * resolution from the start-of-frame positions, re-integration and velocity
 * update, for every cloth of the context, nsteps times. */
int cs_step(cs_ctx *ctx, int nsteps);

/* ---- stages of one cloth, host buffers in and out ------------------------------ */
/* StepTime_InternalDynamicsILU / StepTime_InternalDynamics
 * (solve_internal_sparse.h:255-326 / :185-253): x, v in place. */
int cs_implicit_step(cs_ctx *ctx, int id, double *x, double *v, cs_stats *st);
/* GetIntermidiateVelocityContactResolved, self_collision_cloth.cpp:355-456:
 * v in place, from start-of-frame positions x1. */
int cs_resolve_contacts(cs_ctx *ctx, int id, const double *x1, double *v, cs_stats *st);
/* UpdateIntermidiateVelocity, solve_internal_sparse.h:329-369 */
int cs_update_velocity(cs_ctx *ctx, int id, const double *x, double *v);

/* Assembly half of StepTime_InternalDynamicsILU (solve_internal_sparse.h:276-313):
 * the 3x3 block matrix (diagonal blocks vdia[9 np], off-diagonal vcrs[9 nb] in the
 * pattern's order) and right-hand side b[3 np] at state (x, v).  Any output may be null. */
int cs_assemble(cs_ctx *ctx, int id, const double *x, const double *v, double *vdia, double *vcrs,
                double *b);
/* Block pattern of a cloth: nb and, when non-null, row_ptr[np+1], col_idx[nb]
 * (CMatrixSquareSparse m_colInd / m_rowPtr, matrix_square_sparse.h:40-43). */
int cs_pattern(cs_ctx *ctx, int id, int *nb, int *row_ptr, int *col_idx);
/* CPreconditionerILU::SetValueILU + DoILUDecomp (ilu_sparse.cpp:352-624) on the
 * last assembled matrix; factor blocks out (nullable) and the singular-pivot count. */
int cs_ilu_factor(cs_ctx *ctx, int id, double *fdia, double *fcrs, int *nsing);
/* Solve_PCG (ilu_sparse.cpp:628-709) on the last assembled matrix and factor. */
int cs_solve_pcg(cs_ctx *ctx, int id, const double *b, double tol, int maxit, double *x, double *conv,
                 int *iter);
/* Solve_CG (matrix_square_sparse.cpp:338-406) on the last assembled matrix. */
int cs_solve_cg(cs_ctx *ctx, int id, const double *b, double tol, int maxit, double *x, double *conv,
                int *iter);
/* The residual vector of the cloth's last cs_solve_cg / cs_solve_pcg: the r_vec
 * that Solve_CG / Solve_PCG leave behind (matrix_square_sparse.cpp:338-406,
 * ilu_sparse.cpp:628-709). */
int cs_last_residual(cs_ctx *ctx, int id, double *r);
/* CMatrixSquareSparse::MatVec(1, x, 0, y) (matrix_square_sparse.cpp:167-270) */
int cs_spmv(cs_ctx *ctx, int id, const double *x, double *y);
/* CMatrixSquareSparse::MatVec(alpha, x, beta, y) (matrix_square_sparse.cpp:167-270):
 * y = beta y + alpha A x, y in place, in the reference's operation order. */
int cs_matvec(cs_ctx *ctx, int id, double alpha, const double *x, double beta, double *y);
/* Replaces the cloth's device matrix by caller values (diagonal blocks vdia[9 np],
 * off-diagonal vcrs[9 nb] in the pattern's order; either may be null to keep it):
 * the matrix a CMatrixSquareSparse holds after Mearge / SetBoundaryCondition
 * (matrix_square_sparse.cpp:88-138, 272-302), for the MatVec, Solve_CG,
 * DoILUDecomp and Solve_PCG entries above.  The next frame assembles anew. */
int cs_set_matrix(cs_ctx *ctx, int id, const double *vdia, const double *vcrs);
/* CPreconditionerILU::Solve (ilu_sparse.h:23-26: ForwardSubstitution then
 * BackwardSubstitution, ilu_sparse.cpp:136-350): vec <- (LU)^-1 vec in place
 * with the cloth's last factor (cs_ilu_factor). */
int cs_ilu_solve(cs_ctx *ctx, int id, double *vec);

/* BVH of a cloth: nnode and, when non-null, nodes[3 nnode] = parent, child0,
 * child1 (CNodeBVH, bvh_aabb.h:18-23; child1 == -1 marks a leaf). */
int cs_bvh_nodes(cs_ctx *ctx, int id, int *nnode, int *nodes);
/* BuildBoundingBoxChild_Prx / _CCD (bvh_aabb.cpp:23-106): boxes[7 nnode] =
 * xmin, xmax, ymin, ymax, zmin, zmax, non-empty flag.  boxes may be null. */
int cs_refit_prx(cs_ctx *ctx, int id, const double *x, double delta, double *boxes);
int cs_refit_ccd(cs_ctx *ctx, int id, const double *x, const double *v, double dt, double *boxes);
/* GetContactElement_Proximity / _CCD (bvh_aabb.cpp:441-557, 797-923) after the
 * matching refit: contacts in std::set order, 5 ints each (is_fv, ino0..ino3),
 * up to cap; *n receives the full count (CS_ERR_CAPACITY if it exceeds cap). */
int cs_contacts_prx(cs_ctx *ctx, int id, const double *x, double delta, int *out, int cap, int *n);
int cs_contacts_ccd(cs_ctx *ctx, int id, const double *x, const double *v, double dt, double delta,
                    int *out, int cap, int *n);
/* SelfCollisionImpulse_Proximity / _CCD (self_collision_cloth.cpp:20-212):
 * sequential-order impulses over a contact list, v in place. */
int cs_impulse_prx(cs_ctx *ctx, int id, const double *x, double *v, const int *ce, int n);
int cs_impulse_ccd(cs_ctx *ctx, int id, const double *x, double *v, const int *ce, int n);
/* MakeRigidImpactZone / ApplyRigidImpactZone (self_collision_cloth.cpp:220-348):
 * reset the zones, add contacts, read zone ids per vertex (-1 outside; ids are
 * an arbitrary labelling of the same partition), apply the rigid velocities. */
int cs_riz_reset(cs_ctx *ctx, int id);
int cs_riz_add(cs_ctx *ctx, int id, const int *ce, int n);
int cs_riz_zones(cs_ctx *ctx, int id, int *zone_of_vertex, int *nzone);
int cs_riz_apply(cs_ctx *ctx, int id, const double *x, double *v, const double *v0);

/* Boxes of a cloth's BVH from the last refit (the aBB output of
 * GetIntermidiateVelocityContactResolved, self_collision_cloth.h:33): 7 doubles
 * per node as in cs_refit_prx. */
int cs_get_boxes(cs_ctx *ctx, int id, double *boxes);

/* ---- element kernels on batches (cloth_internal_physics.h) --------------------- */
/* WdWddW_CST (:70-176) for n triangles: C, c [n][9]; W[n], dW[n][9], ddW[n][81] */
int cs_element_cst(cs_ctx *ctx, int n, const double *C, const double *c, double lambda, double myu,
                   double *W, double *dW, double *ddW);
/* WdWddW_Bend (:180-238) for n stencils: C, c [n][12]; W[n], dW[n][12], ddW[n][144] */
int cs_element_bend(cs_ctx *ctx, int n, const double *C, const double *c, double stiff, double *W,
                    double *dW, double *ddW);
/* WdWddW_Contact (:243-280) for n points against the obstacle of prm */
int cs_element_contact(cs_ctx *ctx, int n, const double *c, const cs_params *prm, double *W, double *dW,
                       double *ddW);

/* ---- geometry on batches (bvh_aabb.h:50-61), on the device ---------------------- */
/* DistanceFaceVertex (bvh_aabb.cpp:321-340) for n items: pts[n][12] = face p0 p1 p2
 * and vertex p3; dist[n], w[n][2] = the weights of p0 and p1. */
int cs_distance_fv(cs_ctx *ctx, int n, const double *pts, double *dist, double *w);
/* DistanceEdgeEdge (bvh_aabb.cpp:343-384): pts[n][12] = p0 p1 q0 q1; dist[n],
 * ratio[n][2] = ratio_p, ratio_q. */
int cs_distance_ee(cs_ctx *ctx, int n, const double *pts, double *dist, double *ratio);
/* FindCoplanerInterp (bvh_aabb.cpp:598-662): start points s[n][12], end points
 * e[n][12]; t[n] = first coplanarity time in [0, 1], or -1. */
int cs_coplanar_time(cs_ctx *ctx, int n, const double *s, const double *e, double *t);

/* ---- whole-arena state I/O ------------------------------------------------------ */
/* States of every cloth in the order they were added (x and v of 3 doubles per
 * vertex each, cloths back to back): one copy each way for the whole arena.  Either
 * pointer may be null. */
int cs_set_states(cs_ctx *ctx, const double *x, const double *v);
int cs_get_states(cs_ctx *ctx, double *x, double *v);
/* MakeNormal (self_contact_sparse/main.cpp:183-211, the demo's render normals)
 * into a device-side buffer copied to `normals` (3 doubles per vertex): for
 * cloth `id` at positions x (null: its current state), or, with id = -1 and
 * x = null, for every cloth of the context in the order of cs_get_states, in
 * one launch.  Bit-exact with the reference's loop. */
int cs_vertex_normals(cs_ctx *ctx, int id, const double *x, double *normals);
/* Total vertices of the context (length of the state arrays / 3). */
long long cs_num_vertices(const cs_ctx *ctx);

/* ---- serving: continuous batching of scenes on one GPU ---------------------------- */
/* No counterpart in the reference (its driver steps one cloth in a GLUT loop).  A
 * server owns one context whose arena holds every admitted scene; a worker thread
 * advances all unfinished scenes together, one StepTime frame per loop, while scenes
 * that arrive are packed into the next arena by a builder thread and swapped in at a
 * frame boundary (their positions and velocities stay on the device).  Admission is
 * first come, first served by estimated device bytes: the arena being stepped plus
 * the one being packed stay within hbm_budget_bytes.  A scene computes the same
 * frames alone and in a mix (every reduction, sort and schedule is per cloth). */
typedef struct cs_server cs_server;

typedef struct cs_server_config {
  int device;               /* CUDA device ordinal                                   */
  int precision;            /* CS_PREC_FP64 or CS_PREC_MIXED                         */
  double hbm_budget_bytes;  /* admission limit on estimated device bytes             */
  int max_cloths;           /* limit on scenes per arena, 0 for none                 */
} cs_server_config;

typedef struct cs_request_info {
  int np, nsteps, steps_done;
  int status;               /* CS_OK, or the error that ended the request            */
  double t_submit, t_admit, t_first_frame, t_done;  /* seconds since cs_server_create */
  double step_ms_p50, step_ms_p99;                   /* frames the scene took part in */
} cs_request_info;

typedef struct cs_server_stats {
  long long frames, vertex_steps;
  int submitted, finished, queued, resident, rebuilds;
  int diverged;                              /* requests ended by CS_ERR_DIVERGED        */
  double elapsed_s, busy_s;                  /* since creation; inside frames           */
  double step_ms_p50, step_ms_p99, step_ms_max;  /* over (scene, frame) samples        */
  double admit_ms_p50, admit_ms_p99;         /* submission to first frame               */
  double build_ms_total;                     /* packing new arenas, overlapped with frames */
  double install_ms_total;                   /* frame-boundary swaps                    */
  double arena_bytes, peak_bytes;            /* estimated device bytes                  */
} cs_server_stats;

int cs_server_create(const cs_server_config *cfg, cs_server **out);
/* Queues a scene (mesh as in cs_add_cloth; x, v: initial state, null for X0 and
 * rest) for nsteps frames.  Builds its host topology on the calling thread and
 * returns at once; CS_ERR_CAPACITY if the scene alone exceeds the budget.
 * Thread-safe. */
int cs_server_submit(cs_server *srv, int np, const double *X0, const int *bc, int nt, const int *tri,
                     int nq, const int *quad, const double *x, const double *v, const cs_params *prm,
                     int nsteps, int *req);
/* Waits (timeout_s < 0: without limit; CS_ERR_TIMEOUT when it runs out) until the
 * request has run its frames, then copies its final state (x, v may be null).
 * Returns the request's status. */
int cs_server_wait(cs_server *srv, int req, double timeout_s, double *x, double *v, cs_request_info *info);
/* Frees the host copy of a finished request's final state. */
int cs_server_release(cs_server *srv, int req);
/* Waits until every submitted request has finished. */
int cs_server_drain(cs_server *srv, double timeout_s);
int cs_server_get_stats(cs_server *srv, cs_server_stats *st);
const char *cs_server_last_error(cs_server *srv);
/* Stops the worker after its current frame; unfinished requests are dropped. */
void cs_server_destroy(cs_server *srv);
/* The admission estimate of a scene's device bytes (0 for invalid arguments). */
size_t cs_scene_device_bytes(int np, const double *X0, int nt, const int *tri, int nq, const int *quad,
                             const cs_params *prm);

/* ---- a solve that allocates nothing ---------------------------------------------- */
/* Maximum block rows (vertices) accepted by cs_solve_cg_noalloc. */
#define CS_NOALLOC_MAX_VERTICES 16384
/* No counterpart in the reference: Solve_CG (matrix_square_sparse.cpp:338-406
 * semantics) for callers that cannot allocate device memory, such as an engine
 * that owns all device memory through its own pool, or a real-time loop that
 * must not enter the CUDA allocator.  The caller passes the 3x3 block system in
 * device memory (row_ptr[np+1], col_idx[nb], vcrs[9 nb], vdia[9 np], b[3 np])
 * and the device output x[3 np]; conv and iter are host outputs.  No
 * allocation is made: the work vectors live in one fixed file-scope device array
 * sized for CS_NOALLOC_MAX_VERTICES rows (about 1.2 MB), which every GPU that
 * loads the library holds until the process exits.  Larger systems return
 * CS_ERR_CAPACITY.  The first call on a device looks up that array's device
 * address; make that first call before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race, so serialise them.  Runs on
 * `stream` (a cudaStream_t, null for the default stream); every call copies conv
 * and iter to the host and waits for the stream before it returns. */
int cs_solve_cg_noalloc(const int *row_ptr, const int *col_idx, const double *vcrs, const double *vdia,
                        const double *b, double *x, int np, double tol, int maxit, double *conv, int *iter,
                        void *stream);

/* ---- frame graph ------------------------------------------------------------------ */
/* How cs_step runs a frame.  CS_FRAME_GRAPH (the default): one launch of a
 * CUDA graph captured for the context's cloths, whose loops (refinement cycles
 * or CG iterations, up to 5 CCD passes and up to 100 impact-zone passes of
 * GetIntermidiateVelocityContactResolved, self_collision_cloth.cpp:398-455)
 * are conditional graph nodes decided on the device; the host reads the
 * frame's counters once at its end.  Contact buffers and sorts have fixed sizes
 * in a graph: a frame that outgrows them is restored to its start and re-run
 * host-driven, which grows them, and the graph is captured again.
 * CS_FRAME_HOST: every frame host-driven (the host reads counters after each
 * detection and solver cycle).  Both give the same frames bit for bit.  Frames
 * run host-driven while per-kernel profiling or the contact log is on. */
#define CS_FRAME_HOST 0
#define CS_FRAME_GRAPH 1
int cs_set_frame_mode(cs_ctx *ctx, int mode);
/* Frames run as a graph and host-driven, graph captures, and graph frames that
 * outgrew a fixed size (each then re-run host-driven); any pointer may be null. */
int cs_frame_counts(cs_ctx *ctx, long long *graph_frames, long long *host_frames, long long *captures,
                    long long *overflows);
/* The graph frames re-run host-driven, by reason (a frame may count under
 * several): reasons[0] candidates beyond the graph's padded sort size,
 * [1] impact-zone members beyond its padded sort size, [2] leaf pairs, test
 * queues or candidates beyond the contact buffers (which the host-driven frame
 * then grows), [3] refinement cycles beyond the graph's cap. */
int cs_frame_overflows(cs_ctx *ctx, long long reasons[4]);

/* ---- autotuning of launch shapes ----------------------------------------------------- */
/* No counterpart in the reference.  Times `frames` frames from the current state
 * for candidate launch shapes (coordinate descent over the persistent solver's
 * blocks per SM, the slice count below which it continues in a smaller tail
 * launch, the blocks per SM of the narrow-phase kernels of graph frames,
 * whether the FP64 narrow-phase kernels are capped at 128 registers, the
 * pause between polls of the persistent solver's grid barrier, and the blocks
 * per cloth of the impulse sweep),
 * restoring the state after each, and keeps the fastest.  The frames do not
 * depend on these shapes, so the simulation continues exactly where it was.
 * Results are cached per arena shape (cloths, vertices, slices, precision) for
 * the life of the process: a later call on the same shape only applies them. */
typedef struct cs_tune_result {
  int mx_blocks_per_sm;   /* persistent solver: blocks of 256 threads per SM    */
  int mx_tail_slices;     /* persistent solver: tail launch threshold (0: none)  */
  int graph_grid_per_sm;  /* graph frames: narrow-phase blocks per SM           */
  int narrow_regs;        /* FP64 narrow-phase kernels: 0 free, 128 capped       */
  int bar_sleep_ns;       /* persistent solver: pause between barrier polls (ns) */
  int impulse_cluster;    /* impulse sweep: blocks per cloth (1, or a cluster of 8) */
  double frame_ms;        /* measured time of a frame with these shapes         */
  int candidates;         /* configurations timed                               */
  int cached;             /* 1: taken from an earlier call on the same shape    */
} cs_tune_result;
int cs_autotune(cs_ctx *ctx, int frames, cs_tune_result *out);

/* ---- contact log ------------------------------------------------------------------ */
/* Test facility, off by default: with logging on, every contact resolution
 * (GetIntermidiateVelocityContactResolved, self_collision_cloth.cpp:355-456, in
 * cs_step or cs_resolve_contacts) records, for each cloth it resolves, one entry
 * per detection it runs, in order: kind (0 proximity, 1 swept), the contact count
 * and a digest of the ordered contact list (FNV-1a 64 over its 32-bit words, 5 per
 * contact: is_fv and the canonical key in cloth-local ids).  The log of a cloth
 * holds its last resolution.  Enabling or disabling clears it.  Each logged
 * detection copies the contact lists to the host, so frames run slower. */
int cs_contact_log(cs_ctx *ctx, int enable);
/* The log of cloth `id`: *n entries, up to cap written (CS_ERR_CAPACITY beyond). */
int cs_contact_log_read(cs_ctx *ctx, int id, int *kind, int *count, unsigned long long *digest, int cap,
                        int *n);

/* ---- counters ------------------------------------------------------------------ */
/* Kernel launches issued by this context since creation (for launch accounting). */
long long cs_launch_count(const cs_ctx *ctx);
/* Device timing of kernel classes with CUDA events recorded on the context's
 * stream around each launch: enable (1) / disable (0) and clear the totals; read
 * the total milliseconds and launch count of one class ("cg_spmv", "traverse",
 * "narrow", "refit", "tri_elements", "slot_reduce", "rhs", "ilu_factor", "pcg",
 * "cg_update", "cg_direction", "impulse"). */
int cs_profile(cs_ctx *ctx, int enable);
int cs_profile_read(cs_ctx *ctx, const char *kernel, double *total_ms, long long *launches);
/* Algorithmic bytes moved by the SpMV kernels since profiling was enabled
 * (blocks, column indices, x and y once per processed row; converged cloths
 * excluded): the FP32 inner SpMV and the FP64 CG SpMV. */
int cs_profile_bytes(cs_ctx *ctx, long long *spmv32, long long *spmv64);

#ifdef __cplusplus
}
#endif
#endif
