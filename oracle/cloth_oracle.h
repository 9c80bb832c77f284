/*
 * cloth_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (plain C, FP64, IEEE, no FMA contraction) of the reference's
 * self_contact_sparse step: FEM cloth element energies, 3x3 block-sparse
 * assembly, block ILU(0) + PCG / CG, BVH build + refit + self-collision
 * culling, proximity / CCD impulses, rigid impact zones and the frame glue.
 *
 * It exists only as the checker for the CUDA library: tests/, the smoke()
 * entry point and bench.py's CPU-baseline leg may load it.  The product path
 * never links or calls it.  It is pinned against the reference itself: the
 * companion driver oracle/ref_driver.cpp compiles the reference sources in
 * place and the golden fixtures under tests/golden/ were produced by it.
 *
 * Every function in cloth_oracle.c cites the reference file:line it restates.
 */
#ifndef CLOTH_ORACLE_H
#define CLOTH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Obstacle kinds (the reference passes a host function pointer
 * `penetrationDepth`, self_contact_sparse/main.cpp:110-133). */
enum {
  CO_OBSTACLE_NONE = 0,
  CO_OBSTACLE_PLANE_Z = 1,       /* pd = obs_center[2] - z, n = (0,0,1)      */
  CO_OBSTACLE_SPHERE_SOLID = 2,  /* pd = r - |p-c|, n = (p-c)/|p-c|          */
  CO_OBSTACLE_SPHERE_HOLLOW = 3  /* the reference demo's inside-out sphere   */
};

/* Linear solver used by the implicit step. */
enum {
  CO_SOLVER_ILU_PCG = 0, /* StepTime_InternalDynamicsILU, solve_internal_sparse.h:255 */
  CO_SOLVER_CG = 1       /* StepTime_InternalDynamics,    solve_internal_sparse.h:185 */
};

/* Simulation parameters; the same layout is used by the CUDA library's
 * cs_params (include/clothgpu.h). */
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
  int flags; /* ignored: the oracle always sums inner products serially, like the reference */
} co_params;

/* Per-frame counters, filled by co_step / co_resolve. */
typedef struct {
  int solver_iterations;
  int n_prx;            /* proximity contacts                               */
  int n_ccd_passes;     /* CCD detections run (1..5)                        */
  int n_ccd[5];         /* contacts per CCD detection                       */
  int n_riz_passes;     /* RIZ detections run (0..100)                      */
  int n_riz_last;       /* contacts in the last RIZ detection               */
  int n_riz_total;      /* contacts summed over RIZ detections              */
  int riz_nodes;        /* vertices in impact zones at the end              */
  int impulse_applied;
  int ilu_singular;     /* singular pivots met by the ILU factorisation     */
  double solver_conv;   /* relative residual reported by the solver         */
} co_stats;

/* ---- element level (cloth_internal_physics.h) ---------------------------- */
void co_wdwddw_cst(const double C[9], const double c[9], double lambda, double myu,
                   double *W, double dW[9], double ddW[81]);
void co_wdwddw_bend(const double C[12], const double c[12], double stiff,
                    double *W, double dW[12], double ddW[144]);
void co_wdwddw_contact(const double c[3], const co_params *prm,
                       double *W, double dW[3], double ddW[9]);

/* ---- a simulated cloth --------------------------------------------------- */
typedef struct co_cloth co_cloth;

co_cloth *co_create(int np, const double *X0, const int *bc, int nt, const int *tri,
                    int nq, const int *quad, const co_params *prm);
void co_destroy(co_cloth *h);
void co_set_params(co_cloth *h, const co_params *prm);

int co_num_blocks(const co_cloth *h);          /* off-diagonal 3x3 blocks B  */
void co_pattern(const co_cloth *h, int *row_ptr, int *col_idx);
int co_num_nodes(const co_cloth *h);           /* BVH nodes 2T-1             */
void co_bvh_nodes(const co_cloth *h, int *nodes); /* 3 ints: parent, child0, child1 */
int co_num_edges(const co_cloth *h);           /* 1-ring adjacency entries   */
void co_edges(const co_cloth *h, int *index, int *array);

/* implicit step pieces */
void co_assemble(co_cloth *h, const double *x, const double *v,
                 double *vdia, double *vcrs, double *b);
int co_ilu(co_cloth *h, double *fdia, double *fcrs);  /* after co_assemble; returns singular count */
void co_pcg(co_cloth *h, const double *b, double tol, int maxit, double *x,
            double *conv, int *iter);                 /* after co_ilu */
void co_cg(co_cloth *h, const double *b, double tol, int maxit, double *x,
           double *conv, int *iter);                  /* after co_assemble */
void co_implicit(co_cloth *h, double *x, double *v, co_stats *st);
void co_last_residual(const co_cloth *h, double *r);   /* r_vec after co_cg / co_pcg */
void co_ilu_solve(const co_cloth *h, double *vec);     /* after co_ilu */
void co_matvec(const co_cloth *h, double alpha, const double *x, double beta, double *y); /* after co_assemble */
/* geometry on 12 doubles of points (face p0 p1 p2 + vertex p3; edges p0 p1, q0 q1) */
double co_distance_fv(const double *p, double *w);
double co_distance_ee(const double *p, double *r);
double co_coplanar_time(const double *s, const double *e);
/* IsContact_FV_CCD / IsContact_EE_CCD on n configurations of 24 doubles each
 * (start points, then end points: face p0 p1 p2 and vertex p3, or edges p0 p1
 * and q0 q1), with the distinct indices 0..3; the face-vertex test takes the box
 * (lo[3], hi[3]) for its node; results (0 or 1) into out */
void co_fv_ccd_batch(int n, const double *p, const double *box, int *out);
void co_ee_ccd_batch(int n, const double *p, int *out);

/* collision pieces */
void co_refit_prx(co_cloth *h, const double *x, double delta, double *boxes);
void co_refit_ccd(co_cloth *h, const double *x, const double *v, double dt, double *boxes);
int co_contacts_prx(co_cloth *h, const double *x, double delta, int *out, int cap);
int co_contacts_ccd(co_cloth *h, const double *x, const double *v, double dt, double delta,
                    int *out, int cap);
void co_impulse_prx(co_cloth *h, const double *x, double *v, const int *ce, int n);
void co_impulse_ccd(co_cloth *h, const double *x, double *v, const int *ce, int n);
void co_riz_reset(co_cloth *h);
void co_riz_add(co_cloth *h, const int *ce, int n);
int co_riz_zones(const co_cloth *h, int *zone_of_vertex);
void co_riz_apply(co_cloth *h, const double *x, double *v, const double *v0);
void co_resolve(co_cloth *h, const double *x1, double *v, co_stats *st);
void co_update_velocity(co_cloth *h, const double *x, double *v);
/* MakeNormal (self_contact_sparse/main.cpp:183-211): unit vertex normals */
void co_vertex_normals(const co_cloth *h, const double *x, double *nrm);

/* Contact log: with logging on, co_resolve (and so co_step) records one entry
 * per detection it runs, in order: kind (0 proximity, 1 swept/CCD), contact
 * count and co_contact_digest of the ordered list (5 ints a contact: is_fv,
 * then the canonical key).  co_contact_log clears the log. */
unsigned long long co_contact_digest(const int *ce, int n);
void co_contact_log(co_cloth *h, int enable);
int co_contact_log_read(const co_cloth *h, int *kind, int *count, unsigned long long *digest, int cap);

/* one frame of self_contact_sparse/main.cpp StepTime, in place on x, v */
void co_step(co_cloth *h, double *x, double *v, co_stats *st);

#ifdef __cplusplus
}
#endif
#endif
