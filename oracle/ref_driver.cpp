// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A headless driver around the reference's own sources, compiled in place by
// oracle/Makefile (target `ref`) into oracle/_ref/libclothref.so.  It exposes
// the same C entry points as the oracle restatement (cloth_oracle.h) with the
// prefix `ref_` so tests can compare the two function by function, and so the
// fixture script tests/golden/make_golden.py can record golden vectors.
//
// Everything numeric here is the reference's code: this file only owns the
// objects the reference's GLUT driver keeps as globals
// (self_contact_sparse/main.cpp:137-177), restates its init sequence
// (main.cpp:563-583) and its StepTime glue (main.cpp:213-263), and maps the
// obstacle descriptor onto a penetration-depth callback.  Console output of the
// reference is captured and parsed for contact counters.
#include <cstring>
#include <sstream>
#include <string>
#include <vector>
#include <set>
#include <iostream>

#include "solve_internal_sparse.h"
#include "self_collision_cloth.h"
#include "jagged_array.h"
#include "bvh_aabb.h"

#include "cloth_oracle.h"

// Non-static functions of self_collision_cloth.cpp that its header does not declare.
void SelfCollisionImpulse_Proximity(std::vector<double>& aUVWm, double delta, double stiffness,
                                    double dt, double mass, const std::vector<double>& aXYZ,
                                    const std::vector<int>& aTri,
                                    const std::vector<CContactElement>& aContactElem);
void SelfCollisionImpulse_CCD(std::vector<double>& aUVWm, double delta, double stiffness,
                              double dt, double mass, const std::vector<double>& aXYZ,
                              const std::vector<int>& aTri,
                              const std::vector<CContactElement>& aContactElem);
bool IsContact_FV_CCD(int ino0, int ino1, int ino2, int ino3, const CVector3D& p0, const CVector3D& p1,
                      const CVector3D& p2, const CVector3D& p3, const CVector3D& q0, const CVector3D& q1,
                      const CVector3D& q2, const CVector3D& q3, const CAABB3D& bb);
bool IsContact_EE_CCD(int ino0, int ino1, int jno0, int jno1, const CVector3D& p0s, const CVector3D& p1s,
                      const CVector3D& q0s, const CVector3D& q1s, const CVector3D& p0e, const CVector3D& p1e,
                      const CVector3D& q0e, const CVector3D& q1e);
void MakeRigidImpactZone(std::vector<std::set<int> >& aRIZ,
                         const std::vector<CContactElement>& aContactElem,
                         const CJaggedArray& aEdge);
void ApplyRigidImpactZone(std::vector<double>& aUVWm, const std::vector<std::set<int> >& aRIZ,
                          const std::vector<double>& aXYZ, const std::vector<double>& aUVWm0);

namespace {

co_params g_obstacle;  // the callback below cannot capture

// Penetration-depth callbacks with the reference's signature
// (self_contact_sparse/main.cpp:110-133).
void pd_none(double& pd, double* n, const double* p) {
  (void)p;
  n[0] = 0; n[1] = 0; n[2] = 1;
  pd = -1.0e300;
}
void pd_plane(double& pd, double* n, const double* p) {
  n[0] = 0.0; n[1] = 0.0; n[2] = 1.0;
  pd = g_obstacle.obs_center[2] - p[2];
}
void pd_sphere_solid(double& pd, double* n, const double* p) {
  const double* c = g_obstacle.obs_center;
  n[0] = p[0] - c[0];
  n[1] = p[1] - c[1];
  n[2] = p[2] - c[2];
  const double len = Length3D(n);
  n[0] /= len;
  n[1] /= len;
  n[2] /= len;
  pd = g_obstacle.obs_radius - len;
}
void pd_sphere_hollow(double& pd, double* n, const double* p) {
  const double* c = g_obstacle.obs_center;
  n[0] = p[0] - c[0];
  n[1] = p[1] - c[1];
  n[2] = p[2] - c[2];
  const double len = Length3D(n);
  n[0] /= len;
  n[1] /= len;
  n[2] /= len;
  pd = g_obstacle.obs_radius - len;
  n[0] *= -1;
  n[1] *= -1;
  n[2] *= -1;
  pd *= -1;
}

typedef void (*pd_fn)(double&, double*, const double*);
pd_fn obstacle_fn(const co_params& p) {
  g_obstacle = p;
  switch (p.obstacle_kind) {
    case CO_OBSTACLE_PLANE_Z: return pd_plane;
    case CO_OBSTACLE_SPHERE_SOLID: return pd_sphere_solid;
    case CO_OBSTACLE_SPHERE_HOLLOW: return pd_sphere_hollow;
    default: return pd_none;
  }
}

struct RefCloth {
  co_params prm;
  std::vector<double> aXYZ0;
  std::vector<int> aBCFlag, aTri, aQuad;
  CMatrixSquareSparse mat_A;
  CPreconditionerILU* ilu_A;
  std::vector<CNodeBVH> aNodeBVH;
  std::vector<CAABB3D> aBB;
  int iroot_bvh;
  CJaggedArray aEdge;
  std::vector<std::set<int> > aRIZ;
  std::vector<double> vec_b;  // rhs of the last assembly
  std::vector<double> r_last; // r_vec of the last Solve_CG / Solve_PCG
};

std::vector<CContactElement> to_elems(const int* ce, int n) {
  std::vector<CContactElement> v;
  v.reserve(n);
  for (int i = 0; i < n; i++) {
    // the constructor re-canonicalises; keys from a set are canonical already
    CContactElement e(ce[i * 5] != 0, ce[i * 5 + 1], ce[i * 5 + 2], ce[i * 5 + 3], ce[i * 5 + 4]);
    v.push_back(e);
  }
  return v;
}

int from_set(const std::set<CContactElement>& s, int* out, int cap) {
  int n = 0;
  for (std::set<CContactElement>::const_iterator it = s.begin(); it != s.end(); ++it, ++n) {
    if (n < cap) {
      out[n * 5 + 0] = it->is_fv ? 1 : 0;
      out[n * 5 + 1] = it->ino0;
      out[n * 5 + 2] = it->ino1;
      out[n * 5 + 3] = it->ino2;
      out[n * 5 + 4] = it->ino3;
    }
  }
  return n;
}

void export_boxes(const std::vector<CAABB3D>& bb, double* boxes) {
  for (size_t i = 0; i < bb.size(); i++) {
    boxes[i * 7 + 0] = bb[i].x_min; boxes[i * 7 + 1] = bb[i].x_max;
    boxes[i * 7 + 2] = bb[i].y_min; boxes[i * 7 + 3] = bb[i].y_max;
    boxes[i * 7 + 4] = bb[i].z_min; boxes[i * 7 + 5] = bb[i].z_max;
    boxes[i * 7 + 6] = bb[i].isnt_empty ? 1.0 : 0.0;
  }
}

// Parses the counters the reference prints in GetIntermidiateVelocityContactResolved
// (self_collision_cloth.cpp:386, 415, 448).
void parse_resolve_log(const std::string& log, co_stats* st) {
  std::istringstream is(log);
  std::string line;
  while (std::getline(is, line)) {
    size_t p;
    if ((p = line.find("Proximity")) != std::string::npos) {
      size_t q = line.find("Size:");
      st->n_prx = atoi(line.c_str() + q + 5);
    } else if ((p = line.find("CCD iter:")) != std::string::npos) {
      int it = atoi(line.c_str() + p + 9);
      size_t q = line.find("Size:");
      if (it < 5) st->n_ccd[it] = atoi(line.c_str() + q + 5);
      st->n_ccd_passes = it + 1;
    } else if ((p = line.find("RIZ iter:")) != std::string::npos) {
      size_t q = line.find("Size:");
      size_t r = line.find("RIZ:", q);
      int cnt = atoi(line.c_str() + q + 5);
      st->n_riz_passes += 1;
      st->n_riz_last = cnt;
      st->n_riz_total += cnt;
      st->riz_nodes = atoi(line.c_str() + r + 4);
    }
  }
}

}  // namespace

extern "C" {

void ref_wdwddw_cst(const double C[9], const double c[9], double lambda, double myu, double* W,
                    double dW[9], double ddW[81]) {
  double w = 0;
  WdWddW_CST(w, (double(*)[3])dW, (double(*)[3][3][3])ddW, (const double(*)[3])C,
             (const double(*)[3])c, lambda, myu);
  *W = w;
}

void ref_wdwddw_bend(const double C[12], const double c[12], double stiff, double* W, double dW[12],
                     double ddW[144]) {
  double w = 0;  // the reference accumulates into W without clearing it
  WdWddW_Bend(w, (double(*)[3])dW, (double(*)[4][3][3])ddW, (const double(*)[3])C,
              (const double(*)[3])c, stiff);
  *W = w;
}

void ref_wdwddw_contact(const double c[3], const co_params* prm, double* W, double dW[3],
                        double ddW[9]) {
  double w = 0;
  WdWddW_Contact(w, dW, (double(*)[3])ddW, c, prm->stiff_contact, prm->contact_clearance,
                 obstacle_fn(*prm));
  *W = w;
}

void* ref_create(int np, const double* X0, const int* bc, int nt, const int* tri, int nq,
                 const int* quad, const co_params* prm) {
  RefCloth* h = new RefCloth();
  h->prm = *prm;
  h->aXYZ0.assign(X0, X0 + 3 * np);
  h->aBCFlag.assign(bc, bc + np);
  h->aTri.assign(tri, tri + 3 * nt);
  h->aQuad.assign(quad, quad + 4 * nq);
  // init sequence of self_contact_sparse/main.cpp:576-582
  h->iroot_bvh = MakeBVHTopology_TopDown(h->aTri, h->aXYZ0, h->aNodeBVH);
  h->aEdge.SetEdgeOfElem(h->aTri, (int)h->aTri.size() / 3, 3, np, false);
  h->mat_A.Initialize(np, 3);
  CJaggedArray crs;
  crs.SetEdgeOfElem(h->aQuad, (int)h->aQuad.size() / 4, 4, np, false);
  crs.Sort();
  h->mat_A.SetPattern(crs.index, crs.array);
  h->ilu_A = new CPreconditionerILU();
  h->ilu_A->m_diaInd = 0;  // the constructor leaves it unset
  h->ilu_A->Initialize_ILU0(h->mat_A);
  return h;
}

void ref_destroy(void* p) {
  RefCloth* h = (RefCloth*)p;
  delete h->ilu_A;
  delete h;
}

void ref_set_params(void* p, const co_params* prm) { ((RefCloth*)p)->prm = *prm; }

int ref_num_blocks(void* p) { return ((RefCloth*)p)->mat_A.m_ncrs; }

void ref_pattern(void* p, int* row_ptr, int* col_idx) {
  RefCloth* h = (RefCloth*)p;
  for (int i = 0; i <= h->mat_A.m_nblk; i++) row_ptr[i] = h->mat_A.m_colInd[i];
  for (int i = 0; i < h->mat_A.m_ncrs; i++) col_idx[i] = h->mat_A.m_rowPtr[i];
}

int ref_num_nodes(void* p) { return (int)((RefCloth*)p)->aNodeBVH.size(); }

void ref_bvh_nodes(void* p, int* nodes) {
  RefCloth* h = (RefCloth*)p;
  for (size_t i = 0; i < h->aNodeBVH.size(); i++) {
    nodes[i * 3 + 0] = h->aNodeBVH[i].iroot;
    nodes[i * 3 + 1] = h->aNodeBVH[i].ichild[0];
    nodes[i * 3 + 2] = h->aNodeBVH[i].ichild[1];
  }
}

int ref_num_edges(void* p) { return (int)((RefCloth*)p)->aEdge.array.size(); }

void ref_edges(void* p, int* index, int* array) {
  RefCloth* h = (RefCloth*)p;
  for (size_t i = 0; i < h->aEdge.index.size(); i++) index[i] = h->aEdge.index[i];
  for (size_t i = 0; i < h->aEdge.array.size(); i++) array[i] = h->aEdge.array[i];
}

// The assembly half of StepTime_InternalDynamicsILU (solve_internal_sparse.h:276-313),
// restated as the same sequence of reference calls.
void ref_assemble(void* p, const double* x, const double* v, double* vdia, double* vcrs,
                  double* b) {
  RefCloth* h = (RefCloth*)p;
  const co_params& q = h->prm;
  const int np = (int)h->aXYZ0.size() / 3;
  const int nDof = np * 3;
  std::vector<double> aXYZ(x, x + nDof), aUVW(v, v + nDof);
  double W = 0;
  std::vector<double> vec_b(nDof, 0);
  h->mat_A.SetZero();
  std::vector<int> tmp_buffer(np, -1);
  AddWdWddW_Cloth(W, vec_b, h->mat_A, tmp_buffer, aXYZ, h->aXYZ0, h->aTri, h->aQuad, q.lambda,
                  q.myu, q.stiff_bend);
  AddWdWddW_Contact(W, vec_b, h->mat_A, tmp_buffer, aXYZ, q.stiff_contact, q.contact_clearance,
                    obstacle_fn(q));
  AddWdW_Gravity(W, vec_b, aXYZ, q.gravity, q.mass_point);
  for (int i = 0; i < nDof; i++) vec_b[i] = -vec_b[i] + q.mass_point * aUVW[i] / q.dt;
  for (int ip = 0; ip < np; ip++) {
    h->mat_A.m_valDia[ip * 9 + 0 * 3 + 0] += q.mass_point / (q.dt * q.dt);
    h->mat_A.m_valDia[ip * 9 + 1 * 3 + 1] += q.mass_point / (q.dt * q.dt);
    h->mat_A.m_valDia[ip * 9 + 2 * 3 + 2] += q.mass_point / (q.dt * q.dt);
  }
  h->mat_A.SetBoundaryCondition(h->aBCFlag);
  for (int ip = 0; ip < np; ip++) {
    if (h->aBCFlag[ip] == 0) continue;
    vec_b[ip * 3 + 0] = 0;
    vec_b[ip * 3 + 1] = 0;
    vec_b[ip * 3 + 2] = 0;
  }
  h->vec_b = vec_b;
  if (vdia) memcpy(vdia, h->mat_A.m_valDia, sizeof(double) * 9 * np);
  if (vcrs) memcpy(vcrs, h->mat_A.m_valCrs, sizeof(double) * 9 * h->mat_A.m_ncrs);
  if (b) memcpy(b, vec_b.data(), sizeof(double) * nDof);
}

int ref_ilu(void* p, double* fdia, double* fcrs) {
  RefCloth* h = (RefCloth*)p;
  std::ostringstream sink;
  std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
  h->ilu_A->SetValueILU(h->mat_A);
  h->ilu_A->DoILUDecomp();
  std::cout.rdbuf(old);
  // singular pivots are reported on the console (ilu_sparse.cpp:545)
  int nsing = 0;
  const std::string s = sink.str();
  for (size_t pos = s.find("frac false 3"); pos != std::string::npos;
       pos = s.find("frac false 3", pos + 1))
    nsing++;
  const CMatrixSquareSparse& m = h->ilu_A->mat;
  if (fdia) memcpy(fdia, m.m_valDia, sizeof(double) * 9 * m.m_nblk);
  if (fcrs) memcpy(fcrs, m.m_valCrs, sizeof(double) * 9 * m.m_ncrs);
  return nsing;
}

void ref_pcg(void* p, const double* b, double tol, int maxit, double* x, double* conv, int* iter) {
  RefCloth* h = (RefCloth*)p;
  const int nDof = 3 * h->mat_A.m_nblk;
  std::vector<double> r(b, b + nDof), u;
  double c = tol;
  int it = maxit;
  Solve_PCG(c, it, h->mat_A, *h->ilu_A, r, u);
  memcpy(x, u.data(), sizeof(double) * nDof);
  *conv = c;
  *iter = it;
  h->r_last = r;
}

void ref_cg(void* p, const double* b, double tol, int maxit, double* x, double* conv, int* iter) {
  RefCloth* h = (RefCloth*)p;
  const int nDof = 3 * h->mat_A.m_nblk;
  std::vector<double> r(b, b + nDof), u;
  double c = tol;
  int it = maxit;
  Solve_CG(c, it, h->mat_A, r, u);
  memcpy(x, u.data(), sizeof(double) * nDof);
  *conv = c;
  *iter = it;
  h->r_last = r;
}

void ref_last_residual(void* p, double* r) {
  RefCloth* h = (RefCloth*)p;
  memcpy(r, h->r_last.data(), sizeof(double) * h->r_last.size());
}

void ref_ilu_solve(void* p, double* vec) {
  RefCloth* h = (RefCloth*)p;
  std::vector<double> v(vec, vec + 3 * h->mat_A.m_nblk);
  h->ilu_A->Solve(v);
  memcpy(vec, v.data(), sizeof(double) * v.size());
}

void ref_matvec(void* p, double alpha, const double* x, double beta, double* y) {
  RefCloth* h = (RefCloth*)p;
  const int nDof = 3 * h->mat_A.m_nblk;
  std::vector<double> xv(x, x + nDof), yv(y, y + nDof);
  h->mat_A.MatVec(alpha, xv, beta, yv);
  memcpy(y, yv.data(), sizeof(double) * nDof);
}

static CVector3D v3(const double* a, int k) { return CVector3D(a[3 * k], a[3 * k + 1], a[3 * k + 2]); }

double ref_distance_fv(const double* pt, double* w) {
  return DistanceFaceVertex(v3(pt, 0), v3(pt, 1), v3(pt, 2), v3(pt, 3), w[0], w[1]);
}

double ref_distance_ee(const double* pt, double* r) {
  return DistanceEdgeEdge(v3(pt, 0), v3(pt, 1), v3(pt, 2), v3(pt, 3), r[0], r[1]);
}

double ref_coplanar_time(const double* s, const double* e) {
  return FindCoplanerInterp(v3(s, 0), v3(s, 1), v3(s, 2), v3(s, 3), v3(e, 0), v3(e, 1), v3(e, 2), v3(e, 3));
}

void ref_fv_ccd_batch(int n, const double* p, const double* box, int* out) {
  const CAABB3D bb(box[0], box[3], box[1], box[4], box[2], box[5]);
  for (int i = 0; i < n; i++) {
    const double* a = p + 24 * (size_t)i;
    out[i] = IsContact_FV_CCD(0, 1, 2, 3, v3(a, 0), v3(a, 1), v3(a, 2), v3(a, 3), v3(a, 4), v3(a, 5), v3(a, 6),
                              v3(a, 7), bb);
  }
}

void ref_ee_ccd_batch(int n, const double* p, int* out) {
  for (int i = 0; i < n; i++) {
    const double* a = p + 24 * (size_t)i;
    out[i] = IsContact_EE_CCD(0, 1, 2, 3, v3(a, 0), v3(a, 1), v3(a, 2), v3(a, 3), v3(a, 4), v3(a, 5), v3(a, 6),
                              v3(a, 7));
  }
}

// StepTime_InternalDynamicsILU / StepTime_InternalDynamics with the solver tolerance
// and iteration cap taken from the parameters (the reference hard-codes them at
// solve_internal_sparse.h:245-246 and :318-319).
void ref_implicit(void* p, double* x, double* v, co_stats* st) {
  RefCloth* h = (RefCloth*)p;
  const co_params& q = h->prm;
  const int nDof = (int)h->aXYZ0.size();
  ref_assemble(p, x, v, 0, 0, 0);
  std::vector<double> vec_x;
  std::vector<double> r = h->vec_b;
  double conv = q.tol;
  int it = q.maxit;
  if (q.solver_kind == CO_SOLVER_CG) {
    Solve_CG(conv, it, h->mat_A, r, vec_x);
  } else {
    int ns = ref_ilu(p, 0, 0);
    if (st) st->ilu_singular = ns;
    Solve_PCG(conv, it, h->mat_A, *h->ilu_A, r, vec_x);
  }
  for (int i = 0; i < nDof; i++) x[i] += vec_x[i];
  for (int i = 0; i < nDof; i++) v[i] = vec_x[i] / q.dt;
  if (st) {
    st->solver_iterations = it;
    st->solver_conv = conv;
  }
}

void ref_refit_prx(void* p, const double* x, double delta, double* boxes) {
  RefCloth* h = (RefCloth*)p;
  std::vector<double> aXYZ(x, x + h->aXYZ0.size());
  BuildBoundingBoxChild_Prx(h->iroot_bvh, delta, aXYZ, h->aTri, h->aNodeBVH, h->aBB);
  if (boxes) export_boxes(h->aBB, boxes);
}

void ref_refit_ccd(void* p, const double* x, const double* v, double dt, double* boxes) {
  RefCloth* h = (RefCloth*)p;
  std::vector<double> aXYZ(x, x + h->aXYZ0.size()), aUVW(v, v + h->aXYZ0.size());
  h->aBB.resize(h->aNodeBVH.size());
  BuildBoundingBoxChild_CCD(h->iroot_bvh, dt, aXYZ, aUVW, h->aTri, h->aNodeBVH, h->aBB);
  if (boxes) export_boxes(h->aBB, boxes);
}

int ref_contacts_prx(void* p, const double* x, double delta, int* out, int cap) {
  RefCloth* h = (RefCloth*)p;
  std::vector<double> aXYZ(x, x + h->aXYZ0.size());
  BuildBoundingBoxChild_Prx(h->iroot_bvh, delta, aXYZ, h->aTri, h->aNodeBVH, h->aBB);
  std::set<CContactElement> s;
  GetContactElement_Proximity(s, delta, aXYZ, h->aTri, h->iroot_bvh, h->aNodeBVH, h->aBB);
  return from_set(s, out, cap);
}

int ref_contacts_ccd(void* p, const double* x, const double* v, double dt, double delta, int* out,
                     int cap) {
  RefCloth* h = (RefCloth*)p;
  std::vector<double> aXYZ(x, x + h->aXYZ0.size()), aUVW(v, v + h->aXYZ0.size());
  h->aBB.resize(h->aNodeBVH.size());
  BuildBoundingBoxChild_CCD(h->iroot_bvh, dt, aXYZ, aUVW, h->aTri, h->aNodeBVH, h->aBB);
  std::set<CContactElement> s;
  GetContactElement_CCD(s, dt, delta, aXYZ, aUVW, h->aTri, h->iroot_bvh, h->aNodeBVH, h->aBB);
  return from_set(s, out, cap);
}

void ref_impulse_prx(void* p, const double* x, double* v, const int* ce, int n) {
  RefCloth* h = (RefCloth*)p;
  const co_params& q = h->prm;
  std::vector<double> aXYZ(x, x + h->aXYZ0.size()), aUVW(v, v + h->aXYZ0.size());
  SelfCollisionImpulse_Proximity(aUVW, q.contact_clearance, q.stiff_contact, q.dt, q.mass_point,
                                 aXYZ, h->aTri, to_elems(ce, n));
  memcpy(v, aUVW.data(), sizeof(double) * aUVW.size());
}

void ref_impulse_ccd(void* p, const double* x, double* v, const int* ce, int n) {
  RefCloth* h = (RefCloth*)p;
  const co_params& q = h->prm;
  std::vector<double> aXYZ(x, x + h->aXYZ0.size()), aUVW(v, v + h->aXYZ0.size());
  SelfCollisionImpulse_CCD(aUVW, q.contact_clearance, q.stiff_contact, q.dt, q.mass_point, aXYZ,
                           h->aTri, to_elems(ce, n));
  memcpy(v, aUVW.data(), sizeof(double) * aUVW.size());
}

void ref_riz_reset(void* p) { ((RefCloth*)p)->aRIZ.clear(); }

void ref_riz_add(void* p, const int* ce, int n) {
  RefCloth* h = (RefCloth*)p;
  MakeRigidImpactZone(h->aRIZ, to_elems(ce, n), h->aEdge);
}

int ref_riz_zones(void* p, int* zone_of_vertex) {
  RefCloth* h = (RefCloth*)p;
  const int np = (int)h->aXYZ0.size() / 3;
  for (int i = 0; i < np; i++) zone_of_vertex[i] = -1;
  for (size_t z = 0; z < h->aRIZ.size(); z++)
    for (std::set<int>::const_iterator it = h->aRIZ[z].begin(); it != h->aRIZ[z].end(); ++it)
      zone_of_vertex[*it] = (int)z;
  return (int)h->aRIZ.size();
}

void ref_riz_apply(void* p, const double* x, double* v, const double* v0) {
  RefCloth* h = (RefCloth*)p;
  const size_t n = h->aXYZ0.size();
  std::vector<double> aXYZ(x, x + n), aUVW(v, v + n), aUVW0(v0, v0 + n);
  ApplyRigidImpactZone(aUVW, h->aRIZ, aXYZ, aUVW0);
  memcpy(v, aUVW.data(), sizeof(double) * n);
}

void ref_resolve(void* p, const double* x1, double* v, co_stats* st) {
  RefCloth* h = (RefCloth*)p;
  const co_params& q = h->prm;
  const size_t n = h->aXYZ0.size();
  std::vector<double> aXYZ1(x1, x1 + n), aUVW(v, v + n);
  bool applied = false;
  std::ostringstream sink;
  std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
  GetIntermidiateVelocityContactResolved(aUVW, applied, q.dt, q.contact_clearance, q.mass_point,
                                         q.stiff_contact, aXYZ1, h->aTri, h->aEdge, h->iroot_bvh,
                                         h->aNodeBVH, h->aBB);
  std::cout.rdbuf(old);
  memcpy(v, aUVW.data(), sizeof(double) * n);
  if (st) {
    co_stats s;
    memset(&s, 0, sizeof(s));
    s.solver_iterations = st->solver_iterations;
    s.solver_conv = st->solver_conv;
    s.ilu_singular = st->ilu_singular;
    parse_resolve_log(sink.str(), &s);
    s.impulse_applied = applied ? 1 : 0;
    *st = s;
  }
}

void ref_update_velocity(void* p, const double* x, double* v) {
  RefCloth* h = (RefCloth*)p;
  const co_params& q = h->prm;
  const size_t n = h->aXYZ0.size();
  std::vector<double> aXYZ(x, x + n), aUVW(v, v + n);
  UpdateIntermidiateVelocity(aUVW, aXYZ, h->aXYZ0, h->aBCFlag, h->aTri, h->aQuad, q.dt, q.lambda,
                             q.myu, q.stiff_bend, q.gravity, q.mass_point);
  memcpy(v, aUVW.data(), sizeof(double) * n);
}

// MakeNormal of self_contact_sparse/main.cpp:183-211 (the GLUT file cannot be
// compiled here): the reference's UnitNormalAreaTri3D in the demo's loop.
void ref_vertex_normals(void* p, const double* x, double* nrm) {
  RefCloth* h = (RefCloth*)p;
  const int np = (int)h->aXYZ0.size() / 3, ntri = (int)h->aTri.size() / 3;
  std::vector<double> aNormal(3 * (size_t)np, 0.0);
  for (int itri = 0; itri < ntri; itri++) {
    const int ip[3] = {h->aTri[3 * itri], h->aTri[3 * itri + 1], h->aTri[3 * itri + 2]};
    double n[3], area;
    UnitNormalAreaTri3D(n, area, x + 3 * ip[0], x + 3 * ip[1], x + 3 * ip[2]);
    for (int k = 0; k < 3; k++)
      for (int d = 0; d < 3; d++) aNormal[3 * ip[k] + d] += n[d];
  }
  for (int i = 0; i < np; i++) {
    const double sqlen = +aNormal[3 * i] * aNormal[3 * i] + aNormal[3 * i + 1] * aNormal[3 * i + 1] +
                         aNormal[3 * i + 2] * aNormal[3 * i + 2];
    const double invlen = 1.0 / sqrt(sqlen);
    for (int d = 0; d < 3; d++) nrm[3 * i + d] = aNormal[3 * i + d] * invlen;
  }
}

// StepTime of self_contact_sparse/main.cpp:213-263 without the normals (render only).
void ref_step(void* p, double* x, double* v, co_stats* st) {
  RefCloth* h = (RefCloth*)p;
  const co_params& q = h->prm;
  const size_t n = h->aXYZ0.size();
  co_stats s;
  memset(&s, 0, sizeof(s));
  std::vector<double> aXYZ1(x, x + n);
  {
    std::ostringstream sink;  // the implicit step prints its energy and residual
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    ref_implicit(p, x, v, &s);
    std::cout.rdbuf(old);
  }
  ref_resolve(p, aXYZ1.data(), v, &s);
  if (s.impulse_applied) {
    for (size_t ip = 0; ip < n / 3; ip++) {
      x[ip * 3 + 0] = aXYZ1[ip * 3 + 0] + v[ip * 3 + 0] * q.dt;
      x[ip * 3 + 1] = aXYZ1[ip * 3 + 1] + v[ip * 3 + 1] * q.dt;
      x[ip * 3 + 2] = aXYZ1[ip * 3 + 2] + v[ip * 3 + 2] * q.dt;
    }
    ref_update_velocity(p, x, v);
  }
  if (st) *st = s;
}

// The reference's StepTime_InternalDynamicsILU exactly as shipped (tolerance 1e-4,
// 100 iterations), for the "as shipped" comparison.
void ref_implicit_as_shipped(void* p, double* x, double* v) {
  RefCloth* h = (RefCloth*)p;
  const co_params& q = h->prm;
  const size_t n = h->aXYZ0.size();
  std::vector<double> aXYZ(x, x + n), aUVW(v, v + n);
  std::ostringstream sink;
  std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
  StepTime_InternalDynamicsILU(aXYZ, aUVW, h->mat_A, *h->ilu_A, h->aXYZ0, h->aBCFlag, h->aTri,
                               h->aQuad, q.dt, q.lambda, q.myu, q.stiff_bend, q.gravity,
                               q.mass_point, q.stiff_contact, q.contact_clearance,
                               obstacle_fn(q));
  std::cout.rdbuf(old);
  memcpy(x, aXYZ.data(), sizeof(double) * n);
  memcpy(v, aUVW.data(), sizeof(double) * n);
}

}  // extern "C"
