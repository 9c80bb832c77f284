// clothgpu_dropin.cpp -- the reference's frame functions over the C ABI
// (see clothgpu_dropin.h).
#include "clothgpu_dropin.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "../../include/clothgpu.h"

// ---- containers --------------------------------------------------------------------

CMatrixSquareSparse::CMatrixSquareSparse()
    : m_nblk(0), m_len(0), m_ncrs(0), m_colInd(nullptr), m_rowPtr(nullptr), m_valCrs(nullptr), m_valDia(nullptr) {}

CMatrixSquareSparse::CMatrixSquareSparse(int nblk, int len) : CMatrixSquareSparse() { Initialize(nblk, len); }

CMatrixSquareSparse::~CMatrixSquareSparse() {
  delete[] m_colInd;
  delete[] m_rowPtr;
  delete[] m_valCrs;
  delete[] m_valDia;
}

void CMatrixSquareSparse::Initialize(int nblk, int len) {
  delete[] m_colInd;
  delete[] m_rowPtr;
  delete[] m_valCrs;
  delete[] m_valDia;
  m_nblk = nblk;
  m_len = len;
  m_ncrs = 0;
  m_valDia = new double[(size_t)nblk * len * len]();
  m_colInd = new int[(size_t)nblk + 1]();
  m_rowPtr = nullptr;
  m_valCrs = nullptr;
}

void CMatrixSquareSparse::operator=(const CMatrixSquareSparse& m) {
  if (this == &m) return;
  Initialize(m.m_nblk, m.m_len);
  m_ncrs = m.m_ncrs;
  std::copy(m.m_colInd, m.m_colInd + m_nblk + 1, m_colInd);
  m_rowPtr = new int[(size_t)std::max(m_ncrs, 1)];
  std::copy(m.m_rowPtr, m.m_rowPtr + m_ncrs, m_rowPtr);
  const size_t bs = (size_t)m_len * m_len;
  m_valCrs = new double[std::max<size_t>(bs * m_ncrs, 1)];
  std::copy(m.m_valCrs, m.m_valCrs + bs * m_ncrs, m_valCrs);
  std::copy(m.m_valDia, m.m_valDia + bs * m_nblk, m_valDia);
}

void CMatrixSquareSparse::SetPattern(const std::vector<int>& colind, const std::vector<int>& rowptr) {
  assert((int)colind.size() == m_nblk + 1);
  std::copy(colind.begin(), colind.end(), m_colInd);
  m_ncrs = colind[m_nblk];
  delete[] m_rowPtr;
  delete[] m_valCrs;
  m_rowPtr = new int[(size_t)std::max(m_ncrs, 1)];
  std::copy(rowptr.begin(), rowptr.begin() + m_ncrs, m_rowPtr);
  m_valCrs = new double[std::max<size_t>((size_t)m_len * m_len * m_ncrs, 1)]();
}

bool CMatrixSquareSparse::SetZero() {
  std::fill(m_valDia, m_valDia + (size_t)m_len * m_len * m_nblk, 0.0);
  if (m_valCrs) std::fill(m_valCrs, m_valCrs + (size_t)m_len * m_len * m_ncrs, 0.0);
  return true;
}

// Mearge (matrix_square_sparse.cpp:88-138): adds an element matrix into the
// caller's host container, diagonal blocks to m_valDia and the pattern's
// off-diagonal blocks to m_valCrs (blocks outside the pattern are dropped)
bool CMatrixSquareSparse::Mearge(int nblkel_col, const int* blkel_col, int nblkel_row, const int* blkel_row,
                                 int blksize, const double* emat, std::vector<int>& buf) {
  assert(nblkel_col == nblkel_row && blksize == m_len * m_len);
  if ((int)buf.size() < m_nblk) buf.assign(m_nblk, -1);
  for (int a = 0; a < nblkel_col; a++) {
    const int row = blkel_col[a];
    for (int k = m_colInd[row]; k < m_colInd[row + 1]; k++) buf[m_rowPtr[k]] = k;
    for (int b = 0; b < nblkel_row; b++) {
      const double* in = emat + (size_t)(a * nblkel_row + b) * blksize;
      double* out;
      if (a == b) {
        out = m_valDia + (size_t)row * blksize;
      } else {
        const int slot = buf[blkel_row[b]];
        if (slot < 0) continue;
        out = m_valCrs + (size_t)slot * blksize;
      }
      for (int e = 0; e < blksize; e++) out[e] += in[e];
    }
    for (int k = m_colInd[row]; k < m_colInd[row + 1]; k++) buf[m_rowPtr[k]] = -1;
  }
  return true;
}

// SetBoundaryCondition (matrix_square_sparse.cpp:272-302): identity diagonal
// and zero off-diagonal blocks in the rows and columns of fixed vertices
void CMatrixSquareSparse::SetBoundaryCondition(const std::vector<int>& bc_flag) {
  const size_t bs = (size_t)m_len * m_len;
  for (int i = 0; i < m_nblk; i++) {
    if (bc_flag[i] == 0) continue;
    for (size_t e = 0; e < bs; e++) m_valDia[i * bs + e] = 0.0;
    for (int d = 0; d < m_len; d++) m_valDia[i * bs + (size_t)d * m_len + d] = 1.0;
    for (int k = m_colInd[i]; k < m_colInd[i + 1]; k++)
      for (size_t e = 0; e < bs; e++) m_valCrs[k * bs + e] = 0.0;
  }
  for (int k = 0; k < m_ncrs; k++)
    if (bc_flag[m_rowPtr[k]] != 0)
      for (size_t e = 0; e < bs; e++) m_valCrs[k * bs + e] = 0.0;
}

CPreconditionerILU::CPreconditionerILU() : m_diaInd(nullptr) {}
CPreconditionerILU::~CPreconditionerILU() { delete[] m_diaInd; }

void CPreconditionerILU::Initialize_ILU0(const CMatrixSquareSparse& m) {
  mat = m;
  delete[] m_diaInd;
  m_diaInd = new int[(size_t)std::max(m.m_nblk, 1)];
  for (int i = 0; i < m.m_nblk; i++) {
    m_diaInd[i] = mat.m_colInd[i + 1];
    for (int k = mat.m_colInd[i]; k < mat.m_colInd[i + 1]; k++)
      if (mat.m_rowPtr[k] > i) {
        m_diaInd[i] = k;
        break;
      }
  }
}

void CPreconditionerILU::SetValueILU(const CMatrixSquareSparse& m) {
  const size_t bs = (size_t)mat.m_len * mat.m_len;
  std::copy(m.m_valDia, m.m_valDia + bs * m.m_nblk, mat.m_valDia);
  if (m.m_ncrs == mat.m_ncrs) std::copy(m.m_valCrs, m.m_valCrs + bs * m.m_ncrs, mat.m_valCrs);
}

void CJaggedArray::InitializeSize(int size) {
  index.assign(size + 1, 0);
  array.clear();
}

int CJaggedArray::Size() const { return index.empty() ? 0 : (int)index.size() - 1; }

void CJaggedArray::SetNodeToElem(const std::vector<int>& elem, int nelem, int nnoel, int nnode) {
  index.assign(nnode + 1, 0);
  for (int e = 0; e < nelem * nnoel; e++) index[elem[e] + 1]++;
  for (int v = 0; v < nnode; v++) index[v + 1] += index[v];
  array.assign(index[nnode], 0);
  std::vector<int> fill(index.begin(), index.end() - 1);
  for (int e = 0; e < nelem; e++)
    for (int a = 0; a < nnoel; a++) array[fill[elem[e * nnoel + a]]++] = e;
}

void CJaggedArray::SetEdgeOfElem(const std::vector<int>& elem, int nelem, int nnoel, int nnode, bool is_dia) {
  CJaggedArray n2e;
  n2e.SetNodeToElem(elem, nelem, nnoel, nnode);
  std::vector<int> seen(nnode, -1);
  index.assign(nnode + 1, 0);
  array.clear();
  for (int v = 0; v < nnode; v++) {
    if (!is_dia) seen[v] = v;
    for (int i = n2e.index[v]; i < n2e.index[v + 1]; i++) {
      const int e = n2e.array[i];
      for (int a = 0; a < nnoel; a++) {
        const int w = elem[e * nnoel + a];
        if (seen[w] != v) {
          seen[w] = v;
          array.push_back(w);
        }
      }
    }
    index[v + 1] = (int)array.size();
  }
}

void CJaggedArray::Sort() {
  for (int v = 0; v + 1 < (int)index.size(); v++) std::sort(array.begin() + index[v], array.begin() + index[v + 1]);
}

CContactElement::CContactElement(bool fv, int j0, int j1, int j2, int j3) : is_fv(fv) {
  if (fv) {
    int a = j0, b = j1, c = j2;
    if (a > b) std::swap(a, b);
    if (b > c) std::swap(b, c);
    if (a > b) std::swap(a, b);
    ino0 = a;
    ino1 = b;
    ino2 = c;
    ino3 = j3;
  } else {
    const int lo01 = std::min(j0, j1), lo23 = std::min(j2, j3);
    int o0, o1;
    if (lo01 < lo23) {
      ino0 = lo01;
      ino1 = std::max(j0, j1);
      o0 = j2;
      o1 = j3;
    } else {
      ino0 = lo23;
      ino1 = std::max(j2, j3);
      o0 = j0;
      o1 = j1;
    }
    ino2 = std::min(o0, o1);
    ino3 = std::max(o0, o1);
  }
}

// ---- device side ---------------------------------------------------------------------
namespace {

typedef void (*PdFn)(double&, double*, const double*);

struct Obstacle {
  int kind;
  double center[3];
  double radius;
};

struct ClothKey {
  const int* tri;
  size_t ntri;
  const int* quad;
  size_t nquad;
  bool operator<(const ClothKey& o) const {
    return std::tie(tri, ntri, quad, nquad) < std::tie(o.tri, o.ntri, o.quad, o.nquad);
  }
};

struct State {
  std::mutex mu;
  cs_ctx* ctx = nullptr;
  std::map<PdFn, Obstacle> obstacles;
  std::map<ClothKey, int> cloths;
  std::map<const int*, int> by_tri;
  std::map<const CMatrixSquareSparse*, int> by_matrix;
  std::map<int, int> nverts;  // cloth id -> vertices
  std::map<int, cs_params> params;
  double ilu_tol = 1.0e-4, cg_tol = 1.0e-4;
  int ilu_maxit = 100, cg_maxit = 1000;
  int precision = CS_PREC_FP64;
  int exact = 1;
  int status = CS_OK;
  std::string error;
};

State& S() {
  static State s;
  return s;
}

bool fail(int code, const std::string& msg) {
  S().status = code;
  S().error = msg;
  std::fprintf(stderr, "clothgpu drop-in: %s\n", msg.c_str());
  return false;
}

bool ensure_ctx() {
  State& s = S();
  if (s.ctx) return true;
  if (std::getenv("CLOTHGPU_MIXED")) s.precision = CS_PREC_MIXED;
  if (std::getenv("CLOTHGPU_FAST_DOTS")) s.exact = 0;
  const int rc = cs_create(0, s.precision, &s.ctx);
  if (rc != CS_OK) return fail(rc, "no CUDA device for the cloth step");
  return true;
}

// the cloth of these arrays, admitted on first use
bool cloth_for(const std::vector<double>& X0, const std::vector<int>& bc, const std::vector<int>& tri,
               const std::vector<int>& quad, const cs_params& prm, int* id) {
  State& s = S();
  const ClothKey key{tri.data(), tri.size(), quad.data(), quad.size()};
  auto it = s.cloths.find(key);
  if (it != s.cloths.end()) {
    *id = it->second;
    cs_params& cur = s.params[*id];
    if (std::memcmp(&cur, &prm, sizeof(prm)) != 0) {
      const int rc = cs_set_params(s.ctx, *id, &prm);
      if (rc != CS_OK) return fail(rc, cs_last_error(s.ctx));
      cur = prm;
    }
    return true;
  }
  const int np = (int)X0.size() / 3;
  const int rc = cs_add_cloth(s.ctx, np, X0.data(), bc.empty() ? nullptr : bc.data(), (int)tri.size() / 3,
                              tri.data(), (int)quad.size() / 4, quad.data(), &prm, id);
  if (rc != CS_OK) return fail(rc, cs_last_error(s.ctx));
  s.cloths[key] = *id;
  s.by_tri[tri.data()] = *id;
  s.params[*id] = prm;
  s.nverts[*id] = np;
  return true;
}

bool obstacle_of(PdFn fn, cs_params& p) {
  auto it = S().obstacles.find(fn);
  if (it == S().obstacles.end())
    return fail(CS_ERR_ARG, "penetration-depth callback not registered (ClothGpuRegisterObstacle)");
  p.obstacle_kind = it->second.kind;
  std::copy(it->second.center, it->second.center + 3, p.obs_center);
  p.obs_radius = it->second.radius;
  return true;
}

cs_params make_params(double dt, double lambda, double myu, double stiff_bend, const double g[3], double mass,
                      double stiff_contact, double clearance, int solver) {
  State& s = S();
  cs_params p;
  std::memset(&p, 0, sizeof(p));
  p.dt = dt;
  p.lambda = lambda;
  p.myu = myu;
  p.stiff_bend = stiff_bend;
  std::copy(g, g + 3, p.gravity);
  p.mass_point = mass;
  p.stiff_contact = stiff_contact;
  p.contact_clearance = clearance;
  p.solver_kind = solver;
  p.tol = solver == CS_SOLVER_CG ? s.cg_tol : s.ilu_tol;
  p.maxit = solver == CS_SOLVER_CG ? s.cg_maxit : s.ilu_maxit;
  p.flags = s.exact ? CS_FLAG_EXACT_DOTS : 0;
  return p;
}

void implicit_step(std::vector<double>& aXYZ, std::vector<double>& aUVW, CMatrixSquareSparse& mat_A,
                   CPreconditionerILU* ilu_A, const std::vector<double>& aXYZ0, const std::vector<int>& aBCFlag,
                   const std::vector<int>& aTri, const std::vector<int>& aQuad, cs_params p, PdFn pd) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  if (!ensure_ctx() || !obstacle_of(pd, p)) return;
  int id;
  if (!cloth_for(aXYZ0, aBCFlag, aTri, aQuad, p, &id)) return;
  std::vector<double> x = aXYZ, v = aUVW;
  cs_stats st;
  const int rc = cs_implicit_step(s.ctx, id, x.data(), v.data(), &st);
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  aXYZ.swap(x);
  aUVW.swap(v);
  // the assembled matrix and its factor stay on the device; mat_A / ilu_A keep
  // the caller's pattern (the reference's driver never reads their values) and
  // name the cloth for the matrix functions
  s.by_matrix[&mat_A] = id;
  if (ilu_A) s.by_matrix[&ilu_A->mat] = id;
}

// the cloth whose matrix pattern m carries: the one it was passed with to a
// StepTime function, else an admitted cloth with the same pattern
bool cloth_of_matrix(const CMatrixSquareSparse& m, int* id) {
  State& s = S();
  auto it = s.by_matrix.find(&m);
  if (it != s.by_matrix.end()) {
    *id = it->second;
    return true;
  }
  if (m.m_len != 3) return fail(CS_ERR_ARG, "only 3x3 block matrices run on the device");
  for (const auto& kv : s.nverts) {
    int nb = 0;
    if (kv.second != m.m_nblk || cs_pattern(s.ctx, kv.first, &nb, nullptr, nullptr) != CS_OK || nb != m.m_ncrs)
      continue;
    std::vector<int> rp((size_t)m.m_nblk + 1), ci((size_t)std::max(nb, 1));
    if (cs_pattern(s.ctx, kv.first, nullptr, rp.data(), ci.data()) != CS_OK) continue;
    if (std::equal(rp.begin(), rp.end(), m.m_colInd) && std::equal(ci.begin(), ci.begin() + nb, m.m_rowPtr)) {
      s.by_matrix[&m] = kv.first;
      *id = kv.first;
      return true;
    }
  }
  return fail(CS_ERR_ARG, "matrix pattern belongs to no admitted cloth (pass it to a StepTime function first)");
}

// uploads the values of m as the cloth's device matrix
bool upload_matrix(const CMatrixSquareSparse& m, int* id) {
  State& s = S();
  if (!ensure_ctx() || !cloth_of_matrix(m, id)) return false;
  const int rc = cs_set_matrix(s.ctx, *id, m.m_valDia, m.m_valCrs);
  if (rc != CS_OK) return fail(rc, cs_last_error(s.ctx));
  return true;
}

// the cloth of aTri for the BVH functions (admitted with aXYZ as its rest
// shape, no stencils, when it is new)
bool cloth_of_mesh(const std::vector<int>& aTri, const std::vector<double>& aXYZ, int* id) {
  State& s = S();
  if (!ensure_ctx()) return false;
  auto it = s.by_tri.find(aTri.data());
  if (it != s.by_tri.end()) {
    *id = it->second;
    return true;
  }
  const double g[3] = {0, 0, 0};
  cs_params p = make_params(0.0, 0, 0, 0, g, 1.0, 0.0, 0.0, CS_SOLVER_CG);
  std::vector<int> bc, quad;
  return cloth_for(aXYZ, bc, aTri, quad, p, id);
}

void boxes_to(const std::vector<double>& boxes, int nnode, int ibvh, const std::vector<CNodeBVH>& nodes,
              std::vector<CAABB3D>& aBB) {
  aBB.resize(std::max<size_t>(nodes.size(), (size_t)nnode));
  for (int n = 0; n < nnode; n++) {
    CAABB3D& b = aBB[n];
    b.x_min = boxes[7 * n + 0];
    b.x_max = boxes[7 * n + 1];
    b.y_min = boxes[7 * n + 2];
    b.y_max = boxes[7 * n + 3];
    b.z_min = boxes[7 * n + 4];
    b.z_max = boxes[7 * n + 5];
    b.isnt_empty = boxes[7 * n + 6] != 0.0;
  }
  (void)ibvh;
}

}  // namespace

void StepTime_InternalDynamicsILU(std::vector<double>& aXYZ, std::vector<double>& aUVW, CMatrixSquareSparse& mat_A,
                                  CPreconditionerILU& ilu_A, const std::vector<double>& aXYZ0,
                                  const std::vector<int>& aBCFlag, const std::vector<int>& aTri,
                                  const std::vector<int>& aQuad, const double dt, double lambda, double myu,
                                  double stiff_bend, const double gravity[3], double mass_point, double stiff_contact,
                                  double contact_clearance, void (*penetrationDepth)(double&, double*, const double*)) {
  const cs_params p = make_params(dt, lambda, myu, stiff_bend, gravity, mass_point, stiff_contact, contact_clearance,
                                  CS_SOLVER_ILU_PCG);
  implicit_step(aXYZ, aUVW, mat_A, &ilu_A, aXYZ0, aBCFlag, aTri, aQuad, p, penetrationDepth);
}

void StepTime_InternalDynamics(std::vector<double>& aXYZ, std::vector<double>& aUVW, CMatrixSquareSparse& mat_A,
                               const std::vector<double>& aXYZ0, const std::vector<int>& aBCFlag,
                               const std::vector<int>& aTri, const std::vector<int>& aQuad, const double dt,
                               double lambda, double myu, double stiff_bend, const double gravity[3],
                               double mass_point, double stiff_contact, double contact_clearance,
                               void (*penetrationDepth)(double&, double*, const double*)) {
  const cs_params p = make_params(dt, lambda, myu, stiff_bend, gravity, mass_point, stiff_contact, contact_clearance,
                                  CS_SOLVER_CG);
  implicit_step(aXYZ, aUVW, mat_A, nullptr, aXYZ0, aBCFlag, aTri, aQuad, p, penetrationDepth);
}

void UpdateIntermidiateVelocity(std::vector<double>& aUVW, const std::vector<double>& aXYZ,
                                const std::vector<double>& aXYZ0, const std::vector<int>& aBCFlag,
                                const std::vector<int>& aTri, const std::vector<int>& aQuad, const double dt,
                                double lambda, double myu, double stiff_bend, const double gravity[3],
                                double mass_point) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  if (!ensure_ctx()) return;
  int id;
  auto it = s.cloths.find(ClothKey{aTri.data(), aTri.size(), aQuad.data(), aQuad.size()});
  cs_params p;
  if (it != s.cloths.end()) {
    p = s.params[it->second];
    p.dt = dt;
    p.lambda = lambda;
    p.myu = myu;
    p.stiff_bend = stiff_bend;
    std::copy(gravity, gravity + 3, p.gravity);
    p.mass_point = mass_point;
  } else {
    p = make_params(dt, lambda, myu, stiff_bend, gravity, mass_point, 0.0, 0.0, CS_SOLVER_CG);
  }
  if (!cloth_for(aXYZ0, aBCFlag, aTri, aQuad, p, &id)) return;
  std::vector<double> v = aUVW;
  const int rc = cs_update_velocity(s.ctx, id, aXYZ.data(), v.data());
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  aUVW.swap(v);
}

void GetIntermidiateVelocityContactResolved(std::vector<double>& aUVWm, bool& is_impulse_applied, double dt,
                                            double contact_clearance, double mass_point,
                                            double cloth_contact_stiffness, const std::vector<double>& aXYZ,
                                            const std::vector<int>& aTri, const CJaggedArray& aEdge, int iroot_bvh,
                                            const std::vector<CNodeBVH>& aNodeBVH, std::vector<CAABB3D>& aBB) {
  (void)aEdge;
  (void)iroot_bvh;
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  is_impulse_applied = false;
  if (!ensure_ctx()) return;
  auto it = s.by_tri.find(aTri.data());
  int id;
  if (it == s.by_tri.end()) {
    // a cloth seen first here: admitted with these positions as its rest shape
    const double g[3] = {0, 0, 0};
    cs_params p = make_params(dt, 0, 0, 0, g, mass_point, cloth_contact_stiffness, contact_clearance, CS_SOLVER_CG);
    std::vector<int> bc, quad;
    if (!cloth_for(aXYZ, bc, aTri, quad, p, &id)) return;
  } else {
    id = it->second;
  }
  cs_params& p = s.params[id];
  if (p.dt != dt || p.contact_clearance != contact_clearance || p.mass_point != mass_point ||
      p.stiff_contact != cloth_contact_stiffness) {
    p.dt = dt;
    p.contact_clearance = contact_clearance;
    p.mass_point = mass_point;
    p.stiff_contact = cloth_contact_stiffness;
    const int rc = cs_set_params(s.ctx, id, &p);
    if (rc != CS_OK) {
      fail(rc, cs_last_error(s.ctx));
      return;
    }
  }
  std::vector<double> v = aUVWm;
  cs_stats st;
  int rc = cs_resolve_contacts(s.ctx, id, aXYZ.data(), v.data(), &st);
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  aUVWm.swap(v);
  is_impulse_applied = st.impulse_applied != 0;
  int nnode = 0;
  cs_bvh_nodes(s.ctx, id, &nnode, nullptr);
  std::vector<double> boxes(7 * (size_t)nnode);
  rc = cs_get_boxes(s.ctx, id, boxes.data());
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  boxes_to(boxes, nnode, 0, aNodeBVH, aBB);
}

int MakeBVHTopology_TopDown(const std::vector<int>& aTri, const std::vector<double>& aXYZ,
                            std::vector<CNodeBVH>& aNodeBVH) {
  const int np = (int)aXYZ.size() / 3, nt = (int)aTri.size() / 3;
  int nnode = 0;
  int rc = cs_build_bvh(np, aXYZ.data(), nt, aTri.data(), nullptr, 0, &nnode);
  if (rc != CS_OK) {
    fail(rc, "MakeBVHTopology_TopDown: bad mesh");
    return 0;
  }
  std::vector<int> nodes(3 * (size_t)nnode);
  rc = cs_build_bvh(np, aXYZ.data(), nt, aTri.data(), nodes.data(), (int)nodes.size(), &nnode);
  aNodeBVH.resize(nnode);
  for (int n = 0; n < nnode; n++) {
    aNodeBVH[n].iroot = nodes[3 * n];
    aNodeBVH[n].ichild[0] = nodes[3 * n + 1];
    aNodeBVH[n].ichild[1] = nodes[3 * n + 2];
  }
  return 0;
}

// ---- lower-level functions on the device ------------------------------------------

void CMatrixSquareSparse::MatVec(double alpha, const std::vector<double>& x, double beta,
                                 std::vector<double>& y) const {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id;
  if (!upload_matrix(*this, &id)) return;
  const int rc = cs_matvec(s.ctx, id, alpha, x.data(), beta, y.data());
  if (rc != CS_OK) fail(rc, cs_last_error(s.ctx));
}

void Solve_CG(double& conv_ratio, int& iteration, const CMatrixSquareSparse& mat, std::vector<double>& r_vec,
              std::vector<double>& u_vec) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id;
  if (!upload_matrix(mat, &id)) return;
  u_vec.resize(r_vec.size());
  double conv = 0.0;
  int iter = 0;
  int rc = cs_solve_cg(s.ctx, id, r_vec.data(), conv_ratio, iteration, u_vec.data(), &conv, &iter);
  if (rc == CS_OK) rc = cs_last_residual(s.ctx, id, r_vec.data());
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  conv_ratio = conv;
  iteration = iter;
}

void CPreconditionerILU::DoILUDecomp() {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id;
  if (!upload_matrix(mat, &id)) return;
  int nsing = 0;
  const int rc = cs_ilu_factor(s.ctx, id, mat.m_valDia, mat.m_valCrs, &nsing);
  if (rc != CS_OK) fail(rc, cs_last_error(s.ctx));
}

void CPreconditionerILU::Solve(std::vector<double>& vec) const {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id;
  if (!ensure_ctx() || !cloth_of_matrix(mat, &id)) return;
  const int rc = cs_ilu_solve(s.ctx, id, vec.data());
  if (rc != CS_OK) fail(rc, cs_last_error(s.ctx));
}

void Solve_PCG(double& conv_ratio, int& iteration, const CMatrixSquareSparse& mat, const CPreconditionerILU& ilu,
               std::vector<double>& r_vec, std::vector<double>& u_vec) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id, idf;
  if (!upload_matrix(mat, &id) || !cloth_of_matrix(ilu.mat, &idf)) return;
  if (id != idf) {
    fail(CS_ERR_ARG, "Solve_PCG: the matrix and the preconditioner belong to different cloths");
    return;
  }
  u_vec.resize(r_vec.size());
  double conv = 0.0;
  int iter = 0;
  int rc = cs_solve_pcg(s.ctx, id, r_vec.data(), conv_ratio, iteration, u_vec.data(), &conv, &iter);
  if (rc == CS_OK) rc = cs_last_residual(s.ctx, id, r_vec.data());
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  conv_ratio = conv;
  iteration = iter;
}

void BuildBoundingBoxChild_Prx(int ibvh, double delta, const std::vector<double>& aXYZ, const std::vector<int>& aTri,
                               const std::vector<CNodeBVH>& aNodeBVH, std::vector<CAABB3D>& aBB) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id;
  if (ibvh != 0) {
    fail(CS_ERR_ARG, "BuildBoundingBoxChild_Prx: only the root node (0) is refitted on the device");
    return;
  }
  if (!cloth_of_mesh(aTri, aXYZ, &id)) return;
  int nnode = 0;
  cs_bvh_nodes(s.ctx, id, &nnode, nullptr);
  std::vector<double> boxes(7 * (size_t)nnode);
  const int rc = cs_refit_prx(s.ctx, id, aXYZ.data(), delta, boxes.data());
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  boxes_to(boxes, nnode, ibvh, aNodeBVH, aBB);
}

void BuildBoundingBoxChild_CCD(int ibvh, double dt, const std::vector<double>& aXYZ, const std::vector<double>& aUVW,
                               const std::vector<int>& aTri, const std::vector<CNodeBVH>& aNodeBVH,
                               std::vector<CAABB3D>& aBB) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id;
  if (ibvh != 0) {
    fail(CS_ERR_ARG, "BuildBoundingBoxChild_CCD: only the root node (0) is refitted on the device");
    return;
  }
  if (!cloth_of_mesh(aTri, aXYZ, &id)) return;
  int nnode = 0;
  cs_bvh_nodes(s.ctx, id, &nnode, nullptr);
  std::vector<double> boxes(7 * (size_t)nnode);
  const int rc = cs_refit_ccd(s.ctx, id, aXYZ.data(), aUVW.data(), dt, boxes.data());
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  boxes_to(boxes, nnode, ibvh, aNodeBVH, aBB);
}

namespace {
// contacts of one detection into a std::set (the reference's container)
template <typename F>
void contacts_into(std::set<CContactElement>& out, F&& detect) {
  State& s = S();
  int n = 0;
  std::vector<int> buf(5 * 4096);
  int rc = detect(buf.data(), 4096, &n);
  if (rc == CS_ERR_CAPACITY && n > 4096) {
    buf.assign(5 * (size_t)n, 0);
    rc = detect(buf.data(), n, &n);
  }
  if (rc != CS_OK) {
    fail(rc, cs_last_error(s.ctx));
    return;
  }
  for (int e = 0; e < n; e++) {
    const int* c = buf.data() + 5 * (size_t)e;
    // the stored key is canonical already: the constructor keeps it
    out.insert(CContactElement(c[0] != 0, c[1], c[2], c[3], c[4]));
  }
}
}  // namespace

void GetContactElement_Proximity(std::set<CContactElement>& aContactElem, double delta,
                                 const std::vector<double>& aXYZ, const std::vector<int>& aTri, int ibvh,
                                 const std::vector<CNodeBVH>& aBVH, const std::vector<CAABB3D>& aBB) {
  (void)aBVH;
  (void)aBB;
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id;
  if (ibvh != 0) {
    fail(CS_ERR_ARG, "GetContactElement_Proximity: only the root node (0) is searched on the device");
    return;
  }
  if (!cloth_of_mesh(aTri, aXYZ, &id)) return;
  contacts_into(aContactElem, [&](int* out, int cap, int* n) {
    return cs_contacts_prx(s.ctx, id, aXYZ.data(), delta, out, cap, n);
  });
}

void GetContactElement_CCD(std::set<CContactElement>& aContactElem, double dt, double delta,
                           const std::vector<double>& aXYZ, const std::vector<double>& aUVW,
                           const std::vector<int>& aTri, int ibvh, const std::vector<CNodeBVH>& aBVH,
                           const std::vector<CAABB3D>& aBB) {
  (void)aBVH;
  (void)aBB;
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  int id;
  if (ibvh != 0) {
    fail(CS_ERR_ARG, "GetContactElement_CCD: only the root node (0) is searched on the device");
    return;
  }
  if (!cloth_of_mesh(aTri, aXYZ, &id)) return;
  contacts_into(aContactElem, [&](int* out, int cap, int* n) {
    return cs_contacts_ccd(s.ctx, id, aXYZ.data(), aUVW.data(), dt, delta, out, cap, n);
  });
}

namespace {
void put(double* d, const CVector3D& v) {
  d[0] = v.x;
  d[1] = v.y;
  d[2] = v.z;
}
}  // namespace

double DistanceFaceVertex(const CVector3D& p0, const CVector3D& p1, const CVector3D& p2, const CVector3D& p3,
                          double& w0, double& w1) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  double pts[12], dist = 0.0, w[2] = {0.0, 0.0};
  put(pts, p0);
  put(pts + 3, p1);
  put(pts + 6, p2);
  put(pts + 9, p3);
  if (!ensure_ctx()) return 0.0;
  const int rc = cs_distance_fv(s.ctx, 1, pts, &dist, w);
  if (rc != CS_OK) fail(rc, cs_last_error(s.ctx));
  w0 = w[0];
  w1 = w[1];
  return dist;
}

double DistanceEdgeEdge(const CVector3D& p0, const CVector3D& p1, const CVector3D& q0, const CVector3D& q1,
                        double& ratio_p, double& ratio_q) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  double pts[12], dist = 0.0, r[2] = {0.0, 0.0};
  put(pts, p0);
  put(pts + 3, p1);
  put(pts + 6, q0);
  put(pts + 9, q1);
  if (!ensure_ctx()) return 0.0;
  const int rc = cs_distance_ee(s.ctx, 1, pts, &dist, r);
  if (rc != CS_OK) fail(rc, cs_last_error(s.ctx));
  ratio_p = r[0];
  ratio_q = r[1];
  return dist;
}

double FindCoplanerInterp(const CVector3D& s0, const CVector3D& s1, const CVector3D& s2, const CVector3D& s3,
                          const CVector3D& e0, const CVector3D& e1, const CVector3D& e2, const CVector3D& e3) {
  State& s = S();
  std::lock_guard<std::mutex> lock(s.mu);
  s.status = CS_OK;
  double a[12], b[12], t = -1.0;
  put(a, s0);
  put(a + 3, s1);
  put(a + 6, s2);
  put(a + 9, s3);
  put(b, e0);
  put(b + 3, e1);
  put(b + 6, e2);
  put(b + 9, e3);
  if (!ensure_ctx()) return -1.0;
  const int rc = cs_coplanar_time(s.ctx, 1, a, b, &t);
  if (rc != CS_OK) fail(rc, cs_last_error(s.ctx));
  return t;
}

void ClothGpuRegisterObstacle(void (*penetrationDepth)(double&, double*, const double*), int kind,
                              const double center[3], double radius) {
  Obstacle o;
  o.kind = kind;
  std::copy(center, center + 3, o.center);
  o.radius = radius;
  std::lock_guard<std::mutex> lock(S().mu);
  S().obstacles[penetrationDepth] = o;
}

void ClothGpuSetSolver(double ilu_tol, int ilu_maxit, double cg_tol, int cg_maxit) {
  std::lock_guard<std::mutex> lock(S().mu);
  S().ilu_tol = ilu_tol;
  S().ilu_maxit = ilu_maxit;
  S().cg_tol = cg_tol;
  S().cg_maxit = cg_maxit;
}

void ClothGpuSetMode(int precision, int exact_dots) {
  std::lock_guard<std::mutex> lock(S().mu);
  State& s = S();
  s.precision = precision;
  s.exact = exact_dots;
  if (s.ctx) cs_set_precision(s.ctx, precision);
}

int ClothGpuLastStatus() { return S().status; }
const char* ClothGpuLastError() { return S().error.c_str(); }
