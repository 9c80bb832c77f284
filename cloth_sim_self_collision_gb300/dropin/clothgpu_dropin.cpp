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
  // the caller's pattern (the reference's driver never reads their values)
  (void)mat_A;
  (void)ilu_A;
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
  aBB.resize(std::max<size_t>(aNodeBVH.size(), (size_t)nnode));
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
