// clothgpu_dropin.h -- C++ drop-in for the reference's self_contact_sparse path.
//
// Declares, with the reference's own names and signatures, the classes and
// functions its GLUT driver (self_contact_sparse/main.cpp) uses, so that driver
// compiles unchanged against these headers and runs its frame on the GPU:
//
//   StepTime_InternalDynamicsILU      solve_internal_sparse.h:255-275
//   StepTime_InternalDynamics         solve_internal_sparse.h:185-202
//   UpdateIntermidiateVelocity        solve_internal_sparse.h:329-343
//   GetIntermidiateVelocityContactResolved  self_collision_cloth.h:21-34
//   MakeBVHTopology_TopDown           bvh_aabb.h:25-28
//   BuildBoundingBoxChild_Prx / _CCD  bvh_aabb.h:31-46
//   GetContactElement_Proximity / _CCD                      bvh_aabb.h:110-130
//   DistanceFaceVertex, DistanceEdgeEdge, FindCoplanerInterp bvh_aabb.h:49-61
//   CMatrixSquareSparse (Initialize, SetPattern, SetZero, Mearge, MatVec,
//                        SetBoundaryCondition)              matrix_square_sparse.h:14-48
//   Solve_CG                          matrix_square_sparse.h:58-63
//   CPreconditionerILU (Initialize_ILU0, SetValueILU, DoILUDecomp, Solve)  ilu_sparse.h:16-34
//   Solve_PCG                         ilu_sparse.h:37-43
//   CJaggedArray (SetNodeToElem, SetEdgeOfElem, Sort)       jagged_array.h:20-264
//   CNodeBVH, CAABB3D, CContactElement, CVector3D           bvh_aabb.h:18-106, aabb.h:16-148,
//                                                           vector3d.h
//
// The frame functions forward to the C ABI (include/clothgpu.h): a cloth is
// identified by its triangle and stencil arrays, admitted on first use with
// the rest shape aXYZ0, and its matrix / BVH live on the device.  The
// reference's penetration-depth callback cannot run on a device: register it
// once with ClothGpuRegisterObstacle (an unregistered callback makes the call
// fail, reported by ClothGpuLastStatus, with the state left unchanged).
//
// The lower-level functions run on the device too.  The BVH functions take
// the cloth of aTri (admitted with aXYZ as its rest shape if it is new) and
// recompute the boxes from aXYZ as the matching BuildBoundingBoxChild_* call
// would; they accept the root node only.  The containers stay on the host, as
// in the reference: Mearge, SetZero and SetBoundaryCondition edit the caller's
// arrays, and MatVec, Solve_CG, DoILUDecomp, ILU Solve and Solve_PCG upload
// the matrix values to the cloth whose pattern the matrix carries (the matrix
// passed to a StepTime function, or any matrix with an admitted cloth's
// pattern) and compute there.  DoILUDecomp writes the factor back into the
// preconditioner's matrix; Solve uses the factor of that cloth's last
// DoILUDecomp or implicit step.
//
// Defaults reproduce the reference: FP64 with serial inner products (bit-exact
// frames), PCG tolerance 1e-4 / 100 iterations and CG 1e-4 / 1000 as hard-coded
// in solve_internal_sparse.h:245-246, 318-319.  ClothGpuSetSolver and
// ClothGpuSetMode change them.
#ifndef CLOTHGPU_DROPIN_H
#define CLOTHGPU_DROPIN_H

#include <cassert>
#include <set>
#include <vector>

// ---- containers (host side, the reference's data layout) -------------------------

class CVector3D {
 public:
  CVector3D() : x(0), y(0), z(0) {}
  CVector3D(double vx, double vy, double vz) : x(vx), y(vy), z(vz) {}

 public:
  double x, y, z;
};

class CMatrixSquareSparse {
 public:
  CMatrixSquareSparse();
  CMatrixSquareSparse(int nblk, int len);
  virtual ~CMatrixSquareSparse();
  void Initialize(int nblk, int len);
  void operator=(const CMatrixSquareSparse& m);
  void SetPattern(const std::vector<int>& colind, const std::vector<int>& rowptr);
  bool SetZero();
  bool Mearge(int nblkel_col, const int* blkel_col, int nblkel_row, const int* blkel_row, int blksize,
              const double* emat, std::vector<int>& m_marge_tmp_buffer);
  // {y} = alpha * [A]{x} + beta * {y}
  void MatVec(double alpha, const std::vector<double>& x, double beta, std::vector<double>& y) const;
  void SetBoundaryCondition(const std::vector<int>& bc_flag);

 public:
  int m_nblk;
  int m_len;
  int m_ncrs;
  int* m_colInd;  // row pointers (the reference's naming)
  int* m_rowPtr;  // column indices
  double* m_valCrs;
  double* m_valDia;

 private:
  CMatrixSquareSparse(const CMatrixSquareSparse&);
};

class CPreconditionerILU {
 public:
  CPreconditionerILU();
  ~CPreconditionerILU();
  void Initialize_ILU0(const CMatrixSquareSparse& m);
  void SetValueILU(const CMatrixSquareSparse& m);
  void Solve(std::vector<double>& vec) const;
  void DoILUDecomp();

 public:
  CMatrixSquareSparse mat;
  int* m_diaInd;
};

void Solve_CG(double& conv_ratio, int& iteration, const CMatrixSquareSparse& mat, std::vector<double>& r_vec,
              std::vector<double>& u_vec);

void Solve_PCG(double& conv_ratio, int& iteration, const CMatrixSquareSparse& mat, const CPreconditionerILU& ilu,
               std::vector<double>& r_vec, std::vector<double>& u_vec);

class CJaggedArray {
 public:
  CJaggedArray() {}
  void InitializeSize(int size);
  int Size() const;
  void SetNodeToElem(const std::vector<int>& elem, int nelem, int nnoel, int nnode);
  void SetEdgeOfElem(const std::vector<int>& elem, int nelem, int nnoel, int nnode, bool is_dia);
  void Sort();

 public:
  std::vector<int> index;
  std::vector<int> array;
};

class CNodeBVH {
 public:
  int iroot;
  int ichild[2];
};

class CAABB3D {
 public:
  CAABB3D() : x_min(0), x_max(0), y_min(0), y_max(0), z_min(0), z_max(0), isnt_empty(false) {}
  bool IsIntersect(const CAABB3D& bb) const {
    if (!isnt_empty || !bb.isnt_empty) return false;
    return !(x_max < bb.x_min || x_min > bb.x_max || y_max < bb.y_min || y_min > bb.y_max || z_max < bb.z_min ||
             z_min > bb.z_max);
  }

 public:
  double x_min, x_max, y_min, y_max, z_min, z_max;
  bool isnt_empty;
};

class CContactElement {
 public:
  CContactElement(bool is_fv, int j0, int j1, int j2, int j3);
  bool operator<(const CContactElement& p2) const {
    if (ino0 != p2.ino0) return ino0 < p2.ino0;
    if (ino1 != p2.ino1) return ino1 < p2.ino1;
    if (ino2 != p2.ino2) return ino2 < p2.ino2;
    return ino3 < p2.ino3;
  }

 public:
  bool is_fv;
  int ino0, ino1, ino2, ino3;
};

// ---- the frame on the GPU --------------------------------------------------------

void StepTime_InternalDynamicsILU(std::vector<double>& aXYZ, std::vector<double>& aUVW, CMatrixSquareSparse& mat_A,
                                  CPreconditionerILU& ilu_A, const std::vector<double>& aXYZ0,
                                  const std::vector<int>& aBCFlag, const std::vector<int>& aTri,
                                  const std::vector<int>& aQuad, const double dt, double lambda, double myu,
                                  double stiff_bend, const double gravity[3], double mass_point, double stiff_contact,
                                  double contact_clearance, void (*penetrationDepth)(double&, double*, const double*));

void StepTime_InternalDynamics(std::vector<double>& aXYZ, std::vector<double>& aUVW, CMatrixSquareSparse& mat_A,
                               const std::vector<double>& aXYZ0, const std::vector<int>& aBCFlag,
                               const std::vector<int>& aTri, const std::vector<int>& aQuad, const double dt,
                               double lambda, double myu, double stiff_bend, const double gravity[3],
                               double mass_point, double stiff_contact, double contact_clearance,
                               void (*penetrationDepth)(double&, double*, const double*));

void UpdateIntermidiateVelocity(std::vector<double>& aUVW, const std::vector<double>& aXYZ,
                                const std::vector<double>& aXYZ0, const std::vector<int>& aBCFlag,
                                const std::vector<int>& aTri, const std::vector<int>& aQuad, const double dt,
                                double lambda, double myu, double stiff_bend, const double gravity[3],
                                double mass_point);

void GetIntermidiateVelocityContactResolved(std::vector<double>& aUVWm, bool& is_impulse_applied, double dt,
                                            double contact_clearance, double mass_point,
                                            double cloth_contact_stiffness, const std::vector<double>& aXYZ,
                                            const std::vector<int>& aTri, const CJaggedArray& aEdge, int iroot_bvh,
                                            const std::vector<CNodeBVH>& aNodeBVH, std::vector<CAABB3D>& aBB);

int MakeBVHTopology_TopDown(const std::vector<int>& aTri, const std::vector<double>& aXYZ,
                            std::vector<CNodeBVH>& aNodeBVH);

void BuildBoundingBoxChild_Prx(int ibvh, double delta, const std::vector<double>& aXYZ, const std::vector<int>& aTri,
                               const std::vector<CNodeBVH>& aNodeBVH, std::vector<CAABB3D>& aBB);

void BuildBoundingBoxChild_CCD(int ibvh, double dt, const std::vector<double>& aXYZ, const std::vector<double>& aUVW,
                               const std::vector<int>& aTri, const std::vector<CNodeBVH>& aNodeBVH,
                               std::vector<CAABB3D>& aBB);

double DistanceFaceVertex(const CVector3D& p0, const CVector3D& p1, const CVector3D& p2, const CVector3D& p3,
                          double& w0, double& w1);

double DistanceEdgeEdge(const CVector3D& p0, const CVector3D& p1, const CVector3D& q0, const CVector3D& q1,
                        double& ratio_p, double& ratio_q);

double FindCoplanerInterp(const CVector3D& s0, const CVector3D& s1, const CVector3D& s2, const CVector3D& s3,
                          const CVector3D& e0, const CVector3D& e1, const CVector3D& e2, const CVector3D& e3);

void GetContactElement_Proximity(std::set<CContactElement>& aContactElem, double delta,
                                 const std::vector<double>& aXYZ, const std::vector<int>& aTri, int ibvh,
                                 const std::vector<CNodeBVH>& aBVH, const std::vector<CAABB3D>& aBB);

void GetContactElement_CCD(std::set<CContactElement>& aContactElem, double dt, double delta,
                           const std::vector<double>& aXYZ, const std::vector<double>& aUVW,
                           const std::vector<int>& aTri, int ibvh, const std::vector<CNodeBVH>& aBVH,
                           const std::vector<CAABB3D>& aBB);

// ---- extensions ------------------------------------------------------------------

// obstacle kinds of include/clothgpu.h (CS_OBSTACLE_*)
void ClothGpuRegisterObstacle(void (*penetrationDepth)(double&, double*, const double*), int kind,
                              const double center[3], double radius);
// tolerance / iteration cap of the two frame variants (defaults: the reference's)
void ClothGpuSetSolver(double ilu_tol, int ilu_maxit, double cg_tol, int cg_maxit);
// precision: 0 FP64, 1 mixed; exact_dots: serial inner products (bit-exact FP64)
void ClothGpuSetMode(int precision, int exact_dots);
// status of the last drop-in call (CS_OK or a CS_ERR_* code) and its message
int ClothGpuLastStatus();
const char* ClothGpuLastError();

#endif
