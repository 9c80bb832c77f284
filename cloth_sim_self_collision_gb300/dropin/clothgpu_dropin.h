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
//   CMatrixSquareSparse (Initialize, SetPattern, SetZero)   matrix_square_sparse.h:14-48
//   CPreconditionerILU (Initialize_ILU0, SetValueILU)      ilu_sparse.h:16-34
//   CJaggedArray (SetNodeToElem, SetEdgeOfElem, Sort)       jagged_array.h:20-264
//   CNodeBVH, CAABB3D, CContactElement                      bvh_aabb.h:18-106, aabb.h:16-148
//
// The frame functions forward to the C ABI (include/clothgpu.h): a cloth is
// identified by its triangle and stencil arrays, admitted on first use with
// the rest shape aXYZ0, and its matrix / BVH live on the device.  The
// reference's penetration-depth callback cannot run on a device: register it
// once with ClothGpuRegisterObstacle (an unregistered callback makes the call
// fail, reported by ClothGpuLastStatus, with the state left unchanged).
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

class CMatrixSquareSparse {
 public:
  CMatrixSquareSparse();
  CMatrixSquareSparse(int nblk, int len);
  virtual ~CMatrixSquareSparse();
  void Initialize(int nblk, int len);
  void operator=(const CMatrixSquareSparse& m);
  void SetPattern(const std::vector<int>& colind, const std::vector<int>& rowptr);
  bool SetZero();

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

 public:
  CMatrixSquareSparse mat;
  int* m_diaInd;
};

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
