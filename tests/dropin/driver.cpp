// driver.cpp -- a headless self_contact_sparse-style driver written against the
// reference's API (the init of self_contact_sparse/main.cpp:563-583 and its StepTime,
// main.cpp:213-263), compiled against the GPU drop-in headers.  Used by
// tests/test_gpu_dropin.py: reads a scene, runs N frames, writes x and v; or, in
// the `lower` mode, calls the lower-level functions of the reference's headers
// (BVH refits and contact searches, distances, the coplanarity time, the sparse
// matrix, CG, ILU(0) and PCG) on a given state and writes every result.
//
//   driver <scene.bin> <nframes> <out.bin>
//   driver lower <scene.bin> <state.bin> <out.bin>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <set>
#include <string>
#include <vector>

#include "self_collision_cloth.h"
#include "solve_internal_sparse.h"

static double g_center[3], g_radius;

static void penetration_solid_sphere(double& pd, double* n, const double* p) {
  n[0] = p[0] - g_center[0];
  n[1] = p[1] - g_center[1];
  n[2] = p[2] - g_center[2];
  const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  n[0] /= len;
  n[1] /= len;
  n[2] /= len;
  pd = g_radius - len;
}

template <typename T>
static std::vector<T> read_vec(FILE* f) {
  long long n = 0;
  if (fread(&n, sizeof(n), 1, f) != 1) exit(2);
  std::vector<T> v((size_t)n);
  if (n && fread(v.data(), sizeof(T), (size_t)n, f) != (size_t)n) exit(2);
  return v;
}

template <typename T>
static void write_vec(FILE* f, const std::vector<T>& v) {
  const long long n = (long long)v.size();
  fwrite(&n, sizeof(n), 1, f);
  if (n) fwrite(v.data(), sizeof(T), v.size(), f);
}

static std::vector<double> boxes_of(const std::vector<CAABB3D>& bb) {
  std::vector<double> o;
  for (const CAABB3D& b : bb) {
    const double r[7] = {b.x_min, b.x_max, b.y_min, b.y_max, b.z_min, b.z_max, b.isnt_empty ? 1.0 : 0.0};
    o.insert(o.end(), r, r + 7);
  }
  return o;
}

static std::vector<int> list_of(const std::set<CContactElement>& s) {
  std::vector<int> o;
  for (const CContactElement& e : s) {
    const int r[5] = {e.is_fv ? 1 : 0, e.ino0, e.ino1, e.ino2, e.ino3};
    o.insert(o.end(), r, r + 5);
  }
  return o;
}

static CVector3D pt(const std::vector<double>& a, size_t k) { return CVector3D(a[3 * k], a[3 * k + 1], a[3 * k + 2]); }

// the lower-level functions of bvh_aabb.h, matrix_square_sparse.h and ilu_sparse.h
static int lower(const char* scene_path, const char* state_path, const char* out_path) {
  FILE* f = fopen(scene_path, "rb");
  if (!f) return 1;
  std::vector<double> aXYZ0 = read_vec<double>(f);
  std::vector<int> aTri = read_vec<int>(f), aQuad = read_vec<int>(f);
  std::vector<double> prm = read_vec<double>(f);
  fclose(f);
  f = fopen(state_path, "rb");
  if (!f) return 1;
  std::vector<double> x = read_vec<double>(f), v = read_vec<double>(f), vdia = read_vec<double>(f),
                      vcrs = read_vec<double>(f), b = read_vec<double>(f), geo = read_vec<double>(f),
                      geo_e = read_vec<double>(f);
  fclose(f);
  const double dt = prm[0], lambda = prm[1], myu = prm[2], stiff_bend = prm[3];
  const double gravity[3] = {prm[4], prm[5], prm[6]};
  const double mass_point = prm[7], stiff_contact = prm[8], delta = prm[9];
  g_center[0] = prm[10];
  g_center[1] = prm[11];
  g_center[2] = prm[12];
  g_radius = prm[13];
  ClothGpuRegisterObstacle(penetration_solid_sphere, 2, g_center, g_radius);
  const int np = (int)aXYZ0.size() / 3;
  std::vector<int> aBCFlag(np, 0);
  std::vector<CNodeBVH> aNodeBVH;
  std::vector<CAABB3D> aBB;
  const int iroot = MakeBVHTopology_TopDown(aTri, aXYZ0, aNodeBVH);
  CMatrixSquareSparse mat_A;
  mat_A.Initialize(np, 3);
  CJaggedArray crs;
  crs.SetEdgeOfElem(aQuad, (int)aQuad.size() / 4, 4, np, false);
  crs.Sort();
  mat_A.SetPattern(crs.index, crs.array);
  CPreconditionerILU ilu_A;
  ilu_A.Initialize_ILU0(mat_A);
  {
    // one implicit step on copies admits the cloth and names mat_A / ilu_A
    std::vector<double> xc = aXYZ0, vc(aXYZ0.size(), 0.0);
    StepTime_InternalDynamicsILU(xc, vc, mat_A, ilu_A, aXYZ0, aBCFlag, aTri, aQuad, dt, lambda, myu, stiff_bend,
                                 gravity, mass_point, stiff_contact, delta, penetration_solid_sphere);
  }
  FILE* o = fopen(out_path, "wb");
  // BVH refits and contact searches
  BuildBoundingBoxChild_Prx(iroot, delta, x, aTri, aNodeBVH, aBB);
  write_vec(o, boxes_of(aBB));
  std::set<CContactElement> prx;
  GetContactElement_Proximity(prx, delta, x, aTri, iroot, aNodeBVH, aBB);
  write_vec(o, list_of(prx));
  BuildBoundingBoxChild_CCD(iroot, dt, x, v, aTri, aNodeBVH, aBB);
  write_vec(o, boxes_of(aBB));
  std::set<CContactElement> ccd;
  GetContactElement_CCD(ccd, dt, delta, x, v, aTri, iroot, aNodeBVH, aBB);
  write_vec(o, list_of(ccd));
  // the matrix: caller values, MatVec, Solve_CG, DoILUDecomp, Solve, Solve_PCG
  std::copy(vdia.begin(), vdia.end(), mat_A.m_valDia);
  std::copy(vcrs.begin(), vcrs.end(), mat_A.m_valCrs);
  std::vector<double> y1 = v, y2 = v;
  mat_A.MatVec(1.0, x, 0.0, y1);
  mat_A.MatVec(0.5, x, 2.0, y2);
  write_vec(o, y1);
  write_vec(o, y2);
  for (int maxit : {1000, 5}) {
    double conv = 1.0e-6;
    int iter = maxit;
    std::vector<double> r = b, u;
    Solve_CG(conv, iter, mat_A, r, u);
    write_vec(o, u);
    write_vec(o, r);
    write_vec(o, std::vector<double>{conv, (double)iter});
  }
  ilu_A.SetValueILU(mat_A);
  ilu_A.DoILUDecomp();
  write_vec(o, std::vector<double>(ilu_A.mat.m_valDia, ilu_A.mat.m_valDia + 9 * (size_t)np));
  write_vec(o, std::vector<double>(ilu_A.mat.m_valCrs, ilu_A.mat.m_valCrs + 9 * (size_t)ilu_A.mat.m_ncrs));
  std::vector<double> z = b;
  ilu_A.Solve(z);
  write_vec(o, z);
  {
    double conv = 1.0e-6;
    int iter = 100;
    std::vector<double> r = b, u;
    Solve_PCG(conv, iter, mat_A, ilu_A, r, u);
    write_vec(o, u);
    write_vec(o, r);
    write_vec(o, std::vector<double>{conv, (double)iter});
  }
  // Mearge and SetBoundaryCondition on a second matrix of the same pattern
  CMatrixSquareSparse mat_B;
  mat_B.Initialize(np, 3);
  mat_B.SetPattern(crs.index, crs.array);
  mat_B.SetZero();
  std::vector<int> buf(np, -1);
  const int nq = (int)aQuad.size() / 4;
  for (int q = 0; q < nq; q += 3) {
    double emat[16 * 9];
    for (int k = 0; k < 16 * 9; k++) emat[k] = 0.001 * (double)((q * 131 + k * 17) % 97) - 0.05;
    mat_B.Mearge(4, &aQuad[4 * q], 4, &aQuad[4 * q], 9, emat, buf);
  }
  std::vector<int> bc(np, 0);
  for (int i = 0; i < np; i += 7) bc[i] = 1;
  mat_B.SetBoundaryCondition(bc);
  write_vec(o, std::vector<double>(mat_B.m_valDia, mat_B.m_valDia + 9 * (size_t)np));
  write_vec(o, std::vector<double>(mat_B.m_valCrs, mat_B.m_valCrs + 9 * (size_t)mat_B.m_ncrs));
  // distances and the coplanarity time on probe points (4 points each)
  std::vector<double> geo_out;
  for (size_t g = 0; g + 12 <= geo.size(); g += 12) {
    const size_t k = g / 3;
    double w0, w1, rp, rq;
    const double dfv = DistanceFaceVertex(pt(geo, k), pt(geo, k + 1), pt(geo, k + 2), pt(geo, k + 3), w0, w1);
    const double dee = DistanceEdgeEdge(pt(geo, k), pt(geo, k + 1), pt(geo, k + 2), pt(geo, k + 3), rp, rq);
    const double t = FindCoplanerInterp(pt(geo, k), pt(geo, k + 1), pt(geo, k + 2), pt(geo, k + 3), pt(geo_e, k),
                                        pt(geo_e, k + 1), pt(geo_e, k + 2), pt(geo_e, k + 3));
    const double r[7] = {dfv, w0, w1, dee, rp, rq, t};
    geo_out.insert(geo_out.end(), r, r + 7);
  }
  write_vec(o, geo_out);
  fclose(o);
  if (ClothGpuLastStatus() != 0) {
    fprintf(stderr, "lower: %s\n", ClothGpuLastError());
    return 3;
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 5 && std::string(argv[1]) == "lower") return lower(argv[2], argv[3], argv[4]);
  if (argc < 4) return 1;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 1;
  std::vector<double> aXYZ0 = read_vec<double>(f);
  std::vector<int> aTri = read_vec<int>(f), aQuad = read_vec<int>(f);
  std::vector<double> prm = read_vec<double>(f);  // dt lambda myu bend gx gy gz mass k clearance cx cy cz r solver
  fclose(f);
  const double dt = prm[0], lambda = prm[1], myu = prm[2], stiff_bend = prm[3];
  const double gravity[3] = {prm[4], prm[5], prm[6]};
  const double mass_point = prm[7], stiff_contact = prm[8], contact_clearance = prm[9];
  g_center[0] = prm[10];
  g_center[1] = prm[11];
  g_center[2] = prm[12];
  g_radius = prm[13];
  const bool use_cg = prm[14] != 0;
  ClothGpuRegisterObstacle(penetration_solid_sphere, 2, g_center, g_radius);

  // init (self_contact_sparse/main.cpp:563-583)
  const int np = (int)aXYZ0.size() / 3;
  std::vector<double> aXYZ = aXYZ0, aUVW(aXYZ0.size(), 0.0);
  std::vector<int> aBCFlag(np, 0);
  std::vector<CNodeBVH> aNodeBVH;
  std::vector<CAABB3D> aBB;
  const int iroot_bvh = MakeBVHTopology_TopDown(aTri, aXYZ, aNodeBVH);
  CJaggedArray aEdge;
  aEdge.SetEdgeOfElem(aTri, (int)aTri.size() / 3, 3, np, false);
  CMatrixSquareSparse mat_A;
  mat_A.Initialize(np, 3);
  CJaggedArray crs;
  crs.SetEdgeOfElem(aQuad, (int)aQuad.size() / 4, 4, np, false);
  crs.Sort();
  mat_A.SetPattern(crs.index, crs.array);
  CPreconditionerILU ilu_A;
  ilu_A.Initialize_ILU0(mat_A);

  const int nframes = atoi(argv[2]);
  for (int frame = 0; frame < nframes; frame++) {
    // StepTime (self_contact_sparse/main.cpp:213-263)
    std::vector<double> aXYZ1 = aXYZ;
    if (use_cg)
      StepTime_InternalDynamics(aXYZ, aUVW, mat_A, aXYZ0, aBCFlag, aTri, aQuad, dt, lambda, myu, stiff_bend, gravity,
                                mass_point, stiff_contact, contact_clearance, penetration_solid_sphere);
    else
      StepTime_InternalDynamicsILU(aXYZ, aUVW, mat_A, ilu_A, aXYZ0, aBCFlag, aTri, aQuad, dt, lambda, myu, stiff_bend,
                                   gravity, mass_point, stiff_contact, contact_clearance, penetration_solid_sphere);
    bool is_impulse_applied = false;
    GetIntermidiateVelocityContactResolved(aUVW, is_impulse_applied, dt, contact_clearance, mass_point, stiff_contact,
                                           aXYZ1, aTri, aEdge, iroot_bvh, aNodeBVH, aBB);
    if (is_impulse_applied) {
      for (size_t ip = 0; ip < aXYZ.size() / 3; ip++)
        for (int k = 0; k < 3; k++) aXYZ[ip * 3 + k] = aXYZ1[ip * 3 + k] + aUVW[ip * 3 + k] * dt;
      UpdateIntermidiateVelocity(aUVW, aXYZ, aXYZ0, aBCFlag, aTri, aQuad, dt, lambda, myu, stiff_bend, gravity,
                                 mass_point);
    }
    if (ClothGpuLastStatus() != 0) {
      fprintf(stderr, "frame %d: %s\n", frame, ClothGpuLastError());
      return 3;
    }
  }
  FILE* o = fopen(argv[3], "wb");
  fwrite(aXYZ.data(), sizeof(double), aXYZ.size(), o);
  fwrite(aUVW.data(), sizeof(double), aUVW.size(), o);
  fclose(o);
  return 0;
}
