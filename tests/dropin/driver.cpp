// driver.cpp -- a headless self_contact_sparse-style driver written against the
// reference's API (the init of self_contact_sparse/main.cpp:563-583 and its StepTime,
// main.cpp:213-263), compiled against the GPU drop-in headers.  Used by
// tests/test_gpu_dropin.py: reads a scene, runs N frames, writes x and v.
//
//   driver <scene.bin> <nframes> <out.bin>
#include <cstdio>
#include <cstdlib>
#include <cmath>
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

int main(int argc, char** argv) {
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
