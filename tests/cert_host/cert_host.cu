// Host build of the FP32 continuous-collision certificates (cert.cuh) for the
// CPU tests: the same float arithmetic as the device (round to nearest, no
// contraction), with the outward-rounded bounds one ulp wider.
#include "cert.cuh"

using cs::V3;

namespace {
V3<double> pt(const double* a, int k) { return cs::mk<double>(a[3 * k], a[3 * k + 1], a[3 * k + 2]); }

// x_i = p_i - p0 at the start and v_i = (e_i - e0) - x_i, as FindCoplanerInterp forms them
void diffs(const double* a, V3<double> x[3], V3<double> v[3]) {
  const V3<double> s0 = pt(a, 0), e0 = pt(a, 4);
  for (int i = 0; i < 3; i++) {
    x[i] = pt(a, 1 + i) - s0;
    v[i] = (pt(a, 5 + i) - e0) - x[i];
  }
}
}  // namespace

// configurations of 24 doubles (start points, then end points); 1 where the
// certificate proves the reference's test rejects
extern "C" void cert_fv_batch(int n, const double* p, int* out) {
  for (int i = 0; i < n; i++) {
    V3<double> x[3], v[3];
    diffs(p + 24 * (size_t)i, x, v);
    out[i] = cs::fv_ccd_cert32(x[0], x[1], x[2], v[0], v[1], v[2]);
  }
}

extern "C" void cert_ee_batch(int n, const double* p, int* out) {
  for (int i = 0; i < n; i++) {
    V3<double> x[3], v[3];
    diffs(p + 24 * (size_t)i, x, v);
    out[i] = cs::ee_ccd_cert32(x[0], x[1], x[2], v[0], v[1], v[2]);
  }
}
