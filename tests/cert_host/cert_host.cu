// Host build of the FP32 continuous-collision certificates (cert.cuh) for the
// CPU tests: the same float arithmetic as the device (round to nearest, no
// contraction), with the outward-rounded bounds one ulp wider, and the same
// hi/lo split of positions and displacements as the device's k_ccd_split.
#include "cert.cuh"

namespace {
// point k of a configuration: start position p and end position e, split as
// the device splits x and e - x
cs::PS split(const double* a, int k) {
  cs::PS s;
  for (int c = 0; c < 3; c++) {
    const double p = a[3 * k + c], e = a[12 + 3 * k + c];
    const double d = e - p;
    s.ph[c] = (float)p;
    s.pl[c] = (float)(p - (double)s.ph[c]);
    s.dh[c] = (float)d;
    s.dl[c] = (float)(d - (double)s.dh[c]);
  }
  return s;
}
}  // namespace

// configurations of 24 doubles (start points, then end points); 1 where the
// certificate proves the reference's test rejects
extern "C" void cert_fv_batch(int n, const double* p, int* out) {
  for (int i = 0; i < n; i++) {
    const double* a = p + 24 * (size_t)i;
    out[i] = cs::fv_ccd_cert32(split(a, 0), split(a, 1), split(a, 2), split(a, 3));
  }
}

extern "C" void cert_ee_batch(int n, const double* p, int* out) {
  for (int i = 0; i < n; i++) {
    const double* a = p + 24 * (size_t)i;
    out[i] = cs::ee_ccd_cert32(split(a, 0), split(a, 1), split(a, 2), split(a, 3));
  }
}
