// Host build of the library's point-wise device numerics
// (pressio-demoapps_gb300/csrc/numerics.cuh) for CPU comparison against the
// oracle.  Compiled by tests/test_numerics_host.py with -ffp-contract=off.
#include "numerics.cuh"

extern "C" {
void pdn_weno5_face(const double *q, double *u) { pda::weno5_face(u[0], u[1], q[0], q[1], q[2], q[3], q[4], q[5]); }
void pdn_weno3_face(const double *q, double *u) { pda::weno3_face(u[0], u[1], q[0], q[1], q[2], q[3]); }
void pdn_weno5_face_grad(const double *q, double *u, double *gN, double *gP) {
  pda::weno5_face_grad(u[0], u[1], gN, gP, q[0], q[1], q[2], q[3], q[4], q[5]);
}
void pdn_weno3_face_grad(const double *q, double *u, double *gN, double *gP) {
  pda::weno3_face_grad(u[0], u[1], gN, gP, q[0], q[1], q[2], q[3]);
}
void pdn_point_flux(int family, int ax, const double *qL, const double *qR, double param, double *F, double *JL,
                    double *JR) {
  if (family == 0) {
    pda::euler3_flux(F, qL, qR, param);
    pda::euler3_flux_jac(JL, JR, qL, qR, param);
  } else if (family == 1) {
    if (ax == 0) { pda::euler4_flux<0>(F, qL, qR, param); pda::euler4_flux_jac<0>(JL, JR, qL, qR, param); }
    else { pda::euler4_flux<1>(F, qL, qR, param); pda::euler4_flux_jac<1>(JL, JR, qL, qR, param); }
  } else if (family == 2) {
    if (ax == 0) { pda::euler5_flux<0>(F, qL, qR, param); pda::euler5_flux_jac<0>(JL, JR, qL, qR, param); }
    else if (ax == 1) { pda::euler5_flux<1>(F, qL, qR, param); pda::euler5_flux_jac<1>(JL, JR, qL, qR, param); }
    else { pda::euler5_flux<2>(F, qL, qR, param); pda::euler5_flux_jac<2>(JL, JR, qL, qR, param); }
  } else {
    if (ax == 0) { pda::swe_flux<0>(F, qL, qR, param); pda::swe_flux_jac<0>(JL, JR, qL, qR, param); }
    else { pda::swe_flux<1>(F, qL, qR, param); pda::swe_flux_jac<1>(JL, JR, qL, qR, param); }
  }
}
}
