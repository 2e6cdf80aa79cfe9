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

}  // extern "C"

// the same fluxes through their two halves (one face state each, then the combination)
template <int N, int AX>
static void split_flux(int family, const double *qL, const double *qR, double param, double *F) {
  pda::FluxSide<N> L, R;
  if constexpr (N == 3) {
    if (family == 0) {
      pda::euler3_side(L, qL, param);
      pda::euler3_side(R, qR, param);
      pda::euler3_combine(F, qL, qR, L, R, param);
    } else {
      pda::swe_side<AX>(L, qL, param);
      pda::swe_side<AX>(R, qR, param);
      pda::swe_combine<AX>(F, qL, qR, L, R, param);
    }
  } else if constexpr (N == 4) {
    pda::euler4_side<AX>(L, qL, param);
    pda::euler4_side<AX>(R, qR, param);
    pda::euler4_combine<AX>(F, qL, qR, L, R, param);
  } else {
    pda::euler5_side<AX>(L, qL, param);
    pda::euler5_side<AX>(R, qR, param);
    pda::euler5_combine<AX>(F, qL, qR, L, R, param);
  }
}
extern "C" {
void pdn_point_flux_split(int family, int ax, const double *qL, const double *qR, double param, double *F) {
  if (family == 0) split_flux<3, 0>(family, qL, qR, param, F);
  else if (family == 1) (ax == 0 ? split_flux<4, 0> : split_flux<4, 1>)(family, qL, qR, param, F);
  else if (family == 2) (ax == 0 ? split_flux<5, 0> : ax == 1 ? split_flux<5, 1> : split_flux<5, 2>)(family, qL, qR, param, F);
  else (ax == 0 ? split_flux<3, 0> : split_flux<3, 1>)(family, qL, qR, param, F);
}
}
