// Device problem object: parameters, initial conditions, boundary stencil
// tables, the CSR pattern, kernel dispatch, steppers and the C ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "problem_impl.hpp"

namespace pda {

static thread_local std::string g_last_error;
void set_last_error(const std::string &m) { g_last_error = m; }

}  // namespace pda

namespace pda {
namespace {

// ---------------------------------------------------------------- params
constexpr int kInvalid = -1;

// impl/euler_2d_parametrization_helpers.hpp:60-160
int euler2d_ic_index(int probEn, int icFlag, const std::string &s) {
  if (probEn == 5 /*NormalShock*/ && icFlag == 1 && s == "mach") return 0;
  if (probEn == 7 /*CrossShock*/ && icFlag == 1) {
    if (s == "crossShockDensity") return 1;
    if (s == "crossShockInletXVel") return 2;
    if (s == "crossShockBottomYVel") return 3;
  }
  if (probEn == 4 /*Riemann*/) {
    if (icFlag == 1 && s == "riemannTopRightPressure") return 4;
    if (icFlag == 2) {
      if (s == "riemannTopRightPressure") return 5;
      if (s == "riemannTopRightXVel") return 6;
      if (s == "riemannTopRightYVel") return 7;
      if (s == "riemannTopRightDensity") return 8;
      if (s == "riemannBotLeftPressure") return 9;
    }
  }
  return kInvalid;
}

// impl/swe_2d_parametrization_helpers.hpp:104-128
int swe_ic_index(int icFlag, const std::string &s) {
  if (icFlag == 1) {
    if (s == "pulseMagnitude") return 0;
    if (s == "pulseX") return 1;
    if (s == "pulseY") return 2;
  } else if (icFlag == 2) {
    if (s == "pulseMagnitude1") return 3;
    if (s == "pulseX1") return 4;
    if (s == "pulseY1") return 5;
    if (s == "pulseMagnitude2") return 6;
    if (s == "pulseX2") return 7;
    if (s == "pulseY2") return 8;
  }
  return kInvalid;
}

// -------------------------------------------------------- initial conditions
double energy2(double gm1inv, const double *prim, int n) {
  // euler_compute_energy.hpp:55-110 (prim[last] = p)
  constexpr double half = 1. / 2.;
  if (n == 3) {
    const double usq = prim[1] * prim[1];
    return prim[2] * gm1inv + half * prim[0] * (usq);
  }
  if (n == 4) {
    const double usq = prim[1] * prim[1], vsq = prim[2] * prim[2];
    return prim[3] * gm1inv + half * prim[0] * (usq + vsq);
  }
  const double usq = prim[1] * prim[1], vsq = prim[2] * prim[2], wsq = prim[3] * prim[3];
  return prim[4] * gm1inv + half * prim[0] * (usq + vsq + wsq);
}

// Post-shock primitive state {rho, u, v, p} behind a shock of Mach number
// `mach` moving into gas at rest, the shock normal at `angle` from the x axis
// (computePostShockConditionsFromPreshockAtRest over the normal-shock
// relations, impl/euler_rankine_hugoniot.hpp:55-145).
void post_shock_at_rest(const double pre[4], double angle, double mach, double gamma, double post[4]) {
  const double one = 1., two = 2.;
  const double sinA = std::sin(angle), cosA = std::cos(angle);
  const double rhoPre = pre[0], velPre = 0., pPre = pre[3];
  const double machShockSq = mach * mach;
  const double rhoPost = rhoPre * (gamma + one) * machShockSq / (two + (gamma - one) * machShockSq);
  const double pPost = pPre * (one + two * gamma / (gamma + one) * (machShockSq - one));
  const double aPre = std::sqrt(gamma * pPre / rhoPre);
  const double aPost = std::sqrt(gamma * pPost / rhoPost);
  const double half = one / two;
  const double num = (one + half * (gamma - one) * machShockSq);
  const double den = gamma * machShockSq - half * (gamma - one);
  const double machRelPost = std::sqrt(num / den);
  const double velPost = machRelPost * aPost - mach * aPre + velPre;
  post[0] = rhoPost;
  post[1] = -velPost * cosA;
  post[2] = -velPost * sinA;
  post[3] = pPost;
}

void initial_condition(const pda_problem &P, std::vector<double> &st) {
  const Mesh &m = *P.mesh;
  const int64_t N = m.stencilMeshSize;
  st.assign((size_t)N * P.ndpc, 0.0);
  const double *x = m.x.data(), *y = m.y.data(), *z = m.z.data();
  if (P.family == PDA_EULER1D) {
    // impl/euler_1d_initial_condition.hpp
    const double gamma = P.phys.gamma;
    const double gm1inv = 1. / (gamma - 1.);
    double prim[3] = {0, 0, 0};
    for (int64_t i = 0; i < N; ++i) {
      if (P.probEnum == 0) {
        prim[0] = 1. + 0.2 * std::sin(M_PI * x[i]);
        prim[1] = 1.;
        prim[2] = 1.;
      } else if (P.probEnum == 1) {
        if (x[i] <= 0.) { prim[0] = 1.; prim[1] = 0.; prim[2] = 1.; }
        if (x[i] > 0.) { prim[0] = 0.125; prim[1] = 0.; prim[2] = 0.1; }
      } else if (P.probEnum == 2) {
        if (x[i] <= 0.) { prim[0] = 0.445; prim[1] = 0.698; prim[2] = 3.528; }
        else if (x[i] > 0.) { prim[0] = 0.5; prim[1] = 0.; prim[2] = 0.571; }
      } else {
        if (x[i] <= -4.) { prim[0] = 27. / 7.; prim[1] = 2.629369; prim[2] = 31. / 3.; }
        else { prim[0] = 1. + (1. / 5.) * std::sin(5. * x[i]); prim[1] = 0.; prim[2] = 1.; }
      }
      st[i * 3] = prim[0];
      st[i * 3 + 1] = prim[0] * prim[1];
      st[i * 3 + 2] = energy2(gm1inv, prim, 3);
    }
  } else if (P.family == PDA_EULER2D) {
    const double gamma = P.phys.gamma;
    const double gm1inv = 1. / (gamma - 1.);
    double prim[4] = {0, 0, 0, 0};
    if (P.probEnum == 0) {
      // sin2dEulerIC (impl/euler_2d_initial_condition.hpp:57-83)
      for (int64_t i = 0; i < N; ++i) {
        prim[0] = 1. + (1. / 5.) * std::sin(M_PI * (x[i] + y[i]));
        prim[1] = prim[2] = prim[3] = 1.;
        st[i * 4] = prim[0];
        st[i * 4 + 1] = prim[0] * prim[1];
        st[i * 4 + 2] = prim[0] * prim[2];
        st[i * 4 + 3] = energy2(gm1inv, prim, 4);
      }
    } else if (P.probEnum == 4 && P.icFlag == 1) {
      // riemann2dIC1 (:256-297)
      const double pTR = P.icParams[4];
      const double x0 = 1. / 2., y0 = 1. / 2.;
      for (int64_t i = 0; i < N; ++i) {
        if (x[i] >= x0 && y[i] >= y0) { prim[0] = 0.5313; prim[1] = 0.; prim[2] = 0.; prim[3] = pTR; }
        else if (x[i] < x0 && y[i] >= y0) { prim[0] = 1.; prim[1] = 0.7276; prim[2] = 0.; prim[3] = 1.; }
        else if (x[i] < x0 && y[i] < y0) { prim[0] = 0.8; prim[1] = 0.; prim[2] = 0.; prim[3] = 1.; }
        else if (x[i] > x0 && y[i] < y0) { prim[0] = 1.; prim[1] = 0.; prim[2] = 0.7276; prim[3] = 1.; }
        st[i * 4] = prim[0];
        st[i * 4 + 1] = prim[0] * prim[1];
        st[i * 4 + 2] = prim[0] * prim[2];
        st[i * 4 + 3] = energy2(gm1inv, prim, 4);
      }
    } else if (P.probEnum == 4 && P.icFlag == 2) {
      // riemann2dIC2 (:309-380): unspecified quadrants from the compatibility relations
      const double topRightPressure = P.icParams[5], topRightXVel = P.icParams[6],
                   topRightYVel = P.icParams[7], topRightDensity = P.icParams[8],
                   botLeftPressure = P.icParams[9];
      PDA_REQUIRE(!(topRightPressure <= botLeftPressure), PDA_ERR_INVALID_ARGUMENT,
                  "INVALID: riemannTopRightPressure <= riemannBotLeftPressure");
      const double one = 1., two = 2., four = 4.;
      const double x0 = 0.8, y0 = 0.8;
      const double eps = (gamma - one) / (gamma + one);
      const double fac13 = topRightPressure / botLeftPressure;
      const double fac43 = (one / (two * (one + two * eps))) *
                           (eps * (fac13 + one) +
                            std::sqrt(std::pow(eps * (fac13 + one), 2) + four * (one + two * eps) * fac13));
      const double topLeftPressure = fac43 * botLeftPressure;
      const double botRightPressure = topLeftPressure;
      const double topLeftYVel = topRightYVel;
      const double botRightXVel = topRightXVel;
      const double topLeftDensity = topRightDensity * (topLeftPressure / topRightPressure + eps) /
                                    (1 + eps * topLeftPressure / topRightDensity);
      const double botRightDensity = topLeftDensity;
      const double psi21_sq = (topLeftPressure - topRightPressure) * (topLeftDensity - topRightDensity) /
                              (topLeftDensity * topRightDensity);
      const double topLeftXVel = std::sqrt(psi21_sq) + topRightXVel;
      const double psi41_sq = (botRightPressure - topRightPressure) * (botRightDensity - topRightDensity) /
                              (botRightDensity * topRightDensity);
      const double botRightYVel = std::sqrt(psi41_sq) + topRightYVel;
      const double botLeftXVel = topLeftXVel;
      const double botLeftYVel = botRightYVel;
      const double botLeftDensity = topLeftDensity * (botLeftPressure - topLeftPressure) /
                                    ((botLeftPressure - topLeftPressure) - psi41_sq * topLeftDensity);
      for (int64_t i = 0; i < N; ++i) {
        if (x[i] >= x0 && y[i] >= y0) {
          prim[0] = topRightDensity; prim[1] = topRightXVel; prim[2] = topRightYVel; prim[3] = topRightPressure;
        } else if (x[i] < x0 && y[i] >= y0) {
          prim[0] = topLeftDensity; prim[1] = topLeftXVel; prim[2] = topLeftYVel; prim[3] = topLeftPressure;
        } else if (x[i] < x0 && y[i] < y0) {
          prim[0] = botLeftDensity; prim[1] = botLeftXVel; prim[2] = botLeftYVel; prim[3] = botLeftPressure;
        } else if (x[i] > x0 && y[i] < y0) {
          prim[0] = botRightDensity; prim[1] = botRightXVel; prim[2] = botRightYVel; prim[3] = botRightPressure;
        }
        st[i * 4] = prim[0];
        st[i * 4 + 1] = prim[0] * prim[1];
        st[i * 4 + 2] = prim[0] * prim[2];
        st[i * 4 + 3] = energy2(gm1inv, prim, 4);
      }
    } else if (P.probEnum == 1) {
      // KelvinHelmholtzIC (impl/euler_2d_initial_condition.hpp:87-125)
      const double one = 1.;
      const double gammaMinusOne = gamma - one;
      for (int64_t i = 0; i < N; ++i) {
        const double freq = 4.;
        const double mag = 0.025;
        const double pert = mag * std::cos(2. * 3.14159265 / 10. * freq * x[i]);
        double *u = &st[i * 4];
        if (y[i] > -2 + pert && y[i] < 2 + pert) {
          u[0] = 2.;
          u[1] = u[0] * 0.5;
          u[2] = 0.;
        } else {
          u[0] = 1.;
          u[1] = -u[0] * 0.5;
          u[2] = 0.;
        }
        u[3] = 2.5 / (gammaMinusOne) + 0.5 / u[0] * (u[1] * u[1] + u[2] * u[2]);
      }
    } else if (P.probEnum == 2 || P.probEnum == 3) {
      // sedov2dIC / sedov2dsymmetryIC (impl/euler_2d_initial_condition.hpp:131-249)
      const double zero = 0., one = 1., two = 2.;
      const double dx = m.dx[0], dy = m.dx[1];
      const double gammaMinusOne = gamma - one;
      const double gammaMinusOneInv = one / gammaMinusOne;
      const bool sym = P.probEnum == 3;
      const double sRad = sym ? 3. * std::min(dx, dy) : two * std::min(dx, dy);
      for (int64_t i = 0; i < N; ++i) {
        const double diffx = x[i], diffy = y[i];
        const double myR = std::sqrt(diffx * diffx + diffy * diffy);
        prim[0] = one;
        prim[1] = zero;
        prim[2] = zero;
        if (myR <= sRad) prim[3] = sym ? gammaMinusOne * 0.851072 / (M_PI * sRad * sRad)
                                       : (gammaMinusOne) / (M_PI * sRad * sRad);
        else prim[3] = sym ? 2.5e-5 : 5.e-5;
        st[i * 4] = prim[0];
        st[i * 4 + 1] = prim[0] * prim[1];
        st[i * 4 + 2] = prim[0] * prim[2];
        st[i * 4 + 3] = energy2(gammaMinusOneInv, prim, 4);
      }
    } else if (P.probEnum == 5) {
      // normalShock2dIC (impl/euler_2d_initial_condition.hpp:391-436) with the
      // Rankine-Hugoniot relations of impl/euler_rankine_hugoniot.hpp:55-145
      const double zero = 0., one = 1., two = 2., six = 6.;
      const double angle = zero, xShock = one / six;
      const double gammaMinusOne = gamma - one, gammaMinusOneInv = one / gammaMinusOne;
      const double machShock = P.icParams[0];
      const double pre[4] = {gamma, zero, zero, one};
      double post[4];
      post_shock_at_rest(pre, angle, machShock, gamma, post);
      (void)two;
      for (int64_t i = 0; i < N; ++i) {
        const double *q = x[i] < xShock ? post : pre;
        st[i * 4] = q[0];
        st[i * 4 + 1] = q[0] * q[1];
        st[i * 4 + 2] = q[0] * q[2];
        st[i * 4 + 3] = energy2(gammaMinusOneInv, q, 4);
      }
    } else if (P.probEnum == 6) {
      // doubleMachReflection2dIC (impl/euler_2d_initial_condition.hpp:443-500)
      const double zero = 0., one = 1., six = 6.;
      const double xShockBottom = one / six, angle = M_PI / six;
      const double shockSlope = std::tan(angle);
      const double gammaMinusOneInv = one / (gamma - one);
      const double pre[4] = {gamma, zero, zero, one};
      double post[4];
      post_shock_at_rest(pre, -angle, 10., gamma, post);
      for (int64_t i = 0; i < N; ++i) {
        const double xShock = xShockBottom + shockSlope * y[i];
        const double *q = x[i] < xShock ? post : pre;
        st[i * 4] = q[0];
        st[i * 4 + 1] = q[0] * q[1];
        st[i * 4 + 2] = q[0] * q[2];
        st[i * 4 + 3] = energy2(gammaMinusOneInv, q, 4);
      }
    } else if (P.probEnum == 7) {
      // crossShockIC (impl/euler_2d_initial_condition.hpp:505-526)
      const double gammaMinusOneInv = 1. / (gamma - 1.);
      const double q[4] = {P.icParams[1], P.icParams[2], 0., 1.};
      for (int64_t i = 0; i < N; ++i) {
        st[i * 4] = q[0];
        st[i * 4 + 1] = q[0] * q[1];
        st[i * 4 + 2] = q[0] * q[2];
        st[i * 4 + 3] = energy2(gammaMinusOneInv, q, 4);
      }
    } else if (P.probEnum == 8) {
      // testingonlyneumann: no initial condition (zeros)
    } else {
      throw Error(PDA_ERR_UNSUPPORTED, "Euler2d: initial condition not available for this problem");
    }
  } else if (P.family == PDA_EULER3D && P.probEnum == 1) {
    // sedov3dInitialCondition (impl/euler_3d_initial_condition.hpp:87-141)
    const double gamma = P.phys.gamma;
    const double dx = m.dx[0], dy = m.dx[1], dz = m.dx[2];
    const double sRad = 3. * std::min(dx, std::min(dy, dz));
    const double gammaMinusOne = gamma - 1.;
    const double gammaMinusOneInv = 1. / gammaMinusOne;
    double prim[5];
    for (int64_t i = 0; i < N; ++i) {
      const double xsq = x[i] * x[i], ysq = y[i] * y[i], zsq = z[i] * z[i];
      const double myR = std::sqrt(xsq + ysq + zsq);
      prim[0] = 1.;
      prim[1] = prim[2] = prim[3] = 0.;
      prim[4] = myR <= sRad ? (3. * gammaMinusOne * 0.851072) / (4. * M_PI * sRad * sRad * sRad) : 2.5e-5;
      st[i * 5] = prim[0];
      st[i * 5 + 1] = prim[0] * prim[1];
      st[i * 5 + 2] = prim[0] * prim[2];
      st[i * 5 + 3] = prim[0] * prim[3];
      st[i * 5 + 4] = energy2(gammaMinusOneInv, prim, 5);
    }
  } else if (P.family == PDA_EULER3D) {
    // euler3dsmoothInitialCondition (impl/euler_3d_initial_condition.hpp:57-85)
    const double gamma = P.phys.gamma;
    const double gm1inv = 1. / (gamma - 1.);
    double prim[5];
    for (int64_t i = 0; i < N; ++i) {
      prim[0] = 1.0 + 0.2 * std::sin(M_PI * (x[i] + y[i] + z[i]));
      prim[1] = prim[2] = prim[3] = 1.0;
      prim[4] = 1.;
      st[i * 5] = prim[0];
      st[i * 5 + 1] = prim[0] * prim[1];
      st[i * 5 + 2] = prim[0] * prim[2];
      st[i * 5 + 3] = prim[0] * prim[3];
      st[i * 5 + 4] = energy2(gm1inv, prim, 5);
    }
  } else {
    // GaussianPulse / DoubleGaussianPulse (impl/swe_2d_initial_condition.hpp:55-106)
    const std::vector<double> &c = P.icParams;
    for (int64_t i = 0; i < N; ++i) {
      if (P.icFlag == 1) {
        const double dx1 = x[i] - c[1], dy1 = y[i] - c[2];
        const double r = std::sqrt(dx1 * dx1 + dy1 * dy1);
        st[i * 3] = 1. + c[0] * std::exp(-(r * r));
      } else {
        const double dx1 = x[i] - c[4], dy1 = y[i] - c[5];
        const double r1 = std::sqrt(dx1 * dx1 + dy1 * dy1);
        const double dx2 = x[i] - c[7], dy2 = y[i] - c[8];
        const double r2 = std::sqrt(dx2 * dx2 + dy2 * dy2);
        st[i * 3] = 1. + c[3] * std::exp(-(r1 * r1)) + c[6] * std::exp(-(r2 * r2));
      }
      st[i * 3 + 1] = 0.;
      st[i * 3 + 2] = 0.;
    }
  }
}

// ------------------------------------------------------- stencil tables
// graph column of the neighbour at distance k+1 on the minus / plus side of
// an axis (functor_reconstruct_from_state.hpp:257-262, :432-437, :614-619).
int col_minus(int dim, int ax, int k) {
  if (dim == 1) return 1 + 2 * k;
  if (dim == 2) return (ax == 0 ? 1 : 4) + 4 * k;
  return (ax == 0 ? 1 : ax == 1 ? 4 : 5) + 6 * k;
}
int col_plus(int dim, int ax, int k) {
  if (dim == 1) return 2 + 2 * k;
  if (dim == 2) return (ax == 0 ? 3 : 2) + 4 * k;
  return (ax == 0 ? 3 : ax == 1 ? 2 : 6) + 6 * k;
}

// Source cell of ghost layer L on one side of row r, following the ghost
// fillers: Ghost2dNeumannFiller (euler_2d_ghost_filler_neumann.hpp:101-276)
// and InviscidWallFiller (swe_2d_ghost_filler_inviscid_wall.hpp:99-278), which
// share the index rule, and Ghost1dNeumannFiller
// (euler_1d_ghost_filler.hpp:81-144), whose second and third layers copy the
// opposite-side neighbours also for the second cell from the wall.
int ghost_source(const Mesh &m, int bc, int64_t r, int ax, bool minusSide, int L) {
  auto same = [&](int k) {
    return m.g(r, minusSide ? col_minus(m.dim, ax, k) : col_plus(m.dim, ax, k));
  };
  auto opp = [&](int k) {
    return m.g(r, minusSide ? col_plus(m.dim, ax, k) : col_minus(m.dim, ax, k));
  };
  const int cell = m.g(r, 0);
  if (bc == BC_NEUMANN1D || bc == BC_SEDOVSYM || bc == BC_NORMALSHOCK || bc == BC_DMR || bc == BC_CROSSSHOCK) {
    // euler_1d_ghost_filler.hpp:104-142, euler_2d_ghost_filler_sedov2d_sym.hpp:87-206,
    // euler_2d_ghost_filler_normal_shock.hpp:87-205,
    // euler_2d_ghost_filler_double_mach_reflection.hpp:83-264,
    // euler_2d_ghost_filler_cross_shock.hpp:95-248
    if (L == 0) return cell;
    return opp(L - 1);
  }
  if (bc == BC_MIRROR2D) {
    if (L == 0) return cell;
    if (L == 1) return same(0) == -1 ? opp(0) : same(0);
    const int m0 = same(0), m1 = same(1);
    int ind = cell;
    if (m1 != -1 && m0 != -1) ind = m1;
    if (m1 == -1 && m0 != -1) ind = cell;
    if (m1 == -1 && m0 == -1) ind = opp(1);
    return ind;
  }
  throw Error(PDA_ERR_UNSUPPORTED, "this problem has no ghost-cell rule for meshes with boundaries");
}

// Ghost recipe ids: 0 copies the source cell, 1 negates the face-normal
// momentum (the mesh args' reflect dof), r >= 2 is the problem's recipe r - 2.
constexpr uint8_t kCopy = 0, kReflect = 1;
// double Mach reflection: the moving shock on the top boundary
constexpr uint8_t kDmrShock = 2;
// cross shock: inflow state on the left; bottom layer 0 (cell's density and
// energy) and layers >= 1 (prescribed density, the source's energy), each
// for x < 0.5 (no normal momentum) and x >= 0.5 (the bottom inflow momentum)
constexpr uint8_t kCsInflow = 2, kCsBottom0Lo = 3, kCsBottom0Hi = 4, kCsBottom1Lo = 5, kCsBottom1Hi = 6;
// wedge position of the double Mach reflection (1/6, as the reference writes it)
const double kDmrWedge = 1. / 6.;

// Recipe of ghost layer L on one side of row r: walls of the slip-wall
// problem on every side; the Sedov symmetry planes on the left and bottom;
// the normal-shock walls on the top and bottom; the double Mach reflection
// wall from the wedge on (euler_2d_ghost_filler_double_mach_reflection.hpp:
// 133-147) under the moving shock (:115-129); the cross-shock inflow states
// (euler_2d_ghost_filler_cross_shock.hpp:107-112, :133-147, :173-187).
uint8_t ghost_recipe(const pda_problem &P, int64_t r, int ax, bool minusSide, int L) {
  const Mesh &m = *P.mesh;
  switch (P.bc) {
    case BC_SEDOVSYM: return minusSide ? kReflect : kCopy;
    case BC_NORMALSHOCK: return ax == 1 ? kReflect : kCopy;
    case BC_DMR:
      if (ax == 0) return kCopy;
      if (!minusSide) return kDmrShock;
      return m.x[m.g(r, 0)] < kDmrWedge ? kCopy : kReflect;
    case BC_CROSSSHOCK: {
      if (ax == 0) return minusSide ? kCsInflow : kCopy;
      if (!minusSide) return kCopy;
      const bool lo = m.x[m.g(r, 0)] < 0.5;
      if (L == 0) return lo ? kCsBottom0Lo : kCsBottom0Hi;
      return lo ? kCsBottom1Lo : kCsBottom1Hi;
    }
    default: return kReflect;
  }
}

// whether the recipe reads its source cell (constant states and the moving
// shock do not)
bool recipe_reads_source(const pda_problem &P, uint8_t rid) {
  if (rid < 2) return true;
  const GhostRecipe &g = P.recipes[rid - 2];
  if (g.op[0] == 3) return false;
  for (int d = 0; d < P.ndpc; ++d)
    if (g.op[d] != 2) return true;
  return false;
}

// Source cell and recipe of one ghost entry; the ghost's position
// (cell x, cell y + (L + 1) dy: the points where the double Mach reflection
// filler evaluates the shock distance) when the table keeps positions.
void ghost_entry(const pda_problem &P, int64_t r, int ax, bool minusSide, int L, int *src, uint8_t *rid,
                 double *gx, double *gy) {
  const Mesh &m = *P.mesh;
  *rid = ghost_recipe(P, r, ax, minusSide, L);
  *src = m.g(r, 0);
  if (recipe_reads_source(P, *rid)) {
    *src = ghost_source(m, P.bc, r, ax, minusSide, L);
    PDA_REQUIRE(*src >= 0, PDA_ERR_INVALID_ARGUMENT, "mesh too small for the ghost layers of this scheme");
  }
  if (gx) {
    const int c = m.g(r, 0);
    *gx = m.x[c];
    *gy = m.y[c] + (L + 1.0) * m.dx[1];
  }
}

// Stencil of the scheme (positions -h..h) for every row of the table.
void build_stencil(const pda_problem &P, Table &T, const std::vector<int32_t> &rowList, bool allowGhost) {
  const Mesh &m = *P.mesh;
  const int S = 2 * P.h + 1, D = P.dim;
  T.rows.assign(rowList.begin(), rowList.end());
  T.cell.resize(rowList.size());
  T.src.assign(rowList.size() * D * S, 0);
  T.flip.assign(rowList.size() * D * S, 0);
  T.gsx.assign(P.timeDependent && allowGhost ? rowList.size() * D * S : 0, 0.);
  T.gsy.assign(T.gsx.size(), 0.);
  for (size_t e = 0; e < rowList.size(); ++e) {
    const int64_t r = rowList[e];
    T.cell[e] = m.g(r, 0);
    for (int ax = 0; ax < D; ++ax) {
      const size_t base = (e * D + ax) * S;
      T.src[base + P.h] = m.g(r, 0);
      for (int k = 1; k <= P.h; ++k) {
        for (int side = 0; side < 2; ++side) {
          const bool minus = side == 0;
          const int c = m.g(r, minus ? col_minus(D, ax, k - 1) : col_plus(D, ax, k - 1));
          const size_t pos = base + (minus ? P.h - k : P.h + k);
          if (c != -1) {
            T.src[pos] = c;
          } else {
            PDA_REQUIRE(allowGhost, PDA_ERR_INTERNAL, "unexpected boundary neighbour in an inner row");
            const bool pos_ = !T.gsx.empty();
            ghost_entry(P, r, ax, minus, k - 1, &T.src[pos], &T.flip[pos], pos_ ? &T.gsx[pos] : nullptr,
                        pos_ ? &T.gsy[pos] : nullptr);
          }
        }
      }
    }
  }
}

// ------------------------------------------------------------ CSR pattern
// initializeJacobian (euler_2d_prob_class.hpp:223-237, :314-387 and the
// 1d/3d/swe analogues): Eigen setFromTriplets + makeCompressed gives, per row,
// the sorted distinct columns.
void build_pattern(pda_problem &P) {
  if (P.patternBuilt) return;
  const Mesh &m = *P.mesh;
  const int nd = P.ndpc;
  const int nnbInner = 2 * P.dim * P.h;
  std::vector<char> isNear(m.sampleMeshSize, 0);
  for (int32_t r : m.nearBd) isNear[r] = 1;
  P.rowBlocks.assign(m.sampleMeshSize, {});
  int64_t nnz = 0;
  for (int64_t r = 0; r < m.sampleMeshSize; ++r) {
    std::vector<int32_t> &b = P.rowBlocks[r];
    b.push_back(m.g(r, 0));
    if (isNear[r]) {
      for (int i = 1; i <= 2 * P.dim; ++i)
        if (m.g(r, i) != -1) b.push_back(m.g(r, i));
    } else {
      for (int i = 1; i <= nnbInner; ++i) b.push_back(m.g(r, i));
    }
    std::sort(b.begin(), b.end());
    b.erase(std::unique(b.begin(), b.end()), b.end());
    nnz += (int64_t)b.size() * nd * nd;
  }
  PDA_REQUIRE(nnz < INT32_MAX, PDA_ERR_UNSUPPORTED, "Jacobian has more than 2^31-1 entries (int32 CSR)");
  P.rowptr.assign((size_t)m.sampleMeshSize * nd + 1, 0);
  P.colidx.resize((size_t)nnz);
  int64_t q = 0;
  for (int64_t r = 0; r < m.sampleMeshSize; ++r) {
    const std::vector<int32_t> &b = P.rowBlocks[r];
    for (int k = 0; k < nd; ++k) {
      P.rowptr[(size_t)r * nd + k] = (int)q;
      for (int32_t c : b)
        for (int j = 0; j < nd; ++j) P.colidx[q++] = c * nd + j;
    }
  }
  P.rowptr[(size_t)m.sampleMeshSize * nd] = (int)q;
  P.patternBuilt = true;
}

void pattern_to_device(pda_problem &P) {
  build_pattern(P);
  if (P.d_rowptr.p && P.d_rowptr.n == P.rowptr.size()) return;
  P.d_rowptr.upload(P.rowptr);
  P.d_colidx.upload(P.colidx);
}

int block_offset(const pda_problem &P, int64_t r, int32_t cell) {
  const std::vector<int32_t> &b = P.rowBlocks[r];
  auto it = std::lower_bound(b.begin(), b.end(), cell);
  if (it == b.end() || *it != cell) throw Error(PDA_ERR_INTERNAL, "cell missing from CSR row pattern");
  return (int)(it - b.begin()) * P.ndpc;
}

// BC factors of fillJacFactorsForCellBd (euler_2d_prob_class.hpp:1115-1129,
// swe_2d_prob_class.hpp:839-854; 1d all ones, euler_1d_prob_class.hpp:608-610)
void jac_factors(const pda_problem &P, int64_t r, int ax, double *f) {
  for (int j = 0; j < P.ndpc; ++j) f[j] = 1.;
  if (P.family == PDA_SWE2D) f[ax == 0 ? 1 : 2] = -1.;
  if (P.bc == BC_SEDOVSYM) {
    // euler_2d_prob_class.hpp:1129-1148, euler_3d_prob_class.hpp:626-666 with
    // findCellBdType (:1017-1043): reflective factors on the axis of a left /
    // back / bottom boundary, Neumann otherwise
    const Mesh &m = *P.mesh;
    if (m.g(r, col_minus(P.dim, ax, 0)) == -1) f[1 + ax] = -1.;
  }
  // euler_2d_prob_class.hpp:1150-1162: reflective along y, Neumann along x
  if (P.bc == BC_NORMALSHOCK && ax == 1) f[2] = -1.;
  if (P.bc == BC_DMR && ax == 1) {
    // euler_2d_prob_class.hpp:1164-1193: Neumann along x; along y Neumann
    // before the wedge and reflective after it on the bottom, Dirichlet
    // (shock states) on the top
    const Mesh &m = *P.mesh;
    const bool back = m.g(r, col_minus(2, 1, 0)) == -1;
    const double myX = m.x[m.g(r, 0)];
    if (back && myX >= kDmrWedge) f[2] = -1.;
    else if (!back)
      for (int j = 0; j < 4; ++j) f[j] = 0.;
  }
  if (P.bc == BC_CROSSSHOCK) {
    // euler_2d_prob_class.hpp:1195-1222: Dirichlet on the left, Neumann on
    // the right and top, Dirichlet momentum with Neumann density and energy
    // on the bottom
    const Mesh &m = *P.mesh;
    if (ax == 0 && m.g(r, col_minus(2, 0, 0)) == -1)
      for (int j = 0; j < 4; ++j) f[j] = 0.;
    if (ax == 1 && m.g(r, col_minus(2, 1, 0)) == -1) f[1] = f[2] = 0.;
  }
}

void build_inner_table(pda_problem &P, bool withJ) {
  if (withJ ? P.innerBuiltJ : P.innerBuiltV) return;
  const Mesh &m = *P.mesh;
  build_stencil(P, P.innerT, m.inner, false);
  if (withJ) {
    build_pattern(P);
    P.innerT.jpos.resize(P.innerT.src.size());
    const int S = 2 * P.h + 1;
    for (size_t e = 0; e < m.inner.size(); ++e)
      for (int ax = 0; ax < P.dim; ++ax)
        for (int s = 0; s < S; ++s) {
          const size_t pos = (e * P.dim + ax) * S + s;
          P.innerT.jpos[pos] = block_offset(P, m.inner[e], P.innerT.src[pos]);
        }
    P.innerBuiltJ = true;
  }
  P.innerT.dirty = true;
  P.innerBuiltV = true;
}

void build_near_table(pda_problem &P, bool withJ) {
  const Mesh &m = *P.mesh;
  if (!withJ) {
    build_stencil(P, P.nearT, m.nearBd, true);
    P.nearT.dirty = true;
    return;
  }
  if (P.nearBuiltJ) return;
  build_pattern(P);
  Table &T = P.nearT;
  const size_t n = m.nearBd.size();
  T.src1.assign(n * P.dim * 3, 0);
  T.flip1.assign(n * P.dim * 3, 0);
  T.jpos1.assign(n * P.dim * 3, -1);
  T.jfac.assign(n * P.dim * P.ndpc, 1.0);
  T.gsx1.assign(P.timeDependent ? n * P.dim * 3 : 0, 0.);
  T.gsy1.assign(T.gsx1.size(), 0.);
  const bool keepPos = !T.gsx1.empty();
  for (size_t e = 0; e < n; ++e) {
    const int64_t r = m.nearBd[e];
    for (int ax = 0; ax < P.dim; ++ax) {
      const size_t base = (e * P.dim + ax) * 3;
      T.src1[base + 1] = m.g(r, 0);
      T.jpos1[base + 1] = block_offset(P, r, m.g(r, 0));
      const int cm = m.g(r, col_minus(P.dim, ax, 0)), cp = m.g(r, col_plus(P.dim, ax, 0));
      if (cm != -1) {
        T.src1[base] = cm;
        T.jpos1[base] = block_offset(P, r, cm);
      } else {
        ghost_entry(P, r, ax, true, 0, &T.src1[base], &T.flip1[base], keepPos ? &T.gsx1[base] : nullptr,
                    keepPos ? &T.gsy1[base] : nullptr);
      }
      if (cp != -1) {
        T.src1[base + 2] = cp;
        T.jpos1[base + 2] = block_offset(P, r, cp);
      } else {
        ghost_entry(P, r, ax, false, 0, &T.src1[base + 2], &T.flip1[base + 2],
                    keepPos ? &T.gsx1[base + 2] : nullptr, keepPos ? &T.gsy1[base + 2] : nullptr);
      }
      jac_factors(P, r, ax, &T.jfac[(e * P.dim + ax) * P.ndpc]);
    }
  }
  T.dirty = true;
  P.nearBuiltJ = true;
}

// Evaluations the reference refuses: the 3D Sedov ghost filler has layers
// for stencils 3 and 5 only (euler_3d_ghost_filler_sedov.hpp:220-224,
// euler_3d_prob_class.hpp:320-322)
void check_evaluable(const pda_problem &P) {
  PDA_REQUIRE(!(P.family == PDA_EULER3D && P.probEnum == 1 && P.scheme == PDA_WENO5), PDA_ERR_UNSUPPORTED,
              "Euler3d::SedovSymmetry: For 3d, only 1st order is currently working (WENO5 ghost layers are "
              "missing in the reference)");
}

// the problem's ghost recipes on the device (first evaluation; creation
// stays host-only)
void sync_recipes(pda_problem &P) {
  if (P.recipes.empty() || P.d_recipes.p) return;
  P.d_recipes.alloc(P.recipes.size());
  PDA_CUDA(cudaMemcpy(P.d_recipes.p, P.recipes.data(), P.recipes.size() * sizeof(GhostRecipe),
                      cudaMemcpyHostToDevice));
  P.margs.recipes = P.d_recipes.p;
}

void check_launch(pda_problem &P, int n = 1) {
  P.launches += n;
  PDA_CUDA(cudaGetLastError());
}

// --------------------------------------------------------------- evaluation
void velocity(pda_problem &P, const double *U, double *V, double t, cudaEvent_t *ev = nullptr) {
  check_evaluable(P);
  sync_recipes(P);
  MeshArgs ma = P.margs;
  ma.time = t;
  if (P.useStruct) {
    const Box &b = P.box;
    double *Fb[3] = {nullptr, nullptr, nullptr};
    for (int a = 0; a < P.dim; ++a) {
      long nf = 1;
      for (int c = 0; c < 3; ++c) nf *= (long)(b.hi[c] - b.lo[c] + (c == a ? 1 : 0));
      P.F[a].alloc((size_t)nf * P.ndpc);
      Fb[a] = P.F[a].p;
    }
    int nl = 0;
    if (!ev && P.dim >= 2) {
      // the face passes of different axes are independent (separate face
      // arrays): the y faces run on the side stream beside the x (and z)
      // faces, so each pass's last, partly filled wave overlaps the other's
      // (1024^2 Riemann WENO5: 1.302 ms per velocity against 1.319 ms with
      // the passes in sequence).  The profiling path (ev) keeps the
      // sequence, one pass at a time.
      if (!P.side) {
        PDA_CUDA(cudaStreamCreateWithFlags(&P.side, cudaStreamNonBlocking));
        PDA_CUDA(cudaEventCreateWithFlags(&P.evFork, cudaEventDisableTiming));
        PDA_CUDA(cudaEventCreateWithFlags(&P.evJoin, cudaEventDisableTiming));
      }
      PDA_CUDA(cudaEventRecord(P.evFork, P.stream));
      PDA_CUDA(cudaStreamWaitEvent(P.side, P.evFork, 0));
      P.L->struct_faces(P.scheme, 0, b, P.phys, U, Fb[0], P.stream);
      P.L->struct_faces(P.scheme, 1, b, P.phys, U, Fb[1], P.side);
      if (P.dim == 3) P.L->struct_faces(P.scheme, 2, b, P.phys, U, Fb[2], P.stream);
      PDA_CUDA(cudaEventRecord(P.evJoin, P.side));
      PDA_CUDA(cudaStreamWaitEvent(P.stream, P.evJoin, 0));
      const double *Fc[3] = {Fb[0], Fb[1], Fb[2]};
      P.L->struct_balance(b, ma, P.phys, U, Fc, V, P.stream);
      check_launch(P, P.dim + 1);
    } else {
      P.L->struct_velocity(P.scheme, b, ma, P.phys, U, Fb, V, P.stream, &nl, ev);
      check_launch(P, nl);
    }
  }
  // the row tables in one launch: inner rows (when no structured box covers
  // them) and near-boundary rows
  RowTable none{};
  if (!P.useStruct) {
    build_inner_table(P, false);
    P.innerT.sync();
  }
  if (!P.structAll) P.nearT.sync();
  const RowTable &ta = P.useStruct ? none : P.innerT.t;
  const RowTable &tb = P.structAll ? none : P.nearT.t;
  if (ta.nrows + tb.nrows > 0) {
    P.L->rows_velocity(P.scheme, ta, tb, ma, P.phys, U, V, P.stream);
    check_launch(P);
  }
  if (ev) cudaEventRecord(ev[P.dim + 2], P.stream);
}

void velocity_and_jacobian(pda_problem &P, const double *U, double *V, double *J, double t) {
  check_evaluable(P);
  sync_recipes(P);
  MeshArgs ma = P.margs;
  ma.time = t;
  if (P.jStruct) {
    build_near_table(P, true);
    pattern_to_device(P);
    P.nearT.sync();
    int nl = 0;
    P.L->struct_vj(P.scheme, P.jbox, ma, P.phys, U, P.d_rowptr.p, V, J, P.stream, &nl);
    check_launch(P, nl);
    if (P.nearT.t.nrows > 0) {
      P.L->rows_vj_nearbd(P.scheme, P.nearT.t, ma, P.phys, U, P.d_rowptr.p, V, J, P.stream);
      check_launch(P);
    }
    return;
  }
  build_inner_table(P, true);
  build_near_table(P, true);
  pattern_to_device(P);
  P.innerT.sync();
  P.nearT.sync();
  const bool both = P.innerT.t.nrows > 0 && P.nearT.t.nrows > 0;
  cudaStream_t ns = P.stream;
  if (both) {
    // the two row sets are independent (disjoint rows of V and J): fork the
    // near-boundary rows onto a second stream and join before returning
    if (!P.side) {
      PDA_CUDA(cudaStreamCreateWithFlags(&P.side, cudaStreamNonBlocking));
      PDA_CUDA(cudaEventCreateWithFlags(&P.evFork, cudaEventDisableTiming));
      PDA_CUDA(cudaEventCreateWithFlags(&P.evJoin, cudaEventDisableTiming));
    }
    PDA_CUDA(cudaEventRecord(P.evFork, P.stream));
    PDA_CUDA(cudaStreamWaitEvent(P.side, P.evFork, 0));
    ns = P.side;
  }
  if (P.nearT.t.nrows > 0) {
    P.L->rows_vj_nearbd(P.scheme, P.nearT.t, ma, P.phys, U, P.d_rowptr.p, V, J, ns);
    check_launch(P);
  }
  if (P.innerT.t.nrows > 0) {
    P.L->rows_vj_inner(P.scheme, P.innerT.t, ma, P.phys, U, P.d_rowptr.p, V, J, P.stream);
    check_launch(P);
  }
  if (both) {
    PDA_CUDA(cudaEventRecord(P.evJoin, P.side));
    PDA_CUDA(cudaStreamWaitEvent(P.stream, P.evJoin, 0));
  }
}

// ------------------------------------------------------------------ create
void create_problem(pda_problem &P, const Mesh &m, int family, int probEn, int scheme, int icFlag,
                    const char *const *names, const double *vals, int np, void *stream,
                    bool crossShockFactory = false) {
  PDA_REQUIRE(family >= 0 && family <= 3, PDA_ERR_INVALID_ARGUMENT, "invalid problem family");
  PDA_REQUIRE(scheme >= 0 && scheme <= 2, PDA_ERR_INVALID_ARGUMENT, "invalid reconstruction scheme");
  PDA_REQUIRE(np >= 0 && (np == 0 || (names && vals)), PDA_ERR_INVALID_ARGUMENT, "invalid parameter arrays");
  const int dims[4] = {1, 2, 3, 2};
  const int ndpcs[4] = {3, 4, 5, 3};
  PDA_REQUIRE(m.dim == dims[family], PDA_ERR_INVALID_ARGUMENT, "mesh dimensionality does not match the problem");
  P.mesh = &m;
  P.family = family;
  P.probEnum = probEn;
  P.scheme = scheme;
  P.icFlag = icFlag <= 0 ? 1 : icFlag;
  P.dim = dims[family];
  P.ndpc = ndpcs[family];
  P.h = scheme + 1;
  // stencilSizeCompatibleWithInviscidFluxReconstruction (schemes_info.hpp:96-104)
  PDA_REQUIRE(m.stencil >= 2 * P.h + 1, PDA_ERR_INVALID_ARGUMENT,
              "mesh stencil size too small for the reconstruction scheme");
  P.stream = (cudaStream_t)stream;
  P.dofsSample = m.sampleMeshSize * P.ndpc;
  P.dofsStencil = m.stencilMeshSize * P.ndpc;
  P.phys = Phys{1.4, 9.8, -3.0};
  for (int a = 0; a < 3; ++a) {
    P.margs.hinv[a] = m.dxInv[a];
    P.margs.reflect[a] = -1;
  }
  P.margs.dim = P.dim;
  std::vector<std::pair<std::string, double>> params;
  for (int i = 0; i < np; ++i) {
    PDA_REQUIRE(names[i], PDA_ERR_INVALID_ARGUMENT, "null parameter name");
    params.emplace_back(names[i], vals[i]);
  }
  if (family == PDA_EULER1D) {
    // euler_1d_prob_class.hpp:97-112 (gamma hard-wired 1.4)
    PDA_REQUIRE(probEn >= 0 && probEn <= 3, PDA_ERR_INVALID_ARGUMENT, "invalid Euler1d problem");
    PDA_REQUIRE(params.empty(), PDA_ERR_INVALID_ARGUMENT, "Euler1d takes no parameters");
    P.physParams = {1.4};
    P.bc = probEn == 0 ? BC_NONE : BC_NEUMANN1D;
  } else if (family == PDA_EULER3D) {
    // euler3d.hpp:80-122: PeriodicSmooth, SedovSymmetry (reflective on the
    // left, back and bottom planes, Neumann on the others: Ghost3dSedov,
    // impl/euler_3d_ghost_filler_sedov.hpp:58-226)
    PDA_REQUIRE(probEn == 0 || probEn == 1, PDA_ERR_INVALID_ARGUMENT, "invalid Euler3d problem");
    PDA_REQUIRE(params.empty(), PDA_ERR_INVALID_ARGUMENT, "Euler3d takes no parameters");
    P.physParams = {1.4};
    P.bc = probEn == 1 ? BC_SEDOVSYM : BC_NONE;
    if (probEn == 1)
      for (int a = 0; a < 3; ++a) P.margs.reflect[a] = 1 + a;
  } else if (family == PDA_EULER2D) {
    // euler2d.hpp:88-173; impl/euler_2d_parametrization_helpers.hpp:75-93
    PDA_REQUIRE(probEn >= 0 && probEn <= 8, PDA_ERR_INVALID_ARGUMENT, "invalid Euler2d problem");
    const bool validIc = (probEn == 4) ? (P.icFlag == 1 || P.icFlag == 2) : P.icFlag == 1;
    PDA_REQUIRE(validIc, PDA_ERR_INVALID_ARGUMENT, "Euler2d: invalid icFlag for the given problem enum");
    P.physParams = {1.4};
    P.icParams = {9, 0.1, 10., 1., 0.4, 1.5, 0.0, 0.0, 1.5, 0.029};
    if (!params.empty() && !crossShockFactory)
      PDA_REQUIRE(probEn == 4 || probEn == 5, PDA_ERR_INVALID_ARGUMENT,
                  "Euler2d: custom parametrization only valid for Euler2d::{Riemann, NormalShock}");
    for (auto &kv : params) {
      if (kv.first == "gamma") {
        P.physParams[0] = kv.second;
        continue;
      }
      const int idx = euler2d_ic_index(probEn, P.icFlag, kv.first);
      PDA_REQUIRE(idx != kInvalid, PDA_ERR_INVALID_ARGUMENT, "Euler2d: invalid parameter name " + kv.first);
      P.icParams[idx] = kv.second;
    }
    // ghost rules per problem (euler_2d_prob_class.hpp:466-560): none for the
    // periodic problems, Neumann mirrors for SedovFull / Riemann / testing
    P.bc = (probEn == 0 || probEn == 1) ? BC_NONE
           : probEn == 3                ? BC_SEDOVSYM
           : probEn == 5                ? BC_NORMALSHOCK
           : probEn == 6                ? BC_DMR
           : probEn == 7                ? BC_CROSSSHOCK
                                        : BC_MIRROR2D;
    if (probEn == 3) {
      P.margs.reflect[0] = 1;
      P.margs.reflect[1] = 2;
    }
    if (probEn == 5 || probEn == 6) P.margs.reflect[1] = 2;
    const double gamma = P.physParams[0], one = 1.;
    if (probEn == 6) {
      // DoubleMachReflection2dGhostFiller::computeShockConditions and
      // distanceFromShock (euler_2d_ghost_filler_double_mach_reflection.hpp:
      // 272-305, :320-330): Mach 10 shock at pi/6, pre-shock gas at rest
      const double angle = M_PI / 6.;
      const double pre[4] = {gamma, 0., 0., 1.};
      double post[4];
      post_shock_at_rest(pre, -angle, 10., gamma, post);
      const double gm1inv = one / (gamma - one);
      const double *prim[2] = {pre, post};
      double *cons[2] = {P.margs.pre, P.margs.post};
      for (int k = 0; k < 2; ++k) {
        cons[k][0] = prim[k][0];
        cons[k][1] = prim[k][0] * prim[k][1];
        cons[k][2] = prim[k][0] * prim[k][2];
        cons[k][3] = energy2(gm1inv, prim[k], 4);
      }
      P.margs.shockX0 = kDmrWedge;
      P.margs.shockSpeed = 10. / std::cos(angle);
      P.margs.shockSlope = std::tan(angle);
      GhostRecipe shock{};
      shock.op[0] = 3;
      P.recipes = {shock};
      P.timeDependent = true;
    }
    if (probEn == 7) {
      // CrossShock2dGhostFiller (euler_2d_ghost_filler_cross_shock.hpp:61-93)
      const double rho = P.icParams[1], uIn = P.icParams[2], vBot = P.icParams[3];
      const double prim[4] = {rho, uIn, 0., 1.};
      const double gm1inv = one / (gamma - one);
      GhostRecipe inflow{};
      for (int d = 0; d < 4; ++d) inflow.op[d] = 2;
      inflow.val[0] = prim[0];
      inflow.val[1] = prim[0] * prim[1];
      inflow.val[2] = prim[0] * prim[2];
      inflow.val[3] = energy2(gm1inv, prim, 4);
      GhostRecipe b0lo{}, b0hi{}, b1lo{}, b1hi{};
      for (GhostRecipe *g : {&b0lo, &b0hi, &b1lo, &b1hi}) {
        g->op[1] = g->op[2] = 2;
        g->val[1] = rho * uIn;
      }
      b0hi.val[2] = b1hi.val[2] = rho * vBot;
      b1lo.op[0] = b1hi.op[0] = 2;
      b1lo.val[0] = b1hi.val[0] = rho;
      P.recipes = {inflow, b0lo, b0hi, b1lo, b1hi};
    }
  } else {
    // swe2d.hpp:143-195; impl/swe_2d_parametrization_helpers.hpp:59-95
    PDA_REQUIRE(probEn == 0, PDA_ERR_UNSUPPORTED, "Swe2d: only SlipWall is supported");
    PDA_REQUIRE(P.icFlag == 1 || P.icFlag == 2, PDA_ERR_INVALID_ARGUMENT,
                "2D swe: for Swed2d::SlipWall, invalid icFlag");
    P.physParams = {9.8, -3.};
    P.icParams = {1. / 8, 1, 1, 1. / 10, -2, -2, 1. / 8, 2, 2};
    for (auto &kv : params) {
      if (kv.first == "gravity") { P.physParams[0] = kv.second; continue; }
      if (kv.first == "coriolis") { P.physParams[1] = kv.second; continue; }
      const int idx = swe_ic_index(P.icFlag, kv.first);
      PDA_REQUIRE(idx != kInvalid, PDA_ERR_INVALID_ARGUMENT,
                  "2D swe: create_problem_eigen: one or more params in user-provided map is invalid");
      P.icParams[idx] = kv.second;
    }
    P.bc = BC_MIRROR2D;
    P.margs.reflect[0] = 1;
    P.margs.reflect[1] = 2;
  }
  if (family == PDA_SWE2D) {
    P.phys.gravity = P.physParams[0];
    P.phys.coriolis = P.physParams[1];
  } else {
    P.phys.gamma = P.physParams[0];
  }
  if (P.bc == BC_NONE)
    PDA_REQUIRE(m.nearBd.empty(), PDA_ERR_UNSUPPORTED,
                "this problem defines no boundary conditions: the mesh must be fully periodic");
  switch (family) {
    case PDA_EULER1D: P.L = &launchers_euler1d(); break;
    case PDA_EULER2D: P.L = &launchers_euler2d(); break;
    case PDA_EULER3D: P.L = &launchers_euler3d(); break;
    default: P.L = &launchers_swe2d(); break;
  }
  // Structured box.  With the 2D mirror boundary conditions (Neumann, slip
  // wall) the ghost layers are exact mirror images of interior cells
  // (Ghost2dNeumannFiller / InviscidWallFiller with at least 2*h cells per
  // axis), so the box covers the whole mesh and boundary faces are computed
  // from mirrored loads; otherwise it covers the inner rows and the
  // near-boundary rows go through the per-row kernel.
  P.useStruct = false;
  P.structAll = false;
  if (m.structured) {
    const int hm = (m.stencil - 1) / 2;
    bool mirror = P.bc == BC_MIRROR2D;
    for (int a = 0; a < P.dim; ++a)
      if (!m.periodic[a] && m.n[a] < 2 * hm + 1) mirror = false;
    Box b{};
    long cells = 1;
    for (int a = 0; a < 3; ++a) {
      b.n[a] = a < P.dim ? m.n[a] : 1;
      b.reflect[a] = -1;
      if (a >= P.dim) {
        b.mode[a] = 0;
        b.lo[a] = 0;
        b.hi[a] = 1;
      } else if (m.periodic[a]) {
        b.mode[a] = 1;
        b.lo[a] = 0;
        b.hi[a] = b.n[a];
      } else if (mirror) {
        b.mode[a] = 2;
        b.lo[a] = 0;
        b.hi[a] = b.n[a];
        b.reflect[a] = P.margs.reflect[a];
      } else {
        b.mode[a] = 0;
        b.lo[a] = std::min(hm, b.n[a]);
        b.hi[a] = std::max(b.lo[a], b.n[a] - hm);
      }
      cells *= (long)(b.hi[a] - b.lo[a]);
    }
    // Small 1D meshes take the per-row kernels for every row: the face pass
    // puts a whole face (every dof's reconstructions and the flux) on one
    // thread, and below about 60 faces per SM its blocks cannot fill the GPU,
    // so a call costs one long per-warp FP64 instruction stream (GB300 issues
    // one FP64 warp instruction per ~64 cycles per sub-partition); the row
    // kernel spreads a row's work over warps.
    const bool smallLine = P.dim == 1 && (long)m.sampleMeshSize < kRowsOnlyCells1D;
    if (!smallLine && mirror && cells == (long)m.sampleMeshSize) {
      P.box = b;
      P.useStruct = true;
      P.structAll = true;
    } else if (!smallLine && !mirror && cells == (long)m.inner.size()) {
      P.box = b;
      P.useStruct = true;
    }
  }
  // Jacobian of the inner rows with faces computed once: the inner box
  // (periodic axes whole, others [hm, n - hm)), when no stencil repeats a
  // cell (periodic axes of at least 2h + 1 cells); WENO schemes only
  P.jStruct = false;
  if (m.structured && scheme != PDA_FIRST_ORDER && P.dofsSample == P.dofsStencil) {
    const int hm = (m.stencil - 1) / 2;
    Box jb{};
    long cells = 1;
    bool ok = true;
    for (int a = 0; a < 3; ++a) {
      jb.n[a] = a < P.dim ? m.n[a] : 1;
      jb.reflect[a] = -1;
      jb.mode[a] = 0;
      if (a >= P.dim) {
        jb.lo[a] = 0;
        jb.hi[a] = 1;
      } else if (m.periodic[a]) {
        jb.mode[a] = 1;
        jb.lo[a] = 0;
        jb.hi[a] = jb.n[a];
        if (jb.n[a] < 2 * P.h + 1) ok = false;
      } else {
        jb.lo[a] = std::min(hm, jb.n[a]);
        jb.hi[a] = std::max(jb.lo[a], jb.n[a] - hm);
      }
      cells *= (long)(jb.hi[a] - jb.lo[a]);
    }
    if (ok && cells > 0 && cells == (long)m.inner.size()) {
      P.jbox = jb;
      P.jStruct = true;
    }
  }
  build_near_table(P, false);
}

}  // namespace

// ------------------------------------------------------------------ steppers
namespace {

void stepper_buffers(pda_problem &P, int nr) {
  P.aux.alloc(P.dofsStencil);
  for (int i = 0; i < nr; ++i) P.r[i].alloc(P.dofsSample);
}

// One step of SSP-RK3 (ode_explicit_stepper_without_mass_matrix.hpp:230-282).
void ssprk3_step(pda_problem &P, double *U, double t, double dt) {
  const long n = (long)P.dofsStencil;
  double *r0 = P.r[0].p, *aux = P.aux.p;
  const double tHalf = t + dt / 2., tNext = t + dt;
  velocity(P, U, r0, t);
  launch_axpby_stage(0, aux, U, r0, nullptr, 0., dt, 0., 0., nullptr, nullptr, n, P.stream);
  check_launch(P);
  velocity(P, aux, r0, tNext);
  const double fourInv = 1. / 4., threeOvFour = 3. / 4.;
  launch_axpby_stage(1, aux, U, r0, nullptr, fourInv, threeOvFour, fourInv * dt, 0., nullptr, nullptr, n,
                     P.stream);
  check_launch(P);
  velocity(P, aux, r0, tHalf);
  const double oneOvThree = 1. / 3., twoOvThree = 2. / 3.;
  launch_axpby_stage(1, U, aux, r0, nullptr, oneOvThree, twoOvThree, twoOvThree * dt, 0., nullptr, nullptr,
                     n, P.stream);
  check_launch(P);
}

// One step of RK4 (ode_explicit_stepper_without_mass_matrix.hpp:284-336).
void rk4_step(pda_problem &P, double *U, double t, double dt) {
  const long n = (long)P.dofsStencil;
  const double dt2 = dt / 2., dt6 = dt / 6., dt3 = dt / 3.;
  double *aux = P.aux.p;
  const double tHalf = t + dt2, tNext = t + dt;
  velocity(P, U, P.r[0].p, t);
  launch_axpby_stage(0, aux, U, P.r[0].p, nullptr, 0., dt2, 0., 0., nullptr, nullptr, n, P.stream);
  check_launch(P);
  velocity(P, aux, P.r[1].p, tHalf);
  launch_axpby_stage(0, aux, U, P.r[1].p, nullptr, 0., dt2, 0., 0., nullptr, nullptr, n, P.stream);
  check_launch(P);
  velocity(P, aux, P.r[2].p, tHalf);
  launch_axpby_stage(0, aux, U, P.r[2].p, nullptr, 0., dt, 0., 0., nullptr, nullptr, n, P.stream);
  check_launch(P);
  velocity(P, aux, P.r[3].p, tNext);
  launch_axpby_stage(2, U, P.r[0].p, P.r[1].p, P.r[2].p, 0., dt3, 0., dt6, P.r[3].p, nullptr, n, P.stream);
  check_launch(P);
}

void advance(pda_problem &P, int kind, double *U, double t0, double dt, int64_t nsteps, bool useGraph) {
  PDA_REQUIRE(P.dofsSample == P.dofsStencil, PDA_ERR_UNSUPPORTED,
              "time integration needs a full mesh (sample meshes integrate in a reduced space)");
  PDA_REQUIRE(nsteps >= 0, PDA_ERR_INVALID_ARGUMENT, "negative step count");
  stepper_buffers(P, kind == 0 ? 1 : 4);
  auto step = [&](double t) {
    if (kind == 0) ssprk3_step(P, U, t, dt);
    else rk4_step(P, U, t, dt);
  };
  // time-dependent ghost states take the stage times as kernel arguments:
  // those problems step eagerly
  if (!useGraph || P.stream == nullptr || P.timeDependent) {
    double t = t0;
    for (int64_t s = 0; s < nsteps; ++s) {
      step(t);
      t = t + dt;
    }
    return;
  }
  // Capture one step and replay it: the kernels do not depend on t for these
  // boundary conditions.  The graph bakes in U and dt.
  if (P.stepGraph && (P.stepGraphKind != kind || P.stepGraphDt != dt || P.stepGraphU != U)) {
    cudaGraphExecDestroy(P.stepGraph);
    P.stepGraph = nullptr;
  }
  if (!P.stepGraph) {
    // lazily built tables and buffers must exist before capture
    velocity(P, U, P.r[0].p, t0);
    PDA_CUDA(cudaStreamSynchronize(P.stream));
    cudaGraph_t g;
    PDA_CUDA(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
    const int64_t before = P.launches;
    try {
      step(t0);
    } catch (...) {
      cudaStreamEndCapture(P.stream, &g);
      throw;
    }
    PDA_CUDA(cudaStreamEndCapture(P.stream, &g));
    P.stepGraphLaunches = P.launches - before;
    P.launches = before;
    PDA_CUDA(cudaGraphInstantiate(&P.stepGraph, g, 0));
    cudaGraphDestroy(g);
    P.stepGraphKind = kind;
    P.stepGraphDt = dt;
    P.stepGraphU = U;
  }
  for (int64_t s = 0; s < nsteps; ++s) PDA_CUDA(cudaGraphLaunch(P.stepGraph, P.stream));
  P.launches += nsteps * P.stepGraphLaunches;
}

}  // namespace
}  // namespace pda

namespace pda {
void ensure_device_pattern(pda_problem &P) { pattern_to_device(P); }
void ensure_row_tables(pda_problem &P) {
  check_evaluable(P);
  build_inner_table(P, true);
  build_near_table(P, true);
  pattern_to_device(P);
  P.innerT.sync();
  P.nearT.sync();
  sync_recipes(P);
}
}  // namespace pda

// ===================================================================== C ABI
using pda::Error;

extern "C" {

const char *pda_last_error(void) { return pda::g_last_error.c_str(); }
const char *pda_version(void) { return "pda_gb300 0.1.0"; }

pda_status pda_mesh_load(const char *dir, pda_mesh **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(dir && out, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_ptr<pda_mesh> m(new pda_mesh);
  m->m = pda::mesh_load(dir);
  *out = m.release();
  PDA_API_END
}

pda_status pda_mesh_create_full(const int n[3], const double bounds[6], int stencil, const int periodic[3],
                                pda_mesh **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(n && bounds && periodic && out, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_ptr<pda_mesh> m(new pda_mesh);
  m->m = pda::mesh_generate_full(n, bounds, stencil, periodic);
  *out = m.release();
  PDA_API_END
}

pda_status pda_mesh_create_sample(const pda_mesh *full, const int64_t *gids, int64_t n, pda_mesh **out,
                                  int64_t *stencil_gids_out) {
  PDA_API_BEGIN
  PDA_REQUIRE(full && out && (n == 0 || gids), PDA_ERR_INVALID_ARGUMENT, "null argument");
  PDA_REQUIRE(n > 0, PDA_ERR_INVALID_ARGUMENT, "empty sample mesh");
  std::vector<int64_t> g(gids, gids + n), st;
  std::unique_ptr<pda_mesh> m(new pda_mesh);
  m->m = pda::mesh_sample(full->m, g, &st);
  if (stencil_gids_out) std::copy(st.begin(), st.end(), stencil_gids_out);
  *out = m.release();
  PDA_API_END
}

pda_status pda_mesh_write(const pda_mesh *m, const char *dir) {
  PDA_API_BEGIN
  PDA_REQUIRE(m && dir, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::mesh_write(m->m, dir);
  PDA_API_END
}

pda_status pda_mesh_write_binary(const pda_mesh *m, const char *path) {
  PDA_API_BEGIN
  PDA_REQUIRE(m && path, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::mesh_write_binary(m->m, path);
  PDA_API_END
}

pda_status pda_mesh_load_binary(const char *path, pda_mesh **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(path && out, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_ptr<pda_mesh> m(new pda_mesh);
  m->m = pda::mesh_load_binary(path);
  *out = m.release();
  PDA_API_END
}

pda_status pda_mesh_info(const pda_mesh *mm, int dims[3], int64_t sizes[4], double dx[3], double dxinv[3],
                         int flags[2]) {
  PDA_API_BEGIN
  PDA_REQUIRE(mm, PDA_ERR_INVALID_ARGUMENT, "null mesh");
  const pda::Mesh &m = mm->m;
  if (dims) { dims[0] = m.dim; dims[1] = m.stencil; dims[2] = m.ncols; }
  if (sizes) {
    sizes[0] = m.stencilMeshSize;
    sizes[1] = m.sampleMeshSize;
    sizes[2] = (int64_t)m.inner.size();
    sizes[3] = (int64_t)m.nearBd.size();
  }
  for (int a = 0; a < 3; ++a) {
    if (dx) dx[a] = m.dx[a];
    if (dxinv) dxinv[a] = m.dxInv[a];
  }
  if (flags) { flags[0] = m.fullyPeriodic; flags[1] = m.structured; }
  PDA_API_END
}

pda_status pda_mesh_arrays(const pda_mesh *mm, int32_t *graph, double *x, double *y, double *z,
                           int32_t *inner_rows, int32_t *near_bd_rows) {
  PDA_API_BEGIN
  PDA_REQUIRE(mm, PDA_ERR_INVALID_ARGUMENT, "null mesh");
  const pda::Mesh &m = mm->m;
  if (graph) std::copy(m.graph.begin(), m.graph.end(), graph);
  if (x) std::copy(m.x.begin(), m.x.end(), x);
  if (y) std::copy(m.y.begin(), m.y.end(), y);
  if (z) std::copy(m.z.begin(), m.z.end(), z);
  if (inner_rows) std::copy(m.inner.begin(), m.inner.end(), inner_rows);
  if (near_bd_rows) std::copy(m.nearBd.begin(), m.nearBd.end(), near_bd_rows);
  PDA_API_END
}

void pda_mesh_free(pda_mesh *m) { delete m; }

pda_status pda_problem_create(const pda_mesh *mesh, int family, int problem, int scheme, int ic_flag,
                              const char *const *names, const double *vals, int np, void *stream,
                              pda_problem **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(mesh && out, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_ptr<pda_problem> p(new pda_problem);
  pda::create_problem(*p, mesh->m, family, problem, scheme, ic_flag, names, vals, np, stream);
  *out = p.release();
  PDA_API_END
}

pda_status pda_problem_create_swe_slip_wall(const pda_mesh *mesh, int scheme, double gravity, double coriolis,
                                            double pulse, void *stream, pda_problem **out) {
  const char *names[3] = {"gravity", "coriolis", "pulseMagnitude"};
  const double vals[3] = {gravity, coriolis, pulse};
  return pda_problem_create(mesh, PDA_SWE2D, PDA_SWE2D_SLIP_WALL, scheme, 1, names, vals, 3, stream, out);
}

pda_status pda_problem_create_cross_shock(const pda_mesh *mesh, int scheme, double density, double inlet_x_vel,
                                          double bottom_y_vel, void *stream, pda_problem **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(mesh && out, PDA_ERR_INVALID_ARGUMENT, "null argument");
  const char *names[3] = {"crossShockDensity", "crossShockInletXVel", "crossShockBottomYVel"};
  const double vals[3] = {density, inlet_x_vel, bottom_y_vel};
  std::unique_ptr<pda_problem> p(new pda_problem);
  pda::create_problem(*p, mesh->m, PDA_EULER2D, 7, scheme, 1, names, vals, 3, stream, true);
  *out = p.release();
  PDA_API_END
}

void pda_problem_free(pda_problem *p) { delete p; }

pda_status pda_problem_sizes(const pda_problem *p, int *ndpc, int64_t *ds, int64_t *dst) {
  PDA_API_BEGIN
  PDA_REQUIRE(p, PDA_ERR_INVALID_ARGUMENT, "null problem");
  if (ndpc) *ndpc = p->ndpc;
  if (ds) *ds = p->dofsSample;
  if (dst) *dst = p->dofsStencil;
  PDA_API_END
}

pda_status pda_query_parameter(const pda_problem *p, const char *name, double *value) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && name && value, PDA_ERR_INVALID_ARGUMENT, "null argument");
  const std::string s(name);
  if (p->family == PDA_SWE2D) {
    if (s == "gravity") { *value = p->physParams[0]; return PDA_OK; }
    if (s == "coriolis") { *value = p->physParams[1]; return PDA_OK; }
    const int idx = pda::swe_ic_index(p->icFlag, s);
    PDA_REQUIRE(idx >= 0, PDA_ERR_INVALID_ARGUMENT, "unknown parameter " + s);
    *value = p->icParams[idx];
  } else {
    if (s == "gamma") { *value = p->physParams[0]; return PDA_OK; }
    PDA_REQUIRE(p->family == PDA_EULER2D, PDA_ERR_INVALID_ARGUMENT, "unknown parameter " + s);
    const int idx = pda::euler2d_ic_index(p->probEnum, p->icFlag, s);
    PDA_REQUIRE(idx >= 0, PDA_ERR_INVALID_ARGUMENT, "unknown parameter " + s);
    *value = p->icParams[idx];
  }
  PDA_API_END
}

pda_status pda_initial_condition_host(const pda_problem *p, double *hU) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && hU, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<double> st;
  pda::initial_condition(*p, st);
  std::copy(st.begin(), st.end(), hU);
  PDA_API_END
}

pda_status pda_initial_condition(pda_problem *p, double *dU) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<double> st;
  pda::initial_condition(*p, st);
  PDA_CUDA(cudaMemcpyAsync(dU, st.data(), st.size() * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  PDA_CUDA(cudaStreamSynchronize(p->stream));
  PDA_API_END
}

pda_status pda_velocity(pda_problem *p, const double *dU, double t, double *dV) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU && dV, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::velocity(*p, dU, dV, t);
  PDA_API_END
}

pda_status pda_velocity_noalloc(pda_problem *p, const double *dU, double t, double *dV) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU && dV, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda_problem &P = *p;
  pda::check_evaluable(P);
  pda::MeshArgs ma = P.margs;
  ma.time = t;
  if (!P.useStruct) {
    // every row through the row kernel (small 1D full meshes): no face
    // scratch, only the two row tables, uploaded by the first pda_velocity call
    PDA_REQUIRE(P.mesh->structured && P.innerBuiltV && !P.innerT.dirty && !P.nearT.dirty &&
                    (P.recipes.empty() || P.d_recipes.p),
                PDA_ERR_UNSUPPORTED,
                "pda_velocity_noalloc: full meshes only, and the row tables of this problem are not on the device "
                "yet; one pda_velocity call on the problem uploads them");
    P.L->rows_velocity(P.scheme, P.innerT.t, P.nearT.t, ma, P.phys, dU, dV, P.stream);
    pda::check_launch(P);
    return PDA_OK;
  }
  // the near-boundary row table is uploaded by the first pda_velocity call;
  // uploading it here would allocate
  const bool nearResident =
      (P.structAll || P.nearT.hostRows() == 0 || !P.nearT.dirty) && (P.recipes.empty() || P.d_recipes.p);
  PDA_REQUIRE(nearResident, PDA_ERR_UNSUPPORTED,
              "pda_velocity_noalloc: the near-boundary row table of this problem is not on the device yet; "
              "one pda_velocity call on the problem uploads it");
  // face regions, each rounded up to 32 doubles (256 bytes)
  size_t off[3] = {0, 0, 0}, need = 0;
  for (int a = 0; a < P.dim; ++a) {
    size_t nf = 1;
    for (int c = 0; c < 3; ++c) nf *= (size_t)(P.box.hi[c] - P.box.lo[c] + (c == a ? 1 : 0));
    off[a] = need;
    need += (nf * (size_t)P.ndpc + 31) / 32 * 32;
  }
  if (need > (size_t)PDA_NOALLOC_SCRATCH_DOUBLES)
    throw pda::Error(PDA_ERR_INVALID_ARGUMENT,
                     "pda_velocity_noalloc: this mesh needs " + std::to_string(need) +
                         " doubles of face scratch, more than the static limit of " +
                         std::to_string((size_t)PDA_NOALLOC_SCRATCH_DOUBLES) +
                         " (PDA_NOALLOC_SCRATCH_DOUBLES); use pda_velocity");
  double *scratch = nullptr;
  PDA_CUDA(pda::noalloc_face_scratch(&scratch));
  double *Fb[3] = {nullptr, nullptr, nullptr};
  for (int a = 0; a < P.dim; ++a) Fb[a] = scratch + off[a];
  int nl = 0;
  P.L->struct_velocity(P.scheme, P.box, ma, P.phys, dU, Fb, dV, P.stream, &nl, nullptr);
  pda::check_launch(P, nl);
  if (!P.structAll && P.nearT.t.nrows > 0) {
    pda::RowTable none{};
    P.L->rows_velocity(P.scheme, none, P.nearT.t, ma, P.phys, dU, dV, P.stream);
    pda::check_launch(P);
  }
  PDA_API_END
}

namespace pda {
// pda_velocity_host for 2D meshes that one structured box covers: kHostBands
// row bands whose copies overlap the other bands' kernels.  The copy stream
// moves the bands' rows in order; each band's x faces start on its own
// compute stream as soon as its rows are on the device (x faces read no
// other row), its y faces once the next band's rows are in too (band b
// computes y faces [r_b + 1, r_b+1], band 0 from face 0), its balance after
// its own faces and the previous band's y faces (it reads face r_b), and its
// velocity rows go back as soon as its balance is done.  Earlier bands run
// at higher stream priority, so they finish first while later bands' blocks
// fill their tails.  The first band's copy in and the last band's copy out
// cannot overlap any kernel; more bands shorten them.  The same kernels on
// sub-boxes: V equals pda_velocity's bit for bit.
//
// Repeated calls with the same pinned buffers and time replay the whole
// sequence (copies, kernels, cross-stream events) as one CUDA graph, captured
// on the second consecutive call with the same arguments and device buffers;
// pageable host buffers (not capturable) and changing arguments take the
// direct path.  Returns false when the mesh does not qualify.
bool velocity_host_banded(pda_problem &P, const double *hU, double t, double *hV) {
  constexpr int NB = kHostBands;
  if (!(P.useStruct && P.structAll && P.dim == 2 && P.box.n[1] >= 16 * NB && P.dofsSample == P.dofsStencil))
    return false;
  check_evaluable(P);
  sync_recipes(P);
  if (!P.hostCopy) {
    int least = 0, greatest = 0;
    PDA_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    for (int b = 0; b < NB; ++b) {
      // priorities run from greatest (numerically lowest) to least
      const int prio = greatest + b > least ? least : greatest + b;
      PDA_CUDA(cudaStreamCreateWithPriority(&P.hostBand[b], cudaStreamNonBlocking, prio));
    }
    PDA_CUDA(cudaStreamCreateWithFlags(&P.hostCopy, cudaStreamNonBlocking));
    for (cudaEvent_t &e : P.hostEv) PDA_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  const Box &B = P.box;
  const int nx = B.n[0], ny = B.n[1], nd = P.ndpc;
  int r[NB + 1];
  for (int b = 0; b <= NB; ++b) r[b] = (int)((long)ny * b / NB);
  const size_t rowDofs = (size_t)nx * nd;
  P.d_U.alloc(P.dofsStencil);
  P.d_V.alloc(P.dofsSample);
  P.F[0].alloc((size_t)(nx + 1) * ny * nd);
  P.F[1].alloc((size_t)nx * (ny + 1) * nd);
  double *U = P.d_U.p, *V = P.d_V.p, *Fx = P.F[0].p, *Fy = P.F[1].p;
  MeshArgs ma = P.margs;
  ma.time = t;
  const HostGraphKey key{hU, hV, t, U, V, Fx, Fy};
  bool pinned = false;
  {
    cudaPointerAttributes au{}, av{};
    if (cudaPointerGetAttributes(&au, hU) == cudaSuccess && cudaPointerGetAttributes(&av, hV) == cudaSuccess)
      pinned = au.type == cudaMemoryTypeHost && av.type == cudaMemoryTypeHost;
    cudaGetLastError();  // a pageable pointer may leave an error behind on older drivers
  }
  constexpr int nLaunch = 3 * NB;
  // events: start, rows in [NB], y faces [NB], balance [NB], copies out, graph order
  cudaEvent_t *ev = P.hostEv;
  cudaEvent_t evStart = ev[0], *evIn = ev + 1, *evY = ev + 1 + NB, *evBal = ev + 1 + 2 * NB;
  cudaEvent_t evOut = ev[1 + 3 * NB], evOrder = ev[2 + 3 * NB];
  cudaStream_t *cs = P.hostBand, sc = P.hostCopy;
  // the graph runs on the first band's stream, after whatever the problem's
  // stream holds; later work on the problem's stream follows it
  auto launch_graph = [&]() {
    PDA_CUDA(cudaEventRecord(evOrder, P.stream));
    PDA_CUDA(cudaStreamWaitEvent(cs[0], evOrder, 0));
    PDA_CUDA(cudaGraphLaunch(P.hostGraph, cs[0]));
    PDA_CUDA(cudaEventRecord(evOrder, cs[0]));
    PDA_CUDA(cudaStreamWaitEvent(P.stream, evOrder, 0));
    PDA_CUDA(cudaStreamSynchronize(cs[0]));
  };
  if (pinned && P.hostGraph && P.hostGraphKey == key) {
    launch_graph();
    P.launches += nLaunch;
    return true;
  }
  const bool capture = pinned && P.hostLastKey == key;
  P.hostLastKey = key;
  // ends an open capture if an error leaves this function early
  struct CaptureGuard {
    cudaStream_t s;
    bool open;
    ~CaptureGuard() {
      if (!open) return;
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
    }
  } guard{cs[0], false};
  if (capture) {
    PDA_CUDA(cudaStreamBeginCapture(cs[0], cudaStreamCaptureModeThreadLocal));
    guard.open = true;
  }
  // the sequence starts and ends on `so`: the problem's stream when run
  // directly, the first band's stream (the capture origin) when captured
  const cudaStream_t so = capture ? cs[0] : P.stream;
  PDA_CUDA(cudaEventRecord(evStart, so));
  PDA_CUDA(cudaStreamWaitEvent(sc, evStart, 0));
  for (int b = 0; b < NB; ++b) PDA_CUDA(cudaStreamWaitEvent(cs[b], evStart, 0));
  for (int b = 0; b < NB; ++b) {
    PDA_CUDA(cudaMemcpyAsync(U + r[b] * rowDofs, hU + r[b] * rowDofs, (size_t)(r[b + 1] - r[b]) * rowDofs * 8,
                             cudaMemcpyHostToDevice, sc));
    PDA_CUDA(cudaEventRecord(evIn[b], sc));
  }
  for (int b = 0; b < NB; ++b) {
    PDA_CUDA(cudaStreamWaitEvent(cs[b], evIn[b], 0));
    Box xb = B;
    xb.lo[1] = r[b];
    xb.hi[1] = r[b + 1];
    P.L->struct_faces(P.scheme, 0, xb, P.phys, U, Fx + (size_t)(nx + 1) * r[b] * nd, cs[b]);
  }
  for (int b = 0; b < NB; ++b) {
    // the next band's rows (the copy stream is in order: earlier rows too)
    PDA_CUDA(cudaStreamWaitEvent(cs[b], evIn[b + 1 < NB ? b + 1 : b], 0));
    Box yb = B;
    yb.lo[1] = b == 0 ? 0 : r[b] + 1;
    yb.hi[1] = r[b + 1];
    P.L->struct_faces(P.scheme, 1, yb, P.phys, U, Fy + (size_t)nx * yb.lo[1] * nd, cs[b]);
    PDA_CUDA(cudaEventRecord(evY[b], cs[b]));
  }
  for (int b = 0; b < NB; ++b) {
    if (b > 0) PDA_CUDA(cudaStreamWaitEvent(cs[b], evY[b - 1], 0));  // face r_b, from the previous band
    Box bb = B;
    bb.lo[1] = r[b];
    bb.hi[1] = r[b + 1];
    const double *Fb[3] = {Fx + (size_t)(nx + 1) * r[b] * nd, Fy + (size_t)nx * r[b] * nd, nullptr};
    P.L->struct_balance(bb, ma, P.phys, U, Fb, V, cs[b]);
    PDA_CUDA(cudaEventRecord(evBal[b], cs[b]));
  }
  for (int b = 0; b < NB; ++b) {
    PDA_CUDA(cudaStreamWaitEvent(sc, evBal[b], 0));
    PDA_CUDA(cudaMemcpyAsync(hV + r[b] * rowDofs, V + r[b] * rowDofs, (size_t)(r[b + 1] - r[b]) * rowDofs * 8,
                             cudaMemcpyDeviceToHost, sc));
  }
  PDA_CUDA(cudaEventRecord(evOut, sc));
  // every band stream's last work is awaited by the copy stream, which `so`
  // awaits: the fork joins back (as a capture requires), and later work on
  // `so` follows
  PDA_CUDA(cudaStreamWaitEvent(so, evOut, 0));
  P.launches += nLaunch;
  if (capture) {
    cudaGraph_t g = nullptr;
    guard.open = false;
    PDA_CUDA(cudaStreamEndCapture(cs[0], &g));
    if (P.hostGraph) {
      cudaGraphExecDestroy(P.hostGraph);
      P.hostGraph = nullptr;
    }
    const cudaError_t ie = cudaGraphInstantiate(&P.hostGraph, g, 0);
    cudaGraphDestroy(g);
    PDA_CUDA(ie);
    P.hostGraphKey = key;
    launch_graph();
  } else {
    PDA_CUDA(cudaStreamSynchronize(P.stream));  // the last copy follows every kernel of every band
  }
  PDA_CUDA(cudaGetLastError());
  return true;
}
}  // namespace pda

pda_status pda_velocity_host(pda_problem *p, const double *hU, double t, double *hV) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && hU && hV, PDA_ERR_INVALID_ARGUMENT, "null argument");
  if (pda::velocity_host_banded(*p, hU, t, hV)) return PDA_OK;
  p->d_U.alloc(p->dofsStencil);
  p->d_V.alloc(p->dofsSample);
  PDA_CUDA(cudaMemcpyAsync(p->d_U.p, hU, p->dofsStencil * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  pda::velocity(*p, p->d_U.p, p->d_V.p, t);
  PDA_CUDA(cudaMemcpyAsync(hV, p->d_V.p, p->dofsSample * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  PDA_CUDA(cudaStreamSynchronize(p->stream));
  PDA_API_END
}

pda_status pda_jacobian_shape(pda_problem *p, int64_t *rows, int64_t *cols, int64_t *nnz) {
  PDA_API_BEGIN
  PDA_REQUIRE(p, PDA_ERR_INVALID_ARGUMENT, "null problem");
  pda::build_pattern(*p);
  if (rows) *rows = p->dofsSample;
  if (cols) *cols = p->dofsStencil;
  if (nnz) *nnz = (int64_t)p->colidx.size();
  PDA_API_END
}

pda_status pda_jacobian_pattern(pda_problem *p, int32_t *drp, int32_t *dci) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && drp && dci, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::pattern_to_device(*p);
  PDA_CUDA(cudaMemcpyAsync(drp, p->d_rowptr.p, p->rowptr.size() * sizeof(int), cudaMemcpyDeviceToDevice,
                           p->stream));
  PDA_CUDA(cudaMemcpyAsync(dci, p->d_colidx.p, p->colidx.size() * sizeof(int), cudaMemcpyDeviceToDevice,
                           p->stream));
  PDA_CUDA(cudaStreamSynchronize(p->stream));
  PDA_API_END
}

pda_status pda_jacobian_pattern_host(pda_problem *p, int32_t *hrp, int32_t *hci) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && hrp && hci, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::build_pattern(*p);
  std::copy(p->rowptr.begin(), p->rowptr.end(), hrp);
  std::copy(p->colidx.begin(), p->colidx.end(), hci);
  PDA_API_END
}

pda_status pda_velocity_and_jacobian(pda_problem *p, const double *dU, double t, double *dV, double *dJ) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU && dV && dJ, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::velocity_and_jacobian(*p, dU, dV, dJ, t);
  PDA_API_END
}

pda_status pda_velocity_and_jacobian_host(pda_problem *p, const double *hU, double t, double *hV,
                                          double *hJ) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && hU && hV && hJ, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::build_pattern(*p);
  p->d_U.alloc(p->dofsStencil);
  p->d_V.alloc(p->dofsSample);
  p->d_J.alloc(p->colidx.size());
  PDA_CUDA(cudaMemcpyAsync(p->d_U.p, hU, p->dofsStencil * sizeof(double), cudaMemcpyHostToDevice, p->stream));
  pda::velocity_and_jacobian(*p, p->d_U.p, p->d_V.p, p->d_J.p, t);
  PDA_CUDA(cudaMemcpyAsync(hV, p->d_V.p, p->dofsSample * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  PDA_CUDA(cudaMemcpyAsync(hJ, p->d_J.p, p->colidx.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  PDA_CUDA(cudaStreamSynchronize(p->stream));
  PDA_API_END
}

pda_status pda_jacobian(pda_problem *p, const double *dU, double t, double *dJ) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU && dJ, PDA_ERR_INVALID_ARGUMENT, "null argument");
  p->d_Vscratch.alloc(p->dofsSample);
  pda::velocity_and_jacobian(*p, dU, p->d_Vscratch.p, dJ, t);
  PDA_API_END
}

pda_status pda_apply_jacobian(pda_problem *p, const double *dU, double t, const double *dB, int ncols,
                              double *dR) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU && dB && dR && ncols >= 1, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  pda::pattern_to_device(*p);
  p->d_Vscratch.alloc(p->dofsSample);
  p->d_Jscratch.alloc(p->colidx.size());
  pda::velocity_and_jacobian(*p, dU, p->d_Vscratch.p, p->d_Jscratch.p, t);
  pda::launch_csr_spmm(p->dofsSample, p->d_rowptr.p, p->d_colidx.p, p->d_Jscratch.p, dB, p->dofsStencil, ncols,
                       dR, p->dofsSample, p->stream);
  pda::check_launch(*p);
  PDA_API_END
}

pda_status pda_advance_ssprk3(pda_problem *p, double *dU, double t0, double dt, int64_t n, int use_graph) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::advance(*p, 0, dU, t0, dt, n, use_graph != 0);
  PDA_API_END
}

pda_status pda_advance_rk4(pda_problem *p, double *dU, double t0, double dt, int64_t n, int use_graph) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU, PDA_ERR_INVALID_ARGUMENT, "null argument");
  pda::advance(*p, 1, dU, t0, dt, n, use_graph != 0);
  PDA_API_END
}

int64_t pda_problem_launch_count(const pda_problem *p) { return p ? p->launches : 0; }

pda_status pda_profile_velocity(pda_problem *p, const double *dU, double *dV, int reps, double *ms) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && dU && dV && ms && reps > 0, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  const int ne = p->dim + 3;
  std::vector<cudaEvent_t> ev(ne);
  for (auto &e : ev) PDA_CUDA(cudaEventCreate(&e));
  std::vector<double> acc(ne - 1, 0.0);
  for (int r = 0; r < reps; ++r) {
    pda::velocity(*p, dU, dV, 0.0, p->useStruct ? ev.data() : nullptr);
    if (!p->useStruct) break;
    PDA_CUDA(cudaEventSynchronize(ev[ne - 1]));
    for (int k = 0; k + 1 < ne; ++k) {
      float t = 0;
      PDA_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
      acc[k] += t;
    }
  }
  for (int k = 0; k < 5; ++k) ms[k] = 0.0;
  // order: faces x, faces y, faces z, balance, near-boundary rows
  for (int a = 0; a < p->dim; ++a) ms[a] = acc[a] / reps;
  ms[3] = acc[p->dim] / reps;
  ms[4] = acc[p->dim + 1] / reps;
  for (auto &e : ev) cudaEventDestroy(e);
  PDA_API_END
}

pda_status pda_measure_fp64_peak(double *flops_per_s) {
  PDA_API_BEGIN
  PDA_REQUIRE(flops_per_s, PDA_ERR_INVALID_ARGUMENT, "null argument");
  int dev = 0, sms = 0;
  PDA_CUDA(cudaGetDevice(&dev));
  PDA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  *flops_per_s = pda::measure_fp64_fma_rate(sms * 8, 256, 4096, nullptr);
  PDA_CUDA(cudaGetLastError());
  PDA_API_END
}

pda_status pda_check_divsqrt(int mode, uint64_t seed, int64_t per_thread, int64_t counts[3]) {
  PDA_API_BEGIN
  PDA_REQUIRE(counts && mode >= 0 && mode <= 3 && per_thread > 0, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  long long c[3] = {0, 0, 0};
  pda::check_divsqrt(mode, seed, (long)per_thread, c, nullptr);
  PDA_CUDA(cudaGetLastError());
  for (int k = 0; k < 3; ++k) counts[k] = (int64_t)c[k];
  PDA_API_END
}

pda_status pda_check_products(int mode, uint64_t seed, int64_t per_thread, int64_t counts[5]) {
  PDA_API_BEGIN
  PDA_REQUIRE(counts && mode >= 0 && mode <= 3 && per_thread > 0, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  long long c[5] = {0, 0, 0, 0, 0};
  pda::check_products(mode, seed, (long)per_thread, c, nullptr);
  PDA_CUDA(cudaGetLastError());
  for (int k = 0; k < 5; ++k) counts[k] = (int64_t)c[k];
  PDA_API_END
}

}  // extern "C"
