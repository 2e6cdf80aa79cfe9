// Test infrastructure only (the oracle): a thin C shim over the unmodified
// pressio-demoapps headers, compiled from the reference's own sources by
// oracle/Makefile into oracle/_ref/libpdaref.so.  Used in this container to
// pin the C restatement (oracle/pda_oracle.c) and to generate the golden
// fixtures under tests/golden/.  Serial build (no OpenMP): the reference's
// near-boundary Jacobian loops share a mutable factors array between threads.
//
// API surface wrapped: load_cellcentered_uniform_mesh_eigen (mesh.hpp:87),
// create_problem_eigen (euler1d.hpp:82, euler2d.hpp:88-146, euler3d.hpp:80,
// swe2d.hpp:170-195), create_cross_shock_problem_eigen (euler2d.hpp:258-285), initialCondition, rightHandSide, rightHandSideAndJacobian
// (adapter_cpp.hpp:193-221).
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>

#include "pressiodemoapps/euler1d.hpp"
#include "pressiodemoapps/euler2d.hpp"
#include "pressiodemoapps/euler3d.hpp"
#include "pressiodemoapps/swe2d.hpp"

namespace pda = pressiodemoapps;

namespace {

using mesh_t = pda::cellcentered_uniform_mesh_eigen_type;

struct Base {
  virtual ~Base() = default;
  virtual int ndpc() const = 0;
  virtual long dofsSample() const = 0;
  virtual long dofsStencil() const = 0;
  virtual long nnz() const = 0;
  virtual void ic(double *out) const = 0;
  virtual void velocity(const double *U, double t, double *V) = 0;
  virtual void velocityAndJacobian(const double *U, double t, double *V, int *rowptr, int *colidx,
                                   double *vals) = 0;
};

template <class P> struct Holder : Base {
  std::unique_ptr<mesh_t> mesh;
  P prob;
  typename P::jacobian_type J;
  Holder(std::unique_ptr<mesh_t> m, P &&p) : mesh(std::move(m)), prob(std::move(p)) {
    J = prob.createJacobian();
  }
  int ndpc() const override { return prob.numDofPerCell(); }
  long dofsSample() const override { return (long)prob.totalDofSampleMesh(); }
  long dofsStencil() const override { return (long)prob.totalDofStencilMesh(); }
  long nnz() const override { return (long)J.nonZeros(); }
  void ic(double *out) const override {
    auto s = prob.initialCondition();
    std::memcpy(out, s.data(), sizeof(double) * s.size());
  }
  void velocity(const double *U, double t, double *V) override {
    typename P::state_type u = Eigen::Map<const Eigen::VectorXd>(U, dofsStencil());
    auto v = prob.createRightHandSide();
    prob.rightHandSide(u, t, v);
    std::memcpy(V, v.data(), sizeof(double) * v.size());
  }
  void velocityAndJacobian(const double *U, double t, double *V, int *rowptr, int *colidx,
                           double *vals) override {
    typename P::state_type u = Eigen::Map<const Eigen::VectorXd>(U, dofsStencil());
    auto v = prob.createRightHandSide();
    prob.rightHandSideAndJacobian(u, t, v, J);
    std::memcpy(V, v.data(), sizeof(double) * v.size());
    std::memcpy(rowptr, J.outerIndexPtr(), sizeof(int) * (J.rows() + 1));
    std::memcpy(colidx, J.innerIndexPtr(), sizeof(int) * J.nonZeros());
    std::memcpy(vals, J.valuePtr(), sizeof(double) * J.nonZeros());
  }
};

template <class P> Base *make(std::unique_ptr<mesh_t> m, P &&p) {
  return new Holder<P>(std::move(m), std::move(p));
}

thread_local std::string g_err;

}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

// family: 0 Euler1d, 1 Euler2d, 2 Euler3d, 3 Swe2d; scheme 0/1/2
void *ref_create(const char *meshdir, int family, int problem, int scheme, int icflag, int np,
                 const char *const *names, const double *vals) {
  try {
    auto mesh = std::make_unique<mesh_t>(pda::load_cellcentered_uniform_mesh_eigen(meshdir));
    const auto rec = scheme == 0 ? pda::InviscidFluxReconstruction::FirstOrder
                     : scheme == 1 ? pda::InviscidFluxReconstruction::Weno3
                                   : pda::InviscidFluxReconstruction::Weno5;
    std::unordered_map<std::string, double> params;
    for (int i = 0; i < np; ++i) params[names[i]] = vals[i];
    const mesh_t &mr = *mesh;
    if (family == 0) {
      return make(std::move(mesh), pda::create_problem_eigen(mr, (pda::Euler1d)problem, rec));
    } else if (family == 1 && problem == 7) {
      // CrossShock: the generic factory passes no initial-condition
      // parameters, which this problem reads; use its own factory
      // (euler2d.hpp:258-299) with the defaults or the given values
      double v[3] = {0.1, 10., 1.};
      const char *nm[3] = {"crossShockDensity", "crossShockInletXVel", "crossShockBottomYVel"};
      for (int k = 0; k < 3; ++k)
        if (params.count(nm[k])) v[k] = params[nm[k]];
      return make(std::move(mesh), pda::create_cross_shock_problem_eigen(mr, rec, v[0], v[1], v[2]));
    } else if (family == 1) {
      if (np > 0)
        return make(std::move(mesh), pda::create_problem_eigen(mr, (pda::Euler2d)problem, rec, icflag, params));
      return make(std::move(mesh), pda::create_problem_eigen(mr, (pda::Euler2d)problem, rec, icflag));
    } else if (family == 2) {
      return make(std::move(mesh), pda::create_problem_eigen(mr, (pda::Euler3d)problem, rec));
    } else {
      if (np > 0)
        return make(std::move(mesh), pda::create_problem_eigen(mr, (pda::Swe2d)problem, rec, icflag, params));
      return make(std::move(mesh), pda::create_problem_eigen(mr, (pda::Swe2d)problem, rec, icflag));
    }
  } catch (const std::exception &e) {
    g_err = e.what();
    return nullptr;
  }
}

void ref_destroy(void *h) { delete static_cast<Base *>(h); }

void ref_sizes(void *h, long *out4) {
  Base *b = static_cast<Base *>(h);
  out4[0] = b->ndpc();
  out4[1] = b->dofsSample();
  out4[2] = b->dofsStencil();
  out4[3] = b->nnz();
}

void ref_ic(void *h, double *out) { static_cast<Base *>(h)->ic(out); }

void ref_velocity(void *h, const double *U, double t, double *V) {
  static_cast<Base *>(h)->velocity(U, t, V);
}

void ref_velocity_and_jacobian(void *h, const double *U, double t, double *V, int *rowptr, int *colidx,
                               double *vals) {
  static_cast<Base *>(h)->velocityAndJacobian(U, t, V, rowptr, colidx, vals);
}

// Explicit steppers with the vendored Pressio update formulas
// (tests_cpp/pressio/include/pressio/ode/impl/ode_explicit_stepper_without_mass_matrix.hpp:230-336).
void ref_ssprk3(void *h, double *U, double t0, double dt, long nsteps) {
  Base *b = static_cast<Base *>(h);
  const long n = b->dofsStencil();
  std::vector<double> aux(n), r(n);
  double t = t0;
  for (long s = 0; s < nsteps; ++s) {
    b->velocity(U, t, r.data());
    for (long i = 0; i < n; ++i) aux[i] = U[i] + dt * r[i];
    b->velocity(aux.data(), t + dt, r.data());
    const double c = (1. / 4.) * dt;
    for (long i = 0; i < n; ++i) aux[i] = (1. / 4.) * aux[i] + (3. / 4.) * U[i] + c * r[i];
    b->velocity(aux.data(), t + dt / 2., r.data());
    const double c2 = (2. / 3.) * dt;
    for (long i = 0; i < n; ++i) U[i] = (1. / 3.) * U[i] + (2. / 3.) * aux[i] + c2 * r[i];
    t = t + dt;
  }
}

void ref_rk4(void *h, double *U, double t0, double dt, long nsteps) {
  Base *b = static_cast<Base *>(h);
  const long n = b->dofsStencil();
  std::vector<double> aux(n), r1(n), r2(n), r3(n), r4(n);
  const double dt2 = dt / 2., dt6 = dt / 6., dt3 = dt / 3.;
  double t = t0;
  for (long s = 0; s < nsteps; ++s) {
    b->velocity(U, t, r1.data());
    for (long i = 0; i < n; ++i) aux[i] = U[i] + dt2 * r1[i];
    b->velocity(aux.data(), t + dt2, r2.data());
    for (long i = 0; i < n; ++i) aux[i] = U[i] + dt2 * r2[i];
    b->velocity(aux.data(), t + dt2, r3.data());
    for (long i = 0; i < n; ++i) aux[i] = U[i] + dt * r3[i];
    b->velocity(aux.data(), t + dt, r4.data());
    for (long i = 0; i < n; ++i) U[i] = U[i] + dt6 * r1[i] + dt3 * r2[i] + dt3 * r3[i] + dt6 * r4[i];
    t = t + dt;
  }
}

// WENO known-answer entry points (impl/weno5.hpp, impl/weno3.hpp)
void ref_weno5(const double *q7, double *out4) {
  pda::weno5(out4[0], out4[1], out4[2], out4[3], q7[0], q7[1], q7[2], q7[3], q7[4], q7[5], q7[6]);
}
void ref_weno3(const double *q5, double *out4) {
  pda::weno3(out4[0], out4[1], out4[2], out4[3], q5[0], q5[1], q5[2], q5[3], q5[4]);
}

}  // extern "C"
