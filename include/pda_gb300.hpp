// pda_gb300.hpp -- header-only C++ wrapper over the C ABI (pda_gb300.h) with
// the method names of pressio-demoapps' PublicProblemEigenMixinCpp
// (include/pressiodemoapps/adapter_cpp.hpp:59-264), so a device problem is a
// drop-in beside the Eigen one:
//
//   auto mesh = pda_gb300::load_cellcentered_uniform_mesh("path/to/mesh");
//   auto app  = pda_gb300::create_problem(mesh, pda_gb300::Euler2d::Riemann,
//                                         pda_gb300::InviscidFluxReconstruction::Weno5, 2);
//   Eigen::VectorXd U = app.initialCondition<Eigen::VectorXd>();
//   Eigen::VectorXd V = app.createRightHandSide<Eigen::VectorXd>();
//   app.rightHandSide(U, 0.0, V);                  // host vectors: copies in/out
//   auto J = app.createJacobian<Eigen::SparseMatrix<double, Eigen::RowMajor, int>>();
//   app.rightHandSideAndJacobian(U, 0.0, V, J);    // values filled in place
//
// Host containers need data()/size() (vectors) or the compressed-storage
// accessors of Eigen::SparseMatrix (outerIndexPtr/innerIndexPtr/valuePtr,
// resizeNonZeros).  Device-pointer overloads take d_ pointers directly.
// Errors become std::runtime_error, as in the reference.
#ifndef PDA_GB300_HPP_
#define PDA_GB300_HPP_

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "pda_gb300.h"

namespace pda_gb300 {

enum class InviscidFluxReconstruction { FirstOrder = 0, Weno3 = 1, Weno5 = 2 };
enum class Euler1d { PeriodicSmooth = 0, Sod = 1, Lax = 2, ShuOsher = 3 };
enum class Euler2d {
  PeriodicSmooth = 0, KelvinHelmholtz = 1, SedovFull = 2, SedovSymmetry = 3, Riemann = 4,
  NormalShock = 5, DoubleMachReflection = 6, CrossShock = 7, testingonlyneumann = 8
};
enum class Euler3d { PeriodicSmooth = 0, SedovSymmetry = 1 };
enum class Swe2d { SlipWall = 0, CustomBCs = 1 };

inline void check(pda_status s) {
  if (s != PDA_OK) throw std::runtime_error(std::string("pda_gb300: ") + pda_last_error());
}

class Mesh {
 public:
  explicit Mesh(pda_mesh *h) : h_(h, &pda_mesh_free) {}
  const pda_mesh *get() const { return h_.get(); }
  int dimensionality() const { return info().first[0]; }
  int stencilSize() const { return info().first[1]; }
  int64_t stencilMeshSize() const { return info().second[0]; }
  int64_t sampleMeshSize() const { return info().second[1]; }
  // the library's one-file binary format (load_mesh_binary reads it back)
  void write_binary(const std::string &path) const { check(pda_mesh_write_binary(h_.get(), path.c_str())); }

 private:
  std::pair<std::vector<int>, std::vector<int64_t>> info() const {
    std::vector<int> d(3);
    std::vector<int64_t> s(4);
    check(pda_mesh_info(h_.get(), d.data(), s.data(), nullptr, nullptr, nullptr));
    return {d, s};
  }
  std::shared_ptr<pda_mesh> h_;
};

inline Mesh load_cellcentered_uniform_mesh(const std::string &dir) {
  pda_mesh *m = nullptr;
  check(pda_mesh_load(dir.c_str(), &m));
  return Mesh(m);
}

inline Mesh load_mesh_binary(const std::string &path) {
  pda_mesh *m = nullptr;
  check(pda_mesh_load_binary(path.c_str(), &m));
  return Mesh(m);
}

class Problem {
 public:
  using scalar_type = double;

  Problem(const Mesh &mesh, int family, int problem, int scheme, int icFlag,
          const std::unordered_map<std::string, double> &params, void *stream = nullptr)
      : mesh_(mesh), h_(nullptr, &pda_problem_free) {
    std::vector<const char *> names;
    std::vector<double> vals;
    for (const auto &kv : params) {
      names.push_back(kv.first.c_str());
      vals.push_back(kv.second);
    }
    pda_problem *p = nullptr;
    check(pda_problem_create(mesh.get(), family, problem, scheme, icFlag, names.data(), vals.data(),
                             (int)names.size(), stream, &p));
    h_.reset(p);
    check(pda_problem_sizes(p, &ndpc_, &dofsSample_, &dofsStencil_));
  }
  Problem(const Problem &) = delete;
  Problem &operator=(const Problem &) = delete;
  Problem(Problem &&) = default;

  int numDofPerCell() const { return ndpc_; }
  int64_t totalDofSampleMesh() const { return dofsSample_; }
  int64_t totalDofStencilMesh() const { return dofsStencil_; }
  double queryParameter(const std::string &n) const {
    double v = 0;
    check(pda_query_parameter(h_.get(), n.c_str(), &v));
    return v;
  }
  double gamma() const { return queryParameter("gamma"); }
  double gravity() const { return queryParameter("gravity"); }
  double coriolis() const { return queryParameter("coriolis"); }

  // ---- host containers (Eigen::VectorXd, std::vector<double>, ...)
  template <class Vec> Vec initialCondition() const {
    Vec u(dofsStencil_);
    check(pda_initial_condition_host(h_.get(), u.data()));
    return u;
  }
  template <class Vec> Vec createState() const {
    Vec u(dofsStencil_);
    for (int64_t i = 0; i < dofsStencil_; ++i) u.data()[i] = 0.0;
    return u;
  }
  template <class Vec> Vec createRightHandSide() const {
    Vec v(dofsSample_);
    for (int64_t i = 0; i < dofsSample_; ++i) v.data()[i] = 0.0;
    return v;
  }
  template <class Vec> Vec createRhs() const { return createRightHandSide<Vec>(); }
  template <class Vec> Vec createVelocity() const { return createRightHandSide<Vec>(); }

  template <class Vec> void rightHandSide(const Vec &U, double t, Vec &V) const {
    check(pda_velocity_host(h_.get(), U.data(), t, V.data()));
  }
  template <class Vec> void rhs(const Vec &U, double t, Vec &V) const { rightHandSide(U, t, V); }
  template <class Vec> void velocity(const Vec &U, double t, Vec &V) const { rightHandSide(U, t, V); }
  template <class Vec> void operator()(const Vec &U, double t, Vec &V) const { rightHandSide(U, t, V); }

  // Eigen::SparseMatrix<double, RowMajor, int> (compressed) with the reference's pattern
  template <class SpMat> SpMat createJacobian() const {
    int64_t rows = 0, cols = 0, nnz = 0;
    check(pda_jacobian_shape(h_.get(), &rows, &cols, &nnz));
    SpMat J((typename SpMat::Index)rows, (typename SpMat::Index)cols);
    J.resizeNonZeros((typename SpMat::Index)nnz);
    check(pda_jacobian_pattern_host(h_.get(), J.outerIndexPtr(), J.innerIndexPtr()));
    for (int64_t q = 0; q < nnz; ++q) J.valuePtr()[q] = 0.0;
    return J;
  }
  template <class Vec, class SpMat>
  void rightHandSideAndJacobian(const Vec &U, double t, Vec &V, SpMat &J) const {
    check(pda_velocity_and_jacobian_host(h_.get(), U.data(), t, V.data(), J.valuePtr()));
  }
  template <class Vec, class SpMat> void jacobian(const Vec &U, double t, SpMat &J) const {
    std::vector<double> scratch((size_t)dofsSample_);
    check(pda_velocity_and_jacobian_host(h_.get(), U.data(), t, scratch.data(), J.valuePtr()));
  }

  // ---- device pointers (state resident in HBM)
  void velocity(const double *d_U, double t, double *d_V) { check(pda_velocity(h_.get(), d_U, t, d_V)); }
  void velocityAndJacobian(const double *d_U, double t, double *d_V, double *d_J) {
    check(pda_velocity_and_jacobian(h_.get(), d_U, t, d_V, d_J));
  }
  void jacobian(const double *d_U, double t, double *d_J) { check(pda_jacobian(h_.get(), d_U, t, d_J)); }
  void applyJacobian(const double *d_U, const double *d_B, int nCols, double t, double *d_R) {
    check(pda_apply_jacobian(h_.get(), d_U, t, d_B, nCols, d_R));
  }
  void initialCondition(double *d_U) { check(pda_initial_condition(h_.get(), d_U)); }
  void advanceSSPRK3(double *d_U, double t0, double dt, int64_t nSteps, bool graph = true) {
    check(pda_advance_ssprk3(h_.get(), d_U, t0, dt, nSteps, graph ? 1 : 0));
  }
  void advanceRK4(double *d_U, double t0, double dt, int64_t nSteps, bool graph = true) {
    check(pda_advance_rk4(h_.get(), d_U, t0, dt, nSteps, graph ? 1 : 0));
  }
  pda_problem *native() { return h_.get(); }

 private:
  Mesh mesh_;  // keeps the mesh alive as long as the problem
  std::unique_ptr<pda_problem, void (*)(pda_problem *)> h_;
  int ndpc_ = 0;
  int64_t dofsSample_ = 0, dofsStencil_ = 0;
};

// create_problem_eigen-style factories (euler1d.hpp:82, euler2d.hpp:88-173,
// euler3d.hpp:80-122, swe2d.hpp:143-195)
inline Problem create_problem(const Mesh &m, Euler1d p, InviscidFluxReconstruction r) {
  return Problem(m, PDA_EULER1D, (int)p, (int)r, 1, {});
}
inline Problem create_problem(const Mesh &m, Euler2d p, InviscidFluxReconstruction r, int icFlag = 1,
                              const std::unordered_map<std::string, double> &params = {}) {
  return Problem(m, PDA_EULER2D, (int)p, (int)r, icFlag, params);
}
inline Problem create_problem(const Mesh &m, Euler3d p, InviscidFluxReconstruction r) {
  return Problem(m, PDA_EULER3D, (int)p, (int)r, 1, {});
}
inline Problem create_problem(const Mesh &m, Swe2d p, InviscidFluxReconstruction r, int icFlag = 1,
                              const std::unordered_map<std::string, double> &params = {}) {
  return Problem(m, PDA_SWE2D, (int)p, (int)r, icFlag, params);
}

}  // namespace pda_gb300

#endif  // PDA_GB300_HPP_
