// Test infrastructure only: drives the reference's own hyper-reduced LSPG --
// Pressio (vendored with the reference under tests_cpp/pressio) over the
// reference's own shallow-water problem on a sample mesh -- to produce golden
// latent trajectories for the LSPG oracle and the device LSPG.  Built by
// `make -C oracle lspgref REF=<reference checkout>` into oracle/_ref/ and run
// by tests/golden/make_lspg_golden.py; never part of the library.
//
// Pieces (all the reference's / Pressio's code paths):
//   * FOM: pressiodemoapps::create_problem_eigen on the sample mesh
//     (swe2d.hpp:143-195), slip wall, WENO5;
//   * trial space: pressio::rom::create_trial_column_subspace (affine:
//     y = u_ref + Phi x over the stencil mesh);
//   * hyper-reduction: the updater below, a = alpha a + beta b[stencil of
//     each sample row] (the operation Pressio's
//     LspgUnsteadyResidualJacobianPolicyHypRed asks of it);
//   * problem: pressio::rom::lspg::create_unsteady_problem(BDF1 | BDF2, ...)
//     (rom/lspg_unsteady.hpp:130-153);
//   * solver: pressio::create_gauss_newton_solver with a fixed number of
//     iterations per step (Stop::AfterMaxIters), normal equations solved by
//     Pressio's dense QR linear solver;
//   * pressio::ode::advance_n_steps.
//
// usage: lspg_ref <sample mesh dir> <s2st file> <phi file> <uref file> <x0 file> <k> <dt> <steps>
//                 <order 1|2> <gn iters> <gravity> <coriolis> <pulse> <out file>
// Files are raw little-endian doubles (phi row-major, stencil dofs x k) and
// s2st a raw int64 array; out receives the latent after every step.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "pressio/ode_advancers.hpp"
#include "pressio/ode_steppers_implicit.hpp"
#include "pressio/rom_lspg_unsteady.hpp"
#include "pressio/rom_subspaces.hpp"
#include "pressio/solvers_linear.hpp"
#include "pressio/solvers_nonlinear_gaussnewton.hpp"
#include "pressiodemoapps/swe2d.hpp"

namespace {

template <class T> std::vector<T> read_raw(const std::string &path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  const std::streamsize n = f.tellg();
  f.seekg(0);
  std::vector<T> v((size_t)n / sizeof(T));
  f.read(reinterpret_cast<char *>(v.data()), n);
  return v;
}

// a (sample-mesh operand) = alpha a + beta b (its stencil-mesh counterpart,
// row s2st[i] * ndpc + d of b for row i * ndpc + d of a)
struct HypRedUpdater {
  std::vector<int64_t> s2st;
  int ndpc;
  void updateSampleMeshOperandWithStencilMeshOne(Eigen::VectorXd &a, double alpha, const Eigen::VectorXd &b,
                                                 double beta) const {
    for (size_t i = 0; i < s2st.size(); ++i)
      for (int d = 0; d < ndpc; ++d) {
        const long r = (long)i * ndpc + d, s = (long)s2st[i] * ndpc + d;
        a(r) = alpha * a(r) + beta * b(s);
      }
  }
  void updateSampleMeshOperandWithStencilMeshOne(Eigen::MatrixXd &a, double alpha, const Eigen::MatrixXd &b,
                                                 double beta) const {
    for (size_t i = 0; i < s2st.size(); ++i)
      for (int d = 0; d < ndpc; ++d) {
        const long r = (long)i * ndpc + d, s = (long)s2st[i] * ndpc + d;
        for (long c = 0; c < a.cols(); ++c) a(r, c) = alpha * a(r, c) + beta * b(s, c);
      }
  }
};

}  // namespace

int main(int argc, char **argv) {
  if (argc != 15) {
    std::fprintf(stderr, "usage: %s mesh s2st phi uref x0 k dt steps order iters gravity coriolis pulse out\n",
                 argv[0]);
    return 2;
  }
  namespace pda = pressiodemoapps;
  const std::string meshDir = argv[1];
  const auto s2st = read_raw<int64_t>(argv[2]);
  const auto phiv = read_raw<double>(argv[3]);
  const auto urefv = read_raw<double>(argv[4]);
  const auto x0v = read_raw<double>(argv[5]);
  const int k = std::atoi(argv[6]);
  const double dt = std::atof(argv[7]);
  const int steps = std::atoi(argv[8]);
  const int order = std::atoi(argv[9]);
  const int iters = std::atoi(argv[10]);
  const double gravity = std::atof(argv[11]), coriolis = std::atof(argv[12]), pulse = std::atof(argv[13]);

  const auto mesh = pda::load_cellcentered_uniform_mesh_eigen(meshDir);
  auto fom = pda::create_slip_wall_swe_2d_problem_eigen(mesh, pda::InviscidFluxReconstruction::Weno5, gravity,
                                                        coriolis, pulse);
  const long nst = (long)urefv.size();
  Eigen::MatrixXd phi(nst, k);
  for (long r = 0; r < nst; ++r)
    for (int c = 0; c < k; ++c) phi(r, c) = phiv[(size_t)r * k + c];
  Eigen::VectorXd uref(nst);
  for (long r = 0; r < nst; ++r) uref(r) = urefv[(size_t)r];

  using reduced_state_t = Eigen::VectorXd;
  const auto space = pressio::rom::create_trial_column_subspace<reduced_state_t>(phi, uref, true);
  HypRedUpdater up{s2st, 3};
  const auto scheme = order == 2 ? pressio::ode::StepScheme::BDF2 : pressio::ode::StepScheme::BDF1;
  auto problem = pressio::rom::lspg::create_unsteady_problem(scheme, space, fom, up);
  auto &stepper = problem.lspgStepper();

  using hessian_t = Eigen::MatrixXd;
  using lin_solver_t = pressio::linearsolvers::Solver<pressio::linearsolvers::direct::HouseholderQR, hessian_t>;
  lin_solver_t linSolver;
  auto solver = pressio::create_gauss_newton_solver(stepper, linSolver);
  solver.setStopCriterion(pressio::nonlinearsolvers::Stop::AfterMaxIters);
  solver.setMaxIterations(iters);

  reduced_state_t x(k);
  for (int c = 0; c < k; ++c) x(c) = x0v[(size_t)c];
  std::vector<double> traj;
  auto observer = [&](pressio::ode::StepCount, double, const reduced_state_t &xs) {
    for (int c = 0; c < k; ++c) traj.push_back(xs(c));
  };
  pressio::ode::advance_n_steps(stepper, x, 0.0, dt, pressio::ode::StepCount(steps), observer, solver);
  std::ofstream f(argv[14], std::ios::binary);
  f.write(reinterpret_cast<const char *>(traj.data()), (std::streamsize)(traj.size() * sizeof(double)));
  std::printf("ok %zu latent states\n", traj.size() / (size_t)k);
  return 0;
}
