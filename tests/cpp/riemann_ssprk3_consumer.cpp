// A C++ consumer of the library through include/pda_gb300.hpp, following the
// flow of the reference test tests_cpp/eigen_2d_euler_riemann_explicit/main.cc:
// load a mesh (here also written to and read back from the library's binary
// mesh file), create_problem(Euler2d::Riemann, scheme, icFlag 2), take the
// initial condition, advance SSP-RK3 with dt = 0.01 for 0.6 / dt steps.
//
// Two drivers over the same problem object:
//   * host: the stepper owns std::vector states and calls rightHandSide()
//     with host vectors (each call copies U in and V out), applying the
//     stage updates of Pressio's SSP-RK3
//     (ode_explicit_stepper_without_mass_matrix.hpp:230-282) with Pressio's
//     ops::update association on the host;
//   * device: the state lives in device memory and advanceSSPRK3() runs the
//     steps on the GPU.
// Both final states are written as raw doubles for the test to compare with
// the reference's rho/p golds.  Built by tests/test_cpp_consumer.py with
// host FMA contraction off, so the host updates round like the reference's.
//
// usage: riemann_ssprk3_consumer <mesh dir> <scheme 0|1|2> <dt> <steps> <out host> <out device>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "pda_gb300.hpp"

namespace {

void write(const std::string &path, const std::vector<double> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(double)));
}

bool cuda_ok(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
  return false;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 7) {
    std::fprintf(stderr, "usage: %s mesh scheme dt steps out_host out_device\n", argv[0]);
    return 2;
  }
  namespace pda = pda_gb300;
  // the reference's text mesh, passed through the library's binary mesh
  // file (written next to the outputs, then loaded back)
  const auto textMesh = pda::load_cellcentered_uniform_mesh(argv[1]);
  const std::string binPath = std::string(argv[5]) + ".mesh.bin";
  textMesh.write_binary(binPath);
  const auto mesh = pda::load_mesh_binary(binPath);
  const auto order = static_cast<pda::InviscidFluxReconstruction>(std::atoi(argv[2]));
  const double dt = std::atof(argv[3]);
  const long nsteps = std::atol(argv[4]);
  auto app = pda::create_problem(mesh, pda::Euler2d::Riemann, order, 2);
  using state_t = std::vector<double>;

  // ---- host-driven SSP-RK3 through the host-vector right-hand side
  state_t u = app.initialCondition<state_t>();
  state_t aux = app.createState<state_t>();
  state_t rhs = app.createRightHandSide<state_t>();
  const size_t n = u.size();
  constexpr double one = 1., two = 2., three = 3., four = 4.;
  constexpr double oneOvThree = one / three, twoOvThree = two / three, threeOvFour = three / four,
                   fourInv = one / four;
  double t = 0.0;
  for (long step = 0; step < nsteps; ++step) {
    const double tHalf = t + dt / two, tNext = t + dt;
    app.rightHandSide(u, t, rhs);
    for (size_t i = 0; i < n; ++i) aux[i] = u[i] + dt * rhs[i];  // 0 aux + 1 u + dt rhs
    app.rightHandSide(aux, tNext, rhs);
    const double c2 = fourInv * dt;
    for (size_t i = 0; i < n; ++i) aux[i] = fourInv * aux[i] + threeOvFour * u[i] + c2 * rhs[i];
    app.rightHandSide(aux, tHalf, rhs);
    const double c3 = twoOvThree * dt;
    for (size_t i = 0; i < n; ++i) u[i] = oneOvThree * u[i] + twoOvThree * aux[i] + c3 * rhs[i];
    t = (double)(step + 1) * dt;
  }
  write(argv[5], u);

  // ---- device-resident state, steps on the GPU
  state_t u0 = app.initialCondition<state_t>();
  double *d_u = nullptr;
  if (!cuda_ok(cudaMalloc(&d_u, n * sizeof(double)), "cudaMalloc")) return 1;
  if (!cuda_ok(cudaMemcpy(d_u, u0.data(), n * sizeof(double), cudaMemcpyHostToDevice), "H2D")) return 1;
  app.advanceSSPRK3(d_u, 0.0, dt, nsteps);
  state_t ud(n);
  if (!cuda_ok(cudaMemcpy(ud.data(), d_u, n * sizeof(double), cudaMemcpyDeviceToHost), "D2H")) return 1;
  cudaFree(d_u);
  write(argv[6], ud);
  std::printf("ok %zu dofs, %ld steps\n", n, nsteps);
  return 0;
}
