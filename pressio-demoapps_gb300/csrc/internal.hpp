// Host-side internals shared by the mesh, problem and stepper translation
// units.  Nothing here crosses the C ABI.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pda_gb300.h"

namespace pda {

// Error carried to the C ABI as a status code plus a thread-local message.
struct Error : std::runtime_error {
  pda_status code;
  Error(pda_status c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string &msg);

#define PDA_REQUIRE(cond, code, msg) \
  do {                               \
    if (!(cond)) throw ::pda::Error((code), (msg)); \
  } while (0)

// Cell-centered uniform mesh, the in-memory form of the three mesh files
// (impl/mesh_ccu.hpp:60-473).
struct Mesh {
  int dim = 0;
  double dx[3] = {0, 0, 0};
  double dxInv[3] = {0, 0, 0};
  int stencil = 0;
  int64_t stencilMeshSize = 0;
  int64_t sampleMeshSize = 0;
  int ncols = 0;                 // 1 + (stencil-1)*dim
  std::vector<int32_t> graph;    // [sampleMeshSize][ncols]
  std::vector<double> x, y, z;   // [stencilMeshSize]
  std::vector<int32_t> inner;    // graph rows away from the boundary
  std::vector<int32_t> nearBd;   // graph rows near a non-periodic boundary
  bool fullyPeriodic = false;
  // natural-order full mesh descriptor (structured fast path)
  bool structured = false;
  int n[3] = {1, 1, 1};
  int periodic[3] = {0, 0, 0};
  // extra info.dat entries kept for writing the files back
  double bounds[6] = {0, 0, 0, 0, 0, 0};
  bool hasBounds = false;

  int32_t g(int64_t row, int col) const { return graph[row * ncols + col]; }
  void classify();  // fills inner / nearBd / fullyPeriodic
};

// text round-trip that the reference's files impose on coordinates and dx
double round14(double v);

Mesh mesh_generate_full(const int n[3], const double bounds[6], int stencil, const int periodic[3]);
Mesh mesh_load(const std::string &dir);
void mesh_write(const Mesh &m, const std::string &dir);
void mesh_write_binary(const Mesh &m, const std::string &path);
Mesh mesh_load_binary(const std::string &path);
Mesh mesh_sample(const Mesh &full, const std::vector<int64_t> &gids, std::vector<int64_t> *stencilGids);
void mesh_detect_structure(Mesh &m, const int nInfo[3], bool haveN);

}  // namespace pda
