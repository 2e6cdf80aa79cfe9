// Host-side state of a device problem (pda_problem) and the small device
// buffer / row-table helpers it is built from; shared by problem.cpp and
// batch.cpp.  Nothing here crosses the C ABI.
#pragma once

#include <cstdint>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "internal.hpp"
#include "launch.hpp"

namespace pda {

#define PDA_CUDA(x)                                                                           \
  do {                                                                                        \
    cudaError_t e_ = (x);                                                                     \
    if (e_ != cudaSuccess)                                                                    \
      throw ::pda::Error(PDA_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));      \
  } while (0)

template <class T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count <= n && p) return;
    release();
    if (count == 0) return;
    cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      throw Error(e == cudaErrorMemoryAllocation ? PDA_ERR_OUT_OF_MEMORY : PDA_ERR_CUDA,
                  std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    n = count;
  }
  void upload(const std::vector<T> &v) {
    alloc(v.size());
    if (!v.empty()) PDA_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  }
};

// Host copy + device copy of a row table.
struct Table {
  std::vector<int> rows, cell, src, jpos, src1, jpos1;
  std::vector<uint8_t> flip, flip1;
  std::vector<double> jfac;
  std::vector<double> gsx, gsy, gsx1, gsy1;  // moving-shock ghost positions (empty unless used)
  DevBuf<int> d_rows, d_cell, d_src, d_jpos, d_src1, d_jpos1;
  DevBuf<uint8_t> d_flip, d_flip1;
  DevBuf<double> d_jfac, d_gsx, d_gsy, d_gsx1, d_gsy1;
  RowTable t{};
  bool dirty = true;
  int hostRows() const { return (int)rows.size(); }
  // copy the host tables to the device if they changed since the last copy
  void sync() {
    if (!dirty) return;
    upload();
    dirty = false;
  }
  void upload() {
    d_rows.upload(rows);
    d_cell.upload(cell);
    d_src.upload(src);
    d_flip.upload(flip);
    d_jpos.upload(jpos);
    d_src1.upload(src1);
    d_flip1.upload(flip1);
    d_jpos1.upload(jpos1);
    d_jfac.upload(jfac);
    d_gsx.upload(gsx);
    d_gsy.upload(gsy);
    d_gsx1.upload(gsx1);
    d_gsy1.upload(gsy1);
    t.nrows = (int)rows.size();
    t.rows = d_rows.p;
    t.cell = d_cell.p;
    t.src = d_src.p;
    t.flip = d_flip.p;
    t.jpos = jpos.empty() ? nullptr : d_jpos.p;
    t.src1 = src1.empty() ? nullptr : d_src1.p;
    t.flip1 = flip1.empty() ? nullptr : d_flip1.p;
    t.jpos1 = jpos1.empty() ? nullptr : d_jpos1.p;
    t.jfac = jfac.empty() ? nullptr : d_jfac.p;
    t.gsx = gsx.empty() ? nullptr : d_gsx.p;
    t.gsy = gsy.empty() ? nullptr : d_gsy.p;
    t.gsx1 = gsx1.empty() ? nullptr : d_gsx1.p;
    t.gsy1 = gsy1.empty() ? nullptr : d_gsy1.p;
  }
};

// ghost-cell rules: BC_MIRROR2D = Ghost2dNeumannFiller / InviscidWallFiller,
// BC_NEUMANN1D = Ghost1dNeumannFiller, BC_SEDOVSYM = Sedov2dSymmetryGhostFiller
// (layer L >= 1 copies the opposite-side neighbour L-1; reflective on the
// left and bottom sides, Neumann on the right and top), BC_NORMALSHOCK =
// NormalShock2dGhostFiller (same layer rule; reflective top and bottom,
// Neumann left and right), BC_DMR = DoubleMachReflection2dGhostFiller (same
// layer rule; moving oblique shock on the top, wall behind the wedge on the
// bottom), BC_CROSSSHOCK = CrossShock2dGhostFiller (same layer rule; inflow
// state on the left, prescribed momentum on the bottom)
enum BcKind {
  BC_NONE = 0,
  BC_MIRROR2D = 1,
  BC_NEUMANN1D = 2,
  BC_SEDOVSYM = 3,
  BC_NORMALSHOCK = 4,
  BC_DMR = 5,
  BC_CROSSSHOCK = 6
};

}  // namespace pda

namespace pda {
// row bands of the host-buffer velocity (velocity_host_banded); measured at
// 1024^2 with the copies at about 300 GB/s: 2, 3, 4, 6, 8 bands gave 1.565,
// 1.556, 1.584, 1.535, 1.701 ms per call
constexpr int kHostBands = 6;
// the arguments and device buffers a captured host-buffer velocity graph is
// bound to
struct HostGraphKey {
  const double *hU = nullptr;
  const double *hV = nullptr;
  double t = 0;
  const double *U = nullptr, *V = nullptr, *Fx = nullptr, *Fy = nullptr;
  bool operator==(const HostGraphKey &o) const {
    return hU != nullptr && hU == o.hU && hV == o.hV && t == o.t && U == o.U && V == o.V && Fx == o.Fx &&
           Fy == o.Fy;
  }
};
}  // namespace pda

struct pda_mesh {
  pda::Mesh m;
};

struct pda_problem {
  const pda::Mesh *mesh = nullptr;
  int family = 0, probEnum = 0, scheme = 0, icFlag = 1;
  std::vector<double> icParams, physParams;
  pda::Phys phys{};
  pda::MeshArgs margs{};
  cudaStream_t stream = nullptr;
  // second stream + events: inner and near-boundary row kernels run side by side
  cudaStream_t side = nullptr;
  cudaEvent_t evFork = nullptr, evJoin = nullptr;
  // host-buffer velocity in row bands: one compute stream per band (earlier
  // bands at higher priority), a copy stream and their events (created on
  // first use)
  cudaStream_t hostBand[pda::kHostBands] = {}, hostCopy = nullptr;
  cudaEvent_t hostEv[3 * pda::kHostBands + 3] = {};
  // the host-buffer velocity as one graph, for repeated calls with the same
  // arguments (velocity_host_banded)
  cudaGraphExec_t hostGraph = nullptr;
  pda::HostGraphKey hostGraphKey{}, hostLastKey{};
  int ndpc = 0, dim = 0, h = 0;
  int64_t dofsSample = 0, dofsStencil = 0;
  int bc = pda::BC_NONE;
  bool timeDependent = false;  // ghost states depend on the evaluation time
  std::vector<pda::GhostRecipe> recipes;  // ghost recipes with ids >= 2
  pda::DevBuf<pda::GhostRecipe> d_recipes;
  const pda::Launchers *L = nullptr;
  // velocity
  bool useStruct = false;
  bool structAll = false;  // the structured box covers every cell (mirror boundaries)
  pda::Box box{};
  pda::DevBuf<double> F[3];
  // Jacobian, faces once on the inner box (jfaces.cuh)
  bool jStruct = false;
  pda::Box jbox{};

  pda::Table nearT;   // near-boundary rows: V stencil (+ J first-order tables)
  pda::Table innerT;  // inner rows (sample meshes for V; every mesh for V+J)
  bool innerBuiltV = false, innerBuiltJ = false, nearBuiltJ = false;
  // Jacobian
  bool patternBuilt = false;
  std::vector<int> rowptr, colidx;
  std::vector<std::vector<int32_t>> rowBlocks;  // sorted unique cell ids per graph row
  pda::DevBuf<int> d_rowptr, d_colidx;
  pda::DevBuf<double> d_Jscratch, d_Vscratch;
  // host-buffer entry points and steppers
  pda::DevBuf<double> d_U, d_V, d_J;
  pda::DevBuf<double> aux, r[4];
  cudaGraphExec_t stepGraph = nullptr;
  int stepGraphKind = -1;
  double stepGraphDt = 0;
  double *stepGraphU = nullptr;
  int64_t stepGraphLaunches = 0;
  int64_t launches = 0;
  ~pda_problem() {
    if (stepGraph) cudaGraphExecDestroy(stepGraph);
    if (hostGraph) cudaGraphExecDestroy(hostGraph);
    if (side) cudaStreamDestroy(side);
    if (evFork) cudaEventDestroy(evFork);
    if (evJoin) cudaEventDestroy(evJoin);
    for (cudaStream_t h : hostBand)
      if (h) cudaStreamDestroy(h);
    if (hostCopy) cudaStreamDestroy(hostCopy);
    for (cudaEvent_t e : hostEv)
      if (e) cudaEventDestroy(e);
  }
};

namespace pda {
// build the CSR pattern of the problem and copy it to the device (once)
void ensure_device_pattern(pda_problem &P);
// inner and near-boundary row tables with their Jacobian parts, the CSR
// pattern and the ghost recipes on the device (allocates; call before any
// stream capture)
void ensure_row_tables(pda_problem &P);
}  // namespace pda

// C ABI bodies: exceptions become a status code + the thread-local message
// 1D full meshes below this many cells evaluate every row with the per-row
// kernel: the face pass takes 61 faces per block, so below ~61 x 152 cells its
// grid does not cover GB300's SMs and a call costs one whole-face FP64
// instruction stream per warp
constexpr long kRowsOnlyCells1D = 8192;

#define PDA_API_BEGIN try {
#define PDA_API_END                                   \
  return PDA_OK;                                      \
  }                                                   \
  catch (const pda::Error &e) {                       \
    pda::set_last_error(e.what());                    \
    return e.code;                                    \
  }                                                   \
  catch (const std::bad_alloc &) {                    \
    pda::set_last_error("host out of memory");        \
    return PDA_ERR_OUT_OF_MEMORY;                     \
  }                                                   \
  catch (const std::exception &e) {                   \
    pda::set_last_error(e.what());                    \
    return PDA_ERR_INTERNAL;                          \
  }
