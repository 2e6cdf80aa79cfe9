// Batches of independent problems: packing, tile bookkeeping, the tile-shape
// autotuner, batched velocity and the batched SSP-RK3 integrator (one CUDA
// graph per step for all instances).
//
// The reference has no batch object: a caller that runs many parameter
// instances loops over problem objects, one velocity call (and, on a GPU,
// several kernel launches) per instance and stage.  Here the instances'
// states are packed into one vector and each phase of the residual is one
// launch over all of them (batch.cuh), with per-instance boxes, mesh
// spacings and physical parameters read from a device table.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "problem_impl.hpp"

struct pda_batch {
  std::vector<pda_problem *> probs;
  int family = 0, scheme = 0, ndpc = 0, dim = 0;
  cudaStream_t stream = nullptr;
  std::vector<pda::BatchItem> items;
  std::vector<int64_t> offsets;  // packed dof offsets [n + 1] (instances start on 256-byte boundaries)
  std::vector<int64_t> cells;    // cells per instance
  int64_t totalDofs = 0, totalCells = 0;
  int shape[3] = {0, 0, 0};
  pda::DevBuf<pda::BatchItem> d_items;
  pda::DevBuf<long> d_tileStart[3], d_blockStart;
  pda::BatchArgs args{};
  pda::DevBuf<double> F, aux;
  cudaGraphExec_t graph = nullptr;
  double graphDt = 0;
  double *graphU = nullptr;
  int64_t graphLaunches = 0;
  int64_t launches = 0;
  ~pda_batch() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

namespace pda {
namespace {

constexpr long kAlign = 32;  // doubles (256 bytes)
long align_up(long v) { return (v + kAlign - 1) / kAlign * kAlign; }

int scheme_halo(int scheme) { return scheme == PDA_WENO5 ? 3 : (scheme == PDA_WENO3 ? 2 : 1); }

// tiles of instance `it` along `axis` for the current shape
long tiles_of(const pda_batch &B, const BatchItem &bi, int axis) {
  const Box &b = bi.b;
  const long nfa = (long)(b.hi[axis] - b.lo[axis] + 1);
  if (B.scheme == PDA_FIRST_ORDER) {
    long nf = nfa;
    for (int c = 0; c < 3; ++c)
      if (c != axis) nf *= (long)(b.hi[c] - b.lo[c]);
    return (nf + kFoFacesPerTile - 1) / kFoFacesPerTile;
  }
  const TileShape ts = kTileShapes[B.shape[axis]];
  const long tw = ts.lanes - scheme_halo(B.scheme);
  return bi.groups[axis] * ((nfa + tw - 1) / tw);
}

void refresh_tiles(pda_batch &B, int axis) {
  const TileShape ts = kTileShapes[B.shape[axis]];
  std::vector<long> start(B.items.size() + 1, 0);
  for (size_t i = 0; i < B.items.size(); ++i) {
    BatchItem &bi = B.items[i];
    long lines = 1;
    for (int c = 0; c < 3; ++c)
      if (c != axis) lines *= (long)(bi.b.hi[c] - bi.b.lo[c]);
    bi.groups[axis] = (lines + ts.nr - 1) / ts.nr;
    start[i + 1] = start[i] + tiles_of(B, bi, axis);
  }
  B.d_tileStart[axis].upload(start);
  B.args.tileStart[axis] = B.d_tileStart[axis].p;
  B.args.totalTiles[axis] = start.back();
  B.d_items.upload(B.items);
  B.args.items = B.d_items.p;
  if (B.graph) {
    cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
  }
}

void batch_velocity(pda_batch &B, const double *U, double *V) {
  for (int a = 0; a < B.dim; ++a) {
    B.probs[0]->L->batch_faces(B.scheme, a, B.shape[a], B.args, U, B.F.p, B.stream);
    ++B.launches;
  }
  B.probs[0]->L->batch_balance(B.args, U, B.F.p, V, B.stream);
  ++B.launches;
  PDA_CUDA(cudaGetLastError());
}

void batch_buffers(pda_batch &B) {
  if (B.aux.p) return;
  B.aux.alloc((size_t)B.totalDofs);
  // entries between instances are never written by the kernels: keep them 0
  PDA_CUDA(cudaMemsetAsync(B.aux.p, 0, (size_t)B.totalDofs * sizeof(double), B.stream));
}

// One SSP-RK3 step, the single-problem stage formulas over the packed vector
// (ode_explicit_stepper_without_mass_matrix.hpp:230-282): per stage the face
// passes, then the balance fused with the stage update (no velocity buffer).
void batch_faces_all(pda_batch &B, const double *U) {
  for (int a = 0; a < B.dim; ++a) {
    B.probs[0]->L->batch_faces(B.scheme, a, B.shape[a], B.args, U, B.F.p, B.stream);
    ++B.launches;
  }
}

void batch_ssprk3_step(pda_batch &B, double *U, double dt) {
  double *aux = B.aux.p;
  const pda::Launchers &L = *B.probs[0]->L;
  const double fourInv = 1. / 4., threeOvFour = 3. / 4., oneOvThree = 1. / 3., twoOvThree = 2. / 3.;
  batch_faces_all(B, U);  // u_1 = u_n + dt rhs(u_n)
  L.batch_balance_stage(B.args, U, B.F.p, aux, U, 0, 0., dt, 0., B.stream);
  batch_faces_all(B, aux);  // u_2 = 3/4 u_n + 1/4 u_1 + 1/4 dt rhs(u_1)
  L.batch_balance_stage(B.args, aux, B.F.p, aux, U, 1, fourInv, threeOvFour, fourInv * dt, B.stream);
  batch_faces_all(B, aux);  // u_n+1 = 1/3 u_n + 2/3 u_2 + 2/3 dt rhs(u_2)
  L.batch_balance_stage(B.args, aux, B.F.p, U, aux, 1, oneOvThree, twoOvThree, twoOvThree * dt, B.stream);
  B.launches += 3;
  PDA_CUDA(cudaGetLastError());
}

void create_batch(pda_batch &B, pda_problem *const *probs, int n, void *stream) {
  PDA_REQUIRE(probs && n > 0, PDA_ERR_INVALID_ARGUMENT, "empty batch");
  B.stream = (cudaStream_t)stream;
  B.probs.assign(probs, probs + n);
  const pda_problem &P0 = *probs[0];
  B.family = P0.family;
  B.scheme = P0.scheme;
  B.ndpc = P0.ndpc;
  B.dim = P0.dim;
  B.offsets.assign(n + 1, 0);
  B.cells.assign(n, 0);
  std::vector<long> blockStart(n + 1, 0);
  long fTotal[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    const pda_problem *P = probs[i];
    PDA_REQUIRE(P, PDA_ERR_INVALID_ARGUMENT, "null problem in batch");
    PDA_REQUIRE(P->family == B.family && P->scheme == B.scheme, PDA_ERR_INVALID_ARGUMENT,
                "batch instance " + std::to_string(i) + ": every instance needs the same family and scheme");
    PDA_REQUIRE(P->useStruct && (P->structAll || P->nearT.hostRows() == 0), PDA_ERR_UNSUPPORTED,
                "batch instance " + std::to_string(i) +
                    ": batches take full natural-order meshes whose boundaries are periodic or mirror "
                    "images (slip wall, 2D Neumann)");
    BatchItem bi{};
    bi.b = P->box;
    bi.m = P->margs;
    bi.p = P->phys;
    bi.uOff = (long)B.offsets[i];
    B.offsets[i + 1] = B.offsets[i] + align_up((long)P->dofsStencil);
    long nc = 1;
    for (int c = 0; c < 3; ++c) nc *= (long)(bi.b.hi[c] - bi.b.lo[c]);
    B.cells[i] = nc;
    B.totalCells += nc;
    blockStart[i + 1] = blockStart[i] + (nc + kBalanceBlock - 1) / kBalanceBlock;
    for (int a = 0; a < B.dim; ++a) {
      long nf = (long)B.ndpc;
      for (int c = 0; c < 3; ++c) nf *= (long)(bi.b.hi[c] - bi.b.lo[c] + (c == a ? 1 : 0));
      bi.fOff[a] = fTotal[a];
      fTotal[a] += align_up(nf);
    }
    B.items.push_back(bi);
  }
  B.totalDofs = B.offsets[n];
  // faces of all instances normal to x, then y, then z
  long fBase = 0;
  for (int a = 0; a < B.dim; ++a) {
    for (auto &bi : B.items) bi.fOff[a] += fBase;
    fBase += fTotal[a];
  }
  B.F.alloc((size_t)std::max(fBase, 1L));
  B.args.nItems = n;
  B.d_blockStart.upload(blockStart);
  B.args.blockStart = B.d_blockStart.p;
  B.args.totalBlocks = blockStart.back();
  for (int a = 0; a < B.dim; ++a) refresh_tiles(B, a);
}

}  // namespace
}  // namespace pda

using pda::Error;

extern "C" {

pda_status pda_batch_create(pda_problem *const *problems, int n, void *stream, pda_batch **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(out, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_ptr<pda_batch> b(new pda_batch);
  pda::create_batch(*b, problems, n, stream);
  *out = b.release();
  PDA_API_END
}

void pda_batch_free(pda_batch *b) { delete b; }

pda_status pda_batch_sizes(const pda_batch *b, int *n, int64_t *total_dofs, int64_t *total_cells) {
  PDA_API_BEGIN
  PDA_REQUIRE(b, PDA_ERR_INVALID_ARGUMENT, "null argument");
  if (n) *n = (int)b->probs.size();
  if (total_dofs) *total_dofs = b->totalDofs;
  if (total_cells) *total_cells = b->totalCells;
  PDA_API_END
}

pda_status pda_batch_offsets(const pda_batch *b, int64_t *offsets) {
  PDA_API_BEGIN
  PDA_REQUIRE(b && offsets, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::memcpy(offsets, b->offsets.data(), b->offsets.size() * sizeof(int64_t));
  PDA_API_END
}

pda_status pda_batch_initial_condition(pda_batch *b, double *d_U) {
  PDA_API_BEGIN
  PDA_REQUIRE(b && d_U, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<double> h((size_t)b->totalDofs, 0.0);
  for (size_t i = 0; i < b->probs.size(); ++i) {
    const pda_status s = pda_initial_condition_host(b->probs[i], h.data() + b->offsets[i]);
    if (s != PDA_OK) throw Error(s, pda_last_error());
  }
  PDA_CUDA(cudaMemcpyAsync(d_U, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  PDA_CUDA(cudaStreamSynchronize(b->stream));
  PDA_API_END
}

pda_status pda_batch_velocity(pda_batch *b, const double *d_U, double t, double *d_V) {
  PDA_API_BEGIN
  PDA_REQUIRE(b && d_U && d_V, PDA_ERR_INVALID_ARGUMENT, "null argument");
  (void)t;
  pda::batch_velocity(*b, d_U, d_V);
  PDA_API_END
}

pda_status pda_batch_advance_ssprk3(pda_batch *b, double *d_U, double t0, double dt, int64_t n_steps,
                                    int use_graph) {
  PDA_API_BEGIN
  PDA_REQUIRE(b && d_U, PDA_ERR_INVALID_ARGUMENT, "null argument");
  PDA_REQUIRE(n_steps >= 0, PDA_ERR_INVALID_ARGUMENT, "negative step count");
  (void)t0;
  pda_batch &B = *b;
  pda::batch_buffers(B);
  if (!use_graph || B.stream == nullptr) {
    for (int64_t s = 0; s < n_steps; ++s) pda::batch_ssprk3_step(B, d_U, dt);
    return PDA_OK;
  }
  if (B.graph && (B.graphDt != dt || B.graphU != d_U)) {
    cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
  }
  if (!B.graph) {
    PDA_CUDA(cudaStreamSynchronize(B.stream));
    cudaGraph_t g;
    PDA_CUDA(cudaStreamBeginCapture(B.stream, cudaStreamCaptureModeThreadLocal));
    const int64_t before = B.launches;
    try {
      pda::batch_ssprk3_step(B, d_U, dt);
    } catch (...) {
      cudaStreamEndCapture(B.stream, &g);
      throw;
    }
    PDA_CUDA(cudaStreamEndCapture(B.stream, &g));
    B.graphLaunches = B.launches - before;
    B.launches = before;
    PDA_CUDA(cudaGraphInstantiate(&B.graph, g, 0));
    cudaGraphDestroy(g);
    B.graphDt = dt;
    B.graphU = d_U;
  }
  for (int64_t s = 0; s < n_steps; ++s) PDA_CUDA(cudaGraphLaunch(B.graph, B.stream));
  B.launches += n_steps * B.graphLaunches;
  PDA_API_END
}

int pda_batch_num_tile_shapes(const pda_batch *b) {
  if (!b || b->scheme == 0) return 1;
  return b->probs[0]->L->batch_num_shapes();
}

pda_status pda_batch_set_tile_shape(pda_batch *b, int axis, int shape) {
  PDA_API_BEGIN
  PDA_REQUIRE(b && axis >= 0 && axis < b->dim, PDA_ERR_INVALID_ARGUMENT, "invalid axis");
  PDA_REQUIRE(shape >= 0 && shape < pda_batch_num_tile_shapes(b), PDA_ERR_INVALID_ARGUMENT,
              "tile shape not compiled for this family / scheme");
  if (b->shape[axis] != shape) {
    b->shape[axis] = shape;
    pda::refresh_tiles(*b, axis);
  }
  PDA_API_END
}

pda_status pda_batch_tile_shape(const pda_batch *b, int axis, int *shape, int *lanes, int *lines) {
  PDA_API_BEGIN
  PDA_REQUIRE(b && axis >= 0 && axis < b->dim, PDA_ERR_INVALID_ARGUMENT, "invalid axis");
  const int s = b->shape[axis];
  if (shape) *shape = s;
  if (lanes) *lanes = b->scheme == 0 ? pda::kFoFacesPerTile : pda::kTileShapes[s].lanes;
  if (lines) *lines = b->scheme == 0 ? 1 : pda::kTileShapes[s].nr;
  PDA_API_END
}

pda_status pda_batch_autotune(pda_batch *b, const double *d_U, int reps, double *ms) {
  PDA_API_BEGIN
  PDA_REQUIRE(b && d_U && reps > 0, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  pda_batch &B = *b;
  const int ns = pda_batch_num_tile_shapes(b);
  cudaEvent_t e0, e1;
  PDA_CUDA(cudaEventCreate(&e0));
  PDA_CUDA(cudaEventCreate(&e1));
  for (int a = 0; a < B.dim; ++a) {
    int best = B.shape[a];
    double bestMs = 1e300;
    for (int s = 0; s < ns; ++s) {
      if (B.shape[a] != s) {
        B.shape[a] = s;
        pda::refresh_tiles(B, a);
      }
      B.probs[0]->L->batch_faces(B.scheme, a, s, B.args, d_U, B.F.p, B.stream);  // warm-up
      PDA_CUDA(cudaEventRecord(e0, B.stream));
      for (int r = 0; r < reps; ++r) B.probs[0]->L->batch_faces(B.scheme, a, s, B.args, d_U, B.F.p, B.stream);
      PDA_CUDA(cudaEventRecord(e1, B.stream));
      PDA_CUDA(cudaEventSynchronize(e1));
      PDA_CUDA(cudaGetLastError());
      B.launches += reps + 1;
      float t = 0;
      PDA_CUDA(cudaEventElapsedTime(&t, e0, e1));
      const double m = t / reps;
      if (ms) ms[a * ns + s] = m;
      if (m < bestMs) {
        bestMs = m;
        best = s;
      }
    }
    if (B.shape[a] != best) {
      B.shape[a] = best;
      pda::refresh_tiles(B, a);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  PDA_API_END
}

int64_t pda_batch_launch_count(const pda_batch *b) { return b ? b->launches : 0; }

}  // extern "C"
