// Plain-data descriptors shared by host code and kernels.
#pragma once

#include <stdint.h>

namespace pda {

enum Family : int { Euler1d = 0, Euler2d = 1, Euler3d = 2, Swe2d = 3 };

struct Phys {
  double gamma;
  double gravity;
  double coriolis;
};

// ---------------------------------------------------------------------------
// Row tables (built on the host, see problem.cpp)
// ---------------------------------------------------------------------------
struct RowTable {
  int nrows;
  const int *rows;         // graph row (sample-mesh index) of each entry
  const int *cell;         // stencil-mesh cell id of the row (graph col 0)
  const int *src;          // [nrows][dim][2H+1] stencil source cell per position
  const uint8_t *flip;     // [nrows][dim][2H+1] ghost recipe: 0 copy, 1 negate the reflect dof,
                           // r >= 2 the mesh args' recipe r - 2
  const double *gsx;       // [nrows][dim][2H+1] ghost position for the moving-shock recipe (or null)
  const double *gsy;
  // Jacobian support (may be null for velocity-only tables)
  const int *jpos;         // [nrows][dim][2H+1] block offset in the CSR row, -1 = absent
  const int *src1;         // [nrows][dim][3] first-order stencil (near-boundary rows)
  const uint8_t *flip1;    // [nrows][dim][3]
  const double *gsx1;      // [nrows][dim][3] (or null)
  const double *gsy1;
  const int *jpos1;        // [nrows][dim][3] block offset for existing neighbours, -1 = none
  const double *jfac;      // [nrows][dim][ndpc] ghost-to-cell derivative factors
};

// Ghost state from the source cell, dof by dof: op 0 copy, 1 negate,
// 2 the constant val; op[0] == 3 marks the moving oblique shock of the double
// Mach reflection (post-shock state behind it, pre-shock ahead).
struct GhostRecipe {
  uint8_t op[5];
  double val[5];
};

struct MeshArgs {
  int dim;
  double hinv[3];
  int reflect[3];  // dof negated in a mirrored ghost for a face normal to each axis (-1: none)
  const GhostRecipe *recipes;  // device table for recipe ids >= 2 (or null)
  double time;                 // evaluation time (moving-shock recipe)
  // moving shock: distance = ((x - shockX0) - shockSpeed t) - shockSlope y
  double shockX0, shockSpeed, shockSlope;
  double pre[5], post[5];
};

// Structured box of a natural-order full mesh: cells [lo, hi) per axis,
// faces normal to an axis at [lo, hi].  mode per axis: 0 = the box stays
// inside the mesh, 1 = periodic, 2 = mirror images outside the mesh (the 2D
// Neumann and slip-wall ghost layers), with dof reflect[axis] negated in
// mirrored cells.
struct Box {
  int n[3];
  int lo[3], hi[3];
  int mode[3];
  int reflect[3];
};

// ---------------------------------------------------------------------------
// Batches of independent problems of one family and scheme on structured
// full meshes (uneven sizes and parameters), evaluated by one launch per
// phase over all instances.
// ---------------------------------------------------------------------------
struct BatchItem {
  Box b;
  MeshArgs m;
  Phys p;
  long uOff;       // first dof of the instance in the packed state / residual
  long fOff[3];    // first double of the instance's faces normal to each axis
  long groups[3];  // tile line groups per axis for the current tile shape
};

// Tile shapes the batch autotuner chooses from: LANES threads along the face
// axis x NR lines per block.  Shape 0 is the single-problem default.
struct TileShape {
  int lanes, nr;
};
constexpr int kNumTileShapes = 4;
constexpr TileShape kTileShapes[kNumTileShapes] = {{64, 2}, {32, 4}, {128, 1}, {64, 1}};
constexpr int kFoFacesPerTile = 128;  // first order: faces per tile (one per thread)

// Per-step Gauss-Newton state of an LSPG object (device).
struct LspgFlags {
  int converged;    // correction below tolerance in this step
  int iters;        // iterations taken in this step
  double lastCorr;  // norm of the last correction
  double lastRes;   // residual norm at the last iterate
  double maxRes;    // max over steps of the residual norm at the step's last iterate
};

// blocks per reduction group of the fused LSPG kernel's partial sums
constexpr int kLspgGroup = 16;
__host__ __device__ constexpr int lspg_groups(int nblocks) { return (nblocks + kLspgGroup - 1) / kLspgGroup; }

// Arguments of the fused LSPG iteration kernel (lspg_fused.cuh).
struct LspgArgs {
  const double *y;   // trial state at the stencil dofs
  const double *D;   // its latent Jacobian, [stencil dofs][K]
  int K;             // latent dimension (<= 32)
  double cf;         // -dt (BDF1)
  double *yn;        // y_n at the sample dofs (stored on the step's first iteration)
  int first;
  double *V;         // sample-mesh velocity (written)
  double *partial;   // [blocks + groups][K(K+1)/2 + K + 1] normal-equation partial sums
  unsigned *ticket;  // [1 + groups] last-block counters (return to 0)
  double *x;         // latent state, updated in place
  double tol;
  LspgFlags *f;
  int jac32;         // 1: reconstruction gradients, flux Jacobians and Jf D in
                     // single precision (an inexact Gauss-Newton step; V, R, the
                     // normal equations and the solve stay double)
  // backward-difference history: R = cf V + (y + cn y_n [+ cnm1 y_n-1]) with
  // BDF1 (cf, cn) = (-dt, -1), BDF2 (cf, cn, cnm1) = (-2/3 dt, -4/3, 1/3); the
  // first iteration of a step moves y_n to y_n-1 (ynm1) and stores y(x_n)
  double cn;
  double cnm1;
  double *ynm1;
  int bdf2;
};

struct BatchArgs {
  const BatchItem *items;     // device array [nItems]
  int nItems;
  const long *tileStart[3];   // device prefix sums [nItems + 1] of tiles per axis
  const long *blockStart;     // device prefix sums [nItems + 1] of balance blocks
  long totalTiles[3];
  long totalBlocks;
};
constexpr int kBalanceBlock = 256;

}  // namespace pda
