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
  const uint8_t *flip;     // [nrows][dim][2H+1] 1 = mirrored ghost: negate reflect dof
  // Jacobian support (may be null for velocity-only tables)
  const int *jpos;         // [nrows][dim][2H+1] block offset in the CSR row, -1 = absent
  const int *src1;         // [nrows][dim][3] first-order stencil (near-boundary rows)
  const uint8_t *flip1;    // [nrows][dim][3]
  const int *jpos1;        // [nrows][dim][3] block offset for existing neighbours, -1 = none
  const double *jfac;      // [nrows][dim][ndpc] ghost-to-cell derivative factors
};

struct MeshArgs {
  int dim;
  double hinv[3];
  int reflect[3];  // dof negated in a mirrored ghost for a face normal to each axis (-1: none)
};

struct Box {
  int n[3];       // cells per axis (1 for absent axes)
  int lo[3];      // first box cell per axis
  int hi[3];      // one past the last box cell per axis
  int periodic[3];
};

}  // namespace pda
