// Batched structured velocity: many independent problem instances (uneven
// mesh sizes, own parameters) in one launch per phase.
//
// Work is cut into tiles (the single-problem tile of tiles.cuh: NR lines x
// TW faces of one instance), numbered instance by instance; per-instance
// prefix sums of tile counts let each block find its instance by binary
// search.  One launch per phase covers all instances: the face kernels run
// one block per tile of every instance, the first-order faces and the
// balance passes are persistent (a grid of resident blocks per SM x SMs loops
// over the work), so small instances no longer leave most of the GPU idle
// and one launch replaces one per instance.  Each tile runs exactly the
// single-problem code, so every instance's residual is bit-identical to
// evaluating that problem alone.
#pragma once

#include "kernels.cuh"
#include "tiles.cuh"

namespace pda {

// Largest i in [0, n) with start[i] <= t (start[0] = 0 <= t < start[n]);
// skips instances that own no tiles.
__device__ __forceinline__ int batch_find(const long *__restrict__ start, int n, long t) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(start + mid) <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// One block per tile of any instance (grid = all tiles of the axis), with
// registers capped for 32 resident warps per SM (fewer where the tile's
// shared memory admits fewer blocks, FaceTileMinBlocks).  Measured on 512
// shallow-water instances: 169 ms per SSP-RK3 step, against 193 ms for a
// persistent loop over the tiles (its loop state raised the registers from
// 74 to 80: 6 blocks per SM) and 178 ms for one block per tile without the cap.
template <int FAM, int SCHEME, int AXIS, int NR, int LANES>
__global__ void __launch_bounds__(LANES *NR, (FaceTileMinBlocks<FAM, SCHEME, NR, LANES>::value))
k_batch_faces_tile(BatchArgs a, const double *__restrict__ U, double *__restrict__ F) {
  __shared__ FaceTileSmem<FAM, SCHEME, NR, LANES> sm;
  const long t = blockIdx.x;
  const int it = batch_find(a.tileStart[AXIS], a.nItems, t);
  const BatchItem &bi = a.items[it];
  const Box b = bi.b;
  const Phys p = bi.p;
  const long local = t - a.tileStart[AXIS][it];
  const long g = bi.groups[AXIS];
  face_tile<FAM, SCHEME, AXIS, NR, LANES>(sm, b, p, U + bi.uOff, F + bi.fOff[AXIS], local % g,
                                          (int)(local / g));
}

// first order: one face per thread, kFoFacesPerTile faces per tile
template <int FAM, int AXIS>
__global__ void __launch_bounds__(kFoFacesPerTile)
k_batch_faces_fo(BatchArgs a, const double *__restrict__ U, double *__restrict__ F) {
  const long total = a.totalTiles[AXIS];
  for (long t = blockIdx.x; t < total; t += gridDim.x) {
    const int it = batch_find(a.tileStart[AXIS], a.nItems, t);
    const BatchItem &bi = a.items[it];
    const Box b = bi.b;
    const Phys p = bi.p;
    const long face = (t - a.tileStart[AXIS][it]) * kFoFacesPerTile + threadIdx.x;
    struct_face<FAM, FirstOrder, AXIS>(b, p, U + bi.uOff, F + bi.fOff[AXIS], face);
  }
}

template <int FAM>
__global__ void __launch_bounds__(kBalanceBlock)
k_batch_balance(BatchArgs a, const double *__restrict__ U, const double *__restrict__ F,
                double *__restrict__ V) {
  for (long blk = blockIdx.x; blk < a.totalBlocks; blk += gridDim.x) {
    const int it = batch_find(a.blockStart, a.nItems, blk);
    const BatchItem &bi = a.items[it];
    const Box b = bi.b;
    const MeshArgs m = bi.m;
    const Phys p = bi.p;
    const long cell = (blk - a.blockStart[it]) * kBalanceBlock + threadIdx.x;
    balance_cell<FAM>(b, m, p, U + bi.uOff, F + bi.fOff[0], F + bi.fOff[1], F + bi.fOff[2], V + bi.uOff,
                      cell);
  }
}

// The balance of every instance fused with an SSP-RK3 stage update: the
// velocity r of the cell (state Us) goes straight into
//   kind 0: out = x + cb r
//   kind 1: out = ca out + cb x + cc r
// (the stage formulas of the unfused update kernels, same association), so
// the stage needs no velocity buffer and no separate update pass.  Each
// thread reads its own cell's state before writing, so out may be Us.
template <int FAM>
__global__ void __launch_bounds__(kBalanceBlock)
k_batch_balance_stage(BatchArgs a, const double *Us, const double *__restrict__ F, double *out,
                      const double *x, int kind, double ca, double cb, double cc) {
  constexpr int NDPC = Fam<FAM>::ndpc;
  for (long blk = blockIdx.x; blk < a.totalBlocks; blk += gridDim.x) {
    const int it = batch_find(a.blockStart, a.nItems, blk);
    const BatchItem &bi = a.items[it];
    const Box b = bi.b;
    const MeshArgs m = bi.m;
    const Phys p = bi.p;
    const long t = (blk - a.blockStart[it]) * kBalanceBlock + threadIdx.x;
    double v[NDPC];
    long cell;
    if (!balance_values<FAM>(b, m, p, Us + bi.uOff, F + bi.fOff[0], F + bi.fOff[1], F + bi.fOff[2], t, v, cell))
      continue;
    const long q0 = bi.uOff + cell * NDPC;
#pragma unroll
    for (int d = 0; d < NDPC; ++d) {
      const long q = q0 + d;
      out[q] = kind == 0 ? x[q] + cb * v[d] : ca * out[q] + cb * x[q] + cc * v[d];
    }
  }
}

}  // namespace pda
