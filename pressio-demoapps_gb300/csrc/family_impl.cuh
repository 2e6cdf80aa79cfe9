// Launchers for one problem family; included by kernels_<family>.cu with
// PDA_FAM defined to the family enum value.
#pragma once

#include <type_traits>

#include "kernels.cuh"
#include "tiles.cuh"
#include "batch.cuh"
#include "jfaces.cuh"
#include "lspg_fused.cuh"
#include "launch.hpp"

namespace pda {
namespace fam_impl {
namespace {

constexpr int FAM = PDA_FAM;
using F = Fam<FAM>;

int device_sms();
// whether this family has the given axis
constexpr bool F_dim_ok(int axis) { return axis < Fam<PDA_FAM>::dim; }

template <int SCHEME>
void rows_velocity_s(const RowTable &ta, const RowTable &tb, const MeshArgs &m, const Phys &p, const double *U,
                     double *V, cudaStream_t s) {
  const int rows = ta.nrows + tb.nrows;
  if (rows <= 0) return;
  // rows per block: the fewest blocks that still cover every SM once
  const int rpb = std::max(1, std::min(VelPar<FAM>::RPB_MAX, div_up(rows, device_sms())));
  const int nbA = div_up(ta.nrows, rpb), nb = nbA + div_up(tb.nrows, rpb);
  k_rows_velocity_par<FAM, SCHEME><<<nb, VelPar<FAM>::THREADS, 0, s>>>(ta, tb, nbA, rpb, m, p, U, V);
}

void rows_velocity(int scheme, const RowTable &ta, const RowTable &tb, const MeshArgs &m, const Phys &p,
                   const double *U, double *V, cudaStream_t s) {
  switch (scheme) {
    case FirstOrder: rows_velocity_s<FirstOrder>(ta, tb, m, p, U, V, s); break;
    case Weno3: rows_velocity_s<Weno3>(ta, tb, m, p, U, V, s); break;
    default: rows_velocity_s<Weno5>(ta, tb, m, p, U, V, s); break;
  }
}

template <int SCHEME, int AXIS>
void faces_s(const Box &b, const Phys &p, const double *U, double *Fo, cudaStream_t s, int *launches,
             cudaEvent_t *ev) {
  long nf = 1;
  for (int a = 0; a < 3; ++a) nf *= (long)(b.hi[a] - b.lo[a] + (a == AXIS ? 1 : 0));
  if (nf > 0) {
    if constexpr (SCHEME == FirstOrder) {
      k_struct_faces<FAM, SCHEME, AXIS><<<div_up(nf, 128), 128, 0, s>>>(b, p, U, Fo);
    } else {
      // tiled kernel: lines of the other two axes in grid x, face chunks in grid y
      // 64 x 2 threads: measured against 128 x 1, 128 x 2 and 32 x 4
      constexpr int NR = 2, LANES = 64;
      using Cfg = TileCfg<SCHEME, LANES>;
      long lines = 1;
      for (int a = 0; a < 3; ++a)
        if (a != AXIS) lines *= (long)(b.hi[a] - b.lo[a]);
      const int nfa = b.hi[AXIS] - b.lo[AXIS] + 1;
      dim3 grid(div_up(lines, NR), div_up(nfa, Cfg::TW));
      dim3 block(Cfg::LANES, NR);
      k_faces_tile<FAM, SCHEME, AXIS, NR, LANES><<<grid, block, 0, s>>>(b, p, U, Fo);
    }
    ++*launches;
  }
  if (ev) cudaEventRecord(ev[AXIS + 1], s);
}

template <int SCHEME>
void struct_velocity_s(const Box &b, const MeshArgs &m, const Phys &p, const double *U,
                       double *const Fb[3], double *V, cudaStream_t s, int *launches, cudaEvent_t *ev) {
  long nc = 1;
  for (int a = 0; a < 3; ++a) nc *= (long)(b.hi[a] - b.lo[a]);
  if (ev) cudaEventRecord(ev[0], s);
  if (nc > 0) {
    faces_s<SCHEME, 0>(b, p, U, Fb[0], s, launches, ev);
    if constexpr (F::dim > 1) faces_s<SCHEME, 1>(b, p, U, Fb[1], s, launches, ev);
    if constexpr (F::dim > 2) faces_s<SCHEME, 2>(b, p, U, Fb[2], s, launches, ev);
    k_struct_balance<FAM><<<div_up(nc, 256), 256, 0, s>>>(b, m, p, U, Fb[0], Fb[1], Fb[2], V);
    ++*launches;
  }
  if (ev) cudaEventRecord(ev[F::dim + 1], s);
}

void struct_velocity(int scheme, const Box &b, const MeshArgs &m, const Phys &p, const double *U,
                     double *const Fb[3], double *V, cudaStream_t s, int *launches, cudaEvent_t *ev) {
  switch (scheme) {
    case FirstOrder: struct_velocity_s<FirstOrder>(b, m, p, U, Fb, V, s, launches, ev); break;
    case Weno3: struct_velocity_s<Weno3>(b, m, p, U, Fb, V, s, launches, ev); break;
    default: struct_velocity_s<Weno5>(b, m, p, U, Fb, V, s, launches, ev); break;
  }
}

void struct_faces(int scheme, int axis, const Box &b, const Phys &p, const double *U, double *F, cudaStream_t s) {
  int nl = 0;
  auto go = [&](auto sch) {
    constexpr int SC = decltype(sch)::value;
    if (axis == 0) faces_s<SC, 0>(b, p, U, F, s, &nl, nullptr);
    if constexpr (F_dim_ok(1)) if (axis == 1) faces_s<SC, 1>(b, p, U, F, s, &nl, nullptr);
    if constexpr (F_dim_ok(2)) if (axis == 2) faces_s<SC, 2>(b, p, U, F, s, &nl, nullptr);
  };
  switch (scheme) {
    case FirstOrder: go(std::integral_constant<int, FirstOrder>{}); break;
    case Weno3: go(std::integral_constant<int, Weno3>{}); break;
    default: go(std::integral_constant<int, Weno5>{}); break;
  }
}

void struct_balance(const Box &b, const MeshArgs &m, const Phys &p, const double *U, const double *const F[3],
                    double *V, cudaStream_t s) {
  long nc = 1;
  for (int a = 0; a < 3; ++a) nc *= (long)(b.hi[a] - b.lo[a]);
  if (nc > 0) k_struct_balance<FAM><<<div_up(nc, 256), 256, 0, s>>>(b, m, p, U, F[0], F[1], F[2], V);
}

void rows_vj_inner(int scheme, const RowTable &t, const MeshArgs &m, const Phys &p, const double *U,
                   const int *rowptr, double *V, double *J, cudaStream_t s) {
  if (t.nrows <= 0) return;
  const int g = div_up(t.nrows, 64);
  switch (scheme) {
    case FirstOrder: k_rows_vj_inner<FAM, FirstOrder><<<g, 64, 0, s>>>(t, m, p, U, rowptr, V, J); break;
    case Weno3: {
      using RP = RowPar<FAM, Weno3>;
      k_rows_vj_inner_par<FAM, Weno3><<<div_up(t.nrows, RP::RPB), RP::THREADS, 0, s>>>(t, m, p, U, rowptr, V, J);
      break;
    }
    default: {
      using RP = RowPar<FAM, Weno5>;
      k_rows_vj_inner_par<FAM, Weno5><<<div_up(t.nrows, RP::RPB), RP::THREADS, 0, s>>>(t, m, p, U, rowptr, V, J);
      break;
    }
  }
}

int device_sms() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

// rows per block: the fewest blocks that still cover every SM once, within
// the shared-memory budget
int lspg_fused_rpb(int scheme, int innerRows, int nearRows, int K) {
  const int rows = innerRows + nearRows;
  const int S = 2 * (scheme + 1) + 1;
  const int bySmem = (int)(FusedPar<FAM>::kSmemLimit / FusedPar<FAM>::smem_row(S, K));
  return std::max(1, std::min(std::min(FusedPar<FAM>::RPB_MAX, bySmem), div_up(rows, device_sms())));
}

int lspg_fused_blocks(int scheme, int innerRows, int nearRows, int K) {
  const int rpb = lspg_fused_rpb(scheme, innerRows, nearRows, K);
  return div_up(innerRows, rpb) + div_up(nearRows, rpb);
}

template <typename JT>
void lspg_fused_prepare_t() {
  const int bytes = (int)FusedPar<FAM>::kSmemLimit;
  cudaFuncSetAttribute(k_lspg_fused<FAM, FirstOrder, JT>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_lspg_fused<FAM, Weno3, JT>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_lspg_fused<FAM, Weno5, JT>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

void lspg_fused_prepare() {
  lspg_fused_prepare_t<double>();
  lspg_fused_prepare_t<float>();
}

void lspg_fused(int scheme, const RowTable &ti, const RowTable &tn, const MeshArgs &m, const Phys &p,
                const LspgArgs &a, cudaStream_t s) {
  const int rpb = lspg_fused_rpb(scheme, ti.nrows, tn.nrows, a.K);
  const int nbI = div_up(ti.nrows, rpb);
  const int nb = lspg_fused_blocks(scheme, ti.nrows, tn.nrows, a.K);
  if (nb <= 0) return;
  constexpr int T = FusedPar<FAM>::THREADS;
  const size_t sm = (size_t)rpb * FusedPar<FAM>::smem_row(2 * (scheme + 1) + 1, a.K);
  if (a.jac32) {
    switch (scheme) {
      case FirstOrder: k_lspg_fused<FAM, FirstOrder, float><<<nb, T, sm, s>>>(ti, tn, rpb, nbI, m, p, a); break;
      case Weno3: k_lspg_fused<FAM, Weno3, float><<<nb, T, sm, s>>>(ti, tn, rpb, nbI, m, p, a); break;
      default: k_lspg_fused<FAM, Weno5, float><<<nb, T, sm, s>>>(ti, tn, rpb, nbI, m, p, a); break;
    }
    return;
  }
  switch (scheme) {
    case FirstOrder: k_lspg_fused<FAM, FirstOrder, double><<<nb, T, sm, s>>>(ti, tn, rpb, nbI, m, p, a); break;
    case Weno3: k_lspg_fused<FAM, Weno3, double><<<nb, T, sm, s>>>(ti, tn, rpb, nbI, m, p, a); break;
    default: k_lspg_fused<FAM, Weno5, double><<<nb, T, sm, s>>>(ti, tn, rpb, nbI, m, p, a); break;
  }
}

void rows_vj_nearbd(int scheme, const RowTable &t, const MeshArgs &m, const Phys &p, const double *U,
                    const int *rowptr, double *V, double *J, cudaStream_t s) {
  if (t.nrows <= 0) return;
  const int g = div_up(t.nrows, 64);
  (void)g;
  const int gp = div_up(t.nrows, NearPar<FAM>::RPB);
  constexpr int tp = NearPar<FAM>::THREADS;
  switch (scheme) {
    case FirstOrder: k_rows_vj_nearbd_par<FAM, FirstOrder><<<gp, tp, 0, s>>>(t, m, p, U, rowptr, V, J); break;
    case Weno3: k_rows_vj_nearbd_par<FAM, Weno3><<<gp, tp, 0, s>>>(t, m, p, U, rowptr, V, J); break;
    default: k_rows_vj_nearbd_par<FAM, Weno5><<<gp, tp, 0, s>>>(t, m, p, U, rowptr, V, J); break;
  }
}


// ------------------------------------------------------------------ batches
// persistent grid: resident blocks per SM x SMs (cached per kernel; one GPU
// model per process), never more blocks than tiles
template <class K>
long persistent_grid(K kernel, int threads, long work) {
  static long grid = 0;
  if (grid == 0) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, 0);
    grid = (long)(occ > 0 ? occ : 1) * (sms > 0 ? sms : 1);
  }
  return work < grid ? work : grid;
}

template <int SCHEME, int AXIS, int NR, int LANES>
void batch_tile_launch(const BatchArgs &a, const double *U, double *Fo, cudaStream_t s) {
  auto k = k_batch_faces_tile<FAM, SCHEME, AXIS, NR, LANES>;
  const long g = a.totalTiles[AXIS];  // one block per tile
  if (g > 0) k<<<(unsigned)g, dim3(LANES, NR), 0, s>>>(a, U, Fo);
}

template <int SCHEME, int AXIS>
void batch_faces_axis(int shape, const BatchArgs &a, const double *U, double *Fo, cudaStream_t s) {
  if constexpr (SCHEME == FirstOrder) {
    auto k = k_batch_faces_fo<FAM, AXIS>;
    const long g = persistent_grid(k, kFoFacesPerTile, a.totalTiles[AXIS]);
    if (g > 0) k<<<(unsigned)g, kFoFacesPerTile, 0, s>>>(a, U, Fo);
  } else {
    static_assert(kTileShapes[0].lanes == 64 && kTileShapes[0].nr == 2, "shape table");
    if (shape == 0 || F::dim != 2) {
      batch_tile_launch<SCHEME, AXIS, 2, 64>(a, U, Fo, s);
    } else {
      if constexpr (F::dim == 2) {
        static_assert(kTileShapes[1].lanes == 32 && kTileShapes[1].nr == 4, "shape table");
        static_assert(kTileShapes[2].lanes == 128 && kTileShapes[2].nr == 1, "shape table");
        static_assert(kTileShapes[3].lanes == 64 && kTileShapes[3].nr == 1, "shape table");
        if (shape == 1) batch_tile_launch<SCHEME, AXIS, 4, 32>(a, U, Fo, s);
        else if (shape == 2) batch_tile_launch<SCHEME, AXIS, 1, 128>(a, U, Fo, s);
        else batch_tile_launch<SCHEME, AXIS, 1, 64>(a, U, Fo, s);
      }
    }
  }
}

template <int SCHEME>
void batch_faces_s(int axis, int shape, const BatchArgs &a, const double *U, double *Fo, cudaStream_t s) {
  if (axis == 0) batch_faces_axis<SCHEME, 0>(shape, a, U, Fo, s);
  if constexpr (F::dim > 1)
    if (axis == 1) batch_faces_axis<SCHEME, 1>(shape, a, U, Fo, s);
  if constexpr (F::dim > 2)
    if (axis == 2) batch_faces_axis<SCHEME, 2>(shape, a, U, Fo, s);
}

void batch_faces(int scheme, int axis, int shape, const BatchArgs &a, const double *U, double *Fo,
                 cudaStream_t s) {
  switch (scheme) {
    case FirstOrder: batch_faces_s<FirstOrder>(axis, shape, a, U, Fo, s); break;
    case Weno3: batch_faces_s<Weno3>(axis, shape, a, U, Fo, s); break;
    default: batch_faces_s<Weno5>(axis, shape, a, U, Fo, s); break;
  }
}

void batch_balance(const BatchArgs &a, const double *U, const double *Fo, double *V, cudaStream_t s) {
  auto k = k_batch_balance<FAM>;
  const long g = persistent_grid(k, kBalanceBlock, a.totalBlocks);
  if (g > 0) k<<<(unsigned)g, kBalanceBlock, 0, s>>>(a, U, Fo, V);
}

void batch_balance_stage(const BatchArgs &a, const double *Us, const double *Fo, double *out, const double *x,
                         int kind, double ca, double cb, double cc, cudaStream_t s) {
  auto k = k_batch_balance_stage<FAM>;
  const long g = persistent_grid(k, kBalanceBlock, a.totalBlocks);
  if (g > 0) k<<<(unsigned)g, kBalanceBlock, 0, s>>>(a, Us, Fo, out, x, kind, ca, cb, cc);
}

int batch_num_shapes() { return F::dim == 2 ? kNumTileShapes : 1; }


// ----------------------------------------------------- Jacobian, faces once
template <int SCHEME, int AXIS>
void struct_vj_axis(const Box &b, const MeshArgs &m, const Phys &p, const double *U, const int *rowptr,
                    double *V, double *J, cudaStream_t s) {
  constexpr int LANES = 64;
  using Cfg = JTileCfg<FAM, SCHEME, LANES>;
  constexpr int A1 = AXIS == 0 ? 1 : 0, A2 = AXIS == 2 ? 1 : 2;
  const long lines = (long)(b.hi[A1] - b.lo[A1]) * (b.hi[A2] - b.lo[A2]);
  const int nfa = b.hi[AXIS] - b.lo[AXIS] + 1;
  dim3 grid((unsigned)lines, (unsigned)div_up(nfa, Cfg::TW));
  k_jtile<FAM, SCHEME, AXIS, LANES><<<grid, LANES, 0, s>>>(b, m, p, U, rowptr, V, J);
}

template <int SCHEME>
void struct_vj_s(const Box &b, const MeshArgs &m, const Phys &p, const double *U, const int *rowptr, double *V,
                 double *J, cudaStream_t s, int *launches) {
  long nc = 1;
  for (int a = 0; a < 3; ++a) nc *= (long)(b.hi[a] - b.lo[a]);
  if (nc <= 0) return;
  struct_vj_axis<SCHEME, 0>(b, m, p, U, rowptr, V, J, s);
  if constexpr (F::dim > 1) struct_vj_axis<SCHEME, 1>(b, m, p, U, rowptr, V, J, s);
  if constexpr (F::dim > 2) struct_vj_axis<SCHEME, 2>(b, m, p, U, rowptr, V, J, s);
  *launches += F::dim;
}

void struct_vj(int scheme, const Box &b, const MeshArgs &m, const Phys &p, const double *U, const int *rowptr,
               double *V, double *J, cudaStream_t s, int *launches) {
  if (scheme == Weno3) struct_vj_s<Weno3>(b, m, p, U, rowptr, V, J, s, launches);
  else if (scheme == Weno5) struct_vj_s<Weno5>(b, m, p, U, rowptr, V, J, s, launches);
}

}  // namespace
}  // namespace fam_impl
}  // namespace pda
