// Launchers for one problem family; included by kernels_<family>.cu with
// PDA_FAM defined to the family enum value.
#pragma once

#include "kernels.cuh"
#include "tiles.cuh"
#include "launch.hpp"

namespace pda {
namespace fam_impl {
namespace {

constexpr int FAM = PDA_FAM;
using F = Fam<FAM>;

template <int SCHEME>
void rows_velocity_s(const RowTable &t, const MeshArgs &m, const Phys &p, const double *U, double *V,
                     cudaStream_t s) {
  if (t.nrows <= 0) return;
  k_rows_velocity<FAM, SCHEME><<<div_up(t.nrows, 128), 128, 0, s>>>(t, m, p, U, V);
}

void rows_velocity(int scheme, const RowTable &t, const MeshArgs &m, const Phys &p, const double *U,
                   double *V, cudaStream_t s) {
  switch (scheme) {
    case FirstOrder: rows_velocity_s<FirstOrder>(t, m, p, U, V, s); break;
    case Weno3: rows_velocity_s<Weno3>(t, m, p, U, V, s); break;
    default: rows_velocity_s<Weno5>(t, m, p, U, V, s); break;
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
      constexpr int NR = 2;
      using Cfg = TileCfg<SCHEME>;
      long lines = 1;
      for (int a = 0; a < 3; ++a)
        if (a != AXIS) lines *= (long)(b.hi[a] - b.lo[a]);
      const int nfa = b.hi[AXIS] - b.lo[AXIS] + 1;
      dim3 grid(div_up(lines, NR), div_up(nfa, Cfg::TW));
      dim3 block(Cfg::LANES, NR);
      k_faces_tile<FAM, SCHEME, AXIS, NR><<<grid, block, 0, s>>>(b, p, U, Fo);
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

void rows_vj_inner(int scheme, const RowTable &t, const MeshArgs &m, const Phys &p, const double *U,
                   const int *rowptr, double *V, double *J, cudaStream_t s) {
  if (t.nrows <= 0) return;
  const int g = div_up(t.nrows, 64);
  switch (scheme) {
    case FirstOrder: k_rows_vj_inner<FAM, FirstOrder><<<g, 64, 0, s>>>(t, m, p, U, rowptr, V, J); break;
    case Weno3: k_rows_vj_inner<FAM, Weno3><<<g, 64, 0, s>>>(t, m, p, U, rowptr, V, J); break;
    default: k_rows_vj_inner<FAM, Weno5><<<g, 64, 0, s>>>(t, m, p, U, rowptr, V, J); break;
  }
}

void rows_vj_nearbd(int scheme, const RowTable &t, const MeshArgs &m, const Phys &p, const double *U,
                    const int *rowptr, double *V, double *J, cudaStream_t s) {
  if (t.nrows <= 0) return;
  const int g = div_up(t.nrows, 64);
  switch (scheme) {
    case FirstOrder: k_rows_vj_nearbd<FAM, FirstOrder><<<g, 64, 0, s>>>(t, m, p, U, rowptr, V, J); break;
    case Weno3: k_rows_vj_nearbd<FAM, Weno3><<<g, 64, 0, s>>>(t, m, p, U, rowptr, V, J); break;
    default: k_rows_vj_nearbd<FAM, Weno5><<<g, 64, 0, s>>>(t, m, p, U, rowptr, V, J); break;
  }
}

}  // namespace
}  // namespace fam_impl
}  // namespace pda
