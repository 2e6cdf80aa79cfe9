// Kernel templates for the residual ("velocity") and the CSR Jacobian of the
// cell-centered finite-volume problems.
//
// Two formulations are used:
//  * "rows" kernels evaluate one graph row per thread exactly like the
//    reference's per-cell loops (both faces of a cell computed from the
//    cell's own stencil).  They serve the cells within the stencil half-width
//    of a non-periodic boundary, whose ghost values depend on the row
//    (impl/euler_2d_prob_class.hpp:1045-1113, :833-988), and every row of a
//    sample mesh.  Each row's stencil is pre-resolved on the host into a
//    table of source cells (the ghost-fill rule folded in), so a single
//    kernel serves every boundary condition that mirrors cells.
//  * "structured" kernels evaluate each face of a natural-order full mesh
//    exactly once (the reference computes every interior face twice, once
//    from each side, with identical arguments) and then balance the face
//    fluxes per cell in the reference's axis order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "numerics.cuh"
#include "types.hpp"

namespace pda {

template <int FAM> struct Fam;
template <> struct Fam<Euler1d> {
  static constexpr int dim = 1, ndpc = 3;
  template <int AXIS, bool INL = false, bool IP = false>
  static PDA_HD void flux(double F[3], const double qL[3], const double qR[3], const Phys &p) {
    euler3_flux<INL, IP>(F, qL, qR, p.gamma);
  }
  template <int AXIS, typename T>
  static PDA_HD void flux_jac(T JL[9], T JR[9], const T qL[3], const T qR[3], const Phys &p) {
    euler3_flux_jac(JL, JR, qL, qR, (T)p.gamma);
  }
  template <typename T>
  static PDA_HD void flux_jac_ax(T JL[9], T JR[9], const T qL[3], const T qR[3], const Phys &p, int) {
    euler3_flux_jac(JL, JR, qL, qR, (T)p.gamma);
  }
  // the flux in two halves (one face state, then the combination); bit-identical to flux
  using Side = FluxSide<3>;
  template <int AXIS>
  static PDA_HD void flux_side(Side &o, const double q[3], const Phys &p) {
    euler3_side(o, q, p.gamma);
  }
  static PDA_HD void flux_side_ax(Side &o, const double q[3], const Phys &p, int) { euler3_side(o, q, p.gamma); }
  template <int AXIS>
  static PDA_HD void flux_combine(double F[3], const double qL[3], const double qR[3], const Side &L,
                                  const Side &R, const Phys &p) {
    euler3_combine(F, qL, qR, L, R, p.gamma);
  }
};
template <> struct Fam<Euler2d> {
  static constexpr int dim = 2, ndpc = 4;
  template <int AXIS, bool INL = false, bool IP = false>
  static PDA_HD void flux(double F[4], const double qL[4], const double qR[4], const Phys &p) {
    euler4_flux<AXIS, INL, IP>(F, qL, qR, p.gamma);
  }
  template <int AXIS, typename T>
  static PDA_HD void flux_jac(T JL[16], T JR[16], const T qL[4], const T qR[4], const Phys &p) {
    euler4_flux_jac<AXIS>(JL, JR, qL, qR, (T)p.gamma);
  }
  template <typename T>
  static PDA_HD void flux_jac_ax(T JL[16], T JR[16], const T qL[4], const T qR[4], const Phys &p, int ax) {
    euler4_flux_jac_ax(JL, JR, qL, qR, (T)p.gamma, ax);
  }
  // the flux in two halves (one face state, then the combination); bit-identical to flux
  using Side = FluxSide<4>;
  template <int AXIS>
  static PDA_HD void flux_side(Side &o, const double q[4], const Phys &p) {
    euler4_side<AXIS>(o, q, p.gamma);
  }
  static PDA_HD void flux_side_ax(Side &o, const double q[4], const Phys &p, int ax) {
    euler4_side_ax(o, q, p.gamma, ax);
  }
  template <int AXIS>
  static PDA_HD void flux_combine(double F[4], const double qL[4], const double qR[4], const Side &L,
                                  const Side &R, const Phys &p) {
    euler4_combine<AXIS>(F, qL, qR, L, R, p.gamma);
  }
};
template <> struct Fam<Euler3d> {
  static constexpr int dim = 3, ndpc = 5;
  template <int AXIS, bool INL = false, bool IP = false>
  static PDA_HD void flux(double F[5], const double qL[5], const double qR[5], const Phys &p) {
    euler5_flux<AXIS, INL, IP>(F, qL, qR, p.gamma);
  }
  template <int AXIS, typename T>
  static PDA_HD void flux_jac(T JL[25], T JR[25], const T qL[5], const T qR[5], const Phys &p) {
    euler5_flux_jac<AXIS>(JL, JR, qL, qR, (T)p.gamma);
  }
  template <typename T>
  static PDA_HD void flux_jac_ax(T JL[25], T JR[25], const T qL[5], const T qR[5], const Phys &p, int ax) {
    euler5_flux_jac_ax(JL, JR, qL, qR, (T)p.gamma, ax);
  }
  // the flux in two halves (one face state, then the combination); bit-identical to flux
  using Side = FluxSide<5>;
  template <int AXIS>
  static PDA_HD void flux_side(Side &o, const double q[5], const Phys &p) {
    euler5_side<AXIS>(o, q, p.gamma);
  }
  static PDA_HD void flux_side_ax(Side &o, const double q[5], const Phys &p, int ax) {
    euler5_side_ax(o, q, p.gamma, ax);
  }
  template <int AXIS>
  static PDA_HD void flux_combine(double F[5], const double qL[5], const double qR[5], const Side &L,
                                  const Side &R, const Phys &p) {
    euler5_combine<AXIS>(F, qL, qR, L, R, p.gamma);
  }
};
template <> struct Fam<Swe2d> {
  static constexpr int dim = 2, ndpc = 3;
  template <int AXIS, bool INL = false, bool IP = false>
  static PDA_HD void flux(double F[3], const double qL[3], const double qR[3], const Phys &p) {
    swe_flux<AXIS, INL, IP>(F, qL, qR, p.gravity);
  }
  template <int AXIS, typename T>
  static PDA_HD void flux_jac(T JL[9], T JR[9], const T qL[3], const T qR[3], const Phys &p) {
    swe_flux_jac<AXIS>(JL, JR, qL, qR, (T)p.gravity);
  }
  template <typename T>
  static PDA_HD void flux_jac_ax(T JL[9], T JR[9], const T qL[3], const T qR[3], const Phys &p, int ax) {
    swe_flux_jac_ax(JL, JR, qL, qR, (T)p.gravity, ax);
  }
  // the flux in two halves (one face state, then the combination); bit-identical to flux
  using Side = FluxSide<3>;
  template <int AXIS>
  static PDA_HD void flux_side(Side &o, const double q[3], const Phys &p) {
    swe_side<AXIS>(o, q, p.gravity);
  }
  static PDA_HD void flux_side_ax(Side &o, const double q[3], const Phys &p, int ax) {
    swe_side_ax(o, q, p.gravity, ax);
  }
  template <int AXIS>
  static PDA_HD void flux_combine(double F[3], const double qL[3], const double qR[3], const Side &L,
                                  const Side &R, const Phys &p) {
    swe_combine<AXIS>(F, qL, qR, L, R, p.gravity);
  }
};

// Reconstruct the two states of the face between q[H-1] and q[H] from 2H
// consecutive cell states (H = scheme half-width).  Mirrors
// impl/functor_reconstruct_from_state.hpp:419-499 and weno.hpp:300-328.
template <int NDPC, int SCHEME>
PDA_HD void reconstruct_face(double uNeg[NDPC], double uPos[NDPC], const double (*q)[NDPC]) {
#pragma unroll
  for (int d = 0; d < NDPC; ++d) {
    if constexpr (SCHEME == FirstOrder) {
      uNeg[d] = q[0][d];
      uPos[d] = q[1][d];
    } else if constexpr (SCHEME == Weno3) {
      weno3_face(uNeg[d], uPos[d], q[0][d], q[1][d], q[2][d], q[3][d]);
    } else {
      weno5_face(uNeg[d], uPos[d], q[0][d], q[1][d], q[2][d], q[3][d], q[4][d], q[5][d]);
    }
  }
}

// The Rusanov flux of a face whose axis is a runtime value, as its two sides
// and their combination (bit-identical to flux<AXIS>): threads of one warp
// that hold faces of different axes then run one instruction stream instead
// of each axis's specialised flux in turn.
template <int FAM>
__device__ __forceinline__ void flux_ax(double fl[], const double uN[], const double uP[], const Phys &p, int ax) {
  using F = Fam<FAM>;
  typename F::Side L, R;
  F::flux_side_ax(L, uN, p, ax);
  F::flux_side_ax(R, uP, p, ax);
  F::template flux_combine<0>(fl, uN, uP, L, R, p);
}

// Same with the gradient of each reconstructed value with respect to the 2H
// cell values (per dof): g[d][s].  FirstOrder gradients are {1,0} / {0,1}
// (functor_reconstruct_from_state.hpp:523-536).
template <int NDPC, int SCHEME>
PDA_HD void reconstruct_face_grad(double uNeg[NDPC], double uPos[NDPC],
                                  double gNeg[NDPC][2 * SchemeTraits<SCHEME>::h],
                                  double gPos[NDPC][2 * SchemeTraits<SCHEME>::h],
                                  const double (*q)[NDPC]) {
#pragma unroll
  for (int d = 0; d < NDPC; ++d) {
    if constexpr (SCHEME == FirstOrder) {
      uNeg[d] = q[0][d];
      uPos[d] = q[1][d];
      gNeg[d][0] = 1.;
      gNeg[d][1] = 0.;
      gPos[d][0] = 0.;
      gPos[d][1] = 1.;
    } else if constexpr (SCHEME == Weno3) {
      weno3_face_grad(uNeg[d], uPos[d], gNeg[d], gPos[d], q[0][d], q[1][d], q[2][d], q[3][d]);
    } else {
      weno5_face_grad(uNeg[d], uPos[d], gNeg[d], gPos[d], q[0][d], q[1][d], q[2][d], q[3][d],
                      q[4][d], q[5][d]);
    }
  }
}

// One side of one dof's face reconstruction from its 2H cell values:
// side 0 the left-biased value uNeg, side 1 the right-biased uPos (the
// one-sided halves of reconstruct_face / reconstruct_face_grad, same
// expressions).
template <int SCHEME>
PDA_HD double face_value_side(int side, const double *q) {
  if constexpr (SCHEME == FirstOrder) {
    return q[side];
  } else if constexpr (SCHEME == Weno3) {
    return side == 0 ? weno3_neg(q[0], q[1], q[2]) : weno3_pos(q[1], q[2], q[3]);
  } else {
    return side == 0 ? weno5_neg(q[0], q[1], q[2], q[3], q[4]) : weno5_pos(q[1], q[2], q[3], q[4], q[5]);
  }
}

template <int SCHEME, typename T>
PDA_HD void face_grad_side(int side, T &u, T g[2 * SchemeTraits<SCHEME>::h], const T *q) {
  if constexpr (SCHEME == FirstOrder) {
    u = q[side];
    g[0] = side == 0 ? T(1) : T(0);
    g[1] = side == 0 ? T(0) : T(1);
  } else if constexpr (SCHEME == Weno3) {
    if (side == 0) weno3_neg_grad(u, g, q[0], q[1], q[2], q[3]);
    else weno3_pos_grad(u, g, q[0], q[1], q[2], q[3]);
  } else {
    if (side == 0) weno5_neg_grad(u, g, q[0], q[1], q[2], q[3], q[4], q[5]);
    else weno5_pos_grad(u, g, q[0], q[1], q[2], q[3], q[4], q[5]);
  }
}

template <int NDPC>
__device__ __forceinline__ void load_cell(double q[NDPC], const double *__restrict__ U, int c,
                                          bool flip, int reflectDof) {
#pragma unroll
  for (int d = 0; d < NDPC; ++d) q[d] = __ldg(U + (size_t)c * NDPC + d);
  if (flip && reflectDof >= 0) {
#pragma unroll
    for (int d = 0; d < NDPC; ++d)
      if (d == reflectDof) q[d] = -q[d];
  }
}

// Stencil entry i of a row table: a mesh cell, or a ghost built from a cell
// by the entry's recipe (time enters through the moving-shock recipe).
template <int NDPC>
__device__ __forceinline__ void load_entry(double q[NDPC], const double *__restrict__ U, int c, uint8_t rid,
                                           int reflectDof, const MeshArgs &m, const double *gsx,
                                           const double *gsy, size_t i) {
  if (rid < 2) {
    load_cell<NDPC>(q, U, c, rid == 1, reflectDof);
    return;
  }
  const GhostRecipe &g = m.recipes[rid - 2];
  if (g.op[0] == 3) {
    const double dist = ((gsx[i] - m.shockX0) - m.shockSpeed * m.time) - m.shockSlope * gsy[i];
#pragma unroll
    for (int d = 0; d < NDPC; ++d) q[d] = dist < 0. ? m.post[d] : m.pre[d];
    return;
  }
#pragma unroll
  for (int d = 0; d < NDPC; ++d) {
    const uint8_t op = g.op[d];
    q[d] = op == 2 ? g.val[d] : (op == 1 ? -__ldg(U + (size_t)c * NDPC + d) : __ldg(U + (size_t)c * NDPC + d));
  }
}

// Reference per-cell V (velocityOnlyNearBdCellsImpl / velocityOnlyInnerCellsImpl)
template <int FAM, int SCHEME>
__global__ void __launch_bounds__(128)
k_rows_velocity(RowTable t, MeshArgs m, Phys p, const double *__restrict__ U, double *__restrict__ V) {
  using F = Fam<FAM>;
  constexpr int NDPC = F::ndpc, DIM = F::dim, H = SchemeTraits<SCHEME>::h, S = 2 * H + 1;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= t.nrows) return;
  double v[NDPC];
#pragma unroll
  for (int d = 0; d < NDPC; ++d) v[d] = 0.;
#pragma unroll
  for (int ax = 0; ax < DIM; ++ax) {
    double q[S][NDPC];
    const size_t base = ((size_t)e * DIM + ax) * S;
#pragma unroll
    for (int s = 0; s < S; ++s)
      load_entry<NDPC>(q[s], U, t.src[base + s], t.flip[base + s], m.reflect[ax], m, t.gsx, t.gsy, base + s);
    double uN[NDPC], uP[NDPC], fL[NDPC], fR[NDPC];
    reconstruct_face<NDPC, SCHEME>(uN, uP, q);
    if (ax == 0) F::template flux<0>(fL, uN, uP, p);
    if constexpr (DIM > 1) if (ax == 1) F::template flux<1>(fL, uN, uP, p);
    if constexpr (DIM > 2) if (ax == 2) F::template flux<2>(fL, uN, uP, p);
    reconstruct_face<NDPC, SCHEME>(uN, uP, q + 1);
    if (ax == 0) F::template flux<0>(fR, uN, uP, p);
    if constexpr (DIM > 1) if (ax == 1) F::template flux<1>(fR, uN, uP, p);
    if constexpr (DIM > 2) if (ax == 2) F::template flux<2>(fR, uN, uP, p);
    const double hinv = m.hinv[ax];
#pragma unroll
    for (int d = 0; d < NDPC; ++d) v[d] += hinv * (fL[d] - fR[d]);
  }
  const int r = t.rows[e];
  if constexpr (FAM == Swe2d) {
    // swe_2d_prob_class.hpp:983-994
    const int c = t.cell[e];
    const double u0 = __ldg(U + (size_t)c * 3), u1 = __ldg(U + (size_t)c * 3 + 1),
                 u2 = __ldg(U + (size_t)c * 3 + 2);
    v[1] -= div_rn(p.coriolis * u2, u0);
    v[2] += div_rn(p.coriolis * u1, u0);
  }
#pragma unroll
  for (int d = 0; d < NDPC; ++d) V[(size_t)r * NDPC + d] = v[d];
}

// ---------------------------------------------------------------------------
// Structured full mesh: faces once, then per-cell balance.
// ---------------------------------------------------------------------------
// cell index along an axis for a position that may lie outside [0, n)
__device__ __forceinline__ int map_cell(int c, int n, int mode, bool &mirrored) {
  mirrored = false;
  if (mode == 1) {
    c %= n;
    if (c < 0) c += n;
  } else if (mode == 2) {
    if (c < 0) {
      c = -c - 1;
      mirrored = true;
    } else if (c >= n) {
      c = 2 * n - 1 - c;
      mirrored = true;
    }
  }
  // interior boxes never leave the mesh for faces that are written; clamp
  // the loads of unused tile tails
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

// One thread per face normal to AXIS inside the box; face f lies between
// cells f-1 and f.  Output Fx laid out [outer][mid][f - lo] with the face
// axis fastest.
template <int FAM, int SCHEME, int AXIS>
__device__ __forceinline__ void struct_face(const Box &b, const Phys &p, const double *__restrict__ U,
                                            double *__restrict__ Fout, long t) {
  using F = Fam<FAM>;
  constexpr int NDPC = F::ndpc, H = SchemeTraits<SCHEME>::h;
  const int nf[3] = {b.hi[0] - b.lo[0] + (AXIS == 0), b.hi[1] - b.lo[1] + (AXIS == 1),
                     b.hi[2] - b.lo[2] + (AXIS == 2)};
  const long total = (long)nf[0] * nf[1] * nf[2];
  if (t >= total) return;
  int id[3];
  id[0] = (int)(t % nf[0]);
  id[1] = (int)((t / nf[0]) % nf[1]);
  id[2] = (int)(t / ((long)nf[0] * nf[1]));
  int c[3] = {id[0] + b.lo[0], id[1] + b.lo[1], id[2] + b.lo[2]};
  double q[2 * H][NDPC];
#pragma unroll
  for (int s = 0; s < 2 * H; ++s) {
    int cc[3] = {c[0], c[1], c[2]};
    bool mir;
    cc[AXIS] = map_cell(c[AXIS] - H + s, b.n[AXIS], b.mode[AXIS], mir);
    const long cell = cc[0] + (long)b.n[0] * (cc[1] + (long)b.n[1] * cc[2]);
#pragma unroll
    for (int d = 0; d < NDPC; ++d) {
      q[s][d] = __ldg(U + cell * NDPC + d);
      if (mir && d == b.reflect[AXIS]) q[s][d] = -q[s][d];
    }
  }
  double uN[NDPC], uP[NDPC], f[NDPC];
  reconstruct_face<NDPC, SCHEME>(uN, uP, q);
  F::template flux<AXIS>(f, uN, uP, p);
#pragma unroll
  for (int d = 0; d < NDPC; ++d) Fout[t * NDPC + d] = f[d];
}

template <int FAM, int SCHEME, int AXIS>
__global__ void __launch_bounds__(128)
k_struct_faces(Box b, Phys p, const double *__restrict__ U, double *__restrict__ Fout) {
  struct_face<FAM, SCHEME, AXIS>(b, p, U, Fout, (long)blockIdx.x * blockDim.x + threadIdx.x);
}

// V for every box cell from the face fluxes, in the reference's axis order
// (x, then y, then z, then the shallow-water Coriolis source).
template <int FAM>
__device__ __forceinline__ bool balance_values(const Box &b, const MeshArgs &m, const Phys &p,
                                               const double *__restrict__ U, const double *__restrict__ Fx,
                                               const double *__restrict__ Fy, const double *__restrict__ Fz,
                                               long t, double v[], long &cell) {
  using F = Fam<FAM>;
  constexpr int NDPC = F::ndpc, DIM = F::dim;
  const int nb[3] = {b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]};
  const long total = (long)nb[0] * nb[1] * nb[2];
  if (t >= total) return false;
  const int i = (int)(t % nb[0]);
  const int j = (int)((t / nb[0]) % nb[1]);
  const int k = (int)(t / ((long)nb[0] * nb[1]));
#pragma unroll
  for (int d = 0; d < NDPC; ++d) v[d] = 0.;
  {
    const long f0 = (i + (long)(nb[0] + 1) * (j + (long)nb[1] * k)) * NDPC;
#pragma unroll
    for (int d = 0; d < NDPC; ++d) v[d] += m.hinv[0] * (Fx[f0 + d] - Fx[f0 + NDPC + d]);
  }
  if constexpr (DIM > 1) {
    const long f0 = (i + (long)nb[0] * (j + (long)(nb[1] + 1) * k)) * NDPC;
    const long f1 = f0 + (long)nb[0] * NDPC;
#pragma unroll
    for (int d = 0; d < NDPC; ++d) v[d] += m.hinv[1] * (Fy[f0 + d] - Fy[f1 + d]);
  }
  if constexpr (DIM > 2) {
    const long f0 = (i + (long)nb[0] * (j + (long)nb[1] * k)) * NDPC;
    const long f1 = f0 + (long)nb[0] * nb[1] * NDPC;
#pragma unroll
    for (int d = 0; d < NDPC; ++d) v[d] += m.hinv[2] * (Fz[f0 + d] - Fz[f1 + d]);
  }
  cell = (i + b.lo[0]) + (long)b.n[0] * ((j + b.lo[1]) + (long)b.n[1] * (k + b.lo[2]));
  if constexpr (FAM == Swe2d) {
    const double u0 = __ldg(U + cell * 3), u1 = __ldg(U + cell * 3 + 1), u2 = __ldg(U + cell * 3 + 2);
    v[1] -= div_rn(p.coriolis * u2, u0);
    v[2] += div_rn(p.coriolis * u1, u0);
  }
  return true;
}

template <int FAM>
__device__ __forceinline__ void balance_cell(const Box &b, const MeshArgs &m, const Phys &p,
                                             const double *__restrict__ U, const double *__restrict__ Fx,
                                             const double *__restrict__ Fy, const double *__restrict__ Fz,
                                             double *__restrict__ V, long t) {
  constexpr int NDPC = Fam<FAM>::ndpc;
  double v[NDPC];
  long cell;
  if (!balance_values<FAM>(b, m, p, U, Fx, Fy, Fz, t, v, cell)) return;
#pragma unroll
  for (int d = 0; d < NDPC; ++d) V[cell * NDPC + d] = v[d];
}

template <int FAM>
__global__ void __launch_bounds__(256)
k_struct_balance(Box b, MeshArgs m, Phys p, const double *__restrict__ U,
                 const double *__restrict__ Fx, const double *__restrict__ Fy,
                 const double *__restrict__ Fz, double *__restrict__ V) {
  balance_cell<FAM>(b, m, p, U, Fx, Fy, Fz, V, (long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
// V and J, reference per-cell formulation, rows whose stencil is entirely
// inside the domain (velocityAndJacInnerCellsImpl, euler_2d_prob_class.hpp:
// 632-720; scatter: mixin_directional_flux_balance_jacobian.hpp:120-285).
// J values are accumulated in place at the block offsets of the CSR row, in
// the reference's order, so repeated neighbours on tiny periodic meshes sum
// exactly as Eigen's coeffRef does.
// ---------------------------------------------------------------------------
template <int FAM, int SCHEME>
__global__ void __launch_bounds__(64)
k_rows_vj_inner(RowTable t, MeshArgs m, Phys p, const double *__restrict__ U,
                const int *__restrict__ rowptr, double *__restrict__ V, double *__restrict__ J) {
  using F = Fam<FAM>;
  constexpr int NDPC = F::ndpc, DIM = F::dim, H = SchemeTraits<SCHEME>::h, S = 2 * H + 1;
  constexpr int G = 2 * H;  // gradient length per face
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= t.nrows) return;
  const int r = t.rows[e];
  // zero this row block's entries
#pragma unroll 1
  for (int k = 0; k < NDPC; ++k)
    for (int q = rowptr[r * NDPC + k]; q < rowptr[r * NDPC + k + 1]; ++q) J[q] = 0.;
  double v[NDPC];
#pragma unroll
  for (int d = 0; d < NDPC; ++d) v[d] = 0.;
#pragma unroll 1
  for (int ax = 0; ax < DIM; ++ax) {
    double q[S][NDPC];
    int pos[S];
    const size_t base = ((size_t)e * DIM + ax) * S;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      load_cell<NDPC>(q[s], U, t.src[base + s], false, -1);
      pos[s] = t.jpos[base + s];
    }
    double uN[NDPC], uP[NDPC], fL[NDPC], fR[NDPC];
    double gLN[NDPC][G], gLP[NDPC][G], gRN[NDPC][G], gRP[NDPC][G];
    double JLN[NDPC * NDPC], JLP[NDPC * NDPC], JRN[NDPC * NDPC], JRP[NDPC * NDPC];
    reconstruct_face_grad<NDPC, SCHEME>(uN, uP, gLN, gLP, q);
    if (ax == 0) { F::template flux<0>(fL, uN, uP, p); F::template flux_jac<0>(JLN, JLP, uN, uP, p); }
    if constexpr (DIM > 1) if (ax == 1) { F::template flux<1>(fL, uN, uP, p); F::template flux_jac<1>(JLN, JLP, uN, uP, p); }
    if constexpr (DIM > 2) if (ax == 2) { F::template flux<2>(fL, uN, uP, p); F::template flux_jac<2>(JLN, JLP, uN, uP, p); }
    reconstruct_face_grad<NDPC, SCHEME>(uN, uP, gRN, gRP, q + 1);
    if (ax == 0) { F::template flux<0>(fR, uN, uP, p); F::template flux_jac<0>(JRN, JRP, uN, uP, p); }
    if constexpr (DIM > 1) if (ax == 1) { F::template flux<1>(fR, uN, uP, p); F::template flux_jac<1>(JRN, JRP, uN, uP, p); }
    if constexpr (DIM > 2) if (ax == 2) { F::template flux<2>(fR, uN, uP, p); F::template flux_jac<2>(JRN, JRP, uN, uP, p); }
    const double hinv = m.hinv[ax];
#pragma unroll
    for (int d = 0; d < NDPC; ++d) v[d] += hinv * (fL[d] - fR[d]);
    // scatter, reference order: for k, for j: left face (+=) then right face (-=)
#pragma unroll 1
    for (int k = 0; k < NDPC; ++k) {
      const int rb = rowptr[r * NDPC + k];
#pragma unroll 1
      for (int j = 0; j < NDPC; ++j) {
        const double ln = JLN[k * NDPC + j], lp = JLP[k * NDPC + j];
        const double rn = JRN[k * NDPC + j], rp = JRP[k * NDPC + j];
        if constexpr (SCHEME == FirstOrder) {
          J[rb + pos[0] + j] += ln * hinv;
          J[rb + pos[1] + j] += (lp - rn) * hinv;
          J[rb + pos[2] + j] += -rp * hinv;
        } else {
#pragma unroll
          for (int s = 0; s < G; ++s) {
            J[rb + pos[s] + j] += ln * gLN[j][s] * hinv;
            J[rb + pos[s] + j] += lp * gLP[j][s] * hinv;
          }
#pragma unroll
          for (int s = 0; s < G; ++s) {
            J[rb + pos[s + 1] + j] -= rn * gRN[j][s] * hinv;
            J[rb + pos[s + 1] + j] -= rp * gRP[j][s] * hinv;
          }
        }
      }
    }
  }
  if constexpr (FAM == Swe2d) {
    // swe_2d_prob_class.hpp:997-1012
    const int c = t.cell[e];
    const double u0 = __ldg(U + (size_t)c * 3), u1 = __ldg(U + (size_t)c * 3 + 1),
                 u2 = __ldg(U + (size_t)c * 3 + 2);
    v[1] -= div_rn(p.coriolis * u2, u0);
    v[2] += div_rn(p.coriolis * u1, u0);
    const int self = t.jpos[((size_t)e * DIM + 0) * S + H];
    const int rb1 = rowptr[r * 3 + 1], rb2 = rowptr[r * 3 + 2];
    J[rb1 + self + 0] += div_rn(p.coriolis * u2, (u0 * u0));
    J[rb1 + self + 2] += div_rn(-p.coriolis, u0);
    J[rb2 + self + 1] += div_rn(p.coriolis, u0);
    J[rb2 + self + 0] += div_rn(-p.coriolis * u1, (u0 * u0));
  }
#pragma unroll
  for (int d = 0; d < NDPC; ++d) V[(size_t)r * NDPC + d] = v[d];
}

// ---------------------------------------------------------------------------
// V and J of the rows of a sample mesh (or of any row set), each row's work
// spread over many threads.  GB300's FP64 units give one warp one instruction
// per ~64 cycles, so a row set of a few hundred rows is bound by the longest
// per-thread chain of FP64 instructions, not by the total: the work of a row
// is split until every thread's chain is short.
//   phase 1a  thread (side, row, face, dof): one side of the face's
//             reconstruction (value and, for inner rows, its gradient); the
//             side is uniform per warp, so each warp evaluates one side only
//   phase 1b  thread (part, row, face): the face flux (part 0) or the flux
//             Jacobians (part 1), again one part per warp
//   phase 2   thread (row, k, j): dof k of V (j == 0) and column dof j of row
//             k of the row's J blocks, every entry accumulated in exactly the
//             order of the per-row kernels (k_rows_vj_inner /
//             k_rows_vj_nearbd), then written once.
// Bit-identical to those kernels.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int pad_warp(int n) { return (n + 31) / 32 * 32; }

template <int FAM, int SCHEME> struct RowFace {
  static constexpr int NDPC = Fam<FAM>::ndpc, G = 2 * SchemeTraits<SCHEME>::h;
  double fl[NDPC];
  double JN[NDPC * NDPC], JP[NDPC * NDPC];
  double gN[NDPC][G], gP[NDPC][G];
  double uN[NDPC], uP[NDPC];
};

template <int FAM, int SCHEME> struct RowPar {
  static constexpr int NF = 2 * Fam<FAM>::dim, NDPC = Fam<FAM>::ndpc;
  static constexpr int RPB = 4;                        // rows per block
  static constexpr int SIDE = pad_warp(RPB * NF * NDPC);  // phase-1a threads per side
  static constexpr int PART = pad_warp(RPB * NF);         // phase-1b threads per part
  static constexpr int THREADS = 2 * SIDE;
  static_assert(2 * PART <= THREADS, "phase 1b fits the block");
};

template <int FAM, int SCHEME>
__global__ void __launch_bounds__(RowPar<FAM, SCHEME>::THREADS)
k_rows_vj_inner_par(RowTable t, MeshArgs m, Phys p, const double *__restrict__ U, const int *__restrict__ rowptr,
                    double *__restrict__ V, double *__restrict__ J) {
  using F = Fam<FAM>;
  using RF = RowFace<FAM, SCHEME>;
  using RP = RowPar<FAM, SCHEME>;
  constexpr int NDPC = F::ndpc, DIM = F::dim, H = SchemeTraits<SCHEME>::h, S = 2 * H + 1, G = 2 * H;
  constexpr int NF = RP::NF, RPB = RP::RPB;
  constexpr int NB = 1 + 2 * DIM * H;  // distinct column blocks of an inner row at most
  __shared__ RF fd[RPB][NF];
  const int tid = threadIdx.x;
  {  // phase 1a
    const int side = tid / RP::SIDE, slot = tid % RP::SIDE;
    const int rl = slot / (NF * NDPC), f = (slot / NDPC) % NF, d = slot % NDPC, ax = f >> 1, fs = f & 1;
    const int e = blockIdx.x * RPB + rl;
    if (slot < RPB * NF * NDPC && e < t.nrows) {
      double q[G];
      const size_t base = ((size_t)e * DIM + ax) * S;
#pragma unroll
      for (int s = 0; s < G; ++s) q[s] = __ldg(U + (size_t)t.src[base + fs + s] * NDPC + d);
      RF &o = fd[rl][f];
      double u, g[G];
      face_grad_side<SCHEME>(side, u, g, q);
      double *gs = side == 0 ? o.gN[d] : o.gP[d];
      (side == 0 ? o.uN : o.uP)[d] = u;
#pragma unroll
      for (int s = 0; s < G; ++s) gs[s] = g[s];
    }
  }
  __syncthreads();
  {  // phase 1b
    const int part = tid / RP::PART, slot = tid % RP::PART;
    const int rl = slot / NF, f = slot % NF, ax = f >> 1;
    const int e = blockIdx.x * RPB + rl;
    if (part < 2 && slot < RPB * NF && e < t.nrows) {
      RF &o = fd[rl][f];
      double uN[NDPC], uP[NDPC];
#pragma unroll
      for (int d = 0; d < NDPC; ++d) {
        uN[d] = o.uN[d];
        uP[d] = o.uP[d];
      }
      if (part == 0) {
        flux_ax<FAM>(o.fl, uN, uP, p, ax);  // one stream for all axes of the warp
      } else {
        F::flux_jac_ax(o.JN, o.JP, uN, uP, p, ax);  // one stream for all axes of the warp
      }
    }
  }
  __syncthreads();
  // phase 2: thread (row, k, j)
  for (int w = tid; w < RPB * NDPC * NDPC; w += blockDim.x) {
    const int rl = w / (NDPC * NDPC), k = (w / NDPC) % NDPC, j = w % NDPC;
    const int e = blockIdx.x * RPB + rl;
    if (e >= t.nrows) continue;
    const int r = t.rows[e];
    double acc[NB];
#pragma unroll
    for (int i = 0; i < NB; ++i) acc[i] = 0.;
#pragma unroll 1
    for (int ax = 0; ax < DIM; ++ax) {
      const double hinv = m.hinv[ax];
      const size_t base = ((size_t)e * DIM + ax) * S;
      int blk[S];
#pragma unroll
      for (int s = 0; s < S; ++s) blk[s] = t.jpos[base + s] / NDPC;
      const RF &L = fd[rl][2 * ax], &R = fd[rl][2 * ax + 1];
      const double ln = L.JN[k * NDPC + j], lp = L.JP[k * NDPC + j];
      const double rn = R.JN[k * NDPC + j], rp = R.JP[k * NDPC + j];
#pragma unroll
      for (int s = 0; s < G; ++s) {
        acc[blk[s]] += ln * L.gN[j][s] * hinv;
        acc[blk[s]] += lp * L.gP[j][s] * hinv;
      }
#pragma unroll
      for (int s = 0; s < G; ++s) {
        acc[blk[s + 1]] -= rn * R.gN[j][s] * hinv;
        acc[blk[s + 1]] -= rp * R.gP[j][s] * hinv;
      }
    }
    double vk = 0.;
    if (j == 0) {
#pragma unroll
      for (int ax = 0; ax < DIM; ++ax) vk += m.hinv[ax] * (fd[rl][2 * ax].fl[k] - fd[rl][2 * ax + 1].fl[k]);
    }
    if constexpr (FAM == Swe2d) {
      // swe_2d_prob_class.hpp:983-1012
      const int c = t.cell[e];
      const double u0 = __ldg(U + (size_t)c * 3), u1 = __ldg(U + (size_t)c * 3 + 1),
                   u2 = __ldg(U + (size_t)c * 3 + 2);
      if (j == 0 && k == 1) vk -= div_rn(p.coriolis * u2, u0);
      if (j == 0 && k == 2) vk += div_rn(p.coriolis * u1, u0);
      const int self = t.jpos[((size_t)e * DIM + 0) * S + H] / NDPC;
      if (k == 1 && j == 0) acc[self] += div_rn(p.coriolis * u2, (u0 * u0));
      if (k == 1 && j == 2) acc[self] += div_rn(-p.coriolis, u0);
      if (k == 2 && j == 1) acc[self] += div_rn(p.coriolis, u0);
      if (k == 2 && j == 0) acc[self] += div_rn(-p.coriolis * u1, (u0 * u0));
    }
    if (j == 0) V[(size_t)r * NDPC + k] = vk;
    const int rb = rowptr[r * NDPC + k];
    const int nb = (rowptr[r * NDPC + k + 1] - rb) / NDPC;
    for (int b = 0; b < nb && b < NB; ++b) J[rb + b * NDPC + j] = acc[b];
  }
}

// Near-boundary rows, split the same way: phase 1a one side of the scheme's
// face value (ghost entries through their recipes), phase 1b the face flux
// (part 0) or the first-order flux Jacobians of the face's two cells (part 1),
// phase 2 thread (row, k, j) accumulates exactly as k_rows_vj_nearbd does.
template <int FAM> struct NearFace {
  static constexpr int NDPC = Fam<FAM>::ndpc;
  double fl[NDPC];
  double JN[NDPC * NDPC], JP[NDPC * NDPC];
  double uN[NDPC], uP[NDPC];
};

template <int FAM> struct NearPar {
  static constexpr int NF = 2 * Fam<FAM>::dim, NDPC = Fam<FAM>::ndpc;
  static constexpr int RPB = 4;
  static constexpr int SIDE = pad_warp(RPB * NF * NDPC);
  static constexpr int PART = pad_warp(RPB * NF);
  static constexpr int THREADS = 2 * SIDE;
  static_assert(2 * PART <= THREADS, "phase 1b fits the block");
};

template <int FAM, int SCHEME>
__global__ void __launch_bounds__(NearPar<FAM>::THREADS)
k_rows_vj_nearbd_par(RowTable t, MeshArgs m, Phys p, const double *__restrict__ U, const int *__restrict__ rowptr,
                     double *__restrict__ V, double *__restrict__ J) {
  using F = Fam<FAM>;
  using NP = NearPar<FAM>;
  constexpr int NDPC = F::ndpc, DIM = F::dim, H = SchemeTraits<SCHEME>::h, S = 2 * H + 1, G = 2 * H;
  constexpr int NF = NP::NF, RPB = NP::RPB, NB = 1 + 2 * DIM;
  __shared__ NearFace<FAM> fd[RPB][NF];
  const int tid = threadIdx.x;
  {  // phase 1a
    const int side = tid / NP::SIDE, slot = tid % NP::SIDE;
    const int rl = slot / (NF * NDPC), f = (slot / NDPC) % NF, d = slot % NDPC, ax = f >> 1, fs = f & 1;
    const int e = blockIdx.x * RPB + rl;
    if (slot < RPB * NF * NDPC && e < t.nrows) {
      double q[G];
      const size_t base = ((size_t)e * DIM + ax) * S;
#pragma unroll
      for (int s = 0; s < G; ++s) {
        double qe[NDPC];
        load_entry<NDPC>(qe, U, t.src[base + fs + s], t.flip[base + fs + s], m.reflect[ax], m, t.gsx, t.gsy,
                         base + fs + s);
        q[s] = qe[d];
      }
      (side == 0 ? fd[rl][f].uN : fd[rl][f].uP)[d] = face_value_side<SCHEME>(side, q);
    }
  }
  __syncthreads();
  {  // phase 1b
    const int part = tid / NP::PART, slot = tid % NP::PART;
    const int rl = slot / NF, f = slot % NF, ax = f >> 1, fs = f & 1;
    const int e = blockIdx.x * RPB + rl;
    if (part < 2 && slot < RPB * NF && e < t.nrows) {
      NearFace<FAM> &o = fd[rl][f];
      if (part == 0) {
        double uN[NDPC], uP[NDPC];
#pragma unroll
        for (int d = 0; d < NDPC; ++d) {
          uN[d] = o.uN[d];
          uP[d] = o.uP[d];
        }
        flux_ax<FAM>(o.fl, uN, uP, p, ax);  // one stream for all axes of the warp
      } else {
        double q1[2][NDPC];
        const size_t b1 = ((size_t)e * DIM + ax) * 3;
#pragma unroll
        for (int s = 0; s < 2; ++s)
          load_entry<NDPC>(q1[s], U, t.src1[b1 + fs + s], t.flip1[b1 + fs + s], m.reflect[ax], m, t.gsx1, t.gsy1,
                           b1 + fs + s);
        F::flux_jac_ax(o.JN, o.JP, q1[0], q1[1], p, ax);  // one stream for all axes of the warp
      }
    }
  }
  __syncthreads();
  // phase 2: thread (row, k, j)
  for (int w = tid; w < RPB * NDPC * NDPC; w += blockDim.x) {
    const int rl = w / (NDPC * NDPC), k = (w / NDPC) % NDPC, j = w % NDPC;
    const int e = blockIdx.x * RPB + rl;
    if (e >= t.nrows) continue;
    const int r = t.rows[e];
    double acc[NB];
#pragma unroll
    for (int i = 0; i < NB; ++i) acc[i] = 0.;
#pragma unroll 1
    for (int ax = 0; ax < DIM; ++ax) {
      const double hinv = m.hinv[ax];
      const size_t b1 = ((size_t)e * DIM + ax) * 3;
      const int pl = t.jpos1[b1 + 0], pc = t.jpos1[b1 + 1], pr = t.jpos1[b1 + 2];
      const int bl = pl / NDPC, bc = pc / NDPC, br = pr / NDPC;
      const double *fac = t.jfac + ((size_t)e * DIM + ax) * NDPC;
      const NearFace<FAM> &L = fd[rl][2 * ax], &R = fd[rl][2 * ax + 1];
      const double ln = L.JN[k * NDPC + j], lp = L.JP[k * NDPC + j];
      const double rn = R.JN[k * NDPC + j], rp = R.JP[k * NDPC + j];
      acc[bc] += (lp - rn) * hinv;
      if (pl >= 0) acc[bl] += ln * hinv;
      if (pr >= 0) acc[br] += -rp * hinv;
      if (pl < 0) acc[bc] += (fac[j] * ln) * hinv;
      if (pr < 0) acc[bc] += (fac[j] * -rp) * hinv;
    }
    double vk = 0.;
    if (j == 0) {
#pragma unroll
      for (int ax = 0; ax < DIM; ++ax) vk += m.hinv[ax] * (fd[rl][2 * ax].fl[k] - fd[rl][2 * ax + 1].fl[k]);
    }
    if constexpr (FAM == Swe2d) {
      const int c = t.cell[e];
      const double u0 = __ldg(U + (size_t)c * 3), u1 = __ldg(U + (size_t)c * 3 + 1),
                   u2 = __ldg(U + (size_t)c * 3 + 2);
      if (j == 0 && k == 1) vk -= div_rn(p.coriolis * u2, u0);
      if (j == 0 && k == 2) vk += div_rn(p.coriolis * u1, u0);
      const int self = t.jpos1[((size_t)e * DIM + 0) * 3 + 1] / 3;
      if (k == 1 && j == 0) acc[self] += div_rn(p.coriolis * u2, (u0 * u0));
      if (k == 1 && j == 2) acc[self] += div_rn(-p.coriolis, u0);
      if (k == 2 && j == 1) acc[self] += div_rn(p.coriolis, u0);
      if (k == 2 && j == 0) acc[self] += div_rn(-p.coriolis * u1, (u0 * u0));
    }
    if (j == 0) V[(size_t)r * NDPC + k] = vk;
    const int rb = rowptr[r * NDPC + k];
    const int nb = (rowptr[r * NDPC + k + 1] - rb) / NDPC;
    for (int b = 0; b < nb && b < NB; ++b) J[rb + b * NDPC + j] = acc[b];
  }
}

// V of one or two row sets with each row's work spread over threads (the
// velocity-only counterpart of k_rows_vj_nearbd_par): thread (side, row, face, dof) one
// side of the face value (ghost entries through their recipes), thread (row,
// face) the face flux, thread (row, k) dof k of V in the order of
// k_rows_velocity.  Bit-identical to k_rows_velocity.  Rows per block (rpb <=
// RPB_MAX) are chosen at launch so that small row sets spread over the SMs.
template <int FAM> struct VelPar {
  static constexpr int NF = 2 * Fam<FAM>::dim, NDPC = Fam<FAM>::ndpc;
  static constexpr int RPB_MAX = Fam<FAM>::dim == 3 ? 4 : 8;
  static constexpr int SIDE = pad_warp(RPB_MAX * NF * NDPC);
  static constexpr int THREADS = 2 * SIDE;
  static constexpr int PART = pad_warp(RPB_MAX * NF);  // one warp: the block's faces
  static_assert(2 * PART <= THREADS, "the two face-state halves fit the block");
};

template <int FAM> struct VelFace {
  static constexpr int NDPC = Fam<FAM>::ndpc;
  double fl[NDPC];
  double uN[NDPC], uP[NDPC];
};

template <int FAM, int SCHEME>
__global__ void __launch_bounds__(VelPar<FAM>::THREADS)
k_rows_velocity_par(RowTable ta, RowTable tb, int nbA, int rpb, MeshArgs m, Phys p, const double *__restrict__ U,
                    double *__restrict__ V) {
  using F = Fam<FAM>;
  using VP = VelPar<FAM>;
  constexpr int NDPC = F::ndpc, DIM = F::dim, H = SchemeTraits<SCHEME>::h, S = 2 * H + 1, G = 2 * H;
  constexpr int NF = VP::NF;
  __shared__ VelFace<FAM> fd[VP::RPB_MAX][NF];
  __shared__ typename F::Side sSide[VP::RPB_MAX][NF][2];  // the two face states' halves of each flux
  // blocks [0, nbA) take the rows of table ta, the others those of tb
  const bool first = (int)blockIdx.x < nbA;
  const RowTable &t = first ? ta : tb;
  const int tid = threadIdx.x, e0 = (first ? (int)blockIdx.x : (int)blockIdx.x - nbA) * rpb;
  {  // one side of one dof's face value
    const int side = tid / VP::SIDE, slot = tid % VP::SIDE;
    const int rl = slot / (NF * NDPC), f = (slot / NDPC) % NF, d = slot % NDPC, ax = f >> 1, fs = f & 1;
    const int e = e0 + rl;
    if (slot < rpb * NF * NDPC && e < t.nrows) {
      const size_t base = ((size_t)e * DIM + ax) * S;
      double q[G];
#pragma unroll
      for (int s = 0; s < G; ++s) {
        double qe[NDPC];
        load_entry<NDPC>(qe, U, t.src[base + fs + s], t.flip[base + fs + s], m.reflect[ax], m, t.gsx, t.gsy,
                         base + fs + s);
        q[s] = qe[d];
      }
      (side == 0 ? fd[rl][f].uN : fd[rl][f].uP)[d] = face_value_side<SCHEME>(side, q);
    }
  }
  __syncthreads();
  // the face flux in two halves, so that no warp evaluates a whole flux (a
  // stage costs its longest per-warp FP64 instruction stream): warps 0 / 1
  // the left / right face state's quantities, then warp 0 their combination
  {
    const int part = tid / VP::PART, slot = tid % VP::PART;
    const int rl = slot / NF, f = slot % NF, ax = f >> 1;
    if (part < 2 && slot < rpb * NF && e0 + rl < t.nrows) {
      const double *q = part == 0 ? fd[rl][f].uN : fd[rl][f].uP;
      typename F::Side &so = sSide[rl][f][part];
      F::flux_side_ax(so, q, p, ax);  // one stream for all axes of the warp
    }
  }
  __syncthreads();
  if (tid < rpb * NF) {
    const int rl = tid / NF, f = tid % NF;
    if (e0 + rl < t.nrows) {
      VelFace<FAM> &o = fd[rl][f];
      const typename F::Side &L = sSide[rl][f][0], &R = sSide[rl][f][1];
      F::template flux_combine<0>(o.fl, o.uN, o.uP, L, R, p);  // the combination does not depend on the axis
    }
  }
  __syncthreads();
  if (tid < rpb * NDPC) {  // dof k of the row's velocity
    const int rl = tid / NDPC, k = tid % NDPC;
    const int e = e0 + rl;
    if (e < t.nrows) {
      double vk = 0.;
#pragma unroll
      for (int ax = 0; ax < DIM; ++ax) vk += m.hinv[ax] * (fd[rl][2 * ax].fl[k] - fd[rl][2 * ax + 1].fl[k]);
      if constexpr (FAM == Swe2d) {
        // swe_2d_prob_class.hpp:983-994
        const int c = t.cell[e];
        const double u0 = __ldg(U + (size_t)c * 3), u1 = __ldg(U + (size_t)c * 3 + 1),
                     u2 = __ldg(U + (size_t)c * 3 + 2);
        if (k == 1) vk -= div_rn(p.coriolis * u2, u0);
        if (k == 2) vk += div_rn(p.coriolis * u1, u0);
      }
      V[(size_t)t.rows[e] * NDPC + k] = vk;
    }
  }
}

// V and J for rows near a non-periodic boundary: V with the scheme's stencil
// (ghosts folded into the table), J first order with the ghost dependence
// folded into the diagonal block by the BC factors
// (velocityAndJacNearBDCellsImplDifferentScheme, euler_2d_prob_class.hpp:
// 833-988; ComputeDirectionalFluxBalanceFirstOrderJacobianOnBoundaryCell,
// mixin_directional_flux_balance_jacobian.hpp:287-372).
template <int FAM, int SCHEME>
__global__ void __launch_bounds__(64)
k_rows_vj_nearbd(RowTable t, MeshArgs m, Phys p, const double *__restrict__ U,
                 const int *__restrict__ rowptr, double *__restrict__ V, double *__restrict__ J) {
  using F = Fam<FAM>;
  constexpr int NDPC = F::ndpc, DIM = F::dim, H = SchemeTraits<SCHEME>::h, S = 2 * H + 1;
  constexpr int NB = 1 + 2 * DIM;  // column blocks of a first-order row at most
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= t.nrows) return;
  const int r = t.rows[e];
  // the row's CSR values, accumulated locally in the order of the reference's
  // in-place updates and written once at the end: acc[block][k][j]
  double acc[NB * NDPC * NDPC];
#pragma unroll
  for (int i = 0; i < NB * NDPC * NDPC; ++i) acc[i] = 0.;
  double v[NDPC];
#pragma unroll
  for (int d = 0; d < NDPC; ++d) v[d] = 0.;
#pragma unroll 1
  for (int ax = 0; ax < DIM; ++ax) {
    const double hinv = m.hinv[ax];
    {  // velocity with the scheme's stencil
      double q[S][NDPC];
      const size_t base = ((size_t)e * DIM + ax) * S;
#pragma unroll
      for (int s = 0; s < S; ++s)
        load_entry<NDPC>(q[s], U, t.src[base + s], t.flip[base + s], m.reflect[ax], m, t.gsx, t.gsy, base + s);
      double uN[NDPC], uP[NDPC], fL[NDPC], fR[NDPC];
      reconstruct_face<NDPC, SCHEME>(uN, uP, q);
      if (ax == 0) F::template flux<0>(fL, uN, uP, p);
      if constexpr (DIM > 1) if (ax == 1) F::template flux<1>(fL, uN, uP, p);
      if constexpr (DIM > 2) if (ax == 2) F::template flux<2>(fL, uN, uP, p);
      reconstruct_face<NDPC, SCHEME>(uN, uP, q + 1);
      if (ax == 0) F::template flux<0>(fR, uN, uP, p);
      if constexpr (DIM > 1) if (ax == 1) F::template flux<1>(fR, uN, uP, p);
      if constexpr (DIM > 2) if (ax == 2) F::template flux<2>(fR, uN, uP, p);
#pragma unroll
      for (int d = 0; d < NDPC; ++d) v[d] += hinv * (fL[d] - fR[d]);
    }
    {  // first-order Jacobian with BC factors
      double q[3][NDPC];
      const size_t base = ((size_t)e * DIM + ax) * 3;
#pragma unroll
      for (int s = 0; s < 3; ++s)
        load_entry<NDPC>(q[s], U, t.src1[base + s], t.flip1[base + s], m.reflect[ax], m, t.gsx1, t.gsy1, base + s);
      double JLN[NDPC * NDPC], JLP[NDPC * NDPC], JRN[NDPC * NDPC], JRP[NDPC * NDPC];
      if (ax == 0) { F::template flux_jac<0>(JLN, JLP, q[0], q[1], p); F::template flux_jac<0>(JRN, JRP, q[1], q[2], p); }
      if constexpr (DIM > 1) if (ax == 1) { F::template flux_jac<1>(JLN, JLP, q[0], q[1], p); F::template flux_jac<1>(JRN, JRP, q[1], q[2], p); }
      if constexpr (DIM > 2) if (ax == 2) { F::template flux_jac<2>(JLN, JLP, q[0], q[1], p); F::template flux_jac<2>(JRN, JRP, q[1], q[2], p); }
      const int pl = t.jpos1[base + 0], pc = t.jpos1[base + 1], pr = t.jpos1[base + 2];
      const int bl = pl / NDPC, bc = pc / NDPC, br = pr / NDPC;
      const double *fac = t.jfac + ((size_t)e * DIM + ax) * NDPC;
#pragma unroll 1
      for (int k = 0; k < NDPC; ++k) {
        double *ac = acc + (bc * NDPC + k) * NDPC;
        for (int j = 0; j < NDPC; ++j) ac[j] += (JLP[k * NDPC + j] - JRN[k * NDPC + j]) * hinv;
        if (pl >= 0) {
          double *al = acc + (bl * NDPC + k) * NDPC;
          for (int j = 0; j < NDPC; ++j) al[j] += JLN[k * NDPC + j] * hinv;
        }
        if (pr >= 0) {
          double *ar = acc + (br * NDPC + k) * NDPC;
          for (int j = 0; j < NDPC; ++j) ar[j] += -JRP[k * NDPC + j] * hinv;
        }
        if (pl < 0)
          for (int j = 0; j < NDPC; ++j) ac[j] += (fac[j] * JLN[k * NDPC + j]) * hinv;
        if (pr < 0)
          for (int j = 0; j < NDPC; ++j) ac[j] += (fac[j] * -JRP[k * NDPC + j]) * hinv;
      }
    }
  }
  if constexpr (FAM == Swe2d) {
    const int c = t.cell[e];
    const double u0 = __ldg(U + (size_t)c * 3), u1 = __ldg(U + (size_t)c * 3 + 1),
                 u2 = __ldg(U + (size_t)c * 3 + 2);
    v[1] -= div_rn(p.coriolis * u2, u0);
    v[2] += div_rn(p.coriolis * u1, u0);
    const int self = t.jpos1[((size_t)e * DIM + 0) * 3 + 1] / 3;
    acc[(self * 3 + 1) * 3 + 0] += div_rn(p.coriolis * u2, (u0 * u0));
    acc[(self * 3 + 1) * 3 + 2] += div_rn(-p.coriolis, u0);
    acc[(self * 3 + 2) * 3 + 1] += div_rn(p.coriolis, u0);
    acc[(self * 3 + 2) * 3 + 0] += div_rn(-p.coriolis * u1, (u0 * u0));
  }
#pragma unroll
  for (int d = 0; d < NDPC; ++d) V[(size_t)r * NDPC + d] = v[d];
#pragma unroll 1
  for (int k = 0; k < NDPC; ++k) {
    const int rb = rowptr[r * NDPC + k];
    const int nb = (rowptr[r * NDPC + k + 1] - rb) / NDPC;
    for (int b = 0; b < nb && b < NB; ++b)
      for (int j = 0; j < NDPC; ++j) J[rb + b * NDPC + j] = acc[(b * NDPC + k) * NDPC + j];
  }
}

}  // namespace pda
