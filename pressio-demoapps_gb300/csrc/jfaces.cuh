// Velocity + exact Jacobian on the inner box of a natural-order full mesh,
// each face computed once.
//
// The reference (and k_rows_vj_inner) evaluates, for every row, the WENO
// reconstruction with gradients and the Rusanov flux Jacobians of its left and
// right faces, so every face is computed twice, and accumulates
//     J[row k, col(c_s) j] += (JLNeg(k,j) * gLNeg(j,s)) * h^-1    (left face)
//     J[row k, col(c_s) j] += (JLPos(k,j) * gLPos(j,s)) * h^-1
//     J[row k, col(c_s) j] -= (JRNeg(k,j) * gRNeg(j,s)) * h^-1    (right face)
//     J[row k, col(c_s) j] -= (JRPos(k,j) * gRPos(j,s)) * h^-1
// (mixin_directional_flux_balance_jacobian.hpp:222-282), x then y then z.
// Every product term belongs to one face and is the same for the two cells
// that share it, so:
//  1. k_jfaces: one thread per face writes the face flux and all its product
//     terms (Neg and Pos, per stencil position s, row k, column dof j) to a
//     structure-of-arrays scratch [component][face] (coalesced);
//  2. k_jassemble: one thread per cell gathers the terms of its faces and
//     adds them entry by entry in the reference's order (left Neg, left Pos,
//     right Neg, right Pos; axes in order; the shallow-water Coriolis terms
//     last), writing each CSR value once.  Results are bit-identical to the
//     per-row formulation.
// Used when no stencil repeats a cell (periodic axes of at least 2H+1 cells).
#pragma once

#include "kernels.cuh"

namespace pda {

template <int FAM, int SCHEME> struct JFaceLayout {
  static constexpr int NDPC = Fam<FAM>::ndpc, H = SchemeTraits<SCHEME>::h, G = 2 * H;
  static constexpr int NT = G * NDPC * NDPC;  // product terms per side (Neg or Pos)
  static constexpr int NCOMP = NDPC + 2 * NT;  // flux, Neg terms, Pos terms
  PDA_HD static constexpr int neg(int s, int k, int j) { return NDPC + (s * NDPC + k) * NDPC + j; }
  PDA_HD static constexpr int pos(int s, int k, int j) { return NDPC + NT + (s * NDPC + k) * NDPC + j; }
};

// faces normal to AXIS of box b, same numbering as k_struct_faces
template <int FAM, int SCHEME, int AXIS>
__global__ void __launch_bounds__(128)
k_jfaces(Box b, Phys p, double hinv, const double *__restrict__ U, double *__restrict__ T) {
  using F = Fam<FAM>;
  using Lay = JFaceLayout<FAM, SCHEME>;
  constexpr int NDPC = F::ndpc, H = Lay::H, G = Lay::G;
  const int nf[3] = {b.hi[0] - b.lo[0] + (AXIS == 0), b.hi[1] - b.lo[1] + (AXIS == 1),
                     b.hi[2] - b.lo[2] + (AXIS == 2)};
  const long total = (long)nf[0] * nf[1] * nf[2];
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  int c[3];
  c[0] = (int)(t % nf[0]) + b.lo[0];
  c[1] = (int)((t / nf[0]) % nf[1]) + b.lo[1];
  c[2] = (int)(t / ((long)nf[0] * nf[1])) + b.lo[2];
  double q[G][NDPC];
#pragma unroll
  for (int s = 0; s < G; ++s) {
    int cc[3] = {c[0], c[1], c[2]};
    bool mir;
    cc[AXIS] = map_cell(c[AXIS] - H + s, b.n[AXIS], b.mode[AXIS], mir);
    const long cell = cc[0] + (long)b.n[0] * (cc[1] + (long)b.n[1] * cc[2]);
#pragma unroll
    for (int d = 0; d < NDPC; ++d) q[s][d] = __ldg(U + cell * NDPC + d);
  }
  double uN[NDPC], uP[NDPC], gN[NDPC][G], gP[NDPC][G], fl[NDPC], JN[NDPC * NDPC], JP[NDPC * NDPC];
  reconstruct_face_grad<NDPC, SCHEME>(uN, uP, gN, gP, q);
  F::template flux<AXIS>(fl, uN, uP, p);
  F::template flux_jac<AXIS>(JN, JP, uN, uP, p);
#pragma unroll
  for (int d = 0; d < NDPC; ++d) T[d * total + t] = fl[d];
#pragma unroll
  for (int k = 0; k < NDPC; ++k)
#pragma unroll
    for (int j = 0; j < NDPC; ++j) {
      const double ln = JN[k * NDPC + j], lp = JP[k * NDPC + j];
#pragma unroll
      for (int s = 0; s < G; ++s) {
        T[Lay::neg(s, k, j) * total + t] = ln * gN[j][s] * hinv;
        T[Lay::pos(s, k, j) * total + t] = lp * gP[j][s] * hinv;
      }
    }
}

// one thread per box cell: V row and the CSR values of its NDPC rows
template <int FAM, int SCHEME>
__global__ void __launch_bounds__(128)
k_jassemble(Box b, MeshArgs m, Phys p, const double *__restrict__ U, const double *__restrict__ Tx,
            const double *__restrict__ Ty, const double *__restrict__ Tz, const int *__restrict__ rowptr,
            double *__restrict__ V, double *__restrict__ J) {
  using F = Fam<FAM>;
  using Lay = JFaceLayout<FAM, SCHEME>;
  constexpr int NDPC = F::ndpc, DIM = F::dim, H = Lay::H, G = Lay::G;
  constexpr int NB = 1 + DIM * 2 * H;  // stencil blocks: centre, then per axis offsets -H..-1, 1..H
  const int nb[3] = {b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]};
  const long ncell = (long)nb[0] * nb[1] * nb[2];
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell) return;
  const int i0 = (int)(t % nb[0]), i1 = (int)((t / nb[0]) % nb[1]), i2 = (int)(t / ((long)nb[0] * nb[1]));
  const int c[3] = {i0 + b.lo[0], i1 + b.lo[1], i2 + b.lo[2]};
  const long gid = c[0] + (long)b.n[0] * (c[1] + (long)b.n[1] * c[2]);

  // left / right face of the cell per axis and the face counts (k_jfaces numbering)
  const double *Ta[3] = {Tx, Ty, Tz};
  long fL[3], fR[3], nfT[3];
  nfT[0] = (long)(nb[0] + 1) * nb[1] * nb[2];
  fL[0] = i0 + (long)(nb[0] + 1) * (i1 + (long)nb[1] * i2);
  fR[0] = fL[0] + 1;
  nfT[1] = (long)nb[0] * (nb[1] + 1) * nb[2];
  fL[1] = i0 + (long)nb[0] * (i1 + (long)(nb[1] + 1) * i2);
  fR[1] = fL[1] + nb[0];
  nfT[2] = (long)nb[0] * nb[1] * (nb[2] + 1);
  fL[2] = i0 + (long)nb[0] * (i1 + (long)nb[1] * i2);
  fR[2] = fL[2] + (long)nb[0] * nb[1];

  // column rank of every stencil block in the sorted CSR row
  long gids[NB];
  gids[0] = gid;
#pragma unroll
  for (int a = 0; a < DIM; ++a)
#pragma unroll
    for (int e = 0; e < 2 * H; ++e) {
      const int d = e < H ? e - H : e - H + 1;
      int cc[3] = {c[0], c[1], c[2]};
      bool mir;
      cc[a] = map_cell(c[a] + d, b.n[a], b.mode[a], mir);
      gids[1 + a * 2 * H + e] = cc[0] + (long)b.n[0] * (cc[1] + (long)b.n[1] * cc[2]);
    }
  int rank[NB];
#pragma unroll
  for (int x = 0; x < NB; ++x) {
    int r = 0;
#pragma unroll
    for (int y = 0; y < NB; ++y) r += gids[y] < gids[x] ? 1 : 0;
    rank[x] = r;
  }

  // velocity (same order as the per-row kernel)
  double v[NDPC];
#pragma unroll
  for (int d = 0; d < NDPC; ++d) v[d] = 0.;
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    const double hinv = m.hinv[a];
#pragma unroll
    for (int d = 0; d < NDPC; ++d)
      v[d] += hinv * (__ldg(Ta[a] + d * nfT[a] + fL[a]) - __ldg(Ta[a] + d * nfT[a] + fR[a]));
  }
  double u0 = 0., u1 = 0., u2 = 0.;
  if constexpr (FAM == Swe2d) {
    u0 = __ldg(U + gid * 3);
    u1 = __ldg(U + gid * 3 + 1);
    u2 = __ldg(U + gid * 3 + 2);
    v[1] -= p.coriolis * u2 / u0;
    v[2] += p.coriolis * u1 / u0;
  }
#pragma unroll
  for (int d = 0; d < NDPC; ++d) V[gid * NDPC + d] = v[d];

#pragma unroll 1
  for (int k = 0; k < NDPC; ++k) {
    double *Jrow = J + rowptr[gid * NDPC + k];
    // centre block: every axis contributes
#pragma unroll
    for (int j = 0; j < NDPC; ++j) {
      double acc = 0.;
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        const double *T = Ta[a];
        acc += __ldg(T + Lay::neg(H, k, j) * nfT[a] + fL[a]);
        acc += __ldg(T + Lay::pos(H, k, j) * nfT[a] + fL[a]);
        acc -= __ldg(T + Lay::neg(H - 1, k, j) * nfT[a] + fR[a]);
        acc -= __ldg(T + Lay::pos(H - 1, k, j) * nfT[a] + fR[a]);
      }
      if constexpr (FAM == Swe2d) {
        // swe_2d_prob_class.hpp:997-1012
        if (k == 1 && j == 0) acc += p.coriolis * u2 / (u0 * u0);
        if (k == 1 && j == 2) acc += -p.coriolis / u0;
        if (k == 2 && j == 1) acc += p.coriolis / u0;
        if (k == 2 && j == 0) acc += -p.coriolis * u1 / (u0 * u0);
      }
      Jrow[rank[0] * NDPC + j] = acc;
    }
    // off-centre blocks along each axis
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      const double *T = Ta[a];
#pragma unroll 1
      for (int e = 0; e < 2 * H; ++e) {
        const int d = e < H ? e - H : e - H + 1;
        const int sL = d + H, sR = d + H - 1;  // stencil slot in the left / right face
        int rk = 0;
#pragma unroll
        for (int x = 0; x < 2 * H; ++x)
          if (x == e) rk = rank[1 + a * 2 * H + x];
        double *dst = Jrow + rk * NDPC;
#pragma unroll
        for (int j = 0; j < NDPC; ++j) {
          double acc = 0.;
          if (sL <= G - 1) {
            acc += __ldg(T + Lay::neg(sL, k, j) * nfT[a] + fL[a]);
            acc += __ldg(T + Lay::pos(sL, k, j) * nfT[a] + fL[a]);
          }
          if (sR >= 0) {
            acc -= __ldg(T + Lay::neg(sR, k, j) * nfT[a] + fR[a]);
            acc -= __ldg(T + Lay::pos(sR, k, j) * nfT[a] + fR[a]);
          }
          dst[j] = acc;
        }
      }
    }
  }
}

}  // namespace pda
