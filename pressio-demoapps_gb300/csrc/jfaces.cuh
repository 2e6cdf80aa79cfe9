// Velocity + exact Jacobian on the inner box of a natural-order full mesh,
// each face computed once, the CSR values assembled in the same kernel.
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
// that share it.  k_jtile takes one axis per launch: a block owns LANES
// consecutive faces of one line of the box (LANES - 1 cells; the face at a
// tile's end is computed by both neighbouring tiles), one thread per face.
// For each row dof k in turn the face threads put the row-k product terms
// (Neg and Pos, per stencil position s and column dof j) in shared memory
// and the cell threads add them entry by entry in the reference's order
// (left Neg, left Pos, right Neg, right Pos) into the CSR values.  The
// centre block gathers every axis: the first axis's launch starts it from
// zero, later axes continue the partial sum stored in J (the same
// additions in the same order), and the last adds the shallow-water
// Coriolis terms.  Velocities follow the same pattern.  Results are
// bit-identical to the per-row formulation; DRAM traffic is the state reads,
// the CSR values written (the centre block re-read once per later axis) and
// the velocity.
// Used when no stencil repeats a cell (periodic axes of at least 2H+1 cells).
#pragma once

#include "kernels.cuh"

namespace pda {

template <int FAM, int SCHEME, int LANES_ = 64> struct JTileCfg {
  static constexpr int NDPC = Fam<FAM>::ndpc, DIM = Fam<FAM>::dim, H = SchemeTraits<SCHEME>::h, G = 2 * H;
  static constexpr int LANES = LANES_, TW = LANES - 1;  // faces and cells per tile
};

template <int FAM, int SCHEME, int LANES> struct JTileSmem {
  using C = JTileCfg<FAM, SCHEME, LANES>;
  double fl[C::NDPC][LANES];                 // face fluxes
  double tN[C::G][C::NDPC][LANES];           // row-k terms (JNeg(k,j) gNeg(j,s)) h^-1
  double tP[C::G][C::NDPC][LANES];           // row-k terms (JPos(k,j) gPos(j,s)) h^-1
};

// grid: x = lines of the box along AXIS (first other axis fastest), y = face
// chunks of TW faces
// Resident blocks per SM the register allocation must allow.  The kernel is
// FP64-bound with few warps (one face per thread holds its gradients and flux
// Jacobians); measured at 1024^2 / 96^3, capping registers for 8 blocks of 64
// threads (2D) or 6 (3D) beats the uncapped allocation by 4-6 % / 3 %, the
// few spills included.
template <int DIM> struct JTileMinBlocks {
  static constexpr int value = DIM == 3 ? 6 : 8;
};

template <int FAM, int SCHEME, int AXIS, int LANES>
__global__ void __launch_bounds__(LANES, JTileMinBlocks<Fam<FAM>::dim>::value)
k_jtile(Box b, MeshArgs m, Phys p, const double *__restrict__ U, const int *__restrict__ rowptr,
        double *__restrict__ V, double *__restrict__ J) {
  using F = Fam<FAM>;
  using C = JTileCfg<FAM, SCHEME, LANES>;
  constexpr int NDPC = C::NDPC, DIM = C::DIM, H = C::H, G = C::G, TW = C::TW;
  constexpr bool FIRST = AXIS == 0, LAST = AXIS == DIM - 1;
  constexpr int NB = 1 + DIM * 2 * H;  // stencil blocks: centre, then per axis offsets -H..-1, 1..H
  constexpr int A1 = AXIS == 0 ? 1 : 0, A2 = AXIS == 2 ? 1 : 2;
  __shared__ JTileSmem<FAM, SCHEME, LANES> sm;
  const int tx = threadIdx.x;
  const int nb1 = b.hi[A1] - b.lo[A1], nb2 = b.hi[A2] - b.lo[A2];
  const long line = blockIdx.x;
  const bool lineOk = line < (long)nb1 * nb2;
  int c[3];
  c[A1] = b.lo[A1] + (lineOk ? (int)(line % nb1) : 0);
  c[A2] = b.lo[A2] + (lineOk ? (int)(line / nb1) : 0);
  const int f0 = b.lo[AXIS] + (int)blockIdx.y * TW;
  const int f = f0 + tx;  // this thread's face, between cells f - 1 and f
  const bool faceOk = lineOk && f <= b.hi[AXIS];
  const bool cellOk = lineOk && tx < TW && f < b.hi[AXIS];  // cell f: faces tx (left), tx + 1 (right)
  const double hinv = m.hinv[AXIS];

  // ---- the face: reconstruction with gradients, flux and flux Jacobians
  double gN[NDPC][G], gP[NDPC][G], JN[NDPC * NDPC], JP[NDPC * NDPC];
  if (faceOk) {
    double q[G][NDPC];
#pragma unroll
    for (int s = 0; s < G; ++s) {
      int cc[3] = {c[0], c[1], c[2]};
      bool mir;
      cc[AXIS] = map_cell(f - H + s, b.n[AXIS], b.mode[AXIS], mir);
      const long cell = cc[0] + (long)b.n[0] * (cc[1] + (long)b.n[1] * cc[2]);
#pragma unroll
      for (int d = 0; d < NDPC; ++d) q[s][d] = __ldg(U + cell * NDPC + d);
    }
    double uN[NDPC], uP[NDPC], fl[NDPC];
    reconstruct_face_grad<NDPC, SCHEME>(uN, uP, gN, gP, q);
    F::template flux<AXIS>(fl, uN, uP, p);
    F::template flux_jac<AXIS>(JN, JP, uN, uP, p);
#pragma unroll
    for (int d = 0; d < NDPC; ++d) sm.fl[d][tx] = fl[d];
  }

  // ---- the cell: its row position, block ranks and velocity
  c[AXIS] = f;
  const long gid = c[0] + (long)b.n[0] * (c[1] + (long)b.n[1] * c[2]);
  int rank[NB];
  double u0 = 0., u1 = 0., u2 = 0.;
  if (cellOk) {
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
    // column rank of every stencil block in the sorted CSR row
#pragma unroll
    for (int x = 0; x < NB; ++x) {
      int r = 0;
#pragma unroll
      for (int y = 0; y < NB; ++y) r += gids[y] < gids[x] ? 1 : 0;
      rank[x] = r;
    }
    if constexpr (FAM == Swe2d && LAST) {
      u0 = __ldg(U + gid * 3);
      u1 = __ldg(U + gid * 3 + 1);
      u2 = __ldg(U + gid * 3 + 2);
    }
  }
  __syncthreads();
  if (cellOk) {
    // velocity: sum over the axes in order (the first from zero), sources last
    double v[NDPC];
#pragma unroll
    for (int d = 0; d < NDPC; ++d) {
      const double prev = FIRST ? 0. : V[gid * NDPC + d];
      v[d] = prev + hinv * (sm.fl[d][tx] - sm.fl[d][tx + 1]);
    }
    if constexpr (FAM == Swe2d && LAST) {
      v[1] -= div_rn(p.coriolis * u2, u0);
      v[2] += div_rn(p.coriolis * u1, u0);
    }
#pragma unroll
    for (int d = 0; d < NDPC; ++d) V[gid * NDPC + d] = v[d];
  }

  // ---- CSR values, one row dof at a time
#pragma unroll
  for (int k = 0; k < NDPC; ++k) {
    if (faceOk) {
#pragma unroll
      for (int j = 0; j < NDPC; ++j) {
        const double ln = JN[k * NDPC + j], lp = JP[k * NDPC + j];
#pragma unroll
        for (int s = 0; s < G; ++s) {
          sm.tN[s][j][tx] = ln * gN[j][s] * hinv;
          sm.tP[s][j][tx] = lp * gP[j][s] * hinv;
        }
      }
    }
    __syncthreads();
    if (cellOk) {
      double *Jrow = J + rowptr[gid * NDPC + k];
      // centre block: left face slot H, right face slot H - 1
      double *dst = Jrow + rank[0] * NDPC;
#pragma unroll
      for (int j = 0; j < NDPC; ++j) {
        double acc = FIRST ? 0. : dst[j];
        acc += sm.tN[H][j][tx];
        acc += sm.tP[H][j][tx];
        acc -= sm.tN[H - 1][j][tx + 1];
        acc -= sm.tP[H - 1][j][tx + 1];
        if constexpr (FAM == Swe2d && LAST) {
          // swe_2d_prob_class.hpp:997-1012
          if (k == 1 && j == 0) acc += div_rn(p.coriolis * u2, (u0 * u0));
          if (k == 1 && j == 2) acc += div_rn(-p.coriolis, u0);
          if (k == 2 && j == 1) acc += div_rn(p.coriolis, u0);
          if (k == 2 && j == 0) acc += div_rn(-p.coriolis * u1, (u0 * u0));
        }
        dst[j] = acc;
      }
      // off-centre blocks along AXIS
#pragma unroll
      for (int e = 0; e < 2 * H; ++e) {
        const int d = e < H ? e - H : e - H + 1;
        const int sL = d + H, sR = d + H - 1;  // stencil slot in the left / right face
        double *o = Jrow + rank[1 + AXIS * 2 * H + e] * NDPC;
#pragma unroll
        for (int j = 0; j < NDPC; ++j) {
          double acc = 0.;
          if (sL <= G - 1) {
            acc += sm.tN[sL][j][tx];
            acc += sm.tP[sL][j][tx];
          }
          if (sR >= 0) {
            acc -= sm.tN[sR][j][tx + 1];
            acc -= sm.tP[sR][j][tx + 1];
          }
          o[j] = acc;
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace pda
