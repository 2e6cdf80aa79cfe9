// Tiled face kernels for WENO3 / WENO5 on natural-order full meshes.
//
// The FP64 pipe bounds this path on GB300, so the kernels minimise FP64
// operations while keeping every value bit-identical to the reference:
//  * products by powers of two are fused into the following sum (w5_* in
//    numerics.cuh: the product is exact, so one rounding equals two);
//  * each face is computed once (the reference computes it from both cells);
//  * the smoothness indicators of a cell triple (WENO5) or pair (WENO3) and
//    the alpha terms built from them enter up to three one-sided
//    reconstructions of neighbouring faces with identical expression trees
//    (impl/weno5.hpp:112-178, impl/weno3.hpp:82-131), so they are computed
//    once per cell into shared memory and reused;
//  * the reference's products by small integers, 1/2, 1/4 and constants and
//    its divisions and square roots run on the integer pipe
//    (fp64_intpipe.cuh), bit for bit;
//  * the code stays small enough for the instruction cache: the per-dof
//    loops of the cell and face phases are not unrolled (face states kept in
//    registers by predicated moves) and every division and square root is
//    an out-of-line call.  Fully unrolled with inline divisions the kernel
//    is a straight line of about 10^4 instructions per thread, and
//    instruction-fetch stalls were its largest stall reason;
//  * boundary faces of the mirror-type boundary conditions (2D Neumann and
//    slip wall, whose ghost layers are exact mirror images,
//    euler_2d_ghost_filler_neumann.hpp:101-276,
//    swe_2d_ghost_filler_inviscid_wall.hpp:99-278) are computed in the same
//    pass by mirrored loads, so no per-row boundary kernel is needed.
//
// Block: LANES threads along the face axis x NR lines; a block produces TW
// faces of each of its NR lines (TW = LANES - 3 for WENO5, LANES - 2 for
// WENO3).  Loads along y/z are strided gathers of whole 32-40 byte cells, so
// no sector is fetched for nothing.
#pragma once

#include "kernels.cuh"

namespace pda {

// v[d] = x for a runtime d, with v kept in registers (predicated moves)
template <int N>
__device__ __forceinline__ void set_dof(double (&v)[N], int d, double x) {
#pragma unroll
  for (int k = 0; k < N; ++k)
    if (k == d) v[k] = x;
}

template <int SCHEME, int LANES_ = 64> struct TileCfg;
template <int LANES_> struct TileCfg<Weno5, LANES_> {
  static constexpr int H = 3, LANES = LANES_, TW = LANES - 3, NCELL = TW + 5, NA = 5;
};
template <int LANES_> struct TileCfg<Weno3, LANES_> {
  static constexpr int H = 2, LANES = LANES_, TW = LANES - 2, NCELL = TW + 3, NA = 2;
};

// shared memory of one tile: the cells of NR lines and their alpha terms
template <int FAM, int SCHEME, int NR, int LANES> struct FaceTileSmem {
  using C = TileCfg<SCHEME, LANES>;
  double sU[NR][Fam<FAM>::ndpc][C::NCELL + 1];
  double sA[NR][Fam<FAM>::ndpc][C::NA][LANES];
};

// One tile: lines lineGroup*NR .. +NR-1 of the box (the lines run along AXIS,
// numbered with the first other axis fastest), faces chunk*TW .. +TW-1 of
// each line.  Called by every thread of a LANES x NR block.
template <int FAM, int SCHEME, int AXIS, int NR, int LANES>
__device__ __forceinline__ void face_tile(FaceTileSmem<FAM, SCHEME, NR, LANES> &sm, const Box &b, const Phys &p,
                                          const double *__restrict__ U, double *__restrict__ Fout,
                                          long lineGroup, int chunk) {
  using F = Fam<FAM>;
  using C = TileCfg<SCHEME, LANES>;
  constexpr int NDPC = F::ndpc, TW = C::TW, NCELL = C::NCELL, H = C::H;
  constexpr int A1 = AXIS == 0 ? 1 : 0, A2 = AXIS == 2 ? 1 : 2;  // the two other axes
  auto &sU = sm.sU;
  auto &sA = sm.sA;

  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nb1 = b.hi[A1] - b.lo[A1], nb2 = b.hi[A2] - b.lo[A2];
  const int nf = b.hi[AXIS] - b.lo[AXIS] + 1;
  const long line = lineGroup * NR + ty;
  const bool lineOk = line < (long)nb1 * nb2;
  const int c1 = lineOk ? b.lo[A1] + (int)(line % nb1) : b.lo[A1];
  const int c2 = lineOk ? b.lo[A2] + (int)(line / nb1) : b.lo[A2];
  const int f0 = b.lo[AXIS] + chunk * TW;  // first face of the tile
  long stride[3];
  stride[0] = 1;
  stride[1] = b.n[0];
  stride[2] = (long)b.n[0] * b.n[1];
  const long base = (long)c1 * stride[A1] + (long)c2 * stride[A2];

  // ---- phase A: cells f0-H .. f0+TW+H-2 of this line into shared memory
  for (int k = tx; k < NCELL; k += LANES) {
    bool mir;
    const int c = map_cell(f0 - H + k, b.n[AXIS], b.mode[AXIS], mir);
    const double *src = U + (base + (long)c * stride[AXIS]) * NDPC;
#pragma unroll
    for (int d = 0; d < NDPC; ++d) {
      double v = __ldg(src + d);
      if (mir && d == b.reflect[AXIS]) v = -v;
      sU[ty][d][k] = v;
    }
  }
  __syncthreads();

  // ---- phase B: per-cell alpha terms
  constexpr double epsilon = 1e-6;
  if constexpr (SCHEME == Weno5) {
    // center c = f0 - 2 + tx uses cells c-1, c, c+1 = sU[tx .. tx+2]
    constexpr double oneOvten = 1. / 10., threeOvten = 3. / 10., sixOvten = 6. / 10.,
                     thirteenOvtwelve = 13. / 12.;
    if (tx + 2 < NCELL) {
#pragma unroll 1
      for (int d = 0; d < NDPC; ++d) {
        const double a = sU[ty][d][tx], m = sU[ty][d][tx + 1], c = sU[ty][d][tx + 2];
        const double X = w5_curv<true>(a, m, c);
        const double D = mul_c(X, thirteenOvtwelve) * X;
        const double YL = w5_slopeL<true>(a, m, c);
        const double YC = a - c;
        const double YR = w5_slopeR<true>(a, m, c);
        const double BL = D + quarter_of(YL) * YL;
        const double BC = D + quarter_of(YC) * YC;
        const double BR = D + quarter_of(YR) * YR;
        const double dL = epsilon * epsilon + mul_c(BL, 2. * epsilon) + BL * BL;
        const double dC = epsilon * epsilon + mul_c(BC, 2. * epsilon) + BC * BC;
        const double dR = epsilon * epsilon + mul_c(BR, 2. * epsilon) + BR * BR;
        const Quot2 aL = div2_rn(oneOvten, threeOvten, dL);
        const Quot2 aR = div2_rn(threeOvten, oneOvten, dR);
        sA[ty][d][0][tx] = aL.q0;                 // uNeg alpha0 of face c+1+1/2
        sA[ty][d][1][tx] = aL.q1;                 // uPos alpha0 of face c+1/2
        sA[ty][d][2][tx] = div_rn(sixOvten, dC);  // uNeg alpha1 of face c+1/2, uPos alpha1 of face c-1/2
        sA[ty][d][3][tx] = aR.q0;                 // uNeg alpha2 of face c-1/2
        sA[ty][d][4][tx] = aR.q1;                 // uPos alpha2 of face c-2+1/2
      }
    }
  } else {
    // pair k = (f0 - 2 + tx, f0 - 1 + tx) uses cells sU[tx], sU[tx+1]
    constexpr double two = 2., oneOvthree = 1. / 3., twoOvthree = 2. / 3.;
    if (tx + 1 < NCELL) {
#pragma unroll 1
      for (int d = 0; d < NDPC; ++d) {
        const double a = sU[ty][d][tx], c = sU[ty][d][tx + 1];
        const double B = (a - c) * (a - c);
        const double den = epsilon * epsilon + mul_c(B, two * epsilon) + B * B;
        sA[ty][d][0][tx] = div_rn(oneOvthree, den);
        sA[ty][d][1][tx] = div_rn(twoOvthree, den);
      }
    }
  }
  __syncthreads();

  // ---- phase C: face f = f0 + tx between cells f-1 and f
  const int f = f0 + tx;
  if (!lineOk || tx >= TW || f > b.hi[AXIS]) return;
  double uN[NDPC], uP[NDPC];
  if constexpr (SCHEME == Weno5) {
    constexpr double oneOvsix = 1. / 6.;
#pragma unroll 1
    for (int d = 0; d < NDPC; ++d) {
      // left cell i = f-1: cells i-2..i+3 = sU[tx .. tx+5]; centers i-1..i+2 = sA[.][tx .. tx+3]
      const double qim2 = sU[ty][d][tx], qim1 = sU[ty][d][tx + 1], qi = sU[ty][d][tx + 2];
      const double qip1 = sU[ty][d][tx + 3], qip2 = sU[ty][d][tx + 4], qip3 = sU[ty][d][tx + 5];
      const double p0 = mul_c(w5_pFarL<true>(qim2, qim1, qi), oneOvsix);
      const double p1 = mul_c(w5_pMidL<true>(qim1, qi, qip1), oneOvsix);
      const double p2 = mul_c(w5_pMidR<true>(qi, qip1, qip2), oneOvsix);
      const double p3 = mul_c(w5_pFarR<true>(qip1, qip2, qip3), oneOvsix);
      {
        const double a0 = sA[ty][d][0][tx], a1 = sA[ty][d][2][tx + 1], a2 = sA[ty][d][3][tx + 2];
        const double s = div_rn(1., (a0 + a1 + a2));
        set_dof(uN, d, (a0 * s) * p0 + (a1 * s) * p1 + (a2 * s) * p2);
      }
      {
        const double a0 = sA[ty][d][1][tx + 1], a1 = sA[ty][d][2][tx + 2], a2 = sA[ty][d][4][tx + 3];
        const double s = div_rn(1., (a0 + a1 + a2));
        set_dof(uP, d, (a0 * s) * p1 + (a1 * s) * p2 + (a2 * s) * p3);
      }
    }
  } else {
    // p0 = (-q_{i-1} + 3 q_i) / 2, p1 = (q_i + q_{i+1}) / 2, p2 = (3 q_{i+1} - q_{i+2}) / 2
#pragma unroll 1
    for (int d = 0; d < NDPC; ++d) {
      // left cell i = f-1: cells i-1..i+2 = sU[tx .. tx+3]; pairs i-1, i, i+1 = sA[.][tx .. tx+2]
      const double qim1 = sU[ty][d][tx], qi = sU[ty][d][tx + 1], qip1 = sU[ty][d][tx + 2],
                   qip2 = sU[ty][d][tx + 3];
      const double p0 = half_of(-qim1 + mul_k<3>(qi));
      const double p1 = half_of(qi + qip1);
      const double p2 = half_of(mul_k<3>(qip1) - qip2);
      {
        const double a0 = sA[ty][d][0][tx], a1 = sA[ty][d][1][tx + 1];
        const double s = div_rn(1., (a0 + a1));
        set_dof(uN, d, (a0 * s) * p0 + (a1 * s) * p1);
      }
      {
        const double a0 = sA[ty][d][1][tx + 1], a1 = sA[ty][d][0][tx + 2];
        const double s = div_rn(1., (a0 + a1));
        set_dof(uP, d, (a0 * s) * p1 + (a1 * s) * p2);
      }
    }
  }
  double fl[NDPC];
  F::template flux<AXIS, false, true>(fl, uN, uP, p);
  // output layout of k_struct_faces: face axis index fastest within its line
  // ordering [A2][A1][face] for AXIS=0, [k][face][i] for AXIS=1, [face][j][i] for AXIS=2
  const int fi = f - b.lo[AXIS];
  const int i1 = c1 - b.lo[A1], i2 = c2 - b.lo[A2];
  long o;
  if (AXIS == 0) o = fi + (long)nf * (i1 + (long)nb1 * i2);
  else if (AXIS == 1) o = i1 + (long)nb1 * (fi + (long)nf * i2);
  else o = i1 + (long)nb1 * (i2 + (long)nb2 * fi);
#pragma unroll
  for (int d = 0; d < NDPC; ++d) Fout[o * NDPC + d] = fl[d];
}

// Resident blocks per SM the register allocation must allow: 32 warps per SM,
// or fewer where the tile's shared memory admits fewer blocks (3D: 7), so the
// cap never forces spills that buy no occupancy.  2D Euler, 1024^2: 0.634
// against 0.638 ms per face pass at the uncapped 68 registers.
template <int FAM, int SCHEME, int NR, int LANES>
struct FaceTileMinBlocks {
  static constexpr int kSmemPerSM = 228 * 1024, kReservedPerBlock = 1024;
  static constexpr int bySmem =
      kSmemPerSM / ((int)sizeof(FaceTileSmem<FAM, SCHEME, NR, LANES>) + kReservedPerBlock);
  static constexpr int byWarps = 1024 / (LANES * NR);
  static constexpr int value = bySmem < byWarps ? (bySmem > 0 ? bySmem : 1) : byWarps;
};

// grid: x = line groups of NR lines, y = face chunks of TW faces
template <int FAM, int SCHEME, int AXIS, int NR, int LANES = 64>
__global__ void __launch_bounds__(LANES *NR, (FaceTileMinBlocks<FAM, SCHEME, NR, LANES>::value))
k_faces_tile(Box b, Phys p, const double *__restrict__ U, double *__restrict__ Fout) {
  __shared__ FaceTileSmem<FAM, SCHEME, NR, LANES> sm;
  face_tile<FAM, SCHEME, AXIS, NR, LANES>(sm, b, p, U, Fout, (long)blockIdx.x, (int)blockIdx.y);
}

}  // namespace pda
