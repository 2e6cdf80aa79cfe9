// One Gauss-Newton iteration of hyper-reduced LSPG (BDF1 or BDF2) in one
// launch: sample-mesh velocity V, the product Jf D of the sample-mesh
// Jacobian with the trial space's latent Jacobian D formed face by face
// (never assembling Jf), the LSPG residual R = cf V + (y + cn y_n [+ cnm1
// y_n-1]) and JR = cf Jf D + D at the sample dofs, the block partial sums of
// JR^T JR, JR^T R and R^T R, and, in the last block to finish, their
// reduction, the k x k Cholesky solve and the latent update (Pressio's
// LspgUnsteadyResidualJacobianPolicyHypRed,
// lspg_unsteady_rj_policy_hypred.hpp:180-264).
//
// Jf D row by row: Jf's row is the sum over the row's faces of
// +-h^-1 (JN dU/dq + JP dU/dq) with dU/dq the reconstruction gradients, so
//   (Jf D)_row = sum_faces +-h^-1 (JN (sum_s gN_s D_s) + JP (sum_s gP_s D_s)),
// one face and one latent column per thread.  Near-boundary rows use the
// first-order Jacobian with the ghost dependence folded into the row's own
// cell by the BC factors (the assembled Jacobian's rule), i.e. D of a ghost
// is the factor times D of the cell.  Same products as forming Jf and then
// Jf D (the assembled path), in another order: equal to rounding.
//
// Blocks [0, nbInner) take inner rows, the others near-boundary rows; each
// block takes RPB rows through the phases of k_rows_vj_inner_par /
// k_rows_vj_nearbd_par (GB300's narrow FP64 units make the per-thread
// instruction chain the cost, so the work of a row is spread over threads).
#pragma once

#include "kernels.cuh"

namespace pda {

constexpr int kLspgKMax = 32;

// Rows per block are chosen at launch (rpb <= RPB_MAX) so that the grid
// covers the SMs once where the row count allows (a second block on one SM
// doubles that SM's chain) and the dynamic shared memory fits.
template <int FAM> struct FusedPar {
  static constexpr int NF = 2 * Fam<FAM>::dim, NDPC = Fam<FAM>::ndpc, DIM = Fam<FAM>::dim;
  static constexpr int RPB_MAX = Fam<FAM>::dim == 3 ? 4 : 8;
  static constexpr int SIDE = pad_warp(RPB_MAX * NF * NDPC);
  static constexpr int PART = pad_warp(RPB_MAX * NF);
  static constexpr int THREADS = 2 * SIDE;
  static_assert(4 * PART <= THREADS, "phase B fits the block");
  static_assert(RPB_MAX * NF <= PART && RPB_MAX <= PART, "a warp covers the block's faces and rows");
  static constexpr size_t kSmemLimit = 160 * 1024;  // dynamic shared memory per block
  // dynamic shared memory per row: staged D of the row's stencil cells, the
  // per-face J D columns and the row's JR rows
  static size_t smem_row(int S, int K) {
    return sizeof(double) * ((size_t)DIM * S * NDPC * K + (size_t)NF * NDPC * K + (size_t)NDPC * (K + 1));
  }
};

// Blocks are reduced in groups of kLspgGroup: the last block of a group to
// finish sums the group's partial sums in block order, the last group to
// finish sums the group sums in group order and solves.  Both levels run one
// thread per entry with independent loads, since a chain of dependent FP64
// adds costs ~70 cycles a step on GB300.

// sum of rows [r0, r1) of a [rows][ne] array, entry by entry, in row order
__device__ inline double lspg_sum_rows(const double *__restrict__ a, int ne, int e, int r0, int r1) {
  double s = 0.;
  int r = r0;
  for (; r + 4 <= r1; r += 4) {
    const double v0 = a[(long)r * ne + e], v1 = a[(long)(r + 1) * ne + e], v2 = a[(long)(r + 2) * ne + e],
                 v3 = a[(long)(r + 3) * ne + e];
    s += v0;
    s += v1;
    s += v2;
    s += v3;
  }
  for (; r < r1; ++r) s += a[(long)r * ne + e];
  return s;
}

// reduce the group sums in group order, factor, solve, update (the calling
// block; warp 0 factors): right-looking Cholesky with reciprocal square
// roots of the matrix [H g; g^T .] augmented by the right-hand side, so that
// its last row becomes z = L^-1 g in the trailing updates (no separate
// forward substitution), then a lane-parallel back substitution
__device__ inline void lspg_solve_rt(int K, int nparts, const double *__restrict__ partial, double *__restrict__ x,
                                     double tol, int first, LspgFlags *f) {
  constexpr int KA = kLspgKMax + 1;  // augmented order
  __shared__ double H[KA][KA];
  __shared__ double rdiag[kLspgKMax];
  __shared__ double rr;
  __shared__ unsigned char pi[KA * (KA + 1) / 2], pl[KA * (KA + 1) / 2];
  const int ntri = K * (K + 1) / 2, ne = ntri + K + 1, Ka = K + 1;
  const int lane = threadIdx.x & 31;
  // lower-triangle pairs (i, l), i >= l, of the augmented order, by l
  // descending: the pairs with l > j are the first (Ka-1-j)(Ka-j)/2 entries
  const int ntriA = Ka * (Ka + 1) / 2;
  for (int q = threadIdx.x; q < ntriA; q += blockDim.x) {
    int l = Ka - 1, rem = q;
    while (rem >= Ka - l) {
      rem -= Ka - l;
      --l;
    }
    pi[q] = (unsigned char)(l + rem);
    pl[q] = (unsigned char)l;
  }
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    const double s = lspg_sum_rows(partial, ne, e, 0, nparts);
    if (e < ntri) {
      int a = 0, rem = e;
      while (rem >= K - a) {
        rem -= K - a;
        ++a;
      }
      const int b2 = a + rem;
      H[a][b2] = s;
      H[b2][a] = s;
    } else if (e < ntri + K) {
      H[K][e - ntri] = s;  // the right-hand side as the augmented row
    } else {
      rr = s;
    }
  }
  __syncthreads();
  if (threadIdx.x >= 32) return;
  bool ok = true;
  for (int j = 0; j < K; ++j) {
    const double d = H[j][j];
    // positive and finite, tested on the bits (no FP64 instruction)
    const long long db = __double_as_longlong(d);
    if (!(db > 0 && db < 0x7FF0000000000000LL)) {
      ok = false;
      break;
    }
    const double rs = rsqrt(d);
    if (lane == 0) rdiag[j] = rs;
    for (int i = j + 1 + lane; i <= K; i += 32) H[i][j] *= rs;
    __syncwarp();
    // trailing lower triangle (the augmented row included), its pairs spread over the lanes
    const int np = (Ka - 1 - j) * (Ka - j) / 2;
    for (int q = lane; q < np; q += 32) {
      const int row = pi[q], col = pl[q];
      H[row][col] = fma(-H[row][j], H[col][j], H[row][col]);
    }
    __syncwarp();
  }
  double sv = lane < K ? H[K][lane] : 0.;  // z = L^-1 g
  double corr = 0.;
  if (ok) {
    for (int i = K - 1; i >= 0; --i) {
      const double di = __shfl_sync(0xffffffffu, sv, i) * rdiag[i];
      if (lane == i) sv = di;
      if (lane < i) sv = fma(-H[i][lane], di, sv);
    }
    if (lane < K) x[lane] -= sv;
    double c2 = lane < K ? sv * sv : 0.;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c2 += __shfl_xor_sync(0xffffffffu, c2, o);
    corr = c2;
  }
  if (lane == 0) {
    // the first iteration of a step starts the step's count and flag
    f->iters = first ? 1 : f->iters + 1;
    f->lastCorr = sqrt(corr);
    f->lastRes = sqrt(rr);
    if (!(f->lastRes <= f->maxRes)) f->maxRes = f->lastRes;
    f->converged = (!ok || sqrt(corr) < tol) ? 1 : 0;
  }
}

// one face of a block's rows: the flux and face values in double, the
// Jacobian terms in JT (double, or float for the inexact Gauss-Newton step)
template <int FAM, int SCHEME, typename JT> struct FusedFace {
  static constexpr int NDPC = Fam<FAM>::ndpc, G = 2 * SchemeTraits<SCHEME>::h;
  double fl[NDPC];
  double uN[NDPC], uP[NDPC];
  JT JN[NDPC * NDPC], JP[NDPC * NDPC];
  JT gN[NDPC][G], gP[NDPC][G];
};

// 16-byte global -> shared copy that does not hold up the issuing warp
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// JT: the scalar type of the Jacobian terms (double: the exact Jacobian of
// the sample-mesh residual; float: an approximate one, on GB300's far wider
// FP32 units, for an inexact Gauss-Newton step on the same double residual)
template <int FAM, int SCHEME, typename JT>
__global__ void __launch_bounds__(FusedPar<FAM>::THREADS)
k_lspg_fused(RowTable ti, RowTable tn, int rpb, int nbInner, MeshArgs m, Phys p, LspgArgs a) {
  if (!a.first && a.f->converged) return;
  using F = Fam<FAM>;
  using FP = FusedPar<FAM>;
  using FF = FusedFace<FAM, SCHEME, JT>;
  constexpr bool kExact = sizeof(JT) == sizeof(double);
  constexpr int NDPC = F::ndpc, DIM = F::dim, H = SchemeTraits<SCHEME>::h, S = 2 * H + 1, G = 2 * H;
  constexpr int NF = FP::NF;
  __shared__ FF fd[FP::RPB_MAX][NF];
  __shared__ double sY[FP::RPB_MAX][NDPC];    // state at the row's cell
  __shared__ double sSrc[FP::RPB_MAX][NDPC];  // source-term velocity (shallow water: Coriolis)
  __shared__ double sSJ[FP::RPB_MAX][NDPC * NDPC];  // its Jacobian
  __shared__ typename F::Side sSide[FP::RPB_MAX][NF][2];  // the two face states' halves of the flux
  extern __shared__ double dyn[];
  const int tid = threadIdx.x, K = a.K, RD = rpb * NDPC, CB = NDPC * K;  // CB: D doubles per cell
  double *sD = dyn;                                  // [rpb][DIM][S][NDPC][K] staged D of stencil cells
  double *ctb = sD + (size_t)rpb * DIM * S * CB;     // [rpb][NF][NDPC][K]
  double *sJR = ctb + (size_t)rpb * NF * NDPC * K;   // [RD][K + 1]
  const bool inner = (int)blockIdx.x < nbInner;
  const RowTable &t = inner ? ti : tn;
  const int e0 = (inner ? (int)blockIdx.x : (int)blockIdx.x - nbInner) * rpb;
  // D of the stencil cells (inner rows: the scheme's stencil; near rows: the
  // first-order cells) staged by asynchronous copies that overlap phase A
  {
    const int npos = inner ? S : 3, chunks = CB / 2;
    const int total = rpb * DIM * npos * chunks;
    for (int w = tid; w < total; w += blockDim.x) {
      const int ch = w % chunks, ps = (w / chunks) % npos, ax = (w / (chunks * npos)) % DIM,
                rl = w / (chunks * npos * DIM);
      const int e = e0 + rl;
      if (e >= t.nrows) continue;
      const int cell = inner ? t.src[((size_t)e * DIM + ax) * S + ps] : t.src1[((size_t)e * DIM + ax) * 3 + ps];
      cp_async16(sD + (((size_t)rl * DIM + ax) * S + ps) * CB + 2 * ch, a.D + (size_t)cell * CB + 2 * ch);
    }
  }
  {  // phase A: (side, row, face, dof): one side of the face value (+ gradient for inner rows)
    const int side = tid / FP::SIDE, slot = tid % FP::SIDE;
    const int rl = slot / (NF * NDPC), f = (slot / NDPC) % NF, d = slot % NDPC, ax = f >> 1, fs = f & 1;
    const int e = e0 + rl;
    if (slot < rpb * NF * NDPC && e < t.nrows) {
      const size_t base = ((size_t)e * DIM + ax) * S;
      double q[G];
      FF &o = fd[rl][f];
      if (inner) {
#pragma unroll
        for (int s = 0; s < G; ++s) q[s] = __ldg(a.y + (size_t)t.src[base + fs + s] * NDPC + d);
        JT u, gg[G];
        if constexpr (kExact) {
          face_grad_side<SCHEME>(side, u, gg, q);
        } else {
          // the value in double (it enters V and R); the gradient in float
          JT qf[G];
#pragma unroll
          for (int s = 0; s < G; ++s) qf[s] = (JT)q[s];
          face_grad_side<SCHEME>(side, u, gg, qf);
        }
        JT *gs = side == 0 ? o.gN[d] : o.gP[d];
        (side == 0 ? o.uN : o.uP)[d] = kExact ? (double)u : face_value_side<SCHEME>(side, q);
#pragma unroll
        for (int s = 0; s < G; ++s) gs[s] = gg[s];
      } else {
#pragma unroll
        for (int s = 0; s < G; ++s) {
          double qe[NDPC];
          load_entry<NDPC>(qe, a.y, t.src[base + fs + s], t.flip[base + fs + s], m.reflect[ax], m, t.gsx, t.gsy,
                           base + fs + s);
          q[s] = qe[d];
        }
        (side == 0 ? o.uN : o.uP)[d] = face_value_side<SCHEME>(side, q);
      }
    }
  }
  cp_async_wait_all();
  __syncthreads();
  // GB300 issues one FP64 warp instruction per ~64 cycles per sub-partition
  // whatever the number of active lanes, so a stage costs its longest
  // per-warp FP64 instruction stream.  With single-precision Jacobian terms
  // phase B runs in two stages so that no warp evaluates a whole flux: B1 the
  // two face states' halves of the flux (warps 0 / 1) beside JN / JP (warps
  // 2 / 3), B2 their combination (warp 0) beside the row's source term (warp
  // 1).  With double-precision Jacobian terms the flux Jacobians are the
  // longest streams, so one stage: warp 0 the whole flux, warp 1 the source.
  auto row_state_and_source = [&](int rl) {
    const int e = e0 + rl;
    if (rl >= rpb || e >= t.nrows) return;
    const int cell = t.cell[e];
    double y[NDPC];
#pragma unroll
    for (int d = 0; d < NDPC; ++d) y[d] = __ldg(a.y + (size_t)cell * NDPC + d);
#pragma unroll
    for (int d = 0; d < NDPC; ++d) {
      sY[rl][d] = y[d];
      sSrc[rl][d] = 0.;
    }
#pragma unroll
    for (int i = 0; i < NDPC * NDPC; ++i) sSJ[rl][i] = 0.;
    if constexpr (FAM == Swe2d) {
      // Coriolis source (swe_2d_prob_class.hpp:983-1012) and its Jacobian
      const double u0 = y[0], u1 = y[1], u2 = y[2];
      // (divisions on the integer pipe, the IEEE quotients)
      sSrc[rl][1] = -div_rn(p.coriolis * u2, u0);
      sSrc[rl][2] = div_rn(p.coriolis * u1, u0);
      sSJ[rl][1 * 3 + 0] = div_rn(p.coriolis * u2, (u0 * u0));
      sSJ[rl][1 * 3 + 2] = div_rn(-p.coriolis, u0);
      sSJ[rl][2 * 3 + 1] = div_rn(p.coriolis, u0);
      sSJ[rl][2 * 3 + 0] = div_rn(-p.coriolis * u1, (u0 * u0));
    }
  };
  auto combine = [&](int rl, int f) {
    FF &o = fd[rl][f];
    const typename F::Side &L = sSide[rl][f][0], &R = sSide[rl][f][1];
    F::template flux_combine<0>(o.fl, o.uN, o.uP, L, R, p);  // the combination does not depend on the axis
  };
  {  // phase B1: (part, row, face): parts 0 / 1 the left / right face state's
     // half of the flux (exact Jacobian: part 0 both halves and the flux,
     // part 1 the rows' sources), parts 2 / 3 JN / JP
    const int part = tid / FP::PART, slot = tid % FP::PART;
    const int rl = slot / NF, f = slot % NF, ax = f >> 1, fs = f & 1;
    const int e = e0 + rl;
    if (kExact && part == 1) {
      row_state_and_source(slot);
    } else if (part < 4 && slot < rpb * NF && e < t.nrows) {
      FF &o = fd[rl][f];
      if (part < 2) {
#pragma unroll
        for (int sd = 0; sd < (kExact ? 2 : 1); ++sd) {
          const int side = kExact ? sd : part;
          const double *q = side == 0 ? o.uN : o.uP;
          typename F::Side &so = sSide[rl][f][side];
          F::flux_side_ax(so, q, p, ax);  // one stream for all axes of the warp
        }
        if (kExact) combine(rl, f);
      } else {
        double uN[NDPC], uP[NDPC];
#pragma unroll
        for (int d = 0; d < NDPC; ++d) {
          uN[d] = o.uN[d];
          uP[d] = o.uP[d];
        }
        if (!inner) {
          // first-order Jacobian at the face's two cells (ghosts through their recipes)
          const size_t b1 = ((size_t)e * DIM + ax) * 3;
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            double qe[NDPC];
            load_entry<NDPC>(qe, a.y, t.src1[b1 + fs + s], t.flip1[b1 + fs + s], m.reflect[ax], m, t.gsx1,
                             t.gsy1, b1 + fs + s);
#pragma unroll
            for (int d = 0; d < NDPC; ++d) (s == 0 ? uN : uP)[d] = qe[d];
          }
        }
        JT JN[NDPC * NDPC], JP[NDPC * NDPC], vN[NDPC], vP[NDPC];
#pragma unroll
        for (int d = 0; d < NDPC; ++d) {
          vN[d] = (JT)uN[d];
          vP[d] = (JT)uP[d];
        }
        F::flux_jac_ax(JN, JP, vN, vP, p, ax);  // one stream for all axes of the warp
        // one of the two per warp (the part is warp-uniform): the other's
        // arithmetic is dead and dropped
        if (part == 2) {
#pragma unroll
          for (int i = 0; i < NDPC * NDPC; ++i) o.JN[i] = JN[i];
        } else {
#pragma unroll
          for (int i = 0; i < NDPC * NDPC; ++i) o.JP[i] = JP[i];
        }
      }
    }
  }
  __syncthreads();
  if constexpr (!kExact) {  // phase B2: warp 0 (row, face) the flux from its two halves; warp 1
                            // (row) the row's state and its source term with its Jacobian
    if (tid < FP::PART) {
      const int rl = tid / NF, f = tid % NF;
      if (tid < rpb * NF && e0 + rl < t.nrows) combine(rl, f);
    } else if (tid < 2 * FP::PART) {
      row_state_and_source(tid - FP::PART);
    }
    __syncthreads();
  }
  // phase C: (row, face, column c): the face's (JN dU_N + JP dU_P) D column
  for (int w = tid; w < rpb * NF * K; w += blockDim.x) {
    const int rl = w / (NF * K), f = (w / K) % NF, c = w % K, ax = f >> 1, fs = f & 1;
    const int e = e0 + rl;
    if (e >= t.nrows) continue;
    const FF &o = fd[rl][f];
    const double *Dax = sD + ((size_t)rl * DIM + ax) * S * CB;  // staged D of this axis' positions
    JT dN[NDPC], dP[NDPC];
    if (inner) {
#pragma unroll
      for (int d = 0; d < NDPC; ++d) {
        dN[d] = JT(0);
        dP[d] = JT(0);
      }
#pragma unroll
      for (int s = 0; s < G; ++s) {
        const double *Ds = Dax + (size_t)(fs + s) * CB;
#pragma unroll
        for (int d = 0; d < NDPC; ++d) {
          const JT dv = (JT)Ds[d * K + c];
          dN[d] = fma(o.gN[d][s], dv, dN[d]);
          dP[d] = fma(o.gP[d][s], dv, dP[d]);
        }
      }
    } else {
      const size_t b1 = ((size_t)e * DIM + ax) * 3;
      const double *fac = t.jfac + ((size_t)e * DIM + ax) * NDPC;
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const int pos = fs + s;
        const bool ghost = t.jpos1[b1 + pos] < 0;
        const double *Ds = Dax + (size_t)(ghost ? 1 : pos) * CB;  // position 1 is the row's cell
#pragma unroll
        for (int d = 0; d < NDPC; ++d) {
          const double dv = Ds[d * K + c];
          (s == 0 ? dN : dP)[d] = (JT)(ghost ? fac[d] * dv : dv);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < NDPC; ++k) {
      JT acc = JT(0);
#pragma unroll
      for (int d = 0; d < NDPC; ++d) {
        acc = fma(o.JN[k * NDPC + d], dN[d], acc);
        acc = fma(o.JP[k * NDPC + d], dP[d], acc);
      }
      ctb[(((size_t)rl * NF + f) * NDPC + k) * K + c] = (double)acc;
    }
  }
  __syncthreads();
  // phase D: (row, k, column c <= K): JR = cf Jf D + D and, in column K, R
  for (int w = tid; w < RD * (K + 1); w += blockDim.x) {
    const int rk = w / (K + 1), c = w % (K + 1), rl = rk / NDPC, k = rk % NDPC;
    const int e = e0 + rl;
    double val = 0.;
    if (e < t.nrows) {
      const double *Dself = sD + ((size_t)rl * DIM * S + (inner ? H : 1)) * CB;  // axis 0, the row's cell
      if (c < K) {
        double jd = 0.;
#pragma unroll
        for (int ax = 0; ax < DIM; ++ax)
          jd = fma(m.hinv[ax],
                   ctb[(((size_t)rl * NF + 2 * ax) * NDPC + k) * K + c] -
                       ctb[(((size_t)rl * NF + 2 * ax + 1) * NDPC + k) * K + c],
                   jd);
        if constexpr (FAM == Swe2d) {
#pragma unroll
          for (int j = 0; j < NDPC; ++j) jd = fma(sSJ[rl][k * NDPC + j], Dself[j * K + c], jd);
        }
        val = fma(a.cf, jd, Dself[k * K + c]);
      } else {
        double vk = 0.;
#pragma unroll
        for (int ax = 0; ax < DIM; ++ax) vk += m.hinv[ax] * (fd[rl][2 * ax].fl[k] - fd[rl][2 * ax + 1].fl[k]);
        if constexpr (FAM == Swe2d) vk += sSrc[rl][k];
        const int r = t.rows[e];
        a.V[(size_t)r * NDPC + k] = vk;
        const double ynp1 = sY[rl][k];
        const size_t q = (size_t)r * NDPC + k;
        if (a.first) {
          a.ynm1[q] = a.yn[q];
          a.yn[q] = ynp1;
        }
        // Pressio's ops::update(helper, 0, y_n+1, 1, y_n, cn[, y_n-1, cnm1])
        const double helper = a.bdf2 ? 1. * ynp1 + a.cn * a.yn[q] + a.cnm1 * a.ynm1[q] : 1. * ynp1 + a.cn * a.yn[q];
        val = a.cf * vk + 1. * helper;
      }
    }
    sJR[(size_t)rk * (K + 1) + c] = val;
  }
  __syncthreads();
  // phase E: block partial sums of the upper triangle of JR^T JR, of JR^T R, R^T R
  const int ntri = K * (K + 1) / 2, ne = ntri + K + 1;
  for (int q = tid; q < ne; q += blockDim.x) {
    int ia, ib;
    if (q < ntri) {
      ia = 0;
      int rem = q;
      while (rem >= K - ia) {
        rem -= K - ia;
        ++ia;
      }
      ib = ia + rem;
    } else if (q < ntri + K) {
      ia = q - ntri;
      ib = K;
    } else {
      ia = K;
      ib = K;
    }
    double s = 0.;
    for (int i = 0; i < RD; ++i) s = fma(sJR[(size_t)i * (K + 1) + ia], sJR[(size_t)i * (K + 1) + ib], s);
    a.partial[(long)blockIdx.x * ne + q] = s;
  }
  // the last block of a group reduces the group; the last group solves (no
  // block waits for another).  ticket[0] counts groups, ticket[1 + g] blocks.
  __shared__ unsigned last;
  const int nb = (int)gridDim.x, ng = lspg_groups(nb), grp = (int)blockIdx.x / kLspgGroup;
  const int g0 = grp * kLspgGroup, g1 = min(nb, g0 + kLspgGroup);
  double *gsum = a.partial + (long)nb * ne;  // [groups][ne] after the block sums
  __threadfence();
  __syncthreads();
  if (tid == 0) last = atomicAdd(a.ticket + 1 + grp, 1u) == (unsigned)(g1 - g0 - 1) ? 1u : 0u;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int q = tid; q < ne; q += blockDim.x) gsum[(long)grp * ne + q] = lspg_sum_rows(a.partial, ne, q, g0, g1);
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    a.ticket[1 + grp] = 0u;
    last = atomicAdd(a.ticket, 1u) == (unsigned)(ng - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  lspg_solve_rt(K, ng, gsum, a.x, a.tol, a.first, a.f);
  if (tid == 0) *a.ticket = 0u;
}

}  // namespace pda
