// Host-callable launchers, one set per problem family (kernels_<family>.cu).
#pragma once

#include <cuda_runtime.h>

#include "types.hpp"

namespace pda {

struct Launchers {
  // velocity of the rows of one or two row tables (tb may be empty), one launch
  void (*rows_velocity)(int scheme, const RowTable &ta, const RowTable &tb, const MeshArgs &m, const Phys &p,
                        const double *U, double *V, cudaStream_t s);
  // structured interior: faces once per axis into F[axis], then balance into V
  // ev (may be null): dim+2 events recorded before the first face launch,
  // after each face launch and after the balance launch
  void (*struct_velocity)(int scheme, const Box &b, const MeshArgs &m, const Phys &p,
                          const double *U, double *const F[3], double *V, cudaStream_t s,
                          int *launches, cudaEvent_t *ev);
  // the pieces of struct_velocity over a sub-box (bands of the host-buffer
  // path): faces normal to `axis` into F (the face array of that box), and
  // the balance of the box's cells from F[axis] (offset to the box) into V
  void (*struct_faces)(int scheme, int axis, const Box &b, const Phys &p, const double *U, double *F,
                       cudaStream_t s);
  void (*struct_balance)(const Box &b, const MeshArgs &m, const Phys &p, const double *U,
                         const double *const F[3], double *V, cudaStream_t s);
  // V and J for inner rows / near-boundary rows
  void (*rows_vj_inner)(int scheme, const RowTable &t, const MeshArgs &m, const Phys &p,
                        const double *U, const int *rowptr, double *V, double *J, cudaStream_t s);
  void (*rows_vj_nearbd)(int scheme, const RowTable &t, const MeshArgs &m, const Phys &p,
                         const double *U, const int *rowptr, double *V, double *J, cudaStream_t s);
  // batches: faces normal to one axis of every instance with tile shape
  // `shape` (index into kTileShapes), then the balance of every instance
  void (*batch_faces)(int scheme, int axis, int shape, const BatchArgs &a, const double *U, double *F,
                      cudaStream_t s);
  void (*batch_balance)(const BatchArgs &a, const double *U, const double *F, double *V, cudaStream_t s);
  // the balance fused with an SSP-RK3 stage update (k_batch_balance_stage)
  void (*batch_balance_stage)(const BatchArgs &a, const double *Us, const double *F, double *out,
                              const double *x, int kind, double ca, double cb, double cc, cudaStream_t s);
  int (*batch_num_shapes)();  // tile shapes compiled for this family
  // V + J of the inner box with faces computed once (WENO3 / WENO5), one
  // launch per axis (jfaces.cuh)
  void (*struct_vj)(int scheme, const Box &b, const MeshArgs &m, const Phys &p, const double *U,
                    const int *rowptr, double *V, double *J, cudaStream_t s, int *launches);
  // one fused LSPG Gauss-Newton iteration over the inner rows ti and the
  // near-boundary rows tn (lspg_fused.cuh); grid = lspg_fused_blocks(...)
  void (*lspg_fused)(int scheme, const RowTable &ti, const RowTable &tn, const MeshArgs &m, const Phys &p,
                     const LspgArgs &a, cudaStream_t s);
  int (*lspg_fused_blocks)(int scheme, int innerRows, int nearRows, int K);
  // raise the fused kernels' dynamic shared-memory limit (once, before any capture)
  void (*lspg_fused_prepare)();
};

const Launchers &launchers_euler1d();
const Launchers &launchers_euler2d();
const Launchers &launchers_euler3d();
const Launchers &launchers_swe2d();

// generic device utilities (util.cu)
void launch_axpby_stage(int kind, double *out, const double *a, const double *b, const double *c,
                        double ca, double cb, double cc, double cd, const double *d, const double *e,
                        long n, cudaStream_t s);
// FP64 FMA throughput probe: returns FLOP/s measured with CUDA events
double measure_fp64_fma_rate(int blocks, int threads, int iters, cudaStream_t s);
// counts = {operand sets, division mismatches, square-root mismatches}
void check_divsqrt(int mode, uint64_t seed, long per_thread, long long counts[3], cudaStream_t s);
void check_products(int mode, uint64_t seed, long per_thread, long long counts[5], cudaStream_t s);
void launch_csr_spmm(long rows, const int *rowptr, const int *colidx, const double *vals,
                     const double *B, long ldb, int ncols, double *R, long ldr, cudaStream_t s);

// device address of the static face-flux scratch (noalloc.cu) on the
// current device, looked up once per device
cudaError_t noalloc_face_scratch(double **out);

inline int div_up(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace pda
