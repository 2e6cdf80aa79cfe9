/*
 * pda_gb300.h -- C ABI of the GB300-native finite-volume residual/Jacobian
 * engine (drop-in for pressio-demoapps' cell-centered Euler/shallow-water
 * problems).
 *
 * Conventions
 *   - Every function returns PDA_OK (0) or a negative pda_status; the message
 *     of the last failure on the calling thread is pda_last_error().
 *     No C++ exception crosses this boundary and nothing calls exit().
 *   - Pointers named d_* are device (GB300 HBM) pointers; h_* are host.
 *   - State U and residual V are array-of-structures doubles:
 *       U[cell * ndpc + dof]   cell = stencil-mesh id   (totalDofStencilMesh)
 *       V[row  * ndpc + dof]   row  = sample-mesh row   (totalDofSampleMesh)
 *     exactly as the reference's Eigen vectors.
 *   - The Jacobian is CSR (int32 row pointers and column indices, double
 *     values) with the same row/column order and sparsity as the reference's
 *     Eigen::SparseMatrix<double, RowMajor, int32>; the pattern is built once
 *     and the evaluation calls overwrite the values in place.
 *   - A problem object is bound to one CUDA stream; calls on it are
 *     asynchronous with respect to the host (except *_host variants) and it
 *     is not safe to call one object from two threads at once (as the
 *     reference, whose const methods mutate internal buffers).
 *   - The mesh must outlive every problem created from it (as the reference,
 *     which keeps a reference to the mesh).
 *
 * Reference interfaces replaced (pressio-demoapps v0.16.0, paths relative to
 * include/pressiodemoapps/):
 */
#ifndef PDA_GB300_H_
#define PDA_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int pda_status;
#define PDA_OK 0
#define PDA_ERR_INVALID_ARGUMENT -1
#define PDA_ERR_IO -2
#define PDA_ERR_CUDA -3
#define PDA_ERR_UNSUPPORTED -4
#define PDA_ERR_OUT_OF_MEMORY -5
#define PDA_ERR_INTERNAL -6

/* problem families (euler1d.hpp:64, euler2d.hpp:67, euler3d.hpp:64, swe2d.hpp:66) */
#define PDA_EULER1D 0
#define PDA_EULER2D 1
#define PDA_EULER3D 2
#define PDA_SWE2D 3

/* InviscidFluxReconstruction (schemes_info.hpp:61-63) */
#define PDA_FIRST_ORDER 0
#define PDA_WENO3 1
#define PDA_WENO5 2

/* problem enums, same integer values as the reference enums */
#define PDA_EULER1D_PERIODIC_SMOOTH 0 /* Euler1d::PeriodicSmooth */
#define PDA_EULER1D_SOD 1             /* Euler1d::Sod */
#define PDA_EULER1D_LAX 2             /* Euler1d::Lax */
#define PDA_EULER1D_SHU_OSHER 3       /* Euler1d::ShuOsher */
#define PDA_EULER2D_PERIODIC_SMOOTH 0 /* Euler2d::PeriodicSmooth */
#define PDA_EULER2D_KELVIN_HELMHOLTZ 1 /* Euler2d::KelvinHelmholtz */
#define PDA_EULER2D_SEDOV_FULL 2      /* Euler2d::SedovFull */
#define PDA_EULER2D_SEDOV_SYMMETRY 3  /* Euler2d::SedovSymmetry */
#define PDA_EULER2D_RIEMANN 4         /* Euler2d::Riemann */
#define PDA_EULER2D_NORMAL_SHOCK 5    /* Euler2d::NormalShock */
#define PDA_EULER2D_DOUBLE_MACH_REFLECTION 6 /* Euler2d::DoubleMachReflection */
#define PDA_EULER2D_CROSS_SHOCK 7     /* Euler2d::CrossShock */
#define PDA_EULER2D_TESTING_NEUMANN 8 /* Euler2d::testingonlyneumann */
#define PDA_EULER3D_PERIODIC_SMOOTH 0 /* Euler3d::PeriodicSmooth */
#define PDA_EULER3D_SEDOV_SYMMETRY 1  /* Euler3d::SedovSymmetry (FirstOrder, WENO3) */
#define PDA_SWE2D_SLIP_WALL 0         /* Swe2d::SlipWall */

typedef struct pda_mesh pda_mesh;
typedef struct pda_problem pda_problem;

/* Message of the last failed call on this thread ("" if none). */
const char *pda_last_error(void);

/* Library version string. */
const char *pda_version(void);

/* ---------------------------------------------------------------- meshes */

/* Replaces load_cellcentered_uniform_mesh_eigen(dir) (mesh.hpp:87-91,
 * impl/mesh_ccu.hpp:359-448, impl/mesh_read_{info,connectivity,coords}.hpp).
 * Reads info.dat, connectivity.dat and coordinates.dat.  Missing files are
 * PDA_ERR_IO (the reference calls exit(EXIT_FAILURE)). */
pda_status pda_mesh_load(const char *dir, pda_mesh **out);

/* Native in-memory equivalent of meshing_scripts/create_full_mesh.py
 * (natural row ordering; create_full_mesh.py:32-218 with
 * _impl/{one_dim_mesh,natural_order_mesh_2d,natural_order_mesh_3d}.py).
 * n[3] cells per axis (1 for absent axes, dim = number of n > 1 axes as the
 * script decides), bounds[6] = {xL,xR,yL,yR,zL,zR}, stencil in {3,5,7},
 * periodic[3] flags.  The result equals loading the files the script would
 * write (coordinates and dx pass through the same %.14f text rounding).
 * Extension: 3D meshes with stencil 7 (absent in the reference). */
pda_status pda_mesh_create_full(const int n[3], const double bounds[6], int stencil,
                                const int periodic[3], pda_mesh **out);

/* Equivalent of meshing_scripts/create_sample_mesh.py (lines 28-213): sample
 * mesh of the given full-mesh cell ids plus all their stencil neighbours,
 * renumbered in sorted full-mesh order.  stencil_gids_out (may be NULL)
 * receives the full-mesh id of every stencil-mesh cell (the
 * stencil_mesh_gids.dat file), sized pda_mesh_sizes()'s stencil size. */
pda_status pda_mesh_create_sample(const pda_mesh *full, const int64_t *sample_gids, int64_t n,
                                  pda_mesh **out, int64_t *stencil_gids_out);

/* Write info.dat / connectivity.dat / coordinates.dat in the reference's
 * text format (create_full_mesh.py:150-218). */
pda_status pda_mesh_write(const pda_mesh *m, const char *dir);

/* A binary mesh file (no counterpart in the reference, whose meshes are the
 * three text files above): one little-endian file holding the info.dat
 * entries, the structured-mesh descriptor, the graph (int32) and the
 * coordinates (double), with a 64-bit checksum.  Loading it reads the arrays
 * in a few large reads instead of parsing text (seconds instead of minutes
 * at 256^3); the loaded mesh equals the one written, bit for bit.  A file
 * that is truncated, corrupt, of another version or byte order is
 * PDA_ERR_IO. */
pda_status pda_mesh_write_binary(const pda_mesh *m, const char *path);
pda_status pda_mesh_load_binary(const char *path, pda_mesh **out);

/* dims[0]=dimensionality, dims[1]=stencilSize, dims[2]=graph columns,
 * sizes[0]=stencilMeshSize, sizes[1]=sampleMeshSize, sizes[2]=#inner rows,
 * sizes[3]=#near-boundary rows; dx[3], dxInv[3]; flags[0]=isFullyPeriodic,
 * flags[1]=structured natural-order full mesh (mesh_ccu.hpp:115-159). */
pda_status pda_mesh_info(const pda_mesh *m, int dims[3], int64_t sizes[4], double dx[3],
                         double dxinv[3], int flags[2]);

/* Copies of graph() (row-major int32), viewX/Y/Z(), graphRowsOfCellsAwayFromBd(),
 * graphRowsOfCellsNearBd().  Any pointer may be NULL. */
pda_status pda_mesh_arrays(const pda_mesh *m, int32_t *graph, double *x, double *y, double *z,
                           int32_t *inner_rows, int32_t *near_bd_rows);

void pda_mesh_free(pda_mesh *m);

/* -------------------------------------------------------------- problems */

/* Replaces create_problem_eigen(mesh, family enum, scheme [, icFlag [, params]])
 * (euler1d.hpp:82-99, euler2d.hpp:88-173, euler3d.hpp:80-122,
 * swe2d.hpp:143-195) and the PublicProblemEigenMixinCpp constructor
 * (adapter_cpp.hpp:80-88).  ic_flag <= 0 selects the reference default (1).
 * Parameters are (name, value) pairs with the reference's names
 * (impl/euler_2d_parametrization_helpers.hpp:104-109,
 * impl/swe_2d_parametrization_helpers.hpp:97-102); an unknown name is
 * PDA_ERR_INVALID_ARGUMENT as in the reference.  stream is a cudaStream_t
 * (NULL = legacy default stream).  Device memory for internal tables is
 * allocated here and in pda_jacobian_pattern. */
pda_status pda_problem_create(const pda_mesh *mesh, int family, int problem, int scheme,
                              int ic_flag, const char *const *param_names,
                              const double *param_values, int n_params, void *stream,
                              pda_problem **out);

/* Equivalent of createSlipWall SWE factory create_slip_wall_swe_2d_problem_eigen
 * (swe2d.hpp:278-308): gravity, coriolis, pulse magnitude. */
pda_status pda_problem_create_swe_slip_wall(const pda_mesh *mesh, int scheme, double gravity,
                                            double coriolis, double pulse_magnitude,
                                            void *stream, pda_problem **out);

/* Equivalent of create_cross_shock_problem_eigen(mesh, rec, density,
 * inletXVel, bottomYVel) (euler2d.hpp:258-285): Euler2d::CrossShock with the
 * inflow density, inlet x velocity and bottom-inflow y velocity.  The generic
 * pda_problem_create with PDA_EULER2D_CROSS_SHOCK and no parameters uses the
 * reference's default values (0.1, 10, 1). */
pda_status pda_problem_create_cross_shock(const pda_mesh *mesh, int scheme, double density,
                                          double inlet_x_vel, double bottom_y_vel, void *stream,
                                          pda_problem **out);

void pda_problem_free(pda_problem *p);

/* numDofPerCell(), totalDofSampleMesh(), totalDofStencilMesh()
 * (adapter_cpp.hpp:93-103). */
pda_status pda_problem_sizes(const pda_problem *p, int *ndpc, int64_t *dofs_sample,
                             int64_t *dofs_stencil);

/* queryParameter(name) (euler_2d_prob_class.hpp:188-195, swe_2d_prob_class.hpp:169-179),
 * also gamma(), gravity(), coriolis(). */
pda_status pda_query_parameter(const pda_problem *p, const char *name, double *value);

/* initialCondition() (euler_2d_prob_class.hpp:184-186): computed on the
 * host with the reference's formulas, written to a device / host buffer of
 * totalDofStencilMesh doubles. */
pda_status pda_initial_condition(pda_problem *p, double *d_U);
pda_status pda_initial_condition_host(const pda_problem *p, double *h_U);

/* rightHandSide / operator() / rhs / velocity (adapter_cpp.hpp:162-199,
 * adapter_py.hpp:153-158): V = f(U, t). */
pda_status pda_velocity(pda_problem *p, const double *d_U, double t, double *d_V);

/* The same call with host buffers: copies U in, evaluates, copies V out
 * (synchronous).  This is what a caller holding Eigen/numpy vectors uses. */
pda_status pda_velocity_host(pda_problem *p, const double *h_U, double t, double *h_V);

/* Allocation-free variant of pda_velocity (no counterpart in the reference).
 * For callers that may not allocate device memory while evaluating the
 * right-hand side: fixed-budget real-time loops whose memory is set aside at
 * start-up, hosts whose pool allocator forbids library allocations.
 * pda_velocity allocates its face-flux buffers on a problem's first call;
 * this entry point puts them in one static device array of
 * PDA_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB) inside the library instead
 * and calls no allocator.  Same kernels, same results as pda_velocity.
 *  - Covers full meshes on the structured face pass (natural-order full
 *    meshes); sample meshes return PDA_ERR_UNSUPPORTED.  A mesh whose face
 *    scratch exceeds the limit returns PDA_ERR_INVALID_ARGUMENT with the
 *    required size in pda_last_error().
 *  - Problems with near-boundary rows (non-mirror boundary conditions) need
 *    their row table on the device: one pda_velocity call uploads it, until
 *    then PDA_ERR_UNSUPPORTED.
 *  - The first call on each device looks up the array's device address
 *    (this may load the module that holds it); make that first call before
 *    any stream capture or allocation-free section begins.  The address is
 *    kept per device for the process; like every problem handle it does not
 *    survive cudaDeviceReset.
 *  - Nothing in the array needs to start at zero.  The array is shared by all
 *    problems of the process on a device: calls that overlap in time (other
 *    streams or threads without ordering between them) race on it. */
#define PDA_NOALLOC_SCRATCH_DOUBLES (4u * 1024u * 1024u)
pda_status pda_velocity_noalloc(pda_problem *p, const double *d_U, double t, double *d_V);

/* createJacobian() (adapter_cpp.hpp:121-124; pattern from initializeJacobian,
 * euler_2d_prob_class.hpp:223-237, :314-387): number of rows
 * (totalDofSampleMesh), columns (totalDofStencilMesh) and stored entries. */
pda_status pda_jacobian_shape(pda_problem *p, int64_t *rows, int64_t *cols, int64_t *nnz);

/* Copy the CSR pattern (row pointers rows+1, column indices nnz) into device
 * buffers / host buffers. */
pda_status pda_jacobian_pattern(pda_problem *p, int32_t *d_rowptr, int32_t *d_colidx);
pda_status pda_jacobian_pattern_host(pda_problem *p, int32_t *h_rowptr, int32_t *h_colidx);

/* rightHandSideAndJacobian / rhsAndJacobian / operator()(U,t,V,J,true)
 * (adapter_cpp.hpp:201-221): V and the CSR values (nnz doubles, in the
 * pattern's order) are overwritten. */
pda_status pda_velocity_and_jacobian(pda_problem *p, const double *d_U, double t, double *d_V,
                                     double *d_J);
pda_status pda_velocity_and_jacobian_host(pda_problem *p, const double *h_U, double t,
                                          double *h_V, double *h_J);

/* jacobian(U, t, J) (adapter_cpp.hpp:223-229): V goes to internal scratch. */
pda_status pda_jacobian(pda_problem *p, const double *d_U, double t, double *d_J);

/* applyJacobian(U, B, t, R) (adapter_cpp.hpp:231-259): recomputes J at U and
 * forms R = J * B for a column-major B of n_cols columns (ld = rows of B =
 * totalDofStencilMesh, R ld = totalDofSampleMesh). */
pda_status pda_apply_jacobian(pda_problem *p, const double *d_U, double t, const double *d_B,
                              int n_cols, double *d_R);

/* --------------------------------------------------------------- steppers */

/* Explicit time integration on the device with the vendored Pressio
 * steppers' update formulas: SSP-RK3
 * (ode_explicit_stepper_without_mass_matrix.hpp:230-282) and RK4 (:284-336).
 * U is advanced in place by n_steps steps of size dt from t0.  When
 * use_graph != 0 each step is captured once into a CUDA graph and replayed. */
pda_status pda_advance_ssprk3(pda_problem *p, double *d_U, double t0, double dt, int64_t n_steps,
                              int use_graph);
pda_status pda_advance_rk4(pda_problem *p, double *d_U, double t0, double dt, int64_t n_steps,
                           int use_graph);

/* ----------------------------------------------------------------- batches
 * (no counterpart in the reference, whose callers loop over problem objects)
 *
 * A batch advances many independent problems -- one family and scheme,
 * uneven mesh sizes, own parameters (e.g. the shallow-water gravity,
 * Coriolis and pulse of each instance) -- with one launch per residual phase
 * over all instances.  Instances must be full natural-order meshes whose
 * boundaries are periodic or mirror images (2D Neumann, slip wall).  The
 * problems must outlive the batch; their own entry points stay usable.
 *
 * Packed layout: instance i owns dofs [offsets[i], offsets[i] + its
 * totalDofStencilMesh) of one device vector (offsets from
 * pda_batch_offsets, n+1 values, each instance starting on a 256-byte
 * boundary); entries between instances are not read by the residual and are
 * left untouched in V. */
typedef struct pda_batch pda_batch;
pda_status pda_batch_create(pda_problem *const *problems, int n, void *stream, pda_batch **out);
void pda_batch_free(pda_batch *b);
pda_status pda_batch_sizes(const pda_batch *b, int *n, int64_t *total_dofs, int64_t *total_cells);
pda_status pda_batch_offsets(const pda_batch *b, int64_t *offsets);
/* every instance's initialCondition() at its packed offset (zeros between) */
pda_status pda_batch_initial_condition(pda_batch *b, double *d_U);
/* every instance's velocity; bit-identical to pda_velocity on each problem */
pda_status pda_batch_velocity(pda_batch *b, const double *d_U, double t, double *d_V);
/* n_steps SSP-RK3 steps of size dt for all instances (the single-problem
 * stage formulas); use_graph != 0 replays one captured step */
pda_status pda_batch_advance_ssprk3(pda_batch *b, double *d_U, double t0, double dt, int64_t n_steps,
                                    int use_graph);
/* Tile shapes of the face kernels (threads along the face axis x lines per
 * block).  The autotuner times every compiled shape per axis on d_U (reps
 * launches each) and keeps the fastest; ms (may be NULL) receives the mean
 * times [axis][shape]. */
int pda_batch_num_tile_shapes(const pda_batch *b);
pda_status pda_batch_set_tile_shape(pda_batch *b, int axis, int shape);
pda_status pda_batch_tile_shape(const pda_batch *b, int axis, int *shape, int *lanes, int *lines);
pda_status pda_batch_autotune(pda_batch *b, const double *d_U, int reps, double *ms);
int64_t pda_batch_launch_count(const pda_batch *b);

/* ------------------------------------------------- learned-manifold ROM
 * (no counterpart in the reference; building blocks of the autoencoder
 * trained on snapshots of the batched full-order model)
 *
 * BF16 tensor-core GEMM on tcgen05 with fp32 accumulation in tensor memory:
 * C[M x N] = A[M x K] * B[N x K]^T (+ bias[N]; epilogue 0 none, 1 bias,
 * 2 bias + ELU), A and B row-major bf16 (uint16 storage), K a multiple of 64.
 * Outputs (any may be NULL, not both of d_outF / d_outB): fp32 and / or bf16
 * row-major [M x N], d_preact = fp32 value before the activation.
 * Synchronous on `stream` (cudaStream_t, NULL = legacy default).  Shapes
 * with N <= 16 take the thin blocked kernel and allocate scratch for both
 * operands' blocked copies and the split partial sums on every call (the
 * reduced-order model's decoder keeps its operands pre-blocked instead). */
pda_status pda_tc_gemm_bf16(const void *d_A, const void *d_B, int64_t M, int64_t N, int64_t K,
                            const float *d_bias, int epilogue, float *d_outF, void *d_outB,
                            float *d_preact, void *stream);

/* MLP autoencoder for the learned manifold, trained on the device with the
 * tcgen05 GEMM (bf16 operands, fp32 accumulation) and Adam (fp32 masters):
 *   encoder n -> ha (ELU) -> hb (ELU) -> latent;  decoder latent -> hb (ELU)
 *   -> ha (ELU) -> n (full-width output); loss = mean squared error.
 * n, ha, hb multiples of 64; latent <= 64 (padded to 64 inside).  Data are
 * bf16 rows [ns x n] on the device (uint16 storage).  Layers 0..5 in the
 * order above; padded shapes: W [out x in], b [out]. */
typedef struct pda_ae pda_ae;
pda_status pda_ae_create(int64_t n, int latent, int ha, int hb, uint64_t seed, void *stream, pda_ae **out);
void pda_ae_free(pda_ae *ae);
/* epochs of minibatch Adam over a seeded permutation; losses[epoch] = mean
 * batch loss (may be NULL); batch a multiple of 64 */
pda_status pda_ae_train(pda_ae *ae, const void *d_data, int64_t ns, int batch, int epochs, double lr,
                        uint64_t seed, double *losses);
/* fused = 1 (default): each Adam step runs inside the epilogues of the
 * weight-gradient GEMMs, so the fp32 weight gradients are never stored;
 * fused = 0: gradients are stored, then a separate optimizer pass.  Both give
 * the same weights bit for bit. */
pda_status pda_ae_set_fused(pda_ae *ae, int fused);
/* Y = decoder(encoder(X)) (fp32 [rows x n]); Z (may be NULL) = latent [rows x latent] */
pda_status pda_ae_reconstruct(pda_ae *ae, const void *d_X, int64_t rows, float *d_Y, float *d_Z);
/* loss and all parameter gradients of one batch, no update (gradient checks);
 * d_grads = concatenation over layers of [W, b] with padded shapes */
pda_status pda_ae_gradients(pda_ae *ae, const void *d_X, int batch, double *loss, float *d_grads);
pda_status pda_ae_layer(pda_ae *ae, int layer, float *d_W, float *d_b, int64_t *out_in);
pda_status pda_ae_set_layer(pda_ae *ae, int layer, const float *d_W, const float *d_b);

/* Hyper-reduced LSPG on the device (no counterpart in pressio-demoapps; the
 * algorithm of Pressio's LspgUnsteadyResidualJacobianPolicyHypRed,
 * rom/impl/lspg_unsteady_rj_policy_hypred.hpp:180-264, with BDF1 and a
 * Gauss-Newton solver whose normal equations are formed and factored in
 * FP64).  sample_problem is a problem on a sample mesh; sample_to_stencil[i]
 * is the stencil-mesh index of sample cell i.  Trial spaces:
 *   affine: y = uref + Phi x         (d_phi: stencil dofs x k, row-major)
 *   mlp:    y = uref + scale * (W3 elu(W2 elu(W1 x + b1) + b2) + b3)
 *           (W1: h1 x k, W2: h2 x h1, W3: stencil dofs x h2, row-major fp32;
 *            h1 = 256; the decoder's output rows at the stencil cells)
 * k must be one of 2, 4, 6, 8, 10, 12, 16, 20, 24, 32. */
typedef struct pda_lspg pda_lspg;
pda_status pda_lspg_create_affine(pda_problem *sample_problem, const int64_t *sample_to_stencil, int k,
                                  const double *d_uref, const double *d_phi, pda_lspg **out);
/* mode 0: the decoder in fp32 on the CUDA cores; mode 1: the network's own
 * training numerics -- the output layer as a tcgen05 GEMM with bf16 weights
 * (which must already be bf16 values) and bf16 activations, fp32
 * accumulation (latent at most 15, h2 a multiple of 64). */
pda_status pda_lspg_create_mlp(pda_problem *sample_problem, const int64_t *sample_to_stencil, int k, int h1,
                               int h2, const double *d_uref, const double *d_scale, const float *d_W1,
                               const float *d_b1, const float *d_W2, const float *d_b2, const float *d_W3,
                               const float *d_b3, int mode, pda_lspg **out);
void pda_lspg_free(pda_lspg *rom);
/* y (stencil dofs) of latent x (k doubles, device) */
pda_status pda_lspg_decode(pda_lspg *rom, const double *d_x, double *d_y);
/* n_steps BDF1 steps of size dt from latent d_x (updated in place), at most
 * gn_iters Gauss-Newton iterations per step (stopping early once the
 * correction norm is below tol); use_graph != 0 replays one captured step.
 * info (may be NULL) receives {last correction norm, iterations of the last
 * step, residual norm at the last iterate, max of that norm over the
 * iterates of this call's steps}. */
pda_status pda_lspg_advance_bdf1(pda_lspg *rom, double *d_x, double dt, int64_t n_steps, int gn_iters,
                                 double tol, int use_graph, double *info);
/* The same with the backward-difference order chosen: order 1 (BDF1) or 2
 * (BDF2: R = y_n+1 - 4/3 y_n + 1/3 y_n-1 - 2/3 dt f(y_n+1)).  first_step is
 * the 1-based index, within the trajectory, of the first step this call
 * takes; as in Pressio's BDF2 LSPG (rom/impl/lspg_unsteady_rj_policy_hypred.hpp:
 * 124-134) step 1 is a BDF1 step, and each step's first Gauss-Newton iteration
 * moves the stored y_n to y_n-1, so consecutive calls continue one
 * trajectory when first_step continues its numbering. */
pda_status pda_lspg_advance(pda_lspg *rom, double *d_x, double dt, int64_t n_steps, int gn_iters, double tol,
                            int order, int64_t first_step, int use_graph, double *info);

/* Gauss-Newton iteration form: fused = 1 (default) evaluates the sample-mesh
 * velocity and the product of its Jacobian with the trial space's latent
 * Jacobian face by face in one launch (never forming the CSR Jacobian);
 * fused = 0 assembles the sample-mesh CSR Jacobian with pda_velocity_and_jacobian
 * and multiplies it in a second kernel.  Same LSPG iteration; results agree
 * to rounding. */
pda_status pda_lspg_set_fused(pda_lspg *rom, int fused);

/* Precision of the Jacobian terms in the fused iteration: 64 (default) the
 * exact Jacobian of the sample-mesh residual in double; 32 the reconstruction
 * gradients, flux Jacobians and the Jacobian-times-basis product in single
 * precision, an inexact Gauss-Newton step (relative perturbation ~1e-7 of
 * the step) on the same double-precision velocity, residual, normal
 * equations and solve.  No counterpart in the reference (which has no ROM);
 * the assembled form (fused = 0) is always double. */
pda_status pda_lspg_set_jacobian_precision(pda_lspg *rom, int bits);

/* Implicit steps on the device (the consumer of the Jacobian in the
 * reference's implicit tests, tests_cpp/eigen_2d_euler_riemann_implicit/
 * main.cc:31-44: Pressio's implicit stepper + Newton-Raphson + BiCGSTAB).
 * scheme 0 = BDF1, 1 = Crank-Nicolson.  Per step, Newton iterations with
 * J_R = I - c dt Jf (c = 1 or 1/2) stop before updating once the l2 norm of
 * the correction is below newton_tol (Pressio's default criterion); each
 * correction is BiCGSTAB with a Jacobi preconditioner to a relative residual
 * of linear_tol.  Full meshes only.  info (may be NULL) receives {Newton
 * iterations in total, most in one step, BiCGSTAB iterations in total, worst
 * final relative linear residual}. */
pda_status pda_advance_implicit(pda_problem *p, double *d_U, double t0, double dt, int64_t n_steps, int scheme,
                                double newton_tol, int newton_max_iters, double linear_tol,
                                int linear_max_iters, double *info);

/* --------------------------------------------------------- diagnostics
 * (no counterpart in the reference: measurement support for benchmarks) */

/* Number of kernels this library launched since the problem was created. */
int64_t pda_problem_launch_count(const pda_problem *p);

/* Evaluate the velocity reps times with CUDA events between the kernels of
 * the structured path; ms[5] receives the mean device time of the face
 * kernels along x, y, z, the balance kernel and the near-boundary row
 * kernel (0 where absent).  The kernels run one after another here;
 * pda_velocity runs the face passes of different axes side by side. */
pda_status pda_profile_velocity(pda_problem *p, const double *d_U, double *d_V, int reps,
                                double ms[5]);

/* Measured FP64 FMA throughput of the current device (FLOP/s, FMA = 2). */
pda_status pda_measure_fp64_peak(double *flops_per_s);

/* Self-check of the integer-pipe division and square root the kernels use
 * for every FP64 division and square root: on (SMs x 2048 threads) x
 * per_thread seeded operand sets of the given mode (0 normal-range
 * operands, 1 divisor mantissas near the ends of [1, 2), 2 near-exact
 * quotients and roots, 3 arbitrary bit patterns), compares each result with
 * the FP64 pipe's IEEE division and square root bit for bit.  counts receives
 * {operand sets, division mismatches, square-root mismatches}.  No
 * counterpart in the reference (whose divisions are the CPU's). */
pda_status pda_check_divsqrt(int mode, uint64_t seed, int64_t per_thread, int64_t counts[3]);

/* Self-check of the integer-pipe forms of the products by constants the
 * kernels use (K x for K = 3, 5, 7, 11, 13; x / 2 and x / 4; x c for
 * literals c such as 1/6, 13/12, 2e-6) and of the density guard x + 1e-30:
 * on (SMs x 2048 threads) x per_thread seeded operands of the given mode
 * (0 normal range, 1 exponents at the edges of the fast paths and short
 * mantissas, 2 mantissas near the ends of [1, 2), 3 arbitrary bit patterns),
 * compares each result with the FP64 pipe's operation bit for bit.  counts
 * receives {operands, small-integer product mismatches, power-of-two
 * mismatches, guard mismatches, constant product mismatches}.  No
 * counterpart in the reference. */
pda_status pda_check_products(int mode, uint64_t seed, int64_t per_thread, int64_t counts[5]);

#ifdef __cplusplus
}
#endif

#endif /* PDA_GB300_H_ */
