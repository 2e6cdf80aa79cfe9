/* Test infrastructure only (the oracle).  Plain-C restatement of the
 * pressio-demoapps residual / Jacobian algorithm, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline; never by the
 * product library. */
#ifndef PDA_ORACLE_H_
#define PDA_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mesh orc_mesh;
typedef struct orc_problem orc_problem;

const char *orc_last_error(void);

orc_mesh *orc_mesh_load(const char *dir);
orc_mesh *orc_mesh_from_arrays(int dim, int stencil, int64_t sample_size, int64_t stencil_size,
                               const int32_t *graph, const double *x, const double *y, const double *z,
                               const double dx[3]);
void orc_mesh_free(orc_mesh *m);
void orc_mesh_counts(const orc_mesh *m, int64_t out[4]); /* stencil, sample, inner, nearBd */

orc_problem *orc_problem_create(const orc_mesh *m, int family, int problem, int scheme, int icflag,
                                int nparams, const char *const *names, const double *vals);
void orc_problem_free(orc_problem *p);
void orc_sizes(const orc_problem *p, int64_t out[4]); /* ndpc, dofs sample, dofs stencil, nnz */
void orc_initial_condition(const orc_problem *p, double *U);
void orc_velocity(orc_problem *p, const double *U, double t, double *V);
void orc_velocity_and_jacobian(orc_problem *p, const double *U, double t, double *V, int32_t *rowptr,
                               int32_t *colidx, double *vals);
void orc_ssprk3(orc_problem *p, double *U, double t0, double dt, int64_t nsteps);
void orc_rk4(orc_problem *p, double *U, double t0, double dt, int64_t nsteps);
void orc_ssprk3_py(orc_problem *p, double *U, double t0, double dt, int64_t nsteps);
void orc_weno5(const double q7[7], double out4[4]);
void orc_weno3(const double q5[5], double out4[4]);
/* point-wise functions, exported for tests of the device numerics */
void orc_weno5_face(const double q[6], double u[2]);
void orc_weno3_face(const double q[4], double u[2]);
void orc_weno5_face_grad(const double q[6], double u[2], double gN[6], double gP[6]);
void orc_weno3_face_grad(const double q[4], double u[2], double gN[4], double gP[4]);
void orc_point_flux(int family, int ax, const double *qL, const double *qR, double param, double *F,
                    double *JL, double *JR);
/* 0: pow(x, 3.) as the reference (default); 1: correctly rounded x^3 */
void orc_set_cube_mode(int correctly_rounded);
/* out[i] = strtod(sprintf("%.14f", in[i])): mesh-script coordinates as read back */
void orc_round14(const double *in, double *out, int64_t n);
/* OpenMP threads for the CPU baseline (<= 0: all). Returns the count used. */
int orc_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
