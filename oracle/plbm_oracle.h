/*
 * plbm_oracle.h -- CPU restatement of the periodic-lbm D2Q9 hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path
 * and the timed CPU baseline; the product never links or calls it.
 *
 * Parity status: PINNED for the Taylor-Green driver with the finite-difference
 * Bardow streaming and BGK -- set_properties, set_pdf_to_equilibrium,
 * stream_fdm_bardow, collide_bgk, update_macros -- against the errors the
 * reference binary printed in graphs/fvm_bardow_64.txt (21 runs of 17,558 to
 * 1,755,763 steps on 64 x 64; tests/test_reference_bardow64.py): within half
 * a printed unit + 2.2e-10.  UNPINNED for TRT, RR, the improved BGK and
 * lbm_stream: the reference is Fortran 2008, no Fortran compiler exists on
 * either build machine, and the reference ships no other output or golden
 * vectors for this path.  The restatement follows the Fortran loop for loop
 * and keeps its parenthesisation; it is checked against analytic invariants
 * (mass/momentum conservation, the equilibrium fixed point, Taylor-Green
 * decay) and against an independent numpy restatement
 * (tests/golden/make_golden.py).
 *
 * Layout (reference src/ convention, src/fvm_bardow.F90:144-153):
 *   f(ld,nx,0:8), element (y,x,q) at 0-based offset y + ld*(x + nx*q),
 *   ld = ny rounded up to a multiple of 16.
 * Plugin convention (sim/sim.F90:102-117): f(0:nx+1,0:ny+1,0:8), x fastest,
 *   element (i,j,q) at 0-based offset i + (nx+2)*(j + (ny+2)*q), i,j in 0..n+1.
 */
#ifndef PLBM_ORACLE_H
#define PLBM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

int  oref_pad16(int ny);

/* src/periodic_lbm.f90:45-127 */
void oref_lbm_stream(int nx, int ny, int ld, const double *fsrc, double *fdst);
/* src/collision_bgk.F90:35-82 (split=0) and :84-176 (split=1) */
void oref_collide_bgk(int nx, int ny, int ld, double *f, double omega, int split);
/* src/collision_trt.F90:24-34 */
double oref_magic_number(double le, double ld);
double oref_lambda_d(double omega, double x);
/* src/collision_trt.F90:64-160 (split=0) and :162-290 (split=1) */
void oref_collide_trt(int nx, int ny, int ld, double *f, double lambda_e, double lambda_d, int split);
/* src/collision_regularized.F90:40-202 */
void oref_collide_rr(int nx, int ny, int ld, double *f, double omega);
/* src/collision_bgk_improved.f90:24-107 (dummy f1(ny,nx,0:8): ld is ignored) */
void oref_collide_bgk_improved(int nx, int ny, double *f, double omega);
/* src/fvm_bardow.F90:356-388 */
void oref_update_macros(int nx, int ny, int ld, const double *f, double *rho, double *ux, double *uy);
/* src/vorticity.f90:13-43 and :46-87; arrays (ny,nx) */
void oref_vorticity_2nd(int nx, int ny, const double *ux, const double *uy, double *w);
void oref_vorticity_4th(int nx, int ny, const double *ux, const double *uy, double *w);
/* src/fvm_bardow.F90:242-269; magic may be NULL (absent optional) */
void oref_set_properties(double nu, double dt, const double *magic,
                         double *tau, double *omega, double *trt_magic);
/* src/fvm_bardow.F90:99-126 */
void oref_equilibrium(double rho, double ux, double uy, double feq[9]);
/* src/fvm_bardow.F90:272-305; rho/ux/uy are (ny,nx) */
void oref_set_pdf_to_equilibrium(int nx, int ny, int ld, const double *rho,
                                 const double *ux, const double *uy, double *f);
/* src/periodic_lbm.f90:15-29 with lbm_stream + collision kind; f holds both
 * buffers (ld,nx,9,2); iold/inew are 1-based and updated in place. */
enum { OREF_BGK = 0, OREF_TRT = 1, OREF_RR = 2, OREF_BGKI = 3 };
void oref_perform_lbm_step(int nx, int ny, int ld, double *f, int *iold, int *inew,
                           int kind, double omega, double trt_magic, int nsteps);
/* Finite-volume / finite-difference streaming, src/fvm_bardow.F90:393-886
 * (loops over the whole nx x ny grid; the reference's swapped bounds in
 * stream_fvm_bardow / stream_fdm_sofonea agree with them for nx == ny). */
void oref_stream_fvm_bardow(int nx, int ny, int ld, const double *fold, double *fnew, double dt);
void oref_stream_fdm_bardow(int nx, int ny, int ld, const double *fold, double *fnew, double dt, int variant);
void oref_stream_fdm_sofonea(int nx, int ny, int ld, const double *fold, double *fnew, double dt);
void oref_perform_step_scheme(int nx, int ny, int ld, double *f, int *iold, int *inew, int scheme, double dt,
                              int kind, double omega, double trt_magic, int nsteps);
/* src/benchmarks/taylor_green.f90:51-84.  ref_loop=1 reproduces the reference
 * inner loop bound `y = 1, self%nx` (:68); ref_loop=0 loops y = 1, ny. */
void oref_taylor_green_eval(int nx, int ny, double kx, double ky, double umax, double nu,
                            double t, double *p, double *ux, double *uy, int ref_loop);
/* src/benchmarks/shear_layer.f90:31-50 */
void oref_shear_layer_eval(int nx, int ny, double length, double u0, double k, double delta,
                           double rho0, double *rho, double *ux, double *uy);
/* app/main_taylor_green.f90:174-212: |hypot(u-ua)| / |hypot(ua)| (norm2 = sqrt(sum sq)) */
double oref_tgv_l2_norm(int nx, int ny, const double *ux, const double *uy,
                        const double *uxa, const double *uya);
/* kinetic energy 0.5*sum(rho*(ux^2+uy^2)), summed column by column (x outer) */
double oref_kinetic_energy(int nx, int ny, const double *rho, const double *ux, const double *uy);

/* ---- plugin semantics, sim/sim.F90 (DDF-shifted storage, push streaming) ---- */
/* sim/sim.F90:181-199 */
void oref_sim_eqinit_fields(int nx, int ny, int nhalo, double *f, const double *p,
                            const double *u, const double *v);
/* sim/sim.F90:148-179 */
void oref_sim_macros(int nx, int ny, int nhalo, const double *f, double *rho, double *u, double *v);
/* sim/sim.F90:404-505 (push branch) */
void oref_sim_collide_stream_fused(int nx, int ny, const double *fsrc, double *fdst, double omega);
/* sim/sim.F90:568-624 */
void oref_sim_bc_push(int nx, int ny, double *f);
/* sim/sim_slbm.F90:80-110, nsteps steps with the move_alloc swap (f1 <-> f2 pointers) */
void oref_sim_slbm_steps(int nx, int ny, double *f1, double *f2, double omega, int nsteps);
/* sim/sim_slbm.F90:198-205 */
double oref_sim_norm(int nx, int ny, const double *u, const double *ua);

/* ---- discrete adjoint of the BGK time stepper (no reference counterpart) --
 * Model: f_0 = equilibrium(1, u0) (src/fvm_bardow.F90:99-126), then nsteps of
 * perform_lbm_step with lbm_stream + collide_bgk; u_T = j/rho of the final
 * state.  Given G = dL/du_T (arrays gux, guy of shape (ny,nx)), returns
 * dL/du0 (arrays (ny,nx)) and dL/domega, by reverse-mode differentiation of
 * every step (all states kept: small grids only).  Also writes u_T. */
void oref_adjoint_bgk(int nx, int ny, const double *ux0, const double *uy0, double omega, int nsteps,
                      const double *gux, const double *guy, double *uxT, double *uyT,
                      double *grad_ux0, double *grad_uy0, double *grad_omega);
/* Forward only: u_T of the same model. */
void oref_forward_bgk(int nx, int ny, const double *ux0, const double *uy0, double omega, int nsteps,
                      double *uxT, double *uyT);

/* ---- OpenMP thread count actually used (for the CPU baseline report) ---- */
int oref_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
