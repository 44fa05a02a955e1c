/*
 * plbm_plugin.h -- the reference's simulation-plugin C ABI, served by
 * libplbmgpu.so under the stem "plbmgpu".
 *
 * Replaces the Fortran plugin sim/sim_slbm.F90:135-205 (prototypes in
 * sim/lbm.h:13-19).  A loader derives the symbol names from the library file
 * stem (sim/cases.py:21-32): libplbmgpu.so -> c_plbmgpu_{init,step,vars,free,norm}.
 *
 * Semantics follow sim/sim_slbm.F90 and sim/sim.F90:
 *  - fields are (nx,ny) arrays, x fastest (Fortran order); u is (nx,ny,2);
 *  - the "rho" argument of init carries the pressure p, and the density is
 *    rho = 1 + p/cs^2 (sim/sim.F90:193, sim/cases.py:302-303);
 *  - populations are stored shifted, h_i = f_i - w_i (sim/sim.F90:131,384);
 *  - a step is collide-then-push-stream with periodic wrap
 *    (sim/sim.F90:404-505 + :568-624);
 *  - dt must be 1.0 (sim/sim_slbm.F90:48-51).
 * Where the reference stops the program (error stop), these entry points
 * return NULL / set a sticky error instead; read it with plbm_last_error()
 * and c_plbmgpu_status().
 */
#ifndef PLBM_PLUGIN_H
#define PLBM_PLUGIN_H
#ifdef __cplusplus
extern "C" {
#endif

/* Optional plugin parameters, passed through the params slot of init
 * (the reference passes NULL there, sim/cases.py:95).  NULL selects
 * {BGK, PLBM_F64, trt_magic 0.25}. */
typedef struct plbm_plugin_params {
    int version;       /* 1, or 2 when `math` is filled in                  */
    int kind;          /* PLBM_BGK | PLBM_TRT | PLBM_RR                    */
    int storage;       /* PLBM_F64 | PLBM_F32DEV | PLBM_F16DEV             */
    double trt_magic;  /* TRT magic parameter (Lambda)                     */
    int math;          /* version 2: PLBM_MATH_FMA | PLBM_MATH_STRICT |
                          PLBM_MATH_HYBRID (PLBM_F64: the hybrid binary64
                          arithmetic on the shifted populations)           */
} plbm_plugin_params;

/* siminit -- sim/lbm.h:13-15, c_slbm_init sim/sim_slbm.F90:135-149 (slbm_init :41-78) */
void *c_plbmgpu_init(int nx, int ny, double dt, const double *rho, const double *u,
                     const double *sigma, void *params);
/* simstep -- sim/lbm.h:17, c_slbm_step sim/sim_slbm.F90:152-160 (slbm_step :80-110) */
void c_plbmgpu_step(void *sim, double omega);
/* simvars -- sim/lbm.h:18, c_slbm_vars sim/sim_slbm.F90:163-180 (slbm_vars :112-127) */
void c_plbmgpu_vars(void *sim, double *rho, double *u);
/* simfree -- sim/lbm.h:19, c_slbm_free sim/sim_slbm.F90:184-195 */
void c_plbmgpu_free(void *sim);
/* norm2(u-ua)/norm2(ua) -- c_slbm_norm sim/sim_slbm.F90:198-205 (host arithmetic) */
double c_plbmgpu_norm(int nx, int ny, const double *u, const double *ua);
/* Not in the reference: sticky status of a plugin instance (0 = ok). */
int c_plbmgpu_status(void *sim);
/* Not in the reference: run nsteps steps in one call (same result as nsteps
 * calls of c_plbmgpu_step). */
int c_plbmgpu_steps(void *sim, double omega, int nsteps);
/* Not in the reference: wait until the queued steps have finished (steps run
 * asynchronously on the instance's stream; vars() waits by itself).  Returns
 * the sticky status. */
int c_plbmgpu_synchronize(void *sim);

#ifdef __cplusplus
}
#endif
#endif
