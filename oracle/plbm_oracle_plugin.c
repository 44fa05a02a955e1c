/*
 * plbm_oracle_plugin.c -- the oracle's restatement of the standard-LBM plugin
 * (sim/sim_slbm.F90 over sim/sim.F90) behind the reference's plugin C ABI
 * (sim/lbm.h:13-19), under the stem "oracleplugin": liboracleplugin.so
 * exports c_oracleplugin_{init,step,vars,free,norm}.
 *
 * TEST INFRASTRUCTURE ONLY.  It lets the reference's own Python loader and
 * study code (sim/cases.py SimPlugin, run, TGVStudy) drive the oracle on the
 * CPU, so the loader and studies of the product (plbm.plugin, plbm.studies)
 * can be compared with the reference's, and it yields the expected states of
 * the GPU plugin's parity tests.  The product never links or calls it.
 *
 * Semantics as sim/sim_slbm.F90 (gfortran branch):
 *   init  :41-78 and :135-149 -- dt must be 1 (:48-51; here NULL is returned
 *          where the reference stops), sigma is not implemented (:64-70),
 *          equilibrium initialisation from (p, u, v), f2 = f1 (:76)
 *   step  :80-110 and :152-160 -- fused collide + push into f2, periodic
 *          halo push, move_alloc swap
 *   vars  :112-127 and :163-180 -- macroscopic fields of f1
 *   free  :184-195, norm :198-205
 */
#include <stdlib.h>
#include <string.h>

#include "plbm_oracle.h"

typedef struct {
    int nx, ny;
    double *f1, *f2;  /* halo lattices f(0:nx+1,0:ny+1,0:8) */
} oplugin;

void *c_oracleplugin_init(int nx, int ny, double dt, const double *rho, const double *u,
                          const double *sigma, void *params)
{
    (void)params;
    if (nx < 1 || ny < 1 || dt != 1.0 || sigma || !rho || !u) return NULL;
    oplugin *s = calloc(1, sizeof *s);
    if (!s) return NULL;
    size_t n = (size_t)(nx + 2) * (size_t)(ny + 2) * 9u;
    s->nx = nx;
    s->ny = ny;
    s->f1 = calloc(n, sizeof(double));
    s->f2 = calloc(n, sizeof(double));
    if (!s->f1 || !s->f2) {
        free(s->f1);
        free(s->f2);
        free(s);
        return NULL;
    }
    /* u is (nx,ny,2) in Fortran order: the x block, then the y block */
    oref_sim_eqinit_fields(nx, ny, 1, s->f1, rho, u, u + (size_t)nx * ny);
    memcpy(s->f2, s->f1, n * sizeof(double));
    return s;
}

void c_oracleplugin_step(void *sim, double omega)
{
    oplugin *s = sim;
    if (!s) return;
    oref_sim_collide_stream_fused(s->nx, s->ny, s->f1, s->f2, omega);
    oref_sim_bc_push(s->nx, s->ny, s->f2);
    double *t = s->f1;
    s->f1 = s->f2;
    s->f2 = t;
}

void c_oracleplugin_vars(void *sim, double *rho, double *u)
{
    oplugin *s = sim;
    if (!s) return;
    oref_sim_macros(s->nx, s->ny, 1, s->f1, rho, u, u + (size_t)s->nx * s->ny);
}

void c_oracleplugin_free(void *sim)
{
    oplugin *s = sim;
    if (!s) return;
    free(s->f1);
    free(s->f2);
    free(s);
}

double c_oracleplugin_norm(int nx, int ny, const double *u, const double *ua)
{
    return oref_sim_norm(nx, ny, u, ua);
}
