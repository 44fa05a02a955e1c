/*
 * plbm_gpu.h -- C ABI of libplbmgpu.so, the GB300 (sm_103a) D2Q9 periodic
 * stream-collide library.
 *
 * Every entry point takes plain pointers and sizes, returns 0 (PLBM_OK) or a
 * negative PLBM_E* code, and records a message readable through
 * plbm_last_error() (thread-local).  A handle is not reentrant: calls on one
 * handle must be serialised by the caller (the reference calls one routine at
 * a time from its serial time loop).  Distinct handles are independent.
 *
 * Lattice layout is the reference's (src/fvm_bardow.F90:144-153):
 *   f(ld,nx,0:8,nf), element (y,x,q,b) at 0-based offset
 *   y + ld*(x + nx*(q + 9*b)), ld = ny rounded up to a multiple of 16.
 * Macroscopic fields are (ny,nx) arrays, y fastest (src/fvm_bardow.F90:155).
 * Buffer indices (iold, inew, ibuf) are 1-based, as in the Fortran.
 */
#ifndef PLBM_GPU_H
#define PLBM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PLBM_OK             0
#define PLBM_E_INVALID     -1  /* bad argument: size, kind, index, NULL     */
#define PLBM_E_NOMEM       -2  /* device or pinned allocation failed        */
#define PLBM_E_CUDA        -3  /* CUDA runtime error (message has details)  */
#define PLBM_E_UNSUPPORTED -4  /* valid request this build does not offer   */
#define PLBM_E_TIMEOUT     -5  /* a bounded device-side wait expired        */
#define PLBM_E_NODEVICE    -6  /* no CUDA device visible                    */

/* Largest nx, ny (and ld) accepted: the kernels index cells with 32-bit
 * coordinates, which must not overflow when rounded up to a whole tile.
 * Larger extents are rejected with PLBM_E_INVALID. */
#define PLBM_MAX_EXTENT (1 << 30)

/* ---- collision kinds (grid%collision => collide_*) ---------------------- */
#define PLBM_BGK   0  /* collide_bgk, src/collision_bgk.F90:17-82          */
#define PLBM_TRT   1  /* collide_trt, src/collision_trt.F90:41-160         */
#define PLBM_RR    2  /* collide_rr,  src/collision_regularized.F90:21-202 */
#define PLBM_BGKI  3  /* collide_bgk_improved, src/collision_bgk_improved.f90:16-109 */

/* ---- storage of the populations on the device -------------------------- */
#define PLBM_F64     0  /* f_i in binary64, reference semantics               */
#define PLBM_F32DEV  1  /* h_i = f_i - w_i in binary32, binary32 collision     */
#define PLBM_F16DEV  2  /* h_i = f_i - w_i in binary16 scaled by 2^PLBM_F16_SCALE_LOG2 */
#define PLBM_F16_SCALE_LOG2 15

/* ---- arithmetic of the fused step --------------------------------------
 * PLBM_F64 storage:
 *   FMA    binary64, FMA contraction allowed (default)
 *   STRICT binary64, no contraction: the Fortran's operations in its order,
 *          bit-identical to it
 *   HYBRID BGK, TRT and RR: exact integer moments, double-float for the
 *          small terms, binary64 only for the final combination (FP64
 *          instructions per cell: BGK 18, TRT 10, RR 9, instead of 60-150).
 *          A cell with |f_0| >= 2, |f_axis| >= 1/2 or |f_diagonal| >= 1/4
 *          is evaluated with the FMA binary64 operator instead (see
 *          plbm_hybrid_range_flag)
 * Deviation storage (PLBM_F32DEV / PLBM_F16DEV):
 *   FMA    binary32 collision (default)
 *   STRICT binary64 collision on the stored deviations
 *   HYBRID BGK only: compensated binary32 collision (exact pairwise sums,
 *          hi+lo pairs for the O(h) linear terms, binary32 nonlinear term)
 *   DF64   BGK only: double-float collision on the stored deviations */
#define PLBM_MATH_FMA    0
#define PLBM_MATH_STRICT 1
#define PLBM_MATH_HYBRID 2
#define PLBM_MATH_DF64   3

/* ---- streaming schemes (grid%streaming => ...) ----------------------------
 * LBM       lbm_stream, src/periodic_lbm.f90:32-129 (default; fused with the
 *           collision in plbm_perform_lbm_step)
 * FVM_BARDOW        stream_fvm_bardow, src/fvm_bardow.F90:393-509
 * FDM_BARDOW        stream_fdm_bardow, src/fvm_bardow.F90:511-686, central
 *                   differences (the default build)
 * FDM_BARDOW_ISO    the same with the isotropic differences (FDM_ISO build)
 * FDM_BARDOW_WLS    the same with unweighted least squares (FDM_WLS build)
 * FDM_SOFONEA       stream_fdm_sofonea, src/fvm_bardow.F90:688-886
 * FDM_BARDOW_WLS_GAUSS_V1 / _V2  stream_fdm_bardow with Gaussian-weighted least
 *                   squares (FDM_WLS_GAUSS_V1 / V2 builds, :604-644)
 * The finite-volume / finite-difference schemes use grid%dt (set_properties)
 * and run with PLBM_F64 storage, FMA or STRICT arithmetic. */
#define PLBM_STREAM_LBM            0
#define PLBM_STREAM_FVM_BARDOW     1
#define PLBM_STREAM_FDM_BARDOW     2
#define PLBM_STREAM_FDM_BARDOW_ISO 3
#define PLBM_STREAM_FDM_BARDOW_WLS 4
#define PLBM_STREAM_FDM_SOFONEA    5
#define PLBM_STREAM_FDM_BARDOW_WLS_GAUSS_V1 6
#define PLBM_STREAM_FDM_BARDOW_WLS_GAUSS_V2 7

typedef struct plbm_grid plbm_grid_t;

/* Message of the last failing call on this thread ("" if none). */
const char *plbm_last_error(void);
/* Library ABI version (major*10000 + minor*100 + patch). */
int plbm_version(void);

/* ---- lattice_grid lifecycle -------------------------------------------- */
/* alloc_grid(grid,nx,ny,nf) -- src/fvm_bardow.F90:129-202.  Allocates nf
 * device lattices (ld,nx,0:8), sets inew=1, iold=2, collision BGK.  nf >= 2. */
int plbm_grid_create(int nx, int ny, int nf, int storage, plbm_grid_t **out);
/* dealloc_grid -- src/fvm_bardow.F90:204-240.  NULL is accepted. */
int plbm_grid_destroy(plbm_grid_t *g);
int plbm_grid_info(const plbm_grid_t *g, int *nx, int *ny, int *ld, int *nf, int *storage);
/* grid%iold / grid%inew (1-based). */
int plbm_grid_indices(const plbm_grid_t *g, int *iold, int *inew);
int plbm_grid_set_indices(plbm_grid_t *g, int iold, int inew);
/* grid%iold / grid%inew / grid%imid (imid = 3 when nf > 2, else -1;
 * src/fvm_bardow.F90:172-177). */
int plbm_grid_indices3(const plbm_grid_t *g, int *iold, int *inew, int *imid);
int plbm_grid_set_indices3(plbm_grid_t *g, int iold, int inew, int imid);
/* Run the handle's work on this cudaStream_t (NULL = the handle's own stream). */
int plbm_grid_set_stream(plbm_grid_t *g, void *cuda_stream);
/* Device address of lattice ibuf (for device-resident callers).  A
 * plbm_perform_triple_step permutes which device lattice backs which buffer
 * index: query the address again after one. */
int plbm_grid_device_ptr(const plbm_grid_t *g, int ibuf, void **dptr);

/* ---- properties --------------------------------------------------------- */
/* set_properties(grid,nu,dt[,magic]) -- src/fvm_bardow.F90:242-269.
 * tau = 3 nu, omega = dt/(tau + dt/2), trt_magic = magic or (tau/dt)^2.
 * magic may be NULL (absent optional). */
int plbm_set_properties(plbm_grid_t *g, double nu, double dt, const double *magic);
int plbm_get_properties(const plbm_grid_t *g, double *nu, double *dt, double *tau,
                        double *omega, double *trt_magic);
/* Set omega and the TRT magic parameter directly. */
int plbm_set_relaxation(plbm_grid_t *g, double omega, double trt_magic);
/* Set grid%dt alone (the time step of the finite-volume / finite-difference
 * streaming schemes); omega is left as it is. */
int plbm_set_time_step(plbm_grid_t *g, double dt);
/* grid%collision => collide_bgk | collide_trt | collide_rr | collide_bgk_improved
 * (app/main_taylor_green.f90:39). */
int plbm_set_collision(plbm_grid_t *g, int kind);
/* PLBM_MATH_* for PLBM_F64 storage. */
int plbm_set_math(plbm_grid_t *g, int math);
/* grid%streaming => lbm_stream | stream_fvm_bardow | stream_fdm_bardow |
 * stream_fdm_sofonea (PLBM_STREAM_*; app/main_vortex.f90:44). */
int plbm_set_streaming(plbm_grid_t *g, int scheme);

/* ---- transfers ---------------------------------------------------------- */
/* Copy host f(:,:,:,ibuf) (ld*nx*9 doubles) to/from the device lattice.
 * For deviation storage the values are converted (f - w_i) on the device. */
int plbm_upload(plbm_grid_t *g, const double *f_host, int ibuf);
int plbm_download(plbm_grid_t *g, double *f_host, int ibuf);

/* ---- the hot path ------------------------------------------------------- */
/* set_pdf_to_equilibrium -- src/fvm_bardow.F90:272-305.  rho, ux, uy are host
 * (ny,nx) arrays; writes the equilibrium into f(:,:,:,iold) on the device.
 * Page-locked (pinned, mapped) host arrays are read in place by the kernel;
 * pageable ones are staged through device memory (in x-column slabs that
 * overlap copies and kernels on grids of 2^22 cells or more).  The same holds
 * for the outputs of plbm_update_macros. */
int plbm_set_pdf_to_equilibrium(plbm_grid_t *g, const double *rho, const double *ux,
                                const double *uy);
/* Same from DEVICE (ny,nx) arrays into lattice ibuf, asynchronous. */
int plbm_equilibrium_device(plbm_grid_t *g, int ibuf, const double *rho, const double *ux,
                            const double *uy);
/* grid%streaming() -- lbm_stream (src/periodic_lbm.f90:32-129) or the
 * selected scheme: f(:,:,:,iold) -> f(:,:,:,inew). */
int plbm_stream(plbm_grid_t *g);
/* grid%collision() -- in place on f(:,:,:,inew). */
int plbm_collide(plbm_grid_t *g);
/* perform_lbm_step -- src/periodic_lbm.f90:15-29, nsteps times: one fused
 * pull-stream + collide kernel per step (lbm_stream; another streaming
 * scheme: its kernel, then the collision), then the iold/inew swap. */
int plbm_perform_lbm_step(plbm_grid_t *g, int nsteps);
/* perform_triple_step -- src/fvm_bardow.F90:322-340, nsteps times (needs
 * nf >= 3, PLBM_F64 storage, PLBM_MATH_FMA or _STRICT): stream iold -> inew,
 * keep the streamed populations in iold, collide inew, rotate
 * iold <- inew, inew <- imid, imid <- iold.  One fused kernel per step
 * (read 72 B, write 144 B per cell) writes the pre-collision populations to a
 * spare lattice (allocated on the first call) that then backs buffer index
 * iold; every buffer index holds what the Fortran leaves in it. */
int plbm_perform_triple_step(plbm_grid_t *g, int nsteps);
/* update_macros -- src/fvm_bardow.F90:343-390: moments of f(:,:,:,inew)
 * into host (ny,nx) arrays.  Any of rho/ux/uy may be NULL.
 * With PLBM_MATH_HYBRID and PLBM_F64 storage the moments (here and in
 * plbm_macros_device) and the equilibria (plbm_set_pdf_to_equilibrium,
 * plbm_equilibrium_device) are integer forms: rho = sum f and u = j / rho
 * correctly rounded from the exact sums, feq within 0.5 ulp + w_i 2^-58 of
 * the exact w_i rho (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2); cells outside their
 * range (f_i < 0 or >= 1, rho >= 8; rho outside (0, 2) or |u| >= 1/4) take
 * the reference's binary64 expressions.  The other modes evaluate those. */
int plbm_update_macros(plbm_grid_t *g, double *rho, double *ux, double *uy);
/* Same moments of lattice ibuf into DEVICE (ny,nx) arrays, asynchronous. */
int plbm_macros_device(plbm_grid_t *g, int ibuf, double *rho, double *ux, double *uy);

/* ---- vorticity, src/vorticity.f90 --------------------------------------- */
/* vorticity_2nd (order 2, :13-43) or vorticity_4th (order 4, :46-87) on host
 * (ny,nx) arrays.  order 44 selects the standard 4th-order weights (2/3 on
 * +-1, -1/12 on +-2), which the reference routine does not use. */
int plbm_vorticity(int order, int nx, int ny, const double *ux, const double *uy, double *omega);
/* Same on device arrays, asynchronous on cuda_stream (may be NULL). */
int plbm_vorticity_device(int order, int nx, int ny, const double *ux, const double *uy,
                          double *omega, void *cuda_stream);

/* ---- binary64 reductions ------------------------------------------------- */
/* E = 1/2 sum rho |u|^2 over the moments of lattice ibuf (moments evaluated as
 * in update_macros), accumulated in binary64. */
int plbm_kinetic_energy(plbm_grid_t *g, int ibuf, double *energy);
/* sqrt(sum |u - ua|^2 / sum |ua|^2) for lattice ibuf against host (ny,nx)
 * fields uxa, uya (calc_L2_norm, app/main_taylor_green.f90:174-212). */
int plbm_velocity_l2_error(plbm_grid_t *g, int ibuf, const double *uxa, const double *uya,
                           double *err);

/* Same number as plbm_velocity_l2_error, for callers that cannot allocate
 * device memory when they ask for it: a diagnostic hook inside a run whose
 * lattices fill nearly all of HBM, a program whose device memory is held by
 * another (caching) allocator, or a time loop that must not allocate.  No
 * counterpart in the reference (it has no device memory).
 * f is a DEVICE lattice f(ld,nx,0:8) of the given storage; uxa, uya are host
 * (ny,nx) fields; err is a host double.  Nothing is allocated: the reference
 * fields and the partial sums are staged in one fixed device array of
 * 2*PLBM_NOALLOC_MAX_CELLS + PLBM_NOALLOC_PARTIAL_DOUBLES doubles (about 16 MB),
 * reserved on every GPU that loads the library until exit.
 * nx*ny > PLBM_NOALLOC_MAX_CELLS returns PLBM_E_INVALID, and so do extents
 * above PLBM_MAX_EXTENT.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current; make that first
 * call before any stream capture.  All calls share the array and it keeps the
 * last call's contents, so calls that overlap on the GPU (other streams,
 * other host threads) race; serialise them: the library's lock covers only
 * the first call's address lookup, not the calls.  Runs on cuda_stream (may be
 * NULL) and returns after the result is on the host. */
#define PLBM_NOALLOC_MAX_CELLS (1 << 20)
#define PLBM_NOALLOC_PARTIAL_DOUBLES 3648
int plbm_velocity_l2_error_noalloc(int storage, int nx, int ny, int ld, const void *f,
                                   const double *uxa, const double *uya, double *err,
                                   void *cuda_stream);

/* ---- files (.npy, NumPy format version 1.0) -------------------------------
 * output_npy -- src/fvm_bardow.F90:930-961, src/output/npy.f90:13-26: the
 * moments mf(ny,nx,3) = (rho, ux, uy) of f(:,:,:,inew) (as update_macros
 * computes them) written as a Fortran-order binary64 array of shape
 * (ny, nx, 3). */
int plbm_output_npy(plbm_grid_t *g, const char *path);
/* The same under the reference's name: folder/filename + step as %09d +
 * ".npy" (step < 0: no number), creating folder (mkdir -p) first.  folder
 * NULL or "": the working directory (the reference's concatenation would
 * name the root directory). */
int plbm_output_npy_step(plbm_grid_t *g, const char *folder, const char *filename, int step);
/* Restart files: all nf lattices as binary64 f(ld,nx,0:8,nf), Fortran order
 * (deviation storage is converted).  load_state needs the same ld, nx, nf.
 * Buffer indices are not stored (plbm_grid_indices3 / set_indices3). */
int plbm_save_state(plbm_grid_t *g, const char *path);
int plbm_load_state(plbm_grid_t *g, const char *path);
/* Host-only helpers (no device): write a binary64 array as .npy; read the
 * header of one (shape has room for 8 extents). */
int plbm_write_npy(const char *path, const double *data, int ndim, const long long *shape,
                   int fortran_order);
int plbm_read_npy_header(const char *path, int *ndim, long long *shape, int *fortran_order,
                         long long *data_offset);

/* Wait for all work queued on the handle's stream. */
int plbm_synchronize(plbm_grid_t *g);

/* PLBM_MATH_HYBRID with PLBM_F64 storage evaluates a cell outside its range
 * (|f_0| >= 2, |f_axis| >= 1/2 or |f_diagonal| >= 1/4) with the binary64
 * operator and sets a device flag: results stay valid, the flag only reports
 * that the slower path ran.  Reads it (after synchronising the device) and
 * clears it when reset != 0.  No reference counterpart (the reference has no
 * such mode). */
int plbm_hybrid_range_flag(int *flag, int reset);

/* ---- batched grids ------------------------------------------------------
 * Many independent periodic grids of uneven sizes and relaxation times,
 * stepped together.  No counterpart in the reference (it steps one
 * lattice_grid at a time); each grid's step is the reference's
 * perform_lbm_step with collide_bgk or collide_trt (incompressible TRT with
 * the grid's magic parameter).  Every grid keeps the layout f(ld,nx,0:8),
 * ld = pad16(ny), with two lattices packed in one allocation.
 *
 * Work is cut into tiles of ty rows (y) x threads/ty columns of one grid;
 * ty is chosen per grid from the bucket of its ny (<=48, <=96, <=192,
 * <=384, >384).  persistent = 1 runs all steps of a plbm_batch_run in ONE
 * cooperative launch with a grid-wide barrier between steps (bounded wait:
 * an expired wait is reported as PLBM_E_TIMEOUT by plbm_batch_synchronize);
 * persistent = 0 launches once per step.  Either can be captured into a CUDA
 * graph with plbm_batch_capture and replayed with plbm_batch_launch_graph. */
#define PLBM_BATCH_BUCKETS 5
typedef struct plbm_batch_schedule {
    int threads;       /* threads per CTA, multiple of 32 in [64, 512]          */
    int ctas_per_sm;   /* resident CTAs per SM, 0 = occupancy maximum           */
    int persistent;    /* 1 = one cooperative launch for all steps              */
    int ty[PLBM_BATCH_BUCKETS]; /* tile rows per ny bucket, power of 2 >= 32    */
} plbm_batch_schedule;
typedef struct plbm_batch plbm_batch_t;

int plbm_batch_default_schedule(plbm_batch_schedule *s);
/* kind[i] in {PLBM_BGK, PLBM_TRT}; trt_magic may be NULL (0.25);
 * storage PLBM_F64 or PLBM_F32DEV.  All lattices start at 0. */
int plbm_batch_create(int ngrids, const int *nx, const int *ny, const int *kind,
                      const double *omega, const double *trt_magic, int storage,
                      plbm_batch_t **out);
int plbm_batch_destroy(plbm_batch_t *b);
int plbm_batch_info(const plbm_batch_t *b, int *ngrids, long long *cells, int *ntiles, int *ctas);
int plbm_batch_set_schedule(plbm_batch_t *b, const plbm_batch_schedule *s);
int plbm_batch_get_schedule(const plbm_batch_t *b, plbm_batch_schedule *s);
int plbm_batch_set_stream(plbm_batch_t *b, void *cuda_stream);
/* Collision arithmetic of the batch: PLBM_MATH_FMA (default) for every
 * storage, or PLBM_MATH_HYBRID for PLBM_F64 (BGK and TRT grids alike take
 * the hybrid binary64 arithmetic of plbm_set_math; a cell outside its range
 * takes the FMA binary64 operator). */
int plbm_batch_set_math(plbm_batch_t *b, int math);
/* Equilibrium of host (ny,nx) rho/ux/uy into the current lattice of grid i
 * (set_pdf_to_equilibrium, src/fvm_bardow.F90:272-305). */
int plbm_batch_set_equilibrium(plbm_batch_t *b, int grid, const double *rho, const double *ux,
                               const double *uy);
/* Queue nsteps steps of every grid (asynchronous). */
int plbm_batch_run(plbm_batch_t *b, int nsteps);
/* Capture nsteps steps into a CUDA graph for the current step parity. */
int plbm_batch_capture(plbm_batch_t *b, int nsteps);
int plbm_batch_launch_graph(plbm_batch_t *b);
/* Failure injection for tests of the bounded wait: the next persistent
 * plbm_batch_run starts with a grid-barrier arrival count that can never
 * complete, so every CTA's wait runs out (a few seconds), the kernel returns,
 * and plbm_batch_synchronize reports PLBM_E_TIMEOUT; the lattices are left
 * part-stepped and the context stays usable.  Persistent schedule only. */
int plbm_batch_inject_stall(plbm_batch_t *b);
/* Wait; PLBM_E_TIMEOUT if a persistent run's barrier wait expired. */
int plbm_batch_synchronize(plbm_batch_t *b);
int plbm_batch_steps(const plbm_batch_t *b, long long *steps);
/* Moments (update_macros order for PLBM_F64) of grid i's current state into
 * host (ny,nx) arrays; any may be NULL.  Synchronises. */
int plbm_batch_macros(plbm_batch_t *b, int grid, double *rho, double *ux, double *uy);
/* Current lattice of grid i as binary64 f(ld,nx,0:8) on the host. */
int plbm_batch_download(plbm_batch_t *b, int grid, double *f);

/* ---- discrete adjoint -----------------------------------------------------
 * Reverse-mode derivative of the BGK time stepper: f_0 = equilibrium(1, u0)
 * (src/fvm_bardow.F90:99-126), nsteps x perform_lbm_step with lbm_stream +
 * collide_bgk (src/periodic_lbm.f90:15-29), u_T = j/rho of the final state.
 * No counterpart in the reference.  Hand-written reverse step: the Jacobian
 * transpose of the BGK collision applied matrix-free, then streaming
 * transposed (a push along -c_q).  Memory is bounded by checkpointing every
 * checkpoint_every (K) steps and recomputing each segment: ceil(T/K) + 2K + 4
 * lattices, the recomputation of the next segment running on a second stream
 * of the handle beside the reverse steps of the current one (ordered by
 * events; the call's work still ends on the caller's stream).  When the
 * second K-lattice buffer does not fit, create falls back to one buffer,
 * each recomputation after the previous sweep (same gradients, bit for bit).
 * dL/domega is accumulated in binary64.  storage PLBM_F64 (binary64 arithmetic) or
 * PLBM_F32DEV (binary32 storage and per-cell arithmetic).
 * All field pointers are DEVICE arrays of 2*nx*ny doubles: component a of
 * cell (x,y) at a*nx*ny + y + ny*x (two (ny,nx) fields). */
typedef struct plbm_adjoint plbm_adjoint_t;
int plbm_adjoint_create(int nx, int ny, int storage, int nsteps, int checkpoint_every,
                        plbm_adjoint_t **out);
int plbm_adjoint_destroy(plbm_adjoint_t *a);
int plbm_adjoint_set_stream(plbm_adjoint_t *a, void *cuda_stream);
/* Arithmetic of the reverse step: PLBM_MATH_FMA (default: the storage's own
 * arithmetic) or, for PLBM_F32DEV, PLBM_MATH_HYBRID: compensated binary32 (the
 * O(lambda) sums in double-float, each pair's update from the exact pair sum
 * and difference, one rounding per stored value), about 3x smaller gradient
 * error at about 1.25x the reverse-step time.  No counterpart in the
 * reference. */
int plbm_adjoint_set_math(plbm_adjoint_t *a, int math);
/* Device bytes held by the handle. */
int plbm_adjoint_memory(const plbm_adjoint_t *a, size_t *bytes);
/* Run the model from u0 with relaxation omega; writes u_T (may be NULL) and
 * keeps the checkpoints for the next backward call.  Asynchronous. */
int plbm_adjoint_forward(plbm_adjoint_t *a, const double *u0, double omega, double *uT);
/* Given dL/du_T, writes dL/du0 (device, may be NULL) and dL/domega (host,
 * may be NULL; synchronises when given). */
int plbm_adjoint_backward(plbm_adjoint_t *a, const double *grad_uT, double *grad_u0,
                          double *grad_omega);

/* ---- raw device launches (device-resident callers: batched, autograd) ---- */
/* One fused pull-stream + collide step over device lattices fsrc -> fdst
 * (layout above, PLBM_F64 storage = double, F32DEV = float, F16DEV = half). */
int plbm_launch_step(int storage, int math, int kind, int nx, int ny, int ld,
                     const void *fsrc, void *fdst, double omega, double trt_magic,
                     void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* PLBM_GPU_H */
