/*
 * beachslope.h -- C-ABI of the GB300 (sm_103a) ISPH particle hot path.
 *
 * The reference (Sinchanrc/Beach-Slope, Fortran 2008 + OpenMP) exposes its
 * per-step physics as argument-less module subroutines acting on module
 * globals (dpcell, fmatrix, fvec, fsol, dt, h1: initialize.f90:54-69).  Those
 * derived types hold allocatable/pointer components and are not
 * interoperable, so this boundary replaces them with a context that owns all
 * device state, plus plain SoA host buffers that the caller owns.
 *
 * Every function returns an int status: 0 = ok, negative = error class
 * (BS_E_*).  No exception crosses the ABI, there is no global state, and a
 * context is externally synchronised (one host thread at a time); work is
 * ordered on the context's own CUDA stream.  A Fortran caller must call from
 * outside `!$omp parallel` (or from `!$omp masked` followed by a barrier),
 * because the reference's entry points are called by every thread of the
 * enclosing parallel region (main.f90:238-261).
 *
 * A context holds a batch of one or more scenes.  Each scene has its own cell
 * grid, parameters, time step and solver state; every stage runs over all
 * scenes of the batch in one launch.
 */
#ifndef BEACHSLOPE_H
#define BEACHSLOPE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define BS_OK              0
#define BS_E_ARG          -1   /* bad argument / size                         */
#define BS_E_CUDA         -2   /* CUDA runtime error                          */
#define BS_E_NOMEM        -3   /* device or host allocation failed            */
#define BS_E_CAPACITY     -4   /* particle, neighbour or cell capacity hit    */
#define BS_E_NOTCONV      -5   /* PPE solve did not reach the tolerance       */
#define BS_E_NONFINITE    -6   /* NaN/Inf detected in a checked field         */
#define BS_E_DOMAIN       -7   /* particle outside the interior cell grid     */
#define BS_E_STATE        -8   /* call order violated (e.g. solve before assemble) */

/* device error-word bits (bs_error_bits) */
#define BS_ERR_NBR_OVERFLOW    0x01u  /* neighbour list longer than kmax      */
#define BS_ERR_ZERO_DIAG       0x02u  /* PPE row with zero diagonal (isph.f90:436) */
#define BS_ERR_SOLVER_BREAK    0x04u  /* BiCGStab breakdown (rho or omega = 0) */
#define BS_ERR_NOT_CONVERGED   0x08u  /* maxit reached before tolerance        */
#define BS_ERR_NONFINITE       0x10u  /* NaN/Inf in pressure or positions      */
#define BS_ERR_LOST_PARTICLE   0x20u  /* particle left the interior grid       */
#define BS_ERR_ZERO_SHIFT      0x40u  /* opt2_shift with exactly zero shift (NaN, part_shift.f90:89) */
#define BS_ERR_NO_NEIGHBOUR    0x80u  /* fluid particle with no neighbours     */

/* particle type ids (particle.f90:11): 1 fixed wall, 2 ghost/dummy wall, 3 fluid */
#define BS_TID_WALL   1
#define BS_TID_GHOST  2
#define BS_TID_FLUID  3

/* particle flag bits (particles%free / %vicinity / %buffer, particle.f90:42-43) */
#define BS_FLAG_FREE      0x01u
#define BS_FLAG_VICINITY  0x02u
#define BS_FLAG_BUFFER    0x04u

/* precision modes */
#define BS_PREC_FP64   0   /* plain FP64 drop-in                                      */
#define BS_PREC_MIXED  1   /* pair values stored in FP32 (each the FP32 rounding of the
                              FP64 value); neighbour sweeps on the FP32 pipe, double-float
                              where terms cancel; FP32 multigrid cycle, double-float FGMRES
                              basis; FP64 Krylov loop, residuals and positions */

/* PPE stopping rules */
#define BS_STOP_RELRES     0  /* ||b - A x||_2 / ||b||_2 <= ppe_tol                    */
#define BS_STOP_REFERENCE  1  /* every |dx_i/(x_i+1e-5)| <= 1e-2 (solver.f90:233-242)  */
#define BS_STOP_R0         2  /* ||b - A x||_2 / ||b - A x0||_2 <= ppe_tol: the relative-to-initial-
                                 residual test of the reference's FGMRES (dpar(1), solver.f90:324) */

#define BS_SOLVER_BICGSTAB 0  /* bicgstab, solver.f90:129-254                          */
#define BS_SOLVER_FGMRES   1  /* fgmres, solver.f90:306-350: restarted flexible GMRES   */

/*
 * Scene parameters.  Defaults and formulas follow initialize.f90:21-81 and
 * setup.f90:10-150; bs_params_default() fills the reference's values.
 */
typedef struct bs_params {
    /* resolution and cell grid */
    double h;          /* smoothing length h1 (setup.f90:47)                          */
    double dl;         /* lattice spacing dl = min particle spacing (setup.f90:53)    */
    int32_t cellx;     /* cells in x incl. the empty border ring (setup.f90:51)       */
    int32_t celly;     /* cells in y incl. the empty border ring (setup.f90:52)       */
    /* time */
    double dt;         /* time step (fixed unless adaptive_dt)                        */
    double t0;         /* simulated time at upload                                    */
    int32_t adaptive_dt; /* 1: timestep() rule integrator.f90:927-937 sets dt          */
    int32_t scalar_on;   /* 1: salinity sub-steps run at the start of each step        */
    /* fluid */
    double rho;        /* reference density (initialize.f90:23)                       */
    double rhomin;     /* initialize.f90:24, used at scalar.f90:414                   */
    double rhomax;     /* rho*rel_den (setup.f90:19)                                  */
    double rel_den;    /* initialize.f90:27                                           */
    double g;          /* gravity along y (negative)                                  */
    double mu;         /* viscosity in the timestep rule (initialize.f90:39)          */
    double tschmidt;   /* turbulent Schmidt number (initialize.f90:25)                */
    /* porous medium (porous.f90:111) */
    double por;        /* grain-bed porosity                                          */
    double lamk;       /* Ergun constant                                              */
    double d50;        /* grain diameter                                              */
    /* free surface and shifting */
    double lamfs;      /* 0.8  (initialize.f90:46)                                    */
    double maxdivr;    /* 2.0  (initialize.f90:45)                                    */
    double csh;        /* 0.5  (initialize.f90:24)                                    */
    double maxshift;   /* 0.1  (initialize.f90:40)                                    */
    double sig1;       /* 0.2  CFL factor (initialize.f90:39)                         */
    /* outflow cut-offs used by the second re-bin (integrator.f90:61-62) */
    double xlcutoff;
    double ytcutoff;
    /* PPE */
    double ppe_tol;    /* relative residual tolerance                                 */
    int32_t ppe_maxit;
    int32_t ppe_stop;  /* BS_STOP_*                                                   */
    int32_t precision; /* BS_PREC_*                                                   */
    int32_t kmax;      /* neighbour-list capacity per particle (<= 64)                */
    /* mixed precision: FP32 inner BiCGStab tolerance per refinement sweep and
     * the number of FP64 refinement sweeps (0: solve with the FP64 BiCGStab) */
    double mixed_inner_tol;
    int32_t mixed_max_outer;
    /* PPE preconditioner: 0 none (the reference's plain BiCGStab), 1 cell-grid
     * aggregation multigrid V-cycle (FP64 in BS_PREC_FP64, FP32 in BS_PREC_MIXED) */
    int32_t ppe_precond;
    /* WCSPH (wcsph.f90): speed of sound co (never set by the reference,
     * setup.f90:134; 10*sqrt(g*depth) for the beach scenes), Tait exponent
     * t_gam (7, initialize.f90:46), delta-SPH coefficient delt (0.1,
     * initialize.f90:40), and the still-water level that the reference
     * writes as brrealy*distfac*(2*bl-1)+wc (wcsph.f90:78-82) */
    double wc_c0;
    double wc_gamma;
    double wc_delta;
    double wc_ysurf;
    /* calmasscons form: 0 as the reference writes it (term2 doubles as the
     * pair's hydrostatic difference, so only the last neighbour's y term
     * survives, and the delta-SPH term runs along r_i - r_j, which is
     * anti-diffusive, wcsph.f90:78-117); 1 this library's correction (y term
     * summed over all neighbours, delta term along r_j - r_i; no reference
     * counterpart) */
    int32_t wc_form;
    int32_t wc_pad;
    /* PPE Krylov method (BS_SOLVER_*) and the FGMRES restart length (1..150;
     * the reference's MKL call keeps MKL's default, 150).  Context-wide, taken
     * from scene 0 like ppe_precond.  FGMRES stops on ppe_stop =
     * BS_STOP_RELRES (||r||/||b||) or BS_STOP_R0 (||r||/||r0||, the
     * reference's rule; BS_STOP_REFERENCE is read as BS_STOP_R0 there), with
     * ppe_maxit counting Arnoldi columns over all restart cycles */
    int32_t ppe_solver;
    int32_t ppe_restart;
    /* comp_pos buffer release (integrator.f90:865-872): a buffer particle
     * whose new x lies in (buf_release_lo, buf_release_hi) becomes fluid --
     * the reference's window is (8 prrealx + brrealx + 0.001, xrcutoff).  The
     * default (lo > hi) never releases. */
    double buf_release_lo;
    double buf_release_hi;
} bs_params;

/*
 * Host SoA view of one scene's particles.  On upload only the "state" fields
 * are read (x..flags); on download every non-NULL pointer is filled, in the
 * context's particle order: cell-major (column-major over cells, as resetid,
 * isph.f90:97-108), walls first in each cell, then fluid in slot order.
 */
typedef struct bs_state {
    int32_t n;
    double *x, *y, *vx, *vy, *p, *mass, *rho, *oden, *ovol, *con;
    int32_t *tid, *pid;
    uint8_t *flags;
    /* download-only per-particle fields (may be NULL) */
    double *xs, *ys, *vxs, *vys;
    double *porosity, *resx, *resy, *nut, *tke, *varts, *gradvx, *vel, *cdiff;
    double *coff;      /* 4*n: L-matrix inverse (coff, search.f90:276-278)        */
    int32_t *cell;     /* cell key (j-1)*celly + (i-1)                              */
} bs_state;

/* static grain particles of the porous bed (porlist, boundary.f90:582-585) */
typedef struct bs_grains {
    int32_t n;
    double *x, *y, *mass, *rho;
} bs_grains;

/*
 * Open-boundary buffer zone of a scene: the reference's remove_bufferN +
 * insert_bufferN (internal.f90:447-586) with the schedule of main.f90:218-234.
 * Zone 0 / 1 stand for buffer1 / buffer2.  At an exchange, every buffer
 * particle of the zone's entry cells whose x is at or beyond remove_x
 * (remove_side +1: x >= remove_x, rv_buf_r; -1: x <= remove_x, rv_buf_l) is
 * removed, the survivors keeping their order, then every template particle
 * is appended to the entry cell that contains it, in template order (give the
 * template column by column, as the reference's loops visit bufferN(k,i)),
 * as a buffer fluid particle with the template's position, velocity,
 * pressure and pid (NULL: 0, as the reference's templates) and the zone's
 * mass, density (also oden), ovol and con; xs, ys, vxs, vys = 0.  bs_step
 * runs the exchange after the scalar sub-steps and before projection when
 * (t_old + phase) < k period <= (t_old + dt + phase), k = 1, 2, ... counted
 * per zone from bs_set_inflow (period 0: never).
 */
typedef struct bs_inflow {
    int32_t n;
    const double *x, *y, *vx, *vy, *p;
    const int32_t* pid;
    double mass, rho, ovol, con;
    double period, phase;
    double remove_x;
    int32_t remove_side;
    int32_t ncells;                /* entry cells, dpcell(i, j): 1-based row i, column j */
    const int32_t *cell_i, *cell_j;
} bs_inflow;

/* per-scene scalars reported back to the host */
typedef struct bs_scene_info {
    int32_t n;            /* particles in the scene                         */
    int32_t solsteps;     /* scalar sub-steps for the next step             */
    int32_t ppe_iters;    /* BiCGStab iterations of the last solve          */
    int32_t ppe_outer;    /* refinement sweeps of the last solve (mixed)    */
    double dt, dtsol, t;  /* current step sizes and simulated time          */
    double umax, numax;   /* timestep() maxima (integrator.f90:914-924)     */
    double ppe_relres;    /* true FP64 relative residual of the last solve  */
    uint32_t err_bits;    /* BS_ERR_* seen since the last bs_clear_errors   */
    int32_t pad0;
} bs_scene_info;

/* ---- lifetime ------------------------------------------------------------- */
void bs_params_default(bs_params* p);

/* Select the CUDA device for contexts created afterwards on this host thread
 * (one process per GPU: call with the local rank before bs_create). */
int bs_set_device(int32_t device);

/* Create a context for nscenes scenes; params[s] and capacity[s] (max particles)
 * per scene.  Replaces init/memalloc/matrixid (setup.f90:10, memory.f90:10,80). */
int bs_create(int32_t nscenes, const bs_params* params, const int32_t* capacity,
              const int32_t* grain_capacity, struct bs_ctx** out);
int bs_destroy(struct bs_ctx* ctx);

/* Upload one scene's particles and grains (bins them into cells with the
 * reference's comparison rule; walls first in a cell, then fluid). */
int bs_upload(struct bs_ctx* ctx, int32_t scene, const bs_state* st, const bs_grains* gr);
/* Page-locked host memory for the arrays of bs_upload / bs_download
 * (cudaMallocHost): copies from and to it run at the host link's full rate
 * and overlap.  Any host memory works with both calls; this is the fast kind. */
int bs_host_alloc(size_t bytes, void** p);
int bs_host_free(void* p);
int bs_download(struct bs_ctx* ctx, int32_t scene, bs_state* st);
/* Read-back that overlaps the steps that follow (the reference writes its
 * state between steps, output.f90:188-222; a host loop here can keep the GPU
 * stepping meanwhile).  Snapshots the scene's rows of the non-null fields of
 * st on the device in stream order after the work already submitted (the next
 * bs_step can be called at once), then copies the snapshot into st's buffers
 * on a copy stream.  st's buffers hold the scene's capacity rows (bs_create's
 * capacity rounded up to a multiple of 256; st->n gives their size) and stay
 * untouched until bs_download_wait, which waits for the copy and sets st->n to
 * the particle count at the snapshot; rows beyond it are padding.  cell and
 * coff are not available here (bs_download).  Pinned buffers (bs_host_alloc)
 * let the copy overlap compute; one read-back in flight per scene. */
int bs_download_async(struct bs_ctx* ctx, int32_t scene, bs_state* st);
int bs_download_wait(struct bs_ctx* ctx, int32_t scene, bs_state* st);
int bs_scene_info_get(struct bs_ctx* ctx, int32_t scene, bs_scene_info* out);
int bs_clear_errors(struct bs_ctx* ctx);
int bs_sync(struct bs_ctx* ctx);
const char* bs_last_error(struct bs_ctx* ctx);

/* Neighbour lists for parity tests: counts[n] and idx[n*kmax] as particle
 * indices in download order (list%nh, interactions.f90:26-35). */
int bs_get_neighbours(struct bs_ctx* ctx, int32_t scene, int32_t* counts, int32_t* idx,
                      double* dist, double* kx, double* ky);
/* Assembled, Jacobi-scaled PPE rows (isph.f90:423-444): diag[n], off[n*kmax]
 * aligned with the neighbour list, rhs[n]. */
int bs_get_matrix(struct bs_ctx* ctx, int32_t scene, double* diag, double* off, double* rhs);

/* Re-use scene slot `scene` for another scene (new parameters, particles and
 * grains; a request loop refills slots this way).  The slot keeps the
 * capacities it was created with: rows, grains, and the cell grid given by
 * the parameters passed to bs_create -- the new cellx/celly may not exceed
 * those (BS_E_CAPACITY).  The other scenes are untouched.  No counterpart in
 * the reference (one scene per run). */
int bs_set_scene(struct bs_ctx* ctx, int32_t scene, const bs_params* params, const bs_state* st,
                 const bs_grains* gr);
/* bs_prime for one scene only; the other scenes are left exactly as they
 * are, so a scene joining a running batch does not perturb the others. */
int bs_prime_scene(struct bs_ctx* ctx, int32_t scene);

/* boun_vel, integrator.f90:394-457 (compiled in the reference, never
 * called): wall and ghost particles (tid 1, 2) take minus the Shepard average
 * of their fluid neighbours' velocity (a no-slip mirror), divided only when
 * the Shepard sum reaches 1e-6 (single literal); vxs = vys = 0.  Uses the
 * neighbour lists of the last bs_search. */
int bs_boun_vel(struct bs_ctx* ctx);
/* comp_ghost + ghost_en, mls.f90:114-263 (not compiled in the reference):
 * the same mirror of the velocity, tke and nut onto wall and ghost particles
 * that have neighbours, over their fluid neighbours (the module's list2 is
 * never built; the neighbour list restricted to fluid stands in), 0 where the
 * Shepard sum is 0.  use_mls = 1: the velocity by the module's commented-out
 * moving-least-squares branch -- weights W (b1 + b2 dx + b3 dy) m/rho with b
 * the first column of the inverse 3x3 moment matrix over all neighbours
 * (Wmls, mls.f90:16-111; invertmat3D, functions.f90:134-165), the Shepard
 * average where that determinant is below 1e-5 (single literal), which at the
 * reference's particle sizes is every particle. */
int bs_ghost(struct bs_ctx* ctx, int32_t use_mls);
/* coll_pos_shift (mode 0, part_shift.f90:193-292) and coll_shift (mode 1,
 * 294-410), compiled in the reference and never called.  Every particle's
 * xs, ys (mode 0) or vxs, vys (mode 1) are set to 0; a fluid particle with
 * neighbours, gradvx >= 0.7 and not in a buffer gets, per axis, the
 * mass-weighted push of the neighbours closer than the collision distance
 * pr/sqrt(phi_i) + (fluid ? pr : br)/sqrt(phi_j) (pr, br = prx, brx along x
 * and pry, bry along y: the half particle spacings prrealx, prrealy, brrealx,
 * brrealy of the reference) -- from the overlap (mode 0) or the approaching
 * relative pore velocity (mode 1) -- over m_i + the sum of the neighbour
 * masses.  Then mode 0 moves those particles by (xs, ys); mode 1 adds
 * phi (vxs, vys) to the velocity of every fluid particle not in a buffer.
 * Uses the neighbour lists and stored pair distances of the last bs_search. */
int bs_collision_shift(struct bs_ctx* ctx, int32_t mode, double prx, double pry, double brx, double bry);

/* Set (or, with z->n = 0 and z->ncells = 0, clear) buffer zone `zone` (0 or
 * 1) of a scene; the template is copied.  entrycell1/2 of the reference. */
int bs_set_inflow(struct bs_ctx* ctx, int32_t scene, int32_t zone, const bs_inflow* z);
/* remove_bufferN + insert_bufferN of one zone now (outside the schedule).
 * BS_E_CAPACITY if the scene could exceed its row capacity. */
int bs_buffer_exchange(struct bs_ctx* ctx, int32_t scene, int32_t zone);

/* combined, output.f90:188-222: the scene's fluid particles as text, one
 * line each in the reference's order and format (F10.3 x, y, p; ES10.3 vx,
 * vy; F10.5 con+0.5) -- non-buffer particles to fluid_path, buffer particles
 * to buffer_path (may be NULL: not written). */
int bs_write_combined(struct bs_ctx* ctx, int32_t scene, const char* fluid_path, const char* buffer_path);

/* Solver tunables, set by the project autotuner (beach-slope_gb300/autotune.py):
 * "ppe_solver" (BS_SOLVER_*), "ppe_restart" (FGMRES restart, 1..150),
 * "mg_omega" (Jacobi damping), "mg_cscale" (coarse-correction scale),
 * "mg_pre0" / "mg_prec" (pre-smoothing at the particle / cell levels, 0 or 1),
 * "mg_post0" (1 or 2 particle-level post-sweeps), "mg_coarse_sweeps",
 * "mg_wlev" (coarse levels 1..mg_wlev visit the next level twice: W-cycle on
 * top, V-cycle below), "mg_sub" (0/1: the small levels of a visit as one
 * clustered launch), "ppe_precond", "fg_df" (0/1, default 1: the FGMRES basis
 * of the preconditioned mixed solve as double-float (hi, lo) FP32 pairs, its
 * dots on the FP32 pipe, h_{j+1,j} from the Gram relation), "mg_fp32" (0/1,
 * default 0: the FP64 form's multigrid preconditioner in FP32 like the mixed
 * form's; the Krylov solve, its residuals and stopping test stay FP64, so the
 * pressure solves the same FP64 system to the same tolerance), "mg_tail" (0/1,
 * default 1: each visit of the level above the coarsest, with the coarsest
 * solve, as one block per scene in shared memory -- bit-identical to the
 * separate launches; used where every scene ends on the same two levels of at
 * most 1024 and 256 cells), "sweep_tpb" /
 * "mg0_tpb" (64, 128 or 256 threads per block of the neighbour sweeps / of
 * the particle-level multigrid kernels; every row is computed the same way
 * whatever the block size), "step_graph" (0/1, default 1: each bs_step is
 * one captured CUDA graph with the loops on the device);
 * bs_get_option also reads "mg_levels", "mg_sub_level", "mg_tail_level", "step_graph_steps"
 * and "step_graph_cached". */
int bs_set_option(struct bs_ctx* ctx, const char* name, double value);
int bs_get_option(struct bs_ctx* ctx, const char* name, double* value);

/* Replace the assembled right-hand side (already Jacobi-scaled) of one scene,
 * e.g. with a manufactured source; b[n] in download order. */
int bs_set_rhs(struct bs_ctx* ctx, int32_t scene, const double* b);

/* ---- one entry point per reference subroutine ----------------------------- */
/* Warm-up: neighbour lists, porosity, eddy viscosity and timestep maxima for
 * the uploaded state (what the reference's spin-up leaves behind, main.f90:35-67). */
int bs_prime(struct bs_ctx* ctx);
/* The same without the time-step rule (integrator.f90:885-953): dt keeps the
 * parameters' value and umax stays 0 for the first step, as the reference's
 * own set-up leaves them (main.f90:23-37 calls no timestep before its loop;
 * initialize.f90:32,46). */
int bs_prime_setup(struct bs_ctx* ctx);
int bs_scalar_substep(struct bs_ctx* ctx);  /* scalart_anisotropic+scalarupdate, scalar.f90:242,364 */
int bs_projection(struct bs_ctx* ctx);      /* isph.f90:17                                   */
int bs_cellshift(struct bs_ctx* ctx, int32_t alt); /* integrator.f90:251 (alt=0) / 33 (alt=1); resetid isph.f90:88 */
int bs_search(struct bs_ctx* ctx);          /* neighbour/nsearch2, search.f90:13-399         */
int bs_porosity(struct bs_ctx* ctx);        /* effpor/porsearch, porous.f90:32-224           */
int bs_eddy(struct bs_ctx* ctx);            /* eddyvis, turbulence.f90:12                    */
int bs_int_vel(struct bs_ctx* ctx);         /* int_vel, integrator.f90:459                   */
int bs_ppe_assemble(struct bs_ctx* ctx);    /* ppesolve assembly, isph.f90:115-456           */
int bs_ppe_solve(struct bs_ctx* ctx);       /* bicgstab (solver.f90:129) + scatter isph.f90:468 */
int bs_comp_vel(struct bs_ctx* ctx);        /* comp_vel, integrator.f90:705                  */
int bs_comp_pos(struct bs_ctx* ctx);        /* comp_pos, integrator.f90:845                  */
int bs_free_surface(struct bs_ctx* ctx);    /* freesurf, isph.f90:49                         */
int bs_shift(struct bs_ctx* ctx);           /* opt2_shift, part_shift.f90:12                 */
int bs_density_update(struct bs_ctx* ctx);  /* densityupdate, scalar.f90:399                 */
int bs_timestep(struct bs_ctx* ctx);        /* timestep, integrator.f90:885                  */

/* Full production step (main.f90:199-272) with fused kernels, nsteps times. */
int bs_step(struct bs_ctx* ctx, int32_t nsteps);

/* The step with parts left out, as the reference's settling phases run it:
 * phase 1 (main.f90:39-67) with 0, phase 2 (main.f90:95-155) with
 * BS_STEP_BUFFERS; bs_step = BS_STEP_ALL. */
#define BS_STEP_SCALAR    0x1   /* scalar sub-steps at the start of the step          */
#define BS_STEP_BUFFERS   0x2   /* the buffer-zone schedule (bs_set_inflow)           */
#define BS_STEP_DENSITY   0x4   /* densityupdate after the shift                     */
#define BS_STEP_EDDY_END  0x8   /* eddyvis (and the dispersion) at the end of the step */
#define BS_STEP_ALL       0xf
int bs_step_flags(struct bs_ctx* ctx, int32_t nsteps, int32_t flags);
/* Overwrite vx, vy, p, mass, rho, oden, ovol, con (the non-NULL ones) of a
 * scene in place, in bs_download's particle order; st->n = the scene's
 * count.  The host edits of the reference's driver between its phases. */
int bs_set_fields(struct bs_ctx* ctx, int32_t scene, const bs_state* st);
/* Set a scene's time t (the reference restarts it at 0 for production). */
int bs_set_time(struct bs_ctx* ctx, int32_t scene, double t);

/* ---- WCSPH (wcsph.f90, a module the reference ships but does not call) --- */
int bs_wcsph_continuity(struct bs_ctx* ctx);   /* calmasscons, wcsph.f90:65-129: tden of fluid rows */
int bs_wcsph_update_density(struct bs_ctx* ctx); /* updateden, wcsph.f90:131-154: density = tden   */
int bs_wcsph_eos(struct bs_ctx* ctx);          /* dentopress, wcsph.f90:35-63: Tait pressure      */
int bs_wcsph_pressure_to_density(struct bs_ctx* ctx); /* presstoden, wcsph.f90:13-33              */
/* Wall and ghost pressure for the WCSPH step: Shepard average over fluid
 * neighbours of p_f + rho_f |g| (y_f - y_w).  No counterpart in the
 * reference, which has no WCSPH boundary treatment. */
int bs_wcsph_wall_pressure(struct bs_ctx* ctx);
/* WCSPH step, nsteps times: the production step of bs_step with the PPE
 * assembly and solve replaced by continuity + updateden + dentopress + wall
 * pressure, the density kept from the continuity equation (the porosity pass
 * and densityupdate leave it alone).  The reference has no WCSPH time loop;
 * this composition of its routines is this library's. */
int bs_wcsph_step(struct bs_ctx* ctx, int32_t nsteps);

/* Standalone BiCGStab on a CSR system (solver.f90:129-254 with the CSR
 * operator spmv, solver.f90:53-82) -- the solvertest.f90 driver's path.
 * Host arrays, 0-based row_ptr/col.  Returns iterations and relative residual. */
int bs_bicgstab_csr(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val,
                    const double* b, double* x, double tol, int32_t maxit, int32_t stop_rule,
                    int32_t* iters, double* relres);

/* Standalone restarted FGMRES on a CSR system: the Krylov method of the
 * reference's live PPE solve (fgmres, solver.f90:306-350, which calls MKL's
 * dfgmres with the spmv2 operator), unpreconditioned as there.  restart in
 * 1..150, maxit counts Arnoldi columns, stop_rule BS_STOP_RELRES or
 * BS_STOP_R0.  Host arrays, 0-based row_ptr/col. */
int bs_fgmres_csr(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val,
                  const double* b, double* x, double tol, int32_t maxit, int32_t restart,
                  int32_t stop_rule, int32_t* iters, double* relres);

/* No counterpart in the reference.  The same BiCGStab as bs_bicgstab_csr, but
 * on a CSR system already in device memory (0-based d_row_ptr[n+1], d_col,
 * d_val, d_b; d_x holds the initial guess and receives the solution) and
 * without allocating: for callers that cannot let a library call cudaMalloc
 * or cudaFree (hosts whose device memory belongs to their own pool allocator,
 * or code that must not stall on the implicit synchronisation of those
 * calls).  All solver scratch lives in a fixed ~3.2 MB device array inside the
 * library, which every GPU that loads the library holds until exit.  At most
 * 65,536 rows (larger n returns BS_E_CAPACITY).  The array is shared by all
 * calls: calls whose GPU work overlaps race, so serialise them.  The first call
 * on each device looks up the array's address (cudaGetSymbolAddress, that
 * device current); make it before any stream capture.  Convergence is judged
 * on the recursive residual, as in bs_bicgstab_csr; *relres is the true
 * residual ||b - A x|| / ||b|| after the last iteration; the convergence flag
 * is read back every four iterations (the call waits for `stream` there), so
 * the call must not be made on a stream that is being captured into a graph.
 * `stream` is a cudaStream_t (NULL: the default stream). */
int bs_bicgstab_csr_noalloc(int32_t n, const int32_t* d_row_ptr, const int32_t* d_col, const double* d_val,
                            const double* d_b, double* d_x, double tol, int32_t maxit, void* stream,
                            int32_t* iters, double* relres);

/* ---- timing: CUDA events recorded on the context's stream ------------------ */
int bs_event_record(struct bs_ctx* ctx, int32_t slot);
int bs_event_elapsed_ms(struct bs_ctx* ctx, int32_t slot0, int32_t slot1, float* ms);
/* per-kernel timing: mask = one bit per kernel id (bs_kernel_timing_get
 * gives the name of each id), ~0 for all, 0 to stop; totals are reset. */
int bs_kernel_timing(struct bs_ctx* ctx, uint64_t mask);
int bs_kernel_timing_get(struct bs_ctx* ctx, int32_t idx, const char** name, int32_t* launches,
                         double* total_ms);
/* count of kernels launched by the library since context creation */
int64_t bs_launch_count(struct bs_ctx* ctx);

/* No counterpart in the reference (admission of requests by free device
 * memory): free and total bytes of the current device (cudaMemGetInfo), and
 * the device bytes a context holds (its particle, neighbour, matrix,
 * multigrid and Krylov arrays; the FGMRES basis is allocated at the first
 * FGMRES solve and counted from then on). */
int bs_device_memory(size_t* free_bytes, size_t* total_bytes);
int bs_context_bytes(struct bs_ctx* ctx, size_t* bytes);

/* No counterpart in the reference: a measurement helper for the roofline.
 * FP64 rate of the current device in TFLOP/s, from chains of dependent
 * fused multiply-adds on every SM (best of five timed launches, ~0.5 s). */
int bs_measure_fp64_peak(double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* BEACHSLOPE_H */
