/*
 * bs_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU FP64 restatement of the reference ISPH step (Sinchanrc/Beach-Slope,
 * Fortran).  It is the parity checker for the CUDA library and the timed CPU
 * baseline; nothing in the product links it.  Only tests/, the smoke check
 * and bench.py's cpu_baseline / reference legs may load it.
 *
 * Parity status: pinned by the reference's only known-answer test
 * (solvertest.f90:10-19, 5x5 system -> x=(1,2,3,4,5)) and by analytic
 * identities of the kernel, inverse and porosity routines; the rest is
 * parity against this restatement (the Fortran reference cannot be compiled
 * here: no Fortran compiler, no MKL).
 */
#ifndef BS_ORACLE_H
#define BS_ORACLE_H
#include "../include/beachslope.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_scene or_scene;

/* stage ids for or_stage (one per reference subroutine) */
enum {
    OR_PROJECTION = 1, OR_CELLSHIFT, OR_CELLSHIFTALT, OR_RESETID, OR_NEIGHBOUR,
    OR_EFFPOR, OR_EDDYVIS, OR_INT_VEL, OR_PPE_ASSEMBLE, OR_PPE_SOLVE, OR_COMP_VEL,
    OR_COMP_POS, OR_FREESURF, OR_OPT2_SHIFT, OR_DENSITYUPDATE, OR_TIMESTEP,
    OR_SCALAR_SUBSTEP, OR_PRIME,
    /* wcsph.f90 */
    OR_CALMASSCONS, OR_UPDATEDEN, OR_DENTOPRESS, OR_PRESSTODEN,
    OR_WALL_PRESSURE,   /* the WCSPH step's wall rule (no reference counterpart) */
    OR_EFFPOR_KEEP,     /* effpor without its density write (WCSPH step)        */
    OR_BOUN_VEL,        /* boun_vel, integrator.f90:394-457 (never called)      */
    OR_GHOST,           /* comp_ghost + ghost_en, mls.f90:114-263 (Shepard)     */
    OR_GHOST_MLS,       /* the same with the MLS branch for the velocity        */
    OR_PRIME_SETUP      /* prime without the time-step rule: dt and umax keep
                           their initial values, as after main.f90:23-37        */
};

or_scene* or_create(const bs_params* p, const bs_state* st, const bs_grains* gr);
void or_destroy(or_scene* s);
int or_n(or_scene* s);
void or_set_threads(int nthreads);
int or_get_threads(void);
int or_get(or_scene* s, bs_state* out);
int or_info(or_scene* s, bs_scene_info* out);
int or_neighbours(or_scene* s, int32_t kmax, int32_t* counts, int32_t* idx,
                  double* dist, double* kx, double* ky);
int or_matrix(or_scene* s, int32_t kmax, double* diag, double* off, double* rhs);
int or_stage(or_scene* s, int32_t stage);
int or_ppe_solve(or_scene* s, double tol, int32_t maxit, int32_t rule,
                 int32_t* iters, double* relres);
/* fgmres, solver.f90:306-350: restarted GMRES (rule 0: ||r||/||b||, else ||r||/||r0||) */
int or_ppe_fgmres(or_scene* s, double tol, int32_t maxit, int32_t restart, int32_t rule,
                  int32_t* iters, double* relres);
int or_fgmres_csr(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val,
                  const double* b, double* x, double tol, int32_t maxit, int32_t restart,
                  int32_t rule, int32_t* iters, double* relres);
int or_step(or_scene* s, int32_t nsteps);
/* the step with parts left out (BS_STEP_* flags, main.f90:39-67, 95-155) */
int or_step_flags(or_scene* s, int32_t nsteps, int32_t flags);
int or_set_fields(or_scene* s, const bs_state* st);
int or_set_time(or_scene* s, double t);
/* coll_pos_shift (mode 0) / coll_shift (mode 1), part_shift.f90:193-410;
 * prx, pry, brx, bry: the half particle spacings prrealx, prrealy, brrealx,
 * brrealy the routines read */
int or_collision_shift(or_scene* s, int32_t mode, double prx, double pry, double brx, double bry);
int or_wcsph_step(or_scene* s, int32_t nsteps);
/* combined, output.f90:188-222 (fluid / buffer text files) */
int or_write_combined(or_scene* s, const char* fluid_path, const char* buffer_path);
/* overwrite pressures (used to pin a common PPE guess in tests) */
int or_set_pressure(or_scene* s, const double* p);
/* open-boundary buffer zones (internal.f90:447-586, main.f90:218-234) */
int or_set_inflow(or_scene* s, int32_t zone, const bs_inflow* z);
int or_buffer_exchange(or_scene* s, int32_t zone);
int or_bicgstab_csr(int32_t n, const int32_t* row_ptr, const int32_t* col, const double* val,
                    const double* b, double* x, double tol, int32_t maxit, int32_t rule,
                    int32_t* iters, double* relres);
/* kernel functions for unit tests (kernel.f90:34-162, functions.f90:62-96) */
double or_Wab(double r, double h);
double or_Wo(double h);
void or_gradW(double xj, double yj, double xi, double yi, double r, double h,
              double* wx, double* wy);
void or_invert2(double* a4);
double or_vis(double oden);

#ifdef __cplusplus
}
#endif
#endif
