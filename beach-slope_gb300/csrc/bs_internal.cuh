// bs_internal.cuh -- device data layout and shared device helpers.
//
// Layout in HBM (one context = a batch of scenes):
//  * particle rows: SoA arrays over all scenes; scene s owns rows
//    [row0[s], row0[s] + cap[s]), cap a multiple of BS_ALIGN so that a
//    256-thread block never straddles two scenes; rows beyond n[s] are idle.
//    Inside a scene rows are kept sorted by cell key (column-major over
//    cells, as resetid numbers them, isph.f90:97-108), walls first in a
//    cell, then fluid in the reference's slot order (integrator.f90:319-387).
//  * neighbour lists: sliced ELL, slice = 32 rows, kmax entries per row,
//    element (row,k) at ((row/32)*kmax + k)*32 + row%32, so a warp reading
//    the k-th neighbour of its 32 rows issues one coalesced request.
//  * PPE matrix: values aligned with the neighbour list (the list is the
//    column array), a per-row diagonal (1 after Jacobi scaling except the
//    reference's leftover-entry rows), right-hand side.
//  * cells: per-scene grids concatenated; cell_start/cell_end rows.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/beachslope.h"

#define BS_ALIGN 256
#define BS_THREADS 256
#define BS_NCAT 10      // bucket categories per cell in the re-bin (see k_rank)
#define BS_MAXDOT 8     // partial sums per block in the solver
#define BS_SCAN_CHUNK 1024  // cells per block of the re-bin's cell scan
#define BS_FG_MAXM 150  // longest FGMRES restart cycle (the reference's MKL default)

// constants with the reference's literal precision (default REAL = single)
#define BS_C28 ((double)(28.0f * 3.14f))   // kernel.f90:61
#define BS_C3 ((double)(3.0f * 3.14f))     // kernel.f90:62
#define BS_SP1EM5 ((double)1e-5f)          // functions.f90:75, solver.f90:235
#define BS_SP1EM6 ((double)1e-6f)          // integrator.f90:581
#define BS_SP1EM9 ((double)1e-9f)          // scalar.f90:246 (Dm)

struct ScenePar {                 // per-scene constants
    double h, twoh, lam, dl, cw;  // cw = 4h cell width (setup.f90:51, incr=4)
    double inv_h, inv_h2, inv_h3;
    double cn1, cn2;              // alp*10/(C28 h^2), (1-alp)/(C3 h^2)
    double wo;                    // Wo(h)
    double rho, rhomin, rhomax, rel_den, g, mu, tschmidt;
    double por, lamk, d50;
    double freethr;               // lamfs*maxdivr
    double csh, maxshift, sig1;
    double xlcutoff, ytcutoff;
    double buf_lo, buf_hi;        // comp_pos buffer release window (integrator.f90:865-872)
    double ppe_tol, inner_tol;
    double wc_c0, wc_gamma, wc_delta, wc_ysurf;   // WCSPH (wcsph.f90)
    int wc_form, wc_pad;
    int cellx, celly, ncell, cell0;   // grid dims and first global cell
    int row0, cap, kmax, maxit;
    int adaptive_dt, scalar_on, precision, stop_rule;
    int nblk, blk0, max_outer, mg_lev;   // mg_lev: this scene's coarsest multigrid level
    int grp0, pad_grp;                    // first group of 32 row blocks (two-level reductions)
    // the kernel gradient on the FP32 pipe as F = kq_s g(q), q = r/h:
    // kq_s = fl32(cn1/h^2), (hi, lo) pairs of cn2/cn1, 3 (1 + cn2/cn1) and lam
    float kq_s, kq_rho_h, kq_rho_l, kq_k3_h, kq_k3_l, kq_lam_h, kq_lam_l, kq_pad;
};

struct SceneDyn {                 // per-scene dynamic state (device)
    int n, solsteps, lost, n_prev;
    double t, dt, dtsol, umax, numax;
    // solver scalars
    double rho_old, alpha, omega, beta, rhonew;
    double bnorm2, rnorm2, relres, rtrue2;
    int iters, converged, breakdown, outer;
    unsigned err;
    int hold;                      // 1: row sweeps and timestep leave the scene alone (bs_prime_scene)
    double part_tmp;
    // FGMRES: Arnoldi column of the current cycle, cycle state (0 running,
    // 1 restart, 2 converged, 3 iteration cap) and the columns the update applies
    int fg_j, fg_state, fg_k;
    int asm_split;                 // 1: the mixed assembly wrote aval32/aval_lo with aval (k_mx_convert skips the split)
    double fg_rinv;                // 1 / the norm of the vector the next column normalises
};

// Aggregation multigrid over the cell grid.  Level 1 = half-cells (2h x 2h,
// the four quadrants of a search cell: one aggregate of ~7 rows), level 2 =
// the cells, level l+1 = 2x2 boxes of level l; 9-point Galerkin stencils
// stored per offset k = (dj+1)*3 + (di+1): A[k*n + c].  Levels 1..wlev
// visit the next level twice (W-cycle), deeper levels once (V-cycle).
#define BS_MG_MAXL 16
struct MgDev {
    int nlev;                         // coarsest level index (levels 1..nlev)
    int n[BS_MG_MAXL + 1];            // cells of level l over all scenes
    void* A[BS_MG_MAXL + 1];          // 9*n[l] (double or float)
    void* dinv[BS_MG_MAXL + 1];       // 1/diag (0 for empty rows)
    void* r[BS_MG_MAXL + 1];
    void* z[BS_MG_MAXL + 1];
    const int* scene_of[BS_MG_MAXL + 1];
    const int* off[BS_MG_MAXL + 1];   // per scene: first cell of the scene in level l
    const int* nx[BS_MG_MAXL + 1];    // per scene
    const int* ny[BS_MG_MAXL + 1];
    void* dinv0;                      // level 0: 1/adiag per particle row
    void* adiagT;                     // level 0: adiag in the V-cycle's precision
    void* xin;                        // level 0: V-cycle input in its precision
    void* u;                          // level 0: w * xin / adiag (pre-smoothing from zero)
    void* zz;                         // level 0: u + cscale * e1[cell]  (after the coarse correction)
    double omega, cscale;
    int coarse_sweeps, coarse_max;
    int pre0, prec;                   // pre-smoothing at level 0 / on the cell levels (0 or 1)
    int wlev;                         // levels 1..wlev recurse twice
    int post0;                        // level-0 post-sweeps (1 or 2)
    uint8_t* sub;                     // level 0: quadrant of the row in its cell (bit0 lower, bit1 right)
    int* agg1;                        // level 0: global level-1 index of the row's half-cell
    // exact coarse solve (option mg_exact): each scene's hierarchy ends at
    // its first level of at most BS_MG_EXACT_MAX cells, whose operator is
    // inverted once per step; the visits apply the inverse
    int exact;
    void* ainv;                       // per scene: BS_MG_EXACT_MAX^2 values (the level's precision), row-major
    double* xinv;                     // per scene: BS_MG_EXACT_MAX^2 doubles (the factorisation's work space)
};
#define BS_MG_EXACT_MAX 1024          // cells of an exactly solved level
#define BS_MG_EXACT_BAND 20480        // band entries (doubles, shared memory) of its LU factors

// One cell level's per-scene tables, passed to the level kernels by value
// (__grid_constant__): scene k owns cells [off[k], off[k+1]) of the level, a
// nx[k] x ny[k] grid (empty range if the scene is coarser than the level).
#define BS_MG_MAXS 64
struct MgLevel {
    int l, n, ns;              // level, cells over all scenes, scenes
    int off[BS_MG_MAXS + 1];
    int nx[BS_MG_MAXS], ny[BS_MG_MAXS];
    int lev[BS_MG_MAXS];       // the scene's coarsest level
};
// Per scene, the level solved exactly (0: none) and its grid and offset
struct MgExact {
    int ns;
    int l[BS_MG_MAXS], off[BS_MG_MAXS], nx[BS_MG_MAXS], ny[BS_MG_MAXS];
};

// device pointers of one context (passed by value to kernels)
struct Dev {
    // particle fields (current buffer)
    double *x, *y, *xs, *ys, *vx, *vy, *vxs, *vys, *p, *mass, *rho, *oden, *ovol, *con;
    float *xr, *yr;                 // position relative to the row's cell corner (xleft, ybot), FP32
    float4* pos4;                   // mixed: position as (x hi, x lo, y hi, y lo) FP32 pairs (f2_split2),
                                    // written by k_relpos and by the packs of the sweeps that read it (k_quot)
    double *vol, *nu;               // derived: m/rho, vis(oden)/oden
    int8_t* tid;
    uint8_t* flags;
    int* pid;
    int* cell;                      // global cell index of the row
    // particle fields (alternate buffer, permute target)
    double *x2, *y2, *xs2, *ys2, *vx2, *vy2, *vxs2, *vys2, *p2, *mass2, *rho2, *oden2, *ovol2, *con2;
    double *vol2, *nu2;
    int8_t* tid2;
    uint8_t* flags2;
    int* pid2;
    int* cell2;
    // per-particle properties (recomputed after every re-bin)
    double *por, *resx, *resy, *nut, *tke, *varts, *gradvx, *vel, *cdiff;
    double *c0, *c1, *c2, *c3;      // coff (L^-1), search.f90:276-278
    float4 *cfa, *cfb;              // mixed: the same as (hi, lo) FP32 pairs, (c0, c1) and (c2, c3), written by k_search
    double *Dp0, *Dp1, *Dp2, *Dp3, *Dt;   // scalar dispersion per particle
    double *rho_new, *vol_new;      // effpor output (ping-pong with rho/vol)
    double *tden, *whyd;            // WCSPH: continuity density, hydrostatic Tait density per row
    double *qa, *qu, *qw, *qi;      // per-row quotients of the sweeps (k_quot): rho/phi, u/phi, w/phi, 1/phi
    // mixed: what a neighbour sweep reads of a row's neighbours, packed per
    // row by k_quot right before the sweep (the layout of each sweep is at
    // k_quot); fields whose pair differences cancel as (hi, lo) FP32 pairs
    float4 *rec0, *rec1, *rec2;
    float2* volf2;                  // mixed: volume as an (hi, lo) FP32 pair, written by k_relpos for k_search
    double *con_new;
    // neighbour lists (ELL)
    int* ncount;
    int* nidx;
    void *ndist, *nrinv, *nkx, *nky;   // double (FP64) or float (mixed)
    // PPE
    void* aval;                     // ELL values (double or float hi)
    float* aval32;                  // mixed: FP32 copy of the values (inner operator)
    float* aval_lo;                 // mixed: value - aval32 in FP32 (aval32 + aval_lo: 48 bits)
    float* zf;                      // mixed: the V-cycle output in FP32 (it is FP32-exact)
    double *adiag, *rhs;
    double *sx, *sr, *srhat, *sp, *sp2, *sv, *sv2, *ss, *st, *sxd;  // solver vectors
    float *fr, *fp, *fp2, *fv, *fv2, *fs, *ft, *fd, *frhat;          // mixed inner vectors
    // per-scene
    const ScenePar* par;
    SceneDyn* dyn;
    const int* blk_scene;           // row block -> scene
    const int* cell_scene;          // global cell -> scene
    int* blk_done;                  // per-scene block counters for finisher reductions
    double* part;                   // per-block partial sums [nblk_total][BS_MAXDOT]
    // FGMRES (ppe_solver = BS_SOLVER_FGMRES): Krylov basis V [(m+1) x rows],
    // preconditioned basis Z [m x rows], partials per block and per group of
    // 32 blocks [.. x (2m+4)], per-scene Hessenberg and Gram matrices,
    // rotations and right-hand side [nscene x fg_small]
    double *fg_V, *fg_Z, *fg_part, *fg_gpart, *fg_small;
    int* fg_gdone;                  // per-group block counters
    int fg_m, fg_small_n, fg_ld;    // restart length, doubles per scene, rows per basis vector
    int fg_df;                      // 1: basis stored as (hi, lo) FP32 pairs, dots on the FP32 pipe
    // open-boundary buffer zones: per global cell, the zone bits of the entry
    // cells and, per zone, the cell's template range [zstart, zstart + zcount)
    uint8_t* czone;
    int *zstart[2], *zcount[2];
    // cells
    int *cell_start, *cell_end, *cell_start2, *cell_end2;
    int* bucket;                    // [ncell_total*BS_NCAT] counts then starts
    int* cell_total;                // [ncell_total]
    int* coderank;                  // per row: code<<24 | rank
    double *cell_maxvel, *cell_maxeddy;
    int* scan_part;                 // per scene x chunk of BS_SCAN_CHUNK cells: the chunk's row total (re-bin scan)
    int scan_chunks;                // chunks of the scene with the most cells
    unsigned long long* scene_max;  // per scene: the timestep rule's |vel| and |nut| maxima (bit patterns), k_scene_max
    // grains (static, sorted by cell)
    double *gx, *gy, *gv;           // gv = mass/density
    float *gxr, *gyr;               // grain position relative to its cell corner, FP32
    float4* gpos4;                  // grain position as (x hi, x lo, y hi, y lo) FP32 pairs
    int *gcell_start, *gcell_end;
    int ncell_total, nrow_total, nblk_total, nscene;
    int kmax;
    unsigned* err_word;
    MgDev mg;
    struct LoopCtl* loop;           // device-side loop counters of the captured step (bs_graph)
};

// Counters of the device-side loops of a captured step: the scalar sub-step
// pairs, BiCGStab iterations, FGMRES restart cycles and columns, and the
// kernels the loop bodies launched (for the launch count).
struct LoopCtl {
    int j, it, cycle, col;
    unsigned long long kernels;
};

// ------------------------------------------------------------ helpers
__device__ __forceinline__ long ell(int row, int k, int kmax) {
    return ((long)(row >> 5) * kmax + k) * 32 + (row & 31);
}

// cell bounds exactly as setup.f90:120-123 (local 1-based i,j)
__device__ __forceinline__ double cell_xleft(const ScenePar& P, int j) { return (double)(j - 2) * (4.0 * P.h); }
__device__ __forceinline__ double cell_xright(const ScenePar& P, int j) { return (double)(j - 1) * (4.0 * P.h); }
__device__ __forceinline__ double cell_ybot(const ScenePar& P, int i) { return (double)(-i + P.celly - 1) * (4.0 * P.h); }
__device__ __forceinline__ double cell_ytop(const ScenePar& P, int i) { return (double)(-i + P.celly) * (4.0 * P.h); }

// Hybrid kernel value W(r) (kernel.f90:34-66)
__device__ __forceinline__ double bs_W(double r, const ScenePar& P) {
    const double q = r * P.inv_h;
    double t1, t2;
    if (r < P.h) {
        t1 = 4.0 - 6.0 * q * q + 3.0 * q * q * q;
        t2 = q * q * q - 6.0 * q + 6.0;
    } else {
        const double a = 2.0 - q;
        t1 = a * a * a;
        t2 = t1;
    }
    return P.cn1 * t1 + P.cn2 * t2;
}

// The kernel's constants in FP32, converted once per row (a conversion from
// FP64 issues on the FP64 pipe)
struct KerF {
    float h, ih, ih2, ih3, c1, c2;
};
__device__ __forceinline__ KerF ker_f(const ScenePar& P) {
    KerF K;
    K.h = (float)P.h;
    K.ih = (float)P.inv_h;
    K.ih2 = (float)P.inv_h2;
    K.ih3 = (float)P.inv_h3;
    K.c1 = (float)P.cn1;
    K.c2 = (float)P.cn2;
    return K;
}
__device__ __forceinline__ float bs_Wf(float r, const KerF& K) {
    const float q = r * K.ih;
    float t1, t2;
    if (r < K.h) {
        t1 = 4.0f - 6.0f * q * q + 3.0f * q * q * q;
        t2 = q * q * q - 6.0f * q + 6.0f;
    } else {
        const float a = 2.0f - q;
        t1 = a * a * a;
        t2 = t1;
    }
    return K.c1 * t1 + K.c2 * t2;
}

// r = sqrt(s) and 1/r in FP64 from an FP32 rsqrt seed and one Newton step
// (relative error ~1e-13: far below the FP32 rounding of the stored pair
// values, not correctly rounded): used where the exact IEEE sqrt is not
// required (mixed-mode pair quantities, grain distances).
__device__ __forceinline__ void fast_r64(double s, double& r, double& ir) {
    double y = (double)rsqrtf((float)s);
    y = y * (1.5 - 0.5 * s * y * y);
    ir = y;
    r = s * y;
}
// Compensated FP32 sum (Neumaier's variant of Kahan summation): the running
// error term keeps the sum of n terms within ~1 ulp instead of ~n/2 ulp.
struct Kahan32 {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float t = __fadd_rn(s, x);
        c = __fadd_rn(c, fabsf(s) >= fabsf(x) ? __fadd_rn(__fsub_rn(s, t), x) : __fadd_rn(__fsub_rn(x, t), s));
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// 1/d in FP64 from an FP32 reciprocal seed and one Newton step (~1e-14)
__device__ __forceinline__ double fast_rcp64(double d) {
    double y = (double)__frcp_rn((float)d);
    y = y * (2.0 - d * y);
    return y;
}

// ---------------------------------------------------- pair offsets on the FP32 pipe
// The mixed form's neighbour sweeps take the pair offset x_j - x_i and the
// pair distance from double-float positions (a value as hi + lo, two FP32
// numbers; Dekker 1971, Knuth's TwoSum) instead of FP64 arithmetic: on this
// part the FP64 pipe issues 2 lanes per clock per SM against 128 for FP32, and
// one FP64 instruction per pair costs as much as ~60 FP32 ones.  Every
// rounding is explicit (no contraction).

// a + b = s + e exactly
__device__ __forceinline__ float2 f2_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}
// a + b = s + e exactly, for |a| >= |b|
__device__ __forceinline__ float2 f2_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
// (hi, lo) of a double: hi = fl32(v), lo = fl32(v - hi); |v - hi - lo| <= 2^-48 |v|
__device__ __forceinline__ float2 f2_split(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(__dsub_rn(v, (double)h)));
}
// two doubles as (x hi, x lo, y hi, y lo): a position, a velocity, a pair
// of quotients
__device__ __forceinline__ float4 f2_split2(double x, double y) {
    const float2 a = f2_split(x), b = f2_split(y);
    return make_float4(a.x, a.y, b.x, b.y);
}
// b - a of two double-float values, renormalised (.x = fl32 of the
// difference): the hi parts subtracted exactly, the lo parts added; absolute
// error within ~2^-46 max(|a|, |b|) (1e-13 m for positions on a 4 m domain)
__device__ __forceinline__ float2 f2_diff(float bh, float bl, float ah, float al) {
    const float2 s = f2_two_sum(bh, -ah);
    return f2_two_sum(s.x, __fadd_rn(s.y, __fsub_rn(bl, al)));
}
// Pair distance from a double-float offset (dx, dy): s = dx^2 + dy^2 as
// double-float (TwoProduct by FMA), r = sqrt(s) as (rh, rl) by one Newton
// step from the FP32 reciprocal square root y (r = r0 + (s - r0^2) y / 2,
// r0 = fl(s y); the residual s - r0^2 exact by Sterbenz and FMA), and 1/r
// by one Newton step y (1 + (1 - r y)).  rh = fl32(r) and ir = fl32(1/r)
// up to ties (relative error of r before rounding ~2^-44); s = sh + sl.
struct PairR {
    float rh, rl, ir, sh, sl;
};
__device__ __forceinline__ PairR pair_r(float2 dx, float2 dy) {
    const float p1 = __fmul_rn(dx.x, dx.x);
    const float e1 = __fmaf_rn(__fmul_rn(2.0f, dx.x), dx.y, __fmaf_rn(dx.x, dx.x, -p1));
    const float p2 = __fmul_rn(dy.x, dy.x);
    const float e2 = __fmaf_rn(__fmul_rn(2.0f, dy.x), dy.y, __fmaf_rn(dy.x, dy.x, -p2));
    const float2 s0 = f2_two_sum(p1, p2);
    const float2 s = f2_fast_two_sum(s0.x, __fadd_rn(s0.y, __fadd_rn(e1, e2)));
    const float y = rsqrtf(s.x);
    const float r0 = __fmul_rn(s.x, y);
    const float q = __fmul_rn(r0, r0);
    const float d = __fadd_rn(__fsub_rn(__fsub_rn(s.x, q), __fmaf_rn(r0, r0, -q)), s.y);
    const float2 r = f2_fast_two_sum(r0, __fmul_rn(d, __fmul_rn(0.5f, y)));
    const float t = __fmaf_rn(-r.y, y, __fmaf_rn(-r.x, y, 1.0f));
    PairR o;
    o.rh = r.x;
    o.rl = r.y;
    o.ir = __fmaf_rn(y, t, y);
    o.sh = s.x;
    o.sl = s.y;
    return o;
}
// r < c for a double-float r and a double c given as (ch, cl)
__device__ __forceinline__ bool f2_less(float rh, float rl, float ch, float cl) {
    return rh < ch || (rh == ch && rl < cl);
}
// Double-float arithmetic on (hi, lo) pairs (relative error ~2^-44; the
// lo * lo terms are below it)
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return f2_fast_two_sum(p, e);
}
__device__ __forceinline__ float2 f2_mulf(float2 a, float b) {
    const float p = __fmul_rn(a.x, b);
    return f2_fast_two_sum(p, __fmaf_rn(a.y, b, __fmaf_rn(a.x, b, -p)));
}
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) {
    const float2 s = f2_two_sum(a.x, b.x);
    return f2_fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}
// 1/a by one Newton step from the FP32 reciprocal
__device__ __forceinline__ float2 f2_rcp(float2 a) {
    const float y = __frcp_rn(a.x);
    const float e = __fmaf_rn(-a.y, y, __fmaf_rn(-a.x, y, 1.0f));
    return f2_fast_two_sum(y, __fmul_rn(y, e));
}
// a += (kh + kl)(rh + re) for a double-float accumulator a and two
// double-float factors: the product's rounding error kept in the lo part
__device__ __forceinline__ void f2_acc_prod(float2& a, float2 k, float rh, float re) {
    const float th = __fmul_rn(k.x, rh);
    const float te = __fmaf_rn(k.y, rh, __fmaf_rn(k.x, re, __fmaf_rn(k.x, rh, -th)));
    const float2 t = f2_two_sum(a.x, th);
    a.x = t.x;
    a.y = __fadd_rn(a.y, __fadd_rn(t.y, te));
}

// Radial factor F(r) of the hybrid-kernel gradient: grad_i W_ij = F(r) (r_i - r_j)
// (kernel.f90:94-162: Wabx(p1=j, p2=i) = F * (p2%x - p1%x)).
__device__ __forceinline__ double bs_F(double r, const ScenePar& P) {
    if (r < P.h) {
        const double t1 = 9.0 * r * P.inv_h3 - 12.0 * P.inv_h2;
        const double t2 = 3.0 * r * P.inv_h3 - 6.0 * P.inv_h / r;
        return P.cn1 * t1 + P.cn2 * t2;
    }
    const double a = 2.0 - r * P.inv_h;
    const double c = (3.0 * P.inv_h / r) * a * a;
    return -(P.cn1 + P.cn2) * c;
}
__device__ __forceinline__ float bs_Ff(float r, const KerF& K) {
    if (r < K.h) {
        const float t1 = 9.0f * r * K.ih3 - 12.0f * K.ih2;
        const float t2 = 3.0f * r * K.ih3 - 6.0f * K.ih / r;
        return K.c1 * t1 + K.c2 * t2;
    }
    const float a = 2.0f - r * K.ih;
    const float c = (3.0f * K.ih / r) * a * a;
    return -(K.c1 + K.c2) * c;
}

// viscosity (integrator.f90:12-30)
__device__ __forceinline__ double bs_vis(double oden) {
    const double Sp = oden - 1000.0;
    return (1.002 + 0.001652 * Sp + 0.0000083 * (Sp * Sp)) * 0.001;
}

// A row's gradient-correction matrix C as (hi, lo) pairs for the FP32 pipe:
// a corrected gradient component c_a z1 + c_b z2 with the lo parts added, so
// that its one FP32 error is the rounding of the pair's own value.  C rounded
// to FP32 once per row would give every pair of the row the same relative
// error, which the row's sums (divergences, matrix entries) carry whole.
struct CorrF {
    float c0h, c0l, c1h, c1l, c2h, c2l, c3h, c3l;
    __device__ __forceinline__ float lx(float z1, float z2) const {
        return __fmaf_rn(c0h, z1, __fmaf_rn(c1h, z2, __fmaf_rn(c0l, z1, __fmul_rn(c1l, z2))));
    }
    __device__ __forceinline__ float ly(float z1, float z2) const {
        return __fmaf_rn(c2h, z1, __fmaf_rn(c3h, z2, __fmaf_rn(c2l, z1, __fmul_rn(c3l, z2))));
    }
    // the same components as (hi, lo) pairs
    __device__ __forceinline__ float2 lx2(float z1, float z2) const { return comp(c0h, c0l, c1h, c1l, z1, z2); }
    __device__ __forceinline__ float2 ly2(float z1, float z2) const { return comp(c2h, c2l, c3h, c3l, z1, z2); }
    __device__ __forceinline__ static float2 comp(float ah, float al, float bh, float bl, float z1, float z2) {
        const float p1 = __fmul_rn(ah, z1), p2 = __fmul_rn(bh, z2);
        const float2 s = f2_two_sum(p1, p2);
        float lo = __fmaf_rn(ah, z1, -p1);
        lo = __fadd_rn(lo, __fmaf_rn(bh, z2, -p2));
        lo = __fmaf_rn(al, z1, __fmaf_rn(bl, z2, __fadd_rn(lo, s.y)));
        return f2_fast_two_sum(s.x, lo);
    }
};
// C of row r from the (hi, lo) pairs the mixed search writes
__device__ __forceinline__ CorrF corr_f(const Dev& D, int r) {
    const float4 a = __ldg(D.cfa + r), b = __ldg(D.cfb + r);
    return CorrF{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}

__device__ __forceinline__ void set_err(const Dev& D, int s, unsigned bits) {
    atomicOr(&D.dyn[s].err, bits);
    atomicOr(D.err_word, bits);
}

// block reductions (BS_THREADS threads)
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh /*[NV*32]*/) {
#pragma unroll
    for (int q = 0; q < NV; ++q)
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[q * 32 + w] = v[q];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double a = (l < (int)(blockDim.x >> 5)) ? sh[q * 32 + l] : 0.0;
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            v[q] = a;
        }
    }
}

template <int NV>
__device__ __forceinline__ void block_max(double (&v)[NV], double* sh) {
#pragma unroll
    for (int q = 0; q < NV; ++q)
        for (int o = 16; o > 0; o >>= 1) v[q] = fmax(v[q], __shfl_xor_sync(0xffffffffu, v[q], o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[q * 32 + w] = v[q];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double a = (l < (int)(blockDim.x >> 5)) ? sh[q * 32 + l] : 0.0;
            for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
            v[q] = a;
        }
    }
}

// ---------------------------------------------------------- launchers
// (defined in the kernel translation units, called by the host code)
namespace bs {
// kernel ids for the per-kernel event timer
enum KId {
    K_RANK = 0, K_CELLPREFIX, K_SCANCELLS, K_PERMUTE, K_SEARCH, K_FREESURF, K_EDDY, K_INTVEL,
    K_ASSEMBLE, K_COMPVEL, K_CELLMAX, K_TIMESTEP, K_SHIFT, K_APPLY, K_DISP, K_SCALAR,
    K_BICG_INIT, K_BICG_IT1, K_BICG_IT2, K_BICG_IT3, K_TRUERES, K_ADVANCE, K_DERIVE, K_VELMAG,
    K_PROJECTION, K_MX_INIT, K_MX_IT1, K_MX_IT2, K_MX_IT3, K_MX_RES, K_MX_CONV, K_BICG_PUPD, K_BICG_SUPD,
    K_MX_UPD, K_MG_GAL0, K_MG_GALC, K_MG_L0DOWN, K_MG_DOWN, K_MG_COARSE, K_MG_UP, K_MG_L0UP, K_MG_PROLONG,
    K_MG_RESID, K_RELPOS, K_WC_CONT, K_WC_ROWS, K_WC_WALLP, K_FG_START, K_FG_PUT, K_FG_ARN, K_FG_ORTH, K_FG_UPD, K_BUFX, K_GHOST, K_MG_SUB, K_COLL, K_MG_L0REST, K_MG_TAIL, K_COUNT
};
extern const char* const kernel_names[K_COUNT];
struct KTimer {
    unsigned long long mask = 0;
    static const int NEV = 8192;   // event pool: NEV/2 launch slots used as a ring
    cudaEvent_t ev[NEV];
    int id_of[NEV / 2];
    long long head = 0, tail = 0;  // slots [tail, head) are pending
    bool ready = false;
    double total_ms[K_COUNT] = {};
    long long count[K_COUNT] = {};
};
// A captured chunk of BiCGStab iterations, re-used while the device data match.
struct IterGraph {
    cudaGraphExec_t exec = nullptr;
    Dev key;
    int precond = -1, prec = -1, chunk = 0, solver = -1;
    int64_t nkernels = 0;
    bool valid = false;
};
// The multigrid levels from `l0` down as one clustered launch per visit:
// the op list of the visit (built on the host from the cycle's recursion)
// and the tables of the levels it touches.
#define BS_MG_SUBL 8
#define BS_MG_MAXOPS 128
struct MgSub {
    int l0, nops;
    unsigned char op[BS_MG_MAXOPS], lv[BS_MG_MAXOPS], acc[BS_MG_MAXOPS];   // op: 0 down, 1 resid, 2 up, 3 coarse
    MgLevel G[BS_MG_SUBL];           // levels l0 .. l0 + BS_MG_SUBL - 1
};
struct Launch {
    cudaStream_t stream;
    int nblk_rows;      // total row blocks
    int ncell_total;
    int64_t* launches;  // launch counter
    KTimer* timer;
    IterGraph* graph;   // nullptr: launch kernels one by one
    const MgLevel* mglev;          // host tables of the multigrid levels, indexed by level
    const unsigned char* mgneed;   // per level: bit0 some scene visits it, bit1 restriction and
                                   // prolongation to the next level, bit2 coarsest-level solve
    int mgsub_level, mgsub_cs;     // first level of the clustered subtree (0: per-level launches), CTAs per cluster
    int mgtail;                    // level whose visits run with the coarsest level in one block (0: none)
    int sweep_tpb;                 // threads per block of the neighbour sweeps (64, 128 or 256)
    int mg0_tpb;                   // threads per block of the particle-level multigrid kernels
    const MgExact* exact;          // the scenes' exactly solved levels (when D.mg.exact)
};
// blocks of `tpb` threads over the rows of a batch (scenes own multiples of
// BS_ALIGN rows, so a block never straddles two scenes for tpb | BS_ALIGN)
inline unsigned row_blocks(const Launch& L, int tpb) { return (unsigned)(L.nblk_rows * (BS_THREADS / tpb)); }
// Programmatic dependent launch: a kernel launched by launch_pdl may be
// scheduled while its predecessor in the stream still runs.  Its first
// statement must be BS_PDL_ENTRY(): wait for the predecessor grid to finish
// (its memory visible), then allow the successor to be scheduled.  Without
// the launch attribute both instructions are no-ops.
#define BS_PDL_ENTRY()                                                  \
    do {                                                                \
        asm volatile("griddepcontrol.wait;" ::: "memory");              \
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); \
    } while (0)
template <typename... KArgs, typename... Args>
inline void launch_pdl(const Launch& L, void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                       Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = L.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}
// the same with a 2-D grid
template <typename... KArgs, typename... Args>
inline void launch_pdl_2d(const Launch& L, void (*kernel)(KArgs...), dim3 grid, unsigned block, size_t smem,
                          Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = L.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}
// bracket one launch with timer events (no-op unless the id is enabled)
void timer_collect(KTimer* T, bool wait);
inline int tbegin(const Launch& L, int id) {
    *L.launches += 1;
    KTimer* T = L.timer;
    if (!T || !T->ready || !((T->mask >> id) & 1ull)) return -1;
    if (T->head - T->tail >= KTimer::NEV / 2) timer_collect(T, true);   // ring full: drain
    const int q = (int)(T->head++ % (KTimer::NEV / 2));
    T->id_of[q] = id;
    cudaEventRecord(T->ev[2 * q], L.stream);
    return q;
}
inline void tend(const Launch& L, int q) {
    if (q >= 0) cudaEventRecord(L.timer->ev[2 * q + 1], L.stream);
}

void rebin(const Dev& D, const Launch& L, int projection, int cutoff);
void search(const Dev& D, const Launch& L, int precision, int do_search, int do_effpor);
void freesurf(const Dev& D, const Launch& L);
void boun_vel(const Dev& D, const Launch& L, int precision);
void ghost(const Dev& D, const Launch& L, int precision, int use_mls);
void collision_shift(const Dev& D, const Launch& L, int precision, int mode, double prx, double pry, double brx,
                     double bry);
void eddy(const Dev& D, const Launch& L, int precision, int with_eddy, int with_varts, int with_disp);
void int_vel(const Dev& D, const Launch& L, int precision);
void assemble(const Dev& D, const Launch& L, int precision);
void comp_vel(const Dev& D, const Launch& L, int precision, int do_vel, int do_pos);
void cell_max_timestep(const Dev& D, const Launch& L, int do_cellmax, int do_timestep);
void shift(const Dev& D, const Launch& L, int precision);
void apply_density(const Dev& D, const Launch& L, int do_apply, int do_density);
// one salinity sub-step; with jdev the sub-step index is substep + *jdev
void scalar(const Dev& D, const Launch& L, int precision, int substep, const int* jdev = nullptr);
// WCSPH (wcsph.f90): continuity, row updates (bit0 updateden, bit1
// dentopress, bit2 presstoden), wall pressure of the WCSPH step
void wc_continuity(const Dev& D, const Launch& L, int precision);
void wc_rows(const Dev& D, const Launch& L, int mode);
void wc_wall_pressure(const Dev& D, const Launch& L, int precision);
void advance_time(const Dev& D, const Launch& L);
void derive_fields(const Dev& D, const Launch& L);
// state snapshot of one scene for an asynchronous read-back (k_snapshot):
// nf FP64 fields, and tid (widened to int32), pid and flags where non-null
#define BS_SNAP_MAXF 23
struct SnapArgs {
    const double* src[BS_SNAP_MAXF];
    double* dst[BS_SNAP_MAXF];
    int nf, row0, n;
    const int8_t* tid;
    int* tid_dst;
    const int* pid;
    int* pid_dst;
    const uint8_t* flags;
    uint8_t* flags_dst;
};
void snapshot(const Launch& L, const SnapArgs& a);
// an uploaded scene's rows into their binned order (see k_upload_gather)
void upload_gather(const Dev& D, const Launch& L, int row0, int n, int cell0, int has_flags, int has_pid);
// solver
void solve_fp64(const Dev& D, const Launch& L, int maxit, int check_every, int precond, int mg_precision,
                int* d_all_conv, int* h_all_conv_pinned, cudaEvent_t ev);
// multigrid preconditioner (bs_mg.cu)
void mg_setup(const Dev& D, const Launch& L, int mg_precision);
void mg_apply(const Dev& D, const Launch& L, int mg_precision, const double* in, double* out);
// the level-0 input of the V-cycle, written by the Krylov streams (x = p or s)
template <typename T>
__device__ __forceinline__ void mg_put_input(const Dev& D, int r, double x) {
    ((T*)D.mg.xin)[r] = (T)x;
    ((T*)D.mg.u)[r] = (T)D.mg.omega * (T)x * ((const T*)D.mg.dinv0)[r];
}
void solve_mixed(const Dev& D, const Launch& L, int maxit, int check_every, int* d_all_conv,
                 int* h_all_conv_pinned, cudaEvent_t ev);
// one scene's buffer zone template and exchange rule (remove_bufferN +
// insert_bufferN, internal.f90:447-586)
struct ZoneDev {
    const double *x, *y, *vx, *vy, *p;
    const int* pid;                 // may be null (pid 0)
    double mass, rho, ovol, con, remove_x;
    int remove_side, zone;
};
void buffer_exchange(const Dev& D, const Launch& L, int s, const ScenePar& P, const ZoneDev& Z);
int mg_sub_max_clusters(int mg_precision, int cs, size_t smem);
// allow the exact coarse factorisation its shared memory (once per process)
int mg_exact_prepare();
void solve_fgmres(const Dev& D, const Launch& L, int maxit, int check_every, int precond, int mg_prec,
                  int* d_nconv, int* h_nconv, cudaEvent_t ev);
// The same solves recorded into the stream capture of L.stream with their
// loops on the device (conditional while/if nodes whose condition kernels
// read the converged-scene counters); side[0..2] are streams that capture the
// loop bodies.  Return false when a CUDA call failed (the capture is unusable).
bool capture_fp64(const Dev& D, const Launch& L, const cudaStream_t* side, int maxit, int check_every, int precond,
                  int mg_prec, int* d_nconv);
bool capture_fgmres(const Dev& D, const Launch& L, const cudaStream_t* side, int maxit, int check_every,
                    int precond, int mg_prec, int* d_nconv);
// conditional-node helpers for a capture in progress on `st`
bool cond_handle(cudaStream_t st, unsigned init, cudaGraphConditionalHandle* h);
template <class F>
bool cond_node(cudaStream_t st, cudaStream_t side, cudaGraphConditionalNodeType type, cudaGraphConditionalHandle h,
               F&& body) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive)
        return false;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = type;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &np) != cudaSuccess) return false;
    if (cudaStreamBeginCaptureToGraph(side, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed) != cudaSuccess)
        return false;
    const bool ok = body();
    cudaGraph_t out = nullptr;
    const bool ended = cudaStreamEndCapture(side, &out) == cudaSuccess;
    if (!ok || !ended) return false;
    return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies) ==
           cudaSuccess;
}
// condition kernel of the captured step's scalar sub-step pairs (two more
// sub-steps done; go on while a scene has sub-steps left), launched on st
void cond_scalar(const Dev& D, cudaStream_t st, cudaGraphConditionalHandle h, int body_kernels);
// per-scene small FGMRES storage for restart length m (doubles)
inline int fg_small_size(int m) { return (m + 1) * m + (m + 1) * (m + 1) + 2 * m + (m + 1) + m + (m + 1) + 8; }
__host__ __device__ inline int fg_part_ld(int m) { return 2 * m + 4; }
}  // namespace bs
