// bs_mg.cu -- aggregation multigrid preconditioner for the PPE BiCGStab.
//
// The reference solves the Jacobi-scaled PPE with unpreconditioned FGMRES /
// BiCGStab (solver.f90:129-350); the iteration count then grows with the
// number of particles across the domain.  This multigrid cycle is applied as
// a right preconditioner; the Krylov recurrence, dots and the stopping test
// stay FP64, so the converged pressure is the solution of the same FP64
// system.
//
// Level 0: particle rows (the sliced-ELL PPE).  Level 1: one aggregate per
// half-cell -- the four 2h x 2h quadrants of a search cell (~7 rows each).
// The rows of a cell are contiguous, so the Galerkin product P^T A P
// (P = half-cell indicator) is a warp reduction per cell, and because every
// neighbour lies within 2h the coarse operator is a 9-point stencil on the
// half-cell grid.  Level 2: the cells; level l+1: 2x2 boxes of level l,
// again 9-point Galerkin stencils.  Smoother: damped Jacobi, one pre-sweep
// from zero and one post-sweep; coarse corrections scaled by cscale (over-
// correction for the piecewise-constant prolongation); levels 1..wlev visit
// the next level twice (the second time on the updated residual), so the
// cycle is a W-cycle at the top and a V-cycle below; coarsest level: Jacobi
// sweeps by one block per scene.  Every scene coarsens on its own, so its
// cycle is the same alone and inside a batch.  The particle-level kernels
// skip converged scenes.  T = double (FP64 mode) or float (mixed mode, FP32
// cycle).
#include "bs_internal.cuh"

using namespace bs;

namespace {

__device__ __forceinline__ bool mg_skip(const Dev& D, int s) { return D.dyn[s].converged != 0; }

// ------------------------------------------------------------ setup
// level 0: 1/adiag per row, and the row's half-cell (quadrant of its cell,
// split at the cell's mid-lines as the quadrant search does, search.f90:328)
template <typename T>
__global__ void k_mg_dinv0(Dev D) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const ScenePar& P = D.par[s];
    if (r >= P.row0 + D.dyn[s].n) return;
    const double d = D.adiag[r];
    ((T*)D.mg.dinv0)[r] = (d != 0.0 && isfinite(d)) ? (T)(1.0 / d) : (T)0;
    ((T*)D.mg.adiagT)[r] = (T)d;
    const int lc = D.cell[r] - P.cell0;
    const int i0 = lc % P.celly, j0 = lc / P.celly;
    const double xl = cell_xleft(P, j0 + 1), xr = cell_xright(P, j0 + 1);
    const double yb = cell_ybot(P, i0 + 1), yt = cell_ytop(P, i0 + 1);
    const int lower = D.y[r] <= yb + fabs((yt - yb) / 2.0);
    const int right = D.x[r] > xl + fabs((xl - xr) / 2.0);
    D.mg.sub[r] = (uint8_t)(lower | (right << 1));
    D.mg.agg1[r] = D.mg.off[1][s] + (2 * j0 + right) * (2 * P.celly) + 2 * i0 + lower;
}

// level 1 = P^T A0 P over the half-cells: one warp per cell, a lane per row
// accumulating the row's 9 stencil entries, then one masked warp reduction
// per (half-cell, entry); lane m keeps entry m and m+32 of the 36 results.
// An offset beyond one half-cell (a pair split by rounding at a mid-line)
// is clamped into the stencil.  Sums in the level's type T (FP32 in the
// mixed form, from the FP32 copy of the matrix); the neighbour's cell column
// offset (-1, 0, 1) from two comparisons instead of an integer division.
template <typename T>
__global__ void k_mg_gal0(Dev D) {
    BS_PDL_ENTRY();
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= D.ncell_total) return;
    const int s = D.cell_scene[c];
    const ScenePar& P = D.par[s];
    if (c - P.cell0 >= P.ncell) return;   // reserved cells beyond the scene's current grid
    const int celly = P.celly;
    const int r0 = D.cell_start[c], r1 = D.cell_end[c];
    const T* A = (const T*)(sizeof(T) == 8 ? D.aval : (void*)D.aval32);
    const uint8_t* sub = D.mg.sub;
    T mine0 = 0, mine1 = 0;
    for (int base = r0; base < r1; base += 32) {
        const int r = base + lane;
        T acc[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] = 0;
        int sb = -1;
        if (r < r1) {
            sb = sub[r];
            const int si = sb & 1, sj = sb >> 1;
            acc[4] += (T)D.adiag[r];
            const int n = D.ncount[r];
            for (int k = 0; k < n; ++k) {
                const long e = ell(r, k, D.kmax);
                const int col = D.nidx[e];
                const int d = D.cell[col] - c;
                const int u = d + celly + 1;   // in [0, 2 celly + 2] for the 3x3 neighbour cells
                const int dj = (u >= 2 * celly) ? 1 : ((u >= celly) ? 0 : -1);
                const int di = d - dj * celly;
                const int s2 = sub[col];
                const int dI = min(max(2 * di + (s2 & 1) - si, -1), 1);
                const int dJ = min(max(2 * dj + (s2 >> 1) - sj, -1), 1);
                const int q = (dJ + 1) * 3 + (dI + 1);
                const T v = A[e];
#pragma unroll
                for (int t = 0; t < 9; ++t)
                    if (t == q) acc[t] += v;
            }
        }
#pragma unroll
        for (int t = 0; t < 4; ++t)
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                T v = (sb == t) ? acc[k] : (T)0;
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                const int m = t * 9 + k;
                if (m < 32) { if (lane == m) mine0 += v; }
                else if (lane == m - 32) mine1 += v;
            }
    }
    T* Al = (T*)D.mg.A[1];
    T* dl = (T*)D.mg.dinv[1];
    const int n1 = D.mg.n[1];
    const int lc = c - P.cell0;
    const int i0 = lc % celly, j0 = lc / celly;
    const int o1 = D.mg.off[1][s], ny1 = 2 * celly;
    auto put = [&](int m, T v) {
        const int t = m / 9, k = m - 9 * (m / 9);
        const int Q = o1 + (2 * j0 + (t >> 1)) * ny1 + 2 * i0 + (t & 1);
        Al[(long)k * n1 + Q] = v;
        if (k == 4) dl[Q] = (v != (T)0 && isfinite(v)) ? (T)1 / v : (T)0;
    };
    put(lane, mine0);
    if (lane < 4) put(lane + 32, mine1);
}

// level l+1 from level l: one thread per coarse cell
template <typename T>
__global__ void k_mg_galc(Dev D, int l) {
    BS_PDL_ENTRY();
    const int Q = blockIdx.x * blockDim.x + threadIdx.x;
    const MgDev& M = D.mg;
    if (Q >= M.n[l + 1]) return;
    const int s = M.scene_of[l + 1][Q];
    const int q = Q - M.off[l + 1][s];
    const int nyc = M.ny[l + 1][s];
    if (q >= nyc * M.nx[l + 1][s]) return;   // reserved beyond the scene's current grid
    const int I = q % nyc, J = q / nyc;
    const int nyf = M.ny[l][s], nxf = M.nx[l][s], fo = M.off[l][s];
    const T* Af = (const T*)M.A[l];
    const int nf = M.n[l];
    double acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.0;
    for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a) {
            const int fi = 2 * I + a, fj = 2 * J + b;
            if (fi >= nyf || fj >= nxf) continue;
            const int c = fo + fj * nyf + fi;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const double v = (double)Af[(long)k * nf + c];
                if (v == 0.0) continue;
                const int ni = fi + (k % 3) - 1, nj = fj + (k / 3) - 1;
                const int ci = (ni >= 0 ? ni / 2 : -1) - I, cj = (nj >= 0 ? nj / 2 : -1) - J;
                const int t = (cj + 1) * 3 + (ci + 1);
#pragma unroll
                for (int u = 0; u < 9; ++u)
                    if (u == t) acc[u] += v;
            }
        }
    T* Ac = (T*)M.A[l + 1];
    const int nc = M.n[l + 1];
#pragma unroll
    for (int k = 0; k < 9; ++k) Ac[(long)k * nc + Q] = (T)acc[k];
    ((T*)M.dinv[l + 1])[Q] = (acc[4] != 0.0 && isfinite(acc[4])) ? (T)(1.0 / acc[4]) : (T)0;
}

// ------------------------------------------------------------ cycle
// Level 0 pre-smooth from zero (z0 = w D^-1 in), residual, restriction to
// the half-cells: r1[h] = sum_{i in h} (in_i - (A0 z0)_i).  One warp per
// cell, four sums (one per quadrant); every half-cell is written, empty
// ones with 0.
// sum over the row's off-diagonal nonzeros of A * u (sliced ELL), four
// independent index/value loads in flight before the gathers
template <typename T>
__device__ __forceinline__ T ell_dot(const T* __restrict__ A, const int* __restrict__ idx,
                                     const T* __restrict__ u, int r, int n, int kmax, T acc) {
    long e = ell(r, 0, kmax);
    int k = 0;
    for (; k + 4 <= n; k += 4, e += 128) {
        const int j0 = __ldg(idx + e), j1 = __ldg(idx + e + 32), j2 = __ldg(idx + e + 64), j3 = __ldg(idx + e + 96);
        const T a0 = __ldg(A + e), a1 = __ldg(A + e + 32), a2 = __ldg(A + e + 64), a3 = __ldg(A + e + 96);
        const T u0 = u[j0], u1 = u[j1], u2 = u[j2], u3 = u[j3];
        acc += a0 * u0;
        acc += a1 * u1;
        acc += a2 * u2;
        acc += a3 * u3;
    }
    for (; k < n; ++k, e += 32) acc += __ldg(A + e) * u[__ldg(idx + e)];
    return acc;
}

// Level 0, pass 1: the residual after the pre-sweep from zero, v = xin - A u
// (u = omega xin / adiag, written with the input), one thread per row on the
// aligned row blocks (coalesced slices of the ELL), into zz (free until the
// prolongation)
template <typename T>
__global__ void k_mg_l0_resid(Dev D) {
    BS_PDL_ENTRY();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = D.blk_scene[r / BS_ALIGN];
    if (mg_skip(D, s)) return;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const T* __restrict__ u = (const T*)D.mg.u;
    const T* __restrict__ A = (const T*)(sizeof(T) == 8 ? D.aval : (void*)D.aval32);
    T v = ((const T*)D.mg.xin)[r];
    if (D.mg.pre0) v -= ell_dot<T>(A, D.nidx, u, r, D.ncount[r], D.kmax, ((const T*)D.mg.adiagT)[r] * u[r]);
    ((T*)D.mg.zz)[r] = v;
}

// Level 0, pass 2: restriction of that residual to the half-cells, a thread
// per half-cell summing the rows of its quadrant in row order (the four
// threads of a cell read the cell's rows together; one wave of threads)
template <typename T>
__global__ void k_mg_l0_down(Dev D) {
    BS_PDL_ENTRY();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = t >> 2, quad = t & 3;   // quad = lower | right << 1, as mg.sub
    if (c >= D.ncell_total) return;
    const int s = D.cell_scene[c];
    if (mg_skip(D, s) || c - D.par[s].cell0 >= D.par[s].ncell) return;
    const T* __restrict__ zz = (const T*)D.mg.zz;
    const uint8_t* __restrict__ sub = D.mg.sub;
    const int r0 = D.cell_start[c], r1 = D.cell_end[c];
    T q = 0;
    int r = r0;
    for (; r + 4 <= r1; r += 4) {   // four rows' loads in flight
        const T v0 = zz[r], v1 = zz[r + 1], v2 = zz[r + 2], v3 = zz[r + 3];
        const int t0 = sub[r], t1 = sub[r + 1], t2 = sub[r + 2], t3 = sub[r + 3];
        q += (t0 == quad) ? v0 : (T)0;
        q += (t1 == quad) ? v1 : (T)0;
        q += (t2 == quad) ? v2 : (T)0;
        q += (t3 == quad) ? v3 : (T)0;
    }
    for (; r < r1; ++r) q += (sub[r] == quad) ? zz[r] : (T)0;
    const ScenePar& P = D.par[s];
    const int lc = c - P.cell0;
    const int i0 = lc % P.celly, j0 = lc / P.celly;
    const int Q = D.mg.off[1][s] + (2 * j0 + (quad >> 1)) * (2 * P.celly) + 2 * i0 + (quad & 1);
    ((T*)D.mg.r[1])[Q] = q;
}

// zz = u + cscale * e1[half-cell]: the level-0 value after the coarse correction
template <typename T>
__global__ void k_mg_l0_prolong(Dev D) {
    BS_PDL_ENTRY();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = D.blk_scene[r / BS_ALIGN];
    if (mg_skip(D, s)) return;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const T pre = D.mg.pre0 ? ((const T*)D.mg.u)[r] : (T)0;
    ((T*)D.mg.zz)[r] = pre + (T)D.mg.cscale * ((const T*)D.mg.z[1])[D.mg.agg1[r]];
}

// ---- level operations on the cell levels (l >= 1), one cell per call.
// A scene's view of a level: its grid, its first cell in the level's arrays
// and the level's total size (the stride of the stencil arrays).  The
// per-level kernels build views from the MgLevel tables (kernel arguments,
// in the constant bank: no memory round trip for a cell's scene, offsets and
// grid).  On these
// small levels the kernels are bound by the latency of their dependent
// loads, not by bandwidth.  Converged scenes are not skipped here (their
// cells are few and the result is unused).
struct LevelS {
    int l, n, off, nx, ny;
};

// largest scene index k with G.off[k] <= c (scenes absent from the level
// have empty ranges)
__device__ __forceinline__ int scene_at(const MgLevel& G, int c) {
    int lo = 0, hi = G.ns - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (G.off[mid] <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ LevelS view_of(const MgLevel& G, int k) {
    LevelS v;
    v.l = G.l; v.n = G.n; v.off = G.off[k]; v.nx = G.nx[k]; v.ny = G.ny[k];
    return v;
}

// Levels l -> l+1 for coarse cell q of the scene: pre-smooth from zero,
// residual, restriction (2x2 sum).  The smoothed values w r D^-1 of the 4x4
// fine cells around the box are loaded once and all loads are issued before
// the sums (one round of memory latency instead of one per child: these
// levels are bound by their chains of dependent loads); the sums run in the
// same order as child by child.
template <typename T>
__device__ __forceinline__ void op_down(const MgDev& M, const LevelS& F, const LevelS& C, int q) {
    const int I = q % C.ny, J = q / C.ny;
    const T* __restrict__ A = (const T*)M.A[F.l];
    const T* __restrict__ dinv = (const T*)M.dinv[F.l];
    const T* __restrict__ r = (const T*)M.r[F.l];
    const T w = (T)M.omega;
    T sum = 0;
    if (!M.prec) {
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
                const int fi = 2 * I + a, fj = 2 * J + b;
                if (fi < F.ny && fj < F.nx) sum += r[F.off + fj * F.ny + fi];
            }
        ((T*)M.r[C.l])[C.off + q] = sum;
        return;
    }
    const int fi0 = 2 * I - 1, fj0 = 2 * J - 1;   // the 4x4 neighbourhood's corner
    T y[4][4], rc[2][2];
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int ni = fi0 + a, nj = fj0 + b;
            const bool in = ni >= 0 && nj >= 0 && ni < F.ny && nj < F.nx;
            const int nb = F.off + nj * F.ny + ni;
            y[b][a] = in ? w * r[nb] * __ldg(dinv + nb) : (T)0;
            if (a >= 1 && a <= 2 && b >= 1 && b <= 2) rc[b - 1][a - 1] = in ? r[nb] : (T)0;
        }
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const int fi = 2 * I + a, fj = 2 * J + b;
            if (fi >= F.ny || fj >= F.nx) continue;
            const int c = F.off + fj * F.ny + fi;
            T ax = 0;
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                const int ni = fi + (t % 3) - 1, nj = fj + (t / 3) - 1;
                if (ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx) continue;
                ax += __ldg(A + (long)t * F.n + c) * y[b + t / 3][a + t % 3];
            }
            sum += rc[b][a] - ax;
        }
    ((T*)M.r[C.l])[C.off + q] = sum;
}

// One child (a, b) of coarse cell q's 2x2 box: r_c - (A (w D^-1 r))_c, the
// value op_down adds for it (0 for a child beyond the fine grid); the
// neighbourhood's loads issued before the sum.
template <typename T>
__device__ __forceinline__ T down_child(const MgDev& M, const LevelS& F, const LevelS& C, int q, int a, int b) {
    const int I = q % C.ny, J = q / C.ny;
    const int fi = 2 * I + a, fj = 2 * J + b;
    if (fi >= F.ny || fj >= F.nx) return (T)0;
    const T* __restrict__ A = (const T*)M.A[F.l];
    const T* __restrict__ dinv = (const T*)M.dinv[F.l];
    const T* __restrict__ r = (const T*)M.r[F.l];
    const T w = (T)M.omega;
    const int c = F.off + fj * F.ny + fi;
    const T rc = r[c];
    if (!M.prec) return rc;
    T yv[9], av[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int ni = fi + (t % 3) - 1, nj = fj + (t / 3) - 1;
        const bool in = !(ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx);
        const int nb = F.off + nj * F.ny + ni;
        yv[t] = in ? w * r[nb] * __ldg(dinv + nb) : (T)0;
        av[t] = in ? __ldg(A + (long)t * F.n + c) : (T)0;
    }
    T ax = 0;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int ni = fi + (t % 3) - 1, nj = fj + (t / 3) - 1;
        if (ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx) continue;
        ax += av[t] * yv[t];
    }
    return rc - ax;
}

// In-place residual on level l, cell q of the scene: r = r - A z (between
// the two visits of a W-cycle level; reads its own r and the stencil's z).
template <typename T>
__device__ __forceinline__ void op_resid(const MgDev& M, const LevelS& F, int q) {
    const int i = q % F.ny, j = q / F.ny;
    const int c = F.off + q;
    const T* __restrict__ A = (const T*)M.A[F.l];
    const T* z = (const T*)M.z[F.l];
    T* r = (T*)M.r[F.l];
    T zv[9], av[9];   // loads first (one round of latency), then the sum in stencil order
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int ni = i + (t % 3) - 1, nj = j + (t / 3) - 1;
        const bool in = !(ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx);
        zv[t] = in ? z[F.off + nj * F.ny + ni] : (T)0;
        av[t] = in ? __ldg(A + (long)t * F.n + c) : (T)0;
    }
    const T rc = r[c];
    T ax = 0;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int ni = i + (t % 3) - 1, nj = j + (t / 3) - 1;
        if (ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx) continue;
        ax += av[t] * zv[t];
    }
    r[c] = rc - ax;
}

// Levels l+1 -> l for cell q of the scene: prolongation (constant per box,
// scaled) + one post-sweep; with acc the result is added to z.
template <typename T>
__device__ __forceinline__ void op_up(const MgDev& M, const LevelS& F, const LevelS& C, int acc, int q) {
    const int i = q % F.ny, j = q / F.ny;
    const int c = F.off + q;
    const T* __restrict__ A = (const T*)M.A[F.l];
    const T* __restrict__ dinv = (const T*)M.dinv[F.l];
    const T* __restrict__ r = (const T*)M.r[F.l];
    const T* __restrict__ e = (const T*)M.z[C.l];
    const T w = (T)M.omega, cs = (T)M.cscale;
    const T wp = M.prec ? w : (T)0;
    // every load of the 3x3 neighbourhood issued before the sum (one round
    // of latency), the sum in stencil order
    T zv[9], av[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int ni = i + (t % 3) - 1, nj = j + (t / 3) - 1;
        const bool in = !(ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx);
        const int nb = F.off + nj * F.ny + ni;
        zv[t] = in ? wp * r[nb] * __ldg(dinv + nb) + cs * e[C.off + (nj / 2) * C.ny + (ni / 2)] : (T)0;
        av[t] = in ? __ldg(A + (long)t * F.n + c) : (T)0;
    }
    const T zc = zv[4];
    T ax = 0;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int ni = i + (t % 3) - 1, nj = j + (t / 3) - 1;
        if (ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx) continue;
        ax += av[t] * zv[t];
    }
    const T v = zc + w * __ldg(dinv + c) * (r[c] - ax);
    T* zo = (T*)M.z[F.l];
    zo[c] = acc ? zo[c] + v : v;
}

// Coarsest level of one scene: damped Jacobi sweeps from zero by the whole
// block in shared memory (z, z2: coarse_max values each); with acc the
// result is added to z.  Every thread of the block calls it.
template <typename T>
__device__ __forceinline__ void op_coarse(const MgDev& M, const LevelS& F, int acc, T* z) {
    T* z2 = z + M.coarse_max;
    const int m = F.nx * F.ny;
    const T* __restrict__ A = (const T*)M.A[F.l];
    const T* __restrict__ dinv = (const T*)M.dinv[F.l];
    const T* __restrict__ r = (const T*)M.r[F.l];
    const T w = (T)M.omega;
    for (int q = threadIdx.x; q < m; q += blockDim.x) z[q] = 0;
    __syncthreads();
    if (m <= (int)blockDim.x) {
        // one cell per thread: its stencil, D^-1 and r held in registers
        // across the sweeps, which then touch shared memory only
        const int q = threadIdx.x;
        const bool act = q < m;
        const int i = q % F.ny, j = q / F.ny;
        const int c = F.off + q;
        T a9[9], dc = 0, rcv = 0;
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            const int ni = i + (t % 3) - 1, nj = j + (t / 3) - 1;
            a9[t] = (act && !(ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx)) ? __ldg(A + (long)t * F.n + c) : (T)0;
        }
        if (act) {
            dc = __ldg(dinv + c);
            rcv = r[c];
        }
        for (int it = 0; it < M.coarse_sweeps; ++it) {
            if (act) {
                T ax = 0;
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    const int ni = i + (t % 3) - 1, nj = j + (t / 3) - 1;
                    if (ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx) continue;
                    ax += a9[t] * z[nj * F.ny + ni];
                }
                z2[q] = z[q] + w * dc * (rcv - ax);
            }
            __syncthreads();
            if (act) z[q] = z2[q];
            __syncthreads();
        }
    } else {
        for (int it = 0; it < M.coarse_sweeps; ++it) {
            for (int q = threadIdx.x; q < m; q += blockDim.x) {
                const int i = q % F.ny, j = q / F.ny;
                const int c = F.off + q;
                T ax = 0;
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    const int ni = i + (t % 3) - 1, nj = j + (t / 3) - 1;
                    if (ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx) continue;
                    ax += __ldg(A + (long)t * F.n + c) * z[nj * F.ny + ni];
                }
                z2[q] = z[q] + w * __ldg(dinv + c) * (r[c] - ax);
            }
            __syncthreads();
            for (int q = threadIdx.x; q < m; q += blockDim.x) z[q] = z2[q];
            __syncthreads();
        }
    }
    T* out = (T*)M.z[F.l];
    for (int q = threadIdx.x; q < m; q += blockDim.x) out[F.off + q] = acc ? out[F.off + q] + z[q] : z[q];
}

// ---- the last two levels of a visit in one block (option mg_tail)
// Scene k's visit of level l (F, at most 1024 cells) whose next level C (at
// most BS_MG_TAIL_C cells) is its coarsest: pre-sweep and restriction
// (op_down), the coarsest-level Jacobi sweeps (op_coarse; with wcycle the
// residual op_resid and a second solve added, as a W-cycle level visits its
// next level twice) and prolongation + post-sweep (op_up), one thread per
// cell of F, both levels in shared memory between the operations instead of
// a launch each.  Every value is formed by the same operations in the same
// order as the separate launches (bit-identical).
#define BS_MG_TAIL_F 1024
#define BS_MG_TAIL_C 256
template <typename T>
__global__ void __launch_bounds__(BS_MG_TAIL_F) k_mg_tail(Dev D, __grid_constant__ const MgLevel F,
                                                          __grid_constant__ const MgLevel C, int acc, int wcycle) {
    BS_PDL_ENTRY();
    __shared__ T R[BS_MG_TAIL_F], Y[BS_MG_TAIL_F], RS[BS_MG_TAIL_F], DV[BS_MG_TAIL_F];
    __shared__ T RC[BS_MG_TAIL_C], ZC[BS_MG_TAIL_C], ZC2[BS_MG_TAIL_C], ZA[BS_MG_TAIL_C];
    const MgDev& M = D.mg;
    const int k = blockIdx.x;
    const LevelS f = view_of(F, k), c = view_of(C, k);
    const int mf = f.nx * f.ny, mc = c.nx * c.ny;
    if (mf == 0) return;
    const int t = threadIdx.x;
    const T w = (T)M.omega, cs = (T)M.cscale;
    const T* __restrict__ Af = (const T*)M.A[f.l];
    const T* __restrict__ Ac = (const T*)M.A[c.l];
    // fine cell t: its stencil in registers, r and D^-1 in shared memory
    const bool fa = t < mf;
    const int fi = t % f.ny, fj = t / f.ny;
    T a9[9];
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        const int ni = fi + (s % 3) - 1, nj = fj + (s / 3) - 1;
        a9[s] = (fa && !(ni < 0 || nj < 0 || ni >= f.ny || nj >= f.nx)) ? __ldg(Af + (long)s * f.n + f.off + t) : (T)0;
    }
    if (fa) {
        R[t] = ((const T*)M.r[f.l])[f.off + t];
        DV[t] = __ldg((const T*)M.dinv[f.l] + f.off + t);
    }
    // coarse cell t: its stencil, D^-1 (and r below) in registers
    const bool ca = t < mc;
    const int ci = t % c.ny, cj = t / c.ny;
    T c9[9], dc = 0;
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        const int ni = ci + (s % 3) - 1, nj = cj + (s / 3) - 1;
        c9[s] = (ca && !(ni < 0 || nj < 0 || ni >= c.ny || nj >= c.nx)) ? __ldg(Ac + (long)s * c.n + c.off + t) : (T)0;
    }
    if (ca) dc = __ldg((const T*)M.dinv[c.l] + c.off + t);
    __syncthreads();
    // op_down: the pre-sweep from zero and each fine cell's residual
    if (fa) Y[t] = w * R[t] * DV[t];
    __syncthreads();
    if (fa) {
        T ax = 0;
        if (M.prec) {
#pragma unroll
            for (int s = 0; s < 9; ++s) {
                const int ni = fi + (s % 3) - 1, nj = fj + (s / 3) - 1;
                if (ni < 0 || nj < 0 || ni >= f.ny || nj >= f.nx) continue;
                ax += a9[s] * Y[nj * f.ny + ni];
            }
            RS[t] = R[t] - ax;
        } else {
            RS[t] = R[t];
        }
    }
    __syncthreads();
    // restriction: the 2x2 box's children, b outer, a inner
    T rcv = 0;
    if (ca) {
        T sum = 0;
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {   // a child beyond the grid adds 0, as in k_mg_down
                const int gi = 2 * ci + a, gj = 2 * cj + b;
                sum += (gi < f.ny && gj < f.nx) ? RS[gj * f.ny + gi] : (T)0;
            }
        rcv = sum;
        RC[t] = sum;
    }
    // op_coarse: damped Jacobi from zero, one coarse cell per thread
    auto jacobi = [&](T rhs, T* z, T* z2) {
        if (ca) z[t] = 0;
        __syncthreads();
        for (int it = 0; it < M.coarse_sweeps; ++it) {
            if (ca) {
                T ax = 0;
#pragma unroll
                for (int s = 0; s < 9; ++s) {
                    const int ni = ci + (s % 3) - 1, nj = cj + (s / 3) - 1;
                    if (ni < 0 || nj < 0 || ni >= c.ny || nj >= c.nx) continue;
                    ax += c9[s] * z[nj * c.ny + ni];
                }
                z2[t] = z[t] + w * dc * (rhs - ax);
            }
            __syncthreads();
            if (ca) z[t] = z2[t];
            __syncthreads();
        }
    };
    jacobi(rcv, ZC, ZC2);
    if (wcycle) {
        // op_resid on the coarsest level, then the second solve added to z
        T r2 = 0;
        if (ca) {
            T ax = 0;
#pragma unroll
            for (int s = 0; s < 9; ++s) {
                const int ni = ci + (s % 3) - 1, nj = cj + (s / 3) - 1;
                if (ni < 0 || nj < 0 || ni >= c.ny || nj >= c.nx) continue;
                ax += c9[s] * ZC[nj * c.ny + ni];
            }
            r2 = rcv - ax;
            ZA[t] = ZC[t];
        }
        __syncthreads();
        jacobi(r2, ZC, ZC2);
        if (ca) ZC[t] = ZA[t] + ZC[t];
        __syncthreads();
    }
    // op_up: prolongation (scaled, constant per box) + one post-sweep
    if (fa) {
        const T wp = M.prec ? w : (T)0;
        T zv[9];
#pragma unroll
        for (int s = 0; s < 9; ++s) {
            const int ni = fi + (s % 3) - 1, nj = fj + (s / 3) - 1;
            const bool in = !(ni < 0 || nj < 0 || ni >= f.ny || nj >= f.nx);
            const int nb = nj * f.ny + ni;
            zv[s] = in ? wp * R[nb] * DV[nb] + cs * ZC[(nj / 2) * c.ny + (ni / 2)] : (T)0;
        }
        const T zc = zv[4];
        T ax = 0;
#pragma unroll
        for (int s = 0; s < 9; ++s) {
            const int ni = fi + (s % 3) - 1, nj = fj + (s / 3) - 1;
            if (ni < 0 || nj < 0 || ni >= f.ny || nj >= f.nx) continue;
            ax += a9[s] * zv[s];
        }
        const T v = zc + w * DV[t] * (R[t] - ax);
        T* zo = (T*)M.z[f.l];
        zo[f.off + t] = acc ? zo[f.off + t] + v : v;
    }
}

// ---- one launch per level operation
// A quad of lanes per coarse cell: lane (a, b) smooths child (a, b), the
// first lane adds the four values in op_down's order (b outer, a inner), so
// the result is bit-identical to op_down with a quarter of its loads per
// thread in flight at once.
template <typename T>
__global__ void k_mg_down(Dev D, __grid_constant__ const MgLevel F, __grid_constant__ const MgLevel C) {
    BS_PDL_ENTRY();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int Q = g >> 2, child = g & 3;
    bool ok = false;
    int q = 0, k = 0;
    T val = 0;
    if (Q < C.n) {
        k = scene_at(C, Q);
        q = Q - C.off[k];
        ok = q < C.nx[k] * C.ny[k];   // not reserved beyond the scene's current grid
        if (ok) val = down_child<T>(D.mg, view_of(F, k), view_of(C, k), q, child & 1, child >> 1);
    }
    const int base = (threadIdx.x & 31) & ~3;
    const T v0 = __shfl_sync(0xffffffffu, val, base), v1 = __shfl_sync(0xffffffffu, val, base + 1);
    const T v2 = __shfl_sync(0xffffffffu, val, base + 2), v3 = __shfl_sync(0xffffffffu, val, base + 3);
    if (ok && child == 0) {
        T sum = 0;
        sum += v0;
        sum += v1;
        sum += v2;
        sum += v3;
        ((T*)D.mg.r[C.l])[C.off[k] + q] = sum;
    }
}

template <typename T>
__global__ void k_mg_resid(Dev D, __grid_constant__ const MgLevel F) {
    BS_PDL_ENTRY();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= F.n) return;
    const int k = scene_at(F, c);
    const LevelS f = view_of(F, k);
    const int q = c - f.off;
    if (q >= f.nx * f.ny) return;
    op_resid<T>(D.mg, f, q);
}

template <typename T>
__global__ void k_mg_up(Dev D, __grid_constant__ const MgLevel F, __grid_constant__ const MgLevel C, int acc) {
    BS_PDL_ENTRY();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= F.n) return;
    const int k = scene_at(F, c);
    if (F.l >= F.lev[k]) return;   // the coarse solve wrote this level
    const LevelS f = view_of(F, k);
    const int q = c - f.off;
    if (q >= f.nx * f.ny) return;
    op_up<T>(D.mg, f, view_of(C, k), acc, q);
}

template <typename T>
__global__ void k_mg_coarse(Dev D, __grid_constant__ const MgLevel F, int acc) {
    BS_PDL_ENTRY();
    const int k = blockIdx.x;
    if (F.lev[k] != F.l) return;
    extern __shared__ unsigned char smem[];
    op_coarse<T>(D.mg, view_of(F, k), acc, (T*)smem);
}

// ---- exact coarse solve (option mg_exact).  A scene's level of at most
// BS_MG_EXACT_MAX cells (a 9-point Galerkin stencil on an nx x ny grid,
// cells numbered q = j ny + i) is a band matrix of half-bandwidth b = ny + 1.
// Once per step one block per scene factors it in FP64 (LU without pivoting,
// in shared memory: the Jacobi-scaled PPE and its Galerkin products are
// diagonally dominant M-matrices, whose pivots stay positive) and forms the
// inverse by m forward/back substitutions in parallel, one right-hand side
// per thread (the solution columns in global memory, coalesced across the
// threads).  Each visit of the level then is one mat-vec z = A^-1 r, a warp
// per row, in place of the Jacobi sweeps and the levels below.  Cells with
// no particle (zero diagonal) are decoupled rows whose z stays 0; if a
// pivot is not positive and finite the scene falls back to z = D^-1 r.
template <typename T>
__global__ void __launch_bounds__(1024) k_mg_exact_factor(Dev D, __grid_constant__ const MgExact E) {
    BS_PDL_ENTRY();
    const int k = blockIdx.x;
    const int l = E.l[k];
    if (l <= 0) return;
    const int nx = E.nx[k], ny = E.ny[k], m = nx * ny;
    if (m <= 0 || m > BS_MG_EXACT_MAX) return;
    const int b = ny + 1, W = 2 * b + 1;
    extern __shared__ double band[];   // row i: columns i-b .. i+b
    __shared__ int bad;
    const MgDev& M = D.mg;
    const T* __restrict__ A = (const T*)M.A[l];
    const long n = M.n[l];
    const int off = E.off[k];
    for (int e = threadIdx.x; e < m * W; e += blockDim.x) band[e] = 0.0;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
        const int i = q % ny, j = q / ny;
        const double dq = (double)A[4 * n + off + q];
        if (dq == 0.0) {   // no particle in the cell: an identity row (its r is 0)
            band[q * W + b] = 1.0;
            continue;
        }
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            const int ni = i + (t % 3) - 1, nj = j + (t / 3) - 1;
            if (ni < 0 || nj < 0 || ni >= ny || nj >= nx) continue;
            band[q * W + (nj * ny + ni - q + b)] = (double)A[t * n + off + q];
        }
    }
    __syncthreads();
    for (int kk = 0; kk < m; ++kk) {
        const double piv = band[kk * W + b];
        const int nr = min(m - 1, kk + b) - kk;
        if (threadIdx.x < nr) {
            const int i = kk + 1 + threadIdx.x;
            band[i * W + (kk - i + b)] /= piv;
        }
        if (threadIdx.x == 0 && !(piv > 0.0 && isfinite(piv))) bad = 1;
        __syncthreads();
        for (int e = threadIdx.x; e < nr * nr; e += blockDim.x) {
            const int i = kk + 1 + e / nr, jc = kk + 1 + e % nr;
            band[i * W + (jc - i + b)] -= band[i * W + (kk - i + b)] * band[kk * W + (jc - kk + b)];
        }
        __syncthreads();
    }
    double* X = M.xinv + (long)k * BS_MG_EXACT_MAX * BS_MG_EXACT_MAX;
    T* Ai = (T*)M.ainv + (long)k * BS_MG_EXACT_MAX * BS_MG_EXACT_MAX;
    if (bad) {
        const T* dinv = (const T*)M.dinv[l] + off;
        for (long e = threadIdx.x; e < (long)m * m; e += blockDim.x) Ai[e] = (e / m == e % m) ? dinv[e / m] : (T)0;
        return;
    }
    // column t of the inverse: L y = e_t (unit lower), then U x = y; X[i m + t]
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
        for (int i = 0; i < m; ++i) {
            double y = (i == t) ? 1.0 : 0.0;
            for (int c = max(0, i - b); c < i; ++c) y -= band[i * W + (c - i + b)] * X[(long)c * m + t];
            X[(long)i * m + t] = y;
        }
        for (int i = m - 1; i >= 0; --i) {
            double x = X[(long)i * m + t];
            for (int c = i + 1; c <= min(m - 1, i + b); ++c) x -= band[i * W + (c - i + b)] * X[(long)c * m + t];
            X[(long)i * m + t] = x / band[i * W + b];
        }
    }
    __syncthreads();
    for (long e = threadIdx.x; e < (long)m * m; e += blockDim.x) Ai[e] = (T)X[e];
}

// z = A^-1 r on a scene's exactly solved level (added to z with acc): a warp
// per row, lanes over the row, a fixed-order sum
template <typename T>
__global__ void k_mg_exact_apply(Dev D, __grid_constant__ const MgLevel F, int acc) {
    BS_PDL_ENTRY();
    const int k = blockIdx.y;
    if (F.lev[k] != F.l) return;
    const int m = F.nx[k] * F.ny[k];
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= m) return;
    const T* __restrict__ Ai = (const T*)D.mg.ainv + (long)k * BS_MG_EXACT_MAX * BS_MG_EXACT_MAX + (long)q * m;
    const T* __restrict__ r = (const T*)D.mg.r[F.l] + F.off[k];
    T a = 0;
    for (int p = lane; p < m; p += 32) a += Ai[p] * r[p];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) {
        T* z = (T*)D.mg.z[F.l] + F.off[k];
        z[q] = acc ? z[q] + a : a;
    }
}

// ---- the levels from l0 down in one launch: one thread-block cluster per
// scene (cluster rank r, nt threads over the cluster, one cell per thread
// on the first level), the visit's level operations in order, a cluster
// barrier (release / acquire: the level arrays in global memory, L2
// resident) between them in place of a kernel boundary.  The coarsest-level
// solve runs in the cluster's first block.  Every thread reaches every
// barrier (no early exit).
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned cluster_size() {
    unsigned n;
    asm("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
    return n;
}

template <typename T>
__global__ void __launch_bounds__(1024) k_mg_sub(Dev D, __grid_constant__ const MgSub S) {
    BS_PDL_ENTRY();
    extern __shared__ unsigned char smem[];
    const int cs = (int)cluster_size();
    const int k = blockIdx.x / cs, rank = blockIdx.x % cs;
    const int t = rank * blockDim.x + threadIdx.x, nt = cs * blockDim.x;
    for (int o = 0; o < S.nops; ++o) {
        const int l = S.lv[o];
        const MgLevel& F = S.G[l - S.l0];
        const LevelS f = view_of(F, k);
        switch (S.op[o]) {
            case 0: {   // down l -> l+1
                const LevelS c = view_of(S.G[l + 1 - S.l0], k);
                const int m = c.nx * c.ny;
                for (int q = t; q < m; q += nt) op_down<T>(D.mg, f, c, q);
                break;
            }
            case 1: {   // residual on l
                const int m = f.nx * f.ny;
                for (int q = t; q < m; q += nt) op_resid<T>(D.mg, f, q);
                break;
            }
            case 2: {   // up l+1 -> l (the coarse solve wrote the scene's coarsest level)
                if (l >= F.lev[k]) break;
                const LevelS c = view_of(S.G[l + 1 - S.l0], k);
                const int m = f.nx * f.ny;
                for (int q = t; q < m; q += nt) op_up<T>(D.mg, f, c, S.acc[o], q);
                break;
            }
            default:   // coarsest-level solve of the scenes whose coarsest level is l
                if (rank == 0 && F.lev[k] == l) op_coarse<T>(D.mg, f, S.acc[o], (T*)smem);
                break;
        }
        cluster_sync_all();
    }
}

// Level 0 post-sweep after the prolongation; writes the preconditioned
// vector (FP64).
// mode 0: one sweep from zz into out; with two post-sweeps (mg_post0 = 2)
// mode 1 sweeps zz into u (free after the prolongation) and mode 2 u into out.
template <typename T>
__global__ void k_mg_l0_up(Dev D, double* __restrict__ out, int mode) {
    BS_PDL_ENTRY();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = D.blk_scene[r / BS_ALIGN];
    if (mg_skip(D, s)) return;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const T* __restrict__ zz = (const T*)(mode == 2 ? D.mg.u : D.mg.zz);
    const T* __restrict__ A = (const T*)(sizeof(T) == 8 ? D.aval : (void*)D.aval32);
    const int* __restrict__ idx = D.nidx;
    const T zr = zz[r];
    const T ax = ell_dot<T>(A, idx, zz, r, D.ncount[r], D.kmax, ((const T*)D.mg.adiagT)[r] * zr);
    const T x = ((const T*)D.mg.xin)[r];
    const T v = zr + (T)D.mg.omega * ((const T*)D.mg.dinv0)[r] * (x - ax);
    if (mode == 1) {
        ((T*)D.mg.u)[r] = v;
    } else {
        out[r] = (double)v;
        if (sizeof(T) == 4 && D.zf) D.zf[r] = (float)v;   // the FGMRES pass reads it in FP32
    }
}

inline unsigned gdiv(long a, int b) { return (unsigned)((a + b - 1) / b); }

template <typename T>
void setup_t(const Dev& D, const Launch& L) {
    int q = tbegin(L, K_MG_GAL0);
    launch_pdl(L, k_mg_dinv0<T>, L.nblk_rows, BS_THREADS, 0, D);
    launch_pdl(L, k_mg_gal0<T>, gdiv((long)D.ncell_total * 32, BS_THREADS), BS_THREADS, 0, D);
    tend(L, q);
    *L.launches += 1;
    for (int l = 1; l < D.mg.nlev; ++l) {
        if (D.mg.exact && !(L.mgneed[l + 1] & 1)) break;   // below every scene's exact level
        q = tbegin(L, K_MG_GALC);
        launch_pdl(L, k_mg_galc<T>, gdiv(D.mg.n[l + 1], 128), 128, 0, D, l);
        tend(L, q);
    }
    if (D.mg.exact && L.exact) {
        q = tbegin(L, K_MG_GALC);
        launch_pdl(L, k_mg_exact_factor<T>, D.nscene, 1024, BS_MG_EXACT_BAND * sizeof(double), D, *L.exact);
        tend(L, q);
    }
}

// op list of one visit of level l (the recursion of cycle_t)
void sub_ops(const Dev& D, const Launch& L, int l, int acc, MgSub& S) {
    const unsigned char need = L.mgneed[l];
    if (!(need & 1)) return;
    auto push = [&](int op, int lv, int a) {
        if (S.nops < BS_MG_MAXOPS) {
            S.op[S.nops] = (unsigned char)op;
            S.lv[S.nops] = (unsigned char)lv;
            S.acc[S.nops] = (unsigned char)a;
        }
        S.nops++;
    };
    if (need & 4) push(3, l, acc);
    if (!(need & 2)) return;
    push(0, l, 0);
    sub_ops(D, L, l + 1, 0, S);
    if (l <= D.mg.wlev) {
        push(1, l + 1, 0);
        sub_ops(D, L, l + 1, 1, S);
    }
    push(2, l, acc);
}

// Cycle on level l >= 1 (input r[l], output z[l]); acc: add to z[l].
// Levels 1..wlev visit level l+1 twice (W), deeper levels once (V).
// Levels no scene needs launch nothing.  From the subtree level down, one
// clustered launch per visit.
template <typename T>
void cycle_t(const Dev& D, const Launch& L, int l, int acc) {
    const MgLevel* G = L.mglev;
    const unsigned char need = L.mgneed[l];
    if (!(need & 1)) return;
    int q;
    if (l == L.mgtail) {   // this level and the coarsest below it: one block per scene
        q = tbegin(L, K_MG_TAIL);
        launch_pdl(L, k_mg_tail<T>, D.nscene, BS_MG_TAIL_F, 0, D, G[l], G[l + 1], acc, l <= D.mg.wlev ? 1 : 0);
        tend(L, q);
        return;
    }
    if (l == L.mgsub_level) {   // this level and everything below: one clustered launch
        MgSub S;
        S.l0 = l;
        S.nops = 0;
        sub_ops(D, L, l, acc, S);
        for (int u = 0; u < BS_MG_SUBL && l + u <= D.mg.nlev; ++u) S.G[u] = G[l + u];
        q = tbegin(L, K_MG_SUB);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(D.nscene * L.mgsub_cs));
        cfg.blockDim = dim3(1024);
        cfg.dynamicSmemBytes = 2 * D.mg.coarse_max * sizeof(T);
        cfg.stream = L.stream;
        cudaLaunchAttribute at[2];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)L.mgsub_cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 2;
        cudaLaunchKernelEx(&cfg, k_mg_sub<T>, D, S);
        tend(L, q);
        return;
    }
    if (need & 4) {
        q = tbegin(L, K_MG_COARSE);
        if (D.mg.exact)
            launch_pdl_2d(L, k_mg_exact_apply<T>, dim3(BS_MG_EXACT_MAX / 8, D.nscene), 256, 0, D, G[l], acc);
        else
            launch_pdl(L, k_mg_coarse<T>, D.nscene, 256, 2 * D.mg.coarse_max * sizeof(T), D, G[l], acc);
        tend(L, q);
    }
    if (!(need & 2)) return;
    q = tbegin(L, K_MG_DOWN);
    launch_pdl(L, k_mg_down<T>, gdiv(4L * D.mg.n[l + 1], 128), 128, 0, D, G[l], G[l + 1]);
    tend(L, q);
    cycle_t<T>(D, L, l + 1, 0);
    if (l <= D.mg.wlev) {
        q = tbegin(L, K_MG_RESID);
        launch_pdl(L, k_mg_resid<T>, gdiv(D.mg.n[l + 1], 128), 128, 0, D, G[l + 1]);
        tend(L, q);
        cycle_t<T>(D, L, l + 1, 1);
    }
    q = tbegin(L, K_MG_UP);
    launch_pdl(L, k_mg_up<T>, gdiv(D.mg.n[l], 128), 128, 0, D, G[l], G[l + 1], acc);
    tend(L, q);
}

template <typename T>
void apply_t(const Dev& D, const Launch& L, const double* in, double* out) {
    (void)in;   // the Krylov stream already wrote the input (mg_put_input)
    int q = tbegin(L, K_MG_L0DOWN);
    launch_pdl(L, k_mg_l0_resid<T>, row_blocks(L, L.mg0_tpb), L.mg0_tpb, 0, D);
    tend(L, q);
    q = tbegin(L, K_MG_L0REST);
    launch_pdl(L, k_mg_l0_down<T>, gdiv((long)D.ncell_total * 4, 128), 128, 0, D);
    tend(L, q);
    cycle_t<T>(D, L, 1, 0);
    q = tbegin(L, K_MG_PROLONG);
    launch_pdl(L, k_mg_l0_prolong<T>, row_blocks(L, L.mg0_tpb), L.mg0_tpb, 0, D);
    tend(L, q);
    q = tbegin(L, K_MG_L0UP);
    if (D.mg.post0 == 2) {
        launch_pdl(L, k_mg_l0_up<T>, row_blocks(L, L.mg0_tpb), L.mg0_tpb, 0, D, out, 1);
        launch_pdl(L, k_mg_l0_up<T>, row_blocks(L, L.mg0_tpb), L.mg0_tpb, 0, D, out, 2);
        *L.launches += 1;
    } else {
        launch_pdl(L, k_mg_l0_up<T>, row_blocks(L, L.mg0_tpb), L.mg0_tpb, 0, D, out, 0);
    }
    tend(L, q);
}

}  // namespace

namespace bs {

// clusters of `cs` blocks of k_mg_sub that fit on the device at once (0: the
// cluster shape cannot be launched)
int mg_sub_max_clusters(int mg_precision, int cs, size_t smem) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)cs);
    cfg.blockDim = dim3(1024);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    cudaError_t e;
    if (mg_precision == BS_PREC_MIXED) {
        if (cs > 8) cudaFuncSetAttribute(k_mg_sub<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaOccupancyMaxActiveClusters(&n, k_mg_sub<float>, &cfg);
    } else {
        if (cs > 8) cudaFuncSetAttribute(k_mg_sub<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaOccupancyMaxActiveClusters(&n, k_mg_sub<double>, &cfg);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int mg_exact_prepare() {
    const int bytes = BS_MG_EXACT_BAND * (int)sizeof(double);
    if (cudaFuncSetAttribute(k_mg_exact_factor<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_mg_exact_factor<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
            cudaSuccess)
        return BS_E_CUDA;
    return BS_OK;
}

void mg_setup(const Dev& D, const Launch& L, int mg_precision) {
    if (mg_precision == BS_PREC_MIXED) setup_t<float>(D, L);
    else setup_t<double>(D, L);
}

void mg_apply(const Dev& D, const Launch& L, int mg_precision, const double* in, double* out) {
    if (mg_precision == BS_PREC_MIXED) apply_t<float>(D, L, in, out);
    else apply_t<double>(D, L, in, out);
}

}  // namespace bs
