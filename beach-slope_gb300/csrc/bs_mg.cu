// bs_mg.cu -- aggregation multigrid preconditioner for the PPE BiCGStab.
//
// The reference solves the Jacobi-scaled PPE with unpreconditioned FGMRES /
// BiCGStab (solver.f90:129-350); the iteration count then grows with the
// number of particles across the domain.  This V-cycle is applied as a right
// preconditioner; the Krylov recurrence, dots and the stopping test stay
// FP64, so the converged pressure is the solution of the same FP64 system.
//
// Level 0: particle rows (the sliced-ELL PPE).  Level 1: one aggregate per
// cell of the search grid -- the rows of a cell are contiguous, so the
// Galerkin product P^T A P (P = cell indicator) is a warp reduction per
// cell, and because every neighbour lies in one of the 3x3 surrounding cells
// the coarse operator is a 9-point stencil on the cell grid.  Level l+1:
// 2x2 boxes of level l, again a 9-point Galerkin stencil.  Smoother: damped
// Jacobi, one pre-sweep from zero and one post-sweep; coarsest level: Jacobi
// sweeps by one block per scene.  All kernels skip converged scenes.
// T = double (FP64 mode) or float (mixed mode, FP32 V-cycle).
#include "bs_internal.cuh"

using namespace bs;

namespace {

__device__ __forceinline__ bool mg_skip(const Dev& D, int s) { return D.dyn[s].converged != 0; }

template <typename T>
__device__ __forceinline__ const T* Ap(const Dev& D, int l) { return (const T*)D.mg.A[l]; }

// ------------------------------------------------------------ setup
// level 0: 1/adiag per row
template <typename T>
__global__ void k_mg_dinv0(Dev D) {
    const int s = D.blk_scene[blockIdx.x];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const double d = D.adiag[r];
    ((T*)D.mg.dinv0)[r] = (d != 0.0 && isfinite(d)) ? (T)(1.0 / d) : (T)0;
    ((T*)D.mg.adiagT)[r] = (T)d;
}

// level 1 = P^T A0 P: one warp per cell
template <typename T>
__global__ void k_mg_gal0(Dev D) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= D.ncell_total) return;
    const int s = D.cell_scene[c];
    const int celly = D.par[s].celly;
    const int r0 = D.cell_start[c], r1 = D.cell_end[c];
    const double* A = (const double*)D.aval;
    double acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.0;
    for (int r = r0 + lane; r < r1; r += 32) {
        acc[4] += D.adiag[r];
        const int n = D.ncount[r];
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, D.kmax);
            const int d = D.cell[D.nidx[e]] - c;
            const int dj = (d + celly + 1) / celly - 1;
            const int di = d - dj * celly;
            const int q = (dj + 1) * 3 + (di + 1);
            const double v = A[e];
#pragma unroll
            for (int t = 0; t < 9; ++t)
                if (t == q) acc[t] += v;
        }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k)
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    if (lane == 0) {
        T* Al = (T*)D.mg.A[1];
        const int n1 = D.mg.n[1];
#pragma unroll
        for (int k = 0; k < 9; ++k) Al[(long)k * n1 + c] = (T)acc[k];
        ((T*)D.mg.dinv[1])[c] = (acc[4] != 0.0 && isfinite(acc[4])) ? (T)(1.0 / acc[4]) : (T)0;
    }
}

// level l+1 from level l: one thread per coarse cell
template <typename T>
__global__ void k_mg_galc(Dev D, int l) {
    const int Q = blockIdx.x * blockDim.x + threadIdx.x;
    const MgDev& M = D.mg;
    if (Q >= M.n[l + 1]) return;
    const int s = M.scene_of[l + 1][Q];
    const int q = Q - M.off[l + 1][s];
    const int nyc = M.ny[l + 1][s];
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

// ------------------------------------------------------------ V-cycle
// Level 0 pre-smooth from zero (z0 = w D^-1 in), residual, restriction to
// the cells: r1[c] = sum_{i in c} (in_i - (A0 z0)_i).  One warp per cell.
template <typename T>
__global__ void k_mg_l0_down(Dev D) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= D.ncell_total) return;
    const int s = D.cell_scene[c];
    if (mg_skip(D, s)) return;
    const T* __restrict__ xin = (const T*)D.mg.xin;
    const T* __restrict__ u = (const T*)D.mg.u;
    const T* __restrict__ ad = (const T*)D.mg.adiagT;
    const T* __restrict__ A = (const T*)(sizeof(T) == 8 ? D.aval : (void*)D.aval32);
    const int* __restrict__ idx = D.nidx;
    const int r0 = D.cell_start[c], r1 = D.cell_end[c];
    T sum = 0;
    if (!D.mg.pre0) {   // no pre-smoothing: restrict the input itself
        for (int r = r0 + lane; r < r1; r += 32) sum += xin[r];
    } else {
        for (int r = r0 + lane; r < r1; r += 32) {
            T ax = ad[r] * u[r];
            const int n = D.ncount[r];
            long e = ell(r, 0, D.kmax);
            for (int k = 0; k < n; ++k, e += 32) ax += __ldg(A + e) * u[__ldg(idx + e)];
            sum += xin[r] - ax;
        }
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) ((T*)D.mg.r[1])[c] = sum;
}

// zz = u + cscale * e1[cell]: the level-0 value after the coarse correction
template <typename T>
__global__ void k_mg_l0_prolong(Dev D) {
    const int s = D.blk_scene[blockIdx.x];
    if (mg_skip(D, s)) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const T pre = D.mg.pre0 ? ((const T*)D.mg.u)[r] : (T)0;
    ((T*)D.mg.zz)[r] = pre + (T)D.mg.cscale * ((const T*)D.mg.z[1])[D.cell[r]];
}

template <typename T>
struct LevelView {
    const T* A;
    const T* dinv;
    const T* r;
    int n, off, nx, ny;
};

template <typename T>
__device__ __forceinline__ LevelView<T> view(const MgDev& M, int l, int s) {
    LevelView<T> v;
    v.A = (const T*)M.A[l];
    v.dinv = (const T*)M.dinv[l];
    v.r = (const T*)M.r[l];
    v.n = M.n[l];
    v.off = M.off[l][s];
    v.nx = M.nx[l][s];
    v.ny = M.ny[l][s];
    return v;
}

// Levels l -> l+1: pre-smooth from zero, residual, restriction (2x2 sum).
template <typename T>
__global__ void k_mg_down(Dev D, int l) {
    const int Q = blockIdx.x * blockDim.x + threadIdx.x;
    const MgDev& M = D.mg;
    if (Q >= M.n[l + 1]) return;
    const int s = M.scene_of[l + 1][Q];
    if (mg_skip(D, s)) return;
    const int q = Q - M.off[l + 1][s];
    const int nyc = M.ny[l + 1][s];
    const int I = q % nyc, J = q / nyc;
    const LevelView<T> F = view<T>(M, l, s);
    const T w = (T)M.omega;
    T sum = 0;
    for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a) {
            const int fi = 2 * I + a, fj = 2 * J + b;
            if (fi >= F.ny || fj >= F.nx) continue;
            const int c = F.off + fj * F.ny + fi;
            if (!M.prec) {
                sum += F.r[c];
                continue;
            }
            T ax = 0;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const int ni = fi + (k % 3) - 1, nj = fj + (k / 3) - 1;
                if (ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx) continue;
                const int nb = F.off + nj * F.ny + ni;
                ax += F.A[(long)k * F.n + c] * (w * F.r[nb] * F.dinv[nb]);
            }
            sum += F.r[c] - ax;
        }
    ((T*)M.r[l + 1])[Q] = sum;
}

// Coarsest level: damped Jacobi sweeps from zero, one block per scene.
template <typename T>
__global__ void k_mg_coarse(Dev D) {
    const int s = blockIdx.x;
    if (mg_skip(D, s)) return;
    const MgDev& M = D.mg;
    const int L = D.par[s].mg_lev;
    const LevelView<T> C = view<T>(M, L, s);
    const int m = C.nx * C.ny;
    extern __shared__ unsigned char smem[];
    T* z = (T*)smem;
    T* z2 = z + M.coarse_max;
    const T w = (T)M.omega;
    for (int q = threadIdx.x; q < m; q += blockDim.x) z[q] = 0;
    __syncthreads();
    for (int it = 0; it < M.coarse_sweeps; ++it) {
        for (int q = threadIdx.x; q < m; q += blockDim.x) {
            const int i = q % C.ny, j = q / C.ny;
            const int c = C.off + q;
            T ax = 0;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const int ni = i + (k % 3) - 1, nj = j + (k / 3) - 1;
                if (ni < 0 || nj < 0 || ni >= C.ny || nj >= C.nx) continue;
                ax += C.A[(long)k * C.n + c] * z[nj * C.ny + ni];
            }
            z2[q] = z[q] + w * C.dinv[c] * (C.r[c] - ax);
        }
        __syncthreads();
        for (int q = threadIdx.x; q < m; q += blockDim.x) z[q] = z2[q];
        __syncthreads();
    }
    T* out = (T*)M.z[L];
    for (int q = threadIdx.x; q < m; q += blockDim.x) out[C.off + q] = z[q];
}

// Levels l+1 -> l: prolongation (constant per box, scaled) + one post-sweep.
template <typename T>
__global__ void k_mg_up(Dev D, int l) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const MgDev& M = D.mg;
    if (c >= M.n[l]) return;
    const int s = M.scene_of[l][c];
    if (mg_skip(D, s) || l >= D.par[s].mg_lev) return;   // the coarse solve wrote this level
    const LevelView<T> F = view<T>(M, l, s);
    const int q = c - F.off;
    const int i = q % F.ny, j = q / F.ny;
    const int nyc = M.ny[l + 1][s], oc = M.off[l + 1][s];
    const T* e = (const T*)M.z[l + 1];
    const T w = (T)M.omega, cs = (T)M.cscale;
    const T wp = M.prec ? w : (T)0;
    auto zval = [&](int ii, int jj) -> T {
        const int nb = F.off + jj * F.ny + ii;
        return wp * F.r[nb] * F.dinv[nb] + cs * e[oc + (jj / 2) * nyc + (ii / 2)];
    };
    const T zc = zval(i, j);
    T ax = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int ni = i + (k % 3) - 1, nj = j + (k / 3) - 1;
        if (ni < 0 || nj < 0 || ni >= F.ny || nj >= F.nx) continue;
        ax += F.A[(long)k * F.n + c] * (k == 4 ? zc : zval(ni, nj));
    }
    ((T*)M.z[l])[c] = zc + w * F.dinv[c] * (F.r[c] - ax);
}

// Level 0 post-sweep after the prolongation; writes the preconditioned
// vector (FP64).
template <typename T>
__global__ void k_mg_l0_up(Dev D, double* __restrict__ out) {
    const int s = D.blk_scene[blockIdx.x];
    if (mg_skip(D, s)) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const T* __restrict__ zz = (const T*)D.mg.zz;
    const T* __restrict__ A = (const T*)(sizeof(T) == 8 ? D.aval : (void*)D.aval32);
    const int* __restrict__ idx = D.nidx;
    const T zr = zz[r];
    T ax = ((const T*)D.mg.adiagT)[r] * zr;
    const int n = D.ncount[r];
    long e = ell(r, 0, D.kmax);
    int k = 0;
    for (; k + 2 <= n; k += 2, e += 64) {
        const int j0 = __ldg(idx + e), j1 = __ldg(idx + e + 32);
        const T a0 = __ldg(A + e), a1 = __ldg(A + e + 32);
        ax += a0 * zz[j0];
        ax += a1 * zz[j1];
    }
    if (k < n) ax += __ldg(A + e) * zz[__ldg(idx + e)];
    const T x = ((const T*)D.mg.xin)[r];
    out[r] = (double)(zr + (T)D.mg.omega * ((const T*)D.mg.dinv0)[r] * (x - ax));
}

inline unsigned gdiv(long a, int b) { return (unsigned)((a + b - 1) / b); }

template <typename T>
void setup_t(const Dev& D, const Launch& L) {
    int q = tbegin(L, K_MG_GAL0);
    k_mg_dinv0<T><<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D);
    k_mg_gal0<T><<<gdiv((long)D.ncell_total * 32, BS_THREADS), BS_THREADS, 0, L.stream>>>(D);
    tend(L, q);
    *L.launches += 1;
    for (int l = 1; l < D.mg.nlev; ++l) {
        q = tbegin(L, K_MG_GALC);
        k_mg_galc<T><<<gdiv(D.mg.n[l + 1], 128), 128, 0, L.stream>>>(D, l);
        tend(L, q);
    }
}

template <typename T>
void apply_t(const Dev& D, const Launch& L, const double* in, double* out) {
    (void)in;   // the Krylov stream already wrote the input (mg_put_input)
    int q = tbegin(L, K_MG_L0DOWN);
    k_mg_l0_down<T><<<gdiv((long)D.ncell_total * 32, BS_THREADS), BS_THREADS, 0, L.stream>>>(D);
    tend(L, q);
    for (int l = 1; l < D.mg.nlev; ++l) {
        q = tbegin(L, K_MG_DOWN);
        k_mg_down<T><<<gdiv(D.mg.n[l + 1], 128), 128, 0, L.stream>>>(D, l);
        tend(L, q);
    }
    q = tbegin(L, K_MG_COARSE);
    k_mg_coarse<T><<<D.nscene, 256, 2 * D.mg.coarse_max * sizeof(T), L.stream>>>(D);
    tend(L, q);
    for (int l = D.mg.nlev - 1; l >= 1; --l) {
        q = tbegin(L, K_MG_UP);
        k_mg_up<T><<<gdiv(D.mg.n[l], 128), 128, 0, L.stream>>>(D, l);
        tend(L, q);
    }
    q = tbegin(L, K_MG_PROLONG);
    k_mg_l0_prolong<T><<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D);
    tend(L, q);
    q = tbegin(L, K_MG_L0UP);
    k_mg_l0_up<T><<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D, out);
    tend(L, q);
}

}  // namespace

namespace bs {

void mg_setup(const Dev& D, const Launch& L, int mg_precision) {
    if (mg_precision == BS_PREC_MIXED) setup_t<float>(D, L);
    else setup_t<double>(D, L);
}

void mg_apply(const Dev& D, const Launch& L, int mg_precision, const double* in, double* out) {
    if (mg_precision == BS_PREC_MIXED) apply_t<float>(D, L, in, out);
    else apply_t<double>(D, L, in, out);
}

}  // namespace bs
