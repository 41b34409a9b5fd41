// bs_solver.cu -- batched BiCGStab on the Jacobi-scaled PPE (bicgstab,
// solver.f90:129-254, on the padded-ELL operator spmv2, solver.f90:84-127).
//
// One iteration = three kernels over all scenes:
//   K1: p <- r + beta (p - omega v) folded into v <- A p  (gathers r,p,v)
//   K2: s <- r - alpha v folded into t <- A s            (gathers r,v)
//   K3: x <- x + alpha p + omega s ; r <- s - omega t
// Each kernel ends with per-scene FP64 dot products: block partials plus a
// deterministic finisher (the last block of the scene sums the partials in
// block order and updates the scene's scalars).  Converged scenes return at
// the top of every kernel.  FP64 mode: all vectors FP64.  Mixed mode: the
// inner iteration runs on FP32 vectors and FP32 matrix values; the outer
// loop recomputes the true residual with the FP64 matrix and corrects x
// (iterative refinement), with FP64 dots throughout.
#include <cstring>

#include "bs_internal.cuh"

namespace {

// Sum NV values over the scene's blocks; returns true in the finisher block
// (thread 0 holds the totals in tot[]).
template <int NV>
__device__ __forceinline__ bool scene_sum(const Dev& D, int s, double (&v)[NV], double (&tot)[NV]) {
    __shared__ double sh[NV * 32];
    __shared__ int last;
    const ScenePar& P = D.par[s];
    block_sum<NV>(v, sh);
    if (threadIdx.x == 0) {
        double* part = D.part + (long)blockIdx.x * BS_MAXDOT;
#pragma unroll
        for (int q = 0; q < NV; ++q) part[q] = v[q];
        __threadfence();
        const int prev = atomicAdd(&D.blk_done[s], 1);
        last = (prev == P.nblk - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double a[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) a[q] = 0.0;
    for (int b = threadIdx.x; b < P.nblk; b += blockDim.x) {
        const double* part = D.part + (long)(P.blk0 + b) * BS_MAXDOT;
#pragma unroll
        for (int q = 0; q < NV; ++q) a[q] += __ldcg(part + q);
    }
    __syncthreads();
    block_sum<NV>(a, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) tot[q] = a[q];
        D.blk_done[s] = 0;
    }
    return true;
}

__device__ __forceinline__ bool scene_done(const Dev& D, int s) { return D.dyn[s].converged != 0; }

// ---------------------------------------------------------------- FP64
__global__ void k_init64(Dev D, int* nconv) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (r < P.row0 + D.dyn[s].n) {
        const double* A = (const double*)D.aval;
        double acc = D.adiag[r] * D.p[r];
        const int n = D.ncount[r];
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, D.kmax);
            acc += A[e] * D.p[D.nidx[e]];
        }
        const double b = D.rhs[r];
        const double rr = b - acc;
        D.sr[r] = rr;
        D.srhat[r] = rr;
        D.sp[r] = 0.0;
        D.sv[r] = 0.0;
        v[0] = b * b;
        v[1] = rr * rr;
    }
    double tot[2];
    if (scene_sum<2>(D, s, v, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        Y.bnorm2 = tot[0];
        Y.rnorm2 = tot[1];
        Y.rho_old = tot[1];
        Y.alpha = 1.0;
        Y.omega = 1.0;
        Y.beta = 0.0;
        Y.iters = 0;
        Y.breakdown = 0;
        Y.outer = 0;
        Y.part_tmp = 0.0;
        const bool conv = (tot[0] == 0.0) || (tot[1] <= P.ppe_tol * P.ppe_tol * tot[0]);
        Y.converged = conv;
        if (conv) atomicAdd(nconv, 1);
    }
}

// KP: p = r + beta (p - omega v)   (streaming; beta = 0 on the first iteration);
// also writes the V-cycle input (mgmode 1: FP64, 2: FP32)
__global__ void k_pupd64(Dev D, int mgmode) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (scene_done(D, s)) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const double beta = D.dyn[s].beta, omega = D.dyn[s].omega;
    const double p = D.sr[r] + beta * (D.sp[r] - omega * D.sv[r]);
    D.sp[r] = p;
    if (mgmode == 1) bs::mg_put_input<double>(D, r, p);
    else if (mgmode == 2) bs::mg_put_input<float>(D, r, p);
}

// y = A u for one row (1 DFMA per nonzero)
__device__ __forceinline__ double spmv_row64(const Dev& D, const double* __restrict__ u, int r) {
    const double* __restrict__ A = (const double*)D.aval;
    const int* __restrict__ idx = D.nidx;
    const int n = D.ncount[r];
    const int kmax = D.kmax;
    double acc = D.adiag[r] * u[r];
    long e = ell(r, 0, kmax);
    int k = 0;
    for (; k + 4 <= n; k += 4, e += 128) {   // four independent gathers in flight
        const int j0 = __ldg(idx + e), j1 = __ldg(idx + e + 32), j2 = __ldg(idx + e + 64), j3 = __ldg(idx + e + 96);
        const double a0 = __ldg(A + e), a1 = __ldg(A + e + 32), a2 = __ldg(A + e + 64), a3 = __ldg(A + e + 96);
        const double u0 = u[j0], u1 = u[j1], u2 = u[j2], u3 = u[j3];
        acc += a0 * u0;
        acc += a1 * u1;
        acc += a2 * u2;
        acc += a3 * u3;
    }
    for (; k < n; ++k, e += 32) acc += __ldg(A + e) * u[__ldg(idx + e)];
    return acc;
}

// K1: v = A u (u = p, or M^-1 p when preconditioned);  partial (rhat, v);
// finisher: alpha
__global__ void k_it1_64(Dev D, const double* __restrict__ u) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (scene_done(D, s)) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double q[1] = {0.0};
    if (r < P.row0 + D.dyn[s].n) {
        const double acc = spmv_row64(D, u, r);
        D.sv[r] = acc;
        q[0] = D.srhat[r] * acc;
    }
    double tot[1];
    if (scene_sum<1>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        if (tot[0] == 0.0 || !isfinite(tot[0])) {
            Y.breakdown = 1;
            Y.alpha = 0.0;
        } else {
            Y.alpha = Y.rho_old / tot[0];
        }
    }
}

// KS: s = r - alpha v   (streaming), plus the V-cycle input as in KP
__global__ void k_supd64(Dev D, int mgmode) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (scene_done(D, s)) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const double v = D.sr[r] - D.dyn[s].alpha * D.sv[r];
    D.ss[r] = v;
    if (mgmode == 1) bs::mg_put_input<double>(D, r, v);
    else if (mgmode == 2) bs::mg_put_input<float>(D, r, v);
}

// K2: t = A u (u = s, or M^-1 s);  partials (t,s), (t,t);  finisher: omega
__global__ void k_it2_64(Dev D, const double* __restrict__ u) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (scene_done(D, s)) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double q[2] = {0.0, 0.0};
    if (r < P.row0 + D.dyn[s].n) {
        const double acc = spmv_row64(D, u, r);
        D.st[r] = acc;
        const double si = D.ss[r];
        q[0] = acc * si;
        q[1] = acc * acc;
    }
    double tot[2];
    if (scene_sum<2>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        Y.omega = (tot[1] != 0.0) ? tot[0] / tot[1] : 0.0;
        if (tot[1] == 0.0) Y.breakdown = 1;
    }
}

// K3: x += alpha pu + omega su;  r = s - omega t;  partials (rhat, r), (r,r);
// finisher: beta, convergence
__global__ void k_it3_64(Dev D, const double* __restrict__ pu, const double* __restrict__ su, int* nconv) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (scene_done(D, s)) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = D.dyn[s].alpha, omega = D.dyn[s].omega;
    double q[2] = {0.0, 0.0};
    double mrel = 0.0;
    if (r < P.row0 + D.dyn[s].n) {
        const double si = D.ss[r], ti = D.st[r];
        const double xo = D.p[r];
        const double xn = xo + alpha * pu[r] + omega * su[r];
        D.p[r] = xn;
        const double rr = si - omega * ti;
        D.sr[r] = rr;
        q[0] = D.srhat[r] * rr;
        q[1] = rr * rr;
        if (P.stop_rule == BS_STOP_REFERENCE) mrel = fabs((xn - xo) / (xo + BS_SP1EM5));
    }
    if (P.stop_rule == BS_STOP_REFERENCE) {
        __shared__ double shm[32];
        double mv[1] = {mrel};
        block_max<1>(mv, shm);
        __syncthreads();
        if (threadIdx.x == 0) atomicMax((unsigned long long*)&D.dyn[s].part_tmp, __double_as_longlong(mv[0]));
    }
    double tot[2];
    if (scene_sum<2>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        const double rho_new = tot[0];
        Y.beta = (rho_new / Y.rho_old) * (alpha / omega);
        Y.rho_old = rho_new;
        Y.rnorm2 = tot[1];
        Y.iters += 1;
        bool conv;
        if (P.stop_rule == BS_STOP_REFERENCE) {
            conv = Y.part_tmp <= (double)1e-2f;
            Y.part_tmp = 0.0;
        } else {
            conv = tot[1] <= P.ppe_tol * P.ppe_tol * Y.bnorm2;
        }
        if (!isfinite(tot[1])) {
            conv = true;
            set_err(D, s, BS_ERR_NONFINITE);
        }
        if (Y.breakdown) {
            conv = true;
            if (!(tot[1] <= P.ppe_tol * P.ppe_tol * Y.bnorm2)) set_err(D, s, BS_ERR_SOLVER_BREAK);
        }
        if (!conv && Y.iters >= P.maxit) {
            conv = true;
            set_err(D, s, BS_ERR_NOT_CONVERGED);
        }
        if (conv) {
            Y.converged = 1;
            atomicAdd(nconv, 1);
        }
    }
}

// ---------------------------------------------------------------- mixed
// Outer refinement: r64 = b - A64 x (FP64 matrix, FP64 vectors); the scene
// is done when ||r64|| <= tol ||b||.  Otherwise the inner FP32 BiCGStab
// solves A32 d = r64/||r64|| to inner_tol and x += ||r64|| d.
__global__ void k_mx_res(Dev D, int* nconv) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    const ScenePar& P = D.par[s];
    SceneDyn& Y = D.dyn[s];
    if (Y.outer < 0) return;   // outer-converged
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double q[2] = {0.0, 0.0};
    if (r < P.row0 + Y.n) {
        const double b = D.rhs[r];
        const double rr = b - spmv_row64(D, D.p, r);
        D.sxd[r] = rr;
        q[0] = rr * rr;
        q[1] = b * b;
    }
    double tot[2];
    if (scene_sum<2>(D, s, q, tot) && threadIdx.x == 0) {
        Y.rtrue2 = tot[0];
        Y.bnorm2 = tot[1];
        Y.relres = (tot[1] > 0.0) ? sqrt(tot[0] / tot[1]) : sqrt(tot[0]);
        const bool done = (tot[1] == 0.0) || (tot[0] <= P.ppe_tol * P.ppe_tol * tot[1]) || !isfinite(tot[0]);
        if (!isfinite(tot[0])) set_err(D, s, BS_ERR_NONFINITE);
        if (done || Y.outer >= P.max_outer) {
            if (!done) set_err(D, s, BS_ERR_NOT_CONVERGED);
            Y.outer = -Y.outer - 1;   // mark outer-converged, keep the count
            Y.converged = 1;
            atomicAdd(nconv + 1, 1);
        } else {
            Y.rnorm2 = tot[0];
            Y.converged = 0;
            Y.outer += 1;
        }
    }
}

// inner init: r = r64 / ||r64|| in FP32, rhat = r, p = v = d = 0
__global__ void k_mx_init(Dev D, int* nconv) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    const SceneDyn& Y0 = D.dyn[s];
    if (Y0.outer < 0) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const double scale = 1.0 / sqrt(Y0.rnorm2);
    double q[1] = {0.0};
    if (r < P.row0 + Y0.n) {
        const float rf = (float)(D.sxd[r] * scale);
        D.fr[r] = rf;
        D.frhat[r] = rf;
        D.fp[r] = 0.0f;
        D.fv[r] = 0.0f;
        D.fd[r] = 0.0f;
        q[0] = (double)rf * rf;
    }
    double tot[1];
    if (scene_sum<1>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        Y.rho_old = tot[0];
        Y.part_tmp = tot[0];   // inner ||r0||^2
        Y.alpha = 1.0;
        Y.omega = 1.0;
        Y.beta = 0.0;
        Y.breakdown = 0;
        if (tot[0] == 0.0) {
            Y.converged = 1;
            atomicAdd(nconv, 1);
        }
    }
}

__device__ __forceinline__ bool inner_done(const Dev& D, int s) {
    return D.dyn[s].outer < 0 || D.dyn[s].converged != 0;
}

// FP32 row of A32 applied to u_j = a_j + c (b_j - e g_j) evaluated on the fly
template <int MODE>
__device__ __forceinline__ float spmv_row32(const Dev& D, const float* __restrict__ a, const float* __restrict__ b,
                                            const float* __restrict__ g, float c, float e2, int r, float& own) {
    const float* __restrict__ A = (const float*)D.aval32;   // FP32 values (hi part)
    const int* __restrict__ idx = D.nidx;
    const int n = D.ncount[r];
    const int kmax = D.kmax;
    auto val = [&](int j) -> float {
        if (MODE == 0) return a[j] + c * (b[j] - e2 * g[j]);   // p = r + beta (p - omega v)
        return a[j] - c * b[j];                              // s = r - alpha v
    };
    own = val(r);
    float acc = (float)D.adiag[r] * own;
    long e = ell(r, 0, kmax);
    int k = 0;
    for (; k + 4 <= n; k += 4, e += 128) {
        const int j0 = __ldg(idx + e), j1 = __ldg(idx + e + 32), j2 = __ldg(idx + e + 64), j3 = __ldg(idx + e + 96);
        const float a0 = __ldg(A + e), a1 = __ldg(A + e + 32), a2 = __ldg(A + e + 64), a3 = __ldg(A + e + 96);
        const float u0 = val(j0), u1 = val(j1), u2 = val(j2), u3 = val(j3);
        acc = fmaf(a0, u0, acc);
        acc = fmaf(a1, u1, acc);
        acc = fmaf(a2, u2, acc);
        acc = fmaf(a3, u3, acc);
    }
    for (; k < n; ++k, e += 32) acc = fmaf(__ldg(A + e), val(__ldg(idx + e)), acc);
    return acc;
}

__global__ void k_mx_it1(Dev D, const float* __restrict__ p, const float* __restrict__ v, float* pn, float* vn) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (inner_done(D, s)) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const float beta = (float)D.dyn[s].beta, omega = (float)D.dyn[s].omega;
    double q[1] = {0.0};
    if (r < P.row0 + D.dyn[s].n) {
        float pi;
        const float acc = spmv_row32<0>(D, D.fr, p, v, beta, omega, r, pi);
        pn[r] = pi;
        vn[r] = acc;
        q[0] = (double)D.frhat[r] * acc;
    }
    double tot[1];
    if (scene_sum<1>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        if (tot[0] == 0.0 || !isfinite(tot[0])) {
            Y.breakdown = 1;
            Y.alpha = 0.0;
        } else {
            Y.alpha = Y.rho_old / tot[0];
        }
    }
}

__global__ void k_mx_it2(Dev D, const float* __restrict__ v) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (inner_done(D, s)) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const float alpha = (float)D.dyn[s].alpha;
    double q[2] = {0.0, 0.0};
    if (r < P.row0 + D.dyn[s].n) {
        float si;
        const float acc = spmv_row32<1>(D, D.fr, v, v, alpha, 0.0f, r, si);
        D.fs[r] = si;
        D.ft[r] = acc;
        q[0] = (double)acc * si;
        q[1] = (double)acc * acc;
    }
    double tot[2];
    if (scene_sum<2>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        Y.omega = (tot[1] != 0.0) ? tot[0] / tot[1] : 0.0;
        if (tot[1] == 0.0) Y.breakdown = 1;
    }
}

__global__ void k_mx_it3(Dev D, const float* __restrict__ p, int* nconv) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (inner_done(D, s)) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const float alpha = (float)D.dyn[s].alpha, omega = (float)D.dyn[s].omega;
    double q[2] = {0.0, 0.0};
    if (r < P.row0 + D.dyn[s].n) {
        const float si = D.fs[r], ti = D.ft[r];
        D.fd[r] = D.fd[r] + alpha * p[r] + omega * si;
        const float rr = si - omega * ti;
        D.fr[r] = rr;
        q[0] = (double)D.frhat[r] * rr;
        q[1] = (double)rr * rr;
    }
    double tot[2];
    if (scene_sum<2>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        const double rho_new = tot[0];
        Y.beta = (rho_new / Y.rho_old) * ((double)alpha / (double)omega);
        Y.rho_old = rho_new;
        Y.iters += 1;
        bool conv = tot[1] <= P.inner_tol * P.inner_tol * Y.part_tmp;
        if (!isfinite(tot[1]) || Y.breakdown) conv = true;
        if (Y.iters >= P.maxit) conv = true;
        if (conv) {
            Y.converged = 1;
            atomicAdd(nconv, 1);
        }
    }
}

// x += ||r64|| d
__global__ void k_mx_update(Dev D) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    const SceneDyn& Y = D.dyn[s];
    if (Y.outer < 0) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= D.par[s].row0 + Y.n) return;
    D.p[r] = D.p[r] + sqrt(Y.rnorm2) * (double)D.fd[r];
}

// FP32 copy of the assembled FP64 matrix values (inner operator): hi part
// and the remainder; nothing to do where the mixed assembly already wrote them
__global__ void k_mx_convert(Dev D) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r == D.par[s].row0) {
        D.dyn[s].outer = 0;
        D.dyn[s].iters = 0;
    }
    if (r >= D.par[s].row0 + D.dyn[s].n || D.dyn[s].asm_split) return;
    const double* A = (const double*)D.aval;
    float* F = D.aval32;
    const int n = D.ncount[r];
    for (int k = 0; k < n; ++k) {
        const long e = ell(r, k, D.kmax);
        const float h = (float)A[e];
        F[e] = h;
        D.aval_lo[e] = __double2float_rn(__dsub_rn(A[e], (double)h));
    }
}

// true FP64 residual ||b - A x|| / ||b|| for every scene (no early exit)
__global__ void k_true_res64(Dev D) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double q[2] = {0.0, 0.0};
    if (r < P.row0 + D.dyn[s].n) {
        const double* A = (const double*)D.aval;
        double acc = D.adiag[r] * D.p[r];
        const int n = D.ncount[r];
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, D.kmax);
            acc += A[e] * D.p[D.nidx[e]];
        }
        const double b = D.rhs[r];
        const double rr = b - acc;
        q[0] = rr * rr;
        q[1] = b * b;
    }
    double tot[2];
    if (scene_sum<2>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        Y.rtrue2 = tot[0];
        Y.relres = (tot[1] > 0.0) ? sqrt(tot[0] / tot[1]) : sqrt(tot[0]);
    }
}

// ---------------------------------------------------------------- FGMRES
// Restarted flexible GMRES (Saad, SIAM J. Sci. Comput. 14, 1993), the Krylov
// method of the reference's live solver (fgmres, solver.f90:306-350: MKL's
// RCI dfgmres with spmv2 as the operator, the previous pressure as the first
// guess, memory.f90:144, isph.f90:477).  Per scene: r0 = b - A x0, v0 =
// r0/||r0||; column j: z_j = M^-1 v_j (the multigrid cycle; z_j = v_j
// unpreconditioned), w = A z_j, classical Gram-Schmidt against v_0..v_j
// applied twice in two passes over the basis (the second projection from
// the basis' Gram matrix), h_{j+1,j} = ||w||, v_{j+1} = w / h_{j+1,j}; Givens rotations keep
// the least-squares residual |g_{j+1}| current.  The cycle ends when |g_{j+1}|
// <= ref, h_{j+1,j} <= 1e-12 (lucky breakdown), j+1 = m (restart) or at the
// iteration cap; then y = R^-1 g and x += Z y.  Scenes run their cycles in lock
// step; a scene whose cycle ended returns at the top of every column kernel,
// and the column index lives in the scene's state, so one captured chunk of
// columns serves every cycle.
//
// Two forms of a column.  FP64 basis (fg_df = 0): k_fg_put writes v_j and the
// V-cycle input, pass 1 (k_fg_arn1<0>) the SpMV and the dots, pass 2
// (k_fg_arn2<0>) the projection, the norm and, in its finisher, the
// rotations.  Double-float basis (fg_df = 1, the preconditioned mixed solve):
// the basis is stored as (hi, lo) FP32 pairs and its dots and projection run
// on the FP32 pipe; pass 1 (k_fg_arn1<1>) also sums u.u and its finisher takes
// h_{j+1,j} from the Gram relation and runs the rotations, so pass 2
// (k_fg_arn2<1>) streams v_{j+1} and the next V-cycle input with no reduction
// and k_fg_put runs once per cycle.

// Per-scene small storage: H [(m+1) x m] column-major (R of the rotated
// Hessenberg matrix), Gm [(m+1) x (m+1)] (the Gram matrix V^T V of the
// basis), cs[m], sn[m], g[m+1], y[m], hc[m+1] (the column's coefficients)
struct FgSmall {
    double *H, *Gm, *cs, *sn, *g, *y, *hc;
};
__device__ __forceinline__ FgSmall fg_small(const Dev& D, int s) {
    const int m = D.fg_m;
    double* b = D.fg_small + (long)s * D.fg_small_n;
    FgSmall f;
    f.H = b;
    b += (long)(m + 1) * m;
    f.Gm = b;
    b += (long)(m + 1) * (m + 1);
    f.cs = b;
    b += m;
    f.sn = b;
    b += m;
    f.g = b;
    b += m + 1;
    f.y = b;
    b += m;
    f.hc = b;
    return f;
}

__device__ __forceinline__ bool fg_running(const Dev& D, int s) {
    return D.dyn[s].converged == 0 && D.dyn[s].fg_state == 0;
}

__device__ __forceinline__ double warp_sum(double a) {
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    return a;
}

// Double-float arithmetic (a value as an unevaluated sum hi + lo of two FP32
// numbers, 48 significant bits; Dekker 1971, Knuth's TwoSum, the FMA form of
// TwoProduct) for the Gram-Schmidt passes of the mixed solve: a basis element
// is 8 bytes as in FP64, and its products and sums run on the FP32 pipe, which
// on this part is ~60x faster than the FP64 pipe that bounds the FP64 form.
// Intrinsics keep every rounding explicit (no contraction).
__device__ __forceinline__ float2 df_split(double a) {
    const float h = __double2float_rn(a);
    return make_float2(h, __double2float_rn(__dsub_rn(a, (double)h)));
}
__device__ __forceinline__ double df_to_double(float2 a) { return __dadd_rn((double)a.x, (double)a.y); }
// s += a * b (products to ~2^-48 relative: TwoProduct of the high parts plus
// the cross terms; TwoSum into the running high part, errors into the low)
__device__ __forceinline__ void df_fma(float2& s, float2 a, float2 b) {
    const float ph = __fmul_rn(a.x, b.x);
    float pe = __fmaf_rn(a.x, b.x, -ph);
    pe = __fmaf_rn(a.x, b.y, pe);
    pe = __fmaf_rn(a.y, b.x, pe);
    const float t = __fadd_rn(s.x, ph);
    const float v = __fsub_rn(t, s.x);
    const float e = __fadd_rn(__fsub_rn(s.x, __fsub_rn(t, v)), __fsub_rn(ph, v));
    s.y = __fadd_rn(s.y, __fadd_rn(e, pe));
    s.x = t;
}
// a + b, renormalised
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float t = __fadd_rn(a.x, b.x);
    const float v = __fsub_rn(t, a.x);
    float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(t, v)), __fsub_rn(b.x, v));
    e = __fadd_rn(e, __fadd_rn(a.y, b.y));
    const float h = __fadd_rn(t, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, t)));
}
__device__ __forceinline__ float2 df_shfl_xor(float2 a, int m) {
    return make_float2(__shfl_xor_sync(0xffffffffu, a.x, m), __shfl_xor_sync(0xffffffffu, a.y, m));
}

// Sum `cnt` rows of nv partials (row stride ld) in a fixed order: thread t
// takes value t % nv over rows q, q+Q, ... (q = t / nv, Q = 256 / nv), the
// Q sub-sums are added in q order.  Rows of zeros at the end change nothing,
// so a scene's sums do not depend on its slot's capacity.
__device__ __forceinline__ void fg_sum_rows(const double* __restrict__ src, int cnt, int ld, int nv, double* out,
                                            double* scratch /*[BS_THREADS]*/) {
    const int t = threadIdx.x;
    if (nv <= BS_THREADS) {
        const int Q = BS_THREADS / nv;
        const int i = t % nv, q = t / nv;
        if (q < Q) {
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            int b = q;
            for (; b + 3 * Q < cnt; b += 4 * Q) {   // four loads in flight per thread
                a0 += __ldcg(src + (long)b * ld + i);
                a1 += __ldcg(src + (long)(b + Q) * ld + i);
                a2 += __ldcg(src + (long)(b + 2 * Q) * ld + i);
                a3 += __ldcg(src + (long)(b + 3 * Q) * ld + i);
            }
            for (; b < cnt; b += Q) a0 += __ldcg(src + (long)b * ld + i);
            scratch[q * nv + i] = (a0 + a1) + (a2 + a3);
        }
        __syncthreads();
        if (t < nv) {
            double a = 0.0;
            for (int k = 0; k < Q; ++k) a += scratch[k * nv + t];
            out[t] = a;
        }
    } else {
        for (int i = t; i < nv; i += BS_THREADS) {
            double a0 = 0.0, a1 = 0.0;
            int b = 0;
            for (; b + 1 < cnt; b += 2) {
                a0 += __ldcg(src + (long)b * ld + i);
                a1 += __ldcg(src + (long)(b + 1) * ld + i);
            }
            if (b < cnt) a0 += __ldcg(src + (long)b * ld + i);
            out[i] = a0 + a1;
        }
    }
    __syncthreads();
}

// Two-level scene sum of nv per-block values in vals[] (shared): the last
// block of each group of 32 row blocks sums the group, the last group of the
// scene sums the groups into tot[] (shared); true in that block.
__device__ __forceinline__ bool fg_scene_sum(const Dev& D, int s, int nv, const double* vals, double* tot) {
    __shared__ double scratch[BS_THREADS];
    __shared__ int last;
    const ScenePar& P = D.par[s];
    const int ld = bs::fg_part_ld(D.fg_m);
    const int lb = blockIdx.x - P.blk0, grp = lb >> 5;
    const int gsize = min(32, P.nblk - (grp << 5));
    double* part = D.fg_part + (long)blockIdx.x * ld;
    for (int i = threadIdx.x; i < nv; i += BS_THREADS) part[i] = vals[i];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(&D.fg_gdone[P.grp0 + grp], 1) == gsize - 1);
    __syncthreads();
    if (!last) return false;
    __threadfence();
    fg_sum_rows(D.fg_part + (long)(P.blk0 + (grp << 5)) * ld, gsize, ld, nv, tot, scratch);
    double* gp = D.fg_gpart + (long)(P.grp0 + grp) * ld;
    for (int i = threadIdx.x; i < nv; i += BS_THREADS) gp[i] = tot[i];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        D.fg_gdone[P.grp0 + grp] = 0;
        last = (atomicAdd(&D.blk_done[s], 1) == ((P.nblk + 31) >> 5) - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    fg_sum_rows(D.fg_gpart + (long)P.grp0 * ld, (P.nblk + 31) >> 5, ld, nv, tot, scratch);
    if (threadIdx.x == 0) D.blk_done[s] = 0;
    return true;
}

// Cycle start: r = b - A x (into ss), ||r||, g = ||r|| e1.  first: every
// scene, sets the stopping threshold (tol ||r0|| or tol ||b||).
__global__ void k_fg_start(Dev D, int first, int* nconv, const int* cycle) {
    BS_PDL_ENTRY();
    if (cycle) first = (*cycle == 0);   // the captured solve counts its cycles on the device
    const int s = D.blk_scene[blockIdx.x];
    if (!first && D.dyn[s].converged) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double q[2] = {0.0, 0.0};
    if (r < P.row0 + D.dyn[s].n) {
        const double b = D.rhs[r];
        const double rr = b - spmv_row64(D, D.p, r);
        D.ss[r] = rr;
        q[0] = rr * rr;
        q[1] = b * b;
    }
    double tot[2];
    if (scene_sum<2>(D, s, q, tot) && threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        const double beta = sqrt(tot[0]);
        if (first) {
            Y.bnorm2 = tot[1];
            Y.iters = 0;
            Y.outer = 0;
            Y.converged = 0;
            Y.breakdown = 0;
            Y.part_tmp = P.ppe_tol * (P.stop_rule == BS_STOP_RELRES ? sqrt(tot[1]) : beta);
        }
        Y.rnorm2 = tot[0];
        Y.rho_old = beta;   // norm of the vector the next column normalises
        Y.fg_rinv = beta > 0.0 ? 1.0 / beta : 0.0;
        Y.fg_j = 0;
        Y.fg_k = 0;
        fg_small(D, s).g[0] = beta;
        bool conv = tot[1] == 0.0 || beta <= Y.part_tmp;
        if (!isfinite(tot[0])) {
            conv = true;
            set_err(D, s, BS_ERR_NONFINITE);
        }
        if (conv) {
            Y.fg_state = 2;
            Y.converged = 1;
            atomicAdd(nconv, 1);
            atomicAdd(nconv + 1, 1);
        } else {
            Y.fg_state = 0;
            Y.outer += 1;   // cycles
        }
    }
}

// v_j = pending / its norm (into V), plus the V-cycle input (mgmode 1: FP64,
// 2: FP32); the scene's reciprocal norm is formed once by the producer (an
// FP64 division per row would bound this pass on this part)
__global__ void k_fg_put(Dev D, int mgmode) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (!fg_running(D, s)) return;
    const SceneDyn& Y = D.dyn[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= D.par[s].row0 + Y.n) return;
    const double v = D.ss[r] * Y.fg_rinv;
    if (D.fg_df) reinterpret_cast<float2*>(D.fg_V)[(long)Y.fg_j * D.fg_ld + r] = df_split(v);
    else D.fg_V[(long)Y.fg_j * D.fg_ld + r] = v;
    if (mgmode == 1) bs::mg_put_input<double>(D, r, v);
    else if (mgmode == 2) bs::mg_put_input<float>(D, r, v);
}

// Column finisher (one block, the scene's last): the new column h[0..j] of
// H, with h_{j+1,j} = hn below it, rotated by the cycle's earlier Givens
// rotations (staged in shared memory; the sweep, a dependent chain, run by
// one thread), a new rotation that zeroes hn, the residual estimate
// |g_{j+1}| and the cycle's state.  est: hn was formed from the Gram
// relation rather than summed, and was not trusted (cancellation), so the
// cycle restarts from the true residual instead of going on.
__device__ void fg_finish_column(const Dev& D, int s, const FgSmall& f, int j, double hn, bool est_bad, int* nconv) {
    __shared__ double hcol[BS_FG_MAXM + 2], csh[BS_FG_MAXM], snh[BS_FG_MAXM];
    const ScenePar& P = D.par[s];
    const int m = D.fg_m;
    double* h = f.H + (long)j * (m + 1);
    for (int i = threadIdx.x; i <= j; i += BS_THREADS) hcol[i] = h[i];
    for (int i = threadIdx.x; i < j; i += BS_THREADS) {
        csh[i] = f.cs[i];
        snh[i] = f.sn[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        SceneDyn& Y = D.dyn[s];
        double hi = hcol[0];
        for (int i = 0; i < j; ++i) {   // earlier rotations on the new column
            const double b = hcol[i + 1];
            hcol[i] = csh[i] * hi + snh[i] * b;
            hi = -snh[i] * hi + csh[i] * b;
        }
        const double a = hi;
        const double den = sqrt(a * a + hn * hn);
        const double c = den > 0.0 ? a / den : 1.0, sn = den > 0.0 ? hn / den : 0.0;
        f.cs[j] = c;
        f.sn[j] = sn;
        hcol[j] = den;
        hcol[j + 1] = 0.0;
        const double gj = f.g[j];
        f.g[j] = c * gj;
        f.g[j + 1] = -sn * gj;
        const double res = fabs(f.g[j + 1]);
        Y.rnorm2 = res * res;
        Y.rho_old = hn;
        Y.fg_rinv = hn > 0.0 ? 1.0 / hn : 0.0;
        Y.iters += 1;
        Y.fg_j = j + 1;
        int st = 0;
        if (!isfinite(res) || !isfinite(hn)) {
            st = 3;
            set_err(D, s, BS_ERR_NONFINITE);
        } else if (est_bad) {
            st = Y.iters >= P.maxit ? 3 : 1;
        } else if (res <= Y.part_tmp || hn <= 1e-12) {
            st = 2;
        } else if (Y.iters >= P.maxit) {
            st = 3;
        } else if (j + 1 == m) {
            st = 1;
        }
        Y.fg_state = st;
        if (st) atomicAdd(nconv, 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= j + 1; i += BS_THREADS) h[i] = hcol[i];
}

// s += (a.x + a.y) z for an FP32 z: TwoProduct of the high part, the low
// part's product into the error, TwoSum into the running sum
__device__ __forceinline__ void df_fma1(float2& s, float2 a, float z) {
    const float ph = __fmul_rn(a.x, z);
    float pe = __fmaf_rn(a.x, z, -ph);
    pe = __fmaf_rn(a.y, z, pe);
    const float t = __fadd_rn(s.x, ph);
    const float v = __fsub_rn(t, s.x);
    const float e = __fadd_rn(__fsub_rn(s.x, __fsub_rn(t, v)), __fsub_rn(ph, v));
    s.y = __fadd_rn(s.y, __fadd_rn(e, pe));
    s.x = t;
}

// Row r of A z for an FP32-exact z (the mixed V-cycle output, zf): the
// off-diagonal values as double-float pairs (aval32 + aval_lo, 48 bits) and
// the products and sums on the FP32 pipe; the diagonal term in FP64.
__device__ __forceinline__ double spmv_row_df(const Dev& D, const float* __restrict__ z, int r) {
    const float* __restrict__ Ah = D.aval32;
    const float* __restrict__ Al = D.aval_lo;
    const int* __restrict__ idx = D.nidx;
    const int n = D.ncount[r];
    float2 acc = make_float2(0.f, 0.f);
    long e = ell(r, 0, D.kmax);
    int k = 0;
    for (; k + 4 <= n; k += 4, e += 128) {   // four independent gathers in flight
        const int j0 = __ldg(idx + e), j1 = __ldg(idx + e + 32), j2 = __ldg(idx + e + 64), j3 = __ldg(idx + e + 96);
        const float2 a0 = make_float2(__ldg(Ah + e), __ldg(Al + e));
        const float2 a1 = make_float2(__ldg(Ah + e + 32), __ldg(Al + e + 32));
        const float2 a2 = make_float2(__ldg(Ah + e + 64), __ldg(Al + e + 64));
        const float2 a3 = make_float2(__ldg(Ah + e + 96), __ldg(Al + e + 96));
        const float z0 = z[j0], z1 = z[j1], z2 = z[j2], z3 = z[j3];
        df_fma1(acc, a0, z0);
        df_fma1(acc, a1, z1);
        df_fma1(acc, a2, z2);
        df_fma1(acc, a3, z3);
    }
    for (; k < n; ++k, e += 32) df_fma1(acc, make_float2(__ldg(Ah + e), __ldg(Al + e)), z[__ldg(idx + e)]);
    return __dadd_rn(__dmul_rn(D.adiag[r], (double)z[r]), df_to_double(acc));
}

// Pass 1's dots with a double-float basis: the block's w and v_j split into
// (hi, lo) pairs in shared memory, each lane keeps its 8 rows of both in
// registers; warp `warp` takes basis vectors warp + 8 (4g + u) as in the FP64
// form, the 8 double-float values of a lane summed across the warp by the
// same transposing butterfly in double-float, each block's value converted to
// FP64 once (into dsh) for the FP64 scene sums.
__device__ __forceinline__ void fg_arn1_dots_df(const Dev& D, float2 wd, float2 vjd, int nv, long r0, int rend,
                                                double* dsh) {
    __shared__ float2 wsd[BS_THREADS], vsd[BS_THREADS];
    wsd[threadIdx.x] = wd;
    vsd[threadIdx.x] = vjd;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    constexpr int RPL = BS_THREADS / 32;   // rows per lane
    const float2* Vb = reinterpret_cast<const float2*>(D.fg_V);
    for (int base = warp; base < nv; base += 4 * (BS_THREADS / 32)) {
        // per vector: the lane's 8 rows loaded first, then two accumulation
        // chains; w and v_j read from shared memory (few registers: the grid
        // fits the SMs in one wave)
        float2 x[8];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = base + (BS_THREADS / 32) * u;
            float2 a = make_float2(0.f, 0.f), c = make_float2(0.f, 0.f);
            if (i < nv) {
                const float2* v = Vb + (long)i * D.fg_ld + r0;
                float2 vv[RPL];
#pragma unroll
                for (int k = 0; k < RPL; ++k) {
                    const int t = lane + 32 * k;
                    vv[k] = (r0 + t < rend) ? v[t] : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int k = 0; k < RPL; ++k) {
                    const int t = lane + 32 * k;
                    df_fma(a, vv[k], wsd[t]);
                    df_fma(c, vv[k], vsd[t]);
                }
            }
            x[2 * u] = a;
            x[2 * u + 1] = c;
        }
        float2 y[4], z[2];
#pragma unroll
        for (int k = 0; k < 4; ++k) y[k] = df_add(b4 ? x[k + 4] : x[k], df_shfl_xor(b4 ? x[k] : x[k + 4], 16));
#pragma unroll
        for (int k = 0; k < 2; ++k) z[k] = df_add(b3 ? y[k + 2] : y[k], df_shfl_xor(b3 ? y[k] : y[k + 2], 8));
        float2 tv = df_add(b2 ? z[1] : z[0], df_shfl_xor(b2 ? z[0] : z[1], 4));
        tv = df_add(tv, df_shfl_xor(tv, 2));
        tv = df_add(tv, df_shfl_xor(tv, 1));
        if ((lane & 3) == 0) {
            const int q = lane >> 2;
            const int i = base + (BS_THREADS / 32) * (q >> 1);
            if (i < nv) dsh[(q & 1) ? nv + i : i] = df_to_double(tv);
        }
    }
}

// Column j, pass 1: w = A z_j (z_j = the V-cycle output in sp2, kept as Z_j;
// or v_j) into sv; one read of v_0..v_j gives h = V^T w and the Gram column
// c = V^T v_j.  Finisher: Gm(:,j) = c, then the column's coefficients
// hc = (2I - Gm) h -- classical Gram-Schmidt applied twice,
// (I - V V^T)^2 = I - V (2I - V^T V) V^T, with the second projection
// taken from the Gram matrix instead of a second pass over V.
template <int DF>
__global__ void __launch_bounds__(BS_THREADS, 5) k_fg_arn1(Dev D, int precond, int* nconv) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (!fg_running(D, s)) return;
    __shared__ double ws[BS_THREADS], vs[BS_THREADS];
    __shared__ double dsh[2 * (BS_FG_MAXM + 1)];
    __shared__ double tsh[2 * (BS_FG_MAXM + 1)];
    const int j = D.dyn[s].fg_j, nv = j + 1;
    const int rend = D.par[s].row0 + D.dyn[s].n;
    const long r0 = (long)blockIdx.x * BS_THREADS;
    const int r = (int)r0 + threadIdx.x;
    const long col = (long)j * D.fg_ld;
    const double* u = precond ? D.sp2 : D.fg_V + col;
    double w = 0.0, vj = 0.0;
    float2 vjd = make_float2(0.f, 0.f);
    if (r < rend) {
        w = DF ? spmv_row_df(D, D.zf, r) : spmv_row64(D, u, r);
        D.sv[r] = w;
        if (DF) vjd = reinterpret_cast<const float2*>(D.fg_V)[col + r];
        else vj = D.fg_V[col + r];
        if (precond) D.fg_Z[col + r] = D.sp2[r];
    }
    if (DF) {
        // u.u for the Gram relation of ||w|| (block partial at dsh[2 nv])
        __shared__ double wwp[BS_THREADS / 32];
        const double ww = warp_sum(w * w);
        if ((threadIdx.x & 31) == 0) wwp[threadIdx.x >> 5] = ww;
        fg_arn1_dots_df(D, df_split(w), vjd, nv, r0, rend, dsh);
        if (threadIdx.x == 0) {
            double a = 0.0;
            for (int k = 0; k < BS_THREADS / 32; ++k) a += wwp[k];
            dsh[2 * nv] = a;
        }
    } else {
        ws[threadIdx.x] = w;
        vs[threadIdx.x] = vj;
        __syncthreads();
    // Warp w takes basis vectors w + 8 (4g + u), u = 0..3: lanes across the
    // block's rows (coalesced), 8 values per lane (4 vectors x 2 dots), summed
    // over the lanes by a transposing butterfly -- 9 FP64 adds per lane for
    // the 8 values rather than 5 per value (the FP64 pipe bounds this pass)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    for (int base = warp; base < nv; base += 4 * (BS_THREADS / 32)) {
        double x[8];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = base + (BS_THREADS / 32) * u;
            double a = 0.0, c = 0.0;
            if (i < nv) {
                const double* v = D.fg_V + (long)i * D.fg_ld + r0;
#pragma unroll
                for (int k = 0; k < BS_THREADS / 32; ++k) {
                    const int t = lane + 32 * k;
                    const double vi = (r0 + t < rend) ? v[t] : 0.0;
                    a += vi * ws[t];
                    c += vi * vs[t];
                }
            }
            x[2 * u] = a;
            x[2 * u + 1] = c;
        }
        double y[4], z[2];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            y[k] = (b4 ? x[k + 4] : x[k]) + __shfl_xor_sync(0xffffffffu, b4 ? x[k] : x[k + 4], 16);
#pragma unroll
        for (int k = 0; k < 2; ++k)
            z[k] = (b3 ? y[k + 2] : y[k]) + __shfl_xor_sync(0xffffffffu, b3 ? y[k] : y[k + 2], 8);
        double tv = (b2 ? z[1] : z[0]) + __shfl_xor_sync(0xffffffffu, b2 ? z[0] : z[1], 4);
        tv += __shfl_xor_sync(0xffffffffu, tv, 2);
        tv += __shfl_xor_sync(0xffffffffu, tv, 1);
        if ((lane & 3) == 0) {   // lane holds value q = lane / 4 = 2u + dot
            const int q = lane >> 2;
            const int i = base + (BS_THREADS / 32) * (q >> 1);
            if (i < nv) dsh[(q & 1) ? nv + i : i] = tv;
        }
    }
    }
    __syncthreads();
    if (!fg_scene_sum(D, s, DF ? 2 * nv + 1 : 2 * nv, dsh, tsh)) return;
    const FgSmall f = fg_small(D, s);
    const int ldg = D.fg_m + 1;
    for (int i = threadIdx.x; i < nv; i += BS_THREADS) {
        f.Gm[i + (long)j * ldg] = tsh[nv + i];
        f.Gm[j + (long)i * ldg] = tsh[nv + i];
    }
    __syncthreads();
    // hc = (2I - Gm) h, a warp per row: Gm is symmetric, so row i is read as
    // the contiguous column i (coalesced, a few loads per lane)
    __shared__ double hcs[BS_FG_MAXM + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = wid; i < nv; i += BS_THREADS / 32) {
        const double* gcol = f.Gm + (long)i * ldg;
        double a = 0.0;
        for (int k = lane; k < nv; k += 32) a += __ldcg(gcol + k) * tsh[k];
        a = warp_sum(a);
        if (lane == 0) {
            const double acc = 2.0 * tsh[i] - a;
            f.hc[i] = acc;
            f.H[i + (long)j * ldg] = acc;
            hcs[i] = acc;
        }
    }
    if (!DF) return;
    // h_{j+1,j} = ||w|| for w = u - V c without a pass over w: ||w||^2 =
    // u.u - 2 c.h + c^T Gm c (u = A z_j, h = V^T u, Gm = V^T V, c = hc), so
    // pass 2 can write v_{j+1} and the V-cycle input directly.  When that
    // difference falls below 1e-6 u.u the estimate is not trusted and the
    // cycle restarts from the true residual.
    __shared__ double eparts[BS_THREADS / 32];
    __shared__ double eta2s;
    __syncthreads();
    double part = 0.0;
    for (int i = wid; i < nv; i += BS_THREADS / 32) {
        const double* gcol = f.Gm + (long)i * ldg;
        double g = 0.0;
        for (int k = lane; k < nv; k += 32) g += __ldcg(gcol + k) * hcs[k];
        g = warp_sum(g);
        part += hcs[i] * (g - 2.0 * tsh[i]);
    }
    if (lane == 0) eparts[wid] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double e = tsh[2 * nv];
        for (int w = 0; w < BS_THREADS / 32; ++w) e += eparts[w];
        eta2s = e;
    }
    __syncthreads();
    const double uu = tsh[2 * nv], eta2 = eta2s;
    fg_finish_column(D, s, f, j, sqrt(fmax(eta2, 0.0)), !(eta2 > 1e-6 * uu), nconv);
}

// Column j, pass 2: w -= V hc (the pending vector, into ss), h_{j+1,j} = ||w||;
// finisher: rotations, residual estimate, cycle end
// With the double-float basis (DF): column j = fg_j - 1 was finished by pass
// 1, and this pass writes v_{j+1} = (w - V hc) / h_{j+1,j} into the basis
// and the V-cycle input (mgmode as k_fg_put), with no reduction.
template <int DF>
__global__ void k_fg_arn2(Dev D, int* nconv, int mgmode) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    if (!fg_running(D, s)) return;
    __shared__ double hs[BS_FG_MAXM + 1];
    __shared__ float2 hsd[BS_FG_MAXM + 1];
    const ScenePar& P = D.par[s];
    const int j = DF ? D.dyn[s].fg_j - 1 : D.dyn[s].fg_j;
    const int rend = P.row0 + D.dyn[s].n;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const FgSmall f = fg_small(D, s);
    for (int i = threadIdx.x; i <= j; i += BS_THREADS) {
        hs[i] = f.hc[i];
        if (DF) hsd[i] = df_split(hs[i]);
    }
    __syncthreads();
    double q[1] = {0.0};
    if (DF) {   // w -= (V hc) summed in double-float, then v_{j+1}
        if (r >= rend) return;
        double w = D.sv[r];
        const float2* v = reinterpret_cast<const float2*>(D.fg_V) + r;
        const long ld = D.fg_ld;
        float2 a0 = make_float2(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
        int i = 0;
        for (; i + 4 <= j + 1; i += 4) {   // four loads in flight, four chains
            const float2 v0 = v[i * ld], v1 = v[(i + 1) * ld], v2 = v[(i + 2) * ld], v3 = v[(i + 3) * ld];
            df_fma(a0, hsd[i], v0);
            df_fma(a1, hsd[i + 1], v1);
            df_fma(a2, hsd[i + 2], v2);
            df_fma(a3, hsd[i + 3], v3);
        }
        for (; i <= j; ++i) df_fma(a0, hsd[i], v[i * ld]);
        w = __dsub_rn(w, df_to_double(df_add(df_add(a0, a1), df_add(a2, a3))));
        const double vn = w * D.dyn[s].fg_rinv;
        reinterpret_cast<float2*>(D.fg_V)[(long)(j + 1) * ld + r] = df_split(vn);
        if (mgmode == 1) bs::mg_put_input<double>(D, r, vn);
        else if (mgmode == 2) bs::mg_put_input<float>(D, r, vn);
        return;
    } else if (r < rend) {
        double w = D.sv[r];
        const double* v = D.fg_V + r;
        int i = 0;
        for (; i + 4 <= j + 1; i += 4) {   // four loads in flight
            const double v0 = v[(long)i * D.fg_ld], v1 = v[(long)(i + 1) * D.fg_ld];
            const double v2 = v[(long)(i + 2) * D.fg_ld], v3 = v[(long)(i + 3) * D.fg_ld];
            w -= hs[i] * v0;
            w -= hs[i + 1] * v1;
            w -= hs[i + 2] * v2;
            w -= hs[i + 3] * v3;
        }
        for (; i <= j; ++i) w -= hs[i] * v[(long)i * D.fg_ld];
        D.ss[r] = w;
        q[0] = w * w;
    }
    double tot[1];
    if (!scene_sum<1>(D, s, q, tot)) return;
    fg_finish_column(D, s, f, j, sqrt(tot[0]), false, nconv);
}

// One warp per scene: y = R^-1 g over the cycle's k columns; scenes that
// converged (or met the cap) in this cycle are marked done
__global__ void k_fg_solve(Dev D, int* nconv) {
    BS_PDL_ENTRY();
    const int s = blockIdx.x, lane = threadIdx.x;
    SceneDyn& Y = D.dyn[s];
    if (Y.converged) {
        if (lane == 0) Y.fg_k = 0;
        return;
    }
    __shared__ double ys[BS_FG_MAXM];
    const int k = Y.fg_j;
    const int ld = D.fg_m + 1;
    const FgSmall f = fg_small(D, s);
    for (int i = k - 1; i >= 0; --i) {
        double acc = 0.0;
        for (int l = i + 1 + lane; l < k; l += 32) acc += f.H[i + (long)l * ld] * ys[l];
        acc = warp_sum(acc);
        if (lane == 0) {
            const double d = f.H[i + (long)i * ld];
            ys[i] = d != 0.0 ? (f.g[i] - acc) / d : 0.0;
        }
        __syncwarp();
    }
    for (int i = lane; i < k; i += 32) f.y[i] = ys[i];
    if (lane == 0) {
        Y.fg_k = k;
        if (Y.fg_state >= 2) {
            if (Y.fg_state == 3) set_err(D, s, BS_ERR_NOT_CONVERGED);
            Y.converged = 1;
            atomicAdd(nconv + 1, 1);
        }
    }
}

// x += Z y over the cycle's columns
__global__ void k_fg_update(Dev D, int precond) {
    BS_PDL_ENTRY();
    const int s = D.blk_scene[blockIdx.x];
    const int k = D.dyn[s].fg_k;
    if (k == 0) return;
    __shared__ double ys[BS_FG_MAXM];
    const FgSmall f = fg_small(D, s);
    for (int i = threadIdx.x; i < k; i += BS_THREADS) ys[i] = f.y[i];
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= D.par[s].row0 + D.dyn[s].n) return;
    const double* z = (precond ? D.fg_Z : D.fg_V) + r;
    double dx = 0.0;
    for (int i = 0; i < k; ++i) dx += ys[i] * z[(long)i * D.fg_ld];
    D.p[r] += dx;
}

}  // namespace

namespace bs {

// Host driver of the FP64 solve.  Checks the converged-scene counter every
// `check_every` iterations with one event sync, one chunk behind the launches
// so the GPU never idles on the host.
void solve_fp64(const Dev& D, const Launch& L, int maxit, int check_every, int precond, int mg_prec, int* d_nconv,
                int* h_nconv, cudaEvent_t ev) {
    int q;
    if (precond) {
        if (mg_prec == BS_PREC_MIXED) {
            q = tbegin(L, K_MX_CONV);
            launch_pdl(L, k_mx_convert, L.nblk_rows, BS_THREADS, 0, D);
            tend(L, q);
        }
        mg_setup(D, L, mg_prec);
    }
    const double* pu = precond ? D.sp2 : D.sp;   // M^-1 p
    const double* su = precond ? D.sv2 : D.ss;   // M^-1 s
    cudaMemsetAsync(d_nconv, 0, sizeof(int), L.stream);
    q = tbegin(L, K_BICG_INIT);
    launch_pdl(L, k_init64, L.nblk_rows, BS_THREADS, 0, D, d_nconv);
    tend(L, q);
    const int mgmode = precond ? (mg_prec == BS_PREC_MIXED ? 2 : 1) : 0;
    auto iteration = [&]() {
        int q2 = tbegin(L, K_BICG_PUPD);
        launch_pdl(L, k_pupd64, L.nblk_rows, BS_THREADS, 0, D, mgmode);
        tend(L, q2);
        if (precond) mg_apply(D, L, mg_prec, D.sp, D.sp2);
        q2 = tbegin(L, K_BICG_IT1);
        launch_pdl(L, k_it1_64, L.nblk_rows, BS_THREADS, 0, D, pu);
        tend(L, q2);
        q2 = tbegin(L, K_BICG_SUPD);
        launch_pdl(L, k_supd64, L.nblk_rows, BS_THREADS, 0, D, mgmode);
        tend(L, q2);
        if (precond) mg_apply(D, L, mg_prec, D.ss, D.sv2);
        q2 = tbegin(L, K_BICG_IT2);
        launch_pdl(L, k_it2_64, L.nblk_rows, BS_THREADS, 0, D, su);
        tend(L, q2);
        q2 = tbegin(L, K_BICG_IT3);
        launch_pdl(L, k_it3_64, L.nblk_rows, BS_THREADS, 0, D, pu, su, d_nconv);
        tend(L, q2);
    };
    // capture one convergence-check chunk (check_every iterations; an
    // iteration of a converged scene returns at once) as a CUDA graph, not
    // while per-kernel events are on
    IterGraph* G = L.graph;
    bool use_graph = G && !(L.timer && L.timer->mask);
    if (use_graph && !(G->valid && G->solver == BS_SOLVER_BICGSTAB && G->precond == precond && G->prec == mg_prec &&
                       G->chunk == check_every && std::memcmp(&G->key, &D, sizeof(Dev)) == 0)) {
        if (G->exec) cudaGraphExecDestroy(G->exec);
        G->exec = nullptr;
        G->valid = false;
        const int64_t before = *L.launches;
        cudaGraph_t gr = nullptr;
        if (cudaStreamBeginCapture(L.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            for (int c = 0; c < check_every; ++c) iteration();
            if (cudaStreamEndCapture(L.stream, &gr) == cudaSuccess && gr &&
                cudaGraphInstantiate(&G->exec, gr, 0) == cudaSuccess) {
                G->valid = true;
                G->key = D;
                G->solver = BS_SOLVER_BICGSTAB;
                G->precond = precond;
                G->prec = mg_prec;
                G->chunk = check_every;
                G->nkernels = *L.launches - before;
            }
            if (gr) cudaGraphDestroy(gr);
        }
        *L.launches = before;
        cudaGetLastError();
        use_graph = G->valid;
    }
    int it = 0;
    while (it < maxit) {
        cudaMemcpyAsync(h_nconv, d_nconv, sizeof(int), cudaMemcpyDeviceToHost, L.stream);
        cudaEventRecord(ev, L.stream);
        if (use_graph) {
            cudaGraphLaunch(G->exec, L.stream);
            *L.launches += G->nkernels;
            it += check_every;
        } else {
            for (int c = 0; c < check_every && it < maxit; ++c, ++it) iteration();
        }
        cudaEventSynchronize(ev);
        timer_collect(L.timer, false);
        if (*h_nconv >= D.nscene) break;
    }
    q = tbegin(L, K_TRUERES);
    launch_pdl(L, k_true_res64, L.nblk_rows, BS_THREADS, 0, D);
    tend(L, q);
}

// Host driver of FGMRES: per restart cycle one start kernel and a host read
// of the converged count, then chunks of `check_every` columns (captured as
// one CUDA graph) until every scene's cycle has ended, then the small
// triangular solves and the update.  d_nconv[0] counts scenes whose cycle
// ended, d_nconv[1] converged scenes.
void solve_fgmres(const Dev& D, const Launch& L, int maxit, int check_every, int precond, int mg_prec,
                  int* d_nconv, int* h_nconv, cudaEvent_t ev) {
    int q;
    if (precond) {
        if (mg_prec == BS_PREC_MIXED) {
            q = tbegin(L, K_MX_CONV);
            launch_pdl(L, k_mx_convert, L.nblk_rows, BS_THREADS, 0, D);
            tend(L, q);
        }
        mg_setup(D, L, mg_prec);
    }
    const int mgmode = precond ? (mg_prec == BS_PREC_MIXED ? 2 : 1) : 0;
    // a column: [v_j and the V-cycle input], the V-cycle, pass 1, pass 2.  With
    // the double-float basis pass 2 writes v_{j+1} and the next input, so only
    // a cycle's first vector needs k_fg_put (after k_fg_start).
    auto put = [&]() {
        int q2 = tbegin(L, K_FG_PUT);
        launch_pdl(L, k_fg_put, L.nblk_rows, BS_THREADS, 0, D, mgmode);
        tend(L, q2);
    };
    auto column = [&]() {
        if (!D.fg_df) put();
        if (precond) mg_apply(D, L, mg_prec, D.fg_V, D.sp2);
        int q2 = tbegin(L, K_FG_ARN);
        if (D.fg_df) launch_pdl(L, k_fg_arn1<1>, L.nblk_rows, BS_THREADS, 0, D, precond, d_nconv);
        else launch_pdl(L, k_fg_arn1<0>, L.nblk_rows, BS_THREADS, 0, D, precond, d_nconv);
        tend(L, q2);
        q2 = tbegin(L, K_FG_ORTH);
        if (D.fg_df) launch_pdl(L, k_fg_arn2<1>, L.nblk_rows, BS_THREADS, 0, D, d_nconv, mgmode);
        else launch_pdl(L, k_fg_arn2<0>, L.nblk_rows, BS_THREADS, 0, D, d_nconv, mgmode);
        tend(L, q2);
    };
    IterGraph* G = L.graph;
    bool use_graph = G && !(L.timer && L.timer->mask);
    if (use_graph && !(G->valid && G->solver == BS_SOLVER_FGMRES && G->precond == precond && G->prec == mg_prec &&
                       G->chunk == check_every && std::memcmp(&G->key, &D, sizeof(Dev)) == 0)) {
        if (G->exec) cudaGraphExecDestroy(G->exec);
        G->exec = nullptr;
        G->valid = false;
        const int64_t before = *L.launches;
        cudaGraph_t gr = nullptr;
        if (cudaStreamBeginCapture(L.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            for (int c = 0; c < check_every; ++c) column();
            if (cudaStreamEndCapture(L.stream, &gr) == cudaSuccess && gr &&
                cudaGraphInstantiate(&G->exec, gr, 0) == cudaSuccess) {
                G->valid = true;
                G->key = D;
                G->solver = BS_SOLVER_FGMRES;
                G->precond = precond;
                G->prec = mg_prec;
                G->chunk = check_every;
                G->nkernels = *L.launches - before;
            }
            if (gr) cudaGraphDestroy(gr);
        }
        *L.launches = before;
        cudaGetLastError();
        use_graph = G->valid;
    }
    cudaMemsetAsync(d_nconv, 0, 2 * sizeof(int), L.stream);
    // every cycle does at least one column of each scene it starts, and the
    // column kernels stop a scene at maxit columns
    for (int cycle = 0; cycle <= maxit; ++cycle) {
        cudaMemcpyAsync(d_nconv, d_nconv + 1, sizeof(int), cudaMemcpyDeviceToDevice, L.stream);
        q = tbegin(L, K_FG_START);
        launch_pdl(L, k_fg_start, L.nblk_rows, BS_THREADS, 0, D, cycle == 0 ? 1 : 0, d_nconv, (const int*)nullptr);
        tend(L, q);
        cudaMemcpyAsync(h_nconv, d_nconv, 2 * sizeof(int), cudaMemcpyDeviceToHost, L.stream);
        cudaStreamSynchronize(L.stream);
        timer_collect(L.timer, false);
        if (h_nconv[1] >= D.nscene) break;
        if (D.fg_df) put();
        int it = 0;
        while (it < D.fg_m) {
            cudaMemcpyAsync(h_nconv, d_nconv, sizeof(int), cudaMemcpyDeviceToHost, L.stream);
            cudaEventRecord(ev, L.stream);
            if (use_graph) {
                cudaGraphLaunch(G->exec, L.stream);
                *L.launches += G->nkernels;
                it += check_every;
            } else {
                for (int c = 0; c < check_every && it < D.fg_m; ++c, ++it) column();
            }
            cudaEventSynchronize(ev);
            timer_collect(L.timer, false);
            if (*h_nconv >= D.nscene) break;
        }
        q = tbegin(L, K_FG_UPD);
        launch_pdl(L, k_fg_solve, D.nscene, 32, 0, D, d_nconv);
        launch_pdl(L, k_fg_update, L.nblk_rows, BS_THREADS, 0, D, precond);
        tend(L, q);
    }
    q = tbegin(L, K_TRUERES);
    launch_pdl(L, k_true_res64, L.nblk_rows, BS_THREADS, 0, D);
    tend(L, q);
}

// Mixed solve: outer FP64 refinement around an FP32 BiCGStab.
void solve_mixed(const Dev& D, const Launch& L, int maxit, int check_every, int* d_nconv, int* h_nconv,
                 cudaEvent_t ev) {
    // FP32-inner iterative refinement (kept for systems whose condition number
    // times the FP32 unit round-off is well below one)
    int q = tbegin(L, K_MX_CONV);
    launch_pdl(L, k_mx_convert, L.nblk_rows, BS_THREADS, 0, D);
    tend(L, q);
    cudaMemsetAsync(d_nconv, 0, 2 * sizeof(int), L.stream);
    int max_outer = 0;
    cudaMemcpyAsync(h_nconv + 2, &D.par[0].max_outer, sizeof(int), cudaMemcpyDeviceToHost, L.stream);
    cudaStreamSynchronize(L.stream);
    max_outer = h_nconv[2];
    for (int outer = 0; outer <= max_outer; ++outer) {
        float *p = D.fp, *v = D.fv, *p2 = D.fp2, *v2 = D.fv2;   // k_mx_init zeroes fp, fv
        q = tbegin(L, K_MX_RES);
        launch_pdl(L, k_mx_res, L.nblk_rows, BS_THREADS, 0, D, d_nconv);
        tend(L, q);
        cudaMemcpyAsync(h_nconv, d_nconv, 2 * sizeof(int), cudaMemcpyDeviceToHost, L.stream);
        cudaStreamSynchronize(L.stream);
        if (h_nconv[1] >= D.nscene) break;
        cudaMemsetAsync(d_nconv, 0, sizeof(int), L.stream);
        // inner-converged counter starts with the outer-converged scenes
        cudaMemcpyAsync(d_nconv, d_nconv + 1, sizeof(int), cudaMemcpyDeviceToDevice, L.stream);
        q = tbegin(L, K_MX_INIT);
        launch_pdl(L, k_mx_init, L.nblk_rows, BS_THREADS, 0, D, d_nconv);
        tend(L, q);
        int it = 0;
        while (it < maxit) {
            cudaMemcpyAsync(h_nconv, d_nconv, sizeof(int), cudaMemcpyDeviceToHost, L.stream);
            cudaEventRecord(ev, L.stream);
            for (int c = 0; c < check_every && it < maxit; ++c, ++it) {
                q = tbegin(L, K_MX_IT1);
                launch_pdl(L, k_mx_it1, L.nblk_rows, BS_THREADS, 0, D, p, v, p2, v2);
                tend(L, q);
                q = tbegin(L, K_MX_IT2);
                launch_pdl(L, k_mx_it2, L.nblk_rows, BS_THREADS, 0, D, v2);
                tend(L, q);
                q = tbegin(L, K_MX_IT3);
                launch_pdl(L, k_mx_it3, L.nblk_rows, BS_THREADS, 0, D, p2, d_nconv);
                tend(L, q);
                float* t;
                t = p; p = p2; p2 = t;
                t = v; v = v2; v2 = t;
            }
            cudaEventSynchronize(ev);
            timer_collect(L.timer, false);
            if (*h_nconv >= D.nscene) break;
        }
        q = tbegin(L, K_MX_UPD);
        launch_pdl(L, k_mx_update, L.nblk_rows, BS_THREADS, 0, D);
        tend(L, q);
    }
}


// ---------------------------------------------------------------- captured solves
// The solves above check convergence on the host between chunks of
// iterations.  Inside a captured step the loops run on the device instead:
// a conditional while node repeats a chunk of iterations (or columns, or
// restart cycles) for as long as its condition kernel -- one thread, after
// the chunk -- finds a scene that has not converged and the iteration budget
// not spent.  Every loop is bounded by the same maxit / restart length as the
// host loops, so it ends even if no scene converges.

bool cond_handle(cudaStream_t st, unsigned init, cudaGraphConditionalHandle* h) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive || !g)
        return false;
    return cudaGraphConditionalHandleCreate(h, g, init, cudaGraphCondAssignDefault) == cudaSuccess;
}

// BiCGStab chunk done: go on while a scene is not converged and it < maxit
__global__ void k_cond_iter(Dev D, const int* nconv, cudaGraphConditionalHandle h, int chunk, int maxit,
                            int body_kernels) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    LoopCtl* C = D.loop;
    C->kernels += (unsigned long long)body_kernels;
    C->it += chunk;
    cudaGraphSetConditional(h, (*nconv < D.nscene && C->it < maxit) ? 1u : 0u);
}

// FGMRES cycle started (k_fg_start ran): the cycle's columns run if a scene
// is not converged; another cycle follows while cycle <= maxit
__global__ void k_cond_cycle(Dev D, const int* nconv, cudaGraphConditionalHandle hloop,
                             cudaGraphConditionalHandle hbody, int maxit, int body_kernels) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    LoopCtl* C = D.loop;
    C->kernels += (unsigned long long)body_kernels;
    const bool go = nconv[1] < D.nscene;
    C->cycle += 1;
    cudaGraphSetConditional(hbody, go ? 1u : 0u);
    cudaGraphSetConditional(hloop, (go && C->cycle <= maxit) ? 1u : 0u);
}

// start of a cycle's columns: column counter 0, the column loop armed
__global__ void k_col_init(Dev D, cudaGraphConditionalHandle h, int body_kernels) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    LoopCtl* C = D.loop;
    C->kernels += (unsigned long long)body_kernels;
    C->col = 0;
    cudaGraphSetConditional(h, 1u);
}

// a chunk of columns done: go on while col < restart length and a scene's cycle is open
__global__ void k_cond_col(Dev D, const int* nconv, cudaGraphConditionalHandle h, int chunk, int body_kernels) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    LoopCtl* C = D.loop;
    C->kernels += (unsigned long long)body_kernels;
    C->col += chunk;
    cudaGraphSetConditional(h, (C->col < D.fg_m && nconv[0] < D.nscene) ? 1u : 0u);
}

namespace {

void bicg_iteration(const Dev& D, const Launch& L, int precond, int mg_prec, int* d_nconv) {
    const double* pu = precond ? D.sp2 : D.sp;
    const double* su = precond ? D.sv2 : D.ss;
    const int mgmode = precond ? (mg_prec == BS_PREC_MIXED ? 2 : 1) : 0;
    int q = tbegin(L, K_BICG_PUPD);
    launch_pdl(L, k_pupd64, L.nblk_rows, BS_THREADS, 0, D, mgmode);
    tend(L, q);
    if (precond) mg_apply(D, L, mg_prec, D.sp, D.sp2);
    q = tbegin(L, K_BICG_IT1);
    launch_pdl(L, k_it1_64, L.nblk_rows, BS_THREADS, 0, D, pu);
    tend(L, q);
    q = tbegin(L, K_BICG_SUPD);
    launch_pdl(L, k_supd64, L.nblk_rows, BS_THREADS, 0, D, mgmode);
    tend(L, q);
    if (precond) mg_apply(D, L, mg_prec, D.ss, D.sv2);
    q = tbegin(L, K_BICG_IT2);
    launch_pdl(L, k_it2_64, L.nblk_rows, BS_THREADS, 0, D, su);
    tend(L, q);
    q = tbegin(L, K_BICG_IT3);
    launch_pdl(L, k_it3_64, L.nblk_rows, BS_THREADS, 0, D, pu, su, d_nconv);
    tend(L, q);
}

void fg_put(const Dev& D, const Launch& L, int mgmode) {
    int q = tbegin(L, K_FG_PUT);
    launch_pdl(L, k_fg_put, L.nblk_rows, BS_THREADS, 0, D, mgmode);
    tend(L, q);
}

void fg_column(const Dev& D, const Launch& L, int precond, int mg_prec, int mgmode, int* d_nconv) {
    if (!D.fg_df) fg_put(D, L, mgmode);
    if (precond) mg_apply(D, L, mg_prec, D.fg_V, D.sp2);
    int q = tbegin(L, K_FG_ARN);
    if (D.fg_df) launch_pdl(L, k_fg_arn1<1>, L.nblk_rows, BS_THREADS, 0, D, precond, d_nconv);
    else launch_pdl(L, k_fg_arn1<0>, L.nblk_rows, BS_THREADS, 0, D, precond, d_nconv);
    tend(L, q);
    q = tbegin(L, K_FG_ORTH);
    if (D.fg_df) launch_pdl(L, k_fg_arn2<1>, L.nblk_rows, BS_THREADS, 0, D, d_nconv, mgmode);
    else launch_pdl(L, k_fg_arn2<0>, L.nblk_rows, BS_THREADS, 0, D, d_nconv, mgmode);
    tend(L, q);
}

void precond_setup(const Dev& D, const Launch& L, int precond, int mg_prec) {
    if (!precond) return;
    if (mg_prec == BS_PREC_MIXED) {
        const int q = tbegin(L, K_MX_CONV);
        launch_pdl(L, k_mx_convert, L.nblk_rows, BS_THREADS, 0, D);
        tend(L, q);
    }
    mg_setup(D, L, mg_prec);
}

Launch on_stream(const Launch& L, cudaStream_t st) {
    Launch B = L;
    B.stream = st;
    return B;
}

}  // namespace

bool capture_fp64(const Dev& D, const Launch& L, const cudaStream_t* side, int maxit, int check_every, int precond,
                  int mg_prec, int* d_nconv) {
    precond_setup(D, L, precond, mg_prec);
    cudaMemsetAsync(d_nconv, 0, sizeof(int), L.stream);
    int q = tbegin(L, K_BICG_INIT);
    launch_pdl(L, k_init64, L.nblk_rows, BS_THREADS, 0, D, d_nconv);
    tend(L, q);
    cudaMemsetAsync(&D.loop->it, 0, sizeof(int), L.stream);
    cudaGraphConditionalHandle h;
    if (!cond_handle(L.stream, 1, &h)) return false;
    const bool ok = cond_node(L.stream, side[0], cudaGraphCondTypeWhile, h, [&]() {
        const Launch B = on_stream(L, side[0]);
        const int64_t b0 = *L.launches;
        for (int c = 0; c < check_every; ++c) bicg_iteration(D, B, precond, mg_prec, d_nconv);
        const int nk = (int)(*L.launches - b0) + 1;
        k_cond_iter<<<1, 32, 0, side[0]>>>(D, d_nconv, h, check_every, maxit, nk);
        *L.launches = b0;   // counted on the device per iteration of the loop
        return cudaGetLastError() == cudaSuccess;
    });
    q = tbegin(L, K_TRUERES);
    launch_pdl(L, k_true_res64, L.nblk_rows, BS_THREADS, 0, D);
    tend(L, q);
    return ok;
}

bool capture_fgmres(const Dev& D, const Launch& L, const cudaStream_t* side, int maxit, int check_every,
                    int precond, int mg_prec, int* d_nconv) {
    precond_setup(D, L, precond, mg_prec);
    const int mgmode = precond ? (mg_prec == BS_PREC_MIXED ? 2 : 1) : 0;
    cudaMemsetAsync(d_nconv, 0, 2 * sizeof(int), L.stream);
    cudaMemsetAsync(&D.loop->cycle, 0, sizeof(int), L.stream);
    cudaGraphConditionalHandle hc, hif, hcol;
    if (!cond_handle(L.stream, 1, &hc)) return false;
    const bool ok = cond_node(L.stream, side[0], cudaGraphCondTypeWhile, hc, [&]() {
        // one restart cycle: start (true residual, norms), then its columns
        const Launch B0 = on_stream(L, side[0]);
        const int64_t b0 = *L.launches;
        cudaMemcpyAsync(d_nconv, d_nconv + 1, sizeof(int), cudaMemcpyDeviceToDevice, side[0]);
        int q0 = tbegin(B0, K_FG_START);
        launch_pdl(B0, k_fg_start, L.nblk_rows, BS_THREADS, 0, D, 0, d_nconv, (const int*)&D.loop->cycle);
        tend(B0, q0);
        if (!cond_handle(side[0], 0, &hif)) return false;
        k_cond_cycle<<<1, 32, 0, side[0]>>>(D, d_nconv, hc, hif, maxit, 2);
        const bool ok1 = cond_node(side[0], side[1], cudaGraphCondTypeIf, hif, [&]() {
            const Launch B1 = on_stream(L, side[1]);
            if (D.fg_df) fg_put(D, B1, mgmode);
            if (!cond_handle(side[1], 1, &hcol)) return false;
            // the cycle's own kernels: put (double-float basis), this one, the solve and the update
            k_col_init<<<1, 32, 0, side[1]>>>(D, hcol, (D.fg_df ? 1 : 0) + 3);
            const bool ok2 = cond_node(side[1], side[2], cudaGraphCondTypeWhile, hcol, [&]() {
                const Launch B2 = on_stream(L, side[2]);
                const int64_t b2 = *L.launches;
                for (int c = 0; c < check_every; ++c) fg_column(D, B2, precond, mg_prec, mgmode, d_nconv);
                const int nk = (int)(*L.launches - b2) + 1;
                k_cond_col<<<1, 32, 0, side[2]>>>(D, d_nconv, hcol, check_every, nk);
                *L.launches = b2;
                return cudaGetLastError() == cudaSuccess;
            });
            int q1 = tbegin(B1, K_FG_UPD);
            launch_pdl(B1, k_fg_solve, D.nscene, 32, 0, D, d_nconv);
            launch_pdl(B1, k_fg_update, L.nblk_rows, BS_THREADS, 0, D, precond);
            tend(B1, q1);
            return ok2 && cudaGetLastError() == cudaSuccess;
        });
        *L.launches = b0;
        return ok1 && cudaGetLastError() == cudaSuccess;
    });
    int q = tbegin(L, K_TRUERES);
    launch_pdl(L, k_true_res64, L.nblk_rows, BS_THREADS, 0, D);
    tend(L, q);
    return ok;
}

// scalar sub-step pairs of the captured step
__global__ void k_cond_scalar(Dev D, cudaGraphConditionalHandle h, int body_kernels) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    LoopCtl* C = D.loop;
    C->kernels += (unsigned long long)body_kernels;
    C->j += 2;
    int mx = 1;
    for (int s = 0; s < D.nscene; ++s) mx = max(mx, D.dyn[s].solsteps);
    // the same sub-step count as the host loop (bounded: solsteps is finite)
    cudaGraphSetConditional(h, C->j < mx ? 1u : 0u);
}

void cond_scalar(const Dev& D, cudaStream_t st, cudaGraphConditionalHandle h, int body_kernels) {
    k_cond_scalar<<<1, 32, 0, st>>>(D, h, body_kernels);
}

}  // namespace bs
