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

// K1: p' = r + beta (p - omega v);  v' = A p';  partial (rhat, v')
__global__ void k_it1_64(Dev D, const double* __restrict__ p, const double* __restrict__ v, double* pn, double* vn) {
    const int s = D.blk_scene[blockIdx.x];
    if (scene_done(D, s)) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const double beta = D.dyn[s].beta, omega = D.dyn[s].omega;
    double q[1] = {0.0};
    if (r < P.row0 + D.dyn[s].n) {
        const double* A = (const double*)D.aval;
        const double pi = D.sr[r] + beta * (p[r] - omega * v[r]);
        double acc = D.adiag[r] * pi;
        const int n = D.ncount[r];
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, D.kmax);
            const int j = D.nidx[e];
            acc += A[e] * (D.sr[j] + beta * (p[j] - omega * v[j]));
        }
        pn[r] = pi;
        vn[r] = acc;
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

// K2: s = r - alpha v;  t = A s;  partials (t,s), (t,t)
__global__ void k_it2_64(Dev D, const double* __restrict__ v) {
    const int s = D.blk_scene[blockIdx.x];
    if (scene_done(D, s)) return;
    const ScenePar& P = D.par[s];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = D.dyn[s].alpha;
    double q[2] = {0.0, 0.0};
    if (r < P.row0 + D.dyn[s].n) {
        const double* A = (const double*)D.aval;
        const double si = D.sr[r] - alpha * v[r];
        double acc = D.adiag[r] * si;
        const int n = D.ncount[r];
        for (int k = 0; k < n; ++k) {
            const long e = ell(r, k, D.kmax);
            const int j = D.nidx[e];
            acc += A[e] * (D.sr[j] - alpha * v[j]);
        }
        D.ss[r] = si;
        D.st[r] = acc;
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

// K3: x += alpha p + omega s;  r = s - omega t;  partials (rhat, r), (r,r)
__global__ void k_it3_64(Dev D, const double* __restrict__ p, int* nconv) {
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
        const double xn = xo + alpha * p[r] + omega * si;
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

// true FP64 residual ||b - A x|| / ||b|| for every scene (no early exit)
__global__ void k_true_res64(Dev D) {
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

}  // namespace

namespace bs {

// Host driver of the FP64 solve.  Checks the converged-scene counter every
// `check_every` iterations (one event sync), so the host never waits per
// iteration.
void solve_fp64(const Dev& D, const Launch& L, int maxit, int check_every, const int*, int* d_nconv,
                int* h_nconv, cudaEvent_t ev) {
    cudaMemsetAsync(d_nconv, 0, sizeof(int), L.stream);
    int q = tbegin(L, K_BICG_INIT);
    k_init64<<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D, d_nconv);
    tend(L, q);
    double *p = D.sp, *v = D.sv, *p2 = D.sp2, *v2 = D.sv2;
    int it = 0;
    while (it < maxit) {
        cudaMemcpyAsync(h_nconv, d_nconv, sizeof(int), cudaMemcpyDeviceToHost, L.stream);
        cudaEventRecord(ev, L.stream);
        const int chunk = check_every;
        for (int c = 0; c < chunk && it < maxit; ++c, ++it) {
            q = tbegin(L, K_BICG_IT1);
            k_it1_64<<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D, p, v, p2, v2);
            tend(L, q);
            q = tbegin(L, K_BICG_IT2);
            k_it2_64<<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D, v2);
            tend(L, q);
            q = tbegin(L, K_BICG_IT3);
            k_it3_64<<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D, p2, d_nconv);
            tend(L, q);
            double* t;
            t = p; p = p2; p2 = t;
            t = v; v = v2; v2 = t;
        }
        // the counter copied before this chunk: decide whether to go on
        cudaEventSynchronize(ev);
        timer_collect(L.timer, false);
        if (*h_nconv >= D.nscene) break;
    }
    q = tbegin(L, K_TRUERES);
    k_true_res64<<<L.nblk_rows, BS_THREADS, 0, L.stream>>>(D);
    tend(L, q);
}

void solve_mixed(const Dev& D, const Launch& L, int maxit, int check_every, int* d_nconv, int* h_nconv,
                 cudaEvent_t ev) {
    // mixed precision solver: added with the FP32 inner iteration
    solve_fp64(D, L, maxit, check_every, nullptr, d_nconv, h_nconv, ev);
}

}  // namespace bs
