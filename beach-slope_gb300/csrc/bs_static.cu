// bs_static.cu -- BiCGStab on a caller-owned device CSR system that
// allocates nothing.
//
// Some callers cannot let a library call cudaMalloc/cudaFree: hosts whose
// device memory is owned by their own pool allocator (a framework that
// reserves HBM up front and forbids third-party allocations), or code that
// must not stall -- cudaMalloc and cudaFree may synchronise the device and
// take unbounded time.  This entry point keeps all of its solver scratch
// (the six Krylov vectors, block partial sums and the scalars) in one
// file-scope device array of fixed size, so a call only launches kernels and
// copies a few scalars back to the host.
//
// Limits and rules:
//  * n <= BS_STATIC_MAX_ROWS (65,536) rows; larger systems are rejected with
//    BS_E_CAPACITY before any work.
//  * The array (about 3.2 MB) is part of the library's device image: every
//    GPU that loads the library holds it until the process exits.
//  * Every call shares the array and it keeps the last call's contents; each
//    call clears what must start at zero (p, v, the converged flag).  Calls
//    whose work overlaps on the GPU (different streams, or host threads
//    without ordering) race on the array: serialise them.
//  * The device address of the array is looked up with cudaGetSymbolAddress
//    on the first call on each device (that device current) and cached; make
//    that first call before any stream capture begins.
//  * Convergence is judged on the recursive residual, as bs_bicgstab_csr
//    judges it; *relres reports the true residual ||b - A x|| / ||b||
//    computed after the last iteration.  The flag is read back to the host
//    every four iterations (the call waits for its stream there), so the
//    call cannot run on a stream that is being captured.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "bs_internal.cuh"

#define BS_STATIC_MAX_ROWS 65536
#define BS_STATIC_THREADS 256
#define BS_STATIC_MAX_BLOCKS (BS_STATIC_MAX_ROWS / BS_STATIC_THREADS)
#define BS_STATIC_NPART 4

// scratch layout (doubles): r, rhat, p, v, s, t [MAX_ROWS each] |
// partials [MAX_BLOCKS * NPART] | scalars [32]
#define BS_STATIC_VEC (6L * BS_STATIC_MAX_ROWS)
#define BS_STATIC_WORDS (BS_STATIC_VEC + BS_STATIC_MAX_BLOCKS * BS_STATIC_NPART + 32)

static __device__ __align__(256) double bs_static_scratch[BS_STATIC_WORDS];

namespace {

// scalar slots
enum { S_RHO = 0, S_ALPHA, S_OMEGA, S_BETA, S_BNORM2, S_RNORM2, S_CONV, S_ITERS, S_RTRUE2, S_BREAK };

struct Csr {
    int n;
    const int* rp;
    const int* col;
    const double* val;
};

struct Scr {
    double *r, *rh, *p, *v, *s, *t, *part, *sc;
};

__host__ __device__ inline Scr carve(double* base) {
    Scr q;
    q.r = base;
    q.rh = base + BS_STATIC_MAX_ROWS;
    q.p = base + 2L * BS_STATIC_MAX_ROWS;
    q.v = base + 3L * BS_STATIC_MAX_ROWS;
    q.s = base + 4L * BS_STATIC_MAX_ROWS;
    q.t = base + 5L * BS_STATIC_MAX_ROWS;
    q.part = base + BS_STATIC_VEC;
    q.sc = q.part + BS_STATIC_MAX_BLOCKS * BS_STATIC_NPART;
    return q;
}

__device__ __forceinline__ double csr_row(const Csr& A, const double* __restrict__ u, int i) {
    double acc = 0.0;
    for (int e = A.rp[i]; e < A.rp[i + 1]; ++e) acc += A.val[e] * u[A.col[e]];
    return acc;
}

template <int NV>
__device__ __forceinline__ void block_partials(double (&v)[NV], double* part) {
    __shared__ double sh[NV * 32];
    block_sum<NV>(v, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) part[blockIdx.x * BS_STATIC_NPART + q] = v[q];
}

__device__ __forceinline__ bool done(const Scr& S) { return S.sc[S_CONV] != 0.0; }

__global__ void ks_init(Csr A, const double* __restrict__ b, const double* __restrict__ x, double* base) {
    const Scr S = carve(base);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double q[2] = {0.0, 0.0};
    if (i < A.n) {
        const double ri = b[i] - csr_row(A, x, i);
        S.r[i] = ri;
        S.rh[i] = ri;
        S.p[i] = 0.0;
        S.v[i] = 0.0;
        q[0] = b[i] * b[i];
        q[1] = ri * ri;
    }
    block_partials<2>(q, S.part);
}

// single block: sum the partials in block order and update the scalars
__global__ void ks_reduce(int nblk, int phase, double tol, int maxit, double* base) {
    const Scr S = carve(base);
    // the host launches iterations in groups: once a solve has converged the
    // iteration phases of the rest of the group leave every scalar (and the
    // iteration count) as they are; the flag is read by the whole block, so
    // the early return is uniform
    if (phase >= 1 && phase <= 3 && S.sc[S_CONV] != 0.0) return;
    __shared__ double sh[3 * 32];
    double a[3] = {0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
        for (int q = 0; q < 3; ++q) a[q] += S.part[b * BS_STATIC_NPART + q];
    block_sum<3>(a, sh);
    if (threadIdx.x != 0) return;
    double* sc = S.sc;
    if (phase == 0) {   // init: (b,b), (r,r)
        sc[S_BNORM2] = a[0];
        sc[S_RNORM2] = a[1];
        sc[S_RHO] = a[1];
        sc[S_ALPHA] = 1.0;
        sc[S_OMEGA] = 1.0;
        sc[S_BETA] = 0.0;
        sc[S_ITERS] = 0.0;
        sc[S_BREAK] = 0.0;
        sc[S_CONV] = (a[0] == 0.0 || a[1] <= tol * tol * a[0]) ? 1.0 : 0.0;
    } else if (phase == 1) {   // (rhat, v) -> alpha
        if (a[0] == 0.0 || !isfinite(a[0])) {
            sc[S_BREAK] = 1.0;
            sc[S_ALPHA] = 0.0;
        } else {
            sc[S_ALPHA] = sc[S_RHO] / a[0];
        }
    } else if (phase == 2) {   // (t,s), (t,t) -> omega
        sc[S_OMEGA] = (a[1] != 0.0) ? a[0] / a[1] : 0.0;
        if (a[1] == 0.0) sc[S_BREAK] = 1.0;
    } else if (phase == 3) {   // (rhat, r), (r,r) -> beta, convergence
        sc[S_BETA] = (a[0] / sc[S_RHO]) * (sc[S_ALPHA] / sc[S_OMEGA]);
        sc[S_RHO] = a[0];
        sc[S_RNORM2] = a[1];
        sc[S_ITERS] += 1.0;
        const bool conv = a[1] <= tol * tol * sc[S_BNORM2] || !isfinite(a[1]) || sc[S_BREAK] != 0.0 ||
                          sc[S_ITERS] >= (double)maxit;
        sc[S_CONV] = conv ? 1.0 : 0.0;
    } else {   // true residual
        sc[S_RTRUE2] = a[0];
    }
}

__global__ void ks_p(Csr A, double* base) {
    const Scr S = carve(base);
    if (done(S)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    S.p[i] = S.r[i] + S.sc[S_BETA] * (S.p[i] - S.sc[S_OMEGA] * S.v[i]);
}

__global__ void ks_v(Csr A, double* base) {
    const Scr S = carve(base);
    if (done(S)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double q[1] = {0.0};
    if (i < A.n) {
        const double vi = csr_row(A, S.p, i);
        S.v[i] = vi;
        q[0] = S.rh[i] * vi;
    }
    block_partials<1>(q, S.part);
}

__global__ void ks_s(Csr A, double* base) {
    const Scr S = carve(base);
    if (done(S)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    S.s[i] = S.r[i] - S.sc[S_ALPHA] * S.v[i];
}

__global__ void ks_t(Csr A, double* base) {
    const Scr S = carve(base);
    if (done(S)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double q[2] = {0.0, 0.0};
    if (i < A.n) {
        const double ti = csr_row(A, S.s, i);
        S.t[i] = ti;
        q[0] = ti * S.s[i];
        q[1] = ti * ti;
    }
    block_partials<2>(q, S.part);
}

__global__ void ks_x(Csr A, double* __restrict__ x, double* base) {
    const Scr S = carve(base);
    if (done(S)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double q[2] = {0.0, 0.0};
    if (i < A.n) {
        const double a = S.sc[S_ALPHA], w = S.sc[S_OMEGA];
        x[i] = x[i] + a * S.p[i] + w * S.s[i];
        const double ri = S.s[i] - w * S.t[i];
        S.r[i] = ri;
        q[0] = S.rh[i] * ri;
        q[1] = ri * ri;
    }
    block_partials<2>(q, S.part);
}

__global__ void ks_true(Csr A, const double* __restrict__ b, const double* __restrict__ x, double* base) {
    const Scr S = carve(base);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double q[1] = {0.0};
    if (i < A.n) {
        const double ri = b[i] - csr_row(A, x, i);
        q[0] = ri * ri;
    }
    block_partials<1>(q, S.part);
}

// device address of the scratch array, looked up once per device
std::mutex g_mu;
double* g_addr[64] = {};

int scratch_for_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return BS_E_CUDA;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, bs_static_scratch);
        if (e != cudaSuccess || !p) return BS_E_CUDA;
        g_addr[dev] = (double*)p;
    }
    *out = g_addr[dev];
    return BS_OK;
}

}  // namespace

extern "C" int bs_bicgstab_csr_noalloc(int32_t n, const int32_t* d_row_ptr, const int32_t* d_col,
                                       const double* d_val, const double* d_b, double* d_x, double tol,
                                       int32_t maxit, void* stream, int32_t* iters, double* relres) {
    if (n <= 0 || !d_row_ptr || !d_col || !d_val || !d_b || !d_x || maxit <= 0 || !(tol >= 0.0)) return BS_E_ARG;
    if (n > BS_STATIC_MAX_ROWS) return BS_E_CAPACITY;
    double* base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const Csr A{n, d_row_ptr, d_col, d_val};
    const int nb = (n + BS_STATIC_THREADS - 1) / BS_STATIC_THREADS;
    ks_init<<<nb, BS_STATIC_THREADS, 0, st>>>(A, d_b, d_x, base);
    ks_reduce<<<1, 256, 0, st>>>(nb, 0, tol, maxit, base);
    double sc[32];
    const Scr S = carve(base);
    int it = 0;
    while (true) {
        // check every 4 iterations; kernels of a converged solve return at once
        for (int c = 0; c < 4; ++c, ++it) {
            ks_p<<<nb, BS_STATIC_THREADS, 0, st>>>(A, base);
            ks_v<<<nb, BS_STATIC_THREADS, 0, st>>>(A, base);
            ks_reduce<<<1, 256, 0, st>>>(nb, 1, tol, maxit, base);
            ks_s<<<nb, BS_STATIC_THREADS, 0, st>>>(A, base);
            ks_t<<<nb, BS_STATIC_THREADS, 0, st>>>(A, base);
            ks_reduce<<<1, 256, 0, st>>>(nb, 2, tol, maxit, base);
            ks_x<<<nb, BS_STATIC_THREADS, 0, st>>>(A, d_x, base);
            ks_reduce<<<1, 256, 0, st>>>(nb, 3, tol, maxit, base);
        }
        if (cudaMemcpyAsync(sc, S.sc, sizeof(sc), cudaMemcpyDeviceToHost, st) != cudaSuccess) return BS_E_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return BS_E_CUDA;
        if (sc[S_CONV] != 0.0 || it >= maxit) break;
    }
    ks_true<<<nb, BS_STATIC_THREADS, 0, st>>>(A, d_b, d_x, base);
    ks_reduce<<<1, 256, 0, st>>>(nb, 4, tol, maxit, base);
    if (cudaMemcpyAsync(sc, S.sc, sizeof(sc), cudaMemcpyDeviceToHost, st) != cudaSuccess) return BS_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return BS_E_CUDA;
    if (cudaGetLastError() != cudaSuccess) return BS_E_CUDA;
    if (iters) *iters = (int32_t)sc[S_ITERS];
    if (relres) *relres = sc[S_BNORM2] > 0.0 ? std::sqrt(sc[S_RTRUE2] / sc[S_BNORM2]) : std::sqrt(sc[S_RTRUE2]);
    const bool ok = sc[S_BNORM2] == 0.0 || sc[S_RNORM2] <= tol * tol * sc[S_BNORM2];
    return ok ? BS_OK : BS_E_NOTCONV;
}
