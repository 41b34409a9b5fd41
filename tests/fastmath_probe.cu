// Test harness (built by tests/test_fastmath.py with nvcc): evaluates the
// library's Newton-refined square root / reciprocal helpers (fast_r64,
// fast_rcp64 in bs_internal.cuh) beside CUDA's correctly rounded sqrt and
// IEEE division on the same inputs, so the test can bound their errors.
#include <cuda_runtime.h>

#include "../beach-slope_gb300/csrc/bs_internal.cuh"

__global__ void k_eval(int n, const double* __restrict__ s, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = s[i];
    double r, ir;
    fast_r64(x, r, ir);
    out[6L * i + 0] = r;
    out[6L * i + 1] = ir;
    out[6L * i + 2] = fast_rcp64(x);
    out[6L * i + 3] = sqrt(x);
    out[6L * i + 4] = 1.0 / sqrt(x);
    out[6L * i + 5] = 1.0 / x;
}

// s: n host inputs; out: 6n host outputs (r, 1/r, 1/s from the helpers, then
// sqrt(s), 1/sqrt(s), 1/s from CUDA).  Returns 0 or a CUDA error code.
extern "C" int fm_eval(int n, const double* s, double* out) {
    double *ds = nullptr, *dout = nullptr;
    cudaError_t e = cudaMalloc(&ds, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(double) * 6 * n);
    if (e == cudaSuccess) e = cudaMemcpy(ds, s, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_eval<<<(n + 255) / 256, 256>>>(n, ds, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost);
    cudaFree(ds);
    cudaFree(dout);
    return (int)e;
}
