"""Error bounds of the mixed search's FP64 square root and reciprocal
(fast_r64 / fast_rcp64, bs_internal.cuh): an FP32 hardware seed refined by one
Newton step (for 1/sqrt(s): y <- y (3 - s y^2) / 2; for 1/d: y <- y (2 - d y)).
One step squares the seed's relative error e0: 1.5 e0^2 for 1/sqrt, e0^2 for
1/d.  With e0 of a few FP32 ulp (2^-22) that is ~1e-13 and ~1e-14.  The test
evaluates both on the GPU beside CUDA's correctly rounded sqrt and IEEE
division over a log-uniform sweep of inputs and the pair distances the search
meets (squared spacings of 0.1-2.6 lattice steps at dx = 1e-3 ... 2e-2 m)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    pytest.skip("nvcc not found")


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fastmath") / "libfastmath.so")
    subprocess.check_call([_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                           "-Xcompiler", "-fPIC", "-shared", os.path.join(HERE, "fastmath_probe.cu"), "-o", out])
    lib = C.CDLL(out)
    lib.fm_eval.restype = C.c_int
    lib.fm_eval.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    return lib


def _inputs():
    rng = np.random.default_rng(20261204)
    sweep = 10.0 ** rng.uniform(-14, 4, 400_000)
    dx = 10.0 ** rng.uniform(-3, np.log10(2e-2), 200_000)
    pair = (dx * rng.uniform(0.1, 2.6, dx.size)) ** 2
    lam = 1e-3 * (1.3 * dx) ** 2   # the search's regulariser lambda = 1e-3 h^2 added before 1/(r^2+lambda)
    return np.concatenate([sweep, pair, pair + lam, [1.0, 0.25, 4.0, 2.0 ** -20]])


def test_fast_sqrt_and_reciprocal_error_bounds(probe):
    s = np.ascontiguousarray(_inputs())
    out = np.zeros(6 * s.size)
    rc = probe.fm_eval(s.size, s.ctypes.data, out.ctypes.data)
    assert rc == 0, f"CUDA error {rc}"
    o = out.reshape(-1, 6)
    r, ir, rcp, r_ref, ir_ref, rcp_ref = (o[:, k] for k in range(6))
    e_r = np.max(np.abs(r / r_ref - 1.0))
    e_ir = np.max(np.abs(ir / ir_ref - 1.0))
    e_rcp = np.max(np.abs(rcp / rcp_ref - 1.0))
    print(f"max rel error: sqrt {e_r:.2e}, 1/sqrt {e_ir:.2e}, 1/d {e_rcp:.2e}")
    # bounds: 1.5 e0^2 + rounding with e0 <= 4.8e-7 (2 ulp rsqrtf plus the
    # FP32 conversion of s), e0^2 + rounding with e0 <= 1.2e-7 for 1/d
    assert e_ir <= 4e-13, e_ir
    assert e_r <= 4e-13, e_r
    assert e_rcp <= 2e-14, e_rcp
