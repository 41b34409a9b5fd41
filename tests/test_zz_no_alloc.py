"""GPU test of bs_bicgstab_csr_noalloc, the entry point that allocates
nothing (for callers whose device memory belongs to their own allocator and
that cannot let the library call cudaMalloc/cudaFree).  It is checked through
the C-ABI against the allocating entry point bs_bicgstab_csr on two calls in a
row, which share the library's fixed scratch array.  Device buffers for the
inputs come from torch (plumbing only)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KAT_ROW = np.array([1, 4, 6, 8, 11, 14]) - 1
KAT_COL = np.array([1, 3, 4, 2, 4, 1, 3, 2, 3, 4, 1, 2, 5]) - 1


def _ppe_csr(api):
    """A Jacobi-scaled PPE of a small jittered lattice, as CSR (diagonal included)."""
    from beachslope_gb300 import scene
    p, st, gr = scene.lattice_scene(n=40, dx=1e-3, seed=4)
    ctx = api.Context([p], [st], [None])
    for nm in ("search", "porosity", "int_vel", "ppe_assemble"):
        ctx.stage(nm)
    c, idx, *_ = ctx.neighbours()
    d, off, _ = ctx.matrix()
    n = len(c)
    rows, cols, vals = [], [], []
    for i in range(n):
        rows.append(np.full(c[i] + 1, i))
        cols.append(np.concatenate([[i], idx[i, :c[i]]]))
        vals.append(np.concatenate([[d[i]], off[i, :c[i]]]))
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp)
    b = np.random.default_rng(9).standard_normal(n)
    return rp, cols, vals, b


def test_noalloc_matches_allocating_entry_point(api):
    torch = pytest.importorskip("torch")
    systems = [(KAT_ROW, KAT_COL, np.ones(13), np.array([8.0, 6.0, 4.0, 9.0, 8.0])), _ppe_csr(api)]
    dev = torch.device("cuda:0")
    for rp, col, val, b in systems:   # two calls in a row on the shared scratch
        n = len(b)
        x0 = np.ones(n)
        rc, xref, it_ref, rr_ref = api.bicgstab_csr(rp, col, val, b, x0, tol=1e-12, maxit=5000)
        assert rc == 0
        t = _device_system(torch, dev, rp, col, val, b)
        t_x = torch.tensor(x0, device=dev)
        torch.cuda.synchronize()
        rc, it, rr = api.bicgstab_csr_noalloc(n, *t, t_x.data_ptr(), tol=1e-12, maxit=5000)
        x = t_x.cpu().numpy()
        assert rc == 0, rc
        assert rr <= 1e-11
        # the same recurrence: the same number of iterations
        assert it == it_ref, (it, it_ref)
        # the tolerance the parity tests use for converged FP64 solves
        assert np.linalg.norm(x - xref) / np.linalg.norm(xref) < 1e-9


def _device_system(torch, dev, rp, col, val, b):
    ts = [torch.tensor(np.asarray(rp, np.int32), device=dev), torch.tensor(np.asarray(col, np.int32), device=dev),
          torch.tensor(np.asarray(val, np.float64), device=dev), torch.tensor(np.asarray(b, np.float64), device=dev)]
    _device_system.keep = ts   # the tensors must outlive the call
    return [q.data_ptr() for q in ts]


def test_noalloc_iteration_count(api):
    """An exact initial guess takes no iteration; a capped solve stops at
    maxit, reports maxit iterations and the not-converged status, as the
    allocating entry point does."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    b = np.array([8.0, 6.0, 4.0, 9.0, 8.0])
    t = _device_system(torch, dev, KAT_ROW, KAT_COL, np.ones(13), b)
    t_x = torch.tensor(np.arange(1.0, 6.0), device=dev)   # solvertest.f90's solution
    torch.cuda.synchronize()
    rc, it, rr = api.bicgstab_csr_noalloc(5, *t, t_x.data_ptr(), tol=1e-12, maxit=5)
    assert (rc, it) == (0, 0)
    assert rr == 0.0
    rp, col, val, b = _ppe_csr(api)
    for maxit in (1, 3, 5, 6):
        rc_ref, _, it_ref, _ = api.bicgstab_csr(rp, col, val, b, np.zeros(len(b)), tol=1e-14, maxit=maxit)
        t = _device_system(torch, dev, rp, col, val, b)
        t_x = torch.zeros(len(b), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc, it, rr = api.bicgstab_csr_noalloc(len(b), *t, t_x.data_ptr(), tol=1e-14, maxit=maxit)
        assert rc == -5 and rc_ref == -5, (rc, rc_ref)   # BS_E_NOTCONV
        assert it == maxit == it_ref, (it, maxit, it_ref)


def test_noalloc_rejects_oversize(api):
    rc, it, rr = api.bicgstab_csr_noalloc(70000, 0, 0, 0, 0, 0)
    assert rc == -1 or rc == -4
    rc, it, rr = api.bicgstab_csr_noalloc(70000, 8, 8, 8, 8, 8)
    assert rc == -4   # BS_E_CAPACITY: more rows than the fixed scratch holds
