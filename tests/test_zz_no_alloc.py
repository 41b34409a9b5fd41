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
        rc, xref, _, rr_ref = api.bicgstab_csr(rp, col, val, b, x0, tol=1e-12, maxit=5000)
        assert rc == 0
        t_rp = torch.tensor(np.asarray(rp, np.int32), device=dev)
        t_col = torch.tensor(np.asarray(col, np.int32), device=dev)
        t_val = torch.tensor(np.asarray(val, np.float64), device=dev)
        t_b = torch.tensor(np.asarray(b, np.float64), device=dev)
        t_x = torch.tensor(x0, device=dev)
        torch.cuda.synchronize()
        rc, it, rr = api.bicgstab_csr_noalloc(n, t_rp.data_ptr(), t_col.data_ptr(), t_val.data_ptr(),
                                              t_b.data_ptr(), t_x.data_ptr(), tol=1e-12, maxit=5000)
        x = t_x.cpu().numpy()
        assert rc == 0, rc
        assert rr <= 1e-11
        # the tolerance the parity tests use for converged FP64 solves
        assert np.linalg.norm(x - xref) / np.linalg.norm(xref) < 1e-9


def test_noalloc_rejects_oversize(api):
    rc, it, rr = api.bicgstab_csr_noalloc(70000, 0, 0, 0, 0, 0)
    assert rc == -1 or rc == -4
    rc, it, rr = api.bicgstab_csr_noalloc(70000, 8, 8, 8, 8, 8)
    assert rc == -4   # BS_E_CAPACITY: more rows than the fixed scratch holds
