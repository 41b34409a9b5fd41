"""bench.py's roofline arithmetic on a fake context (no GPU): the basis
vectors an FGMRES solve reads, the algorithmic bytes and FP64 work per
launch of the candidate kernels, and the peak lookup."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


class _Fake:
    nscenes = 2

    def neighbour_counts(self, s):
        return np.full(1000 * (s + 1), 20, np.int32)   # 1000 and 2000 rows, 20 neighbours each


def test_fg_columns(bench):
    assert bench.fg_columns(37, 120) == 37 * 38 // 2
    assert bench.fg_columns(200, 150) == 150 * 151 // 2 + 50 * 51 // 2
    assert bench.fg_columns(0, 50) == 0


def test_algorithmic_bytes(bench):
    f = _Fake()
    n, nnz = 3000.0, 60000.0
    assert bench.algorithmic_bytes(f, "fg_arnoldi_spmv", "mixed", basis_reads=10) == \
        nnz * 12 + n * 28 + n * 16 + 10 * n * 8
    assert bench.algorithmic_bytes(f, "fg_project", "mixed", basis_reads=10) == n * 16 + 10 * n * 8
    assert bench.algorithmic_bytes(f, "bicg_it1_spmv", "fp64") == nnz * 12 + n * 36
    # the particle-level sweeps read 4-byte matrix values in the mixed form, 8 in FP64
    m, d = (bench.algorithmic_bytes(f, "mg_l0_up", p) for p in ("mixed", "fp64"))
    assert d - m == nnz * 4 + n * 4
    # the search stores four pair values per neighbour: 4 bytes each in the
    # mixed form, 8 in FP64 (copies the mixed form keeps for the FP32 pipe,
    # such as the correction matrix as (hi, lo) pairs, are not algorithmic)
    m, d = (bench.algorithmic_bytes(f, "search_effpor", p) for p in ("mixed", "fp64"))
    assert d - m == nnz * 16


def test_fp64_work(bench):
    f = _Fake()
    n, nnz = 3000.0, 60000.0
    assert bench.fp64_flops(f, "fg_arnoldi_spmv", 10, df=False) == 2 * nnz + 2 * n + 40 * n
    assert bench.fp64_flops(f, "fg_arnoldi_spmv", 10, df=True) == 4 * n
    assert bench.fp64_flops(f, "fg_project", 10, df=True) == 2 * n
    assert bench.fp64_flops(f, "search_effpor", 10) is None


def test_peaks_measured_or_fallback(bench):
    v, src = bench.peaks()
    assert src in ("measured", "fallback") and v > 1000
