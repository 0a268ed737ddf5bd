"""Pins the oracle to the reference: the reference's own kernels, compiled
from its sources (oracle/build_ref.py), run on the GPU and are compared with
the CPU restatement bit for bit.  Together with tests/test_parity_gpu.py this
chains library == oracle == reference.

The reference's solver kernels apply ILU(0) with busy-wait triangular solves
that spin until a neighbour's value is finite; they are only run on inputs for
which the oracle (the same arithmetic) shows every system converging with
finite values, and only at sizes within the reference's limits (n <= 512 for
the busy-wait solves, nnz <= 2560 for its true-residual kernel).  The
spin-waiting ILU approaches 2 and 3 are never run."""
import numpy as np
import pytest

import bilu
import helpers as H
import oracle as O
import ref as R

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not R.available(), reason="reference kernels not built")]

FAMILIES = ["2d5_8x8", "2d5_16x16", "cd2d_12x12", "3d7_5x5x5", "3d7_7x7x7"]
NSYS = 12


def _safe(o):
    assert np.all(o["conv"] == 1) and np.all(np.isfinite(o["x"])), "input would not be safe for the reference"


def _cmp(a, b, what, fields=("iters", "conv", "x", "res")):
    for f in fields:
        H.assert_bitwise(a[f], b[f], f"{what}: {f}")


@pytest.mark.parametrize("family", FAMILIES)
def test_reference_merged_solver(cuda, family):
    rp, ci, v, b = H.workload(family, NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0, approach=1)
    _safe(o)
    r = R.merged_solve(cuda, rp, ci, v, b)
    _cmp(r, o, f"reference merged solver {family}", fields=("iters", "conv", "x", "res", "true_res"))
    H.assert_bitwise(r["lu"], o["lu"], f"reference merged solver {family}: in-kernel ILU(0) factors")
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0)
    _cmp(g, r, f"library vs reference merged solver {family}", fields=("iters", "conv", "x", "res", "true_res"))


@pytest.mark.parametrize("family", FAMILIES)
@pytest.mark.parametrize("approach", [1, 4])
def test_reference_ilu0_kernels(cuda, family, approach):
    rp, ci, v, _ = H.workload(family, NSYS)
    H.assert_bitwise(R.ilu0(cuda, rp, ci, v, approach), O.ilu0(rp, ci, v, approach),
                     f"reference ILU(0) approach {approach} {family}")


@pytest.mark.parametrize("family", ["2d5_16x16", "3d7_7x7x7"])
@pytest.mark.parametrize("approach", [1, 3])
def test_reference_split_solver(cuda, family, approach):
    rp, ci, v, b = H.workload(family, NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0_SPLIT, approach=approach)
    _safe(o)
    r = R.split_solve(cuda, rp, ci, v, b, o["lu"])
    _cmp(r, o, f"reference split solver {family} approach {approach}")


@pytest.mark.parametrize("family", FAMILIES)
def test_reference_isai_kernels(cuda, family):
    rp, ci, v, _ = H.workload(family, NSYS)
    lu = O.ilu0(rp, ci, v, 3)
    lrp, lci, urp, uci = O.split_pattern(rp, ci)
    Lv, Uv = O.split_values(rp, ci, lu)
    for (trp, tci, T, tri, nm) in ((lrp, lci, Lv, 0, "L"), (urp, uci, Uv, 1, "U")):
        arp, aci = O.isai_pattern(trp, tci, 2, T[0])  # the reference's numeric pattern of page 0
        H.assert_bitwise(R.isai(cuda, trp, tci, T, tri, arp, aci), O.isai_values(trp, tci, T, tri, arp, aci),
                         f"reference ISAI({nm}) {family}")


@pytest.mark.parametrize("family", ["2d5_16x16", "3d7_5x5x5", "3d7_7x7x7"])
def test_reference_isai_solver(cuda, family):
    rp, ci, v, b = H.workload(family, NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0_ISAI, approach=3)
    _safe(o)
    r = R.isai_solve(cuda, rp, ci, v, b, (*o["ail_pattern"], o["ail"]), (*o["aiu_pattern"], o["aiu"]))
    _cmp(r, o, f"reference ILU-ISAI solver {family}")
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0_ISAI, ilu_approach=3)
    _cmp(g, r, f"library vs reference ILU-ISAI solver {family}")


@pytest.mark.parametrize("family", ["2d5_8x8", "3d7_5x5x5"])
def test_reference_parilu_reaches_the_same_fixed_point(cuda, family):
    """The reference sweeps update in place without a barrier (order depends on thread timing), so
    single sweeps are not comparable bit for bit; after enough sweeps both schedules reach the exact
    ILU(0) fixed point."""
    rp, ci, v, _ = H.workload(family, NSYS)
    r = R.parilu(cuda, rp, ci, v, 80)
    j = O.parilu0(rp, ci, v, 80)
    a3 = O.ilu0(rp, ci, v, 3)
    np.testing.assert_allclose(r, a3, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(j, a3, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("family", ["2d5_8x8", "2d5_16x16", "cd2d_12x12", "3d7_5x5x5"])
def test_reference_general_isai(cuda, family):
    """GenerateISAI_gpu(aiA, A, general, 1)'s kernels (Gauss-Jordan with partial pivoting) and the general-ISAI
    solver kernel, against the oracle and the library."""
    rp, ci, v, b = H.workload(family, NSYS)
    arp, aci = O.isai_pattern(rp, ci, 1, v[0])
    ai = O.isai_values(rp, ci, v, 2, arp, aci)
    H.assert_bitwise(R.isai(cuda, rp, ci, v, 2, arp, aci), ai, f"reference general ISAI {family}")
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_GENERAL_ISAI, isai_power=1)
    _safe(o)
    r = R.general_isai_solve(cuda, rp, ci, v, b, (arp, aci, ai))
    _cmp(r, o, f"reference general-ISAI solver {family}")
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_GENERAL_ISAI, isai_power=1)
    _cmp(g, r, f"library vs reference general-ISAI solver {family}")

