"""The library against the reference's own kernels on the same GPU.

The reference's solver kernels (compiled from its sources into oracle/_ref by
oracle/build_ref.py, launched by oracle/ref_launch.cpp) and the library solve
the same seeded batches with the reference's stopping rule (absolute
recursive-residual tolerance 1e-11, at most 500 iterations):

* the merged ILU(0)-BiCGSTAB solver (PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu,
  the reference's namesake path) on 16384 systems of the 2D 5-point 16x16
  pattern and 4096 systems of the 3D 7-point 7x7x7 pattern;
* the ILU-ISAI solver kernel (PrecondBiCGSTAB_ilu_isai_gpu.cu:49-262) with
  ISAI factors given, on the 16x16 batch; the library's time includes
  generating its factors, the reference's does not.

The library's reference-order mode reproduces the reference's iteration
counts exactly; both library modes must be faster than the reference kernel.
The times are printed (pytest -s) in one line per case, prefixed "speed:".

The reference kernels apply ILU(0) with busy-wait triangular solves, so they
only run after the library's reference-order solve of the same batch (bit
identical to the reference, tests/test_ref_pin.py) shows every system
converging with finite values, and only at n <= 512."""
import time

import numpy as np
import pytest

import bilu
import helpers as H
import oracle as O
import ref as R

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not R.available(), reason="reference kernels not built")]

ABS = dict(tol_mode=bilu.TOL_ABS, tol=1e-11, max_iter=500)


def _time_ours(dev, plan, V, B, reps=5):
    import torch
    nsys = B.shape[0]
    X = torch.empty_like(B)
    it = torch.empty(nsys, dtype=torch.float32, device=dev)
    cv = torch.empty(nsys, dtype=torch.int32, device=dev)
    rs = torch.empty(nsys, dtype=torch.float64, device=dev)
    plan.solve(V, B, X, it, cv, rs)
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.solve(V, B, X, it, cv, rs)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts)), it.cpu().numpy(), cv.cpu().numpy(), X.cpu().numpy()


def _time_ref(fn, args, reps=3):
    import torch
    R._call(fn, *args)  # warm-up (module load, first launch)
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        R._call(fn, *args)  # synchronous: returns after the kernel finished
        ts.append(1e3 * (time.perf_counter() - t0))
    return float(np.median(ts))


def _report(case, nsys, ref_ms, ours):
    parts = [f"speed: {case}, {nsys} systems: reference kernel {ref_ms:.3f} ms ({nsys / ref_ms * 1e3:,.0f} systems/s)"]
    for name, ms in ours:
        parts.append(f"library {name} {ms:.3f} ms ({nsys / ms * 1e3:,.0f} systems/s, {ref_ms / ms:.2f}x)")
    print("; ".join(parts))


@pytest.mark.parametrize("family,nsys", [("2d5_16x16", 16384), ("3d7_7x7x7", 4096)])
def test_merged_solver_faster_than_reference(cuda, family, nsys):
    import torch
    rp, ci, v, b = H.workload(family, nsys)
    n, nnz = len(rp) - 1, len(ci)
    assert n <= 512
    V = torch.from_numpy(v).to(cuda)
    B = torch.from_numpy(b).to(cuda)
    with bilu.Plan(rp, ci, precond=bilu.PRECOND_ILU0, **ABS) as plan:
        ref_order_ms, it_lib, cv_lib, x_lib = _time_ours(cuda, plan, V, B)
    assert np.all(cv_lib == 1) and np.all(np.isfinite(x_lib)), "input would not be safe for the reference"
    with bilu.Plan(rp, ci, precond=bilu.PRECOND_ILU0, reduction=bilu.REDUCE_FAST, **ABS) as plan:
        fast_ms, it_fast, cv_fast, _ = _time_ours(cuda, plan, V, B)
    assert np.all(cv_fast == 1)

    RP = torch.from_numpy(rp.astype(np.int32)).to(cuda)
    CI = torch.from_numpy(ci.astype(np.int32)).to(cuda)
    D = torch.from_numpy(O.find_diag(rp, ci).astype(np.int32)).to(cuda)
    X = torch.zeros_like(B)
    F = torch.empty_like(V)
    it = torch.zeros(nsys, dtype=torch.float32, device=cuda)
    cv = torch.zeros(nsys, dtype=torch.int32, device=cuda)
    rs = torch.zeros(nsys, dtype=torch.float64, device=cuda)
    ref_ms = _time_ref(R.lib().ref_merged, (n, nnz, nsys, RP, CI, V, B, X, F, D, it, cv, rs))
    H.assert_bitwise(it.cpu().numpy(), it_lib, f"{family}: iteration counts, library reference order vs reference")
    H.assert_bitwise(X.cpu().numpy(), x_lib, f"{family}: solutions, library reference order vs reference")
    assert np.all(np.abs(it_fast - it_lib) <= 1.0)
    _report(f"merged ILU(0) BiCGSTAB, {family}", nsys, ref_ms,
            [("reference order", ref_order_ms), ("FAST order", fast_ms)])
    assert ref_order_ms < ref_ms and fast_ms < ref_ms


def test_ilu_isai_solver_faster_than_reference(cuda):
    import torch
    family, nsys = "2d5_16x16", 16384
    rp, ci, v, b = H.workload(family, nsys)
    n, nnz = len(rp) - 1, len(ci)
    V = torch.from_numpy(v).to(cuda)
    B = torch.from_numpy(b).to(cuda)
    opts = dict(precond=bilu.PRECOND_ILU0_ISAI, ilu_approach=1, **ABS)
    with bilu.Plan(rp, ci, **opts) as plan:
        ref_order_ms, it_lib, cv_lib, x_lib = _time_ours(cuda, plan, V, B)
        assert np.all(cv_lib == 1) and np.all(np.isfinite(x_lib)), "input would not be safe for the reference"
        # the reference solver kernel's inputs: the library's ISAI factors (bit-identical to the reference's
        # ISAI kernels, tests/test_ref_pin.py) on the reference's pattern of |L|^2 and |U|^2
        LU = torch.empty_like(V)
        plan.ilu0(V, LU, 1)
        arp, aci = plan.pattern(1)
        urp, uci = plan.pattern(2)
        AIL = torch.empty((nsys, len(aci)), dtype=torch.float64, device=cuda)
        AIU = torch.empty((nsys, len(uci)), dtype=torch.float64, device=cuda)
        plan.isai(LU, AIL, AIU)
        torch.cuda.synchronize()
    with bilu.Plan(rp, ci, reduction=bilu.REDUCE_FAST, factor_precision=bilu.FP32, **opts) as plan:
        fast_ms, _, cv_fast, _ = _time_ours(cuda, plan, V, B)
    assert np.all(cv_fast == 1)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).to(cuda)
    X = torch.zeros_like(B)
    it = torch.zeros(nsys, dtype=torch.float32, device=cuda)
    cv = torch.zeros(nsys, dtype=torch.int32, device=cuda)
    rs = torch.zeros(nsys, dtype=torch.float64, device=cuda)
    ref_ms = _time_ref(R.lib().ref_isai_solve, (n, nnz, nsys, T(rp), T(ci), V, B, X, len(aci), T(arp), T(aci), AIL,
                                                len(uci), T(urp), T(uci), AIU, it, cv, rs))
    H.assert_bitwise(it.cpu().numpy(), it_lib, "ILU-ISAI: iteration counts, library reference order vs reference")
    _report("ILU(0)-ISAI BiCGSTAB (reference: solver kernel only, factors given), 2d5_16x16", nsys, ref_ms,
            [("reference order, factors included", ref_order_ms), ("FAST order, FP32 ISAI, factors included",
                                                                   fast_ms)])
    assert ref_order_ms < ref_ms and fast_ms < ref_ms
