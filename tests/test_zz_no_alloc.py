"""bilu_solve_noalloc: the solve for callers that cannot allocate device memory
(for example a simulation's time-step loop that fixes its GPU memory at
start-up; cudaMalloc would also synchronise the device mid-step).

It runs bilu_solve's own scratch layout and launches (SELL-32 operand copies
and the autotuner's kernel variant included) with its scratch in one fixed
32 MiB device array.  This file is collected last so that a run stopping at the first
failure has already run every other test; it also passes on its own in a
fresh process."""
import numpy as np
import pytest

import bilu
import helpers as H

pytestmark = pytest.mark.gpu

FIELDS = ("x", "iters", "conv", "res", "true_res", "status")


def _buffers(torch, dev, nsys, n):
    return (torch.empty((nsys, n), dtype=torch.float64, device=dev),
            torch.empty(nsys, dtype=torch.float32, device=dev), torch.empty(nsys, dtype=torch.int32, device=dev),
            torch.empty(nsys, dtype=torch.float64, device=dev), torch.empty(nsys, dtype=torch.float64, device=dev),
            torch.empty(nsys, dtype=torch.int32, device=dev))


def _host(bufs):
    return {k: t.cpu().numpy() for k, t in zip(FIELDS, bufs)}


@pytest.mark.parametrize("family,opts", [
    ("3d7_5x5x5", dict(precond=bilu.PRECOND_PARILU0_ISAI, parilu_sweeps=5)),
    ("2d5_16x16", dict(precond=bilu.PRECOND_ILU0_SPLIT, ilu_approach=1)),
    ("cd2d_12x12", dict(precond=bilu.PRECOND_PARILU0, factor_precision=bilu.FP32, tol_mode=bilu.TOL_REL,
                        tol=1e-10)),
    ("cd2d_12x12", dict(precond=bilu.PRECOND_GENERAL_ISAI, isai_power=2)),
    # ILU factors at n = 1000 in FAST order: the register-resident solver reads a SELL-32 copy of A by default
    ("3d7_10x10x10", dict(precond=bilu.PRECOND_ILU0_SPLIT, ilu_approach=1, reduction=bilu.REDUCE_FAST,
                          tol_mode=bilu.TOL_REL, tol=1e-10)),
    ("3d7_10x10x10", dict(precond=bilu.PRECOND_PARILU0, reduction=bilu.REDUCE_FAST, factor_precision=bilu.FP32,
                          tol_mode=bilu.TOL_REL, tol=1e-10)),
    # the 4-CTA-per-SM kernel variant (staging bit 4) with FP32 ISAI
    ("3d7_7x7x7", dict(precond=bilu.PRECOND_PARILU0_ISAI, reduction=bilu.REDUCE_FAST, factor_precision=bilu.FP32,
                       smem_staging=16, tol_mode=bilu.TOL_REL, tol=1e-10)),
    # SELL-32 copies of A and aiU (staging bit 3) with FP64 ISAI
    ("3d7_7x7x7", dict(precond=bilu.PRECOND_PARILU0_ISAI, reduction=bilu.REDUCE_FAST, smem_staging=8,
                       tol_mode=bilu.TOL_REL, tol=1e-10)),
])
def test_noalloc_matches_bilu_solve_twice(cuda, family, opts):
    import torch
    rp, ci, v, b = H.workload(family, 16 if family == "3d7_10x10x10" else 32)
    nsys, n = b.shape
    with bilu.Plan(rp, ci, **opts) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        _matches_solve_twice(torch, cuda, plan, V, B, nsys, n)
        info = plan.info()
    if opts.get("reduction") == bilu.REDUCE_FAST and family == "3d7_10x10x10":
        assert info["operands_in_smem"] & 8, "the SELL-32 copy of A was not selected"
    if opts.get("smem_staging") == 16:
        assert info["operands_in_smem"] & 16, "the 4-CTA kernel variant was not selected"


def test_noalloc_matches_autotuned_headline_plan(cuda):
    """The headline configuration: ParILU(0) 5 sweeps + FP32 ISAI at n = 1000, the plan autotuned on the batch
    (threads, staging, SELL-32 copies, kernel variant), then bilu_solve and bilu_solve_noalloc on that plan."""
    import torch
    rp, ci, v, b = H.workload("3d7_10x10x10", 24)
    nsys, n = b.shape
    opts = dict(precond=bilu.PRECOND_PARILU0_ISAI, parilu_sweeps=5, reduction=bilu.REDUCE_FAST,
                factor_precision=bilu.FP32, tol_mode=bilu.TOL_REL, tol=1e-10)
    with bilu.Plan(rp, ci, **opts) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        plan.autotune(V, B, torch.empty_like(B))
        _matches_solve_twice(torch, cuda, plan, V, B, nsys, n)


def _matches_solve_twice(torch, cuda, plan, V, B, nsys, n):
    """bilu_solve once, then bilu_solve_noalloc twice in a row on the same plan: equal bit for bit."""
    ref = _buffers(torch, cuda, nsys, n)
    plan.solve(V, B, *ref)
    torch.cuda.synchronize()
    want = _host(ref)
    out = _buffers(torch, cuda, nsys, n)
    for call in range(2):  # two calls in a row: the shared scratch holds the previous call's values
        for t in out:
            t.fill_(-1)
        plan.solve_noalloc(V, B, *out)
        torch.cuda.synchronize()
        got = _host(out)
        for f in FIELDS:
            H.assert_bitwise(got[f], want[f], f"noalloc call {call}: {f}")
    assert np.all(want["conv"] == 1)


def test_noalloc_allocates_nothing(cuda):
    import torch
    rp, ci, v, b = H.workload("3d7_5x5x5", 16)
    with bilu.Plan(rp, ci, precond=bilu.PRECOND_PARILU0_ISAI) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        out = _buffers(torch, cuda, *b.shape)
        plan.solve_noalloc(V, B, *out)  # first call on the device: address look-up, module already loaded
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            plan.solve_noalloc(V, B, *out)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0


def test_noalloc_rejects_batches_beyond_its_scratch(cuda):
    import torch
    # n = 1000 ParILU + ISAI needs ~187 KB of scratch per system: 256 systems exceed 32 MiB
    rp, ci, v, b = bilu.gen_stencil(2, 10, 10, 10, 256)
    with bilu.Plan(rp, ci, precond=bilu.PRECOND_PARILU0_ISAI) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        out = _buffers(torch, cuda, *b.shape)
        with pytest.raises(bilu.BiluError) as e:
            plan.solve_noalloc(V, B, *out)
        assert e.value.code == bilu.ERR_CAPACITY
        assert "split the batch" in str(e.value)
