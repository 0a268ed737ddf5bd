"""The benchmark configurations at their full sizes on the GPU, through the
autotuned plans the benchmark uses: every system converges, the true residual
of every system stays within a small factor of the relative tolerance, x is
finite, and 32 systems sampled across the batch equal the oracle's FAST-order
restatement bit for bit (systems are independent, so the oracle on the sample
alone gives the same bits as inside the full batch)."""
import numpy as np
import pytest

import bilu
import helpers as H

pytestmark = pytest.mark.gpu

TOL = dict(tol_mode=bilu.TOL_REL, tol=1e-10)
CONFIGS = [
    # (name, generator kind and grid, systems, options)
    ("headline ParILU(5) + FP32 ISAI, 3D 10x10x10", (2, 10, 10, 10), 4096,
     dict(precond=bilu.PRECOND_PARILU0_ISAI, parilu_sweeps=5, factor_precision=bilu.FP32)),
    ("plain merged FP64 ILU(0), 2D 16x16", (1, 16, 16, 1), 16384, dict(precond=bilu.PRECOND_ILU0)),
    ("precision variant ILU(0) + FP32 ISAI, conv-diff 24x24", (4, 24, 24, 1), 32768,
     dict(precond=bilu.PRECOND_ILU0_ISAI, ilu_approach=3, factor_precision=bilu.FP32)),
    ("plain merged FP64 ILU(0), 3D 7x7x7", (5, 7, 7, 7), 16384, dict(precond=bilu.PRECOND_ILU0)),
]


@pytest.mark.parametrize("name,grid,nsys,opts", CONFIGS, ids=[c[0].split(",")[0].replace(" ", "_") for c in CONFIGS])
def test_full_size_batch(cuda, name, grid, nsys, opts):
    import torch
    kind, gx, gy, gz = grid
    rp, ci, v, b = bilu.gen_stencil(kind, gx, gy, gz, nsys, H.SEED)
    opts = dict(opts, reduction=bilu.REDUCE_FAST, **TOL)
    with bilu.Plan(rp, ci, **opts) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        X = torch.full_like(B, float("nan"))
        info = plan.autotune(V, B, torch.empty_like(B))
        it = torch.empty(nsys, dtype=torch.float32, device=cuda)
        cv = torch.empty(nsys, dtype=torch.int32, device=cuda)
        rs = torch.empty(nsys, dtype=torch.float64, device=cuda)
        tr = torch.empty(nsys, dtype=torch.float64, device=cuda)
        st = torch.empty(nsys, dtype=torch.int32, device=cuda)
        plan.solve(V, B, X, it, cv, rs, tr, st)
        torch.cuda.synchronize()
        x, iters, conv, res, true_res, status = (t.cpu().numpy() for t in (X, it, cv, rs, tr, st))
    bn = np.linalg.norm(b, axis=1)
    assert np.all(conv == 1) and np.all(status == bilu.SYS_CONVERGED), f"{name}: not every system converged"
    assert np.all(np.isfinite(x))
    assert np.all(res < 1e-10 * bn), f"{name}: recursive residual above the threshold"
    assert np.all(true_res < 1e-8 * bn), f"{name}: true residual {np.max(true_res / bn):.3g} of ||b||"
    sample = np.linspace(0, nsys - 1, 32).astype(np.int64)
    o = H.oracle_fast(rp, ci, v[sample], b[sample], opts["precond"], info["threads"],
                      opts.get("factor_precision", 0) == bilu.FP32, approach=opts.get("ilu_approach", 1),
                      sweeps=opts.get("parilu_sweeps", 5), **TOL)
    g = dict(x=x[sample], iters=iters[sample], conv=conv[sample], res=res[sample], true_res=true_res[sample],
             status=status[sample])
    for f in ("iters", "conv", "status", "res", "x", "true_res"):
        H.assert_bitwise(g[f], o[f], f"{name}, systems {sample[:3].tolist()}...: {f}")
