"""The benchmark configurations at their full sizes on the GPU, through the
autotuned plans the benchmark uses: every system converges, the true residual
of every system stays within a small factor of the relative tolerance, x is
finite, and 32 systems sampled across the batch equal the oracle's FAST-order
restatement bit for bit (systems are independent, so the oracle on the sample
alone gives the same bits as inside the full batch). The uneven batch (8192
systems of their own sizes and patterns) is checked the same way, each sampled
system against the oracle at its bucket's threads per system."""
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


@pytest.mark.parametrize("fp32", [False, True])
def test_full_size_uneven_batch(cuda, fp32):
    """The uneven configuration at full size: 8192 systems with n log-uniform in [64, 1024] and their own
    random patterns, merged ILU(0), autotuned buckets, one graph launch; every system converges and 32 sampled
    systems equal the oracle's FAST order for their bucket's threads per system bit for bit."""
    import torch
    import oracle as O
    nsys = 8192
    sn, sz, rp, ci, v, b = bilu.gen_uneven(nsys, H.SEED, 64, 1024, 5, 12)
    with bilu.UnevenPlan(sn, sz, rp, ci, reduction=bilu.REDUCE_FAST, factor_precision=bilu.FP32 if fp32 else bilu.FP64,
                         **TOL) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        X = torch.full_like(B, float("nan"))
        plan.autotune(V, B, torch.empty_like(B))
        info = plan.info()
        out = [torch.empty(nsys, dtype=dt, device=cuda) for dt in (torch.float32, torch.int32, torch.float64,
                                                                    torch.float64, torch.int32)]
        plan.solve(V, B, X, *out)
        torch.cuda.synchronize()
        x = X.cpu().numpy()
        iters, conv, res, true_res, status = (t.cpu().numpy() for t in out)
    assert np.all(conv == 1) and np.all(np.isfinite(x))
    parts = H.uneven_split(sn, sz, rp, ci, v, b)
    offs = np.concatenate([[0], np.cumsum(sn)])
    for s in np.linspace(0, nsys - 1, 32).astype(np.int64):
        r, c, vv, bb = parts[s]
        n = int(sn[s])
        nt = next(i["threads"] for i in info if i["n_lo"] < n <= i["n_hi"])
        lu = O.ilu0(r, c, vv[None, :], 1)
        o = O.bicgstab_fast(r, c, vv[None, :], bb[None, :], nt, pv=3, ail=(r, c, lu), fp32=fp32, **TOL)
        H.assert_bitwise(x[offs[s]:offs[s + 1]], o["x"][0], f"uneven system {s}: x")
        for f, g in (("iters", iters), ("conv", conv), ("res", res), ("true_res", true_res), ("status", status)):
            H.assert_bitwise(g[s], o[f][0], f"uneven system {s}: {f}")
