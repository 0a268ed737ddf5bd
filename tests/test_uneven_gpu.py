"""Uneven batches (own size and pattern per system): one graph-launched solve
of persistent, size-bucketed kernels, checked per system against the oracle
bit for bit in the reference operation order."""
import numpy as np
import pytest

import bilu
import helpers as H

pytestmark = pytest.mark.gpu


def _run(dev, plan, v, b, nsys):
    import torch
    V = torch.from_numpy(v).to(dev)
    B = torch.from_numpy(b).to(dev)
    X = torch.full_like(B, float("nan"))
    it = torch.full((nsys,), -7.0, dtype=torch.float32, device=dev)
    cv = torch.full((nsys,), 7, dtype=torch.int32, device=dev)
    rs = torch.full((nsys,), -1.0, dtype=torch.float64, device=dev)
    tr = torch.full((nsys,), -1.0, dtype=torch.float64, device=dev)
    st = torch.full((nsys,), 99, dtype=torch.int32, device=dev)
    plan.solve(V, B, X, it, cv, rs, tr, st)
    torch.cuda.synchronize()
    return {"x": X.cpu().numpy(), "iters": it.cpu().numpy(), "conv": cv.cpu().numpy(), "res": rs.cpu().numpy(),
            "true_res": tr.cpu().numpy(), "status": st.cpu().numpy()}, (V, B, X, it, cv, rs, tr, st)


def _cmp(g, o, what):
    for f in ("iters", "conv", "x", "res", "true_res", "status"):
        H.assert_bitwise(g[f], o[f], f"{what}: {f}")


@pytest.mark.parametrize("fp32", [False, True])
def test_uneven_ref_bitwise(cuda, fp32):
    sn, sz, rp, ci, v, b = bilu.gen_uneven(40, seed=11, nmin=16, nmax=300)
    kw = dict(tol_mode=bilu.TOL_REL, tol=1e-10) if fp32 else {}
    o = H.oracle_uneven(sn, sz, rp, ci, v, b, fp32=fp32, **({"tol_mode": 1, "tol": 1e-10} if fp32 else {}))
    with bilu.UnevenPlan(sn, sz, rp, ci, precond=bilu.PRECOND_ILU0,
                         factor_precision=bilu.FP32 if fp32 else bilu.FP64, **kw) as plan:
        g, _ = _run(cuda, plan, v, b, len(sn))
        info = plan.info()
    _cmp(g, o, f"uneven fp32={fp32}")
    assert sum(i["systems"] for i in info) == len(sn)
    assert sum(1 for i in info if i["systems"]) >= 2  # the batch spans several buckets
    assert np.all(g["conv"] == 1)


def test_uneven_autotune_keeps_bits_and_graph_replays(cuda):
    import torch
    sn, sz, rp, ci, v, b = bilu.gen_uneven(64, seed=5, nmin=16, nmax=600)
    o = H.oracle_uneven(sn, sz, rp, ci, v, b)
    with bilu.UnevenPlan(sn, sz, rp, ci) as plan:
        g1, bufs = _run(cuda, plan, v, b, len(sn))
        V, B, X = bufs[:3]
        plan.autotune(V, B, torch.empty_like(X))
        torch.cuda.synchronize()
        tuned = plan.info()
        g2, _ = _run(cuda, plan, v, b, len(sn))          # new buffers: graph re-captured
        X2 = torch.empty_like(X)
        plan.solve(V, B, X2, *bufs[3:])                   # another re-capture
        plan.solve(V, B, X2, *bufs[3:])                   # replay of the same graph
        torch.cuda.synchronize()
    _cmp(g1, o, "uneven untuned")
    _cmp(g2, o, "uneven autotuned")  # REF results do not depend on the CTA size
    H.assert_bitwise(X2.cpu().numpy(), o["x"], "graph replay")
    for i in tuned:
        if i["systems"]:
            assert i["threads"] in (64, 128, 256, 512, 1024) and i["grid"] > 0 and i["tuned_ms"] > 0


def test_uneven_fast_mode(cuda):
    sn, sz, rp, ci, v, b = bilu.gen_uneven(48, seed=9, nmin=64, nmax=1024)
    with bilu.UnevenPlan(sn, sz, rp, ci, tol_mode=bilu.TOL_REL, tol=1e-10, reduction=bilu.REDUCE_FAST) as plan:
        g, _ = _run(cuda, plan, v, b, len(sn))
    parts = H.uneven_split(sn, sz, rp, ci, v, b)
    bn = np.array([np.linalg.norm(p[3]) for p in parts])
    assert np.all(g["conv"] == 1)
    assert np.all(g["res"] < 1e-10 * bn)
    assert np.all(g["true_res"] < 1e-8 * bn)


def test_uneven_rejects_missing_diagonal(cuda):
    sn, sz, rp, ci, v, b = bilu.gen_uneven(3, seed=2, nmin=16, nmax=32)
    # drop the diagonal of row 0 of system 1
    parts = H.uneven_split(sn, sz, rp, ci, v, b)
    r, c = parts[1][0].copy(), parts[1][1].copy()
    k = int(np.where(c[r[0]:r[1]] == 0)[0][0])
    c2 = np.delete(c, k)
    r2 = r.copy()
    r2[1:] -= 1
    rp2 = np.concatenate([parts[0][0], r2, parts[2][0]])
    ci2 = np.concatenate([parts[0][1], c2, parts[2][1]])
    sz2 = sz.copy()
    sz2[1] -= 1
    with pytest.raises(bilu.BiluError) as e:
        bilu.UnevenPlan(sn, sz2, rp2, ci2)
    assert e.value.code == bilu.ERR_PATTERN
