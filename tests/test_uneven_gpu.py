"""Uneven batches (own size and pattern per system): one graph-launched solve
of size-bucketed kernels, checked per system against the oracle bit for bit,
in the reference operation order (persistent shared-memory kernels) and in
FAST order (the register-resident solver with its bucket's threads per system,
one CTA per system or persistent over the bucket's work queue)."""
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


def _oracle_uneven_fast(sn, sz, rp, ci, v, b, info, fp32, precond=bilu.PRECOND_ILU0, **tol):
    """orc_bicgstab_fast per system with its bucket's threads per system (merged ILU(0), approach 1)."""
    import oracle as O
    out = {f: [] for f in ("x", "iters", "conv", "res", "true_res", "status")}
    for s, (r, c, vv, bb) in enumerate(H.uneven_split(sn, sz, rp, ci, v, b)):
        n = int(sn[s])
        nt = next(i["threads"] for i in info if i["n_lo"] < n <= i["n_hi"])
        if precond == bilu.PRECOND_NONE:
            o = O.bicgstab_fast(r, c, vv[None, :], bb[None, :], nt, pv=0, **tol)
        else:
            lu = O.ilu0(r, c, vv[None, :], 1)
            o = O.bicgstab_fast(r, c, vv[None, :], bb[None, :], nt, pv=3, ail=(r, c, lu), fp32=fp32, **tol)
        for f in out:
            out[f].append(o[f][0])
    return {"x": np.concatenate(out["x"]), "iters": np.array(out["iters"], np.float32),
            "conv": np.array(out["conv"], np.int32), "res": np.array(out["res"]),
            "true_res": np.array(out["true_res"]), "status": np.array(out["status"], np.int32)}


@pytest.mark.parametrize("fp32", [False, True])
def test_uneven_fast_bitwise(cuda, fp32):
    """FAST order: every bucket with n <= 1024 runs the register-resident solver; bit for bit against the
    oracle's restatement of its order, before and after autotuning (which changes threads per system)."""
    import torch
    sn, sz, rp, ci, v, b = bilu.gen_uneven(48, seed=9, nmin=16, nmax=1024)
    tol = dict(tol_mode=bilu.TOL_REL, tol=1e-10)
    with bilu.UnevenPlan(sn, sz, rp, ci, reduction=bilu.REDUCE_FAST,
                         factor_precision=bilu.FP32 if fp32 else bilu.FP64, **tol) as plan:
        g, bufs = _run(cuda, plan, v, b, len(sn))
        info = plan.info()
        assert sum(1 for i in info if i["systems"]) >= 3
        _cmp(g, _oracle_uneven_fast(sn, sz, rp, ci, v, b, info, fp32, **tol), f"uneven FAST fp32={fp32}")
        V, B, X = bufs[:3]
        plan.autotune(V, B, torch.empty_like(X))
        torch.cuda.synchronize()
        g2, _ = _run(cuda, plan, v, b, len(sn))
        info2 = plan.info()
        _cmp(g2, _oracle_uneven_fast(sn, sz, rp, ci, v, b, info2, fp32, **tol), f"uneven FAST autotuned fp32={fp32}")
    parts = H.uneven_split(sn, sz, rp, ci, v, b)
    bn = np.array([np.linalg.norm(p[3]) for p in parts])
    assert np.all(g["conv"] == 1)
    assert np.all(g["res"] < 1e-10 * bn)
    assert np.all(g["true_res"] < 1e-8 * bn)


@pytest.mark.parametrize("fp32", [False, True])
def test_uneven_fast_persistent_queue_bitwise(cuda, fp32):
    """Register-resident buckets as persistent grids over their work queues (bilu_uneven_set_config with 1 to
    3 CTAs, so every CTA takes several systems from the queue) give the same bits as the oracle; a second
    solve on the same buffers replays the captured graph, whose queue heads it zeroes itself."""
    import torch
    sn, sz, rp, ci, v, b = bilu.gen_uneven(40, seed=13, nmin=16, nmax=700)
    tol = dict(tol_mode=bilu.TOL_REL, tol=1e-10)
    with bilu.UnevenPlan(sn, sz, rp, ci, reduction=bilu.REDUCE_FAST,
                         factor_precision=bilu.FP32 if fp32 else bilu.FP64, **tol) as plan:
        for k, i in enumerate(plan.info()):
            if i["systems"] > 1:
                plan.set_config(k, 0, 1 + k % 3)
        info = plan.info()
        assert any(0 < i["grid"] < i["systems"] for i in info)
        g, bufs = _run(cuda, plan, v, b, len(sn))
        V, B, X, it, cv, rs, tr, st = bufs
        for t, fill in ((X, float("nan")), (it, -7.0), (cv, 7), (rs, -1.0), (tr, -1.0), (st, 99)):
            t.fill_(fill)
        plan.solve(V, B, X, it, cv, rs, tr, st)
        torch.cuda.synchronize()
        g2 = {"x": X.cpu().numpy(), "iters": it.cpu().numpy(), "conv": cv.cpu().numpy(), "res": rs.cpu().numpy(),
              "true_res": tr.cpu().numpy(), "status": st.cpu().numpy()}
    want = _oracle_uneven_fast(sn, sz, rp, ci, v, b, info, fp32, **tol)
    _cmp(g, want, f"uneven FAST persistent fp32={fp32}")
    _cmp(g2, want, f"uneven FAST persistent replay fp32={fp32}")
    assert np.all(g["conv"] == 1)


def test_uneven_set_config_rejects_bad_configurations(cuda):
    """bilu_uneven_set_config: buckets out of range, negative sizes and CTA sizes the register-resident solver
    cannot take (more than 8 rows per thread, not a multiple of 32) are errors that leave the plan usable."""
    sn, sz, rp, ci, v, b = bilu.gen_uneven(24, seed=3, nmin=16, nmax=1000)
    with bilu.UnevenPlan(sn, sz, rp, ci, reduction=bilu.REDUCE_FAST, tol_mode=bilu.TOL_REL, tol=1e-10) as plan:
        info = plan.info()
        k = max(i for i, x in enumerate(info) if x["systems"])
        bad = [(len(info), 0, 0), (-1, 0, 0), (k, -32, 0), (k, 0, -1), (k, 33, 0)]
        if info[k]["n_lo"] >= 256:
            bad.append((k, 32, 0))  # more than 8 rows per thread
        for args in bad:
            with pytest.raises(bilu.BiluError) as e:
                plan.set_config(*args)
            assert e.value.code == bilu.ERR_INVALID, args
        g, _ = _run(cuda, plan, v, b, len(sn))
        assert np.all(g["conv"] == 1)


def test_uneven_fast_unpreconditioned_bitwise(cuda):
    sn, sz, rp, ci, v, b = bilu.gen_uneven(24, seed=4, nmin=16, nmax=400)
    tol = dict(tol_mode=bilu.TOL_ABS, tol=1e-11, max_iter=60)
    with bilu.UnevenPlan(sn, sz, rp, ci, precond=bilu.PRECOND_NONE, reduction=bilu.REDUCE_FAST, **tol) as plan:
        g, _ = _run(cuda, plan, v, b, len(sn))
        info = plan.info()
    _cmp(g, _oracle_uneven_fast(sn, sz, rp, ci, v, b, info, False, precond=bilu.PRECOND_NONE, **tol),
         "uneven FAST, no preconditioner")


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
