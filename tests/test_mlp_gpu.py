"""Learned ParILU(0) warm start: the GPU features, forward pass and gradients
against the oracle, training, the ILU-residual gate with its fallback, and
what the trained network saves over the plain A-value initialisation."""
import numpy as np
import pytest

import bilu
import helpers as H
import oracle as O

pytestmark = pytest.mark.gpu


def _setup(cuda, nsys, seed=H.SEED):
    import torch
    rp, ci, v, b = bilu.gen_stencil(5, 7, 7, 7, nsys, seed)
    plan = bilu.Plan(rp, ci, precond=bilu.PRECOND_PARILU0)
    V = torch.from_numpy(v).to(cuda)
    LU = torch.empty_like(V)
    plan.parilu0(V, LU, 40)  # converged ParILU(0) factors: the training targets
    torch.cuda.synchronize()
    return rp, ci, v, b, plan, V, LU


def test_features_and_forward_match_oracle(cuda):
    rp, ci, v, b, plan, V, LU = _setup(cuda, 8)
    rng = np.random.default_rng(3)
    idx = rng.integers(0, v.size, 500).astype(np.int32)
    with bilu.Mlp(seed=7) as m:
        feat, out, base = m.eval(plan, V, idx)
        of, ob = O.mlp_features(rp, ci, v, idx)
        H.assert_bitwise(feat, of, "features")
        H.assert_bitwise(base, ob, "first-order estimates")
        y = np.zeros(len(idx), np.float32)
        _, _, oo = O.mlp_loss_grad(m.params(), of, y)
        np.testing.assert_allclose(out, oo, rtol=1e-4, atol=1e-5)
    plan.close()


def test_gradient_matches_oracle(cuda):
    rp, ci, v, b, plan, V, LU = _setup(cuda, 8)
    rng = np.random.default_rng(4)
    idx = rng.integers(0, v.size, 1000).astype(np.int32)
    with bilu.Mlp(seed=11) as m:
        m.train(plan, V, LU, 20, 512, 3e-3, seed=1)  # move away from the initialisation
        loss, grad = m.loss_grad(plan, V, LU, idx)
        feat, base = O.mlp_features(rp, ci, v, idx)
        lut = LU.cpu().numpy().reshape(-1)[idx]
        a = v.reshape(-1)[idx]
        y = (lut / (a * base) - 1.0).astype(np.float32)
        oloss, ograd, _ = O.mlp_loss_grad(m.params(), feat, y)
    assert abs(loss - oloss) <= 1e-3 * abs(oloss) + 1e-9
    assert np.linalg.norm(grad - ograd) <= 2e-3 * np.linalg.norm(ograd)
    plan.close()


def test_tensor_core_inference_matches_oracle(cuda):
    """The warm start's predictions (64x64 layer on tcgen05.mma with TMEM accumulators, hardware tanh)
    against the oracle's FP64 forward pass on the same BF16 weights; no system fell back for lack of a
    completed tensor-core round (ILU residual -1)."""
    import torch
    rp, ci, v, b, plan, V, LU = _setup(cuda, 12)
    with bilu.Mlp(seed=21) as m:
        m.train(plan, V, LU, 50, 2048, 3e-3, seed=2)
        LU0 = torch.empty_like(V)
        res = torch.empty(V.shape[0], dtype=torch.float64, device=cuda)
        m.warm_start(plan, V, LU0, 1e30, res)  # accept everything
        LU1 = torch.full_like(V, float("nan"))
        m.warm_start(plan, V, LU1, 1e30)  # a second call gives the same bits
        torch.cuda.synchronize()
        params = m.params()
    got = LU0.cpu().numpy()
    assert np.all(res.cpu().numpy() >= 0.0)
    H.assert_bitwise(LU1.cpu().numpy(), got, "repeated warm start")
    d = O.find_diag(rp, ci)
    n = len(rp) - 1
    deps = O.parilu0(rp, ci, v[:1], 0)  # shape only
    idx = []
    for s in range(v.shape[0]):
        for i in range(n):
            for k in range(rp[i], rp[i + 1]):
                if ci[k] < i:
                    idx.append(s * len(ci) + k)
    idx = np.array(idx, np.int32)
    feat, base = O.mlp_features(rp, ci, v, idx)
    _, _, out = O.mlp_loss_grad(params, feat, np.zeros(len(idx), np.float32))
    want = v.reshape(-1)[idx] * base * (1.0 + out)
    np.testing.assert_allclose(got.reshape(-1)[idx], want, rtol=2e-4)
    assert deps.shape == v[:1].shape
    plan.close()


def test_training_and_warm_start_gain(cuda, tmp_path):
    import torch
    rp, ci, v, b, plan, V, LU = _setup(cuda, 4096)
    with bilu.Mlp(seed=3) as m:
        losses = m.train(plan, V, LU, 1500, 16384, 2e-3, seed=5)
        assert losses[-20:].mean() < 0.05 * losses[:5].mean()
        path = str(tmp_path / "warm.bin")
        m.save(path)
        # fresh systems
        rp2, ci2, v2, b2 = bilu.gen_stencil(5, 7, 7, 7, 256, seed=999)
        V2 = torch.from_numpy(v2).to(cuda)
        LU0 = torch.empty_like(V2)
        res = torch.empty(256, dtype=torch.float64, device=cuda)
        used = torch.empty(256, dtype=torch.int32, device=cuda)
        m.warm_start(plan, V2, LU0, 1e-3, res, used)
        with bilu.Mlp(seed=0) as m2:
            m2.load(path)
            LU0b = torch.empty_like(V2)
            m2.warm_start(plan, V2, LU0b, 1e-3)
            torch.cuda.synchronize()
            H.assert_bitwise(LU0b.cpu().numpy(), LU0.cpu().numpy(), "saved / loaded model")
    u = used.cpu().numpy()
    r = res.cpu().numpy()
    assert u.mean() > 0.9, f"warm start accepted for only {u.mean():.2f} of the systems (median residual {np.median(r)})"
    # sweeps to ILU residual 1e-6: warm vs plain start
    sw_cold = torch.empty(256, dtype=torch.int32, device=cuda)
    sw_warm = torch.empty(256, dtype=torch.int32, device=cuda)
    with bilu.Plan(rp2, ci2, precond=bilu.PRECOND_PARILU0, parilu_sweeps=40, parilu_res_tol=1e-6,
                   tol_mode=bilu.TOL_REL, tol=1e-10) as p2:
        B2 = torch.from_numpy(b2).to(cuda)
        X = torch.empty_like(B2)
        it = torch.empty(256, dtype=torch.float32, device=cuda)
        cv = torch.empty(256, dtype=torch.int32, device=cuda)
        p2.solve(V2, B2, X, it, cv, sweeps=sw_cold)
        p2.solve(V2, B2, X, it, cv, sweeps=sw_warm, lu_init=LU0)
        torch.cuda.synchronize()
        assert np.all(cv.cpu().numpy() == 1)
    c, w = sw_cold.cpu().numpy(), sw_warm.cpu().numpy()
    print(f"sweeps to ILU residual 1e-6: plain {c.mean():.2f}, learned warm start {w.mean():.2f}")
    assert w.mean() < c.mean()
    plan.close()


def test_fallback_writes_a_values(cuda):
    import torch
    rp, ci, v, b, plan, V, LU = _setup(cuda, 16)
    with bilu.Mlp(seed=1) as m:
        LU0 = torch.empty_like(V)
        used = torch.empty(16, dtype=torch.int32, device=cuda)
        m.warm_start(plan, V, LU0, 1e-12, None, used)  # unattainable threshold: every system falls back
        torch.cuda.synchronize()
    assert np.all(used.cpu().numpy() == 0)
    H.assert_bitwise(LU0.cpu().numpy(), v, "fallback = A values")
    plan.close()


def test_adaptive_parilu_reports_residual(cuda):
    import torch
    rp, ci, v, b = H.workload("3d7_5x5x5", 8)
    with bilu.Plan(rp, ci, precond=bilu.PRECOND_PARILU0, parilu_sweeps=30, parilu_res_tol=1e-8) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        X = torch.empty_like(B)
        sw = torch.empty(8, dtype=torch.int32, device=cuda)
        rr = torch.empty(8, dtype=torch.float64, device=cuda)
        plan.solve(V, B, X, sweeps=sw, ilu_res=rr)
        torch.cuda.synchronize()
    s, r = sw.cpu().numpy(), rr.cpu().numpy()
    assert np.all(r <= 1e-8) and np.all(s > 0) and np.all(s < 30)
    # the residual the kernel reports for the last iterate equals the oracle's ILU residual of the
    # factors after the same number of Jacobi sweeps
    for k in range(8):
        lu = O.parilu0(rp, ci, v[k:k + 1], int(s[k]))
        np.testing.assert_allclose(r[k], O.ilu_residual(rp, ci, v[k:k + 1], lu)[0], rtol=1e-6)
