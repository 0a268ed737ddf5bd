"""GPU parity: the CUDA path, called through the C ABI, against the oracle.

In the reference operation order (BILU_REDUCE_REF) every output is compared
bit for bit: iteration counts, convergence flags, statuses, the solution,
the recursive residual norm and the true residual norm, for every
preconditioner family on small members of the benchmark workloads."""
import numpy as np
import pytest

import bilu
import helpers as H
import oracle as O

pytestmark = pytest.mark.gpu

NSYS = 24


def _compare(g, o, what, fields=("iters", "conv", "x", "res", "true_res")):
    for f in fields:
        H.assert_bitwise(g[f], o[f], f"{what}: {f}")
    np.testing.assert_array_equal(g["status"], o["status"], err_msg=f"{what}: status")


@pytest.mark.parametrize("family", ["2d5_8x8", "2d5_16x16", "3d7_5x5x5", "cd2d_12x12", "3d7_7x7x7"])
@pytest.mark.parametrize("approach", [1, 2, 3, 4])
def test_merged_ilu0_bitwise(cuda, family, approach):
    rp, ci, v, b = H.workload(family, NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0, approach=approach)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0, ilu_approach=approach)
    _compare(g, o, f"merged ILU(0) {family} approach {approach}")
    assert np.all(o["conv"] == 1)


@pytest.mark.parametrize("family", ["2d5_16x16", "3d7_5x5x5"])
@pytest.mark.parametrize("approach", [1, 3])
def test_split_ilu0_bitwise(cuda, family, approach):
    rp, ci, v, b = H.workload(family, NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0_SPLIT, approach=approach)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0_SPLIT, ilu_approach=approach)
    _compare(g, o, f"split ILU(0) {family} approach {approach}")


@pytest.mark.parametrize("family", ["2d5_16x16", "3d7_7x7x7"])
@pytest.mark.parametrize("sweeps", [0, 1, 5])
def test_parilu0_bitwise(cuda, family, sweeps):
    rp, ci, v, b = H.workload(family, NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_PARILU0, sweeps=sweeps)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_PARILU0, parilu_sweeps=sweeps)
    _compare(g, o, f"ParILU(0) {family} sweeps {sweeps}")


def _random_pattern_batch(nsys, seed=3):
    """A random pattern of the uneven generator (n in [200, 300]) shared by nsys systems whose off-diagonal
    values are those of the generated system times 1 + U(-0.05, 0.05): unlike the stencil families, many of
    its entries below the diagonal have ILU(0) dependency pairs."""
    sn, sz, rp, ci, v, b = bilu.gen_uneven(4, H.SEED, 200, 300, 5, 12)
    r, c, vv, bb = H.uneven_split(sn, sz, rp, ci, v, b)[0]
    r, c = np.ascontiguousarray(r - r[0], np.int32), np.ascontiguousarray(c, np.int32)
    rng = np.random.default_rng(seed)
    row = np.repeat(np.arange(len(r) - 1), np.diff(r))
    scale = np.where(c[None, :] == row[None, :], 1.0, 1.0 + 0.05 * rng.uniform(-1.0, 1.0, (nsys, len(c))))
    vals = np.ascontiguousarray(vv[None, :] * scale)
    bs = np.ascontiguousarray(np.repeat(bb[None, :], nsys, 0) * (1.0 + 0.1 * rng.uniform(-1.0, 1.0, (nsys, len(bb)))))
    low_with_pairs = 0
    cols = [set(c[r[i]:r[i + 1]].tolist()) for i in range(len(r) - 1)]
    for i in range(len(r) - 1):
        for j in c[r[i]:r[i + 1]]:
            if j < i and any(k < j and j in cols[k] for k in cols[i]):
                low_with_pairs += 1
    assert low_with_pairs > 50
    return r, c, vals, bs


@pytest.mark.parametrize("precond", [bilu.PRECOND_PARILU0, bilu.PRECOND_PARILU0_ISAI])
def test_parilu0_lower_entries_with_pairs_bitwise(cuda, precond):
    """ParILU sweeps (and ISAI on their factors) on a random pattern whose lower entries have dependency
    pairs, the kernel's own class of entries that no stencil family has, and whose ISAI rows differ in
    length (the ISAI kernels' row order): the reference order end to end."""
    rp, ci, v, b = _random_pattern_batch(NSYS)
    # ISAI on the factors' own pattern (power 1): |T|^2 rows of this pattern pass the 32-entry limit
    o = H.oracle_pipeline(rp, ci, v, b, precond, sweeps=5, isai_power=1)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, parilu_sweeps=5, isai_power=1)
    _compare(g, o, f"ParILU(0) random pattern precond {precond}")


@pytest.mark.parametrize("precond,fp32", [(bilu.PRECOND_PARILU0, False), (bilu.PRECOND_PARILU0, True),
                                          (bilu.PRECOND_PARILU0_ISAI, False), (bilu.PRECOND_PARILU0_ISAI, True)])
def test_parilu0_fast_lower_entries_with_pairs_bitwise(cuda, precond, fp32):
    """The FAST pipeline on the same random pattern (FAST ParILU sweeps with the diagonal reciprocal, FAST
    ISAI in FP64 or FP32, the register-resident FAST solve) bit for bit against the oracle's FAST order.
    (bilu_parilu0, the drop-in for the reference's factorisation, always runs the reference's division.)"""
    rp, ci, v, b = _random_pattern_batch(NSYS)
    tol = dict(tol_mode=bilu.TOL_REL, tol=1e-10)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, parilu_sweeps=5, isai_power=1, reduction=bilu.REDUCE_FAST,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, threads_per_system=128, **tol)
    assert g["info"]["solver_kernel"] == 1 and g["info"]["threads"] == 128
    o = H.oracle_fast(rp, ci, v, b, precond, 128, fp32, sweeps=5, power=1, **tol)
    for f in ("iters", "conv", "status", "res", "x", "true_res"):
        H.assert_bitwise(g[f], o[f], f"FAST random pattern precond {precond} fp32={fp32}: {f}")
    assert np.all(g["conv"] == 1)


@pytest.mark.parametrize("family", ["2d5_16x16", "3d7_5x5x5", "3d7_7x7x7"])
@pytest.mark.parametrize("precond", [bilu.PRECOND_ILU0_ISAI, bilu.PRECOND_PARILU0_ISAI])
def test_isai_bitwise(cuda, family, precond):
    rp, ci, v, b = H.workload(family, NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, precond, approach=3, sweeps=5)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, ilu_approach=3, parilu_sweeps=5)
    _compare(g, o, f"ISAI precond {precond} {family}")


@pytest.mark.parametrize("family", ["2d5_16x16", "3d7_5x5x5", "cd2d_12x12"])
@pytest.mark.parametrize("fp32", [False, True])
def test_general_isai_bitwise(cuda, family, fp32):
    rp, ci, v, b = H.workload(family, NSYS)
    kw = dict(tol_mode=1, tol=1e-10) if fp32 else {}
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_GENERAL_ISAI, fp32=fp32, **kw)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_GENERAL_ISAI,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, **kw)
    _compare(g, o, f"general ISAI {family} fp32={fp32}")
    assert np.all(g["conv"] == 1)


def test_general_isai_entry_point_bitwise(cuda):
    import torch
    rp, ci, v, b = H.workload("cd2d_12x12", NSYS)
    with bilu.Plan(rp, ci, precond=bilu.PRECOND_GENERAL_ISAI, isai_power=2) as plan:
        arp, aci = plan.pattern(1)
        orp, oci = O.isai_pattern(rp, ci, 2)
        np.testing.assert_array_equal(arp, orp)
        np.testing.assert_array_equal(aci, oci)
        V = torch.from_numpy(v).to(cuda)
        AI = torch.empty((NSYS, len(aci)), dtype=torch.float64, device=cuda)
        plan.isai(V, AI, None)
        torch.cuda.synchronize()
    H.assert_bitwise(AI.cpu().numpy(), O.isai_values(rp, ci, v, 2, orp, oci), "bilu_isai general")


@pytest.mark.parametrize("precond", [bilu.PRECOND_ILU0, bilu.PRECOND_PARILU0, bilu.PRECOND_PARILU0_ISAI])
def test_fp32_factors_bitwise(cuda, precond):
    rp, ci, v, b = H.workload("cd2d_12x12", NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, precond, fp32=True, tol_mode=1, tol=1e-10)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, factor_precision=bilu.FP32, tol_mode=1, tol=1e-10)
    _compare(g, o, f"FP32 factors precond {precond}")
    assert np.all(g["conv"] == 1)


@pytest.mark.parametrize("precond", [bilu.PRECOND_NONE])
def test_unpreconditioned_bitwise(cuda, precond):
    rp, ci, v, b = H.workload("2d5_8x8", NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, precond)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond)
    _compare(g, o, "no preconditioner")


@pytest.mark.parametrize("family,threads", [("3d7_7x7x7", 0), ("3d7_7x7x7", 128), ("3d7_7x7x7", 256),
                                            ("cd2d_24x24", 0), ("3d7_10x10x10", 0)],
                         ids=["7x7x7-2warps", "7x7x7-4warps", "7x7x7-8warps", "24x24-3warps", "10x10x10-4warps"])
@pytest.mark.parametrize("precond,fp32", [(bilu.PRECOND_ILU0, False), (bilu.PRECOND_ILU0, True),
                                          (bilu.PRECOND_NONE, False)], ids=["ilu0", "ilu0-fp32", "none"])
def test_reference_order_several_warps_bitwise(cuda, family, threads, precond, fp32):
    """The register-resident kernel in the reference order with several warps per system: each inner
    product chains through the warps (warp w holds a block of every lane's rows), so it equals the
    reference's warp-0 sum, and the true residual its serial sum, bit for bit."""
    nsys = 8
    rp, ci, v, b = H.workload(family, nsys)
    kw = dict(tol_mode=1, tol=1e-10) if fp32 else {}
    o = H.oracle_pipeline(rp, ci, v, b, precond, fp32=fp32, **kw)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, threads_per_system=threads,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, **kw)
    assert g["info"]["solver_kernel"] == 1
    if threads:
        assert g["info"]["threads"] == threads
    _compare(g, o, f"reference order {family} threads {g['info']['threads']} precond {precond} fp32={fp32}")
    assert np.all(g["conv"] == 1)


def test_relative_tolerance_bitwise(cuda):
    rp, ci, v, b = H.workload("2d5_16x16", NSYS)
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0, tol_mode=1, tol=1e-10)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0, tol_mode=bilu.TOL_REL, tol=1e-10)
    _compare(g, o, "relative tolerance")
    assert np.all(g["res"] < 1e-10 * np.linalg.norm(b, axis=1))


@pytest.mark.parametrize("precond", [bilu.PRECOND_ILU0, bilu.PRECOND_PARILU0, bilu.PRECOND_PARILU0_ISAI])
def test_fast_mode_properties(cuda, precond):
    """FAST order is not bit-comparable; it must converge to the same accuracy in about as many iterations."""
    rp, ci, v, b = H.workload("3d7_7x7x7", NSYS)
    ref = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, tol_mode=1, tol=1e-10)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, tol_mode=1, tol=1e-10, reduction=bilu.REDUCE_FAST)
    bn = np.linalg.norm(b, axis=1)
    assert np.all(g["conv"] == 1)
    assert np.all(np.abs(g["iters"] - ref["iters"]) <= 1.0)
    assert np.all(g["res"] < 1e-10 * bn)
    # true residual within a small factor of the recursive one (rounding drift)
    assert np.all(g["true_res"] < 1e-9 * bn)
    xd = O.dense_solve(rp, ci, v, b)
    assert np.max(np.abs(g["x"] - xd)) < 1e-8


# ---------------------------------------------------------------- separate entry points
def test_factorisation_entry_points_bitwise(cuda):
    import torch
    rp, ci, v, b = H.workload("3d7_5x5x5", NSYS)
    with bilu.Plan(rp, ci, precond=bilu.PRECOND_PARILU0_ISAI) as plan:
        V = torch.from_numpy(v).to(cuda)
        for approach in (1, 2, 3, 4):
            LU = torch.empty_like(V)
            plan.ilu0(V, LU, approach)
            H.assert_bitwise(LU.cpu().numpy(), O.ilu0(rp, ci, v, approach), f"bilu_ilu0 approach {approach}")
        for sweeps in (1, 3, 7):
            LU = torch.empty_like(V)
            plan.parilu0(V, LU, sweeps)
            H.assert_bitwise(LU.cpu().numpy(), O.parilu0(rp, ci, v, sweeps), f"bilu_parilu0 sweeps {sweeps}")
        lu = O.ilu0(rp, ci, v, 3)
        LU = torch.from_numpy(lu).to(cuda)
        Lr, Ur = O.split_values(rp, ci, lu)
        Lg = torch.empty((NSYS, Lr.shape[1]), dtype=torch.float64, device=cuda)
        Ug = torch.empty((NSYS, Ur.shape[1]), dtype=torch.float64, device=cuda)
        plan.split_lu(LU, Lg, Ug)
        H.assert_bitwise(Lg.cpu().numpy(), Lr, "bilu_split_lu L")
        H.assert_bitwise(Ug.cpu().numpy(), Ur, "bilu_split_lu U")
        lrp, lci, urp, uci = O.split_pattern(rp, ci)
        arp, aci = O.isai_pattern(lrp, lci, 2)
        brp, bci = O.isai_pattern(urp, uci, 2)
        grp, gci = plan.pattern(1)
        np.testing.assert_array_equal(grp, arp)
        np.testing.assert_array_equal(gci, aci)
        grp, gci = plan.pattern(2)
        np.testing.assert_array_equal(grp, brp)
        np.testing.assert_array_equal(gci, bci)
        AIL = torch.empty((NSYS, len(aci)), dtype=torch.float64, device=cuda)
        AIU = torch.empty((NSYS, len(bci)), dtype=torch.float64, device=cuda)
        plan.isai(LU, AIL, AIU)
        H.assert_bitwise(AIL.cpu().numpy(), O.isai_values(lrp, lci, Lr, 0, arp, aci), "bilu_isai aiL")
        H.assert_bitwise(AIU.cpu().numpy(), O.isai_values(urp, uci, Ur, 1, brp, bci), "bilu_isai aiU")
        X = torch.from_numpy(np.random.default_rng(1).standard_normal(b.shape)).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        out = torch.empty(NSYS, dtype=torch.float64, device=cuda)
        plan.true_residual(V, B, X, out)
        H.assert_bitwise(out.cpu().numpy(), O.true_residual(rp, ci, v, b, X.cpu().numpy()), "bilu_true_residual")


# ---------------------------------------------------------------- edge cases
def test_zero_and_tiny_rhs(cuda):
    rp, ci, v, b = H.workload("2d5_8x8", 6)
    b[1] = 0.0           # x = 0 without iterating (reference: "RHS ... is 0")
    b[3] *= 1e-14        # initial residual already below ATOL
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0)
    _compare(g, o, "zero / tiny rhs")
    assert g["status"][1] == bilu.SYS_ZERO_RHS and g["iters"][1] == 0 and np.all(g["x"][1] == 0)
    assert g["status"][3] == bilu.SYS_INITIAL_OK and g["iters"][3] == 0


@pytest.mark.parametrize("max_iter", [0, 1, 3])
def test_iteration_cap(cuda, max_iter):
    rp, ci, v, b = H.workload("3d7_5x5x5", 8)
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_NONE, max_iter=max_iter)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_NONE, max_iter=max_iter)
    _compare(g, o, f"max_iter {max_iter}")
    assert np.all(g["conv"] == -1) and np.all(g["status"] == bilu.SYS_MAX_ITER)
    assert np.all(g["iters"] == max_iter)


def test_missing_diagonal_split_path(cuda):
    rp, ci, v, b = H.workload("2d5_8x8", NSYS)
    # drop the diagonal of rows 5 and 40 from the pattern (values follow), make rows still solvable
    keep = np.ones(len(ci), bool)
    for row in (5, 40):
        k = rp[row] + int(np.where(ci[rp[row]:rp[row + 1]] == row)[0][0])
        keep[k] = False
    nrp = np.concatenate([[0], np.cumsum([keep[rp[i]:rp[i + 1]].sum() for i in range(len(rp) - 1)])]).astype(np.int32)
    nci = ci[keep]
    nv = np.ascontiguousarray(v[:, keep])
    # exact ILU(0) gives the inserted zero diagonals nonzero pivots through the updates of earlier rows
    g = H.gpu_solve(cuda, nrp, nci, nv, b, precond=bilu.PRECOND_ILU0_SPLIT, max_iter=20)
    o = H.oracle_pipeline(nrp, nci, nv, b, bilu.PRECOND_ILU0_SPLIT, max_iter=20)
    _compare(g, o, "missing diagonals (split ILU path)")
    assert g["info"]["missing_diag"] == 2
    with pytest.raises(bilu.BiluError) as e:
        bilu.Plan(nrp, nci, precond=bilu.PRECOND_ILU0)
    assert e.value.code == bilu.ERR_PATTERN


def test_isai_row_limit(cuda):
    # dense lower band: |L|^2 rows exceed the 32-entry limit of the ISAI row solve
    n = 48
    rows = [list(range(max(0, i - 20), min(n, i + 2))) for i in range(n)]
    rp = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    ci = np.concatenate(rows).astype(np.int32)
    with pytest.raises(bilu.BiluError) as e:
        bilu.Plan(rp, ci, precond=bilu.PRECOND_ILU0_ISAI)
    assert e.value.code == bilu.ERR_CAPACITY


def test_empty_batch(cuda):
    import torch
    rp, ci, v, b = H.workload("2d5_8x8", 1)
    with bilu.Plan(rp, ci) as plan:
        z = torch.empty((0, len(ci)), dtype=torch.float64, device=cuda)
        zb = torch.empty((0, 64), dtype=torch.float64, device=cuda)
        plan.solve(z, zb, zb.clone())
        torch.cuda.synchronize()


def test_nonfinite_status(cuda):
    rp, ci, v, b = H.workload("2d5_8x8", 4)
    v[2, :] = np.nan
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0, max_iter=50)
    assert g["conv"][2] == -1 and g["status"][2] == bilu.SYS_NONFINITE
    assert np.all(g["conv"][[0, 1, 3]] == 1)


# ---------------------------------------------------------------- forward error
@pytest.mark.parametrize("family", ["2d5_8x8", "cd2d_12x12", "3d7_5x5x5"])
def test_dense_lu_bitwise_and_forward_error(cuda, family):
    import torch
    rp, ci, v, b = H.workload(family, 16)
    ids = np.array([0, 3, 7, 15], np.int32)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0, tol_mode=bilu.TOL_REL, tol=1e-10)
    with bilu.Plan(rp, ci) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        X = torch.from_numpy(g["x"]).to(cuda)
        XD = torch.empty((len(ids), b.shape[1]), dtype=torch.float64, device=cuda)
        fe = plan.forward_error(V, B, X, ids, x_dense=XD)
        torch.cuda.synchronize()
    xd = O.dense_solve(rp, ci, v, b, ids)
    H.assert_bitwise(XD.cpu().numpy(), xd, f"GPU dense LU vs oracle {family}")
    ref = np.linalg.norm(g["x"][ids] - xd, axis=1) / np.linalg.norm(xd, axis=1)
    np.testing.assert_allclose(fe, ref, rtol=1e-12, atol=1e-30)
    assert np.all(fe < 1e-8)


def test_fp64_rate_probe(cuda):
    """bilu_probe_fp64_rate, the FP64 roofline's peak in the benchmark: a positive DFMA rate below the
    part's nominal FP64 figure (2 lane-FMAs per clock per SM), with the SM clock it ran at."""
    import torch
    gflops, mhz = bilu.probe_fp64_rate()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert 100.0 < mhz < 4000.0
    assert 0.0 < gflops <= 2 * 2 * sms * mhz * 1e-3 * 1.02



def test_integer_fp_matches_hardware(cuda):
    """The FP32 preconditioner paths round and widen with integer operations, and the FAST ParILU / ISAI take
    the correctly rounded reciprocal of the diagonal by integer Newton-Raphson (k_intfp.cuh), leaving the
    special cases to the hardware: every bit equal to the hardware conversions and to __drcp_rn on about 160
    million patterns of each kind (random doubles, every float exponent boundary with rounding ties, random
    floats, doubles with short, long and zero mantissas)."""
    assert bilu.check_integer_fp(1024, seed=7) == (0, 0, 0)
