"""The register-resident FAST solver (csrc/k_solve_rr.cu) against the oracle's
restatement of its reduction order (orc_bicgstab_fast), bit for bit: ISAI of
L and U (exact ILU or FAST ParILU factors), general ISAI, in-place ILU factors
(the merged form factorising in the kernel, split ILU(0) approaches and FAST
ParILU) and no preconditioner; FP64 and FP32 preconditioner values; several
threads-per-system choices (1 to 8 rows per thread); edge cases with their
status words."""
import numpy as np
import pytest

import bilu
import helpers as H
import oracle as O

pytestmark = pytest.mark.gpu
NSYS = 10
TOL = dict(tol_mode=bilu.TOL_REL, tol=1e-10)


_oracle_fast = H.oracle_fast


def _check(g, o, what, fields=("iters", "conv", "status", "res", "x", "true_res")):
    assert g["info"]["solver_kernel"] == 1, f"{what}: the register-resident kernel was not selected"
    for f in fields:
        H.assert_bitwise(g[f], o[f], f"{what}: {f}")


CASES = [
    ("2d5_16x16", bilu.PRECOND_ILU0_ISAI, dict(ilu_approach=3)),
    ("3d7_7x7x7", bilu.PRECOND_PARILU0_ISAI, dict(parilu_sweeps=5)),
    ("cd2d_12x12", bilu.PRECOND_GENERAL_ISAI, dict(isai_power=1)),
    ("3d7_5x5x5", bilu.PRECOND_GENERAL_ISAI, dict(isai_power=2)),
    ("2d5_8x8", bilu.PRECOND_NONE, {}),
]


@pytest.mark.parametrize("fam,precond,kw", CASES, ids=[f"{c[0]}-p{c[1]}" for c in CASES])
@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("nt", [0, 64, 128])
def test_rr_solver_bitwise(cuda, fam, precond, kw, fp32, nt):
    if precond == bilu.PRECOND_NONE and fp32:
        pytest.skip("no preconditioner values to round")
    rp, ci, v, b = H.workload(fam, NSYS)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, reduction=bilu.REDUCE_FAST,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, threads_per_system=nt, **kw, **TOL)
    used = g["info"]["threads"]
    if nt:
        assert used == nt
    o = _oracle_fast(rp, ci, v, b, precond, used, fp32, approach=kw.get("ilu_approach", 3),
                     sweeps=kw.get("parilu_sweeps", 5), power=kw.get("isai_power", 2), **TOL)
    _check(g, o, f"{fam} precond {precond} fp32={fp32} threads={used}")
    assert np.all(g["conv"] == 1)


def test_rr_large_system_eight_rows_per_thread(cuda):
    """n = 1000 (the benchmark's 3D 10x10x10 pattern): 128 threads, 8 rows each, FP32 ISAI."""
    rp, ci, v, b = bilu.gen_stencil(2, 10, 10, 10, 6, seed=11)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_PARILU0_ISAI, parilu_sweeps=5,
                    reduction=bilu.REDUCE_FAST, factor_precision=bilu.FP32, **TOL)
    assert g["info"]["threads"] == 128
    o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_PARILU0_ISAI, 128, True, **TOL)
    _check(g, o, "3D 10x10x10 ParILU+ISAI FP32")


HEADLINE_OPTS = dict(precond=bilu.PRECOND_PARILU0_ISAI, parilu_sweeps=5, isai_power=2, reduction=bilu.REDUCE_FAST,
                     factor_precision=bilu.FP32, max_iter=500, **TOL)


@pytest.mark.parametrize("threads,staging", [(128, 16), (128, 6), (128, 0), (256, 16)])
def test_headline_configuration_bitwise(cuda, threads, staging):
    """The benchmark's headline path (PrecondBiCGSTAB_ilu_isai_gpu.cu:267-339: ParILU, ISAI of L and U, solver)
    on 16 systems of its 3D 7-point 10x10x10 pattern: ParILU(0) 5 sweeps (k_parilu0, FAST), ISAI computed in
    FP32 (k_isai_f32), then the solver.  256 threads with staging 16 is the configuration the autotuner picks
    for the 4096-system headline on GB300: the occupancy variant with 4 rows per thread
    (k_bicgstab_rr_occ<4, 1, float>, 4 CTAs of 256 threads per SM, 64 registers) with every operand read
    through L1.  With 128 threads (8 rows each): staging 16 runs k_bicgstab_rr_occ<8, 1, float> (4 CTAs, 128
    registers), 6 stages aiL and aiU in shared memory (3 CTAs per SM), 0 stages nothing.  x, iterations,
    status, both norms and the true residual equal the oracle's FAST order bit for bit."""
    rp, ci, v, b = H.workload("3d7_10x10x10", 16)
    g = H.gpu_solve(cuda, rp, ci, v, b, smem_staging=staging, threads_per_system=threads, **HEADLINE_OPTS)
    info = g["info"]
    assert info["threads"] == threads
    assert bool(info["operands_in_smem"] & 16) == (staging == 16), info
    o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_PARILU0_ISAI, threads, True, **TOL)
    _check(g, o, f"headline 3D 10x10x10 ParILU(5)+FP32 ISAI, {threads} threads, staging {staging}")
    assert np.all(g["conv"] == 1) and np.all(g["status"] == bilu.SYS_CONVERGED)


def test_headline_autotuned_plan_bitwise(cuda):
    """The headline plan as the benchmark uses it: bilu_plan_autotune on the batch, then solves with the same
    plan (whatever thread count, staging, SELL-32 copies or kernel variant it kept) equal the oracle."""
    import torch
    rp, ci, v, b = H.workload("3d7_10x10x10", 24)
    with bilu.Plan(rp, ci, **HEADLINE_OPTS) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        X = torch.empty_like(B)
        info = plan.autotune(V, B, X)
        assert info["solver_kernel"] == 1
        nsys, n = b.shape
        out = dict(x=torch.full_like(B, float("nan")), iters=torch.full((nsys,), -7.0, device=cuda),
                   conv=torch.full((nsys,), 7, dtype=torch.int32, device=cuda),
                   res=torch.full((nsys,), -1.0, dtype=torch.float64, device=cuda),
                   true_res=torch.full((nsys,), -1.0, dtype=torch.float64, device=cuda),
                   status=torch.full((nsys,), 99, dtype=torch.int32, device=cuda))
        plan.solve(V, B, out["x"], out["iters"], out["conv"], out["res"], out["true_res"], out["status"])
        torch.cuda.synchronize()
        g = {k: t.cpu().numpy() for k, t in out.items()}
        g["info"] = plan.info()
    o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_PARILU0_ISAI, info["threads"], True, **TOL)
    _check(g, o, f"autotuned headline plan (threads {info['threads']}, staging {info['operands_in_smem']})")


@pytest.mark.parametrize("nt,staging", [(96, 16), (96, 6), (192, -1), (384, -1)])
def test_cd2d_24x24_fp32_isai_bitwise(cuda, nt, staging):
    """The precision-variant workload: 2D 5-point 24x24 convection-diffusion (n = 576), ILU(0) approach 3 +
    ISAI of L and U computed, stored and applied in FP32, FAST order, at the autotuner's thread counts (96
    threads with 8 rows each, on the 4-CTA kernel or with the ISAI values staged; 192 and 384 threads)."""
    rp, ci, v, b = H.workload("cd2d_24x24", 8)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0_ISAI, ilu_approach=3, reduction=bilu.REDUCE_FAST,
                    factor_precision=bilu.FP32, threads_per_system=nt, smem_staging=staging, **TOL)
    assert g["info"]["threads"] == nt
    if staging == 16:
        assert g["info"]["operands_in_smem"] & 16
    o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_ILU0_ISAI, nt, True, approach=3, **TOL)
    _check(g, o, f"cd2d 24x24 ILU(0)+FP32 ISAI, {nt} threads, staging {staging}")
    assert np.all(g["conv"] == 1)


def test_rr_edge_cases(cuda):
    """Zero right-hand side, one already below the threshold, an iteration limit and a NaN in A."""
    rp, ci, v, b = H.workload("2d5_8x8", 6)
    b = b.copy()
    v = v.copy()
    b[1] = 0.0
    b[2] *= 1e-14           # below the absolute threshold from the start
    v[4, 3] = np.nan        # non-finite recurrences
    for max_iter in (500, 2):
        kw = dict(tol_mode=bilu.TOL_ABS, tol=1e-11, max_iter=max_iter)
        g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0_ISAI, ilu_approach=3,
                        reduction=bilu.REDUCE_FAST, **kw)
        o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_ILU0_ISAI, g["info"]["threads"], False, **kw)
        _check(g, o, f"edge cases, max_iter {max_iter}")
        assert g["status"][1] == 2 and g["status"][2] == 3 and g["status"][4] == -3
        if max_iter == 2:
            assert g["status"][0] == -1


def test_rr_matches_reference_order_in_iterations(cuda):
    """Same method as the reference-order kernel: iteration counts within one of it."""
    rp, ci, v, b = H.workload("3d7_7x7x7", NSYS)
    ref = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0_ISAI, ilu_approach=3, **TOL)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0_ISAI, ilu_approach=3,
                    reduction=bilu.REDUCE_FAST, **TOL)
    assert ref["info"]["solver_kernel"] == 0 and g["info"]["solver_kernel"] == 1
    assert np.all(np.abs(g["iters"] - ref["iters"]) <= 1.0)
    np.testing.assert_allclose(g["x"], ref["x"], rtol=0, atol=1e-8 * np.abs(ref["x"]).max())


def test_rr_autotuned_plan_bitwise(cuda):
    """bilu_plan_autotune picks threads per system and shared-memory staging; the solves that follow
    still equal the oracle's order for the chosen thread count."""
    import torch
    rp, ci, v, b = H.workload("3d7_7x7x7", 64)
    opts = dict(precond=bilu.PRECOND_PARILU0_ISAI, parilu_sweeps=5, reduction=bilu.REDUCE_FAST,
                factor_precision=bilu.FP32, **TOL)
    with bilu.Plan(rp, ci, **opts) as plan:
        V = torch.from_numpy(v).to(cuda)
        B = torch.from_numpy(b).to(cuda)
        X = torch.empty_like(B)
        info = plan.autotune(V, B, X)
        assert info["solver_kernel"] == 1 and info["threads"] in (64, 128, 256)
    g = H.gpu_solve(cuda, rp, ci, v, b, threads_per_system=info["threads"], **opts)
    o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_PARILU0_ISAI, info["threads"], True, **TOL)
    _check(g, o, f"autotuned threads {info['threads']}")


LU_CASES = [
    ("2d5_16x16", bilu.PRECOND_ILU0, dict(ilu_approach=1)),
    ("3d7_7x7x7", bilu.PRECOND_ILU0, dict(ilu_approach=4)),
    ("cd2d_12x12", bilu.PRECOND_ILU0, dict(ilu_approach=2)),
    ("3d7_5x5x5", bilu.PRECOND_ILU0, dict(ilu_approach=3)),
    ("cd2d_12x12", bilu.PRECOND_ILU0_SPLIT, dict(ilu_approach=3)),
    ("3d7_5x5x5", bilu.PRECOND_ILU0_SPLIT, dict(ilu_approach=2)),
    ("3d7_7x7x7", bilu.PRECOND_PARILU0, dict(parilu_sweeps=4)),
]


@pytest.mark.parametrize("fam,precond,kw", LU_CASES, ids=[f"{c[0]}-p{c[1]}-{list(c[2].values())[0]}" for c in LU_CASES])
@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("nt", [0, 64, 128])
def test_rr_lu_solver_bitwise(cuda, fam, precond, kw, fp32, nt):
    """In-place ILU factors in shared memory, level-scheduled triangular solves over the CTA."""
    rp, ci, v, b = H.workload(fam, NSYS)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, reduction=bilu.REDUCE_FAST,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, threads_per_system=nt, **kw, **TOL)
    used = g["info"]["threads"]
    if nt:
        assert used == nt
    o = _oracle_fast(rp, ci, v, b, precond, used, fp32, approach=kw.get("ilu_approach", 1),
                     sweeps=kw.get("parilu_sweeps", 5), **TOL)
    _check(g, o, f"{fam} precond {precond} fp32={fp32} threads={used}")
    assert np.all(g["conv"] == 1)


@pytest.mark.parametrize("fp32", [False, True])
def test_rr_lu_large_system(cuda, fp32):
    """n = 1000 (3D 10x10x10): the merged form factorises 6400 entries in shared memory, 128 threads with
    8 rows each; FP32 factors are rounded in place after the FP64 factorisation."""
    rp, ci, v, b = bilu.gen_stencil(2, 10, 10, 10, 6, seed=11)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0, reduction=bilu.REDUCE_FAST,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, **TOL)
    assert g["info"]["threads"] == 128
    o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_ILU0, 128, fp32, approach=1, **TOL)
    _check(g, o, f"3D 10x10x10 merged ILU(0) fp32={fp32}")


def test_rr_lu_missing_diagonal(cuda):
    """Split ILU(0) on a pattern without two diagonal entries: the factor pattern has them inserted, A*x
    keeps the caller's pattern."""
    rp, ci, v, b = H.workload("2d5_8x8", NSYS)
    keep = np.ones(len(ci), bool)
    for row in (5, 40):
        keep[rp[row] + int(np.where(ci[rp[row]:rp[row + 1]] == row)[0][0])] = False
    nrp = np.concatenate([[0], np.cumsum([keep[rp[i]:rp[i + 1]].sum() for i in range(len(rp) - 1)])]).astype(np.int32)
    nci = ci[keep]
    nv = np.ascontiguousarray(v[:, keep])
    kw = dict(tol_mode=bilu.TOL_ABS, tol=1e-11, max_iter=20)
    g = H.gpu_solve(cuda, nrp, nci, nv, b, precond=bilu.PRECOND_ILU0_SPLIT, reduction=bilu.REDUCE_FAST, **kw)
    assert g["info"]["missing_diag"] == 2
    o = _oracle_fast(nrp, nci, nv, b, bilu.PRECOND_ILU0_SPLIT, g["info"]["threads"], False, approach=1, **kw)
    _check(g, o, "missing diagonals, split ILU(0)")


def test_rr_lu_edge_cases(cuda):
    """Merged form: zero right-hand side, one below the threshold from the start, an iteration limit and a
    NaN in A (non-finite factors)."""
    rp, ci, v, b = H.workload("2d5_8x8", 6)
    b = b.copy()
    v = v.copy()
    b[1] = 0.0
    b[2] *= 1e-14
    v[4, 3] = np.nan
    for max_iter in (500, 2):
        kw = dict(tol_mode=bilu.TOL_ABS, tol=1e-11, max_iter=max_iter)
        g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0, reduction=bilu.REDUCE_FAST, **kw)
        o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_ILU0, g["info"]["threads"], False, approach=1, **kw)
        _check(g, o, f"LU edge cases, max_iter {max_iter}")
        assert g["status"][1] == 2 and g["status"][2] == 3 and g["status"][4] == -3
        if max_iter == 2:
            assert g["status"][0] == -1


@pytest.mark.parametrize("fam,precond,kw", [("3d7_7x7x7", bilu.PRECOND_PARILU0_ISAI, dict(parilu_sweeps=5)),
                                            ("cd2d_12x12", bilu.PRECOND_ILU0, dict(ilu_approach=1)),
                                            ("3d7_5x5x5", bilu.PRECOND_GENERAL_ISAI, dict(isai_power=2))],
                         ids=["parilu_isai", "merged_ilu0", "general_isai"])
@pytest.mark.parametrize("staging", [0, 8, 9, 14, 16, 26])
@pytest.mark.parametrize("fp32", [False, True])
def test_rr_operand_layouts_bitwise(cuda, fam, precond, kw, staging, fp32):
    """Shared-memory staging and the SELL-32 copies of A and aiU change where the SpMVs read their operands,
    never the arithmetic: every layout equals the oracle bit for bit."""
    rp, ci, v, b = H.workload(fam, NSYS)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, reduction=bilu.REDUCE_FAST, smem_staging=staging,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, **kw, **TOL)
    o = _oracle_fast(rp, ci, v, b, precond, g["info"]["threads"], fp32, approach=kw.get("ilu_approach", 1),
                     sweeps=kw.get("parilu_sweeps", 5), power=kw.get("isai_power", 2), **TOL)
    _check(g, o, f"{fam} precond {precond} staging {staging} fp32={fp32}")


@pytest.mark.parametrize("precond,kw", [(bilu.PRECOND_NONE, {}), (bilu.PRECOND_GENERAL_ISAI, dict(isai_power=1)),
                                       (bilu.PRECOND_PARILU0_ISAI, dict(parilu_sweeps=5))],
                         ids=["none", "general_isai", "parilu_isai"])
@pytest.mark.parametrize("fp32", [False, True])
def test_rr_four_ctas_per_sm_bitwise(cuda, precond, kw, fp32):
    """The 4-CTAs-per-SM kernel variant (staging bit 4; 8 rows per thread at n = 343) for every
    preconditioner kind it serves gives the oracle's FAST-order bits."""
    if precond == bilu.PRECOND_NONE and fp32:
        pytest.skip("no preconditioner values to round")
    rp, ci, v, b = H.workload("3d7_7x7x7", NSYS)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, reduction=bilu.REDUCE_FAST, smem_staging=16,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, **kw, **TOL)
    assert g["info"]["operands_in_smem"] & 16, "the 4-CTA variant was not selected"
    o = _oracle_fast(rp, ci, v, b, precond, g["info"]["threads"], fp32, sweeps=kw.get("parilu_sweeps", 5),
                     power=kw.get("isai_power", 2), **TOL)
    _check(g, o, f"4 CTAs per SM, precond {precond} fp32={fp32}")
    assert np.all(g["conv"] == 1)


OCC_CASES = [
    ("3d7_10x10x10", bilu.PRECOND_ILU0, dict(ilu_approach=1), 256),        # ILU factors, 4 rows per thread
    ("2d5_16x16", bilu.PRECOND_ILU0, dict(ilu_approach=1), 128),           # ILU factors, 2 rows per thread
    ("cd2d_24x24", bilu.PRECOND_ILU0_SPLIT, dict(ilu_approach=3), 192),    # given factors, 4 rows per thread
    ("3d7_7x7x7", bilu.PRECOND_PARILU0_ISAI, dict(parilu_sweeps=5), 128),  # ISAI, 4 rows per thread
    ("3d7_7x7x7", bilu.PRECOND_GENERAL_ISAI, dict(isai_power=2), 256),     # general ISAI, 2 rows per thread
    ("2d5_16x16", bilu.PRECOND_NONE, {}, 128),                             # none, 2 rows per thread
]


@pytest.mark.parametrize("fam,precond,kw,nt", OCC_CASES,
                         ids=[f"{c[0]}-p{c[1]}-t{c[3]}" for c in OCC_CASES])
@pytest.mark.parametrize("fp32", [False, True])
def test_rr_occupancy_variants_bitwise(cuda, fam, precond, kw, nt, fp32):
    """The occupancy variants of the register-resident kernel (staging bit 4, k_bicgstab_rr_occ: fewer
    registers, more threads per SM) at 2 and 4 rows per thread, for ILU factors (in-kernel and given), ISAI
    and no preconditioner: the same bits as the oracle's FAST order for that thread count."""
    if precond == bilu.PRECOND_NONE and fp32:
        pytest.skip("no preconditioner values to round")
    rp, ci, v, b = H.workload(fam, NSYS)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, reduction=bilu.REDUCE_FAST, smem_staging=16,
                    threads_per_system=nt, factor_precision=bilu.FP32 if fp32 else bilu.FP64, **kw, **TOL)
    assert g["info"]["threads"] == nt and g["info"]["operands_in_smem"] & 16, g["info"]
    o = _oracle_fast(rp, ci, v, b, precond, nt, fp32, approach=kw.get("ilu_approach", 1),
                     sweeps=kw.get("parilu_sweeps", 5), power=kw.get("isai_power", 2), **TOL)
    _check(g, o, f"occupancy variant {fam} precond {precond} threads {nt} fp32={fp32}")
    assert np.all(g["conv"] == 1)


def _wide_level_pattern(n=1000, seed=5):
    """Rows with a diagonal, upper entries (i, i+1) and (i, i+7), and lower entries only in every 97th row:
    the lower solve (and the ILU(0) schedule) has a first level of ~990 rows, far wider than the CTA, and
    the upper solve is a chain of n levels."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n):
        cols = {i}
        if i + 1 < n:
            cols.add(i + 1)
        if i + 7 < n:
            cols.add(i + 7)
        if i % 97 == 0 and i > 0:
            cols.add(i - 1)
            cols.add(i // 2)
        rows.append(sorted(cols))
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    ci = np.concatenate([np.array(r, np.int32) for r in rows])
    return rp, ci, rng


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("precond", [bilu.PRECOND_ILU0, bilu.PRECOND_ILU0_SPLIT])
def test_rr_lu_levels_wider_than_cta(cuda, fp32, precond):
    """Level widths above the CTA size take the solve programs' and the ILU program's second-slot paths."""
    rp, ci, rng = _wide_level_pattern()
    nsys, n = 4, len(rp) - 1
    v = np.empty((nsys, len(ci)))
    for s in range(nsys):
        for i in range(n):
            for k in range(rp[i], rp[i + 1]):
                v[s, k] = 2.0 + rng.random() if ci[k] == i else -(0.5 + rng.random())
    b = rng.uniform(-1, 1, (nsys, n))
    kw = dict(ilu_approach=1) if precond == bilu.PRECOND_ILU0 else dict(ilu_approach=3)
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=precond, reduction=bilu.REDUCE_FAST,
                    factor_precision=bilu.FP32 if fp32 else bilu.FP64, **kw, **TOL)
    assert g["info"]["threads"] == 128 and g["info"]["levels_lower"] < 10
    o = _oracle_fast(rp, ci, v, b, precond, 128, fp32, approach=kw["ilu_approach"], **TOL)
    _check(g, o, f"wide levels precond {precond} fp32={fp32}")
    assert np.all(g["conv"] == 1)


@pytest.mark.parametrize("n", [1, 2, 3, 33])
@pytest.mark.parametrize("reduction", [bilu.REDUCE_REF, bilu.REDUCE_FAST])
def test_rr_tiny_systems(cuda, n, reduction):
    """Systems of 1 to 33 rows (one or two slots of 32 rows, single-level solves) on the register-resident
    kernel, in both orders, merged ILU(0): bit for bit against the oracle."""
    rng = np.random.default_rng(n)
    nsys = 5
    rows = [sorted({min(max(i + d, 0), n - 1) for d in (-3, -1, 0, 1, 2)}) for i in range(n)]
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    ci = np.concatenate([np.array(r, np.int32) for r in rows])
    v = np.where(np.concatenate([np.array(r) == i for i, r in enumerate(rows)])[None, :],
                 3.0 + rng.random((nsys, len(ci))), -rng.random((nsys, len(ci))))
    b = rng.uniform(-1, 1, (nsys, n))
    g = H.gpu_solve(cuda, rp, ci, v, b, precond=bilu.PRECOND_ILU0, reduction=reduction, **TOL)
    assert g["info"]["solver_kernel"] == 1 and g["info"]["threads"] == 32
    if reduction == bilu.REDUCE_FAST:
        o = _oracle_fast(rp, ci, v, b, bilu.PRECOND_ILU0, 32, False, approach=1, **TOL)
    else:
        o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0, **TOL)
    _check(g, o, f"n={n} reduction={reduction}")
    assert np.all(g["conv"] == 1)
