"""CPU tests: the C ABI library loads and exports every declared symbol, host
logic (generators, pattern validation), and the oracle's own consistency."""
import ctypes
import os
import re
import sys

import numpy as np
import pytest

import bilu
import helpers as H
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bilu_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(bilu.LIBPATH)
    names = _declared("bilu.h")
    assert "bilu_solve" in names and "bilu_plan_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared in include/bilu.h but not exported: {missing}"


def test_default_options_match_reference_constants(built):
    o = bilu.default_options()
    assert o.precond == bilu.PRECOND_ILU0 and o.ilu_approach == 1
    assert o.tol == 1e-11 and o.tol_mode == bilu.TOL_ABS  # ATOL, PrecondBiCGSTAB.h:12
    assert o.max_iter == 500                               # MAX_ITER, PrecondBiCGSTAB.h:10
    assert o.isai_power == 2 and o.factor_precision == bilu.FP64 and o.reduction == bilu.REDUCE_REF


def test_generator_is_seeded_per_system(built):
    rp, ci, v5, b5 = bilu.gen_stencil(1, 16, 16, 1, 5, seed=7)
    _, _, v9, b9 = bilu.gen_stencil(1, 16, 16, 1, 9, seed=7)
    np.testing.assert_array_equal(v5, v9[:5])
    np.testing.assert_array_equal(b5, b9[:5])
    _, _, v5b, _ = bilu.gen_stencil(1, 16, 16, 1, 5, seed=8)
    assert not np.array_equal(v5, v5b)


@pytest.mark.parametrize("kind,grid,n,nnz", [(1, (16, 16, 1), 256, 1216), (2, (10, 10, 10), 1000, 6400),
                                             (4, (24, 24, 1), 576, 2784), (5, (7, 7, 7), 343, 2107)])
def test_generator_shapes_and_ranges(built, kind, grid, n, nnz):
    rp, ci, v, b = bilu.gen_stencil(kind, *grid, 3)
    assert len(rp) == n + 1 and len(ci) == nnz and v.shape == (3, nnz) and b.shape == (3, n)
    d = O.find_diag(rp, ci)
    assert np.all(d >= 0)
    diag = v[:, d]
    off = np.delete(v, d, axis=1)
    if kind == 1:
        assert diag.min() >= 4 and diag.max() < 5
        assert off.min() >= -1.2 - 0.3 and off.max() <= -0.8 + 0.3
    if kind == 2:
        assert diag.min() >= 6 and diag.max() < 7 and off.min() >= -1.25 - 0.25 and off.max() <= -0.75 + 0.25
    if kind == 5:
        assert diag.min() >= 6 and diag.max() < 7 and off.min() >= -1.3 and off.max() <= -0.7
    assert np.abs(b).max() <= 1.0
    for i in range(n):  # sorted columns
        assert np.all(np.diff(ci[rp[i]:rp[i + 1]]) > 0)


def test_uneven_generator(built):
    lib = bilu.lib()
    nsys = 64
    sn = np.zeros(nsys, np.int32)
    sz = np.zeros(nsys, np.int32)
    ip = ctypes.POINTER(ctypes.c_int)
    f = lib.bilu_gen_uneven
    f.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, ip, ip, ip,
                  ctypes.c_void_p, ctypes.c_void_p]
    assert f(nsys, 3, 64, 1024, 5, 12, sn.ctypes.data_as(ip), sz.ctypes.data_as(ip), None, None, None, None) == 0
    assert sn.min() >= 64 and sn.max() <= 1024
    rp = np.zeros(int(sn.sum()) + nsys, np.int32)
    ci = np.zeros(int(sz.sum()), np.int32)
    v = np.zeros(int(sz.sum()))
    b = np.zeros(int(sn.sum()))
    assert f(nsys, 3, 64, 1024, 5, 12, sn.ctypes.data_as(ip), sz.ctypes.data_as(ip), rp.ctypes.data_as(ip),
             ci.ctypes.data_as(ip), v.ctypes.data, b.ctypes.data) == 0
    ro = zo = 0
    for s in range(nsys):
        n = sn[s]
        r = rp[ro + s: ro + s + n + 1]
        c = ci[zo: zo + sz[s]]
        vv = v[zo: zo + sz[s]]
        assert r[0] == 0 and r[-1] == sz[s]
        for i in range(n):
            cols = c[r[i]:r[i + 1]]
            assert np.all(np.diff(cols) > 0) and i in cols
            k = 5 <= len(cols) - 1 <= 12
            assert k
            dv = vv[r[i] + int(np.where(cols == i)[0][0])]
            offs = np.abs(vv[r[i]:r[i + 1]]).sum() - abs(dv)
            assert abs(abs(dv) - 1.2 * offs) <= 1e-12 * max(1.0, offs)
        ro += n
        zo += sz[s]


def test_pattern_validation_without_device(built):
    rp = np.array([0, 2, 3], np.int32)
    for ci, code in ((np.array([1, 0, 1], np.int32), bilu.ERR_PATTERN),   # unsorted
                     (np.array([0, 2, 1], np.int32), bilu.ERR_PATTERN)):  # out of range
        with pytest.raises(bilu.BiluError) as e:
            bilu.Plan(rp, ci)
        assert e.value.code == code
    with pytest.raises(bilu.BiluError) as e:
        bilu.Plan(np.array([0, 1, 1], np.int32), np.array([0], np.int32), tol_mode=5)
    assert e.value.code == bilu.ERR_INVALID


def test_plan_without_device_reports_no_device(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    rp, ci, _, _ = H.workload("2d5_8x8", 1)
    with pytest.raises(bilu.BiluError) as e:
        bilu.Plan(rp, ci)
    assert e.value.code == bilu.ERR_NO_DEVICE


# ---------------------------------------------------------------- oracle consistency
def test_oracle_ilu_approaches(built):
    rp, ci, v, _ = H.workload("3d7_5x5x5", 4)
    a1, a2, a3, a4 = (O.ilu0(rp, ci, v, a) for a in (1, 2, 3, 4))
    H.assert_bitwise(a1, a4, "approach 1 vs 4")             # same per-entry update order
    np.testing.assert_allclose(a3, a1, rtol=1e-13, atol=0)  # different rounding, same factors
    np.testing.assert_allclose(a2, a1, rtol=1e-13, atol=0)
    # ILU(0) property: (L U)_ij = a_ij on the pattern
    assert O.ilu_residual(rp, ci, v, a1).max() < 1e-15


def test_oracle_parilu_reaches_exact_ilu_fixed_point(built):
    """Jacobi ParILU with the approach-3 formula: once every dependency has
    converged, a sweep reproduces ILU(0) approach 3 bit for bit."""
    rp, ci, v, _ = H.workload("2d5_8x8", 3)
    a3 = O.ilu0(rp, ci, v, 3)
    lu = O.parilu0(rp, ci, v, 200)
    H.assert_bitwise(lu, a3, "ParILU(200) vs ILU(0) approach 3")
    r = [O.ilu_residual(rp, ci, v, O.parilu0(rp, ci, v, s)).max() for s in (0, 1, 3, 6)]
    assert r[0] > r[1] > r[2] > r[3]


def test_oracle_isai_is_approximate_inverse_on_its_pattern(built):
    rp, ci, v, _ = H.workload("2d5_16x16", 2)
    lu = O.ilu0(rp, ci, v, 3)
    lrp, lci, urp, uci = O.split_pattern(rp, ci)
    L, U = O.split_values(rp, ci, lu)
    for (trp, tci, T, tri) in ((lrp, lci, L, 0), (urp, uci, U, 1)):
        arp, aci = O.isai_pattern(trp, tci, 2)
        # numeric pattern of page 0 equals the structural pattern here
        arpn, acin = O.isai_pattern(trp, tci, 2, T[0])
        np.testing.assert_array_equal(arpn, arp)
        np.testing.assert_array_equal(acin, aci)
        M = O.isai_values(trp, tci, T, tri, arp, aci)
        n = len(trp) - 1
        Td = np.zeros((n, n))
        Md = np.zeros((n, n))
        for i in range(n):
            Td[i, tci[trp[i]:trp[i + 1]]] = T[0, trp[i]:trp[i + 1]]
            Md[i, aci[arp[i]:arp[i + 1]]] = M[0, arp[i]:arp[i + 1]]
        P = Md @ Td
        for i in range(n):
            J = aci[arp[i]:arp[i + 1]]
            e = (J == i).astype(float)
            np.testing.assert_allclose(P[i, J], e, atol=1e-13)


@pytest.mark.parametrize("precond", range(6))
def test_oracle_solver_converges(built, precond):
    rp, ci, v, b = H.workload("2d5_16x16", 6)
    r = H.oracle_pipeline(rp, ci, v, b, precond, approach=3 if precond == 3 else 1)
    assert np.all(r["conv"] == 1) and np.all(r["status"] == 1)
    assert np.all(r["res"] < 1e-11)
    assert np.all(r["true_res"] < 1e-10)
    xd = O.dense_solve(rp, ci, v, b)
    assert np.abs(xd - r["x"]).max() < 1e-10


def test_oracle_half_step_exit_and_caps(built):
    rp, ci, v, b = H.workload("2d5_8x8", 8)
    r = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_NONE, max_iter=2)
    assert np.all(r["iters"] == 2) and np.all(r["conv"] == -1)
    r = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0)
    assert np.all(np.mod(r["iters"] * 2, 1) == 0)  # multiples of 0.5


def test_bench_reference_arm_json_line(built):
    """bench.py --impl reference times the CPU restatement on the host cores and prints the same JSON line
    as the GPU arm, with impl, cpu_baseline and a zero-copy e2e."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "systems/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    # the same workload as the GPU arm's line: its config key for key, the same dtype, the same CPU sample
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench.headline_config(1)
    assert line["dtype"] == bench.headline_dtype() == "f64 (ISAI FP32)"
    assert str(bench.CPU_SAMPLE) in cb["sample"] and cb["host"]["nproc"] >= 1 and cb["host"]["model"]
    assert "reference_gpu_kernels" in line


def test_oracle_pipeline_pattern_cache_keeps_results(built):
    """The pattern cache that the CPU timing runs use reproduces the uncached pipeline bit for bit."""
    rp, ci, v, b = H.workload("3d7_5x5x5", 4)
    kw = dict(sweeps=3, fp32=True, tol_mode=1, tol=1e-10)
    want = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_PARILU0_ISAI, **kw)
    cache = {}
    H.oracle_pipeline(rp, ci, v[:1], b[:1], bilu.PRECOND_PARILU0_ISAI, patterns=cache, **kw)
    got = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_PARILU0_ISAI, patterns=cache, **kw)
    assert set(cache) == {"diag", "split", "isai_l", "isai_u"}
    for k in ("x", "iters", "res", "true_res", "ail", "aiu"):
        H.assert_bitwise(got[k], want[k], k)


def test_bench_names_the_solver_kernel_from_the_plan(built):
    """bench.solver_kernel_name reads the plan's configuration: rows per thread from n and the CTA size, the
    occupancy variant from staging bit 4, the preconditioner values' type."""
    sys.path.insert(0, ROOT)
    import bench
    isai32 = dict(precond=4, factor_precision=1)
    info = dict(solver_kernel=1, threads=256, operands_in_smem=16)
    assert bench.solver_kernel_name(info, 1000, isai32).startswith("k_bicgstab_rr_occ<4, 1, float>")
    info = dict(solver_kernel=1, threads=128, operands_in_smem=6)
    assert bench.solver_kernel_name(info, 1000, isai32).startswith("k_bicgstab_rr<8, 1, float>")
    assert bench.solver_kernel_name(dict(solver_kernel=1, threads=32, operands_in_smem=0), 256,
                                    dict(precond=0)).startswith("k_bicgstab_rr<8, 3, double>")
    assert bench.solver_kernel_name(dict(solver_kernel=0, threads=1024, operands_in_smem=0), 1000,
                                    isai32).startswith("k_bicgstab ")
    assert bench.launches_per_step(dict(operands_in_smem=16)) == 3
    assert bench.launches_per_step(dict(operands_in_smem=8)) == 5

