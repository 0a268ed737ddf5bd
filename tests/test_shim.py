"""The drop-in C++ interface (libbilu_ref.so, merging-ilu0_gb300/shim/).

CPU: every function of the original headers is exported with the original
C++ signature; the original's five driver programs compile against these
headers and against their own and link unchanged (where the original sources
are present); the container classes have the original's size; the Matrix
Market batch reader builds the pages the way ReadWriteData.cpp does.
GPU: each of the five solver entry points and the factorisation / ISAI
functions, driven through the containers and files like the original drivers,
give results bit-identical to the oracle's restatement of the same computation.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import bilu
import helpers as H
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "merging-ilu0_gb300")
SHIM_INC = os.path.join(PKG, "shim", "include")
SHIM_LIB = os.path.join(PKG, "libbilu_ref.so")
DRIVER_SRC = os.path.join(ROOT, "tests", "shim_driver.cpp")
# the reference checkout: MERGING_ILU0_REFERENCE names its root (default /root/reference)
REF_DIR = os.path.join(os.environ.get("MERGING_ILU0_REFERENCE", "/root/reference"), "Batched-ILU0-merged",
                       "ILU0_ISAI_bicgstab")
DRIVERS = ["main_bicgstab_ilu", "main_bicgstab_ilu_merged", "main_bicgstab_ilu_segregated",
           "main_bicgstab_ilu_isai", "main_bicgstab_general_isai"]

# the original interface, as `nm -DC` prints it
SIGNATURES = [
    "Batched_ILU_Preconditioned_BiCGSTAB_Gpu(std::vector<std::__cxx11::basic_string<char, std::char_traits<char>, "
    "std::allocator<char> >, std::allocator<std::__cxx11::basic_string<char, std::char_traits<char>, "
    "std::allocator<char> > > > const&, PagedCSRMatrices const&, PagedVectors const&, PagedVectors&, bool, "
    "SolverResults&, bool, int, int, double&, double&, double&)",
    "Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu(",
    "Batched_General_ISAI_Preconditioned_BiCGSTAB_Gpu(",
    "Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_merged_Gpu(",
    "Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_segregated_Gpu(",
    "ILU_0_Factorization_Gpu(PagedCSRMatrices const&, PagedCSRMatrices&, PagedCSRMatrices&, int)",
    "ComputeILU0Approach1(PagedCSRMatrices&, int const*)",
    "ParILU_0_Factorization_Gpu(PagedCSRMatrices const&, PagedCSRMatrices&, PagedCSRMatrices&, int)",
    "GenerateISAI_gpu(PagedCSRMatrices&, PagedCSRMatrices const&, mat_type, int)",
    "FillSubdir(std::__cxx11::basic_string<char, std::char_traits<char>, std::allocator<char> > const&, ",
    "ReadData(int, std::vector<",
    "Print_ans(std::vector<",
    "PrintSolverResults(std::vector<",
    "PagedCSRMatrices::CopyFromCpuToGpu()", "PagedCSRMatrices::CopyFromGpuToCpu()",
    "PagedCSRMatrices::AllocateMemory(LOCATION)", "PagedCSRMatrices::DeallocateMemory(LOCATION)",
    "PagedCOOMatrices::CopyFromCpuToGpu()", "PagedVectors::AllocateMemory(LOCATION)",
    "PagedVectors::CopyFromGpuToCpu()", "SolverResults::SolverResults(int, double, CPU_EXISTENCE, GPU_EXISTENCE)",
    "SolverResults::CopyFromGpuToCpu()", "SolverResults::~SolverResults()", "PagedVectors::~PagedVectors()",
]


def _cuda_inc():
    import bilu_build
    return bilu_build._cuda_dirs()[0]


@pytest.fixture(scope="module")
def driver(built, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("drv") / "shim_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-I", SHIM_INC, "-I", _cuda_inc(), DRIVER_SRC, "-o", exe, "-L", PKG,
           "-lbilu_ref", f"-Wl,-rpath,{PKG}"]
    import bilu_build
    for d in bilu_build._cuda_dirs()[1]:
        cmd += [f"-L{d}"]
    cmd += ["-lcudart"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


# ---------------------------------------------------------------- Matrix Market files
def _write_system(d, rp, ci, vals, b, scaled=False, symmetric=False, integer=False, shuffle=None):
    os.makedirs(d, exist_ok=True)
    n = len(rp) - 1
    ents = []
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            if symmetric and ci[k] > i:
                continue
            ents.append((i + 1, ci[k] + 1, vals[k]))
    if shuffle is not None:
        shuffle.shuffle(ents)
    field = "integer" if integer else "real"
    sym = "symmetric" if symmetric else "general"
    fmt = (lambda v: "%d" % int(v)) if integer else (lambda v: "%.17g" % v)
    with open(os.path.join(d, "A_scaled.mtx" if scaled else "A.mtx"), "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {sym}\n% written by the tests\n")
        f.write(f"{n} {n} {len(ents)}\n")
        for i, j, v in ents:
            f.write(f"{i} {j} {fmt(v)}\n")
    with open(os.path.join(d, "b_scaled.mtx" if scaled else "b.mtx"), "w") as f:
        f.write("%%MatrixMarket matrix array real general\n")
        f.write(f"{n} 1\n")
        for v in b:
            f.write("%.17g\n" % v)


def _write_batch(root, rp, ci, vals, b, **kw):
    for s in range(vals.shape[0]):
        _write_system(os.path.join(root, f"sys{s:02d}"), rp, ci, vals[s], b[s], **kw)
    return root + "/"


def _run(driver, root, out, cmd, *args, problem_size=1, scaled=False, check=True):
    os.makedirs(out, exist_ok=True)
    r = subprocess.run([driver, root, str(problem_size), "1" if scaled else "0", out, cmd, *map(str, args)],
                       capture_output=True, text=True, timeout=600)
    if check and r.returncode != 0:
        raise AssertionError(f"shim_driver {cmd} failed ({r.returncode}):\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    return r


def _page_systems(out):
    subs = open(os.path.join(out, "subdirs.txt")).read().split()
    return subs, [int(os.path.basename(s)[3:]) for s in subs]


def _read_csr(path):
    raw = open(path, "rb").read()
    n, nnz, npages = struct.unpack("3i", raw[:12])
    o = 12
    rp = np.frombuffer(raw, np.int32, n + 1, o)
    o += 4 * (n + 1)
    ci = np.frombuffer(raw, np.int32, nnz, o)
    o += 4 * nnz
    v = np.frombuffer(raw, np.float64, nnz * npages, o).reshape(npages, nnz)
    return rp, ci, v


def _read_results(out):
    raw = open(os.path.join(out, "results.bin"), "rb").read()
    rec = np.frombuffer(raw, np.dtype([("it", "<f4"), ("cv", "<i4"), ("res", "<f8"), ("tr", "<f8")]))
    return {"iters": rec["it"].copy(), "conv": rec["cv"].copy(), "res": rec["res"].copy(), "true_res": rec["tr"].copy()}


def _read_x(path):
    lines = open(path).read().split("\n")
    assert lines[0] == "%%MatrixMarket matrix array real general"
    m, one = map(int, lines[1].split())
    assert one == 1
    return np.array([float(t) for t in lines[2:2 + m]])


# ---------------------------------------------------------------- CPU
def test_shim_exports_original_signatures(built):
    out = subprocess.run(["nm", "-DC", "--defined-only", SHIM_LIB], capture_output=True, text=True, check=True).stdout
    missing = [s for s in SIGNATURES if s not in out]
    assert not missing, f"not exported: {missing}"


@pytest.mark.skipif(not os.path.isdir(REF_DIR), reason="original sources not present")
@pytest.mark.parametrize("headers", ["shim", "original"])
def test_original_drivers_link_unchanged(built, tmp_path, headers):
    inc = ["-I", SHIM_INC] if headers == "shim" else ["-I", REF_DIR, "-I", _cuda_inc()]
    for m in DRIVERS:
        exe = str(tmp_path / m)
        r = subprocess.run(["g++", "-std=c++17", *inc, os.path.join(REF_DIR, m + ".cpp"), "-o", exe, "-L", PKG,
                            "-lbilu_ref", f"-Wl,-rpath,{PKG}"], capture_output=True, text=True)
        assert r.returncode == 0, f"{m} with {headers} headers:\n{r.stderr[-3000:]}"


@pytest.mark.skipif(not os.path.isdir(REF_DIR), reason="original sources not present")
def test_container_layout_matches_original(tmp_path):
    src = tmp_path / "layout.cpp"
    src.write_text('#include <cstdio>\n#include "matrix.h"\n#include "SolverResults.h"\n'
                   'int main(){std::printf("%zu %zu %zu %zu", sizeof(PagedCSRMatrices), sizeof(PagedCOOMatrices),'
                   ' sizeof(PagedVectors), sizeof(SolverResults));}\n')
    sizes = []
    for inc in (["-I", SHIM_INC], ["-I", REF_DIR, "-I", _cuda_inc()]):
        exe = str(tmp_path / f"lay{len(sizes)}")
        subprocess.run(["g++", "-std=c++17", *inc, str(src), "-o", exe], check=True, capture_output=True)
        sizes.append(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert sizes[0] == sizes[1]


def test_matrix_market_batch_reader(driver, tmp_path):
    """General, symmetric and integer files with entries in any order; Problem_Size repeats the subdirectories."""
    rp, ci, v, b = H.workload("2d5_8x8", 3)
    rng = np.random.default_rng(7)
    root = str(tmp_path / "cat") + "/"
    _write_system(root + "sys00", rp, ci, v[0], b[0], shuffle=rng)
    # a symmetric matrix on the same pattern, stored as its lower triangle
    sym = v[1].copy()
    n = len(rp) - 1
    pos = {(i, ci[k]): k for i in range(n) for k in range(rp[i], rp[i + 1])}
    for (i, j), k in pos.items():
        if j > i:
            sym[k] = sym[pos[(j, i)]]
    _write_system(root + "sys01", rp, ci, sym, b[1], symmetric=True, shuffle=rng)
    ints = np.round(v[2] * 4.0)
    _write_system(root + "sys02", rp, ci, ints, b[2], integer=True)
    out = str(tmp_path / "out")
    _run(driver, root, out, "read", problem_size=2)
    subs, sysid = _page_systems(out)
    assert sorted(sysid) == [0, 1, 2]
    arp, aci, av = _read_csr(os.path.join(out, "A.bin"))
    np.testing.assert_array_equal(arp, rp)
    np.testing.assert_array_equal(aci, ci)
    want = {0: v[0], 1: sym, 2: ints}
    bb = np.fromfile(os.path.join(out, "b.bin")).reshape(6, n)
    for p in range(6):
        s = sysid[p % 3]
        H.assert_bitwise(av[p], want[s], f"page {p} values")
        H.assert_bitwise(bb[p], b[s], f"page {p} rhs")


def test_matrix_market_pattern_mismatch_exits(driver, tmp_path):
    rp, ci, v, b = H.workload("2d5_8x8", 2)
    rp2, ci2, v2, b2 = H.workload("2d5_16x16", 1)
    root = str(tmp_path / "cat") + "/"
    _write_system(root + "a", rp, ci, v[0], b[0])
    _write_system(root + "b", rp2, ci2, v2[0], b2[0])
    r = _run(driver, root, str(tmp_path / "out"), "read", check=False)
    assert r.returncode == 1 and "size differs from the first system" in r.stdout


# ---------------------------------------------------------------- GPU
SOLVERS = [
    ("ilu", (0, 1, 0), dict(precond=bilu.PRECOND_ILU0_SPLIT, approach=1), "x_gpu_conv_ILU_app_1_bicgstab.mtx"),
    ("ilu", (0, 2, 0), dict(precond=bilu.PRECOND_ILU0_SPLIT, approach=2), "x_gpu_conv_ILU_app_2_bicgstab.mtx"),
    ("ilu", (0, 3, 0), dict(precond=bilu.PRECOND_ILU0_SPLIT, approach=3), "x_gpu_conv_ILU_app_3_bicgstab.mtx"),
    ("ilu", (0, 4, 0), dict(precond=bilu.PRECOND_ILU0_SPLIT, approach=4), "x_gpu_conv_ILU_app_4_bicgstab.mtx"),
    ("ilu", (1, 0, 5), dict(precond=bilu.PRECOND_PARILU0, sweeps=5), "x_gpu_parILU_5_bicgstab.mtx"),
    ("ilu_isai", (0, 0), dict(precond=bilu.PRECOND_ILU0_ISAI, approach=3), "x_gpu_ilu_isai_bicgstab.mtx"),
    ("ilu_isai", (1, 3), dict(precond=bilu.PRECOND_PARILU0_ISAI, sweeps=3), "x_gpu_ilu_isai_bicgstab.mtx"),
    ("general", (), dict(precond=bilu.PRECOND_GENERAL_ISAI, isai_power=1), "x_gpu_general_isai_bicgstab.mtx"),
    ("merged", (), dict(precond=bilu.PRECOND_ILU0, approach=1), "x_gpu_conv_ilu_merged_app1_bicgstab.mtx"),
    ("segregated", (), dict(precond=bilu.PRECOND_ILU0, approach=1), "x_gpu_conv_ilu_segregated_app1_bicgstab.mtx"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("cmd,args,pipe,xfile", SOLVERS, ids=[f"{s[0]}-{'-'.join(map(str, s[1]))}" for s in SOLVERS])
def test_shim_solver_entry_points_bitwise(driver, tmp_path, cmd, args, pipe, xfile):
    fam = "cd2d_12x12" if cmd == "general" else "2d5_8x8"
    rp, ci, v, b = H.workload(fam, 5)
    root = _write_batch(str(tmp_path / "cat"), rp, ci, v, b)
    out = str(tmp_path / "out")
    _run(driver, root, out, cmd, *args, problem_size=2)
    subs, sysid = _page_systems(out)
    o = H.oracle_pipeline(rp, ci, v, b, **pipe)
    res = _read_results(out)
    order = [sysid[p % len(subs)] for p in range(2 * len(subs))]
    for f in ("iters", "conv", "res", "true_res"):
        H.assert_bitwise(res[f], o[f][order], f"{cmd}{args}: {f}")
    for p, s in enumerate(subs):  # the entry point's own solution files, first #subdir pages
        H.assert_bitwise(_read_x(os.path.join(s, xfile)), o["x"][sysid[p]], f"{cmd}{args}: {xfile} of {s}")
    lines = open(os.path.join(out, "Results.txt")).read().splitlines()
    assert [(int(a), float(c)) for a, c in (ln.split() for ln in lines)] == \
        [(int(o["conv"][s]), float(o["iters"][s])) for s in sysid]
    pst, ist, oet, taken = map(float, open(os.path.join(out, "timing.txt")).read().split())
    assert taken > 0
    if cmd in ("ilu", "ilu_isai", "general"):  # merged / segregated have no PST / IST / OET outputs
        assert oet == pytest.approx(taken, abs=1e-5)
        assert 0 <= ist <= oet and pst == pytest.approx(oet - ist, abs=1e-3)


@pytest.mark.gpu
def test_shim_scaled_file_names(driver, tmp_path):
    rp, ci, v, b = H.workload("2d5_8x8", 2)
    root = _write_batch(str(tmp_path / "cat"), rp, ci, v, b, scaled=True)
    _run(driver, root, str(tmp_path / "out"), "merged", scaled=True)
    for s in range(2):
        assert os.path.exists(os.path.join(root, f"sys{s:02d}", "x_scaled_gpu_conv_ilu_merged_app1_bicgstab.mtx"))


@pytest.mark.gpu
@pytest.mark.parametrize("cmd,arg", [("factor_ilu", 1), ("factor_ilu", 2), ("factor_ilu", 3), ("factor_ilu", 4),
                                     ("factor_parilu", 0), ("factor_parilu", 6)])
def test_shim_factorisations_bitwise(driver, tmp_path, cmd, arg):
    rp, ci, v, b = H.workload("cd2d_12x12", 4)
    root = _write_batch(str(tmp_path / "cat"), rp, ci, v, b)
    out = str(tmp_path / "out")
    _run(driver, root, out, cmd, arg)
    _, sysid = _page_systems(out)
    lu = O.ilu0(rp, ci, v, arg) if cmd == "factor_ilu" else O.parilu0(rp, ci, v, arg)
    lrp, lci, urp, uci = O.split_pattern(rp, ci)
    Lv, Uv = O.split_values(rp, ci, lu)
    for name, (trp, tci, tv) in (("L", (lrp, lci, Lv)), ("U", (urp, uci, Uv))):
        grp, gci, gv = _read_csr(os.path.join(out, name + ".bin"))
        np.testing.assert_array_equal(grp, trp)
        np.testing.assert_array_equal(gci, tci)
        H.assert_bitwise(gv, tv[sysid], f"{cmd} {arg}: {name}")


@pytest.mark.gpu
def test_shim_compute_ilu0_approach1_in_place(driver, tmp_path):
    rp, ci, v, b = H.workload("3d7_5x5x5", 3)
    root = _write_batch(str(tmp_path / "cat"), rp, ci, v, b)
    out = str(tmp_path / "out")
    _run(driver, root, out, "approach1")
    _, sysid = _page_systems(out)
    _, _, fv = _read_csr(os.path.join(out, "F.bin"))
    H.assert_bitwise(fv, O.ilu0(rp, ci, v, 1)[sysid], "ComputeILU0Approach1")


def _triangle(rp, ci, v, lower):
    n = len(rp) - 1
    trp, tci, keep = [0], [], []
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            if (ci[k] <= i) if lower else (ci[k] >= i):
                tci.append(ci[k])
                keep.append(k)
        trp.append(len(tci))
    return np.array(trp, np.int32), np.array(tci, np.int32), v[:, keep]


@pytest.mark.gpu
@pytest.mark.parametrize("kind,power", [("general", 1), ("general", 2), ("lower", 2), ("lower", 3), ("upper", 2),
                                        ("lower_unit", 2)])
def test_shim_generate_isai_bitwise(driver, tmp_path, kind, power):
    rp, ci, v, b = H.workload("cd2d_12x12", 4)
    if kind == "general":
        trp, tci, tv, tri = rp, ci, v, 2
    elif kind == "lower_unit":  # the L factor the solvers pass: unit diagonal stored last
        lrp, lci, _, _ = O.split_pattern(rp, ci)
        Lv, _ = O.split_values(rp, ci, O.ilu0(rp, ci, v, 3))
        trp, tci, tv, tri = lrp, lci, Lv, 0
    else:  # a stand-alone triangle of A, diagonal not 1
        trp, tci, tv = _triangle(rp, ci, v, kind == "lower")
        tri = 0 if kind == "lower" else 1
    root = _write_batch(str(tmp_path / "cat"), trp, tci, tv, b)
    out = str(tmp_path / "out")
    _run(driver, root, out, "isai", {"general": 0, "upper": 2}.get(kind, 1), power)
    _, sysid = _page_systems(out)
    arp, aci = O.isai_pattern(trp, tci, power)
    grp, gci, gv = _read_csr(os.path.join(out, "AI.bin"))
    np.testing.assert_array_equal(grp, arp)
    np.testing.assert_array_equal(gci, aci)
    H.assert_bitwise(gv, O.isai_values(trp, tci, tv, tri, arp, aci)[sysid], f"GenerateISAI_gpu {kind} power {power}")
