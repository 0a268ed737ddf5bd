"""ORACLE -- test infrastructure only.

ctypes front end of oracle/liboracle.so, the CPU restatement of the
reference's arithmetic (oracle/oracle.cpp).  Only tests/, the smoke check
and bench.py's CPU-baseline leg use it; the library product never does.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "liboracle.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            import importlib.util
            spec = importlib.util.spec_from_file_location("build_oracle", os.path.join(HERE, "build_oracle.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        _lib = C.CDLL(LIBPATH)
        _lib.orc_isai_pattern.restype = C.c_int
        _lib.orc_isai_values.restype = C.c_int
        _lib.orc_count_missing_diag.restype = C.c_int
        _lib.orc_num_threads.restype = C.c_int
    return _lib


def _i(a):
    # the array must outlive the call: no conversion here (callers pass int32 arrays)
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous, "int32 contiguous array required"
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _ia(a):
    return np.ascontiguousarray(a, np.int32)


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _f(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def num_threads():
    return lib().orc_num_threads()


def set_num_threads(t):
    lib().orc_set_num_threads(int(t))


def count_missing_diag(rp, ci):
    rp, ci = _ia(rp), _ia(ci)
    return lib().orc_count_missing_diag(len(rp) - 1, _i(rp), _i(ci))


def add_missing_diag(rp, ci):
    rp, ci = _ia(rp), _ia(ci)
    n = len(rp) - 1
    m = count_missing_diag(rp, ci)
    nrp = np.zeros(n + 1, np.int32)
    nci = np.zeros(len(ci) + m, np.int32)
    src = np.zeros(len(ci) + m, np.int32)
    lib().orc_add_missing_diag(n, _i(rp), _i(ci), _i(nrp), _i(nci), _i(src))
    return nrp, nci, src


def find_diag(rp, ci):
    rp, ci = _ia(rp), _ia(ci)
    n = len(rp) - 1
    d = np.zeros(n, np.int32)
    lib().orc_find_diag(n, _i(rp), _i(ci), _i(d))
    return d


def split_pattern(rp, ci):
    rp, ci = _ia(rp), _ia(ci)
    n = len(rp) - 1
    d = find_diag(rp, ci)
    nl = int(np.sum(d - rp[:-1])) + n
    nu = int(np.sum(rp[1:] - d))
    lrp, lci = np.zeros(n + 1, np.int32), np.zeros(nl, np.int32)
    urp, uci = np.zeros(n + 1, np.int32), np.zeros(nu, np.int32)
    lib().orc_split_pattern(n, _i(rp), _i(ci), _i(d), _i(lrp), _i(lci), _i(urp), _i(uci))
    return lrp, lci, urp, uci


def split_values(rp, ci, lu):
    rp, ci = _ia(rp), _ia(ci)
    n = len(rp) - 1
    d = find_diag(rp, ci)
    lrp, lci, urp, uci = split_pattern(rp, ci)
    nsys = lu.shape[0]
    L = np.zeros((nsys, len(lci)))
    U = np.zeros((nsys, len(uci)))
    lu = np.ascontiguousarray(lu, np.float64)
    lib().orc_split_values(n, lu.shape[1], _i(rp), _i(d), nsys, _d(lu), len(lci), _d(L), len(uci), _d(U))
    return L, U


def ilu0(rp, ci, vals, approach=1):
    rp, ci = _ia(rp), _ia(ci)
    vals = np.ascontiguousarray(vals, np.float64)
    out = np.zeros_like(vals)
    lib().orc_ilu0(len(rp) - 1, vals.shape[1], _i(rp), _i(ci), vals.shape[0], _d(vals), _d(out), int(approach))
    return out


def parilu0(rp, ci, vals, sweeps, init=None, fast=False):
    """fast: the reciprocal-multiply sweep of BILU_REDUCE_FAST."""
    rp, ci = _ia(rp), _ia(ci)
    vals = np.ascontiguousarray(vals, np.float64)
    init = None if init is None else np.ascontiguousarray(init, np.float64)
    out = np.zeros_like(vals)
    lib().orc_parilu0_ex(len(rp) - 1, vals.shape[1], _i(rp), _i(ci), vals.shape[0], _d(vals), _d(init), int(sweeps),
                         _d(out), int(bool(fast)))
    return out


def ilu_residual(rp, ci, vals, lu):
    rp, ci = _ia(rp), _ia(ci)
    vals = np.ascontiguousarray(vals, np.float64)
    lu = np.ascontiguousarray(lu, np.float64)
    out = np.zeros(vals.shape[0])
    lib().orc_ilu_residual(len(rp) - 1, vals.shape[1], _i(rp), _i(ci), vals.shape[0], _d(vals), _d(lu), _d(out))
    return out


def isai_pattern(rp, ci, power, vals0=None):
    rp, ci = _ia(rp), _ia(ci)
    n = len(rp) - 1
    v0 = None if vals0 is None else np.ascontiguousarray(vals0, np.float64)
    nz = lib().orc_isai_pattern(n, _i(rp), _i(ci), int(power), _d(v0), None, None)
    arp = np.zeros(n + 1, np.int32)
    aci = np.zeros(nz, np.int32)
    lib().orc_isai_pattern(n, _i(rp), _i(ci), int(power), _d(v0), _i(arp), _i(aci))
    return arp, aci


def isai_values(trp, tci, tvals, tri, arp, aci, fast=False):
    """fast: True (1) = the reciprocal-multiply upper-triangle ISAI of BILU_REDUCE_FAST; 2 = the FAST ISAI
    stored in FP32, computed in FP32 (values returned widened to float64)."""
    trp, tci, arp, aci = _ia(trp), _ia(tci), _ia(arp), _ia(aci)
    tvals = np.ascontiguousarray(tvals, np.float64)
    out = np.zeros((tvals.shape[0], len(aci)))
    r = lib().orc_isai_values_ex(len(trp) - 1, _i(trp), _i(tci), tvals.shape[1], tvals.shape[0], _d(tvals),
                                 int(tri), _i(arp), _i(aci), len(aci), _d(out), int(fast))
    if r != 0:
        raise ValueError("ISAI row longer than 32")
    return out


PREC_LU, PREC_ISAI, PREC_NONE, PREC_LU_F32, PREC_ISAI_F32, PREC_GISAI, PREC_GISAI_F32 = 0, 1, 2, 3, 4, 5, 6


def bicgstab(rp, ci, A, b, prec=PREC_LU, lu=None, ail=None, aiu=None, dot=0, tol_mode=0, tol=1e-11, max_iter=500,
             lu_f32=None, ail_f32=None, aiu_f32=None, factor_pattern=None):
    """ail / aiu: (row_ptrs, col_idxs, values) tuples; factor_pattern: (row_ptrs, col_idxs) of lu when it
    differs from A's (inserted diagonals).  Returns dict of x, iters, conv, res, status."""
    rp, ci = _ia(rp), _ia(ci)
    frp, fci = (None, None) if factor_pattern is None else (_ia(factor_pattern[0]), _ia(factor_pattern[1]))
    A = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    nsys, n = b.shape
    x = np.zeros_like(b)
    iters = np.zeros(nsys, np.float32)
    conv = np.zeros(nsys, np.int32)
    res = np.zeros(nsys)
    status = np.zeros(nsys, np.int32)
    lu = None if lu is None else np.ascontiguousarray(lu, np.float64)
    lu_f32 = None if lu_f32 is None else np.ascontiguousarray(lu_f32, np.float32)
    empty = (np.zeros(1, np.int32), np.zeros(1, np.int32), None)
    ailt = (_ia(ail[0]), _ia(ail[1]), ail[2]) if ail is not None else empty
    aiut = (_ia(aiu[0]), _ia(aiu[1]), aiu[2]) if aiu is not None else empty
    ailv = None if ailt[2] is None else np.ascontiguousarray(ailt[2], np.float64)
    aiuv = None if aiut[2] is None else np.ascontiguousarray(aiut[2], np.float64)
    ailf = None if ail_f32 is None else np.ascontiguousarray(ail_f32, np.float32)
    aiuf = None if aiu_f32 is None else np.ascontiguousarray(aiu_f32, np.float32)
    lib().orc_bicgstab(n, A.shape[1], _i(rp), _i(ci), nsys, _d(A), _d(b), 0 if fci is None else len(fci), _i(frp),
                       _i(fci), int(prec), _d(lu), _f(lu_f32),
                       len(ailt[1]), _i(ailt[0]), _i(ailt[1]), _d(ailv), _f(ailf),
                       len(aiut[1]), _i(aiut[0]), _i(aiut[1]), _d(aiuv), _f(aiuf),
                       int(dot), int(tol_mode), C.c_double(tol), int(max_iter), _d(x), _f(iters), _i(conv), _d(res),
                       _i(status))
    return {"x": x, "iters": iters, "conv": conv, "res": res, "status": status}


def bicgstab_fast(rp, ci, A, b, nt, pv=1, ail=None, aiu=None, fp32=False, tol_mode=0, tol=1e-11, max_iter=500):
    """BILU_REDUCE_FAST order of the register-resident solver with `nt` threads per system.  pv: 0 none,
    1 ISAI of L and U (ail, aiu = (row_ptrs, col_idxs, values)), 2 general ISAI (ail), 3 in-place ILU
    factors (ail = (factor row_ptrs, col_idxs, LU values)).  fp32: preconditioner values rounded to float
    and applied in float.  Returns x, iters, conv, res, status, true_res."""
    rp, ci = _ia(rp), _ia(ci)
    A = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    nsys, n = b.shape
    out = {"x": np.zeros_like(b), "iters": np.zeros(nsys, np.float32), "conv": np.zeros(nsys, np.int32),
           "res": np.zeros(nsys), "status": np.zeros(nsys, np.int32), "true_res": np.zeros(nsys)}
    empty = (np.zeros(1, np.int32), np.zeros(1, np.int32), None)
    tri = []
    for m in (ail, aiu):
        if m is None:
            tri.append((empty[0], empty[1], 0, None, None))
            continue
        vd = np.ascontiguousarray(m[2], np.float64)
        vf = np.ascontiguousarray(m[2], np.float32) if fp32 else None
        tri.append((_ia(m[0]), _ia(m[1]), len(m[1]), None if fp32 else vd, vf))
    (lr, lc, ln, ld, lf), (ur, uc, un, ud, uf) = tri
    rc = lib().orc_bicgstab_fast(n, A.shape[1], _i(rp), _i(ci), nsys, _d(A), _d(b), int(pv), int(bool(fp32)),
                                 _i(lr), _i(lc), ln, _d(ld), _f(lf), _i(ur), _i(uc), un, _d(ud), _f(uf), int(nt),
                                 int(tol_mode), C.c_double(tol), int(max_iter), _d(out["x"]), _f(out["iters"]),
                                 _i(out["conv"]), _d(out["res"]), _i(out["status"]), _d(out["true_res"]))
    if rc != 0:
        raise ValueError("orc_bicgstab_fast: threads must be a multiple of 32 with at most 8 rows per thread")
    return out


def true_residual(rp, ci, A, b, x):
    rp, ci = _ia(rp), _ia(ci)
    A = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros(b.shape[0])
    lib().orc_true_residual(b.shape[1], A.shape[1], _i(rp), _i(ci), b.shape[0], _d(A), _d(b), _d(x), _d(out))
    return out


def dense_solve(rp, ci, A, b, sys_ids=None):
    rp, ci = _ia(rp), _ia(ci)
    A = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    ids = None if sys_ids is None else np.ascontiguousarray(sys_ids, np.int32)
    m = b.shape[0] if ids is None else len(ids)
    out = np.zeros((m, b.shape[1]))
    lib().orc_dense_solve(b.shape[1], A.shape[1], _i(rp), _i(ci), m, _i(ids), _d(A), _d(b), _d(out))
    return out


# ---------------------------------------------------------------- learned warm start
def mlp_features(rp, ci, vals, idx):
    rp, ci = _ia(rp), _ia(ci)
    vals = np.ascontiguousarray(vals, np.float64)
    idx = _ia(idx)
    feat = np.zeros((len(idx), 9), np.float32)
    base = np.zeros(len(idx))
    lib().orc_mlp_features(len(rp) - 1, vals.shape[1], _i(rp), _i(ci), vals.shape[0], _d(vals), len(idx), _i(idx),
                           _f(feat), _d(base))
    return feat, base


def mlp_loss_grad(params, feat, y):
    lib().orc_mlp_loss_grad.restype = C.c_double
    params = np.ascontiguousarray(params, np.float32)
    feat = np.ascontiguousarray(feat, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    grad = np.zeros(len(params))
    out = np.zeros(len(y))
    loss = lib().orc_mlp_loss_grad(_f(params), len(y), _f(feat), _f(y), _d(grad), _d(out))
    return loss, grad, out
