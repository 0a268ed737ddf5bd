"""ORACLE -- test infrastructure only.

Python front end of oracle/_ref/libreflaunch.so: runs the reference's own
kernels (compiled from its sources by oracle/build_ref.py) on torch CUDA
tensors.  The reference's host-side preparation that these kernels need is
restated here from its source (pattern-only integer work):

  diag_ptrs                 factorization.cu:192-212, 472-480
  L/U split patterns        factorization.cu:216-344
  ParILU dependency graph   parILU_0_gpu.cu:118-220
  approach-4 era lists      ILU_0_gpu.cu:947-1053
  ISAI pattern of |T|^p     isai_gpu.cu:40-179 (oracle.isai_pattern)

Kernels the reference can only run with grid-wide spin-waits (ILU approaches
2 and 3) are not available here.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFDIR = os.path.join(HERE, "_ref")
LIBPATH = os.path.join(REFDIR, "libreflaunch.so")
_lib = None


def available():
    return os.path.exists(LIBPATH) and all(
        os.path.exists(os.path.join(REFDIR, u + ".cubin"))
        for u in ("merged", "ilu_split", "ilu_isai", "ilu0", "parilu", "isai", "general_isai"))


def lib(device=0):
    global _lib
    if _lib is None:
        L = C.CDLL(LIBPATH)
        L.ref_last_error.restype = C.c_char_p
        L.ref_load.argtypes = [C.c_char_p, C.c_int]
        r = L.ref_load(REFDIR.encode(), device)
        if r != 0:
            raise RuntimeError("ref_load: " + L.ref_last_error().decode())
        _lib = L
    return _lib


def _p(t):
    return C.c_void_p(t.data_ptr())


def _call(fn, *args):
    conv = []
    for a in args:
        if isinstance(a, int):
            conv.append(C.c_int(a))
        else:
            conv.append(_p(a))
    r = fn(*conv)
    if r != 0:
        raise RuntimeError(f"{fn.__name__}: " + lib().ref_last_error().decode())


# ---------------------------------------------------------------- host preparation restated
def parilu_dependencies(rp, ci, lrp, lci, urp, uci):
    """create_dependency_graph_parilu (parILU_0_gpu.cu:118-220)."""
    n = len(rp) - 1
    deps = []
    nzp = [0]
    for row in range(n):
        rs, re = rp[row], rp[row + 1]
        for loc in range(rs, re):
            col = ci[loc]
            if row > col:
                deps.append(loc - rs + lrp[row])
            else:
                deps.append((urp[row + 1] - 1) - (re - 1 - loc))
            kmax = min(row, col) - 1
            nd = 0
            for li in range(lrp[row], lrp[row + 1]):
                k = lci[li]
                if k > kmax:
                    continue
                for ui in range(urp[k], urp[k + 1]):
                    if uci[ui] == col:
                        deps += [li, ui]
                        nd += 2
            if row > col:
                deps.append(urp[col])
                nd += 1
            nzp.append(nzp[-1] + nd + 1)
    return np.array(deps, np.int32), np.array(nzp, np.int32)


def approach4_lists(rp, ci):
    """create_dependency_list (ILU_0_gpu.cu:947-1053)."""
    n = len(rp) - 1
    deps, starters, era = [], [], [0]
    d_start = 0
    era_start = 0
    for cur in range(n):
        temp = {}
        for j in range(rp[cur], rp[cur + 1]):
            temp[ci[j]] = j
        for below in range(cur + 1, n):
            loc_row = -1
            for loc in range(rp[below], rp[below + 1]):
                col = ci[loc]
                if col < cur:
                    continue
                if col == cur:
                    deps += [loc, temp.get(cur, -1)]
                    starters.append(d_start)
                    d_start += 2
                    era_start += 1
                    loc_row = loc
                else:
                    if loc_row == -1:
                        break
                    lc = temp.get(col, -1)
                    if lc == -1:
                        continue
                    deps += [loc, lc]
                    d_start += 2
        if era[-1] < era_start:
            era.append(era_start)
    starters.append(d_start)
    return np.array(deps, np.int32), np.array(starters, np.int32), np.array(era, np.int32)


# ---------------------------------------------------------------- kernels
def merged_solve(dev, rp, ci, vals, b):
    """Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_merged_Gpu's kernel sequence (no file output):
    diagonal pointers, the merged solver kernel, then KernelFillTrueResNorms."""
    import torch
    import oracle as O
    nsys, n = b.shape
    nnz = len(ci)
    T = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    RP, CI, D = T(rp, torch.int32), T(ci, torch.int32), T(O.find_diag(rp, ci), torch.int32)
    V, B = T(vals, torch.float64), T(b, torch.float64)
    X = torch.zeros_like(B)
    F = torch.empty_like(V)
    it = torch.zeros(nsys, dtype=torch.float32, device=dev)
    cv = torch.zeros(nsys, dtype=torch.int32, device=dev)
    rs = torch.zeros(nsys, dtype=torch.float64, device=dev)
    tr = torch.zeros(nsys, dtype=torch.float64, device=dev)
    L = lib()
    _call(L.ref_merged, n, nnz, nsys, RP, CI, V, B, X, F, D, it, cv, rs)
    _call(L.ref_true_residual, n, nnz, nsys, RP, CI, V, B, X, tr)
    return {"x": X.cpu().numpy(), "iters": it.cpu().numpy(), "conv": cv.cpu().numpy(), "res": rs.cpu().numpy(),
            "true_res": tr.cpu().numpy(), "lu": F.cpu().numpy()}


def ilu0(dev, rp, ci, vals, approach):
    import torch
    import oracle as O
    nsys, nnz = vals.shape
    n = len(rp) - 1
    V = torch.as_tensor(np.ascontiguousarray(vals), device=dev)
    if approach == 1:
        RP = torch.as_tensor(rp, dtype=torch.int32, device=dev)
        CI = torch.as_tensor(ci, dtype=torch.int32, device=dev)
        D = torch.as_tensor(O.find_diag(rp, ci), dtype=torch.int32, device=dev)
        _call(lib().ref_ilu0_app1, nsys, n, nnz, RP, CI, V, D)
    elif approach == 4:
        deps, starters, era = approach4_lists(rp, ci)
        Dp = torch.as_tensor(deps if len(deps) else np.zeros(1, np.int32), device=dev)
        S = torch.as_tensor(starters, device=dev)
        E = torch.as_tensor(era, device=dev)
        _call(lib().ref_ilu0_app4, nsys, nnz, V, Dp, S, E, len(era), len(deps))
    else:
        raise ValueError("approaches 2 and 3 spin across the grid and are not run")
    return V.cpu().numpy()


def split_solve(dev, rp, ci, vals, b, lu):
    """PrecondBiCGSTAB_ilu_gpu.cu's solver kernel with the given in-place factors split into L and U."""
    import torch
    import oracle as O
    nsys, n = b.shape
    lrp, lci, urp, uci = O.split_pattern(rp, ci)
    Lv, Uv = O.split_values(rp, ci, lu)
    T = lambda a, dt=None: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    X = torch.zeros((nsys, n), dtype=torch.float64, device=dev)
    it = torch.zeros(nsys, dtype=torch.float32, device=dev)
    cv = torch.zeros(nsys, dtype=torch.int32, device=dev)
    rs = torch.zeros(nsys, dtype=torch.float64, device=dev)
    _call(lib().ref_split_solve, n, len(ci), nsys, T(rp, torch.int32), T(ci, torch.int32), T(vals), T(b), X,
          len(lci), T(lrp, torch.int32), T(lci, torch.int32), T(Lv), len(uci), T(urp, torch.int32),
          T(uci, torch.int32), T(Uv), it, cv, rs)
    return {"x": X.cpu().numpy(), "iters": it.cpu().numpy(), "conv": cv.cpu().numpy(), "res": rs.cpu().numpy()}


def parilu(dev, rp, ci, vals, sweeps):
    """ParILU0_Approach2's kernel (parILU_0_gpu.cu:255-287); returns in-place factors."""
    import torch
    import oracle as O
    nsys, nnz = vals.shape
    n = len(rp) - 1
    lrp, lci, urp, uci = O.split_pattern(rp, ci)
    Lv, Uv = O.split_values(rp, ci, vals)  # Fill_L_and_U: L = strict lower + I, U = upper
    deps, nzp = parilu_dependencies(rp, ci, lrp, lci, urp, uci)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    LV, UV = T(Lv), T(Uv)
    _call(lib().ref_parilu, nsys, n, nnz, T(vals), len(lci), LV, len(uci), UV, sweeps, T(deps), T(nzp))
    # back to the in-place layout
    Lh, Uh = LV.cpu().numpy(), UV.cpu().numpy()
    d = O.find_diag(rp, ci)
    out = np.zeros_like(vals)
    for i in range(n):
        nl = d[i] - rp[i]
        out[:, rp[i]:d[i]] = Lh[:, lrp[i]:lrp[i] + nl]
        out[:, d[i]:rp[i + 1]] = Uh[:, urp[i]:urp[i + 1]]
    return out


def isai(dev, trp, tci, tvals, tri, arp, aci):
    """GenerateISAI_gpu's two kernels on a triangular factor T (reference split CSR) and ISAI pattern."""
    import torch
    nsys = tvals.shape[0]
    n = len(trp) - 1
    T = lambda a, dt=None: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    dense = torch.full((n * 32 * 32,), -1, dtype=torch.int32, device=dev)
    rhs1 = torch.full((n,), -1, dtype=torch.int32, device=dev)
    sizes = torch.zeros(n, dtype=torch.int32, device=dev)
    TRP, TCI, ARP, ACI = T(trp, torch.int32), T(tci, torch.int32), T(arp, torch.int32), T(aci, torch.int32)
    _call(lib().ref_isai_extract, n, TRP, TCI, len(tci), ARP, ACI, len(aci), dense, rhs1, sizes)
    M = torch.zeros((nsys, len(aci)), dtype=torch.float64, device=dev)
    _call(lib().ref_isai_fill, nsys, n, ARP, ACI, M, len(aci), TRP, TCI, T(tvals), len(tci), dense, rhs1, sizes, tri)
    return M.cpu().numpy()


def isai_solve(dev, rp, ci, vals, b, ail, aiu):
    """KernelBatchedPreconditionedBiCGSTAB_ILU_ISAI with (row_ptrs, col_idxs, values) ISAI factors."""
    import torch
    nsys, n = b.shape
    T = lambda a, dt=None: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    X = torch.zeros((nsys, n), dtype=torch.float64, device=dev)
    it = torch.zeros(nsys, dtype=torch.float32, device=dev)
    cv = torch.zeros(nsys, dtype=torch.int32, device=dev)
    rs = torch.zeros(nsys, dtype=torch.float64, device=dev)
    _call(lib().ref_isai_solve, n, len(ci), nsys, T(rp, torch.int32), T(ci, torch.int32), T(vals), T(b), X,
          len(ail[1]), T(ail[0], torch.int32), T(ail[1], torch.int32), T(ail[2]), len(aiu[1]),
          T(aiu[0], torch.int32), T(aiu[1], torch.int32), T(aiu[2]), it, cv, rs)
    return {"x": X.cpu().numpy(), "iters": it.cpu().numpy(), "conv": cv.cpu().numpy(), "res": rs.cpu().numpy()}


def general_isai_solve(dev, rp, ci, vals, b, ai):
    """KernelBatchedPreconditionedBiCGSTABGeneralISAI with (row_ptrs, col_idxs, values) of aiA."""
    import torch
    nsys, n = b.shape
    T = lambda a, dt=None: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    X = torch.zeros((nsys, n), dtype=torch.float64, device=dev)
    it = torch.zeros(nsys, dtype=torch.float32, device=dev)
    cv = torch.zeros(nsys, dtype=torch.int32, device=dev)
    rs = torch.zeros(nsys, dtype=torch.float64, device=dev)
    _call(lib().ref_general_isai_solve, n, len(ci), nsys, T(rp, torch.int32), T(ci, torch.int32), T(vals), T(b), X,
          len(ai[1]), T(ai[0], torch.int32), T(ai[1], torch.int32), T(ai[2]), it, cv, rs)
    return {"x": X.cpu().numpy(), "iters": it.cpu().numpy(), "conv": cv.cpu().numpy(), "res": rs.cpu().numpy()}

