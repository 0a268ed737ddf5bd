"""Shared helpers of the test suite: seeded workloads, the oracle pipeline
that mirrors each preconditioner family, and GPU calls through the C ABI."""
import numpy as np

import bilu
import oracle as O

SEED = 20261203

# Small members of the benchmark families (kind, gx, gy, gz): every parity
# case runs the same generator as the benchmark with a smaller grid.
FAMILIES = {
    "2d5_8x8": (1, 8, 8, 1),
    "2d5_16x16": (1, 16, 16, 1),
    "3d7_5x5x5": (2, 5, 5, 5),
    "cd2d_12x12": (4, 12, 12, 1),
    "3d7_7x7x7": (5, 7, 7, 7),
    "cd2d_24x24": (4, 24, 24, 1),
    "3d7_10x10x10": (2, 10, 10, 10),
}


def workload(name, nsys, seed=SEED):
    kind, gx, gy, gz = FAMILIES[name]
    return bilu.gen_stencil(kind, gx, gy, gz, nsys, seed)


def oracle_pipeline(rp, ci, vals, b, precond, approach=1, sweeps=5, fp32=False, tol_mode=0, tol=1e-11,
                    max_iter=500, isai_power=2, lu_init=None, patterns=None):
    """The reference's computation for one preconditioner family, restated on the CPU.

    patterns: an optional dict that keeps the pattern-only work (diagonal insertion, L/U split and ISAI
    patterns) of the first call for the later calls on the same pattern, as a plan does; timing runs
    fill it untimed."""
    out = {}
    memo = patterns if patterns is not None else {}

    def once(key, f):
        if key not in memo:
            memo[key] = f()
        return memo[key]
    if precond == bilu.PRECOND_NONE:
        r = O.bicgstab(rp, ci, vals, b, prec=O.PREC_NONE, dot=0, tol_mode=tol_mode, tol=tol, max_iter=max_iter)
        r["true_res"] = O.true_residual(rp, ci, vals, b, r["x"])
        return r
    nrp, nci, src = once("diag", lambda: O.add_missing_diag(rp, ci))
    fvals = np.where(src[None, :] >= 0, vals[:, np.maximum(src, 0)], 0.0)
    if precond == bilu.PRECOND_GENERAL_ISAI:
        arp, aci = once("gisai", lambda: O.isai_pattern(nrp, nci, isai_power))
        ai = O.isai_values(nrp, nci, fvals, 2, arp, aci)
        out.update(ai=ai, ai_pattern=(arp, aci))
        if fp32:
            r = O.bicgstab(rp, ci, vals, b, prec=O.PREC_GISAI_F32, ail=(arp, aci, None), ail_f32=ai.astype(np.float32),
                           dot=1, tol_mode=tol_mode, tol=tol, max_iter=max_iter)
        else:
            r = O.bicgstab(rp, ci, vals, b, prec=O.PREC_GISAI, ail=(arp, aci, ai), dot=1, tol_mode=tol_mode, tol=tol,
                           max_iter=max_iter)
        out.update(r)
        out["true_res"] = O.true_residual(rp, ci, vals, b, r["x"])
        return out
    if precond in (bilu.PRECOND_ILU0, bilu.PRECOND_ILU0_SPLIT, bilu.PRECOND_ILU0_ISAI):
        lu = O.ilu0(nrp, nci, fvals, approach)
    else:
        lu = O.parilu0(nrp, nci, fvals, sweeps, init=lu_init)
    out["lu"] = lu
    if precond in (bilu.PRECOND_ILU0_ISAI, bilu.PRECOND_PARILU0_ISAI):
        lrp, lci, urp, uci = once("split", lambda: O.split_pattern(nrp, nci))
        L, U = O.split_values(nrp, nci, lu)
        arp, aci = once("isai_l", lambda: O.isai_pattern(lrp, lci, isai_power))
        brp, bci = once("isai_u", lambda: O.isai_pattern(urp, uci, isai_power))
        ail = O.isai_values(lrp, lci, L, 0, arp, aci)
        aiu = O.isai_values(urp, uci, U, 1, brp, bci)
        out.update(ail=ail, aiu=aiu, ail_pattern=(arp, aci), aiu_pattern=(brp, bci))
        if fp32:
            r = O.bicgstab(rp, ci, vals, b, prec=O.PREC_ISAI_F32, ail=(arp, aci, None), aiu=(brp, bci, None),
                           ail_f32=ail.astype(np.float32), aiu_f32=aiu.astype(np.float32), dot=1,
                           tol_mode=tol_mode, tol=tol, max_iter=max_iter)
        else:
            r = O.bicgstab(rp, ci, vals, b, prec=O.PREC_ISAI, ail=(arp, aci, ail), aiu=(brp, bci, aiu), dot=1,
                           tol_mode=tol_mode, tol=tol, max_iter=max_iter)
    else:
        fp = (nrp, nci)
        if fp32:
            r = O.bicgstab(rp, ci, vals, b, prec=O.PREC_LU_F32, lu_f32=lu.astype(np.float32), dot=0,
                           tol_mode=tol_mode, tol=tol, max_iter=max_iter, factor_pattern=fp)
        else:
            r = O.bicgstab(rp, ci, vals, b, prec=O.PREC_LU, lu=lu, dot=0, tol_mode=tol_mode, tol=tol,
                           max_iter=max_iter, factor_pattern=fp)
    out.update(r)
    out["true_res"] = O.true_residual(rp, ci, vals, b, r["x"])
    return out


def oracle_fast(rp, ci, v, b, precond, nt, fp32, approach=3, sweeps=5, power=2, **tol):
    """The oracle's restatement of the FAST order (orc_bicgstab_fast) for one preconditioner family with `nt`
    threads per system: factors, ISAI values and the solve, as the register-resident kernel computes them."""
    nrp, nci, src = O.add_missing_diag(rp, ci)
    fv = np.where(src[None, :] >= 0, v[:, np.maximum(src, 0)], 0.0)
    if precond == bilu.PRECOND_NONE:
        return O.bicgstab_fast(rp, ci, v, b, nt, pv=0, **tol)
    if precond == bilu.PRECOND_GENERAL_ISAI:
        arp, aci = O.isai_pattern(nrp, nci, power)
        ai = O.isai_values(nrp, nci, fv, 2, arp, aci)
        return O.bicgstab_fast(rp, ci, v, b, nt, pv=2, ail=(arp, aci, ai), fp32=fp32, **tol)
    if precond in (bilu.PRECOND_ILU0, bilu.PRECOND_ILU0_SPLIT, bilu.PRECOND_PARILU0):
        if precond == bilu.PRECOND_PARILU0:
            lu = O.parilu0(nrp, nci, fv, sweeps, fast=True)
        else:
            lu = O.ilu0(nrp, nci, fv, approach)
        return O.bicgstab_fast(rp, ci, v, b, nt, pv=3, ail=(nrp, nci, lu), fp32=fp32, **tol)
    if precond == bilu.PRECOND_ILU0_ISAI:
        lu = O.ilu0(nrp, nci, fv, approach)
    else:
        lu = O.parilu0(nrp, nci, fv, sweeps, fast=True)
    lrp, lci, urp, uci = O.split_pattern(nrp, nci)
    Lv, Uv = O.split_values(nrp, nci, lu)
    arp, aci = O.isai_pattern(lrp, lci, power)
    brp, bci = O.isai_pattern(urp, uci, power)
    ail = O.isai_values(lrp, lci, Lv, 0, arp, aci, fast=2 if fp32 else False)
    aiu = O.isai_values(urp, uci, Uv, 1, brp, bci, fast=2 if fp32 else True)
    return O.bicgstab_fast(rp, ci, v, b, nt, pv=1, ail=(arp, aci, ail), aiu=(brp, bci, aiu), fp32=fp32, **tol)


def gpu_solve(dev, rp, ci, vals, b, lu_init=None, **opts):
    """Solve through the C ABI; returns numpy results and the plan info."""
    import torch
    nsys, n = b.shape
    with bilu.Plan(rp, ci, **opts) as plan:
        V = torch.from_numpy(vals).to(dev)
        B = torch.from_numpy(b).to(dev)
        X = torch.full_like(B, float("nan"))
        it = torch.full((nsys,), -7.0, dtype=torch.float32, device=dev)
        cv = torch.full((nsys,), 7, dtype=torch.int32, device=dev)
        rs = torch.full((nsys,), -1.0, dtype=torch.float64, device=dev)
        tr = torch.full((nsys,), -1.0, dtype=torch.float64, device=dev)
        st = torch.full((nsys,), 99, dtype=torch.int32, device=dev)
        LI = None if lu_init is None else torch.from_numpy(lu_init).to(dev)
        plan.solve(V, B, X, it, cv, rs, tr, st, lu_init=LI)
        torch.cuda.synchronize()
        info = plan.info()
    return {"x": X.cpu().numpy(), "iters": it.cpu().numpy(), "conv": cv.cpu().numpy(), "res": rs.cpu().numpy(),
            "true_res": tr.cpu().numpy(), "status": st.cpu().numpy(), "info": info}


def assert_bitwise(a, b, what):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    same = (a == b) | (np.isnan(a) & np.isnan(b)) if a.dtype.kind == "f" else (a == b)
    if not np.all(same):
        idx = np.argwhere(~same)[:5]
        raise AssertionError(f"{what}: {int((~same).sum())} of {a.size} differ, first at {idx.tolist()}: "
                             f"{a[tuple(idx[0])]!r} vs {b[tuple(idx[0])]!r}")


def uneven_split(sn, sz, rp, ci, v, b):
    """Per-system views (row_ptrs, col_idxs, values, b) of a concatenated uneven batch."""
    out = []
    ro = zo = 0
    for s in range(len(sn)):
        n, nz = int(sn[s]), int(sz[s])
        out.append((rp[ro + s: ro + s + n + 1], ci[zo: zo + nz], v[zo: zo + nz], b[ro: ro + n]))
        ro += n
        zo += nz
    return out


def oracle_uneven(sn, sz, rp, ci, v, b, precond=0, approach=1, tol_mode=0, tol=1e-11, max_iter=500, fp32=False):
    """Oracle per system (each its own pattern); concatenated outputs."""
    xs, its, cvs, rss, trs, sts = [], [], [], [], [], []
    for (r, c, vv, bb) in uneven_split(sn, sz, rp, ci, v, b):
        o = oracle_pipeline(r, c, vv[None, :], bb[None, :], precond, approach=approach, tol_mode=tol_mode, tol=tol,
                            max_iter=max_iter, fp32=fp32)
        xs.append(o["x"][0]); its.append(o["iters"][0]); cvs.append(o["conv"][0]); rss.append(o["res"][0])
        trs.append(o["true_res"][0]); sts.append(o["status"][0])
    return {"x": np.concatenate(xs), "iters": np.array(its, np.float32), "conv": np.array(cvs, np.int32),
            "res": np.array(rss), "true_res": np.array(trs), "status": np.array(sts, np.int32)}
