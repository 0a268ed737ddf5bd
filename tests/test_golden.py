"""The oracle against golden outputs of the reference's own kernels
(tests/golden/ref_*.npz, made by tests/golden/make_golden.py on a GB300 from
kernels compiled out of the reference sources).  CPU only."""
import glob
import os

import numpy as np
import pytest

import helpers as H
import oracle as O

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_*.npz")))


@pytest.mark.skipif(not GOLD, reason="no golden fixtures")
@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p) for p in GOLD])
def test_oracle_matches_reference_golden(built, path):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(path), "make_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    g = np.load(path)
    fam, nsys = str(g["family"]), int(g["nsys"])
    rp, ci, v, b = H.workload(fam, nsys, int(g["seed"]))
    assert mk.checksum(rp, ci, v, b) == str(g["input_sha256"]), "generator drift: inputs differ from the fixture's"
    # merged ILU(0) solver (approach 1 factors, warp-0 inner products)
    lu = O.ilu0(rp, ci, v, 1)
    H.assert_bitwise(lu, g["merged_lu"], f"{fam}: in-kernel ILU(0)")
    r = O.bicgstab(rp, ci, v, b, prec=O.PREC_LU, lu=lu, dot=0)
    for f in ("x", "iters", "conv", "res"):
        H.assert_bitwise(r[f], g["merged_" + f], f"{fam}: merged solver {f}")
    H.assert_bitwise(O.true_residual(rp, ci, v, b, r["x"]), g["merged_true_res"], f"{fam}: true residual")
    H.assert_bitwise(O.ilu0(rp, ci, v, 4), g["ilu_app4"], f"{fam}: ILU(0) approach 4")
    # ISAI of approach-3 factors and the ILU-ISAI solver (serial inner products)
    lu3 = O.ilu0(rp, ci, v, 3)
    lrp, lci, urp, uci = O.split_pattern(rp, ci)
    Lv, Uv = O.split_values(rp, ci, lu3)
    arp, aci = O.isai_pattern(lrp, lci, 2, Lv[0])
    brp, bci = O.isai_pattern(urp, uci, 2, Uv[0])
    ail = O.isai_values(lrp, lci, Lv, 0, arp, aci)
    aiu = O.isai_values(urp, uci, Uv, 1, brp, bci)
    H.assert_bitwise(ail, g["isai_L"], f"{fam}: ISAI(L)")
    H.assert_bitwise(aiu, g["isai_U"], f"{fam}: ISAI(U)")
    s = O.bicgstab(rp, ci, v, b, prec=O.PREC_ISAI, ail=(arp, aci, ail), aiu=(brp, bci, aiu), dot=1)
    for f in ("x", "iters", "conv", "res"):
        H.assert_bitwise(s[f], g["isai_" + f], f"{fam}: ILU-ISAI solver {f}")
