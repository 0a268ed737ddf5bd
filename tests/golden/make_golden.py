"""Generates the golden fixtures tests/golden/ref_*.npz from the reference's own kernels.

  python tests/golden/make_golden.py [outdir]      (needs a GPU and oracle/_ref built)

Inputs are the seeded synthetic workloads (regenerated by the tests from
family / nsys / seed; a checksum of the values guards against generator
drift).  Outputs are those of the reference kernels compiled from its sources:
the merged ILU(0) solver (solution, half-iteration counts, flags, recursive and
true residual norms, in-kernel factors), ILU(0) approach 4, ISAI of L and U
(on the numeric pattern of page 0) and the ILU-ISAI solver.
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
for sub in ("merging-ilu0_gb300", "oracle", "tests"):
    sys.path.insert(0, os.path.join(ROOT, sub))

CASES = [("2d5_8x8", 8), ("2d5_16x16", 3), ("cd2d_12x12", 4), ("3d7_5x5x5", 6)]


def checksum(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main(outdir):
    import torch
    import helpers as H
    import oracle as O
    import ref as R
    dev = torch.device("cuda:0")
    os.makedirs(outdir, exist_ok=True)
    for fam, nsys in CASES:
        rp, ci, v, b = H.workload(fam, nsys)
        m = R.merged_solve(dev, rp, ci, v, b)
        a4 = R.ilu0(dev, rp, ci, v, 4)
        lu3 = O.ilu0(rp, ci, v, 3)  # factors fed to the ISAI kernels (approach 3 spins, so it is not run)
        lrp, lci, urp, uci = O.split_pattern(rp, ci)
        Lv, Uv = O.split_values(rp, ci, lu3)
        arp, aci = O.isai_pattern(lrp, lci, 2, Lv[0])
        brp, bci = O.isai_pattern(urp, uci, 2, Uv[0])
        ail = R.isai(dev, lrp, lci, Lv, 0, arp, aci)
        aiu = R.isai(dev, urp, uci, Uv, 1, brp, bci)
        s = R.isai_solve(dev, rp, ci, v, b, (arp, aci, ail), (brp, bci, aiu))
        np.savez_compressed(os.path.join(outdir, f"ref_{fam}.npz"), family=fam, nsys=nsys, seed=H.SEED,
                            input_sha256=checksum(rp, ci, v, b),
                            merged_x=m["x"], merged_iters=m["iters"], merged_conv=m["conv"], merged_res=m["res"],
                            merged_true_res=m["true_res"], merged_lu=m["lu"], ilu_app4=a4,
                            isai_L=ail, isai_U=aiu, isai_x=s["x"], isai_iters=s["iters"], isai_conv=s["conv"],
                            isai_res=s["res"])
        print(fam, nsys, "iters", m["iters"].tolist(), "isai iters", s["iters"].tolist())


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
