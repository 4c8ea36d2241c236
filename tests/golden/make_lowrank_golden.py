"""
Generate tests/golden/lowrank_n2000.npz by running the reference implementation itself on the low-rank case of
tests/strong_inputs.py (LR2000): fasterlmm.lowrank.loco_scan_lowrank (fasterlmm/lowrank.py:320-359) with a
400-marker kinship factor (LOCO ranks ~300 < N = 2,000), and single_k_scan_lowrank (lowrank.py:362-373).

Usage (in a checkout where the reference is present):
    python tests/golden/make_lowrank_golden.py [--reference PATH]

The inputs are not stored (tests/strong_inputs.py regenerates them; genotype checksums guard that).  Both factor and
test genotypes are standardised by the reference's io.standardise_columns; the fixture holds its FP64 outputs f,
beta, se, sfve, nullh2 and max_F for the LOCO scan and, prefixed sk_, for the single-kinship scan.
"""
from __future__ import annotations

import argparse
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE))

from make_golden import _import_reference, _res_dict  # noqa: E402
from strong_inputs import LR2000, genotype_checksum, lowrank_dataset  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("FASTERLMM_REFERENCE", ""))
    args = ap.parse_args()
    if not args.reference:
        sys.exit("pass --reference PATH (or set FASTERLMM_REFERENCE) to the reference checkout")
    core, fio, perms, torch = _import_reference(args.reference)
    import fasterlmm.lowrank as lowrank
    c = LR2000
    G, X, Y, chrom, Gk, chrom_kin = lowrank_dataset(c)
    Z = fio.standardise_columns(torch.from_numpy(G.astype(np.float64)))
    Zk = fio.standardise_columns(torch.from_numpy(Gk.astype(np.float64)))
    Xt, Yt = torch.from_numpy(X.copy()), torch.from_numpy(Y.copy())
    B = len(c["specs"])
    res = lowrank.loco_scan_lowrank(Zk, chrom_kin, Z, chrom, Xt, Yt, n_real=B)
    res1 = lowrank.single_k_scan_lowrank(Zk, Z, Xt, Yt, n_real=B)
    out = _res_dict(res)
    out.update({"sk_" + k: v for k, v in _res_dict(res1).items()})
    np.savez_compressed(HERE / "lowrank_n2000.npz", g_checksum=np.int64(genotype_checksum(G)),
                        gk_checksum=np.int64(genotype_checksum(Gk)), X=X, Y=Y, n_real=B, **out)
    print("wrote", HERE / "lowrank_n2000.npz", "max F", float(out["f"].max()))


if __name__ == "__main__":
    main()
