"""
Generate tests/golden/strong_n5000.npz by running the reference implementation itself on the N = 5,000
strong-association case of tests/strong_inputs.py (N5000).

Usage (in a checkout where the reference is present):
    python tests/golden/make_strong_golden.py [--reference PATH]

The inputs are not stored: tests/strong_inputs.py regenerates them bit for bit from numpy's PCG64 raw uniforms on
any host, and the fixture keeps a checksum of the genotypes so a host that produced different data fails loudly.
The fixture holds the reference's FP64 outputs of ``perm_threshold`` (LOCO over three chromosomes, ten
permutations per phenotype): f, beta, se, sfve, max_F, the permutation maxima and the fitted log delta of every
chromosome.
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

from make_golden import _DeltaRecorder, _import_reference, _res_dict  # noqa: E402
from strong_inputs import N5000, genotype_checksum, strong_dataset  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("FASTERLMM_REFERENCE", ""))
    args = ap.parse_args()
    if not args.reference:
        sys.exit("pass --reference PATH (or set FASTERLMM_REFERENCE) to the reference checkout")
    core, fio, perms, torch = _import_reference(args.reference)
    c = N5000
    G, X, Y, chrom = strong_dataset(c["N"], c["sizes"], c["D"], c["specs"], seed=c["seed"])
    Zf = G.astype(np.float64)
    data = fio.AlignedDataset(iid=[str(i) for i in range(Zf.shape[0])], Z=torch.from_numpy(Zf),
                              Y=torch.from_numpy(Y.copy()), X=torch.from_numpy(X.copy()), chrom=chrom,
                              pos=np.arange(Zf.shape[1]), snp_id=[str(i) for i in range(Zf.shape[1])],
                              pheno_names=[f"p{i}" for i in range(Y.shape[1])], Z_kin=None, chrom_kin=None)
    B = Y.shape[1]
    with _DeltaRecorder(core) as rec:
        res, pmf = perms.perm_threshold(data, list(range(B)), n_perm=c["n_perm"], seed=19930909, loco=True)
    out = {k: v for k, v in _res_dict(res).items() if k != "nullh2"}
    out["perm_max_F"] = pmf.numpy()
    out["log_delta"] = np.stack([cc[1].numpy() for cc in rec.calls])
    np.savez_compressed(HERE / "strong_n5000.npz", g_checksum=np.int64(genotype_checksum(G)), X=X, Y=Y,
                        n_perm=c["n_perm"], **out)
    print("wrote", HERE / "strong_n5000.npz", "max F", float(out["f"].max()))


if __name__ == "__main__":
    main()
