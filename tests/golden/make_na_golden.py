"""
Generate tests/golden/na_groups_n1600.npz by running the reference implementation itself on the NaN-group case of
tests/strong_inputs.py (NA1600): phenotypes in four missingness patterns, each pattern scanned on its own strain
subset as the CLI's grouped path does (fasterlmm/cli.py:351-375, fasterlmm/io.py:187-218), with one
``perm_threshold`` per (pattern, permutation count) -- the reference takes one count per run, so the three
phenotypes with forty permutations run apart from the rest of their pattern.

Usage (in a checkout where the reference is present):
    python tests/golden/make_na_golden.py [--reference PATH]

The inputs are not stored (tests/strong_inputs.py regenerates them; a genotype checksum guards that); for each run
r the fixture holds its strain rows and columns (r{r}_keep, r{r}_cols, r{r}_n_perm) and the reference's FP64
outputs f, beta, se, sfve, max_F, the permutation maxima and the per-chromosome log delta.
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
from strong_inputs import NA1600, genotype_checksum, na_dataset  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("FASTERLMM_REFERENCE", ""))
    args = ap.parse_args()
    if not args.reference:
        sys.exit("pass --reference PATH (or set FASTERLMM_REFERENCE) to the reference checkout")
    core, fio, perms, torch = _import_reference(args.reference)
    c = NA1600
    G, X, Y, chrom = na_dataset(c)
    Zf = G.astype(np.float64)
    data = fio.AlignedDataset(iid=[str(i) for i in range(Zf.shape[0])], Z=torch.from_numpy(Zf),
                              Y=torch.from_numpy(Y.copy()), X=torch.from_numpy(X.copy()), chrom=chrom,
                              pos=np.arange(Zf.shape[1]), snp_id=[str(i) for i in range(Zf.shape[1])],
                              pheno_names=[f"p{i}" for i in range(Y.shape[1])], Z_kin=None, chrom_kin=None)
    B = Y.shape[1]
    out, r = {}, 0
    for keep, cols in fio.group_by_na(data.Y, list(range(B))):
        counts: dict[int, list[int]] = {}
        for col in cols:
            counts.setdefault(int(c["n_perm_of"].get(col, c["n_perm"])), []).append(col)
        for n_perm, sel in counts.items():
            sub = fio.subset_dataset(data, keep, sel)
            with _DeltaRecorder(core) as rec:
                res, pmf = perms.perm_threshold(sub, list(range(len(sel))), n_perm=n_perm, seed=19930909,
                                                loco=True, seed_idx=sel)
            vals = {k: v for k, v in _res_dict(res).items() if k != "nullh2"}
            vals["perm_max_F"] = pmf.numpy()
            vals["log_delta"] = np.stack([cc[1].numpy() for cc in rec.calls])
            out.update({f"r{r}_{k}": v for k, v in vals.items()})
            out[f"r{r}_keep"] = np.asarray(keep, dtype=np.int32)
            out[f"r{r}_cols"] = np.asarray(sel, dtype=np.int32)
            out[f"r{r}_n_perm"] = np.int64(n_perm)
            print(f"run {r}: {len(keep)} samples, columns {sel}, {n_perm} permutations", flush=True)
            r += 1
    np.savez_compressed(HERE / "na_groups_n1600.npz", g_checksum=np.int64(genotype_checksum(G)), X=X, Y=Y,
                        n_runs=r, **out)
    print("wrote", HERE / "na_groups_n1600.npz")


if __name__ == "__main__":
    main()
