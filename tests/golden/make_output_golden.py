"""
Generate tests/golden/output_files.npz: the files the reference CLI writes for a phenotype, made by the reference's
own writer (``fasterlmm.cli._write_pheno``, fasterlmm/cli.py:114-161) on seeded synthetic result columns.

Usage (in a checkout where the reference and pyarrow are present):
    python tests/golden/make_output_golden.py [--reference PATH]

The reference is imported from PATH (default: the FASTERLMM_REFERENCE environment variable); pandas, which
``fasterlmm.inflation`` imports at module top but the per-phenotype writer never calls, is replaced by an empty
stand-in package when it is not installed.  The writer context is built the way the CLI builds it
(fasterlmm/cli.py:248-252).  The result columns carry the values a scan produces at the edges: NaN p (NaN F),
p = 0 (underflow), tied p, p = 1, negative and tiny effects, the huge SE of a variant with no variance left, and
numbers on both sides of every switch between fixed and exponent notation.

The fixture stores the inputs and, per phenotype, the bytes of gwas.tsv, perms.tsv, threshold.txt and
lambda_gc.txt from the per-phenotype directory route, plus the streamed parquet bundle's columns (the bundle route,
fasterlmm/bundle.py:36-117) read back as arrays.
"""

from __future__ import annotations

import argparse
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _import_cli(path: str):
    import pyarrow as pa
    pa.array(["x"])  # pyarrow settles whether pandas is importable before the stand-in is on the path
    try:
        import pandas  # noqa: F401
    except ImportError:
        stub = Path(tempfile.mkdtemp()) / "pandas"
        stub.mkdir()
        (stub / "__init__.py").write_text("")
        sys.path.insert(0, str(stub.parent))
    sys.path.insert(0, path)
    import fasterlmm.bundle as bundle
    import fasterlmm.cli as cli
    return cli, bundle


def make_inputs(seed: int = 20240611) -> dict:
    rng = np.random.default_rng(seed)
    M, B, n_perm = 240, 3, 10
    chrom = np.repeat(np.arange(1, 5, dtype=np.float64), M // 4)
    pos = np.concatenate([np.sort(rng.choice(10**8, M // 4, replace=False)) for _ in range(4)]).astype(np.float64)
    snp = [f"chr{int(c)}_{int(p)}_{'ACGT'[i % 4]}_{'TGCA'[i % 4]}" for i, (c, p) in enumerate(zip(chrom, pos))]
    g_var = rng.uniform(0.05, 0.5, M)
    g_var[7] = 0.0  # monomorphic variant
    cols = {}
    for name in ("p", "beta", "se", "sfve", "nullh2"):
        cols[name] = np.empty((M, B))
    for b in range(B):
        p = 10.0 ** -rng.uniform(0, 12, M)
        p[rng.choice(M, 6, replace=False)] = np.nan          # NaN F
        p[rng.choice(M, 4, replace=False)] = 0.0             # underflow
        p[rng.choice(M, 5, replace=False)] = 0.125           # ties
        p[rng.choice(M, 3, replace=False)] = 1.0
        p[rng.choice(M, 3, replace=False)] = [1e-6, 1e-7, 9.99999e-7]
        beta = rng.normal(0, 1, M) * 10.0 ** rng.uniform(-9, 11, M)
        beta[7] = 0.0
        se = np.abs(rng.normal(0, 1, M)) * 10.0 ** rng.uniform(-3, 3, M)
        se[7] = 3.5e150  # sqrt(rWr / df / 1e-300), the reference's clamp
        sfve = rng.uniform(0, 1, M)
        sfve[7] = 0.0
        nullh2 = np.full(M, rng.uniform(0, 1))
        nullh2[M // 2:] = rng.uniform(0, 1)  # two chromosome groups with different fits
        for name, v in zip(("p", "beta", "se", "sfve", "nullh2"), (p, beta, se, sfve, nullh2)):
            cols[name][:, b] = v
    perm_min_p = 10.0 ** -rng.uniform(0, 9, (B, n_perm))
    perm_min_p[1, 3] = 0.0
    p_var = rng.uniform(0.5, 2.0, B)
    return dict(M=M, B=B, n_perm=n_perm, chrom=chrom, pos=pos, snp=np.array(snp), g_var=g_var,
                pheno=np.array(["height", "yield at 30C", "growth_rate"]), p_var=p_var, perm_min_p=perm_min_p,
                perm_quantile=0.05, **cols)


def run_reference(cli, bundle, inp: dict, outdir: Path) -> dict:
    import pyarrow as pa
    import pyarrow.parquet as pq
    M, n_perm = inp["M"], inp["n_perm"]
    ctx = {"snp_id": pa.array(list(inp["snp"]), type=pa.string()), "chrom": inp["chrom"], "pos": inp["pos"],
           "g_var": inp["g_var"], "sid_index": np.arange(M, dtype=np.int64), "gendist": pa.nulls(M, pa.float64()),
           "mixing": np.zeros(M), "phenocount": np.full(M, 1 + n_perm),
           "pheno_idx": pa.array(np.zeros(M, dtype=np.int32)), "lambda_rows": []}
    writer = bundle.BundleWriter(outdir / bundle.BUNDLE_FILENAME)
    for j, name in enumerate(inp["pheno"]):
        cli._write_pheno(ctx, str(outdir), str(name), p_col=inp["p"][:, j], beta_col=inp["beta"][:, j],
                         se_col=inp["se"][:, j], sfve_col=inp["sfve"][:, j], nullh2_col=inp["nullh2"][:, j],
                         p_var=float(inp["p_var"][j]), perm_min_p=inp["perm_min_p"][j],
                         perm_quantile=inp["perm_quantile"], per_pheno_dirs=True, bundle_writer=None)
        cli._write_pheno(ctx, str(outdir), str(name), p_col=inp["p"][:, j], beta_col=inp["beta"][:, j],
                         se_col=inp["se"][:, j], sfve_col=inp["sfve"][:, j], nullh2_col=inp["nullh2"][:, j],
                         p_var=float(inp["p_var"][j]), perm_min_p=inp["perm_min_p"][j],
                         perm_quantile=inp["perm_quantile"], per_pheno_dirs=False, bundle_writer=writer)
    path = writer.close()
    table = pq.read_table(path)
    out = {}
    for j, name in enumerate(inp["pheno"]):
        sub = outdir / str(name)
        for fname in ("gwas.tsv", "perms.tsv", "threshold.txt", "lambda_gc.txt"):
            out[f"file_{j}_{fname}"] = np.frombuffer((sub / fname).read_bytes(), dtype=np.uint8)
    # each phenotype was written twice (directory route, bundle route): one row per phenotype, in column order
    first = {}
    for r in ctx["lambda_rows"]:
        first.setdefault(r[0], r)
    rows = [first[str(n)] for n in inp["pheno"]]
    out["lambda"] = np.array([r[1] for r in rows])
    out["lambda_n"] = np.array([r[2] for r in rows])
    # the bundle: one row group per phenotype appended in call order; columns read back as arrays
    out["bundle_columns"] = np.array(table.column_names)
    for c in table.column_names:
        col = table.column(c)
        if pa.types.is_string(col.type):
            out[f"bundle_{c}"] = np.array(col.to_pylist())
        elif c == "GenDist":
            out[f"bundle_{c}_nulls"] = np.array([v is None for v in col.to_pylist()])
        else:
            out[f"bundle_{c}"] = col.to_numpy()
    out["bundle_types"] = np.array([str(table.schema.field(c).type) for c in table.column_names])
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("FASTERLMM_REFERENCE", ""))
    args = ap.parse_args()
    if not args.reference:
        sys.exit("pass --reference PATH or set FASTERLMM_REFERENCE")
    cli, bundle = _import_cli(args.reference)
    inp = make_inputs()
    with tempfile.TemporaryDirectory() as tmp:
        ref = run_reference(cli, bundle, inp, Path(tmp))
    np.savez_compressed(HERE / "output_files.npz", **inp, **ref)
    print("wrote", HERE / "output_files.npz")


if __name__ == "__main__":
    main()
