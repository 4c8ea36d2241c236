"""
Output files (fasterlmm_gb300.output) against the reference's own writer: tests/golden/output_files.npz holds the
files fasterlmm.cli._write_pheno wrote for seeded result columns (tests/golden/make_output_golden.py).  The text
routes must match byte for byte; the parquet bundle column for column.  CPU only: the writer is host code of the
library, which loads without a GPU.
"""
from __future__ import annotations

import numpy as np
import pytest


@pytest.fixture(scope="module")
def built():
    from fasterlmm_gb300 import build
    return build()


@pytest.fixture(scope="module")
def gold(golden):
    return golden("output_files")


def _ctx(g):
    from fasterlmm_gb300.output import VariantTable
    return VariantTable.of(list(g["snp"]), g["chrom"], g["pos"], g["g_var"], int(g["n_perm"]))


def _cols(g, j):
    return dict(p_col=g["p"][:, j], beta_col=g["beta"][:, j], se_col=g["se"][:, j], sfve_col=g["sfve"][:, j],
                nullh2_col=g["nullh2"][:, j])


FILES = ("gwas.tsv", "perms.tsv", "threshold.txt", "lambda_gc.txt")


def test_per_pheno_files_match_reference_bytes(built, gold, tmp_path):
    from fasterlmm_gb300.output import write_pheno
    ctx = _ctx(gold)
    rows = []
    for j, name in enumerate(gold["pheno"]):
        # (M, B) tables are passed as strided column views, as write_batch does
        write_pheno(ctx, str(tmp_path), str(name), **_cols(gold, j), p_var=float(gold["p_var"][j]),
                    perm_min_p=gold["perm_min_p"][j], perm_quantile=float(gold["perm_quantile"]),
                    per_pheno_dirs=True, bundle_writer=None, lambda_rows=rows)
        for fname in FILES:
            got = (tmp_path / str(name) / fname).read_bytes()
            want = bytes(gold[f"file_{j}_{fname}"])
            assert got == want, f"{name}/{fname} differs from the reference's file"
    assert [r[0] for r in rows] == [str(n) for n in gold["pheno"]]
    np.testing.assert_array_equal([r[1] for r in rows], gold["lambda"])
    np.testing.assert_array_equal([r[2] for r in rows], gold["lambda_n"])


def test_contiguous_columns_give_the_same_file(built, gold, tmp_path):
    from fasterlmm_gb300.output import write_gwas_tsv
    ctx = _ctx(gold)
    j = 2
    cols = {k: np.ascontiguousarray(v) for k, v in _cols(gold, j).items()}
    write_gwas_tsv(tmp_path / "g.tsv", ctx, str(gold["pheno"][j]), cols["p_col"], cols["beta_col"], cols["se_col"],
                   cols["sfve_col"], cols["nullh2_col"], float(gold["p_var"][j]))
    assert (tmp_path / "g.tsv").read_bytes() == bytes(gold[f"file_{j}_gwas.tsv"])


def test_bundle_matches_reference(built, gold, tmp_path):
    pytest.importorskip("pyarrow")
    import pyarrow.parquet as pq
    from fasterlmm_gb300.output import BUNDLE_COLUMNS, BundleWriter, write_pheno
    ctx = _ctx(gold)
    w = BundleWriter(tmp_path / "gwas_bundle.parquet")
    for j, name in enumerate(gold["pheno"]):
        write_pheno(ctx, str(tmp_path), str(name), **_cols(gold, j), p_var=float(gold["p_var"][j]),
                    perm_min_p=gold["perm_min_p"][j], perm_quantile=float(gold["perm_quantile"]),
                    per_pheno_dirs=False, bundle_writer=w)
    table = pq.read_table(w.close())
    assert table.column_names == list(gold["bundle_columns"]) == BUNDLE_COLUMNS
    assert [str(table.schema.field(c).type) for c in table.column_names] == list(gold["bundle_types"])
    for c in table.column_names:
        col = table.column(c)
        if c == "GenDist":
            assert col.null_count == len(col) and gold[f"bundle_{c}_nulls"].all()
        elif str(col.type) == "string":
            assert col.to_pylist() == list(gold[f"bundle_{c}"])
        else:
            np.testing.assert_array_equal(col.to_numpy(), gold[f"bundle_{c}"], err_msg=c)
    assert not (tmp_path / "gwas_bundle.parquet.tmp").exists()


# (value, text) pairs as pyarrow's CSV writer prints them: both sides of each notation switch, extremes, specials
KNOWN = [(0.1, "0.1"), (1.0, "1"), (-2.5, "-2.5"), (1e-5, "0.00001"), (1e-6, "0.000001"), (1e-7, "1e-7"),
         (1.5e-6, "0.0000015"), (1.2345e-7, "1.2345e-7"), (123456789.0, "123456789"), (1e9, "1000000000"),
         (9999999999.0, "9999999999"), (1e10, "1e+10"), (1.2345678901e10, "1.2345678901e+10"),
         (1.0000000000000002, "1.0000000000000002"), (5e-324, "5e-324"), (2.2250738585072014e-308,
         "2.2250738585072014e-308"), (1.7976931348623157e308, "1.7976931348623157e+308"), (1e21, "1e+21"),
         (0.0, "0"), (-0.0, "-0"), (float("nan"), "nan"), (float("inf"), "inf"), (float("-inf"), "-inf"),
         (0.000020332011720086887, "0.000020332011720086887"), (8.379874136692308e+15, "8.379874136692308e+15")]


def test_number_format_known_cases(built):
    from fasterlmm_gb300.output import format_f64
    got = format_f64([v for v, _ in KNOWN])
    assert got == [t for _, t in KNOWN]


def test_number_format_matches_pyarrow(built):
    pa = pytest.importorskip("pyarrow")
    import io

    import pyarrow.csv as pacsv
    from fasterlmm_gb300.output import format_f64
    rng = np.random.default_rng(7)
    with np.errstate(over="ignore"):
        v = np.concatenate([rng.standard_normal(40000) * 10.0 ** rng.uniform(-320, 308, 40000),
                            np.frombuffer(rng.bytes(8 * 20000), dtype=np.float64),
                            rng.uniform(0, 1, 20000) * 10.0 ** rng.integers(-9, 12, 20000)])
    b = io.BytesIO()
    pacsv.write_csv(pa.table({"x": v}), b, write_options=pacsv.WriteOptions(delimiter="\t", include_header=False,
                                                                           quoting_style="none"))
    want = b.getvalue().decode().split("\n")[:-1]
    assert format_f64(v) == want


def test_lambda_table(built, tmp_path):
    from fasterlmm_gb300.output import write_lambda_table
    rows = [("b", 1.25, 90), ("a", float("nan"), 0), ("c", 0.9876543219, 100)]
    p = write_lambda_table(tmp_path, None, rows, {"a": 0, "b": 1, "c": 2})
    assert p.name == "lambda_gc.tsv"
    assert p.read_text() == ("Pheno\tPhenoIndex\tLambdaGC\tNVariants\na\t0\t\t0\nb\t1\t1.250000\t90\n"
                             "c\t2\t0.987654\t100\n")
    assert write_lambda_table(tmp_path, 3, rows[:1], {"b": 1}).name == "lambda_gc.shard3.tsv"


def test_write_errors(built, gold, tmp_path):
    from fasterlmm_gb300 import _lib
    from fasterlmm_gb300.output import write_gwas_tsv
    ctx = _ctx(gold)
    cols = [np.ascontiguousarray(v) for v in _cols(gold, 0).values()]
    with pytest.raises(_lib.FlmmError) as e:
        write_gwas_tsv(tmp_path / "missing_dir" / "g.tsv", ctx, "x", *cols, 1.0)
    assert e.value.status == 7
    bad = np.arange(ctx.M, dtype=np.int64)
    bad[5] = ctx.M
    with pytest.raises(_lib.FlmmError) as e:
        write_gwas_tsv(tmp_path / "g.tsv", ctx, "x", *cols, 1.0, order=bad)
    assert e.value.status == 1
