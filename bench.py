#!/usr/bin/env python
"""
Benchmark of the batched LMM association scan (FaST-ER-LMM's perm_threshold -> loco_scan_compat path) on GB300.

Metric: variant-phenotype tests per second, tests = M variants x B phenotypes x (1 + n_perm) (the reference's
"Wald ops", fasterlmm/watch.py:194-199).  Workload: 1,000 samples x 100,000 variants over 20 chromosomes, 6,484
phenotypes x 10 permutations (71,324 scan columns), 5 covariate columns, seeded synthetic inputs.

One step = one full permutation scan of that workload through fasterlmm_gb300.perms.perm_threshold: standardise,
per-chromosome kinship Grams, the batched eigendecomposition of the 20 LOCO kinships, then 20 x (rotations, delta
fit, fused Wald scan), permutation orders drawn per step.  ``value`` times steps with the inputs already on the
device; ``e2e`` times the same call with host (pinned) inputs and host outputs, copies included.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form fast|plain] [--impl ours|reference]
                  [--delta grid|learned] [--no-pipeline] [--B B] [--M M] [--no-e2e] [--no-cpu-baseline]
                  [--no-plain] [--plain-chroms C] [--workload headline|c3|c5]

Besides ``value`` and ``e2e`` the line carries the metric's own ratio (``chosen_vs_plain``: the plain FP64 form and
the chosen form timed on the same bounded subset of the workload, its first C chromosomes), the real-only rate,
the fused Wald kernel's roofline on the tensor pipe and in HBM bytes, the delta fit's FP32 roofline and per-stage
times of one step with nothing overlapped.

``--delta learned`` switches the fast form's delta fit to the learned proposal's narrow bracket; ``--no-pipeline``
runs each chromosome's delta fit on the main stream instead of one chromosome ahead on a side stream.

``--workload c3`` runs the uneven-batching shape instead: 5,000 samples x 500,000 variants over 22 chromosomes of
human proportions, 2,000 phenotypes in 12 missingness patterns (groups of 3,000-5,000 samples), 1,000 permutations
for 50 phenotypes and 10 for the rest, every group on its own strain subset (fasterlmm_gb300.groups).

``--workload c5`` runs the low-rank large-cohort shape (fasterlmm_gb300.lowrank_fast): 50,000 samples, a 2,000-marker
kinship factor, 100 phenotypes x (1 + 10 permutations), int8 genotypes streamed from pinned host memory in 8,192-
variant blocks (200,000 tested variants by default, --M up to 1,000,000).

``--impl reference`` times the reference's own CPU path on the host's cores on a bounded sample of the same workload
(one chromosome x one 256-phenotype batch per step): the reference package's functions in FP64 torch where it is
installed under baseline/_ref, else the CPU restatement of its algorithm (oracle/flmm_oracle.py).  The line's
``cpu_baseline`` is the same measurement inside the GPU run.
Under torchrun (N > 1) every rank runs its own replica of the workload (the scan has no cross-GPU exchange) and
the line reports the total over ranks against the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path
from types import SimpleNamespace

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "fast-er-lmm_gb300", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

WORKLOAD = "n1000_m100k_b6484_perm10"
METRIC = "variant-phenotype tests/s, 1 GB300: chosen vs plain form at |Δ-log10p|≤1e-3"
UNIT = "tests/s"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int) -> float:
    """The slowest rank's value (the job's time), over the initialised process group when world > 1."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.device_index = device_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs"), "tensor_tflops": d.get("bf16_tflops"),
                "tensor_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "tensor_tflops": 1900.0, "tensor_tflops_sustained": 1700.0, "source": "fallback"}


# --workload: the headline shape, or the uneven-batching shape (5,000 samples x 500,000 variants over 22
# human-sized chromosomes, 2,000 phenotypes in 12 missingness patterns, 1,000 permutations for 50 of them and 10
# for the rest)
WORKLOADS = {"headline": WORKLOAD, "c3": "n5000_m500k_b2000_na12", "c5": "n50000_k2000_m1m_b100_perm10"}


def make_inputs(B: int | None, M: int | None, name: str = WORKLOAD):
    from fasterlmm_gb300.synth import make_workload
    d, w = make_workload(name, B=B, M=M)
    return d, w


# ---- CPU baseline: the reference (or the oracle) on a bounded sample ---------------------------------------------

REF_DIR = ROOT / "baseline" / "_ref"


def _reference_modules():
    """
    The reference package itself (pure Python/torch), installed under baseline/_ref by the one offline install
    ``pip install --no-deps --target baseline/_ref <reference checkout>``; None where it is absent.  Its modules
    fasterlmm.io and fasterlmm.normalize import pandas at module top although the scan never calls it; where
    pandas is not installed an empty stand-in module serves the import and is removed again afterwards.
    """
    if not (REF_DIR / "fasterlmm" / "core.py").exists():
        return None
    stub = None
    try:
        import pandas  # noqa: F401
    except ImportError:
        import types
        stub = sys.modules["pandas"] = types.ModuleType("pandas")
    if str(REF_DIR) not in sys.path:
        sys.path.insert(0, str(REF_DIR))
    try:
        import fasterlmm.core as ref_core
        import fasterlmm.io as ref_io
    except Exception:  # an install that does not import here (another Python, a missing dependency)
        return None
    finally:
        if stub is not None and sys.modules.get("pandas") is stub:
            del sys.modules["pandas"]
    return ref_core, ref_io


def cpu_sample_run(d, w, B_sample: int, chrom_id: int = 1, ref=None) -> tuple[float, int]:
    """
    One CLI-sized batch (B_sample phenotypes + their permutations) through one LOCO chromosome on the CPU: the
    kinship without the chromosome, the compat rotation, the delta fit and the Wald scan of its variants
    (fasterlmm/core.py:712-716).  ``ref`` = (fasterlmm.core, fasterlmm.io) runs the reference's own functions in
    FP64 torch on the host threads; None runs the oracle's numpy restatement.  Standardisation and the
    permutation packing happen before the clock starts.
    """
    import flmm_oracle as orc
    Zn = orc.standardise_columns(d.Z_float())
    n_perm = w["n_perm"]
    orders = orc.perm_orders(Zn.shape[0], range(B_sample), n_perm)
    Y_all = orc.pack_perms(d.Y[:, :B_sample], orders)
    mask = d.chrom == chrom_id
    tests = int(mask.sum()) * B_sample * (1 + n_perm)
    grid_kw = dict(n_grid=w["n_grid"], log_delta_min=w["log_delta_min"], log_delta_max=w["log_delta_max"])
    if ref is not None:
        import torch
        core, fio = ref
        Z = torch.from_numpy(np.ascontiguousarray(Zn))
        X = torch.from_numpy(np.ascontiguousarray(d.X))
        Yt = torch.from_numpy(np.ascontiguousarray(Y_all))
        Zk = Z[:, torch.from_numpy(~mask)].contiguous()
        Zc = Z[:, torch.from_numpy(mask)].contiguous()
        t0 = time.perf_counter()
        K = fio.grm(Zk)
        spec = core.fastlmm_compat_rotate(K, X, Yt)
        ld = core.fit_delta_grid_compat(spec, **grid_kw)
        core.snp_wald_scan_compat(spec, ld, Zc, n_real=B_sample)
        return time.perf_counter() - t0, tests
    t0 = time.perf_counter()
    K = orc.grm(Zn[:, ~mask])
    spec = orc.compat_rotate(K, d.X, Y_all)
    ld = orc.fit_delta_grid_compat(spec["s"], spec["UY"], **grid_kw)
    orc.snp_wald_scan_compat(spec, ld, Zn[:, mask], n_real=B_sample)
    return time.perf_counter() - t0, tests


def _host_cores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def _cpu_kind():
    """(kind, ref modules, description) of the CPU path the baseline times."""
    ref = _reference_modules()
    if ref is not None:
        return "reference", ref, "the reference's own fasterlmm.core / fasterlmm.io functions, FP64 torch"
    return "port", None, "the oracle's numpy FP64 restatement (the reference is not installed here)"


class _TorchThreads:
    """torch's intra-op thread count set to the host's cores for the duration (the reference CLI's --device cpu
    setting, fasterlmm/cli.py:221), then put back."""

    def __init__(self, n: int):
        self.n = n

    def __enter__(self):
        import torch
        self.prev = torch.get_num_threads()
        torch.set_num_threads(self.n)

    def __exit__(self, *exc):
        import torch
        torch.set_num_threads(self.prev)


def cpu_baseline(d, w, target_s: float = 12.0) -> dict:
    B_sample = min(256, w["B"])
    total_t, total_tests, runs = 0.0, 0, 0
    chroms = sorted(np.unique(d.chrom).tolist())
    cores = _host_cores()
    kind, ref, what = _cpu_kind()
    with _TorchThreads(cores):
        while total_t < target_s and runs < len(chroms):
            dt, n = cpu_sample_run(d, w, B_sample, chroms[runs], ref)
            total_t += dt
            total_tests += n
            runs += 1
    return {"value": total_tests / total_t, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"{runs} LOCO chromosome(s) x one {B_sample}-phenotype batch with {w['n_perm']} permutations each "
                      f"(GRM, compat rotation, 64-point grid + golden section, Wald) through {what} on {cores} host "
                      f"threads; {total_tests} tests in {total_t:.1f} s"}


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    d, w = make_inputs(args.B, args.M)
    B_sample = min(256, w["B"])
    chroms = sorted(np.unique(d.chrom).tolist())
    cores = _host_cores()
    kind, ref, what = _cpu_kind()
    times, tests = [], []
    with _TorchThreads(cores):
        for i in range(args.warmup):
            cpu_sample_run(d, w, B_sample, chroms[i % len(chroms)], ref)
        for i in range(args.steps):
            dt, n = cpu_sample_run(d, w, B_sample, chroms[i % len(chroms)], ref)
            times.append(dt)
            tests.append(n)
    value = sum(tests) / sum(times)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "N": w["N"], "M": w["M"], "B": w["B"], "n_perm": w["n_perm"],
                       "step": f"one LOCO chromosome x one {B_sample}-phenotype batch (+{w['n_perm']} perms each)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"one chromosome x {B_sample} phenotypes per step through {what}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- GPU arm ----------------------------------------------------------------------------------------------------

def run_ours(args):
    import torch
    rank, world, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from fasterlmm_gb300 import _lib, build, fast, perms
    build()
    if args.delta is not None:
        fast.DELTA_PROPOSAL = args.delta
    if args.no_pipeline:
        fast.PIPELINE = False
    d, w = make_inputs(args.B, args.M)
    N, M, B, n_perm = w["N"], w["M"], w["B"], w["n_perm"]
    P = B * (1 + n_perm)
    tests_per_step = M * B * (1 + n_perm)
    grid_kw = dict(n_grid=w["n_grid"], log_delta_min=w["log_delta_min"], log_delta_max=w["log_delta_max"])
    host_bufs = e2e_buffers(d, w) if (rank == 0 and world == 1 and not args.no_e2e) else None
    Zf = d.Z_float()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))
    data_dev = SimpleNamespace(Z=t(Zf).to(dev), Y=t(d.Y).to(dev), X=t(d.X).to(dev), chrom=d.chrom, Z_kin=None,
                               chrom_kin=None)
    pheno = list(range(B))

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    timers: dict = {}

    def step(tm=None):
        return perms.perm_threshold(data_dev, pheno, n_perm=n_perm, form=args.form, timers=tm, **grid_kw)

    for _ in range(args.warmup):
        step()
    barrier()
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    launches0 = _lib.kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        res, pmf = step(timers)
        del res, pmf
    ev1.record()
    barrier()
    wall = time.perf_counter() - w0
    launches = _lib.kernel_launches() - launches0
    clk = clocks.stop()
    elapsed = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, world)
    value = world * tests_per_step * args.steps / elapsed

    # dominant kernel: the fused Wald scan, timed by events around its launches inside the timed steps
    wald_ms = [a.elapsed_time(b) for a, b in timers.get("wald", []) if b is not None]
    peaks = measured_peaks()
    Neff = N - w["D"]
    mc_mean = M / w["n_chrom"]
    roof = None
    if wald_ms:
        from fasterlmm_gb300.fast import interp_nodes
        mean_s = statistics.mean(wald_ms) / 1e3
        alg_flop = 4.0 * Neff * P * mc_mean
        achieved = alg_flop / mean_s / 1e12
        # what the tensor pipe executes: sWy (K = Neff) and the interpolated sWs (K = R nodes), three split products
        R = interp_nodes(w["log_delta_min"], w["log_delta_max"])[1]
        exec_flop = 3 * 2.0 * (Neff + R) * P * mc_mean
        peak = peaks["tensor_tflops"]
        # DRAM bytes per launch from the committed ncu summary of this workload (measured at full size)
        traffic = None
        tp = ROOT / "profiles" / f"wald_k_pair2_{WORKLOAD}.md"
        if tp.exists() and args.B is None and args.M is None and args.form == "fast":
            for line in tp.read_text().splitlines():
                if line.startswith("traffic_bytes_per_launch:"):
                    traffic = int(line.split(":")[1])
        # algorithmic HBM bytes of one launch: the split FP16 hi/lo operands read once (columns: w~ o UY over Neff
        # and the Lagrange weights over R; variants: US over Neff and the sWs node table over R) and the FP64
        # detail of the real columns (f, beta, se, sfve) written once
        ldk, ldr = -(-Neff // 8) * 8, -(-R // 8) * 8
        alg_bytes = 4.0 * P * (ldk + ldr) + 4.0 * mc_mean * (ldk + ldr) + 32.0 * mc_mean * B
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": "k_pair<2> (fused split-FP16 Wald, tcgen05 CTA pairs)", "launch_ms": 1e3 * mean_s,
                "algorithmic_flop_per_launch": alg_flop, "executed_flop_per_launch": exec_flop,
                "executed_tensor_frac": exec_flop / mean_s / 1e12 / peak,
                "peak_source": peaks["source"] + " bf16 dense (FP16 rate is the same)",
                "hbm": {"algorithmic_bytes_per_launch": alg_bytes, "achieved_gbs": alg_bytes / mean_s / 1e9,
                        "measured_gbs": None if traffic is None else traffic / mean_s / 1e9,
                        "peak_gbs": peaks["hbm_gbs"], "frac": alg_bytes / mean_s / 1e9 / peaks["hbm_gbs"],
                        "note": "fused: ~1e3 flop per HBM byte, so the tensor pipe binds, not HBM"}}

    # the phenotype rotation UY = U_eff^T Y_r per chromosome (split-FP16 tcgen05 GEMM): 2 N Neff P algorithmic flop
    rot_ms = [a.elapsed_time(b) for a, b in timers.get("rotate", []) if b is not None]
    rotation = None
    if rot_ms:
        mean_s = statistics.mean(rot_ms) / 1e3
        alg = 2.0 * N * Neff * P
        rotation = {"kernel": "k_pair<1> (split-FP16 GEMM, UY = U_eff^T Y_r)", "launch_ms": 1e3 * mean_s,
                    "algorithmic_tflops": alg / mean_s / 1e12, "frac": alg / mean_s / 1e12 / peaks["tensor_tflops"],
                    "executed_tensor_frac": 3 * alg / mean_s / 1e12 / peaks["tensor_tflops"],
                    "peak_source": peaks["source"] + " bf16 dense"}
    stages = {k: round(sum(a.elapsed_time(b) for a, b in v if b is not None) / args.steps, 3)
              for k, v in timers.items()}

    iso = isolated_stages(args, step, w) if (args.form == "fast" and rank == 0) else None
    delta_roof = None
    if iso and iso.get("delta"):
        # per chromosome: the FP32 grid product (G x Neff) x (Neff x P), 2 flop per term, and the Newton passes,
        # ~30 FP32 operations per element for each of ~4.5 evaluations of a column
        d_s = iso["delta"] / w["n_chrom"] / 1e3
        grid_flop = 2.0 * w["n_grid"] * Neff * P
        newton_flop = 30.0 * 4.5 * Neff * P
        fp32_peak = fp32_peak_tflops()
        delta_roof = {"kernels": "k_grid_argmin_f32 + k_newton_refine (FP32 pipe)", "ms_per_chromosome": 1e3 * d_s,
                      "algorithmic_flop": grid_flop + newton_flop, "grid_flop": grid_flop,
                      "achieved_tflops": (grid_flop + newton_flop) / d_s / 1e12, "peak_tflops": fp32_peak,
                      "frac": (grid_flop + newton_flop) / d_s / 1e12 / fp32_peak,
                      "peak_source": "nominal FP32 CUDA-core rate: SMs x 128 lanes x 2 flop x max SM clock",
                      "timed": "one untimed step with the delta fit on the main stream (not overlapped)"}
    plain = None
    if rank == 0 and world == 1 and args.form == "fast" and not args.no_plain:
        plain = plain_comparison(args, d, w, grid_kw)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "fp16x2-split tensor (FP32 acc) + f64" if args.form == "fast" else "f64",
            "data": "synthetic (seeded: Binomial(2, MAF~U[0.01,0.5]) genotypes, RINT phenotypes, 0-50 causal)",
            "config": {"workload": WORKLOAD, "N": N, "M": M, "B": B, "n_perm": n_perm, "P": P, "chromosomes": w["n_chrom"],
                       "covariates": w["D"], "grid": w["n_grid"], "form": args.form,
                       "delta_fit": fast.DELTA_PROPOSAL, "pipelined_delta_fit": bool(fast.PIPELINE),
                       "l2": "inputs larger than L2 (Z 0.8 GB FP64, operands >100 MB per chromosome)",
                       "parallelism": f"{world} replica(s), no cross-GPU exchange"},
            "real_tests_per_s": value * B / P,
            "wall_s_timed": wall, "gpu_launches": launches, "roofline": roof, "rotation_roofline": rotation,
            "delta_roofline": delta_roof, "chosen_vs_plain": plain,
            "stage_ms_per_step": stages, "stage_ms_isolated": iso, "autotune": _lib.autotune_report(), "clocks": clk}

    data_dev = None  # the e2e leg starts from host data only
    if host_bufs is not None:
        line["e2e"] = e2e_leg(args, w, pheno, grid_kw, *host_bufs)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(d, w)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_grouped(args):
    """
    The uneven-batching workload: every missingness group scanned on its own strain subset through
    fasterlmm_gb300.groups.perm_threshold_grouped, each group's two permutation counts in one joint scan.  One step =
    the whole grouped permutation scan; inputs on the device (int8 dosages uploaded and widened there once).
    """
    import torch
    rank, world, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from fasterlmm_gb300 import _lib, build, fast
    from fasterlmm_gb300.groups import group_by_na, perm_threshold_grouped
    build()
    if args.no_pipeline:
        fast.PIPELINE = False
    name = WORKLOADS[args.workload]
    t_gen = time.perf_counter()
    d, w = make_inputs(args.B, args.M, name)
    t_gen = time.perf_counter() - t_gen
    N, M, B, n_perm, D = w["N"], w["M"], w["B"], w["n_perm"], w["D"]
    n_perm_of = {b: w["n_perm_hi"] for b in range(min(w.get("B_hi", 0), B))}
    groups = [(keep, cols) for keep, cols in group_by_na(d.Y, range(B)) if len(keep) - D - 1 >= 1]
    P_of = [sum(1 + n_perm_of.get(b, n_perm) for b in cols) for _, cols in groups]
    tests_per_step = M * sum(P_of)
    grid_kw = dict(n_grid=w["n_grid"], log_delta_min=w["log_delta_min"], log_delta_max=w["log_delta_max"])
    G = torch.from_numpy(d.G).to(dev)
    Z = G.to(torch.float64)
    Z[G < 0] = float("nan")
    del G
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    data_dev = SimpleNamespace(Z=Z, Y=t(d.Y), X=t(d.X), chrom=d.chrom, Z_kin=None, chrom_kin=None)

    def step(tm=None):
        return perm_threshold_grouped(data_dev, list(range(B)), n_perm=n_perm, n_perm_of=n_perm_of, form=args.form,
                                      timers=tm, **grid_kw)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    launches0 = _lib.kernel_launches()
    timers: dict = {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        out = step(timers)
        del out
    ev1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    launches = _lib.kernel_launches() - launches0
    clk = clocks.stop()
    elapsed = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, world)
    value = world * tests_per_step * args.steps / elapsed
    stages = {k: round(sum(a.elapsed_time(b) for a, b in v if b is not None) / args.steps, 3)
              for k, v in timers.items()}
    # the fused Wald launches of a step: 4 Neff_g P_g Mc algorithmic flop each, summed over groups and chromosomes
    peaks = measured_peaks()
    wald_s = sum(a.elapsed_time(b) for a, b in timers.get("wald", []) if b is not None) / 1e3 / args.steps
    wald_flop = sum(4.0 * (len(keep) - D) * Pg * M for (keep, _), Pg in zip(groups, P_of))
    roof = None
    if wald_s > 0:
        ach = wald_flop / wald_s / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": peaks["tensor_tflops"], "unit": "TFLOP/s",
                "frac": ach / peaks["tensor_tflops"], "traffic": None,
                "kernel": "k_pair<2> (fused split-FP16 Wald, tcgen05 CTA pairs), all launches of a step",
                "wald_ms_per_step": 1e3 * wald_s, "algorithmic_flop_per_step": wald_flop,
                "peak_source": peaks["source"] + " bf16 dense (FP16 rate is the same)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "fp16x2-split tensor (FP32 acc) + f64" if args.form == "fast" else "f64",
            "data": "synthetic (seeded: Binomial(2, MAF~U[0.01,0.5]) genotypes, RINT phenotypes, 0-50 causal, "
                    f"{len(groups)} missingness patterns)",
            "config": {"workload": name, "N": N, "M": M, "B": B, "n_perm": n_perm,
                       "n_perm_hi": w.get("n_perm_hi"), "B_hi": len(n_perm_of), "chromosomes": w["n_chrom"],
                       "covariates": D, "grid": w["n_grid"], "form": args.form,
                       "groups": [{"samples": len(keep), "phenotypes": len(cols), "columns": Pg}
                                  for (keep, cols), Pg in zip(groups, P_of)],
                       "columns": sum(P_of), "pipelined_delta_fit": bool(fast.PIPELINE),
                       "l2": "inputs larger than L2 (Z 20 GB FP64)",
                       "parallelism": f"{world} replica(s), no cross-GPU exchange"},
            "wall_s_timed": wall, "gpu_launches": launches, "roofline": roof, "stage_ms_per_step": stages,
            "generate_s": round(t_gen, 1), "e2e": None, "cpu_baseline": None,
            "notes": "device-resident inputs; no e2e leg and no CPU sample for this shape (one N=5,000 LOCO GRM "
                     "alone is ~2e13 flop on the host)",
            "clocks": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_lowrank(args):
    """
    The low-rank large-cohort shape through fasterlmm_gb300.lowrank_fast: 50,000 samples, a 2,000-marker kinship
    factor, tested variants (int8 dosages in pinned host memory) streamed to the device in 8,192-variant blocks
    while the previous block is scanned, 100 phenotypes x (1 + 10 permutations).  One step = the whole LOCO scan:
    22 per-chromosome bases (FP64 k x k eigendecompositions), phenotype rotations and FP64 delta fits, and every
    block's split-FP16 products and fused Wald.  The tested-variant count defaults to 200,000 (10 GB of dosages on
    the host; --M sets it, up to the spec's 1,000,000).
    """
    import torch
    rank, world, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from fasterlmm_gb300 import _lib, build, lowrank_fast, perms
    from fasterlmm_gb300.core import _ptr, transpose
    from fasterlmm_gb300.synth import make_lowrank_workload
    build()
    name = WORKLOADS[args.workload]
    t_gen = time.perf_counter()
    d, w = make_lowrank_workload(name, M=args.M or 200_000, B=args.B)
    t_gen = time.perf_counter() - t_gen
    N, k, M, B, n_perm, D = w["N"], w["k_kin"], w["M"], w["B"], w["n_perm"], w["D"]
    P = B * (1 + n_perm)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    Gkt = t(d.Gk.T)                                                   # (k, N) int8, marker-major
    Zkt = torch.empty((k, N), dtype=torch.float64, device=dev)
    _lib.call("flmm_standardise_dosage", _ptr(Gkt), N, N, k, _ptr(Zkt), N, None)
    Gk_std = transpose(Zkt)                                           # (N, k) standardised factor
    orders = torch.from_numpy(perms.perm_orders(N, range(B), n_perm)).to(dev)
    Yt_all = perms.pack_perm_columns(transpose(t(d.Y)), orders)
    Y_all = transpose(Yt_all)                                         # (N, P): reals, then permutations
    X = t(d.X)
    Gt_host = torch.from_numpy(d.Gt).pin_memory()
    del d.Gt
    rows_of = {int(c): np.flatnonzero(d.chrom == c) for c in np.unique(d.chrom)}
    chroms = sorted(rows_of)
    grid_kw = dict(n_grid=w["n_grid"], log_delta_min=w["log_delta_min"], log_delta_max=w["log_delta_max"])

    def step(tm=None):
        src = lowrank_fast.dosage_blocks(Gt_host, rows_of, dev)
        return lowrank_fast.loco_scan_blocks_fast(Gk_std, d.chrom_kin, src, M, chroms, X, Y_all, n_real=B, timers=tm,
                                                  **grid_kw)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    launches0 = _lib.kernel_launches()
    timers: dict = {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        out = step(timers)
        del out
    ev1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    launches = _lib.kernel_launches() - launches0
    clk = clocks.stop()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    value = M * P * args.steps / elapsed
    stages = {kk: round(sum(a.elapsed_time(b) for a, b in v if b is not None) / args.steps, 3)
              for kk, v in timers.items()}
    peaks = measured_peaks()
    # the fused Wald launches of a step: 4 (k_c + N) flop per test (the on-rank and off-rank dot products)
    wald_s = stages.get("wald", 0.0) / 1e3
    wald_flop = 4.0 * (k + N) * P * M
    roof = None
    if wald_s > 0:
        ach = wald_flop / wald_s / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": peaks["tensor_tflops"], "unit": "TFLOP/s",
                "frac": ach / peaks["tensor_tflops"], "traffic": None,
                "kernel": "k_pair<2> over K = k + N (fused split-FP16 low-rank Wald) with its block's operand prep",
                "wald_ms_per_step": 1e3 * wald_s, "algorithmic_flop_per_step": wald_flop,
                "peak_source": peaks["source"] + " bf16 dense (FP16 rate is the same)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp16x2-split tensor (FP32 acc) + f64",
            "data": "synthetic (seeded: Binomial(2, MAF~U[0.05,0.5]) int8 genotypes, RINT phenotypes, "
                    "h2~U[0.1,0.7], 10 causal)",
            "config": {"workload": name, "N": N, "k_kin": k, "M": M, "B": B, "n_perm": n_perm, "P": P,
                       "chromosomes": w["n_chrom"], "covariates": D, "grid": w["n_grid"], "block": lowrank_fast.BLOCK,
                       "h2d_bytes_per_step": int(M) * N,
                       "stream": "int8 dosages in pinned host memory, copied per block on a side stream beside the "
                                 "previous block's scan, standardised on the device",
                       "l2": "inputs larger than L2 (each block's split operands 1.7 GB)",
                       "parallelism": f"{world} replica(s), no cross-GPU exchange"},
            "wall_s_timed": wall, "gpu_launches": launches, "roofline": roof, "stage_ms_per_step": stages,
            "generate_s": round(t_gen, 1), "e2e": None, "cpu_baseline": None,
            "notes": "genotypes cross from host memory inside every step; outputs stay on the device; no CPU sample "
                     "for this shape (one LOCO basis at N = 50,000 is ~4e11 flop on the host)",
            "clocks": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)


def fp32_peak_tflops() -> float:
    import torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    mhz = 2070.0
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        mhz = float(json.loads(p.read_text()).get("sm_max_mhz") or mhz)
    return props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12


def isolated_stages(args, step, w) -> dict:
    """Stage times of one untimed step with every stage on the main stream (nothing overlapped), CUDA events."""
    import torch
    from fasterlmm_gb300 import fast
    saved = fast.PIPELINE
    fast.PIPELINE = False
    tm: dict = {}
    try:
        step(tm)
        torch.cuda.synchronize()
    finally:
        fast.PIPELINE = saved
    return {k: round(sum(a.elapsed_time(b) for a, b in v if b is not None), 3) for k, v in tm.items()}


def plain_comparison(args, d, w, grid_kw) -> dict:
    """
    The metric's denominator: the plain FP64 form (FP64 kernels, FP64 eigendecomposition, the reference's golden
    section) and the chosen form on the same bounded subset of the workload -- its first ``--plain-chroms``
    chromosomes with every phenotype and permutation -- device-resident inputs, CUDA events, one warm-up step each.
    """
    import torch
    from fasterlmm_gb300 import perms
    keep = np.isin(d.chrom, sorted(np.unique(d.chrom))[: args.plain_chroms])
    dev = torch.device("cuda", torch.cuda.current_device())
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    sub = SimpleNamespace(Z=t(d.Z_float()[:, keep]), Y=t(d.Y), X=t(d.X), chrom=d.chrom[keep], Z_kin=None,
                          chrom_kin=None)
    B, n_perm = w["B"], w["n_perm"]
    tests = int(keep.sum()) * B * (1 + n_perm)
    out = {"subset": f"{args.plain_chroms} of {w['n_chrom']} chromosomes ({int(keep.sum())} variants), all {B} "
                     f"phenotypes x {n_perm} permutations, LOCO within the subset"}
    for form, reps in (("plain", 1), ("fast", 3)):
        perms.perm_threshold(sub, list(range(B)), n_perm=n_perm, form=form, **grid_kw)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            res, pmf = perms.perm_threshold(sub, list(range(B)), n_perm=n_perm, form=form, **grid_kw)
            del res, pmf
        e1.record()
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3 / reps
        out[form] = {"ms_per_step": 1e3 * sec, "tests_per_s": tests / sec}
    out["ratio"] = out["fast"]["tests_per_s"] / out["plain"]["tests_per_s"]
    return out


def e2e_buffers(d, w):
    """Pinned host inputs and preallocated pinned host outputs of the e2e leg, made before any device work (the
    state a caller that keeps its buffers between scans is in)."""
    import torch
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    data_host = SimpleNamespace(Z=t(d.Z_float()), Y=t(d.Y), X=t(d.X), chrom=d.chrom, Z_kin=None, chrom_kin=None)
    M, B, n_perm = w["M"], w["B"], w["n_perm"]
    out = {k: torch.empty((M, B), dtype=torch.float64).pin_memory() for k in ("f", "beta", "se", "sfve", "nullh2")}
    out["max_F"] = torch.empty(B * (1 + n_perm), dtype=torch.float64).pin_memory()
    return data_host, out


def e2e_leg(args, w, pheno, grid_kw, data_host, out) -> dict:
    """Same scan through the public call with pinned host inputs and preallocated pinned host outputs."""
    import torch
    from fasterlmm_gb300 import perms
    torch.cuda.synchronize()
    torch.cuda.empty_cache()  # start from the allocator state a fresh caller would see
    M, B, n_perm = w["M"], w["B"], w["n_perm"]
    steps = max(1, min(args.steps, 5))
    perms.perm_threshold(data_host, pheno, n_perm=n_perm, form=args.form, out=out, **grid_kw)  # warm
    torch.cuda.synchronize()
    step_ms = []
    t0 = time.perf_counter()
    for _ in range(steps):
        t1 = time.perf_counter()
        perms.perm_threshold(data_host, pheno, n_perm=n_perm, form=args.form, out=out, **grid_kw)
        torch.cuda.synchronize()
        step_ms.append(round(1e3 * (time.perf_counter() - t1), 2))
    dt = (time.perf_counter() - t0) / steps
    h2d = sum(x.numel() * x.element_size() for x in (data_host.Z, data_host.Y, data_host.X))
    d2h = sum(x.numel() * x.element_size() for k, x in out.items() if k != "nullh2")
    # the fast form streams nullh2 as one (B,) vector per chromosome and fills its rows on the host
    d2h += (w["n_chrom"] * B * 8) if args.form == "fast" else out["nullh2"].numel() * 8
    return {"value": M * B * (1 + n_perm) / dt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": 1e3 * dt, "steps": steps, "step_ms": step_ms}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--form", choices=["fast", "plain"], default="fast")
    ap.add_argument("--B", type=int, default=None, help="override the phenotype count (quick runs)")
    ap.add_argument("--M", type=int, default=None, help="override the variant count (quick runs)")
    ap.add_argument("--delta", choices=["grid", "learned"], default=None,
                    help="fast form's delta fit: full FP32 grid, or the learned proposal's narrow bracket")
    ap.add_argument("--no-pipeline", action="store_true",
                    help="run each chromosome's delta fit on the main stream instead of one chromosome ahead")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 form's bounded run (the denominator of the chosen-vs-plain ratio)")
    ap.add_argument("--plain-chroms", type=int, default=2,
                    help="chromosomes of the workload that the plain-form comparison scans (default 2 of 20)")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="headline",
                    help="headline: 1,000 x 100,000 x 6,484 phenotypes; c3: the uneven-batching shape; c5: the "
                         "low-rank large cohort (50,000 samples, streamed genotypes)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c5":
        run_lowrank(args)
    elif args.workload != "headline":
        run_grouped(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
