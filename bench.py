#!/usr/bin/env python
"""Headline benchmark: exact Khatri-Rao-product leverage-score sampling.

Workload (the reference's headline sampling configuration): N = 3 factor
matrices of I = 2^23 rows x R = 32 columns, float64 N(0,1) entries with 1% of
each factor's rows scaled x100 (seeded, synthetic -- no dataset), J = 50,000
samples per draw from the full Khatri-Rao product (no mode excluded, the
reference's KRPDrawSamples(N+1)).  One step = one draw: computeM (Hadamard
products, FP64 pseudo-inverse and eigendecompositions, eigen trees) plus the
fused descent of all modes plus the weights, with the partition trees
resident in HBM.  The trees (3 x 1.1 GB FP32, 3 x 2.2 GB FP64) are larger
than L2, so no separate flush is done between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp32|fp64]
  python bench.py --impl reference ...   # the reference arm: the CPU oracle port

Multi-GPU (torchrun): every rank runs an independent replica of the workload
(sampling needs no exchange); value = all samples / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import shutil
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "samples/s at I=2^23,R=32 (exact KRP leverage sampling, N=3, J=50000)"
UNIT = "samples/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--N", type=int, default=3)
    ap.add_argument("--log2I", type=int, default=23)
    ap.add_argument("--R", type=int, default=32)
    ap.add_argument("--J", type=int, default=50000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="sampling",
                    choices=["sampling", "als", "serve", "lowrank", "tree", "launcher-check"],
                    help="als: randomized CP-ALS on the synthetic sparse tensor (seconds per sweep); "
                         "serve: Poisson stream of sampling and CP-ALS requests (p50/p99 latency)")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: mean arrivals per second")
    ap.add_argument("--duration", type=float, default=10.0, help="serve: seconds of arrivals")
    ap.add_argument("--als-fraction", type=float, default=0.2)
    ap.add_argument("--hbm-budget-gb", type=float, default=160.0)
    ap.add_argument("--max-active", type=int, default=32)
    ap.add_argument("--nnz", type=float, default=1.5e8)
    ap.add_argument("--als-scale", type=float, default=1.0,
                    help="als: dims and nnz times this factor (a smaller case of the same kernels, for profiling)")
    ap.add_argument("--sweeps", type=int, default=20)
    ap.add_argument("--snr-db", type=lambda v: None if v.lower() == "none" else float(v), default=20.0,
                    help="lowrank: signal-to-noise ratio of the counter-hash Gaussian noise (none: --snr-db none)")
    ap.add_argument("--no-fp64-arm", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="sampling: skip the tree-build, CP-ALS and serving legs of the default line")
    return ap.parse_args()


# ------------------------------------------------------------- distributed

def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int, device=None) -> float:
    """The largest value of x over the ranks (x itself on one rank): the
    timed region of the slowest replica sets the whole-job time."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def free_port() -> int:
    import socket
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def spawn_command(argv: list[str], nproc: int, port: int | None = None) -> list[str]:
    """The launch of this script as `nproc` ranks on one node (one process
    per GPU, RANK / LOCAL_RANK / WORLD_SIZE set by torch.distributed.run,
    rendezvous on 127.0.0.1)."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={nproc}",
            "--master-addr", "127.0.0.1", "--master-port", str(port or free_port()),
            str(Path(__file__).resolve()), *argv]


def launcher_check(ws: int, rank: int, local: int):
    """The multi-rank plumbing without a GPU: gloo ranks agree on the max
    over ranks and on the whole-job rate (used by the CPU tests)."""
    import torch.distributed as dist
    dist.init_process_group("gloo")
    slowest = max_over_ranks(1.0 + rank, ws)
    line = {"n_gpus": ws, "rank": rank, "local_rank": local, "max_over_ranks": slowest,
            "whole_job_rate": whole_job_rate(ws, 100.0, slowest), "seeds": replica_seeds(rank)}
    dist.destroy_process_group()
    return line if rank == 0 else None


def replica_seeds(rank: int) -> dict:
    """Seeds of one replica: every rank draws its own factors and uniforms,
    so the replicas do independent work (weak scaling, no exchange)."""
    return {"factors": 1234 + rank, "sampler": 7 + rank, "sparse": 2024 + rank, "serve": 2024 + rank}


def whole_job_rate(ws: int, units_per_rank: float, seconds: float) -> float:
    """Units all ranks processed per second of the slowest rank's time."""
    return ws * units_per_rank / seconds


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        exe = shutil.which("nvidia-smi")
        if not exe:
            return
        self.proc = subprocess.Popen(
            [exe, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
             "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- workload

def make_factors_device(N, I, R, seed, device):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    U = []
    for _ in range(N):
        u = torch.randn(I, R, device=device, dtype=torch.float64, generator=g)
        rows = torch.randperm(I, device=device, generator=g)[: max(1, I // 100)]
        u[rows] *= 100.0
        U.append(u)
    return U


def algorithmic_bytes(samples, dims, R, J, N, j, prec_bytes, shadow=False):
    """Bytes one descent launch must move at minimum (each distinct node or
    leaf block read once): per included mode, distinct Gram-tree nodes read
    (root + left child of every internal node on a sampled path) x P x s_G,
    (P = values per node in the tree's layout), distinct leaf blocks x rows x
    R x 8 (FP64 factor rows of the leaf scan;
    x 4 when the scan reads the FP32 factor copies, plus distinct sampled
    rows x R x 8 for the FP64 rows that update h), the whole eigen tree
    (2R-1) x P x s_G and its R x R FP64 row table; plus the outputs
    (samples N x J x 8, h J x R x 8, weights J x 8)."""
    import torch
    from fast_tensor_leverage_gb300 import _lib
    # values per node in the trees' layout (packed triangle, or the 544-value
    # wrapped-diagonal node of FP32 trees at 16 < R <= 32)
    P = _lib.node_layout(R, 0 if prec_bytes == 8 else 1)[1]
    total = 0
    for k in range(N):
        if k == j:
            continue
        F = min(R, dims[k])
        g = _lib.tree_geometry(dims[k], F)
        rows = samples[k].to(torch.int64)
        leaf = rows // F
        partial = g.node_count - g.nodes_upto_lfill
        node = torch.where(leaf < partial, g.nodes_upto_lfill + leaf, leaf + g.complete_level_offset)
        leaves = torch.unique(leaf)
        reads = [torch.zeros(1, dtype=torch.int64, device=rows.device)]
        cur = node
        while True:
            cur = cur[cur > 0]
            if cur.numel() == 0:
                break
            parent = (cur - 1) // 2
            reads.append(torch.unique(2 * parent + 1))
            cur = torch.unique(parent)
        n_nodes = int(torch.unique(torch.cat(reads)).numel())
        if shadow:
            total += n_nodes * P * prec_bytes + int(leaves.numel()) * F * R * 4
            total += int(torch.unique(rows).numel()) * R * 8
        else:
            total += n_nodes * P * prec_bytes + int(leaves.numel()) * F * R * 8
        total += (2 * R - 1) * P * prec_bytes + R * R * 8
    n_inc = sum(1 for k in range(N) if k != j)
    total += n_inc * J * 8 + J * R * 8 + J * 8
    return total


def source_tag() -> str:
    """Hash of the descent kernel's sources; a committed ncu summary carries
    the tag of the sources it was captured from, so a stale one is detected."""
    import hashlib
    h = hashlib.sha256()
    for f in ("descent.cuh", "krp_draw.cu", "ftl_common.cuh"):
        h.update((REPO / "fast_tensor_leverage_gb300" / "csrc" / f).read_bytes())
    return h.hexdigest()[:16]


def read_traffic(precision):
    """DRAM bytes per C2 descent launch from the committed ncu summary
    (profiles/krp_draw*_<precision>_*.md, lines 'traffic_bytes_per_launch:'
    and 'source_tag:').  None when no summary matches the current sources."""
    tag = source_tag()
    for f in sorted((REPO / "profiles").glob(f"krp_draw*_{precision}_*.md")):
        vals = {}
        for line in f.read_text().splitlines():
            for key in ("traffic_bytes_per_launch:", "source_tag:"):
                if line.strip().startswith(key):
                    vals[key] = line.split(":", 1)[1].strip().split()[0]
        if vals.get("source_tag:") == tag and "traffic_bytes_per_launch:" in vals:
            try:
                return float(vals["traffic_bytes_per_launch:"]), f.name
            except ValueError:
                pass
    return None, f"no ncu summary for source tag {tag}"


def measured_peak():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def binom_upper(k: int, n: int, z: float = 1.96) -> float:
    """Wilson upper bound of a binomial proportion (k of n)."""
    if n == 0:
        return 1.0
    p = k / n
    den = 1 + z * z / n
    c = p + z * z / (2 * n)
    r = z * ((p * (1 - p) / n + z * z / (4 * n * n)) ** 0.5)
    return (c + r) / den


def small_krp_tv(ftl, precision, seed=2023, N=3, I=8, R=4, J=1 << 20, reps=64):
    """Total-variation distance between 2^26 draws of the sampler and the
    exact leverage distribution of a 512-row KRP (1% of entries x10), the
    exact scores by brute force in FP64 (K pinv(K^T K) K^T on the
    materialised KRP), with the sampling-noise level of that many draws."""
    import torch
    rng = np.random.default_rng(seed)
    U = [rng.normal(size=(I, R)) for _ in range(N)]
    for u in U:
        u[rng.random(u.shape) < 0.01] *= 10.0
    K = np.ones((1, R))
    for u in U:
        K = (K[:, None, :] * u[None, :, :]).reshape(-1, R)
    lev = np.einsum("ij,jk,ik->i", K, np.linalg.pinv(K.T @ K), K)
    p = lev / lev.sum()
    s = ftl.Sampler(U, J, R, "efficient", precision=precision, seed=99)
    counts = torch.zeros(I ** N, dtype=torch.int64, device=s.device)
    offs = torch.tensor([I ** (N - 1 - k) for k in range(N)], device=s.device, dtype=torch.int64)
    for _ in range(reps):
        samples, _, _ = s.draw(N + 1)
        counts += torch.bincount((samples * offs[:, None]).sum(0), minlength=I ** N)
    emp = counts.cpu().numpy() / (reps * J)
    return {"tv": float(0.5 * np.abs(emp - p).sum()),
            "noise": float(0.5 * np.sum(np.sqrt(2 * p / (np.pi * reps * J)))),
            "draws": reps * J, "krp_rows": I ** N}


# ------------------------------------------------------------ our arm

def run_ours(args, ws, rank, local):
    import torch
    import fast_tensor_leverage_gb300 as ftl
    from fast_tensor_leverage_gb300 import _lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    N, I, R, J = args.N, 1 << args.log2I, args.R, args.J
    j = N + 1
    seeds = replica_seeds(rank)
    U = make_factors_device(N, I, R, seeds["factors"], dev)
    st = torch.cuda.current_stream(dev)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    def time_draws(sampler, steps, warmup, clocks=None, jj=None):
        """Mean ms per draw over `steps` timed draws, and the mean duration
        of the descent launches inside that same timed region (CUDA events
        on the launching stream)."""
        jj = j if jj is None else jj
        for _ in range(warmup):
            sampler.draw(jj)
        barrier()
        torch.cuda.synchronize(dev)
        if clocks:
            clocks.start()
            time.sleep(0.25)
        sampler.descent_events = []
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            sampler.draw(jj)
        e1.record(st)
        torch.cuda.synchronize(dev)
        barrier()
        clk = clocks.stop() if clocks else None
        kms = statistics.fmean(a.elapsed_time(b) for a, b in sampler.descent_events)
        sampler.descent_events = None
        ms = max_over_ranks(e0.elapsed_time(e1) / steps, ws, dev)
        return ms, max_over_ranks(kms, ws, dev), clk

    s = ftl.Sampler(U, J, R, "efficient", precision=args.precision, seed=seeds["sampler"], autotune=False)
    # the autotuner times the draw variants on this workload (set-up, outside
    # the timed region) and selects the fastest for the timed draws
    from fast_tensor_leverage_gb300 import autotune as AT
    tuning = AT.tune_draw(s, store=False)
    clocks = ClockSampler(local) if rank == 0 else None
    ms, kernel_ms, clk = time_draws(s, args.steps, args.warmup, clocks)
    value = whole_job_rate(ws, J, ms / 1e3)
    prec_bytes = 4 if args.precision == "fp32" else 8
    alg = algorithmic_bytes(s.samples_dev, s.dims, R, J, N, j, prec_bytes, shadow=s.U32 is not None)
    peak, peak_kind = measured_peak()
    achieved = alg / (kernel_ms / 1e3) / 1e9
    traffic, traffic_src = read_traffic(args.precision)

    # end to end through the public numpy API: host uniforms in (pinned),
    # samples / h / weights back into host arrays, every step
    e2e_steps = max(5, min(50, args.steps // 5))
    draws_host = torch.empty(2 * N * J, dtype=torch.float64, pin_memory=True)
    draws_host.uniform_(0.0, 1.0, generator=torch.Generator().manual_seed(99))
    samples_np = np.zeros((N, J), dtype=np.uint64)
    h_np = np.zeros((J, R))
    w_np = np.zeros(J)
    for _ in range(3):
        s.KRPDrawSamples_materialize(j, samples_np, h_np, w_np, draws=draws_host)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.KRPDrawSamples_materialize(j, samples_np, h_np, w_np, draws=draws_host)
    t_e2e = max_over_ranks(time.perf_counter() - t0, ws, dev)
    e2e = {"value": whole_job_rate(ws, J * e2e_steps, t_e2e), "unit": UNIT,
           "h2d_bytes_per_step": 2 * N * J * 8,
           "d2h_bytes_per_step": N * J * 8 + J * R * 8 + J * 8,
           "api": "Sampler.KRPDrawSamples_materialize(j, samples, h_out, weights_out, draws=pinned host uniforms)"}

    # the other C2 variant: one mode excluded (j = 0, two descents per sample)
    ms_j0, kms_j0, _ = time_draws(s, max(20, args.steps // 5), max(3, args.warmup // 4), jj=0)
    one_excluded = {"j": 0, "value": whole_job_rate(ws, J, ms_j0 / 1e3), "ms_per_step": ms_j0,
                    "descent_ms": kms_j0}

    # the plain FP64 GPU path on the same workload (the like-for-like
    # precision of the reference), and the accuracy of the mixed path
    # against it: both drawn with the same uniforms
    fp64 = None
    acc = {}
    shared = torch.empty(2 * N * J, dtype=torch.float64, device=dev)
    shared.uniform_(0.0, 1.0, generator=torch.Generator(device=dev).manual_seed(4242))
    smp, _, w_mixed = s.draw(j, shared)
    samples_mixed, w_mixed = smp.clone(), w_mixed.clone()
    if args.precision == "fp32" and not args.no_fp64_arm:
        s.descent_events = None
        del s
        torch.cuda.empty_cache()
        s64 = ftl.Sampler(U, J, R, "efficient", precision="fp64", seed=seeds["sampler"])
        ms64, kms64, _ = time_draws(s64, max(10, args.steps // 5), max(3, args.warmup // 4))
        fp64 = {"value": whole_job_rate(ws, J, ms64 / 1e3), "ms_per_step": ms64, "descent_ms": kms64}
        smp64, _, w64 = s64.draw(j, shared)
        same = (samples_mixed == smp64).all(dim=0)
        mism = int((~same).sum())
        wrel = ((w_mixed - w64).abs() / w64.abs())[same]
        acc["mixed_vs_fp64_same_uniforms"] = {
            "samples": J, "index_agreement": 1.0 - mism / J, "mismatches": mism,
            "tv_upper_bound_95": binom_upper(mism, J),
            "weights_rel_err_max": float(wrel.max()) if wrel.numel() else None,
            "weights_rel_err_median": float(wrel.median()) if wrel.numel() else None,
            "note": "coupling: TV(mixed law, FP64 law) <= P(indices differ under shared uniforms)"}
        samples64_host = smp64.cpu().numpy().astype(np.uint64)
        if not args.no_extras:
            # the tensor-core tree precisions on the same workload and uniforms
            per = {}
            for tp in ("tf32x3", "bf16"):
                st_ = ftl.Sampler(U, J, R, "efficient", precision=tp, seed=seeds["sampler"], overlap_computem=False)
                smp_t, _, w_t = st_.draw(j, shared)
                same_t = (smp_t == smp64).all(dim=0)
                mism_t = int((~same_t).sum())
                wrel_t = ((w_t - w64).abs() / w64.abs())[same_t]
                per[tp] = {"index_agreement": 1.0 - mism_t / J, "mismatches": mism_t,
                           "tv_upper_bound_95": binom_upper(mism_t, J),
                           "weights_rel_err_max": float(wrel_t.max()) if wrel_t.numel() else None}
                del st_, smp_t, w_t
                torch.cuda.empty_cache()
            per["fp32"] = {k: acc["mixed_vs_fp64_same_uniforms"][k]
                           for k in ("index_agreement", "mismatches", "tv_upper_bound_95", "weights_rel_err_max")}
            acc["tree_precisions_vs_fp64_same_uniforms"] = per
        del s64
        torch.cuda.empty_cache()
    else:
        samples64_host = None
        del s
    if rank == 0:
        acc["small_krp_tv"] = {p: small_krp_tv(ftl, p) for p in
                               (("fp32", "fp64") if args.no_extras else ("fp32", "tf32x3", "bf16", "fp64"))}
    extras = {}
    if not args.no_extras:
        extras["tree_build"] = tree_build_rates(U[0], R, ("fp32", "tf32x3", "bf16"), reps=5)
        extras["tree_build"]["shape"] = f"I={I}, R={R} (one factor of the workload)"

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        U_host = [u.cpu().numpy() for u in U]
        del U
        torch.cuda.empty_cache()
        cpu, par = cpu_baseline(U_host, J, R, j, reps=3, shared=shared.cpu().numpy(),
                                samples64=samples64_host, samples_mixed=samples_mixed.cpu().numpy())
        if par is not None:
            acc.update(par)

    if not args.no_extras:
        # CP-ALS at 1/6 of the C3 size (5 sweeps) and a short serving run at a
        # sustainable rate, measured in the same process as the headline
        extras["als"] = als_summary(dev, replica_seeds(rank)["sparse"], scale=0.167, sweeps=5,
                                    cpu_sweeps=1 if rank == 0 else 0)
        torch.cuda.empty_cache()
        extras["serve"] = serve_summary(dev, replica_seeds(rank)["serve"], rate=8.0, duration=10.0)
    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.precision, "data": "synthetic (seeded N(0,1), 1% rows x100)",
        "config": {"workload": "exact KRP leverage sampling, N=3, I=2^23, R=32, J=50000, no mode excluded",
                   "N": N, "I": I, "R": R, "J": J, "j": j, "precision": args.precision,
                   "value_is": ("mixed precision (FP32 node Grams and forms, FP64 h, weights, pseudo-inverse): "
                                "the mixed-precision mode this workload targets; fp64_path is the reference's "
                                "precision")
                   if args.precision == "fp32" else "FP64 throughout (the reference's precision)",
                   "l2": "inputs larger than L2 (partition trees 3 x %.2f GB)" % (
                       (2 * (I // R) - 1) * (R * (R + 1) // 2) * prec_bytes / 1e9),
                   "parallelism": f"replicas x{ws}"},
        "e2e": e2e,
        # per draw: computem_pinv_kernel, computem_eig_kernel, krp_draw_kernel,
        # krp_fixup_kernel (FP32; FP64 draws have no fix-up pass)
        "gpu_launches": (4 if args.precision == "fp32" else 3) * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "peak_kind": peak_kind,
                     "kernel": "krp_draw_d32_kernel" if args.precision != "fp64" and 16 < R <= 32 else "krp_draw_kernel",
                     "kernel_ms": kernel_ms, "kernel_ms_source": "mean of the descent launches in the timed loop "
                     "(krp_draw_kernel + its fix-up pass), CUDA events on the launching stream",
                     "algorithmic_bytes_per_launch": alg},
        "clocks": clk,
        "cpu_baseline": cpu,
        "one_mode_excluded": one_excluded,
        "autotune": {"family": "draw", "variant": tuning["variant"],
                     "samples_per_warp": (1, 2, 3, 3, 4, 6)[tuning["variant"]] if tuning["ms"] else 1,
                     "weights_in_shared_memory": bool(tuning["ms"]) and tuning["variant"] >= 3,
                     "descent_ms_by_variant": {str(k): v for k, v in tuning["ms"].items()}},
        "accuracy": acc,
    }
    if fp64 is not None:
        line["fp64_path"] = fp64
        line["mixed_vs_fp64"] = value / fp64["value"]
    line.update(extras)
    return line


def cpu_baseline(U_host, J, R, j, reps=3, shared=None, samples64=None, samples_mixed=None):
    """The CPU oracle port (C restatement of the reference's sampler with
    OpenMP over samples) on the same workload: full-size trees (built outside
    the timing), one warm-up draw, median of `reps` draws of J samples.
    As the checker it then draws with the uniforms the GPU paths used and
    compares indices: the FP64 GPU path must match it except at near-ties
    (decision margin < 1e-10), and the mixed path's mismatches are binned by
    the oracle's margin."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    N = len(U_host)
    o = O.OracleKRPSampler(U_host, J, R)
    rng = np.random.default_rng(5)
    draws = rng.random(2 * N * J)
    o.draw(j, draws)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        o.draw(j, draws)
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    cpu = {"value": J / t, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{reps} draws of J={J} (median) at the full workload, trees prebuilt",
           "note": "the port parallelises over samples with OpenMP; the reference calls cblas_dsymv once per "
                   "sample and level, so this baseline is stronger than the reference itself"}
    par = None
    if shared is not None:
        ref = o.draw(j, shared, want_margin=True).astype(np.uint64)
        margin = o.margin
        par = {}

        def bins(bad):
            m = margin[bad]
            return {"margin_lt_1e-10": int((m < 1e-10).sum()), "margin_lt_1e-6": int((m < 1e-6).sum()),
                    "margin_lt_1e-3": int((m < 1e-3).sum()), "total": int(bad.sum())}

        if samples64 is not None:
            bad = (samples64 != ref).any(axis=0)
            par["fp64_vs_oracle"] = {"samples": J, "index_exact": float(1 - bad.mean()),
                                     "mismatches": bins(bad),
                                     "ok": bool(np.all(margin[bad] < 1e-10))}
        if samples_mixed is not None:
            bad = (samples_mixed.astype(np.uint64) != ref).any(axis=0)
            par["mixed_vs_oracle"] = {"samples": J, "index_agreement": float(1 - bad.mean()),
                                      "mismatches": bins(bad)}
    return cpu, par


# ------------------------------------------------------- reference arm

def run_reference(args, ws, rank):
    if rank != 0:
        return None
    N, I, R, J = args.N, 1 << args.log2I, args.R, args.J
    j = N + 1
    rng = np.random.default_rng(1234)
    U = []
    for _ in range(N):
        u = rng.standard_normal((I, R))
        u[rng.choice(I, size=max(1, I // 100), replace=False)] *= 100.0
        U.append(u)
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    # each step: one draw of J samples, the GPU arm's configuration
    o = O.OracleKRPSampler(U, J, R)
    draws = rng.random(2 * N * J)
    for _ in range(max(1, args.warmup)):
        o.draw(j, draws)
    steps = max(1, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.draw(j, draws)
    t = time.perf_counter() - t0
    value = steps * J / t
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded N(0,1), 1% rows x100)",
        "config": {"workload": "exact KRP leverage sampling, N=3, I=2^23, R=32, J=50000, no mode excluded",
                   "N": N, "I": I, "R": R, "J": J, "j": j, "samples_per_step": J},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} draws of J={J} samples at the full workload (the GPU arm's config)",
                         "note": "C restatement of the reference's sampler (the reference's sources are not on "
                                 "the GPU box); it parallelises over samples with OpenMP, where the reference "
                                 "calls cblas_dsymv per sample and level"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def tree_build_rates(U, R, precisions, reps=10):
    """Device time of one partition-tree build (leaf Grams, the FP32 factor
    copy for FP32-node trees, internal levels) per precision on the factor U,
    and its HBM rate: bytes = read U (n R 8) + write the FP32 copy (n R 4) +
    write the leaf level + read and write the internal levels (each internal
    node is written once and read by its parent)."""
    import torch
    from fast_tensor_leverage_gb300 import _lib
    n = U.shape[0]
    F = min(R, n)
    g = _lib.tree_geometry(n, F)
    st = torch.cuda.current_stream(U.device)
    peak, _ = measured_peak()
    out = {}
    for prec in precisions:
        p = _lib.PREC[prec]
        _, S, _ = _lib.node_layout(R, p)
        es = 8 if prec == "fp64" else 4
        G = torch.empty(_lib.tree_bytes(n, F, R, p) // es, dtype=torch.float64 if es == 8 else torch.float32,
                        device=U.device)
        U32 = torch.empty((n, R), dtype=torch.float32, device=U.device) if es == 4 else None

        def build():
            _lib.call("ftl_tree_build_ex", U.data_ptr(), n, R, F, p, G.data_ptr(),
                      U32.data_ptr() if U32 is not None else None, st.cuda_stream)

        for _ in range(3):
            build()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            build()
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        node_b = S * es
        internal = g.node_count - g.leaf_count
        byts = n * R * 8 + (n * R * 4 if es == 4 else 0) + g.leaf_count * node_b + 2 * internal * node_b
        out[prec] = {"ms": ms, "GBps": byts / ms / 1e6, "frac_of_hbm": byts / ms / 1e6 / peak,
                     "bytes": byts, "leaf_path": ("tensor cores (tcgen05)" if prec in ("tf32x3", "bf16") and R <= 32
                                                  else "CUDA cores")}
        del G, U32
    out["device_status"] = _lib.device_status()
    return out


def run_tree(args, ws, rank, local):
    """Partition-tree build throughput at the sampling workload's factor shape
    (I = 2^log2I rows x R, N(0,1) with 1% of rows x100), per tree precision."""
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    I, R = 1 << args.log2I, args.R
    U = make_factors_device(1, I, R, replica_seeds(rank)["factors"], dev)[0]
    res = tree_build_rates(U, R, ("fp32", "tf32x3", "bf16", "fp64"), reps=max(3, args.steps))
    if rank != 0:
        return None
    return {"metric": f"partition-tree build, I=2^{args.log2I}, R={R}", "unit": "ms", "value": res["fp32"]["ms"],
            "higher_is_better": False, "n_gpus": ws, "builds": res,
            "peak_hbm_gbs": measured_peak()[0], "data": "synthetic (seeded N(0,1), 1% rows x100)"}


def als_summary(dev, seed, scale, sweeps, cpu_sweeps=1):
    """Randomized CP-ALS on the synthetic sparse stand-in for amazon-reviews
    at `scale` of its size (dims 4.8e6 x 1.8e6 x 1.8e6 and 1.5e8 nonzeros
    times scale; Zipf(1.1) indices, log1p(lognormal) values; R = 25,
    J = 2^16; factors from the range finder), `sweeps` sweeps with
    mixed-precision and with FP64 sampling: update-only device s/sweep and
    exact fits.  With cpu_sweeps, the CPU port of the same ALS (the oracle's
    restatement of ALS::execute_ds_als_update over its C sampler, all host
    cores) runs that many sweeps from the same initial factors: its s/sweep
    is the CPU baseline."""
    import torch
    import fast_tensor_leverage_gb300 as ftl
    from fast_tensor_leverage_gb300.synthetic import sparse_powerlaw_tensor
    dims = [int(d * scale) for d in (4_800_000, 1_800_000, 1_800_000)]
    R, J = 25, 1 << 16
    idx, vals = sparse_powerlaw_tensor(dims, int(1.5e8 * scale), 1.1, seed=seed, device=dev)
    sp = ftl.SparseTensor(idx, vals, "sort", dims=dims)
    rhs = type("Rhs", (), {})()
    rhs.ten = sp
    out = {"dims": dims, "nnz": sp.nnz, "R": R, "J": J, "sweeps": sweeps}
    init = None
    # FP64 twice (sampler seeds 11 and 12): randomized ALS trajectories depend
    # on the sample stream, so the FP64 seed-to-seed fit spread is the
    # yardstick for the mixed-vs-FP64 fit gap
    for prec, sseed in (("fp32", 11), ("fp64", 11), ("fp64_seed12", 12)):
        lhs = ftl.PyLowRank(dims, R, seed=7, sync_host=False)
        sp.execute_rrf(lhs.ten, seed=7)
        if init is None:
            init = ([u.cpu().numpy() for u in lhs.ten.U_dev], lhs.ten.sigma_dev.cpu().numpy())
        als = ftl.ALS(lhs.ten, sp)
        als.initialize_ds_als(J, "efficient", precision=prec[:4], seed=sseed)
        fit0 = lhs.compute_exact_fit(rhs)
        st = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(st)
        for _ in range(sweeps):
            for j in range(3):
                als.execute_ds_als_update(j, True, True)
        e1.record(st)
        torch.cuda.synchronize(dev)
        out[prec] = {"s_per_sweep": e0.elapsed_time(e1) / 1e3 / sweeps, "fit_initial": fit0,
                     "fit_final": lhs.compute_exact_fit(rhs)}
        del als, lhs
        torch.cuda.empty_cache()
    out["fit_gap_mixed_vs_fp64"] = out["fp32"]["fit_final"] - out["fp64"]["fit_final"]
    out["fit_gap_fp64_seed_to_seed"] = out["fp64_seed12"]["fit_final"] - out["fp64"]["fit_final"]
    if cpu_sweeps:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        O.set_threads(threads)
        # the port's per-mode lookups (nonzeros stably sorted by their fiber
        # key over the other modes, as its constructor sorts them), sorted on
        # the GPU to keep this leg short
        lookups = []
        for j in range(3):
            key = torch.zeros(idx.shape[0], dtype=torch.int64, device=dev)
            for k in range(3):
                if k != j:
                    key = key * dims[k] + idx[:, k].to(torch.int64)
            ks, perm = torch.sort(key, stable=True)
            lookups.append((ks.cpu().numpy().astype(np.uint64), idx[perm, j].to(torch.int64).cpu().numpy(),
                            vals[perm].cpu().numpy()))
            del key, ks, perm
        idx_h = idx.cpu().numpy().astype(np.uint32)
        vals_h = vals.cpu().numpy()
        del idx, vals
        t0 = time.perf_counter()
        o = O.OracleALS(init[0], init[1], idx_h, vals_h, J, dims=dims, lookups=lookups)
        t_setup = time.perf_counter() - t0
        t0 = time.perf_counter()
        ctr = 0
        for _ in range(cpu_sweeps):
            for j in range(3):
                o.update(j, O.philox_uniforms(11, ctr, 2 * 3 * J))
                ctr += 2 * 3 * J
        t = (time.perf_counter() - t0) / cpu_sweeps
        out["cpu_baseline"] = {"s_per_sweep": t, "unit": "s/sweep", "cores": threads, "kind": "port",
                               "sample": f"{cpu_sweeps} sweep(s) of the CPU port from the same initial factors "
                                         f"(set-up {t_setup:.1f} s not counted)"}
        out["mixed_vs_cpu"] = t / out["fp32"]["s_per_sweep"]
    return out


def serve_summary(dev, seed, rate, duration, max_active=32, budget_gb=160.0):
    """A short Poisson stream of sampling and 5-sweep CP-ALS requests (the
    serving mix: N 3..6, I 1e4..1e7, R 8..128, J 2^10..2^17) through the
    serving engine; p50/p99 latency from scheduled arrival to results on the
    host, and the completed rate."""
    import torch
    from fast_tensor_leverage_gb300 import serving as S
    warm = S.ServingEngine(int(budget_gb * 1e9), max_active=4, device=dev)
    for _, r in S.poisson_request_stream(99, 1000.0, 0.01, als_fraction=0.5, I_range=(1e4, 1e5),
                                         J_log2_range=(10, 12), nnz_range=(1e5, 2e5)):
        warm.submit(r, arrival=0.0)
    while not warm.idle():
        warm.tick()
    del warm
    torch.cuda.synchronize(dev)
    torch.cuda.empty_cache()
    stream = S.poisson_request_stream(seed, rate, duration, als_fraction=0.2)
    for _, r in stream:
        if isinstance(r, S.ALSRequest) and isinstance(r.idx, S.SyntheticSparse):
            r.idx, r.vals = r.idx.materialize(dev)
    torch.cuda.synchronize(dev)
    eng = S.ServingEngine(int(budget_gb * 1e9), max_active=max_active, device=dev, reserve=True)
    done = eng.run(stream)
    torch.cuda.synchronize(dev)
    makespan = max(h.done for h in done) - min(h.arrival for h in done)
    tot = S.latency_stats(done)
    samp = [h for h in done if isinstance(h.request, S.SampleRequest)]
    als = [h for h in done if isinstance(h.request, S.ALSRequest)]
    return {"offered_rate": rate, "duration_s": duration, "requests": len(stream), "completed": len(done),
            "completed_rate": len(done) / makespan, "p50_ms": tot["p50_ms"], "p99_ms": tot["p99_ms"],
            "sampling": S.latency_stats(samp), "als": S.latency_stats(als)}


def run_als(args, ws, rank, local):
    """Randomized CP-ALS on the synthetic stand-in for amazon-reviews:
    dims 4.8e6 x 1.8e6 x 1.8e6, Zipf(1.1) indices, nnz unique tuples,
    log(1 + lognormal) values; R = 25, J = 2^16; factors initialised by the
    reference's randomized range finder (SparseTensor.execute_rrf, seeded,
    renormalised), then `sweeps` sweeps of one sampled update per mode.
    (From Gaussian factors the first update of this tensor hits ~3 nonzeros:
    J = 2^16 fibers drawn near-uniformly from 3.2e12, 1.5e8 of them occupied;
    whether a trajectory recovers from a factor with one nonzero row or
    collapses to a zero factor then turns on single samples.)
    Reports update-only seconds per sweep (device time) and the exact fit
    after the last sweep, for mixed-precision and FP64 sampling."""
    import torch
    import fast_tensor_leverage_gb300 as ftl
    from fast_tensor_leverage_gb300.synthetic import sparse_powerlaw_tensor
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dims = [int(d * args.als_scale) for d in (4_800_000, 1_800_000, 1_800_000)]
    R, J = 25, 1 << 16
    idx, vals = sparse_powerlaw_tensor(dims, int(args.nnz * args.als_scale), 1.1, seed=replica_seeds(rank)["sparse"],
                                       device=dev)
    t0 = time.perf_counter()
    sp = ftl.SparseTensor(idx, vals, "sort", dims=dims)
    torch.cuda.synchronize(dev)
    t_build = time.perf_counter() - t0
    del idx, vals
    rhs = type("Rhs", (), {})()
    rhs.ten = sp
    out = {}
    # FP64 twice (sampler seeds 11 and 12): randomized ALS trajectories depend
    # on the sample stream, so the seed-to-seed spread of the FP64 fit is the
    # yardstick for the mixed-vs-FP64 fit gap
    for prec, sseed in (("fp32", 11), ("fp64", 11), ("fp64_seed12", 12)):
        lhs = ftl.PyLowRank(dims, R, seed=7, sync_host=False)
        sp.execute_rrf(lhs.ten, seed=7)
        als = ftl.ALS(lhs.ten, sp)
        als.initialize_ds_als(J, "efficient", precision=prec[:4], seed=sseed)
        fit0 = lhs.compute_exact_fit(rhs)
        st = torch.cuda.current_stream(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(st)
        for _ in range(args.sweeps):
            for j in range(3):
                als.execute_ds_als_update(j, True, True)
        e1.record(st)
        torch.cuda.synchronize(dev)
        s_per_sweep = e0.elapsed_time(e1) / 1e3 / args.sweeps
        t0 = time.perf_counter()
        fit = lhs.compute_exact_fit(rhs)
        t_fit = time.perf_counter() - t0
        out[prec] = {"s_per_sweep": s_per_sweep, "fit_initial": fit0, "fit_final": fit, "fit_seconds": t_fit,
                     "unique_samples_last_update": als.num_unique_samples()}
        del als, lhs
        torch.cuda.empty_cache()
    if rank != 0:
        return None
    return {
        "metric": "CP-ALS s/sweep (update only), synthetic sparse {} x {} x {}, R=25, J=2^16".format(*dims),
        "value": out["fp32"]["s_per_sweep"], "unit": "s/sweep", "higher_is_better": False, "n_gpus": ws,
        "sweeps": args.sweeps, "dtype": "fp32 trees / fp64 solve", "data": "synthetic (seeded Zipf 1.1, log1p lognormal)",
        "config": {"workload": "randomized CP-ALS (STS-CP)", "dims": dims, "nnz": sp.nnz, "R": R, "J": J,
                   "init": "execute_rrf (randomized range finder), seed 7"},
        "tensor_build_s": t_build, "mixed": out["fp32"], "fp64": out["fp64"], "fp64_seed12": out["fp64_seed12"],
        "fit_gap_mixed_vs_fp64": out["fp32"]["fit_final"] - out["fp64"]["fit_final"],
        "fit_gap_fp64_seed_to_seed": out["fp64_seed12"]["fit_final"] - out["fp64"]["fit_final"],
    }


def run_lowrank(args, ws, rank, local):
    """Randomized CP-ALS of a low-rank tensor (a LowRankTensor right-hand
    side): 4 modes of I = 65,536, true rank 16, float64 N(0,1) factors made
    on the device (no noise: a noisy tensor has no low-rank MTTKRP shortcut),
    decomposed at R = 16 and R = 64 with J = 2^17 samples per update, from
    PyLowRank(seed) factors renormalised once.  Reports update-only device
    seconds per sweep and the exact fit (low-rank vs low-rank residual) before
    and after `sweeps` sweeps, for mixed-precision and FP64 sampling."""
    import torch
    import fast_tensor_leverage_gb300 as ftl
    from fast_tensor_leverage_gb300.serving import GaussianFactors
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dims, Rt, J = [65536] * 4, 16, 1 << 17
    rhs_ten = ftl.LowRankTensor(Rt, 10000, GaussianFactors(dims, Rt, seed=77 + rank).materialize(dev),
                                sync_host=False)
    noise_sigma = rhs_ten.set_noise_snr(args.snr_db, seed=91 + rank) if args.snr_db is not None else 0.0
    rhs = type("Rhs", (), {})()
    rhs.ten = rhs_ten
    out = {}
    study = {}
    precisions = ("fp64", "fp32", "tf32x3", "bf16")
    for R in (16, 64):
        for prec in precisions:
            lhs = ftl.PyLowRank(dims, R, seed=7, sync_host=False)
            lhs.ten.renormalize_columns(-1)
            als = ftl.ALS(lhs.ten, rhs_ten)
            als.initialize_ds_als(J, "efficient", precision=prec, seed=11)
            fits = [lhs.compute_exact_fit(rhs)]
            st = torch.cuda.current_stream(dev)
            ms = 0.0
            # sweep 0 is a warm-up (its fit is in the trace, its time is not);
            # the fit after every sweep is computed outside the timed spans
            for sweep in range(args.sweeps + 1):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                for j in range(4):
                    als.execute_ds_als_update(j, True, True)
                e1.record(st)
                torch.cuda.synchronize(dev)
                if sweep > 0:
                    ms += e0.elapsed_time(e1)
                fits.append(lhs.compute_exact_fit(rhs))
            out[f"R{R}_{prec}"] = {"s_per_sweep": ms / 1e3 / args.sweeps, "fit_initial": fits[0],
                                   "fit_final": fits[-1], "sweeps": args.sweeps + 1, "fit_trace": fits}
            del als, lhs
            torch.cuda.empty_cache()
        ref = out[f"R{R}_fp64"]["fit_trace"]
        study[f"R{R}"] = {p: {"max_abs_fit_diff_vs_fp64_per_sweep": max(abs(a - b) for a, b in
                                                                      zip(out[f"R{R}_{p}"]["fit_trace"], ref)),
                              "final_fit_diff_vs_fp64": out[f"R{R}_{p}"]["fit_final"] - ref[-1]}
                          for p in precisions if p != "fp64"}
    if rank != 0:
        return None
    return {
        "metric": "CP-ALS s/sweep on a rank-16 low-rank tensor, 4 x 65536, J=2^17", "value":
        out["R16_fp32"]["s_per_sweep"], "unit": "s/sweep", "higher_is_better": False, "n_gpus": ws,
        "dtype": "fp32 trees / fp64 solve",
        "data": "synthetic (seeded N(0,1) rank-16 factors" + (f", counter-hash Gaussian noise at SNR {args.snr_db} dB)"
                                                          if args.snr_db is not None else ", no noise)"),
        "config": {"workload": "randomized CP-ALS of a low-rank tensor", "dims": dims, "true_rank": Rt, "J": J,
                   "snr_db": args.snr_db, "noise_sigma": noise_sigma,
                   "fit_of_true_factors": (1.0 - float(np.sqrt(1.0 / (1.0 + 10.0 ** (args.snr_db / 10.0))))
                                           if args.snr_db is not None else 1.0)},
        "runs": out, "precision_study": study,
        "note": "same initial factors and sampler seed per precision; fit_trace[s] = exact fit after sweep s "
                "(s = 0: before the first); randomized trajectories differ once one sample differs",
    }


def run_serve(args, ws, rank, local):
    """Serving under load: a seeded Poisson stream (mean --rate per second,
    --duration seconds of arrivals) of sampling and 5-sweep CP-ALS requests,
    N in {3..6}, I log-uniform in [1e4, 1e7], R in {8, 16, 32, 64, 128}, J
    log-uniform in [2^10, 2^17], float64 N(0,1) factors, fed to the serving
    engine (HBM-budget admission, resident trees, packed draw launches,
    graph-captured sweeps).  Latency = completion (results copied to the
    host) - scheduled arrival, so queueing behind a slow engine counts.
    Every rank serves its own stream (replicas)."""
    import torch
    from fast_tensor_leverage_gb300 import serving as S
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    budget = int(args.hbm_budget_gb * 1e9)
    # warm-up: one small request of each kind through a throwaway engine
    warm = S.ServingEngine(budget, max_active=4, device=dev)
    for t, r in S.poisson_request_stream(99, 1000.0, 0.01, als_fraction=0.5, I_range=(1e4, 1e5),
                                         J_log2_range=(10, 12), nnz_range=(1e5, 2e5)):
        warm.submit(r, arrival=0.0)
    while not warm.idle():
        warm.tick()
    del warm
    torch.cuda.synchronize(dev)
    torch.cuda.empty_cache()   # the warm-up engine's cached blocks belong to its streams
    stream = S.poisson_request_stream(replica_seeds(rank)["serve"], args.rate, args.duration,
                                      als_fraction=args.als_fraction)
    # the sparse tensors of CP-ALS requests are request payloads: made on the
    # device before the clock starts (sampling factors are made at admission)
    for _, r in stream:
        if isinstance(r, S.ALSRequest) and isinstance(r.idx, S.SyntheticSparse):
            r.idx, r.vals = r.idx.materialize(dev)
    torch.cuda.synchronize(dev)
    eng = S.ServingEngine(budget, max_active=args.max_active, device=dev, reserve=True)
    clocks = ClockSampler(local)
    clocks.start()
    done = eng.run(stream)
    torch.cuda.synchronize(dev)
    cl = clocks.stop()
    makespan = max(h.done for h in done) - min(h.arrival for h in done)
    samp = [h for h in done if isinstance(h.request, S.SampleRequest)]
    als = [h for h in done if isinstance(h.request, S.ALSRequest)]
    n_samples = sum(h.request.J for h in samp)
    n_als_samples = sum(h.request.J * len(h.request.dims) * h.request.sweeps for h in als)
    tot = S.latency_stats(done)
    if rank != 0:
        return None
    return {
        "metric": "serve p50/p99 latency (Poisson mix of sampling and 5-sweep CP-ALS requests)",
        "value": tot["p99_ms"], "unit": "ms (p99)", "higher_is_better": False, "n_gpus": ws,
        "dtype": "fp32 trees / fp64 pinv, solve, fit", "data": "synthetic (seeded request stream, device-made factors)",
        "p50_ms": tot["p50_ms"], "p99_ms": tot["p99_ms"], "mean_ms": tot["mean_ms"],
        "sampling": S.latency_stats(samp), "als": S.latency_stats(als),
        "requests": len(stream), "completed": len(done), "offered_rate": args.rate,
        "completed_rate": len(done) / makespan, "makespan_s": makespan,
        "samples_per_s": n_samples / makespan, "als_samples_per_s": n_als_samples / makespan,
        "packed_launches": eng.packed_launches, "max_hbm_in_use_gb": eng.max_in_use / 1e9,
        "engine_host_s": eng.host_s,
        "admission_host_ms": {"p50": float(np.percentile(eng.start_s, 50) * 1e3),
                              "p99": float(np.percentile(eng.start_s, 99) * 1e3),
                              "max": float(np.max(eng.start_s) * 1e3)},
        "slowest_admissions": [list(x) for x in sorted(eng.start_log, reverse=True)[:12]],
        "allocator": {k: v for k, v in torch.cuda.memory_stats(dev).items()
                      if k in ("num_alloc_retries", "num_device_alloc", "num_device_free",
                               "reserved_bytes.all.peak", "allocated_bytes.all.peak")},
        "config": {"workload": "C5 serving mix", "rate_per_s": args.rate, "duration_s": args.duration,
                   "als_fraction": args.als_fraction, "hbm_budget_gb": args.hbm_budget_gb,
                   "max_active": args.max_active, "N": "3..6", "I": "log-uniform [1e4, 1e7]",
                   "R": [8, 16, 32, 64, 128], "J": "log-uniform [2^10, 2^17]", "precision": "fp32",
                   "als_nnz": "log-uniform [1e5, 3e6]"},
        "clocks": cl,
    }


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch this script as args.gpus ranks
        sys.exit(subprocess.call(spawn_command(sys.argv[1:], args.gpus)))
    ws, rank, local = dist_setup()
    if args.workload == "launcher-check":
        line = launcher_check(ws, rank, local)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.workload == "serve":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving loop"}), flush=True)
            return
        os.environ.setdefault("PYTORCH_CUDA_ALLOC_CONF", "expandable_segments:True")
        line = run_serve(args, ws, rank, local)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.workload == "tree":
        line = run_tree(args, ws, rank, local)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.workload == "lowrank":
        line = run_lowrank(args, ws, rank, local)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.workload == "als":
        line = run_als(args, ws, rank, local)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.impl == "reference":
        line = run_reference(args, ws, rank)
    else:
        line = run_ours(args, ws, rank, local)
    if line is not None:
        print(json.dumps(line), flush=True)
    if ws > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
