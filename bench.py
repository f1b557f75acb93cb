"""Benchmark: PhyloCSF region scoring on GB300 (one JSON line on rank 0).

Workload (default): 58mammals tree, strategy=mle (find_init + Brent over rho),
10,000 synthetic alignments (half coding / half noncoding ECM), lengths
log-uniform 50-3000 codons, per-species gap+N fraction U(5%,40%), 0-20% of
species entirely missing.  A step scores every region once (both models, full
rho MLE).  Inputs (7.2 M columns x 58 leaves, ~0.42 GB) are larger than L2.

  value       regions/s with the batch resident in HBM (device-timed, CUDA
              events on the engine's stream)
  e2e         the same through pcsf_score_batch with pinned host buffers
              (upload, scoring, results back inside the timed region)
  roofline    the pruning kernel: algorithmic FLOPs (8192(nl-2)+64(nl-1)+128
              per column-evaluation) / its device time
  cpu_baseline  the FP64 oracle port (the reference's loop structure, dense
              leaves) on a length-stratified sample of regions, a persistent
              pool of one process per core fed longest-first
  fp64_gpu    the plain FP64 GPU path (oracle-matched iterates) timed on a
              length-stratified sample of the same workload: the denominator of
              the split-precision engine's speed-up

``--impl reference`` times that CPU port alone (the reference is OCaml + GSL,
which cannot be built here).  It builds its sample of regions with the numpy
restatement of the column simulator (oracle/synth_np.py) and never loads the
engine library.  Multi-GPU (torchrun): replicas, each rank scores its own
workload (no data-path collective), weak scaling.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "codon-column·branches/s and regions scored/s at |Δscore|≤1e-3 dB vs FP64 oracle"
DATA = "synthetic (seeded simulation along the tree; no public benchmark exists)"
L2_BYTES = 129 * 1024 * 1024
DTYPES = {"fp32": "f32", "fp32c": "f32 (compensated)", "fp32b": "f32 (blocked compensation)", "fp64": "f64",
          "tf32x3": "tf32x3 search, f32 (compensated) reported",
          "tf32x3b": "tf32x3 search, f32 (blocked compensation) reported",
          "bf16x3b": "3xbf16 split search, f32 (blocked compensation) reported"}


def flops_per_column(nl: int) -> int:
    """One column-evaluation of the inside pass: a 64x64 contraction per internal child, the
    children's products, the root dot."""
    return 8192 * (nl - 2) + 64 * (nl - 1) + 128


def flops_per_column_grad(nl: int) -> int:
    """Inside pass plus the adjoint: per branch a Q contraction and, for internal children, a
    P^T contraction."""
    return flops_per_column(nl) + 8192 * ((2 * nl - 2) + (nl - 2)) + 64 * 3 * (2 * nl - 2)


def flops_per_column_tangent(nl: int) -> int:
    """Forward-mode pass: three contractions per internal child (E alpha, E alpha', Q v), one per
    leaf (Q v), the products of values and tangents."""
    return 8192 * (3 * (nl - 2) + nl) + 64 * 4 * (nl - 1) + 256


KERNEL_NAMES = {0: "k_prune (SIMT, {prec} returned values)", 1: "{tc} (tcgen05 search)",
                2: "k_grad (adjoint)", 3: "k_prune_tc_dual (tcgen05 tangent)",
                4: "k_prune_ff (float-float returned values of long regions)"}
KERNEL_KEYS = {0: "simt_prune", 1: "tc_prune", 2: "grad", 3: "tc_tangent", 4: "ff_prune"}
NKINDS = len(KERNEL_KEYS)


# ---------------------------------------------------------------- distributed
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, gpu: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU port
_CPU = {}


def _cpu_init(name: str):
    """Pool initialiser: the oracle's models of parameter set `name`, the reference's dense loop."""
    from oracle import oracle as O
    from phylocsf_gb300 import synth
    ps = synth.load_params(name)
    t = ps.tree
    n = t.n
    lch = np.full(n, -1, np.int32)
    rch = np.full(n, -1, np.int32)
    for i in range(n - 1):
        p = t.parent[i]
        if lch[p] < 0:
            lch[p] = i
        else:
            rch[p] = i
    ot = O.OTree(O.Tree(t.labels, t.parent, lch, rch, t.branch))
    _CPU.update(O=O, mc=O.OModel.from_ecm(ps.S_c, ps.pi_c), mn=O.OModel.from_ecm(ps.S_n, ps.pi_n), ot=ot)
    O.set_sparse_leaves(False)          # the reference's dense loop (PhyloLik.ml:87-90)


def _cpu_noop(_):
    return os.getpid()


def _cpu_worker(job):
    key, lv, strategy = job
    O = _CPU["O"]
    x = lv.astype(np.int32)
    x[x >= 64] = -1
    t0 = time.perf_counter()
    r = O.score_region(_CPU["mc"], _CPU["mn"], _CPU["ot"], strategy, x)
    return key, r.score, r.status, r.evals, time.perf_counter() - t0


class CpuPool:
    """A persistent pool of one process per core (spawned, so no CUDA context crosses a fork),
    started and warmed up outside any timed region.  score() feeds a region list longest-first,
    one region per task, as the reference's `-p N` mode schedules its region list
    (src/PhyloCSF.ml:303-308)."""

    def __init__(self, name: str, cores: int):
        self.cores = cores
        self.pool = mp.get_context("spawn").Pool(cores, initializer=_cpu_init, initargs=(name,))
        self.pool.map(_cpu_noop, range(cores), chunksize=1)

    def score(self, jobs):
        """jobs: (key, leaves uint8 [L][nl], strategy); returns {key: (score, status, evals, seconds)}, wall."""
        order = sorted(jobs, key=lambda j: -j[1].shape[0])
        t0 = time.perf_counter()
        out = {k: v for k, *v in self.pool.imap_unordered(_cpu_worker, order, chunksize=1)}
        return out, time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()


def stratified(col_offsets, n: int, offset: int = 0):
    """n regions at evenly spaced length quantiles (sorted by length, ties by index)."""
    L = np.diff(col_offsets)
    order = np.lexsort((np.arange(len(L)), L))
    n = min(n, len(L))
    pos = np.unique(np.linspace(0, len(L) - 1, n).round().astype(np.int64))
    return order[(pos + offset) % len(L)]


def sample_leaves_np(spec, idx):
    """Leaf codes of regions idx of a workload, from the numpy restatement of the simulator."""
    from oracle import synth_np
    from phylocsf_gb300 import synth
    P, prior = synth.simulation_inputs(spec.params)
    out, L = [], np.diff(spec.col_offsets)
    lv = synth_np.simulate_regions(spec.params.tree.parent, P, prior, spec.col_offsets, spec.models, spec.gap_frac,
                                   spec.seed, idx)
    o = 0
    for r in idx:
        out.append(lv[o:o + L[r]])
        o += L[r]
    return out


def loaded_native_libs():
    """Shared libraries from this repository mapped into this process."""
    libs = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.startswith(ROOT) and ".so" in path:
                    libs.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(libs)


def workload_config(spec, world: int) -> dict:
    """The workload description both arms print (identical keys and values)."""
    nbytes = spec.total_cols * spec.params.tree.nl
    return {"workload": spec.name, "tree": spec.params.name, "strategy": "mle" if spec.strategy else "fixed",
            "regions_per_gpu": spec.n_regions, "columns_per_gpu": spec.total_cols,
            "l2": ("L2 flushed before every timed step (inputs %.0f MB)" if nbytes < 2 * L2_BYTES
                   else "inputs larger than L2 (%.0f MB)") % (nbytes / 1e6),
            "parallelism": "replicas" if world > 1 else "single GPU"}


# ---------------------------------------------------------------- reference arm
def run_reference(args, world, rank):
    if rank != 0:
        return
    spec = make_spec(args, seed=0)
    cores = args.cpu_cores or os.cpu_count() or 1
    nb = spec.params.tree.n - 1
    K = args.steps
    per_step = max(1, -(-args.ref_regions // K))
    sample = stratified(spec.col_offsets, per_step * K)
    steps = [sample[k::K] for k in range(K)]                 # each step a stratified slice
    warm = stratified(spec.col_offsets, 4 * cores)[:cores]   # the shortest regions: warm-up only
    lv = dict(zip(list(sample) + list(warm), sample_leaves_np(spec, list(sample) + list(warm))))
    pool = CpuPool(spec.params.name, cores)
    for _ in range(args.warmup):
        pool.score([(int(r), lv[r], spec.strategy) for r in warm])
    # the K steps' regions go to the pool as one longest-first list, so no core idles at a
    # step boundary; ms_per_step = wall / K
    jobs = [(int(r), lv[r], spec.strategy) for st in steps for r in st]
    out, wall = pool.score(jobs)
    pool.close()
    regions = len(jobs)
    L = np.diff(spec.col_offsets)
    cols = int(sum(L[r] for r in sample))
    v = regions / wall
    line = {"metric": METRIC, "value": v, "unit": "regions/s", "n_gpus": world, "steps": K,
            "warmup": args.warmup, "ms_per_step": 1000 * wall / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA, "impl": "reference",
            "config": workload_config(spec, world),
            "cpu_baseline": {"value": v, "unit": "regions/s", "cores": cores, "kind": "port",
                             "sample": "%d regions (%d codon columns) at evenly spaced length quantiles of the "
                                       "workload, %d per step, fed longest-first to a persistent pool of %d "
                                       "processes (nproc %d); FP64 oracle with the reference's dense loop"
                                       % (regions, cols, per_step, cores, os.cpu_count() or 0)},
            "e2e": {"value": v, "unit": "regions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "column_branches_per_s": sum(o[2] * L[k] for k, o in out.items()) * nb / wall,
            "columns_per_s": cols / wall,
            "evaluations": int(sum(o[2] for o in out.values())),
            "failed_regions": int(sum(1 for o in out.values() if o[1] != 0)),
            "native_libs_loaded": loaded_native_libs(),
            "note": "the reference is OCaml+GSL and cannot be built on this image; this arm times the C FP64 "
                    "restatement of its loop structure (oracle/)"}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm
def make_spec(args, seed):
    from phylocsf_gb300 import synth
    import phylocsf_gb300 as P
    if args.workload == "58mammals_mle":
        spec = synth.spec_58mammals_mle(n_regions=args.regions, seed=seed)
    elif args.workload == "12flies_fixed":
        spec = synth.spec_12flies_fixed(seed=seed)
    elif args.workload == "120mammals_fixed":
        spec = synth.spec_120mammals_fixed(total_cols=args.cols, seed=seed)
    elif args.workload == "100vertebrates_mle":
        spec = synth.spec_100vertebrates_mle(n_regions=args.regions, seed=seed)
    else:
        raise SystemExit("unknown workload " + args.workload + " (the reference arm takes the simulated-column "
                         "workloads: 58mammals_mle, 12flies_fixed, 120mammals_fixed, 100vertebrates_mle)")
    if args.strategy is not None:
        spec.strategy = P.FIXED if args.strategy == "fixed" else P.MLE
        spec.name = spec.name.replace("_mle", "_" + args.strategy).replace("_fixed", "_" + args.strategy)
    return spec


def measure_matmul_peaks(local):
    """Dense GEMM throughput of this GPU for the arithmetic types the kernels use but the
    driver's peak file does not cover: TF32 tensor cores (the search's products), FP32 on
    the CUDA cores (the SIMT kernels) and FP64 (the FP64 engine); cuBLAS through torch,
    best of 5 CUDA-event-timed multiplies after 2 warm-ups, 2 n^3 FLOPs each."""
    import torch
    dev = torch.device("cuda", local)
    keep = (torch.backends.cuda.matmul.allow_tf32, torch.backends.cudnn.allow_tf32)
    out = {}
    try:
        for name, dt, tf32, n in (("tf32", torch.float32, True, 8192), ("fp32", torch.float32, False, 8192),
                                  ("fp64", torch.float64, False, 4096)):
            torch.backends.cuda.matmul.allow_tf32 = tf32
            a = torch.randn(n, n, dtype=dt, device=dev)
            b = torch.randn(n, n, dtype=dt, device=dev)
            c = torch.empty(n, n, dtype=dt, device=dev)
            for _ in range(2):
                torch.matmul(a, b, out=c)
            best = 1e30
            for _ in range(5):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                torch.matmul(a, b, out=c)
                e1.record()
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            out[name + "_tflops"] = 2.0 * n ** 3 / (best / 1000.0) / 1e12
            del a, b, c
    finally:
        torch.backends.cuda.matmul.allow_tf32, torch.backends.cudnn.allow_tf32 = keep
    return out


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def load_traffic(kernel: str):
    """Per-column DRAM bytes of a kernel from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def run_ours(args, world, rank, local):
    import torch
    import phylocsf_gb300 as P

    from phylocsf_gb300 import synth
    if args.workload == "100vertebrates_6frame":
        # regions enumerated in six frames from nucleotide alignments and packed natively (the
        # MFA driver's path); the workload object carries what the config needs
        wl = spec = synth.workload_100vertebrates_6frame(n_regions=args.regions, seed=rank)
    else:
        spec = make_spec(args, seed=rank)
        wl = synth.realize(spec)
    ps = wl.params
    nl = ps.tree.nl
    nb = ps.tree.n - 1
    eng = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision=args.precision, device=local)
    stream = torch.cuda.ExternalStream(eng.stream_handle(), device=torch.device("cuda", local))
    batch = eng.batch(wl.col_offsets, wl.leaves)
    # column tile of the compensated FP32 kernel chosen by measurement on this tree and workload
    t_at = time.perf_counter()
    tile = eng.autotune(batch) if not args.no_autotune else None
    autotune_s = time.perf_counter() - t_at
    tc_shape_ms = None
    if tile is not None and eng.stats()["tc_shape"] >= 0:
        tc_shape_ms = {P.Engine.TC_SHAPES[k]: round(float(v), 3) for k, v in enumerate(eng.tc_shape_times())}
    gemm_peaks = measure_matmul_peaks(local) if rank == 0 else {}

    # inputs smaller than twice the L2 (129 MB) get an L2 flush before every timed step
    flush = None
    if wl.leaves.nbytes < 2 * L2_BYTES:
        flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=torch.device("cuda", local))

    def step():
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.fill_(0.0)
        return eng.score(batch, wl.strategy)

    for _ in range(args.warmup):
        res = step()
    clocks = ClockSampler(local) if rank == 0 else None
    eng.reset_stats()
    barrier(world)
    torch.cuda.synchronize(local)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        res = step()
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize(local)
    barrier(world)
    ms = ev0.elapsed_time(ev1)
    st = eng.stats()
    clk = clocks.stop() if clocks else None
    ms_max = max_over_ranks(ms, world)
    value = world * wl.n_regions * args.steps / (ms_max / 1000.0)
    colb_per_s = world * st["column_branches"] / (ms_max / 1000.0)

    # e2e: host buffers (pinned) -> pcsf_score_batch -> results on the host
    pin = torch.from_numpy(wl.leaves).pin_memory()
    leaves_pinned = pin.numpy()
    offs_pinned = torch.from_numpy(wl.col_offsets).pin_memory().numpy()
    barrier(world)
    torch.cuda.synchronize(local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.fill_(0.0)
        res_e2e = eng.score_batch(offs_pinned, leaves_pinned, wl.strategy)
    e1.record(stream)
    e1.synchronize()
    barrier(world)
    ms_e2e = max_over_ranks(e0.elapsed_time(e1), world)
    e2e_value = world * wl.n_regions * args.steps / (ms_e2e / 1000.0)
    same = bool(np.array_equal(res_e2e["score"], res["score"]))

    # roofline of the dominant pruning kernel (by device time): algorithmic FLOPs of its launches
    # (one product per contraction, whatever the split) over their device time.  The SIMT kernels
    # are CUDA-core FMA bound; they are reported against the measured tensor peak as the contract
    # requires, with the FP32 FMA ceiling alongside.
    peaks, peak_kind = load_peaks()
    kind = int(np.argmax(st["kind_ms"]))
    kname = KERNEL_NAMES[kind].format(prec=args.precision,
                                      tc="k_prune_bf16 (6 BF16 products)" if args.precision.startswith("bf16")
                                      else "k_prune_tc<3>")
    kcols = st["kind_columns"][kind]
    kflops = kcols * {0: flops_per_column, 1: flops_per_column, 2: flops_per_column_grad,
                      3: flops_per_column_tangent, 4: flops_per_column}[kind](nl)
    kms = st["kind_ms"][kind]
    launches = max(st["kind_launches"][kind], 1)
    achieved_tflops = kflops / (kms / 1000.0) / 1e12 if kms > 0 else 0.0
    peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
    sm_mhz = (clk or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    # the TF32 search executes three products per contraction (hi x hi, hi x lo, lo x hi)
    nprod = {"tf32x3": 3, "tf32x3b": 3, "tf32x3_direct": 3, "tf32": 1, "tf32_direct": 1}.get(args.precision)
    tf32_measured = gemm_peaks.get("tf32_tflops")
    traffic = load_traffic(KERNEL_KEYS[kind])
    traffic_per_launch = (traffic * kcols / launches) if traffic else None
    shares = {KERNEL_KEYS[k]: st["kind_ms"][k] / args.steps for k in range(NKINDS)}
    shares["pform"] = st["pform_ms"] / args.steps
    kinds = {KERNEL_KEYS[k]: {"launches_per_step": st["kind_launches"][k] / args.steps,
                              "column_evals_per_step": st["kind_columns"][k] / args.steps,
                              "ns_per_column_eval": (1e6 * st["kind_ms"][k] / st["kind_columns"][k]
                                                     if st["kind_columns"][k] else None)} for k in range(NKINDS)}

    line = {"metric": METRIC, "value": value, "unit": "regions/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPES.get(args.precision, args.precision),
            "data": DATA,
            "config": workload_config(spec, world),
            "precision": args.precision,
            "launch": {"ctas": {"simt_prune": st["prune_grid"], "tensor_core_prune": st["tc_grid"]},
                       "simt_tile": st["simt_tile"],
                       "tc_shape": P.Engine.TC_SHAPES.get(st["tc_shape"]),
                       "autotune": None if tile is None else {"chosen_tile": tile, "seconds": autotune_s,
                                                              "candidates": [64, 32],
                                                              "tc_shape_ms": tc_shape_ms}},
            "column_branches_per_s": colb_per_s,
            "e2e": {"value": e2e_value, "unit": "regions/s", "h2d_bytes_per_step": int(wl.leaves.nbytes +
                                                                                       wl.col_offsets.nbytes),
                    "d2h_bytes_per_step": int(res_e2e.nbytes), "same_scores_as_resident": same},
            "gpu_launches": int(st["kernel_launches"]),
            "rounds_per_step": st["rounds"] / args.steps,
            "evaluations_per_step": st["evaluations"] / args.steps,
            "roofline": {"kernel": kname, "bound": "tensor", "achieved": achieved_tflops,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved_tflops / peak,
                         "peak_kind": peak_kind + " bf16 sustained",
                         "traffic": traffic_per_launch, "alg_flops_per_launch": kflops / launches,
                         "avg_launch_ms": kms / launches, "launches": int(launches),
                         "fp32_fma_peak_tflops": fp32_peak, "frac_of_fp32_fma_peak": achieved_tflops / fp32_peak,
                         "gemm_peaks_measured": {k: round(v, 2) for k, v in gemm_peaks.items()},
                         "executed_tf32_tflops": (nprod * achieved_tflops if kind == 1 and nprod else None),
                         "frac_executed_of_tf32_measured": (nprod * achieved_tflops / tf32_measured
                                                            if kind == 1 and nprod and tf32_measured else None)},
            "kernel_ms_per_step": dict(shares, other=st["other_ms"] / args.steps),
            # P(t) formation as its own line: 2 * 64^3 FLOPs per branch of every P set when done
            # as GEMMs; one P set per (region, model, rho) evaluation at most (P sets are shared
            # by requests with the same model and rho), so this is an upper bound
            "pform": {"ms_per_step": st["pform_ms"] / args.steps, "launches_per_step": st["pform_launches"] / args.steps,
                      "psets_per_step_at_most": st["evaluations"] / args.steps,
                      "gemm_flops_per_pset": 2 * 64 ** 3 * nb,
                      "tflops_at_most": (st["evaluations"] * 2 * 64 ** 3 * nb / (st["pform_ms"] / 1000.0) / 1e12
                                         if st["pform_ms"] > 0 else None)},
            "pruning_kernels": kinds,
            "clocks": clk}

    if args.latency_batches > 0:
        # serving view: the regions arrive as B consecutive batches (host buffers, one
        # pcsf_score_batch call each); a region's latency is the time from the first
        # submission until its batch's results are on the host
        B = args.latency_batches
        cuts = np.linspace(0, wl.n_regions, B + 1).astype(np.int64)
        batch_ms, done_ms = [], []
        torch.cuda.synchronize(local)
        t_start = time.perf_counter()
        for k in range(B):
            r0, r1 = cuts[k], cuts[k + 1]
            o = wl.col_offsets[r0:r1 + 1] - wl.col_offsets[r0]
            lv = wl.leaves[wl.col_offsets[r0]:wl.col_offsets[r1]]
            t0 = time.perf_counter()
            eng.score_batch(np.ascontiguousarray(o), np.ascontiguousarray(lv), wl.strategy)
            t1 = time.perf_counter()
            batch_ms.append(1000 * (t1 - t0))
            done_ms.extend([1000 * (t1 - t_start)] * int(r1 - r0))
        total_s = time.perf_counter() - t_start
        line["latency"] = {"batches": B, "regions_per_batch": int(wl.n_regions // B),
                           "batch_ms_p50": float(np.percentile(batch_ms, 50)),
                           "batch_ms_p99": float(np.percentile(batch_ms, 99)),
                           "region_latency_ms_p50": float(np.percentile(done_ms, 50)),
                           "region_latency_ms_p99": float(np.percentile(done_ms, 99)),
                           "throughput_regions_per_s": wl.n_regions / total_s,
                           "clock": "host wall clock around each call (synchronous API)"}
    if rank == 0 and not args.no_fp64:
        # the plain FP64 GPU path (oracle-matched iterates) on a length-stratified sample: the
        # path the split-precision engine is compared against (time) and the accuracy
        # reference (scores)
        sub = stratified(wl.col_offsets, args.fp64_regions)
        parts = [wl.leaves[wl.col_offsets[i]:wl.col_offsets[i + 1]] for i in sub]
        so = np.zeros(len(sub) + 1, np.int64)
        so[1:] = np.cumsum([p.shape[0] for p in parts])
        e64 = P.Engine(ps.tree, ps.S_c, ps.pi_c, ps.S_n, ps.pi_n, precision="fp64", device=local)
        s64 = torch.cuda.ExternalStream(e64.stream_handle(), device=torch.device("cuda", local))
        b64 = e64.batch(so, np.concatenate(parts))
        warm = e64.batch(so[:9] - so[0], np.concatenate(parts[:8]))   # first launches (attributes, module load)
        e64.score(warm, wl.strategy)
        warm.close()
        torch.cuda.synchronize(local)
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(s64)
        r64 = e64.score(b64, wl.strategy)
        f1.record(s64)
        f1.synchronize()
        ms64 = f0.elapsed_time(f1)
        # the split-precision engine on the same sample, same clock, for a like-for-like ratio
        bs = eng.batch(so, np.concatenate(parts))
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(local)
        g0.record(stream)
        rs = eng.score(bs, wl.strategy)
        g1.record(stream)
        g1.synchronize()
        ms_s = g0.elapsed_time(g1)
        bs.close()
        b64.close()
        e64.close()
        d = np.abs(r64["score"] - res["score"][sub])
        line["fp64_gpu"] = {"regions": int(len(sub)), "columns": int(so[-1]), "ms": ms64,
                            "value": len(sub) / (ms64 / 1000.0), "unit": "regions/s",
                            "split_precision_ms_same_sample": ms_s,
                            "speedup_same_sample": ms64 / ms_s,
                            "speedup_vs_headline_value": value / (len(sub) / (ms64 / 1000.0)),
                            "sample": "regions at evenly spaced length quantiles of the workload"}
        line.setdefault("accuracy", {})["vs_fp64_gpu"] = {
            "regions": int(len(sub)), "max_abs_db": float(d.max()), "median_abs_db": float(np.median(d)),
            "frac_le_1e-3_db": float((d <= 1e-3).mean()),
            "failed": int((r64["status"] != 0).sum() + (res["status"][sub] != 0).sum()),
            "same_scores_on_sample": bool(np.array_equal(rs["score"], res["score"][sub]))}
    if rank == 0 and not args.no_cpu_baseline:
        # the FP64 oracle port (the reference's dense loop) on a length-stratified sample: its time
        # is the CPU baseline, its scores the oracle check of the returned scores
        cores = args.cpu_cores or os.cpu_count() or 1
        idx = stratified(wl.col_offsets, args.cpu_regions, offset=1)
        pool = CpuPool(ps.name, cores)
        out, wall = pool.score([(int(i), wl.leaves[wl.col_offsets[i]:wl.col_offsets[i + 1]], wl.strategy)
                                for i in idx])
        pool.close()
        d = np.abs(np.array([out[int(i)][0] for i in idx]) - res["score"][idx])
        cols = int(sum(wl.col_offsets[i + 1] - wl.col_offsets[i] for i in idx))
        line["cpu_baseline"] = {"value": len(idx) / wall, "unit": "regions/s", "cores": cores, "kind": "port",
                                "sample": "%d regions (%d codon columns) at evenly spaced length quantiles of the "
                                          "workload, fed longest-first to a persistent pool of %d processes "
                                          "(nproc %d); FP64 oracle with the reference's dense loop"
                                          % (len(idx), cols, cores, os.cpu_count() or 0),
                                "wall_s": wall}
        line.setdefault("accuracy", {})["vs_fp64_oracle"] = {
            "regions": int(len(idx)), "max_abs_db": float(d.max()), "median_abs_db": float(np.median(d)),
            "frac_le_1e-3_db": float((d <= 1e-3).mean())}
    if rank == 0:
        line["native_libs_loaded"] = loaded_native_libs()
        print(json.dumps(line), flush=True)
    batch.close()
    eng.close()


def run_omega(args, world, rank, local):
    """The differentiation configuration: the OmegaModel gradient with respect to every branch
    length, rho, kappa and omega for alignments of 200-2,000 codons on 100vertebrates simulated at
    per-alignment omega; one step = one pcsf_omega_grad over the whole batch."""
    import torch
    import phylocsf_gb300 as P
    from phylocsf_gb300 import synth, omega_fit
    wl = synth.workload_100vertebrates_omega(n_alignments=args.regions, seed=rank)
    prec = args.precision if args.precision != "tf32x3b" else "fp32b"
    eng = P.Engine.for_tree(wl.tree, precision=prec, device=local)
    stream = torch.cuda.ExternalStream(eng.stream_handle(), device=torch.device("cuda", local))
    b = eng.batch(wl.col_offsets, wl.leaves)
    for _ in range(args.warmup):
        g = eng.omega_grad(b, wl.kappa, wl.omega, 1.0, wl.sigma)
    clocks = ClockSampler(local) if rank == 0 else None
    barrier(world)
    torch.cuda.synchronize(local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        g = eng.omega_grad(b, wl.kappa, wl.omega, 1.0, wl.sigma)
    e1.record(stream)
    e1.synchronize()
    barrier(world)
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    clk = clocks.stop() if clocks else None
    value = world * wl.n_regions * args.steps / (ms / 1000.0)
    nbr = wl.tree.n - 1
    line = {"metric": "OmegaModel gradient (every branch, rho, kappa, omega): alignments/s", "value": value,
            "unit": "alignments/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPES.get(prec, prec) + ", P(t) and its eigenbasis derivative f64", "data": DATA,
            "config": {"workload": wl.name, "tree": "100vertebrates", "alignments_per_gpu": wl.n_regions,
                       "columns_per_gpu": wl.total_cols, "gradient_entries_per_alignment": nbr + 3,
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (%.0f MB)" % (wl.leaves.nbytes / 1e6)},
            "column_branches_per_s": world * wl.total_cols * nbr * args.steps / (ms / 1000.0),
            "clocks": clk}
    if rank == 0:
        # against the FP64 engine on alignments at evenly spaced length quantiles
        sub = stratified(wl.col_offsets, args.fp64_regions)
        parts = [wl.leaves[wl.col_offsets[i]:wl.col_offsets[i + 1]] for i in sub]
        so = np.zeros(len(sub) + 1, np.int64)
        so[1:] = np.cumsum([x.shape[0] for x in parts])
        e64 = P.Engine.for_tree(wl.tree, precision="fp64", device=local)
        b64 = e64.batch(so, np.concatenate(parts))
        t0 = time.perf_counter()
        g64 = e64.omega_grad(b64, wl.kappa, wl.omega[sub], 1.0, wl.sigma)
        t64 = time.perf_counter() - t0
        # the gradient is taken at the simulated parameters, near the optimum, where the true
        # derivatives are small: besides the relative error (floor 1e-2) report the absolute
        # error and the absolute error over sqrt(columns), the scale of the derivative's
        # column-to-column fluctuation
        rel, med, absmax, per_sqrt = {}, {}, {}, {}
        ncol = np.diff(so).astype(np.float64)
        for k in ("d_kappa", "d_omega", "d_rho", "d_branch"):
            a, c = g64[k], g[k][sub]
            err = np.abs(c - a)
            r = err / (np.abs(a) + 1e-2)
            rel[k] = float(np.max(r))
            med[k] = float(np.median(r))
            absmax[k] = float(np.max(err))
            scale = np.sqrt(ncol).reshape((-1,) + (1,) * (err.ndim - 1))
            per_sqrt[k] = float(np.max(err / scale))
        line["accuracy"] = {"vs_fp64_gpu": {"alignments": int(len(sub)), "max_rel_error": rel,
                                            "median_rel_error": med, "max_abs_error": absmax,
                                            "max_abs_error_per_sqrt_column": per_sqrt,
                                            "lpr_max_rel": float(np.max(np.abs(g["lpr"][sub] - g64["lpr"]) /
                                                                        np.abs(g64["lpr"])))},
                            "fp64_seconds_on_sample": t64}
        # gradient MAP (rho, kappa at omega = 1) beside the reference's Brent coordinate ascent (H0)
        bs = eng.batch(so, np.concatenate(parts))
        t0 = time.perf_counter()
        brent = eng.omega_score(bs)
        tb = time.perf_counter() - t0
        t0 = time.perf_counter()
        gm = omega_fit.gradient_map(eng, bs, omega=1.0, sigma=1.0)
        tg = time.perf_counter() - t0
        t0 = time.perf_counter()
        fo = omega_fit.gradient_map(eng, bs, sigma=1.0, fit_omega=True, iters=60)
        to = time.perf_counter() - t0
        gap = gm["objective"] - (brent["lpr_h0"] + omega_fit.log_prior_rho(brent["rho_h0"]))
        L = np.diff(so)
        line["fits"] = {"alignments": int(len(sub)),
                        "brent_kr_map_seconds": tb, "brent_evaluations_mean": float(np.mean(brent["evals"])),
                        "gradient_map_seconds": tg, "gradient_map_evaluations_mean": float(np.mean(gm["evals"])),
                        "objective_gap_gradient_minus_brent": {"min": float(gap.min()), "max": float(gap.max())},
                        "omega_mle_seconds": to,
                        "omega_mle_log_ratio_to_simulated": {
                            "median_abs": float(np.median(np.abs(np.log(fo["omega"] / wl.omega[sub])))),
                            "median_abs_1000_codons_or_more": float(np.median(np.abs(
                                np.log(fo["omega"][L >= 1000] / wl.omega[sub][L >= 1000])))) if (L >= 1000).any() else None}}
        line["native_libs_loaded"] = loaded_native_libs()
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="58mammals_mle")
    ap.add_argument("--regions", type=int, default=10000)
    ap.add_argument("--cols", type=int, default=2_000_000)
    ap.add_argument("--precision", default="tf32x3b")
    ap.add_argument("--strategy", default=None, choices=[None, "fixed", "mle"],
                    help="override the workload's strategy (fixed: one likelihood pass, used for profiling)")
    ap.add_argument("--fp64-regions", type=int, default=1024,
                    help="regions of the workload timed on the FP64 GPU path (and compared with it)")
    ap.add_argument("--cpu-regions", type=int, default=64,
                    help="regions of the workload timed on the CPU port (and compared with it)")
    ap.add_argument("--ref-regions", type=int, default=128,
                    help="reference arm: regions timed over all steps")
    ap.add_argument("--cpu-cores", type=int, default=0)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default column tile of the FP32 kernel")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--latency-batches", type=int, default=0,
                    help="also score the workload as this many consecutive batches and report latency percentiles")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    world, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "100vertebrates_omega":
        run_omega(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
