"""Benchmark of the RDME timestep on GB300.

Default workload: the 256^3, 16-slot, 16-species / 30-reaction multi-region
lattice (the roofline configuration), production path (Philox, FP32
propensities with FP64 clock), the autotuned step variant (the sweep stream:
two or three launches per frame, or one persistent launch per call).  `value`
is voxel-steps/s over the whole job with the lattice resident in HBM; the
lattice (2 x 256 MiB) is larger
than L2, so no flush is needed between timed frames.  Five more timed calls
of the same length follow (`repeats`: their median and spread; the headline
is the first call alone).  Also reported: the
batched 512-replicate ensemble vs the plain one-launch-group-per-replicate
path (replicate-steps/s), the reference-RNG CUDA path on the same lattice,
an end-to-end number through the C ABI, the frame's roofline (algorithmic
bytes over the frame time, with the profiled DRAM traffic of its longest
launch) and a CPU baseline (the oracle's reference-semantics port, OpenMP on
the host cores).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --ensemble-only --variant V --steps K   (the ensemble leg alone, for profiling)
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "voxel-steps/s and replicate-steps/s, batched vs plain, 1 GB300, KS-matched"
UNIT = "voxel-steps/s"
N_REPEATS = 5  # timed calls after the headline one, for the median and spread
# lattices the main leg can run (--workload): the 256^3 multi-region cell is the headline
WORKLOADS = {"c1": "c1_plain_2d", "c2": "c2_single_cell", "c3": "c3_multi_region", "c5": "c5_stiff"}


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier and max-over-ranks via torch.distributed when WORLD_SIZE > 1."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms with a host timestamp per row.

    A timed region of a few milliseconds is shorter than nvidia-smi's sampling interval, so the
    benchmark keeps the GPU busy with untimed frames right after the timed region until the
    window that starts at the timed region holds at least three rows, and reports the rows of that
    window (`window` in the result says so)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.rows: list[tuple[float, list[str]]] = []

    def start(self, wait_s: float = 5.0):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, bufsize=1)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.rows and time.perf_counter() - t0 < wait_s and self.proc.poll() is None:
            time.sleep(0.02)

    def _read(self):
        for line in self.proc.stdout:
            if line.count(",") >= 8:
                self.rows.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def rows_since(self, t: float) -> int:
        return sum(1 for ts, _ in self.rows if ts >= t)

    def alive(self) -> bool:
        return self.proc is not None and self.proc.poll() is None

    def stop(self, t_from: float, t_to: float):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        rows = [r for ts, r in self.rows if t_from <= ts <= t_to]
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(r[1]) for r in rows) if v is not None]
        mx = [v for v in (num(r[2]) for r in rows) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "window": "the timed region, the end-to-end and repeat calls after it and the untimed "
                          "frames that follow (one window; the GPU idles only in the end-to-end loop's "
                          "host waits)"}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu summaries."""
    key = re.escape(f"{kernel}/{workload}")
    for f in sorted((ROOT / "profiles").glob("*.md")):
        m = re.search(rf"traffic_bytes_per_launch\[{key}\]:\s*([0-9.eE+]+)", f.read_text())
        if m:
            return float(m.group(1))
    return None


def central_slab(workload, nx: int):
    """The nx planes through the centre of a workload's lattice, cut out of the full lattice (same
    particles, regions and tables): reference-layout arguments and state for the oracle.  The slab's
    faces act as the lattice boundary."""
    import oracle

    sim = workload.sim
    i = sim.info()
    X, Y, Z = (int(r) for r in i.res)
    K, S1 = i.max_particles_site, i.n_species + 1
    x0 = max(0, X // 2 - nx // 2)
    x1 = min(X, x0 + nx)
    s, o, c = sim.get_lattice()
    tab = sim.tables()
    cut = lambda a, w: np.ascontiguousarray(a.reshape(X, Y, Z * w)[x0:x1]).reshape(-1)
    t = type(tab)(cut(tab.regions, 1), tab.diffusion, tab.stoich, tab.reactants, tab.rates, cut(tab.reservoir, 1))
    s, o, c = cut(s, K), cut(o, 1), cut(c, S1)
    st = c.reshape(-1, S1).sum(0).astype(np.int32)
    args = ((x1 - x0, Y, Z), K, i.n_regions, i.n_species, i.n_reactions, float(np.float32(i.tau)),
            float(np.float32(i.lambda_)), t)
    V = (x1 - x0) * Y * Z
    desc = (f"the {x1 - x0}x{Y}x{Z} x-slab through the centre of {workload.name}, cut out of the full lattice "
            f"({V} voxels, {int((s > 0).sum())} particles: the full lattice's own particles and regions)")
    return args, oracle.RefState(s, o, c, st), V, desc


def cpu_reference_rate(workload, nx: int, budget_s: float, threads: int, max_frames: int = 100_000):
    """The oracle's reference-semantics step (gather form, OpenMP) on a slab of a workload:
    frames until budget_s has passed; returns (voxel-steps/s, sample description)."""
    import oracle

    oracle.build()
    args, state, V, desc = central_slab(workload, nx)
    it = (np.arange(max_frames + 1, dtype=np.uint64) * 7919 + 12345).astype(np.uint32)
    oracle.ref_run(*args, state, it[:1], mode=1, threads=threads)  # warm-up
    t0 = time.perf_counter()
    n, chunk = 0, 1
    while time.perf_counter() - t0 < budget_s and n + chunk <= max_frames:
        oracle.ref_run(*args, state, it[1 + n:1 + n + chunk], mode=1, threads=threads)
        n += chunk
        if time.perf_counter() - t0 < budget_s / 20:
            chunk = min(chunk * 2, 1000)
    dt = time.perf_counter() - t0
    return V * n / dt, f"{n} reference-semantics frames of {desc}"


CPU_SLAB = 8  # planes of the 256^3 cell in the CPU samples (cpu_baseline and the reference arm)
CPU_SLABS = {"c1": 64, "c2": 16, "c3": CPU_SLAB, "c5": 8}  # the same, per workload (c1: the whole lattice)


def reference_arm(args, rank, world):
    """The reference's algorithm on the host cores: the oracle's restatement of the WGSL shaders
    (the reference itself needs Vulkan and a Rust toolchain), on the same central slab of the
    workload's lattice as cpu_baseline (the 256^3 cell by default).  The slab is cut from the
    lattice the product library's host model builder makes (outside the timed region); the timed
    loop runs the oracle alone."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle
    from cell_simulation_gb300 import configs

    oracle.build()
    w = getattr(configs, WORKLOADS[args.workload])()
    nx = CPU_SLABS[args.workload]
    a, state, V, desc = central_slab(w, nx)
    n_total = args.warmup + args.steps
    it = (np.arange(n_total, dtype=np.uint64) * 7919 + 12345).astype(np.uint32)
    oracle.ref_run(*a, state, it[:args.warmup], mode=1, threads=threads)
    t0 = time.perf_counter()
    oracle.ref_run(*a, state, it[args.warmup:], mode=1, threads=threads)
    dt = time.perf_counter() - t0
    value = V * args.steps / dt
    sample = f"each step: one reference-semantics frame of {desc}"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": f"{w.name} ({nx}-plane central x-slab)",
                       "rng": "reference PCG", "threads": threads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def describe_variant(i):
    from cell_simulation_gb300 import tiling_kinds, tiling_launches, tiling_variants
    k, ty, tz, nt = tiling_variants()[i]
    kind, bx = tiling_kinds()[i]
    if kind == 1:
        return {"index": i, "kind": "brick", "slots": k, "brick": [bx, ty, tz], "threads": nt}
    if kind == 3:  # one block per replicate, every frame of a step call in one launch
        return {"index": i, "kind": "resident", "slots": k, "threads": nt, "multi_frame": True,
                "launches_per_call": 1}
    if kind == 2:
        if ty == 1:  # the persistent form: every frame of a step call in one launch
            return {"index": i, "kind": "stream", "slots": k, "words_per_group": 32, "threads": nt,
                    "passes_per_frame": 2, "multi_frame": True, "launches_per_call": 1}
        return {"index": i, "kind": "stream", "slots": k, "words_per_group": 32, "threads": nt,
                "passes_per_frame": tiling_launches()[i]}
    return {"index": i, "kind": "tile", "slots": k, "tile": [ty, tz], "threads": nt}


def launches_per_frame(i):
    """Kernel launches per frame of variant i once a run is under way: the sweep stream's passes
    (two where the Y and Z sweeps are one launch, else three), a brick pass and the pass over its
    spilled bricks, or one tile-pipeline launch.  The persistent sweep stream runs a whole step
    call in one launch: 1 here, see launches_in_call."""
    from cell_simulation_gb300 import tiling_launches
    return tiling_launches()[i]


def launches_in_call(i, frames):
    """Kernel launches of one step call of `frames` frames with variant i (none for pass 0, which
    runs only when the x-decisions are stale)."""
    if describe_variant(i).get("multi_frame"):
        return 1
    return frames * launches_per_frame(i)


def frame_kernels(desc):
    """The kernels of one frame of a variant, as named in the committed ncu summaries."""
    if desc["kind"] == "stream":
        if desc.get("multi_frame"):
            return ["sweep_frames_kernel"]
        if desc["passes_per_frame"] == 2:
            return ["sweep_pass_kernel<1>", "sweep_pass_kernel<5>"]
        return ["sweep_pass_kernel<1>", "sweep_pass_kernel<2>", "sweep_pass_kernel<3>"]
    if desc["kind"] == "resident":
        return ["resident_frames_kernel"]
    return ["brick_step_kernel"] if desc["kind"] == "brick" else ["prod_step_kernel"]


def ensemble_numbers(device, steps_batched=5000, steps_plain=200, variant=-1):
    """The 512-replicate ensemble: batched (one launch per pass for all replicates) against plain
    (one launch group per replicate), replicate-steps/s."""
    from cell_simulation_gb300 import Ensemble, configs

    tmpl = configs.c4_ensemble_template(K=8)
    res, seeds, mult, init = configs.c4_ensemble_spec()
    ens = Ensemble(tmpl, res, seeds, mult, init, device=device)
    tot, items = ens.info()
    if variant >= 0:
        ens.set_tiling(variant)
    else:
        variant, _ = ens.autotune(3)
    per_frame = launches_per_frame(variant)
    ens.step(3, batched=True)
    ms_b = ens.step_timed(steps_batched, batched=True)
    ens.step(1, batched=False)
    ms_p = ens.step_timed(steps_plain, batched=False)
    n = len(res)
    rb = n * steps_batched / (ms_b / 1e3)
    rp = n * steps_plain / (ms_p / 1e3)
    peak, _ = measured_peaks()
    out = {"workload": f"c4_ensemble_{n}rep_L32-96_K8", "total_voxels": int(tot), "work_items": int(items),
           "replicate_steps_per_s_batched": rb, "replicate_steps_per_s_plain": rp,
           "voxel_steps_per_s_batched": tot * steps_batched / (ms_b / 1e3),
           "batched_over_plain": rb / rp, "steps_batched": steps_batched, "steps_plain": steps_plain,
           "ms_per_step_batched": ms_b / steps_batched, "ms_per_step_plain": ms_p / steps_plain,
           "roofline_frac_batched": tot * steps_batched / (ms_b / 1e3) * 17 / 1e9 / peak,
           "launches_per_frame_batched": per_frame,
           "launches_per_frame_plain": n * (2 if describe_variant(variant).get("multi_frame") else per_frame),
           "variant": describe_variant(variant)}
    ens.close()
    return out


def philox_leg(workload, device, steps, warmup=5, tune_frames=5):
    """The production step of one workload (autotuned), timed with CUDA events."""
    from cell_simulation_gb300 import PREC_MIXED, RNG_PHILOX
    sim = workload.sim
    info = sim.info()
    V, K = int(info.n_voxels), info.max_particles_site
    sim.prepare_for_gpu(RNG_PHILOX, device)
    sim.set_precision(PREC_MIXED)
    variant, _ = sim.autotune(tune_frames)
    sim.step_philox(warmup, 7)
    ms = sim.step_philox_timed(steps, 7)
    sim.close()
    peak, _ = measured_peaks()
    rate = V * steps / (ms / 1e3)
    return {"voxel_steps_per_s": rate, "ms_per_step": ms / steps, "steps": steps, "voxels": V,
            "roofline_frac": rate * (2 * K + 1) / 1e9 / peak, "variant": describe_variant(variant)}


def reference_rng_leg(workload, device, steps, warmup=3):
    """The reference-RNG (bit-parity) CUDA path of one workload, timed with CUDA events."""
    from cell_simulation_gb300 import RNG_REFERENCE
    sim = workload.sim
    V = int(sim.info().n_voxels)
    sim.prepare_for_gpu(RNG_REFERENCE, device)
    it = (np.arange(warmup + steps, dtype=np.uint64) * 7919 + 12345).astype(np.uint32)
    sim.step(it[:warmup])
    ms = sim.step_timed(it[warmup:])
    sim.close()
    return {"voxel_steps_per_s": V * steps / (ms / 1e3), "ms_per_step": ms / steps, "steps": steps, "voxels": V}


def config_legs(device, cpu_budget, threads, with_cpu):
    """Every named configuration other than the headline: GPU production and reference-RNG paths,
    and the CPU restatement on a slab of the same lattice."""
    from cell_simulation_gb300 import configs
    out = {}
    c1 = {"philox": philox_leg(configs.c1_plain_2d(), device, 10_000, tune_frames=20),
          "reference_rng": reference_rng_leg(configs.c1_plain_2d(), device, 10_000)}
    c2 = {"philox": philox_leg(configs.c2_single_cell(), device, 1000),
          "reference_rng": reference_rng_leg(configs.c2_single_cell(), device, 100)}
    c5 = {"philox": philox_leg(configs.c5_stiff(), device, 200),
          "reference_rng": reference_rng_leg(configs.c5_stiff(), device, 50)}
    if with_cpu:
        for leg, w, nx in ((c1, configs.c1_plain_2d(), 64), (c2, configs.c2_single_cell(), 16),
                           (c5, configs.c5_stiff(), 8)):
            rate, sample = cpu_reference_rate(w, nx, cpu_budget, threads)
            leg["cpu_reference_semantics"] = {"voxel_steps_per_s": rate, "cores": threads, "sample": sample}
    out["c1_plain_64x64x1_K8"] = c1
    out["c2_single_cell_128x128x128_K16"] = c2
    out["c5_stiff_192x192x192_K16"] = c5
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="skip the ensemble, other configurations, "
                                                             "reference-RNG, e2e and CPU legs")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--variant", type=int, default=-1, help="step variant index (default: autotuned)")
    ap.add_argument("--workload", default="c3", choices=sorted(WORKLOADS),
                    help="the lattice of the main leg (default: the 256^3 multi-region cell)")
    ap.add_argument("--ensemble-only", action="store_true",
                    help="only the 512-replicate ensemble leg: --steps batched frames, a tenth as many plain ones "
                         "(for profiling; prints that leg's numbers)")
    ap.add_argument("--refrng-only", action="store_true",
                    help="only the reference-RNG CUDA path on the --workload lattice: --steps frames (for profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = env_rank()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return

    import __graft_entry__
    __graft_entry__.build()
    from cell_simulation_gb300 import PREC_MIXED, RNG_PHILOX, configs
    if args.ensemble_only:
        print(json.dumps(ensemble_numbers(local, args.steps, max(1, args.steps // 10), args.variant)), flush=True)
        return
    if args.refrng_only:
        w = getattr(configs, WORKLOADS[args.workload])()
        print(json.dumps(reference_rng_leg(w, local, args.steps, args.warmup)), flush=True)
        return

    dist = Dist(world)
    device = local
    seed = 0xC0FFEE + rank
    t_setup = time.perf_counter()
    w = getattr(configs, WORKLOADS[args.workload])()
    sim = w.sim
    info = sim.info()
    V, K, S1 = int(info.n_voxels), info.max_particles_site, info.n_species + 1
    t_build = time.perf_counter() - t_setup
    t0 = time.perf_counter()
    sim.prepare_for_gpu(RNG_PHILOX, device)
    t_upload = time.perf_counter() - t0
    sim.set_precision(PREC_MIXED)
    if args.variant >= 0:
        variant = args.variant
        sim.set_tiling(variant)
    else:
        variant, _ = sim.autotune(10)  # state restored: the timed frames start from the same lattice
    clocks = ClockSampler(device)
    clocks.start()
    sim.step_philox(args.warmup, seed)
    sim.synchronize()
    dist.barrier()
    t_region = time.perf_counter()
    ms = sim.step_philox_timed(args.steps, seed)
    dist.barrier()
    # end to end through the C ABI, right after the timed frames (the frame time grows slowly as the
    # lattice evolves, so both numbers cover the same stretch of frames): every frame one step call
    # (its frame number up, 4 bytes; the seed is uploaded only when it changes) and one blocking
    # read of the species counts (down), like the reference's per-frame itime write, submit and
    # stats readback
    n_e2e = 500  # step calls timed, whatever --steps is: a call lasts about 0.17 ms
    # untimed warm-up calls of the same loop: one-frame calls of either parity run their own
    # captured graph, made on its first use
    for _ in range(args.warmup):
        sim.step_philox(1, seed)
        sim.counts()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        sim.step_philox(1, seed)
        sim.counts()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * V * n_e2e / dist.max(e2e_s), "unit": UNIT, "h2d_bytes_per_step": 4,
           "d2h_bytes_per_step": S1 * 8, "steps": n_e2e,
           "setup_s": {"host_model_build": t_build, "upload_prepare_for_gpu": t_upload}}
    # five more timed calls of the same length, continuing from the lattice the timed call left:
    # their median and spread beside the single timed call the headline is taken from
    rep_ms = []
    for _ in range(N_REPEATS):
        r = sim.step_philox_timed(args.steps, seed)
        dist.barrier()
        rep_ms.append(dist.max(r) / args.steps)
    # keep the GPU busy (untimed frames) until the clock window holds three samples
    t_hold = time.perf_counter()
    while clocks.alive() and clocks.rows_since(t_region) < 3 and time.perf_counter() - t_hold < 5.0:
        sim.step_philox(200, seed)
        sim.synchronize()
    clk = clocks.stop(t_region, time.perf_counter())
    ms_max = dist.max(ms)
    value = world * V * args.steps / (ms_max / 1e3)
    frame_s = ms / 1e3 / args.steps
    lat_mib = V * K / 2**20
    l2_note = (f"inputs larger than L2 (2 x {lat_mib:.0f} MiB lattice buffers)" if 2 * V * K > 129e6 else
               f"inputs smaller than L2 (2 x {lat_mib * 1024:.0f} KiB lattice buffers), not flushed")
    peak, peak_kind = measured_peaks()
    alg_bytes = V * (2 * K + 1)
    achieved = alg_bytes / frame_s / 1e9
    desc = describe_variant(variant)
    kernels = frame_kernels(desc)
    longest = "sweep_pass_kernel<5>" if "sweep_pass_kernel<5>" in kernels else (
        "sweep_pass_kernel<3>" if "sweep_pass_kernel<3>" in kernels else kernels[0])
    traffic = profiled_traffic(longest, w.name)
    per_kernel = {k: profiled_traffic(k, w.name) for k in kernels}
    frame_dram = sum(per_kernel.values()) if all(v is not None for v in per_kernel.values()) else None
    diag = sim.diagnostics()

    sim.close()

    extras = {}
    threads = os.cpu_count() or 1
    if not args.no_extras and rank == 0:
        extras["ensemble"] = ensemble_numbers(device)
        extras["reference_rng_path"] = reference_rng_leg(configs.c3_multi_region(), device, 100)
        extras["configs"] = config_legs(device, min(args.cpu_budget, 4.0), threads, world == 1)
    cpu = None
    if not args.no_extras and rank == 0 and world == 1:
        rate, sample = cpu_reference_rate(getattr(configs, WORKLOADS[args.workload])(), CPU_SLABS[args.workload],
                                          args.cpu_budget, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    dist.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8", "data": "synthetic",
        "config": {"workload": w.name, "voxels": V, "slots_per_voxel": K, "species": S1 - 1,
                   "reactions": int(info.n_reactions), "rng": "philox4x32-10", "precision": "fp32 propensities, fp64 clock",
                   "l2": l2_note, "parallelism": f"replicas x{world}",
                   "variant": desc},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes, "kernel": longest,
                     "achieved_over": "frame time (every launch of the frame)",
                     # the persistent kernel runs every frame of a call in one launch: its bytes are
                     # per frame of that launch
                     "traffic_per": "frame" if desc.get("multi_frame") else "launch",
                     "frame_dram_bytes": frame_dram, "frame_dram_bytes_per_kernel": per_kernel,
                     "dram_frac": (frame_dram / frame_s / 1e9 / peak) if frame_dram else None,
                     "dram_frac_note": "the frame's profiled DRAM bytes (every launch, one cold-cache ncu capture) "
                                       "over the measured frame time, against the measured copy bandwidth"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches_in_call(variant, args.steps),
        "clocks": clk,
        "repeats": {"calls": N_REPEATS, "frames_per_call": args.steps, "ms_per_step": rep_ms,
                    "median_ms_per_step": statistics.median(rep_ms),
                    "median_value": world * V / (statistics.median(rep_ms) / 1e3),
                    "note": "further timed calls after the one the headline is taken from, each continuing "
                            "from the lattice the previous call left"},
        "diagnostics": {"events": int(diag[0]), "rejected_capacity": int(diag[1]), "event_cap": int(diag[2]),
                        "fp64_selections": int(diag[3]), "ssa_voxels": int(diag[6]), "wait_timeouts": int(diag[7])},
    }
    line.update(extras)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
