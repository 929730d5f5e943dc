"""Benchmark of the RDME timestep on GB300.

Default workload: the 256^3, 16-slot, 16-species / 30-reaction multi-region
lattice (the roofline configuration), production path (Philox, FP32
propensities with FP64 clock), the autotuned step variant (the sweep stream:
three or four launches per frame).  `value` is voxel-steps/s over the whole
job with the lattice resident in HBM; the lattice (2 x 256 MiB) is larger
than L2, so no flush is needed between timed frames.  Also reported: the
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
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        rows = [[x.strip() for x in l.split(",")] for l in self.lines if l.count(",") >= 8]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


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


def cpu_reference_rate(budget_s: float, threads: int):
    """Oracle reference-semantics step (gather + OpenMP) on an x-slab through
    the centre of the 256^3 multi-region cell; returns (voxel-steps/s, sample)."""
    import oracle
    from cell_simulation_gb300 import configs

    oracle.build()
    nx = 8
    w = configs.c3_multi_region(res=(nx, 256, 256), total_particles=int(1_000_000 * nx / 256))
    sim = w.sim
    i = sim.info()
    s, o, c = sim.get_lattice()
    st = c.reshape(-1, i.n_species + 1).sum(0).astype(np.int32)
    state = oracle.RefState(s, o, c, st)
    args = (tuple(i.res), i.max_particles_site, i.n_regions, i.n_species, i.n_reactions, float(np.float32(i.tau)),
            float(np.float32(i.lambda_)), sim.tables())
    it = (np.arange(10_000, dtype=np.uint64) * 7919 + 12345).astype(np.uint32)
    oracle.ref_run(*args, state, it[:1], mode=1, threads=threads)  # warm-up
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < budget_s and n < len(it) - 1:
        oracle.ref_run(*args, state, it[1 + n:2 + n], mode=1, threads=threads)
        n += 1
    dt = time.perf_counter() - t0
    V = int(np.prod(i.res))
    return V * n / dt, f"{n} reference-semantics frames of the {nx}x256x256 x-slab through the cell centre " \
                       f"(membrane, cytoplasm, nucleus; {V} voxels, same particle density)"


def reference_arm(args, rank, world):
    """The reference's algorithm on the host cores (the oracle's port of the
    WGSL shaders: the reference itself needs Vulkan and a Rust toolchain)."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle
    from cell_simulation_gb300 import configs

    oracle.build()
    nx = 4
    w = configs.c3_multi_region(res=(nx, 256, 256), total_particles=int(1_000_000 * nx / 256))
    sim = w.sim
    i = sim.info()
    s, o, c = sim.get_lattice()
    st = c.reshape(-1, i.n_species + 1).sum(0).astype(np.int32)
    state = oracle.RefState(s, o, c, st)
    a = (tuple(i.res), i.max_particles_site, i.n_regions, i.n_species, i.n_reactions, float(np.float32(i.tau)),
         float(np.float32(i.lambda_)), sim.tables())
    n_total = args.warmup + args.steps
    it = (np.arange(n_total, dtype=np.uint64) * 7919 + 12345).astype(np.uint32)
    oracle.ref_run(*a, state, it[:args.warmup], mode=1, threads=threads)
    t0 = time.perf_counter()
    oracle.ref_run(*a, state, it[args.warmup:], mode=1, threads=threads)
    dt = time.perf_counter() - t0
    V = int(np.prod(i.res))
    value = V * args.steps / dt
    sample = (f"each step: one reference-semantics frame of the {nx}x256x256 x-slab through the centre of the "
              f"256^3 multi-region cell ({V} voxels, same particle density)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "c3_multi_region_256x256x256_K16 (x-slab sample)", "rng": "reference PCG",
                       "threads": threads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def describe_variant(i):
    from cell_simulation_gb300 import tiling_kinds, tiling_variants
    k, ty, tz, nt = tiling_variants()[i]
    kind, bx = tiling_kinds()[i]
    if kind == 1:
        return {"index": i, "kind": "brick", "slots": k, "brick": [bx, ty, tz], "threads": nt}
    if kind == 2:
        from cell_simulation_gb300 import tiling_launches
        return {"index": i, "kind": "stream", "slots": k, "words_per_group": 32, "threads": nt,
                "passes_per_frame": tiling_launches()[i]}
    return {"index": i, "kind": "tile", "slots": k, "tile": [ty, tz], "threads": nt}


def launches_per_frame(i):
    """Kernel launches per frame of variant i: a brick pass with bounded pools is
    followed by the pass over its spilled bricks; the sweep stream is four passes,
    or three where the Y and Z sweeps are one launch."""
    from cell_simulation_gb300 import tiling_launches
    return tiling_launches()[i]


def ensemble_numbers(device, steps_batched=200, steps_plain=20, variant=-1):
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
    out = {"workload": f"c4_ensemble_{n}rep_L32-96_K8", "total_voxels": int(tot), "work_items": int(items),
           "replicate_steps_per_s_batched": rb, "replicate_steps_per_s_plain": rp,
           "voxel_steps_per_s_batched": tot * steps_batched / (ms_b / 1e3),
           "batched_over_plain": rb / rp, "steps_batched": steps_batched, "steps_plain": steps_plain,
           "launches_per_frame_batched": per_frame, "launches_per_frame_plain": n * per_frame,
           "variant": describe_variant(variant)}
    ens.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="skip ensemble, reference-RNG, e2e and CPU legs")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--variant", type=int, default=-1, help="step variant index (default: autotuned)")
    ap.add_argument("--ensemble-only", action="store_true",
                    help="only the 512-replicate ensemble leg: --steps batched frames, a tenth as many plain ones "
                         "(for profiling; prints that leg's numbers)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = env_rank()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return

    import __graft_entry__
    __graft_entry__.build()
    if args.ensemble_only:
        print(json.dumps(ensemble_numbers(local, args.steps, max(1, args.steps // 10), args.variant)), flush=True)
        return
    from cell_simulation_gb300 import PREC_MIXED, RNG_PHILOX, RNG_REFERENCE, configs

    dist = Dist(world)
    device = local
    seed = 0xC0FFEE + rank
    t_setup = time.perf_counter()
    w = configs.c3_multi_region()
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
    sim.step_philox(args.warmup, seed)
    sim.synchronize()
    clocks = ClockSampler(device)
    clocks.start()
    dist.barrier()
    ms = sim.step_philox_timed(args.steps, seed)
    dist.barrier()
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = world * V * args.steps / (ms_max / 1e3)
    per_launch_s = ms / 1e3 / args.steps
    peak, peak_kind = measured_peaks()
    alg_bytes = V * (2 * K + 1)
    achieved = alg_bytes / per_launch_s / 1e9
    desc = describe_variant(variant)
    kernel = {"brick": "brick_step_kernel", "stream": "sweep_pass_kernel"}.get(desc["kind"], "prod_step_kernel")
    if desc["kind"] == "stream":
        # the frame's longest launch: pass 3, or the fused Y and Z sweeps (template pass 5)
        kernel += "<5>" if desc["passes_per_frame"] == 3 else "<3>"
    traffic = profiled_traffic(kernel, w.name)
    diag = sim.diagnostics()

    # end to end through the C ABI: every frame one step call (its frame number
    # up, 4 bytes; the seed is uploaded only when it changes) and one blocking
    # read of the species counts (down), like the reference's per-frame itime
    # write, submit and stats readback
    n_e2e = min(args.steps, 500)
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        sim.step_philox(1, seed)
        sim.counts()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * V * n_e2e / dist.max(e2e_s), "unit": UNIT, "h2d_bytes_per_step": 4,
           "d2h_bytes_per_step": S1 * 8, "steps": n_e2e,
           "setup_s": {"host_model_build": t_build, "upload_prepare_for_gpu": t_upload}}

    extras = {}
    if not args.no_extras and rank == 0:
        extras["ensemble"] = ensemble_numbers(device)
        # reference-RNG (bit-parity) CUDA path on the same lattice
        w2 = configs.c3_multi_region()
        s2 = w2.sim
        s2.prepare_for_gpu(RNG_REFERENCE, device)
        it = (np.arange(200, dtype=np.uint64) * 7919 + 12345).astype(np.uint32)
        s2.step(it[:3])
        ms_ref = s2.step_timed(it[3:103])
        extras["reference_rng_path"] = {"voxel_steps_per_s": V * 100 / (ms_ref / 1e3), "launches_per_frame": 5,
                                        "steps": 100}
        s2.close()
    cpu = None
    if not args.no_extras and rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        rate, sample = cpu_reference_rate(args.cpu_budget, threads)
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
                   "l2": "inputs larger than L2 (2 x 256 MiB lattice buffers)", "parallelism": f"replicas x{world}",
                   "variant": describe_variant(variant)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": alg_bytes, "kernel": kernel,
                     "achieved_over": "frame time (every launch of the frame)"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": args.steps * launches_per_frame(variant),
        "clocks": clk,
        "diagnostics": {"events": int(diag[0]), "rejected_capacity": int(diag[1]), "event_cap": int(diag[2]),
                        "fp64_selections": int(diag[3]), "ssa_voxels": int(diag[6])},
    }
    line.update(extras)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
