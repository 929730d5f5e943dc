"""bench.py's multi-rank path on the CPU.  Under torchrun every rank times its
own replica and rank 0 reports the maximum over ranks after a barrier; two
gloo ranks here check that the barrier completes and that both ranks agree
on that maximum.  The reference arm does its work on rank 0 only: another
rank exits at once without output."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out: str) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    d = bench.Dist(world)
    d.barrier()
    m = d.max(1.0 + 2.5 * rank)  # each rank's own frame time
    d.barrier()
    d.close()
    Path(f"{out}.{rank}").write_text(repr(m))


def test_max_over_two_gloo_ranks(tmp_path):
    out = str(tmp_path / "max")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    for r in range(2):
        assert float(Path(f"{out}.{r}").read_text()) == 3.5


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    d = bench.Dist(1)
    d.barrier()
    assert d.max(2.0) == 2.0
    d.close()


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    res = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert res.stdout.strip() == ""


def test_profiled_traffic_covers_the_reported_kernels():
    """bench.py reads the DRAM traffic of the frame's longest launch from the committed ncu
    summaries: every kernel it can report on the 256^3 workload has an entry."""
    sys.path.insert(0, str(ROOT))
    import bench

    for kernel in ("sweep_pass_kernel<5>", "sweep_pass_kernel<3>", "brick_step_kernel", "prod_step_kernel"):
        t = bench.profiled_traffic(kernel, "c3_multi_region_256x256x256_K16")
        assert t is not None and t > 1e7, kernel


def test_reference_arm_follows_the_workload():
    """`--workload` picks the lattice of the main leg and of the reference arm: the 64 x 64 x 1 case
    runs on the host cores as a whole lattice (its CPU sample is all 64 planes)."""
    import json

    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    res = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "c1", "--steps", "2",
                          "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["config"]["workload"].startswith("c1_plain_64x64x1_K8 (64-plane")
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]


def test_every_variant_is_described():
    """bench.py names every compiled variant (tile pipeline, bricks, the sweep stream's forms and
    the resident form), its frame's kernels and its launches per step call."""
    sys.path.insert(0, str(ROOT))
    import bench
    from cell_simulation_gb300 import tiling_kinds, tiling_variants

    kinds = tiling_kinds()
    for i in range(len(tiling_variants())):
        d = bench.describe_variant(i)
        assert d["index"] == i and d["kind"] in ("tile", "brick", "stream", "resident")
        assert bench.frame_kernels(d)
        if d["kind"] == "resident" or d.get("multi_frame"):
            assert bench.launches_in_call(i, 20) == 1
        else:
            assert bench.launches_in_call(i, 20) == 20 * bench.launches_per_frame(i)
    assert sum(1 for k in kinds if k[0] == 3) == 2
