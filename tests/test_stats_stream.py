"""Statistics stream (SolverStatisticSample samples every write_freq frames,
src/simulation.rs:391-418) and its CSV output (examples/no_window.rs:16-62)."""
import numpy as np
import pytest

from cell_simulation_gb300 import RNG_PHILOX, RNG_REFERENCE
from cell_simulation_gb300.stats import StatisticContainer, drain, make_all_stats, rust_f32
from tests.helpers import itime_schedule, multi_region_model


def test_rust_f32_display():
    assert rust_f32(5000) == "5000" and rust_f32(0) == "0" and rust_f32(-3) == "-3"
    assert rust_f32(0.1) == "0.1" and rust_f32(2.5) == "2.5"
    assert rust_f32(16777217) == "16777216"  # f32 rounding of the i32 value


def test_container_ring_and_csv(tmp_path):
    c = StatisticContainer(capacity=3)
    for i, v in enumerate([10, 11, 12, 13]):
        c.add(i * 5, v)
    assert list(c.x) == [5, 10, 15] and c.last() == 13.0 and c.mean() == 12.0
    p = tmp_path / "A.csv"
    c.to_csv(p)
    assert p.read_text() == "5;11\n10;12\n15;13\n"
    assert not c.x


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [RNG_PHILOX, RNG_REFERENCE])
def test_samples_every_write_freq(mode, tmp_path):
    """Samples of the logged species at every frame f > 0 with f % write_freq == 0,
    each equal to the species count after f frames."""
    sim = multi_region_model(res=(10, 10, 12), K=16, counts=(80, 60, 40, 20))
    sim.prepare_for_gpu(mode, 0)
    it = itime_schedule(40)
    want = {}
    ref = multi_region_model(res=(10, 10, 12), K=16, counts=(80, 60, 40, 20))
    ref.prepare_for_gpu(mode, 0)
    for f in range(1, 41):
        if mode == RNG_REFERENCE:
            ref.step(it[f - 1:f])
        else:
            ref.step_philox(1, 77)
        want[f] = ref.counts()
    if mode == RNG_REFERENCE:
        sim.step(it, write_freq=8)
    else:
        sim.step_philox(40, 77, write_freq=8)
    stats = make_all_stats(sim.particle_names[1:])
    assert drain(sim, stats) > 0
    names = sim.particle_names
    for n, c in stats.items():
        assert list(c.x) == [8, 16, 24, 32], n
        # the sample labelled f is the count after f frames (the reference maps the
        # stats buffer inside step(f), before frame f's passes are submitted)
        q = names.index(n)
        assert [int(v) for v in c.y] == [int(want[f][q]) for f in (8, 16, 24, 32)], n
        c.to_csv(tmp_path / f"{n}.csv")
        assert (tmp_path / f"{n}.csv").read_text().count(";") == 4
