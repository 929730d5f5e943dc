"""Checkpoint/resume (cs_checkpoint_*) and the headless visualisation views
(cs_render_view, final_stage.wgsl:35-68)."""
import numpy as np
import pytest

from cell_simulation_gb300 import RNG_PHILOX, RNG_REFERENCE
from cell_simulation_gb300.simulation import Simulation
from tests.helpers import itime_schedule, multi_region_model


def test_checkpoint_roundtrip_host_model(tmp_path, lib):
    """Before prepare_for_gpu a checkpoint carries the host model unchanged."""
    a = multi_region_model(res=(9, 10, 11), K=8, reservoir=True, transition=True)
    p = tmp_path / "model.ckpt"
    a.save_checkpoint(p)
    b = Simulation.load_checkpoint(p)
    ta, tb = a.tables(), b.tables()
    for f in ("regions", "diffusion", "stoich", "reactants", "rates", "reservoir"):
        assert np.array_equal(getattr(ta, f), getattr(tb, f)), f
    for x, y in zip(a.get_lattice(), b.get_lattice()):
        assert np.array_equal(x, y)
    assert a.particle_names == b.particle_names
    assert a.info().n_reactions == b.info().n_reactions


def test_checkpoint_rejects_garbage(tmp_path, lib):
    from cell_simulation_gb300 import CellsimError
    p = tmp_path / "bad.ckpt"
    p.write_bytes(b"not a checkpoint at all")
    with pytest.raises(CellsimError):
        Simulation.load_checkpoint(p)


def _step(sim, mode, it):
    if mode == RNG_REFERENCE:
        sim.step(it)
    else:
        sim.step_philox(len(it), 4321)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [RNG_PHILOX, RNG_REFERENCE])
def test_checkpoint_resume_bit_exact(tmp_path, mode):
    it = itime_schedule(30)
    a = multi_region_model(res=(12, 14, 30), K=16, reservoir=True, counts=(90, 70, 50, 40))
    a.prepare_for_gpu(mode, 0)
    _step(a, mode, it[:10])
    p = tmp_path / "run.ckpt"
    a.save_checkpoint(p)
    _step(a, mode, it[10:30])
    b = Simulation.load_checkpoint(p, device=0)
    _step(b, mode, it[10:30])
    for x, y in zip(a.get_lattice(), b.get_lattice()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.counts(), b.counts())


def views_numpy(sim, view, axis, slice_):
    i = sim.info()
    X, Y, Z = (int(r) for r in i.res)
    K = i.max_particles_site
    s, _, _ = sim.get_lattice()
    t = sim.tables()
    s = s.reshape(X * Y * Z, K)
    out = np.zeros(X * Y * Z, np.float32)
    for v in range(X * Y * Z):
        if view == 1:
            val = t.regions[v]
        elif view == 2:
            val = t.reservoir[v]
        else:
            sl = [q for q in s[v] if q]
            best, val = 0, 0
            for a in sl:
                c = sl.count(a)
                if c > best:
                    best, val = c, a
        out[v] = np.float32(val) / np.float32(255.0)
    coord = np.indices((X, Y, Z)).reshape(3, -1)[axis]
    out[(np.array([X, Y, Z])[axis] - coord) < slice_] = 0.0
    return out.reshape(X, Y, Z)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [RNG_PHILOX, RNG_REFERENCE])
def test_render_views_match_numpy(mode):
    sim = multi_region_model(res=(10, 9, 12), K=16, reservoir=True, counts=(300, 200, 150, 60))
    sim.prepare_for_gpu(mode, 0)
    _step(sim, mode, itime_schedule(5))
    for view, axis, sl in ((0, 0, 0), (1, 1, 0), (2, 2, 0), (0, 2, 5), (1, 0, 3)):
        got = sim.render_view(view, axis, sl)
        want = views_numpy(sim, view, axis, sl)
        assert np.array_equal(got, want), (view, axis, sl)
