"""Production (Philox) fused kernel against the plain per-sweep oracle:
identical lattices and counts after N frames for every tiling, plus exact
conservation, region confinement and batched-ensemble equivalence."""
import numpy as np
import pytest

from cell_simulation_gb300 import (CellsimError, Ensemble, PREC_FP32, PREC_FP64, PREC_MIXED, RNG_PHILOX, configs,
                                   tiling_kinds, tiling_launches, tiling_variants)
from tests.helpers import crowded_model, multi_region_model, oracle_args, patchy_model

pytestmark = pytest.mark.gpu


def compact(slots_u32, K):
    s = slots_u32.reshape(-1, K)
    out = np.zeros_like(s, dtype=np.uint8)
    for v in np.flatnonzero((s > 0).any(1)):
        nz = s[v][s[v] > 0]
        out[v, :len(nz)] = nz
    return out.reshape(-1)


def oracle_prod(orc, sim, n, seed, frame0=0, precision=0):
    res, K, NR, S, R, tau, lam, tab = oracle_args(sim)
    s, o, c = sim.get_lattice()
    slots = compact(s, K)
    counts = np.bincount(s, minlength=S + 1).astype(np.int64)
    counts[0] = 0
    for q in tab.reservoir[tab.reservoir > 0]:
        counts[q] += 1
    diag = orc.prod_run(res, K, NR, S, R, tau, lam, tab, slots, counts, seed, frame0, n, precision=precision)
    return slots, counts, diag


def gpu_prod(sim, n, seed, tiling=None, seg=0, chunks=1, precision=PREC_MIXED):
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    sim.set_precision(precision)
    if tiling is not None:
        sim.set_tiling(tiling, seg)
    for part in np.array_split(np.arange(n), chunks):
        if len(part):
            sim.step_philox(len(part), seed)
    s, o, c = sim.get_lattice()
    K = sim.info().max_particles_site
    return s.astype(np.uint8), sim.counts(), sim.diagnostics()


def tilings_for(K):
    return [i for i, t in enumerate(tiling_variants()) if t[0] == K]


@pytest.mark.parametrize("K", [8, 16])
def test_fused_kernel_matches_oracle(orc, K):
    sim = multi_region_model(res=(11, 13, 37), K=K, counts=(60, 50, 40, 30))
    want_s, want_c, want_d = oracle_prod(orc, sim, 40, seed=1234)
    for ti in tilings_for(K):
        got_s, got_c, got_d = gpu_prod(multi_region_model(res=(11, 13, 37), K=K, counts=(60, 50, 40, 30)), 40, 1234,
                                       tiling=ti, seg=5)
        assert np.array_equal(got_s, want_s), (ti, np.flatnonzero(got_s != want_s)[:8])
        assert np.array_equal(got_c, want_c), ti
        assert np.array_equal(got_d[:4], want_d[:4]), (ti, got_d, want_d)
    assert want_d[0] > 0  # reactions fired


@pytest.mark.parametrize("precision", [PREC_MIXED, PREC_FP32, PREC_FP64])
def test_precision_modes_match_oracle(orc, precision):
    mk = lambda: multi_region_model(res=(9, 8, 20), K=16, counts=(70, 60, 50, 40), reservoir=True)
    want_s, want_c, want_d = oracle_prod(orc, mk(), 30, seed=99, precision=precision)
    got_s, got_c, got_d = gpu_prod(mk(), 30, 99, precision=precision, chunks=3)
    assert np.array_equal(got_s, want_s)
    assert np.array_equal(got_c, want_c)
    assert np.array_equal(got_d[:4], want_d[:4])


def brick_tilings(K):
    return [i for i, (t, (kind, _)) in enumerate(zip(tiling_variants(), tiling_kinds())) if t[0] == K and kind == 1]


@pytest.mark.parametrize("K", [8, 16])
def test_brick_pass_with_spilled_bricks_matches_oracle(orc, K):
    """Sparse bricks run in the brick pass, the crowded cube's bricks overflow
    its pools and are finished by the full-capacity second pass: the frame is
    the same."""
    mk = lambda: patchy_model(K=K)
    want_s, want_c, want_d = oracle_prod(orc, mk(), 24, seed=77)
    for ti in brick_tilings(K):
        got_s, got_c, got_d = gpu_prod(mk(), 24, 77, tiling=ti, chunks=2)
        assert np.array_equal(got_s, want_s), (ti, np.flatnonzero(got_s != want_s)[:8])
        assert np.array_equal(got_c, want_c), ti
        assert np.array_equal(got_d[:4], want_d[:4]), (ti, got_d, want_d)
        spilled, lost = int(got_d[4]), int(got_d[5])
        assert lost == 0
        if tiling_kinds()[ti][1] == 2:
            assert spilled == 0  # full-capacity pools
        else:
            planes = tiling_kinds()[ti][1]
            n_bricks = -(-19 // planes) * 3 * 3  # (19/planes, 21/8, 70/32) rounded up
            assert 0 < spilled < 24 * n_bricks, spilled  # some bricks spill, most do not


@pytest.mark.parametrize("K", [8, 16])
def test_one_region_windows_match_oracle(orc, K):
    """A small cell in a large lattice: bricks far from it see one region in their whole region
    window and skip the region rows, the bricks around it stage them; the frame is the same."""
    mk = lambda: multi_region_model(res=(40, 36, 70), K=K, counts=(120, 400, 80, 40), transition=True)
    want_s, want_c, want_d = oracle_prod(orc, mk(), 30, seed=4242)
    for ti in brick_tilings(K):
        got_s, got_c, got_d = gpu_prod(mk(), 30, 4242, tiling=ti, chunks=2)
        assert np.array_equal(got_s, want_s), (ti, np.flatnonzero(got_s != want_s)[:8])
        assert np.array_equal(got_c, want_c), ti
        assert np.array_equal(got_d[:4], want_d[:4]), (ti, got_d, want_d)


def stream_tilings(K):
    return [i for i, (t, (kind, _)) in enumerate(zip(tiling_variants(), tiling_kinds())) if t[0] == K and kind == 2]


@pytest.mark.parametrize("K", [8, 16])
def test_sweep_stream_matches_oracle(orc, K):
    """The sweep stream on the crowded patchy lattice and on a multi-region lattice with
    reservoirs, in runs split over several step calls: each call after the first starts from the
    x-decisions that the previous call's last pass made.  The frames are the oracle's."""
    models = (lambda: patchy_model(K=K),
              lambda: multi_region_model(res=(9, 8, 40), K=K, counts=(70, 60, 50, 40), reservoir=True))
    assert stream_tilings(K)
    for mk in models:
        want_s, want_c, want_d = oracle_prod(orc, mk(), 24, seed=77)
        for ti in stream_tilings(K):
            got_s, got_c, got_d = gpu_prod(mk(), 24, 77, tiling=ti, chunks=5)
            assert np.array_equal(got_s, want_s), (ti, np.flatnonzero(got_s != want_s)[:8])
            assert np.array_equal(got_c, want_c), ti
            assert np.array_equal(got_d[:4], want_d[:4]), (ti, got_d, want_d)


def test_fused_sweep_stream_needs_short_rows(orc):
    """The fused Y and Z sweeps need rows of at most 32 bitmap words: on a lattice with Z = 1056
    (33 words) cs_set_tiling refuses them and the handle keeps stepping with its own variant."""
    mk = lambda: multi_region_model(res=(3, 4, 1056), K=16, counts=(40, 30, 20, 10))
    want_s, want_c, _ = oracle_prod(orc, mk(), 3, seed=31)
    sim = mk()
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    launches = tiling_launches()
    fused = next(i for i in stream_tilings(16) if launches[i] == 2)
    with pytest.raises(CellsimError, match="at most 32 bitmap words"):
        sim.set_tiling(fused)
    sim.step_philox(3, 31)
    assert np.array_equal(sim.get_lattice()[0].astype(np.uint8), want_s)
    assert np.array_equal(sim.counts(), want_c)


def test_sweep_stream_recomputes_stale_decisions(orc):
    """A seed change and a lattice upload between step calls make the next frame's x-decisions
    (made by the last pass of the previous call) stale: the lattice still follows the oracle.
    The upload comes after an odd number of frames, so the frame parity restarts at 0 while the
    parity-0 work counters were used last (the brick pass is checked on that too)."""
    mk = lambda: multi_region_model(res=(11, 13, 37), K=16, counts=(60, 50, 40, 30))
    ref = mk()
    want_s, want_c, _ = oracle_prod(orc, ref, 6, seed=11)
    res, K, NR, S, R, tau, lam, tab = oracle_args(ref)
    orc.prod_run(res, K, NR, S, R, tau, lam, tab, want_s, want_c, 12, 6, 9)
    for ti in stream_tilings(16) + brick_tilings(16)[-1:]:
        sim = mk()
        sim.prepare_for_gpu(RNG_PHILOX, 0)
        sim.set_tiling(ti)
        sim.step_philox(6, 11)
        sim.step_philox(5, 12)  # new seed
        sim.set_lattice(sim.get_lattice()[0])  # same content, fresh upload
        sim.step_philox(4, 12)
        assert np.array_equal(sim.get_lattice()[0].astype(np.uint8), want_s), ti
        assert np.array_equal(sim.counts(), want_c), ti


def test_sparse_lattice_never_spills():
    sim = multi_region_model(res=(24, 20, 40), K=16, counts=(60, 50, 40, 30))
    _, _, d = gpu_prod(sim, 10, 5)
    assert d[4] == 0


def test_crowded_capacity_rule(orc):
    mk = lambda: crowded_model(res=(6, 5, 7), K=8, counts=(60, 50, 40))
    want_s, want_c, _ = oracle_prod(orc, mk(), 50, seed=5)
    got_s, got_c, _ = gpu_prod(mk(), 50, 5)
    assert np.array_equal(got_s, want_s)
    assert np.array_equal(got_c, want_c)
    v = got_s.reshape(-1, 8)
    # compacted: no zero before a particle
    assert not ((v[:, :-1] == 0) & (v[:, 1:] != 0)).any()


def test_conservation_and_confinement():
    sim = multi_region_model(res=(16, 16, 24), K=16, counts=(200, 150, 100, 80))
    tab = sim.tables()
    before = np.bincount(sim.get_lattice()[0], minlength=5)[1:]
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    # no reactions: rates zeroed through the drop-in table setter is not allowed after prepare, so use a model copy
    sim2 = multi_region_model(res=(16, 16, 24), K=16, counts=(200, 150, 100, 80))
    t2 = sim2.tables()
    i2 = sim2.info()
    sim2.set_tables(i2.n_regions, i2.n_species, i2.n_reactions, t2.regions, t2.diffusion, t2.stoich, t2.reactants,
                    np.zeros_like(t2.rates))
    sim2.set_lattice(sim.get_lattice()[0])
    sim2.prepare_for_gpu(RNG_PHILOX, 0)
    sim2.step_philox(200, 7)
    s, _, _ = sim2.get_lattice()
    after = np.bincount(s, minlength=5)[1:]
    assert np.array_equal(before, after)
    assert np.array_equal(sim2.counts()[1:], before)
    # off-diagonal D = 0: every particle stays in the region it started in
    reg = tab.regions
    s0 = sim.get_lattice()[0].reshape(-1, 16)
    s1 = s.reshape(-1, 16)
    for q in range(1, 5):
        r0 = np.bincount(np.repeat(reg, (s0 == q).sum(1)), minlength=4)
        r1 = np.bincount(np.repeat(reg, (s1 == q).sum(1)), minlength=4)
        assert np.array_equal(r0, r1), q


@pytest.mark.parametrize("form", ["default", "frames"])
def test_graph_replay_equals_single_launches(form):
    """25 frames in one call equal 25 one-frame calls: the default step's two-frame graph against
    its one-frame graphs, and the persistent multi-frame launch against the per-pass launches its
    variant takes for one-frame calls; calls of mixed lengths as well."""
    a = multi_region_model(res=(10, 12, 30), K=16)
    b = multi_region_model(res=(10, 12, 30), K=16)
    c = multi_region_model(res=(10, 12, 30), K=16)
    for sim in (a, b, c):
        sim.prepare_for_gpu(RNG_PHILOX, 0)
        if form == "frames":
            launches = tiling_launches()
            sim.set_tiling(next(i for i in stream_tilings(16) if launches[i] == 1))
    a.step_philox(25, 3)
    for _ in range(25):
        b.step_philox(1, 3)
    for n in (1, 2, 1, 3, 1, 4, 1, 5, 7):
        c.step_philox(n, 3)
    for other in (b, c):
        assert np.array_equal(a.get_lattice()[0], other.get_lattice()[0])
        assert np.array_equal(a.counts(), other.counts())
    assert a.diagnostics()[7] == 0


@pytest.mark.parametrize("variant", ["default", "unfused", "fused_last", "frames", "resident"])
def test_ensemble_batched_equals_plain_and_oracle(orc, variant):
    """Replicates of different sizes in one launch per pass: batched frames equal per-replicate
    (plain) frames and the oracle, for the default step (fused Y and Z sweeps), the sweep stream
    with the Y and Z sweeps apart, the fused stream at four blocks per SM, the persistent
    multi-frame stream (batched: every frame of a step call in one launch) and the resident form
    (one block per replicate, every frame of a call in one launch)."""
    tmpl = configs.c4_ensemble_template(K=8)
    res = np.array([[9, 9, 9], [12, 12, 12], [7, 7, 7], [16, 16, 16]], np.uint32)
    seeds = np.array([11, 22, 33, 44], np.uint64)
    mult = np.array([0.5, 1.0, 1.7, 2.0], np.float32)
    init = np.array([0, 40, 40, 5], np.uint32)
    eb = Ensemble(tmpl, res, seeds, mult, init)
    ep = Ensemble(tmpl, res, seeds, mult, init)
    if variant == "resident":
        ti = next(i for i, (t, k) in enumerate(zip(tiling_variants(), tiling_kinds())) if t[0] == 8 and k[0] == 3)
        eb.set_tiling(ti)
        ep.set_tiling(ti)
    elif variant != "default":
        launches = tiling_launches()
        want = {"unfused": 3, "fused_last": 2, "frames": 1}[variant]
        ti = [i for i in stream_tilings(8) if launches[i] == want][-1]
        eb.set_tiling(ti)
        ep.set_tiling(ti)
    s0 = eb.slots()
    eb.step(30, batched=True)
    ep.step(30, batched=False)
    assert np.array_equal(eb.slots(), ep.slots())
    assert np.array_equal(eb.counts(), ep.counts())
    # each replicate against the oracle
    tab = tmpl.tables()
    info = tmpl.info()
    off = 0
    got = eb.slots()
    counts = eb.counts()
    for r in range(len(res)):
        V = int(np.prod(res[r]))
        sl = s0[off * 8:(off + V) * 8].copy()
        c0 = np.bincount(sl, minlength=4).astype(np.int64)
        c0[0] = 0
        t = type(tab)(np.zeros(V, np.uint32), tab.diffusion, tab.stoich, tab.reactants, tab.rates,
                      np.zeros(V, np.uint32))
        orc.prod_run(tuple(int(x) for x in res[r]), 8, info.n_regions, info.n_species, info.n_reactions,
                     float(np.float32(info.tau)), float(np.float32(info.lambda_)), t, sl, c0, int(seeds[r]), 0, 30,
                     rate_mult=float(mult[r]))
        assert np.array_equal(got[off * 8:(off + V) * 8], sl), r
        assert np.array_equal(counts[r], c0), r
        off += V


def test_switching_step_kinds_mid_run_matches_oracle(orc):
    """Tile-pipeline frames do not maintain the occupancy bitmaps of the brick
    pass; switching back rebuilds them.  A lattice upload in between does too."""
    mk = lambda: multi_region_model(res=(13, 17, 40), K=16, counts=(90, 70, 50, 40))
    want_s, want_c, _ = oracle_prod(orc, mk(), 18, seed=321)
    sim = mk()
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    kinds = tiling_kinds()
    tile = next(i for i, (t, k) in enumerate(zip(tiling_variants(), kinds)) if t[0] == 16 and k[0] == 0)
    brick = next(i for i, (t, k) in enumerate(zip(tiling_variants(), kinds)) if t[0] == 16 and k == (1, 8))
    sim.set_tiling(brick)
    sim.step_philox(6, 321)
    sim.set_tiling(tile)
    sim.step_philox(6, 321)
    sim.set_tiling(brick)
    s_mid = sim.get_lattice()[0]
    sim.set_lattice(s_mid)  # same content, fresh upload
    sim.step_philox(6, 321)
    got_s, _, _ = sim.get_lattice()
    assert np.array_equal(got_s.astype(np.uint8), want_s)
    assert np.array_equal(sim.counts(), want_c)


def test_switching_to_and_from_the_sweep_stream_matches_oracle(orc):
    """Brick, sweep-stream (three launches, Y and Z sweeps fused, and the persistent multi-frame
    form) and tile frames in one run:
    frames of another kind (and an upload) make the x-decisions the last stream frame left for the
    next frame stale, so the stream recomputes them.  Odd frame counts change the parity the kinds
    hand over; the fused variant keeps its records in buffers of fixed roles."""
    mk = lambda: multi_region_model(res=(13, 17, 40), K=16, counts=(90, 70, 50, 40))
    want_s, want_c, _ = oracle_prod(orc, mk(), 29, seed=777)
    sim = mk()
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    kinds = tiling_kinds()
    tile = next(i for i, (t, k) in enumerate(zip(tiling_variants(), kinds)) if t[0] == 16 and k[0] == 0)
    brick = next(i for i, (t, k) in enumerate(zip(tiling_variants(), kinds)) if t[0] == 16 and k == (1, 8))
    launches = tiling_launches()
    stream = [i for i in stream_tilings(16) if launches[i] == 3][-1]
    fused = next(i for i in stream_tilings(16) if launches[i] == 2)
    frames = next(i for i in stream_tilings(16) if launches[i] == 1)
    for ti, n in ((stream, 3), (brick, 4), (frames, 3), (fused, 5), (tile, 3), (frames, 2), (stream, 2), (fused, 3)):
        sim.set_tiling(ti)
        sim.step_philox(n, 777)
    sim.set_lattice(sim.get_lattice()[0])
    sim.step_philox(4, 777)
    assert np.array_equal(sim.get_lattice()[0].astype(np.uint8), want_s)
    assert np.array_equal(sim.counts(), want_c)


def test_autotune_keeps_state_and_results(orc):
    """The autotuner times every variant on a copy of the live state: the
    simulation does not advance and the following frames equal the oracle."""
    mk = lambda: multi_region_model(res=(16, 18, 45), K=16, counts=(90, 70, 50, 40))
    want_s, want_c, _ = oracle_prod(orc, mk(), 12, seed=5150)
    sim = mk()
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    sim.step_philox(4, 5150)
    before = sim.get_lattice()[0].copy()
    idx, ms = sim.autotune(frames_per_trial=2)
    assert 0 <= idx < len(tiling_variants()) and tiling_variants()[idx][0] == 16 and ms > 0
    assert sim.get_tiling() == idx
    assert np.array_equal(sim.get_lattice()[0], before)
    sim.step_philox(8, 5150)
    got_s, _, _ = sim.get_lattice()
    assert np.array_equal(got_s.astype(np.uint8), want_s)
    assert np.array_equal(sim.counts(), want_c)


def test_counts_follow_a_change_of_species_count():
    """cs_set_tables may raise the species count after a preparation: the next preparation's
    counts have the new length and equal the new lattice's particles plus reservoir species."""
    sim = multi_region_model(res=(12, 10, 14), K=8)
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    assert len(sim.counts()) == 5
    other = multi_region_model(res=(12, 10, 14), K=8, reservoir=True)
    t, i = other.tables(), other.info()
    sim.set_tables(i.n_regions, i.n_species, i.n_reactions, t.regions, t.diffusion, t.stoich, t.reactants, t.rates,
                   t.reservoir)
    slots = other.get_lattice()[0]
    sim.set_lattice(slots)
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    want = np.bincount(slots, minlength=i.n_species + 1).astype(np.int64)
    want[0] = 0
    for q in t.reservoir[t.reservoir > 0]:
        want[q] += 1
    got = sim.counts()
    assert len(got) == i.n_species + 1 == 6
    assert np.array_equal(got, want)
