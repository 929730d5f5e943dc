"""The oracle against published known answers, libm accuracy bounds and its
own two formulations (serial order vs gather + OpenMP)."""
import numpy as np
import pytest

from cell_simulation_gb300 import configs
from tests.helpers import crowded_model, itime_schedule, multi_region_model, oracle_args, ref_state

# Random123 known-answer vectors for Philox4x32-10 (published with the algorithm)
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_philox_known_answers(orc):
    lib = orc.load()
    for ctr, key, want in PHILOX_KAT:
        c, k, o = np.array(ctr, np.uint32), np.array(key, np.uint32), np.zeros(4, np.uint32)
        lib.orc_philox4x32_10(c.ctypes.data, k.ctypes.data, o.ctypes.data)
        assert tuple(int(x) for x in o) == want


def _py_pcg(s):
    # res/shader/random.wgsl:14-20, written out independently in numpy
    s = np.uint32(s)
    word = np.uint32(((s >> ((s >> np.uint32(28)) + np.uint32(4))) ^ s) * np.uint32(277803737))
    return np.uint32((word >> np.uint32(22)) ^ word)


def _py_xorshift(s):
    s = np.uint32(s)
    s ^= np.uint32(s << np.uint32(13))
    s ^= np.uint32(s >> np.uint32(17))
    s ^= np.uint32(s << np.uint32(5))
    return s


def test_pcg_xorshift_uniform(orc):
    lib = orc.load()
    rng = np.random.default_rng(1)
    with np.errstate(over="ignore"):
        for s in list(rng.integers(0, 2 ** 32, 2000, dtype=np.uint64)) + [0, 1, 0xFFFFFFFF, 0x80000000]:
            s = int(s)
            assert lib.orc_pcg(s) == int(_py_pcg(s))
            assert lib.orc_xorshift(s) == int(_py_xorshift(s))
            u = np.float32(np.float32(int(_py_xorshift(s))) * np.float32(2.0 ** -32))
            assert np.float32(lib.orc_uniform_float(s)) == u
    # 0 maps to 0 and the largest u32 rounds to exactly 1.0
    assert lib.orc_uniform_float(0) == 0.0
    inv = [s for s in range(1, 1 << 20) if int(_py_xorshift(s)) >= 0xFFFFFF80][:1]
    if inv:
        assert lib.orc_uniform_float(inv[0]) == 1.0


def _ulp_err(got, want):
    got = np.float32(got)
    spacing = np.spacing(np.float32(abs(want)) if want != 0 else np.float32(1e-45))
    return abs(float(got) - want) / float(spacing)


def test_expf_accuracy(orc):
    lib = orc.load()
    xs = np.concatenate([np.linspace(-87.3, 88.7, 20001), -np.logspace(-8, 1.9, 3000), np.logspace(-8, 1.9, 3000)])
    worst = max(_ulp_err(lib.orc_expf(float(np.float32(x))), float(np.exp(np.float64(np.float32(x))))) for x in xs)
    assert worst <= 2.0, worst
    assert lib.orc_expf(0.0) == 1.0
    assert lib.orc_expf(-100.0) == 0.0


def test_logf_accuracy(orc):
    lib = orc.load()
    xs = np.concatenate([np.logspace(-40, 38, 20000), (np.arange(1, 1 << 14) * 2.0 ** -14)])
    worst = 0.0
    for x in xs:
        x32 = np.float32(x)
        want = float(np.log(np.float64(x32)))
        if want == 0.0:
            assert lib.orc_logf(float(x32)) == 0.0
            continue
        worst = max(worst, _ulp_err(lib.orc_logf(float(x32)), want))
    assert worst <= 3.0, worst


def _run_both(orc, sim, n, threads=4):
    args = oracle_args(sim)
    s, o, c, st = ref_state(sim)
    it = itime_schedule(n)
    a = orc.ref_run(*args, orc.RefState(s, o, c, st), it, mode=0)
    b = orc.ref_run(*args, orc.RefState(s, o, c, st), it, mode=1, threads=threads)
    return a, b


def _same(a, b):
    assert np.array_equal(a.slots, b.slots)
    assert np.array_equal(a.occ, b.occ)
    assert np.array_equal(a.conc, b.conc)
    assert np.array_equal(a.stat, b.stat)
    for k in (0, 1, 3, 4):  # spill, occupancy range, rollbacks, fired
        assert a.diag[k] == b.diag[k], (k, a.diag, b.diag)


def test_serial_equals_gather_c1(orc):
    from cell_simulation_gb300 import configs
    a, b = _run_both(orc, configs.c1_plain_2d().sim, 1500)
    _same(a, b)
    assert a.diag[4] > 0  # some reactions fired


@pytest.mark.parametrize("reservoir,transition", [(False, False), (True, False), (False, True)])
def test_serial_equals_gather_multi_region(orc, reservoir, transition):
    sim = multi_region_model(reservoir=reservoir, transition=transition)
    a, b = _run_both(orc, sim, 400)
    _same(a, b)


def test_gather_falls_back_under_contention(orc):
    # crowded K=4 lattice: some frames cannot be resolved by the gather rule
    sim = crowded_model()
    a, b = _run_both(orc, sim, 200)
    _same(a, b)
    assert b.diag[2] > 0  # slow (serial) frames happened
    assert a.diag[0] >= 0


def test_conservation_without_reactions(orc):
    sim = multi_region_model(res=(9, 8, 7), K=8)
    args = list(oracle_args(sim))
    tab = args[-1]
    tab.rates[:] = 0.0
    s, o, c, st = ref_state(sim)
    before = np.bincount(s, minlength=8)
    a = orc.ref_run(*args, orc.RefState(s, o, c, st), itime_schedule(300), mode=0)
    after = np.bincount(a.slots, minlength=8)
    assert np.array_equal(before[1:], after[1:])
    # per-species concentrations agree with the slots
    S1 = sim.info().n_species + 1
    conc = a.conc.reshape(-1, S1)
    K = sim.info().max_particles_site
    sl = a.slots.reshape(-1, K)
    for q in range(1, S1):
        assert np.array_equal(conc[:, q], (sl == q).sum(1))


def quiet_threshold(a0: np.float32, tau: np.float32) -> int:
    """The production step's tabulated bound: draws m <= this give dt > tau."""
    if not a0 > 0:
        return 1 << 24
    x = float(a0) * float(tau) * (1.0 + 2.0 ** -12)
    ub = np.exp(-x) * 16777216.0
    return 16777215 if ub >= 16777215.0 else int(np.floor(ub))


@pytest.mark.parametrize("tau", [configs.stable_tau(1e-12), configs.stable_tau(1e-11)])
def test_quiet_threshold_is_exact(orc, tau):
    """Exhaustively over every draw m <= threshold: the exact waiting time
    -logf(m 2^-24) / a0 exceeds tau, so skipping the SSA there changes nothing."""
    tau = np.float32(tau)
    for a0 in (1e-30, 1e-8, 1e-3, 0.37, 5.0, 120.0, 3e3, 1e4, 6e4, 1e6, 1e8):
        a0 = np.float32(a0)
        m = quiet_threshold(a0, tau)
        if m >= 1:
            assert orc.first_event_inside(a0, tau, 1, m) == 0, (a0, m)
        # the bound is useful: the draws above it that are still quiet are few
        if 1 <= m < (1 << 24) - 1:
            hi = min((1 << 24), m + 4096)
            assert orc.first_event_inside(a0, tau, m + 1, hi) > 0 or float(a0) * float(tau) < 1e-6, (a0, m)
