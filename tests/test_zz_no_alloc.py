"""cs_ref_frame_noalloc: the reference-RNG frame for callers that own every
device buffer and may not allocate device memory at run time.

The caller's buffers here come from torch (standing in for a host engine's
own arena).  Two frames in a row through the allocation-free entry point
must give exactly the lattice, occupancy, concentrations, species counts and
diagnostics of the same two frames through cs_step (integer state: the
tolerance is zero, as in every parity test here).  This file is collected
last so that a failure here does not hide the other tests."""
import ctypes as C

import numpy as np
import pytest

from cell_simulation_gb300 import RNG_REFERENCE, CellsimError, native
from tests.helpers import crowded_model, itime_schedule, multi_region_model

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    """Caller-owned device copy of a numpy array (bits preserved)."""
    a = np.ascontiguousarray(a)
    view = {1: np.uint8, 4: np.int32}[a.dtype.itemsize]
    return torch.from_numpy(a.view(view).copy()).cuda()


def _host(t, dtype):
    return t.cpu().numpy().view(dtype)


@pytest.mark.parametrize("model", ["multi_region", "crowded"])
def test_noalloc_frames_match_cs_step(lib, model):
    """Two frames through each entry point.  On the crowded lattice the first frame has moves
    that compete for room, so it takes the serial-resolution branch, which reads the contention
    flag the frame set in the library's shared scratch; the second frame takes the gather
    branch and must find that flag cleared."""
    torch = pytest.importorskip("torch")
    if model == "crowded":
        sim = crowded_model()
    else:
        sim = multi_region_model(res=(12, 10, 14), K=8, reservoir=True)
    info = sim.info()
    K, S1, R, NR = info.max_particles_site, info.n_species + 1, info.n_reactions, info.n_regions
    V = int(info.n_voxels)
    tab = sim.tables()
    slots, occ, conc = sim.get_lattice()
    counts0 = conc.reshape(V, S1).sum(0).astype(np.int32)
    f = np.float32
    prob = (tab.diffusion.astype(f) * f(info.tau)) / (f(info.lambda_) * f(info.lambda_))
    itimes = itime_schedule(2, seed=424242)

    # caller-owned buffers: frame 1 reads A and writes B, frame 2 reads B and writes A
    A = [_dev(torch, slots.astype(np.uint8)), _dev(torch, occ), _dev(torch, conc)]
    B = [torch.zeros_like(A[0]), torch.zeros_like(A[1]), torch.zeros_like(A[2])]
    tables = dict(regions=_dev(torch, tab.regions.astype(np.uint8)), reservoir=_dev(torch, tab.reservoir.astype(np.uint8)),
                  probabilities=_dev(torch, prob.astype(np.float32)), stoich=_dev(torch, tab.stoich),
                  reactants=_dev(torch, tab.reactants), rates=_dev(torch, tab.rates))
    counts = _dev(torch, counts0)
    diag = torch.zeros(8, dtype=torch.int32, device="cuda")
    itime_dev = [_dev(torch, itimes[i:i + 1]) for i in range(2)]

    # the existing entry point on the same model
    sim.prepare_for_gpu(RNG_REFERENCE, 0)

    def frame(src, dst, it):
        a = native.RefFrameNoAllocArgsC()
        a.device, a.stream = 0, None
        a.res[:] = list(info.res)
        a.max_particles_site, a.n_regions, a.n_species, a.n_reactions = K, NR, S1 - 1, R
        a.tau = info.tau
        a.slots_in, a.occupancy_in, a.conc_in = (t.data_ptr() for t in src)
        a.slots_out, a.occupancy_out, a.conc_out = (t.data_ptr() for t in dst)
        for k, t in tables.items():
            setattr(a, k, t.data_ptr())
        a.itime, a.counts, a.diag = it.data_ptr(), counts.data_ptr(), diag.data_ptr()
        torch.cuda.synchronize()
        native.check(lib.cs_ref_frame_noalloc(C.byref(a)))
        torch.cuda.synchronize()

    for i, (src, dst) in enumerate(((A, B), (B, A))):
        frame(src, dst, itime_dev[i])
        sim.step(itimes[i:i + 1])
        ws, wo, wc = sim.get_lattice()
        assert np.array_equal(_host(dst[0], np.uint8).astype(np.uint32), ws), f"slots differ after frame {i + 1}"
        assert np.array_equal(_host(dst[1], np.uint32), wo), f"occupancy differs after frame {i + 1}"
        assert np.array_equal(_host(dst[2], np.int32), wc), f"concentrations differ after frame {i + 1}"
        assert np.array_equal(_host(counts, np.int32).astype(np.int64), sim.counts()), f"counts differ after frame {i + 1}"
        assert np.array_equal(_host(diag, np.uint32), sim.diagnostics()), f"diagnostics differ after frame {i + 1}"
        if model == "crowded":
            assert _host(diag, np.uint32)[2] == 1  # frame 1 resolved serially, frame 2 by the gather


def test_noalloc_rejects_oversized_lattice(lib):
    a = native.RefFrameNoAllocArgsC()
    a.res[:] = [512, 256, 256]
    a.max_particles_site, a.n_regions, a.n_species, a.n_reactions = 8, 1, 1, 0
    with pytest.raises(CellsimError) as e:
        native.check(lib.cs_ref_frame_noalloc(C.byref(a)))
    assert e.value.status == 3 and "16777216" in str(e.value)
