"""Python mirror of the reference's host API (src/simulation.rs,
src/lattice_params.rs, src/region.rs, src/statistics.rs) over the libcellsim
C ABI.  Method names, argument meaning and order follow the reference;
errors raise CellsimError where the reference panics.
"""
from __future__ import annotations

import ctypes as C
from collections import deque
from dataclasses import dataclass, field
from typing import Iterable, Sequence

import numpy as np

from . import native as N


@dataclass
class LatticeParams:
    """LatticeParams::new(dimensions, resolution, tau, lambda), src/lattice_params.rs:97-118."""

    dimensions: Sequence[float]
    resolution: Sequence[int]
    tau: float
    lambda_: float
    max_particles_site: int = 8  # MAX_PARTICLES_SITE, src/lib.rs:15

    def to_c(self) -> N.LatticeParamsC:
        p = N.LatticeParamsC()
        p.dims[:] = [float(x) for x in self.dimensions]
        p.res[:] = [int(x) for x in self.resolution]
        p.tau, p.lambda_, p.max_particles_site = float(self.tau), float(self.lambda_), int(self.max_particles_site)
        return p


class RegionType:
    """Constructors for the RegionType variants of src/region.rs:10-20."""

    @staticmethod
    def _desc(kind, **kw) -> N.RegionDescC:
        d = N.RegionDescC()
        d.type = kind
        keep = []
        for k, v in kw.items():
            if isinstance(v, str):
                b = v.encode()
                keep.append(b)
                setattr(d, k, b)
            elif isinstance(v, (list, tuple, np.ndarray)):
                getattr(d, k)[:] = [float(x) for x in v]
            else:
                setattr(d, k, float(v))
        d._keep = keep  # keep the byte strings alive
        return d

    @staticmethod
    def Cube(name, p0, pf):
        return RegionType._desc(N.REGION_CUBE, name=name, p0=p0, pf=pf)

    @staticmethod
    def Sphere(name, center, radius):
        return RegionType._desc(N.REGION_SPHERE, name=name, center=center, radius=radius)

    @staticmethod
    def SemiSphere(name, center, radius, direction):
        return RegionType._desc(N.REGION_SEMISPHERE, name=name, center=center, radius=radius, direction=direction)

    @staticmethod
    def Cylinder(name, p0, pf, radius):
        return RegionType._desc(N.REGION_CYLINDER, name=name, p0=p0, pf=pf, radius=radius)

    @staticmethod
    def SphericalShell(shell_name, interior_name, center, internal_radius, external_radius):
        return RegionType._desc(N.REGION_SPHERICAL_SHELL, shell_name=shell_name, interior_name=interior_name,
                                center=center, internal_radius=internal_radius, external_radius=external_radius)

    @staticmethod
    def CylindricalShell(shell_name, interior_name, p0, pf, internal_radius, external_radius):
        return RegionType._desc(N.REGION_CYLINDRICAL_SHELL, shell_name=shell_name, interior_name=interior_name,
                                p0=p0, pf=pf, internal_radius=internal_radius, external_radius=external_radius)

    @staticmethod
    def Capsid(shell_name, interior_name, center, dir, internal_radius, external_radius, total_length):
        return RegionType._desc(N.REGION_CAPSID, shell_name=shell_name, interior_name=interior_name, center=center,
                                direction=dir, internal_radius=internal_radius, external_radius=external_radius,
                                total_length=total_length)


@dataclass
class SolverStatisticSample:
    """SolverStatisticSample<i32>, src/statistics.rs:4-9."""

    name: str
    value: int
    iteration_count: int


@dataclass
class Tables:
    regions: np.ndarray
    diffusion: np.ndarray
    stoich: np.ndarray
    reactants: np.ndarray
    rates: np.ndarray
    reservoir: np.ndarray


class Simulation:
    """Simulation (src/simulation.rs:29-46) backed by libcellsim."""

    def __init__(self, lattice_params: LatticeParams | None = None, *, _handle=None):
        self._lib = N.load()
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            N.check(self._lib.cs_create(C.byref(lattice_params.to_c()), C.byref(self._h)))
        self.stats: deque[SolverStatisticSample] = deque()
        self.rng_mode: int | None = None
        # species count (+1) of the prepared model, read once per preparation for counts();
        # every call that can change the model clears it
        self._s1: int | None = None
        # counts() reads into one persistent buffer (its ctypes pointer made once) and returns a copy
        self._counts_buf: np.ndarray | None = None
        self._counts_ptr = None

    @classmethod
    def from_file(cls, path: str, placement_seed: int = 0) -> "Simulation":
        """Simulation::from_file, src/simulation.rs:210-232 (no texture is created)."""
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.cs_from_json_file(str(path).encode(), placement_seed, C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def from_json(cls, text: str, placement_seed: int = 0) -> "Simulation":
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.cs_from_json_string(text.encode(), placement_seed, C.byref(h)))
        return cls(_handle=h)

    def close(self) -> None:
        if self._h:
            self._lib.cs_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- model
    def seed_placement(self, seed: int) -> None:
        N.check(self._lib.cs_seed_placement(self._h, seed))

    def add_region(self, region: N.RegionDescC, diffusion_rate: float) -> None:
        self._s1 = None
        N.check(self._lib.cs_add_region(self._h, C.byref(region), diffusion_rate))

    def prepare_regions(self) -> None:
        N.check(self._lib.cs_prepare_regions(self._h))

    def add_particle_count(self, name, to_region, count, logging, is_reservoir) -> None:
        self._s1 = None
        N.check(self._lib.cs_add_particle_count(self._h, name.encode(), to_region.encode(), count, int(logging),
                                                int(is_reservoir)))

    def add_particle_concentration(self, name, to_region, concentration, logging, is_reservoir) -> None:
        self._s1 = None
        N.check(self._lib.cs_add_particle_concentration(self._h, name.encode(), to_region.encode(), concentration,
                                                        int(logging), int(is_reservoir)))

    def fill_region(self, name, to_region, logging) -> None:
        self._s1 = None
        N.check(self._lib.cs_fill_region(self._h, name.encode(), to_region.encode(), int(logging)))

    def set_diffusion_rate(self, region, diffusion_rate) -> None:
        N.check(self._lib.cs_set_diffusion_rate(self._h, region.encode(), diffusion_rate))

    def set_diffusion_rate_particle(self, particle, region, diffusion_rate) -> None:
        N.check(self._lib.cs_set_diffusion_rate_particle(self._h, particle.encode(), region.encode(), diffusion_rate))

    def set_transition_rate(self, from_region, to_region, transition_rate) -> None:
        N.check(self._lib.cs_set_transition_rate(self._h, from_region.encode(), to_region.encode(), transition_rate))

    def set_transition_rate_particle(self, particle, from_region, to_region, transition_rate) -> None:
        N.check(self._lib.cs_set_transition_rate_particle(self._h, particle.encode(), from_region.encode(),
                                                          to_region.encode(), transition_rate))

    def add_reaction(self, reactants: Iterable[str], products: Iterable[str], k: float) -> None:
        self._s1 = None
        re = [r.encode() for r in reactants]
        pr = [p.encode() for p in products]
        ra = (C.c_char_p * max(len(re), 1))(*re)
        pa = (C.c_char_p * max(len(pr), 1))(*pr)
        N.check(self._lib.cs_add_reaction(self._h, ra, len(re), pa, len(pr), k))

    # ---------------------------------------------------------- introspection
    def info(self) -> N.InfoC:
        i = N.InfoC()
        N.check(self._lib.cs_get_info(self._h, C.byref(i)))
        return i

    @property
    def shape(self) -> tuple[int, int, int]:
        i = self.info()
        return tuple(int(x) for x in i.res)

    def name(self, kind: int, index: int) -> str:
        buf = C.create_string_buffer(256)
        N.check(self._lib.cs_get_name(self._h, kind, index, buf, 256))
        return buf.value.decode()

    @property
    def particle_names(self) -> list[str]:
        return [self.name(0, i) for i in range(self.info().n_species + 1)]

    @property
    def region_names(self) -> list[str]:
        return [self.name(1, i) for i in range(self.info().n_regions)]

    def region_volumes(self) -> np.ndarray:
        v = np.zeros(self.info().n_regions, np.uint32)
        N.check(self._lib.cs_get_region_volumes(self._h, N.ptr(v, C.c_uint32)))
        return v

    def tables(self) -> Tables:
        i = self.info()
        V, S1, R, NR = int(i.n_voxels), i.n_species + 1, i.n_reactions, i.n_regions
        t = Tables(np.zeros(V, np.uint32), np.zeros(NR * NR * S1, np.float32), np.zeros((R + 1) * S1, np.int32),
                   np.zeros((R + 1) * 3, np.uint32), np.zeros(R + 1, np.float32), np.zeros(V, np.uint32))
        N.check(self._lib.cs_get_tables(self._h, N.ptr(t.regions, C.c_uint32), N.ptr(t.diffusion, C.c_float),
                                        N.ptr(t.stoich, C.c_int32), N.ptr(t.reactants, C.c_uint32),
                                        N.ptr(t.rates, C.c_float), N.ptr(t.reservoir, C.c_uint32)))
        return t

    def set_tables(self, n_regions, n_species, n_reactions, regions, diffusion, stoich, reactants, rates,
                   reservoir=None) -> None:
        self._s1 = None
        arrs = [np.ascontiguousarray(a, dt) for a, dt in ((regions, np.uint32), (diffusion, np.float32),
                                                            (stoich, np.int32), (reactants, np.uint32),
                                                            (rates, np.float32))]
        res = None if reservoir is None else np.ascontiguousarray(reservoir, np.uint32)
        N.check(self._lib.cs_set_tables(self._h, n_regions, n_species, n_reactions, N.ptr(arrs[0], C.c_uint32),
                                        N.ptr(arrs[1], C.c_float), N.ptr(arrs[2], C.c_int32),
                                        N.ptr(arrs[3], C.c_uint32), N.ptr(arrs[4], C.c_float),
                                        N.ptr(res, C.c_uint32)))

    # ---------------------------------------------------------------- state
    def set_lattice(self, slots, occupancy=None, concentrations=None) -> None:
        s = np.ascontiguousarray(slots, np.uint32)
        o = None if occupancy is None else np.ascontiguousarray(occupancy, np.uint32)
        c = None if concentrations is None else np.ascontiguousarray(concentrations, np.int32)
        N.check(self._lib.cs_set_lattice(self._h, N.ptr(s, C.c_uint32), N.ptr(o, C.c_uint32), N.ptr(c, C.c_int32)))

    def get_lattice(self):
        i = self.info()
        V, K, S1 = int(i.n_voxels), i.max_particles_site, i.n_species + 1
        s = np.zeros(V * K, np.uint32)
        o = np.zeros(V, np.uint32)
        c = np.zeros(V * S1, np.int32)
        N.check(self._lib.cs_get_lattice(self._h, N.ptr(s, C.c_uint32), N.ptr(o, C.c_uint32), N.ptr(c, C.c_int32)))
        return s, o, c

    # ---------------------------------------------------------------- device
    def prepare_for_gpu(self, rng_mode: int = N.RNG_PHILOX, device: int = 0) -> None:
        """Simulation::prepare_for_gpu, src/simulation.rs:152-208."""
        self._s1 = None
        N.check(self._lib.cs_prepare_for_gpu(self._h, rng_mode, device))
        self.rng_mode = rng_mode
        self._s1 = self.info().n_species + 1

    def step(self, itimes: Sequence[int], write_freq: int = 0) -> None:
        """Simulation::step (src/simulation.rs:99-150) for len(itimes) frames with the reference RNG."""
        it = np.ascontiguousarray(itimes, np.uint32)
        N.check(self._lib.cs_step(self._h, len(it), N.ptr(it, C.c_uint32), write_freq))
        if write_freq:  # samples come only from calls that log
            self._drain_stats()

    def step_philox(self, n_steps: int, seed: int, write_freq: int = 0) -> None:
        N.check(self._lib.cs_step_philox(self._h, n_steps, seed, write_freq))
        if write_freq:
            self._drain_stats()

    def step_timed(self, itimes: Sequence[int]) -> float:
        it = np.ascontiguousarray(itimes, np.uint32)
        ms = C.c_float()
        N.check(self._lib.cs_step_timed(self._h, len(it), N.ptr(it, C.c_uint32), C.byref(ms)))
        return ms.value

    def step_philox_timed(self, n_steps: int, seed: int) -> float:
        ms = C.c_float()
        N.check(self._lib.cs_step_philox_timed(self._h, n_steps, seed, C.byref(ms)))
        return ms.value

    def set_precision(self, precision: int) -> None:
        N.check(self._lib.cs_set_precision(self._h, precision))

    def set_tiling(self, index: int, segment_length: int = 0) -> None:
        N.check(self._lib.cs_set_tiling(self._h, index, segment_length))

    def save_checkpoint(self, path) -> None:
        """Full state to a file (cs_checkpoint_save)."""
        N.check(self._lib.cs_checkpoint_save(self._h, str(path).encode()))

    @classmethod
    def load_checkpoint(cls, path, device: int = 0) -> "Simulation":
        """A handle resumed from a checkpoint file (cs_checkpoint_load)."""
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.cs_checkpoint_load(str(path).encode(), device, C.byref(h)))
        return cls(_handle=h)

    def render_view(self, view: int = 0, slice_axis: int = 0, slice: int = 0) -> np.ndarray:
        """The final_stage.wgsl views as a float32 (X, Y, Z) volume: 0 majority
        species, 1 regions, 2 reservoirs, each / 255 (cs_render_view)."""
        X, Y, Z = self.shape
        out = np.zeros((X, Y, Z), np.float32)
        N.check(self._lib.cs_render_view(self._h, view, slice_axis, slice, N.ptr(out, C.c_float), None))
        return out

    def autotune(self, frames_per_trial: int = 10) -> tuple[int, float]:
        """Time every compiled variant on this lattice (state restored afterwards)
        and keep the fastest: (chosen variant index, ms per frame)."""
        i, ms = C.c_int32(), C.c_float()
        N.check(self._lib.cs_autotune(self._h, frames_per_trial, C.byref(i), C.byref(ms)))
        return i.value, ms.value

    def get_tiling(self) -> int:
        i = C.c_int32()
        N.check(self._lib.cs_get_tiling(self._h, C.byref(i)))
        return i.value

    def counts(self) -> np.ndarray:
        """Species counts (StatisticsGroup buffer 0, src/statistics.rs:11-69)."""
        s1 = self._s1 if self._s1 is not None else self.info().n_species + 1
        buf = self._counts_buf
        if buf is None or buf.shape[0] != s1:
            buf = self._counts_buf = np.zeros(s1, np.int64)
            self._counts_ptr = N.ptr(buf, C.c_int64)
        N.check(self._lib.cs_get_counts(self._h, self._counts_ptr))
        return buf.copy()

    def diagnostics(self, n: int = 8) -> np.ndarray:
        d = np.zeros(n, np.uint32)
        N.check(self._lib.cs_get_diagnostics(self._h, N.ptr(d, C.c_uint32), n))
        return d

    def synchronize(self) -> None:
        N.check(self._lib.cs_synchronize(self._h))

    def debug_stall_group(self, group: int) -> None:
        """Test hook (cs_debug_stall_group): the next multi-frame launch's waits for `group` run out."""
        N.check(self._lib.cs_debug_stall_group(self._h, group))

    def _drain_stats(self) -> None:
        buf = (N.StatSampleC * 256)()
        names = None
        while True:
            n = C.c_uint32()
            N.check(self._lib.cs_pop_stats(self._h, buf, 256, C.byref(n)))
            if n.value == 0:
                break
            if names is None:
                names = self.particle_names
            for k in range(n.value):
                s = buf[k]
                self.stats.append(SolverStatisticSample(names[s.species], s.value, s.iteration_count))


def tiling_variants() -> list[tuple[int, int, int, int]]:
    """(K, TY, TZ, threads) of every compiled fused-kernel variant."""
    lib = N.load()
    n = C.c_int32()
    N.check(lib.cs_tiling_count(C.byref(n)))
    out = []
    for i in range(n.value):
        k, ty, tz, nt = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        N.check(lib.cs_tiling_describe(i, C.byref(k), C.byref(ty), C.byref(tz), C.byref(nt)))
        out.append((k.value, ty.value, tz.value, nt.value))
    return out


def tiling_kinds() -> list[tuple[int, int]]:
    """(kind, brick_planes) of every compiled variant: kind 0 = tile pipeline,
    kind 1 = sparse brick pass (crowded bricks finished by a full-capacity brick
    pass), kind 2 = sweep stream (the default; brick_planes 0), kind 3 = resident
    form (one block per replicate, its lattice in shared memory for every frame
    of a step call; small lattices only)."""
    lib = N.load()
    n = C.c_int32()
    N.check(lib.cs_tiling_count(C.byref(n)))
    out = []
    for i in range(n.value):
        kind, bx = C.c_int32(), C.c_int32()
        N.check(lib.cs_tiling_kind(i, C.byref(kind), C.byref(bx)))
        out.append((kind.value, bx.value))
    return out


def tiling_launches() -> list[int]:
    """Kernel launches per frame of every compiled variant, once a run is under
    way (cs_tiling_launches)."""
    lib = N.load()
    n = C.c_int32()
    N.check(lib.cs_tiling_count(C.byref(n)))
    out = []
    for i in range(n.value):
        k = C.c_int32()
        N.check(lib.cs_tiling_launches(i, C.byref(k)))
        out.append(k.value)
    return out


class Ensemble:
    """Replicates of one model stepped by one launch per frame (cs_ensemble_*)."""

    def __init__(self, model: Simulation, resolutions, seeds, rate_multipliers, initial_counts, device: int = 0):
        self._lib = N.load()
        self._h = C.c_void_p()
        res = np.ascontiguousarray(resolutions, np.uint32).reshape(-1, 3)
        sd = np.ascontiguousarray(seeds, np.uint64)
        mu = np.ascontiguousarray(rate_multipliers, np.float32)
        ic = np.ascontiguousarray(initial_counts, np.uint32)
        self.n = res.shape[0]
        self.resolutions = res
        self.S1 = model.info().n_species + 1
        self.K = model.info().max_particles_site
        N.check(self._lib.cs_ensemble_create(model._h, self.n, N.ptr(res, C.c_uint32), N.ptr(sd, C.c_uint64),
                                             N.ptr(mu, C.c_float), N.ptr(ic, C.c_uint32), device, C.byref(self._h)))

    def close(self):
        if self._h:
            self._lib.cs_ensemble_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n_steps: int, batched: bool = True) -> None:
        N.check(self._lib.cs_ensemble_step(self._h, n_steps, int(batched)))

    def step_timed(self, n_steps: int, batched: bool = True) -> float:
        ms = C.c_float()
        N.check(self._lib.cs_ensemble_step_timed(self._h, n_steps, int(batched), C.byref(ms)))
        return ms.value

    def set_precision(self, precision: int) -> None:
        N.check(self._lib.cs_ensemble_set_precision(self._h, precision))

    def set_tiling(self, index: int, segment_length: int = 0) -> None:
        N.check(self._lib.cs_ensemble_set_tiling(self._h, index, segment_length))

    def autotune(self, frames_per_trial: int = 5) -> tuple[int, float]:
        """Time every compiled variant on these replicates (state restored
        afterwards) and keep the fastest: (chosen variant index, ms per frame)."""
        i, ms = C.c_int32(), C.c_float()
        N.check(self._lib.cs_ensemble_autotune(self._h, frames_per_trial, C.byref(i), C.byref(ms)))
        return i.value, ms.value

    def counts(self) -> np.ndarray:
        out = np.zeros((self.n, self.S1), np.int64)
        N.check(self._lib.cs_ensemble_get_counts(self._h, N.ptr(out, C.c_int64)))
        return out

    def slots(self) -> np.ndarray:
        tot = C.c_uint64()
        N.check(self._lib.cs_ensemble_info(self._h, C.byref(tot), None))
        out = np.zeros(tot.value * self.K, np.uint8)
        N.check(self._lib.cs_ensemble_get_slots(self._h, N.ptr(out, C.c_uint8)))
        return out

    def diagnostics(self, n: int = 8) -> np.ndarray:
        d = np.zeros(n, np.uint32)
        N.check(self._lib.cs_ensemble_get_diagnostics(self._h, N.ptr(d, C.c_uint32), n))
        return d

    def info(self) -> tuple[int, int]:
        tot, items = C.c_uint64(), C.c_uint32()
        N.check(self._lib.cs_ensemble_info(self._h, C.byref(tot), C.byref(items)))
        return tot.value, items.value

    def synchronize(self) -> None:
        N.check(self._lib.cs_ensemble_synchronize(self._h))
