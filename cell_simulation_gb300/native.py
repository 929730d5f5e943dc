"""ctypes binding of libcellsim.so (include/cellsim.h).

The library is built in-tree (``cell_simulation_gb300/libcellsim.so``); a
missing library is an error, never a silent fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libcellsim.so"

CS_OK = 0
STATUS_NAMES = {
    0: "CS_OK", 1: "CS_ERR_INVALID_ARG", 2: "CS_ERR_NOT_FOUND", 3: "CS_ERR_LIMIT", 4: "CS_ERR_STATE",
    5: "CS_ERR_PARSE", 6: "CS_ERR_IO", 7: "CS_ERR_CUDA", 8: "CS_ERR_CAPACITY", 9: "CS_ERR_DEVICE_STATUS",
}
RNG_REFERENCE, RNG_PHILOX = 0, 1
PREC_MIXED, PREC_FP32, PREC_FP64 = 0, 1, 2
REGION_CUBE, REGION_SPHERE, REGION_SEMISPHERE, REGION_CYLINDER = 0, 1, 2, 3
REGION_SPHERICAL_SHELL, REGION_CYLINDRICAL_SHELL, REGION_CAPSID = 4, 5, 6


class CellsimError(RuntimeError):
    """A libcellsim call returned a non-zero cs_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class LatticeParamsC(C.Structure):
    _fields_ = [("dims", C.c_float * 3), ("res", C.c_uint32 * 3), ("tau", C.c_float), ("lambda_", C.c_float),
                ("max_particles_site", C.c_uint32)]


class RegionDescC(C.Structure):
    _fields_ = [("type", C.c_int32), ("name", C.c_char_p), ("shell_name", C.c_char_p), ("interior_name", C.c_char_p),
                ("p0", C.c_float * 3), ("pf", C.c_float * 3), ("center", C.c_float * 3), ("direction", C.c_float * 3),
                ("radius", C.c_float), ("internal_radius", C.c_float), ("external_radius", C.c_float),
                ("total_length", C.c_float)]


class InfoC(C.Structure):
    _fields_ = [("res", C.c_uint32 * 3), ("max_particles_site", C.c_uint32), ("n_regions", C.c_uint32),
                ("n_species", C.c_uint32), ("n_reactions", C.c_uint32), ("n_logging", C.c_uint32),
                ("n_voxels", C.c_uint64), ("frame", C.c_uint64), ("tau", C.c_float), ("lambda_", C.c_float),
                ("dims", C.c_float * 3), ("rng_mode", C.c_int32), ("device", C.c_int32)]


class RefFrameNoAllocArgsC(C.Structure):
    _fields_ = [("device", C.c_int32), ("stream", C.c_void_p), ("res", C.c_uint32 * 3),
                ("max_particles_site", C.c_uint32), ("n_regions", C.c_uint32), ("n_species", C.c_uint32),
                ("n_reactions", C.c_uint32), ("tau", C.c_float)] + [
        (n, C.c_void_p) for n in ("slots_in", "occupancy_in", "conc_in", "slots_out", "occupancy_out", "conc_out",
                                  "regions", "reservoir", "probabilities", "stoich", "reactants", "rates", "itime",
                                  "counts", "diag")]


class StatSampleC(C.Structure):
    _fields_ = [("species", C.c_uint32), ("value", C.c_int32), ("iteration_count", C.c_uint32)]


P = C.c_void_p
u32p, i32p, f32p, u64p, i64p, u8p = (C.POINTER(C.c_uint32), C.POINTER(C.c_int32), C.POINTER(C.c_float),
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.POINTER(C.c_uint8))
st = C.c_int32

# name -> (restype, argtypes); this table lists every symbol include/cellsim.h declares
SIGNATURES = {
    "cs_version": (C.c_char_p, []),
    "cs_last_error": (C.c_char_p, []),
    "cs_create": (st, [C.POINTER(LatticeParamsC), C.POINTER(P)]),
    "cs_from_json_file": (st, [C.c_char_p, C.c_uint64, C.POINTER(P)]),
    "cs_from_json_string": (st, [C.c_char_p, C.c_uint64, C.POINTER(P)]),
    "cs_destroy": (None, [P]),
    "cs_seed_placement": (st, [P, C.c_uint64]),
    "cs_add_region": (st, [P, C.POINTER(RegionDescC), C.c_float]),
    "cs_prepare_regions": (st, [P]),
    "cs_add_particle_count": (st, [P, C.c_char_p, C.c_char_p, C.c_uint32, C.c_int32, C.c_int32]),
    "cs_add_particle_concentration": (st, [P, C.c_char_p, C.c_char_p, C.c_float, C.c_int32, C.c_int32]),
    "cs_fill_region": (st, [P, C.c_char_p, C.c_char_p, C.c_int32]),
    "cs_set_diffusion_rate": (st, [P, C.c_char_p, C.c_float]),
    "cs_set_diffusion_rate_particle": (st, [P, C.c_char_p, C.c_char_p, C.c_float]),
    "cs_set_transition_rate": (st, [P, C.c_char_p, C.c_char_p, C.c_float]),
    "cs_set_transition_rate_particle": (st, [P, C.c_char_p, C.c_char_p, C.c_char_p, C.c_float]),
    "cs_add_reaction": (st, [P, C.POINTER(C.c_char_p), C.c_uint32, C.POINTER(C.c_char_p), C.c_uint32, C.c_float]),
    "cs_get_info": (st, [P, C.POINTER(InfoC)]),
    "cs_get_tables": (st, [P, u32p, f32p, i32p, u32p, f32p, u32p]),
    "cs_get_region_volumes": (st, [P, u32p]),
    "cs_get_name": (st, [P, C.c_int32, C.c_uint32, C.c_char_p, C.c_uint32]),
    "cs_set_tables": (st, [P, C.c_uint32, C.c_uint32, C.c_uint32, u32p, f32p, i32p, u32p, f32p, u32p]),
    "cs_set_lattice": (st, [P, u32p, u32p, i32p]),
    "cs_get_lattice": (st, [P, u32p, u32p, i32p]),
    "cs_prepare_for_gpu": (st, [P, C.c_int32, C.c_int32]),
    "cs_step": (st, [P, C.c_uint32, u32p, C.c_uint32]),
    "cs_step_philox": (st, [P, C.c_uint32, C.c_uint64, C.c_uint32]),
    "cs_set_precision": (st, [P, C.c_int32]),
    "cs_get_counts": (st, [P, i64p]),
    "cs_pop_stats": (st, [P, C.POINTER(StatSampleC), C.c_uint32, u32p]),
    "cs_get_diagnostics": (st, [P, u32p, C.c_uint32]),
    "cs_synchronize": (st, [P]),
    "cs_debug_stall_group": (st, [P, C.c_uint32]),
    "cs_ref_frame_noalloc": (st, [C.POINTER(RefFrameNoAllocArgsC)]),
    "cs_step_timed": (st, [P, C.c_uint32, u32p, f32p]),
    "cs_step_philox_timed": (st, [P, C.c_uint32, C.c_uint64, f32p]),
    "cs_tiling_count": (st, [i32p]),
    "cs_tiling_describe": (st, [C.c_int32, i32p, i32p, i32p, i32p]),
    "cs_tiling_kind": (st, [C.c_int32, i32p, i32p]),
    "cs_tiling_launches": (st, [C.c_int32, i32p]),
    "cs_autotune": (st, [P, C.c_uint32, i32p, C.POINTER(C.c_float)]),
    "cs_checkpoint_save": (st, [P, C.c_char_p]),
    "cs_checkpoint_load": (st, [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "cs_render_view": (st, [P, C.c_int32, C.c_int32, C.c_uint32, C.POINTER(C.c_float), C.c_void_p]),
    "cs_ensemble_autotune": (st, [P, C.c_uint32, i32p, C.POINTER(C.c_float)]),
    "cs_set_tiling": (st, [P, C.c_int32, C.c_uint32]),
    "cs_get_tiling": (st, [P, i32p]),
    "cs_ensemble_create": (st, [P, C.c_uint32, u32p, u64p, f32p, u32p, C.c_int32, C.POINTER(P)]),
    "cs_ensemble_destroy": (None, [P]),
    "cs_ensemble_step": (st, [P, C.c_uint32, C.c_int32]),
    "cs_ensemble_step_timed": (st, [P, C.c_uint32, C.c_int32, f32p]),
    "cs_ensemble_set_precision": (st, [P, C.c_int32]),
    "cs_ensemble_set_tiling": (st, [P, C.c_int32, C.c_uint32]),
    "cs_ensemble_get_counts": (st, [P, i64p]),
    "cs_ensemble_get_slots": (st, [P, u8p]),
    "cs_ensemble_get_diagnostics": (st, [P, u32p, C.c_uint32]),
    "cs_ensemble_synchronize": (st, [P]),
    "cs_ensemble_info": (st, [P, u64p, u32p]),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libcellsim.so (once) and attach the prototypes."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise CellsimError(7, f"{p} is missing: run __graft_entry__.build() (there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int) -> None:
    if status != CS_OK:
        msg = load().cs_last_error()
        raise CellsimError(status, msg.decode() if msg else "")


def ptr(arr, ctype):
    """Pointer to a contiguous numpy array (or None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(C.POINTER(ctype))
