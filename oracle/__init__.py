"""CPU oracle of the RDME timestep — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this
package, as the checker or as the timed CPU baseline; the product library
never links or calls it.  See oracle.h for the parity status.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRCS = ["oracle_math.c", "ref_semantics.c", "prod_semantics.c", "ssa_fp64.c"]


def build(force: bool = False) -> Path:
    """gcc -O2 -fopenmp -ffp-contract=off: every float op a single binary32 op."""
    srcs = [HERE / s for s in SRCS]
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in srcs + [HERE / "oracle.h"]):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-o", str(tmp), *map(str, srcs), "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(tmp, LIB)
    return LIB


class Params(C.Structure):
    _fields_ = [("res", C.c_uint32 * 3), ("K", C.c_uint32), ("n_regions", C.c_uint32), ("n_species", C.c_uint32),
                ("n_reactions", C.c_uint32), ("tau", C.c_float), ("lambda_", C.c_float)]


class Tables(C.Structure):
    _fields_ = [("regions", C.c_void_p), ("diffusion", C.c_void_p), ("stoich", C.c_void_p),
                ("reactants", C.c_void_p), ("rates", C.c_void_p), ("reservoir", C.c_void_p)]


class ProdParams(C.Structure):
    _fields_ = [("res", C.c_uint32 * 3), ("K", C.c_uint32), ("n_regions", C.c_uint32), ("n_species", C.c_uint32),
                ("n_reactions", C.c_uint32), ("precision", C.c_uint32), ("max_events", C.c_uint32),
                ("tau", C.c_float), ("lambda_", C.c_float), ("rate_mult", C.c_float), ("seed", C.c_uint64)]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.orc_pcg.restype = C.c_uint32
        lib.orc_pcg.argtypes = [C.c_uint32]
        lib.orc_xorshift.restype = C.c_uint32
        lib.orc_xorshift.argtypes = [C.c_uint32]
        lib.orc_uniform_float.restype = C.c_float
        lib.orc_uniform_float.argtypes = [C.c_uint32]
        lib.orc_expf.restype = C.c_float
        lib.orc_expf.argtypes = [C.c_float]
        lib.orc_logf.restype = C.c_float
        lib.orc_logf.argtypes = [C.c_float]
        lib.orc_philox4x32_10.restype = None
        lib.orc_philox4x32_10.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.orc_ref_run.restype = C.c_int
        lib.orc_ref_run.argtypes = [C.POINTER(Params), C.POINTER(Tables), C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        lib.orc_prod_run.restype = C.c_int
        lib.orc_prod_run.argtypes = [C.POINTER(ProdParams), C.POINTER(Tables), C.c_void_p, C.c_void_p, C.c_uint32,
                                     C.c_uint32, C.c_void_p]
        lib.orc_first_event_inside.restype = C.c_uint32
        lib.orc_first_event_inside.argtypes = [C.c_float, C.c_float, C.c_uint32, C.c_uint32]
        lib.orc_ssa_fp64_batch.restype = C.c_int64
        lib.orc_ssa_fp64_batch.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                           C.c_int32, C.c_int64, C.c_void_p]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class RefState:
    """Reference-layout state arrays (numpy) for the oracle and the library."""

    def __init__(self, slots, occ, conc, stat):
        self.slots = np.ascontiguousarray(slots, np.uint32).copy()
        self.occ = np.ascontiguousarray(occ, np.uint32).copy()
        self.conc = np.ascontiguousarray(conc, np.int32).copy()
        self.stat = np.ascontiguousarray(stat, np.int32).copy()
        self.diag = np.zeros(8, np.uint32)


def _tables(tab):
    arrs = dict(regions=np.ascontiguousarray(tab.regions, np.uint32),
                diffusion=np.ascontiguousarray(tab.diffusion, np.float32),
                stoich=np.ascontiguousarray(tab.stoich, np.int32),
                reactants=np.ascontiguousarray(tab.reactants, np.uint32),
                rates=np.ascontiguousarray(tab.rates, np.float32),
                reservoir=np.ascontiguousarray(tab.reservoir, np.uint32))
    t = Tables(*(a.ctypes.data for a in arrs.values()))
    return t, arrs


def ref_run(res, K, n_regions, n_species, n_reactions, tau, lam, tab, state: RefState, itimes, mode=0, threads=0):
    """Runs len(itimes) reference frames in place on `state` (mode 0 serial, 1 gather/OpenMP)."""
    lib = load()
    p = Params((C.c_uint32 * 3)(*res), K, n_regions, n_species, n_reactions, tau, lam)
    t, keep = _tables(tab)
    it = np.ascontiguousarray(itimes, np.uint32)
    rc = lib.orc_ref_run(C.byref(p), C.byref(t), _p(state.slots), _p(state.occ), _p(state.conc), _p(state.stat),
                         len(it), _p(it), _p(state.diag), mode, threads)
    if rc != 0:
        raise ValueError(f"orc_ref_run failed: {rc}")
    return state


def prod_run(res, K, n_regions, n_species, n_reactions, tau, lam, tab, slots_u8, counts, seed, frame0, n_steps,
             precision=0, max_events=64, rate_mult=1.0, diag=None):
    lib = load()
    p = ProdParams((C.c_uint32 * 3)(*res), K, n_regions, n_species, n_reactions, precision, max_events, tau, lam,
                   rate_mult, seed)
    t, keep = _tables(tab)
    if diag is None:
        diag = np.zeros(8, np.uint32)
    rc = lib.orc_prod_run(C.byref(p), C.byref(t), _p(slots_u8), _p(counts), frame0, n_steps, _p(diag))
    if rc != 0:
        raise ValueError(f"orc_prod_run failed: {rc}")
    return diag


def first_event_inside(a0, tau, lo, hi) -> int:
    """Draws m in [lo, hi] (u1 = m 2^-24) whose first reaction event lands inside tau."""
    return int(load().orc_first_event_inside(float(a0), float(tau), int(lo), int(hi)))


def ssa_batch(S, reactants, rates, ch_species, ch_delta, x0, seed0, n_rep, t_samples, fpt_species=0, fpt_threshold=0):
    """Well-mixed FP64 SSA over n_rep replicates; returns (samples[n_rep][n_t][S+1], fpt[n_rep])."""
    lib = load()
    re = np.ascontiguousarray(reactants, np.uint8)
    R = re.shape[0]
    rt = np.ascontiguousarray(rates, np.float64)
    cs = np.ascontiguousarray(ch_species, np.uint8)
    cd = np.ascontiguousarray(ch_delta, np.int8)
    x = np.ascontiguousarray(x0, np.int64)
    ts = np.ascontiguousarray(t_samples, np.float64)
    out = np.zeros((n_rep, len(ts), S + 1), np.int64)
    fpt = np.zeros(n_rep, np.float64)
    lib.orc_ssa_fp64_batch(S, R, _p(re), _p(rt), _p(cs), _p(cd), _p(x), seed0, n_rep, len(ts), _p(ts), _p(out),
                           fpt_species, fpt_threshold, _p(fpt))
    return out, fpt
