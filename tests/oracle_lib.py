"""ctypes access to the CPU oracle (oracle/libcbmref.so).

Test infrastructure: used only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "libcbmref.so")
# the CPU-baseline build (FMA contraction, unrolling): timed by bench.py,
# never used as the parity checker
TIMING_LIB_PATH = os.path.join(ORACLE_DIR, "libcbmref_timing.so")

_libs = {}
# which build init_state / run / run_calls / forcing use: False the parity
# build, True the timing build (bench.py's CPU legs set it)
TIMING = False


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib(timing=None):
    timing = TIMING if timing is None else timing
    path = TIMING_LIB_PATH if timing else LIB_PATH
    _lib = _libs.get(path)
    if _lib is None:
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        dp, ip, fp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_float)
        L.cbmref_state_field_name.restype = C.c_char_p
        L.cbmref_diag_name.restype = C.c_char_p
        L.cbmref_init.argtypes = [C.c_int, C.c_int, ip, ip, dp, dp, dp, dp, dp, dp]
        L.cbmref_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, ip, ip, dp, dp, fp,
                                 C.c_uint64, C.c_int, fp, fp, fp, fp, dp, dp, C.c_int]
        L.cbmref_run_calls.argtypes = [C.c_int, C.c_int, ip, C.c_double, C.c_int, C.c_int, ip, ip, dp, dp, fp,
                                       C.c_uint64, C.c_int, fp, fp, fp, fp, dp, dp, C.c_int]
        L.cbmref_forcing.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int, C.c_double, fp, fp, fp, fp, fp]
        for n in ("cbmref_psim", "cbmref_psis"):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [C.c_double]
        L.cbmref_qsat.restype = C.c_double
        L.cbmref_qsat.argtypes = [C.c_double, C.c_double]
        L.cbmref_spitter.restype = C.c_double
        L.cbmref_spitter.argtypes = [C.c_int, C.c_double, C.c_double]
        L.cbmref_trimb.argtypes = [dp, dp, dp, dp, C.c_int]
        L.cbmref_photosynthesis.restype = C.c_double
        L.cbmref_photosynthesis.argtypes = [C.c_double] * 11
        L.cbmref_pft_value.restype = C.c_double
        L.cbmref_pft_value.argtypes = [C.c_char_p, C.c_int]
        L.cbmref_soil_value.restype = C.c_double
        L.cbmref_soil_value.argtypes = [C.c_char_p, C.c_int]
        L.cbmref_params.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp]
        L.cbmref_soil_thermal_fix.argtypes = [C.c_int, dp, dp, dp, dp]
        _libs[path] = _lib = L
    return _lib


def _switch_mask(**switches):
    """The science-switch bits (the same as the library's, cable_gb300.runtime.switch_mask)."""
    from cable_gb300.runtime import switch_mask
    return switch_mask(**switches)


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def state_layout():
    """[(name, width)] of the flat state vector, in slot order."""
    L = lib()
    return [(L.cbmref_state_field_name(i).decode(), L.cbmref_state_field_width(i))
            for i in range(L.cbmref_num_state_fields())]


def diag_names():
    L = lib()
    return [L.cbmref_diag_name(i).decode() for i in range(L.cbmref_num_diag())]


def split_state(flat):
    """flat [slots, mp] -> {name: array [width, mp]}"""
    out, j = {}, 0
    for name, w in state_layout():
        out[name] = flat[j:j + w]
        j += w
    return out


def init_state(ts, precision=0):
    L = lib()
    mp = ts.mp
    st = np.zeros((L.cbmref_state_slots(), mp), np.float64)
    iveg = np.ascontiguousarray(ts.iveg, np.int32)
    isoil = np.ascontiguousarray(ts.isoilm, np.int32)
    d = lambda a: np.ascontiguousarray(a, np.float64)
    vlai, lat, sn, tg, wb = d(ts.vlai), d(ts.lat), d(ts.snowd0), d(ts.tgg0), d(ts.wb0)
    rc = L.cbmref_init(mp, precision, _p(iveg, C.c_int), _p(isoil, C.c_int), _p(vlai, C.c_double),
                       _p(lat, C.c_double), _p(sn, C.c_double), _p(tg, C.c_double), _p(wb, C.c_double),
                       _p(st, C.c_double))
    assert rc == 0
    return st


def run(ts, state, nsteps, ktau0=1, forcing=None, precision=0, nthreads=None, **switches):
    """Advance ``state`` (modified in place) by ``nsteps``; return the last
    step's diagnostics as {name: array[mp]}."""
    L = lib()
    mp = ts.mp
    nd = L.cbmref_num_diag()
    diag = np.zeros((nd, mp), np.float64)
    iveg = np.ascontiguousarray(ts.iveg, np.int32)
    isoil = np.ascontiguousarray(ts.isoilm, np.int32)
    vlai = np.ascontiguousarray(ts.vlai, np.float64)
    lat = np.ascontiguousarray(ts.lat, np.float64)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    tl, tp, tb, tsw = f32(ts.lat), f32(ts.lonphase), f32(ts.tbase), f32(ts.swscale)
    fptr = None
    if forcing is not None:
        forcing = np.ascontiguousarray(forcing, np.float32)
        assert forcing.shape == (nsteps, L.cbmref_num_forcing_fields(), mp)
        fptr = _p(forcing, C.c_float)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    assert state.flags["C_CONTIGUOUS"] and state.dtype == np.float64
    rc = L.cbmref_run(mp, nsteps, ktau0, float(ts.dels), precision, _switch_mask(**switches), _p(iveg, C.c_int),
                      _p(isoil, C.c_int), _p(vlai, C.c_double), _p(lat, C.c_double), fptr, ts.seed, ts.doy0,
                      _p(tl, C.c_float), _p(tp, C.c_float), _p(tb, C.c_float), _p(tsw, C.c_float),
                      _p(state, C.c_double), _p(diag, C.c_double), nthreads)
    assert rc == 0
    return dict(zip(diag_names(), diag))


def run_calls(ts, state, calls, forcing=None, precision=0, nthreads=None, **switches):
    """A sequence of offline / coupled calls on ``state`` (modified in place):
    calls = [(ktau, mode, final_cycle, lai_refresh), ...] with mode 0 cbm(),
    1 cbm_expl, 2 cbm_impl; forcing [ncalls][13][mp] or None (the synthetic
    record of each call's ktau).  Returns the last call's diagnostics."""
    L = lib()
    mp = ts.mp
    cl = np.ascontiguousarray(np.asarray(calls, np.int32).reshape(-1, 4))
    diag = np.zeros((L.cbmref_num_diag(), mp), np.float64)
    iveg = np.ascontiguousarray(ts.iveg, np.int32)
    isoil = np.ascontiguousarray(ts.isoilm, np.int32)
    vlai = np.ascontiguousarray(ts.vlai, np.float64)
    lat = np.ascontiguousarray(ts.lat, np.float64)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    tl, tp, tb, tsw = f32(ts.lat), f32(ts.lonphase), f32(ts.tbase), f32(ts.swscale)
    fptr = None
    if forcing is not None:
        forcing = np.ascontiguousarray(forcing, np.float32)
        assert forcing.shape == (len(cl), L.cbmref_num_forcing_fields(), mp)
        fptr = _p(forcing, C.c_float)
    assert state.flags["C_CONTIGUOUS"] and state.dtype == np.float64
    rc = L.cbmref_run_calls(mp, len(cl), _p(cl, C.c_int), float(ts.dels), precision, _switch_mask(**switches),
                            _p(iveg, C.c_int), _p(isoil, C.c_int), _p(vlai, C.c_double), _p(lat, C.c_double), fptr,
                            ts.seed, ts.doy0, _p(tl, C.c_float), _p(tp, C.c_float), _p(tb, C.c_float),
                            _p(tsw, C.c_float), _p(state, C.c_double), _p(diag, C.c_double),
                            nthreads or os.cpu_count() or 1)
    assert rc == 0
    return dict(zip(diag_names(), diag))


def forcing(ts, step0, nsteps):
    L = lib()
    mp = ts.mp
    out = np.zeros((nsteps, L.cbmref_num_forcing_fields(), mp), np.float32)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    tl, tp, tb, tsw = f32(ts.lat), f32(ts.lonphase), f32(ts.tbase), f32(ts.swscale)
    L.cbmref_forcing(mp, step0, nsteps, ts.seed, ts.doy0, float(ts.dels), _p(tl, C.c_float), _p(tp, C.c_float),
                     _p(tb, C.c_float), _p(tsw, C.c_float), _p(out, C.c_float))
    return out


FORCING_FIELDS = ["fsd1", "fsd2", "fld", "precip", "precip_sn", "tk", "pmb", "ua", "qv", "ca", "coszen", "doy", "hod"]
