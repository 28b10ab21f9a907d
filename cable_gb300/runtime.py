"""ctypes binding of the C ABI in ``include/cablegpu.h``.

:class:`CableGPU` owns one device context: the per-tile parameters and
state of ``mp`` tiles resident in GPU memory, advanced by the fused timestep
kernel.  Field arrays cross the boundary in the reference's Fortran layout,
``(mp, nlayer)`` column-major, i.e. numpy arrays of shape ``(nlayer, mp)``.

There is no CPU fallback: if the CUDA library cannot be loaded, or no GPU is
present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

F32, F64, I32 = 0, 1, 2
KIND_PARAM, KIND_STATE, KIND_OUTPUT, KIND_DIAG, KIND_FORCING = 0, 1, 2, 3, 4
NFORCING = 13
FORCING_FIELDS = ["fsd_vis", "fsd_nir", "fld", "precip", "precip_sn", "tk", "pmb", "ua", "qv", "ca", "coszen", "doy",
                  "hod"]
OUTPUT_FIELDS = ["fe", "fh", "fgpp", "frday", "tv", "rnet", "ga", "trad"]
_NP = {F32: np.float32, F64: np.float64, I32: np.int32}

ERRORS = {-1: "CABLEGPU_ERR_ARG", -2: "CABLEGPU_ERR_CUDA", -3: "CABLEGPU_ERR_NONFINITE", -4: "CABLEGPU_ERR_STATE",
          -5: "CABLEGPU_ERR_IO"}

# Every symbol include/cablegpu.h declares.
EXPORTS = [
    "cablegpu_create", "cablegpu_destroy", "cablegpu_cold_start", "cablegpu_num_fields", "cablegpu_field_info",
    "cablegpu_field_id", "cablegpu_set_field", "cablegpu_get_field", "cablegpu_field_device_ptr",
    "cablegpu_set_forcing", "cablegpu_set_synthetic_forcing", "cablegpu_set_options", "cablegpu_step",
    "cablegpu_run", "cablegpu_synchronize", "cablegpu_run_timed", "cablegpu_kernel_timed",
    "cablegpu_launch_count", "cablegpu_param_table", "cablegpu_last_error", "cablegpu_phase_timed",
    "cablegpu_cold_start_noalloc", "cablegpu_harvest", "cablegpu_harvest_rows", "cablegpu_surrogate_train",
    "cablegpu_surrogate_weights", "cablegpu_set_surrogate", "cablegpu_surrogate_stats", "cablegpu_mlp_sizes",
    "cablegpu_mlp_forward", "cablegpu_mlp_grad", "cablegpu_mlp_fit", "cablegpu_mlp_last_error",
    "cablegpu_set_blocks", "cablegpu_get_config", "cablegpu_autotune", "cablegpu_step_host",
    "cablegpu_restart_write", "cablegpu_restart_read", "cablegpu_forcing_file_write", "cablegpu_file_info",
    "cablegpu_run_forcing_file", "cablegpu_set_host_layout", "cablegpu_tile_order",
    "cablegpu_step_explicit", "cablegpu_step_implicit", "cablegpu_coupled_timed", "cablegpu_set_soil_solve",
    "cablegpu_set_canopy_schedule", "cablegpu_check_tile_param", "cablegpu_tune_blocks",
    "cablegpu_host_register", "cablegpu_host_unregister", "cablegpu_get_fields",
    "cablegpu_host_alloc", "cablegpu_host_free",
]
NOALLOC_MAX_TILES = 65536
MAX_TILES = 33554176      # CABLEGPU_MAX_TILES: the most tiles one context takes
# soil tridiagonal solve arithmetic (cablegpu_set_soil_solve)
SOLVE_FP64 = 0
SOLVE_FP32_CHANGE = 1
# canopy dryLeaf pass scheduling (cablegpu_set_canopy_schedule)
CANOPY_POOL = 0
CANOPY_LANES = 1
# science switch bits of cablegpu_set_options (include/cablegpu.h)
SW_MEDLYN = 1
SW_SOIL_THERMAL_FIX = 2
SW_LITTER = 4
SW_L_REV_CORR = 8
SW_FWSOIL_NONLINEAR = 16
SW_FWSOIL_LAI_KTAUL = 32
SW_POTEV_PM = 64
SW_NEW_REDUCE_SOILEVP = 128
SW_NEW_RUNOFF_SPEED = 256
SW_DIAG_SOIL_RESP_OFF = 512
# per-tile status bits of the field "tile_status" (include/cablegpu.h)
TILE_NONFINITE = 1
TILE_DRYLEAF_NOCONV = 2
TILE_FORCING_RANGE = 4
TILE_OUTPUT_RANGE = 8
TILE_EVAPFBL = 16
FWSOIL_SWITCH = {"standard": 0, "non-linear extrapolation": SW_FWSOIL_NONLINEAR,
                 "Lai and Ktaul 2000": SW_FWSOIL_LAI_KTAUL}


def switch_mask(medlyn=False, soil_thermal_fix=False, litter=False, l_rev_corr=False, fwsoil_switch="standard",
                ssnow_potev="HDM", l_new_reduce_soilevp=False, l_new_runoff_speed=False, diag_soil_resp="ON") -> int:
    """cablegpu_set_options mask of the reference's science switches
    (``cable_user`` names and values; the defaults are the offline ones)."""
    if fwsoil_switch not in FWSOIL_SWITCH:
        raise ValueError("fwsoil_switch %r: one of %s" % (fwsoil_switch, list(FWSOIL_SWITCH)))
    if ssnow_potev not in ("HDM", "P-M"):
        raise ValueError("ssnow_potev %r: 'HDM' or 'P-M'" % ssnow_potev)
    if diag_soil_resp.strip().upper() not in ("ON", "OFF"):
        raise ValueError("diag_soil_resp %r: 'ON' or 'OFF'" % diag_soil_resp)
    return ((SW_MEDLYN if medlyn else 0) | (SW_SOIL_THERMAL_FIX if soil_thermal_fix else 0) |
            (SW_LITTER if litter else 0) | (SW_L_REV_CORR if l_rev_corr else 0) | FWSOIL_SWITCH[fwsoil_switch] |
            (SW_POTEV_PM if ssnow_potev == "P-M" else 0) | (SW_NEW_REDUCE_SOILEVP if l_new_reduce_soilevp else 0) |
            (SW_NEW_RUNOFF_SPEED if l_new_runoff_speed else 0) |
            (SW_DIAG_SOIL_RESP_OFF if diag_soil_resp.strip().upper() == "OFF" else 0))


def param_table(table: int, name: str) -> np.ndarray:
    """A built-in parameter table (cablegpu_param_table): table 0 per plant
    type (17 values; "froot" 6 x 17, layer-major), 1 per soil type (9), 2 the
    per-soil table with the soil_thermal_fix set applied."""
    L = load()
    out = np.zeros(6 * 17, np.float32)
    rc = L.cablegpu_param_table(int(table), name.encode(), _ptr(out, C.c_float), out.size)
    if rc != 0:
        raise CableGPUError(rc, "param_table: no entry %r in table %d" % (name, table))
    n = 6 * 17 if name == "froot" else (17 if table == 0 else 9)
    return out[:n].copy()


def forcing_file_write(path, forcing, doy0: int = 1, dels: float = 1800.0):
    """Binary forcing file from [nsteps][13][mp] float32 met forcing."""
    f = np.ascontiguousarray(forcing, np.float32)
    assert f.ndim == 3 and f.shape[1] == NFORCING
    L = load()
    rc = L.cablegpu_forcing_file_write(os.fsencode(path), f.shape[2], f.shape[0], int(doy0), float(dels),
                                       _ptr(f, C.c_float))
    if rc != 0:
        raise CableGPUError(rc, "forcing_file_write failed for %s" % path)


def file_info(path) -> dict:
    """Header of a restart, forcing or output file."""
    L = load()
    kind, nrec, nf, ktau, doy0 = (C.c_int() for _ in range(5))
    mp, dels = C.c_longlong(), C.c_float()
    rc = L.cablegpu_file_info(os.fsencode(path), C.byref(kind), C.byref(mp), C.byref(nrec), C.byref(nf),
                              C.byref(ktau), C.byref(doy0), C.byref(dels))
    if rc != 0:
        raise CableGPUError(rc, "not a readable CABLEGPU file: %s" % path)
    return {"kind": kind.value, "mp": mp.value, "nrecords": nrec.value, "nfields": nf.value, "ktau": ktau.value,
            "doy0": doy0.value, "dels": dels.value}

PHASES = ["radiation", "canopy", "snow_pack", "soil_heat", "soil_water", "surrogate_net"]

_lib = None


class CableGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


class _Tiles(C.Structure):
    _fields_ = [("mp", C.c_int), ("iveg", C.POINTER(C.c_int)), ("isoilm", C.POINTER(C.c_int)),
                ("vlai", C.POINTER(C.c_float)), ("lat", C.POINTER(C.c_float)), ("lonphase", C.POINTER(C.c_float)),
                ("tbase", C.POINTER(C.c_float)), ("swscale", C.POINTER(C.c_float)), ("order", C.c_int)]


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library and declare its ABI."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("cable_gb300 CUDA library missing (%s); run cable_gb300.build.build()" % _build.LIB)
    L = C.CDLL(_build.LIB)
    vp, ip = C.c_void_p, C.c_int
    L.cablegpu_create.argtypes = [C.POINTER(_Tiles), ip, C.POINTER(vp)]
    L.cablegpu_destroy.argtypes = [vp]
    L.cablegpu_cold_start.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.cablegpu_cold_start_noalloc.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.POINTER(C.c_double)]
    fp = C.POINTER(C.c_float)
    L.cablegpu_mlp_sizes.argtypes = [C.POINTER(ip), C.POINTER(ip), C.POINTER(ip)]
    L.cablegpu_mlp_forward.argtypes = [fp, fp, fp, C.c_longlong, fp]
    L.cablegpu_mlp_grad.argtypes = [fp, fp, fp, C.c_longlong, fp, fp]
    L.cablegpu_mlp_fit.argtypes = [fp, C.c_longlong, C.c_longlong, ip, ip, C.c_float, C.c_ulonglong, fp, fp, fp]
    L.cablegpu_harvest.argtypes = [vp, ip, ip, C.c_float, C.c_float, C.c_ulonglong, C.c_longlong,
                                   C.POINTER(C.c_longlong)]
    L.cablegpu_harvest_rows.argtypes = [vp, fp, C.c_longlong]
    L.cablegpu_surrogate_train.argtypes = [vp, ip, ip, C.c_float, C.c_float, C.c_ulonglong, fp]
    L.cablegpu_surrogate_weights.argtypes = [vp, fp, fp, ip]
    L.cablegpu_set_surrogate.argtypes = [vp, ip, C.c_float]
    L.cablegpu_surrogate_stats.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), ip]
    L.cablegpu_mlp_last_error.argtypes = []
    L.cablegpu_mlp_last_error.restype = C.c_char_p
    L.cablegpu_num_fields.argtypes = []
    L.cablegpu_field_info.argtypes = [ip, C.POINTER(C.c_char_p), C.POINTER(ip), C.POINTER(ip), C.POINTER(ip)]
    L.cablegpu_field_id.argtypes = [C.c_char_p]
    L.cablegpu_set_field.argtypes = [vp, ip, vp]
    L.cablegpu_get_field.argtypes = [vp, ip, vp]
    L.cablegpu_field_device_ptr.argtypes = [vp, ip, C.POINTER(vp), C.POINTER(ip)]
    L.cablegpu_set_forcing.argtypes = [vp, C.POINTER(C.c_float)]
    L.cablegpu_set_synthetic_forcing.argtypes = [vp, C.c_ulonglong, ip]
    L.cablegpu_set_options.argtypes = [vp, ip, ip, ip]
    L.cablegpu_set_soil_solve.argtypes = [vp, ip]
    L.cablegpu_set_canopy_schedule.argtypes = [vp, ip]
    L.cablegpu_check_tile_param.argtypes = [vp, C.c_char_p, C.POINTER(C.c_float)]
    L.cablegpu_step.argtypes = [vp, ip, C.c_float]
    L.cablegpu_step_explicit.argtypes = [vp, ip, C.c_float, ip]
    L.cablegpu_coupled_timed.argtypes = [vp, ip, ip, C.c_float, ip, C.POINTER(C.c_float)]
    L.cablegpu_step_implicit.argtypes = [vp, ip, C.c_float, ip, ip]
    L.cablegpu_run.argtypes = [vp, ip, ip, C.c_float]
    L.cablegpu_synchronize.argtypes = [vp]
    L.cablegpu_run_timed.argtypes = [vp, ip, ip, C.c_float, C.POINTER(C.c_float)]
    L.cablegpu_kernel_timed.argtypes = [vp, ip, ip, C.c_float, C.POINTER(C.c_float)]
    L.cablegpu_phase_timed.argtypes = [vp, ip, ip, C.c_float, C.POINTER(C.c_float)]
    L.cablegpu_step_host.argtypes = [vp, ip, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.cablegpu_set_blocks.argtypes = [vp, C.POINTER(ip)]
    L.cablegpu_get_config.argtypes = [vp, C.POINTER(ip), C.POINTER(ip)]
    L.cablegpu_get_fields.argtypes = [vp, ip, C.POINTER(ip), C.POINTER(vp)]
    L.cablegpu_host_register.argtypes = [vp, C.c_size_t]
    L.cablegpu_host_unregister.argtypes = [vp]
    L.cablegpu_host_alloc.argtypes = [C.c_size_t, C.POINTER(vp)]
    L.cablegpu_host_free.argtypes = [vp]
    L.cablegpu_tune_blocks.argtypes = [vp, ip, ip, C.c_float, C.POINTER(ip), C.POINTER(C.c_float)]
    L.cablegpu_autotune.argtypes = [C.POINTER(_Tiles), ip, ip, ip, C.POINTER(ip), C.POINTER(ip), C.POINTER(C.c_float)]
    L.cablegpu_launch_count.argtypes = [vp]
    L.cablegpu_launch_count.restype = C.c_longlong
    L.cablegpu_param_table.argtypes = [ip, C.c_char_p, C.POINTER(C.c_float), ip]
    L.cablegpu_restart_write.argtypes = [vp, C.c_char_p, ip]
    L.cablegpu_restart_read.argtypes = [vp, C.c_char_p, C.POINTER(ip)]
    L.cablegpu_forcing_file_write.argtypes = [C.c_char_p, ip, ip, ip, C.c_float, C.POINTER(C.c_float)]
    L.cablegpu_file_info.argtypes = [C.c_char_p, C.POINTER(ip), C.POINTER(C.c_longlong), C.POINTER(ip), C.POINTER(ip),
                                     C.POINTER(ip), C.POINTER(ip), C.POINTER(C.c_float)]
    L.cablegpu_run_forcing_file.argtypes = [vp, C.c_char_p, ip, ip, ip, C.c_char_p]
    L.cablegpu_set_host_layout.argtypes = [vp, ip]
    L.cablegpu_tile_order.argtypes = [vp, C.POINTER(ip)]
    L.cablegpu_last_error.argtypes = [vp]
    L.cablegpu_last_error.restype = C.c_char_p
    _lib = L
    return L


def fields():
    """{name: (id, nlayer, dtype, kind)} of the library's field registry."""
    L = load()
    out = {}
    for i in range(L.cablegpu_num_fields()):
        n, nl, dt, kd = C.c_char_p(), C.c_int(), C.c_int(), C.c_int()
        L.cablegpu_field_info(i, C.byref(n), C.byref(nl), C.byref(dt), C.byref(kd))
        out[n.value.decode()] = (i, nl.value, dt.value, kd.value)
    return out


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


# ---------------------------------------------------------------- surrogate network
MLP_NPARAM, MLP_NNORM, MLP_ROW = 5187, 30, 16


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    if shape is not None:
        assert a.shape == shape, (a.shape, shape)
    return a


def _mlp_check(rc):
    if rc != 0:
        raise CableGPUError(rc, load().cablegpu_mlp_last_error().decode())


def mlp_forward(params, norm, rows):
    """Raw network outputs [n][3] for training-format rows [n][16]."""
    L = load()
    rows = _f32(rows)
    n = rows.shape[0]
    y = np.empty((n, 3), np.float32)
    _mlp_check(L.cablegpu_mlp_forward(_ptr(_f32(params, (MLP_NPARAM,)), C.c_float),
                                      _ptr(_f32(norm, (MLP_NNORM,)), C.c_float), _ptr(rows, C.c_float), n,
                                      _ptr(y, C.c_float)))
    return y


def mlp_grad(params, norm, rows):
    """(mean squared normalised error, its gradient w.r.t. the parameters)."""
    L = load()
    rows = _f32(rows)
    g = np.empty(MLP_NPARAM, np.float32)
    loss = C.c_float()
    _mlp_check(L.cablegpu_mlp_grad(_ptr(_f32(params, (MLP_NPARAM,)), C.c_float),
                                   _ptr(_f32(norm, (MLP_NNORM,)), C.c_float), _ptr(rows, C.c_float),
                                   rows.shape[0], _ptr(g, C.c_float), C.byref(loss)))
    return float(loss.value), g


def mlp_fit(rows, nval, epochs=20, batch=65536, lr=1e-3, seed=1):
    """Trains a fresh network on rows[:-nval] (validation rows[-nval:]);
    returns (params, norm, losses [epochs][2] = train, validation MSE)."""
    L = load()
    rows = _f32(rows)
    ntrain = rows.shape[0] - nval
    p = np.empty(MLP_NPARAM, np.float32)
    nrm = np.empty(MLP_NNORM, np.float32)
    losses = np.empty((epochs, 2), np.float32)
    _mlp_check(L.cablegpu_mlp_fit(_ptr(rows, C.c_float), ntrain, nval, epochs, batch, lr, seed,
                                  _ptr(p, C.c_float), _ptr(nrm, C.c_float), _ptr(losses, C.c_float)))
    return p, nrm, losses


def mlp_unpack(params):
    """{W1, b1, W2, b2, W3, b3} views of a parameter vector."""
    p = np.asarray(params)
    return {"W1": p[0:768].reshape(64, 12), "b1": p[768:832], "W2": p[832:4928].reshape(64, 64),
            "b2": p[4928:4992], "W3": p[4992:5184].reshape(3, 64), "b3": p[5184:5187]}


def mlp_pack(d):
    return np.concatenate([np.ravel(d[k]) for k in ("W1", "b1", "W2", "b2", "W3", "b3")]).astype(np.float32)


class CableGPU:
    """One device context holding ``mp`` tiles (see module docstring)."""

    def __init__(self, tiles, device: int = 0, order: int = 0):
        """order: 0 grouped by plant and soil type, 1 as given, 2 grouped by
        plant type, local solar hour, latitude band and LAI, -1 autotuned."""
        self.L = load()
        self.fields = fields()
        self.mp = int(tiles.mp)
        self._keep = dict(
            iveg=np.ascontiguousarray(tiles.iveg, np.int32), isoilm=np.ascontiguousarray(tiles.isoilm, np.int32),
            vlai=np.ascontiguousarray(tiles.vlai, np.float32), lat=np.ascontiguousarray(tiles.lat, np.float32),
            lonphase=np.ascontiguousarray(tiles.lonphase, np.float32),
            tbase=np.ascontiguousarray(tiles.tbase, np.float32),
            swscale=np.ascontiguousarray(tiles.swscale, np.float32))
        t = self._tiles_struct(order)
        h = C.c_void_p()
        rc = self.L.cablegpu_create(C.byref(t), device, C.byref(h))
        self.h = h
        if rc != 0:
            msg = self.L.cablegpu_last_error(h).decode() if h.value else "invalid tile description"
            if h.value:
                self.L.cablegpu_destroy(h)
            self.h = C.c_void_p()
            raise CableGPUError(rc, msg)

    def _tiles_struct(self, order):
        k = self._keep
        return _Tiles(self.mp, _ptr(k["iveg"], C.c_int), _ptr(k["isoilm"], C.c_int), _ptr(k["vlai"], C.c_float),
                      _ptr(k["lat"], C.c_float), _ptr(k["lonphase"], C.c_float), _ptr(k["tbase"], C.c_float),
                      _ptr(k["swscale"], C.c_float), int(order))

    # ------------------------------------------------------------------ util
    def _check(self, rc):
        if rc != 0:
            raise CableGPUError(rc, self.L.cablegpu_last_error(self.h).decode())

    def close(self):
        if self.h and self.h.value:
            self.L.cablegpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------ setup
    def cold_start(self, snowd0, tgg0, wb0):
        a = [np.ascontiguousarray(x, np.float64) for x in (snowd0, tgg0, wb0)]
        self._check(self.L.cablegpu_cold_start(self.h, *[_ptr(x, C.c_double) for x in a]))

    def cold_start_noalloc(self, snowd0, tgg0, wb0):
        """cold_start through the allocation-free entry point (at most
        NOALLOC_MAX_TILES tiles; calls must not overlap)."""
        a = [np.ascontiguousarray(x, np.float64) for x in (snowd0, tgg0, wb0)]
        self._check(self.L.cablegpu_cold_start_noalloc(self.h, *[_ptr(x, C.c_double) for x in a]))

    def set_options(self, diag=False, capture_forcing=False, **switches):
        """Output options and the reference's science switches, by their
        ``cable_user`` names (see :func:`switch_mask`; unset = the offline
        defaults)."""
        self._check(self.L.cablegpu_set_options(self.h, switch_mask(**switches), int(diag), int(capture_forcing)))

    def set_soil_solve(self, mode):
        """Soil heat and moisture Thomas solves: SOLVE_FP64 (default, the
        reference's FP64 direct form) or SOLVE_FP32_CHANGE (FP32 on the
        step's change)."""
        if isinstance(mode, str):
            mode = {"fp64": SOLVE_FP64, "fp32_change": SOLVE_FP32_CHANGE}[mode]
        self._check(self.L.cablegpu_set_soil_solve(self.h, int(mode)))

    def set_canopy_schedule(self, mode):
        """Canopy dryLeaf passes: CANOPY_LANES (default) or CANOPY_POOL, or
        "lanes" / "pool"."""
        if isinstance(mode, str):
            mode = {"pool": CANOPY_POOL, "lanes": CANOPY_LANES}[mode]
        self._check(self.L.cablegpu_set_canopy_schedule(self.h, int(mode)))

    def check_tile_param(self, name, values):
        """Raises CableGPUError unless the per-tile parameter equals each
        tile's built-in per-type table value (cablegpu_check_tile_param)."""
        v = np.ascontiguousarray(values, np.float32)
        self._check(self.L.cablegpu_check_tile_param(self.h, name.encode(), _ptr(v, C.c_float)))

    def set_synthetic_forcing(self, seed: int, doy0: int = 1):
        self._check(self.L.cablegpu_set_synthetic_forcing(self.h, int(seed), int(doy0)))

    def set_forcing(self, forcing):
        f = np.ascontiguousarray(forcing, np.float32)
        assert f.shape == (NFORCING, self.mp)
        self._check(self.L.cablegpu_set_forcing(self.h, _ptr(f, C.c_float)))

    # ------------------------------------------------------------------ fields
    def get(self, name):
        fid, nl, dt, _ = self.fields[name]
        out = np.empty((nl, self.mp), _NP[dt])
        self._check(self.L.cablegpu_get_field(self.h, fid, out.ctypes.data_as(C.c_void_p)))
        return out

    def get_many(self, names):
        """Several fields in one call (cablegpu_get_fields): {name: array}."""
        outs = {n: np.empty((self.fields[n][1], self.mp), _NP[self.fields[n][2]]) for n in names}
        ids = (C.c_int * len(names))(*[self.fields[n][0] for n in names])
        ptrs = (C.c_void_p * len(names))(*[outs[n].ctypes.data for n in names])
        self._check(self.L.cablegpu_get_fields(self.h, len(names), ids, ptrs))
        return outs

    def set(self, name, value):
        fid, nl, dt, _ = self.fields[name]
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(value, _NP[dt]), (nl, self.mp)))
        self._check(self.L.cablegpu_set_field(self.h, fid, a.ctypes.data_as(C.c_void_p)))

    def outputs(self):
        o = self.get("out")
        return dict(zip(OUTPUT_FIELDS, o))

    def device_ptr(self, name):
        p, ld = C.c_void_p(), C.c_int()
        self._check(self.L.cablegpu_field_device_ptr(self.h, self.fields[name][0], C.byref(p), C.byref(ld)))
        return p.value, ld.value

    # ------------------------------------------------------------------ time
    def step(self, ktau: int, dels: float = 1800.0):
        self._check(self.L.cablegpu_step(self.h, int(ktau), float(dels)))

    def step_explicit(self, ktau: int, dels: float = 1800.0, lai_refresh: bool = True):
        """cbm_expl of the ACCESS coupling: radiation and canopy fluxes from
        the current state, which is left unchanged but for rtsoil, ga and
        (lai_refresh) the carried snow-reduced LAI."""
        self._check(self.L.cablegpu_step_explicit(self.h, int(ktau), float(dels), 1 if lai_refresh else 0))

    def step_implicit(self, ktau: int, dels: float = 1800.0, cycleno: int = 1, numcycles: int = 1):
        """cbm_impl of the ACCESS coupling; only the last of numcycles cycles
        advances the prognostic state."""
        self._check(self.L.cablegpu_step_implicit(self.h, int(ktau), float(dels), int(cycleno), int(numcycles)))

    def run(self, ktau0: int, nsteps: int, dels: float = 1800.0):
        self._check(self.L.cablegpu_run(self.h, int(ktau0), int(nsteps), float(dels)))

    def step_host(self, ktau, forcing, out, dels: float = 1800.0):
        """Pipelined step with host I/O: forcing [13][mp] float32 in, out
        [8][mp] float32 filled asynchronously (valid after synchronize())."""
        assert forcing.dtype == np.float32 and forcing.flags["C_CONTIGUOUS"] and forcing.shape == (NFORCING, self.mp)
        assert out.dtype == np.float32 and out.flags["C_CONTIGUOUS"] and out.shape == (8, self.mp)
        self._check(self.L.cablegpu_step_host(self.h, int(ktau), float(dels), _ptr(forcing, C.c_float),
                                              _ptr(out, C.c_float)))

    def host_register(self, a: np.ndarray):
        """Page-locks the memory of a C-contiguous array (cablegpu_host_register)."""
        assert a.flags["C_CONTIGUOUS"]
        self._check(self.L.cablegpu_host_register(a.ctypes.data, a.nbytes))

    def host_unregister(self, a: np.ndarray):
        self._check(self.L.cablegpu_host_unregister(a.ctypes.data))

    def synchronize(self):
        self._check(self.L.cablegpu_synchronize(self.h))

    def set_host_layout(self, layout: int):
        """0: step_host buffers in the caller's tile order; 1: in device order."""
        self._check(self.L.cablegpu_set_host_layout(self.h, int(layout)))

    def tile_order(self) -> np.ndarray:
        """The caller's index of the tile in each device slot."""
        o = np.empty(self.mp, np.int32)
        self._check(self.L.cablegpu_tile_order(self.h, _ptr(o, C.c_int)))
        return o

    # ------------------------------------------------------------------ files
    def restart_write(self, path, ktau: int):
        """Binary restart file of the state after step ``ktau``."""
        self._check(self.L.cablegpu_restart_write(self.h, os.fsencode(path), int(ktau)))

    def restart_read(self, path) -> int:
        """Loads a restart file's state; returns the step it was written after."""
        k = C.c_int()
        self._check(self.L.cablegpu_restart_read(self.h, os.fsencode(path), C.byref(k)))
        return k.value

    def run_forcing_file(self, forcing_path, ktau0: int, nsteps: int, record0: int = 0, output_path=None):
        """Steps ktau0.. on the records record0.. of a forcing file, with file
        reads and output writes overlapping the steps."""
        self._check(self.L.cablegpu_run_forcing_file(self.h, os.fsencode(forcing_path), int(record0), int(ktau0),
                                                     int(nsteps), os.fsencode(output_path) if output_path else None))

    def run_timed(self, ktau0, nsteps, dels=1800.0) -> float:
        ms = C.c_float()
        self._check(self.L.cablegpu_run_timed(self.h, int(ktau0), int(nsteps), float(dels), C.byref(ms)))
        return ms.value

    def coupled_timed(self, ktau0, nsteps, dels=1800.0, numcycles=2) -> float:
        """Milliseconds (CUDA events) of nsteps coupled timesteps: an explicit
        call and numcycles implicit cycles each."""
        ms = C.c_float()
        self._check(self.L.cablegpu_coupled_timed(self.h, int(ktau0), int(nsteps), float(dels), int(numcycles),
                                                  C.byref(ms)))
        return ms.value

    def kernel_timed(self, ktau0, nsteps, dels=1800.0) -> float:
        ms = C.c_float()
        self._check(self.L.cablegpu_kernel_timed(self.h, int(ktau0), int(nsteps), float(dels), C.byref(ms)))
        return ms.value

    def phase_timed(self, ktau0, nsteps, dels=1800.0) -> dict:
        """Average milliseconds of each kernel of a step, {phase: ms}."""
        ms = (C.c_float * len(PHASES))()
        self._check(self.L.cablegpu_phase_timed(self.h, int(ktau0), int(nsteps), float(dels), ms))
        return dict(zip(PHASES, [float(x) for x in ms]))

    # ---------------------------------------------------------- surrogate
    def harvest(self, ktau0, nsteps, prob, seed=7, capacity=None, dels=1800.0) -> int:
        """Runs nsteps plain steps that record dryLeaf training rows; returns
        the number of rows filled."""
        if capacity is None:
            capacity = max(1024, int(self.mp * nsteps * 4 * prob * 1.3) + 1024)
        n = C.c_longlong()
        self._check(self.L.cablegpu_harvest(self.h, int(ktau0), int(nsteps), float(dels), float(prob), int(seed),
                                            int(capacity), C.byref(n)))
        return int(n.value)

    def harvest_rows(self, n):
        out = np.empty((int(n), MLP_ROW), np.float32)
        self._check(self.L.cablegpu_harvest_rows(self.h, _ptr(out, C.c_float), int(n)))
        return out

    def surrogate_train(self, epochs=20, batch=65536, lr=1e-3, val_frac=0.1, seed=1):
        losses = np.zeros((epochs, 2), np.float32)
        self._check(self.L.cablegpu_surrogate_train(self.h, int(epochs), int(batch), float(lr), float(val_frac),
                                                    int(seed), _ptr(losses, C.c_float)))
        return losses

    def surrogate_weights(self, params=None, norm=None):
        """Returns (params, norm); sets them first when given."""
        if params is not None:
            p, n = _f32(params, (MLP_NPARAM,)), _f32(norm, (MLP_NNORM,))
            self._check(self.L.cablegpu_surrogate_weights(self.h, _ptr(p, C.c_float), _ptr(n, C.c_float), 1))
            return p, n
        p = np.empty(MLP_NPARAM, np.float32)
        n = np.empty(MLP_NNORM, np.float32)
        self._check(self.L.cablegpu_surrogate_weights(self.h, _ptr(p, C.c_float), _ptr(n, C.c_float), 0))
        return p, n

    def set_surrogate(self, mode=1, gate=0.1):
        """mode 0 off, 1 strict (unclosed predictions restart the plain
        iteration), 2 warm (the iteration continues from the prediction)."""
        self._check(self.L.cablegpu_set_surrogate(self.h, int(mode), float(gate)))

    def surrogate_stats(self, reset=False):
        tried, acc = C.c_longlong(), C.c_longlong()
        self._check(self.L.cablegpu_surrogate_stats(self.h, C.byref(tried), C.byref(acc), int(reset)))
        return int(tried.value), int(acc.value)

    def tune_blocks(self, ktau0=1, nsteps=4, dels=1800.0):
        """Times block sizes 32..256 of each step kernel on this context's own
        tiles and state (restored afterwards), keeps the fastest; returns
        (blocks, ms per step)."""
        b = (C.c_int * 5)()
        ms = C.c_float()
        self._check(self.L.cablegpu_tune_blocks(self.h, int(ktau0), int(nsteps), float(dels), b, C.byref(ms)))
        return list(b), ms.value

    def set_blocks(self, blocks):
        b = (C.c_int * 5)(*[int(x) for x in blocks])
        self._check(self.L.cablegpu_set_blocks(self.h, b))

    def config(self):
        """(tile order, [block size of the five step kernels])"""
        o = C.c_int()
        b = (C.c_int * 5)()
        self._check(self.L.cablegpu_get_config(self.h, C.byref(o), b))
        return int(o.value), list(b)

    def launch_count(self) -> int:
        return int(self.L.cablegpu_launch_count(self.h))


def autotune(ts, device: int = 0, sample_tiles: int = 262144, nsteps: int = 8):
    """(best tile order, [block sizes], sample ms/step) for a TileSet."""
    g = object.__new__(CableGPU)
    g.L = load()
    g.mp = int(ts.mp)
    g._keep = dict(
        iveg=np.ascontiguousarray(ts.iveg, np.int32), isoilm=np.ascontiguousarray(ts.isoilm, np.int32),
        vlai=np.ascontiguousarray(ts.vlai, np.float32), lat=np.ascontiguousarray(ts.lat, np.float32),
        lonphase=np.ascontiguousarray(ts.lonphase, np.float32), tbase=np.ascontiguousarray(ts.tbase, np.float32),
        swscale=np.ascontiguousarray(ts.swscale, np.float32))
    t = g._tiles_struct(0)
    o, ms = C.c_int(), C.c_float()
    b = (C.c_int * 5)()
    rc = g.L.cablegpu_autotune(C.byref(t), device, int(sample_tiles), int(nsteps), C.byref(o), b, C.byref(ms))
    if rc != 0:
        raise CableGPUError(rc, "autotune failed")
    return int(o.value), list(b), float(ms.value)


class HostBlock:
    """Page-locked host memory from cablegpu_host_alloc (the CUDA driver's
    pinned allocator), carved into arrays for cablegpu_step_host's forcing
    and output buffers.
    ``HostBlock([(13, mp), (8, mp)])`` -> ``.arrays``; ``free()`` releases it
    (the arrays must not be used after)."""

    ALIGN = 1 << 16

    def __init__(self, shapes, dtype=np.float32):
        L = load()
        dt = np.dtype(dtype)
        counts = [int(np.prod(sh)) for sh in shapes]
        offs, tot = [], 0
        for n in counts:
            offs.append(tot)
            tot += -(-n * dt.itemsize // self.ALIGN) * self.ALIGN
        p = C.c_void_p()
        rc = L.cablegpu_host_alloc(C.c_size_t(max(tot, 1)), C.byref(p))
        if rc != 0:
            raise CableGPUError(rc, "host_alloc of %d bytes failed" % tot)
        self.L, self.ptr, self.nbytes = L, p.value, tot
        self.arrays = [np.ctypeslib.as_array((C.c_byte * (n * dt.itemsize)).from_address(self.ptr + o))
                       .view(dt).reshape(sh) for o, n, sh in zip(offs, counts, shapes)]

    def free(self):
        if self.ptr:
            self.arrays = []
            rc = self.L.cablegpu_host_free(C.c_void_p(self.ptr))
            self.ptr = None
            if rc != 0:
                raise CableGPUError(rc, "host_free failed")


def from_tileset(ts, device: int = 0, seed=None, order: int = 0) -> CableGPU:
    """Context for a :class:`cable_gb300.workloads.TileSet`, cold-started and
    driven by the built-in synthetic forcing."""
    g = CableGPU(ts, device, order)
    g.cold_start(ts.snowd0, ts.tgg0, ts.wb0)
    g.set_synthetic_forcing(ts.seed if seed is None else seed, ts.doy0)
    return g
