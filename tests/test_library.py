"""The C-ABI library (no GPU needed): build, exported symbols, field
registry, parameter tables against the oracle's copy, argument validation."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from cable_gb300 import build as B
from cable_gb300 import runtime as R
from cable_gb300 import workloads as W

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "cablegpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(cablegpu_\w+)\s*\(", txt)))


def test_library_builds_and_exports_every_declared_symbol():
    lib = C.CDLL(B.build())
    syms = declared_symbols()
    assert len(syms) >= 19
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(R.EXPORTS)   # the Python binding lists exactly the declared entry points


def test_binding_constants_match_the_header():
    """Values the Python binding copies from include/cablegpu.h: a change to
    the header must not leave the binding (and the tests built on it)
    checking a stale value."""
    txt = open(HEADER).read()
    defs = dict(re.findall(r"#define\s+(CABLEGPU_\w+)\s+\(?(-?\d+)\)?", txt))
    assert int(defs["CABLEGPU_NOALLOC_MAX_TILES"]) == R.NOALLOC_MAX_TILES
    assert int(defs["CABLEGPU_MAX_TILES"]) == R.MAX_TILES
    assert int(defs["CABLEGPU_NFORCING"]) == R.NFORCING
    for name in ("MEDLYN", "SOIL_THERMAL_FIX", "LITTER", "L_REV_CORR", "FWSOIL_NONLINEAR", "FWSOIL_LAI_KTAUL",
                 "POTEV_PM", "NEW_REDUCE_SOILEVP", "NEW_RUNOFF_SPEED", "DIAG_SOIL_RESP_OFF"):
        assert int(defs["CABLEGPU_SW_" + name]) == getattr(R, "SW_" + name), name
    for name in ("NONFINITE", "DRYLEAF_NOCONV", "FORCING_RANGE", "OUTPUT_RANGE", "EVAPFBL"):
        assert int(defs["CABLEGPU_TILE_" + name]) == getattr(R, "TILE_" + name), name
    for code, name in R.ERRORS.items():
        assert int(defs[name]) == code, name


def test_field_registry_is_consistent():
    f = R.fields()
    assert len(f) == R.load().cablegpu_num_fields()
    for name in ("wb", "wbice", "tgg", "tggsn", "ssdn", "smass", "sdepth", "snowd", "cansto", "out", "forcing_in"):
        assert name in f
    assert f["wb"][1] == 6 and f["wb"][2] == R.F64
    assert f["tggsn"][1] == 3 and f["out"][1] == 8
    assert f["forcing_in"][1] == R.NFORCING
    ids = sorted(v[0] for v in f.values())
    assert ids == list(range(len(f)))
    assert R.load().cablegpu_field_id(b"no_such_field") < 0


def test_create_rejects_bad_tiles_without_a_gpu():
    """Argument validation happens before any CUDA call."""
    ts = W.grid(16)
    ts.iveg = ts.iveg.copy()
    ts.iveg[3] = 18
    with pytest.raises(R.CableGPUError) as e:
        R.CableGPU(ts)
    assert e.value.code == -1
    ts.iveg[3] = 5
    ts.isoilm = ts.isoilm.copy()
    ts.isoilm[0] = 0
    with pytest.raises(R.CableGPUError):
        R.CableGPU(ts)
    # more tiles than 32-bit row offsets address: refused before the arrays
    # are read (these hold 16 tiles) and before any CUDA call
    ts.isoilm[0] = 1
    L = R.load()
    t = R._Tiles(R.MAX_TILES + 1, ts.iveg.ctypes.data_as(C.POINTER(C.c_int)),
                 ts.isoilm.ctypes.data_as(C.POINTER(C.c_int)), ts.vlai.ctypes.data_as(C.POINTER(C.c_float)),
                 ts.lat.ctypes.data_as(C.POINTER(C.c_float)), None, None, None, 0)
    h = C.c_void_p()
    assert L.cablegpu_create(C.byref(t), 0, C.byref(h)) == -1 and not h.value
    # and an empty or negative tile count
    for mp in (0, -5):
        t.mp = mp
        assert L.cablegpu_create(C.byref(t), 0, C.byref(h)) == -1 and not h.value


def test_host_alloc_arguments_and_failure_leave_nothing_behind():
    """cablegpu_host_alloc refuses zero bytes and a null out; without a GPU
    its registration fails and it returns CABLEGPU_ERR_CUDA with the mapping
    undone and *out null; cablegpu_host_free refuses unknown addresses."""
    L = R.load()
    p = C.c_void_p()
    assert L.cablegpu_host_alloc(C.c_size_t(0), C.byref(p)) == -1 and not p.value
    assert L.cablegpu_host_alloc(C.c_size_t(4096), None) == -1
    buf = np.zeros(16, np.float32)
    assert L.cablegpu_host_free(C.c_void_p(buf.ctypes.data)) == -1
    assert L.cablegpu_host_free(None) == -1
    import torch
    if not torch.cuda.is_available():
        assert L.cablegpu_host_alloc(C.c_size_t(1 << 20), C.byref(p)) == -2 and not p.value


def test_null_arguments_are_errors():
    L = R.load()
    assert L.cablegpu_create(None, 0, None) == -1
    assert L.cablegpu_step(None, 1, C.c_float(1800.0)) == -1
    assert L.cablegpu_destroy(None) == -1
    assert L.cablegpu_field_info(10 ** 6, None, None, None, None) == -1


def test_parameter_tables_match_the_oracle(oracle):
    """The product's derived per-type tables equal the oracle's restatement."""
    L = R.load()
    buf = (C.c_float * 17)()
    for name in ("vcmax", "a1gs", "hc", "frac4", "xfang", "rp20", "vegcf", "g1", "refl1", "taul2"):
        assert L.cablegpu_param_table(0, name.encode(), buf, 17) == 0
        ref = [oracle.lib().cbmref_pft_value(name.encode(), v) for v in range(1, 18)]
        np.testing.assert_allclose(np.frombuffer(buf, np.float32), np.float32(ref), rtol=1e-7)
    sbuf = (C.c_float * 9)()
    for name in ("bch", "ssat", "sfc", "swilt", "hyds", "css", "rhosoil"):
        assert L.cablegpu_param_table(1, name.encode(), sbuf, 9) == 0
        ref = [oracle.lib().cbmref_soil_value(name.encode(), s) for s in range(1, 10)]
        np.testing.assert_allclose(np.frombuffer(sbuf, np.float32), np.float32(ref), rtol=1e-7)
    # derived: root fractions and leaf width
    fr = (C.c_float * (6 * 17))()
    assert L.cablegpu_param_table(0, b"froot", fr, 6 * 17) == 0
    fr = np.frombuffer(fr, np.float32).reshape(6, 17)
    dl = (C.c_float * 17)()
    assert L.cablegpu_param_table(0, b"dleaf", dl, 17) == 0
    dp = lambda: C.c_double()
    for v in range(1, 18):
        f6 = (C.c_double * 6)(); a, b_, c_ = dp(), dp(), dp()
        oracle.lib().cbmref_params(v, 1, f6, C.byref(a), C.byref(b_), C.byref(c_))
        np.testing.assert_allclose(fr[:, v - 1], np.array(f6[:]), rtol=2e-6, atol=1e-7)
        assert np.frombuffer(dl, np.float32)[v - 1] == pytest.approx(a.value, rel=1e-6)
    assert abs(fr.sum(0) - 1).max() < 1e-5


FORTRAN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cable_gb300", "fortran")
SHIM = os.path.join(FORTRAN, "cable_cbm_gpu.F90")
COUPLED_SHIM = os.path.join(FORTRAN, "cable_cbm_coupled_gpu.F90")
SHIM_FILES = [os.path.join(FORTRAN, n) for n in ("cablegpu_c.F90", "cablegpu_shim.F90", "cable_cbm_gpu.F90",
                                                  "cable_cbm_coupled_gpu.F90")]


def test_fortran_shim_binds_exported_symbols_and_registry_fields():
    """No Fortran compiler is available, so the ISO_C_BINDING shim is checked
    textually: every BIND(C) name is an exported symbol declared in the
    header, every field it moves is in the registry with the width and type
    the shim's buffer assumes, and the forcing order matches the ABI's."""
    src = "\n".join(open(f).read() for f in SHIM_FILES)
    lib = C.CDLL(B.build())
    binds = re.findall(r'BIND\(C,\s*name="(\w+)"\)', src)
    assert len(binds) >= 10
    declared = set(declared_symbols())
    for b in binds:
        assert b in declared and hasattr(lib, b), b
    f = R.fields()
    used = set(re.findall(r"CALL (?:put|get)\('(\w+)'", src))
    assert used, "no field transfers found"
    missing = used - set(f)
    assert not missing, missing
    # buffers the shim uses: r8 (REAL(c_double)) for F64, r4 for F32, flags for I32
    for name in used:
        dt = f[name][2]
        m = re.search(r"CALL (?:put|get)\('%s', C_LOC\((\w+)\)\)" % name, src)
        buf = m.group(1)
        want = {R.F64: ("r8",), R.F32: ("r4", "outb"), R.I32: ("flags",)}[dt]
        assert buf in want, (name, buf, want)
    # forcing gathered into device order through the slot -> tile index, the
    # outputs scattered back through it
    src = open(SHIM).read() + open(SHIM_FILES[1]).read()
    order = re.findall(r"forc\(:, (\d+)\) = met%(\w+)\(slot_tile(?:, (\d))?\)", src)
    names = []
    for idx, comp, band in order:
        names.append("fsd_" + ("vis" if band == "1" else "nir") if comp == "fsd" else comp)
    assert names == R.FORCING_FIELDS
    assert [int(o[0]) for o in order] == list(range(1, R.NFORCING + 1))
    outs = re.findall(r"(?:canopy|rad)%(\w+)\(slot_tile\) = outb\(:, (\d)\)", src)
    assert [o[0] for o in sorted(outs, key=lambda x: int(x[1]))] == R.OUTPUT_FIELDS
    assert "cablegpu_set_host_layout(ctx, 1_c_int)" in src and "cablegpu_tile_order(ctx, C_LOC(slot_tile))" in src


def test_coupled_fortran_shim_matches_the_cm3_interface():
    """The ACCESS (CM3) replacement of cable_cbm_module: cbm_expl and cbm_impl
    with the reference's argument lists (cbl_cbm_mod.F90:10-11, :184-186),
    the forcing in the ABI's field order, the eight outputs back into their
    components, and the two coupled entry points."""
    src = open(COUPLED_SHIM).read()
    assert re.search(r"^MODULE cable_cbm_module", src, re.M)
    assert re.search(r"PUBLIC cbm_expl, cbm_impl", src)

    def args(name):
        m = re.search(r"SUBROUTINE %s\(([^)]*)\)" % name, src, re.S)
        return [a.strip() for a in m.group(1).replace("&", "").split(",")]

    tail = ["air", "bgc", "canopy", "met", "bal", "rad", "rough", "soil", "ssnow", "sum_flux", "veg", "climate"]
    assert args("cbm_expl") == ["mp", "nrb", "ktau", "dels"] + tail
    assert args("cbm_impl") == ["cycleno", "numcycles", "mp", "nrb", "ktau", "dels"] + tail
    order = re.findall(r"forc\(:, (\d+)\) = met%(\w+)(?:\(:, (\d)\))?", src)
    names = ["fsd_" + ("vis" if band == "1" else "nir") if comp == "fsd" else comp for _, comp, band in order]
    assert names == R.FORCING_FIELDS
    assert [int(o[0]) for o in order] == list(range(1, R.NFORCING + 1))
    outs = re.findall(r"(?:canopy|rad)%(\w+) = outb\(:, (\d)\)", src)
    assert [o[0] for o in sorted(outs, key=lambda x: int(x[1]))] == R.OUTPUT_FIELDS
    assert "cablegpu_step_explicit(ctx" in src and "cablegpu_step_implicit(ctx" in src
    assert "CALL put('vlaiw', C_LOC(r4))" in src and R.fields()["vlaiw"][2] == R.F32


def test_soil_thermal_fix_tables_match_the_oracle(oracle):
    """The soil_thermal_fix parameter set (css, rhosoil, dry conductivity and
    the saturated-conductivity factor of total_soil_conductivity) equals the
    oracle's restatement of cable_parameters.F90:2165-2227 and
    cbl_conductivity.F90:36-43; table 1 keeps the default values."""
    L = R.load()
    got = {}
    for name in ("css", "rhosoil", "cnsd", "cnsdv", "ktmp"):
        b = (C.c_float * 9)()
        assert L.cablegpu_param_table(2, name.encode(), b, 9) == 0
        got[name] = np.frombuffer(b, np.float32).copy()
    d = [C.c_double() for _ in range(4)]
    for s in range(1, 10):
        assert oracle.lib().cbmref_soil_thermal_fix(s, *[C.byref(x) for x in d]) == 0
        css, rho, cnsdv, ktmp = (x.value for x in d)
        assert got["css"][s - 1] == pytest.approx(css, rel=1e-6)
        assert got["rhosoil"][s - 1] == pytest.approx(rho, rel=1e-6)
        assert got["cnsdv"][s - 1] == pytest.approx(cnsdv, rel=1e-6)
        assert got["cnsd"][s - 1] == got["cnsdv"][s - 1]
        assert got["ktmp"][s - 1] == pytest.approx(ktmp, rel=1e-6)
    # rhosoil / (1 - ssat) for the table's first soil (1600 kg/m3, ssat .398)
    assert got["rhosoil"][0] == pytest.approx(1600.0 / (1 - 0.398), rel=1e-6)
    b = (C.c_float * 9)()
    assert L.cablegpu_param_table(1, b"css", b, 9) == 0
    assert np.frombuffer(b, np.float32)[0] == 850.0


def test_phase_launchers_are_not_merged_across_translation_units():
    """Each phase translation unit launches its own kernel: a launch helper
    with external (weak) linkage and the same name in several units would be
    merged by the linker into one, so every phase would launch the same
    kernel.  The helpers must have internal linkage."""
    import shutil
    import subprocess
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-C", B.build()], capture_output=True, text=True, check=True).stdout
    weak = [ln for ln in out.splitlines() if re.search(r"\s[WVuw]\s", ln) and "cg::" in ln and "launch" in ln.lower()]
    assert not weak, weak[:5]
