"""Binary restart and forcing files on the GPU: a run resumed from a restart
file is bitwise the uninterrupted run, and a run driven from a forcing file
(reader and writer threads overlapping the steps) is bitwise the run driven
step by step from the same forcing in host memory, outputs included."""
import numpy as np
import pytest

import oracle_lib as O
from cable_gb300 import cgfile
from cable_gb300 import workloads as W

pytestmark = pytest.mark.gpu

STATE = ["wb", "wbice", "gammzz1", "tgg", "tggsn", "ssdn", "smass", "sdepth", "flags", "snowd", "ssdnn", "snage",
         "pudsto", "owetfac", "rtsoil", "tss", "wb_lake", "wbtot1", "wbtot2", "cansto", "cplant", "csoil", "owb",
         "ebal_tot", "wbal_tot"]


@pytest.fixture(scope="module")
def runtime():
    from cable_gb300 import runtime as R
    R.load()
    return R


@pytest.mark.parametrize("switches", [{}, {"ssnow_potev": "P-M", "litter": True}])
def test_restart_file_resumes_bitwise(runtime, tmp_path, switches):
    """Also with Penman-Monteith soil evaporation, which reads the last
    step's canopy%ga: the restart file carries the output rows."""
    R = runtime
    ts = W.snow_grid(6000, nsteps=48)
    path = str(tmp_path / "restart.cgf")
    a = R.from_tileset(ts)
    a.set_options(**switches)
    a.run(1, 24)
    a.restart_write(path, 24)
    a.run(25, 24)
    a.synchronize()
    sa = {k: a.get(k) for k in STATE}
    out_a = a.get("out")
    a.close()
    b = R.from_tileset(ts)
    b.set_options(**switches)
    assert b.restart_read(path) == 24
    b.run(25, 24)
    b.synchronize()
    for k in STATE:
        np.testing.assert_array_equal(b.get(k), sa[k], err_msg=k)
    np.testing.assert_array_equal(b.get("out"), out_a)
    b.close()
    # the file: tile description plus state, the soil water as exact word pairs
    f = cgfile.read(path)
    assert f.kind == "restart" and f.header["ktau"] == 24 and f.mp == ts.mp and "out" in f.fields
    assert f.fields["wb"][0] == cgfile.DF32 and f.fields["tgg"][:2] == (cgfile.F32, 6)
    np.testing.assert_array_equal(f.read("iveg")[0], ts.iveg)
    hi, lo = f.read_pairs("wb")
    assert np.all(np.abs(lo) <= np.abs(hi) * 2.0 ** -23)
    # a restart of other tiles is refused
    other = W.snow_grid(6000, seed=7, nsteps=48)
    c = R.from_tileset(other)
    with pytest.raises(R.CableGPUError) as e:
        c.restart_read(path)
    assert e.value.code == -1
    c.close()


def test_forcing_file_run_matches_host_forcing(runtime, tmp_path):
    R = runtime
    ts = W.snow_grid(5000, nsteps=20)
    n = 20
    F = O.forcing(ts, 0, n)
    fpath, opath = str(tmp_path / "met.cgf"), str(tmp_path / "out.cgf")
    R.forcing_file_write(fpath, F, doy0=ts.doy0, dels=ts.dels)
    a = R.from_tileset(ts)
    a.run_forcing_file(fpath, ktau0=1, nsteps=n, output_path=opath)
    sa = {k: a.get(k) for k in STATE}
    a.close()
    b = R.from_tileset(ts)
    outs = []
    for k in range(n):
        b.set_forcing(F[k])
        b.step(k + 1, ts.dels)
        outs.append(b.get("out"))
    b.synchronize()
    for k in STATE:
        np.testing.assert_array_equal(b.get(k), sa[k], err_msg=k)
    b.close()
    o = cgfile.read(opath)
    assert o.kind == "output" and o.header["nrecords"] == n and o.header["ktau"] == 1
    for k in range(n):
        np.testing.assert_array_equal(o.read("out", k), outs[k], err_msg="output record %d" % k)
    # a window of the file: records 10.. continue a run restarted at step 10
    c = R.from_tileset(ts)
    for k in range(10):
        c.set_forcing(F[k])
        c.step(k + 1, ts.dels)
    c.run_forcing_file(fpath, ktau0=11, nsteps=n - 10, record0=10)
    for k in ("wb", "tgg", "snowd", "cansto"):
        np.testing.assert_array_equal(c.get(k), sa[k], err_msg=k)
    with pytest.raises(R.CableGPUError):
        c.run_forcing_file(fpath, ktau0=21, nsteps=5, record0=18)   # past the end of the file
    c.close()
