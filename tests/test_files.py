"""Binary restart / forcing / output files: the container written by the
library (host code, no GPU needed) against the numpy reader, and the error
paths of a damaged file."""
import os

import numpy as np
import pytest

from cable_gb300 import cgfile
from cable_gb300 import runtime as R


def test_forcing_file_layout_matches_the_reader(tmp_path):
    rng = np.random.default_rng(3)
    mp, n = 1000, 5
    F = rng.standard_normal((n, R.NFORCING, mp)).astype(np.float32)
    p = str(tmp_path / "met.cgf")
    R.forcing_file_write(p, F, doy0=32, dels=1800.0)
    info = R.file_info(p)
    assert info == {"kind": 2, "mp": mp, "nrecords": n, "nfields": 1, "ktau": 1, "doy0": 32, "dels": 1800.0}
    f = cgfile.read(p)
    assert f.kind == "forcing" and f.fields == {"met": (cgfile.F32, R.NFORCING, 0)}
    rb = f.header["record_bytes"]
    assert rb % 4096 == 0 and rb >= 4 * R.NFORCING * mp
    assert os.path.getsize(p) == cgfile.DATA_OFFSET + n * rb
    for k in range(n):
        np.testing.assert_array_equal(f.read("met", k), F[k])


def test_damaged_files_are_rejected(tmp_path):
    mp, n = 64, 3
    F = np.ones((n, R.NFORCING, mp), np.float32)
    p = str(tmp_path / "met.cgf")
    R.forcing_file_write(p, F)
    raw = open(p, "rb").read()
    bad = tmp_path / "bad_magic.cgf"
    bad.write_bytes(b"XABLEGPU" + raw[8:])
    short = tmp_path / "truncated.cgf"
    short.write_bytes(raw[:-100])
    for q in (bad, short, tmp_path / "missing.cgf"):
        with pytest.raises(R.CableGPUError) as e:
            R.file_info(str(q))
        assert e.value.code == -5
    with pytest.raises(ValueError):
        cgfile.read(str(bad))
    with pytest.raises(ValueError):
        cgfile.read(str(short))
    # bad arguments of the writer
    L = R.load()
    assert L.cablegpu_forcing_file_write(p.encode(), 0, 1, 1, 1800.0, None) == -1
