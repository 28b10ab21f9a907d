"""The soil solver's FP64 arithmetic on the GPU: its reciprocal (rcp64 in
cbm_physics.cuh: two fused multiply-adds from the FP32 reciprocal) against CUDA's FP64
division, within 2 units in the last place and a relative error below
4.5e-16 on 2^22 values over 1e-20..1e20 and over the soil systems' pivot
range; and its Thomas elimination (trimb64, reciprocals seeded from the
pivots' FP32 shadow) against the same elimination in long double on the
host, on 2^18 six-row and 2^18 nine-row systems shaped like the soil heat
and moisture systems: its largest error (relative to each system's largest
value) at most twice that of the host's double elimination with IEEE
division, the reference's arithmetic; and its FP32 <-> FP64 conversions on
the integer pipe (f2d, d2f), bit for bit equal to the hardware conversion
instructions on 2^23 inputs of every class."""
import os
import subprocess
import tempfile

import pytest

from cable_gb300 import build as B

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_rcp64_matches_cuda_fp64_division():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "fp64_reciprocal")
        subprocess.run([B._nvcc(), "-O3", "-std=c++17"] + B.ARCH + ["-I", B.CSRC,
                        os.path.join(HERE, "kernels", "fp64_reciprocal.cu"), "-o", exe], check=True)
        r = subprocess.run([exe, "2", "4.5e-16"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_trimb64_matches_long_double_elimination():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "fp64_thomas")
        subprocess.run([B._nvcc(), "-O3", "-std=c++17"] + B.ARCH + ["-I", B.CSRC,
                        os.path.join(HERE, "kernels", "fp64_thomas.cu"), "-o", exe], check=True)
        r = subprocess.run([exe, "2.0"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_integer_pipe_conversions_equal_the_hardware_conversions():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "fp64_convert")
        subprocess.run([B._nvcc(), "-O3", "-std=c++17"] + B.ARCH + ["-I", B.CSRC,
                        os.path.join(HERE, "kernels", "fp64_convert.cu"), "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
