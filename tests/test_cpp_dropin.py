"""The C++ drop-in layer (include/quantit_gb300.hpp) compiled with g++ against
libqtt_gb300.so: structure cases and QuantiT's exception types on the CPU; contraction,
SVD and both dmrg overloads (with loggers) on the GPU, the DMRG energy checked
against exact diagonalisation of the L = 8 Heisenberg chain."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "quantit_gb300")


@pytest.fixture(scope="module")
def binary(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ is not installed")
    if not os.path.exists(os.path.join(LIBDIR, "libqtt_gb300.so")):
        pytest.fail("libqtt_gb300.so is missing: build it with `python -m quantit_gb300.build`")
    out = str(tmp_path_factory.mktemp("cpp") / "test_dropin")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"), "-L", LIBDIR, "-lqtt_gb300",
           "-Wl,-rpath," + LIBDIR, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "warning" not in r.stderr, r.stderr
    return out


def test_structure_and_exceptions(binary):
    r = subprocess.run([binary, "structure"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "structure: 0 failure(s)" in r.stdout


@pytest.mark.gpu
def test_numeric_and_dmrg(binary):
    r = subprocess.run([binary, "numeric"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [x for x in r.stdout.splitlines() if x.startswith("ENERGY")][0]
    e1, e2 = (float(v) for v in line.split()[1:])
    L = 8
    sx = np.array([[0, .5], [.5, 0]])
    sy = np.array([[0, -.5j], [.5j, 0]])
    sz = np.diag([.5, -.5])

    def op(a, i):
        m = np.eye(1)
        for j in range(L):
            m = np.kron(m, a if j == i else np.eye(2))
        return m
    H = sum((op(sx, i) @ op(sx, i + 1) + op(sy, i) @ op(sy, i + 1) + op(sz, i) @ op(sz, i + 1)).real
            for i in range(L - 1))
    e0 = np.linalg.eigvalsh(H)[0]
    assert e1 == pytest.approx(e0, abs=1e-9)
    assert e2 == pytest.approx(e0, abs=1e-9)
