"""The C++ drop-in header (include/nrgcore_gpu.hpp) used the way the
reference's drivers use nrgcore: a driver written like
examples/entropyKondo/main.cpp (tests/cpp/shim_kondo.cpp), with models that
follow the reference's model concept, built with g++ against libnrggpu.so."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden
from parity import check_eigs
from nrgplusplus_gb300 import models as M
from nrgplusplus_gb300 import workloads

SRC = os.path.join(ROOT, "tests", "cpp", "shim_kondo.cpp")


def _gxx():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    return gxx


def _write_models(path, imp, bath, temps):
    with open(path, "wb") as f:
        for site in (imp, bath):
            nq = len(site.qnums[0])
            f.write(struct.pack("<ii", nq, len(site.qnums)))
            for q in site.qnums:
                f.write(struct.pack("<%di" % nq, *q))
            for e in site.energies:
                f.write(struct.pack("<i", len(e)))
                f.write(np.asarray(e, "<f8").tobytes())
            f.write(np.asarray(site.chi, "<f8").tobytes())
            f.write(struct.pack("<i", len(site.fdag)))
            for op in site.fdag:
                f.write(struct.pack("<i", len(op)))
                for (i, j), m in sorted(op.items()):
                    m = np.ascontiguousarray(m, "<f8")
                    f.write(struct.pack("<iiii", i, j, m.shape[0], m.shape[1]))
                    f.write(m.tobytes())
        f.write(struct.pack("<i", len(temps)))
        f.write(np.asarray(temps, "<f8").tobytes())


def test_shim_header_compiles(tmp_path):
    gxx = _gxx()
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Wextra", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_shim_kondo_against_shipped_fixture(tmp_path):
    from nrgplusplus_gb300.build import build
    lib = build(verbose=False)
    gxx = _gxx()
    exe = str(tmp_path / "shim_kondo")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    imp, bath = M.spinhalf_kondo(0.25, 0.5), M.spinhalf(0.0, 0.0)
    models = str(tmp_path / "models.bin")
    _write_models(models, imp, bath, workloads.temperature_grid())
    out = str(tmp_path / "out.bin")
    r = subprocess.run([exe, models, out, "1", "41", "2.0", "1024"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    with open(out, "rb") as f:
        n = struct.unpack("<i", f.read(4))[0]
        eigs = []
        for _ in range(n):
            m = struct.unpack("<i", f.read(4))[0]
            eigs.append(np.frombuffer(f.read(8 * m), "<f8"))
        ns = struct.unpack("<i", f.read(4))[0]
        entropy = np.frombuffer(f.read(8 * ns), "<f8")
    fx = golden("shipped_kondo_J0.25")
    assert n == 41
    check_eigs(fx, eigs, 2.0)
    assert np.abs(entropy - fx["entropy"]).max() < 1e-8
