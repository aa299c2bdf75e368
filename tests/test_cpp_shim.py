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
SRC_SIAM = os.path.join(ROOT, "tests", "cpp", "shim_entropy_siam.cpp")


def _gxx():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    return gxx


def _write_ops(f, ops):
    f.write(struct.pack("<i", len(ops)))
    for op in ops:
        f.write(struct.pack("<i", len(op)))
        for (i, j), m in sorted(op.items()):
            m = np.ascontiguousarray(m, "<f8")
            f.write(struct.pack("<iiii", i, j, m.shape[0], m.shape[1]))
            f.write(m.tobytes())


def _write_models(path, imp, bath, temps, extra_ops=None):
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
            _write_ops(f, site.fdag)
        if extra_ops is not None:
            _write_ops(f, extra_ops)
        f.write(struct.pack("<i", len(temps)))
        f.write(np.asarray(temps, "<f8").tobytes())


@pytest.mark.parametrize("src", [SRC, SRC_SIAM])
def test_shim_header_compiles(tmp_path, src):
    gxx = _gxx()
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Wextra", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        src], capture_output=True, text=True)
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


def _read_vecs(path):
    with open(path, "rb") as f:
        b = f.read()
    p, out = 0, []
    n = struct.unpack_from("<i", b, p)[0]
    p += 4
    eigs = []
    for _ in range(n):
        m = struct.unpack_from("<i", b, p)[0]
        p += 4
        eigs.append(np.frombuffer(b, "<f8", m, p))
        p += 8 * m
    while p < len(b):
        m = struct.unpack_from("<i", b, p)[0]
        p += 4
        out.append(np.frombuffer(b, "<f8", m, p))
        p += 8 * m
    return eigs, out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_shim_entropy_siam_driver(tmp_path, precision):
    """The entropySIAM-form driver: reference constructor nrgcore(imp, bath),
    update_system_operator(&siam, nd) with the rotated blocks copied back,
    `siam.nrg_iterations_cnt--; rawData.loadCurrentData();`, class template
    argument deduction for NrgData / fdmThermodynamics, setSystemOperator;
    eigenvalues, entropy and <n_d>(T) against the reference's own output."""
    from nrgplusplus_gb300.build import build
    from oracle.nrg_oracle import siam_run
    lib = build(verbose=False)
    gxx = _gxx()
    exe = str(tmp_path / "shim_entropy_siam")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC_SIAM, lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    imp, bath = M.spinhalf(-0.25, 0.8), M.spinhalf(0.0, 0.0)
    models = str(tmp_path / "models.bin")
    _write_models(models, imp, bath, workloads.temperature_grid(), extra_ops=M.n_d())
    out = str(tmp_path / "out.bin")
    env = dict(os.environ, NRG_GPU_PRECISION=precision)
    r = subprocess.run([exe, models, out, "30", "2.0", "256", "0.15"], capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr
    eigs, (entropy, nd, extra) = _read_vecs(out)
    fx = golden("ref_siam_thermo_nd_nk256")
    assert len(eigs) == 30
    check_eigs(fx, eigs, 2.0)
    assert np.abs(entropy - fx["entropy"]).max() < 1e-8
    assert np.abs(nd - fx["qsysOPeratorExpValue0"]).max() < 1e-9
    ref = siam_run(imp, bath, 256, 30, 2.0, V=0.15, track_ops=M.n_d(), fdm=True, full_fdag=False)
    # Frobenius norm of the rotated n_d: basis-invariant, so the copied-back
    # blocks must carry the oracle's value
    norm2 = sum(float(np.sum(m * m)) for m in ref["snaps"][max(ref["snaps"])]["ops"][0].values())
    assert abs(extra[0] - norm2) <= 1e-9 * norm2
    assert extra[1] == 1 and extra[2] > 0  # loadqOperator rebuilt one operator with its blocks
