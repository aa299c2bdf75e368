"""The C-ABI library builds, loads and exports every entry point that
include/nrg_gpu.h declares; without a GPU it refuses to run (no CPU fallback)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "nrg_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nrg_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    from nrgplusplus_gb300.build import build
    return build(verbose=False)


def test_header_declares_entry_points():
    names = _declared()
    assert len(names) >= 35
    assert "nrg_run_add_site" in names and "nrg_fdm_calc" in names


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_api_binds_every_declared_symbol():
    from nrgplusplus_gb300 import api
    assert sorted(api.EXPORTS) == _declared()


def test_no_gpu_means_loud_failure(libpath):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from nrgplusplus_gb300 import api
    with pytest.raises(api.NrgError) as ei:
        api.Engine()
    assert ei.value.code == 6  # NRG_E_NOCUDA
