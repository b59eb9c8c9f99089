"""The C ABI library builds, loads without a GPU and exports every symbol include/fednl_gpu.h
declares; without a device its entry points fail loudly (no CPU fallback)."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "fednl_gpu.h")


def header_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|int32_t|double|const char\*|void\*)\s+(fednl_(?:gpu|mx|server)_\w+|doptExecute\w+)\s*\(",
                                 txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    from ufednl_gb300 import build, fednl
    build.build()
    return fednl


def test_header_declares_the_binding_table(lib):
    assert header_symbols() == sorted(lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib.lib_path()], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\bT (fednl_(?:gpu|mx|server)_\w+|doptExecute\w+)", out.stdout))
    missing = [s for s in header_symbols() if s not in exported]
    assert not missing, missing
    L = lib.load()
    for s in header_symbols():
        assert getattr(L, s) is not None


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_entry_points_fail_loudly_without_a_device(lib):
    with pytest.raises(lib.FedNLError) as e:
        lib.get_topk_from_upper_diagonal_part(np.zeros(16), 4, 4, 2)
    assert e.value.code == -6
    from ufednl_gb300 import datagen
    p = datagen.binary_problem(0, 5, [4, 4], 0.5, 1e-3)
    with pytest.raises(lib.FedNLError):
        lib.FedNL(p, "topk", 3, 1.0)
