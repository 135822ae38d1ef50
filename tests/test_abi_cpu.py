"""CPU-side checks of the C ABI: the library builds, loads and exports every
entry point declared in include/espins_gpu.h (no GPU work is done here)."""
import ctypes
import os
import re

import pytest

from espins_gb300 import build as B
from espins_gb300 import lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "espins_gpu.h")) as fh:
        txt = fh.read()
    return sorted(set(re.findall(r"^int\s+(esp_\w+)\s*\(", txt, flags=re.M)))


def test_header_and_binding_list_agree():
    assert _declared() == sorted(L.EXPORTED)


def test_library_exports_every_declared_symbol():
    path = B.build()
    lib = ctypes.CDLL(path)
    for name in _declared():
        assert hasattr(lib, name), name


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(L.EspError) as ei:
        L.Engine(8, 1, (2, 2, 2), 1)
    assert ei.value.code in (L.ESP_ECUDA,)
