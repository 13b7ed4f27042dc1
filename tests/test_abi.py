"""The C ABI library builds, loads and exports every symbol include/frg.h
declares; host-side argument checks and error reporting work without a GPU.
No compute calls here (CPU only)."""
import ctypes
import os
import re

import pytest

import frg
from frg import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(frg_\w+)\s*\(", text))
    return names


def test_header_matches_binding_table():
    assert declared_symbols() == set(native.EXPORTED)


def test_library_exports_every_declared_symbol(built_lib):
    L = ctypes.CDLL(built_lib)
    for name in sorted(declared_symbols()):
        assert hasattr(L, name), name


def test_status_strings_and_defaults(built_lib):
    L = frg.lib()
    assert L.frg_status_string(0) == b"ok"
    assert L.frg_status_string(2) == b"CUDA error"
    opt = native.Options()
    opt.device = 5
    L.frg_options_default(ctypes.byref(opt))
    assert (opt.device, opt.vel_damping, opt.mpc_mode, opt.warps_per_cta, opt.ctas_per_sm) == (0, 0, 0, 0, 0)


def test_null_context_is_rejected_not_crashing(built_lib):
    L = frg.lib()
    assert L.frg_gradient(None, 4, None, None, None, None, None, None, None) == 1
    assert L.frg_plan_launch(None, None) == 1
    L.frg_destroy(None)
    L.frg_plan_destroy(None)
    assert L.frg_create(None, None) == 1
    assert b"NULL" in L.frg_last_error(None)


def test_create_without_gpu_reports_error(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(frg.FrgError) as ei:
        frg.Context()
    assert ei.value.status == 2
