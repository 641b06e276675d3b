"""The engine library builds, loads and exports every entry point its header declares (no GPU)."""
import ctypes as C
import os
import re

import pytest

from stablercwa_gb300 import abi
from stablercwa_gb300.engine import EngineError, load_library

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|void|long long|double)\s+\**(rcwa_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    L = load_library()
    names = declared_functions()
    assert len(names) >= 12
    for name in sorted(names):
        assert hasattr(L, name), name


def test_struct_layouts_match_header():
    # sizes the C compiler gives the header's structs on LP64 targets
    assert C.sizeof(abi.rcwa_complex) == 16
    assert C.sizeof(abi.rcwa_layer1d) == 8 + 8 + 16 + 8 + 8 + 8 + 8
    assert C.sizeof(abi.rcwa_stack1d) == 16 + 16 + 8 + 8 + 8
    assert C.sizeof(abi.rcwa_options) == 24 + 8
    assert C.sizeof(abi.rcwa_result1d) == 10 * 8
    assert C.sizeof(abi.rcwa_result_conical) == 16 * 8
    assert C.sizeof(abi.rcwa_server_config) == 4 + 4 + 8 + 4 + 4
    assert C.sizeof(abi.rcwa_response) == 4 + 4 + 4 * 8 + 8
    assert C.sizeof(abi.rcwa_xprofile2d) == 8 + 8 + 8
    assert C.sizeof(abi.rcwa_layer2d) == 8 + 8 + 16 + 8 + 8 + 8
    assert C.sizeof(abi.rcwa_stack2d) == 8 + 16 + 8 + 8 + 8 + 8
    assert C.sizeof(abi.rcwa_point2d) == 24 + 32
    assert C.sizeof(abi.rcwa_result2d) == 24 * 8


def test_abi_version_and_defaults():
    L = load_library()
    assert L.rcwa_gpu_abi_version() == 1
    o = abi.rcwa_options()
    L.rcwa_options_default(C.byref(o))
    assert (o.eig_method, o.linear_solver, o.homogeneous_fast_path, o.eig_max_iter) == (0, 0, 1, 30)
    assert o.eig_eps == 2.220446049250313e-16


def test_create_without_device_reports_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from stablercwa_gb300.engine import Engine
    with pytest.raises(EngineError):
        Engine()


def test_server_create_without_device_reports_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from stablercwa_gb300.engine import Server
    with pytest.raises(EngineError):
        Server(slots=1)


def test_autotune_set_validates_forms():
    from stablercwa_gb300.engine import autotune_set, autotune_table
    assert autotune_set(False, 77, 1000, 12) == -1      # not a kernel form
    assert autotune_set(True, 77, 1000, -1) == -1       # no cluster form for the Hermitian solver
    assert autotune_set(False, 77, 1000, 16) == 0
    assert "general 77 512 16" in autotune_table()      # batch 1000 falls in the bucket of 512
