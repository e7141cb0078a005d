"""CPU checks of the C ABI: the library builds, loads, and exports every
symbol declared in include/qsim_gb300.h.  No compute calls (no GPU here)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "qsim_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(qsg_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_core_entry_points():
    syms = declared_symbols()
    for s in ("qsg_apply_gate", "qsg_apply_controlled_gate",
              "qsg_expectation_value", "qsg_norm", "qsg_inner_product",
              "qsg_sample", "qsg_collapse", "qsg_set_state_zero",
              "qsg_measure", "qsg_partial_norms", "qsg_find_measured_bits"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from qsim_gb300 import _native
    lib = C.CDLL(_native.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert missing == []


def test_python_binding_covers_header():
    from qsim_gb300 import _native
    missing = [s for s in declared_symbols() if s not in _native.SIGNATURES]
    assert missing == []


def test_min_size_and_chunks():
    from qsim_gb300 import _native
    assert _native.lib.qsg_min_size(0) == 64
    assert _native.lib.qsg_min_size(5) == 64
    assert _native.lib.qsg_min_size(6) == 128
    assert _native.lib.qsg_min_size(30) == 2 << 30
    assert _native.lib.qsg_num_chunks(13) == 1
    assert _native.lib.qsg_num_chunks(20) == 1 << 7


def test_errors_without_gpu_are_status_codes():
    """Calls that fail argument checks return a status and a message."""
    from qsim_gb300 import _native
    assert _native.lib.qsg_ctx_create(0, None, None) == 1
    assert b"null" in _native.lib.qsg_last_error()
