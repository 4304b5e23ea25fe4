"""C ABI checks that need no GPU: the library builds for sm_103a, loads, exports
every entry point include/lpg.h declares, and rejects bad settings before any
device work (the reference aborts on unknown keys, ellipticSettings.cpp:144-146)."""
import ctypes

import pytest

from libparanumal_gb300.build import build_library


@pytest.fixture(scope="module")
def L():
    build_library()
    import libparanumal_gb300 as lpg
    return lpg.lib()


def test_exports_every_declared_symbol(L):
    import libparanumal_gb300 as lpg
    names = lpg.declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_unknown_setting_is_rejected_before_device_work(L):
    h = ctypes.c_void_p()
    st = L.lpg_elliptic_create(b"[BOX NX]\n4\n\n[NOT A KEY]\n1\n", ctypes.byref(h))
    assert st == -6
    assert b"NOT A KEY" in L.lpg_last_error()
    assert not h.value


def test_null_arguments_are_rejected(L):
    assert L.lpg_elliptic_create(None, None) == -1
    assert L.lpg_ax_hex_f64(7, 1, None, None, None, 0, None, 0, None, 1.0, None, None, None, 0, None) == -1
    assert L.lpg_ax_hex_f64(9, 1, None, None, None, 0, None, 0, None, 1.0, None, None, None, 0, None) == -3
    assert L.lpg_dot_f64(-1, None, None, None, None) == -1


def test_version(L):
    assert b"sm_103a" in L.lpg_version()


def test_info_keys_match_the_header():
    """The Python object's info() names map to the LPG_INFO_* values include/lpg.h defines."""
    import os
    import re
    import libparanumal_gb300 as lpg
    header = open(os.path.join(os.path.dirname(__file__), "..", "include", "lpg.h")).read()
    defs = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"#define LPG_INFO_(\w+) (\d+)", header)}
    assert defs == lpg.INFO
