"""The C-ABI library loads and exports every function include/fia.h declares (no GPU calls)."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "fia.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(fia_[A-Za-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("fia_create", "fia_destroy", "fia_move_substances_3D", "fia_advect_velocity_xyz",
                 "fia_calc_pressure_3D", "fia_calc_pressure_gradient_term_3D", "fia_max_abs_velocity"):
        assert must in names


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_library_exports_every_declared_symbol():
    import fia
    path = fia.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.fia_api_version() == 1
    lib.fia_error_string.restype = ctypes.c_char_p
    assert lib.fia_error_string(-3) == b"unsupported option"
