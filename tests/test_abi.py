"""The C-ABI library loads and exports every entry point include/sam_gpu.h
declares (no GPU needed: nothing here calls into the device)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sam_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(sam_gpu_\w+)\s*\(", text, re.M)))


def test_header_declares_the_drop_in_surface():
    syms = declared_symbols()
    for name in ("rhs", "xy_trans_f", "xy_trans_b", "z_trans_f", "z_trans_b", "x2z_decomp", "z2x_decomp",
                 "x_deriv", "y_deriv", "vel_max", "init", "stage", "step", "upload", "download"):
        assert f"sam_gpu_{name}" in syms


def test_library_builds_and_exports_every_declared_symbol():
    from sam_gb300 import build as B
    from sam_gb300 import sam_gpu
    path = B.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # the Python mirror binds exactly the declared surface
    assert set(sam_gpu.EXPORTS) <= set(declared_symbols())


def test_calls_before_init_fail_cleanly():
    """Every entry point returns an error code, never traps, without a context
    (no device work is issued on this path)."""
    from sam_gb300 import build as B
    lib = ctypes.CDLL(B.build())
    assert lib.sam_gpu_stage(1) == -2
    assert lib.sam_gpu_dims(None) == -2
    lib.sam_gpu_error_string.restype = ctypes.c_char_p
    assert b"sam_gpu_init" in lib.sam_gpu_error_string()


def test_fortran_module_binds_every_symbol():
    """include/sam_gpu.f90 (the ISO_C_BINDING module sam.f uses) has one
    bind(C) interface per routine the header declares, with the same number
    of arguments."""
    f90 = open(os.path.join(ROOT, "include", "sam_gpu.f90")).read().replace("&\n", " ")
    bound = dict((m.group(2), m.group(1)) for m in
                 re.finditer(r"function\s+\w+\(([^)]*)\)\s*bind\(C,\s*name=\"(sam_gpu_\w+)\"\)", f90))
    header = open(os.path.join(ROOT, "include", "sam_gpu.h")).read()
    for sym in declared_symbols():
        assert sym in bound, sym
        m = re.search(r"^\s*(?:int|const char\*)\s+" + sym + r"\s*\(([^)]*)\)", header, re.M)
        c_args = [a for a in m.group(1).replace("\n", " ").split(",") if a.strip() not in ("", "void")]
        f_args = [a for a in bound[sym].split(",") if a.strip()]
        assert len(c_args) == len(f_args), (sym, c_args, f_args)
