"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/fealpy_gb300.h (no GPU compute calls here)."""
import ctypes
import os
import re

import pytest

from fealpy_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "fealpy_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fgb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(header_symbols()) == set(_lib.exported_symbols())


def test_host_only_entry_points():
    lib = _lib.lib()
    assert lib.fgb_abi_version() == 2
    assert lib.fgb_status_string(0) == b"ok"
    assert b"pattern" in lib.fgb_status_string(4)
    assert lib.fgb_pcg_workspace_bytes(1000) >= 5 * 8 * 1000
    assert lib.fgb_scan_workspace_bytes(10) > 0


def test_argument_validation_without_gpu():
    lib = _lib.lib()
    # invalid sizes are rejected before any CUDA call
    assert lib.fgb_csr_spmv(1, 0, None, None, None, None, None, 0, None) == 1
    assert lib.fgb_cell_factors(4, 10, None, None, 1, None, None, None, None, 1, None, None, None) == 1
    assert lib.fgb_pcg_f64(0, None, None, None, None, None, None, 0.0, 0.0, 1, 1, 0, 0, 0, None, 0, None, None) == 1
    assert lib.fgb_pcg_f64_noalloc(0, None, None, None, None, None, None, 0.0, 0.0, 1, 1, 0, 0, None, None) == 1
    assert lib.fgb_pattern_build(0, None, None, None, 4, 1, None, None, 0, None, None, None, 0, None) == 1
    assert lib.fgb_pattern_compact(0, None, None, None, 4, None, None, None, None, None, 0, None) == 1
    # batched solver: sizes, bad capacities and bad launch shapes are refused on the host
    assert lib.fgb_batch_bytes(0, 1, 1) == 0 and lib.fgb_batch_bytes(4, 16, 16) > 0
    h = ctypes.c_void_p()
    assert lib.fgb_batch_create(0, 1, 1, 256, None, 0, ctypes.byref(h)) == 1
    assert lib.fgb_batch_create(4, 16, 16, 100, None, 0, ctypes.byref(h)) == 1
    assert lib.fgb_batch_create(4, 16, 16, 256, None, 0, ctypes.byref(h)) == 2
    assert lib.fgb_batch_destroy(None) == 1
    # delta-coded SELL copy: sizes, block lists and missing arrays are refused on the host
    one = ctypes.c_void_p(16)  # a non-null stand-in: nothing is dereferenced on these paths
    sizes = (ctypes.c_int64 * 3)(4, 4, 4)
    assert lib.fgb_sell_d16_workspace_bytes(0) == 0 and lib.fgb_sell_d16_workspace_bytes(100) > 0
    assert lib.fgb_sell_renumber(0, one, one, 0, None, one, one, None, 0, None) == 1
    assert lib.fgb_sell_renumber(12, one, one, 17, sizes, one, one, None, 0, None) == 1   # too many blocks
    assert lib.fgb_sell_renumber(13, one, one, 3, sizes, one, one, None, 0, None) == 1    # sizes do not add up
    assert lib.fgb_sell_renumber(12, one, one, 1, None, one, one, None, 0, None) == 1     # no sizes
    assert lib.fgb_sell_renumber(12, one, one, 0, None, one, one, None, 0, None) == 2     # min-column order: workspace
    assert lib.fgb_csr_permute(0, one, one, None, None, one, one, one, one, None, None, None, 0, None) == 1
    assert lib.fgb_sell_d16_indptr(5, one, one, None, None, 0, None) == 1
    assert lib.fgb_sell_fill_d16(5, one, one, None, None, one, one, one, None, None, None, None) == 1
    assert lib.fgb_permute(1, 5, one, one, one, 0, None) == 1                             # src == dst
    assert lib.fgb_permute(7, 5, one, one, ctypes.c_void_p(32), 0, None) == 1             # bad dtype
    # node-triple copy: rows must come in whole triples
    assert lib.fgb_sell_b3_indptr(10, one, one, one, one, 1 << 20, None) == 1
    assert lib.fgb_sell_b3_indptr(9, one, one, one, None, 0, None) == 2
    assert lib.fgb_sell_fill_b3(10, one, one, one, None, one, one, one, None, None, None) == 1
    assert lib.fgb_sell_fill_b3(9, one, one, None, None, one, one, one, one, None, None) == 1  # values, no source


def test_build_targets_sm103a():
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.ARCH_FLAGS)


def test_header_compiles_as_c99_and_cxx(tmp_path):
    """include/fealpy_gb300.h is a plain C header (the boundary a cgo/ctypes/
    JNI binding includes): it compiles as C99 and as C++17 on its own."""
    import shutil
    import subprocess
    src = tmp_path / "use.c"
    src.write_text('#include "fealpy_gb300.h"\n'
                   'int probe(void) { fgb_sell s; fgb_pcg_info i; (void)s; (void)i;\n'
                   '  return (int)sizeof(fgb_batch_state) + (int)FGB_PCG_STAGNATED; }\n')
    inc = os.path.join(ROOT, "include")
    for cc, std in (("gcc", "-std=c99"), ("g++", "-std=c++17")):
        if shutil.which(cc) is None:
            pytest.skip(f"{cc} not found")
        lang = ["-x", "c++"] if cc == "g++" else []
        res = subprocess.run([cc, std, "-Wall", "-Werror", "-fsyntax-only", "-I", inc] + lang + [str(src)],
                             capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
