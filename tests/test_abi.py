"""The C ABI: header, field table, exported symbols, and the product library's refusal to run
without a GPU (no CPU fallback)."""
import ctypes as C
import re
from pathlib import Path

import pytest

from gom_release_gb300.core import ABI_VERSION, FIELDS, GomCore, GomDims, GomError, load_library

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gom_core.h"


def _declared_functions():
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^[\w\s\*]*?\b(gom_\w+)\s*\(", txt, flags=re.M)))


def test_field_table_matches_header():
    txt = HEADER.read_text()
    body = txt[txt.index("typedef enum gom_field"):txt.index("} gom_field;")]
    names = re.findall(r"GOM_F_(\w+)", body)
    names = [n for n in names if n != "COUNT"]
    assert [n.lower() for n in names] == [f.replace("dz1", "dz1") for f in
                                          [x.upper().lower() for x in FIELDS]], "FIELDS order differs from gom_field"


def test_cuda_library_exports_every_declared_function(core_so):
    lib = C.CDLL(str(core_so))
    missing = [f for f in _declared_functions() if not hasattr(lib, f)]
    assert not missing, missing
    assert len(_declared_functions()) >= 25


def test_oracle_exports_the_time_loop_abi(oracle_so):
    lib = C.CDLL(str(oracle_so))
    needed = [f for f in _declared_functions() if f != "gom_pcg_solve_noalloc"]
    assert not [f for f in needed if not hasattr(lib, f)]


def test_abi_version_and_field_sizes(core_so, oracle_so):
    for so in (core_so, oracle_so):
        lib = load_library(so)
        assert lib.gom_abi_version() == ABI_VERSION
        d = GomDims(10, 23, 14, 5, 12, 3, 1, 0)
        n = C.c_int64()
        eb = C.c_int32()
        expect = {"eta_cell": (10, 8), "wn_cell": (60, 8), "un_face": (115, 8), "u_node": (84, 8),
                  "top_layer_face": (23, 4), "qu_boundary": (1, 8), "elm_foot": (115, 4), "av": (138, 8)}
        for name, (cnt, size) in expect.items():
            assert lib.gom_field_info(C.byref(d), FIELDS.index(name) + 1, C.byref(n), C.byref(eb)) == 0
            assert (n.value, eb.value) == (cnt, size), name
        assert lib.gom_field_info(C.byref(d), 999, C.byref(n), C.byref(eb)) == 1


def test_cuda_library_fails_loudly_without_gpu(core_so):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from gom_release_gb300.deck import tidal_basin
    deck = tidal_basin(nx=6, ny=4)
    with pytest.raises(GomError):
        GomCore(deck, lib=load_library(core_so))
