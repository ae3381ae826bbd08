"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol
(no compute call: runs without a GPU)."""
import ctypes

from autopdex_gb300 import _native as N
from autopdex_gb300 import build


def test_library_exports_every_header_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    declared = N.header_symbols()
    assert len(declared) >= 18
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    assert sorted(N._SIGNATURES) == N.header_symbols()


def test_struct_layouts_match_header():
    # sizes of the option/info structs as laid out by the C compiler for this ABI
    assert ctypes.sizeof(N.SolveOpts) == 4 + 4 + 8 + 8 + 4 + 4
    assert ctypes.sizeof(N.NewtonInfo) == 4 + 4 + 8 + 8 + 4 + 4 + 4 + 4 + 64 * 8 + 64 * 4
