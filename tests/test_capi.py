"""CPU tests of the C-ABI library: it loads, exports every symbol the
header declares, and its host-side checks reject malformed input before
any device work (no kernel is launched here)."""
import re
from pathlib import Path

from gls.capi import EXPORTED

HEADER = Path(__file__).resolve().parent.parent / "include" / "gls.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(gls_[a-z_0-9]+)\s*\(", text, re.M)))


def test_header_lists_the_binding():
    assert declared_symbols() == sorted(EXPORTED)


def test_library_exports_every_declared_symbol(libgls):
    for name in declared_symbols():
        assert hasattr(libgls, name), name


def test_abi_version(libgls):
    assert libgls.gls_abi_version() == 2


def test_create_rejects_bad_calc_mode(libgls):
    import ctypes as C
    from gls.capi import Opts
    o = Opts(0, 7, 0, 1.0, 0, 0, None)
    h = C.c_void_p()
    assert libgls.gls_create(C.byref(o), C.byref(h)) != 0
    assert not h.value
