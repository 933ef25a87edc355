"""The C-ABI library loads and exports every symbol declared in include/*.h (no GPU calls)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(mm_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    assert "mm_compute" in declared_symbols() and "mm_create" in declared_symbols()


def test_library_exports_all_declared_symbols():
    from micmec_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    lib = ctypes.CDLL(build.LIB)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
