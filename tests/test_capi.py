"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol
(no compute calls: these run without a GPU)."""
import ctypes
import os
import re

import pytest

from conftest import REPO


def _declared():
    names = []
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        if h.endswith(".h"):
            txt = open(os.path.join(REPO, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(cmt_\w+)\s*\(", txt, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from cmtip_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = _declared()
    for must in ("cmt_plan_create", "cmt_set_pts", "cmt_execute", "cmt_plan_destroy", "cmt_last_error"):
        assert must in names


def test_library_exports_all_declared_symbols(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from cmtip_gb300 import _lib
    assert set(_declared()) <= set(_lib.SIGNATURES)


def test_library_reports_version(lib):
    lib.cmt_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.cmt_version()
