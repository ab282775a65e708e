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


# ---- argument checking: rejected before any CUDA call, so these run without a GPU

def _err(lib):
    lib.cmt_last_error.restype = ctypes.c_char_p
    return lib.cmt_last_error().decode()


def test_bad_arguments_return_arg_error(lib):
    vp, out = ctypes.c_void_p, ctypes.c_void_p()
    lib.cmt_plan_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_double, vp, ctypes.POINTER(vp)]
    assert lib.cmt_plan_create(3, 21, 32, 1e-6, 1, 0.0, None, ctypes.byref(out)) == 1
    assert "type must be 1 or 2" in _err(lib) and not out.value
    assert lib.cmt_plan_create(1, 21, 16, 1e-6, 1, 0.0, None, ctypes.byref(out)) == 1
    assert "prec must be 32 or 64" in _err(lib)
    lib.cmt_phase_create.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.POINTER(vp)]
    assert lib.cmt_phase_create(0, 64, None, ctypes.byref(out)) == 1 and "M must be in" in _err(lib)
    assert lib.cmt_phase_create(21, 16, None, ctypes.byref(out)) == 1 and "prec" in _err(lib)
    lib.cmt_cg_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.POINTER(vp)]
    assert lib.cmt_cg_create(1, 32, 0, None, ctypes.byref(out)) == 1 and "M must be in [2, 512]" in _err(lib)
    lib.cmt_match_create.argtypes = [ctypes.c_int64, ctypes.c_int, vp, ctypes.POINTER(vp)]
    assert lib.cmt_match_create(16384, 7, None, ctypes.byref(out)) == 1 and "mode must be" in _err(lib)


def test_noalloc_filter_rejects_grids_beyond_its_scratch(lib):
    # the allocation-free support filter checks M against its fixed scratch first
    vp = ctypes.c_void_p
    lib.cmt_support_from_estimate_noalloc.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp]
    dummy = vp(16)  # never dereferenced: the size check fails before any device work
    assert lib.cmt_support_from_estimate_noalloc(dummy, 129, dummy, 0, None) == 1
    assert "128" in _err(lib)
    assert lib.cmt_support_from_estimate_noalloc(None, 21, dummy, 0, None) == 1


def test_python_binding_maps_status_codes():
    from cmtip_gb300 import _lib
    with pytest.raises(ValueError, match="type must be 1 or 2"):
        _lib.call("cmt_plan_create", 3, 21, 32, 1e-6, 1, 0.0, None, ctypes.byref(ctypes.c_void_p()))
    with pytest.raises(ValueError, match="null"):
        _lib.call("cmt_phase_er", None, None, None, None, None, float("inf"), 1)


def test_missing_library_fails_loudly(tmp_path):
    # no fallback: without the built library the package's first call raises ImportError
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from cmtip_gb300 import _lib\n"
            "try:\n"
            "    _lib.load(%r)\n"
            "except ImportError as e:\n"
            "    print('ImportError:', e)\n"
            "else:\n"
            "    print('loaded')\n") % (REPO, str(tmp_path / "absent.so"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120).stdout
    assert out.startswith("ImportError:") and "no non-CUDA implementation" in out


def test_every_entry_point_rejects_null_arguments():
    # every function, called with null pointers and zero sizes, returns CMT_ERR_ARG before any
    # CUDA call (destroy functions accept null, like free); run in a child so that a missing
    # check would show as a crash of that child only
    import subprocess
    import sys
    code = ("import ctypes, sys; sys.path.insert(0, %r)\n"
            "from cmtip_gb300 import _lib\n"
            "lib = _lib.load()\n"
            "ints = (ctypes.c_int, ctypes.c_int64, ctypes.c_long, ctypes.c_uint, ctypes.c_size_t)\n"
            "for name, args in sorted(_lib.SIGNATURES.items()):\n"
            "    if name in ('cmt_version', 'cmt_last_error'):\n"
            "        continue\n"
            "    vals = [0.0 if a in (ctypes.c_double, ctypes.c_float) else 0 if a in ints else None\n"
            "            for a in args]\n"
            "    print(name, getattr(lib, name)(*vals), flush=True)\n") % REPO
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    got = dict(line.split() for line in r.stdout.splitlines())
    from cmtip_gb300 import _lib
    assert len(got) == len(_lib.SIGNATURES) - 2
    for name, rc in got.items():
        assert rc == ("0" if name.endswith("_destroy") else "1"), (name, rc)
