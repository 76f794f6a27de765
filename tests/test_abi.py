"""The C-ABI library loads and exports every symbol the headers declare (CPU only)."""
import ctypes
import os
import re
import subprocess

from conftest import REPO

HEADERS = [os.path.join(REPO, "include", f) for f in sorted(os.listdir(os.path.join(REPO, "include")))
           if f.endswith(".h")]


def _lib_path():
    import __graft_entry__ as ge
    ge.build_library()
    import gpumemefficient_gb300 as g
    return g.LIB_PATH


def declared_c_functions():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gme_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


def test_headers_declare_entry_points():
    names = declared_c_functions()
    for must in ("gme_create", "gme_destroy", "gme_align", "gme_align_device"):
        assert must in names


def test_library_exports_all_declared_symbols():
    path = _lib_path()
    L = ctypes.CDLL(path)
    missing = [n for n in declared_c_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_reference_cpp_signatures_exported():
    path = _lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    for sym in ["_Z3LCSiiPiS_iiS_", "_Z3LCSiiPiS_", "_Z2EDiiPiS_iiS_ii", "_Z2EDiiPiS_iiS_",
                "_Z2EDiiPiS_", "_Z2SWiiPiS_iiS_ii", "_Z2SWiiPiS_iiS_", "_Z2SWiiPiS_", "_Z3SORiiPiii", "_Z3SORiiPi"]:
        assert sym in out, sym


def test_status_strings_without_gpu():
    L = ctypes.CDLL(_lib_path())
    L.gme_status_string.restype = ctypes.c_char_p
    assert L.gme_status_string(4) == b"device wait timed out"
    import gpumemefficient_gb300 as g
    s = g.lib().gme_default_scoring()
    assert (s.match, s.mismatch, s.gap, s.ed_boundary) == (3, -3, -2, 0)
