"""The reference's own drivers build unchanged on this library: every driver program of
the LCS, EditDistance, SmithWaterman and SAT directories (GPU_Hyperlane_Share.cpp,
GPU_Hyperlane_Cache.cpp, GPU_TILE_SHARE.cpp, GPU_TILE_NOSHARE.cpp, GPU.cpp), compiled from
its own unmodified source with `-include include/gme_reference.h` and linked against
libgme.so in place of the reference's .cu files.  Runs only where the reference checkout
is present (the first of $GME_REFERENCE_ROOT and a `reference` directory beside this
repository); the programs themselves need a GPU and are exercised through gme-refcheck
in test_refsig_gpu.py."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(REPO, "gpumemefficient_gb300", "_lib")


def reference_root():
    for cand in (os.environ.get("GME_REFERENCE_ROOT"), os.path.join(os.path.dirname(REPO), "reference")):
        if cand and os.path.isfile(os.path.join(cand, "LCS", "LCS.cpp")):
            return cand
    return None


DRIVERS = [(d, f) for d in ("LCS", "EditDistance", "SmithWaterman")
           for f in ("GPU_Hyperlane_Share", "GPU_Hyperlane_Cache", "GPU_TILE_SHARE", "GPU_TILE_NOSHARE", "GPU")]
DRIVERS += [("SAT", "GPU_Hyperlane_Share"), ("SAT", "GPU_Hyperlane_Cache")]


@pytest.mark.parametrize("d,f", DRIVERS)
def test_reference_driver_links(tmp_path, d, f):
    ref = reference_root()
    if ref is None:
        pytest.skip("no reference checkout on this machine")
    if not os.path.exists(os.path.join(LIB, "libgme.so")):
        pytest.skip("libgme.so not built")
    src = os.path.join(ref, d, f + ".cpp")
    if not os.path.exists(src):
        pytest.skip(f"{d}/{f}.cpp not in this checkout")
    exe = str(tmp_path / f"{d}-{f}")
    cmd = [shutil.which("g++") or "g++", "-O1", "-w", "-include", os.path.join(REPO, "include", "gme_reference.h"),
           "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(ref, d), src, "-L" + LIB, "-lgme",
           "-Wl,-rpath," + LIB, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.exists(exe)
