"""Builds libgme.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled to an object in parallel, then linked as a
shared library against the shared CUDA runtime (so the process shares one
runtime with any other CUDA user, e.g. PyTorch).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUTDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUTDIR, "libgme.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _deps():
    d = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    d.append(os.path.join(REPO, "include", "gme.h"))
    d.append(os.path.join(REPO, "include", "gme_reference.h"))
    return [x for x in d if os.path.exists(x)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(x) <= t for x in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    if not force and up_to_date():
        build_tools()
        return LIB
    os.makedirs(OUTDIR, exist_ok=True)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    common = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I" + os.path.join(REPO, "include"), *extra_flags]

    def one(src):
        obj = os.path.join(OUTDIR, os.path.basename(src) + ".o")
        cmd = [nvcc(), *common, "-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd.insert(1, "-x=cu")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, sources()))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs,
           "-Xlinker", "-rpath=" + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_tools()
    return LIB


TOOLS = os.path.join(HERE, "tools")
TOOL_BINS = {"gme-align": ("gme_align.cpp", True), "gme-generate": ("gme_generate.cpp", False),
             "gme-refcheck": ("gme_refcheck.cpp", True)}


def build_tools() -> dict:
    """The command-line tools (host C++): gme-align (the reference's drivers on the
    library), gme-generate (the reference's data files from a seeded PRNG) and
    gme-refcheck (every reference host-function signature called once)."""
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    out = {}
    for name, (src, uses_lib) in TOOL_BINS.items():
        exe = os.path.join(OUTDIR, name)
        deps = [os.path.join(TOOLS, src), os.path.join(TOOLS, "gme_datafile.h"),
                os.path.join(REPO, "include", "gme.h"),
                os.path.join(REPO, "include", "gme_reference.h")] + ([LIB] if uses_lib else [])
        if not (os.path.exists(exe) and all(os.path.getmtime(d) <= os.path.getmtime(exe) for d in deps)):
            cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-I" + os.path.join(REPO, "include"),
                   "-I" + TOOLS, os.path.join(TOOLS, src), "-o", exe + f".tmp{os.getpid()}"]
            if uses_lib:
                cmd += ["-L" + OUTDIR, "-lgme", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{name} failed:\n{r.stdout}\n{r.stderr}")
            os.replace(exe + f".tmp{os.getpid()}", exe)
        out[name] = exe
    return out


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
