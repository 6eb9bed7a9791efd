"""Build libsph_gb300.so in-tree: nvcc for sm_103a only, translation units in parallel.

    python npr-sph_gb300/build.py          # incremental
    python npr-sph_gb300/build.py --force  # rebuild everything

The library is self-contained (CUDA runtime linked statically) and exports the
C ABI declared in include/sph_gb300.h.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libsph_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers():
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((REPO / "include").glob("*.h"))


def _compile_cmd(src: Path, obj: Path, cuda: Path) -> list[str]:
    inc = ["-I", str(REPO / "include"), "-I", str(CSRC)]
    if src.suffix == ".cu":
        return [str(cuda / "bin" / "nvcc"), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills", *inc, "-c", str(src), "-o", str(obj)]
    return ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", str(cuda / "include"), *inc,
            "-c", str(src), "-o", str(obj)]


def build(force: bool = False, verbose: bool = False) -> Path:
    cuda = _cuda_home()
    OBJ.mkdir(exist_ok=True)
    # Objects built on another host architecture (the tree is copied between x86-64 and
    # aarch64 machines) are rebuilt.
    stamp = OBJ / "MACHINE"
    machine = platform.machine()
    if not stamp.exists() or stamp.read_text().strip() != machine or not LIB.exists():
        force = True
    hdr_mtime = max(p.stat().st_mtime for p in _headers())
    jobs = []
    for src in _sources():
        obj = OBJ / (src.name + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_mtime):
            jobs.append((src, obj))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = {ex.submit(subprocess.run, _compile_cmd(s, o, cuda), capture_output=True, text=True): s for s, o in jobs}
        for fut in cf.as_completed(futs):
            r = fut.result()
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"compile failed: {futs[fut].name}")
    objs = [OBJ / (s.name + ".o") for s in _sources()]
    if force or jobs or not LIB.exists():
        cmd = [str(cuda / "bin" / "nvcc"), *ARCH, "-shared", "-cudart", "static", "-o", str(LIB),
               *map(str, objs), "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("link failed")
    stamp.write_text(machine)
    build_headless(force or bool(jobs), verbose)
    return LIB


HEADLESS = PKG / "sph_headless"


def build_headless(force: bool = False, verbose: bool = False) -> Path:
    """The C++ host loop (host/sph_headless.cpp) linked against libsph_gb300.so."""
    src = PKG / "host" / "sph_headless.cpp"
    if not force and HEADLESS.exists() and HEADLESS.stat().st_mtime >= max(src.stat().st_mtime, LIB.stat().st_mtime):
        return HEADLESS
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", str(REPO / "include"), str(src), "-o", str(HEADLESS),
           "-L", str(PKG), "-lsph_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
    if r.returncode:
        raise RuntimeError("headless driver build failed")
    return HEADLESS


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
