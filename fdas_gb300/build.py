"""Build the sm_103a shared library ``fdas_gb300/libfdas_gb300.so`` with nvcc.

Each ``csrc/*.cu`` translation unit is compiled in parallel, then linked with
``-shared``; objects go to ``fdas_gb300/_build``.  No CMake, no torch
extension machinery: the library exposes a plain C ABI (include/fdas_gb300.h).
"""

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libfdas_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                   f"-I{ROOT / 'include'}", f"-I{CSRC}", "-Xptxas", "-warn-spills"]


def sources():
    return sorted(CSRC.glob("*.cu"))


def _needs_rebuild(obj, src):
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    deps = [src] + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose=False, force=False, ptxas_verbose=False):
    BUILD.mkdir(exist_ok=True)
    exe = nvcc()
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        if force or _needs_rebuild(obj, src):
            cmd = [exe] + flags() + (["-Xptxas", "-v"] if ptxas_verbose else []) + ["-c", str(src), "-o", str(obj)]
            jobs.append((src, cmd))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): src for src, cmd in jobs}
        for fut in cf.as_completed(futs):
            r = fut.result()
            if verbose or r.returncode != 0 or ptxas_verbose:
                sys.stderr.write(r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {futs[fut].name}")
    objs = [str(BUILD / (s.stem + ".o")) for s in sources()]
    if jobs or not LIB.exists() or force:
        cmd = [exe] + ARCH + ["-shared", "-o", str(LIB)] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stderr)
            raise RuntimeError("link failed")
    build_driver(force=force)
    return LIB


DRIVER_SRC = ROOT / "tests" / "cpp" / "fdas_drive.cpp"
DRIVER = BUILD / "fdas_drive"


def build_driver(force=False):
    """C++ driver over include/FDAS.hpp (the reference-style host class), linked
    against the library; used by the GPU tests."""
    if not DRIVER_SRC.exists():
        return None
    if not force and DRIVER.exists() and DRIVER.stat().st_mtime > max(
            DRIVER_SRC.stat().st_mtime, LIB.stat().st_mtime, (ROOT / "include" / "FDAS.hpp").stat().st_mtime):
        return DRIVER
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(DRIVER_SRC), f"-L{PKG}", "-lfdas_gb300",
           f"-Wl,-rpath,{PKG}", "-o", str(DRIVER)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stderr)
        raise RuntimeError("C++ driver build failed")
    return DRIVER


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv)
    print(LIB)
