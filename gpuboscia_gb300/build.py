"""In-tree build of libgpuboscia_gb300.so for sm_103a.

Every translation unit compiles in parallel (one ``-gencode``), then one link.
Objects are rebuilt only when a source or header is newer. The CUDA runtime is
linked statically so the library loads without a library path.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libgpuboscia_gb300.so"
INCLUDE = ROOT / "include"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", ARCH,
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall"]


def _cuda_home() -> pathlib.Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return pathlib.Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return pathlib.Path(nvcc).resolve().parent.parent
    return pathlib.Path("/usr/local/cuda")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _deps():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.rglob("*.h"))


def _stale(target: pathlib.Path, inputs) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _compile(src: pathlib.Path, obj: pathlib.Path, cuda: pathlib.Path, extra) -> str:
    if src.suffix == ".cu":
        cmd = [str(cuda / "bin" / "nvcc"), *NVCC_FLAGS, *extra, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-I", str(INCLUDE), "-I", str(cuda / "include"),
               "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose: bool = False, force: bool = False, extra_nvcc=()) -> pathlib.Path:
    """Compile and link the library; returns its path."""
    cuda = _cuda_home()
    BUILD.mkdir(parents=True, exist_ok=True)
    deps = _deps()
    jobs = []
    objs = []
    for src in _sources():
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *deps]):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            futs = {ex.submit(_compile, s, o, cuda, list(extra_nvcc)): s for s, o in jobs}
            for f in cf.as_completed(futs):
                log = f.result()
                if verbose and log:
                    print(log)
    if force or jobs or _stale(LIB, objs):
        cmd = [str(cuda / "bin" / "nvcc"), "-shared", ARCH, "-cudart", "static", "-o", str(LIB),
               *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
