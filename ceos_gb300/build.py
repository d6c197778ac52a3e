"""Compile the CUDA library in-tree for sm_103a, and the pybind11 module.

    python -m ceos_gb300.build            # -> ceos_gb300/_lib/libceos_gb300.so
                                          #    ceos_gb300/_lib/CEOs<ext suffix>

Every translation unit under ceos_gb300/csrc is compiled in parallel with
nvcc (one -gencode, sm_103a) and linked into one shared library that exports
the C ABI declared in include/ceos_gb300.h. Objects go to ceos_gb300/_build.

The drop-in Python module `CEOs` (ceos_gb300/pybind/ceos_module.cpp, the
reference's pybind11 module name and bindings) is compiled with g++ against
pybind11's headers - from the pybind11 package, or the copy that PyTorch
ships in its include directory - and links the library above;
`import CEOs` works with ceos_gb300/_lib on the module search path.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libceos_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--extended-lambda", "-Xcompiler", "-fPIC,-O3",
         "-diag-suppress", "177"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CEOs GPU library needs the CUDA toolkit to build")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_digest() -> str:
    h = hashlib.sha1()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cuh", ".h")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(fh.read())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def _compile(src: str, digest: str, force: bool) -> str:
    obj = os.path.join(BUILD, src[:-3] + ".o")
    stamp = obj + ".stamp"
    path = os.path.join(CSRC, src)
    with open(path, "rb") as fh:
        key = digest + hashlib.sha1(fh.read()).hexdigest()
    if not force and os.path.exists(obj) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read() == key:
                return obj
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as fh:
        fh.write(key)
    return obj


PYMOD_SRC = os.path.join(HERE, "pybind", "ceos_module.cpp")


def pymodule_path() -> str:
    return os.path.join(LIBDIR, "CEOs" + sysconfig.get_config_var("EXT_SUFFIX"))


def _pybind11_include() -> str:
    try:
        import pybind11

        return pybind11.get_include()
    except ImportError:
        pass
    import importlib.util

    spec = importlib.util.find_spec("torch")
    if spec and spec.origin:
        inc = os.path.join(os.path.dirname(spec.origin), "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    raise RuntimeError("pybind11 headers not found (neither the pybind11 package nor PyTorch's copy)")


def build_pymodule(force: bool = False) -> str:
    """Compile the `CEOs` pybind11 module against libceos_gb300.so."""
    out = pymodule_path()
    deps = [PYMOD_SRC, LIB, os.path.join(ROOT, "include", "ceos_gb300.h")]
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
        return out
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
           "-I" + sysconfig.get_paths()["include"], "-I" + _pybind11_include(),
           "-I" + os.path.join(ROOT, "include"), PYMOD_SRC, "-o", out,
           "-L" + LIBDIR, "-lceos_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the CEOs module failed:\n{r.stdout}\n{r.stderr}")
    return out


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    digest = _headers_digest()
    srcs = _sources()
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, digest, force), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-Xlinker", "--no-undefined", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_pymodule(force)
    if verbose:
        print(LIB)
        print(pymodule_path())
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
