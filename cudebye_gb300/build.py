"""Build recipe of the native engine: nvcc for sm_103a, in-tree outputs.

Produces, under ``cudebye_gb300/_build/``:

* ``libcudebye.so`` — the C-ABI library (include/cudebye.h)
* ``cudebye`` — the command-line drop-in for ``cuDebye.exe <file.deb>``

Translation units are compiled in parallel and skipped when up to date.
``python -m cudebye_gb300.build`` builds from the command line.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-Wall", "-I", INCLUDE]
# Per-file flags. hist.cu must never contract the reference's unfused FP32
# distance arithmetic into FMAs (it also uses explicit _rn intrinsics).
EXTRA = {"hist.cu": ["--fmad=false"], "hist_noalloc.cu": ["--fmad=false"]}
LIB_SOURCES = ["hist.cu", "hist_noalloc.cu", "debye.cu", "debye_tc.cu",
               "model.cu", "spatial_sort.cu", "capi.cu", "serve.cu", "debio.cpp",
               "xyz2deb.cpp"]
CLI_SOURCES = ["cli.cpp"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"),
              "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
             if f.endswith((".h", ".cuh"))]
    files.append(os.path.join(INCLUDE, "cudebye.h"))
    return max(os.path.getmtime(f) for f in files)


def _compile(src, hdr_mtime, force):
    s = os.path.join(CSRC, src)
    o = os.path.join(OUT, src + ".o")
    if (not force and os.path.exists(o)
            and os.path.getmtime(o) >= max(os.path.getmtime(s), hdr_mtime)):
        return o
    cmd = [nvcc(), *ARCH, *COMMON, *EXTRA.get(src, []), "-c", s, "-o", o]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd),
                                                           r.stderr))
    return o


def build(force=False, verbose=False):
    """Compile the engine; returns the path of libcudebye.so."""
    os.makedirs(OUT, exist_ok=True)
    hdr = _deps()
    with cf.ThreadPoolExecutor(max_workers=len(LIB_SOURCES) + 1) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr, force),
                           LIB_SOURCES + CLI_SOURCES))
    lib = os.path.join(OUT, "libcudebye.so")
    lib_objs = objs[:len(LIB_SOURCES)]
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < max(
            os.path.getmtime(o) for o in lib_objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *lib_objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr)
    cli = os.path.join(OUT, "cudebye")
    if force or not os.path.exists(cli) or os.path.getmtime(cli) < max(
            os.path.getmtime(lib), os.path.getmtime(objs[-1])):
        cmd = [nvcc(), *ARCH, "-o", cli, objs[-1], "-L", OUT, "-lcudebye",
               "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("CLI link failed:\n%s" % r.stderr)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
