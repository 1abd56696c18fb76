"""Builds the CUDA extension libks.so in-tree (kynema_sgf_gb300/_build/).

Each translation unit is compiled by nvcc for sm_103a in parallel, then
linked into one shared library with the C ABI of include/ks.h.  Nothing is
installed outside the package directory.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
SOURCES = ["ks_host.cpp", "ks_adjoint_host.cpp", "ks_io.cpp", "ks_kernels.cu", "ks_godunov.cu", "ks_mol.cu", "ks_implicit.cu", "ks_temperature.cu", "ks_mg.cu", "ks_adjoint.cu", "ks_noalloc.cu", "ks_probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    lang = ["-x", "cu"] if src.endswith(".cu") else []
    cmd = [nvcc()] + ARCH + FLAGS + extra + lang + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libks.so")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "ks.h")]
    exe = driver_path()
    if (os.path.exists(lib) and os.path.exists(exe) and not extra
            and all(min(os.path.getmtime(lib), os.path.getmtime(exe)) >= os.path.getmtime(d) for d in deps)):
        return lib
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, lib)
    # deck-compatible driver executable over the C ABI (reference: src/main.cpp)
    cmd = [nvcc(), "-O2", "-std=c++17", os.path.join(CSRC, "ks_main.cpp"), "-L" + OUT, "-lks", "-Xlinker", "-rpath",
           "-Xlinker", "$ORIGIN", "-o", exe + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(exe + ".tmp", exe)
    return lib


def driver_path():
    """The ks_run executable: `ks_run <input_file> [param=value ...]`."""
    return os.path.join(OUT, "ks_run")


if __name__ == "__main__":
    print(build(verbose=True, extra=tuple(sys.argv[1:])))
