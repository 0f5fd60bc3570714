"""Builds libfasttau.so in-tree (fast_gb300/_build/) with nvcc for sm_103a.

The translation units compile in parallel; the library links the CUDA
runtime statically so it loads beside any torch build.  Rebuilds only when a
source or header is newer than the library.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfasttau.so")
CLI = os.path.join(OUT, "fast")  # the `fast tau` command-line drop-in

CUDA_SOURCES = ["kern_f64.cu", "kern_f32.cu", "kern_misc.cu", "tau_host.cu", "noalloc.cu", "ccl.cu", "serve.cu",
                "volume_ops.cu", "alpha.cu"]
CXX_SOURCES = ["gen.cpp", "tiff_folder.cpp"]
CLI_SOURCE = "fast_cli.cpp"
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfasttau.so")


def _inputs():
    files = [os.path.join(CSRC, f) for f in CUDA_SOURCES + CXX_SOURCES + [CLI_SOURCE]]
    files += glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    files += glob.glob(os.path.join(CSRC, "*.inc"))
    files += glob.glob(os.path.join(INCLUDE, "*.h"))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI))
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-I", INCLUDE, "-I", CSRC] + os.environ.get("FAST_TAU_NVCC_FLAGS", "").split()
    procs, objs = [], []
    for src in CUDA_SOURCES:
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [nvcc, *GENCODE, "-lineinfo", *common, "-Xcompiler", "-fPIC,-fvisibility=hidden",
               "-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    for src in CXX_SOURCES:
        obj = os.path.join(OUT, src.replace(".cpp", ".o"))
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off",
               "-I", INCLUDE, "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode:
            failed.append(" ".join(cmd))
    if failed:
        raise RuntimeError("compilation failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *GENCODE, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    # The CLI links the library from its own directory.
    tmp = CLI + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-I", INCLUDE, os.path.join(CSRC, CLI_SOURCE), "-o", tmp,
           "-L", OUT, "-lfasttau", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode:
        raise RuntimeError("CLI build failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
