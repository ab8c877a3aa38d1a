"""In-tree build of the CUDA library for sm_103a (GB300).

``python -m simkit_gb300.build`` compiles each translation unit of
``simkit_gb300/csrc`` in parallel with nvcc (one -gencode, sm_103a) and links
``simkit_gb300/_build/libsimkit_gb300.so`` against the shared CUDA runtime.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsimkit_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def build_library(verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    procs = []
    objs = []
    t0 = time.time()
    for f in cu:
        obj = os.path.join(OUT_DIR, f + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", os.path.join(CSRC, f), "-o", obj]
        procs.append((f, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    for f in cpp:
        obj = os.path.join(OUT_DIR, f + ".o")
        cmd = ["g++", *CXX_FLAGS, "-c", os.path.join(CSRC, f), "-o", obj]
        procs.append((f, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for f, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append((f, text))
        elif verbose and text.strip():
            print(f"--- {f}\n{text}")
    if failed:
        msg = "\n".join(f"--- {f}\n{t}" for f, t in failed)
        raise RuntimeError(f"CUDA build failed:\n{msg}")
    link = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", LIB, *objs,
            "-Xlinker", "-rpath,$ORIGIN", "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    if verbose:
        print(f"built {LIB} in {time.time() - t0:.1f} s")
    return LIB


if __name__ == "__main__":
    build_library(verbose="-v" in sys.argv)
