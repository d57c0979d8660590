"""Build the GB300 ADS library (libadsgpu.so) in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into
ads_mpi_gb300/libadsgpu.so with the static CUDA runtime.  The driver API
(cuTensorMapEncodeTiled) is resolved at run time, so the library links
against nothing beyond the C/C++ runtime and can be loaded on a machine
without a GPU (for symbol checks).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libadsgpu.so")
SOURCES = ["ads_api.cu", "k_assemble.cu", "k_assemble_oil.cu", "k_assemble_df.cu", "k_general.cu", "k_sweep.cu", "k_csweep.cu", "k_misc.cu", "noalloc.cu", "setup.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src, verbose):
    f = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden"]
    if src.endswith(".cu"):
        f += ARCH + ["-lineinfo"]
        if verbose:
            f += ["-Xptxas", "-v"]
    return f


def _compile(src, verbose):
    out = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + _flags(src, verbose) + ["-c", os.path.join(CSRC, src), "-o", out]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++"] + cmd[1:]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, r.returncode, r.stdout + r.stderr, out


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "ads_gpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, jobs=None):
    """Compile libadsgpu.so if any source is newer than it; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 1)
    logs = []
    objs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        for src, rc, log, out in ex.map(lambda s: _compile(s, verbose), SOURCES):
            logs.append((src, log))
            if rc != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{log}")
            objs.append(out)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared"] + ARCH + ["-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        for src, log in logs:
            if log.strip():
                print(f"== {src}\n{log}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
