"""Builds the engine's CUDA library in-tree: fdtd_method_gb300/libfdtd_gb300.so.

Each .cu file under csrc/ is compiled for sm_103a only (one -gencode), in
parallel, then linked with -shared.  No cmake; needs nvcc and g++.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfdtd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _newest_input():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(HERE, "cpp", f) for f in os.listdir(os.path.join(HERE, "cpp"))]
    files.append(os.path.join(HERE, "..", "include", "fdtd_gb300.h"))
    files.append(os.path.join(HERE, "..", "include", "fdtd_gb300.hpp"))
    files.append(__file__)
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def up_to_date():
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input()


def build(force=False, verbose=False, extra_flags=()):
    if not force and up_to_date():
        return LIB
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + CSRC, "-I" + os.path.join(HERE, "..", "include")]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, *inc, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    build_programs()
    return LIB


CPP = os.path.join(HERE, "cpp")
PROGRAMS = ("fdtd_sample", "convergence_tests", "fdtd_coarray_sample")


def build_programs():
    """C++ programs over the drop-in header include/fdtd_gb300.hpp: the GPU
    twin of the reference's sample driver and its convergence tests."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    inc = os.path.join(HERE, "..", "include")
    for name in PROGRAMS:
        cmd = [cxx, "-O2", "-std=c++17", "-I" + inc, os.path.join(CPP, name + ".cpp"), "-L" + HERE,
               "-lfdtd_gb300", "-Wl,-rpath,$ORIGIN", "-o", os.path.join(HERE, name)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build of %s failed:\n%s" % (name, r.stderr))


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
