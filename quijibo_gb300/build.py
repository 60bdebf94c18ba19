"""Build recipe of the CUDA library: every .cu and .cpp under csrc/ compiled
in parallel for sm_103a and linked into _lib/libquijibo_gpu.so (in-tree).

    python -m quijibo_gb300.build [--verbose]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libquijibo_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src, cuda, verbose):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJDIR, src + ".o")
    if src.endswith(".cu"):
        cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-lineinfo", "-O3", "-std=c++17",
               "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", path, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
               "-I" + os.path.join(cuda, "include"), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return src, r.stderr


def build(verbose=False):
    cuda = _cuda_home()
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(2, len(srcs))) as ex:
        for src, log in ex.map(lambda s: _compile(s, cuda, verbose), srcs):
            if verbose and log:
                print("==", src, "\n", log, file=sys.stderr)
    objs = [os.path.join(OBJDIR, s + ".o") for s in srcs]
    cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv))
