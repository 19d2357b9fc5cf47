"""Build recipe for the in-tree native libraries (no cmake).

    libdim3gpu.so  CUDA kernels + C ABI (nvcc, sm_103a only)
    libdim3gen.so  seeded workload generators (gcc, OpenMP)

The CUDA translation units compile in parallel to objects under _build/,
then link into one shared library.  Both libraries are written next to this
file; `python build.py` builds them.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
GPU_SO = os.path.join(HERE, "libdim3gpu.so")
GEN_SO = os.path.join(HERE, "libdim3gen.so")
GPU_TUS = ["dim3gpu.cu", "batch.cu", "tune.cu", "noalloc.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _sources(ext):
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(ext)]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _obj(tu):
    return os.path.join(OBJ, tu.replace(".cu", ".o"))


def commands(force=False):
    """Two stages: [compile commands], [link commands]."""
    compile_cmds, link_cmds = [], []
    headers = _sources(".cuh") + _sources(".h") + [os.path.join(REPO, "include", "dim3gpu.h")]
    objs = []
    for tu in GPU_TUS:
        src, obj = os.path.join(CSRC, tu), _obj(tu)
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            compile_cmds.append([_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj])
    if force or compile_cmds or _stale(GPU_SO, objs):
        link_cmds.append([_nvcc()] + ARCH + ["-shared"] + objs + ["-o", GPU_SO])
    gen_deps = [os.path.join(CSRC, "dim3gen.c"), os.path.join(CSRC, "dim3gen.h")]
    if force or _stale(GEN_SO, gen_deps):
        compile_cmds.append(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                             os.path.join(CSRC, "dim3gen.c"), "-o", GEN_SO])
    return compile_cmds, link_cmds


def run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
    if failed:
        msg = "\n".join("$ " + " ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("native build failed:\n" + msg)


def build(force=False):
    os.makedirs(OBJ, exist_ok=True)
    compile_cmds, link_cmds = commands(force)
    run_parallel(compile_cmds)
    run_parallel(link_cmds)
    return GPU_SO, GEN_SO


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built", GPU_SO, GEN_SO)
