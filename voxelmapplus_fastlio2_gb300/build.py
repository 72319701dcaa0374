"""In-tree build of the native parts (no cmake, no setuptools).

* ``_build/libvmp.so``        CUDA kernels + C ABI, nvcc for sm_103a only.
* ``_build/libvmp_synth.so``  host C++ synthetic sequence generator.

Translation units compile in parallel; the link is one nvcc call.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(ROOT, "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no contraction of double/float multiply-add pairs, so the
# device reproduces the reference's (x86-64, no FMA) rounding of every
# expression that feeds a voxel key, a gate or a float output.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC", "-I" + INC,
              "-I" + CSRC, "--expt-relaxed-constexpr"]

CU_SOURCES = [
    "vmp_api.cu",
    "k_sort.cu",
    "k_points.cu",
    "k_filter.cu",
    "k_predict.cu",
    "k_iekf.cu",
    "k_map.cu",
    "k_merge.cu",
    "k_fit.cu",
    "k_std.cu",
    "vmp_noalloc.cu",
    "vmp_server.cu",
]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout)
        raise RuntimeError("build step failed: " + os.path.basename(cmd[-1]))
    return r.stdout


def build_synth():
    os.makedirs(OUT, exist_ok=True)
    out = os.path.join(OUT, "libvmp_synth.so")
    src = os.path.join(CSRC, "synth.cpp")
    if os.path.exists(out) and os.path.getmtime(out) > os.path.getmtime(src):
        return out
    _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-I" + INC, "-o", out, src])
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_vmp(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INC, "vmp.h"))
    objs = []
    jobs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s.replace(".cu", ".o"))
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [NVCC] + ARCH + NVCC_FLAGS + list(extra) + ["-rdc=false", "-c", "-o", obj, src]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    so = os.path.join(OUT, "libvmp.so")
    if _stale(so, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", so] + objs + ["-lcudart", "-lpthread"])
    return so


def build_all(verbose=False):
    build_synth()
    return build_vmp(verbose=verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
