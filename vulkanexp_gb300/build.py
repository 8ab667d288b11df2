"""Builds libddgi_gb300.so in-tree with nvcc for sm_103a.

Each .cu translation unit is compiled in parallel to an object file under
vulkanexp_gb300/_build/, then linked into vulkanexp_gb300/_lib/libddgi_gb300.so
(the CUDA runtime is linked statically).  Host code is compiled with
-ffp-contract=off: the ray-direction table and instance inverses computed on
the host are part of the hit-ID contract.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libddgi_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-warn-spills"]
SOURCES = ["lbvh.cu", "trace.cu", "wavefront.cu", "blend.cu", "blend_tc.cu", "adjoint.cu", "ddgi_api.cu",
           "noalloc.cu", "batch.cu", "schedule.cu", "gather.cu", "wide.cu", "sah.cu", "blend_shared.cu", "sbvh.cu", "sky.cu",
           "gbuild.cu"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
    if not _stale(obj, [src] + _headers() + [__file__]):
        return obj
    tmp = obj + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", tmp]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    if verbose and (r.stdout or r.stderr):
        sys.stdout.write(r.stdout + r.stderr)
    os.replace(tmp, obj)
    return obj


def build(verbose=False, force=False):
    """Compile every CUDA translation unit and link the shared library.
    Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    if force:
        for s in srcs:
            o = os.path.join(BUILD, os.path.splitext(os.path.basename(s))[0] + ".o")
            if os.path.exists(o):
                os.remove(o)
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 1)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
