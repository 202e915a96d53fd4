"""Build the CUDA library libanneal_gb300.so in-tree for sm_103a (GB300).

The translation units under csrc/ are compiled in parallel with nvcc and linked into
anneal_gb300/_lib/libanneal_gb300.so. ``python -m anneal_gb300.build`` runs it;
``--debug`` builds the bounds-checked variant (-DANL_DEBUG=1, ANL_IN_RANGE in
csrc/anl_common.cuh) into anneal_gb300/_lib_debug/, which ANL_DEBUG_LIB=1 loads.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libanneal_gb300.so")
DEBUG_DIR = os.path.join(HERE, "_lib_debug")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.isfile(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build anneal_gb300")


def _stale(obj, deps):
    if not os.path.isfile(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=(), debug=False):
    out_dir = DEBUG_DIR if debug else OUT_DIR
    lib = os.path.join(out_dir, "libanneal_gb300.so")
    if debug:
        extra = (*extra, "-DANL_DEBUG=1")
    os.makedirs(os.path.join(out_dir, "obj"), exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [
        os.path.join(os.path.dirname(HERE), "include", "anneal_gb300.h")]
    exe = nvcc()
    jobs = []
    for src in srcs:
        obj = os.path.join(out_dir, "obj", os.path.basename(src)[:-3] + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        tmp = obj + f".{os.getpid()}.tmp"
        cmd = [exe, *ARCH, *FLAGS, *extra, "-c", src, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        os.replace(tmp, obj)
        return src, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for src, err in ex.map(compile_one, jobs):
            if verbose and err.strip():
                print(f"[{os.path.basename(src)}]\n{err}", file=sys.stderr)
    objs = [os.path.join(out_dir, "obj", os.path.basename(s)[:-3] + ".o") for s in srcs]
    if force or jobs or not os.path.isfile(lib):
        tmp = lib + f".{os.getpid()}.tmp"
        subprocess.check_call([exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, debug="--debug" in sys.argv))
