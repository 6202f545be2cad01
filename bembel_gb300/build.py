"""Build the in-tree shared library bembel_gb300/_build/libbembel_gb300.so.

CUDA sources are compiled for sm_103a only (GB300) with nvcc; the host setup
is plain C++17. Translation units compile in parallel; the build is skipped
when the library is newer than every source and header.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libbembel_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the bembel_gb300 CUDA library cannot be built")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    deps = cu + cpp + glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    return cu, cpp, deps


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    _, _, deps = _sources()
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OUT, exist_ok=True)
    cu, cpp, _ = _sources()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
    jobs = []
    for src in cu:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        jobs.append([nvcc] + ARCH + common + ["-lineinfo", "-diag-suppress", "1444", "-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        jobs.append([nvcc] + common + ["-Xcompiler", "-pthread", "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return cmd[-1]

    with ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 2))) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    link = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static", "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
