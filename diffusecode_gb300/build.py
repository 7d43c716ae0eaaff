"""Builds libdiscus_gpu.so in-tree (diffusecode_gb300/lib/) with nvcc for
sm_103a.  Translation units compile in parallel; no CMake, no torch.

    python -m diffusecode_gb300.build
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libdiscus_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _compile(args):
    src, obj, kind = args
    if kind == "cu":
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, r.returncode, r.stdout + r.stderr


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    cu, cpp = sources()
    jobs = []
    for f in cu:
        jobs.append((os.path.join(CSRC, f), os.path.join(OBJ_DIR, f + ".o"), "cu"))
    for f in cpp:
        jobs.append((os.path.join(CSRC, f), os.path.join(OBJ_DIR, f + ".o"), "cpp"))
    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(_compile, jobs))
    failed = False
    for src, rc, log in results:
        if rc != 0 or (verbose and log.strip()):
            sys.stderr.write(f"--- {os.path.basename(src)} (rc={rc})\n{log}\n")
        failed = failed or rc != 0
    if failed:
        raise RuntimeError("libdiscus_gpu build failed")
    objs = [j[1] for j in jobs]
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("libdiscus_gpu link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
