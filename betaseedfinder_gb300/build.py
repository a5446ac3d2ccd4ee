"""Build libbsf.so and bsf_worker for sm_103a with nvcc (in-tree, parallel).

Outputs go to betaseedfinder_gb300/_build/. FP64 exactness flags: no FMA
contraction (--fmad=false), IEEE division/sqrt, no flush-to-zero.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
CU_SOURCES = ["bsf_stage0.cu", "bsf_stage0_fast.cu", "bsf_coarse.cu", "bsf_coarse_fast.cu", "bsf_exact.cu",
              "bsf_sweep.cu", "bsf_probe.cu", "bsf_api.cu", "bsf_noalloc.cu", "bsf_server.cu"]
LIB = os.path.join(BUILD, "libbsf.so")
WORKER = os.path.join(BUILD, "bsf_worker")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "--fmad=false", "--prec-div=true", "--prec-sqrt=true", "--ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    "-I", os.path.join(ROOT, "include"),
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))] + \
        [os.path.join(ROOT, "include", "bsf.h")]


def build(verbose=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = _headers()
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([cc, *NVCC_FLAGS, *extra_flags, "-c", s, "-o", o])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed for %s" % cmd[-3])
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        subprocess.check_call([cc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", tmp, *objs,
                               "-lcudart", "-lpthread"])
        os.replace(tmp, LIB)
    wsrc = [os.path.join(CSRC, "bsf_worker.cpp"), os.path.join(CSRC, "bsf_hunt.cpp")]
    if _stale(WORKER, wsrc + [LIB, os.path.join(ROOT, "include", "bsf.h")]):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-o", WORKER, *wsrc, "-L" + BUILD, "-lbsf",
                               "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
