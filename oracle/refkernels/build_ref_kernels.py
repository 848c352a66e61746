"""Build CUDIMOT's own GPU kernels for the GB300 (test infrastructure).

    python oracle/refkernels/build_ref_kernels.py --reference CUDIMOT_TREE [--models ...]

Where the CUDIMOT source tree is present: compiles GridSearch.cu,
Levenberg_Marquardt.cu, MCMC.cu, BIC_AIC.cu and getPredictedSignal.cu of the
CUDIMOT tree, unmodified, against a model's unmodified plugin, to sm_103a
cubins in oracle/_ref/<Model>/ (flags of CUDIMOT's Makefile:13-22: -O3,
-maxrregcount 128 for double plugins). FSL's utils/options.h, log.h and
tracer_plus.h are replaced by the stubs in oracle/refkernels/stubs (the
host classes they serve are never run).

On a machine with the GPU but without the CUDIMOT tree, build_harness()
compiles refharness.cpp (driver API) into oracle/_ref/librefharness.so,
which loads those cubins.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REF_OUT = os.path.join(ORACLE, "_ref")
FILES = ("GridSearch", "Levenberg_Marquardt", "MCMC", "BIC_AIC", "getPredictedSignal")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc")


MODELS = ("Ball_1_Stick", "NODDI_Watson", "DiffusionTensor", "Ball_2_Sticks", "NODDI_Bingham")


def build_cubins(reference, models=MODELS, jobs=8):
    todo = []
    for m in models:
        out = os.path.join(REF_OUT, m)
        os.makedirs(out, exist_ok=True)
        for f in FILES:
            src = os.path.join(reference, f + ".cu")
            dst = os.path.join(out, f + ".cubin")
            if os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(src):
                continue
            cmd = [nvcc(), "-cubin", ARCH, "-O3", "-maxrregcount", "128", "-w",
                   "-I", os.path.join(HERE, "stubs"), "-I", reference,
                   "-I", os.path.join(reference, "mymodels", m), src, "-o", dst + ".tmp"]
            todo.append((cmd, dst))

    def run(t):
        cmd, dst = t
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode == 0:
            os.replace(dst + ".tmp", dst)
            return None
        return dst + "\n" + r.stderr[-3000:]

    with cf.ThreadPoolExecutor(jobs) as ex:
        errs = [e for e in ex.map(run, todo) if e]
    return errs


def build_harness():
    src = os.path.join(HERE, "refharness.cpp")
    out = os.path.join(REF_OUT, "librefharness.so")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-I", os.path.join(cuda, "include"),
           "-L", os.path.join(cuda, "lib64", "stubs"), "-L", os.path.join(cuda, "lib64"), "-lcuda",
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return None if r.returncode == 0 else r.stderr[-3000:]


def available(model):
    d = os.path.join(REF_OUT, model)
    return all(os.path.exists(os.path.join(d, f + ".cubin")) for f in FILES)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--models", nargs="*", default=list(MODELS))
    a = ap.parse_args()
    errs = build_cubins(a.reference, a.models)
    for e in errs:
        print("FAILED", e, file=sys.stderr)
    sys.exit(1 if errs else 0)
