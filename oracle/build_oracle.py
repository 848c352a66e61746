"""Build the CPU oracle (test infrastructure, never part of the library).

    python oracle/build_oracle.py                 # oracle for the shipped plugins
    python oracle/build_oracle.py --reference DIR # also CUDIMOT's own plugins

The oracle (oracle_capi.cpp + cudimot_oracle.hpp) is compiled once per model
plugin with g++ into oracle/_build/liboracle_<Model>.so. With --reference,
the same sources are compiled against each plugin directory DIR/<Model>
of the CUDIMOT tree (its unchanged modelfunctions.h / modelparameters.*)
into oracle/_ref/libref_<Model>.so; those libraries produce the golden
fixtures that pin the shipped plugins to CUDIMOT's. Nothing is copied out of
the reference tree; only the compiled libraries land in oracle/_ref/.

Flags: -O2, OpenMP, no -march (the same code builds on x86 and Arm) and
-ffp-contract=off so both machines round identically.
"""
import argparse
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# Where this recipe looks for CUDIMOT's source tree unless CUDIMOT_REFERENCE
# names another (the tree exists only on the build machine).
DEFAULT_REFERENCE = "/root/reference"


def reference_tree():
    """CUDIMOT's source tree if it is present (CUDIMOT_REFERENCE, else the
    default location), else None."""
    ref = os.environ.get("CUDIMOT_REFERENCE", DEFAULT_REFERENCE)
    return ref if ref and os.path.isdir(os.path.join(ref, "mymodels")) else None
PRELUDE = os.path.join(ROOT, "cudimot_gb300", "csrc", "prelude")
KERNELS = os.path.join(ROOT, "cudimot_gb300", "csrc", "kernels")
INCLUDE = os.path.join(ROOT, "include")
MODELS = os.path.join(ROOT, "cudimot_gb300", "mymodels")


def shipped_models():
    return sorted(d for d in os.listdir(MODELS)
                  if os.path.isfile(os.path.join(MODELS, d, "modelfunctions.h")))


def compile_one(model_dir, name, out):
    os.makedirs(os.path.dirname(out), exist_ok=True)
    deps = [os.path.join(HERE, "oracle_capi.cpp"), os.path.join(HERE, "cudimot_oracle.hpp"),
            os.path.join(HERE, "host_prelude.h")]
    deps += [os.path.join(PRELUDE, f) for f in os.listdir(PRELUDE)]
    deps += [os.path.join(model_dir, f) for f in os.listdir(model_dir)
             if f.endswith((".h", ".cc"))]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out, None
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-w", f'-DCDM_MODEL_NAME="{name}"',
           "-I", HERE, "-I", PRELUDE, "-I", KERNELS, "-I", INCLUDE, "-I", model_dir,
           os.path.join(HERE, "oracle_capi.cpp"), "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, r.stderr[-4000:]
    os.replace(out + ".tmp", out)
    return out, None


def build(models=None, reference=None, ref_models=None, jobs=None):
    jobs = jobs or min(8, os.cpu_count() or 1)
    todo = []
    for m in (models or shipped_models()):
        todo.append((os.path.join(MODELS, m), m,
                     os.path.join(HERE, "_build", f"liboracle_{m}.so")))
    if reference:
        ref_dir = os.path.join(reference, "mymodels")
        names = ref_models or sorted(
            d for d in os.listdir(ref_dir)
            if os.path.isfile(os.path.join(ref_dir, d, "modelfunctions.h")))
        for m in names:
            todo.append((os.path.join(ref_dir, m), m, os.path.join(HERE, "_ref", f"libref_{m}.so")))
    errors = {}
    with cf.ThreadPoolExecutor(jobs) as ex:
        for out, err in ex.map(lambda t: compile_one(*t), todo):
            if err:
                errors[out] = err
    return errors


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="CUDIMOT source tree")
    ap.add_argument("--models", nargs="*", default=None)
    ap.add_argument("--ref-models", nargs="*", default=None)
    a = ap.parse_args()
    errors = build(a.models, a.reference, a.ref_models)
    for out, err in errors.items():
        print(f"FAILED {out}\n{err}", file=sys.stderr)
    sys.exit(1 if errors else 0)


if __name__ == "__main__":
    main()
