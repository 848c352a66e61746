"""Build the library from CUDIMOT's own, unchanged plugins (test
infrastructure: the drop-in parity tests run these libraries on the GPU).

    python oracle/build_dropin.py --reference CUDIMOT_TREE   # device halves + host halves
    python oracle/build_dropin.py                             # host halves only

The library's split build (cudimot_gb300/build.py) is used: where CUDIMOT's
source tree is present, the device half of each library (every kernel, as a
sm_103a cubin) is compiled against the plugin directory as it lies in the
tree, next to the generated model description, into
oracle/_ref/dropin/<Model>_<eval>/. The host half is compiled from those two
files alone, on whichever machine runs the tests; it embeds the cubin.
Nothing of the tree is copied: only compiled modules and generated headers
land in oracle/_ref/.

The plugins and the precision each is evaluated in: CUDIMOT's NODDI-Watson
closed forms cancel terms of ~1e10 and are usable in double only, so it is
built with --eval double (and once in float, to report what single precision
does to it); NODDI-Bingham (its signal misses the single-precision bound by
two orders of magnitude) and the SSFP model are built in double as well.
"""
import argparse
import concurrent.futures as cf
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from cudimot_gb300 import build  # noqa: E402

OUT = os.path.join(HERE, "_ref", "dropin")
DROPIN = (("Ball_1_Stick", "float"), ("NODDI_Watson", "double"), ("NODDI_Watson", "float"),
          ("DiffusionTensor", "float"), ("Ball_2_Sticks", "float"), ("NODDI_Bingham", "double"),
          ("toymodel", "float"), ("Ball_2_Sticks_1Shell_SSFP", "double"))


def outdir(model, eval_type):
    return os.path.join(OUT, f"{model}_{eval_type}")


def lib_path(model, eval_type):
    return build.split_lib_path(outdir(model, eval_type))


def available(model, eval_type):
    d = outdir(model, eval_type)
    return all(os.path.exists(os.path.join(d, f)) for f in ("cdm_module.cubin", "cdm_model_desc.h"))


def build_all(reference=None, jobs=None):
    errors = {}
    jobs = jobs or min(8, os.cpu_count() or 1)
    if reference:
        def dev(t):
            m, ev = t
            # no source-line tables: the modules travel with the tests
            return build.split_device(os.path.join(reference, "mymodels", m), outdir(m, ev),
                                      name=m, eval_type=ev, lineinfo=False)
        with cf.ThreadPoolExecutor(jobs) as ex:
            for out, err in ex.map(dev, DROPIN):
                if err:
                    errors[out] = err
    todo = [(m, ev) for m, ev in DROPIN if available(m, ev)]
    with cf.ThreadPoolExecutor(jobs) as ex:
        for out, err in ex.map(lambda t: build.split_host(outdir(*t)), todo):
            if err:
                errors[out] = err
    return errors


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="CUDIMOT source tree")
    a = ap.parse_args()
    errs = build_all(a.reference)
    for k, v in errs.items():
        print(f"FAILED {k}\n{v}", file=sys.stderr)
    sys.exit(1 if errs else 0)
