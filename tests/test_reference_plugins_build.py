"""Every model plugin of CUDIMOT's tree compiles, unchanged, into this
library's kernels (the drop-in promise of the plugin surface).

Runs where CUDIMOT's source tree is present (skipped elsewhere). Each
plugin directory is compiled as it lies in the tree through
cudimot_gb300/build.py's compile check: the device module with every kernel
of the library at one lane count, the plugin included in CUDIMOT's order
(functions_gpu.h, modelparameters.h, macro_numerical.h, modelfunctions.h).
Plugin macros such as NODDI-Watson's `#define H 0.4` must not reach any
name of the kernels or of the headers included after the plugin."""
import concurrent.futures as cf
import os

import pytest

from cudimot_gb300 import build
from oracle import build_oracle


def test_every_cudimot_plugin_compiles():
    ref = build_oracle.reference_tree()
    if not ref:
        pytest.skip("CUDIMOT's source tree is not present")
    root = os.path.join(ref, "mymodels")
    models = sorted(d for d in os.listdir(root)
                    if os.path.isfile(os.path.join(root, d, "modelfunctions.h")))
    assert len(models) >= 18
    with cf.ThreadPoolExecutor(min(8, os.cpu_count() or 1)) as ex:
        errs = dict(zip(models, ex.map(lambda m: build.check_plugin(os.path.join(root, m)), models)))
    failed = {m: e for m, e in errs.items() if e}
    assert not failed, "\n\n".join(f"{m}:\n{e[-1500:]}" for m, e in failed.items())
