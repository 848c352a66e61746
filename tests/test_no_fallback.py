"""The product path never routes through the oracle or a CPU fallback.

* no module of the package imports `oracle`, and no C/C++/CUDA source of the
  package includes a file from `oracle/`;
* a model library that was never built is an error at load time, not a
  silent substitute.
"""
import ast
import os
import re

import pytest

from cudimot_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cudimot_gb300")


def _files(exts):
    for d, _, names in os.walk(PKG):
        if os.sep + "_" in d[len(PKG):]:   # build outputs (_build, _lib, _tune)
            continue
        for n in names:
            if n.endswith(exts):
                yield os.path.join(d, n)


def test_package_python_does_not_import_oracle():
    bad = []
    for f in _files((".py",)):
        tree = ast.parse(open(f).read(), f)
        for node in ast.walk(tree):
            names = []
            if isinstance(node, ast.Import):
                names = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom) and node.module:
                names = [node.module]
            bad += [(f, n) for n in names if n == "oracle" or n.startswith("oracle.")]
    assert not bad, bad


def test_package_sources_do_not_include_oracle():
    inc = re.compile(r'#\s*include\s*[<"][^>"]*oracle/')
    bad = [f for f in _files((".cu", ".cuh", ".cpp", ".h", ".hpp"))
           if inc.search(open(f, errors="replace").read())]
    assert not bad, bad


def test_missing_library_is_an_error():
    with pytest.raises(capi.CdmError, match="not built"):
        capi.load_library("No_Such_Model")
