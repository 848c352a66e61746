"""The public headers are a C ABI: each compiles on its own and all together
as strict C99 and C11 (gcc -pedantic -Werror) and as C++17, and a plain C
program links against a model library and calls its host-only entry points
(what a cgo, JNI or N-API binding does first); two threads that fail at
the same time each read their own cdm_last_error. No GPU is needed.
"""
import os
import shutil
import subprocess

import pytest

from cudimot_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
HEADERS = sorted(h for h in os.listdir(INC) if h.endswith(".h"))

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None or shutil.which("g++") is None,
                                reason="needs gcc and g++")


def _compile(tmp_path, compiler, std, src, name):
    f = tmp_path / name
    f.write_text(src)
    lang = ["-x", "c++"] if compiler == "g++" else []
    r = subprocess.run([compiler, f"-std={std}", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I", INC, *lang, "-c", str(f), "-o", str(tmp_path / (name + ".o"))],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("compiler,std", [("gcc", "c99"), ("gcc", "c11"), ("g++", "c++17")])
def test_headers_compile(tmp_path, compiler, std):
    for h in HEADERS:
        _compile(tmp_path, compiler, std, f'#include "{h}"\nint main(void) {{ return 0; }}\n',
                 f"one_{h}.c")
    both = "".join(f'#include "{h}"\n' for h in HEADERS) + "int main(void) { return 0; }\n"
    _compile(tmp_path, compiler, std, both, "all.c")


C_PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "cudimot_gb300.h"

int main(void) {
  cdm_model_info info;
  cdm_model_cfg cfg;
  cdm_ctx* ctx = NULL;
  int fixed[CDM_MAX_PARAMS];
  cdm_status bad;
  if (cdm_get_model_info(&info) != CDM_OK) return 2;
  if (cdm_default_cfg(&cfg) != CDM_OK) return 3;
  memset(fixed, 0, sizeof fixed);
  if (cdm_parse_fixed("1,3", fixed) != CDM_OK) return 4;
  printf("name=%s nparams=%d cfp_tsize=%d fixp_tsize=%d\n", info.name, info.nparams,
         info.cfp_tsize, info.fixp_tsize);
  printf("nburn=%d njumps=%d se=%d seed=%llu iter=%d\n", cfg.nburn, cfg.njumps,
         cfg.sampleevery, (unsigned long long)cfg.seed, cfg.iter_levmar);
  printf("fixed=%d%d%d%d%d\n", fixed[0], fixed[1], fixed[2], fixed[3], fixed[4]);
  cfg.nparams = info.nparams - 1;
  bad = cdm_create(&cfg, &ctx);
  printf("bad_create=%d msg=%d\n", (int)bad, cdm_last_error()[0] != 0);
  printf("status=%s\n", cdm_status_string(CDM_BAD_ARG));
  return 0;
}
"""


def test_c_program_links_and_calls(built, tmp_path):
    src = tmp_path / "prog.c"
    src.write_text(C_PROGRAM)
    libdir = os.path.dirname(capi.lib_path("NODDI_Watson"))
    exe = tmp_path / "prog"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", INC, str(src), "-o", str(exe),
                        "-L", libdir, "-lcudimot_NODDI_Watson", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    out = dict(kv.split("=", 1) for line in r.stdout.split("\n") for kv in line.split())
    assert out["name"] == "NODDI_Watson" and out["nparams"] == "5"
    assert out["cfp_tsize"] == "4" and out["fixp_tsize"] == "1"
    # cudimotoptions.h defaults
    assert (out["nburn"], out["njumps"], out["se"], out["seed"], out["iter"]) == \
        ("1000", "1250", "25", "8219", "200")
    assert out["fixed"] == "01010"
    assert out["bad_create"] == "1" and out["msg"] == "1"
    assert out["status"]


THREAD_PROGRAM = r"""
#include <pthread.h>
#include <stdio.h>
#include <string.h>
#include "cudimot_gb300.h"

static pthread_barrier_t bar;
static int ok[2];

static void* create_bad(void* arg) {
  cdm_model_cfg cfg;
  cdm_ctx* ctx = NULL;
  (void)arg;
  cdm_default_cfg(&cfg);
  cfg.nparams = 4;
  int st = cdm_create(&cfg, &ctx);
  pthread_barrier_wait(&bar);   /* both threads have failed */
  ok[0] = st == CDM_BAD_ARG && strstr(cdm_last_error(), "nparams") != NULL &&
          strstr(cdm_last_error(), "Wrong number") == NULL;
  return NULL;
}

static void* parse_bad(void* arg) {
  int fixed[CDM_MAX_PARAMS];
  (void)arg;
  int st = cdm_parse_fixed("9", fixed);
  pthread_barrier_wait(&bar);
  ok[1] = st == CDM_BAD_ARG && strstr(cdm_last_error(), "Wrong number of parameter 9") != NULL;
  return NULL;
}

int main(void) {
  pthread_t a, b;
  pthread_barrier_init(&bar, NULL, 2);
  pthread_create(&a, NULL, create_bad, NULL);
  pthread_create(&b, NULL, parse_bad, NULL);
  pthread_join(a, NULL);
  pthread_join(b, NULL);
  printf("%d %d\n", ok[0], ok[1]);
  return ok[0] && ok[1] ? 0 : 1;
}
"""


def test_last_error_is_per_thread(built, tmp_path):
    """cdm_last_error reports the failure of the calling thread: two threads
    fail differently at the same time and each reads its own message."""
    src = tmp_path / "threads.c"
    src.write_text(THREAD_PROGRAM)
    libdir = os.path.dirname(capi.lib_path("NODDI_Watson"))
    exe = tmp_path / "threads"
    r = subprocess.run(["gcc", "-std=gnu99", "-Wall", "-Werror", "-pthread", "-I", INC, str(src),
                        "-o", str(exe), "-L", libdir, "-lcudimot_NODDI_Watson",
                        f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.stdout, r.stderr)
