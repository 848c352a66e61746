"""Build libcudimot_<Model>.so for sm_103a, in-tree.

    python -m cudimot_gb300.build                 # every plugin in mymodels/
    python -m cudimot_gb300.build --model-dir DIR # any CUDIMOT plugin directory
    python -m cudimot_gb300.build --model-dir DIR --split OUT  # device half only
    python -m cudimot_gb300.build --module-host OUT            # host half of a split build

Like CUDIMOT's Makefile (one binary per mymodels/<Model>), each model plugin
is compiled into its own library: the generic kernels include the plugin's
unchanged modelparameters.h / modelfunctions.h / modelparameters.cc. The
plugin's CFP/FixP block sizes are read from modelparameters.cc into a
generated header so the kernels can size their register arrays at compile
time. Libraries land in cudimot_gb300/_lib/ (git-ignored).

Split build: the device half (every kernel, cdm_module.cu) is compiled
against the plugin into a cubin, next to a generated description of the
model (sizes and hooks, cdm_model_desc.h); the host half (cdm_model.cu with
CDM_MODULE_HOST) is compiled later from the description alone and embeds the
cubin. The two halves can be built on different machines: the plugin's
sources are needed only for the first.

--eval double (-DCDM_EVAL_DOUBLE) evaluates the plugin in double precision:
for plugins whose closed forms are not usable in single precision.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
GENDIR = os.path.join(HERE, "_build")
MODELS = os.path.join(HERE, "mymodels")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found")


def shipped_models():
    return sorted(d for d in os.listdir(MODELS)
                  if os.path.isfile(os.path.join(MODELS, d, "modelfunctions.h")))


def block_sizes(model_dir):
    """CFP_size / FixP_size initialisers of modelparameters.cc."""
    txt = open(os.path.join(model_dir, "modelparameters.cc")).read()
    txt = re.sub(r"//[^\n]*", "", txt)
    out = {}
    for name in ("CFP_size", "FixP_size"):
        m = re.search(name + r"\s*\[\s*\]\s*=\s*\{([^}]*)\}", txt)
        if not m:
            raise ValueError(f"{model_dir}: cannot find MODEL::{name}[] in modelparameters.cc")
        vals = [int(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]
        out[name] = vals
    return out


def sources():
    files = [os.path.join(CSRC, "cdm_model.cu"), os.path.join(CSRC, "cdm_module.cu"),
             os.path.join(ROOT, "include", "cudimot_gb300.h")]
    for sub in ("prelude", "kernels", "host"):
        d = os.path.join(CSRC, sub)
        files += [os.path.join(d, f) for f in sorted(os.listdir(d))]
    return files


def digest(model_dir, flags):
    h = hashlib.sha256()
    for f in sources() + sorted(os.path.join(model_dir, x) for x in os.listdir(model_dir)
                               if x.endswith((".h", ".cc", ".cu", ".hpp"))):
        h.update(f.encode())
        h.update(open(f, "rb").read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def lib_path(name):
    return os.path.join(LIBDIR, f"libcudimot_{name}.so")


def _write_sizes(gen, sizes):
    with open(os.path.join(gen, "cdm_model_sizes.h"), "w") as f:
        f.write("// generated from modelparameters.cc by cudimot_gb300/build.py\n#pragma once\n")
        f.write(f"#define CDM_CFP_TSIZE {sum(sizes['CFP_size'])}\n")
        f.write(f"#define CDM_FIXP_TSIZE {sum(sizes['FixP_size'])}\n")


def _includes(gen, model_dir):
    return ["-I", os.path.join(CSRC, "prelude"), "-I", os.path.join(CSRC, "kernels"),
            "-I", os.path.join(CSRC, "host"), "-I", os.path.join(ROOT, "include"), "-I", gen,
            "-I", model_dir]


def _build_flops(model_dir, gen, fl):
    """Operation-count build of the plugin (host g++; roofline FLOP basis and
    the model description of split builds)."""
    cmd = ["g++", "-O1", "-std=c++17", "-fPIC", "-shared", "-w",
           "-I", os.path.join(CSRC, "prelude"), "-I", os.path.join(CSRC, "host"), "-I", gen,
           "-I", model_dir, os.path.join(CSRC, "host", "cdm_flops.cpp"), "-o", fl + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return (r.stdout + r.stderr)[-6000:]
    os.replace(fl + ".tmp", fl)
    return None


def eval_flags(eval_type):
    if eval_type in (None, "float"):
        return []
    if eval_type == "double":
        return ["-DCDM_EVAL_DOUBLE"]
    raise ValueError("eval must be 'float' or 'double'")


def build_model(model_dir, name=None, extra_flags=(), verbose=False, force=False, eval_type=None):
    model_dir = os.path.abspath(model_dir)
    name = name or os.path.basename(model_dir.rstrip("/"))
    flags = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-shared",
             "-Xcompiler", "-ffp-contract=off"] + eval_flags(eval_type) + list(extra_flags)
    out = lib_path(name)
    stamp = out + ".sha256"
    dig = digest(model_dir, flags)
    if not force and os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == dig:
        return out, None
    gen = os.path.join(GENDIR, name)
    os.makedirs(gen, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    _write_sizes(gen, block_sizes(model_dir))
    # modelparameters.cc defines the MODEL:: size arrays the ABI reports.
    with open(os.path.join(gen, "cdm_model_params.cpp"), "w") as f:
        f.write('#include "modelparameters.cc"\n')
    cmd = [nvcc_path()] + flags + [f'-DCDM_MODEL_NAME="{name}"'] + _includes(gen, model_dir) + [
        os.path.join(CSRC, "cdm_model.cu"), os.path.join(CSRC, "host", "cdm_host.cpp"),
        os.path.join(gen, "cdm_model_params.cpp"),
        "-o", out + ".tmp"]
    if verbose:
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, (r.stdout + r.stderr)[-6000:]
    os.replace(out + ".tmp", out)
    if verbose:
        sys.stderr.write(r.stdout + r.stderr)
    err = _build_flops(model_dir, gen, os.path.join(LIBDIR, f"libcdm_flops_{name}.so"))
    if err:
        return os.path.join(LIBDIR, f"libcdm_flops_{name}.so"), err
    with open(stamp, "w") as f:
        f.write(dig)
    return out, None


HOOK_MACROS = ("CDM_SIGNAL_PAIR", "CDM_SHELL_SERIES", "CDM_SHELL_KEY", "CDM_SHELL_NCOEF",
               "CDM_SHELL_MCOLS", "CDM_MLP_HEAD", "CDM_MLP_NMU", "CDM_MLP_NSIG", "CDM_MLP_GROUPS")


def device_hooks(known, extra):
    """#define lines of the plugin's optional hooks as the device compilation
    of cdm_module.cu sees them (a plugin may define a hook for CUDA only),
    except those already in `known`. extra = (includes, flags) of that
    compilation."""
    includes, flags = extra
    cmd = [nvcc_path(), "-E", "-std=c++17", "-Xcompiler", "-dM"] + list(flags) + list(includes) + \
        [os.path.join(CSRC, "cdm_module.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("macro dump of the device module failed:\n" + r.stderr[-3000:])
    out = ""
    for line in r.stdout.splitlines():
        m = re.match(r"#define (\w+)(\s.*)?$", line)
        if m and m.group(1) in HOOK_MACROS and f"#define {m.group(1)} " not in known:
            out += line.rstrip() + "\n"
    return out


def describe(flops_lib, sizes, name, eval_type=None, extra=((), ())):
    """Text of cdm_model_desc.h from the host build of the plugin (sizes) and
    the device compilation's macros (hooks)."""
    import ctypes
    lib = ctypes.CDLL(flops_lib)
    buf = ctypes.create_string_buffer(1 << 14)
    n = lib.cdm_describe(buf, len(buf))
    if n < 0:
        raise RuntimeError("model description does not fit")
    pad = lambda v: "{" + ", ".join(str(x) for x in (v or [0])) + "}"  # noqa: E731
    txt = ("// generated by cudimot_gb300/build.py from the plugin: the host half of a\n"
           "// split build is compiled with this instead of the plugin\n#pragma once\n")
    txt += buf.value.decode()
    txt += device_hooks(txt, extra)
    txt += f"#define CDM_CFP_SIZES {pad(sizes['CFP_size'])}\n"
    txt += f"#define CDM_FIXP_SIZES {pad(sizes['FixP_size'])}\n"
    if eval_type == "double":
        txt += "#define CDM_EVAL_DOUBLE 1\n"
    txt += f'#define CDM_SPLIT_MODEL_NAME "{name}"\n'
    return txt


def split_device(model_dir, outdir, name=None, eval_type=None, force=False, lineinfo=True):
    """Device half of a split build: outdir/cdm_module.cubin and
    outdir/cdm_model_desc.h from the plugin in model_dir. lineinfo=False
    leaves out the source-line tables (a third of the size)."""
    model_dir = os.path.abspath(model_dir)
    outdir = os.path.abspath(outdir)
    name = name or os.path.basename(model_dir.rstrip("/"))
    os.makedirs(outdir, exist_ok=True)
    flags = ["-O3", "-std=c++17", ARCH] + (["-lineinfo"] if lineinfo else []) + ["-cubin"] + \
        eval_flags(eval_type)
    cubin = os.path.join(outdir, "cdm_module.cubin")
    stamp = cubin + ".sha256"
    dig = digest(model_dir, flags + [name])
    if not force and os.path.exists(cubin) and os.path.exists(stamp) and open(stamp).read() == dig:
        return cubin, None
    gen = os.path.join(outdir, "gen")
    os.makedirs(gen, exist_ok=True)
    sizes = block_sizes(model_dir)
    _write_sizes(gen, sizes)
    fl = os.path.join(gen, "libcdm_describe.so")
    err = _build_flops(model_dir, gen, fl)
    if err:
        return fl, err
    with open(os.path.join(outdir, "cdm_model_desc.h"), "w") as f:
        f.write(describe(fl, sizes, name, eval_type,
                         (_includes(gen, model_dir), [ARCH] + eval_flags(eval_type))))
    cmd = [nvcc_path()] + flags + _includes(gen, model_dir) + [
        os.path.join(CSRC, "cdm_module.cu"), "-o", cubin + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return cubin, (r.stdout + r.stderr)[-6000:]
    os.replace(cubin + ".tmp", cubin)
    with open(stamp, "w") as f:
        f.write(dig)
    return cubin, None


def check_plugin(model_dir, eval_type=None, lanes=2):
    """Compile check of a plugin: the device module with one lane count
    (every kernel, cubin discarded). Returns None or the compiler's error."""
    import tempfile
    model_dir = os.path.abspath(model_dir)
    with tempfile.TemporaryDirectory() as gen:
        _write_sizes(gen, block_sizes(model_dir))
        cmd = [nvcc_path(), "-O3", "-std=c++17", ARCH, "-cubin", f"-DCDM_CHECK_LANES={lanes}"] + \
            eval_flags(eval_type) + _includes(gen, model_dir) + \
            [os.path.join(CSRC, "cdm_module.cu"), "-o", os.path.join(gen, "check.cubin")]
        r = subprocess.run(cmd, capture_output=True, text=True)
    return None if r.returncode == 0 else (r.stdout + r.stderr)[-6000:]


def split_lib_path(outdir):
    return os.path.join(os.path.abspath(outdir), "libcudimot_split.so")


def split_host(outdir, force=False):
    """Host half of a split build: outdir/libcudimot_split.so from
    outdir/cdm_model_desc.h, embedding outdir/cdm_module.cubin."""
    outdir = os.path.abspath(outdir)
    cubin = os.path.join(outdir, "cdm_module.cubin")
    desc = os.path.join(outdir, "cdm_model_desc.h")
    out = split_lib_path(outdir)
    deps = [cubin, desc, os.path.join(CSRC, "cdm_model.cu"), os.path.join(CSRC, "host", "cdm_host.cpp")]
    deps += [os.path.join(CSRC, "host", f) for f in os.listdir(os.path.join(CSRC, "host"))]
    deps += [os.path.join(CSRC, "kernels", "cdm_args.h"), os.path.join(ROOT, "include", "cudimot_gb300.h")]
    if not (os.path.exists(cubin) and os.path.exists(desc)):
        return out, f"{outdir} holds no device module (cdm_module.cubin, cdm_model_desc.h)"
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(map(os.path.getmtime, deps)):
        return out, None
    name = re.search(r'CDM_SPLIT_MODEL_NAME "([^"]*)"', open(desc).read())
    image = os.path.join(outdir, "cdm_module_image.cpp")
    with open(image, "w") as f:
        f.write("// generated by cudimot_gb300/build.py: the device module, embedded\n")
        f.write('__asm__(".section .rodata\\n.balign 64\\n.globl cdm_module_image\\n'
                'cdm_module_image:\\n.incbin \\"' + cubin + '\\"\\n.byte 0\\n.previous\\n");\n')
    cmd = [nvcc_path(), "-O3", "-std=c++17", ARCH, "-Xcompiler", "-fPIC", "-shared",
           "-DCDM_MODULE_HOST", f'-DCDM_MODEL_NAME="{name.group(1) if name else "model"}"',
           "-I", os.path.join(CSRC, "kernels"), "-I", os.path.join(CSRC, "host"),
           "-I", os.path.join(ROOT, "include"), "-I", outdir,
           os.path.join(CSRC, "cdm_model.cu"), os.path.join(CSRC, "host", "cdm_host.cpp"), image,
           "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, (r.stdout + r.stderr)[-6000:]
    os.replace(out + ".tmp", out)
    return out, None


def build_peak(force=False):
    """FP32 FMA probe library (roofline peak)."""
    src = os.path.join(CSRC, "cdm_peak.cu")
    out = os.path.join(LIBDIR, "libcdm_peak.so")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out, None
    os.makedirs(LIBDIR, exist_ok=True)
    cmd = [nvcc_path(), "-O3", ARCH, "-Xcompiler", "-fPIC", "-shared", src, "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, (r.stdout + r.stderr)[-4000:]
    os.replace(out + ".tmp", out)
    return out, None


def build_batch(force=False):
    """Graph batching library over model contexts (include/cdm_batch.h)."""
    src = os.path.join(CSRC, "batch", "cdm_batch.cpp")
    hdr = os.path.join(ROOT, "include", "cdm_batch.h")
    out = os.path.join(LIBDIR, "libcdm_batch.so")
    newest = max(os.path.getmtime(src), os.path.getmtime(hdr))
    if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out, None
    os.makedirs(LIBDIR, exist_ok=True)
    cmd = [nvcc_path(), "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"), src, "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, (r.stdout + r.stderr)[-4000:]
    os.replace(out + ".tmp", out)
    return out, None


def build_mlp(force=False):
    """Learned-initialiser library: tcgen05 GEMMs, training and inference
    (include/cdm_mlp.h)."""
    src = os.path.join(CSRC, "mlp", "cdm_mlp.cu")
    deps = [src, os.path.join(CSRC, "mlp", "cdm_umma.cuh"), os.path.join(ROOT, "include", "cdm_mlp.h")]
    out = os.path.join(LIBDIR, "libcdm_mlp.so")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(map(os.path.getmtime, deps)):
        return out, None
    os.makedirs(LIBDIR, exist_ok=True)
    cmd = [nvcc_path(), "-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CSRC, "mlp"), src,
           "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, (r.stdout + r.stderr)[-4000:]
    os.replace(out + ".tmp", out)
    return out, None


def zlib_flags():
    """-DCDM_HAVE_ZLIB -lz when zlib's header and library are present (gzip
    NIfTI support in libcdm_utils), else nothing."""
    probe = "#include <zlib.h>\nint main() { return zlibVersion() == 0; }\n"
    try:
        r = subprocess.run(["g++", "-x", "c++", "-", "-lz", "-o", os.devnull], input=probe,
                           capture_output=True, text=True, timeout=60)
    except (OSError, subprocess.SubprocessError):
        return []
    return ["-DCDM_HAVE_ZLIB", "-lz"] if r.returncode == 0 else []


def build_utils(force=False):
    """DTI initialiser, post-processing, part files and NIfTI volumes
    (include/cdm_utils.h, include/cdm_volumes.h)."""
    srcs = [os.path.join(CSRC, "utils", "cdm_utils.cu"), os.path.join(CSRC, "utils", "cdm_volumes.cpp")]
    hdrs = [os.path.join(ROOT, "include", "cdm_utils.h"), os.path.join(ROOT, "include", "cdm_volumes.h")]
    out = os.path.join(LIBDIR, "libcdm_utils.so")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(f) for f in srcs + hdrs):
        return out, None
    os.makedirs(LIBDIR, exist_ok=True)
    zl = zlib_flags()
    cmd = [nvcc_path(), "-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include")] + [f for f in zl if f.startswith("-D")] + srcs + \
        ["-o", out + ".tmp"] + [f for f in zl if f.startswith("-l")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, (r.stdout + r.stderr)[-4000:]
    os.replace(out + ".tmp", out)
    return out, None


# The models of the multi-model library built by default: the mix of the
# heterogeneous workload (tensor, ball & two sticks, NODDI-Watson).
HETERO_MODELS = ("DiffusionTensor", "Ball_2_Sticks", "NODDI_Watson")
HETERO_LANES = (1, 2, 4)
# bytes of a model's MCMC argument block in the persistent kernel's
# parameters (one slot per entry; models with up to 17 parameters)
HETERO_ARGS_BLOCK = 640


def hetero_lib_path(tag="default"):
    return os.path.join(LIBDIR, f"libcdm_hetero_{tag}.so")


def build_hetero(models=HETERO_MODELS, lanes=HETERO_LANES, tag="default", model_dirs=None,
                 eval_types=None, force=False, verbose=False, jobs=None, lto=False, maxrreg=128,
                 whole=False):
    """libcdm_hetero_<tag>.so: one persistent MCMC kernel over several models
    (cdm_hetero.h). Each model's part (cdm_hetero_part.cu) is compiled with
    relocatable device code in a translation unit of its own, against that
    model's plugin; the parts and the persistent kernel are device-linked
    into one cubin, which the host half embeds."""
    model_dirs = list(model_dirs or [os.path.join(MODELS, m) for m in models])
    eval_types = list(eval_types or [None] * len(model_dirs))
    names = [os.path.basename(d.rstrip("/")) for d in model_dirs]
    out = hetero_lib_path(tag)
    hdir = os.path.join(GENDIR, f"hetero_{tag}")
    os.makedirs(hdir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hsrc = os.path.join(CSRC, "hetero")
    h = hashlib.sha256()
    for f in sources() + sorted(os.path.join(hsrc, x) for x in os.listdir(hsrc)) + \
            [os.path.join(ROOT, "include", "cdm_hetero.h")]:
        h.update(open(f, "rb").read())
    for d, e in zip(model_dirs, eval_types):
        h.update(f"{d}|{e}".encode())
        for x in sorted(os.listdir(d)):
            if x.endswith((".h", ".cc", ".cu", ".hpp")):
                h.update(open(os.path.join(d, x), "rb").read())
    h.update(repr((tuple(lanes), lto, maxrreg, whole)).encode())
    dig = h.hexdigest()
    stamp = out + ".sha256"
    if not force and os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == dig:
        return out, None
    lane_list = " ".join(f"X({g}, {li})" for li, g in enumerate(lanes))
    with open(os.path.join(hdir, "cdm_hx_dispatch.h"), "w") as f:
        f.write("// generated by cudimot_gb300/build.py: entries of the linked models\n#pragma once\n")
        entries = []
        for i in range(len(names)):
            for g in lanes:
                for r in (0, 1):
                    nm = f"cdm_hx_{i}_mcmc_{g}_{r}"
                    f.write(f'extern "C" __device__ void {nm}(int, unsigned char*);\n')
                    entries.append(nm)
        # entry k reads its argument block from slot k of the constant
        # table cdm_hx_args
        f.write("__device__ __forceinline__ void cdm_hx_dispatch(int fn, int tile, "
                "unsigned char* scratch) {\n  switch (fn) {\n")
        for k, nm in enumerate(entries):
            f.write(f"    case {k}: {nm}(tile, scratch); break;\n")
        f.write("    default: break;\n  }\n}\n")
    with open(os.path.join(hdir, "cdm_hx_entries.h"), "w") as f:
        f.write("// generated by cudimot_gb300/build.py\n#pragma once\n")
        f.write(f"#define CDM_HX_ENTRIES {len(entries)}\n#define CDM_HX_ARGS_BLOCK {HETERO_ARGS_BLOCK}\n")
        f.write(f"#define CDM_HX_NLANES {len(lanes)}\n#define CDM_HX_LANES(X) {lane_list}\n")
    with open(os.path.join(hdir, "cdm_hx_set.h"), "w") as f:
        f.write("// generated by cudimot_gb300/build.py: the linked models\n#pragma once\n")
        f.write(f"constexpr int kHxNumModels = {len(names)};\n")
        f.write("static const char* const kHxModels[] = {" + ", ".join(f'"{n}"' for n in names) + "};\n")
        f.write("static const int kHxEvalDouble[] = {" +
                ", ".join("1" if e == "double" else "0" for e in eval_types) + "};\n")
        f.write(f"constexpr int kHxNumLanes = {len(lanes)};\n")
        f.write("static const int kHxLanes[] = {" + ", ".join(str(g) for g in lanes) + "};\n")
        f.write("constexpr int kHxThreads = 128;\n")
    # lto: the parts reach the device link as IR and the entries are
    # inlined into the persistent kernel; otherwise each entry is compiled
    # on its own, as a kernel of the model library is, and called through
    # the ABI once per tile (saving and restoring the registers it uses)
    gen_flag = "-gencode=arch=compute_103a,code=lto_103a" if lto else ARCH
    # registers per thread: 128 gives 4 resident CTAs of 128 threads per
    # SM, as the model libraries' MCMC kernels have
    base = [nvcc_path(), "-O3", "-std=c++17", gen_flag, "-lineinfo", "-rdc=true",
            f"-maxrregcount={maxrreg}", f"-DCDM_MCMC_MIN_BLOCKS={65536 // (128 * maxrreg)}",
            "-Xcompiler", "-ffp-contract=off"]
    if verbose:
        base += ["-Xptxas", "-v"]

    def part(i):
        d, e, n = model_dirs[i], eval_types[i], names[i]
        gen = os.path.join(hdir, f"gen_{i}")
        os.makedirs(gen, exist_ok=True)
        _write_sizes(gen, block_sizes(d))
        o = os.path.join(hdir, f"part_{i}.o")
        cmd = base + eval_flags(e) + [f"-DCDM_HX_ID={i}", "-I", hdir] + _includes(gen, d) + \
            ["-c", os.path.join(hsrc, "cdm_hetero_part.cu"), "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        return o, None if r.returncode == 0 else f"{n}: " + (r.stdout + r.stderr)[-6000:]

    cubin = os.path.join(hdir, "cdm_hetero.cubin")
    if whole:
        # one model: the part and the persistent kernel in one translation
        # unit, compiled as a whole program (no device link)
        if len(names) != 1:
            return out, "whole-program build of the multi-model kernel takes one model"
        gen = os.path.join(hdir, "gen_0")
        os.makedirs(gen, exist_ok=True)
        _write_sizes(gen, block_sizes(model_dirs[0]))
        tu = os.path.join(hdir, "cdm_hetero_whole.cu")
        with open(tu, "w") as f:
            f.write("// generated by cudimot_gb300/build.py\n#define CDM_HX_ID 0\n")
            f.write(f'#include "{os.path.join(hsrc, "cdm_hetero_part.cu")}"\n')
            f.write(f'#include "{os.path.join(hsrc, "cdm_hetero_kernel.cu")}"\n')
        cmd = [nvcc_path(), "-O3", "-std=c++17", ARCH, "-lineinfo", "-cubin",
               "-Xcompiler", "-ffp-contract=off", "-I", hdir, "-I", hsrc] + eval_flags(eval_types[0]) + \
            _includes(gen, model_dirs[0]) + [tu, "-o", cubin]
        if verbose:
            cmd[1:1] = ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            return out, (r.stdout + r.stderr)[-6000:]
        parts = None
    kobj = os.path.join(hdir, "kernel.o")
    if not whole:
        kcmd = base + ["-I", hdir, "-I", hsrc, "-c", os.path.join(hsrc, "cdm_hetero_kernel.cu"),
                       "-o", kobj]
        with cf.ThreadPoolExecutor(jobs or min(len(names) + 1, os.cpu_count() or 1)) as ex:
            parts = list(ex.map(part, range(len(names))))
            kr = subprocess.run(kcmd, capture_output=True, text=True)
        for _, err in parts:
            if err:
                return out, err
        if kr.returncode != 0:
            return out, (kr.stdout + kr.stderr)[-6000:]
        lcmd = [nvcc_path(), "-arch=sm_103a"] + (["-dlto"] if lto else []) + ["-dlink", "--cubin"] + \
            [o for o, _ in parts] + [kobj, "-o", cubin]
        if verbose:
            lcmd[1:1] = ["-Xnvlink", "-v"]
        r = subprocess.run(lcmd, capture_output=True, text=True)
        if r.returncode != 0:
            return out, (r.stdout + r.stderr)[-6000:]
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
    image = os.path.join(hdir, "cdm_hetero_image.cpp")
    with open(image, "w") as f:
        f.write("// generated by cudimot_gb300/build.py: the multi-model module, embedded\n")
        f.write('__asm__(".section .rodata\\n.balign 64\\n.globl cdm_hetero_image\\n'
                'cdm_hetero_image:\\n.incbin \\"' + cubin + '\\"\\n.byte 0\\n.previous\\n");\n')
    cmd = [nvcc_path(), "-O3", "-std=c++17", ARCH, "-Xcompiler", "-fPIC", "-shared",
           "-I", hdir, "-I", hsrc, "-I", os.path.join(ROOT, "include"),
           os.path.join(hsrc, "cdm_hetero_host.cu"), image, "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return out, (r.stdout + r.stderr)[-6000:]
    os.replace(out + ".tmp", out)
    with open(stamp, "w") as f:
        f.write(dig)
    return out, None


def build_all(models=None, model_dirs=(), jobs=None, verbose=False, force=False):
    todo = [(os.path.join(MODELS, m), m) for m in (models or shipped_models())]
    todo += [(d, None) for d in model_dirs]
    jobs = jobs or max(1, min(len(todo), os.cpu_count() or 1))
    errors = {}
    with cf.ThreadPoolExecutor(jobs + 1) as ex:
        futs = {ex.submit(build_model, d, n, (), verbose, force): (d, n) for d, n in todo}
        futs[ex.submit(build_peak, force)] = ("peak", None)
        futs[ex.submit(build_batch, force)] = ("batch", None)
        futs[ex.submit(build_mlp, force)] = ("mlp", None)
        futs[ex.submit(build_utils, force)] = ("utils", None)
        futs[ex.submit(build_hetero, force=force)] = ("hetero", None)
        for f in cf.as_completed(futs):
            out, err = f.result()
            if err:
                errors[out] = err
    return errors


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--models", nargs="*", default=None)
    ap.add_argument("--model-dir", action="append", default=[])
    ap.add_argument("--eval", choices=["float", "double"], default=None,
                    help="plugin evaluation precision of --model-dir builds (default float)")
    ap.add_argument("--split", default=None,
                    help="with one --model-dir: build only the device half into this directory")
    ap.add_argument("--module-host", default=None,
                    help="build the host half of a split build from this directory")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    if a.split or a.module_host:
        errs = {}
        if a.split:
            if len(a.model_dir) != 1:
                ap.error("--split takes exactly one --model-dir")
            out, err = split_device(a.model_dir[0], a.split, eval_type=a.eval, force=a.force)
            if err:
                errs[out] = err
        if a.module_host and not errs:
            out, err = split_host(a.module_host, force=a.force)
            if err:
                errs[out] = err
    elif a.eval:
        errs = {}
        for d in a.model_dir:
            out, err = build_model(d, None, (), a.verbose, a.force, eval_type=a.eval)
            if err:
                errs[out] = err
    else:
        errs = build_all(a.models, a.model_dir, verbose=a.verbose, force=a.force)
    for k, v in errs.items():
        print(f"FAILED {k}\n{v}", file=sys.stderr)
    sys.exit(1 if errs else 0)


if __name__ == "__main__":
    main()
