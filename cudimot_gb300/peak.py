"""Measured FP32 FMA peak of the current GPU (the roofline denominator of
the FP32-pipe-bound fitting kernels)."""
import ctypes as C
import os

from .capi import LIBDIR


def _lib():
    path = os.path.join(LIBDIR, "libcdm_peak.so")
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = C.CDLL(path)
    lib.cdm_ffma_probe.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    lib.cdm_ffma_probe.restype = C.c_int
    lib.cdm_ffma2_probe.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    lib.cdm_ffma2_probe.restype = C.c_int
    lib.cdm_ffma_probe_fmas.argtypes = [C.c_int, C.c_int]
    lib.cdm_ffma_probe_fmas.restype = C.c_double
    return lib


def measure_fp32(dev, iters=4096, repeats=5):
    """Best FP32 FMA rate of the scalar (FFMA) and paired (FFMA2) probes;
    the peak is the larger."""
    import torch
    lib = _lib()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks = sms * 8
    out = torch.zeros(blocks * 256, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    res = {}
    for name, fn in (("ffma", lib.cdm_ffma_probe), ("ffma2", lib.cdm_ffma2_probe)):
        for _ in range(2):
            fn(C.c_void_p(out.data_ptr()), iters, blocks, C.c_void_p(st.cuda_stream))
        torch.cuda.synchronize(dev)
        best = None
        for _ in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn(C.c_void_p(out.data_ptr()), iters, blocks, C.c_void_p(st.cuda_stream))
            e1.record(st)
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        res[name] = 2.0 * lib.cdm_ffma_probe_fmas(iters, blocks) / (best / 1e3) / 1e12
    top = max(res, key=res.get)
    return {"tflops": res[top], "ffma_tflops": res["ffma"], "ffma2_tflops": res["ffma2"],
            "source": f"measured: {top.upper()} loop, {blocks} CTAs x 256 threads, best of {repeats} "
                      f"(FFMA {res['ffma']:.1f}, FFMA2 {res['ffma2']:.1f} TFLOP/s)"}
