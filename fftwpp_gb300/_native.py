"""ctypes binding of lib_fftwpp.so (the C ABI of include/cfftw++.h and
include/fftwpp_gb300.h).

Loading fails loudly when the library is missing: there is no CPU fallback
anywhere in this package.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib_fftwpp.so")

PAD, CENTERED, HERMITIAN, REAL = 0, 1, 2, 3
F64, F32, FF = 0, 1, 2
PRECISIONS = {"f64": F64, "f32": F32, "ff": FF}
MULT = {"none": 0, "binary": 1, "realbinary": 2, "correlation": 3,
        "realjacobian": 4, "jacobian": 5, "realjacadj": 6, "dot": 7,
        "realdot": 8, "user": 9}

_lib = None


class NativeLibraryMissing(RuntimeError):
    pass


def load():
    """Load lib_fftwpp.so and declare every prototype."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise NativeLibraryMissing(
            f"{LIB_PATH} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` "
            "(the GPU path has no fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    sz = ctypes.c_size_t
    vp = ctypes.c_void_p
    P = ctypes.POINTER

    lib.fgb_create.restype = vp
    lib.fgb_create.argtypes = [ctypes.c_int, P(ctypes.c_int), P(sz), P(sz),
                               P(sz), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                               ctypes.c_int, sz]
    lib.fgb_convolve_device.restype = ctypes.c_int
    lib.fgb_convolve_device.argtypes = [vp, P(vp), P(vp), vp]
    lib.fgb_convolve_host.restype = ctypes.c_int
    lib.fgb_convolve_host.argtypes = [vp, P(vp), P(vp)]
    lib.fgb_convolve_device_with.restype = ctypes.c_int
    lib.fgb_convolve_device_with.argtypes = [vp, vp, P(vp), P(vp), vp]
    lib.fgb_convolve_host_with.restype = ctypes.c_int
    lib.fgb_convolve_host_with.argtypes = [vp, vp, P(vp), P(vp)]
    lib.fgb_fft_origin_shift_device.restype = ctypes.c_int
    lib.fgb_fft_origin_shift_device.argtypes = [vp, sz, sz, sz, ctypes.c_int,
                                                vp]
    lib.fgb_set_ff_range_guard.restype = None
    lib.fgb_set_ff_range_guard.argtypes = [ctypes.c_int]
    lib.fgb_set_strides.restype = ctypes.c_int
    lib.fgb_set_strides.argtypes = [vp, P(sz)]
    lib.fgb_info.restype = ctypes.c_int
    lib.fgb_info.argtypes = [vp, P(ctypes.c_long)]
    lib.fgb_timing.restype = ctypes.c_int
    lib.fgb_timing.argtypes = [vp, ctypes.c_int]
    lib.fgb_timing_collect.restype = ctypes.c_int
    lib.fgb_timing_collect.argtypes = [vp, P(ctypes.c_double), ctypes.c_int]
    lib.fgb_measure_fma_rate.restype = ctypes.c_int
    lib.fgb_measure_fma_rate.argtypes = [P(ctypes.c_double), P(ctypes.c_double)]
    lib.fgb_scale_columns_device.restype = ctypes.c_int
    lib.fgb_scale_columns_device.argtypes = [sz, sz, ctypes.c_double,
                                             ctypes.c_double, vp,
                                             ctypes.c_int, vp]
    lib.fgb_hconv2d_convolve_noalloc.restype = ctypes.c_int
    lib.fgb_hconv2d_convolve_noalloc.argtypes = [vp, vp, vp, sz, sz, vp]
    lib.fgb_batch_create.restype = vp
    lib.fgb_batch_create.argtypes = [ctypes.c_int, P(sz), P(sz), ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int]
    lib.fgb_batch_convolve_device.restype = ctypes.c_int
    lib.fgb_batch_convolve_device.argtypes = [vp, P(vp), P(vp), vp,
                                              ctypes.c_int]
    lib.fgb_batch_info.restype = ctypes.c_int
    lib.fgb_batch_info.argtypes = [vp, P(ctypes.c_long)]
    lib.fgb_batch_choice.restype = ctypes.c_long
    lib.fgb_batch_choice.argtypes = [vp, ctypes.c_int]
    lib.fgb_batch_error.restype = ctypes.c_int
    lib.fgb_batch_error.argtypes = [vp]
    lib.fgb_batch_destroy.restype = None
    lib.fgb_batch_destroy.argtypes = [vp]
    lib.fgb_batch_set_spin_limit.restype = ctypes.c_int
    lib.fgb_batch_set_spin_limit.argtypes = [vp, ctypes.c_longlong]
    lib.fgb_batch_block_problem.restype = ctypes.c_int
    lib.fgb_batch_block_problem.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    lib.fgb_pad_create.restype = vp
    lib.fgb_pad_create.argtypes = [ctypes.c_int, sz, sz, sz, sz, ctypes.c_int]
    lib.fgb_pad_forward_device.restype = ctypes.c_int
    lib.fgb_pad_forward_device.argtypes = [vp, vp, vp, vp]
    lib.fgb_pad_backward_device.restype = ctypes.c_int
    lib.fgb_pad_backward_device.argtypes = [vp, vp, vp, vp]
    lib.fgb_pad_info.restype = ctypes.c_int
    lib.fgb_pad_info.argtypes = [vp, P(ctypes.c_long)]
    lib.fgb_pad_index.restype = sz
    lib.fgb_pad_index.argtypes = [vp, sz, sz]
    lib.fgb_pad_destroy.restype = None
    lib.fgb_pad_destroy.argtypes = [vp]
    lib.fgb_fft_create.restype = vp
    lib.fgb_fft_create.argtypes = [ctypes.c_int, sz, ctypes.c_int, sz, sz, sz,
                                   sz, sz, sz, ctypes.c_int]
    lib.fgb_fft_execute_device.restype = ctypes.c_int
    lib.fgb_fft_execute_device.argtypes = [vp, vp, vp, vp]
    lib.fgb_fft_destroy.restype = None
    lib.fgb_fft_destroy.argtypes = [vp]
    lib.fgb_debug_fail_allocation_after.restype = None
    lib.fgb_debug_fail_allocation_after.argtypes = [ctypes.c_long]
    lib.fgb_set_autotune.restype = None
    lib.fgb_set_autotune.argtypes = [ctypes.c_int]
    lib.fgb_wisdom_export.restype = sz
    lib.fgb_wisdom_export.argtypes = [ctypes.c_char_p, sz]
    lib.fgb_wisdom_import.restype = ctypes.c_int
    lib.fgb_wisdom_import.argtypes = [ctypes.c_char_p]
    lib.fgb_wisdom_forget.restype = None
    lib.fgb_wisdom_forget.argtypes = []
    lib.fgb_set_residue_search.restype = None
    lib.fgb_set_residue_search.argtypes = [ctypes.c_int]
    lib.fgb_set_drop_in_precision.restype = ctypes.c_int
    lib.fgb_set_drop_in_precision.argtypes = [ctypes.c_int]
    lib.fgb_get_drop_in_precision.restype = ctypes.c_int
    lib.fgb_get_drop_in_precision.argtypes = []
    lib.fgb_set_zero_copy.restype = None
    lib.fgb_set_zero_copy.argtypes = [ctypes.c_int]
    lib.fgb_set_host_path.restype = None
    lib.fgb_set_host_path.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.fgb_host_path.restype = ctypes.c_int
    lib.fgb_host_path.argtypes = [vp, P(ctypes.c_int), P(ctypes.c_int)]
    lib.fgb_destroy.restype = None
    lib.fgb_destroy.argtypes = [vp]
    lib.fgb_last_error.restype = ctypes.c_char_p
    lib.fgb_last_error.argtypes = []
    lib.fgb_parameters.restype = None
    lib.fgb_parameters.argtypes = [sz, sz, sz, ctypes.c_int, P(sz), P(sz), P(sz)]
    lib.fgb_nextfftsize.restype = sz
    lib.fgb_nextfftsize.argtypes = [sz]
    lib.fgb_batch_task_order.restype = ctypes.c_int
    lib.fgb_batch_task_order.argtypes = [
        ctypes.c_int, P(sz), P(ctypes.c_int), P(ctypes.c_int),
        P(ctypes.c_int), ctypes.c_int, ctypes.c_int, ctypes.c_int, sz,
        P(ctypes.c_int), P(ctypes.c_int), ctypes.c_int]
    lib.fgb_fft_radices.restype = ctypes.c_int
    lib.fgb_fft_radices.argtypes = [sz, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, P(ctypes.c_int),
                                    ctypes.c_int]
    lib.fgb_index.restype = sz
    lib.fgb_index.argtypes = [ctypes.c_int, sz, sz, sz, sz, sz, sz, sz]
    lib.fgb_hermitian_symmetrize_x_device.restype = ctypes.c_int
    lib.fgb_hermitian_symmetrize_x_device.argtypes = [sz, sz, sz, vp,
                                                      ctypes.c_int, vp]

    # FFTW++-compatible entry points (wrappers/cfftw++.h).
    for name in ("conv1d", "hconv1d", "conv2d", "hconv2d", "conv3d",
                 "hconv3d"):
        create = getattr(lib, f"fftwpp_create_{name}")
        create.restype = vp
        dims = {"1d": 1, "2d": 2, "3d": 3}[name[-2:]]
        create.argtypes = [sz] * dims
        conv = getattr(lib, f"fftwpp_{name}_convolve")
        conv.restype = None
        conv.argtypes = [vp, vp, vp]
        delete = getattr(lib, f"fftwpp_{name}_delete")
        delete.restype = None
        delete.argtypes = [vp]
        # Dot-product and work-array forms (declared in FFTW++'s header).
        cdot = getattr(lib, f"fftwpp_create_{name}_dot")
        cdot.restype = vp
        cdot.argtypes = [sz] * dims + [sz]
        nwork = {"conv1d": 2, "hconv1d": 3, "conv2d": 4, "hconv2d": 5,
                 "conv3d": 6, "hconv3d": 7}[name]
        cwork = getattr(lib, f"fftwpp_create_{name}_work")
        cwork.restype = vp
        cwork.argtypes = [sz] * dims + [vp] * nwork
        if name != "conv3d":
            cwd = getattr(lib, f"fftwpp_create_{name}_work_dot")
            cwd.restype = vp
            cwd.argtypes = [sz] * dims + [vp] * nwork + [sz]
        dot = getattr(lib, f"fftwpp_{name}_convolve_dot")
        dot.restype = None
        dot.argtypes = [vp, P(vp), P(vp)]
        if name != "hconv3d":
            dotf = getattr(lib, f"fftwpp_{name}_convolve_dotf")
            dotf.restype = None
            dotf.argtypes = [vp, vp, vp]
    lib.create_doublealign.restype = vp
    lib.create_doublealign.argtypes = [sz]
    lib.fftwpp_HermitianSymmetrize.argtypes = [vp]
    lib.fftwpp_HermitianSymmetrizeX.argtypes = [sz, sz, sz, vp]
    lib.fftwpp_HermitianSymmetrizeXY.argtypes = [sz, sz, sz, sz, sz, vp]
    lib.create_complexAlign.restype = vp
    lib.create_complexAlign.argtypes = [sz]
    lib.delete_complexAlign.argtypes = [vp]
    lib.create_doubleAlign.restype = vp
    lib.create_doubleAlign.argtypes = [sz]
    lib.delete_doubleAlign.argtypes = [vp]
    lib.get_fftwpp_maxthreads.restype = sz
    lib.set_fftwpp_maxthreads.argtypes = [sz]
    _lib = lib
    return lib


def last_error() -> str:
    return load().fgb_last_error().decode(errors="replace")


def header_symbols() -> list[str]:
    """Every function declared in include/*.h (for the export check)."""
    import re
    inc = os.path.join(os.path.dirname(HERE), "include")
    names = []
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"([A-Za-z_][A-Za-z_0-9]*)\s*\(", text):
            name = m.group(1)
            if name in ("if", "for", "while", "sizeof", "return", "defined"):
                continue
            if name.startswith(("fftwpp_", "fgb_", "create_", "delete_",
                                "get_fftwpp", "set_fftwpp")):
                names.append(name)
    return sorted(set(names))
