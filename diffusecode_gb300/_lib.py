"""Loader of the in-tree C-ABI library (lib/libdiscus_gpu.so).

There is no CPU fallback: if the library is missing or no CUDA device is
visible, calls raise.  Signatures mirror include/discus_gpu.h.
"""
import ctypes as C
import os

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libdiscus_gpu.so")
_lib = None

# every entry point declared in include/discus_gpu.h
EXPORTS = [
    "dgpu_ctx_create", "dgpu_ctx_destroy", "dgpu_last_error", "dgpu_default_opts",
    "dgpu_four_run", "dgpu_four_run_device", "dgpu_four_strucf", "dgpu_fourier_lmn",
    "dgpu_four_stltab", "dgpu_four_formtab", "dgpu_four_increments", "dgpu_chi2_grad",
    "dgpu_batch_run", "dgpu_batch_last_ms", "dgpu_batch_graph_nodes", "dgpu_four_strucf_noalloc", "dgpu_tc_last_kernel_ms",
    "dgpu_four_weight", "dgpu_four_weight_device", "dgpu_four_accumulate", "dgpu_set_symmetry", "dgpu_qval",
    "dgpu_calc_hkl", "dgpu_powder_npkt", "dgpu_powder_complete", "dgpu_chi2_grad_device",
    "dgpu_calc_hkl_files", "dgpu_output_write", "dgpu_four_filter",
]


class DiscusGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"discus_gpu error {code}: {msg}")
        self.code = code


def load():
    """Load the shared library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} not built: run `python -m diffusecode_gb300.build`")
    L = C.CDLL(LIB_PATH)
    dp, ip, i64p = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)
    vp = C.c_void_p
    CR, GR, OP, IN = (C.POINTER(_abi.Crystal), C.POINTER(_abi.Grid), C.POINTER(_abi.Opts),
                      C.POINTER(_abi.Info))
    L.dgpu_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.dgpu_ctx_destroy.argtypes = [vp]
    L.dgpu_last_error.argtypes = [vp]
    L.dgpu_last_error.restype = C.c_char_p
    L.dgpu_default_opts.argtypes = [OP]
    L.dgpu_default_opts.restype = None
    L.dgpu_four_run.argtypes = [vp, CR, GR, OP, dp, dp, dp, IN]
    L.dgpu_four_run_device.argtypes = [vp, CR, GR, OP, vp, vp, vp, IN]
    L.dgpu_four_strucf.argtypes = [vp, dp, C.c_int64, dp, dp, dp, dp, ip, ip, ip, dp, ip, dp]
    L.dgpu_fourier_lmn.argtypes = [dp, dp, ip, ip, dp]
    L.dgpu_four_stltab.argtypes = [vp, GR, dp, ip]
    L.dgpu_four_formtab.argtypes = [vp, CR, OP, dp]
    L.dgpu_four_increments.argtypes = [vp, dp, C.c_int64, dp, dp, dp, dp, i64p]
    L.dgpu_chi2_grad.argtypes = [vp, CR, GR, OP, dp, dp, dp, dp, dp, IN]
    L.dgpu_chi2_grad_device.argtypes = [vp, CR, GR, OP, vp, vp, dp, vp, vp, IN]
    PP = C.POINTER(dp)
    L.dgpu_batch_run.argtypes = [vp, C.c_int32, CR, GR, OP, PP, PP, PP, dp, PP, PP]
    L.dgpu_batch_last_ms.argtypes = [vp]
    L.dgpu_batch_last_ms.restype = C.c_double
    L.dgpu_batch_graph_nodes.argtypes = [vp, C.POINTER(C.c_int64)]
    L.dgpu_batch_graph_nodes.restype = C.c_int64
    L.dgpu_tc_last_kernel_ms.argtypes = [vp]
    L.dgpu_tc_last_kernel_ms.restype = C.c_double
    L.dgpu_four_strucf_noalloc.argtypes = [vp, vp, C.c_int64, dp, dp, dp, dp, ip, ip, ip, vp, vp, vp]
    L.dgpu_four_weight.argtypes = [vp, CR, GR, OP, dp, dp]
    L.dgpu_four_weight_device.argtypes = [vp, CR, GR, OP, vp, vp]
    L.dgpu_four_accumulate.argtypes = [vp, C.c_int32, C.c_int32, GR, C.c_double, dp, dp]
    L.dgpu_set_symmetry.argtypes = [vp, C.c_int32, dp]
    L.dgpu_qval.argtypes = [vp, CR, GR, OP, C.c_int32, C.c_int32, dp, dp, dp, dp, dp]
    L.dgpu_calc_hkl.argtypes = [vp, CR, OP, ip, C.c_int64, C.c_double, C.c_double, C.c_double, dp, dp, dp]
    L.dgpu_calc_hkl_files.argtypes = [vp, CR, OP, C.c_char_p, C.c_char_p, C.c_int32, C.c_double, C.c_double,
                                      C.c_double]
    L.dgpu_output_write.argtypes = [C.c_char_p, C.POINTER(_abi.Output), dp, dp, dp, C.c_int64]
    L.dgpu_four_filter.argtypes = [vp, ip, OP, dp]
    PW = C.POINTER(_abi.Powder)
    L.dgpu_powder_npkt.argtypes = [PW]
    L.dgpu_powder_npkt.restype = C.c_int32
    L.dgpu_powder_complete.argtypes = [vp, CR, PW, OP, dp, C.POINTER(_abi.PowderInfo)]
    _lib = L
    return L


class Context:
    """One device context (stream + cached device buffers)."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.dgpu_ctx_create(int(device), C.byref(h))
        if rc != 0:
            raise DiscusGpuError(rc, "no CUDA device / context creation failed")
        self.h = h

    def check(self, rc):
        if rc < 0:
            raise DiscusGpuError(rc, self.lib.dgpu_last_error(self.h).decode(errors="replace"))
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.dgpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx
