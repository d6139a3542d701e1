"""ctypes binding of the C ABI in include/acc_gb300.h.

The structures below mirror the C structs field for field; `check_layout`
compares their sizes with the library's own `mcv_struct_sizes`.  The
library is the in-tree `acc_gb300/libacc_gb300.so` built by
`acc_gb300._build`; there is no fallback: every entry point raises if the
library or a CUDA device is missing.
"""

import ctypes
import os
import threading

MCV_MAX_COMPONENTS = 32
MCV_NPARAM = 24
MCV_NIPARAM = 8
MCV_MAX_INTERSECTIONS = 10
MCV_MAX_BOUNCES = 100000
MCV_MAX_VARIANTS = 1024
MCV_MS_MAX_SCATTERED = 48
MCV_COMPOSITE_MAX = 16
MCV_ANYSHAPE_MAX_FACES = 99
MCV_ANYSHAPE_MAX_VERTICES = 16
MCV_EXPR_STACK = 8
MCV_EXPR_MAX_OPS = 256
MCV_SNS_E_NODES = 4096
MCV_SNS_T_NODES = 512
MCV_SNS_TAIL_MAX = 65536
MCV_NOALLOC_MAX_VARIANTS = 64
MCV_VARIANT_FP64_FMA = 4
MCV_SMEM_TALLY_MAX = 2048

MCV_OK, MCV_EINVAL, MCV_ECUDA, MCV_ECOUNT, MCV_EBOUNCE = 0, 1, 2, 3, 4
MCV_ENONFINITE, MCV_EBIN, MCV_ENODEV, MCV_ECAPACITY = 5, 6, 7, 8

OP_ARM = 0
OP_SOURCE_SIMPLE = 1
OP_GUIDE = 2
OP_HSS = 3
OP_PSD_MONITOR = 4
OP_PSD_MONITOR_4PI = 5
OP_WAVELENGTH_MONITOR = 6
OP_POSDIV_MONITOR = 7
OP_IQE_MONITOR = 8
OP_ENERGY_MONITOR = 9
OP_THETA_TOF_4PI = 10
OP_CYL_IQE_DETECTOR = 11
OP_BANKED_DETECTOR = 12
OP_SLIT = 13
OP_BEAMSTOP = 14
OP_HMS = 15
OP_GUIDE_TAPERING = 16
OP_SNS_SOURCE = 17
OP_NEUTRON_STORAGE = 18
OP_KERNEL_ELEMENT = 19
OP_GUIDE_ANYSHAPE = 20
OP_NEUTRON_TO_STORAGE = 21

SHAPE_SPHERE, SHAPE_CYLINDER, SHAPE_BOX = 1, 2, 3
CSG_PRIMITIVE, CSG_DIFFERENCE, CSG_UNION, CSG_INTERSECTION = 0, 1, 2, 3
KERNEL_ISOTROPIC, KERNEL_POWDER, KERNEL_SQE_GRID = 1, 2, 3
KERNEL_CONSTANT_QE, KERNEL_E_Q, KERNEL_COMPOSITE, KERNEL_SANS2D = 4, 5, 6, 7
KERNEL_DGSSXRES = 8

FLAG_IDENTITY_ROT = 1
FLAG_AGGREGATE = 2
FLAG_SMEM_TALLY = 4
FP32, FP64 = 32, 64


class mcv_component(ctypes.Structure):
    _fields_ = [
        ("opcode", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("ip", ctypes.c_int32 * MCV_NIPARAM),
        ("dp", ctypes.c_double * MCV_NPARAM),
        ("fp", ctypes.c_float * MCV_NPARAM),
        ("tally", ctypes.c_void_p),
        ("table", ctypes.c_void_p),
        ("ftable", ctypes.c_void_p),
        ("table_len", ctypes.c_uint64),
    ]


class mcv_chain(ctypes.Structure):
    _fields_ = [
        ("ncomp", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("weight_exp2", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("comp", mcv_component * MCV_MAX_COMPONENTS),
        ("rot", (ctypes.c_double * 9) * MCV_MAX_COMPONENTS),
        ("off", (ctypes.c_double * 3) * MCV_MAX_COMPONENTS),
        ("frot", (ctypes.c_float * 9) * MCV_MAX_COMPONENTS),
        ("foff", (ctypes.c_float * 3) * MCV_MAX_COMPONENTS),
    ]


class mcv_launch(ctypes.Structure):
    _fields_ = [
        ("threads_per_block", ctypes.c_int32),
        ("blocks", ctypes.c_int32),
        ("chunk", ctypes.c_int32),
        ("variant", ctypes.c_int32),
    ]


class mcv_grad(ctypes.Structure):
    _fields_ = [
        ("dout", ctypes.c_void_p * MCV_MAX_COMPONENTS),
        ("dparam", ctypes.c_void_p * MCV_MAX_COMPONENTS),
        ("dtable", ctypes.c_void_p * MCV_MAX_COMPONENTS),
    ]


class mcv_status(ctypes.Structure):
    _fields_ = [
        ("code", ctypes.c_int32),
        ("first_bad_component", ctypes.c_int32),
        ("processed", ctypes.c_uint64),
        ("bounce_overflow", ctypes.c_uint64),
        ("nonfinite", ctypes.c_uint64),
        ("bin_oob", ctypes.c_uint64),
        ("message", ctypes.c_char * 256),
    ]


class EngineError(RuntimeError):
    """A C-ABI call returned a nonzero status."""

    def __init__(self, code, message):
        super().__init__(f"[mcv error {code}] {message}")
        self.code = code


LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                        "libacc_gb300.so")

_lib = None
_lock = threading.Lock()

_SIGNATURES = {
    "mcv_abi_version": (ctypes.c_int, []),
    "mcv_struct_sizes": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint64)] * 4),
    "mcv_ctx_create": (ctypes.c_int, [ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_void_p)]),
    "mcv_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "mcv_ctx_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_uint64,
                                      ctypes.POINTER(mcv_status)]),
    "mcv_run_chain": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.POINTER(mcv_chain), ctypes.c_uint64,
        ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
        ctypes.POINTER(mcv_launch), ctypes.c_void_p,
        ctypes.POINTER(mcv_status)]),
    "mcv_replay_uniforms": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.POINTER(mcv_chain), ctypes.c_uint64,
        ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.POINTER(mcv_launch), ctypes.c_void_p,
        ctypes.POINTER(mcv_status)]),
    "mcv_process_buffer": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.POINTER(mcv_chain), ctypes.c_void_p,
        ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
        ctypes.POINTER(mcv_launch), ctypes.c_void_p,
        ctypes.POINTER(mcv_status)]),
    "mcv_run_batched": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(mcv_launch),
        ctypes.c_void_p, ctypes.POINTER(mcv_status)]),
    "mcv_graph_create_batched": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(mcv_launch),
        ctypes.POINTER(ctypes.c_void_p)]),
    "mcv_run_batched_noalloc": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_int, ctypes.POINTER(mcv_launch), ctypes.c_void_p,
        ctypes.POINTER(mcv_status)]),
    "mcv_graph_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "mcv_graph_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "mcv_backward": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.POINTER(mcv_chain), ctypes.POINTER(mcv_grad),
        ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
        ctypes.POINTER(mcv_launch), ctypes.c_void_p,
        ctypes.POINTER(mcv_status)]),
    "mcv_probe_fma_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_double)]),
    "mcv_probe_sfu_rate": (ctypes.c_int, [ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_double)]),
    "mcv_probe_atomic_rate": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint64,
                                             ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_double)]),
    "mcv_intersect": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.POINTER(mcv_component), ctypes.c_void_p,
        ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
        ctypes.c_void_p, ctypes.POINTER(mcv_status)]),
}


def lib():
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"the CUDA engine {LIB_PATH} is not built; run "
                    "acc_gb300._build.build_engine() (needs nvcc)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in _SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
            check_layout(L)
        return _lib


def check_layout(L):
    sizes = [ctypes.c_uint64() for _ in range(4)]
    L.mcv_struct_sizes(*[ctypes.byref(s) for s in sizes])
    mine = [ctypes.sizeof(mcv_component), ctypes.sizeof(mcv_chain),
            ctypes.sizeof(mcv_status), ctypes.sizeof(mcv_launch)]
    theirs = [s.value for s in sizes]
    if mine != theirs:
        raise RuntimeError(f"ABI layout mismatch: python {mine} vs C {theirs}")


def check(rc, st=None):
    if rc != MCV_OK:
        msg = st.message.decode(errors="replace") if st is not None else ""
        raise EngineError(rc, msg or "engine call failed")


class Context:
    """Owns one mcv_ctx (the per-device status counters)."""

    def __init__(self, device=0):
        self.device = device
        self.handle = ctypes.c_void_p()
        rc = lib().mcv_ctx_create(device, ctypes.byref(self.handle))
        if rc == MCV_ENODEV:
            raise EngineError(rc, "no CUDA device is visible")
        check(rc)

    def close(self):
        if self.handle:
            lib().mcv_ctx_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_contexts = {}


def context(device=None):
    """The shared context of `device` (default: the current torch device)."""
    if device is None:
        import torch
        device = torch.cuda.current_device()
    with _lock:
        ctx = _contexts.get(device)
    if ctx is None:
        ctx = Context(device)
        with _lock:
            _contexts[device] = ctx
    return ctx


def current_stream_handle():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
