"""The C-ABI library loads, exports every entry point of include/*.h, and
its struct layout matches the Python mirror and the oracle (no GPU needed)."""

import ctypes
import glob
import os
import re

from acc_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:int|void|uint64_t)\s+(mcv_\w+)\s*\(",
                            text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("mcv_run_chain", "mcv_replay_uniforms", "mcv_process_buffer",
              "mcv_ctx_create", "mcv_ctx_destroy", "mcv_ctx_status"):
        assert n in names


def test_library_exports_every_declared_symbol(engine_lib):
    for name in declared_functions():
        assert hasattr(engine_lib, name), f"{name} not exported"


def test_struct_layout_matches(engine_lib, oracle_lib):
    nat.check_layout(engine_lib)
    assert oracle_lib.oracle_sizeof_chain() == ctypes.sizeof(nat.mcv_chain)
    assert oracle_lib.oracle_sizeof_component() == \
        ctypes.sizeof(nat.mcv_component)
    assert engine_lib.mcv_abi_version() == 3


def _bad_chain():
    ch = nat.mcv_chain()
    ch.ncomp = 1
    ch.comp[0].opcode = nat.OP_PSD_MONITOR  # zero bins: invalid
    return ch


def test_invalid_chain_rejected_before_any_device_work(engine_lib):
    st = nat.mcv_status()
    rc = engine_lib.mcv_run_chain(None, ctypes.byref(_bad_chain()), 10, 0, 1,
                                  64, None, None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL
    assert b"bin counts" in st.message
    ch = nat.mcv_chain()
    ch.ncomp = 0
    rc = engine_lib.mcv_run_chain(None, ctypes.byref(ch), 10, 0, 1, 64, None,
                                  None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"components" in st.message
    ch.ncomp = 1
    ch.comp[0].opcode = 99
    rc = engine_lib.mcv_process_buffer(None, ctypes.byref(ch), None, 1, 0, 1,
                                       64, None, None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"opcode" in st.message


def test_bad_precision_and_null_context(engine_lib):
    ch = nat.mcv_chain()
    ch.ncomp = 1  # an Arm
    st = nat.mcv_status()
    rc = engine_lib.mcv_run_chain(None, ctypes.byref(ch), 10, 0, 1, 16, None,
                                  None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"precision" in st.message
    rc = engine_lib.mcv_run_chain(None, ctypes.byref(ch), 10, 0, 1, 32, None,
                                  None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"context" in st.message


def test_hss_validation(engine_lib):
    ch = nat.mcv_chain()
    ch.ncomp = 1
    c = ch.comp[0]
    c.opcode = nat.OP_HSS
    c.ip[0] = nat.CSG_PRIMITIVE
    c.ip[1] = nat.KERNEL_POWDER
    c.ip[2] = nat.SHAPE_SPHERE
    st = nat.mcv_status()
    rc = engine_lib.mcv_run_chain(None, ctypes.byref(ch), 1, 0, 1, 32, None,
                                  None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"powder" in st.message
    c.ip[2] = 7
    rc = engine_lib.mcv_run_chain(None, ctypes.byref(ch), 1, 0, 1, 32, None,
                                  None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"shape" in st.message


def test_e_q_kernel_validation(engine_lib):
    """The E(Q) kernel needs both programs (1..MCV_EXPR_MAX_OPS
    instructions) and 1 <= max_iter <= 1e6; a kernel kind past DGSSXRES is
    unknown."""
    from acc_gb300.components.samples.homogeneous_single_scatterer import \
        factory
    from acc_gb300.engine import build_chain
    from acc_gb300.geometry import Block
    from acc_gb300.kernels import E_Q_Kernel
    from acc_gb300.memory import HostBinder
    H = factory(Block(0.01, 0.01, 0.01), E_Q_Kernel("Q", "1", 0, 5, 1, 1))
    st = nat.mcv_status()

    def run(ch):
        return engine_lib.mcv_run_chain(None, ctypes.byref(ch), 1, 0, 1, 32,
                                        None, None, ctypes.byref(st))
    for field, value in (("ip4", 0), ("ip4", nat.MCV_EXPR_MAX_OPS + 1),
                         ("ip5", 0), ("dp12", 0.0), ("dp12", 2e6),
                         ("table", None)):
        ch = build_chain([H("s")], binder=HostBinder())
        c = ch.comp[0]
        if field == "ip4":
            c.ip[4] = value
        elif field == "ip5":
            c.ip[5] = value
        elif field == "dp12":
            c.dp[12] = value
        else:
            c.table = value
        assert run(ch) == nat.MCV_EINVAL and b"E(Q)" in st.message, field
    ch = build_chain([H("s")], binder=HostBinder())
    ch.comp[0].ip[1] = nat.KERNEL_DGSSXRES + 1
    assert run(ch) == nat.MCV_EINVAL and b"unknown scattering" in st.message


def test_composite_kernel_validation(engine_lib):
    """A composite kernel's elements fill the slots after it, each a kernel
    element (not composite) with a positive weight, running weights that
    reach 1."""
    from acc_gb300.components.samples.homogeneous_single_scatterer import \
        factory
    from acc_gb300.engine import build_chain
    from acc_gb300.geometry import Block
    from acc_gb300.kernels import CompositeKernel, IsotropicKernel
    from acc_gb300.memory import HostBinder
    kern = CompositeKernel([IsotropicKernel(1, 2), IsotropicKernel(3, 4)])
    H = factory(Block(0.01, 0.01, 0.01), kern)
    st = nat.mcv_status()

    def run(ch):
        return engine_lib.mcv_run_chain(None, ctypes.byref(ch), 1, 0, 1, 32,
                                        None, None, ctypes.byref(st))
    ch = build_chain([H("s")], binder=HostBinder())
    assert run(ch) == nat.MCV_EINVAL and b"context" in st.message  # valid
    ch = build_chain([H("s")], binder=HostBinder())
    ch.ncomp = 2  # the second element is cut off
    assert run(ch) == nat.MCV_EINVAL and b"follow" in st.message
    ch = build_chain([H("s")], binder=HostBinder())
    ch.comp[2].dp[23] = 0.9  # running weight short of 1
    assert run(ch) == nat.MCV_EINVAL and b"running weight" in st.message
    ch = build_chain([H("s")], binder=HostBinder())
    ch.comp[1].ip[1] = nat.KERNEL_COMPOSITE  # nested
    assert run(ch) == nat.MCV_EINVAL and b"composite" in st.message
    ch = build_chain([H("s")], binder=HostBinder())
    ch.comp[2].opcode = nat.OP_ARM
    assert run(ch) == nat.MCV_EINVAL and b"bad slot" in st.message


def test_context_create(engine_lib):
    from conftest import HAS_GPU
    h = ctypes.c_void_p()
    rc = engine_lib.mcv_ctx_create(0, ctypes.byref(h))
    if HAS_GPU:
        assert rc == nat.MCV_OK
        engine_lib.mcv_ctx_destroy(h)
    else:
        assert rc == nat.MCV_ENODEV


def test_weight_exp2_out_of_range_rejected(engine_lib):
    from acc_gb300.memory import HostBinder
    from acc_gb300.components.optics.arm import Arm
    from acc_gb300.engine import build_chain
    ch = build_chain([Arm("a")], binder=HostBinder())
    ch.weight_exp2 = 127
    st = nat.mcv_status()
    rc = engine_lib.mcv_run_chain(None, ctypes.byref(ch), 1, 0, 1, 32, None,
                                  None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"weight_exp2" in st.message


def test_multiple_scatterer_rejected_where_unsupported(engine_lib):
    """The fan-out runs in the fused run only: buffered mode, replay,
    backward and batched launches reject a chain with an HMS before any
    device work."""
    from acc_gb300 import instruments
    from acc_gb300.engine import build_chain
    from acc_gb300.instrument import calcTransformations
    from acc_gb300.memory import HostBinder
    ins = instruments.ms_hollow_cylinder()
    off, rot = calcTransformations(ins)
    ch = build_chain(ins.components, off, rot, HostBinder())
    st = nat.mcv_status()
    rc = engine_lib.mcv_process_buffer(None, ctypes.byref(ch), None, 0, 0, 1,
                                       64, None, None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"multiple scatterer" in st.message
    g = nat.mcv_grad()
    rc = engine_lib.mcv_backward(None, ctypes.byref(ch), ctypes.byref(g), 1,
                                 0, 1, 64, None, None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"multiple scatterer" in st.message
    rc = engine_lib.mcv_replay_uniforms(None, ctypes.byref(ch), 1, 0, 1, 64,
                                        None, 0, None, None, None, None,
                                        ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"multiple scatterer" in st.message
    cnt = (ctypes.c_uint64 * 1)(1)
    sd = (ctypes.c_uint64 * 1)(1)
    rc = engine_lib.mcv_run_batched(None, ctypes.byref(ch), 1, cnt, sd, 64,
                                    None, None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"multiple scatterer" in st.message
    # more than one multiple scatterer
    ch2 = build_chain([ins.components[1], ins.components[1]],
                      binder=HostBinder())
    rc = engine_lib.mcv_run_chain(None, ctypes.byref(ch2), 1, 0, 1, 64, None,
                                  None, ctypes.byref(st))
    assert rc == nat.MCV_EINVAL and b"at most one" in st.message
