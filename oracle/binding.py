"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
to check or time the CUDA engine; the product path never imports it.  The
oracle consumes the same mcv_chain struct as the engine (include/
acc_gb300.h) with host pointers for tallies and tables (acc_gb300.memory.
HostBinder).
"""

import ctypes

import numpy as np

from . import build as _build

_lib = None
_timing_lib = None

c_double_p = ctypes.POINTER(ctypes.c_double)


def lib():
    """The checker build (multiply-adds never contracted)."""
    global _lib
    if _lib is None:
        _lib = _bind(ctypes.CDLL(_build.build()))
    return _lib


def timing_lib():
    """The timed-baseline build (-O3, contraction allowed): the same
    functions, for bench.py's CPU legs."""
    global _timing_lib
    if _timing_lib is None:
        _timing_lib = _bind(ctypes.CDLL(_build.build(timing=True)))
    return _timing_lib


def _bind(L):
    """Declare the argument and return types of the oracle's entry points."""
    L.oracle_philox4x32_10.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
    L.oracle_philox4x32_10.restype = None
    for name in ("oracle_intersect_sphere",):
        getattr(L, name).argtypes = [ctypes.c_double] * 7 + [c_double_p] * 2
    L.oracle_intersect_cylinder.argtypes = [ctypes.c_double] * 8 + [c_double_p] * 2
    L.oracle_intersect_box.argtypes = [ctypes.c_double] * 9 + [c_double_p] * 2
    L.oracle_locate.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 3
    L.oracle_locate.restype = ctypes.c_int
    L.oracle_insert_sorted.argtypes = [ctypes.c_double, c_double_p,
                                       ctypes.c_int, ctypes.c_int]
    L.oracle_insert_sorted.restype = ctypes.c_int
    L.oracle_intersect.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 6 + [c_double_p]
    L.oracle_intersect.restype = ctypes.c_int
    L.oracle_time_to_scatter.argtypes = [c_double_p, ctypes.c_int,
                                         ctypes.c_double, c_double_p]
    L.oracle_time_to_scatter.restype = None
    L.oracle_total_time_in_shape.argtypes = [c_double_p, ctypes.c_int]
    L.oracle_total_time_in_shape.restype = ctypes.c_double
    L.oracle_time_to_enter.argtypes = [c_double_p, ctypes.c_int]
    L.oracle_time_to_enter.restype = ctypes.c_double
    L.oracle_rotate.argtypes = [c_double_p, c_double_p, ctypes.c_double,
                                ctypes.c_double]
    L.oracle_rotate.restype = None
    L.oracle_reflectivity.argtypes = [ctypes.c_double] * 6
    L.oracle_reflectivity.restype = ctypes.c_double
    L.oracle_propagate_out.argtypes = [ctypes.c_void_p, c_double_p]
    L.oracle_tof_before_first_exit.argtypes = [ctypes.c_void_p, c_double_p]
    L.oracle_tof_before_first_exit.restype = ctypes.c_double
    L.oracle_propagate_to_next_incident_surface.argtypes = [ctypes.c_void_p, c_double_p]
    L.oracle_propagate_to_next_incident_surface.restype = ctypes.c_int
    L.oracle_propagate_to_next_exiting_surface.argtypes = [ctypes.c_void_p, c_double_p]
    L.oracle_run_chain.argtypes = [
        ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
        ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    L.oracle_run_chain.restype = ctypes.c_int
    L.oracle_process_buffer.argtypes = [
        ctypes.c_void_p, c_double_p, ctypes.c_uint64, ctypes.c_uint64,
        ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    L.oracle_process_buffer.restype = ctypes.c_int
    L.oracle_guide_reflections.argtypes = [
        ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
        ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    L.oracle_guide_reflections.restype = ctypes.c_int
    L.oracle_ms_step.argtypes = [
        ctypes.c_void_p, ctypes.c_int, c_double_p, ctypes.c_uint64,
        ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int, c_double_p]
    L.oracle_ms_step.restype = ctypes.c_int
    L.oracle_sns_generate.argtypes = [
        ctypes.c_void_p, ctypes.c_double, ctypes.c_double, c_double_p,
        c_double_p]
    L.oracle_guide_one.argtypes = [ctypes.c_void_p, c_double_p]
    L.oracle_guide_one.restype = ctypes.c_int
    L.oracle_source_one.argtypes = [ctypes.c_void_p, ctypes.c_void_p, c_double_p]
    L.oracle_hss_one.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_int, c_double_p]
    L.oracle_anyshape_one.argtypes = [ctypes.c_void_p, c_double_p]
    L.oracle_kernel_scatter_one.argtypes = [ctypes.c_void_p, c_double_p,
                                            ctypes.c_uint64, ctypes.c_uint64]
    L.oracle_expr_eval.restype = ctypes.c_double
    L.oracle_expr_eval.argtypes = [c_double_p, ctypes.c_int, ctypes.c_double]
    L.oracle_apply_transform.argtypes = [c_double_p, c_double_p, c_double_p]
    L.oracle_sqe_lookup.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
    L.oracle_sqe_lookup.restype = ctypes.c_double
    L.oracle_sizeof_chain.restype = ctypes.c_int
    L.oracle_sizeof_component.restype = ctypes.c_int
    return L


def _dp(a):
    return a.ctypes.data_as(c_double_p)


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().oracle_philox4x32_10(c, k, o)
    return list(o)


def intersect_sphere(x, y, z, vx, vy, vz, R):
    a, b = ctypes.c_double(), ctypes.c_double()
    lib().oracle_intersect_sphere(x, y, z, vx, vy, vz, R, ctypes.byref(a),
                                  ctypes.byref(b))
    return a.value, b.value


def intersect_cylinder(x, y, z, vx, vy, vz, R, H):
    a, b = ctypes.c_double(), ctypes.c_double()
    lib().oracle_intersect_cylinder(x, y, z, vx, vy, vz, R, H, ctypes.byref(a),
                                    ctypes.byref(b))
    return a.value, b.value


def intersect_box(x, y, z, vx, vy, vz, W, H, D):
    a, b = ctypes.c_double(), ctypes.c_double()
    lib().oracle_intersect_box(x, y, z, vx, vy, vz, W, H, D, ctypes.byref(a),
                               ctypes.byref(b))
    return a.value, b.value


def locate(comp_struct, x, y, z):
    return lib().oracle_locate(ctypes.byref(comp_struct), x, y, z)


def intersect(comp_struct, ray):
    ts = np.full(10, np.nan)
    n = lib().oracle_intersect(ctypes.byref(comp_struct), *[float(v) for v in ray], _dp(ts))
    return ts[:n]


def insert_sorted(d, l, N):
    l = np.ascontiguousarray(l, dtype=np.float64)
    n = lib().oracle_insert_sorted(float(d), _dp(l), int(N), l.size)
    return n, l


def time_to_scatter(ts, ninter, rand):
    ts = np.ascontiguousarray(ts, dtype=np.float64)
    o = np.zeros(3)
    lib().oracle_time_to_scatter(_dp(ts), int(ninter), float(rand), _dp(o))
    return tuple(o)


def total_time_in_shape(ts, ninter):
    ts = np.ascontiguousarray(ts, dtype=np.float64)
    return lib().oracle_total_time_in_shape(_dp(ts), int(ninter))


def time_to_enter(ts, ninter):
    ts = np.ascontiguousarray(ts, dtype=np.float64)
    return lib().oracle_time_to_enter(_dp(ts), int(ninter))


def rotate(v, c, angle, epsilon=1e-7):
    v = np.array(v, dtype=np.float64)
    c = np.array(c, dtype=np.float64)
    lib().oracle_rotate(_dp(v), _dp(c), float(angle), float(epsilon))
    return v


def reflectivity(Q, R0, Qc, alpha, m, W):
    return lib().oracle_reflectivity(Q, R0, Qc, alpha, m, W)


def _neutron_op(fn, comp_struct, neutron):
    st = np.array(neutron, dtype=np.float64)
    r = fn(ctypes.byref(comp_struct), _dp(st))
    return st, r


def propagate_out(comp, n):
    return _neutron_op(lib().oracle_propagate_out, comp, n)[0]


def tof_before_first_exit(comp, n):
    return _neutron_op(lib().oracle_tof_before_first_exit, comp, n)[1]


def propagate_to_next_incident_surface(comp, n):
    return _neutron_op(lib().oracle_propagate_to_next_incident_surface, comp, n)


def propagate_to_next_exiting_surface(comp, n):
    return _neutron_op(lib().oracle_propagate_to_next_exiting_surface, comp, n)[0]


def guide_one(comp, n):
    return _neutron_op(lib().oracle_guide_one, comp, n)


def source_one(comp, uniforms):
    st = np.zeros(10)
    u = np.ascontiguousarray(uniforms, dtype=np.float32)
    lib().oracle_source_one(ctypes.byref(comp), u.ctypes.data, _dp(st))
    return st


def hss_one(comp, neutron, uniforms):
    st = np.array(neutron, dtype=np.float64)
    u = np.ascontiguousarray(uniforms, dtype=np.float32)
    lib().oracle_hss_one(ctypes.byref(comp), u.ctypes.data, u.size, _dp(st))
    return st


def anyshape_one(comp, neutron):
    """The mesh guide (Guide_anyshape) on one neutron state; returns
    (state, 1 if the bounce limit was reached)."""
    st = np.array(neutron, dtype=np.float64)
    over = lib().oracle_anyshape_one(ctypes.byref(comp), _dp(st))
    return st, over


def kernel_scatter_one(comp, neutron, seed=1, index=0):
    """The HSS kernel's scatter (p *= sigma, then S) on one neutron."""
    st = np.array(neutron, dtype=np.float64)
    lib().oracle_kernel_scatter_one(ctypes.byref(comp), _dp(st), int(seed),
                                    int(index))
    return st


def expr_eval(prog, Q):
    """An E_Q kernel program ({opcode, argument} rows) at Q."""
    p = np.ascontiguousarray(prog, dtype=np.float64).reshape(-1)
    return lib().oracle_expr_eval(_dp(p), p.size // 2, float(Q))


def sqe_lookup(comp, Q, E):
    return lib().oracle_sqe_lookup(ctypes.byref(comp), float(Q), float(E))


def run_chain(chain, ncount, seed=1, first=0, uniforms=None, record=False,
              nthreads=0, timing=False):
    """Run the chain on the CPU (`timing`: on the timed-baseline build).
    Tallies land in the host memory the chain's components were bound to.
    Returns (stats dict, neutrons, last)."""
    stats = (ctypes.c_uint64 * 4)()
    out = np.zeros((ncount, 10)) if record else None
    last = np.zeros(ncount, dtype=np.int32) if record else None
    uptr, stride = None, 0
    if uniforms is not None:
        u = np.ascontiguousarray(uniforms, dtype=np.float32)
        assert u.ndim == 2 and u.shape[0] == ncount
        uptr, stride = u.ctypes.data, u.shape[1]
    L = timing_lib() if timing else lib()
    rc = L.oracle_run_chain(
        ctypes.byref(chain), int(ncount), int(first), int(seed), uptr, stride,
        out.ctypes.data if record else None,
        last.ctypes.data if record else None, int(nthreads), stats)
    if rc != 0:
        raise RuntimeError(f"oracle_run_chain failed ({rc}); stats {list(stats)}")
    return ({"processed": stats[0], "bounce_overflow": stats[1],
             "nonfinite": stats[2]}, out, last)


def guide_reflections(chain, ncount, seed=1, first=0, nbins=64,
                      nthreads=0):
    """Histogram (ncomp, nbins) of reflections per guide traversal: row k
    counts the neutrons that entered guide component k by how many
    reflections they made there (last bin: nbins - 1 or more)."""
    h = np.zeros((chain.ncomp, nbins), dtype=np.uint64)
    rc = lib().oracle_guide_reflections(ctypes.byref(chain), int(ncount),
                                        int(first), int(seed), int(nthreads),
                                        h.ctypes.data, int(nbins))
    if rc != 0:
        raise RuntimeError(f"oracle_guide_reflections failed ({rc})")
    return h


MS_STEPS = {"interactM1": 0, "interactM_path1": 1, "scatterM": 2}


def ms_step(comp, step, neutron, seed=1, index=0, uniforms=None):
    """One step of the multiple scatterer (homogeneous_multiple_scatterer.py)
    on a neutron state: returns (output neutrons (N, 10), the input state as
    the step left it)."""
    st = np.array(neutron, dtype=np.float64).reshape(10).copy()
    out = np.zeros((64, 10))
    uptr, stride = None, 0
    if uniforms is not None:
        u = np.ascontiguousarray(uniforms, dtype=np.float32).reshape(-1)
        uptr, stride = u.ctypes.data, u.size
    n = lib().oracle_ms_step(ctypes.byref(comp), MS_STEPS[step], _dp(st),
                             int(seed), int(index), uptr, stride, _dp(out))
    return out[:n].copy(), st


def sns_generate(comp, randE, randt):
    """The SNS source's (E in meV, t in s) for two uniforms
    (SNS_source.generate)."""
    E, t = ctypes.c_double(), ctypes.c_double()
    lib().oracle_sns_generate(ctypes.byref(comp), float(randE), float(randt),
                              ctypes.byref(E), ctypes.byref(t))
    return E.value, t.value


def process_buffer(chain, neutrons, seed=1, first=0, nthreads=0):
    a = np.array(neutrons, dtype=np.float64).reshape(-1, 10)
    stats = (ctypes.c_uint64 * 4)()
    rc = lib().oracle_process_buffer(ctypes.byref(chain), _dp(a), a.shape[0],
                                     int(first), int(seed), int(nthreads), stats)
    if rc != 0:
        raise RuntimeError(f"oracle_process_buffer failed ({rc})")
    return a
