"""Shared helpers for the parity tests: run one instrument on the CPU oracle
and on the GPU engine with the same Philox stream, and compare."""

import numpy as np

from acc_gb300.engine import chain_for_instrument
from acc_gb300.memory import HostBinder
from acc_gb300.stats import chi2_per_dof  # noqa: F401


def oracle_run(ins, ncount, seed=7, first=0, record=False, uniforms=None,
               nthreads=0):
    """Oracle run of `ins`; returns (tallies {component: (3, *shape)},
    stats, neutrons, last)."""
    from oracle import binding as O
    b = HostBinder()
    ch = chain_for_instrument(ins, b)
    stats, out, last = O.run_chain(ch, ncount, seed=seed, first=first,
                                   record=record, uniforms=uniforms,
                                   nthreads=nthreads)
    tallies = {c: b.out(c) for c in ins.components if id(c) in b.tallies}
    return tallies, stats, out, last


def gpu_tallies(ins):
    from acc_gb300.components.monitors.MonitorBase import MonitorBase
    return {c: c.out for c in ins.components if isinstance(c, MonitorBase)}


def field_scale(ref):
    """Per-field scale of a (N, 10) neutron array: the RMS magnitude of
    each slot over the batch (floors the denominator of relative errors
    for slots that cross zero)."""
    s = np.sqrt(np.mean(np.where(np.isfinite(ref), ref, 0.0) ** 2, axis=0))
    return np.where(s > 0, s, 1.0)


def rel_err(a, b):
    """|a - b| / max(|b|, field RMS), elementwise; NaN pairs count as 0."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b) / np.maximum(np.abs(b), field_scale(b))
    d[both_nan] = 0.0
    d[np.isnan(d)] = np.inf
    return d
