"""Constant-(Q, E) and E(Q) kernels: the oracle against the reference's
kernel tests, and the host-side expression compiler.

tests/kernels/test_constant_qe.py:25-65 scatters one 60 meV neutron along z
with Q = 3 /A, E = 30 meV and checks the transfer to 7 decimals;
tests/kernels/test_E_Q.py:15-34 scatters 2000 m/s neutrons along z with
E(Q) = 5 sin(Q)^2 + 5, S(Q) = 1 over Q 0-15 /A and checks E = E(Q) for
each.  The same checks run here on the oracle over many seeds and incident
directions.
"""

import math

import numpy as np
import pytest

from acc_gb300 import _native as nat
from acc_gb300.components.samples.homogeneous_single_scatterer import factory
from acc_gb300.conversion import V2K, e2v, v2e
from acc_gb300.geometry import Block
from acc_gb300.kernels import ConstantQEKernel, E_Q_Kernel
from acc_gb300.kernels.expression import compile_expression, evaluate
from acc_gb300.memory import HostBinder
from oracle import binding as O


def _comp(kernel):
    return factory(Block(0.06, 0.10, 0.01), kernel)("s").to_struct(HostBinder())


def _transfer(n0, n1):
    vi, vf = np.asarray(n0[3:6]), np.asarray(n1[3:6])
    E = v2e(np.linalg.norm(vi)) - v2e(np.linalg.norm(vf))
    Q = V2K * np.linalg.norm(vi - vf)
    return Q, E


DIRECTIONS = [(0, 0, 1), (1, 0, 0), (0, 1, 0), (0.3, -0.2, 0.9),
              (0.05, 0.05, 1.0), (-1, 0.01, 0.02)]


@pytest.mark.parametrize("d", DIRECTIONS)
def test_constant_qe_transfer(oracle_lib, d):
    Q, E, Ei = 3.0, 30.0, 60.0
    comp = _comp(ConstantQEKernel(Q, E, 0.0, 1.0))
    d = np.asarray(d, float) / np.linalg.norm(d)
    n0 = np.r_[0, 0, 0, d * e2v(Ei), 0, 0, 0, 1.0]
    for seed in range(1, 51):
        n1 = O.kernel_scatter_one(comp, n0, seed=seed, index=seed * 7)
        q, e = _transfer(n0, n1)
        np.testing.assert_almost_equal(e, E)
        np.testing.assert_almost_equal(q, Q)
        assert n1[9] == 1.0  # p *= sigma = 1, no other factor


def test_constant_qe_weight_and_closed_transfers(oracle_lib):
    n0 = np.r_[0, 0, 0, 0, 0, e2v(60.0), 0, 0, 0, 0.5]
    n1 = O.kernel_scatter_one(_comp(ConstantQEKernel(3.0, 30.0, 0.0, 7.0)), n0)
    assert n1[9] == 0.5 * 7.0
    # E above Ei, and Q beyond ki + kf: absorbed
    for Q, E in ((3.0, 61.0), (20.0, 30.0), (0.1, 30.0)):
        n1 = O.kernel_scatter_one(_comp(ConstantQEKernel(Q, E, 0.0, 1.0)), n0)
        assert n1[9] == -1.0, (Q, E)


@pytest.mark.parametrize("d", DIRECTIONS)
def test_e_q_dispersion(oracle_lib, d):
    E_Q = "5*sin(Q)**2+5"
    comp = _comp(E_Q_Kernel(E_Q, "1", 0.0, 15.0, 0.0, 1.0))
    d = np.asarray(d, float) / np.linalg.norm(d)
    n0 = np.r_[0, 0, 0, d * 2000.0, 0, 0, 0, 1.0]
    for seed in range(1, 101):
        n1 = O.kernel_scatter_one(comp, n0, seed=seed, index=seed)
        assert n1[9] > 0
        q, e = _transfer(n0, n1)
        assert np.isclose(e, eval(E_Q, dict(Q=q, sin=np.sin))), (seed, q, e)


def test_e_q_weight(oracle_lib):
    """p = sigma S(Q) (vf/vi) Q (Qmax-Qmin) / (2 ki kf) / tries
    (E_Q.py:94-95); elastic E(Q) = 0 with Q < 2 ki accepts the first
    draw, so tries = 1."""
    Qmin, Qmax, sigma = 0.5, 5.0, 3.0
    comp = _comp(E_Q_Kernel("0", "exp(-Q/4)", Qmin, Qmax, 0.0, sigma))
    vi = 2000.0
    n0 = np.r_[0, 0, 0, 0, 0, vi, 0, 0, 0, 1.0]
    ki = V2K * vi
    assert 2 * ki > Qmax
    for seed in range(1, 41):
        n1 = O.kernel_scatter_one(comp, n0, seed=seed)
        q, e = _transfer(n0, n1)
        assert abs(e) < 1e-6  # VS2E and SE2V agree to ~1e-9
        vf = np.linalg.norm(n1[3:6])
        kf = V2K * vf
        want = sigma * math.exp(-q / 4) * (vf / vi) * q * (Qmax - Qmin) / (kf * ki) / 2
        np.testing.assert_allclose(n1[9], want, rtol=1e-7)


def test_e_q_counts_rejected_draws(oracle_lib):
    """Only Q above 2 ki is closed for an elastic dispersion: the weight
    carries 1 / (number of draws), and the mean weight over many neutrons
    is sigma E[S (vf/vi) Q (Qmax-Qmin) / (2 ki kf) / tries]; with
    Qmax = 4 ki the accepted fraction is 1/2, and p never exceeds the
    single-draw value."""
    vi = 2000.0
    ki = V2K * vi
    comp = _comp(E_Q_Kernel("0", "1", 0.0, 4 * ki, 0.0, 1.0))
    n0 = np.r_[0, 0, 0, 0, 0, vi, 0, 0, 0, 1.0]
    tries = []
    for seed in range(1, 401):
        n1 = O.kernel_scatter_one(comp, n0, seed=seed)
        q, _ = _transfer(n0, n1)
        single = q * (4 * ki) / (ki * ki) / 2
        t = single / n1[9]
        assert abs(t - round(t)) < 1e-9 and round(t) >= 1
        tries.append(round(t))
    # geometric with success 1/2: mean 2
    assert 1.7 < np.mean(tries) < 2.3


def test_e_q_no_accepted_draw_zeroes_the_weight(oracle_lib):
    comp = _comp(E_Q_Kernel("1000", "1", 0.0, 5.0, 0.0, 1.0))
    n0 = np.r_[0, 0, 0, 0, 0, 2000.0, 0, 0, 0, 1.0]
    n1 = O.kernel_scatter_one(comp, n0)
    assert n1[9] == 0.0
    np.testing.assert_array_equal(n1[3:6], n0[3:6])


EXPRESSIONS = [
    "5*sin(Q)**2+5", "30+20*sin(Q)", "1", "Q", "-Q**3 + 2*Q - 1",
    "exp(-Q/4)*cos(2*pi*Q)", "sqrt(Q+1) / (1 + Q^2)", "log(Q+2, 3)",
    "atan2(Q, 2) + tanh(Q - 3)", "abs(Q - 4) % 1.5", "Q // 2",
    "pow(Q, 2.5) - pow(Q, 2)", "min(Q, 3) + max(Q, 5)", "erf(Q/3)*erfc(Q/5)",
    "floor(Q) + ceil(Q/2)", "asinh(Q) + acosh(Q+1) + atanh(Q/20)",
    "log10(Q+1) + sinh(Q/5) + cosh(Q/7)", "1/Q**2", "e**(-Q)",
    "asin(Q/20) + acos(Q/20) + atan(Q) + tan(Q/10)",
    "((((Q+1)*(Q+2))*((Q+3)*(Q+4)))*(((Q+5)*(Q+6))*((Q+7)*(Q+8))))",
]


@pytest.mark.parametrize("text", EXPRESSIONS)
def test_expression_compiler_matches_python(oracle_lib, text):
    import math as m
    prog = compile_expression(text)
    ns = {k: getattr(m, k) for k in dir(m) if not k.startswith("_")}
    ns.update(abs=abs, min=min, max=max)
    for Q in np.linspace(0.05, 14.9, 37):
        want = eval(text.replace("^", "**"), dict(ns, Q=float(Q)))
        got = evaluate(prog, Q)
        ora = O.expr_eval(prog, Q)
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-300)
        np.testing.assert_allclose(ora, want, rtol=1e-13, atol=1e-300)


def test_expression_folds_constants_and_bounds_the_stack():
    assert compile_expression("2*pi*3").shape == (1, 2)
    # x**n with integer n is binary powering
    assert compile_expression("Q**3")[-1, 0] == 9
    deep = "Q+(Q+(Q+(Q+(Q+(Q+(Q+(Q+Q)))))))"
    with pytest.raises(ValueError, match="stack"):
        compile_expression(deep)
    for bad in ("Q if Q > 1 else 2", "foo(Q)", "x + 1", "Q < 3",
                "factorial(Q)", "[Q]", "sin(Q, 2)", "'a'"):
        with pytest.raises(ValueError):
            compile_expression(bad)


def test_malformed_program_gives_nan(oracle_lib):
    # stack underflow, overflow and an unknown opcode
    assert math.isnan(O.expr_eval(np.array([[3, 0]]), 1.0))
    assert math.isnan(O.expr_eval(np.array([[2, 0]] * 9 + [[3, 0]] * 8), 1.0))
    assert math.isnan(O.expr_eval(np.array([[2, 0], [99, 0]]), 1.0))
    assert math.isnan(O.expr_eval(np.array([[2, 0], [2, 0]]), 1.0))


def test_composite_picks_elements_by_weight(oracle_lib):
    """composite.py:62-75, 101-104: one uniform picks element i with
    probability w_i (weights 1 and 3, normalised), the element scatters
    (p *= its sigma, then its S) and p /= w_i.  Two constant-(Q, E)
    elements tell which one scattered by the energy transfer."""
    from acc_gb300.engine import build_chain
    from acc_gb300.kernels import CompositeKernel
    k1 = ConstantQEKernel(2.0, 10.0, 0.0, 5.0)
    k2 = ConstantQEKernel(3.0, 20.0, 0.0, 7.0)
    H = factory(Block(0.06, 0.10, 0.01), CompositeKernel([k1, k2], [1, 3]))
    ch = build_chain([H("s")], binder=HostBinder())
    assert ch.ncomp == 3 and ch.comp[0].ip[4] == 2
    assert [ch.comp[i].opcode for i in (1, 2)] == [nat.OP_KERNEL_ELEMENT] * 2
    np.testing.assert_allclose([ch.comp[1].dp[22], ch.comp[2].dp[22]],
                               [0.25, 0.75])
    assert ch.comp[2].dp[23] == 1.0
    assert ch.comp[0].dp[9] == 12.0  # sigma: the sum (not averaged)
    n0 = np.r_[0, 0, 0, 0, 0, e2v(60.0), 0, 0, 0, 1.0]
    first = 0
    N = 2000
    for seed in range(N):
        n1 = O.kernel_scatter_one(ch.comp[0], n0, seed=seed + 1, index=seed)
        q, e = _transfer(n0, n1)
        if abs(e - 10.0) < 1e-6:
            first += 1
            assert abs(q - 2.0) < 1e-6 and n1[9] == pytest.approx(5.0 / 0.25)
        else:
            assert abs(e - 20.0) < 1e-6 and abs(q - 3.0) < 1e-6
            assert n1[9] == pytest.approx(7.0 / 0.75)
    assert abs(first / N - 0.25) < 4 * np.sqrt(0.25 * 0.75 / N)


def test_un_kernel_packs_the_reference_sample(oracle_lib):
    """tests/kernels/UN/UN-scatterer.xml: 8 E(Q) levels averaged; sigma
    and mu of the composite are then those of one level."""
    from acc_gb300 import instruments
    from acc_gb300.engine import chain_for_instrument
    ch = chain_for_instrument(instruments.un_ms(), HostBinder())
    c = ch.comp[1]
    assert c.opcode == nat.OP_HMS and c.ip[1] == nat.KERNEL_COMPOSITE
    assert c.ip[4] == 8 and c.ip[6] == 33
    np.testing.assert_allclose([c.dp[8], c.dp[9], c.dp[10]],
                               [32.395, 69.847, 0.125])
    # level 3: E = 150 meV, S = (a Q^2)^3 / 3! exp(-a Q^2)
    from acc_gb300.kernels.expression import evaluate
    k3 = instruments.un_kernel().elements[3]
    a = 0.00276
    for Q in (1.0, 7.5, 20.0):
        assert evaluate(k3.E_prog, Q) == 150.0
        want = (a * Q * Q) ** 3 / 6 * math.exp(-a * Q * Q)
        np.testing.assert_allclose(evaluate(k3.S_prog, Q), want, rtol=1e-14)


def test_sans2d_transfer_and_weight(oracle_lib):
    """SANS2D_ongrid.S (acc/kernels/SANS2D_ongrid.py:24-56): the drawn
    (Qx, Qy) comes back from the velocity change as (vi - vf) V2K in x and
    y; vz = sqrt(vi^2 - vx^2 vy^2) (the reference's expression); p = sigma
    times S bilinear on cells of width (Qmax - Qmin) / n, indices clamped
    to [0, n-2]; the image is indexed (y, x)."""
    from acc_gb300.kernels import SANS2D_ongrid_Kernel
    rng = np.random.default_rng(3)
    img = rng.random((7, 9))  # (ny, nx)
    qx0, qx1, qy0, qy1 = -0.01, 0.02, -0.005, 0.004
    sigma = 3.0
    comp = _comp(SANS2D_ongrid_Kernel(img, qx0, qx1, qy0, qy1, 0.0, sigma))
    v0 = np.array([1.5, -0.7, 400.0])
    n0 = np.r_[0, 0, 0, v0, 0, 0, 0, 1.0]
    S = img.T
    nx, ny = S.shape
    for seed in range(1, 200):
        n1 = O.kernel_scatter_one(comp, n0, seed=seed)
        Qx = (v0[0] - n1[3]) * V2K
        Qy = (v0[1] - n1[4]) * V2K
        assert qx0 <= Qx < qx1 and qy0 <= Qy < qy1
        vi2 = v0 @ v0
        np.testing.assert_allclose(n1[5], math.sqrt(vi2 - n1[3] ** 2 * n1[4] ** 2),
                                   rtol=1e-14)
        dx, dy = (qx1 - qx0) / nx, (qy1 - qy0) / ny
        xi = min(max(int((Qx - qx0) / dx), 0), nx - 2)
        yi = min(max(int((Qy - qy0) / dy), 0), ny - 2)
        fx, fy = (Qx - qx0) / dx - xi, (Qy - qy0) / dy - yi
        s = (S[xi, yi] * (1 - fx) * (1 - fy) + S[xi + 1, yi] * fx * (1 - fy)
             + S[xi, yi + 1] * (1 - fx) * fy + S[xi + 1, yi + 1] * fx * fy)
        np.testing.assert_allclose(n1[9], sigma * s, rtol=1e-9)


def test_dgssxres_kernel_reference_case(oracle_lib):
    """tests/kernels/test_DGSSXRes.py:23-66: a 3000 m/s neutron along z at
    t = 1 s scattering towards a target 3 m along x (radius 0.025 m), to
    arrive at 1.001 s +- 5 us: elastic within 0.5 meV, Q = 6.74 /A within
    1%.  Also: the direction lies in the target's cone, and the weight is
    sigma * solid angle / 4 pi * dtof * (2 Ef / tof) * vf / vi."""
    from acc_gb300.kernels import DGSSXResKernel
    sigma = 2.0
    comp = _comp(DGSSXResKernel((3.0, 0.0, 0.0), 0.025, 1.001, 1e-5, 0.0,
                                sigma))
    n0 = np.r_[0, 0, 0, 0, 0, 3000.0, 0, 0, 1.0, 1.0]
    cmax = math.sqrt(9.0 / (0.025 ** 2 + 9.0))
    for seed in range(1, 101):
        n1 = O.kernel_scatter_one(comp, n0, seed=seed)
        q, e = _transfer(n0, n1)
        np.testing.assert_allclose(e, 0.0, atol=0.5)
        np.testing.assert_allclose(q, 6.74, rtol=1e-2)
        vf = n1[3:6]
        vfl = np.linalg.norm(vf)
        assert vf[0] / vfl >= cmax - 1e-9  # inside the cone towards +x
        tof = 3.0 / vfl + 1.0
        assert abs(tof - 1.001) <= 5e-6 * (1 + 1e-9)
        Ef = v2e(vfl)
        want = sigma * 2 * math.pi * (1 - cmax) / (4 * math.pi) * 1e-5 \
            * (2 * Ef / tof) * vfl / 3000.0
        np.testing.assert_allclose(n1[9], want, rtol=1e-9)
