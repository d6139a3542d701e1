"""Backward replay (mcv_backward through acc_gb300.autograd) against
common-random-number finite differences.

With the Philox stream fixed, a tally is a smooth function of every
differentiated parameter (they enter only neutron weights), so a central
difference of the FP64 forward with the same seed converges to the
replayed gradient.  Tolerances: 1e-6 relative for the coefficient-type
parameters (central difference, step 1e-4 relative, O(step^2) truncation);
S(Q,E) nodes enter linearly, checked to 1e-7 relative (the loss
difference of a 1% node change is a sum over many bins); FP32 backward
against FP64 backward within 1e-3 relative for dL/d ln S on the nodes
that carry 1% or more of the largest sensitivity.
"""

import numpy as np
import pytest
import torch

from acc_gb300 import instruments
from acc_gb300.autograd import GradRun

pytestmark = pytest.mark.gpu

N = 200_000


@pytest.fixture(scope="module", autouse=True)
def _engine(engine_lib):
    torch.cuda.init()
    yield


def weights(shape, seed=0):
    g = np.random.default_rng(seed)
    return torch.tensor(g.standard_normal(shape), dtype=torch.float64,
                        device="cuda")


def sqe_run(floattype="float64"):
    ins = instruments.sqe_hollow_cylinder()
    sample, det = ins.components[1], ins.components[2]
    run = GradRun(ins, det, N, seed=5, floattype=floattype,
                  params={"S": ("sqe_table", sample),
                          "mu": ("hss_mu", sample),
                          "sigma": ("hss_sigma", sample)})
    S = torch.tensor(sample.kernel.S, device="cuda")
    mu = torch.tensor(sample.kernel.absorption_coefficient,
                      dtype=torch.float64)
    sigma = torch.tensor(sample.kernel.scattering_coefficient,
                         dtype=torch.float64)
    return run, det, S, mu, sigma


def loss(run, w, **v):
    return float((w * run.forward_hist(v)).sum())


def test_sqe_mu_sigma_gradients_match_crn_differences():
    run, det, S, mu, sigma = sqe_run()
    w = weights(det.hist_shape)
    mu_r = mu.clone().requires_grad_(True)
    sg_r = sigma.clone().requires_grad_(True)
    L = (w * run(S=S, mu=mu_r, sigma=sg_r)).sum()
    L.backward()
    for name, val, grad in (("mu", mu, mu_r.grad), ("sigma", sigma,
                                                    sg_r.grad)):
        h = 1e-4 * float(val)
        kw = dict(S=S, mu=mu, sigma=sigma)
        kw[name] = val + h
        lp = loss(run, w, **kw)
        kw[name] = val - h
        lm = loss(run, w, **kw)
        fd = (lp - lm) / (2 * h)
        assert float(grad) == pytest.approx(fd, rel=1e-6), name


def test_sqe_table_gradient_is_exact_for_linear_nodes():
    run, det, S, mu, sigma = sqe_run()
    w = weights(det.hist_shape, seed=1)
    S_r = S.clone().requires_grad_(True)
    L = (w * run(S=S_r, mu=mu, sigma=sigma)).sum()
    L.backward()
    g = S_r.grad.cpu().numpy()
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    # nodes whose change moves L the most (|dL/dS| S), so that a 1% change
    # is resolved in double
    effect = np.abs(g * S.cpu().numpy())
    for flat in np.argsort(-effect.ravel())[:4]:
        i, j = np.unravel_index(flat, g.shape)
        base = float(S[i, j])
        Sp, Sm = S.clone(), S.clone()
        Sp[i, j] = base * 1.01
        Sm[i, j] = base * 0.99
        d = float(Sp[i, j]) - float(Sm[i, j])
        fd = (loss(run, w, S=Sp, mu=mu, sigma=sigma)
              - loss(run, w, S=Sm, mu=mu, sigma=sigma)) / d
        assert g[i, j] == pytest.approx(fd, rel=1e-7), (i, j)


def test_guide_coating_gradients_match_crn_differences():
    ins = instruments.guide_chain()
    g1, g2, psd = ins.components[1], ins.components[2], ins.components[3]
    run = GradRun(ins, psd, N, seed=3, floattype="float64",
                  params={"m": ("guide_m", [g1, g2]),
                          "alpha": ("guide_alpha", [g1, g2]),
                          "W": ("guide_W", [g1, g2])})
    vals = {"m": torch.tensor(3.0, dtype=torch.float64),
            "alpha": torch.tensor(3.0, dtype=torch.float64),
            "W": torch.tensor(0.003, dtype=torch.float64)}
    w = weights(psd.hist_shape, seed=2)
    req = {k: v.clone().requires_grad_(True) for k, v in vals.items()}
    L = (w * run(**req)).sum()
    L.backward()
    for k in vals:
        h = 1e-4 * float(vals[k])
        kp, km = dict(vals), dict(vals)
        kp[k] = vals[k] + h
        km[k] = vals[k] - h
        fd = (loss(run, w, **kp) - loss(run, w, **km)) / (2 * h)
        assert float(req[k].grad) == pytest.approx(fd, rel=1e-5, abs=1e-12), k


def test_powder_F2_gradient_matches_crn_differences():
    ins = instruments.powder_banked(ntubes=16, npixels=16, ntof=50)
    sample, det = ins.components[5], ins.components[6]
    run = GradRun(ins, det, N, seed=8, floattype="float64",
                  params={"F2": ("powder_F2", sample)})
    F2 = torch.tensor([p.F_squared for p in sample.kernel.peaks],
                      dtype=torch.float64)
    w = weights(det.hist_shape, seed=3)
    F2_r = F2.clone().requires_grad_(True)
    L = (w * run(F2=F2_r)).sum()
    L.backward()
    g = F2_r.grad.numpy()
    for j in np.argsort(-np.abs(g))[:4]:
        h = 1e-4 * float(F2[j])
        Fp, Fm = F2.clone(), F2.clone()
        Fp[j] += h
        Fm[j] -= h
        fd = (loss(run, w, F2=Fp) - loss(run, w, F2=Fm)) / (2 * h)
        assert g[j] == pytest.approx(fd, rel=1e-5), j


def test_fp32_backward_close_to_fp64():
    out = {}
    for ft in ("float64", "float32"):
        run, det, S, mu, sigma = sqe_run(ft)
        w = weights(det.hist_shape, seed=4)
        S_r = S.clone().requires_grad_(True)
        mu_r = mu.clone().requires_grad_(True)
        L = (w * run(S=S_r, mu=mu_r, sigma=sigma)).sum()
        L.backward()
        out[ft] = (S_r.grad.cpu().numpy(), float(mu_r.grad))
    g64, g32 = out["float64"], out["float32"]
    assert g32[1] == pytest.approx(g64[1], rel=1e-3)
    # compare dL/d ln S = S dL/dS: where S is tiny (far tails) the FP32
    # weights are subnormal and dL/dS is large but moves L by nothing
    S = sqe_run()[2].cpu().numpy()
    e64, e32 = g64[0] * S, g32[0] * S
    big = np.abs(e64) > 1e-2 * np.abs(e64).max()
    assert big.sum() > 100
    np.testing.assert_allclose(e32[big], e64[big], rtol=1e-3)


@pytest.mark.parametrize("variant", ["regen", "regen_noqueue"])
def test_fp32_regeneration_backward_equals_thread_backward(variant):
    """The FP32 replay of a chain with guides runs with the forward's
    structure (regeneration, tail queue carrying the tracker state); it
    replays the same neutrons with the same arithmetic as the one-neutron-
    per-thread replay.  The kernels may contract different multiply-adds
    into FMAs, which moves a neutron within an ulp of a bin edge into the
    next bin (a different dL/d(sum p) weight); the sums have random-sign
    terms, so the bound is on the gradient vector's scale: every component
    within 1e-6 relative or 2e-5 of the largest component.  A lost tracker
    state would move components by their own size."""
    from acc_gb300 import engine
    ins = instruments.powder_banked(ntubes=16, npixels=16, ntof=50)
    sample, det = ins.components[5], ins.components[6]
    run = GradRun(ins, det, N, seed=8, floattype="float32",
                  params={"F2": ("powder_F2", sample),
                          "m": ("guide_m", [ins.components[1],
                                            ins.components[2]])})
    dout = weights(det.hist_shape, seed=6).reshape(-1).contiguous()
    kF = run._index(sample)
    kg = [run._index(ins.components[1]), run._index(ins.components[2])]
    out = {}
    for v in (variant, "thread"):
        dF = torch.zeros(run.chain.comp[kF].ip[4], dtype=torch.float64,
                         device="cuda")
        dm = {k: torch.zeros(3, dtype=torch.float64, device="cuda")
              for k in kg}
        engine.backward(run.chain, N, {run.mon_index: dout}, dm, {kF: dF},
                        seed=8, floattype="float32", variant=v)
        out[v] = (dF.cpu().numpy(), [dm[k].cpu().numpy() for k in kg])
    a, b = out[variant], out["thread"]
    assert np.abs(b[0]).max() > 0 and np.abs(b[1][0]).max() > 0
    np.testing.assert_allclose(a[0], b[0], rtol=1e-6,
                               atol=2e-5 * np.abs(b[0]).max())
    for x, y in zip(a[1], b[1]):
        np.testing.assert_allclose(x, y, rtol=1e-6,
                                   atol=2e-5 * np.abs(y).max())
