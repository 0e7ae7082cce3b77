"""Forward-mode sensitivities d s_H / d theta, Fisher scores and the differentiable window cost.

Tolerances: J within 1e-3 (per-window Frobenius relative error) of FP64 central differences of
the oracle with h = 1e-6; Fisher matrices within 1e-5 of the same reduction in FP64; the
autograd gradient within 1e-3 of FP64 central differences of the oracle's cost.
"""
import numpy as np
import pytest
import torch

from oracle import cost as oc
from oracle import dynamics as dyn
from oracle import fisher as ofi
from oracle import go2_model as gm
from helpers import oracle_windows, random_theta

pytestmark = pytest.mark.gpu
H_FD = 1e-6


def _fd_jacobian(x0, acts, theta, sim):
    """Central differences of the oracle's final states: [N, W, 37, 13]."""
    N, W = theta.shape[0], x0.shape[0]
    out = np.zeros((N, W, 37, 13))
    for k in range(13):
        tp, tm = theta.copy(), theta.copy()
        tp[:, k] += H_FD
        tm[:, k] -= H_FD
        th = np.concatenate([np.repeat(tp, W, 0), np.repeat(tm, W, 0)])
        xs = dyn.rollout(np.tile(x0, (2 * N, 1)), np.tile(acts, (2 * N, 1, 1)), th, sim)
        out[..., k] = ((xs[:N * W] - xs[N * W:]) / (2 * H_FD)).reshape(N, W, 37)
    return out


@pytest.fixture(scope="module")
def case(built):
    from spi_gb300.engine import Engine
    rng = np.random.default_rng(41)
    _, init, actions, target = oracle_windows(8, n_traj=2, T=26, H=20)
    sel = rng.choice(init.shape[0], 4, replace=False)
    init, actions, target = init[sel], actions[sel], target[sel]
    theta = random_theta(rng, 2)
    e = Engine()
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
    return e, init.astype(np.float64), actions.astype(np.float64), target.astype(np.float64), theta


def test_sensitivity_matches_fp64_central_differences(case):
    from spi_gb300.sensitivity import sensitivities
    e, x0, acts, target, theta = case
    th32 = theta.astype(np.float32)
    J, xH = sensitivities(e, torch.from_numpy(th32), list(range(13)))
    J = J.cpu().numpy().astype(np.float64)
    ref = _fd_jacobian(x0, acts, th32.astype(np.float64), gm.SimParams())
    num = np.sqrt(((J - ref) ** 2).sum(axis=(2, 3)))
    den = np.sqrt((ref ** 2).sum(axis=(2, 3)))
    assert (num / den).max() <= 1e-3, (num / den)
    # the primal part of the dual rollout is the ordinary rollout
    xs = dyn.rollout(np.tile(x0, (2, 1)), np.tile(acts, (2, 1, 1)), np.repeat(th32.astype(np.float64), 4, 0),
                     gm.SimParams())
    np.testing.assert_allclose(xH.cpu().numpy().reshape(8, 37), xs, rtol=1e-4, atol=1e-4)


def test_fisher_and_logdet_match_fp64(case):
    from spi_gb300.sensitivity import block_weights, fisher, sensitivities
    e, x0, acts, target, theta = case
    J, _ = sensitivities(e, torch.from_numpy(theta.astype(np.float32)), list(range(13)))
    q = block_weights((10.0, 5.0, 0.1, 0.1, 1.0, 0.01))
    F, logdet, trace = fisher(J, q, eps=1e-9)
    Jn = J.cpu().numpy().astype(np.float64)
    Fr = ofi.fisher_matrix(Jn, q.astype(np.float64))
    np.testing.assert_allclose(F.cpu().numpy(), Fr, rtol=1e-5, atol=1e-6 * np.abs(Fr).max())
    np.testing.assert_allclose(logdet.cpu().numpy(), ofi.fisher_logdet(Fr, 1e-9), rtol=1e-4)
    np.testing.assert_allclose(trace.cpu().numpy(), np.trace(Fr, axis1=1, axis2=2), rtol=1e-5)


def test_fisher_on_tensor_cores(case):
    """BF16 operands, FP32 accumulation: within 1e-2 of the FP64 reduction (BF16 has 8 mantissa bits)."""
    from spi_gb300.sensitivity import block_weights, fisher, sensitivities
    e, x0, acts, target, theta = case
    J, _ = sensitivities(e, torch.from_numpy(theta.astype(np.float32)), list(range(13)))
    q = block_weights((10.0, 5.0, 0.1, 0.1, 1.0, 0.01))
    F, logdet, trace = fisher(J, q, eps=1e-9, tensor_cores=True)
    Fr = ofi.fisher_matrix(J.cpu().numpy().astype(np.float64), q.astype(np.float64))
    err = np.abs(F.cpu().numpy() - Fr).max(axis=(1, 2)) / np.abs(Fr).max(axis=(1, 2))
    assert err.max() <= 1e-2, err
    np.testing.assert_allclose(trace.cpu().numpy(), np.trace(Fr, axis1=1, axis2=2), rtol=1e-2)


def test_window_cost_autograd_matches_fd(case):
    from spi_gb300.sensitivity import WindowCost, block_weights
    e, x0, acts, target, theta = case
    w6 = (10.0, 5.0, 0.1, 0.1, 1.0, 0.01)
    th = torch.from_numpy(theta.astype(np.float32)).cuda().requires_grad_(True)
    cost = WindowCost.apply(th, e, w6)
    cost.sum().backward()
    g = th.grad.cpu().numpy().astype(np.float64)
    q = block_weights(w6).astype(np.float64)

    def oracle_cost(t):
        xs = dyn.rollout(np.tile(x0, (t.shape[0], 1)), np.tile(acts, (t.shape[0], 1, 1)), np.repeat(t, 4, 0),
                         gm.SimParams())
        d = xs - np.tile(target, (t.shape[0], 1))
        return (q * d * d).sum(-1).reshape(t.shape[0], 4).mean(1)

    base = theta.astype(np.float32).astype(np.float64)
    ref = np.zeros_like(g)
    for k in range(13):
        tp, tm = base.copy(), base.copy()
        tp[:, k] += H_FD
        tm[:, k] -= H_FD
        ref[:, k] = (oracle_cost(tp) - oracle_cost(tm)) / (2 * H_FD)
    np.testing.assert_allclose(cost.detach().cpu().numpy(), oracle_cost(base), rtol=1e-4)
    rel = np.linalg.norm(g - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert rel.max() <= 1e-3, rel


def test_excitation_scoring_end_to_end(built):
    from spi_gb300.engine import Engine
    from spi_gb300.robot import THETA_NOMINAL
    from spi_gb300.sensitivity import multisine_actions, score_excitations
    e = Engine()
    cfg = e.cfg
    acts, _ = multisine_actions(16, 4 * 20, cfg.control_dt, cfg.action_scale, seed=3, settle=100)
    r = score_excitations(e, THETA_NOMINAL, acts, windows_per_cand=4, horizon=20, settle=100)
    assert np.isfinite(r["logdet"]).all() and np.isfinite(r["trace"]).all()
    assert r["best"] == int(np.argmax(r["logdet"]))
    F = r["F"].cpu().numpy()
    np.testing.assert_allclose(np.trace(F, axis1=1, axis2=2), r["trace"], rtol=1e-5)


@pytest.fixture(scope="module")
def adj_case(built):
    """16 theta x 24 windows x H = 20 with window weights: the C3 shape (13 parameters, H = 20)."""
    from spi_gb300.engine import Engine
    rng = np.random.default_rng(43)
    _, init, actions, target = oracle_windows(9, n_traj=3, T=30, H=20)
    sel = rng.choice(init.shape[0], 24, replace=False)
    init, actions, target = init[sel], actions[sel], target[sel]
    target = target + (0.01 * rng.standard_normal(target.shape)).astype(np.float32)
    weight = (rng.random(24) > 0.25).astype(np.float32)
    theta = random_theta(rng, 16)
    e = Engine()
    e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target),
                   torch.from_numpy(weight), norm=float(weight.sum()))
    return e, init.astype(np.float64), actions.astype(np.float64), target.astype(np.float64), weight, theta


def _oracle_cost(x0, acts, target, weight, t, mode, w6=(10.0, 5.0, 0.1, 0.1, 1.0, 0.01)):
    from spi_gb300.sensitivity import block_weights
    W = x0.shape[0]
    xs = dyn.rollout(np.tile(x0, (t.shape[0], 1)), np.tile(acts, (t.shape[0], 1, 1)), np.repeat(t, W, 0),
                     gm.SimParams())
    d = (xs - np.tile(target, (t.shape[0], 1))).reshape(t.shape[0], W, 37)
    if mode == 1:
        c = (block_weights(w6).astype(np.float64) * d * d).sum(-1)
    else:
        c = (10 * np.linalg.norm(d[..., 0:3], axis=-1) + 5 * np.linalg.norm(d[..., 3:7], axis=-1)
             + np.linalg.norm(d[..., 13:25], axis=-1))
    return (c * weight).sum(1) / weight.sum()


@pytest.mark.parametrize("mode", [1, 0])
def test_adjoint_gradient_matches_fp64_central_differences(adj_case, mode):
    """The hand-written adjoint (spi_adjoint) against FP64 central differences (h = 1e-6) of the
    oracle's cost, for both cost modes: <= 1e-3 in |g - ref| / |ref| per theta sample."""
    from spi_gb300.engine import COST_REF, COST_SQ
    from spi_gb300.sensitivity import adjoint
    e, x0, acts, target, weight, theta = adj_case
    e.set_cost(COST_SQ if mode == 1 else COST_REF)
    th32 = theta.astype(np.float32)
    cost, grad = adjoint(e, torch.from_numpy(th32))
    torch.cuda.synchronize()
    assert e.sync() == 0
    base = th32.astype(np.float64)
    ref = np.zeros((base.shape[0], 13))
    for k in range(13):
        tp, tm = base.copy(), base.copy()
        tp[:, k] += H_FD
        tm[:, k] -= H_FD
        ref[:, k] = (_oracle_cost(x0, acts, target, weight, tp, mode)
                     - _oracle_cost(x0, acts, target, weight, tm, mode)) / (2 * H_FD)
    np.testing.assert_allclose(cost.cpu().numpy(), _oracle_cost(x0, acts, target, weight, base, mode), rtol=1e-4)
    g = grad.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(g - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert rel.max() <= 1e-3, rel
    e.set_cost(COST_SQ)


def test_adjoint_equals_forward_mode_gradient(adj_case):
    """One reverse sweep and 13 tangent sweeps give the same gradient (unit window weights)."""
    from spi_gb300.engine import Engine
    from spi_gb300.sensitivity import adjoint, tangent_gradient
    _, x0, acts, target, _, theta = adj_case
    e = Engine()
    e.load_windows(torch.from_numpy(x0.astype(np.float32)), torch.from_numpy(acts.astype(np.float32)),
                   torch.from_numpy(target.astype(np.float32)))
    th = torch.from_numpy(theta.astype(np.float32))
    c_adj, g_adj = adjoint(e, th)
    c_fwd, g_fwd = tangent_gradient(e, th)
    torch.cuda.synchronize()
    np.testing.assert_allclose(c_adj.cpu().numpy(), c_fwd.cpu().numpy(), rtol=1e-4)
    ga, gf = g_adj.cpu().numpy().astype(np.float64), g_fwd.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(ga - gf, axis=1) / np.linalg.norm(gf, axis=1)
    assert rel.max() <= 1e-3, rel


def test_adjoint_checkpoint_segments_cover_ragged_horizons(built):
    """Horizons that are not a multiple of the 5-step checkpoint interval (H = 7, 13) and a
    window count that is not a multiple of 8: against FP64 central differences."""
    from spi_gb300.engine import Engine
    from spi_gb300.sensitivity import adjoint
    rng = np.random.default_rng(44)
    for H in (7, 13):
        _, init, actions, target = oracle_windows(10 + H, n_traj=2, T=H + 8, H=H)
        init, actions, target = init[:11], actions[:11], target[:11]
        weight = np.ones(11, np.float32)
        theta = random_theta(rng, 3)
        e = Engine()
        e.load_windows(torch.from_numpy(init), torch.from_numpy(actions), torch.from_numpy(target))
        _, grad = adjoint(e, torch.from_numpy(theta.astype(np.float32)))
        base = theta.astype(np.float32).astype(np.float64)
        x0, a64, t64 = init.astype(np.float64), actions.astype(np.float64), target.astype(np.float64)
        ref = np.zeros((3, 13))
        for k in range(13):
            tp, tm = base.copy(), base.copy()
            tp[:, k] += H_FD
            tm[:, k] -= H_FD
            ref[:, k] = (_oracle_cost(x0, a64, t64, weight, tp, 1) - _oracle_cost(x0, a64, t64, weight, tm, 1)) / (2 * H_FD)
        g = grad.cpu().numpy().astype(np.float64)
        rel = np.linalg.norm(g - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert rel.max() <= 1e-3, (H, rel)
