"""The kernel's dynamics source (csrc/dynamics.cuh), built for the host in FP64, against the oracle.

Proves on the CPU that the equations the sm_103a kernel executes are the oracle's
equations; the GPU tests then only have FP32 rounding and the lane plumbing to check.
"""
import ctypes

import numpy as np
import pytest

from oracle import dynamics as dyn
from oracle import go2_model as gm
from oracle import spatial
from oracle import sysid as osy
from helpers import random_theta

# Instrumented counts at the default configuration and a standing state (base-box corners off
# the ground): the articulated-body formulation of the oracle (csrc/aba_reference.h), the
# roofline's algorithmic figure, and the kernel's condensed formulation (csrc/dynamics.cuh; the
# joint targets of the actions are formed once per control step, outside the substep).
FLOPS_PER_SUBSTEP = 7053
EXECUTED_FLOPS_PER_SUBSTEP = 5149


def _emu(built, cfg, x0, acts, th):
    from spi_gb300 import _lib, robot
    r = robot.to_struct(cfg)
    B, H = acts.shape[:2]
    out = np.zeros((B, H, 37))
    x0c, ac, tc = (np.ascontiguousarray(a, dtype=np.float64) for a in (x0, acts, th))
    rc = _lib.hostemu_lib().spi_hostemu_rollout(ctypes.byref(r), x0c.ctypes.data, ac.ctypes.data,
                                                tc.ctypes.data, B, H, out.ctypes.data)
    assert rc == 0
    return out, r


@pytest.fixture
def oracle_f32_constants(monkeypatch):
    """Patch the oracle's constants to the float32 values the C struct carries."""
    from spi_gb300 import robot
    r = robot.to_struct(robot.SimConfig())
    org = np.zeros((13, 3))
    Irig = dyn._I_RIGID.copy()
    for b in range(12):
        h = np.array(r.body_h[b][:], dtype=np.float64)
        I6 = np.array(r.body_I[b][:], dtype=np.float64)
        M6 = np.zeros((6, 6))
        M6[:3, :3] = [[I6[0], I6[3], I6[4]], [I6[3], I6[1], I6[5]], [I6[4], I6[5], I6[2]]]
        M6[:3, 3:] = spatial.skew(h)
        M6[3:, :3] = spatial.skew(h).T
        M6[3:, 3:] = r.body_mass[b] * np.eye(3)
        Irig[b + 1] = M6
        org[b + 1] = np.array(r.body_origin[b][:], dtype=np.float64)
    fI = np.array(r.fixed_I[:], dtype=np.float64)
    fh = np.array(r.fixed_h[:], dtype=np.float64)
    H6 = np.zeros((6, 6))
    H6[:3, :3] = [[fI[0], fI[3], fI[4]], [fI[3], fI[1], fI[5]], [fI[4], fI[5], fI[2]]]
    H6[:3, 3:] = spatial.skew(fh)
    H6[3:, :3] = spatial.skew(fh).T
    H6[3:, 3:] = r.fixed_mass * np.eye(3)
    f = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)   # noqa: E731
    monkeypatch.setattr(dyn, "_ORIGIN", org)
    monkeypatch.setattr(dyn, "_I_RIGID", Irig)
    monkeypatch.setattr(dyn, "_I_HEADS", H6)
    for name in ("BASE_COM", "BASE_INERTIA", "FOOT_IN_CALF", "BASE_CORNERS"):
        monkeypatch.setattr(gm, name, f(getattr(gm, name)))
    return gm.SimParams(sim_dt=float(np.float32(0.00125)), gravity=float(np.float32(9.81)),
                        contact_mu=float(np.float32(0.8)), foot_radius=float(np.float32(0.022)),
                        friction_vel=float(np.float32(0.2)), torque_limit=f(gm.TORQUE_LIMIT),
                        contact_ramp=1.0 / float(np.float32(1.0) / np.float32(1e-3)),
                        velocity_limit=f(gm.VELOCITY_LIMIT), default_dof_pos=f(gm.DEFAULT_DOF_POS))


def _inputs(seed, B=12, H=8):
    from spi_gb300 import robot
    rng = np.random.default_rng(seed)
    cfg = robot.SimConfig()
    th = np.asarray(random_theta(rng, B), dtype=np.float32).astype(np.float64)
    x0 = osy.standing_state(B, z=0.30)
    x0[:, 7:13] = 0.3 * rng.normal(size=(B, 6))
    x0[:, 25:] = rng.normal(size=(B, 12))
    acts = osy.sine_actions(H, rng.uniform(0.1, 0.4, (B, 12)), rng.uniform(1, 3, (B, 12)),
                            rng.uniform(0, 6.28, (B, 12)), cfg.control_dt, cfg.action_scale)
    return cfg, x0, acts, th


def test_kernel_equations_equal_oracle(built, oracle_f32_constants):
    cfg, x0, acts, th = _inputs(11)
    emu, _ = _emu(built, cfg, x0, acts, th)
    ref = dyn.rollout(x0, acts, th, oracle_f32_constants, trace=True)
    assert np.abs(emu - ref).max() < 1e-9


def test_kernel_equations_reference_motor_variants(built, oracle_f32_constants):
    """Reference torque path (plain clip), tanh motor model and hip x0.5, contacts off/on."""
    from spi_gb300 import robot
    cfg, x0, acts, th = _inputs(12)
    for kw in (dict(torque_speed=False), dict(tanh_a=(15.0, 18.0, 25.0), hip_action_scale=0.5),
               dict(base_contact=False, motor_gain=(0.9, 1.1, 1.05))):
        c = robot.SimConfig(**kw)
        emu, _ = _emu(built, c, x0, acts, th)
        sp = oracle_f32_constants
        sp2 = gm.SimParams(**{**sp.__dict__, **{k: (np.asarray(v, dtype=np.float32).astype(np.float64) if isinstance(v, tuple) else v)
                                                 for k, v in kw.items()}})
        ref = dyn.rollout(x0, acts, th, sp2, trace=True)
        assert np.abs(emu - ref).max() < 1e-9, kw


def test_condensed_legs_equal_articulated_body_algorithm(built):
    """The kernel's leg condensation (joint-space inertia + Schur complement) and the oracle's
    articulated-body algorithm, both in FP64 with the same constants, agree to rounding, in
    and out of contact."""
    from spi_gb300 import _lib, robot
    cfg, x0, acts, th = _inputs(15, B=16, H=12)
    x0[:8, 2] = 0.26                                   # half the rollouts start with feet pressed in
    emu, r = _emu(built, cfg, x0, acts, th)
    out = np.zeros_like(emu)
    x0c, ac, tc = (np.ascontiguousarray(a, dtype=np.float64) for a in (x0, acts, th))
    rc = _lib.hostemu_lib().spi_hostemu_rollout_aba(ctypes.byref(r), x0c.ctypes.data, ac.ctypes.data,
                                                    tc.ctypes.data, x0.shape[0], acts.shape[1], out.ctypes.data)
    assert rc == 0
    assert np.abs(emu - out).max() < 1e-9


def test_kernel_vs_oracle_with_urdf_constants(built):
    """Float32 model constants move states by < 1e-5 (well inside the 1e-4 parity bar)."""
    cfg, x0, acts, th = _inputs(13)
    emu, _ = _emu(built, cfg, x0, acts, th)
    ref = dyn.rollout(x0, acts, th, gm.SimParams(), trace=True)
    err = np.abs(emu - ref) / np.maximum(np.abs(ref), 1.0)
    assert err.max() < 1e-5


def test_flop_count_constant(built):
    from spi_gb300 import _lib, robot
    cfg, x0, acts, th = _inputs(14, B=1, H=1)
    r = robot.to_struct(cfg)
    n1, n2 = ctypes.c_longlong(), ctypes.c_longlong()
    x0c = np.ascontiguousarray(x0[0], dtype=np.float64)
    tc = np.ascontiguousarray(th[0], dtype=np.float64)
    ac = np.ascontiguousarray(acts[0, 0], dtype=np.float64)
    lib = _lib.hostemu_lib()
    rc = lib.spi_hostemu_count_ops_aba(ctypes.byref(r), x0c.ctypes.data, tc.ctypes.data,
                                       ac.ctypes.data, ctypes.byref(n1), ctypes.byref(n2))
    assert rc == 0
    assert n1.value == FLOPS_PER_SUBSTEP
    rc = lib.spi_hostemu_count_ops(ctypes.byref(r), x0c.ctypes.data, tc.ctypes.data,
                                   ac.ctypes.data, ctypes.byref(n1), ctypes.byref(n2))
    assert rc == 0
    assert n1.value == EXECUTED_FLOPS_PER_SUBSTEP
    from spi_gb300 import flops
    assert flops.flops_per_rollout_step(cfg) == cfg.decimation * FLOPS_PER_SUBSTEP
    assert flops.executed_flops_per_rollout_step(cfg) == cfg.decimation * EXECUTED_FLOPS_PER_SUBSTEP
