"""FP64 rollout dynamics of the Go2 model: motor model, contact, ABA, integrator.

Test infrastructure (the checker of the CUDA rollout kernel). Equations:

* Action clip and PD law: reference spigym/envs/legged_base_task/
  legged_robot_base.py:185-187 (clip +-action_clip_value) and :542-560
  (tau = kp_scale*Kp*(action_scale*a + q0 - q) - kd_scale*Kd*qd, clipped to
  +-torque_limits). The hip-action halving of spigym/envs/locomotion/
  go2_omni.py:437 is ``hip_action_scale``.
* Motor models: per-group gain (act2tau_vec3, spigym/envs/sysid/
  active_sysid_openloop.py:365-379) and a*tanh(tau/a) (act2tau_vec3_tanh,
  :381-400), applied after the clip as in ActiveSysId_OpenLoop._compute_torques
  (:174-187).
* Extended motor terms (13-slot theta): per leg group Kp scale, Coulomb joint
  friction -Fc*tanh(qd/w), armature (added to the joint-space inertia inside
  ABA) and torque-limit scale, with a linear torque-speed limit.
* Torques are recomputed from the current state at every physics substep, as
  in legged_robot_base.py:201-209.
* Dynamics: floating-base articulated-body algorithm (Featherstone), penalty
  contact at the four foot spheres (r = 0.022 m) and the eight corners of the
  base collision box: fn = max(0, k*pen - c*s(pen)*vz) for pen > 0 with the
  damping ramp s = min(1, pen/ramp), tangential force -min(ct*|vt|, mu*fn) *
  vt/|vt|. Contact damping is linearly implicit: an active contact point adds a
  point mass dt*max(c, ct)*s(pen) at the contact to its body's inertia in the
  ABA (exact for linear damping; keeps the stiff contact mode stable). Semi-implicit Euler on the base's
  body-coordinate spatial velocity and the joint velocities; the orientation is
  advanced with the new body angular velocity (q <- normalise(q + dt/2 q (x) w_b))
  and the new body velocity is mapped to world coordinates with the new pose. Root state layout follows the reference's root-state rows
  (spigym/simulator/isaacgym/isaacgym.py:567-577): pos, quat xyzw, linear and
  angular velocity in world coordinates; linear velocity is that of the base
  frame origin.
"""
from __future__ import annotations

import numpy as np

from . import go2_model as gm
from .spatial import crf, crm, plucker, rigid_inertia, rot_axis, skew, mv

_ORIGIN, _MASS, _COM, _INERTIA = gm.body_tables()
_I_RIGID = np.stack([rigid_inertia(_MASS[i], _COM[i], _INERTIA[i]) for i in range(gm.N_BODIES)])
_I_HEADS = gm.head_spatial_inertia()
CALVES = (3, 6, 9, 12)


def quat_to_R(quat):
    x, y, z, w = (quat[..., i] for i in range(4))
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


def base_inertia(theta, sim: gm.SimParams):
    """Spatial inertia of the base (theta slots 0-4) plus the collapsed head links."""
    theta = np.asarray(theta, dtype=np.float64)
    m = theta[..., 0]
    c = gm.BASE_COM + theta[..., 1:4]
    Ic = np.broadcast_to(gm.BASE_INERTIA, theta.shape[:-1] + (3, 3)).copy()
    if sim.inertia_follows_mass:
        Ic = Ic * (m / gm.BASE_MASS)[..., None, None]
    d = np.arange(3)
    Ic[..., d, d] = Ic[..., d, d] * theta[..., 4:5]
    return rigid_inertia(m, c, Ic) + _I_HEADS


def joint_groups():
    """Leg group (0 front: FL, FR; 1 rear: RL, RR) and joint type (0 hip, 1 thigh, 2 calf)."""
    j = np.arange(gm.N_JOINTS)
    return (j // 3 >= 2).astype(int), j % 3


def motor_torques(q, qd, action, theta, sim: gm.SimParams):
    """Joint torques (motor output minus Coulomb friction) and per-joint armature."""
    grp, jtype = joint_groups()
    th = np.asarray(theta, dtype=np.float64)
    kp_s = th[..., 5 + 4 * grp]
    fc = th[..., 6 + 4 * grp]
    arm = th[..., 7 + 4 * grp]
    ts = th[..., 8 + 4 * grp]
    a = np.clip(action, -sim.action_clip, sim.action_clip)
    scaled = a * sim.action_scale
    scaled = scaled * np.where(jtype == 0, sim.hip_action_scale, 1.0)
    target = scaled + sim.default_dof_pos
    tau = kp_s * sim.kp * (target - q) - sim.kd_scale * sim.kd * qd
    lim = ts * sim.torque_limit
    if sim.torque_speed:
        lim = lim * np.maximum(0.0, 1.0 - np.abs(qd) / sim.velocity_limit)
    tau = np.clip(tau, -lim, lim)
    tau = tau * sim.motor_gain[jtype]
    a_t = sim.tanh_a[jtype]
    on = a_t > 0
    safe_a = np.where(on, a_t, 1.0)
    tau = np.where(on, safe_a * np.tanh(tau / safe_a), tau)
    tau = tau - fc * np.tanh(qd / sim.friction_vel)
    return tau, arm


def damping_ramp(pen, sim: gm.SimParams):
    """Fraction of the contact damping active at penetration pen (0 at touchdown, 1 past the ramp)."""
    return np.clip(pen / sim.contact_ramp, 0.0, 1.0)


def implicit_mass(pen, sim: gm.SimParams):
    """Point mass dt*c_imp*ramp added at a contact point: linearly implicit contact damping."""
    return sim.sim_dt * max(sim.contact_c, sim.contact_ct) * damping_ramp(pen, sim)


def foot_force(p_foot, v_foot, sim: gm.SimParams, radius=None):
    """Penalty contact force (world frame) on a contact point (foot sphere or box corner)."""
    pen = (sim.foot_radius if radius is None else radius) - p_foot[..., 2]
    fn = np.where(pen > 0, np.maximum(0.0, sim.contact_k * pen
                                      - sim.contact_c * damping_ramp(pen, sim) * v_foot[..., 2]), 0.0)
    vt = v_foot[..., :2]
    vtn = np.sqrt(np.sum(vt * vt, -1))
    lim = sim.contact_mu * fn
    visc = sim.contact_ct * vtn
    stick = visc <= lim
    scale = np.where(stick, sim.contact_ct, lim / np.where(stick, 1.0, vtn))
    ft = -scale[..., None] * vt
    return np.concatenate([ft, fn[..., None]], -1)


def _unit(axis):
    s = np.zeros(6)
    s[axis] = 1.0
    return s


def substep(x, action, theta, sim: gm.SimParams, return_aux=False, tau_override=None):
    """One physics substep for a batch. x [B,37], action [B,12], theta [B,13].

    ``tau_override`` [B,12] replaces the motor model's joint torques (armature
    still comes from theta); the golden-vector harness uses it to drive this
    physics with torques computed by the reference's own torque code.
    """
    x = np.asarray(x, dtype=np.float64)
    B = x.shape[0]
    p, quat, vw, ww = x[:, 0:3], x[:, 3:7], x[:, 7:10], x[:, 10:13]
    q, qd = x[:, 13:25], x[:, 25:37]
    R = quat_to_R(quat)
    Rt = np.swapaxes(R, -1, -2)
    tau, arm = motor_torques(q, qd, action, theta, sim)
    if tau_override is not None:
        tau = np.asarray(tau_override, dtype=np.float64)

    nb = gm.N_BODIES
    Xup = [None] * nb
    v = [None] * nb
    c = [np.zeros((B, 6))] * nb
    Rw = [None] * nb
    pw = [None] * nb
    v[0] = np.concatenate([mv(Rt, ww), mv(Rt, vw)], -1)
    Rw[0], pw[0] = R, p
    for i in range(1, nb):
        lam, ax, j = gm.PARENT[i], gm.AXIS[i], i - 1
        RJ = rot_axis(ax, q[:, j])
        Xup[i] = plucker(np.swapaxes(RJ, -1, -2), _ORIGIN[i])
        vJ = _unit(ax)[None, :] * qd[:, j:j + 1]
        v[i] = mv(Xup[i], v[lam]) + vJ
        c[i] = mv(crm(v[i]), vJ)
        Rw[i] = Rw[lam] @ RJ
        pw[i] = pw[lam] + mv(Rw[lam], np.broadcast_to(_ORIGIN[i], (B, 3)))

    fext = [np.zeros((B, 6)) for _ in range(nb)]
    I_imp = [np.zeros((B, 6, 6)) for _ in range(nb)]   # implicit contact damping
    foot_F = np.zeros((B, 4, 3))
    for l, i in enumerate(CALVES):
        r = np.broadcast_to(gm.FOOT_IN_CALF, (B, 3))
        pf = pw[i] + mv(Rw[i], r)
        vfb = v[i][:, 3:] + np.cross(v[i][:, :3], r)
        vf = mv(Rw[i], vfb)
        F = foot_force(pf, vf, sim)
        foot_F[:, l] = F
        fl = mv(np.swapaxes(Rw[i], -1, -2), F)
        fext[i] = np.concatenate([np.cross(r, fl), fl], -1)
        I_imp[i] = rigid_inertia(implicit_mass(sim.foot_radius - pf[:, 2], sim), r, np.zeros((B, 3, 3)))

    if sim.base_contact:
        for corner in gm.BASE_CORNERS:
            r = np.broadcast_to(corner, (B, 3))
            pc = p + mv(R, r)
            vcb = v[0][:, 3:] + np.cross(v[0][:, :3], r)
            F = foot_force(pc, mv(R, vcb), sim, radius=0.0)
            fl = mv(Rt, F)
            fext[0] = fext[0] + np.concatenate([np.cross(r, fl), fl], -1)
            I_imp[0] = I_imp[0] + rigid_inertia(implicit_mass(-pc[:, 2], sim), r, np.zeros((B, 3, 3)))

    IA = [None] * nb
    pA = [None] * nb
    IA[0] = base_inertia(theta, sim)
    if IA[0].ndim == 2:
        IA[0] = np.broadcast_to(IA[0], (B, 6, 6))
    IA[0] = IA[0].copy()
    for i in range(nb):
        if i > 0:
            IA[i] = np.broadcast_to(_I_RIGID[i], (B, 6, 6)).copy()
        pA[i] = mv(crf(v[i]), mv(IA[i], v[i])) - fext[i]
        # the implicit term acts on the true acceleration; the ABA runs in the gravity-shifted
        # frame (a' = a - (0, g)), so the shift's share I_imp (0, g_i) joins the bias
        g_i = mv(np.swapaxes(Rw[i], -1, -2), np.broadcast_to(np.array([0.0, 0.0, -sim.gravity]), (B, 3)))
        pA[i] = pA[i] + mv(I_imp[i], np.concatenate([np.zeros((B, 3)), g_i], -1))
        IA[i] = IA[i] + I_imp[i]

    U = [None] * nb
    D = [None] * nb
    u = [None] * nb
    for i in range(nb - 1, 0, -1):
        lam, ax, j = gm.PARENT[i], gm.AXIS[i], i - 1
        U[i] = IA[i][:, :, ax]
        D[i] = U[i][:, ax] + arm[:, j]
        u[i] = tau[:, j] - pA[i][:, ax]
        Ia = IA[i] - np.einsum("bi,bj->bij", U[i], U[i]) / D[i][:, None, None]
        pa = pA[i] + mv(Ia, c[i]) + U[i] * (u[i] / D[i])[:, None]
        XT = np.swapaxes(Xup[i], -1, -2)
        IA[lam] = IA[lam] + XT @ Ia @ Xup[i]
        pA[lam] = pA[lam] + mv(XT, pa)

    a = [None] * nb
    a[0] = -np.linalg.solve(IA[0], pA[0][..., None])[..., 0]
    qdd = np.zeros((B, gm.N_JOINTS))
    for i in range(1, nb):
        lam, ax, j = gm.PARENT[i], gm.AXIS[i], i - 1
        a[i] = mv(Xup[i], a[lam]) + c[i]
        qdd[:, j] = (u[i] - np.sum(U[i] * a[i], -1)) / D[i]
        a[i] = a[i] + _unit(ax)[None, :] * qdd[:, j:j + 1]
    g_b = mv(Rt, np.broadcast_to(np.array([0.0, 0.0, -sim.gravity]), (B, 3)))
    a0 = a[0] + np.concatenate([np.zeros((B, 3)), g_b], -1)

    dt = sim.sim_dt
    nu = v[0] + dt * a0                       # base velocity, body coordinates, end of step
    qd_n = qd + dt * qdd
    wb = nu[:, :3]
    wq = np.concatenate([                     # quat (x) (w_body, 0)
        quat[:, 3:4] * wb + np.cross(quat[:, :3], wb),
        -np.sum(wb * quat[:, :3], -1, keepdims=True)], -1)
    quat_n = quat + 0.5 * dt * wq
    quat_n = quat_n / np.linalg.norm(quat_n, axis=-1, keepdims=True)
    R_n = quat_to_R(quat_n)                   # body coordinates are those of the new pose
    ww_n = mv(R_n, wb)
    vw_n = mv(R_n, nu[:, 3:])
    p_n = p + dt * vw_n
    q_n = q + dt * qd_n
    xn = np.concatenate([p_n, quat_n, vw_n, ww_n, q_n, qd_n], -1)
    if return_aux:
        return xn, dict(a0=a0, qdd=qdd, tau=tau, foot_force=foot_F, v=v, Rw=Rw, pw=pw, I_imp=I_imp,
                        fext=fext)
    return xn


def control_step(x, action, theta, sim: gm.SimParams):
    for _ in range(sim.decimation):
        x = substep(x, action, theta, sim)
    return x


def rollout(x0, actions, theta, sim: gm.SimParams, trace=False):
    """Roll H control steps. x0 [B,37], actions [B,H,12], theta [B,13] (or [13]).

    Returns the final state [B,37], or the states after every control step
    [B,H,37] when ``trace`` is set.
    """
    x = np.asarray(x0, dtype=np.float64)
    actions = np.asarray(actions, dtype=np.float64)
    theta = np.broadcast_to(np.asarray(theta, dtype=np.float64), (x.shape[0], gm.THETA_DIM))
    H = actions.shape[1]
    out = []
    for h in range(H):
        x = control_step(x, actions[:, h], theta, sim)
        if trace:
            out.append(x)
    return np.stack(out, 1) if trace else x
