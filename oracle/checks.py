"""Independent inverse-dynamics (RNEA) and mass-matrix (CRBA-by-columns) checks.

Test infrastructure: used only to validate the oracle's forward dynamics
(ABA in ``dynamics.substep``) through the identity ID(FD(tau)) = tau.
"""
from __future__ import annotations

import numpy as np

from . import go2_model as gm
from .dynamics import _I_RIGID, _ORIGIN, _unit, base_inertia, quat_to_R
from .spatial import crf, crm, mv, plucker, rot_axis


def rnea(x, a0_true, qdd, theta, sim, fext=None, gravity=True, I_extra=None):
    """Floating-base RNEA. Returns (base wrench [B,6], joint torques [B,12]).

    a0_true is the base spatial acceleration in base coordinates (Featherstone
    convention, gravity not removed); fext is a list of 13 [B,6] body-frame forces;
    I_extra an optional list of 13 [B,6,6] inertias acting on the true accelerations
    (the implicit contact-damping terms).
    """
    B = x.shape[0]
    quat, vw, ww = x[:, 3:7], x[:, 7:10], x[:, 10:13]
    q, qd = x[:, 13:25], x[:, 25:37]
    Rt = np.swapaxes(quat_to_R(quat), -1, -2)
    nb = gm.N_BODIES
    g_b = mv(Rt, np.broadcast_to(np.array([0.0, 0.0, -sim.gravity if gravity else 0.0]), (B, 3)))
    v = [None] * nb
    a = [None] * nb
    f = [None] * nb
    X = [None] * nb
    I = [None] * nb
    v[0] = np.concatenate([mv(Rt, ww), mv(Rt, vw)], -1)
    a[0] = a0_true - np.concatenate([np.zeros((B, 3)), g_b], -1)
    I[0] = np.broadcast_to(base_inertia(theta, sim), (B, 6, 6))
    for i in range(1, nb):
        lam, ax, j = gm.PARENT[i], gm.AXIS[i], i - 1
        X[i] = plucker(np.swapaxes(rot_axis(ax, q[:, j]), -1, -2), _ORIGIN[i])
        S = _unit(ax)[None, :]
        v[i] = mv(X[i], v[lam]) + S * qd[:, j:j + 1]
        a[i] = mv(X[i], a[lam]) + S * qdd[:, j:j + 1] + mv(crm(v[i]), S * qd[:, j:j + 1])
        I[i] = np.broadcast_to(_I_RIGID[i], (B, 6, 6))
    # true (unshifted) body accelerations for the implicit-damping terms
    at = [None] * nb
    at[0] = a0_true
    for i in range(1, nb):
        lam, ax, j = gm.PARENT[i], gm.AXIS[i], i - 1
        S = _unit(ax)[None, :]
        at[i] = mv(X[i], at[lam]) + S * qdd[:, j:j + 1] + mv(crm(v[i]), S * qd[:, j:j + 1])
    for i in range(nb):
        f[i] = mv(I[i], a[i]) + mv(crf(v[i]), mv(I[i], v[i]))
        if fext is not None:
            f[i] = f[i] - fext[i]
        if I_extra is not None:
            f[i] = f[i] + mv(I_extra[i], at[i])
    tau = np.zeros((B, gm.N_JOINTS))
    for i in range(nb - 1, 0, -1):
        lam, ax, j = gm.PARENT[i], gm.AXIS[i], i - 1
        tau[:, j] = f[i][:, ax]
        f[lam] = f[lam] + mv(np.swapaxes(X[i], -1, -2), f[i])
    return f[0], tau


def mass_matrix(x, theta, sim):
    """18x18 joint-space inertia (base 6 in body coordinates, then 12 joints) by unit RNEA columns."""
    B = x.shape[0]
    x0 = x.copy()
    x0[:, 7:13] = 0.0
    x0[:, 25:37] = 0.0
    M = np.zeros((B, 18, 18))
    for k in range(18):
        a0 = np.zeros((B, 6))
        qdd = np.zeros((B, 12))
        if k < 6:
            a0[:, k] = 1.0
        else:
            qdd[:, k - 6] = 1.0
        fb, tau = rnea(x0, a0, qdd, theta, sim, gravity=False)
        M[:, :6, k] = fb
        M[:, 6:, k] = tau
    return M


def momentum_world(x, theta, sim):
    """Total spatial momentum (angular about world origin; linear) in world coordinates."""
    from .dynamics import substep
    _, aux = substep(x, np.zeros((x.shape[0], 12)), theta, sim, return_aux=True)
    B = x.shape[0]
    h = np.zeros((B, 6))
    I0 = np.broadcast_to(base_inertia(theta, sim), (B, 6, 6))
    for i in range(gm.N_BODIES):
        Ii = I0 if i == 0 else np.broadcast_to(_I_RIGID[i], (B, 6, 6))
        hb = mv(Ii, aux["v"][i])            # body-frame momentum (moment about body origin; force)
        R, p = aux["Rw"][i], aux["pw"][i]
        lin = mv(R, hb[:, 3:])
        ang = mv(R, hb[:, :3]) + np.cross(p, lin)
        h += np.concatenate([ang, lin], -1)
    return h


def energy_world(x, theta, sim):
    """Kinetic energy 1/2 sum_i v_i . (I_i v_i) plus gravitational potential energy
    g sum_i m_i z_com,i of all bodies (contact and motor terms excluded)."""
    from .dynamics import substep
    _, aux = substep(x, np.zeros((x.shape[0], 12)), theta, sim, return_aux=True)
    B = x.shape[0]
    E = np.zeros(B)
    I0 = np.broadcast_to(base_inertia(theta, sim), (B, 6, 6))
    for i in range(gm.N_BODIES):
        Ii = I0 if i == 0 else np.broadcast_to(_I_RIGID[i], (B, 6, 6))
        v = aux["v"][i]
        E += 0.5 * np.einsum("bk,bk->b", v, mv(Ii, v))
        m = Ii[:, 3, 3]
        h = np.stack([Ii[:, 2, 4], Ii[:, 0, 5], Ii[:, 1, 3]], -1)   # [h]x sits in the upper-right block
        com = aux["pw"][i] + mv(aux["Rw"][i], h / m[:, None])
        E += sim.gravity * m * com[:, 2]
    return E
