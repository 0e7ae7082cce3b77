"""Go2 model constants and simulation settings, packed into the C ``spi_robot`` struct.

Constants (paths inside the reference project):
* link inertials, joint origins / axes, foot sphere and base collision box:
  spigym/data/robots/go2/urdf/go2.urdf (base :9-41, head links :45-120, FL_hip
  :121-175, FL_thigh :176-230, FL_calf :231-285, FL_foot :330-379 and the
  mirrored FR / RL / RR blocks).
* default joint pose, effort and velocity limits, action scale and clip:
  spigym/config/robot/go2/go2.yaml:36-39, 56-68, 105-109. The default PD gains
  are Kp = 20, Kd = 0.5 (the synthetic identification workload); the
  reference's own go2.yaml:78-103 values (25 / 0.6) are available through
  ``SimConfig(kp=25.0, kd=0.6)``.
* joint order FL, FR, RL, RR x hip, thigh, calf: go2.yaml:29.

Fixed joints are collapsed the way Isaac Gym's ``collapse_fixed_joints`` does:
the foot (0.04 kg) is merged into the calf and the two head links (0.001 kg
each) into the base.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

LEGS = ("FL", "FR", "RL", "RR")
STATE_DIM = 37
THETA_DIM = 13
N_COMP = 9
THETA_NAMES = (
    "base_mass", "com_x", "com_y", "com_z", "inertia_scale",
    "front_kp_scale", "front_friction", "front_armature", "front_tau_scale",
    "rear_kp_scale", "rear_friction", "rear_armature", "rear_tau_scale",
)

BASE_MASS = 6.921
BASE_COM = (0.021112, 0.0, -0.005366)
BASE_INERTIA = (0.02448, 0.098077, 0.107, 0.00012166, 0.0014849, -3.12e-05)  # xx yy zz xy xz yz
HEAD_MASS = 0.001
HEAD_POS = ((0.285, 0.0, 0.01), (0.293, 0.0, -0.06))
SMALL_INERTIA = 9.6e-6
FOOT_MASS = 0.04
FOOT_IN_CALF = (0.0, 0.0, -0.213)
FOOT_RADIUS = 0.022
BASE_BOX = (0.3762, 0.0935, 0.114)
DEFAULT_DOF_POS = (0.1, 0.8, -1.5, -0.1, 0.8, -1.5, 0.1, 1.0, -1.5, -0.1, 1.0, -1.5)
TORQUE_LIMIT = (23.7, 23.7, 35.55) * 4
VELOCITY_LIMIT = (30.1, 30.1, 20.07) * 4

THETA_NOMINAL = np.array([BASE_MASS, 0, 0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 1], dtype=np.float64)
THETA_PRIOR_LO = np.array([5.0, -0.05, -0.05, -0.05, 0.7, 0.8, 0.0, 0.0, 0.8, 0.8, 0.0, 0.0, 0.8])
THETA_PRIOR_HI = np.array([9.0, 0.05, 0.05, 0.05, 1.3, 1.2, 0.3, 0.02, 1.0, 1.2, 0.3, 0.02, 1.0])

# sign of x (front +) and y (left +) per leg
_SX = (1.0, 1.0, -1.0, -1.0)
_SY = (1.0, -1.0, 1.0, -1.0)


def _sym(xx, yy, zz, xy, xz, yz):
    return np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]], dtype=np.float64)


def _about_origin(m, c, Ic):
    """(mass, first moment m*c, inertia about the body origin) from CoM-frame data."""
    c = np.asarray(c, dtype=np.float64)
    return m, m * c, Ic + m * (c @ c * np.eye(3) - np.outer(c, c))


def leg_links(leg: int):
    """URDF hip, thigh, calf(+foot) as (mass, com, inertia about com) for leg index 0..3."""
    sx, sy = _SX[leg], _SY[leg]
    hip = (0.678, (-0.0054 * sx, 0.00194 * sy, -0.000105),
           _sym(0.00048, 0.000884, 0.000596, -3.01e-06 * sx * sy, 1.11e-06 * sx, -1.42e-06 * sy))
    thigh = (1.152, (-0.00374, -0.0223 * sy, -0.0327),
             _sym(0.00584, 0.0058, 0.00103, 8.72e-05 * sy, -0.000289, 0.000808 * sy))
    calf_m, calf_c = 0.154, np.array([0.00548, -0.000975 * sy, -0.115])
    calf_I = _sym(0.00108, 0.0011, 3.29e-05, 3.4e-07 * sy, 1.72e-05, 8.28e-06 * sy)
    foot_c = np.array(FOOT_IN_CALF)
    m = calf_m + FOOT_MASS
    c = (calf_m * calf_c + FOOT_MASS * foot_c) / m
    I = np.zeros((3, 3))
    for mm, cc, II in ((calf_m, calf_c, calf_I), (FOOT_MASS, foot_c, SMALL_INERTIA * np.eye(3))):
        d = cc - c
        I += II + mm * (d @ d * np.eye(3) - np.outer(d, d))
    return hip, thigh, (m, tuple(c), I)


def joint_origins(leg: int):
    sx, sy = _SX[leg], _SY[leg]
    return ((0.1934 * sx, 0.0465 * sy, 0.0), (0.0, 0.0955 * sy, 0.0), (0.0, 0.0, -0.213))


def _s6(I):
    return (I[0, 0], I[1, 1], I[2, 2], I[0, 1], I[0, 2], I[1, 2])


class SpiRobot(ctypes.Structure):
    """ctypes mirror of ``spi_robot`` in include/spi_engine.h."""
    _fields_ = [
        ("body_origin", (ctypes.c_float * 3) * 12),
        ("body_mass", ctypes.c_float * 12),
        ("body_h", (ctypes.c_float * 3) * 12),
        ("body_I", (ctypes.c_float * 6) * 12),
        ("base_mass_nominal", ctypes.c_float),
        ("base_com", ctypes.c_float * 3),
        ("base_Ic", ctypes.c_float * 6),
        ("fixed_mass", ctypes.c_float),
        ("fixed_h", ctypes.c_float * 3),
        ("fixed_I", ctypes.c_float * 6),
        ("foot", ctypes.c_float * 3),
        ("foot_radius", ctypes.c_float),
        ("corners", (ctypes.c_float * 3) * 8),
        ("contact_k", ctypes.c_float), ("contact_c", ctypes.c_float),
        ("contact_ct", ctypes.c_float), ("contact_mu", ctypes.c_float),
        ("contact_ramp", ctypes.c_float),
        ("kp", ctypes.c_float * 12), ("kd", ctypes.c_float * 12),
        ("kd_scale", ctypes.c_float), ("action_scale", ctypes.c_float),
        ("action_clip", ctypes.c_float), ("hip_action_scale", ctypes.c_float),
        ("default_q", ctypes.c_float * 12), ("torque_limit", ctypes.c_float * 12),
        ("velocity_limit", ctypes.c_float * 12),
        ("motor_gain", ctypes.c_float * 3), ("tanh_a", ctypes.c_float * 3),
        ("friction_vel", ctypes.c_float),
        ("sim_dt", ctypes.c_float), ("gravity", ctypes.c_float),
        ("decimation", ctypes.c_int32), ("torque_speed", ctypes.c_int32),
        ("base_contact", ctypes.c_int32), ("inertia_follows_mass", ctypes.c_int32),
    ]


@dataclass
class SimConfig:
    """Simulation / motor settings. Defaults: the synthetic Go2 identification workload."""
    sim_dt: float = 0.00125
    decimation: int = 4
    gravity: float = 9.81
    contact_k: float = 2.0e4
    contact_c: float = 200.0
    contact_ct: float = 200.0
    contact_mu: float = 0.8
    contact_ramp: float = 1e-3
    foot_radius: float = FOOT_RADIUS
    base_contact: bool = True
    kp: object = 20.0
    kd: object = 0.5
    kd_scale: float = 1.0
    action_scale: float = 0.25
    action_clip: float = 20.0
    hip_action_scale: float = 1.0
    default_dof_pos: tuple = DEFAULT_DOF_POS
    torque_limit: tuple = TORQUE_LIMIT
    velocity_limit: tuple = VELOCITY_LIMIT
    torque_speed: bool = True
    motor_gain: tuple = (1.0, 1.0, 1.0)
    tanh_a: tuple = (0.0, 0.0, 0.0)
    friction_vel: float = 0.2
    inertia_follows_mass: bool = False

    @property
    def control_dt(self) -> float:
        return self.sim_dt * self.decimation

    @classmethod
    def reference_compatible(cls, **kw):
        """Torque path of the reference's LeggedRobotBase (PD + plain clip, no speed limit)."""
        kw.setdefault("torque_speed", False)
        return cls(**kw)


def to_struct(cfg: SimConfig) -> SpiRobot:
    r = SpiRobot()
    for leg in range(4):
        links = leg_links(leg)
        origins = joint_origins(leg)
        for k in range(3):
            b = 3 * leg + k
            m, h, Io = _about_origin(*links[k])
            r.body_origin[b][:] = origins[k]
            r.body_mass[b] = m
            r.body_h[b][:] = tuple(h)
            r.body_I[b][:] = _s6(Io)
    r.base_mass_nominal = BASE_MASS
    r.base_com[:] = BASE_COM
    r.base_Ic[:] = BASE_INERTIA
    fm, fh, fI = 0.0, np.zeros(3), np.zeros((3, 3))
    for pos in HEAD_POS:
        m, h, Io = _about_origin(HEAD_MASS, pos, SMALL_INERTIA * np.eye(3))
        fm, fh, fI = fm + m, fh + h, fI + Io
    r.fixed_mass = fm
    r.fixed_h[:] = tuple(fh)
    r.fixed_I[:] = _s6(fI)
    r.foot[:] = FOOT_IN_CALF
    r.foot_radius = cfg.foot_radius
    half = np.array(BASE_BOX) / 2.0
    for i, (sx, sy, sz) in enumerate((a, b, c) for a in (1, -1) for b in (1, -1) for c in (1, -1)):
        r.corners[i][:] = tuple(half * np.array([sx, sy, sz]))
    r.contact_k, r.contact_c, r.contact_ct, r.contact_mu = (cfg.contact_k, cfg.contact_c,
                                                            cfg.contact_ct, cfg.contact_mu)
    r.contact_ramp = cfg.contact_ramp
    r.kp[:] = tuple(np.broadcast_to(np.asarray(cfg.kp, dtype=np.float64), (12,)))
    r.kd[:] = tuple(np.broadcast_to(np.asarray(cfg.kd, dtype=np.float64), (12,)))
    r.kd_scale, r.action_scale, r.action_clip = cfg.kd_scale, cfg.action_scale, cfg.action_clip
    r.hip_action_scale = cfg.hip_action_scale
    r.default_q[:] = tuple(cfg.default_dof_pos)
    r.torque_limit[:] = tuple(cfg.torque_limit)
    r.velocity_limit[:] = tuple(cfg.velocity_limit)
    r.motor_gain[:] = tuple(cfg.motor_gain)
    r.tanh_a[:] = tuple(cfg.tanh_a)
    r.friction_vel = cfg.friction_vel
    r.sim_dt, r.gravity, r.decimation = cfg.sim_dt, cfg.gravity, int(cfg.decimation)
    r.torque_speed = int(bool(cfg.torque_speed))
    r.base_contact = int(bool(cfg.base_contact))
    r.inertia_follows_mass = int(bool(cfg.inertia_follows_mass))
    return r
