"""Go2 robot description and simulation settings for the FP64 oracle.

Oracle-side copy of the model constants (test infrastructure). The product
package builds its own copy; ``tests/test_model_constants.py`` checks that the
two agree and, where the reference checkout is present, that both match the
URDF.

Sources (paths inside the reference project):
* link inertials, joint origins and axes: spigym/data/robots/go2/urdf/go2.urdf
  (base :9-23, FL_hip :121-136, FL_hip_joint :158-175, FL_thigh :176-191,
  FL_thigh_joint :213-230, FL_calf :231-246, FL_calf_joint :268-285,
  FL_foot :330-366 incl. sphere r=0.022 :363, FL_foot_joint :367-379, and the
  mirrored FR/RL/RR blocks; Head_upper/Head_lower :45-120).
* default pose, effort / velocity limits, PD gains, action scale and clip:
  spigym/config/robot/go2/go2.yaml:36-39, 56-68, 78-109.
* joint order (Isaac Gym DFS order FL, FR, RL, RR x hip, thigh, calf):
  spigym/config/robot/go2/go2.yaml:29.

Fixed joints are collapsed as Isaac Gym does with ``collapse_fixed_joints``
(go2.yaml asset block): the foot (0.04 kg) merges into the calf, the two head
links (0.001 kg each) merge into the base; imu/radar are massless.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

LEGS = ("FL", "FR", "RL", "RR")
N_BODIES = 13
N_JOINTS = 12
STATE_DIM = 37            # pos3 quat4(xyzw) linvel3 angvel3 q12 qd12
THETA_DIM = 13
# parent of each body; body 0 is the floating base
PARENT = np.array([-1, 0, 1, 2, 0, 4, 5, 0, 7, 8, 0, 10, 11])
# joint axis of body i (0 = x, 1 = y); hip abduction about x, thigh/calf about y
AXIS = np.array([-1, 0, 1, 1, 0, 1, 1, 0, 1, 1, 0, 1, 1])

_SIDE_X = {"FL": 1.0, "FR": 1.0, "RL": -1.0, "RR": -1.0}
_SIDE_Y = {"FL": 1.0, "FR": -1.0, "RL": 1.0, "RR": -1.0}


def _sym(ixx, ixy, ixz, iyy, iyz, izz):
    return np.array([[ixx, ixy, ixz], [ixy, iyy, iyz], [ixz, iyz, izz]], dtype=np.float64)


def _combine(m1, c1, I1, m2, c2, I2):
    """Merge two rigid bodies given in the same frame (inertia about own CoM)."""
    m = m1 + m2
    c = (m1 * c1 + m2 * c2) / m
    def shift(mm, cc, II):
        d = cc - c
        return II + mm * (np.dot(d, d) * np.eye(3) - np.outer(d, d))
    return m, c, shift(m1, c1, I1) + shift(m2, c2, I2)


# --- URDF link inertials (mass, CoM in link frame, inertia about CoM) ---------
BASE_MASS = 6.921
BASE_COM = np.array([0.021112, 0.0, -0.005366])
BASE_INERTIA = _sym(0.02448, 0.00012166, 0.0014849, 0.098077, -3.12e-05, 0.107)
HEAD_UPPER_POS = np.array([0.285, 0.0, 0.01])
HEAD_LOWER_POS = HEAD_UPPER_POS + np.array([0.008, 0.0, -0.07])
HEAD_MASS = 0.001
HEAD_INERTIA = 9.6e-6 * np.eye(3)

FOOT_MASS = 0.04
FOOT_INERTIA = 9.6e-6 * np.eye(3)
FOOT_IN_CALF = np.array([0.0, 0.0, -0.213])
FOOT_RADIUS = 0.022
# base collision box 0.3762 x 0.0935 x 0.114 m centred on the base origin (go2.urdf:39-41);
# its 8 corners are penalty contact points so a tipped-over base rests on the ground
BASE_BOX_HALF = np.array([0.3762, 0.0935, 0.114]) / 2.0
BASE_CORNERS = np.array([[sx, sy, sz] for sx in (1, -1) for sy in (1, -1) for sz in (1, -1)]) * BASE_BOX_HALF


def _leg_links(leg):
    """(mass, com, inertia) of hip, thigh, calf(+foot) for one leg, from the URDF."""
    sx, sy = _SIDE_X[leg], _SIDE_Y[leg]
    # hip: com x flips front/rear, y flips left/right; ixy, iyz flip with y, ixz with x
    hip = (0.678, np.array([-0.0054 * sx, 0.00194 * sy, -0.000105]),
           _sym(0.00048, -3.01e-06 * sx * sy, 1.11e-06 * sx, 0.000884, -1.42e-06 * sy, 0.000596))
    thigh = (1.152, np.array([-0.00374, -0.0223 * sy, -0.0327]),
             _sym(0.00584, 8.72e-05 * sy, -0.000289, 0.0058, 0.000808 * sy, 0.00103))
    calf = (0.154, np.array([0.00548, -0.000975 * sy, -0.115]),
            _sym(0.00108, 3.4e-07 * sy, 1.72e-05, 0.0011, 8.28e-06 * sy, 3.29e-05))
    calf = _combine(*calf, FOOT_MASS, FOOT_IN_CALF, FOOT_INERTIA)
    return hip, thigh, calf


def _joint_origins(leg):
    sx, sy = _SIDE_X[leg], _SIDE_Y[leg]
    return (np.array([0.1934 * sx, 0.0465 * sy, 0.0]),
            np.array([0.0, 0.0955 * sy, 0.0]),
            np.array([0.0, 0.0, -0.213]))


def body_tables():
    """Per-body (origin in parent, mass, com, inertia about com); base row is nominal."""
    origin = np.zeros((N_BODIES, 3))
    mass = np.zeros(N_BODIES)
    com = np.zeros((N_BODIES, 3))
    inertia = np.zeros((N_BODIES, 3, 3))
    mass[0], com[0], inertia[0] = BASE_MASS, BASE_COM, BASE_INERTIA
    for l, leg in enumerate(LEGS):
        links = _leg_links(leg)
        origins = _joint_origins(leg)
        for k in range(3):
            b = 1 + 3 * l + k
            origin[b] = origins[k]
            mass[b], com[b], inertia[b] = links[k]
    return origin, mass, com, inertia


def head_spatial_inertia():
    """6x6 spatial inertia (about base origin) of the two collapsed head links."""
    from .spatial import rigid_inertia
    I = rigid_inertia(HEAD_MASS, HEAD_UPPER_POS, HEAD_INERTIA)
    return I + rigid_inertia(HEAD_MASS, HEAD_LOWER_POS, HEAD_INERTIA)


# --- go2.yaml control constants ------------------------------------------------
DEFAULT_DOF_POS = np.array([0.1, 0.8, -1.5, -0.1, 0.8, -1.5, 0.1, 1.0, -1.5, -0.1, 1.0, -1.5])
TORQUE_LIMIT = np.array([23.7, 23.7, 35.55] * 4)
VELOCITY_LIMIT = np.array([30.1, 30.1, 20.07] * 4)

# Nominal 13-slot theta (layout documented in THETA_NAMES).
THETA_NAMES = (
    "base_mass", "com_x", "com_y", "com_z", "inertia_scale",
    "front_kp_scale", "front_friction", "front_armature", "front_tau_scale",
    "rear_kp_scale", "rear_friction", "rear_armature", "rear_tau_scale",
)
THETA_NOMINAL = np.array([BASE_MASS, 0.0, 0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 1.0])
THETA_PRIOR_LO = np.array([5.0, -0.05, -0.05, -0.05, 0.7, 0.8, 0.0, 0.0, 0.8, 0.8, 0.0, 0.0, 0.8])
THETA_PRIOR_HI = np.array([9.0, 0.05, 0.05, 0.05, 1.3, 1.2, 0.3, 0.02, 1.0, 1.2, 0.3, 0.02, 1.0])


@dataclass
class SimParams:
    """Simulation and motor-model settings shared by every rollout."""
    sim_dt: float = 0.00125           # physics substep [s]
    decimation: int = 4               # substeps per control step
    gravity: float = 9.81
    contact_k: float = 2.0e4          # N/m
    contact_c: float = 200.0          # N s/m (normal damping)
    contact_ct: float = 200.0         # N s/m (tangential viscous slope, capped at mu*fn)
    contact_mu: float = 0.8
    contact_ramp: float = 1e-3        # m: normal damping fades in over the first mm of penetration
    foot_radius: float = FOOT_RADIUS
    base_contact: bool = True          # base box corners collide with the ground
    kp: np.ndarray = field(default_factory=lambda: np.full(12, 20.0))
    kd: np.ndarray = field(default_factory=lambda: np.full(12, 0.5))
    kd_scale: float = 1.0             # reference _kd_scale
    action_scale: float = 0.25
    action_clip: float = 20.0
    hip_action_scale: float = 1.0     # 0.5 reproduces go2_omni_interface
    default_dof_pos: np.ndarray = field(default_factory=lambda: DEFAULT_DOF_POS.copy())
    torque_limit: np.ndarray = field(default_factory=lambda: TORQUE_LIMIT.copy())
    velocity_limit: np.ndarray = field(default_factory=lambda: VELOCITY_LIMIT.copy())
    torque_speed: bool = True         # limit falls linearly to 0 at velocity_limit
    motor_gain: np.ndarray = field(default_factory=lambda: np.ones(3))   # act2tau_vec3 gains
    tanh_a: np.ndarray = field(default_factory=lambda: np.zeros(3))      # act2tau_vec3_tanh a (0 = off)
    friction_vel: float = 0.2         # rad/s, Coulomb friction tanh width
    inertia_follows_mass: bool = False

    @property
    def control_dt(self) -> float:
        return self.sim_dt * self.decimation
