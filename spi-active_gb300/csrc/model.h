// model.h -- spi_robot (public C struct) -> DevModel (kernel layout); shared by the CUDA
// engine and the host emulation.
#pragma once

#include <math.h>
#include <string.h>

#include "dynamics.cuh"

namespace spi {

// Returns 0 on success, or a negative code with a message in *why.
inline int build_dev_model(const spi_robot& r, DevModel* M, const char** why) {
  memset(M, 0, sizeof(*M));
  for (int leg = 0; leg < 4; ++leg) {
    for (int k = 0; k < 3; ++k) {
      const int b = 3 * leg + k;
      for (int c = 0; c < 3; ++c) {
        M->org[k][c][leg] = r.body_origin[b][c];
        M->h[k][c][leg] = r.body_h[b][c];
      }
      M->m[k][leg] = r.body_mass[b];
      for (int c = 0; c < 6; ++c) M->I[k][c][leg] = r.body_I[b][c];
      M->kp[k][leg] = r.kp[b];
      M->kd[k][leg] = r.kd[b];
      M->q0[k][leg] = r.default_q[b];
      M->tlim[k][leg] = r.torque_limit[b];
      M->vlim[k][leg] = r.velocity_limit[b];
      F4* lc = M->legc[leg];
      lc[k] = F4{r.body_origin[b][0], r.body_origin[b][1], r.body_origin[b][2], r.kd_scale * r.kd[b]};
      lc[3 + 3 * k] = F4{r.body_mass[b], r.body_h[b][0], r.body_h[b][1], r.body_h[b][2]};
      lc[4 + 3 * k] = F4{r.body_I[b][0], r.body_I[b][1], r.body_I[b][2], r.body_I[b][3]};
      lc[5 + 3 * k] = F4{r.body_I[b][4], r.body_I[b][5],
                         r.torque_speed ? (float)(1.0 / (double)r.velocity_limit[b]) : 0.0f, 0.0f};
      if (!(r.body_mass[b] > 0.0f)) { *why = "leg body mass must be > 0"; return SPI_EINVAL; }
      // the kernel's transforms assume hip joints in the base's x-y plane, thigh joints offset
      // along y and calf joints along z
      if (k == 0 && r.body_origin[b][2] != 0.0f) {
        *why = "hip joint origins must lie in the base frame's x-y plane"; return SPI_EINVAL;
      }
      if (k == 1 && (r.body_origin[b][0] != 0.0f || r.body_origin[b][2] != 0.0f)) {
        *why = "thigh joint origins must lie on the hip frame's y axis"; return SPI_EINVAL;
      }
      if (k == 2 && (r.body_origin[b][0] != 0.0f || r.body_origin[b][1] != 0.0f)) {
        *why = "calf joint origins must lie on the thigh frame's z axis"; return SPI_EINVAL;
      }
      if (r.torque_speed && !(r.velocity_limit[b] > 0.0f)) {
        *why = "velocity_limit must be > 0 with torque_speed"; return SPI_EINVAL;
      }
    }
  }
  memcpy(M->corner, r.corners, sizeof(M->corner));
  for (int leg = 0; leg < 4; ++leg) {
    const float* c0 = r.corners[2 * leg];
    const float* c1 = r.corners[2 * leg + 1];
    M->legc[leg][12] = F4{c0[0], c0[1], c0[2], c1[0]};
    M->legc[leg][13] = F4{c1[1], c1[2], 0.0f, 0.0f};
  }
  M->corner_reach = 0.0f;
  for (int i = 0; i < 8; ++i) {
    const float d = sqrtf(r.corners[i][0] * r.corners[i][0] + r.corners[i][1] * r.corners[i][1] +
                          r.corners[i][2] * r.corners[i][2]);
    M->corner_reach = d > M->corner_reach ? d : M->corner_reach;
  }
  M->corner_reach *= 1.001f;   // margin over float rounding of the corner coordinates
  memcpy(M->foot, r.foot, sizeof(M->foot));
  if (r.foot[0] != 0.0f || r.foot[1] != 0.0f) { *why = "the foot must lie on the calf frame's z axis"; return SPI_EINVAL; }
  memcpy(M->gain, r.motor_gain, sizeof(M->gain));
  memcpy(M->tanh_a, r.tanh_a, sizeof(M->tanh_a));
  memcpy(M->base_com, r.base_com, sizeof(M->base_com));
  memcpy(M->base_Ic, r.base_Ic, sizeof(M->base_Ic));
  M->base_m0 = r.base_mass_nominal;
  M->fixed_m = r.fixed_mass;
  memcpy(M->fixed_h, r.fixed_h, sizeof(M->fixed_h));
  memcpy(M->fixed_I, r.fixed_I, sizeof(M->fixed_I));
  M->foot_r = r.foot_radius;
  M->k = r.contact_k; M->c = r.contact_c; M->ct = r.contact_ct; M->mu = r.contact_mu;
  if (!(r.contact_ramp > 0.0f)) { *why = "contact_ramp must be > 0"; return SPI_EINVAL; }
  M->ramp_inv = 1.0f / r.contact_ramp;
  M->imp_c = r.contact_c > r.contact_ct ? r.contact_c : r.contact_ct;
  M->dt_imp_c = r.sim_dt * M->imp_c;
  M->kd_scale = r.kd_scale; M->act_scale = r.action_scale; M->act_clip = r.action_clip;
  M->hip_scale = r.hip_action_scale; M->fric_vel = r.friction_vel;
  M->dt = r.sim_dt; M->g = r.gravity;
  M->decimation = r.decimation; M->torque_speed = r.torque_speed;
  M->base_contact = r.base_contact; M->inertia_follows_mass = r.inertia_follows_mass;
  if (!(r.sim_dt > 0.0f) || r.decimation < 1 || r.decimation > 64) {
    *why = "sim_dt must be > 0 and decimation in [1, 64]"; return SPI_EINVAL;
  }
  if (!(r.friction_vel > 0.0f)) { *why = "friction_vel must be > 0"; return SPI_EINVAL; }
  M->fric_k2 = (float)(2.0 / (log(2.0) * (double)r.friction_vel));
  if (r.inertia_follows_mass && !(r.base_mass_nominal > 0.0f)) {
    *why = "base_mass_nominal must be > 0 with inertia_follows_mass"; return SPI_EINVAL;
  }
  return SPI_OK;
}

}  // namespace spi
