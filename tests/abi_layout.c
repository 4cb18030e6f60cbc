/* Prints the size of each C-ABI parameter struct of include/fest_gpu.h
 * and the offset of each field, one per line ("struct.field offset"):
 * tests/test_abi_cpu.py compares them with the ctypes mirrors in
 * fest3d/abi.py. */
#include <stddef.h>
#include <stdio.h>
#include "fest_gpu.h"

int main(void) {
  printf("fest_extent %zu\n", sizeof(fest_extent));
  printf("fest_extent.imx %zu\n", offsetof(fest_extent, imx));
  printf("fest_extent.jmx %zu\n", offsetof(fest_extent, jmx));
  printf("fest_extent.kmx %zu\n", offsetof(fest_extent, kmx));
  printf("fest_extent.n_var %zu\n", offsetof(fest_extent, n_var));
  printf("fest_flow %zu\n", sizeof(fest_flow));
  printf("fest_flow.density_inf %zu\n", offsetof(fest_flow, density_inf));
  printf("fest_flow.x_speed_inf %zu\n", offsetof(fest_flow, x_speed_inf));
  printf("fest_flow.y_speed_inf %zu\n", offsetof(fest_flow, y_speed_inf));
  printf("fest_flow.z_speed_inf %zu\n", offsetof(fest_flow, z_speed_inf));
  printf("fest_flow.pressure_inf %zu\n", offsetof(fest_flow, pressure_inf));
  printf("fest_flow.tk_inf %zu\n", offsetof(fest_flow, tk_inf));
  printf("fest_flow.tw_inf %zu\n", offsetof(fest_flow, tw_inf));
  printf("fest_flow.vel_mag %zu\n", offsetof(fest_flow, vel_mag));
  printf("fest_flow.MInf %zu\n", offsetof(fest_flow, MInf));
  printf("fest_flow.gm %zu\n", offsetof(fest_flow, gm));
  printf("fest_flow.R_gas %zu\n", offsetof(fest_flow, R_gas));
  printf("fest_flow.mu_ref %zu\n", offsetof(fest_flow, mu_ref));
  printf("fest_flow.T_ref %zu\n", offsetof(fest_flow, T_ref));
  printf("fest_flow.Sutherland_temp %zu\n", offsetof(fest_flow, Sutherland_temp));
  printf("fest_flow.Pr %zu\n", offsetof(fest_flow, Pr));
  printf("fest_flow.tPr %zu\n", offsetof(fest_flow, tPr));
  printf("fest_flow.mu_variation %zu\n", offsetof(fest_flow, mu_variation));
  printf("fest_flow.reserved %zu\n", offsetof(fest_flow, reserved));
  printf("fest_flow.tv_inf %zu\n", offsetof(fest_flow, tv_inf));
  printf("fest_flow.tkl_inf %zu\n", offsetof(fest_flow, tkl_inf));
  printf("fest_flow.tu_inf %zu\n", offsetof(fest_flow, tu_inf));
  printf("fest_flow.tgm_inf %zu\n", offsetof(fest_flow, tgm_inf));
  printf("fest_scheme %zu\n", sizeof(fest_scheme));
  printf("fest_scheme.scheme_name %zu\n", offsetof(fest_scheme, scheme_name));
  printf("fest_scheme.interpolant %zu\n", offsetof(fest_scheme, interpolant));
  printf("fest_scheme.time_stepping_method %zu\n", offsetof(fest_scheme, time_stepping_method));
  printf("fest_scheme.time_step_accuracy %zu\n", offsetof(fest_scheme, time_step_accuracy));
  printf("fest_scheme.global_time_step %zu\n", offsetof(fest_scheme, global_time_step));
  printf("fest_scheme.ilimiter_switch %zu\n", offsetof(fest_scheme, ilimiter_switch));
  printf("fest_scheme.jlimiter_switch %zu\n", offsetof(fest_scheme, jlimiter_switch));
  printf("fest_scheme.klimiter_switch %zu\n", offsetof(fest_scheme, klimiter_switch));
  printf("fest_scheme.itlimiter_switch %zu\n", offsetof(fest_scheme, itlimiter_switch));
  printf("fest_scheme.jtlimiter_switch %zu\n", offsetof(fest_scheme, jtlimiter_switch));
  printf("fest_scheme.ktlimiter_switch %zu\n", offsetof(fest_scheme, ktlimiter_switch));
  printf("fest_scheme.iPB_switch %zu\n", offsetof(fest_scheme, iPB_switch));
  printf("fest_scheme.jPB_switch %zu\n", offsetof(fest_scheme, jPB_switch));
  printf("fest_scheme.kPB_switch %zu\n", offsetof(fest_scheme, kPB_switch));
  printf("fest_scheme.turbulence %zu\n", offsetof(fest_scheme, turbulence));
  printf("fest_scheme.accur %zu\n", offsetof(fest_scheme, accur));
  printf("fest_scheme.limiter %zu\n", offsetof(fest_scheme, limiter));
  printf("fest_scheme.transition %zu\n", offsetof(fest_scheme, transition));
  printf("fest_bc %zu\n", sizeof(fest_bc));
  printf("fest_bc.id %zu\n", offsetof(fest_bc, id));
  printf("fest_bc.partner_block %zu\n", offsetof(fest_bc, partner_block));
  printf("fest_bc.partner_face %zu\n", offsetof(fest_bc, partner_face));
  printf("fest_bc.fixed_density %zu\n", offsetof(fest_bc, fixed_density));
  printf("fest_bc.fixed_pressure %zu\n", offsetof(fest_bc, fixed_pressure));
  printf("fest_bc.fixed_x_speed %zu\n", offsetof(fest_bc, fixed_x_speed));
  printf("fest_bc.fixed_y_speed %zu\n", offsetof(fest_bc, fixed_y_speed));
  printf("fest_bc.fixed_z_speed %zu\n", offsetof(fest_bc, fixed_z_speed));
  printf("fest_bc.fixed_tk %zu\n", offsetof(fest_bc, fixed_tk));
  printf("fest_bc.fixed_tw %zu\n", offsetof(fest_bc, fixed_tw));
  printf("fest_bc.fixed_wall_temperature %zu\n", offsetof(fest_bc, fixed_wall_temperature));
  printf("fest_bc.fixed_Tpressure %zu\n", offsetof(fest_bc, fixed_Tpressure));
  printf("fest_bc.fixed_Ttemperature %zu\n", offsetof(fest_bc, fixed_Ttemperature));
  printf("fest_bc.block_id %zu\n", offsetof(fest_bc, block_id));
  printf("fest_bc.partner_orient %zu\n", offsetof(fest_bc, partner_orient));
  printf("fest_bc.fixed_tv %zu\n", offsetof(fest_bc, fixed_tv));
  printf("fest_bc.fixed_tkl %zu\n", offsetof(fest_bc, fixed_tkl));
  printf("fest_bc.fixed_tgm %zu\n", offsetof(fest_bc, fixed_tgm));
  return 0;
}
