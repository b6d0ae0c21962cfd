// host_math.h -- FP32 setup math of the solver (see host_math.cpp).
#pragma once

namespace bbg {

void build_grid(const double dmin[3], const double dmax[3], double spacing, double scale,
                int dims[3], float minp[3], float len[3], float bmin[3], float bmax[3]);
float compute_mass(int lattice_kind, float target_density, float spacing, float kernel_radius);
float compute_delta_denom(float spacing, float kernel_radius);
float compute_delta(float mass_over_density_sq, float delta_denom, float dt);
unsigned number_of_time_steps(float time_step, float sound_speed, float scale, float kernel_radius,
                              float mass, float max_force);
float float_above(double t);

}  // namespace bbg
