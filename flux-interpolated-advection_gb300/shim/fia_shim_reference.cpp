// fia_shim_reference.cpp -- the reference's 3D entry points, under its own names and
// signatures, forwarded to libfia through fia_shim.hpp.
//
// Added to the reference build (its makefile's object list, makefile:7) in place of
// src/move_substances_3d.cpp, src/advect_velocity_flux_advection_3d.cpp,
// src/update_fluid_velocity_3d.cpp and src/calc_pressure_3d.cpp, and linked with libfia; it
// compiles against the reference's own headers (include/), with MY_FLOAT_TYPE float as shipped
// or double.  The rest of the reference (main.cpp's 3D loop, Grid_3D, the output) stays as it
// is.  Dropping those four files also drops the build's amgcl dependency.  The CFL time step
// (calc_time_step_length_from_CFL_number_3D) shares its translation unit with the 1D/2D
// versions, so it is not replaced here; fia_shim::calc_time_step_length_from_CFL_number_3D is
// the device-reduction version for a caller that wants it.
//
// Declarations followed: move_substances_3d.h:48-66, advect_velocity_flux_advection_3d.h:107-124,
// update_fluid_velocity_3d.h:38-56, calc_pressure_3d.h:6-9.
#include "grid_3d.h"
#include "move_substances_3d.h"
#include "advect_velocity_flux_advection_3d.h"
#include "update_fluid_velocity_3d.h"
#include "calc_pressure_3d.h"

#include "fia_shim.hpp"

namespace smoke_simulation {

void move_substances_3D(Grid_3D& all_grid, int i_frame, const MY_FLOAT_TYPE time_step_length,
                        const bool use_flux_advection, const bool use_MacCormack_scheme,
                        const bool use_clamping_in_MacCormack_scheme, const int num_gauss_quad_boundary,
                        const int num_gauss_quad_bulk, const bool enable_eliminate_zero_velocity_false_diffusion,
                        const std::string split_method, const std::string integral_method,
                        const int num_gauss_quadrature_points, const std::string interpolation_method,
                        bool use_integral, const int num_gauss_quadrature_point_for_integrate_density,
                        const bool enable_cell_volume_correction, const MY_FLOAT_TYPE minimal_area) {
    fia_shim::move_substances_3D(all_grid, i_frame, time_step_length, use_flux_advection, use_MacCormack_scheme,
                                 use_clamping_in_MacCormack_scheme, num_gauss_quad_boundary, num_gauss_quad_bulk,
                                 enable_eliminate_zero_velocity_false_diffusion, split_method, integral_method,
                                 num_gauss_quadrature_points, interpolation_method, use_integral,
                                 num_gauss_quadrature_point_for_integrate_density, enable_cell_volume_correction,
                                 minimal_area);
}

void advect_velocity_xyz_flux_advection_3D_std_thread(
    Grid_3D& all_grid, const MY_FLOAT_TYPE time_step_length, const bool use_MacCormack_scheme,
    const bool use_clamping_in_MacCormack_scheme, const int num_gauss_quad_boundary, const int num_gauss_quad_bulk,
    const bool enable_eliminate_zero_velocity_false_diffusion, const std::string integral_method,
    const int num_gauss_quadrature_points_on_one_triangle, const std::string interpolation_method, bool use_integral,
    const int num_gauss_quadrature_point_for_integrate_density, const bool enable_cell_volume_correction,
    const MY_FLOAT_TYPE minimal_area) {
    fia_shim::advect_velocity_xyz_flux_advection_3D_std_thread(
        all_grid, time_step_length, use_MacCormack_scheme, use_clamping_in_MacCormack_scheme, num_gauss_quad_boundary,
        num_gauss_quad_bulk, enable_eliminate_zero_velocity_false_diffusion, integral_method,
        num_gauss_quadrature_points_on_one_triangle, interpolation_method, use_integral,
        num_gauss_quadrature_point_for_integrate_density, enable_cell_volume_correction, minimal_area);
}

void update_fluid_velocity_3D(Grid_3D& all_grid, int i_frame, const MY_FLOAT_TYPE time_step_length,
                              const bool use_flux_advection, const bool use_MacCormack_scheme,
                              const bool use_clamping_in_MacCormack_scheme, const int num_gauss_quad_boundary,
                              const int num_gauss_quad_bulk, const bool enable_eliminate_zero_velocity_false_diffusion,
                              const std::string split_method, const std::string integral_method,
                              const std::string interpolation_method, const bool enable_cell_volume_correction,
                              const bool fix_velocity, const int num_gauss_quadrature_point_for_integrate_density,
                              const bool use_integral, const MY_FLOAT_TYPE minimal_area) {
    fia_shim::update_fluid_velocity_3D(all_grid, i_frame, time_step_length, use_flux_advection, use_MacCormack_scheme,
                                       use_clamping_in_MacCormack_scheme, num_gauss_quad_boundary, num_gauss_quad_bulk,
                                       enable_eliminate_zero_velocity_false_diffusion, split_method, integral_method,
                                       interpolation_method, enable_cell_volume_correction, fix_velocity,
                                       num_gauss_quadrature_point_for_integrate_density, use_integral, minimal_area);
}

void calc_pressure_3D(Grid_3D& all_grid) { fia_shim::calc_pressure_3D(all_grid); }

void calc_pressure_gradient_term_3D(Grid_3D& all_grid) { fia_shim::calc_pressure_gradient_term_3D(all_grid); }

}  // namespace smoke_simulation
