// Driver of the reference-signature shim (flux-interpolated-advection_gb300/shim/): calls the
// reference's 3D entry points on a grid, as the reference's main loop does (main.cpp:600-721),
// and writes what each call left in the grid.
//
// Built two ways:
//   -DFIA_REFERENCE_GRID  the reference's own Grid_3D and declarations (its include/ directory
//                         on the include path, fia_shim_reference.cpp linked): the maintainer's
//                         build, compiled and linked where the reference checkout exists;
//   otherwise             a stand-in grid with the Grid_3D members the path touches
//                         (grid_3d.h:31-52), calling the fia_shim templates directly: runs on
//                         GPU hosts, which have no reference checkout.
// -DFIA_GRID_REAL=float|double selects the scalar type (the reference's MY_FLOAT_TYPE).
//
// usage: shim_driver <input> <output>
//   input : int32 n, float64 h, float64 dt, then density, u, v, w as float64 (Grid_3D order)
//   output: float64 arrays, in order: density after move_substances_3D; u, v, w after
//           advect_velocity_xyz_flux_advection_3D_std_thread; u, v, w, pressure and the three
//           wall momentum totals after calc_pressure_gradient_term_3D; pressure after
//           calc_pressure_3D; u, v, w after update_fluid_velocity_3D (frame 1: advect, then
//           project); the CFL time step (CFL 2, now 0, movie frame 0, 60 fps) and its
//           write-frame flag.
#include <cstdio>
#include <string>
#include <vector>

#ifdef FIA_REFERENCE_GRID
#include "grid_3d.h"
#include "move_substances_3d.h"
#include "advect_velocity_flux_advection_3d.h"
#include "update_fluid_velocity_3d.h"
#include "calc_pressure_3d.h"
#include "fia_shim.hpp"
typedef MY_FLOAT_TYPE Real;
typedef smoke_simulation::Grid_3D Grid;
using smoke_simulation::move_substances_3D;
using smoke_simulation::advect_velocity_xyz_flux_advection_3D_std_thread;
using smoke_simulation::update_fluid_velocity_3D;
using smoke_simulation::calc_pressure_3D;
using smoke_simulation::calc_pressure_gradient_term_3D;
#else
#include "fia_shim.hpp"
#ifndef FIA_GRID_REAL
#define FIA_GRID_REAL double
#endif
typedef FIA_GRID_REAL Real;
// the members of the reference's Grid_3D that the shim reads and writes
struct Grid {
    const int Grid_num_x, Grid_num_y, Grid_num_z;
    const Real _cell_length;
    std::vector<Real> velocity_in_voxel_face_x, velocity_in_voxel_face_y, velocity_in_voxel_face_z;
    std::vector<Real> pressure, substance_density;
    Real total_loss_of_momentum_x = 0, total_loss_of_momentum_y = 0, total_loss_of_momentum_z = 0;
    Grid(int nx, int ny, int nz, Real h)
        : Grid_num_x(nx), Grid_num_y(ny), Grid_num_z(nz), _cell_length(h),
          velocity_in_voxel_face_x((size_t)(nx + 1) * ny * nz), velocity_in_voxel_face_y((size_t)nx * (ny + 1) * nz),
          velocity_in_voxel_face_z((size_t)nx * ny * (nz + 1)), pressure((size_t)nx * ny * nz),
          substance_density((size_t)nx * ny * nz) {}
};
using fia_shim::move_substances_3D;
using fia_shim::advect_velocity_xyz_flux_advection_3D_std_thread;
using fia_shim::update_fluid_velocity_3D;
using fia_shim::calc_pressure_3D;
using fia_shim::calc_pressure_gradient_term_3D;
#endif

static bool read_array(FILE* f, std::vector<Real>& a) {
    std::vector<double> t(a.size());
    if (std::fread(t.data(), sizeof(double), t.size(), f) != t.size()) return false;
    for (size_t i = 0; i < t.size(); ++i) a[i] = (Real)t[i];
    return true;
}
static void write_array(FILE* f, const std::vector<Real>& a) {
    std::vector<double> t(a.begin(), a.end());
    std::fwrite(t.data(), sizeof(double), t.size(), f);
}
static void write_value(FILE* f, double x) { std::fwrite(&x, sizeof(double), 1, f); }

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: shim_driver <input> <output>\n");
        return 2;
    }
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int n = 0;
    double h = 0, dt = 0;
    if (std::fread(&n, sizeof(int), 1, in) != 1 || std::fread(&h, sizeof(double), 1, in) != 1 ||
        std::fread(&dt, sizeof(double), 1, in) != 1 || n < 2)
        return 2;
    Grid g(n, n, n, (Real)h);
    if (!read_array(in, g.substance_density) || !read_array(in, g.velocity_in_voxel_face_x) ||
        !read_array(in, g.velocity_in_voxel_face_y) || !read_array(in, g.velocity_in_voxel_face_z))
        return 2;
    std::fclose(in);
    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    const Real step = (Real)dt, minimal_area = (Real)1.0;
    // the benchmark flags: flux advection, WENO6, xz-CellFaceAligned, k = 3, y-integral,
    // zero-velocity correction, no MacCormack, no volume correction, no triangulation
    move_substances_3D(g, 0, step, true, false, false, 1, 1, true, std::string("xz-CellFaceAligned"),
                       std::string("gauss"), 1, std::string("WENO6"), true, 3, false, minimal_area);
    write_array(out, g.substance_density);
    advect_velocity_xyz_flux_advection_3D_std_thread(g, step, false, false, 1, 1, true, std::string("gauss"), 1,
                                                     std::string("WENO6"), true, 3, false, minimal_area);
    write_array(out, g.velocity_in_voxel_face_x);
    write_array(out, g.velocity_in_voxel_face_y);
    write_array(out, g.velocity_in_voxel_face_z);
    calc_pressure_gradient_term_3D(g);
    write_array(out, g.velocity_in_voxel_face_x);
    write_array(out, g.velocity_in_voxel_face_y);
    write_array(out, g.velocity_in_voxel_face_z);
    write_array(out, g.pressure);
    write_value(out, (double)g.total_loss_of_momentum_x);
    write_value(out, (double)g.total_loss_of_momentum_y);
    write_value(out, (double)g.total_loss_of_momentum_z);
    calc_pressure_3D(g);
    write_array(out, g.pressure);
    update_fluid_velocity_3D(g, 1, step, true, false, false, 1, 1, true, std::string("xz-CellFaceAligned"),
                             std::string("gauss"), std::string("WENO6"), false, false, 3, true, minimal_area);
    write_array(out, g.velocity_in_voxel_face_x);
    write_array(out, g.velocity_in_voxel_face_y);
    write_array(out, g.velocity_in_voxel_face_z);
    bool write_frame = false;
    const Real cfl_dt = fia_shim::calc_time_step_length_from_CFL_number_3D(g, (Real)0, 0, write_frame, 2, (Real)60);
    write_value(out, (double)cfl_dt);
    write_value(out, write_frame ? 1.0 : 0.0);
    std::fclose(out);
    return 0;
}
