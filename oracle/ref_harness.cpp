// ref_harness.cpp -- C entry points over the reference's own translation units.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles the reference's hot-path
// sources (where they lie in the reference checkout) together with this file into
// oracle/_ref/libfia_ref_{float,double}.so.  The tests use it to pin the oracle and to
// write the golden fixtures under tests/golden/.
//
// The orchestration of move_substances_3D (move_substances_3d.cpp:38-240) and of
// advect_velocity_flux_advection_3D_std_thread (advect_velocity_flux_advection_3d.cpp:252-576)
// lives in translation units that include amgcl, which is not available, so the few
// calls they make are restated here; every numerical step runs in the reference's code.

#include <vector>
#include <string>
#include <cstring>
#include <thread>

#include "grid_3d.h"
#include "utils.h"
#include "calc_psi_3D.h"
#include "gauss_quadrature_points.h"
#include "split_face_3D.h"
#include "backtrace_and_calc_all_quadrature_point_list.h"
#include "backtrace_and_calc_all_quadrature_point_list_for_integrate_density.h"
#include "calc_density_in_cell_from_quadrature_point_list.h"
#include "calc_density_in_cell_from_quadrature_point_list_for_integrate_density.h"
#include "calc_velocity_from_quadrature_point_list.h"
#include "calc_velocity_from_quadrature_point_list_use_integral.h"
#include "linear_interpolation_1d.h"
#include "linear_interpolation_3d.h"
#include "WENO6_interpolation_1d.h"
#include "WENO6_interpolation_3d.h"

using namespace smoke_simulation;

namespace {

const char* interp_name(int c) {
    switch (c) { case 0: return "WENO6"; case 1: return "linear"; case 2: return "1Dy_linear"; default: return "WENO6"; }
}
const char* split_name(int c) {
    switch (c) {
        case 0: return "xz-CellFaceAligned";
        case 1: return "xz-AxisAligned";
        case 2: return "x-CellFaceAligned_z-AxisAligned";
        case 3: return "x-AxisAligned_z-CellFaceAligned";
        default: return "no-split";
    }
}

template <typename T>
void to_vec(std::vector<MY_FLOAT_TYPE>& v, const T* a, long n) { v.resize(n); for (long i = 0; i < n; ++i) v[i] = (MY_FLOAT_TYPE)a[i]; }

void fill_velocity(Grid_3D& g, const double* u, const double* v, const double* w) {
    int nx = g.Grid_num_x, ny = g.Grid_num_y, nz = g.Grid_num_z;
    to_vec(g.velocity_in_voxel_face_x, u, (long)(nx + 1) * ny * nz);
    to_vec(g.velocity_in_voxel_face_y, v, (long)nx * (ny + 1) * nz);
    to_vec(g.velocity_in_voxel_face_z, w, (long)nx * ny * (nz + 1));
}

// one density pass (advect_density_flux_advection_3D_std_thread, move_substances_3d.cpp:585-841),
// single-threaded: i_thread = 0 over the whole face range.
void density_pass(Grid_3D& g, std::vector<MY_FLOAT_TYPE>& values, MY_FLOAT_TYPE dt,
                  const std::string& split, const std::string& interp, const std::string& interp_psi,
                  bool zero_vel, bool use_integral, int k, MY_FLOAT_TYPE minimal_area, bool maccormack = false) {
    const size_t nface = (size_t)g.Grid_num_x * g.Grid_num_y * g.Grid_num_z * 6;
    calc_psi_on_cell_face_from_density_on_cell_center_3D(
        g, g.psi_substance_density_cell_face_x, g.psi_substance_density_cell_face_y,
        g.psi_substance_density_cell_face_z, values, g.Grid_num_x, g.Grid_num_y, g.Grid_num_z,
        g._cell_length, interp_psi, k, use_integral);
    std::vector<MY_FLOAT_TYPE> after(values.size(), 0.0);
    if (use_integral) {
        quadrature_point_vector qd, qp, qv;
        backtrace_and_calc_all_quadrature_point_list_for_integrate_density(
            -1, qd, qp, qv, 0, nface, maccormack, g, dt, split, "gauss", 1, 0, interp, zero_vel, k, false,
            "density", minimal_area);
        calc_density_in_cell_from_quadrature_point_list_for_integrate_density(qd, qp, g, after, 0, interp, values);
    } else {
        quadrature_point_vector q;
        backtrace_and_calc_all_quadrature_point_list(-1, q, 0, nface, maccormack, g, dt, split, "gauss", 1, 0,
                                                     interp, zero_vel, minimal_area);
        calc_density_in_cell_from_quadrature_point_list(q, g, after, 0, interp);
    }
    values = after;
}

// one velocity-component pass (advect_velocity_flux_advection_3d.cpp:252-576).
void velocity_pass(Grid_3D& g, int dim, std::vector<MY_FLOAT_TYPE>& values, MY_FLOAT_TYPE dt,
                   const std::string& split, const std::string& interp, const std::string& interp_psi,
                   bool zero_vel, bool use_integral, int k, MY_FLOAT_TYPE minimal_area) {
    int dx = dim == 0, dy = dim == 1, dz = dim == 2;
    const size_t nface = (size_t)(g.Grid_num_x + dx) * (g.Grid_num_y + dy) * (g.Grid_num_z + dz) * 6;
    std::vector<MY_FLOAT_TYPE>& psi = dim == 0 ? g.psi_velocity_x_cell_face : (dim == 1 ? g.psi_velocity_y_cell_face : g.psi_velocity_z_cell_face);
    calc_discrete_psi_velocity_3D(dim, g, psi, values, g.Grid_num_x, g.Grid_num_y, g.Grid_num_z, g._cell_length,
                                  interp_psi, k, use_integral);
    std::vector<MY_FLOAT_TYPE> after(values.size(), 0.0);
    if (use_integral) {
        quadrature_point_vector qd, qp, qv;
        backtrace_and_calc_all_quadrature_point_list_for_integrate_velocity(
            dim, qd, qp, qv, 0, nface, false, g, dt, split, "gauss", 1, 0, interp, zero_vel, k, false, minimal_area);
        calc_velocity_from_quadrature_point_list_use_integral(dim, qd, qp, g, after, 0, interp, values);
    } else {
        quadrature_point_vector q;
        backtrace_and_calc_all_quadrature_point_list(dim, q, 0, nface, false, g, dt, split, "gauss", 1, 0,
                                                     interp, zero_vel, minimal_area);
        calc_velocity_from_quadrature_point_list(dim, q, g, after, 0, interp);
    }
    values = after;
}

}  // namespace

extern "C" {

int fr_scalar_bytes(void) { return (int)sizeof(MY_FLOAT_TYPE); }

// kind: 0 WENO6 centre, 1/2/3 WENO6 x/y/z faces, 4 linear centre, 5/6/7 linear faces,
//       8 WENO6 1Dy centre, 9/10/11 1Dy-linear faces x/y/z, 12 1Dy-linear psi_y (density)
int fr_interp(int kind, const double* a, int nx, int ny, int nz, double h, const double* pts, long n, double* out) {
    Grid_3D g(nx, ny, nz, (MY_FLOAT_TYPE)h);
    long na = (kind == 1 || kind == 5 || kind == 9) ? (long)(nx + 1) * ny * nz
            : (kind == 2 || kind == 6 || kind == 10 || kind == 12) ? (long)nx * (ny + 1) * nz
            : (kind == 3 || kind == 7 || kind == 11) ? (long)nx * ny * (nz + 1) : (long)nx * ny * nz;
    std::vector<MY_FLOAT_TYPE> A; to_vec(A, a, na);
    for (long i = 0; i < n; ++i) {
        VEC3_TYPE p((MY_FLOAT_TYPE)pts[3 * i], (MY_FLOAT_TYPE)pts[3 * i + 1], (MY_FLOAT_TYPE)pts[3 * i + 2]);
        MY_FLOAT_TYPE r = 0;
        switch (kind) {
            case 0: r = WENO6_interpolation_3D_cell_center_values(p, A, g); break;
            case 1: r = WENO6_interpolation_3D_cell_face_x_values(p, A, g); break;
            case 2: r = WENO6_interpolation_3D_cell_face_y_values(p, A, g); break;
            case 3: r = WENO6_interpolation_3D_cell_face_z_values(p, A, g); break;
            case 4: r = linear_interpolation_3D_cell_center_values(p, A, g); break;
            case 5: r = linear_interpolation_3D_cell_face_x_values(p, A, g); break;
            case 6: r = linear_interpolation_3D_cell_face_y_values(p, A, g); break;
            case 7: r = linear_interpolation_3D_cell_face_z_values(p, A, g); break;
            case 8: r = WENO6_interpolation_1Dy_cell_center_values(p, A, g); break;
            case 9: r = linear_interpolation_1Dy_cell_face_x_values(p, A, g); break;
            case 10: r = linear_interpolation_1Dy_cell_face_y_values(p, A, g); break;
            case 11: r = linear_interpolation_1Dy_cell_face_z_values(p, A, g); break;
            case 12: g.psi_substance_density_cell_face_y = A;
                     r = g.calc_interpolated_psi_density(p, "1Dy_linear")[1]; break;
            default: return -1;
        }
        out[i] = (double)r;
    }
    return 0;
}

// psi_y of a density field; interp code 0 WENO6, 1 linear, 3 const
int fr_psi_density(const double* rho, int nx, int ny, int nz, double h, int interp, int k, int use_integral, double* psi_y) {
    Grid_3D g(nx, ny, nz, (MY_FLOAT_TYPE)h);
    std::vector<MY_FLOAT_TYPE> R; to_vec(R, rho, (long)nx * ny * nz);
    std::string m = interp == 3 ? "const" : interp_name(interp);
    calc_psi_on_cell_face_from_density_on_cell_center_3D(
        g, g.psi_substance_density_cell_face_x, g.psi_substance_density_cell_face_y, g.psi_substance_density_cell_face_z,
        R, nx, ny, nz, g._cell_length, m, k, use_integral != 0);
    for (size_t i = 0; i < g.psi_substance_density_cell_face_y.size(); ++i) psi_y[i] = g.psi_substance_density_cell_face_y[i];
    return 0;
}

// Pieces of one face: (centroid xyz, scaled normal xyz) per piece, in emission order.
int fr_split_face(const double* verts12, double h, int split, double minimal_area, int max_out, double* out6, int* nout) {
    Grid_3D g(4, 4, 4, (MY_FLOAT_TYPE)h);
    cell_face_3D face;
    for (int i = 0; i < 4; ++i)
        face._vertex_list[i]._vertex_pos = VEC3_TYPE((MY_FLOAT_TYPE)verts12[3 * i], (MY_FLOAT_TYPE)verts12[3 * i + 1], (MY_FLOAT_TYPE)verts12[3 * i + 2]);
    quadrature_point_vector q;
    split_face_and_add_quadrature_points_3D_ref(q, g, face, split_name(split), 0, 0, 0, 0, "gauss", 1, 1.0, (MY_FLOAT_TYPE)minimal_area);
    int n = (int)q._quadtarure_position[0].size();
    *nout = n;
    for (int i = 0; i < n && i < max_out; ++i)
        for (int d = 0; d < 3; ++d) {
            out6[6 * i + d] = q._quadtarure_position[0][i][d];
            out6[6 * i + 3 + d] = q._weighted_area_normal[0][i][d];
        }
    return 0;
}

// One density pass.  interp: 0 WENO6 1 linear 2 1Dy_linear; psi: 0 WENO6 1 linear 3 const.
int fr_density_pass(int nx, int ny, int nz, double h, const double* u, const double* v, const double* w,
                    const double* rho, double dt, int interp, int psi, int use_integral, int zero_vel,
                    int split, int k, double minimal_area, double* out, int maccormack) {
    Grid_3D g(nx, ny, nz, (MY_FLOAT_TYPE)h);
    fill_velocity(g, u, v, w);
    std::vector<MY_FLOAT_TYPE> R; to_vec(R, rho, (long)nx * ny * nz);
    std::string ps = psi == 3 ? "const" : interp_name(psi);
    density_pass(g, R, (MY_FLOAT_TYPE)dt, split_name(split), interp_name(interp), ps, zero_vel != 0, use_integral != 0, k,
                 (MY_FLOAT_TYPE)minimal_area, maccormack != 0);
    for (size_t i = 0; i < R.size(); ++i) out[i] = R[i];
    return 0;
}

// move_substances_3D, flux branch with the zero-velocity correction, restated from
// move_substances_3d.cpp:58-226 (interp 0 WENO6 or 1 linear).
int fr_move_substances_3D(int nx, int ny, int nz, double h, const double* u, const double* v, const double* w,
                          double* rho, double dt, int interp, int split, int k, int correction, int use_integral,
                          double minimal_area, int maccormack) {
    Grid_3D g(nx, ny, nz, (MY_FLOAT_TYPE)h);
    fill_velocity(g, u, v, w);
    long n = (long)nx * ny * nz;
    std::vector<MY_FLOAT_TYPE> before; to_vec(before, rho, n);
    std::vector<MY_FLOAT_TYPE> R = before;
    std::string im = interp_name(interp), ipsi = interp == 0 ? "WENO6" : "linear";
    const bool mc = maccormack != 0;
    density_pass(g, R, (MY_FLOAT_TYPE)dt, split_name(split), im, ipsi, false, use_integral != 0, k, (MY_FLOAT_TYPE)minimal_area, mc);
    if (correction) {
        std::vector<MY_FLOAT_TYPE> c = before;
        density_pass(g, c, (MY_FLOAT_TYPE)dt, split_name(split), im, ipsi, true, false, k, (MY_FLOAT_TYPE)minimal_area, mc);
        for (long i = 0; i < n; ++i) { c[i] *= -1.0; c[i] += before[i]; }
        density_pass(g, c, (MY_FLOAT_TYPE)dt, "xz-AxisAligned", "1Dy_linear", "const", false, false, k, (MY_FLOAT_TYPE)minimal_area, mc);
        for (long i = 0; i < n; ++i) R[i] += c[i];
    }
    for (long i = 0; i < n; ++i) rho[i] = R[i];
    return 0;
}

// Advected cell volumes of a density main pass (integral branch): the volume points the
// reference collects with enable_cell_volume_correction, summed by its
// calc_cell_volumes_from_quadrature_point_list (calc_density_in_cell_from_quadrature_point_list.cpp:135-156).
int fr_cell_volumes(int nx, int ny, int nz, double h, const double* u, const double* v, const double* w, double dt,
                    int interp, int split, int k, double minimal_area, int maccormack, double* out) {
    Grid_3D g(nx, ny, nz, (MY_FLOAT_TYPE)h);
    fill_velocity(g, u, v, w);
    const size_t nface = (size_t)nx * ny * nz * 6;
    std::vector<MY_FLOAT_TYPE> vol((size_t)nx * ny * nz, 0.0);
    quadrature_point_vector qd, qp, qv;
    backtrace_and_calc_all_quadrature_point_list_for_integrate_density(
        -1, qd, qp, qv, 0, nface, maccormack != 0, g, (MY_FLOAT_TYPE)dt, split_name(split), "gauss", 1, 0,
        interp_name(interp), false, k, true, "density", (MY_FLOAT_TYPE)minimal_area);
    calc_cell_volumes_from_quadrature_point_list(qv, g, vol, 0);
    for (size_t i = 0; i < vol.size(); ++i) out[i] = vol[i];
    return 0;
}

// One velocity-component pass in the reference's defined ("linear") form, integral path:
// advect_velocity_{x,y,z}_flux_advection_3D_std_thread with the correction off.
int fr_velocity_pass_linear(int nx, int ny, int nz, double h, const double* u, const double* v, const double* w,
                            int dim, double dt, int k, double minimal_area, double* out) {
    Grid_3D g(nx, ny, nz, (MY_FLOAT_TYPE)h);
    fill_velocity(g, u, v, w);
    const char* split = dim == 0 ? "x-AxisAligned_z-CellFaceAligned" : (dim == 1 ? "xz-CellFaceAligned" : "x-CellFaceAligned_z-AxisAligned");
    std::vector<MY_FLOAT_TYPE> vals = dim == 0 ? g.velocity_in_voxel_face_x : (dim == 1 ? g.velocity_in_voxel_face_y : g.velocity_in_voxel_face_z);
    velocity_pass(g, dim, vals, (MY_FLOAT_TYPE)dt, split, "linear", "linear", false, true, k, (MY_FLOAT_TYPE)minimal_area);
    for (size_t i = 0; i < vals.size(); ++i) out[i] = vals[i];
    return 0;
}

}  // extern "C"
