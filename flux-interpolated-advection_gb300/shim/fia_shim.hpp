// fia_shim.hpp -- the reference's 3D entry points over libfia's C ABI (include/fia.h).
//
// The reference program (nyhirasawa/Flux-Interpolated-Advection) advances its 3D smoke through
// five functions that take a Grid_3D& and mutate its std::vectors in place:
//
//   move_substances_3D                                 move_substances_3d.h:48-66
//   advect_velocity_xyz_flux_advection_3D_std_thread   advect_velocity_flux_advection_3d.h:107-124
//   update_fluid_velocity_3D                           update_fluid_velocity_3d.h:38-56
//   calc_pressure_3D, calc_pressure_gradient_term_3D   calc_pressure_3d.h:6-9
//   calc_time_step_length_from_CFL_number_3D           calc_time_step_length_from_CFL_number.h:33-39
//
// This header implements each of them, with the same parameter lists and meaning, as a
// template over the grid type: any type with the Grid_3D members the path touches
// (grid_3d.h:31-52: Grid_num_x/y/z, _cell_length, substance_density, pressure,
// velocity_in_voxel_face_x/y/z, total_loss_of_momentum_x/y/z; std::vector<float> or
// std::vector<double>, the reference's MY_FLOAT_TYPE).  fia_shim_reference.cpp instantiates it
// for the reference's own Grid_3D under the reference's names, which is the translation unit
// a maintainer links into the reference build in place of move_substances_3d.cpp,
// advect_velocity_flux_advection_3d.cpp, update_fluid_velocity_3d.cpp and calc_pressure_3d.cpp.
//
// Every call copies the fields it reads from the grid to the device and the fields it writes
// back (host-buffer round trip, synchronous, like the reference's void functions).  One
// device session is kept per (grid size, cell length, precision) and reused by later calls.
//
// Settings (fia_shim::options(), initialised from the environment on first use):
//   FIA_SHIM_PRECISION  fp64 (default: the plain form, FP64 throughout) or fp32c (the chosen
//                       form: FP32 advection with compensated sums, FP64 reductions)
//   FIA_SHIM_SOLVER     pcg (default: Jacobi-PCG) or learned (flexible CG with the learned
//                       preconditioner; fp32c only; needs FIA_SHIM_WEIGHTS)
//   FIA_SHIM_WEIGHTS    path of the learned preconditioner's weights (float32, as written by
//                       fia_learned_get_weights)
//   FIA_SHIM_TOL        pressure tolerance, relative residual (default 1e-8: the reference's
//                       amgcl solve receives no tolerance, calc_pressure_3d.cpp:157-160, so it
//                       runs to the library default of its solver, which is not in this tree)
//
// Errors: the reference has no error convention (void functions; its clipper exit(0)s on a
// failed cut, facecutter.h:191-204).  The shim keeps the void signatures: a negative return
// of the library (bad argument, CUDA failure, unsupported option) prints the library's
// message and exits with status 1; positive status bits (numerical warnings) are printed and
// the run continues.  Options the library does not implement exit the same way: the
// semi-Lagrangian branch (use_flux_advection == false) and split or interpolation methods
// outside the four split methods and WENO6 / linear (the reference's "1Dy_linear" and
// "WENO6-optimized" are internal choices of its passes, not user settings of this path).
#pragma once

#include "fia.h"

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

namespace fia_shim {

struct Options {
    int precision = FIA_FP64;
    int solver = FIA_SOLVER_PCG_JACOBI;
    double pressure_tol = 1e-8;
    int max_iter = 100000;
    int fallback_iter = 200;
    std::string weights;
};

inline Options options_from_env() {
    Options o;
    if (const char* p = std::getenv("FIA_SHIM_PRECISION")) o.precision = std::string(p) == "fp32c" ? FIA_FP32C : FIA_FP64;
    if (const char* s = std::getenv("FIA_SHIM_SOLVER")) o.solver = std::string(s) == "learned" ? FIA_SOLVER_FCG_LEARNED
                                                                                           : FIA_SOLVER_PCG_JACOBI;
    if (const char* w = std::getenv("FIA_SHIM_WEIGHTS")) o.weights = w;
    if (const char* t = std::getenv("FIA_SHIM_TOL")) o.pressure_tol = std::atof(t);
    return o;
}

// Settings of the shim; change them before the first call (sessions keep their precision).
inline Options& options() {
    static Options o = options_from_env();
    return o;
}

[[noreturn]] inline void fatal(const char* what, const char* msg) {
    std::fprintf(stderr, "%s: %s\n", what, msg);
    std::exit(1);
}

inline int check(int rc, const char* what) {
    if (rc < 0) fatal(what, fia_error_string(rc));
    if (rc > 0) std::fprintf(stderr, "%s: status bits 0x%x\n", what, rc);
    return rc;
}

struct SessionKey {
    int nx, ny, nz, precision;
    double h;
    bool operator<(const SessionKey& o) const {
        return std::tie(nx, ny, nz, precision, h) < std::tie(o.nx, o.ny, o.nz, o.precision, o.h);
    }
};

// The sessions of this process, one per grid size, cell length and precision; destroyed at exit.
struct Sessions {
    std::map<SessionKey, fia_session*> map;
    std::mutex mu;
    ~Sessions() {
        for (auto& kv : map) fia_destroy(kv.second);
    }
};
inline Sessions& sessions() {
    static Sessions s;
    return s;
}

inline std::vector<float> read_weights(const std::string& path) {
    std::vector<float> w((size_t)fia_learned_num_parameters());
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) fatal("fia_shim", ("cannot open FIA_SHIM_WEIGHTS file " + path).c_str());
    const size_t got = std::fread(w.data(), sizeof(float), w.size(), f);
    std::fclose(f);
    if (got != w.size()) fatal("fia_shim", ("short weights file " + path).c_str());
    return w;
}

inline fia_session* session(int nx, int ny, int nz, double h) {
    const Options& o = options();
    Sessions& S = sessions();
    std::lock_guard<std::mutex> lock(S.mu);
    const SessionKey key{nx, ny, nz, o.precision, h};
    auto it = S.map.find(key);
    if (it != S.map.end()) return it->second;
    fia_session* s = fia_create(nx, ny, nz, h, o.precision);
    if (!s) fatal("fia_create", fia_error_string(FIA_ERR_CUDA));
    if (o.solver == FIA_SOLVER_FCG_LEARNED) {
        if (o.precision != FIA_FP32C) fatal("fia_shim", "the learned solver needs FIA_SHIM_PRECISION=fp32c");
        if (o.weights.empty()) fatal("fia_shim", "the learned solver needs FIA_SHIM_WEIGHTS");
        const std::vector<float> w = read_weights(o.weights);
        check(fia_learned_set_weights(s, w.data(), (long long)w.size()), "fia_learned_set_weights");
    }
    S.map[key] = s;
    return s;
}

template <class G>
using RealOf = typename std::decay<decltype(std::declval<G&>().substance_density[0])>::type;

template <class G>
constexpr int host_type() {
    static_assert(std::is_same<RealOf<G>, double>::value || std::is_same<RealOf<G>, float>::value,
                  "grid fields must be float or double");
    return std::is_same<RealOf<G>, double>::value ? FIA_HOST_F64 : FIA_HOST_F32;
}

// the session of a grid, after checking that its arrays have the Grid_3D sizes (grid_3d.cpp:13-47)
template <class G>
fia_session* session_for(const G& g) {
    const size_t nx = (size_t)g.Grid_num_x, ny = (size_t)g.Grid_num_y, nz = (size_t)g.Grid_num_z;
    if (g.substance_density.size() != nx * ny * nz || g.pressure.size() != nx * ny * nz ||
        g.velocity_in_voxel_face_x.size() != (nx + 1) * ny * nz ||
        g.velocity_in_voxel_face_y.size() != nx * (ny + 1) * nz ||
        g.velocity_in_voxel_face_z.size() != nx * ny * (nz + 1))
        fatal("fia_shim", "grid arrays do not have the Grid_3D sizes");
    return session(g.Grid_num_x, g.Grid_num_y, g.Grid_num_z, (double)g._cell_length);
}

// split_face_3D.cpp:26-41; the reference leaves the colours at zero (no cut) for any other name
inline int split_method_of(const std::string& s) {
    if (s == "xz-CellFaceAligned") return FIA_SPLIT_XZ_CELLFACE;
    if (s == "xz-AxisAligned") return FIA_SPLIT_XZ_AXIS;
    if (s == "x-CellFaceAligned_z-AxisAligned") return FIA_SPLIT_XCELLFACE_ZAXIS;
    if (s == "x-AxisAligned_z-CellFaceAligned") return FIA_SPLIT_XAXIS_ZCELLFACE;
    fatal("fia_shim", ("split_method not supported by the GPU path: " + s).c_str());
}

inline int interpolation_method_of(const std::string& s) {
    if (s == "WENO6") return FIA_INTERP_WENO6;
    if (s == "linear") return FIA_INTERP_LINEAR;
    fatal("fia_shim", ("interpolation_method not supported by the GPU path: " + s).c_str());
}

inline fia_advect_params advect_params(int split, const std::string& interpolation_method, bool use_integral, int k,
                                       bool zero_velocity_correction, bool maccormack, bool volume_correction,
                                       double minimal_area) {
    fia_advect_params p;
    fia_default_advect_params(&p);
    p.interpolation_method = interpolation_method_of(interpolation_method);
    p.split_method = split;
    p.num_gauss_quadrature_point_for_integrate_density = k;
    p.use_integral = use_integral ? 1 : 0;
    p.enable_eliminate_zero_velocity_false_diffusion = zero_velocity_correction ? 1 : 0;
    p.use_MacCormack_scheme = maccormack ? 1 : 0;
    p.enable_cell_volume_correction = volume_correction ? 1 : 0;
    p.minimal_area = minimal_area;
    return p;
}

inline fia_solver_params solver_params() {
    const Options& o = options();
    fia_solver_params sp;
    fia_default_solver_params(&sp);
    sp.tol = o.pressure_tol;
    sp.max_iter = o.max_iter;
    sp.method = o.solver;
    sp.fallback_iter = o.fallback_iter;
    return sp;
}

// move_substances_3D (move_substances_3d.cpp:38-240), flux-advection branch.  The clamping
// flag and the Gauss counts of the semi-Lagrangian and triangle quadratures have no role on
// this path (the reference passes them through unused there); integral_method likewise.
template <class G, class R>
void move_substances_3D(G& g, int /*i_frame*/, R time_step_length, bool use_flux_advection, bool use_MacCormack_scheme,
                        bool /*use_clamping_in_MacCormack_scheme*/, int /*num_gauss_quad_boundary*/,
                        int /*num_gauss_quad_bulk*/, bool enable_eliminate_zero_velocity_false_diffusion,
                        const std::string& split_method, const std::string& /*integral_method*/,
                        int /*num_gauss_quadrature_points*/, const std::string& interpolation_method, bool use_integral,
                        int num_gauss_quadrature_point_for_integrate_density, bool enable_cell_volume_correction,
                        R minimal_area) {
    if (!use_flux_advection) fatal("move_substances_3D", "the semi-Lagrangian branch is not part of the GPU path");
    fia_session* s = session_for(g);
    const fia_advect_params p = advect_params(split_method_of(split_method), interpolation_method, use_integral,
                                              num_gauss_quadrature_point_for_integrate_density,
                                              enable_eliminate_zero_velocity_false_diffusion, use_MacCormack_scheme,
                                              enable_cell_volume_correction, (double)minimal_area);
    check(fia_move_substances_3D_host(s, host_type<G>(), g.substance_density.data(), g.velocity_in_voxel_face_x.data(),
                                      g.velocity_in_voxel_face_y.data(), g.velocity_in_voxel_face_z.data(),
                                      (double)time_step_length, &p),
          "move_substances_3D");
}

// advect_velocity_xyz_flux_advection_3D_std_thread (advect_velocity_flux_advection_3d.cpp:1138-1272):
// each staggered component with its own split method (:620-628 and the y/z equivalents);
// enable_cell_volume_correction is accepted and, as in the reference, not applied to velocity.
template <class G, class R>
void advect_velocity_xyz_flux_advection_3D_std_thread(G& g, R time_step_length, bool use_MacCormack_scheme,
                                                      bool /*use_clamping_in_MacCormack_scheme*/,
                                                      int /*num_gauss_quad_boundary*/, int /*num_gauss_quad_bulk*/,
                                                      bool enable_eliminate_zero_velocity_false_diffusion,
                                                      const std::string& /*integral_method*/,
                                                      int /*num_gauss_quadrature_points_on_one_triangle*/,
                                                      const std::string& interpolation_method, bool use_integral,
                                                      int num_gauss_quadrature_point_for_integrate_density,
                                                      bool /*enable_cell_volume_correction*/, R minimal_area) {
    fia_session* s = session_for(g);
    const fia_advect_params p = advect_params(FIA_SPLIT_XZ_CELLFACE, interpolation_method, use_integral,
                                              num_gauss_quadrature_point_for_integrate_density,
                                              enable_eliminate_zero_velocity_false_diffusion, use_MacCormack_scheme,
                                              false, (double)minimal_area);
    check(fia_advect_velocity_xyz_host(s, host_type<G>(), g.velocity_in_voxel_face_x.data(),
                                       g.velocity_in_voxel_face_y.data(), g.velocity_in_voxel_face_z.data(),
                                       (double)time_step_length, &p),
          "advect_velocity_xyz_flux_advection_3D_std_thread");
}

// calc_pressure_3D (calc_pressure_3d.cpp:18-181): the pressure of the grid's velocity, the
// last cell pinned to zero; the velocity is not changed.
template <class G>
void calc_pressure_3D(G& g) {
    fia_session* s = session_for(g);
    const int ht = host_type<G>();
    check(fia_set_field(s, FIA_FIELD_U, g.velocity_in_voxel_face_x.data(), ht), "calc_pressure_3D");
    check(fia_set_field(s, FIA_FIELD_V, g.velocity_in_voxel_face_y.data(), ht), "calc_pressure_3D");
    check(fia_set_field(s, FIA_FIELD_W, g.velocity_in_voxel_face_z.data(), ht), "calc_pressure_3D");
    const fia_solver_params sp = solver_params();
    fia_solver_report rep;
    check(fia_calc_pressure_3D(s, &sp, &rep), "calc_pressure_3D");
    check(fia_get_field(s, FIA_FIELD_PRESSURE, g.pressure.data(), ht), "calc_pressure_3D");
}

// calc_pressure_gradient_term_3D (calc_pressure_3d.cpp:183-270): solve, subtract the gradient
// on interior faces, and add this call's wall momentum losses to the grid's running totals.
template <class G>
void calc_pressure_gradient_term_3D(G& g) {
    fia_session* s = session_for(g);
    double before[3], after[3];
    check(fia_wall_momentum_loss(s, before), "calc_pressure_gradient_term_3D");
    const fia_solver_params sp = solver_params();
    fia_solver_report rep;
    check(fia_calc_pressure_gradient_term_3D_host(s, host_type<G>(), g.velocity_in_voxel_face_x.data(),
                                                  g.velocity_in_voxel_face_y.data(), g.velocity_in_voxel_face_z.data(),
                                                  g.pressure.data(), &sp, &rep),
          "calc_pressure_gradient_term_3D");
    check(fia_wall_momentum_loss(s, after), "calc_pressure_gradient_term_3D");
    using R = RealOf<G>;
    g.total_loss_of_momentum_x += (R)(after[0] - before[0]);
    g.total_loss_of_momentum_y += (R)(after[1] - before[1]);
    g.total_loss_of_momentum_z += (R)(after[2] - before[2]);
}

// update_fluid_velocity_3D (update_fluid_velocity_3d.cpp:88-193): frame 0 projects and then
// advects, later frames advect and then project; the body force is commented out in the
// reference (:109) and fix_velocity is not read there.
template <class G, class R>
void update_fluid_velocity_3D(G& g, int i_frame, R time_step_length, bool use_flux_advection,
                              bool use_MacCormack_scheme, bool use_clamping_in_MacCormack_scheme,
                              int num_gauss_quad_boundary, int num_gauss_quad_bulk,
                              bool enable_eliminate_zero_velocity_false_diffusion,
                              const std::string& /*split_method*/, const std::string& integral_method,
                              const std::string& interpolation_method, bool enable_cell_volume_correction,
                              bool /*fix_velocity*/, int num_gauss_quadrature_point_for_integrate_density,
                              bool use_integral, R minimal_area) {
    if (!use_flux_advection) fatal("update_fluid_velocity_3D", "the semi-Lagrangian branch is not part of the GPU path");
    auto advect = [&]() {
        advect_velocity_xyz_flux_advection_3D_std_thread(
            g, time_step_length, use_MacCormack_scheme, use_clamping_in_MacCormack_scheme, num_gauss_quad_boundary,
            num_gauss_quad_bulk, enable_eliminate_zero_velocity_false_diffusion, integral_method, num_gauss_quad_bulk,
            interpolation_method, use_integral, num_gauss_quadrature_point_for_integrate_density,
            enable_cell_volume_correction, minimal_area);
    };
    if (i_frame == 0) {
        calc_pressure_gradient_term_3D(g);
        advect();
    } else {
        advect();
        calc_pressure_gradient_term_3D(g);
    }
}

// calc_time_step_length_from_CFL_number_3D (calc_time_step_length_from_CFL_number.cpp:81-132):
// dt = CFL h / max|u| over all faces, shortened to end at the next movie frame (which then
// sets write_frame_to_movie_file).  The reduction runs on the device.
template <class G, class R>
R calc_time_step_length_from_CFL_number_3D(const G& g, R now_time, int i_movie_frame, bool& write_frame_to_movie_file,
                                           int CFL_number, R movie_fps) {
    fia_session* s = session_for(g);
    const int ht = host_type<G>();
    check(fia_set_field(s, FIA_FIELD_U, g.velocity_in_voxel_face_x.data(), ht), "calc_time_step_length_from_CFL_number_3D");
    check(fia_set_field(s, FIA_FIELD_V, g.velocity_in_voxel_face_y.data(), ht), "calc_time_step_length_from_CFL_number_3D");
    check(fia_set_field(s, FIA_FIELD_W, g.velocity_in_voxel_face_z.data(), ht), "calc_time_step_length_from_CFL_number_3D");
    double umax = 0.0;
    check(fia_max_abs_velocity(s, &umax), "calc_time_step_length_from_CFL_number_3D");
    const R from_cfl = (R)CFL_number * g._cell_length / (R)umax;
    const R next_frame = (R)(i_movie_frame + 1) / movie_fps;
    if (now_time + from_cfl > next_frame) {
        write_frame_to_movie_file = true;
        return next_frame - now_time;
    }
    write_frame_to_movie_file = false;
    return from_cfl;
}

}  // namespace fia_shim
