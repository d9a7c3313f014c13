"""Host-side mirror of the reference's 3D entry points over the C ABI of libfia.so.

The reference (nyhirasawa/Flux-Interpolated-Advection) is a C++ program; its hot path is
called as

    move_substances_3D(Grid_3D&, i_frame, dt, ...flags)            move_substances_3d.h:48-66
    advect_velocity_xyz_flux_advection_3D_std_thread(Grid_3D&, dt, ...)   advect_velocity_flux_advection_3d.h:107-124
    calc_pressure_3D(Grid_3D&) / calc_pressure_gradient_term_3D(Grid_3D&)  calc_pressure_3d.h:6-9

This module keeps those names and flag names; a `Grid3D` owns a device-resident session
(fia_create) with the Grid_3D arrays.  There is no CPU fallback: if libfia.so is not
built for this machine, or no GPU is present, the calls raise.
"""
import ctypes
import os
import platform
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libfia_%s.so" % platform.machine())
SOURCES = ["fia_api.cu", "fia_advect.cu", "fia_advect32.cu", "fia_pressure.cu", "fia_noalloc.cu", "fia_unet.cu"]
HEADERS = ["fia_device.cuh", "fia_advect.cuh", "fia_local.cuh", "fia_clip32.cuh", "fia_pressure.cuh", "fia_unet.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

FIA_OK, FIA_ERR_INVALID, FIA_ERR_CUDA, FIA_ERR_UNSUPPORTED, FIA_ERR_NOMEM = 0, -1, -2, -3, -4
FIA_FP64, FIA_FP32C = 0, 1
FIA_HOST_F64, FIA_HOST_F32 = 0, 1
FIELD = {"density": 0, "u": 1, "v": 2, "w": 3, "pressure": 4}
INTERP = {"WENO6": 0, "linear": 1}
SPLIT = {"xz-CellFaceAligned": 0, "xz-AxisAligned": 1, "x-CellFaceAligned_z-AxisAligned": 2,
         "x-AxisAligned_z-CellFaceAligned": 3}
STATUS_BITS = {1: "clip overflow", 2: "odd cut", 4: "non-finite flux", 8: "subdivision overflow",
               16: "solver cap", 32: "solver fallback"}


class FiaError(RuntimeError):
    pass


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def build(force=False, jobs=None):
    """Compile libfia for sm_103a into lib/ (in-tree).  Returns the library path."""
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(REPO, "include", "fia.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    objdir = os.path.join(HERE, "_build", platform.machine())
    os.makedirs(objdir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    flags = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(REPO, "include")]
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        procs.append(subprocess.Popen([nvcc] + flags + ["-c", s, "-o", o]))
    for p in procs:
        if p.wait() != 0:
            raise FiaError("nvcc failed building libfia")
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    """Load libfia (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = ctypes.CDLL(LIB)
        _declare(lib)
        _lib = lib
    return _lib


class AdvectParams(ctypes.Structure):
    """Flags of move_substances_3D (main.cpp:48-83), same names."""
    _fields_ = [("interpolation_method", ctypes.c_int), ("split_method", ctypes.c_int),
                ("num_gauss_quadrature_point_for_integrate_density", ctypes.c_int),
                ("use_integral", ctypes.c_int), ("enable_eliminate_zero_velocity_false_diffusion", ctypes.c_int),
                ("use_MacCormack_scheme", ctypes.c_int), ("enable_cell_volume_correction", ctypes.c_int),
                ("minimal_area", ctypes.c_double)]


class SolverParams(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iter", ctypes.c_int), ("method", ctypes.c_int),
                ("fallback_iter", ctypes.c_int)]


class SolverReport(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("rel_residual", ctypes.c_double), ("status", ctypes.c_int),
                ("fcg_iterations", ctypes.c_int), ("precond_ms", ctypes.c_double)]


class StepParams(ctypes.Structure):
    """fia_step_params: one smoke step (main.cpp:600-721 order) plus the plume harness."""
    _fields_ = [("advect", AdvectParams), ("solver", SolverParams), ("cfl", ctypes.c_double),
                ("max_dt", ctypes.c_double), ("buoyancy", ctypes.c_double), ("source", ctypes.c_int),
                ("source_center", ctypes.c_double * 3), ("source_radius", ctypes.c_double),
                ("source_density", ctypes.c_double), ("mass_correction", ctypes.c_int), ("frame", ctypes.c_int),
                ("capture_pair", ctypes.c_int), ("capture_tol", ctypes.c_double)]


class StepReport(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("max_velocity", ctypes.c_double),
                ("mass_before_advection", ctypes.c_double), ("mass_after_advection", ctypes.c_double),
                ("mass_after", ctypes.c_double), ("solver_iterations", ctypes.c_int),
                ("solver_rel_residual", ctypes.c_double), ("status", ctypes.c_int),
                ("solver_fcg_iterations", ctypes.c_int), ("precond_ms", ctypes.c_double)]


def _declare(lib):
    vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
    lib.fia_create.restype = vp
    lib.fia_create.argtypes = [ip, ip, ip, ctypes.c_double, ip]
    lib.fia_destroy.argtypes = [vp]
    lib.fia_error_string.restype = ctypes.c_char_p
    lib.fia_stream.restype = vp
    lib.fia_stream.argtypes = [vp]
    for name in ("fia_last_status", "fia_synchronize"):
        getattr(lib, name).argtypes = [vp]
    lib.fia_set_field.argtypes = [vp, ip, vp, ip]
    lib.fia_get_field.argtypes = [vp, ip, vp, ip]
    lib.fia_field_device_ptr.argtypes = [vp, ip, ctypes.POINTER(vp)]
    lib.fia_move_substances_3D.argtypes = [vp, ctypes.c_double, ctypes.POINTER(AdvectParams)]
    lib.fia_advect_velocity_xyz.argtypes = [vp, ctypes.c_double, ctypes.POINTER(AdvectParams)]
    lib.fia_calc_pressure_3D.argtypes = [vp, ctypes.POINTER(SolverParams), ctypes.POINTER(SolverReport)]
    lib.fia_calc_pressure_gradient_term_3D.argtypes = [vp, ctypes.POINTER(SolverParams), ctypes.POINTER(SolverReport)]
    lib.fia_max_abs_velocity.argtypes = [vp, dp]
    lib.fia_total_mass.argtypes = [vp, dp]
    lib.fia_wall_momentum_loss.argtypes = [vp, dp]
    lib.fia_total_momentum.argtypes = [vp, dp]
    lib.fia_write_density_frame.argtypes = [vp, ctypes.c_char_p, ip]
    lib.fia_append_totals.argtypes = [vp, ctypes.c_char_p, ctypes.c_double]
    lib.fia_pass_counters.argtypes = [vp, ctypes.POINTER(ctypes.c_ulonglong)]
    lib.fia_move_substances_3D_host.argtypes = [vp, ip, vp, vp, vp, vp, ctypes.c_double, ctypes.POINTER(AdvectParams)]
    lib.fia_advect_velocity_xyz_host.argtypes = [vp, ip, vp, vp, vp, ctypes.c_double, ctypes.POINTER(AdvectParams)]
    lib.fia_calc_pressure_gradient_term_3D_host.argtypes = [vp, ip, vp, vp, vp, vp, ctypes.POINTER(SolverParams),
                                                           ctypes.POINTER(SolverReport)]
    lib.fia_debug_flux_pass.argtypes = [vp, ip, dp, ctypes.c_double, ip, ip, ip, ip, dp, ip, ctypes.c_double, dp]
    lib.fia_debug_backtrace.argtypes = [vp, ip, ctypes.c_double, ip, dp]
    lib.fia_debug_psi.argtypes = [vp, ip, dp, ip, ip, dp]
    lib.fia_gauss_rule.argtypes = [ip, dp, dp]
    lib.fia_default_advect_params.argtypes = [ctypes.POINTER(AdvectParams)]
    lib.fia_default_solver_params.argtypes = [ctypes.POINTER(SolverParams)]
    lib.fia_default_step_params.argtypes = [ctypes.POINTER(StepParams)]
    lib.fia_profile_faces.argtypes = [vp, ip]
    lib.fia_profile_faces_read.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_int)]
    lib.fia_step.argtypes = [vp, ctypes.POINTER(StepParams), ctypes.POINTER(StepReport)]
    fp = ctypes.POINTER(ctypes.c_float)
    lib.fia_set_solid_spheres.argtypes = [vp, ip, dp, dp]
    lib.fia_get_solid_mask.argtypes = [vp, vp]
    lib.fia_learned_num_parameters.restype = ctypes.c_longlong
    lib.fia_learned_num_parameters.argtypes = []
    lib.fia_learned_init.argtypes = [vp, ctypes.c_ulonglong]
    lib.fia_learned_set_weights.argtypes = [vp, fp, ctypes.c_longlong]
    lib.fia_learned_get_weights.argtypes = [vp, fp, ctypes.c_longlong]
    lib.fia_learned_add_pair.argtypes = [vp, fp, fp]
    lib.fia_learned_num_pairs.argtypes = [vp]
    lib.fia_learned_loss.argtypes = [vp, ip, dp]
    lib.fia_learned_calibrate.argtypes = [vp, ip]
    lib.fia_learned_train_step.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ip, ctypes.c_double, dp]
    lib.fia_learned_level_dims.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int)]
    lib.fia_debug_unet_forward.argtypes = [vp, fp, fp]
    lib.fia_debug_unet_backward.argtypes = [vp, fp, fp, fp]
    lib.fia_debug_precondition.argtypes = [vp, fp, fp]
    lib.fia_debug_learned_tc.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_uint)]
    lib.fia_debug_clip_fast.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_ulonglong)]
    lib.fia_debug_full_weno.argtypes = [vp, ip]
    lib.fia_debug_piece_pipeline.argtypes = [vp, ip]
    lib.fia_debug_vertex_jitter.argtypes = [vp, ctypes.c_double]
    lib.fia_debug_learned_grad.argtypes = [vp, ip, fp, dp]
    lib.fia_debug_grid_op.argtypes = [vp, ip, fp, fp]
    lib.fia_debug_solve_rhs.argtypes = [vp, fp, fp, ctypes.POINTER(SolverParams), ctypes.POINTER(SolverReport)]
    lib.fia_debug_set_piece_capacity.argtypes = [vp, ctypes.c_longlong]
    lib.fia_debug_piece_capacity.argtypes = [vp]
    lib.fia_debug_piece_capacity.restype = ctypes.c_longlong


def _check(rc, what):
    if rc < 0:
        raise FiaError("%s failed: %s" % (what, load().fia_error_string(rc).decode()))
    return rc


def advect_params(interpolation_method="WENO6", split_method="xz-CellFaceAligned",
                  num_gauss_quadrature_point_for_integrate_density=3, use_integral=True,
                  enable_eliminate_zero_velocity_false_diffusion=True, use_MacCormack_scheme=False,
                  enable_cell_volume_correction=False, minimal_area=1.0):
    p = AdvectParams()
    p.interpolation_method = INTERP[interpolation_method]
    p.split_method = SPLIT[split_method]
    p.num_gauss_quadrature_point_for_integrate_density = num_gauss_quadrature_point_for_integrate_density
    p.use_integral = int(bool(use_integral))
    p.enable_eliminate_zero_velocity_false_diffusion = int(bool(enable_eliminate_zero_velocity_false_diffusion))
    p.use_MacCormack_scheme = int(bool(use_MacCormack_scheme))
    p.enable_cell_volume_correction = int(bool(enable_cell_volume_correction))
    p.minimal_area = minimal_area
    return p


FIA_SOLVER_PCG_JACOBI, FIA_SOLVER_FCG_LEARNED = 0, 1
FIA_STATUS_SOLVER_CAP, FIA_STATUS_SOLVER_FALLBACK = 16, 32


def solver_params(tol=1e-6, max_iter=10000, method=0, fallback_iter=200):
    p = SolverParams()
    p.tol, p.max_iter, p.method, p.fallback_iter = tol, max_iter, method, fallback_iter
    return p


def step_params(**kw):
    """Defaults of fia_default_step_params (the plume), overridden by keyword."""
    p = StepParams()
    load().fia_default_step_params(ctypes.byref(p))
    for k, v in kw.items():
        if k == "advect" and isinstance(v, dict):
            p.advect = advect_params(**v)
        elif k == "solver" and isinstance(v, dict):
            p.solver = solver_params(**v)
        elif k == "source_center":
            p.source_center = (ctypes.c_double * 3)(*v)
        else:
            setattr(p, k, v)
    return p


def gauss_rule(k):
    """(nodes, weights) of the library's Gauss rule for k points per half cell (host only)"""
    x, w = np.zeros(k), np.zeros(k)
    _check(load().fia_gauss_rule(k, _dp(x), _dp(w)), "fia_gauss_rule")
    return x, w


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def num_learned_parameters():
    return int(load().fia_learned_num_parameters())


class Grid3D:
    """Device-resident Grid_3D (grid_3d.h:14-88): nx*ny*nz cells of length cell_length."""

    def __init__(self, nx, ny, nz, cell_length, precision=FIA_FP64):
        self.lib = load()
        self.N = (nx, ny, nz)
        self.h = cell_length
        self.precision = precision
        self.s = self.lib.fia_create(nx, ny, nz, ctypes.c_double(cell_length), precision)
        if not self.s:
            raise FiaError("fia_create failed: " + self.lib.fia_error_string(FIA_ERR_CUDA).decode())

    def close(self):
        if self.s:
            self.lib.fia_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sizes(self):
        nx, ny, nz = self.N
        return {"density": nx * ny * nz, "pressure": nx * ny * nz, "u": (nx + 1) * ny * nz,
                "v": nx * (ny + 1) * nz, "w": nx * ny * (nz + 1)}

    # ---- field access ----
    def set(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        if a.size != self.sizes()[name]:
            raise FiaError("field %s: expected %d values, got %d" % (name, self.sizes()[name], a.size))
        _check(self.lib.fia_set_field(self.s, FIELD[name], a.ctypes.data, FIA_HOST_F64), "fia_set_field")

    def get(self, name):
        a = np.empty(self.sizes()[name], dtype=np.float64)
        _check(self.lib.fia_get_field(self.s, FIELD[name], a.ctypes.data, FIA_HOST_F64), "fia_get_field")
        return a

    def device_ptr(self, name):
        p = ctypes.c_void_p()
        _check(self.lib.fia_field_device_ptr(self.s, FIELD[name], ctypes.byref(p)), "fia_field_device_ptr")
        return p.value

    def stream(self):
        return self.lib.fia_stream(self.s)

    def synchronize(self):
        _check(self.lib.fia_synchronize(self.s), "fia_synchronize")

    def last_status(self):
        return _check(self.lib.fia_last_status(self.s), "fia_last_status")

    # ---- the reference's entry points ----
    def move_substances_3D(self, time_step_length, params=None):
        p = params or advect_params()
        return _check(self.lib.fia_move_substances_3D(self.s, ctypes.c_double(time_step_length), ctypes.byref(p)),
                      "move_substances_3D")

    def advect_velocity_xyz_flux_advection_3D(self, time_step_length, params=None):
        p = params or advect_params()
        return _check(self.lib.fia_advect_velocity_xyz(self.s, ctypes.c_double(time_step_length), ctypes.byref(p)),
                      "advect_velocity_xyz_flux_advection_3D")

    def calc_pressure_3D(self, sp=None):
        rep = SolverReport()
        _check(self.lib.fia_calc_pressure_3D(self.s, ctypes.byref(sp or solver_params()), ctypes.byref(rep)),
               "calc_pressure_3D")
        return rep

    def calc_pressure_gradient_term_3D(self, sp=None):
        rep = SolverReport()
        _check(self.lib.fia_calc_pressure_gradient_term_3D(self.s, ctypes.byref(sp or solver_params()),
                                                           ctypes.byref(rep)), "calc_pressure_gradient_term_3D")
        return rep

    def step(self, params=None):
        """One smoke step (fia_step); returns the StepReport."""
        rep = StepReport()
        _check(self.lib.fia_step(self.s, ctypes.byref(params or step_params()), ctypes.byref(rep)), "fia_step")
        return rep

    def profile_faces(self, capacity):
        """Start timing each face-kernel launch with CUDA events (see read_face_profile)."""
        _check(self.lib.fia_profile_faces(self.s, capacity), "fia_profile_faces")

    def read_face_profile(self):
        """(summed device ms, number of face-kernel launches) since profile_faces."""
        ms = ctypes.c_double(0); n = ctypes.c_int(0)
        _check(self.lib.fia_profile_faces_read(self.s, ctypes.byref(ms), ctypes.byref(n)), "fia_profile_faces_read")
        return ms.value, n.value

    def max_abs_velocity(self):
        out = ctypes.c_double(0)
        _check(self.lib.fia_max_abs_velocity(self.s, ctypes.byref(out)), "fia_max_abs_velocity")
        return out.value

    def total_mass(self):
        out = ctypes.c_double(0)
        _check(self.lib.fia_total_mass(self.s, ctypes.byref(out)), "fia_total_mass")
        return out.value

    def wall_momentum_loss(self):
        out = (ctypes.c_double * 3)()
        _check(self.lib.fia_wall_momentum_loss(self.s, out), "fia_wall_momentum_loss")
        return tuple(out)

    def total_momentum(self):
        out = (ctypes.c_double * 3)()
        _check(self.lib.fia_total_momentum(self.s, out), "fia_total_momentum")
        return tuple(out)

    # ---- frame output (main.cpp:515-654) ----
    def write_density_frame(self, path, frame):
        """dense density frame (header + float32, see read_density_frame)"""
        _check(self.lib.fia_write_density_frame(self.s, os.fsencode(path), int(frame)), "fia_write_density_frame")

    def append_totals(self, prefix, now_time):
        """one line per log: total mass, momenta, wall momentum losses and their sums"""
        _check(self.lib.fia_append_totals(self.s, os.fsencode(prefix), ctypes.c_double(now_time)), "fia_append_totals")

    def pass_counters(self):
        """Cumulative (faces, pieces, faces clipped from both sides, FP32 point
        interpolations, kernel launches) since the session was created."""
        out = (ctypes.c_ulonglong * 5)()
        _check(self.lib.fia_pass_counters(self.s, out), "fia_pass_counters")
        return tuple(int(x) for x in out)

    # ---- solids ----
    def set_solid_spheres(self, centers, radii):
        """Solid spheres (physical centres, radii); an empty list removes them."""
        c = np.ascontiguousarray(centers, dtype=np.float64).reshape(-1)
        r = np.ascontiguousarray(radii, dtype=np.float64).reshape(-1)
        if c.size != 3 * r.size:
            raise FiaError("set_solid_spheres: %d centre values for %d radii" % (c.size, r.size))
        _check(self.lib.fia_set_solid_spheres(self.s, r.size, _dp(c), _dp(r)), "fia_set_solid_spheres")

    def solid_mask(self):
        m = np.empty(self.sizes()["density"], dtype=np.uint8)
        _check(self.lib.fia_get_solid_mask(self.s, m.ctypes.data), "fia_get_solid_mask")
        return m

    # ---- learned preconditioner ----
    def learned_init(self, seed=1):
        _check(self.lib.fia_learned_init(self.s, seed), "fia_learned_init")

    def learned_set_weights(self, w):
        a = np.ascontiguousarray(w, dtype=np.float32)
        _check(self.lib.fia_learned_set_weights(self.s, _fp(a), a.size), "fia_learned_set_weights")

    def learned_get_weights(self):
        a = np.empty(num_learned_parameters(), dtype=np.float32)
        _check(self.lib.fia_learned_get_weights(self.s, _fp(a), a.size), "fia_learned_get_weights")
        return a

    def learned_add_pair(self, r, p):
        a = np.ascontiguousarray(r, dtype=np.float32)
        b = np.ascontiguousarray(p, dtype=np.float32)
        _check(self.lib.fia_learned_add_pair(self.s, _fp(a), _fp(b)), "fia_learned_add_pair")

    def learned_num_pairs(self):
        return self.lib.fia_learned_num_pairs(self.s)

    def learned_loss(self, pair):
        out = ctypes.c_double(0)
        _check(self.lib.fia_learned_loss(self.s, pair, ctypes.byref(out)), "fia_learned_loss")
        return out.value

    def learned_calibrate(self, pair=0):
        _check(self.lib.fia_learned_calibrate(self.s, pair), "fia_learned_calibrate")

    def learned_train_step(self, pairs, lr):
        idx = (ctypes.c_int * len(pairs))(*[int(i) for i in pairs])
        losses = np.zeros(len(pairs))
        _check(self.lib.fia_learned_train_step(self.s, idx, len(pairs), ctypes.c_double(lr), _dp(losses)),
               "fia_learned_train_step")
        return losses

    def learned_level_dims(self, level):
        d = (ctypes.c_int * 3)()
        _check(self.lib.fia_learned_level_dims(self.s, level, d), "fia_learned_level_dims")
        return tuple(d)

    def debug_unet_forward(self, x0):
        a = np.ascontiguousarray(x0, dtype=np.float32).ravel()
        y = np.empty_like(a)
        _check(self.lib.fia_debug_unet_forward(self.s, _fp(a), _fp(y)), "fia_debug_unet_forward")
        return y

    def debug_unet_backward(self, x0, gy):
        a = np.ascontiguousarray(x0, dtype=np.float32).ravel()
        g = np.ascontiguousarray(gy, dtype=np.float32).ravel()
        out = np.empty(num_learned_parameters(), dtype=np.float32)
        _check(self.lib.fia_debug_unet_backward(self.s, _fp(a), _fp(g), _fp(out)), "fia_debug_unet_backward")
        return out

    def debug_solve_rhs(self, rhs, sp):
        """x with B x = rhs (B = -A), FP32 sessions; returns (x, SolverReport)"""
        a = np.ascontiguousarray(rhs, dtype=np.float32).ravel()
        x = np.empty_like(a)
        rep = SolverReport()
        _check(self.lib.fia_debug_solve_rhs(self.s, _fp(a), _fp(x), ctypes.byref(sp), ctypes.byref(rep)),
               "fia_debug_solve_rhs")
        return x, rep

    def debug_set_piece_capacity(self, pieces):
        _check(self.lib.fia_debug_set_piece_capacity(self.s, pieces), "fia_debug_set_piece_capacity")

    def debug_piece_capacity(self):
        return int(self.lib.fia_debug_piece_capacity(self.s))

    def debug_grid_op(self, op, values):
        """restriction (0), prolongation (1) or its adjoint (2) of the learned preconditioner"""
        a = np.ascontiguousarray(values, dtype=np.float32).ravel()
        d0 = self.learned_level_dims(0)
        out = np.empty(int(np.prod(self.N)) if op == 1 else int(np.prod(d0)), dtype=np.float32)
        _check(self.lib.fia_debug_grid_op(self.s, op, _fp(a), _fp(out)), "fia_debug_grid_op")
        return out

    def debug_learned_grad(self, pair):
        out = np.empty(num_learned_parameters(), dtype=np.float32)
        loss = ctypes.c_double(0)
        _check(self.lib.fia_debug_learned_grad(self.s, pair, _fp(out), ctypes.byref(loss)), "fia_debug_learned_grad")
        return out, loss.value

    def debug_learned_tc(self, enable=-1):
        """switch the network's tcgen05 convolution path (1 on, 0 off, -1 leave); returns its
        error bits"""
        st = ctypes.c_uint(0)
        _check(self.lib.fia_debug_learned_tc(self.s, enable, ctypes.byref(st)), "fia_debug_learned_tc")
        return st.value

    def debug_clip_fast(self, enable=-1):
        """switch the face clipper's shared-memory path (1 on, 0 off, -1 leave); returns the
        number of faces the local-memory clipper took so far"""
        n = ctypes.c_ulonglong(0)
        _check(self.lib.fia_debug_clip_fast(self.s, enable, ctypes.byref(n)), "fia_debug_clip_fast")
        return n.value

    def debug_full_weno(self, enable=-1):
        """FP64 form: 1 evaluates every WENO6 in full, 0 collapses it on node planes (default),
        -1 leaves it; returns the setting"""
        return _check(self.lib.fia_debug_full_weno(self.s, enable), "fia_debug_full_weno")

    def debug_piece_pipeline(self, enable=-1):
        """FP64 form: 1 runs the faces as the piece pipeline (default), 0 as one thread per face,
        -1 leaves it; returns the setting"""
        return _check(self.lib.fia_debug_piece_pipeline(self.s, enable), "fia_debug_piece_pipeline")

    def debug_vertex_jitter(self, cells):
        """FP64 form: move every backtraced vertex by up to `cells` cells per axis (independent,
        hashed, per pass); 0 switches it off"""
        _check(self.lib.fia_debug_vertex_jitter(self.s, ctypes.c_double(cells)), "fia_debug_vertex_jitter")

    def debug_precondition(self, r):
        a = np.ascontiguousarray(r, dtype=np.float32).ravel()
        z = np.empty_like(a)
        _check(self.lib.fia_debug_precondition(self.s, _fp(a), _fp(z)), "fia_debug_precondition")
        return z

    # ---- test hooks ----
    def debug_flux_pass(self, comp, field, dt, interp, psi_mode, use_integral, zero_velocity, color_off, k,
                        minimal_area=1.0):
        f = np.ascontiguousarray(field, dtype=np.float64)
        out = np.zeros(f.size)
        co = np.array(color_off, dtype=np.float64)
        st = _check(self.lib.fia_debug_flux_pass(self.s, comp, _dp(f), ctypes.c_double(dt), interp, psi_mode,
                                                 use_integral, zero_velocity, _dp(co), k,
                                                 ctypes.c_double(minimal_area), _dp(out)), "fia_debug_flux_pass")
        return out, st

    def debug_backtrace(self, comp, dt, interp):
        L = [self.N[d] + 1 + (d == comp) for d in range(3)]
        out = np.zeros(L[0] * L[1] * L[2] * 3)
        _check(self.lib.fia_debug_backtrace(self.s, comp, ctypes.c_double(dt), interp, _dp(out)), "fia_debug_backtrace")
        return out.reshape(L[0], L[1], L[2], 3)

    def debug_psi(self, comp, field, mode, k):
        f = np.ascontiguousarray(field, dtype=np.float64)
        M = [self.N[d] + (d == comp) for d in range(3)]
        out = np.zeros(M[0] * (M[1] + 1) * M[2])
        _check(self.lib.fia_debug_psi(self.s, comp, _dp(f), mode, k, _dp(out)), "fia_debug_psi")
        return out


def read_density_frame(path):
    """(density array (nx, ny, nz) float32, header dict) of a frame written by
    Grid3D.write_density_frame / fia_write_density_frame"""
    raw = open(path, "rb").read()
    if raw[:8] != b"FIAFRM1\0":
        raise FiaError("%s: not a density frame" % path)
    nx, ny, nz, frame = np.frombuffer(raw[8:24], dtype="<i4")
    origin = np.frombuffer(raw[24:48], dtype="<f8")
    voxel = float(np.frombuffer(raw[48:56], dtype="<f8")[0])
    data = np.frombuffer(raw[64:], dtype="<f4").reshape(int(nx), int(ny), int(nz))
    return data, {"frame": int(frame), "origin": tuple(float(x) for x in origin), "voxel_size": voxel}
