"""ctypes loader for the CPU oracle (oracle/fia_oracle.cpp) and, where it was built,
the reference build (oracle/_ref/libfia_ref_{float,double}.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline / reference legs.  The product library never imports this module.
"""
import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SRC = os.path.join(HERE, "fia_oracle.cpp")
ORACLE_DEPS = [ORACLE_SRC, os.path.join(HERE, "cpu_stream.inl")]
ORACLE_SO = os.path.join(HERE, "_build", "liboracle_%s.so" % platform.machine())
REF_DIR = os.path.join(HERE, "_ref")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def build_oracle(force=False):
    """Compile the oracle for this host (x86-64 here, aarch64 on the GPU host)."""
    if not force and os.path.exists(ORACLE_SO) and os.path.getmtime(ORACLE_SO) >= max(map(os.path.getmtime,
                                                                                         ORACLE_DEPS)):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17",
                           "-o", tmp, ORACLE_SRC, "-lpthread"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_reference():
    """Compile oracle/_ref from the reference checkout (only where it is present)."""
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")])


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """Thin wrapper over the oracle's C entry points (all arrays float64, z fastest)."""

    def __init__(self):
        self.lib = ctypes.CDLL(build_oracle())
        L = self.lib
        L.fo_interp.restype = ctypes.c_int
        L.fo_max_abs_velocity.restype = ctypes.c_double

    # ---- pieces ----
    def gauss(self, k):
        x = np.zeros(k); w = np.zeros(k)
        assert self.lib.fo_gauss(k, _ptr(x), _ptr(w)) == 0
        return x, w

    def interp(self, a, M, off, h, method, pts):
        a = _f64(a); pts = _f64(pts).reshape(-1, 3)
        out = np.zeros(len(pts))
        Mi = (ctypes.c_int * 3)(*M); Of = (ctypes.c_double * 3)(*off)
        self.lib.fo_interp(_ptr(a), Mi, Of, ctypes.c_double(h), method, _ptr(pts), ctypes.c_long(len(pts)), _ptr(out))
        return out

    def psi(self, a, M, off, h, mode, k):
        a = _f64(a)
        out = np.zeros(M[0] * (M[1] + 1) * M[2])
        Mi = (ctypes.c_int * 3)(*M); Of = (ctypes.c_double * 3)(*off)
        self.lib.fo_psi(_ptr(a), Mi, Of, ctypes.c_double(h), mode, k, _ptr(out))
        return out

    def split_face(self, verts, h, color_off, minimal_area=1.0, max_out=256):
        v = _f64(verts).reshape(12)
        out = np.zeros(6 * max_out); n = ctypes.c_int(0)
        co = (ctypes.c_double * 2)(*color_off)
        st = self.lib.fo_split_face(_ptr(v), ctypes.c_double(h), co, ctypes.c_double(minimal_area), max_out,
                                    _ptr(out), ctypes.byref(n))
        return out[:6 * min(n.value, max_out)].reshape(-1, 6), st

    def backtrace_vertices(self, N, h, u, v, w, dt, comp, interp):
        u, v, w = _f64(u), _f64(v), _f64(w)
        L = [N[d] + 1 + (d == comp) for d in range(3)]
        out = np.zeros(L[0] * L[1] * L[2] * 3)
        self.lib.fo_backtrace_vertices(N[0], N[1], N[2], ctypes.c_double(h), _ptr(u), _ptr(v), _ptr(w),
                                       ctypes.c_double(dt), comp, interp, _ptr(out))
        return out.reshape(L[0], L[1], L[2], 3)

    def flux_pass(self, N, h, u, v, w, comp, field, dt, interp, psi_mode, use_integral, zero_velocity,
                  color_off, k, minimal_area=1.0, nthreads=1, c0=0, c1=-1, maccormack=0):
        u, v, w, field = _f64(u), _f64(v), _f64(w), _f64(field)
        out = np.zeros(field.size)
        co = (ctypes.c_double * 2)(*color_off)
        nf = ctypes.c_long(0); npoly = ctypes.c_long(0)
        st = self.lib.fo_flux_pass(N[0], N[1], N[2], ctypes.c_double(h), _ptr(u), _ptr(v), _ptr(w), comp,
                                   _ptr(field), ctypes.c_double(dt), interp, psi_mode, use_integral,
                                   zero_velocity, co, k, ctypes.c_double(minimal_area), nthreads,
                                   ctypes.c_long(c0), ctypes.c_long(c1), _ptr(out), ctypes.byref(nf),
                                   ctypes.byref(npoly), int(maccormack))
        return out, st, nf.value, npoly.value

    # ---- reference entry points ----
    def move_substances_3D(self, N, h, u, v, w, rho, dt, interp=0, k=3, correction=1, use_integral=1,
                           split_off=(0.5, 0.5), minimal_area=1.0, nthreads=1, maccormack=0, volume_correction=0):
        u, v, w = _f64(u), _f64(v), _f64(w)
        r = _f64(rho).copy()
        so = (ctypes.c_double * 2)(*split_off)
        st = self.lib.fo_move_substances_3D(N[0], N[1], N[2], ctypes.c_double(h), _ptr(u), _ptr(v), _ptr(w),
                                            _ptr(r), ctypes.c_double(dt), interp, k, correction, use_integral,
                                            so, ctypes.c_double(minimal_area), nthreads, int(maccormack),
                                            int(volume_correction))
        return r, st

    def move_substances_slab(self, N, h, u, v, w, rho, dt, x0, x1, margin, interp=0, k=3, correction=1,
                             use_integral=1, split_off=(0.5, 0.5), minimal_area=1.0, nthreads=1, out=None):
        """move_substances_3D on the cells of the x-slab [x0, x1) (the CPU baseline's work unit);
        returns (out, status, faces visited) with only the slab's cells of out written"""
        u, v, w, rho = _f64(u), _f64(v), _f64(w), _f64(rho)
        if out is None:
            out = np.zeros(rho.size)
        so = (ctypes.c_double * 2)(*split_off)
        nf = ctypes.c_long(0)
        st = self.lib.fo_move_substances_slab(N[0], N[1], N[2], ctypes.c_double(h), _ptr(u), _ptr(v), _ptr(w),
                                              _ptr(rho), ctypes.c_double(dt), interp, k, correction, use_integral, so,
                                              ctypes.c_double(minimal_area), nthreads, x0, x1, margin, _ptr(out),
                                              ctypes.byref(nf))
        return out, st, nf.value

    def stream_move_substances_slab(self, N, h, u, v, w, rho, dt, x0, x1, margin, interp=0, k=3, correction=1,
                                    use_integral=1, split_off=(0.5, 0.5), minimal_area=1.0, nthreads=1, out=None):
        """the streaming-tile CPU baseline (oracle/cpu_stream.inl) on the x-slab [x0, x1), the same
        interface as move_substances_slab"""
        u, v, w, rho = _f64(u), _f64(v), _f64(w), _f64(rho)
        if out is None:
            out = np.zeros(rho.size)
        so = (ctypes.c_double * 2)(*split_off)
        nf = ctypes.c_long(0)
        st = self.lib.fo_stream_move_substances_slab(N[0], N[1], N[2], ctypes.c_double(h), _ptr(u), _ptr(v), _ptr(w),
                                                     _ptr(rho), ctypes.c_double(dt), interp, k, correction,
                                                     use_integral, so, ctypes.c_double(minimal_area), nthreads, x0, x1,
                                                     margin, _ptr(out), ctypes.byref(nf))
        return out, st, nf.value

    def cell_volumes(self, N, h, u, v, w, dt, interp=0, k=3, use_integral=1, split_off=(0.5, 0.5), minimal_area=1.0,
                     nthreads=1, maccormack=0):
        """advected cell volumes of the density's main pass (sum of y n_y of the pieces)"""
        u, v, w = _f64(u), _f64(v), _f64(w)
        out = np.zeros(N[0] * N[1] * N[2])
        so = (ctypes.c_double * 2)(*split_off)
        st = self.lib.fo_cell_volumes(N[0], N[1], N[2], ctypes.c_double(h), _ptr(u), _ptr(v), _ptr(w),
                                      ctypes.c_double(dt), interp, k, use_integral, so, ctypes.c_double(minimal_area),
                                      nthreads, int(maccormack), _ptr(out))
        return out, st

    def advect_velocity_3D(self, N, h, u, v, w, dt, interp=0, k=3, correction=1, use_integral=1,
                           minimal_area=1.0, nthreads=1, maccormack=0):
        u, v, w = _f64(u).copy(), _f64(v).copy(), _f64(w).copy()
        st = self.lib.fo_advect_velocity_3D(N[0], N[1], N[2], ctypes.c_double(h), _ptr(u), _ptr(v), _ptr(w),
                                            ctypes.c_double(dt), interp, k, correction, use_integral,
                                            ctypes.c_double(minimal_area), nthreads, int(maccormack))
        return u, v, w, st

    def pressure_rhs(self, N, h, u, v, w):
        b = np.zeros(N[0] * N[1] * N[2])
        self.lib.fo_pressure_rhs(N[0], N[1], N[2], ctypes.c_double(h), _ptr(_f64(u)), _ptr(_f64(v)),
                                 _ptr(_f64(w)), _ptr(b))
        return b

    def apply_laplacian(self, N, p):
        p = _f64(p); out = np.zeros_like(p)
        self.lib.fo_apply_laplacian(N[0], N[1], N[2], _ptr(p), _ptr(out))
        return out

    def pressure_solve(self, N, b, tol=1e-12, maxit=100000):
        b = _f64(b); p = np.zeros_like(b); rr = ctypes.c_double(0)
        it = self.lib.fo_pressure_solve(N[0], N[1], N[2], _ptr(b), _ptr(p), ctypes.c_double(tol), maxit,
                                        ctypes.byref(rr))
        return p, it, rr.value

    def subtract_gradient(self, N, h, p, u, v, w):
        u, v, w = _f64(u).copy(), _f64(v).copy(), _f64(w).copy()
        self.lib.fo_subtract_gradient(N[0], N[1], N[2], ctypes.c_double(h), _ptr(_f64(p)), _ptr(u), _ptr(v), _ptr(w))
        return u, v, w

    def max_abs_velocity(self, N, u, v, w):
        return self.lib.fo_max_abs_velocity(N[0], N[1], N[2], _ptr(_f64(u)), _ptr(_f64(v)), _ptr(_f64(w)))


class Reference:
    """The reference's own translation units (oracle/_ref), float or double scalars."""

    def __init__(self, precision="double"):
        path = os.path.join(REF_DIR, "libfia_ref_%s.so" % precision)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        self.scalar_bytes = self.lib.fr_scalar_bytes()

    def interp(self, kind, a, N, h, pts):
        a = _f64(a); pts = _f64(pts).reshape(-1, 3); out = np.zeros(len(pts))
        self.lib.fr_interp(kind, _ptr(a), N[0], N[1], N[2], ctypes.c_double(h), _ptr(pts), ctypes.c_long(len(pts)), _ptr(out))
        return out

    def psi_density(self, rho, N, h, interp, k, use_integral):
        out = np.zeros(N[0] * (N[1] + 1) * N[2])
        self.lib.fr_psi_density(_ptr(_f64(rho)), N[0], N[1], N[2], ctypes.c_double(h), interp, k, use_integral, _ptr(out))
        return out

    def split_face(self, verts, h, split, minimal_area=1.0, max_out=256):
        v = _f64(verts).reshape(12); out = np.zeros(6 * max_out); n = ctypes.c_int(0)
        self.lib.fr_split_face(_ptr(v), ctypes.c_double(h), split, ctypes.c_double(minimal_area), max_out, _ptr(out), ctypes.byref(n))
        return out[:6 * min(n.value, max_out)].reshape(-1, 6)

    def density_pass(self, N, h, u, v, w, rho, dt, interp, psi, use_integral, zero_vel, split, k, minimal_area=1.0,
                     maccormack=0):
        out = np.zeros(N[0] * N[1] * N[2])
        self.lib.fr_density_pass(N[0], N[1], N[2], ctypes.c_double(h), _ptr(_f64(u)), _ptr(_f64(v)), _ptr(_f64(w)),
                                 _ptr(_f64(rho)), ctypes.c_double(dt), interp, psi, use_integral, zero_vel, split, k,
                                 ctypes.c_double(minimal_area), _ptr(out), int(maccormack))
        return out

    def move_substances_3D(self, N, h, u, v, w, rho, dt, interp=0, split=0, k=3, correction=1, use_integral=1,
                           minimal_area=1.0, maccormack=0):
        r = _f64(rho).copy()
        self.lib.fr_move_substances_3D(N[0], N[1], N[2], ctypes.c_double(h), _ptr(_f64(u)), _ptr(_f64(v)), _ptr(_f64(w)),
                                       _ptr(r), ctypes.c_double(dt), interp, split, k, correction, use_integral,
                                       ctypes.c_double(minimal_area), int(maccormack))
        return r

    def cell_volumes(self, N, h, u, v, w, dt, interp=0, split=0, k=3, minimal_area=1.0, maccormack=0):
        """advected cell volumes of the density's main pass (integral branch) from the reference's
        own volume points and calc_cell_volumes_from_quadrature_point_list"""
        out = np.zeros(N[0] * N[1] * N[2])
        self.lib.fr_cell_volumes(N[0], N[1], N[2], ctypes.c_double(h), _ptr(_f64(u)), _ptr(_f64(v)), _ptr(_f64(w)),
                                 ctypes.c_double(dt), interp, split, k, ctypes.c_double(minimal_area), int(maccormack),
                                 _ptr(out))
        return out

    def velocity_pass_linear(self, N, h, u, v, w, dim, dt, k, minimal_area=1.0):
        sizes = [(N[0] + 1) * N[1] * N[2], N[0] * (N[1] + 1) * N[2], N[0] * N[1] * (N[2] + 1)]
        out = np.zeros(sizes[dim])
        self.lib.fr_velocity_pass_linear(N[0], N[1], N[2], ctypes.c_double(h), _ptr(_f64(u)), _ptr(_f64(v)), _ptr(_f64(w)),
                                         dim, ctypes.c_double(dt), k, ctypes.c_double(minimal_area), _ptr(out))
        return out
