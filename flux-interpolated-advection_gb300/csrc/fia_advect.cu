// fia_advect.cu -- the flux-interpolated advection pass on the GPU.
//
// One pass of the reference (advect_density_flux_advection_3D_std_thread,
// move_substances_3d.cpp:585-841, and its velocity counterpart
// advect_velocity_flux_advection_3d.cpp:252-576) becomes four kernels:
//
//   k_psi        one thread per (x,z) column: psi = running y-integral of the field
//                (calc_psi_3D.cpp:10-308, :311-537)
//   k_backtrace  one thread per UNIQUE cell vertex: x' = x - dt u(x), pin rule, clamp
//                (calc_backtraced_face_3D.cpp:9-160).  The reference backtraces every
//                vertex once per face that uses it (up to 24 times).
//   k_faces      one thread per UNIQUE face: clip the backtraced face in (xi,eta) space
//                at the integer iso-lines of its vertex colours (facecutter.h:59-324,
//                split_face_3D.cpp:17-93), and for every piece evaluate the quadrature
//                of polygon_3D.cpp:257-487 with WENO6 / linear interpolation; the face
//                flux is accumulated in registers.  The reference computes each interior
//                face twice (once per adjacent cell, with reversed vertex order); the two
//                computations produce the same pieces with opposite normals, so one
//                signed flux per face is exact.
//   k_gather     one thread per cell: rho' = (sum of the six signed face fluxes) / V.
//                Deterministic, no atomics (the reference's per-thread += is racy).
#include "fia_advect.cuh"

#include <cmath>
#include <vector>
#include <algorithm>

namespace fia {

// ------------------------------------------------------------------------------------
// host helpers
// ------------------------------------------------------------------------------------
static void legendre(int n, double x, double* p, double* dp) {
    double p0 = 1.0, p1 = x;
    for (int m = 2; m <= n; ++m) {
        double p2 = ((2.0 * m - 1.0) * x * p1 - (m - 1.0) * p0) / m;
        p0 = p1; p1 = p2;
    }
    if (n == 0) { *p = 1.0; *dp = 0.0; return; }
    *p = p1;
    *dp = n * (x * p1 - p0) / (x * x - 1.0);
}

// Gauss-Legendre rule on [-1,1]: Newton iteration on P_k from Chebyshev-like starting
// points; nodes ordered centre first then -/+ pairs by increasing |x| (the order of
// gauss_quadrature_points.cpp:18-60); weights normalised to sum 1.  Fixed arrays only (no
// heap), so the allocation-free entry point shares it.
void make_gauss(int k, double* x, double* w) {
    const double pi = 3.14159265358979323846;
    double nx[kMaxGauss + 1], nw[kMaxGauss + 1];
    int n = 0;
    for (int i = 0; i < (k + 1) / 2; ++i) {
        double z = std::cos(pi * (i + 0.75) / (k + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p, dp; legendre(k, z, &p, &dp);
            double dz = p / dp; z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        double p, dp; legendre(k, z, &p, &dp);
        double wt = 2.0 / ((1.0 - z * z) * dp * dp);
        if (std::fabs(z) < 1e-15) { nx[n] = 0.0; nw[n++] = wt; }
        else { nx[n] = -std::fabs(z); nw[n++] = wt; nx[n] = std::fabs(z); nw[n++] = wt; }
    }
    // stable insertion sort by |x|
    for (int i = 1; i < n; ++i)
        for (int j = i; j > 0 && std::fabs(nx[j]) < std::fabs(nx[j - 1]); --j) {
            std::swap(nx[j], nx[j - 1]); std::swap(nw[j], nw[j - 1]);
        }
    for (int i = 0; i < k; ++i) { x[i] = nx[i]; w[i] = nw[i] / 2.0; }
}

NodeField cell_field(const int* N, int comp) {
    NodeField F;
    F.Mx = N[0] + (comp == 0); F.My = N[1] + (comp == 1); F.Mz = N[2] + (comp == 2);
    F.ox = comp == 0 ? 0.0 : 0.5; F.oy = comp == 1 ? 0.0 : 0.5; F.oz = comp == 2 ? 0.0 : 0.5;
    return F;
}

NodeField psi_field(const NodeField& A) {
    NodeField P = A;
    P.My = A.My + 1;
    P.oy = A.oy - 0.5;
    return P;
}

NodeField field32(NodeField F) {
    F.oxf = (float)F.ox; F.oyf = (float)F.oy; F.ozf = (float)F.oz;
    return F;
}

PassDesc desc32(const PassDesc& d) {
    PassDesc e = d;
    e.A = field32(d.A);
    e.P = field32(d.P);
    for (int q = 0; q < kMaxGauss; ++q) { e.gxf[q] = (float)d.gx[q]; e.gwf[q] = (float)d.gw[q]; }
    e.hf = (float)d.h;
    e.invhf = (float)(1.0 / d.h);
    e.dthf = (float)(d.dt / d.h);
    e.color_off_f[0] = (float)d.color_off[0]; e.color_off_f[1] = (float)d.color_off[1];
    e.minimal_area_f = (float)d.minimal_area;
    return e;
}

// ------------------------------------------------------------------------------------
// psi: one thread per column (i,k); psi(.,0,.) = 0, psi(.,j,.) = psi(.,j-1,.) + incr(j-1)
// ------------------------------------------------------------------------------------
template <typename T>
__global__ void k_psi(PassDesc d, const T* __restrict__ a, T* __restrict__ psi) {
    const int Mx = d.A.Mx, My = d.A.My, Mz = d.A.Mz;
    const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (long long)Mx * Mz) return;
    const int i = (int)(col / Mz), k = (int)(col % Mz);
    const T h = T(d.h);
    const T px = (T(i) + T(d.A.ox)) * h, pz = (T(k) + T(d.A.oz)) * h;
    T acc = T(0);
    psi[idx3(d.P, i, 0, k)] = T(0);
    for (int j = 1; j <= My; ++j) {
        if (d.psi_mode == PSI_PLAIN) {
            acc = acc + ldg(a + idx3(d.A, i, j - 1, k)) * h;
        } else if (d.psi_mode == PSI_WENO6) {
            // cell j-1 spans [(j-1+oy-.5)h, (j+oy-.5)h]; k Gauss points per half
            const T ylo = (T(j) - T(1.0) + T(d.A.oy) - T(0.5)) * h;
            const T ymid = (T(j) - T(0.5) + T(d.A.oy) - T(0.5)) * h;
            const T yhi = (T(j) + T(d.A.oy) - T(0.5)) * h;
            for (int half = 0; half < 2; ++half) {
                const T lo = half ? ymid : ylo, hi = half ? yhi : ymid;
                const T L = hi - lo;
                for (int q = 0; q < d.k; ++q) {
                    const T py = (L / T(2)) * T(d.gx[q]) + (L / T(2)) + lo;
                    acc += weno6_1dy(a, d.A, h, px, py, pz) * (h / T(2)) * T(d.gw[q]);
                }
            }
        } else {
            const T y0 = ((T(j - 1) + T(0.25)) + T(d.A.oy) - T(0.5)) * h;
            const T y1 = ((T(j - 1) + T(0.75)) + T(d.A.oy) - T(0.5)) * h;
            const T a0 = lin3d(a, d.A, h, px, y0, pz), a1 = lin3d(a, d.A, h, px, y1, pz);
            acc = acc + a0 * (h / T(2)) + a1 * (h / T(2));
        }
        psi[idx3(d.P, i, j, k)] = acc;
    }
}

// ------------------------------------------------------------------------------------
// vertex positions
// ------------------------------------------------------------------------------------
// interp with WENO6 collapsed along the axes on which the point lies on a node plane of F
// (equal in exact arithmetic; the vertices at rest and the psi points of the pieces sit there)
// (PassDesc::full_weno switches it off, to measure what it saves)
template <typename T>
__device__ __forceinline__ T interp_c(const PassDesc& d, int method, const T* __restrict__ a, const NodeField& F, T h,
                                      T px, T py, T pz) {
    if (method == INTERP_WENO6 && !d.full_weno) return weno6_3d_collapse(a, F, h, px, py, pz);
    return interp(method, a, F, h, px, py, pz);
}

template <typename T>
__device__ __forceinline__ void vertex_rest_position(const PassDesc& d, int i, int j, int k, T* p) {
    const T h = T(d.h);
    p[0] = T(i) * h; p[1] = T(j) * h; p[2] = T(k) * h;
    if (d.comp >= 0) p[d.comp] -= T(1) * T(0.5) * h;
}

// uniform in [-1, 1) from a vertex index, an axis and a seed (splitmix64 finaliser)
__device__ __forceinline__ double jitter_unit(long long id, int axis, unsigned seed) {
    unsigned long long x = (unsigned long long)id * 3ull + (unsigned long long)axis + ((unsigned long long)seed << 40);
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    x ^= x >> 31;
    return (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

template <typename T>
__global__ void k_backtrace(PassDesc d, const T* __restrict__ u, const T* __restrict__ v,
                            const T* __restrict__ w, NodeField fu, NodeField fv, NodeField fw,
                            T* __restrict__ verts) {
    const int Lx = d.A.Mx + 1, Ly = d.A.My + 1, Lz = d.A.Mz + 1;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)Lx * Ly * Lz) return;
    const int k = (int)(id % Lz);
    const int j = (int)((id / Lz) % Ly);
    const int i = (int)(id / ((long long)Lz * Ly));
    const T h = T(d.h);
    T p[3];
    vertex_rest_position(d, i, j, k, p);
    bool pinned = false;
    if (d.comp >= 0) {
        const int vi = d.comp == 0 ? i : (d.comp == 1 ? j : k);
        pinned = (vi <= 1 || vi >= d.N[d.comp]);
    }
    if (!pinned) {
        // at the rest position WENO6 collapses along the axes on which the vertex lies on a node
        // plane of the component's lattice (weno6_3d_collapse)
        const T vx = interp_c(d, d.interp, u, fu, h, p[0], p[1], p[2]);
        const T vy = interp_c(d, d.interp, v, fv, h, p[0], p[1], p[2]);
        const T vz = interp_c(d, d.interp, w, fw, h, p[0], p[1], p[2]);
        const T dt = T(d.dt);
        p[0] -= vx * dt; p[1] -= vy * dt; p[2] -= vz * dt;
        if (d.vertex_jitter != 0.0)
            for (int c = 0; c < 3; ++c) p[c] += T(d.vertex_jitter * jitter_unit(id, c, d.jitter_seed)) * h;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int e = (c == d.comp);
        const T lo = T(0) - T(e) * T(0.5) * h;
        const T hi = T(0) + h * T(d.N[c]) + T(e) * T(0.5) * h;
        if (p[c] < lo) p[c] = lo;
        if (p[c] > hi) p[c] = hi;
    }
    verts[3 * id + 0] = p[0]; verts[3 * id + 1] = p[1]; verts[3 * id + 2] = p[2];
}

// Second trace of the flux MacCormack scheme (calc_backtraced_face_3D.cpp:9-128, time
// direction "backward"): x2 = x1 + dt u(x1), the velocity interpolated at the backtraced
// position x1, the pin rule of the first trace, then the clamp (:131-160).
template <typename T>
__global__ void k_forward_trace(PassDesc d, const T* __restrict__ u, const T* __restrict__ v,
                                const T* __restrict__ w, NodeField fu, NodeField fv, NodeField fw,
                                const T* __restrict__ verts, T* __restrict__ verts2) {
    const int Lx = d.A.Mx + 1, Ly = d.A.My + 1, Lz = d.A.Mz + 1;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)Lx * Ly * Lz) return;
    const int k = (int)(id % Lz);
    const int j = (int)((id / Lz) % Ly);
    const int i = (int)(id / ((long long)Lz * Ly));
    const T h = T(d.h);
    T p[3] = {verts[3 * id], verts[3 * id + 1], verts[3 * id + 2]};
    bool pinned = false;
    if (d.comp >= 0) {
        const int vi = d.comp == 0 ? i : (d.comp == 1 ? j : k);
        pinned = (vi <= 1 || vi >= d.N[d.comp]);
    }
    if (!pinned) {
        const T vx = interp(d.interp, u, fu, h, p[0], p[1], p[2]);
        const T vy = interp(d.interp, v, fv, h, p[0], p[1], p[2]);
        const T vz = interp(d.interp, w, fw, h, p[0], p[1], p[2]);
        const T dt = T(d.dt);
        p[0] += vx * dt; p[1] += vy * dt; p[2] += vz * dt;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int e = (c == d.comp);
        const T lo = T(0) - T(e) * T(0.5) * h;
        const T hi = T(0) + h * T(d.N[c]) + T(e) * T(0.5) * h;
        if (p[c] < lo) p[c] = lo;
        if (p[c] > hi) p[c] = hi;
    }
    verts2[3 * id + 0] = p[0]; verts2[3 * id + 1] = p[1]; verts2[3 * id + 2] = p[2];
}

// ------------------------------------------------------------------------------------
// clipping in (xi, eta) space with an explicit stack
// ------------------------------------------------------------------------------------
template <typename T>
struct CV { T p0, p1, c0, c1; };   // xi, eta, colour component 0, colour component 1

constexpr int kPool = 144;     // vertex pool (LIFO) for pending pieces
constexpr int kMaxVerts = 32;  // vertices per piece (MAX_TMP_POINTS of facecutter.h)
constexpr int kMaxStack = 48;

template <typename T> __device__ __forceinline__ T cv_c(const CV<T>& v, int dim) { return dim ? v.c1 : v.c0; }

// Robust bilinear map: v0 + xi (v1-v0) + eta (v3-v0) + xi eta (v0-v1+v2-v3); exact for
// faces lying in a grid plane (the form the oracle uses).
template <typename T>
__device__ __forceinline__ T bilin(const T* v, T xi, T eta) {
    const T a = v[1] - v[0], b = v[3] - v[0], c = (v[0] - v[1]) + (v[2] - v[3]);
    return v[0] + xi * a + eta * b + (xi * eta) * c;
}

template <typename T>
struct FaceGeom {
    T x[4], y[4], z[4];   // backtraced vertex coordinates in face order
};

// centroid and area of a polygon in (xi,eta) (facecutter.h:226-253)
template <typename T>
__device__ __forceinline__ void centroid(const T* px, const T* py, int num, T& cx, T& cy, T& area) {
    T a = T(0), sx = T(0), sy = T(0);
    for (int n = 0; n < num; ++n) {
        const int m = (n + 1 == num) ? 0 : n + 1;
        const T c = px[n] * py[m] - px[m] * py[n];
        a += c;
        sx += c * (px[n] + px[m]);
        sy += c * (py[n] + py[m]);
    }
    a = fabs(T(0.5) * a);
    if (a != T(0)) {
        const T s = T(1.0) / (T(6.0) * a);
        cx = sx * s; cy = sy * s;
    } else {
        sx = T(0); sy = T(0);
        for (int n = 0; n < num; ++n) { sx = sx + px[n]; sy = sy + py[n]; }
        const T s = T(1.0) / T(num);
        cx = sx * s; cy = sy * s;
    }
    area = a;
}

// 3D centroid and the y component of the scaled normal of an emitted piece (xi-eta polygon
// px/py with centroid (cxi, ceta); split_face_3D.cpp:67-93)
template <typename T>
__device__ __forceinline__ void piece_geom(const FaceGeom<T>& g, const T* px, const T* py, int num, T cxi, T ceta,
                                           T& cx, T& cy, T& cz, T& ny) {
    cx = bilin(g.x, cxi, ceta); cy = bilin(g.y, cxi, ceta); cz = bilin(g.z, cxi, ceta);
    if (num == 3) {
        const T ax = bilin(g.x, px[1], py[1]) - bilin(g.x, px[0], py[0]);
        const T az = bilin(g.z, px[1], py[1]) - bilin(g.z, px[0], py[0]);
        const T bx = bilin(g.x, px[2], py[2]) - bilin(g.x, px[0], py[0]);
        const T bz = bilin(g.z, px[2], py[2]) - bilin(g.z, px[0], py[0]);
        ny = T(0.5) * (az * bx - ax * bz);
    } else {
        T acc = T(0);
        T x0 = bilin(g.x, px[0], py[0]) - cx, z0 = bilin(g.z, px[0], py[0]) - cz;
        const T xs = x0, zs = z0;
        for (int n = 0; n < num; ++n) {
            T x1, z1;
            if (n + 1 == num) { x1 = xs; z1 = zs; }
            else { x1 = bilin(g.x, px[n + 1], py[n + 1]) - cx; z1 = bilin(g.z, px[n + 1], py[n + 1]) - cz; }
            acc += z0 * x1 - x0 * z1;
            x0 = x1; z0 = z1;
        }
        ny = acc * T(0.5);
    }
}

// weno6_3d_collapse at points that share x and z (the density quadrature points of a piece,
// polygon_3D.cpp:286-453) and whose stencils start in two consecutive y rows: the z-pass of
// the 6 x 7 (x, y) stencil rows is evaluated once into the thread's column zs (word
// (7 ix + r) * stride, shared memory), and each point takes its y- and x-passes from it.  The
// same evaluations on the same values as weno6_3d_collapse point by point, so the same results,
// in 42 + 7 per point 1D evaluations instead of 43 per point.  point(m, y, w) gives point m in
// [ya, yb]; acc += value * w in order.  A point whose row falls outside the column is evaluated
// on its own.
template <typename T, class Pt>
__device__ void weno6_column(const T* __restrict__ a, const NodeField& F, T h, T px, T pz, T ya, T yb, int npts,
                             const Pt& point, T& acc, T* zs, int stride) {
    const T rx = (px - T(F.ox) * h) / h, rz = (pz - T(F.oz) * h) / h;
    const T sx = snap_int(rx), sz = snap_int(rz);
    const bool cxn = sx == rint(sx), czn = sz == rint(sz);
    const int bx = cxn ? (int)sx : (int)floor(rx);
    const int bz = czn ? (int)sz : (int)floor(rz);
    auto row_of = [&](T py) {
        const T ry = (py - T(F.oy) * h) / h;
        const T sy = snap_int(ry);
        return sy == rint(sy) ? (int)sy : (int)floor(ry);
    };
    const int by0 = row_of(ya);
    const int nr = row_of(yb) > by0 ? 7 : 6;
    T tx[6], tz[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        tx[i] = rx - T(bx - 2 + i);
        tz[i] = rz - T(bz - 2 + i);
    }
    const WenoCoef<T> cx = weno_coef(tx), cz = weno_coef(tz);
    int kk[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) kk[i] = clampi(bz - 2 + i, F.Mz - 1);
    const int x0 = cxn ? 2 : 0, x1 = cxn ? 3 : 6;
#pragma unroll 1
    for (int ix = x0; ix < x1; ++ix) {
        const int ii = clampi(bx - 2 + ix, F.Mx - 1);
#pragma unroll 1
        for (int r = 0; r < nr; ++r) {
            const int jj = clampi(by0 - 2 + r, F.My - 1);
            const T* row = a + (long long)F.Mz * ((long long)F.My * ii + jj);
            T v;
            if (czn) {
                v = ldg(row + kk[2]);
            } else {
                T f[6];
#pragma unroll
                for (int iz = 0; iz < 6; ++iz) f[iz] = ldg(row + kk[iz]);
                v = weno6_eval(f, cz);
            }
            zs[(7 * ix + r) * stride] = v;
        }
    }
#pragma unroll 1
    for (int m = 0; m < npts; ++m) {
        T y, w;
        point(m, y, w);
        const T ry = (y - T(F.oy) * h) / h;
        const T sy = snap_int(ry);
        const bool cyn = sy == rint(sy);
        const int by = cyn ? (int)sy : (int)floor(ry);
        T val;
        if (by < by0 || by - by0 > nr - 6) {
            val = weno6_3d_collapse(a, F, h, px, y, pz);
        } else {
            T ty[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) ty[i] = ry - T(by - 2 + i);
            const WenoCoef<T> cy = weno_coef(ty);
            const T* zb = zs + (by - by0) * stride;
            T yv[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
#pragma unroll 1
            for (int ix = x0; ix < x1; ++ix) {
                if (cyn) {
                    yv[ix] = zb[(7 * ix + 2) * stride];
                } else {
                    T zv[6];
#pragma unroll
                    for (int iy = 0; iy < 6; ++iy) zv[iy] = zb[(7 * ix + iy) * stride];
                    yv[ix] = weno6_eval(zv, cy);
                }
            }
            val = cxn ? yv[2] : weno6_eval(yv, cx);
        }
        acc += val * w;
    }
}

// The quadrature of one piece with centroid (cx, cy, cz) and y-normal ny (polygon_3D.cpp:257-487).
// With a column zs (42 words at stride `stride`, see weno6_column) the WENO6 density points
// share their z-pass.
template <typename T>
__device__ __forceinline__ T piece_quad(const PassDesc& d, T cx, T cy, T cz, T ny, const T* __restrict__ a,
                                        const T* __restrict__ psi, T* zs = nullptr, int stride = 0) {
    if (ny == T(0)) return T(0);
    const T h = T(d.h);
    T F = T(0);
    if (d.use_integral) {
        // polygon_3D.cpp:257-487 with the grid origin shifted by -h/2 along a staggered axis
        const T oy = (d.comp == 1) ? T(-1) * T(0.5) * h : T(0);
        const T ry = snap_int((cy - oy) / h);
        const int iy0 = (int)floor(ry);
        const T f = ry - T(iy0);
        if (zs && d.interp == INTERP_WENO6 && !d.full_weno) {
            // the same points, weights and order as below
            const int k = d.k;
            if (f < T(0.5)) {
                const T lo = T(iy0) * h + oy, L = cy - lo;
                auto pt = [&](int q, T& y, T& w) {
                    y = (L / T(2)) * T(d.gx[q]) + (L / T(2)) + lo;
                    w = ny * f * h * T(d.gw[q]);
                };
                weno6_column(a, d.A, h, cx, cz, lo, cy, k, pt, F, zs, stride);
            } else {
                const T lo0 = T(iy0) * h + oy, hi0 = (T(iy0) + T(0.5)) * h + oy, L0 = hi0 - lo0;
                const T lo1 = (T(iy0) + T(0.5)) * h + oy, hi1 = (T(iy0) + f) * h + oy, L1 = hi1 - lo1;
                auto pt = [&](int m, T& y, T& w) {
                    if (m < k) {
                        y = (L0 / T(2)) * T(d.gx[m]) + (L0 / T(2)) + lo0;
                        w = ny * T(0.5) * h * T(d.gw[m]);
                    } else {
                        y = (L1 / T(2)) * T(d.gx[m - k]) + (L1 / T(2)) + lo1;
                        w = ny * (f - T(0.5)) * h * T(d.gw[m - k]);
                    }
                };
                weno6_column(a, d.A, h, cx, cz, lo0, hi1, 2 * k, pt, F, zs, stride);
            }
        } else if (f < T(0.5)) {
            const T lo = T(iy0) * h + oy, L = cy - lo;
            for (int q = 0; q < d.k; ++q) {
                const T yq = (L / T(2)) * T(d.gx[q]) + (L / T(2)) + lo;
                F += interp_c(d, d.interp, a, d.A, h, cx, yq, cz) * (ny * f * h * T(d.gw[q]));
            }
        } else {
            T lo = T(iy0) * h + oy, hi = (T(iy0) + T(0.5)) * h + oy, L = hi - lo;
            for (int q = 0; q < d.k; ++q) {
                const T yq = (L / T(2)) * T(d.gx[q]) + (L / T(2)) + lo;
                F += interp_c(d, d.interp, a, d.A, h, cx, yq, cz) * (ny * T(0.5) * h * T(d.gw[q]));
            }
            lo = (T(iy0) + T(0.5)) * h + oy; hi = (T(iy0) + f) * h + oy; L = hi - lo;
            for (int q = 0; q < d.k; ++q) {
                const T yq = (L / T(2)) * T(d.gx[q]) + (L / T(2)) + lo;
                F += interp_c(d, d.interp, a, d.A, h, cx, yq, cz) * (ny * (f - T(0.5)) * h * T(d.gw[q]));
            }
        }
        F += interp_c(d, d.interp, psi, d.P, h, cx, T(iy0) * h + oy, cz) * ny;
    } else {
        F += interp_c(d, d.interp, psi, d.P, h, cx, cy, cz) * ny;
    }
    return F;
}

// Accumulates the flux of one emitted piece (xi-eta polygon px/py with centroid c) and its
// volume point y n_y (polygon_3D.cpp:480-486).
template <typename T>
__device__ __forceinline__ T piece_flux(const PassDesc& d, const FaceGeom<T>& g, const T* px, const T* py,
                                        int num, T cxi, T ceta, const T* __restrict__ a,
                                        const T* __restrict__ psi, T* vol) {
    T cx, cy, cz, ny;
    piece_geom(g, px, py, num, cxi, ceta, cx, cy, cz, ny);
    if (vol) *vol += cy * ny;
    return piece_quad(d, cx, cy, cz, ny, a, psi);
}

// What the clipper does with each emitted piece: the per-face kernel evaluates it at once
// (EvalPiece), the piece pipeline stores it (StorePiece, below).
template <typename T>
struct EvalPiece {
    const PassDesc& d;
    const T* __restrict__ a;
    const T* __restrict__ psi;
    T* vol;
    __device__ __forceinline__ T operator()(const FaceGeom<T>& g, const T* px, const T* py, int num, T cxi,
                                            T ceta) const {
        return piece_flux(d, g, px, py, num, cxi, ceta, a, psi, vol);
    }
};

// Emits a polygon (optionally triangulated to minimal_area, facecutter.h:255-324).
template <typename T, class Emit>
__device__ T emit_polygon(const PassDesc& d, const FaceGeom<T>& g, const T* px, const T* py, int num,
                          const Emit& emit, unsigned& st, int& npieces) {
    T cx, cy, area;
    centroid(px, py, num, cx, cy, area);
    const T minA = T(d.minimal_area);
    if (!(area > minA)) {
        if (area != T(0)) { ++npieces; return emit(g, px, py, num, cx, cy); }
        return T(0);
    }
    // triangulate: fan from the centroid (num > 3) then recursive longest-edge bisection
    T F = T(0);
    T tri[24][6];
    int top = 0;
    if (num == 3) {
        tri[top][0] = px[0]; tri[top][1] = py[0]; tri[top][2] = px[1]; tri[top][3] = py[1];
        tri[top][4] = px[2]; tri[top][5] = py[2]; ++top;
    } else {
        for (int n = num - 1; n >= 0; --n) {
            const int m = (n + 1 == num) ? 0 : n + 1;
            if (top >= 24) { st |= ST_SUBDIV_OVERFLOW; return F; }
            tri[top][0] = cx; tri[top][1] = cy; tri[top][2] = px[n]; tri[top][3] = py[n];
            tri[top][4] = px[m]; tri[top][5] = py[m]; ++top;
        }
    }
    while (top > 0) {
        --top;
        T tx[3] = {tri[top][0], tri[top][2], tri[top][4]};
        T ty[3] = {tri[top][1], tri[top][3], tri[top][5]};
        T tcx, tcy, tarea;
        centroid(tx, ty, 3, tcx, tcy, tarea);
        if (tarea > minA) {
            // the first of the longest edges, lengths within kLongestEdgeTie counting as equal
            int mi = 0; T ml = T(-1);
            for (int n = 0; n < 3; ++n) {
                const int m = (n + 1) % 3;
                const T len = (tx[n] - tx[m]) * (tx[n] - tx[m]) + (ty[n] - ty[m]) * (ty[n] - ty[m]);
                if (len > ml * T(1.0 + kLongestEdgeTie)) { ml = len; mi = n; }
            }
            const int i1 = (mi + 1) % 3, i2 = (mi + 2) % 3;
            const T mx = T(0.5) * (tx[mi] + tx[i1]), my = T(0.5) * (ty[mi] + ty[i1]);
            if (top + 2 > 24) { st |= ST_SUBDIV_OVERFLOW; return F; }
            // push second half first so the first half is processed first
            tri[top][0] = mx; tri[top][1] = my; tri[top][2] = tx[i1]; tri[top][3] = ty[i1];
            tri[top][4] = tx[i2]; tri[top][5] = ty[i2]; ++top;
            tri[top][0] = tx[mi]; tri[top][1] = ty[mi]; tri[top][2] = mx; tri[top][3] = my;
            tri[top][4] = tx[i2]; tri[top][5] = ty[i2]; ++top;
        } else if (tarea != T(0)) {
            ++npieces;
            F += emit(g, tx, ty, 3, tcx, tcy);
        }
    }
    return F;
}

// Clips one face and returns its flux (sum over pieces of the quadrature terms).
// `multi` is set when some iso-line crosses a piece more than twice: the piece that holds
// the first vertex then merges several disjoint parts (facecutter.h:163-181), so the
// partition depends on the vertex order and the two adjacent cells see different pieces.
template <typename T, class Emit>
__device__ T clip_face(const PassDesc& d, const FaceGeom<T>& g, const Emit& emit, unsigned& st, int& npieces,
                       bool& multi) {
    const T h = T(d.h);
    CV<T> pool[kPool];
    unsigned char sstart[kMaxStack], snum[kMaxStack], sdim[kMaxStack];
    int sp = 0, top = 4;
    const T xi[4] = {T(0), T(1), T(1), T(0)}, eta[4] = {T(0), T(0), T(1), T(1)};
    bool finite = true;
    for (int q = 0; q < 4; ++q) {
        pool[q].p0 = xi[q]; pool[q].p1 = eta[q];
        pool[q].c0 = snap_int(g.x[q] / h - T(d.color_off[0]));
        pool[q].c1 = snap_int(g.z[q] / h - T(d.color_off[1]));
        finite = finite && isfinite(pool[q].c0) && isfinite(pool[q].c1) && isfinite(g.y[q]);
    }
    // every cut narrows the range of a polygon's finite colours, which bounds the loop below;
    // a face with a non-finite vertex (NaN or infinite velocity upstream) is not clipped
    if (!finite) { st |= ST_NONFINITE; return T(0); }
    sstart[0] = 0; snum[0] = 4; sdim[0] = 0; sp = 1;
    T F = T(0);
    CV<T> tmp0[kMaxVerts + 2];
    while (sp > 0) {
        --sp;
        const int pstart = sstart[sp], num = snum[sp], dim = sdim[sp];
        const CV<T>* poly = pool + pstart;
        T mn = cv_c(poly[0], dim), mx = mn;
        for (int n = 1; n < num; ++n) { const T c = cv_c(poly[n], dim); mn = fmin(mn, c); mx = fmax(mx, c); }
        int start = (int)ceil(mn), end = (int)floor(mx);
        if (mn - T(start) == T(0)) start += 1;
        if (mx - T(end) == T(0)) end -= 1;
        bool cut = false;
        if (start <= end) {
            if (pstart + 3 * num + 2 > kPool) { st |= ST_CLIP_OVERFLOW; top = pstart; continue; }
            const T iso = T(start);
            int h0 = 0, h1 = 0, slot = 0;
            int wpos = pstart + num;          // pieces on the far side are written here
            int p1start = wpos;
            int nchild = 0;
            unsigned char cst[kMaxStack], cnum[kMaxStack];
            tmp0[h0++] = poly[0];
            bool bad = false;
            for (int n = 0; n < num && !bad; ++n) {
                const int m = (n + 1 == num) ? 0 : n + 1;
                const T v0 = cv_c(poly[n], dim) - iso, v1 = cv_c(poly[m], dim) - iso;
                if ((v0 < T(0)) != (v1 < T(0))) {
                    const T inv = T(1.0) / (v1 - v0);
                    const T t0 = v1 * inv, t1 = -v0 * inv;
                    cut = true;
                    CV<T> X;
                    X.p0 = t0 * poly[n].p0 + t1 * poly[m].p0;
                    X.p1 = t0 * poly[n].p1 + t1 * poly[m].p1;
                    const T other = snap_int(t0 * cv_c(poly[n], 1 - dim) + t1 * cv_c(poly[m], 1 - dim));
                    if (dim == 0) { X.c0 = iso; X.c1 = other; } else { X.c1 = iso; X.c0 = other; }
                    if (slot == 0) {
                        tmp0[h0++] = X;
                        slot = 1; h1 = 0; p1start = wpos;
                        if (t1 < T(1.0)) pool[p1start + h1++] = X;
                    } else {
                        pool[p1start + h1++] = X;
                        if (nchild >= kMaxStack - 1) { bad = true; break; }
                        cst[nchild] = (unsigned char)p1start; cnum[nchild] = (unsigned char)h1; ++nchild;
                        wpos = p1start + h1;
                        slot = 0;
                        if (t1 < T(1.0)) tmp0[h0++] = X;
                    }
                }
                if (n < num - 1) {
                    if (slot == 0) tmp0[h0++] = poly[m];
                    else pool[p1start + h1++] = poly[m];
                }
                if (h0 >= kMaxVerts || h1 >= kMaxVerts || p1start + h1 + 2 >= kPool) bad = true;
            }
            if (bad) { st |= ST_CLIP_OVERFLOW; top = pstart; continue; }
            if (nchild > 1) multi = true;
            if (cut) {
                if (slot != 0) { st |= ST_CLIP_ODD_CUT; top = pstart; continue; }
                if (wpos + h0 >= kPool || sp + nchild + 1 > kMaxStack) { st |= ST_CLIP_OVERFLOW; top = pstart; continue; }
                // piece 0 goes after the far-side pieces; then the block moves down over the parent
                for (int q = 0; q < h0; ++q) pool[wpos + q] = tmp0[q];
                const int src = pstart + num, len = wpos + h0 - src;
                for (int q = 0; q < len; ++q) pool[pstart + q] = pool[src + q];
                for (int c = 0; c < nchild; ++c) {
                    sstart[sp] = (unsigned char)(cst[c] - num); snum[sp] = cnum[c]; sdim[sp] = (unsigned char)dim; ++sp;
                }
                sstart[sp] = (unsigned char)(wpos - num); snum[sp] = (unsigned char)h0; sdim[sp] = (unsigned char)dim; ++sp;
                top = pstart + len;
            }
        }
        if (!cut) {
            if (dim == 0) {
                sstart[sp] = (unsigned char)pstart; snum[sp] = (unsigned char)num; sdim[sp] = 1; ++sp;
                top = pstart + num;
            } else {
                if (num >= 3) {
                    T px[kMaxVerts], py[kMaxVerts];
                    for (int q = 0; q < num; ++q) { px[q] = poly[q].p0; py[q] = poly[q].p1; }
                    F += emit_polygon(d, g, px, py, num, emit, st, npieces);
                }
                top = pstart;
            }
        }
    }
    (void)top;
    return F;
}

// Face families: 0 = faces normal to x, 1 = normal to y, 2 = normal to z, in the vertex
// order of the face as seen from the lower cell (faces 1, 2, 5 of
// backtrace_..._for_integrate_density.cpp:83-112).
__device__ __forceinline__ void face_corners(int fam, int i, int j, int k, int* ci, int* cj, int* ck) {
    if (fam == 0) {
        ci[0] = i; cj[0] = j;     ck[0] = k;
        ci[1] = i; cj[1] = j + 1; ck[1] = k;
        ci[2] = i; cj[2] = j + 1; ck[2] = k + 1;
        ci[3] = i; cj[3] = j;     ck[3] = k + 1;
    } else if (fam == 1) {
        ci[0] = i;     cj[0] = j; ck[0] = k;
        ci[1] = i;     cj[1] = j; ck[1] = k + 1;
        ci[2] = i + 1; cj[2] = j; ck[2] = k + 1;
        ci[3] = i + 1; cj[3] = j; ck[3] = k;
    } else {
        ci[0] = i;     cj[0] = j;     ck[0] = k;
        ci[1] = i + 1; cj[1] = j;     ck[1] = k;
        ci[2] = i + 1; cj[2] = j + 1; ck[2] = k;
        ci[3] = i;     cj[3] = j + 1; ck[3] = k;
    }
}

// the four corners of face id of family fam: backtraced (verts) or at rest
template <typename T>
__device__ __forceinline__ void face_geom(const PassDesc& d, int fam, long long id, const T* __restrict__ verts,
                                          FaceGeom<T>& g) {
    const int Fy = d.A.My + (fam == 1), Fz = d.A.Mz + (fam == 2);
    const int k = (int)(id % Fz);
    const int j = (int)((id / Fz) % Fy);
    const int i = (int)(id / ((long long)Fz * Fy));
    int ci[4], cj[4], ck[4];
    face_corners(fam, i, j, k, ci, cj, ck);
    const int Ly = d.A.My + 1, Lz = d.A.Mz + 1;
    for (int q = 0; q < 4; ++q) {
        if (d.zero_velocity) {
            T p[3];
            vertex_rest_position(d, ci[q], cj[q], ck[q], p);
            g.x[q] = p[0]; g.y[q] = p[1]; g.z[q] = p[2];
        } else {
            const long long vid = ((long long)ci[q] * Ly + cj[q]) * Lz + ck[q];
            g.x[q] = verts[3 * vid]; g.y[q] = verts[3 * vid + 1]; g.z[q] = verts[3 * vid + 2];
        }
    }
}

// the upper cell's own face: vertex order (v0, v3, v2, v1), which is the reference's x-/y-/z-
// face order (backtrace_..._for_integrate_density.cpp:77-112)
template <typename T>
__device__ __forceinline__ FaceGeom<T> upper_face(const FaceGeom<T>& g) {
    FaceGeom<T> r = g;
    r.x[1] = g.x[3]; r.y[1] = g.y[3]; r.z[1] = g.z[3];
    r.x[3] = g.x[1]; r.y[3] = g.y[1]; r.z[3] = g.z[1];
    return r;
}

// The flux of face id of family fam, clipped and integrated piece by piece as the clipper emits
// them: flux = wgt * F (acc = 0) or flux + wgt * F (acc = 1) -- the weighted faces of the flux
// MacCormack scheme accumulate into one flux per face (wgt = 1, acc = 0 otherwise).
template <typename T>
__device__ __forceinline__ void face_eval(const PassDesc& d, int fam, long long id, const T* __restrict__ a,
                                          const T* __restrict__ psi, const T* __restrict__ verts,
                                          T* __restrict__ flux, T* __restrict__ flux_rev, T wgt, int acc,
                                          T* __restrict__ fvol, T* __restrict__ fvol_rev, unsigned& st,
                                          int& npieces, int& nmulti) {
    FaceGeom<T> g;
    face_geom(d, fam, id, verts, g);
    bool multi = false;
    T V = T(0), Vr = T(0);
    const T F = clip_face(d, g, EvalPiece<T>{d, a, psi, fvol ? &V : nullptr}, st, npieces, multi);
    T Fr = -F;
    Vr = -V;
    if (multi) {
        const FaceGeom<T> r = upper_face(g);
        int np2 = 0; bool m2 = false;
        Vr = T(0);
        Fr = clip_face(d, r, EvalPiece<T>{d, a, psi, fvol ? &Vr : nullptr}, st, np2, m2);
        ++nmulti;
    }
    if (!isfinite(F) || !isfinite(Fr)) st |= ST_NONFINITE;
    flux[id] = acc ? flux[id] + wgt * F : wgt * F;
    flux_rev[id] = acc ? flux_rev[id] + wgt * Fr : wgt * Fr;
    if (fvol) {
        fvol[id] = acc ? fvol[id] + wgt * V : wgt * V;
        fvol_rev[id] = acc ? fvol_rev[id] + wgt * Vr : wgt * Vr;
    }
}

template <typename T>
__global__ void __launch_bounds__(128) k_faces(PassDesc d, int fam, const T* __restrict__ a,
                                               const T* __restrict__ psi, const T* __restrict__ verts,
                                               T* __restrict__ flux, T* __restrict__ flux_rev,
                                               unsigned* status, unsigned long long* counters, T wgt, int acc,
                                               T* __restrict__ fvol, T* __restrict__ fvol_rev) {
    const int Fx = d.A.Mx + (fam == 0), Fy = d.A.My + (fam == 1), Fz = d.A.Mz + (fam == 2);
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nface = (long long)Fx * Fy * Fz;
    unsigned st = 0;
    int npieces = 0, nmulti = 0;
    if (id < nface) face_eval(d, fam, id, a, psi, verts, flux, flux_rev, wgt, acc, fvol, fvol_rev, st, npieces, nmulti);
    // warp-aggregated counters and status
    unsigned long long pc = (unsigned long long)npieces;
    unsigned fc = id < nface ? 1u : 0u, mc = (unsigned)nmulti;
    for (int o = 16; o > 0; o >>= 1) {
        pc += __shfl_down_sync(0xffffffffu, pc, o);
        fc += __shfl_down_sync(0xffffffffu, fc, o);
        mc += __shfl_down_sync(0xffffffffu, mc, o);
        st |= __shfl_down_sync(0xffffffffu, st, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (fc) { atomicAdd(&counters[0], (unsigned long long)fc); atomicAdd(&counters[1], pc); }
        if (mc) atomicAdd(&counters[2], (unsigned long long)mc);
        if (st) atomicOr(status, st);
    }
}

// ------------------------------------------------------------------------------------
// The plain form's piece pipeline: k_clip64 (one thread per face: the clip, its pieces
// appended contiguously per face), k_quad64 (one thread per piece: the quadrature) and
// k_facesum64 (one thread per face: its pieces' fluxes summed in emission order).  The clip,
// the per-piece arithmetic and the order of every sum are those of k_faces, which evaluates
// each piece as the clipper emits it: there the lanes of a warp wait for the face with the
// most pieces (a third of them active on average); here each lane has one piece.
// ------------------------------------------------------------------------------------
constexpr int kMaxPieces64 = 64;   // pieces of one face, both clips (as the FP32 store)

struct StorePiece64 {
    double4_32a* p;
    int* n;
    bool* spill;   // the face has more pieces than the buffer: it is evaluated by k_faces_deferred64
    __device__ __forceinline__ double operator()(const FaceGeom<double>& g, const double* px, const double* py, int num,
                                                 double cxi, double ceta) const {
        if (*n >= kMaxPieces64) { *spill = true; return 0.0; }
        double cx, cy, cz, ny;
        piece_geom(g, px, py, num, cxi, ceta, cx, cy, cz, ny);
        p[(*n)++] = make_double4_32a(cx, cy, cz, ny);
        return 0.0;
    }
};

__device__ __forceinline__ int2* range64(const PieceStore64& ps, int fam) {
    return fam == 0 ? ps.range[0] : (fam == 1 ? ps.range[1] : ps.range[2]);
}

__global__ void __launch_bounds__(128) k_clip64(PassDesc d, int fam, const double* __restrict__ verts, PieceStore64 ps,
                                                unsigned* status, unsigned long long* counters) {
    const long long nface = (long long)(d.A.Mx + (fam == 0)) * (d.A.My + (fam == 1)) * (d.A.Mz + (fam == 2));
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    unsigned st = 0;
    int npieces = 0, n = 0, nfwd = 0;
    bool multi = false, spill = false;
    double4_32a buf[kMaxPieces64];
    if (id < nface) {
        FaceGeom<double> g;
        face_geom(d, fam, id, verts, g);
        clip_face(d, g, StorePiece64{buf, &n, &spill}, st, npieces, multi);
        nfwd = n;
        if (multi) {
            int np2 = 0;
            bool m2 = false;
            clip_face(d, upper_face(g), StorePiece64{buf, &n, &spill}, st, np2, m2);
        }
        if (spill) {
            // too many pieces for the buffer (triangulated faces at high CFL): the face is
            // listed and evaluated as a whole by k_faces_deferred64
            n = 0;
            ps.deferred[atomicAdd(ps.count + 1, 1u)] = (fam << 29) | (int)id;
        }
    }
    const long long start = warp_slots(ps.count, n, lane);
    if (id < nface) {
        // a range beyond the capacity is kept as it is: the host sees the count, grows the
        // store and clips again
        if (start + n <= ps.cap)
            for (int q = 0; q < n; ++q) ps.rec[start + q] = buf[q];
        range64(ps, fam)[id] = spill ? make_int2(-1, 0)
                                     : make_int2((int)start, nfwd | ((n - nfwd) << 15) | ((multi ? 1 : 0) << 30));
    }
    unsigned long long pc = (unsigned long long)npieces;
    unsigned fc = id < nface ? 1u : 0u, mc = multi ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) {
        pc += __shfl_down_sync(0xffffffffu, pc, o);
        fc += __shfl_down_sync(0xffffffffu, fc, o);
        mc += __shfl_down_sync(0xffffffffu, mc, o);
        st |= __shfl_down_sync(0xffffffffu, st, o);
    }
    if (lane == 0) {
        if (fc) { atomicAdd(&counters[0], (unsigned long long)fc); atomicAdd(&counters[1], pc); }
        if (mc) atomicAdd(&counters[2], (unsigned long long)mc);
        if (st) atomicOr(status, st);
    }
}

constexpr int kQuad64Threads = 128;

__global__ void __launch_bounds__(kQuad64Threads) k_quad64(PassDesc d, const double* __restrict__ a,
                                                           const double* __restrict__ psi, PieceStore64 ps,
                                                           long long npc) {
    __shared__ double zcol[42 * kQuad64Threads];   // each thread's z-pass column (weno6_column)
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npc; t += (long long)gridDim.x * blockDim.x) {
        const double4_32a p = ps.rec[t];
        ps.flux[t] = piece_quad(d, p.x, p.y, p.z, p.w, a, psi, zcol + threadIdx.x, kQuad64Threads);
    }
}

__global__ void k_facesum64(PassDesc d, int fam, PieceStore64 ps, double* __restrict__ flux,
                            double* __restrict__ flux_rev, unsigned* status, double wgt, int acc,
                            double* __restrict__ fvol, double* __restrict__ fvol_rev) {
    const long long nface = (long long)(d.A.Mx + (fam == 0)) * (d.A.My + (fam == 1)) * (d.A.Mz + (fam == 2));
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nface) return;
    const int2 r = range64(ps, fam)[id];
    if (r.x < 0) return;   // a listed face: k_faces_deferred64 writes it
    const int nf = r.y & 0x7fff, nr = (r.y >> 15) & 0x7fff;
    const bool multi = (r.y >> 30) & 1;
    double F = 0.0, V = 0.0;
    for (int q = 0; q < nf; ++q) {
        F += ps.flux[(long long)r.x + q];
        if (fvol) { const double4_32a p = ps.rec[(long long)r.x + q]; V += p.y * p.w; }
    }
    double Fr = -F, Vr = -V;
    if (multi) {
        Fr = 0.0; Vr = 0.0;
        for (int q = nf; q < nf + nr; ++q) {
            Fr += ps.flux[(long long)r.x + q];
            if (fvol) { const double4_32a p = ps.rec[(long long)r.x + q]; Vr += p.y * p.w; }
        }
    }
    if (!isfinite(F) || !isfinite(Fr)) atomicOr(status, (unsigned)ST_NONFINITE);
    flux[id] = acc ? flux[id] + wgt * F : wgt * F;
    flux_rev[id] = acc ? flux_rev[id] + wgt * Fr : wgt * Fr;
    if (fvol) {
        fvol[id] = acc ? fvol[id] + wgt * V : wgt * V;
        fvol_rev[id] = acc ? fvol_rev[id] + wgt * Vr : wgt * Vr;
    }
}

// The faces k_clip64 listed (all families), evaluated as k_faces does; their counters were
// counted by k_clip64.  Grid-stride over the list length in ps.count[1].
__global__ void __launch_bounds__(128) k_faces_deferred64(PassDesc d, const double* __restrict__ a,
                                                          const double* __restrict__ psi,
                                                          const double* __restrict__ verts, PieceStore64 ps,
                                                          double* fx, double* fy, double* fz, double* rx, double* ry,
                                                          double* rz, unsigned* status, double wgt, int acc,
                                                          double* vx, double* vy, double* vz, double* vrx,
                                                          double* vry, double* vrz) {
    const long long nd = (long long)ps.count[1];
    unsigned st = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nd; t += (long long)gridDim.x * blockDim.x) {
        const int tag = ps.deferred[t];
        const int fam = tag >> 29;
        const long long id = tag & ((1 << 29) - 1);
        int np = 0, nm = 0;
        double* f = fam == 0 ? fx : (fam == 1 ? fy : fz);
        double* r = fam == 0 ? rx : (fam == 1 ? ry : rz);
        double* v = vx ? (fam == 0 ? vx : (fam == 1 ? vy : vz)) : nullptr;
        double* vr = vx ? (fam == 0 ? vrx : (fam == 1 ? vry : vrz)) : nullptr;
        face_eval(d, fam, id, a, psi, verts, f, r, wgt, acc, v, vr, st, np, nm);
    }
    if (st) atomicOr(status, st);
}

// rho'(i,j,k) = (Fx(i+1) + Rx(i) + Fy(j+1) + Ry(j) + Fz(k+1) + Rz(k)) / V, where F is the
// flux of a face as the lower cell's face and R as the upper cell's (R = -F unless the
// clip partition depends on the vertex order).
template <typename T>
__global__ void k_gather(PassDesc d, const T* __restrict__ fx, const T* __restrict__ fy,
                         const T* __restrict__ fz, const T* __restrict__ rx, const T* __restrict__ ry,
                         const T* __restrict__ rz, const T* __restrict__ in, T* __restrict__ out, int mode) {
    const int Mx = d.A.Mx, My = d.A.My, Mz = d.A.Mz;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)Mx * My * Mz) return;
    const int k = (int)(id % Mz);
    const int j = (int)((id / Mz) % My);
    const int i = (int)(id / ((long long)Mz * My));
    const T h = T(d.h);
    const T V = h * h * h;
    const long long ix0 = ((long long)i * My + j) * Mz + k;             // (Mx+1) x My x Mz
    const long long ix1 = ((long long)(i + 1) * My + j) * Mz + k;
    const long long iy0 = ((long long)i * (My + 1) + j) * Mz + k;       // Mx x (My+1) x Mz
    const long long iy1 = ((long long)i * (My + 1) + j + 1) * Mz + k;
    const long long iz0 = ((long long)i * My + j) * (Mz + 1) + k;       // Mx x My x (Mz+1)
    const T s = ((fx[ix1] + rx[ix0]) + (fy[iy1] + ry[iy0])) + (fz[iz0 + 1] + rz[iz0]);
    const T val = s / V;
    if (mode == 0) out[id] = val;
    else if (mode == 1) out[id] = in[id] - val;
    else if (mode == 2) out[id] = out[id] + val;
    else out[id] = s;
}

// ------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------
static inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

template <typename T>
cudaError_t launch_psi(const PassDesc& d, const T* a, T* psi, cudaStream_t s) {
    const long long cols = (long long)d.A.Mx * d.A.Mz;
    k_psi<T><<<blocks_for(cols, 128), 128, 0, s>>>(d, a, psi);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_backtrace(const PassDesc& d, const VelocityFields& vel, T* verts, cudaStream_t s) {
    const long long n = (long long)(d.A.Mx + 1) * (d.A.My + 1) * (d.A.Mz + 1);
    k_backtrace<T><<<blocks_for(n, 128), 128, 0, s>>>(d, (const T*)vel.u, (const T*)vel.v, (const T*)vel.w,
                                                      vel.fu, vel.fv, vel.fw, verts);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_faces_from(const PassDesc& d, const T* a, const PassWork<T>& w, const T* verts, T wgt,
                                     int acc, cudaStream_t s) {
    for (int fam = 0; fam < 3; ++fam) {
        const long long n = (long long)(d.A.Mx + (fam == 0)) * (d.A.My + (fam == 1)) * (d.A.Mz + (fam == 2));
        prof_mark(w, 0, s);
        k_faces<T><<<blocks_for(n, 128), 128, 0, s>>>(d, fam, a, w.psi, verts, w.flux[fam], w.flux_rev[fam],
                                                      w.status, w.counters, wgt, acc,
                                                      d.volumes ? w.fvol[fam] : nullptr,
                                                      d.volumes ? w.fvol_rev[fam] : nullptr);
        prof_mark(w, 1, s);
    }
    return cudaGetLastError();
}

// One face stage of the piece pipeline: clip (growing the store and clipping again when it is
// too small), per-piece quadrature, per-face sums weighted into the face fluxes.
static cudaError_t face_stage64(const PassDesc& d, const double* a, const PassWork<double>& w, const double* verts,
                                double wgt, int acc, cudaStream_t s) {
    PieceStore64& ps = *w.pieces64;
    long long nface[3], big = 0;
    for (int fam = 0; fam < 3; ++fam) {
        nface[fam] = (long long)(d.A.Mx + (fam == 0)) * (d.A.My + (fam == 1)) * (d.A.Mz + (fam == 2));
        big = nface[fam] > big ? nface[fam] : big;
    }
    unsigned npc = 0;
    // the work counters as they were before the clip: a second attempt starts from them again
    cudaError_t ec = cudaMemcpyAsync(ps.saved, w.counters, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s);
    if (ec != cudaSuccess) return ec;
    for (int attempt = 0; attempt < 2; ++attempt) {
        cudaError_t e = cudaMemsetAsync(ps.count, 0, 2 * sizeof(unsigned), s);
        if (e == cudaSuccess && attempt > 0)
            e = cudaMemcpyAsync(w.counters, ps.saved, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        for (int fam = 0; fam < 3; ++fam)
            k_clip64<<<blocks_for(nface[fam], 128), 128, 0, s>>>(d, fam, verts, ps, w.status, w.counters);
        e = cudaMemcpyAsync(&npc, ps.count, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        if ((long long)npc <= ps.cap) break;
        // more pieces than the store holds: grow it and clip again
        e = piece_store64_reserve(ps, (long long)npc + npc / 4 + 1024, big);
        if (e != cudaSuccess) return e;
    }
    if ((long long)npc > ps.cap) return cudaErrorMemoryAllocation;
    if (npc > 0) {
        const long long nb = std::min<long long>(blocks_for(npc, kQuad64Threads), 152LL * 16);
        prof_mark(w, 0, s);
        k_quad64<<<(unsigned)nb, kQuad64Threads, 0, s>>>(d, a, w.psi, ps, (long long)npc);
        prof_mark(w, 1, s);
    }
    for (int fam = 0; fam < 3; ++fam)
        k_facesum64<<<blocks_for(nface[fam], 256), 256, 0, s>>>(d, fam, ps, w.flux[fam], w.flux_rev[fam], w.status, wgt,
                                                              acc, d.volumes ? w.fvol[fam] : nullptr,
                                                              d.volumes ? w.fvol_rev[fam] : nullptr);
    const bool vol = d.volumes != 0;
    k_faces_deferred64<<<152, 128, 0, s>>>(d, a, w.psi, verts, ps, w.flux[0], w.flux[1], w.flux[2], w.flux_rev[0],
                                           w.flux_rev[1], w.flux_rev[2], w.status, wgt, acc,
                                           vol ? w.fvol[0] : nullptr, vol ? w.fvol[1] : nullptr,
                                           vol ? w.fvol[2] : nullptr, vol ? w.fvol_rev[0] : nullptr,
                                           vol ? w.fvol_rev[1] : nullptr, vol ? w.fvol_rev[2] : nullptr);
    return cudaGetLastError();
}

// The piece pipeline where its face tags (family << 29 | index) hold every face; one thread
// per face otherwise (grids beyond about 800^3) and where the session has no piece store.
template <typename T>
static cudaError_t faces_weighted(const PassDesc& d, const T* a, const PassWork<T>& w, const T* verts, T wgt, int acc,
                                  cudaStream_t s) {
    if constexpr (sizeof(T) == sizeof(double)) {
        long long big = 0;
        for (int fam = 0; fam < 3; ++fam) {
            const long long nf = (long long)(d.A.Mx + (fam == 0)) * (d.A.My + (fam == 1)) * (d.A.Mz + (fam == 2));
            big = nf > big ? nf : big;
        }
        if (w.pieces64 && big < (1LL << 29)) return face_stage64(d, a, w, verts, wgt, acc, s);
    }
    return launch_faces_from<T>(d, a, w, verts, wgt, acc, s);
}

template <typename T>
cudaError_t launch_faces(const PassDesc& d, const T* a, const PassWork<T>& w, cudaStream_t s) {
    return faces_weighted<T>(d, a, w, w.verts, T(1), 0, s);
}

cudaError_t piece_store64_reserve(PieceStore64& p, long long pieces, long long faces_per_family) {
    cudaDeviceSynchronize();
    // ranges hold 31-bit starts
    if (pieces >= (1LL << 31)) pieces = (1LL << 31) - 1;
    if (pieces > p.cap) {
        cudaFree(p.rec); cudaFree(p.flux);
        p.rec = nullptr; p.flux = nullptr; p.cap = 0;
        cudaError_t e = cudaMalloc(&p.rec, pieces * sizeof(double4_32a));
        if (e == cudaSuccess) e = cudaMalloc(&p.flux, pieces * sizeof(double));
        if (e != cudaSuccess) return e;
        p.cap = pieces;
    }
    if (!p.count) {
        cudaError_t e = cudaMalloc(&p.count, 2 * sizeof(unsigned));
        if (e == cudaSuccess) e = cudaMalloc(&p.saved, 5 * sizeof(unsigned long long));
        if (e != cudaSuccess) return e;
    }
    if (!p.range[0]) {
        for (int f = 0; f < 3; ++f) {
            cudaError_t e = cudaMalloc(&p.range[f], faces_per_family * sizeof(int2));
            if (e != cudaSuccess) return e;
        }
        cudaError_t e = cudaMalloc(&p.deferred, 3 * faces_per_family * sizeof(int));
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void piece_store64_free(PieceStore64& p) {
    cudaFree(p.rec); cudaFree(p.flux); cudaFree(p.count); cudaFree(p.deferred); cudaFree(p.saved);
    for (int f = 0; f < 3; ++f) cudaFree(p.range[f]);
    p = PieceStore64();
}

template <typename T>
cudaError_t launch_gather(const PassDesc& d, const PassWork<T>& w, const T* in, T* out, int mode, cudaStream_t s) {
    const long long n = (long long)d.A.Mx * d.A.My * d.A.Mz;
    k_gather<T><<<blocks_for(n, 256), 256, 0, s>>>(d, w.flux[0], w.flux[1], w.flux[2], w.flux_rev[0],
                                                   w.flux_rev[1], w.flux_rev[2], in, out, mode);
    return cudaGetLastError();
}

template <typename T>
cudaError_t run_pass(const PassDesc& d, const VelocityFields& vel, const T* a, const PassWork<T>& w,
                     const T* in, T* out, int mode, cudaStream_t s) {
    cudaError_t e = launch_psi<T>(d, a, w.psi, s);
    if (e != cudaSuccess) return e;
    if (!d.zero_velocity) {
        e = launch_backtrace<T>(d, vel, w.verts, s);
        if (e != cudaSuccess) return e;
    }
    if (!d.maccormack || d.zero_velocity) {
        // one face per face slot; with zero velocity the MacCormack faces coincide and their
        // weights sum to one
        e = launch_faces<T>(d, a, w, s);
    } else {
        if (!w.verts2) return cudaErrorInvalidValue;
        const long long nv = (long long)(d.A.Mx + 1) * (d.A.My + 1) * (d.A.Mz + 1);
        k_forward_trace<T><<<blocks_for(nv, 128), 128, 0, s>>>(d, (const T*)vel.u, (const T*)vel.v, (const T*)vel.w,
                                                              vel.fu, vel.fv, vel.fw, w.verts, w.verts2);
        PassDesc rest = d;
        rest.zero_velocity = 1;
        e = faces_weighted<T>(rest, a, w, w.verts, T(0.5), 0, s);            // the face at rest
        if (e == cudaSuccess) e = faces_weighted<T>(d, a, w, w.verts, T(1), 1, s);   // backtraced
        if (e == cudaSuccess) e = faces_weighted<T>(d, a, w, w.verts2, T(-0.5), 1, s);   // traced back
    }
    if (e != cudaSuccess) return e;
    if (d.volumes) {
        if (!w.vol || !w.fvol[0]) return cudaErrorInvalidValue;
        const long long n = (long long)d.A.Mx * d.A.My * d.A.Mz;
        k_gather<T><<<blocks_for(n, 256), 256, 0, s>>>(d, w.fvol[0], w.fvol[1], w.fvol[2], w.fvol_rev[0],
                                                       w.fvol_rev[1], w.fvol_rev[2], nullptr, w.vol, 3);
    }
    return launch_gather<T>(d, w, in, out, mode, s);
}

template cudaError_t launch_psi<double>(const PassDesc&, const double*, double*, cudaStream_t);
template cudaError_t launch_backtrace<double>(const PassDesc&, const VelocityFields&, double*, cudaStream_t);
template cudaError_t launch_faces<double>(const PassDesc&, const double*, const PassWork<double>&, cudaStream_t);
template cudaError_t launch_gather<double>(const PassDesc&, const PassWork<double>&, const double*, double*, int, cudaStream_t);
template cudaError_t run_pass<double>(const PassDesc&, const VelocityFields&, const double*, const PassWork<double>&,
                                      const double*, double*, int, cudaStream_t);

}  // namespace fia
