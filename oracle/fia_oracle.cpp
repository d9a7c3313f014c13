// fia_oracle.cpp -- CPU restatement (FP64) of the flux-interpolated advection step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA library is checked
// against: only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
// legs load it.  The product path (libfia.so) never links, loads or calls it.
//
// It restates the reference program (nyhirasawa/Flux-Interpolated-Advection, the 3D
// branch) in double precision, following the structure of the reference closely:
// every cell enumerates its own six faces (as the reference does), every face
// backtraces its own four vertices, the clipper is the recursive iso-line cutter,
// and quadrature values are accumulated straight into the owning cell.  The GPU
// library restructures all of this (unique vertices, unique faces, deterministic
// gather); the two are independent implementations of the same arithmetic.
//
// Compiled with -ffp-contract=off so that x86-64 and aarch64 hosts round alike.
//
// Parity pinning: tests/golden/ holds outputs of the reference's own translation units
// (compiled from the reference sources by oracle/build_ref.sh); the oracle is checked
// against them in tests/test_oracle_golden.py.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <thread>
#include <algorithm>
#include <functional>

namespace {

typedef double real;

// ---------------------------------------------------------------------------------
// Grid description.  A "node field" is an array of M[0]*M[1]*M[2] values, z fastest,
// x slowest (utils.h:65-165 all use  Mz*(My*ix+iy)+iz ), whose node (i,j,k) sits at
// ((i+off[0])h, (j+off[1])h, (k+off[2])h).
//   density        M=(N,N,N)     off=(.5,.5,.5)   (grid_3d.h:42)
//   u (x-faces)    M=(N+1,N,N)   off=(0,.5,.5)    (grid_3d.cpp:30)
//   v (y-faces)    M=(N,N+1,N)   off=(.5,0,.5)
//   w (z-faces)    M=(N,N,N+1)   off=(.5,.5,0)
//   psi of a field with offsets off lives on its y-faces: M=(Mx,My+1,Mz), off-(0,.5,0)
// ---------------------------------------------------------------------------------
struct Field {
    const real* a;
    int M[3];
    real off[3];
};

inline long idx3(const int* M, int i, int j, int k) { return (long)M[2] * ((long)M[1] * i + j) + k; }
inline int clampi(int i, int lo, int hi) { return i < lo ? lo : (i > hi ? hi : i); }

// Values within a few units in the last place of an integer are taken as that integer.
// The scheme makes discrete decisions on exact integers (iso-line crossings of vertex
// colours, the cell holding a centroid); in exact arithmetic a vertex on the lattice or
// clamped to a wall has an integer colour, but n*h/h rounds to either side of n when h
// is not a power of two, and the resulting piece structure then flips under ulp-sized
// changes (measured: 1e-15 relative velocity noise moved a 9^3 error pass by 1e-6).
// The GPU library applies the same rule.
inline real snap_int(real x) {
    const real r = std::nearbyint(x);
    const real tol = 8.0 * 2.220446049250313e-16 * std::max(1.0, std::fabs(x));
    return std::fabs(x - r) <= tol ? r : x;
}

struct Grid {
    int N[3];
    real h;
};

// ----------------------------- Gauss-Legendre rule --------------------------------
// gauss_quadrature_points.cpp:18-33, :382-431: nodes on [-1,1] ordered centre first,
// then -/+ pairs by increasing |x|; weights normalised to sum 1.  The nodes are the
// roots of P_k found by Newton's method (our own computation from the definition).
struct Gauss1D {
    int k;
    real x[64];
    real w[64];
};

static void legendre(int n, real x, real* p, real* dp) {
    real p0 = 1.0, p1 = x;
    if (n == 0) { *p = 1.0; *dp = 0.0; return; }
    for (int m = 2; m <= n; ++m) {
        real p2 = ((2.0 * m - 1.0) * x * p1 - (m - 1.0) * p0) / m;
        p0 = p1; p1 = p2;
    }
    *p = p1;
    *dp = n * (x * p1 - p0) / (x * x - 1.0);
}

static Gauss1D make_gauss(int k) {
    Gauss1D g; g.k = k;
    std::vector<std::pair<real, real>> nodes;
    const real pi = 3.14159265358979323846;
    for (int i = 0; i < (k + 1) / 2; ++i) {
        real x = std::cos(pi * (i + 0.75) / (k + 0.5));
        for (int it = 0; it < 100; ++it) {
            real p, dp; legendre(k, x, &p, &dp);
            real dx = p / dp; x -= dx;
            if (std::fabs(dx) < 1e-17) break;
        }
        real p, dp; legendre(k, x, &p, &dp);
        real w = 2.0 / ((1.0 - x * x) * dp * dp);
        if (std::fabs(x) < 1e-15) { nodes.push_back({0.0, w}); }
        else { nodes.push_back({-std::fabs(x), w}); nodes.push_back({std::fabs(x), w}); }
    }
    std::stable_sort(nodes.begin(), nodes.end(), [](const std::pair<real,real>& a, const std::pair<real,real>& b) {
        return std::fabs(a.first) < std::fabs(b.first);
    });
    for (int i = 0; i < k; ++i) { g.x[i] = nodes[i].first; g.w[i] = nodes[i].second / 2.0; }
    return g;
}

// positions of the rule on [a,b]  (gauss_quadrature_points.cpp:419-428)
inline real gauss_pos(const Gauss1D& g, int q, real a, real b) {
    real L = b - a;
    return (L / 2.0) * g.x[q] + (L / 2.0) + a;
}

// --------------------------------- WENO6 ------------------------------------------
// One 1D WENO6 interpolation on 6 samples f[0..5] with signed distances d[i]=p-x_i
// (WENO6_interpolation_3d.cpp:70-123): three cubic candidates, ideal weights from the
// distances, smoothness indicators with integer coefficients over 180, and
// alpha = C / (eps + beta)^2 with eps = 1e-6.
inline real weno6_1d(const real* f, const real* d, real h) {
    real cand[3];
    for (int i = 0; i < 3; ++i) {
        cand[i] = f[i]
            + (f[i + 1] - f[i]) * d[i] / (h)
            + (f[i + 2] - 2 * f[i + 1] + f[i]) * d[i] * d[i + 1] / (2 * h * h)
            + (f[i + 3] - 3 * f[i + 2] + 3 * f[i + 1] - f[i]) * d[i] * d[i + 1] * d[i + 2] / (6 * h * h * h);
    }
    real C[3];
    C[0] = d[4] * d[5] / (20 * h * h);
    C[1] = -d[5] * d[0] / (10 * h * h);
    C[2] = d[0] * d[1] / (20 * h * h);
    real b[3];
    b[0] = (-3579 * f[3] * f[2] + 2634 * f[3] * f[1] - 683 * f[3] * f[0]
            - 6927 * f[2] * f[1] + 1854 * f[2] * f[0] - 1659 * f[1] * f[0]
            + 814 * f[3] * f[3] + 4326 * f[2] * f[2] + 2976 * f[1] * f[1]
            + 244 * f[0] * f[0]) / 180.0;
    b[1] = (-3777 * f[3] * f[2] + 1074 * f[3] * f[1] - 1269 * f[2] * f[1]
            + 1986 * f[3] * f[3] + 1986 * f[2] * f[2] + 244 * f[1] * f[1]
            + 244 * f[4] * f[4] - 1269 * f[4] * f[3] + 1074 * f[4] * f[2]
            - 293 * f[4] * f[1]) / 180.0;
    b[2] = (-3579 * f[3] * f[2] + 4326 * f[3] * f[3] + 814 * f[2] * f[2]
            + 2976 * f[4] * f[4] + 244 * f[5] * f[5] - 683 * f[5] * f[2]
            - 6927 * f[4] * f[3] + 2634 * f[4] * f[2] - 1659 * f[5] * f[4]
            + 1854 * f[5] * f[3]) / 180.0;
    real alpha[3];
    for (int i = 0; i < 3; ++i) {
        real eps = 0.000001;
        alpha[i] = C[i] / ((eps + b[i]) * (eps + b[i]));
    }
    real wsum = alpha[0] + alpha[1] + alpha[2];
    real w0 = alpha[0] / wsum, w1 = alpha[1] / wsum, w2 = alpha[2] / wsum;
    return w0 * cand[0] + w1 * cand[1] + w2 * cand[2];
}

// Tensor-product WENO6 (z, then y, then x) of a node field at p, stencil indices
// clamped to the array (WENO6_interpolation_3d.cpp:7-258 and the face variants).
static real weno6_3d(const Field& F, const real* p, real h) {
    int base[3];
    for (int d = 0; d < 3; ++d) base[d] = (int)std::floor((p[d] - F.off[d] * h) / h);
    real dist[3][6];
    for (int d = 0; d < 3; ++d)
        for (int i = 0; i < 6; ++i) dist[d][i] = p[d] - (base[d] - 2 + i + F.off[d]) * h;
    real zv[6][6];
    for (int ix = 0; ix < 6; ++ix) {
        int ii = clampi(base[0] - 2 + ix, 0, F.M[0] - 1);
        for (int iy = 0; iy < 6; ++iy) {
            int jj = clampi(base[1] - 2 + iy, 0, F.M[1] - 1);
            real f[6];
            for (int iz = 0; iz < 6; ++iz) {
                int kk = clampi(base[2] - 2 + iz, 0, F.M[2] - 1);
                f[iz] = F.a[idx3(F.M, ii, jj, kk)];
            }
            zv[ix][iy] = weno6_1d(f, dist[2], h);
        }
    }
    real yv[6];
    for (int ix = 0; ix < 6; ++ix) yv[ix] = weno6_1d(zv[ix], dist[1], h);
    return weno6_1d(yv, dist[0], h);
}

// WENO6 along y only; x and z pick the node whose cell holds p
// (WENO6_interpolation_1d.cpp:315-430:  index_x = floor(p_x/h) for cell centres).
static real weno6_1dy(const Field& F, const real* p, real h) {
    int ix = clampi((int)std::floor(snap_int((p[0] - (F.off[0] * h - 0.5 * h)) / h)), 0, F.M[0] - 1);
    int iz = clampi((int)std::floor(snap_int((p[2] - (F.off[2] * h - 0.5 * h)) / h)), 0, F.M[2] - 1);
    int base = (int)std::floor((p[1] - F.off[1] * h) / h);
    real d[6], f[6];
    for (int i = 0; i < 6; ++i) {
        d[i] = p[1] - (base - 2 + i + F.off[1]) * h;
        f[i] = F.a[idx3(F.M, ix, clampi(base - 2 + i, 0, F.M[1] - 1), iz)];
    }
    return weno6_1d(f, d, h);
}

// Trilinear interpolation with clamped indices (linear_interpolation_3d.cpp:7-95).
static real lin3d(const Field& F, const real* p, real h) {
    int base[3]; real t[3];
    for (int d = 0; d < 3; ++d) {
        real o = F.off[d] * h;
        base[d] = (int)std::floor((p[d] - o) / h);
        t[d] = (p[d] - o) / h - base[d];
    }
    real zv[2][2];
    for (int ix = 0; ix < 2; ++ix)
        for (int iy = 0; iy < 2; ++iy) {
            int ii = clampi(base[0] + ix, 0, F.M[0] - 1), jj = clampi(base[1] + iy, 0, F.M[1] - 1);
            real f0 = F.a[idx3(F.M, ii, jj, clampi(base[2], 0, F.M[2] - 1))];
            real f1 = F.a[idx3(F.M, ii, jj, clampi(base[2] + 1, 0, F.M[2] - 1))];
            zv[ix][iy] = (1.0 - t[2]) * f0 + t[2] * f1;
        }
    real yv[2];
    for (int ix = 0; ix < 2; ++ix) yv[ix] = (1.0 - t[1]) * zv[ix][0] + t[1] * zv[ix][1];
    return (1.0 - t[0]) * yv[0] + t[0] * yv[1];
}

// Linear along y, nearest cell in x and z (linear_interpolation_1d.cpp:314-374).
static real lin1dy(const Field& F, const real* p, real h) {
    int ix = clampi((int)std::floor(snap_int((p[0] - (F.off[0] * h - 0.5 * h)) / h)), 0, F.M[0] - 1);
    int iz = clampi((int)std::floor(snap_int((p[2] - (F.off[2] * h - 0.5 * h)) / h)), 0, F.M[2] - 1);
    real o = F.off[1] * h;
    int base = (int)std::floor((p[1] - o) / h);
    real f0 = F.a[idx3(F.M, ix, clampi(base, 0, F.M[1] - 1), iz)];
    real f1 = F.a[idx3(F.M, ix, clampi(base + 1, 0, F.M[1] - 1), iz)];
    real b0 = (p[1] - o) / h - base;
    return (1.0 - b0) * f0 + b0 * f1;
}

enum Interp { I_WENO6 = 0, I_LINEAR = 1, I_1DY_LINEAR = 2 };

static real interp(int method, const Field& F, const real* p, real h) {
    if (method == I_WENO6) return weno6_3d(F, p, h);
    if (method == I_LINEAR) return lin3d(F, p, h);
    return lin1dy(F, p, h);
}

// ------------------------------------ psi ------------------------------------------
// psi of a node field F along y: psi(.,0,.) = 0, psi(.,j,.) = psi(.,j-1,.) + increment.
//   plain   : + F(.,j-1,.) h                     (calc_psi_3D.cpp:274-306, :520-535)
//   WENO6   : + sum over two half cells, k Gauss points each, of the 1Dy-WENO6
//             interpolant times h/2 w_q          (calc_psi_3D.cpp:177-272)
//   linear  : + trilinear at 1/4 and 3/4 of the cell, times h/2  (calc_psi_3D.cpp:92-131)
enum PsiMode { PSI_PLAIN = 0, PSI_WENO6 = 1, PSI_LINEAR = 2 };

// Columns [xlo, xhi) only (xhi < 0: all); the others stay zero (the bounded CPU baseline
// computes the columns its cells read).
static void compute_psi(const Field& F, real h, int mode, const Gauss1D& g, std::vector<real>& psi, int xlo = 0,
                        int xhi = -1) {
    int Mp[3] = {F.M[0], F.M[1] + 1, F.M[2]};
    psi.assign((size_t)Mp[0] * Mp[1] * Mp[2], 0.0);
    if (xhi < 0 || xhi > Mp[0]) xhi = Mp[0];
    if (xlo < 0) xlo = 0;
    for (int j = 1; j < Mp[1]; ++j)
        for (int i = xlo; i < xhi; ++i)
            for (int k = 0; k < Mp[2]; ++k) {
                real acc = psi[idx3(Mp, i, j - 1, k)];
                if (mode == PSI_PLAIN) {
                    acc = acc + F.a[idx3(F.M, i, j - 1, k)] * h;
                } else if (mode == PSI_WENO6) {
                    // cell j-1 spans [(j-1+off_y-0.5)h, (j+off_y-0.5)h]
                    real ylo = (j - 1.0 + F.off[1] - 0.5) * h;
                    real ymid = (j - 0.5 + F.off[1] - 0.5) * h;
                    real yhi = (j + F.off[1] - 0.5) * h;
                    real p[3] = {(i + F.off[0]) * h, 0.0, (k + F.off[2]) * h};
                    for (int q = 0; q < g.k; ++q) {
                        p[1] = gauss_pos(g, q, ylo, ymid);
                        acc += weno6_1dy(F, p, h) * (h / 2.0) * g.w[q];
                    }
                    for (int q = 0; q < g.k; ++q) {
                        p[1] = gauss_pos(g, q, ymid, yhi);
                        acc += weno6_1dy(F, p, h) * (h / 2.0) * g.w[q];
                    }
                } else {
                    real p0[3] = {(i + F.off[0]) * h, ((j - 1) + 0.25 + F.off[1] - 0.5) * h, (k + F.off[2]) * h};
                    real p1[3] = {(i + F.off[0]) * h, ((j - 1) + 0.75 + F.off[1] - 0.5) * h, (k + F.off[2]) * h};
                    real a0 = lin3d(F, p0, h), a1 = lin3d(F, p1, h);
                    acc = acc + a0 * (h / 2.0) + a1 * (h / 2.0);
                }
                psi[idx3(Mp, i, j, k)] = acc;
            }
}

// ------------------------------- face clipping -------------------------------------
// The clipper of facecutter.h:59-324 restated in double: a quad in (xi,eta) space with
// a two-component "colour" per vertex is cut at interior integer iso-lines of colour
// component 0 (smallest first, recursively), then of component 1; pieces with
// non-zero area are emitted with their centroid.
struct V2 { real p[2]; real c[2]; };
typedef std::function<void(const real (*pts)[2], int num, const real* ctr)> PolyOut;

// multi: some cut produced more than one part on the far side of its iso-line (the line
// crossed the polygon more than twice), so the partition depends on the vertex order
struct ClipStatus { int overflow = 0; int odd_cut = 0; int multi = 0; };

static void cut_face_rec(const V2* poly, int num, int dim, const std::function<void(const V2*, int)>& out, ClipStatus& st) {
    real mn = 1e308, mx = -1e308;
    for (int n = 0; n < num; ++n) { mn = std::min(mn, poly[n].c[dim]); mx = std::max(mx, poly[n].c[dim]); }
    int start = (int)std::ceil(mn), end = (int)std::floor(mx);
    if (mn - start == 0.0) start += 1;
    if (mx - end == 0.0) end -= 1;
    bool cut = false;
    if (start <= end) {
        const real iso = start;
        V2 arr[2][40];
        int head[2] = {0, 0};
        int slot = 0, parts = 0;
        arr[0][head[0]++] = poly[0];
        for (int n = 0; n < num; ++n) {
            int m = (n + 1) % num;
            real v0 = poly[n].c[dim] - iso, v1 = poly[m].c[dim] - iso;
            if ((v0 < 0.0) != (v1 < 0.0)) {
                real inv = 1.0 / (v1 - v0);
                real t0 = v1 * inv, t1 = -v0 * inv;
                cut = true;
                V2 add;
                add.p[0] = t0 * poly[n].p[0] + t1 * poly[m].p[0];
                add.p[1] = t0 * poly[n].p[1] + t1 * poly[m].p[1];
                add.c[dim] = iso;
                add.c[1 - dim] = snap_int(t0 * poly[n].c[1 - dim] + t1 * poly[m].c[1 - dim]);
                if (slot == 0) {
                    arr[0][head[0]++] = add;
                    slot = 1; head[1] = 0;
                    if (t1 < 1.0) arr[1][head[1]++] = add;
                } else {
                    arr[1][head[1]++] = add;
                    if (head[1] > 32) { st.overflow = 1; return; }
                    if (++parts > 1) st.multi = 1;
                    cut_face_rec(arr[1], head[1], dim, out, st);
                    slot = 0;
                    if (t1 < 1.0) arr[0][head[0]++] = add;
                }
            }
            if (n < num - 1) arr[slot][head[slot]++] = poly[m];
            if (head[0] >= 32 || head[1] >= 32) { st.overflow = 1; return; }
        }
        if (cut) {
            if (slot != 0) { st.odd_cut = 1; return; }
            cut_face_rec(arr[0], head[0], dim, out, st);
        }
    }
    if (!cut) {
        if (dim == 0) cut_face_rec(poly, num, 1, out, st);
        else out(poly, num);
    }
}

static void center_of_gravity(const real (*pts)[2], int num, real* ctr, real* area) {
    ctr[0] = ctr[1] = 0.0; real a = 0.0;
    for (int n = 0; n < num; ++n) {
        const real* p0 = pts[n]; const real* p1 = pts[(n + 1) % num];
        real c = p0[0] * p1[1] - p1[0] * p0[1];
        a += c;
        ctr[0] += c * (p0[0] + p1[0]);
        ctr[1] += c * (p0[1] + p1[1]);
    }
    a = std::fabs(0.5 * a);
    if (a != 0.0) {
        real s = 1.0 / (6.0 * a);
        ctr[0] = ctr[0] * s; ctr[1] = ctr[1] * s;
    } else {
        ctr[0] = ctr[1] = 0.0;
        for (int n = 0; n < num; ++n) { ctr[0] = ctr[0] + pts[n][0]; ctr[1] = ctr[1] + pts[n][1]; }
        real s = 1.0 / num;
        ctr[0] = ctr[0] * s; ctr[1] = ctr[1] * s;
    }
    *area = a;
}

// facecutter.h:255-324; with the default minimal_area (1.0) a polygon is emitted as is.  The
// longest edge is the first of the longest: edges whose squared lengths agree to within a
// relative 4e-6 count as equally long (equal in exact arithmetic they are, as in a fan triangle
// of a square, whose rounding would otherwise pick the edge differently in every precision;
// the GPU library applies the same rule in both forms).
constexpr real kLongestEdgeTie = 4e-6;
static void subdivide(const real (*poly)[2], int num, real minimal_area, const PolyOut& out) {
    std::function<void(const real (*)[2])> tri_split = [&](const real (*t)[2]) {
        real ctr[2], area;
        center_of_gravity(t, 3, ctr, &area);
        if (area > minimal_area) {
            int maxi = 0; real maxlen = -1e308;
            for (int n = 0; n < 3; ++n) {
                real dx = t[n][0] - t[(n + 1) % 3][0], dy = t[n][1] - t[(n + 1) % 3][1];
                real len = dx * dx + dy * dy;
                if (len > maxlen * (1.0 + kLongestEdgeTie)) { maxlen = len; maxi = n; }
            }
            const real* p0 = t[maxi]; const real* p1 = t[(maxi + 1) % 3]; const real* p2 = t[(maxi + 2) % 3];
            real mid[2] = {0.5 * (p0[0] + p1[0]), 0.5 * (p0[1] + p1[1])};
            real t0[3][2] = {{p0[0], p0[1]}, {mid[0], mid[1]}, {p2[0], p2[1]}};
            real t1[3][2] = {{mid[0], mid[1]}, {p1[0], p1[1]}, {p2[0], p2[1]}};
            tri_split(t0); tri_split(t1);
        } else if (area != 0.0) {
            out(t, 3, ctr);
        }
    };
    if (num == 3) { tri_split(poly); return; }
    real ctr[2], area;
    center_of_gravity(poly, num, ctr, &area);
    if (area > minimal_area) {
        for (int n = 0; n < num; ++n) {
            real t[3][2] = {{ctr[0], ctr[1]}, {poly[n][0], poly[n][1]}, {poly[(n + 1) % num][0], poly[(n + 1) % num][1]}};
            tri_split(t);
        }
    } else if (area != 0.0) {
        out(poly, num, ctr);
    }
}

// Bilinear map of the backtraced face (cell_face_3D.cpp:54-59), evaluated in the
// equivalent form v0 + xi (v1-v0) + eta (v3-v0) + xi eta (v0-v1+v2-v3).  Where all four
// vertices share a coordinate (a face lying in a grid plane: zero-velocity passes, wall
// faces, clamped faces) this returns that coordinate exactly, so the quadrature branch
// taken on floor(y/h) does not depend on how xi and eta were rounded.  The reference's
// weighted-sum form rounds such centroids to either side of the plane (its own float and
// double builds disagree there); the GPU library uses this same form.
inline void bilinear(const real (*v)[3], real xi, real eta, real* out) {
    for (int d = 0; d < 3; ++d) {
        real a = v[1][d] - v[0][d], b = v[3][d] - v[0][d], c = (v[0][d] - v[1][d]) + (v[2][d] - v[3][d]);
        out[d] = v[0][d] + xi * a + eta * b + (xi * eta) * c;
    }
}

inline void cross(const real* a, const real* b, real* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// split_face_3D.cpp:17-93: colours from the split method, clip, and per piece the 3D
// centroid position and the scaled normal.
struct SubPoly { real pos[3]; real n[3]; };

static int split_face(const real (*v)[3], real h, const real* color_off, real minimal_area,
                      std::vector<SubPoly>& outv, int* multi = nullptr) {
    V2 quad[4];
    const real xi[4][2] = {{0.0, 0.0}, {1.0, 0.0}, {1.0, 1.0}, {0.0, 1.0}};
    for (int i = 0; i < 4; ++i) {
        quad[i].p[0] = xi[i][0]; quad[i].p[1] = xi[i][1];
        quad[i].c[0] = snap_int(v[i][0] / h - color_off[0]);
        quad[i].c[1] = snap_int(v[i][2] / h - color_off[1]);
    }
    ClipStatus st;
    cut_face_rec(quad, 4, 0, [&](const V2* poly, int num) {
        if (num >= 3) {
            real tmp[40][2];
            for (int i = 0; i < num; ++i) { tmp[i][0] = poly[i].p[0]; tmp[i][1] = poly[i].p[1]; }
            subdivide(tmp, num, minimal_area, [&](const real (*pts)[2], int n, const real* ctr) {
                SubPoly sp;
                bilinear(v, ctr[0], ctr[1], sp.pos);
                real P[40][3];
                for (int i = 0; i < n; ++i) bilinear(v, pts[i][0], pts[i][1], P[i]);
                if (n == 3) {
                    real a[3], b[3], c[3];
                    for (int d = 0; d < 3; ++d) { a[d] = P[1][d] - P[0][d]; b[d] = P[2][d] - P[0][d]; }
                    cross(a, b, c);
                    for (int d = 0; d < 3; ++d) sp.n[d] = 0.5 * c[d];
                } else {
                    real acc[3] = {0.0, 0.0, 0.0};
                    for (int i = 0; i < n; ++i) {
                        real a[3], b[3], c[3];
                        for (int d = 0; d < 3; ++d) { a[d] = P[i][d] - sp.pos[d]; b[d] = P[(i + 1) % n][d] - sp.pos[d]; }
                        cross(a, b, c);
                        for (int d = 0; d < 3; ++d) acc[d] += c[d];
                    }
                    for (int d = 0; d < 3; ++d) sp.n[d] = acc[d] * 0.5;
                }
                outv.push_back(sp);
            });
        }
    }, st);
    if (multi) *multi = st.multi;
    return (st.overflow ? 1 : 0) | (st.odd_cut ? 2 : 0);
}

// ----------------------------------- one pass ---------------------------------------
// Face vertex tables, cell-relative (backtrace_...for_integrate_density.cpp:77-112).
static const int kFaceVerts[6][4][3] = {
    {{0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}},   // 0: z-
    {{1, 0, 0}, {1, 1, 0}, {1, 1, 1}, {1, 0, 1}},   // 1: x+
    {{0, 1, 0}, {0, 1, 1}, {1, 1, 1}, {1, 1, 0}},   // 2: y+
    {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0}},   // 3: x-
    {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}},   // 4: y-
    {{0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}},   // 5: z+
};

struct PassParams {
    int comp;            // -1 density, 0/1/2 velocity component (pin rule + staggering)
    int interp;          // Interp: velocity for the backtrace, values and psi
    int psi_mode;        // PsiMode
    int use_integral;    // 1: density-integral quadrature (A6), 0: psi at centroid only
    int zero_velocity;   // backtrace skipped
    real color_off[2];   // split method: 0.5 = CellFaceAligned, 0.0 = AxisAligned (x, z)
    int k;               // Gauss points per half cell
    real minimal_area;
    real dt;
    int maccormack = 0;  // flux MacCormack: faces at rest (0.5), backtraced (1), traced back (-0.5)
};

struct Velocity { Field u, v, w; };

// Backtrace one vertex (calc_backtraced_face_3D.cpp:9-160).
static void backtrace_vertex(const Grid& G, const Velocity& vel, const PassParams& P,
                             const int* vidx, real* pos) {
    real h = G.h;
    for (int d = 0; d < 3; ++d) {
        pos[d] = vidx[d] * h;
        if (d == P.comp) pos[d] -= 1 * 0.5 * h;
    }
    if (P.zero_velocity) return;
    bool pinned = false;
    if (P.comp >= 0) {
        int c = P.comp;
        if (vidx[c] <= 1 || vidx[c] >= G.N[c]) pinned = true;
    }
    real u[3];
    u[0] = interp(P.interp, vel.u, pos, h);
    u[1] = interp(P.interp, vel.v, pos, h);
    u[2] = interp(P.interp, vel.w, pos, h);
    if (!pinned) {
        for (int d = 0; d < 3; ++d) pos[d] -= u[d] * P.dt;
    }
    for (int d = 0; d < 3; ++d) {
        int e = (d == P.comp);
        real lo = 0.0 - e * 0.5 * h;
        real hi = 0.0 + h * G.N[d] + e * 0.5 * h;
        if (pos[d] < lo) pos[d] = lo;
        if (pos[d] > hi) pos[d] = hi;
    }
}

// Second trace of the flux MacCormack scheme (calc_backtraced_face_3D.cpp:9-128 with
// time_direction "backward"): from the backtraced position x1, x2 = x1 + dt u(x1) with the
// velocity interpolated at x1, the same pin rule (by the vertex's lattice index), then clamped
// (clamp_vertex_position_by_grid_3D, :131-160).
static void forward_trace_vertex(const Grid& G, const Velocity& vel, const PassParams& P, const int* vidx,
                                 const real* x1, real* pos) {
    const real h = G.h;
    for (int d = 0; d < 3; ++d) pos[d] = x1[d];
    if (P.zero_velocity) return;
    bool pinned = false;
    if (P.comp >= 0) {
        int c = P.comp;
        if (vidx[c] <= 1 || vidx[c] >= G.N[c]) pinned = true;
    }
    real u[3];
    u[0] = interp(P.interp, vel.u, x1, h);
    u[1] = interp(P.interp, vel.v, x1, h);
    u[2] = interp(P.interp, vel.w, x1, h);
    if (!pinned) {
        for (int d = 0; d < 3; ++d) pos[d] += u[d] * P.dt;
    }
    for (int d = 0; d < 3; ++d) {
        int e = (d == P.comp);
        real lo = 0.0 - e * 0.5 * h;
        real hi = 0.0 + h * G.N[d] + e * 0.5 * h;
        if (pos[d] < lo) pos[d] = lo;
        if (pos[d] > hi) pos[d] = hi;
    }
}

struct PassCounters { long faces = 0; long polys = 0; int status = 0; };

// One flux pass over the cells [c0, c1) of the advected field A (node field of the
// advected quantity), writing out[cell] for those cells.
static void pass_range(const Grid& G, const Velocity& vel, const Field& A, const Field& Psi,
                       const PassParams& P, const Gauss1D& g, real* out, long c0, long c1,
                       PassCounters& cnt, real* vol) {
    const real h = G.h;
    const real V = h * h * h;
    const int* M = A.M;
    real origin[3] = {0.0, 0.0, 0.0};
    if (P.comp >= 0) origin[P.comp] = -1 * 0.5 * h;
    std::vector<SubPoly> polys;
    for (long cell = c0; cell < c1; ++cell) {
        int iz = (int)(cell % M[2]);
        int iy = (int)((cell / M[2]) % M[1]);
        int ix = (int)(cell / ((long)M[2] * M[1]));
        real acc = 0.0, vacc = 0.0;
        for (int f = 0; f < 6; ++f) {
            real vb[4][3], v0[4][3], v2[4][3];
            for (int q = 0; q < 4; ++q) {
                int vi[3] = {ix + kFaceVerts[f][q][0], iy + kFaceVerts[f][q][1], iz + kFaceVerts[f][q][2]};
                backtrace_vertex(G, vel, P, vi, vb[q]);
                if (P.maccormack) {
                    // the face before the backtrace (backtrace_..._for_integrate_density.cpp:139-144)
                    for (int d = 0; d < 3; ++d) v0[q][d] = vi[d] * h - ((d == P.comp) ? 1 * 0.5 * h : 0.0);
                    forward_trace_vertex(G, vel, P, vi, vb[q], v2[q]);
                }
            }
            // the flux MacCormack branch adds the quadrature of three faces with weights 0.5, 1
            // and -0.5 (backtrace_..._for_integrate_density.cpp:146-234); otherwise one face
            const int nstage = P.maccormack ? 3 : 1;
            for (int stage = 0; stage < nstage; ++stage) {
            const real (*v)[3] = !P.maccormack ? vb : (stage == 0 ? v0 : (stage == 1 ? vb : v2));
            const real wgt = !P.maccormack ? 1.0 : (stage == 0 ? 0.5 : (stage == 1 ? 1.0 : -0.5));
            polys.clear();
            cnt.status |= split_face(v, h, P.color_off, P.minimal_area, polys);
            cnt.faces++;
            cnt.polys += (long)polys.size();
            for (const SubPoly& sp : polys) {
                // the volume point of the piece (polygon_3D.cpp:480-486): y n_y summed per cell
                // (calc_density_in_cell_from_quadrature_point_list.cpp:135-156)
                vacc += sp.pos[1] * (sp.n[1] * wgt);
                if (P.use_integral) {
                    // polygon_3D.cpp:257-487
                    const real ry = snap_int((sp.pos[1] - origin[1]) / h);
                    int iy0 = (int)std::floor(ry);
                    real f01 = ry - iy0;
                    real q[3] = {sp.pos[0], 0.0, sp.pos[2]};
                    if (f01 < 0.5) {
                        real a = iy0 * h + origin[1], b = sp.pos[1];
                        for (int t = 0; t < g.k; ++t) {
                            q[1] = gauss_pos(g, t, a, b);
                            real wy = sp.n[1] * f01 * h * g.w[t] * wgt;
                            acc += interp(P.interp, A, q, h) * wy / V;
                        }
                    } else {
                        real a = iy0 * h + origin[1], b = (iy0 + 0.5) * h + origin[1];
                        for (int t = 0; t < g.k; ++t) {
                            q[1] = gauss_pos(g, t, a, b);
                            real wy = sp.n[1] * 0.5 * h * g.w[t] * wgt;
                            acc += interp(P.interp, A, q, h) * wy / V;
                        }
                        a = (iy0 + 0.5) * h + origin[1]; b = (iy0 + f01) * h + origin[1];
                        for (int t = 0; t < g.k; ++t) {
                            q[1] = gauss_pos(g, t, a, b);
                            real wy = sp.n[1] * (f01 - 0.5) * h * g.w[t] * wgt;
                            acc += interp(P.interp, A, q, h) * wy / V;
                        }
                    }
                    real qp[3] = {sp.pos[0], iy0 * h + origin[1], sp.pos[2]};
                    acc += interp(P.interp, Psi, qp, h) * (sp.n[1] * wgt) / V;
                } else {
                    // calc_density_in_cell_from_quadrature_point_list.cpp:101-131
                    acc += interp(P.interp, Psi, sp.pos, h) * (sp.n[1] * wgt) / V;
                }
            }
            }
        }
        out[cell] = acc;
        if (vol) vol[cell] = vacc;
    }
}

static int run_pass(const Grid& G, const Velocity& vel, const Field& A, const PassParams& P,
                    real* out, int nthreads, long c0, long c1, long* faces, long* polys, real* vol = nullptr,
                    int psi_x0 = 0, int psi_x1 = -1) {
    Gauss1D g = make_gauss(P.k);
    std::vector<real> psi;
    compute_psi(A, G.h, P.psi_mode, g, psi, psi_x0, psi_x1);
    Field Psi;
    Psi.a = psi.data();
    Psi.M[0] = A.M[0]; Psi.M[1] = A.M[1] + 1; Psi.M[2] = A.M[2];
    Psi.off[0] = A.off[0]; Psi.off[1] = A.off[1] - 0.5; Psi.off[2] = A.off[2];
    long ncell = (long)A.M[0] * A.M[1] * A.M[2];
    if (c1 < 0 || c1 > ncell) c1 = ncell;
    if (c0 < 0) c0 = 0;
    if (nthreads < 1) nthreads = 1;
    std::vector<PassCounters> cnt(nthreads);
    std::vector<std::thread> th;
    long span = c1 - c0;
    for (int t = 0; t < nthreads; ++t) {
        long a = c0 + span * t / nthreads, b = c0 + span * (t + 1) / nthreads;
        th.emplace_back([&, a, b, t]() { pass_range(G, vel, A, Psi, P, g, out, a, b, cnt[t], vol); });
    }
    for (auto& x : th) x.join();
    int status = 0; long nf = 0, np = 0;
    for (auto& c : cnt) { status |= c.status; nf += c.faces; np += c.polys; }
    if (faces) *faces = nf;
    if (polys) *polys = np;
    return status;
}

static Field make_field(const real* a, const Grid& G, int comp) {
    Field F; F.a = a;
    for (int d = 0; d < 3; ++d) { F.M[d] = G.N[d] + (d == comp); F.off[d] = (d == comp) ? 0.0 : 0.5; }
    return F;
}

static Velocity make_velocity(const Grid& G, const real* u, const real* v, const real* w) {
    Velocity vel; vel.u = make_field(u, G, 0); vel.v = make_field(v, G, 1); vel.w = make_field(w, G, 2);
    return vel;
}

// Split offsets (colour = position/h - off) per field for the main pass and the
// error-advection pass (move_substances_3d.cpp:189, advect_velocity_flux_advection_3d.cpp:622-628,
// :721, :805-810, :913, :999-1002, :1096).
static void split_offsets(int comp, int error_pass, const real* density_main, real* off) {
    if (comp < 0) {
        if (error_pass) { off[0] = 0.0; off[1] = 0.0; }
        else { off[0] = density_main[0]; off[1] = density_main[1]; }
        return;
    }
    // main pass: cut where psi of the component lives; error pass: the other lines
    real main_x = (comp == 0) ? 0.0 : 0.5;
    real main_z = (comp == 2) ? 0.0 : 0.5;
    if (!error_pass) { off[0] = main_x; off[1] = main_z; }
    else {
        if (comp == 1) { off[0] = 0.0; off[1] = 0.0; }
        else { off[0] = 0.5 - main_x; off[1] = 0.5 - main_z; }
    }
}

// CG on -A (the reference operator, last cell pinned): A p = b to a relative residual tol.
static int solve_A(const int* N, const real* b, real* p, real tol, int maxit);

// Cell-volume correction (move_substances_3d.cpp:243-493): A p = -(V - V0) on the pinned
// operator, then density moves between face neighbours by -(p_hi - p_lo) / V0 times the mean
// of their densities before the correction, x faces, then y, then z.  The reference stops
// its AMG-CG at a relative residual of 0.1 (:363); here the solve is run to 1e-13, the
// correction that the reference approximates.
static void volume_correction(const Grid& G, real* rho, const real* vol) {
    const int* N = G.N;
    const long n = (long)N[0] * N[1] * N[2];
    const real V0 = G.h * G.h * G.h;
    std::vector<real> b(n), p(n), before(rho, rho + n);
    for (long c = 0; c < n - 1; ++c) b[c] = -(vol[c] - V0);
    b[n - 1] = 0.0;
    solve_A(N, b.data(), p.data(), 1e-13, 100000);
    const long st[3] = {(long)N[1] * N[2], (long)N[2], 1};
    for (int a = 0; a < 3; ++a)
        for (int ix = 0; ix < N[0]; ++ix) for (int iy = 0; iy < N[1]; ++iy) for (int iz = 0; iz < N[2]; ++iz) {
            const int id[3] = {ix, iy, iz};
            if (id[a] < 1) continue;
            const long c = idx3(N, ix, iy, iz), cm = c - st[a];
            const real flux = -(p[c] - p[cm]) / V0;
            const real dens = (before[cm] * V0 + before[c] * V0) / (2.0 * V0);
            rho[cm] -= 1.0 * flux * dens;
            rho[c] += 1.0 * flux * dens;
        }
}

// move_substances_3d.cpp:38-240 (density) and advect_velocity_..._3D_std_thread for one
// velocity component: pass 1 (+ the zero-velocity / error-advection correction).
static int advect_field(const Grid& G, const Velocity& vel, int comp, const real* in, real* out,
                        real dt, int interp_method, int k, int correction, int use_integral,
                        const real* density_split, real minimal_area, int nthreads,
                        long* faces, long* polys, int maccormack, int volume = 0) {
    Field A = make_field(in, G, comp);
    if (comp < 0) { for (int d = 0; d < 3; ++d) { A.M[d] = G.N[d]; A.off[d] = 0.5; } }
    long n = (long)A.M[0] * A.M[1] * A.M[2];
    PassParams P;
    P.comp = comp; P.interp = interp_method; P.k = k; P.minimal_area = minimal_area; P.dt = dt;
    P.psi_mode = use_integral ? (interp_method == I_WENO6 ? PSI_WENO6 : PSI_LINEAR) : PSI_PLAIN;
    P.use_integral = use_integral; P.zero_velocity = 0; P.maccormack = maccormack;
    split_offsets(comp, 0, density_split, P.color_off);
    std::vector<real> vol(volume && comp < 0 ? n : 0);
    int status = run_pass(G, vel, A, P, out, nthreads, 0, n, faces, polys, vol.empty() ? nullptr : vol.data());
    if (!vol.empty()) volume_correction(G, out, vol.data());
    if (!correction) return status;
    // pass 2: zero velocity, no integral, plain psi
    std::vector<real> c(n);
    P.zero_velocity = 1; P.use_integral = 0; P.psi_mode = PSI_PLAIN;
    status |= run_pass(G, vel, A, P, c.data(), nthreads, 0, n, nullptr, nullptr);
    for (long i = 0; i < n; ++i) c[i] = in[i] - c[i];
    // pass 3: error advection with 1Dy-linear interpolation, plain psi, error split
    Field C = A; C.a = c.data();
    std::vector<real> c2(n);
    P.zero_velocity = 0; P.use_integral = 0; P.psi_mode = PSI_PLAIN; P.interp = I_1DY_LINEAR;
    split_offsets(comp, 1, density_split, P.color_off);
    status |= run_pass(G, vel, C, P, c2.data(), nthreads, 0, n, nullptr, nullptr);
    for (long i = 0; i < n; ++i) out[i] += c2[i];
    return status;
}

}  // namespace

// =================================== C ABI =========================================
extern "C" {

int fo_version(void) { return 4; }

// Gauss rule (for tests): writes k nodes on [-1,1] and normalised weights.
int fo_gauss(int k, double* x, double* w) {
    if (k < 1 || k > 63 || (k % 2) == 0) return -1;
    Gauss1D g = make_gauss(k);
    for (int i = 0; i < k; ++i) { x[i] = g.x[i]; w[i] = g.w[i]; }
    return 0;
}

// Point interpolation of a node field (M, off) at n points; method 0=WENO6 1=linear 2=1Dy-linear 3=1Dy-WENO6.
int fo_interp(const double* a, const int* M, const double* off, double h, int method,
              const double* pts, long n, double* out) {
    Field F; F.a = a;
    for (int d = 0; d < 3; ++d) { F.M[d] = M[d]; F.off[d] = off[d]; }
    for (long i = 0; i < n; ++i) {
        if (method == 3) out[i] = weno6_1dy(F, pts + 3 * i, h);
        else out[i] = interp(method, F, pts + 3 * i, h);
    }
    return 0;
}

// psi of a node field (mode 0 plain, 1 WENO6 integral, 2 linear integral).
int fo_psi(const double* a, const int* M, const double* off, double h, int mode, int k, double* psi_out) {
    Field F; F.a = a;
    for (int d = 0; d < 3; ++d) { F.M[d] = M[d]; F.off[d] = off[d]; }
    std::vector<double> psi;
    compute_psi(F, h, mode, make_gauss(k), psi);
    std::memcpy(psi_out, psi.data(), psi.size() * sizeof(double));
    return 0;
}

// Clip one face (4 vertices, xyz) and return the pieces (centroid xyz, scaled normal xyz).
int fo_split_face(const double* verts12, double h, const double* color_off, double minimal_area,
                  int max_out, double* out6, int* nout) {
    real v[4][3];
    for (int i = 0; i < 4; ++i) for (int d = 0; d < 3; ++d) v[i][d] = verts12[3 * i + d];
    std::vector<SubPoly> polys;
    int st = split_face(v, h, color_off, minimal_area, polys);
    int n = (int)polys.size();
    *nout = n;
    for (int i = 0; i < n && i < max_out; ++i) {
        for (int d = 0; d < 3; ++d) { out6[6 * i + d] = polys[i].pos[d]; out6[6 * i + 3 + d] = polys[i].n[d]; }
    }
    return st;
}

// Backtraced positions of all vertices of a field's cell lattice (for tests).
// comp=-1: (N+1)^3 density vertices; comp=c: staggered lattice of component c.
int fo_backtrace_vertices(int nx, int ny, int nz, double h, const double* u, const double* v,
                          const double* w, double dt, int comp, int interp_method, double* out) {
    Grid G; G.N[0] = nx; G.N[1] = ny; G.N[2] = nz; G.h = h;
    Velocity vel = make_velocity(G, u, v, w);
    PassParams P; P.comp = comp; P.interp = interp_method; P.zero_velocity = 0; P.dt = dt;
    int L[3];
    for (int d = 0; d < 3; ++d) L[d] = G.N[d] + 1 + (d == comp);
    long o = 0;
    for (int i = 0; i < L[0]; ++i) for (int j = 0; j < L[1]; ++j) for (int k = 0; k < L[2]; ++k) {
        int vi[3] = {i, j, k};
        backtrace_vertex(G, vel, P, vi, out + 3 * o);
        ++o;
    }
    return 0;
}

// One flux pass of a field (density when comp=-1), written to out.  Only cells in
// [c0, c1) are computed (c1 < 0 means all); used by the bounded CPU baseline.
int fo_flux_pass(int nx, int ny, int nz, double h, const double* u, const double* v, const double* w,
                 int comp, const double* field, double dt, int interp_method, int psi_mode,
                 int use_integral, int zero_velocity, const double* color_off, int k,
                 double minimal_area, int nthreads, long c0, long c1, double* out,
                 long* faces, long* polys, int maccormack) {
    Grid G; G.N[0] = nx; G.N[1] = ny; G.N[2] = nz; G.h = h;
    Velocity vel = make_velocity(G, u, v, w);
    Field A = make_field(field, G, comp);
    PassParams P;
    P.comp = comp; P.interp = interp_method; P.psi_mode = psi_mode; P.use_integral = use_integral;
    P.zero_velocity = zero_velocity; P.color_off[0] = color_off[0]; P.color_off[1] = color_off[1];
    P.k = k; P.minimal_area = minimal_area; P.dt = dt; P.maccormack = maccormack;
    return run_pass(G, vel, A, P, out, nthreads, c0, c1, faces, polys);
}

// move_substances_3D (flux advection branch), density in/out.
int fo_move_substances_3D(int nx, int ny, int nz, double h, const double* u, const double* v,
                          const double* w, double* rho, double dt, int interp_method, int k,
                          int correction, int use_integral, const double* split_off,
                          double minimal_area, int nthreads, int maccormack, int volume_correction) {
    Grid G; G.N[0] = nx; G.N[1] = ny; G.N[2] = nz; G.h = h;
    Velocity vel = make_velocity(G, u, v, w);
    long n = (long)nx * ny * nz;
    std::vector<double> in(rho, rho + n);
    return advect_field(G, vel, -1, in.data(), rho, dt, interp_method, k, correction, use_integral,
                        split_off, minimal_area, nthreads, nullptr, nullptr, maccormack, volume_correction);
}

// move_substances_3D (flux branch, density) on the cells of the x-slab [x0, x1) only: the work
// unit of the bounded CPU baseline, which times the step slab by slab.  The main pass and the
// error-advection pass run on the slab's cells; the zero-velocity pass, whose result the error
// pass reads within the backtrace reach, on the slab widened by `margin` cells each way (the
// caller passes ceil(max displacement) + 1); psi is computed on the columns those cells read
// (the WENO6 stencil reaches 3 more).  out[cell] is written for the slab's cells only.
int fo_move_substances_slab(int nx, int ny, int nz, double h, const double* u, const double* v, const double* w,
                            const double* rho, double dt, int interp_method, int k, int correction,
                            int use_integral, const double* split_off, double minimal_area, int nthreads, int x0,
                            int x1, int margin, double* out, long* faces) {
    Grid G; G.N[0] = nx; G.N[1] = ny; G.N[2] = nz; G.h = h;
    if (x0 < 0 || x1 > nx || x0 >= x1 || margin < 0) return -1;
    Velocity vel = make_velocity(G, u, v, w);
    Field A = make_field(rho, G, -1);
    for (int d = 0; d < 3; ++d) { A.M[d] = G.N[d]; A.off[d] = 0.5; }
    const long plane = (long)ny * nz, n = (long)nx * plane;
    PassParams P;
    P.comp = -1; P.interp = interp_method; P.k = k; P.minimal_area = minimal_area; P.dt = dt;
    P.psi_mode = use_integral ? (interp_method == I_WENO6 ? PSI_WENO6 : PSI_LINEAR) : PSI_PLAIN;
    P.use_integral = use_integral; P.zero_velocity = 0; P.maccormack = 0;
    split_offsets(-1, 0, split_off, P.color_off);
    const int reach = margin + 3;
    int status = run_pass(G, vel, A, P, out, nthreads, x0 * plane, x1 * plane, faces, nullptr, nullptr, x0 - reach,
                          x1 + reach);
    if (!correction) return status;
    const int xa = std::max(0, x0 - margin), xb = std::min(nx, x1 + margin);
    std::vector<real> c(n, 0.0), c2(n, 0.0);
    P.zero_velocity = 1; P.use_integral = 0; P.psi_mode = PSI_PLAIN;
    status |= run_pass(G, vel, A, P, c.data(), nthreads, xa * plane, xb * plane, nullptr, nullptr, nullptr, xa - 3,
                       xb + 3);
    for (long i = xa * plane; i < xb * plane; ++i) c[i] = rho[i] - c[i];
    Field C = A; C.a = c.data();
    P.zero_velocity = 0; P.interp = I_1DY_LINEAR;
    split_offsets(-1, 1, split_off, P.color_off);
    status |= run_pass(G, vel, C, P, c2.data(), nthreads, x0 * plane, x1 * plane, nullptr, nullptr, nullptr, xa, xb);
    for (long i = x0 * plane; i < x1 * plane; ++i) out[i] += c2[i];
    return status;
}

// The advected cell volumes of the density's main pass (the volume points of its pieces).
int fo_cell_volumes(int nx, int ny, int nz, double h, const double* u, const double* v, const double* w,
                    double dt, int interp_method, int k, int use_integral, const double* split_off,
                    double minimal_area, int nthreads, int maccormack, double* vol) {
    Grid G; G.N[0] = nx; G.N[1] = ny; G.N[2] = nz; G.h = h;
    Velocity vel = make_velocity(G, u, v, w);
    long n = (long)nx * ny * nz;
    std::vector<double> zero(n, 0.0), out(n);
    Field A = make_field(zero.data(), G, -1);
    for (int d = 0; d < 3; ++d) { A.M[d] = G.N[d]; A.off[d] = 0.5; }
    PassParams P;
    P.comp = -1; P.interp = interp_method; P.k = k; P.minimal_area = minimal_area; P.dt = dt;
    P.psi_mode = use_integral ? (interp_method == I_WENO6 ? PSI_WENO6 : PSI_LINEAR) : PSI_PLAIN;
    P.use_integral = use_integral; P.zero_velocity = 0; P.maccormack = maccormack;
    P.color_off[0] = split_off[0]; P.color_off[1] = split_off[1];
    return run_pass(G, vel, A, P, out.data(), nthreads, 0, n, nullptr, nullptr, vol);
}

// advect_velocity_xyz_flux_advection_3D: all three components advected by the old
// velocity (advect_velocity_flux_advection_3d.cpp:1138-1272), in place.
int fo_advect_velocity_3D(int nx, int ny, int nz, double h, double* u, double* v, double* w,
                          double dt, int interp_method, int k, int correction, int use_integral,
                          double minimal_area, int nthreads, int maccormack) {
    Grid G; G.N[0] = nx; G.N[1] = ny; G.N[2] = nz; G.h = h;
    long nu = (long)(nx + 1) * ny * nz, nv = (long)nx * (ny + 1) * nz, nw = (long)nx * ny * (nz + 1);
    std::vector<double> u0(u, u + nu), v0(v, v + nv), w0(w, w + nw);
    Velocity vel = make_velocity(G, u0.data(), v0.data(), w0.data());
    double* outs[3] = {u, v, w};
    const double* ins[3] = {u0.data(), v0.data(), w0.data()};
    int status = 0;
    const real dummy[2] = {0.5, 0.5};
    for (int c = 0; c < 3; ++c)
        status |= advect_field(G, vel, c, ins[c], outs[c], dt, interp_method, k, correction, use_integral,
                               dummy, minimal_area, nthreads, nullptr, nullptr, maccormack);
    return status;
}

// ------------------------------ pressure (A10) ---------------------------------------
// The reference operator (calc_pressure_3d.cpp:18-181): 7-point Laplacian, +1 off the
// diagonal, -6 + (number of walls) on it, over all cells but the last (pinned to 0),
// right-hand side div(u)*h.  Solved here by plain CG to a relative residual `tol`.
static void apply_A(const int* N, const double* p, double* Ap) {
    long n = (long)N[0] * N[1] * N[2];
    for (long c = 0; c < n - 1; ++c) {
        int iz = (int)(c % N[2]), iy = (int)((c / N[2]) % N[1]), ix = (int)(c / ((long)N[2] * N[1]));
        double diag = -6;
        double s = 0.0;
        if (ix == 0) diag += 1; else { long o = c - (long)N[1] * N[2]; if (o != n - 1) s += p[o]; }
        if (ix == N[0] - 1) diag += 1; else { long o = c + (long)N[1] * N[2]; if (o != n - 1) s += p[o]; }
        if (iy == 0) diag += 1; else { long o = c - N[2]; if (o != n - 1) s += p[o]; }
        if (iy == N[1] - 1) diag += 1; else { long o = c + N[2]; if (o != n - 1) s += p[o]; }
        if (iz == 0) diag += 1; else { long o = c - 1; if (o != n - 1) s += p[o]; }
        if (iz == N[2] - 1) diag += 1; else { long o = c + 1; if (o != n - 1) s += p[o]; }
        Ap[c] = diag * p[c] + s;
    }
    Ap[n - 1] = 0.0;
}

int fo_pressure_rhs(int nx, int ny, int nz, double h, const double* u, const double* v, const double* w, double* b) {
    int N[3] = {nx, ny, nz};
    for (int ix = 0; ix < nx; ++ix) for (int iy = 0; iy < ny; ++iy) for (int iz = 0; iz < nz; ++iz) {
        long c = idx3(N, ix, iy, iz);
        int Mu[3] = {nx + 1, ny, nz}, Mv[3] = {nx, ny + 1, nz}, Mw[3] = {nx, ny, nz + 1};
        b[c] = (u[idx3(Mu, ix + 1, iy, iz)] - u[idx3(Mu, ix, iy, iz)]
              + v[idx3(Mv, ix, iy + 1, iz)] - v[idx3(Mv, ix, iy, iz)]
              + w[idx3(Mw, ix, iy, iz + 1)] - w[idx3(Mw, ix, iy, iz)]) * h;
    }
    b[(long)nx * ny * nz - 1] = 0.0;
    return 0;
}

int fo_apply_laplacian(int nx, int ny, int nz, const double* p, double* Ap) {
    int N[3] = {nx, ny, nz};
    apply_A(N, p, Ap);
    return 0;
}

// CG on -A (SPD).  Returns iterations; p has the pinned last cell = 0.
int fo_pressure_solve(int nx, int ny, int nz, const double* b, double* p, double tol, int maxit, double* relres) {
    int N[3] = {nx, ny, nz};
    long n = (long)nx * ny * nz;
    std::vector<double> r(n), d(n), q(n);
    for (long i = 0; i < n; ++i) p[i] = 0.0;
    double bn = 0.0;
    for (long i = 0; i < n - 1; ++i) { r[i] = -b[i]; bn += r[i] * r[i]; }
    r[n - 1] = 0.0;
    bn = std::sqrt(bn);
    if (bn == 0.0) { if (relres) *relres = 0.0; return 0; }
    d = r;
    double rr = 0.0; for (long i = 0; i < n; ++i) rr += r[i] * r[i];
    int it = 0;
    for (; it < maxit; ++it) {
        if (std::sqrt(rr) <= tol * bn) break;
        apply_A(N, d.data(), q.data());
        for (long i = 0; i < n; ++i) q[i] = -q[i];
        double dq = 0.0; for (long i = 0; i < n; ++i) dq += d[i] * q[i];
        double alpha = rr / dq;
        for (long i = 0; i < n; ++i) { p[i] += alpha * d[i]; r[i] -= alpha * q[i]; }
        double rr2 = 0.0; for (long i = 0; i < n; ++i) rr2 += r[i] * r[i];
        double beta = rr2 / rr; rr = rr2;
        for (long i = 0; i < n; ++i) d[i] = r[i] + beta * d[i];
    }
    p[n - 1] = 0.0;
    if (relres) *relres = std::sqrt(rr) / bn;
    return it;
}

// u -= grad p / h on interior faces (calc_pressure_3d.cpp:196-232).
int fo_subtract_gradient(int nx, int ny, int nz, double h, const double* p, double* u, double* v, double* w) {
    int N[3] = {nx, ny, nz};
    int Mu[3] = {nx + 1, ny, nz}, Mv[3] = {nx, ny + 1, nz}, Mw[3] = {nx, ny, nz + 1};
    for (int ix = 1; ix < nx; ++ix) for (int iy = 0; iy < ny; ++iy) for (int iz = 0; iz < nz; ++iz)
        u[idx3(Mu, ix, iy, iz)] -= (p[idx3(N, ix, iy, iz)] - p[idx3(N, ix - 1, iy, iz)]) / (h);
    for (int ix = 0; ix < nx; ++ix) for (int iy = 1; iy < ny; ++iy) for (int iz = 0; iz < nz; ++iz)
        v[idx3(Mv, ix, iy, iz)] -= (p[idx3(N, ix, iy, iz)] - p[idx3(N, ix, iy - 1, iz)]) / (h);
    for (int ix = 0; ix < nx; ++ix) for (int iy = 0; iy < ny; ++iy) for (int iz = 1; iz < nz; ++iz)
        w[idx3(Mw, ix, iy, iz)] -= (p[idx3(N, ix, iy, iz)] - p[idx3(N, ix, iy, iz - 1)]) / (h);
    return 0;
}

// Largest |face velocity| (calc_time_step_length_from_CFL_number.cpp:90-117).
double fo_max_abs_velocity(int nx, int ny, int nz, const double* u, const double* v, const double* w) {
    long nu = (long)(nx + 1) * ny * nz, nv = (long)nx * (ny + 1) * nz, nw = (long)nx * ny * (nz + 1);
    double m = 0.0;
    for (long i = 0; i < nu; ++i) m = std::max(m, std::fabs(u[i]));
    for (long i = 0; i < nv; ++i) m = std::max(m, std::fabs(v[i]));
    for (long i = 0; i < nw; ++i) m = std::max(m, std::fabs(w[i]));
    return m;
}

}  // extern "C"

namespace {
static int solve_A(const int* N, const real* b, real* p, real tol, int maxit) {
    double rr = 0.0;
    return fo_pressure_solve(N[0], N[1], N[2], b, p, tol, maxit, &rr);
}
}  // namespace

// the streaming-tile CPU baseline (uses the clipper and fields above)
#include "cpu_stream.inl"
