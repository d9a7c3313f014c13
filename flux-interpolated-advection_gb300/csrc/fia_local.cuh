// fia_local.cuh -- FP32 building blocks in local cell coordinates (the chosen form).
//
// Positions are carried as an integer anchor (a cell-lattice index) plus a small FP32
// offset q, both in units of the cell length: X = anchor + q.  Every quantity the FP32
// arithmetic sees is then O(CFL): stencil distances, colours, centroids and normals keep
// FP32's full relative precision regardless of where in a 256^3 or 384^3 grid the face is.
// Absolute FP32 coordinates would lose ~1.5e-5 of a cell at 256^3.
//
// psi is carried as a double-float pair (hi, lo) in cell units (psi / h).  A face
// interpolates psi - Psi0 for a base node Psi0 of its own, formed from the pairs as
// (hi - hi0) + (lo - lo0): WENO6, trilinear and 1Dy-linear interpolation all commute with
// adding a constant (the smoothness indicators are quadratic forms of differences and the
// weights sum to one), so this is the same interpolant without FP32 cancellation.
#pragma once
#include "fia_device.cuh"

namespace fia {

// One 1D WENO6 evaluation as a real call.  Inlined, the face kernel held some sixty copies
// of weno6_eval (the unrolled z-passes of a stencil), more code than the instruction cache
// holds; ncu showed most warps waiting on instruction fetch.  Arguments travel in registers.
__device__ __noinline__ float weno6_f(float f0, float f1, float f2, float f3, float f4, float f5, WenoCoef<float> w) {
    const float f[6] = {f0, f1, f2, f3, f4, f5};
    return weno6_eval<float, true>(f, w);
}
__device__ __forceinline__ float weno6_call(const float* f, const WenoCoef<float>& w) {
    return weno6_f(f[0], f[1], f[2], f[3], f[4], f[5], w);
}
// Two evaluations with the same coefficients in one call: the two dependency chains (the
// weights end in a serial max / reciprocal / normalise tail) interleave, which a call per
// evaluation prevents, at half the calls.  Each result equals weno6_f's.
__device__ __noinline__ float2 weno6_f2(float a0, float a1, float a2, float a3, float a4, float a5, float b0, float b1,
                                        float b2, float b3, float b4, float b5, WenoCoef<float> w) {
    const float fa[6] = {a0, a1, a2, a3, a4, a5}, fb[6] = {b0, b1, b2, b3, b4, b5};
    return make_float2(weno6_eval<float, true>(fa, w), weno6_eval<float, true>(fb, w));
}
__device__ __forceinline__ float2 weno6_call2(const float* a, const float* b, const WenoCoef<float>& w) {
    return weno6_f2(a[0], a[1], a[2], a[3], a[4], a[5], b[0], b[1], b[2], b[3], b[4], b[5], w);
}

// Two evaluations with shared coefficients, inlined: for a loop whose body is one pair (the
// z-pass of the quadrature kernel), so one copy of the code serves the whole loop and the
// coefficients stay in registers across its iterations.
__device__ __forceinline__ float2 weno6_pair(const float* a, const float* b, const WenoCoef<float>& w) {
    return make_float2(weno6_eval<float, true>(a, w), weno6_eval<float, true>(b, w));
}

// error-free sum of two floats (Knuth TwoSum)
__host__ __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// running sum with a compensation term
struct Kahan {
    float s = 0.f, c = 0.f;
    __host__ __device__ __forceinline__ void add(float x) {
        float t, e;
        two_sum(s, x, t, e);
        s = t;
        c += e;
    }
    __host__ __device__ __forceinline__ float value() const { return s + c; }
};

// Loads node values as floats: plain array, or psi pairs relative to a base pair.
// row(i) gives a row pointer; at(row, k) the value k nodes further along the row (k a
// compile-time constant in an unrolled loop, so one load with an immediate offset).
// Node offsets are 32-bit: fia_create admits grids with (nx+2)(ny+2)(nz+2) <= 2^31, which
// bounds every node field of the path.
struct PlainLoad {
    const float* __restrict__ a;
    __device__ __forceinline__ float operator()(int i) const { return __ldg(a + i); }
    __device__ __forceinline__ const float* row(int i) const { return a + i; }
    __device__ __forceinline__ float at(const float* p, int k) const { return __ldg(p + k); }
};
struct PsiLoad {
    const float2* __restrict__ a;
    float hi0, lo0;
    __device__ __forceinline__ float operator()(int i) const {
        const float2 v = __ldg(a + i);
        return (v.x - hi0) + (v.y - lo0);
    }
    __device__ __forceinline__ const float2* row(int i) const { return a + i; }
    __device__ __forceinline__ float at(const float2* p, int k) const {
        const float2 v = __ldg(p + k);
        return (v.x - hi0) + (v.y - lo0);
    }
};

// the six z-values of two stencil rows: row pointers and immediate offsets when the z-stencil
// lies inside the field (zin), else the clamped indices kk
template <class L>
__device__ __forceinline__ void load_rows(const L& load, int row0, int row1, bool zin, int bz,
                                          const int* kk, float* f0, float* f1) {
    if (zin) {
        const auto p0 = load.row(row0 + bz - 2), p1 = load.row(row1 + bz - 2);
#pragma unroll
        for (int iz = 0; iz < 6; ++iz) { f0[iz] = load.at(p0, iz); f1[iz] = load.at(p1, iz); }
    } else {
#pragma unroll
        for (int iz = 0; iz < 6; ++iz) { f0[iz] = load(row0 + kk[iz]); f1[iz] = load(row1 + kk[iz]); }
    }
}

// stencil base and fractional offset of the local position along one axis
__device__ __forceinline__ void locate(int anchor, float q, float off, int& base, float& s) {
    const float r = q - off;
    const float f = floorf(r);
    base = anchor + (int)f;
    s = r - f;
}
// the cell holding the local position along one axis (a discrete decision: snapped)
__device__ __forceinline__ int cell_of(int anchor, float q, float off) {
    return anchor + (int)floorf(snap_int(q - off));
}

template <class L>
__device__ float weno6_3d_loc(const L& load, const NodeField& F, const int* anc, const float* q) {
    int bx, by, bz;
    float sx, sy, sz;
    locate(anc[0], q[0], F.oxf, bx, sx);
    locate(anc[1], q[1], F.oyf, by, sy);
    locate(anc[2], q[2], F.ozf, bz, sz);
    float tx[6], ty[6], tz[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        tx[i] = sx + float(2 - i);
        ty[i] = sy + float(2 - i);
        tz[i] = sz + float(2 - i);
    }
    const WenoCoef<float> cx = weno_coef(tx), cy = weno_coef(ty), cz = weno_coef(tz);
    int kk[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) kk[i] = clampi(bz - 2 + i, F.Mz - 1);
    float yv[6];
#pragma unroll 1
    for (int ix = 0; ix < 6; ++ix) {
        const int ii = clampi(bx - 2 + ix, F.Mx - 1);
        float zv[6];
#pragma unroll
        for (int iy = 0; iy < 6; iy += 2) {
            const int j0 = clampi(by - 2 + iy, F.My - 1), j1 = clampi(by - 1 + iy, F.My - 1);
            const int row0 = F.Mz * (F.My * ii + j0), row1 = F.Mz * (F.My * ii + j1);
            float f0[6], f1[6];
#pragma unroll
            for (int iz = 0; iz < 6; ++iz) { f0[iz] = load(row0 + kk[iz]); f1[iz] = load(row1 + kk[iz]); }
            const float2 v = weno6_call2(f0, f1, cz);
            zv[iy] = v.x; zv[iy + 1] = v.y;
        }
        yv[ix] = weno6_call(zv, cy);
    }
    return weno6_call(yv, cx);
}

// WENO6 at npts points that share x and z and lie within one cell in y (the density
// quadrature points of one piece, polygon_3D.cpp:286-453): the z-pass over the 6 x 7
// (x, y) stencil rows is done once and shared; each point then needs 6 y- and 1 x-
// evaluation instead of 43.  Bit-identical to evaluating the points one by one.  The points
// come from point(m, y, w) and lie in [ya, yb]; returns the number of 1D evaluations made, or
// 0 (nothing accumulated) if [ya, yb] spans more than one cell of the field.
// The 6 x 7 z-pass results live in shared memory, zs[(7 ix + r) * stride] (the calling
// thread's column of a block-wide array, stride = threads per block, 48 words: in registers
// they held 42 of the face kernel's 128); a point's six y-pass results stay in registers.
template <int STRIDE, class L, class P>
__device__ int weno6_ycolumn(const L& load, const NodeField& F, const int* anc, float qx, float qz, float ya,
                             float yb, int npts, const P& point, Kahan& acc, float* zs) {
    int bx, bz, by0, by1;
    float sx, sz, s;
    locate(anc[0], qx, F.oxf, bx, sx);
    locate(anc[2], qz, F.ozf, bz, sz);
    locate(anc[1], ya, F.oyf, by0, s);
    locate(anc[1], yb, F.oyf, by1, s);
    if (by1 - by0 > 1) return 0;
    const bool seven = by1 > by0;
    float tx[6], tz[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) { tx[i] = sx + float(2 - i); tz[i] = sz + float(2 - i); }
    const WenoCoef<float> cx = weno_coef(tx), cz = weno_coef(tz);
    int kk[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) kk[i] = clampi(bz - 2 + i, F.Mz - 1);
    const int nr = seven ? 7 : 6;
    const bool zin = bz >= 2 && bz + 3 <= F.Mz - 1;
#pragma unroll 1
    for (int ix = 0; ix < 6; ix += 2) {
        const int i0 = clampi(bx - 2 + ix, F.Mx - 1), i1 = clampi(bx - 1 + ix, F.Mx - 1);
        float* z0 = zs + 7 * ix * STRIDE;
        float* z1 = z0 + 7 * STRIDE;
        // two rows per iteration: two independent pairs of evaluations in flight
        int r = 0;
#pragma unroll 1
        for (; r + 1 < nr; r += 2) {
            const int ja = clampi(by0 - 2 + r, F.My - 1), jb = clampi(by0 - 1 + r, F.My - 1);
            float fa0[6], fa1[6], fb0[6], fb1[6];
            load_rows(load, F.Mz * (F.My * i0 + ja), F.Mz * (F.My * i1 + ja), zin, bz, kk, fa0, fa1);
            load_rows(load, F.Mz * (F.My * i0 + jb), F.Mz * (F.My * i1 + jb), zin, bz, kk, fb0, fb1);
            const float2 va = weno6_pair(fa0, fa1, cz);
            const float2 vb = weno6_pair(fb0, fb1, cz);
            z0[r * STRIDE] = va.x; z1[r * STRIDE] = va.y;
            z0[(r + 1) * STRIDE] = vb.x; z1[(r + 1) * STRIDE] = vb.y;
        }
        if (r < nr) {
            const int jj = clampi(by0 - 2 + r, F.My - 1);
            const int row0 = F.Mz * (F.My * i0 + jj), row1 = F.Mz * (F.My * i1 + jj);
            float f0[6], f1[6];
            load_rows(load, row0, row1, zin, bz, kk, f0, f1);
            const float2 v = weno6_pair(f0, f1, cz);
            z0[r * STRIDE] = v.x; z1[r * STRIDE] = v.y;
        }
    }
    for (int m = 0; m < npts; ++m) {
        float y, w;
        point(m, y, w);
        int by;
        float sy;
        locate(anc[1], y, F.oyf, by, sy);
        const bool up = by > by0;
        float ty[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) ty[i] = sy + float(2 - i);
        const WenoCoef<float> cy = weno_coef(ty);
        const float* zb = zs + (up ? STRIDE : 0);
        float yv[6];
#pragma unroll
        for (int ix = 0; ix < 6; ix += 2) {
            float f0[6], f1[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                f0[i] = zb[(7 * ix + i) * STRIDE];
                f1[i] = zb[(7 * ix + 7 + i) * STRIDE];
            }
            const float2 v = weno6_pair(f0, f1, cy);
            yv[ix] = v.x; yv[ix + 1] = v.y;
        }
        acc.add(weno6_eval<float, true>(yv, cx) * w);
    }
    return (seven ? 42 : 36) + 7 * npts;
}

template <class L>
__device__ float weno6_1dy_loc(const L& load, const NodeField& F, const int* anc, const float* q) {
    int by;
    float sy;
    const int ix = clampi(cell_of(anc[0], q[0], F.oxf - 0.5f), F.Mx - 1);
    const int iz = clampi(cell_of(anc[2], q[2], F.ozf - 0.5f), F.Mz - 1);
    locate(anc[1], q[1], F.oyf, by, sy);
    float t[6], f[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        t[i] = sy + float(2 - i);
        f[i] = load(F.Mz * (F.My * ix + clampi(by - 2 + i, F.My - 1)) + iz);
    }
    return weno6_call(f, weno_coef(t));
}

template <class L>
__device__ float lin3d_loc(const L& load, const NodeField& F, const int* anc, const float* q) {
    int bx, by, bz;
    float sx, sy, sz;
    locate(anc[0], q[0], F.oxf, bx, sx);
    locate(anc[1], q[1], F.oyf, by, sy);
    locate(anc[2], q[2], F.ozf, bz, sz);
    const int k0 = clampi(bz, F.Mz - 1), k1 = clampi(bz + 1, F.Mz - 1);
    float yv[2];
#pragma unroll
    for (int ix = 0; ix < 2; ++ix) {
        const int ii = clampi(bx + ix, F.Mx - 1);
        float zv[2];
#pragma unroll
        for (int iy = 0; iy < 2; ++iy) {
            const int jj = clampi(by + iy, F.My - 1);
            const int row = F.Mz * (F.My * ii + jj);
            zv[iy] = (1.f - sz) * load(row + k0) + sz * load(row + k1);
        }
        yv[ix] = (1.f - sy) * zv[0] + sy * zv[1];
    }
    return (1.f - sx) * yv[0] + sx * yv[1];
}

template <class L>
__device__ float lin1dy_loc(const L& load, const NodeField& F, const int* anc, const float* q) {
    int by;
    float sy;
    const int ix = clampi(cell_of(anc[0], q[0], F.oxf - 0.5f), F.Mx - 1);
    const int iz = clampi(cell_of(anc[2], q[2], F.ozf - 0.5f), F.Mz - 1);
    locate(anc[1], q[1], F.oyf, by, sy);
    const float f0 = load(F.Mz * (F.My * ix + clampi(by, F.My - 1)) + iz);
    const float f1 = load(F.Mz * (F.My * ix + clampi(by + 1, F.My - 1)) + iz);
    return (1.f - sy) * f0 + sy * f1;
}

// WENO6 at a point whose y lies on a node row of F (fractional offset exactly 0, as for the
// psi point of a piece, which sits on the y-face below the centroid).  Every candidate
// polynomial of the y-pass interpolates that node and the weights sum to one, so the y-pass
// returns the row's value: the interpolant is the (x, z) WENO6 of the row, 7 evaluations
// instead of 43, equal to the full form in exact arithmetic.  Returns the number of 1D
// evaluations, or 0 (out untouched) if y is not on a node row.  The six z-pass results pass
// through words 42-47 of the thread's shared column zs (as in weno6_ycolumn).
template <int STRIDE, class L>
__device__ int weno6_3d_noderow(const L& load, const NodeField& F, const int* anc, const float* q, float& out,
                                float* zs) {
    int bx, by, bz;
    float sx, sy, sz;
    locate(anc[1], q[1], F.oyf, by, sy);
    if (sy != 0.f) return 0;
    locate(anc[0], q[0], F.oxf, bx, sx);
    locate(anc[2], q[2], F.ozf, bz, sz);
    float tx[6], tz[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) { tx[i] = sx + float(2 - i); tz[i] = sz + float(2 - i); }
    const WenoCoef<float> cx = weno_coef(tx), cz = weno_coef(tz);
    int kk[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) kk[i] = clampi(bz - 2 + i, F.Mz - 1);
    const int jj = clampi(by, F.My - 1);
    const bool zin = bz >= 2 && bz + 3 <= F.Mz - 1;
#pragma unroll 1
    for (int ix = 0; ix < 6; ix += 2) {
        const int i0 = clampi(bx - 2 + ix, F.Mx - 1), i1 = clampi(bx - 1 + ix, F.Mx - 1);
        const int row0 = F.Mz * (F.My * i0 + jj), row1 = F.Mz * (F.My * i1 + jj);
        float f0[6], f1[6];
        load_rows(load, row0, row1, zin, bz, kk, f0, f1);
        const float2 v = weno6_pair(f0, f1, cz);
        zs[(42 + ix) * STRIDE] = v.x; zs[(43 + ix) * STRIDE] = v.y;
    }
    float xv[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) xv[i] = zs[(42 + i) * STRIDE];
    out = weno6_eval<float, true>(xv, cx);
    return 7;
}

// WENO6 in which every axis whose fractional offset is exactly 0 is collapsed to its centre
// node (all candidate polynomials interpolate the node and the weights sum to one, so the pass
// along that axis returns the node value): the vertices' rest positions lie on node planes of
// the staggered fields along one or two axes.  Equal to weno6_3d_loc in exact arithmetic.
template <class L>
__device__ float weno6_3d_collapse(const L& load, const NodeField& F, const int* anc, const float* q) {
    int bx, by, bz;
    float sx, sy, sz;
    locate(anc[0], q[0], F.oxf, bx, sx);
    locate(anc[1], q[1], F.oyf, by, sy);
    locate(anc[2], q[2], F.ozf, bz, sz);
    const bool cxn = sx == 0.f, cyn = sy == 0.f, czn = sz == 0.f;
    float tx[6], ty[6], tz[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        tx[i] = sx + float(2 - i);
        ty[i] = sy + float(2 - i);
        tz[i] = sz + float(2 - i);
    }
    const WenoCoef<float> cx = weno_coef(tx), cy = weno_coef(ty), cz = weno_coef(tz);
    int kk[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) kk[i] = clampi(bz - 2 + i, F.Mz - 1);
    const int x0 = cxn ? 2 : 0, x1 = cxn ? 3 : 6, y0 = cyn ? 2 : 0, y1 = cyn ? 3 : 6;
    float yv[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
    for (int ix = x0; ix < x1; ++ix) {
        const int ii = clampi(bx - 2 + ix, F.Mx - 1);
        float zv[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
        for (int iy = y0; iy < y1; ++iy) {
            const int row = F.Mz * (F.My * ii + clampi(by - 2 + iy, F.My - 1));
            if (czn) {
                zv[iy] = load(row + kk[2]);
            } else {
                float f[6];
#pragma unroll
                for (int iz = 0; iz < 6; ++iz) f[iz] = load(row + kk[iz]);
                zv[iy] = weno6_call(f, cz);
            }
        }
        yv[ix] = cyn ? zv[2] : weno6_call(zv, cy);
    }
    return cxn ? yv[2] : weno6_call(yv, cx);
}

template <class L>
__device__ __forceinline__ float interp_loc(int method, const L& load, const NodeField& F, const int* anc,
                                            const float* q) {
    if (method == INTERP_WENO6) return weno6_3d_loc(load, F, anc, q);
    if (method == INTERP_LINEAR) return lin3d_loc(load, F, anc, q);
    return lin1dy_loc(load, F, anc, q);
}

}  // namespace fia
