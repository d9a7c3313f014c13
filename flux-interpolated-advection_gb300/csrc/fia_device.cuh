// fia_device.cuh -- device building blocks of the flux-interpolated advection path.
//
// Node fields: an array of M.x*M.y*M.z values, z fastest and x slowest (the reference
// layout, utils.h:65-165), whose node (i,j,k) sits at ((i+off.x)h, (j+off.y)h, (k+off.z)h).
//   density M=(N,N,N) off=(.5,.5,.5); u M=(N+1,N,N) off=(0,.5,.5); v, w likewise;
//   psi of a field with offsets off: M=(Mx,My+1,Mz), off-(0,.5,0).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fia {

struct NodeField {
    int Mx, My, Mz;
    double ox, oy, oz;  // node offsets in units of the cell length
    float oxf, oyf, ozf;   // the same in FP32 for the FP32 kernels (set by the host, desc32)
};

__device__ __forceinline__ int clampi(int i, int hi) { return i < 0 ? 0 : (i > hi ? hi : i); }
__device__ __forceinline__ long long idx3(const NodeField& F, int i, int j, int k) {
    return (long long)F.Mz * ((long long)F.My * i + j) + k;
}

// Values within a few units in the last place of an integer are taken as that integer:
// the discrete decisions of the scheme (iso-line crossings of vertex colours, the cell
// holding a centroid) are made on integers that exact arithmetic hits exactly (lattice
// vertices, vertices clamped to a wall) but n*h/h does not when h is not a power of two.
// Without this, ulp-level differences flip the clipped piece structure.  The oracle
// applies the same rule.
__device__ __forceinline__ double snap_int(double x) {
    const double r = rint(x);
    const double tol = 8.0 * 2.220446049250313e-16 * fmax(1.0, fabs(x));
    return fabs(x - r) <= tol ? r : x;
}
__host__ __device__ __forceinline__ float snap_int(float x) {
    const float r = rintf(x);
    const float tol = 8.0f * 1.1920928955078125e-7f * fmaxf(1.0f, fabsf(x));
    return fabsf(x - r) <= tol ? r : x;
}

// Contiguous store slots for the pieces of a warp's faces (cnt per lane): warp prefix sum and
// one atomic per warp on the store's counter.  Every lane of the warp calls it.
__device__ __forceinline__ long long warp_slots(unsigned* count, int cnt, int lane) {
    int pre = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, pre, o);
        if (lane >= o) pre += t;
    }
    const int total = __shfl_sync(0xffffffffu, pre, 31);
    unsigned base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(count, (unsigned)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return (long long)base + pre - cnt;
}

// Read-only load through the non-coherent cache.
template <typename T> __device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

// --------------------------------------------------------------------------------
// WENO6 coefficients that depend only on the sample position: for signed distances
// t_i = (p - x_i)/h of the six nodes, the three cubic candidates are
//   P_i = f_i + (f_{i+1}-f_i) a_i + (f_{i+2}-2f_{i+1}+f_i) b_i + (f_{i+3}-3f_{i+2}+3f_{i+1}-f_i) c_i
// with a_i = t_i, b_i = t_i t_{i+1}/2, c_i = t_i t_{i+1} t_{i+2}/6, and the ideal weights
// C = (t4 t5/20, -t5 t0/10, t0 t1/20)  (WENO6_interpolation_3d.cpp:70-92).  The divisions by
// constants are products here (one rounding more each: on GB300 an FP64 division is a dozen
// FP64-pipe instructions), and C is kept scaled by 20.
// --------------------------------------------------------------------------------
template <typename T>
struct WenoCoef {
    T a[3], b[3], c[3], C[3];
};

template <typename T>
__device__ __forceinline__ WenoCoef<T> weno_coef(const T* t) {
    WenoCoef<T> w;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const T p = t[i] * t[i + 1];
        w.a[i] = t[i];
        w.b[i] = T(0.5) * p;
        w.c[i] = (p * t[i + 2]) * (T(1) / T(6));
    }
    // the ideal weights scaled by 20, which the normalised weights of weno6_eval do not see
    w.C[0] = t[4] * t[5];
    w.C[1] = T(-2) * (t[5] * t[0]);
    w.C[2] = t[0] * t[1];
    return w;
}

// One 1D WENO6 evaluation: smoothness indicators with integer coefficients over 180,
// alpha_i = C_i / (1e-6 + beta_i)^2, normalised weights (WENO6_interpolation_3d.cpp:94-123).
// The smoothness indicators are evaluated as quadratic forms of the first differences
// D_i = f_{i+1} - f_i.  Expanding the reference's forms (products of the samples,
// WENO6_interpolation_3d.cpp:95-110) in D gives exactly
//   beta0 = (244 D0^2 - 1171 D0 D1 + 683 D0 D2 + 1561 D1^2 - 1951 D1 D2 + 814 D2^2) / 180
//   beta1 = (244 D1^2 - 781 D1 D2 + 293 D1 D3 + 961 D2^2 - 781 D2 D3 + 244 D3^2) / 180
//   beta2 = (814 D2^2 - 1951 D2 D3 + 683 D2 D4 + 1561 D3^2 - 1171 D3 D4 + 244 D4^2) / 180
// (no term in the samples themselves survives: the indicators are shift invariant).  In
// FP32 the sample-product form cancels to an absolute error of ~1e-3 f^2, far above the
// 1e-6 regularisation; the difference form keeps full relative accuracy and costs less.
template <typename T, bool FASTDIV = false>
__device__ __forceinline__ T weno6_eval(const T* f, const WenoCoef<T>& w) {
    const T D0 = f[1] - f[0], D1 = f[2] - f[1], D2 = f[3] - f[2], D3 = f[4] - f[3], D4 = f[5] - f[4];
    const T S0 = D1 - D0, S1 = D2 - D1, S2 = D3 - D2;      // second differences
    const T D[3] = {D0, D1, D2}, S[3] = {S0, S1, S2};
    const T Tt[3] = {S1 - S0, S2 - S1, (D4 - D3) - S2};    // third differences
    T P[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) P[i] = f[i] + D[i] * w.a[i] + S[i] * w.b[i] + Tt[i] * w.c[i];
    if constexpr (FASTDIV) {
        // FP32 form: the indicators in Horner form, all three (and eps) scaled by 180, which
        // cancels in the normalised weights, with 180 eps as the start of each chain; then
        // alpha_i = C_i r_i^2 with r_i = 1/e_i (approximate reciprocals, 1 ulp) and one
        // approximate division by the weight sum.  Range: e_i >= 180 eps = 1.8e-4, so
        // r_i^2 <= 3.1e7; for sample differences of order 1 the e_i stay far below the 1e19
        // at which r_i^2 would leave the normal range.
        const T eps180 = T(0.00018);
        const T w2 = T(814) * D2;
        const T e0 = fmaf(D0, T(244) * D0 - T(1171) * D1 + T(683) * D2,
                          fmaf(D1, T(1561) * D1 - T(1951) * D2, fmaf(w2, D2, eps180)));
        const T e1 = fmaf(D1, T(244) * D1 - T(781) * D2 + T(293) * D3,
                          fmaf(D2, T(961) * D2 - T(781) * D3, fmaf(T(244) * D3, D3, eps180)));
        const T e2 = fmaf(D2, w2 - T(1951) * D3 + T(683) * D4,
                          fmaf(D3, T(1561) * D3 - T(1171) * D4, fmaf(T(244) * D4, D4, eps180)));
        const T r0 = __fdividef(T(1), e0), r1 = __fdividef(T(1), e1), r2 = __fdividef(T(1), e2);
        const T a0 = (w.C[0] * r0) * r0, a1 = (w.C[1] * r1) * r1, a2 = (w.C[2] * r2) * r2;
        return __fdividef(fmaf(a2, P[2], fmaf(a1, P[1], a0 * P[0])), (a0 + a1) + a2);
    } else {
        const T r180 = T(1) / T(180);
        const T b0 = (T(244) * D0 * D0 - T(1171) * D0 * D1 + T(683) * D0 * D2 + T(1561) * D1 * D1
                      - T(1951) * D1 * D2 + T(814) * D2 * D2) * r180;
        const T b1 = (T(244) * D1 * D1 - T(781) * D1 * D2 + T(293) * D1 * D3 + T(961) * D2 * D2
                      - T(781) * D2 * D3 + T(244) * D3 * D3) * r180;
        const T b2 = (T(814) * D2 * D2 - T(1951) * D2 * D3 + T(683) * D2 * D4 + T(1561) * D3 * D3
                      - T(1171) * D3 * D4 + T(244) * D4 * D4) * r180;
        const T eps = T(0.000001);
        const T e0 = eps + b0, e1 = eps + b1, e2 = eps + b2;
        // alpha_i = C_i / e_i^2 and w_i = alpha_i / sum(alpha).  Multiplying every alpha by
        // e0^2 e1^2 e2^2 leaves the weights unchanged and needs one division instead of six; in
        // FP64 the products stay in range (e_i >= 1e-6, and e_i^4 overflows only for sample
        // differences beyond 1e75).
        const T q0 = e0 * e0, q1 = e1 * e1, q2 = e2 * e2;
        const T a0 = w.C[0] * (q1 * q2), a1 = w.C[1] * (q0 * q2), a2 = w.C[2] * (q0 * q1);
        return (a0 * P[0] + a1 * P[1] + a2 * P[2]) / (a0 + a1 + a2);
    }
}

// Tensor-product WENO6 of a node field at p (z, then y, then x), stencil indices clamped
// to the array (WENO6_interpolation_3d.cpp:7-258 and the face-value variants).
template <typename T>
__device__ T weno6_3d(const T* __restrict__ a, const NodeField& F, T h, T px, T py, T pz) {
    // positions in cells from the field's node 0; the stencil offsets t are these minus the
    // stencil nodes (the reference divides each offset by h)
    const T rx = (px - T(F.ox) * h) / h, ry = (py - T(F.oy) * h) / h, rz = (pz - T(F.oz) * h) / h;
    const int bx = (int)floor(rx), by = (int)floor(ry), bz = (int)floor(rz);
    T tx[6], ty[6], tz[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        tx[i] = rx - T(bx - 2 + i);
        ty[i] = ry - T(by - 2 + i);
        tz[i] = rz - T(bz - 2 + i);
    }
    const WenoCoef<T> cx = weno_coef(tx), cy = weno_coef(ty), cz = weno_coef(tz);
    int kk[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) kk[i] = clampi(bz - 2 + i, F.Mz - 1);
    T yv[6];
#pragma unroll 1
    for (int ix = 0; ix < 6; ++ix) {
        const int ii = clampi(bx - 2 + ix, F.Mx - 1);
        T zv[6];
#pragma unroll
        for (int iy = 0; iy < 6; ++iy) {
            const int jj = clampi(by - 2 + iy, F.My - 1);
            const T* row = a + (long long)F.Mz * ((long long)F.My * ii + jj);
            T f[6];
#pragma unroll
            for (int iz = 0; iz < 6; ++iz) f[iz] = ldg(row + kk[iz]);
            zv[iy] = weno6_eval(f, cz);
        }
        yv[ix] = weno6_eval(zv, cy);
    }
    return weno6_eval(yv, cx);
}

// weno6_3d with every axis on which p lies on a node plane of F (its offset from the lattice,
// in cells, is an integer up to the snap tolerance) collapsed to that node: every candidate
// polynomial along such an axis interpolates the node and the weights sum to one, so the pass
// along it returns the node's value.  Equal to weno6_3d in exact arithmetic, with fewer 1D
// evaluations: a vertex at rest lies on node planes of the staggered velocity components
// along one or two axes (21 evaluations instead of 129 for a density vertex), the psi point of
// a piece lies on a node row of psi (7 instead of 43), and a face at rest has its centroid on
// node planes.  The remaining axes use weno6_3d's arithmetic.
template <typename T>
__device__ T weno6_3d_collapse(const T* __restrict__ a, const NodeField& F, T h, T px, T py, T pz) {
    const T rx = (px - T(F.ox) * h) / h, ry = (py - T(F.oy) * h) / h, rz = (pz - T(F.oz) * h) / h;
    const T sx = snap_int(rx), sy = snap_int(ry), sz = snap_int(rz);
    const bool cxn = sx == rint(sx), cyn = sy == rint(sy), czn = sz == rint(sz);
    const int bx = cxn ? (int)sx : (int)floor(rx);
    const int by = cyn ? (int)sy : (int)floor(ry);
    const int bz = czn ? (int)sz : (int)floor(rz);
    T tx[6], ty[6], tz[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        tx[i] = rx - T(bx - 2 + i);
        ty[i] = ry - T(by - 2 + i);
        tz[i] = rz - T(bz - 2 + i);
    }
    const WenoCoef<T> cx = weno_coef(tx), cy = weno_coef(ty), cz = weno_coef(tz);
    int kk[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) kk[i] = clampi(bz - 2 + i, F.Mz - 1);
    const int x0 = cxn ? 2 : 0, x1 = cxn ? 3 : 6, y0 = cyn ? 2 : 0, y1 = cyn ? 3 : 6;
    T yv[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
#pragma unroll 1
    for (int ix = x0; ix < x1; ++ix) {
        const int ii = clampi(bx - 2 + ix, F.Mx - 1);
        T zv[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
#pragma unroll 1
        for (int iy = y0; iy < y1; ++iy) {
            const int jj = clampi(by - 2 + iy, F.My - 1);
            const T* row = a + (long long)F.Mz * ((long long)F.My * ii + jj);
            if (czn) {
                zv[iy] = ldg(row + kk[2]);
            } else {
                T f[6];
#pragma unroll
                for (int iz = 0; iz < 6; ++iz) f[iz] = ldg(row + kk[iz]);
                zv[iy] = weno6_eval(f, cz);
            }
        }
        yv[ix] = cyn ? zv[2] : weno6_eval(zv, cy);
    }
    return cxn ? yv[2] : weno6_eval(yv, cx);
}

// WENO6 along y only; x and z take the node whose cell holds p
// (WENO6_interpolation_1d.cpp:315-430).
template <typename T>
__device__ T weno6_1dy(const T* __restrict__ a, const NodeField& F, T h, T px, T py, T pz) {
    const int ix = clampi((int)floor(snap_int((px - (T(F.ox) * h - T(0.5) * h)) / h)), F.Mx - 1);
    const int iz = clampi((int)floor(snap_int((pz - (T(F.oz) * h - T(0.5) * h)) / h)), F.Mz - 1);
    const T ry = (py - T(F.oy) * h) / h;
    const int by = (int)floor(ry);
    T t[6], f[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        t[i] = ry - T(by - 2 + i);
        f[i] = ldg(a + idx3(F, ix, clampi(by - 2 + i, F.My - 1), iz));
    }
    return weno6_eval(f, weno_coef(t));
}

// Trilinear interpolation with clamped indices (linear_interpolation_3d.cpp:7-95).
template <typename T>
__device__ T lin3d(const T* __restrict__ a, const NodeField& F, T h, T px, T py, T pz) {
    const T ox = T(F.ox) * h, oy = T(F.oy) * h, oz = T(F.oz) * h;
    const int bx = (int)floor((px - ox) / h), by = (int)floor((py - oy) / h), bz = (int)floor((pz - oz) / h);
    const T sx = (px - ox) / h - T(bx), sy = (py - oy) / h - T(by), sz = (pz - oz) / h - T(bz);
    const int k0 = clampi(bz, F.Mz - 1), k1 = clampi(bz + 1, F.Mz - 1);
    T yv[2];
#pragma unroll
    for (int ix = 0; ix < 2; ++ix) {
        const int ii = clampi(bx + ix, F.Mx - 1);
        T zv[2];
#pragma unroll
        for (int iy = 0; iy < 2; ++iy) {
            const int jj = clampi(by + iy, F.My - 1);
            const T* row = a + (long long)F.Mz * ((long long)F.My * ii + jj);
            zv[iy] = (T(1) - sz) * ldg(row + k0) + sz * ldg(row + k1);
        }
        yv[ix] = (T(1) - sy) * zv[0] + sy * zv[1];
    }
    return (T(1) - sx) * yv[0] + sx * yv[1];
}

// Linear along y, nearest cell in x and z (linear_interpolation_1d.cpp:314-374).
template <typename T>
__device__ T lin1dy(const T* __restrict__ a, const NodeField& F, T h, T px, T py, T pz) {
    const int ix = clampi((int)floor(snap_int((px - (T(F.ox) * h - T(0.5) * h)) / h)), F.Mx - 1);
    const int iz = clampi((int)floor(snap_int((pz - (T(F.oz) * h - T(0.5) * h)) / h)), F.Mz - 1);
    const T oy = T(F.oy) * h;
    const int by = (int)floor((py - oy) / h);
    const T f0 = ldg(a + idx3(F, ix, clampi(by, F.My - 1), iz));
    const T f1 = ldg(a + idx3(F, ix, clampi(by + 1, F.My - 1), iz));
    const T b0 = (py - oy) / h - T(by);
    return (T(1) - b0) * f0 + b0 * f1;
}

enum Interp : int { INTERP_WENO6 = 0, INTERP_LINEAR = 1, INTERP_1DY_LINEAR = 2 };

template <typename T>
__device__ __forceinline__ T interp(int method, const T* __restrict__ a, const NodeField& F, T h, T px, T py, T pz) {
    if (method == INTERP_WENO6) return weno6_3d(a, F, h, px, py, pz);
    if (method == INTERP_LINEAR) return lin3d(a, F, h, px, py, pz);
    return lin1dy(a, F, h, px, py, pz);
}

}  // namespace fia
