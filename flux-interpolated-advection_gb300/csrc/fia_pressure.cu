// fia_pressure.cu -- pressure projection (calc_pressure_3d.cpp:18-270) on the GPU.
//
// The reference assembles a CSR 7-point Laplacian over all cells but the last one (pinned
// to p = 0), right-hand side b = div(u) h, and solves it with amgcl (SA-AMG + CG).  Here
// the same operator is applied matrix-free and solved with CG on B = -A (symmetric positive
// definite on the free cells): Jacobi-preconditioned, or flexible CG around a preconditioner
// supplied by the caller (the learned one).  Solid cells are excluded like walls.
//
// Element arithmetic is in the field's own type; every dot product and norm is accumulated
// to FP64 accuracy: per thread exactly in double (FP64 form) or as an unevaluated float
// pair with FMA-exact products (FP32 form), across threads and blocks in double, with
// fixed per-block partials summed in block order by the last block of each kernel (no
// atomics on values, so the result does not depend on scheduling).
#include "fia_pressure.cuh"

#include <algorithm>
#include <cmath>

namespace fia {

constexpr int kRedBlocks = 152 * 6;
constexpr int kRedThreads = 256;
constexpr int kCgBatch = 16;

// scal layout
enum : int {
    S_ALPHA = 0, S_BETA = 1, S_RZ = 2, S_RR = 3, S_THRESH = 4, S_DONE = 5, S_ITERS = 6, S_DQ = 7,
    S_BETAJ = 8,                        // flexible CG: beta of direction slot j
    S_DQJ = S_BETAJ + kFcgMaxDirs + 1   // flexible CG: d.q of direction slot j
};
static_assert(S_DQJ + kFcgMaxDirs + 1 <= kScalDoubles, "scalar block too small for the FCG direction ring");

// ---------------------------------------------------------------------------------
// per-thread dot accumulators
// ---------------------------------------------------------------------------------
template <typename T>
struct DotAcc;

template <>
struct DotAcc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
};

template <>
struct DotAcc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float a, float b) {
        const float p = __fmul_rn(a, b);
        const float pe = __fmaf_rn(a, b, -p);          // exact product error
        const float s = __fadd_rn(hi, p);
        const float bb = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(e, pe));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-level sums of NV values written to part[b + nb*q].
template <int NV>
__device__ __forceinline__ void block_sums(const double (&v)[NV], double* part) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const double s = warp_sum(v[q]);
        if (lane == 0) sh[q][wid] = s;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = lane < nw ? sh[q][lane] : 0.0;
            s = warp_sum(s);
            if (lane == 0) part[blockIdx.x + gridDim.x * q] = s;
        }
    }
}

__device__ __forceinline__ bool last_block(unsigned* ticket) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    return last;
}

// sum of one partial row by the last block, in block order
__device__ double block_total(const double* part, int nblocks, int q) {
    __shared__ double sh[32];
    __shared__ double tot;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += __ldcg(part + b + nblocks * q);
    s = warp_sum(s);
    if (lane == 0) sh[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        tot = t;
    }
    __syncthreads();
    return tot;
}

// ---------------------------------------------------------------------------------
// the operator
// ---------------------------------------------------------------------------------
struct Cell {
    int ix, iy, iz;
};
__device__ __forceinline__ Cell decode(unsigned c, int ny, int nz) {
    Cell r;
    r.iz = (int)(c % (unsigned)nz);
    const unsigned t = c / (unsigned)nz;
    r.iy = (int)(t % (unsigned)ny);
    r.ix = (int)(t / (unsigned)ny);
    return r;
}

__device__ __forceinline__ bool excluded(const PoissonGrid& g, unsigned c) {
    return (int)c == g.pin || (g.solid && g.solid[c]);
}

// Visits the six neighbours of free cell c: f(o) for coupled neighbours (fluid, not the
// pinned cell); returns the diagonal of B (coupled neighbours + the pinned one).
template <typename F>
__device__ __forceinline__ int for_neighbours(const PoissonGrid& g, unsigned c, Cell k, F&& f) {
    const unsigned sx = (unsigned)g.ny * g.nz, sy = (unsigned)g.nz;
    int diag = 0;
    auto nb = [&](unsigned o) {
        if (g.solid && g.solid[o]) return;          // zero-flux face, like a wall
        ++diag;
        if ((int)o != g.pin) f(o);                  // the pinned cell holds p = 0
    };
    if (k.ix > 0) nb(c - sx);
    if (k.ix < g.nx - 1) nb(c + sx);
    if (k.iy > 0) nb(c - sy);
    if (k.iy < g.ny - 1) nb(c + sy);
    if (k.iz > 0) nb(c - 1);
    if (k.iz < g.nz - 1) nb(c + 1);
    return diag;
}

// Net outflow of free cell c, summed over its six faces in the accumulation type A.  A face
// shared with a solid cell carries the solid's zero velocity whatever the array holds there
// (advection and buoyancy write every face), so the right-hand side matches the operator,
// whose rows drop solid neighbours, and the projected field is divergence-free next to solids.
template <typename A, typename T>
__device__ __forceinline__ A net_outflow(const PoissonGrid& g, unsigned c, Cell k, const T* __restrict__ u,
                                         const T* __restrict__ v, const T* __restrict__ w) {
    const int ny = g.ny, nz = g.nz;
    const unsigned sx = (unsigned)ny * nz;
    const unsigned u0 = c, u1 = c + sx;
    const unsigned v0 = ((unsigned)k.ix * (ny + 1) + k.iy) * nz + k.iz, v1 = v0 + nz;
    const unsigned w0 = ((unsigned)k.ix * ny + k.iy) * (nz + 1) + k.iz, w1 = w0 + 1;
    A fu0 = (A)u[u0], fu1 = (A)u[u1], fv0 = (A)v[v0], fv1 = (A)v[v1], fw0 = (A)w[w0], fw1 = (A)w[w1];
    if (g.solid) {
        if (k.ix > 0 && g.solid[c - sx]) fu0 = A(0);
        if (k.ix < g.nx - 1 && g.solid[c + sx]) fu1 = A(0);
        if (k.iy > 0 && g.solid[c - nz]) fv0 = A(0);
        if (k.iy < ny - 1 && g.solid[c + nz]) fv1 = A(0);
        if (k.iz > 0 && g.solid[c - 1]) fw0 = A(0);
        if (k.iz < nz - 1 && g.solid[c + 1]) fw1 = A(0);
    }
    return (fu1 - fu0) + (fv1 - fv0) + (fw1 - fw0);
}

template <typename T>
__device__ __forceinline__ T inv_count(int d) {
    return d > 0 ? T(1) / T(d) : T(0);
}

// ---------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------

// r = -b - B p (warm) or r = -b, p = 0; partials |b|^2 and |r|^2
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_rhs(PoissonGrid g, T h, const T* __restrict__ u,
                                                      const T* __restrict__ v, const T* __restrict__ w,
                                                      T* __restrict__ r, T* __restrict__ p, int warm, double* part) {
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    const int ny = g.ny, nz = g.nz;
    DotAcc<T> bb, rr;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const Cell k = decode(c, ny, nz);
        T b = T(0), rc = T(0);
        if (!excluded(g, c)) {
            b = net_outflow<T>(g, c, k, u, v, w) * h;
            rc = -b;
            if (warm) {
                T s = T(0);
                const int diag = for_neighbours(g, c, k, [&](unsigned o) { s += p[o]; });
                rc -= T(diag) * p[c] - s;
            }
        }
        if (!warm) p[c] = T(0);
        r[c] = rc;
        bb.add(b, b);
        rr.add(rc, rc);
    }
    const double acc[2] = {bb.value(), rr.value()};
    block_sums<2>(acc, part);
}

// Final sums of nv partial rows into sums[0..nv).
__global__ void k_finish(const double* part, int nblocks, int nv, double* sums) {
    __shared__ double sh[4][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < nv; ++q) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += part[b + nblocks * q];
        s = warp_sum(s);
        if (lane == 0) sh[q][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < nv; ++q) {
            double t = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[q][w];
            sums[q] = t;
        }
    }
}

// z = r / diag(B); rz; solver scalars initialised by the last block
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_pcg_init(PoissonGrid g, const T* __restrict__ r, T* __restrict__ z,
                                                           double* scal, double threshold, double rr0, double* part,
                                                           unsigned* ticket) {
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    DotAcc<T> rz;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        T zc = T(0);
        if (!excluded(g, c)) {
            const int diag = for_neighbours(g, c, decode(c, g.ny, g.nz), [](unsigned) {});
            zc = r[c] * inv_count<T>(diag);
        }
        z[c] = zc;
        rz.add(r[c], zc);
    }
    const double acc[1] = {rz.value()};
    block_sums<1>(acc, part);
    if (last_block(ticket)) {
        const double t = block_total(part, gridDim.x, 0);
        if (threadIdx.x == 0) {
            scal[S_ALPHA] = 0.0; scal[S_BETA] = 0.0; scal[S_RZ] = t; scal[S_RR] = rr0;
            scal[S_THRESH] = threshold; scal[S_DONE] = rr0 <= threshold ? 1.0 : 0.0; scal[S_ITERS] = 0.0;
            scal[S_DQ] = 0.0;
            *ticket = 0;
        }
    }
}

// ---------------------------------------------------------------------------------
// per-iteration kernels, W consecutive cells of a z-line per thread and loop trip
// (float4 / double2 loads when nz is a multiple of W; W = 1 otherwise)
// ---------------------------------------------------------------------------------
template <typename T, int W>
__device__ __forceinline__ void ldv(const T* __restrict__ p, T (&v)[W]) {
    if constexpr (W == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else if constexpr (W == 2) {
        const double2 t = *reinterpret_cast<const double2*>(p);
        v[0] = t.x; v[1] = t.y;
    } else {
        v[0] = p[0];
    }
}
template <typename T, int W>
__device__ __forceinline__ void stv(T* __restrict__ p, const T (&v)[W]) {
    if constexpr (W == 4) *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    else if constexpr (W == 2) *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    else p[0] = v[0];
}

// warp sum of a float-float accumulator; lane 0 holds the total
__device__ __forceinline__ double warp_total(const DotAcc<float>& a) {
    float hi = a.hi, lo = a.lo;
    for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, hi, o), l2 = __shfl_down_sync(0xffffffffu, lo, o);
        const float s = __fadd_rn(hi, h2);
        const float bb = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
        hi = s;
        lo = __fadd_rn(__fadd_rn(lo, l2), e);
    }
    return (double)hi + (double)lo;
}
__device__ __forceinline__ double warp_total(const DotAcc<double>& a) { return warp_sum(a.s); }

// block sums of NV accumulators into part[b + nb*q] (FP64 conversions only per warp)
template <typename T, int NV>
__device__ __forceinline__ void block_dots(const DotAcc<T> (&acc)[NV], double* part) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const double t = warp_total(acc[q]);
        if (lane == 0) sh[q][wid] = t;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double v = lane < nw ? sh[q][lane] : 0.0;
            v = warp_sum(v);
            if (lane == 0) part[blockIdx.x + gridDim.x * q] = v;
        }
    }
}

// diagonal of B at cell c0 + e of a group (walls and solid neighbours removed)
template <int W>
__device__ __forceinline__ int diag_at(const PoissonGrid& g, unsigned c0, const Cell& k, int e) {
    const unsigned sx = (unsigned)g.ny * g.nz, sy = (unsigned)g.nz, c = c0 + e;
    int d = 0;
    auto nb = [&](bool ok, unsigned o) { if (ok && !(g.solid && g.solid[o])) ++d; };
    nb(k.ix > 0, c - sx);
    nb(k.ix < g.nx - 1, c + sx);
    nb(k.iy > 0, c - sy);
    nb(k.iy < g.ny - 1, c + sy);
    nb(e > 0 || k.iz > 0, c - 1);
    nb(e < W - 1 || k.iz + W < g.nz, c + 1);
    return d;
}

// d_new = z + beta d_old (d_new = z on the first iteration);  q = B d_new;
// alpha = rz / (d_new.q), or (d_new.r) / (d_new.q) when r is given (flexible CG: exact line
// search along d whatever the preconditioner did)
template <typename T, int W>
__global__ void __launch_bounds__(kRedThreads) k_cg_direction_apply(PoissonGrid g, double* __restrict__ scal,
                                                                     const T* __restrict__ z, const T* __restrict__ dold,
                                                                     T* __restrict__ dnew, T* __restrict__ q, int first,
                                                                     const T* __restrict__ rres, double* part,
                                                                     unsigned* ticket) {
    if (scal[S_DONE] != 0.0) return;
    const unsigned n = (unsigned)g.nx * g.ny * g.nz, ngr = n / W;
    const unsigned sx = (unsigned)g.ny * g.nz, sy = (unsigned)g.nz;
    const T beta = (T)scal[S_BETA];
    auto dvec = [&](unsigned o0, T (&o)[W]) {
        ldv<T, W>(z + o0, o);
        if (!first) {
            T b[W];
            ldv<T, W>(dold + o0, b);
#pragma unroll
            for (int e = 0; e < W; ++e) o[e] += beta * b[e];
        }
    };
    auto d1 = [&](unsigned o) -> T { return first ? z[o] : z[o] + beta * dold[o]; };
    DotAcc<T> acc[2];
    for (unsigned gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngr; gi += gridDim.x * blockDim.x) {
        const unsigned c0 = gi * W;
        const Cell k = decode(c0, g.ny, g.nz);
        T dc[W], s[W];
        int dg[W];
        dvec(c0, dc);
#pragma unroll
        for (int e = 0; e < W; ++e) { s[e] = T(0); dg[e] = 0; }
        auto side = [&](bool ok, unsigned o0) {
            if (!ok) return;
            T nv[W];
            dvec(o0, nv);
#pragma unroll
            for (int e = 0; e < W; ++e) {
                const unsigned o = o0 + e;
                if (g.solid && g.solid[o]) continue;
                ++dg[e];
                if ((int)o != g.pin) s[e] += nv[e];
            }
        };
        side(k.ix > 0, c0 - sx);
        side(k.ix < g.nx - 1, c0 + sx);
        side(k.iy > 0, c0 - sy);
        side(k.iy < g.ny - 1, c0 + sy);
#pragma unroll
        for (int e = 0; e < W; ++e) {
            const unsigned c = c0 + e;
            if (e > 0 || k.iz > 0) {
                const unsigned o = c - 1;
                if (!(g.solid && g.solid[o])) { ++dg[e]; if ((int)o != g.pin) s[e] += e > 0 ? dc[e - 1] : d1(o); }
            }
            if (e < W - 1 || k.iz + W < g.nz) {
                const unsigned o = c + 1;
                if (!(g.solid && g.solid[o])) { ++dg[e]; if ((int)o != g.pin) s[e] += e < W - 1 ? dc[e + 1] : d1(o); }
            }
        }
        T qv[W];
#pragma unroll
        for (int e = 0; e < W; ++e) {
            qv[e] = excluded(g, c0 + e) ? T(0) : T(dg[e]) * dc[e] - s[e];
            acc[0].add(dc[e], qv[e]);
        }
        stv<T, W>(dnew + c0, dc);
        stv<T, W>(q + c0, qv);
        if (rres) {
            T rv[W];
            ldv<T, W>(rres + c0, rv);
#pragma unroll
            for (int e = 0; e < W; ++e) acc[1].add(dc[e], rv[e]);
        }
    }
    block_dots<T, 2>(acc, part);
    if (last_block(ticket)) {
        const double t = block_total(part, gridDim.x, 0);
        const double tr = rres ? block_total(part, gridDim.x, 1) : 0.0;
        if (threadIdx.x == 0) {
            const double num = rres ? tr : scal[S_RZ];
            scal[S_ALPHA] = t != 0.0 ? num / t : 0.0;
            scal[S_DQ] = t;
            *ticket = 0;
        }
    }
}

// r = rhs - B p on the free cells; partials |r|^2
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_residual(PoissonGrid g, const T* __restrict__ rhs,
                                                           const T* __restrict__ p, T* __restrict__ r, double* part) {
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    DotAcc<T> rr;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        T rc = T(0);
        if (!excluded(g, c)) {
            T s = T(0);
            const int diag = for_neighbours(g, c, decode(c, g.ny, g.nz), [&](unsigned o) { s += p[o]; });
            rc = rhs[c] - (T(diag) * p[c] - s);
        }
        r[c] = rc;
        rr.add(rc, rc);
    }
    const double acc[1] = {rr.value()};
    block_sums<1>(acc, part);
}

// x += alpha d; r -= alpha q; rr; with jacobi: z = r / diag, rz, beta = rz_new / rz_old.
template <typename T, int W>
__global__ void __launch_bounds__(kRedThreads) k_cg_update(PoissonGrid g, double* __restrict__ scal, T* __restrict__ x,
                                                            T* __restrict__ r, const T* __restrict__ d,
                                                            const T* __restrict__ q, T* __restrict__ z, int jacobi,
                                                            double* part, unsigned* ticket) {
    if (scal[S_DONE] != 0.0) return;
    const unsigned n = (unsigned)g.nx * g.ny * g.nz, ngr = n / W;
    const T a = (T)scal[S_ALPHA];
    DotAcc<T> acc[2];   // rz, rr
    for (unsigned gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngr; gi += gridDim.x * blockDim.x) {
        const unsigned c0 = gi * W;
        T xv[W], dv[W], rv[W], qv[W];
        ldv<T, W>(x + c0, xv); ldv<T, W>(d + c0, dv); ldv<T, W>(r + c0, rv); ldv<T, W>(q + c0, qv);
#pragma unroll
        for (int e = 0; e < W; ++e) {
            xv[e] += a * dv[e];
            rv[e] -= a * qv[e];
            acc[1].add(rv[e], rv[e]);
        }
        stv<T, W>(x + c0, xv);
        stv<T, W>(r + c0, rv);
        if (jacobi) {
            const Cell k = decode(c0, g.ny, g.nz);
            T zv[W];
#pragma unroll
            for (int e = 0; e < W; ++e) {
                zv[e] = excluded(g, c0 + e) ? T(0) : rv[e] * inv_count<T>(diag_at<W>(g, c0, k, e));
                acc[0].add(rv[e], zv[e]);
            }
            stv<T, W>(z + c0, zv);
        }
    }
    block_dots<T, 2>(acc, part);
    if (last_block(ticket)) {
        const double trz = block_total(part, gridDim.x, 0);
        const double trr = block_total(part, gridDim.x, 1);
        if (threadIdx.x == 0) {
            if (jacobi) {
                scal[S_BETA] = scal[S_RZ] != 0.0 ? trz / scal[S_RZ] : 0.0;
                scal[S_RZ] = trz;
            }
            scal[S_RR] = trr;
            scal[S_ITERS] += 1.0;
            if (trr <= scal[S_THRESH]) scal[S_DONE] = 1.0;
            *ticket = 0;
        }
    }
}

// flexible CG with m kept directions (Notay's FCG(m)):
//   beta_j = -(z.q_j)/(d_j.q_j) for the kept directions j;  d = z + sum_j beta_j d_j;
//   q = B d;  alpha = (d.r)/(d.q)
template <typename T>
struct DirSet {
    const T* v[kFcgMaxDirs];
    int slot[kFcgMaxDirs];
    int n;
};

template <typename T, int W>
__global__ void __launch_bounds__(kRedThreads) k_fcgm_dots(unsigned n, double* __restrict__ scal, const T* __restrict__ z,
                                                            const T* __restrict__ r, DirSet<T> qs, double* part,
                                                            unsigned* ticket) {
    if (scal[S_DONE] != 0.0) return;
    const unsigned ngr = n / W;
    DotAcc<T> acc[kFcgMaxDirs + 1];   // z.q_j, then z.r
    for (unsigned gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngr; gi += gridDim.x * blockDim.x) {
        const unsigned c0 = gi * W;
        T zv[W], v[W];
        ldv<T, W>(z + c0, zv);
        ldv<T, W>(r + c0, v);
#pragma unroll
        for (int e = 0; e < W; ++e) acc[kFcgMaxDirs].add(zv[e], v[e]);
#pragma unroll
        for (int j = 0; j < kFcgMaxDirs; ++j) {
            if (j >= qs.n) break;
            ldv<T, W>(qs.v[j] + c0, v);
#pragma unroll
            for (int e = 0; e < W; ++e) acc[j].add(zv[e], v[e]);
        }
    }
    block_dots<T, kFcgMaxDirs + 1>(acc, part);
    if (last_block(ticket)) {
        double t[kFcgMaxDirs + 1];
        for (int j = 0; j <= kFcgMaxDirs; ++j) t[j] = (j < qs.n || j == kFcgMaxDirs) ? block_total(part, gridDim.x, j) : 0.0;
        if (threadIdx.x == 0) {
            for (int j = 0; j < qs.n; ++j) {
                const double dq = scal[S_DQJ + qs.slot[j]];
                scal[S_BETAJ + qs.slot[j]] = dq != 0.0 ? -t[j] / dq : 0.0;
            }
            scal[S_RZ] = t[kFcgMaxDirs];
            *ticket = 0;
        }
    }
}

// d_new = z + sum_j beta_j d_j (streamed once; the stencil kernel below then reads d_new
// instead of recomputing it for each neighbour)
template <typename T, int W>
__global__ void __launch_bounds__(kRedThreads) k_fcgm_combine(unsigned n, const double* __restrict__ scal,
                                                               const T* __restrict__ z, DirSet<T> ds,
                                                               T* __restrict__ dnew) {
    if (scal[S_DONE] != 0.0) return;
    const unsigned ngr = n / W;
    T beta[kFcgMaxDirs];
#pragma unroll
    for (int j = 0; j < kFcgMaxDirs; ++j) beta[j] = j < ds.n ? (T)scal[S_BETAJ + ds.slot[j]] : T(0);
    for (unsigned gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngr; gi += gridDim.x * blockDim.x) {
        const unsigned c0 = gi * W;
        T o[W];
        ldv<T, W>(z + c0, o);
#pragma unroll
        for (int j = 0; j < kFcgMaxDirs; ++j) {
            if (j >= ds.n) break;
            T b[W];
            ldv<T, W>(ds.v[j] + c0, b);
#pragma unroll
            for (int e = 0; e < W; ++e) o[e] += beta[j] * b[e];
        }
        stv<T, W>(dnew + c0, o);
    }
}

// q = B d for d = z + sum_j beta_j d_j (with ds.n = 0 and dnew null: d = z, already combined);
// d.q and d.r; the last block sets alpha = d.r / d.q
template <typename T, int W>
__global__ void __launch_bounds__(kRedThreads) k_fcgm_direction(PoissonGrid g, double* __restrict__ scal,
                                                                 const T* __restrict__ z, DirSet<T> ds,
                                                                 T* __restrict__ dnew, T* __restrict__ qnew, int newslot,
                                                                 const T* __restrict__ rres, double* part,
                                                                 unsigned* ticket) {
    if (scal[S_DONE] != 0.0) return;
    const unsigned n = (unsigned)g.nx * g.ny * g.nz, ngr = n / W;
    const unsigned sx = (unsigned)g.ny * g.nz, sy = (unsigned)g.nz;
    T beta[kFcgMaxDirs];
#pragma unroll
    for (int j = 0; j < kFcgMaxDirs; ++j) beta[j] = j < ds.n ? (T)scal[S_BETAJ + ds.slot[j]] : T(0);
    auto dvec = [&](unsigned o0, T (&o)[W]) {
        ldv<T, W>(z + o0, o);
#pragma unroll
        for (int j = 0; j < kFcgMaxDirs; ++j) {
            if (j >= ds.n) break;
            T b[W];
            ldv<T, W>(ds.v[j] + o0, b);
#pragma unroll
            for (int e = 0; e < W; ++e) o[e] += beta[j] * b[e];
        }
    };
    auto d1 = [&](unsigned o) -> T {
        T v = z[o];
        for (int j = 0; j < ds.n; ++j) v += beta[j] * ds.v[j][o];
        return v;
    };
    DotAcc<T> acc[2];
    for (unsigned gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngr; gi += gridDim.x * blockDim.x) {
        const unsigned c0 = gi * W;
        const Cell k = decode(c0, g.ny, g.nz);
        T dc[W], s[W];
        int dg[W];
        dvec(c0, dc);
#pragma unroll
        for (int e = 0; e < W; ++e) { s[e] = T(0); dg[e] = 0; }
        auto side = [&](bool ok, unsigned o0) {
            if (!ok) return;
            T nv[W];
            dvec(o0, nv);
#pragma unroll
            for (int e = 0; e < W; ++e) {
                const unsigned o = o0 + e;
                if (g.solid && g.solid[o]) continue;
                ++dg[e];
                if ((int)o != g.pin) s[e] += nv[e];
            }
        };
        side(k.ix > 0, c0 - sx);
        side(k.ix < g.nx - 1, c0 + sx);
        side(k.iy > 0, c0 - sy);
        side(k.iy < g.ny - 1, c0 + sy);
#pragma unroll
        for (int e = 0; e < W; ++e) {
            const unsigned c = c0 + e;
            if (e > 0 || k.iz > 0) {
                const unsigned o = c - 1;
                if (!(g.solid && g.solid[o])) { ++dg[e]; if ((int)o != g.pin) s[e] += e > 0 ? dc[e - 1] : d1(o); }
            }
            if (e < W - 1 || k.iz + W < g.nz) {
                const unsigned o = c + 1;
                if (!(g.solid && g.solid[o])) { ++dg[e]; if ((int)o != g.pin) s[e] += e < W - 1 ? dc[e + 1] : d1(o); }
            }
        }
        T qv[W], rv[W];
        ldv<T, W>(rres + c0, rv);
#pragma unroll
        for (int e = 0; e < W; ++e) {
            qv[e] = excluded(g, c0 + e) ? T(0) : T(dg[e]) * dc[e] - s[e];
            acc[0].add(dc[e], qv[e]);
            acc[1].add(dc[e], rv[e]);
        }
        if (dnew) stv<T, W>(dnew + c0, dc);
        stv<T, W>(qnew + c0, qv);
    }
    block_dots<T, 2>(acc, part);
    if (last_block(ticket)) {
        const double t = block_total(part, gridDim.x, 0);
        const double tr = block_total(part, gridDim.x, 1);
        if (threadIdx.x == 0) {
            scal[S_ALPHA] = t != 0.0 ? tr / t : 0.0;
            scal[S_DQJ + newslot] = t;
            *ticket = 0;
        }
    }
}

__global__ void k_fcg_begin(double* scal, double threshold, double rr0) {
    scal[S_ALPHA] = 0.0; scal[S_BETA] = 0.0; scal[S_RZ] = 0.0; scal[S_RR] = rr0;
    scal[S_THRESH] = threshold; scal[S_DONE] = rr0 <= threshold ? 1.0 : 0.0; scal[S_ITERS] = 0.0; scal[S_DQ] = 0.0;
}

// u -= (p_i - p_{i-1}) / h on faces between two fluid cells (calc_pressure_3d.cpp:196-232);
// faces touching a solid cell are set to the solid's (zero) velocity.
template <typename T, typename P>
__global__ void k_subtract_gradient(PoissonGrid g, P invh, const P* __restrict__ p, T* __restrict__ u,
                                    T* __restrict__ v, T* __restrict__ w) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const unsigned nu = (unsigned)(nx + 1) * ny * nz, nv = (unsigned)nx * (ny + 1) * nz;
    const unsigned nw = (unsigned)nx * ny * (nz + 1);
    const unsigned tot = nu + nv + nw;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += gridDim.x * blockDim.x) {
        T* f; unsigned i, c, cm; bool interior;
        if (t < nu) {
            i = t; f = u;
            const Cell k = decode(i, ny, nz);
            interior = k.ix >= 1 && k.ix < nx;
            c = ((unsigned)k.ix * ny + k.iy) * nz + k.iz; cm = c - (unsigned)ny * nz;
        } else if (t < nu + nv) {
            i = t - nu; f = v;
            const Cell k = decode(i, ny + 1, nz);
            interior = k.iy >= 1 && k.iy < ny;
            c = ((unsigned)k.ix * ny + k.iy) * nz + k.iz; cm = c - nz;
        } else {
            i = t - nu - nv; f = w;
            const Cell k = decode(i, ny, nz + 1);
            interior = k.iz >= 1 && k.iz < nz;
            c = ((unsigned)k.ix * ny + k.iy) * nz + k.iz; cm = c - 1;
        }
        if (!interior) continue;
        if (g.solid && (g.solid[c] || g.solid[cm])) f[i] = T(0);
        else f[i] = (T)((P)f[i] - (p[c] - p[cm]) * invh);
    }
}

// wall momentum loss tallies (calc_pressure_3d.cpp:235-268)
template <typename T>
__global__ void k_wall_loss(int nx, int ny, int nz, double h, const T* __restrict__ p, double* part) {
    double acc[3] = {0.0, 0.0, 0.0};
    const long long nyz = (long long)ny * nz, nxz = (long long)nx * nz, nxy = (long long)nx * ny;
    const long long tot = nyz + nxz + nxy;
    const double h2 = h * h;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
        if (t < nyz) {
            const int iy = (int)(t / nz), iz = (int)(t % nz);
            acc[0] += -(double)p[((long long)0 * ny + iy) * nz + iz] * h2 + (double)p[((long long)(nx - 1) * ny + iy) * nz + iz] * h2;
        } else if (t < nyz + nxz) {
            const long long s = t - nyz;
            const int ix = (int)(s / nz), iz = (int)(s % nz);
            acc[1] += -(double)p[((long long)ix * ny + 0) * nz + iz] * h2 + (double)p[((long long)ix * ny + ny - 1) * nz + iz] * h2;
        } else {
            const long long s = t - nyz - nxz;
            const int ix = (int)(s / ny), iy = (int)(s % ny);
            acc[2] += -(double)p[((long long)ix * ny + iy) * nz + 0] * h2 + (double)p[((long long)ix * ny + iy) * nz + nz - 1] * h2;
        }
    }
    block_sums<3>(acc, part);
}

// ---------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------
template <typename T> struct VecW;
template <> struct VecW<float> { static constexpr int W = 4; };
template <> struct VecW<double> { static constexpr int W = 2; };

template <typename T>
void launch_direction(const PressureWork<T>& W, const PoissonGrid& g, const T* dold, T* dnew, bool first, const T* rres,
                      double* part, unsigned* ticket, cudaStream_t s) {
    constexpr int V = VecW<T>::W;
    if (g.nz % V == 0)
        k_cg_direction_apply<T, V><<<kRedBlocks, kRedThreads, 0, s>>>(g, W.scal, W.z, dold, dnew, W.q, first ? 1 : 0,
                                                                       rres, part, ticket);
    else
        k_cg_direction_apply<T, 1><<<kRedBlocks, kRedThreads, 0, s>>>(g, W.scal, W.z, dold, dnew, W.q, first ? 1 : 0,
                                                                       rres, part, ticket);
}

template <typename T>
void launch_update(const PressureWork<T>& W, const PoissonGrid& g, const T* d, bool jacobi, double* part,
                   unsigned* ticket, cudaStream_t s, const T* q = nullptr) {
    constexpr int V = VecW<T>::W;
    if (!q) q = W.q;
    if (g.nz % V == 0)
        k_cg_update<T, V><<<kRedBlocks, kRedThreads, 0, s>>>(g, W.scal, W.p, W.r, d, q, W.z, jacobi ? 1 : 0, part,
                                                              ticket);
    else
        k_cg_update<T, 1><<<kRedBlocks, kRedThreads, 0, s>>>(g, W.scal, W.p, W.r, d, q, W.z, jacobi ? 1 : 0, part,
                                                              ticket);
}
template <typename T>
cudaError_t pressure_rhs(const PressureWork<T>& W, const PoissonGrid& g, double h, const T* u, const T* v,
                         const T* w, bool warm, double* bb_rr_host, cudaStream_t s) {
    k_rhs<T><<<kRedBlocks, kRedThreads, 0, s>>>(g, (T)h, u, v, w, W.r, W.p, warm ? 1 : 0, W.part);
    k_finish<<<1, 256, 0, s>>>(W.part, kRedBlocks, 2, W.sums);
    cudaMemcpyAsync(bb_rr_host, W.sums, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    return cudaStreamSynchronize(s);
}

template <typename T>
cudaError_t pressure_pcg(const PressureWork<T>& W, const PoissonGrid& g, double bb, double rr0, double tol,
                         int max_iter, PressureReport* rep, cudaStream_t s) {
    const int nb = kRedBlocks, nt = kRedThreads;
    rep->launches = 1;
    k_pcg_init<T><<<nb, nt, 0, s>>>(g, W.r, W.z, W.scal, tol * tol * bb, rr0, W.part, W.ticket);
    // iterations are enqueued in batches; the device flag turns the rest of a batch into
    // empty launches once the residual is below tolerance
    T* dold = W.d;
    T* dnew = W.d2;
    int launched = 0;
    double st[3] = {rr0 <= tol * tol * bb ? 1.0 : 0.0, 0.0, rr0};   // done, iterations, rr
    while (launched < max_iter && st[0] == 0.0) {
        const int batch = std::min(kCgBatch, max_iter - launched);
        for (int b = 0; b < batch; ++b) {
            launch_direction<T>(W, g, dold, dnew, launched + b == 0, nullptr, W.part, W.ticket, s);
            launch_update<T>(W, g, dnew, true, W.part + 2 * nb, W.ticket + 1, s);
            std::swap(dold, dnew);
        }
        launched += batch;
        rep->launches += 2 * batch;
        double tail[4];
        cudaMemcpyAsync(tail, W.scal + S_RR, 4 * sizeof(double), cudaMemcpyDeviceToHost, s);
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        st[0] = tail[S_DONE - S_RR]; st[1] = tail[S_ITERS - S_RR]; st[2] = tail[0];
    }
    rep->iterations = (int)st[1];
    rep->rel_residual = bb > 0.0 ? std::sqrt(st[2] / bb) : 0.0;
    rep->status = st[0] == 0.0 ? 1 : 0;
    return cudaGetLastError();
}

template <typename T>
cudaError_t pressure_solve(const PressureWork<T>& W, const PoissonGrid& g, double h, const T* u, const T* v,
                           const T* w, double tol, int max_iter, PressureReport* rep, cudaStream_t s) {
    double br[2];
    cudaError_t e = pressure_rhs<T>(W, g, h, u, v, w, false, br, s);
    if (e != cudaSuccess) return e;
    rep->iterations = 0; rep->rel_residual = 0.0; rep->status = 0; rep->launches = 2; rep->bb = br[0];
    if (br[0] == 0.0) return cudaGetLastError();
    PressureReport r2;
    e = pressure_pcg<T>(W, g, br[0], br[1], tol, max_iter, &r2, s);
    r2.launches += 2;
    r2.bb = br[0];
    *rep = r2;
    return e;
}

template <typename T>
cudaError_t pressure_residual(const PressureWork<T>& W, const PoissonGrid& g, const T* rhs, double* rr_host,
                              cudaStream_t s) {
    k_residual<T><<<kRedBlocks, kRedThreads, 0, s>>>(g, rhs, W.p, W.r, W.part);
    k_finish<<<1, 256, 0, s>>>(W.part, kRedBlocks, 1, W.sums);
    cudaMemcpyAsync(rr_host, W.sums, sizeof(double), cudaMemcpyDeviceToHost, s);
    return cudaStreamSynchronize(s);
}

template <typename T>
cudaError_t fcg_begin(const PressureWork<T>& W, double bb, double rr0, double tol, cudaStream_t s) {
    k_fcg_begin<<<1, 1, 0, s>>>(W.scal, tol * tol * bb, rr0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t fcg_iteration(const PressureWork<T>& W, const PoissonGrid& g, const FcgBuffers<T>& B, int it, int m,
                          cudaStream_t s) {
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    const int nb = kRedBlocks, nt = kRedThreads;
    m = std::max(1, std::min(m, kFcgMaxDirs));
    const int ring = m + 1, newslot = it % ring;
    DirSet<T> qs, ds;
    qs.n = ds.n = std::min(it, m);
    for (int j = 0; j < qs.n; ++j) {
        const int sl = (it - 1 - j) % ring;
        qs.v[j] = B.q[sl]; qs.slot[j] = sl;
        ds.v[j] = B.d[sl]; ds.slot[j] = sl;
    }
    constexpr int V = VecW<T>::W;
    DirSet<T> none = ds;
    none.n = 0;
    if (g.nz % V == 0) {
        k_fcgm_dots<T, V><<<nb, nt, 0, s>>>(n, W.scal, W.z, W.r, qs, W.part, W.ticket);
        k_fcgm_combine<T, V><<<nb, nt, 0, s>>>(n, W.scal, W.z, ds, B.d[newslot]);
        k_fcgm_direction<T, V><<<nb, nt, 0, s>>>(g, W.scal, B.d[newslot], none, (T*)nullptr, B.q[newslot], newslot,
                                                 W.r, W.part + (kFcgMaxDirs + 1) * nb, W.ticket + 1);
    } else {
        k_fcgm_dots<T, 1><<<nb, nt, 0, s>>>(n, W.scal, W.z, W.r, qs, W.part, W.ticket);
        k_fcgm_combine<T, 1><<<nb, nt, 0, s>>>(n, W.scal, W.z, ds, B.d[newslot]);
        k_fcgm_direction<T, 1><<<nb, nt, 0, s>>>(g, W.scal, B.d[newslot], none, (T*)nullptr, B.q[newslot], newslot,
                                                 W.r, W.part + (kFcgMaxDirs + 1) * nb, W.ticket + 1);
    }
    launch_update<T>(W, g, B.d[newslot], false, W.part, W.ticket + 2, s, B.q[newslot]);
    return cudaGetLastError();
}

cudaError_t solver_state(const double* scal, double out[3], cudaStream_t s) {
    double tail[4];
    cudaMemcpyAsync(tail, scal + S_RR, 4 * sizeof(double), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    out[0] = tail[0]; out[1] = tail[S_DONE - S_RR]; out[2] = tail[S_ITERS - S_RR];
    return e;
}

template <typename T>
cudaError_t subtract_gradient(const T* p, T* u, T* v, T* w, const PoissonGrid& g, double h, double* loss_part,
                              double* loss_sums, cudaStream_t s) {
    k_subtract_gradient<T, T><<<kRedBlocks, kRedThreads, 0, s>>>(g, (T)(1.0 / h), p, u, v, w);
    k_wall_loss<T><<<kRedBlocks, kRedThreads, 0, s>>>(g.nx, g.ny, g.nz, h, p, loss_part);
    k_finish<<<1, 256, 0, s>>>(loss_part, kRedBlocks, 3, loss_sums);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// FP64 residual refinement of the FP32 form
// ---------------------------------------------------------------------------------
// r = -b - B p64 in FP64 arithmetic (b = div(u) h from the FP32 velocities), stored as FP32
// for the next correction solve; partial |r|^2
__global__ void __launch_bounds__(kRedThreads) k_true_residual(PoissonGrid g, double h, const float* __restrict__ u,
                                                                const float* __restrict__ v, const float* __restrict__ w,
                                                                const double* __restrict__ p, float* __restrict__ r,
                                                                double* part) {
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    const int ny = g.ny, nz = g.nz;
    double acc = 0.0;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        double rc = 0.0;
        if (!excluded(g, c)) {
            const Cell k = decode(c, ny, nz);
            const double b = net_outflow<double>(g, c, k, u, v, w) * h;
            double s = 0.0;
            const int diag = for_neighbours(g, c, k, [&](unsigned o) { s += p[o]; });
            rc = -b - ((double)diag * p[c] - s);
        }
        r[c] = (float)rc;
        acc += rc * rc;
    }
    const double a[1] = {acc};
    block_sums<1>(a, part);
}

__global__ void k_to_double(const float* __restrict__ a, double* __restrict__ b, unsigned n, int accumulate) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        b[i] = accumulate ? b[i] + (double)a[i] : (double)a[i];
}
__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, unsigned n) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = (float)a[i];
}

cudaError_t true_residual(const PressureWork<float>& W, const PoissonGrid& g, double h, const float* u,
                          const float* v, const float* w, const double* p64, double* rr_host, cudaStream_t s) {
    k_true_residual<<<kRedBlocks, kRedThreads, 0, s>>>(g, h, u, v, w, p64, W.r, W.part);
    k_finish<<<1, 256, 0, s>>>(W.part, kRedBlocks, 1, W.sums);
    cudaMemcpyAsync(rr_host, W.sums, sizeof(double), cudaMemcpyDeviceToHost, s);
    return cudaStreamSynchronize(s);
}

cudaError_t widen(const float* a, double* b, long long n, bool accumulate, cudaStream_t s) {
    k_to_double<<<kRedBlocks, kRedThreads, 0, s>>>(a, b, (unsigned)n, accumulate ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t narrow(const double* a, float* b, long long n, cudaStream_t s) {
    k_to_float<<<kRedBlocks, kRedThreads, 0, s>>>(a, b, (unsigned)n);
    return cudaGetLastError();
}

cudaError_t subtract_gradient_p64(const double* p64, float* u, float* v, float* w, const PoissonGrid& g, double h,
                                  double* loss_part, double* loss_sums, cudaStream_t s) {
    k_subtract_gradient<float, double><<<kRedBlocks, kRedThreads, 0, s>>>(g, 1.0 / h, p64, u, v, w);
    k_wall_loss<double><<<kRedBlocks, kRedThreads, 0, s>>>(g.nx, g.ny, g.nz, h, p64, loss_part);
    k_finish<<<1, 256, 0, s>>>(loss_part, kRedBlocks, 3, loss_sums);
    return cudaGetLastError();
}

// partial rows: the FCG dot kernel's kFcgMaxDirs + 1 and the direction kernel's 2 (the CG
// kernels use fewer)
size_t pressure_partials() { return (size_t)kRedBlocks * (kFcgMaxDirs + 4); }

#define FIA_PRESSURE_INST(T)                                                                                       \
    template cudaError_t pressure_rhs<T>(const PressureWork<T>&, const PoissonGrid&, double, const T*, const T*,    \
                                         const T*, bool, double*, cudaStream_t);                                    \
    template cudaError_t pressure_pcg<T>(const PressureWork<T>&, const PoissonGrid&, double, double, double, int,   \
                                         PressureReport*, cudaStream_t);                                            \
    template cudaError_t pressure_solve<T>(const PressureWork<T>&, const PoissonGrid&, double, const T*, const T*,  \
                                           const T*, double, int, PressureReport*, cudaStream_t);                   \
    template cudaError_t fcg_begin<T>(const PressureWork<T>&, double, double, double, cudaStream_t);               \
    template cudaError_t pressure_residual<T>(const PressureWork<T>&, const PoissonGrid&, const T*, double*,         \
                                              cudaStream_t);                                                          \
    template cudaError_t fcg_iteration<T>(const PressureWork<T>&, const PoissonGrid&, const FcgBuffers<T>&, int, int, \
                                          cudaStream_t);                                                              \
    template cudaError_t subtract_gradient<T>(const T*, T*, T*, T*, const PoissonGrid&, double, double*, double*,   \
                                              cudaStream_t);
FIA_PRESSURE_INST(double)
FIA_PRESSURE_INST(float)
#undef FIA_PRESSURE_INST

}  // namespace fia
