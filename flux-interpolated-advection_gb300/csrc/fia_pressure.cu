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

constexpr int kRedBlocks = 152 * 4;
constexpr int kRedThreads = 256;
constexpr int kCgBatch = 16;

// scal layout
enum : int { S_ALPHA = 0, S_BETA = 1, S_RZ = 2, S_RR = 3, S_THRESH = 4, S_DONE = 5, S_ITERS = 6, S_DQ = 7 };

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
            const unsigned u0 = c, u1 = c + (unsigned)ny * nz;
            const unsigned v0 = ((unsigned)k.ix * (ny + 1) + k.iy) * nz + k.iz, v1 = v0 + nz;
            const unsigned w0 = ((unsigned)k.ix * ny + k.iy) * (nz + 1) + k.iz, w1 = w0 + 1;
            b = ((u[u1] - u[u0]) + (v[v1] - v[v0]) + (w[w1] - w[w0])) * h;
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

// d_new = z + beta d_old (d_new = z on the first iteration);  q = B d_new;  alpha = rz / (d_new.q)
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_cg_direction_apply(PoissonGrid g, double* __restrict__ scal,
                                                                     const T* __restrict__ z, const T* __restrict__ dold,
                                                                     T* __restrict__ dnew, T* __restrict__ q, int first,
                                                                     double* part, unsigned* ticket) {
    if (scal[S_DONE] != 0.0) return;
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    const T beta = (T)scal[S_BETA];
    auto dval = [&](unsigned o) -> T { return first ? z[o] : z[o] + beta * dold[o]; };
    DotAcc<T> dq;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const T dc = dval(c);
        T qc = T(0);
        if (!excluded(g, c)) {
            T s = T(0);
            const int diag = for_neighbours(g, c, decode(c, g.ny, g.nz), [&](unsigned o) { s += dval(o); });
            qc = T(diag) * dc - s;
        }
        dnew[c] = dc;
        q[c] = qc;
        dq.add(dc, qc);
    }
    const double acc[1] = {dq.value()};
    block_sums<1>(acc, part);
    if (last_block(ticket)) {
        const double t = block_total(part, gridDim.x, 0);
        if (threadIdx.x == 0) {
            scal[S_ALPHA] = t != 0.0 ? scal[S_RZ] / t : 0.0;
            scal[S_DQ] = t;
            *ticket = 0;
        }
    }
}

// x += alpha d; r -= alpha q; rr; with jacobi: z = r / diag, rz, beta = rz_new / rz_old.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_cg_update(PoissonGrid g, double* __restrict__ scal, T* __restrict__ x,
                                                            T* __restrict__ r, const T* __restrict__ d,
                                                            const T* __restrict__ q, T* __restrict__ z, int jacobi,
                                                            double* part, unsigned* ticket) {
    if (scal[S_DONE] != 0.0) return;
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    const T a = (T)scal[S_ALPHA];
    DotAcc<T> rz, rr;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        x[c] = x[c] + a * d[c];
        const T rc = r[c] - a * q[c];
        r[c] = rc;
        rr.add(rc, rc);
        if (jacobi) {
            T zc = T(0);
            if (!excluded(g, c)) {
                const int diag = for_neighbours(g, c, decode(c, g.ny, g.nz), [](unsigned) {});
                zc = rc * inv_count<T>(diag);
            }
            z[c] = zc;
            rz.add(rc, zc);
        }
    }
    const double acc[2] = {rz.value(), rr.value()};
    block_sums<2>(acc, part);
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

// flexible CG: beta = -(z.q_old)/(d_old.q_old) (first: 0); rz = z.r
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_fcg_dots(unsigned n, double* __restrict__ scal, const T* __restrict__ z,
                                                           const T* __restrict__ qold, const T* __restrict__ r, int first,
                                                           double* part, unsigned* ticket) {
    if (scal[S_DONE] != 0.0) return;
    DotAcc<T> zq, zr;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const T zc = z[c];
        if (!first) zq.add(zc, qold[c]);
        zr.add(zc, r[c]);
    }
    const double acc[2] = {zq.value(), zr.value()};
    block_sums<2>(acc, part);
    if (last_block(ticket)) {
        const double tzq = block_total(part, gridDim.x, 0);
        const double tzr = block_total(part, gridDim.x, 1);
        if (threadIdx.x == 0) {
            scal[S_BETA] = (first || scal[S_DQ] == 0.0) ? 0.0 : -tzq / scal[S_DQ];
            scal[S_RZ] = tzr;
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
template <typename T>
__global__ void k_subtract_gradient(PoissonGrid g, T invh, const T* __restrict__ p, T* __restrict__ u,
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
        else f[i] = f[i] - (p[c] - p[cm]) * invh;
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
            k_cg_direction_apply<T><<<nb, nt, 0, s>>>(g, W.scal, W.z, dold, dnew, W.q, launched + b == 0 ? 1 : 0,
                                                      W.part, W.ticket);
            k_cg_update<T><<<nb, nt, 0, s>>>(g, W.scal, W.p, W.r, dnew, W.q, W.z, 1, W.part + 2 * nb, W.ticket + 1);
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
    rep->iterations = 0; rep->rel_residual = 0.0; rep->status = 0; rep->launches = 2;
    if (br[0] == 0.0) return cudaGetLastError();
    PressureReport r2;
    e = pressure_pcg<T>(W, g, br[0], br[1], tol, max_iter, &r2, s);
    r2.launches += 2;
    *rep = r2;
    return e;
}

template <typename T>
cudaError_t fcg_begin(const PressureWork<T>& W, double bb, double rr0, double tol, cudaStream_t s) {
    k_fcg_begin<<<1, 1, 0, s>>>(W.scal, tol * tol * bb, rr0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t fcg_iteration(const PressureWork<T>& W, const PoissonGrid& g, bool first, T* dold, T* dnew,
                          cudaStream_t s) {
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    const int nb = kRedBlocks, nt = kRedThreads;
    k_fcg_dots<T><<<nb, nt, 0, s>>>(n, W.scal, W.z, W.q, W.r, first ? 1 : 0, W.part, W.ticket);
    k_cg_direction_apply<T><<<nb, nt, 0, s>>>(g, W.scal, W.z, dold, dnew, W.q, first ? 1 : 0, W.part + 2 * nb,
                                              W.ticket + 1);
    k_cg_update<T><<<nb, nt, 0, s>>>(g, W.scal, W.p, W.r, dnew, W.q, W.z, 0, W.part, W.ticket + 2);
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
    k_subtract_gradient<T><<<kRedBlocks, kRedThreads, 0, s>>>(g, (T)(1.0 / h), p, u, v, w);
    k_wall_loss<T><<<kRedBlocks, kRedThreads, 0, s>>>(g.nx, g.ny, g.nz, h, p, loss_part);
    k_finish<<<1, 256, 0, s>>>(loss_part, kRedBlocks, 3, loss_sums);
    return cudaGetLastError();
}

size_t pressure_partials() { return (size_t)kRedBlocks * 4; }

#define FIA_PRESSURE_INST(T)                                                                                       \
    template cudaError_t pressure_rhs<T>(const PressureWork<T>&, const PoissonGrid&, double, const T*, const T*,    \
                                         const T*, bool, double*, cudaStream_t);                                    \
    template cudaError_t pressure_pcg<T>(const PressureWork<T>&, const PoissonGrid&, double, double, double, int,   \
                                         PressureReport*, cudaStream_t);                                            \
    template cudaError_t pressure_solve<T>(const PressureWork<T>&, const PoissonGrid&, double, const T*, const T*,  \
                                           const T*, double, int, PressureReport*, cudaStream_t);                   \
    template cudaError_t fcg_begin<T>(const PressureWork<T>&, double, double, double, cudaStream_t);               \
    template cudaError_t fcg_iteration<T>(const PressureWork<T>&, const PoissonGrid&, bool, T*, T*, cudaStream_t);  \
    template cudaError_t subtract_gradient<T>(const T*, T*, T*, T*, const PoissonGrid&, double, double*, double*,   \
                                              cudaStream_t);
FIA_PRESSURE_INST(double)
FIA_PRESSURE_INST(float)
#undef FIA_PRESSURE_INST

}  // namespace fia
