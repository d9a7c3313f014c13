// fia_pressure.cu -- pressure projection (calc_pressure_3d.cpp:18-270) on the GPU.
//
// The reference assembles a CSR 7-point Laplacian over all cells but the last one (pinned
// to p = 0), right-hand side b = div(u) h, and solves it with amgcl (SA-AMG + CG).  Here
// the same operator is applied matrix-free and solved with Jacobi-preconditioned CG on -A
// (symmetric positive definite on the N-1 free cells).  Dot products and norms are
// reduced deterministically (fixed per-block partials, one final block) in FP64.
#include "fia_pressure.cuh"

#include <cmath>

namespace fia {

constexpr int kRedBlocks = 1024;
constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-level sum of up to 3 values written to part[b + nb*slot].
template <int NV>
__device__ __forceinline__ void block_sums(double (&v)[NV], double* part) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = warp_sum(v[q]);
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

// -(A p) for the pinned operator; cells are (ix,iy,iz), z fastest.
template <typename T>
__device__ __forceinline__ double neg_apply(const T* __restrict__ p, int nx, int ny, int nz, long long c, long long last) {
    if (c == last) return 0.0;
    const int iz = (int)(c % nz), iy = (int)((c / nz) % ny), ix = (int)(c / ((long long)nz * ny));
    double diag = -6.0, s = 0.0;
    const long long sx = (long long)ny * nz, sy = nz;
    if (ix == 0) diag += 1.0; else { long long o = c - sx; if (o != last) s += (double)p[o]; }
    if (ix == nx - 1) diag += 1.0; else { long long o = c + sx; if (o != last) s += (double)p[o]; }
    if (iy == 0) diag += 1.0; else { long long o = c - sy; if (o != last) s += (double)p[o]; }
    if (iy == ny - 1) diag += 1.0; else { long long o = c + sy; if (o != last) s += (double)p[o]; }
    if (iz == 0) diag += 1.0; else { long long o = c - 1; if (o != last) s += (double)p[o]; }
    if (iz == nz - 1) diag += 1.0; else { long long o = c + 1; if (o != last) s += (double)p[o]; }
    return -(diag * (double)p[c] + s);
}

__device__ __forceinline__ double neg_diag(int nx, int ny, int nz, long long c) {
    const int iz = (int)(c % nz), iy = (int)((c / nz) % ny), ix = (int)(c / ((long long)nz * ny));
    double diag = -6.0;
    if (ix == 0) diag += 1.0;
    if (ix == nx - 1) diag += 1.0;
    if (iy == 0) diag += 1.0;
    if (iy == ny - 1) diag += 1.0;
    if (iz == 0) diag += 1.0;
    if (iz == nz - 1) diag += 1.0;
    return -diag;
}

// b = div(u) h (the last cell's equation is dropped); also |b|^2 partials.
template <typename T>
__global__ void k_rhs(int nx, int ny, int nz, double h, const T* __restrict__ u, const T* __restrict__ v,
                      const T* __restrict__ w, T* __restrict__ r, double* part) {
    const long long n = (long long)nx * ny * nz;
    double acc[1] = {0.0};
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(c % nz), iy = (int)((c / nz) % ny), ix = (int)(c / ((long long)nz * ny));
        double b = 0.0;
        if (c != n - 1) {
            const long long u0 = ((long long)ix * ny + iy) * nz + iz, u1 = ((long long)(ix + 1) * ny + iy) * nz + iz;
            const long long v0 = ((long long)ix * (ny + 1) + iy) * nz + iz, v1 = v0 + nz;
            const long long w0 = ((long long)ix * ny + iy) * (nz + 1) + iz, w1 = w0 + 1;
            b = ((double)u[u1] - (double)u[u0] + (double)v[v1] - (double)v[v0] + (double)w[w1] - (double)w[w0]) * h;
        }
        // CG works on -A p = -b; r0 = -b with p0 = 0
        r[c] = (T)(-b);
        acc[0] += b * b;
    }
    block_sums<1>(acc, part);
}

// q = -A d ; partial d.q
template <typename T>
__global__ void k_spmv(int nx, int ny, int nz, const T* __restrict__ d, T* __restrict__ q, double* part) {
    const long long n = (long long)nx * ny * nz;
    double acc[1] = {0.0};
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double qc = neg_apply(d, nx, ny, nz, c, n - 1);
        q[c] = (T)qc;
        acc[0] += (double)d[c] * qc;
    }
    block_sums<1>(acc, part);
}

// x += a d; r -= a q; z = r / diag; partials r.z and r.r   (a = scal[0])
template <typename T>
__global__ void k_update(int nx, int ny, int nz, const double* __restrict__ scal, T* __restrict__ x,
                         T* __restrict__ r, const T* __restrict__ d, const T* __restrict__ q, T* __restrict__ z,
                         double* part) {
    const long long n = (long long)nx * ny * nz;
    const double a = scal[0];
    double acc[2] = {0.0, 0.0};
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double xc = (double)x[c] + a * (double)d[c];
        const double rc = (double)r[c] - a * (double)q[c];
        x[c] = (T)xc;
        r[c] = (T)rc;
        const double zc = (c == n - 1) ? 0.0 : rc / neg_diag(nx, ny, nz, c);
        z[c] = (T)zc;
        acc[0] += rc * zc;
        acc[1] += rc * rc;
    }
    block_sums<2>(acc, part);
}

// z = r / diag, partial r.z (first iteration)
template <typename T>
__global__ void k_precond(int nx, int ny, int nz, const T* __restrict__ r, T* __restrict__ z, T* __restrict__ d,
                          T* __restrict__ x, double* part) {
    const long long n = (long long)nx * ny * nz;
    double acc[1] = {0.0};
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double rc = (double)r[c];
        const double zc = (c == n - 1) ? 0.0 : rc / neg_diag(nx, ny, nz, c);
        z[c] = (T)zc; d[c] = (T)zc; x[c] = (T)0;
        acc[0] += rc * zc;
    }
    block_sums<1>(acc, part);
}

// d = z + b d   (b = scal[1])
template <typename T>
__global__ void k_direction(long long n, const double* __restrict__ scal, const T* __restrict__ z, T* __restrict__ d) {
    const double b = scal[1];
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        d[c] = (T)((double)z[c] + b * (double)d[c]);
}

// Final reduction of the partials and the CG scalars, on one block.
//  op 0: sums[0..nv) = totals
//  op 1: alpha = rz / dq                      (scal[0]);  dq = total
//  op 2: beta = rz_new / rz; rz = rz_new      (scal[1], scal[2]); rr = total1
__global__ void k_finish(const double* part, int nblocks, int nv, int op, double* scal, double* sums) {
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
        double t[4] = {0, 0, 0, 0};
        for (int q = 0; q < nv; ++q) for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t[q] += sh[q][w];
        for (int q = 0; q < nv; ++q) sums[q] = t[q];
        if (op == 1) scal[0] = (t[0] != 0.0) ? scal[2] / t[0] : 0.0;
        if (op == 2) { scal[1] = (scal[2] != 0.0) ? t[0] / scal[2] : 0.0; scal[2] = t[0]; }
        if (op == 3) scal[2] = t[0];
    }
}

// u -= (p_i - p_{i-1}) / h on interior faces (calc_pressure_3d.cpp:196-232)
template <typename T>
__global__ void k_subtract_gradient(int nx, int ny, int nz, double h, const T* __restrict__ p, T* __restrict__ u,
                                    T* __restrict__ v, T* __restrict__ w) {
    const long long nu = (long long)(nx + 1) * ny * nz, nv = (long long)nx * (ny + 1) * nz;
    const long long nw = (long long)nx * ny * (nz + 1);
    const long long tot = nu + nv + nw;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
        if (t < nu) {
            const int iz = (int)(t % nz), iy = (int)((t / nz) % ny), ix = (int)(t / ((long long)nz * ny));
            if (ix >= 1 && ix < nx) {
                const long long c = ((long long)ix * ny + iy) * nz + iz, cm = c - (long long)ny * nz;
                u[t] = (T)((double)u[t] - ((double)p[c] - (double)p[cm]) / h);
            }
        } else if (t < nu + nv) {
            const long long s = t - nu;
            const int iz = (int)(s % nz), iy = (int)((s / nz) % (ny + 1)), ix = (int)(s / ((long long)nz * (ny + 1)));
            if (iy >= 1 && iy < ny) {
                const long long c = ((long long)ix * ny + iy) * nz + iz, cm = c - nz;
                v[s] = (T)((double)v[s] - ((double)p[c] - (double)p[cm]) / h);
            }
        } else {
            const long long s = t - nu - nv;
            const int iz = (int)(s % (nz + 1)), iy = (int)((s / (nz + 1)) % ny), ix = (int)(s / ((long long)(nz + 1) * ny));
            if (iz >= 1 && iz < nz) {
                const long long c = ((long long)ix * ny + iy) * nz + iz, cm = c - 1;
                w[s] = (T)((double)w[s] - ((double)p[c] - (double)p[cm]) / h);
            }
        }
    }
}

// wall momentum loss tallies (calc_pressure_3d.cpp:235-268)
template <typename T>
__global__ void k_wall_loss(int nx, int ny, int nz, double h, const T* __restrict__ p, double* part) {
    double acc[3] = {0.0, 0.0, 0.0};
    const long long nyz = (long long)ny * nz, nxz = (long long)nx * nz, nxy = (long long)nx * ny;
    const long long tot = nyz + nxz + nxy;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
        if (t < nyz) {
            const int iy = (int)(t / nz), iz = (int)(t % nz);
            acc[0] += -(double)p[((long long)0 * ny + iy) * nz + iz] * h * h + (double)p[((long long)(nx - 1) * ny + iy) * nz + iz] * h * h;
        } else if (t < nyz + nxz) {
            const long long s = t - nyz;
            const int ix = (int)(s / nz), iz = (int)(s % nz);
            acc[1] += -(double)p[((long long)ix * ny + 0) * nz + iz] * h * h + (double)p[((long long)ix * ny + ny - 1) * nz + iz] * h * h;
        } else {
            const long long s = t - nyz - nxz;
            const int ix = (int)(s / ny), iy = (int)(s % ny);
            acc[2] += -(double)p[((long long)ix * ny + iy) * nz + 0] * h * h + (double)p[((long long)ix * ny + iy) * nz + nz - 1] * h * h;
        }
    }
    block_sums<3>(acc, part);
}

template <typename T>
cudaError_t pressure_solve(const PressureWork<T>& W, int nx, int ny, int nz, double h, const T* u, const T* v,
                           const T* w, double tol, int max_iter, PressureReport* rep, cudaStream_t s) {
    const long long n = (long long)nx * ny * nz;
    const int nb = kRedBlocks, nt = kRedThreads;
    double* part = W.part; double* scal = W.scal; double* sums = W.sums;
    k_rhs<T><<<nb, nt, 0, s>>>(nx, ny, nz, h, u, v, w, W.r, part);
    k_finish<<<1, 256, 0, s>>>(part, nb, 1, 0, scal, sums);
    double bb = 0.0;
    cudaMemcpyAsync(&bb, sums, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    const double bn = std::sqrt(bb);
    rep->iterations = 0; rep->rel_residual = 0.0; rep->status = 0;
    k_precond<T><<<nb, nt, 0, s>>>(nx, ny, nz, W.r, W.z, W.d, W.p, part);
    k_finish<<<1, 256, 0, s>>>(part, nb, 1, 3, scal, sums);
    if (bn == 0.0) return cudaGetLastError();
    double rr = bb;
    int it = 0;
    for (; it < max_iter; ++it) {
        if (std::sqrt(rr) <= tol * bn) break;
        k_spmv<T><<<nb, nt, 0, s>>>(nx, ny, nz, W.d, W.q, part);
        k_finish<<<1, 256, 0, s>>>(part, nb, 1, 1, scal, sums);
        k_update<T><<<nb, nt, 0, s>>>(nx, ny, nz, scal, W.p, W.r, W.d, W.q, W.z, part);
        k_finish<<<1, 256, 0, s>>>(part, nb, 2, 2, scal, sums);
        k_direction<T><<<nb, nt, 0, s>>>(n, scal, W.z, W.d);
        cudaMemcpyAsync(&rr, sums + 1, sizeof(double), cudaMemcpyDeviceToHost, s);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
    }
    rep->iterations = it;
    rep->rel_residual = std::sqrt(rr) / bn;
    if (!(std::sqrt(rr) <= tol * bn)) rep->status = 1;
    return cudaGetLastError();
}

template <typename T>
cudaError_t subtract_gradient(const T* p, T* u, T* v, T* w, int nx, int ny, int nz, double h, double* loss_part,
                              double* loss_sums, cudaStream_t s) {
    k_subtract_gradient<T><<<kRedBlocks, kRedThreads, 0, s>>>(nx, ny, nz, h, p, u, v, w);
    k_wall_loss<T><<<kRedBlocks, kRedThreads, 0, s>>>(nx, ny, nz, h, p, loss_part);
    k_finish<<<1, 256, 0, s>>>(loss_part, kRedBlocks, 3, 0, nullptr, loss_sums);
    return cudaGetLastError();
}

size_t pressure_partials() { return (size_t)kRedBlocks * 4; }

template cudaError_t pressure_solve<double>(const PressureWork<double>&, int, int, int, double, const double*, const double*,
                                            const double*, double, int, PressureReport*, cudaStream_t);
template cudaError_t subtract_gradient<double>(const double*, double*, double*, double*, int, int, int, double, double*,
                                               double*, cudaStream_t);
template cudaError_t pressure_solve<float>(const PressureWork<float>&, int, int, int, double, const float*, const float*,
                                           const float*, double, int, PressureReport*, cudaStream_t);
template cudaError_t subtract_gradient<float>(const float*, float*, float*, float*, int, int, int, double, double*,
                                              double*, cudaStream_t);

}  // namespace fia
