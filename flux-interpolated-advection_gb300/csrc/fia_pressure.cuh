// fia_pressure.cuh -- matrix-free pressure projection (calc_pressure_3d.cpp:18-270).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace fia {

// The Poisson problem of one projection.  Cells flagged in `solid` (nullptr: none) are
// excluded like walls (zero-flux faces, p = 0 there); cell `pin` is held at p = 0 (the
// reference pins the last cell, calc_pressure_3d.cpp:25).
struct PoissonGrid {
    int nx, ny, nz;
    int pin;
    const unsigned char* solid;
};

// index of r.r in PressureWork::scal (read by the learned preconditioner)
constexpr int kScalRR = 3;

template <typename T>
struct PressureWork {
    T *p, *r, *z, *d, *d2, *q;  // N^3 each; p is the pressure
    double* part;               // pressure_partials() doubles
    double* scal;               // 8 doubles: alpha beta rz rr threshold done iterations dq
    double* sums;               // 4 doubles
    unsigned* ticket;           // 4 last-block counters (zero between kernels)
};

struct PressureReport {
    int iterations;
    double rel_residual;
    int status;               // 1: iteration cap reached before the tolerance
    int launches;             // kernels launched by the solve
};

size_t pressure_partials();

// r = -b - B p (warm) or r = -b, p = 0 (cold), b = div(u) h, B = -A; |b|^2 and |r|^2 into
// bb_rr_host[0..2) (synchronises the stream).
template <typename T>
cudaError_t pressure_rhs(const PressureWork<T>& W, const PoissonGrid& g, double h, const T* u, const T* v,
                         const T* w, bool warm, double* bb_rr_host, cudaStream_t s);

// Jacobi-PCG on B p = -b from the residual left by pressure_rhs, to |r|^2 <= tol^2 bb.
template <typename T>
cudaError_t pressure_pcg(const PressureWork<T>& W, const PoissonGrid& g, double bb, double rr0, double tol,
                         int max_iter, PressureReport* rep, cudaStream_t s);

// Solves A p = div(u) h for the reference operator to |r| <= tol |b| (Jacobi-PCG, cold start).
template <typename T>
cudaError_t pressure_solve(const PressureWork<T>& W, const PoissonGrid& g, double h, const T* u, const T* v,
                           const T* w, double tol, int max_iter, PressureReport* rep, cudaStream_t s);

// u -= grad p / h on faces between two fluid cells, 0 on faces touching a solid cell; wall
// momentum loss sums into loss_sums[0..3).
template <typename T>
cudaError_t subtract_gradient(const T* p, T* u, T* v, T* w, const PoissonGrid& g, double h, double* loss_part,
                              double* loss_sums, cudaStream_t s);

// Flexible CG (FCG(1)) around a preconditioner that writes z = M(r) between iterations:
//   dots:       beta = -(z.q_old)/(d_old.q_old) (0 on the first iteration), rz = z.r
//   direction:  d = z + beta d_old, q = B d, alpha = rz / (d.q)
//   update:     p += alpha d, r -= alpha q, rr = r.r, done flag when rr <= tol^2 bb
template <typename T>
cudaError_t fcg_begin(const PressureWork<T>& W, double bb, double rr0, double tol, cudaStream_t s);
template <typename T>
cudaError_t fcg_iteration(const PressureWork<T>& W, const PoissonGrid& g, bool first, T* dold, T* dnew,
                          cudaStream_t s);

// out = {rr, done, iterations} (synchronises the stream)
cudaError_t solver_state(const double* scal, double out[3], cudaStream_t s);

}  // namespace fia
