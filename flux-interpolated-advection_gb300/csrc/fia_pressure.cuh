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
constexpr int kScalDoubles = 48;
// directions kept by flexible CG (FCG(m), m <= kFcgMaxDirs)
constexpr int kFcgMaxDirs = 8;

// ring of m+1 direction vectors d and their images q = B d (N^3 each)
template <typename T>
struct FcgBuffers {
    T* d[kFcgMaxDirs + 1];
    T* q[kFcgMaxDirs + 1];
};

template <typename T>
struct PressureWork {
    T *p, *r, *z, *d, *d2, *q;  // N^3 each; p is the pressure
    double* part;               // pressure_partials() doubles
    double* scal;               // kScalDoubles doubles (layout in fia_pressure.cu)
    double* sums;               // 4 doubles
    unsigned* ticket;           // 4 last-block counters (zero between kernels)
};

struct PressureReport {
    int iterations;
    double rel_residual;
    int status;               // 1: iteration cap reached before the tolerance
    int launches;             // kernels launched by the solve
    double bb = 0.0;          // |b|^2 of the right-hand side
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

// r = rhs - B p; |r|^2 into rr_host (synchronises the stream).
template <typename T>
cudaError_t pressure_residual(const PressureWork<T>& W, const PoissonGrid& g, const T* rhs, double* rr_host,
                              cudaStream_t s);

// Solves A p = div(u) h for the reference operator to |r| <= tol |b| (Jacobi-PCG, cold start).
template <typename T>
cudaError_t pressure_solve(const PressureWork<T>& W, const PoissonGrid& g, double h, const T* u, const T* v,
                           const T* w, double tol, int max_iter, PressureReport* rep, cudaStream_t s);

// u -= grad p / h on faces between two fluid cells, 0 on faces touching a solid cell; wall
// momentum loss sums into loss_sums[0..3).
template <typename T>
cudaError_t subtract_gradient(const T* p, T* u, T* v, T* w, const PoissonGrid& g, double h, double* loss_part,
                              double* loss_sums, cudaStream_t s);

// Flexible CG (FCG(m), the last m directions kept) around a preconditioner that writes
// z = M(r) between iterations:
//   dots:       beta_j = -(z.q_j)/(d_j.q_j) for the kept directions j
//   direction:  d = z + sum_j beta_j d_j, q = B d, alpha = (d.r) / (d.q)   (ring slot it % (m+1))
//   update:     p += alpha d, r -= alpha q, rr = r.r, done flag when rr <= tol^2 bb
template <typename T>
cudaError_t fcg_begin(const PressureWork<T>& W, double bb, double rr0, double tol, cudaStream_t s);
template <typename T>
cudaError_t fcg_iteration(const PressureWork<T>& W, const PoissonGrid& g, const FcgBuffers<T>& B, int it, int m,
                          cudaStream_t s);

// FP64 residual refinement of the FP32 form: r = -b - B p64 computed in FP64 from the FP32
// velocities (stored as FP32 in W.r), |r|^2 into rr_host (synchronises); conversions; the
// gradient subtraction from the FP64 pressure.
cudaError_t true_residual(const PressureWork<float>& W, const PoissonGrid& g, double h, const float* u,
                          const float* v, const float* w, const double* p64, double* rr_host, cudaStream_t s);
cudaError_t widen(const float* a, double* b, long long n, bool accumulate, cudaStream_t s);
cudaError_t narrow(const double* a, float* b, long long n, cudaStream_t s);
cudaError_t subtract_gradient_p64(const double* p64, float* u, float* v, float* w, const PoissonGrid& g, double h,
                                  double* loss_part, double* loss_sums, cudaStream_t s);

// out = {rr, done, iterations} (synchronises the stream)
cudaError_t solver_state(const double* scal, double out[3], cudaStream_t s);

}  // namespace fia
