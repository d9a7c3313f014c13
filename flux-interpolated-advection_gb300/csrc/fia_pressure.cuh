// fia_pressure.cuh -- matrix-free pressure projection (calc_pressure_3d.cpp:18-270).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace fia {

template <typename T>
struct PressureWork {
    T *p, *r, *z, *d, *q;     // N^3 each; p is the pressure (last cell pinned to 0)
    double* part;             // pressure_partials() doubles
    double* scal;             // 4 doubles: alpha, beta, rz
    double* sums;             // 4 doubles
};

struct PressureReport {
    int iterations;
    double rel_residual;
    int status;               // 1: iteration cap reached before the tolerance
};

size_t pressure_partials();

// Solves A p = div(u) h for the reference operator to |r| <= tol |b| (Jacobi-PCG).
template <typename T>
cudaError_t pressure_solve(const PressureWork<T>& W, int nx, int ny, int nz, double h, const T* u, const T* v,
                           const T* w, double tol, int max_iter, PressureReport* rep, cudaStream_t s);

// u -= grad p / h on interior faces; wall momentum loss sums into loss_sums[0..3).
template <typename T>
cudaError_t subtract_gradient(const T* p, T* u, T* v, T* w, int nx, int ny, int nz, double h, double* loss_part,
                              double* loss_sums, cudaStream_t s);

}  // namespace fia
