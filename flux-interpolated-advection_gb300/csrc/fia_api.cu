// fia_api.cu -- the C ABI of include/fia.h: device-resident Grid_3D session and the
// orchestration of the reference's entry points on one CUDA stream.
#include "../../include/fia.h"
#include "fia_advect.cuh"
#include "fia_pressure.cuh"
#include "fia_unet.cuh"

#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <algorithm>

using namespace fia;

struct fia_session {
    int N[3];
    double h;
    int precision;
    size_t es;                   // element size on the device
    cudaStream_t stream;
    int last_status;
    bool status_pending;
    bool counters_pending;
    unsigned long long counters_host[5];
    unsigned long long launches;   // kernels launched by this session (host-side count)
    std::vector<cudaEvent_t> prof_ev;   // face-kernel timing (fia_profile_faces)
    int prof_n;
    double wall_loss[3];
    // device buffers
    void* rho; void* rho_next; void* pres;
    void* vel[3]; void* vel_next[3];
    void* cbuf;                  // correction field (pass 2 result)
    void* psi; void* verts; void* flux[3]; void* flux_rev[3];
    void* verts2 = nullptr;      // flux MacCormack: the vertices traced back (allocated on first use)
    // cell-volume correction (allocated on first use): per-face y n_y sums, cell volumes, the
    // right-hand side and the potential of its Poisson solve
    void* fvol[3] = {nullptr, nullptr, nullptr};
    void* fvol_rev[3] = {nullptr, nullptr, nullptr};
    void* vol = nullptr; void* vol_rhs = nullptr; void* vol_p = nullptr;
    size_t verts_bytes = 0;      // one coordinate of every vertex of the largest field
    void* pw[5];                 // pressure work vectors r z d q (+ spare)
    double* part; double* scal; double* sums;
    unsigned* status; unsigned long long* counters;
    unsigned* ticket;            // last-block counters of the fused CG kernels
    double* red_part; double* red_out;
    std::vector<void*> allocations;
    // solids and the pinned pressure cell
    unsigned char* solid = nullptr;
    int pin = 0;
    long long n_free = 0;
    // learned preconditioner (created by fia_learned_init / fia_learned_set_weights)
    unet::Net* net = nullptr;
    cudaEvent_t pev[2] = {nullptr, nullptr};
    // clipped pieces of a pass (FP32 form)
    PieceStore pieces;
    // flexible-CG direction ring (allocated on first use)
    FcgBuffers<float> fcg{};
    bool fcg_ready = false;
    double* p64 = nullptr;       // FP32 form: pressure accumulated in FP64 by the refinement
    int full_weno = 0;           // FP64 form: no WENO6 collapse on node planes (fia_debug_full_weno)
    double vertex_jitter = 0.0;  // FP64 form: backtraced vertices jittered (fia_debug_vertex_jitter)
    mutable unsigned jitter_calls = 0;
    // clipped pieces of a pass (FP64 form); piece_pipeline 0: one thread per face instead
    PieceStore64 pieces64;
    int piece_pipeline = 1;
};

namespace {

thread_local std::string g_last_error;
thread_local std::string g_last_unsupported;   // why the last FIA_ERR_UNSUPPORTED of this thread

int set_cuda_error(cudaError_t e, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return FIA_ERR_CUDA;
}
#define CK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return set_cuda_error(e_, #call); } while (0)

long long field_count(const fia_session* s, int field) {
    const long long nx = s->N[0], ny = s->N[1], nz = s->N[2];
    switch (field) {
        case FIA_FIELD_DENSITY: case FIA_FIELD_PRESSURE: return nx * ny * nz;
        case FIA_FIELD_U: return (nx + 1) * ny * nz;
        case FIA_FIELD_V: return nx * (ny + 1) * nz;
        case FIA_FIELD_W: return nx * ny * (nz + 1);
        default: return -1;
    }
}

void* field_ptr(fia_session* s, int field) {
    switch (field) {
        case FIA_FIELD_DENSITY: return s->rho;
        case FIA_FIELD_PRESSURE: return s->pres;
        case FIA_FIELD_U: return s->vel[0];
        case FIA_FIELD_V: return s->vel[1];
        case FIA_FIELD_W: return s->vel[2];
        default: return nullptr;
    }
}

// element-type conversion on the device
template <typename D, typename S>
__global__ void k_convert(const S* __restrict__ src, D* __restrict__ dst, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = (D)src[i];
}

// FP64 sum (kind 0) or max |x| (kind 1) of n values: per-block partials then one block.
template <typename T>
__global__ void k_reduce_part(const T* __restrict__ a, long long n, int kind, double* part) {
    double acc = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double x = (double)a[i];
        acc = kind == 0 ? acc + x : fmax(acc, fabs(x));
    }
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_down_sync(0xffffffffu, acc, o);
        acc = kind == 0 ? acc + y : fmax(acc, y);
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, acc, o);
            acc = kind == 0 ? acc + y : fmax(acc, y);
        }
        if (threadIdx.x == 0) part[blockIdx.x] = acc;
    }
}

__global__ void k_reduce_final(const double* part, int nb, int kind, double* out, int accumulate) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) acc = kind == 0 ? acc + part[b] : fmax(acc, part[b]);
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_down_sync(0xffffffffu, acc, o);
        acc = kind == 0 ? acc + y : fmax(acc, y);
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = kind == 0 ? 0.0 : 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = kind == 0 ? t + sh[w] : fmax(t, sh[w]);
        if (accumulate && kind == 1) t = fmax(t, *out);
        else if (accumulate) t += *out;
        *out = t;
    }
}

constexpr int kRedBlocks = 512;

template <typename T>
cudaError_t reduce(fia_session* s, const void* a, long long n, int kind, bool accumulate) {
    k_reduce_part<T><<<kRedBlocks, 256, 0, s->stream>>>((const T*)a, n, kind, s->red_part);
    k_reduce_final<<<1, 256, 0, s->stream>>>(s->red_part, kRedBlocks, kind, s->red_out, accumulate ? 1 : 0);
    s->launches += 2;
    return cudaGetLastError();
}

// kernels launched by one run_pass: psi, backtrace (moving passes), the face stages (one, or
// three for the flux MacCormack scheme, plus its second trace), gather.  A face stage is three
// face-family launches (FP64), or three clips, the per-piece quadrature and three per-face
// sums (FP32 form).
inline unsigned pass_launches(const PassDesc& d, int precision) {
    // FP32 form: faces at rest clip and sum the y-faces only (the others emit no piece)
    const unsigned stage = precision == FIA_FP64 ? 3u : 8u, rest = precision == FIA_FP64 ? 3u : 4u;
    if (d.zero_velocity) return 2u + rest;
    if (d.maccormack) return 4u + rest + 2u * stage;
    return 3u + stage;
}

// Split offsets (colour = pos/h - off) per field for the main and the error-advection pass
// (move_substances_3d.cpp:189; advect_velocity_flux_advection_3d.cpp:622-628, :721,
// :805-810, :913, :999-1002, :1096).
void split_offsets(int comp, int error_pass, int density_split, double* off) {
    static const double tbl[4][2] = {{0.5, 0.5}, {0.0, 0.0}, {0.5, 0.0}, {0.0, 0.5}};
    if (comp < 0) {
        const int m = error_pass ? FIA_SPLIT_XZ_AXIS : density_split;
        off[0] = tbl[m][0]; off[1] = tbl[m][1];
        return;
    }
    const double main_x = comp == 0 ? 0.0 : 0.5, main_z = comp == 2 ? 0.0 : 0.5;
    if (!error_pass) { off[0] = main_x; off[1] = main_z; }
    else if (comp == 1) { off[0] = 0.0; off[1] = 0.0; }
    else { off[0] = 0.5 - main_x; off[1] = 0.5 - main_z; }
}

int check_params(const fia_advect_params* p) {
    if (!p) return FIA_ERR_INVALID;
    if (p->interpolation_method != FIA_INTERP_WENO6 && p->interpolation_method != FIA_INTERP_LINEAR) return FIA_ERR_INVALID;
    if (p->split_method < 0 || p->split_method > 3) return FIA_ERR_INVALID;
    const int k = p->num_gauss_quadrature_point_for_integrate_density;
    if (k < 1 || k > kMaxGauss || (k % 2) == 0) return FIA_ERR_INVALID;
    if (!(p->minimal_area > 0.0)) return FIA_ERR_INVALID;
    return FIA_OK;
}

// The chosen form does not triangulate pieces (minimal_area < 1; a piece's xi-eta area is at
// most 1, so minimal_area >= 1, the reference's default, never triangulates).  The bisection
// of the longest edge jumps where two edges are equally long, and FP32 vertex positions,
// through crossing points on edges almost parallel to an iso-line, put a face on the other
// side of such a tie often enough to move a pass by 1-6% against the oracle; the plain form
// matches it.
int check_form(const fia_session* s, double minimal_area) {
    if (s->precision == FIA_FP32C && minimal_area < 1.0) {
        g_last_unsupported = "minimal_area < 1 (triangulated pieces) is supported by the FP64 form only";
        return FIA_ERR_UNSUPPORTED;
    }
    return FIA_OK;
}

PassDesc base_desc(const fia_session* s, int comp, double dt) {
    PassDesc d;
    std::memset(&d, 0, sizeof(d));
    for (int c = 0; c < 3; ++c) d.N[c] = s->N[c];
    d.comp = comp;
    d.A = comp < 0 ? cell_field(s->N, -1) : cell_field(s->N, comp);
    d.P = psi_field(d.A);
    d.h = s->h;
    d.dt = dt;
    d.full_weno = s->full_weno;
    if (s->vertex_jitter != 0.0) {
        d.vertex_jitter = s->vertex_jitter;
        d.jitter_seed = ++s->jitter_calls;
    }
    return d;
}

template <typename T>
PassWork<T> work(fia_session* s) {
    PassWork<T> w;
    w.psi = (T*)s->psi; w.verts = (T*)s->verts; w.verts2 = (T*)s->verts2;
    for (int f = 0; f < 3; ++f) { w.fvol[f] = (T*)s->fvol[f]; w.fvol_rev[f] = (T*)s->fvol_rev[f]; }
    w.vol = (T*)s->vol;
    for (int f = 0; f < 3; ++f) { w.flux[f] = (T*)s->flux[f]; w.flux_rev[f] = (T*)s->flux_rev[f]; }
    w.status = s->status; w.counters = s->counters;
    w.prof_ev = s->prof_ev.empty() ? nullptr : s->prof_ev.data();
    w.prof_n = &s->prof_n;
    w.prof_cap = (int)(s->prof_ev.size() / 2);
    w.pieces = &s->pieces;
    w.pieces64 = (s->precision == FIA_FP64 && s->piece_pipeline) ? &s->pieces64 : nullptr;
    return w;
}

VelocityFields velocity(fia_session* s, void* const* v) {
    VelocityFields vel;
    vel.u = v[0]; vel.v = v[1]; vel.w = v[2];
    vel.fu = cell_field(s->N, 0); vel.fv = cell_field(s->N, 1); vel.fw = cell_field(s->N, 2);
    return vel;
}

// ------------------------------ cell-volume correction -----------------------------
// move_substances_3d.cpp:243-493: A p = -(V - V0) on the reference operator (last cell pinned,
// no solids), i.e. B p = V - V0 for B = -A; then density moves between face neighbours by
// -(p_hi - p_lo) / V0 times the mean of their densities before the correction, x faces, then
// y, then z (each cell gathers its six faces in that order).
template <typename T>
__global__ void k_volume_rhs(const T* __restrict__ vol, T* __restrict__ rhs, T* __restrict__ before,
                             const T* __restrict__ rho, long long n, T V0) {
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        rhs[c] = c == n - 1 ? T(0) : vol[c] - V0;
        before[c] = rho[c];
    }
}

template <typename T>
__global__ void k_volume_exchange(int nx, int ny, int nz, const T* __restrict__ p, const T* __restrict__ before,
                                  T* __restrict__ rho, T V0) {
    const long long n = (long long)nx * ny * nz;
    const long long sx = (long long)ny * nz, sy = nz;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(c % nz), iy = (int)((c / nz) % ny), ix = (int)(c / sx);
        const int id[3] = {ix, iy, iz}, lim[3] = {nx, ny, nz};
        const long long st[3] = {sx, sy, 1};
        T val = rho[c];
        for (int a = 0; a < 3; ++a) {
            if (id[a] >= 1) {            // the face below: this cell is its upper cell
                const long long o = c - st[a];
                const T flux = -(p[c] - p[o]) / V0;
                const T dens = (before[o] * V0 + before[c] * V0) / (T(2) * V0);
                val += T(1) * flux * dens;
            }
            if (id[a] < lim[a] - 1) {    // the face above: this cell is its lower cell
                const long long o = c + st[a];
                const T flux = -(p[o] - p[c]) / V0;
                const T dens = (before[c] * V0 + before[o] * V0) / (T(2) * V0);
                val -= T(1) * flux * dens;
            }
        }
        rho[c] = val;
    }
}

// relative residual of the volume solve: FP64 form, FP32 form (FP32 Jacobi-PCG with FP64 dots)
constexpr double kVolumeTol = 1e-12, kVolumeTol32 = 1e-6;

template <typename T>
PressureWork<T> pressure_work(fia_session* s);

// allocates the buffers of the cell-volume correction on first use
cudaError_t volume_buffers(fia_session* s) {
    if (s->vol) return cudaSuccess;
    const size_t fb = s->verts_bytes;                    // one value per node of the largest field
    const size_t pb = s->verts_bytes / s->es * 8;        // one double, or one float pair (FP32 form)
    auto A = [&](void*& dst, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(&dst, bytes);
        if (e == cudaSuccess) { s->allocations.push_back(dst); cudaMemsetAsync(dst, 0, bytes, s->stream); }
        return e;
    };
    for (int f = 0; f < 3; ++f) {
        cudaError_t e = A(s->fvol[f], pb);
        if (e == cudaSuccess) e = A(s->fvol_rev[f], pb);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = A(s->vol, fb);
    if (e == cudaSuccess) e = A(s->vol_rhs, fb);
    if (e == cudaSuccess) e = A(s->vol_p, fb);
    return e;
}

// rho (the main pass's result) corrected by the cell volumes in s->vol (FP64 form: absolute
// volumes, V0 = h^3; FP32 form: volumes in cells, V0 = 1: the potential scales with the
// volumes and the exchanged fraction -(p_hi - p_lo) / V0 is the same)
template <typename T>
cudaError_t volume_correction(fia_session* s, T* rho) {
    const int nx = s->N[0], ny = s->N[1], nz = s->N[2];
    const long long n = (long long)nx * ny * nz;
    const bool fp64 = s->precision == FIA_FP64;
    const T V0 = fp64 ? T(s->h * s->h * s->h) : T(1);
    T* before = (T*)s->vol;   // the volumes are consumed by the right-hand side first
    k_volume_rhs<T><<<1024, 256, 0, s->stream>>>((const T*)s->vol, (T*)s->vol_rhs, before, rho, n, V0);
    PressureWork<T> W = pressure_work<T>(s);
    W.p = (T*)s->vol_p;
    const PoissonGrid g{nx, ny, nz, (int)(n - 1), nullptr};
    cudaError_t e = cudaMemsetAsync(W.p, 0, n * sizeof(T), s->stream);
    double rr = 0.0;
    if (e == cudaSuccess) e = pressure_residual<T>(W, g, (const T*)s->vol_rhs, &rr, s->stream);
    PressureReport rep{};
    if (e == cudaSuccess && rr > 0.0)
        e = pressure_pcg<T>(W, g, rr, rr, fp64 ? kVolumeTol : kVolumeTol32, 50000, &rep, s->stream);
    if (e != cudaSuccess) return e;
    s->launches += 3 + (unsigned long long)rep.launches;
    k_volume_exchange<T><<<1024, 256, 0, s->stream>>>(nx, ny, nz, (const T*)W.p, before, rho, V0);
    return cudaGetLastError();
}

// One field through move_substances_3D's pass structure (move_substances_3d.cpp:58-226);
// velocity components follow the same structure with their own split methods.
template <typename T>
cudaError_t advect_field(fia_session* s, int comp, const T* in, T* out, double dt, const fia_advect_params* p,
                         void* const* vel_fields) {
    PassDesc d = base_desc(s, comp, dt);
    d.k = p->num_gauss_quadrature_point_for_integrate_density;
    make_gauss(d.k, d.gx, d.gw);
    d.minimal_area = p->minimal_area;
    d.maccormack = p->use_MacCormack_scheme ? 1 : 0;
    if (d.maccormack && !s->verts2) {
        const size_t bytes = 3 * s->verts_bytes;
        if (cudaMalloc(&s->verts2, bytes) != cudaSuccess) return cudaErrorMemoryAllocation;
        s->allocations.push_back(s->verts2);
    }
    const VelocityFields vel = velocity(s, vel_fields);
    const PassWork<T> w = work<T>(s);
    // pass 1
    d.interp = p->interpolation_method == FIA_INTERP_WENO6 ? INTERP_WENO6 : INTERP_LINEAR;
    d.use_integral = p->use_integral ? 1 : 0;
    d.psi_mode = p->use_integral ? (d.interp == INTERP_WENO6 ? PSI_WENO6 : PSI_LINEAR) : PSI_PLAIN;
    d.zero_velocity = 0;
    split_offsets(comp, 0, p->split_method, d.color_off);
    // cell-volume correction of the density (move_substances_3d.cpp:106-112; the velocity
    // version is commented out in the reference)
    const bool volumes = p->enable_cell_volume_correction && comp < 0;
    d.volumes = volumes ? 1 : 0;
    cudaError_t e = run_pass<T>(d, vel, in, w, in, out, 0, s->stream);
    s->launches += pass_launches(d, s->precision) + (volumes ? 1 : 0);
    if (e == cudaSuccess && volumes) e = volume_correction<T>(s, out);
    d.volumes = 0;
    if (e != cudaSuccess || !p->enable_eliminate_zero_velocity_false_diffusion) return e;
    // pass 2: zero velocity, psi at the piece centroid, plain psi; c = in - A2(in)
    T* c = (T*)s->cbuf;
    d.zero_velocity = 1; d.use_integral = 0; d.psi_mode = PSI_PLAIN;
    e = run_pass<T>(d, vel, in, w, in, c, 1, s->stream);
    s->launches += pass_launches(d, s->precision);
    if (e != cudaSuccess) return e;
    // pass 3: advect the error with 1Dy-linear interpolation and the error split
    d.zero_velocity = 0; d.interp = INTERP_1DY_LINEAR;
    split_offsets(comp, 1, p->split_method, d.color_off);
    s->launches += pass_launches(d, s->precision);
    return run_pass<T>(d, vel, c, w, nullptr, out, 2, s->stream);
}

// Status bits are per call; the work counters accumulate over the session's lifetime.
cudaError_t reset_counters(fia_session* s) {
    s->status_pending = true; s->counters_pending = true;
    return cudaMemsetAsync(s->status, 0, sizeof(unsigned), s->stream);
}

int finish_status(fia_session* s) {
    if (!s->status_pending) return s->last_status;
    unsigned st = 0;
    if (cudaMemcpyAsync(&st, s->status, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream) != cudaSuccess) return FIA_ERR_CUDA;
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return FIA_ERR_CUDA;
    s->status_pending = false;
    s->last_status = (int)st;
    return s->last_status;
}

template <typename T>
int move_substances(fia_session* s, double dt, const fia_advect_params* p) {
    if (p->enable_cell_volume_correction) CK(volume_buffers(s));
    CK(reset_counters(s));
    CK(advect_field<T>(s, -1, (const T*)s->rho, (T*)s->rho_next, dt, p, s->vel));
    std::swap(s->rho, s->rho_next);
    return FIA_OK;
}

template <typename T>
int advect_velocity(fia_session* s, double dt, const fia_advect_params* p) {
    CK(reset_counters(s));
    for (int c = 0; c < 3; ++c)
        CK(advect_field<T>(s, c, (const T*)s->vel[c], (T*)s->vel_next[c], dt, p, s->vel));
    for (int c = 0; c < 3; ++c) std::swap(s->vel[c], s->vel_next[c]);
    return FIA_OK;
}

template <typename T>
PressureWork<T> pressure_work(fia_session* s) {
    PressureWork<T> W;
    W.p = (T*)s->pres; W.r = (T*)s->pw[0]; W.z = (T*)s->pw[1]; W.d = (T*)s->pw[2]; W.q = (T*)s->pw[3];
    W.d2 = (T*)s->pw[4]; W.ticket = s->ticket;
    W.part = s->part; W.scal = s->scal; W.sums = s->sums;
    return W;
}

PoissonGrid poisson_grid(const fia_session* s) {
    return PoissonGrid{s->N[0], s->N[1], s->N[2], s->pin, s->solid};
}

// Flexible CG with the learned preconditioner (FP32C sessions), Jacobi-PCG after
// fallback_iter iterations, or earlier when 20 iterations reduced the best |r| by less than 1%.
// The right-hand side is -div(u) h of the session velocity, or rhs (device, B p = rhs).
int pressure_fcg(fia_session* s, const fia_solver_params* sp, PressureReport& r, int& fcg_its, double& pms,
                 const float* rhs = nullptr) {
    if (!s->net) return FIA_ERR_INVALID;
    using T = float;
    PressureWork<T> W = pressure_work<T>(s);
    const PoissonGrid g = poisson_grid(s);
    const T *u = (const T*)s->vel[0], *v = (const T*)s->vel[1], *w = (const T*)s->vel[2];
    const long long nc = (long long)s->N[0] * s->N[1] * s->N[2];
    double br[2];
    if (rhs) {
        CK(cudaMemsetAsync(W.p, 0, nc * sizeof(T), s->stream));
        CK(pressure_residual<T>(W, g, rhs, &br[1], s->stream));
        br[0] = br[1];
    } else {
        CK(pressure_rhs<T>(W, g, s->h, u, v, w, false, br, s->stream));
    }
    s->launches += 2;
    r.iterations = 0; r.status = 0; r.rel_residual = 0.0; r.launches = 0; r.bb = br[0];
    fcg_its = 0; pms = 0.0;
    if (br[0] == 0.0) return FIA_OK;
    CK(fcg_begin<T>(W, br[0], br[1], sp->tol, s->stream));
    s->launches += 1;
    if (!s->pev[0]) { CK(cudaEventCreate(&s->pev[0])); CK(cudaEventCreate(&s->pev[1])); }
    if (!s->fcg_ready) {
        for (int j = 0; j <= kFcgMaxDirs; ++j) {
            CK(cudaMalloc(&s->fcg.d[j], nc * sizeof(T)));
            CK(cudaMalloc(&s->fcg.q[j], nc * sizeof(T)));
        }
        s->fcg_ready = true;
    }
    const int cap = std::min(sp->fallback_iter, sp->max_iter);
    double st[3] = {br[1], br[1] <= sp->tol * sp->tol * br[0] ? 1.0 : 0.0, 0.0};
    // stalled: the best |r| of the last 20 iterations is not 1% below the best before them
    std::vector<double> best(1, br[1]);
    int it = 0;
    bool stalled = false;
    while (it < cap && st[1] == 0.0 && !stalled) {
        CK(cudaEventRecord(s->pev[0], s->stream));
        CK(unet::net_apply(s->net, g, W.r, W.z, W.scal + kScalRR, (double)s->n_free, s->stream));
        CK(cudaEventRecord(s->pev[1], s->stream));
        CK(fcg_iteration<T>(W, g, s->fcg, it, kFcgMaxDirs, s->stream));
        s->launches += (unsigned long long)unet::net_launches(s->net) + 4;
        CK(solver_state(W.scal, st, s->stream));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->pev[0], s->pev[1]));
        pms += ms;
        ++it;
        best.push_back(std::min(best.back(), st[0]));
        if (it >= 20 && best[it] > 0.9801 * best[it - 20]) stalled = true;
    }
    fcg_its = it;
    r.iterations = it;
    r.rel_residual = std::sqrt(st[0] / br[0]);
    if (st[1] != 0.0) return FIA_OK;
    // fallback: Jacobi-PCG from the current pressure
    double br2[2];
    if (rhs) CK(pressure_residual<T>(W, g, rhs, &br2[1], s->stream));
    else CK(pressure_rhs<T>(W, g, s->h, u, v, w, true, br2, s->stream));
    PressureReport r2;
    CK(pressure_pcg<T>(W, g, br[0], br2[1], sp->tol, std::max(0, sp->max_iter - it), &r2, s->stream));
    s->launches += 2 + (unsigned long long)r2.launches;
    r.iterations = it + r2.iterations;
    r.rel_residual = r2.rel_residual;
    r.status = r2.status;
    return FIA_STATUS_SOLVER_FALLBACK;
}

// FP32 form: the FP32 solve is followed by FP64 residual refinement.  The true residual
// -b - B p is formed in FP64 with the pressure accumulated in FP64; while it is above the
// tolerance, B e = r is solved in FP32 from e = 0 (same solver) and p += e.  The reported
// residual is this FP64 residual, so both precision forms stop at the same true residual.
constexpr int kMaxRefinements = 4;

int refine_fp32(fia_session* s, const fia_solver_params* sp, PressureReport& r, int& fcg_its, double& pms,
                int& extra) {
    using T = float;
    PressureWork<T> W = pressure_work<T>(s);
    const PoissonGrid g = poisson_grid(s);
    const T *u = (const T*)s->vel[0], *v = (const T*)s->vel[1], *w = (const T*)s->vel[2];
    const long long nc = (long long)s->N[0] * s->N[1] * s->N[2];
    const double bb = r.bb;
    if (!(bb > 0.0)) return FIA_OK;
    if (!s->p64) CK(cudaMalloc(&s->p64, nc * sizeof(double)));
    CK(widen(W.p, s->p64, nc, false, s->stream));
    double rr = 0.0;
    CK(true_residual(W, g, s->h, u, v, w, s->p64, &rr, s->stream));
    s->launches += 3;
    int used = r.iterations;
    for (int k = 0; k < kMaxRefinements && rr > sp->tol * sp->tol * bb && used < sp->max_iter; ++k) {
        fia_solver_params in = *sp;
        in.tol = std::min(0.5, std::max(1e-5, 0.3 * sp->tol * std::sqrt(bb / rr)));
        in.max_iter = sp->max_iter - used;
        PressureReport r2;
        if (sp->method == FIA_SOLVER_FCG_LEARNED) {
            float* rhs = (float*)s->cbuf;
            CK(cudaMemcpyAsync(rhs, W.r, nc * sizeof(T), cudaMemcpyDeviceToDevice, s->stream));
            int its2 = 0;
            double pms2 = 0.0;
            in.fallback_iter = std::min(in.fallback_iter, in.max_iter);
            const int rc = pressure_fcg(s, &in, r2, its2, pms2, rhs);
            if (rc < 0) return rc;
            extra |= rc;
            fcg_its += its2;
            pms += pms2;
        } else {
            CK(cudaMemsetAsync(W.p, 0, nc * sizeof(T), s->stream));
            CK(pressure_pcg<T>(W, g, rr, rr, in.tol, in.max_iter, &r2, s->stream));
            s->launches += (unsigned long long)r2.launches + 1;
        }
        used += r2.iterations;
        CK(widen(W.p, s->p64, nc, true, s->stream));
        CK(true_residual(W, g, s->h, u, v, w, s->p64, &rr, s->stream));
        s->launches += 3;
    }
    CK(narrow(s->p64, W.p, nc, s->stream));
    s->launches += 1;
    r.iterations = used;
    r.rel_residual = std::sqrt(rr / bb);
    r.status = rr > sp->tol * sp->tol * bb ? 1 : 0;
    return FIA_OK;
}

template <typename T>
int pressure(fia_session* s, const fia_solver_params* sp, fia_solver_report* rep, bool subtract) {
    fia_solver_params def;
    fia_default_solver_params(&def);
    if (!sp) sp = &def;
    if (sp->method != FIA_SOLVER_PCG_JACOBI && sp->method != FIA_SOLVER_FCG_LEARNED) return FIA_ERR_INVALID;
    if (!(sp->tol > 0.0) || sp->max_iter < 1) return FIA_ERR_INVALID;
    PressureWork<T> W = pressure_work<T>(s);
    const PoissonGrid g = poisson_grid(s);
    PressureReport r;
    int extra = 0, fcg_its = 0;
    double pms = 0.0;
    if (sp->method == FIA_SOLVER_FCG_LEARNED) {
        if (s->precision != FIA_FP32C) {
            g_last_unsupported = "the learned preconditioner needs an FP32C session";
            return FIA_ERR_UNSUPPORTED;
        }
        if (!s->net) return FIA_ERR_INVALID;
        if (sp->fallback_iter < 1) return FIA_ERR_INVALID;
        const int rc = pressure_fcg(s, sp, r, fcg_its, pms);
        if (rc < 0) return rc;
        extra = rc;
    } else {
        CK(pressure_solve<T>(W, g, s->h, (const T*)s->vel[0], (const T*)s->vel[1], (const T*)s->vel[2], sp->tol,
                             sp->max_iter, &r, s->stream));
        s->launches += (unsigned long long)r.launches;
    }
    const bool refined = s->precision == FIA_FP32C && r.bb > 0.0;
    if (refined) {
        const int rc = refine_fp32(s, sp, r, fcg_its, pms, extra);
        if (rc < 0) return rc;
    }
    if (subtract) {
        if (refined)
            CK(subtract_gradient_p64(s->p64, (float*)s->vel[0], (float*)s->vel[1], (float*)s->vel[2], g, s->h, s->part,
                                     s->sums, s->stream));
        else
            CK(subtract_gradient<T>((const T*)s->pres, (T*)s->vel[0], (T*)s->vel[1], (T*)s->vel[2], g, s->h, s->part,
                                    s->sums, s->stream));
        s->launches += 3;
        double loss[3];
        CK(cudaMemcpyAsync(loss, s->sums, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (int c = 0; c < 3; ++c) s->wall_loss[c] += loss[c];
    }
    const int status = (r.status ? FIA_STATUS_SOLVER_CAP : 0) | extra;
    if (rep) {
        rep->iterations = r.iterations; rep->rel_residual = r.rel_residual; rep->status = status;
        rep->fcg_iterations = fcg_its; rep->precond_ms = pms;
    }
    return status;
}

// Solves the projection of the current velocity to tol with Jacobi-PCG (pressure untouched)
// and keeps (r = -div(u) h, p) as a training pair of the learned preconditioner.
int capture_pair(fia_session* s, double tol) {
    if (s->precision != FIA_FP32C || !s->net) return FIA_ERR_INVALID;
    using T = float;
    PressureWork<T> W = pressure_work<T>(s);
    const PoissonGrid g = poisson_grid(s);
    // the solve runs on a copy of the pressure so that the session's pressure is kept
    PressureWork<T> C = W;
    const long long nc = (long long)s->N[0] * s->N[1] * s->N[2];
    T* pkeep = (T*)s->cbuf;
    CK(cudaMemcpyAsync(pkeep, s->pres, nc * sizeof(T), cudaMemcpyDeviceToDevice, s->stream));
    PressureReport r;
    CK(pressure_solve<T>(C, g, s->h, (const T*)s->vel[0], (const T*)s->vel[1], (const T*)s->vel[2], tol, 100000, &r,
                         s->stream));
    s->launches += (unsigned long long)r.launches;
    // r = -b into W.z (its pressure argument W.q is a scratch that gets zeroed)
    PressureWork<T> R = W;
    R.r = W.z; R.p = W.q;
    double br[2];
    CK(pressure_rhs<T>(R, g, s->h, (const T*)s->vel[0], (const T*)s->vel[1], (const T*)s->vel[2], false, br,
                       s->stream));
    const int id = unet::net_add_pair(s->net, g, W.z, (const float*)s->pres, s->stream);
    CK(cudaMemcpyAsync(s->pres, pkeep, nc * sizeof(T), cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return id < 0 ? FIA_ERR_CUDA : FIA_OK;
}

template <typename T>
int debug_flux_pass(fia_session* s, int comp, const double* field, double dt, int interp, int psi_mode,
                    int use_integral, int zero_velocity, const double* co, int k, double minimal_area, double* out) {
    PassDesc d = base_desc(s, comp, dt);
    d.k = k; make_gauss(k, d.gx, d.gw);
    d.interp = interp; d.psi_mode = psi_mode; d.use_integral = use_integral; d.zero_velocity = zero_velocity;
    d.color_off[0] = co[0]; d.color_off[1] = co[1]; d.minimal_area = minimal_area;
    const long long n = (long long)d.A.Mx * d.A.My * d.A.Mz;
    double* tmp = nullptr;
    CK(cudaMallocAsync((void**)&tmp, n * sizeof(double), s->stream));
    CK(cudaMemcpyAsync(tmp, field, n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    T* a = (T*)s->cbuf;
    k_convert<T, double><<<256, 256, 0, s->stream>>>(tmp, a, n);
    CK(reset_counters(s));
    CK(run_pass<T>(d, velocity(s, s->vel), a, work<T>(s), a, (T*)s->rho_next, 0, s->stream));
    k_convert<double, T><<<256, 256, 0, s->stream>>>((const T*)s->rho_next, tmp, n);
    CK(cudaMemcpyAsync(out, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaFreeAsync(tmp, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return finish_status(s);
}

// FP32 form: vertex displacements in cells -> absolute positions; psi pairs -> psi.
__global__ void k_disp_to_pos(const float* __restrict__ disp, double* __restrict__ out, int Ly, int Lz, int comp,
                              double h, long long nv) {
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x) {
        const int idx[3] = {(int)(v / ((long long)Ly * Lz)), (int)((v / Lz) % Ly), (int)(v % Lz)};
        for (int c = 0; c < 3; ++c)
            out[3 * v + c] = ((double)idx[c] - (c == comp ? 0.5 : 0.0) + (double)disp[3 * v + c]) * h;
    }
}
__global__ void k_pairs_to_psi(const float2* __restrict__ p, double* __restrict__ out, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (double)p[i].x + (double)p[i].y;
}

void export_verts(fia_session* s, const PassDesc& d, const double* verts, double* tmp, long long n) {
    k_convert<double, double><<<256, 256, 0, s->stream>>>(verts, tmp, n);
}
void export_verts(fia_session* s, const PassDesc& d, const float* verts, double* tmp, long long n) {
    k_disp_to_pos<<<256, 256, 0, s->stream>>>(verts, tmp, d.A.My + 1, d.A.Mz + 1, d.comp, s->h, n / 3);
}
void export_psi(fia_session* s, const double* psi, double* tmp, long long n) {
    k_convert<double, double><<<256, 256, 0, s->stream>>>(psi, tmp, n);
}
void export_psi(fia_session* s, const float* psi, double* tmp, long long n) {
    k_pairs_to_psi<<<256, 256, 0, s->stream>>>((const float2*)psi, tmp, n);
}

template <typename T>
int debug_backtrace(fia_session* s, int comp, double dt, int interp, double* out) {
    PassDesc d = base_desc(s, comp, dt);
    d.interp = interp;
    const long long n = 3LL * (d.A.Mx + 1) * (d.A.My + 1) * (d.A.Mz + 1);
    CK(launch_backtrace<T>(d, velocity(s, s->vel), (T*)s->verts, s->stream));
    double* tmp = nullptr;
    CK(cudaMallocAsync((void**)&tmp, n * sizeof(double), s->stream));
    export_verts(s, d, (const T*)s->verts, tmp, n);
    CK(cudaMemcpyAsync(out, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaFreeAsync(tmp, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

template <typename T>
int debug_psi(fia_session* s, int comp, const double* field, int mode, int k, double* out) {
    PassDesc d = base_desc(s, comp, 0.0);
    d.k = k; make_gauss(k, d.gx, d.gw); d.psi_mode = mode;
    const long long n = (long long)d.A.Mx * d.A.My * d.A.Mz;
    const long long np = (long long)d.P.Mx * d.P.My * d.P.Mz;
    double* tmp = nullptr;
    CK(cudaMallocAsync((void**)&tmp, np * sizeof(double), s->stream));
    CK(cudaMemcpyAsync(tmp, field, n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    k_convert<T, double><<<256, 256, 0, s->stream>>>(tmp, (T*)s->cbuf, n);
    CK(launch_psi<T>(d, (const T*)s->cbuf, (T*)s->psi, s->stream));
    export_psi(s, (const T*)s->psi, tmp, np);
    CK(cudaMemcpyAsync(out, tmp, np * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaFreeAsync(tmp, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

// ------------------------------- the smoke step -----------------------------------
// density = max(density, value) in the cells whose centre lies in the sphere
template <typename T>
__global__ void k_source(T* __restrict__ rho, int nx, int ny, int nz, double h, double cx, double cy, double cz,
                         double r, double value, const unsigned char* __restrict__ solid) {
    const long long n = (long long)nx * ny * nz;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(c % nz), iy = (int)((c / nz) % ny), ix = (int)(c / ((long long)nz * ny));
        const double x = (ix + 0.5) * h - cx, y = (iy + 0.5) * h - cy, z = (iz + 0.5) * h - cz;
        if (solid && solid[c]) continue;
        if (x * x + y * y + z * z <= r * r && (double)rho[c] < value) rho[c] = (T)value;
    }
}

// v += dt * b * (rho_below + rho_above) / 2 on interior y-faces between fluid cells
template <typename T>
__global__ void k_buoyancy(T* __restrict__ v, const T* __restrict__ rho, int nx, int ny, int nz, double a,
                           const unsigned char* __restrict__ solid) {
    const long long n = (long long)nx * (ny + 1) * nz;
    for (long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(f % nz), iy = (int)((f / nz) % (ny + 1)), ix = (int)(f / ((long long)nz * (ny + 1)));
        if (iy == 0 || iy == ny) continue;
        const long long c = ((long long)ix * ny + iy) * nz + iz;
        if (solid && (solid[c] || solid[c - nz])) continue;
        v[f] = (T)((double)v[f] + a * 0.5 * ((double)rho[c - nz] + (double)rho[c]));
    }
}

// density = 0 in solid cells
template <typename T>
__global__ void k_clear_solid(T* __restrict__ rho, long long n, const unsigned char* __restrict__ solid) {
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        if (solid[c]) rho[c] = (T)0;
}

// zero velocity on faces touching a solid cell (all three families)
template <typename T>
__global__ void k_solid_faces(T* __restrict__ u, T* __restrict__ v, T* __restrict__ w, int nx, int ny, int nz,
                              const unsigned char* __restrict__ solid) {
    const long long nu = (long long)(nx + 1) * ny * nz, nv = (long long)nx * (ny + 1) * nz;
    const long long nw = (long long)nx * ny * (nz + 1);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nu + nv + nw; t += (long long)gridDim.x * blockDim.x) {
        if (t < nu) {
            const int iz = (int)(t % nz), iy = (int)((t / nz) % ny), ix = (int)(t / ((long long)nz * ny));
            const long long c = ((long long)ix * ny + iy) * nz + iz, sx = (long long)ny * nz;
            if ((ix < nx && solid[c]) || (ix > 0 && solid[c - sx])) u[t] = (T)0;
        } else if (t < nu + nv) {
            const long long f = t - nu;
            const int iz = (int)(f % nz), iy = (int)((f / nz) % (ny + 1)), ix = (int)(f / ((long long)nz * (ny + 1)));
            const long long c = ((long long)ix * ny + iy) * nz + iz;
            if ((iy < ny && solid[c]) || (iy > 0 && solid[c - nz])) v[f] = (T)0;
        } else {
            const long long f = t - nu - nv;
            const int iz = (int)(f % (nz + 1)), iy = (int)((f / (nz + 1)) % ny), ix = (int)(f / ((long long)(nz + 1) * ny));
            const long long c = ((long long)ix * ny + iy) * nz + iz;
            if ((iz < nz && solid[c]) || (iz > 0 && solid[c - 1])) w[f] = (T)0;
        }
    }
}

template <typename T>
__global__ void k_scale(T* __restrict__ a, long long n, double s) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        a[i] = (T)((double)a[i] * s);
}

template <typename T>
int read_reduction(fia_session* s, const void* a, long long n, int kind, double* out) {
    CK(reduce<T>(s, a, n, kind, false));
    CK(cudaMemcpyAsync(out, s->red_out, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

template <typename T>
int step(fia_session* s, const fia_step_params* p, fia_step_report* rep) {
    const int nx = s->N[0], ny = s->N[1], nz = s->N[2];
    const long long nc = (long long)nx * ny * nz;
    const double V = s->h * s->h * s->h;
    int status = 0, r;
    if (p->source) {
        k_source<T><<<1024, 256, 0, s->stream>>>((T*)s->rho, nx, ny, nz, s->h, p->source_center[0],
                                                 p->source_center[1], p->source_center[2], p->source_radius,
                                                 p->source_density, s->solid);
        s->launches += 1;
    }
    double umax = 0.0, m;
    for (int c = 0; c < 3; ++c) {
        if ((r = read_reduction<T>(s, s->vel[c], field_count(s, FIA_FIELD_U + c), 1, &m)) != FIA_OK) return r;
        umax = std::max(umax, m);
    }
    double dt = p->max_dt;
    if (umax > 0.0) dt = std::min(dt, p->cfl * s->h / umax);
    if (p->buoyancy != 0.0) {
        k_buoyancy<T><<<1024, 256, 0, s->stream>>>((T*)s->vel[1], (const T*)s->rho, nx, ny, nz, dt * p->buoyancy,
                                                   s->solid);
        s->launches += 1;
    }
    fia_solver_report sr;
    std::memset(&sr, 0, sizeof(sr));
    auto project = [&]() -> int {
        if (p->capture_pair) {
            const int c = capture_pair(s, p->capture_tol);
            if (c < 0) return c;
        }
        return pressure<T>(s, &p->solver, &sr, true);
    };
    if (p->frame == 0) {
        if ((r = project()) < 0) return r;
        status |= r;
        if ((r = advect_velocity<T>(s, dt, &p->advect)) < 0) return r;
    } else {
        if ((r = advect_velocity<T>(s, dt, &p->advect)) < 0) return r;
        if ((r = project()) < 0) return r;
        status |= r;
    }
    status |= finish_status(s);
    double m0, m1;
    if ((r = read_reduction<T>(s, s->rho, nc, 0, &m0)) != FIA_OK) return r;
    if ((r = move_substances<T>(s, dt, &p->advect)) < 0) return r;
    status |= finish_status(s);
    if (s->solid) {
        k_clear_solid<T><<<1024, 256, 0, s->stream>>>((T*)s->rho, nc, s->solid);
        s->launches += 1;
    }
    if ((r = read_reduction<T>(s, s->rho, nc, 0, &m1)) != FIA_OK) return r;
    double m2 = m1;
    if (p->mass_correction && m1 != 0.0 && m0 != 0.0) {
        k_scale<T><<<1024, 256, 0, s->stream>>>((T*)s->rho, nc, m0 / m1);
        s->launches += 1;
        if ((r = read_reduction<T>(s, s->rho, nc, 0, &m2)) != FIA_OK) return r;
    }
    if (rep) {
        rep->dt = dt; rep->max_velocity = umax;
        rep->mass_before_advection = m0 * V; rep->mass_after_advection = m1 * V; rep->mass_after = m2 * V;
        rep->solver_iterations = sr.iterations; rep->solver_rel_residual = sr.rel_residual;
        rep->status = status;
        rep->solver_fcg_iterations = sr.fcg_iterations;
        rep->precond_ms = sr.precond_ms;
    }
    return status;
}

}  // namespace

// =====================================================================================
extern "C" {

void fia_default_step_params(fia_step_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    fia_default_advect_params(&p->advect);
    fia_default_solver_params(&p->solver);
    p->cfl = 1.0;
    p->max_dt = 1.0 / 60.0;
    p->buoyancy = 1.0;
    p->source = 1;
    p->source_center[0] = 0.5; p->source_center[1] = 0.15; p->source_center[2] = 0.5;
    p->source_radius = 0.1;
    p->source_density = 1.0;
    p->mass_correction = 1;
    p->frame = 0;
    p->capture_pair = 0;
    p->capture_tol = 1e-10;
}

int fia_step(fia_session* s, const fia_step_params* p, fia_step_report* rep) {
    if (!s || !p || !(p->cfl > 0.0) || !(p->max_dt > 0.0)) return FIA_ERR_INVALID;
    int c = check_params(&p->advect);
    if (c == FIA_OK) c = check_form(s, p->advect.minimal_area);
    if (c != FIA_OK) return c;
    return s->precision == FIA_FP64 ? step<double>(s, p, rep) : step<float>(s, p, rep);
}

int fia_api_version(void) { return FIA_API_VERSION; }

int fia_gauss_rule(int k, double* nodes, double* weights) {
    if (!nodes || !weights || k < 1 || k > kMaxGauss || (k % 2) == 0) return FIA_ERR_INVALID;
    make_gauss(k, nodes, weights);
    return FIA_OK;
}

const char* fia_error_string(int code) {
    switch (code) {
        case FIA_OK: return "ok";
        case FIA_ERR_INVALID: return "invalid argument";
        case FIA_ERR_CUDA: return g_last_error.empty() ? "CUDA error" : g_last_error.c_str();
        case FIA_ERR_UNSUPPORTED: return g_last_unsupported.empty() ? "unsupported option" : g_last_unsupported.c_str();
        case FIA_ERR_NOMEM: return "device allocation failed";
        default: return code > 0 ? "completed with numerical status bits set" : "unknown error";
    }
}

void fia_default_advect_params(fia_advect_params* p) {
    if (!p) return;
    p->interpolation_method = FIA_INTERP_WENO6;
    p->split_method = FIA_SPLIT_XZ_CELLFACE;
    p->num_gauss_quadrature_point_for_integrate_density = 3;
    p->use_integral = 1;
    p->enable_eliminate_zero_velocity_false_diffusion = 1;
    p->use_MacCormack_scheme = 0;
    p->enable_cell_volume_correction = 0;
    p->minimal_area = 1.0;
}

void fia_default_solver_params(fia_solver_params* p) {
    if (!p) return;
    p->tol = 1e-6;
    p->max_iter = 10000;
    p->method = FIA_SOLVER_PCG_JACOBI;
    p->fallback_iter = 200;
}

fia_session* fia_create(int nx, int ny, int nz, double cell_length, int precision) {
    if (nx < 2 || ny < 2 || nz < 2 || !(cell_length > 0.0)) { g_last_error = "fia_create: bad grid"; return nullptr; }
    if (precision != FIA_FP64 && precision != FIA_FP32C) { g_last_error = "fia_create: unknown precision"; return nullptr; }
    if ((long long)(nx + 2) * (ny + 2) * (nz + 2) > (1LL << 31)) { g_last_error = "fia_create: grid too large"; return nullptr; }
    fia_session* s = new fia_session();
    std::memset(s->wall_loss, 0, sizeof(s->wall_loss));
    s->N[0] = nx; s->N[1] = ny; s->N[2] = nz; s->h = cell_length; s->precision = precision;
    s->es = precision == FIA_FP64 ? sizeof(double) : sizeof(float);
    s->last_status = 0; s->status_pending = false; s->counters_pending = false; s->launches = 0;
    s->counters_host[0] = s->counters_host[1] = s->counters_host[2] = s->counters_host[3] = s->counters_host[4] = 0;
    s->pin = nx * ny * nz - 1;
    s->n_free = (long long)nx * ny * nz - 1;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        g_last_error = "fia_create: stream"; delete s; return nullptr;
    }
    const long long big = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    auto alloc = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, bytes);
        s->allocations.push_back(p);
        return p;
    };
    bool ok = true;
    auto A = [&](void*& dst, size_t bytes) { dst = alloc(bytes); ok = ok && dst != nullptr; };
    const size_t fb = (size_t)big * s->es;
    const size_t pb = (size_t)big * 8;   // psi and face fluxes: one double or one float pair per node
    A(s->rho, fb); A(s->rho_next, fb); A(s->pres, fb); A(s->cbuf, (size_t)big * 8); A(s->psi, pb);
    for (int c = 0; c < 3; ++c) { A(s->vel[c], fb); A(s->vel_next[c], fb); A(s->flux[c], pb); A(s->flux_rev[c], pb); }
    A(s->verts, 3 * fb);
    s->verts_bytes = fb;
    for (int q = 0; q < 5; ++q) A(s->pw[q], fb);
    { void* t2; A(t2, 4 * sizeof(unsigned)); s->ticket = (unsigned*)t2; }
    void* t;
    A(t, pressure_partials() * sizeof(double)); s->part = (double*)t;
    A(t, kScalDoubles * sizeof(double)); s->scal = (double*)t;
    A(t, 8 * sizeof(double)); s->sums = (double*)t;
    A(t, sizeof(unsigned)); s->status = (unsigned*)t;
    A(t, 5 * sizeof(unsigned long long)); s->counters = (unsigned long long*)t;
    A(t, kRedBlocks * sizeof(double)); s->red_part = (double*)t;
    A(t, 4 * sizeof(double)); s->red_out = (double*)t;
    if (ok && precision == FIA_FP32C) {
        // about 2.8 pieces per face at CFL 2, three face families per pass; grown on demand
        // faces of one family of any (staggered) field fit in (nx+2)(ny+2)(nz+2)
        ok = piece_store_reserve(s->pieces, 10 * big + 1024, big) == cudaSuccess;
    }
    if (ok && precision == FIA_FP64) ok = piece_store64_reserve(s->pieces64, 10 * big + 1024, big) == cudaSuccess;
    if (!ok) {
        g_last_error = "fia_create: device allocation failed";
        fia_destroy(s);
        return nullptr;
    }
    cudaDeviceSynchronize();
    return s;
}

int fia_profile_faces(fia_session* s, int capacity) {
    if (!s || capacity < 0) return FIA_ERR_INVALID;
    CK(cudaStreamSynchronize(s->stream));
    for (cudaEvent_t e : s->prof_ev) cudaEventDestroy(e);
    s->prof_ev.assign(2 * (size_t)capacity, nullptr);
    for (auto& e : s->prof_ev) CK(cudaEventCreate(&e));
    s->prof_n = 0;
    return FIA_OK;
}

int fia_profile_faces_read(fia_session* s, double* total_ms, int* launches) {
    if (!s || !total_ms || !launches) return FIA_ERR_INVALID;
    CK(cudaStreamSynchronize(s->stream));
    double t = 0.0;
    for (int i = 0; i < s->prof_n; ++i) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->prof_ev[2 * i], s->prof_ev[2 * i + 1]));
        t += ms;
    }
    *total_ms = t;
    *launches = s->prof_n;
    for (cudaEvent_t e : s->prof_ev) cudaEventDestroy(e);
    s->prof_ev.clear();
    s->prof_n = 0;
    return FIA_OK;
}

void fia_destroy(fia_session* s) {
    if (!s) return;
    cudaStreamSynchronize(s->stream);
    for (cudaEvent_t e : s->prof_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : s->pev) if (e) cudaEventDestroy(e);
    if (s->fcg_ready)
        for (int j = 0; j <= kFcgMaxDirs; ++j) { cudaFree(s->fcg.d[j]); cudaFree(s->fcg.q[j]); }
    unet::net_destroy(s->net);
    piece_store_free(s->pieces);
    piece_store64_free(s->pieces64);
    if (s->p64) cudaFree(s->p64);
    if (s->solid) cudaFree(s->solid);
    for (void* p : s->allocations) cudaFree(p);
    cudaStreamDestroy(s->stream);
    delete s;
}

int fia_last_status(const fia_session* s) {
    if (!s) return FIA_ERR_INVALID;
    return finish_status(const_cast<fia_session*>(s));
}

void* fia_stream(fia_session* s) { return s ? (void*)s->stream : nullptr; }

int fia_synchronize(fia_session* s) {
    if (!s) return FIA_ERR_INVALID;
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_set_field(fia_session* s, int field, const void* host, int host_dtype) {
    if (!s || !host) return FIA_ERR_INVALID;
    const long long n = field_count(s, field);
    void* dst = field_ptr(s, field);
    if (n < 0 || !dst) return FIA_ERR_INVALID;
    const size_t hb = host_dtype == FIA_HOST_F64 ? 8 : (host_dtype == FIA_HOST_F32 ? 4 : 0);
    if (!hb) return FIA_ERR_INVALID;
    if (hb == s->es) {
        CK(cudaMemcpyAsync(dst, host, n * hb, cudaMemcpyHostToDevice, s->stream));
    } else {
        CK(cudaMemcpyAsync(s->cbuf, host, n * hb, cudaMemcpyHostToDevice, s->stream));
        if (hb == 4) k_convert<double, float><<<512, 256, 0, s->stream>>>((const float*)s->cbuf, (double*)dst, n);
        else k_convert<float, double><<<512, 256, 0, s->stream>>>((const double*)s->cbuf, (float*)dst, n);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_get_field(fia_session* s, int field, void* host, int host_dtype) {
    if (!s || !host) return FIA_ERR_INVALID;
    const long long n = field_count(s, field);
    void* src = field_ptr(s, field);
    if (n < 0 || !src) return FIA_ERR_INVALID;
    const size_t hb = host_dtype == FIA_HOST_F64 ? 8 : (host_dtype == FIA_HOST_F32 ? 4 : 0);
    if (!hb) return FIA_ERR_INVALID;
    if (hb == s->es) {
        CK(cudaMemcpyAsync(host, src, n * hb, cudaMemcpyDeviceToHost, s->stream));
    } else {
        if (hb == 4) k_convert<float, double><<<512, 256, 0, s->stream>>>((const double*)src, (float*)s->cbuf, n);
        else k_convert<double, float><<<512, 256, 0, s->stream>>>((const float*)src, (double*)s->cbuf, n);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(host, s->cbuf, n * hb, cudaMemcpyDeviceToHost, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_field_device_ptr(fia_session* s, int field, void** dev_ptr) {
    if (!s || !dev_ptr) return FIA_ERR_INVALID;
    void* p = field_ptr(s, field);
    if (!p) return FIA_ERR_INVALID;
    *dev_ptr = p;
    return FIA_OK;
}

int fia_move_substances_3D(fia_session* s, double dt, const fia_advect_params* p) {
    if (!s || !(dt >= 0.0)) return FIA_ERR_INVALID;
    int c = check_params(p);
    if (c == FIA_OK) c = check_form(s, p->minimal_area);
    if (c != FIA_OK) return c;
    return s->precision == FIA_FP64 ? move_substances<double>(s, dt, p) : move_substances<float>(s, dt, p);
}

int fia_advect_velocity_xyz(fia_session* s, double dt, const fia_advect_params* p) {
    if (!s || !(dt >= 0.0)) return FIA_ERR_INVALID;
    int c = check_params(p);
    if (c == FIA_OK) c = check_form(s, p->minimal_area);
    if (c != FIA_OK) return c;
    return s->precision == FIA_FP64 ? advect_velocity<double>(s, dt, p) : advect_velocity<float>(s, dt, p);
}

int fia_calc_pressure_3D(fia_session* s, const fia_solver_params* sp, fia_solver_report* rep) {
    if (!s) return FIA_ERR_INVALID;
    return s->precision == FIA_FP64 ? pressure<double>(s, sp, rep, false) : pressure<float>(s, sp, rep, false);
}

int fia_calc_pressure_gradient_term_3D(fia_session* s, const fia_solver_params* sp, fia_solver_report* rep) {
    if (!s) return FIA_ERR_INVALID;
    return s->precision == FIA_FP64 ? pressure<double>(s, sp, rep, true) : pressure<float>(s, sp, rep, true);
}

int fia_max_abs_velocity(fia_session* s, double* out) {
    if (!s || !out) return FIA_ERR_INVALID;
    CK(cudaMemsetAsync(s->red_out, 0, sizeof(double), s->stream));
    for (int c = 0; c < 3; ++c) {
        const long long n = field_count(s, FIA_FIELD_U + c);
        CK(s->precision == FIA_FP64 ? reduce<double>(s, s->vel[c], n, 1, true) : reduce<float>(s, s->vel[c], n, 1, true));
    }
    CK(cudaMemcpyAsync(out, s->red_out, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_total_mass(fia_session* s, double* out) {
    if (!s || !out) return FIA_ERR_INVALID;
    const long long n = field_count(s, FIA_FIELD_DENSITY);
    CK(s->precision == FIA_FP64 ? reduce<double>(s, s->rho, n, 0, false) : reduce<float>(s, s->rho, n, 0, false));
    double m = 0.0;
    CK(cudaMemcpyAsync(&m, s->red_out, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *out = m * (s->h * s->h * s->h);
    return FIA_OK;
}

int fia_wall_momentum_loss(fia_session* s, double* out3) {
    if (!s || !out3) return FIA_ERR_INVALID;
    for (int c = 0; c < 3; ++c) out3[c] = s->wall_loss[c];
    return FIA_OK;
}

int fia_total_momentum(fia_session* s, double* out3) {
    if (!s || !out3) return FIA_ERR_INVALID;
    const double V = s->h * s->h * s->h;
    for (int c = 0; c < 3; ++c) {
        const long long n = field_count(s, FIA_FIELD_U + c);
        CK(s->precision == FIA_FP64 ? reduce<double>(s, s->vel[c], n, 0, false) : reduce<float>(s, s->vel[c], n, 0, false));
        double m = 0.0;
        CK(cudaMemcpyAsync(&m, s->red_out, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        out3[c] = m * V;
    }
    return FIA_OK;
}

int fia_write_density_frame(fia_session* s, const char* path, int frame) {
    if (!s || !path) return FIA_ERR_INVALID;
    static_assert(sizeof(fia_frame_header) == 64, "frame header layout");
    fia_frame_header hd;
    std::memset(&hd, 0, sizeof(hd));
    std::memcpy(hd.magic, "FIAFRM1", 8);
    hd.nx = s->N[0]; hd.ny = s->N[1]; hd.nz = s->N[2];
    hd.frame = frame;
    for (int c = 0; c < 3; ++c) hd.origin[c] = -0.5 * s->h * s->N[c];
    hd.voxel_size = s->h;
    const long long n = field_count(s, FIA_FIELD_DENSITY);
    std::vector<float> data((size_t)n);
    int r = fia_get_field(s, FIA_FIELD_DENSITY, data.data(), FIA_HOST_F32);
    if (r != FIA_OK) return r;
    FILE* f = std::fopen(path, "wb");
    if (!f) { g_last_error = std::string("fia_write_density_frame: cannot open ") + path; return FIA_ERR_INVALID; }
    const bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 && std::fwrite(data.data(), sizeof(float), (size_t)n, f) == (size_t)n;
    if (std::fclose(f) != 0 || !ok) { g_last_error = std::string("fia_write_density_frame: write failed: ") + path; return FIA_ERR_INVALID; }
    return FIA_OK;
}

int fia_append_totals(fia_session* s, const char* prefix, double now_time) {
    if (!s || !prefix) return FIA_ERR_INVALID;
    double mass = 0.0, mom[3], loss[3];
    int r = fia_total_mass(s, &mass);
    if (r == FIA_OK) r = fia_total_momentum(s, mom);
    if (r == FIA_OK) r = fia_wall_momentum_loss(s, loss);
    if (r != FIA_OK) return r;
    auto append = [&](const std::string& name, double v) -> bool {
        FILE* f = std::fopen((std::string(prefix) + name).c_str(), "a");
        if (!f) return false;
        const bool ok = std::fprintf(f, "%.16g %.16g\n", now_time, v) > 0;
        return std::fclose(f) == 0 && ok;
    };
    bool ok = append("total_mass.dat", mass);
    static const char* ax[3] = {"x", "y", "z"};
    for (int c = 0; c < 3 && ok; ++c) {
        ok = append(std::string("total_momentum_") + ax[c] + ".dat", mom[c]) &&
             append(std::string("total_loss_of_momentum_") + ax[c] + ".dat", loss[c]) &&
             append(std::string("momentum_") + ax[c] + "_plus_total_loss_of_momentum_" + ax[c] + ".dat", mom[c] + loss[c]);
    }
    if (!ok) { g_last_error = std::string("fia_append_totals: cannot write under ") + prefix; return FIA_ERR_INVALID; }
    return FIA_OK;
}

int fia_pass_counters(fia_session* s, unsigned long long* out5) {
    if (!s || !out5) return FIA_ERR_INVALID;
    if (s->counters_pending) {
        CK(cudaMemcpyAsync(s->counters_host, s->counters, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        s->counters_pending = false;
    }
    for (int q = 0; q < 4; ++q) out5[q] = s->counters_host[q];
    out5[4] = s->launches;
    return FIA_OK;
}

int fia_move_substances_3D_host(fia_session* s, int host_dtype, void* rho, const void* u, const void* v,
                                const void* w, double dt, const fia_advect_params* p) {
    int r;
    if ((r = fia_set_field(s, FIA_FIELD_DENSITY, rho, host_dtype)) != FIA_OK) return r;
    if ((r = fia_set_field(s, FIA_FIELD_U, u, host_dtype)) != FIA_OK) return r;
    if ((r = fia_set_field(s, FIA_FIELD_V, v, host_dtype)) != FIA_OK) return r;
    if ((r = fia_set_field(s, FIA_FIELD_W, w, host_dtype)) != FIA_OK) return r;
    if ((r = fia_move_substances_3D(s, dt, p)) < 0) return r;
    if ((r = fia_get_field(s, FIA_FIELD_DENSITY, rho, host_dtype)) != FIA_OK) return r;
    return fia_last_status(s);
}

int fia_advect_velocity_xyz_host(fia_session* s, int host_dtype, void* u, void* v, void* w, double dt,
                                 const fia_advect_params* p) {
    int r;
    void* f[3] = {u, v, w};
    for (int c = 0; c < 3; ++c) if ((r = fia_set_field(s, FIA_FIELD_U + c, f[c], host_dtype)) != FIA_OK) return r;
    if ((r = fia_advect_velocity_xyz(s, dt, p)) < 0) return r;
    for (int c = 0; c < 3; ++c) if ((r = fia_get_field(s, FIA_FIELD_U + c, f[c], host_dtype)) != FIA_OK) return r;
    return fia_last_status(s);
}

int fia_calc_pressure_gradient_term_3D_host(fia_session* s, int host_dtype, void* u, void* v, void* w,
                                            void* pressure_out, const fia_solver_params* sp,
                                            fia_solver_report* rep) {
    int r;
    void* f[3] = {u, v, w};
    for (int c = 0; c < 3; ++c) if ((r = fia_set_field(s, FIA_FIELD_U + c, f[c], host_dtype)) != FIA_OK) return r;
    const int st = fia_calc_pressure_gradient_term_3D(s, sp, rep);
    if (st < 0) return st;
    for (int c = 0; c < 3; ++c) if ((r = fia_get_field(s, FIA_FIELD_U + c, f[c], host_dtype)) != FIA_OK) return r;
    if (pressure_out && (r = fia_get_field(s, FIA_FIELD_PRESSURE, pressure_out, host_dtype)) != FIA_OK) return r;
    return st;
}

int fia_debug_flux_pass(fia_session* s, int comp, const double* field, double dt, int interp, int psi_mode,
                        int use_integral, int zero_velocity, const double* co, int k, double minimal_area,
                        double* out) {
    if (!s || !field || !out || !co || comp < -1 || comp > 2 || k < 1 || k > kMaxGauss || interp < 0 || interp > 2 ||
        psi_mode < 0 || psi_mode > 2 || !(minimal_area > 0.0))
        return FIA_ERR_INVALID;
    const int c = check_form(s, minimal_area);
    if (c != FIA_OK) return c;
    if (s->precision == FIA_FP64)
        return debug_flux_pass<double>(s, comp, field, dt, interp, psi_mode, use_integral, zero_velocity, co, k,
                                       minimal_area, out);
    return debug_flux_pass<float>(s, comp, field, dt, interp, psi_mode, use_integral, zero_velocity, co, k,
                                  minimal_area, out);
}

int fia_debug_backtrace(fia_session* s, int comp, double dt, int interp, double* out) {
    if (!s || !out || comp < -1 || comp > 2 || interp < 0 || interp > 2) return FIA_ERR_INVALID;
    return s->precision == FIA_FP64 ? debug_backtrace<double>(s, comp, dt, interp, out)
                                    : debug_backtrace<float>(s, comp, dt, interp, out);
}

int fia_debug_psi(fia_session* s, int comp, const double* field, int mode, int k, double* out) {
    if (!s || !field || !out || comp < -1 || comp > 2 || mode < 0 || mode > 2 || k < 1 || k > kMaxGauss)
        return FIA_ERR_INVALID;
    return s->precision == FIA_FP64 ? debug_psi<double>(s, comp, field, mode, k, out)
                                    : debug_psi<float>(s, comp, field, mode, k, out);
}

// ------------------------------- solids -------------------------------------------
int fia_set_solid_spheres(fia_session* s, int count, const double* centers, const double* radii) {
    if (!s || count < 0 || (count > 0 && (!centers || !radii))) return FIA_ERR_INVALID;
    const int nx = s->N[0], ny = s->N[1], nz = s->N[2];
    const long long nc = (long long)nx * ny * nz;
    CK(cudaStreamSynchronize(s->stream));
    if (count == 0) {
        if (s->solid) CK(cudaFree(s->solid));
        s->solid = nullptr;
        s->pin = (int)(nc - 1);
        s->n_free = nc - 1;
        return FIA_OK;
    }
    std::vector<unsigned char> m(nc, 0);
    long long nsolid = 0;
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < ny; ++iy)
            for (int iz = 0; iz < nz; ++iz) {
                const double x = (ix + 0.5) * s->h, y = (iy + 0.5) * s->h, z = (iz + 0.5) * s->h;
                for (int k = 0; k < count; ++k) {
                    const double dx = x - centers[3 * k], dy = y - centers[3 * k + 1], dz = z - centers[3 * k + 2];
                    if (dx * dx + dy * dy + dz * dz <= radii[k] * radii[k]) {
                        m[((long long)ix * ny + iy) * nz + iz] = 1;
                        ++nsolid;
                        break;
                    }
                }
            }
    long long pin = nc - 1;
    while (pin >= 0 && m[pin]) --pin;
    if (pin < 0) return FIA_ERR_INVALID;   // no fluid cell left
    if (!s->solid) CK(cudaMalloc(&s->solid, nc));
    CK(cudaMemcpy(s->solid, m.data(), nc, cudaMemcpyHostToDevice));
    s->pin = (int)pin;
    s->n_free = nc - nsolid - 1;
    // no velocity through solid faces, no density inside
    if (s->precision == FIA_FP64) {
        k_solid_faces<double><<<1024, 256, 0, s->stream>>>((double*)s->vel[0], (double*)s->vel[1], (double*)s->vel[2],
                                                           nx, ny, nz, s->solid);
        k_clear_solid<double><<<1024, 256, 0, s->stream>>>((double*)s->rho, nc, s->solid);
    } else {
        k_solid_faces<float><<<1024, 256, 0, s->stream>>>((float*)s->vel[0], (float*)s->vel[1], (float*)s->vel[2], nx,
                                                          ny, nz, s->solid);
        k_clear_solid<float><<<1024, 256, 0, s->stream>>>((float*)s->rho, nc, s->solid);
    }
    s->launches += 2;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_get_solid_mask(fia_session* s, unsigned char* out) {
    if (!s || !out) return FIA_ERR_INVALID;
    const long long nc = (long long)s->N[0] * s->N[1] * s->N[2];
    if (!s->solid) { std::memset(out, 0, nc); return FIA_OK; }
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(out, s->solid, nc, cudaMemcpyDeviceToHost));
    return FIA_OK;
}

// ------------------------------- learned preconditioner ---------------------------
static int ensure_net(fia_session* s) {
    if (s->precision != FIA_FP32C) {
        g_last_unsupported = "the learned preconditioner needs an FP32C session";
        return FIA_ERR_UNSUPPORTED;
    }
    if (!s->net) {
        s->net = unet::net_create(s->N[0], s->N[1], s->N[2], s->stream);
        if (!s->net) { g_last_error = "fia_learned: device allocation failed"; return FIA_ERR_NOMEM; }
    }
    return FIA_OK;
}

long long fia_learned_num_parameters(void) { return unet::num_parameters(); }

int fia_learned_init(fia_session* s, unsigned long long seed) {
    if (!s) return FIA_ERR_INVALID;
    int r = ensure_net(s);
    if (r != FIA_OK) return r;
    CK(unet::net_init(s->net, seed));
    return FIA_OK;
}

int fia_learned_set_weights(fia_session* s, const float* w, long long count) {
    if (!s || !w || count != unet::num_parameters()) return FIA_ERR_INVALID;
    int r = ensure_net(s);
    if (r != FIA_OK) return r;
    CK(unet::net_set_weights(s->net, w, count));
    return FIA_OK;
}

int fia_learned_get_weights(fia_session* s, float* w, long long count) {
    if (!s || !w || !s->net || count != unet::num_parameters()) return FIA_ERR_INVALID;
    CK(unet::net_get_weights(s->net, w, count));
    return FIA_OK;
}

int fia_learned_add_pair(fia_session* s, const float* r, const float* p) {
    if (!s || !r || !p || !s->net) return FIA_ERR_INVALID;
    const long long nc = (long long)s->N[0] * s->N[1] * s->N[2];
    float *dr = (float*)s->pw[0], *dp = (float*)s->pw[1];
    CK(cudaMemcpyAsync(dr, r, nc * 4, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(dp, p, nc * 4, cudaMemcpyHostToDevice, s->stream));
    const int id = unet::net_add_pair(s->net, poisson_grid(s), dr, dp, s->stream);
    return id < 0 ? FIA_ERR_INVALID : FIA_OK;
}

int fia_learned_num_pairs(fia_session* s) {
    if (!s || !s->net) return 0;
    return unet::net_num_pairs(s->net);
}

int fia_learned_loss(fia_session* s, int pair, double* loss) {
    if (!s || !s->net || !loss || pair < 0 || pair >= unet::net_num_pairs(s->net)) return FIA_ERR_INVALID;
    CK(unet::net_loss(s->net, poisson_grid(s), pair, false, loss, s->stream));
    return FIA_OK;
}

int fia_learned_calibrate(fia_session* s, int pair) {
    if (!s || !s->net || pair < 0 || pair >= unet::net_num_pairs(s->net)) return FIA_ERR_INVALID;
    CK(unet::net_calibrate(s->net, poisson_grid(s), pair, s->stream));
    return FIA_OK;
}

int fia_learned_train_step(fia_session* s, const int* pairs, int batch, double lr, double* losses) {
    if (!s || !s->net || !pairs || batch < 1 || !(lr > 0.0)) return FIA_ERR_INVALID;
    const int np = unet::net_num_pairs(s->net);
    for (int i = 0; i < batch; ++i)
        if (pairs[i] < 0 || pairs[i] >= np) return FIA_ERR_INVALID;
    const PoissonGrid g = poisson_grid(s);
    for (int i = 0; i < batch; ++i) {
        double l = 0.0;
        CK(unet::net_loss(s->net, g, pairs[i], true, &l, s->stream));
        if (losses) losses[i] = l;
    }
    CK(unet::net_adam_step(s->net, lr, batch, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_learned_level_dims(fia_session* s, int level, int* dims3) {
    if (!s || !dims3 || level < 0 || level > 3) return FIA_ERR_INVALID;
    int r = ensure_net(s);
    if (r != FIA_OK) return r;
    unet::net_level_dims(s->net, level, dims3);
    return FIA_OK;
}

int fia_debug_unet_forward(fia_session* s, const float* x0, float* y) {
    if (!s || !s->net || !x0 || !y) return FIA_ERR_INVALID;
    int d[3];
    unet::net_level_dims(s->net, 0, d);
    const long long n = (long long)d[0] * d[1] * d[2];
    float *dx = (float*)s->pw[0], *dy = (float*)s->pw[1];
    CK(cudaMemcpyAsync(dx, x0, n * 4, cudaMemcpyHostToDevice, s->stream));
    CK(unet::net_forward_level0(s->net, dx, dy, s->stream));
    CK(cudaMemcpyAsync(y, dy, n * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_debug_unet_backward(fia_session* s, const float* x0, const float* gy, float* grads) {
    if (!s || !s->net || !x0 || !gy || !grads) return FIA_ERR_INVALID;
    int d[3];
    unet::net_level_dims(s->net, 0, d);
    const long long n = (long long)d[0] * d[1] * d[2];
    float *dx = (float*)s->pw[0], *dg = (float*)s->pw[1];
    CK(cudaMemcpyAsync(dx, x0, n * 4, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(dg, gy, n * 4, cudaMemcpyHostToDevice, s->stream));
    CK(unet::net_zero_grad(s->net, s->stream));
    CK(unet::net_forward_level0(s->net, dx, nullptr, s->stream));
    CK(unet::net_backward_level0(s->net, dg, s->stream));
    CK(unet::net_get_grads(s->net, grads, unet::num_parameters()));
    CK(unet::net_zero_grad(s->net, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_debug_learned_grad(fia_session* s, int pair, float* grads, double* loss) {
    if (!s || !s->net || !grads || pair < 0 || pair >= unet::net_num_pairs(s->net)) return FIA_ERR_INVALID;
    CK(unet::net_zero_grad(s->net, s->stream));
    double l = 0.0;
    CK(unet::net_loss(s->net, poisson_grid(s), pair, true, &l, s->stream));
    CK(unet::net_get_grads(s->net, grads, unet::num_parameters()));
    CK(unet::net_zero_grad(s->net, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (loss) *loss = l;
    return FIA_OK;
}

int fia_debug_set_piece_capacity(fia_session* s, long long pieces) {
    if (!s || pieces < 1) return FIA_ERR_INVALID;
    CK(cudaStreamSynchronize(s->stream));
    const long long big = (long long)(s->N[0] + 2) * (s->N[1] + 2) * (s->N[2] + 2);
    if (s->precision == FIA_FP64) {
        piece_store64_free(s->pieces64);
        CK(piece_store64_reserve(s->pieces64, pieces, big));
        return FIA_OK;
    }
    const int fast = s->pieces.clip_fast;
    piece_store_free(s->pieces);
    s->pieces.clip_fast = fast;
    CK(piece_store_reserve(s->pieces, pieces, big));
    return FIA_OK;
}

int fia_debug_vertex_jitter(fia_session* s, double cells) {
    if (!s || s->precision != FIA_FP64 || !(cells >= 0.0) || cells > 0.5) return FIA_ERR_INVALID;
    s->vertex_jitter = cells;
    return FIA_OK;
}

int fia_debug_piece_pipeline(fia_session* s, int enable) {
    if (!s || enable < -1 || enable > 1) return FIA_ERR_INVALID;
    if (enable >= 0) {
        if (s->precision != FIA_FP64) return FIA_ERR_INVALID;
        CK(cudaStreamSynchronize(s->stream));
        s->piece_pipeline = enable;
    }
    return s->precision == FIA_FP64 ? s->piece_pipeline : 0;
}

int fia_debug_full_weno(fia_session* s, int enable) {
    if (!s || enable < -1 || enable > 1) return FIA_ERR_INVALID;
    if (enable >= 0) s->full_weno = enable;
    return s->full_weno;
}

int fia_debug_clip_fast(fia_session* s, int enable, unsigned long long* deferred) {
    if (!s || s->precision != FIA_FP32C || enable < -1 || enable > 1) return FIA_ERR_INVALID;
    if (enable >= 0) s->pieces.clip_fast = enable;
    if (deferred) {
        CK(cudaMemcpyAsync(deferred, s->counters + 4, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return FIA_OK;
}

long long fia_debug_piece_capacity(fia_session* s) {
    if (!s) return -1;
    return s->precision == FIA_FP64 ? s->pieces64.cap : s->pieces.cap;
}

int fia_debug_solve_rhs(fia_session* s, const float* rhs, float* x, const fia_solver_params* sp,
                        fia_solver_report* rep) {
    if (!s || !rhs || !x || !sp || s->precision != FIA_FP32C) return FIA_ERR_INVALID;
    const long long nc = (long long)s->N[0] * s->N[1] * s->N[2];
    float* drhs = (float*)s->cbuf;
    CK(cudaMemcpyAsync(drhs, rhs, nc * 4, cudaMemcpyHostToDevice, s->stream));
    PressureReport r;
    int fcg_its = 0, extra = 0;
    double pms = 0.0;
    if (sp->method == FIA_SOLVER_FCG_LEARNED) {
        if (!s->net) return FIA_ERR_INVALID;
        const int rc = pressure_fcg(s, sp, r, fcg_its, pms, drhs);
        if (rc < 0) return rc;
        extra = rc;
    } else {
        PressureWork<float> W = pressure_work<float>(s);
        const PoissonGrid g = poisson_grid(s);
        double rr;
        CK(cudaMemsetAsync(W.p, 0, nc * 4, s->stream));
        CK(pressure_residual<float>(W, g, drhs, &rr, s->stream));
        CK(pressure_pcg<float>(W, g, rr, rr, sp->tol, sp->max_iter, &r, s->stream));
    }
    CK(cudaMemcpyAsync(x, s->pres, nc * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const int status = (r.status ? FIA_STATUS_SOLVER_CAP : 0) | extra;
    if (rep) {
        rep->iterations = r.iterations; rep->rel_residual = r.rel_residual; rep->status = status;
        rep->fcg_iterations = fcg_its; rep->precond_ms = pms;
    }
    return status;
}

int fia_debug_grid_op(fia_session* s, int op, const float* in, float* out) {
    if (!s || !s->net || !in || !out || op < 0 || op > 2) return FIA_ERR_INVALID;
    int d[3];
    unet::net_level_dims(s->net, 0, d);
    const long long nc = (long long)s->N[0] * s->N[1] * s->N[2], n0 = (long long)d[0] * d[1] * d[2];
    const long long nin = op == 1 ? n0 : nc, nout = op == 1 ? nc : n0;
    float *din = (float*)s->pw[0], *dout = (float*)s->pw[1];
    CK(cudaMemcpyAsync(din, in, nin * 4, cudaMemcpyHostToDevice, s->stream));
    CK(unet::net_grid_op(s->net, poisson_grid(s), op, din, dout, s->stream));
    CK(cudaMemcpyAsync(out, dout, nout * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

int fia_debug_learned_tc(fia_session* s, int enable, unsigned* status) {
    if (!s || enable < -1 || enable > 1) return FIA_ERR_INVALID;
    int r = ensure_net(s);
    if (r != FIA_OK) return r;
    if (enable >= 0) unet::net_set_tc(s->net, enable == 1);
    if (status) CK(unet::net_tc_status(s->net, status, s->stream));
    return FIA_OK;
}

int fia_debug_precondition(fia_session* s, const float* r, float* z) {
    if (!s || !s->net || !r || !z) return FIA_ERR_INVALID;
    const long long nc = (long long)s->N[0] * s->N[1] * s->N[2];
    float *dr = (float*)s->pw[0], *dz = (float*)s->pw[1];
    CK(cudaMemcpyAsync(dr, r, nc * 4, cudaMemcpyHostToDevice, s->stream));
    // r.r into the solver scalar the preconditioner reads
    std::vector<float> h(r, r + nc);
    double rr = 0.0;
    for (long long i = 0; i < nc; ++i) rr += (double)h[i] * h[i];
    CK(cudaMemcpyAsync(s->scal + kScalRR, &rr, sizeof(double), cudaMemcpyHostToDevice, s->stream));
    CK(unet::net_apply(s->net, poisson_grid(s), dr, dz, s->scal + kScalRR, (double)s->n_free, s->stream));
    CK(cudaMemcpyAsync(z, dz, nc * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FIA_OK;
}

}  // extern "C"
