// fia_noalloc.cu -- density flux advection on caller-owned device buffers with no device
// allocation (fia_move_substances_3D_noalloc in include/fia.h).
//
// Some callers cannot call cudaMalloc: a host application that owns all device memory and
// hands a plug-in only the buffers it may touch (a renderer or game-engine integration with
// a fixed memory budget), or a real-time loop where an allocation's latency, and the chance
// that it fails mid-run, are not acceptable.  Such a caller passes its density and velocity
// buffers and gets the advected density back; the scratch the pass needs (psi, the
// backtraced vertex lattice, the face fluxes, the zero-velocity correction field, the status
// word) lives in a file-scope device array of fixed size, held by every GPU that has loaded
// this module until the process exits.
//
// When the scratch is reserved: CUDA loads a module's device code lazily by default, so the
// driver reserves the 23.6 MB on a device when this module is first used there, i.e. during
// the first call on that device (which also looks up the array's device address).  A caller
// whose memory budget must be settled up front makes one call at initialisation (any small
// grid), or sets CUDA_MODULE_LOADING=EAGER so that the reservation happens when the context
// is created; that first call must come before any stream capture.  The looked-up address
// is kept for the life of the process: a cudaDeviceReset after the first call on a device is
// not supported.
//
// Limit: at most kMaxCells cells per axis (64, i.e. up to 64^3 cells; 23.6 MB of scratch).
// Calls share the scratch: two calls whose work overlaps on the GPU (different streams, or
// different host threads) race on it and produce wrong results.  Each call clears what must
// start at zero (the status word) itself.
#include "../../include/fia.h"
#include "fia_advect.cuh"

#include <cmath>
#include <cstring>
#include <mutex>

namespace {

using namespace fia;

constexpr int kMaxCells = 64;
constexpr size_t kPsi = (size_t)kMaxCells * (kMaxCells + 1) * kMaxCells;
constexpr size_t kVerts = 3 * (size_t)(kMaxCells + 1) * (kMaxCells + 1) * (kMaxCells + 1);
constexpr size_t kFlux = (size_t)(kMaxCells + 1) * kMaxCells * kMaxCells;
constexpr size_t kCells = (size_t)kMaxCells * kMaxCells * kMaxCells;
constexpr size_t kScratchDoubles = kPsi + kVerts + 6 * kFlux + kCells;

// The scratch.  In host code these names are host-side stand-ins, not device addresses:
// the device address of each is obtained with cudaGetSymbolAddress below.
__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];
__device__ __align__(256) unsigned long long g_noalloc_words[8];   // [0] status, [1..4] counters

struct DeviceScratch {
    double* scratch = nullptr;
    unsigned long long* words = nullptr;
};
constexpr int kMaxDevices = 64;
DeviceScratch g_dev[kMaxDevices];
std::mutex g_mu;
thread_local char g_msg[256];

// Device addresses of the scratch on the current device, looked up on its first use.
int device_scratch(DeviceScratch* out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FIA_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    DeviceScratch& d = g_dev[dev];
    if (!d.scratch) {
        double* s = nullptr;
        unsigned long long* w = nullptr;
        if (cudaGetSymbolAddress((void**)&s, g_noalloc_scratch) != cudaSuccess) return FIA_ERR_CUDA;
        if (cudaGetSymbolAddress((void**)&w, g_noalloc_words) != cudaSuccess) return FIA_ERR_CUDA;
        d.scratch = s;
        d.words = w;
    }
    *out = d;
    return FIA_OK;
}

int fail(int code, const char* msg) {
    std::strncpy(g_msg, msg, sizeof(g_msg) - 1);
    g_msg[sizeof(g_msg) - 1] = 0;
    return code;
}

}  // namespace

extern "C" {

const char* fia_noalloc_error_string(void) { return g_msg; }

int fia_move_substances_3D_noalloc(int nx, int ny, int nz, double cell_length, const double* density_in,
                                   double* density_out, const double* u, const double* v, const double* w,
                                   double time_step_length, const fia_advect_params* p, void* stream) {
    if (nx < 2 || ny < 2 || nz < 2 || !(cell_length > 0.0) || !(time_step_length >= 0.0))
        return fail(FIA_ERR_INVALID, "fia_move_substances_3D_noalloc: bad grid size, cell length or time step");
    if (nx > kMaxCells || ny > kMaxCells || nz > kMaxCells)
        return fail(FIA_ERR_INVALID, "fia_move_substances_3D_noalloc: grid exceeds the static scratch "
                                     "(at most 64 cells per axis); use a session (fia_create) instead");
    if (!density_in || !density_out || !u || !v || !w || !p || density_in == density_out)
        return fail(FIA_ERR_INVALID, "fia_move_substances_3D_noalloc: null buffer, or input and output alias");
    if (p->use_MacCormack_scheme || p->enable_cell_volume_correction)
        return fail(FIA_ERR_UNSUPPORTED, "fia_move_substances_3D_noalloc: MacCormack / cell-volume correction");
    const int k = p->num_gauss_quadrature_point_for_integrate_density;
    if ((p->interpolation_method != FIA_INTERP_WENO6 && p->interpolation_method != FIA_INTERP_LINEAR) ||
        p->split_method < 0 || p->split_method > 3 || k < 1 || k > kMaxGauss || (k % 2) == 0 ||
        !(p->minimal_area > 0.0))
        return fail(FIA_ERR_INVALID, "fia_move_substances_3D_noalloc: invalid advection parameters");
    DeviceScratch ds;
    if (device_scratch(&ds) != FIA_OK) return fail(FIA_ERR_CUDA, "fia_move_substances_3D_noalloc: scratch lookup");
    cudaStream_t s = (cudaStream_t)stream;

    // scratch layout
    PassWork<double> work;
    double* base = ds.scratch;
    work.psi = base; base += kPsi;
    work.verts = base; base += kVerts;
    for (int f = 0; f < 3; ++f) { work.flux[f] = base; base += kFlux; }
    for (int f = 0; f < 3; ++f) { work.flux_rev[f] = base; base += kFlux; }
    double* corr = base;
    work.status = (unsigned*)ds.words;
    work.counters = ds.words + 1;
    work.prof_ev = nullptr; work.prof_n = nullptr; work.prof_cap = 0;
    if (cudaMemsetAsync(ds.words, 0, 8 * sizeof(unsigned long long), s) != cudaSuccess)
        return fail(FIA_ERR_CUDA, "fia_move_substances_3D_noalloc: clearing the status word");

    PassDesc d;
    std::memset(&d, 0, sizeof(d));
    d.N[0] = nx; d.N[1] = ny; d.N[2] = nz;
    d.comp = -1;
    d.A.Mx = nx; d.A.My = ny; d.A.Mz = nz; d.A.ox = d.A.oy = d.A.oz = 0.5;
    d.P = d.A; d.P.My = ny + 1; d.P.oy = 0.0;
    d.h = cell_length; d.dt = time_step_length;
    d.k = k;
    make_gauss(k, d.gx, d.gw);   // the session's rule (fixed arrays, no heap)
    d.minimal_area = p->minimal_area;
    static const double split_tbl[4][2] = {{0.5, 0.5}, {0.0, 0.0}, {0.5, 0.0}, {0.0, 0.5}};

    VelocityFields vel;
    vel.u = u; vel.v = v; vel.w = w;
    vel.fu.Mx = nx + 1; vel.fu.My = ny; vel.fu.Mz = nz; vel.fu.ox = 0.0; vel.fu.oy = 0.5; vel.fu.oz = 0.5;
    vel.fv.Mx = nx; vel.fv.My = ny + 1; vel.fv.Mz = nz; vel.fv.ox = 0.5; vel.fv.oy = 0.0; vel.fv.oz = 0.5;
    vel.fw.Mx = nx; vel.fw.My = ny; vel.fw.Mz = nz + 1; vel.fw.ox = 0.5; vel.fw.oy = 0.5; vel.fw.oz = 0.0;

    // move_substances_3d.cpp:58-226: main pass, zero-velocity pass, error advection
    d.interp = p->interpolation_method == FIA_INTERP_WENO6 ? INTERP_WENO6 : INTERP_LINEAR;
    d.use_integral = p->use_integral ? 1 : 0;
    d.psi_mode = p->use_integral ? (d.interp == INTERP_WENO6 ? PSI_WENO6 : PSI_LINEAR) : PSI_PLAIN;
    d.zero_velocity = 0;
    d.color_off[0] = split_tbl[p->split_method][0]; d.color_off[1] = split_tbl[p->split_method][1];
    if (run_pass<double>(d, vel, density_in, work, density_in, density_out, 0, s) != cudaSuccess)
        return fail(FIA_ERR_CUDA, "fia_move_substances_3D_noalloc: launch");
    if (p->enable_eliminate_zero_velocity_false_diffusion) {
        d.zero_velocity = 1; d.use_integral = 0; d.psi_mode = PSI_PLAIN;
        if (run_pass<double>(d, vel, density_in, work, density_in, corr, 1, s) != cudaSuccess)
            return fail(FIA_ERR_CUDA, "fia_move_substances_3D_noalloc: launch");
        d.zero_velocity = 0; d.interp = INTERP_1DY_LINEAR;
        d.color_off[0] = split_tbl[FIA_SPLIT_XZ_AXIS][0]; d.color_off[1] = split_tbl[FIA_SPLIT_XZ_AXIS][1];
        if (run_pass<double>(d, vel, corr, work, nullptr, density_out, 2, s) != cudaSuccess)
            return fail(FIA_ERR_CUDA, "fia_move_substances_3D_noalloc: launch");
    }
    unsigned long long status = 0;
    if (cudaMemcpyAsync(&status, ds.words, sizeof(status), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail(FIA_ERR_CUDA, "fia_move_substances_3D_noalloc: reading the status word");
    return (int)(status & 0xffffffffu);
}

}  // extern "C"
