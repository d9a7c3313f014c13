// fia_advect.cuh -- host-side description of one flux-advection pass and the launchers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "fia_device.cuh"

namespace fia {

constexpr int kMaxGauss = 15;

// Triangulation of pieces above minimal_area bisects each triangle's longest edge
// (facecutter.h:255-324).  Edges whose squared lengths agree to within this relative amount
// count as equally long and the first of them is taken, as for an exact tie: equal lengths in
// exact arithmetic (the fan triangles of a square) would otherwise be ordered by rounding,
// differently in FP32 and FP64.  The oracle applies the same rule.
constexpr double kLongestEdgeTie = 4e-6;

// Everything one flux pass needs; passed to the kernels by value.
struct PassDesc {
    NodeField A;            // advected node field (its cells are the control volumes)
    NodeField P;            // psi of A (y-faces of A's cells)
    int N[3];               // base grid (cells of the density)
    int comp;               // -1 density, 0/1/2 velocity component: staggering + pin rule
    int interp;             // Interp for the backtrace velocity, the values and psi
    int psi_mode;           // PSI_PLAIN / PSI_WENO6 / PSI_LINEAR
    int use_integral;       // 1: y-integral quadrature per piece (polygon_3D.cpp:257-487)
    int zero_velocity;      // 1: faces are not moved (zero-velocity pass)
    int maccormack;         // flux MacCormack: faces at rest (0.5), backtraced (1), traced back (-0.5)
    int volumes;            // also sum y n_y of the pieces per face into PassWork::fvol (cell volumes)
    int full_weno;          // FP64 form: evaluate every WENO6 in full (no collapse on node planes)
    double vertex_jitter;   // FP64 form, sensitivity studies: backtraced vertices moved by up to this many
    unsigned jitter_seed;   //   cells, independently per vertex and axis (a hash of vertex, axis and seed)
    double color_off[2];    // split method: colour = x/h - off0, z/h - off1
    int k;                  // Gauss points per half cell
    double gx[kMaxGauss];   // Gauss nodes on [-1,1] (centre first, then -/+ pairs)
    double gw[kMaxGauss];   // weights normalised to sum 1
    double minimal_area;    // xi-eta area above which pieces are triangulated
    double dt, h;
    // FP32 copies for the FP32 kernels, filled on the host by desc32(): on GB300 every
    // double-to-float conversion in a kernel runs on the (slow) FP64 pipe
    float gxf[kMaxGauss], gwf[kMaxGauss];
    float hf, invhf, dthf;  // h, 1/h, dt/h
    float color_off_f[2], minimal_area_f;
};

// PassDesc / NodeField with their FP32 copies filled (host)
NodeField field32(NodeField F);
PassDesc desc32(const PassDesc& d);

enum PsiMode : int { PSI_PLAIN = 0, PSI_WENO6 = 1, PSI_LINEAR = 2 };

// Status bits (OR-ed into the device status word).
enum StatusBits : unsigned {
    ST_CLIP_OVERFLOW = 1u,      // a piece exceeded 32 vertices or the clip pool
    ST_CLIP_ODD_CUT = 2u,       // odd number of iso-line crossings (facecutter.h:191-204)
    ST_NONFINITE = 4u,          // a non-finite flux was produced
    ST_SUBDIV_OVERFLOW = 8u,    // triangle subdivision stack exhausted
};

// Pieces of the FP32 face pipeline (clip -> per-piece quadrature -> per-face sum): the
// clipped pieces of every face of a pass, contiguous per face, and per face its range.
struct PieceStore {
    float4* rec = nullptr;       // (cx, cy, cz, ny): centroid in cells relative to the face anchor, y-normal
    int* face = nullptr;         // family << 29 | face index
    float* flux = nullptr;       // flux of each piece
    int2* range[3] = {nullptr, nullptr, nullptr};   // per face: start, nfwd | nrev << 15 | multi << 30
    float2* normal[3] = {nullptr, nullptr, nullptr};  // per face: y-normal sums of both clips (lower, upper cell)
    unsigned* count = nullptr;   // device counters: [0] pieces, [1] faces listed for the local-memory clipper
    int* deferred = nullptr;     // those faces (family << 29 | face index), room for every face
    float4* rest = nullptr;      // the pieces of a face at rest (same for every face of a family)
    unsigned long long* saved = nullptr;   // the session's work counters before a clip (restored on a retry)
    long long cap = 0;           // pieces the buffers hold
    int clip_fast = 1;           // 0: every face through the local-memory clipper
};
// (re)allocates the piece buffers for at least `pieces` pieces; ranges for `faces` per family
cudaError_t piece_store_reserve(PieceStore& p, long long pieces, long long faces_per_family);
void piece_store_free(PieceStore& p);

// Pieces of the plain form's face pipeline (clip -> per-piece quadrature -> per-face sum),
// as PieceStore: every face's pieces contiguous, in emission order, forward clip first.
struct PieceStore64 {
    double4_32a* rec = nullptr;      // (cx, cy, cz, ny): centroid (absolute), y component of the scaled normal
    double* flux = nullptr;      // flux of each piece
    int2* range[3] = {nullptr, nullptr, nullptr};   // per face: start, nfwd | nrev << 15 | multi << 30
    unsigned* count = nullptr;   // device counters: [0] pieces appended, [1] faces listed for whole-face evaluation
    int* deferred = nullptr;     // those faces (family << 29 | face index), room for every face
    unsigned long long* saved = nullptr;   // the session's work counters before a clip (restored on a retry)
    long long cap = 0;           // pieces the buffers hold
};
cudaError_t piece_store64_reserve(PieceStore64& p, long long pieces, long long faces_per_family);
void piece_store64_free(PieceStore64& p);

// Workspace owned by the caller (device pointers).
template <typename T>
struct PassWork {
    T* psi;            // P.Mx*P.My*P.Mz
    T* verts;          // 3 * (A.Mx+1)(A.My+1)(A.Mz+1)  backtraced vertex positions
    T* verts2 = nullptr;   // the same, traced back from verts (flux MacCormack only)
    T* fvol[3] = {nullptr, nullptr, nullptr};      // per face: sum of y n_y of its pieces (PassDesc::volumes)
    T* fvol_rev[3] = {nullptr, nullptr, nullptr};  // the same seen from the upper cell
    T* vol = nullptr;  // cells: the advected cell volumes (PassDesc::volumes)
    T* flux[3];        // per face family: (Mx+1)MyMz, Mx(My+1)Mz, MxMy(Mz+1); lower cell's view
    T* flux_rev[3];    // the same faces seen from the upper cell (its own clip when needed)
    unsigned* status;  // one word
    unsigned long long* counters;  // [0] faces, [1] pieces, [2] faces clipped twice, [3] WENO6 evaluations
    // optional timing of the face kernels: an event pair is recorded around each launch
    cudaEvent_t* prof_ev;   // 2 * prof_cap events, or null
    int* prof_n;            // pairs recorded so far
    int prof_cap;
    PieceStore* pieces = nullptr;   // FP32 form only
    PieceStore64* pieces64 = nullptr;   // FP64 form: the piece pipeline; null: one thread per face (k_faces)
};

// records the opening / closing event of a timed face-kernel launch
template <typename T>
inline void prof_mark(const PassWork<T>& w, int closing, cudaStream_t s) {
    if (!w.prof_ev || *w.prof_n >= w.prof_cap) return;
    cudaEventRecord(w.prof_ev[2 * *w.prof_n + closing], s);
    if (closing) ++*w.prof_n;
}

struct VelocityFields {
    const void* u; const void* v; const void* w;   // T* on the device
    NodeField fu, fv, fw;
};

void make_gauss(int k, double* x, double* w);
NodeField cell_field(const int* N, int comp);
NodeField psi_field(const NodeField& A);

// Launchers (one CUDA stream); all return cudaError_t of the launches.
template <typename T>
cudaError_t launch_psi(const PassDesc& d, const T* a, T* psi, cudaStream_t s);
template <typename T>
cudaError_t launch_backtrace(const PassDesc& d, const VelocityFields& vel, T* verts, cudaStream_t s);
template <typename T>
cudaError_t launch_faces(const PassDesc& d, const T* a, const PassWork<T>& w, cudaStream_t s);
// mode 0: out = div F / V; 1: out = in - div F / V; 2: out += div F / V; 3: out = div F (raw)
template <typename T>
cudaError_t launch_gather(const PassDesc& d, const PassWork<T>& w, const T* in, T* out, int mode, cudaStream_t s);

// One complete pass: psi, backtrace (unless zero velocity), faces, gather.
template <typename T>
cudaError_t run_pass(const PassDesc& d, const VelocityFields& vel, const T* a, const PassWork<T>& w,
                     const T* in, T* out, int mode, cudaStream_t s);

// The chosen form (fia_advect32.cu): FP32 in local cell coordinates; psi is stored as
// (hi, lo) float pairs in cell units, fluxes as (flux, y-normal sum) float pairs, vertex
// displacements in cells.
template <>
cudaError_t run_pass<float>(const PassDesc& d, const VelocityFields& vel, const float* a, const PassWork<float>& w,
                            const float* in, float* out, int mode, cudaStream_t s);
template <>
cudaError_t launch_psi<float>(const PassDesc& d, const float* a, float* psi, cudaStream_t s);
template <>
cudaError_t launch_backtrace<float>(const PassDesc& d, const VelocityFields& vel, float* verts, cudaStream_t s);

}  // namespace fia
