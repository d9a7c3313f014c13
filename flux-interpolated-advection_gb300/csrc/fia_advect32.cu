// fia_advect32.cu -- the chosen form of the flux pass: FP32 arithmetic in local cell
// coordinates, double-float psi, compensated face and cell sums.
//
// Same kernels as fia_advect.cu (psi column scan, unique-vertex backtrace, unique-face
// clip + quadrature + WENO6, deterministic gather), with these differences:
//  * all geometry is in cell units relative to an integer anchor (fia_local.cuh);
//  * psi is stored as (hi, lo) float pairs in the reference's units (density x length):
//    the WENO6 weights are not scale invariant (alpha = C / (1e-6 + beta)^2), so psi must
//    carry the same scale as in the reference for the same interpolant;
//  * a face interpolates psi - Psi0(f), Psi0(f) = the psi node at the face's anchor, and
//    stores (Ft, Ny): the compensated flux of psi - Psi0 plus the density terms, and the
//    sum of the pieces' scaled y-normals;
//  * the gather forms, per cell c with base node Psi_c,
//        rho' = sum_f s_f [ Ft(f) + (Psi0(f) - Psi_c) Ny(f) ],
//    which equals sum_f s_f F(f) - Psi_c sum_f s_f Ny(f); the last sum is the y-component
//    of the vector area of the closed surface of the backtraced cell, zero in exact
//    arithmetic, and is dropped so that no O(psi) term survives in FP32.
#include "fia_advect.cuh"
#include "fia_local.cuh"
#include "fia_clip32.cuh"

#include <algorithm>

namespace fia {

namespace {

// ---------------------------------------------------------------------------------
// psi as hi/lo pairs, one thread per (x,z) column
// ---------------------------------------------------------------------------------
__global__ void k_psi32(PassDesc d, const float* __restrict__ a, float2* __restrict__ psi) {
    const int Mx = d.A.Mx, My = d.A.My, Mz = d.A.Mz;
    const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (long long)Mx * Mz) return;
    const int i = (int)(col / Mz), k = (int)(col % Mz);
    const PlainLoad L{a};
    const float hf = d.hf;
    float hi = 0.f, lo = 0.f;
    psi[idx3(d.P, i, 0, k)] = make_float2(0.f, 0.f);
    const float oy = d.A.oyf;
    for (int j = 1; j <= My; ++j) {
        Kahan inc;
        if (d.psi_mode == PSI_PLAIN) {
            inc.add(__ldg(a + idx3(d.A, i, j - 1, k)) * hf);
        } else if (d.psi_mode == PSI_WENO6) {
            // cell j-1 spans [j-1+oy-.5, j+oy-.5] in cells; anchor (i, j-1, k)
            const int anc[3] = {i, j - 1, k};
            for (int half = 0; half < 2; ++half) {
                const float lo_y = (oy - 0.5f) + 0.5f * float(half);
                for (int q = 0; q < d.k; ++q) {
                    const float qq[3] = {d.A.oxf, lo_y + 0.25f * (1.0f + d.gxf[q]), d.A.ozf};
                    inc.add(weno6_1dy_loc(L, d.A, anc, qq) * (0.5f * hf) * d.gwf[q]);
                }
            }
        } else {
            const int anc[3] = {i, j - 1, k};
            const float q0[3] = {d.A.oxf, 0.25f + oy - 0.5f, d.A.ozf};
            const float q1[3] = {d.A.oxf, 0.75f + oy - 0.5f, d.A.ozf};
            inc.add(lin3d_loc(L, d.A, anc, q0) * (0.5f * hf));
            inc.add(lin3d_loc(L, d.A, anc, q1) * (0.5f * hf));
        }
        // (hi, lo) += inc
        float s, e;
        two_sum(hi, inc.s, s, e);
        e += lo + inc.c;
        two_sum(s, e, hi, lo);
        psi[idx3(d.P, i, j, k)] = make_float2(hi, lo);
    }
}

// ---------------------------------------------------------------------------------
// backtrace: displacement in cells of every unique vertex, clamped to the domain
// ---------------------------------------------------------------------------------
__global__ void k_backtrace32(PassDesc d, const float* __restrict__ u, const float* __restrict__ v,
                              const float* __restrict__ w, NodeField fu, NodeField fv, NodeField fw,
                              float* __restrict__ disp) {
    const int Lx = d.A.Mx + 1, Ly = d.A.My + 1, Lz = d.A.Mz + 1;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)Lx * Ly * Lz) return;
    const int k = (int)(id % Lz);
    const int j = (int)((id / Lz) % Ly);
    const int i = (int)(id / ((long long)Lz * Ly));
    const int anc[3] = {i, j, k};
    float q[3] = {0.f, 0.f, 0.f};
    if (d.comp >= 0) q[d.comp] = -0.5f;
    float dx[3] = {0.f, 0.f, 0.f};
    bool pinned = false;
    if (d.comp >= 0) {
        const int vi = anc[d.comp];
        pinned = (vi <= 1 || vi >= d.N[d.comp]);
    }
    if (!pinned) {
        // dt/h converts the velocity to cells per step; at the rest position WENO6 collapses
        // along the axes on which it lies on a node plane of the component's lattice
        const float s = d.dthf;
        if (d.interp == INTERP_WENO6) {
            dx[0] = -weno6_3d_collapse(PlainLoad{u}, fu, anc, q) * s;
            dx[1] = -weno6_3d_collapse(PlainLoad{v}, fv, anc, q) * s;
            dx[2] = -weno6_3d_collapse(PlainLoad{w}, fw, anc, q) * s;
        } else {
            dx[0] = -interp_loc(d.interp, PlainLoad{u}, fu, anc, q) * s;
            dx[1] = -interp_loc(d.interp, PlainLoad{v}, fv, anc, q) * s;
            dx[2] = -interp_loc(d.interp, PlainLoad{w}, fw, anc, q) * s;
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float e = (c == d.comp) ? 0.5f : 0.f;
        const float rest = float(anc[c]) + q[c];          // exact (small integers and halves)
        const float lo = -e, hi = float(d.N[c]) + e;
        if (rest + dx[c] < lo) dx[c] = lo - rest;
        if (rest + dx[c] > hi) dx[c] = hi - rest;
    }
    disp[3 * id + 0] = dx[0]; disp[3 * id + 1] = dx[1]; disp[3 * id + 2] = dx[2];
}

// Second trace of the flux MacCormack scheme: from the backtraced position (rest + disp),
// disp2 = disp + dt/h u(rest + disp), the pin rule and clamp of k_backtrace32
// (calc_backtraced_face_3D.cpp:9-160, time direction "backward").
__global__ void k_forward32(PassDesc d, const float* __restrict__ u, const float* __restrict__ v,
                            const float* __restrict__ w, NodeField fu, NodeField fv, NodeField fw,
                            const float* __restrict__ disp, float* __restrict__ disp2) {
    const int Lx = d.A.Mx + 1, Ly = d.A.My + 1, Lz = d.A.Mz + 1;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)Lx * Ly * Lz) return;
    const int k = (int)(id % Lz);
    const int j = (int)((id / Lz) % Ly);
    const int i = (int)(id / ((long long)Lz * Ly));
    const int anc[3] = {i, j, k};
    float q0[3] = {0.f, 0.f, 0.f};
    if (d.comp >= 0) q0[d.comp] = -0.5f;
    float dx[3] = {disp[3 * id], disp[3 * id + 1], disp[3 * id + 2]};
    bool pinned = false;
    if (d.comp >= 0) {
        const int vi = anc[d.comp];
        pinned = (vi <= 1 || vi >= d.N[d.comp]);
    }
    if (!pinned) {
        const float q[3] = {q0[0] + dx[0], q0[1] + dx[1], q0[2] + dx[2]};
        const float s = d.dthf;
        const float v0 = interp_loc(d.interp, PlainLoad{u}, fu, anc, q);
        const float v1 = interp_loc(d.interp, PlainLoad{v}, fv, anc, q);
        const float v2 = interp_loc(d.interp, PlainLoad{w}, fw, anc, q);
        dx[0] += v0 * s; dx[1] += v1 * s; dx[2] += v2 * s;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float e = (c == d.comp) ? 0.5f : 0.f;
        const float rest = float(anc[c]) + q0[c];
        const float lo = -e, hi = float(d.N[c]) + e;
        if (rest + dx[c] < lo) dx[c] = lo - rest;
        if (rest + dx[c] > hi) dx[c] = hi - rest;
    }
    disp2[3 * id + 0] = dx[0]; disp2[3 * id + 1] = dx[1]; disp2[3 * id + 2] = dx[2];
}

// ---------------------------------------------------------------------------------
// faces
// ---------------------------------------------------------------------------------
// The quadrature of one piece (polygon_3D.cpp:257-487): density points on the y-interval
// below the centroid and one psi point; returns the number of 1D WENO6 evaluations.
constexpr int kQuadThreads = 128;

__device__ int piece_quad32(const PassDesc& d, const int* anc, float cx, float cy, float cz, float ny,
                            const float* __restrict__ a, const PsiLoad& pl, Kahan& F, float* zs) {
    const PlainLoad al{a};
    const float invh = d.invhf;   // psi carries a length; the face terms are per cell volume
    int evals = 0;
    if (d.use_integral) {
        const float oy = (d.comp == 1) ? -0.5f : 0.f;
        const float r = snap_int(cy - oy);
        const float fl = floorf(r);
        const float f = r - fl;
        const float ylo = fl + oy;   // local y of the y-face below the centroid
        // the density quadrature points (polygon_3D.cpp:286-453): k on [ylo, cy] when the
        // centroid is in the lower half of the cell, else k on each of [ylo, ylo+1/2], [ylo+1/2, cy];
        // point m is generated on demand (no per-thread arrays)
        const bool two = !(f < 0.5f);
        const float lo0 = ylo, hl0 = two ? 0.25f : (cy - ylo) * 0.5f, wf0 = two ? ny * 0.5f : ny * f;
        const float lo1 = ylo + 0.5f, hl1 = (cy - lo1) * 0.5f, wf1 = ny * (f - 0.5f);
        const int k = d.k, np = two ? 2 * k : k;
        auto point = [&](int m, float& y, float& w) {
            const bool second = m >= k;
            const int q = second ? m - k : m;
            const float hl = second ? hl1 : hl0;
            y = hl * d.gxf[q] + hl + (second ? lo1 : lo0);
            w = (second ? wf1 : wf0) * d.gwf[q];
        };
        bool shared = false;
        if (d.interp == INTERP_WENO6) {
            const int n1d = weno6_ycolumn<kQuadThreads>(al, d.A, anc, cx, cz, ylo, cy, np, point, F, zs);
            shared = n1d > 0;
            evals += n1d;          // 1D WENO6 evaluations executed
        }
        if (!shared) {
            for (int m = 0; m < np; ++m) {
                float y, w;
                point(m, y, w);
                const float qq[3] = {cx, y, cz};
                F.add(interp_loc(d.interp, al, d.A, anc, qq) * w);
            }
            if (d.interp == INTERP_WENO6) evals += 43 * np;
        }
        // the psi point lies on the psi node row of the y-face below the centroid
        const float qp[3] = {cx, ylo, cz};
        float v;
        const int n1d = d.interp == INTERP_WENO6 ? weno6_3d_noderow<kQuadThreads>(pl, d.P, anc, qp, v, zs) : 0;
        if (n1d == 0) {
            v = interp_loc(d.interp, pl, d.P, anc, qp);
            if (d.interp == INTERP_WENO6) evals += 43;
        }
        evals += n1d;
        F.add(v * (ny * invh));
    } else {
        // psi at the centroid; on an unmoved y-face (the zero-velocity pass) the centroid lies
        // on a psi node row
        const float qp[3] = {cx, cy, cz};
        float v;
        const int n1d = d.interp == INTERP_WENO6 ? weno6_3d_noderow<kQuadThreads>(pl, d.P, anc, qp, v, zs) : 0;
        if (n1d == 0) {
            v = interp_loc(d.interp, pl, d.P, anc, qp);
            if (d.interp == INTERP_WENO6) evals += 43;
        }
        evals += n1d;
        F.add(v * (ny * invh));
    }
    return evals;
}

__device__ __forceinline__ void corners(int fam, int i, int j, int k, int* ci, int* cj, int* ck) {
    if (fam == 0) {
        ci[0] = i; cj[0] = j; ck[0] = k;   ci[1] = i; cj[1] = j + 1; ck[1] = k;
        ci[2] = i; cj[2] = j + 1; ck[2] = k + 1;   ci[3] = i; cj[3] = j; ck[3] = k + 1;
    } else if (fam == 1) {
        ci[0] = i; cj[0] = j; ck[0] = k;   ci[1] = i; cj[1] = j; ck[1] = k + 1;
        ci[2] = i + 1; cj[2] = j; ck[2] = k + 1;   ci[3] = i + 1; cj[3] = j; ck[3] = k;
    } else {
        ci[0] = i; cj[0] = j; ck[0] = k;   ci[1] = i + 1; cj[1] = j; ck[1] = k;
        ci[2] = i + 1; cj[2] = j + 1; ck[2] = k;   ci[3] = i; cj[3] = j + 1; ck[3] = k;
    }
}

// psi base node of a face / cell anchored at (i,j,k), clamped into the psi array
__device__ __forceinline__ long long psi_node(const NodeField& P, int i, int j, int k) {
    return idx3(P, clampi(i, P.Mx - 1), clampi(j, P.My - 1), clampi(k, P.Mz - 1));
}

// a family's arrays of the store, selected without indexing the kernel parameter (an indexed
// parameter array is copied to the stack frame)
__device__ __forceinline__ int2* range_of(const PieceStore& ps, int fam) {
    return fam == 0 ? ps.range[0] : (fam == 1 ? ps.range[1] : ps.range[2]);
}
__device__ __forceinline__ float2* normal_of(const PieceStore& ps, int fam) {
    return fam == 0 ? ps.normal[0] : (fam == 1 ? ps.normal[1] : ps.normal[2]);
}

// Face pipeline of the chosen form, per pass:
//  k_clip32     one thread per unique face: backtraced corners, clip in shared memory (twice
//               when an iso-line crosses a piece more than twice), pieces appended
//               contiguously per face (warp prefix sum + one atomic per warp), y-normal sums;
//               a face the shared pool cannot hold goes to a list
//  k_clip32_deferred  the listed faces, clipped in local memory, appended the same way
//  k_quad32     one thread per piece: quadrature + WENO6 (uniform work per thread, no clip
//               code, so fewer registers and no divergence from the piece count);
//  k_facesum32  one thread per face: compensated sum of its pieces in emission order.
__device__ __forceinline__ void face_of(int fam, const NodeField& A, long long id, int& i, int& j, int& k) {
    const int Fy = A.My + (fam == 1), Fz = A.Mz + (fam == 2);
    k = (int)(id % Fz);
    j = (int)((id / Fz) % Fy);
    i = (int)(id / ((long long)Fz * Fy));
}

// face_of for the tags of the piece store (face ids below 2^29): two 32-bit divisions
__device__ __forceinline__ void face_of32(int fam, const NodeField& A, unsigned id, int& i, int& j, int& k) {
    const unsigned Fy = A.My + (fam == 1), Fz = A.Mz + (fam == 2);
    const unsigned t = id / Fz;
    k = (int)(id - t * Fz);
    const unsigned ii = t / Fy;
    i = (int)ii;
    j = (int)(t - ii * Fy);
}

// corners of face id of family fam, in cells relative to its anchor, backtraced by disp
__device__ __forceinline__ void face_geometry(const PassDesc& d, int fam, long long id, const float* __restrict__ disp,
                                              LocalFace& g) {
    int i, j, k;
    face_of(fam, d.A, id, i, j, k);
    int ci[4], cj[4], ck[4];
    corners(fam, i, j, k, ci, cj, ck);
    g.anc[0] = i; g.anc[1] = j; g.anc[2] = k;
    const int Ly = d.A.My + 1, Lz = d.A.Mz + 1;
    const float sx = d.comp == 0 ? -0.5f : 0.f, sy = d.comp == 1 ? -0.5f : 0.f, sz = d.comp == 2 ? -0.5f : 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float dx = 0.f, dy = 0.f, dz = 0.f;
        if (!d.zero_velocity) {
            const long long vid = ((long long)ci[q] * Ly + cj[q]) * Lz + ck[q];
            dx = disp[3 * vid]; dy = disp[3 * vid + 1]; dz = disp[3 * vid + 2];
        }
        g.x[q] = float(ci[q] - i) + sx + dx;
        g.y[q] = float(cj[q] - j) + sy + dy;
        g.z[q] = float(ck[q] - k) + sz + dz;
    }
}

__device__ __forceinline__ void warp_counters(unsigned long long pc, unsigned fc, unsigned mc, unsigned st, int lane,
                                              unsigned* status, unsigned long long* counters) {
    for (int o = 16; o > 0; o >>= 1) {
        pc += __shfl_down_sync(0xffffffffu, pc, o);
        fc += __shfl_down_sync(0xffffffffu, fc, o);
        mc += __shfl_down_sync(0xffffffffu, mc, o);
        st |= __shfl_down_sync(0xffffffffu, st, o);
    }
    if (lane == 0) {
        if (fc) { atomicAdd(&counters[0], (unsigned long long)fc); atomicAdd(&counters[1], pc); }
        if (mc) atomicAdd(&counters[2], (unsigned long long)mc);
        if (st) atomicOr(status, st);
    }
}

// fast = 0 sends every face to the list (the local-memory clipper alone)
__global__ void __launch_bounds__(kClipThreads, 4) k_clip32(PassDesc d, int fam, const float* __restrict__ disp,
                                                            PieceStore ps, unsigned* status,
                                                            unsigned long long* counters, int fast) {
    extern __shared__ float clip_smem[];
    const FastPool P{clip_smem + threadIdx.x};
    const int Fx = d.A.Mx + (fam == 0), Fy = d.A.My + (fam == 1), Fz = d.A.Mz + (fam == 2);
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nface = (long long)Fx * Fy * Fz;
    const int lane = threadIdx.x & 31;
    int npieces = 0, nst = 0, nfwd = 0;
    bool multi = false, ok = false;
    if (id < nface) {
        LocalFace g;
        face_geometry(d, fam, id, disp, g);
        Kahan ny;
        ok = fast != 0 && clip32_fast(d, g, npieces, multi, nst, ny, P);
        float N = 0.f, Nr = 0.f;
        if (ok) {
            nfwd = nst;
            N = ny.value();
            Nr = -N;
            if (multi) {
                ny = Kahan();
                int np2 = 0;
                bool m2 = false;
                ok = clip32_fast(d, reversed_face(g), np2, m2, nst, ny, P);
                Nr = ny.value();
            }
        }
        if (ok) {
            normal_of(ps, fam)[id] = make_float2(N, Nr);
        } else {
            const unsigned q = atomicAdd(ps.count + 1, 1u);
            ps.deferred[q] = (fam << 29) | (int)id;
            npieces = 0; nst = 0; multi = false;
        }
    }
    const int cnt = nst;
    const long long start = warp_slots(ps.count, cnt, lane);
    if (ok) {
        if (start + cnt <= ps.cap) {
            const int tag = (fam << 29) | (int)id;
            for (int q = 0; q < cnt; ++q) {
                const int e = kFastR - 1 - q;
                ps.rec[start + q] = make_float4(P.at(e, 0), P.at(e, 1), P.at(e, 2), P.at(e, 3));
                ps.face[start + q] = tag;
            }
        }
        // a range beyond the capacity is kept as it is: the host sees the count, grows the
        // store and runs the pass again
        range_of(ps, fam)[id] = make_int2((int)start, nfwd | ((cnt - nfwd) << 15) | ((multi ? 1 : 0) << 30));
    }
    warp_counters((unsigned long long)npieces, ok ? 1u : 0u, (ok && multi) ? 1u : 0u, 0u, lane, status, counters);
}

// The faces k_clip32 listed (all families), clipped by clip32 in local memory; grid-stride
// over the list length the clip kernels left in ps.count[1].
__global__ void __launch_bounds__(128) k_clip32_deferred(PassDesc d, const float* __restrict__ disp, PieceStore ps,
                                                         unsigned* status, unsigned long long* counters) {
    const long long nd = (long long)ps.count[1];
    const int lane = threadIdx.x & 31;
    if (blockIdx.x == 0 && threadIdx.x == 0 && nd > 0) atomicAdd(&counters[4], (unsigned long long)nd);
    for (long long base = (long long)blockIdx.x * blockDim.x; base < nd; base += (long long)gridDim.x * blockDim.x) {
        const long long t = base + threadIdx.x;
        const bool valid = t < nd;
        const int tag = valid ? ps.deferred[t] : 0;
        const int fam = tag >> 29;
        const long long id = tag & ((1 << 29) - 1);
        unsigned st = 0;
        int npieces = 0, nmulti = 0, nfwd = 0;
        bool multi = false;
        PieceSink sink;
        if (valid) {
            LocalFace g;
            face_geometry(d, fam, id, disp, g);
            clip32(d, g, st, npieces, multi, sink);
            nfwd = sink.n;
            const float N = sink.ny.value();
            float Nr = -N;
            if (multi) {
                int np2 = 0;
                bool m2 = false;
                sink.ny = Kahan();
                clip32(d, reversed_face(g), st, np2, m2, sink);
                Nr = sink.ny.value();
                ++nmulti;
            }
            normal_of(ps, fam)[id] = make_float2(N, Nr);
        }
        const int cnt = sink.n;
        const long long start = warp_slots(ps.count, cnt, lane);
        if (valid) {
            if (start + cnt <= ps.cap)
                for (int q = 0; q < cnt; ++q) { ps.rec[start + q] = sink.p[q]; ps.face[start + q] = tag; }
            range_of(ps, fam)[id] = make_int2((int)start, nfwd | ((cnt - nfwd) << 15) | ((multi ? 1 : 0) << 30));
        }
        warp_counters((unsigned long long)npieces, valid ? 1u : 0u, (unsigned)nmulti, st, lane, status, counters);
    }
}

// Faces at rest (the zero-velocity pass, the MacCormack face at rest) are the same square in
// every face's local coordinates, so they all have the same pieces: k_rest_clip32 clips one
// with clip32 (one thread) into ps.rest -- [0] (count, range bits, pieces with area, status)
// as ints, [1] (N, Nr), [2..] the pieces -- and k_rest_fill32 gives every face of the family a
// copy, face-major (face id's pieces at id * count): the pieces, order and sums of a clip per
// face.  Only y-faces emit pieces at rest.
__global__ void k_rest_clip32(PassDesc d, int fam, PieceStore ps) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    LocalFace g;
    face_geometry(d, fam, 0, nullptr, g);
    unsigned st = 0;
    int npieces = 0;
    bool multi = false;
    PieceSink sink;
    clip32(d, g, st, npieces, multi, sink);
    const int nfwd = sink.n;
    const float N = sink.ny.value();
    float Nr = -N;
    if (multi) {
        int np2 = 0;
        bool m2 = false;
        sink.ny = Kahan();
        clip32(d, reversed_face(g), st, np2, m2, sink);
        Nr = sink.ny.value();
    }
    reinterpret_cast<int4*>(ps.rest)[0] =
        make_int4(sink.n, nfwd | ((sink.n - nfwd) << 15) | ((multi ? 1 : 0) << 30), npieces, (int)st);
    ps.rest[1] = make_float4(N, Nr, 0.f, 0.f);
    for (int q = 0; q < sink.n; ++q) ps.rest[2 + q] = sink.p[q];
}

__global__ void k_rest_fill32(PassDesc d, int fam, PieceStore ps, unsigned* status, unsigned long long* counters) {
    const long long nface = (long long)(d.A.Mx + (fam == 0)) * (d.A.My + (fam == 1)) * (d.A.Mz + (fam == 2));
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int4 hd = reinterpret_cast<const int4*>(ps.rest)[0];
    const int cnt = hd.x;
    if (id == 0) {
        atomicAdd(ps.count, (unsigned)(cnt * nface));
        atomicAdd(&counters[0], (unsigned long long)nface);
        atomicAdd(&counters[1], (unsigned long long)hd.z * (unsigned long long)nface);
        if ((hd.y >> 30) & 1) atomicAdd(&counters[2], (unsigned long long)nface);
        if (hd.w) atomicOr(status, (unsigned)hd.w);
    }
    if (id >= nface) return;
    const long long start = id * cnt;
    if (start + cnt <= ps.cap) {
        const int tag = (fam << 29) | (int)id;
        for (int q = 0; q < cnt; ++q) { ps.rec[start + q] = ps.rest[2 + q]; ps.face[start + q] = tag; }
    }
    range_of(ps, fam)[id] = make_int2((int)start, hd.y);
    const float4 nr = ps.rest[1];
    normal_of(ps, fam)[id] = make_float2(nr.x, nr.y);
}

__global__ void __launch_bounds__(kQuadThreads, 4) k_quad32(PassDesc d, const float* __restrict__ a,
                                                         const float2* __restrict__ psi, PieceStore ps, long long npc,
                                                         unsigned long long* counters) {
    __shared__ float zcol[48 * kQuadThreads];   // each thread's z- and y-pass column (weno6_ycolumn)
    unsigned long long ec = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npc; t += (long long)gridDim.x * blockDim.x) {
        const float4 p = ps.rec[t];
        const int tag = ps.face[t];
        const int fam = tag >> 29;
        int anc[3];
        face_of32(fam, d.A, (unsigned)(tag & ((1 << 29) - 1)), anc[0], anc[1], anc[2]);
        const float2 b = __ldg(psi + psi_node(d.P, anc[0], anc[1], anc[2]));
        const PsiLoad pl{psi, b.x, b.y};
        Kahan F;
        ec += (unsigned long long)piece_quad32(d, anc, p.x, p.y, p.z, p.w, a, pl, F, zcol + threadIdx.x);
        ps.flux[t] = F.value();
    }
    for (int o = 16; o > 0; o >>= 1) ec += __shfl_down_sync(0xffffffffu, ec, o);
    if ((threadIdx.x & 31) == 0 && ec) atomicAdd(&counters[3], ec);
}

// flux = wgt (F, N) (acc = 0) or flux + wgt (F, N) (acc = 1): the weighted faces of the flux
// MacCormack scheme accumulate into one (flux, y-normal sum) pair per face
// With fvol: (M, Mr) = sums of y n_y of the face's pieces in cells (y relative to the face
// anchor), the same weighting, for the cell volumes of the cell-volume correction.
__global__ void k_facesum32(PassDesc d, int fam, PieceStore ps, float2* __restrict__ flux, float2* __restrict__ flux_rev,
                            unsigned* status, float wgt, int acc, float2* __restrict__ fvol) {
    const long long nface = (long long)(d.A.Mx + (fam == 0)) * (d.A.My + (fam == 1)) * (d.A.Mz + (fam == 2));
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nface) return;
    const int2 r = range_of(ps, fam)[id];
    const int nf = r.y & 0x7fff, nr = (r.y >> 15) & 0x7fff;
    const bool multi = (r.y >> 30) & 1;
    Kahan F, Fr;
    for (int q = 0; q < nf; ++q) F.add(ps.flux[(long long)r.x + q]);
    for (int q = 0; q < nr; ++q) Fr.add(ps.flux[(long long)r.x + nf + q]);
    const float f = F.value(), fr = multi ? Fr.value() : -f;
    const float2 nrm = normal_of(ps, fam)[id];
    float2 a = make_float2(wgt * f, wgt * nrm.x), b = make_float2(wgt * fr, wgt * nrm.y);
    if (acc) {
        const float2 a0 = flux[id], b0 = flux_rev[id];
        a.x += a0.x; a.y += a0.y; b.x += b0.x; b.y += b0.y;
    }
    flux[id] = a;
    flux_rev[id] = b;
    if (!isfinite(f) || !isfinite(fr)) atomicOr(status, (unsigned)ST_NONFINITE);
    if (fvol) {
        Kahan M, Mr;
        for (int q = 0; q < nf; ++q) { const float4 p = ps.rec[(long long)r.x + q]; M.add(p.y * p.w); }
        for (int q = 0; q < nr; ++q) { const float4 p = ps.rec[(long long)r.x + nf + q]; Mr.add(p.y * p.w); }
        const float m = M.value(), mr = multi ? Mr.value() : -m;
        float2 v = make_float2(wgt * m, wgt * mr);
        if (acc) { const float2 v0 = fvol[id]; v.x += v0.x; v.y += v0.y; }
        fvol[id] = v;
    }
}

// Advected cell volumes in cells (cell-volume correction, density only): the volume points
// y n_y of a cell's pieces, from the per-face sums with y relative to each face's anchor.  The
// faces of cell (i, j, k) are anchored at row j except its upper y-face (row j + 1), which
// adds its y-normal sum; the term j sum_f s_f N_f of the common row is zero for a closed
// surface and is dropped (in FP32 it would only carry rounding).
__global__ void k_volume_gather32(PassDesc d, const float2* __restrict__ vx, const float2* __restrict__ vy,
                                  const float2* __restrict__ vz, const float2* __restrict__ fy, float* __restrict__ vol) {
    const int Mx = d.A.Mx, My = d.A.My, Mz = d.A.Mz;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)Mx * My * Mz) return;
    const int k = (int)(id % Mz);
    const int j = (int)((id / Mz) % My);
    const int i = (int)(id / ((long long)Mz * My));
    Kahan s;
    s.add(vx[((long long)(i + 1) * My + j) * Mz + k].x);
    s.add(vx[((long long)i * My + j) * Mz + k].y);
    s.add(vy[((long long)i * (My + 1) + j + 1) * Mz + k].x);
    s.add(vy[((long long)i * (My + 1) + j) * Mz + k].y);
    s.add(vz[((long long)i * My + j) * (Mz + 1) + k + 1].x);
    s.add(vz[((long long)i * My + j) * (Mz + 1) + k].y);
    s.add(fy[((long long)i * (My + 1) + j + 1) * Mz + k].y);
    vol[id] = s.value();
}

// rho'(c) = sum_f s_f [Ft + (Psi0(f) - Psi_c) Ny], compensated
__global__ void k_gather32(PassDesc d, const float2* __restrict__ fx, const float2* __restrict__ fy,
                           const float2* __restrict__ fz, const float2* __restrict__ rx,
                           const float2* __restrict__ ry, const float2* __restrict__ rz,
                           const float2* __restrict__ psi, const float* __restrict__ in, float* __restrict__ out,
                           int mode) {
    const int Mx = d.A.Mx, My = d.A.My, Mz = d.A.Mz;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)Mx * My * Mz) return;
    const int k = (int)(id % Mz);
    const int j = (int)((id / Mz) % My);
    const int i = (int)(id / ((long long)Mz * My));
    const float2 pc = __ldg(psi + psi_node(d.P, i, j, k));
    const float invh = d.invhf;
    auto base_diff = [&](int a, int b, int c) {
        const float2 p = __ldg(psi + psi_node(d.P, a, b, c));
        return ((p.x - pc.x) + (p.y - pc.y)) * invh;
    };
    // lower faces (anchor = the cell itself): base difference 0
    const float2 lx = rx[((long long)i * My + j) * Mz + k];
    const float2 ly = ry[((long long)i * (My + 1) + j) * Mz + k];
    const float2 lz = rz[((long long)i * My + j) * (Mz + 1) + k];
    const float2 ux = fx[((long long)(i + 1) * My + j) * Mz + k];
    const float2 uy = fy[((long long)i * (My + 1) + j + 1) * Mz + k];
    const float2 uz = fz[((long long)i * My + j) * (Mz + 1) + k + 1];
    Kahan s;
    s.add(lx.x); s.add(ly.x); s.add(lz.x);
    s.add(ux.x); s.add(uy.x); s.add(uz.x);
    s.add(base_diff(i + 1, j, k) * ux.y);
    s.add(base_diff(i, j + 1, k) * uy.y);
    s.add(base_diff(i, j, k + 1) * uz.y);
    const float val = s.value();
    if (mode == 0) out[id] = val;
    else if (mode == 1) out[id] = in[id] - val;
    else out[id] = out[id] + val;
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// One face stage of the FP32 pipeline: clip (growing the piece store and clipping again when
// it is too small), per-piece quadrature, per-face sums weighted into the face fluxes.
static cudaError_t face_stage32(const PassDesc& d, const float* a, const float2* psi, const float* disp,
                                const PassWork<float>& w, float wgt, int acc, cudaStream_t s) {
    PieceStore& ps = *w.pieces;
    long long nface[3];
    for (int fam = 0; fam < 3; ++fam)
        nface[fam] = (long long)(d.A.Mx + (fam == 0)) * (d.A.My + (fam == 1)) * (d.A.Mz + (fam == 2));
    if (std::max(nface[0], std::max(nface[1], nface[2])) >= (1LL << 29)) return cudaErrorInvalidValue;
    // Faces at rest (the zero-velocity pass, the MacCormack face at rest): an x- or z-face keeps
    // its four corners at one x (z), so every piece's y-normal is exactly zero and the face
    // emits no piece; its flux, normal and volume sums are zero and only the y-faces are clipped.
    const bool rest = d.zero_velocity != 0;
    if (rest && !acc) {
        for (int fam = 0; fam < 3; fam += 2) {
            cudaMemsetAsync(w.flux[fam], 0, nface[fam] * sizeof(float2), s);
            cudaMemsetAsync(w.flux_rev[fam], 0, nface[fam] * sizeof(float2), s);
            if (d.volumes) cudaMemsetAsync(w.fvol[fam], 0, nface[fam] * sizeof(float2), s);
        }
    }
    unsigned npc = 0;
    cudaError_t ea = cudaFuncSetAttribute(k_clip32, cudaFuncAttributeMaxDynamicSharedMemorySize, kClipSmem);
    if (ea == cudaSuccess)
        ea = cudaFuncSetAttribute(k_clip32, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (ea != cudaSuccess) return ea;
    // the work counters as they were before the clip: a second attempt starts from them again
    ea = cudaMemcpyAsync(ps.saved, w.counters, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s);
    if (ea != cudaSuccess) return ea;
    for (int attempt = 0; attempt < 2; ++attempt) {
        cudaMemsetAsync(ps.count, 0, 2 * sizeof(unsigned), s);
        if (attempt > 0)
            cudaMemcpyAsync(w.counters, ps.saved, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s);
        if (rest && ps.clip_fast) {
            k_rest_clip32<<<1, 32, 0, s>>>(d, 1, ps);
            k_rest_fill32<<<nblk(nface[1], 256), 256, 0, s>>>(d, 1, ps, w.status, w.counters);
        } else {
            for (int fam = 0; fam < 3; ++fam)
                if (!rest || fam == 1)
                    k_clip32<<<nblk(nface[fam], kClipThreads), kClipThreads, kClipSmem, s>>>(d, fam, disp, ps, w.status,
                                                                                             w.counters, ps.clip_fast);
            k_clip32_deferred<<<152 * 8, 128, 0, s>>>(d, disp, ps, w.status, w.counters);
        }
        cudaError_t e = cudaMemcpyAsync(&npc, ps.count, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        if ((long long)npc <= ps.cap) break;
        // more pieces than the store holds: grow it and clip again
        e = piece_store_reserve(ps, (long long)npc + npc / 4 + 1024, std::max(nface[0], std::max(nface[1], nface[2])));
        if (e != cudaSuccess) return e;
    }
    if ((long long)npc > ps.cap) return cudaErrorMemoryAllocation;
    if (npc > 0) {
        prof_mark(w, 0, s);
        k_quad32<<<152 * 8, kQuadThreads, 0, s>>>(d, a, psi, ps, (long long)npc, w.counters);
        prof_mark(w, 1, s);
    }
    for (int fam = 0; fam < 3; ++fam)
        if (!rest || fam == 1)
            k_facesum32<<<nblk(nface[fam], 256), 256, 0, s>>>(d, fam, ps, (float2*)w.flux[fam], (float2*)w.flux_rev[fam],
                                                              w.status, wgt, acc,
                                                              d.volumes ? (float2*)w.fvol[fam] : nullptr);
    return cudaGetLastError();
}

template <>
cudaError_t run_pass<float>(const PassDesc& d64, const VelocityFields& vel64, const float* a, const PassWork<float>& w,
                            const float* in, float* out, int mode, cudaStream_t s) {
    const PassDesc d = desc32(d64);
    VelocityFields vel = vel64;
    vel.fu = field32(vel64.fu); vel.fv = field32(vel64.fv); vel.fw = field32(vel64.fw);
    float2* psi = (float2*)w.psi;
    const long long cols = (long long)d.A.Mx * d.A.Mz;
    k_psi32<<<nblk(cols, 128), 128, 0, s>>>(d, a, psi);
    const long long nv = (long long)(d.A.Mx + 1) * (d.A.My + 1) * (d.A.Mz + 1);
    if (!d.zero_velocity)
        k_backtrace32<<<nblk(nv, 128), 128, 0, s>>>(d, (const float*)vel.u, (const float*)vel.v, (const float*)vel.w,
                                                   vel.fu, vel.fv, vel.fw, w.verts);
    cudaError_t e;
    if (!d.maccormack || d.zero_velocity) {
        // one face per face slot; with zero velocity the MacCormack faces coincide and their
        // weights sum to one
        e = face_stage32(d, a, psi, w.verts, w, 1.f, 0, s);
    } else {
        if (!w.verts2) return cudaErrorInvalidValue;
        k_forward32<<<nblk(nv, 128), 128, 0, s>>>(d, (const float*)vel.u, (const float*)vel.v, (const float*)vel.w,
                                                 vel.fu, vel.fv, vel.fw, w.verts, w.verts2);
        PassDesc rest = d;
        rest.zero_velocity = 1;
        e = face_stage32(rest, a, psi, w.verts, w, 0.5f, 0, s);                       // the face at rest
        if (e == cudaSuccess) e = face_stage32(d, a, psi, w.verts, w, 1.f, 1, s);     // backtraced
        if (e == cudaSuccess) e = face_stage32(d, a, psi, w.verts2, w, -0.5f, 1, s);  // traced back
    }
    if (e != cudaSuccess) return e;
    const long long nc = (long long)d.A.Mx * d.A.My * d.A.Mz;
    if (d.volumes) {
        if (!w.vol || !w.fvol[0] || d.comp >= 0) return cudaErrorInvalidValue;
        k_volume_gather32<<<nblk(nc, 256), 256, 0, s>>>(d, (const float2*)w.fvol[0], (const float2*)w.fvol[1],
                                                        (const float2*)w.fvol[2], (const float2*)w.flux[1], w.vol);
    }
    k_gather32<<<nblk(nc, 256), 256, 0, s>>>(d, (const float2*)w.flux[0], (const float2*)w.flux[1],
                                             (const float2*)w.flux[2], (const float2*)w.flux_rev[0],
                                             (const float2*)w.flux_rev[1], (const float2*)w.flux_rev[2], psi, in, out,
                                             mode);
    return cudaGetLastError();
}

cudaError_t piece_store_reserve(PieceStore& p, long long pieces, long long faces_per_family) {
    cudaDeviceSynchronize();
    if (pieces > p.cap) {
        cudaFree(p.rec); cudaFree(p.face); cudaFree(p.flux);
        p.rec = nullptr; p.face = nullptr; p.flux = nullptr; p.cap = 0;
        cudaError_t e = cudaMalloc(&p.rec, pieces * sizeof(float4));
        if (e == cudaSuccess) e = cudaMalloc(&p.face, pieces * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc(&p.flux, pieces * sizeof(float));
        if (e != cudaSuccess) return e;
        p.cap = pieces;
    }
    if (!p.count) {
        cudaError_t e = cudaMalloc(&p.count, 2 * sizeof(unsigned));
        if (e == cudaSuccess) e = cudaMalloc(&p.saved, 5 * sizeof(unsigned long long));
        if (e != cudaSuccess) return e;
    }
    if (!p.range[0]) {
        for (int f = 0; f < 3; ++f) {
            cudaError_t e = cudaMalloc(&p.range[f], faces_per_family * sizeof(int2));
            if (e == cudaSuccess) e = cudaMalloc(&p.normal[f], faces_per_family * sizeof(float2));
            if (e != cudaSuccess) return e;
        }
        cudaError_t e = cudaMalloc(&p.deferred, 3 * faces_per_family * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc(&p.rest, (2 + kMaxPieces32) * sizeof(float4));
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void piece_store_free(PieceStore& p) {
    cudaFree(p.rec); cudaFree(p.face); cudaFree(p.flux); cudaFree(p.count); cudaFree(p.deferred); cudaFree(p.rest);
    cudaFree(p.saved);
    for (int f = 0; f < 3; ++f) { cudaFree(p.range[f]); cudaFree(p.normal[f]); }
    p = PieceStore();
}

template <>
cudaError_t launch_psi<float>(const PassDesc& d64, const float* a, float* psi, cudaStream_t s) {
    const PassDesc d = desc32(d64);
    const long long cols = (long long)d.A.Mx * d.A.Mz;
    k_psi32<<<nblk(cols, 128), 128, 0, s>>>(d, a, (float2*)psi);
    return cudaGetLastError();
}

template <>
cudaError_t launch_backtrace<float>(const PassDesc& d64, const VelocityFields& vel, float* verts, cudaStream_t s) {
    const PassDesc d = desc32(d64);
    const long long nv = (long long)(d.A.Mx + 1) * (d.A.My + 1) * (d.A.Mz + 1);
    k_backtrace32<<<nblk(nv, 128), 128, 0, s>>>(d, (const float*)vel.u, (const float*)vel.v, (const float*)vel.w,
                                               field32(vel.fu), field32(vel.fv), field32(vel.fw), verts);
    return cudaGetLastError();
}

}  // namespace fia
