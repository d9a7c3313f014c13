// fia_clip32.cuh -- the FP32 face clipper: the reference's facecutter (facecutter.h:59-224)
// on a face's local colours, producing its pieces (centroid, scaled y-normal) in emission
// order.  Two stores for its polygons: clip32 keeps them in per-thread arrays (local memory),
// clip32_fast in a slice of the CTA's shared memory.  Host and device code: the face kernels
// in fia_advect32.cu run it on the GPU, tests/clip_host_check.cu compares the two stores on
// the host.
#pragma once
#include "fia_advect.cuh"
#include "fia_local.cuh"

#include <cstdio>
#include <cstdlib>

namespace fia {

struct CVf { float p0, p1, c0, c1; };
__host__ __device__ __forceinline__ float cvc(const CVf& v, int dim) { return dim ? v.c1 : v.c0; }

__host__ __device__ __forceinline__ float bilinf(const float* v, float xi, float eta) {
    const float a = v[1] - v[0], b = v[3] - v[0], c = (v[0] - v[1]) + (v[2] - v[3]);
    return v[0] + xi * a + eta * b + (xi * eta) * c;
}

struct LocalFace {
    int anc[3];          // lattice index of vertex 0
    float x[4], y[4], z[4];   // vertex positions in cells relative to the anchor
};

// pieces of one face, both clips, in the local-memory clipper (CFL 4 needs about 36 per clip;
// triangulation at a small minimal_area several times that)
constexpr int kMaxPieces32 = 128;

// Pieces emitted by the clipper of one face: centroid (cells, relative to the face anchor)
// and scaled y-normal, collected in order; the y-normals are summed here.
struct PieceSink {
    float4 p[kMaxPieces32];
    int n = 0;
    bool full = false;   // a piece was dropped: the clip stops (its flux is flagged anyway)
    Kahan ny;
    __host__ __device__ __forceinline__ void add(float cx, float cy, float cz, float nyv, unsigned& st) {
        ny.add(nyv);
        if (n >= kMaxPieces32) { st |= ST_CLIP_OVERFLOW; full = true; return; }
        p[n++] = make_float4(cx, cy, cz, nyv);
    }
};

// The clippers' loops are bounded by the colours: every cut strictly narrows the range of a
// polygon's finite colours.  A non-finite vertex (a NaN or infinite velocity upstream) would
// break that bound, so a face with one is not clipped: it emits no piece and is flagged.  The
// y coordinates are checked too, so no piece with a non-finite centroid reaches the quadrature.
__host__ __device__ __forceinline__ bool colours_finite(const float* c0, const float* c1, const float* y) {
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 4; ++q) ok = ok && isfinite(c0[q]) && isfinite(c1[q]) && isfinite(y[q]);
    return ok;
}

// Polygon vertices (xi, eta) as two arrays, for the clipper in local memory.
struct ArrayVerts {
    const float* px;
    const float* py;
    __host__ __device__ __forceinline__ float x(int n) const { return px[n]; }
    __host__ __device__ __forceinline__ float y(int n) const { return py[n]; }
};

// Centroid and area of a polygon in (xi, eta) (facecutter.h:226-253), the shoelace sums taken
// relative to the polygon's first vertex.  Equal in exact arithmetic to the sums over absolute
// coordinates; in FP32 the absolute form cancels for a sliver (a piece a few 1e-4 wide beside an
// iso-line, whose vertices are O(1) from the origin): its centroid came out up to ~1e-4 off,
// on the far side of the iso-line that bounds it, and the error pass's nearest-cell
// interpolation (1Dy-linear) then read psi of the wrong column.  Relative to the first vertex
// the products are of the sliver's own size and its centroid is accurate to FP32 rounding.
template <class V>
__host__ __device__ __forceinline__ void centroid_v(const V& v, int num, float& cx, float& cy, float& area) {
    const float x0 = v.x(0), y0 = v.y(0);
    float a = 0.f, sx = 0.f, sy = 0.f;
    for (int n = 0; n < num; ++n) {
        const int m = (n + 1 == num) ? 0 : n + 1;
        const float xn = v.x(n) - x0, yn = v.y(n) - y0, xm = v.x(m) - x0, ym = v.y(m) - y0;
        const float c = xn * ym - xm * yn;
        a += c; sx += c * (xn + xm); sy += c * (yn + ym);
    }
    a = fabsf(0.5f * a);
    if (a != 0.f) { const float s = 1.0f / (6.0f * a); cx = x0 + sx * s; cy = y0 + sy * s; }
    else {
        sx = 0.f; sy = 0.f;
        for (int n = 0; n < num; ++n) { sx += v.x(n) - x0; sy += v.y(n) - y0; }
        cx = x0 + sx / float(num); cy = y0 + sy / float(num);
    }
    area = a;
}
__host__ __device__ __forceinline__ void centroidf(const float* px, const float* py, int num, float& cx, float& cy, float& area) {
    centroid_v(ArrayVerts{px, py}, num, cx, cy, area);
}

// 3D centroid and scaled y-normal of a piece (split_face_3D.cpp:67-93); false when the
// normal vanishes (the piece is not emitted).
template <class V>
__host__ __device__ __forceinline__ bool piece_geom_v(const LocalFace& g, const V& v, int num, float cxi, float ceta,
                                             float4& out) {
    const float cx = bilinf(g.x, cxi, ceta), cy = bilinf(g.y, cxi, ceta), cz = bilinf(g.z, cxi, ceta);
    float ny;
    if (num == 3) {
        const float x0 = bilinf(g.x, v.x(0), v.y(0)), z0 = bilinf(g.z, v.x(0), v.y(0));
        const float ax = bilinf(g.x, v.x(1), v.y(1)) - x0, az = bilinf(g.z, v.x(1), v.y(1)) - z0;
        const float bx = bilinf(g.x, v.x(2), v.y(2)) - x0, bz = bilinf(g.z, v.x(2), v.y(2)) - z0;
        ny = 0.5f * (az * bx - ax * bz);
    } else {
        float acc = 0.f;
        float x0 = bilinf(g.x, v.x(0), v.y(0)) - cx, z0 = bilinf(g.z, v.x(0), v.y(0)) - cz;
        const float xs = x0, zs = z0;
        for (int n = 0; n < num; ++n) {
            float x1, z1;
            if (n + 1 == num) { x1 = xs; z1 = zs; }
            else { x1 = bilinf(g.x, v.x(n + 1), v.y(n + 1)) - cx; z1 = bilinf(g.z, v.x(n + 1), v.y(n + 1)) - cz; }
            acc += z0 * x1 - x0 * z1;
            x0 = x1; z0 = z1;
        }
        ny = acc * 0.5f;
    }
    out = make_float4(cx, cy, cz, ny);
    return ny != 0.f;
}
static __host__ __device__ void piece_geom32(const LocalFace& g, const float* px, const float* py, int num, float cxi, float ceta,
                             PieceSink& sink, unsigned& st) {
    float4 p;
    if (piece_geom_v(g, ArrayVerts{px, py}, num, cxi, ceta, p)) sink.add(p.x, p.y, p.z, p.w, st);
}

static __host__ __device__ void emit32(const PassDesc& d, const LocalFace& g, const float* px, const float* py, int num,
                       unsigned& st, int& npieces, PieceSink& sink) {
    float cx, cy, area;
    centroidf(px, py, num, cx, cy, area);
    const float minA = d.minimal_area_f;
    if (!(area > minA)) {
        if (area != 0.f) { ++npieces; piece_geom32(g, px, py, num, cx, cy, sink, st); }
        return;
    }
    float tri[24][6];
    int top = 0;
    if (num == 3) {
        tri[0][0] = px[0]; tri[0][1] = py[0]; tri[0][2] = px[1]; tri[0][3] = py[1]; tri[0][4] = px[2]; tri[0][5] = py[2];
        top = 1;
    } else {
        for (int n = num - 1; n >= 0; --n) {
            const int m = (n + 1 == num) ? 0 : n + 1;
            if (top >= 24) { st |= ST_SUBDIV_OVERFLOW; return; }
            tri[top][0] = cx; tri[top][1] = cy; tri[top][2] = px[n]; tri[top][3] = py[n];
            tri[top][4] = px[m]; tri[top][5] = py[m]; ++top;
        }
    }
    while (top > 0) {
        --top;
        float tx[3] = {tri[top][0], tri[top][2], tri[top][4]};
        float ty[3] = {tri[top][1], tri[top][3], tri[top][5]};
        float tcx, tcy, ta;
        centroidf(tx, ty, 3, tcx, tcy, ta);
        if (ta > minA) {
            // the first of the longest edges, lengths within kLongestEdgeTie counting as equal
            int mi = 0; float ml = -1.f;
            for (int n = 0; n < 3; ++n) {
                const int m = (n + 1) % 3;
                const float len = (tx[n] - tx[m]) * (tx[n] - tx[m]) + (ty[n] - ty[m]) * (ty[n] - ty[m]);
                if (len > ml * float(1.0 + kLongestEdgeTie)) { ml = len; mi = n; }
            }
            const int i1 = (mi + 1) % 3, i2 = (mi + 2) % 3;
            const float mx = 0.5f * (tx[mi] + tx[i1]), my = 0.5f * (ty[mi] + ty[i1]);
            if (top + 2 > 24) { st |= ST_SUBDIV_OVERFLOW; return; }
            tri[top][0] = mx; tri[top][1] = my; tri[top][2] = tx[i1]; tri[top][3] = ty[i1]; tri[top][4] = tx[i2]; tri[top][5] = ty[i2]; ++top;
            tri[top][0] = tx[mi]; tri[top][1] = ty[mi]; tri[top][2] = mx; tri[top][3] = my; tri[top][4] = tx[i2]; tri[top][5] = ty[i2]; ++top;
        } else if (ta != 0.f) {
            ++npieces;
            piece_geom32(g, tx, ty, 3, tcx, tcy, sink, st);
        }
    }
}

constexpr int kPool32 = 144, kMaxV32 = 32, kStack32 = 48;

// The point where edge a -> b crosses the iso-line (v0, v1: the edge ends' cut coordinate
// minus the iso value, of opposite signs); returns the edge parameter t1 of b.
__host__ __device__ __forceinline__ float cross_point(const CVf& a, const CVf& b, float v0, float v1, float iso, int dim, CVf& X) {
    const float inv = 1.0f / (v1 - v0);
    const float t0 = v1 * inv, t1 = -v0 * inv;
    X.p0 = t0 * a.p0 + t1 * b.p0;
    X.p1 = t0 * a.p1 + t1 * b.p1;
    const float other = snap_int(t0 * cvc(a, 1 - dim) + t1 * cvc(b, 1 - dim));
    if (dim == 0) { X.c0 = iso; X.c1 = other; } else { X.c1 = iso; X.c0 = other; }
    return t1;
}

// The clipper of fia_advect.cu (facecutter.h:59-224) on local colours.
static __host__ __device__ void clip32(const PassDesc& d, const LocalFace& g, unsigned& st, int& npieces, bool& multi,
                       PieceSink& sink) {
    CVf pool[kPool32];
    unsigned char sstart[kStack32], snum[kStack32], sdim[kStack32];
    const float xi[4] = {0.f, 1.f, 1.f, 0.f}, eta[4] = {0.f, 0.f, 1.f, 1.f};
    float col0[4], col1[4];
    for (int q = 0; q < 4; ++q) {
        col0[q] = snap_int(g.x[q] - d.color_off_f[0]);
        col1[q] = snap_int(g.z[q] - d.color_off_f[1]);
        pool[q].p0 = xi[q]; pool[q].p1 = eta[q];
        pool[q].c0 = col0[q];
        pool[q].c1 = col1[q];
    }
    if (!colours_finite(col0, col1, g.y)) { st |= ST_NONFINITE; return; }
    sstart[0] = 0; snum[0] = 4; sdim[0] = 0;
    int sp = 1;
    CVf tmp0[kMaxV32 + 2];
    while (sp > 0 && !sink.full) {
        --sp;
        const int pstart = sstart[sp], num = snum[sp], dim = sdim[sp];
        const CVf* poly = pool + pstart;
        float mn = cvc(poly[0], dim), mx = mn;
        for (int n = 1; n < num; ++n) { const float c = cvc(poly[n], dim); mn = fminf(mn, c); mx = fmaxf(mx, c); }
        int start = (int)ceilf(mn), end = (int)floorf(mx);
        if (mn - float(start) == 0.f) start += 1;
        if (mx - float(end) == 0.f) end -= 1;
        bool cut = false;
        if (start <= end) {
            if (pstart + 3 * num + 2 > kPool32) { st |= ST_CLIP_OVERFLOW; continue; }
            const float iso = float(start);
            int h0 = 0, h1 = 0, slot = 0, wpos = pstart + num, p1start = wpos, nchild = 0;
            unsigned char cst[kStack32], cnum[kStack32];
            tmp0[h0++] = poly[0];
            bool bad = false;
            for (int n = 0; n < num && !bad; ++n) {
                const int m = (n + 1 == num) ? 0 : n + 1;
                const float v0 = cvc(poly[n], dim) - iso, v1 = cvc(poly[m], dim) - iso;
                if ((v0 < 0.f) != (v1 < 0.f)) {
                    cut = true;
                    CVf X;
                    const float t1 = cross_point(poly[n], poly[m], v0, v1, iso, dim, X);
                    if (slot == 0) {
                        tmp0[h0++] = X;
                        slot = 1; h1 = 0; p1start = wpos;
                        if (t1 < 1.0f) pool[p1start + h1++] = X;
                    } else {
                        pool[p1start + h1++] = X;
                        if (nchild >= kStack32 - 1) { bad = true; break; }
                        cst[nchild] = (unsigned char)p1start; cnum[nchild] = (unsigned char)h1; ++nchild;
                        wpos = p1start + h1;
                        slot = 0;
                        if (t1 < 1.0f) tmp0[h0++] = X;
                    }
                }
                if (n < num - 1) {
                    if (slot == 0) tmp0[h0++] = poly[m];
                    else pool[p1start + h1++] = poly[m];
                }
                if (h0 >= kMaxV32 || h1 >= kMaxV32 || p1start + h1 + 2 >= kPool32) bad = true;
            }
            if (bad) { st |= ST_CLIP_OVERFLOW; continue; }
            if (nchild > 1) multi = true;
            if (cut) {
                if (slot != 0) { st |= ST_CLIP_ODD_CUT; continue; }
                if (wpos + h0 >= kPool32 || sp + nchild + 1 > kStack32) { st |= ST_CLIP_OVERFLOW; continue; }
                for (int q = 0; q < h0; ++q) pool[wpos + q] = tmp0[q];
                const int src = pstart + num, len = wpos + h0 - src;
                for (int q = 0; q < len; ++q) pool[pstart + q] = pool[src + q];
                for (int c = 0; c < nchild; ++c) {
                    sstart[sp] = (unsigned char)(cst[c] - num); snum[sp] = cnum[c]; sdim[sp] = (unsigned char)dim; ++sp;
                }
                sstart[sp] = (unsigned char)(wpos - num); snum[sp] = (unsigned char)h0; sdim[sp] = (unsigned char)dim; ++sp;
            }
        }
        if (!cut) {
            if (dim == 0) {
                sstart[sp] = (unsigned char)pstart; snum[sp] = (unsigned char)num; sdim[sp] = 1; ++sp;
            } else if (num >= 3) {
                float px[kMaxV32], py[kMaxV32];
                for (int q = 0; q < num; ++q) { px[q] = poly[q].p0; py[q] = poly[q].p1; }
                emit32(d, g, px, py, num, st, npieces, sink);
            }
        }
    }
}

// The clipper in shared memory.  Each thread owns kFastR vertex slots (xi, eta and the two
// colours, one word each) and kFastS stack words of the CTA's dynamic shared memory, laid
// out word-major ([word][thread]): a warp's access to one word of its threads' slots is one
// conflict-free wavefront however far apart the threads' polygons are, where the same pool
// in local memory costs a line per thread and, with 36 warps per SM, is written back to
// DRAM (about 360 bytes per face).  The pool grows upward from slot 0 and the face's pieces
// downward from the top slot.  It is clip32 -- the same cuts, pieces, emission order and
// arithmetic -- except that a face needing more room (about 0.2% of the faces of a developed
// flow at CFL 2), cutting a polygon an odd number of times, or holding a piece above the
// triangulation area returns false and is clipped again by clip32 in local memory.
constexpr int kFastR = 26, kFastS = 6, kClipThreads = 128;
constexpr int kFastWords = 4 * kFastR + kFastS;
constexpr int kClipSmem = kFastWords * kClipThreads * (int)sizeof(float);   // 56,320 B: 4 CTAs per SM
static_assert(4 * (kClipSmem + 1024) <= 233472, "four clip CTAs per SM");

#ifndef __CUDA_ARCH__
// host builds of the clipper (the host check of the shared-pool clipper) stop on a slot outside
// the pool; on the device the bounds are the checks in clip32_fast
[[noreturn]] inline void fast_pool_range_error(int e, int c) {
    std::fprintf(stderr, "fast clip pool: slot %d word %d out of range\n", e, c);
    std::abort();
}
#endif

struct FastPool {
    float* w;   // this thread's word 0
    __host__ __device__ __forceinline__ float& at(int e, int c) const {
#ifndef __CUDA_ARCH__
        if (e < 0 || e >= kFastR || c < 0 || c > 3) fast_pool_range_error(e, c);
#endif
        return w[(4 * e + c) * kClipThreads];
    }
    __host__ __device__ __forceinline__ CVf get(int e) const { return CVf{at(e, 0), at(e, 1), at(e, 2), at(e, 3)}; }
    __host__ __device__ __forceinline__ void put(int e, const CVf& v) const {
        at(e, 0) = v.p0; at(e, 1) = v.p1; at(e, 2) = v.c0; at(e, 3) = v.c1;
    }
    __host__ __device__ __forceinline__ unsigned& stk(int i) const {
#ifndef __CUDA_ARCH__
        if (i < 0 || i >= kFastS) fast_pool_range_error(kFastR + i, -1);
#endif
        return reinterpret_cast<unsigned*>(w)[(4 * kFastR + i) * kClipThreads];
    }
};
struct PoolVerts {
    FastPool P;
    int s;
    __host__ __device__ __forceinline__ float x(int n) const { return P.at(s + n, 0); }
    __host__ __device__ __forceinline__ float y(int n) const { return P.at(s + n, 1); }
};
__host__ __device__ __forceinline__ unsigned stack_word(int start, int num, int dim) {
    return (unsigned)start | ((unsigned)num << 8) | ((unsigned)dim << 16);
}

// One clip of a face (facecutter.h:59-224) in the shared pool.  nst pieces are stored so far
// (slot kFastR - 1 - q holds piece q as cx, cy, cz, ny); ny sums the y-normals of this clip.
static __host__ __device__ bool clip32_fast(const PassDesc& d, const LocalFace& g, int& npieces, bool& multi, int& nst, Kahan& ny,
                            const FastPool& P) {
    if (4 > kFastR - nst) return false;
    const float xi[4] = {0.f, 1.f, 1.f, 0.f}, eta[4] = {0.f, 0.f, 1.f, 1.f};
    float col0[4], col1[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        col0[q] = snap_int(g.x[q] - d.color_off_f[0]);
        col1[q] = snap_int(g.z[q] - d.color_off_f[1]);
    }
    if (!colours_finite(col0, col1, g.y)) return false;    // flagged by clip32
#pragma unroll
    for (int q = 0; q < 4; ++q) P.put(q, CVf{xi[q], eta[q], col0[q], col1[q]});
    P.stk(0) = stack_word(0, 4, 0);
    int sp = 1;
    const float minA = d.minimal_area_f;
    while (sp > 0) {
        --sp;
        const unsigned e = P.stk(sp);
        const int pstart = (int)(e & 0xffu), num = (int)((e >> 8) & 0xffu), dim = (int)(e >> 16);
        const int cc = 2 + dim;
        float mn = P.at(pstart, cc), mx = mn;
        for (int n = 1; n < num; ++n) { const float c = P.at(pstart + n, cc); mn = fminf(mn, c); mx = fmaxf(mx, c); }
        int start = (int)ceilf(mn), end = (int)floorf(mx);
        if (mn - float(start) == 0.f) start += 1;
        if (mx - float(end) == 0.f) end -= 1;
        bool cut = false;
        if (start <= end) {
            const float iso = float(start);
            // the crossings bound what the cut writes: the parts away from vertex 0 (at most
            // num - 1 + ncross vertices) from pstart + num, the part holding vertex 0 (at most
            // num + ncross) from b0, after them
            int ncross = 0;
            bool sprev = (P.at(pstart + num - 1, cc) - iso) < 0.f;
            for (int n = 0; n < num; ++n) {
                const bool sn = (P.at(pstart + n, cc) - iso) < 0.f;
                ncross += sn != sprev ? 1 : 0;
                sprev = sn;
            }
            const int b0 = pstart + 2 * num - 1 + ncross;
            if (b0 + num + ncross > kFastR - nst) return false;
            int h0 = 0, h1 = 0, slot = 0, wpos = pstart + num, p1start = wpos, nchild = 0;
            const CVf V0 = P.get(pstart);
            CVf A = V0;
            P.put(b0 + h0++, V0);
            for (int n = 0; n < num; ++n) {
                const CVf B = (n + 1 == num) ? V0 : P.get(pstart + n + 1);
                const float v0 = cvc(A, dim) - iso, v1 = cvc(B, dim) - iso;
                if ((v0 < 0.f) != (v1 < 0.f)) {
                    cut = true;
                    CVf X;
                    const float t1 = cross_point(A, B, v0, v1, iso, dim, X);
                    if (slot == 0) {
                        P.put(b0 + h0++, X);
                        slot = 1; h1 = 0; p1start = wpos;
                        if (t1 < 1.0f) P.put(p1start + h1++, X);
                    } else {
                        P.put(p1start + h1++, X);
                        // the part is complete: pushed where it lands after the parent is dropped
                        if (sp >= kFastS) return false;
                        P.stk(sp++) = stack_word(p1start - num, h1, dim);
                        ++nchild;
                        wpos = p1start + h1;
                        slot = 0;
                        if (t1 < 1.0f) P.put(b0 + h0++, X);
                    }
                }
                if (n < num - 1) {
                    if (slot == 0) P.put(b0 + h0++, B);
                    else P.put(p1start + h1++, B);
                }
                A = B;
            }
            if (nchild > 1) multi = true;
            if (cut) {
                if (slot != 0 || sp >= kFastS) return false;
                // drop the parent: the parts move down by num, the part of vertex 0 follows them
                for (int q = pstart + num; q < wpos; ++q) P.put(q - num, P.get(q));
                for (int q = 0; q < h0; ++q) P.put(wpos - num + q, P.get(b0 + q));
                P.stk(sp++) = stack_word(wpos - num, h0, dim);
            }
        }
        if (!cut) {
            if (dim == 0) {
                if (sp >= kFastS) return false;
                P.stk(sp++) = stack_word(pstart, num, 1);
            } else if (num >= 3) {
                const PoolVerts V{P, pstart};
                float cx, cy, area;
                centroid_v(V, num, cx, cy, area);
                if (area > minA) return false;      // triangulated by clip32
                if (area != 0.f) {
                    ++npieces;
                    float4 pc;
                    if (piece_geom_v(g, V, num, cx, cy, pc)) {
                        ny.add(pc.w);
                        const int slotp = kFastR - 1 - nst;
                        if (slotp < pstart) return false;   // the polygon above pstart is spent
                        P.at(slotp, 0) = pc.x; P.at(slotp, 1) = pc.y; P.at(slotp, 2) = pc.z; P.at(slotp, 3) = pc.w;
                        ++nst;
                    }
                }
            }
        }
    }
    return true;
}

// the upper cell's vertex order (v0, v3, v2, v1)
__host__ __device__ __forceinline__ LocalFace reversed_face(const LocalFace& g) {
    LocalFace r = g;
    r.x[1] = g.x[3]; r.y[1] = g.y[3]; r.z[1] = g.z[3];
    r.x[3] = g.x[1]; r.y[3] = g.y[1]; r.z[3] = g.z[1];
    return r;
}


}  // namespace fia
