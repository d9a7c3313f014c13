// cpu_stream.inl -- the streaming-tile CPU baseline, compiled into the oracle library (this
// file is included at the end of fia_oracle.cpp and uses its clipper and field descriptions).
//
// TEST AND BASELINE INFRASTRUCTURE: bench.py times it as the CPU baseline; tests check it
// against the oracle.  It is not the oracle (which keeps the reference's structure) and not
// the product (the GPU library).
//
// The reference's fastest CPU interpolator, sginterp3::interpolate (sginterp3.cpp:204-385),
// presorts the points to be interpolated by the cell of their stencil and streams each column
// of cells with a rolling 6x6x6 cache of samples, one new plane per cell, under OpenMP with an
// ISPC kernel.  This restates that design in plain C++ (std::thread, no ISPC) around a density
// step organised for a CPU rather than per cell:
//   psi           columns in parallel;
//   vertices      every lattice vertex backtraced once (the reference: once per face using it);
//   faces         every face clipped once in the lower cell's vertex order, and again in the
//                 upper cell's only where the partition depends on it (the reference: twice);
//   points        the quadrature points of all pieces (polygon_3D.cpp:257-487) presorted by
//                 the cell of their WENO6 stencil and evaluated column by column along x with
//                 a ring of six (y, z) planes of 6 x 6 samples;
//   fluxes        summed per face side in piece order, then gathered per cell.
// FP64 throughout; WENO6 in the difference form of the smoothness indicators and collapsed
// along axes on which a point lies on a node plane, both equal to the reference's
// evaluation in exact arithmetic (so the results match the oracle to rounding).

namespace {

struct SWCoef { real a[3], b[3], c[3], C[3]; };

inline SWCoef sw_coef(const real* t) {
    SWCoef w;
    for (int i = 0; i < 3; ++i) {
        w.a[i] = t[i];
        w.b[i] = t[i] * t[i + 1] / 2.0;
        w.c[i] = t[i] * t[i + 1] * t[i + 2] / 6.0;
    }
    w.C[0] = t[4] * t[5] / 20.0;
    w.C[1] = -t[5] * t[0] / 10.0;
    w.C[2] = t[0] * t[1] / 20.0;
    return w;
}

// WENO6 of six samples: the candidates as Newton forms in the distances t (cells), the
// smoothness indicators as quadratic forms of the first differences (the reference's
// indicators, WENO6_interpolation_3d.cpp:95-110, expanded), alpha = C / (1e-6 + beta)^2.
inline real sw_eval(const real* f, const SWCoef& w) {
    const real D0 = f[1] - f[0], D1 = f[2] - f[1], D2 = f[3] - f[2], D3 = f[4] - f[3], D4 = f[5] - f[4];
    const real S0 = D1 - D0, S1 = D2 - D1, S2 = D3 - D2;
    const real T0 = S1 - S0, T1 = S2 - S1, T2 = (D4 - D3) - S2;
    const real P0 = f[0] + D0 * w.a[0] + S0 * w.b[0] + T0 * w.c[0];
    const real P1 = f[1] + D1 * w.a[1] + S1 * w.b[1] + T1 * w.c[1];
    const real P2 = f[2] + D2 * w.a[2] + S2 * w.b[2] + T2 * w.c[2];
    const real r180 = 1.0 / 180.0;
    const real b0 = (244 * D0 * D0 - 1171 * D0 * D1 + 683 * D0 * D2 + 1561 * D1 * D1 - 1951 * D1 * D2 + 814 * D2 * D2) * r180;
    const real b1 = (244 * D1 * D1 - 781 * D1 * D2 + 293 * D1 * D3 + 961 * D2 * D2 - 781 * D2 * D3 + 244 * D3 * D3) * r180;
    const real b2 = (814 * D2 * D2 - 1951 * D2 * D3 + 683 * D2 * D4 + 1561 * D3 * D3 - 1171 * D3 * D4 + 244 * D4 * D4) * r180;
    const real e0 = 1e-6 + b0, e1 = 1e-6 + b1, e2 = 1e-6 + b2;
    const real q0 = e0 * e0, q1 = e1 * e1, q2 = e2 * e2;
    const real qm = std::max(q0, std::max(q1, q2));
    const real t0 = q0 / qm, t1 = q1 / qm, t2 = q2 / qm;
    const real a0 = w.C[0] * (t1 * t2), a1 = w.C[1] * (t0 * t2), a2 = w.C[2] * (t0 * t1);
    return (a0 * P0 + a1 * P1 + a2 * P2) / (a0 + a1 + a2);
}

// Stencil base of a coordinate along one axis: the node index when the point lies on a node
// plane (the axis then collapses), else the floor.
inline int sw_base(real p, real off, real h, bool& on_node) {
    const real r = (p - off * h) / h;
    const real s = snap_int(r);
    on_node = s == std::nearbyint(s);
    return on_node ? (int)s : (int)std::floor(r);
}

struct SPt { real p[3]; real w; long out; };   // a point to evaluate: position, weight, result slot

// body(i) for i in [0, n), contiguous ranges per thread
template <class F>
static void parallel_for(int nthreads, long n, const F& body) {
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t]() {
            for (long i = n * t / nthreads; i < n * (t + 1) / nthreads; ++i) body(i);
        });
    for (auto& x : th) x.join();
}

// res[pts[i].out] = pts[i].w * WENO6(F, pts[i].p), collapsed on node planes.  The points are
// presorted by the cell of their stencil (a counting sort over the (y, z) columns, then by x
// within a column) and each thread takes a run of columns; within a column it walks x upwards,
// keeping the six (y, z) planes of 6 x 6 samples of the current stencil in a ring and loading
// one plane per step.
static void stream_eval(const Field& F, real h, const std::vector<SPt>& pts, real* res, int nthreads) {
    const int B = 4;                                     // bases lie in [-1, M]; margin 4
    const long NBY = F.M[1] + 2 * B, NBZ = F.M[2] + 2 * B;
    const long npt = (long)pts.size();
    if (npt == 0) return;
    std::vector<long> col_of(npt);
    std::vector<int> bx_of(npt);
    const long ncol = NBY * NBZ;
    // counting sort by column: per-thread histograms, offsets, scatter
    std::vector<std::vector<long>> hist(nthreads, std::vector<long>(ncol, 0));
    {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; ++t)
            th.emplace_back([&, t]() {
                const long a = npt * t / nthreads, b = npt * (t + 1) / nthreads;
                for (long i = a; i < b; ++i) {
                    bool c;
                    bx_of[i] = sw_base(pts[i].p[0], F.off[0], h, c);
                    const long by = std::min(std::max((long)sw_base(pts[i].p[1], F.off[1], h, c) + B, 0L), NBY - 1);
                    const long bz = std::min(std::max((long)sw_base(pts[i].p[2], F.off[2], h, c) + B, 0L), NBZ - 1);
                    col_of[i] = by * NBZ + bz;
                    ++hist[t][col_of[i]];
                }
            });
        for (auto& x : th) x.join();
    }
    std::vector<long> start(ncol + 1, 0);
    {
        long acc = 0;
        for (long k = 0; k < ncol; ++k) {
            start[k] = acc;
            for (int t = 0; t < nthreads; ++t) { const long c = hist[t][k]; hist[t][k] = acc; acc += c; }
        }
        start[ncol] = acc;
    }
    std::vector<long> order(npt);
    {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; ++t)
            th.emplace_back([&, t]() {
                const long a = npt * t / nthreads, b = npt * (t + 1) / nthreads;
                for (long i = a; i < b; ++i) order[hist[t][col_of[i]]++] = i;
            });
        for (auto& x : th) x.join();
    }
    hist.clear();
    // columns split between threads by point count
    std::vector<long> colcut(nthreads + 1, ncol);
    colcut[0] = 0;
    for (int t = 1; t < nthreads; ++t) {
        const long target = npt * t / nthreads;
        long c = colcut[t - 1];
        while (c < ncol && start[c] < target) ++c;
        colcut[t] = c;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t]() {
            real ring[6][36];
            for (long col = colcut[t]; col < colcut[t + 1]; ++col) {
                const long p0 = start[col], p1 = start[col + 1];
                if (p0 == p1) continue;
                std::sort(order.begin() + p0, order.begin() + p1, [&](long a, long b) {
                    return bx_of[a] != bx_of[b] ? bx_of[a] < bx_of[b] : a < b;
                });
                const int by = (int)(col / NBZ) - B, bz = (int)(col % NBZ) - B;
                int cur = -1 << 30, head = 0;
                auto load_plane = [&](int slot, int x) {
                    const int ii = clampi(x, 0, F.M[0] - 1);
                    for (int iy = 0; iy < 6; ++iy) {
                        const int jj = clampi(by - 2 + iy, 0, F.M[1] - 1);
                        const real* row = F.a + (long)F.M[2] * ((long)F.M[1] * ii + jj);
                        for (int iz = 0; iz < 6; ++iz) ring[slot][iy * 6 + iz] = row[clampi(bz - 2 + iz, 0, F.M[2] - 1)];
                    }
                };
                for (long q = p0; q < p1; ++q) {
                    const SPt& P = pts[order[q]];
                    bool cxn, cyn, czn;
                    const int bx = sw_base(P.p[0], F.off[0], h, cxn);
                    sw_base(P.p[1], F.off[1], h, cyn);
                    sw_base(P.p[2], F.off[2], h, czn);
                    if (bx != cur) {
                        if (bx == cur + 1) {                      // slide the ring by one plane
                            load_plane(head, bx + 3);
                            head = (head + 1) % 6;
                        } else {
                            for (int s = 0; s < 6; ++s) load_plane(s, bx - 2 + s);
                            head = 0;
                        }
                        cur = bx;
                    }
                    real tx[6], ty[6], tz[6];
                    for (int i = 0; i < 6; ++i) {
                        tx[i] = (P.p[0] - ((bx - 2 + i) + F.off[0]) * h) / h;
                        ty[i] = (P.p[1] - ((by - 2 + i) + F.off[1]) * h) / h;
                        tz[i] = (P.p[2] - ((bz - 2 + i) + F.off[2]) * h) / h;
                    }
                    const SWCoef wx = sw_coef(tx), wy = sw_coef(ty), wz = sw_coef(tz);
                    const int x0 = cxn ? 2 : 0, x1 = cxn ? 3 : 6, y0 = cyn ? 2 : 0, y1 = cyn ? 3 : 6;
                    real yv[6] = {0, 0, 0, 0, 0, 0};
                    for (int ix = x0; ix < x1; ++ix) {
                        const real* plane = ring[(head + ix) % 6];
                        real zv[6] = {0, 0, 0, 0, 0, 0};
                        for (int iy = y0; iy < y1; ++iy)
                            zv[iy] = czn ? plane[iy * 6 + 2] : sw_eval(plane + iy * 6, wz);
                        yv[ix] = cyn ? zv[2] : sw_eval(zv, wy);
                    }
                    res[P.out] = P.w * (cxn ? yv[2] : sw_eval(yv, wx));
                }
            }
        });
    for (auto& x : th) x.join();
}

// psi on the columns [xlo, xhi), columns split between threads; WENO6 increments use sw_eval
static void stream_psi(const Field& F, real h, int mode, const Gauss1D& g, std::vector<real>& psi, int xlo, int xhi,
                       int nthreads) {
    const int Mp[3] = {F.M[0], F.M[1] + 1, F.M[2]};
    psi.assign((size_t)Mp[0] * Mp[1] * Mp[2], 0.0);
    xlo = std::max(xlo, 0);
    xhi = std::min(xhi, Mp[0]);
    if (xlo >= xhi) return;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t]() {
            const long ncol = (long)(xhi - xlo) * Mp[2];
            for (long col = ncol * t / nthreads; col < ncol * (t + 1) / nthreads; ++col) {
                const int i = xlo + (int)(col / Mp[2]), k = (int)(col % Mp[2]);
                real acc = 0.0;
                for (int j = 1; j < Mp[1]; ++j) {
                    if (mode == PSI_PLAIN) {
                        acc = acc + F.a[idx3(F.M, i, j - 1, k)] * h;
                    } else if (mode == PSI_WENO6) {
                        const real ylo = (j - 1.0 + F.off[1] - 0.5) * h, ymid = (j - 0.5 + F.off[1] - 0.5) * h;
                        const real yhi = (j + F.off[1] - 0.5) * h;
                        for (int half = 0; half < 2; ++half) {
                            const real a = half ? ymid : ylo, b = half ? yhi : ymid;
                            for (int q = 0; q < g.k; ++q) {
                                const real py = gauss_pos(g, q, a, b);
                                const int base = (int)std::floor((py - F.off[1] * h) / h);
                                real f[6], tt[6];
                                for (int s = 0; s < 6; ++s) {
                                    tt[s] = (py - (base - 2 + s + F.off[1]) * h) / h;
                                    f[s] = F.a[idx3(F.M, i, clampi(base - 2 + s, 0, F.M[1] - 1), k)];
                                }
                                acc += sw_eval(f, sw_coef(tt)) * (h / 2.0) * g.w[q];
                            }
                        }
                    } else {
                        const real p0[3] = {(i + F.off[0]) * h, ((j - 1) + 0.25 + F.off[1] - 0.5) * h, (k + F.off[2]) * h};
                        const real p1[3] = {(i + F.off[0]) * h, ((j - 1) + 0.75 + F.off[1] - 0.5) * h, (k + F.off[2]) * h};
                        acc = acc + lin3d(F, p0, h) * (h / 2.0) + lin3d(F, p1, h) * (h / 2.0);
                    }
                    psi[idx3(Mp, i, j, k)] = acc;
                }
            }
        });
    for (auto& x : th) x.join();
}

// One flux pass of the density on the cells with x in [cx0, cx1); psi on columns
// [psi_x0, psi_x1).  out[cell] for those cells.
static int stream_pass(const Grid& G, const Velocity& vel, const Field& A, const PassParams& P, real* out,
                       int nthreads, int cx0, int cx1, int psi_x0, int psi_x1, long* faces_out) {
    const real h = G.h, V = h * h * h;
    const int nx = A.M[0], ny = A.M[1], nz = A.M[2];
    const Gauss1D g = make_gauss(P.k);
    std::vector<real> psi;
    stream_psi(A, h, P.psi_mode, g, psi, psi_x0, psi_x1, nthreads);
    Field Psi;
    Psi.a = psi.data();
    Psi.M[0] = nx; Psi.M[1] = ny + 1; Psi.M[2] = nz;
    Psi.off[0] = A.off[0]; Psi.off[1] = A.off[1] - 0.5; Psi.off[2] = A.off[2];
    // vertices of the slab (x in [cx0, cx1]); the velocity samples are sorted and streamed
    // like the quadrature points
    const int Ly = ny + 1, Lz = nz + 1, Lx = cx1 - cx0 + 1;
    const long nv = (long)Lx * Ly * Lz;
    std::vector<real> verts(3 * nv);
    for (long v = 0; v < nv; ++v) {
        verts[3 * v] = (cx0 + v / ((long)Ly * Lz)) * h;
        verts[3 * v + 1] = ((v / Lz) % Ly) * h;
        verts[3 * v + 2] = (v % Lz) * h;
    }
    if (!P.zero_velocity) {
        std::vector<real> vel3(3 * nv);
        if (P.interp == I_WENO6) {
            const Field* f[3] = {&vel.u, &vel.v, &vel.w};
            std::vector<SPt> pts(nv);
            for (int c = 0; c < 3; ++c) {
                for (long v = 0; v < nv; ++v) {
                    for (int d = 0; d < 3; ++d) pts[v].p[d] = verts[3 * v + d];
                    pts[v].w = 1.0; pts[v].out = 3 * v + c;
                }
                stream_eval(*f[c], h, pts, vel3.data(), nthreads);
            }
        } else {
            parallel_for(nthreads, nv, [&](long v) {
                const real* p = &verts[3 * v];
                vel3[3 * v] = interp(P.interp, vel.u, p, h);
                vel3[3 * v + 1] = interp(P.interp, vel.v, p, h);
                vel3[3 * v + 2] = interp(P.interp, vel.w, p, h);
            });
        }
        for (long v = 0; v < nv; ++v)
            for (int d = 0; d < 3; ++d) {
                real p = verts[3 * v + d] - vel3[3 * v + d] * P.dt;
                if (p < 0.0) p = 0.0;
                if (p > h * G.N[d]) p = h * G.N[d];
                verts[3 * v + d] = p;
            }
    }
    auto vert = [&](int i, int j, int k) { return &verts[3 * (((long)(i - cx0) * Ly + j) * Lz + k)]; };
    // faces of the slab: x-faces on planes [cx0, cx1], y- and z-faces of its cells
    const long nfx = (long)(cx1 - cx0 + 1) * ny * nz, nfy = (long)(cx1 - cx0) * (ny + 1) * nz;
    const long nfz = (long)(cx1 - cx0) * ny * (nz + 1), nf = nfx + nfy + nfz;
    // per face: the two sides' fluxes (lower cell's vertex order, upper cell's)
    std::vector<real> side(2 * nf, 0.0);
    std::vector<int> multi(nf, 0);
    // per thread (a contiguous run of faces): the density points and the psi point of every
    // piece in piece order, the slot (2 face + side) of each psi point and the number of
    // density points before it that belong to its piece
    std::vector<std::vector<SPt>> apts(nthreads), ppts(nthreads);
    std::vector<std::vector<long>> pslot(nthreads);
    std::vector<std::vector<int>> pna(nthreads);
    std::vector<PassCounters> cnt(nthreads);
    {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; ++t)
            th.emplace_back([&, t]() {
                std::vector<SubPoly> polys;
                for (long f = nf * t / nthreads; f < nf * (t + 1) / nthreads; ++f) {
                    int fam, i, j, k;
                    if (f < nfx) {
                        fam = 0; i = cx0 + (int)(f / ((long)ny * nz)); j = (int)((f / nz) % ny); k = (int)(f % nz);
                    } else if (f < nfx + nfy) {
                        const long r = f - nfx; fam = 1;
                        i = cx0 + (int)(r / ((long)(ny + 1) * nz)); j = (int)((r / nz) % (ny + 1)); k = (int)(r % nz);
                    } else {
                        const long r = f - nfx - nfy; fam = 2;
                        i = cx0 + (int)(r / ((long)ny * (nz + 1))); j = (int)((r / (nz + 1)) % ny); k = (int)(r % (nz + 1));
                    }
                    // the lower cell's vertex order (backtrace_..._for_integrate_density.cpp:83-112);
                    // the upper cell sees v0, v3, v2, v1
                    static const int corner[3][4][3] = {{{0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1}},
                                                        {{0, 0, 0}, {0, 0, 1}, {1, 0, 1}, {1, 0, 0}},
                                                        {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}}};
                    real v[4][3];
                    for (int a = 0; a < 4; ++a) {
                        const real* p = vert(i + corner[fam][a][0], j + corner[fam][a][1], k + corner[fam][a][2]);
                        v[a][0] = p[0]; v[a][1] = p[1]; v[a][2] = p[2];
                    }
                    for (int s = 0; s < 2; ++s) {
                        if (s == 1 && !multi[f]) break;
                        real vs[4][3];
                        for (int a = 0; a < 4; ++a) {
                            const int src = s == 0 ? a : (a == 1 ? 3 : (a == 3 ? 1 : a));
                            vs[a][0] = v[src][0]; vs[a][1] = v[src][1]; vs[a][2] = v[src][2];
                        }
                        polys.clear();
                        int m = 0;
                        cnt[t].status |= split_face(vs, h, P.color_off, P.minimal_area, polys, &m);
                        if (s == 0) { multi[f] = m; cnt[t].faces++; }
                        cnt[t].polys += (long)polys.size();
                        const long slot = 2 * f + s;
                        for (const SubPoly& sp : polys) {
                            SPt pp; pp.p[0] = sp.pos[0]; pp.p[2] = sp.pos[2]; pp.w = sp.n[1] / V; pp.out = 0;
                            int na = 0;
                            if (P.use_integral) {
                                // polygon_3D.cpp:257-487 (density grid: y origin 0)
                                const real ry = snap_int(sp.pos[1] / h);
                                const int iy0 = (int)std::floor(ry);
                                const real f01 = ry - iy0;
                                SPt pt; pt.p[0] = sp.pos[0]; pt.p[2] = sp.pos[2]; pt.out = 0;
                                auto add = [&](real a, real b, real frac) {
                                    for (int q = 0; q < g.k; ++q) {
                                        pt.p[1] = gauss_pos(g, q, a, b);
                                        pt.w = sp.n[1] * frac * h * g.w[q] / V;
                                        apts[t].push_back(pt);
                                        ++na;
                                    }
                                };
                                if (f01 < 0.5) {
                                    add(iy0 * h, sp.pos[1], f01);
                                } else {
                                    add(iy0 * h, (iy0 + 0.5) * h, 0.5);
                                    add((iy0 + 0.5) * h, (iy0 + f01) * h, f01 - 0.5);
                                }
                                pp.p[1] = iy0 * h;
                            } else {
                                pp.p[1] = sp.pos[1];
                            }
                            ppts[t].push_back(pp);
                            pslot[t].push_back(slot);
                            pna[t].push_back(na);
                        }
                    }
                }
            });
        for (auto& x : th) x.join();
    }
    // all points in face order (thread t held a contiguous run of faces), evaluated streaming
    std::vector<SPt> A_all, P_all;
    std::vector<long> P_slot;
    std::vector<int> P_na;
    for (int t = 0; t < nthreads; ++t) {
        A_all.insert(A_all.end(), apts[t].begin(), apts[t].end());
        P_all.insert(P_all.end(), ppts[t].begin(), ppts[t].end());
        P_slot.insert(P_slot.end(), pslot[t].begin(), pslot[t].end());
        P_na.insert(P_na.end(), pna[t].begin(), pna[t].end());
        std::vector<SPt>().swap(apts[t]);
        std::vector<SPt>().swap(ppts[t]);
    }
    for (long i = 0; i < (long)A_all.size(); ++i) A_all[i].out = i;
    for (long i = 0; i < (long)P_all.size(); ++i) P_all[i].out = i;
    std::vector<real> A_res(A_all.size()), P_res(P_all.size());
    if (P.interp == I_WENO6) {
        stream_eval(A, h, A_all, A_res.data(), nthreads);
        stream_eval(Psi, h, P_all, P_res.data(), nthreads);
    } else {
        parallel_for(nthreads, (long)A_all.size(), [&](long i) { A_res[i] = A_all[i].w * interp(P.interp, A, A_all[i].p, h); });
        parallel_for(nthreads, (long)P_all.size(), [&](long i) { P_res[i] = P_all[i].w * interp(P.interp, Psi, P_all[i].p, h); });
    }
    // per face side, in piece order: each piece's density points, then its psi point
    {
        long ia = 0;
        for (long ip = 0; ip < (long)P_all.size(); ++ip) {
            real acc = side[P_slot[ip]];
            for (int q = 0; q < P_na[ip]; ++q) acc += A_res[ia++];
            side[P_slot[ip]] = acc + P_res[ip];
        }
    }
    // gather: a cell's x+ face is the lower side of face x = i + 1, its x- face the upper side
    // of face x = i (the negated lower side unless the partition depends on the vertex order)
    auto fx = [&](int i, int j, int k) { return (long)(i - cx0) * ny * nz + (long)j * nz + k; };
    auto fy = [&](int i, int j, int k) { return nfx + (long)(i - cx0) * (ny + 1) * nz + (long)j * nz + k; };
    auto fz = [&](int i, int j, int k) { return nfx + nfy + (long)(i - cx0) * ny * (nz + 1) + (long)j * (nz + 1) + k; };
    auto up = [&](long f) { return multi[f] ? side[2 * f + 1] : -side[2 * f]; };
    parallel_for(nthreads, (long)(cx1 - cx0) * ny * nz, [&](long c) {
        const int i = cx0 + (int)(c / ((long)ny * nz)), j = (int)((c / nz) % ny), k = (int)(c % nz);
        out[idx3(A.M, i, j, k)] = side[2 * fx(i + 1, j, k)] + up(fx(i, j, k)) + side[2 * fy(i, j + 1, k)] +
                                  up(fy(i, j, k)) + side[2 * fz(i, j, k + 1)] + up(fz(i, j, k));
    });
    int status = 0;
    long nfaces = 0;
    for (auto& c : cnt) { status |= c.status; nfaces += c.faces; }
    if (faces_out) *faces_out = nfaces;
    return status;
}

}  // namespace

// move_substances_3D (flux branch, density) with the streaming passes on the x-slab [x0, x1),
// organised as fo_move_substances_slab (the same margins); x0 = 0, x1 = nx is the whole step.
extern "C" int fo_stream_move_substances_slab(int nx, int ny, int nz, double h, const double* u, const double* v,
                                              const double* w, const double* rho, double dt, int interp_method,
                                              int k, int correction, int use_integral, const double* split_off,
                                              double minimal_area, int nthreads, int x0, int x1, int margin,
                                              double* out, long* faces) {
    Grid G; G.N[0] = nx; G.N[1] = ny; G.N[2] = nz; G.h = h;
    if (x0 < 0 || x1 > nx || x0 >= x1 || margin < 0 || nthreads < 1) return -1;
    Velocity vel = make_velocity(G, u, v, w);
    Field A = make_field(rho, G, -1);
    for (int d = 0; d < 3; ++d) { A.M[d] = G.N[d]; A.off[d] = 0.5; }
    const long plane = (long)ny * nz, n = (long)nx * plane;
    PassParams P;
    P.comp = -1; P.interp = interp_method; P.k = k; P.minimal_area = minimal_area; P.dt = dt;
    P.psi_mode = use_integral ? (interp_method == I_WENO6 ? PSI_WENO6 : PSI_LINEAR) : PSI_PLAIN;
    P.use_integral = use_integral; P.zero_velocity = 0; P.maccormack = 0;
    split_offsets(-1, 0, split_off, P.color_off);
    const int reach = margin + 3;
    int status = stream_pass(G, vel, A, P, out, nthreads, x0, x1, x0 - reach, x1 + reach, faces);
    if (!correction) return status;
    const int xa = std::max(0, x0 - margin), xb = std::min(nx, x1 + margin);
    std::vector<real> c(n, 0.0), c2(n, 0.0);
    P.zero_velocity = 1; P.use_integral = 0; P.psi_mode = PSI_PLAIN;
    status |= stream_pass(G, vel, A, P, c.data(), nthreads, xa, xb, xa - 3, xb + 3, nullptr);
    for (long i = xa * plane; i < xb * plane; ++i) c[i] = rho[i] - c[i];
    Field C = A; C.a = c.data();
    P.zero_velocity = 0; P.interp = I_1DY_LINEAR;
    split_offsets(-1, 1, split_off, P.color_off);
    status |= stream_pass(G, vel, C, P, c2.data(), nthreads, x0, x1, xa, xb, nullptr);
    for (long i = x0 * plane; i < x1 * plane; ++i) out[i] += c2[i];
    return status;
}
