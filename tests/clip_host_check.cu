// Host check of the FP32 face clipper (csrc/fia_clip32.cuh): the shared-pool clipper
// (clip32_fast, as k_clip32 runs it) against the local-memory clipper (clip32, as
// k_clip32_deferred runs it) on seeded random faces, compiled for the host from the library's
// own header.  For every face the fast clipper accepts, the pieces, their order, the
// piece count, the both-sides flag and the y-normal sums must be bitwise equal; a slot or
// stack word outside the shared pool stops the program (the host bounds checks of FastPool).
//
// Faces: the three face families and four staggerings, corners displaced by a common
// translation of up to `cfl` cells plus a per-corner perturbation (rigid, mildly deformed,
// strongly deformed so that polygons turn non-convex), translations rounded to half cells in a
// share of the cases (iso-lines through vertices and edges), both colour offsets, and
// minimal areas that triangulate pieces in a share of the cases.
//
// usage: clip_host_check [faces] [seed]; prints one summary line, exit status 1 on a mismatch.
// clip_host_check dump <faces file> <pieces file>: the local-memory clipper on given faces.
// clip_host_check status: faces that must set a status bit (non-finite, overflowing).
#include "../flux-interpolated-advection_gb300/csrc/fia_clip32.cuh"

#include <cstdint>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

using namespace fia;

namespace {

struct Result {
    bool ok = true;
    int npieces = 0, n = 0, nfwd = 0;
    bool multi = false;
    unsigned st = 0;
    float N = 0.f, Nr = 0.f;
    float4 p[kMaxPieces32];
};

LocalFace make_face(std::mt19937_64& rng, int fam, int comp, float cfl, float def, bool half) {
    std::uniform_real_distribution<float> U(-1.f, 1.f);
    static const int cx[3][4] = {{0, 0, 0, 0}, {0, 0, 1, 1}, {0, 1, 1, 0}};
    static const int cy[3][4] = {{0, 1, 1, 0}, {0, 0, 0, 0}, {0, 0, 1, 1}};
    static const int cz[3][4] = {{0, 0, 1, 1}, {0, 1, 1, 0}, {0, 0, 0, 0}};
    float T[3] = {cfl * U(rng), cfl * U(rng), cfl * U(rng)};
    if (half)
        for (float& t : T) t = 0.5f * std::nearbyint(2.f * t);
    const float s[3] = {comp == 0 ? -0.5f : 0.f, comp == 1 ? -0.5f : 0.f, comp == 2 ? -0.5f : 0.f};
    LocalFace g;
    g.anc[0] = g.anc[1] = g.anc[2] = 0;
    for (int q = 0; q < 4; ++q) {
        g.x[q] = float(cx[fam][q]) + s[0] + T[0] + def * U(rng);
        g.y[q] = float(cy[fam][q]) + s[1] + T[1] + def * U(rng);
        g.z[q] = float(cz[fam][q]) + s[2] + T[2] + def * U(rng);
    }
    return g;
}

// k_clip32_deferred's sequence
Result slow(const PassDesc& d, const LocalFace& g) {
    Result r;
    PieceSink sink;
    clip32(d, g, r.st, r.npieces, r.multi, sink);
    r.nfwd = sink.n;
    r.N = sink.ny.value();
    r.Nr = -r.N;
    if (r.multi) {
        int np2 = 0;
        bool m2 = false;
        sink.ny = Kahan();
        clip32(d, reversed_face(g), r.st, np2, m2, sink);
        r.Nr = sink.ny.value();
    }
    r.n = sink.n;
    for (int q = 0; q < sink.n; ++q) r.p[q] = sink.p[q];
    return r;
}

// k_clip32's sequence on thread 0's slice of a CTA's pool
Result fast(const PassDesc& d, const LocalFace& g, std::vector<float>& pool) {
    Result r;
    const FastPool P{pool.data()};
    Kahan ny;
    int nst = 0;
    r.ok = clip32_fast(d, g, r.npieces, r.multi, nst, ny, P);
    if (r.ok) {
        r.nfwd = nst;
        r.N = ny.value();
        r.Nr = -r.N;
        if (r.multi) {
            ny = Kahan();
            int np2 = 0;
            bool m2 = false;
            r.ok = clip32_fast(d, reversed_face(g), np2, m2, nst, ny, P);
            r.Nr = ny.value();
        }
    }
    r.n = nst;
    for (int q = 0; q < nst && r.ok; ++q) {
        const int e = kFastR - 1 - q;
        r.p[q] = make_float4(P.at(e, 0), P.at(e, 1), P.at(e, 2), P.at(e, 3));
    }
    return r;
}

bool same_bits(float a, float b) { return std::memcmp(&a, &b, sizeof(float)) == 0; }

}  // namespace

// dump mode: faces from a file (per face 12 floats: x, y, z of the four corners in cells, then
// the two colour offsets and the minimal area), the local-memory clipper's result to a file
// (per face: int pieces, int both-sides flag, float N, float Nr, then cx, cy, cz, ny per piece)
int dump(const char* in_path, const char* out_path) {
    FILE* fi = std::fopen(in_path, "rb");
    FILE* fo = std::fopen(out_path, "wb");
    if (!fi || !fo) return 2;
    float rec[15];
    while (std::fread(rec, sizeof(float), 15, fi) == 15) {
        PassDesc d;
        std::memset(&d, 0, sizeof(d));
        d.color_off_f[0] = rec[12];
        d.color_off_f[1] = rec[13];
        d.minimal_area_f = rec[14];
        LocalFace g;
        g.anc[0] = g.anc[1] = g.anc[2] = 0;
        for (int q = 0; q < 4; ++q) { g.x[q] = rec[3 * q]; g.y[q] = rec[3 * q + 1]; g.z[q] = rec[3 * q + 2]; }
        const Result r = slow(d, g);
        const int hd[2] = {r.n, r.multi ? 1 : 0};
        const float nn[2] = {r.N, r.Nr};
        std::fwrite(hd, sizeof(int), 2, fo);
        std::fwrite(nn, sizeof(float), 2, fo);
        std::fwrite(r.p, sizeof(float4), r.n, fo);
    }
    std::fclose(fi);
    return std::fclose(fo) == 0 ? 0 : 2;
}

// status mode: faces that must set a status bit, each clipped by both stores; prints per face
// "name st pieces fast_ok" (fast_ok: the shared-pool clipper accepted the face).  The process
// ending at all is part of the check: no clip loop may depend on a non-finite colour.
int status_cases() {
    const float nan = std::numeric_limits<float>::quiet_NaN(), inf = std::numeric_limits<float>::infinity();
    struct Case { const char* name; float x[4], y[4], z[4]; };
    // y-faces (corners in the order of face family 1) in cells
    const Case cases[] = {
        {"normal", {0.3f, 0.3f, 1.3f, 1.3f}, {0.f, 0.f, 0.f, 0.f}, {0.2f, 1.2f, 1.2f, 0.2f}},
        {"nan_x", {0.3f, 0.3f, nan, 1.3f}, {0.f, 0.f, 0.f, 0.f}, {0.2f, 1.2f, 1.2f, 0.2f}},
        {"nan_y", {0.3f, 0.3f, 1.3f, 1.3f}, {0.f, nan, 0.f, 0.f}, {0.2f, 1.2f, 1.2f, 0.2f}},
        {"inf_z", {0.3f, 0.3f, 1.3f, 1.3f}, {0.f, 0.f, 0.f, 0.f}, {0.2f, inf, 1.2f, 0.2f}},
        {"neg_inf_x", {-inf, 0.3f, 1.3f, 1.3f}, {0.f, 0.f, 0.f, 0.f}, {0.2f, 1.2f, 1.2f, 0.2f}},
        {"all_nan", {nan, nan, nan, nan}, {nan, nan, nan, nan}, {nan, nan, nan, nan}},
        // 12 x 12 cells: 144 pieces, more than a face's piece store holds
        {"stretched", {0.f, 0.f, 12.f, 12.f}, {0.f, 0.f, 0.f, 0.f}, {0.f, 12.f, 12.f, 0.f}},
        // finite but absurd colours (10^7 cells): the clip stops when the store is full
        {"huge", {0.f, 0.f, 1.e7f, 1.e7f}, {0.f, 0.f, 0.f, 0.f}, {0.f, 0.6f, 0.6f, 0.f}},
    };
    std::vector<float> pool((size_t)kFastWords * kClipThreads, 0.f);
    for (const Case& c : cases) {
        PassDesc d;
        std::memset(&d, 0, sizeof(d));
        d.color_off_f[0] = 0.5f; d.color_off_f[1] = 0.5f; d.minimal_area_f = 1.0f;
        LocalFace g;
        g.anc[0] = g.anc[1] = g.anc[2] = 0;
        for (int q = 0; q < 4; ++q) { g.x[q] = c.x[q]; g.y[q] = c.y[q]; g.z[q] = c.z[q]; }
        const Result a = slow(d, g);
        const Result b = fast(d, g, pool);
        std::printf("%s %u %d %d\n", c.name, a.st, a.n, b.ok ? 1 : 0);
    }
    return 0;
}

int main(int argc, char** argv) {
    if (argc == 4 && std::strcmp(argv[1], "dump") == 0) return dump(argv[2], argv[3]);
    if (argc == 2 && std::strcmp(argv[1], "status") == 0) return status_cases();
    const long long faces = argc > 1 ? std::atoll(argv[1]) : 200000;
    const unsigned long long seed = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    std::mt19937_64 rng(seed);
    std::vector<float> pool((size_t)kFastWords * kClipThreads, 0.f);
    long long accepted = 0, listed = 0, mismatches = 0, multi = 0, pieces = 0, flagged = 0;
    static const float cfls[4] = {0.f, 1.f, 2.f, 4.f};
    static const float defs[4] = {0.f, 0.02f, 0.2f, 0.8f};
    for (long long t = 0; t < faces; ++t) {
        PassDesc d;
        std::memset(&d, 0, sizeof(d));
        d.color_off_f[0] = (rng() & 1) ? 0.5f : 0.f;
        d.color_off_f[1] = (rng() & 1) ? 0.5f : 0.f;
        d.minimal_area_f = (rng() % 8 == 0) ? 0.05f : 1.0f;
        const int fam = (int)(rng() % 3), comp = (int)(rng() % 4) - 1;
        const float cfl = cfls[rng() % 4], def = defs[rng() % 4];
        const bool half = rng() % 4 == 0;
        const LocalFace g = make_face(rng, fam, comp, cfl, def, half);
        const Result a = slow(d, g);
        const Result b = fast(d, g, pool);
        if (!b.ok) { ++listed; continue; }
        ++accepted;
        multi += a.multi ? 1 : 0;
        pieces += a.n;
        flagged += a.st != 0 ? 1 : 0;
        bool eq = a.npieces == b.npieces && a.n == b.n && a.nfwd == b.nfwd && a.multi == b.multi && a.st == 0 &&
                  same_bits(a.N, b.N) && same_bits(a.Nr, b.Nr);
        for (int q = 0; eq && q < a.n; ++q)
            eq = same_bits(a.p[q].x, b.p[q].x) && same_bits(a.p[q].y, b.p[q].y) && same_bits(a.p[q].z, b.p[q].z) &&
                 same_bits(a.p[q].w, b.p[q].w);
        if (!eq) {
            if (mismatches < 5)
                std::fprintf(stderr, "mismatch at face %lld: fam %d comp %d pieces %d/%d multi %d/%d st %u\n", t, fam,
                             comp, a.n, b.n, (int)a.multi, (int)b.multi, a.st);
            ++mismatches;
        }
    }
    std::printf("faces %lld accepted %lld listed %lld mismatches %lld multi %lld pieces %lld flagged %lld\n", faces,
                accepted, listed, mismatches, multi, pieces, flagged);
    return mismatches == 0 ? 0 : 1;
}
