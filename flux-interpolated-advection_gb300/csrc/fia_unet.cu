// fia_unet.cu -- the learned preconditioner's U-Net: convolution kernels (forward, backward
// data, backward weights) on the tensor cores, the fine-grid pieces of the two-level
// preconditioner (restriction, prolongation, energy-norm loss), Adam, and the host side.
// Layout, layer table and the formula of the preconditioner: fia_unet.cuh.
#include "fia_unet.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>

namespace fia {
namespace unet {

// ---------------------------------------------------------------------------------
// layer table
// ---------------------------------------------------------------------------------
enum TensorId : int {
    T_X0 = 0, T_A0, T_S0, T_A1, T_S1, T_A2, T_S2, T_A3, T_B3, T_U2, T_C2, T_U1, T_C1, T_U0, T_C0, T_Y
};
enum InMode : int { IN_PLAIN = 0, IN_POOL = 1, IN_UPCAT = 2, IN_SCALAR = 3 };

struct LayerDef {
    LayerShape shape;
    int mode;      // how the input is formed
    int in0, in1;  // IN_UPCAT: in0 is upsampled (coarse), in1 the skip tensor
    int out;
};

static const LayerDef kDefs[kLayers] = {
    {{0, 1, 16, 1}, IN_SCALAR, T_X0, -1, T_A0},
    {{0, 16, 16, 1}, IN_PLAIN, T_A0, -1, T_S0},
    {{1, 16, 32, 1}, IN_POOL, T_S0, -1, T_A1},
    {{1, 32, 32, 1}, IN_PLAIN, T_A1, -1, T_S1},
    {{2, 32, 48, 1}, IN_POOL, T_S1, -1, T_A2},
    {{2, 48, 48, 1}, IN_PLAIN, T_A2, -1, T_S2},
    {{3, 48, 64, 1}, IN_POOL, T_S2, -1, T_A3},
    {{3, 64, 64, 1}, IN_PLAIN, T_A3, -1, T_B3},
    {{2, 112, 48, 1}, IN_UPCAT, T_B3, T_S2, T_U2},
    {{2, 48, 48, 1}, IN_PLAIN, T_U2, -1, T_C2},
    {{1, 80, 32, 1}, IN_UPCAT, T_C2, T_S1, T_U1},
    {{1, 32, 32, 1}, IN_PLAIN, T_U1, -1, T_C1},
    {{0, 48, 16, 1}, IN_UPCAT, T_C1, T_S0, T_U0},
    {{0, 16, 16, 1}, IN_PLAIN, T_U0, -1, T_C0},
    {{0, 16, 1, 0}, IN_PLAIN, T_C0, -1, T_Y},
};
// level and channels of each tensor
static const int kTensorLevel[kTensors] = {0, 0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0};
static const int kTensorC[kTensors] = {1, 16, 16, 32, 32, 48, 48, 64, 64, 48, 48, 32, 32, 16, 16, 1};

const LayerShape& layer_shape(int l) { return kDefs[l].shape; }

long long layer_offset(int l) {
    long long o = 0;
    for (int i = 0; i < l; ++i) o += 27LL * kDefs[i].shape.cin * kDefs[i].shape.cout;
    return o;
}
long long num_parameters() { return layer_offset(kLayers) + 1; }   // + omega (last)

// ---------------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------------
constexpr int TX = 2, TY = 4, TZ = 16;          // output brick of one CTA (128 voxels)
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;
constexpr int HV = HX * HY * HZ;                // 432 halo voxels
constexpr int kConvThreads = 128;               // 4 warps x 2 lines of 16 voxels

enum SrcKind : int { SRC_BF16 = 1, SRC_BF16_UP = 2, SRC_BF16_POOL = 3, SRC_F32 = 4, SRC_F32_GATED = 5 };

struct Src {
    int kind;
    const void* p;
    const __nv_bfloat16* gate;   // SRC_F32_GATED: value x (gate > 0)
    int C, cstride, coff;        // channels taken; channel stride and offset in the tensor
    int gstride, goff;           // same for the gate tensor
    int dims[3];                 // grid of the source tensor
};

enum OutKind : int { OUT_BF16 = 0, OUT_F32 = 1 };

struct ConvArgs {
    Src s0, s1;
    int cin;              // staged channels (1: scalar input packed over taps)
    int dims[3];          // grid of the convolution (output = input grid)
    const uint2* wfrag;   // weights in fragment order
    const uint4* wtc;     // forward weights for k_conv_tc, (tap, unit, n) x 8 channels; null: not eligible
    int out_kind;
    void* out;
    int out_cstride, out_coff, cout_real;
    int relu;
    int nt;               // n-tiles (8 output channels) of the weight fragments
    int nsplit;           // CTAs sharing one brick, each with nt / nsplit n-tiles
};

__device__ __forceinline__ int swz(int u) { return (u & ~7) | ((u ^ (u >> 3)) & 7); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);   // .x = lo (low 16 bits)
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ long long vox(const int* d, int x, int y, int z) {
    return ((long long)x * d[1] + y) * d[2] + z;
}

// 8 channels [c, c+8) of source s at voxel (x,y,z) of the convolution's grid, as bf16x8
__device__ uint4 load_unit(const Src& s, int x, int y, int z, int c) {
    float f[8];
    switch (s.kind) {
        case SRC_BF16:
        case SRC_BF16_UP: {
            if (s.kind == SRC_BF16_UP) { x >>= 1; y >>= 1; z >>= 1; }
            const __nv_bfloat16* p = (const __nv_bfloat16*)s.p + vox(s.dims, x, y, z) * s.cstride + s.coff + c;
            return *reinterpret_cast<const uint4*>(p);
        }
        case SRC_BF16_POOL: {
            for (int i = 0; i < 8; ++i) f[i] = 0.f;
            int cnt = 0;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    for (int k = 0; k < 2; ++k) {
                        const int cx = 2 * x + i, cy = 2 * y + j, cz = 2 * z + k;
                        if (cx >= s.dims[0] || cy >= s.dims[1] || cz >= s.dims[2]) continue;
                        const uint4 u = *reinterpret_cast<const uint4*>(
                            (const __nv_bfloat16*)s.p + vox(s.dims, cx, cy, cz) * s.cstride + s.coff + c);
                        const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
                        for (int q = 0; q < 4; ++q) {
                            const float2 t = __bfloat1622float2(h[q]);
                            f[2 * q] += t.x; f[2 * q + 1] += t.y;
                        }
                        ++cnt;
                    }
            const float inv = 1.f / (float)cnt;
            for (int i = 0; i < 8; ++i) f[i] *= inv;
            break;
        }
        default: {   // SRC_F32, SRC_F32_GATED
            const long long v = vox(s.dims, x, y, z);
            const float4* p = reinterpret_cast<const float4*>((const float*)s.p + v * s.cstride + s.coff + c);
            const float4 a = p[0], b = p[1];
            f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w; f[4] = b.x; f[5] = b.y; f[6] = b.z; f[7] = b.w;
            if (s.kind == SRC_F32_GATED) {
                const uint4 u = *reinterpret_cast<const uint4*>(s.gate + v * s.gstride + s.goff + c);
                const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&u);
                for (int i = 0; i < 8; ++i)
                    if (!(__bfloat162float(h[i]) > 0.f)) f[i] = 0.f;
            }
        }
    }
    uint4 r;
    r.x = pack_bf16(f[0], f[1]); r.y = pack_bf16(f[2], f[3]); r.z = pack_bf16(f[4], f[5]); r.w = pack_bf16(f[6], f[7]);
    return r;
}

// one scalar (channel 0) of an fp32 source at (x,y,z)
__device__ __forceinline__ float load_scalar(const Src& s, int x, int y, int z) {
    return ((const float*)s.p)[vox(s.dims, x, y, z) * s.cstride + s.coff];
}

// Stages the halo brick of the convolution input (channels-last, swizzled 16-byte units).
__device__ void stage_units(const ConvArgs& a, uint4* sm, int bx, int by, int bz) {
    const int ncu = a.cin >> 3;
    const int total = HV * ncu;
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int hv = u / ncu, cu = u - hv * ncu;
        const int hz = hv % HZ, hy = (hv / HZ) % HY, hx = hv / (HZ * HY);
        const int x = bx + hx - 1, y = by + hy - 1, z = bz + hz - 1;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (x >= 0 && y >= 0 && z >= 0 && x < a.dims[0] && y < a.dims[1] && z < a.dims[2]) {
            const int c = cu << 3;
            val = c < a.s0.C ? load_unit(a.s0, x, y, z, c) : load_unit(a.s1, x, y, z, c - a.s0.C);
        }
        sm[swz(u)] = val;
    }
}

__device__ void stage_scalars(const ConvArgs& a, __nv_bfloat16* sm, int bx, int by, int bz) {
    for (int hv = threadIdx.x; hv < HV; hv += blockDim.x) {
        const int hz = hv % HZ, hy = (hv / HZ) % HY, hx = hv / (HZ * HY);
        const int x = bx + hx - 1, y = by + hy - 1, z = bz + hz - 1;
        float v = 0.f;
        if (x >= 0 && y >= 0 && z >= 0 && x < a.dims[0] && y < a.dims[1] && z < a.dims[2]) v = load_scalar(a.s0, x, y, z);
        sm[hv] = __float2bfloat16_rn(v);
    }
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void tap_offsets(int tap, int& dx, int& dy, int& dz) {
    dx = tap / 9; dy = (tap / 3) % 3; dz = tap % 3;
}

// ---------------------------------------------------------------------------------
// convolution (forward; backward data with flipped/transposed weights): a CTA of 4 warps computes a brick of MT x 4 x 16 output voxels
// (warp w: the MT z-lines at y = w) and NTL n-tiles of output channels (the n-tiles of a
// layer are split over nsplit CTAs on the coarse levels, where a brick per CTA would leave
// the GPU nearly empty).  The halo brick is staged channels-last with an odd number of
// 16-byte units per voxel, so the 8 rows of an ldmatrix (8 consecutive voxels) fall into 8
// different bank groups; plain and upsampled BF16 sources are copied with cp.async (zero
// fill outside the grid).
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::); }

__host__ __device__ __forceinline__ int odd_units(int cin) { return (cin >> 3) | 1; }

__device__ __forceinline__ void stage_one(const Src& src, int x, int y, int z, int c, bool in, uint32_t dst,
                                          uint4* dptr) {
    if (src.kind == SRC_BF16 || src.kind == SRC_BF16_UP) {
        int sx = x, sy = y, sz = z;
        if (src.kind == SRC_BF16_UP) { sx >>= 1; sy >>= 1; sz >>= 1; }
        const __nv_bfloat16* gp = (const __nv_bfloat16*)src.p;
        if (in) gp += vox(src.dims, sx, sy, sz) * src.cstride + src.coff + c;
        cp_async16(dst, gp, in ? 16 : 0);
    } else {
        *dptr = in ? load_unit(src, x, y, z, c) : make_uint4(0, 0, 0, 0);
    }
}

template <int MT>
__device__ void stage2(const ConvArgs& a, uint4* sm, int bx, int by, int bz) {
    constexpr int HY = 6, HZ = 18, HV = (MT + 2) * HY * HZ;
    const int ncu = a.cin >> 3, ncp = odd_units(a.cin);
    const int total = HV * ncu;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int hv = u / ncu, cu = u - hv * ncu;
        const int hz = hv % HZ, hy = (hv / HZ) % HY, hx = hv / (HZ * HY);
        const int x = bx + hx - 1, y = by + hy - 1, z = bz + hz - 1;
        const bool in = x >= 0 && y >= 0 && z >= 0 && x < a.dims[0] && y < a.dims[1] && z < a.dims[2];
        const int c = cu << 3, su = hv * ncp + cu;
        if (c < a.s0.C) stage_one(a.s0, x, y, z, c, in, sbase + su * 16, sm + su);
        else stage_one(a.s1, x, y, z, c - a.s0.C, in, sbase + su * 16, sm + su);
    }
}

template <int MT>
__device__ void stage2_scalar(const ConvArgs& a, __nv_bfloat16* sm, int bx, int by, int bz) {
    constexpr int HY = 6, HZ = 18, HV = (MT + 2) * HY * HZ;
    for (int hv = threadIdx.x; hv < HV; hv += blockDim.x) {
        const int hz = hv % HZ, hy = (hv / HZ) % HY, hx = hv / (HZ * HY);
        const int x = bx + hx - 1, y = by + hy - 1, z = bz + hz - 1;
        float v = 0.f;
        if (x >= 0 && y >= 0 && z >= 0 && x < a.dims[0] && y < a.dims[1] && z < a.dims[2]) v = load_scalar(a.s0, x, y, z);
        sm[hv] = __float2bfloat16_rn(v);
    }
}

template <int NTL, int MT, bool TAP>
__global__ void __launch_bounds__(kConvThreads) k_conv2(ConvArgs a) {
    extern __shared__ __align__(128) uint4 smem[];
    constexpr int HY = 6, HZ = 18;
    const int nsplit = a.nsplit;
    const int zb = blockIdx.x / nsplit, part = blockIdx.x - zb * nsplit;
    const int n0 = part * NTL;
    const int bz = zb * 16, by = blockIdx.y * 4, bx = blockIdx.z * MT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NT = a.nt;
    if (TAP) stage2_scalar<MT>(a, reinterpret_cast<__nv_bfloat16*>(smem), bx, by, bz);
    else stage2<MT>(a, smem, bx, by, bz);
    cp_async_wait_all();
    __syncthreads();

    float acc[MT][NTL][4];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int n = 0; n < NTL; ++n)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[m][n][e] = 0.f;

    if (!TAP) {
        const int nc16 = a.cin >> 4, ncp = odd_units(a.cin);
        const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
        const int j = lane >> 3, i = lane & 7;
        const int m = i + ((j & 1) << 3), ku = j >> 1;
        for (int tap = 0; tap < 27; ++tap) {
            int dx, dy, dz;
            tap_offsets(tap, dx, dy, dz);
            uint32_t addr[MT];
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                const int hv = ((mt + dx) * HY + (warp + dy)) * HZ + m + dz;
                addr[mt] = sbase + (uint32_t)(hv * ncp + ku) * 16u;
            }
            const uint2* wt = a.wfrag + ((size_t)tap * nc16 * NT + n0) * 32 + lane;
            for (int c16 = 0; c16 < nc16; ++c16) {
                uint32_t A[MT][4];
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) ldsm_x4(A[mt], addr[mt] + c16 * 32);
#pragma unroll
                for (int n = 0; n < NTL; ++n) {
                    const uint2 b = __ldg(wt + (c16 * NT + n) * 32);
#pragma unroll
                    for (int mt = 0; mt < MT; ++mt) mma_bf16(acc[mt][n], A[mt], b.x, b.y);
                }
            }
        }
    } else {
        const unsigned short* shu = reinterpret_cast<const unsigned short*>(smem);
        const int g = lane >> 2, q = lane & 3;
        for (int kc = 0; kc < 2; ++kc) {
            int off[4];
            bool ok[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int k = (t < 2 ? 2 * q + t : 2 * q + 8 + (t - 2));
                const int tap = 16 * kc + k;
                ok[t] = tap < 27;
                int dx, dy, dz;
                tap_offsets(ok[t] ? tap : 0, dx, dy, dz);
                off[t] = (dx * HY + dy) * HZ + dz;
            }
            uint32_t A[MT][4];
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                const int base = (mt * HY + warp) * HZ;
                auto v = [&](int row, int t) -> uint32_t { return ok[t] ? (uint32_t)shu[base + row + off[t]] : 0u; };
                A[mt][0] = v(g, 0) | (v(g, 1) << 16);
                A[mt][1] = v(g + 8, 0) | (v(g + 8, 1) << 16);
                A[mt][2] = v(g, 2) | (v(g, 3) << 16);
                A[mt][3] = v(g + 8, 2) | (v(g + 8, 3) << 16);
            }
#pragma unroll
            for (int n = 0; n < NTL; ++n) {
                const uint2 b = __ldg(a.wfrag + (kc * NT + n0 + n) * 32 + lane);
#pragma unroll
                for (int mt = 0; mt < MT; ++mt) mma_bf16(acc[mt][n], A[mt], b.x, b.y);
            }
        }
    }

    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
        const int x = bx + mt, y = by + warp;
        if (x >= a.dims[0] || y >= a.dims[1]) continue;
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
            const int z = bz + g + 8 * hf;
            if (z >= a.dims[2]) continue;
            const long long v = vox(a.dims, x, y, z);
#pragma unroll
            for (int n = 0; n < NTL; ++n) {
                const int c = (n0 + n) * 8 + 2 * q;
                if (c >= a.cout_real) continue;
                float v0 = acc[mt][n][2 * hf], v1 = acc[mt][n][2 * hf + 1];
                if (a.relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                if (a.out_kind == OUT_BF16) {
                    __nv_bfloat16* o = (__nv_bfloat16*)a.out + v * a.out_cstride + a.out_coff + c;
                    *reinterpret_cast<uint32_t*>(o) = pack_bf16(v0, v1);
                } else {
                    float* o = (float*)a.out + v * a.out_cstride + a.out_coff + c;
                    if (a.cout_real == 1) o[0] = v0;
                    else *reinterpret_cast<float2*>(o) = make_float2(v0, v1);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// forward convolution on the 5th-generation tensor cores: tcgen05.mma (BF16 operands in
// shared memory, FP32 accumulators in tensor memory).
//
// A CTA computes TXC tiles of M = 128 output voxels, each an x-plane of 16 y-lines x 8 z-voxels,
// for all N output channels (N = 16..64).  The halo brick (TXC+2) x 18 x 10 is staged
// unit-major: 16-byte unit u (8 channels) of halo voxel hv at (u * HVP + hv) * 16, HVP odd so
// that the staging writes of consecutive units spread over the banks.  In this layout the A
// operand of every tap is the canonical K-major, no-swizzle layout at a shifted start
// address: rows m = 8 ly + lz, the 8 rows of a core matrix are one z-line (16 bytes apart),
// the 8-row groups are the y-lines (SBO = 10 voxels = 160 bytes), the K chunks are the units
// (LBO = HVP * 16).  The weights (B = N x K per tap, K-major) are laid out (tap, unit, n) x 16
// bytes (SBO = 128, LBO = N * 16) and streamed in chunks of TPC taps through two shared
// buffers by one-dimensional bulk copies (cp.async.bulk, completion counted in bytes on the
// buffer's "full" mbarrier).  Thread 0 issues the MMAs of a chunk once its buffer is full and
// commits them to the buffer's "empty" mbarrier, which thread 32 waits on before refilling
// the buffer.  The CTA has 256 or 512 threads (8 or 16 warps, for the halo staging); the
// epilogue reads the accumulators with tcgen05.ld (warps w, w + 4, ...: TMEM lanes 32 (w mod 4)
// .. + 31 = rows, splitting the 16-column blocks), applies ReLU and stores BF16 channels-last.
//
// Every wait is bounded; on a timeout the kernel sets bit 0 of *status, skips the epilogue
// and still frees its tensor memory.
// ---------------------------------------------------------------------------------
constexpr int TCY = 16, TCZ = 8, HCY = TCY + 2, HCZ = TCZ + 2;
constexpr int kTcThreadsMax = 512;
constexpr int kTcWaitLimit = 1 << 22;
constexpr size_t kTcSmemBudget = 110 * 1024;   // two CTAs per SM
constexpr int kTcSmemMax = 112 * 1024;

__host__ __device__ constexpr int tc_hvp(int txc) { return ((txc + 2) * HCY * HCZ) | 1; }

__device__ __forceinline__ uint64_t umma_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);   // descriptor version of tcgen05; base offset 0, no swizzle
}
// kind::f16 instruction descriptor: FP32 accumulate, BF16 A and B, both K-major, M = 128
__host__ __device__ __forceinline__ uint32_t umma_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}
__device__ __forceinline__ bool mbar_wait(uint32_t mb, uint32_t parity) {
    for (int it = 0; it < kTcWaitLimit; ++it) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, q;\n\t}"
                     : "=r"(done) : "r"(mb), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

template <int TXC, int NU, int THREADS>
__global__ void __launch_bounds__(THREADS) k_conv_tc(ConvArgs a, int n_out, int tpc, unsigned* status) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    __shared__ __align__(8) uint64_t bar_full[2], bar_empty[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int failed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int nu = NU, hvp = tc_hvp(TXC);   // NU = cin / 8
    const int bz = blockIdx.x * TCZ, by = blockIdx.y * TCY, bx = blockIdx.z * TXC;
    const uint32_t halo = (uint32_t)__cvta_generic_to_shared(tsm);
    const uint32_t halo_bytes = ((uint32_t)(hvp * nu * 16) + 127u) & ~127u;
    const uint32_t chunk_bytes = (uint32_t)(tpc * nu * n_out * 16);
    const uint32_t wbuf0 = halo + halo_bytes;
    const int nchunks = (27 + tpc - 1) / tpc;
    uint32_t ncols = 32;
    while (ncols < (uint32_t)(TXC * n_out)) ncols <<= 1;

    if (warp == 0) {
        const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&tmem_slot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        failed = 0;
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&bar_full[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&bar_empty[b])));
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tbase = tmem_slot;
    // weight chunk c into buffer c & 1 (one thread), completion counted on the buffer's full barrier
    const unsigned char* wg = reinterpret_cast<const unsigned char*>(a.wtc);
    auto issue_chunk = [&](int c) {
        const int b = c & 1;
        const uint32_t full = (uint32_t)__cvta_generic_to_shared(&bar_full[b]);
        const int t0 = c * tpc, nt = min(tpc, 27 - t0);
        const uint32_t bytes = (uint32_t)(nt * nu * n_out * 16);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(wbuf0 + (uint32_t)b * chunk_bytes), "l"(wg + (size_t)t0 * nu * n_out * 16), "r"(bytes),
                     "r"(full)
                     : "memory");
    };
    // the first two chunks load while the halo is staged
    if (tid == 32) for (int c = 0; c < min(2, nchunks); ++c) issue_chunk(c);
    // halo: plain and upsampled BF16 by cp.async (zero fill outside the grid), the rest computed
    const int total = ((TXC + 2) * HCY * HCZ) * nu;
    for (int i = tid; i < total; i += THREADS) {
        const int hv = i / nu, u = i - hv * nu;
        const int hz = hv % HCZ, hy = (hv / HCZ) % HCY, hx = hv / (HCZ * HCY);
        const int x = bx + hx - 1, y = by + hy - 1, z = bz + hz - 1;
        const bool in = x >= 0 && y >= 0 && z >= 0 && x < a.dims[0] && y < a.dims[1] && z < a.dims[2];
        const int c = u << 3;
        const uint32_t off = (uint32_t)(u * hvp + hv) * 16u;
        uint4* dptr = reinterpret_cast<uint4*>(tsm + off);
        if (c < a.s0.C) stage_one(a.s0, x, y, z, c, in, halo + off, dptr);
        else stage_one(a.s1, x, y, z, c - a.s0.C, in, halo + off, dptr);
    }
    cp_async_wait_all();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();

    if (tid == 32) {
        // producer: the remaining chunks, each once the MMAs of the chunk two before are done
        for (int c = 2; c < nchunks; ++c) {
            if (!mbar_wait((uint32_t)__cvta_generic_to_shared(&bar_empty[c & 1]), (uint32_t)((c >> 1) - 1) & 1u)) {
                failed = 1;
                break;
            }
            issue_chunk(c);
        }
    } else if (tid == 0) {
        // MMA issue.  The descriptors of the halo and of each weight buffer are built once; an
        // operand at a later address adds its offset in 16-byte units to the start-address
        // field (shared addresses stay below 256 KB, so the 14-bit field does not overflow).
        const uint32_t idesc = umma_idesc(n_out);
        const uint64_t adesc0 = umma_sdesc(halo, (uint32_t)hvp * 16u, HCZ * 16u);
        for (int c = 0; c < nchunks; ++c) {
            const int b = c & 1;
            if (!mbar_wait((uint32_t)__cvta_generic_to_shared(&bar_full[b]), (uint32_t)(c >> 1) & 1u)) {
                failed = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int t0 = c * tpc, nt = min(tpc, 27 - t0);
            const uint64_t bdesc0 = umma_sdesc(wbuf0 + (uint32_t)b * chunk_bytes, (uint32_t)n_out * 16u, 128u);
            for (int tl = 0; tl < nt; ++tl) {
                const int tap = t0 + tl;
                const int dx = tap / 9, dy = (tap / 3) % 3, dz = tap % 3;
                const uint32_t hvt = (uint32_t)((dx * HCY + dy) * HCZ + dz);
#pragma unroll
                for (int ks = 0; ks < NU / 2; ++ks) {
                    const uint64_t bd = bdesc0 + (uint64_t)((tl * NU + 2 * ks) * n_out);
                    const uint32_t acc = (tap > 0 || ks > 0) ? 1u : 0u;
#pragma unroll
                    for (int tx = 0; tx < TXC; ++tx) {
                        const uint64_t ad = adesc0 + (uint64_t)(2 * ks * hvp + hvt + tx * HCY * HCZ);
                        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                                     ::"r"(tbase + (uint32_t)(tx * n_out)), "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                                     : "memory");
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"((uint32_t)__cvta_generic_to_shared(&bar_empty[b]))
                         : "memory");
        }
    }
    __syncthreads();
    // all MMAs complete: the last chunk's commit tracks every earlier MMA of thread 0; the
    // decision is made block-wide (tcgen05.ld is warp-collective)
    bool ok = !failed;
    if (ok) {
        const int cl = nchunks - 1;
        ok = mbar_wait((uint32_t)__cvta_generic_to_shared(&bar_empty[cl & 1]), (uint32_t)(cl >> 1) & 1u);
    }
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok) {
        if (lane == 0) atomicOr(status, 1u);
    } else {
        // warp w reads TMEM lanes 32 (w mod 4) ..; the warp groups split the 16-column blocks
        const int q4 = warp & 3, grp = warp >> 2;
        const int m = q4 * 32 + lane, ly = m >> 3, lz = m & 7;
        const int y = by + ly, z = bz + lz;
        const int nblk = n_out >> 4;
        for (int item = grp; item < TXC * nblk; item += THREADS / 128) {
            const int tx = item / nblk, c0 = (item - tx * nblk) * 16;
            const int x = bx + tx;
            const bool st = x < a.dims[0] && y < a.dims[1] && z < a.dims[2];
            const long long ov = st ? vox(a.dims, x, y, z) * a.out_cstride + a.out_coff : 0;
            {
                uint32_t r[16];
                const uint32_t ta = tbase + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(tx * n_out + c0);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                               "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                               "=r"(r[14]), "=r"(r[15])
                             : "r"(ta));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (st && a.out_kind == OUT_BF16) {
                    uint32_t pk[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float v0 = __uint_as_float(r[2 * j]), v1 = __uint_as_float(r[2 * j + 1]);
                        if (a.relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                        pk[j] = pack_bf16(v0, v1);
                    }
                    uint4* dst = reinterpret_cast<uint4*>((__nv_bfloat16*)a.out + ov + c0);
                    dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                } else if (st) {   // FP32 output of the first cout_real channels (the last layer)
                    float* dst = (float*)a.out + ov;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        if (c0 + j >= a.cout_real) break;
                        float v = __uint_as_float(r[j]);
                        if (a.relu) v = fmaxf(v, 0.f);
                        dst[c0 + j] = v;
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(ncols));
}

// ---------------------------------------------------------------------------------
// backward weights: dW[tap][ci][co] += sum_v x[v + off(tap)][ci] g[v][co]
// ---------------------------------------------------------------------------------
template <int COUT>
__global__ void __launch_bounds__(kConvThreads) k_wgrad(ConvArgs a, Src gs, float* __restrict__ dW) {
    extern __shared__ __align__(128) uint4 smem[];
    constexpr int GU = COUT / 8;
    const int bz = blockIdx.x * TZ, by = blockIdx.y * TY, bx = blockIdx.z * TX;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ncu = a.cin >> 3, nc16 = a.cin >> 4;
    const int xunits = ((HV * ncu + 7) / 8) * 8;
    stage_units(a, smem, bx, by, bz);
    uint4* gsm = smem + xunits;
    for (int u = threadIdx.x; u < TX * TY * TZ * GU; u += blockDim.x) {
        const int vrow = u / GU, cu = u - vrow * GU;
        const int L = vrow / TZ, z = vrow % TZ;
        const int x = bx + L / TY, y = by + L % TY, zz = bz + z;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (x < a.dims[0] && y < a.dims[1] && zz < a.dims[2]) val = load_unit(gs, x, y, zz, cu * 8);
        gsm[swz(u)] = val;
    }
    __syncthreads();
    const uint32_t xb = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t gb = (uint32_t)__cvta_generic_to_shared(gsm);
    const int j = lane >> 3, i = lane & 7;
    const int g = lane >> 2, q = lane & 3;
    const int nM = 27 * nc16;
    for (int mt = warp; mt < nM; mt += kConvThreads / 32) {
        const int tap = mt / nc16, c16 = mt - tap * nc16;
        int dx, dy, dz;
        tap_offsets(tap, dx, dy, dz);
        float acc[GU][4];
#pragma unroll
        for (int n = 0; n < GU; ++n)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[n][e] = 0.f;
        for (int L = 0; L < TX * TY; ++L) {
            const int lx = L / TY, ly = L % TY;
            uint32_t A[4];
            const int vrow = i + 8 * (j >> 1);
            const int hv = ((lx + dx) * HY + (ly + dy)) * HZ + vrow + dz;
            ldsm_x4_t(A, xb + swz(hv * ncu + 2 * c16 + (j & 1)) * 16);
#pragma unroll
            for (int n16 = 0; n16 < GU / 2; ++n16) {
                uint32_t B[4];
                const int vr = L * TZ + i + 8 * (j & 1);
                ldsm_x4_t(B, gb + swz(vr * GU + 2 * n16 + (j >> 1)) * 16);
                mma_bf16(acc[2 * n16], A, B[0], B[1]);
                mma_bf16(acc[2 * n16 + 1], A, B[2], B[3]);
            }
        }
#pragma unroll
        for (int n = 0; n < GU; ++n) {
            const int co = n * 8 + 2 * q;
            const int ci0 = c16 * 16 + g, ci1 = ci0 + 8;
            float* w0 = dW + ((size_t)tap * a.cin + ci0) * COUT + co;
            float* w1 = dW + ((size_t)tap * a.cin + ci1) * COUT + co;
            atomicAdd(w0, acc[n][0]); atomicAdd(w0 + 1, acc[n][1]);
            atomicAdd(w1, acc[n][2]); atomicAdd(w1 + 1, acc[n][3]);
        }
    }
}

// Weight gradient of the scalar-input (cin 1) and scalar-output (cout 1) layers on the FP32 pipe.
__global__ void __launch_bounds__(kConvThreads) k_wgrad_small(ConvArgs a, Src gs, int cout, float* __restrict__ dW) {
    extern __shared__ __align__(16) float fsm[];
    const int cin = a.cin;
    float* xs = fsm;                       // HV x cin
    float* gsh = fsm + HV * cin;           // 128 x cout
    const int bz = blockIdx.x * TZ, by = blockIdx.y * TY, bx = blockIdx.z * TX;
    for (int u = threadIdx.x; u < HV * cin; u += blockDim.x) {
        const int hv = u / cin, c = u - hv * cin;
        const int hz = hv % HZ, hy = (hv / HZ) % HY, hx = hv / (HZ * HY);
        const int x = bx + hx - 1, y = by + hy - 1, z = bz + hz - 1;
        float v = 0.f;
        if (x >= 0 && y >= 0 && z >= 0 && x < a.dims[0] && y < a.dims[1] && z < a.dims[2]) {
            if (a.s0.kind == SRC_F32) v = load_scalar(a.s0, x, y, z);
            else v = __bfloat162float(((const __nv_bfloat16*)a.s0.p)[vox(a.s0.dims, x, y, z) * a.s0.cstride + a.s0.coff + c]);
        }
        xs[u] = __bfloat162float(__float2bfloat16_rn(v));
    }
    for (int u = threadIdx.x; u < TX * TY * TZ * cout; u += blockDim.x) {
        const int vrow = u / cout, c = u - vrow * cout;
        const int L = vrow / TZ, z = vrow % TZ;
        const int x = bx + L / TY, y = by + L % TY, zz = bz + z;
        float v = 0.f;
        if (x < a.dims[0] && y < a.dims[1] && zz < a.dims[2]) {
            const long long o = vox(gs.dims, x, y, zz);
            v = ((const float*)gs.p)[o * gs.cstride + gs.coff + c];
            if (gs.kind == SRC_F32_GATED && !(__bfloat162float(gs.gate[o * gs.gstride + gs.goff + c]) > 0.f)) v = 0.f;
        }
        gsh[u] = __bfloat162float(__float2bfloat16_rn(v));
    }
    __syncthreads();
    const int nw = 27 * cin * cout;
    for (int w = threadIdx.x; w < nw; w += blockDim.x) {
        const int co = w % cout, ci = (w / cout) % cin, tap = w / (cout * cin);
        int dx, dy, dz;
        tap_offsets(tap, dx, dy, dz);
        float s = 0.f;
        for (int vrow = 0; vrow < TX * TY * TZ; ++vrow) {
            const int L = vrow / TZ, z = vrow % TZ;
            const int hv = ((L / TY + dx) * HY + (L % TY + dy)) * HZ + z + dz;
            s = fmaf(xs[hv * cin + ci], gsh[vrow * cout + co], s);
        }
        atomicAdd(dW + w, s);
    }
}

// ---------------------------------------------------------------------------------
// weights: FP32 master [tap][cin][cout] -> bf16 fragments
// ---------------------------------------------------------------------------------
// fwd: frag[(tap*nc16 + c16)*nt + n][lane] (unit input) or frag[(kc*nt + n)][lane] (scalar input)
// with transposed = 1 the layer is read as W'[t][co][ci] = W[26-t][ci][co] (backward data)
__global__ void k_pack(const float* __restrict__ W, int cin, int cout, int transposed, uint2* __restrict__ frag) {
    const int ci_n = transposed ? cout : cin;     // input channels of the packed convolution
    const int co_n = transposed ? cin : cout;
    const int nt = (co_n + 7) / 8;
    const bool scalar_in = ci_n == 1;
    const int nk = scalar_in ? 2 : 27 * (ci_n / 16);
    const int total = nk * nt * 32;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int lane = e & 31, n = (e >> 5) % nt, kk = (e >> 5) / nt;
        const int g = lane >> 2, q = lane & 3;
        const int co = n * 8 + g;
        auto wv = [&](int k) -> float {     // k within the 16-chunk kk
            int tap, ci;
            if (scalar_in) { tap = 16 * kk + k; ci = 0; if (tap >= 27) return 0.f; }
            else { const int nc16 = ci_n / 16; tap = kk / nc16; ci = (kk % nc16) * 16 + k; }
            if (co >= co_n) return 0.f;
            if (!transposed) return W[((size_t)tap * cin + ci) * cout + co];
            return W[((size_t)(26 - tap) * cin + co) * cout + ci];
        };
        uint2 r;
        r.x = pack_bf16(wv(2 * q), wv(2 * q + 1));
        r.y = pack_bf16(wv(2 * q + 8), wv(2 * q + 9));
        frag[e] = r;
    }
}

// forward weights for k_conv_tc: unit (tap, u, n) = W[tap][8u .. 8u+7][n] as BF16, n < nout
// (columns n >= cout are zero)
__global__ void k_pack_tc(const float* __restrict__ W, int cin, int cout, int nout, uint4* __restrict__ out) {
    const int nu = cin / 8;
    const int total = 27 * nu * nout;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int n = e % nout, u = (e / nout) % nu, tap = e / (nout * nu);
        if (n >= cout) { out[e] = make_uint4(0, 0, 0, 0); continue; }
        const float* w = W + ((size_t)tap * cin + 8 * u) * cout + n;
        out[e] = make_uint4(pack_bf16(w[0], w[(size_t)cout]), pack_bf16(w[2 * (size_t)cout], w[3 * (size_t)cout]),
                            pack_bf16(w[4 * (size_t)cout], w[5 * (size_t)cout]),
                            pack_bf16(w[6 * (size_t)cout], w[7 * (size_t)cout]));
    }
}

size_t frag_count(int cin, int cout, bool transposed) {
    const int ci_n = transposed ? cout : cin, co_n = transposed ? cin : cout;
    const int nt = (co_n + 7) / 8;
    const int nk = ci_n == 1 ? 2 : 27 * (ci_n / 16);
    return (size_t)nk * nt * 32;
}

// ---------------------------------------------------------------------------------
// gradient routing of the backward pass
// ---------------------------------------------------------------------------------
enum ScatterMode : int { SC_COPY = 0, SC_DOWNSUM = 1, SC_POOLADJ = 2 };
// dst[v][c] (+)= ... over the destination grid ddims, from src (fp32 [v][sstride] at soff)
__global__ void k_scatter(const float* __restrict__ src, int sstride, int soff, const int* sdims_unused, int sd0,
                          int sd1, int sd2, float* __restrict__ dst, int C, int dd0, int dd1, int dd2, int mode,
                          int accumulate) {
    const int sd[3] = {sd0, sd1, sd2}, dd[3] = {dd0, dd1, dd2};
    const long long nv = (long long)dd0 * dd1 * dd2;
    const long long tot = nv * C;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const long long v = e / C;
        const int c = (int)(e - v * C);
        const int z = (int)(v % dd2), y = (int)((v / dd2) % dd1), x = (int)(v / ((long long)dd2 * dd1));
        float s = 0.f;
        if (mode == SC_COPY) {
            s = src[v * sstride + soff + c];
        } else if (mode == SC_DOWNSUM) {   // dst coarse, src fine: sum of the children
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    for (int k = 0; k < 2; ++k) {
                        const int fx = 2 * x + i, fy = 2 * y + j, fz = 2 * z + k;
                        if (fx < sd[0] && fy < sd[1] && fz < sd[2]) s += src[vox(sd, fx, fy, fz) * sstride + soff + c];
                    }
        } else {   // SC_POOLADJ: dst fine, src coarse: parent / number of its children
            const int px = x >> 1, py = y >> 1, pz = z >> 1;
            const int cnt = (min(2, dd[0] - 2 * px)) * (min(2, dd[1] - 2 * py)) * (min(2, dd[2] - 2 * pz));
            s = src[vox(sd, px, py, pz) * sstride + soff + c] / (float)cnt;
        }
        float* d = dst + v * C + c;
        *d = accumulate ? *d + s : s;
    }
}

// ---------------------------------------------------------------------------------
// fine-grid pieces: restriction, prolongation (+ Jacobi term), loss
// ---------------------------------------------------------------------------------
__device__ __forceinline__ bool excl(const PoissonGrid& g, unsigned c) {
    return (int)c == g.pin || (g.solid && g.solid[c]);
}
__device__ __forceinline__ int bdiag(const PoissonGrid& g, int x, int y, int z) {
    if (!g.solid) return (x > 0) + (x < g.nx - 1) + (y > 0) + (y < g.ny - 1) + (z > 0) + (z < g.nz - 1);
    const unsigned sx = (unsigned)g.ny * g.nz, sy = g.nz;
    const unsigned c = ((unsigned)x * g.ny + y) * g.nz + z;
    int d = 0;
    auto nb = [&](unsigned o) { if (!g.solid[o]) ++d; };
    if (x > 0) nb(c - sx);
    if (x < g.nx - 1) nb(c + sx);
    if (y > 0) nb(c - sy);
    if (y < g.ny - 1) nb(c + sy);
    if (z > 0) nb(c - 1);
    if (z < g.nz - 1) nb(c + 1);
    return d;
}

__device__ __forceinline__ float rms_scale(const double* rr, double n_free) {
    if (!rr) return 1.f;
    const double v = *rr;
    return v > 0.0 ? (float)sqrt(n_free / v) : 0.f;
}

// x0[c] = scale * mean of the fine children of coarse cell c
__global__ void k_restrict(PoissonGrid g, const float* __restrict__ r, float* __restrict__ x0, int c0, int c1, int c2,
                           const double* rr, double n_free) {
    const float sc = rms_scale(rr, n_free);
    const unsigned n = (unsigned)c0 * c1 * c2;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const unsigned t = c / (unsigned)c2;
        const int z = (int)(c - t * (unsigned)c2), y = (int)(t % (unsigned)c1), x = (int)(t / (unsigned)c1);
        float s = 0.f;
        int cnt = 0;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    const int fx = 2 * x + i, fy = 2 * y + j, fz = 2 * z + k;
                    if (fx >= g.nx || fy >= g.ny || fz >= g.nz) continue;
                    s += r[((unsigned)fx * g.ny + fy) * g.nz + fz];
                    ++cnt;
                }
        x0[c] = sc * s / (float)cnt;
    }
}

// cell-centred linear prolongation along one axis: fine i -> coarse (j0, w0), (j1, w1)
__device__ __forceinline__ void pro1(int i, int nc, int& j0, float& w0, int& j1, float& w1) {
    if (i & 1) { j0 = i >> 1; j1 = j0 + 1; w0 = 0.75f; w1 = 0.25f; }
    else { j0 = (i >> 1) - 1; j1 = i >> 1; w0 = 0.25f; w1 = 0.75f; }
    j0 = max(0, min(nc - 1, j0));
    j1 = max(0, min(nc - 1, j1));
}

// z = omega r / diag + (1/scale) P y   (0 on excluded cells); omega_on = 0 drops the first term
__global__ void k_combine(PoissonGrid g, const float* __restrict__ r, const float* __restrict__ y, int c0, int c1,
                          int c2, const float* __restrict__ omega, int omega_on, const double* rr, double n_free,
                          float* __restrict__ z) {
    const float sc = rms_scale(rr, n_free);
    const float inv = sc > 0.f ? 1.f / sc : 0.f;
    const float om = omega_on ? *omega : 0.f;
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        if (excl(g, c)) { z[c] = 0.f; continue; }
        const unsigned t = c / (unsigned)g.nz;
        const int iz = (int)(c - t * (unsigned)g.nz), iy = (int)(t % (unsigned)g.ny), ix = (int)(t / (unsigned)g.ny);
        int xa, xb, ya, yb, za, zb;
        float wxa, wxb, wya, wyb, wza, wzb;
        pro1(ix, c0, xa, wxa, xb, wxb);
        pro1(iy, c1, ya, wya, yb, wyb);
        pro1(iz, c2, za, wza, zb, wzb);
        auto Y = [&](int x, int yy, int zz) { return y[((unsigned)x * c1 + yy) * c2 + zz]; };
        const float p = wxa * (wya * (wza * Y(xa, ya, za) + wzb * Y(xa, ya, zb)) + wyb * (wza * Y(xa, yb, za) + wzb * Y(xa, yb, zb))) +
                        wxb * (wya * (wza * Y(xb, ya, za) + wzb * Y(xb, ya, zb)) + wyb * (wza * Y(xb, yb, za) + wzb * Y(xb, yb, zb)));
        const int d = bdiag(g, ix, iy, iz);
        const float jac = d > 0 ? r[c] / (float)d : 0.f;
        z[c] = om * jac + inv * p;
    }
}

// weight of coarse cell m in the prolongation to fine cell i along one axis: 3/4 for the two
// children (2m, 2m+1), 1/4 for the next fine cells out (2m-1, 2m+2); at the ends of the axis
// the clamped neighbour adds its 1/4 to the end cell (fine 0 -> coarse 0, fine 2nc-1 ->
// coarse nc-1); 0 outside the fine grid
__device__ __forceinline__ float pro_weight(int i, int m, int nf, int nc) {
    if (i < 0 || i >= nf) return 0.f;
    if ((m == 0 && i == 0) || (m == nc - 1 && i == 2 * nc - 1)) return 1.f;
    if (i == 2 * m || i == 2 * m + 1) return 0.75f;
    if (i == 2 * m - 1 || i == 2 * m + 2) return 0.25f;
    return 0.f;
}

// gy = P^T gz  (gather over the fine cells 2m-1 .. 2m+2 per axis whose prolongation stencil
// holds coarse cell m)
__global__ void k_prolong_adj(PoissonGrid g, const float* __restrict__ gz, int c0, int c1, int c2, float* __restrict__ gy) {
    const unsigned n = (unsigned)c0 * c1 * c2;
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const unsigned t = c / (unsigned)c2;
        const int z = (int)(c - t * (unsigned)c2), y = (int)(t % (unsigned)c1), x = (int)(t / (unsigned)c1);
        float s = 0.f;
        for (int a = 0; a < 4; ++a) {
            const int fx = 2 * x - 1 + a;
            const float wx = pro_weight(fx, x, g.nx, c0);
            if (wx == 0.f) continue;
            for (int b = 0; b < 4; ++b) {
                const int fy = 2 * y - 1 + b;
                const float wy = pro_weight(fy, y, g.ny, c1);
                if (wy == 0.f) continue;
                for (int d = 0; d < 4; ++d) {
                    const int fz = 2 * z - 1 + d;
                    const float wz = pro_weight(fz, z, g.nz, c2);
                    if (wz == 0.f) continue;
                    s += wx * wy * wz * gz[((unsigned)fx * g.ny + fy) * g.nz + fz];
                }
            }
        }
        gy[c] = s;
    }
}

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
template <int NV>
__device__ void block_sums_d(const double (&v)[NV], double* part) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < NV; ++q) {
        const double s = warp_sum_d(v[q]);
        if (lane == 0) sh[q][wid] = s;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        for (int q = 0; q < NV; ++q) {
            double s = lane < nw ? sh[q][lane] : 0.0;
            s = warp_sum_d(s);
            if (lane == 0) part[blockIdx.x + gridDim.x * q] = s;
        }
    }
}

// e = z - p; partials of e.Be and, with backward, gz = 2 Be / denom and gz.(r/diag)
// mode 1 (calibration): partials of z.Bz and z.B(p - omega r/diag) instead
__global__ void k_loss(PoissonGrid g, const float* __restrict__ z, const float* __restrict__ p,
                       const float* __restrict__ r, const float* __restrict__ omega, double inv_denom, int backward,
                       int mode, float* __restrict__ gz, double* part) {
    const unsigned n = (unsigned)g.nx * g.ny * g.nz;
    const unsigned sx = (unsigned)g.ny * g.nz, sy = g.nz;
    const float om = *omega;
    double a0 = 0.0, a1 = 0.0;
    auto jac = [&](unsigned c, int ix, int iy, int iz) {
        const int d = bdiag(g, ix, iy, iz);
        return d > 0 ? r[c] / (float)d : 0.f;
    };
    for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        float gc = 0.f;
        if (!excl(g, c)) {
            const unsigned t = c / (unsigned)g.nz;
            const int iz = (int)(c - t * (unsigned)g.nz), iy = (int)(t % (unsigned)g.ny), ix = (int)(t / (unsigned)g.ny);
            // value at a cell: e (mode 0) or z (mode 1)
            auto val = [&](unsigned o) { return mode == 0 ? (double)z[o] - (double)p[o] : (double)z[o]; };
            double s = 0.0;
            int d = 0;
            auto nb = [&](unsigned o) {
                if (g.solid && g.solid[o]) return;
                ++d;
                if ((int)o != g.pin) s += val(o);
            };
            if (ix > 0) nb(c - sx);
            if (ix < g.nx - 1) nb(c + sx);
            if (iy > 0) nb(c - sy);
            if (iy < g.ny - 1) nb(c + sy);
            if (iz > 0) nb(c - 1);
            if (iz < g.nz - 1) nb(c + 1);
            const double vc = val(c);
            const double Bv = d * vc - s;
            if (mode == 0) {
                a0 += vc * Bv;
                if (backward) {
                    gc = (float)(2.0 * Bv * inv_denom);
                    a1 += (double)gc * (double)jac(c, ix, iy, iz);
                }
            } else {
                a0 += vc * Bv;                                                   // z.Bz
                a1 += Bv * ((double)p[c] - (double)om * (double)jac(c, ix, iy, iz));   // Bz.(p - omega r/d)
            }
        }
        if (backward && mode == 0) gz[c] = gc;
    }
    const double acc[2] = {a0, a1};
    block_sums_d<2>(acc, part);
}

__global__ void k_sum_parts(const double* part, int nb, int nv, double* out) {
    __shared__ double sh[32];
    for (int q = 0; q < nv; ++q) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[b + nb * q];
        s = warp_sum_d(s);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
            out[q] = t;
        }
        __syncthreads();
    }
}

// normalise a pair: r, p /= rms(r) (over the free cells)
__global__ void k_scale2(float* a, float* b, long long n, const double* sums, double n_free) {
    const double rr = sums[0];
    const float s = rr > 0.0 ? (float)sqrt(n_free / rr) : 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        a[i] *= s; b[i] *= s;
    }
}
// partials of r.r and r.p for a pair
__global__ void k_pair_dots(const float* r, const float* p, long long n, double* part) {
    double a0 = 0.0, a1 = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        a0 += (double)r[i] * r[i];
        a1 += (double)r[i] * p[i];
    }
    const double acc[2] = {a0, a1};
    block_sums_d<2>(acc, part);
}

__global__ void k_adam(float* __restrict__ w, float* __restrict__ gw, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2, float inv_batch) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gr = gw[i] * inv_batch;
        const float mi = b1 * m[i] + (1.f - b1) * gr;
        const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
        m[i] = mi; v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        gw[i] = 0.f;
    }
}

__global__ void k_scale_range(float* w, long long n, const double* factor) {
    const float f = (float)*factor;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        w[i] *= f;
}
__global__ void k_ratio(const double* sums, double* out) { out[0] = sums[0] > 0.0 ? sums[1] / sums[0] : 1.0; }

// ---------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------
constexpr int kRedBlocks = 304;

// a training pair with the Poisson problem it belongs to (solid mask copy, pinned cell)
struct Pair { float* r; float* p; unsigned char* solid; int pin; double denom; };

struct Net {
    int fine[3];
    int dims[4][3];
    cudaStream_t stream;
    float *w, *gw, *m, *v;
    uint2* wf[kLayers];
    uint2* wb[kLayers];
    uint4* wt[kLayers];   // k_conv_tc weights (layers with cin, cout multiples of 16)
    unsigned* tc_status;  // bit 0: a k_conv_tc wait ran out
    bool use_tc;
    size_t tc_budget;     // shared memory per k_conv_tc CTA
    void* act[kTensors];
    float* grad[kTensors];
    float* temp;       // backward data output of concat / pool inputs
    float* z;          // fine-grid preconditioner output (training)
    float* gz;         // fine-grid gradient
    double* part;
    double* sums;
    int adam_t;
    int launches;
    std::vector<Pair> pairs;
    std::vector<void*> allocs;
};

namespace {

#define UCK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return e_; } while (0)

int grid_for(long long n) { return (int)std::max(1LL, std::min<long long>(4 * 152, (n + 255) / 256)); }

void* dalloc(Net* n, size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, bytes);
    n->allocs.push_back(p);
    return p;
}

long long nvox(const int* d) { return (long long)d[0] * d[1] * d[2]; }

Src make_src(int kind, const void* p, int C, int cstride, int coff, const int* dims) {
    Src s;
    std::memset(&s, 0, sizeof(s));
    s.kind = kind; s.p = p; s.C = C; s.cstride = cstride; s.coff = coff;
    for (int i = 0; i < 3; ++i) s.dims[i] = dims[i];
    return s;
}

size_t conv_smem(int cin) {
    if (cin == 1) return (size_t)((HV * 2 + 15) / 16) * 16;
    return (size_t)((HV * (cin / 8) + 7) / 8) * 8 * 16;
}

size_t conv2_smem(int cin, int mt) {
    const int hv = (mt + 2) * 6 * 18;
    if (cin == 1) return (size_t)((hv * 2 + 15) / 16) * 16;
    return (size_t)hv * odd_units(cin) * 16;
}

template <int NTL, int MT, bool TAP>
cudaError_t launch_conv2_t(ConvArgs a, int nsplit, cudaStream_t s) {
    const size_t sm = conv2_smem(a.cin, MT);
    static bool attr = false;
    if (!attr) {
        UCK(cudaFuncSetAttribute(k_conv2<NTL, MT, TAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, 120 * 1024));
        attr = true;
    }
    if (sm > 120 * 1024) return cudaErrorInvalidValue;
    a.nsplit = nsplit;
    const dim3 grid(((a.dims[2] + 15) / 16) * nsplit, (a.dims[1] + 3) / 4, (a.dims[0] + MT - 1) / MT);
    k_conv2<NTL, MT, TAP><<<grid, kConvThreads, sm, s>>>(a);
    return cudaGetLastError();
}

template <int TXC, int NU, int THREADS>
cudaError_t launch_conv_tc_k(const ConvArgs& a, int n_out, int tpc, size_t smem, unsigned* status, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        UCK(cudaFuncSetAttribute(k_conv_tc<TXC, NU, THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemMax));
        attr = true;
    }
    const dim3 grid((a.dims[2] + TCZ - 1) / TCZ, (a.dims[1] + TCY - 1) / TCY, (a.dims[0] + TXC - 1) / TXC);
    k_conv_tc<TXC, NU, THREADS><<<grid, THREADS, smem, s>>>(a, n_out, tpc, status);
    return cudaGetLastError();
}

// 256 threads where the CTA is small enough for many CTAs per SM, else 512 (measured at
// 256^3: the 16 -> 16 layers 92 us with 256 threads, 130 with 512; the 48 -> 16 layer 379 us
// with 256, 352 with 512)
template <int TXC, int NU>
cudaError_t launch_conv_tc_t(const ConvArgs& a, int n_out, int tpc, size_t smem, unsigned* status, cudaStream_t s) {
    if (smem <= 40 * 1024) return launch_conv_tc_k<TXC, NU, 256>(a, n_out, tpc, smem, status, s);
    return launch_conv_tc_k<TXC, NU, kTcThreadsMax>(a, n_out, tpc, smem, status, s);
}

template <int TXC>
cudaError_t launch_conv_tc_nu(const ConvArgs& a, int n_out, int tpc, size_t smem, unsigned* status, cudaStream_t s) {
    switch (a.cin / 8) {
        case 2: return launch_conv_tc_t<TXC, 2>(a, n_out, tpc, smem, status, s);
        case 4: return launch_conv_tc_t<TXC, 4>(a, n_out, tpc, smem, status, s);
        case 6: return launch_conv_tc_t<TXC, 6>(a, n_out, tpc, smem, status, s);
        case 8: return launch_conv_tc_t<TXC, 8>(a, n_out, tpc, smem, status, s);
        case 10: return launch_conv_tc_t<TXC, 10>(a, n_out, tpc, smem, status, s);
        case 14: return launch_conv_tc_t<TXC, 14>(a, n_out, tpc, smem, status, s);
        default: return cudaErrorInvalidValue;
    }
}

size_t conv_tc_smem(int txc, int cin, int n_out, int tpc) {
    const size_t halo = ((size_t)tc_hvp(txc) * (cin / 8) * 16 + 127) & ~(size_t)127;
    const int nbuf = (27 + tpc - 1) / tpc > 1 ? 2 : 1;
    return halo + (size_t)nbuf * tpc * (cin / 8) * n_out * 16;
}

// The tensor-core path when the layer qualifies (cin a multiple of 16; BF16 output with cout a
// multiple of 16 up to 64, or the single FP32 output channel of the last layer, computed as 16
// with zero weights) and its tiles make at least one wave.  Configurations, best first: all
// 27 taps in one or two weight chunks (no refill wait, both loads overlap the halo staging),
// two x-planes per CTA before one; then 9-, 3- and 1-tap chunks; each within 110 KB of shared
// memory (two CTAs per SM).  Returns false (nothing launched) otherwise.
int tc_nout(int cout) { return cout == 1 ? 16 : cout; }

bool try_conv_tc(const ConvArgs& a, int cout, size_t budget, unsigned* status, cudaStream_t s, cudaError_t* err) {
    if (!a.wtc || a.cin % 16 || cout != a.cout_real) return false;
    const bool f32_single = a.out_kind == OUT_F32 && cout == 1;
    if (!f32_single && (a.out_kind != OUT_BF16 || cout % 16 || cout > 64)) return false;
    const int n_out = tc_nout(cout);
    const long long tiles1 = (long long)((a.dims[2] + TCZ - 1) / TCZ) * ((a.dims[1] + TCY - 1) / TCY) * a.dims[0];
    if (tiles1 < 152) return false;
    static const int order[][2] = {{2, 27}, {2, 14}, {1, 27}, {1, 14}, {2, 9}, {1, 9}, {2, 3}, {1, 3}, {2, 1}, {1, 1}};
    for (const auto& o : order) {
        const int txc = o[0], tpc = o[1];
        if (txc == 2 && tiles1 / 2 < 2 * 152) continue;
        const size_t sm = conv_tc_smem(txc, a.cin, n_out, tpc);
        if (sm > budget) continue;
        *err = txc == 2 ? launch_conv_tc_nu<2>(a, n_out, tpc, sm, status, s)
                        : launch_conv_tc_nu<1>(a, n_out, tpc, sm, status, s);
        return true;
    }
    return false;
}

// Chooses the brick (MT) and the n-tile split for a convolution with cout_padded output
// channels: whole bricks of 4 x 4 x 16 voxels (up to 32 output channels) or 2 x 4 x 16 where
// the grid gives at least two CTAs per SM, else 2 x 4 x 16 bricks with the output channels
// split 16 per CTA.  (Staging the weights in shared memory as well was measured slower: it
// costs CTAs per SM, and the weights stay in L1.)
cudaError_t launch_conv(ConvArgs a, int cout_padded, cudaStream_t s) {
    const int nt = cout_padded / 8;
    a.nt = nt;
    const long long bricks4 = (long long)((a.dims[2] + 15) / 16) * ((a.dims[1] + 3) / 4) * ((a.dims[0] + 3) / 4);
    const bool big = bricks4 >= 2 * 152;
    if (a.cin == 1) {
        if (nt != 2) return cudaErrorInvalidValue;
        return big ? launch_conv2_t<2, 4, true>(a, 1, s) : launch_conv2_t<2, 2, true>(a, 1, s);
    }
    if (a.cin % 16 != 0) return cudaErrorInvalidValue;
    if (big) {
        switch (nt) {
            case 1: return launch_conv2_t<1, 4, false>(a, 1, s);
            case 2: return launch_conv2_t<2, 4, false>(a, 1, s);
            case 4: return launch_conv2_t<4, 4, false>(a, 1, s);
            case 6: return launch_conv2_t<6, 2, false>(a, 1, s);
            case 8: return launch_conv2_t<8, 2, false>(a, 1, s);
            case 10: return launch_conv2_t<10, 2, false>(a, 1, s);
            case 14: return launch_conv2_t<14, 2, false>(a, 1, s);
            default: return cudaErrorInvalidValue;
        }
    }
    if (nt == 1) return launch_conv2_t<1, 2, false>(a, 1, s);
    if (nt % 2 != 0) return cudaErrorInvalidValue;
    return launch_conv2_t<2, 2, false>(a, nt / 2, s);
}

template <int COUT>
cudaError_t launch_wgrad_t(const ConvArgs& a, const Src& gs, float* dW, cudaStream_t s) {
    const size_t sm = conv_smem(a.cin) + (size_t)TX * TY * TZ * (COUT / 8) * 16;
    static bool attr = false;
    if (!attr) {
        UCK(cudaFuncSetAttribute(k_wgrad<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 140 * 1024));
        attr = true;
    }
    const dim3 grid((a.dims[2] + TZ - 1) / TZ, (a.dims[1] + TY - 1) / TY, (a.dims[0] + TX - 1) / TX);
    k_wgrad<COUT><<<grid, kConvThreads, sm, s>>>(a, gs, dW);
    return cudaGetLastError();
}

cudaError_t launch_wgrad(const ConvArgs& a, const Src& gs, int cout, float* dW, cudaStream_t s) {
    const dim3 grid((a.dims[2] + TZ - 1) / TZ, (a.dims[1] + TY - 1) / TY, (a.dims[0] + TX - 1) / TX);
    if (a.cin == 1 || cout == 1) {
        const size_t sm = ((size_t)HV * a.cin + (size_t)TX * TY * TZ * cout) * sizeof(float);
        k_wgrad_small<<<grid, kConvThreads, sm, s>>>(a, gs, cout, dW);
        return cudaGetLastError();
    }
    switch (cout) {
        case 16: return launch_wgrad_t<16>(a, gs, dW, s);
        case 32: return launch_wgrad_t<32>(a, gs, dW, s);
        case 48: return launch_wgrad_t<48>(a, gs, dW, s);
        case 64: return launch_wgrad_t<64>(a, gs, dW, s);
        default: return cudaErrorInvalidValue;
    }
}

// input sources of layer l (forward)
void layer_sources(const Net* n, int l, ConvArgs& a) {
    const LayerDef& d = kDefs[l];
    const int lev = d.shape.level;
    std::memset(&a.s0, 0, sizeof(Src));
    std::memset(&a.s1, 0, sizeof(Src));
    switch (d.mode) {
        case IN_SCALAR: a.s0 = make_src(SRC_F32, n->act[d.in0], 1, 1, 0, n->dims[lev]); break;
        case IN_PLAIN: a.s0 = make_src(SRC_BF16, n->act[d.in0], d.shape.cin, d.shape.cin, 0, n->dims[lev]); break;
        case IN_POOL: a.s0 = make_src(SRC_BF16_POOL, n->act[d.in0], d.shape.cin, d.shape.cin, 0, n->dims[lev - 1]); break;
        case IN_UPCAT: {
            const int cu = kTensorC[d.in0], cs = kTensorC[d.in1];
            a.s0 = make_src(SRC_BF16_UP, n->act[d.in0], cu, cu, 0, n->dims[lev + 1]);
            a.s1 = make_src(SRC_BF16, n->act[d.in1], cs, cs, 0, n->dims[lev]);
            break;
        }
    }
    a.cin = d.shape.cin;
    for (int i = 0; i < 3; ++i) a.dims[i] = n->dims[lev][i];
}

cudaError_t forward(Net* n, cudaStream_t s) {
    for (int l = 0; l < kLayers; ++l) {
        const LayerDef& d = kDefs[l];
        ConvArgs a;
        layer_sources(n, l, a);
        a.wfrag = n->wf[l];
        a.relu = d.shape.relu;
        a.cout_real = d.shape.cout;
        if (d.out == T_Y) { a.out_kind = OUT_F32; a.out = n->act[T_Y]; a.out_cstride = 1; a.out_coff = 0; }
        else { a.out_kind = OUT_BF16; a.out = n->act[d.out]; a.out_cstride = d.shape.cout; a.out_coff = 0; }
        a.wtc = n->use_tc ? n->wt[l] : nullptr;
        cudaError_t e = cudaSuccess;
        if (try_conv_tc(a, d.shape.cout, n->tc_budget, n->tc_status, s, &e)) UCK(e);
        else UCK(launch_conv(a, std::max(8, d.shape.cout), s));
        ++n->launches;
    }
    return cudaSuccess;
}

// backward through the network from grad[T_Y] (= dL/dy, fp32 level 0)
cudaError_t backward(Net* n, cudaStream_t s) {
    for (int t : {T_S0, T_S1, T_S2})
        UCK(cudaMemsetAsync(n->grad[t], 0, sizeof(float) * nvox(n->dims[kTensorLevel[t]]) * kTensorC[t], s));
    for (int l = kLayers - 1; l >= 0; --l) {
        const LayerDef& d = kDefs[l];
        const int lev = d.shape.level;
        // gated output gradient
        Src gs;
        if (d.shape.relu) {
            gs = make_src(SRC_F32_GATED, n->grad[d.out], d.shape.cout, d.shape.cout, 0, n->dims[lev]);
            gs.gate = (const __nv_bfloat16*)n->act[d.out];
            gs.gstride = d.shape.cout; gs.goff = 0;
        } else {
            gs = make_src(SRC_F32, n->grad[d.out], d.shape.cout, d.shape.cout, 0, n->dims[lev]);
        }
        ConvArgs a;
        layer_sources(n, l, a);
        a.wtc = nullptr;
        UCK(launch_wgrad(a, gs, d.shape.cout, n->gw + layer_offset(l), s));
        if (l == 0) break;
        // backward data: conv of gs with the flipped/transposed weights
        ConvArgs b;
        std::memset(&b, 0, sizeof(b));
        b.s0 = gs;
        b.cin = d.shape.cout;
        for (int i = 0; i < 3; ++i) b.dims[i] = n->dims[lev][i];
        b.wfrag = n->wb[l];
        b.relu = 0;
        b.out_kind = OUT_F32;
        b.cout_real = d.shape.cin;
        b.out_cstride = d.shape.cin;
        b.out_coff = 0;
        const bool direct = d.mode == IN_PLAIN;
        b.out = direct ? (void*)n->grad[d.in0] : (void*)n->temp;
        int gdims[3];
        for (int i = 0; i < 3; ++i) gdims[i] = n->dims[lev][i];
        UCK(launch_conv(b, d.shape.cin, s));
        if (d.mode == IN_POOL) {
            const int* fd = n->dims[lev - 1];
            k_scatter<<<grid_for(nvox(fd) * d.shape.cin), 256, 0, s>>>(n->temp, d.shape.cin, 0, nullptr, gdims[0], gdims[1],
                                                                         gdims[2], n->grad[d.in0], d.shape.cin, fd[0],
                                                                         fd[1], fd[2], SC_POOLADJ, 1);
        } else if (d.mode == IN_UPCAT) {
            const int cu = kTensorC[d.in0], cs = kTensorC[d.in1];
            const int* cd = n->dims[lev + 1];
            k_scatter<<<grid_for(nvox(cd) * cu), 256, 0, s>>>(n->temp, d.shape.cin, 0, nullptr, gdims[0], gdims[1], gdims[2],
                                                              n->grad[d.in0], cu, cd[0], cd[1], cd[2], SC_DOWNSUM, 0);
            k_scatter<<<grid_for(nvox(gdims) * cs), 256, 0, s>>>(n->temp, d.shape.cin, cu, nullptr, gdims[0], gdims[1],
                                                                 gdims[2], n->grad[d.in1], cs, gdims[0], gdims[1],
                                                                 gdims[2], SC_COPY, 1);
        }
        UCK(cudaGetLastError());
    }
    return cudaSuccess;
}

cudaError_t pack_all(Net* n, cudaStream_t s) {
    for (int l = 0; l < kLayers; ++l) {
        const LayerShape& sh = kDefs[l].shape;
        const float* W = n->w + layer_offset(l);
        k_pack<<<grid_for((long long)frag_count(sh.cin, sh.cout, false)), 256, 0, s>>>(W, sh.cin, sh.cout, 0, n->wf[l]);
        if (l > 0)
            k_pack<<<grid_for((long long)frag_count(sh.cin, sh.cout, true)), 256, 0, s>>>(W, sh.cin, sh.cout, 1, n->wb[l]);
        if (n->wt[l])
            k_pack_tc<<<grid_for(27LL * (sh.cin / 8) * tc_nout(sh.cout)), 256, 0, s>>>(W, sh.cin, sh.cout,
                                                                                    tc_nout(sh.cout), n->wt[l]);
    }
    return cudaGetLastError();
}

}  // namespace

Net* net_create(int nx, int ny, int nz, cudaStream_t s) {
    Net* n = new Net();
    n->fine[0] = nx; n->fine[1] = ny; n->fine[2] = nz;
    n->stream = s;
    n->adam_t = 0;
    n->launches = 0;
    for (int i = 0; i < 3; ++i) {
        int d = (n->fine[i] + 1) / 2;
        for (int l = 0; l < 4; ++l) { n->dims[l][i] = d; d = (d + 1) / 2; }
    }
    bool ok = true;
    auto A = [&](size_t bytes) { void* p = dalloc(n, bytes); ok = ok && p; return p; };
    const long long np = num_parameters();
    n->w = (float*)A(np * 4); n->gw = (float*)A(np * 4); n->m = (float*)A(np * 4); n->v = (float*)A(np * 4);
    for (int l = 0; l < kLayers; ++l) {
        const LayerShape& sh = kDefs[l].shape;
        n->wf[l] = (uint2*)A(frag_count(sh.cin, sh.cout, false) * sizeof(uint2));
        n->wb[l] = l > 0 ? (uint2*)A(frag_count(sh.cin, sh.cout, true) * sizeof(uint2)) : nullptr;
        const bool tc = sh.cin % 16 == 0 && ((sh.cout % 16 == 0 && sh.cout <= 64) || sh.cout == 1);
        n->wt[l] = tc ? (uint4*)A(27LL * (sh.cin / 8) * tc_nout(sh.cout) * sizeof(uint4)) : nullptr;
    }
    n->tc_status = (unsigned*)A(sizeof(unsigned));
    n->use_tc = true;
    // FIA_TC_SMEM_KB overrides the shared memory per tensor-core convolution CTA (tuning)
    n->tc_budget = kTcSmemBudget;
    if (const char* e = std::getenv("FIA_TC_SMEM_KB")) {
        const long kb = std::strtol(e, nullptr, 10);
        if (kb >= 16 && kb * 1024 <= kTcSmemMax) n->tc_budget = (size_t)kb * 1024;
    }
    size_t tmax = 0;
    for (int t = 0; t < kTensors; ++t) {
        const long long nv = nvox(n->dims[kTensorLevel[t]]);
        const size_t es = (t == T_X0 || t == T_Y) ? 4 : 2;
        n->act[t] = A((size_t)nv * kTensorC[t] * es + 64);
        n->grad[t] = (float*)A((size_t)nv * kTensorC[t] * 4 + 64);
    }
    for (int l = 0; l < kLayers; ++l) {
        const LayerDef& d = kDefs[l];
        if (d.mode == IN_POOL || d.mode == IN_UPCAT)
            tmax = std::max(tmax, (size_t)nvox(n->dims[d.shape.level]) * d.shape.cin);
    }
    n->temp = (float*)A(tmax * 4 + 64);
    const long long nf = (long long)nx * ny * nz;
    n->z = (float*)A(nf * 4); n->gz = (float*)A(nf * 4);
    n->part = (double*)A(kRedBlocks * 4 * sizeof(double));
    n->sums = (double*)A(8 * sizeof(double));
    if (!ok) { net_destroy(n); return nullptr; }
    return n;
}

void net_destroy(Net* n) {
    if (!n) return;
    cudaStreamSynchronize(n->stream);
    for (void* p : n->allocs) cudaFree(p);
    for (auto& pr : n->pairs) { cudaFree(pr.r); cudaFree(pr.p); if (pr.solid) cudaFree(pr.solid); }
    delete n;
}

cudaError_t net_set_weights(Net* n, const float* host, long long count) {
    if (count != num_parameters()) return cudaErrorInvalidValue;
    UCK(cudaMemcpyAsync(n->w, host, count * 4, cudaMemcpyHostToDevice, n->stream));
    UCK(pack_all(n, n->stream));
    return cudaStreamSynchronize(n->stream);
}

cudaError_t net_get_weights(Net* n, float* host, long long count) {
    if (count != num_parameters()) return cudaErrorInvalidValue;
    UCK(cudaMemcpyAsync(host, n->w, count * 4, cudaMemcpyDeviceToHost, n->stream));
    return cudaStreamSynchronize(n->stream);
}

cudaError_t net_grid_op(Net* n, const PoissonGrid& g, int op, const float* in, float* out, cudaStream_t s) {
    const int* d0 = n->dims[0];
    const long long nf = (long long)g.nx * g.ny * g.nz;
    if (op == 0) k_restrict<<<grid_for(nvox(d0)), 256, 0, s>>>(g, in, out, d0[0], d0[1], d0[2], nullptr, 0.0);
    else if (op == 1)
        k_combine<<<grid_for(nf), 256, 0, s>>>(g, in, in, d0[0], d0[1], d0[2], n->w + num_parameters() - 1, 0,
                                               nullptr, 0.0, out);
    else if (op == 2) k_prolong_adj<<<grid_for(nvox(d0)), 256, 0, s>>>(g, in, d0[0], d0[1], d0[2], out);
    else return cudaErrorInvalidValue;
    UCK(cudaGetLastError());
    return cudaStreamSynchronize(s);
}

cudaError_t net_get_grads(Net* n, float* host, long long count) {
    if (count != num_parameters()) return cudaErrorInvalidValue;
    UCK(cudaMemcpyAsync(host, n->gw, count * 4, cudaMemcpyDeviceToHost, n->stream));
    return cudaStreamSynchronize(n->stream);
}

cudaError_t net_init(Net* n, unsigned long long seed) {
    std::mt19937_64 rng(seed);
    std::vector<float> w(num_parameters());
    for (int l = 0; l < kLayers; ++l) {
        const LayerShape& sh = kDefs[l].shape;
        const double sd = std::sqrt((sh.relu ? 2.0 : 1.0) / (27.0 * sh.cin));
        std::normal_distribution<double> nd(0.0, sd);
        const long long o = layer_offset(l), c = 27LL * sh.cin * sh.cout;
        for (long long i = 0; i < c; ++i) w[o + i] = (float)nd(rng);
    }
    w.back() = 2.0f / 3.0f;
    n->adam_t = 0;
    UCK(cudaMemsetAsync(n->m, 0, w.size() * 4, n->stream));
    UCK(cudaMemsetAsync(n->v, 0, w.size() * 4, n->stream));
    UCK(cudaMemsetAsync(n->gw, 0, w.size() * 4, n->stream));
    return net_set_weights(n, w.data(), (long long)w.size());
}

void net_level_dims(const Net* n, int level, int dims[3]) {
    for (int i = 0; i < 3; ++i) dims[i] = n->dims[level][i];
}
int net_launches(const Net* n) { return n->launches; }

cudaError_t net_forward_level0(Net* n, const float* x0, float* y, cudaStream_t s) {
    const long long nv = nvox(n->dims[0]);
    UCK(cudaMemcpyAsync(n->act[T_X0], x0, nv * 4, cudaMemcpyDeviceToDevice, s));
    n->launches = 0;
    UCK(forward(n, s));
    if (y) UCK(cudaMemcpyAsync(y, n->act[T_Y], nv * 4, cudaMemcpyDeviceToDevice, s));
    return cudaSuccess;
}

cudaError_t net_backward_level0(Net* n, const float* gy, cudaStream_t s) {
    const long long nv = nvox(n->dims[0]);
    UCK(cudaMemcpyAsync(n->grad[T_Y], gy, nv * 4, cudaMemcpyDeviceToDevice, s));
    return backward(n, s);
}

cudaError_t net_zero_grad(Net* n, cudaStream_t s) {
    return cudaMemsetAsync(n->gw, 0, num_parameters() * 4, s);
}

cudaError_t net_apply(Net* n, const PoissonGrid& g, const float* r, float* z, const double* rr, double n_free,
                      cudaStream_t s) {
    const int* d0 = n->dims[0];
    n->launches = 0;
    k_restrict<<<grid_for(nvox(d0)), 256, 0, s>>>(g, r, (float*)n->act[T_X0], d0[0], d0[1], d0[2], rr, n_free);
    UCK(forward(n, s));
    k_combine<<<grid_for((long long)g.nx * g.ny * g.nz), 256, 0, s>>>(g, r, (const float*)n->act[T_Y], d0[0], d0[1],
                                                                      d0[2], n->w + num_parameters() - 1, 1, rr,
                                                                      n_free, z);
    n->launches += 2;
    return cudaGetLastError();
}

int net_add_pair(Net* n, const PoissonGrid& g, const float* r_dev, const float* p_dev, cudaStream_t s) {
    const long long nf = (long long)g.nx * g.ny * g.nz;
    Pair pr;
    pr.solid = nullptr;
    pr.pin = g.pin;
    if (cudaMalloc(&pr.r, nf * 4) != cudaSuccess) return -1;
    if (cudaMalloc(&pr.p, nf * 4) != cudaSuccess) { cudaFree(pr.r); return -1; }
    auto fail = [&]() { cudaFree(pr.r); cudaFree(pr.p); if (pr.solid) cudaFree(pr.solid); return -1; };
    cudaMemcpyAsync(pr.r, r_dev, nf * 4, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(pr.p, p_dev, nf * 4, cudaMemcpyDeviceToDevice, s);
    long long nfree = nf - 1;
    if (g.solid) {
        if (cudaMalloc(&pr.solid, nf) != cudaSuccess) return fail();
        cudaMemcpyAsync(pr.solid, g.solid, nf, cudaMemcpyDeviceToDevice, s);
        std::vector<unsigned char> m(nf);
        if (cudaMemcpyAsync(m.data(), g.solid, nf, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return fail();
        nfree = 0;
        for (long long i = 0; i < nf; ++i) nfree += (m[i] == 0 && i != g.pin);
    }
    k_pair_dots<<<kRedBlocks, 256, 0, s>>>(pr.r, pr.p, nf, n->part);
    k_sum_parts<<<1, 256, 0, s>>>(n->part, kRedBlocks, 2, n->sums);
    k_scale2<<<grid_for(nf), 256, 0, s>>>(pr.r, pr.p, nf, n->sums, (double)nfree);
    double h[2];
    cudaMemcpyAsync(h, n->sums, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || !(h[0] > 0.0)) return fail();
    pr.denom = h[1] / h[0] * (double)nfree;   // p^T B p = p^T r after scaling both by sqrt(nfree/rr)
    n->pairs.push_back(pr);
    return (int)n->pairs.size() - 1;
}

int net_num_pairs(const Net* n) { return (int)n->pairs.size(); }

void net_set_tc(Net* n, bool on) { n->use_tc = on; }

cudaError_t net_tc_status(Net* n, unsigned* out, cudaStream_t s) {
    UCK(cudaMemcpyAsync(out, n->tc_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    return cudaStreamSynchronize(s);
}

cudaError_t net_loss(Net* n, const PoissonGrid& g0, int pair, bool backward_pass, double* loss, cudaStream_t s) {
    if (pair < 0 || pair >= (int)n->pairs.size()) return cudaErrorInvalidValue;
    const Pair& pr = n->pairs[pair];
    const PoissonGrid g{g0.nx, g0.ny, g0.nz, pr.pin, pr.solid};
    const int* d0 = n->dims[0];
    const long long nf = (long long)g.nx * g.ny * g.nz;
    const float* omega = n->w + num_parameters() - 1;
    k_restrict<<<grid_for(nvox(d0)), 256, 0, s>>>(g, pr.r, (float*)n->act[T_X0], d0[0], d0[1], d0[2], nullptr, 0.0);
    UCK(forward(n, s));
    k_combine<<<grid_for(nf), 256, 0, s>>>(g, pr.r, (const float*)n->act[T_Y], d0[0], d0[1], d0[2], omega, 1, nullptr,
                                           0.0, n->z);
    k_loss<<<kRedBlocks, 256, 0, s>>>(g, n->z, pr.p, pr.r, omega, 1.0 / pr.denom, backward_pass ? 1 : 0, 0, n->gz,
                                      n->part);
    k_sum_parts<<<1, 256, 0, s>>>(n->part, kRedBlocks, 2, n->sums);
    double h[2];
    UCK(cudaMemcpyAsync(h, n->sums, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (backward_pass) {
        k_prolong_adj<<<grid_for(nvox(d0)), 256, 0, s>>>(g, n->gz, d0[0], d0[1], d0[2], n->grad[T_Y]);
        UCK(backward(n, s));
    }
    UCK(cudaStreamSynchronize(s));
    if (backward_pass) {
        // d loss / d omega accumulates on the host side copy of the last gradient entry
        float go = 0.f;
        UCK(cudaMemcpy(&go, n->gw + num_parameters() - 1, 4, cudaMemcpyDeviceToHost));
        go += (float)h[1];
        UCK(cudaMemcpy(n->gw + num_parameters() - 1, &go, 4, cudaMemcpyHostToDevice));
    }
    if (loss) *loss = h[0] / pr.denom;
    return cudaGetLastError();
}

cudaError_t net_calibrate(Net* n, const PoissonGrid& g0, int pair, cudaStream_t s) {
    if (pair < 0 || pair >= (int)n->pairs.size()) return cudaErrorInvalidValue;
    const Pair& pr = n->pairs[pair];
    const PoissonGrid g{g0.nx, g0.ny, g0.nz, pr.pin, pr.solid};
    const int* d0 = n->dims[0];
    const long long nf = (long long)g.nx * g.ny * g.nz;
    const float* omega = n->w + num_parameters() - 1;
    k_restrict<<<grid_for(nvox(d0)), 256, 0, s>>>(g, pr.r, (float*)n->act[T_X0], d0[0], d0[1], d0[2], nullptr, 0.0);
    UCK(forward(n, s));
    k_combine<<<grid_for(nf), 256, 0, s>>>(g, pr.r, (const float*)n->act[T_Y], d0[0], d0[1], d0[2], omega, 0, nullptr,
                                           0.0, n->z);
    k_loss<<<kRedBlocks, 256, 0, s>>>(g, n->z, pr.p, pr.r, omega, 1.0, 0, 1, nullptr, n->part);
    k_sum_parts<<<1, 256, 0, s>>>(n->part, kRedBlocks, 2, n->sums);
    k_ratio<<<1, 1, 0, s>>>(n->sums, n->sums + 4);
    const long long o = layer_offset(kLayers - 1), c = 27LL * kDefs[kLayers - 1].shape.cin;
    k_scale_range<<<grid_for(c), 256, 0, s>>>(n->w + o, c, n->sums + 4);
    UCK(pack_all(n, s));
    return cudaStreamSynchronize(s);
}

cudaError_t net_adam_step(Net* n, double lr, int batch, cudaStream_t s) {
    ++n->adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)n->adam_t), c2 = 1.f - std::pow(b2, (float)n->adam_t);
    const long long np = num_parameters();
    k_adam<<<grid_for(np), 256, 0, s>>>(n->w, n->gw, n->m, n->v, np, (float)lr, b1, b2, 1e-8f, c1, c2,
                                        1.f / (float)std::max(1, batch));
    UCK(pack_all(n, s));
    return cudaGetLastError();
}

}  // namespace unet
}  // namespace fia
