// fia_unet.cuh -- the learned pressure preconditioner: a 3D U-Net (4 levels, 16/32/48/64
// channels, 3x3x3 convolutions, BF16 weights and activations, FP32 accumulation) used as the
// coarse solver of a two-level preconditioner inside flexible CG:
//
//     z = M(r) = omega D^-1 r + P net(R r)
//
// R: average of the 2x2x2 children (fine grid -> half-resolution grid, the U-Net's level 0),
// P: cell-centred trilinear prolongation (weights 3/4, 1/4 per axis, clamped at the walls),
// D: the diagonal of B = -A, omega a trained scalar.  The input of the network is scaled
// by 1/rms(r) and its output by rms(r), so M(c r) = c M(r) for c > 0.
//
// Convolutions are implicit GEMMs on the tensor cores (mma.sync m16n8k16, BF16 in, FP32
// accumulate): a CTA of 4 warps stages the halo of an MT x 4 x 16 voxel brick channels-last in
// shared memory (an odd number of 16-byte units per voxel, so ldmatrix rows never share a bank
// group; plain and upsampled BF16 sources by cp.async), reads A fragments with ldmatrix and B
// fragments (weights pre-arranged in fragment order) through L1; on the coarse levels the
// output channels are split over several CTAs per brick.  The backward data pass is the same
// kernel run on the gated output gradient with the weights flipped in space and transposed in
// channels; the backward weight pass reduces im2col(x)^T g per CTA on the tensor cores
// (ldmatrix.trans fragments) and adds the result to an FP32 gradient with atomics.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "fia_pressure.cuh"

namespace fia {
namespace unet {

constexpr int kLayers = 15;
constexpr int kTensors = 16;

struct LayerShape {
    int level;       // U-Net level of the output (0 = half resolution of the fine grid)
    int cin, cout;   // cin 1: scalar input (packed over taps); cout 1: scalar output
    int relu;
};
const LayerShape& layer_shape(int l);
long long num_parameters();              // conv weights of all layers + omega
long long layer_offset(int l);           // offset of layer l's weights [tap][cin][cout]

// Device state of one network on one grid size (the fine grid's nx, ny, nz).
struct Net;
Net* net_create(int nx, int ny, int nz, cudaStream_t s);
void net_destroy(Net* n);
cudaError_t net_set_weights(Net* n, const float* host, long long count);    // FP32 master
cudaError_t net_get_weights(Net* n, float* host, long long count);
cudaError_t net_init(Net* n, unsigned long long seed);                      // He-normal, omega 2/3

// z = M(r) for the preconditioner of fia_pressure's flexible CG.  rr: device pointer to
// r.r (the CG scalar); n_free the number of free cells.  Excluded cells get z = 0.
cudaError_t net_apply(Net* n, const PoissonGrid& g, const float* r, float* z, const double* rr, double n_free,
                      cudaStream_t s);

// Training pairs (B p = r on the fine grid, stored normalised to rms(r) = 1).
int net_add_pair(Net* n, const PoissonGrid& g, const float* r_dev, const float* p_dev, cudaStream_t s);
int net_num_pairs(const Net* n);
// Energy-norm loss (z - p)^T B (z - p) / p^T B p of pair i; grads accumulated if backward.
cudaError_t net_loss(Net* n, const PoissonGrid& g, int pair, bool backward, double* loss, cudaStream_t s);
// Adam on the accumulated gradients (divided by `batch`), then zero them and repack.
cudaError_t net_adam_step(Net* n, double lr, int batch, cudaStream_t s);
cudaError_t net_zero_grad(Net* n, cudaStream_t s);
// Scales the output layer to the energy-norm least-squares fit of pair i.
cudaError_t net_calibrate(Net* n, const PoissonGrid& g, int pair, cudaStream_t s);
cudaError_t net_get_grads(Net* n, float* host, long long count);
// test hook: op 0 restriction (fine -> level 0), 1 prolongation (level 0 -> fine, excluded
// cells 0), 2 adjoint of the prolongation (fine -> level 0); device arrays
cudaError_t net_grid_op(Net* n, const PoissonGrid& g, int op, const float* in, float* out, cudaStream_t s);

// Test hooks: run the network on a given level-0 input (scalar field, fp32 on the device),
// output the level-0 scalar result; activations stay inside.
cudaError_t net_forward_level0(Net* n, const float* x0, float* y, cudaStream_t s);
// Backward from a given dL/dy (level 0, fp32 device) after net_forward_level0.
cudaError_t net_backward_level0(Net* n, const float* gy, cudaStream_t s);
void net_level_dims(const Net* n, int level, int dims[3]);
int net_launches(const Net* n);   // kernels launched by the last net_apply
// the tcgen05 convolution path (on by default) and its error bits (bit 0: a wait ran out)
void net_set_tc(Net* n, bool on);
cudaError_t net_tc_status(Net* n, unsigned* out, cudaStream_t s);

}  // namespace unet
}  // namespace fia
