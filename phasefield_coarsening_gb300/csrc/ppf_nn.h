// ppf_nn.h -- the learned time-stepping surrogate's device side: data
// layout of activations, and launchers of the tcgen05 implicit-GEMM 3x3x3
// convolutions and their helpers.  Internal (not part of include/ppf.h).
//
// Activation layout ("planar padded"): a tensor of C channels on an
// (nz, ny, nx) domain with a one-voxel halo is stored as C/8 planes of
// 16-byte voxels (8 BF16 channels each):
//   byte (j, x, y, z) = (j * Pst + p(x, y, z)) * 16,  p = (z+1) YX + (y+1) X + (x+1)
// with X = nx+2, YX = (ny+2)(nx+2), Pst >= (nz+2) YX.  A run of voxels
// along x is then a run of 16-byte rows, which is exactly the no-swizzle
// core-matrix layout of the tensor-core operands: shifting a convolution
// tap by one voxel in x moves an operand's start address by 16 bytes.
// Halo voxels hold the periodic (or mirrored, no-flux) images, written by
// the kernel that produces the tensor.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ppf_internal.h"

namespace ppf {
namespace nn {

constexpr int kTileX = 128;                 // voxels of one tile (the MMA's M)
constexpr int kSegRows = kTileX + 2;        // a tile plus one voxel on each side in x
constexpr int kSegPlane = kSegRows * 16;    // bytes of one 8-channel plane of a segment

struct NNGeom {
    int nx, ny, nz, bc;
    int X;           // nx + 2
    int64_t YX;      // (ny + 2)(nx + 2)
    int64_t Pst;     // voxels per channel plane
    __host__ __device__ __forceinline__ int64_t p(int x, int y, int z) const {
        return (int64_t)(z + 1) * YX + (int64_t)(y + 1) * X + (x + 1);
    }
};

inline NNGeom make_nngeom(int nz, int ny, int nx, int bc) {
    NNGeom g;
    g.nx = nx; g.ny = ny; g.nz = nz; g.bc = bc;
    g.X = nx + 2;
    g.YX = (int64_t)(ny + 2) * (nx + 2);
    g.Pst = ((int64_t)(nz + 2) * g.YX + 7) / 8 * 8;
    return g;
}

inline size_t act_bytes(const NNGeom &g, int C) { return (size_t)(C / 8) * (size_t)g.Pst * 16; }

enum Epi : int {
    EPI_ACT = 0,        // out = silu(acc + b)
    EPI_ACT_TRAIN = 1,  // out = silu(acc + b), zout = acc + b
    EPI_DGRAD = 2,      // out = acc * silu'(zlow), bias-gradient sums
    EPI_STATE = 3,      // state s1 = s0 + oscale * (acc + b), channels 0..2
    EPI_LOSS = 4,       // loss against (s1 - s0) / oscale, out = dLoss/dpred
};

struct ConvArgs {
    NNGeom g;
    const uint16_t *x;      // input, CI channels (planar padded)
    const uint16_t *wimg;   // weight image: [dz][dx][CI/8][dy][CO][8] BF16
    const float *bias;      // CO
    uint16_t *out;          // output, CO channels (planar padded)
    uint16_t *zout;         // pre-activations (EPI_ACT_TRAIN), interior only
    const uint16_t *zlow;   // pre-activations of the layer below (EPI_DGRAD)
    float *partials;        // per CTA: CO bias-gradient sums, then the loss (EPI_DGRAD, EPI_LOSS)
    double *mass_part;      // per CTA: FP64 sum of the new c (EPI_STATE)
    Geom sg;                // state geometry (EPI_STATE, EPI_LOSS)
    Fields<const float> s0; // state at the start of the call
    Fields<float> s1;       // EPI_STATE: state written; EPI_LOSS: target state (read)
    float oscale[3];        // output scale per state channel
    float lw[3];            // loss weight per channel, including 1/count
    int yc;                 // rows per work item
    int items;
    int *err;
    unsigned long long limit_ns;
    int inject_stall;       // test hook: one input row's copies never complete
};

struct WgradArgs {
    NNGeom g;
    const uint16_t *x;      // layer input, CX channels
    const uint16_t *dz;     // gradient of the layer's pre-activation, CZ channels
    float *partials;        // per CTA: [27][CZ][CX]
    int ntiles;
    int *err;
    unsigned long long limit_ns;
};

int conv_smem_bytes(int ci, int co);
int conv_ctas_per_sm(int ci, int co);
int wgrad_smem_bytes(int cx, int cz);
cudaError_t conv_setup(int max_smem_optin);
cudaError_t launch_conv(int ci, int co, int epi, const ConvArgs &a, int grid, cudaStream_t s);
cudaError_t launch_wgrad(int cx, int cz, const WgradArgs &a, int grid, cudaStream_t s);

}  // namespace nn
}  // namespace ppf
