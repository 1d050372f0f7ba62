// Activation layout and 3x3x3 convolution kernels of the learned
// preconditioner (BF16 storage, FP32 accumulation on the tcgen05 tensor cores).
//
// Layout of one grid level (nz, ny, nx) with C channels (C a multiple of 8):
// the grid is zero-padded by one cell on every side (padded dims nz+2, ny+2,
// nx+2; voxel o = padded linear index, x fastest) and the channels are stored
// in blocks of 8 (16 bytes per voxel and block).  Block g of voxel o sits at
// element (g * S + GD + o) of a uint4 array; GD guard voxels before and after
// each block keep every window a conv tile reads inside the allocation.  Pads
// and guards hold zeros.  In this layout a 3x3x3 tap (dz, dy, dx) is a constant
// shift dz*P + dy*R + dx of the voxel index, so a tile of 128 consecutive
// padded voxels reads, per (dz, dy), one contiguous window of 130 voxels.
#pragma once

#include "nn_internal.cuh"

struct nn_act_geom {
    int nz = 0, ny = 0, nx = 0;
    int64_t R = 0, P = 0, Np = 0;   // padded row, plane, volume (voxels)
    int64_t GD = 0, S = 0;          // guard, block stride (voxels)
    int64_t o_first = 0, o_last = 0;  // first / last interior voxel
    int64_t tiles = 0;              // 128-voxel tiles covering [o_first, o_last]
};

inline nn_act_geom nn_act_geometry(int nz, int ny, int nx)
{
    nn_act_geom g;
    g.nz = nz; g.ny = ny; g.nx = nx;
    g.R = nx + 2;
    g.P = g.R * (ny + 2);
    g.Np = g.P * (nz + 2);
    g.GD = g.P + g.R + 2 + 128;
    g.S = g.Np + 2 * g.GD;
    g.o_first = g.P + g.R + 1;
    g.o_last = (int64_t)nz * g.P + (int64_t)ny * g.R + nx;
    g.tiles = (g.o_last - g.o_first + 128) / 128;
    return g;
}

// Bytes of an activation tensor with C channels.
inline size_t nn_act_bytes(const nn_act_geom& g, int C) { return (size_t)(C / 8) * g.S * 16; }

bool nn_conv_supported(int cin, int cout);
size_t nn_conv_packed_weight_bytes(int cin, int cout);

// y = act(conv(x) + bias) [* (mask > 0)], BF16 in and out, on ctx's stream.
// y32 (nullable): channel 0 of the result also written as a dense FP32 grid,
// times (float)*y32_scale when y32_scale (device) is given.  up (nullable):
// the result also written, nearest-upsampled (each voxel to its eight
// children), into the first COUT/8 channel blocks of the activation up of
// geometry *gup (twice the sides).  Launched as a programmatic dependent of
// the kernel before it (nn_launch_pdl).
nn_status nn_conv_forward(nn_ctx* ctx, const nn_act_geom& g, int cin, int cout, const void* x, const void* wpacked,
                          const float* bias, int relu, const void* mask, void* y, float* y32, int* err,
                          const double* y32_scale = nullptr, void* up = nullptr, const nn_act_geom* gup = nullptr);
// dw[27][cin][cout] += sum over voxels of x(o + tap) gy(o); db[cout] += sum gy.
// err (device int) is set when a pipeline wait gives up.
nn_status nn_conv_wgrad(nn_ctx* ctx, const nn_act_geom& g, int cin, int cout, const void* x, const void* gy,
                        float* dw, float* db, int* err);
// Pack FP32 weights w[27][cin][cout] (tap = (dz+1)*9 + (dy+1)*3 + dx+1) into
// the tile-ordered BF16 blocks the forward kernel streams.  With flip set the
// packed operator is the adjoint (taps mirrored, cin and cout exchanged),
// i.e. the input-gradient convolution of a cout x cin layer.
nn_status nn_conv_pack(nn_ctx* ctx, int cin, int cout, const float* w, int flip, void* packed);
nn_status nn_act_pack_dense(nn_ctx* ctx, const nn_act_geom& g, int C, const float* dense, void* act);
nn_status nn_act_unpack_dense(nn_ctx* ctx, const nn_act_geom& g, int C, const void* act, float* dense);
