// lbm_ensemble.h - batched time stepping of many FP32/FP16 lattices in one launch per stage.
//
// Members keep their own buffers (each is an ordinary handle); the ensemble builds a
// device table of member descriptors (geometry, constants, buffer pointers, buffer
// parity) and a packed tile table (member, first cell) over all members of one
// dimension, and advances every member with one flow and one thermal launch per step.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "lbm_fast.h"

namespace lbm {

struct EnsMemberHost {
    Geo geo;          // the member's geometry (wall terms in full-g form)
    PhysC phys;
    FastState* F;     // buffers and parity of the member
    int dim;
};

struct EnsLaunchCfg {
    int block = 128;        // threads per block
    int tile_cells = 1024;  // cells per tile (a multiple of `block`)
    int grid_mul = 8;       // grid = min(tiles, SMs * grid_mul)
};

struct EnsPlan {
    int precision = LBM_FP32;
    int nmembers[2] = {0, 0};  // [0] = 2D, [1] = 3D
    void* d_members[2] = {nullptr, nullptr};
    int2* d_tiles[2] = {nullptr, nullptr};
    int ntiles[2] = {0, 0};
    long long cells = 0;
    EnsLaunchCfg cfg;
    int sms = 152;
};

// Build the device tables (allocates with cudaMalloc; frees the previous tables).
cudaError_t ens_build(EnsPlan& plan, const std::vector<EnsMemberHost>& members, const EnsLaunchCfg& cfg, int sms);
void ens_free(EnsPlan& plan);
// One time step of every member; flip = number of batched steps since the build, mod 2.
void ens_step(const EnsPlan& plan, int flip, cudaStream_t s);

}  // namespace lbm
