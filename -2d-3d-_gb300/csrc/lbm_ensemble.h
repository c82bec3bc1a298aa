// lbm_ensemble.h - batched time stepping of many FP32/FP16 lattices in one launch per stage.
//
// Members keep their own buffers (each is an ordinary handle); the ensemble builds a
// device table of member descriptors (geometry, constants, buffer pointers, buffer
// parity) and a packed tile table (member, first cell) per member list, and advances every
// member with one flow and one thermal launch per list and step.  Lists: 2D and 3D members
// taken one cell per thread, and 2D and 3D members with even nx taken two x-adjacent cells
// per thread (2-element vector loads and stores) when the launch configuration pairs.
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
    int grid_mul = 32;      // grid = min(tiles, SMs * grid_mul)
    int pairs = 1;          // members with even nx two cells per thread: bit 0 2D, bit 1 3D
};

// Member lists of a plan: index (dim == 3) + 2 * paired.
constexpr int kEnsLists = 4;

struct EnsPlan {
    int precision = LBM_FP32;
    int nmembers[kEnsLists] = {};
    void* d_members[kEnsLists] = {};
    int2* d_tiles[kEnsLists] = {};
    int ntiles[kEnsLists] = {};
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
