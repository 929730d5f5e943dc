// resident_kernel.cuh — the resident form of the production step.
//
// A lattice small enough for one block's shared memory (about 5,300 voxels at
// K = 16, 8,800 at K = 8: two copies of the slots, a decision word, two list
// entries and a region code per voxel) steps every frame of a step call inside
// one launch, one block per replicate.  Each frame is the oracle's order
// itself: for each axis the move decisions of every occupied voxel, a block
// barrier, the new content of every voxel, a barrier; then the quiet-voxel
// test of every occupied voxel and the SSA of the rest, one warp per voxel
// (react_voxel_warp).  Every step works on lists, not on the whole lattice:
// the block keeps the list of occupied voxels from sweep to sweep, the
// decisions add the voxels that receive a particle (a shared bitmap keeps
// each voxel on the list once), the new contents are formed for the listed
// voxels only, and those that end up occupied make the next sweep's list.
// So a frame costs work in proportion to the particles, not to the lattice.
// The same per-voxel functions as the sweep stream's (decide_moves, combine,
// calm_voxel, react_voxel_warp) compute every value, so the lattice, the
// counts and the diagnostics equal the other forms'.  There is no global
// record, bitmap or dependency wait: a frame costs a few block barriers
// instead of the launch boundaries or completion values through L2 that the
// stream pays, which is what bounds a lattice of a few thousand voxels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "prod_kernel.cuh"

namespace cellsim {

constexpr int RESIDENT_THREADS = 512;
constexpr int RESIDENT_SSA_WARPS = 8;  // the warps that run the SSA (1408 bytes of scratch each)

struct ResidentParams {
    ProdParams P;          // tables, replicates, counts, diagnostics; P.src holds the call's first
                           // frame, P.dst receives its last; block 0 zeroes P.reset[0 .. n_reset)
    uint32_t frame0;       // frame number of the call's first frame
    uint32_t n_frames;
    uint32_t rep0;         // block b runs replicate rep0 + b
    uint32_t stepbuf_out;  // P.stepbuf[stepbuf_out] receives frame0 + n_frames
    uint32_t vmax;         // voxels of the largest replicate of the launch (the shared-memory layout)
    uint32_t thr_words;    // threshold-table words staged in shared memory (0: read from global)
};

// Dynamic shared memory of one block for replicates of at most vmax voxels.
size_t resident_smem(int K, uint64_t vmax, uint32_t thr_words);
// Lets the resident kernels use the device's whole opt-in shared memory.
void resident_set_attrs(int device);
void resident_launch(int K, const ResidentParams& RP, int grid, size_t smem, cudaStream_t s);

}  // namespace cellsim
