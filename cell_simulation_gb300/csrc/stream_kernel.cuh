// stream_kernel.cuh — the sweep-stream form of the production step.
//
// One frame is barrier-free passes over the occupancy bitmaps:
//
//   pass 0  x-move decisions of every occupied voxel of the source lattice
//   pass 1  X sweep (new content along x), y-move decisions
//   pass 2  Y sweep, z-move decisions
//   pass 3  Z sweep, reactions, store into the destination lattice and its
//           occupancy bitmap; voxels that became empty get zeros
//
// Pass 3 decides for every occupied voxel whether an event can fire at all
// (the exact quiet-voxel bound).  The few voxels whose first event may fall
// within the frame are set aside by the lane that meets them, and once the
// group's items are done the whole warp runs their SSA together
// (react_voxel_warp), then stores them and makes their next-frame decisions.
// So no lane runs a long single-voxel SSA while the others wait, and no launch
// of its own (and no launch boundary) is spent on them.
//
// Pass 0 of frame f + 1 needs only the final contents of frame f, so pass 3
// also makes the next frame's x-decisions while the contents are in
// registers, and consecutive frames run passes 1-3 only.  The host runs a
// standalone pass 0 when those decisions are absent or stale (the first
// frame, a new lattice, seed, frame number or step configuration).
//
// The Z sweep of a row needs nothing but that row's z-decisions, and a group
// holds whole rows when a row has at most 32 words (Z <= 1024).  The fused
// variants then run passes 2 and 3 as one launch (PASS_YZ): each warp sweeps
// its group along y and at once along z, the z-decision words passing
// through the warp's shared memory and registers instead of global arrays.
// Their records take three buffers with fixed roles (x-, y- and z-decisions),
// because the Y sweep of one group still reads the y-decision records of the
// neighbouring groups' rows while another group's Z sweep writes next-frame
// x-decisions.
//
// A warp takes a word group: up to 32 bitmap words of one replicate, one per
// lane (rows of one x plane, z fastest).  Each lane builds the word's work
// mask from its own words and those of the neighbouring rows (or, for the
// Z sweep, the neighbouring bits), the warp lists the set bits in shared
// memory and runs the list with every lane busy.  Nothing synchronises
// beyond the warp, so every SM keeps as many warps in flight as its
// registers allow.
//
// Between passes a voxel's state is a 32-byte record (content, move
// decisions, and the words of its Philox block B(v, 0) that later passes
// still need).  Records are packed per group: the record of work bit b of a
// word is base[word] + popcount(work[word] below b), where work and base are
// the producing pass's per-word arrays.  The records a pass writes are
// therefore contiguous, so L2 holds whole lines of them between passes.
//
// The per-voxel operations (decide_moves, combine, calm_voxel,
// react_voxel) are those of the brick pass and the tile pipeline, so all
// three forms compute the same lattice bit for bit.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "prod_common.cuh"
#include "prod_kernel.cuh"

namespace cellsim {

// Lane i of a group holds word k0 + i % nk of row (x, y0 + i / nk).
struct WordGroup {
    uint32_t rep, x, y0, nrows, k0, nk;
    uint64_t rbase;  // first record index of the group (capacity nrows * nk * 32 records)
};
static_assert(sizeof(WordGroup) == 32, "WordGroup is 32 bytes");

// Per-word arrays of one pass boundary (indexed like the occupancy bitmaps).
struct SweepWords {
    uint32_t* occ;   // voxels with content after the sweep
    uint32_t* mv_m;  // voxels whose next-axis decision moves something to the lower neighbour
    uint32_t* mv_p;  // ... to the upper neighbour
    uint32_t* work;  // work mask of the producing pass (record index)
    uint32_t* base;  // first record index of the word
};

struct StreamParams {
    ProdParams P;
    const WordGroup* groups;
    uint32_t n_groups;
    uint32_t* queue;  // group counter of this pass (zero at launch); null: groups dealt round-robin
    uint32_t batch;   // consecutive groups taken per increment of the counter (at least 1)
    // per bitmap word: the region code shared by every lattice voxel of the word's window
    // (rows x-1..x+1, y-1..y+1, z from 32k-1 to 32k+32), or 0; null for one-region replicates
    const uint8_t* wcode;
    // pass 3: nonzero when it also makes the next frame's x-decisions (the
    // work of pass 0 for frame + 1) from the final contents, so that the next
    // frame starts at pass 1
    uint32_t fuse;
    SweepWords in;   // produced by the previous pass (pass 0: unused)
    SweepWords out;  // produced by this pass (pass 3: the next frame's x-decisions when fused)
    const uint4* rec_in;
    uint4* rec_mid;  // PASS_YZ: the z-decision records its Y sweep writes and its Z sweep reads
    uint4* rec_out;
    // pass 3: per warp of the launch (block * warps per block + warp), room for a group's items:
    // the voxels set aside for the warp's SSA beyond its shared buffer (record index, item)
    uint2* ssa_over;
    // the persistent multi-frame form: the lattice buffers of frames of parity 1 (those of parity 0
    // are in.occ, P.odst and P.dst)
    const uint32_t* in_occ1;
    uint32_t* odst1;
    uint8_t* dst1;
};

// Template value of the fused Y and Z sweep (passes 2 and 3 in one launch).
constexpr int PASS_YZ = 5;

// The persistent multi-frame form of the fused stream: one launch runs pass 1 and the fused Y and
// Z sweeps of every word group (of every replicate) for n_frames frames.  Tasks come from one
// counter in the order frame, pass, group (groups heaviest first), so that a warp that finishes
// early takes the next pass's or the next frame's groups instead of idling in a launch's tail.  A
// task first waits until the tasks it reads from, and those that read what it overwrites, are
// done: pass 1 of a group after the previous frame's fused pass of the group, of the groups with
// the same rows at x - 1 and x + 1 and of the previous and next group of its plane; the fused pass
// after this frame's pass 1 of the same five groups.  Within a pass the groups are taken heaviest
// first, or in plane order (a wavefront in x, for lattices whose occupancy is spread evenly).
struct FramesParams {
    StreamParams sp[2];    // [0] pass 1, [1] the fused Y and Z sweeps (parity 0's lattice buffers;
                           // parity 1's in in_occ1, odst1 and dst1)
    const uint32_t* nbr;   // per group: x - 1, x + 1, previous and next group of the plane, or
                           // 0xFFFFFFFF
    const uint32_t* order; // the group of each task rank within a pass (plane order); null: the
                           // groups' own order (heaviest first)
    uint32_t* done1;       // per group: seq + frame index + 1 of its last finished pass 1
    uint32_t* done2;       // ... of its last finished fused pass
    uint32_t* tasks;       // the launch's task counter, zero between launches
    uint32_t* exits;       // warps of the launch that have finished, zero between launches
    uint32_t* reset;       // queue counters of the per-pass launches, cleared at the start
    unsigned long long* fault;  // counts waits that timed out (the host then reports an error)
    uint32_t n_reset;
    uint32_t n_groups;
    uint32_t n_frames;     // n_frames * 2 * n_groups + the launch's warps < 2^32
    uint32_t cur0;         // parity of the first frame
    uint32_t seq;          // completion values of this launch are seq + frame index + 1
};

// Compiled launch shapes ("variants": threads per block and minimum resident
// blocks per SM) of the four passes.
int stream_variant_count();
int stream_variant_threads(int variant);
// True when the variant runs passes 2 and 3 as one launch (PASS_YZ, launched
// as its pass 2); it needs rows of at most 32 bitmap words.
bool stream_variant_fused(int variant);
// Launches pass `pass` (0..3) of variant `variant` for slot count K.
// Returns false when no such kernel is compiled.
bool stream_launch(int K, int variant, int pass, int grid, size_t smem, cudaStream_t s, const StreamParams& SP);
// Resident blocks per SM of that kernel with `smem` dynamic shared memory.
int stream_blocks_per_sm(int K, int variant, int pass, size_t smem);
// Dynamic shared memory of one block of NT threads whose warps stage `recs` records each.
size_t stream_smem(int NT, uint32_t S1, uint32_t thr_words, int recs);
// ... of pass `pass` of a variant (0-3 as stream_launch; 4: the multi-frame kernel).
size_t stream_pass_smem(int variant, int pass, uint32_t S1, uint32_t thr_words);
// Sets the kernel attributes (shared-memory size and carveout) of every pass.
void stream_set_attrs(int K, int variant, uint32_t S1, uint32_t thr_words);
// True when the variant runs in the persistent multi-frame form (stream_frames_launch), and when
// that form takes a pass's groups in plane order (FramesParams::order).
bool stream_variant_frames(int variant);
bool stream_variant_plane_order(int variant);
// Resident blocks per SM of the multi-frame kernel of the variant (0: not compiled).
int stream_frames_blocks_per_sm(int K, int variant, size_t smem);
// Launches the multi-frame kernel; false when none is compiled for K and the variant.
bool stream_frames_launch(int K, int variant, int grid, size_t smem, cudaStream_t s, const FramesParams& FP);
// Entries of StreamParams::ssa_over per warp of a pass-3 launch.
constexpr uint32_t STREAM_SSA_OVER_PER_WARP = 1024;

}  // namespace cellsim
