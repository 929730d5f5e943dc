// views.cuh — the headless visualisation views of final_stage.wgsl:35-68,
// written to a float volume in lattice order instead of a storage texture.
//
//   view 0  majority species of the voxel's slots / 255 (the first slot whose
//           species count is strictly largest wins, final_stage.wgsl:43-57)
//   view 1  region id / 255 (final_stage.wgsl:60-62)
//   view 2  reservoir species / 255 (final_stage.wgsl:64-66)
//
// Voxels cut away by the slice, res[axis] - coord[axis] < slice
// (final_stage.wgsl:35-38), are 0.
#pragma once
#include <cstdint>

namespace cellsim {

struct ViewParams {
    const uint8_t* slots;      // [V][K], compacted
    uint32_t K;
    uint32_t X, Y, Z;
    const uint8_t* region_id;  // [V] region ids, or null
    const uint8_t* region_pad; // padded region codes (id + 1), rows of Zr bytes with z at column z + 2, or null
    uint32_t Zr;
    const uint8_t* reservoir;  // [V], or null (no reservoirs)
    int32_t view;
    int32_t slice_axis;
    uint32_t slice;
    float* out;                // [V]
};

static __global__ void render_view_kernel(ViewParams p) {
    const uint64_t V = (uint64_t)p.X * p.Y * p.Z;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t z = (uint32_t)(v % p.Z);
        const uint64_t xy = v / p.Z;
        const uint32_t y = (uint32_t)(xy % p.Y), x = (uint32_t)(xy / p.Y);
        const uint32_t res[3] = {p.X, p.Y, p.Z}, coord[3] = {x, y, z};
        const int a = p.slice_axis < 0 || p.slice_axis > 2 ? 0 : p.slice_axis;
        if (res[a] - coord[a] < p.slice) {
            p.out[v] = 0.0f;
            continue;
        }
        uint32_t value = 0;
        if (p.view == 1) {
            if (p.region_id) value = p.region_id[v];
            else if (p.region_pad) value = (uint32_t)p.region_pad[xy * p.Zr + z + 2] - 1u;
        } else if (p.view == 2) {
            value = p.reservoir ? p.reservoir[v] : 0u;
        } else {
            const uint8_t* s = p.slots + v * p.K;
            uint32_t n = 0;
            while (n < p.K && s[n]) n++;
            uint32_t best = 0;
            for (uint32_t i = 0; i < n; i++) {
                uint32_t c = 0;
                for (uint32_t j = 0; j < n; j++) c += s[i] == s[j];
                if (c > best) {
                    best = c;
                    value = s[i];
                }
            }
        }
        p.out[v] = __fdiv_rn((float)value, 255.0f);
    }
}

}  // namespace cellsim
