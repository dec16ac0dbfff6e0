// sph_grid.cuh -- the hashed cell grid shared by both SPH forms.
//
// Space is cut into cubic cells of a given side; a cell's bucket is the low
// bits of its Morton code (3-way interleave of the offset cell coordinates)
// in a table of 2^k >= 2N buckets.  Bodies radix sorted by bucket are also
// sorted in space, and a cell's bodies are one contiguous run of sorted
// slots.  Cells far apart (further than the table's period) can share a
// bucket; such buckets are marked and filtered by the packed cell key.
// The packed cell key clamps coordinates to +-2^20 cells; a body beyond
// that (a clamp) is reported through SFGPU_STATUS_SPH_CELLS: its candidates
// are still tested pair by pair, but cells that share its clamped key and
// bucket are no longer told apart.
#pragma once

#include "internal.cuh"

namespace sfgrid {

constexpr int CELL_BITS = 21;  // per axis in the packed cell key
constexpr int32_t CELL_OFF = 1 << (CELL_BITS - 1);

__device__ __forceinline__ int3 cell_of(float x, float y, float z, float inv) {
    return make_int3((int)floorf(x * inv), (int)floorf(y * inv), (int)floorf(z * inv));
}
__device__ __forceinline__ bool cell_clamped(int3 c) {
    return c.x < -CELL_OFF || c.x >= CELL_OFF || c.y < -CELL_OFF || c.y >= CELL_OFF || c.z < -CELL_OFF ||
           c.z >= CELL_OFF;
}
__device__ __forceinline__ int clamp_cell(int v) { return max(-CELL_OFF, min(CELL_OFF - 1, v)); }
__device__ __forceinline__ uint64_t pack_cell(int3 c) {
    auto f = [](int v) { return (uint64_t)(uint32_t)(clamp_cell(v) + CELL_OFF); };
    return (f(c.x) << (2 * CELL_BITS)) | (f(c.y) << CELL_BITS) | f(c.z);
}
__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // low 10 bits to every third bit
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
// The bucket comes from the unclamped coordinates, so two cells that clamp
// to the same key still land in different buckets (unless a table period
// apart), and a stencil offset never finds the same body twice.
__device__ __forceinline__ uint32_t bucket_of(int3 c, uint32_t mask) {
    const uint32_t x = (uint32_t)(c.x + CELL_OFF), y = (uint32_t)(c.y + CELL_OFF), z = (uint32_t)(c.z + CELL_OFF);
    return ((spread3(x) << 2) | (spread3(y) << 1) | spread3(z)) & mask;
}

// Squared distances from a point to the nearest and the farthest point of
// the box [lo, lo + side)^3 (FP32; callers compare them with margins).
__device__ __forceinline__ void box_dist2(float x, float y, float z, float lx, float ly, float lz, float side,
                                          float& dmin2, float& dmax2) {
    const float ax = lx - x, bx = x - (lx + side);
    const float ay = ly - y, by = y - (ly + side);
    const float az = lz - z, bz = z - (lz + side);
    const float nx = fmaxf(0.f, fmaxf(ax, bx)), ny = fmaxf(0.f, fmaxf(ay, by)), nz = fmaxf(0.f, fmaxf(az, bz));
    const float fx = fmaxf(fabsf(ax), fabsf(bx)), fy = fmaxf(fabsf(ay), fabsf(by)), fz = fmaxf(fabsf(az), fabsf(bz));
    dmin2 = nx * nx + ny * ny + nz * nz;
    dmax2 = fx * fx + fy * fy + fz * fz;
}

}  // namespace sfgrid
