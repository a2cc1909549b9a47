// sm_grid.h - uniform-grid conventions shared by the CUDA kernels and the CPU oracle:
// cell size rules, cell coordinates and the 8-phase order of the greedy sampler.
//
// The reference thins a cloud greedily in k-d-tree leaf order (util.cpp:107-139): a point
// is kept unless an already kept point lies within the sampling step (squared distance <
// step^2). The GPU keeps the greedy rule but fixes a parallel-friendly order: cells of
// side g >= step * (1 + 2^-10) are coloured by the parity of their three coordinates
// (8 phases); phases run one after the other, cells of one phase are at least one cell
// apart and cannot interact, and inside a cell points are visited by ascending index.
// The result is the sequential greedy thinning in the order (phase, cell, index), which
// the oracle computes sequentially and the GPU computes one phase per launch.
#pragma once

#include "sm_math.h"

namespace smg {

constexpr long long kMaxCells = 1ll << 22; // dense grid size cap (4M cells, 16 MB of u32)

SM_HD int dim_of(float extent, float g) { return (int)smm::ffloor(smm::fdiv(extent, g)) + 1; }

SM_HD long long cells_of(const float ext[3], float g) {
    return (long long)dim_of(ext[0], g) * (long long)dim_of(ext[1], g) *
           (long long)dim_of(ext[2], g);
}

// Cell side of the grid-order greedy sampler at `step`: slightly larger than the step so
// that two cells of the same phase never hold a conflicting pair. The sampler's grid is
// hashed (occupied cells only), so the side is doubled only while an axis would reach 2^20
// cells (cell keys stay within 60 bits).
SM_HD float thin_cell(float step, const float ext[3]) {
    float g = step * (1.0f + 1.0f / 1024.0f);
    // dim_of(e, g) >= 2^20  <=>  e / g >= 2^20 - 1 (compared in float: no int overflow)
    const float lim = (float)((1 << 20) - 1);
    for (int it = 0; it < 256; it++) {
        if (smm::fdiv(ext[0], g) < lim && smm::fdiv(ext[1], g) < lim && smm::fdiv(ext[2], g) < lim)
            break;
        g = g * 2.0f;
    }
    return g;
}

// Cell side of a dense acceleration grid for searches within `step` (the reference-order
// sampler's cell lists): slightly larger than the step, doubled until the dense grid fits
// the cap.
SM_HD float sample_cell(float step, const float ext[3]) {
    float g = step * (1.0f + 1.0f / 1024.0f);
    while (cells_of(ext, g) > kMaxCells)
        g = g * 2.0f;
    return g;
}

// Cell side for k-nearest / nearest-neighbour / radius queries: `want`, enlarged until
// the dense grid fits the cap.
SM_HD float query_cell(float want, const float ext[3]) {
    float g = want;
    while (cells_of(ext, g) > kMaxCells)
        g = g * 2.0f;
    return g;
}

SM_HD int coord(float x, float origin, float g, int dim) {
    int c = (int)smm::ffloor(smm::fdiv(x - origin, g));
    if (c < 0)
        c = 0;
    if (c > dim - 1)
        c = dim - 1;
    return c;
}

SM_HD int phase_of(int cx, int cy, int cz) { return (cx & 1) | ((cy & 1) << 1) | ((cz & 1) << 2); }

// After the cells within Chebyshev radius s of the query's cell have been searched, every
// other point lies at least s cells' width away from the query: lower bound s * g, less a
// 1% cell margin for the rounding of cell coordinates.
SM_HD float ring_bound(int s, float g) { return s <= 0 ? 0.0f : ((float)s - 0.01f) * g; }

} // namespace smg
