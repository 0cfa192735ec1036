// warp_union.cuh — warp-cooperative traversal of 27-cell stencils.
//
// Every 27-cell loop of the reference (compute_delta_pos, find_cover_vector,
// find_surface, compute_distance_to_surface, merge_mark_gpu,
// update_upsampled_cuda) visits cells in the order
// m = (dx+1)*9 + (dy+1)*3 + (dz+1) and, inside a cell, candidates by index.
// The cell key is lexicographic in (x, y, z) and the arrays are sorted by
// key, so that order is increasing candidate index within increasing key:
// one lane's visit order is a subsequence of the sorted array.
//
// warp_union_visit lets a warp walk the union of its lanes' stencils in that
// order.  Lanes are grouped by query column (q.x, q.y); for each of the nine
// neighbour columns the group's z-run is one contiguous index range, staged
// 32 candidates at a time into shared memory with one coalesced load, then
// visited by every lane whose stencil holds the candidate's cell.  Each
// candidate is read from global memory once per warp and each lane still
// sees exactly its own candidates in the reference order.
#pragma once

#include <climits>

#include "common.cuh"

namespace gg {

// masks m0, m1, m2: per axis, bit k set when offset k-1 is visited.
// stage(j, slot, ok): lane `slot` stores candidate j (when ok) into its
//   per-warp staging slot.
// visit(j, slot): called for each candidate j of this lane's stencil, in
//   order, with the staging slot holding it.
template <class StageF, class VisitF>
__device__ __forceinline__ void warp_union_visit(const Grid& g, const int32_t* __restrict__ cs, bool active,
                                                 int3 q, unsigned m0, unsigned m1, unsigned m2, StageF&& stage,
                                                 VisitF&& visit) {
  const int lane = threadIdx.x & 31;
  int zoff_lo = 2, zoff_hi = -2;
  for (int k = 0; k < 3; ++k)
    if ((m2 >> k) & 1u) {
      zoff_lo = min(zoff_lo, k - 1);
      zoff_hi = max(zoff_hi, k - 1);
    }
  unsigned pending = __ballot_sync(0xffffffffu, active);
  while (pending) {
    const int leader = __ffs(pending) - 1;
    const int gx = __shfl_sync(0xffffffffu, q.x, leader);
    const int gy = __shfl_sync(0xffffffffu, q.y, leader);
    const bool mine = active && ((pending >> lane) & 1u) && q.x == gx && q.y == gy;
    pending &= ~__ballot_sync(0xffffffffu, mine);
    for (int ox = 0; ox < 3; ++ox) {
      for (int oy = 0; oy < 3; ++oy) {
        const bool colin = mine && ((m0 >> ox) & 1u) && ((m1 >> oy) & 1u) && zoff_lo <= zoff_hi;
        if (!__any_sync(0xffffffffu, colin)) continue;
        const long long cxl = (long long)gx + ox - 1, cyl = (long long)gy + oy - 1;
        if (cxl < 0 || cxl >= g.nx || cyl < 0 || cyl >= g.ny) continue;
        int zl = colin ? q.z + zoff_lo : INT_MAX;
        int zh = colin ? q.z + zoff_hi : INT_MIN;
        for (int o = 16; o > 0; o >>= 1) {
          zl = min(zl, __shfl_xor_sync(0xffffffffu, zl, o));
          zh = max(zh, __shfl_xor_sync(0xffffffffu, zh, o));
        }
        zl = max(zl, 0);
        zh = min(zh, g.nz - 1);
        if (zl > zh) continue;
        const int key0 = ((int)cxl * g.ny + (int)cyl) * g.nz + zl;
        auto in_cell = [&](int cz) {
          const int oz = cz - q.z + 1;
          return colin && oz >= 0 && oz <= 2 && ((m2 >> oz) & 1u);
        };
        const int J1 = cs[key0 + (zh - zl + 1)];
        int cz = zl;
        int cnext = cs[key0 + 1];
        bool in = in_cell(cz);
        for (int base = cs[key0]; base < J1; base += 32) {
          stage(base + lane, lane, base + lane < J1);
          __syncwarp();
          const int m = min(32, J1 - base);
          for (int k = 0; k < m; ++k) {
            const int j = base + k;
            while (j >= cnext) {
              ++cz;
              cnext = cs[key0 + (cz - zl) + 1];
              in = in_cell(cz);
            }
            if (in) visit(j, k);
          }
          __syncwarp();
        }
      }
    }
  }
}

}  // namespace gg
