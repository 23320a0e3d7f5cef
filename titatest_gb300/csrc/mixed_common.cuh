// Pieces shared by the two complex64 band factorisations (the barrier-stepped
// kernel of factor.cu and the pipelined kernel of factor_pipe.cu): staging of
// entering rows, fast complex square root / reciprocal and the refill of a
// register tile from the entering rows.
#pragma once

#include "async.cuh"
#include "device.cuh"

namespace crgpu {

constexpr int kStageSteps = 4;  // block steps of look-ahead for entering rows

// issue the cp.async copies of the 4 rows r0..r0+3 (padded pattern values,
// columns, right-hand side) into ring slot sl; called by the staging warp
__device__ __forceinline__ void stage_issue4(const DevProblem &P, const double2 *as, const double2 *bv, int r0,
                                             int ln, int rw, int fuse, double2 (*rv)[32], int (*rc)[32],
                                             double2 *rb) {
    const int r = ln >> 3, e0 = ln & 7;
    const int rr = r0 + r;
    if (rr < P.n) {
        for (int e = e0; e < rw; e += 8) {
            cp_async16(&rv[r][e], as + (size_t)rr * rw + e);
            cp_async4(&rc[r][e], P.col + (size_t)rr * rw + e);
        }
        if (e0 == 7 && fuse) cp_async16(&rb[r], bv + rr);
    }
    cp_commit();
}

// Principal complex square root and reciprocal from the approximate MUFU
// reciprocal square root / reciprocal (a few ulp): the complex64 factor is a
// preconditioner for the FP64 refinement.
__device__ __forceinline__ float2 csqrt_fast(float2 z) {
    const float r2 = z.x * z.x + z.y * z.y;
    if (r2 == 0.f) return cf(0.f, 0.f);
    const float r = r2 * rsqrtf(r2);
    if (z.x >= 0.f) {
        const float t2 = 0.5f * (r + z.x);
        const float it = rsqrtf(t2);
        return cf(t2 * it, 0.5f * z.y * it);
    }
    const float t2 = 0.5f * (r - z.x);
    const float it = rsqrtf(t2);
    return cf(0.5f * fabsf(z.y) * it, copysignf(t2 * it, z.y));
}
__device__ __forceinline__ float2 crecip_fast(float2 d) {
    const float q = __fdividef(1.0f, d.x * d.x + d.y * d.y);
    return cf(d.x * q, -d.y * q);
}

// Tile entries from the 4 entering rows staged by slot in nb[4][WP]: a tile
// of block row B takes row a's slots of its column block, a tile of block
// column B takes row b's slots of its row block, the diagonal tile takes the
// rows among themselves.  128-bit shared loads.
template <int WP>
__device__ __forceinline__ void refill_tile(float2 (&w)[4][4], const float2 (*nb)[WP], bool rowB, bool colB,
                                            int sa0, int sb0) {
    if (rowB && colB) {
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) w[a][b] = nb[a > b ? a : b][sb0 + (a > b ? b : a)];
    } else if (rowB) {
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const float4 v0 = *(const float4 *)&nb[a][sb0];
            const float4 v1 = *(const float4 *)&nb[a][sb0 + 2];
            w[a][0] = cf(v0.x, v0.y);
            w[a][1] = cf(v0.z, v0.w);
            w[a][2] = cf(v1.x, v1.y);
            w[a][3] = cf(v1.z, v1.w);
        }
    } else {
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const float4 v0 = *(const float4 *)&nb[b][sa0];
            const float4 v1 = *(const float4 *)&nb[b][sa0 + 2];
            w[0][b] = cf(v0.x, v0.y);
            w[1][b] = cf(v0.z, v0.w);
            w[2][b] = cf(v1.x, v1.y);
            w[3][b] = cf(v1.z, v1.w);
        }
    }
}

}  // namespace crgpu
