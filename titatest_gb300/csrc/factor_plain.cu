// Complex128 band factorisation (src/chol.f90:7-88) with the active window
// held in registers, for band widths mb < kPlainRegMaxW.
//
// The active window at column j is the trailing block of rows and columns
// j .. j+mb (W = mb+1 of them); row r sits in slot r mod W.  Its entries are
// complex symmetric, so the window is stored once per unordered slot pair
// {x, y}: W(W+1)/2 entries.  For every j exactly one orientation of a pair is
// inside the window (the pairs of the pivot slot p = j mod W hold the pivot
// column; once that column retires, the same pairs hold the row entering at
// slot p), so the storage needs no orientation logic, and the rank-1 update
//     A(x, y) -= l_x l_y   (no conjugation, src/chol.f90:58)
// is the same for either orientation.  Thread t owns the pairs t, t + NT, ...
// of the packed triangle for the whole factorisation, values in registers.
//
// Column j: the owners of the pivot slot's pairs publish the pivot column
// (barrier); one thread takes the square root and reciprocal of the diagonal
// and the fused forward substitution y_j = b_j / l_jj (src/vre.f90:45-56),
// while a staging warp scatters the row entering at slot p from its cp.async
// ring (barrier); one thread per window row forms its entry of L, stores it
// in the band layout a((mb+1)*sanz) and updates its right-hand side
// (barrier); then every thread updates its pairs, and the pivot slot's pairs
// take the entering row.  The FP64 pipe bounds the update: W(W-1)/2 complex
// multiply-adds per column, one system per SM.
#include "async.cuh"
#include "crgpu_internal.h"
#include "device.cuh"
#include "kernels.h"

namespace crgpu {

namespace {

constexpr int kPlainRegThreads = 512;
constexpr int kPlainRegMaxW = 128;  // slots (mb + 1); W(W+1)/2 pairs over 512 threads, at most 16 each
constexpr int kRingRows = 4;        // entering rows staged ahead
constexpr int kRingCap = 64;        // padded row width the ring holds
constexpr int kStageWarp = kPlainRegThreads / 32 - 1;

// x >= y of packed index k = x(x+1)/2 + y
__device__ __forceinline__ void unpack_pair(int k, int &x, int &y) {
    int a = (int)((sqrtf(8.f * (float)k + 1.f) - 1.f) * 0.5f);
    while ((a + 1) * (a + 2) / 2 <= k) a++;
    while (a * (a + 1) / 2 > k) a--;
    x = a;
    y = k - a * (a + 1) / 2;
}

// the padded lower-pattern row r (its rw entries) and b(r) into ring slot sl;
// one commit group per lane
__device__ __forceinline__ void ring_issue(const DevProblem &P, const double2 *as, const double2 *bv, int r, int ln,
                                           double2 (*rv)[kRingCap], int (*rc)[kRingCap], double2 *rb, int sl,
                                           int fuse) {
    if (r < P.n) {
        for (int e = ln; e < P.rw; e += 32) {
            cp_async16(&rv[sl][e], as + (size_t)r * P.rw + e);
            cp_async4(&rc[sl][e], P.col + (size_t)r * P.rw + e);
        }
        if (ln == 0 && fuse) cp_async16(&rb[sl], bv + r);
    }
    cp_commit();
}

template <int NP>
__global__ __launch_bounds__(kPlainRegThreads, 1) void k_factor_plain_reg(DevProblem P, DevBatch B, int fuse) {
    constexpr int NT = kPlainRegThreads;
    const int n = P.n, mb = P.mb, W = mb + 1, rw = P.rw;
    const int T = W * (W + 1) / 2;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    __shared__ double2 pcol[kPlainRegMaxW];     // the pivot column by slot (pcol[p]: the diagonal)
    __shared__ double2 lsh[kPlainRegMaxW];      // this column's L entries by slot (0 at the pivot slot)
    __shared__ double2 nrow[2][kPlainRegMaxW];  // the entering row by slot of its column
    __shared__ double2 bsh[kPlainRegMaxW];      // right-hand side by slot
    __shared__ __align__(16) double2 ring_val[kRingRows][kRingCap];
    __shared__ int ring_col[kRingRows][kRingCap];
    __shared__ __align__(16) double2 ring_b[kRingRows];
    __shared__ double2 dinv_sh, y_sh, bnext;
    __shared__ int bad;

    // this thread's pairs: slots packed as x | y << 8 (0xffff: none)
    uint32_t xy[NP];
#pragma unroll
    for (int i = 0; i < NP; i++) {
        const int k = tid + i * NT;
        int x = 0, y = 0;
        if (k < T) unpack_pair(k, x, y);
        xy[i] = k < T ? (uint32_t)(x | (y << 8)) : 0xffffu;
    }

    for (int s = blockIdx.x; s < B.nsys; s += gridDim.x) {
        double2 *L = (double2 *)B.L + (size_t)s * B.lpitch;
        const double2 *as = B.As + (size_t)s * P.nnz;
        const double2 *bv = B.b + (size_t)s * n;
        double2 *yv = (double2 *)B.y + (size_t)s * n;
        __syncthreads();
        if (tid == 0) bad = 0;
        // band entries before column 0 (rows 0..mb-1) are outside the matrix: zero
        for (int q = tid; q < mb * W; q += NT) {
            const int r = q / W, o = q % W;
            if (r < n && o < mb - r) L[(size_t)r * W + o] = cz(0.0, 0.0);
        }
        for (int q = tid; q < W; q += NT) bsh[q] = (q < n && fuse) ? bv[q] : cz(0.0, 0.0);
        // the initial window (rows 0..mb in slots 0..mb): each pair from its row's pattern
        double2 v[NP];
#pragma unroll
        for (int i = 0; i < NP; i++) {
            v[i] = cz(0.0, 0.0);
            if (xy[i] == 0xffffu) continue;
            const int x = xy[i] & 0xff, y = xy[i] >> 8;
            if (x >= n) continue;
            for (int e = 0; e < rw; e++) {
                if (P.col[(size_t)x * rw + e] == y) {
                    v[i] = as[(size_t)x * rw + e];
                    break;
                }
            }
        }
        if (warp == kStageWarp) {
            for (int q = 0; q < kRingRows; q++) ring_issue(P, as, bv, W + q, lane, ring_val, ring_col, ring_b, q, fuse);
        }
        __syncthreads();

        for (int j = 0; j < n; j++) {
            const int p = j % W, cur = j & 1;
            // ---- 1. the pivot column (and diagonal) from the owners of slot p's pairs;
            //      the staging warp clears the entering row's buffer meanwhile
#pragma unroll
            for (int i = 0; i < NP; i++) {
                const int x = xy[i] & 0xff, y = xy[i] >> 8;
                if (x == p || y == p) pcol[x == p ? y : x] = v[i];
            }
            if (warp == kStageWarp)
                for (int q = lane; q < W; q += 32) nrow[cur][q] = cz(0.0, 0.0);
            __syncthreads();
            // ---- 2. l_jj = sqrt(a_jj), its reciprocal, y_j; the row j + W that enters
            //      slot p after this column, from the ring
            if (tid == 0) {
                const double2 a = pcol[p];
                if (!(cabsd(a) > 0.0) || (P.ldc && !(a.x > 0.0))) bad = 28;  // src/chol.f90:67-71, choldc.f90:66-70
                const double2 d = csqrtd(a);
                L[(size_t)j * W + mb] = d;
                const double2 di = crecip(d);
                dinv_sh = di;
                if (fuse) {
                    const double2 yj = cmul(bsh[p], di);
                    yv[j] = yj;
                    y_sh = yj;
                }
            }
            if (warp == kStageWarp) {
                const int sl = j % kRingRows, r = j + W;
                cp_wait<kRingRows - 1>();
                __syncwarp();
                if (r < n) {
                    for (int e = lane; e < rw; e += 32) {
                        const int c = ring_col[sl][e];
                        if (c >= 0) nrow[cur][c % W] = ring_val[sl][e];
                    }
                }
                if (lane == 0) bnext = (r < n && fuse) ? ring_b[sl] : cz(0.0, 0.0);
                __syncwarp();
                ring_issue(P, as, bv, r + kRingRows, lane, ring_val, ring_col, ring_b, sl, fuse);
            }
            __syncthreads();
            // ---- 3. L entries of column j and the right-hand sides (one thread per window row)
            if (tid < W) {
                const int x = tid;
                if (x == p) {
                    lsh[x] = cz(0.0, 0.0);
                    bsh[x] = bnext;  // the entering row's right-hand side
                } else {
                    const int a = x > p ? x - p : x - p + W;  // slot x holds row j + a
                    const int r = j + a;
                    double2 l = cz(0.0, 0.0);
                    if (r < n) {
                        l = cmul(pcol[x], dinv_sh);
                        L[(size_t)r * W + (mb - a)] = l;
                        if (fuse) bsh[x] = cfms(bsh[x], l, y_sh);
                    }
                    lsh[x] = l;
                }
            }
            __syncthreads();
            // ---- 4. rank-1 update of the window; the pivot slot's pairs take the entering row
#pragma unroll
            for (int i = 0; i < NP; i++) {
                if (xy[i] == 0xffffu) continue;
                const int x = xy[i] & 0xff, y = xy[i] >> 8;
                if (x == p || y == p) {
                    v[i] = nrow[cur][x == p ? y : x];
                } else {
                    v[i] = cfms(v[i], lsh[x], lsh[y]);
                }
            }
        }
        if (warp == kStageWarp) cp_wait<0>();
        __syncthreads();
        if (tid == 0 && bad) atomicCAS(&B.status[s], 0, bad);
    }
}

}  // namespace

// pairs per thread for band width mb (0: the window does not fit in registers)
static int plain_reg_np(int mb) {
    const int W = mb + 1;
    if (W > kPlainRegMaxW) return 0;
    const int T = W * (W + 1) / 2;
    const int np = (T + kPlainRegThreads - 1) / kPlainRegThreads;
    return np <= 4 ? 4 : np <= 8 ? 8 : np <= 12 ? 12 : np <= 16 ? 16 : 0;
}

bool launch_factor_plain_reg(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st) {
    const int np = plain_reg_np(P.mb);
    if (!np || P.rw > kRingCap) return false;
    const int grid = B.nsys < nsm ? B.nsys : nsm;
    switch (np) {
        case 4: k_factor_plain_reg<4><<<grid, kPlainRegThreads, 0, st>>>(P, B, fuse); break;
        case 8: k_factor_plain_reg<8><<<grid, kPlainRegThreads, 0, st>>>(P, B, fuse); break;
        case 12: k_factor_plain_reg<12><<<grid, kPlainRegThreads, 0, st>>>(P, B, fuse); break;
        default: k_factor_plain_reg<16><<<grid, kPlainRegThreads, 0, st>>>(P, B, fuse); break;
    }
    return true;
}

}  // namespace crgpu
