// Banded complex-symmetric L L^T factorisation (no conjugation) of the scaled
// systems, src/chol.f90:7-88, with the forward substitution of
// src/vre.f90:45-56 fused in.
//
// Band layout (the reference's a((mb+1)*sanz)): row i occupies
// L[i*(mb+1) .. i*(mb+1)+mb], entry (i, c) at offset c - i + mb, diagonal
// last.  Rows are materialised from the sparse scaled values just before they
// enter the active window.
//
// Both kernels are right-looking: at step j the pivot column j is divided by
// sqrt(a_jj) and the (mb x mb) trailing triangle receives the rank-1 update.
// Each entry therefore sees its updates in increasing j, the same summation
// order as the reference's left-looking dot products.
//
//  * k_factor_plain (complex128): the window is updated in place in the band
//    buffer (global memory; the active ~(mb+1)^2 * 16 B stays in L2).  On
//    GB300 the FP64 pipe, not memory, bounds this kernel.
//  * k_factor_mixed<WP> (complex64): the (mb+1) x (mb+1) window lives in
//    registers.  Window rows rotate through W = mb+1 slots (row r in slot
//    r mod W); every thread owns a fixed 4x4 tile of the lower triangle of
//    slot pairs, so a step needs no data movement: the retiring pivot row's
//    slot is refilled with the entering row.
#include "device.cuh"
#include "crgpu_internal.h"
#include "kernels.h"

namespace crgpu {

// ---------------------------------------------------------------------------
// complex128, window in L2
// ---------------------------------------------------------------------------
__device__ __forceinline__ void materialize_row_c128(const DevProblem &P, const double2 *as, double2 *L,
                                                     int r, int lane) {
    const int W = P.mb + 1;
    double2 *row = L + (size_t)r * W;
    for (int o = lane; o < W; o += 32) row[o] = cz(0.0, 0.0);
    __syncwarp();
    int p0 = P.rowptr[r], p1 = P.rowptr[r + 1];
    for (int p = p0 + lane; p < p1; p += 32) row[P.col[p] - r + P.mb] = as[p];
    __syncwarp();
}

constexpr int kPlainThreads = 256;

__global__ __launch_bounds__(kPlainThreads) void k_factor_plain(DevProblem P, DevBatch B, int fuse) {
    const int n = P.n, mb = P.mb, W = mb + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = kPlainThreads / 32;
    extern __shared__ double2 sm_plain[];
    double2 *lcol = sm_plain;          // W
    __shared__ double2 dsh, ysh;
    __shared__ int bad;
    for (int s = blockIdx.x; s < B.nsys; s += gridDim.x) {
        double2 *L = (double2 *)B.L + (size_t)s * n * W;
        const double2 *as = B.As + (size_t)s * P.nnz;
        double2 *bv = B.b + (size_t)s * n;
        double2 *yv = (double2 *)B.y + (size_t)s * n;
        if (tid == 0) bad = 0;
        int r0 = min(W, n);
        for (int r = warp; r < r0; r += nwarps) materialize_row_c128(P, as, L, r, lane);
        __syncthreads();
        for (int j = 0; j < n; j++) {
            if (tid == 0) {
                double2 a = L[(size_t)j * W + mb];
                if (!(cabsd(a) > 0.0)) bad = 28;  // src/chol.f90:67-71
                double2 d = csqrtd(a);
                L[(size_t)j * W + mb] = d;
                dsh = d;
                if (fuse) {
                    double2 yj = cdiv(bv[j], d);
                    yv[j] = yj;
                    ysh = yj;
                }
            }
            __syncthreads();
            const double2 d = dsh;
            const int R = min(mb, n - 1 - j);
            for (int t = tid; t < R; t += kPlainThreads) {
                int r = j + 1 + t;
                size_t idx = (size_t)r * W + (mb - 1 - t);
                double2 l = cdiv(L[idx], d);
                L[idx] = l;
                lcol[t] = l;
                if (fuse) bv[r] = cfms(bv[r], l, ysh);
            }
            __syncthreads();
            // trailing update: rows r = j+1+a, columns c = j+1+b, b <= a
            for (int a = warp; a < R; a += nwarps) {
                double2 la = lcol[a];
                double2 *row = L + (size_t)(j + 1 + a) * W + (mb - a);  // column j+1
                for (int b = lane; b <= a; b += 32) row[b] = cfms(row[b], la, lcol[b]);
            }
            if (j + W < n && warp == nwarps - 1) materialize_row_c128(P, as, L, j + W, lane);
            __syncthreads();
        }
        if (tid == 0 && bad) atomicCAS(&B.status[s], 0, bad);
        __syncthreads();
    }
}

void launch_factor_plain(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st) {
    int grid = B.nsys < nsm * 4 ? B.nsys : nsm * 4;
    size_t smem = sizeof(double2) * (P.mb + 1);
    k_factor_plain<<<grid, kPlainThreads, smem, st>>>(P, B, fuse);
}

// ---------------------------------------------------------------------------
// complex64, window in registers
// ---------------------------------------------------------------------------
template <int WP>
struct MixCfg {
    static constexpr int NB = WP / 4;
    static constexpr int T = NB * (NB + 1) / 2;
    static constexpr int NT = ((T + 31) / 32) * 32;
};

// value of the scaled matrix entry (row, col), row >= col, from the pattern
__device__ __forceinline__ float2 lookup_f(const DevProblem &P, const double2 *as, int row, int col) {
    for (int p = P.rowptr[row]; p < P.rowptr[row + 1]; p++)
        if (P.col[p] == col) return to_f(as[p]);
    return cf(0.f, 0.f);
}

template <int WP>
__global__ __launch_bounds__(MixCfg<WP>::NT, 1) void k_factor_mixed(DevProblem P, DevBatch B, int fuse) {
    constexpr int T = MixCfg<WP>::T;
    const int n = P.n, mb = P.mb, W = mb + 1;
    const int tid = threadIdx.x;
    __shared__ float2 lsh[WP];
    __shared__ float2 nrow[3][WP];
    __shared__ float2 bsh[WP];
    __shared__ float2 bnew[3];
    __shared__ float2 dsh, ysh;
    __shared__ int bad;
    // tile of this thread: (bi, bj), bi >= bj
    const bool has = tid < T;
    int bi = 0, bj = 0;
    if (has) {
        int t = tid;
        bi = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
        while ((bi + 1) * (bi + 2) / 2 <= t) bi++;
        while (bi * (bi + 1) / 2 > t) bi--;
        bj = t - bi * (bi + 1) / 2;
    }
    const int sa0 = 4 * bi, sb0 = 4 * bj;
    for (int s = blockIdx.x; s < B.nsys; s += gridDim.x) {
        float2 *L = (float2 *)B.L + (size_t)s * n * W;
        float2 *yv = (float2 *)B.y + (size_t)s * n;
        const double2 *as = B.As + (size_t)s * P.nnz;
        const double2 *bv = B.b + (size_t)s * n;
        float2 w[4][4];
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int a = q >> 2, b = q & 3;
            const int sa = sa0 + a, sb = sb0 + b;
            float2 v = cf(0.f, 0.f);
            if (has && sa < W && sb < W && sa < n && sb < n) {
                const int rr = max(sa, sb), cc = min(sa, sb);
                const int p1 = P.rowptr[rr + 1];
                for (int pp = P.rowptr[rr]; pp < p1; pp++)
                    if (P.col[pp] == cc) v = to_f(as[pp]);
            }
            w[a][b] = v;
        }
        for (int q = tid; q < WP; q += blockDim.x) {
            lsh[q] = cf(0.f, 0.f);
            bsh[q] = (q < W && q < n && fuse) ? to_f(bv[q]) : cf(0.f, 0.f);
            nrow[0][q] = nrow[1][q] = nrow[2][q] = cf(0.f, 0.f);
        }
        if (tid == 0) {
            bad = 0;
            bnew[0] = bnew[1] = bnew[2] = cf(0.f, 0.f);
        }
        __syncthreads();
        // stage row W (enters at step 0) in nrow[0]
        if (tid < 32 && W < n) {
            int rn = W;
            for (int p = P.rowptr[rn] + tid; p < P.rowptr[rn + 1]; p += 32) nrow[0][P.col[p] % W] = to_f(as[p]);
            if (tid == 0 && fuse) bnew[0] = to_f(bv[rn]);
        }
        int p = 0;  // slot of row j
        for (int j = 0; j < n; j++) {
            const int cur = j % 3;
            // ---- phase A: pivot
            if (has && bi == bj && (p >> 2) == bi) {
                // explicit select: an indexed read would move the tile to local memory
                const int q3 = p & 3;
                const float2 v = q3 == 0 ? w[0][0] : (q3 == 1 ? w[1][1] : (q3 == 2 ? w[2][2] : w[3][3]));
                if (!(cabsf_(v) > 0.f) || !isfinite(v.x) || !isfinite(v.y)) bad = 28;
                float2 d = csqrtf_(v);
                dsh = d;
                L[(size_t)j * W + mb] = d;
            }
            __syncthreads();
            // ---- phase B: pivot column, refill of the retiring slot
            const float2 d = dsh;
            if (has && ((p >> 2) == bi || (p >> 2) == bj)) {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int a = q >> 2, b = q & 3;
                    const int sa = sa0 + a, sb = sb0 + b;
                    const bool ra = sa == p, rb = sb == p;
                    if (ra && rb) {
                        w[a][b] = nrow[cur][p];
                        lsh[p] = cf(0.f, 0.f);
                    } else if (ra || rb) {
                        const int other = ra ? sb : sa;
                        if (other < W) {
                            float2 l = cdivf(w[a][b], d);
                            lsh[other] = l;
                            int dist = other - p;
                            if (dist < 0) dist += W;
                            const int r = j + dist;
                            if (r < n && sa > sb) L[(size_t)r * W + (mb - dist)] = l;
                        }
                        w[a][b] = nrow[cur][other];
                    }
                }
            }
            if (fuse && tid == p) {
                float2 yj = cdivf(bsh[p], d);
                yv[j] = yj;
                ysh = yj;
                bsh[p] = bnew[cur];
            }
            __syncthreads();
            // ---- phase C: rank-1 update of the window
            if (has) {
                float2 la[4], lb[4];
#pragma unroll
                for (int a = 0; a < 4; a++) la[a] = lsh[sa0 + a];
#pragma unroll
                for (int b = 0; b < 4; b++) lb[b] = lsh[sb0 + b];
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) w[a][b] = cfmsf(w[a][b], la[a], lb[b]);
            }
            if (fuse && tid < W && tid != p) bsh[tid] = cfmsf(bsh[tid], lsh[tid], ysh);
            // stage row j+1+W for the next step; clear the buffer after it
            if (tid < W) nrow[(j + 2) % 3][tid] = cf(0.f, 0.f);
            const int rn = j + 1 + W;
            if (rn < n && tid >= blockDim.x - 32) {
                int ln = tid - (blockDim.x - 32);
                for (int q = P.rowptr[rn] + ln; q < P.rowptr[rn + 1]; q += 32)
                    nrow[(j + 1) % 3][P.col[q] % W] = to_f(as[q]);
                if (ln == 0 && fuse) bnew[(j + 1) % 3] = to_f(bv[rn]);
            } else if (rn >= n && tid == blockDim.x - 1) {
                bnew[(j + 1) % 3] = cf(0.f, 0.f);
            }
            p = (p + 1 == W) ? 0 : p + 1;
        }
        __syncthreads();
        if (tid == 0 && bad) atomicCAS(&B.status[s], 0, bad);
    }
}

#define CRGPU_MIXED_SIZES(X) X(36) X(64) X(80) X(104) X(124) X(144) X(164) X(176)

int mixed_window_supported(int W) {
#define X(S) if (W <= S) return S;
    CRGPU_MIXED_SIZES(X)
#undef X
    return 0;
}

int launch_factor_mixed(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st) {
    int W = P.mb + 1;
    int grid = B.nsys < nsm ? B.nsys : nsm;
#define X(S)                                                                   \
    if (W <= S) {                                                              \
        k_factor_mixed<S><<<grid, MixCfg<S>::NT, 0, st>>>(P, B, fuse);         \
        return 0;                                                              \
    }
    CRGPU_MIXED_SIZES(X)
#undef X
    return ERR_UNSUPPORTED;
}

}  // namespace crgpu
