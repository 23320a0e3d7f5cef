// Complex64 band factorisation (src/chol.f90:7-88, with the forward
// substitution of src/vre.f90:45-56 fused in) for band widths up to 207,
// where the window no longer fits in registers.
//
// The algorithm is that of k_factor_mixed (factor.cu): rows j .. j+WP-1 in
// slots r mod WP, the lower triangle of slot pairs in 4x4 tiles, 4 pivot
// columns per step (gather -> panel -> rank-4 update with refill of the
// entering rows), two block barriers per step.  The tiles live in shared
// memory instead of registers, entry-major (entry k of tile t at
// tiles[k][t]) so that consecutive threads touch consecutive banks; each of
// kSmemTileThreads threads owns ceil(T / kSmemTileThreads) tiles and loads,
// updates and stores them once per step.  At WP = 208 the tiles take 176 KB
// of the block's 227 KB.
#include <mutex>

#include "async.cuh"
#include "crgpu_internal.h"
#include "device.cuh"
#include "kernels.h"
#include "mixed_common.cuh"

namespace crgpu {

namespace {

constexpr int kSmemTileThreads = 512;
constexpr int kSmemThreads = kSmemTileThreads + 32;  // + the staging warp

template <int WP>
struct SmemWin {
    static constexpr int NB = WP / 4;
    static constexpr int T = NB * (NB + 1) / 2;
    static constexpr int TPT = (T + kSmemTileThreads - 1) / kSmemTileThreads;  // tiles per thread
    float2 tiles[16][T];               // entry-major
    float2 panel[4][WP];               // pivot columns by slot
    float2 lp[4][2][NB][2];            // L entries: lp[q][(s&3)>>1][s>>2][s&1]
    float2 nbuf[3][4][WP];             // entering rows by slot, triple buffered
    double2 ring_val[kStageSteps][4][32];
    double2 ring_b[kStageSteps][4];
    int ring_col[kStageSteps][4][32];
    float2 bsh[WP];                    // right-hand side by slot
    float2 bnew[3][4];
    float2 ysh[4];
    float2 Ldsh[4][4];                 // factor of the next 4x4 diagonal block
    float2 dinvsh[4];
    int bad;
};

__device__ __forceinline__ void tile_of(int t, int &bi, int &bj) {
    bi = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
    while ((bi + 1) * (bi + 2) / 2 <= t) bi++;
    while (bi * (bi + 1) / 2 > t) bi--;
    bj = t - bi * (bi + 1) / 2;
}

template <int T>
__device__ __forceinline__ void load_tile(const float2 (*tl)[T], int t, float2 (&w)[4][4]) {
#pragma unroll
    for (int k = 0; k < 16; k++) w[k >> 2][k & 3] = tl[k][t];
}

template <int T>
__device__ __forceinline__ void store_tile(float2 (*tl)[T], int t, const float2 (&w)[4][4]) {
#pragma unroll
    for (int k = 0; k < 16; k++) tl[k][t] = w[k >> 2][k & 3];
}

// In-place L L^T of a 4x4 diagonal tile (rows j0..j0+3; rows beyond n get a
// unit pivot); publishes L and 1/diag
__device__ __forceinline__ void factor_diag4_s(float2 (&w)[4][4], int j0, int n, float2 (*Ld)[4], float2 *dinv,
                                               int *bad, int ldc) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float2 d;
        if (j0 + q < n) {
            const float2 v = w[q][q];
            const float r2 = v.x * v.x + v.y * v.y;
            if (!(r2 > 0.f) || !isfinite(r2) || (ldc && !(v.x > 0.f))) *bad = 28;
            d = csqrt_fast(v);
        } else {
            d = cf(1.f, 0.f);
        }
        const float2 di = crecip_fast(d);
        w[q][q] = d;
        Ld[q][q] = d;
        dinv[q] = di;
#pragma unroll
        for (int r = q + 1; r < 4; r++) {
            w[r][q] = cmulf(w[r][q], di);
            Ld[r][q] = w[r][q];
        }
#pragma unroll
        for (int r = q + 1; r < 4; r++)
#pragma unroll
            for (int c = q + 1; c <= r; c++) w[r][c] = cfmsf(w[r][c], w[r][q], w[c][q]);
    }
}

}  // namespace

template <int WP>
__global__ __launch_bounds__(kSmemThreads, 1) void k_factor_mixed_smem(DevProblem P, DevBatch B, int fuse) {
    using W = SmemWin<WP>;
    constexpr int NB = W::NB, T = W::T, TPT = W::TPT;
    constexpr int D = kStageSteps;
    extern __shared__ __align__(16) unsigned char smw_raw[];
    W &S = *reinterpret_cast<W *>(smw_raw);
    const int n = P.n, mb = P.mb, Wb = mb + 1, rw = P.rw;
    const int tid = threadIdx.x;
    const int ln = tid - kSmemTileThreads;  // lane in the staging warp (< 0 elsewhere)
    const bool tile_thread = ln < 0;
    int tbi[TPT], tbj[TPT];
#pragma unroll
    for (int u = 0; u < TPT; u++) {
        const int t = tid + u * kSmemTileThreads;
        tbi[u] = tbj[u] = -1;
        if (tile_thread && t < T) tile_of(t, tbi[u], tbj[u]);
    }
    const int nblk = (n + 3) / 4;
    for (int s = blockIdx.x; s < B.nsys; s += gridDim.x) {
        float2 *L = (float2 *)B.L + (size_t)s * B.lpitch;
        float2 *yv = (float2 *)B.y + (size_t)s * n;
        const double2 *as = B.As + (size_t)s * P.nnz;
        const double2 *bv = B.b + (size_t)s * n;
        // ---- initial window: slot q holds row q; the rows enter 4 at a time
        for (int q = tid; q < WP; q += blockDim.x) {
            S.bsh[q] = (q < n && fuse) ? to_f(bv[q]) : cf(0.f, 0.f);
#pragma unroll
            for (int r = 0; r < 4; r++) S.nbuf[0][r][q] = S.nbuf[1][r][q] = S.nbuf[2][r][q] = cf(0.f, 0.f);
        }
        for (int q = tid; q < 16 * T; q += blockDim.x) (&S.tiles[0][0])[q] = cf(0.f, 0.f);
        if (tid < 12) S.bnew[tid / 4][tid % 4] = cf(0.f, 0.f);
        if (tid == 0) S.bad = 0;
        for (int Jw = 0; Jw < NB; Jw++) {
            __syncthreads();
            if (ln >= 0) {
                const int r = ln >> 3, e0 = ln & 7, rr = 4 * Jw + r;
                if (rr < n)
                    for (int e = e0; e < rw; e += 8) {
                        const int c = P.col[(size_t)rr * rw + e];
                        if (c >= 0) S.nbuf[0][r][c] = to_f(as[(size_t)rr * rw + e]);
                    }
            }
            __syncthreads();
#pragma unroll
            for (int u = 0; u < TPT; u++) {
                const int bi = tbi[u], bj = tbj[u];
                if (bi >= 0 && (bi == Jw || bj == Jw)) {
                    float2 w[4][4];
                    refill_tile(w, S.nbuf[0], bi == Jw, bj == Jw, 4 * bi, 4 * bj);
                    store_tile(S.tiles, tid + u * kSmemTileThreads, w);
                }
            }
            __syncthreads();
            if (tid < WP) {
#pragma unroll
                for (int r = 0; r < 4; r++) S.nbuf[0][r][tid] = cf(0.f, 0.f);
            }
        }
        __syncthreads();
        if (tid == 0) {  // tile (0, 0) is tile 0
            float2 w[4][4];
            load_tile(S.tiles, 0, w);
            factor_diag4_s(w, 0, n, S.Ldsh, S.dinvsh, &S.bad, P.ldc);
            store_tile(S.tiles, 0, w);
        }
        if (ln >= 0) {
            // rows WP..WP+3 enter at block step 0: staged directly
            const int r = ln >> 3, e0 = ln & 7, rr = WP + r;
            if (rr < n) {
                for (int e = e0; e < rw; e += 8) {
                    const int c = P.col[(size_t)rr * rw + e];
                    if (c >= 0) S.nbuf[0][r][c % WP] = to_f(as[(size_t)rr * rw + e]);
                }
                if (e0 == 7 && fuse) S.bnew[0][r] = to_f(bv[rr]);
            }
            for (int q = 0; q < D; q++) {
                const int sl = (q + 1) % D;
                stage_issue4(P, as, bv, WP + 4 * (q + 1), ln, rw, fuse, S.ring_val[sl], S.ring_col[sl], S.ring_b[sl]);
            }
        }
        int Bk = 0;
        for (int J = 0; J < nblk; J++) {
            const int j = 4 * J, cur = J % 3;
            // ---- 1. gather the pivot columns
#pragma unroll
            for (int u = 0; u < TPT; u++) {
                const int bi = tbi[u], bj = tbj[u];
                if (bi >= 0 && (bi == Bk) != (bj == Bk)) {
                    float2 w[4][4];
                    load_tile(S.tiles, tid + u * kSmemTileThreads, w);
                    if (bi == Bk) {
#pragma unroll
                        for (int a = 0; a < 4; a++) {
                            float4 *d = (float4 *)&S.panel[a][4 * bj];
                            d[0] = make_float4(w[a][0].x, w[a][0].y, w[a][1].x, w[a][1].y);
                            d[1] = make_float4(w[a][2].x, w[a][2].y, w[a][3].x, w[a][3].y);
                        }
                    } else {
#pragma unroll
                        for (int b = 0; b < 4; b++) {
                            float4 *d = (float4 *)&S.panel[b][4 * bi];
                            d[0] = make_float4(w[0][b].x, w[0][b].y, w[1][b].x, w[1][b].y);
                            d[1] = make_float4(w[2][b].x, w[2][b].y, w[3][b].x, w[3][b].y);
                        }
                    }
                }
            }
            __syncthreads();
            // ---- 2. panel: L entries of every window row for columns j..j+3
            if (tid < WP) {
                const int sl = tid, blk = sl >> 2, b4 = sl & 3;
                int dist = sl - 4 * Bk;
                if (dist < 0) dist += WP;
                const int r_s = j + dist;
                float2 a[4];
                int band0;
                if (blk == Bk) {
                    if (j + b4 < n) {  // row j+b4 of the diagonal block factor
                        float2 *row = L + (size_t)(j + b4) * Wb + (mb - b4);
                        for (int q = 0; q <= b4; q++)
                            if (mb - b4 + q >= 0) row[q] = S.Ldsh[b4][q];
                    }
                    band0 = WP + b4 - mb;  // the entering row's first pivot column in its band
#pragma unroll
                    for (int q = 0; q < 4; q++) a[q] = (q >= band0) ? S.nbuf[cur][b4][4 * Bk + q] : cf(0.f, 0.f);
                } else {
                    band0 = dist - mb;
#pragma unroll
                    for (int q = 0; q < 4; q++) a[q] = S.panel[q][sl];
                }
                const int r_l = (blk == Bk) ? j + WP + b4 : r_s;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 l = cmulf(a[q], S.dinvsh[q]);
#pragma unroll
                    for (int r = q + 1; r < 4; r++) a[r] = cfmsf(a[r], l, S.Ldsh[r][q]);
                    a[q] = l;
                    S.lp[q][b4 >> 1][blk][b4 & 1] = l;
                }
                if (r_l < n && band0 < 4) {
                    float2 *row = L + (size_t)r_l * Wb + (j - r_l + mb);  // column j
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (q >= band0) row[q] = a[q];
                }
            }
            if (ln == 0 && fuse) {  // forward substitution of the 4 pivot entries
                float2 bb[4];
#pragma unroll
                for (int q = 0; q < 4; q++) bb[q] = S.bsh[4 * Bk + q];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 yq = cmulf(bb[q], S.dinvsh[q]);
                    S.ysh[q] = yq;
                    if (j + q < n) yv[j + q] = yq;
#pragma unroll
                    for (int r = q + 1; r < 4; r++) bb[r] = cfmsf(bb[r], S.Ldsh[r][q], yq);
                }
            }
            __syncthreads();
            // ---- 3. rank-4 update, or refill with the entering rows
            const int Bn = (Bk + 1 == NB) ? 0 : Bk + 1;
#pragma unroll
            for (int u = 0; u < TPT; u++) {
                const int bi = tbi[u], bj = tbj[u];
                if (bi < 0) continue;
                const int t = tid + u * kSmemTileThreads;
                float2 w[4][4];
                if (bi == Bk || bj == Bk) refill_tile(w, S.nbuf[cur], bi == Bk, bj == Bk, 4 * bi, 4 * bj);
                else load_tile(S.tiles, t, w);
#pragma unroll 1
                for (int q = 0; q < 4; q++) {
                    const float4 a01 = *(const float4 *)&S.lp[q][0][bi][0];
                    const float4 a23 = *(const float4 *)&S.lp[q][1][bi][0];
                    const float4 b01 = *(const float4 *)&S.lp[q][0][bj][0];
                    const float4 b23 = *(const float4 *)&S.lp[q][1][bj][0];
                    const float2 la[4] = {cf(a01.x, a01.y), cf(a01.z, a01.w), cf(a23.x, a23.y), cf(a23.z, a23.w)};
                    const float2 lb[4] = {cf(b01.x, b01.y), cf(b01.z, b01.w), cf(b23.x, b23.y), cf(b23.z, b23.w)};
#pragma unroll
                    for (int a = 0; a < 4; a++)
#pragma unroll
                        for (int b = 0; b < 4; b++) w[a][b] = cfmsf(w[a][b], la[a], lb[b]);
                }
                if (bi == Bn && bj == Bn) factor_diag4_s(w, j + 4, n, S.Ldsh, S.dinvsh, &S.bad, P.ldc);
                store_tile(S.tiles, t, w);
            }
            if (ln >= 0) {
                // staging warp: right-hand side update, clearing of the buffer
                // after next, entering rows of the next step
                if (fuse)
                    for (int t = ln; t < WP; t += 32) {
                        const int blk = t >> 2, b4 = t & 3;
                        float2 v = (blk == Bk) ? S.bnew[cur][b4] : S.bsh[t];
#pragma unroll
                        for (int q = 0; q < 4; q++) v = cfmsf(v, S.lp[q][b4 >> 1][blk][b4 & 1], S.ysh[q]);
                        S.bsh[t] = v;
                    }
                for (int t = ln; t < WP; t += 32) {
#pragma unroll
                    for (int r = 0; r < 4; r++) S.nbuf[(J + 2) % 3][r][t] = cf(0.f, 0.f);
                }
                __syncwarp();
                const int sl = (J + 1) % D, r = ln >> 3, e0 = ln & 7;
                const int rr = j + 4 + WP + r;
                cp_wait<D - 1>();
                if (rr < n) {
                    for (int e = e0; e < rw; e += 8) {
                        const int c = S.ring_col[sl][r][e];
                        if (c >= 0) S.nbuf[(J + 1) % 3][r][c % WP] = to_f(S.ring_val[sl][r][e]);
                    }
                    if (e0 == 7 && fuse) S.bnew[(J + 1) % 3][r] = to_f(S.ring_b[sl][r]);
                } else if (e0 == 7) {
                    S.bnew[(J + 1) % 3][r] = cf(0.f, 0.f);
                }
                stage_issue4(P, as, bv, rr - r + 4 * D, ln, rw, fuse, S.ring_val[sl], S.ring_col[sl], S.ring_b[sl]);
            }
            Bk = Bn;
        }
        if (ln >= 0) cp_wait<0>();
        __syncthreads();
        if (tid == 0 && S.bad) atomicCAS(&B.status[s], 0, S.bad);
    }
}

#define CRGPU_SMEM_SIZES(X) X(192) X(208)

int mixed_smem_window_supported(int W) {
#define X(S) if (W <= S) return S;
    CRGPU_SMEM_SIZES(X)
#undef X
    return 0;
}

int launch_factor_mixed_smem(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st) {
    const int W = P.mb + 1;
    const int grid = B.nsys < nsm ? B.nsys : nsm;
#define X(S)                                                                                          \
    if (W <= S) {                                                                                     \
        static_assert(sizeof(SmemWin<S>) <= 227 * 1024, "window exceeds the shared memory of a block"); \
        static std::once_flag once_##S;                                                               \
        std::call_once(once_##S, [] {                                                                 \
            cudaFuncSetAttribute(k_factor_mixed_smem<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                 (int)sizeof(SmemWin<S>));                                            \
        });                                                                                           \
        k_factor_mixed_smem<S><<<grid, kSmemThreads, sizeof(SmemWin<S>), st>>>(P, B, fuse);          \
        return 0;                                                                                     \
    }
    CRGPU_SMEM_SIZES(X)
#undef X
    return ERR_UNSUPPORTED;
}

}  // namespace crgpu
