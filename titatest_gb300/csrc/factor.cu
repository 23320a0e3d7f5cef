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
//  * complex128: k_factor_plain_reg (factor_plain.cu) keeps the window in
//    registers for mb < 127; wider bands use k_factor_plain, which updates the
//    window in place in the band buffer (global memory; the active
//    ~(mb+1)^2 * 16 B stays in L2).
//  * complex64, mb <= 124: k_factor_tc (tc_factor.cu) keeps the window in
//    tensor memory and applies the trailing updates with tcgen05.mma.
//  * complex64, mb > 175: k_factor_mixed_smem<WP> (factor_smem.cu), the same
//    algorithm with the tiles in shared memory.
//  * complex64, larger mb: k_factor_mixed<WP>: the (mb+1) x (mb+1) window
//    lives in registers.  Window rows rotate through W = mb+1 slots (row r in
//    slot r mod W); every thread owns a fixed 4x4 tile of the lower triangle
//    of slot pairs, so a step needs no data movement: the retiring pivot
//    row's slot is refilled with the entering row.
#include "async.cuh"
#include "device.cuh"
#include "crgpu_internal.h"
#include "kernels.h"
#include "mixed_common.cuh"

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
    for (int p = p0 + lane; p < p1; p += 32) {
        int c = P.col[p];
        if (c >= 0) row[c - r + P.mb] = as[p];
    }
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
        double2 *L = (double2 *)B.L + (size_t)s * B.lpitch;
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
                if (!(cabsd(a) > 0.0) || (P.ldc && !(a.x > 0.0))) bad = 28;  // src/chol.f90:67-71, choldc.f90:66-70
                double2 d = csqrtd(a);
                L[(size_t)j * W + mb] = d;
                double2 dinv = crecip(d);
                dsh = dinv;
                if (fuse) {
                    double2 yj = cmul(bv[j], dinv);
                    yv[j] = yj;
                    ysh = yj;
                }
            }
            __syncthreads();
            const double2 dinv = dsh;
            const int R = min(mb, n - 1 - j);
            for (int t = tid; t < R; t += kPlainThreads) {
                int r = j + 1 + t;
                size_t idx = (size_t)r * W + (mb - 1 - t);
                double2 l = cmul(L[idx], dinv);
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
    if (launch_factor_plain_reg(P, B, fuse, nsm, st)) return;  // mb < 127: window in registers
    int grid = B.nsys < nsm * 2 ? B.nsys : nsm * 2;
    size_t smem = sizeof(double2) * (P.mb + 1);
    k_factor_plain<<<grid, kPlainThreads, smem, st>>>(P, B, fuse);
}

// ---------------------------------------------------------------------------
// complex64, window in registers, 4 columns per step
//
// The window holds rows j .. j+WP-1 (WP a multiple of 4, WP >= mb+1).  Row r
// sits in slot r mod WP; slot s belongs to slot block s/4.  The 4 rows that
// enter at a block step (they replace the pivot rows, in slot block B) may
// reach back into the pivot columns when WP < mb+4: their L entries there are
// computed in the panel step like those of any other window row.  Thread t owns
// tile (bi, bj), bi >= bj, of the lower triangle of slot-block pairs and keeps
// its 4x4 complex entries in registers for the whole factorisation.
//
// Block step J factors columns j = 4J .. j+3 (pivot slot block B = J mod NB):
//   1. owners of tiles in block row/column B copy the 4 pivot columns into
//      the panel (shared memory);
//   2. one thread per slot computes its 4 entries of L from the 4x4 diagonal
//      block factor (computed at the end of the previous step by the owner
//      of that tile) by the same right-looking recurrence as chol; thread 0
//      does the forward substitution of the 4 right-hand-side entries;
//   3. every tile applies the rank-4 update; the tiles of block row/column B
//      first take the values of the 4 entering rows (staged through a
//      cp.async ring) and then get the same update.
// Two barriers per 4 columns.
// ---------------------------------------------------------------------------
template <int WP>
struct MixCfg {
    static constexpr int NB = WP / 4;
    static constexpr int T = NB * (NB + 1) / 2;      // tiles, one per thread
    static constexpr int NT = ((T + 31) / 32) * 32 + 32;  // + a staging warp without tiles
};

// In-place L L^T of the 4x4 diagonal tile held in registers (rows j0..j0+3);
// rows beyond n get a unit pivot.  Publishes L and 1/diag to shared memory.
__device__ __forceinline__ void factor_diag4(float2 (&w)[4][4], int j0, int n, float2 (*Ld)[4], float2 *dinv,
                                             int *bad, int ldc) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float2 d;
        if (j0 + q < n) {
            const float2 v = w[q][q];
            if (!(cabsf_(v) > 0.f) || !isfinite(v.x) || !isfinite(v.y) || (ldc && !(v.x > 0.f))) *bad = 28;
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

template <int WP>
__global__ __launch_bounds__(MixCfg<WP>::NT, (WP <= 64 ? 4 : 1)) void k_factor_mixed(DevProblem P, DevBatch B, int fuse) {
    constexpr int NB = MixCfg<WP>::NB, T = MixCfg<WP>::T;
    constexpr int D = kStageSteps;
    const int n = P.n, mb = P.mb, Wb = mb + 1, rw = P.rw;
    const int tid = threadIdx.x;
    const int ln = tid - (int)(blockDim.x - 32);  // lane in the staging warp (< 0 elsewhere)
    __shared__ __align__(16) float2 panel[4][WP];  // pivot columns: panel[q][s] = a(row of slot s, j+q)
    // L entries of the step: L(row of slot s, j+q) at lp[q][(s&3)>>1][s>>2][s&1]
    __shared__ __align__(16) float2 lp[4][2][NB][2];
    __shared__ __align__(16) float2 nbuf[3][4][WP];  // entering rows by slot, triple buffered
    __shared__ float2 bsh[WP];              // right-hand side by slot
    __shared__ float2 bnew[3][4];
    __shared__ float2 ysh[4];
    __shared__ float2 Ldsh[4][4];           // factor of the next 4x4 diagonal block (lower)
    __shared__ float2 dinvsh[4];            // reciprocals of its diagonal
    __shared__ int bad;
    __shared__ __align__(16) double2 ring_val[D][4][32];
    __shared__ int ring_col[D][4][32];
    __shared__ __align__(16) double2 ring_b[D][4];
    // tile of this thread
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
    const int nblk = (n + 3) / 4;
    for (int s = blockIdx.x; s < B.nsys; s += gridDim.x) {
        float2 *L = (float2 *)B.L + (size_t)s * B.lpitch;
        float2 *yv = (float2 *)B.y + (size_t)s * n;
        const double2 *as = B.As + (size_t)s * P.nnz;
        const double2 *bv = B.b + (size_t)s * n;
        // ---- initial window: slot q holds row q.  The rows enter 4 at a time
        // through the refill path (rows only reach back, so block bi's rows
        // complete every tile of block row bi when they enter).
        float2 w[4][4];
#pragma unroll
        for (int q = 0; q < 16; q++) w[q >> 2][q & 3] = cf(0.f, 0.f);
        for (int q = tid; q < WP; q += blockDim.x) {
            bsh[q] = (q < n && fuse) ? to_f(bv[q]) : cf(0.f, 0.f);
#pragma unroll
            for (int r = 0; r < 4; r++) nbuf[0][r][q] = nbuf[1][r][q] = nbuf[2][r][q] = cf(0.f, 0.f);
        }
        if (tid < 12) bnew[tid / 4][tid % 4] = cf(0.f, 0.f);
        if (tid == 0) bad = 0;
        for (int Jw = 0; Jw < NB; Jw++) {
            __syncthreads();
            if (ln >= 0) {
                const int r = ln >> 3, e0 = ln & 7, rr = 4 * Jw + r;
                if (rr < n)
                    for (int e = e0; e < rw; e += 8) {
                        int c = P.col[(size_t)rr * rw + e];
                        if (c >= 0) nbuf[0][r][c] = to_f(as[(size_t)rr * rw + e]);
                    }
            }
            __syncthreads();
            if (has && (bi == Jw || bj == Jw)) refill_tile(w, nbuf[0], bi == Jw, bj == Jw, sa0, sb0);
            __syncthreads();
            if (tid < WP) {
#pragma unroll
                for (int r = 0; r < 4; r++) nbuf[0][r][tid] = cf(0.f, 0.f);
            }
        }
        __syncthreads();
        if (has && bi == 0 && bj == 0) factor_diag4(w, 0, n, Ldsh, dinvsh, &bad, P.ldc);
        if (ln >= 0) {
            // rows WP..WP+3 enter at block step 0: staged directly
            const int r = ln >> 3, e0 = ln & 7, rr = WP + r;
            if (rr < n) {
                for (int e = e0; e < rw; e += 8) {
                    int c = P.col[(size_t)rr * rw + e];
                    if (c >= 0) nbuf[0][r][c % WP] = to_f(as[(size_t)rr * rw + e]);
                }
                if (e0 == 7 && fuse) bnew[0][r] = to_f(bv[rr]);
            }
            // block steps 1..D ahead of time
            for (int q = 0; q < D; q++) {
                const int sl = (q + 1) % D;
                stage_issue4(P, as, bv, WP + 4 * (q + 1), ln, rw, fuse, ring_val[sl], ring_col[sl], ring_b[sl]);
            }
        }
        int Bk = 0;  // pivot slot block of the current step
        for (int J = 0; J < nblk; J++) {
            const int j = 4 * J, cur = J % 3;
            // ---- 1. gather the pivot columns
            if (has && (bi == Bk) != (bj == Bk)) {
                if (bi == Bk) {
#pragma unroll
                    for (int a = 0; a < 4; a++) {
                        float4 *d = (float4 *)&panel[a][sb0];
                        d[0] = make_float4(w[a][0].x, w[a][0].y, w[a][1].x, w[a][1].y);
                        d[1] = make_float4(w[a][2].x, w[a][2].y, w[a][3].x, w[a][3].y);
                    }
                } else {
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        float4 *d = (float4 *)&panel[b][sa0];
                        d[0] = make_float4(w[0][b].x, w[0][b].y, w[1][b].x, w[1][b].y);
                        d[1] = make_float4(w[2][b].x, w[2][b].y, w[3][b].x, w[3][b].y);
                    }
                }
            }
            __syncthreads();
            // ---- 2. panel: L entries of every window row for columns j..j+3
            if (tid < WP) {
                const int sl = tid;
                const int blk = sl >> 2, b4 = sl & 3;
                int dist = sl - 4 * Bk;
                if (dist < 0) dist += WP;
                const int r_s = j + dist;
                float2 a[4];
                int band0;  // first pivot column (0..4) inside the band of this row
                if (blk == Bk) {
                    // pivot row j+b4: its row of the diagonal block factor
                    if (j + b4 < n) {
                        float2 *row = L + (size_t)(j + b4) * Wb + (mb - b4);  // column j
                        for (int q = 0; q <= b4; q++)
                            if (mb - b4 + q >= 0) row[q] = Ldsh[b4][q];
                    }
                    // the row entering this slot: its entries in the pivot columns
                    band0 = WP + b4 - mb;  // >= b4 + 1
#pragma unroll
                    for (int q = 0; q < 4; q++) a[q] = (q >= band0) ? nbuf[cur][b4][4 * Bk + q] : cf(0.f, 0.f);
                } else {
                    band0 = dist - mb;
#pragma unroll
                    for (int q = 0; q < 4; q++) a[q] = panel[q][sl];
                }
                const int r_l = (blk == Bk) ? j + WP + b4 : r_s;  // row whose L entries these are
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 l = cmulf(a[q], dinvsh[q]);
#pragma unroll
                    for (int r = q + 1; r < 4; r++) a[r] = cfmsf(a[r], l, Ldsh[r][q]);
                    a[q] = l;
                    lp[q][b4 >> 1][blk][b4 & 1] = l;
                }
                if (r_l < n && band0 < 4) {
                    float2 *row = L + (size_t)r_l * Wb + (j - r_l + mb);  // column j
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (q >= band0) row[q] = a[q];
                }
            }
            if (ln == 0 && fuse) {
                // forward substitution of the 4 pivot entries (staging warp)
                float2 bb[4];
#pragma unroll
                for (int q = 0; q < 4; q++) bb[q] = bsh[4 * Bk + q];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 yq = cmulf(bb[q], dinvsh[q]);
                    ysh[q] = yq;
                    if (j + q < n) yv[j + q] = yq;
#pragma unroll
                    for (int r = q + 1; r < 4; r++) bb[r] = cfmsf(bb[r], Ldsh[r][q], yq);
                }
            }
            __syncthreads();
            // ---- 3. rank-4 update, or refill with the entering rows
            if (has) {
                if (bi == Bk || bj == Bk) refill_tile(w, nbuf[cur], bi == Bk, bj == Bk, sa0, sb0);
                // one column at a time: keeps 16 registers of L values live
#pragma unroll 1
                for (int q = 0; q < 4; q++) {
                    float2 la[4], lb[4];
                    {
                        const float4 a01 = *(const float4 *)&lp[q][0][bi][0];
                        const float4 a23 = *(const float4 *)&lp[q][1][bi][0];
                        const float4 b01 = *(const float4 *)&lp[q][0][bj][0];
                        const float4 b23 = *(const float4 *)&lp[q][1][bj][0];
                        la[0] = cf(a01.x, a01.y); la[1] = cf(a01.z, a01.w);
                        la[2] = cf(a23.x, a23.y); la[3] = cf(a23.z, a23.w);
                        lb[0] = cf(b01.x, b01.y); lb[1] = cf(b01.z, b01.w);
                        lb[2] = cf(b23.x, b23.y); lb[3] = cf(b23.z, b23.w);
                    }
#pragma unroll
                    for (int a = 0; a < 4; a++)
#pragma unroll
                        for (int b = 0; b < 4; b++) w[a][b] = cfmsf(w[a][b], la[a], lb[b]);
                }
                // the next pivot block: factor it now, off the critical path
                const int Bn = (Bk + 1 == NB) ? 0 : Bk + 1;
                if (bi == Bn && bj == Bn) factor_diag4(w, j + 4, n, Ldsh, dinvsh, &bad, P.ldc);
            }
            if (ln >= 0) {
                // staging warp: right-hand side update, clearing of the buffer
                // after next, entering rows of the next step
                if (fuse)
                    for (int t = ln; t < WP; t += 32) {
                        const int blk = t >> 2, b4 = t & 3;
                        float2 v = (blk == Bk) ? bnew[cur][b4] : bsh[t];
#pragma unroll
                        for (int q = 0; q < 4; q++) v = cfmsf(v, lp[q][b4 >> 1][blk][b4 & 1], ysh[q]);
                        bsh[t] = v;
                    }
                for (int t = ln; t < WP; t += 32) {
#pragma unroll
                    for (int r = 0; r < 4; r++) nbuf[(J + 2) % 3][r][t] = cf(0.f, 0.f);
                }
                __syncwarp();
                // rows of block step J+1 (issued D steps ago) -> nbuf[(J+1)%3];
                // then issue the rows of block step J+1+D
                const int sl = (J + 1) % D, r = ln >> 3, e0 = ln & 7;
                const int rr = j + 4 + WP + r;
                cp_wait<D - 1>();
                if (rr < n) {
                    for (int e = e0; e < rw; e += 8) {
                        int c = ring_col[sl][r][e];
                        if (c >= 0) nbuf[(J + 1) % 3][r][c % WP] = to_f(ring_val[sl][r][e]);
                    }
                    if (e0 == 7 && fuse) bnew[(J + 1) % 3][r] = to_f(ring_b[sl][r]);
                } else if (e0 == 7) {
                    bnew[(J + 1) % 3][r] = cf(0.f, 0.f);
                }
                stage_issue4(P, as, bv, rr - r + 4 * D, ln, rw, fuse, ring_val[sl], ring_col[sl], ring_b[sl]);
            }
            Bk = (Bk + 1 == NB) ? 0 : Bk + 1;
        }
        if (ln >= 0) cp_wait<0>();
        __syncthreads();
        if (tid == 0 && bad) atomicCAS(&B.status[s], 0, bad);
    }
}

#define CRGPU_MIXED_SIZES(X) X(36) X(64) X(84) X(104) X(124) X(128) X(144) X(160) X(176)

// smallest instantiated window holding W = mb + 1 rows (registers, then shared memory)
int mixed_window_supported(int W) {
#define X(S) if (W <= S) return S;
    CRGPU_MIXED_SIZES(X)
#undef X
    return mixed_smem_window_supported(W);
}

// Kernel by P.tune_factor (0: one warp per system when mb <= 63, else tensor
// cores when the band fits their window, else the smallest SIMT window),
// blocks per SM of the SIMT tile kernels by P.tune_ctas (0: one).
int mixed_factor_kind(const DevProblem &P) {
    const int W = P.mb + 1;
    int kind = P.tune_factor;
    if (kind == 4 && (W > 64 || P.rw > 32)) kind = 0;
    if (kind == 1 && P.mb + 4 > 128) kind = 0;
    if (kind == 2 && mixed_window_supported(W) > 176) kind = 0;
    if (kind == 0) kind = (W <= 64 && P.rw <= 32) ? 4 : P.mb + 4 <= 128 ? 1 : (mixed_window_supported(W) <= 176 ? 2 : 3);
    return kind;
}

int launch_factor_mixed(const DevProblem &P, const DevBatch &B, int fuse, int nsm, bool exclusive,
                        cudaStream_t st) {
    const int W = P.mb + 1;
    const int kind = mixed_factor_kind(P);
    if (kind == 4) return launch_factor_warp(P, B, fuse, nsm, st) ? 0 : ERR_UNSUPPORTED;
    if (kind == 1) return launch_factor_tc(P, B, fuse, nsm, st, exclusive);
    const int per_sm = P.tune_ctas > 0 ? P.tune_ctas : 1;
    if (kind == 3) return launch_factor_mixed_smem(P, B, fuse, nsm * per_sm, st);
    int grid = B.nsys < nsm * per_sm ? B.nsys : nsm * per_sm;
#define X(S)                                                                   \
    if (W <= S) {                                                              \
        k_factor_mixed<S><<<grid, MixCfg<S>::NT, 0, st>>>(P, B, fuse);         \
        return 0;                                                              \
    }
    CRGPU_MIXED_SIZES(X)
#undef X
    return launch_factor_mixed_smem(P, B, fuse, nsm, st);
}

}  // namespace crgpu
