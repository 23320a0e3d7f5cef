// Band triangular solves (src/vre.f90:5-71), FP64 iterative refinement of the
// mixed mode, and the unscaling into kpot (src/fem.f90:383-394).
//
// One warp solves one right-hand side, kRB = 8 band rows at a time.  A
// block's rows are contiguous in the band layout (8 * (mb+1) entries), so one
// bulk copy per block brings them into shared memory S blocks ahead;
// the working vector lives in a shared window.  Per block the dependent
// chain is one warp reduction (forward) and an 8-step triangle of shuffles;
// the rest is independent multiply-adds over the lanes' columns.  Launches
// of few sweeps (up to kFewItems) give each right-hand side kSweepWarps
// warps instead (k_fwd_mw, k_bwd_mw), since each sweep is then latency bound.
#include <mutex>

#include "async.cuh"
#include "bulk.cuh"
#include "crgpu_internal.h"
#include "device.cuh"
#include "kernels.h"

namespace crgpu {

template <typename T>
struct Ops;
template <>
struct Ops<double2> {
    __device__ static double2 div(double2 a, double2 b) { return cdiv(a, b); }
    __device__ static double2 fms(double2 s, double2 a, double2 b) { return cfms(s, a, b); }
    __device__ static double2 from(double2 a) { return a; }
    __device__ static double2 shfl(double2 a, int src) {
        return cz(__shfl_sync(0xffffffffu, a.x, src), __shfl_sync(0xffffffffu, a.y, src));
    }
    __device__ static double2 add(double2 a, double2 b) { return cadd(a, b); }
    __device__ static double2 mul(double2 a, double2 b) { return cmul(a, b); }
    __device__ static double2 rcp(double2 a) { return crecip(a); }
    __device__ static double2 shfl_xor(double2 a, int m) {
        return cz(__shfl_xor_sync(0xffffffffu, a.x, m), __shfl_xor_sync(0xffffffffu, a.y, m));
    }
};
template <>
struct Ops<float2> {
    __device__ static float2 div(float2 a, float2 b) { return cdivf(a, b); }
    __device__ static float2 fms(float2 s, float2 a, float2 b) { return cfmsf(s, a, b); }
    __device__ static float2 from(double2 a) { return to_f(a); }
    __device__ static float2 shfl(float2 a, int src) {
        return cf(__shfl_sync(0xffffffffu, a.x, src), __shfl_sync(0xffffffffu, a.y, src));
    }
    __device__ static float2 add(float2 a, float2 b) { return caddf(a, b); }
    __device__ static float2 mul(float2 a, float2 b) { return cmulf(a, b); }
    __device__ static float2 rcp(float2 a) {  // approximate reciprocal: the solves refine in FP64
        const float q = __fdividef(1.0f, a.x * a.x + a.y * a.y);
        return cf(a.x * q, -a.y * q);
    }
    __device__ static float2 shfl_xor(float2 a, int m) {
        return cf(__shfl_xor_sync(0xffffffffu, a.x, m), __shfl_xor_sync(0xffffffffu, a.y, m));
    }
};

constexpr int kRB = 8;  // rows per block of a sweep
// blocks of band rows in flight per warp: 2 when many sweeps share the GPU
// (together they saturate HBM), 8 when few do and each is latency bound
constexpr int kStagesMany = 2, kStagesFew = 8;
constexpr int kFewItems = 256;  // sweeps per launch up to which kStagesFew is used
// warps per right-hand side of the few-sweeps kernels (k_fwd_mw, k_bwd_mw)
constexpr int kSweepWarps = 4;

// Per-warp shared memory (byte offsets): stage barriers, the right-hand side
// of each staged block (forward sweep), the staged band rows, the window of
// the working vector (entry j in slot j & wmask) and the vector entries that
// enter the window with each block (backward sweep); the multi-warp kernels
// add the per-warp row sums (forward) or the block's solution (backward).
struct SolveLayout {
    int bars, rhs, rows, win, ent, part, total;
};
template <typename T, int S>
__host__ __device__ inline SolveLayout solve_layout(int W, int WW) {
    SolveLayout s;
    s.bars = 0;  // S <= 8 barriers
    s.rhs = 64;
    s.rows = s.rhs + S * kRB * (int)sizeof(double2);
    s.win = s.rows + S * kRB * W * (int)sizeof(T);
    s.ent = s.win + WW * (int)sizeof(T);
    s.part = s.ent + S * kRB * (int)sizeof(T);
    s.total = (s.part + kSweepWarps * kRB * (int)sizeof(T) + 127) & ~127;
    return s;
}

// window size: a power of two holding mb + kRB consecutive entries
static int solve_window(int mb) {
    int w = 16;
    while (w < mb + kRB) w <<= 1;
    return w;
}

// Reduce eight per-lane partial sums a[0..7] (one per block row) over the
// warp; lane l returns the total of row l >> 2.  Halving exchanges: nine
// complex shuffles instead of eight full butterflies.
template <typename T>
__device__ __forceinline__ T reduce_rows8(const T (&a)[kRB], int lane) {
    const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
    T b[4], c[2];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const T send = h16 ? a[k] : a[k + 4];
        const T keep = h16 ? a[k + 4] : a[k];
        b[k] = Ops<T>::add(keep, Ops<T>::shfl_xor(send, 16));
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const T send = h8 ? b[k] : b[k + 2];
        const T keep = h8 ? b[k + 2] : b[k];
        c[k] = Ops<T>::add(keep, Ops<T>::shfl_xor(send, 8));
    }
    const T send = h4 ? c[0] : c[1];
    const T keep = h4 ? c[1] : c[0];
    T d = Ops<T>::add(keep, Ops<T>::shfl_xor(send, 4));
    d = Ops<T>::add(d, Ops<T>::shfl_xor(d, 2));
    d = Ops<T>::add(d, Ops<T>::shfl_xor(d, 1));
    return d;
}

template <int S>
__device__ __forceinline__ void solve_timeout(const DevProblem &P, uint64_t *bar, int next_use, int last_use) {
    // report, then let the copies still in flight land before the block exits
    if ((threadIdx.x & 31) == 0) atomicCAS(P.err, 0, ERR_TIMEOUT);
    for (int u = next_use; u <= last_use; u++) mbar_wait(&bar[u % S], (u / S) & 1);
    cp_wait<0>();
}

// Forward substitution y = L^{-1} rin, one warp per right-hand side, in
// blocks of kRB rows.  For block rows i0..i0+7:
//   (1) t_r = rin_r - sum_{j < i0} L(r, j) y_j   lanes own columns, 8 sums
//   (2) warp reduction of the 8 sums
//   (3) the 8x8 triangle, y_q broadcast from the lanes of row q
// The block's band rows (contiguous, 8 W entries) and right-hand side arrive
// by bulk copy S blocks ahead.
template <typename T, int S>
__global__ __launch_bounds__(32) void k_fwd(DevProblem P, DevBatch B, int nrhs, const double2 *__restrict__ rin,
                                             int wmask) {
    extern __shared__ __align__(128) unsigned char sm_raw[];
    const int n = P.n, mb = P.mb, W = mb + 1, lane = threadIdx.x;
    const int item = blockIdx.x;
    if (item >= B.nsys * nrhs) return;
    if (B.nprev && *B.nprev == 0) return;
    if (B.active && !B.active[item]) return;
    const SolveLayout lay = solve_layout<T, S>(W, wmask + 1);
    uint64_t *bar = (uint64_t *)(sm_raw + lay.bars);
    double2 *rv = (double2 *)(sm_raw + lay.rhs);
    T *rows = (T *)(sm_raw + lay.rows);
    T *win = (T *)(sm_raw + lay.win);
    const T *L = (const T *)B.L + (size_t)(item / nrhs) * B.lpitch;
    const double2 *r = rin + (size_t)item * n;
    T *y = (T *)B.y + (size_t)item * n;
    const int nblk = (n + kRB - 1) / kRB;
    auto issue = [&](int t) {
        if (t >= nblk) return;
        const int st = t % S, i0 = t * kRB, nr = min(kRB, n - i0);
        const uint32_t bl = ((uint32_t)(nr * W * (int)sizeof(T)) + 15u) & ~15u;
        const uint32_t br = (uint32_t)nr * (uint32_t)sizeof(double2);
        mbar_expect_tx(&bar[st], bl + br);
        bulk_g2s(rows + (size_t)st * kRB * W, L + (size_t)i0 * W, bl, &bar[st]);
        bulk_g2s(rv + st * kRB, r + i0, br, &bar[st]);
    };
    if (lane == 0) {
        for (int q = 0; q < S; q++) mbar_init(&bar[q], 1);
        mbar_init_fence();
        for (int t = 0; t < S; t++) issue(t);
    }
    __syncwarp();
    const int myr = lane >> 2;
    for (int t = 0; t < nblk; t++) {
        const int st = t % S, i0 = t * kRB, nr = min(kRB, n - i0);
        const bool ok = mbar_wait(&bar[st], (t / S) & 1);
        if (!__all_sync(0xffffffffu, ok)) {
            solve_timeout<S>(P, bar, t, min(nblk - 1, t + S - 1));
            return;
        }
        const T *Lb = rows + (size_t)st * kRB * W;
        T acc[kRB];
#pragma unroll
        for (int q = 0; q < kRB; q++) acc[q] = T{};
        for (int c = lane; c < mb; c += 32) {
            const int j = i0 - mb + c;
            if (j < 0) continue;
            const T yv = win[j & wmask];
#pragma unroll
            for (int q = 0; q < kRB; q++)
                if (c >= q) acc[q] = Ops<T>::fms(acc[q], Lb[q * W + c - q], yv);
        }
        T tv = Ops<T>::add(Ops<T>::from(rv[st * kRB + myr]), reduce_rows8<T>(acc, lane));
        const T rinv = Ops<T>::rcp(Lb[myr * W + mb]);
        T lt[kRB];
#pragma unroll
        for (int q = 0; q < kRB; q++) {
            const int off = mb - myr + q;  // column i0 + q of row i0 + myr
            lt[q] = (q < myr && off >= 0) ? Lb[myr * W + off] : T{};
        }
#pragma unroll
        for (int q = 0; q < kRB - 1; q++) {
            const T yq = Ops<T>::shfl(Ops<T>::mul(tv, rinv), 4 * q);
            if (q < myr) tv = Ops<T>::fms(tv, lt[q], yq);
        }
        const T ymine = Ops<T>::mul(tv, rinv);
        if ((lane & 3) == 0 && myr < nr) {
            win[(i0 + myr) & wmask] = ymine;
            y[i0 + myr] = ymine;
        }
        __syncwarp();
        if (lane == 0) {
            fence_proxy_async();
            issue(t + S);
        }
    }
}

// Backward substitution L^T x = y in place (y -> x), the column sweep of
// src/vre.f90:58-69 in blocks of kRB rows from the bottom:
//   (1) the 8x8 triangle: x_q = w_q / L(q,q), w_r -= L(q,r) x_q (r < q)
//   (2) w_j -= sum_r L(r, j) x_r for the columns j < i0, lanes own columns
// w lives in the shared window; entries enter it (w_j = y_j) when the first
// block that touches column j is processed.
template <typename T, int S>
__global__ __launch_bounds__(32) void k_bwd(DevProblem P, DevBatch B, int nrhs, int wmask) {
    extern __shared__ __align__(128) unsigned char sm_raw[];
    const int n = P.n, mb = P.mb, W = mb + 1, lane = threadIdx.x;
    const int item = blockIdx.x;
    if (item >= B.nsys * nrhs) return;
    if (B.nprev && *B.nprev == 0) return;
    if (B.active && !B.active[item]) return;
    const SolveLayout lay = solve_layout<T, S>(W, wmask + 1);
    uint64_t *bar = (uint64_t *)(sm_raw + lay.bars);
    T *rows = (T *)(sm_raw + lay.rows);
    T *win = (T *)(sm_raw + lay.win);
    T *ent = (T *)(sm_raw + lay.ent);
    const T *L = (const T *)B.L + (size_t)(item / nrhs) * B.lpitch;
    T *y = (T *)B.y + (size_t)item * n;
    const int nblk = (n + kRB - 1) / kRB;
    // use u = 0, 1, ... processes block t = nblk - 1 - u
    auto issue = [&](int u) {
        const int t = nblk - 1 - u;
        if (t >= 0) {
            const int st = u % S, i0 = t * kRB;
            if (lane == 0) {
                const int nr = min(kRB, n - i0);
                const uint32_t bl = ((uint32_t)(nr * W * (int)sizeof(T)) + 15u) & ~15u;
                mbar_expect_tx(&bar[st], bl);
                bulk_g2s(rows + (size_t)st * kRB * W, L + (size_t)i0 * W, bl, &bar[st]);
            }
            const int j = i0 - mb + lane;  // entering column (not for the last block)
            if (u > 0 && lane < kRB && j >= 0) cp_async_elem<T>(ent + st * kRB + lane, y + j);
        }
        cp_commit();
    };
    const int i0l = (nblk - 1) * kRB;
    for (int j = max(0, i0l - mb) + lane; j < n; j += 32) win[j & wmask] = y[j];
    if (lane == 0) {
        for (int q = 0; q < S; q++) mbar_init(&bar[q], 1);
        mbar_init_fence();
    }
    __syncwarp();
    for (int u = 0; u < S; u++) issue(u);
    const int myr = lane >> 2;
    for (int u = 0; u < nblk; u++) {
        const int t = nblk - 1 - u, st = u % S, i0 = t * kRB, nr = min(kRB, n - i0);
        const bool ok = mbar_wait(&bar[st], (u / S) & 1);
        cp_wait<S - 1>();
        if (!__all_sync(0xffffffffu, ok)) {
            solve_timeout<S>(P, bar, u, min(nblk - 1, u + S - 1));
            return;
        }
        {
            const int j = i0 - mb + lane;
            if (u > 0 && lane < kRB && j >= 0) win[j & wmask] = ent[st * kRB + lane];
        }
        __syncwarp();
        const T *Lb = rows + (size_t)st * kRB * W;
        T wv = win[(i0 + myr) & wmask];
        const T rinv = Ops<T>::rcp(Lb[myr * W + mb]);
        T lt[kRB];
#pragma unroll
        for (int q = 0; q < kRB; q++) {
            const int off = mb - q + myr;  // column i0 + myr of row i0 + q
            lt[q] = (myr < q && q < nr && off >= 0) ? Lb[q * W + off] : T{};
        }
        T xq[kRB];
#pragma unroll
        for (int q = kRB - 1; q >= 0; q--) {
            xq[q] = Ops<T>::shfl(Ops<T>::mul(wv, rinv), 4 * q);
            if (myr < q && q < nr) wv = Ops<T>::fms(wv, lt[q], xq[q]);
        }
        if ((lane & 3) == 0 && myr < nr) y[i0 + myr] = Ops<T>::mul(wv, rinv);
        for (int c = lane; c < mb; c += 32) {
            const int j = i0 - mb + c;
            if (j < 0) continue;
            T w2 = win[j & wmask];
#pragma unroll
            for (int q = 0; q < kRB; q++)
                if (q < nr && c >= q) w2 = Ops<T>::fms(w2, Lb[q * W + c - q], xq[q]);
            win[j & wmask] = w2;
        }
        __syncwarp();
        if (lane == 0) fence_proxy_async();
        issue(u + S);
    }
    cp_wait<0>();
}

// Few sweeps per launch (the last, partial round of a batch; small problems):
// a sweep is a chain of n / 8 dependent blocks, and one warp alone spends
// most of each block on its own issue and shuffle latency.  Here
// kSweepWarps warps share one right-hand side: the columns are split over
// all threads, warp 0 adds the per-warp row sums in warp order and solves
// the 8x8 triangle, and two block barriers separate the phases of a block.
// The staging (thread 0's bulk copies, warp 0's entering elements) is that
// of k_fwd / k_bwd.
template <typename T, int S>
__global__ __launch_bounds__(32 * kSweepWarps) void k_fwd_mw(DevProblem P, DevBatch B, int nrhs,
                                                             const double2 *__restrict__ rin, int wmask) {
    extern __shared__ __align__(128) unsigned char sm_raw[];
    constexpr int NT = 32 * kSweepWarps;
    const int n = P.n, mb = P.mb, W = mb + 1, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int item = blockIdx.x;
    if (item >= B.nsys * nrhs) return;
    if (B.nprev && *B.nprev == 0) return;
    if (B.active && !B.active[item]) return;
    const SolveLayout lay = solve_layout<T, S>(W, wmask + 1);
    uint64_t *bar = (uint64_t *)(sm_raw + lay.bars);
    double2 *rv = (double2 *)(sm_raw + lay.rhs);
    T *rows = (T *)(sm_raw + lay.rows);
    T *win = (T *)(sm_raw + lay.win);
    T *part = (T *)(sm_raw + lay.part);  // [kSweepWarps][kRB]
    const T *L = (const T *)B.L + (size_t)(item / nrhs) * B.lpitch;
    const double2 *r = rin + (size_t)item * n;
    T *y = (T *)B.y + (size_t)item * n;
    const int nblk = (n + kRB - 1) / kRB;
    auto issue = [&](int t) {  // thread 0
        if (t >= nblk) return;
        const int st = t % S, i0 = t * kRB, nr = min(kRB, n - i0);
        const uint32_t bl = ((uint32_t)(nr * W * (int)sizeof(T)) + 15u) & ~15u;
        const uint32_t br = (uint32_t)nr * (uint32_t)sizeof(double2);
        mbar_expect_tx(&bar[st], bl + br);
        bulk_g2s(rows + (size_t)st * kRB * W, L + (size_t)i0 * W, bl, &bar[st]);
        bulk_g2s(rv + st * kRB, r + i0, br, &bar[st]);
    };
    if (tid == 0) {
        for (int q = 0; q < S; q++) mbar_init(&bar[q], 1);
        mbar_init_fence();
        for (int t = 0; t < S; t++) issue(t);
    }
    __syncthreads();
    const int myr = lane >> 2;
    for (int t = 0; t < nblk; t++) {
        const int st = t % S, i0 = t * kRB, nr = min(kRB, n - i0);
        const bool ok = mbar_wait(&bar[st], (t / S) & 1);
        if (!__syncthreads_and(ok)) {
            if (wid == 0) solve_timeout<S>(P, bar, t, min(nblk - 1, t + S - 1));
            return;
        }
        const T *Lb = rows + (size_t)st * kRB * W;
        T acc[kRB];
#pragma unroll
        for (int q = 0; q < kRB; q++) acc[q] = T{};
        for (int c = tid; c < mb; c += NT) {
            const int j = i0 - mb + c;
            if (j < 0) continue;
            const T yv = win[j & wmask];
#pragma unroll
            for (int q = 0; q < kRB; q++)
                if (c >= q) acc[q] = Ops<T>::fms(acc[q], Lb[q * W + c - q], yv);
        }
        const T red = reduce_rows8<T>(acc, lane);
        if ((lane & 3) == 0) part[wid * kRB + myr] = red;
        __syncthreads();
        if (wid == 0) {
            T tv = Ops<T>::from(rv[st * kRB + myr]);
#pragma unroll
            for (int w = 0; w < kSweepWarps; w++) tv = Ops<T>::add(tv, part[w * kRB + myr]);
            const T rinv = Ops<T>::rcp(Lb[myr * W + mb]);
            T lt[kRB];
#pragma unroll
            for (int q = 0; q < kRB; q++) {
                const int off = mb - myr + q;  // column i0 + q of row i0 + myr
                lt[q] = (q < myr && off >= 0) ? Lb[myr * W + off] : T{};
            }
#pragma unroll
            for (int q = 0; q < kRB - 1; q++) {
                const T yq = Ops<T>::shfl(Ops<T>::mul(tv, rinv), 4 * q);
                if (q < myr) tv = Ops<T>::fms(tv, lt[q], yq);
            }
            const T ymine = Ops<T>::mul(tv, rinv);
            if ((lane & 3) == 0 && myr < nr) {
                win[(i0 + myr) & wmask] = ymine;
                y[i0 + myr] = ymine;
            }
        }
        __syncthreads();
        if (tid == 0) {
            fence_proxy_async();
            issue(t + S);
        }
    }
}

template <typename T, int S>
__global__ __launch_bounds__(32 * kSweepWarps) void k_bwd_mw(DevProblem P, DevBatch B, int nrhs, int wmask) {
    extern __shared__ __align__(128) unsigned char sm_raw[];
    constexpr int NT = 32 * kSweepWarps;
    const int n = P.n, mb = P.mb, W = mb + 1, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int item = blockIdx.x;
    if (item >= B.nsys * nrhs) return;
    if (B.nprev && *B.nprev == 0) return;
    if (B.active && !B.active[item]) return;
    const SolveLayout lay = solve_layout<T, S>(W, wmask + 1);
    uint64_t *bar = (uint64_t *)(sm_raw + lay.bars);
    T *rows = (T *)(sm_raw + lay.rows);
    T *win = (T *)(sm_raw + lay.win);
    T *ent = (T *)(sm_raw + lay.ent);
    T *xs = (T *)(sm_raw + lay.part);  // the block's kRB solution entries
    const T *L = (const T *)B.L + (size_t)(item / nrhs) * B.lpitch;
    T *y = (T *)B.y + (size_t)item * n;
    const int nblk = (n + kRB - 1) / kRB;
    // warp 0: use u = 0, 1, ... processes block t = nblk - 1 - u
    auto issue = [&](int u) {
        const int t = nblk - 1 - u;
        if (t >= 0) {
            const int st = u % S, i0 = t * kRB;
            if (lane == 0) {
                const int nr = min(kRB, n - i0);
                const uint32_t bl = ((uint32_t)(nr * W * (int)sizeof(T)) + 15u) & ~15u;
                mbar_expect_tx(&bar[st], bl);
                bulk_g2s(rows + (size_t)st * kRB * W, L + (size_t)i0 * W, bl, &bar[st]);
            }
            const int j = i0 - mb + lane;  // entering column (not for the last block)
            if (u > 0 && lane < kRB && j >= 0) cp_async_elem<T>(ent + st * kRB + lane, y + j);
        }
        cp_commit();
    };
    const int i0l = (nblk - 1) * kRB;
    for (int j = max(0, i0l - mb) + tid; j < n; j += NT) win[j & wmask] = y[j];
    if (tid == 0) {
        for (int q = 0; q < S; q++) mbar_init(&bar[q], 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (wid == 0)
        for (int u = 0; u < S; u++) issue(u);
    const int myr = lane >> 2;
    for (int u = 0; u < nblk; u++) {
        const int t = nblk - 1 - u, st = u % S, i0 = t * kRB, nr = min(kRB, n - i0);
        const bool ok = mbar_wait(&bar[st], (u / S) & 1);
        if (wid == 0) cp_wait<S - 1>();
        if (!__syncthreads_and(ok)) {
            if (wid == 0) solve_timeout<S>(P, bar, u, min(nblk - 1, u + S - 1));
            return;
        }
        const T *Lb = rows + (size_t)st * kRB * W;
        if (wid == 0) {
            {
                const int j = i0 - mb + lane;
                if (u > 0 && lane < kRB && j >= 0) win[j & wmask] = ent[st * kRB + lane];
            }
            __syncwarp();
            T wv = win[(i0 + myr) & wmask];
            const T rinv = Ops<T>::rcp(Lb[myr * W + mb]);
            T lt[kRB];
#pragma unroll
            for (int q = 0; q < kRB; q++) {
                const int off = mb - q + myr;  // column i0 + myr of row i0 + q
                lt[q] = (myr < q && q < nr && off >= 0) ? Lb[q * W + off] : T{};
            }
            T xq[kRB];
#pragma unroll
            for (int q = kRB - 1; q >= 0; q--) {
                xq[q] = Ops<T>::shfl(Ops<T>::mul(wv, rinv), 4 * q);
                if (myr < q && q < nr) wv = Ops<T>::fms(wv, lt[q], xq[q]);
            }
            if ((lane & 3) == 0 && myr < nr) y[i0 + myr] = Ops<T>::mul(wv, rinv);
            if (lane == 0) {
#pragma unroll
                for (int q = 0; q < kRB; q++) xs[q] = xq[q];
            }
        }
        __syncthreads();
        T xb[kRB];
#pragma unroll
        for (int q = 0; q < kRB; q++) xb[q] = xs[q];
        for (int c = tid; c < mb; c += NT) {
            const int j = i0 - mb + c;
            if (j < 0) continue;
            T w2 = win[j & wmask];
#pragma unroll
            for (int q = 0; q < kRB; q++)
                if (q < nr && c >= q) w2 = Ops<T>::fms(w2, Lb[q * W + c - q], xb[q]);
            win[j & wmask] = w2;
        }
        __syncthreads();
        if (tid == 0) fence_proxy_async();
        if (wid == 0) issue(u + S);
    }
    if (wid == 0) cp_wait<0>();
}

// The kernels' dynamic shared memory depends on the band width; contexts of
// different widths may launch concurrently from several host threads, so the
// limit is raised once to the device's opt-in maximum instead of per width.
template <typename T, int S>
static int set_solve_smem(int W, int WW) {
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0, optin = 48 * 1024;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if constexpr (S == kStagesFew) {
            cudaFuncSetAttribute(k_fwd_mw<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(k_bwd_mw<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        } else {
            cudaFuncSetAttribute(k_fwd<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
            cudaFuncSetAttribute(k_bwd<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        }
    });
    return solve_layout<T, S>(W, WW).total;
}

template <typename T, int S>
static void fwd_launch(const DevProblem &P, const DevBatch &B, int nrhs, const double2 *rin, cudaStream_t st) {
    const int nitems = B.nsys * nrhs, W = P.mb + 1, WW = solve_window(P.mb);
    const int bytes = set_solve_smem<T, S>(W, WW);
    if constexpr (S == kStagesFew)
        k_fwd_mw<T, S><<<nitems, 32 * kSweepWarps, bytes, st>>>(P, B, nrhs, rin, WW - 1);
    else
        k_fwd<T, S><<<nitems, 32, bytes, st>>>(P, B, nrhs, rin, WW - 1);
}

template <typename T, int S>
static void bwd_launch(const DevProblem &P, const DevBatch &B, int nrhs, cudaStream_t st) {
    const int nitems = B.nsys * nrhs, W = P.mb + 1, WW = solve_window(P.mb);
    const int bytes = set_solve_smem<T, S>(W, WW);
    if constexpr (S == kStagesFew)
        k_bwd_mw<T, S><<<nitems, 32 * kSweepWarps, bytes, st>>>(P, B, nrhs, WW - 1);
    else
        k_bwd<T, S><<<nitems, 32, bytes, st>>>(P, B, nrhs, WW - 1);
}

// the deep pipeline with several warps per sweep for few sweeps, when its
// staging fits the block's shared memory
template <typename T>
static bool use_few(const DevProblem &P, int nitems) {
    return nitems <= kFewItems && solve_layout<T, kStagesFew>(P.mb + 1, solve_window(P.mb)).total <= 200 * 1024;
}

void launch_forward_solve(const DevProblem &P, const DevBatch &B, int nrhs, bool mixed, const double2 *rin,
                          cudaStream_t st) {
    const bool few = mixed ? use_few<float2>(P, B.nsys * nrhs) : use_few<double2>(P, B.nsys * nrhs);
    if (mixed) few ? fwd_launch<float2, kStagesFew>(P, B, nrhs, rin, st) : fwd_launch<float2, kStagesMany>(P, B, nrhs, rin, st);
    else few ? fwd_launch<double2, kStagesFew>(P, B, nrhs, rin, st) : fwd_launch<double2, kStagesMany>(P, B, nrhs, rin, st);
}

void launch_back_solve(const DevProblem &P, const DevBatch &B, int nrhs, bool mixed, cudaStream_t st) {
    const bool few = mixed ? use_few<float2>(P, B.nsys * nrhs) : use_few<double2>(P, B.nsys * nrhs);
    if (mixed) few ? bwd_launch<float2, kStagesFew>(P, B, nrhs, st) : bwd_launch<float2, kStagesMany>(P, B, nrhs, st);
    else few ? bwd_launch<double2, kStagesFew>(P, B, nrhs, st) : bwd_launch<double2, kStagesMany>(P, B, nrhs, st);
}
// r = b - A x with the full symmetric pattern (FP64)
__global__ void k_residual(DevProblem P, DevBatch B, int nrhs) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t nitems = (size_t)B.nsys * nrhs;
    if (gid >= nitems * P.n) return;
    int item = (int)(gid / P.n), i = (int)(gid % P.n);
    if (B.nprev && *B.nprev == 0) return;
    if (B.active && !B.active[item]) return;
    int s = item / nrhs;
    const double2 *as = B.As + (size_t)s * P.nnz;
    const double2 *x = B.x + (size_t)item * P.n;
    double2 acc = cz(0.0, 0.0);
    for (int q = P.fptr[i]; q < P.fptr[i + 1]; q++) {
        double2 a = as[P.fidx[q]], xv = x[P.fcol[q]];
        acc.x = fma(a.x, xv.x, acc.x);
        acc.x = fma(-a.y, xv.y, acc.x);
        acc.y = fma(a.x, xv.y, acc.y);
        acc.y = fma(a.y, xv.x, acc.y);
    }
    double2 b = B.b[gid];
    B.r[gid] = cz(b.x - acc.x, b.y - acc.y);
}

void launch_residual(const DevProblem &P, const DevBatch &B, int nrhs, cudaStream_t st) {
    size_t tot = (size_t)B.nsys * nrhs * P.n;
    int nt = 256;
    k_residual<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, B, nrhs);
}

// x (+)= z where z is the complex64 correction left in B.y; a system stops
// refining once max|z| <= tol * max|x|.
__global__ void k_accumulate(DevProblem P, DevBatch B, int nrhs, int first, double tol) {
    int item = blockIdx.x;
    if (B.nprev && *B.nprev == 0) return;
    if (B.active && !B.active[item]) return;
    const float2 *z = (const float2 *)B.y + (size_t)item * P.n;
    double2 *x = B.x + (size_t)item * P.n;
    double mz = 0.0, mx = 0.0;
    for (int i = threadIdx.x; i < P.n; i += blockDim.x) {
        double2 zi = to_d(z[i]);
        double2 xi = first ? zi : cz(x[i].x + zi.x, x[i].y + zi.y);
        x[i] = xi;
        mz = fmax(mz, fmax(fabs(zi.x), fabs(zi.y)));
        mx = fmax(mx, fmax(fabs(xi.x), fabs(xi.y)));
    }
    __shared__ double red[2][32];
    for (int o = 16; o > 0; o >>= 1) {
        mz = fmax(mz, __shfl_xor_sync(0xffffffffu, mz, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    if (lane == 0) { red[0][wl] = mz; red[1][wl] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); q++) { mz = fmax(mz, red[0][q]); mx = fmax(mx, red[1][q]); }
        mz = fmax(mz, red[0][0]);
        mx = fmax(mx, red[1][0]);
        if (!first && B.active && !(mz > tol * mx)) B.active[item] = 0;
        if (B.active && B.active[item] && B.nactive) atomicAdd(B.nactive, 1);
        if (B.zmax && mx > 0.0) {
            // relative corrections are non-negative: compare their bit patterns
            unsigned long long rel = (unsigned long long)__double_as_longlong(mz / mx);
            atomicMax((unsigned long long *)B.zmax, rel);
        }
        if (!isfinite(mz) || !isfinite(mx)) {
            atomicCAS(&B.status[item / nrhs], 0, 28);
            if (B.active) B.active[item] = 0;
        }
    }
}

void launch_accumulate(const DevProblem &P, const DevBatch &B, int nrhs, bool first, double tol,
                       cudaStream_t st) {
    int nitems = B.nsys * nrhs;
    k_accumulate<<<nitems, 256, 0, st>>>(P, B, nrhs, first ? 1 : 0, tol);
}

// every item of the batch starts refining
__global__ void k_fill_active(DevBatch B, int nitems) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nitems) B.active[i] = 1;
}

void launch_fill_active(const DevBatch &B, int nrhs, cudaStream_t st) {
    const int nitems = B.nsys * nrhs;
    k_fill_active<<<(nitems + 255) / 256, 256, 0, st>>>(B, nitems);
}

// plain mode: the back sweep left x (complex128) in B.y; copy to B.x
__global__ void k_copy_solution(DevProblem P, DevBatch B, int nrhs) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t tot = (size_t)B.nsys * nrhs * P.n;
    if (gid >= tot) return;
    B.x[gid] = ((const double2 *)B.y)[gid];
}

void launch_copy_solution(const DevProblem &P, const DevBatch &B, int nrhs, cudaStream_t st) {
    size_t tot = (size_t)B.nsys * nrhs * P.n;
    int nt = 256;
    k_copy_solution<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, B, nrhs);
}

// kpot(j, l, k) = pot(j) * fak(j) with pot = -x (src/fem.f90:388-389); for the
// mixed Jacobian also kpot as two complex64 planes hi + lo
__global__ void k_kpot(DevProblem P, DevBatch B, int nrhs, double2 *kpot, float2 *kpot32) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t tot = (size_t)B.nsys * nrhs * P.n;
    if (gid >= tot) return;
    int item = (int)(gid / P.n), i = (int)(gid % P.n);
    int s = item / nrhs, r = item % nrhs;
    int k = B.ks[s], l = (nrhs == 1) ? B.ls[s] : r;
    double f = B.fak[(size_t)s * P.n + i];
    double2 x = B.x[gid];
    double2 v = cz(-x.x * f, -x.y * f);
    if (P.lsr) v = cadd(v, B.pota[(size_t)s * P.n + i]);  // src/fem.f90:390-391
    const size_t at = ((size_t)k * P.eanz + l) * P.n + i;
    kpot[at] = v;
    if (kpot32) {  // complex64 hi plane, then the lo plane (v - hi)
        const float2 hi = to_f(v);
        kpot32[at] = hi;
        kpot32[at + (size_t)P.K * P.eanz * P.n] = cf((float)(v.x - (double)hi.x), (float)(v.y - (double)hi.y));
    }
}

void launch_kpot(const DevProblem &P, const DevBatch &B, int nrhs, double2 *kpot, float2 *kpot32,
                 cudaStream_t st) {
    size_t tot = (size_t)B.nsys * nrhs * P.n;
    int nt = 256;
    k_kpot<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, B, nrhs, kpot, kpot32);
}

}  // namespace crgpu
