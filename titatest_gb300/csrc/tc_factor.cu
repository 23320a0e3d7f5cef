// Complex64 band factorisation on the 5th-generation tensor cores
// (src/chol.f90:7-88, with the forward substitution of src/vre.f90:45-56
// fused in), for band widths mb <= 124.
//
// The active window (rows j .. j+127 of the band, row r in slot r mod 128)
// lives in tensor memory as FP32: TMEM lane s = slot s, columns 2c / 2c+1 =
// real / imaginary part of the entry with the row of slot c.  One step
// eliminates the 4 pivot columns j..j+3 (pivot slot block Bk = J mod 32):
//
//   1. every thread (= slot) holds its row's 4 entries A(r, j..j+3) in the
//      pivot columns (read ahead, see below);
//   2. SIMT panel: L D L^T of the 4x4 diagonal block (in every thread),
//      m_r = A(r, j..j+3) Lu^{-T} and l_r = m_r D^{-1} of the slot's row;
//   3. one elected thread issues, into the TMEM window,
//        D += A . B^T  (M=128, N=256, K=8, kind::tf32)
//      with A row r = [Re m_r | Im m_r] and B rows 2c, 2c+1 =
//      [-Re l_c | Im l_c], [-Im l_c | -Re l_c]: D -= m l^T in complex
//      arithmetic (the Schur complement A - a P^{-1} a^T of the pivot block
//      P).  Three products (hi.hi + hi.lo + lo.hi of the tf32 splits) keep
//      FP32 accuracy; pivot rows contribute zero.
//   4. the 4 rows entering at this step take over the pivot slots.  Their
//      row part D(p, :) is set by a fourth MMA whose A is one-hot on the
//      pivot lanes and whose B holds new value - old value (hi + lo); the
//      old value of D(p, c) is, by symmetry, the pivot column entry that
//      thread c holds in step 1.  Their column part D(:, p) is written by
//      tcgen05.st once the MMAs of the step have completed.
// Entering rows never reach back into eliminated columns because the window
// has 128 >= mb + 4 rows, so they need no update of earlier steps.
//
// One-step look-ahead: before handing step J over, the panel reads the
// next pivot columns from TMEM as they stand after the MMAs of step J-1 and
// applies step J's rank-4 update to them itself (4x4 complex products per
// row), so the MMAs of step J have a whole panel step to complete.
//
// Roles: warps 0-3 (128 threads, thread t <-> TMEM lane t) run the panel;
// warp 4 stages the entering rows from the scaled sparse values (cp.async
// ring, three steps ahead of their use); warp 5 issues the MMAs when the
// panel hands over a step's operands, then, while they run, does the pivot
// block's share of the factor (its rows of L, the fused forward substitution
// and 1/sqrt(d), u = D^{-1} Lu^{-1} b for the panel, which stores its rows of L
// and updates its right-hand side one step later).  All six warps meet at
// one named barrier per step.  Every mbarrier wait is bounded in time and
// failures are agreed on by a barrier reduction, so all roles leave
// together.
#include <mutex>

#include "bulk.cuh"
#include "crgpu_internal.h"
#include "device.cuh"
#include "kernels.h"
#include "mixed_common.cuh"
#include "tc_common.cuh"

namespace crgpu {

using namespace tc;

namespace {

constexpr int kTcWP = 128;     // window slots = TMEM lanes = MMA M
constexpr int kTcCols = 256;   // TMEM columns = MMA N
constexpr int kTcNB = kTcWP / 4;
constexpr int kTcThreads = 192;
constexpr int kTcNNB = 4;      // buffers of entering rows
constexpr int kTcSmemRequest = 110 * 1024;  // at most two blocks (2 x 256 TMEM columns) per SM

struct TcOperands {
    // K-major canonical layout without swizzle: 8-row x 16-byte core
    // matrices, K-adjacent cores 128 B apart, row groups 256 B apart.
    float a_hi[kTcWP * 8], a_lo[kTcWP * 8], a_e[kTcWP * 8];
    float b_hi[kTcCols * 8], b_lo[kTcCols * 8], b_e[kTcCols * 8];
};

struct TcSmem {
    TcOperands op[2];               // double buffered by step parity
    float2 nbuf[kTcNNB][4][kTcWP];  // entering rows by slot of column
    float2 bnew[kTcNNB][4];         // their right-hand sides
    double2 ring_val[kStageSteps][4][32];
    double2 ring_b[kStageSteps][4];
    int ring_col[kStageSteps][4][32];
    float2 dm[2][4][4];  // diagonal block of the step
    float2 bp[2][4];     // right-hand side of the pivot rows
    float2 lnx[2][4][4];  // l of the next step's pivot rows [row][k]
    float2 mp[2][4][4];   // m of the last step of the pivot rows [row][k]
    float2 isq_s[2][4];   // 1/sqrt(d) of the step's pivots
    float2 u_s[2][4];     // u = D^{-1} Lu^{-1} b of the step's pivot rows
    uint64_t bar_m;  // the MMAs of a step completed
    uint32_t tmem_base;
    int bad;
    int abort_flag;
    int panel_fail;
    int stop_issue;
};

// barrier of the 128 panel threads that also returns the OR of `fail`
__device__ __forceinline__ bool panel_bar_or(bool fail) {
    uint32_t r;
    asm volatile(
        "{\n"
        " .reg .pred pi, po;\n"
        " setp.ne.u32 pi, %1, 0;\n"
        " bar.red.or.pred po, 1, 128, pi;\n"
        " selp.u32 %0, 1, 0, po;\n"
        "}\n"
        : "=r"(r)
        : "r"((uint32_t)fail)
        : "memory");
    return r != 0;
}

// entry between entering rows a and b of pivot block Bk: the scatter stores
// each row's lower pattern, so it sits in the row with the larger index
__device__ __forceinline__ float2 entering_pair(const float2 (*nb)[kTcWP], int Bk, int a, int b) {
    return a >= b ? nb[a][4 * Bk + b] : nb[b][4 * Bk + a];
}



// named barrier 2: the panel threads hand a step's operands to the MMA warp
__device__ __forceinline__ void handoff_arrive() { asm volatile("bar.arrive 2, 192;\n" ::: "memory"); }
__device__ __forceinline__ void handoff_sync() { asm volatile("bar.sync 2, 192;\n" ::: "memory"); }

// L D L^T of the 4x4 pivot block (rows j..j+3, complex symmetric; rows
// beyond n get a unit pivot): unit lower Lu, d and 1/d.  The only
// operations on the step's critical path; the square roots for the stored
// Cholesky factor Lc = Lu D^{1/2} come after the MMAs are issued.
__device__ __forceinline__ void pivot_ldlt(const float2 (&a)[4][4], int j, int n, float2 (&Lu)[4][4],
                                           float2 (&dv)[4], float2 (&dinv)[4], int &bad, int ldc) {
    float2 dm[4][4];
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int q = 0; q < 4; q++) dm[r][q] = a[r][q];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float2 d = dm[q][q];
        if (j + q >= n) {
            d = cf(1.f, 0.f);
        } else {
            const float r2 = d.x * d.x + d.y * d.y;
            if (!(r2 > 0.f) || !isfinite(r2) || (ldc && !(d.x > 0.f))) bad = 28;
        }
        const float2 di = crecip_fast(d);
        dv[q] = d;
        dinv[q] = di;
#pragma unroll
        for (int r = q + 1; r < 4; r++) Lu[r][q] = cmulf(dm[r][q], di);
#pragma unroll
        for (int r = q + 1; r < 4; r++)
#pragma unroll
            for (int c = q + 1; c <= r; c++) dm[r][c] = cfmsf(dm[r][c], Lu[r][q], dm[c][q]);
    }
}

// MMAs of one step over TMEM columns [c0, c0 + N): the rank-4 update as
// three tf32 products and the injection of the entering rows
__device__ __forceinline__ void issue_range(uint32_t tbase, const TcOperands &o, int c0, int N) {
    const uint32_t idesc = tf32_idesc(kTcWP, N);
    const uint32_t d = tbase + (uint32_t)c0;
    const int boff = c0 * 8;  // floats: 8-row groups of 256 B
    const uint64_t ah = smem_desc(o.a_hi), al = smem_desc(o.a_lo), ae = smem_desc(o.a_e);
    const uint64_t bh = smem_desc(o.b_hi + boff), bl = smem_desc(o.b_lo + boff), be = smem_desc(o.b_e + boff);
    tc_mma_tf32(d, ah, bh, idesc);
    tc_mma_tf32(d, ah, bl, idesc);
    tc_mma_tf32(d, al, bh, idesc);
    tc_mma_tf32(d, ae, be, idesc);
}

}  // namespace

// MULTI = false: the systems of one batch (P1, B1).  MULTI = true: a table of
// (problem, system) items over several problems (uneven meshes), whose
// descriptors Ps[p], Bs[p] are in device memory; the table lists the longest
// systems first, so the persistent blocks finish together.
template <bool MULTI>
__global__ __launch_bounds__(kTcThreads, 2) void k_factor_tc(DevProblem P1, DevBatch B1,
                                                             const DevProblem *__restrict__ Ps,
                                                             const DevBatch *__restrict__ Bs,
                                                             const int2 *__restrict__ items, int nitems, int fuse) {
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    TcSmem &S = *reinterpret_cast<TcSmem *>(tc_smem_raw);
    volatile int *abort_flag = &S.abort_flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool is_panel = warp < 4, is_stage = warp == 4, is_mma = warp == 5;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&S.tmem_base)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = S.tmem_base;
    const uint32_t tlane = tbase + ((uint32_t)(32 * (warp & 3)) << 16);  // this warp's lanes

    bool stop = false;
    const int total = MULTI ? nitems : B1.nsys;
    for (int it = blockIdx.x; it < total && !stop; it += gridDim.x) {
        const DevProblem &P = MULTI ? Ps[items[it].x] : P1;
        const DevBatch &B = MULTI ? Bs[items[it].x] : B1;
        const int s = MULTI ? items[it].y : it;
        const int n = P.n, mb = P.mb, Wb = mb + 1, rw = P.rw;
        const int nblk = (n + 3) / 4;
        float2 *L = (float2 *)B.L + (size_t)s * B.lpitch;
        float2 *yv = (float2 *)B.y + (size_t)s * n;
        const double2 *as = B.As + (size_t)s * P.nnz;
        const double2 *bv = B.b + (size_t)s * n;
        __syncthreads();
        if (tid == 0) {
            mbar_init(&S.bar_m, 1);
            mbar_init_fence();
            S.bad = 0;
            S.abort_flag = 0;
            S.panel_fail = 0;
            S.stop_issue = 0;
        }
        for (int q = tid; q < kTcNNB * 4 * kTcWP; q += blockDim.x) (&S.nbuf[0][0][0])[q] = cf(0.f, 0.f);
        for (int q = tid; q < kTcWP * 8; q += blockDim.x) S.op[0].a_e[q] = S.op[1].a_e[q] = 0.f;
        if (tid < 4 * kTcNNB) S.bnew[tid / 4][tid % 4] = cf(0.f, 0.f);
        __syncthreads();
        // ---- initial window (rows 0..127) from the full symmetric pattern;
        //      entering rows of steps 0..kTcNNB-1
        float2 bsh = cf(0.f, 0.f);
        if (is_panel) {
            const int r = tid;
            if (r < n && fuse) bsh = to_f(bv[r]);
            const int f0 = r < n ? P.fptr[r] : 0, f1 = r < n ? P.fptr[r + 1] : 0;
            for (int cb = 0; cb < kTcNB; cb++) {  // 4 slots = 8 columns per store
                float v[8];
#pragma unroll
                for (int q = 0; q < 8; q++) v[q] = 0.f;
                for (int f = f0; f < f1; f++) {
                    const int c = P.fcol[f];
                    if ((c >> 2) != cb) continue;
                    const float2 a = to_f(as[P.fidx[f]]);
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if ((c & 3) == q) {
                            v[2 * q] = a.x;
                            v[2 * q + 1] = a.y;
                        }
                }
                tmem_st8(tlane + 8 * cb, v);
            }
        } else if (is_stage) {
            const int ln = lane;
            for (int m = 0; m < kTcNNB; m++) {
                const int r = ln >> 3, e0 = ln & 7, rr = 4 * m + kTcWP + r;
                if (rr < n) {
                    for (int e = e0; e < rw; e += 8) {
                        const int c = P.col[(size_t)rr * rw + e];
                        if (c >= 0) S.nbuf[m][r][c % kTcWP] = to_f(as[(size_t)rr * rw + e]);
                    }
                    if (e0 == 7 && fuse) S.bnew[m][r] = to_f(bv[rr]);
                }
            }
            for (int q = 0; q < kStageSteps; q++) {
                const int m = kTcNNB + q;
                stage_issue4(P, as, bv, 4 * m + kTcWP, ln, rw, fuse, S.ring_val[m % kStageSteps],
                             S.ring_col[m % kStageSteps], S.ring_b[m % kStageSteps]);
            }
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();

        if (is_panel) {
            // ================= panel warps: one thread per slot =================
            const int t = tid, b4 = t & 3, blk = t >> 2;
            int Bk = 0, Bp = kTcNB - 1;  // pivot block of this step, of the last step
            int issued = 0;              // steps handed to the MMA warp
            int bad = 0;
            bool failed = false;
            // this row's entries in the pivot columns of the coming step, as in
            // TMEM before the last step's update (which the panel applies itself)
            float2 pre[4], mprev[4];
            {
                float v[8];
                tmem_ld8(tlane, v);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    pre[q] = cf(v[2 * q], v[2 * q + 1]);
                    mprev[q] = cf(0.f, 0.f);
                }
            }
            for (int J = 0; J < nblk; J++) {
                const int j = 4 * J, cn = J % kTcNNB, cp = (J + kTcNNB - 1) % kTcNNB, ob = J & 1;
                const int Bn = (Bk + 1 == kTcNB) ? 0 : Bk + 1;
                bool ok = !failed;
                // ---- this row's entries in the pivot columns: the rows that entered at the
                //      last step as staged, the others with the last step's update applied
                float2 a[4], mold[4];
#pragma unroll
                for (int q = 0; q < 4; q++) mold[q] = mprev[q];
                if (J >= 1 && blk == Bp) {
#pragma unroll
                    for (int q = 0; q < 4; q++) a[q] = S.nbuf[cp][b4][4 * Bk + q];
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        float2 x = pre[q];
                        if (J >= 1) {
#pragma unroll
                            for (int p = 0; p < 4; p++) x = cfmsf(x, mprev[p], S.lnx[ob ^ 1][q][p]);
                        }
                        a[q] = x;
                    }
                }
                if (blk == Bk) {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        S.dm[ob][b4][q] = a[q];
                        S.mp[ob][b4][q] = mprev[q];
                    }
                    S.bp[ob][b4] = bsh;
                }
                if (panel_bar_or(!ok)) {  // the same decision in every panel thread
                    if (t == 0) {
                        S.panel_fail = 1;
                        S.stop_issue = 1;
                    }
                    handoff_arrive();  // release the MMA warp, which then stops
                    break;
                }
                // ---- L D L^T of the pivot block (every thread, in registers)
                float2 Lu[4][4], dv[4], dinv[4];
                {
                    float2 d0[4][4];
#pragma unroll
                    for (int r = 0; r < 4; r++)
#pragma unroll
                        for (int q = 0; q < 4; q++) d0[r][q] = S.dm[ob][r][q];
                    pivot_ldlt(d0, j, n, Lu, dv, dinv, bad, P.ldc);
                }
                // ---- m = a Lu^{-T} and l = m D^{-1} of this slot's row (zero for the pivot rows)
                float2 m[4], l[4];
                int dist = t - 4 * Bk;
                if (dist < 0) dist += kTcWP;
                if (blk == Bk) {
#pragma unroll
                    for (int q = 0; q < 4; q++) m[q] = l[q] = cf(0.f, 0.f);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        float2 x = a[q];
#pragma unroll
                        for (int p = 0; p < q; p++) x = cfmsf(x, m[p], Lu[q][p]);
                        m[q] = x;
                        l[q] = cmulf(x, dinv[q]);
                    }
                }
                if (blk == Bn) {  // the next pivot rows' l, for the next step's update of its pivot columns
#pragma unroll
                    for (int q = 0; q < 4; q++) S.lnx[ob][b4][q] = l[q];
                }
                // ---- MMA operands of this step (buffer ob; its last reader, the MMAs of
                //      step J-2, completed before step J-1 ended)
                {
                    TcOperands &o = S.op[ob];
                    float ah[8], al[8], bh0[8], bl0[8], bh1[8], bl1[8], be0[8], be1[8];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const float mr = m[q].x, mi = m[q].y, re = l[q].x, im = l[q].y;
                        const float mrh = tf32_hi(mr), mih = tf32_hi(mi);
                        const float reh = tf32_hi(re), imh = tf32_hi(im);
                        ah[q] = mrh;
                        ah[4 + q] = mih;
                        al[q] = mr - mrh;
                        al[4 + q] = mi - mih;
                        bh0[q] = -reh;
                        bh0[4 + q] = imh;
                        bl0[q] = -(re - reh);
                        bl0[4 + q] = im - imh;
                        bh1[q] = -imh;
                        bh1[4 + q] = -reh;
                        bl1[q] = -(im - imh);
                        bl1[4 + q] = -(re - reh);
                        // new - old value of entering row q at this slot's column; the old
                        // value D(pivot q, t) equals this thread's pivot entry a[q] by symmetry
                        const float2 nv = (blk == Bk) ? entering_pair(S.nbuf[cn], Bk, q, b4) : S.nbuf[cn][q][t];
                        const float dr = nv.x - a[q].x, di = nv.y - a[q].y;
                        const float drh = tf32_hi(dr), dih = tf32_hi(di);
                        be0[q] = drh;
                        be0[4 + q] = dr - drh;
                        be1[q] = dih;
                        be1[4 + q] = di - dih;
                    }
                    put_row8(o.a_hi, t, ah);
                    put_row8(o.a_lo, t, al);
                    put_row8(o.b_hi, 2 * t, bh0);
                    put_row8(o.b_lo, 2 * t, bl0);
                    put_row8(o.b_hi, 2 * t + 1, bh1);
                    put_row8(o.b_lo, 2 * t + 1, bl1);
                    // A of the injection: one-hot rows on the pivot lanes; the rows set
                    // in this buffer two steps ago go back to zero
                    const int B2 = Bk >= 2 ? Bk - 2 : Bk + kTcNB - 2;
                    if (blk == Bk || (J >= 2 && blk == B2)) {
                        float ae[8];
#pragma unroll
                        for (int q = 0; q < 4; q++) ae[q] = ae[4 + q] = (blk == Bk && b4 == q) ? 1.f : 0.f;
                        put_row8(o.a_e, t, ae);
                    }
                    put_row8(o.b_e, 2 * t, be0);
                    put_row8(o.b_e, 2 * t + 1, be1);
                }
                // ---- the last step's MMAs have landed: column part of the rows that
                //      entered then (the MMAs of this step update it), and the next
                //      pivot columns as they stand before this step's update
                if (J >= 1) {
                    ok = __all_sync(0xffffffffu, mbar_wait_abort(&S.bar_m, (J - 1) & 1, abort_flag, 0u));
                    tc_fence_after();
                    if (ok) {
                        float v[8];
#pragma unroll
                        for (int b = 0; b < 4; b++) {
                            // entries among the entering rows sit in the later row's pattern
                            const float2 x = (blk == Bp) ? entering_pair(S.nbuf[cp], Bp, b, b4) : S.nbuf[cp][b][t];
                            v[2 * b] = x.x;
                            v[2 * b + 1] = x.y;
                        }
                        tmem_st8(tlane + 8 * Bp, v);
                    }
                }
                if (ok && J + 1 < nblk) {
                    float v[8];
                    tmem_ld8(tlane + 8 * Bn, v);
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        pre[q] = cf(v[2 * q], v[2 * q + 1]);
                        mprev[q] = m[q];
                    }
                }
                failed = !ok;
                if (!ok && t == 0) S.panel_fail = 1;
                fence_proxy_async();
                tc_fence_before();
                handoff_sync();  // also orders this step's lnx before the next step's reads
                issued = J + 1;
                // ---- while the MMAs run: this row's entries of Lc = Lu D^{1/2} (as
                //      src/chol.f90 stores it) in the last step's pivot columns,
                //      l sqrt(d) = m / sqrt(d), and the last step's update of the fused
                //      forward substitution, b -= l (Lu^{-1} b_p) = m u, from 1/sqrt(d)
                //      and u of the pivot block that the MMA warp left in shared memory
                if (J >= 1 && blk != Bp && fuse) {
#pragma unroll
                    for (int q = 0; q < 4; q++) bsh = cfmsf(bsh, mold[q], S.u_s[ob ^ 1][q]);
                }
                if (blk == Bk) bsh = fuse ? S.bnew[cn][b4] : cf(0.f, 0.f);  // the entering row's right-hand side
                Bp = Bk;
                Bk = Bn;
            }
            // the MMAs issued last must land before the next system or the dealloc
            if (issued > 0) {
                mbar_wait(&S.bar_m, (issued - 1) & 1);
                tc_fence_after();
            }
            if (bad) S.bad = bad;
        } else if (is_stage) {
            // ================= staging warp =================
            // The buffer of step i-1's entering rows is free once step i has been
            // handed over (its last reader is step i's column store): after
            // handoff i it takes the rows of step i+3, which step i+3 reads after
            // handoff i+2.  The per-step handoff barrier orders both sides.
            const int ln = lane;
            for (int i = 0; i < nblk; i++) {
                handoff_sync();
                if (S.stop_issue) break;
                if (i == 0) continue;
                const int m = i + kTcNNB - 1, cn = m % kTcNNB;
                for (int q = ln; q < kTcWP; q += 32) {
#pragma unroll
                    for (int r = 0; r < 4; r++) S.nbuf[cn][r][q] = cf(0.f, 0.f);
                }
                if (ln < 4) S.bnew[cn][ln] = cf(0.f, 0.f);
                __syncwarp();
                const int sl = m % kStageSteps, r = ln >> 3, e0 = ln & 7;
                const int rr = 4 * m + kTcWP + r;
                cp_wait<kStageSteps - 1>();
                __syncwarp();
                if (rr < n) {
                    for (int e = e0; e < rw; e += 8) {
                        const int c = S.ring_col[sl][r][e];
                        if (c >= 0) S.nbuf[cn][r][c % kTcWP] = to_f(S.ring_val[sl][r][e]);
                    }
                    if (e0 == 7 && fuse) S.bnew[cn][r] = to_f(S.ring_b[sl][r]);
                }
                __syncwarp();
                stage_issue4(P, as, bv, 4 * (m + kStageSteps) + kTcWP, ln, rw, fuse, S.ring_val[sl], S.ring_col[sl],
                             S.ring_b[sl]);
            }
            cp_wait<0>();
        } else if (is_mma) {
            // ================= MMA warp =================
            // Issues each step's MMAs; then, while they run, lanes 0-3 do the pivot
            // block's share of the factor: its rows of Lc, the fused forward
            // substitution y = D^{-1/2} Lu^{-1} b and, for the panel's update of the
            // other rows, 1/sqrt(d) and u = D^{-1} Lu^{-1} b.
            float2 up[4];
#pragma unroll
            for (int q = 0; q < 4; q++) up[q] = cf(0.f, 0.f);
            for (int J = 0; J < nblk; J++) {
                handoff_sync();
                if (S.stop_issue) break;
                tc_fence_after();
                const int ob = J & 1;
                if (lane == 0) {
                    issue_range(tbase, S.op[ob], 0, kTcCols);
                    tc_commit(&S.bar_m);
                }
                if (lane < 4) {
                    const int j = 4 * J, q = lane;
                    float2 d0[4][4], Lu[4][4], dv[4], dinv[4];
#pragma unroll
                    for (int r = 0; r < 4; r++)
#pragma unroll
                        for (int c = 0; c < 4; c++) d0[r][c] = S.dm[ob][r][c];
                    int bad_m = 0;  // reported by the panel, which factors the same block
                    pivot_ldlt(d0, j, n, Lu, dv, dinv, bad_m, P.ldc);
                    // right-hand side of the pivot rows with the last step's update, then Lu^{-1}
                    float2 w[4];
#pragma unroll
                    for (int r = 0; r < 4; r++) {
                        float2 x = S.bp[ob][r];
#pragma unroll
                        for (int p = 0; p < 4; p++) x = cfmsf(x, S.mp[ob][r][p], up[p]);
                        w[r] = x;
                    }
#pragma unroll
                    for (int c = 0; c < 4; c++)
#pragma unroll
                        for (int r = c + 1; r < 4; r++) w[r] = cfmsf(w[r], Lu[r][c], w[c]);
                    float2 sq[4];
#pragma unroll
                    for (int p = 0; p < 4; p++) {
                        sq[p] = csqrt_fast(dv[p]);
                        up[p] = cmulf(w[p], dinv[p]);
                    }
                    float2 sqq = sq[0], dinvq = dinv[0], wq = w[0], uq = up[0];
#pragma unroll
                    for (int p = 1; p < 4; p++)
                        if (q == p) {
                            sqq = sq[p];
                            dinvq = dinv[p];
                            wq = w[p];
                            uq = up[p];
                        }
                    const float2 isqq = cmulf(sqq, dinvq);  // 1/sqrt(d) = sqrt(d)/d
                    if (j + q < n) {
                        if (fuse) yv[j + q] = cmulf(wq, isqq);
                        float2 *row = L + (size_t)(j + q) * Wb + (mb - q);  // row j+q of the pivot block
#pragma unroll
                        for (int r = 0; r < 4; r++)
                            if (r == q) {
#pragma unroll
                                for (int p = 0; p <= r; p++)
                                    if (mb - r + p >= 0) row[p] = (p == r) ? sq[p] : cmulf(Lu[r][p], sq[p]);
                            }
                    }
                    S.isq_s[ob][q] = isqq;
                    S.u_s[ob][q] = uq;
                }
                __syncwarp();
                // the step's entries of Lc = m / sqrt(d) for the other rows of the window:
                // m rebuilt exactly from its tf32 hi + lo operand rows, which stay in this
                // buffer until step J+2 writes it (after the next handoff)
                {
                    const int j = 4 * J, Bk = J % kTcNB;
                    float2 isq[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) isq[q] = S.isq_s[ob][q];
                    const TcOperands &o = S.op[ob];
#pragma unroll
                    for (int w = 0; w < 4; w++) {
                        const int t = lane + 32 * w;
                        int dist = t - 4 * Bk;
                        if (dist < 0) dist += kTcWP;
                        const int r_l = j + dist, band0 = dist - mb;
                        if ((t >> 2) == Bk || r_l >= n || band0 >= 4) continue;  // pivot rows: stored above
                        const float4 h0 = *(const float4 *)&o.a_hi[kmaj(t, 0)], h1 = *(const float4 *)&o.a_hi[kmaj(t, 4)];
                        const float4 l0 = *(const float4 *)&o.a_lo[kmaj(t, 0)], l1 = *(const float4 *)&o.a_lo[kmaj(t, 4)];
                        const float2 mq[4] = {cf(h0.x + l0.x, h1.x + l1.x), cf(h0.y + l0.y, h1.y + l1.y),
                                              cf(h0.z + l0.z, h1.z + l1.z), cf(h0.w + l0.w, h1.w + l1.w)};
                        float2 *row = L + (size_t)r_l * Wb + (j - r_l + mb);  // column j
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            if (q >= band0) row[q] = cmulf(mq[q], isq[q]);
                    }
                }
                __syncwarp();
            }
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            if (S.abort_flag || S.panel_fail) atomicCAS(&B.status[s], 0, ERR_TIMEOUT);
            else if (S.bad) atomicCAS(&B.status[s], 0, S.bad);
            mbar_inval(&S.bar_m);
        }
        stop = S.abort_flag || S.panel_fail;
        __syncthreads();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(kTcCols) : "memory");
}

static int tc_smem_optin() {
    static std::once_flag once;
    static int optin = kTcSmemRequest;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (optin < kTcSmemRequest) optin = kTcSmemRequest;
        cudaFuncSetAttribute(k_factor_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        cudaFuncSetAttribute(k_factor_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    });
    return optin;
}

int launch_factor_tc(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st, bool exclusive) {
    if (P.mb + 4 > kTcWP) return ERR_UNSUPPORTED;
    const int optin = tc_smem_optin();
    static_assert(sizeof(TcSmem) <= kTcSmemRequest, "shared memory layout exceeds the request");
    const int per_sm = exclusive ? 1 : 2;
    const int grid = B.nsys < per_sm * nsm ? B.nsys : per_sm * nsm;
    k_factor_tc<false><<<grid, kTcThreads, exclusive ? optin : kTcSmemRequest, st>>>(P, B, nullptr, nullptr, nullptr, 0,
                                                                                      fuse);
    return 0;
}

// the band factors of several problems' batches in one launch: items (problem,
// system) in device memory, every problem's mb + 4 <= 128 (checked by the caller)
void launch_factor_tc_multi(const DevProblem *Ps, const DevBatch *Bs, const int2 *items, int nitems, int fuse, int nsm,
                            cudaStream_t st) {
    tc_smem_optin();
    const int grid = nitems < 2 * nsm ? nitems : 2 * nsm;
    k_factor_tc<true><<<grid, kTcThreads, kTcSmemRequest, st>>>(DevProblem{}, DevBatch{}, Ps, Bs, items, nitems, fuse);
}

}  // namespace crgpu
