// Complex64 band factorisation (src/chol.f90:7-88, with the forward
// substitution of src/vre.f90:45-56 fused in) of narrow bands, mb <= 63, with
// one warp per system and the whole active window in that warp's registers:
// k_factor_warp one column a step (below), k_factor_warp2 two columns a step
// for mb <= 62 (further down).
//
// Window: rows j .. j+63, row r in slot r mod 64, slots in 8 blocks of 8.
// The window is complex symmetric; its strictly lower slot pairs are held
// once, as 8x8 register tiles R[a][c]:
//   * lanes 0-27: the off-diagonal block pairs (I, J), I > J:
//       R[a][c] = A(slot 8I+a, slot 8J+c);
//   * lanes 28-31: two diagonal blocks I, I' = I+1 each (strict triangles):
//       R[a][c] = A(8I+a, 8I+c) for c < a, A(8I'+c, 8I'+a) for c > a
//       (R[a][a] unused);
// and the diagonal A(x, x) in the lane x mod 32 (d0: x = lane, d1: x =
// lane + 32).  With this storage the pairs of pivot slot p = 8P+pp are row pp
// or column pp of the tiles of block P, for every lane, so the unrolled
// column loop touches static registers under per-lane predicates.
//
// Column j (pivot slot p, LDL^T form of the rank-1 update, the same
// right-looking order as the other factor kernels):
//   1. the owners publish the pivot column pcol[x] = A(x, p) (pcol[p] = a_pp);
//   2. every lane: inv = 1/a_pp, its two slots' scaled entries pcs = pcol*inv,
//      the L entries pcol/sqrt(a_pp) of its two slots (stored in the band
//      layout a((mb+1)*sanz)) and the right-hand-side update;
//   3. every lane: R[a][c] -= pcol[x(a)] * pcs[y(c)] over its tile (64
//      complex multiply-adds), d -= pcol*pcs;
//   4. the row j+64 enters slot p: the positions of slot p take its values
//      from a dense row staged two-level ahead (cp.async of the sparse
//      pattern row, then expanded by slot).
// Two __syncwarp per column, no block barrier; a block is one warp.  Two
// register budgets: 168 registers (12 systems an SM resident) for launches of
// more than 8 systems an SM, else ~250 (8 an SM, each column ~1.3x faster).
#include "async.cuh"
#include "crgpu_internal.h"
#include "device.cuh"
#include "kernels.h"
#include "mixed_common.cuh"

namespace crgpu {

namespace {

constexpr int kWW = 64;      // window slots
constexpr int kDense = 4;    // entering rows expanded by slot ahead of use
constexpr int kRaw = 4;      // sparse pattern rows in flight (cp.async)
constexpr int kRawCap = 32;  // padded pattern row width held per raw row
constexpr int kPad = kWW + kWW / 4;  // slot arrays with 16 bytes of padding after every block of 8

// index of slot x in a padded slot array: the 16-byte loads of one block by
// the lanes of the eight blocks fall into disjoint bank groups
__device__ __forceinline__ int pad(int x) { return x + 2 * (x >> 3); }

struct WarpSmem {
    __align__(16) float2 pcol[2][kPad];        // pivot column by padded slot, double buffered by column parity
    __align__(16) float2 pcs[2][kPad];         // pcol * 1/a_pp
    __align__(16) float2 dense[kDense][kPad];  // entering rows by padded slot of their column
    float2 dense_b[kDense];
    __align__(16) double2 raw_val[kRaw][kRawCap];
    int raw_col[kRaw][kRawCap];
    __align__(16) double2 raw_b[kRaw];
};

// row r's lower pattern into dense slot sl (zeros elsewhere), plain loads
template <class SM>
__device__ __forceinline__ void load_dense_row(const DevProblem &P, const double2 *as, const double2 *bv, int r,
                                               int fuse, SM &S, int sl, int lane) {
    S.dense[sl][pad(lane)] = cf(0.f, 0.f);
    S.dense[sl][pad(lane + 32)] = cf(0.f, 0.f);
    __syncwarp();
    if (r < P.n) {
        for (int e = lane; e < P.rw; e += 32) {
            const int c = P.col[(size_t)r * P.rw + e];
            if (c >= 0) S.dense[sl][pad(c & (kWW - 1))] = to_f(as[(size_t)r * P.rw + e]);
        }
    }
    if (lane == 31) S.dense_b[sl] = (r < P.n && fuse) ? to_f(bv[r]) : cf(0.f, 0.f);
    __syncwarp();
}

template <class SM>
__device__ __forceinline__ void raw_issue(const DevProblem &P, const double2 *as, const double2 *bv, int r, int fuse,
                                          SM &S, int lane) {
    const int q = r & (kRaw - 1);
    if (r < P.n) {
        if (lane < P.rw) {
            cp_async16(&S.raw_val[q][lane], as + (size_t)r * P.rw + lane);
            cp_async4(&S.raw_col[q][lane], P.col + (size_t)r * P.rw + lane);
        }
        if (lane == 31 && fuse) cp_async16(&S.raw_b[q], bv + r);
    }
    cp_commit();
}

// Lane tile and its padded slot bases.  xl/xh: base of the rows of the lower /
// upper part (c < a / c > a) of R, yl/yh: of its columns.
struct WarpTile {
    int I, J, diag;
    int xl, xh, yl, yh;
};

__device__ __forceinline__ WarpTile warp_tile(int lane) {
    WarpTile t;
    if (lane < 28) {
        int i = 1, k = lane;
        while (k >= i) {
            k -= i;
            i++;
        }
        t.I = i;
        t.J = k;
        t.diag = 0;
        t.xl = t.xh = 10 * t.I;
        t.yl = t.yh = 10 * t.J;
    } else {
        t.I = 2 * (lane - 28);
        t.J = t.I + 1;
        t.diag = 1;
        t.xl = t.yl = 10 * t.I;
        t.xh = t.yh = 10 * t.J;
    }
    return t;
}

// predicates of one block step (pivot block P) for the positions of slot 8P+pp:
// row pp at c < pp / c > pp / c == pp, column pp at a < pp / a > pp / a == pp
struct WarpPred {
    bool rl, rh, re, cl, ch, ce;
};

__device__ __forceinline__ WarpPred warp_pred(const WarpTile &t, int P) {
    const bool fRow = !t.diag && t.I == P, fCol = !t.diag && t.J == P;
    const bool fL = t.diag && t.I == P, fH = t.diag && t.J == P;
    WarpPred w;
    w.rl = fRow || fL;
    w.rh = fRow || fH;
    w.re = fRow;
    w.cl = fCol || fH;
    w.ch = fCol || fL;
    w.ce = fCol;
    return w;
}

// the pairs of slot 8P+PP: publish them into pcol (by the other slot)
template <int PP>
__device__ __forceinline__ void publish(const float2 (&R)[8][8], const WarpTile &t, const WarpPred &w, float2 *pc) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
        if (c < PP) {
            if (w.rl) pc[t.yl + c] = R[PP][c];
        } else if (c > PP) {
            if (w.rh) pc[t.yh + c] = R[PP][c];
        } else {
            if (w.re) pc[t.yh + c] = R[PP][c];
        }
    }
#pragma unroll
    for (int a = 0; a < 8; a++) {
        if (a < PP) {
            if (w.cl) pc[t.xh + a] = R[a][PP];
        } else if (a > PP) {
            if (w.ch) pc[t.xl + a] = R[a][PP];
        } else {
            if (w.ce) pc[t.xl + a] = R[a][PP];
        }
    }
}

// the pairs of slot 8P+PP take the entering row's values (dense by slot)
template <int PP>
__device__ __forceinline__ void enter(float2 (&R)[8][8], const WarpTile &t, const WarpPred &w, const float2 *nr) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
        if (c < PP) {
            if (w.rl) R[PP][c] = nr[t.yl + c];
        } else if (c > PP) {
            if (w.rh) R[PP][c] = nr[t.yh + c];
        } else {
            if (w.re) R[PP][c] = nr[t.yh + c];
        }
    }
#pragma unroll
    for (int a = 0; a < 8; a++) {
        if (a < PP) {
            if (w.cl) R[a][PP] = nr[t.xh + a];
        } else if (a > PP) {
            if (w.ch) R[a][PP] = nr[t.xl + a];
        } else {
            if (w.ce) R[a][PP] = nr[t.xl + a];
        }
    }
}

__device__ __forceinline__ float4 ld4(const float2 *p) { return *reinterpret_cast<const float4 *>(p); }

// rank-1 update of the tile: R[a][c] -= pcol[x(a)] pcs[y(c)]
__device__ __forceinline__ void tile_update(float2 (&R)[8][8], const WarpTile &t, const float2 *pc, const float2 *ps) {
    float2 yl[8], yh[8];
#pragma unroll
    for (int c = 0; c < 8; c += 2) {
        const float4 u = ld4(ps + t.yl + c), v = ld4(ps + t.yh + c);
        yl[c] = cf(u.x, u.y);
        yl[c + 1] = cf(u.z, u.w);
        yh[c] = cf(v.x, v.y);
        yh[c + 1] = cf(v.z, v.w);
    }
#pragma unroll
    for (int a = 0; a < 8; a += 2) {
        const float4 u = ld4(pc + t.xl + a), v = ld4(pc + t.xh + a);
        const float2 xl0 = cf(u.x, u.y), xl1 = cf(u.z, u.w), xh0 = cf(v.x, v.y), xh1 = cf(v.z, v.w);
#pragma unroll
        for (int c = 0; c < 8; c++) {
            R[a][c] = cfmsf(R[a][c], c < a ? xl0 : xh0, c < a ? yl[c] : yh[c]);
            R[a + 1][c] = cfmsf(R[a + 1][c], c < a + 1 ? xl1 : xh1, c < a + 1 ? yl[c] : yh[c]);
        }
    }
}

#define CRGPU_PP_SWITCH(pp, CALL) \
    switch (pp) {                   \
        case 0: CALL(0); break;     \
        case 1: CALL(1); break;     \
        case 2: CALL(2); break;     \
        case 3: CALL(3); break;     \
        case 4: CALL(4); break;     \
        case 5: CALL(5); break;     \
        case 6: CALL(6); break;     \
        default: CALL(7); break;    \
    }

// One column: pivot slot p = 8P+pp, column j, buffer pb.  pp selects the
// register positions of publish/enter through a switch; the rest of the
// column (the bulk of the instructions) is shared by the eight positions.
// The scalar chain of the pivot (reciprocal, scaled copy) sits between the
// two __syncwarp; the L entries, the right-hand side and the staging follow
// the tile update, branch-free, so that they interleave with its
// multiply-adds.
template <int FUSE>
__device__ __forceinline__ void warp_column(float2 (&R)[8][8], float2 &d0, float2 &d1, float2 &b0, float2 &b1,
                                            const WarpTile &t, const WarpPred &w, WarpSmem &S, const DevProblem &P,
                                            const double2 *as, const double2 *bv, float2 *L, float2 *yv, int j,
                                            int p, int pp, int lane, int &bad) {
    const int n = P.n, mb = P.mb, Wb = mb + 1;
    const int pb = j & 1;
    float2 *pc = S.pcol[pb];
    float2 *ps = S.pcs[pb];
    // ---- 1. publish the pivot column
#define CRGPU_PUB(K) publish<K>(R, t, w, pc)
    CRGPU_PP_SWITCH(pp, CRGPU_PUB)
#undef CRGPU_PUB
    if (lane == (p & 31)) pc[pad(p)] = (p >> 5) ? d1 : d0;
    // the raw row scattered below (committed kRaw - 1 groups ago) has landed
    cp_wait<kRaw - 1>();
    __syncwarp();
    // ---- 2. pivot, reciprocal, scaled copy, square root; the dense slot of
    //      row j+63 (entered at column j-1) is cleared for row j+63+kDense
    const float2 app = pc[pad(p)];
    const float r2 = app.x * app.x + app.y * app.y;
    bad |= (!(r2 > 0.f) || !(r2 < INFINITY) || (P.ldc && !(app.x > 0.f))) ? 28 : 0;  // src/chol.f90:67-71, choldc.f90:66-70
    const float ir2 = __fdividef(1.f, r2);
    const float2 inv = cf(app.x * ir2, -app.y * ir2);
    const float2 pc0 = pc[pad(lane)], pc1 = pc[pad(lane + 32)];
    const float2 ps0 = cmulf(pc0, inv), ps1 = cmulf(pc1, inv);
    ps[pad(lane)] = ps0;
    ps[pad(lane + 32)] = ps1;
    const int qd = (j + kWW - 1) & (kDense - 1);  // dense slot of rows j+63 and j+63+kDense
    *reinterpret_cast<float4 *>(&S.dense[qd][pad(2 * lane)]) = make_float4(0.f, 0.f, 0.f, 0.f);
    d0 = cfmsf(d0, pc0, ps0);
    d1 = cfmsf(d1, pc1, ps1);
    const float2 sq = csqrt_fast(app);
    const float2 isq = cmulf(sq, inv);  // 1/sqrt(a_pp) = sqrt(a_pp)/a_pp
    __syncwarp();
    // ---- 3. rank-1 update of the tile; in the same basic block (branch-free)
    //      the L entries of column j (Cholesky form, as src/chol.f90 stores
    //      them), the fused forward substitution and the staging of row
    //      j+63+kDense from its raw pattern row into dense slot qd, then the
    //      raw row kRaw further ahead into the freed raw slot
    tile_update(R, t, pc, ps);
    const float2 l0 = cmulf(pc0, isq), l1 = cmulf(pc1, isq);
    {
        const int dd0 = (lane - p) & (kWW - 1), dd1 = (lane + 32 - p) & (kWW - 1);
        if (dd0 == 0 || dd1 == 0) L[(size_t)j * Wb + mb] = sq;
        if (dd0 != 0 && dd0 <= mb && j + dd0 < n) L[(size_t)(j + dd0) * Wb + (mb - dd0)] = l0;
        if (dd1 != 0 && dd1 <= mb && j + dd1 < n) L[(size_t)(j + dd1) * Wb + (mb - dd1)] = l1;
    }
    if (FUSE) {
        const float2 bsel = (p >> 5) ? b1 : b0;
        const float2 bp = cf(__shfl_sync(0xffffffffu, bsel.x, p & 31), __shfl_sync(0xffffffffu, bsel.y, p & 31));
        const float2 yj = cmulf(bp, isq);
        if (lane == (p & 31)) yv[j] = yj;
        b0 = cfmsf(b0, l0, yj);
        b1 = cfmsf(b1, l1, yj);
    }
    {
        const int r = j + kWW - 1 + kDense, q = r & (kRaw - 1);
        const bool live = r < n && lane < P.rw;
        const int c = live ? S.raw_col[q][lane] : -1;
        if (c >= 0) S.dense[qd][pad(c & (kWW - 1))] = to_f(S.raw_val[q][lane]);
        if (lane == 31) S.dense_b[qd] = (FUSE && r < n) ? to_f(S.raw_b[q]) : cf(0.f, 0.f);
        raw_issue(P, as, bv, r + kRaw, FUSE, S, lane);
    }
    // ---- 4. row j+64 enters slot p
    {
        const int qe = j & (kDense - 1);
        const float2 *nr = S.dense[qe];
#define CRGPU_ENT(K) enter<K>(R, t, w, nr)
        CRGPU_PP_SWITCH(pp, CRGPU_ENT)
#undef CRGPU_ENT
        const float2 nd = nr[pad(p)];
        const bool own = lane == (p & 31), hi = p >> 5;
        d0 = (own && !hi) ? nd : d0;
        d1 = (own && hi) ? nd : d1;
        if (FUSE) {
            const float2 nbv = S.dense_b[qe];
            b0 = (own && !hi) ? nbv : b0;
            b1 = (own && hi) ? nbv : b1;
        }
    }
}

template <int PP, class SM>
__device__ __forceinline__ void warp_enter_initial(float2 (&R)[8][8], float2 &d0, float2 &d1, float2 &b0,
                                                   float2 &b1, const WarpTile &t, const WarpPred &w, SM &S,
                                                   int p, int lane) {
    enter<PP>(R, t, w, S.dense[0]);
    if (lane == (p & 31)) {
        if (p >> 5) {
            d1 = S.dense[0][pad(p)];
            b1 = S.dense_b[0];
        } else {
            d0 = S.dense[0][pad(p)];
            b0 = S.dense_b[0];
        }
    }
    __syncwarp();
}

// MINB: warps an SM the register budget is sized for.  12 (168 registers)
// keeps up to 12 systems an SM resident; 8 leaves the compiler ~206
// registers, which makes one system's column ~1.5x faster, for launches of
// at most 8 systems an SM.
template <int FUSE, int MINB>
__global__ __launch_bounds__(32, MINB) void k_factor_warp(DevProblem P, DevBatch B) {
    constexpr int fuse = FUSE;
    __shared__ WarpSmem S;
    const int lane = threadIdx.x;
    const int s = blockIdx.x;
    if (s >= B.nsys) return;
    const int n = P.n, mb = P.mb, Wb = mb + 1;
    float2 *L = (float2 *)B.L + (size_t)s * B.lpitch;
    float2 *yv = (float2 *)B.y + (size_t)s * n;
    const double2 *as = B.As + (size_t)s * P.nnz;
    const double2 *bv = B.b + (size_t)s * n;
    const WarpTile t = warp_tile(lane);
    int bad = 0;

    // band entries before column 0 (rows 0..mb-1) are outside the matrix: zero
    for (int q = lane; q < mb * Wb; q += 32) {
        const int r = q / Wb, o = q % Wb;
        if (r < n && o < mb - r) L[(size_t)r * Wb + o] = cf(0.f, 0.f);
    }
    float2 R[8][8];
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int c = 0; c < 8; c++) R[a][c] = cf(0.f, 0.f);
    float2 d0 = cf(0.f, 0.f), d1 = cf(0.f, 0.f), b0 = cf(0.f, 0.f), b1 = cf(0.f, 0.f);

    // ---- initial window: rows 0..63 enter slots 0..63 in order (each pair takes
    //      its value from the later row's pattern)
    for (int P8 = 0; P8 < 8; P8++) {
        const WarpPred w = warp_pred(t, P8);
#define CRGPU_ENTER0(PP)                                                          \
    load_dense_row(P, as, bv, 8 * P8 + PP, fuse, S, 0, lane);                    \
    warp_enter_initial<PP>(R, d0, d1, b0, b1, t, w, S, 8 * P8 + PP, lane);
        CRGPU_ENTER0(0) CRGPU_ENTER0(1) CRGPU_ENTER0(2) CRGPU_ENTER0(3)
        CRGPU_ENTER0(4) CRGPU_ENTER0(5) CRGPU_ENTER0(6) CRGPU_ENTER0(7)
#undef CRGPU_ENTER0
    }
    // the diagonal pairs' unused positions R[a][a] of the diagonal-block lanes
    // are never read; entering rows 64..66 as dense rows, 67.. in flight
    for (int q = 0; q < kDense - 1; q++) load_dense_row(P, as, bv, kWW + q, fuse, S, (kWW + q) & (kDense - 1), lane);
    for (int q = 0; q < kRaw; q++) raw_issue(P, as, bv, kWW - 1 + kDense + q, fuse, S, lane);

    const int nstep = (n + 7) / 8;
    for (int J8 = 0; J8 < nstep; J8++) {
        const int P8 = J8 & 7;
        const WarpPred w = warp_pred(t, P8);
        const int j0 = 8 * J8;
#pragma unroll 1
        for (int pp = 0; pp < 8 && j0 + pp < n; pp++)
            warp_column<FUSE>(R, d0, d1, b0, b1, t, w, S, P, as, bv, L, yv, j0 + pp, 8 * P8 + pp, pp, lane, bad);
    }
    cp_wait<0>();
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (lane == 0 && bad) atomicCAS(&B.status[s], 0, bad);
}

// ---------------------------------------------------------------------------
// Two columns a step (mb <= 62).  The pivot slots p1 = 8P+2h, p2 = p1+1 lie in
// one block; their columns are published together, the 2x2 pivot block is
// factored (L D L^T) in every lane, and the tile takes the two rank-1 updates
// back to back.  The rows j+64 and j+65 then enter slots p1 and p2: with
// mb <= 62 neither has an entry in column j+1 (63 or more columns before it),
// so no entering row misses an update of the step.
// ---------------------------------------------------------------------------
struct WarpSmem2 {
    __align__(16) float2 pcol[2][2][kPad];  // [step parity][column of the step] by padded slot; the second
                                            // column after the first's elimination
    __align__(16) float2 pcs[2][2][kPad];   // scaled: pcol / d
    __align__(16) float2 dense[kDense][kPad];
    float2 dense_b[kDense];
    // the cp.async ring of the 12-warp variant (no registers to spare for rows ahead)
    __align__(16) double2 raw_val[kRaw][kRawCap];
    int raw_col[kRaw][kRawCap];
    __align__(16) double2 raw_b[kRaw];
};

// the pattern rows r and r+1 into their raw slots, one commit group
__device__ __forceinline__ void raw_issue2(const DevProblem &P, const double2 *as, const double2 *bv, int r,
                                           int fuse, WarpSmem2 &S, int lane) {
#pragma unroll
    for (int u = 0; u < 2; u++) {
        const int rr = r + u, q = rr & (kRaw - 1);
        if (rr < P.n) {
            if (lane < P.rw) {
                cp_async16(&S.raw_val[q][lane], as + (size_t)rr * P.rw + lane);
                cp_async4(&S.raw_col[q][lane], P.col + (size_t)rr * P.rw + lane);
            }
            if (lane == 31 && fuse) cp_async16(&S.raw_b[q], bv + rr);
        }
    }
    cp_commit();
}

// Two pattern rows one step ahead in registers (plain loads, so nothing waits
// on them until the next step scatters them): lane e < rw holds entry e of
// each row, lane 31 also its right-hand side.
struct RowsAhead {
    int col[2];
    double2 val[2], b[2];
};

__device__ __forceinline__ void rows_load(RowsAhead &A, const DevProblem &P, const double2 *as, const double2 *bv,
                                          int r, int fuse, int lane) {
#pragma unroll
    for (int u = 0; u < 2; u++) {
        const int rr = r + u;
        const bool live = rr < P.n && lane < P.rw;
        A.col[u] = live ? P.col[(size_t)rr * P.rw + lane] : -1;
        A.val[u] = live ? as[(size_t)rr * P.rw + lane] : make_double2(0.0, 0.0);
        A.b[u] = (rr < P.n && fuse && lane == 31) ? bv[rr] : make_double2(0.0, 0.0);
    }
}

#define CRGPU_H_SWITCH(h, CALL) \
    switch (h) {                  \
        case 0: CALL(0); break;   \
        case 1: CALL(2); break;   \
        case 2: CALL(4); break;   \
        default: CALL(6); break;  \
    }

template <int FUSE, int MINB>
__device__ __forceinline__ void warp_step2(float2 (&R)[8][8], float2 &d0, float2 &d1, float2 &b0, float2 &b1,
                                           const WarpTile &t, const WarpPred &w, WarpSmem2 &S, RowsAhead &A,
                                           const DevProblem &P, const double2 *as, const double2 *bv, float2 *L,
                                           float2 *yv, int j, int p1, int h, int lane, int &bad) {
    const int n = P.n, mb = P.mb, Wb = mb + 1;
    const int p2 = p1 + 1, pb = (j >> 1) & 1;
    const bool two = j + 1 < n;  // the second column exists
    float2 *pc1 = S.pcol[pb][0], *pc2 = S.pcol[pb][1];
    float2 *ps1 = S.pcs[pb][0], *ps2 = S.pcs[pb][1];
    // ---- 1. publish both pivot columns
#define CRGPU_PUB2(K)                 \
    publish<K>(R, t, w, pc1);         \
    publish<K + 1>(R, t, w, pc2);
    CRGPU_H_SWITCH(h, CRGPU_PUB2)
#undef CRGPU_PUB2
    {
        const bool own1 = lane == (p1 & 31), own2 = lane == (p2 & 31);
        if (own1) pc1[pad(p1)] = (p1 >> 5) ? d1 : d0;
        if (own2) pc2[pad(p2)] = (p2 >> 5) ? d1 : d0;
    }
    if (MINB != 8) cp_wait<1>();  // the raw rows scattered below (committed one step before the last) have landed
    __syncwarp();
    // ---- 2. the 2x2 pivot block (L D L^T), the second column after the first's
    //      elimination, the scaled copies, the diagonal, the square roots
    const float2 a11 = pc1[pad(p1)], a21 = pc1[pad(p2)], a22 = pc2[pad(p2)];
    const float r1 = a11.x * a11.x + a11.y * a11.y;
    const float2 inv1 = cf(a11.x * __fdividef(1.f, r1), -a11.y * __fdividef(1.f, r1));
    const float2 l21 = cmulf(a21, inv1);
    const float2 dd2 = two ? cfmsf(a22, l21, a21) : cf(1.f, 0.f);
    const float r2 = dd2.x * dd2.x + dd2.y * dd2.y;
    const float2 inv2 = cf(dd2.x * __fdividef(1.f, r2), -dd2.y * __fdividef(1.f, r2));
    bad |= (!(r1 > 0.f) || !(r1 < INFINITY) || (P.ldc && !(a11.x > 0.f))) ? 28 : 0;  // src/chol.f90:67-71, choldc.f90:66-70
    bad |= (!(r2 > 0.f) || !(r2 < INFINITY) || (P.ldc && !(dd2.x > 0.f))) ? 28 : 0;
    const float2 c10 = pc1[pad(lane)], c11 = pc1[pad(lane + 32)];
    const float2 c20 = two ? cfmsf(pc2[pad(lane)], l21, c10) : cf(0.f, 0.f);
    const float2 c21 = two ? cfmsf(pc2[pad(lane + 32)], l21, c11) : cf(0.f, 0.f);
    const float2 s10 = cmulf(c10, inv1), s11 = cmulf(c11, inv1);
    const float2 s20 = cmulf(c20, inv2), s21 = cmulf(c21, inv2);
    __syncwarp();  // every lane has read pc2 before it takes the eliminated values
    pc2[pad(lane)] = c20;
    pc2[pad(lane + 32)] = c21;
    ps1[pad(lane)] = s10;
    ps1[pad(lane + 32)] = s11;
    ps2[pad(lane)] = s20;
    ps2[pad(lane + 32)] = s21;
    d0 = cfmsf(cfmsf(d0, c10, s10), c20, s20);
    d1 = cfmsf(cfmsf(d1, c11, s11), c21, s21);
    const int qa = (j + kWW - 2) & (kDense - 1), qb = (j + kWW - 1) & (kDense - 1);  // slots of rows j+62, j+63
    *reinterpret_cast<float4 *>(&S.dense[qa][pad(2 * lane)]) = make_float4(0.f, 0.f, 0.f, 0.f);
    *reinterpret_cast<float4 *>(&S.dense[qb][pad(2 * lane)]) = make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 sq1 = csqrt_fast(a11), isq1 = cmulf(sq1, inv1);
    const float2 sq2 = csqrt_fast(dd2), isq2 = cmulf(sq2, inv2);
    __syncwarp();
    // ---- 3. the two rank-1 updates of the tile
    tile_update(R, t, pc1, ps1);
    if (two) tile_update(R, t, pc2, ps2);
    // ---- the L entries of columns j and j+1 (Cholesky form) and the fused
    //      forward substitution
    {
        const float2 l10 = cmulf(c10, isq1), l11 = cmulf(c11, isq1);
        const float2 l20 = cmulf(c20, isq2), l21c = cmulf(c21, isq2);
        const int e0 = (lane - p1) & (kWW - 1), e1 = (lane + 32 - p1) & (kWW - 1);  // row offsets from j
        if (e0 == 0 || e1 == 0) L[(size_t)j * Wb + mb] = sq1;
        if (e0 != 0 && e0 <= mb && j + e0 < n) L[(size_t)(j + e0) * Wb + (mb - e0)] = l10;
        if (e1 != 0 && e1 <= mb && j + e1 < n) L[(size_t)(j + e1) * Wb + (mb - e1)] = l11;
        if (two) {
            if (e0 == 1 || e1 == 1) L[(size_t)(j + 1) * Wb + mb] = sq2;
            if (e0 > 1 && e0 - 1 <= mb && j + e0 < n) L[(size_t)(j + e0) * Wb + (mb - e0 + 1)] = l20;
            if (e1 > 1 && e1 - 1 <= mb && j + e1 < n) L[(size_t)(j + e1) * Wb + (mb - e1 + 1)] = l21c;
        }
        if (FUSE) {
            const float2 bs1 = (p1 >> 5) ? b1 : b0;
            const float2 bp1 = cf(__shfl_sync(0xffffffffu, bs1.x, p1 & 31), __shfl_sync(0xffffffffu, bs1.y, p1 & 31));
            const float2 y1 = cmulf(bp1, isq1);
            b0 = cfmsf(b0, l10, y1);
            b1 = cfmsf(b1, l11, y1);
            const float2 bs2 = (p2 >> 5) ? b1 : b0;
            const float2 bp2 = cf(__shfl_sync(0xffffffffu, bs2.x, p2 & 31), __shfl_sync(0xffffffffu, bs2.y, p2 & 31));
            const float2 y2 = cmulf(bp2, isq2);
            if (lane == (p1 & 31)) yv[j] = y1;
            if (two && lane == (p2 & 31)) yv[j + 1] = y2;
            if (two) {
                b0 = cfmsf(b0, l20, y2);
                b1 = cfmsf(b1, l21c, y2);
            }
        }
    }
    // ---- staging: rows j+66, j+67 into the dense slots cleared above; 8 warps an
    //      SM: loaded into registers one step ago, and rows j+68, j+69 are loaded
    //      now; 12 warps an SM: from the cp.async ring, which then takes the
    //      rows four further ahead
    if (MINB == 8) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int qd = (j + kWW + 2 + u) & (kDense - 1);
            if (A.col[u] >= 0) S.dense[qd][pad(A.col[u] & (kWW - 1))] = to_f(A.val[u]);
            if (lane == 31) S.dense_b[qd] = to_f(A.b[u]);
        }
        rows_load(A, P, as, bv, j + kWW + 4, FUSE, lane);
    } else {
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int r = j + kWW + 2 + u, q = r & (kRaw - 1), qd = r & (kDense - 1);
            const bool live = r < n && lane < P.rw;
            const int c = live ? S.raw_col[q][lane] : -1;
            if (c >= 0) S.dense[qd][pad(c & (kWW - 1))] = to_f(S.raw_val[q][lane]);
            if (lane == 31) S.dense_b[qd] = (FUSE && r < n) ? to_f(S.raw_b[q]) : cf(0.f, 0.f);
        }
        raw_issue2(P, as, bv, j + kWW + 6, FUSE, S, lane);
    }
    // ---- 4. rows j+64 and j+65 enter slots p1 and p2 (in this order: the pair
    //      (p1, p2) takes its value from row j+65's pattern)
    {
        const float2 *na = S.dense[(j + kWW) & (kDense - 1)], *nb = S.dense[(j + kWW + 1) & (kDense - 1)];
#define CRGPU_ENT2(K)              \
    enter<K>(R, t, w, na);         \
    enter<K + 1>(R, t, w, nb);
        CRGPU_H_SWITCH(h, CRGPU_ENT2)
#undef CRGPU_ENT2
        const bool hi = p1 >> 5;  // p1, p2 lie in the same half
        const bool own1 = lane == (p1 & 31), own2 = lane == (p2 & 31);
        const float2 nd1 = na[pad(p1)], nd2 = nb[pad(p2)];
        d0 = (own1 && !hi) ? nd1 : (own2 && !hi) ? nd2 : d0;
        d1 = (own1 && hi) ? nd1 : (own2 && hi) ? nd2 : d1;
        if (FUSE) {
            const float2 nb1 = S.dense_b[(j + kWW) & (kDense - 1)], nb2 = S.dense_b[(j + kWW + 1) & (kDense - 1)];
            b0 = (own1 && !hi) ? nb1 : (own2 && !hi) ? nb2 : b0;
            b1 = (own1 && hi) ? nb1 : (own2 && hi) ? nb2 : b1;
        }
    }
}

template <int FUSE, int MINB>
__global__ __launch_bounds__(32, MINB) void k_factor_warp2(DevProblem P, DevBatch B) {
    constexpr int fuse = FUSE;
    __shared__ WarpSmem2 S;
    const int lane = threadIdx.x;
    const int s = blockIdx.x;
    if (s >= B.nsys) return;
    const int n = P.n, mb = P.mb, Wb = mb + 1;
    float2 *L = (float2 *)B.L + (size_t)s * B.lpitch;
    float2 *yv = (float2 *)B.y + (size_t)s * n;
    const double2 *as = B.As + (size_t)s * P.nnz;
    const double2 *bv = B.b + (size_t)s * n;
    const WarpTile t = warp_tile(lane);
    int bad = 0;
    for (int q = lane; q < mb * Wb; q += 32) {
        const int r = q / Wb, o = q % Wb;
        if (r < n && o < mb - r) L[(size_t)r * Wb + o] = cf(0.f, 0.f);
    }
    float2 R[8][8];
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int c = 0; c < 8; c++) R[a][c] = cf(0.f, 0.f);
    float2 d0 = cf(0.f, 0.f), d1 = cf(0.f, 0.f), b0 = cf(0.f, 0.f), b1 = cf(0.f, 0.f);
    for (int P8 = 0; P8 < 8; P8++) {
        const WarpPred w = warp_pred(t, P8);
#define CRGPU_ENTER0(PP)                                                          \
    load_dense_row(P, as, bv, 8 * P8 + PP, fuse, S, 0, lane);                    \
    warp_enter_initial<PP>(R, d0, d1, b0, b1, t, w, S, 8 * P8 + PP, lane);
        CRGPU_ENTER0(0) CRGPU_ENTER0(1) CRGPU_ENTER0(2) CRGPU_ENTER0(3)
        CRGPU_ENTER0(4) CRGPU_ENTER0(5) CRGPU_ENTER0(6) CRGPU_ENTER0(7)
#undef CRGPU_ENTER0
    }
    // rows 64, 65 (step 0) as dense rows; 66, 67 in registers
    load_dense_row(P, as, bv, kWW, fuse, S, kWW & (kDense - 1), lane);
    load_dense_row(P, as, bv, kWW + 1, fuse, S, (kWW + 1) & (kDense - 1), lane);
    RowsAhead A;
    if (MINB == 8) {
        rows_load(A, P, as, bv, kWW + 2, fuse, lane);
    } else {
        raw_issue2(P, as, bv, kWW + 2, fuse, S, lane);
        raw_issue2(P, as, bv, kWW + 4, fuse, S, lane);
    }
    const int nstep = (n + 7) / 8;
    for (int J8 = 0; J8 < nstep; J8++) {
        const int P8 = J8 & 7;
        const WarpPred w = warp_pred(t, P8);
        const int j0 = 8 * J8;
#pragma unroll 1
        for (int h = 0; h < 4 && j0 + 2 * h < n; h++)
            warp_step2<FUSE, MINB>(R, d0, d1, b0, b1, t, w, S, A, P, as, bv, L, yv, j0 + 2 * h, 8 * P8 + 2 * h, h,
                                   lane, bad);
    }
    cp_wait<0>();
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (lane == 0 && bad) atomicCAS(&B.status[s], 0, bad);
}

}  // namespace

bool launch_factor_warp(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st) {
    if (P.mb + 1 > kWW || P.rw > kRawCap || P.rw > 32) return false;
    if (B.nsys <= 0) return true;
    const bool few = B.nsys <= 8 * nsm;
    if (P.mb <= 62) {  // two columns a step
        if (few)
            fuse ? k_factor_warp2<1, 8><<<B.nsys, 32, 0, st>>>(P, B) : k_factor_warp2<0, 8><<<B.nsys, 32, 0, st>>>(P, B);
        else
            fuse ? k_factor_warp2<1, 12><<<B.nsys, 32, 0, st>>>(P, B) : k_factor_warp2<0, 12><<<B.nsys, 32, 0, st>>>(P, B);
    } else if (few) {
        fuse ? k_factor_warp<1, 8><<<B.nsys, 32, 0, st>>>(P, B) : k_factor_warp<0, 8><<<B.nsys, 32, 0, st>>>(P, B);
    } else {
        fuse ? k_factor_warp<1, 12><<<B.nsys, 32, 0, st>>>(P, B) : k_factor_warp<0, 12><<<B.nsys, 32, 0, st>>>(P, B);
    }
    return true;
}

}  // namespace crgpu
