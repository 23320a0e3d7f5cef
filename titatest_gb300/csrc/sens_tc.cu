// Jacobian of CRMod (src/bsens.f90:23-197) on the tensor cores, in the Gram
// form of the element contraction.
//
// For element e, wavenumber k and measurement i with current electrodes
// (e1, e2) and voltage electrodes (e3, e4) the reference sums
//   hsens_k = sum_{m,n} K_k[m][n] (u_m(e4) - u_m(e3)) (u_n(e2) - u_n(e1)),
// u_m(a) = kpot(node_m, a, k), K_k the element matrix elbg.  The form is
// bilinear in the two dipoles, so with the electrode Gram matrix of the
// element
//   P[a][b] = sum_k w_k sum_{m,n} u_m(a) K_k[m][n] u_n(b)        (eanz x eanz)
// every measurement is P[e4][e2] - P[e4][e1] - P[e3][e2] + P[e3][e1].
// P is one complex GEMM per element: P = sum_k U_k W_k^T with U_k the
// element's potentials (eanz x nk) and W_k = w_k U_k K_k.  In real form, per
// wavenumber, one tcgen05.mma.kind::tf32 with M = 128 (electrodes a),
// N = 2 eanz (electrode b, real / imaginary part) and K = 8:
//   A row a      = [Re U(a, 0..3) | Im U(a, 0..3)]
//   B row 2b     = [Re W(b, 0..3) | -Im W(b, 0..3)]   -> Re P[a][b]
//   B row 2b + 1 = [Im W(b, 0..3) |  Re W(b, 0..3)]   -> Im P[a][b]
// Three products of the tf32 hi/lo splits (hi.hi + hi.lo + lo.hi) keep FP32
// accuracy; an absent electrode (-1, zero potential) is one more row and
// column of P, which stays zero.  The accumulator stays in TMEM over the
// wavenumbers; the epilogue copies P to shared memory and one thread per
// measurement forms its four-term combination and the reference's scaling,
// written coalesced into sens(e, :).
//
// Accuracy: P is rounded relative to its own size in the FP32 accumulator,
// and the four-term combination cancels what the two potential (or current)
// electrodes have in common at the element.  Relative to max|J| of
// src/bsens.f90 that stays below 1e-6 (8.7e-7 on a 96-electrode survey).
// src/bsensi.f90 divides by V_i, which amplifies the cancellation of long
// dipole-dipole measurements (1.3e-5 on a 30-electrode survey); that mode
// keeps the SIMT contraction of post.cu, which forms the dipole differences
// before the products.
//
// 256 threads per block, one element at a time (persistent over elements);
// the element potentials of wavenumber k+1 are fetched by cp.async while the
// operands of k are built, operands are double buffered against the MMAs of
// the previous wavenumber.  eanz + 1 <= 128 (one M tile).
#include <mutex>

#include "async.cuh"
#include "crgpu_internal.h"
#include "device.cuh"
#include "kernels.h"
#include "tc_common.cuh"

namespace crgpu {

using namespace tc;

namespace {

constexpr int kStThreads = 256;
constexpr int kStM = 128;       // MMA M: electrodes a
constexpr int kStCols = 256;    // TMEM columns allocated (N <= 256)
static constexpr double kStPi = 3.14159265358979323846264338327950288;

// dynamic shared memory layout (bytes); the operand buffers and P alias
struct StLayout {
    int N;                   // MMA N = 2 E rounded up to 16 (E = eanz + 1 rows of P)
    int off_b;               // offset of the B buffers inside one operand buffer
    int op_bytes;            // one operand buffer: A hi, A lo (128 x 8), B hi, B lo (N x 8) floats
    int p_bytes;             // P: E x E float2
    int u_off, u_bytes;      // element potentials, two wavenumbers: [2][4][eanz] float2 (sized for E)
    int ctl_off;             // StCtl
    int scale_off;           // -strom_i / pi per measurement (FP32), or 0: read in FP64
    int total;
};

__host__ __device__ inline StLayout st_layout(int E, int nanz) {
    StLayout L;
    L.N = ((2 * E + 15) / 16) * 16;
    L.off_b = 2 * kStM * 8 * 4;
    L.op_bytes = L.off_b + 2 * L.N * 8 * 4;
    L.p_bytes = E * E * 8;
    const int region = (2 * L.op_bytes > L.p_bytes ? 2 * L.op_bytes : L.p_bytes);
    L.u_off = (region + 127) / 128 * 128;
    L.u_bytes = 2 * 4 * E * 8;
    L.ctl_off = L.u_off + L.u_bytes;
    L.total = L.ctl_off + 128;  // barriers and flags
    L.scale_off = 0;
    if (L.total + nanz * 4 <= 200 * 1024) {
        L.scale_off = L.total;
        L.total += (nanz * 4 + 15) / 16 * 16;
    }
    return L;
}

// FP32 -> FP64 from the bit fields (exact for normal numbers; zero and
// subnormals give a signed zero, inf / nan stay inf / nan) without the FP64
// pipe, which runs at a small fraction of the FP32 rate here
__device__ __forceinline__ double widen(float x) {
    const uint32_t u = __float_as_uint(x), e8 = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    const uint32_t e11 = e8 == 0u ? 0u : (e8 == 0xFFu ? 0x7FFu : e8 + 896u);
    const uint32_t hi = (u & 0x80000000u) | (e11 << 20) | (e8 == 0u ? 0u : (m >> 3));
    const uint32_t lo = e8 == 0u ? 0u : (m << 29);
    return __hiloint2double((int)hi, (int)lo);
}

struct StCtl {
    uint64_t bar[2];  // MMAs of the wavenumbers using operand buffer 0 / 1 completed
    uint32_t uses[2];
    uint32_t tmem_base;
    int fail;
};

}  // namespace

__global__ __launch_bounds__(kStThreads) void k_sens_tc(DevProblem P, const float2 *__restrict__ kpot,
                                                         double2 *__restrict__ sens, int e_first, int e_end) {
    extern __shared__ __align__(1024) unsigned char st_raw[];
    const int eanz = P.eanz, nanz = P.nanz, n = P.n, K = P.K;
    const int E = eanz + 1;  // electrodes and the zero-potential one (index eanz)
    const StLayout Ly = st_layout(E, nanz);
    const int N = Ly.N;
    auto opb = [&](int b) { return (float *)(st_raw + (size_t)b * Ly.op_bytes); };  // operand buffer b
    float2 *Psh = (float2 *)st_raw;
    float2 *ush = (float2 *)(st_raw + Ly.u_off);  // [2][4][eanz]
    StCtl &C = *(StCtl *)(st_raw + Ly.ctl_off);
    float *scale = Ly.scale_off ? (float *)(st_raw + Ly.scale_off) : nullptr;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&C.tmem_base)),
                     "r"(kStCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&C.bar[0], 1);
        mbar_init(&C.bar[1], 1);
        mbar_init_fence();
        C.fail = 0;
        C.uses[0] = C.uses[1] = 0u;
    }
    if (scale)  // the measurements' scaling of src/bsens.f90, once per block
        for (int i = tid; i < nanz; i += kStThreads)
            scale[i] = (float)(-(P.swrtr ? P.strom[i] * (1.0 / kStPi) : P.strom[i]));
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = C.tmem_base;
    const uint32_t idesc = tf32_idesc(kStM, N);
    uint32_t *uses = C.uses;  // commits on each buffer's barrier (kept by thread 0)
    bool fail = false;

    // potentials of element nodes, wavenumber k, all electrodes -> ush[slot]
    auto fetch_u = [&](int e, int nk, int k, int slot) {
        float2 *dst = ush + (size_t)slot * 4 * eanz;
        for (int t = tid; t < nk * eanz; t += kStThreads) {
            const int m = t / eanz, l = t % eanz;
            cp_async8(&dst[m * eanz + l], kpot + ((size_t)k * eanz + l) * n + P.enodes[e * 4 + m]);
        }
        cp_commit();
    };

    for (int e = e_first + blockIdx.x; e < e_end && !fail; e += gridDim.x) {
        const int nk = P.etype[e] == 3 ? 3 : 4;
        // A rows a >= E and B rows beyond 2 E stay zero
        for (int t = tid; t < 2 * (kStM - E) * 16; t += kStThreads) {
            const int buf = t / ((kStM - E) * 16), r = t % ((kStM - E) * 16);
            const int row = E + r / 16, k8 = r % 8, hl = (r / 8) & 1;
            opb(buf)[hl * kStM * 8 + kmaj(row, k8)] = 0.f;
        }
        for (int t = tid; t < 2 * (N - 2 * E) * 16; t += kStThreads) {
            const int buf = t / ((N - 2 * E) * 16), r = t % ((N - 2 * E) * 16);
            const int row = 2 * E + r / 16, k8 = r % 8, hl = (r / 8) & 1;
            opb(buf)[Ly.off_b / 4 + hl * N * 8 + kmaj(row, k8)] = 0.f;
        }
        fetch_u(e, nk, 0, 0);
        for (int k = 0; k < K; k++) {
            const int kb = k & 1;
            if (k + 1 < K) fetch_u(e, nk, k + 1, kb ^ 1);
            else cp_commit();
            // the MMAs that last read buffer kb (wavenumber k-2) must have completed
            if (tid == 0 && k >= 2) {
                if (!mbar_wait(&C.bar[kb], (uses[kb] - 1) & 1)) C.fail = 1;
                tc_fence_after();
            }
            cp_wait<1>();
            __syncthreads();
            if (C.fail) {
                fail = true;
                break;
            }
            // ---- operands of wavenumber k into buffer kb
            {
                const float2 *u = ush + (size_t)kb * 4 * eanz;
                float *A = opb(kb), *Bm = opb(kb) + Ly.off_b / 4;
                // potential of electrode a at node m in FP32 (a == eanz: zero)
                auto dev = [&](int m, int a) -> float2 {
                    return (m < nk && a < eanz) ? u[m * eanz + a] : cf(0.f, 0.f);
                };
                if (tid >= kStThreads - kStM) {  // A row a: [Re U | Im U]
                    const int a = tid - (kStThreads - kStM);
                    if (a < E) {
                        float hi[8], lo[8];
#pragma unroll
                        for (int m = 0; m < 4; m++) {
                            const float2 x = dev(m, a);
                            hi[m] = tf32_hi(x.x);
                            hi[4 + m] = tf32_hi(x.y);
                            lo[m] = x.x - hi[m];
                            lo[4 + m] = x.y - hi[4 + m];
                        }
                        put_row8(A, a, hi);
                        put_row8(A + kStM * 8, a, lo);
                    }
                } else if (tid < E) {  // B rows 2b, 2b+1 from W(b) = w_k U(b) K_k
                    const int b = tid;
                    const double *kel = P.elbg + ((size_t)k * P.elanz + e) * 10;
                    const float w = P.swrtr ? (float)P.kwnwi[k] : 1.f;
                    float2 ub[4];
#pragma unroll
                    for (int m = 0; m < 4; m++) ub[m] = dev(m, b);
                    float hr[8], hi2[8], lr[8], li[8];
#pragma unroll
                    for (int m = 0; m < 4; m++) {
                        float2 s = cf(0.f, 0.f);
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const int mx = m > q ? m : q, mn = m < q ? m : q;
                            const float kk = (q < nk && m < nk) ? (float)kel[mx * (mx + 1) / 2 + mn] * w : 0.f;
                            s.x = fmaf(kk, ub[q].x, s.x);
                            s.y = fmaf(kk, ub[q].y, s.y);
                        }
                        const float rh = tf32_hi(s.x), ih = tf32_hi(s.y);
                        const float rl = s.x - rh, il = s.y - ih;
                        hr[m] = rh;       // row 2b:   [Re W | -Im W]
                        hr[4 + m] = -ih;
                        lr[m] = rl;
                        lr[4 + m] = -il;
                        hi2[m] = ih;      // row 2b+1: [Im W | Re W]
                        hi2[4 + m] = rh;
                        li[m] = il;
                        li[4 + m] = rl;
                    }
                    put_row8(Bm, 2 * b, hr);
                    put_row8(Bm, 2 * b + 1, hi2);
                    put_row8(Bm + N * 8, 2 * b, lr);
                    put_row8(Bm + N * 8, 2 * b + 1, li);
                }
            }
            fence_proxy_async();
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
                const float *A = opb(kb), *Bm = opb(kb) + Ly.off_b / 4;
                const uint64_t ah = smem_desc(A), al = smem_desc(A + kStM * 8);
                const uint64_t bh = smem_desc(Bm), bl = smem_desc(Bm + N * 8);
                tc_mma_tf32(tbase, ah, bh, idesc, k > 0 ? 1u : 0u);
                tc_mma_tf32(tbase, ah, bl, idesc);
                tc_mma_tf32(tbase, al, bh, idesc);
                tc_commit(&C.bar[kb]);
                uses[kb]++;
            }
        }
        cp_wait<0>();
        if (fail) break;
        // ---- all MMAs of the element completed (the last commit covers them all)
        if (tid == 0) {
            const int kb = (K - 1) & 1;
            if (!mbar_wait(&C.bar[kb], (uses[kb] - 1) & 1)) C.fail = 1;
            if (K >= 2 && !mbar_wait(&C.bar[kb ^ 1], (uses[kb ^ 1] - 1) & 1)) C.fail = 1;
        }
        __syncthreads();
        tc_fence_after();
        if (C.fail) break;
        // ---- P from TMEM to shared memory: warp w reads lanes 32 (w % 4) ..,
        //      columns of half w / 4
        {
            const int q4 = warp & 3, half = warp >> 2, a = 32 * q4 + lane;
            const uint32_t tl = tbase + ((uint32_t)(32 * q4) << 16);
            for (int c0 = half * (N / 2); c0 < (half + 1) * (N / 2); c0 += 8) {
                float v[8];
                tmem_ld8(tl + (uint32_t)c0, v);
                if (a < E) {
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int b = c0 / 2 + j;
                        if (b < E) Psh[a * E + b] = cf(v[2 * j], v[2 * j + 1]);
                    }
                }
            }
        }
        tc_fence_before();
        __syncthreads();
        // ---- one thread per measurement: the dipole combination and the scaling
        //      of src/bsens.f90 (-strom / pi)
        {
            const int4 *meas4 = (const int4 *)P.meas;
            for (int i = tid; i < nanz; i += kStThreads) {
                const int4 ee = meas4[i];  // e1, e2, e3, e4 (-1: none -> the zero-potential row)
                const int x1 = ee.x >= 0 ? ee.x : eanz, x2 = ee.y >= 0 ? ee.y : eanz;
                const int x3 = ee.z >= 0 ? ee.z : eanz, x4 = ee.w >= 0 ? ee.w : eanz;
                const float2 p42 = Psh[x4 * E + x2], p41 = Psh[x4 * E + x1];
                const float2 p32 = Psh[x3 * E + x2], p31 = Psh[x3 * E + x1];
                const float dx = (p42.x - p41.x) - (p32.x - p31.x), dy = (p42.y - p41.y) - (p32.y - p31.y);
                if (scale) {
                    const float f = scale[i];
                    sens[(size_t)e * nanz + i] = cz(widen(dx * f), widen(dy * f));
                } else {
                    const double f = P.swrtr ? P.strom[i] * (1.0 / kStPi) : P.strom[i];
                    sens[(size_t)e * nanz + i] = cz(-(double)dx * f, -(double)dy * f);
                }
            }
        }
        __syncthreads();  // P is overwritten by the next element's operands
    }
    cp_wait<0>();
    // MMAs still in flight after a failure must land before the dealloc
    if (tid == 0) {
        for (int b = 0; b < 2; b++)
            if (uses[b] > 0) mbar_wait(&C.bar[b], (uses[b] - 1) & 1);
        if (C.fail) atomicCAS(P.err, 0, ERR_TIMEOUT);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
        mbar_inval(&C.bar[0]);
        mbar_inval(&C.bar[1]);
    }
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(kStCols) : "memory");
}

bool sens_tc_supported(const DevProblem &P, int mode) { return mode == 0 && P.eanz >= 1 && P.eanz + 1 <= kStM; }

void launch_sens_tc(const DevProblem &P, const float2 *kpot, double2 *sens, cudaStream_t st, int e_first,
                    int e_count) {
    const StLayout Ly = st_layout(P.eanz + 1, P.nanz);
    static std::once_flag once;
    static int nsm = 0;
    std::call_once(once, [] {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_sens_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    });
    const int per_sm = Ly.total <= 110 * 1024 ? 2 : 1;  // two 256-column TMEM allocations per SM at most
    const int grid = e_count < per_sm * nsm ? e_count : per_sm * nsm;
    if (grid <= 0) return;
    k_sens_tc<<<grid, kStThreads, Ly.total, st>>>(P, kpot, sens, e_first, e_first + e_count);
}

}  // namespace crgpu
