// Band triangular solves (src/vre.f90:5-71), FP64 iterative refinement of the
// mixed mode, and the unscaling into kpot (src/fem.f90:383-394).
//
// One warp solves one right-hand side.  Both sweeps read the band rows of L
// contiguously, streamed kRing rows ahead into shared memory by cp.async, and
// keep a W = mb+1 window of the working vector in shared memory (entry i in
// slot i mod W):
//   forward  L y = b : row-oriented, a warp-reduced dot product per row;
//   backward L^T x = y: the column sweep of vre (x_i broadcast, W updates).
#include "async.cuh"
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
    __device__ static double2 reduce(double2 a) {
        for (int o = 16; o > 0; o >>= 1) {
            a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
            a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
        }
        return a;
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
    __device__ static float2 reduce(float2 a) {
        for (int o = 16; o > 0; o >>= 1) {
            a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
            a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
        }
        return a;
    }
};

constexpr int kSolveWarps = 4;
constexpr int kRing = 8;  // rows of look-ahead streamed by cp.async

// per-warp shared memory: kRing vector entries, kRing rows, the W window;
// rounded to 16 bytes so every warp's region keeps cp.async alignment
template <typename T>
__host__ __device__ constexpr size_t solve_smem_per_warp(int W) {
    return (((size_t)kRing * W * sizeof(T) + (size_t)W * sizeof(T) + (size_t)kRing * sizeof(double2)) + 15) & ~(size_t)15;
}

// issue row rr of L (W entries) and vector entry vv (if >= 0) into ring slot sl
template <typename T>
__device__ __forceinline__ void ring_issue(const T *L, int W, int rr, int n, T *slot, const double2 *vsrc,
                                           double2 *vdst, int lane) {
    if (rr >= 0 && rr < n) {
        const T *row = L + (size_t)rr * W;
        for (int o = lane; o < W; o += 32) cp_async_elem<T>(slot + o, row + o);
        if (lane == 0 && vsrc) cp_async16(vdst, vsrc);
    }
    cp_commit();
}

// the same with a vector entry of type T (the back sweep's entering y values)
template <typename T>
__device__ __forceinline__ void ring_issue_v(const T *L, int W, int rr, int n, T *slot, const T *vsrc, T *vdst,
                                             int lane) {
    if (rr >= 0 && rr < n) {
        const T *row = L + (size_t)rr * W;
        for (int o = lane; o < W; o += 32) cp_async_elem<T>(slot + o, row + o);
        if (lane == 0 && vsrc) cp_async_elem<T>(vdst, vsrc);
    }
    cp_commit();
}

// Row-oriented forward substitution y = L^{-1} rin:
//   y_i = (rin_i - sum_{j=i-mb}^{i-1} L(i,j) y_j) / L(i,i)
// rows stream through a ring of kRing slots; the last W values of y sit in
// a shared-memory window (y_j in slot j mod W, tracked incrementally).
// Items whose active flag is 0 are skipped.
template <typename T>
__global__ __launch_bounds__(kSolveWarps * 32) void k_fwd(DevProblem P, DevBatch B, int nrhs,
                                                           const double2 *__restrict__ rin) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int n = P.n, mb = P.mb, W = mb + 1;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    unsigned char *base = sm_raw + (size_t)wl * solve_smem_per_warp<T>(W);
    double2 *rv = (double2 *)base;                       // [kRing]
    T *ring = (T *)(base + kRing * sizeof(double2));     // [kRing][W]
    T *pw = ring + (size_t)kRing * W;                    // [W]
    const int item = blockIdx.x * kSolveWarps + wl;
    if (item >= B.nsys * nrhs) return;
    if (B.active && !B.active[item]) return;
    const int s = item / nrhs;
    const T *L = (const T *)B.L + (size_t)s * n * W;
    const double2 *r = rin + (size_t)item * n;
    T *y = (T *)B.y + (size_t)item * n;
    for (int q = lane; q < W; q += 32) pw[q] = T{};
    for (int q = 0; q < kRing; q++) ring_issue<T>(L, W, q, n, ring + (size_t)q * W, r + q, rv + q, lane);
    int sb = 1;  // slot of column i - mb (== (i - mb) mod W); row i's slot is sb + mb - W or sb - 1
    int sl = 0;  // ring slot of row i
    for (int i = 0; i < n; i++) {
        const T *row = ring + (size_t)sl * W;
        cp_wait<kRing - 1>();
        __syncwarp();
        // read the diagonal and the right-hand side before any lane can
        // re-issue copies into this ring slot
        const T dg = row[mb];
        const double2 rhs = rv[sl];
        T acc{};
        const int o0 = i < mb ? mb - i : 0;
        for (int o = o0 + lane; o < mb; o += 32) {
            int sw = sb + o;
            if (sw >= W) sw -= W;
            acc = Ops<T>::fms(acc, row[o], pw[sw]);
        }
        acc = Ops<T>::reduce(acc);  // acc = -sum
        const int si = sb == 0 ? W - 1 : sb - 1;  // slot of row i == (i - mb - 1) mod W
        if (lane == 0) {
            const T v = Ops<T>::mul(Ops<T>::add(Ops<T>::from(rhs), acc), Ops<T>::rcp(dg));
            pw[si] = v;
            y[i] = v;
        }
        ring_issue<T>(L, W, i + kRing, n, ring + (size_t)sl * W, i + kRing < n ? r + i + kRing : nullptr,
                      rv + sl, lane);
        sb = sb + 1 == W ? 0 : sb + 1;
        sl = sl + 1 == kRing ? 0 : sl + 1;
    }
    cp_wait<0>();
}

// Backward substitution L^T x = y in place (y -> x), the column sweep of
// src/vre.f90:58-69: x_i = w_i / L(i,i); w_j -= L(i,j) x_i for j < i.
template <typename T>
__global__ __launch_bounds__(kSolveWarps * 32) void k_bwd(DevProblem P, DevBatch B, int nrhs) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int n = P.n, mb = P.mb, W = mb + 1;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    unsigned char *base = sm_raw + (size_t)wl * solve_smem_per_warp<T>(W);
    double2 *rv = (double2 *)base;  // entering entries y[i - W], as raw bytes of T
    T *ring = (T *)(base + kRing * sizeof(double2));
    T *pw = ring + (size_t)kRing * W;
    const int item = blockIdx.x * kSolveWarps + wl;
    if (item >= B.nsys * nrhs) return;
    if (B.active && !B.active[item]) return;
    const int s = item / nrhs;
    const T *L = (const T *)B.L + (size_t)s * n * W;
    T *y = (T *)B.y + (size_t)item * n;
    // window slot of entry j is j mod W
    const int j0 = n - W < 0 ? 0 : n - W;
    for (int q = j0 + lane; q < n; q += 32) pw[q % W] = y[q];
    for (int q = 0; q < kRing; q++) {
        const int rr = n - 1 - q;
        ring_issue_v<T>(L, W, rr, n, ring + (size_t)q * W, rr - W >= 0 ? y + (rr - W) : nullptr, (T *)(rv + q), lane);
    }
    int si = (n - 1) % W;            // slot of row i
    int sb = si + 1 == W ? 0 : si + 1;  // slot of column i - mb (== (i + 1) mod W)
    int sl = 0;
    for (int i = n - 1; i >= 0; i--) {
        const T *row = ring + (size_t)sl * W;
        cp_wait<kRing - 1>();
        __syncwarp();
        T v{};
        if (lane == 0) {
            v = Ops<T>::mul(pw[si], Ops<T>::rcp(row[mb]));
            y[i] = v;
        }
        v = Ops<T>::shfl(v, 0);
        const int o0 = i < mb ? mb - i : 0;
        for (int o = o0 + lane; o < mb; o += 32) {
            int sw = sb + o;
            if (sw >= W) sw -= W;
            pw[sw] = Ops<T>::fms(pw[sw], row[o], v);
        }
        if (lane == 0 && i - W >= 0) pw[si] = *(const T *)(rv + sl);
        const int rr = i - kRing;
        ring_issue_v<T>(L, W, rr, n, ring + (size_t)sl * W, rr - W >= 0 ? y + (rr - W) : nullptr, (T *)(rv + sl),
                        lane);
        si = si == 0 ? W - 1 : si - 1;
        sb = sb == 0 ? W - 1 : sb - 1;
        sl = sl + 1 == kRing ? 0 : sl + 1;
    }
    cp_wait<0>();
}

template <typename T>
static void set_solve_smem(int W) {
    static int done_w = -1;
    if (done_w == W) return;
    size_t bytes = kSolveWarps * solve_smem_per_warp<T>(W);
    cudaFuncSetAttribute(k_fwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    cudaFuncSetAttribute(k_bwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    done_w = W;
}

void launch_forward_solve(const DevProblem &P, const DevBatch &B, int nrhs, bool mixed, const double2 *rin,
                          cudaStream_t st) {
    int nitems = B.nsys * nrhs;
    int grid = (nitems + kSolveWarps - 1) / kSolveWarps;
    int W = P.mb + 1;
    if (mixed) {
        set_solve_smem<float2>(W);
        k_fwd<float2><<<grid, kSolveWarps * 32, kSolveWarps * solve_smem_per_warp<float2>(W), st>>>(P, B, nrhs, rin);
    } else {
        set_solve_smem<double2>(W);
        k_fwd<double2><<<grid, kSolveWarps * 32, kSolveWarps * solve_smem_per_warp<double2>(W), st>>>(P, B, nrhs, rin);
    }
}

void launch_back_solve(const DevProblem &P, const DevBatch &B, int nrhs, bool mixed, cudaStream_t st) {
    int nitems = B.nsys * nrhs;
    int grid = (nitems + kSolveWarps - 1) / kSolveWarps;
    int W = P.mb + 1;
    if (mixed) {
        set_solve_smem<float2>(W);
        k_bwd<float2><<<grid, kSolveWarps * 32, kSolveWarps * solve_smem_per_warp<float2>(W), st>>>(P, B, nrhs);
    } else {
        set_solve_smem<double2>(W);
        k_bwd<double2><<<grid, kSolveWarps * 32, kSolveWarps * solve_smem_per_warp<double2>(W), st>>>(P, B, nrhs);
    }
}

// r = b - A x with the full symmetric pattern (FP64)
__global__ void k_residual(DevProblem P, DevBatch B, int nrhs) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t nitems = (size_t)B.nsys * nrhs;
    if (gid >= nitems * P.n) return;
    int item = (int)(gid / P.n), i = (int)(gid % P.n);
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

// kpot(j, l, k) = pot(j) * fak(j) with pot = -x (src/fem.f90:388-389)
__global__ void k_kpot(DevProblem P, DevBatch B, int nrhs, double2 *kpot) {
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
    kpot[((size_t)k * P.eanz + l) * P.n + i] = v;
}

void launch_kpot(const DevProblem &P, const DevBatch &B, int nrhs, double2 *kpot, cudaStream_t st) {
    size_t tot = (size_t)B.nsys * nrhs * P.n;
    int nt = 256;
    k_kpot<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, B, nrhs, kpot);
}

}  // namespace crgpu
