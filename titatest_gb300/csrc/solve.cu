// Band triangular solves (src/vre.f90:5-71), FP64 iterative refinement of the
// mixed mode, and the unscaling into kpot (src/fem.f90:383-394).
//
// One warp solves one right-hand side.  Both sweeps keep a W = mb+1 window of
// the working vector in shared memory (entry i in slot i mod W):
//   forward  L y = b : column j of L is gathered from the rows j+1..j+mb
//                      (addresses step by mb; the same sectors serve the next
//                      three columns, so L1 absorbs the gather);
//   backward L^T x = y: row i of L is read contiguously (the vre update
//                      pot(j) += a(i,j) * pot(i)).
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
};
template <>
struct Ops<float2> {
    __device__ static float2 div(float2 a, float2 b) { return cdivf(a, b); }
    __device__ static float2 fms(float2 s, float2 a, float2 b) { return cfmsf(s, a, b); }
    __device__ static float2 from(double2 a) { return to_f(a); }
    __device__ static float2 shfl(float2 a, int src) {
        return cf(__shfl_sync(0xffffffffu, a.x, src), __shfl_sync(0xffffffffu, a.y, src));
    }
};

constexpr int kSolveWarps = 4;

// y = L^{-1} rin (rin FP64, converted to T); items whose active flag is 0 are skipped
template <typename T>
__global__ __launch_bounds__(kSolveWarps * 32) void k_fwd(DevProblem P, DevBatch B, int nrhs,
                                                           const double2 *__restrict__ rin) {
    extern __shared__ unsigned char sm_raw[];
    const int n = P.n, mb = P.mb, W = mb + 1;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    T *pw = (T *)sm_raw + (size_t)wl * W;
    int item = blockIdx.x * kSolveWarps + wl;
    int nitems = B.nsys * nrhs;
    if (item >= nitems) return;
    if (B.active && !B.active[item]) return;
    int s = item / nrhs;
    const T *L = (const T *)B.L + (size_t)s * n * W;
    const double2 *r = rin + (size_t)item * n;
    T *y = (T *)B.y + (size_t)item * n;
    for (int q = lane; q < W; q += 32) pw[q] = (q < n) ? Ops<T>::from(r[q]) : T{};
    __syncwarp();
    for (int j = 0; j < n; j++) {
        T v{};
        if (lane == 0) {
            v = Ops<T>::div(pw[j % W], L[(size_t)j * W + mb]);
            y[j] = v;
        }
        v = Ops<T>::shfl(v, 0);
        const int R = min(mb, n - 1 - j);
        for (int o = lane; o < R; o += 32) {
            int rr = j + 1 + o;
            int sl = rr % W;
            pw[sl] = Ops<T>::fms(pw[sl], L[(size_t)rr * W + (mb - 1 - o)], v);
        }
        __syncwarp();
        if (lane == 0 && j + W < n) pw[j % W] = Ops<T>::from(r[j + W]);
        __syncwarp();
    }
}

// x = L^{-T} y in place (y -> x); items whose active flag is 0 are skipped
template <typename T>
__global__ __launch_bounds__(kSolveWarps * 32) void k_bwd(DevProblem P, DevBatch B, int nrhs) {
    extern __shared__ unsigned char sm_raw[];
    const int n = P.n, mb = P.mb, W = mb + 1;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    T *pw = (T *)sm_raw + (size_t)wl * W;
    int item = blockIdx.x * kSolveWarps + wl;
    int nitems = B.nsys * nrhs;
    if (item >= nitems) return;
    if (B.active && !B.active[item]) return;
    int s = item / nrhs;
    const T *L = (const T *)B.L + (size_t)s * n * W;
    T *y = (T *)B.y + (size_t)item * n;
    int j0 = n - W < 0 ? 0 : n - W;
    for (int q = j0 + lane; q < n; q += 32) pw[q % W] = y[q];
    __syncwarp();
    for (int i = n - 1; i >= 0; i--) {
        const T *row = L + (size_t)i * W;
        T v{};
        if (lane == 0) {
            v = Ops<T>::div(pw[i % W], row[mb]);
            y[i] = v;
        }
        v = Ops<T>::shfl(v, 0);
        int o0 = mb - i;  // first offset with column >= 0
        if (o0 < 0) o0 = 0;
        for (int o = o0 + lane; o < mb; o += 32) {
            int jj = i - mb + o;
            int sl = jj % W;
            pw[sl] = Ops<T>::fms(pw[sl], row[o], v);
        }
        __syncwarp();
        if (lane == 0 && i - W >= 0) pw[i % W] = y[i - W];
        __syncwarp();
    }
}

void launch_forward_solve(const DevProblem &P, const DevBatch &B, int nrhs, bool mixed, const double2 *rin,
                          cudaStream_t st) {
    int nitems = B.nsys * nrhs;
    int grid = (nitems + kSolveWarps - 1) / kSolveWarps;
    size_t W = P.mb + 1;
    if (mixed) k_fwd<float2><<<grid, kSolveWarps * 32, kSolveWarps * W * sizeof(float2), st>>>(P, B, nrhs, rin);
    else k_fwd<double2><<<grid, kSolveWarps * 32, kSolveWarps * W * sizeof(double2), st>>>(P, B, nrhs, rin);
}

void launch_back_solve(const DevProblem &P, const DevBatch &B, int nrhs, bool mixed, cudaStream_t st) {
    int nitems = B.nsys * nrhs;
    int grid = (nitems + kSolveWarps - 1) / kSolveWarps;
    size_t W = P.mb + 1;
    if (mixed) k_bwd<float2><<<grid, kSolveWarps * 32, kSolveWarps * W * sizeof(float2), st>>>(P, B, nrhs);
    else k_bwd<double2><<<grid, kSolveWarps * 32, kSolveWarps * W * sizeof(double2), st>>>(P, B, nrhs);
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
    kpot[((size_t)k * P.eanz + l) * P.n + i] = cz(-x.x * f, -x.y * f);
}

void launch_kpot(const DevProblem &P, const DevBatch &B, int nrhs, double2 *kpot, cudaStream_t st) {
    size_t tot = (size_t)B.nsys * nrhs * P.n;
    int nt = 256;
    k_kpot<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, B, nrhs, kpot);
}

}  // namespace crgpu
