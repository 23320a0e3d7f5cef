// Model update of the Gauss-Newton step: src/update.f90:27-353 with the
// complex preconditioned CG of src/cg_mod.f90:426-726 (cjggra, bap, bp,
// bptri, bb), or in the final phase improvement (lfpi) the real CG of
// src/cg_mod.f90:136-400 (cjggdc, bapdc, bpdc, bpdctri, bbdc) on Re(J) and the
// phases.  The Jacobian is column-major (nanz, manz): column j is
// contiguous, so the column reductions (preconditioner, right-hand side,
// J^H W (J p)) read coalesced columns, and J p is formed from column chunks
// with fixed-order partial sums (deterministic, no atomics).
#include <algorithm>
#include <cmath>
#include <vector>

#include "crgpu_internal.h"
#include "kernels.h"

namespace crgpu {

namespace {

constexpr int kRowTile = 256;   // rows of J per block in J p
constexpr int kColChunk = 64;   // columns of J per block in J p
constexpr int kRedThreads = 256;

// R v (optionally R (w o v)): structured 5-point stencil (ltri 0,
// src/cg_mod.f90:547-577 / src/update.f90:63-91) or the neighbour stencil
// (ltri 1, 2: src/cg_mod.f90:579-613 / src/update.f90:99-120)
__global__ void k_rmul(CGArgs a, const double2 *__restrict__ v, const double *__restrict__ w,
                       double2 *__restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int manz = a.manz;
    if (i >= manz) return;
    auto wv = [&](int j) -> double2 {
        double2 x = v[j];
        if (w) {
            double f = w[j];
            return cz(x.x * f, x.y * f);
        }
        return x;
    };
    double2 c = cz(0.0, 0.0);
    if (a.ltri == 0) {
        const double *sm1 = a.smatm, *sm2 = a.smatm + manz, *sm3 = a.smatm + 2 * (size_t)manz;
        const int nx = a.nx;
        if (i > 0) c = cscale(wv(i - 1), sm2[i - 1]);
        if (i < manz - 1) c = cadd(c, cscale(wv(i + 1), sm2[i]));
        if (i >= nx) c = cadd(c, cscale(wv(i - nx), sm3[i - nx]));
        if (i < manz - nx) c = cadd(c, cscale(wv(i + nx), sm3[i]));
        out[i] = cadd(c, cscale(wv(i), sm1[i]));
    } else {
        for (int q = 0; q < a.maxnk; q++) {
            int nb = a.nachbar[(size_t)q * manz + i];
            if (nb != 0) c = cadd(c, cscale(wv(nb - 1), a.smatm[(size_t)q * manz + i]));
        }
        out[i] = cadd(c, cscale(wv(i), a.smatm[(size_t)a.maxnk * manz + i]));
    }
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One block per column j: g_j = sum_i conj(s_ij) w_i vec_i and (mode 0)
// diag_j = sum_i |s_ij|^2 w_i (w_i = wmatd_i * wdfak_i).
// mode 0 (update.f90 RHS): cgfac_j = 1/sqrt(diag_j + lam R_jj),
//                          out_j = (g_j - lam rm_j) cgfac_j
// mode 1 (cg_mod.f90 bb):  out_j = (g_j + lam rm_j) cgfac_j
__global__ __launch_bounds__(kRedThreads) void k_colred(CGArgs a, int mode, const double2 *__restrict__ vec,
                                                        const double2 *rm, double *cgfac,
                                                        double2 *out) {  // out may alias rm
    const int j = blockIdx.x;
    const double2 *col = a.sens + (size_t)j * a.nanz;
    double gr = 0.0, gi = 0.0, dg = 0.0;
    for (int i = threadIdx.x; i < a.nanz; i += kRedThreads) {
        double2 s = col[i];
        if (a.part) s.y = 0.0;  // DBLE(sens) / sensdc of src/update.f90:182-192, 243-252
        const double w = a.wmatd[i] * (double)a.wdfak[i];
        if (mode == 0) dg = fma(s.x * s.x + s.y * s.y, w, dg);
        const double2 v = vec[i];
        // conj(s) * (w v)
        const double vx = w * v.x, vy = w * v.y;
        gr = fma(s.x, vx, gr);
        gr = fma(s.y, vy, gr);
        gi = fma(s.x, vy, gi);
        gi = fma(-s.y, vx, gi);
    }
    __shared__ double red[3][kRedThreads / 32];
    gr = warp_sum(gr);
    gi = warp_sum(gi);
    dg = warp_sum(dg);
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][wl] = gr;
        red[1][wl] = gi;
        red[2][wl] = dg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        gr = gi = dg = 0.0;
        for (int q = 0; q < kRedThreads / 32; q++) {
            gr += red[0][q];
            gi += red[1][q];
            dg += red[2][q];
        }
        double cf;
        if (mode == 0) {
            const double diagR = a.ltri == 0 ? a.smatm[j] : a.smatm[(size_t)a.maxnk * a.manz + j];
            cf = 1.0 / sqrt(dg + a.lam * diagR);
            cgfac[j] = cf;
            out[j] = cz((gr - a.lam * rm[j].x) * cf, (gi - a.lam * rm[j].y) * cf);
        } else {
            cf = cgfac[j];
            out[j] = cz((gr + a.lam * rm[j].x) * cf, (gi + a.lam * rm[j].y) * cf);
        }
    }
}

// wv_i = w_i v_i (w_i = wmatd_i wdfak_i), once per CG step for k_colred_bb
__global__ void k_weight(CGArgs a, const double2 *__restrict__ v, double2 *__restrict__ wv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nanz) return;
    const double w = a.wmatd[i] * (double)a.wdfak[i];
    wv[i] = cz(w * v[i].x, w * v[i].y);
}

// k_colred mode 1 (src/cg_mod.f90 bb) on a weighted vector: four FP64 FMAs
// per element of J, the FP64 pipe's minimum for a complex product
//   out_j = (sum_i conj(s_ij) wv_i + lam rm_j) cgfac_j
__global__ __launch_bounds__(kRedThreads) void k_colred_bb(CGArgs a, const double2 *__restrict__ wv,
                                                           const double2 *rm, double2 *out) {  // out may alias rm
    const int j = blockIdx.x;
    const double2 *col = a.sens + (size_t)j * a.nanz;
    double gr = 0.0, gi = 0.0;
    for (int i = threadIdx.x; i < a.nanz; i += kRedThreads) {
        double2 s = col[i];
        if (a.part) s.y = 0.0;
        const double2 v = wv[i];
        gr = fma(s.x, v.x, gr);
        gr = fma(s.y, v.y, gr);
        gi = fma(s.x, v.y, gi);
        gi = fma(-s.y, v.x, gi);
    }
    __shared__ double red[2][kRedThreads / 32];
    gr = warp_sum(gr);
    gi = warp_sum(gi);
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][wl] = gr;
        red[1][wl] = gi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        gr = gi = 0.0;
        for (int q = 0; q < kRedThreads / 32; q++) {
            gr += red[0][q];
            gi += red[1][q];
        }
        const double cf = a.cgfac[j];
        out[j] = cz((gr + a.lam * rm[j].x) * cf, (gi + a.lam * rm[j].y) * cf);
    }
}

// partial[chunk][i] = sum_{j in chunk} s_ij (cgfac_j p_j)   (src/cg_mod.f90:520-545)
__global__ __launch_bounds__(kRowTile) void k_jp_partial(CGArgs a, const double2 *__restrict__ p,
                                                         double2 *__restrict__ partial) {
    __shared__ double2 q[kColChunk];
    const int i = blockIdx.x * kRowTile + threadIdx.x;
    const int j0 = blockIdx.y * kColChunk;
    const int j1 = min(j0 + kColChunk, a.manz);
    for (int t = threadIdx.x; t < j1 - j0; t += kRowTile) {
        double2 v = p[j0 + t];
        double f = a.cgfac[j0 + t];
        q[t] = cz(v.x * f, v.y * f);
    }
    __syncthreads();
    if (i >= a.nanz) return;
    double ar = 0.0, ai = 0.0;
    for (int j = j0; j < j1; j++) {
        double2 s = a.sens[(size_t)j * a.nanz + i];
        if (a.part) s.y = 0.0;  // bapdc, src/cg_mod.f90:222-230
        const double2 v = q[j - j0];
        ar = fma(s.x, v.x, ar);
        ar = fma(-s.y, v.y, ar);
        ai = fma(s.x, v.y, ai);
        ai = fma(s.y, v.x, ai);
    }
    partial[(size_t)blockIdx.y * a.nanz + i] = cz(ar, ai);
}

__global__ void k_jp_reduce(CGArgs a, int nchunk, const double2 *__restrict__ partial, double2 *__restrict__ ap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nanz) return;
    double2 s = cz(0.0, 0.0);
    for (int c = 0; c < nchunk; c++) s = cadd(s, partial[(size_t)c * a.nanz + i]);
    ap[i] = s;
}

// block partial sums of Re(conj(x) y) (x == y: |x|^2), then a second pass
__global__ __launch_bounds__(kRedThreads) void k_dot_partial(int n, const double2 *__restrict__ x,
                                                             const double2 *__restrict__ y, double *part) {
    double s = 0.0;
    for (int i = blockIdx.x * kRedThreads + threadIdx.x; i < n; i += gridDim.x * kRedThreads) {
        double2 a = x[i], b = y[i];
        s = fma(a.x, b.x, s);
        s = fma(a.y, b.y, s);
    }
    __shared__ double red[kRedThreads / 32];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < kRedThreads / 32; q++) t += red[q];
        part[blockIdx.x] = t;
    }
}

__global__ void k_dot_final(int nb, const double *part, double *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < nb; q++) t += part[q];
        *out = t;
    }
}

// x = y + c z   (elementwise, complex with real c)
__global__ void k_axpy(int n, double2 *x, const double2 *y, double c, const double2 *z) {  // x may alias y or z
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 a = y[i], b = z[i];
    x[i] = cz(a.x + c * b.x, a.y + c * b.y);
}

// d = (y - f) for the right-hand side, dpar = 0, ...
__global__ void k_sub(int n, const double2 *__restrict__ a, const double2 *__restrict__ b, double2 *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = csub(a[i], b[i]);
}

// the real CG runs on Im(bvec) (part 1) or Re(bvec) (part 2) (cjggdc,
// src/cg_mod.f90:160-164)
__global__ void k_take_part(int n, double2 *v, int part) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v[i] = cz(part == 1 ? v[i].y : v[i].x, 0.0);
}

// dpar = cgfac o dpar (part 1: i Re(dpar), src/update.f90:299-302; part 2:
// Re(dpar)), par += step dpar
__global__ void k_final(int n, double2 *dpar, const double *__restrict__ cgfac, double step, double2 *par,
                        int part) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 d = dpar[i];
    double f = cgfac[i];
    d = part == 1 ? cz(0.0, d.x * f) : part == 2 ? cz(d.x * f, 0.0) : cz(d.x * f, d.y * f);
    dpar[i] = d;
    double2 p = par[i];
    par[i] = cz(p.x + step * d.x, p.y + step * d.y);
}

inline unsigned nblk(int n, int t) { return (unsigned)((n + t - 1) / t); }

__global__ void k_fill_one(int n, double2 *v, double *f) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    v[i] = cz(1.0, 0.0);
    f[i] = 1.0;
}

__global__ void k_abs(int n, const double2 *__restrict__ v, double *out) {  // out may not alias v
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = hypot(v[i].x, v[i].y);
}

}  // namespace

// work layout (double2 units): bvec, rvec, pvec, dpar(out) | ap, dmf (nanz) |
// partial (nchunk * nanz) | scalars
size_t update_work_bytes(int nanz, int manz) {
    int nchunk = (manz + kColChunk - 1) / kColChunk;
    return sizeof(double2) * ((size_t)3 * manz + 2 * (size_t)nanz + (size_t)nchunk * nanz) + sizeof(double) * 1024;
}

int run_update(const CGArgs &a, cudaStream_t st, int *ncg_out, float *cgres_host) {
    const int manz = a.manz, nanz = a.nanz;
    const int nchunk = (manz + kColChunk - 1) / kColChunk;
    double2 *bvec = a.work, *rvec = bvec + manz, *pvec = rvec + manz;
    double2 *ap = pvec + manz, *dmf = ap + nanz, *partial = dmf + nanz;
    double *scal = (double *)(partial + (size_t)nchunk * nanz);
    double *dots = scal;          // [0]: result
    double *dpart = scal + 8;     // block partials
    const int nbm = 120;
    auto dot = [&](const double2 *x, const double2 *y) -> double {
        k_dot_partial<<<nbm, kRedThreads, 0, st>>>(manz, x, y, dpart);
        k_dot_final<<<1, 32, 0, st>>>(nbm, dpart, dots);
        double h = 0.0;
        cudaMemcpyAsync(&h, dots, sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        return h;
    };
    const int T = 256;
    // bvec = R m ; right-hand side and preconditioner
    k_rmul<<<nblk(manz, T), T, 0, st>>>(a, a.par, nullptr, bvec);
    k_sub<<<nblk(nanz, T), T, 0, st>>>(nanz, a.dat, a.sigmaa, dmf);
    k_colred<<<manz, kRedThreads, 0, st>>>(a, 0, dmf, bvec, a.cgfac, bvec);
    if (a.part) k_take_part<<<nblk(manz, T), T, 0, st>>>(manz, bvec, a.part);
    // cjggra (complex) or cjggdc (parts 1, 2: the same recursion on real vectors)
    cudaMemsetAsync(a.dpar, 0, sizeof(double2) * manz, st);
    cudaMemcpyAsync(rvec, bvec, sizeof(double2) * manz, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(pvec, 0, sizeof(double2) * manz, st);
    std::vector<float> cgres(a.ncgmax + 2, 0.f);
    double dr = 0, dr0 = 0, dr1 = 0, beta = 0;
    int ncg = a.ncgmax, k;
    for (k = 1; k <= a.ncgmax; k++) {
        ncg = k - 1;
        dr = dot(rvec, rvec);
        if (k == 1) {
            dr0 = dr * a.eps;
            beta = 0.0;
            if (a.part && dr <= dr0) break;  // cjggdc tests the first step too
        } else {
            if (dr <= dr0) break;
            beta = dr / dr1;
        }
        k_axpy<<<nblk(manz, T), T, 0, st>>>(manz, pvec, rvec, beta, pvec);
        dim3 g1(nblk(nanz, kRowTile), nchunk);
        k_jp_partial<<<g1, kRowTile, 0, st>>>(a, pvec, partial);
        k_jp_reduce<<<nblk(nanz, T), T, 0, st>>>(a, nchunk, partial, ap);
        k_rmul<<<nblk(manz, T), T, 0, st>>>(a, pvec, a.cgfac, bvec);
        k_weight<<<nblk(nanz, T), T, 0, st>>>(a, ap, dmf);  // d - f is not needed after the right-hand side
        k_colred_bb<<<manz, kRedThreads, 0, st>>>(a, dmf, bvec, bvec);
        dr1 = dot(pvec, bvec);
        const double alpha = dr / dr1;
        k_axpy<<<nblk(manz, T), T, 0, st>>>(manz, a.dpar, a.dpar, alpha, pvec);
        k_axpy<<<nblk(manz, T), T, 0, st>>>(manz, rvec, rvec, -alpha, bvec);
        dr1 = dr;
        cgres[k] = (float)(a.eps * dr / dr0);
    }
    if (k > a.ncgmax) ncg = a.ncgmax;
    cgres[0] = (float)ncg;
    k_final<<<nblk(manz, T), T, 0, st>>>(manz, a.dpar, a.cgfac, a.step, a.par, a.part);
    for (size_t q = 0; q < cgres.size(); q++) cgres_host[q] = cgres[q];
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    *ncg_out = ncg;
    return e == cudaSuccess ? 0 : ERR_CUDA;
}

// |(J^H W J 1)_j| of src/blam0.f90:60-130 (phase only: Re(J)): the double
// sum over data and model cells as two products with J.  Reads a.sens,
// a.wmatd, a.wdfak and the work space; a.smatm, a.nachbar, a.par, a.dpar,
// a.dat and a.sigmaa are not used (k_colred reads smatm in mode 0 only).
int run_jhwj1(CGArgs a, cudaStream_t st, double *jtj_host) {
    const int manz = a.manz, nanz = a.nanz;
    const int nchunk = (manz + kColChunk - 1) / kColChunk;
    double2 *bvec = a.work, *ones = bvec + manz, *pvec = ones + manz;
    double2 *ap = pvec + manz, *dmf = ap + nanz, *partial = dmf + nanz;
    (void)dmf;
    const int T = 256;
    k_fill_one<<<nblk(manz, T), T, 0, st>>>(manz, ones, a.cgfac);
    cudaMemsetAsync(bvec, 0, sizeof(double2) * manz, st);
    dim3 g1(nblk(nanz, kRowTile), nchunk);
    k_jp_partial<<<g1, kRowTile, 0, st>>>(a, ones, partial);
    k_jp_reduce<<<nblk(nanz, T), T, 0, st>>>(a, nchunk, partial, ap);
    a.lam = 0.0;
    k_colred<<<manz, kRedThreads, 0, st>>>(a, 1, ap, bvec, a.cgfac, pvec);
    k_abs<<<nblk(manz, T), T, 0, st>>>(manz, pvec, (double *)bvec);
    cudaMemcpyAsync(jtj_host, bvec, sizeof(double) * manz, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? 0 : ERR_CUDA;
}

}  // namespace crgpu
