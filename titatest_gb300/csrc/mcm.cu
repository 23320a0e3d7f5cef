// Model uncertainty and resolution (src/bmcm_mod.f90: buncert, bata,
// bata_reg, bmcm, bres, bmcm2) and the coverage sums (src/bbsens.f90) on the
// sensitivities held on the device.
//
//   ata     = Re(J^H W J) = S^T S               (bata; S = [sqrt(w) Re J; sqrt(w) Im J])
//   ata_reg = ata + lam R                       (bata_reg)
//   cov     = ata_reg^-1 = L^-T L^-1            (bmcm: blocked Cholesky, triangular inverse, Y^T Y)
//   res     = cov ata          -> diag          (bres: row-column dots, O(manz^2))
//   cov2    = cov ata cov      -> diag          (bmcm2: = (S cov)^T (S cov), column sums of squares)
//
// The dense steps are this library's own FP64 kernels (dense.cu); the kernels
// here form the weighted operand, the regularisation entries and the
// diagonals.
#include <algorithm>
#include <string>

#include "kernels.h"

namespace crgpu {

namespace {

// A (2 nanz x manz, column-major): rows i = sqrt(w_i) Re J_ij, rows nanz + i
// = sqrt(w_i) Im J_ij (w_i = wmatd_i wdfak_i), so that A^T A = Re(J^H W J)
__global__ void k_weighted_split(int nanz, int manz, const double2 *__restrict__ sens,
                                 const double *__restrict__ wmatd, const int32_t *__restrict__ wdfak,
                                 double *__restrict__ A) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)nanz * manz) return;
    const int j = (int)(idx / nanz), i = (int)(idx % nanz);
    const double sw = sqrt(wmatd[i] * (double)wdfak[i]);
    const double2 s = sens[idx];
    A[(size_t)j * 2 * nanz + i] = sw * s.x;
    A[(size_t)j * 2 * nanz + nanz + i] = sw * s.y;
}

// upper triangle from the lower one (column-major n x n)
__global__ void k_symmetrize_lower(int n, double *M) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n * n) return;
    const int c = (int)(idx / n), r = (int)(idx % n);
    if (r < c) M[(size_t)c * n + r] = M[(size_t)r * n + c];
}

__global__ void k_diag(int n, const double *__restrict__ M, double *__restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = M[(size_t)i * n + i];
}

// ata_reg = ata + lam R for the neighbour regularisation (ltri 1, 2),
// src/bmcm_mod.f90:357-370 in its order: column by column, the diagonal,
// then the first nachbar(j, nk+1) neighbour slots (a neighbour in a later
// slot is not reached, as in the reference), each write mirrored.  One
// thread: the later column's write of a mirrored pair must win.
__global__ void k_reg_neighbours(int manz, int nk, double lam, const double *__restrict__ smatm,
                                 const int32_t *__restrict__ nachbar, const double *__restrict__ ata,
                                 double *__restrict__ reg) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int j = 0; j < manz; j++) {
        reg[(size_t)j * manz + j] = ata[(size_t)j * manz + j] + lam * smatm[(size_t)nk * manz + j];
        const int cnt = nachbar[(size_t)nk * manz + j];
        for (int k = 0; k < cnt && k < nk; k++) {
            const int ik = nachbar[(size_t)k * manz + j];
            if (ik == 0) continue;
            const double v = ata[(size_t)j * manz + (ik - 1)] + lam * smatm[(size_t)k * manz + j];
            reg[(size_t)j * manz + (ik - 1)] = v;
            reg[(size_t)(ik - 1) * manz + j] = v;
        }
    }
}

// ata_reg = ata + lam R for the structured 5-point regularisation (ltri 0):
// the stencil of src/update.f90:63-91 (smatm(:,1) diagonal, smatm(:,2) the
// x neighbour, smatm(:,3) the z neighbour), one thread per cell
__global__ void k_reg_stencil(int manz, int nx, double lam, const double *__restrict__ smatm, double *reg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= manz) return;
    reg[(size_t)i * manz + i] += lam * smatm[i];
    if (i + 1 < manz) {
        reg[(size_t)i * manz + i + 1] += lam * smatm[manz + i];
        reg[(size_t)(i + 1) * manz + i] += lam * smatm[manz + i];
    }
    if (i + nx < manz) {
        reg[(size_t)i * manz + i + nx] += lam * smatm[2 * (size_t)manz + i];
        reg[(size_t)(i + nx) * manz + i] += lam * smatm[2 * (size_t)manz + i];
    }
}

// d_i = sum_k X_ik Y_ki (column-major n x n): the diagonal of X Y
__global__ void k_diag_of_product(int n, const double *__restrict__ X, const double *__restrict__ Y, double *d) {
    const int i = blockIdx.x;
    double s = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) s = fma(X[(size_t)k * n + i], Y[(size_t)i * n + k], s);
    __shared__ double red[256 / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q];
        d[i] = t;
    }
}

// column sums of src/bbsens.f90 and the FPI diagonal of src/bmcm_mod.f90
// bata: c1_j = sum_i |J_ij| wa_i, c2_j = sum_i |Re J_ij| wb_i,
// c3_j = sum_i Re(J_ij)^2 wc_i (the weights already carry wdfak)
__global__ void k_column_sums(int nanz, const double2 *__restrict__ sens, const double *__restrict__ wa,
                              const double *__restrict__ wb, const double *__restrict__ wc, double *c1,
                              double *c2, double *c3) {
    const int j = blockIdx.x;
    const double2 *col = sens + (size_t)j * nanz;
    double s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int i = threadIdx.x; i < nanz; i += blockDim.x) {
        const double2 v = col[i];
        s1 = fma(hypot(v.x, v.y), wa[i], s1);
        s2 = fma(fabs(v.x), wb[i], s2);
        s3 = fma(v.x * v.x, wc[i], s3);
    }
    __shared__ double red[3][256 / 32];
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        s3 += __shfl_xor_sync(0xffffffffu, s3, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s1;
        red[1][threadIdx.x >> 5] = s2;
        red[2][threadIdx.x >> 5] = s3;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t1 = 0.0, t2 = 0.0, t3 = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
            t1 += red[0][q];
            t2 += red[1][q];
            t3 += red[2][q];
        }
        c1[j] = t1;
        c2[j] = t2;
        c3[j] = t3;
    }
}

inline unsigned nb(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void launch_column_sums(int nanz, int manz, const double2 *sens, const double *wa, const double *wb,
                        const double *wc, double *c1, double *c2, double *c3, cudaStream_t st) {
    if (manz > 0) k_column_sums<<<manz, 256, 0, st>>>(nanz, sens, wa, wb, wc, c1, c2, c3);
}

int run_mcm(const McmArgs &a, cudaStream_t st, std::string &msg) {
    const int n = a.manz, m = a.nanz;
    const size_t nn = (size_t)n * n;
    double *A = nullptr, *ata = nullptr, *reg = nullptr, *Y = nullptr, *cov = nullptr, *d = nullptr, *work = nullptr;
    int *info = nullptr;
    int rc = 0;
    auto fail = [&](int code, const std::string &what) {
        if (!rc) {
            rc = code;
            msg = what;
        }
    };
    auto dal = [&](void **p, size_t bytes) {
        if (!rc && cudaMallocAsync(p, bytes, st) != cudaSuccess) fail(97, "uncertainty work space");
    };
    dal((void **)&A, sizeof(double) * 2 * (size_t)m * n);
    dal((void **)&ata, sizeof(double) * nn);
    dal((void **)&reg, sizeof(double) * nn);
    dal((void **)&d, sizeof(double) * n);
    dal((void **)&info, sizeof(int));
    const int T = 256;
    if (!rc) {
        // bata: ata = S^T S (lower), S the weighted split of J
        k_weighted_split<<<nb((size_t)m * n, T), T, 0, st>>>(m, n, a.sens, a.wmatd, a.wdfak, A);
        dense_syrk_t(n, 2 * m, A, 2 * m, ata, st);
        k_symmetrize_lower<<<nb(nn, T), T, 0, st>>>(n, ata);
        k_diag<<<nb(n, T), T, 0, st>>>(n, ata, d);
        cudaMemcpyAsync(a.diag_ata, d, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        // bata_reg
        cudaMemcpyAsync(reg, ata, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st);
        if (a.ltri == 0)
            k_reg_stencil<<<nb(n, T), T, 0, st>>>(n, a.nx, a.lam, a.smatm, reg);
        else
            k_reg_neighbours<<<1, 1, 0, st>>>(n, a.nk, a.lam, a.smatm, a.nachbar, ata, reg);
        k_diag<<<nb(n, T), T, 0, st>>>(n, reg, d);
        cudaMemcpyAsync(a.diag_reg, d, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        // bmcm: Cholesky factor L of ata_reg (in place, lower)
        cudaMemsetAsync(info, 0, sizeof(int), st);
        dense_potrf(n, reg, info, st);
        int h_info = 0;
        cudaMemcpyAsync(&h_info, info, sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        if (h_info != 0) fail(108, "CHOLD mcm :: matrix not pos definite..");  // src/bmcm_mod.f90:447-451
    }
    dal((void **)&Y, sizeof(double) * nn);
    dal((void **)&cov, sizeof(double) * nn);
    if (!rc) {
        // cov = L^-T L^-1 (lower), then both triangles
        dense_potri(n, reg, Y, cov, st);
        k_symmetrize_lower<<<nb(nn, T), T, 0, st>>>(n, cov);
        k_diag<<<nb(n, T), T, 0, st>>>(n, cov, d);
        cudaMemcpyAsync(a.diag_cov1, d, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        if (a.want_res) {  // bres: diag(cov ata)
            k_diag_of_product<<<n, 256, 0, st>>>(n, cov, ata, d);
            cudaMemcpyAsync(a.diag_res, d, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        }
    }
    if (!rc && a.want_res && a.want_cov2) {  // bmcm2: diag(cov ata cov) = column sums of (S cov)^2
        dal((void **)&work, sizeof(double) * (size_t)((2 * m + 63) / 64) * n);
        if (!rc) {
            dense_col_sq_of_product(2 * m, n, A, 2 * m, cov, work, d, st);
            cudaMemcpyAsync(a.diag_cov2, d, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        }
    }
    cudaError_t ce = cudaStreamSynchronize(st);
    if (!rc && ce != cudaSuccess) fail(1000, cudaGetErrorString(ce));
    ce = cudaGetLastError();
    if (!rc && ce != cudaSuccess) fail(1000, cudaGetErrorString(ce));
    for (void *p : {(void *)A, (void *)ata, (void *)reg, (void *)Y, (void *)cov, (void *)d, (void *)work,
                    (void *)info})
        if (p) cudaFreeAsync(p, st);
    return rc;
}

}  // namespace crgpu
