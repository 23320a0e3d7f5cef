// Dense FP64 kernels for the model uncertainty and resolution of
// src/bmcm_mod.f90 (bata, bmcm, bres, bmcm2): a tiled matrix product, and the
// blocked Cholesky factor, triangular inverse and inverse product that
// replace DPOTRF / DPOTRI.  All matrices are column-major with leading
// dimension ld; blocks are kNB = 64 wide.
//
// On GB300 these run on the FP64 pipe (a small fraction of the FP32 rate):
// each thread of a 256-thread block accumulates a 4x4 tile of the 64x64
// output block in registers from 16-deep slices of the operands staged in
// shared memory, which is far more data reuse than the FP64 pipe needs.
#include <algorithm>
#include <mutex>

#include "kernels.h"

namespace crgpu {

namespace {

constexpr int kNB = 64;   // block size of the tiles and of the blocked factorisations
constexpr int kBK = 16;   // depth of a staged operand slice
constexpr int kGT = 256;  // threads of a product block

// Operand access: element (row i of the product, depth k).  kmaj: the depth
// index is contiguous (A^T of a column-major matrix, stored A(k, i) at
// i*ld + k); otherwise the row index is (A(i, k) at k*ld + i).
template <bool KMAJ>
__device__ __forceinline__ double opnd(const double *__restrict__ A, int ld, int i, int k) {
    return KMAJ ? A[(size_t)i * ld + k] : A[(size_t)k * ld + i];
}

// C(i, j) = alpha * sum_k A(i, k) B(j, k) + beta * C(i, j) for the 64x64
// output block (blockIdx.x, blockIdx.y) of an M x N product, depth K.
// lower: only blocks on or below the diagonal; tri_k: the depth starts at the
// block row's first index (operands lower triangular in k, as Y^T Y with Y
// lower).  partial_sq: instead of storing C, store the sums over each 64-row
// block of the squared entries, sq[(bi) * N + j] (the diagonal of G^T G).
template <bool AK, bool BK>
__global__ __launch_bounds__(kGT) void k_gemm(int M, int N, int K, double alpha, const double *__restrict__ A, int lda,
                                              const double *__restrict__ B, int ldb, double beta, double *C, int ldc,
                                              int lower, int tri_k, double *sq) {
    const int bi = blockIdx.x, bj = blockIdx.y;
    if (lower && bi < bj) return;
    __shared__ double As[kBK][kNB + 1], Bs[kBK][kNB + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = bi * kNB, j0 = bj * kNB;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
    const int kbeg = tri_k ? max(i0, j0) : 0;
    for (int k0 = kbeg; k0 < K; k0 += kBK) {
        // stage the 64 x 16 slices: 1024 values of each operand, 4 per thread
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = tid + q * kGT;
            // depth-contiguous operands load along k, the others along the row index
            const int r = AK ? e >> 4 : e & 63, kk = AK ? e & 15 : e >> 6;
            const int gi = i0 + r, gk = k0 + kk;
            As[kk][r] = (gi < M && gk < K) ? opnd<AK>(A, lda, gi, gk) : 0.0;
            const int r2 = BK ? e >> 4 : e & 63, kk2 = BK ? e & 15 : e >> 6;
            const int gj = j0 + r2, gk2 = k0 + kk2;
            Bs[kk2][r2] = (gj < N && gk2 < K) ? opnd<BK>(B, ldb, gj, gk2) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; kk++) {
            double av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; a++) av[a] = As[kk][ty + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; b++) bv[b] = Bs[kk][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
        }
        __syncthreads();
    }
    if (sq) {  // column sums of squares of this row block, in a fixed order
        __shared__ double red[16][kNB];
#pragma unroll
        for (int b = 0; b < 4; b++) {
            double s = 0.0;
#pragma unroll
            for (int a = 0; a < 4; a++)
                if (i0 + ty + 16 * a < M) s = fma(acc[a][b], acc[a][b], s);
            red[ty][tx + 16 * b] = s;
        }
        __syncthreads();
        if (tid < kNB && j0 + tid < N) {
            double s = 0.0;
            for (int q = 0; q < 16; q++) s += red[q][tid];
            sq[(size_t)bi * N + j0 + tid] = s;
        }
        return;
    }
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const int i = i0 + ty + 16 * a;
        if (i >= M) continue;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int j = j0 + tx + 16 * b;
            if (j >= N || (lower && i < j)) continue;
            double *c = C + (size_t)j * ldc + i;
            *c = alpha * acc[a][b] + (beta == 0.0 ? 0.0 : beta * *c);
        }
    }
}

// Cholesky factor of the diagonal block at (c0, c0), nb x nb (nb <= 64), in
// shared memory: right-looking, one column per step.  info: first column
// (1-based) whose pivot is not positive.
__global__ __launch_bounds__(256) void k_potf2(int n, double *A, int lda, int c0, int *info) {
    const int nb = min(kNB, n - c0);
    __shared__ double S[kNB][kNB + 1];
    __shared__ double dsq;
    __shared__ int bad;
    const int tid = threadIdx.x;
    if (tid == 0) bad = 0;
    for (int e = tid; e < nb * nb; e += blockDim.x) {
        const int r = e % nb, c = e / nb;
        S[r][c] = r >= c ? A[(size_t)(c0 + c) * lda + c0 + r] : 0.0;
    }
    __syncthreads();
    for (int c = 0; c < nb; c++) {
        if (tid == 0) {
            const double d = S[c][c];
            if (!(d > 0.0) && !bad) bad = c0 + c + 1;
            dsq = sqrt(d > 0.0 ? d : 1.0);
            S[c][c] = dsq;
        }
        __syncthreads();
        const double dinv = 1.0 / dsq;
        for (int r = c + 1 + tid; r < nb; r += blockDim.x) S[r][c] *= dinv;
        __syncthreads();
        const int m = nb - c - 1;
        for (int e = tid; e < m * m; e += blockDim.x) {
            const int r = c + 1 + e % m, q = c + 1 + e / m;
            if (r >= q) S[r][q] = fma(-S[r][c], S[q][c], S[r][q]);
        }
        __syncthreads();
    }
    for (int e = tid; e < nb * nb; e += blockDim.x) {
        const int r = e % nb, c = e / nb;
        if (r >= c) A[(size_t)(c0 + c) * lda + c0 + r] = S[r][c];
    }
    if (tid == 0 && bad && *info == 0) *info = bad;
}

// X = A21 L11^-T for the rows below the diagonal block c0 (blockIdx.x: a
// 64-row block of them), overwriting A21: each thread solves one row with the
// factor block in shared memory.
__global__ __launch_bounds__(kNB) void k_trsm_panel(int n, double *A, int lda, int c0) {
    const int nb = min(kNB, n - c0);
    extern __shared__ double dsm[];  // two kNB x (kNB+1) blocks (dynamic: above the 48 KB static limit)
    double(*Lb)[kNB + 1] = reinterpret_cast<double(*)[kNB + 1]>(dsm);
    double(*X)[kNB + 1] = Lb + kNB;
    const int tid = threadIdx.x;
    for (int e = tid; e < nb * nb; e += blockDim.x) {
        const int r = e % nb, c = e / nb;
        Lb[r][c] = A[(size_t)(c0 + c) * lda + c0 + r];
    }
    const int r0 = c0 + nb + blockIdx.x * kNB;
    const int nr = min(kNB, n - r0);
    for (int e = tid; e < nr * nb; e += blockDim.x) {
        const int r = e % nr, c = e / nr;
        X[r][c] = A[(size_t)(c0 + c) * lda + r0 + r];
    }
    __syncthreads();
    if (tid < nr) {
        for (int c = 0; c < nb; c++) {
            double s = X[tid][c];
            for (int p = 0; p < c; p++) s = fma(-X[tid][p], Lb[c][p], s);
            X[tid][c] = s / Lb[c][c];
        }
    }
    __syncthreads();
    for (int e = tid; e < nr * nb; e += blockDim.x) {
        const int r = e % nr, c = e / nr;
        A[(size_t)(c0 + c) * lda + r0 + r] = X[r][c];
    }
}

// Y_ii = L_ii^-1 for the diagonal block at (c0, c0) of the lower factor L,
// into Y (the same positions); then, for every block column j < i,
// Y_ij = -Y_ii acc_ij, where acc_ij (kept in Y_ij) holds sum_k L_ik Y_kj.
// blockIdx.x = 0: the diagonal block; blockIdx.x = 1 + j: block column j.
__global__ __launch_bounds__(256) void k_trtri_row(int n, const double *L, double *Y, int ld, int i) {
    const int c0 = i * kNB, nb = min(kNB, n - c0);
    extern __shared__ double dsm[];  // three kNB x (kNB+1) blocks
    double(*Li)[kNB + 1] = reinterpret_cast<double(*)[kNB + 1]>(dsm);
    double(*Yi)[kNB + 1] = Li + kNB;
    double(*T)[kNB + 1] = Yi + kNB;
    const int tid = threadIdx.x;
    for (int e = tid; e < nb * nb; e += blockDim.x) {
        const int r = e % nb, c = e / nb;
        Li[r][c] = r >= c ? L[(size_t)(c0 + c) * ld + c0 + r] : 0.0;
        Yi[r][c] = 0.0;
    }
    __syncthreads();
    // the inverse of the lower triangular block, column by column: thread c
    // solves Li y = e_c by forward substitution
    if (tid < nb) {
        const int c = tid;
        for (int r = c; r < nb; r++) {
            double s = r == c ? 1.0 : 0.0;
            for (int p = c; p < r; p++) s = fma(-Li[r][p], Yi[p][c], s);
            Yi[r][c] = s / Li[r][r];
        }
    }
    __syncthreads();
    if (blockIdx.x == 0) {
        for (int e = tid; e < nb * nb; e += blockDim.x) {
            const int r = e % nb, c = e / nb;
            Y[(size_t)(c0 + c) * ld + c0 + r] = r >= c ? Yi[r][c] : 0.0;
        }
        return;
    }
    const int j0 = (blockIdx.x - 1) * kNB;  // block column j < i (width kNB)
    for (int e = tid; e < nb * kNB; e += blockDim.x) {
        const int r = e % nb, c = e / nb;
        T[r][c] = Y[(size_t)(j0 + c) * ld + c0 + r];
    }
    __syncthreads();
    for (int e = tid; e < nb * kNB; e += blockDim.x) {
        const int r = e % nb, c = e / nb;
        double s = 0.0;
        for (int p = 0; p <= r; p++) s = fma(Yi[r][p], T[p][c], s);
        Y[(size_t)(j0 + c) * ld + c0 + r] = -s;
    }
}

// x = a (n doubles)
__global__ void k_fill(size_t n, double *x, double a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = a;
}

// d_j = sum over the row blocks of sq (nblk x n), in block order
__global__ void k_sum_blocks(int nblk, int n, const double *__restrict__ sq, double *__restrict__ d) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += sq[(size_t)b * n + j];
    d[j] = s;
}

inline int nblk(int n) { return (n + kNB - 1) / kNB; }

constexpr size_t kBlockBytes = sizeof(double) * kNB * (kNB + 1);

void set_dense_smem() {
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(k_trsm_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(2 * kBlockBytes));
        cudaFuncSetAttribute(k_trtri_row, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(3 * kBlockBytes));
    });
}

template <bool AK, bool BK>
void gemm(int M, int N, int K, double alpha, const double *A, int lda, const double *B, int ldb, double beta,
          double *C, int ldc, int lower, int tri_k, double *sq, cudaStream_t st) {
    if (M <= 0 || N <= 0) return;
    dim3 grid(nblk(M), nblk(N));
    k_gemm<AK, BK><<<grid, kGT, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, lower, tri_k, sq);
}

}  // namespace

void dense_syrk_t(int n, int k, const double *S, int lds, double *C, cudaStream_t st) {
    // C (lower) = S^T S, S k x n column-major: both operands depth-contiguous
    gemm<true, true>(n, n, k, 1.0, S, lds, S, lds, 0.0, C, n, 1, 0, nullptr, st);
}

void dense_potrf(int n, double *A, int *info_dev, cudaStream_t st) {
    set_dense_smem();
    const int nb = nblk(n);
    for (int b = 0; b < nb; b++) {
        const int c0 = b * kNB, w = std::min(kNB, n - c0), rest = n - c0 - w;
        k_potf2<<<1, 256, 0, st>>>(n, A, n, c0, info_dev);
        if (rest <= 0) break;
        k_trsm_panel<<<nblk(rest), kNB, 2 * kBlockBytes, st>>>(n, A, n, c0);
        // trailing update A22 -= X X^T, X = the panel (row-index contiguous)
        const double *X = A + (size_t)c0 * n + c0 + w;
        double *A22 = A + (size_t)(c0 + w) * n + c0 + w;
        gemm<false, false>(rest, rest, w, -1.0, X, n, X, n, 1.0, A22, n, 1, 0, nullptr, st);
    }
}

void dense_potri(int n, const double *L, double *Y, double *C, cudaStream_t st) {
    // Y = L^-1 (lower), block row by block row
    set_dense_smem();
    const int nb = nblk(n);
    k_fill<<<(unsigned)(((size_t)n * n + 255) / 256), 256, 0, st>>>((size_t)n * n, Y, 0.0);
    for (int i = 0; i < nb; i++) {
        k_trtri_row<<<1 + i, 256, 3 * kBlockBytes, st>>>(n, L, Y, n, i);
        const int r0 = (i + 1) * kNB;
        if (r0 >= n) break;
        // acc_(i', j) += L_(i', i) Y_(i, j) for the block rows below, j <= i
        const int w = std::min(kNB, n - i * kNB);
        gemm<false, true>(n - r0, r0, w, 1.0, L + (size_t)(i * kNB) * n + r0, n, Y + (size_t)(i * kNB), n, 1.0,
                          Y + r0, n, 0, 0, nullptr, st);
    }
    // C (lower) = Y^T Y with the depth starting at each block row (Y lower)
    gemm<true, true>(n, n, n, 1.0, Y, n, Y, n, 0.0, C, n, 1, 1, nullptr, st);
}

void dense_col_sq_of_product(int m, int n, const double *S, int lds, const double *C, double *work, double *d,
                             cudaStream_t st) {
    // G = S C (m x n): S(l, k) row-index contiguous, C(k, j) depth-contiguous;
    // d_j = sum_l G(l, j)^2 through per-row-block partial sums in work
    gemm<false, true>(m, n, n, 1.0, S, lds, C, n, 0.0, nullptr, 0, 0, 0, work, st);
    k_sum_blocks<<<(n + 255) / 256, 256, 0, st>>>(nblk(m), n, work, d);
}

}  // namespace crgpu
