// Adjoint of the forward block: the exact derivative of a linear functional
// of the voltages, L = sum_i g_i V_i, with respect to the conductivities.
// No single reference routine does this: CRTomo forms the Jacobian with
// src/bsensi.f90 (reciprocity, without the mixed-boundary term) and applies
// J^H in src/update.f90.  Here, with kpot_(k,l) = A_(k,l)^{-1} e_l and
//   V_i = sum_k w_k/pi [(kpot_(k,e2) - kpot_(k,e1))(P4) - (...)(P3)]
// (src/bvolt.f90, src/rtrafo.f90):
//   dL/dsigma_e = -sum_(k,l) w_k/pi lambda_(k,l)^T (dA_(k,l)/dsigma_e) kpot_(k,l),
//   lambda_(k,l) = A_(k,l)^{-1} c_l,  c_l = sum_(i: e2=l) g_i (e_P4 - e_P3)
//                                        - sum_(i: e1=l) g_i (e_P4 - e_P3).
// dA/dsigma_e is the element matrix of src/precal.f90 plus, for elements
// carrying a mixed boundary (src/kompab.f90:112-139), the boundary matrix
// relbg * beta(k, l).
#include "device.cuh"
#include "kernels.h"

namespace crgpu {

static constexpr double kPiA = 3.14159265358979323846264338327950288;

__device__ __forceinline__ void atomic_add_c(double2 *p, double2 v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
}

// c_l for every electrode l: [eanz][n]
__global__ void k_adj_sources(DevProblem P, const double2 *__restrict__ g, double2 *src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nanz) return;
    const int e1 = P.meas[i * 4], e2 = P.meas[i * 4 + 1], e3 = P.meas[i * 4 + 2], e4 = P.meas[i * 4 + 3];
    const double2 gi = g[i];
    const double2 mg = cz(-gi.x, -gi.y);
    const int p3 = e3 >= 0 ? P.enr0[e3] : -1, p4 = e4 >= 0 ? P.enr0[e4] : -1;
    if (e2 >= 0) {
        if (p4 >= 0) atomic_add_c(&src[(size_t)e2 * P.n + p4], gi);
        if (p3 >= 0) atomic_add_c(&src[(size_t)e2 * P.n + p3], mg);
    }
    if (e1 >= 0) {
        if (p4 >= 0) atomic_add_c(&src[(size_t)e1 * P.n + p4], mg);
        if (p3 >= 0) atomic_add_c(&src[(size_t)e1 * P.n + p3], gi);
    }
}

void launch_adjoint_sources(const DevProblem &P, const double2 *g, double2 *src, int lsink, int nsink,
                            cudaStream_t st) {
    (void)lsink;
    (void)nsink;  // the sink enters b, not the measured functional
    cudaMemsetAsync(src, 0, sizeof(double2) * (size_t)P.eanz * P.n, st);
    const int nt = 128;
    if (P.nanz > 0) k_adj_sources<<<(P.nanz + nt - 1) / nt, nt, 0, st>>>(P, g, src);
}

// scaled right-hand side D c_l of item (s, r) (src/scalab.f90 scaling);
// Dirichlet rows keep b = 0 (src/randb.f90)
__global__ void k_adj_rhs(DevProblem P, DevBatch B, int nrhs, const double2 *__restrict__ src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, item = blockIdx.y;
    if (i >= P.n) return;
    const int s = item / nrhs, r = item % nrhs;
    const int l = (nrhs == 1) ? B.ls[s] : r;
    const double f = B.fak[(size_t)s * P.n + i];
    const double2 v = P.dirichlet[i] ? cz(0.0, 0.0) : src[(size_t)l * P.n + i];
    B.b[(size_t)item * P.n + i] = cz(v.x * f, v.y * f);
}

void launch_adjoint_rhs(const DevProblem &P, const DevBatch &B, int nrhs, const double2 *src, cudaStream_t st) {
    const int nt = 128;
    k_adj_rhs<<<dim3((P.n + nt - 1) / nt, B.nsys * nrhs), nt, 0, st>>>(P, B, nrhs, src);
}

// lambda_(k,l) = D x in the layout of kpot, [K][eanz][n]
__global__ void k_adj_lambda(DevProblem P, DevBatch B, int nrhs, double2 *lambda) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, item = blockIdx.y;
    if (i >= P.n) return;
    const int s = item / nrhs, r = item % nrhs;
    const int k = B.ks[s], l = (nrhs == 1) ? B.ls[s] : r;
    const double f = B.fak[(size_t)s * P.n + i];
    const double2 x = B.x[(size_t)item * P.n + i];
    lambda[((size_t)k * P.eanz + l) * P.n + i] = cz(x.x * f, x.y * f);
}

void launch_adjoint_lambda(const DevProblem &P, const DevBatch &B, int nrhs, double2 *lambda, cudaStream_t st) {
    const int nt = 128;
    k_adj_lambda<<<dim3((P.n + nt - 1) / nt, B.nsys * nrhs), nt, 0, st>>>(P, B, nrhs, lambda);
}

constexpr int kAdjThreads = 128;

// one block per element: its threads run over the (k, l) pairs
__global__ __launch_bounds__(kAdjThreads) void k_adj_grad(DevProblem P, const double2 *__restrict__ kpot,
                                                           const double2 *__restrict__ lambda,
                                                           const int32_t *__restrict__ ebnd_ptr,
                                                           const int32_t *__restrict__ ebnd_list, double2 *grad) {
    const int e = blockIdx.x;
    const int nk = P.etype[e] == 3 ? 3 : 4;
    int nodes[4];
    bool dir[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        nodes[q] = q < nk ? P.enodes[e * 4 + q] : 0;
        dir[q] = q >= nk || P.dirichlet[nodes[q]] != 0;
    }
    const int b0 = ebnd_ptr[e], b1 = ebnd_ptr[e + 1];
    double2 acc = cz(0.0, 0.0);
    const int npairs = P.K * P.eanz;
    for (int t = threadIdx.x; t < npairs; t += blockDim.x) {
        const int k = t / P.eanz;
        const size_t base = (size_t)t * P.n;  // (k * eanz + l) * n
        double2 kv[4], lv[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            // a Dirichlet node keeps its potential (its value enters the other
            // rows through the moved column, src/randb2.f90); lambda is 0 there
            kv[q] = q >= nk ? cz(0.0, 0.0) : kpot[base + nodes[q]];
            lv[q] = dir[q] ? cz(0.0, 0.0) : lambda[base + nodes[q]];
        }
        const double *K = P.elbg + ((size_t)k * P.elanz + e) * 10;
        double2 qv = cz(0.0, 0.0);
#pragma unroll
        for (int m = 0; m < 4; m++) {
            double2 kk = cz(0.0, 0.0);
#pragma unroll
            for (int n2 = 0; n2 < 4; n2++) {
                const int imax = m > n2 ? m : n2, imin = m < n2 ? m : n2;
                const double a = (m < nk && n2 < nk) ? K[imax * (imax + 1) / 2 + imin] : 0.0;
                kk = cz(fma(a, kv[n2].x, kk.x), fma(a, kv[n2].y, kk.y));
            }
            qv = cadd(qv, cmul(lv[m], kk));
        }
        for (int q = b0; q < b1; q++) {  // mixed boundaries carried by this element
            const int rb = ebnd_list[q];
            const int n0 = P.bnodes[rb * 2], n1 = P.bnodes[rb * 2 + 1];
            const double beta = P.kg[(size_t)t * P.relanz + rb];
            const double r0 = P.relbg[rb * 3] * beta, r1 = P.relbg[rb * 3 + 1] * beta, r2 = P.relbg[rb * 3 + 2] * beta;
            const bool d0 = P.dirichlet[n0] != 0, d1 = P.dirichlet[n1] != 0;
            const double2 k0 = kpot[base + n0], k1 = kpot[base + n1];
            const double2 l0 = d0 ? cz(0.0, 0.0) : lambda[base + n0], l1 = d1 ? cz(0.0, 0.0) : lambda[base + n1];
            const double2 u0 = cz(r0 * k0.x + r1 * k1.x, r0 * k0.y + r1 * k1.y);
            const double2 u1 = cz(r1 * k0.x + r2 * k1.x, r1 * k0.y + r2 * k1.y);
            qv = cadd(qv, cadd(cmul(l0, u0), cmul(l1, u1)));
        }
        const double w = P.swrtr ? P.kwnwi[k] / kPiA : 1.0;
        acc = cz(acc.x - w * qv.x, acc.y - w * qv.y);
    }
    __shared__ double2 red[kAdjThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 s = red[0];
        for (int q = 1; q < kAdjThreads / 32; q++) s = cadd(s, red[q]);
        grad[e] = s;
    }
}

void launch_adjoint_grad(const DevProblem &P, const double2 *kpot, const double2 *lambda, const int32_t *ebnd_ptr,
                         const int32_t *ebnd_list, double2 *grad, cudaStream_t st) {
    if (P.elanz > 0) k_adj_grad<<<P.elanz, kAdjThreads, 0, st>>>(P, kpot, lambda, ebnd_ptr, ebnd_list, grad);
}

}  // namespace crgpu
