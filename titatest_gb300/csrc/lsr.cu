// Singularity removal (crmod.cfg mswitch bit 2): the reference conductivity
// of src/refsig.f90:7-73, the analytic half-space potential of
// src/potana.f90:7-99, the right-hand side of the lsr branch of
// src/kompab.f90:129-133 and the addition of the analytic part to kpot
// (src/fem.f90:390-391).
#include "bessel.cuh"
#include "device.cuh"
#include "kernels.h"

namespace crgpu {

namespace {
constexpr double kPiL = 3.14159265358979323846264338327950288;
constexpr int kRefThreads = 256;
}  // namespace

// sigma0 = exp( sum_e area_e log(sigma_e) / sum_e area_e ), one block
__global__ __launch_bounds__(kRefThreads) void k_refsig(DevProblem P, const double2 *__restrict__ sigma,
                                                        double2 *sigma0) {
    double sr = 0.0, si = 0.0, sa = 0.0;
    for (int e = threadIdx.x; e < P.elanz; e += kRefThreads) {
        const double a = P.earea[e];
        const double2 z = sigma[e];
        sr += a * log(sqrt(z.x * z.x + z.y * z.y));
        si += a * atan2(z.y, z.x);
        sa += a;
    }
    __shared__ double red[3][kRefThreads];
    red[0][threadIdx.x] = sr;
    red[1][threadIdx.x] = si;
    red[2][threadIdx.x] = sa;
    __syncthreads();
    if (threadIdx.x == 0) {
        sr = si = sa = 0.0;
        for (int t = 0; t < kRefThreads; t++) {
            sr += red[0][t];
            si += red[1][t];
            sa += red[2][t];
        }
        const double mr = sr / sa, mi = si / sa;
        const double ex = exp(mr);
        *sigma0 = cz(ex * cos(mi), ex * sin(mi));
    }
}

void launch_refsig(const DevProblem &P, const double2 *sigma, double2 *sigma0, cudaStream_t st) {
    k_refsig<<<1, kRefThreads, 0, st>>>(P, sigma, sigma0);
}

// pota(j) = K0(k r-) + K0(k r+) for every node but the source (image source
// mirrored at y = 0), and the per-system maximum
__global__ void k_pota_raw(DevProblem P, DevBatch B) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (size_t)B.nsys * P.n) return;
    const int s = (int)(gid / P.n), j = (int)(gid % P.n);
    const int src = P.enr0[B.ls[s]];
    if (j == src) {
        B.pota[gid] = cz(0.0, 0.0);
        return;
    }
    const double kw = P.kwn[B.ks[s]];
    const double x1 = P.x[src], y1 = P.y[src];
    const double x21 = P.x[j] - x1, y21m = P.y[j] - y1, y21p = P.y[j] + y1;
    const double rm = sqrt(x21 * x21 + y21m * y21m), rp = sqrt(x21 * x21 + y21p * y21p);
    const double dum = as_k0(rm * kw) + as_k0(rp * kw);
    B.pota[gid] = cz(dum, 0.0);
    // K0 > 0: the bit patterns of non-negative doubles order like the values
    atomicMax((unsigned long long *)&B.potmax[s], (unsigned long long)__double_as_longlong(dum));
}

// source node = 5 * max, then the scale (1/2pi) / sigma0
__global__ void k_pota_scale(DevProblem P, DevBatch B, const double2 *__restrict__ sigma0) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (size_t)B.nsys * P.n) return;
    const int s = (int)(gid / P.n), j = (int)(gid % P.n);
    double2 v = B.pota[gid];
    if (j == P.enr0[B.ls[s]]) v = cz(5.0 * B.potmax[s], 0.0);
    const double2 d2 = cdiv(cz(0.5 / kPiL, 0.0), *sigma0);
    B.pota[gid] = cmul(v, d2);
}

// b = D pota with D_ij = sum over the element contributions of (i, j) of
// dum (sigma - sigma0), symmetric; the fictitious sink overrides; scaled by fak
__global__ void k_rhs_lsr(DevProblem P, DevBatch B, const double2 *__restrict__ sigma,
                          const double2 *__restrict__ sigma0, int lsink, int nsink) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (size_t)B.nsys * P.n) return;
    const int s = (int)(gid / P.n), i = (int)(gid % P.n);
    const int k = B.ks[s], l = B.ls[s];
    const double2 s0 = *sigma0;
    const double *eb = P.elbg + (size_t)k * P.elanz * 10;
    const double *kgl = P.kg + ((size_t)k * P.eanz + l) * P.relanz;
    const double2 *pota = B.pota + (size_t)s * P.n;
    double2 acc = cz(0.0, 0.0);
    for (int q = P.fptr[i]; q < P.fptr[i + 1]; q++) {
        const int p = P.fidx[q];
        double2 d = cz(0.0, 0.0);
        for (int t = P.dom_ptr[p]; t < P.dom_ptr[p + 1]; t++) {
            const int code = P.dom_list[t];
            const double dum = eb[(size_t)(code >> 4) * 10 + (code & 15)];
            const double2 ds = csub(sigma[code >> 4], s0);
            d = cadd(d, cz(dum * ds.x, dum * ds.y));
        }
        for (int t = P.bnd_ptr[p]; t < P.bnd_ptr[p + 1]; t++) {
            const int code = P.bnd_list[t];
            const int rb = code >> 4;
            const double dum = P.relbg[rb * 3 + (code & 15)] * kgl[rb];
            const double2 ds = csub(sigma[P.brnr[rb]], s0);
            d = cadd(d, cz(dum * ds.x, dum * ds.y));
        }
        acc = cadd(acc, cmul(d, pota[P.fcol[q]]));
    }
    if (lsink && i == nsink) acc = cz(1.0, 0.0);
    const double f = B.fak[(size_t)s * P.n + i];
    B.b[gid] = cz(acc.x * f, acc.y * f);
}

void launch_pota_rhs(const DevProblem &P, const DevBatch &B, const double2 *sigma, const double2 *sigma0, int lsink,
                     int nsink, cudaStream_t st) {
    size_t tot = (size_t)B.nsys * P.n;
    int nt = 256;
    unsigned g = (unsigned)((tot + nt - 1) / nt);
    cudaMemsetAsync(B.potmax, 0, sizeof(double) * B.nsys, st);
    k_pota_raw<<<g, nt, 0, st>>>(P, B);
    k_pota_scale<<<g, nt, 0, st>>>(P, B, sigma0);
    k_rhs_lsr<<<g, nt, 0, st>>>(P, B, sigma, sigma0, lsink, nsink);
}

}  // namespace crgpu
