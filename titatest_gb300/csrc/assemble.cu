// Complex band assembly, Dirichlet rows, diagonal scaling and the right-hand
// sides: src/kompab.f90:11-194, src/randb.f90:1-84, src/randb2.f90:1-82,
// src/scalab.f90:14-87, src/kompb.f90:1-69.
//
// The matrix lives in a lower-triangular sparse pattern (Pattern in
// host.cpp); each entry sums its element contributions in element order,
// area elements first, as kompab does.  The area part does not depend on the
// current electrode and is assembled once per wavenumber (k_adom); the
// mixed-boundary part is added per (wavenumber, electrode) system.
#include "device.cuh"
#include "kernels.h"

namespace crgpu {

// Adom[k][p] = sum_e elbg[k][e][imn] * sigma_e  (area elements of entry p)
__global__ void k_adom(DevProblem P, const double2 *__restrict__ sigma, double2 *__restrict__ adom) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (size_t)P.K * P.nnz) return;
    int k = (int)(gid / P.nnz), p = (int)(gid % P.nnz);
    double2 v = cz(0.0, 0.0);
    const double *eb = P.elbg + (size_t)k * P.elanz * 10;
    for (int q = P.dom_ptr[p]; q < P.dom_ptr[p + 1]; q++) {
        int code = P.dom_list[q];
        int e = code >> 4, imn = code & 15;
        double dum = eb[(size_t)e * 10 + imn];
        double2 s = sigma[e];
        v = cadd(v, cz(dum * s.x, dum * s.y));
    }
    adom[gid] = v;
}

// Value of lower-pattern entry p of system (k, l) as kompab assembles it:
// area part plus the mixed-boundary terms.
__device__ __forceinline__ double2 entry_raw(const DevProblem &P, const double2 *__restrict__ ad,
                                             const double *__restrict__ kgl, const double2 *__restrict__ sigma,
                                             int p) {
    double2 v = ad[p];
    for (int q = P.bnd_ptr[p]; q < P.bnd_ptr[p + 1]; q++) {
        const int code = P.bnd_list[q];
        const int rb = code >> 4, imn = code & 15;
        const double dum = P.relbg[rb * 3 + imn] * kgl[rb];
        const double2 sg = sigma[P.brnr[rb]];
        v = cadd(v, cz(dum * sg.x, dum * sg.y));
    }
    return v;
}

// The same before scaling, with Dirichlet rows and columns replaced
// (src/randb.f90, src/randb2.f90: diagonal 1, the rest of the row and column 0).
__device__ __forceinline__ double2 entry_value(const DevProblem &P, const double2 *__restrict__ ad,
                                               const double *__restrict__ kgl, const double2 *__restrict__ sigma,
                                               int p, int i, int c, bool dir_i) {
    if (dir_i || P.dirichlet[c]) return (c == i) ? cz(1.0, 0.0) : cz(0.0, 0.0);
    return entry_raw(P, ad, kgl, sigma, p);
}

// 1/sqrt(|v|) = (re^2 + im^2)^(-1/4) without FP64 division or square root
// (both cost tens of FP64 operations, and FP64 runs at a small fraction of the
// FP32 rate here): an FP32 estimate refined by two Newton steps for
// y^-4 = x, y <- y (5 - x y^4) / 4, which square the relative error
// (~1e-7 -> ~1e-13 -> FP64 rounding).  Outside the FP32 range of x the FP64
// functions are used.
__device__ __forceinline__ double inv_sqrt_abs(double2 v) {
    const double x = v.x * v.x + v.y * v.y;
    if (!(x > 1e-30 && x < 1e30)) return 1.0 / sqrt(sqrt(x));
    double y = (double)rsqrtf(sqrtf((float)x));
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const double y2 = y * y;
        y = y * (5.0 - x * y2 * y2) * 0.25;
    }
    return y;
}

// lower-pattern entry of the diagonal of row i (-1: none)
__device__ __forceinline__ int diag_entry(const DevProblem &P, int i) {
    int pd = -1;
    for (int p = P.rowptr[i]; p < P.rowptr[i + 1]; p++)
        if (P.col[p] == i) pd = p;
    return pd;
}

// fak of the area part alone, per wavenumber and row (0: zero diagonal).  A
// row whose diagonal has no mixed-boundary term and which is not a
// Dirichlet row has this fak in every system of the wavenumber, whatever the
// current electrode.
__global__ void k_fak_area(DevProblem P, const double2 *__restrict__ adom, double *__restrict__ fak_area) {
    const size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (size_t)P.K * P.n) return;
    const int k = (int)(gid / P.n), i = (int)(gid % P.n);
    const int pd = diag_entry(P, i);
    double f = 0.0;
    if (pd >= 0) {
        const double2 d = adom[(size_t)k * P.nnz + pd];
        if (d.x * d.x + d.y * d.y > 0.0) f = inv_sqrt_abs(d);
    }
    fak_area[gid] = f;
}

// the area parts of every wavenumber (adom[k][p]), followed in the same
// allocation by fak_area[k][i]
void launch_adom(const DevProblem &P, const double2 *sigma, double2 *adom, cudaStream_t st) {
    const size_t tot = (size_t)P.K * P.nnz, totn = (size_t)P.K * P.n;
    const int nt = 256;
    k_adom<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, sigma, adom);
    k_fak_area<<<(unsigned)((totn + nt - 1) / nt), nt, 0, st>>>(P, adom, (double *)(adom + tot));
}

// fak of every row (src/scalab.f90:50-64): grid (row blocks, systems).  The
// rows of the lower pattern are sorted by column, so the diagonal is the
// last entry that is not padding.  Rows without a mixed-boundary term in the
// diagonal (and not Dirichlet rows) take the wavenumber's fak_area.
__global__ void k_fak(DevProblem P, DevBatch B, const double2 *__restrict__ sigma,
                      const double2 *__restrict__ adom) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= P.n) return;
    const int k = B.ks[s], l = B.ls[s];
    const double2 *ad = adom + (size_t)k * P.nnz;
    const double *kgl = P.kg + ((size_t)k * P.eanz + l) * P.relanz;
    const int pd = diag_entry(P, i);
    double f = 1.0;
    if (pd >= 0 && !P.dirichlet[i] && P.bnd_ptr[pd] == P.bnd_ptr[pd + 1]) {
        const double fa = ((const double *)(adom + (size_t)P.K * P.nnz))[(size_t)k * P.n + i];
        if (fa > 0.0) f = fa;
        else atomicCAS(&B.status[s], 0, 27);  // src/scalab.f90:57-61
    } else {
        double2 d = cz(0.0, 0.0);
        if (pd >= 0) d = entry_value(P, ad, kgl, sigma, pd, i, i, P.dirichlet[i] != 0);
        if (!(d.x * d.x + d.y * d.y > 0.0)) {  // src/scalab.f90:57-61
            atomicCAS(&B.status[s], 0, 27);
        } else {
            f = inv_sqrt_abs(d);
        }
    }
    B.fak[(size_t)s * P.n + i] = f;
}

// Scaled values (src/kompab.f90 + src/scalab.f90:63-80), one thread per
// pattern entry: a_ij fak_i fak_j, which makes the diagonal a_ii / |a_ii| as
// scalab sets it.  Grid (entry blocks, systems).
__global__ void k_assemble_entries(DevProblem P, DevBatch B, const double2 *__restrict__ sigma,
                                   const double2 *__restrict__ adom) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (p >= P.nnz) return;
    double2 *as = B.As + (size_t)s * P.nnz;
    const int c = P.col[p];
    if (c < 0) {
        as[p] = cz(0.0, 0.0);
        return;
    }
    const int i = P.row[p];
    const int k = B.ks[s], l = B.ls[s];
    const double2 *ad = adom + (size_t)k * P.nnz;
    const double *kgl = P.kg + ((size_t)k * P.eanz + l) * P.relanz;
    const double *f = B.fak + (size_t)s * P.n;
    const double2 v = entry_value(P, ad, kgl, sigma, p, i, c, P.dirichlet[i] != 0);
    const double fk = f[i] * f[c];
    as[p] = cz(v.x * fk, v.y * fk);
}

void launch_assemble(const DevProblem &P, const DevBatch &B, const double2 *sigma, const double2 *adom,
                     cudaStream_t st) {
    const int nt = 128;
    k_fak<<<dim3((P.n + nt - 1) / nt, B.nsys), nt, 0, st>>>(P, B, sigma, adom);
    k_assemble_entries<<<dim3((P.nnz + nt - 1) / nt, B.nsys), nt, 0, st>>>(P, B, sigma, adom);
}

// Right-hand sides.  nrhs == 1: one system per (k, l), b of kompab (unit
// sink -1 at the current electrode, +1 at the fictitious sink, zero on
// Dirichlet nodes) scaled by fak.  nrhs == eanz: one factor per k; rhs 0 as
// kompab, rhs l > 0 as kompb (b(enr(l)) = -fak(enr(l)), b(nsink) = fak(nsink)).
__global__ void k_rhs(DevProblem P, DevBatch B, int nrhs, int lsink, int nsink) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t nitems = (size_t)B.nsys * nrhs;
    if (gid >= nitems * P.n) return;
    int item = (int)(gid / P.n), i = (int)(gid % P.n);
    int s = item / nrhs, r = item % nrhs;
    int l = (nrhs == 1) ? B.ls[s] : r;
    double f = B.fak[(size_t)s * P.n + i];
    double2 v = cz(0.0, 0.0);
    if (nrhs == 1 || r == 0) {
        if (i == P.enr0[l]) v = cz(-1.0, 0.0);
        if (lsink && i == nsink) v = cz(1.0, 0.0);
        if (P.dirichlet[i]) v = cz(0.0, 0.0);
        v = cz(v.x * f, v.y * f);
    } else {
        if (i == P.enr0[l]) v = cz(-f, 0.0);
        if (lsink && i == nsink) v = cz(f, 0.0);
    }
    B.b[gid] = v;
}

void launch_rhs(const DevProblem &P, const DevBatch &B, int nrhs, int lsink, int nsink, cudaStream_t st) {
    size_t tot = (size_t)B.nsys * nrhs * P.n;
    int nt = 256;
    k_rhs<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, B, nrhs, lsink, nsink);
}

// Valued Dirichlet nodes (src/randb2.f90:37-79) in the right-hand sides that
// kompab built: every system when nrhs == 1, right-hand side 0 of each
// wavenumber when nrhs == eanz (the others are kompb's, src/fem.f90:355-376,
// which leaves the values out).  A valued node's b is -value; any other row
// that is not a Dirichlet row gains value * a(i, m) for each valued neighbour
// m, with a(i, m) as kompab assembled it.  b is already scaled by fak; fak is 1
// on Dirichlet rows.  Grid (row blocks, systems).
__global__ void k_rhs_randb2(DevProblem P, DevBatch B, int nrhs, const double2 *__restrict__ sigma,
                             const double2 *__restrict__ adom) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= P.n) return;
    double2 *b = B.b + ((size_t)s * nrhs) * P.n;
    const uint8_t di = P.dirichlet[i];
    if (di == 2) {
        const double2 v = P.rwd_b[i];
        b[i] = cz(-v.x, -v.y);
        return;
    }
    if (di) return;
    const int k = B.ks[s], l = B.ls[s];
    const double2 *ad = adom + (size_t)k * P.nnz;
    const double *kgl = P.kg + ((size_t)k * P.eanz + l) * P.relanz;
    double2 acc = cz(0.0, 0.0);
    bool any = false;
    for (int q = P.fptr[i]; q < P.fptr[i + 1]; q++) {
        const double2 w = P.rwd_col[P.fcol[q]];
        if (w.x == 0.0 && w.y == 0.0) continue;
        acc = cadd(acc, cmul(w, entry_raw(P, ad, kgl, sigma, P.fidx[q])));
        any = true;
    }
    if (!any) return;
    const double f = B.fak[(size_t)s * P.n + i];
    const double2 v = b[i];
    b[i] = cz(v.x + acc.x * f, v.y + acc.y * f);
}

void launch_rhs_randb2(const DevProblem &P, const DevBatch &B, int nrhs, const double2 *sigma,
                       const double2 *adom, cudaStream_t st) {
    if (!P.lrandb2) return;
    const int nt = 128;
    k_rhs_randb2<<<dim3((P.n + nt - 1) / nt, B.nsys), nt, 0, st>>>(P, B, nrhs, sigma, adom);
}

}  // namespace crgpu
