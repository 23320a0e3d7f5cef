// Complex band assembly, Dirichlet rows, diagonal scaling and the right-hand
// sides: src/kompab.f90:11-194, src/randb.f90:1-84, src/scalab.f90:14-87,
// src/kompb.f90:1-69.
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

void launch_adom(const DevProblem &P, const double2 *sigma, double2 *adom, cudaStream_t st) {
    size_t tot = (size_t)P.K * P.nnz;
    int nt = 256;
    k_adom<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, sigma, adom);
}

// One thread per (system, row): raw values of the row (area part + mixed
// boundary part), Dirichlet rows and columns, and fak of the row.
__global__ void k_assemble_rows(DevProblem P, DevBatch B, const double2 *__restrict__ sigma,
                                const double2 *__restrict__ adom) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (size_t)B.nsys * P.n) return;
    int s = (int)(gid / P.n), i = (int)(gid % P.n);
    int k = B.ks[s], l = B.ls[s];
    const double2 *ad = adom + (size_t)k * P.nnz;
    double2 *as = B.As + (size_t)s * P.nnz;
    const double *kgl = P.kg + ((size_t)k * P.eanz + l) * P.relanz;
    bool dir_i = P.dirichlet[i] != 0;
    int p0 = P.rowptr[i], p1 = P.rowptr[i + 1];
    double2 diag = cz(0.0, 0.0);
    for (int p = p0; p < p1; p++) {
        double2 v = ad[p];
        for (int q = P.bnd_ptr[p]; q < P.bnd_ptr[p + 1]; q++) {
            int code = P.bnd_list[q];
            int rb = code >> 4, imn = code & 15;
            double dum = P.relbg[rb * 3 + imn] * kgl[rb];
            double2 sg = sigma[P.brnr[rb]];
            v = cadd(v, cz(dum * sg.x, dum * sg.y));
        }
        int c = P.col[p];
        if (c < 0) {
            as[p] = cz(0.0, 0.0);
            continue;
        }
        if (dir_i || P.dirichlet[c]) v = (c == i) ? cz(1.0, 0.0) : cz(0.0, 0.0);
        as[p] = v;
        if (c == i) diag = v;
    }
    double dum = cabsd(diag);
    if (!(dum > 0.0)) {  // src/scalab.f90:57-61
        atomicCAS(&B.status[s], 0, 27);
        dum = 1.0;
    }
    B.fak[(size_t)s * P.n + i] = 1.0 / sqrt(dum);
}

// scaling of every entry with the factors of its row and column
__global__ void k_scale(DevProblem P, DevBatch B) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (size_t)B.nsys * P.nnz) return;
    int s = (int)(gid / P.nnz), p = (int)(gid % P.nnz);
    double2 *a = B.As + gid;
    int i = P.row[p], c = P.col[p];
    if (c < 0) return;
    if (i == c) {
        double2 v = *a;
        double dum = cabsd(v);
        if (dum > 0.0) *a = cdiv(v, cz(dum, 0.0));
    } else {
        const double *f = B.fak + (size_t)s * P.n;
        double fk = f[i] * f[c];
        double2 v = *a;
        *a = cz(v.x * fk, v.y * fk);
    }
}

void launch_assemble(const DevProblem &P, const DevBatch &B, const double2 *sigma, const double2 *adom,
                     cudaStream_t st) {
    int nt = 256;
    size_t t1 = (size_t)B.nsys * P.n;
    k_assemble_rows<<<(unsigned)((t1 + nt - 1) / nt), nt, 0, st>>>(P, B, sigma, adom);
    size_t t2 = (size_t)B.nsys * P.nnz;
    k_scale<<<(unsigned)((t2 + nt - 1) / nt), nt, 0, st>>>(P, B);
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

}  // namespace crgpu
