// Element matrices and mixed-boundary factors on the device:
// src/precal.f90:13-222 with src/elem1.f90, src/elem3.f90, src/elem5.f90,
// src/elem8.f90, src/beta.f90 and the Bessel approximations of
// src/bessk0.f90, src/bessk1.f90, src/bessi0.f90, src/bessi1.f90.
#include "bessel.cuh"
#include "device.cuh"
#include "kernels.h"

namespace crgpu {

__device__ static void raise_err(const DevProblem &P, int code) { atomicCAS(P.err, 0, code); }

// integer base matrices of the linear triangle (src/elem3.f90:62-65)
__constant__ int c_s1[3][3] = {{1, -1, 0}, {-1, 1, 0}, {0, 0, 0}};
__constant__ int c_s2[3][3] = {{2, -1, -1}, {-1, 0, 1}, {-1, 1, 0}};
__constant__ int c_s3[3][3] = {{1, 0, -1}, {0, 0, 0}, {-1, 0, 1}};
__constant__ int c_s4[3][3] = {{2, 1, 1}, {1, 2, 1}, {1, 1, 2}};
// bilinear parallelogram (src/elem5.f90)
__constant__ int c_p1[4][4] = {{2, -2, -1, 1}, {-2, 2, 1, -1}, {-1, 1, 2, -2}, {1, -1, -2, 2}};
__constant__ int c_p2[4][4] = {{1, 0, -1, 0}, {0, -1, 0, 1}, {-1, 0, 1, 0}, {0, 1, 0, -1}};
__constant__ int c_p3[4][4] = {{2, 1, -1, -2}, {1, 2, -2, -1}, {-1, -2, 2, 1}, {-2, -1, 1, 2}};
__constant__ int c_p4[4][4] = {{4, 2, 1, 2}, {2, 4, 2, 1}, {1, 2, 4, 2}, {2, 1, 2, 4}};

// One thread per (wavenumber, area element): elbg[k][e][imn] = S1 + k^2 S2
// packed lower-triangular (m >= n, row by row).
__global__ void k_elbg(DevProblem P) {
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= P.K * P.elanz) return;
    int k = gid / P.elanz, e = gid % P.elanz;
    int typ = P.etype[e];
    double xk[4], yk[4];
    for (int q = 0; q < 4; q++) {
        int nd = P.enodes[e * 4 + q];
        xk[q] = nd >= 0 ? P.x[nd] : 0.0;
        yk[q] = nd >= 0 ? P.y[nd] : 0.0;
    }
    double kw = P.kwn[k];
    double out[10];
    for (int q = 0; q < 10; q++) out[q] = 0.0;
    if (typ == 3) {
        double x21 = xk[1] - xk[0], x31 = xk[2] - xk[0];
        double y21 = yk[1] - yk[0], y31 = yk[2] - yk[0];
        double det = x21 * y31 - x31 * y21;
        if (det <= 0.0) { raise_err(P, 26); return; }
        double a = (x31 * x31 + y31 * y31) / det;
        double b = -(x31 * x21 + y31 * y21) / det;
        double c = (x21 * x21 + y21 * y21) / det;
        int imn = 0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j <= i; j++, imn++) {
                double s = (a * c_s1[i][j] + b * c_s2[i][j] + c * c_s3[i][j]) / 2.0;
                double m = det * c_s4[i][j] / 24.0;
                out[imn] = s + m * kw * kw;
            }
    } else if (typ == 5) {
        double x21 = xk[1] - xk[0], x31 = xk[3] - xk[0];
        double y21 = yk[1] - yk[0], y31 = yk[3] - yk[0];
        double det = x21 * y31 - x31 * y21;
        if (det <= 0.0) { raise_err(P, 26); return; }
        double a = (x31 * x31 + y31 * y31) / det;
        double b = -(x31 * x21 + y31 * y21) / det;
        double c = (x21 * x21 + y21 * y21) / det;
        int imn = 0;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j <= i; j++, imn++) {
                double s = (a * c_p1[i][j] + 3.0 * b * c_p2[i][j] + c * c_p3[i][j]) / 6.0;
                double m = det * c_p4[i][j] / 36.0;
                out[imn] = s + m * kw * kw;
            }
    } else {  // 8: four sub-triangles about the diagonal intersection, centre condensed
        double ms[5][5], mm[5][5], xd[5], yd[5];
        for (int i = 0; i < 5; i++)
            for (int j = 0; j < 5; j++) { ms[i][j] = 0.0; mm[i][j] = 0.0; }
        double a1 = xk[2] - xk[0], a2 = xk[3] - xk[1];
        if (fabs(a1) <= 1e-12 || fabs(a2) <= 1e-12) { raise_err(P, 26); return; }
        a1 = (yk[2] - yk[0]) / a1;
        a2 = (yk[3] - yk[1]) / a2;
        if (fabs(a1 - a2) <= 1e-12) { raise_err(P, 26); return; }
        xd[4] = (a1 * xk[0] - yk[0] - a2 * xk[1] + yk[1]) / (a1 - a2);
        yd[4] = yk[0] + a1 * (xd[4] - xk[0]);
        for (int i = 0; i < 4; i++) { xd[i] = xk[i]; yd[i] = yk[i]; }
        const int ik_tab[4][3] = {{0, 1, 4}, {1, 2, 4}, {4, 2, 3}, {0, 4, 3}};
        for (int t = 0; t < 4; t++) {
            int i0 = ik_tab[t][0], i1 = ik_tab[t][1], i2 = ik_tab[t][2];
            double x21 = xd[i1] - xd[i0], x31 = xd[i2] - xd[i0];
            double y21 = yd[i1] - yd[i0], y31 = yd[i2] - yd[i0];
            double det = x21 * y31 - x31 * y21;
            if (det <= 1e-12) { raise_err(P, 26); return; }
            double a = (x31 * x31 + y31 * y31) / det;
            double b = -(x31 * x21 + y31 * y21) / det;
            double c = (x21 * x21 + y21 * y21) / det;
            int ik[3] = {i0, i1, i2};
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    ms[ik[i]][ik[j]] += (a * c_s1[i][j] + b * c_s2[i][j] + c * c_s3[i][j]) / 2.0;
                    mm[ik[i]][ik[j]] += det * c_s4[i][j] / 24.0;
                }
        }
        for (int i = 0; i < 5; i++)
            for (int j = 0; j < 5; j++) ms[i][j] = ms[i][j] + kw * kw * mm[i][j];
        int imn = 0;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j <= i; j++, imn++) out[imn] = ms[i][j] - ms[i][4] * ms[4][j] / ms[4][4];
    }
    double *dst = P.elbg + ((size_t)k * P.elanz + e) * 10;
    for (int q = 0; q < 10; q++) dst[q] = out[q];
}

// relbg of the type-11 boundary lines (src/elem1.f90: L/6 [2 1; 1 2])
__global__ void k_relbg(DevProblem P) {
    int rb = blockIdx.x * blockDim.x + threadIdx.x;
    if (rb >= P.relanz) return;
    int n0 = P.bnodes[rb * 2], n1 = P.bnodes[rb * 2 + 1];
    double x21 = P.x[n1] - P.x[n0], y21 = P.y[n1] - P.y[n0];
    double l = sqrt(x21 * x21 + y21 * y21);
    P.relbg[rb * 3 + 0] = l * 2.0 / 6.0;
    P.relbg[rb * 3 + 1] = l * 1.0 / 6.0;
    P.relbg[rb * 3 + 2] = l * 2.0 / 6.0;
}

// kg[k][l][rel] = beta(l, k) of src/beta.f90:38-135
__global__ void k_kg(DevProblem P) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t total = (size_t)P.K * P.eanz * P.relanz;
    if (gid >= total) return;
    int rb = (int)(gid % P.relanz);
    int l = (int)((gid / P.relanz) % P.eanz);
    int k = (int)(gid / ((size_t)P.relanz * P.eanz));
    if (P.btype[rb] != 11) { P.kg[gid] = 0.0; return; }
    int n0 = P.bnodes[rb * 2], n1 = P.bnodes[rb * 2 + 1];
    double xk0 = P.x[n0], yk0 = P.y[n0], xk1 = P.x[n1], yk1 = P.y[n1];
    int en = P.enr0[l];
    double xs = P.x[en], ys = P.y[en], sytop = P.sytop;
    double xr = (xk0 + xk1) / 2.0, yr = (yk0 + yk1) / 2.0;
    double x3 = xr - xs;
    double y3m = (yr - sytop) - (ys - sytop);
    double y3p = (yr - sytop) + (ys - sytop);
    double r1m = sqrt(x3 * x3 + y3m * y3m), r1p = sqrt(x3 * x3 + y3p * y3p);
    double x4 = yk0 - yk1, y4 = xk1 - xk0;
    double r2 = sqrt(x4 * x4 + y4 * y4);
    if (r1m < 1e-12 || r1p < 1e-12 || r2 < 1e-12) { raise_err(P, 35); P.kg[gid] = 0.0; return; }
    double cthetm = (x3 * x4 + y3m * y4) / r1m / r2;
    double cthetp = (x3 * x4 + y3p * y4) / r1p / r2;
    double kw = P.kwn[k];
    double bk0m = as_k0(r1m * kw), bk0p = as_k0(r1p * kw);
    double bk1m = as_k1(r1m * kw), bk1p = as_k1(r1p * kw);
    double b;
    if (bk0m + bk0p == 0.0) b = (cthetm + cthetp) / 2.0;
    else b = (cthetm * bk1m + cthetp * bk1p) / (bk0m + bk0p);
    P.kg[gid] = kw * b;
}

void launch_precal(const DevProblem &P, cudaStream_t st) {
    int nt = 128;
    if (P.K * P.elanz > 0) k_elbg<<<(P.K * P.elanz + nt - 1) / nt, nt, 0, st>>>(P);
    if (P.relanz > 0) {
        k_relbg<<<(P.relanz + nt - 1) / nt, nt, 0, st>>>(P);
        size_t tot = (size_t)P.K * P.eanz * P.relanz;
        k_kg<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P);
    }
}

}  // namespace crgpu
