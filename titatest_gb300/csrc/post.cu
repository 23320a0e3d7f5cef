// Wavenumber back-transform, voltages and sensitivities:
// src/rtrafo.f90:13-92, src/bvolt.f90:7-89, src/bvolti.f90:8-100,
// src/bsens.f90:23-197, src/bsensi.f90:23-194.
#include "device.cuh"
#include "kernels.h"

namespace crgpu {

static constexpr double kPi = 3.14159265358979323846264338327950288;

// hpot(j, l) = sum_k kpot(j, l, k) * kwnwi(k) / pi  (2D: kpot(j, l, 1))
__global__ void k_rtrafo(DevProblem P, const double2 *__restrict__ kpot, double2 *__restrict__ hpot) {
    size_t gid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t tot = (size_t)P.eanz * P.n;
    if (gid >= tot) return;
    if (P.swrtr == 0) {
        hpot[gid] = kpot[gid];
        return;
    }
    double2 s = cz(0.0, 0.0);
    for (int k = 0; k < P.K; k++) {
        double2 v = kpot[(size_t)k * tot + gid];
        double w = P.kwnwi[k];
        s = cadd(s, cz(v.x * w, v.y * w));
    }
    hpot[gid] = cz(s.x / kPi, s.y / kPi);
}

void launch_rtrafo(const DevProblem &P, const double2 *kpot, double2 *hpot, cudaStream_t st) {
    size_t tot = (size_t)P.eanz * P.n;
    int nt = 256;
    k_rtrafo<<<(unsigned)((tot + nt - 1) / nt), nt, 0, st>>>(P, kpot, hpot);
}

// V_i = (phi_e2(P_e4) - phi_e1(P_e4)) - (phi_e2(P_e3) - phi_e1(P_e3))
__global__ void k_bvolt(DevProblem P, const double2 *__restrict__ hpot, int mode,
                        const double *__restrict__ kfak, double2 *volt, double2 *sigmaa) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nanz) return;
    int e1 = P.meas[i * 4], e2 = P.meas[i * 4 + 1], e3 = P.meas[i * 4 + 2], e4 = P.meas[i * 4 + 3];
    auto hp = [&](int node_e, int src_e) -> double2 {
        if (node_e < 0 || src_e < 0) return cz(0.0, 0.0);
        return hpot[(size_t)src_e * P.n + P.enr0[node_e]];
    };
    double2 d1 = hp(e4, e2), d2 = hp(e4, e1), d3 = hp(e3, e2), d4 = hp(e3, e1);
    double2 v = csub(csub(d1, d2), csub(d3, d4));
    if (P.ldc) v.y = 0.0;  // dcmplx of the real DC voltage (src/bvolti.f90:56-62): -log(V < 0) = -ln|V| - i pi
    if (volt) volt[i] = v;
    if (mode == 0) {
        double kf = kfak ? kfak[i] : 1.0;
        if (sigmaa) sigmaa[i] = cz(kf * v.x, kf * v.y);
    } else {
        double a = cabsd(v);
        if (!(a > 0.0)) {  // src/bvolti.f90:80-85
            atomicCAS(P.err, 0, 82);
            if (sigmaa) sigmaa[i] = cz(0.0, 0.0);
            return;
        }
        if (sigmaa) sigmaa[i] = cz(-log(a), -atan2(v.y, v.x));
    }
}

__global__ void k_real_part(double2 *v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i].y = 0.0;
}

void launch_real_part(double2 *v, int n, cudaStream_t st) {
    if (n > 0) k_real_part<<<(n + 127) / 128, 128, 0, st>>>(v, n);
}

void launch_bvolt(const DevProblem &P, const double2 *hpot, int mode, const double *kfak, double2 *volt,
                  double2 *sigmaa, cudaStream_t st) {
    int nt = 128;
    k_bvolt<<<(P.nanz + nt - 1) / nt, nt, 0, st>>>(P, hpot, mode, kfak, volt, sigmaa);
}

// ---------------------------------------------------------------------------
// Sensitivities by reciprocity.  For element e, wavenumber k and measurement
// i with current electrodes (e1, e2) and voltage electrodes (e3, e4):
//   hsens_k = sum_{m,n} K_k[m][n] (kpot(node_m,e4) - kpot(node_m,e3))
//                                 (kpot(node_n,e2) - kpot(node_n,e1))
// with K_k the element matrix elbg; then the quadrature over k.
// One block per element; the element's kpot values of all electrodes are
// staged in shared memory one wavenumber at a time, threads run over
// measurements and keep their k-sums in registers.
// ---------------------------------------------------------------------------
constexpr int kSensThreads = 256;
constexpr int kSensMPT = 16;  // measurements per thread per pass (4096 per pass)

template <typename R>
struct SensT;
template <>
struct SensT<double> {
    using C = double2;
    __device__ static C mk(double a, double b) { return cz(a, b); }
};
template <>
struct SensT<float> {
    using C = float2;
    __device__ static C mk(float a, float b) { return cf(a, b); }
};

// MODE 0: src/bsens.f90, MODE 1: src/bsensi.f90.  R: arithmetic type of the
// element contraction (double: the reference arithmetic, from kpot; float: the
// mixed mode, from its complex64 copy, with FP64 output).
template <int MODE, typename R>
__global__ __launch_bounds__(kSensThreads) void k_bsens(DevProblem P,
                                                         const typename SensT<R>::C *__restrict__ kpot,
                                                         const double2 *__restrict__ sigma,
                                                         const double2 *__restrict__ volt,
                                                         double2 *__restrict__ sens, int e_first) {
    using C = typename SensT<R>::C;
    constexpr bool kTwoPlanes = sizeof(R) == 4;  // complex64: hi and lo planes of kpot
    extern __shared__ __align__(16) unsigned char kp_raw[];
    C *kp_sh = (C *)kp_raw;  // [4][eanz]
    C *kl_sh = kp_sh + 4 * P.eanz;  // [4][eanz] lo plane (complex64 only)
    const size_t plane = (size_t)P.K * P.eanz * P.n;
    __shared__ R kel[10];
    const int e = e_first + blockIdx.x;
    const int nk = P.etype[e] == 3 ? 3 : 4;
    int nodes[4];
#pragma unroll
    for (int q = 0; q < 4; q++) nodes[q] = P.enodes[e * 4 + q];
    const int eanz = P.eanz;
    const int4 *meas4 = (const int4 *)P.meas;
    for (int i0 = 0; i0 < P.nanz; i0 += kSensThreads * kSensMPT) {
        C acc[kSensMPT];
#pragma unroll
        for (int m = 0; m < kSensMPT; m++) acc[m] = SensT<R>::mk(0, 0);
        for (int k = 0; k < P.K; k++) {
            __syncthreads();
            for (int t = threadIdx.x; t < nk * eanz; t += kSensThreads) {
                int q = t / eanz, l = t % eanz;
                const size_t at = ((size_t)k * eanz + l) * P.n + nodes[q];
                kp_sh[t] = kpot[at];
                if (kTwoPlanes) kl_sh[t] = kpot[at + plane];
            }
            if (threadIdx.x < 10) kel[threadIdx.x] = (R)P.elbg[((size_t)k * P.elanz + e) * 10 + threadIdx.x];
            __syncthreads();
            const R w = P.swrtr ? (R)P.kwnwi[k] : (R)1;
#pragma unroll
            for (int m = 0; m < kSensMPT; m++) {
                int i = i0 + m * kSensThreads + threadIdx.x;
                if (i >= P.nanz) continue;
                const int4 ee = meas4[i];  // electrodes e1..e4 (-1: none), L1-resident
                C u[4], v[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    C s1 = ee.x >= 0 ? kp_sh[q * eanz + ee.x] : SensT<R>::mk(0, 0);
                    C s2 = ee.y >= 0 ? kp_sh[q * eanz + ee.y] : SensT<R>::mk(0, 0);
                    C s3 = ee.z >= 0 ? kp_sh[q * eanz + ee.z] : SensT<R>::mk(0, 0);
                    C s4 = ee.w >= 0 ? kp_sh[q * eanz + ee.w] : SensT<R>::mk(0, 0);
                    u[q] = SensT<R>::mk(s2.x - s1.x, s2.y - s1.y);
                    v[q] = SensT<R>::mk(s4.x - s3.x, s4.y - s3.y);
                    if (kTwoPlanes) {  // the dipole differences to ~complex64 accuracy of the difference
                        const C z = SensT<R>::mk(0, 0);
                        C t1 = ee.x >= 0 ? kl_sh[q * eanz + ee.x] : z, t2 = ee.y >= 0 ? kl_sh[q * eanz + ee.y] : z;
                        C t3 = ee.z >= 0 ? kl_sh[q * eanz + ee.z] : z, t4 = ee.w >= 0 ? kl_sh[q * eanz + ee.w] : z;
                        u[q] = SensT<R>::mk(u[q].x + (t2.x - t1.x), u[q].y + (t2.y - t1.y));
                        v[q] = SensT<R>::mk(v[q].x + (t4.x - t3.x), v[q].y + (t4.y - t3.y));
                    }
                    if (q >= nk) { u[q] = SensT<R>::mk(0, 0); v[q] = SensT<R>::mk(0, 0); }
                }
                C hs = SensT<R>::mk(0, 0);
#pragma unroll
                for (int mi = 0; mi < 4; mi++) {
                    if (mi >= nk) continue;
                    C ku = SensT<R>::mk(0, 0);
#pragma unroll
                    for (int mj = 0; mj < 4; mj++) {
                        if (mj >= nk) continue;
                        int imax = mi > mj ? mi : mj, imin = mi < mj ? mi : mj;
                        R kk = kel[imax * (imax + 1) / 2 + imin];
                        ku.x = fma(kk, u[mj].x, ku.x);
                        ku.y = fma(kk, u[mj].y, ku.y);
                    }
                    hs.x = fma(v[mi].x, ku.x, hs.x);
                    hs.x = fma(-v[mi].y, ku.y, hs.x);
                    hs.y = fma(v[mi].x, ku.y, hs.y);
                    hs.y = fma(v[mi].y, ku.x, hs.y);
                }
                acc[m].x = fma(hs.x, w, acc[m].x);
                acc[m].y = fma(hs.y, w, acc[m].y);
            }
        }
#pragma unroll
        for (int m = 0; m < kSensMPT; m++) {
            int i = i0 + m * kSensThreads + threadIdx.x;
            if (i >= P.nanz) continue;
            double2 d = cz((double)acc[m].x, (double)acc[m].y);
            double2 out;
            if (MODE == 0) {
                double f = P.swrtr ? P.strom[i] / kPi : P.strom[i];
                out = cz(-d.x * f, -d.y * f);
            } else {
                if (P.swrtr) d = cz(d.x / kPi, d.y / kPi);
                out = cdiv(cmul(d, sigma[e]), volt[i]);
            }
            sens[(size_t)e * P.nanz + i] = out;
        }
    }
}

void launch_bsens(const DevProblem &P, const double2 *kpot, const float2 *kpot32, const double2 *sigma,
                  const double2 *volt, int mode, bool single, double2 *sens, cudaStream_t st, int e_first,
                  int e_count) {
    if (e_count < 0) e_count = P.elanz - e_first;
    if (e_count <= 0) return;
    if (single && sens_tc_supported(P, mode) && P.tune_sens != 2) {
        launch_sens_tc(P, kpot32, sens, st, e_first, e_count);
        return;
    }
    if (single) {
        size_t smem = sizeof(float2) * 8 * P.eanz;  // hi and lo planes
        if (mode == 0) k_bsens<0, float><<<e_count, kSensThreads, smem, st>>>(P, kpot32, sigma, volt, sens, e_first);
        else k_bsens<1, float><<<e_count, kSensThreads, smem, st>>>(P, kpot32, sigma, volt, sens, e_first);
    } else {
        size_t smem = sizeof(double2) * 4 * P.eanz;
        if (mode == 0) k_bsens<0, double><<<e_count, kSensThreads, smem, st>>>(P, kpot, sigma, volt, sens, e_first);
        else k_bsens<1, double><<<e_count, kSensThreads, smem, st>>>(P, kpot, sigma, volt, sens, e_first);
    }
}

}  // namespace crgpu
