// Kernel launchers (defined in the .cu files) used by the C ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "device.cuh"

namespace crgpu {

void launch_precal(const DevProblem &P, cudaStream_t st);

// assembly (src/kompab.f90, src/randb.f90, src/scalab.f90, src/kompb.f90)
void launch_adom(const DevProblem &P, const double2 *sigma, double2 *adom, cudaStream_t st);
void launch_assemble(const DevProblem &P, const DevBatch &B, const double2 *sigma,
                     const double2 *adom, cudaStream_t st);
void launch_rhs(const DevProblem &P, const DevBatch &B, int nrhs, int lsink, int nsink,
                cudaStream_t st);
void launch_rhs_randb2(const DevProblem &P, const DevBatch &B, int nrhs, const double2 *sigma,
                       const double2 *adom, cudaStream_t st);

// singularity removal (src/refsig.f90, src/potana.f90, kompab lsr branch)
void launch_refsig(const DevProblem &P, const double2 *sigma, double2 *sigma0, cudaStream_t st);
void launch_pota_rhs(const DevProblem &P, const DevBatch &B, const double2 *sigma, const double2 *sigma0,
                     int lsink, int nsink, cudaStream_t st);

// factorisation (src/chol.f90) with fused forward substitution when fuse != 0
void launch_factor_plain(const DevProblem &P, const DevBatch &B, int fuse, int nsm,
                         cudaStream_t st);
// complex128 factor with the window in registers (factor_plain.cu); false
// when the band is too wide for it
bool launch_factor_plain_reg(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st);
bool launch_factor_warp(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st);
// the complex64 factor kernel launch_factor_mixed runs (the values of tune_factor)
int mixed_factor_kind(const DevProblem &P);
// the tensor-core factors of several problems' batches in one persistent
// launch over (problem, system) items (tc_factor.cu)
void launch_factor_tc_multi(const DevProblem *Ps, const DevBatch *Bs, const int2 *items, int nitems, int fuse, int nsm,
                            cudaStream_t st);
int launch_factor_mixed(const DevProblem &P, const DevBatch &B, int fuse, int nsm, bool exclusive,
                        cudaStream_t st);
int mixed_window_supported(int W);
// shared-memory window variant (factor_smem.cu) for 176 < mb + 1 <= 208
int mixed_smem_window_supported(int W);
int launch_factor_mixed_smem(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st);
// tensor-core variant (tc_factor.cu) for band widths mb <= 124
// exclusive: each block asks for the whole shared memory of its SM, so that
// no other kernel's blocks share the SM with it (the partial last round,
// which runs beside the full rounds' solves)
int launch_factor_tc(const DevProblem &P, const DevBatch &B, int fuse, int nsm, cudaStream_t st,
                     bool exclusive = false);

// triangular solves (src/vre.f90); item = system * nrhs + rhs
void launch_forward_solve(const DevProblem &P, const DevBatch &B, int nrhs, bool mixed,
                          const double2 *rin, cudaStream_t st);
void launch_back_solve(const DevProblem &P, const DevBatch &B, int nrhs, bool mixed,
                       cudaStream_t st);
// refinement helpers (FP64)
void launch_residual(const DevProblem &P, const DevBatch &B, int nrhs, cudaStream_t st);
void launch_fill_active(const DevBatch &B, int nrhs, cudaStream_t st);
void launch_accumulate(const DevProblem &P, const DevBatch &B, int nrhs, bool first,
                       double tol, cudaStream_t st);
void launch_copy_solution(const DevProblem &P, const DevBatch &B, int nrhs, cudaStream_t st);
// kpot (complex128) and, when kpot32 is given, its complex64 copy for the
// mixed-precision Jacobian
void launch_kpot(const DevProblem &P, const DevBatch &B, int nrhs, double2 *kpot, float2 *kpot32,
                 cudaStream_t st);

// back-transform and voltages (src/rtrafo.f90, src/bvolt.f90, src/bvolti.f90)
void launch_rtrafo(const DevProblem &P, const double2 *kpot, double2 *hpot, cudaStream_t st);
void launch_bvolt(const DevProblem &P, const double2 *hpot, int mode, const double *kfak,
                  double2 *volt, double2 *sigmaa, cudaStream_t st);

// sensitivities (src/bsens.f90, src/bsensi.f90)
// elements e_first .. e_first + e_count - 1 (e_count < 0: to the last)
// Jacobian on the tensor cores (Gram form, complex64 contraction; src/bsens.f90
// mode, eanz <= 127)
bool sens_tc_supported(const DevProblem &P, int mode);
void launch_sens_tc(const DevProblem &P, const float2 *kpot32, double2 *sens, cudaStream_t st, int e_first,
                    int e_count);
// single: the complex64 contraction from kpot32 (mixed precision); else the
// complex128 one from kpot
void launch_bsens(const DevProblem &P, const double2 *kpot, const float2 *kpot32, const double2 *sigma,
                  const double2 *volt, int mode, bool single, double2 *sens, cudaStream_t st,
                  int e_first = 0, int e_count = -1);

// adjoint of the forward block (adjoint.cu)
void launch_adjoint_sources(const DevProblem &P, const double2 *g, double2 *src, int lsink, int nsink,
                            cudaStream_t st);
void launch_adjoint_rhs(const DevProblem &P, const DevBatch &B, int nrhs, const double2 *src, cudaStream_t st);
void launch_adjoint_lambda(const DevProblem &P, const DevBatch &B, int nrhs, double2 *lambda, cudaStream_t st);
void launch_adjoint_grad(const DevProblem &P, const double2 *kpot, const double2 *lambda, const int32_t *ebnd_ptr,
                         const int32_t *ebnd_list, double2 *grad, cudaStream_t st);

// model uncertainty and resolution (mcm.cu, src/bmcm_mod.f90); device
// inputs, host outputs (manz doubles each; diag_res / diag_cov2 only when
// wanted)
struct McmArgs {
    int nanz, manz, ltri, nx, nk;
    double lam;
    const double2 *sens;     // column-major (nanz, manz)
    const double *wmatd;     // nanz
    const int32_t *wdfak;    // nanz
    const double *smatm;     // column-major (manz, 3) or (manz, nk+1)
    const int32_t *nachbar;  // column-major (manz, nk+1)
    int want_res, want_cov2;
    double *diag_ata, *diag_reg, *diag_cov1, *diag_res, *diag_cov2;
};
// dense FP64 kernels (dense.cu), column-major: C (lower) = S^T S for S k x n;
// the Cholesky factor of A (n x n, lower, in place; info_dev: first
// non-positive pivot, 1-based, 0 if none); C (lower) = (L L^T)^-1 with work Y
// (n x n); d_j = sum_l (S C)_lj^2 for S m x n, with work (ceil(m/64) x n)
void dense_syrk_t(int n, int k, const double *S, int lds, double *C, cudaStream_t st);
void dense_potrf(int n, double *A, int *info_dev, cudaStream_t st);
void dense_potri(int n, const double *L, double *Y, double *C, cudaStream_t st);
void dense_col_sq_of_product(int m, int n, const double *S, int lds, const double *C, double *work, double *d,
                             cudaStream_t st);
int run_mcm(const McmArgs &a, cudaStream_t st, std::string &msg);
void launch_column_sums(int nanz, int manz, const double2 *sens, const double *wa, const double *wb,
                        const double *wc, double *c1, double *c2, double *c3, cudaStream_t st);

// v.y = 0 (DC: the real parts of the conductivities)
void launch_real_part(double2 *v, int n, cudaStream_t st);

// update / CG (src/update.f90, src/cg_mod.f90); all pointers device memory
struct CGArgs {
    int nanz, manz, ltri, nx, maxnk, ncgmax;
    double lam, eps, step;
    const double2 *sens;    // column-major (nanz, manz)
    const double *wmatd;    // nanz
    const int32_t *wdfak;   // nanz
    const double2 *dat, *sigmaa;
    const double *smatm;    // column-major (manz, 3) or (manz, maxnk+1)
    const int32_t *nachbar; // column-major (manz, maxnk+1)
    double2 *par, *dpar;    // in/out model, out update
    double *cgfac;          // out preconditioner
    double2 *work;          // update_work_bytes(nanz, manz)
    int part;               // 0 complex CG; real CG of cjggdc on Re(J): 1 the phases (final phase
                            // improvement, lfpi), 2 the real parts (DC, ldc)
};
size_t update_work_bytes(int nanz, int manz);
// runs update + cjggra; cgres (host, ncgmax+2 floats) receives the CG record
int run_update(const CGArgs &a, cudaStream_t st, int *ncg_out, float *cgres_host);
// |(J^H W J 1)_j| for the first regularisation parameter (src/blam0.f90); jtj_host: manz doubles
int run_jhwj1(CGArgs a, cudaStream_t st, double *jtj_host);

}  // namespace crgpu
