/*
 * crtomo_gb300 -- C ABI of the GB300 (sm_103a) implementation of the
 * CRMod/CRTomo forward + sensitivity hot path.
 *
 * Every entry point replaces one reference routine (or one block of a
 * reference driver); the comment above each names it (paths relative to the
 * reference project root).  A Fortran host binds these with ISO_C_BINDING
 * (a module of BIND(C) interfaces, one per function below).
 *
 * Conventions
 *  - All array arguments are HOST pointers unless the name ends in _device.
 *  - Integer arrays keep the reference's 1-based numbering (node numbers in
 *    nrel/enr, element numbers in rnr, electrodes in strnr/vnr encoded as
 *    A*10000+B) and its Fortran column-major layout.
 *  - Complex values are interleaved (re, im) double pairs, i.e. Fortran
 *    COMPLEX(KIND(0D0)).
 *  - Every function returns 0 on success or the reference's error number
 *    (src/error.txt: 19 band width exceeded, 26 bad element geometry,
 *    27 zero diagonal, 28 zero pivot, 35 degenerate boundary element,
 *    73 duplicate electrodes, 82 zero voltage, 93 zero geometry factor,
 *    94/97 allocation, 101 mixed and Dirichlet boundaries together).
 *    Codes >= 1000 are this library's own (1000 CUDA error, 1001 bad
 *    argument, 1002 unsupported option, 1003 a bounded device-side wait
 *    gave up).  crgpu_last_error() gives the text
 *    (the reference's fetxt).
 *  - One context owns one CUDA stream; calls on one context must not overlap.
 */
#ifndef CRTOMO_GB300_H
#define CRTOMO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct crgpu_ctx crgpu_ctx;

/* FE grid as read by src/relem.f90 (module elemmod, src/elemmod.f90). */
typedef struct {
    int32_t sanz, typanz, mb;
    const int32_t *typ, *nelanz, *selanz; /* typanz each; boundary types (>10) last */
    const int32_t *snr;                   /* sanz: node -> coordinate index */
    const double *sx, *sy;                /* sanz */
    const int32_t *nrel;                  /* nrel(ld_nrel, maxnk), column-major */
    int32_t ld_nrel;                      /* elanz + relanz */
    const int32_t *rnr;                   /* relanz: boundary element -> element */
} crgpu_grid;

/* Electrodes, measurements and wavenumbers (src/electrmod.f90,
 * src/datmod.f90, src/wavenmod.f90) and the crmod.cfg switches. */
typedef struct {
    int32_t eanz;
    const int32_t *enr;      /* eanz: electrode node numbers */
    int32_t nanz;
    const int32_t *strnr;    /* nanz: current electrodes  A*10000+B */
    const int32_t *vnr;      /* nanz: voltage electrodes  M*10000+N */
    const double *strom;     /* nanz or NULL (unit current) */
    int32_t kwnanz;
    const double *kwn;       /* kwnanz wavenumbers (src/rwaven.f90) */
    const double *kwnwi;     /* kwnanz quadrature weights */
    int32_t swrtr;           /* 0: 2D (kwnanz = 1, kwn = 0), 1: 2.5D */
    int32_t lsr;             /* singularity removal, mswitch bit 2 */
    int32_t lsink, nsink;    /* fictitious sink node */
    int32_t lsytop;          /* image plane at mean Neumann-boundary y */
} crgpu_survey;

/* Precision of the factorisation. */
enum {
    CRGPU_PLAIN = 0, /* complex128 throughout (reference arithmetic) */
    CRGPU_MIXED = 1  /* complex64 factor + FP64 iterative refinement */
};

/* ------------------------------------------------------------------ */
/* set-up                                                               */
/* ------------------------------------------------------------------ */

/* Uploads grid and survey and computes the element matrices, the mixed-
 * boundary factors and the band pattern on the device.
 * Replaces src/precal.f90:13-222 (with src/elem1.f90, src/elem3.f90,
 * src/elem5.f90, src/elem8.f90, src/beta.f90, src/bessk0.f90,
 * src/bessk1.f90, src/bsytop.f90) and the allocations of src/fem.f90:314-327. */
int crgpu_create(const crgpu_grid *grid, const crgpu_survey *survey, int32_t precision,
                 crgpu_ctx **ctx);

/* crgpu_create with the choice of the complex64 factor's node order (no
 * counterpart in the reference, which factors in the cutmckee band):
 * band_order 0 keeps the grid's band; 1 (crgpu_create's default) lets a
 * CRGPU_MIXED context number its nodes by their coordinate along the mesh's
 * longer extent when that band is narrower than the grid's (for a grid band
 * too wide for the tensor-core window, mb > 124, only when the new band fits
 * it); 2 lets any context (either precision) factor in that order whenever
 * its band is narrower.  The refinement's FP64 residuals use the same matrix, so only the
 * preconditioner changes; potentials,
 * voltages and sensitivities come back in the grid's order and numbering.
 * Such a context returns 1002 from crgpu_factor_system and
 * crgpu_factor_system_noalloc; its device buffers
 * (crgpu_device_buffers) are in the order crgpu_node_order reports. */
int crgpu_create2(const crgpu_grid *grid, const crgpu_survey *survey, int32_t precision, int32_t band_order,
                  crgpu_ctx **ctx);

/* No counterpart in the reference.  grid_node[j] (1-based, sanz entries):
 * the grid node in position j of the context's device arrays (j + 1 unless
 * the context factors in the geometric order of crgpu_create2). */
int crgpu_node_order(const crgpu_ctx *ctx, int32_t *grid_node);

/* Frees the context and its device memory. */
int crgpu_destroy(crgpu_ctx *ctx);

/* Message of the last error on this context (the reference's fetxt). */
const char *crgpu_last_error(const crgpu_ctx *ctx);

/* Iterative refinement of the mixed mode: at most maxit corrections
 * (0 <= maxit <= 64, else 1001), stop a system when max|dx| <= tol * max|x|.
 * Defaults: 8, 1e-10.  The steps run without host synchronisation; a step
 * after the last system stopped returns at once. */
int crgpu_set_refinement(crgpu_ctx *ctx, int32_t maxit, double tol);

/* Stream the context's work is issued on (a cudaStream_t; NULL restores the
 * context's own stream).  The caller keeps the stream alive. */
int crgpu_set_stream(crgpu_ctx *ctx, void *stream);

/* Dirichlet boundary values (lrandb2 with the file read by src/rrandb.f90,
 * src/fem.f90:296-299): node rwdnr[i] (1-based, band numbering) is held at
 * the complex value (rwd[2i], rwd[2i+1]) by src/randb2.f90:1-82, applied
 * after src/randb.f90 in every system assembled by src/kompab.f90
 * (src/fem.f90:363).  Systems whose right-hand side src/kompb.f90 builds
 * (no mixed boundary, electrodes after the first) keep the rows and columns
 * eliminated with zero values, as the reference does.  rwdanz = 0 removes
 * the values.  A node outside 1..sanz returns 30. */
int crgpu_set_boundary_values(crgpu_ctx *ctx, int32_t rwdanz, const int32_t *rwdnr, const double *rwd);

/* DC mode (CRTomo ldc): the DC twins of the hot path (src/kompadc.f90,
 * src/scaldc.f90, src/choldc.f90, src/vredc.f90, src/bsendc.f90) on the
 * complex path: the real parts of sigma, an error 28 for a pivot <= 0
 * (src/choldc.f90:66-70, where src/chol.f90 stops only on 0), the real
 * voltage with a +0 imaginary part for -log V (src/bvolti.f90:56-62).  With
 * real conductivities every other complex operation of the path keeps its
 * imaginary parts 0, so the values are those of the real routines.
 * ldc: 0 or 1. */
int crgpu_set_dc(crgpu_ctx *ctx, int32_t ldc);

/* Upper bound of device memory for the per-system band factors; systems are
 * processed in batches that fit.  Default: 60% of free device memory. */
int crgpu_set_memory_budget(crgpu_ctx *ctx, int64_t bytes);

/* No counterpart in the reference.  Free and total memory of the current
 * device (cudaMemGetInfo), for hosts that size memory budgets. */
int crgpu_device_memory(int64_t *free_bytes, int64_t *total_bytes);

/* ------------------------------------------------------------------ */
/* forward modelling                                                    */
/* ------------------------------------------------------------------ */

/* Forward block of src/fem.f90:327-400 (== src/inv.f90:426-491): for every
 * wavenumber k and current electrode l: src/potana.f90 (if lsr),
 * src/kompab.f90 / src/kompb.f90, src/randb.f90, src/randb2.f90, src/scalab.f90,
 * src/chol.f90, src/vre.f90 and the unscaling into kpot; then
 * src/rtrafo.f90, then src/bvolt.f90 (volt_mode 0: sigmaa = kfak*V, kfak
 * may be NULL) or src/bvolti.f90 (volt_mode 1: sigmaa = -log V).
 *   sigma  : elanz complex (src/sigmamod.f90)
 *   kpot   : kpot(sanz, eanz, kwnanz) complex, or NULL
 *   hpot   : hpot(sanz, eanz) complex, or NULL
 *   volt, sigmaa : nanz complex (either may be NULL) */
int crgpu_forward(crgpu_ctx *ctx, const double *sigma, double *kpot, double *hpot,
                  int32_t volt_mode, const double *kfak, double *volt, double *sigmaa);

/* The same with every array in device memory (inputs resident in HBM). */
int crgpu_forward_device(crgpu_ctx *ctx, const void *sigma_device, int32_t volt_mode,
                         const void *kfak_device, void *volt_device, void *sigmaa_device);

/* Sensitivities of the last forward: src/bsens.f90:23-197 (mode 0, CRMod:
 * sens -= strom/pi * sum_k w_k ...) or src/bsensi.f90:23-194 (mode 1,
 * CRTomo: sens += sum_k w_k/pi ... * sigma_e / V_i).
 *   sens : sens(nanz, elanz) complex, column-major (src/alloci.f90)
 * Mode 0 into page-locked host memory is written by the kernel directly;
 * otherwise the device result is copied in chunks, overlapped with the
 * computation (mode 1 keeps the device copy for crgpu_update).  sens NULL:
 * the device copy only, nothing copied to the host. */
int crgpu_sens(crgpu_ctx *ctx, int32_t mode, double *sens);
int crgpu_sens_device(crgpu_ctx *ctx, int32_t mode, void *sens_device);

/* Several problems at once (uneven meshes; no single counterpart in the
 * reference, which runs one mesh per CRMod call: src/fem.f90:327-470 for each).
 * The forward of every context (sigma[p] host, elanz complex), its voltages
 * into volt[p] (host, nanz complex: V for volt_mode 0, the CRTomo data for
 * 1) and, for sens_mode 0 or 1, its Jacobian kept on the device (as
 * crgpu_sens(ctx, mode, NULL)); sens_mode -1: none.  The band factors of all
 * problems' systems run in one persistent tensor-core launch over a table of
 * (problem, system) items, longest systems first; assembly and the solves run
 * on each context's own stream.  Every context must be CRGPU_MIXED with a band
 * that fits the tensor-core window (as created; see crgpu_create2), without
 * singularity removal, DC mode or boundary values, and its systems must fit
 * one batch in device memory (crgpu_memory_need); else 1002 or a CUDA error. */
int crgpu_forward_sens_batch(crgpu_ctx *const *ctxs, int32_t nprob, const double *const *sigma, int32_t volt_mode,
                             double *const *volt, int32_t sens_mode);

/* No counterpart in the reference.  Device memory a forward + Jacobian of
 * this context still has to allocate (its batch of all systems and the
 * Jacobian), for hosts that group problems to fit. */
int crgpu_memory_need(const crgpu_ctx *ctx, int64_t *bytes);

/* Device buffers of the last forward (valid until the next call):
 * kpot(sanz, eanz, kwnanz), hpot(sanz, eanz), fak per system. */
int crgpu_device_buffers(crgpu_ctx *ctx, void **kpot_device, void **hpot_device);

/* Band factor of one system (k, l) (1-based) as src/chol.f90 leaves it in
 * a((mb+1)*sanz) -- complex128 even in the mixed mode (converted) -- and the
 * scaling vector fak(sanz) of src/scalab.f90.  Recomputes that system. */
int crgpu_factor_system(crgpu_ctx *ctx, const double *sigma, int32_t k, int32_t l,
                        double *a, double *fak);

/* No counterpart in the reference.  The same band factor and fak as
 * crgpu_factor_system (plain precision, non-DC contexts only), for callers
 * that cannot allocate device memory when they call: a host framework that
 * hands out all device memory from its own pool, or a host that must not
 * make the implicit device-wide synchronisation of cudaMalloc/cudaFree in the
 * middle of its work.  sigma_device (elanz complex), a_device
 * (sanz*(mb+1) complex) and fak_device (sanz) are caller-owned device
 * buffers; stream may be NULL (the context's stream).  The call allocates
 * nothing: its scratch, error word included, is one fixed 8 MiB device array
 * in the library (held on every GPU that loads it until exit); systems
 * needing more (16 + 32*(nnz + sanz) bytes) are rejected with 1001.  The
 * first call on a device looks the array up (cudaGetSymbolAddress) and
 * should come before any stream capture.  Every call shares the array, which
 * keeps the last call's contents: calls that overlap on the GPU race.  The
 * call waits for its kernels on `stream` and returns their status. */
int crgpu_factor_system_noalloc(crgpu_ctx *ctx, const void *sigma_device, int32_t k, int32_t l,
                                void *a_device, void *fak_device, void *stream);

/* No single counterpart in the reference, which forms the Jacobian with
 * src/bsensi.f90 (reciprocity, no mixed-boundary term) and applies J^H in
 * src/update.f90.  The exact derivative of L = sum_i g_i V_i, the voltages
 * of the last crgpu_forward (V of src/bvolt.f90, before kfak or log), with
 * respect to sigma: one adjoint solve per (k, l) system that reuses the
 * forward's band factors (refactored batch by batch when the systems did not
 * fit in one batch) and an element-wise contraction with the element and
 * mixed-boundary matrices.  V is holomorphic in sigma, so grad_e =
 * sum_i g_i dV_i/dsigma_e.  Not available with singularity removal (1002).
 *   g    : nanz complex;  grad : elanz complex */
int crgpu_adjoint(crgpu_ctx *ctx, const double *g, double *grad);
int crgpu_adjoint_device(crgpu_ctx *ctx, const void *g_device, void *grad_device);

/* ------------------------------------------------------------------ */
/* inversion update                                                     */
/* ------------------------------------------------------------------ */

/* src/update.f90:27-353 with the complex PCG of src/cg_mod.f90:426-726
 * (cjggra, bap, bp / bptri, bb) on the sensitivities of the last
 * crgpu_sens(ctx, 1, ...) call.
 *   ltri  : 0 structured smoothness (smatm(manz,3), nx) or 1/2 triangular
 *           (smatm(manz,maxnk+1) over nachbar(manz,maxnk+1))
 *   par   : in/out model (log sigma), manz complex
 *   dpar  : out update, manz complex;  cgfac : out, manz
 *   cgres : out, ncgmax+2 floats (cgres(1) = number of CG steps)
 * Returns the error code; *ncg receives the number of CG steps. */
int crgpu_update(crgpu_ctx *ctx, const double *wmatd, const int32_t *wdfak, const double *dat,
                 const double *sigmaa, int32_t ltri, const double *smatm, int32_t nx,
                 const int32_t *nachbar, double lam, double eps, int32_t ncgmax, double step,
                 double *par, double *dpar, double *cgfac, float *cgres, int32_t *ncg);

/* The same update in the final phase improvement (lfpi of src/update.f90 and
 * src/cg_mod.f90): preconditioner and right-hand side from Re(J), the real
 * CG of cjggdc (src/cg_mod.f90:136-400) on the imaginary part of the
 * right-hand side, and the update i cgfac o dpar in the phases only. */
int crgpu_update_fpi(crgpu_ctx *ctx, const double *wmatd, const int32_t *wdfak, const double *dat,
                     const double *sigmaa, int32_t ltri, const double *smatm, int32_t nx,
                     const int32_t *nachbar, double lam, double eps, int32_t ncgmax, double step,
                     double *par, double *dpar, double *cgfac, float *cgres, int32_t *ncg);

/* The same for DC inversion (ldc, src/update.f90 with sensdc and cjggdc):
 * the real CG on the real part of the right-hand side; the update real. */
int crgpu_update_dc(crgpu_ctx *ctx, const double *wmatd, const int32_t *wdfak, const double *dat,
                    const double *sigmaa, int32_t ltri, const double *smatm, int32_t nx,
                    const int32_t *nachbar, double lam, double eps, int32_t ncgmax, double step,
                    double *par, double *dpar, double *cgfac, float *cgres, int32_t *ncg);

/* The column sums of src/blam0.f90:60-130 for the first regularisation
 * parameter: jtj[j] = |sum_i sum_k conj(J_ij) J_ik w_i| (w_i = wmatd_i
 * wdfak_i; phase_only: Re(J), the final phase improvement) on the
 * sensitivities of the last crgpu_sens(ctx, 1, ...), computed as two
 * products with J (J 1, then J^H W (J 1)).  lam_0 = 5 sum_j jtj[j] / manz *
 * 2 / (alfx + alfz).  jtj: manz doubles. */
int crgpu_blam0_jtj(crgpu_ctx *ctx, const double *wmatd, const int32_t *wdfak, int32_t phase_only,
                    double *jtj);

/* Model uncertainty and resolution of src/bmcm_mod.f90 (buncert) on the
 * sensitivities of the last crgpu_sens(ctx, 1, ...):
 *   ata = Re(J^H W J) (bata), ata_reg = ata + lam R (bata_reg; ltri 1, 2 as
 *   the reference builds it; ltri 0 the 5-point stencil of src/update.f90),
 *   cov = ata_reg^-1 (bmcm, Cholesky), res = cov ata (bres, flags bit 0),
 *   cov2 = cov ata cov (bmcm2, flags bits 0 and 1).
 * Outputs the diagonals, manz doubles each (diag_res / diag_cov2 may be NULL
 * when not asked for).  A non positive definite ata_reg returns 108. */
int crgpu_mcm(crgpu_ctx *ctx, const double *wmatd, const int32_t *wdfak, int32_t ltri, const double *smatm,
              int32_t nx, const int32_t *nachbar, double lam, int32_t flags, double *diag_ata,
              double *diag_reg, double *diag_cov1, double *diag_res, double *diag_cov2);

/* Column sums of the sensitivities for the coverage (src/bbsens.f90) and
 * the FPI diagonal of bata: c1_j = sum_i |J_ij| wa_i, c2_j = sum_i
 * |Re J_ij| wb_i, c3_j = sum_i Re(J_ij)^2 wc_i (nanz weights in, manz sums
 * out). */
int crgpu_column_sums(crgpu_ctx *ctx, const double *wa, const double *wb, const double *wc, double *c1,
                      double *c2, double *c3);

/* ------------------------------------------------------------------ */
/* host-side set-up routines                                            */
/* ------------------------------------------------------------------ */

/* src/rwaven.f90:22-171 with the Gauss-Legendre / Gauss-Laguerre rules of
 * src/gauleg.f90 and src/gaulag.f90.  kwn, kwnwi: room for 30. */
int crgpu_rwaven(const crgpu_grid *grid, int32_t eanz, const int32_t *enr, int32_t nanz,
                 const int32_t *strnr, const int32_t *vnr, double *kwn, double *kwnwi,
                 int32_t *kwnanz);

/* Cuthill-McKee renumbering of cutmckee/cutmck.f:125-337: renumbers nrel,
 * snr and enr in place and returns the band width in *mb. */
int crgpu_cutmck(int32_t sanz, int32_t typanz, const int32_t *typ, const int32_t *nelanz,
                 const int32_t *selanz, int32_t *nrel, int32_t ld_nrel, int32_t *snr,
                 int32_t eanz, int32_t *enr, int32_t *mb);

/* Geometric factors of src/bkfak.f90:7-149 (kfak(nanz)). */
int crgpu_bkfak(const crgpu_grid *grid, const crgpu_survey *survey, double *kfak);

/* Counters of the last call: kernels launched, device time (ms) of the
 * forward, factorisation, solve, sensitivity and update phases, refinement
 * steps taken and the largest relative correction max|dx|/max|x| of the
 * last refinement step. */
typedef struct {
    int64_t kernel_launches;
    double ms_forward, ms_factor, ms_solve, ms_sens, ms_update;
    int32_t refine_iterations;
    int32_t nsystems, nbatches;
    double refine_last_correction;
    double ms_adjoint;
} crgpu_stats;
int crgpu_get_stats(const crgpu_ctx *ctx, crgpu_stats *stats);

/* Forward (crgpu_forward_device, volt_mode 0) and Jacobian
 * (crgpu_sens_device) of device buffers as one CUDA graph: the first call,
 * and any call after the buffers, the mode or the context's settings
 * changed, runs them as usual and records the kernel sequence; later calls
 * with the same buffers replay it (one launch) and check for errors.
 * Problems whose systems need several batches run the ordinary path. */
int crgpu_forward_sens_graph(crgpu_ctx *ctx, const void *sigma_device, void *volt_device, int32_t mode,
                             void *sens_device);

/* Autotuner (mixed precision): times the band-factor kernels that can run
 * this problem (one warp per system; tensor cores; SIMT register tiles at
 * 1, 2 and 4 blocks per SM; SIMT shared-memory tiles) on its first batch of
 * systems, and the two
 * CRMod Jacobian kernels (tensor-core Gram form, SIMT direct form), for the
 * conductivities sigma (elanz complex, host), and keeps the fastest for
 * this context.  Choices are cached for the process by problem shape (n, mb,
 * systems, electrodes, measurements, wavenumbers, SMs); flags & 1 re-times.
 * Complex128 contexts return 0 without timing.  Leaves a forward done. */
int crgpu_autotune(crgpu_ctx *ctx, const double *sigma, int32_t flags);

/* The context's launch choices: out[0] factor kernel (0 default, 1 tensor
 * cores, 2 SIMT register tiles, 3 SIMT shared-memory tiles, 4 one warp per
 * system with the window in its registers, mb <= 63), out[1] SIMT
 * blocks per SM (0 default), out[2] CRMod Jacobian (0 default, 1 tensor
 * cores, 2 SIMT). */
int crgpu_get_tune(const crgpu_ctx *ctx, int32_t *out);

/* Sets the launch choices in the layout of crgpu_get_tune (a kernel that
 * cannot run this problem falls back to the default); blocks per SM 0..8. */
int crgpu_set_tune(crgpu_ctx *ctx, const int32_t *in);

#ifdef __cplusplus
}
#endif
#endif
