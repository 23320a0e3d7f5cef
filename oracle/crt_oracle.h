/*
 * CPU oracle for the CRMod/CRTomo forward + sensitivity hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Fortran routines, written to check the CUDA implementation.  Only the test
 * suite, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
 * load it.  The product library (titatest_gb300) never links or calls it.
 *
 * Every function follows the loop order and the operation order of the
 * reference routine named in its comment (paths are relative to the
 * reference project root).
 *
 * Index conventions are the reference's: node, element, electrode and
 * boundary-element numbers stored in the integer arrays are 1-based.
 * Two-dimensional Fortran arrays are passed in Fortran column-major order:
 *   nrel(iel, m)        -> nrel[(m-1)*ld_nrel + (iel-1)]
 *   kpot(j, l, k)       -> kpot[((k-1)*eanz + (l-1))*sanz + (j-1)]
 *   hpot(j, l)          -> hpot[(l-1)*sanz + (j-1)]
 *   sens(i, m)          -> sens[(m-1)*nanz + (i-1)]
 * Complex values are interleaved (re, im) pairs of double.
 */
#ifndef CRT_ORACLE_H
#define CRT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    /* mesh (src/elemmod.f90) */
    int sanz, typanz, mb;
    const int *typ, *nelanz, *selanz;  /* typanz */
    const int *snr;                    /* sanz   */
    const double *sx, *sy;             /* sanz   */
    const int *nrel;                   /* ld_nrel x maxnk, column-major */
    int ld_nrel;                       /* = elanz + relanz */
    const int *rnr;                    /* relanz */
    /* electrodes and measurements (src/electrmod.f90, src/datmod.f90) */
    int eanz;
    const int *enr;                    /* eanz */
    int nanz;
    const int *strnr, *vnr;            /* nanz */
    const double *strom;               /* nanz */
} or_mesh;

typedef struct {
    int swrtr;      /* 0 = 2D, 1 = 2.5D with wavenumber back-transform */
    int lsr;        /* singularity removal (mswitch bit 2) */
    int lana;       /* analytic only (mswitch bit 0) */
    int lsink;      /* fictitious sink */
    int nsink;      /* sink node */
    int lsytop;     /* use mean y of Neumann boundary as the image plane */
    int nthreads;   /* OpenMP threads (<=0: leave default) */
    int rwdanz;     /* Dirichlet boundary values of src/randb2.f90 (lrandb2); 0: none */
    const int *rwdnr;   /* rwdanz node numbers, 1-based */
    const double *rwd;  /* rwdanz complex values (re, im pairs) */
    int ldc;            /* DC twins (src/kompadc.f90 ... src/choldc.f90): Re(sigma), pivots > 0 */
} or_opts;

/* derived mesh counts */
int or_counts(const or_mesh *m, int *elanz, int *relanz, int *maxnk);

/* src/rwaven.f90:22-171 -> returns kwnanz (<=30) or -errnr */
int or_rwaven(const or_mesh *m, double *kwn, double *kwnwi);

/* src/refsig.f90 */
void or_refsig(const or_mesh *m, const double *sigma, double *sigma0);

/* src/bsytop.f90 */
double or_bsytop(const or_mesh *m);

/* src/precal.f90 -> elbg[(imn-1)*elanz + iel-1 + k*elanz*10] as in the
 * Fortran elbg(elanz, 10, kwnanz); relbg(relanz, 10); kg(relanz, eanz, kwnanz).
 * Returns errnr; *lbeta set. */
int or_precal(const or_mesh *m, int kwnanz, const double *kwn, double sytop,
              double *elbg, double *relbg, double *kg, int *lbeta, int *lrandb);

/* Forward block of src/fem.f90:327-397: kpot(sanz, eanz, kwnanz).
 * Returns errnr. */
int or_forward(const or_mesh *m, const or_opts *o, int kwnanz,
               const double *kwn, const double *kwnwi,
               const double *sigma, double *kpot);

/* The same for a subset of (k, l) pairs (CPU baseline sampling): solves
 * npairs systems, pairs[2*p] = k (1-based), pairs[2*p+1] = l (1-based),
 * writing kpot for those pairs only.  Returns errnr. */
int or_forward_pairs(const or_mesh *m, const or_opts *o, int kwnanz,
                     const double *kwn, const double *kwnwi,
                     const double *sigma, int npairs, const int *pairs,
                     double *kpot);

/* one system (k, l), 1-based: kompab + randb + randb2 + scalab + chol; a_out has
 * (mb+1)*sanz complex entries, fak_out sanz.  Returns errnr. */
int or_factor(const or_mesh *m, const or_opts *o, int kwnanz, const double *kwn,
              const double *sigma, int k, int l, double *a_out, double *fak_out);

/* src/rtrafo.f90 : hpot(sanz, eanz) */
void or_rtrafo(const or_mesh *m, int swrtr, int kwnanz, const double *kwnwi,
               const double *kpot, double *hpot);

/* src/bkfak.f90 ; returns errnr */
int or_bkfak(const or_mesh *m, double *kfak);

/* src/bvolt.f90 (mode 0: sigmaa = kfak*V) and src/bvolti.f90 (mode 1:
 * sigmaa = -log V; mode 2: DC, V = dcmplx(Re V)).  kfak may be NULL (= 1).
 * Returns errnr. */
int or_bvolt(const or_mesh *m, int mode, const double *hpot, const double *kfak,
             double *volt, double *sigmaa);

/* precal element matrices only: elbg(elanz, 10, kwnanz) */
int or_elbg(const or_mesh *m, int kwnanz, const double *kwn, double sytop,
            double *elbg);

/* precal outputs: flags[0] = lbeta, flags[1] = lrandb */
int or_precal_all(const or_mesh *m, int kwnanz, const double *kwn, double sytop,
                  double *elbg, double *relbg, double *kg, int *flags);

/* src/bsens.f90:23-197 (mode 0, CRMod: sens -= strom/pi * ...) and
 * src/bsensi.f90:23-194 (mode 1, CRTomo: sens += ... * sigma/V):
 * sens(nanz, manz) with mnr = identity. */
void or_bsens_elbg(const or_mesh *m, const or_opts *o, int mode, int swrtr,
                   int kwnanz, const double *kwnwi, const double *elbg,
                   const double *kpot, const double *sigma, const double *volt,
                   double *sens);

/* A&S 9.8.5 - 9.8.8 (src/bessk0.f90, src/bessk1.f90) */
double or_bessk0(double x);
double or_bessk1(double x);

/* src/potana.f90 : pota(sanz) for electrode l, wavenumber kwn */
void or_potana(const or_mesh *m, int l, double kwn, const double *sigma0,
               double *pota);

/* cutmckee/cutmck.f:125-337.  nrel (in/out, renumbered), snr (in/out),
 * enr (in/out); returns the new band width or -errnr. */
int or_cutmck(int sanz, int typanz, const int *typ, const int *nelanz,
              const int *selanz, int *nrel, int ld_nrel, int *snr, int eanz,
              int *enr);

/* src/bnachbar.f90 : nachbar(manz, maxnk+1) column-major */
void or_bnachbar(const or_mesh *m, int *nachbar);

/* src/bsmatm_mod.f90:190-362 (ltri = 0): smatm(manz, 3) */
void or_bsmatmreg(const or_mesh *m, int nx, int nz, double alfx, double alfz,
                  double *smatm);

/* src/bsmatm_mod.f90:364-460 (ltri = 1, 2): smatm(manz, maxnk+1) */
void or_bsmatmtri(const or_mesh *m, const int *nachbar, double alfx,
                  double alfz, double *smatm);

/* src/update.f90:27-353 with src/cg_mod.f90 cjggra (complex, no prior, no
 * reference model, no difference inversion).  par (in/out), dpar (out),
 * cgres (out, ncgmax+2 floats).  Returns ncg. */
int or_update(int nanz, int manz, const double *sens, const double *wmatd,
              const int *wdfak, const double *dat, const double *sigmaa,
              int ltri, const double *smatm, int nx, const int *nachbar,
              int maxnk, double lam, double eps, int ncgmax, double step,
              double *par, double *dpar, double *cgfac, float *cgres);

/* src/bmcm_mod.f90 buncert (bata, bata_reg, bmcm, bres, bmcm2) on a host
 * Jacobian: the diagonals of ata, ata_reg, cov, cov ata and cov ata cov
 * (d_res / d_cov2 may be NULL).  Returns 108 if ata_reg is not positive
 * definite. */
int or_mcm(int nanz, int manz, const double *sens, const double *wmatd, const int *wdfak, int ltri,
           const double *smatm, int nx, const int *nachbar, int maxnk, double lam, double *d_ata,
           double *d_reg, double *d_cov1, double *d_res, double *d_cov2);

/* the same in the final phase improvement (lfpi; cjggdc on Re(J)); and for
 * DC inversion (ldc; cjggdc on Re(J) and Re(bvec)) */
int or_update_dc(int nanz, int manz, const double *sens, const double *wmatd,
                 const int *wdfak, const double *dat, const double *sigmaa,
                 int ltri, const double *smatm, int nx, const int *nachbar,
                 int maxnk, double lam, double eps, int ncgmax, double step,
                 double *par, double *dpar, double *cgfac, float *cgres);
int or_update_fpi(int nanz, int manz, const double *sens, const double *wmatd,
                  const int *wdfak, const double *dat, const double *sigmaa,
                  int ltri, const double *smatm, int nx, const int *nachbar,
                  int maxnk, double lam, double eps, int ncgmax, double step,
                  double *par, double *dpar, double *cgfac, float *cgres);

#ifdef __cplusplus
}
#endif
#endif
