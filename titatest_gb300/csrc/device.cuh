// Device-side problem description shared by the kernels.
#pragma once

#include <cstdint>

#include "cplx.cuh"

namespace crgpu {

struct DevProblem {
    int n, mb, W, elanz, relanz, eanz, nanz, K, nnz, nnz_full;
    int rw;               // padded row width of the lower pattern (row i at i*rw)
    int swrtr;
    int lsr;              // singularity removal
    int ldc;              // DC (src/kompadc.f90 ... src/bsendc.f90): Re(sigma), pivots > 0 (src/choldc.f90)
    // launch choices of the autotuner (0: the built-in default)
    int tune_factor;      // mixed factor: 1 tensor cores, 2 SIMT register tiles, 3 SIMT shared-memory tiles,
                          // 4 one warp per system (mb <= 63)
    int tune_ctas;        // SIMT factor: blocks per SM
    int tune_sens;        // mixed CRMod Jacobian: 1 tensor cores (Gram form), 2 SIMT (direct form)
    double sytop;
    const double *earea;  // elanz: element areas of src/refsig.f90
    // grid (node order, 0-based)
    const double *x, *y;
    const int32_t *etype, *enodes;          // elanz, elanz*4
    const int32_t *btype, *bnodes, *brnr;   // relanz, relanz*2, relanz
    const uint8_t *dirichlet;               // n: 1 type-13 node (src/randb.f90), 2 valued node (src/randb2.f90)
    // valued Dirichlet nodes (src/randb2.f90), when lrandb2: rwd_b[i] the value
    // whose negative becomes b(i); rwd_col[i] the value whose column is moved to
    // the other rows' right-hand sides (0 where that column was already removed)
    int lrandb2;
    const double2 *rwd_b, *rwd_col;         // n, n
    // band pattern
    const int32_t *rowptr, *col, *row;
    const int32_t *dom_ptr, *dom_list, *bnd_ptr, *bnd_list;
    const int32_t *fptr, *fcol, *fidx;
    // survey
    const int32_t *enr0;   // eanz: electrode -> node (0-based)
    const int32_t *meas;   // nanz*4: electrodes e1,e2,e3,e4 (0-based, -1 = none)
    const double *strom;   // nanz
    const double *kwn, *kwnwi;
    // element matrices (src/precal.f90)
    double *elbg;          // [K][elanz][10]
    double *relbg;         // [relanz][3]
    double *kg;            // [K][eanz][relanz]
    int *err;              // first error code raised on the device
};

// Batch of band systems: system s solves wavenumber ks[s], electrode ls[s].
struct DevBatch {
    int nsys;
    const int32_t *ks, *ls;
    double2 *As;      // [nsys][nnz]   scaled lower-pattern values (FP64)
    double *fak;      // [nsys][n]     scaling factors of src/scalab.f90
    double2 *b;       // [nsys][n]     scaled right-hand side (FP64)
    double2 *x;       // [nsys][n]     solution of A x = b (FP64)
    double2 *r;       // [nsys][n]     residual / work (FP64)
    void *L;          // [nsys][lpitch] band factor (complex128 or complex64), row i at i*(mb+1)
    size_t lpitch;    // elements of L's type between systems: n*(mb+1) rounded up to even, + 2,
                      // so every system starts 16-byte aligned and a block copy rounded up to
                      // 16 bytes stays inside its own system
    void *y;          // [nsys][n]     forward-substitution vector (L's type)
    int *status;      // [nsys]        0 or reference error code
    int *active;      // [nsys]        refinement still running
    int *nactive;     // count of items still refining after the last correction
    const int *nprev; // that count after the previous refinement step (0: the step's kernels return at once)
    double *zmax;     // largest relative correction of the last refinement step
    double2 *pota;    // [nsys][n] analytic potentials (singularity removal)
    double *potmax;   // [nsys]
};

}  // namespace crgpu
