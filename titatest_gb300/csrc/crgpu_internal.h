// Internal declarations shared by the host and device translation units of
// libcrtomo_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "crtomo_gb300.h"

namespace crgpu {

enum : int {
    ERR_CUDA = 1000,
    ERR_ARG = 1001,
    ERR_UNSUPPORTED = 1002,
    ERR_TIMEOUT = 1003,  // a bounded device-side wait gave up
};

// ---------------------------------------------------------------------------
// Host-side description of the problem after validation (0-based indices).
// ---------------------------------------------------------------------------
struct HostGrid {
    int n = 0;        // sanz
    int mb = 0;       // band width
    int elanz = 0;    // area elements
    int relanz = 0;   // boundary elements (types 11, 12, 13)
    int nmixed = 0;   // boundary elements of type 11
    std::vector<double> x, y;       // node coordinates in node order
    std::vector<int32_t> etype;     // elanz (3, 5 or 8)
    std::vector<int32_t> enodes;    // elanz x 4 (0-based nodes, -1 padding)
    std::vector<int32_t> btype;     // relanz
    std::vector<int32_t> bnodes;    // relanz x 2
    std::vector<int32_t> brnr;      // relanz (0-based element)
    std::vector<uint8_t> dirichlet; // n: node on a type-13 boundary
    bool lbeta = false;             // mixed boundaries present
    bool lrandb = false;            // homogeneous Dirichlet boundaries present
};

// Lower-triangular sparsity pattern of the band matrix with the ordered list
// of element contributions of every entry (the summation order of
// src/kompab.f90:80-138: element order, area elements before boundary ones).
struct Pattern {
    int n = 0, nnz = 0, nnz_full = 0, rw = 1;
    std::vector<int32_t> rowptr, col, row;    // lower incl. diagonal, rows padded to rw (col -1)
    std::vector<int32_t> dom_ptr, dom_list;   // nnz+1, packed (element << 4) | imn
    std::vector<int32_t> bnd_ptr, bnd_list;   // nnz+1, packed (rel << 4) | imn
    std::vector<int32_t> fptr, fcol, fidx;    // full symmetric CSR -> lower index
};

int build_grid(const crgpu_grid *g, HostGrid &hg, std::string &msg);
int build_pattern(const HostGrid &hg, Pattern &pat, std::string &msg);
int host_rwaven(const HostGrid &hg, int eanz, const int32_t *enr, int nanz, const int32_t *strnr,
                const int32_t *vnr, double *kwn, double *kwnwi, int32_t *kwnanz);
int host_cutmck(int32_t sanz, int32_t typanz, const int32_t *typ, const int32_t *nelanz,
                const int32_t *selanz, int32_t *nrel, int32_t ld_nrel, int32_t *snr, int32_t eanz,
                int32_t *enr, int32_t *mb);
double host_sytop(const crgpu_grid *g);
int host_geometric_order(const HostGrid &hg, std::vector<int32_t> &old_of_new, std::vector<int32_t> &new_of_old);
void host_permute_grid(HostGrid &hg, const std::vector<int32_t> &old_of_new, const std::vector<int32_t> &new_of_old,
                       int mb);

}  // namespace crgpu
