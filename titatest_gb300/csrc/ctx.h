// Definition of the context behind the opaque crgpu_ctx handle, shared by
// the translation units of the C ABI.
#pragma once

#include <string>
#include <vector>

#include "crgpu_internal.h"
#include "kernels.h"

struct crgpu_ctx {
    // everything below is owned by the context
    crgpu::HostGrid hg;
    // node order of the device arrays when the complex64 factor runs on a
    // narrower geometric band (empty: the grid's own order)
    std::vector<int32_t> old_of_new, new_of_old;
    crgpu::Pattern pat;
    crgpu::DevProblem P{};
    int precision = CRGPU_PLAIN;
    int eanz = 0, nanz = 0, K = 0;
    int swrtr = 1, lsr = 0, lsink = 0, nsink = -1, lsytop = 0;
    cudaStream_t st = nullptr, own_st = nullptr;
    cudaStream_t copy_st = nullptr;  // device -> host copies overlapped with compute
    cudaStream_t st_hi = nullptr;    // high priority: the last, partial round of factors and its solves
    cudaEvent_t ev_join = nullptr;
    int nsm = 0, device = 0;
    std::vector<void *> allocs;
    // device state
    double2 *d_sigma = nullptr, *d_adom = nullptr, *d_kpot = nullptr, *d_hpot = nullptr;
    double2 *d_volt = nullptr, *d_sigmaa = nullptr, *d_sens = nullptr;
    float2 *d_kpot32 = nullptr;  // kpot as complex64 hi and lo planes (mixed precision: the Jacobian's input)
    double *d_kfak = nullptr;
    double2 *d_rwd = nullptr;     // [2][n] valued Dirichlet nodes: b values, moved-column values
    double2 *d_sigma0 = nullptr;  // reference conductivity (singularity removal)
    int *d_err = nullptr;
    // batch buffers
    int batch_cap = 0, nrhs = 1;
    crgpu::DevBatch Bmax{};
    int32_t *d_ks = nullptr, *d_ls = nullptr;
    std::vector<int32_t> sys_k, sys_l;
    // options
    int refine_maxit = 8;
    double refine_tol = 1e-10;
    // refinement step counters on the device, one array per sub-batch of the
    // current batch: {active count, pad, largest relative correction} per step
    void *d_refine = nullptr;
    int refine_used[2] = {};  // steps launched on each array since the last collection
    // forward + Jacobian as one CUDA graph (crgpu_forward_sens_graph)
    bool capturing = false;       // recording: no host copies, synchronisation or timing
    cudaGraphExec_t graph = nullptr;
    const void *graph_key[3] = {nullptr, nullptr, nullptr};  // sigma, volt, sens of the recorded graph
    int graph_mode = -1;
    int graph_refine_used[2] = {};  // refinement steps recorded in the graph per counter array
    int64_t mem_budget = 0;
    bool have_forward = false;
    bool factors_resident = false;  // band factors of every system still in Bmax (one batch)
    // adjoint
    double2 *d_lambda = nullptr, *d_adjsrc = nullptr, *d_adjg = nullptr, *d_adjgrad = nullptr;
    const int32_t *d_ebnd_ptr = nullptr, *d_ebnd_list = nullptr;  // element -> mixed boundary elements
    std::string last_error;
    crgpu_stats stats{};
    // update work space and the sensitivities it uses
    void *d_upd = nullptr;
    size_t upd_bytes = 0;
    const double2 *last_sens = nullptr;
};

