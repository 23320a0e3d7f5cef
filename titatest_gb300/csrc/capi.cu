// C ABI of libcrtomo_gb300 (include/crtomo_gb300.h): context management and
// the orchestration of the forward block (src/fem.f90:327-400), the
// sensitivities (src/bsens.f90, src/bsensi.f90) and the model update
// (src/update.f90).
#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"

using namespace crgpu;

namespace {

// counters of one refinement step (written by k_accumulate)
struct RefineCount {
    int n;     // items still refining after the step
    int pad;
    double z;  // largest relative correction of the step
};
constexpr int kRefineCap = 64;  // refinement steps at most (crgpu_set_refinement)
constexpr int kRefineSlots = 2;  // counter arrays: the full rounds' solves and the last round's

int fail(crgpu_ctx *c, int code, const std::string &msg) {
    if (c) c->last_error = msg;
    return code;
}

#define CUCHECK(c, call)                                                              \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return fail(c, ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int dalloc(crgpu_ctx *c, T **p, size_t count) {
    void *q = nullptr;
    if (count == 0) count = 1;
    // stream-ordered: no device-wide synchronisation on free, so contexts on
    // different streams (ensembles) do not serialise each other
    cudaError_t e = cudaMallocAsync(&q, count * sizeof(T), c->st);
    if (e != cudaSuccess) return fail(c, 94, std::string("device allocation: ") + cudaGetErrorString(e));
    c->allocs.push_back(q);
    *p = (T *)q;
    return 0;
}

template <typename T>
int upload(crgpu_ctx *c, const T **dst, const std::vector<T> &v) {
    T *p = nullptr;
    int e = dalloc(c, &p, std::max<size_t>(v.size(), 1));
    if (e) return e;
    if (!v.empty()) {
        cudaError_t ce = cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->st);
        if (ce != cudaSuccess) return fail(c, ERR_CUDA, cudaGetErrorString(ce));
    }
    *dst = p;
    return 0;
}

// The contexts allocate from the device's default stream-ordered pool.  With
// its default release threshold (0) every synchronisation hands freed memory
// back to the driver, which made creating and destroying many contexts (an
// ensemble of meshes) cost ~10 ms each; freed memory is kept for reuse
// instead (it stays reserved by the process).
void keep_pool_memory(int dev) {
    static std::once_flag once;
    std::call_once(once, [dev] {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    });
}

// the recorded forward + Jacobian graph refers to the batch buffers and the
// launch choices: dropped when either changes
void drop_graph(crgpu_ctx *c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_mode = -1;
}

void free_batch(crgpu_ctx *c) {
    drop_graph(c);
    void *ptrs[] = {c->Bmax.As, c->Bmax.fak, c->Bmax.b, c->Bmax.x, c->Bmax.r, c->Bmax.L, c->Bmax.y,
                    c->Bmax.status, c->Bmax.active, c->Bmax.pota, c->Bmax.potmax, c->d_ks, c->d_ls};
    for (void *p : ptrs)
        if (p) {
            cudaFreeAsync(p, c->st);
            c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), p), c->allocs.end());
        }
    c->Bmax = DevBatch{};
    c->d_ks = c->d_ls = nullptr;
    c->batch_cap = 0;
}

// elements between the band factors of consecutive systems (see DevBatch)
size_t lpitch_of(size_t n, size_t W) { return ((n * W + 1) & ~(size_t)1) + 2; }

size_t bytes_per_system(const crgpu_ctx *c) {
    const size_t n = c->hg.n, W = c->hg.mb + 1, nnz = c->pat.nnz, nr = c->nrhs;
    size_t esz = c->precision == CRGPU_MIXED ? sizeof(float2) : sizeof(double2);
    return lpitch_of(n, W) * esz + nnz * sizeof(double2) + n * sizeof(double) +
           nr * n * (3 * sizeof(double2) + esz) + 64;
}

int ensure_batch(crgpu_ctx *c, int want) {
    if (c->batch_cap >= want) return 0;
    free_batch(c);
    const size_t n = c->hg.n, W = c->hg.mb + 1, nnz = c->pat.nnz, nr = c->nrhs;
    size_t esz = c->precision == CRGPU_MIXED ? sizeof(float2) : sizeof(double2);
    DevBatch &B = c->Bmax;
    int e = 0;
    e = e ? e : dalloc(c, &B.As, (size_t)want * nnz);
    e = e ? e : dalloc(c, &B.fak, (size_t)want * n);
    e = e ? e : dalloc(c, &B.b, (size_t)want * nr * n);
    e = e ? e : dalloc(c, &B.x, (size_t)want * nr * n);
    e = e ? e : dalloc(c, &B.r, (size_t)want * nr * n);
    char *L = nullptr, *y = nullptr;
    e = e ? e : dalloc(c, &L, (size_t)want * lpitch_of(n, W) * esz);
    e = e ? e : dalloc(c, &y, (size_t)want * nr * n * esz);
    e = e ? e : dalloc(c, &B.status, (size_t)want);
    e = e ? e : dalloc(c, &B.active, (size_t)want * nr);
    if (!e && !c->d_refine) {
        char *cnt = nullptr;  // [kRefineSlots][kRefineCap] steps of {int count, pad, double zmax}
        e = dalloc(c, &cnt, kRefineSlots * kRefineCap * sizeof(RefineCount));
        c->d_refine = cnt;
    }
    e = e ? e : dalloc(c, &c->d_ks, (size_t)want);
    e = e ? e : dalloc(c, &c->d_ls, (size_t)want);
    if (!e && c->lsr) {
        e = dalloc(c, &B.pota, (size_t)want * n);
        e = e ? e : dalloc(c, &B.potmax, (size_t)want);
    }
    if (e) return e;
    B.L = L;
    B.lpitch = lpitch_of(n, W);
    B.y = y;
    c->batch_cap = want;
    return 0;
}

int check_device_errors(crgpu_ctx *c, const int *d_status, int nsys) {
    int h_err = 0;
    CUCHECK(c, cudaMemcpyAsync(&h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    std::vector<int> st(nsys > 0 ? nsys : 0);
    if (nsys > 0) CUCHECK(c, cudaMemcpyAsync(st.data(), d_status, sizeof(int) * nsys, cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaStreamSynchronize(c->st));
    if (h_err) return fail(c, h_err, "device reported error " + std::to_string(h_err));
    for (int s = 0; s < nsys; s++)
        if (st[s]) {
            int k = c->sys_k.empty() ? 0 : c->sys_k[s];
            return fail(c, st[s], "system (k=" + std::to_string(k + 1) + ") failed with error " +
                                      std::to_string(st[s]));
        }
    return 0;
}

// systems per batch under the memory budget (at least one)
int batch_size(crgpu_ctx *c) {
    const int nsys_total = (int)c->sys_k.size();
    size_t per = bytes_per_system(c);
    int64_t budget = c->mem_budget;
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = (int64_t)(0.6 * (double)(fr + (size_t)c->batch_cap * per));
    }
    int bs = (int)std::max<int64_t>(1, std::min<int64_t>(nsys_total, budget / (int64_t)per));
    if (c->batch_cap > 0 && c->batch_cap < bs && c->batch_cap >= nsys_total) bs = c->batch_cap;
    return bs;
}

// the batch of systems s0 .. s0+ns-1
DevBatch batch_view(crgpu_ctx *c, int ns) {
    DevBatch B = c->Bmax;
    B.nsys = ns;
    B.ks = c->d_ks;
    B.ls = c->d_ls;
    return B;
}

// systems s0 .. s0+m-1 of a batch view as a batch of their own
DevBatch sub_view(const crgpu_ctx *c, const DevBatch &B, int s0, int m) {
    const size_t n = c->hg.n, nnz = c->pat.nnz, nr = c->nrhs;
    const size_t esz = c->precision == CRGPU_MIXED ? sizeof(float2) : sizeof(double2);
    DevBatch S = B;
    S.nsys = m;
    S.ks += s0;
    S.ls += s0;
    S.As += s0 * nnz;
    S.fak += s0 * n;
    S.b += s0 * nr * n;
    S.x += s0 * nr * n;
    S.r += s0 * nr * n;
    S.L = (char *)B.L + s0 * B.lpitch * esz;
    S.y = (char *)B.y + s0 * nr * n * esz;
    S.status += s0;
    S.active += s0 * nr;
    if (B.pota) S.pota += s0 * n;
    if (B.potmax) S.potmax += s0;
    return S;
}

int load_batch(crgpu_ctx *c, int s0, int ns) {
    CUCHECK(c, cudaMemcpyAsync(c->d_ks, c->sys_k.data() + s0, sizeof(int32_t) * ns, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(c->d_ls, c->sys_l.data() + s0, sizeof(int32_t) * ns, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemsetAsync(c->Bmax.status, 0, sizeof(int) * ns, c->st));
    return 0;
}

// Solves the systems of batch view B, whose band factors are in B.L, for the
// right-hand sides in B.b (src/vre.f90) on stream st; the forward sweep was
// already done inside the factorisation when fused.  Mixed precision adds the
// FP64 refinement: every step is launched without waiting for the host (a
// step whose predecessor left no item active returns at once), with its
// counters in refinement array `slot`.  The FP64 solution ends in B.x.
int solve_view(crgpu_ctx *c, const DevBatch &B, bool fused, cudaStream_t st, int slot) {
    DevProblem &P = c->P;
    const bool mixed = c->precision == CRGPU_MIXED;
    const int nr = c->nrhs;
    DevBatch Bs = B;
    Bs.active = nullptr;
    Bs.nactive = nullptr;
    Bs.zmax = nullptr;
    Bs.nprev = nullptr;
    if (!fused) {
        launch_forward_solve(P, Bs, nr, mixed, B.b, st);
        c->stats.kernel_launches += 1;
    }
    launch_back_solve(P, Bs, nr, mixed, st);
    c->stats.kernel_launches += 1;
    if (!mixed) {
        launch_copy_solution(P, B, nr, st);
        c->stats.kernel_launches += 1;
        return 0;
    }
    RefineCount *cnt = (RefineCount *)c->d_refine + (size_t)slot * kRefineCap;
    const int steps = std::min(c->refine_maxit, kRefineCap);
    CUCHECK(c, cudaMemsetAsync(cnt, 0, sizeof(RefineCount) * kRefineCap, st));
    launch_fill_active(B, nr, st);
    DevBatch B0 = B;
    B0.zmax = nullptr;
    B0.nactive = nullptr;
    B0.nprev = nullptr;
    launch_accumulate(P, B0, nr, true, c->refine_tol, st);
    c->stats.kernel_launches += 2;
    for (int it = 0; it < steps; it++) {
        DevBatch Bi = B;
        Bi.nactive = &cnt[it].n;
        Bi.zmax = &cnt[it].z;
        Bi.nprev = it > 0 ? &cnt[it - 1].n : nullptr;
        launch_residual(P, Bi, nr, st);
        launch_forward_solve(P, Bi, nr, true, B.r, st);
        launch_back_solve(P, Bi, nr, true, st);
        launch_accumulate(P, Bi, nr, false, c->refine_tol, st);
        c->stats.kernel_launches += 4;
    }
    c->refine_used[slot] = std::max(c->refine_used[slot], steps);
    return 0;
}

int solve_batch(crgpu_ctx *c, int ns, bool fused) { return solve_view(c, batch_view(c, ns), fused, c->st, 0); }

// refinement statistics of the steps launched since the last collection (the
// streams must be idle): steps that ran, and the largest relative correction
// of the last one
int collect_refine_stats(crgpu_ctx *c) {
    for (int slot = 0; slot < kRefineSlots; slot++) {
        const int used = c->refine_used[slot];
        if (!used) continue;
        std::vector<RefineCount> h(used);
        CUCHECK(c, cudaMemcpy(h.data(), (RefineCount *)c->d_refine + (size_t)slot * kRefineCap,
                              sizeof(RefineCount) * used, cudaMemcpyDeviceToHost));
        int ran = 0;  // step it ran if it was the first or its predecessor left items active
        for (int it = 0; it < used; it++)
            if (it == 0 || h[it - 1].n > 0) ran = it + 1;
        c->stats.refine_iterations = std::max(c->stats.refine_iterations, ran);
        if (ran > 0) c->stats.refine_last_correction = std::max(c->stats.refine_last_correction, h[ran - 1].z);
        c->refine_used[slot] = 0;
    }
    return 0;
}

// assembly and scaling (src/kompab.f90, src/scalab.f90) of the current batch
int assemble_batch(crgpu_ctx *c, const double2 *d_sigma, int ns) {
    DevProblem &P = c->P;
    DevBatch B = batch_view(c, ns);
    launch_assemble(P, B, d_sigma, c->d_adom, c->st);
    c->stats.kernel_launches += 2;
    return 0;
}

// band factorisation of the current batch (src/chol.f90); with fuse the
// forward sweep of the right-hand sides in B.b runs inside the factor
int run_factor_view(crgpu_ctx *c, const DevBatch &B, int fuse, cudaStream_t st, bool exclusive = false,
                    int kind = 0) {
    if (c->precision == CRGPU_MIXED) {
        DevProblem P = c->P;
        if (kind) P.tune_factor = kind;
        int e = launch_factor_mixed(P, B, fuse, c->nsm, exclusive, st);
        if (e) return fail(c, e, "mixed precision: band width beyond the supported window");
    } else {
        launch_factor_plain(c->P, B, fuse, c->nsm, st);
    }
    c->stats.kernel_launches += 1;
    return 0;
}

int run_factor(crgpu_ctx *c, int ns, int fuse) { return run_factor_view(c, batch_view(c, ns), fuse, c->st); }

// systems of a batch beyond the last full round of the factor: they are
// factored and solved on the high priority stream while the full rounds'
// systems are solved.  0: no split.  Tensor cores: rounds of two blocks per
// SM.  One warp per system: up to 8 systems an SM take the faster register
// budget in one wave, so a batch at most one system an SM beyond that splits
// off the excess (config 2: 1248 = 1216 + 32).
int tail_systems(const crgpu_ctx *c, int ns) {
    if (c->precision != CRGPU_MIXED || c->nsm <= 0) return 0;
    const int kind = mixed_factor_kind(c->P);
    if (kind == 1) {
        const int round = 2 * c->nsm, tail = ns % round;
        return (ns > round && tail > 0 && tail <= round / 2) ? tail : 0;
    }
    if (kind == 4) {
        const int wave = 8 * c->nsm, tail = ns - wave;
        return (tail > 0 && tail <= c->nsm) ? tail : 0;
    }
    return 0;
}

// the forward block on device-resident sigma
int run_forward(crgpu_ctx *c, const double2 *d_sigma, int volt_mode, const double *d_kfak, double2 *d_volt,
                double2 *d_sigmaa) {
    DevProblem &P = c->P;
    const bool cap = c->capturing;  // graph capture: no host copies, synchronisation or timing
    c->stats = crgpu_stats{};
    c->factors_resident = false;
    cudaEvent_t ev[4];
    for (auto &e : ev) cudaEventCreate(&e);
    if (!cap) cudaEventRecord(ev[0], c->st);
    CUCHECK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
    if (d_sigma != c->d_sigma)  // keep the model of this forward (adjoint, refactorisation)
        CUCHECK(c, cudaMemcpyAsync(c->d_sigma, d_sigma, sizeof(double2) * c->hg.elanz, cudaMemcpyDeviceToDevice, c->st));
    d_sigma = c->d_sigma;
    if (P.ldc) {  // the DC routines take DBLE(sigma) (src/kompadc.f90:114-119, src/bsendc.f90:172)
        launch_real_part(c->d_sigma, c->hg.elanz, c->st);
        c->stats.kernel_launches += 1;
    }
    launch_adom(P, d_sigma, c->d_adom, c->st);
    c->stats.kernel_launches += 1;
    if (c->lsr) {
        launch_refsig(P, d_sigma, c->d_sigma0, c->st);
        c->stats.kernel_launches += 1;
    }
    const int nsys_total = (int)c->sys_k.size();
    const int bs = cap ? nsys_total : batch_size(c);  // recording: one batch, allocated by the ordinary run
    int e = ensure_batch(c, bs);
    if (e) return e;
    c->stats.nsystems = nsys_total;
    float t_factor = 0.f, t_solve = 0.f;
    cudaEvent_t f0, f1, f2;
    cudaEventCreate(&f0);
    cudaEventCreate(&f1);
    cudaEventCreate(&f2);
    int worst = 0;
    for (int s0 = 0; s0 < nsys_total; s0 += bs) {
        const int ns = std::min(bs, nsys_total - s0);
        const int nr = c->nrhs;
        const int fuse = nr == 1 ? 1 : 0;
        DevBatch B = batch_view(c, ns);
        if (cap) {  // one batch: its systems' (k, l) are on the device already
            CUCHECK(c, cudaMemsetAsync(c->Bmax.status, 0, sizeof(int) * ns, c->st));
        } else {
            e = load_batch(c, s0, ns);
        }
        if (!e) e = assemble_batch(c, d_sigma, ns);
        if (e) return e;
        if (c->lsr) {
            launch_pota_rhs(P, B, d_sigma, c->d_sigma0, c->lsink, c->nsink, c->st);
            c->stats.kernel_launches += 3;
        } else {
            launch_rhs(P, B, nr, c->lsink, c->nsink, c->st);
            c->stats.kernel_launches += 1;
        }
        if (P.lrandb2) {
            launch_rhs_randb2(P, B, nr, d_sigma, c->d_adom, c->st);
            c->stats.kernel_launches += 1;
        }
        const int tail = tail_systems(c, ns);
        if (!cap) cudaEventRecord(f0, c->st);
        if (!tail) {
            e = run_factor(c, ns, fuse);
            if (e) return e;
            if (!cap) cudaEventRecord(f1, c->st);
            e = solve_view(c, B, fuse != 0, c->st, 0);
            if (e) return e;
        } else {
            // full rounds on st; the last, partial round starts on st_hi once they are
            // done, beside the full rounds' solves, and is solved there.  (Factor
            // launches per round with each round's solves beside the next round's
            // factor were slower: the sweeps' blocks slowed the latency-bound factor
            // more than they gained, 46.8 against 37.2 ms per unit on config 2.)
            const DevBatch Bf = sub_view(c, B, 0, ns - tail), Bt = sub_view(c, B, ns - tail, tail);
            e = run_factor_view(c, Bf, fuse, c->st);
            if (e) return e;
            cudaEventRecord(f1, c->st);
            CUCHECK(c, cudaStreamWaitEvent(c->st_hi, f1, 0));
            // SMs of their own; the few tail systems of the warp-per-system factor
            // take the tensor cores, which factor one lone system faster
            const int tkind = (mixed_factor_kind(P) == 4 && P.mb + 4 <= 128) ? 1 : 0;
            e = run_factor_view(c, Bt, fuse, c->st_hi, true, tkind);
            if (!e) e = solve_view(c, Bt, fuse != 0, c->st_hi, 1);
            if (!e) e = solve_view(c, Bf, fuse != 0, c->st, 0);
            if (e) return e;
            CUCHECK(c, cudaEventRecord(c->ev_join, c->st_hi));
            CUCHECK(c, cudaStreamWaitEvent(c->st, c->ev_join, 0));
        }
        launch_kpot(P, B, nr, c->d_kpot, c->d_kpot32, c->st);
        c->stats.kernel_launches += 1;
        c->stats.nbatches++;
        if (cap) continue;
        cudaEventRecord(f2, c->st);
        int ce = check_device_errors(c, B.status, ns);
        if (ce) {
            worst = ce;
            break;
        }
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, f0, f1);
        cudaEventElapsedTime(&b, f1, f2);
        t_factor += a;
        t_solve += b;
    }
    cudaEventDestroy(f0);
    cudaEventDestroy(f1);
    cudaEventDestroy(f2);
    if (worst) {
        for (auto &ev_ : ev) cudaEventDestroy(ev_);
        return worst;
    }
    launch_rtrafo(P, c->d_kpot, c->d_hpot, c->st);
    launch_bvolt(P, c->d_hpot, volt_mode, d_kfak, d_volt, d_sigmaa, c->st);
    c->stats.kernel_launches += 2;
    if (cap) {
        for (auto &ev_ : ev) cudaEventDestroy(ev_);
        c->have_forward = true;
        c->factors_resident = true;
        return 0;
    }
    cudaEventRecord(ev[1], c->st);
    int ce = check_device_errors(c, nullptr, 0);
    if (!ce) ce = collect_refine_stats(c);
    float tf = 0.f;
    cudaEventElapsedTime(&tf, ev[0], ev[1]);
    c->stats.ms_forward = tf;
    c->stats.ms_factor = t_factor;
    c->stats.ms_solve = t_solve;
    for (auto &ev_ : ev) cudaEventDestroy(ev_);
    CUCHECK(c, cudaGetLastError());
    if (ce) return ce;
    c->have_forward = true;
    c->factors_resident = c->stats.nbatches == 1;
    return 0;
}

// Exact derivative of L = sum_i g_i V_i (the voltages of the last forward)
// with respect to sigma: lambda_(k,l) = A_(k,l)^{-1} c_l with the adjoint
// sources c_l of the measurements, solved with the forward's band factors
// (refactored batch by batch when the forward needed several batches), then
// grad_e = -sum_(k,l) w_k/pi lambda^T (dA/dsigma_e) kpot.
int run_adjoint(crgpu_ctx *c, const double2 *d_g, double2 *d_grad) {
    DevProblem &P = c->P;
    if (!c->have_forward) return fail(c, ERR_ARG, "adjoint before a forward");
    if (c->lsr) return fail(c, ERR_UNSUPPORTED, "adjoint with singularity removal");
    if (!c->d_lambda) {
        int e = dalloc(c, &c->d_lambda, (size_t)c->K * c->eanz * c->hg.n);
        if (!e) e = dalloc(c, &c->d_adjsrc, (size_t)c->eanz * c->hg.n);
        if (e) return e;
    }
    cudaEvent_t a0, a1;
    cudaEventCreate(&a0);
    cudaEventCreate(&a1);
    cudaEventRecord(a0, c->st);
    CUCHECK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
    launch_adjoint_sources(P, d_g, c->d_adjsrc, c->lsink, c->nsink, c->st);
    c->stats.kernel_launches += 2;
    const int nsys_total = (int)c->sys_k.size();
    const int nr = c->nrhs;
    int e = 0;
    if (c->factors_resident) {
        DevBatch B = batch_view(c, nsys_total);
        launch_adjoint_rhs(P, B, nr, c->d_adjsrc, c->st);
        e = solve_batch(c, nsys_total, false);
        if (e) return e;
        launch_adjoint_lambda(P, B, nr, c->d_lambda, c->st);
        c->stats.kernel_launches += 2;
        e = check_device_errors(c, B.status, nsys_total);
        if (e) return e;
    } else {
        const int bs = c->batch_cap;
        for (int s0 = 0; s0 < nsys_total; s0 += bs) {
            const int ns = std::min(bs, nsys_total - s0);
            DevBatch B = batch_view(c, ns);
            e = load_batch(c, s0, ns);
            if (!e) e = assemble_batch(c, c->d_sigma, ns);
            if (e) return e;
            launch_adjoint_rhs(P, B, nr, c->d_adjsrc, c->st);
            e = run_factor(c, ns, 0);
            if (!e) e = solve_batch(c, ns, false);
            if (e) return e;
            launch_adjoint_lambda(P, B, nr, c->d_lambda, c->st);
            c->stats.kernel_launches += 2;
            e = check_device_errors(c, B.status, ns);
            if (e) return e;
        }
        c->factors_resident = nsys_total <= bs;
    }
    launch_adjoint_grad(P, c->d_kpot, c->d_lambda, c->d_ebnd_ptr, c->d_ebnd_list, d_grad, c->st);
    c->stats.kernel_launches += 1;
    cudaEventRecord(a1, c->st);
    e = check_device_errors(c, nullptr, 0);
    if (!e) e = collect_refine_stats(c);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a0, a1);
    c->stats.ms_adjoint = ms;
    cudaEventDestroy(a0);
    cudaEventDestroy(a1);
    CUCHECK(c, cudaGetLastError());
    return e;
}

}  // namespace

// autotuner state (crgpu_autotune)
namespace {
struct TuneKey {
    int n, mb, nsys, eanz, nanz, K, nsm;
    bool operator<(const TuneKey &o) const {
        return std::tie(n, mb, nsys, eanz, nanz, K, nsm) < std::tie(o.n, o.mb, o.nsys, o.eanz, o.nanz, o.K, o.nsm);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, std::array<int, 3>> g_tune;

// device time of fn() on the context's stream, best of two after a warm-up
template <typename F>
float time_on(crgpu_ctx *c, F &&fn) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(a, c->st);
        fn();
        cudaEventRecord(b, c->st);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (r > 0) best = std::min(best, ms);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return best;
}
}  // namespace

extern "C" {

int crgpu_create(const crgpu_grid *grid, const crgpu_survey *sv, int32_t precision, crgpu_ctx **out) {
    return crgpu_create2(grid, sv, precision, 1, out);
}

int crgpu_create2(const crgpu_grid *grid, const crgpu_survey *sv, int32_t precision, int32_t band_order,
                  crgpu_ctx **out) {
    if (!out) return ERR_ARG;
    *out = nullptr;
    crgpu_ctx *c = new crgpu_ctx();
    int e = build_grid(grid, c->hg, c->last_error);
    if (!e && (!sv || sv->eanz <= 0 || !sv->enr || sv->nanz < 0 || sv->kwnanz <= 0 || !sv->kwn || !sv->kwnwi)) {
        e = ERR_ARG;
        c->last_error = "crgpu_survey: missing arrays";
    }
    if (!e && precision != CRGPU_PLAIN && precision != CRGPU_MIXED) {
        e = ERR_ARG;
        c->last_error = "precision";
    }
    if (!e && (band_order < 0 || band_order > 2)) {
        e = ERR_ARG;
        c->last_error = "band_order";
    }
    // band_order 1: a complex64 context factors in the geometric node order
    // when that band is narrower (a narrower band is fewer factor flops and
    // fewer bytes for every sweep; a band too wide for the tensor-core window
    // only when the geometric band fits it); 2: either precision, whenever
    // narrower.  The results are mapped back to the grid's node order at the
    // boundary.
    const bool mixed = precision == CRGPU_MIXED;
    if (!e && (band_order == 2 || (band_order == 1 && mixed))) {
        const int mb2 = host_geometric_order(c->hg, c->old_of_new, c->new_of_old);
        const bool fits = band_order == 2 || c->hg.mb + 4 <= 128 || mb2 + 4 <= 128;
        if (fits && mb2 < c->hg.mb) {
            host_permute_grid(c->hg, c->old_of_new, c->new_of_old, mb2);
        } else {
            c->old_of_new.clear();
            c->new_of_old.clear();
        }
    }
    if (!e) e = build_pattern(c->hg, c->pat, c->last_error);
    if (e) {
        *out = c;  // keep the message available
        return e;
    }
    c->precision = precision;
    c->eanz = sv->eanz;
    c->nanz = sv->nanz;
    c->K = sv->kwnanz;
    c->swrtr = sv->swrtr;
    c->lsink = sv->lsink;
    c->nsink = sv->lsink ? sv->nsink - 1 : -1;
    if (c->nsink >= 0 && !c->new_of_old.empty()) c->nsink = c->new_of_old[c->nsink];
    c->lsytop = sv->lsytop;
    // src/fem.f90:311 (no mixed boundaries: no singularity removal) and 2D
    c->lsr = (sv->lsr && c->hg.lbeta && sv->swrtr != 0) ? 1 : 0;
    cudaError_t ce = cudaStreamCreateWithFlags(&c->own_st, cudaStreamNonBlocking);
    c->st = c->own_st;
    if (ce == cudaSuccess) {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        ce = cudaStreamCreateWithPriority(&c->st_hi, cudaStreamNonBlocking, hi);
    }
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
    if (ce != cudaSuccess) {
        c->last_error = cudaGetErrorString(ce);
        *out = c;
        return ERR_CUDA;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    c->device = dev;
    cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev);
    keep_pool_memory(dev);
    // device problem
    DevProblem &P = c->P;
    const HostGrid &hg = c->hg;
    P.n = hg.n;
    P.mb = hg.mb;
    P.W = hg.mb + 1;
    P.elanz = hg.elanz;
    P.relanz = hg.relanz;
    P.eanz = c->eanz;
    P.nanz = c->nanz;
    P.K = c->K;
    P.nnz = c->pat.nnz;
    P.nnz_full = c->pat.nnz_full;
    P.rw = c->pat.rw;
    P.swrtr = c->swrtr;
    P.lsr = c->lsr;
    P.sytop = sv->lsytop ? host_sytop(grid) : 0.0;
    std::vector<int32_t> enr0(c->eanz), meas((size_t)c->nanz * 4);
    for (int i = 0; i < c->eanz; i++) {
        if (sv->enr[i] < 1 || sv->enr[i] > hg.n) {
            c->last_error = "electrode node beyond sanz";
            *out = c;
            return 29;
        }
        enr0[i] = c->new_of_old.empty() ? sv->enr[i] - 1 : c->new_of_old[sv->enr[i] - 1];
    }
    for (int i = 0; i < c->nanz; i++) {
        int a1 = sv->strnr[i] % 10000, a2 = (sv->strnr[i] - a1) / 10000;
        int a3 = sv->vnr[i] % 10000, a4 = (sv->vnr[i] - a3) / 10000;
        int el[4] = {a1, a2, a3, a4};
        for (int q = 0; q < 4; q++) {
            if (el[q] < 0 || el[q] > c->eanz) {
                c->last_error = "Electrode pair " + std::to_string(i + 1) + " not correct";
                *out = c;
                return 46;
            }
            meas[(size_t)i * 4 + q] = el[q] - 1;
        }
    }
    std::vector<double> strom(c->nanz, 1.0), kwn(sv->kwn, sv->kwn + c->K), kwnwi(sv->kwnwi, sv->kwnwi + c->K);
    if (sv->strom)
        for (int i = 0; i < c->nanz; i++) strom[i] = sv->strom[i];
    if (!e) e = upload(c, &P.x, hg.x);
    if (!e) e = upload(c, &P.y, hg.y);
    if (!e) e = upload(c, &P.etype, hg.etype);
    if (!e) e = upload(c, &P.enodes, hg.enodes);
    if (!e) e = upload(c, &P.btype, hg.btype);
    if (!e) e = upload(c, &P.bnodes, hg.bnodes);
    if (!e) e = upload(c, &P.brnr, hg.brnr);
    if (!e) e = upload(c, &P.dirichlet, hg.dirichlet);
    if (!e) e = upload(c, &P.rowptr, c->pat.rowptr);
    if (!e) e = upload(c, &P.col, c->pat.col);
    if (!e) e = upload(c, &P.row, c->pat.row);
    if (!e) e = upload(c, &P.dom_ptr, c->pat.dom_ptr);
    if (!e) e = upload(c, &P.dom_list, c->pat.dom_list);
    if (!e) e = upload(c, &P.bnd_ptr, c->pat.bnd_ptr);
    if (!e) e = upload(c, &P.bnd_list, c->pat.bnd_list);
    if (!e) e = upload(c, &P.fptr, c->pat.fptr);
    if (!e) e = upload(c, &P.fcol, c->pat.fcol);
    if (!e) e = upload(c, &P.fidx, c->pat.fidx);
    if (!e) e = upload(c, &P.enr0, enr0);
    if (!e) e = upload(c, &P.meas, meas);
    if (!e) e = upload(c, &P.strom, strom);
    if (!e) e = upload(c, &P.kwn, kwn);
    if (!e) e = upload(c, &P.kwnwi, kwnwi);
    {
        // element areas as src/refsig.f90:38-62 computes them
        std::vector<double> area(hg.elanz, 0.0);
        for (int q = 0; q < hg.elanz; q++) {
            const int *nd = &hg.enodes[(size_t)q * 4];
            double xk = hg.x[nd[0]], yk = hg.y[nd[0]];
            double ax = hg.x[nd[1]] - xk, ay = hg.y[nd[1]] - yk, bx = hg.x[nd[2]] - xk, by = hg.y[nd[2]] - yk;
            if (hg.etype[q] == 3) {
                area[q] = std::fabs(ax * by - ay * bx) / 2.0;
            } else {
                double cx = hg.x[nd[3]] - xk, cy = hg.y[nd[3]] - yk;
                area[q] = (std::fabs(ax * by - ay * bx) + std::fabs(bx * cy - by * cx)) / 2.0;
            }
        }
        if (!e) e = upload(c, &P.earea, area);
    }
    {
        // mixed boundary elements (type 11) carried by each area element, for the adjoint
        std::vector<int32_t> ptr(hg.elanz + 1, 0), lst;
        for (int rb = 0; rb < hg.relanz; rb++)
            if (hg.btype[rb] == 11) ptr[hg.brnr[rb] + 1]++;
        for (int q = 0; q < hg.elanz; q++) ptr[q + 1] += ptr[q];
        lst.assign(std::max(ptr[hg.elanz], 1), 0);
        std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
        for (int rb = 0; rb < hg.relanz; rb++)
            if (hg.btype[rb] == 11) lst[fill[hg.brnr[rb]]++] = rb;
        if (!e) e = upload(c, &c->d_ebnd_ptr, ptr);
        if (!e) e = upload(c, &c->d_ebnd_list, lst);
    }
    if (!e) e = dalloc(c, &c->d_sigma0, 1);
    if (!e) e = dalloc(c, &P.elbg, (size_t)c->K * hg.elanz * 10);
    if (!e) e = dalloc(c, &P.relbg, (size_t)std::max(hg.relanz, 1) * 3);
    if (!e) e = dalloc(c, &P.kg, (size_t)c->K * c->eanz * std::max(hg.relanz, 1));
    if (!e) e = dalloc(c, &c->d_err, 1);
    if (!e) e = dalloc(c, &c->d_sigma, (size_t)hg.elanz);
    // area parts adom[K][nnz], then fak_area[K][n] (doubles) in the same allocation
    if (!e) e = dalloc(c, &c->d_adom, (size_t)c->K * c->pat.nnz + ((size_t)c->K * hg.n + 1) / 2);
    if (!e) e = dalloc(c, &c->d_kpot, (size_t)c->K * c->eanz * hg.n);
    if (!e && precision == CRGPU_MIXED) e = dalloc(c, &c->d_kpot32, 2 * (size_t)c->K * c->eanz * hg.n);  // hi, lo
    if (!e) e = dalloc(c, &c->d_hpot, (size_t)c->eanz * hg.n);
    if (!e) e = dalloc(c, &c->d_volt, (size_t)std::max(c->nanz, 1));
    if (!e) e = dalloc(c, &c->d_sigmaa, (size_t)std::max(c->nanz, 1));
    if (!e) e = dalloc(c, &c->d_kfak, (size_t)std::max(c->nanz, 1));
    if (e) {
        *out = c;
        return e;
    }
    P.err = c->d_err;
    cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st);
    launch_precal(P, c->st);
    c->stats.kernel_launches += 3;
    // systems: one factorisation per (k, l) with mixed boundaries, else one
    // per k shared by all electrodes (src/fem.f90:355-376)
    if (hg.lbeta) {
        c->nrhs = 1;
        for (int k = 0; k < c->K; k++)
            for (int l = 0; l < c->eanz; l++) {
                c->sys_k.push_back(k);
                c->sys_l.push_back(l);
            }
    } else {
        c->nrhs = c->eanz;
        for (int k = 0; k < c->K; k++) {
            c->sys_k.push_back(k);
            c->sys_l.push_back(0);
        }
    }
    if (precision == CRGPU_MIXED && !mixed_window_supported(hg.mb + 1)) {
        c->last_error = "mixed precision supports band widths up to 207";
        *out = c;
        return ERR_UNSUPPORTED;
    }
    int ce2 = check_device_errors(c, nullptr, 0);
    *out = c;
    return ce2;
}

int crgpu_destroy(crgpu_ctx *c) {
    if (!c) return 0;
    drop_graph(c);
    for (void *p : c->allocs) cudaFreeAsync(p, c->st);
    if (c->d_upd) cudaFreeAsync(c->d_upd, c->st);
    if (c->own_st) cudaStreamDestroy(c->own_st);
    if (c->copy_st) cudaStreamDestroy(c->copy_st);
    if (c->st_hi) cudaStreamDestroy(c->st_hi);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    delete c;
    return 0;
}

const char *crgpu_last_error(const crgpu_ctx *c) { return c ? c->last_error.c_str() : "null context"; }

int crgpu_set_refinement(crgpu_ctx *c, int32_t maxit, double tol) {
    if (!c || maxit < 0 || maxit > kRefineCap || !(tol >= 0.0)) return ERR_ARG;
    drop_graph(c);
    c->refine_maxit = maxit;
    c->refine_tol = tol;
    return 0;
}

int crgpu_set_boundary_values(crgpu_ctx *c, int32_t rwdanz, const int32_t *rwdnr, const double *rwd) {
    if (!c || rwdanz < 0 || (rwdanz > 0 && (!rwdnr || !rwd))) return ERR_ARG;
    const int n = (int)c->hg.n;
    for (int ir = 0; ir < rwdanz; ir++)  // src/rrandb.f90 (error 30)
        if (rwdnr[ir] < 1 || rwdnr[ir] > n)
            return fail(c, 30, "boundary value node " + std::to_string(rwdnr[ir]) + " outside 1.." +
                                   std::to_string(n));
    drop_graph(c);
    c->factors_resident = false;
    // type-13 nodes (src/randb.f90) first; src/randb2.f90 then sets b(k) = -value
    // (the last value of a node listed twice) and moves the column of a node
    // whose column is still in the matrix (the first value)
    std::vector<uint8_t> dir(c->hg.dirichlet);
    std::vector<double2> vals((size_t)2 * n, make_double2(0.0, 0.0));
    for (int ir = 0; ir < rwdanz; ir++) {
        const int k = c->new_of_old.empty() ? rwdnr[ir] - 1 : c->new_of_old[rwdnr[ir] - 1];
        const double2 v = make_double2(rwd[2 * ir], rwd[2 * ir + 1]);
        vals[k] = v;
        if (dir[k] == 0) vals[(size_t)n + k] = v;
        dir[k] = 2;
    }
    if (!c->d_rwd) {
        int e = dalloc(c, &c->d_rwd, (size_t)2 * n);
        if (e) return e;
    }
    CUCHECK(c, cudaMemcpyAsync((void *)c->P.dirichlet, dir.data(), (size_t)n, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(c->d_rwd, vals.data(), vals.size() * sizeof(double2), cudaMemcpyHostToDevice,
                               c->st));
    CUCHECK(c, cudaStreamSynchronize(c->st));
    c->P.lrandb2 = rwdanz > 0;
    c->P.rwd_b = c->d_rwd;
    c->P.rwd_col = c->d_rwd + n;
    return 0;
}

int crgpu_set_dc(crgpu_ctx *c, int32_t ldc) {
    if (!c || (ldc != 0 && ldc != 1)) return ERR_ARG;
    drop_graph(c);
    c->factors_resident = false;
    c->P.ldc = ldc;
    return 0;
}

int crgpu_set_stream(crgpu_ctx *c, void *stream) {
    if (!c) return ERR_ARG;
    c->st = stream ? (cudaStream_t)stream : c->own_st;
    return 0;
}

int crgpu_set_memory_budget(crgpu_ctx *c, int64_t bytes) {
    if (!c) return ERR_ARG;
    c->mem_budget = bytes;
    free_batch(c);
    return 0;
}

int crgpu_device_memory(int64_t *free_bytes, int64_t *total_bytes) {
    if (!free_bytes || !total_bytes) return ERR_ARG;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return ERR_CUDA;
    *free_bytes = (int64_t)fr;
    *total_bytes = (int64_t)tot;
    return 0;
}

int crgpu_forward_device(crgpu_ctx *c, const void *sigma_device, int32_t volt_mode, const void *kfak_device,
                         void *volt_device, void *sigmaa_device) {
    if (!c || !sigma_device) return ERR_ARG;
    return run_forward(c, (const double2 *)sigma_device, volt_mode, (const double *)kfak_device,
                       (double2 *)volt_device, (double2 *)sigmaa_device);
}

int crgpu_forward(crgpu_ctx *c, const double *sigma, double *kpot, double *hpot, int32_t volt_mode,
                  const double *kfak, double *volt, double *sigmaa) {
    if (!c || !sigma) return ERR_ARG;
    const size_t ne = c->hg.elanz, nn = c->hg.n;
    CUCHECK(c, cudaMemcpyAsync(c->d_sigma, sigma, ne * sizeof(double2), cudaMemcpyHostToDevice, c->st));
    const double *dk = nullptr;
    if (kfak) {
        CUCHECK(c, cudaMemcpyAsync(c->d_kfak, kfak, c->nanz * sizeof(double), cudaMemcpyHostToDevice, c->st));
        dk = c->d_kfak;
    }
    int e = run_forward(c, c->d_sigma, volt_mode, dk, c->d_volt, c->d_sigmaa);
    if (e) return e;
    if (kpot)
        CUCHECK(c, cudaMemcpyAsync(kpot, c->d_kpot, (size_t)c->K * c->eanz * nn * sizeof(double2),
                                   cudaMemcpyDeviceToHost, c->st));
    if (hpot)
        CUCHECK(c, cudaMemcpyAsync(hpot, c->d_hpot, (size_t)c->eanz * nn * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    if (!c->old_of_new.empty() && (kpot || hpot)) {  // back to the grid's node order
        CUCHECK(c, cudaStreamSynchronize(c->st));
        std::vector<double2> tmp(nn);
        auto unpermute = [&](double *arr, size_t blocks) {
            double2 *a = (double2 *)arr;
            for (size_t b = 0; b < blocks; b++) {
                std::copy(a + b * nn, a + (b + 1) * nn, tmp.begin());
                for (size_t j = 0; j < nn; j++) a[b * nn + c->old_of_new[j]] = tmp[j];
            }
        };
        if (kpot) unpermute(kpot, (size_t)c->K * c->eanz);
        if (hpot) unpermute(hpot, (size_t)c->eanz);
    }
    if (volt)
        CUCHECK(c, cudaMemcpyAsync(volt, c->d_volt, (size_t)c->nanz * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    if (sigmaa)
        CUCHECK(c, cudaMemcpyAsync(sigmaa, c->d_sigmaa, (size_t)c->nanz * sizeof(double2), cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaStreamSynchronize(c->st));
    return 0;
}

// Forward + Jacobian on device buffers as one CUDA graph.  The first call
// (and any call after the buffers, the mode, the launch choices, the
// refinement settings or the batching changed) runs the ordinary path, then
// records the same kernel sequence, both streams included, without its host
// copies, synchronisation and timing; later calls replay it and check for
// errors once.  Problems that need several batches run the ordinary path.
int crgpu_forward_sens_graph(crgpu_ctx *c, const void *sigma_device, void *volt_device, int32_t mode,
                             void *sens_device) {
    if (!c || !sigma_device || !volt_device || !sens_device || (mode != 0 && mode != 1)) return ERR_ARG;
    const bool same = c->graph && c->graph_key[0] == sigma_device && c->graph_key[1] == volt_device &&
                      c->graph_key[2] == sens_device && c->graph_mode == mode;
    if (same) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, c->st);
        CUCHECK(c, cudaGraphLaunch(c->graph, c->st));
        cudaEventRecord(b, c->st);
        int e = check_device_errors(c, c->Bmax.status, (int)c->sys_k.size());
        c->stats.refine_iterations = 0;
        c->stats.refine_last_correction = 0.0;
        for (int q = 0; q < kRefineSlots; q++) c->refine_used[q] = c->graph_refine_used[q];
        if (!e) e = collect_refine_stats(c);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        c->stats.ms_forward = ms;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        c->last_sens = (const double2 *)sens_device;
        return e;
    }
    drop_graph(c);
    // the ordinary path: results of this call, buffers and uploads for the recording
    int e = run_forward(c, (const double2 *)sigma_device, 0, nullptr, (double2 *)volt_device, nullptr);
    if (!e) e = crgpu_sens_device(c, mode, sens_device);
    if (e) return e;
    if (c->stats.nbatches != 1) return 0;
    const crgpu_stats keep = c->stats;  // this call's figures: the recording measures nothing
    c->capturing = true;
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
        e = run_forward(c, (const double2 *)sigma_device, 0, nullptr, (double2 *)volt_device, nullptr);
        if (!e) {
            launch_bsens(c->P, c->d_kpot, c->d_kpot32, c->d_sigma, (const double2 *)volt_device, mode,
                         c->precision == CRGPU_MIXED, (double2 *)sens_device, c->st);
            c->stats.kernel_launches += 1;
        }
        ce = cudaStreamEndCapture(c->st, &graph);
    }
    c->capturing = false;
    c->stats = keep;
    for (int q = 0; q < kRefineSlots; q++) {
        c->graph_refine_used[q] = c->refine_used[q];
        c->refine_used[q] = 0;
    }
    if (!e && ce == cudaSuccess && graph) ce = cudaGraphInstantiate(&c->graph, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e || ce != cudaSuccess) {  // no graph: later calls record again; this call's results stand
        c->graph = nullptr;
        cudaGetLastError();
        return e;
    }
    c->graph_key[0] = sigma_device;
    c->graph_key[1] = volt_device;
    c->graph_key[2] = sens_device;
    c->graph_mode = mode;
    return 0;
}

int crgpu_sens_device(crgpu_ctx *c, int32_t mode, void *sens_device) {
    if (!c || !sens_device || (mode != 0 && mode != 1)) return ERR_ARG;
    if (!c->have_forward) return fail(c, ERR_ARG, "crgpu_sens before crgpu_forward");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, c->st);
    launch_bsens(c->P, c->d_kpot, c->d_kpot32, c->d_sigma, c->d_volt, mode, c->precision == CRGPU_MIXED,
                 (double2 *)sens_device, c->st);
    c->last_sens = (const double2 *)sens_device;
    cudaEventRecord(b, c->st);
    c->stats.kernel_launches += 1;
    CUCHECK(c, cudaStreamSynchronize(c->st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    c->stats.ms_sens = ms;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    CUCHECK(c, cudaGetLastError());
    return 0;
}

// The Jacobian to host memory: computed in chunks of elements, each chunk's
// columns (contiguous in sens(nanz, manz)) copied by a second stream while
// the next chunk is computed.
int crgpu_memory_need(const crgpu_ctx *c, int64_t *bytes) {
    if (!c || !bytes) return ERR_ARG;
    const int nsys = (int)c->sys_k.size();
    int64_t need = c->batch_cap >= nsys ? 0 : (int64_t)bytes_per_system(c) * nsys;
    if (!c->d_sens) need += (int64_t)c->nanz * c->hg.elanz * (int64_t)sizeof(double2);
    *bytes = need;
    return 0;
}

// Forward and Jacobian of several mixed-precision contexts (uneven meshes):
// each problem is assembled on its own stream, the band factors of all their
// systems run in one persistent tensor-core launch over a table of (problem,
// system) items, longest systems first, and each problem's solves,
// refinement, back-transform, voltages and Jacobian then run on its own
// stream again.  Every problem must fit one batch (crgpu_memory_need).
int crgpu_forward_sens_batch(crgpu_ctx *const *ctxs, int32_t nprob, const double *const *sigma, int32_t volt_mode,
                             double *const *volt, int32_t sens_mode) {
    if (!ctxs || nprob <= 0 || !sigma || !volt || (sens_mode < -1 || sens_mode > 1)) return ERR_ARG;
    for (int p = 0; p < nprob; p++) {
        crgpu_ctx *c = ctxs[p];
        if (!c || !sigma[p] || !volt[p]) return ERR_ARG;
        if (c->precision != CRGPU_MIXED || c->hg.mb + 4 > 128 || c->lsr || c->P.ldc || c->P.lrandb2 ||
            c->nrhs != 1 || c->device != ctxs[0]->device)
            return fail(c, ERR_UNSUPPORTED, "batched forward: mixed precision on the tensor-core window only");
    }
    cudaStream_t st0 = ctxs[0]->st;
    std::vector<DevProblem> hp(nprob);
    std::vector<DevBatch> hb(nprob);
    std::vector<int> order(nprob);
    for (int p = 0; p < nprob; p++) {  // assembly and right-hand sides, each on its stream
        crgpu_ctx *c = ctxs[p];
        const int ns = (int)c->sys_k.size();
        c->stats = crgpu_stats{};
        c->factors_resident = false;
        drop_graph(c);
        int e = ensure_batch(c, ns);
        if (e) return e;
        CUCHECK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
        CUCHECK(c, cudaMemcpyAsync(c->d_sigma, sigma[p], sizeof(double2) * c->hg.elanz, cudaMemcpyHostToDevice, c->st));
        launch_adom(c->P, c->d_sigma, c->d_adom, c->st);
        e = load_batch(c, 0, ns);
        if (!e) e = assemble_batch(c, c->d_sigma, ns);
        if (e) return e;
        const DevBatch B = batch_view(c, ns);
        launch_rhs(c->P, B, 1, c->lsink, c->nsink, c->st);
        c->stats.kernel_launches += 3;
        c->stats.nsystems = ns;
        CUCHECK(c, cudaEventRecord(c->ev_join, c->st));
        CUCHECK(c, cudaStreamWaitEvent(st0, c->ev_join, 0));
        hp[p] = c->P;
        hb[p] = B;
        order[p] = p;
    }
    // the item table, longest systems first
    std::sort(order.begin(), order.end(), [&](int a, int b) { return ctxs[a]->hg.n > ctxs[b]->hg.n; });
    std::vector<int2> items;
    for (int p : order)
        for (int q = 0; q < hb[p].nsys; q++) items.push_back(make_int2(p, q));
    DevProblem *dP = nullptr;
    DevBatch *dB = nullptr;
    int2 *dI = nullptr;
    crgpu_ctx *c0 = ctxs[0];
    CUCHECK(c0, cudaMallocAsync((void **)&dP, sizeof(DevProblem) * nprob, st0));
    CUCHECK(c0, cudaMallocAsync((void **)&dB, sizeof(DevBatch) * nprob, st0));
    CUCHECK(c0, cudaMallocAsync((void **)&dI, sizeof(int2) * items.size(), st0));
    CUCHECK(c0, cudaMemcpyAsync(dP, hp.data(), sizeof(DevProblem) * nprob, cudaMemcpyHostToDevice, st0));
    CUCHECK(c0, cudaMemcpyAsync(dB, hb.data(), sizeof(DevBatch) * nprob, cudaMemcpyHostToDevice, st0));
    CUCHECK(c0, cudaMemcpyAsync(dI, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, st0));
    launch_factor_tc_multi(dP, dB, dI, (int)items.size(), 1, c0->nsm, st0);
    CUCHECK(c0, cudaGetLastError());
    CUCHECK(c0, cudaEventRecord(c0->ev_join, st0));
    for (int p = 0; p < nprob; p++) {  // solves, refinement, voltages and Jacobian, each on its stream
        crgpu_ctx *c = ctxs[p];
        if (p > 0) CUCHECK(c, cudaStreamWaitEvent(c->st, c0->ev_join, 0));
        int e = solve_view(c, hb[p], true, c->st, 0);
        if (e) return e;
        launch_kpot(c->P, hb[p], 1, c->d_kpot, c->d_kpot32, c->st);
        launch_rtrafo(c->P, c->d_kpot, c->d_hpot, c->st);
        launch_bvolt(c->P, c->d_hpot, volt_mode, nullptr, c->d_volt, c->d_sigmaa, c->st);
        c->stats.kernel_launches += 4;
        if (sens_mode >= 0) {
            if (!c->d_sens) {
                e = dalloc(c, &c->d_sens, (size_t)c->nanz * c->hg.elanz);
                if (e) return e;
            }
            launch_bsens(c->P, c->d_kpot, c->d_kpot32, c->d_sigma, c->d_volt, sens_mode, true, c->d_sens, c->st);
            c->stats.kernel_launches += 1;
            c->last_sens = c->d_sens;
        }
    }
    // the voltages once every problem's work is queued (a copy into pageable
    // host memory returns only when it is done)
    int worst = 0;
    for (int p = 0; p < nprob; p++) {
        crgpu_ctx *c = ctxs[p];
        CUCHECK(c, cudaMemcpyAsync(volt[p], volt_mode == 0 ? c->d_volt : c->d_sigmaa, sizeof(double2) * c->nanz,
                                   cudaMemcpyDeviceToHost, c->st));
        c->stats.kernel_launches += p == 0 ? 1 : 0;  // the shared factor launch
        int e = check_device_errors(c, hb[p].status, hb[p].nsys);
        if (!e) e = collect_refine_stats(c);
        if (e && !worst) worst = e;
        c->have_forward = !e;
        c->factors_resident = !e;
        c->stats.nbatches = 1;
    }
    cudaFreeAsync(dP, st0);
    cudaFreeAsync(dB, st0);
    cudaFreeAsync(dI, st0);
    CUCHECK(c0, cudaStreamSynchronize(st0));
    return worst;
}

int crgpu_sens(crgpu_ctx *c, int32_t mode, double *sens) {
    if (!c || (mode != 0 && mode != 1)) return ERR_ARG;
    if (!c->have_forward) return fail(c, ERR_ARG, "crgpu_sens before crgpu_forward");
    const size_t nanz = c->nanz, manz = c->hg.elanz, cnt = nanz * manz;
    if (!c->d_sens) {
        int e = dalloc(c, &c->d_sens, cnt);
        if (e) return e;
    }
    if (!sens) {  // kept on the device only, for crgpu_update
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, c->st);
        launch_bsens(c->P, c->d_kpot, c->d_kpot32, c->d_sigma, c->d_volt, mode, c->precision == CRGPU_MIXED,
                     c->d_sens, c->st);
        c->stats.kernel_launches += 1;
        cudaEventRecord(b, c->st);
        CUCHECK(c, cudaStreamSynchronize(c->st));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        c->stats.ms_sens = ms;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        c->last_sens = c->d_sens;
        CUCHECK(c, cudaGetLastError());
        return 0;
    }
    // CRMod sensitivities into pinned (page-locked) host memory are written by
    // the kernel itself, over the host link, while it computes; otherwise
    // chunked copies of the device array (which crgpu_update reads for mode 1)
    cudaPointerAttributes pa{};
    if (mode == 0 && cudaPointerGetAttributes(&pa, sens) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
        pa.devicePointer) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, c->st);
        launch_bsens(c->P, c->d_kpot, c->d_kpot32, c->d_sigma, c->d_volt, mode, c->precision == CRGPU_MIXED,
                     (double2 *)pa.devicePointer, c->st);
        c->stats.kernel_launches += 1;
        cudaEventRecord(b, c->st);
        CUCHECK(c, cudaStreamSynchronize(c->st));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        c->stats.ms_sens = ms;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        CUCHECK(c, cudaGetLastError());
        return 0;
    }
    cudaGetLastError();  // a pageable pointer is not an error
    if (!c->copy_st) CUCHECK(c, cudaStreamCreateWithFlags(&c->copy_st, cudaStreamNonBlocking));
    constexpr int kChunks = 8;
    cudaEvent_t a, b, done[kChunks];
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    for (auto &d : done) cudaEventCreateWithFlags(&d, cudaEventDisableTiming);
    cudaEventRecord(a, c->st);
    const int per = (int)((manz + kChunks - 1) / kChunks);
    for (int q = 0; q < kChunks; q++) {
        const int e0 = q * per, ne = std::min<int>(per, (int)manz - e0);
        if (ne <= 0) break;
        launch_bsens(c->P, c->d_kpot, c->d_kpot32, c->d_sigma, c->d_volt, mode, c->precision == CRGPU_MIXED,
                     c->d_sens, c->st, e0,
                     ne);
        c->stats.kernel_launches += 1;
        CUCHECK(c, cudaEventRecord(done[q], c->st));
        CUCHECK(c, cudaStreamWaitEvent(c->copy_st, done[q], 0));
        CUCHECK(c, cudaMemcpyAsync(sens + 2 * (size_t)e0 * nanz, c->d_sens + (size_t)e0 * nanz,
                                   (size_t)ne * nanz * sizeof(double2), cudaMemcpyDeviceToHost, c->copy_st));
    }
    cudaEventRecord(b, c->st);
    CUCHECK(c, cudaStreamSynchronize(c->copy_st));
    CUCHECK(c, cudaStreamSynchronize(c->st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    c->stats.ms_sens = ms;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    for (auto &d : done) cudaEventDestroy(d);
    c->last_sens = c->d_sens;
    CUCHECK(c, cudaGetLastError());
    return 0;
}

int crgpu_adjoint_device(crgpu_ctx *c, const void *g_device, void *grad_device) {
    if (!c || !g_device || !grad_device) return ERR_ARG;
    return run_adjoint(c, (const double2 *)g_device, (double2 *)grad_device);
}

int crgpu_adjoint(crgpu_ctx *c, const double *g, double *grad) {
    if (!c || !g || !grad) return ERR_ARG;
    if (!c->d_adjg) {
        int e = dalloc(c, &c->d_adjg, (size_t)std::max(c->nanz, 1));
        if (!e) e = dalloc(c, &c->d_adjgrad, (size_t)std::max(c->hg.elanz, 1));
        if (e) return e;
    }
    CUCHECK(c, cudaMemcpyAsync(c->d_adjg, g, sizeof(double2) * c->nanz, cudaMemcpyHostToDevice, c->st));
    int e = run_adjoint(c, c->d_adjg, c->d_adjgrad);
    if (e) return e;
    CUCHECK(c, cudaMemcpyAsync(grad, c->d_adjgrad, sizeof(double2) * c->hg.elanz, cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaStreamSynchronize(c->st));
    return 0;
}

int crgpu_node_order(const crgpu_ctx *c, int32_t *grid_node) {
    if (!c || !grid_node) return ERR_ARG;
    for (int j = 0; j < c->hg.n; j++) grid_node[j] = c->old_of_new.empty() ? j + 1 : c->old_of_new[j] + 1;
    return 0;
}

int crgpu_device_buffers(crgpu_ctx *c, void **kpot_device, void **hpot_device) {
    if (!c) return ERR_ARG;
    if (kpot_device) *kpot_device = c->d_kpot;
    if (hpot_device) *hpot_device = c->d_hpot;
    return 0;
}

int crgpu_factor_system(crgpu_ctx *c, const double *sigma, int32_t k, int32_t l, double *a, double *fak) {
    if (!c || !sigma || k < 1 || k > c->K || l < 1 || l > c->eanz) return ERR_ARG;
    if (!c->old_of_new.empty())
        return fail(c, ERR_UNSUPPORTED, "this context factors in the geometric node order (create it with band order 0 "
                                        "to read the grid's band)");
    c->factors_resident = false;  // system 0's factor is overwritten below
    const int n = c->hg.n, W = c->hg.mb + 1;
    CUCHECK(c, cudaMemcpyAsync(c->d_sigma, sigma, c->hg.elanz * sizeof(double2), cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
    launch_adom(c->P, c->d_sigma, c->d_adom, c->st);
    int e = ensure_batch(c, std::max(1, c->batch_cap));
    if (e) return e;
    DevBatch B = c->Bmax;
    B.nsys = 1;
    B.ks = c->d_ks;
    B.ls = c->d_ls;
    int32_t kk = k - 1, ll = c->P.relanz && c->hg.lbeta ? l - 1 : 0;
    CUCHECK(c, cudaMemcpyAsync(c->d_ks, &kk, sizeof(int32_t), cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(c->d_ls, &ll, sizeof(int32_t), cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemsetAsync(B.status, 0, sizeof(int), c->st));
    launch_assemble(c->P, B, c->d_sigma, c->d_adom, c->st);
    launch_rhs(c->P, B, 1, c->lsink, c->nsink, c->st);
    if (c->precision == CRGPU_MIXED) {
        e = launch_factor_mixed(c->P, B, 1, c->nsm, false, c->st);
        if (e) return fail(c, e, "mixed window");
    } else {
        launch_factor_plain(c->P, B, 1, c->nsm, c->st);
    }
    e = check_device_errors(c, B.status, 1);
    if (e) return e;
    if (a) {
        if (c->precision == CRGPU_MIXED) {
            std::vector<float> tmp((size_t)n * W * 2);
            CUCHECK(c, cudaMemcpy(tmp.data(), B.L, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost));
            for (size_t q = 0; q < tmp.size(); q++) a[q] = tmp[q];
        } else {
            CUCHECK(c, cudaMemcpy(a, B.L, (size_t)n * W * sizeof(double2), cudaMemcpyDeviceToHost));
        }
    }
    if (fak) CUCHECK(c, cudaMemcpy(fak, B.fak, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int crgpu_rwaven(const crgpu_grid *grid, int32_t eanz, const int32_t *enr, int32_t nanz, const int32_t *strnr,
                 const int32_t *vnr, double *kwn, double *kwnwi, int32_t *kwnanz) {
    if (!grid || !enr || !strnr || !vnr || !kwn || !kwnwi || !kwnanz) return ERR_ARG;
    HostGrid hg;
    std::string msg;
    int e = build_grid(grid, hg, msg);
    if (e) return e;
    for (int i = 0; i < eanz; i++)
        if (enr[i] < 1 || enr[i] > hg.n) return 29;
    return host_rwaven(hg, eanz, enr, nanz, strnr, vnr, kwn, kwnwi, kwnanz);
}

int crgpu_cutmck(int32_t sanz, int32_t typanz, const int32_t *typ, const int32_t *nelanz, const int32_t *selanz,
                 int32_t *nrel, int32_t ld_nrel, int32_t *snr, int32_t eanz, int32_t *enr, int32_t *mb) {
    if (!typ || !nelanz || !selanz || !nrel || !snr || !mb || (eanz > 0 && !enr)) return ERR_ARG;
    return host_cutmck(sanz, typanz, typ, nelanz, selanz, nrel, ld_nrel, snr, eanz, enr, mb);
}

int crgpu_bkfak(const crgpu_grid *grid, const crgpu_survey *sv, double *kfak) {
    if (!grid || !sv || !kfak) return ERR_ARG;
    HostGrid hg;
    std::string msg;
    int e = build_grid(grid, hg, msg);
    if (e) return e;
    const double pi = 3.14159265358979323846264338327950288;
    double xk[4] = {0, 0, 0, 0}, yk[4] = {0, 0, 0, 0};
    for (int i = 0; i < sv->nanz; i++) {
        int el[4];
        el[0] = sv->strnr[i] % 10000;
        el[1] = (sv->strnr[i] - el[0]) / 10000;
        el[2] = sv->vnr[i] % 10000;
        el[3] = (sv->vnr[i] - el[2]) / 10000;
        for (int q = 0; q < 4; q++)
            if (el[q] > 0) {
                int nd = sv->enr[el[q] - 1] - 1;
                xk[q] = hg.x[nd];
                yk[q] = hg.y[nd];
            }
        // r1 (4,2), r2 (4,1), r3 (3,2), r4 (3,1): src/bkfak.f90:79-134
        const int pr[4][2] = {{3, 1}, {3, 0}, {2, 1}, {2, 0}};
        double r[4];
        for (int q = 0; q < 4; q++) {
            int a = pr[q][0], b = pr[q][1];
            if (el[a] > 0 && el[b] > 0) {
                double dx = xk[a] - xk[b], dym = yk[a] - yk[b], dyp = yk[a] + yk[b];
                dym = 1.0 / std::sqrt(dx * dx + dym * dym);
                dyp = 1.0 / std::sqrt(dx * dx + dyp * dyp);
                r[q] = dym + dyp;
            } else {
                r[q] = 0.0;
            }
        }
        double dum = (r[0] - r[1]) - (r[2] - r[3]);
        if (std::fabs(dum) == 0.0) return 93;
        kfak[i] = 4.0 * pi / dum;
    }
    return 0;
}

// ---- autotuner: the fastest mixed factor kernel (and its blocks per SM) and
//      CRMod Jacobian kernel for this problem, timed on its own systems.
//      Choices are cached for the process by problem shape.

int crgpu_autotune(crgpu_ctx *c, const double *sigma, int32_t flags) {
    if (!c || !sigma) return ERR_ARG;
    if (c->precision != CRGPU_MIXED) return 0;  // complex128 has one kernel per step
    drop_graph(c);
    const TuneKey key{(int)c->hg.n, c->hg.mb, (int)c->sys_k.size(), c->eanz, c->nanz, c->K, c->nsm};
    if (!(flags & 1)) {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            c->P.tune_factor = it->second[0];
            c->P.tune_ctas = it->second[1];
            c->P.tune_sens = it->second[2];
            return 0;
        }
    }
    // a forward with the current choices: sigma on the device, kpot for the Jacobian
    int e = crgpu_forward(c, sigma, nullptr, nullptr, 0, nullptr, nullptr, nullptr);
    if (e) return e;
    DevProblem &P = c->P;
    // ---- factor: the first batch of systems, assembled as the forward does
    const int nsys_total = (int)c->sys_k.size(), ns = std::min(batch_size(c), nsys_total);
    e = ensure_batch(c, ns);
    if (!e) e = load_batch(c, 0, ns);
    if (!e) e = assemble_batch(c, c->d_sigma, ns);
    if (e) return e;
    const int fuse = c->nrhs == 1 ? 1 : 0;
    DevBatch B = batch_view(c, ns);
    launch_rhs(P, B, c->nrhs, c->lsink, c->nsink, c->st);
    std::vector<std::array<int, 2>> cand;
    if (P.mb + 1 <= 64 && P.rw <= 32) cand.push_back({4, 0});
    if (P.mb + 4 <= 128) cand.push_back({1, 0});
    if (mixed_window_supported(P.mb + 1) <= 176 && mixed_window_supported(P.mb + 1) > 0)
        for (int k : {1, 2, 4}) cand.push_back({2, k});
    else if (mixed_window_supported(P.mb + 1) > 0)
        for (int k : {1, 2}) cand.push_back({3, k});
    float best = 1e30f;
    std::array<int, 2> pick = {P.tune_factor, P.tune_ctas};
    for (auto &cd : cand) {
        P.tune_factor = cd[0];
        P.tune_ctas = cd[1];
        int fe = 0;
        // as the forward runs it: a batch that splits (tail_systems) is timed as
        // its main launch and then its tail launch
        const int tail = tail_systems(c, ns);
        const float ms = time_on(c, [&] {
            if (!tail) {
                fe = fe ? fe : run_factor(c, ns, fuse);
                return;
            }
            const int tkind = (mixed_factor_kind(P) == 4 && P.mb + 4 <= 128) ? 1 : 0;
            fe = fe ? fe : run_factor_view(c, sub_view(c, B, 0, ns - tail), fuse, c->st);
            fe = fe ? fe : run_factor_view(c, sub_view(c, B, ns - tail, tail), fuse, c->st, true, tkind);
        });
        if (fe) return fe;
        int ce = check_device_errors(c, B.status, ns);
        if (ce) return ce;
        if (ms < best) {
            best = ms;
            pick = cd;
        }
    }
    P.tune_factor = pick[0];
    P.tune_ctas = pick[1];
    c->factors_resident = false;
    // ---- CRMod Jacobian: tensor cores or SIMT
    if (sens_tc_supported(P, 0)) {
        if (!c->d_sens) {
            e = dalloc(c, &c->d_sens, (size_t)c->nanz * c->hg.elanz);
            if (e) return e;
        }
        float bs = 1e30f;
        int spick = 1;
        for (int k : {1, 2}) {
            P.tune_sens = k;
            const float ms = time_on(c, [&] {
                launch_bsens(P, c->d_kpot, c->d_kpot32, c->d_sigma, c->d_volt, 0, true, c->d_sens, c->st);
            });
            if (ms < bs) {
                bs = ms;
                spick = k;
            }
        }
        P.tune_sens = spick;
    }
    e = check_device_errors(c, nullptr, 0);
    if (e) return e;
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune[key] = {P.tune_factor, P.tune_ctas, P.tune_sens};
    return 0;
}

int crgpu_set_tune(crgpu_ctx *c, const int32_t *in) {
    if (!c || !in || in[0] < 0 || in[0] > 4 || in[1] < 0 || in[1] > 8 || in[2] < 0 || in[2] > 2) return ERR_ARG;
    drop_graph(c);
    c->P.tune_factor = in[0];
    c->P.tune_ctas = in[1];
    c->P.tune_sens = in[2];
    return 0;
}

int crgpu_get_tune(const crgpu_ctx *c, int32_t *out) {
    if (!c || !out) return ERR_ARG;
    out[0] = c->P.tune_factor;
    out[1] = c->P.tune_ctas;
    out[2] = c->P.tune_sens;
    return 0;
}

int crgpu_get_stats(const crgpu_ctx *c, crgpu_stats *s) {
    if (!c || !s) return ERR_ARG;
    *s = c->stats;
    return 0;
}

static int update_common(crgpu_ctx *c, int part, const double *wmatd, const int32_t *wdfak,
                         const double *dat, const double *sigmaa, int32_t ltri, const double *smatm, int32_t nx,
                         const int32_t *nachbar, double lam, double eps, int32_t ncgmax, double step, double *par,
                         double *dpar, double *cgfac, float *cgres, int32_t *ncg) {
    if (!c || !wmatd || !wdfak || !dat || !sigmaa || !smatm || !par || !dpar || !cgfac || !cgres || !ncg ||
        ncgmax < 1)
        return ERR_ARG;
    if (!c->last_sens) return fail(c, ERR_ARG, "crgpu_update needs the sensitivities (crgpu_sens mode 1) first");
    if (ltri != 0 && ltri != 1 && ltri != 2)
        return fail(c, ERR_UNSUPPORTED, "crgpu_update: regularisation types 0, 1 and 2 only");
    if (ltri != 0 && !nachbar) return ERR_ARG;
    const int nanz = c->nanz, manz = c->hg.elanz;
    int maxnk = 0;
    for (int e = 0; e < manz; e++) maxnk = std::max(maxnk, c->hg.etype[e] == 3 ? 3 : 4);
    if (ltri == 0 && (nx <= 0 || manz % nx != 0)) return fail(c, ERR_ARG, "nx must divide manz");
    const int ncol = ltri == 0 ? 3 : maxnk + 1;
    // device layout of the inputs and outputs, then the CG work space
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    const size_t o_w = take(sizeof(double) * nanz), o_wd = take(sizeof(int32_t) * nanz);
    const size_t o_dat = take(sizeof(double2) * nanz), o_sa = take(sizeof(double2) * nanz);
    const size_t o_sm = take(sizeof(double) * (size_t)manz * ncol);
    const size_t o_nb = take(sizeof(int32_t) * (size_t)manz * (maxnk + 1));
    const size_t o_par = take(sizeof(double2) * manz), o_dpar = take(sizeof(double2) * manz);
    const size_t o_cg = take(sizeof(double) * manz);
    const size_t o_work = take(update_work_bytes(nanz, manz));
    if (c->upd_bytes < off) {
        if (c->d_upd) cudaFreeAsync(c->d_upd, c->st);
        c->d_upd = nullptr;
        c->upd_bytes = 0;
        cudaError_t e = cudaMallocAsync(&c->d_upd, off, c->st);
        if (e != cudaSuccess) return fail(c, 94, std::string("update work space: ") + cudaGetErrorString(e));
        c->upd_bytes = off;
    }
    char *base = (char *)c->d_upd;
    CUCHECK(c, cudaMemcpyAsync(base + o_w, wmatd, sizeof(double) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(base + o_wd, wdfak, sizeof(int32_t) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(base + o_dat, dat, sizeof(double2) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(base + o_sa, sigmaa, sizeof(double2) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(base + o_sm, smatm, sizeof(double) * (size_t)manz * ncol, cudaMemcpyHostToDevice, c->st));
    if (ltri != 0)
        CUCHECK(c, cudaMemcpyAsync(base + o_nb, nachbar, sizeof(int32_t) * (size_t)manz * (maxnk + 1),
                                   cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(base + o_par, par, sizeof(double2) * manz, cudaMemcpyHostToDevice, c->st));
    CGArgs a{};
    a.nanz = nanz;
    a.manz = manz;
    a.ltri = ltri;
    a.nx = nx;
    a.maxnk = maxnk;
    a.ncgmax = ncgmax;
    a.lam = lam;
    a.eps = eps;
    a.step = step;
    a.sens = c->last_sens;
    a.wmatd = (const double *)(base + o_w);
    a.wdfak = (const int32_t *)(base + o_wd);
    a.dat = (const double2 *)(base + o_dat);
    a.sigmaa = (const double2 *)(base + o_sa);
    a.smatm = (const double *)(base + o_sm);
    a.nachbar = (const int32_t *)(base + o_nb);
    a.par = (double2 *)(base + o_par);
    a.dpar = (double2 *)(base + o_dpar);
    a.cgfac = (double *)(base + o_cg);
    a.work = (double2 *)(base + o_work);
    a.part = part;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c->st);
    int n_cg = 0;
    int rc = run_update(a, c->st, &n_cg, cgres);
    cudaEventRecord(e1, c->st);
    if (rc) return fail(c, rc, "update kernels failed");
    CUCHECK(c, cudaMemcpyAsync(par, a.par, sizeof(double2) * manz, cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaMemcpyAsync(dpar, a.dpar, sizeof(double2) * manz, cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaMemcpyAsync(cgfac, a.cgfac, sizeof(double) * manz, cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaStreamSynchronize(c->st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    c->stats.ms_update = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ncg = n_cg;
    return 0;
}

int crgpu_blam0_jtj(crgpu_ctx *c, const double *wmatd, const int32_t *wdfak, int32_t phase_only, double *jtj) {
    if (!c || !wmatd || !wdfak || !jtj) return ERR_ARG;
    if (!c->last_sens) return fail(c, ERR_ARG, "crgpu_blam0_jtj needs the sensitivities (crgpu_sens mode 1) first");
    const int nanz = c->nanz, manz = c->hg.elanz;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    const size_t o_w = take(sizeof(double) * nanz), o_wd = take(sizeof(int32_t) * nanz);
    const size_t o_cg = take(sizeof(double) * manz), o_work = take(update_work_bytes(nanz, manz));
    if (c->upd_bytes < off) {
        if (c->d_upd) cudaFreeAsync(c->d_upd, c->st);
        c->d_upd = nullptr;
        c->upd_bytes = 0;
        cudaError_t e = cudaMallocAsync(&c->d_upd, off, c->st);
        if (e != cudaSuccess) return fail(c, 94, std::string("blam0 work space: ") + cudaGetErrorString(e));
        c->upd_bytes = off;
    }
    char *base = (char *)c->d_upd;
    CUCHECK(c, cudaMemcpyAsync(base + o_w, wmatd, sizeof(double) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(base + o_wd, wdfak, sizeof(int32_t) * nanz, cudaMemcpyHostToDevice, c->st));
    CGArgs a{};
    a.nanz = nanz;
    a.manz = manz;
    a.sens = c->last_sens;
    a.wmatd = (const double *)(base + o_w);
    a.wdfak = (const int32_t *)(base + o_wd);
    a.cgfac = (double *)(base + o_cg);
    a.work = (double2 *)(base + o_work);
    a.part = phase_only ? 1 : 0;  // Re(J) for the final phase improvement and for DC
    int rc = run_jhwj1(a, c->st, jtj);
    if (rc) return fail(c, rc, "blam0 kernels failed");
    return 0;
}

int crgpu_mcm(crgpu_ctx *c, const double *wmatd, const int32_t *wdfak, int32_t ltri, const double *smatm,
              int32_t nx, const int32_t *nachbar, double lam, int32_t flags, double *diag_ata, double *diag_reg,
              double *diag_cov1, double *diag_res, double *diag_cov2) {
    if (!c || !wmatd || !wdfak || !smatm || !diag_ata || !diag_reg || !diag_cov1) return ERR_ARG;
    if (!c->last_sens) return fail(c, ERR_ARG, "crgpu_mcm needs the sensitivities (crgpu_sens mode 1) first");
    if (ltri != 0 && ltri != 1 && ltri != 2)
        return fail(c, ERR_UNSUPPORTED, "crgpu_mcm: regularisation types 0, 1 and 2 only");
    if (ltri != 0 && !nachbar) return ERR_ARG;
    if ((flags & 1) && !diag_res) return ERR_ARG;
    if ((flags & 2) && !diag_cov2) return ERR_ARG;
    const int nanz = c->nanz, manz = c->hg.elanz;
    int nk = 0;
    for (int e = 0; e < manz; e++) nk = std::max(nk, c->hg.etype[e] == 3 ? 3 : 4);
    const int ncol = ltri == 0 ? 3 : nk + 1;
    double *d_w = nullptr, *d_sm = nullptr;
    int32_t *d_wd = nullptr, *d_nb = nullptr;
    int e = dalloc(c, &d_w, nanz);
    if (!e) e = dalloc(c, &d_wd, nanz);
    if (!e) e = dalloc(c, &d_sm, (size_t)manz * ncol);
    if (!e && ltri != 0) e = dalloc(c, &d_nb, (size_t)manz * (nk + 1));
    if (e) return e;
    CUCHECK(c, cudaMemcpyAsync(d_w, wmatd, sizeof(double) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(d_wd, wdfak, sizeof(int32_t) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(d_sm, smatm, sizeof(double) * (size_t)manz * ncol, cudaMemcpyHostToDevice, c->st));
    if (ltri != 0)
        CUCHECK(c, cudaMemcpyAsync(d_nb, nachbar, sizeof(int32_t) * (size_t)manz * (nk + 1), cudaMemcpyHostToDevice,
                                   c->st));
    McmArgs a{};
    a.nanz = nanz;
    a.manz = manz;
    a.ltri = ltri;
    a.nx = nx;
    a.nk = nk;
    a.lam = lam;
    a.sens = c->last_sens;
    a.wmatd = d_w;
    a.wdfak = d_wd;
    a.smatm = d_sm;
    a.nachbar = d_nb;
    a.want_res = (flags & 1) != 0;
    a.want_cov2 = (flags & 2) != 0;
    a.diag_ata = diag_ata;
    a.diag_reg = diag_reg;
    a.diag_cov1 = diag_cov1;
    a.diag_res = diag_res;
    a.diag_cov2 = diag_cov2;
    std::string msg;
    const int rc = run_mcm(a, c->st, msg);
    for (void *p : {(void *)d_w, (void *)d_wd, (void *)d_sm, (void *)d_nb}) {
        if (!p) continue;
        cudaFreeAsync(p, c->st);
        c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), p), c->allocs.end());
    }
    if (rc) return fail(c, rc, msg);
    return 0;
}

int crgpu_column_sums(crgpu_ctx *c, const double *wa, const double *wb, const double *wc, double *c1, double *c2,
                      double *c3) {
    if (!c || !wa || !wb || !wc || !c1 || !c2 || !c3) return ERR_ARG;
    if (!c->last_sens) return fail(c, ERR_ARG, "crgpu_column_sums needs the sensitivities first");
    const int nanz = c->nanz, manz = c->hg.elanz;
    double *w = nullptr, *out = nullptr;
    int e = dalloc(c, &w, (size_t)3 * nanz);
    if (!e) e = dalloc(c, &out, (size_t)3 * manz);
    if (e) return e;
    CUCHECK(c, cudaMemcpyAsync(w, wa, sizeof(double) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(w + nanz, wb, sizeof(double) * nanz, cudaMemcpyHostToDevice, c->st));
    CUCHECK(c, cudaMemcpyAsync(w + 2 * (size_t)nanz, wc, sizeof(double) * nanz, cudaMemcpyHostToDevice, c->st));
    launch_column_sums(nanz, manz, c->last_sens, w, w + nanz, w + 2 * (size_t)nanz, out, out + manz,
                       out + 2 * (size_t)manz, c->st);
    CUCHECK(c, cudaMemcpyAsync(c1, out, sizeof(double) * manz, cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaMemcpyAsync(c2, out + manz, sizeof(double) * manz, cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaMemcpyAsync(c3, out + 2 * (size_t)manz, sizeof(double) * manz, cudaMemcpyDeviceToHost, c->st));
    CUCHECK(c, cudaStreamSynchronize(c->st));
    for (void *p : {(void *)w, (void *)out}) {
        cudaFreeAsync(p, c->st);
        c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), p), c->allocs.end());
    }
    CUCHECK(c, cudaGetLastError());
    return 0;
}

int crgpu_update(crgpu_ctx *c, const double *wmatd, const int32_t *wdfak, const double *dat, const double *sigmaa,
                 int32_t ltri, const double *smatm, int32_t nx, const int32_t *nachbar, double lam, double eps,
                 int32_t ncgmax, double step, double *par, double *dpar, double *cgfac, float *cgres,
                 int32_t *ncg) {
    return update_common(c, 0, wmatd, wdfak, dat, sigmaa, ltri, smatm, nx, nachbar, lam, eps, ncgmax, step, par,
                         dpar, cgfac, cgres, ncg);
}

int crgpu_update_fpi(crgpu_ctx *c, const double *wmatd, const int32_t *wdfak, const double *dat,
                     const double *sigmaa, int32_t ltri, const double *smatm, int32_t nx, const int32_t *nachbar,
                     double lam, double eps, int32_t ncgmax, double step, double *par, double *dpar, double *cgfac,
                     float *cgres, int32_t *ncg) {
    return update_common(c, 1, wmatd, wdfak, dat, sigmaa, ltri, smatm, nx, nachbar, lam, eps, ncgmax, step, par,
                         dpar, cgfac, cgres, ncg);
}

int crgpu_update_dc(crgpu_ctx *c, const double *wmatd, const int32_t *wdfak, const double *dat,
                    const double *sigmaa, int32_t ltri, const double *smatm, int32_t nx, const int32_t *nachbar,
                    double lam, double eps, int32_t ncgmax, double step, double *par, double *dpar, double *cgfac,
                    float *cgres, int32_t *ncg) {
    return update_common(c, 2, wmatd, wdfak, dat, sigmaa, ltri, smatm, nx, nachbar, lam, eps, ncgmax, step, par,
                         dpar, cgfac, cgres, ncg);
}

}  // extern "C"
