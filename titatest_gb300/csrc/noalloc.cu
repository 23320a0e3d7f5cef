// crgpu_factor_system_noalloc: the band factor of one (wavenumber, electrode)
// system for callers that cannot allocate device memory when they call: a
// host framework that hands out all device memory from its own pool (its
// budget leaves nothing for allocations outside it), or a host that must not
// make the implicit device-wide synchronisation of cudaMalloc/cudaFree in the
// middle of its work.  The caller passes the conductivities and the two
// output buffers (device memory); everything the kernels need in between,
// including their error word, lives in one file-scope device array.
//
// The array (kScratchBytes) exists once on every GPU that loads the library
// and stays allocated until the process exits.  Its device address is looked
// up (cudaGetSymbolAddress) by the first call on each device, with that
// device current; make that first call before any stream capture starts.
// Every call shares the array and leaves its contents behind, so calls whose
// work overlaps on the GPU (other streams, other host threads) race.
#include <mutex>

#include "ctx.h"

using namespace crgpu;

namespace {

constexpr size_t kScratchBytes = 8u << 20;  // 8 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

// status word, system wavenumber (relative), electrode of the batch of one,
// and the problem-wide error word (kept here, not in the context)
__global__ void k_noalloc_init(int *ints, int l) {
    ints[0] = 0;  // status: the kernels record errors with atomicCAS from 0
    ints[1] = 0;  // k relative to the shifted element arrays
    ints[2] = l;
    ints[3] = 0;  // error word of the assembly and factor kernels
}

int fail(crgpu_ctx *c, int code, const std::string &msg) {
    c->last_error = msg;
    return code;
}

}  // namespace

extern "C" int crgpu_factor_system_noalloc(crgpu_ctx *c, const void *sigma_device, int32_t k, int32_t l,
                                           void *a_device, void *fak_device, void *stream) {
    if (!c || !sigma_device || !a_device || !fak_device) return ERR_ARG;
    if (k < 1 || k > c->K || l < 1 || l > c->eanz) return fail(c, ERR_ARG, "system (k, l) out of range");
    if (c->precision != CRGPU_PLAIN) return fail(c, ERR_UNSUPPORTED, "no-alloc factor: plain precision only");
    if (c->P.ldc) return fail(c, ERR_UNSUPPORTED, "no-alloc factor: not available in DC mode");
    if (!c->old_of_new.empty())
        return fail(c, ERR_UNSUPPORTED, "no-alloc factor: the context factors in the geometric node order");
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != c->device || dev >= kMaxDevices)
        return fail(c, ERR_ARG, "no-alloc factor: the context's device must be current");
    const DevProblem &P = c->P;
    const size_t nnz = P.nnz, n = P.n;
    const size_t need = 16 + 16 * (2 * nnz + 2 * n);
    if (need > kScratchBytes)
        return fail(c, ERR_ARG, "no-alloc factor: the system needs " + std::to_string(need) +
                                    " bytes of scratch, more than the fixed " + std::to_string(kScratchBytes));
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_addr[dev]) {
            void *ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return fail(c, ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_addr[dev] = ptr;
        }
        base = (unsigned char *)g_scratch_addr[dev];
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : c->st;
    int *ints = (int *)base;
    // launch_adom writes the area parts (nnz) and then fak_area (n doubles) into
    // the start of `as`; k_fak reads fak_area there before k_assemble_entries
    // overwrites the region with the scaled entries (same stream)
    double2 *adom = (double2 *)(base + 16);
    double2 *as = adom + nnz;
    double2 *b = as + nnz;
    double2 *y = b + n;
    // element arrays shifted to wavenumber k, so that the batch sees k = 0
    DevProblem Pk = P;
    Pk.K = 1;
    Pk.err = ints + 3;  // the context's own error word is left alone
    Pk.elbg = P.elbg + (size_t)(k - 1) * P.elanz * 10;
    Pk.kg = P.kg + (size_t)(k - 1) * P.eanz * P.relanz;
    const int32_t ll = c->hg.lbeta ? l - 1 : 0;
    DevBatch B{};
    B.nsys = 1;
    B.ks = ints + 1;
    B.ls = ints + 2;
    B.As = as;
    B.fak = (double *)fak_device;
    B.b = b;
    B.y = y;
    B.L = a_device;
    B.lpitch = (size_t)c->hg.n * (c->hg.mb + 1);  // one system
    B.status = ints;
    k_noalloc_init<<<1, 1, 0, st>>>(ints, ll);
    launch_adom(Pk, (const double2 *)sigma_device, adom, st);
    launch_assemble(Pk, B, (const double2 *)sigma_device, adom, st);
    launch_rhs(Pk, B, 1, c->lsink, c->nsink, st);
    launch_factor_plain(Pk, B, 1, c->nsm, st);
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) return fail(c, ERR_CUDA, cudaGetErrorString(ce));
    // the call waits for its kernels and reads the two status words back
    int h[4] = {0, 0, 0, 0};
    if (cudaMemcpyAsync(h, ints, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(c, ERR_CUDA, "no-alloc factor: status read-back failed");
    if (h[3]) return fail(c, h[3], "device reported error " + std::to_string(h[3]));
    if (h[0]) return fail(c, h[0], "system failed with error " + std::to_string(h[0]));
    return 0;
}
