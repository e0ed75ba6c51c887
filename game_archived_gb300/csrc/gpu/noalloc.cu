/*
 * game_gpu_weighted_sums_noalloc: the compensated weighted-sum reduction of
 * global_scalar_integrator / game_gpu_write_out_integral (the k_integral
 * kernel of diag_f64.cu) for callers that must not allocate device memory.
 *
 * Who cannot allocate, and why: cudaMalloc and cudaFree synchronise the whole
 * device, so a host model that keeps several streams busy (transfers of the
 * next step overlapping the current one, other libraries' work) would stall
 * all of them for one diagnostic; and an application that has handed its
 * device memory to its own pool up front has nothing left for a library to
 * take.  The context-based entry points allocate only in game_gpu_init, but
 * they need that context and host buffers; this entry point needs neither.
 *
 * Scratch.  The reduction needs, per field, one (hi, lo) pair of doubles per
 * block and one counter.  They live in the file-scope array below, fixed at
 * INTEGRAL_MAX_FIELDS fields x INTEGRAL_MAX_BLOCKS blocks: 77,824 bytes of
 * partial sums plus 8 counters (77,856 bytes, 256-byte aligned).  The
 * counters must be zero when a launch starts.  A __device__ variable is
 * zero-initialised when the device code is loaded, and every launch leaves
 * the counters at zero again (the last block of each field resets its
 * counter), so no call ever writes them from the host: a host-side clear
 * would be ordered only on the stream it was issued on, not before a kernel
 * on the caller's non-blocking stream.  The partial sums need no initial
 * value.
 *
 * First call per device.  The first call with a given device current looks
 * up the device address of the scratch array (cudaGetSymbolAddress, which
 * may load this library's device code) and keeps it for that device.  Make
 * that first call before any stream capture begins, e.g. once right after
 * selecting the device.  Later calls only launch the kernel.  The address is
 * kept for the life of the process: after cudaDeviceReset the device code is
 * loaded anew at another address, so do not call this entry point on a
 * device that has been reset since its first call.
 *
 * Concurrency.  All calls on one device share the one scratch array.  Two
 * calls whose kernels can run at the same time (different streams without an
 * event between them, or different host threads) race on it and return
 * wrong sums.  Issue the calls of one device in one stream, or order them.
 */
#include <mutex>
#include <string>

#include "context.h"
#include "diag.h"
#include "game_gb300.h"

namespace game {
namespace {

struct NoallocScratch {
    double partials[2 * INTEGRAL_MAX_BLOCKS * INTEGRAL_MAX_FIELDS];
    unsigned counters[INTEGRAL_MAX_FIELDS];
};
static_assert(sizeof(NoallocScratch) == 77856, "scratch size as documented");

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

constexpr int MAX_DEVICES = 64;
NoallocScratch *g_scratch_ptr[MAX_DEVICES] = {};
std::mutex g_setup_mutex;

/* device address of the scratch on the current device, set up on first use */
NoallocScratch *scratch_for_current_device()
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        fail(std::string("weighted_sums_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return nullptr;
    }
    if (dev < 0 || dev >= MAX_DEVICES) {
        fail("weighted_sums_noalloc: device ordinal beyond the 64 this library tracks");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_ptr[dev]) return g_scratch_ptr[dev];
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        fail(std::string("weighted_sums_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return nullptr;
    }
    NoallocScratch *s = (NoallocScratch *)p;
    g_scratch_ptr[dev] = s;
    return s;
}

}  // namespace
}  // namespace game

using namespace game;

extern "C" int game_gpu_weighted_sums_noalloc(const double *fields, int n_fields, long long n, const double *weights,
                                              double *sums, void *stream)
{
    if (n_fields < 1 || n_fields > INTEGRAL_MAX_FIELDS)
        return fail("weighted_sums_noalloc: n_fields must be between 1 and 8 (the scratch holds 8 fields), got " +
                    std::to_string(n_fields));
    if (n < 0) return fail("weighted_sums_noalloc: negative field length");
    if ((n > 0 && (!fields || !weights)) || !sums) return fail("weighted_sums_noalloc: null device pointer");
    NoallocScratch *s = scratch_for_current_device();
    if (!s) return -1;
    return launch_integral(fields, n, n_fields, n, nullptr, weights, s->partials, s->counters, sums,
                           (cudaStream_t)stream);
}
