/*
 * Health check of a State on the device: non-finite values (NaN, +-Inf) in
 * any prognostic field and negative densities of any constituent.
 *
 * The reference aborts when it reads an initial state with a negative
 * density (src/io/set_initial_state.c:318-328) and clips the tracer column
 * solutions at zero (src/time_stepping/column_solvers.c:621-627); a NaN or a
 * negative density in a State after a step therefore means the run has
 * broken down (an unstable time step, corrupted input).  One reduction over
 * the State's device copy counts both and records the first offending
 * element, reported in the reference's State layout; the host reads the
 * counts at the call, which is a synchronisation point.  manage_rkhevi runs
 * it on state_new after every n-th step when game_gpu_set_health_check(n)
 * is on, and then returns GAME_GPU_UNHEALTHY instead of 0.
 */
#include <algorithm>
#include <climits>
#include <string>

#include "context.h"
#include "game_gb300.h"

namespace game {
namespace {

/* counts[0] non-finite, counts[1] negative densities; first[0], first[1]
 * the smallest reference-layout position of each (map: device position ->
 * reference position) */
__global__ void k_health(const double *s, const int *map, long long n_rho, long long n, unsigned long long *counts,
                         unsigned long long *first)
{
    const unsigned lane = threadIdx.x & 31u;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i - lane < n;
         i += (long long)gridDim.x * blockDim.x) {
        const bool in = i < n;
        const double x = in ? s[i] : 0.0;
        const unsigned long long b = in ? (unsigned long long)__double_as_longlong(x) : 0ull;
        const bool bad = in && ((b >> 52) & 0x7ffull) == 0x7ffull; /* exponent all ones: Inf or NaN */
        const bool neg = in && !bad && i < n_rho && x < 0.0;
        const unsigned mb = __ballot_sync(0xffffffffu, bad), mn = __ballot_sync(0xffffffffu, neg);
        if (lane == 0) {
            if (mb) atomicAdd(&counts[0], (unsigned long long)__popc(mb));
            if (mn) atomicAdd(&counts[1], (unsigned long long)__popc(mn));
        }
        if (bad) atomicMin(&first[0], (unsigned long long)map[i]);
        if (neg) atomicMin(&first[1], (unsigned long long)map[i]);
    }
}

}  // namespace

/* checks a State mirror; fills the report (reference-layout indices) and
 * returns 0 when healthy, GAME_GPU_UNHEALTHY when not, -1 on a CUDA error */
int check_mirror(Context *c, StateMirror *m, struct game_gpu_health *report, const char *what)
{
    if (!c->health) {
        void *p = nullptr;
        CK(cudaMalloc(&p, 4 * sizeof(unsigned long long)));
        c->health = (unsigned long long *)p;
    }
    const unsigned long long init[4] = {0ull, 0ull, ULLONG_MAX, ULLONG_MAX};
    CK(cudaMemcpyAsync(c->health, init, sizeof init, cudaMemcpyHostToDevice, c->stream));
    const long long n_rho = (long long)c->n_const * c->ns, n = c->state_len;
    int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 8);
    k_health<<<blocks, 256, 0, c->stream>>>(m->dev, c->map_state, n_rho, n, c->health, c->health + 2);
    c->kernel_launches++;
    CK(cudaGetLastError());
    unsigned long long out[4];
    CK(cudaMemcpyAsync(out, c->health, sizeof out, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    game_gpu_health r{};
    r.nonfinite = (long long)out[0];
    r.negative_density = (long long)out[1];
    r.first_nonfinite = out[0] ? (long long)out[2] : -1;
    r.first_negative_density = out[1] ? (long long)out[3] : -1;
    if (report) *report = r;
    if (r.nonfinite == 0 && r.negative_density == 0) return 0;
    set_error(std::string(what) + ": " + std::to_string(r.nonfinite) + " non-finite values (first at State double " +
              std::to_string(r.first_nonfinite) + ") and " + std::to_string(r.negative_density) +
              " negative densities (first at State double " + std::to_string(r.first_negative_density) + ")");
    return GAME_GPU_UNHEALTHY;
}

}  // namespace game

using namespace game;

extern "C" int game_gpu_check_state(struct state *state, struct game_gpu_health *report)
{
    Context *c = ctx();
    if (!c) return fail("game_gpu_init has not been called");
    if (!state) return fail("check_state: null state");
    StateMirror *m = nullptr;
    if (c->resident) m = mirror(state, 0);
    if (!m) {
        /* host State: checked on the library's scratch copy */
        if (ensure_sub_buffers(c)) return -1;
        m = &c->sub.so;
        if (upload_state(state, m)) return -1;
    }
    return check_mirror(c, m, report, "check_state");
}

extern "C" int game_gpu_set_health_check(int every)
{
    Context *c = ctx();
    if (!c) return fail("game_gpu_init has not been called");
    if (every < 0) return fail("set_health_check: a step count >= 0 expected (0 switches the check off)");
    c->health_every = every;
    c->health_count = 0;
    return 0;
}
