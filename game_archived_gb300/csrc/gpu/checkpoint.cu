/*
 * Checkpoints for a bit-identical resume of a run.
 *
 * The reference restarts a run from an initial-state file that holds the
 * prognostic State only (src/io/set_initial_state.c:244-336,
 * read_init_data) and begins it as a first step; the lagged fields the step
 * carries from one call to the next (the pressure gradient, the vorticity
 * flux and the kinetic-energy gradient in Forcings, the sedimentation heat
 * and the diffusion branch's fields in Irreversible_quantities, the boundary
 * entries of Diagnostics) start again from scratch, so a restarted run does
 * not continue the uninterrupted one bit for bit.  A checkpoint here holds
 * the State the next step starts from together with the whole Diagnostics,
 * Forcings, Irreversible_quantities and Config structs, after the library's
 * device copies of the lagged fields have been written back into them, so
 * that a run continued from it -- in this process or a new one, resident or
 * not -- performs exactly the operations the uninterrupted run performs.
 *
 * File (little-endian):
 *   8 bytes  magic "GAMECK01"
 *   4 x int32  format version (1), RES_ID, NO_OF_LAYERS, MOISTURE_ON
 *   5 x uint64 sizes of the State, Diagnostics, Forcings,
 *              Irreversible_quantities and Config structs
 *   uint64   FNV-1a (64-bit) digest of the payload, taken over its 64-bit words
 *   payload  the five structs' bytes, in that order
 */
#include <cstdint>
#include <cstdio>
#include <string>

#include "context.h"
#include "game_gb300.h"

namespace game {
void forget_imports();
}

using namespace game;

namespace {

const char CK_MAGIC[8] = {'G', 'A', 'M', 'E', 'C', 'K', '0', '1'};
constexpr int CK_VERSION = 1;
constexpr int N_PARTS = 5;

struct CkHeader {
    char magic[8];
    int32_t version, res_id, n_layers, moisture_on;
    uint64_t sizes[N_PARTS];
    uint64_t digest;
};
static_assert(sizeof(CkHeader) == 8 + 16 + 8 * N_PARTS + 8, "checkpoint header has padding");

/* FNV-1a over 64-bit words (the sizes of the structs are multiples of 8) */
struct Fnv {
    uint64_t h = 1469598103934665603ULL;
    void add(const void *p, size_t bytes)
    {
        const uint64_t *w = (const uint64_t *)p;
        for (size_t i = 0; i < bytes / 8; ++i) {
            h ^= w[i];
            h *= 1099511628211ULL;
        }
        const unsigned char *b = (const unsigned char *)p + (bytes / 8) * 8;
        for (size_t i = 0; i < bytes % 8; ++i) {
            h ^= b[i];
            h *= 1099511628211ULL;
        }
    }
};

int part_sizes(Context *c, uint64_t sizes[N_PARTS])
{
    const int sids[N_PARTS] = {GAME_STATE, GAME_DIAGNOSTICS, GAME_FORCINGS, GAME_IRREV, GAME_CONFIG};
    for (int k = 0; k < N_PARTS; ++k) sizes[k] = (uint64_t)game_layout_sizeof(&c->dims, sids[k]);
    return 0;
}

}  // namespace

extern "C" int game_gpu_write_checkpoint(const char *path, struct state *state, struct diagnostics *diagnostics,
                                         struct forcings *forcings, struct irreversible_quantities *irrev,
                                         struct config *config)
{
    Context *c = ctx();
    if (!c) return fail("game_gpu_init has not been called");
    if (!path || !state || !diagnostics || !forcings || !irrev || !config)
        return fail("write_checkpoint: null argument");
    /* the device copies: the State of a resident run, and the lagged fields
     * (always device-resident between steps) */
    if (c->resident && mirror(state, 0) && game_gpu_sync_to_host(state)) return -1;
    if (game_gpu_sync_aux_to_host(diagnostics, forcings, irrev)) return -1;
    CkHeader h{};
    for (int k = 0; k < 8; ++k) h.magic[k] = CK_MAGIC[k];
    h.version = CK_VERSION;
    h.res_id = c->dims.res_id;
    h.n_layers = c->nl;
    h.moisture_on = c->moist;
    part_sizes(c, h.sizes);
    const void *parts[N_PARTS] = {state, diagnostics, forcings, irrev, config};
    Fnv f;
    for (int k = 0; k < N_PARTS; ++k) f.add(parts[k], h.sizes[k]);
    h.digest = f.h;
    const std::string tmp = std::string(path) + ".partial";
    FILE *fp = fopen(tmp.c_str(), "wb");
    if (!fp) return fail(std::string("write_checkpoint: cannot open ") + tmp);
    bool ok = fwrite(&h, sizeof h, 1, fp) == 1;
    for (int k = 0; k < N_PARTS && ok; ++k) ok = fwrite(parts[k], 1, h.sizes[k], fp) == h.sizes[k];
    ok = (fclose(fp) == 0) && ok;
    if (!ok) {
        remove(tmp.c_str());
        return fail(std::string("write_checkpoint: writing ") + tmp + " failed");
    }
    if (rename(tmp.c_str(), path) != 0) return fail(std::string("write_checkpoint: cannot rename to ") + path);
    return 0;
}

extern "C" int game_gpu_read_checkpoint(const char *path, struct state *state, struct diagnostics *diagnostics,
                                        struct forcings *forcings, struct irreversible_quantities *irrev,
                                        struct config *config)
{
    Context *c = ctx();
    if (!c) return fail("game_gpu_init has not been called");
    if (!path || !state || !diagnostics || !forcings || !irrev || !config)
        return fail("read_checkpoint: null argument");
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(std::string("read_checkpoint: cannot open ") + path);
    CkHeader h{};
    if (fread(&h, sizeof h, 1, fp) != 1) {
        fclose(fp);
        return fail(std::string("read_checkpoint: ") + path + " is too short");
    }
    for (int k = 0; k < 8; ++k)
        if (h.magic[k] != CK_MAGIC[k]) {
            fclose(fp);
            return fail(std::string("read_checkpoint: ") + path + " is not a checkpoint");
        }
    uint64_t sizes[N_PARTS];
    part_sizes(c, sizes);
    bool match = h.version == CK_VERSION && h.res_id == c->dims.res_id && h.n_layers == c->nl &&
                 h.moisture_on == c->moist;
    for (int k = 0; k < N_PARTS; ++k) match = match && h.sizes[k] == sizes[k];
    if (!match) {
        fclose(fp);
        return fail("read_checkpoint: the checkpoint was written for RES_ID " + std::to_string(h.res_id) + ", " +
                    std::to_string(h.n_layers) + " layers, moisture " + std::to_string(h.moisture_on) +
                    " (format " + std::to_string(h.version) + "); this context has RES_ID " +
                    std::to_string(c->dims.res_id) + ", " + std::to_string(c->nl) + " layers, moisture " +
                    std::to_string(c->moist));
    }
    void *parts[N_PARTS] = {state, diagnostics, forcings, irrev, config};
    bool ok = true;
    Fnv f;
    for (int k = 0; k < N_PARTS && ok; ++k) {
        ok = fread(parts[k], 1, h.sizes[k], fp) == h.sizes[k];
        if (ok) f.add(parts[k], h.sizes[k]);
    }
    fclose(fp);
    if (!ok) return fail(std::string("read_checkpoint: ") + path + " is truncated; the structs are undefined");
    if (f.h != h.digest)
        return fail(std::string("read_checkpoint: ") + path +
                    " does not match its digest (corrupted); the structs are undefined");
    /* the next step imports the lagged fields from these structs again */
    forget_imports();
    if (c->resident && game_gpu_sync_to_device(state)) return -1;
    return 0;
}
