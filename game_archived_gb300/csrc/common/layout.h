/*
 * Run-time byte layout of GAME's data structures (src/game_types.h:62-238).
 *
 * The reference fixes the grid size, layer count and moisture switch as
 * compile-time enums (src/game_types.h:12-60), so the size of every struct
 * member depends on them.  This module computes each member's offset from
 * those three numbers with the C ABI's rules for int/double members (natural
 * alignment, identical on x86_64 and aarch64), so that a library built once
 * can accept the reference's own Grid*, Dualgrid*, State*, Diagnostics*,
 * Forcings*, Irreversible_quantities* and Config* pointers.
 */
#ifndef GAME_LAYOUT_H
#define GAME_LAYOUT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum game_struct_id {
    GAME_GRID = 0, GAME_DUALGRID, GAME_STATE, GAME_DIAGNOSTICS, GAME_FORCINGS,
    GAME_IRREV, GAME_CONFIG, GAME_N_STRUCTS
};

typedef struct game_dims {
    int res_id, n_layers, moisture_on;
    /* derived */
    long n_cells, n_edges, n_triangles;          /* NO_OF_SCALARS_H, NO_OF_VECTORS_H, NO_OF_DUAL_SCALARS_H */
    long n_scalars, n_vectors, n_dual_vectors;   /* NO_OF_SCALARS, NO_OF_VECTORS, NO_OF_DUAL_VECTORS */
    long n_curl;                                 /* NO_OF_LAYERS*2*NO_OF_VECTORS_H + NO_OF_VECTORS_H */
    long vpl, dpl;                               /* NO_OF_VECTORS_PER_LAYER, NO_OF_DUAL_VECTORS_PER_LAYER */
    int n_constituents, n_condensed, n_soil;
    long n_latlon;                               /* NO_OF_LATLON_IO_POINTS */
} game_dims;

typedef struct game_member {
    const char *name;
    int is_int;        /* 1: int members, 0: double members */
    long count;        /* elements */
    size_t offset;     /* bytes from the start of the struct */
} game_member;

/* fills d from (res_id, n_layers, moisture_on); returns 0 or -1 on invalid input */
int game_dims_init(game_dims *d, int res_id, int n_layers, int moisture_on);
/* number of members of a struct, or -1 */
int game_layout_count(int struct_id);
/* member i of a struct under dims d; returns 0 or -1 */
int game_layout_member(const game_dims *d, int struct_id, int i, game_member *m);
/* byte offset of a named member, or (size_t)-1 */
size_t game_layout_offset(const game_dims *d, int struct_id, const char *name);
/* sizeof the struct under dims d */
size_t game_layout_sizeof(const game_dims *d, int struct_id);

#ifdef __cplusplus
}
#endif
#endif
