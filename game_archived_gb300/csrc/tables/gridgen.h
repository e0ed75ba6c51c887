/*
 * Icosahedral-hexagonal C-grid table builder.
 *
 * Produces every grid table the RKHEVI step reads, in the reference's own
 * array layout (Scalar_field = [layer][cell], Vector_field = level blocks of
 * (cells | edges), Dual_vector_field = level blocks of (edges | triangles)),
 * with the grid sizes given at run time instead of as compile-time enums.
 *
 * The algorithms follow GAME's grid generator
 * (grid_generator/src/coordinator.c:112-338): recursive icosahedron bisection,
 * Lloyd iterations towards an SCVT (optimize.c:17-31), the vertical grid
 * (vertical_grid.c:27-348), inner-product weights (inner_product.c:15-60),
 * rhombus interpolation (rhombus_averaging.c:16-273) and the modified TRSK
 * weights of Gassmann (2018) (coriolis.c:16-440).  Topology is built with
 * hash maps and cell rings, so every stage is O(N) per iteration instead of
 * the reference's O(N^2) searches.  Cell, edge and triangle numbering is this
 * builder's own; cells 0..11 are the pentagons, as the step requires.
 */
#ifndef GAME_GRIDGEN_H
#define GAME_GRIDGEN_H

#ifdef __cplusplus
extern "C" {
#endif

enum { GT_DOUBLE = 0, GT_INT = 1 };

typedef struct gt_array {
    char name[48];
    int type;          /* GT_DOUBLE or GT_INT */
    long n;            /* element count */
    void *ptr;
} gt_array;

#define GT_MAX_ARRAYS 96

typedef struct game_tables {
    int res_id, n_layers, n_oro_layers, n_lloyd;
    int n_cells, n_edges, n_triangles;
    double toa, stretching, radius, radius_rescale;
    int n_arrays;
    gt_array arrays[GT_MAX_ARRAYS];
} game_tables;

/* oro_kind: 0 = flat, 1 = Gaussian mountain h*exp(-(d/half_width)^2 * ln 2)
 * centred at (lat0, lon0) in radians; oro_params = {h, half_width_m, lat0, lon0}. */
game_tables *gt_build(int res_id, int n_layers, int n_oro_layers, double toa,
                      double stretching, double radius_rescale, int n_lloyd,
                      int oro_kind, const double *oro_params, int n_threads);
int gt_count(const game_tables *t);
int gt_info(const game_tables *t, int i, const char **name, int *type, long *n, void **ptr);
void *gt_get(const game_tables *t, const char *name, long *n);
void gt_free(game_tables *t);
int gt_dims(const game_tables *t, int *out8);
const char *gt_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
