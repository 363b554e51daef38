/*
 * mat_prod.h -- tiled-matrix status and helpers (drop-in for Hybrid3's
 * mat_prod.h:12-67; same struct layout, macro names and prototypes).
 *
 * Tile (i,j) of an MT x NT grid of NB x NB tiles starts at (i + j*MT)*NB*NB
 * and is column-major with leading dimension NB.  With one rank (the only
 * configuration of this library) my_* fields equal the global ones.
 */
#ifndef HYBRID3_GB300_MAT_PROD_H_
#define HYBRID3_GB300_MAT_PROD_H_
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* mat_stat_t (mat_prod.h:12-25 of the reference). */
typedef struct mstatus {
    unsigned long int mat_M;     /* rows */
    unsigned long int mat_N;     /* columns */
    unsigned long int my_mat_M;  /* rows held by this rank */
    unsigned long int my_mat_N;  /* columns held by this rank */
    unsigned int tile_M;         /* tile rows (NB) */
    unsigned int tile_N;         /* tile columns (NB) */
    unsigned int glob_tile_M;    /* MT */
    unsigned int glob_tile_N;    /* NT */
    unsigned int my_tile_M;      /* tile rows held by this rank */
    unsigned int my_tile_N;      /* tile columns held by this rank */
} mat_stat_t;

/* mat_init (mat_prod.c:15-37): tile counts mat / tile (truncating); rank
 * my_rank of proc_num holds every tile row and tile columns g with
 * g % proc_num == my_rank, so my_mat_N = tile_n * (its tile columns) while
 * my_mat_M = mat_m as given, as in the reference. */
void mat_init(mat_stat_t *status, long int mat_m, long int mat_n, int tile_m, int tile_n,
              int my_rank, int proc_num);

#define mat_mysize(st) (unsigned long int)(((st)->my_mat_M) * ((st)->my_mat_N))
#define mat_myTAU(st) (unsigned long int)(((st)->my_mat_M / 2) * ((st)->my_mat_N / 2))
#define mat_TileSize(st) (unsigned int)(((st)->tile_M) * ((st)->tile_N))
#define mat_getTileM(st) ((st)->tile_M)
#define mat_getTileN(st) ((st)->tile_N)
#define mat_getM(st) ((st)->mat_M)
#define mat_getN(st) ((st)->mat_N)
#define mat_getMyM(st) ((st)->my_mat_M)
#define mat_getMyN(st) ((st)->my_mat_N)
#define mat_getGTileM(st) ((st)->glob_tile_M)
#define mat_getGTileN(st) ((st)->glob_tile_N)
#define mat_getLTileM(st) ((st)->my_tile_M)
#define mat_getLTileN(st) ((st)->my_tile_N)
#define mat_getPosID(st, ti, tj, si, sj) \
    (((ti) + (tj) * ((st)->my_tile_M)) * ((st)->tile_M) * ((st)->tile_N) + (si) + (sj) * ((st)->tile_M))
#define mat_getMatPos(st, i, j) \
    (((i) + (j) * ((st)->my_tile_M)) * ((unsigned int)(((st)->tile_M) * ((st)->tile_N))))
#define mat_getVecPos(st, i, j) (((i) + (j) * ((st)->my_tile_M)) * ((unsigned int)((st)->tile_N)))

/* Error measures (mat_prod.c:42-154).  mat_comp3 returns the largest column
 * abs-sum (the 1-norm) of a column-major array and propagates NaN.  mat_comp
 * and mat_comp2 start their sums at zero (the reference reads an
 * uninitialised accumulator there). */
double mat_comp(mat_stat_t *status, double *matA, unsigned int seed, int my_rank, int proc_num);
double mat_comp2(mat_stat_t *status, double *matA, double *matB, int my_rank, int proc_num);
double mat_comp3(mat_stat_t *status, double *matE, int my_rank, int proc_num);

/* Input generators (mat_prod.c:157-208): rand()/RAND_MAX after srand(seed+rank). */
void mat_make(mat_stat_t *status, double *matA, unsigned int seed, int my_rank);
void mat_remv(mat_stat_t *status, double *matA, unsigned int seed, int my_rank);

/* Printing (mat_prod.c:211-298); mat_dprint converts tile layout to column-major. */
void mat_print(mat_stat_t *status, FILE *out, double *mat, const char *head_string);
void mat_dprint(mat_stat_t *status, double *out, double *mat);
void mat_print_tile(FILE *out, double *tile, const char *head_string, const int tile_row,
                    const int tile_col);

#ifdef __cplusplus
}
#endif
#endif
