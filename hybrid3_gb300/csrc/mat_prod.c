/* mat_prod.c -- host helpers of the tiled matrix (Hybrid3 mat_prod.c:15-298):
 * status initialisation, the rand()-based input generator, error norms and
 * printing.  One rank only: the MPI gathers of the reference reduce to the
 * local value. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "mat_prod.h"

void mat_init(mat_stat_t *status, long int mat_m, long int mat_n, int tile_m, int tile_n,
              int my_rank, int proc_num)
{
    long int tiles_m = mat_m / tile_m, tiles_n = mat_n / tile_n;
    long int mine = tiles_n / proc_num + ((tiles_n % proc_num) > my_rank ? 1 : 0);
    status->mat_M = mat_m;
    status->mat_N = mat_n;
    status->my_mat_M = mat_m;
    status->my_tile_M = (unsigned)tiles_m;
    status->glob_tile_M = (unsigned)tiles_m;
    status->glob_tile_N = (unsigned)tiles_n;
    status->my_mat_N = (unsigned long)(tile_n * mine);
    status->my_tile_N = (unsigned)mine;
    status->tile_M = (unsigned)tile_m;
    status->tile_N = (unsigned)tile_n;
}

/* Sum over the tile array, column by column, of ||a| - |b||; the largest
 * column sum.  (The reference leaves its accumulator uninitialised; it starts
 * at zero here and, as there, is not reset between columns.) */
double mat_comp2(mat_stat_t *status, double *matA, double *matB, int my_rank, int proc_num)
{
    double e = 0.0, s = 0.0;
    (void)my_rank; (void)proc_num;
    for (unsigned j = 0; j < mat_getLTileN(status); j++)
        for (unsigned jj = 0; jj < mat_getTileN(status); jj++) {
            for (unsigned i = 0; i < mat_getLTileM(status); i++)
                for (unsigned ii = 0; ii < mat_getTileM(status); ii++) {
                    unsigned long p = mat_getPosID(status, i, j, ii, jj);
                    s += fabs(fabs(matA[p]) - fabs(matB[p]));
                }
            s = fabs(s);
            if (s > e) e = s;
        }
    return e;
}

double mat_comp(mat_stat_t *status, double *matA, unsigned int seed, int my_rank, int proc_num)
{
    double e = 0.0, s = 0.0;
    (void)proc_num;
    srand(seed + my_rank);
    for (unsigned j = 0; j < mat_getLTileN(status); j++)
        for (unsigned jj = 0; jj < mat_getTileN(status); jj++) {
            for (unsigned i = 0; i < mat_getLTileM(status); i++)
                for (unsigned ii = 0; ii < mat_getTileM(status); ii++) {
                    double n = (double)rand() / (double)RAND_MAX;
                    s += fabs(fabs(matA[mat_getPosID(status, i, j, ii, jj)]) - fabs(n));
                }
            s = fabs(s);
            if (s > e) e = s;
        }
    return e;
}

double mat_comp3(mat_stat_t *status, double *matE, int my_rank, int proc_num)
{
    double e = 0.0;
    (void)my_rank; (void)proc_num;
    for (unsigned long i = 0; i < mat_getMyN(status); i++) {
        double s = 0.0;
        for (unsigned long j = 0; j < mat_getMyM(status); j++) s += fabs(matE[i * mat_getMyM(status) + j]);
        if (s > e) e = s;
        if (isnan(s)) { e = s; break; }
    }
    return e;
}

static void fill(mat_stat_t *status, double *matA, unsigned int seed, int my_rank, int subtract)
{
    srand(seed + my_rank);
    for (unsigned j = 0; j < mat_getLTileN(status); j++)
        for (unsigned jj = 0; jj < mat_getTileN(status); jj++)
            for (unsigned i = 0; i < mat_getLTileM(status); i++)
                for (unsigned ii = 0; ii < mat_getTileM(status); ii++) {
                    double n = (double)rand() / (double)RAND_MAX;
                    unsigned long p = mat_getPosID(status, i, j, ii, jj);
                    if (subtract) matA[p] -= n; else matA[p] = n;
                }
}

void mat_make(mat_stat_t *status, double *matA, unsigned int seed, int my_rank)
{
    fill(status, matA, seed, my_rank, 0);
}

void mat_remv(mat_stat_t *status, double *matA, unsigned int seed, int my_rank)
{
    fill(status, matA, seed, my_rank, 1);
}

void mat_print(mat_stat_t *status, FILE *out, double *mat, const char *head_string)
{
    const unsigned tr = mat_getTileM(status), tc = mat_getTileN(status);
    const unsigned trn = mat_getLTileM(status), tcn = mat_getLTileN(status);
    fprintf(out, "[%5d] %s\n", 0, head_string);
    for (unsigned i = 0; i < trn; i++)
        for (unsigned k = 0; k < tr; k++) {
            for (unsigned j = 0; j < tcn; j++)
                for (unsigned l = 0; l < tc; l++)
                    fprintf(out, "%lf\t", (mat + (i + trn * j) * tr * tc)[k + tr * l]);
            fprintf(out, "\n");
        }
    fprintf(out, "\n");
    fflush(out);
}

void mat_dprint(mat_stat_t *status, double *out, double *mat)
{
    const unsigned tr = mat_getTileM(status), tc = mat_getTileN(status);
    const unsigned trn = mat_getLTileM(status), tcn = mat_getLTileN(status);
    unsigned long c = 0;
    for (unsigned j = 0; j < tcn; j++)
        for (unsigned l = 0; l < tc; l++)
            for (unsigned i = 0; i < trn; i++)
                for (unsigned k = 0; k < tr; k++) out[c++] = (mat + (i + trn * j) * tr * tc)[k + tr * l];
}

void mat_print_tile(FILE *out, double *tile, const char *head_string, const int tile_row,
                    const int tile_col)
{
    fprintf(out, "%s\n", head_string);
    for (int i = 0; i < tile_row; i++) {
        for (int j = 0; j < tile_col; j++) fprintf(out, "%lf\t", tile[i + tile_row * j]);
        fprintf(out, "\n");
    }
    fprintf(out, "\n");
}
