/* tilesch.c -- the TileSch ready-task FIFO (Hybrid3 TileSch.c:10-173) as a
 * thread-safe host ring.  A process-wide mutex plays the part of the
 * reference's `omp critical (tilsch)`. */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>

#include "TileSch.h"

static pthread_mutex_t tilsch_mu = PTHREAD_MUTEX_INITIALIZER;

void TilSch_init(TilSch_List_t *list, long int max)
{
    list->head = 0;
    list->tail = 0;
    list->max = max;
    list->max_size = 0;
    list->list = (TilSch_t *)calloc((size_t)(max > 0 ? max : 1), sizeof(TilSch_t));
}

int TilSch_pop(TilSch_List_t *list, TilSch_t *data)
{
    int ok = 0;
    pthread_mutex_lock(&tilsch_mu);
    if (list->tail > list->head) {
        *data = list->list[list->head % list->max];
        list->head++;
        ok = 1;
    }
    pthread_mutex_unlock(&tilsch_mu);
    return ok;
}

int TilSch_push(TilSch_List_t *list, TilSch_t data)
{
    int ok = 0;
    pthread_mutex_lock(&tilsch_mu);
    if (list->tail - list->head < list->max) {
        list->list[list->tail % list->max] = data;
        list->tail++;
        if (list->tail - list->head > list->max_size) list->max_size = list->tail - list->head;
        ok = 1;
    }
    pthread_mutex_unlock(&tilsch_mu);
    return ok;
}

int TilSch_empty(TilSch_List_t *list)
{
    pthread_mutex_lock(&tilsch_mu);
    int r = list->tail <= list->head;
    pthread_mutex_unlock(&tilsch_mu);
    return r;
}

int TilSch_fully(TilSch_List_t *list)
{
    pthread_mutex_lock(&tilsch_mu);
    int r = list->max <= list->tail - list->head;
    pthread_mutex_unlock(&tilsch_mu);
    return r;
}

void TilSch_end(TilSch_List_t *list)
{
    printf("Q_size[%ld,%ld,%ld,%ld]\n", list->head, list->tail, list->max, list->max_size);
}

/* The queued entries live at ring positions head..tail-1 (taken modulo max;
 * the reference indexes them without the modulo). */
int TilSch_depend(TilSch_List_t *list, TilSch_t data, unsigned int add_depend)
{
    int flag = 0;
    pthread_mutex_lock(&tilsch_mu);
    if (add_depend == TSDep_END) {
        flag = 1;
    } else {
        long l, found = -1;
        for (l = list->head; l < list->tail; l++) {
            TilSch_t *e = &list->list[l % list->max];
            if (e->i == data.i && e->j == data.j && e->k == data.k) { found = l; break; }
        }
        if (found >= 0) {
            TilSch_t *e = &list->list[found % list->max];
            e->data |= add_depend;
            flag = ((e->data & TSFilter1) == TSDep_END);
        } else if (list->tail - list->head < list->max) {
            list->list[list->tail % list->max] = data;
            list->list[list->tail % list->max].data = add_depend;
            list->tail++;
            if (list->tail - list->head > list->max_size) list->max_size = list->tail - list->head;
        }
    }
    pthread_mutex_unlock(&tilsch_mu);
    return flag;
}

int TilSch_delete(TilSch_List_t *list, TilSch_t data)
{
    int flag = 0;
    pthread_mutex_lock(&tilsch_mu);
    long l;
    for (l = list->head; l < list->tail; l++) {
        TilSch_t *e = &list->list[l % list->max];
        if (e->i == data.i && e->j == data.j && e->k == data.k &&
            (e->data & TSFilter3) == ((unsigned)data.i & TSFilter3)) { flag = 1; break; }
    }
    if (flag) {
        for (l++; l < list->tail; l++) list->list[(l - 1) % list->max] = list->list[l % list->max];
        list->tail--;
    }
    pthread_mutex_unlock(&tilsch_mu);
    return flag;
}
