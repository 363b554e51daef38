/*
 * TileSch.h -- the reference's ready-task FIFO (Hybrid3 TileSch.h:17-123), same
 * types, constants and prototypes.  These host functions are thread-safe (a
 * mutex replaces `omp critical (tilsch)`).  The GPU factorization does not use
 * them: its scheduler is the device-resident equivalent (dependency counters
 * plus lock-free FIFOs of task ids inside the persistent DAG kernel).
 */
#ifndef HYBRID3_GB300_TILESCH_H_
#define HYBRID3_GB300_TILESCH_H_
#include <stdio.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct list_data {
    long int i;
    long int j;
    long int k;
    unsigned int priority;
    unsigned int data;
} TilSch_t;

typedef struct list_data_pry {
    TilSch_t pos;
    unsigned int priority;
} TilSch_sch_t;

typedef struct list_data_table {
    TilSch_t pos;
    unsigned int depend;
} TilSch_table_t;

typedef struct list_data_buff {
    TilSch_t pos;
    double *pointer;
    long int life;
} TilSch_buff_t;

typedef struct sche_list {
    TilSch_t *list;
    long int head;
    long int tail;
    long int max;
    long int max_size;
} TilSch_List_t;

typedef struct sche_table {
    TilSch_table_t *list;
    long int head;
    long int tail;
    long int max;
    long int use;
} TilSch_Table_t;

typedef struct sche_buff {
    TilSch_buff_t *list;
    long int head;
    long int tail;
    long int max;
    long int use;
    int buff_size;
} TilSch_Buff_t;

/* TileSch.c:10 -- empty ring of `max` entries. */
void TilSch_init(TilSch_List_t *list, long int max);
/* TileSch.c:19 -- 1 and the oldest entry, or 0 when empty. */
int TilSch_pop(TilSch_List_t *list, TilSch_t *data);
/* TileSch.c:40 -- 1, or 0 when full. */
int TilSch_push(TilSch_List_t *list, TilSch_t data);
/* TileSch.c:64 */
int TilSch_empty(TilSch_List_t *list);
/* TileSch.c:77 */
int TilSch_fully(TilSch_List_t *list);
/* TileSch.c:89 -- prints the ring counters (debug aid); frees nothing, like the reference. */
void TilSch_end(TilSch_List_t *list);
/* TileSch.c:96 -- OR add_depend into the queued entry (i,j,k); returns 1 when
 * its dependency bits reach TSDep_END; a missing entry is appended. */
int TilSch_depend(TilSch_List_t *list, TilSch_t data, unsigned int add_depend);
/* TileSch.c:146 -- remove the entry (i,j,k); 1 if found. */
int TilSch_delete(TilSch_List_t *list, TilSch_t data);

#define TSNONE (0x0000)
#define TSFULL (0xffff)
#define TSFilter1 (0x000f)
#define TSFilter2 (0x00f0)
#define TSFilter3 (0x0f00)
#define TSFilter4 (0xf000)
#define TSDep_MEM (0x0001)
#define TSDep_LIN (0x0002)
#define TSDep_YT (0x0004)
#define TSDep_END (0x0007)
#define TSKa_GEQ (0x0010)
#define TSKa_TSQ (0x0020)
#define TSKa_LAR (0x0030)
#define TSKa_SSR (0x0040)
#define TSKa_SEC (0x00a0)
#define TSKa_REC (0x00b0)

#ifdef __cplusplus
}
#endif
#endif
