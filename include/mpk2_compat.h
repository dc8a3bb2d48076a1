/*
 * mpk2-compatible C ABI exported by libmpk_gb300.so.
 *
 * These are the entry points and data structures of the reference mpk2
 * library (vatai/mpk, mpk2/lib.h).  The structures keep the reference's
 * field order and types so that programs written against mpk2/lib.h
 * (mpk2/mpktest.c, mpk2/comp.c, mpk2/skirt.c, ...) relink against this
 * library unchanged.  Each declaration names the reference declaration it
 * replaces.
 *
 * Differences from the reference, by design:
 *  - exec_mpk* run the task lists on the GPU (one CUDA stream per mpk_t);
 *    `nthread` is accepted and ignored.  The first call uploads the graph
 *    and task lists; later calls reuse them until del_mpk().
 *  - comp_level, update_level and comp_skirt use bounded breadth-first
 *    searches instead of whole-graph min-plus sweeps; their outputs are
 *    identical to the reference's.
 *  - Errors never call exit(): functions that return a pointer return
 *    NULL, functions that return void record the error, readable with
 *    mpk2_last_error(), and leave their outputs untouched.
 */
#ifndef MPK2_COMPAT_H
#define MPK2_COMPAT_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* mpk2/lib.h:10-14 */
typedef struct {
  int n;    /* number of vertices (rows) */
  int *ptr; /* row pointers, n+1 entries */
  int *col; /* 0-based column indices, capacity 2*ne */
} crs0_t;

/* mpk2/lib.h:16 */ crs0_t *new_crs(int nv, int ne);
/* mpk2/lib.h:17 */ void del_crs(crs0_t *g);
/* mpk2/lib.h:18 (METIS text graph; closes f) */ crs0_t *read_crs(FILE *f);
/* mpk2/lib.h:19 (closes f) */ void write_crs(FILE *f, crs0_t *g);

/* mpk2/lib.h:21-25 */
typedef struct {
  crs0_t *g;
  double *x;
  double *y;
} coord_t;

/* mpk2/lib.h:27 */ coord_t *new_coord(crs0_t *g);
/* mpk2/lib.h:28 (closes f) */ void read_coord(FILE *f, coord_t *cg);

/* mpk2/lib.h:30-34 */
typedef struct {
  crs0_t *g;
  int n_part;
  int *part;
} part_t;

/* mpk2/lib.h:36 */ part_t *new_part(crs0_t *g);
/* mpk2/lib.h:37 */ void del_part(part_t *pg);
/* mpk2/lib.h:38 (does not close f, as the reference) */ void read_part(FILE *f, part_t *pg);
/* mpk2/lib.h:39 (closes f) */ void write_part_c(FILE *f, part_t *pg, coord_t *cg);

/* mpk2/lib.h:41-44 */
typedef struct {
  part_t *pg;
  int *level;
} level_t;

/* mpk2/lib.h:46 */ level_t *new_level(part_t *pg);
/* mpk2/lib.h:47 */ void del_level(level_t *lg);
/* mpk2/lib.h:48 */ void comp_level(level_t *lg);
/* mpk2/lib.h:49 */ void update_level(level_t *lg, level_t *lg_org);
/* mpk2/lib.h:50 (closes f) */ void read_level(FILE *f, level_t *lg);
/* mpk2/lib.h:51 (closes f) */ void write_level(FILE *f, level_t *lg);
/* mpk2/lib.h:52 (closes f) */ void write_level_c(FILE *f, level_t *lg, coord_t *cg);

/* mpk2/lib.h:54-58 */
typedef struct {
  crs0_t *g;
  int *wv;
  int *we;
} wcrs_t;

/* mpk2/lib.h:60 */ wcrs_t *new_wcrs(crs0_t *g);
/* mpk2/lib.h:61 */ void del_wcrs(wcrs_t *wg);
/* mpk2/lib.h:62 (closes f) */ void write_wcrs(FILE *f, wcrs_t *wg);
/* mpk2/lib.h:64 */ void level2wcrs(level_t *lg, wcrs_t *wg);

/* mpk2/lib.h:66-69 */
typedef struct {
  part_t *pg;
  int *levels; /* n_part * n entries */
} skirt_t;

/* mpk2/lib.h:71 */ skirt_t *new_skirt(part_t *pg);
/* mpk2/lib.h:72 */ void del_skirt(skirt_t *sg);
/* mpk2/lib.h:73 */ void comp_skirt(skirt_t *sg);
/* mpk2/lib.h:75 (closes f) */ void read_skirt(FILE *f, skirt_t *sg, int level);
/* mpk2/lib.h:76 (closes f) */ void write_skirt(FILE *f, skirt_t *sg, level_t *lg, int level);

/* mpk2/lib.h:78-83 */
typedef struct {
  int n;
  long *idx;
  int th;
  double t0, t1;
} task_t;

/* mpk2/lib.h:85-99 */
typedef struct {
  int n;
  int npart;
  int nlevel;
  int nphase;

  crs0_t *g0;
  part_t **plist;
  level_t **llist;
  skirt_t *sg;

  task_t *tlist;
  long *idxsrc;
  long idxallocsize;
} mpk_t;

/* mpk2/lib.h:101 */ mpk_t *new_mpk(crs0_t *g0, int npart, int nlevel, int nphase);
/* mpk2/lib.h:102 (directory named ghead_npart_nlevel_nphase) */ mpk_t *read_mpk(char *dir);
/* mpk2/lib.h:103 (declared there as a TODO; implemented here) */ void del_mpk(mpk_t *mg);
/* mpk2/lib.h:104 (vv: (nlevel+1)*n doubles of scratch, as the reference) */
void prep_mpk(mpk_t *mg, double *vv);
/* mpk2/lib.h:105-109: GPU execution of the task lists, 1/deg operator */
void exec_mpk(mpk_t *mg, double *vv, int nthread);
void exec_mpk_xs(mpk_t *mg, double *vv, int nthread);
void exec_mpk_xd(mpk_t *mg, double *vv, int nthread);
void exec_mpk_is(mpk_t *mg, double *vv, int nthread);
void exec_mpk_id(mpk_t *mg, double *vv, int nthread);
/* mpk2/lib.h:110-111: k chained SpMVs on the GPU, 1/deg operator */
void spmv_exec_seq(crs0_t *g0, double *vv, int nlevel);
void spmv_exec_par(crs0_t *g0, double *vv, int nlevel, int nth);
/* mpk2/mpkvexec.c:41 (declared ad hoc in mpk2/mpkrun.c:10): valued operator */
void vexec_mpk(mpk_t *mg, double *vv, double *val);
/* mpk2/mpktexec.c:39: transposed layout vv[i*(nlevel+1)+l] */
void exec_mpkt(mpk_t *mg, double *vv, int nth);

/* ---- MPI-2 prep (mpk2/comm_data.h, mpk2/buffers.h) ---------------------- */

/* mpk2/comm_data.h:10-22 */
typedef struct comm_table {
  char *dir;
  int n;
  int nlevel;
  int npart;
  int nphase;
  int rank;
  crs0_t *graph;
  part_t **plist;
  level_t **llist;
  skirt_t *skirt;
} comm_data_t;

/* mpk2/comm_data.h:24 (records the error instead of exiting) */ void dir_name_error(char *dir);
/* mpk2/comm_data.h:26: dir/loop.g0 */ crs0_t *read_matrix(char *dir);
/* mpk2/comm_data.h:28: <dir up to its first '_'>.loop.val */ double *alloc_read_val(crs0_t *g0, char *dir);
/* mpk2/comm_data.h:30 */ comm_data_t *new_comm_data(char *dir, int rank);
/* mpk2/comm_data.h:32 */ void del_comm_data(comm_data_t *cd);

/* mpk2/buffers.h:18-100 */
typedef struct buffers_t {
  int n;
  int npart;
  int nlevel;
  int nphase;
  int rank;
  int buf_count;
  int buf_scount;
  int mptr_count;
  int mcol_count;
  int *recvcounts;
  int *sendcounts;
  int *rdispls;
  int *sdispls;
  int *rcount;
  int *mcount;
  int *scount;
  int *rbuf_offsets;
  int *mbuf_offsets;
  int *sbuf_offsets;
  int *mptr_offsets;
  int *mcol_offsets;
  long *idx_buf;
  long *idx_sbuf;
  long *mptr_buf;
  long *mcol_buf;
  double *vv_buf;
  double *vv_sbuf;
  double *mval_buf;
} buffers_t;

/* mpk2/buffers.h:107 (a command-line helper: exits on argc != 2, as the
 * reference) */ void check_args(int argc, char *argv0);
/* mpk2/buffers.h:120 */ buffers_t *new_bufs(comm_data_t *cd);
/* mpk2/buffers.h:128 */ void alloc_val_bufs(buffers_t *bufs);
/* mpk2/buffers.h:136 */ void del_bufs(buffers_t *bufs);
/* mpk2/buffers.h:158: computed for all ranks with sparse communication
 * sets; relabels cd->plist for phases > 0 as the reference does */
void fill_buffers(comm_data_t *cd, buffers_t *bufs);
/* mpk2/buffers.h:171 */ void write_buffers(buffers_t *bufs, char *dir);
/* mpk2/buffers.h:183 */ buffers_t *read_buffers(char *dir, int rank);

/* New: text of the last error recorded by the functions above on the
 * calling thread ("" when none). */
const char *mpk2_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
