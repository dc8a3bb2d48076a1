/*
 * CPU oracle for the matrix powers kernel (MPK) hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the
 * algorithms of the reference mpk2 code (vatai/mpk) so that tests,
 * `__graft_entry__.smoke()` and the `cpu_baseline` leg of `bench.py`
 * can check the CUDA path against it.  The product library never links,
 * loads or calls anything built from this file.
 *
 * Every function cites the reference file:line it restates.  Parity of
 * this restatement with the reference itself is pinned by the tests in
 * tests/test_oracle_pin.py (against the reference compiled from its own
 * sources into oracle/_ref/) and by the committed golden fixtures in
 * tests/golden/ (generated by tests/golden/make_golden.py from the
 * reference binaries).
 *
 * Arithmetic modes for the FP64 row sums:
 *   mode 0 ("separate"): s = s + (a * x), two roundings per term; this is
 *          what the reference computes when the compiler does not contract
 *          (x86-64 gcc -O2: no FMA instructions are emitted).
 *   mode 1 ("fma"):      s = fma(a, x, s), one rounding per term; this is
 *          what the reference computes when gcc contracts a*b+c (aarch64
 *          gcc -O2 default), and what the CUDA kernels compute by default.
 * The file is compiled with -ffp-contract=off so mode 0 stays mode 0.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>

#define ORC_OK 0
#define ORC_EIO -1
#define ORC_EFORMAT -2
#define ORC_ERANGE -3
#define ORC_ESTRUCT -4

static double row_term(double s, double a, double x, int mode) {
  return mode ? fma(a, x, s) : s + a * x;
}

/* ------------------------------------------------------------------ */
/* Graph input: METIS text format, 1-based columns, header "n ne".      */
/* Restates read_crs (mpk2/lib.c:69-129): one line per vertex, columns  */
/* in file order, col[] capacity 2*ne, every column in [1, n].          */
/* ------------------------------------------------------------------ */

/* Pass 1: header values (n, ne) and the exact number of column tokens. */
long orc_graph_count(const char *path, int *n_out, long *ne_out) {
  FILE *f = fopen(path, "r");
  if (!f) return ORC_EIO;
  int nv = 0, ne = 0, p = 0, q = 0;
  char line[1 << 16];
  if (!fgets(line, sizeof line, f)) { fclose(f); return ORC_EFORMAT; }
  if (sscanf(line, "%d %d %d %d", &nv, &ne, &p, &q) != 2 || nv <= 0 || ne <= 0) {
    fclose(f); return ORC_EFORMAT;
  }
  long cnt = 0;
  int rows = 0;
  int c;
  int in_tok = 0;
  /* count integer tokens on the next nv lines */
  while (rows < nv && (c = fgetc(f)) != EOF) {
    if (c == '\n') { if (in_tok) { cnt++; in_tok = 0; } rows++; continue; }
    if (isdigit(c)) in_tok = 1;
    else if (in_tok) { cnt++; in_tok = 0; }
  }
  if (in_tok) cnt++;
  fclose(f);
  *n_out = nv; *ne_out = ne;
  return cnt;
}

/* Pass 2: fill ptr[n+1], col[cap] (0-based). */
int orc_graph_read(const char *path, int n, long cap, int *ptr, int *col) {
  FILE *f = fopen(path, "r");
  if (!f) return ORC_EIO;
  char line[1 << 16];
  if (!fgets(line, sizeof line, f)) { fclose(f); return ORC_EFORMAT; }
  long p = 0;
  int i = 0;
  ptr[0] = 0;
  int c, in_tok = 0;
  long v = 0;
  while (i < n && (c = fgetc(f)) != EOF) {
    if (isdigit(c)) { v = v * 10 + (c - '0'); in_tok = 1; continue; }
    if (in_tok) {
      if (p >= cap || v < 1 || v > n) { fclose(f); return ORC_ERANGE; }
      col[p++] = (int)(v - 1);
      in_tok = 0; v = 0;
    }
    if (c == '\n') ptr[++i] = (int)p;
  }
  if (in_tok && i < n) {
    if (p >= cap || v < 1 || v > n) { fclose(f); return ORC_ERANGE; }
    col[p++] = (int)(v - 1);
  }
  while (i < n) ptr[++i] = (int)p; /* missing trailing lines: empty rows */
  fclose(f);
  return ORC_OK;
}

/* Values file (.loop.val): whitespace separated doubles in CSR order.
 * Restates alloc_read_val (mpk2/comm_data.c:160-187). */
int orc_read_values(const char *path, long nnz, double *val) {
  FILE *f = fopen(path, "r");
  if (!f) return ORC_EIO;
  for (long i = 0; i < nnz; i++)
    if (fscanf(f, "%lf ", val + i) != 1) { fclose(f); return ORC_EFORMAT; }
  fclose(f);
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* Min-plus relaxation sweeps (mpk2/lib.c:164-219).                      */
/* mode 0: all rows, 1: rows with part[i]==r, 2: rows with part[i]!=r.   */
/* y[i] = min(x[i], x[col]+1); returns the number of strict decreases    */
/* counted per column visit, exactly as the reference counts them.       */
/* ------------------------------------------------------------------ */
long orc_minplus(int n, const int *ptr, const int *col, const int *x, int *y,
                 int r, const int *part, int mode) {
  long k = 0;
  for (int i = 0; i < n; i++) {
    if (mode == 1 && part[i] != r) continue;
    if (mode == 2 && part[i] == r) continue;
    int t = x[i];
    for (int j = ptr[i]; j < ptr[i + 1]; j++) {
      int s = x[col[j]] + 1;
      if (s < t) { t = s; k++; }
    }
    y[i] = t;
  }
  return k;
}

/* Swap-until-no-change loop shared by comp_level, update_level and
 * comp_skirt: the reference iterates minplus_{r,x} between t0 and t1
 * and keeps the array produced by the last sweep. */
static int *fixed_point(int n, const int *ptr, const int *col, int *t0, int *t1,
                        int r, const int *part, int mode) {
  long ch;
  do {
    ch = orc_minplus(n, ptr, col, t0, t1, r, part, mode);
    int *tt = t0; t0 = t1; t1 = tt;
  } while (ch > 0);
  return t1; /* == array written by the last sweep */
}

/* comp_level (mpk2/lib.c:330-371): per part, start from n+1 inside and
 * -1 outside, sweep inside the part to a fixed point. */
int orc_comp_level(int n, const int *ptr, const int *col, const int *part,
                   int npart, int *level) {
  int *t0 = malloc(sizeof(int) * n), *t1 = malloc(sizeof(int) * n);
  if (!t0 || !t1) { free(t0); free(t1); return ORC_EIO; }
  for (int p = 0; p < npart; p++) {
    for (int j = 0; j < n; j++) t0[j] = t1[j] = (part[j] == p) ? n + 1 : -1;
    int *res = fixed_point(n, ptr, col, t0, t1, p, part, 1);
    for (int j = 0; j < n; j++) if (part[j] == p) level[j] = res[j];
  }
  free(t0); free(t1);
  return ORC_OK;
}

/* update_level (mpk2/lib.c:373-412): like comp_level, but vertices
 * outside the part keep the previous phase's level, and vertices inside
 * start from max(level_org) + n + 1. */
int orc_update_level(int n, const int *ptr, const int *col, const int *part,
                     int npart, const int *level_org, int *level) {
  int *t0 = malloc(sizeof(int) * n), *t1 = malloc(sizeof(int) * n);
  if (!t0 || !t1) { free(t0); free(t1); return ORC_EIO; }
  int mx = level_org[0];
  for (int i = 1; i < n; i++) if (mx < level_org[i]) mx = level_org[i];
  for (int p = 0; p < npart; p++) {
    for (int j = 0; j < n; j++) t0[j] = t1[j] = (part[j] == p) ? mx + n + 1 : level_org[j];
    int *res = fixed_point(n, ptr, col, t0, t1, p, part, 1);
    for (int j = 0; j < n; j++) if (part[j] == p) level[j] = res[j];
  }
  free(t0); free(t1);
  return ORC_OK;
}

/* level2wcrs (mpk2/lib.c:504-537): vertex weight max+1-l_i, edge weight
 * (int)(1e6/(l_i + l_j - 2*min + 1)) clamped to >= 1. */
void orc_level2weights(int n, const int *ptr, const int *col, const int *level,
                       int *wv, int *we) {
  int mx = level[0], mn = level[0];
  for (int i = 1; i < n; i++) {
    if (mx < level[i]) mx = level[i];
    if (mn > level[i]) mn = level[i];
  }
  for (int i = 0; i < n; i++) {
    wv[i] = mx + 1 - level[i];
    int l0 = level[i];
    for (int j = ptr[i]; j < ptr[i + 1]; j++) {
      double w = l0 + level[col[j]] - 2 * mn;
      w = 1e+6 / (w + 1);
      we[j] = (w < 1.0) ? 1 : (int)w;
    }
  }
}

/* comp_skirt for one part (mpk2/lib.c:584-615): 0 inside the part, n+1
 * outside, sweep the outside to a fixed point: dist[j] is the graph
 * distance of j to part p (n+1 when unreachable). */
int orc_skirt_dist(int n, const int *ptr, const int *col, const int *part,
                   int p, int *dist) {
  int *t0 = malloc(sizeof(int) * n), *t1 = malloc(sizeof(int) * n);
  if (!t0 || !t1) { free(t0); free(t1); return ORC_EIO; }
  for (int j = 0; j < n; j++) t0[j] = t1[j] = (part[j] == p) ? 0 : n + 1;
  int *res = fixed_point(n, ptr, col, t0, t1, p, part, 2);
  memcpy(dist, res, sizeof(int) * n);
  free(t0); free(t1);
  return ORC_OK;
}

/* write_skirt (mpk2/lib.c:617-654) over comp_skirt distances: header
 * "skirt N nodes, P parts", then per part "partition p" and lines
 * "j level-dist" for dist < level (lev == NULL, PA1) or for
 * lev[j] < level - dist (multi-phase). */
int orc_write_skirt(const char *path, int n, const int *ptr, const int *col,
                    const int *part, int npart, const int *lev, int level) {
  FILE *f = fopen(path, "w");
  if (!f) return ORC_EIO;
  int *dist = malloc(sizeof(int) * n);
  if (!dist) { fclose(f); return ORC_EIO; }
  fprintf(f, "skirt %d nodes, %d parts\n", n, npart);
  for (int p = 0; p < npart; p++) {
    fprintf(f, "partition %d\n", p);
    orc_skirt_dist(n, ptr, col, part, p, dist);
    for (int j = 0; j < n; j++) {
      int keep = lev ? (lev[j] < level - dist[j]) : (dist[j] < level);
      if (keep) fprintf(f, "%d %d\n", j, level - dist[j]);
    }
  }
  free(dist);
  fclose(f);
  return ORC_OK;
}

/* read_skirt (mpk2/lib.c:656-707) into a dense npart*n array: entries
 * not listed are -1, listed entries hold level - m. */
int orc_read_skirt(const char *path, int n, int npart, int level, int *sl) {
  FILE *f = fopen(path, "r");
  if (!f) return ORC_EIO;
  char line[256];
  int a = -1, b = -1;
  if (!fgets(line, sizeof line, f) || sscanf(line, "skirt %d nodes, %d parts", &a, &b) != 2 ||
      a != n || b != npart) { fclose(f); return ORC_EFORMAT; }
  for (long i = 0; i < (long)npart * n; i++) sl[i] = -1;
  int p = -1;
  while (fgets(line, sizeof line, f)) {
    if (line[0] == 'p') {
      int q;
      if (sscanf(line, "partition %d", &q) != 1 || q != p + 1) { fclose(f); return ORC_EFORMAT; }
      p = q;
      continue;
    }
    int k, m;
    if (sscanf(line, "%d %d", &k, &m) != 2) continue;
    if (p < 0 || k < 0 || k >= n || m < 0 || m > level) { fclose(f); return ORC_ERANGE; }
    sl[(long)p * n + k] = level - m;
  }
  fclose(f);
  return (p == npart - 1) ? ORC_OK : ORC_EFORMAT;
}

/* ------------------------------------------------------------------ */
/* Task lists: restates prep_mpk (mpk2/mpkprep.c:7-258) without its      */
/* printing.  parts: nphase (or 1 when nphase==0) arrays of n part ids;  */
/* levels: nphase arrays of n levels; sl: dense npart*n skirt (-1 = not  */
/* in the skirt).  Output: task (phase, part) = tasks[off[t]..off[t+1]), */
/* t = phase*npart + part, each entry l*n+i.  Returns the total number of */
/* entries, or ORC_ESTRUCT when the reference's dependency checks fail,  */
/* or ORC_ERANGE when cap is too small.                                   */
/* ------------------------------------------------------------------ */
long orc_prep_tasks(int n, const int *ptr, const int *col, int npart, int nlevel,
                    int nphase, const int *parts, const int *levels, const int *sl,
                    long *off, long *tasks, long cap) {
  long erc = 0;
  /* level monotonicity (mpkprep.c:21-49) */
  for (int ph = 0; ph < nphase; ph++) {
    const int *l1 = levels + (long)ph * n;
    for (int i = 0; i < n; i++) {
      if (ph == 0 && l1[i] < 0) erc++;
      if (ph > 0 && levels[(long)(ph - 1) * n + i] > l1[i]) erc++;
    }
  }
  /* skirt consistency (mpkprep.c:52-84) */
  for (int p = 0; p < npart; p++)
    for (int i = 0; i < n; i++) {
      int s = sl[(long)p * n + i];
      if (s < 0) continue;
      if (nphase == 0 && nlevel - s < 0) erc++;
      if (nphase > 0 && levels[(long)(nphase - 1) * n + i] > nlevel - s) erc++;
    }
  if (erc) return ORC_ESTRUCT;

  long nvv = (long)n * (nlevel + 1);
  double *vv = malloc(sizeof(double) * nvv);
  int *l0 = calloc(n, sizeof(int));
  long *tsize = calloc(npart, sizeof(long));
  if (!vv || !l0 || !tsize) { free(vv); free(l0); free(tsize); return ORC_EIO; }
  for (long i = 0; i < nvv; i++) vv[i] = -1.0;
  const int *pl = parts;
  for (int i = 0; i < n; i++) vv[i] = pl[i] * 100.0;

  long tcount = 0;
  const int *prevl = l0;
  int prevlmin = 0;
  for (int ph = 0; ph < nphase; ph++) {
    pl = parts + (long)ph * n;
    const int *ll = levels + (long)ph * n;
    int lmin = ll[0], lmax = ll[0];
    for (int i = 1; i < n; i++) { if (lmin > ll[i]) lmin = ll[i]; if (lmax < ll[i]) lmax = ll[i]; }
    if (lmax > nlevel) lmax = nlevel;
    for (int p = 0; p < npart; p++) tsize[p] = 0;
    /* dependency check with part*100+phase tags (mpkprep.c:134-162) */
    for (int l = prevlmin + 1; l <= lmax; l++)
      for (int i = 0; i < n; i++)
        if (prevl[i] < l && l <= ll[i]) {
          if (vv[(long)l * n + i] >= 0) erc++;
          for (int j = ptr[i]; j < ptr[i + 1]; j++) {
            int k = col[j];
            double t = vv[(long)(l - 1) * n + k];
            if (t < 0.0 || (pl[i] != pl[k] && ((int)t) % 100 == ph)) erc++;
          }
          vv[(long)l * n + i] = pl[i] * 100.0 + ph;
          tsize[pl[i]]++;
        }
    long base = tcount;
    for (int p = 0; p < npart; p++) {
      off[(long)ph * npart + p] = base;
      base += tsize[p];
      tsize[p] = 0;
    }
    if (base > cap) { free(vv); free(l0); free(tsize); return ORC_ERANGE; }
    for (int l = prevlmin + 1; l <= lmax; l++)
      for (int i = 0; i < n; i++)
        if (prevl[i] < l && l <= ll[i]) {
          int p = pl[i];
          tasks[off[(long)ph * npart + p] + tsize[p]++] = (long)l * n + i;
        }
    tcount = base;
    prevl = ll;
    prevlmin = lmin;
  }
  if (erc) { free(vv); free(l0); free(tsize); return ORC_ESTRUCT; }

  /* skirt tasks (mpkprep.c:185-233) */
  pl = parts;
  for (int p = 0; p < npart; p++) {
    long t = (long)nphase * npart + p;
    off[t] = tcount;
    long cnt = 0;
    const int *sp = sl + (long)p * n;
    for (int l = prevlmin + 1; l <= nlevel; l++)
      for (int i = 0; i < n; i++)
        if (prevl[i] < l && sp[i] >= 0 && l <= nlevel - sp[i]) {
          if (vv[(long)l * n + i] > 0.0) erc++;
          for (int j = ptr[i]; j < ptr[i + 1]; j++)
            if (vv[(long)(l - 1) * n + col[j]] < 0.0) erc++;
          vv[(long)l * n + i] = pl[i] * 100.0 + nphase;
          if (tcount + cnt >= cap) { free(vv); free(l0); free(tsize); return ORC_ERANGE; }
          tasks[tcount + cnt++] = (long)l * n + i;
        }
    for (int l = prevlmin + 1; l <= nlevel; l++)
      for (int i = 0; i < n; i++)
        if (prevl[i] < l && sp[i] >= 0 && l <= nlevel - sp[i]) vv[(long)l * n + i] = -0.1;
    tcount += cnt;
  }
  off[(long)(nphase + 1) * npart] = tcount;
  /* final level fully computed (mpkprep.c:238-242) */
  for (int i = 0; i < n; i++) if (vv[(long)nlevel * n + i] < -0.5) erc++;
  free(vv); free(l0); free(tsize);
  return erc ? ORC_ESTRUCT : tcount;
}

/* ------------------------------------------------------------------ */
/* Execution                                                             */
/* ------------------------------------------------------------------ */

/* do_task over every task list in (phase, part) order: restates
 * exec_mpk (mpk2/mpkexec.c:10-59, 1/deg weights when val == NULL) and
 * vexec_mpk (mpk2/mpkvexec.c:10-55, explicit values). */
void orc_exec_tasks(int n, const int *ptr, const int *col, const double *val,
                    long ntask_lists, const long *off, const long *tasks,
                    double *vv, int mode) {
  for (long t = 0; t < ntask_lists; t++)
    for (long q = off[t]; q < off[t + 1]; q++) {
      long tidx = tasks[q];
      long level = tidx / n;
      long i = tidx - level * n;
      const double *src = vv + (level - 1) * n;
      double s = 0.0;
      if (val) {
        for (int j = ptr[i]; j < ptr[i + 1]; j++) s = row_term(s, val[j], src[col[j]], mode);
      } else {
        double a = 1.0 / (ptr[i + 1] - ptr[i]);
        for (int j = ptr[i]; j < ptr[i + 1]; j++) s = row_term(s, a, src[col[j]], mode);
      }
      vv[level * n + i] = s;
    }
}

/* Transposed layout vv[i*(nlevel+1)+l] (mpk2/mpktexec.c:8-37). */
void orc_exec_tasks_t(int n, int nlevel, const int *ptr, const int *col,
                      long ntask_lists, const long *off, const long *tasks,
                      double *vv, int mode) {
  int nl1 = nlevel + 1;
  for (long t = 0; t < ntask_lists; t++)
    for (long q = off[t]; q < off[t + 1]; q++) {
      long tidx = tasks[q];
      long level = tidx / n;
      long i = tidx - level * n;
      double a = 1.0 / (ptr[i + 1] - ptr[i]);
      double s = 0.0;
      for (int j = ptr[i]; j < ptr[i + 1]; j++)
        s = row_term(s, a, vv[(long)col[j] * nl1 + level - 1], mode);
      vv[i * nl1 + level] = s;
    }
}

/* k chained SpMVs: spmv_exec_seq (mpk2/spmvexec.c:8-28) when val == NULL,
 * the verify_val gold chain (mpk2/verify_val.c:44-75) otherwise. */
void orc_spmv_chain(int n, const int *ptr, const int *col, const double *val,
                    int nlevel, double *vv, int mode) {
  for (int l = 1; l <= nlevel; l++) {
    const double *src = vv + (long)(l - 1) * n;
    double *dst = vv + (long)l * n;
    for (int i = 0; i < n; i++) {
      double s = 0.0;
      if (val) {
        for (int j = ptr[i]; j < ptr[i + 1]; j++) s = row_term(s, val[j], src[col[j]], mode);
      } else {
        double a = 1.0 / (ptr[i + 1] - ptr[i]);
        for (int j = ptr[i]; j < ptr[i + 1]; j++) s = row_term(s, a, src[col[j]], mode);
      }
      dst[i] = s;
    }
  }
}

/* The same chain with OpenMP over rows, for timing the CPU baseline on
 * many host cores (spmv_exec_par, mpk2/spmvexec.c:30-50). */
void orc_spmv_chain_par(int n, const int *ptr, const int *col, const double *val,
                        int nlevel, double *vv, int mode, int nth) {
  for (int l = 1; l <= nlevel; l++) {
    const double *src = vv + (long)(l - 1) * n;
    double *dst = vv + (long)l * n;
#pragma omp parallel for num_threads(nth) schedule(static)
    for (int i = 0; i < n; i++) {
      double s = 0.0;
      if (val) {
        for (int j = ptr[i]; j < ptr[i + 1]; j++) s = row_term(s, val[j], src[col[j]], mode);
      } else {
        double a = 1.0 / (ptr[i + 1] - ptr[i]);
        for (int j = ptr[i]; j < ptr[i + 1]; j++) s = row_term(s, a, src[col[j]], mode);
      }
      dst[i] = s;
    }
  }
}

/* exec over task lists with OpenMP: phases in order, parts in parallel
 * with dynamic scheduling, as exec_mpk_xd (mpk2/mpkexec.c:79-95). */
void orc_exec_tasks_par(int n, const int *ptr, const int *col, const double *val,
                        int nphase, int npart, const long *off, const long *tasks,
                        double *vv, int mode, int nth) {
  for (int ph = 0; ph <= nphase; ph++) {
#pragma omp parallel for num_threads(nth) schedule(dynamic, 1)
    for (int p = 0; p < npart; p++) {
      long t = (long)ph * npart + p;
      orc_exec_tasks(n, ptr, col, val, 1, off + t, tasks, vv, mode);
    }
  }
}

/* ------------------------------------------------------------------ */
/* MPI-2 rank buffers (mpk2/buffers.h:18-100).                           */
/* ------------------------------------------------------------------ */
typedef struct {
  int n, npart, nlevel, nphase, rank, buf_count, buf_scount, mptr_count, mcol_count;
  int *recvcounts, *sendcounts, *rdispls, *sdispls;           /* npart*(nphase+1) */
  int *rcount, *mcount, *scount, *rbuf_offsets, *mbuf_offsets, *sbuf_offsets, *mptr_offsets,
      *mcol_offsets;                                          /* nphase+1 */
  long *idx_buf, *idx_sbuf, *mptr_buf, *mcol_buf;
  double *mval_buf;                                           /* NULL when absent */
} orc_bufs;

/* Reads rank<N>.bufs as written by write_buffers (mpk2/buffers.c:588-631):
 * nine ints, four int arrays of npart*(nphase+1), eight int arrays of
 * nphase+1, then idx_buf, idx_sbuf, mptr_buf, mcol_buf (longs) and an
 * optional mval_buf (doubles). */
orc_bufs *orc_bufs_read(const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  orc_bufs *b = calloc(1, sizeof *b);
  int hdr[9];
  if (fread(hdr, sizeof(int), 9, f) != 9) { fclose(f); free(b); return NULL; }
  b->n = hdr[0]; b->npart = hdr[1]; b->nlevel = hdr[2]; b->nphase = hdr[3]; b->rank = hdr[4];
  b->buf_count = hdr[5]; b->buf_scount = hdr[6]; b->mptr_count = hdr[7]; b->mcol_count = hdr[8];
  long np = (long)b->npart * (b->nphase + 1), ph = b->nphase + 1;
  int **a4[4] = {&b->recvcounts, &b->sendcounts, &b->rdispls, &b->sdispls};
  for (int i = 0; i < 4; i++) {
    *a4[i] = malloc(sizeof(int) * np);
    if (fread(*a4[i], sizeof(int), np, f) != (size_t)np) goto bad;
  }
  int **a8[8] = {&b->rcount, &b->mcount, &b->scount, &b->rbuf_offsets, &b->mbuf_offsets, &b->sbuf_offsets,
                 &b->mptr_offsets, &b->mcol_offsets};
  for (int i = 0; i < 8; i++) {
    *a8[i] = malloc(sizeof(int) * ph);
    if (fread(*a8[i], sizeof(int), ph, f) != (size_t)ph) goto bad;
  }
  b->idx_buf = malloc(sizeof(long) * (b->buf_count + 1));
  b->idx_sbuf = malloc(sizeof(long) * (b->buf_scount + 1));
  b->mptr_buf = malloc(sizeof(long) * (b->mptr_count + 1));
  b->mcol_buf = malloc(sizeof(long) * (b->mcol_count + 1));
  if (fread(b->idx_buf, sizeof(long), b->buf_count, f) != (size_t)b->buf_count) goto bad;
  if (fread(b->idx_sbuf, sizeof(long), b->buf_scount, f) != (size_t)b->buf_scount) goto bad;
  if (fread(b->mptr_buf, sizeof(long), b->mptr_count, f) != (size_t)b->mptr_count) goto bad;
  if (fread(b->mcol_buf, sizeof(long), b->mcol_count, f) != (size_t)b->mcol_count) goto bad;
  b->mval_buf = malloc(sizeof(double) * (b->mcol_count + 1));
  if (fread(b->mval_buf, sizeof(double), b->mcol_count, f) < (size_t)b->mcol_count) {
    free(b->mval_buf);
    b->mval_buf = NULL;
  }
  fclose(f);
  return b;
bad:
  fclose(f);
  return NULL; /* leaks on malformed input; test infrastructure only */
}

/* One process's computation for `phase` (mpk2/mpi2_mpkexecbufs_val.c:13-30). */
static void orc_bufs_task(orc_bufs *b, double *vv_buf, int phase, int mode) {
  int mcount = b->mcount[phase];
  long *mptr = b->mptr_buf + b->mptr_offsets[phase];
  long *mcol = b->mcol_buf + b->mcol_offsets[phase];
  double *mval = b->mval_buf + b->mcol_offsets[phase];
  double *vv_mbuf = vv_buf + b->mbuf_offsets[phase];
  for (int mi = 0; mi < mcount; mi++) {
    double tmp = 0.0;
    for (long mj = mptr[mi]; mj < mptr[mi + 1]; mj++) tmp = row_term(tmp, mval[mj], vv_buf[mcol[mj]], mode);
    vv_mbuf[mi] = tmp;
  }
}

/* All ranks of the MPI-2 valued exec in one process: the input placed in
 * every rank's rbuf[0] (mpi2_mpkexecbufs_val.c:86-87, here vv_buf[i] =
 * x[idx_buf[i]] instead of 1.0), phase 0 computed, then per phase the
 * send-buffer gather and the Alltoallv (mpi2_mpkexecbufs_val.c:32-48)
 * emulated by copies, and finally collect_results (mpk2/mpi2_mpkexec.c:
 * 122-146): vv[idx_buf[i]] = vv_buf[i], rank 0 first.  Returns 0, or -1
 * when a buffer has no values. */
int orc_bufs_exec(int P, orc_bufs **b, const double *x, double *vv, int mode) {
  double **vb = malloc(sizeof(double *) * P), **sb = malloc(sizeof(double *) * P);
  for (int p = 0; p < P; p++) {
    if (!b[p]->mval_buf) { free(vb); free(sb); return -1; }
    vb[p] = calloc(b[p]->buf_count + 1, sizeof(double));
    sb[p] = calloc(b[p]->buf_scount + 1, sizeof(double));
    for (int i = 0; i < b[p]->rcount[0]; i++) vb[p][i] = x[b[p]->idx_buf[i]];
  }
  for (int p = 0; p < P; p++) orc_bufs_task(b[p], vb[p], 0, mode);
  for (int ph = 1; ph <= b[0]->nphase; ph++) {
    for (int p = 0; p < P; p++) {
      long *is = b[p]->idx_sbuf + b[p]->sbuf_offsets[ph];
      double *s = sb[p] + b[p]->sbuf_offsets[ph];
      for (int i = 0; i < b[p]->scount[ph]; i++) s[i] = vb[p][is[i]];
    }
    for (int dst = 0; dst < P; dst++)
      for (int src = 0; src < P; src++) {
        int off = P * ph;
        int cnt = b[dst]->recvcounts[off + src];
        double *r = vb[dst] + b[dst]->rbuf_offsets[ph] + b[dst]->rdispls[off + src];
        double *s = sb[src] + b[src]->sbuf_offsets[ph] + b[src]->sdispls[off + dst];
        memcpy(r, s, sizeof(double) * cnt);
      }
    for (int p = 0; p < P; p++) orc_bufs_task(b[p], vb[p], ph, mode);
  }
  for (int p = 0; p < P; p++) {
    for (int i = 0; i < b[p]->buf_count; i++) vv[b[p]->idx_buf[i]] = vb[p][i];
    free(vb[p]);
    free(sb[p]);
  }
  free(vb);
  free(sb);
  return 0;
}

/* ------------------------------------------------------------------ */
/* pdmpk buffers (pdmpk/buffers.h:30-166, written by Buffers::Dump,     */
/* pdmpk/buffers.cc:194-224; vectors as size_t count + raw elements,   */
/* pdmpk/utils.hpp DumpVec).                                            */
/* ------------------------------------------------------------------ */
typedef struct {
  size_t max_sbuf_size;
  int mbuf_idx;
  size_t n_mbuf_pb; size_t *mbuf_pb;
  size_t n_home; int *home;
  size_t n_orig; int *orig;
  size_t n_pd; short *pd;            /* bottom, mid, top per phase */
  size_t n_res; int *res_mbuf;
  size_t n_sc; int *sendcounts, *sdispls, *recvcounts, *rdispls;
  size_t n_sbi; int *sbuf_idcs; size_t n_sbpb; size_t *sbuf_pb;
  size_t n_init; int *init; size_t n_initpb; size_t *init_pb;   /* (src, tgt) pairs */
  size_t n_mptr; int *mptr; size_t n_mptrpb; size_t *mptr_pb;
  size_t n_mcol; int *mcol; size_t n_mval; double *mval;
  size_t n_rorig; int *rorig;        /* results.bin: original indices */
} orc_pd;

static void *rdvec(FILE *f, size_t elem, size_t *count) {
  if (fread(count, sizeof(size_t), 1, f) != 1) return NULL;
  void *p = malloc(elem * (*count + 1));
  if (*count && fread(p, elem, *count, f) != *count) { free(p); return NULL; }
  return p;
}

orc_pd *orc_pd_read(const char *buf_path, const char *res_path) {
  FILE *f = fopen(buf_path, "rb");
  if (!f) return NULL;
  orc_pd *b = calloc(1, sizeof *b);
  int ok = fread(&b->max_sbuf_size, sizeof(size_t), 1, f) == 1 && fread(&b->mbuf_idx, sizeof(int), 1, f) == 1;
  ok = ok && (b->mbuf_pb = rdvec(f, sizeof(size_t), &b->n_mbuf_pb));
  ok = ok && (b->home = rdvec(f, sizeof(int), &b->n_home));
  ok = ok && (b->orig = rdvec(f, sizeof(int), &b->n_orig));
  ok = ok && (b->pd = rdvec(f, 3 * sizeof(short), &b->n_pd));
  ok = ok && (b->res_mbuf = rdvec(f, sizeof(int), &b->n_res));
  size_t c1, c2, c3;
  ok = ok && (b->sendcounts = rdvec(f, sizeof(int), &b->n_sc));
  ok = ok && (b->sdispls = rdvec(f, sizeof(int), &c1)) && (b->recvcounts = rdvec(f, sizeof(int), &c2)) &&
       (b->rdispls = rdvec(f, sizeof(int), &c3));
  ok = ok && c1 == b->n_sc && c2 == b->n_sc && c3 == b->n_sc;
  ok = ok && (b->sbuf_idcs = rdvec(f, sizeof(int), &b->n_sbi)) && (b->sbuf_pb = rdvec(f, sizeof(size_t), &b->n_sbpb));
  ok = ok && (b->init = rdvec(f, 2 * sizeof(int), &b->n_init)) && (b->init_pb = rdvec(f, sizeof(size_t), &b->n_initpb));
  ok = ok && (b->mptr = rdvec(f, sizeof(int), &b->n_mptr)) && (b->mptr_pb = rdvec(f, sizeof(size_t), &b->n_mptrpb));
  ok = ok && (b->mcol = rdvec(f, sizeof(int), &b->n_mcol)) && (b->mval = rdvec(f, sizeof(double), &b->n_mval));
  fclose(f);
  if (!ok) return NULL;
  f = fopen(res_path, "rb");
  if (!f) return NULL;
  b->rorig = rdvec(f, sizeof(int), &b->n_rorig);
  fclose(f);
  return b->rorig ? b : NULL;
}

/* All ranks of pdmpk's exec in one process: LoadInput with x (the
 * reference loads 1.0, pdmpk/buffers.cc:353-358, here x[original_idcs]),
 * then AsyncExec (pdmpk/buffers.cc:286-323) with every batch's
 * MPI_Ialltoallv emulated by copies before the batch's DoComp
 * (pdmpk/buffers.cc:242-263, partial sums seeded from init_idcs), then
 * SendHome (pdmpk/buffers.cc:346-351) and the results scatter
 * (Results::FillVal/FillResults, pdmpk/results.cc:16-29): out[i] = A^k x.
 * Returns 0, or -1 on inconsistent buffers. */
int orc_pd_exec(int P, orc_pd **b, const double *x, double *out, int mode) {
  double **mb = malloc(sizeof(double *) * P), **sb = malloc(sizeof(double *) * P);
  for (int p = 0; p < P; p++) {
    mb[p] = calloc(b[p]->mbuf_idx + 1, sizeof(double));
    sb[p] = calloc(b[p]->max_sbuf_size + 1, sizeof(double));
    for (size_t i = 0; i < b[p]->mbuf_pb[0] && i < b[p]->n_orig; i++) mb[p][i] = x[b[p]->orig[i]];
  }
  size_t batch = 0;
  for (size_t ph = 0; ph < b[0]->n_pd; ph++) {
    const short bottom = b[0]->pd[3 * ph], top = b[0]->pd[3 * ph + 2];
    for (int lvl = bottom; lvl < top; lvl++, batch++) {
      const size_t off = (size_t)P * batch;
      for (int p = 0; p < P; p++) {  /* fill send buffers */
        if (off + P > b[p]->n_sc || batch + 1 >= b[p]->n_mptrpb) return -1;
        const size_t sc = (size_t)b[p]->sendcounts[off + P - 1] + b[p]->sdispls[off + P - 1];
        const int *si = b[p]->sbuf_idcs + b[p]->sbuf_pb[batch];
        for (size_t i = 0; i < sc; i++) sb[p][i] = mb[p][si[i]];
      }
      for (int dst = 0; dst < P; dst++) {  /* Alltoallv into the batch's rbuf */
        const size_t msz = b[dst]->mptr_pb[batch + 1] - b[dst]->mptr_pb[batch];
        double *rbuf = mb[dst] + b[dst]->mbuf_pb[batch] + msz;
        for (int src = 0; src < P; src++) {
          const int cnt = b[dst]->recvcounts[off + src];
          memcpy(rbuf + b[dst]->rdispls[off + src], sb[src] + b[src]->sdispls[off + dst], sizeof(double) * cnt);
        }
      }
      for (int p = 0; p < P; p++) {  /* DoComp */
        orc_pd *q = b[p];
        const size_t mcount = q->mptr_pb[batch + 1] - q->mptr_pb[batch];
        double *cur = mb[p] + q->mbuf_pb[batch];
        const int *mp = q->mptr + q->mptr_pb[batch];
        size_t ii = q->init_pb[batch];
        for (size_t mi = 0; mi < mcount; mi++) {
          double tmp = 0.0;
          if (ii < q->init_pb[batch + 1] && q->mbuf_pb[batch] + mi == (size_t)q->init[2 * ii + 1]) {
            tmp = mb[p][q->init[2 * ii]];
            ii++;
          }
          for (int mj = mp[mi]; mj < mp[mi + 1]; mj++) tmp = row_term(tmp, q->mval[mj], mb[p][q->mcol[mj]], mode);
          cur[mi] = tmp;
        }
      }
    }
  }
  for (int p = 0; p < P; p++) {
    for (size_t i = 0; i < b[p]->n_home; i++) mb[p][i] = mb[p][b[p]->home[i]];
    for (size_t i = 0; i < b[p]->n_res && i < b[p]->n_rorig; i++) out[b[p]->rorig[i]] = mb[p][b[p]->res_mbuf[i]];
    free(mb[p]);
    free(sb[p]);
  }
  free(mb);
  free(sb);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Batched block-vector MPK in FP32 (no reference counterpart: the      */
/* batching form of the task).  V_l = A V_(l-1) for nrhs right-hand     */
/* sides stored row-major (row i: V[i*nrhs .. i*nrhs+nrhs)), each row a  */
/* single-precision fused multiply-add per entry in CSR order starting  */
/* from 0 -- the arithmetic the GPU kernel performs.  vb holds          */
/* (nlevel+1) levels of n*nrhs floats, level 0 = input.                 */
/* ------------------------------------------------------------------ */
void orc_spmm_f32(int n, const int *ptr, const int *col, const float *val, int nrhs, int nlevel, float *vb) {
  const size_t lv = (size_t)n * nrhs;
  for (int l = 1; l <= nlevel; l++) {
    const float *src = vb + (l - 1) * lv;
    float *dst = vb + l * lv;
    for (int i = 0; i < n; i++)
      for (int r = 0; r < nrhs; r++) {
        float s = 0.0f;
        for (int q = ptr[i]; q < ptr[i + 1]; q++) s = fmaf(val[q], src[(size_t)col[q] * nrhs + r], s);
        dst[(size_t)i * nrhs + r] = s;
      }
  }
}

/* ------------------------------------------------------------------ */
/* PA1 task lists at sizes where the reference's dense skirt is out of  */
/* reach (npart*n ints).  Same lists as comp_skirt (mpk2/lib.c:584-615)  */
/* -> write_skirt/read_skirt (lib.c:617-707, PA1 branch: dist < nlevel)  */
/* -> prep_mpk's skirt loop (mpk2/mpkprep.c:186-233, prevl = 0): part p  */
/* computes level l on {i : dist_p(i) <= nlevel - l}, level-major,      */
/* vertex-ascending.  The distance is restated as a breadth-first       */
/* search bounded at nlevel - 1: minplus_x lowers row i to 1 + the      */
/* smallest distance among its columns, so distances spread from a     */
/* vertex j to every row i holding column j (the transpose's edges).    */
/* Returns the number of entries (off: npart + 1), ORC_ERANGE when cap  */
/* is too small (pass cap = 0 and tasks = NULL to count).               */
/* ------------------------------------------------------------------ */
static int cmp_int(const void *a, const void *b) {
  const int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

long orc_pa1_tasks(int n, const int *ptr, const int *col, const int *part, int npart,
                   int nlevel, long *off, long *tasks, long cap) {
  /* transpose: rows holding column j */
  long nnz = ptr[n];
  int *tptr = calloc((size_t)n + 1, sizeof(int)), *trow = malloc(sizeof(int) * (nnz ? nnz : 1));
  int *fill = malloc(sizeof(int) * (size_t)n), *dist = malloc(sizeof(int) * (size_t)n);
  int *ball = malloc(sizeof(int) * (size_t)n);
  long *pstart = calloc((size_t)npart + 1, sizeof(long));
  int *pverts = malloc(sizeof(int) * (size_t)n);
  if (!tptr || !trow || !fill || !dist || !ball || !pstart || !pverts) {
    free(tptr); free(trow); free(fill); free(dist); free(ball); free(pstart); free(pverts);
    return ORC_EIO;
  }
  for (long j = 0; j < nnz; j++) tptr[col[j] + 1]++;
  for (int i = 0; i < n; i++) tptr[i + 1] += tptr[i];
  memcpy(fill, tptr, sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++)
    for (int j = ptr[i]; j < ptr[i + 1]; j++) trow[fill[col[j]]++] = i;
  /* vertices of each part, ascending */
  for (int i = 0; i < n; i++) pstart[part[i] + 1]++;
  for (int p = 0; p < npart; p++) pstart[p + 1] += pstart[p];
  {
    long *pf = malloc(sizeof(long) * (size_t)(npart + 1));
    memcpy(pf, pstart, sizeof(long) * (size_t)(npart + 1));
    for (int i = 0; i < n; i++) pverts[pf[part[i]]++] = i;
    free(pf);
  }
  for (int i = 0; i < n; i++) dist[i] = -1;
  long total = 0;
  off[0] = 0;
  for (int p = 0; p < npart; p++) {
    int nb = 0;
    for (long q = pstart[p]; q < pstart[p + 1]; q++) {
      ball[nb++] = pverts[q];
      dist[pverts[q]] = 0;
    }
    int lo = 0;
    for (int d = 1; d <= nlevel - 1; d++) {
      const int hi = nb;
      for (int q = lo; q < hi; q++) {
        const int j = ball[q];
        for (int t = tptr[j]; t < tptr[j + 1]; t++) {
          const int i = trow[t];
          if (dist[i] < 0) {
            dist[i] = d;
            ball[nb++] = i;
          }
        }
      }
      lo = hi;
    }
    /* the ball in vertex order; keep each vertex's distance */
    int *sorted = malloc(sizeof(int) * (size_t)(nb ? nb : 1));
    memcpy(sorted, ball, sizeof(int) * (size_t)nb);
    qsort(sorted, (size_t)nb, sizeof(int), cmp_int);
    for (int l = 1; l <= nlevel; l++)
      for (int q = 0; q < nb; q++) {
        const int i = sorted[q];
        if (dist[i] <= nlevel - l) {
          if (tasks) {
            if (total >= cap) {
              free(sorted);
              free(tptr); free(trow); free(fill); free(dist); free(ball); free(pstart); free(pverts);
              return ORC_ERANGE;
            }
            tasks[total] = (long)l * n + i;
          }
          total++;
        }
      }
    off[p + 1] = total;
    for (int q = 0; q < nb; q++) dist[ball[q]] = -1;
    free(sorted);
  }
  free(tptr); free(trow); free(fill); free(dist); free(ball); free(pstart); free(pverts);
  return total;
}

/* ------------------------------------------------------------------ */
/* Workload generators for the CPU arms of the benchmark, so that those */
/* arms need nothing but the oracle and the reference.  Definitions of  */
/* this project's own workload (no reference counterpart): the 3-D      */
/* 7-point Laplacian on nx*ny*nz (x fastest; columns ascending: z-, y-, */
/* x-, diagonal, x+, y+, z+), and uniform[-1,1] doubles from a          */
/* splitmix64 stream (2u - 1 with u = (z >> 11) * 2^-53).               */
/* ------------------------------------------------------------------ */
long orc_gen_laplacian(int nx, int ny, int nz, double diag, double offd, int *ptr, int *col, double *val) {
  const long sy = nx, sz = (long)nx * ny, n = sz * nz;
  long e = 0;
  ptr[0] = 0;
  for (long i = 0; i < n; i++) {
    const long x = i % nx, y = (i / nx) % ny, z = i / sz;
    const long c[7] = {i - sz, i - sy, i - 1, i, i + 1, i + sy, i + sz};
    const int ok[7] = {z > 0, y > 0, x > 0, 1, x < nx - 1, y < ny - 1, z < nz - 1};
    for (int t = 0; t < 7; t++)
      if (ok[t]) {
        col[e] = (int)c[t];
        val[e] = (t == 3) ? diag : offd;
        e++;
      }
    ptr[i + 1] = (int)e;
  }
  return e;
}

void orc_uniform(unsigned long long seed, long n, double *out) {
  unsigned long long s = seed;
  for (long i = 0; i < n; i++) {
    s += 0x9E3779B97F4A7C15ULL;
    unsigned long long z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    out[i] = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
  }
}
