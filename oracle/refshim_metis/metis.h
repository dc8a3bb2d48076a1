/* METIS 5.1 interface for compiling the reference pdmpk prep against the
 * real METIS (TEST INFRASTRUCTURE ONLY).  The reference code uses a 32-bit
 * idx_t (METIS's default build, and the width of its buf.bin vectors); the
 * METIS library bundled with the CUDA toolkit is built with a 64-bit
 * idx_t.  This header keeps idx_t 32-bit for the reference code and widens
 * every array on its way into the library's METIS_PartGraphKway (declared
 * under another C++ name through an asm label), and narrows the parts on
 * the way back.  Option values and order are METIS 5.1's. */
#ifndef ORACLE_REFSHIM_METIS_REAL_H
#define ORACLE_REFSHIM_METIS_REAL_H
#include <stdint.h>
#include <stdlib.h>
typedef int32_t idx_t;
typedef float real_t;
#define METIS_NOPTIONS 40
enum { METIS_OK = 1 };
enum {
  METIS_OPTION_PTYPE, METIS_OPTION_OBJTYPE, METIS_OPTION_CTYPE, METIS_OPTION_IPTYPE, METIS_OPTION_RTYPE,
  METIS_OPTION_DBGLVL, METIS_OPTION_NITER, METIS_OPTION_NCUTS, METIS_OPTION_SEED, METIS_OPTION_NO2HOP,
  METIS_OPTION_MINCONN, METIS_OPTION_CONTIG, METIS_OPTION_COMPRESS, METIS_OPTION_CCORDER, METIS_OPTION_PFACTOR,
  METIS_OPTION_NSEPS, METIS_OPTION_UFACTOR, METIS_OPTION_NUMBERING
};
enum { METIS_PTYPE_RB, METIS_PTYPE_KWAY };
enum { METIS_OBJTYPE_CUT, METIS_OBJTYPE_VOL, METIS_OBJTYPE_NODE };
enum { METIS_CTYPE_RM, METIS_CTYPE_SHEM };
enum { METIS_IPTYPE_GROW, METIS_IPTYPE_RANDOM, METIS_IPTYPE_EDGE, METIS_IPTYPE_NODE, METIS_IPTYPE_METISRB };
enum { METIS_RTYPE_FM, METIS_RTYPE_GREEDY, METIS_RTYPE_SEP2SIDED, METIS_RTYPE_SEP1SIDED };

extern "C" int refshim_metis_set_default(int64_t *options) __asm__("METIS_SetDefaultOptions");
extern "C" int refshim_metis_kway(int64_t *nvtxs, int64_t *ncon, int64_t *xadj, int64_t *adjncy, int64_t *vwgt,
                                  int64_t *vsize, int64_t *adjwgt, int64_t *nparts, void *tpwgts, void *ubvec,
                                  int64_t *options, int64_t *edgecut, int64_t *part) __asm__("METIS_PartGraphKway");

static inline int64_t *refshim_widen(const idx_t *a, long count) {
  if (!a) return NULL;
  int64_t *w = (int64_t *)malloc(sizeof(int64_t) * (count > 0 ? count : 1));
  for (long i = 0; i < count; i++) w[i] = a[i];
  return w;
}

static inline int METIS_SetDefaultOptions(idx_t *o) {
  int64_t w[METIS_NOPTIONS];
  const int rc = refshim_metis_set_default(w);
  for (int i = 0; i < METIS_NOPTIONS; i++) o[i] = (idx_t)w[i];
  return rc;
}

static inline int METIS_PartGraphKway(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy, idx_t *vwgt,
                                      idx_t *vsize, idx_t *adjwgt, idx_t *nparts, real_t *tpwgts, real_t *ubvec,
                                      idx_t *options, idx_t *edgecut, idx_t *part) {
  const long n = *nvtxs, nnz = xadj[n];
  int64_t nv = n, nc = *ncon, np = *nparts, cut = 0;
  int64_t *wx = refshim_widen(xadj, n + 1), *wa = refshim_widen(adjncy, nnz);
  int64_t *wv = refshim_widen(vwgt, n * nc), *ws = refshim_widen(vsize, n), *we = refshim_widen(adjwgt, nnz);
  int64_t *wo = refshim_widen(options, METIS_NOPTIONS);
  int64_t *wp = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
  const int rc = refshim_metis_kway(&nv, &nc, wx, wa, wv, ws, we, &np, (void *)tpwgts, (void *)ubvec, wo, &cut, wp);
  for (long i = 0; i < n; i++) part[i] = (idx_t)wp[i];
  *edgecut = (idx_t)cut;
  free(wx); free(wa); free(wv); free(ws); free(we); free(wo); free(wp);
  return rc;
}
#endif
