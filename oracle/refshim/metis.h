/* Stand-in for METIS 5.1 (not available to this oracle), enough to compile
 * the reference pdmpk code as a test oracle.  METIS_PartGraphKway is
 * replaced by a deterministic rule of this file's own: call c of a process
 * assigns vertex i to part ((i + shift_c) mod n) * nparts / n, shift_c =
 * c * n / (2 * nparts) (contiguous blocks, shifted by half a block per
 * call, so that successive phases see different boundaries).  Weights and
 * options are ignored.  The product's pdmpk prep uses the same rule when
 * asked for it, so both sides see identical partitions. */
#ifndef ORACLE_REFSHIM_METIS_H
#define ORACLE_REFSHIM_METIS_H
#include <stdint.h>
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
static inline int METIS_SetDefaultOptions(idx_t *o) {
  for (int i = 0; i < METIS_NOPTIONS; i++) o[i] = -1;
  return METIS_OK;
}
static inline int refshim_partition_calls(void) {
  static int calls = 0;
  return calls++;
}
static inline int METIS_PartGraphKway(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy, idx_t *vwgt,
                                      idx_t *vsize, idx_t *adjwgt, idx_t *nparts, real_t *tpwgts, real_t *ubvec,
                                      idx_t *options, idx_t *edgecut, idx_t *part) {
  (void)ncon; (void)xadj; (void)adjncy; (void)vwgt; (void)vsize; (void)adjwgt; (void)tpwgts; (void)ubvec;
  (void)options;
  const long n = *nvtxs, np = *nparts;
  const long shift = (long)refshim_partition_calls() * n / (2 * np);
  for (long i = 0; i < n; i++) part[i] = (idx_t)((((i + shift) % n) * np) / n);
  *edgecut = 0;
  return METIS_OK;
}
#endif
