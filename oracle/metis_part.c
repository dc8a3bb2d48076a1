/*
 * gpmetis-style k-way partitions for the CPU arms of the benchmark and for
 * the tests (TEST INFRASTRUCTURE ONLY; the product links METIS itself).
 *
 * The reference partitions with METIS 5.1 (mpk2/driver.c:63-66 runs
 * `gpmetis -ufactor=100 g P`; pdmpk/pdmpk_buffers.cc:183-202 calls
 * METIS_PartGraphKway).  The METIS library bundled with the CUDA toolkit
 * (libmetis_static.a: 64-bit idx_t, the METIS 5.1 option layout) is linked
 * here and called through its public API only.  The graph handed to METIS
 * is the matrix pattern without its diagonal (the reference's `g0` graph
 * files hold no self loops), in CSR order.
 */
#include <stdint.h>
#include <stdlib.h>

typedef int64_t idx_t;
int METIS_SetDefaultOptions(idx_t *options);
int METIS_PartGraphKway(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *vsize,
                        idx_t *adjwgt, idx_t *nparts, void *tpwgts, void *ubvec, idx_t *options, idx_t *edgecut,
                        idx_t *part);
enum { kNOptions = 40, kOptUfactor = 16, kOptNumbering = 17, kMetisOk = 1 };

/* Returns 0 and part[n] in [0, npart), or -1.  ufactor <= 0 keeps METIS's
 * default imbalance.  vwgt (n) and adjwgt (one per stored entry) may be
 * NULL; the weights of dropped diagonal entries go with them. */
int orc_metis_kway(int n, const int *ptr, const int *col, const int *vwgt, const int *adjwgt, int npart,
                   int ufactor, int *part, long *edgecut) {
  if (npart == 1) {
    for (int i = 0; i < n; i++) part[i] = 0;
    if (edgecut) *edgecut = 0;
    return 0;
  }
  idx_t *xadj = malloc(sizeof(idx_t) * ((size_t)n + 1));
  idx_t *adj = malloc(sizeof(idx_t) * ((size_t)ptr[n] + 1));
  idx_t *ew = malloc(sizeof(idx_t) * ((size_t)ptr[n] + 1));
  idx_t *vw = malloc(sizeof(idx_t) * ((size_t)n + 1));
  idx_t *pp = malloc(sizeof(idx_t) * (size_t)n);
  if (!xadj || !adj || !ew || !vw || !pp) { free(xadj); free(adj); free(ew); free(vw); free(pp); return -1; }
  idx_t e = 0;
  for (int i = 0; i < n; i++) {
    xadj[i] = e;
    if (vwgt) vw[i] = vwgt[i];
    for (int j = ptr[i]; j < ptr[i + 1]; j++)
      if (col[j] != i) {
        if (adjwgt) ew[e] = adjwgt[j];
        adj[e++] = col[j];
      }
  }
  xadj[n] = e;
  idx_t opt[kNOptions];
  METIS_SetDefaultOptions(opt);
  opt[kOptNumbering] = 0;
  if (ufactor > 0) opt[kOptUfactor] = ufactor;
  idx_t nv = n, ncon = 1, np = npart, cut = 0;
  int rc = METIS_PartGraphKway(&nv, &ncon, xadj, adj, vwgt ? vw : NULL, NULL, adjwgt ? ew : NULL, &np, NULL, NULL,
                               opt, &cut, pp);
  for (int i = 0; i < n; i++) part[i] = (int)pp[i];
  if (edgecut) *edgecut = (long)cut;
  free(xadj); free(adj); free(ew); free(vw); free(pp);
  return rc == kMetisOk ? 0 : -1;
}
