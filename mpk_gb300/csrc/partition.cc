// Partition providers.  The reference partitions with METIS 5.1
// (mpk2/driver.c:63-66 runs `gpmetis -ufactor=100`; pdmpk/pdmpk_buffers.cc:
// 183-202 calls METIS_PartGraphKway).  When the CUDA toolkit bundles METIS
// (libmetis_static.a: 64-bit idx_t, the METIS 5.1 option layout) the
// library links it and calls it through its public API (metis_kway below).
// Besides METIS: partition files in gpmetis's output format (the
// reference's partition contract, mpk2/lib.c:273-284), and two project
// partitioners, recursive coordinate bisection for grids with known
// coordinates and breadth-first recursive bisection for any graph.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <queue>
#include <string>
#include <vector>

#include "host.h"

#ifdef MPKG_HAVE_METIS
extern "C" {
int METIS_SetDefaultOptions(int64_t *options);
int METIS_PartGraphKway(int64_t *nvtxs, int64_t *ncon, int64_t *xadj, int64_t *adjncy, int64_t *vwgt,
                        int64_t *vsize, int64_t *adjwgt, int64_t *nparts, void *tpwgts, void *ubvec,
                        int64_t *options, int64_t *edgecut, int64_t *part);
}
#endif

namespace mpkg {

bool have_metis() {
#ifdef MPKG_HAVE_METIS
  return true;
#else
  return false;
#endif
}

int metis_kway(int n, const int *ptr, const int *col, const int *vwgt, const int *adjwgt, int npart,
               const int *options, int *part, long *edgecut) {
  if (npart <= 0 || npart > n) return fail(kEInval, "npart must be in [1, n]");
  if (npart == 1) {
    std::fill(part, part + n, 0);
    if (edgecut) *edgecut = 0;
    return kOk;
  }
#ifdef MPKG_HAVE_METIS
  const long nnz = ptr[n];
  std::vector<int64_t> xadj(ptr, ptr + n + 1), adj(col, col + nnz), pp(n), vw, ew, opt;
  if (vwgt) vw.assign(vwgt, vwgt + n);
  if (adjwgt) ew.assign(adjwgt, adjwgt + nnz);
  if (options) opt.assign(options, options + kMetisNOptions);
  int64_t nv = n, ncon = 1, np = npart, cut = 0;
  const int rc = METIS_PartGraphKway(&nv, &ncon, xadj.data(), adj.data(), vwgt ? vw.data() : nullptr, nullptr,
                                     adjwgt ? ew.data() : nullptr, &np, nullptr, nullptr,
                                     options ? opt.data() : nullptr, &cut, pp.data());
  if (rc != 1) return fail(kEInval, "METIS_PartGraphKway failed (" + std::to_string(rc) + ")");
  for (int i = 0; i < n; i++) {
    if (pp[i] < 0 || pp[i] >= npart) return fail(kERange, "METIS returned a part out of range");
    part[i] = (int)pp[i];
  }
  if (edgecut) *edgecut = (long)cut;
  return kOk;
#else
  (void)ptr; (void)col; (void)vwgt; (void)adjwgt; (void)options; (void)edgecut;
  return fail(kEInval, "this build has no METIS (the CUDA toolkit's libmetis_static.a was not found)");
#endif
}

int partition_metis(const Csr &g, const int *vwgt, const int *adjwgt, int npart, int ufactor, std::vector<int> *part,
                    long *edgecut) {
  // gpmetis's input: the graph without self loops (the reference's g0 and
  // weighted gN files hold none), weights kept with their entries
  Csr h;
  h.n = g.n;
  h.ptr.assign(g.n + 1, 0);
  h.col.reserve(g.col.size());
  std::vector<int> ew;
  for (int i = 0; i < g.n; i++) {
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++)
      if (g.col[j] != i) {
        h.col.push_back(g.col[j]);
        if (adjwgt) ew.push_back(adjwgt[j]);
      }
    h.ptr[i + 1] = (int)h.col.size();
  }
  int opt[kMetisNOptions];
  std::fill(opt, opt + kMetisNOptions, -1);  // METIS_SetDefaultOptions
  opt[kMetisOptNumbering] = 0;
  if (ufactor > 0) opt[kMetisOptUfactor] = ufactor;
  part->assign(g.n, 0);
  return metis_kway(h.n, h.ptr.data(), h.col.data(), vwgt, adjwgt ? ew.data() : nullptr, npart, opt, part->data(),
                    edgecut);
}

int read_partition(const std::string &path, int n, std::vector<int> *part, int *npart) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) return fail(kEIo, "cannot open " + path);
  part->resize(n);
  int mx = 0;
  for (int i = 0; i < n; i++) {
    int p;
    if (std::fscanf(f, "%d", &p) != 1) {
      std::fclose(f);
      return fail(kEFormat, path + ": fewer part ids than vertices");
    }
    if (p < 0) {
      std::fclose(f);
      return fail(kERange, path + ": negative part id");
    }
    if (mx < p) mx = p;
    (*part)[i] = p;
  }
  std::fclose(f);
  *npart = mx + 1;  // as read_part: n_part = max + 1
  return kOk;
}

int write_partition(const std::string &path, const std::vector<int> &part) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return fail(kEIo, "cannot open " + path);
  for (int p : part) std::fprintf(f, "%d\n", p);
  std::fclose(f);
  return kOk;
}

namespace {
void rcb_rec(std::vector<int> &ids, long lo, long hi, const std::vector<int> &coords, int dim,
             int p0, int np, std::vector<int> *part) {
  if (np == 1) {
    for (long i = lo; i < hi; i++) (*part)[ids[i]] = p0;
    return;
  }
  // longest extent; ties go to the lowest dimension
  int best = 0;
  int bext = -1;
  for (int d = 0; d < dim; d++) {
    int mn = 0x7fffffff, mx = -0x7fffffff;
    for (long i = lo; i < hi; i++) {
      int c = coords[(long)ids[i] * dim + d];
      mn = std::min(mn, c);
      mx = std::max(mx, c);
    }
    if (mx - mn > bext) { bext = mx - mn; best = d; }
  }
  std::stable_sort(ids.begin() + lo, ids.begin() + hi, [&](int a, int b) {
    return coords[(long)a * dim + best] < coords[(long)b * dim + best];
  });
  int nl = np / 2;
  long cut = lo + (long)((double)(hi - lo) * nl / np + 0.5);
  rcb_rec(ids, lo, cut, coords, dim, p0, nl, part);
  rcb_rec(ids, cut, hi, coords, dim, p0 + nl, np - nl, part);
}
}  // namespace

int partition_rcb(int n, const std::vector<int> &coords, int dim, int npart,
                  std::vector<int> *part) {
  if (npart <= 0 || npart > n) return fail(kEInval, "npart must be in [1, n]");
  if ((long)coords.size() < (long)n * dim) return fail(kEInval, "coords too short");
  std::vector<int> ids(n);
  std::iota(ids.begin(), ids.end(), 0);
  part->assign(n, 0);
  rcb_rec(ids, 0, n, coords, dim, 0, npart, part);
  return kOk;
}

namespace {
// BFS order of the vertices in `set` (marked by `in`==tag) starting at s.
void bfs_order(const Csr &g, const std::vector<int> &in, int tag, int s, std::vector<int> &order,
               std::vector<int> &seen, int stamp) {
  order.clear();
  order.push_back(s);
  seen[s] = stamp;
  for (size_t h = 0; h < order.size(); h++) {
    int v = order[h];
    for (int j = g.ptr[v]; j < g.ptr[v + 1]; j++) {
      int u = g.col[j];
      if (in[u] == tag && seen[u] != stamp) {
        seen[u] = stamp;
        order.push_back(u);
      }
    }
  }
}
}  // namespace

int partition_bfs(const Csr &g, int npart, std::vector<int> *part) {
  const int n = g.n;
  if (npart <= 0 || npart > n) return fail(kEInval, "npart must be in [1, n]");
  part->assign(n, 0);
  std::vector<int> in(n, 0), seen(n, -1);
  int stamp = 0;
  // work stack of (part range start, count, tag)
  struct Job { int p0, np, tag; };
  std::vector<Job> stack{{0, npart, 0}};
  std::vector<std::vector<int>> members(1);
  members[0].resize(n);
  std::iota(members[0].begin(), members[0].end(), 0);
  int next_tag = 1;
  std::vector<int> order, comp;
  while (!stack.empty()) {
    Job jb = stack.back();
    stack.pop_back();
    std::vector<int> mem;
    mem.swap(members[jb.tag]);
    if (jb.np == 1) {
      for (int v : mem) (*part)[v] = jb.p0;
      continue;
    }
    // order all members: BFS per connected component, each from a
    // pseudo-peripheral vertex (two sweeps)
    std::vector<int> full;
    full.reserve(mem.size());
    stamp++;
    int comp_stamp = stamp;
    for (int v : mem) {
      if (seen[v] == comp_stamp) continue;
      bfs_order(g, in, jb.tag, v, comp, seen, comp_stamp);
      int far = comp.back();
      stamp++;
      bfs_order(g, in, jb.tag, far, order, seen, stamp);
      for (int u : order) seen[u] = comp_stamp;
      full.insert(full.end(), order.begin(), order.end());
    }
    int nl = jb.np / 2;
    size_t cut = (size_t)((double)full.size() * nl / jb.np + 0.5);
    int ta = next_tag++, tb = next_tag++;
    members.resize(next_tag);
    members[ta].assign(full.begin(), full.begin() + cut);
    members[tb].assign(full.begin() + cut, full.end());
    for (int v : members[ta]) in[v] = ta;
    for (int v : members[tb]) in[v] = tb;
    stack.push_back({jb.p0 + nl, jb.np - nl, tb});
    stack.push_back({jb.p0, nl, ta});
  }
  return kOk;
}

}  // namespace mpkg
