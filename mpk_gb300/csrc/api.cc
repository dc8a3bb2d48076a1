// C ABI: host prep entry points (mpk_gb300.h) and the mpk2-compatible names
// (mpk2_compat.h).
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/mpk2_compat.h"
#include "../../include/mpk_gb300.h"
#include "host.h"

using namespace mpkg;

namespace {

Csr view_csr(int n, const int *ptr, const int *col) {
  Csr g;
  g.n = n;
  g.ptr.assign(ptr, ptr + n + 1);
  g.col.assign(col, col + ptr[n]);
  return g;
}

int check_csr_host(int n, const int *ptr, const int *col) {
  if (n <= 0 || !ptr || !col) return fail(kEInval, "empty matrix or null arrays");
  if (ptr[0] != 0) return fail(kEInval, "ptr[0] must be 0");
  for (int i = 0; i < n; i++)
    if (ptr[i + 1] < ptr[i]) return fail(kEInval, "ptr must be non-decreasing");
  for (long j = 0; j < ptr[n]; j++)
    if (col[j] < 0 || col[j] >= n) return fail(kERange, "column index out of range");
  return kOk;
}

template <typename T>
T *dup(const std::vector<T> &v) {
  T *p = (T *)std::malloc(sizeof(T) * std::max<size_t>(v.size(), 1));
  if (p && !v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}

}  // namespace

extern "C" {

void mpkg_free(void *p) { std::free(p); }

int mpkg_read_metis(const char *path, int *n, long *nnz, int **ptr, int **col) {
  clear_error();
  if (!path || !n || !nnz || !ptr || !col) return fail(kEInval, "null argument");
  Csr g;
  int rc = read_metis(path, &g);
  if (rc) return rc;
  *n = g.n;
  *nnz = g.nnz();
  *ptr = dup(g.ptr);
  *col = dup(g.col);
  if (!*ptr || !*col) return fail(kENoMem, "allocation failed");
  return kOk;
}

int mpkg_read_values(const char *path, long nnz, double **val) {
  clear_error();
  if (!path || !val || nnz < 0) return fail(kEInval, "bad argument");
  std::vector<double> v;
  int rc = read_values(path, nnz, &v);
  if (rc) return rc;
  *val = dup(v);
  return *val ? kOk : fail(kENoMem, "allocation failed");
}

int mpkg_levels(int n, const int *ptr, const int *col, const int *part, int npart,
                const int *level_org, int *level) {
  clear_error();
  int rc = check_csr_host(n, ptr, col);
  if (rc) return rc;
  if (!part || !level || npart <= 0) return fail(kEInval, "null argument");
  Csr g = view_csr(n, ptr, col);
  std::vector<int> pv(part, part + n), lo, out;
  if (level_org) lo.assign(level_org, level_org + n);
  rc = comp_levels(g, pv, npart, level_org ? &lo : nullptr, &out);
  if (rc) return rc;
  std::copy(out.begin(), out.end(), level);
  return kOk;
}

int mpkg_level_weights(int n, const int *ptr, const int *col, const int *level, int *wv, int *we) {
  clear_error();
  int rc = check_csr_host(n, ptr, col);
  if (rc) return rc;
  if (!level || !wv || !we) return fail(kEInval, "null argument");
  Csr g = view_csr(n, ptr, col);
  std::vector<int> lv(level, level + n), a, b;
  level_weights(g, lv, &a, &b);
  std::copy(a.begin(), a.end(), wv);
  std::copy(b.begin(), b.end(), we);
  return kOk;
}

int mpkg_skirt_write(const char *path, int n, const int *ptr, const int *col, const int *part,
                     int npart, const int *lev, int nlevel) {
  clear_error();
  int rc = check_csr_host(n, ptr, col);
  if (rc) return rc;
  if (!path || !part || npart <= 0 || nlevel <= 0) return fail(kEInval, "bad argument");
  Csr g = view_csr(n, ptr, col);
  std::vector<int> pv(part, part + n), lv;
  if (lev) lv.assign(lev, lev + n);
  std::vector<PartSkirt> sk;
  if ((rc = comp_skirts(g, pv, npart, lev ? &lv : nullptr, nlevel, &sk))) return rc;
  return write_skirt_file(path, n, nlevel, sk);
}

int mpkg_tasks(int n, const int *ptr, const int *col, int npart, int nlevel, int nphase,
               const int *parts, const int *levels, int check, long *off, long **idx,
               long *count) {
  clear_error();
  int rc = check_csr_host(n, ptr, col);
  if (rc) return rc;
  if (!parts || (nphase > 0 && !levels) || !off || !idx || !count || npart <= 0 || nlevel <= 0 ||
      nphase < 0)
    return fail(kEInval, "bad argument");
  Csr g = view_csr(n, ptr, col);
  std::vector<std::vector<int>> pv, lv;
  for (int ph = 0; ph < std::max(nphase, 1); ph++) pv.emplace_back(parts + (long)ph * n, parts + (long)(ph + 1) * n);
  for (int ph = 0; ph < nphase; ph++) lv.emplace_back(levels + (long)ph * n, levels + (long)(ph + 1) * n);
  for (auto &p : pv)
    for (int q : p) if (q < 0 || q >= npart) return fail(kERange, "part id out of range");
  std::vector<PartSkirt> sk;
  if ((rc = comp_skirts(g, pv[0], npart, nphase ? &lv[nphase - 1] : nullptr, nlevel, &sk))) return rc;
  TaskLists tl;
  if ((rc = build_tasks(g, npart, nlevel, nphase, pv, lv, sk, check != 0, &tl))) return rc;
  std::copy(tl.off.begin(), tl.off.end(), off);
  *idx = dup(tl.idx);
  *count = (long)tl.idx.size();
  return *idx ? kOk : fail(kENoMem, "allocation failed");
}

int mpkg_partition_rcb(int n, const int *coords, int dim, int npart, int *part) {
  clear_error();
  if (n <= 0 || !coords || dim <= 0 || !part) return fail(kEInval, "bad argument");
  std::vector<int> c(coords, coords + (long)n * dim), out;
  int rc = partition_rcb(n, c, dim, npart, &out);
  if (rc) return rc;
  std::copy(out.begin(), out.end(), part);
  return kOk;
}

int mpkg_partition_bfs(int n, const int *ptr, const int *col, int npart, int *part) {
  clear_error();
  int rc = check_csr_host(n, ptr, col);
  if (rc) return rc;
  if (!part) return fail(kEInval, "null argument");
  Csr g = view_csr(n, ptr, col);
  std::vector<int> out;
  rc = partition_bfs(g, npart, &out);
  if (rc) return rc;
  std::copy(out.begin(), out.end(), part);
  return kOk;
}

int mpkg_gen_stencil(const char *type, int size, int *n, long *nnz, int **ptr, int **col,
                     double **val) {
  clear_error();
  if (!type || !n || !nnz || !ptr || !col || !val) return fail(kEInval, "null argument");
  Csr g;
  int rc = gen_reference_stencil(type, size, &g);
  if (rc) return rc;
  *n = g.n; *nnz = g.nnz();
  *ptr = dup(g.ptr); *col = dup(g.col); *val = dup(g.val);
  return kOk;
}

int mpkg_gen_laplacian(int nx, int ny, int nz, double diag, double offd, int *n, long *nnz,
                       int **ptr, int **col, double **val, int **coords) {
  clear_error();
  if (!n || !nnz || !ptr || !col || !val) return fail(kEInval, "null argument");
  Csr g;
  std::vector<int> c;
  int rc = gen_laplacian(nx, ny, nz, diag, offd, &g, coords ? &c : nullptr);
  if (rc) return rc;
  *n = g.n; *nnz = g.nnz();
  *ptr = dup(g.ptr); *col = dup(g.col); *val = dup(g.val);
  if (coords) *coords = dup(c);
  return kOk;
}

void mpkg_uniform(uint64_t seed, long n, double *out) {
  if (out && n > 0) uniform_vector(seed, n, out);
}

}  // extern "C"

// ==========================================================================
// mpk2-compatible names (include/mpk2_compat.h)
// ==========================================================================
namespace {

std::string slurp_file(FILE *f) {
  std::string s;
  char buf[1 << 16];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, k);
  return s;
}

Csr csr_of(const crs0_t *g) {
  Csr c;
  c.n = g->n;
  c.ptr.assign(g->ptr, g->ptr + g->n + 1);
  c.col.assign(g->col, g->col + g->ptr[g->n]);
  return c;
}

std::mutex g_plan_mu;
// cached device plans of mpk_t handles, keyed by (mpk_t, values, kind)
std::map<std::tuple<const void *, const void *, int>, mpkg_plan *> g_plans;

int legacy_arith() {
  const char *e = std::getenv("MPK_GB300_ARITH");
  if (e && std::strcmp(e, "separate") == 0) return MPKG_ARITH_SEPARATE;
  return MPKG_ARITH_FMA;
}

void drop_plans(const void *owner) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  for (auto it = g_plans.begin(); it != g_plans.end();) {
    if (std::get<0>(it->first) == owner) {
      mpkg_plan_destroy(it->second);
      it = g_plans.erase(it);
    } else {
      ++it;
    }
  }
}

// Task-list plan of an mpk_t (the lists need not be contiguous in idxsrc).
mpkg_plan *plan_for(mpk_t *mg, const double *val, int kind) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto key = std::make_tuple((const void *)mg, (const void *)val, kind);
  auto it = g_plans.find(key);
  if (it != g_plans.end()) return it->second;
  const long nl = (long)(mg->nphase + 1) * mg->npart;
  std::vector<long> off(nl + 1, 0), idx;
  for (long t = 0; t < nl; t++) {
    off[t] = (long)idx.size();
    const task_t &tk = mg->tlist[t];
    if (tk.n > 0 && tk.idx) idx.insert(idx.end(), tk.idx, tk.idx + tk.n);
  }
  off[nl] = (long)idx.size();
  mpkg_plan *p = nullptr;
  int rc = mpkg_plan_tasks(mg->n, mg->g0->ptr, mg->g0->col, val, mg->npart, mg->nlevel, mg->nphase,
                           off.data(), idx.data(), legacy_arith(), &p);
  if (rc) return nullptr;
  g_plans[key] = p;
  return p;
}

void legacy_exec(mpk_t *mg, double *vv, const double *val) {
  clear_error();
  if (!mg || !vv || !mg->tlist) { fail(kEInval, "exec_mpk: null mpk_t/vv or prep_mpk not run"); return; }
  mpkg_plan *p = plan_for(mg, val, 0);
  if (!p) return;
  mpkg_exec_host(p, vv);
}

}  // namespace

extern "C" {

const char *mpk2_last_error(void) { return last_error(); }

crs0_t *new_crs(int nv, int ne) {
  if (nv <= 0 || ne < 0) return nullptr;
  crs0_t *g = (crs0_t *)std::malloc(sizeof(crs0_t));
  if (!g) return nullptr;
  g->n = nv;
  g->ptr = (int *)std::malloc(sizeof(int) * (nv + 1));
  g->col = (int *)std::malloc(sizeof(int) * std::max(2L * ne, 1L));
  if (!g->ptr || !g->col) { std::free(g->ptr); std::free(g->col); std::free(g); return nullptr; }
  g->ptr[0] = 0;
  return g;
}

void del_crs(crs0_t *g) {
  if (!g) return;
  std::free(g->ptr);
  std::free(g->col);
  std::free(g);
}

crs0_t *read_crs(FILE *f) {
  clear_error();
  if (!f) { fail(kEInval, "read_crs: null file"); return nullptr; }
  std::string s = slurp_file(f);
  std::fclose(f);
  // parse through a temporary file-free path: reuse the METIS parser on a
  // memory copy by writing it to a unique temporary file would be wasteful,
  // so parse here with the same rules as mpkg::read_metis.
  const char *p = s.c_str(), *end = p + s.size();
  const char *eol = (const char *)std::memchr(p, '\n', end - p);
  if (!eol) eol = end;
  std::string head(p, eol);
  long nv = 0, ne = 0, a = 0, b = 0;
  if (std::sscanf(head.c_str(), "%ld %ld %ld %ld", &nv, &ne, &a, &b) != 2 || nv <= 0 || ne <= 0) {
    fail(kEFormat, "read_crs: header must be 'n ne'");
    return nullptr;
  }
  crs0_t *g = new_crs((int)nv, (int)ne);
  if (!g) { fail(kENoMem, "read_crs: allocation failed"); return nullptr; }
  p = eol < end ? eol + 1 : end;
  long cnt = 0;
  int row = 0;
  while (row < nv && p < end) {
    const char *le = (const char *)std::memchr(p, '\n', end - p);
    if (!le) le = end;
    const char *t = p;
    while (t < le) {
      while (t < le && (unsigned char)*t <= ' ') t++;
      if (t >= le || !std::isdigit((unsigned char)*t)) break;
      long v = 0;
      while (t < le && std::isdigit((unsigned char)*t)) { v = v * 10 + (*t - '0'); t++; if (v > nv + 1) v = nv + 1; }
      if (cnt >= 2 * ne || v < 1 || v > nv) {
        fail(cnt >= 2 * ne ? kEFormat : kERange, "read_crs: too many edges or column out of range");
        del_crs(g);
        return nullptr;
      }
      g->col[cnt++] = (int)(v - 1);
    }
    g->ptr[++row] = (int)cnt;
    p = le < end ? le + 1 : end;
  }
  if (row < nv) { fail(kEFormat, "read_crs: fewer rows than n"); del_crs(g); return nullptr; }
  return g;
}

void write_crs(FILE *f, crs0_t *g) {
  if (!f || !g) return;
  std::fprintf(f, "%d %d\n", g->n, g->ptr[g->n] / 2);
  for (int i = 0; i < g->n; i++) {
    for (int j = g->ptr[i]; j < g->ptr[i + 1]; j++) std::fprintf(f, "%d ", g->col[j] + 1);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
}

coord_t *new_coord(crs0_t *g) {
  if (!g) return nullptr;
  coord_t *c = (coord_t *)std::malloc(sizeof(coord_t));
  c->g = g;
  c->x = (double *)std::malloc(sizeof(double) * g->n);
  c->y = (double *)std::malloc(sizeof(double) * g->n);
  return c;
}

void read_coord(FILE *f, coord_t *cg) {
  if (!f || !cg) return;
  for (int i = 0; i < cg->g->n; i++)
    if (std::fscanf(f, "%lf %lf\n", &cg->x[i], &cg->y[i]) != 2) break;
  std::fclose(f);
}

part_t *new_part(crs0_t *g) {
  if (!g) return nullptr;
  part_t *pg = (part_t *)std::malloc(sizeof(part_t));
  pg->g = g;
  pg->n_part = -1;
  pg->part = (int *)std::malloc(sizeof(int) * g->n);
  return pg;
}

void del_part(part_t *pg) {
  if (!pg) return;
  std::free(pg->part);
  std::free(pg);
}

void read_part(FILE *f, part_t *pg) {
  if (!f || !pg) return;
  int mx = 0;
  for (int i = 0; i < pg->g->n; i++) {
    int p = 0;
    if (std::fscanf(f, "%d", &p) != 1) { fail(kEFormat, "read_part: fewer part ids than vertices"); p = 0; }
    if (mx < p) mx = p;
    pg->part[i] = p;
  }
  pg->n_part = mx + 1;
}

void write_part_c(FILE *f, part_t *pg, coord_t *cg) {
  if (!f || !pg || !cg) return;
  for (int j = 0; j < pg->g->n; j++) {
    if (j > 0 && cg->x[j] != cg->x[j - 1]) std::fprintf(f, "\n");
    std::fprintf(f, "%e %e %d\n", cg->x[j], cg->y[j], pg->part[j]);
  }
  std::fclose(f);
}

level_t *new_level(part_t *pg) {
  if (!pg) return nullptr;
  level_t *lg = (level_t *)std::malloc(sizeof(level_t));
  lg->pg = pg;
  lg->level = (int *)std::malloc(sizeof(int) * pg->g->n);
  return lg;
}

void del_level(level_t *lg) {
  if (!lg) return;
  std::free(lg->level);
  std::free(lg);
}

void comp_level(level_t *lg) {
  clear_error();
  if (!lg) return;
  Csr g = csr_of(lg->pg->g);
  std::vector<int> pv(lg->pg->part, lg->pg->part + g.n), out;
  if (comp_levels(g, pv, lg->pg->n_part, nullptr, &out)) return;
  std::copy(out.begin(), out.end(), lg->level);
}

void update_level(level_t *lg, level_t *lg_org) {
  clear_error();
  if (!lg || !lg_org) return;
  Csr g = csr_of(lg->pg->g);
  std::vector<int> pv(lg->pg->part, lg->pg->part + g.n), lo(lg_org->level, lg_org->level + g.n), out;
  if (comp_levels(g, pv, lg->pg->n_part, &lo, &out)) return;
  std::copy(out.begin(), out.end(), lg->level);
}

void read_level(FILE *f, level_t *lg) {
  if (!f || !lg) return;
  for (int i = 0; i < lg->pg->g->n; i++)
    if (std::fscanf(f, "%d\n", &lg->level[i]) != 1) { fail(kEFormat, "read_level: short file"); break; }
  std::fclose(f);
}

void write_level(FILE *f, level_t *lg) {
  if (!f || !lg) return;
  for (int i = 0; i < lg->pg->g->n; i++) std::fprintf(f, "%d\n", lg->level[i]);
  std::fclose(f);
}

void write_level_c(FILE *f, level_t *lg, coord_t *cg) {
  if (!f || !lg || !cg) return;
  for (int i = 0; i < lg->pg->g->n; i++) {
    if (i > 0 && cg->x[i] != cg->x[i - 1]) std::fprintf(f, "\n");
    std::fprintf(f, "%e %e %d\n", cg->x[i], cg->y[i], lg->level[i]);
  }
  std::fclose(f);
}

wcrs_t *new_wcrs(crs0_t *g) {
  if (!g) return nullptr;
  wcrs_t *w = (wcrs_t *)std::malloc(sizeof(wcrs_t));
  w->g = g;
  w->wv = (int *)std::malloc(sizeof(int) * g->n);
  w->we = (int *)std::malloc(sizeof(int) * std::max(g->ptr[g->n], 1));
  return w;
}

void del_wcrs(wcrs_t *wg) {
  if (!wg) return;
  std::free(wg->we);
  std::free(wg->wv);
  std::free(wg);
}

void write_wcrs(FILE *f, wcrs_t *wg) {
  if (!f || !wg) return;
  crs0_t *g = wg->g;
  std::fprintf(f, "%d %d 011\n", g->n, g->ptr[g->n] / 2);
  for (int i = 0; i < g->n; i++) {
    std::fprintf(f, "1 ");
    for (int j = g->ptr[i]; j < g->ptr[i + 1]; j++) std::fprintf(f, "%d %d ", g->col[j] + 1, wg->we[j]);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
}

void level2wcrs(level_t *lg, wcrs_t *wg) {
  if (!lg || !wg) return;
  Csr g = csr_of(wg->g);
  std::vector<int> lv(lg->level, lg->level + g.n), a, b;
  level_weights(g, lv, &a, &b);
  std::copy(a.begin(), a.end(), wg->wv);
  std::copy(b.begin(), b.end(), wg->we);
}

skirt_t *new_skirt(part_t *pg) {
  if (!pg) return nullptr;
  skirt_t *s = (skirt_t *)std::malloc(sizeof(skirt_t));
  s->pg = pg;
  s->levels = (int *)std::malloc(sizeof(int) * (size_t)pg->n_part * pg->g->n);
  if (!s->levels) { std::free(s); fail(kENoMem, "new_skirt: n_part*n ints do not fit"); return nullptr; }
  return s;
}

void del_skirt(skirt_t *sg) {
  if (!sg) return;
  std::free(sg->levels);
  std::free(sg);
}

// comp_skirt fills the full distance of every vertex to every part (n+1
// when unreachable), like mpk2/lib.c:584-615, by one BFS per part.
void comp_skirt(skirt_t *sg) {
  clear_error();
  if (!sg) return;
  Csr g = csr_of(sg->pg->g);
  const int n = g.n, np = sg->pg->n_part;
  std::vector<std::vector<int>> tr(n);
  for (int i = 0; i < n; i++)
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) tr[g.col[j]].push_back(i);
  std::vector<int> q;
  q.reserve(n);
  for (int p = 0; p < np; p++) {
    int *d = sg->levels + (size_t)p * n;
    q.clear();
    for (int j = 0; j < n; j++) {
      if (sg->pg->part[j] == p) { d[j] = 0; q.push_back(j); }
      else d[j] = n + 1;
    }
    for (size_t h = 0; h < q.size(); h++) {
      int v = q[h];
      for (int i : tr[v])
        if (d[i] > d[v] + 1) { d[i] = d[v] + 1; q.push_back(i); }
    }
  }
}

void write_skirt(FILE *f, skirt_t *sg, level_t *lg, int level) {
  if (!f || !sg) return;
  const int n = sg->pg->g->n, np = sg->pg->n_part;
  std::fprintf(f, "skirt %d nodes, %d parts\n", n, np);
  for (int p = 0; p < np; p++) {
    std::fprintf(f, "partition %d\n", p);
    const int *s = sg->levels + (size_t)p * n;
    for (int j = 0; j < n; j++) {
      bool keep = lg ? (lg->level[j] < level - s[j]) : (s[j] < level);
      if (keep) std::fprintf(f, "%d %d\n", j, level - s[j]);
    }
  }
  std::fclose(f);
}

void read_skirt(FILE *f, skirt_t *sg, int level) {
  clear_error();
  if (!f || !sg || level <= 0) return;
  const int n = sg->pg->g->n, np = sg->pg->n_part;
  char line[256];
  int a = -1, b = -1;
  if (!std::fgets(line, sizeof line, f) || std::sscanf(line, "skirt %d nodes, %d parts", &a, &b) != 2 ||
      a != n || b != np) {
    fail(kEFormat, "read_skirt: header does not match");
    std::fclose(f);
    return;
  }
  for (size_t i = 0; i < (size_t)n * np; i++) sg->levels[i] = -1;
  int p = -1;
  while (std::fgets(line, sizeof line, f)) {
    if (line[0] == 'p') {
      int q = -1;
      std::sscanf(line, "partition %d", &q);
      if (q != p + 1) { fail(kEFormat, "read_skirt: partitions out of order"); break; }
      p = q;
      continue;
    }
    int k, m;
    if (std::sscanf(line, "%d %d", &k, &m) != 2) continue;
    if (p < 0 || p >= np || k < 0 || k >= n || m < 0 || m > level) {
      fail(kERange, "read_skirt: entry out of range");
      break;
    }
    sg->levels[(size_t)p * n + k] = level - m;
  }
  std::fclose(f);
}

mpk_t *new_mpk(crs0_t *g0, int npart, int nlevel, int nphase) {
  if (!g0 || npart <= 0 || nlevel <= 0 || nphase < 0) return nullptr;
  mpk_t *mg = (mpk_t *)std::calloc(1, sizeof(mpk_t));
  mg->n = g0->n;
  mg->npart = npart;
  mg->nlevel = nlevel;
  mg->nphase = nphase;
  mg->g0 = g0;
  int np = nphase == 0 ? 1 : nphase;
  mg->plist = (part_t **)std::calloc(np, sizeof(part_t *));
  mg->llist = nphase == 0 ? nullptr : (level_t **)std::calloc(nphase, sizeof(level_t *));
  mg->sg = nullptr;
  mg->tlist = (task_t *)std::calloc((size_t)npart * (nphase + 1), sizeof(task_t));
  for (long i = 0; i < (long)npart * (nphase + 1); i++) { mg->tlist[i].n = -1; mg->tlist[i].idx = nullptr; }
  mg->idxsrc = nullptr;
  mg->idxallocsize = 0;
  return mg;
}

// read_mpk (mpk2/mpkread.c:49-185): directory ghead_npart_nlevel_nphase
// holding g0, g<ph>.part.<npart>, l<ph> and s<nphase>.
mpk_t *read_mpk(char *dir) {
  clear_error();
  if (!dir) { fail(kEInval, "read_mpk: null dir"); return nullptr; }
  int len = (int)std::strlen(dir), cnt = 0, j = len;
  for (; j >= 0 && cnt < 3; j--)
    if (dir[j] == '_' && ++cnt == 3) break;
  int npart = -1, nlevel = -1, nphase = -1;
  if (cnt != 3 || j < 0 || std::sscanf(dir + j, "_%d_%d_%d", &npart, &nlevel, &nphase) != 3 ||
      npart <= 0 || nlevel <= 0 || nphase < 0) {
    fail(kEFormat, std::string("read_mpk: directory must be named ghead_npart_nlevel_nphase: ") + dir);
    return nullptr;
  }
  std::string d(dir);
  FILE *f = std::fopen((d + "/g0").c_str(), "r");
  if (!f) { fail(kEIo, "read_mpk: cannot open " + d + "/g0"); return nullptr; }
  crs0_t *g0 = read_crs(f);
  if (!g0) return nullptr;
  mpk_t *mg = new_mpk(g0, npart, nlevel, nphase);
  auto load_part = [&](int ph) -> part_t * {
    std::string fn = d + "/g" + std::to_string(ph) + ".part." + std::to_string(npart);
    FILE *pf = std::fopen(fn.c_str(), "r");
    if (!pf) { fail(kEIo, "read_mpk: cannot open " + fn); return nullptr; }
    part_t *pg = new_part(g0);
    read_part(pf, pg);
    std::fclose(pf);
    return pg;
  };
  for (int ph = 0; ph < nphase; ph++) {
    part_t *pg = load_part(ph);
    if (!pg) { del_mpk(mg); return nullptr; }
    mg->plist[ph] = pg;
    std::string fn = d + "/l" + std::to_string(ph);
    FILE *lf = std::fopen(fn.c_str(), "r");
    if (!lf) { fail(kEIo, "read_mpk: cannot open " + fn); del_mpk(mg); return nullptr; }
    level_t *lg = new_level(pg);
    read_level(lf, lg);
    mg->llist[ph] = lg;
  }
  if (nphase == 0) {
    part_t *pg = load_part(0);
    if (!pg) { del_mpk(mg); return nullptr; }
    mg->plist[0] = pg;
  }
  std::string fn = d + "/s" + std::to_string(nphase);
  FILE *sf = std::fopen(fn.c_str(), "r");
  if (!sf) { fail(kEIo, "read_mpk: cannot open " + fn); del_mpk(mg); return nullptr; }
  // the skirt is sized by the partition read for phase 0 (as the reference)
  mg->plist[0]->n_part = std::max(mg->plist[0]->n_part, npart);
  skirt_t *sk = new_skirt(mg->plist[0]);
  if (!sk) { std::fclose(sf); del_mpk(mg); return nullptr; }
  read_skirt(sf, sk, nlevel);
  mg->sg = sk;
  long c = (long)mg->n * nlevel;
  for (long i = 0; i < (long)npart * mg->n; i++)
    if (sk->levels[i] >= 0) c += nlevel - sk->levels[i] + 1;
  mg->idxsrc = (long *)std::malloc(sizeof(long) * std::max(c, 1L));
  mg->idxallocsize = c;
  return mg;
}

void del_mpk(mpk_t *mg) {
  if (!mg) return;
  drop_plans(mg);
  if (mg->sg) del_skirt(mg->sg);
  int np = mg->nphase == 0 ? 1 : mg->nphase;
  for (int i = 0; i < np; i++) if (mg->plist && mg->plist[i]) del_part(mg->plist[i]);
  for (int i = 0; i < mg->nphase; i++) if (mg->llist && mg->llist[i]) del_level(mg->llist[i]);
  std::free(mg->plist);
  std::free(mg->llist);
  std::free(mg->tlist);
  std::free(mg->idxsrc);
  if (mg->g0) del_crs(mg->g0);
  std::free(mg);
}

// prep_mpk (mpk2/mpkprep.c:7-258): builds the task lists into idxsrc and
// runs the reference's dependency checks; vv is not used as scratch.
void prep_mpk(mpk_t *mg, double *vv) {
  clear_error();
  (void)vv;
  if (!mg || !mg->sg || !mg->plist || !mg->plist[0]) { fail(kEInval, "prep_mpk: incomplete mpk_t"); return; }
  drop_plans(mg);
  const int n = mg->n, np = mg->npart;
  Csr g = csr_of(mg->g0);
  std::vector<std::vector<int>> parts, levels;
  for (int ph = 0; ph < std::max(mg->nphase, 1); ph++)
    parts.emplace_back(mg->plist[ph]->part, mg->plist[ph]->part + n);
  for (int ph = 0; ph < mg->nphase; ph++) levels.emplace_back(mg->llist[ph]->level, mg->llist[ph]->level + n);
  std::vector<PartSkirt> sk(np);
  for (int p = 0; p < np; p++) {
    const int *s = mg->sg->levels + (size_t)p * n;
    for (int i = 0; i < n; i++)
      if (s[i] >= 0) { sk[p].vert.push_back(i); sk[p].dist.push_back(s[i]); }
  }
  TaskLists tl;
  if (build_tasks(g, np, mg->nlevel, mg->nphase, parts, levels, sk, true, &tl)) return;
  if ((long)tl.idx.size() > mg->idxallocsize || !mg->idxsrc) {
    std::free(mg->idxsrc);
    mg->idxsrc = (long *)std::malloc(sizeof(long) * std::max<size_t>(tl.idx.size(), 1));
    mg->idxallocsize = (long)tl.idx.size();
  }
  std::copy(tl.idx.begin(), tl.idx.end(), mg->idxsrc);
  for (long t = 0; t < (long)(mg->nphase + 1) * np; t++) {
    mg->tlist[t].n = (int)(tl.off[t + 1] - tl.off[t]);
    mg->tlist[t].idx = mg->idxsrc + tl.off[t];
  }
}

void exec_mpk(mpk_t *mg, double *vv, int nthread) { (void)nthread; legacy_exec(mg, vv, nullptr); }
void exec_mpk_xs(mpk_t *mg, double *vv, int nthread) { (void)nthread; legacy_exec(mg, vv, nullptr); }
void exec_mpk_xd(mpk_t *mg, double *vv, int nthread) { (void)nthread; legacy_exec(mg, vv, nullptr); }
void exec_mpk_is(mpk_t *mg, double *vv, int nthread) { (void)nthread; legacy_exec(mg, vv, nullptr); }
void exec_mpk_id(mpk_t *mg, double *vv, int nthread) { (void)nthread; legacy_exec(mg, vv, nullptr); }
void vexec_mpk(mpk_t *mg, double *vv, double *val) { legacy_exec(mg, vv, val); }

void exec_mpkt(mpk_t *mg, double *vv, int nth) {
  (void)nth;
  if (!mg || !vv) return;
  const int n = mg->n, nl1 = mg->nlevel + 1;
  std::vector<double> lm((size_t)n * nl1);
  for (int i = 0; i < n; i++)
    for (int l = 0; l < nl1; l++) lm[(size_t)l * n + i] = vv[(size_t)i * nl1 + l];
  legacy_exec(mg, lm.data(), nullptr);
  for (int i = 0; i < n; i++)
    for (int l = 1; l < nl1; l++) vv[(size_t)i * nl1 + l] = lm[(size_t)l * n + i];
}

static void legacy_spmv(crs0_t *g0, double *vv, int nlevel) {
  clear_error();
  if (!g0 || !vv || nlevel <= 0) { fail(kEInval, "spmv_exec: bad argument"); return; }
  mpkg_plan *p = nullptr;
  if (mpkg_plan_spmv(g0->n, g0->ptr, g0->col, nullptr, nlevel, legacy_arith(), &p)) return;
  mpkg_exec_host(p, vv);
  mpkg_plan_destroy(p);
}

void spmv_exec_seq(crs0_t *g0, double *vv, int nlevel) { legacy_spmv(g0, vv, nlevel); }
void spmv_exec_par(crs0_t *g0, double *vv, int nlevel, int nth) { (void)nth; legacy_spmv(g0, vv, nlevel); }

}  // extern "C"
