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

int mpkg_pdmpk_info(int npart, const char *const *buf_paths, const char *const *results_paths, int *n,
                    int *nlevel, int *nbatch, long *rows) {
  clear_error();
  if (npart <= 0 || !buf_paths || !results_paths) return fail(kEInval, "bad argument");
  std::vector<pdmpk_gb300::Buffers> bufs(npart, pdmpk_gb300::Buffers(npart));
  int rc;
  for (int r = 0; r < npart; r++) {
    if (!buf_paths[r] || !results_paths[r]) return fail(kEInval, "null path");
    if ((rc = bufs[r].Load(buf_paths[r], results_paths[r]))) return rc;
  }
  PdExecMaps m;
  if ((rc = pd_exec_maps(bufs, &m))) return rc;
  if (n) *n = m.n;
  if (nlevel) *nlevel = m.nlevel;
  if (nbatch) *nbatch = m.nbatch;
  if (rows) *rows = (long)m.row_dst.size();
  return kOk;
}

int mpkg_read_mtx(const char *path, int *n, long *nnz, int **ptr, int **col, double **val) {
  clear_error();
  if (!path || !n || !nnz || !ptr || !col || !val) return fail(kEInval, "null argument");
  Csr g;
  int rc = read_mtx(path, &g);
  if (rc) return rc;
  *n = g.n;
  *nnz = g.nnz();
  *ptr = dup(g.ptr);
  *col = dup(g.col);
  *val = dup(g.val);
  if (!*ptr || (g.nnz() && (!*col || !*val))) return fail(kENoMem, "allocation failed");
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

int mpkg_have_metis(void) { return have_metis() ? 1 : 0; }

int mpkg_partition_metis(int n, const int *ptr, const int *col, const int *vwgt, const int *adjwgt, int npart,
                         int ufactor, int *part, long *edgecut) {
  clear_error();
  int rc = check_csr_host(n, ptr, col);
  if (rc) return rc;
  if (!part) return fail(kEInval, "null argument");
  Csr g = view_csr(n, ptr, col);
  std::vector<int> out;
  rc = partition_metis(g, vwgt, adjwgt, npart, ufactor, &out, edgecut);
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

int mpkg_gen_diffusion(int nx, int ny, int nz, double sigma, double wx, double wy, double wdiag,
                       double dominance, uint64_t seed, int *n, long *nnz, int **ptr, int **col, double **val) {
  clear_error();
  if (!n || !nnz || !ptr || !col || !val) return fail(kEInval, "null argument");
  Csr g;
  int rc = nz <= 1 ? gen_diffusion_9pt(nx, ny, sigma, wx, wy, wdiag, dominance, seed, &g)
                   : gen_diffusion_7pt(nx, ny, nz, sigma, dominance, seed, &g);
  if (rc) return rc;
  *n = g.n; *nnz = g.nnz();
  *ptr = dup(g.ptr); *col = dup(g.col); *val = dup(g.val);
  return kOk;
}

int mpkg_gen_banded(long n, int bw, int nmin, int nmax, uint64_t seed, int *nout, long *nnz, int **ptr, int **col,
                    double **val) {
  clear_error();
  if (!nout || !nnz || !ptr || !col || !val) return fail(kEInval, "null argument");
  Csr g;
  int rc = gen_banded(n, bw, nmin, nmax, seed, &g);
  if (rc) return rc;
  *nout = g.n; *nnz = g.nnz();
  *ptr = dup(g.ptr); *col = dup(g.col); *val = dup(g.val);
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
  // Task lists that cover every (level, vertex) write every entry of vv
  // levels 1..nlevel, each with its row's FMA chain in CSR order whichever
  // task computes it; the wavefront computes each entry once and gives the
  // same bits, so it runs such lists (PA1 and every complete DMPK list
  // set).  Lists that leave entries untouched keep the task executor.
  const long n = mg->n, cells = n * mg->nlevel;
  std::vector<unsigned char> cov((size_t)cells, 0);
  long covered = 0;
  for (long v : idx) {
    const long l = v / n, i = v - l * n;
    if (l >= 1 && l <= mg->nlevel && !cov[(size_t)((l - 1) * n + i)]) {
      cov[(size_t)((l - 1) * n + i)] = 1;
      covered++;
    }
  }
  int rc = 1;
  if (covered == cells) {
    rc = mpkg_plan_wave(mg->n, mg->g0->ptr, mg->g0->col, val, mg->nlevel, legacy_arith(), &p);
    if (rc) clear_error();
  }
  if (rc) rc = mpkg_plan_tasks(mg->n, mg->g0->ptr, mg->g0->col, val, mg->npart, mg->nlevel, mg->nphase,
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

// ==========================================================================
// MPI-2 prep: comm_data_t and buffers_t (mpk2/comm_data.h, mpk2/buffers.h)
// ==========================================================================
namespace {

// "ghead_npart_nlevel_nphase" parsed from the end of the directory name.
bool parse_dir(const char *dir, int *npart, int *nlevel, int *nphase) {
  int len = (int)std::strlen(dir), cnt = 0, j = len;
  for (; j >= 0; j--)
    if (dir[j] == '_' && ++cnt == 3) break;
  *npart = *nlevel = *nphase = -1;
  return cnt == 3 && j >= 0 && std::sscanf(dir + j, "_%d_%d_%d", npart, nlevel, nphase) == 3 && *npart > 0 &&
         *nlevel > 0 && *nphase >= 0;
}

// <dir up to its first '_'>.loop.val (mpk2/comm_data.c:160-187)
std::string values_path(const char *dir) {
  std::string d(dir);
  size_t u = d.find('_');
  return (u == std::string::npos ? d : d.substr(0, u)) + ".loop.val";
}

buffers_t *to_legacy(const RankBuffers &b) {
  buffers_t *o = (buffers_t *)std::calloc(1, sizeof(buffers_t));
  o->n = b.n; o->npart = b.npart; o->nlevel = b.nlevel; o->nphase = b.nphase; o->rank = b.rank;
  o->buf_count = b.buf_count; o->buf_scount = b.buf_scount; o->mptr_count = b.mptr_count;
  o->mcol_count = b.mcol_count;
  o->recvcounts = dup(b.recvcounts); o->sendcounts = dup(b.sendcounts);
  o->rdispls = dup(b.rdispls); o->sdispls = dup(b.sdispls);
  o->rcount = dup(b.rcount); o->mcount = dup(b.mcount); o->scount = dup(b.scount);
  o->rbuf_offsets = dup(b.rbuf_offsets); o->mbuf_offsets = dup(b.mbuf_offsets);
  o->sbuf_offsets = dup(b.sbuf_offsets); o->mptr_offsets = dup(b.mptr_offsets);
  o->mcol_offsets = dup(b.mcol_offsets);
  o->idx_buf = dup(b.idx_buf); o->idx_sbuf = dup(b.idx_sbuf);
  o->mptr_buf = dup(b.mptr_buf); o->mcol_buf = dup(b.mcol_buf);
  o->mval_buf = b.mval_buf.empty() ? nullptr : dup(b.mval_buf);
  return o;
}

RankBuffers from_legacy(const buffers_t *o) {
  RankBuffers b;
  b.n = o->n; b.npart = o->npart; b.nlevel = o->nlevel; b.nphase = o->nphase; b.rank = o->rank;
  b.buf_count = o->buf_count; b.buf_scount = o->buf_scount; b.mptr_count = o->mptr_count;
  b.mcol_count = o->mcol_count;
  const size_t np = (size_t)o->npart * (o->nphase + 1), ph = (size_t)o->nphase + 1;
  b.recvcounts.assign(o->recvcounts, o->recvcounts + np); b.sendcounts.assign(o->sendcounts, o->sendcounts + np);
  b.rdispls.assign(o->rdispls, o->rdispls + np); b.sdispls.assign(o->sdispls, o->sdispls + np);
  b.rcount.assign(o->rcount, o->rcount + ph); b.mcount.assign(o->mcount, o->mcount + ph);
  b.scount.assign(o->scount, o->scount + ph);
  b.rbuf_offsets.assign(o->rbuf_offsets, o->rbuf_offsets + ph);
  b.mbuf_offsets.assign(o->mbuf_offsets, o->mbuf_offsets + ph);
  b.sbuf_offsets.assign(o->sbuf_offsets, o->sbuf_offsets + ph);
  b.mptr_offsets.assign(o->mptr_offsets, o->mptr_offsets + ph);
  b.mcol_offsets.assign(o->mcol_offsets, o->mcol_offsets + ph);
  b.idx_buf.assign(o->idx_buf, o->idx_buf + o->buf_count);
  b.idx_sbuf.assign(o->idx_sbuf, o->idx_sbuf + o->buf_scount);
  b.mptr_buf.assign(o->mptr_buf, o->mptr_buf + o->mptr_count);
  b.mcol_buf.assign(o->mcol_buf, o->mcol_buf + o->mcol_count);
  if (o->mval_buf) b.mval_buf.assign(o->mval_buf, o->mval_buf + o->mcol_count);
  return b;
}

// The inputs of the MPI-2 prep from a comm_data_t.
void comm_inputs(const comm_data_t *cd, Csr *g, std::vector<std::vector<int>> *parts,
                 std::vector<std::vector<int>> *levels, std::vector<PartSkirt> *sk) {
  *g = csr_of(cd->graph);
  const int n = cd->n;
  parts->clear();
  levels->clear();
  for (int ph = 0; ph < std::max(cd->nphase, 1); ph++)
    parts->emplace_back(cd->plist[ph]->part, cd->plist[ph]->part + n);
  for (int ph = 0; ph < cd->nphase; ph++) levels->emplace_back(cd->llist[ph]->level, cd->llist[ph]->level + n);
  sk->assign(cd->npart, PartSkirt());
  for (int p = 0; p < cd->npart; p++) {
    const int *s = cd->skirt->levels + (size_t)p * n;
    for (int i = 0; i < n; i++)
      if (s[i] >= 0) { (*sk)[p].vert.push_back(i); (*sk)[p].dist.push_back(s[i]); }
  }
}

}  // namespace

extern "C" {

void dir_name_error(char *dir) {
  fail(kEFormat, std::string("unknown directory naming ") + (dir ? dir : "") +
                     " (expecting ghead_npart_nlevel_nphase)");
}

crs0_t *read_matrix(char *dir) {
  clear_error();
  if (!dir) return nullptr;
  FILE *f = std::fopen((std::string(dir) + "/loop.g0").c_str(), "r");
  if (!f) { fail(kEIo, std::string("cannot open ") + dir + "/loop.g0"); return nullptr; }
  return read_crs(f);
}

double *alloc_read_val(crs0_t *g0, char *dir) {
  clear_error();
  if (!g0 || !dir) return nullptr;
  std::vector<double> v;
  if (read_values(values_path(dir), g0->ptr[g0->n], &v)) return nullptr;
  return dup(v);
}

comm_data_t *new_comm_data(char *dir, int rank) {
  clear_error();
  int npart, nlevel, nphase;
  if (!dir || !parse_dir(dir, &npart, &nlevel, &nphase)) { dir_name_error(dir); return nullptr; }
  crs0_t *g = read_matrix(dir);
  if (!g) return nullptr;
  comm_data_t *cd = (comm_data_t *)std::calloc(1, sizeof(comm_data_t));
  cd->dir = dir; cd->rank = rank; cd->npart = npart; cd->nlevel = nlevel; cd->nphase = nphase;
  cd->graph = g;
  cd->n = g->n;
  const int np = nphase == 0 ? 1 : nphase;
  cd->plist = (part_t **)std::calloc(np, sizeof(part_t *));
  cd->llist = nphase == 0 ? nullptr : (level_t **)std::calloc(nphase, sizeof(level_t *));
  std::string d(dir);
  bool ok = true;
  for (int ph = 0; ph < np && ok; ph++) {
    std::string fn = d + "/g" + std::to_string(ph) + ".part." + std::to_string(npart);
    FILE *f = std::fopen(fn.c_str(), "r");
    if (!f) { fail(kEIo, "cannot open " + fn); ok = false; break; }
    cd->plist[ph] = new_part(g);
    read_part(f, cd->plist[ph]);
    std::fclose(f);
    if (nphase > 0) {
      fn = d + "/l" + std::to_string(ph);
      f = std::fopen(fn.c_str(), "r");
      if (!f) { fail(kEIo, "cannot open " + fn); ok = false; break; }
      cd->llist[ph] = new_level(cd->plist[ph]);
      read_level(f, cd->llist[ph]);
    }
  }
  if (ok) {
    std::string fn = d + "/s" + std::to_string(nphase);
    FILE *f = std::fopen(fn.c_str(), "r");
    if (!f) { fail(kEIo, "cannot open " + fn); ok = false; }
    else {
      cd->plist[0]->n_part = std::max(cd->plist[0]->n_part, npart);
      cd->skirt = new_skirt(cd->plist[0]);
      if (!cd->skirt) { std::fclose(f); ok = false; }
      else read_skirt(f, cd->skirt, nlevel);
    }
  }
  if (!ok) { del_comm_data(cd); return nullptr; }
  return cd;
}

void del_comm_data(comm_data_t *cd) {
  if (!cd) return;
  const int np = cd->nphase == 0 ? 1 : cd->nphase;
  for (int ph = 0; ph < np; ph++) if (cd->plist && cd->plist[ph]) del_part(cd->plist[ph]);
  for (int ph = 0; ph < cd->nphase; ph++) if (cd->llist && cd->llist[ph]) del_level(cd->llist[ph]);
  std::free(cd->plist);
  std::free(cd->llist);
  if (cd->skirt) del_skirt(cd->skirt);
  if (cd->graph) del_crs(cd->graph);
  std::free(cd);
}

void check_args(int argc, char *argv0) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s dirname\n", argv0 ? argv0 : "prog");
    std::exit(1);
  }
}

buffers_t *new_bufs(comm_data_t *cd) {
  if (!cd) return nullptr;
  buffers_t *b = (buffers_t *)std::calloc(1, sizeof(buffers_t));
  b->n = cd->n; b->npart = cd->npart; b->nlevel = cd->nlevel; b->nphase = cd->nphase; b->rank = cd->rank;
  return b;
}

void alloc_val_bufs(buffers_t *b) {
  if (!b) return;
  std::free(b->vv_buf);
  std::free(b->vv_sbuf);
  b->vv_buf = (double *)std::calloc(std::max(b->buf_count, 1), sizeof(double));
  b->vv_sbuf = (double *)std::calloc(std::max(b->buf_scount, 1), sizeof(double));
}

void del_bufs(buffers_t *b) {
  if (!b) return;
  for (void *q : {(void *)b->recvcounts, (void *)b->sendcounts, (void *)b->rdispls, (void *)b->sdispls,
                  (void *)b->rcount, (void *)b->mcount, (void *)b->scount, (void *)b->rbuf_offsets,
                  (void *)b->mbuf_offsets, (void *)b->sbuf_offsets, (void *)b->mptr_offsets,
                  (void *)b->mcol_offsets, (void *)b->idx_buf, (void *)b->idx_sbuf, (void *)b->mptr_buf,
                  (void *)b->mcol_buf, (void *)b->vv_buf, (void *)b->vv_sbuf, (void *)b->mval_buf})
    std::free(q);
  std::free(b);
}

void fill_buffers(comm_data_t *cd, buffers_t *bufs) {
  clear_error();
  if (!cd || !bufs) { fail(kEInval, "fill_buffers: null argument"); return; }
  Csr g;
  std::vector<std::vector<int>> parts, levels;
  std::vector<PartSkirt> sk;
  comm_inputs(cd, &g, &parts, &levels, &sk);
  std::vector<RankBuffers> all;
  if (fill_all_buffers(g, cd->npart, cd->nlevel, cd->nphase, &parts, levels, sk, &all)) return;
  for (int ph = 1; ph < cd->nphase; ph++)  // the relabelling reduce_comm applies
    std::copy(parts[ph].begin(), parts[ph].end(), cd->plist[ph]->part);
  buffers_t *o = to_legacy(all[cd->rank]);
  double *vv = bufs->vv_buf, *vs = bufs->vv_sbuf;
  for (void *q : {(void *)bufs->recvcounts, (void *)bufs->sendcounts, (void *)bufs->rdispls, (void *)bufs->sdispls,
                  (void *)bufs->rcount, (void *)bufs->mcount, (void *)bufs->scount, (void *)bufs->rbuf_offsets,
                  (void *)bufs->mbuf_offsets, (void *)bufs->sbuf_offsets, (void *)bufs->mptr_offsets,
                  (void *)bufs->mcol_offsets, (void *)bufs->idx_buf, (void *)bufs->idx_sbuf, (void *)bufs->mptr_buf,
                  (void *)bufs->mcol_buf, (void *)bufs->mval_buf})
    std::free(q);
  *bufs = *o;
  bufs->vv_buf = vv;
  bufs->vv_sbuf = vs;
  bufs->mval_buf = nullptr;  // filled by the caller, as mpi2_mpkwrtbufs does
  std::free(o);
}

void write_buffers(buffers_t *bufs, char *dir) {
  clear_error();
  if (!bufs || !dir) return;
  write_rank_buffers(std::string(dir) + "/rank" + std::to_string(bufs->rank) + ".bufs", from_legacy(bufs));
}

buffers_t *read_buffers(char *dir, int rank) {
  clear_error();
  if (!dir) return nullptr;
  RankBuffers b;
  if (read_rank_buffers(std::string(dir) + "/rank" + std::to_string(rank) + ".bufs", &b)) return nullptr;
  return to_legacy(b);
}

int mpkg_bufs_prepare(const char *dir) {
  clear_error();
  if (!dir) return fail(kEInval, "null dir");
  comm_data_t *cd = new_comm_data(const_cast<char *>(dir), 0);
  if (!cd) return kEIo;
  Csr g;
  std::vector<std::vector<int>> parts, levels;
  std::vector<PartSkirt> sk;
  comm_inputs(cd, &g, &parts, &levels, &sk);
  int rc = read_values(values_path(dir), g.nnz(), &g.val);
  std::vector<RankBuffers> all;
  if (!rc) rc = fill_all_buffers(g, cd->npart, cd->nlevel, cd->nphase, &parts, levels, sk, &all);
  for (int r = 0; !rc && r < cd->npart; r++)
    rc = write_rank_buffers(std::string(dir) + "/rank" + std::to_string(r) + ".bufs", all[r]);
  del_comm_data(cd);
  return rc;
}

}  // extern "C"

// ==========================================================================
// Verification counts (mpk2/work_count.c) and the label assignment
// (mpk2/lapjv.c:366 lapjv)
// ==========================================================================
extern "C" {

int mpkg_work_count(const char *dir, long *comm, long *ops, long *minops, long *nvert, long *redundant) {
  clear_error();
  if (!dir || !comm || !ops || !minops || !nvert) return fail(kEInval, "null argument");
  int npart, nlevel, nphase;
  if (!parse_dir(dir, &npart, &nlevel, &nphase)) {
    dir_name_error(const_cast<char *>(dir));
    return kEFormat;
  }
  crs0_t *g = read_matrix(const_cast<char *>(dir));
  if (!g) return kEIo;
  const int n = g->n;
  const long nnz = g->ptr[n];
  del_crs(g);
  std::vector<RankBuffers> bufs(npart);
  for (int r = 0; r < npart; r++) {
    int rc = read_rank_buffers(std::string(dir) + "/rank" + std::to_string(r) + ".bufs", &bufs[r]);
    if (rc) return rc;
    if (bufs[r].n != n || bufs[r].npart != npart || bufs[r].nlevel != nlevel || bufs[r].nphase != nphase)
      return fail(kEFormat, "rank " + std::to_string(r) + ": buffer header does not match " + dir);
  }
  int rc = check_rank_buffers(bufs);
  if (rc) return rc;
  // count_comm: received doubles minus those a rank keeps for itself
  long c = 0, o = 0, red = 0;
  for (int ph = 0; ph <= nphase; ph++)
    for (int p = 0; p < npart; p++) {
      const RankBuffers &b = bufs[p];
      const long self = (long)npart * ph + p;
      if (b.sendcounts[self] != b.recvcounts[self]) return fail(kEFormat, "send/receive counts differ");
      c += b.rcount[ph] - b.recvcounts[self];
    }
  // count_ops: the row lengths of every rank's local CSR, all phases
  for (int ph = 0; ph <= nphase; ph++)
    for (int p = 0; p < npart; p++) {
      const RankBuffers &b = bufs[p];
      const long *mp = b.mptr_buf.data() + b.mptr_offsets[ph];
      for (int t = 0; t < b.mcount[ph]; t++) o += mp[t + 1] - mp[t];
    }
  // redundancy: an index received in some phase that the rank also
  // computes (received once and computed once: the reference's tmp == 3)
  const long size = (long)n * (nlevel + 1);
  std::vector<unsigned char> computed(size), got(size);
  for (int p = 0; p < npart; p++) {
    const RankBuffers &b = bufs[p];
    std::fill(computed.begin(), computed.end(), 0);
    for (int ph = 0; ph <= nphase; ph++)
      for (int mi = 0; mi < b.mcount[ph]; mi++) {
        const long e = b.idx_buf[b.mbuf_offsets[ph] + mi];
        if (e < 0 || e >= size) return fail(kEFormat, "buffer index out of range");
        if (computed[e] < 255) computed[e]++;
      }
    for (int ph = 0; ph <= nphase; ph++) {
      std::fill(got.begin(), got.end(), 0);
      for (int ri = 0; ri < b.rcount[ph]; ri++) {
        const long e = b.idx_buf[b.rbuf_offsets[ph] + ri];
        if (e < 0 || e >= size) return fail(kEFormat, "buffer index out of range");
        if (got[e] < 255) got[e]++;
      }
      for (long e = 0; e < size; e++) red += got[e] == 1 && computed[e] == 1;
    }
  }
  *comm = c;
  *ops = o;
  *minops = (long)nlevel * nnz;
  *nvert = (long)n * nlevel;
  if (redundant) *redundant = red;
  return kOk;
}

int mpkg_lapjv(const int *sums, int npart, int *perm) {
  clear_error();
  if (!sums || !perm || npart <= 0) return fail(kEInval, "bad argument");
  std::vector<long> s(sums, sums + (long)npart * npart);
  std::vector<int> pv;
  assign_max_trace(s, npart, &pv);
  std::copy(pv.begin(), pv.end(), perm);
  return kOk;
}

}  // extern "C"
