// Graph and matrix input/output and the synthetic matrix generators.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "host.h"

namespace mpkg {

namespace {
thread_local std::string g_last_error;

// Reads a whole file into memory.
int slurp(const std::string &path, std::string *out) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(kEIo, "cannot open " + path);
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out->resize(sz > 0 ? sz : 0);
  if (sz > 0 && std::fread(&(*out)[0], 1, sz, f) != (size_t)sz) {
    std::fclose(f);
    return fail(kEIo, "short read on " + path);
  }
  std::fclose(f);
  return kOk;
}
}  // namespace

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}
const char *last_error() { return g_last_error.c_str(); }
void clear_error() { g_last_error.clear(); }

// METIS text graph reader.  Semantics follow read_crs (mpk2/lib.c:69-129):
// the header must hold exactly two integers n and ne (n, ne > 0); each of
// the next n lines lists 1-based neighbours; parsing of a line stops at
// the first token that is not an unsigned integer; at most 2*ne columns;
// every column in [1, n].  A file with fewer than n rows is an error here
// (the reference leaves those row pointers uninitialised).
int read_metis(const std::string &path, Csr *g, long *ne_header) {
  std::string buf;
  int rc = slurp(path, &buf);
  if (rc) return rc;
  const char *s = buf.c_str();
  const char *end = s + buf.size();
  const char *eol = (const char *)std::memchr(s, '\n', end - s);
  if (!eol) eol = end;
  std::string head(s, eol);
  long nv = 0, ne = 0, p = 0, q = 0;
  int nf = std::sscanf(head.c_str(), "%ld %ld %ld %ld", &nv, &ne, &p, &q);
  if (nf != 2) return fail(kEFormat, path + ": header must be 'n ne' (weighted formats are not read)");
  if (nv <= 0 || ne <= 0 || nv > 0x7fffffffL) return fail(kEFormat, path + ": bad n/ne in header");
  s = eol < end ? eol + 1 : end;
  g->n = (int)nv;
  g->ptr.assign(nv + 1, 0);
  g->col.clear();
  g->col.reserve(std::min<long>(2 * ne, 1L << 31));
  g->val.clear();
  long row = 0;
  while (row < nv && s < end) {
    const char *le = (const char *)std::memchr(s, '\n', end - s);
    if (!le) le = end;
    const char *t = s;
    while (t < le) {
      while (t < le && (unsigned char)*t <= ' ') t++;
      if (t >= le) break;
      if (!std::isdigit((unsigned char)*t)) break;  // non-numeric token ends the row
      long v = 0;
      while (t < le && std::isdigit((unsigned char)*t)) { v = v * 10 + (*t - '0'); t++; if (v > nv + 1) v = nv + 1; }
      if ((long)g->col.size() >= 2 * ne)
        return fail(kEFormat, path + ": too many edges (more than 2*ne columns)");
      if (v < 1 || v > nv) return fail(kERange, path + ": column out of range in row " + std::to_string(row));
      g->col.push_back((int)(v - 1));
    }
    row++;
    g->ptr[row] = (int)g->col.size();
    s = le < end ? le + 1 : end;
  }
  if (row < nv) return fail(kEFormat, path + ": fewer rows than the header's n");
  if (ne_header) *ne_header = ne;
  return kOk;
}

int write_metis(const std::string &path, const Csr &g, long ne_header) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return fail(kEIo, "cannot open " + path);
  std::fprintf(f, "%d %ld\n", g.n, ne_header);
  for (int i = 0; i < g.n; i++) {
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) std::fprintf(f, "%d ", g.col[j] + 1);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
  return kOk;
}

int read_values(const std::string &path, long nnz, std::vector<double> *val) {
  std::string buf;
  int rc = slurp(path, &buf);
  if (rc) return rc;
  val->resize(nnz);
  const char *s = buf.c_str();
  char *e = nullptr;
  for (long i = 0; i < nnz; i++) {
    double v = std::strtod(s, &e);
    if (e == s) return fail(kEFormat, path + ": fewer values than nonzeros");
    (*val)[i] = v;
    s = e;
  }
  return kOk;
}

int write_values(const std::string &path, const std::vector<double> &val) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return fail(kEIo, "cannot open " + path);
  for (double v : val) std::fprintf(f, "%.17g ", v);
  std::fclose(f);
  return kOk;
}

// Matrix Market reader with the semantics of pdmpk/csr.cc:9-122:
// banner "%%MatrixMarket matrix coordinate real|pattern general|symmetric",
// comment lines, "m n nnz" with m == n, 1-based entries kept per row in file
// order, symmetric off-diagonal entries mirrored into the column's row,
// pattern matrices get 1/deg values per row.  The row pointers count every
// stored entry, mirrored ones included.
int read_mtx(const std::string &path, Csr *g) {
  std::ifstream file(path);
  if (!file) return fail(kEIo, "cannot open " + path);
  std::string line, word;
  std::getline(file, line);
  std::stringstream banner(line);
  std::string w0, w1, w2, w3, w4;
  banner >> w0 >> w1 >> w2 >> w3 >> w4;
  if (w0 != "%%MatrixMarket" || w1 != "matrix") return fail(kEFormat, "incorrect mtx banner");
  if (w2 != "coordinate") return fail(kEFormat, "not a coordinate (sparse) matrix");
  bool pattern = (w3 == "pattern");
  if (!pattern && w3 != "real") return fail(kEFormat, "not a real or pattern matrix");
  bool symmetric = (w4 == "symmetric");
  if (!symmetric && w4 != "general") return fail(kEFormat, "not a general or symmetric matrix");
  do {
    if (!std::getline(file, line)) return fail(kEFormat, "missing size line");
  } while (!line.empty() && line[0] == '%');
  long m = 0, n = 0, nnz = 0;
  {
    std::stringstream ss(line);
    ss >> m >> n >> nnz;
  }
  if (m != n || n <= 0) return fail(kEFormat, "matrix not square");
  std::vector<std::vector<int>> js(n);
  std::vector<std::vector<double>> vs(n);
  while (std::getline(file, line)) {
    if (line.empty() || line[0] == '%') continue;
    std::stringstream ss(line);
    long i, j;
    double v = 1.0;
    if (!(ss >> i >> j)) continue;
    if (!pattern) ss >> v;
    i--; j--;
    if (i < 0 || i >= n || j < 0 || j >= n) return fail(kERange, "entry out of range");
    js[i].push_back((int)j);
    vs[i].push_back(v);
    if (symmetric && i != j) {
      js[j].push_back((int)i);
      vs[j].push_back(v);
    }
  }
  g->n = (int)n;
  g->ptr.assign(n + 1, 0);
  g->col.clear();
  g->val.clear();
  for (long i = 0; i < n; i++) {
    g->ptr[i + 1] = g->ptr[i] + (int)js[i].size();
    g->col.insert(g->col.end(), js[i].begin(), js[i].end());
    if (pattern) {
      double a = js[i].empty() ? 0.0 : 1.0 / (double)js[i].size();
      g->val.insert(g->val.end(), js[i].size(), a);
    } else {
      g->val.insert(g->val.end(), vs[i].begin(), vs[i].end());
    }
  }
  return kOk;
}

// The five stencil families of mpk2/gen2.c:59-267 (rows, column order and
// values as gen2 writes them).
int gen_reference_stencil(const std::string &type, int size, Csr *g) {
  if (size <= 0) return fail(kEInval, "size must be positive");
  const int n = size;
  g->ptr.clear(); g->col.clear(); g->val.clear();
  g->ptr.push_back(0);
  auto put = [&](int c, double v) { g->col.push_back(c); g->val.push_back(v); };
  if (type == "m5p" || type == "t5p" || type == "m7p" || type == "m9p") {
    g->n = n * n;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        int me = i * n + j;
        if (type == "m5p") {
          if (i > 0) put((i - 1) * n + j, 1);
          if (j > 0) put(me - 1, 1);
          put(me, -4);
          if (j < n - 1) put(me + 1, 1);
          if (i < n - 1) put((i + 1) * n + j, 1);
        } else if (type == "t5p") {
          if (i == n - 1) put(j, 1);
          if (i > 0) put((i - 1) * n + j, 1);
          if (j == n - 1) put(i * n, 1);
          if (j > 0) put(me - 1, 1);
          put(me, -4);
          if (i < n - 1) put((i + 1) * n + j, 1);
          if (j < n - 1) put(me + 1, 1);
          if (i == 0) put((n - 1) * n + j, 1);
          if (j == 0) put(i * n + n - 1, 1);
        } else if (type == "m7p") {
          if (i > 0 && j > 0) put((i - 1) * n + j - 1, 1);
          if (i > 0) put((i - 1) * n + j, 1);
          if (j > 0) put(me - 1, 1);
          put(me, -6);
          if (j < n - 1) put(me + 1, 1);
          if (i < n - 1) put((i + 1) * n + j, 1);
          if (i < n - 1 && j < n - 1) put((i + 1) * n + j + 1, 1);
        } else {  // m9p
          if (i > 0) put((i - 1) * n + j, 1);
          if (i < n - 1) put((i + 1) * n + j, 1);
          if (j > 0) put(me - 1, 1);
          if (j < n - 1) put(me + 1, 1);
          put(me, -8);
          if (i > 0 && j > 0) put((i - 1) * n + j - 1, 1);
          if (i < n - 1 && j < n - 1) put((i + 1) * n + j + 1, 1);
          if (i > 0 && j < n - 1) put((i - 1) * n + j + 1, 1);
          if (i < n - 1 && j > 0) put((i + 1) * n + j - 1, 1);
        }
        g->ptr.push_back((int)g->col.size());
      }
  } else if (type == "cube") {
    g->n = n * n * n;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        for (int k = 0; k < n; k++) {
          int me = (i * n + j) * n + k;
          put(me, -6);
          if (i > 0) put(((i - 1) * n + j) * n + k, 1);
          if (i < n - 1) put(((i + 1) * n + j) * n + k, 1);
          if (j > 0) put((i * n + j - 1) * n + k, 1);
          if (j < n - 1) put((i * n + j + 1) * n + k, 1);
          if (k > 0) put(me - 1, 1);
          if (k < n - 1) put(me + 1, 1);
          g->ptr.push_back((int)g->col.size());
        }
  } else {
    return fail(kEInval, "unknown graph type " + type);
  }
  return kOk;
}

int gen_laplacian(int nx, int ny, int nz, double diag, double off, Csr *g,
                  std::vector<int> *coords) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return fail(kEInval, "grid sizes must be positive");
  long n = (long)nx * ny * nz;
  if (n > 0x7fffffffL / 8) return fail(kERange, "grid too large for int32 indices");
  g->n = (int)n;
  g->ptr.assign(n + 1, 0);
  g->col.clear(); g->val.clear();
  g->col.reserve(n * 7); g->val.reserve(n * 7);
  if (coords) coords->resize(3 * n);
  const long sy = nx, sz = (long)nx * ny;
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        long i = z * sz + y * sy + x;
        auto put = [&](long c, double v) { g->col.push_back((int)c); g->val.push_back(v); };
        if (z > 0) put(i - sz, off);
        if (y > 0) put(i - sy, off);
        if (x > 0) put(i - 1, off);
        put(i, diag);
        if (x < nx - 1) put(i + 1, off);
        if (y < ny - 1) put(i + sy, off);
        if (z < nz - 1) put(i + sz, off);
        g->ptr[i + 1] = (int)g->col.size();
        if (coords) { (*coords)[3 * i] = x; (*coords)[3 * i + 1] = y; (*coords)[3 * i + 2] = z; }
      }
  return kOk;
}

void uniform_vector(uint64_t seed, long n, double *out) {
  uint64_t s = seed;
  for (long i = 0; i < n; i++) {
    s += 0x9E3779B97F4A7C15ULL;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
    out[i] = 2.0 * u - 1.0;
  }
}

}  // namespace mpkg

namespace mpkg {

namespace {
// splitmix64 -> standard normal by Box-Muller (one value per call).
struct Normal {
  uint64_t s;
  explicit Normal(uint64_t seed) : s(seed) {}
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ULL;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform01() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double operator()() {
    const double u1 = uniform01(), u2 = uniform01();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

// Assemble a symmetric operator from per-vertex neighbour offsets with a
// coefficient per undirected edge.
int assemble(long n, const std::vector<std::vector<std::pair<long, double>>> &nbr, double dominance, Csr *g) {
  g->n = (int)n;
  g->ptr.assign(n + 1, 0);
  g->col.clear();
  g->val.clear();
  for (long i = 0; i < n; i++) {
    std::vector<std::pair<long, double>> row = nbr[i];
    double d = 0.0;
    for (auto &e : row) d += std::fabs(e.second);
    row.emplace_back(i, (1.0 + dominance) * d);
    std::sort(row.begin(), row.end());
    for (auto &e : row) {
      g->col.push_back((int)e.first);
      g->val.push_back(e.first == i ? e.second : -std::fabs(e.second));
    }
    g->ptr[i + 1] = (int)g->col.size();
  }
  return kOk;
}
}  // namespace

int gen_diffusion_9pt(int nx, int ny, double sigma, double wx, double wy, double wdiag, double dominance,
                      uint64_t seed, Csr *g) {
  if (nx <= 0 || ny <= 0) return fail(kEInval, "grid sizes must be positive");
  const long n = (long)nx * ny;
  if (n * 9 > 0x7fffffffL) return fail(kERange, "grid too large for int32 indices");
  Normal rnd(seed);
  std::vector<std::vector<std::pair<long, double>>> nbr(n);
  // forward edges: +x, +y, +x+y, -x+y (each undirected edge once)
  const int dx[4] = {1, 0, 1, -1}, dy[4] = {0, 1, 1, 1};
  const double w[4] = {wx, wy, wdiag, wdiag};
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++)
      for (int d = 0; d < 4; d++) {
        const int x2 = x + dx[d], y2 = y + dy[d];
        if (x2 < 0 || x2 >= nx || y2 >= ny) continue;
        const double c = w[d] * std::exp(sigma * rnd());
        const long i = (long)y * nx + x, j = (long)y2 * nx + x2;
        nbr[i].emplace_back(j, c);
        nbr[j].emplace_back(i, c);
      }
  return assemble(n, nbr, dominance, g);
}

int gen_diffusion_7pt(int nx, int ny, int nz, double sigma, double dominance, uint64_t seed, Csr *g) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return fail(kEInval, "grid sizes must be positive");
  const long n = (long)nx * ny * nz;
  if (n * 7 > 0x7fffffffL) return fail(kERange, "grid too large for int32 indices");
  Normal rnd(seed);
  std::vector<std::vector<std::pair<long, double>>> nbr(n);
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        const long i = ((long)z * ny + y) * nx + x;
        if (x + 1 < nx) { const double c = std::exp(sigma * rnd()); nbr[i].emplace_back(i + 1, c); nbr[i + 1].emplace_back(i, c); }
        if (y + 1 < ny) { const double c = std::exp(sigma * rnd()); nbr[i].emplace_back(i + nx, c); nbr[i + nx].emplace_back(i, c); }
        if (z + 1 < nz) {
          const double c = std::exp(sigma * rnd());
          nbr[i].emplace_back(i + (long)nx * ny, c);
          nbr[i + (long)nx * ny].emplace_back(i, c);
        }
      }
  return assemble(n, nbr, dominance, g);
}

// Random banded operator: row i holds its diagonal plus m-1 distinct
// off-diagonal columns drawn uniformly from [i-bw, i+bw] (m uniform in
// [nmin, nmax], capped by the band), values N(0,1); the diagonal is
// N(0,1) + sum |off-diagonals| + 1 (diagonally dominant).  Columns
// ascending; seeded.
int gen_banded(long n, int bw, int nmin, int nmax, uint64_t seed, Csr *g) {
  if (n <= 0 || n > INT32_MAX / 2 || bw < 1 || nmin < 1 || nmax < nmin) return fail(kEInval, "bad banded parameters");
  Normal rng(seed);
  g->n = (int)n;
  g->ptr.assign(n + 1, 0);
  g->col.clear();
  g->val.clear();
  std::vector<long> pool;
  std::vector<std::pair<long, double>> row;
  for (long i = 0; i < n; i++) {
    const long lo = std::max(0L, i - bw), hi = std::min(n - 1, i + (long)bw);
    const long avail = hi - lo;  // off-diagonal candidates
    long m = nmin + (long)(rng.next() % (uint64_t)(nmax - nmin + 1));
    m = std::min(m - 1, avail);
    pool.clear();
    for (long j = lo; j <= hi; j++)
      if (j != i) pool.push_back(j);
    for (long k = 0; k < m; k++) {  // partial Fisher-Yates
      const long r = k + (long)(rng.next() % (uint64_t)(pool.size() - k));
      std::swap(pool[k], pool[r]);
    }
    row.clear();
    double off = 0.0;
    for (long k = 0; k < m; k++) {
      const double v = rng();
      off += std::fabs(v);
      row.emplace_back(pool[k], v);
    }
    row.emplace_back(i, rng() + off + 1.0);
    std::sort(row.begin(), row.end());
    for (auto &e : row) {
      g->col.push_back((int)e.first);
      g->val.push_back(e.second);
    }
    g->ptr[i + 1] = (int)g->col.size();
  }
  return kOk;
}

}  // namespace mpkg
