// Host prep: levels, edge weights, skirts, task lists and the device plans
// (PA1 tiles and the level pipeline).  The level and skirt computations are
// bounded breadth-first searches that give the same results as the
// reference's whole-graph min-plus sweeps (mpk2/lib.c:164-219, 330-412,
// 584-615) at a fraction of the cost.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "host.h"

namespace mpkg {

namespace {

// Transpose adjacency: tr.col[tr.ptr[j]..tr.ptr[j+1]) = rows i whose row
// lists column j.  Information in the min-plus sweeps flows from column j
// to row i, so the searches below walk these reversed arcs.
struct Adj {
  std::vector<long> ptr;
  std::vector<int> col;
};

void transpose(const Csr &g, Adj *tr) {
  const int n = g.n;
  tr->ptr.assign(n + 1, 0);
  for (long j = 0; j < g.nnz(); j++) tr->ptr[g.col[j] + 1]++;
  for (int i = 0; i < n; i++) tr->ptr[i + 1] += tr->ptr[i];
  tr->col.resize(g.nnz());
  std::vector<long> fill(tr->ptr.begin(), tr->ptr.end() - 1);
  for (int i = 0; i < n; i++)
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) tr->col[fill[g.col[j]]++] = i;
}

}  // namespace

// comp_level (mpk2/lib.c:330-371) and update_level (mpk2/lib.c:373-412).
// For a vertex i of part p the reference's fixed point is
//   level[i] = min(BIG, min over arc paths i -> v1 -> ... -> vm, with
//              v1..v(m-1) in p and vm outside p, of init(vm) + m)
// where init = -1 (first phase) or the previous level, and BIG = n + 1
// (first phase) or max(previous level) + n + 1.  That is a multi-source
// shortest path with unit arcs and per-source offsets, solved here with
// a two-queue merge (seeds sorted by value, FIFO for relaxations).
int comp_levels(const Csr &g, const std::vector<int> &part, int npart,
                const std::vector<int> *level_org, std::vector<int> *level) {
  const int n = g.n;
  (void)npart;
  if ((int)part.size() != n) return fail(kEInval, "partition size != n");
  if (level_org && (int)level_org->size() != n) return fail(kEInval, "level size != n");
  long big;
  if (level_org) {
    int mx = (*level_org)[0];
    for (int i = 1; i < n; i++) mx = std::max(mx, (*level_org)[i]);
    big = (long)mx + n + 1;
  } else {
    big = (long)n + 1;
  }
  std::vector<long> dist(n, big);
  // seeds: one arc into another part
  for (int i = 0; i < n; i++)
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) {
      int c = g.col[j];
      if (part[c] != part[i]) {
        long v = (level_org ? (long)(*level_org)[c] : -1L) + 1;
        if (v < dist[i]) dist[i] = v;
      }
    }
  std::vector<int> seeds;
  for (int i = 0; i < n; i++) if (dist[i] < big) seeds.push_back(i);
  std::stable_sort(seeds.begin(), seeds.end(), [&](int a, int b) { return dist[a] < dist[b]; });
  Adj tr;
  transpose(g, &tr);
  std::vector<int> fifo;
  fifo.reserve(n);
  std::vector<char> done(n, 0);
  size_t si = 0, fh = 0;
  while (si < seeds.size() || fh < fifo.size()) {
    int v;
    if (fh < fifo.size() && (si >= seeds.size() || dist[fifo[fh]] <= dist[seeds[si]])) v = fifo[fh++];
    else v = seeds[si++];
    if (done[v]) continue;
    done[v] = 1;
    long dv = dist[v] + 1;
    for (long t = tr.ptr[v]; t < tr.ptr[v + 1]; t++) {
      int i = tr.col[t];
      if (part[i] == part[v] && !done[i] && dv < dist[i]) {
        dist[i] = dv;
        fifo.push_back(i);
      }
    }
  }
  level->resize(n);
  for (int i = 0; i < n; i++) (*level)[i] = (int)dist[i];
  return kOk;
}

// level2wcrs (mpk2/lib.c:504-537).
void level_weights(const Csr &g, const std::vector<int> &level, std::vector<int> *wv,
                   std::vector<int> *we) {
  const int n = g.n;
  int mx = level[0], mn = level[0];
  for (int i = 1; i < n; i++) { mx = std::max(mx, level[i]); mn = std::min(mn, level[i]); }
  wv->resize(n);
  we->resize(g.nnz());
  for (int i = 0; i < n; i++) {
    (*wv)[i] = mx + 1 - level[i];
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) {
      double w = level[i] + level[g.col[j]] - 2 * mn;
      w = 1e+6 / (w + 1);
      (*we)[j] = (w < 1.0) ? 1 : (int)w;
    }
  }
}

// write_wcrs (mpk2/lib.c:482-502): header "n ne 011", then per vertex
// "1 " and (neighbour, weight) pairs.
int write_weighted_graph(const std::string &path, const Csr &g, const std::vector<int> &we) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return fail(kEIo, "cannot open " + path);
  std::fprintf(f, "%d %d 011\n", g.n, g.ptr[g.n] / 2);
  for (int i = 0; i < g.n; i++) {
    std::fprintf(f, "1 ");
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) std::fprintf(f, "%d %d ", g.col[j] + 1, we[j]);
    std::fprintf(f, "\n");
  }
  std::fclose(f);
  return kOk;
}

int write_levels(const std::string &path, const std::vector<int> &level) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return fail(kEIo, "cannot open " + path);
  for (int v : level) std::fprintf(f, "%d\n", v);
  std::fclose(f);
  return kOk;
}

int read_levels(const std::string &path, int n, std::vector<int> *level) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) return fail(kEIo, "cannot open " + path);
  level->resize(n);
  for (int i = 0; i < n; i++)
    if (std::fscanf(f, "%d", &(*level)[i]) != 1) {
      std::fclose(f);
      return fail(kEFormat, path + ": fewer levels than vertices");
    }
  std::fclose(f);
  return kOk;
}

namespace {
// Vertices at distance <= maxd from part p (breadth first over reversed
// arcs, i.e. dist[i] = 1 + min over columns j of row i of dist[j]), in BFS
// order with their distances.  `mark` must be all -1 on entry and is
// restored on exit.
void part_ball(const Adj &tr, const std::vector<int> &members, int maxd, std::vector<int> &mark,
               std::vector<int> *verts, std::vector<int> *dists) {
  verts->clear();
  dists->clear();
  for (int v : members) {
    mark[v] = 0;
    verts->push_back(v);
    dists->push_back(0);
  }
  for (size_t h = 0; h < verts->size(); h++) {
    int v = (*verts)[h];
    int d = (*dists)[h];
    if (d >= maxd) continue;
    for (long t = tr.ptr[v]; t < tr.ptr[v + 1]; t++) {
      int i = tr.col[t];
      if (mark[i] < 0) {
        mark[i] = d + 1;
        verts->push_back(i);
        dists->push_back(d + 1);
      }
    }
  }
  for (int v : *verts) mark[v] = -1;
}

std::vector<std::vector<int>> members_of(const std::vector<int> &part, int npart) {
  std::vector<std::vector<int>> m(npart);
  for (int i = 0; i < (int)part.size(); i++) m[part[i]].push_back(i);
  return m;
}
}  // namespace

// comp_skirt + the selection of write_skirt (mpk2/lib.c:584-654).
int comp_skirts(const Csr &g, const std::vector<int> &part, int npart,
                const std::vector<int> *lev, int level, std::vector<PartSkirt> *sk) {
  const int n = g.n;
  if ((int)part.size() != n) return fail(kEInval, "partition size != n");
  if (level <= 0) return fail(kEInval, "level must be positive");
  for (int p : part) if (p < 0 || p >= npart) return fail(kERange, "part id out of range");
  Adj tr;
  transpose(g, &tr);
  auto mem = members_of(part, npart);
  std::vector<int> mark(n, -1), verts, dists;
  sk->assign(npart, PartSkirt());
  for (int p = 0; p < npart; p++) {
    part_ball(tr, mem[p], level - 1, mark, &verts, &dists);
    std::vector<std::pair<int, int>> keep;
    keep.reserve(verts.size());
    for (size_t t = 0; t < verts.size(); t++) {
      int j = verts[t], d = dists[t];
      bool k = lev ? ((*lev)[j] < level - d) : (d < level);
      if (k) keep.emplace_back(j, d);
    }
    std::sort(keep.begin(), keep.end());
    PartSkirt &s = (*sk)[p];
    s.vert.resize(keep.size());
    s.dist.resize(keep.size());
    for (size_t t = 0; t < keep.size(); t++) { s.vert[t] = keep[t].first; s.dist[t] = keep[t].second; }
  }
  return kOk;
}

int write_skirt_file(const std::string &path, int n, int level, const std::vector<PartSkirt> &sk) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return fail(kEIo, "cannot open " + path);
  std::fprintf(f, "skirt %d nodes, %d parts\n", n, (int)sk.size());
  for (size_t p = 0; p < sk.size(); p++) {
    std::fprintf(f, "partition %d\n", (int)p);
    for (size_t t = 0; t < sk[p].vert.size(); t++)
      std::fprintf(f, "%d %d\n", sk[p].vert[t], level - sk[p].dist[t]);
  }
  std::fclose(f);
  return kOk;
}

// read_skirt (mpk2/lib.c:656-707): entries "k m" with 0 <= k < n and
// 0 <= m <= level; the stored skirt value is level - m.
int read_skirt_file(const std::string &path, int n, int npart, int level,
                    std::vector<PartSkirt> *sk) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) return fail(kEIo, "cannot open " + path);
  char line[256];
  int a = -1, b = -1;
  if (!std::fgets(line, sizeof line, f) ||
      std::sscanf(line, "skirt %d nodes, %d parts", &a, &b) != 2 || a != n || b != npart) {
    std::fclose(f);
    return fail(kEFormat, path + ": skirt header does not match n/npart");
  }
  sk->assign(npart, PartSkirt());
  int p = -1;
  std::vector<int> slot(n, -1);
  while (std::fgets(line, sizeof line, f)) {
    if (line[0] == 'p') {
      int q = -1;
      if (std::sscanf(line, "partition %d", &q) != 1 || q != p + 1 || q >= npart) {
        std::fclose(f);
        return fail(kEFormat, path + ": partitions out of order");
      }
      if (p >= 0) for (int v : (*sk)[p].vert) slot[v] = -1;
      p = q;
      continue;
    }
    int k, m;
    if (std::sscanf(line, "%d %d", &k, &m) != 2) continue;
    if (p < 0 || k < 0 || k >= n || m < 0 || m > level) {
      std::fclose(f);
      return fail(kERange, path + ": skirt entry out of range");
    }
    PartSkirt &s = (*sk)[p];
    if (slot[k] >= 0) {
      s.dist[slot[k]] = level - m;  // a repeated vertex overwrites, as the reference
    } else {
      slot[k] = (int)s.vert.size();
      s.vert.push_back(k);
      s.dist.push_back(level - m);
    }
  }
  std::fclose(f);
  if (p != npart - 1) return fail(kEFormat, path + ": missing partitions");
  for (auto &s : *sk) {  // keep vertex-ascending order
    std::vector<int> ord(s.vert.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](int x, int y) { return s.vert[x] < s.vert[y]; });
    PartSkirt t;
    for (int o : ord) { t.vert.push_back(s.vert[o]); t.dist.push_back(s.dist[o]); }
    s = t;
  }
  return kOk;
}

// prep_mpk (mpk2/mpkprep.c:7-258).  Dependency tags follow the reference:
// a computed (level, vertex) carries part*100 + phase, level 0 carries
// part0*100; `check` reports the reference's structure errors.
int build_tasks(const Csr &g, int npart, int nlevel, int nphase,
                const std::vector<std::vector<int>> &parts,
                const std::vector<std::vector<int>> &levels,
                const std::vector<PartSkirt> &sk, bool check, TaskLists *tl) {
  const int n = g.n;
  if (npart <= 0 || nlevel <= 0 || nphase < 0) return fail(kEInval, "bad npart/nlevel/nphase");
  if ((int)parts.size() < std::max(nphase, 1) || (int)levels.size() < nphase || (int)sk.size() != npart)
    return fail(kEInval, "missing partitions, levels or skirts");
  // level and skirt sanity (mpkprep.c:21-87)
  for (int ph = 0; ph < nphase; ph++)
    for (int i = 0; i < n; i++) {
      if (ph == 0 && levels[0][i] < 0) return fail(kEStruct, "level error: negative level");
      if (ph > 0 && levels[ph - 1][i] > levels[ph][i]) return fail(kEStruct, "level error: level decreases");
    }
  for (int p = 0; p < npart; p++)
    for (size_t t = 0; t < sk[p].vert.size(); t++) {
      int i = sk[p].vert[t], s = sk[p].dist[t];
      if (s < 0) continue;
      if (nphase == 0 && nlevel - s < 0) return fail(kEStruct, "skirt level error");
      if (nphase > 0 && levels[nphase - 1][i] > nlevel - s) return fail(kEStruct, "skirt level error");
    }
  tl->n = n; tl->npart = npart; tl->nlevel = nlevel; tl->nphase = nphase;
  tl->off.assign((long)(nphase + 1) * npart + 1, 0);
  tl->idx.clear();

  // tags: -1 never computed, -2 computed by a skirt task, else part*100+phase
  std::vector<int> tag;
  if (check) {
    tag.assign((size_t)n * (nlevel + 1), -1);
    for (int i = 0; i < n; i++) tag[i] = parts[0][i] * 100;
  }
  std::vector<int> zero(n, 0);
  const int *prevl = zero.data();
  int prevlmin = 0;
  long errors = 0;
  for (int ph = 0; ph < nphase; ph++) {
    const std::vector<int> &pl = parts[ph];
    const std::vector<int> &ll = levels[ph];
    int lmin = ll[0], lmax = ll[0];
    for (int i = 1; i < n; i++) { lmin = std::min(lmin, ll[i]); lmax = std::max(lmax, ll[i]); }
    if (lmax > nlevel) lmax = nlevel;
    // count per (part, level) to lay out level-major lists
    int nl = std::max(lmax - prevlmin, 0);
    std::vector<long> cnt((size_t)npart * (nl + 1), 0);
    for (int i = 0; i < n; i++) {
      int lo = std::max(prevl[i] + 1, prevlmin + 1), hi = std::min(ll[i], lmax);
      for (int l = lo; l <= hi; l++) cnt[(size_t)pl[i] * (nl + 1) + (l - prevlmin - 1)]++;
    }
    long base = (long)tl->idx.size();
    std::vector<long> pos((size_t)npart * (nl + 1));
    for (int p = 0; p < npart; p++) {
      tl->off[(long)ph * npart + p] = base;
      for (int l = 0; l <= nl; l++) {
        pos[(size_t)p * (nl + 1) + l] = base;
        base += cnt[(size_t)p * (nl + 1) + l];
      }
    }
    tl->idx.resize(base);
    for (int i = 0; i < n; i++) {
      int lo = std::max(prevl[i] + 1, prevlmin + 1), hi = std::min(ll[i], lmax);
      for (int l = lo; l <= hi; l++) tl->idx[pos[(size_t)pl[i] * (nl + 1) + (l - prevlmin - 1)]++] = (long)l * n + i;
    }
    if (check) {
      for (int l = prevlmin + 1; l <= lmax; l++)
        for (int i = 0; i < n; i++)
          if (prevl[i] < l && l <= ll[i]) {
            if (tag[(size_t)l * n + i] >= 0) errors++;
            for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) {
              int k = g.col[j];
              int t = tag[(size_t)(l - 1) * n + k];
              if (t == -1 || (pl[i] != pl[k] && t >= 0 && t % 100 == ph)) errors++;
            }
            tag[(size_t)l * n + i] = pl[i] * 100 + ph;
          }
    }
    prevl = ll.data();
    prevlmin = lmin;
  }
  if (errors) return fail(kEStruct, "structure error in phase task lists");
  // skirt tasks (mpkprep.c:185-233): per part, levels above prevlmin
  for (int p = 0; p < npart; p++) {
    long t = (long)nphase * npart + p;
    tl->off[t] = (long)tl->idx.size();
    const PartSkirt &s = sk[p];
    for (int l = prevlmin + 1; l <= nlevel; l++)
      for (size_t q = 0; q < s.vert.size(); q++) {
        int i = s.vert[q], d = s.dist[q];
        if (prevl[i] < l && d >= 0 && l <= nlevel - d) tl->idx.push_back((long)l * n + i);
      }
    if (check) {
      for (long q = tl->off[t]; q < (long)tl->idx.size(); q++) {
        long e = tl->idx[q];
        int l = (int)(e / n), i = (int)(e - (long)l * n);
        int tg = tag[(size_t)l * n + i];
        if (tg > 0) errors++;  // the reference flags only tags > 0.0
        for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++)
          if (tag[(size_t)(l - 1) * n + g.col[j]] == -1) errors++;
        tag[(size_t)l * n + i] = parts[0][i] * 100 + nphase;
      }
      for (long q = tl->off[t]; q < (long)tl->idx.size(); q++) tag[tl->idx[q]] = -2;
    }
  }
  tl->off[(long)(nphase + 1) * npart] = (long)tl->idx.size();
  if (check) {
    for (int i = 0; i < n; i++) if (tag[(size_t)nlevel * n + i] == -1) errors++;
    if (errors) return fail(kEStruct, "structure error in skirt task lists");
  }
  return kOk;
}

// PA1 tiles.
// Launch order of the parts: breadth-first over the part graph (parts
// adjacent when an entry of one reads a vertex of the other), from a part
// of least degree, neighbours in ascending id; unconnected parts start new
// searches.  Consecutive tiles are then neighbours, so the halo rows two
// tiles share are read while the first tile's are still in L2.  The order
// only schedules work: every tile computes the same rows whatever it is.
void part_order(const Csr &g, const std::vector<int> &part, int npart, std::vector<int> *order) {
  std::vector<std::pair<int, int>> pairs;
  for (int i = 0; i < g.n; i++)
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) {
      const int a = part[i], b = part[g.col[j]];
      if (a != b) pairs.emplace_back(a, b);
    }
  std::sort(pairs.begin(), pairs.end());
  pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
  std::vector<int> aptr(npart + 1, 0), adj(pairs.size());
  for (auto &e : pairs) aptr[e.first + 1]++;
  for (int p = 0; p < npart; p++) aptr[p + 1] += aptr[p];
  for (size_t k = 0; k < pairs.size(); k++) adj[k] = pairs[k].second;  // sorted by (first, second)
  std::vector<int> byd(npart);
  std::iota(byd.begin(), byd.end(), 0);
  std::stable_sort(byd.begin(), byd.end(),
                   [&](int a, int b) { return aptr[a + 1] - aptr[a] < aptr[b + 1] - aptr[b]; });
  std::vector<char> seen(npart, 0);
  order->clear();
  order->reserve(npart);
  for (int s0 : byd) {
    if (seen[s0]) continue;
    size_t head = order->size();
    order->push_back(s0);
    seen[s0] = 1;
    while (head < order->size()) {
      const int p = (*order)[head++];
      for (int k = aptr[p]; k < aptr[p + 1]; k++)
        if (!seen[adj[k]]) {
          seen[adj[k]] = 1;
          order->push_back(adj[k]);
        }
    }
  }
}

int build_tile_plan(const Csr &g, const std::vector<int> &part, int npart, int nlevel,
                    TilePlan *tp) {
  const int n = g.n;
  if ((int)part.size() != n) return fail(kEInval, "partition size != n");
  for (int p : part) if (p < 0 || p >= npart) return fail(kERange, "part id out of range");
  Adj tr;
  transpose(g, &tr);
  auto mem = members_of(part, npart);
  tp->n = n; tp->npart = npart; tp->nlevel = nlevel;
  part_order(g, part, npart, &tp->order);
  tp->slot_off.assign(npart + 1, 0);
  tp->shell.assign((size_t)npart * (nlevel + 1), 0);
  tp->slot_vert.clear();
  tp->slice_off.assign(npart + 1, 0);
  tp->ell_off.assign(1, 0);
  tp->ell_col.clear();
  tp->ell_width.clear();
  tp->max_slots = 0;
  tp->total_rows = 0;
  std::vector<int> mark(n, -1), verts, dists, loc(n, -1);
  for (int p = 0; p < npart; p++) {
    if (mem[p].empty()) return fail(kEInval, "empty part " + std::to_string(p));
    part_ball(tr, mem[p], nlevel, mark, &verts, &dists);
    std::vector<std::pair<int, int>> sd(verts.size());
    for (size_t t = 0; t < verts.size(); t++) sd[t] = {dists[t], verts[t]};
    std::sort(sd.begin(), sd.end());
    if (sd.size() > 0xFFFE) return fail(kERange, "tile of part " + std::to_string(p) + " exceeds 65534 slots");
    int *shell = &tp->shell[(size_t)p * (nlevel + 1)];
    for (auto &e : sd) for (int d = e.first; d <= nlevel; d++) shell[d]++;
    tp->slot_off[p] = (long)tp->slot_vert.size();
    for (size_t s = 0; s < sd.size(); s++) {
      loc[sd[s].second] = (int)s;
      tp->slot_vert.push_back(sd[s].second);
    }
    tp->max_slots = std::max(tp->max_slots, (int)sd.size());
    for (int l = 1; l <= nlevel; l++) tp->total_rows += shell[nlevel - l];
    // sliced ELL over the rows computed at level 1 (distance <= nlevel-1)
    int nrows = shell[nlevel - 1];
    tp->slice_off[p] = (long)tp->ell_width.size();
    for (int r0 = 0; r0 < nrows; r0 += 32) {
      int r1 = std::min(nrows, r0 + 32);
      int w = 0;
      for (int r = r0; r < r1; r++) {
        int v = sd[r].second;
        w = std::max(w, g.ptr[v + 1] - g.ptr[v]);
      }
      if (w > 255) return fail(kERange, "row degree above 255 is not supported by tiles");
      long base = tp->ell_off.back();
      tp->ell_col.resize(base + 32L * w, 0xFFFF);
      for (int r = r0; r < r1; r++) {
        int v = sd[r].second;
        for (int j = g.ptr[v], t = 0; j < g.ptr[v + 1]; j++, t++) {
          int c = loc[g.col[j]];
          if (c < 0) return fail(kEStruct, "tile column outside the halo");
          tp->ell_col[base + (long)t * 32 + (r - r0)] = (uint16_t)c;
        }
      }
      tp->ell_width.push_back((uint8_t)w);
      tp->ell_off.push_back(base + 32L * w);
    }
    for (auto &e : sd) loc[e.second] = -1;
  }
  tp->slot_off[npart] = (long)tp->slot_vert.size();
  tp->slice_off[npart] = (long)tp->ell_width.size();
  return kOk;
}

int build_pipe_plan(const Csr &g, int nlevel, int chunk, PipePlan *pp) {
  const int n = g.n;
  if (chunk <= 0 || chunk % 32) return fail(kEInval, "chunk must be a positive multiple of 32");
  pp->n = n; pp->nlevel = nlevel; pp->chunk = chunk;
  pp->nchunk = (n + chunk - 1) / chunk;
  pp->dep_lo.assign(pp->nchunk, 0);
  pp->dep_hi.assign(pp->nchunk, 0);
  pp->reach = 0;
  for (int c = 0; c < pp->nchunk; c++) {
    int lo = c, hi = c;
    int r1 = std::min(n, (c + 1) * chunk);
    for (int i = c * chunk; i < r1; i++)
      for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) {
        int cc = g.col[j] / chunk;
        lo = std::min(lo, cc);
        hi = std::max(hi, cc);
      }
    pp->dep_lo[c] = lo;
    pp->dep_hi[c] = hi;
    pp->reach = std::max(pp->reach, std::max(c - lo, hi - c));
  }
  return kOk;
}

}  // namespace mpkg
