// MPI-2 rank buffers: file format and consistency checks.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <vector>

#include "host.h"

namespace mpkg {

namespace {
template <typename T>
bool rd(FILE *f, T *p, size_t count) {
  return count == 0 || std::fread(p, sizeof(T), count, f) == count;
}
template <typename T>
bool wr(FILE *f, const T *p, size_t count) {
  return count == 0 || std::fwrite(p, sizeof(T), count, f) == count;
}
}  // namespace

// Layout of write_buffers (mpk2/buffers.c:588-631): nine int scalars
// (n, npart, nlevel, nphase, rank, buf_count, buf_scount, mptr_count,
// mcol_count); recvcounts, sendcounts, rdispls, sdispls (npart*(nphase+1)
// ints each); rcount, mcount, scount, rbuf_offsets, mbuf_offsets,
// sbuf_offsets, mptr_offsets, mcol_offsets (nphase+1 ints each);
// idx_buf, idx_sbuf, mptr_buf, mcol_buf (longs); optionally mval_buf.
int read_rank_buffers(const std::string &path, RankBuffers *b) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(kEIo, "cannot open " + path);
  int h[9];
  bool ok = rd(f, h, 9);
  if (ok) {
    b->n = h[0]; b->npart = h[1]; b->nlevel = h[2]; b->nphase = h[3]; b->rank = h[4];
    b->buf_count = h[5]; b->buf_scount = h[6]; b->mptr_count = h[7]; b->mcol_count = h[8];
    ok = b->n > 0 && b->npart > 0 && b->nlevel > 0 && b->nphase >= 0 && b->rank >= 0 && b->rank < b->npart &&
         b->buf_count >= 0 && b->buf_scount >= 0 && b->mptr_count >= 0 && b->mcol_count >= 0 &&
         (long)b->npart * (b->nphase + 1) < (1L << 28);
  }
  if (!ok) { std::fclose(f); return fail(kEFormat, path + ": bad buffer header"); }
  const size_t np = (size_t)b->npart * (b->nphase + 1), ph = (size_t)b->nphase + 1;
  for (std::vector<int> *v : {&b->recvcounts, &b->sendcounts, &b->rdispls, &b->sdispls}) {
    v->resize(np);
    ok = ok && rd(f, v->data(), np);
  }
  for (std::vector<int> *v : {&b->rcount, &b->mcount, &b->scount, &b->rbuf_offsets, &b->mbuf_offsets,
                              &b->sbuf_offsets, &b->mptr_offsets, &b->mcol_offsets}) {
    v->resize(ph);
    ok = ok && rd(f, v->data(), ph);
  }
  b->idx_buf.resize(b->buf_count);
  b->idx_sbuf.resize(b->buf_scount);
  b->mptr_buf.resize(b->mptr_count);
  b->mcol_buf.resize(b->mcol_count);
  ok = ok && rd(f, b->idx_buf.data(), b->idx_buf.size()) && rd(f, b->idx_sbuf.data(), b->idx_sbuf.size()) &&
       rd(f, b->mptr_buf.data(), b->mptr_buf.size()) && rd(f, b->mcol_buf.data(), b->mcol_buf.size());
  if (!ok) { std::fclose(f); return fail(kEFormat, path + ": truncated buffer file"); }
  b->mval_buf.resize(b->mcol_count);
  if (!rd(f, b->mval_buf.data(), b->mval_buf.size())) b->mval_buf.clear();  // as read_buffers
  std::fclose(f);
  return kOk;
}

int write_rank_buffers(const std::string &path, const RankBuffers &b) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return fail(kEIo, "cannot open " + path);
  const int h[9] = {b.n, b.npart, b.nlevel, b.nphase, b.rank, b.buf_count, b.buf_scount, b.mptr_count,
                    b.mcol_count};
  bool ok = wr(f, h, 9);
  for (const std::vector<int> *v : {&b.recvcounts, &b.sendcounts, &b.rdispls, &b.sdispls, &b.rcount, &b.mcount,
                                    &b.scount, &b.rbuf_offsets, &b.mbuf_offsets, &b.sbuf_offsets, &b.mptr_offsets,
                                    &b.mcol_offsets})
    ok = ok && wr(f, v->data(), v->size());
  ok = ok && wr(f, b.idx_buf.data(), b.idx_buf.size()) && wr(f, b.idx_sbuf.data(), b.idx_sbuf.size()) &&
       wr(f, b.mptr_buf.data(), b.mptr_buf.size()) && wr(f, b.mcol_buf.data(), b.mcol_buf.size());
  if (!b.mval_buf.empty()) ok = ok && wr(f, b.mval_buf.data(), b.mval_buf.size());
  std::fclose(f);
  return ok ? kOk : fail(kEIo, "short write on " + path);
}

int check_rank_buffers(const std::vector<RankBuffers> &bufs) {
  if (bufs.empty()) return fail(kEInval, "no rank buffers");
  const RankBuffers &b0 = bufs[0];
  const int P = (int)bufs.size();
  if (b0.npart != P) return fail(kEInval, "number of rank buffers != npart");
  const long nvv = (long)b0.n * (b0.nlevel + 1);
  for (int r = 0; r < P; r++) {
    const RankBuffers &b = bufs[r];
    if (b.rank != r || b.n != b0.n || b.npart != P || b.nlevel != b0.nlevel || b.nphase != b0.nphase)
      return fail(kEFormat, "rank buffers disagree on n/npart/nlevel/nphase or rank order");
    if (b.mval_buf.empty()) return fail(kEFormat, "rank buffers hold no matrix values");
    for (int ph = 0; ph <= b.nphase; ph++) {
      if (b.rbuf_offsets[ph] < 0 || b.rbuf_offsets[ph] + (long)b.rcount[ph] > b.buf_count ||
          b.mbuf_offsets[ph] < 0 || b.mbuf_offsets[ph] + (long)b.mcount[ph] > b.buf_count ||
          b.sbuf_offsets[ph] < 0 || b.sbuf_offsets[ph] + (long)b.scount[ph] > b.buf_scount ||
          b.mptr_offsets[ph] < 0 || b.mptr_offsets[ph] + (long)b.mcount[ph] + 1 > b.mptr_count ||
          b.mcol_offsets[ph] < 0)
        return fail(kERange, "rank buffer offsets out of range");
      const long *mptr = b.mptr_buf.data() + b.mptr_offsets[ph];
      for (int mi = 0; mi < b.mcount[ph]; mi++)
        if (mptr[mi] > mptr[mi + 1] || b.mcol_offsets[ph] + mptr[mi + 1] > b.mcol_count)
          return fail(kERange, "rank buffer mptr out of range");
      for (int src = 0; src < P; src++) {
        const long k = (long)P * ph + src;
        if (bufs[src].sendcounts[(long)P * ph + r] != b.recvcounts[k])
          return fail(kEFormat, "send and receive counts do not match");
        if (b.rdispls[k] < 0 || b.rdispls[k] + (long)b.recvcounts[k] > b.rcount[ph])
          return fail(kERange, "receive displacement out of range");
        if (b.sdispls[k] < 0 || b.sdispls[k] + (long)b.sendcounts[k] > b.scount[ph])
          return fail(kERange, "send displacement out of range");
      }
    }
    for (long i : b.idx_buf)
      if (i < 0 || i >= nvv) return fail(kERange, "idx_buf entry out of range");
    for (long i : b.idx_sbuf)
      if (i < 0 || i >= b.buf_count) return fail(kERange, "idx_sbuf entry out of range");
    for (long i : b.mcol_buf)
      if (i < 0 || i >= b.buf_count) return fail(kERange, "mcol entry out of range");
    for (int i = 0; i < b.rcount[0]; i++)
      if (b.idx_buf[b.rbuf_offsets[0] + i] >= b.n) return fail(kEFormat, "phase-0 receive entry is not level 0");
  }
  return kOk;
}

}  // namespace mpkg

namespace mpkg {

// Linear assignment by the Jonker-Volgenant shortest augmenting path
// algorithm (R. Jonker, A. Volgenant, Computing 38 (1987) 325-340) on the
// cost max(sums) - sums: rows are old parts, columns new labels, and the
// optimum keeps the most communication on one rank.  Optimal assignments
// are often not unique (zero blocks), so the steps follow the published
// procedure in order -- column reduction scanning columns from the last,
// reduction transfer, two passes of augmenting row reduction, then
// shortest-path augmentation of the remaining free rows -- with the same
// strict/non-strict comparisons, which is what the reference's lapjv
// (mpk2/lapjv.c:366-390, pdmpk/lapjv.c) implements; ties then resolve
// identically.
void assign_max_trace(const std::vector<long> &sums, int np, std::vector<int> *perm) {
  perm->assign(np, 0);
  if (np <= 1) return;
  long mx = sums[0];
  for (long s : sums) mx = std::max(mx, s);
  const int n = np;
  std::vector<long> c((size_t)n * n);
  for (size_t k = 0; k < c.size(); k++) c[k] = mx - sums[k];
  auto C = [&](int i, int j) { return c[(size_t)i * n + j]; };
  const int kFree = -1;
  std::vector<int> x(n, kFree), y(n, kFree);  // x[row] = column, y[column] = row
  std::vector<long> v(n, 0);                   // column duals
  std::vector<int> cols(n);                    // column scan order of the augmentation
  std::vector<char> multi(n, 0);               // row picked by more than one column
  // column reduction
  for (int j = n - 1; j >= 0; j--) {
    cols[j] = j;
    long h = C(0, j);
    int imin = 0;
    for (int i = 1; i < n; i++)
      if (C(i, j) < h) { h = C(i, j); imin = i; }
    v[j] = h;
    if (x[imin] == kFree && !multi[imin]) {
      x[imin] = j;
      y[j] = imin;
    } else {
      multi[imin] = 1;
      y[j] = kFree;
    }
  }
  // reduction transfer; rows never picked are free
  std::vector<int> fr;
  for (int i = 0; i < n; i++) {
    if (x[i] == kFree) {
      fr.push_back(i);
    } else if (!multi[i]) {
      const int j1 = x[i];
      long mn = LONG_MAX;
      for (int j = 0; j < n; j++)
        if (j != j1) mn = std::min(mn, C(i, j) - v[j]);
      v[j1] -= mn;
    }
  }
  // augmenting row reduction, twice; the list of free rows is rewritten
  // in place while it is consumed
  for (int pass = 0; pass < 2; pass++) {
    const int f0 = (int)fr.size();
    int k = 0, f = 0;
    while (k < f0) {
      const int i = fr[k++];
      long u1 = C(i, 0) - v[0], u2 = LONG_MAX;
      int j1 = 0, j2 = 0;
      for (int j = 1; j < n; j++) {
        const long h = C(i, j) - v[j];
        if (h < u2) {
          if (h >= u1) {
            u2 = h;
            j2 = j;
          } else {
            u2 = u1;
            u1 = h;
            j2 = j1;
            j1 = j;
          }
        }
      }
      int i1 = y[j1];
      if (u1 < u2) {
        v[j1] = v[j1] - u2 + u1;
      } else if (i1 != kFree) {
        j1 = j2;
        i1 = y[j1];
      }
      if (i1 != kFree) {
        if (u1 < u2) fr[--k] = i1;
        else fr[f++] = i1;
      }
      x[i] = j1;
      y[j1] = i;
    }
    fr.resize(f);
  }
  // augmentation: Dijkstra-like shortest path from every remaining free row
  std::vector<long> d(n);
  std::vector<int> pred(n);
  for (int i1 : fr) {
    for (int j = 0; j < n; j++) {
      d[j] = C(i1, j) - v[j];
      pred[j] = i1;
    }
    int low = 0, up = 0, last = 0, jend = -1;
    long mn = 0;
    while (jend < 0) {
      if (up == low) {  // next set of columns at minimum distance
        last = low;
        mn = d[cols[up++]];
        for (int k = up; k < n; k++) {
          const int j = cols[k];
          const long h = d[j];
          if (h <= mn) {
            if (h < mn) {
              up = low;
              mn = h;
            }
            cols[k] = cols[up];
            cols[up++] = j;
          }
        }
        for (int h = low; h < up && jend < 0; h++)
          if (y[cols[h]] == kFree) jend = cols[h];
        if (jend >= 0) break;
      }
      // scan the row matched to the next ready column
      const int j1 = cols[low++];
      const int i = y[j1];
      const long u1 = C(i, j1) - v[j1] - mn;
      for (int k = up; k < n; k++) {
        const int j = cols[k];
        const long h = C(i, j) - v[j] - u1;
        if (h < d[j]) {
          d[j] = h;
          pred[j] = i;
          if (h == mn) {
            if (y[j] == kFree) {
              jend = j;
              break;
            }
            cols[k] = cols[up];
            cols[up++] = j;
          }
        }
      }
    }
    for (int k = 0; k < last; k++) {
      const int j = cols[k];
      v[j] += d[j] - mn;
    }
    int j = jend, i;
    do {
      i = pred[j];
      y[j] = i;
      const int k = j;
      j = x[i];
      x[i] = k;
    } while (i != i1);
  }
  for (int j = 0; j < n; j++) (*perm)[j] = y[j];
}

namespace {
struct Triple {
  int src, tgt;
  long v;
};
bool by_tgt(const Triple &a, const Triple &b) {
  return a.tgt != b.tgt ? a.tgt < b.tgt : a.src != b.src ? a.src < b.src : a.v < b.v;
}
void unique_triples(std::vector<Triple> *t) {
  std::sort(t->begin(), t->end(), by_tgt);
  t->erase(std::unique(t->begin(), t->end(),
                       [](const Triple &a, const Triple &b) { return a.src == b.src && a.tgt == b.tgt && a.v == b.v; }),
           t->end());
}
}  // namespace

// See host.h.  The phase ranges follow the reference: phase ph computes
// level l of vertex i when prevl[i] < l <= level_ph[i] (l up to
// min(max level_ph, nlevel)); the skirt phase computes, for part p, level
// l of skirt vertex i when prevl[i] < l <= nlevel - dist_p(i).  A needed
// value (l-1, k) travels from the part that computed it last (store_part)
// to the computing part unless they coincide (proc_vertex,
// mpk2/buffers.c:53-66).
int fill_all_buffers(const Csr &g, int npart, int nlevel, int nphase, std::vector<std::vector<int>> *parts,
                     const std::vector<std::vector<int>> &levels, const std::vector<PartSkirt> &sk,
                     std::vector<RankBuffers> *out) {
  const int n = g.n, P = npart, L = nlevel;
  if ((int)parts->size() < std::max(nphase, 1) || (int)levels.size() < nphase || (int)sk.size() != P)
    return fail(kEInval, "missing partitions, levels or skirts");
  const size_t nvv = (size_t)n * (L + 1);
  std::vector<int> store(nvv, -1);
  for (int i = 0; i < n; i++) store[i] = (*parts)[0][i];
  auto lmin = [&](int ph) {  // min_or_0 (mpk2/buffers.c:68-77)
    if (nphase == 0 || ph < 0) return 0;
    return *std::min_element(levels[ph].begin(), levels[ph].end());
  };
  auto lmax = [&](int ph) {  // max_or_nlevel (mpk2/buffers.c:79-90)
    if (ph == nphase) return L;
    return std::min(L, *std::max_element(levels[ph].begin(), levels[ph].end()));
  };
  std::vector<std::vector<Triple>> ct(nphase + 1);
  std::vector<std::vector<std::vector<long>>> mlist(nphase + 1, std::vector<std::vector<long>>(P));
  int err = 0;
  auto proc = [&](int cur, int i, int level, std::vector<Triple> &t) {
    for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) {
      const long kv = (long)n * (level - 1) + g.col[j];
      const int sp = store[kv];
      if (sp == -1) err = 1;
      else if (sp != cur) t.push_back({sp, cur, kv});
    }
  };
  std::vector<Triple> init;
  for (int i = 0; i < n; i++) init.push_back({(*parts)[0][i], (*parts)[0][i], (long)i});
  for (int ph = 0; ph < nphase; ph++) {
    const std::vector<int> &ll = levels[ph];
    const int *prevl = ph ? levels[ph - 1].data() : nullptr;
    const int lo = lmin(ph - 1), hi = lmax(ph);
    if (ph > 0) {  // collect_comm + reduce_comm (mpk2/buffers.c:92-123, reduce_comm.c:44-59)
      std::vector<Triple> cc;
      for (int level = lo + 1; level <= hi; level++)
        for (int i = 0; i < n; i++)
          if (prevl[i] < level && level <= ll[i]) {
            const int tgt = (*parts)[ph][i];
            for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) {
              const long kv = (long)n * (level - 1) + g.col[j];
              if (store[kv] != -1) cc.push_back({store[kv], tgt, kv});
            }
          }
      unique_triples(&cc);
      std::vector<long> sums((size_t)P * P, 0);
      for (const Triple &t : cc) sums[(size_t)t.src * P + t.tgt]++;
      std::vector<int> perm;
      assign_max_trace(sums, P, &perm);
      for (int &q : (*parts)[ph]) q = perm[q];
    }
    std::vector<Triple> &t = ct[ph];
    if (ph == 0) t = init;
    for (int level = lo + 1; level <= hi; level++)
      for (int i = 0; i < n; i++) {
        const int pv = prevl ? prevl[i] : 0;
        if (pv < level && level <= ll[i] && store[(size_t)level * n + i] == -1) {
          const int cur = (*parts)[ph][i];
          proc(cur, i, level, t);
          store[(size_t)level * n + i] = cur;
          mlist[ph][cur].push_back((long)level * n + i);
        }
      }
  }
  {  // skirt_comm_table + iterator(skirt_cond) (mpk2/buffers.c:155-179, 203-238)
    std::vector<Triple> &t = ct[nphase];
    if (nphase == 0) t = init;
    const int *prevl = nphase ? levels[nphase - 1].data() : nullptr;
    const int lo = lmin(nphase - 1);
    for (int p = 0; p < P; p++)
      for (int level = lo + 1; level <= L; level++)
        for (size_t q = 0; q < sk[p].vert.size(); q++) {
          const int i = sk[p].vert[q], d = sk[p].dist[q];
          const int pv = prevl ? prevl[i] : 0;
          if (pv < level && d >= 0 && level <= L - d) {
            proc(p, i, level, t);
            store[(size_t)level * n + i] = p;
            mlist[nphase][p].push_back((long)level * n + i);
          }
        }
  }
  if (err) return fail(kEStruct, "a needed value is computed by no part (inconsistent levels/skirt)");
  for (auto &t : ct) unique_triples(&t);
  out->assign(P, RankBuffers());
  for (int r = 0; r < P; r++) {
    RankBuffers &b = (*out)[r];
    b.n = n; b.npart = P; b.nlevel = L; b.nphase = nphase; b.rank = r;
    const size_t np = (size_t)P * (nphase + 1), ph1 = nphase + 1;
    b.recvcounts.assign(np, 0); b.sendcounts.assign(np, 0); b.rdispls.assign(np, 0); b.sdispls.assign(np, 0);
    for (auto *v : {&b.rcount, &b.mcount, &b.scount, &b.rbuf_offsets, &b.mbuf_offsets, &b.sbuf_offsets,
                    &b.mptr_offsets, &b.mcol_offsets})
      v->assign(ph1, 0);
    std::vector<std::vector<long>> rlist(ph1), slist(ph1);
    for (int ph = 0; ph <= nphase; ph++) {
      // fill_idx_rsbuf order (mpk2/buffers.c:354-377): by peer, then vv index
      for (const Triple &t : ct[ph])
        if (t.tgt == r) { rlist[ph].push_back(t.v); b.recvcounts[(size_t)P * ph + t.src]++; }
      std::vector<Triple> sends;
      for (const Triple &t : ct[ph])
        if (t.src == r) sends.push_back(t);
      std::sort(sends.begin(), sends.end(), [](const Triple &a, const Triple &c) {
        return a.tgt != c.tgt ? a.tgt < c.tgt : a.v < c.v;
      });
      for (const Triple &t : sends) { slist[ph].push_back(t.v); b.sendcounts[(size_t)P * ph + t.tgt]++; }
      // by_tgt sorted the receive list by (src, v) within tgt == r
      b.rcount[ph] = (int)rlist[ph].size();
      b.scount[ph] = (int)slist[ph].size();
      b.mcount[ph] = (int)mlist[ph][r].size();
      for (int q = 1; q < P; q++) {
        const size_t k = (size_t)P * ph + q;
        b.sdispls[k] = b.sdispls[k - 1] + b.sendcounts[k - 1];
        b.rdispls[k] = b.rdispls[k - 1] + b.recvcounts[k - 1];
      }
    }
    // alloc_bufs (mpk2/buffers.c:317-352)
    long count = 0, scount = 0, mptrcount = 0;
    for (int ph = 0; ph <= nphase; ph++) {
      b.rbuf_offsets[ph] = (int)count;
      count += b.rcount[ph];
      b.mbuf_offsets[ph] = (int)count;
      count += b.mcount[ph];
      b.sbuf_offsets[ph] = (int)scount;
      scount += b.scount[ph];
      b.mptr_offsets[ph] = (int)mptrcount;
      mptrcount += b.mcount[ph] + 1;
    }
    b.buf_count = (int)count;
    b.buf_scount = (int)scount;
    b.mptr_count = (int)mptrcount;
    b.idx_buf.clear();
    b.idx_sbuf.clear();
    b.mptr_buf.clear();
    for (int ph = 0; ph <= nphase; ph++) {
      b.idx_buf.insert(b.idx_buf.end(), rlist[ph].begin(), rlist[ph].end());
      b.idx_buf.insert(b.idx_buf.end(), mlist[ph][r].begin(), mlist[ph][r].end());
      b.idx_sbuf.insert(b.idx_sbuf.end(), slist[ph].begin(), slist[ph].end());
      long acc = 0;  // fill_mptr (mpk2/buffers.c:379-390)
      b.mptr_buf.push_back(0);
      for (long idx : mlist[ph][r]) {
        const int i = (int)(idx % n);
        acc += g.ptr[i + 1] - g.ptr[i];
        b.mptr_buf.push_back(acc);
      }
    }
    // fill_mcol_sbuf (mpk2/buffers.c:413-474): columns and send entries
    // become positions of the first occurrence in idx_buf
    std::unordered_map<long, long> find;
    find.reserve(b.idx_buf.size() * 2);
    for (size_t i = 0; i < b.idx_buf.size(); i++) find.emplace(b.idx_buf[i], (long)i);
    auto first = [&](long v) {
      auto it = find.find(v);
      return it == find.end() ? -1L : it->second;
    };
    long mcol_count = 0;
    b.mcol_buf.clear();
    b.mval_buf.clear();
    for (int ph = 0; ph <= nphase; ph++) {
      b.mcol_offsets[ph] = (int)mcol_count;
      for (long idx : mlist[ph][r]) {
        const long i = idx % n, level = idx / n;
        for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) {
          b.mcol_buf.push_back(first(g.col[j] + (long)n * (level - 1)));
          if (!g.val.empty()) b.mval_buf.push_back(g.val[j]);  // alloc_fill_mval (mpi2_mpkwrtbufs.c:12-29)
        }
      }
      mcol_count = (long)b.mcol_buf.size();
    }
    b.mcol_count = (int)mcol_count;
    for (long &v : b.idx_sbuf) v = first(v);
  }
  return kOk;
}

}  // namespace mpkg
