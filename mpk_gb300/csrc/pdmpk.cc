// pdmpk buffers: the prep (CommCompPatterns), the buf.bin / results.bin
// format and the reference class methods declared in
// include/pdmpk_gb300.h.  Host code only; the buffers execute on the GPU
// through mpkg_plan_pdmpk (device.cu).
#include "../../include/pdmpk_gb300.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <map>
#include <set>
#include <stdexcept>

#include "../../include/mpk_gb300.h"
#include "host.h"

namespace pdmpk_gb300 {

using mpkg::fail;

// ---- Csr -------------------------------------------------------------------

Csr::Csr(const std::string &fname) {
  mpkg::Csr g;
  if (mpkg::read_mtx(fname, &g) != mpkg::kOk) throw std::logic_error(mpkg::last_error());
  n = g.n;
  nnz = (idx_t)g.nnz();
  ptr = std::move(g.ptr);
  col = std::move(g.col);
  val = std::move(g.val);
  FILE *f = fopen(fname.c_str(), "r");
  char banner[256] = {0};
  if (f) {
    if (!fgets(banner, sizeof banner, f)) banner[0] = 0;
    fclose(f);
  }
  const std::string b(banner);
  pattern = b.find(" pattern") != std::string::npos;
  symmetric = b.find(" symmetric") != std::string::npos;
}

int Csr::MPK(const int &nlevels, std::vector<double> &vec) const {
  if ((idx_t)vec.size() != n || nlevels < 0) return fail(mpkg::kEInval, "Csr::MPK: vector size or level count");
  if (nlevels == 0) return mpkg::kOk;
  mpkg_plan *p = nullptr;
  int rc = mpkg_plan_spmv(n, ptr.data(), col.data(), val.data(), nlevels, MPKG_ARITH_SEPARATE, &p);
  if (rc) return rc;
  std::vector<double> vv((size_t)(nlevels + 1) * n, 0.0);
  std::copy(vec.begin(), vec.end(), vv.begin());
  rc = mpkg_exec_host(p, vv.data());
  mpkg_plan_destroy(p);
  if (rc) return rc;
  std::copy(vv.end() - n, vv.end(), vec.begin());
  return mpkg::kOk;
}

// ---- MpiBuffers, Buffers ---------------------------------------------------

void MpiBuffers::PhaseInit() {
  const size_t size = recvcounts.size() + npart;
  recvcounts.resize(size);
  sendcounts.resize(size);
  rdispls.resize(size);
  sdispls.resize(size);
  sbuf_idcs.rec_phase_begin();
  init_idcs.rec_phase_begin();
}

void MpiBuffers::FillDispls() {
  const size_t o = sendcounts.size() - npart;
  sdispls[o] = rdispls[o] = 0;
  for (idx_t i = 1; i < npart; i++) {
    sdispls[o + i] = sdispls[o + i - 1] + sendcounts[o + i - 1];
    rdispls[o + i] = rdispls[o + i - 1] + recvcounts[o + i - 1];
  }
}

void MpiBuffers::SortInitIdcs() {
  std::sort(init_idcs.begin() + init_idcs.phase_begin.back(), init_idcs.end(),
            [](const sidx_tidx_t &a, const sidx_tidx_t &b) { return a.second < b.second; });
}

size_t MpiBuffers::SbufSize(const int &phase) const {
  const size_t k = (size_t)npart * phase + npart - 1;
  return sendcounts[k] + sdispls[k];
}

size_t MpiBuffers::RbufSize(const int &phase) const {
  const size_t k = (size_t)npart * phase + npart - 1;
  return recvcounts[k] + rdispls[k];
}

void Buffers::PreBatch() {
  mpi_bufs.PhaseInit();
  mcsr.mptr.rec_phase_begin();
  mbuf.phase_begin.push_back(mbuf_idx);
}

void Buffers::PostBatch(const int &batch) {
  mpi_bufs.FillDispls();
  const size_t s = mpi_bufs.SbufSize(batch);
  max_sbuf_size = std::max(max_sbuf_size, s);
  mpi_bufs.sbuf_idcs.resize(mpi_bufs.sbuf_idcs.size() + s);
  mbuf_idx += (idx_t)mpi_bufs.RbufSize(batch);
}

namespace {

// Vectors as the reference's Utils::DumpVec writes them: size_t count,
// then the raw elements.
template <typename T>
void put_vec(FILE *f, const std::vector<T> &v, bool *ok) {
  const size_t c = v.size();
  *ok = *ok && fwrite(&c, sizeof c, 1, f) == 1 && (c == 0 || fwrite(v.data(), sizeof(T), c, f) == c);
}

template <typename T>
void get_vec(FILE *f, std::vector<T> *v, bool *ok) {
  size_t c = 0;
  if (!*ok || fread(&c, sizeof c, 1, f) != 1 || c > ((size_t)1 << 36) / sizeof(T)) {
    *ok = false;
    return;
  }
  v->resize(c);
  *ok = c == 0 || fread(v->data(), sizeof(T), c, f) == c;
}

}  // namespace

static_assert(sizeof(PhaseDescriptor) == 3 * sizeof(level_t), "PhaseDescriptor is three shorts");
static_assert(sizeof(sidx_tidx_t) == 2 * sizeof(idx_t), "init pairs are two ints");

int Buffers::Dump(const std::string &buf_bin, const std::string &results_bin) const {
  FILE *f = fopen(buf_bin.c_str(), "wb");
  if (!f) return fail(mpkg::kEIo, "cannot write " + buf_bin);
  bool ok = fwrite(&max_sbuf_size, sizeof max_sbuf_size, 1, f) == 1 && fwrite(&mbuf_idx, sizeof mbuf_idx, 1, f) == 1;
  put_vec(f, mbuf.phase_begin, &ok);
  put_vec(f, home_idcs, &ok);
  put_vec(f, original_idcs, &ok);
  put_vec(f, phase_descriptors, &ok);
  put_vec(f, results.mbuf_idcs, &ok);
  put_vec(f, mpi_bufs.sendcounts, &ok);
  put_vec(f, mpi_bufs.sdispls, &ok);
  put_vec(f, mpi_bufs.recvcounts, &ok);
  put_vec(f, mpi_bufs.rdispls, &ok);
  put_vec<idx_t>(f, mpi_bufs.sbuf_idcs, &ok);
  put_vec(f, mpi_bufs.sbuf_idcs.phase_begin, &ok);
  put_vec<sidx_tidx_t>(f, mpi_bufs.init_idcs, &ok);
  put_vec(f, mpi_bufs.init_idcs.phase_begin, &ok);
  put_vec<idx_t>(f, mcsr.mptr, &ok);
  put_vec(f, mcsr.mptr.phase_begin, &ok);
  put_vec(f, mcsr.mcol, &ok);
  put_vec(f, mcsr.mval, &ok);
  ok = (fclose(f) == 0) && ok;
  if (!ok) return fail(mpkg::kEIo, "write failed: " + buf_bin);
  f = fopen(results_bin.c_str(), "wb");
  if (!f) return fail(mpkg::kEIo, "cannot write " + results_bin);
  put_vec(f, results.original_idcs, &ok);
  put_vec(f, results.values, &ok);
  ok = (fclose(f) == 0) && ok;
  return ok ? mpkg::kOk : fail(mpkg::kEIo, "write failed: " + results_bin);
}

int Buffers::Load(const std::string &buf_bin, const std::string &results_bin) {
  FILE *f = fopen(buf_bin.c_str(), "rb");
  if (!f) return fail(mpkg::kEIo, "cannot open " + buf_bin);
  bool ok = fread(&max_sbuf_size, sizeof max_sbuf_size, 1, f) == 1 && fread(&mbuf_idx, sizeof mbuf_idx, 1, f) == 1;
  get_vec(f, &mbuf.phase_begin, &ok);
  get_vec(f, &home_idcs, &ok);
  get_vec(f, &original_idcs, &ok);
  get_vec(f, &phase_descriptors, &ok);
  get_vec(f, &results.mbuf_idcs, &ok);
  get_vec(f, &mpi_bufs.sendcounts, &ok);
  get_vec(f, &mpi_bufs.sdispls, &ok);
  get_vec(f, &mpi_bufs.recvcounts, &ok);
  get_vec(f, &mpi_bufs.rdispls, &ok);
  get_vec<idx_t>(f, &mpi_bufs.sbuf_idcs, &ok);
  get_vec(f, &mpi_bufs.sbuf_idcs.phase_begin, &ok);
  get_vec<sidx_tidx_t>(f, &mpi_bufs.init_idcs, &ok);
  get_vec(f, &mpi_bufs.init_idcs.phase_begin, &ok);
  get_vec<idx_t>(f, &mcsr.mptr, &ok);
  get_vec(f, &mcsr.mptr.phase_begin, &ok);
  get_vec(f, &mcsr.mcol, &ok);
  get_vec(f, &mcsr.mval, &ok);
  fclose(f);
  if (!ok) return fail(mpkg::kEFormat, "truncated or malformed " + buf_bin);
  f = fopen(results_bin.c_str(), "rb");
  if (!f) return fail(mpkg::kEIo, "cannot open " + results_bin);
  get_vec(f, &results.original_idcs, &ok);
  get_vec(f, &results.values, &ok);
  fclose(f);
  if (!ok) return fail(mpkg::kEFormat, "truncated or malformed " + results_bin);
  if (mpi_bufs.sendcounts.size() % std::max<idx_t>(mpi_bufs.npart, 1) != 0)
    return fail(mpkg::kEFormat, buf_bin + ": count vectors do not match npart");
  return mpkg::kOk;
}

std::string Filename(const std::string &mtxname, int npart, int nlevel, int mirror_method, int weight_update_method,
                     int rank, const std::string &branch, const std::string &hash, const std::string &suffix) {
  std::string s = mtxname + "-np" + std::to_string(npart) + "-nl" + std::to_string(nlevel) + "-mm" +
                  std::to_string(mirror_method) + "-wm" + std::to_string(weight_update_method);
  if (rank > -1) s += "-r" + std::to_string(rank);
  return s + "-" + branch + "-" + hash + "." + suffix;
}

Partitioner BlockShiftPartitioner() {
  return [](const Csr &csr, const idx_t *, int npart, int call, idx_t *part) {
    const long n = csr.n, shift = (long)call * n / (2L * npart);
    for (long i = 0; i < n; i++) part[i] = (idx_t)((((i + shift) % n) * npart) / n);
    return 0;
  };
}

Partitioner BfsPartitioner() {
  return [](const Csr &csr, const idx_t *, int npart, int, idx_t *part) {
    mpkg::Csr g;
    g.n = csr.n;
    g.ptr = csr.ptr;
    g.col = csr.col;
    std::vector<int> p;
    const int rc = mpkg::partition_bfs(g, npart, &p);
    if (rc == 0) std::copy(p.begin(), p.end(), part);
    return rc;
  };
}

Partitioner MetisPartitioner() {
  return [](const Csr &csr, const idx_t *adjwgt, int npart, int, idx_t *part) {
    // MetisPartition passes options = NULL; MetisPartitionWithWeights passes
    // args.opt, METIS_SetDefaultOptions's all -1 unless the command line
    // changed it (pdmpk/args.cc:24-31)
    int opt[mpkg::kMetisNOptions];
    std::fill(opt, opt + mpkg::kMetisNOptions, -1);
    return mpkg::metis_kway(csr.n, csr.ptr.data(), csr.col.data(), nullptr, adjwgt, npart, adjwgt ? opt : nullptr,
                            part, nullptr);
  };
}

// ---- CommCompPatterns ---------------------------------------------------------
//
// The prep walks the levels of every vertex upwards in batches.  A batch
// (one `lbelow`) lets every vertex at level lbelow add the columns whose
// source value (level lbelow) lives in the vertex's current part; a row
// whose columns are all added moves up a level.  Values living in another
// part are received in the batch's rbuf, recorded in a communication
// dictionary ordered by (src part, tgt part) then (source mbuf slot,
// kind), and back-patched when the batch closes.  Phases re-partition the
// graph (weights from the levels) so that the stalled vertices progress.

namespace {

enum Kind { kMcol = 0, kInitIdcs = 1, kFinished = 2 };

struct Prep {
  const Csr &csr;
  const Args &args;
  Partitioner partition;
  const int n, P, L;
  std::vector<Buffers> *bufs;

  // vertex state (pdmpk/pdmpk_buffers.h:14-175)
  struct State {
    std::vector<level_t> levels;
    std::vector<char> partials;
    std::vector<idx_t> partitions;
    bool can_add(const Csr &c, idx_t i, int lbelow, idx_t t) const {
      const idx_t j = c.col[t];
      return !partials[t] && partitions[i] == partitions[j] && levels[j] >= lbelow;
    }
    bool partial_empty(const Csr &c, idx_t i) const {
      for (idx_t t = c.ptr[i]; t < c.ptr[i + 1]; t++)
        if (partials[t]) return false;
      return true;
    }
    bool partial_full(const Csr &c, idx_t i) const {
      for (idx_t t = c.ptr[i]; t < c.ptr[i + 1]; t++)
        if (!partials[t]) return false;
      return true;
    }
    double partial_completed(const Csr &c, idx_t i) const {
      int cnt = 0;
      for (idx_t t = c.ptr[i]; t < c.ptr[i + 1]; t++) cnt += partials[t] ? 1 : 0;
      return double(cnt) / double(c.ptr[i + 1] - c.ptr[i]);
    }
    void inc_level(const Csr &c, idx_t i) {
      if (!partial_full(c, i)) return;
      levels[i]++;
      for (idx_t t = c.ptr[i]; t < c.ptr[i + 1]; t++) partials[t] = 0;
    }
  };
  State cur, sim;  // sim: the trial run that chooses label permutations
  std::vector<idx_t> weights;
  int calls = 0;

  // (vertex, level) -> (part, mbuf slot); part -1 = absent
  std::vector<std::pair<idx_t, idx_t>> store;
  std::pair<idx_t, idx_t> &at(idx_t i, int l) { return store[(size_t)i * (L + 1) + l]; }

  typedef std::pair<idx_t, int> SrcKey;  // (source mbuf slot, kind)
  std::map<std::pair<idx_t, idx_t>, std::map<SrcKey, std::set<idx_t>>> comm_dict;
  std::vector<std::set<idx_t>> comm_table;  // P*P, trial communication sets
  std::vector<idx_t> home;
  std::vector<std::vector<idx_t>> history;
  int batch = -1;
  int err = 0;

  Prep(const Csr &c, const Args &a, std::vector<Buffers> *b)
      : csr(c), args(a), partition(a.partitioner ? a.partitioner : BlockShiftPartitioner()), n(c.n), P(a.npart),
        L(a.nlevel), bufs(b) {}

  int call_partitioner(const idx_t *w) {
    std::vector<idx_t> part(n);
    if (partition(csr, w, P, calls++, part.data()) != 0) return fail(mpkg::kEInval, "partitioner failed");
    for (idx_t p : part)
      if (p < 0 || p >= P) return fail(mpkg::kERange, "partitioner returned a part out of range");
    cur.partitions = part;
    return mpkg::kOk;
  }

  void finalize(idx_t i, int l, idx_t part) {
    at(i, l) = {part, (*bufs)[part].mbuf_idx};
    (*bufs)[part].mbuf_idx++;
  }

  // pdmpk/comm_comp_patterns.cc SendHome: finished values not at home are
  // sent there in the next batch.
  void send_home(idx_t i) {
    const auto &s = at(i, L);
    if (s.first < 0) return;
    if (s.first != home[i]) comm_dict[{s.first, home[i]}][{s.second, kFinished}].insert(i);
  }

  void pre_batch() {
    batch++;
    for (Buffers &b : *bufs) b.PreBatch();
    for (idx_t i = 0; i < n; i++)
      if (cur.levels[i] == L) send_home(i);
  }

  void post_batch(int lbelow) {
    for (const auto &e : comm_dict) {
      const idx_t src = e.first.first, tgt = e.first.second;
      const int size = (int)e.second.size();
      (*bufs)[tgt].mpi_bufs.recvcounts[(size_t)batch * P + src] += size;
      (*bufs)[src].mpi_bufs.sendcounts[(size_t)batch * P + tgt] += size;
    }
    for (Buffers &b : *bufs) b.PostBatch(batch);
    std::vector<char> needs_wait(P, 0);
    for (const auto &e : comm_dict) {
      const idx_t src = e.first.first, tgt = e.first.second;
      needs_wait[tgt] = 1;
      Buffers &sb = (*bufs)[src], &tb = (*bufs)[tgt];
      const size_t send0 = sb.mpi_bufs.sbuf_idcs.phase_begin[batch] + sb.mpi_bufs.sdispls[(size_t)batch * P + tgt];
      const size_t recv0 = tb.mbuf.phase_begin[batch] + tb.mcsr.mptr.size() - tb.mcsr.mptr.phase_begin[batch] +
                           tb.mpi_bufs.rdispls[(size_t)batch * P + src];
      size_t k = 0;
      for (const auto &m : e.second) {
        const idx_t slot = (idx_t)(recv0 + k);
        if (m.first.second == kMcol) {
          for (idx_t t : m.second) tb.mcsr.mcol[t] = slot;
        } else if (m.first.second == kInitIdcs) {
          tb.mpi_bufs.init_idcs.push_back({slot, *m.second.begin()});
        } else {
          at(*m.second.begin(), L) = {tgt, slot};
        }
        sb.mpi_bufs.sbuf_idcs[send0 + k] = m.first.first;
        k++;
      }
    }
    comm_dict.clear();
    for (int r = 0; r < P; r++) {
      PhaseDescriptor &pd = (*bufs)[r].phase_descriptors.back();
      pd.UpdateBottom((level_t)lbelow);
      pd.UpdateTop((level_t)lbelow);
      if (needs_wait[r]) pd.UpdateMid((level_t)lbelow);
      (*bufs)[r].mpi_bufs.SortInitIdcs();
    }
  }

  void add_adjacent(idx_t i, int lbelow, idx_t t) {
    cur.partials[t] = 1;
    const idx_t j = csr.col[t], part = cur.partitions[i];
    const auto src = at(j, lbelow);
    if (src.first < 0) {
      err = err ? err : fail(mpkg::kEStruct, "pdmpk prep: source value missing");
      return;
    }
    Buffers &b = (*bufs)[part];
    b.mcsr.mval.push_back(csr.val[t]);
    if (src.first == part) {
      b.mcsr.mcol.push_back(src.second);
    } else {
      comm_dict[{src.first, part}][{src.second, kMcol}].insert((idx_t)b.mcsr.mcol.size());
      b.mcsr.mcol.push_back(-1);
    }
  }

  void add_init(idx_t i, int level) {
    const auto src = at(i, level);
    if (src.first < 0) {
      err = err ? err : fail(mpkg::kEStruct, "pdmpk prep: partial value missing");
      return;
    }
    const idx_t tgt = cur.partitions[i], slot = (*bufs)[tgt].mbuf_idx;
    if (src.first != tgt)
      comm_dict[{src.first, tgt}][{src.second, kInitIdcs}].insert(slot);
    else
      (*bufs)[tgt].mpi_bufs.init_idcs.push_back({src.second, slot});
  }

  bool proc_vertex(idx_t i, int lbelow) {
    bool any = false;
    const idx_t part = cur.partitions[i];
    const bool send_partial = !cur.partial_empty(csr, i);
    for (idx_t t = csr.ptr[i]; t < csr.ptr[i + 1]; t++) {
      if (!cur.can_add(csr, i, lbelow, t)) continue;
      if (!any) (*bufs)[part].mcsr.NextMcolIdxToMptr();
      add_adjacent(i, lbelow, t);
      any = true;
    }
    if (any) {
      if (send_partial) add_init(i, lbelow + 1);
      cur.inc_level(csr, i);
      finalize(i, lbelow + 1, part);
    }
    return any;
  }

  void proc_phase(int min_level) {
    for (Buffers &b : *bufs) b.phase_descriptors.emplace_back();
    bool active = true;
    for (int lbelow = min_level; active && lbelow < L && !err; lbelow++) {
      pre_batch();
      active = false;
      for (idx_t i = 0; i < n; i++)
        if (cur.levels[i] == lbelow && proc_vertex(i, lbelow)) active = true;
      post_batch(lbelow);
    }
  }

  // Edge weights for the re-partition (pdmpk/pdmpk_buffers.cc:80-150).
  void update_weights(int min) {
    for (idx_t i = 0; i < n; i++)
      for (idx_t t = csr.ptr[i]; t < csr.ptr[i + 1]; t++) {
        const idx_t j = csr.col[t];
        const int li = cur.levels[i], lj = cur.levels[j], m = std::min(li, lj);
        switch (args.weight_update_method) {
          case 0: {
            const double eps = cur.partial_completed(csr, i) + cur.partial_completed(csr, j);
            const double w = 1.0e+4 / ((li + lj - 2 * min + 0.5 * eps) + 1.0);
            weights[t] = w < 1.0 ? 1 : (idx_t)w;
            break;
          }
          case 1: {
            const idx_t w = (L - m + min) + 1;
            weights[t] = cur.partials[t] ? 1 : w * w;
            break;
          }
          case 2: {
            const idx_t w = (L - m + min) + 1;
            weights[t] = cur.partials[t] ? w : (idx_t)(1ul << w);
            break;
          }
          default: {
            const double e = li < lj ? cur.partial_completed(csr, i) : cur.partial_completed(csr, j);
            const size_t w = (size_t)(L - m + min);
            weights[t] = (!cur.partials[t] && m == min) ? (idx_t)(w * (size_t)(1 << int(w * e))) : (idx_t)(w * w + 1);
            break;
          }
        }
      }
  }

  // Trial run of the coming phase on a copy of the state: counts, per (old
  // part, new label), the distinct values that would move, then relabels
  // the new partition to keep the most of them in place (maximum-trace
  // assignment, the reference's lapjv).
  int optimize_labels(int min_level) {
    sim = cur;
    comm_table.assign((size_t)P * P, std::set<idx_t>());
    bool active = true;
    for (int lbelow = min_level; active && lbelow < L; lbelow++) {
      active = false;
      for (idx_t i = 0; i < n; i++) {
        if (sim.levels[i] != lbelow) continue;
        bool any = false;
        const idx_t tgt = sim.partitions[i];
        const bool send_partial = !sim.partial_empty(csr, i);
        for (idx_t t = csr.ptr[i]; t < csr.ptr[i + 1]; t++) {
          if (!sim.can_add(csr, i, lbelow, t)) continue;
          sim.partials[t] = 1;
          const auto &s = at(csr.col[t], lbelow);
          if (s.first >= 0) {
            comm_table[(size_t)s.first * P + tgt].insert(s.second);
            any = true;
          }
        }
        if (any) {
          if (send_partial) {
            const auto &s = at(i, lbelow + 1);
            if (s.first < 0) return fail(mpkg::kEStruct, "pdmpk prep: trial partial value missing");
            comm_table[(size_t)s.first * P + tgt].insert(s.second);
          }
          sim.inc_level(csr, i);
          active = true;
        }
      }
    }
    std::vector<long> sums((size_t)P * P);
    long mn = 0;
    for (size_t k = 0; k < sums.size(); k++) {
      sums[k] = (long)comm_table[k].size();
      mn = k == 0 ? sums[k] : std::min(mn, sums[k]);
    }
    for (long &s : sums) s -= mn;
    std::vector<int> perm;
    mpkg::assign_max_trace(sums, P, &perm);
    for (idx_t &p : cur.partitions) p = perm[p];
    comm_table.clear();
    return mpkg::kOk;
  }

  int new_partition_labels(int min_level) {
    update_weights(min_level);
    int rc = call_partitioner(weights.data());
    if (rc) return rc;
    for (idx_t i = 0; i < n; i++) {
      if (cur.levels[i] != min_level) continue;
      for (idx_t t = csr.ptr[i]; t < csr.ptr[i + 1]; t++)
        if (!cur.partials[t]) cur.partitions[csr.col[t]] = cur.partitions[i];
    }
    if ((rc = optimize_labels(min_level))) return rc;
    history.push_back(cur.partitions);
    return mpkg::kOk;
  }

  bool finished() const {
    for (level_t l : cur.levels)
      if (l != L) return false;
    return true;
  }

  size_t exact_level_sum() const {
    size_t s = 0;
    for (idx_t i = 0; i < n; i++) {
      s += (size_t)cur.levels[i] * (csr.ptr[i + 1] - csr.ptr[i]);
      for (idx_t t = csr.ptr[i]; t < csr.ptr[i + 1]; t++) s += cur.partials[t] ? 1 : 0;
    }
    return s;
  }

  level_t min_level() const { return *std::min_element(cur.levels.begin(), cur.levels.end()); }

  // The six phase strategies (pdmpk/comm_comp_patterns.cc ProcAllPhases0..5):
  // when to re-partition (and whether to stop on no progress) versus reuse
  // an earlier partition.
  int all_phases() {
    const int mm = args.mirror_method;
    const bool check_progress = (mm == 0 || mm == 1 || mm == 2 || mm == 5);
    size_t old_sum = 0;
    while (!finished() && (mm == 0 || !history.empty())) {
      const int ml = min_level();
      const size_t sum = exact_level_sum();
      bool fresh;
      switch (mm) {
        case 0: fresh = true; break;
        case 1: case 3: fresh = ml < L / 2; break;
        case 2: case 4: fresh = ml == 0; break;
        default: fresh = 2 * ml < 3 * L; break;
      }
      if (fresh) {
        if (check_progress) {
          if (old_sum == sum) break;
          old_sum = sum;
        }
        int rc = new_partition_labels(ml);
        if (rc) return rc;
      } else if (mm == 2 || mm == 4) {
        cur.partitions = history[(size_t)batch % history.size()];
      } else {
        cur.partitions = history.back();
        history.pop_back();
      }
      proc_phase(ml);
      if (err) return err;
    }
    if (!finished()) return fail(mpkg::kEStruct, "pdmpk prep: the mirror method could not finish (no progress)");
    return mpkg::kOk;
  }

  void epilogue() {
    for (idx_t i = 0; i < n; i++) {
      if (home[i] != at(i, L).first) {
        for (Buffers &b : *bufs) b.phase_descriptors.emplace_back();
        pre_batch();
        post_batch(L - 1);
        break;
      }
    }
    for (Buffers &b : *bufs) {
      b.mcsr.mptr.rec_phase_begin();
      b.mcsr.NextMcolIdxToMptr();
      b.mpi_bufs.init_idcs.rec_phase_begin();
    }
    for (idx_t i = 0; i < n; i++) {
      const auto fin = at(i, L), first = at(i, 0);
      if (fin.first < 0 || fin.first != first.first) {
        err = err ? err : fail(mpkg::kEStruct, "pdmpk prep: a result did not return to its home part");
        return;
      }
      Buffers &b = (*bufs)[fin.first];
      b.home_idcs[first.second] = fin.second;
      b.results.SaveIndex(i, fin.second);
    }
  }

  int run() {
    if (P <= 0 || L <= 0 || L > 32000 || n <= 0) return fail(mpkg::kEInval, "pdmpk prep: bad npart/nlevel/n");
    if (args.mirror_method < 0 || args.mirror_method > 5) return fail(mpkg::kEInval, "mirror method must be 0..5");
    if (args.weight_update_method < 0 || args.weight_update_method > 3)
      return fail(mpkg::kEInval, "weight update method must be 0..3");
    if ((long)csr.ptr.size() != (long)n + 1 || (long)csr.col.size() < csr.ptr[n] || (long)csr.val.size() < csr.ptr[n])
      return fail(mpkg::kEInval, "pdmpk prep: inconsistent CSR");
    for (idx_t i = 0; i < n; i++)
      if (csr.ptr[i + 1] <= csr.ptr[i]) return fail(mpkg::kEInval, "pdmpk prep: empty row");
    bufs->assign(P, Buffers(P));
    cur.levels.assign(n, 0);
    cur.partials.assign(csr.ptr[n], 0);
    weights.assign(csr.ptr[n], 0);
    store.assign((size_t)n * (L + 1), {-1, -1});
    int rc = call_partitioner(nullptr);
    if (rc) return rc;
    history.push_back(cur.partitions);
    home = cur.partitions;
    for (idx_t i = 0; i < n; i++) {
      const idx_t part = cur.partitions[i];
      (*bufs)[part].home_idcs.push_back(0);
      (*bufs)[part].original_idcs.push_back(i);
      finalize(i, 0, part);
    }
    batch = -1;
    proc_phase(0);
    if (err) return err;
    for (Buffers &b : *bufs) b.phase_descriptors.back().UpdateMid(-1);
    if ((rc = all_phases())) return rc;
    epilogue();
    return err;
  }
};

}  // namespace

int CommCompPatterns(const Csr &csr, const Args &args, std::vector<Buffers> *bufs) {
  mpkg::clear_error();
  if (!bufs) return fail(mpkg::kEInval, "bufs is null");
  Prep prep(csr, args, bufs);
  const int rc = prep.run();
  if (rc) bufs->clear();
  return rc;
}

}  // namespace pdmpk_gb300

// ---- execution maps ---------------------------------------------------------

namespace mpkg {

using pdmpk_gb300::Buffers;

int pd_exec_maps(const std::vector<Buffers> &bufs, PdExecMaps *m) {
  const int P = (int)bufs.size();
  if (P <= 0) return fail(kEInval, "no pdmpk buffers");
  *m = PdExecMaps();
  const size_t nb = bufs[0].mbuf.phase_begin.size();
  std::vector<long> goff(P + 1, 0);
  long n = 0;
  int nlevel = 0;
  for (int r = 0; r < P; r++) {
    const Buffers &b = bufs[r];
    const std::string who = "pdmpk rank " + std::to_string(r) + ": ";
    if (b.mpi_bufs.npart != P && b.mpi_bufs.npart != 0) return fail(kEFormat, who + "npart mismatch");
    if (b.mbuf.phase_begin.size() != nb || b.mcsr.mptr.phase_begin.size() != nb + 1 ||
        b.mpi_bufs.init_idcs.phase_begin.size() != nb + 1 || b.mpi_bufs.sbuf_idcs.phase_begin.size() != nb ||
        b.mpi_bufs.sendcounts.size() != nb * P || b.mpi_bufs.recvcounts.size() != nb * P ||
        b.mpi_bufs.sdispls.size() != nb * P || b.mpi_bufs.rdispls.size() != nb * P)
      return fail(kEFormat, who + "batch counts disagree");
    if (b.mbuf_idx < 0 || b.mcsr.mcol.size() != b.mcsr.mval.size() || b.home_idcs.size() != b.original_idcs.size() ||
        b.results.mbuf_idcs.size() != b.results.original_idcs.size() ||
        (nb && b.mbuf.phase_begin[0] != b.original_idcs.size()))
      return fail(kEFormat, who + "inconsistent sizes");
    long pd_sum = 0;
    for (const auto &pd : b.phase_descriptors) {
      pd_sum += pd.top - pd.bottom;
      nlevel = std::max<int>(nlevel, pd.top);
    }
    if (pd_sum != (long)nb) return fail(kEFormat, who + "phase descriptors do not cover the batches");
    goff[r + 1] = goff[r] + b.mbuf_idx;
    n += (long)b.original_idcs.size();
  }
  if (n <= 0 || nlevel <= 0 || n > INT32_MAX) return fail(kEFormat, "pdmpk buffers hold no rows");
  m->n = (int)n;
  m->nlevel = nlevel;
  m->nbatch = (int)nb;
  m->mbuf_total = goff[P];
  std::vector<char> seen(n, 0), seen_out(n, 0);
  for (int r = 0; r < P; r++) {
    const Buffers &b = bufs[r];
    for (size_t q = 0; q < b.original_idcs.size(); q++) {
      const long v = b.original_idcs[q];
      if (v < 0 || v >= n || seen[v]) return fail(kEFormat, "pdmpk: original indices are not a permutation");
      seen[v] = 1;
      m->in_dst.push_back(goff[r] + (long)q);
      m->in_src.push_back(v);
    }
    for (size_t q = 0; q < b.results.original_idcs.size(); q++) {
      const long v = b.results.original_idcs[q];
      long slot = b.results.mbuf_idcs[q];
      if (v < 0 || v >= n || seen_out[v] || slot < 0 || slot >= b.mbuf_idx)
        return fail(kEFormat, "pdmpk: result indices out of range or repeated");
      // SendHome (mbuf[i] = mbuf[home_idcs[i]]) runs before the results
      // are read: follow it for results that point into the home region.
      if ((size_t)slot < b.home_idcs.size()) {
        slot = b.home_idcs[slot];
        if (slot < (long)b.home_idcs.size() || slot >= b.mbuf_idx)
          return fail(kEFormat, "pdmpk: home index chain not supported");
      }
      seen_out[v] = 1;
      m->out_src.push_back(goff[r] + slot);
      m->out_dst.push_back(v);
    }
  }
  for (long v = 0; v < n; v++)
    if (!seen_out[v]) return fail(kEFormat, "pdmpk: some rows have no result");
  m->cm_off.assign(nb + 1, 0);
  m->row_off.assign(nb + 1, 0);
  m->row_ptr.assign(1, 0);
  for (size_t bt = 0; bt < nb; bt++) {
    m->cm_off[bt] = (long)m->cm_dst.size();
    for (int dst = 0; dst < P; dst++) {
      const Buffers &d = bufs[dst];
      const long rbuf0 = (long)d.mbuf.phase_begin[bt] + (long)d.mcsr.MptrSize((int)bt);
      for (int src = 0; src < P; src++) {
        const Buffers &s = bufs[src];
        const size_t kd = bt * P + src, ks = bt * P + dst;
        const long cnt = d.mpi_bufs.recvcounts[kd];
        if (cnt != s.mpi_bufs.sendcounts[ks] || cnt < 0) return fail(kEFormat, "pdmpk: send/receive counts differ");
        const long r0 = rbuf0 + d.mpi_bufs.rdispls[kd];
        const long s0 = (long)s.mpi_bufs.sbuf_idcs.phase_begin[bt] + s.mpi_bufs.sdispls[ks];
        if (r0 < 0 || r0 + cnt > d.mbuf_idx || s0 < 0 || s0 + cnt > (long)s.mpi_bufs.sbuf_idcs.size())
          return fail(kEFormat, "pdmpk: communication range out of bounds");
        for (long q = 0; q < cnt; q++) {
          const long from = s.mpi_bufs.sbuf_idcs[s0 + q];
          if (from < 0 || from >= s.mbuf_idx) return fail(kEFormat, "pdmpk: send index out of range");
          m->cm_dst.push_back(goff[dst] + r0 + q);
          m->cm_src.push_back(goff[src] + from);
        }
      }
    }
    m->row_off[bt] = (long)m->row_dst.size();
    for (int r = 0; r < P; r++) {
      const Buffers &b = bufs[r];
      const size_t p0 = b.mcsr.mptr.phase_begin[bt], p1 = b.mcsr.mptr.phase_begin[bt + 1];
      if (p1 < p0 || p1 + 1 > b.mcsr.mptr.size())
        return fail(kEFormat, "pdmpk: row pointers out of range");
      size_t ii = b.mpi_bufs.init_idcs.phase_begin[bt];
      const size_t i1 = b.mpi_bufs.init_idcs.phase_begin[bt + 1];
      if (i1 > b.mpi_bufs.init_idcs.size() || ii > i1) return fail(kEFormat, "pdmpk: init ranges out of range");
      for (size_t mi = 0; mi < p1 - p0; mi++) {
        const long slot = (long)b.mbuf.phase_begin[bt] + (long)mi;
        if (slot >= b.mbuf_idx) return fail(kEFormat, "pdmpk: row slot out of range");
        long init = -1;  // Buffers::DoComp: the next seed whose target is this row
        if (ii < i1 && (long)b.mpi_bufs.init_idcs[ii].second == slot) {
          const long from = b.mpi_bufs.init_idcs[ii].first;
          if (from < 0 || from >= b.mbuf_idx) return fail(kEFormat, "pdmpk: init source out of range");
          init = goff[r] + from;
          ii++;
        }
        const long j0 = b.mcsr.mptr[p0 + mi], j1 = b.mcsr.mptr[p0 + mi + 1];
        if (j0 < 0 || j1 < j0 || j1 > (long)b.mcsr.mcol.size()) return fail(kEFormat, "pdmpk: mptr out of range");
        for (long j = j0; j < j1; j++) {
          const long c = b.mcsr.mcol[j];
          if (c < 0 || c >= b.mbuf_idx) return fail(kEFormat, "pdmpk: mcol out of range");
          m->gcol.push_back(goff[r] + c);
          m->gval.push_back(b.mcsr.mval[j]);
        }
        m->row_dst.push_back(goff[r] + slot);
        m->row_init.push_back(init);
        m->row_ptr.push_back((long)m->gcol.size());
      }
    }
  }
  m->cm_off[nb] = (long)m->cm_dst.size();
  m->row_off[nb] = (long)m->row_dst.size();
  return kOk;
}

}  // namespace mpkg
