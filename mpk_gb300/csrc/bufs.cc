// MPI-2 rank buffers: file format and consistency checks.
#include <cstdio>
#include <string>
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
