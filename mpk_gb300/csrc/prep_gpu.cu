// PA1 prep on the GPU.  For every part, the distance-bounded ball (the
// vertices within r arcs of the part under the reference's skirt distance,
// mpk2/lib.c:584-615: row i is one arc from every column it reads), then
//  * tiles (r = nlevel): the ball sorted by (distance, vertex) and the
//    tiles' sliced-ELL local structure -- the TilePlan of build_tile_plan;
//  * task lists (r = nlevel - 1): the ball sorted by vertex (the skirt of
//    comp_skirts) and the level-major task lists of build_tasks
//    (mpk2/mpkprep.c:185-233 for nphase = 0).
// Results equal the host builds (prep.cc) byte for byte; the host builds
// stay the fallback for balls beyond the GPU path's capacity and for every
// error case, so errors keep their codes and messages.
//
// Layout: one persistent CTA per SM.  Each CTA owns an n-entry mark array
// (distance during the search, slot index while the local structure is
// built, -1 otherwise) that it restores after every part, so one memset per
// call prepares all parts.  A part's ball (at most kBallCap vertices) is
// gathered level by level into its own row of a [npart][kBallCap] array and
// sorted in shared memory as 32-bit keys.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <numeric>
#include <vector>

#include "../../include/mpk_gb300.h"
#include "host.h"

namespace mpkg {
namespace {

constexpr int kBallCap = 32768;             // vertices per ball (keys sorted in 128 KB of shared memory)
constexpr int kSliceCap = kBallCap / 32;    // slices of 32 rows per ball
constexpr int kThreads = 1024;
constexpr int kVertBits = 27;               // vertex field of a sort key
constexpr int kDistBits = 5;                // distance field of a (vertex, distance) key
constexpr long kMaxBallBytes = 8L << 30;    // the [npart][kBallCap] array

#define PG_TRY(x)                                                                  \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess) return fail(kECuda, std::string("prep: ") + cudaGetErrorString(e_)); \
  } while (0)

struct BallArgs {
  int n, npart, nlevel, radius;
  const int *ptr;                 // CSR rows (degrees)
  const long *trptr;              // transpose: the rows that read vertex u
  const int *tridx;
  const int *mptr, *mvert;        // members of each part, ascending
  int *mark;                      // gridDim.x * n, -1 when idle
  int *ball;                      // npart * kBallCap: vertices (tiles) or (vertex, distance) keys
  int *bsize;                     // ball size; -1 beyond capacity, -2 empty part
  int *shell;                     // npart * (nlevel + 1): vertices within distance d <= radius
  unsigned char *width;           // npart * kSliceCap: slice widths (255 caps)
  long long *ell;                 // npart: sum of 32 * width; -1 when a row is longer than 255
};

template <bool TILES>
__global__ void __launch_bounds__(kThreads, 1) ball_kernel(BallArgs a) {
  extern __shared__ unsigned int keys[];  // kBallCap
  __shared__ int s_cnt, s_over, s_wide;
  __shared__ unsigned long long s_ell;
  int *mark = a.mark + (size_t)blockIdx.x * a.n;
  for (int p = blockIdx.x; p < a.npart; p += gridDim.x) {
    int *list = a.ball + (size_t)p * kBallCap;
    const int m0 = a.mptr[p + 1] - a.mptr[p];
    if (m0 == 0 || m0 > kBallCap) {
      if (threadIdx.x == 0) a.bsize[p] = m0 == 0 ? -2 : -1;
      for (int d = threadIdx.x; d <= a.nlevel; d += blockDim.x) a.shell[(size_t)p * (a.nlevel + 1) + d] = 0;
      continue;
    }
    if (threadIdx.x == 0) { s_cnt = m0; s_over = 0; s_wide = 0; s_ell = 0; }
    for (int t = threadIdx.x; t < m0; t += blockDim.x) {
      const int v = a.mvert[a.mptr[p] + t];
      mark[v] = 0;
      list[t] = v;
    }
    __syncthreads();
    int *shell = a.shell + (size_t)p * (a.nlevel + 1);
    int lo = 0, hi = m0;
    for (int d = 0; d < a.radius; d++) {
      if (threadIdx.x == 0) shell[d] = hi;
      for (int q = lo + (int)threadIdx.x; q < hi; q += blockDim.x) {
        const int u = list[q];
        for (long t = a.trptr[u]; t < a.trptr[u + 1]; t++) {
          const int i = a.tridx[t];
          if (mark[i] < 0 && atomicCAS(&mark[i], -1, d + 1) == -1) {
            const int pos = atomicAdd(&s_cnt, 1);
            if (pos < kBallCap) {
              list[pos] = i;
            } else {  // beyond capacity: leave the mark as it was
              mark[i] = -1;
              s_over = 1;
            }
          }
        }
      }
      __syncthreads();
      lo = hi;
      hi = min(s_cnt, kBallCap);
      const int over = s_over;
      __syncthreads();
      if (over) break;
    }
    if (s_over) {
      for (int q = threadIdx.x; q < hi; q += blockDim.x) mark[list[q]] = -1;
      if (threadIdx.x == 0) a.bsize[p] = -1;
      __syncthreads();
      continue;
    }
    const int m = hi;
    if (threadIdx.x == 0) shell[a.radius] = m;
    // sort by (distance, vertex) for tiles, by vertex for task lists
    int p2 = 2;
    while (p2 < m) p2 <<= 1;
    for (int q = threadIdx.x; q < p2; q += blockDim.x) {
      unsigned key = 0xFFFFFFFFu;
      if (q < m) {
        const unsigned v = (unsigned)list[q], d = (unsigned)mark[v];
        key = TILES ? (d << kVertBits) | v : (v << kDistBits) | d;
      }
      keys[q] = key;
    }
    __syncthreads();
    for (int k2 = 2; k2 <= p2; k2 <<= 1)
      for (int j = k2 >> 1; j > 0; j >>= 1) {
        for (int q = threadIdx.x; q < p2; q += blockDim.x) {
          const int r = q ^ j;
          if (r > q) {
            const unsigned x0 = keys[q], x1 = keys[r];
            if ((x0 > x1) == ((q & k2) == 0)) {
              keys[q] = x1;
              keys[r] = x0;
            }
          }
        }
        __syncthreads();
      }
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
      const int v = TILES ? (int)(keys[q] & ((1u << kVertBits) - 1)) : (int)(keys[q] >> kDistBits);
      list[q] = TILES ? v : (int)keys[q];
      mark[v] = -1;
    }
    __syncthreads();
    if (!TILES) {
      if (threadIdx.x == 0) {
        a.bsize[p] = m;
        a.ell[p] = 0;
      }
      __syncthreads();
      continue;
    }
    // widths of the slices of the rows computed at level 1 (distance <= nlevel - 1)
    const int nrows = shell[a.nlevel - 1];
    unsigned char *wd = a.width + (size_t)p * kSliceCap;
    for (int s = threadIdx.x; s * 32 < nrows; s += blockDim.x) {
      int w = 0;
      for (int r = s * 32; r < min(nrows, s * 32 + 32); r++) {
        const int v = list[r];
        w = max(w, a.ptr[v + 1] - a.ptr[v]);
      }
      if (w > 255) s_wide = 1;
      wd[s] = (unsigned char)min(w, 255);
      atomicAdd(&s_ell, 32ull * (unsigned)w);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      a.bsize[p] = m;
      a.ell[p] = s_wide ? -1 : (long long)s_ell;
    }
    __syncthreads();
  }
}

struct EllArgs {
  int n, npart, nlevel;
  const int *ptr, *col;
  const int *ball, *bsize, *shell;
  const long *slot_off, *slice_off, *ell_off;
  int *mark;
  int *slot_vert;
  unsigned short *ell_col;   // prefilled with 0xFFFF (padding)
  int *err;
};

__global__ void __launch_bounds__(kThreads, 1) ell_kernel(EllArgs a) {
  int *mark = a.mark + (size_t)blockIdx.x * a.n;
  for (int p = blockIdx.x; p < a.npart; p += gridDim.x) {
    const int *list = a.ball + (size_t)p * kBallCap;
    const int m = a.bsize[p];
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
      mark[list[q]] = q;
      a.slot_vert[a.slot_off[p] + q] = list[q];
    }
    __syncthreads();
    const int nrows = a.shell[(size_t)p * (a.nlevel + 1) + a.nlevel - 1];
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
      const int v = list[r];
      const long base = a.ell_off[a.slice_off[p] + r / 32] + (r & 31);
      for (int j = a.ptr[v], t = 0; j < a.ptr[v + 1]; j++, t++) {
        const int c = mark[a.col[j]];
        if (c < 0) atomicExch(a.err, 1);
        else a.ell_col[base + 32L * t] = (unsigned short)c;
      }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < m; q += blockDim.x) mark[list[q]] = -1;
    __syncthreads();
  }
}

// Level-major task lists of every part from its vertex-sorted skirt: level
// l takes the skirt vertices at distance <= nlevel - l, in vertex order
// (an order-keeping compaction per level: per-thread runs, block scan).
struct TaskArgs {
  int n, npart, nlevel;
  const int *ball, *bsize;
  const long *off;
  long *idx;
};

__global__ void __launch_bounds__(kThreads, 1) task_kernel(TaskArgs a) {
  __shared__ int s_warp[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int p = blockIdx.x; p < a.npart; p += gridDim.x) {
    const unsigned *keys = reinterpret_cast<const unsigned *>(a.ball + (size_t)p * kBallCap);
    const int m = max(a.bsize[p], 0);
    const int per = (m + blockDim.x - 1) / blockDim.x;
    const int q0 = min(m, (int)threadIdx.x * per), q1 = min(m, q0 + per);
    long base = a.off[p];
    for (int l = 1; l <= a.nlevel; l++) {
      const unsigned dmax = (unsigned)(a.nlevel - l);
      int c = 0;
      for (int q = q0; q < q1; q++) c += (keys[q] & ((1u << kDistBits) - 1)) <= dmax;
      int x = c;  // inclusive scan within the warp
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) s_warp[warp] = x;
      __syncthreads();
      if (warp == 0) {
        int w = s_warp[lane];
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xFFFFFFFFu, w, o);
          if (lane >= o) w += y;
        }
        s_warp[lane] = w;
      }
      __syncthreads();
      long r = base + (x - c) + (warp ? s_warp[warp - 1] : 0);
      for (int q = q0; q < q1; q++)
        if ((keys[q] & ((1u << kDistBits) - 1)) <= dmax) a.idx[r++] = (long)l * a.n + (long)(keys[q] >> kDistBits);
      base += s_warp[kThreads / 32 - 1];
      __syncthreads();
    }
  }
}

// Device buffers released on every exit path.
struct DevBufs {
  std::vector<void *> ptrs;
  ~DevBufs() {
    for (void *q : ptrs) cudaFree(q);
  }
  template <typename T>
  int alloc(T **out, size_t count) {
    *out = nullptr;
    PG_TRY(cudaMalloc((void **)out, sizeof(T) * std::max<size_t>(count, 1)));
    ptrs.push_back(*out);
    return kOk;
  }
  template <typename T>
  int upload(T **out, const T *src, size_t count) {
    int rc = alloc(out, count);
    if (rc) return rc;
    if (count) PG_TRY(cudaMemcpy(*out, src, sizeof(T) * count, cudaMemcpyHostToDevice));
    return kOk;
  }
};

// The ball search of every part on the GPU: inputs uploaded once, results
// (sizes, shells, slice widths) copied back.
struct BallRun {
  DevBufs db;
  int n = 0, npart = 0, nlevel = 0, grid = 0;
  int *d_ptr = nullptr, *d_col = nullptr, *d_mark = nullptr, *d_ball = nullptr, *d_bsize = nullptr,
      *d_shell = nullptr;
  unsigned char *d_width = nullptr;
  long long *d_ell = nullptr;
  std::vector<int> bsize, shell;
  std::vector<long long> ell;
  std::vector<unsigned char> width;

  // false: the GPU path does not apply (sizes beyond its limits)
  static bool fits(int n, int npart, int nlevel) {
    return n < (1 << kVertBits) - 1 && nlevel >= 1 && nlevel <= 31 && (long)npart * kBallCap * 4 <= kMaxBallBytes;
  }

  int run(const Csr &g, const std::vector<int> &part, int npart_, int nlevel_, int radius, bool tiles) {
    n = g.n; npart = npart_; nlevel = nlevel_;
    int dev = 0, nsm = 0;
    PG_TRY(cudaGetDevice(&dev));
    PG_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    // one CTA per SM, fewer when the mark arrays would pass 4 GB
    const long per_cta = 4L * n;
    grid = (int)std::max(1L, std::min<long>(std::min(nsm, npart), (4L << 30) / std::max(per_cta, 1L)));
    // members (ascending) and the transpose, on the host: O(n + nnz)
    std::vector<int> mptr(npart + 1, 0), mvert(n);
    for (int v = 0; v < n; v++) mptr[part[v] + 1]++;
    for (int p = 0; p < npart; p++) mptr[p + 1] += mptr[p];
    {
      std::vector<int> fill(mptr.begin(), mptr.end() - 1);
      for (int v = 0; v < n; v++) mvert[fill[part[v]]++] = v;
    }
    std::vector<long> trptr(n + 1, 0);
    std::vector<int> tridx(g.nnz());
    for (long j = 0; j < g.nnz(); j++) trptr[g.col[j] + 1]++;
    for (int i = 0; i < n; i++) trptr[i + 1] += trptr[i];
    {
      std::vector<long> fill(trptr.begin(), trptr.end() - 1);
      for (int i = 0; i < n; i++)
        for (int j = g.ptr[i]; j < g.ptr[i + 1]; j++) tridx[fill[g.col[j]]++] = i;
    }
    int rc;
    int *d_tridx, *d_mptr, *d_mvert;
    long *d_trptr;
    if ((rc = db.upload(&d_ptr, g.ptr.data(), g.ptr.size()))) return rc;
    if ((rc = db.upload(&d_col, g.col.data(), g.col.size()))) return rc;
    if ((rc = db.upload(&d_trptr, trptr.data(), trptr.size()))) return rc;
    if ((rc = db.upload(&d_tridx, tridx.data(), tridx.size()))) return rc;
    if ((rc = db.upload(&d_mptr, mptr.data(), mptr.size()))) return rc;
    if ((rc = db.upload(&d_mvert, mvert.data(), mvert.size()))) return rc;
    if ((rc = db.alloc(&d_mark, (size_t)grid * n))) return rc;
    PG_TRY(cudaMemset(d_mark, 0xFF, sizeof(int) * (size_t)grid * n));
    if ((rc = db.alloc(&d_ball, (size_t)npart * kBallCap))) return rc;
    if ((rc = db.alloc(&d_bsize, npart))) return rc;
    if ((rc = db.alloc(&d_shell, (size_t)npart * (nlevel + 1)))) return rc;
    if ((rc = db.alloc(&d_width, tiles ? (size_t)npart * kSliceCap : 1))) return rc;
    if ((rc = db.alloc(&d_ell, npart))) return rc;
    BallArgs ba;
    std::memset(&ba, 0, sizeof(ba));
    ba.n = n; ba.npart = npart; ba.nlevel = nlevel; ba.radius = radius;
    ba.ptr = d_ptr; ba.trptr = d_trptr; ba.tridx = d_tridx; ba.mptr = d_mptr; ba.mvert = d_mvert;
    ba.mark = d_mark; ba.ball = d_ball; ba.bsize = d_bsize; ba.shell = d_shell; ba.width = d_width; ba.ell = d_ell;
    const size_t smem = sizeof(unsigned int) * kBallCap;
    if (tiles) {
      PG_TRY(cudaFuncSetAttribute(ball_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      ball_kernel<true><<<grid, kThreads, smem>>>(ba);
    } else {
      PG_TRY(cudaFuncSetAttribute(ball_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      ball_kernel<false><<<grid, kThreads, smem>>>(ba);
    }
    PG_TRY(cudaGetLastError());
    bsize.resize(npart);
    ell.resize(npart);
    shell.resize((size_t)npart * (nlevel + 1));
    PG_TRY(cudaMemcpy(bsize.data(), d_bsize, sizeof(int) * npart, cudaMemcpyDeviceToHost));
    PG_TRY(cudaMemcpy(ell.data(), d_ell, sizeof(long long) * npart, cudaMemcpyDeviceToHost));
    PG_TRY(cudaMemcpy(shell.data(), d_shell, sizeof(int) * shell.size(), cudaMemcpyDeviceToHost));
    if (tiles) {
      width.resize((size_t)npart * kSliceCap);
      PG_TRY(cudaMemcpy(width.data(), d_width, width.size(), cudaMemcpyDeviceToHost));
    }
    return kOk;
  }
};

int check_part(int n, const std::vector<int> &part, int npart) {
  if ((int)part.size() != n) return fail(kEInval, "partition size != n");
  for (int q : part) if (q < 0 || q >= npart) return fail(kERange, "part id out of range");
  return kOk;
}

int host_pa1_tasks(const Csr &g, const std::vector<int> &part, int npart, int nlevel, TaskLists *tl) {
  std::vector<PartSkirt> sk;
  int rc = comp_skirts(g, part, npart, nullptr, nlevel, &sk);
  if (rc) return rc;
  return build_tasks(g, npart, nlevel, 0, {part}, {}, sk, false, tl);
}

}  // namespace

int build_pa1_tasks_gpu(const Csr &g, const std::vector<int> &part, int npart, int nlevel, TaskLists *tl,
                        bool *on_gpu) {
  *on_gpu = false;
  const int n = g.n;
  int rc = check_part(n, part, npart);
  if (rc) return rc;
  if (!BallRun::fits(n, npart, nlevel)) return host_pa1_tasks(g, part, npart, nlevel, tl);
  BallRun br;
  if ((rc = br.run(g, part, npart, nlevel, nlevel - 1, false))) return rc;
  for (int p = 0; p < npart; p++)
    if (br.bsize[p] == -1) return host_pa1_tasks(g, part, npart, nlevel, tl);  // beyond capacity
  tl->n = n; tl->npart = npart; tl->nlevel = nlevel; tl->nphase = 0;
  tl->off.assign((size_t)npart + 1, 0);
  for (int p = 0; p < npart; p++) {
    const int *sh = &br.shell[(size_t)p * (nlevel + 1)];
    long c = 0;
    for (int l = 1; l <= nlevel; l++) c += sh[nlevel - l];
    tl->off[p + 1] = tl->off[p] + c;
  }
  const long total = tl->off[npart];
  long *d_off, *d_idx;
  if ((rc = br.db.upload(&d_off, tl->off.data(), tl->off.size()))) return rc;
  if ((rc = br.db.alloc(&d_idx, total))) return rc;
  TaskArgs ta;
  ta.n = n; ta.npart = npart; ta.nlevel = nlevel;
  ta.ball = br.d_ball; ta.bsize = br.d_bsize; ta.off = d_off; ta.idx = d_idx;
  task_kernel<<<br.grid, kThreads>>>(ta);
  PG_TRY(cudaGetLastError());
  tl->idx.resize(total);
  if (total) PG_TRY(cudaMemcpy(tl->idx.data(), d_idx, sizeof(long) * total, cudaMemcpyDeviceToHost));
  *on_gpu = true;
  return kOk;
}

int build_tile_plan_gpu(const Csr &g, const std::vector<int> &part, int npart, int nlevel, TilePlan *tp,
                        bool *on_gpu) {
  *on_gpu = false;
  const int n = g.n;
  int rc = check_part(n, part, npart);
  if (rc) return rc;
  if (!BallRun::fits(n, npart, nlevel)) return build_tile_plan(g, part, npart, nlevel, tp);
  BallRun br;
  if ((rc = br.run(g, part, npart, nlevel, nlevel, true))) return rc;
  const std::vector<int> &bsize = br.bsize, &shell = br.shell;
  const std::vector<long long> &ell = br.ell;
  const std::vector<unsigned char> &width = br.width;
  // empty parts, balls beyond capacity, rows beyond 255 entries: the host
  // build decides (and reports the first error in part order)
  for (int p = 0; p < npart; p++)
    if (bsize[p] < 0 || ell[p] < 0) return build_tile_plan(g, part, npart, nlevel, tp);
  tp->n = n; tp->npart = npart; tp->nlevel = nlevel;
  part_order(g, part, npart, &tp->order);
  tp->shell = shell;
  tp->slot_off.assign(npart + 1, 0);
  tp->slice_off.assign(npart + 1, 0);
  tp->ell_off.assign(1, 0);
  tp->ell_width.clear();
  tp->max_slots = 0;
  tp->total_rows = 0;
  for (int p = 0; p < npart; p++) {
    const int *sh = &shell[(size_t)p * (nlevel + 1)];
    tp->slot_off[p + 1] = tp->slot_off[p] + bsize[p];
    tp->max_slots = std::max(tp->max_slots, bsize[p]);
    for (int l = 1; l <= nlevel; l++) tp->total_rows += sh[nlevel - l];
    const int nsl = (sh[nlevel - 1] + 31) / 32;
    tp->slice_off[p + 1] = tp->slice_off[p] + nsl;
    for (int s = 0; s < nsl; s++) {
      const unsigned char w = width[(size_t)p * kSliceCap + s];
      tp->ell_width.push_back(w);
      tp->ell_off.push_back(tp->ell_off.back() + 32L * w);
    }
  }
  const long nslots = tp->slot_off[npart], nell = tp->ell_off.back();
  DevBufs &db = br.db;
  const int grid = br.grid;
  int *d_ptr = br.d_ptr, *d_col = br.d_col, *d_ball = br.d_ball, *d_bsize = br.d_bsize, *d_shell = br.d_shell,
      *d_mark = br.d_mark;
  long *d_slot_off, *d_slice_off, *d_ell_off;
  int *d_slot_vert, *d_err;
  unsigned short *d_ell_col;
  if ((rc = db.upload(&d_slot_off, tp->slot_off.data(), tp->slot_off.size()))) return rc;
  if ((rc = db.upload(&d_slice_off, tp->slice_off.data(), tp->slice_off.size()))) return rc;
  if ((rc = db.upload(&d_ell_off, tp->ell_off.data(), tp->ell_off.size()))) return rc;
  if ((rc = db.alloc(&d_slot_vert, nslots))) return rc;
  if ((rc = db.alloc(&d_ell_col, nell))) return rc;
  if ((rc = db.alloc(&d_err, 1))) return rc;
  PG_TRY(cudaMemset(d_ell_col, 0xFF, sizeof(unsigned short) * std::max<long>(nell, 1)));
  PG_TRY(cudaMemset(d_err, 0, sizeof(int)));
  EllArgs ea;
  ea.n = n; ea.npart = npart; ea.nlevel = nlevel;
  ea.ptr = d_ptr; ea.col = d_col; ea.ball = d_ball; ea.bsize = d_bsize; ea.shell = d_shell;
  ea.slot_off = d_slot_off; ea.slice_off = d_slice_off; ea.ell_off = d_ell_off;
  ea.mark = d_mark; ea.slot_vert = d_slot_vert; ea.ell_col = d_ell_col; ea.err = d_err;
  ell_kernel<<<grid, kThreads>>>(ea);
  PG_TRY(cudaGetLastError());
  int err = 0;
  PG_TRY(cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return build_tile_plan(g, part, npart, nlevel, tp);  // a column outside its tile's halo
  tp->slot_vert.resize(nslots);
  tp->ell_col.resize(nell);
  if (nslots) PG_TRY(cudaMemcpy(tp->slot_vert.data(), d_slot_vert, sizeof(int) * nslots, cudaMemcpyDeviceToHost));
  if (nell) PG_TRY(cudaMemcpy(tp->ell_col.data(), d_ell_col, sizeof(unsigned short) * nell, cudaMemcpyDeviceToHost));
  *on_gpu = true;
  return kOk;
}

// The host build of the same lists (comp_skirts + build_tasks, nphase = 0).
int check_part_host(const Csr &g, const std::vector<int> &part, int npart, int nlevel, TaskLists *tl) {
  int rc = check_part(g.n, part, npart);
  if (rc) return rc;
  return host_pa1_tasks(g, part, npart, nlevel, tl);
}

// ---- DMPK phase levels and METIS weights on the GPU -----------------------
// comp_level / update_level (mpk2/lib.c:330-412): per part, the fixed point
// of minplus_r from BIG inside the part and init outside (-1, or the
// previous phase's levels).  Every part's fixed point at once: a vertex
// reads its own part's values and the fixed init of the others, so the
// parts never interact.  Jacobi sweeps from BIG descend to the same least
// values the reference's sweeps reach (the shortest-path fixed point, at
// most BIG), one launch per sweep until a sweep changes nothing.
__global__ void level_sweep_kernel(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                                   const int *__restrict__ part, const int *__restrict__ init,
                                   const long long *__restrict__ src, long long *__restrict__ dst,
                                   int *__restrict__ changed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    long long t = src[i];
    const int pi = part[i];
    for (int j = ptr[i]; j < ptr[i + 1]; j++) {
      const int c = col[j];
      const long long v = (part[c] != pi ? (init ? (long long)init[c] : -1LL) : src[c]) + 1;
      if (v < t) t = v;
    }
    dst[i] = t;
    if (t != src[i]) *changed = 1;
  }
}

__global__ void level_minmax_kernel(int n, const int *__restrict__ lev, int *mm) {
  int lo = 0x7fffffff, hi = -0x7fffffff - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    lo = min(lo, lev[i]);
    hi = max(hi, lev[i]);
  }
  atomicMin(mm, lo);
  atomicMax(mm + 1, hi);
}

// level2wcrs (mpk2/lib.c:504-537): vertex weight max + 1 - l_i; edge weight
// 1e6 / (l_i + l_j - 2 min + 1) truncated, at least 1 (IEEE division, the
// host's bits).
__global__ void level_weight_kernel(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                                    const int *__restrict__ lev, const int *__restrict__ mm, int *__restrict__ wv,
                                    int *__restrict__ we) {
  const int mn = mm[0], mx = mm[1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int l0 = lev[i];
    wv[i] = mx + 1 - l0;
    for (int j = ptr[i]; j < ptr[i + 1]; j++) {
      double w = (double)(l0 + lev[col[j]] - 2 * mn);
      w = __ddiv_rn(1e+6, __dadd_rn(w, 1.0));
      we[j] = w < 1.0 ? 1 : __double2int_rz(w);
    }
  }
}

template <typename T>
struct DevArr {
  T *p = nullptr;
  ~DevArr() { cudaFree(p); }
  cudaError_t alloc(size_t count) { return cudaMalloc((void **)&p, sizeof(T) * std::max<size_t>(count, 1)); }
  cudaError_t put(const T *src, size_t count) {
    cudaError_t e = alloc(count);
    return e != cudaSuccess || !count ? e : cudaMemcpy(p, src, sizeof(T) * count, cudaMemcpyHostToDevice);
  }
};

#define PG_TRY(expr)                                                                             \
  do {                                                                                           \
    cudaError_t e_ = (expr);                                                                     \
    if (e_ != cudaSuccess) return fail(kECuda, std::string(#expr ": ") + cudaGetErrorString(e_)); \
  } while (0)

int levels_gpu(int n, const int *ptr, const int *col, const int *part, const int *level_org, int *level) {
  const long nnz = ptr[n];
  long long big;
  if (level_org) {
    int mx = level_org[0];
    for (int i = 1; i < n; i++) mx = std::max(mx, level_org[i]);
    big = (long long)mx + n + 1;
  } else {
    big = (long long)n + 1;
  }
  DevArr<int> dptr, dcol, dpart, dinit, dchg;
  DevArr<long long> d0, d1;
  PG_TRY(dptr.put(ptr, (size_t)n + 1));
  PG_TRY(dcol.put(col, (size_t)nnz));
  PG_TRY(dpart.put(part, (size_t)n));
  if (level_org) PG_TRY(dinit.put(level_org, (size_t)n));
  PG_TRY(dchg.alloc(1));
  PG_TRY(d0.alloc(n));
  PG_TRY(d1.alloc(n));
  std::vector<long long> h(n, big);
  PG_TRY(cudaMemcpy(d0.p, h.data(), sizeof(long long) * n, cudaMemcpyHostToDevice));
  const int grid = (int)std::min<long>((n + 255) / 256, 4096);
  long long *src = d0.p, *dst = d1.p;
  for (long sweep = 0; sweep <= (long)n + 1; sweep++) {  // a fixed point is reached within n + 1 sweeps
    int chg = 0;
    PG_TRY(cudaMemsetAsync(dchg.p, 0, sizeof(int)));
    level_sweep_kernel<<<grid, 256>>>(n, dptr.p, dcol.p, dpart.p, level_org ? dinit.p : nullptr, src, dst, dchg.p);
    PG_TRY(cudaGetLastError());
    PG_TRY(cudaMemcpy(&chg, dchg.p, sizeof(int), cudaMemcpyDeviceToHost));
    std::swap(src, dst);
    if (!chg) break;
  }
  PG_TRY(cudaMemcpy(h.data(), src, sizeof(long long) * n, cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; i++) level[i] = (int)h[i];
  return kOk;
}

int level_weights_gpu(int n, const int *ptr, const int *col, const int *level, int *wv, int *we) {
  const long nnz = ptr[n];
  DevArr<int> dptr, dcol, dlev, dmm, dwv, dwe;
  PG_TRY(dptr.put(ptr, (size_t)n + 1));
  PG_TRY(dcol.put(col, (size_t)nnz));
  PG_TRY(dlev.put(level, (size_t)n));
  const int mm0[2] = {0x7fffffff, -0x7fffffff - 1};
  PG_TRY(dmm.put(mm0, 2));
  PG_TRY(dwv.alloc(n));
  PG_TRY(dwe.alloc(nnz));
  const int grid = (int)std::min<long>((n + 255) / 256, 4096);
  level_minmax_kernel<<<grid, 256>>>(n, dlev.p, dmm.p);
  level_weight_kernel<<<grid, 256>>>(n, dptr.p, dcol.p, dlev.p, dmm.p, dwv.p, dwe.p);
  PG_TRY(cudaGetLastError());
  PG_TRY(cudaMemcpy(wv, dwv.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
  if (nnz) PG_TRY(cudaMemcpy(we, dwe.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
  return kOk;
}

}  // namespace mpkg

extern "C" {

int mpkg_levels_gpu(int n, const int *ptr, const int *col, const int *part, int npart, const int *level_org,
                    int *level) {
  using namespace mpkg;
  clear_error();
  if (n <= 0 || !ptr || !col || ptr[0] != 0 || !part || !level || npart <= 0) return fail(kEInval, "bad argument");
  for (int i = 0; i < n; i++)
    if (ptr[i + 1] < ptr[i]) return fail(kEInval, "ptr must be non-decreasing");
  for (long j = 0; j < ptr[n]; j++)
    if (col[j] < 0 || col[j] >= n) return fail(kERange, "column index out of range");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  return levels_gpu(n, ptr, col, part, level_org, level);
}

int mpkg_level_weights_gpu(int n, const int *ptr, const int *col, const int *level, int *wv, int *we) {
  using namespace mpkg;
  clear_error();
  if (n <= 0 || !ptr || !col || ptr[0] != 0 || !level || !wv || !we) return fail(kEInval, "bad argument");
  for (int i = 0; i < n; i++)
    if (ptr[i + 1] < ptr[i]) return fail(kEInval, "ptr must be non-decreasing");
  for (long j = 0; j < ptr[n]; j++)
    if (col[j] < 0 || col[j] >= n) return fail(kERange, "column index out of range");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  return level_weights_gpu(n, ptr, col, level, wv, we);
}

int mpkg_tile_prep(int n, const int *ptr, const int *col, const int *part, int npart, int nlevel, int on_gpu,
                   mpkg_tiles_t *out) {
  using namespace mpkg;
  clear_error();
  if (!out || !part || npart <= 0 || nlevel <= 0) return fail(kEInval, "bad argument");
  std::memset(out, 0, sizeof(*out));
  if (n <= 0 || !ptr || !col || ptr[0] != 0) return fail(kEInval, "bad CSR");
  for (int i = 0; i < n; i++)
    if (ptr[i + 1] < ptr[i]) return fail(kEInval, "ptr must be non-decreasing");
  for (long j = 0; j < ptr[n]; j++)
    if (col[j] < 0 || col[j] >= n) return fail(kERange, "column index out of range");
  Csr g;
  g.n = n;
  g.ptr.assign(ptr, ptr + n + 1);
  g.col.assign(col, col + ptr[n]);
  std::vector<int> pv(part, part + n);
  TilePlan tp;
  bool gpu = false;
  int rc = on_gpu ? build_tile_plan_gpu(g, pv, npart, nlevel, &tp, &gpu) : build_tile_plan(g, pv, npart, nlevel, &tp);
  if (rc) return rc;
  auto dup = [](const auto &v) {
    using T = typename std::decay_t<decltype(v)>::value_type;
    T *q = (T *)std::malloc(sizeof(T) * std::max<size_t>(v.size(), 1));
    if (q && !v.empty()) std::memcpy(q, v.data(), sizeof(T) * v.size());
    return q;
  };
  out->npart = npart;
  out->nlevel = nlevel;
  out->max_slots = tp.max_slots;
  out->total_rows = tp.total_rows;
  out->nslots = (long)tp.slot_vert.size();
  out->nslices = (long)tp.ell_width.size();
  out->nell = (long)tp.ell_col.size();
  out->built_on_gpu = gpu ? 1 : 0;
  out->slot_off = dup(tp.slot_off);
  out->shell = dup(tp.shell);
  out->slot_vert = dup(tp.slot_vert);
  out->slice_off = dup(tp.slice_off);
  out->ell_off = dup(tp.ell_off);
  out->ell_col = dup(tp.ell_col);
  out->ell_width = dup(tp.ell_width);
  if (!out->slot_off || !out->shell || !out->slot_vert || !out->slice_off || !out->ell_off || !out->ell_col ||
      !out->ell_width) {
    mpkg_tiles_free(out);
    return fail(kENoMem, "allocation failed");
  }
  return kOk;
}

int mpkg_pa1_tasks(int n, const int *ptr, const int *col, const int *part, int npart, int nlevel, int on_gpu,
                   long *off, long **idx, long *count, int *built_on_gpu) {
  using namespace mpkg;
  clear_error();
  if (!part || !off || !idx || !count || npart <= 0 || nlevel <= 0) return fail(kEInval, "bad argument");
  *idx = nullptr;
  *count = 0;
  if (built_on_gpu) *built_on_gpu = 0;
  if (n <= 0 || !ptr || !col || ptr[0] != 0) return fail(kEInval, "bad CSR");
  for (int i = 0; i < n; i++)
    if (ptr[i + 1] < ptr[i]) return fail(kEInval, "ptr must be non-decreasing");
  for (long j = 0; j < ptr[n]; j++)
    if (col[j] < 0 || col[j] >= n) return fail(kERange, "column index out of range");
  Csr g;
  g.n = n;
  g.ptr.assign(ptr, ptr + n + 1);
  g.col.assign(col, col + ptr[n]);
  std::vector<int> pv(part, part + n);
  TaskLists tl;
  bool gpu = false;
  int rc = on_gpu ? build_pa1_tasks_gpu(g, pv, npart, nlevel, &tl, &gpu) : check_part_host(g, pv, npart, nlevel, &tl);
  if (rc) return rc;
  std::copy(tl.off.begin(), tl.off.end(), off);
  *idx = (long *)std::malloc(sizeof(long) * std::max<size_t>(tl.idx.size(), 1));
  if (!*idx) return fail(kENoMem, "allocation failed");
  if (!tl.idx.empty()) std::memcpy(*idx, tl.idx.data(), sizeof(long) * tl.idx.size());
  *count = (long)tl.idx.size();
  if (built_on_gpu) *built_on_gpu = gpu ? 1 : 0;
  return kOk;
}

void mpkg_tiles_free(mpkg_tiles_t *t) {
  if (!t) return;
  std::free(t->slot_off);
  std::free(t->shell);
  std::free(t->slot_vert);
  std::free(t->slice_off);
  std::free(t->ell_off);
  std::free(t->ell_col);
  std::free(t->ell_width);
  std::memset(t, 0, sizeof(*t));
}

}  // extern "C"
