// CUDA kernels (sm_103a) and device plans of the GB300 matrix powers kernel.
//
// Executors (see include/mpk_gb300.h):
//   tasks  - the reference's (phase, part) task lists, one CTA per list,
//            levels separated by __syncthreads (mpk2/mpkexec.c:10-39);
//   tiles  - PA1 diamond tiles: one CTA per part, its k-deep skirt staged in
//            shared memory, k levels computed in place, owned rows written;
//   pipe   - zero-redundancy level pipeline: chunks of rows keep their
//            matrix rows in shared memory and advance level by level once
//            the neighbouring chunks have finished the previous level;
//   spmv   - k separate SpMV launches (baseline, spmv_exec_*).
// All executors evaluate each row sum over the stored columns in CSR order,
// so for a given arithmetic mode every executor produces the same bits.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/mpk_gb300.h"
#include "host.h"

using namespace mpkg;

namespace {

constexpr int kErrTimeout = 2;
constexpr int kErrBounds = 3;
constexpr long kSpinLimit = 4000000;  // polls of one flag (~1 s with backoff)

#define CUDA_TRY(expr)                                                             \
  do {                                                                             \
    cudaError_t e_ = (expr);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(kECuda, std::string(#expr) + ": " + cudaGetErrorString(e_));     \
  } while (0)

template <int ARITH>
__device__ __forceinline__ double row_term(double s, double a, double x) {
  if (ARITH == MPKG_ARITH_SEPARATE) return __dadd_rn(s, __dmul_rn(a, x));
  return __fma_rn(a, x, s);
}

__device__ __forceinline__ double ld_cg(const double *p) { return __ldcg(p); }

// ------------------------------------------------------------------------
// k-SpMV: one launch per level, one thread per row.
// ------------------------------------------------------------------------
template <int ARITH, bool VALUED>
__global__ void __launch_bounds__(256) spmv_level_kernel(int n, const int *__restrict__ ptr,
                                                         const int *__restrict__ col,
                                                         const double *__restrict__ coef,
                                                         const double *__restrict__ x,
                                                         double *__restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int j0 = ptr[i], j1 = ptr[i + 1];
  double s = 0.0;
  if (VALUED) {
    for (int j = j0; j < j1; j++) s = row_term<ARITH>(s, coef[j], x[col[j]]);
  } else {
    double a = coef[i];  // 1/deg, rounded on the host exactly as 1.0/deg
    for (int j = j0; j < j1; j++) s = row_term<ARITH>(s, a, x[col[j]]);
  }
  y[i] = s;
}

// ------------------------------------------------------------------------
// Task lists: one CTA per (phase, part) list; a list is a sequence of
// level segments of vertex ids, computed in order with a CTA barrier in
// between.  vv is read through L2 (ld.global.cg) because the skirt phase
// lets several CTAs write the same (level, vertex) with identical values.
// ------------------------------------------------------------------------
template <int ARITH, bool VALUED>
__global__ void __launch_bounds__(256) tasks_kernel(int n, int list_base,
                                                    const long *__restrict__ list_seg,
                                                    const int *__restrict__ seg_level,
                                                    const long *__restrict__ seg_off,
                                                    const int *__restrict__ rows,
                                                    const int *__restrict__ ptr,
                                                    const int *__restrict__ col,
                                                    const double *__restrict__ coef,
                                                    double *vv) {
  const int list = list_base + blockIdx.x;
  for (long sg = list_seg[list]; sg < list_seg[list + 1]; sg++) {
    const long l = seg_level[sg];
    const double *src = vv + (l - 1) * (long)n;
    double *dst = vv + l * (long)n;
    for (long q = seg_off[sg] + threadIdx.x; q < seg_off[sg + 1]; q += blockDim.x) {
      int i = rows[q];
      int j0 = ptr[i], j1 = ptr[i + 1];
      double s = 0.0;
      if (VALUED) {
        for (int j = j0; j < j1; j++) s = row_term<ARITH>(s, coef[j], ld_cg(src + col[j]));
      } else {
        double a = coef[i];
        for (int j = j0; j < j1; j++) s = row_term<ARITH>(s, a, ld_cg(src + col[j]));
      }
      dst[i] = s;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------
// PA1 tiles.  Tile p: slots [slot_off[p], slot_off[p+1]) sorted by
// (distance to part p, vertex); shell[p*(k+1)+d] = slots with distance
// <= d.  Level l is computed on slots [0, shell[k-l]); rows of slots with
// distance 0 (the part itself) are written to vv.  Local structure is
// sliced ELL (32 rows per slice, column-major inside a slice, 0xFFFF pads).
// Level buffers live in shared memory (SMEM) or, for tiles too large for
// it, in a global scratch area of 2*max_slots doubles per CTA.
// ------------------------------------------------------------------------
struct TileArgs {
  int n, nlevel, max_slots;
  const int *order;
  const long *slot_off;
  const int *shell;
  const int *slot_vert;
  const int *slot_coef;  // per slot: first value offset (valued) or vertex (1/deg)
  const long *slice_off;
  const long *ell_off;
  const uint16_t *ell_col;
  const uint8_t *ell_width;
  const int *ptr;       // global row pointers (value offsets)
  const double *coef;   // values (nnz) or 1/deg (n)
  const double *x;
  double *vv;
  double *scratch;      // used when !SMEM
  int *err;
};

// One tile row in FP64: the slice entries are loaded (and their gathers
// issued) before the first FMA for rows of up to 8 entries; the sum runs
// over the entries in CSR order.
template <int ARITH, bool VALUED>
__device__ __forceinline__ double tile_row_fp64(const TileArgs &a, long sl, int lane, int co, const double *in) {
  const int w = a.ell_width[sl];
  const uint16_t *cp = a.ell_col + a.ell_off[sl] + lane;
  double s = 0.0;
  if (w <= 8) {
    double xv[8], cv[8];
    bool ok[8];
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int c = t < w ? cp[t * 32] : 0xFFFF;
      ok[t] = c != 0xFFFF;
      xv[t] = ok[t] ? in[c] : 0.0;
      cv[t] = ok[t] ? (VALUED ? a.coef[co + t] : 0.0) : 0.0;
    }
    const double cf = VALUED ? 0.0 : a.coef[co];
#pragma unroll
    for (int t = 0; t < 8; t++)
      if (ok[t]) s = row_term<ARITH>(s, VALUED ? cv[t] : cf, xv[t]);
  } else {
    const double cf = VALUED ? 0.0 : a.coef[co];
    for (int t = 0; t < w; t++) {
      const int c = cp[t * 32];
      if (c == 0xFFFF) break;
      s = row_term<ARITH>(s, VALUED ? a.coef[co + t] : cf, in[c]);
    }
  }
  return s;
}

template <int ARITH, bool VALUED, bool SMEM>
__global__ void __launch_bounds__(512) tiles_kernel(TileArgs a) {
  extern __shared__ double smem_buf[];
  const int p = a.order[blockIdx.x];
  const long s0 = a.slot_off[p];
  const int ns = (int)(a.slot_off[p + 1] - s0);
  const int *shell = a.shell + (long)p * (a.nlevel + 1);
  const long sl0 = a.slice_off[p];
  double *buf0 = SMEM ? smem_buf : a.scratch + (long)blockIdx.x * 2 * a.max_slots;
  double *buf1 = buf0 + a.max_slots;
  if (ns > a.max_slots) {  // plan invariant; never true for a valid plan
    if (threadIdx.x == 0) atomicExch(a.err, kErrBounds);
    return;
  }
  for (int s = threadIdx.x; s < ns; s += blockDim.x) buf0[s] = a.x[a.slot_vert[s0 + s]];
  __syncthreads();
  const int owned = shell[0];
  for (int l = 1; l <= a.nlevel; l++) {
    const double *in = (l & 1) ? buf0 : buf1;
    double *out = (l & 1) ? buf1 : buf0;
    const int nrows = shell[a.nlevel - l];
    double *dst = a.vv + (long)l * a.n;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
      const double v = tile_row_fp64<ARITH, VALUED>(a, sl0 + (r >> 5), r & 31, a.slot_coef[s0 + r], in);
      out[r] = v;
      if (r < owned) dst[a.slot_vert[s0 + r]] = v;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------
// Level pipeline.  A persistent grid of CTAs takes chunks of `chunk`
// consecutive rows in ticket order.  The CTA copies the chunk's matrix
// rows into shared memory once, then for l = 1..k waits until every chunk
// its rows reference has published level l-1 (flags[c] = epoch*32 + level,
// bounded spin), computes the chunk's rows of level l into vv and publishes
// level l.  No row is computed twice.  A CTA waiting for level l-1 of chunk
// c + d needs that chunk to be running, so the plan requires the grid to
// hold more than (k-1)*reach chunks at once; a wait that exceeds the spin
// limit sets the error word and the whole grid drains.
// ------------------------------------------------------------------------
struct PipeArgs {
  int n, nlevel, chunk, nchunk, ngroups;
  uint32_t epoch;
  uint32_t stall;      // test hook: waits target counts this far beyond the real ones
  const int *gdep_lo, *gdep_hi;  // per chunk: first/last counter group it reads
  const int *ptr, *col;
  const double *coef;  // FP64 values (nnz) or 1/deg (n)
  const float2 *coef2; // double-float values (nnz) or 1/deg (n)
  const double *x;
  double *vv;
  float2 *ring;        // double-float level values, two slots of n
  unsigned int *ticket;
  unsigned int *counts;  // (nlevel+1) x ngroups completion counters
  int *err;
  int max_chunk_nnz;
  bool bulk_ok;        // col/coef bases are 16-byte aligned: stage with bulk copies
  const int *items;    // dataflow order: (level << 26) | chunk, topologically sorted
  int nitems;
};

constexpr int kPipeThreads = 256;
constexpr int kPipeChunk = kPipeThreads;  // rows per chunk, one per thread
constexpr int kPipeGroup = 1;             // chunks per completion counter

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned int group_size(const PipeArgs &a, int g) {
  return (unsigned)min(kPipeGroup, a.nchunk - g * kPipeGroup);
}

// Every thread of the CTA calls this.  Threads poll one completion counter
// each (acquire loads) until its group has finished `level` in this call;
// a poll count above kSpinLimit, or an error raised elsewhere, aborts the
// CTA.  Returns false on abort.  After the barrier, every thread's plain
// loads observe the data the producers released (acquire + CTA barrier).
__device__ __forceinline__ bool pipe_wait(const PipeArgs &a, int glo, int ghi, int level, int *s_abort) {
  for (int g = glo + (int)threadIdx.x; g <= ghi; g += blockDim.x) {
    const unsigned int want = a.epoch * group_size(a, g) + a.stall * 1024u;
    const unsigned int *cp = a.counts + (long)level * a.ngroups + g;
    long spins = 0;
    while (ld_acquire(cp) < want) {
      if (++spins > kSpinLimit || *((volatile int *)a.err)) {
        atomicCAS(a.err, 0, kErrTimeout);
        *s_abort = 1;
        break;
      }
      __nanosleep(spins < 16 ? 32 : 256);
    }
  }
  __syncthreads();
  return *s_abort == 0;
}

// Release of one chunk's level: the CTA synchronises, then one thread
// fences (cumulative over the CTA's writes ordered by the barrier) and
// bumps the chunk's counter.
__device__ __forceinline__ void pipe_publish(const PipeArgs &a, int c, int level) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(a.counts + (long)level * a.ngroups + c / kPipeGroup, 1u);
  }
}

// ---- 1-D bulk copies (TMA) of a chunk's CSR slice into shared memory ----
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar) {
  asm volatile("mbarrier.init.shared.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned long long *bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok) : "r"(smem_u32(bar)), "r"(phase) : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Element range [g0, g1) of a global array (16-byte aligned base, element
// size E) goes to smem buffer `dst` (16-byte aligned) so that element g0
// lands at dst[g0 % (16/E)].  The 16-byte-aligned body [ga, gb) moves by
// one bulk copy issued by thread 0, the ragged tail by plain loads.
template <typename T>
struct StageRange {
  long ga, gb, g1;
  __device__ __forceinline__ StageRange(long g0, long g1_, bool bulk_ok) {
    constexpr int per = 16 / sizeof(T);
    ga = g0 - (g0 % per);
    g1 = g1_;
    gb = bulk_ok ? (g1 / per) * per : ga;
    if (gb < ga) gb = ga;
  }
  __device__ __forceinline__ unsigned bulk_bytes() const { return (unsigned)((gb - ga) * sizeof(T)); }
  __device__ __forceinline__ void issue(T *dst, const T *src, unsigned long long *bar) const {
    if (threadIdx.x == 0 && gb > ga) bulk_g2s(dst, src + ga, bulk_bytes(), bar);
    for (long j = gb + threadIdx.x; j < g1; j += blockDim.x) dst[j - ga] = src[j];
  }
};

// Takes the next chunk and stages its rows in shared memory: row pointers
// by plain loads, columns and (valued operator) coefficients of type T by
// bulk copies completing on `bar`.  Returns the chunk id, or -1 when the
// work is exhausted or an error (bounds, copy timeout) occurred.  *cols_out
// and *vals_out point at the chunk's first entry inside the buffers.
template <typename T, bool VALUED>
__device__ __forceinline__ int pipe_take(const PipeArgs &a, const T *coef, int *rptr, int *cols_buf, T *vals_buf,
                                         int **cols_out, T **vals_out, unsigned long long *bar,
                                         unsigned *phase, unsigned int *s_chunk, int *s_abort) {
  if (threadIdx.x == 0) {
    *s_chunk = atomicAdd(a.ticket, 1u);
    *s_abort = 0;
  }
  __syncthreads();
  const int c = (int)*s_chunk;
  if (c >= a.nchunk) return -1;
  const int r0 = c * a.chunk;
  const int nr = min(a.chunk, a.n - r0);
  const long j00 = a.ptr[r0];
  const long j01 = a.ptr[r0 + nr];
  if (j01 - j00 > a.max_chunk_nnz) {  // plan invariant
    if (threadIdx.x == 0) atomicExch(a.err, kErrBounds);
    return -1;
  }
  for (int r = threadIdx.x; r <= a.chunk; r += blockDim.x) rptr[r] = (int)(a.ptr[r0 + min(r, nr)] - j00);
  const bool bulk_ok = a.bulk_ok;
  if (threadIdx.x == 0 && bulk_ok) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  const StageRange<int> rc(j00, j01, bulk_ok);
  const StageRange<T> rv(j00, j01, bulk_ok);
  if (bulk_ok && threadIdx.x == 0) mbar_expect(bar, rc.bulk_bytes() + (VALUED ? rv.bulk_bytes() : 0u));
  rc.issue(cols_buf, a.col, bar);
  if (VALUED) rv.issue(vals_buf, coef, bar);
  *cols_out = cols_buf + (j00 - rc.ga);
  *vals_out = vals_buf + (j00 - rv.ga);
  if (bulk_ok) {
    long spins = 0;
    while (!mbar_try(bar, *phase)) {
      if (++spins > kSpinLimit) {  // copy never completed: report, drain with a second bound
        if (threadIdx.x == 0) atomicCAS(a.err, 0, kErrTimeout);
        for (long s2 = 0; s2 < kSpinLimit && !mbar_try(bar, *phase); s2++) __nanosleep(256);
        return -1;
      }
    }
    *phase ^= 1u;
  }
  __syncthreads();
  return c;
}

// Shared memory of one pipeline CTA: row pointers, column buffer and value
// buffer (element size vsize), each 16-byte aligned with 16 bytes of slack
// for the alignment shift of a bulk copy.
__host__ __device__ __forceinline__ size_t pipe_cols_offset(int chunk) {
  return (((size_t)(chunk + 1) * sizeof(int) + 15) & ~(size_t)15);
}
__host__ __device__ __forceinline__ size_t pipe_vals_offset(int chunk, int max_nnz) {
  return pipe_cols_offset(chunk) + (((size_t)(max_nnz + 4) * sizeof(int) + 15) & ~(size_t)15);
}
__host__ __device__ __forceinline__ size_t pipe_smem_size(int chunk, int max_nnz, bool valued, size_t vsize) {
  return pipe_vals_offset(chunk, max_nnz) +
         (valued ? (((size_t)max_nnz + 16 / vsize) * vsize + 15) & ~(size_t)15 : 0);
}

// One row sum in FP64 over the entries [q0, q1) in CSR order; rows of up
// to 8 entries issue every gather before the first FMA.
template <int ARITH, bool VALUED>
__device__ __forceinline__ double pipe_row_fp64(int q0, int q1, const int *cols, const double *vals, double cf,
                                                const double *src) {
  double s = 0.0;
  if (q1 - q0 <= 8) {
    double xv[8];
#pragma unroll
    for (int t = 0; t < 8; t++)
      if (q0 + t < q1) xv[t] = src[cols[q0 + t]];
#pragma unroll
    for (int t = 0; t < 8; t++)
      if (q0 + t < q1) s = row_term<ARITH>(s, VALUED ? vals[q0 + t] : cf, xv[t]);
  } else {
    for (int q = q0; q < q1; q++) s = row_term<ARITH>(s, VALUED ? vals[q] : cf, src[cols[q]]);
  }
  return s;
}

template <int ARITH, bool VALUED>
__global__ void __launch_bounds__(kPipeThreads) pipe_kernel(PipeArgs a) {
  extern __shared__ __align__(16) unsigned char pipe_smem[];
  int *rptr = reinterpret_cast<int *>(pipe_smem);
  int *cols_buf = reinterpret_cast<int *>(pipe_smem + pipe_cols_offset(a.chunk));
  double *vals_buf = reinterpret_cast<double *>(pipe_smem + pipe_vals_offset(a.chunk, a.max_chunk_nnz));
  __shared__ unsigned int s_chunk;
  __shared__ int s_abort;
  __shared__ __align__(8) unsigned long long s_bar;
  unsigned phase = 0;
  if (threadIdx.x == 0 && a.bulk_ok) mbar_init(&s_bar);
  __syncthreads();
  for (;;) {
    int *cols;
    double *vals;
    const int c = pipe_take<double, VALUED>(a, a.coef, rptr, cols_buf, vals_buf, &cols, &vals, &s_bar, &phase,
                                            &s_chunk, &s_abort);
    if (c < 0) return;
    const int r0 = c * a.chunk;
    const int nr = min(a.chunk, a.n - r0);
    const int r = threadIdx.x;
    const bool active = r < nr;
    const double cf = (!VALUED && active) ? a.coef[r0 + r] : 0.0;
    const int q0 = rptr[r], q1 = active ? rptr[r + 1] : q0;
    const int glo = a.gdep_lo[c], ghi = a.gdep_hi[c];
    for (int l = 1; l <= a.nlevel; l++) {
      if (l > 1 && !pipe_wait(a, glo, ghi, l - 1, &s_abort)) return;
      const double *src = l == 1 ? a.x : a.vv + (long)(l - 1) * a.n;
      const double v = pipe_row_fp64<ARITH, VALUED>(q0, q1, cols, vals, cf, src);
      if (active) a.vv[(long)l * a.n + r0 + r] = v;
      pipe_publish(a, c, l);
    }
  }
}

// ------------------------------------------------------------------------
// Double-float ("df64") arithmetic on the FP32 pipes.  A value is an
// unevaluated sum h + l of two floats with |l| <= ulp(h)/2 after
// normalisation (48 significand bits).  Products use the exact FMA
// residual; sums use Knuth's TwoSum.  Intrinsics (__fmul_rn, __fadd_rn)
// keep the compiler from contracting the error-free transformations.
// FP64 <-> df64 conversions use integer bit manipulation so that they do
// not occupy the narrow FP64 pipe.
// ------------------------------------------------------------------------
__device__ __forceinline__ float2 df_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  const int E = e - 1023;
  const unsigned int sgn = (unsigned int)(b >> 63) << 31;
  if (e == 0x7FF || E > 127) {  // inf/nan or beyond the float range
    const float h = __double2float_rn(x);
    return make_float2(h, 0.0f);
  }
  if (E < -126) return make_float2(0.0f, 0.0f);  // below the df64 range
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  const float h = __uint_as_float(sgn | ((unsigned)(E + 127) << 23) | (unsigned)(m >> 29));
  const unsigned int rem = (unsigned int)(m & 0x1FFFFFFFull);  // low 29 bits, weight 2^(E-52)
  float lo = 0.0f;
  if (rem != 0 && E - 52 >= -126) {
    lo = __fmul_rn(__uint2float_rn(rem), __uint_as_float((unsigned)(E - 52 + 127) << 23));
    lo = __uint_as_float(__float_as_uint(lo) | sgn);
  }
  return make_float2(h, lo);
}

__device__ __forceinline__ double df_widen(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int e = (u >> 23) & 0xFF;
  if (e == 0) return __longlong_as_double((long long)((unsigned long long)(u >> 31) << 63));  // +-0
  if (e == 0xFF) return (double)f;
  return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) |
                                          ((unsigned long long)(e + 896) << 52) |
                                          ((unsigned long long)(u & 0x7FFFFF) << 29)));
}

__device__ __forceinline__ double df_to_double(float2 v) { return __dadd_rn(df_widen(v.x), df_widen(v.y)); }

// s += a * x in double-float
__device__ __forceinline__ void df_mac(float2 a, float2 x, float &sh, float &sl) {
  const float p = __fmul_rn(a.x, x.x);
  float e = __fmaf_rn(a.x, x.x, -p);
  e = __fmaf_rn(a.x, x.y, e);
  e = __fmaf_rn(a.y, x.x, e);
  const float s = __fadd_rn(sh, p);
  const float bp = __fadd_rn(s, -sh);
  const float t = __fadd_rn(__fadd_rn(sh, -__fadd_rn(s, -bp)), __fadd_rn(p, -bp));
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(t, e));
}

__device__ __forceinline__ float2 df_norm(float sh, float sl) {
  const float h = __fadd_rn(sh, sl);
  const float l = __fadd_rn(sl, -__fadd_rn(h, -sh));
  return make_float2(h, l);
}

// s += x in double-float (two-sum of the high parts, low parts added)
__device__ __forceinline__ void df_acc(float2 x, float &sh, float &sl) {
  const float s = __fadd_rn(sh, x.x);
  const float bp = __fadd_rn(s, -sh);
  const float t = __fadd_rn(__fadd_rn(sh, -__fadd_rn(s, -bp)), __fadd_rn(x.x, -bp));
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(t, x.y));
}

// a * v in double-float (v normalised)
__device__ __forceinline__ float2 df_scale(float2 a, float2 v) {
  const float p = __fmul_rn(a.x, v.x);
  float e = __fmaf_rn(a.x, v.x, -p);
  e = __fmaf_rn(a.x, v.y, e);
  e = __fmaf_rn(a.y, v.x, e);
  return df_norm(p, e);
}

// Pipeline in double-float: levels travel between chunks through a
// two-slot ring of df64 values (level l in slot l&1); vv receives the FP64
// rounding of every level.  Level 1 splits the gathered FP64 x values.  A
// slot is overwritten (level l+2) only after every chunk within reach has
// finished level l+1, i.e. no longer reads level l.
// One row sum in double-float over the entries [q0, q1) in CSR order.
template <bool VALUED>
__device__ __forceinline__ float2 pipe_row_df(int q0, int q1, const int *cols, const float2 *vals, float2 cf,
                                              const float2 *src) {
  float sh = 0.f, sl = 0.f;
  if (q1 - q0 <= 8) {
    float2 xv[8];
#pragma unroll
    for (int t = 0; t < 8; t++)
      if (q0 + t < q1) xv[t] = src[cols[q0 + t]];
#pragma unroll
    for (int t = 0; t < 8; t++)
      if (q0 + t < q1) df_mac(VALUED ? vals[q0 + t] : cf, xv[t], sh, sl);
  } else {
    for (int q = q0; q < q1; q++) df_mac(VALUED ? vals[q] : cf, src[cols[q]], sh, sl);
  }
  return df_norm(sh, sl);
}

// ------------------------------------------------------------------------
// Dataflow pipeline.  Work items are (chunk, level) pairs in a precomputed
// topological order: key = chunk + D*(level-1), D larger than the
// dependency reach, levels ascending within a key.  CTAs take items in
// ticket order; an item waits (bounded) until the chunks its rows read
// have published the previous level, computes its 256 rows straight from
// global memory (the matrix of recent chunks stays in L2) and publishes.
// Every dependency of an item has a smaller ticket and so belongs to a CTA
// that is already running: the schedule cannot deadlock, whatever the
// grid size, and no CTA sits idle holding a chunk.
// ------------------------------------------------------------------------
__device__ __forceinline__ int flow_next(const PipeArgs &a, int *s_t) {
  __syncthreads();
  const int t = *s_t;
  __syncthreads();
  if (t < a.nitems && threadIdx.x == 0) *s_t = (int)atomicAdd(a.ticket, 1u);  // prefetch
  return t;
}

template <int ARITH, bool VALUED>
__global__ void __launch_bounds__(kPipeThreads) flow_kernel(PipeArgs a) {
  __shared__ int s_t;
  __shared__ int s_abort;
  if (threadIdx.x == 0) {
    s_t = (int)atomicAdd(a.ticket, 1u);
    s_abort = 0;
  }
  for (;;) {
    const int t = flow_next(a, &s_t);
    if (t >= a.nitems) return;
    const int item = a.items[t];
    const int c = item & ((1 << 26) - 1), l = item >> 26;
    if (l > 1 && !pipe_wait(a, a.gdep_lo[c], a.gdep_hi[c], l - 1, &s_abort)) return;
    const int r = c * a.chunk + (int)threadIdx.x;
    if (r < a.n) {
      const int q0 = a.ptr[r], q1 = a.ptr[r + 1];
      const double cf = VALUED ? 0.0 : a.coef[r];
      const double *src = l == 1 ? a.x : a.vv + (long)(l - 1) * a.n;
      a.vv[(long)l * a.n + r] = pipe_row_fp64<ARITH, VALUED>(q0, q1, a.col, a.coef, cf, src);
    }
    pipe_publish(a, c, l);
  }
}

template <bool VALUED>
__global__ void __launch_bounds__(kPipeThreads, 6) flow_df_kernel(PipeArgs a) {
  __shared__ int s_t;
  __shared__ int s_abort;
  if (threadIdx.x == 0) {
    s_t = (int)atomicAdd(a.ticket, 1u);
    s_abort = 0;
  }
  for (;;) {
    const int t = flow_next(a, &s_t);
    if (t >= a.nitems) return;
    const int item = a.items[t];
    const int c = item & ((1 << 26) - 1), l = item >> 26;
    if (l > 1 && !pipe_wait(a, a.gdep_lo[c], a.gdep_hi[c], l - 1, &s_abort)) return;
    const int r = c * a.chunk + (int)threadIdx.x;
    if (r < a.n) {
      const int q0 = a.ptr[r], q1 = a.ptr[r + 1];
      const float2 cf = VALUED ? make_float2(0.f, 0.f) : a.coef2[r];
      float2 v;
      if (l == 1) {
        float sh = 0.f, sl = 0.f;
        for (int q = q0; q < q1; q++) df_mac(VALUED ? a.coef2[q] : cf, df_split(a.x[a.col[q]]), sh, sl);
        v = df_norm(sh, sl);
      } else {
        v = pipe_row_df<VALUED>(q0, q1, a.col, a.coef2, cf, a.ring + (long)((l - 1) & 1) * a.n);
      }
      a.ring[(long)(l & 1) * a.n + r] = v;
      a.vv[(long)l * a.n + r] = df_to_double(v);
    }
    pipe_publish(a, c, l);
  }
}

// PA1 tiles in double-float: same schedule as tiles_kernel, level buffers
// of float2 in shared memory.
template <bool VALUED>
__device__ __forceinline__ float2 tile_row_df(const TileArgs &a, const float2 *coef2, long sl, int lane, int co,
                                              const float2 *in) {
  const int w = a.ell_width[sl];
  const uint16_t *cp = a.ell_col + a.ell_off[sl] + lane;
  float sh = 0.f, slo = 0.f;
  if (w <= 8) {
    float2 xv[8], cv[8];
    bool ok[8];
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int c = t < w ? cp[t * 32] : 0xFFFF;
      ok[t] = c != 0xFFFF;
      xv[t] = ok[t] ? in[c] : make_float2(0.f, 0.f);
      cv[t] = (ok[t] && VALUED) ? coef2[co + t] : make_float2(0.f, 0.f);
    }
    const float2 cf = VALUED ? make_float2(0.f, 0.f) : coef2[co];
#pragma unroll
    for (int t = 0; t < 8; t++)
      if (ok[t]) df_mac(VALUED ? cv[t] : cf, xv[t], sh, slo);
  } else {
    const float2 cf = VALUED ? make_float2(0.f, 0.f) : coef2[co];
    for (int t = 0; t < w; t++) {
      const int c = cp[t * 32];
      if (c == 0xFFFF) break;
      df_mac(VALUED ? coef2[co + t] : cf, in[c], sh, slo);
    }
  }
  return df_norm(sh, slo);
}

template <bool VALUED, bool SMEM>
__global__ void __launch_bounds__(512) tiles_df_kernel(TileArgs a, const float2 *coef2) {
  extern __shared__ float2 smem_f2[];
  const int p = a.order[blockIdx.x];
  const long s0 = a.slot_off[p];
  const int ns = (int)(a.slot_off[p + 1] - s0);
  const int *shell = a.shell + (long)p * (a.nlevel + 1);
  const long sl0 = a.slice_off[p];
  float2 *buf0 = SMEM ? smem_f2 : reinterpret_cast<float2 *>(a.scratch) + (long)blockIdx.x * 2 * a.max_slots;
  float2 *buf1 = buf0 + a.max_slots;
  if (ns > a.max_slots) {
    if (threadIdx.x == 0) atomicExch(a.err, kErrBounds);
    return;
  }
  for (int s = threadIdx.x; s < ns; s += blockDim.x) buf0[s] = df_split(a.x[a.slot_vert[s0 + s]]);
  __syncthreads();
  const int owned = shell[0];
  for (int l = 1; l <= a.nlevel; l++) {
    const float2 *in = (l & 1) ? buf0 : buf1;
    float2 *out = (l & 1) ? buf1 : buf0;
    const int nrows = shell[a.nlevel - l];
    double *dst = a.vv + (long)l * a.n;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
      const float2 res = tile_row_df<VALUED>(a, coef2, sl0 + (r >> 5), r & 31, a.slot_coef[s0 + r], in);
      out[r] = res;
      if (r < owned) dst[a.slot_vert[s0 + r]] = df_to_double(res);
    }
    __syncthreads();
  }
}

// FP64 -> double-float conversion of a coefficient array (plan set-up).
__global__ void split_kernel(const double *__restrict__ src, float2 *__restrict__ dst, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = df_split(src[i]);
}

// ------------------------------------------------------------------------
// MPI-2 rank buffers on one GPU.  Every rank's vv_buf lives in one device
// array; a phase's computation is one launch with one CTA per rank (level
// segments separated by barriers, rows summed in CSR order), and the
// phase's MPI_Alltoallv (mpk2/mpi2_mpkexecbufs_val.c:32-48) becomes one
// gather: receive slot <- the sender's send-list entry.
// ------------------------------------------------------------------------
__global__ void gather_map_kernel(const double *__restrict__ src, const long *__restrict__ sidx,
                                  double *__restrict__ dst, const long *__restrict__ didx, long cnt) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < cnt; t += (long)gridDim.x * blockDim.x)
    dst[didx[t]] = src[sidx[t]];
}

template <int ARITH>
__global__ void __launch_bounds__(256) bufs_phase_kernel(int list_base, const long *__restrict__ list_seg,
                                                         const long *__restrict__ seg_off,
                                                         const long *__restrict__ row_dst,
                                                         const long *__restrict__ row_ptr,
                                                         const long *__restrict__ gcol,
                                                         const double *__restrict__ gval, double *vall) {
  const int list = list_base + blockIdx.x;
  for (long sg = list_seg[list]; sg < list_seg[list + 1]; sg++) {
    for (long q = seg_off[sg] + threadIdx.x; q < seg_off[sg + 1]; q += blockDim.x) {
      double s = 0.0;
      for (long j = row_ptr[q]; j < row_ptr[q + 1]; j++) s = row_term<ARITH>(s, gval[j], vall[gcol[j]]);
      vall[row_dst[q]] = s;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------
// Wavefront executor: one persistent (cooperative) launch; CTA b owns the
// contiguous rows [row_lo[b], row_lo[b+1]) (equal nonzeros) at every level
// and computes level l as soon as the CTAs owning the columns those rows
// read (the plan's exact list dep_idx[dep_ptr[b] ..)) have published level
// l-1.  No grid-wide barrier and no redundant rows; the matrix slices stay
// in L2 across levels.  FP64 levels are written to fresh addresses of vv;
// the double-float and fixed-point forms carry levels in a two-slot ring,
// reused two levels later only after the CTAs reading this CTA's rows have
// moved on (their flags are in the list too), and read after an acquire
// of the writers' flags, so L1 never serves a stale line.
// ------------------------------------------------------------------------
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }

struct WaveArgs {
  int n, nlevel, nblk;
  uint32_t base;               // flags of this call start at base (level l publishes base + l)
  uint32_t stall;              // test hook: extra levels to wait for (never published)
  // matrix in sliced ELL (32 rows per slice, entry t of row 32s+j at
  // sell_off[s] + 32t + j, CSR order within the row), so that a warp's
  // column and value loads are coalesced; columns as int16 offsets from
  // the row when every |col - row| < 32768, else int32
  const long *sell_off;        // nslice + 1
  const unsigned short *len;   // entries per row
  const int *scol;             // column of each slot (int32 form) ...
  const short *srel;           // ... or col - row (int16 form), pattern-compressed: a slice whose 32
                               // rows share one offset list stores it once (runi != 0, padded to 8)
  const long *rel_off;         // nslice + 1: start of each slice in srel
  const unsigned char *runi;   // per slice: 0 = per-lane offsets; else a shared offset list, and
                               // 1 + the rows' common length (255: read the lengths)
  const double *sval;          // value of each slot (valued) ...
  const float2 *sval2;         // ... or its double-float split
  const double *rdeg;          // 1/deg per row (1/deg operator) ...
  const float2 *rdeg2;         // ... or its double-float split
  const double *lut;           // 1/d for d < 256 (exactly the rows' 1/deg) ...
  const float2 *lut2;          // ... and its double-float split
  double *vv;
  float2 *ring;                // 2 * n: double-float copies of levels l-1 and l
  int stage_rel_bytes;         // > 0: the CTA's int16 offsets and lengths are staged in shared memory
                               // once per call (offsets first, this many bytes, then the lengths,
  int stage_len_bytes;         // this many bytes, then per slice its start (int) and flag (byte),
  int stage_slices;            // room for this many slices)
  const int *row_lo;           // nblk + 1
  const int *dep_ptr;          // nblk + 1: CTA b waits for dep_idx[dep_ptr[b] .. dep_ptr[b+1]):
  const int *dep_idx;          // the other CTAs owning columns of its rows (and, for the ring
                               // forms, those reading its rows)
  unsigned int *flags;         // per CTA: last level published
  int *err;
  // fixed-point form (1/deg operator): the ring holds int64 values v * 2^S
  const unsigned long long *fix_mul;  // 256: ceil(2^64 / d), d >= 2
  unsigned long long *fix_word;       // per call: (base << 32) | largest biased exponent of |x|
  int fix_dbits;                      // ceil(log2(longest row))
  // mixed form: the values are larger than L2, so they are loaded
  // evict-first (they would only push the level vectors out of L2)
  int stream_vals;
  // FP64 forms, host execution on page-locked vv: the caller's vv through
  // its host mapping (x read from it, every level written to it as well as
  // to the device copy the next level reads); null otherwise
  double *hv;
};

__device__ __forceinline__ bool wave_wait(const WaveArgs &a, int b, unsigned int want, int *s_abort) {
  const int lo = a.dep_ptr[b], hi = a.dep_ptr[b + 1];
  for (int k = lo + (int)threadIdx.x; k < hi; k += blockDim.x) {
    const int c = a.dep_idx[k];
    long spins = 0;
    while (ld_acquire(a.flags + c) < want + a.stall) {
      if (++spins > kSpinLimit || *((volatile int *)a.err)) {
        atomicCAS(a.err, 0, kErrTimeout);
        *s_abort = 1;
        break;
      }
      __nanosleep(spins < 16 ? 32 : 256);
    }
  }
  __syncthreads();
  return *s_abort == 0;
}

// Release of a CTA's level: the barrier orders the CTA's row writes before
// thread 0's store, and the store's release (a GPU-scope acq_rel fence
// followed by the store) is cumulative over them, so no separate fence.
__device__ __forceinline__ void wave_publish(const WaveArgs &a, int b, unsigned int v) {
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a.flags + b), "r"(v) : "memory");
  }
}

// Copies the CTA's slab of int16 offsets (whole slices, 64-byte aligned) and
// its rows' lengths into shared memory; the CTA owns the same rows at every
// level, so this happens once per call.
__device__ __forceinline__ void wave_stage(const WaveArgs &a, int r0, int r1, unsigned char *smem) {
  if (r0 >= r1) return;
  const long e_lo = a.rel_off[r0 >> 5], e_hi = a.rel_off[(r1 + 31) >> 5];
  const int4 *g = reinterpret_cast<const int4 *>(a.srel + e_lo);
  int4 *d = reinterpret_cast<int4 *>(smem);
  const long nvec = (e_hi - e_lo) / 8;  // every slice holds a multiple of 8 offsets
  for (long v = threadIdx.x; v < nvec; v += blockDim.x) d[v] = __ldg(g + v);
  unsigned char *sl = smem + a.stage_rel_bytes;  // staged rows are at most 255 long
  for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x) sl[i - r0] = (unsigned char)__ldg(a.len + i);
  // per slice of the range: start in the slab (relative) and the shared-list flag
  const int s0 = r0 >> 5, ns = ((r1 + 31) >> 5) - s0;
  int *srs = reinterpret_cast<int *>(smem + a.stage_rel_bytes + a.stage_len_bytes);
  unsigned char *sus = reinterpret_cast<unsigned char *>(srs + a.stage_slices);
  for (int k = threadIdx.x; k < ns; k += blockDim.x) {
    srs[k] = (int)(a.rel_off[s0 + k] - e_lo);
    sus[k] = a.runi[s0 + k];
  }
}

// An int16 offset from the staged slab (shared memory: plain load) or
// from global memory (read-only path).  __ldg must never see a shared
// address.
template <bool STAGE>
__device__ __forceinline__ int ld_off(const short *p) {
  if (STAGE) return (int)*p;
  return (int)__ldg(p);
}

// One row's sum over its entries (CSR order): the row's int16 offsets are
// RS apart (32: per-lane layout, a constant after inlining; 1: a slice's
// shared list), values and int32 columns 32 apart.  Up to 8 (12 for FP32) entries have all their
// loads in flight together.
template <int ARITH, bool VALUED, bool REL, bool STAGE>
__device__ __forceinline__ double fp_row(int len, int RS, double cf, const short *cr, const int *cc,
                                         const double *cv, const double *xb, const double *src) {
  double s = 0.0;
  int t = 0;
  if (len <= 8) {
    double x[8], v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      if (u < len) {
        x[u] = REL ? xb[ld_off<STAGE>(cr + RS * u)] : src[__ldg(cc + 32 * u)];
        v[u] = VALUED ? __ldg(cv + 32 * u) : cf;
      }
    }
#pragma unroll
    for (int u = 0; u < 8; u++)
      if (u < len) s = row_term<ARITH>(s, v[u], x[u]);
    t = len;
  }
  for (; t < len; t++)
    s = row_term<ARITH>(s, VALUED ? __ldg(cv + 32L * t) : cf,
                        REL ? xb[ld_off<STAGE>(cr + RS * t)] : src[__ldg(cc + 32L * t)]);
  return s;
}

template <bool VALUED, bool REL, bool STAGE>
__device__ __forceinline__ void df_row(int len, int RS, const short *cr, const int *cc, const float2 *cv,
                                       const float2 *xb, const float2 *src, float &sh, float &sl_) {
  int t = 0;
  if (len <= 8) {
    float2 x[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      if (u < len) x[u] = REL ? xb[ld_off<STAGE>(cr + RS * u)] : src[__ldg(cc + 32 * u)];
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      if (u < len) {
        if (VALUED) df_mac(cv[32 * u], x[u], sh, sl_);
        else df_acc(x[u], sh, sl_);
      }
    }
    t = len;
  }
  for (; t < len; t++) {
    const float2 x = REL ? xb[ld_off<STAGE>(cr + RS * t)] : src[__ldg(cc + 32L * t)];
    if (VALUED) df_mac(cv[32L * t], x, sh, sl_);
    else df_acc(x, sh, sl_);
  }
}

template <bool STREAM, typename VT>
__device__ __forceinline__ VT ld_val(const VT *p) {
  if (STREAM) return __ldcs(p);
  return __ldg(p);
}

template <typename VT, bool REL, bool STREAM>
__device__ __forceinline__ float mix_row(int len, int RS, const short *cr, const int *cc, const VT *cv,
                                         const float *xb, const float *src) {
  float s = 0.f;
  int t = 0;
  if (len <= 12) {
    float x[12], v[12];
#pragma unroll
    for (int u = 0; u < 12; u++) {
      if (u < len) {
        x[u] = REL ? xb[__ldg(cr + RS * u)] : src[__ldg(cc + 32 * u)];
        v[u] = to_f32(ld_val<STREAM>(cv + 32 * u));
      }
    }
#pragma unroll
    for (int u = 0; u < 12; u++)
      if (u < len) s = __fmaf_rn(v[u], x[u], s);
    t = len;
  }
  for (; t < len; t++)
    s = __fmaf_rn(to_f32(ld_val<STREAM>(cv + 32L * t)), REL ? xb[__ldg(cr + RS * t)] : src[__ldg(cc + 32L * t)], s);
  return s;
}

constexpr int kWaveXGroups = 8;  // host execution: CTA groups that copy x in turn

// FP64 rows (fma or separate multiply/add, CSR order as the reference).
// A warp computes one 32-row slice; CTA row ranges start on slices.  The
// previous level is read from vv: every address of it is fresh in this
// launch, so L1 holds no stale copy.
template <int ARITH, bool VALUED, bool REL, bool STAGE, bool UNI>
__global__ void __launch_bounds__(256, 4) wave_kernel(WaveArgs a) {
  extern __shared__ __align__(16) unsigned char wave_smem[];
  __shared__ int s_abort;
  __shared__ double s_lut[256];
  if (threadIdx.x == 0) s_abort = 0;
  if (!VALUED) s_lut[threadIdx.x] = a.lut[threadIdx.x];
  const int b = blockIdx.x, r0 = a.row_lo[b], r1 = a.row_lo[b + 1];
  if (STAGE) wave_stage(a, r0, r1, wave_smem);
  __syncthreads();
  const short *s_rel = reinterpret_cast<const short *>(wave_smem);
  const unsigned char *s_len = wave_smem + a.stage_rel_bytes;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (a.hv) {  // x from the host mapping into the device copy, own rows
    // in kWaveXGroups groups of CTAs taken in order: group g copies once
    // group g-1 has published level 0, so the first groups' levels already
    // travel down the host link (which carries both directions at once)
    // while the later groups' x still travels up
    const int grp = (int)((long)b * kWaveXGroups / a.nblk);
    if (grp > 0) {
      const int c0 = (int)(((long)(grp - 1) * a.nblk + kWaveXGroups - 1) / kWaveXGroups);
      const int c1 = (int)(((long)grp * a.nblk + kWaveXGroups - 1) / kWaveXGroups);
      for (int c = c0 + (int)threadIdx.x; c < c1; c += blockDim.x) {
        long spins = 0;
        while (ld_acquire(a.flags + c) < a.base + a.stall) {
          if (++spins > kSpinLimit || *((volatile int *)a.err)) {
            atomicCAS(a.err, 0, kErrTimeout);
            s_abort = 1;
            break;
          }
          __nanosleep(spins < 16 ? 32 : 256);
        }
      }
      __syncthreads();
      if (s_abort) return;
    }
    for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x) a.vv[i] = a.hv[i];
    wave_publish(a, b, a.base);
  }
  for (int l = 1; l <= a.nlevel; l++) {
    if ((l > 1 || a.hv) && !wave_wait(a, b, a.base + (unsigned)(l - 1), &s_abort)) return;
    const double *src = a.vv + (size_t)(l - 1) * a.n;
    double *dst = a.vv + (size_t)l * a.n;
    double *hdst = a.hv ? a.hv + (size_t)l * a.n : nullptr;
    for (int sl = (r0 >> 5) + warp; r0 < r1 && (sl << 5) < r1; sl += nw) {
      const int i = (sl << 5) + lane;
      if (i >= r1) continue;
      const int len = STAGE ? s_len[i - r0] : __ldg(a.len + i);
      const long e0 = __ldg(a.sell_off + sl) + lane;
      const double cf = VALUED ? 0.0 : (len < 256 ? s_lut[len] : __ldg(a.rdeg + i));
      const int *s_srs = reinterpret_cast<const int *>(wave_smem + a.stage_rel_bytes + a.stage_len_bytes);
      const unsigned char *s_sus = reinterpret_cast<const unsigned char *>(s_srs + a.stage_slices);
      const int k_sl = sl - (r0 >> 5);
      const bool uni = UNI && REL && (STAGE ? s_sus[k_sl] != 0 : __ldg(a.runi + sl) != 0);
      const short *cr = (STAGE ? s_rel + s_srs[k_sl] : a.srel + (REL ? __ldg(a.rel_off + sl) : 0)) + (uni ? 0 : lane);
      const int *cc = a.scol + e0;
      const double *cv = a.sval + e0;
      const double *xb = src + i;
      // the stride is the constant 32 unless the plan compresses offsets
      const double s = fp_row<ARITH, VALUED, REL, STAGE>(len, UNI ? (uni ? 1 : 32) : 32, cf, cr, cc, cv, xb, src);
      __stcs(dst + i, s);
      if (hdst) hdst[i] = s;
    }
    wave_publish(a, b, a.base + (unsigned)l);
  }
}

// Double-float rows.  1/deg operator: the row's values are summed in
// double-float, then scaled once by 1/deg; valued operator: double-float
// multiply-add per entry.  Levels travel through a two-slot ring of
// double-float copies (level l in slot l&1); a CTA overwrites a slot only
// after every CTA that reads its rows has finished the level before, which
// the symmetric dependency ranges guarantee.  Level 0 splits the CTA's
// own rows of x.
template <bool VALUED, bool REL, bool STAGE, bool UNI>
__global__ void __launch_bounds__(256, 5) wave_df_kernel(WaveArgs a) {
  extern __shared__ __align__(16) unsigned char wave_smem[];
  __shared__ int s_abort;
  __shared__ float2 s_lut[256];
  if (threadIdx.x == 0) s_abort = 0;
  if (!VALUED) s_lut[threadIdx.x] = a.lut2[threadIdx.x];
  const int b = blockIdx.x, r0 = a.row_lo[b], r1 = a.row_lo[b + 1];
  if (STAGE) wave_stage(a, r0, r1, wave_smem);
  __syncthreads();
  const short *s_rel = reinterpret_cast<const short *>(wave_smem);
  const unsigned char *s_len = wave_smem + a.stage_rel_bytes;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x) a.ring[i] = df_split(a.vv[i]);
  wave_publish(a, b, a.base);
  for (int l = 1; l <= a.nlevel; l++) {
    if (!wave_wait(a, b, a.base + (unsigned)(l - 1), &s_abort)) return;
    const float2 *src = a.ring + (size_t)((l - 1) & 1) * a.n;
    float2 *sdst = a.ring + (size_t)(l & 1) * a.n;
    double *dst = a.vv + (size_t)l * a.n;
    for (int sl = (r0 >> 5) + warp; r0 < r1 && (sl << 5) < r1; sl += nw) {
      const int i = (sl << 5) + lane;
      if (i >= r1) continue;
      const int len = STAGE ? s_len[i - r0] : __ldg(a.len + i);
      const long e0 = __ldg(a.sell_off + sl) + lane;
      const int *s_srs = reinterpret_cast<const int *>(wave_smem + a.stage_rel_bytes + a.stage_len_bytes);
      const unsigned char *s_sus = reinterpret_cast<const unsigned char *>(s_srs + a.stage_slices);
      const int k_sl = sl - (r0 >> 5);
      const bool uni = UNI && REL && (STAGE ? s_sus[k_sl] != 0 : __ldg(a.runi + sl) != 0);
      const short *cr = (STAGE ? s_rel + s_srs[k_sl] : a.srel + (REL ? __ldg(a.rel_off + sl) : 0)) + (uni ? 0 : lane);
      // per-lane bases: slot t of this row is 32*t elements further (the
      // offsets of a shared-list slice: t further), an immediate offset
      const int *cc = a.scol + e0;
      const float2 *cv = a.sval2 + e0;
      const float2 *xb = src + i;
      float sh = 0.f, sl_ = 0.f;
      // the stride is the constant 32 unless the plan compresses offsets
      df_row<VALUED, REL, STAGE>(len, UNI ? (uni ? 1 : 32) : 32, cr, cc, cv, xb, src, sh, sl_);
      float2 v = df_norm(sh, sl_);
      if (!VALUED) v = df_scale(len < 256 ? s_lut[len] : a.rdeg2[i], v);
      sdst[i] = v;
      __stcs(dst + i, df_to_double(v));
    }
    wave_publish(a, b, a.base + (unsigned)l);
  }
}

// 64-bit fixed-point rows for the 1/deg operator.  The operator averages
// (|A^l x| <= max|x| entrywise), so one scale 2^S fixed per call keeps every
// level exact to 2^-S: S = 62 - ceil(log2(longest row)) - e, max|x| < 2^e,
// which leaves room for the row sums.  A row is then an exact int64 sum of
// its neighbours, one division by its length (reciprocal multiply, within
// one unit) and one conversion to FP64.  The error against FP64 is about
// 2^-S relative to max|x| per level.  Phase A agrees on e across the grid
// (all CTAs are resident), phase B converts x, then levels 1..k follow
// the wavefront rule.  Tags of a call: base (e published), base + 1 (x
// converted), base + 1 + l (level l).
__device__ __forceinline__ long long fix_div(long long s, int d, unsigned long long m) {
  if (d <= 1) return s;
  const unsigned long long t = (unsigned long long)(s < 0 ? -s : s) + (unsigned long long)(d >> 1);
  const long long q = (long long)__umul64hi(t, m);
  return s < 0 ? -q : q;
}

// q * 2^-S rounded to nearest-even in integer arithmetic (the FP64 pipe's
// conversions are scarce on this part).  |q| < 2^63 and q * 2^-S stays a
// normal double for every S the kernel uses (S <= 1022, |q| >= 1).
__device__ __forceinline__ double fix_to_double(long long q, int S) {
  if (q == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)q & 0x8000000000000000ull;
  const unsigned long long m = q < 0 ? 0ull - (unsigned long long)q : (unsigned long long)q;
  const int lz = __clzll((long long)m);
  const unsigned long long t = m << lz;  // leading one at bit 63
  unsigned long long mant = t >> 11;     // 53 bits, implicit one at bit 52
  const unsigned int rem = (unsigned int)(t & 0x7FFu);
  mant += (rem > 0x400u || (rem == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
  // the implicit one adds 1 to the exponent field (a carry to 2^53 adds one more)
  return __longlong_as_double((long long)(sgn | (((unsigned long long)(1022 + 63 - lz - S) << 52) + mant)));
}

// x * 2^S rounded to the nearest integer, ties to even, in integer
// arithmetic.  |x| * 2^S < 2^62 for every x of the call (S is chosen so).
__device__ __forceinline__ long long double_to_fix(double x, int S) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (e ? 0x10000000000000ull : 0ull);
  const int sh = (e ? e - 1075 : -1074) + S;  // x * 2^S = m * 2^sh
  unsigned long long q;
  if (sh >= 0) {
    q = m << sh;
  } else if (sh < -54) {
    q = 0;  // below 1/2
  } else {
    const int r = -sh;
    q = m >> r;
    const unsigned long long rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
    q += (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
  }
  return (long long)(b >> 63 ? 0ull - q : q);
}

// ------------------------------------------------------------------------
// k separate SpMV launches in the wavefront's other arithmetic forms (the
// "k SpMVs" baseline of mpk2/spmvexec.c:8-50 in the same arithmetic as the
// MPK it is compared with): one thread per CSR row per level, levels kept
// in a two-slot device ring like the wavefront's, FP64 results written to
// vv.  Double-float: the rows of wave_df_kernel; fixed point: the rows of
// wave_fix_kernel with the scale chosen from max|x| per call.
// ------------------------------------------------------------------------
template <bool VALUED>
__global__ void __launch_bounds__(256) spmv_df_kernel(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                                                      const float2 *__restrict__ coef2, const float2 *src,
                                                      float2 *sdst, double *__restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float sh = 0.f, sl = 0.f;
  const int j0 = ptr[i], j1 = ptr[i + 1];
  for (int j = j0; j < j1; j++) {
    const float2 x = src[col[j]];
    if (VALUED) df_mac(coef2[j], x, sh, sl);
    else df_acc(x, sh, sl);
  }
  float2 v = df_norm(sh, sl);
  if (!VALUED) v = df_scale(coef2[i], v);
  sdst[i] = v;
  y[i] = df_to_double(v);
}

__global__ void fix_emax_kernel(int n, const double *__restrict__ x, unsigned int *word) {
  int e = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    e = max(e, (int)(((unsigned long long)__double_as_longlong(x[i]) >> 52) & 0x7FF));
  e = (int)__reduce_max_sync(0xFFFFFFFFu, (unsigned)e);
  if ((threadIdx.x & 31) == 0) atomicMax(word, (unsigned)e);
}

// word[0]: the largest biased exponent of |x|; word[1] receives S
__global__ void fix_convert_kernel(int n, const double *__restrict__ x, unsigned int *word, int dbits,
                                   long long *__restrict__ ring) {
  const int emax = (int)word[0] - 1022;  // max|x| < 2^emax
  const int S = min(62 - dbits - emax, 1022);
  if (blockIdx.x == 0 && threadIdx.x == 0) word[1] = (unsigned)S;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    ring[i] = double_to_fix(x[i], S);
}

__global__ void __launch_bounds__(256) spmv_fix_kernel(int n, const int *__restrict__ ptr,
                                                       const int *__restrict__ col,
                                                       const unsigned long long *__restrict__ mul,
                                                       const unsigned int *__restrict__ word, const long long *src,
                                                       long long *dst, double *__restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int S = (int)word[1];
  const int j0 = ptr[i], len = ptr[i + 1] - j0;
  long long sum = 0;
  for (int j = 0; j < len; j++) sum += src[col[j0 + j]];
  const long long q = fix_div(sum, len, mul[len & 255]);
  dst[i] = q;
  y[i] = fix_to_double(q, S);
}

template <bool STAGE>
__global__ void __launch_bounds__(256, 5) wave_fix_kernel(WaveArgs a) {
  extern __shared__ __align__(16) unsigned char wave_smem[];
  __shared__ int s_abort, s_emax;
  __shared__ unsigned long long s_mul[256];
  if (threadIdx.x == 0) { s_abort = 0; s_emax = 0; }
  s_mul[threadIdx.x] = a.fix_mul[threadIdx.x];
  const int b = blockIdx.x, r0 = a.row_lo[b], r1 = a.row_lo[b + 1];
  if (STAGE) wave_stage(a, r0, r1, wave_smem);
  __syncthreads();
  const short *s_rel = reinterpret_cast<const short *>(wave_smem);
  const unsigned char *s_len = wave_smem + a.stage_rel_bytes;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long *ring = reinterpret_cast<long long *>(a.ring);
  // phase A: the largest exponent of |x| over the grid
  int e = 0;
  for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x)
    e = max(e, (int)(((unsigned long long)__double_as_longlong(a.vv[i]) >> 52) & 0x7FF));
  e = (int)__reduce_max_sync(0xFFFFFFFFu, (unsigned)e);
  if ((threadIdx.x & 31) == 0) atomicMax(&s_emax, e);
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(a.fix_word, ((unsigned long long)a.base << 32) | (unsigned)s_emax);
  wave_publish(a, b, a.base);
  for (int c = (int)threadIdx.x; c < a.nblk; c += blockDim.x) {  // every CTA has contributed
    long spins = 0;
    while (ld_acquire(a.flags + c) < a.base + a.stall) {
      if (++spins > kSpinLimit || *((volatile int *)a.err)) {
        atomicCAS(a.err, 0, kErrTimeout);
        s_abort = 1;
        break;
      }
      __nanosleep(spins < 16 ? 32 : 256);
    }
  }
  __syncthreads();
  if (s_abort) return;
  // one read of the grid maximum per CTA (the acquire loads above order it
  // after every CTA's atomicMax), broadcast through shared memory
  if (threadIdx.x == 0) s_emax = (int)(atomicOr(a.fix_word, 0ull) & 0xFFFFFFFFull);
  __syncthreads();
  const int emax = s_emax - 1022;  // max|x| < 2^emax
  const int S = min(62 - a.fix_dbits - emax, 1022);
  // phase B: x in fixed point
  for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x) ring[i] = double_to_fix(a.vv[i], S);
  wave_publish(a, b, a.base + 1);
  for (int l = 1; l <= a.nlevel; l++) {
    if (!wave_wait(a, b, a.base + (unsigned)l, &s_abort)) return;
    const long long *src = ring + (size_t)((l - 1) & 1) * a.n;
    long long *sdst = ring + (size_t)(l & 1) * a.n;
    double *dst = a.vv + (size_t)l * a.n;
    for (int sl = (r0 >> 5) + warp; r0 < r1 && (sl << 5) < r1; sl += nw) {
      const int i = (sl << 5) + lane;
      if (i >= r1) continue;
      const int len = STAGE ? s_len[i - r0] : __ldg(a.len + i);
      const int *s_srs = reinterpret_cast<const int *>(wave_smem + a.stage_rel_bytes + a.stage_len_bytes);
      const int k_sl = sl - (r0 >> 5);
      const short *cr = (STAGE ? s_rel + s_srs[k_sl] : a.srel + __ldg(a.rel_off + sl)) + lane;
      const long long *xb = src + i;
      long long sum = 0;
      int t = 0;
      if (len <= 8) {
        long long x[8];
#pragma unroll
        for (int u = 0; u < 8; u++)
          if (u < len) x[u] = xb[ld_off<STAGE>(cr + 32 * u)];
#pragma unroll
        for (int u = 0; u < 8; u++)
          if (u < len) sum += x[u];
        t = len;
      }
      for (; t < len; t++) sum += xb[ld_off<STAGE>(cr + 32L * t)];
      const long long q = fix_div(sum, len, s_mul[len & 255]);
      sdst[i] = q;
      __stcs(dst + i, fix_to_double(q, S));
    }
    wave_publish(a, b, a.base + 1 + (unsigned)l);
  }
}

// Mixed-precision rows on the wavefront schedule: FP32 or BF16 values in
// the sliced layout, FP32 basis, FP32 FMA in CSR order from 0, each level
// scaled by the exact power of two `scale` (the same arithmetic as
// mix_pipe_kernel, so both give identical bits).  Levels live at fresh
// addresses of the FP32 vv.
template <typename VT, bool REL, bool UNI, bool STREAM>
__global__ void __launch_bounds__(256, 5) wave_mix_kernel(WaveArgs a, const VT *__restrict__ sv, float *vf, float scale) {
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = 0;
  __syncthreads();
  const int b = blockIdx.x, r0 = a.row_lo[b], r1 = a.row_lo[b + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int l = 1; l <= a.nlevel; l++) {
    if (l > 1 && !wave_wait(a, b, a.base + (unsigned)(l - 1), &s_abort)) return;
    const float *src = vf + (size_t)(l - 1) * a.n;
    float *dst = vf + (size_t)l * a.n;
    for (int sl = (r0 >> 5) + warp; r0 < r1 && (sl << 5) < r1; sl += nw) {
      const int i = (sl << 5) + lane;
      if (i >= r1) continue;
      // a shared-list slice carries its rows' common length in runi: the
      // streaming build takes it from there (less HBM traffic, but the
      // other slices' length loads wait for runi); the other loads both
      int len;
      bool uni;
      if (STREAM) {
        const int ru = UNI && REL ? __ldg(a.runi + sl) : 0;
        uni = ru != 0;
        len = ru != 0 && ru != 255 ? ru - 1 : __ldg(a.len + i);
      } else {
        len = __ldg(a.len + i);
        uni = UNI && REL && __ldg(a.runi + sl);
      }
      const long e0 = __ldg(a.sell_off + sl) + lane;
      const short *cr = a.srel + (REL ? __ldg(a.rel_off + sl) : 0) + (uni ? 0 : lane);
      const int *cc = a.scol + e0;
      const VT *cv = sv + e0;
      const float *xb = src + i;
      // one loop for both offset layouts (a runtime stride keeps the
      // registers of a single copy of the 12-wide body)
      const float s = mix_row<VT, REL, STREAM>(len, UNI && uni ? 1 : 32, cr, cc, cv, xb, src);
      __stcs(dst + i, s * scale);
    }
    wave_publish(a, b, a.base + (unsigned)l);
  }
}

// ------------------------------------------------------------------------
// Mixed-precision PA1 tiles: temporal blocking for matrices larger than L2
// (the reference's PA1 diamond schedule, mpk2/mpkprep.c:186-233, run in
// FP32).  A tile is a part plus every vertex within nlevel arcs, its slots
// sorted by (distance, vertex), so the rows of level l are the prefix
// with distance <= nlevel - l.  A persistent CTA takes tiles in the plan's
// order from a ticket and, per tile:
//   * gathers the tile's level-0 values into shared memory (the halo read
//     that replaces the reference's MPI exchange);
//   * loads the local columns and the values of its rows ONCE into
//     registers (thread t owns rows t and t + kTmThreads of every level),
//     so the matrix is read once for all nlevel levels;
//   * computes the levels in place, ping-ponging two shared-memory
//     vectors, recomputing the skirt rows, and writes the part's own rows
//     of each level to vv.
// Rows beyond the registers' reach, or wider than W entries, read their
// columns and values again at each level (L2 hits).  Row sums: FP32 FMA in
// CSR order, then the exact scaling by 2^-e: the bits of the wavefront and
// pipeline mixed forms.
// ------------------------------------------------------------------------
struct TileMixArgs {
  int n, nlevel, npart, max_slots;
  const int *order;          // tiles in launch order
  const long *slot_off;      // per tile: first slot (npart + 1)
  const int *shell;          // per tile: (nlevel + 1) prefix counts by distance
  const int *slot_vert;      // vertex of each slot
  const int *slot_coef;      // CSR offset of each slot's row
  const long *slice_off;     // per tile: first slice
  const long *ell_off;       // per slice: first entry
  const uint16_t *ell_col;   // local slot of each entry, 0xFFFF = padding
  const uint8_t *ell_width;  // per slice
  const void *val;           // CSR values, float or __nv_bfloat16
  const float *x;            // level 0 (vf[0..n))
  float *vf;                 // (nlevel + 1) * n
  float scale;               // 2^-e
  unsigned int *ticket;
  int *err;
};

constexpr int kTmThreads = 1024;
constexpr int kTmRows = 2;  // rows per thread held in registers

// A row read from global memory (no register copy): columns of the
// tile-local ELL, values from the CSR.
template <typename VT>
__device__ __forceinline__ float tm_row_global(const TileMixArgs &a, const VT *val, long sl, int lane, int co,
                                               const float *in) {
  const int w = a.ell_width[sl];
  const uint16_t *cp = a.ell_col + a.ell_off[sl] + lane;
  float s = 0.f;
  for (int t = 0; t < w; t++) {
    const int c = cp[32 * t];
    if (c == 0xFFFF) break;
    s = __fmaf_rn(to_f32(val[co + t]), in[c], s);
  }
  return s;
}

template <typename VT, int W>
__global__ void __launch_bounds__(kTmThreads, 1) tiles_mix_kernel(TileMixArgs a) {
  extern __shared__ __align__(16) float tm_buf[];
  __shared__ int s_q, s_nrows[32];
  float *buf0 = tm_buf, *buf1 = tm_buf + a.max_slots;
  const VT *val = static_cast<const VT *>(a.val);
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();  // the previous tile's buffers and s_q are free
    if (tid == 0) s_q = (int)atomicAdd(a.ticket, 1u);
    __syncthreads();
    const int q = s_q;
    if (q >= a.npart) return;
    const int p = a.order[q];
    const long s0 = a.slot_off[p];
    const int ns = (int)(a.slot_off[p + 1] - s0);
    if (ns > a.max_slots) {  // plan invariant; never true for a valid plan
      if (tid == 0) atomicExch(a.err, kErrBounds);
      return;
    }
    const int *shell = a.shell + (long)p * (a.nlevel + 1);
    const long sl0 = a.slice_off[p];
    const int nrow1 = a.nlevel >= 1 ? shell[a.nlevel - 1] : 0;
    for (int sv = tid; sv < ns; sv += kTmThreads) buf0[sv] = __ldg(a.x + a.slot_vert[s0 + sv]);
    // this thread's rows: columns (two per word) and values in registers
    uint32_t cw[kTmRows][(W + 1) / 2];
    float v[kTmRows][W];
    int len[kTmRows], vert[kTmRows];
    const int owned = shell[0];
#pragma unroll
    for (int j = 0; j < kTmRows; j++) {
      len[j] = -1;
      const int r = tid + j * kTmThreads;
      vert[j] = r < owned ? a.slot_vert[s0 + r] : 0;  // the part's own rows are written at every level
#pragma unroll
      for (int t = 0; t < (W + 1) / 2; t++) cw[j][t] = 0;
#pragma unroll
      for (int t = 0; t < W; t++) v[j][t] = 0.f;
      if (r < nrow1) {
        const long sl = sl0 + (r >> 5);
        const int w = a.ell_width[sl];
        if (w <= W) {
          const uint16_t *cp = a.ell_col + a.ell_off[sl] + (r & 31);
          const int co = a.slot_coef[s0 + r];
          int L = 0;
#pragma unroll
          for (int t = 0; t < W; t++) {
            const int c = t < w ? (int)__ldg(cp + 32 * t) : 0xFFFF;
            if (c != 0xFFFF && L == t) {
              cw[j][t >> 1] |= (uint32_t)c << (16 * (t & 1));
              v[j][t] = to_f32(val[co + t]);
              L = t + 1;
            }
          }
          len[j] = L;
        }
      }
    }
    if (tid >= 1 && tid <= a.nlevel) s_nrows[tid] = shell[a.nlevel - tid];  // rows of each level
    __syncthreads();
    for (int l = 1; l <= a.nlevel; l++) {
      const float *in = (l & 1) ? buf0 : buf1;
      float *out = (l & 1) ? buf1 : buf0;
      const int nrows = s_nrows[l];
      float *dst = a.vf + (size_t)l * a.n;
#pragma unroll
      for (int j = 0; j < kTmRows; j++) {
        const int r = tid + j * kTmThreads;
        if (r < nrows) {
          float s = 0.f;
          if (len[j] >= 0) {
#pragma unroll
            for (int t = 0; t < W; t++)
              if (t < len[j]) s = __fmaf_rn(v[j][t], in[(cw[j][t >> 1] >> (16 * (t & 1))) & 0xFFFF], s);
          } else {
            s = tm_row_global(a, val, sl0 + (r >> 5), r & 31, a.slot_coef[s0 + r], in);
          }
          s *= a.scale;
          out[r] = s;
          if (r < owned) __stcs(dst + vert[j], s);
        }
      }
      for (int r = tid + kTmRows * kTmThreads; r < nrows; r += kTmThreads) {
        float s = tm_row_global(a, val, sl0 + (r >> 5), r & 31, a.slot_coef[s0 + r], in);
        s *= a.scale;
        out[r] = s;
        if (r < owned) __stcs(dst + a.slot_vert[s0 + r], s);
      }
      __syncthreads();
    }
  }
}

// ------------------------------------------------------------------------
// Register-resident PA1 tiles (the mixed form's temporal blocking for
// tiles of at most kTrThreads * kTrRows computed rows).  A tile's slot s
// lives in the level buffers at position (s & ~31) | ((s + rot) & 31), rot
// chosen per 32-slot group by the plan so that the 32 gathers of one
// warp-wide load fall into distinct shared-memory banks as far as it can.
// The plan writes each tile as two contiguous, 16-byte aligned images in
// execution order,
//   vert image:   header (positions, nrow1, owned, nslice, shells
//                 c_0..c_nlevel, rotation count at [31]), the rotation of
//                 every 32-slot group, then the vertex at every position
//                 (-1 where no slot sits),
//   matrix image: [slice][t / 2][lane] pairs of byte offsets of the local
//                 columns' positions (uint16 each, position * 4; entry t in
//                 half t & 1 of the word) then [slice][t][lane]
//                 values, every row padded to W entries with value -0 and
//                 the zero position,
// so a tile is two bulk copies.  Thread t holds rows t, t + T, t + 2T of
// every level in registers (value and byte offset per entry), so an entry
// costs one shared-memory gather and one FMA.  While a tile computes its
// levels, the next tile's images stream in (TMA bulk copies on two
// mbarriers) and, once its vertices have landed, its level-0 x is gathered
// into a third buffer (cp.async), copied into the first level buffer when
// that tile starts.  Padding entries add
// fma(-0, +0, s) = s exactly, so the row sums are the FP32 FMA chains in
// CSR order of the wavefront and pipeline mixed forms, bit for bit.
// ------------------------------------------------------------------------
constexpr int kTrThreads = 768;
constexpr int kTrRows = 3;
constexpr int kTrHdrInts = 32;  // header of a vert image: 4 counts, c_0..c_nlevel, [31] rotation ints

struct TileRegArgs {
  int n, nlevel, ntile, zs;      // zs: the zero position (a +0 in every level buffer)
  const unsigned char *vimg;     // vert images
  const unsigned char *mimg;     // matrix images
  const long *voff, *moff;       // per tile (execution order): byte offsets
  const int *vbytes, *mbytes;    // per tile: image sizes (multiples of 16)
  int max_vbytes, max_mbytes, buf_floats;
  const float *x;
  float *vf;
  float scale;
  int *err;
};

__device__ __forceinline__ bool tr_wait(unsigned long long *bar, unsigned phase, int *err) {
  long spins = 0;
  while (!mbar_try(bar, phase)) {
    if (spins > 16) __nanosleep(64);
    if (++spins > kSpinLimit) {  // a copy of this CTA never completed: report, drain with a second bound
      if (threadIdx.x == 0) atomicCAS(err, 0, kErrTimeout);
      for (long s2 = 0; s2 < kSpinLimit && !mbar_try(bar, phase); s2++) __nanosleep(256);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One entry's operands in registers: FP32 values beside packed byte
// offsets.
template <typename VT, int W>
struct TrRow;
template <int W>
struct TrRow<float, W> {
  float v[W];
  uint32_t c[(W + 1) / 2];
  __device__ __forceinline__ void load(const uint32_t *cols, const float *vals) {
#pragma unroll
    for (int t = 0; t < W; t++) v[t] = vals[32 * t];
#pragma unroll
    for (int p = 0; p < (W + 1) / 2; p++) c[p] = cols[32 * p];
  }
  __device__ __forceinline__ float sum(const unsigned char *in) const {
    float s = 0.f;
#pragma unroll
    for (int t = 0; t < W; t++) {
      const uint32_t off = (t & 1) ? (c[t / 2] >> 16) : (c[t / 2] & 0xFFFFu);
      s = __fmaf_rn(v[t], *reinterpret_cast<const float *>(in + off), s);
    }
    return s;
  }
};
template <int W>
struct TrRow<__nv_bfloat16, W> : TrRow<float, W> {
  // BF16 values widened once, as the tile enters the registers (a BF16
  // value is the high half of its FP32 bit pattern): the level loop is the
  // FP32 one, and only the image in HBM and shared memory is narrower.
  __device__ __forceinline__ void load(const uint32_t *cols, const __nv_bfloat16 *vals) {
    const uint16_t *vb = reinterpret_cast<const uint16_t *>(vals);
#pragma unroll
    for (int t = 0; t < W; t++) this->v[t] = __uint_as_float((uint32_t)vb[32 * t] << 16);
#pragma unroll
    for (int p = 0; p < (W + 1) / 2; p++) this->c[p] = cols[32 * p];
  }
};

// One level of a tile: rows r = tid + j * kTrThreads below nr read the
// level buffer at byte offset IN of the dynamic shared memory and write the
// one at OUT (compile-time offsets, so a gather is one shared load with an
// immediate displacement); the part's own rows also go to dst.
template <typename VT, int W, int IN, int OUT>
__device__ __forceinline__ void tr_level(const TrRow<VT, W> (&row)[kTrRows], const int (&prow)[kTrRows],
                                         const int (&vert)[kTrRows], int nr, int owned, float *dst, float scale,
                                         unsigned char *smem) {
#pragma unroll
  for (int j = 0; j < kTrRows; j++) {
    const int r = (int)threadIdx.x + j * kTrThreads;
    if (r < nr) {
      const float s = row[j].sum(smem + IN) * scale;
      *reinterpret_cast<float *>(smem + OUT + 4 * prow[j]) = s;
      if (r < owned) __stcs(dst + vert[j], s);
    }
  }
}

// Level buffers: X0 and X1 at fixed offsets (the levels ping-pong between
// them), XG receives the next tile's level 0 and is copied to X0 when that
// tile starts; then the matrix image and the vert image.
constexpr int kTrXBytes = 16384;  // positions per level buffer: 4096 (the zero position included)

template <typename VT, int W>
__global__ void __launch_bounds__(kTrThreads, 1) tiles_reg_kernel(TileRegArgs a) {
  extern __shared__ __align__(128) unsigned char tr_smem[];
  __shared__ __align__(8) unsigned long long bar_v, bar_m;
  __shared__ int s_nrows[33];
  constexpr int X0 = 0, X1 = kTrXBytes, XG = 2 * kTrXBytes;
  float *xg = reinterpret_cast<float *>(tr_smem + XG);
  unsigned char *mbuf = tr_smem + 3 * kTrXBytes;                     // matrix image
  int *vbuf = reinterpret_cast<int *>(mbuf + a.max_mbytes);          // vert image
  const int tid = threadIdx.x, G = gridDim.x;
  int q = blockIdx.x;
  if (q >= a.ntile) return;
  if (tid == 0) {
    reinterpret_cast<float *>(tr_smem + X0)[a.zs] = 0.f;
    reinterpret_cast<float *>(tr_smem + X1)[a.zs] = 0.f;
  }
  long nvo = 0, nmo = 0;  // thread 0: offsets and sizes of this CTA's next tile, loaded a tile ahead
  int nvb = 0, nmb = 0;
  if (tid == 0) {
    mbar_init(&bar_v);
    mbar_init(&bar_m);
    mbar_expect(&bar_v, (unsigned)a.vbytes[q]);
    bulk_g2s(vbuf, a.vimg + a.voff[q], (unsigned)a.vbytes[q], &bar_v);
    mbar_expect(&bar_m, (unsigned)a.mbytes[q]);
    bulk_g2s(mbuf, a.mimg + a.moff[q], (unsigned)a.mbytes[q], &bar_m);
    if (q + G < a.ntile) {
      nvo = a.voff[q + G]; nmo = a.moff[q + G]; nvb = a.vbytes[q + G]; nmb = a.mbytes[q + G];
    }
  }
  __syncthreads();
  unsigned phase = 0;
  // the first tile's level 0
  if (!tr_wait(&bar_v, phase, a.err)) return;
  {
    const int npos = vbuf[0];
    const int *pv = vbuf + kTrHdrInts + vbuf[31];
    for (int s = tid; s < npos; s += kTrThreads) {
      const int v = pv[s];
      if (v >= 0) cp_async4(xg + s, a.x + v);
    }
  }
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int kWarps = kTrThreads / 32;
  for (;;) {
    // this tile: header, vertices and matrix image in shared memory
    if (!tr_wait(&bar_m, phase, a.err)) return;
    phase ^= 1u;
    const int npos = vbuf[0], nrow1 = vbuf[1], owned = vbuf[2], nslice = vbuf[3];
    if (tid >= 1 && tid <= a.nlevel) s_nrows[tid] = vbuf[4 + a.nlevel - tid];
    TrRow<VT, W> row[kTrRows];
    int vert[kTrRows], prow[kTrRows];
    const int *pv = vbuf + kTrHdrInts + vbuf[31];
    const uint32_t *cols = reinterpret_cast<const uint32_t *>(mbuf);  // two entries' offsets per word
    const VT *vals = reinterpret_cast<const VT *>(mbuf + (size_t)nslice * ((W + 1) / 2) * 128);
#pragma unroll
    for (int j = 0; j < kTrRows; j++) {
      const int r = tid + j * kTrThreads;
      prow[j] = r < nrow1 ? (r & ~31) | ((r + vbuf[kTrHdrInts + (r >> 5)]) & 31) : 0;
      vert[j] = r < owned ? pv[prow[j]] : 0;
      const long sl = warp + j * kWarps;  // slice r / 32
      if (r < nrow1) row[j].load(cols + (sl * ((W + 1) / 2)) * 32 + lane, vals + (sl * W) * 32 + lane);
    }
    cp_async_wait_all();  // this tile's level 0 (gathered during the previous tile)
    __syncthreads();      // both images fully read: the buffers take the next tile
    const int qn = q + G;
    const bool has_next = qn < a.ntile;
    if (tid == 0 && has_next) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect(&bar_v, (unsigned)nvb);
      bulk_g2s(vbuf, a.vimg + nvo, (unsigned)nvb, &bar_v);
      mbar_expect(&bar_m, (unsigned)nmb);
      bulk_g2s(mbuf, a.mimg + nmo, (unsigned)nmb, &bar_m);
      if (qn + G < a.ntile) {
        nvo = a.voff[qn + G]; nmo = a.moff[qn + G]; nvb = a.vbytes[qn + G]; nmb = a.mbytes[qn + G];
      }
    }
    for (int s = tid; s < npos; s += kTrThreads) reinterpret_cast<float *>(tr_smem + X0)[s] = xg[s];
    __syncthreads();
    const int lg = (a.nlevel + 1) / 2;  // level after which the next tile's x is gathered into XG
    for (int l = 1; l <= a.nlevel; l++) {
      float *dst = a.vf + (size_t)l * a.n;
      if (l & 1) tr_level<VT, W, X0, X1>(row, prow, vert, s_nrows[l], owned, dst, a.scale, tr_smem);
      else tr_level<VT, W, X1, X0>(row, prow, vert, s_nrows[l], owned, dst, a.scale, tr_smem);
      if (l == lg && has_next) {
        if (!tr_wait(&bar_v, phase, a.err)) return;
        const int nposn = vbuf[0];
        const int *pn = vbuf + kTrHdrInts + vbuf[31];
        for (int s = tid; s < nposn; s += kTrThreads) {
          const int v = pn[s];
          if (v >= 0) cp_async4(xg + s, a.x + v);
        }
      }
      __syncthreads();
    }
    if (!has_next) break;
    q = qn;
  }
}

using TrKernel = void (*)(TileRegArgs);
inline TrKernel tr_kernel_ptr(int value_type, int w) {
  if (value_type == MPKG_VALUE_F32)
    return w == 5 ? tiles_reg_kernel<float, 5> : w == 9 ? tiles_reg_kernel<float, 9> : tiles_reg_kernel<float, 12>;
  return w == 5 ? tiles_reg_kernel<__nv_bfloat16, 5>
                : w == 9 ? tiles_reg_kernel<__nv_bfloat16, 9> : tiles_reg_kernel<__nv_bfloat16, 12>;
}
inline int tr_width(int wmax) { return wmax <= 5 ? 5 : wmax <= 9 ? 9 : wmax <= 12 ? 12 : 0; }

using TmKernel = void (*)(TileMixArgs);
inline TmKernel tm_kernel_ptr(int value_type, int w) {
  if (value_type == MPKG_VALUE_F32)
    return w == 8 ? tiles_mix_kernel<float, 8> : w == 12 ? tiles_mix_kernel<float, 12> : tiles_mix_kernel<float, 16>;
  return w == 8 ? tiles_mix_kernel<__nv_bfloat16, 8>
                : w == 12 ? tiles_mix_kernel<__nv_bfloat16, 12> : tiles_mix_kernel<__nv_bfloat16, 16>;
}

// ------------------------------------------------------------------------
// Batched block-vector MPK (FP32): many independent matrices, nrhs
// right-hand sides each, in ONE persistent cooperative launch.  The
// matrices are concatenated into one block-diagonal CSR and cut into
// groups whose matrix + two levels of vectors fit in L2; every CTA owns a
// row range of every group and walks (group, level) in order, waiting
// only for the CTAs that own its columns (the wavefront rule), so a group's
// matrix is read from HBM once for all levels.  A row is computed by LPR
// lanes, each holding VW consecutive right-hand sides (vector loads);
// entries are accumulated with single-precision FMA in CSR order.
// ------------------------------------------------------------------------
struct BatchArgs {
  long N;                      // rows of all matrices
  int nrhs, nlevel, nblk, ngroup;
  uint32_t base, stall;
  const int *ptr, *col;        // block-diagonal CSR (global columns)
  const float *val;
  float *vb;                   // (nlevel + 1) * N * nrhs, level 0 = input
  const int *row_lo;           // ngroup * (nblk + 1)
  const int *dep_ptr;          // ngroup * nblk + 1: CTA b of group g waits for
  const int *dep_idx;          // dep_idx[dep_ptr[g*nblk+b] ..), the other CTAs owning its columns
  unsigned int *flags;
  int *err;
  const int *win;              // staged form: ngroup * nblk pairs [w0, w1) of previous-level rows in smem
};

template <int VW>
struct VecF;
template <>
struct VecF<1> {
  static __device__ __forceinline__ void ld(const float *p, float *v) { v[0] = *p; }
  static __device__ __forceinline__ void st(float *p, const float *v) { __stcs(p, v[0]); }
};
template <>
struct VecF<2> {
  static __device__ __forceinline__ void ld(const float *p, float *v) {
    const float2 t = *reinterpret_cast<const float2 *>(p);
    v[0] = t.x; v[1] = t.y;
  }
  static __device__ __forceinline__ void st(float *p, const float *v) {
    __stcs(reinterpret_cast<float2 *>(p), make_float2(v[0], v[1]));
  }
};
template <>
struct VecF<4> {
  static __device__ __forceinline__ void ld(const float *p, float *v) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
  static __device__ __forceinline__ void st(float *p, const float *v) {
    __stcs(reinterpret_cast<float4 *>(p), make_float4(v[0], v[1], v[2], v[3]));
  }
};

template <int LPR, int VW>
__global__ void __launch_bounds__(256) batch_kernel(BatchArgs a) {
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = 0;
  __syncthreads();
  const int b = blockIdx.x, nrhs = LPR * VW;
  const int lane = (int)threadIdx.x % LPR, rpp = (int)blockDim.x / LPR;
  for (int g = 0; g < a.ngroup; g++) {
    const int r0 = a.row_lo[(size_t)g * (a.nblk + 1) + b], r1 = a.row_lo[(size_t)g * (a.nblk + 1) + b + 1];
    const unsigned tag = a.base + (unsigned)g * (unsigned)(a.nlevel + 1);
    const int dlo = a.dep_ptr[(size_t)g * a.nblk + b], dhi = a.dep_ptr[(size_t)g * a.nblk + b + 1];
    for (int l = 1; l <= a.nlevel; l++) {
      if (l > 1) {  // the CTAs owning this range's columns have published level l-1 of group g
        for (int k = dlo + (int)threadIdx.x; k < dhi; k += blockDim.x) {
          const int c = a.dep_idx[k];
          long spins = 0;
          while (ld_acquire(a.flags + c) < tag + (unsigned)(l - 1) + a.stall) {
            if (++spins > kSpinLimit || *((volatile int *)a.err)) {
              atomicCAS(a.err, 0, kErrTimeout);
              s_abort = 1;
              break;
            }
            __nanosleep(spins < 16 ? 32 : 256);
          }
        }
        __syncthreads();
        if (s_abort) return;
      }
      const float *src = a.vb + (size_t)(l - 1) * a.N * nrhs + lane * VW;
      float *dst = a.vb + (size_t)l * a.N * nrhs + lane * VW;
      for (int i = r0 + (int)threadIdx.x / LPR; i < r1; i += rpp) {
        float acc[VW];
#pragma unroll
        for (int u = 0; u < VW; u++) acc[u] = 0.0f;
        const int q0 = __ldg(a.ptr + i), q1 = __ldg(a.ptr + i + 1);
        int q = q0;
        // four entries in flight: column and value loads first, then the
        // four vector loads, then the FMAs in CSR order
        for (; q + 4 <= q1; q += 4) {
          int c[4];
          float v[4], xv[4][VW];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            c[u] = __ldg(a.col + q + u);
            v[u] = __ldg(a.val + q + u);
          }
#pragma unroll
          for (int u = 0; u < 4; u++) VecF<VW>::ld(src + (size_t)c[u] * nrhs, xv[u]);
#pragma unroll
          for (int u = 0; u < 4; u++)
#pragma unroll
            for (int w = 0; w < VW; w++) acc[w] = __fmaf_rn(v[u], xv[u][w], acc[w]);
        }
        for (; q < q1; q++) {
          float x0[VW];
          const float v0 = __ldg(a.val + q);
          VecF<VW>::ld(src + (size_t)__ldg(a.col + q) * nrhs, x0);
#pragma unroll
          for (int u = 0; u < VW; u++) acc[u] = __fmaf_rn(v0, x0[u], acc[u]);
        }
        VecF<VW>::st(dst + (size_t)i * nrhs, acc);
      }
      __syncthreads();  // as in wave_publish: the release store is cumulative
      if (threadIdx.x == 0) {
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a.flags + b), "r"(tag + (unsigned)l) : "memory");
      }
    }
  }
}

// The batched rows with the previous level staged in shared memory.  Per
// (group, level) the CTA copies rows [w0, w1) of the previous level (its
// own rows and the halo its columns reach, as far as the window holds)
// with one bulk copy on an mbarrier; an entry whose column falls in the
// window reads shared memory, any other reads global memory through the
// same generic load.  Rows of the window that no row of the CTA reads may
// be stale: they are never used.  Same rows, CSR order and FMAs as
// batch_kernel, so the same bits.
template <int LPR, int VW>
__global__ void __launch_bounds__(1024) batch_stage_kernel(BatchArgs a) {
  extern __shared__ __align__(128) float bs_win[];
  __shared__ int s_abort;
  __shared__ __align__(8) unsigned long long s_bar;
  if (threadIdx.x == 0) {
    s_abort = 0;
    mbar_init(&s_bar);
  }
  __syncthreads();
  unsigned phase = 0;
  const int b = blockIdx.x, nrhs = LPR * VW;
  const int lane = (int)threadIdx.x % LPR, rpp = (int)blockDim.x / LPR;
  for (int g = 0; g < a.ngroup; g++) {
    const int r0 = a.row_lo[(size_t)g * (a.nblk + 1) + b], r1 = a.row_lo[(size_t)g * (a.nblk + 1) + b + 1];
    const unsigned tag = a.base + (unsigned)g * (unsigned)(a.nlevel + 1);
    const int dlo = a.dep_ptr[(size_t)g * a.nblk + b], dhi = a.dep_ptr[(size_t)g * a.nblk + b + 1];
    const int w0 = a.win[2 * ((size_t)g * a.nblk + b)], w1 = a.win[2 * ((size_t)g * a.nblk + b) + 1];
    const unsigned wn = (unsigned)(w1 - w0);
    for (int l = 1; l <= a.nlevel; l++) {
      if (l > 1) {  // the CTAs owning this range's columns have published level l-1 of group g
        for (int k = dlo + (int)threadIdx.x; k < dhi; k += blockDim.x) {
          const int c = a.dep_idx[k];
          long spins = 0;
          while (ld_acquire(a.flags + c) < tag + (unsigned)(l - 1) + a.stall) {
            if (++spins > kSpinLimit || *((volatile int *)a.err)) {
              atomicCAS(a.err, 0, kErrTimeout);
              s_abort = 1;
              break;
            }
            __nanosleep(spins < 16 ? 32 : 256);
          }
        }
        __syncthreads();
        if (s_abort) return;
      }
      const float *src = a.vb + (size_t)(l - 1) * a.N * nrhs;
      if (wn > 0) {
        if (threadIdx.x == 0) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier reads of the window first
          const unsigned bytes = wn * (unsigned)nrhs * 4u;
          mbar_expect(&s_bar, bytes);
          bulk_g2s(bs_win, src + (size_t)w0 * nrhs, bytes, &s_bar);
        }
        if (!tr_wait(&s_bar, phase, a.err)) return;
        phase ^= 1u;
      }
      const float *gl = src + lane * VW;
      const float *wl = bs_win + lane * VW;
      float *dst = a.vb + (size_t)l * a.N * nrhs + lane * VW;
      for (int i = r0 + (int)threadIdx.x / LPR; i < r1; i += rpp) {
        float acc[VW];
#pragma unroll
        for (int u = 0; u < VW; u++) acc[u] = 0.0f;
        const int q0 = __ldg(a.ptr + i), q1 = __ldg(a.ptr + i + 1);
        int q = q0;
        for (; q + 4 <= q1; q += 4) {
          const float *xp[4];
          float v[4], xv[4][VW];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const int c = __ldg(a.col + q + u);
            v[u] = __ldg(a.val + q + u);
            const unsigned o = (unsigned)(c - w0);
            xp[u] = o < wn ? wl + (size_t)o * nrhs : gl + (size_t)c * nrhs;
          }
#pragma unroll
          for (int u = 0; u < 4; u++) VecF<VW>::ld(xp[u], xv[u]);
#pragma unroll
          for (int u = 0; u < 4; u++)
#pragma unroll
            for (int w = 0; w < VW; w++) acc[w] = __fmaf_rn(v[u], xv[u][w], acc[w]);
        }
        for (; q < q1; q++) {
          float x0[VW];
          const int c = __ldg(a.col + q);
          const float v0 = __ldg(a.val + q);
          const unsigned o = (unsigned)(c - w0);
          VecF<VW>::ld(o < wn ? wl + (size_t)o * nrhs : gl + (size_t)c * nrhs, x0);
#pragma unroll
          for (int u = 0; u < VW; u++) acc[u] = __fmaf_rn(v0, x0[u], acc[u]);
        }
        VecF<VW>::st(dst + (size_t)i * nrhs, acc);
      }
      __syncthreads();  // rows written and the window read; the release store is cumulative
      if (threadIdx.x == 0) {
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a.flags + b), "r"(tag + (unsigned)l) : "memory");
      }
    }
  }
}

// One pdmpk batch of every rank (Buffers::DoComp, pdmpk/buffers.cc:76-97):
// a row starts from its partial-sum seed (or 0.0) and adds val*mbuf[col]
// in CSR order.  Thread per row; rows of a batch are independent.
template <int ARITH>
__global__ void __launch_bounds__(256) pd_batch_kernel(long r0, long r1, const long *__restrict__ row_dst,
                                                       const long *__restrict__ row_init,
                                                       const long *__restrict__ row_ptr,
                                                       const long *__restrict__ gcol,
                                                       const double *__restrict__ gval, double *mbuf) {
  for (long q = r0 + blockIdx.x * (long)blockDim.x + threadIdx.x; q < r1; q += (long)gridDim.x * blockDim.x) {
    const long s0 = row_init[q];
    double s = s0 >= 0 ? mbuf[s0] : 0.0;
    for (long j = row_ptr[q]; j < row_ptr[q + 1]; j++) {
      if (ARITH == MPKG_ARITH_SEPARATE) s = __dadd_rn(s, __dmul_rn(gval[j], mbuf[gcol[j]]));
      else s = fma(gval[j], mbuf[gcol[j]], s);
    }
    mbuf[row_dst[q]] = s;
  }
}

// ------------------------------------------------------------------------
// Mixed-precision pipeline: matrix values stored as FP32 or BF16, basis
// vectors FP32, FP32 accumulation (FMA, CSR order).  Each level is scaled by
// a fixed power of two 2^-e with 2^e >= ||A||_inf, so the stored basis
// never grows (|v_l| <= |v_(l-1)|) and the scaling itself is exact; the
// caller recovers A^l x = 2^(l e) v_l.  Chunk-affine schedule as
// pipe_kernel: the chunk's columns and values are staged in shared memory
// by bulk copies once and reused for every level.
// ------------------------------------------------------------------------
struct MixArgs {
  int n, nlevel, chunk, nchunk;
  uint32_t epoch;
  const int *gdep_lo, *gdep_hi;
  const int *ptr, *col;
  const void *val;   // float or __nv_bfloat16, nnz entries
  float *vv;         // (nlevel+1)*n FP32, x in vv[0..n)
  float scale;       // 2^-e
  unsigned int *ticket;
  unsigned int *counts;
  int *err;
  int max_chunk_nnz;
  bool bulk_ok;
};


template <typename VT>
__global__ void __launch_bounds__(kPipeThreads) mix_pipe_kernel(MixArgs m) {
  extern __shared__ __align__(16) unsigned char pipe_smem[];
  // reuse the FP64 pipeline's take/wait/publish through a PipeArgs view
  PipeArgs a{};
  a.n = m.n; a.nlevel = m.nlevel; a.chunk = m.chunk; a.nchunk = m.nchunk; a.ngroups = m.nchunk;
  a.epoch = m.epoch; a.stall = 0; a.ptr = m.ptr; a.col = m.col; a.ticket = m.ticket; a.counts = m.counts;
  a.err = m.err; a.max_chunk_nnz = m.max_chunk_nnz; a.bulk_ok = m.bulk_ok;
  int *rptr = reinterpret_cast<int *>(pipe_smem);
  int *cols_buf = reinterpret_cast<int *>(pipe_smem + pipe_cols_offset(m.chunk));
  VT *vals_buf = reinterpret_cast<VT *>(pipe_smem + pipe_vals_offset(m.chunk, m.max_chunk_nnz));
  __shared__ unsigned int s_chunk;
  __shared__ int s_abort;
  __shared__ __align__(8) unsigned long long s_bar;
  unsigned phase = 0;
  if (threadIdx.x == 0 && m.bulk_ok) mbar_init(&s_bar);
  __syncthreads();
  const VT *val = static_cast<const VT *>(m.val);
  for (;;) {
    int *cols;
    VT *vals;
    const int c = pipe_take<VT, true>(a, val, rptr, cols_buf, vals_buf, &cols, &vals, &s_bar, &phase, &s_chunk,
                                      &s_abort);
    if (c < 0) return;
    const int r0 = c * m.chunk;
    const int nr = min(m.chunk, m.n - r0);
    const int r = threadIdx.x;
    const bool active = r < nr;
    const int q0 = rptr[r], q1 = active ? rptr[r + 1] : q0;
    const int glo = m.gdep_lo[c], ghi = m.gdep_hi[c];
    for (int l = 1; l <= m.nlevel; l++) {
      if (l > 1 && !pipe_wait(a, glo, ghi, l - 1, &s_abort)) return;
      const float *src = m.vv + (long)(l - 1) * m.n;
      float s = 0.f;
      if (q1 - q0 <= 12) {
        float xv[12];
#pragma unroll
        for (int t = 0; t < 12; t++)
          if (q0 + t < q1) xv[t] = src[cols[q0 + t]];
#pragma unroll
        for (int t = 0; t < 12; t++)
          if (q0 + t < q1) s = __fmaf_rn(to_f32(vals[q0 + t]), xv[t], s);
      } else {
        for (int q = q0; q < q1; q++) s = __fmaf_rn(to_f32(vals[q]), src[cols[q]], s);
      }
      if (active) m.vv[(long)l * m.n + r0 + r] = s * m.scale;
      pipe_publish(a, c, l);
    }
  }
}

}  // namespace

// ==========================================================================
// Plans
// ==========================================================================
struct mpkg_plan {
  int n = 0, nlevel = 0, nphase = 0, npart = 0;
  int exec = MPKG_EXEC_TASKS, arith = MPKG_ARITH_FMA;
  bool valued = false;
  bool full_coverage = true;
  long nnz = 0;
  long rows_computed = 0;
  long device_bytes = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  int *d_ptr = nullptr, *d_col = nullptr;
  double *d_coef = nullptr;  // values (nnz) or 1/deg (n)
  float2 *d_coef2 = nullptr; // double-float split of d_coef (ARITH_DF64)
  int *d_err = nullptr;
  double *d_vv = nullptr;    // staging for host execution
  // tasks
  std::vector<long> list_seg_h;
  long *d_list_seg = nullptr;
  int *d_seg_level = nullptr;
  long *d_seg_off = nullptr;
  int *d_rows = nullptr;
  // tiles
  TileArgs tiles{};
  bool tiles_smem = true;
  size_t tiles_smem_bytes = 0;
  int max_tile_slots = 0;
  std::vector<void *> owned;
  // pipe
  PipeArgs pipe{};
  int pipe_grid = 0, pipe_reach = 0;
  size_t pipe_smem_bytes = 0;
  // mixed-precision pipeline
  MixArgs mix{};
  int mix_vt = 0;    // 0: FP32 values, 1: BF16 values
  int mix_e = 0;     // levels are scaled by 2^-mix_e
  long mix_inexact = 0;  // values not exactly representable in the storage type
  // MPI-2 rank buffers
  double *b_vall = nullptr;
  long *b_in_dst = nullptr, *b_in_src = nullptr, *b_out_src = nullptr, *b_out_dst = nullptr;
  long b_nin = 0, b_nout = 0;
  long *b_cm_dst = nullptr, *b_cm_src = nullptr;
  std::vector<long> b_cm_off;  // per phase: range of the comm gather
  long *b_list_seg = nullptr, *b_seg_off = nullptr, *b_row_dst = nullptr, *b_row_ptr = nullptr,
       *b_gcol = nullptr;
  double *b_gval = nullptr;
  // wavefront executor
  WaveArgs wave{};
  int wave_grid = 0;
  bool wave_rel = false;
  bool wave_uni = false;  // pattern-compressed offsets (plans with matrix values)
  // batched block-vector form
  BatchArgs batch{};
  int batch_lpr = 0, batch_vw = 0, batch_nmat = 0;
  int batch_threads = 256;   // CTA size of the persistent launch
  bool batch_staged = false; // batch_stage_kernel: previous level windowed in shared memory
  size_t batch_smem = 0;     // its window bytes per CTA
  long batch_group_bytes = 0;
  double batch_tune_ms = 0.0;
  int batch_candidates = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  const void *graph_key = nullptr;
  bool graph_ok = false;
  float *d_fb = nullptr;  // staging of mpkg_exec_batch_host
  // k-SpMV in double-float or fixed point: level ring, fixed-point tables
  void *sp_ring = nullptr;
  unsigned long long *sp_mul = nullptr;
  unsigned int *sp_word = nullptr;
  int sp_dbits = 0;
  // mixed form on PA1 tiles (temporal blocking)
  TileMixArgs tm{};
  bool tm_on = false;
  int tm_w = 0, tm_grid = 0;
  size_t tm_smem = 0;
  double tune_ms = 0.0;    // mpkg_plan_mixed_tiles_tuned: time spent choosing the part size
  int tune_candidates = 0;  // part sizes it timed
  TileRegArgs tr{};  // register-resident tiles (replaces tm when every tile fits)
  bool tr_on = false;
  int tr_w = 0, tr_grid = 0;
  size_t tr_smem = 0;
  mpkg_plan *inner = nullptr;  // mixed form: the wavefront layout it runs on
  void *mix_sval = nullptr;    // mixed form: sliced FP32 / BF16 values
  // pdmpk buffers (b_vall, b_in_*, b_out_*, b_cm_* shared with the above)
  long *d_row_init = nullptr;
  std::vector<long> pd_row_off;  // per batch: range of rows
  uint32_t epoch = 0;
  int launches = 0;
  std::vector<double> h_x;  // x staging when a tasks plan leaves entries uncovered
};

namespace {

template <typename T>
int dev_copy(mpkg_plan *p, T **dst, const T *src, size_t count) {
  *dst = nullptr;
  if (count == 0) return kOk;
  CUDA_TRY(cudaMalloc((void **)dst, sizeof(T) * count));
  p->owned.push_back(*dst);
  p->device_bytes += (long)(sizeof(T) * count);
  CUDA_TRY(cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice));
  return kOk;
}

template <typename T>
int dev_alloc(mpkg_plan *p, T **dst, size_t count) {
  *dst = nullptr;
  if (count == 0) return kOk;
  CUDA_TRY(cudaMalloc((void **)dst, sizeof(T) * count));
  p->owned.push_back(*dst);
  p->device_bytes += (long)(sizeof(T) * count);
  return kOk;
}

int check_csr(int n, const int *ptr, const int *col) {
  if (n <= 0 || !ptr || !col) return fail(kEInval, "empty matrix or null arrays");
  if (ptr[0] != 0) return fail(kEInval, "ptr[0] must be 0");
  if (ptr[n] <= 0) return fail(kEInval, "the matrix has no entries");
  for (int i = 0; i < n; i++)
    if (ptr[i + 1] < ptr[i]) return fail(kEInval, "ptr must be non-decreasing");
  for (long j = 0; j < ptr[n]; j++)
    if (col[j] < 0 || col[j] >= n) return fail(kERange, "column index out of range");
  return kOk;
}

int plan_common(mpkg_plan *p, int n, const int *ptr, const int *col, const double *val,
                int nlevel, int arith, bool allow_fixed = false) {
  int rc = check_csr(n, ptr, col);
  if (rc) return rc;
  if (nlevel <= 0 || nlevel > 31) return fail(kEInval, "nlevel must be in [1, 31]");
  if (arith == MPKG_ARITH_FIXED && !(allow_fixed && val == nullptr))
    return fail(kEInval, "fixed-point arithmetic runs the 1/deg operator only (wavefront and k-SpMV executors)");
  if (arith != MPKG_ARITH_FMA && arith != MPKG_ARITH_SEPARATE && arith != MPKG_ARITH_DF64 &&
      arith != MPKG_ARITH_FIXED)
    return fail(kEInval, "unknown arith mode");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  CUDA_TRY(cudaGetDevice(&p->device));
  p->n = n;
  p->nlevel = nlevel;
  p->arith = arith;
  p->valued = val != nullptr;
  p->nnz = ptr[n];
  CUDA_TRY(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  if ((rc = dev_copy(p, &p->d_ptr, ptr, (size_t)n + 1))) return rc;
  if ((rc = dev_copy(p, &p->d_col, col, (size_t)p->nnz))) return rc;
  if (val) {
    if ((rc = dev_copy(p, &p->d_coef, val, (size_t)p->nnz))) return rc;
  } else {
    std::vector<double> rdeg(n);
    // as mpk2/mpkexec.c:28; an empty row sums no terms (0 in the reference),
    // so its unused coefficient is 0 rather than 1/0 (a row-sum-then-scale
    // kernel would otherwise form 0 * inf)
    for (int i = 0; i < n; i++) rdeg[i] = ptr[i + 1] > ptr[i] ? 1.0 / (ptr[i + 1] - ptr[i]) : 0.0;
    if ((rc = dev_copy(p, &p->d_coef, rdeg.data(), (size_t)n))) return rc;
  }
  if (arith == MPKG_ARITH_DF64) {
    const long m = val ? p->nnz : n;
    if ((rc = dev_alloc(p, &p->d_coef2, (size_t)m))) return rc;
    split_kernel<<<256, 256, 0, p->stream>>>(p->d_coef, p->d_coef2, m);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(p->stream));
  }
  if ((rc = dev_alloc(p, &p->d_err, 1))) return rc;
  CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
  return kOk;
}

int build_task_device(mpkg_plan *p, int npart, int nphase, const long *off, const long *idx) {
  const int n = p->n;
  const long nlists = (long)(nphase + 1) * npart;
  std::vector<long> list_seg(nlists + 1, 0);
  std::vector<int> seg_level;
  std::vector<long> seg_off;
  std::vector<int> rows;
  rows.reserve(off[nlists]);
  std::vector<unsigned char> covered((size_t)n * (p->nlevel + 1), 0);
  for (long t = 0; t < nlists; t++) {
    list_seg[t] = (long)seg_level.size();
    if (off[t + 1] < off[t]) return fail(kEInval, "task offsets must be non-decreasing");
    int cur = -1;
    for (long q = off[t]; q < off[t + 1]; q++) {
      long e = idx[q];
      long l = e / n;
      if (e < 0 || l < 1 || l > p->nlevel) return fail(kERange, "task entry outside levels 1..nlevel");
      int i = (int)(e - l * n);
      if (l < cur) return fail(kEInval, "task list is not level-major");
      if (l != cur) {
        seg_level.push_back((int)l);
        seg_off.push_back((long)rows.size());
        cur = (int)l;
      }
      rows.push_back(i);
      covered[(size_t)e] = 1;
    }
  }
  list_seg[nlists] = (long)seg_level.size();
  seg_off.push_back((long)rows.size());
  p->full_coverage = true;
  for (size_t e = (size_t)n; e < covered.size(); e++)
    if (!covered[e]) { p->full_coverage = false; break; }
  p->rows_computed = (long)rows.size();
  p->list_seg_h = list_seg;
  int rc;
  if ((rc = dev_copy(p, &p->d_list_seg, list_seg.data(), list_seg.size()))) return rc;
  if ((rc = dev_copy(p, &p->d_seg_level, seg_level.data(), seg_level.size()))) return rc;
  if ((rc = dev_copy(p, &p->d_seg_off, seg_off.data(), seg_off.size()))) return rc;
  if ((rc = dev_copy(p, &p->d_rows, rows.data(), rows.size()))) return rc;
  return kOk;
}

int build_tile_device(mpkg_plan *p, const TilePlan &tp, const int *ptr_host_) {
  int rc;
  TileArgs &a = p->tiles;
  a.n = p->n;
  a.nlevel = p->nlevel;
  a.max_slots = tp.max_slots;
  p->max_tile_slots = tp.max_slots;
  p->rows_computed = tp.total_rows;
  int *order, *shell, *slot_vert;
  long *slot_off, *slice_off, *ell_off;
  uint16_t *ell_col;
  uint8_t *ell_width;
  if ((rc = dev_copy(p, &order, tp.order.data(), tp.order.size()))) return rc;
  if ((rc = dev_copy(p, &slot_off, tp.slot_off.data(), tp.slot_off.size()))) return rc;
  if ((rc = dev_copy(p, &shell, tp.shell.data(), tp.shell.size()))) return rc;
  if ((rc = dev_copy(p, &slot_vert, tp.slot_vert.data(), tp.slot_vert.size()))) return rc;
  int *slot_coef;
  {
    std::vector<int> sc(tp.slot_vert.size());
    for (size_t q = 0; q < sc.size(); q++) sc[q] = p->valued ? ptr_host_[tp.slot_vert[q]] : tp.slot_vert[q];
    if ((rc = dev_copy(p, &slot_coef, sc.data(), sc.size()))) return rc;
  }
  a.slot_coef = slot_coef;
  if ((rc = dev_copy(p, &slice_off, tp.slice_off.data(), tp.slice_off.size()))) return rc;
  if ((rc = dev_copy(p, &ell_off, tp.ell_off.data(), tp.ell_off.size()))) return rc;
  std::vector<uint16_t> ec = tp.ell_col;
  if (ec.empty()) ec.push_back(0xFFFF);
  if ((rc = dev_copy(p, &ell_col, ec.data(), ec.size()))) return rc;
  std::vector<uint8_t> ew = tp.ell_width;
  if (ew.empty()) ew.push_back(0);
  if ((rc = dev_copy(p, &ell_width, ew.data(), ew.size()))) return rc;
  a.order = order; a.slot_off = slot_off; a.shell = shell; a.slot_vert = slot_vert;
  a.slice_off = slice_off; a.ell_off = ell_off; a.ell_col = ell_col; a.ell_width = ell_width;
  a.ptr = p->d_ptr;
  a.coef = p->d_coef;
  a.err = p->d_err;
  size_t need = 2 * (size_t)tp.max_slots * sizeof(double);
  int maxsm = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device));
  p->tiles_smem = need <= (size_t)maxsm;
  p->tiles_smem_bytes = p->tiles_smem ? need : 0;
  a.scratch = nullptr;
  if (!p->tiles_smem) {
    double *scr;
    if ((rc = dev_alloc(p, &scr, 2 * (size_t)tp.max_slots * tp.npart))) return rc;
    a.scratch = scr;
  }
  return kOk;
}

template <int ARITH, bool VALUED, bool SMEM>
int set_tiles_attr(size_t bytes) {
  CUDA_TRY(cudaFuncSetAttribute(tiles_kernel<ARITH, VALUED, SMEM>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return kOk;
}

template <bool VALUED>
int pipe_setup_df(mpkg_plan *p, int *grid) {
  int per_sm = 0, nsm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, flow_df_kernel<VALUED>, kPipeThreads, 0));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
  *grid = per_sm * nsm;
  return kOk;
}

template <bool VALUED, bool SMEM>
int set_tiles_df_attr(size_t bytes) {
  CUDA_TRY(cudaFuncSetAttribute(tiles_df_kernel<VALUED, SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)bytes));
  return kOk;
}

template <int ARITH, bool VALUED>
int pipe_setup_t(mpkg_plan *p, int *grid) {
  int per_sm = 0, nsm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, flow_kernel<ARITH, VALUED>, kPipeThreads, 0));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
  *grid = per_sm * nsm;
  return kOk;
}

template <typename K>
int wave_occupancy(mpkg_plan *p, K kernel, int *grid) {
  int per_sm = 0, nsm = 0, coop = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, p->device));
  if (!coop) return fail(kECuda, "device does not support cooperative launches");
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
  if (per_sm <= 0) return fail(kECuda, "wavefront kernel cannot be resident");
  *grid = per_sm * nsm;
  return kOk;
}

void *wave_kernel_ptr(const mpkg_plan *p) {
  const bool rel = p->wave_rel, stage = p->wave.stage_rel_bytes > 0, uni = p->wave_uni;
  if (p->arith == MPKG_ARITH_FIXED) return stage ? (void *)wave_fix_kernel<true> : (void *)wave_fix_kernel<false>;
#define MPKG_WK(REL, ST, UN)                                                                                  \
  if (p->arith == MPKG_ARITH_DF64)                                                                            \
    return p->valued ? (void *)wave_df_kernel<true, REL, ST, UN> : (void *)wave_df_kernel<false, REL, ST, UN>; \
  if (p->arith == MPKG_ARITH_SEPARATE)                                                                        \
    return p->valued ? (void *)wave_kernel<MPKG_ARITH_SEPARATE, true, REL, ST, UN>                            \
                     : (void *)wave_kernel<MPKG_ARITH_SEPARATE, false, REL, ST, UN>;                          \
  return p->valued ? (void *)wave_kernel<MPKG_ARITH_FMA, true, REL, ST, UN>                                   \
                   : (void *)wave_kernel<MPKG_ARITH_FMA, false, REL, ST, UN>;
  if (rel && stage && uni) { MPKG_WK(true, true, true) }
  if (rel && stage) { MPKG_WK(true, true, false) }
  if (rel && uni) { MPKG_WK(true, false, true) }
  if (rel) { MPKG_WK(true, false, false) }
  MPKG_WK(false, false, false)
#undef MPKG_WK
}

// Dynamic shared memory of a wave launch (the staged slab).
size_t wave_dyn_smem(const mpkg_plan *p) {
  const WaveArgs &w = p->wave;
  return w.stage_rel_bytes > 0 ? (size_t)w.stage_rel_bytes + w.stage_len_bytes + 5L * w.stage_slices : 0;
}

int launch_wave(mpkg_plan *p, double *d_vv, cudaStream_t st, double *hv = nullptr) {
  WaveArgs &w = p->wave;
  const unsigned step = (unsigned)p->nlevel + (p->arith == MPKG_ARITH_FIXED ? 2 : 1);
  if (w.base == 0 || w.base > (1u << 30)) {  // first call, or the flags would wrap: start over
    CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(unsigned int) * (size_t)w.nblk, st));
    if (w.fix_word) CUDA_TRY(cudaMemsetAsync(w.fix_word, 0, sizeof(unsigned long long), st));
    w.base = 1;
  } else {
    w.base += step;
  }
  WaveArgs a = w;
  a.vv = d_vv;
  a.hv = hv;
  void *args[] = {&a};
  CUDA_TRY(cudaLaunchCooperativeKernel(wave_kernel_ptr(p), dim3(w.nblk), dim3(256), args, wave_dyn_smem(p), st));
  return kOk;
}

// ---- batched form: kernel choice, layout, launch -------------------------
typedef void (*BatchKernel)(BatchArgs);

BatchKernel batch_kernel_for(int lpr, int vw) {
#define MPKG_BK(L, V) if (lpr == L && vw == V) return batch_kernel<L, V>;
  MPKG_BK(1, 1) MPKG_BK(2, 1) MPKG_BK(4, 1) MPKG_BK(8, 1) MPKG_BK(16, 1) MPKG_BK(32, 1)
  MPKG_BK(1, 2) MPKG_BK(2, 2) MPKG_BK(4, 2) MPKG_BK(8, 2) MPKG_BK(16, 2) MPKG_BK(32, 2)
  MPKG_BK(1, 4) MPKG_BK(2, 4) MPKG_BK(4, 4) MPKG_BK(8, 4) MPKG_BK(16, 4) MPKG_BK(32, 4)
#undef MPKG_BK
  return nullptr;
}

BatchKernel batch_stage_kernel_for(int lpr, int vw) {
#define MPKG_BK(L, V) if (lpr == L && vw == V) return batch_stage_kernel<L, V>;
  MPKG_BK(1, 4) MPKG_BK(2, 4) MPKG_BK(4, 4) MPKG_BK(8, 4) MPKG_BK(16, 4) MPKG_BK(32, 4)
#undef MPKG_BK
  return nullptr;
}

// Host description of the concatenated matrices.
struct BatchHost {
  long N = 0;
  std::vector<int> ptr, col;
  std::vector<float> val;
  std::vector<long> mat_row0;  // nmat + 1
};

// Groups of consecutive matrices within `budget` bytes (matrix + two
// levels of vectors); per group, CTA row ranges of equal nonzeros and the
// CTAs owning each range's columns.  With cap_rows > 0, also each (group,
// CTA)'s window [w0, w1) of previous-level rows for shared memory: the span
// of its columns when that fits cap_rows rows, else cap_rows rows around
// its own rows (columns beyond are read from global memory).
void batch_layout(const BatchHost &h, int nrhs, long budget, int grid, long cap_rows, std::vector<int> *row_lo,
                  std::vector<int> *dptr, std::vector<int> *didx, std::vector<int> *win, int *ngroup) {
  const int nmat = (int)h.mat_row0.size() - 1;
  std::vector<long> g0(1, 0);
  long bytes = 0;
  for (int m = 0; m < nmat; m++) {
    const long r0 = h.mat_row0[m], r1 = h.mat_row0[m + 1];
    const long mb = (long)(h.ptr[r1] - h.ptr[r0]) * 8 + (r1 - r0) * (4 + 8L * nrhs);
    if (bytes > 0 && bytes + mb > budget) {
      g0.push_back(r0);
      bytes = 0;
    }
    bytes += mb;
  }
  g0.push_back(h.N);
  *ngroup = (int)g0.size() - 1;
  row_lo->assign((size_t)*ngroup * (grid + 1), 0);
  dptr->assign((size_t)*ngroup * grid + 1, 0);
  win->assign((size_t)*ngroup * grid * 2, 0);
  didx->clear();
  std::vector<int> seen(grid, -1);
  for (int g = 0; g < *ngroup; g++) {
    int *lo = row_lo->data() + (size_t)g * (grid + 1);
    const long a = g0[g], z = g0[g + 1];
    const long q0 = h.ptr[a], nz = h.ptr[z] - q0;
    lo[0] = (int)a;
    for (int b = 1; b < grid; b++) {
      const long target = q0 + nz * b / grid;
      const int r = (int)(std::lower_bound(h.ptr.begin() + a, h.ptr.begin() + z + 1, (int)target) - h.ptr.begin());
      lo[b] = std::max(std::min(r, (int)z), lo[b - 1]);
    }
    lo[grid] = (int)z;
    // the exact set of other CTAs whose rows CTA b reads (its own rows of
    // the previous level are ordered by its barrier)
    for (int b = 0; b < grid; b++) {
      const size_t u = (size_t)g * grid + b;
      const size_t first = didx->size();
      for (long q = h.ptr[lo[b]]; q < h.ptr[lo[b + 1]]; q++) {
        const int c = h.col[q];
        if (c >= lo[b] && c < lo[b + 1]) continue;
        const int o = (int)(std::upper_bound(lo, lo + grid, c) - lo) - 1;  // last CTA starting at or before c
        if (seen[o] != (int)u) { seen[o] = (int)u; didx->push_back(o); }
      }
      std::sort(didx->begin() + first, didx->end());
      (*dptr)[u + 1] = (int)didx->size();
      if (cap_rows > 0 && lo[b + 1] > lo[b]) {
        long cmin = lo[b], cmax = lo[b + 1] - 1;
        for (long q = h.ptr[lo[b]]; q < h.ptr[lo[b + 1]]; q++) {
          cmin = std::min<long>(cmin, h.col[q]);
          cmax = std::max<long>(cmax, h.col[q]);
        }
        long w0 = cmin, w1 = cmax + 1;
        if (w1 - w0 > cap_rows) {  // around the own rows, within the column span
          const long own = lo[b + 1] - lo[b];
          w0 = own >= cap_rows ? lo[b] : std::max(cmin, lo[b] - (cap_rows - own) / 2);
          w1 = std::min(cmax + 1, w0 + cap_rows);
          w0 = std::max(cmin, w1 - cap_rows);
        }
        (*win)[2 * u] = (int)w0;
        (*win)[2 * u + 1] = (int)w1;
      }
    }
    std::fill(seen.begin(), seen.end(), -1);
  }
  if (didx->empty()) didx->push_back(0);
}

int batch_launch_raw(mpkg_plan *p, float *d_vb, cudaStream_t st, bool capture) {
  BatchArgs a = p->batch;
  a.vb = d_vb;
  if (capture) {
    a.base = 1;  // the graph resets the flags before every replay
  } else {
    BatchArgs &w = p->batch;
    const unsigned step = (unsigned)w.ngroup * (unsigned)(w.nlevel + 1);
    if (w.base == 0 || w.base > (1u << 30)) {
      CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(unsigned int) * (size_t)w.nblk, st));
      w.base = 1;
    } else {
      w.base += step;
    }
    a.base = w.base;
  }
  if (capture) CUDA_TRY(cudaMemsetAsync(a.flags, 0, sizeof(unsigned int) * (size_t)a.nblk, st));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nblk);
  cfg.blockDim = dim3(p->batch_threads);
  cfg.dynamicSmemBytes = p->batch_staged ? p->batch_smem : 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CUDA_TRY(cudaLaunchKernelEx(&cfg,
                              p->batch_staged ? batch_stage_kernel_for(p->batch_lpr, p->batch_vw)
                                              : batch_kernel_for(p->batch_lpr, p->batch_vw),
                              a));
  return kOk;
}

// One replayable graph per output buffer: flag reset + the persistent
// kernel.  Falls back to a direct launch when capture is not possible.
int batch_launch(mpkg_plan *p, float *d_vb, cudaStream_t st) {
  if (p->graph_ok && p->graph_key == d_vb) {
    CUDA_TRY(cudaGraphLaunch(p->graph_exec, st));
    return kOk;
  }
  if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }
  if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
  p->graph_ok = false;
  cudaStream_t cs = nullptr;
  bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess;
  if (ok) ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    const int rc = batch_launch_raw(p, d_vb, cs, true);
    cudaGraph_t g = nullptr;
    const bool ended = cudaStreamEndCapture(cs, &g) == cudaSuccess;
    ok = rc == kOk && ended && g != nullptr;
    if (ok) {
      p->graph = g;
      ok = cudaGraphInstantiate(&p->graph_exec, g, 0) == cudaSuccess;
    } else if (g) {
      cudaGraphDestroy(g);
    }
  }
  if (cs) cudaStreamDestroy(cs);
  cudaGetLastError();  // a failed capture leaves no sticky error
  clear_error();
  if (ok) {
    p->graph_ok = true;
    p->graph_key = d_vb;
    CUDA_TRY(cudaGraphLaunch(p->graph_exec, st));
    return kOk;
  }
  return batch_launch_raw(p, d_vb, st, false);
}

int launch_spmv(int n, const int *ptr, const int *col, const double *coef, bool valued, int nlevel,
                double *vv, int arith, cudaStream_t st) {
  dim3 blk(256), grd((n + 255) / 256);
  for (int l = 1; l <= nlevel; l++) {
    const double *x = vv + (long)(l - 1) * n;
    double *y = vv + (long)l * n;
    if (arith == MPKG_ARITH_SEPARATE) {
      if (valued) spmv_level_kernel<MPKG_ARITH_SEPARATE, true><<<grd, blk, 0, st>>>(n, ptr, col, coef, x, y);
      else spmv_level_kernel<MPKG_ARITH_SEPARATE, false><<<grd, blk, 0, st>>>(n, ptr, col, coef, x, y);
    } else {
      if (valued) spmv_level_kernel<MPKG_ARITH_FMA, true><<<grd, blk, 0, st>>>(n, ptr, col, coef, x, y);
      else spmv_level_kernel<MPKG_ARITH_FMA, false><<<grd, blk, 0, st>>>(n, ptr, col, coef, x, y);
    }
  }
  CUDA_TRY(cudaGetLastError());
  return kOk;
}

template <int ARITH, bool VALUED>
void launch_tasks_t(mpkg_plan *p, double *vv, cudaStream_t st) {
  for (int ph = 0; ph <= p->nphase; ph++) {
    tasks_kernel<ARITH, VALUED><<<p->npart, 256, 0, st>>>(p->n, ph * p->npart, p->d_list_seg,
                                                         p->d_seg_level, p->d_seg_off, p->d_rows,
                                                         p->d_ptr, p->d_col, p->d_coef, vv);
  }
}

template <int ARITH, bool VALUED>
void launch_tiles_t(mpkg_plan *p, const double *x, double *vv, cudaStream_t st) {
  TileArgs a = p->tiles;
  a.x = x;
  a.vv = vv;
  if (p->tiles_smem)
    tiles_kernel<ARITH, VALUED, true><<<p->npart, 512, p->tiles_smem_bytes, st>>>(a);
  else
    tiles_kernel<ARITH, VALUED, false><<<p->npart, 512, 0, st>>>(a);
}

template <bool VALUED>
void launch_tiles_df(mpkg_plan *p, const double *x, double *vv, cudaStream_t st) {
  TileArgs a = p->tiles;
  a.x = x;
  a.vv = vv;
  if (p->tiles_smem)
    tiles_df_kernel<VALUED, true><<<p->npart, 512, p->tiles_smem_bytes, st>>>(a, p->d_coef2);
  else
    tiles_df_kernel<VALUED, false><<<p->npart, 512, 0, st>>>(a, p->d_coef2);
}

template <bool VALUED>
void launch_pipe_df(mpkg_plan *p, const double *x, double *vv, cudaStream_t st) {
  PipeArgs a = p->pipe;
  a.x = x;
  a.vv = vv;
  a.epoch = p->epoch;
  flow_df_kernel<VALUED><<<p->pipe_grid, kPipeThreads, 0, st>>>(a);
}

template <int ARITH, bool VALUED>
void launch_pipe_t(mpkg_plan *p, const double *x, double *vv, cudaStream_t st) {
  PipeArgs a = p->pipe;
  a.x = x;
  a.vv = vv;
  a.epoch = p->epoch;
  flow_kernel<ARITH, VALUED><<<p->pipe_grid, kPipeThreads, 0, st>>>(a);
}

#define DISPATCH2(fn, ...)                                                   \
  do {                                                                       \
    if (p->arith == MPKG_ARITH_SEPARATE) {                                        \
      if (p->valued) fn<MPKG_ARITH_SEPARATE, true>(__VA_ARGS__);                  \
      else fn<MPKG_ARITH_SEPARATE, false>(__VA_ARGS__);                           \
    } else {                                                                 \
      if (p->valued) fn<MPKG_ARITH_FMA, true>(__VA_ARGS__);                       \
      else fn<MPKG_ARITH_FMA, false>(__VA_ARGS__);                                \
    }                                                                        \
  } while (0)

int plan_launch(mpkg_plan *p, double *d_vv, cudaStream_t st) {
  p->launches = 0;
  switch (p->exec) {
    case MPKG_EXEC_TASKS:
      DISPATCH2(launch_tasks_t, p, d_vv, st);
      p->launches = p->nphase + 1;
      break;
    case MPKG_EXEC_TILES:
      if (p->arith == MPKG_ARITH_DF64) {
        if (p->valued) launch_tiles_df<true>(p, d_vv, d_vv, st);
        else launch_tiles_df<false>(p, d_vv, d_vv, st);
      } else {
        DISPATCH2(launch_tiles_t, p, d_vv, d_vv, st);
      }
      p->launches = 1;
      break;
    case MPKG_EXEC_PIPE: {
      p->epoch++;
      if (p->epoch >= (1u << 27)) {  // counters would wrap: start over
        CUDA_TRY(cudaMemsetAsync(p->pipe.counts, 0,
                                 sizeof(unsigned int) * (size_t)(p->nlevel + 1) * p->pipe.ngroups, st));
        p->epoch = 1;
      }
      CUDA_TRY(cudaMemsetAsync(p->pipe.ticket, 0, sizeof(unsigned int), st));
      if (p->arith == MPKG_ARITH_DF64) {
        if (p->valued) launch_pipe_df<true>(p, d_vv, d_vv, st);
        else launch_pipe_df<false>(p, d_vv, d_vv, st);
      } else {
        DISPATCH2(launch_pipe_t, p, d_vv, d_vv, st);
      }
      p->launches = 1;
      break;
    }
    case MPKG_EXEC_BUFS: {
      const int P = p->npart;
      if (p->b_nin) gather_map_kernel<<<592, 256, 0, st>>>(d_vv, p->b_in_src, p->b_vall, p->b_in_dst, p->b_nin);
      for (int ph = 0; ph <= p->nphase; ph++) {
        const long c0 = p->b_cm_off[ph], c1 = p->b_cm_off[ph + 1];
        if (ph > 0 && c1 > c0)
          gather_map_kernel<<<592, 256, 0, st>>>(p->b_vall, p->b_cm_src + c0, p->b_vall, p->b_cm_dst + c0, c1 - c0);
        if (p->arith == MPKG_ARITH_SEPARATE)
          bufs_phase_kernel<MPKG_ARITH_SEPARATE><<<P, 256, 0, st>>>(ph * P, p->b_list_seg, p->b_seg_off,
                                                                   p->b_row_dst, p->b_row_ptr, p->b_gcol,
                                                                   p->b_gval, p->b_vall);
        else
          bufs_phase_kernel<MPKG_ARITH_FMA><<<P, 256, 0, st>>>(ph * P, p->b_list_seg, p->b_seg_off, p->b_row_dst,
                                                              p->b_row_ptr, p->b_gcol, p->b_gval, p->b_vall);
      }
      if (p->b_nout) gather_map_kernel<<<592, 256, 0, st>>>(p->b_vall, p->b_out_src, d_vv, p->b_out_dst, p->b_nout);
      p->launches = 2 + 2 * p->nphase + 1;
      break;
    }
    case MPKG_EXEC_BATCH:
      return fail(kEInval, "batch plans run through mpkg_exec_batch_device / mpkg_exec_batch_host");
    case MPKG_EXEC_WAVE: {
      int rc = launch_wave(p, d_vv, st);
      if (rc) return rc;
      p->launches = 1;
      break;
    }
    case MPKG_EXEC_PDMPK: {
      int nl = 0;
      if (p->b_nin) { gather_map_kernel<<<592, 256, 0, st>>>(d_vv, p->b_in_src, p->b_vall, p->b_in_dst, p->b_nin); nl++; }
      for (size_t bt = 0; bt + 1 < p->b_cm_off.size(); bt++) {
        const long c0 = p->b_cm_off[bt], c1 = p->b_cm_off[bt + 1];
        if (c1 > c0) {
          gather_map_kernel<<<(unsigned)std::min<long>((c1 - c0 + 255) / 256, 1216), 256, 0, st>>>(
              p->b_vall, p->b_cm_src + c0, p->b_vall, p->b_cm_dst + c0, c1 - c0);
          nl++;
        }
        const long r0 = p->pd_row_off[bt], r1 = p->pd_row_off[bt + 1];
        if (r1 <= r0) continue;
        const unsigned g = (unsigned)std::min<long>((r1 - r0 + 255) / 256, 1216);
        if (p->arith == MPKG_ARITH_SEPARATE)
          pd_batch_kernel<MPKG_ARITH_SEPARATE><<<g, 256, 0, st>>>(r0, r1, p->b_row_dst, p->d_row_init, p->b_row_ptr,
                                                                  p->b_gcol, p->b_gval, p->b_vall);
        else
          pd_batch_kernel<MPKG_ARITH_FMA><<<g, 256, 0, st>>>(r0, r1, p->b_row_dst, p->d_row_init, p->b_row_ptr,
                                                             p->b_gcol, p->b_gval, p->b_vall);
        nl++;
      }
      if (p->b_nout) {
        gather_map_kernel<<<592, 256, 0, st>>>(p->b_vall, p->b_out_src, d_vv + (size_t)p->nlevel * p->n, p->b_out_dst,
                                               p->b_nout);
        nl++;
      }
      p->launches = nl;
      break;
    }
    case MPKG_EXEC_SPMV: {
      const int n = p->n;
      const dim3 blk(256), grd((n + 255) / 256);
      if (p->arith == MPKG_ARITH_DF64) {
        float2 *ring = static_cast<float2 *>(p->sp_ring);
        split_kernel<<<592, 256, 0, st>>>(d_vv, ring, n);
        for (int l = 1; l <= p->nlevel; l++) {
          const float2 *src = ring + (size_t)((l - 1) & 1) * n;
          float2 *dst = ring + (size_t)(l & 1) * n;
          if (p->valued)
            spmv_df_kernel<true><<<grd, blk, 0, st>>>(n, p->d_ptr, p->d_col, p->d_coef2, src, dst, d_vv + (size_t)l * n);
          else
            spmv_df_kernel<false><<<grd, blk, 0, st>>>(n, p->d_ptr, p->d_col, p->d_coef2, src, dst, d_vv + (size_t)l * n);
        }
        CUDA_TRY(cudaGetLastError());
        p->launches = p->nlevel + 1;
        break;
      }
      if (p->arith == MPKG_ARITH_FIXED) {
        long long *ring = static_cast<long long *>(p->sp_ring);
        CUDA_TRY(cudaMemsetAsync(p->sp_word, 0, 2 * sizeof(unsigned int), st));
        fix_emax_kernel<<<592, 256, 0, st>>>(n, d_vv, p->sp_word);
        fix_convert_kernel<<<592, 256, 0, st>>>(n, d_vv, p->sp_word, p->sp_dbits, ring);
        for (int l = 1; l <= p->nlevel; l++)
          spmv_fix_kernel<<<grd, blk, 0, st>>>(n, p->d_ptr, p->d_col, p->sp_mul, p->sp_word,
                                               ring + (size_t)((l - 1) & 1) * n, ring + (size_t)(l & 1) * n,
                                               d_vv + (size_t)l * n);
        CUDA_TRY(cudaGetLastError());
        p->launches = p->nlevel + 2;
        break;
      }
      int rc = launch_spmv(p->n, p->d_ptr, p->d_col, p->d_coef, p->valued, p->nlevel, d_vv, p->arith, st);
      if (rc) return rc;
      p->launches = p->nlevel;
      break;
    }
    default:
      return fail(kEInval, "unknown executor");
  }
  CUDA_TRY(cudaGetLastError());
  return kOk;
}

mpkg_plan *new_plan() { return new (std::nothrow) mpkg_plan(); }

}  // namespace

// ==========================================================================
// C ABI
// ==========================================================================
extern "C" {

const char *mpkg_last_error(void) { return last_error(); }
int mpkg_version(void) { return 1; }

void mpkg_plan_destroy(mpkg_plan *p) {
  if (p && p->inner) mpkg_plan_destroy(p->inner);
  if (p && p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
  if (p && p->graph) cudaGraphDestroy(p->graph);
  if (!p) return;
  for (void *q : p->owned) cudaFree(q);
  if (p->d_vv) cudaFree(p->d_vv);
  if (p->d_fb) cudaFree(p->d_fb);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
}

int mpkg_plan_tasks(int n, const int *ptr, const int *col, const double *val, int npart,
                    int nlevel, int nphase, const long *off, const long *idx, int arith,
                    mpkg_plan **out) {
  clear_error();
  if (!out) return fail(kEInval, "out is null");
  *out = nullptr;
  if (npart <= 0 || nphase < 0 || !off || (!idx && off[(long)(nphase + 1) * npart] > 0))
    return fail(kEInval, "bad task list arguments");
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  int rc = arith == MPKG_ARITH_DF64 ? fail(kEInval, "the tasks executor computes in FP64 only")
                                    : plan_common(p, n, ptr, col, val, nlevel, arith);
  if (!rc) {
    p->exec = MPKG_EXEC_TASKS;
    p->npart = npart;
    p->nphase = nphase;
    rc = build_task_device(p, npart, nphase, off, idx);
  }
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

int mpkg_plan_pa1(int n, const int *ptr, const int *col, const double *val, const int *part,
                  int npart, int nlevel, int exec, int arith, mpkg_plan **out) {
  clear_error();
  if (!out) return fail(kEInval, "out is null");
  *out = nullptr;
  if (!part || npart <= 0) return fail(kEInval, "bad partition");
  if (exec != MPKG_EXEC_TILES && exec != MPKG_EXEC_TASKS)
    return fail(kEInval, "PA1 plans use the tiles or tasks executor");
  int rc = check_csr(n, ptr, col);
  if (rc) return rc;
  Csr g;
  g.n = n;
  g.ptr.assign(ptr, ptr + n + 1);
  g.col.assign(col, col + ptr[n]);
  std::vector<int> pv(part, part + n);
  for (int q : pv) if (q < 0 || q >= npart) return fail(kERange, "part id out of range");
  if (exec == MPKG_EXEC_TASKS) {
    TaskLists tl;
    bool tasks_on_gpu = false;
    if ((rc = build_pa1_tasks_gpu(g, pv, npart, nlevel, &tl, &tasks_on_gpu))) return rc;
    return mpkg_plan_tasks(n, ptr, col, val, npart, nlevel, 0, tl.off.data(), tl.idx.data(), arith, out);
  }
  TilePlan tp;
  bool prep_on_gpu = false;
  if ((rc = build_tile_plan_gpu(g, pv, npart, nlevel, &tp, &prep_on_gpu))) return rc;
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  rc = plan_common(p, n, ptr, col, val, nlevel, arith);
  if (!rc) {
    p->exec = MPKG_EXEC_TILES;
    p->npart = npart;
    rc = build_tile_device(p, tp, ptr);
  }
  if (!rc && p->tiles_smem && p->arith == MPKG_ARITH_DF64) {
    rc = p->valued ? set_tiles_df_attr<true, true>(p->tiles_smem_bytes)
                   : set_tiles_df_attr<false, true>(p->tiles_smem_bytes);
  } else if (!rc && p->tiles_smem) {
    if (p->arith == MPKG_ARITH_SEPARATE) {
      rc = p->valued ? set_tiles_attr<MPKG_ARITH_SEPARATE, true, true>(p->tiles_smem_bytes)
                     : set_tiles_attr<MPKG_ARITH_SEPARATE, false, true>(p->tiles_smem_bytes);
    } else {
      rc = p->valued ? set_tiles_attr<MPKG_ARITH_FMA, true, true>(p->tiles_smem_bytes)
                     : set_tiles_attr<MPKG_ARITH_FMA, false, true>(p->tiles_smem_bytes);
    }
  }
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

int mpkg_plan_pipe(int n, const int *ptr, const int *col, const double *val, int nlevel,
                   int chunk, int arith, mpkg_plan **out) {
  clear_error();
  if (!out) return fail(kEInval, "out is null");
  *out = nullptr;
  if (chunk <= 0) chunk = kPipeChunk;
  if (chunk != kPipeChunk) return fail(kEInval, "the pipeline executor uses 256-row chunks");
  int rc = check_csr(n, ptr, col);
  if (rc) return rc;
  Csr g;
  g.n = n;
  g.ptr.assign(ptr, ptr + n + 1);
  g.col.assign(col, col + ptr[n]);
  PipePlan pp;
  if ((rc = build_pipe_plan(g, nlevel, chunk, &pp))) return rc;
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  rc = plan_common(p, n, ptr, col, val, nlevel, arith);
  if (!rc) {
    p->exec = MPKG_EXEC_PIPE;
    p->npart = pp.nchunk;
    p->rows_computed = (long)n * nlevel;
    PipeArgs &a = p->pipe;
    a.n = n; a.nlevel = nlevel; a.chunk = chunk; a.nchunk = pp.nchunk;
    a.ngroups = (pp.nchunk + kPipeGroup - 1) / kPipeGroup;
    int maxnnz = 0;
    for (int c = 0; c < pp.nchunk; c++) {
      int r1 = std::min(n, (c + 1) * chunk);
      maxnnz = std::max(maxnnz, ptr[r1] - ptr[c * chunk]);
    }
    a.max_chunk_nnz = std::max(maxnnz, 1);
    p->pipe_smem_bytes = pipe_smem_size(chunk, a.max_chunk_nnz, p->valued, 8);
    // dependencies in counter groups, and the reach they imply in chunks
    std::vector<int> glo(pp.nchunk), ghi(pp.nchunk);
    long reach = 0;
    for (int c = 0; c < pp.nchunk; c++) {
      glo[c] = pp.dep_lo[c] / kPipeGroup;
      ghi[c] = pp.dep_hi[c] / kPipeGroup;
      long hi_chunk = std::min<long>((long)ghi[c] * kPipeGroup + kPipeGroup - 1, pp.nchunk - 1);
      reach = std::max(reach, std::max(hi_chunk - c, (long)c - (long)glo[c] * kPipeGroup));
    }
    int *dlo, *dhi;
    unsigned int *ticket, *counts;
    const size_t ncount = (size_t)(nlevel + 1) * a.ngroups;
    if (!rc) rc = dev_copy(p, &dlo, glo.data(), glo.size());
    if (!rc) rc = dev_copy(p, &dhi, ghi.data(), ghi.size());
    if (!rc) rc = dev_alloc(p, &ticket, 1);
    if (!rc) rc = dev_alloc(p, &counts, ncount);
    if (!rc && p->arith == MPKG_ARITH_DF64) {
      float2 *ring;
      rc = dev_alloc(p, &ring, 2 * (size_t)n);
      a.ring = ring;
      a.coef2 = p->d_coef2;
    }
    if (!rc) {
      cudaMemset(counts, 0, sizeof(unsigned int) * ncount);
      a.gdep_lo = dlo; a.gdep_hi = dhi; a.ticket = ticket; a.counts = counts;
      a.ptr = p->d_ptr; a.col = p->d_col; a.coef = p->d_coef; a.err = p->d_err;
      a.bulk_ok = true;  // cudaMalloc'd arrays are 256-byte aligned
    }
    if (!rc) {
      int grid = 0;
      if (p->arith == MPKG_ARITH_DF64)
        rc = p->valued ? pipe_setup_df<true>(p, &grid) : pipe_setup_df<false>(p, &grid);
      else if (p->arith == MPKG_ARITH_SEPARATE)
        rc = p->valued ? pipe_setup_t<MPKG_ARITH_SEPARATE, true>(p, &grid) : pipe_setup_t<MPKG_ARITH_SEPARATE, false>(p, &grid);
      else
        rc = p->valued ? pipe_setup_t<MPKG_ARITH_FMA, true>(p, &grid) : pipe_setup_t<MPKG_ARITH_FMA, false>(p, &grid);
      if (!rc) {
        p->pipe_reach = (int)reach;
        // topological item order: key = chunk + D*(level-1), levels ascending
        // within a key; D leaves about one grid's worth of items between an
        // item and its latest dependency
        const long D = reach + std::max<long>(1, ((long)grid + nlevel - 1) / nlevel);
        std::vector<int> items;
        items.reserve((size_t)pp.nchunk * nlevel);
        for (long K = 0; K < pp.nchunk + D * (nlevel - 1); K++)
          for (int l = 1; l <= nlevel; l++) {
            const long c = K - D * (l - 1);
            if (c >= 0 && c < pp.nchunk) items.push_back((l << 26) | (int)c);
          }
        int *ditems = nullptr;
        rc = dev_copy(p, &ditems, items.data(), items.size());
        a.items = ditems;
        a.nitems = (int)items.size();
        p->pipe_grid = (int)std::min<long>(grid, (long)items.size());
      }
    }
  }
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

int mpkg_plan_spmv(int n, const int *ptr, const int *col, const double *val, int nlevel, int arith,
                   mpkg_plan **out) {
  clear_error();
  if (!out) return fail(kEInval, "out is null");
  *out = nullptr;
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  int rc = plan_common(p, n, ptr, col, val, nlevel, arith, true);
  if (!rc) {
    p->exec = MPKG_EXEC_SPMV;
    p->npart = 1;
    p->rows_computed = (long)n * nlevel;
  }
  if (!rc && arith == MPKG_ARITH_DF64) {
    float2 *ring = nullptr;
    rc = dev_alloc(p, &ring, (size_t)2 * n);
    p->sp_ring = ring;
  }
  if (!rc && arith == MPKG_ARITH_FIXED) {
    int maxlen = 0;
    for (int i = 0; i < n; i++) maxlen = std::max(maxlen, ptr[i + 1] - ptr[i]);
    if (maxlen > 255) rc = fail(kERange, "fixed-point form: rows are limited to 255 entries");
    while ((1 << p->sp_dbits) < maxlen) p->sp_dbits++;
    std::vector<unsigned long long> mul(256, 0);
    for (int d = 2; d < 256; d++) mul[d] = ~0ull / (unsigned long long)d + 1;  // ceil(2^64 / d)
    long long *ring = nullptr;
    if (!rc) rc = dev_copy(p, &p->sp_mul, mul.data(), mul.size());
    if (!rc) rc = dev_alloc(p, &p->sp_word, 2);
    if (!rc) rc = dev_alloc(p, &ring, (size_t)2 * n);
    p->sp_ring = ring;
  }
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

int mpkg_plan_bufs(const char *dir, int npart, int arith, mpkg_plan **out) {
  clear_error();
  if (!out || !dir || npart <= 0) return fail(kEInval, "bad argument");
  *out = nullptr;
  if (arith != MPKG_ARITH_FMA && arith != MPKG_ARITH_SEPARATE)
    return fail(kEInval, "rank buffers run in FP64 (fma or separate)");
  std::vector<RankBuffers> bufs(npart);
  int rc;
  for (int r = 0; r < npart; r++)
    if ((rc = read_rank_buffers(std::string(dir) + "/rank" + std::to_string(r) + ".bufs", &bufs[r]))) return rc;
  if ((rc = check_rank_buffers(bufs))) return rc;
  const int n = bufs[0].n, nlevel = bufs[0].nlevel, nphase = bufs[0].nphase, P = npart;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  p->exec = MPKG_EXEC_BUFS;
  p->n = n; p->nlevel = nlevel; p->nphase = nphase; p->npart = P;
  p->arith = arith; p->valued = true;
  rc = cudaGetDevice(&p->device) == cudaSuccess ? kOk : fail(kECuda, "cudaGetDevice failed");
  if (!rc && cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(kECuda, "stream creation failed");
  std::vector<long> off(P + 1, 0);
  for (int r = 0; r < P; r++) off[r + 1] = off[r] + bufs[r].buf_count;
  // input gather, output scatter
  std::vector<long> in_dst, in_src, out_src, out_dst;
  for (int r = 0; r < P; r++) {
    const RankBuffers &b = bufs[r];
    for (int i = 0; i < b.rcount[0]; i++) {
      in_dst.push_back(off[r] + b.rbuf_offsets[0] + i);
      in_src.push_back(b.idx_buf[b.rbuf_offsets[0] + i]);
    }
    for (int i = 0; i < b.buf_count; i++) {
      out_src.push_back(off[r] + i);
      out_dst.push_back(b.idx_buf[i]);
    }
  }
  // communication per phase: receive slot of dst from src's send list
  std::vector<long> cm_dst, cm_src, cm_off(nphase + 2, 0);
  for (int ph = 0; ph <= nphase; ph++) {
    cm_off[ph] = (long)cm_dst.size();
    if (ph == 0) continue;
    for (int dst = 0; dst < P; dst++)
      for (int src = 0; src < P; src++) {
        const long k = (long)P * ph;
        const int cnt = bufs[dst].recvcounts[k + src];
        for (int t = 0; t < cnt; t++) {
          cm_dst.push_back(off[dst] + bufs[dst].rbuf_offsets[ph] + bufs[dst].rdispls[k + src] + t);
          cm_src.push_back(off[src] + bufs[src].idx_sbuf[bufs[src].sbuf_offsets[ph] + bufs[src].sdispls[k + dst] + t]);
        }
      }
  }
  cm_off[nphase + 1] = (long)cm_dst.size();
  // computation rows, segmented per (phase, rank) by level
  std::vector<long> list_seg((size_t)(nphase + 1) * P + 1, 0), seg_off, row_dst, row_ptr(1, 0), gcol;
  std::vector<double> gval;
  long rows_total = 0;
  for (int ph = 0; ph <= nphase; ph++)
    for (int r = 0; r < P; r++) {
      const RankBuffers &b = bufs[r];
      list_seg[(size_t)ph * P + r] = (long)seg_off.size();
      const long *idx_m = b.idx_buf.data() + b.mbuf_offsets[ph];
      const long *mptr = b.mptr_buf.data() + b.mptr_offsets[ph];
      const long *mcol = b.mcol_buf.data() + b.mcol_offsets[ph];
      const double *mval = b.mval_buf.data() + b.mcol_offsets[ph];
      long cur = -1;
      for (int mi = 0; mi < b.mcount[ph]; mi++) {
        const long level = idx_m[mi] / n;
        if (level < cur) { rc = rc ? rc : fail(kEFormat, "rank buffer rows are not level-major"); break; }
        if (level != cur) {
          seg_off.push_back((long)row_dst.size());
          cur = level;
        }
        row_dst.push_back(off[r] + b.mbuf_offsets[ph] + mi);
        for (long mj = mptr[mi]; mj < mptr[mi + 1]; mj++) {
          gcol.push_back(off[r] + mcol[mj]);
          gval.push_back(mval[mj]);
        }
        row_ptr.push_back((long)gcol.size());
        rows_total++;
      }
    }
  list_seg[(size_t)(nphase + 1) * P] = (long)seg_off.size();
  seg_off.push_back((long)row_dst.size());
  p->rows_computed = rows_total;
  p->nnz = (long)gcol.size();
  if (!rc) rc = dev_alloc(p, &p->b_vall, std::max<long>(off[P], 1));
  if (!rc) rc = dev_copy(p, &p->b_in_dst, in_dst.data(), in_dst.size());
  if (!rc) rc = dev_copy(p, &p->b_in_src, in_src.data(), in_src.size());
  if (!rc) rc = dev_copy(p, &p->b_out_src, out_src.data(), out_src.size());
  if (!rc) rc = dev_copy(p, &p->b_out_dst, out_dst.data(), out_dst.size());
  if (!rc) rc = dev_copy(p, &p->b_cm_dst, cm_dst.data(), cm_dst.size());
  if (!rc) rc = dev_copy(p, &p->b_cm_src, cm_src.data(), cm_src.size());
  if (!rc) rc = dev_copy(p, &p->b_list_seg, list_seg.data(), list_seg.size());
  if (!rc) rc = dev_copy(p, &p->b_seg_off, seg_off.data(), seg_off.size());
  if (!rc) rc = dev_copy(p, &p->b_row_dst, row_dst.data(), row_dst.size());
  if (!rc) rc = dev_copy(p, &p->b_row_ptr, row_ptr.data(), row_ptr.size());
  if (!rc) rc = dev_copy(p, &p->b_gcol, gcol.data(), gcol.size());
  if (!rc) rc = dev_copy(p, &p->b_gval, gval.data(), gval.size());
  if (!rc) rc = dev_alloc(p, &p->d_err, 1);
  if (!rc && cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess) rc = fail(kECuda, "memset failed");
  p->b_nin = (long)in_dst.size();
  p->b_nout = (long)out_src.size();
  p->b_cm_off = cm_off;
  // every (level, vertex) of levels 1..nlevel must be produced by some rank
  std::vector<unsigned char> cov((size_t)n * (nlevel + 1), 0);
  for (long v : out_dst) cov[(size_t)v] = 1;
  p->full_coverage = true;
  for (size_t e = (size_t)n; e < cov.size(); e++)
    if (!cov[e]) { p->full_coverage = false; break; }
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

}  // extern "C"

namespace {
thread_local int g_wave_ctas_per_sm = 0;  // mpkg_plan_wave_ctas: cap on resident CTAs per SM (0: occupancy)
int plan_wave_impl(int n, const int *ptr, const int *col, const double *val, int nlevel, int arith,
                   int occ_value_type, mpkg_plan **out);
const void *mix_wave_kernel_ptr(int value_type, bool rel, bool uni, bool stream);
}  // namespace

extern "C" {

int mpkg_plan_wave(int n, const int *ptr, const int *col, const double *val, int nlevel, int arith,
                   mpkg_plan **out) {
  return plan_wave_impl(n, ptr, col, val, nlevel, arith, -1, out);
}

int mpkg_plan_wave_ctas(int n, const int *ptr, const int *col, const double *val, int nlevel, int arith,
                        int ctas_per_sm, mpkg_plan **out) {
  if (ctas_per_sm <= 0 || ctas_per_sm > 32) return fail(kEInval, "ctas_per_sm must be in [1, 32]");
  g_wave_ctas_per_sm = ctas_per_sm;
  const int rc = plan_wave_impl(n, ptr, col, val, nlevel, arith, -1, out);
  g_wave_ctas_per_sm = 0;
  return rc;
}

}  // extern "C"

namespace {

// occ_value_type >= 0: size the grid for the mixed-precision kernel of that
// value type instead of the plan's own kernel
int plan_wave_impl(int n, const int *ptr, const int *col, const double *val, int nlevel, int arith,
                   int occ_value_type, mpkg_plan **out) {
  clear_error();
  if (!out) return fail(kEInval, "out is null");
  *out = nullptr;
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  p->exec = MPKG_EXEC_WAVE;
  int rc = plan_common(p, n, ptr, col, val, nlevel, arith, true);
  if (!rc && arith == MPKG_ARITH_FIXED) {
    int maxlen = 0;
    for (int i = 0; i < n; i++) maxlen = std::max(maxlen, ptr[i + 1] - ptr[i]);
    if (maxlen > 255) rc = fail(kERange, "fixed-point form: rows are limited to 255 entries");
    int dbits = 0;
    while ((1 << dbits) < maxlen) dbits++;
    p->wave.fix_dbits = dbits;
  }
  if (!rc) {
    bool rel = true;
    for (int i = 0; i < n && rel; i++) {
      if (ptr[i + 1] - ptr[i] > 65535) rc = fail(kERange, "wavefront executor: a row has more than 65535 entries");
      for (int q = ptr[i]; q < ptr[i + 1]; q++)
        if (col[q] - i < -32768 || col[q] - i > 32767) { rel = false; break; }
    }
    p->wave_rel = rel;
    if (!rc && arith == MPKG_ARITH_FIXED && !rel)
      rc = fail(kERange, "fixed-point form: every |column - row| must be below 32768");
    // shared offset lists pay where values dominate the bytes; the pattern
    // operator keeps the per-lane layout (fewer instructions per entry)
    p->wave_uni = rel && val != nullptr;
  }
  int grid = 0;
  if (!rc)
    rc = wave_occupancy(p, occ_value_type >= 0 ? mix_wave_kernel_ptr(occ_value_type, p->wave_rel, p->wave_uni, false)
                                               : (const void *)wave_kernel_ptr(p), &grid);
  if (!rc && g_wave_ctas_per_sm > 0) {
    int nsm = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
    grid = std::min(grid, g_wave_ctas_per_sm * nsm);
  }
  if (!rc) {
    const long nnz = ptr[n];
    const int nslice = (n + 31) / 32;
    grid = (int)std::max<long>(1, std::min<long>(grid, nslice));
    // contiguous row ranges of (nearly) equal nonzeros, starting on slices
    auto ranges = [&](int g) {
      std::vector<int> r(g + 1, 0);
      for (int b = 1; b < g; b++) {
        const long target = nnz * b / g;
        int q = (int)(std::lower_bound(ptr, ptr + n + 1, (int)target) - ptr);
        q = std::min(n, (q + 16) / 32 * 32);
        r[b] = std::max(q, r[b - 1]);
      }
      r[g] = n;
      return r;
    };
    std::vector<int> lo = ranges(grid);
    // sliced ELL copy of the matrix: values (and int32 columns) 32 x width
    // per slice; int16 offsets pattern-compressed (one list per slice whose
    // rows share it)
    std::vector<long> soff(nslice + 1, 0), roff(nslice + 1, 0);
    std::vector<unsigned char> runi(nslice, 0);
    std::vector<unsigned short> len(n);
    for (int sl = 0; sl < nslice; sl++) {
      const int i0 = sl * 32, i1 = std::min(n, sl * 32 + 32);
      int w = 0;
      for (int i = i0; i < i1; i++) w = std::max(w, ptr[i + 1] - ptr[i]);
      soff[sl + 1] = soff[sl] + 32L * w;
      bool uni = p->wave_uni && i1 - i0 == 32;
      for (int i = i0 + 1; i < i1 && uni; i++) {
        if (ptr[i + 1] - ptr[i] != ptr[i0 + 1] - ptr[i0]) { uni = false; break; }
        for (int t = 0; t < ptr[i + 1] - ptr[i]; t++)
          if (col[ptr[i] + t] - i != col[ptr[i0] + t] - i0) { uni = false; break; }
      }
      runi[sl] = uni ? (unsigned char)std::min(w + 1, 255) : 0;
      roff[sl + 1] = roff[sl] + (uni ? (w + 7) / 8 * 8 : 32L * w);
    }
    std::vector<int> scol(p->wave_rel ? 0 : soff[nslice], 0);
    std::vector<short> srel(p->wave_rel ? roff[nslice] : 0, 0);
    std::vector<double> sval(val ? soff[nslice] : 0, 0.0);
    for (int i = 0; i < n; i++) {
      len[i] = (unsigned short)(ptr[i + 1] - ptr[i]);
      const int sl = i / 32;
      const long e0 = soff[sl] + (i % 32);
      for (int t = 0; t < len[i]; t++) {
        if (p->wave_rel) {
          if (runi[sl]) srel[roff[sl] + t] = (short)(col[ptr[i] + t] - i);
          else srel[roff[sl] + 32L * t + (i % 32)] = (short)(col[ptr[i] + t] - i);
        } else {
          scol[e0 + 32L * t] = col[ptr[i] + t];
        }
        if (val) sval[e0 + 32L * t] = val[ptr[i] + t];
      }
    }
    // stage each CTA's int16 offsets and uint8 lengths in shared memory when
    // the slabs fit next to the kernel's own shared memory at this occupancy
    int maxlen = 0;
    for (int i = 0; i < n; i++) maxlen = std::max(maxlen, ptr[i + 1] - ptr[i]);
    if (p->wave_rel && occ_value_type < 0 && maxlen <= 255) {
      long relb = 0, lenb = 0;
      for (int b = 0; b < grid; b++) {
        if (lo[b] >= lo[b + 1]) continue;
        relb = std::max(relb, 2 * (roff[(lo[b + 1] + 31) / 32] - roff[lo[b] / 32]));
        lenb = std::max<long>(lenb, lo[b + 1] - lo[b]);
      }
      relb = (relb + 15) / 16 * 16;
      lenb = (lenb + 15) / 16 * 16;
      long nsl = 0;
      for (int b = 0; b < grid; b++)
        if (lo[b] < lo[b + 1]) nsl = std::max<long>(nsl, (lo[b + 1] + 31) / 32 - lo[b] / 32);
      nsl = (nsl + 15) / 16 * 16;
      int nsm = 0, per_sm = 0;
      CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
      p->wave.stage_rel_bytes = (int)relb;
      p->wave.stage_len_bytes = (int)lenb;
      p->wave.stage_slices = (int)nsl;
      const size_t dyn = wave_dyn_smem(p);
      const void *k = wave_kernel_ptr(p);
      bool ok = dyn <= 200 * 1024 &&
                cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) == cudaSuccess &&
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, dyn) == cudaSuccess &&
                (long)per_sm * nsm >= grid;
      if (!ok) {
        cudaGetLastError();
        p->wave.stage_rel_bytes = 0;
        p->wave.stage_len_bytes = 0;
        p->wave.stage_slices = 0;
      }
    }
    // CTA owning column c: the last b' with lo[b'] <= c (empty ranges skipped)
    auto owner = [&](int c) { return (int)(std::upper_bound(lo.begin(), lo.end() - 1, c) - lo.begin()) - 1; };
    // the exact set of other CTAs whose rows CTA b reads (a CTA's own rows
    // of the previous level are ordered by its barrier)
    std::vector<std::vector<int>> reads(grid);
    {
      std::vector<int> seen(grid, -1);
      for (int b = 0; b < grid; b++)
        for (long q = ptr[lo[b]]; q < ptr[lo[b + 1]]; q++) {
          const int c = col[q];
          if (c >= lo[b] && c < lo[b + 1]) continue;
          const int o = owner(c);
          if (seen[o] != b) { seen[o] = b; reads[b].push_back(o); }
        }
    }
    const bool ring = arith == MPKG_ARITH_DF64 || arith == MPKG_ARITH_FIXED;
    std::vector<std::vector<int>> waits(reads);
    if (ring)  // symmetric closure: a ring slot is reused two levels later, so
               // also wait for the CTAs that read this one's rows
      for (int c = 0; c < grid; c++)
        for (int b : reads[c]) waits[b].push_back(c);
    std::vector<int> dptr(grid + 1, 0), didx;
    long reach = 0;
    for (int b = 0; b < grid; b++) {
      std::sort(waits[b].begin(), waits[b].end());
      waits[b].erase(std::unique(waits[b].begin(), waits[b].end()), waits[b].end());
      for (int c : waits[b]) {
        didx.push_back(c);
        reach = std::max<long>(reach, std::abs(c - b));
      }
      dptr[b + 1] = (int)didx.size();
    }
    if (didx.empty()) didx.push_back(0);
    p->wave_grid = grid;
    p->pipe_grid = grid;
    WaveArgs &w = p->wave;
    w.n = n; w.nlevel = nlevel; w.nblk = grid; w.base = 0; w.err = p->d_err;
    if (!val) { w.rdeg = p->d_coef; w.rdeg2 = p->d_coef2; }
    std::vector<double> lut(256, 0.0);
    for (int d = 1; d < 256; d++) lut[d] = 1.0 / d;  // as the plan's 1/deg (mpk2/mpkexec.c:28)
    int *d_lo = nullptr, *d_dlo = nullptr, *d_dhi = nullptr;
    rc = dev_copy(p, (long **)&w.sell_off, soff.data(), soff.size());
    if (!rc) rc = dev_copy(p, (unsigned short **)&w.len, len.data(), len.size());
    if (!rc && !scol.empty()) rc = dev_copy(p, (int **)&w.scol, scol.data(), scol.size());
    if (!rc && !srel.empty()) rc = dev_copy(p, (short **)&w.srel, srel.data(), srel.size());
    if (!rc && p->wave_rel) rc = dev_copy(p, (long **)&w.rel_off, roff.data(), roff.size());
    if (!rc && p->wave_rel) rc = dev_copy(p, (unsigned char **)&w.runi, runi.data(), runi.size());
    if (!rc && val) rc = dev_copy(p, (double **)&w.sval, sval.data(), sval.size());
    if (!rc) rc = dev_copy(p, (double **)&w.lut, lut.data(), lut.size());
    if (!rc && arith == MPKG_ARITH_DF64) {
      float2 *l2 = nullptr;
      rc = dev_alloc(p, &l2, 256);
      if (!rc) {
        split_kernel<<<1, 256, 0, p->stream>>>(w.lut, l2, 256);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(p->stream) != cudaSuccess)
          rc = fail(kECuda, "split of the degree table failed");
      }
      w.lut2 = l2;
    }
    if (!rc && val && arith == MPKG_ARITH_DF64) {
      float2 *sv2 = nullptr;
      rc = dev_alloc(p, &sv2, sval.size());
      if (!rc) {
        split_kernel<<<256, 256, 0, p->stream>>>(w.sval, sv2, (long)sval.size());
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(p->stream) != cudaSuccess)
          rc = fail(kECuda, "split of the sliced values failed");
      }
      w.sval2 = sv2;
    }
    if (!rc) rc = dev_copy(p, &d_lo, lo.data(), lo.size());
    if (!rc) rc = dev_copy(p, &d_dlo, dptr.data(), dptr.size());
    if (!rc) rc = dev_copy(p, &d_dhi, didx.data(), didx.size());
    if (!rc) rc = dev_alloc(p, &w.flags, (size_t)grid);
    if (!rc && ring) rc = dev_alloc(p, &w.ring, (size_t)2 * n);
    if (!rc && arith == MPKG_ARITH_FIXED) {
      std::vector<unsigned long long> mul(256, 0);
      for (int d = 2; d < 256; d++) mul[d] = ~0ull / (unsigned long long)d + 1;  // ceil(2^64 / d)
      rc = dev_copy(p, (unsigned long long **)&w.fix_mul, mul.data(), mul.size());
      if (!rc) rc = dev_alloc(p, &w.fix_word, 1);
      if (!rc && cudaMemset(w.fix_word, 0, sizeof(unsigned long long)) != cudaSuccess)
        rc = fail(kECuda, "memset failed");
    }
    w.row_lo = d_lo; w.dep_ptr = d_dlo; w.dep_idx = d_dhi;
    p->pipe_reach = (int)reach;
    p->rows_computed = (long)n * nlevel;
  }
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

}  // namespace

extern "C" {

namespace {

// Device state of one (lpr, vw, budget, grid) configuration of a batch plan.
int batch_configure(mpkg_plan *p, const BatchHost &h, int lpr, int vw, long budget, int grid, bool staged,
                    int threads, size_t smem) {
  std::vector<int> lo, dlo, dhi, win;
  int ngroup = 0;
  const long cap_rows = staged ? (long)(smem / (4 * (size_t)p->batch.nrhs)) : 0;
  batch_layout(h, p->batch.nrhs, budget, grid, cap_rows, &lo, &dlo, &dhi, &win, &ngroup);
  BatchArgs &a = p->batch;
  // previous layout arrays are freed with the plan (owned list); small
  int *d_lo = nullptr, *d_dlo = nullptr, *d_dhi = nullptr, *d_win = nullptr;
  unsigned int *d_flags = nullptr;
  int rc = dev_copy(p, &d_lo, lo.data(), lo.size());
  if (!rc) rc = dev_copy(p, &d_dlo, dlo.data(), dlo.size());
  if (!rc) rc = dev_copy(p, &d_dhi, dhi.data(), dhi.size());
  if (!rc && staged) rc = dev_copy(p, &d_win, win.data(), win.size());
  if (!rc) rc = dev_alloc(p, &d_flags, (size_t)grid);
  if (!rc && staged &&
      cudaFuncSetAttribute((const void *)batch_stage_kernel_for(lpr, vw),
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    rc = fail(kECuda, "shared memory attribute");
  if (rc) return rc;
  a.row_lo = d_lo; a.dep_ptr = d_dlo; a.dep_idx = d_dhi; a.flags = d_flags; a.win = d_win;
  a.nblk = grid; a.ngroup = ngroup; a.base = 0;
  p->batch_lpr = lpr; p->batch_vw = vw; p->batch_group_bytes = budget;
  p->batch_staged = staged; p->batch_threads = threads; p->batch_smem = staged ? smem : 0;
  p->pipe_grid = grid;
  if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }
  if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
  p->graph_ok = false;
  p->graph_key = nullptr;
  return kOk;
}

}  // namespace

int mpkg_plan_batch(int nmat, const int *n, const int *const *ptr, const int *const *col, const float *const *val,
                    int nrhs, int nlevel, int tune, mpkg_plan **out) {
  clear_error();
  if (!out || nmat <= 0 || !n || !ptr || !col || !val) return fail(kEInval, "bad argument");
  *out = nullptr;
  if (nlevel <= 0 || nlevel > 64) return fail(kEInval, "nlevel must be in [1, 64]");
  if (nrhs <= 0 || nrhs > 128 || (nrhs & (nrhs - 1)) != 0) return fail(kEInval, "nrhs must be a power of two <= 128");
  if (tune < MPKG_BATCH_DEFAULT || tune > MPKG_BATCH_STAGED4) return fail(kEInval, "unknown tune mode");
  BatchHost h;
  h.mat_row0.assign(nmat + 1, 0);
  long nnz = 0;
  for (int m = 0; m < nmat; m++) {
    int rc = check_csr(n[m], ptr[m], col[m]);
    if (rc) return rc;
    if (!val[m]) return fail(kEInval, "the batched form needs matrix values");
    h.mat_row0[m + 1] = h.mat_row0[m] + n[m];
    nnz += ptr[m][n[m]];
  }
  h.N = h.mat_row0[nmat];
  if (h.N > INT32_MAX / 2 || nnz > INT32_MAX) return fail(kERange, "batch exceeds 2^30 rows or 2^31 nonzeros");
  if ((double)(nlevel + 1) * h.N * nrhs * 4 > 1.5e11) return fail(kERange, "batch vectors exceed 150 GB");
  h.ptr.resize(h.N + 1);
  h.col.resize(nnz);
  h.val.resize(nnz);
  long q = 0;
  for (int m = 0; m < nmat; m++) {
    const long r0 = h.mat_row0[m];
    for (int i = 0; i < n[m]; i++) {
      h.ptr[r0 + i] = (int)q;
      for (int t = ptr[m][i]; t < ptr[m][i + 1]; t++, q++) {
        h.col[q] = (int)(col[m][t] + r0);
        h.val[q] = val[m][t];
      }
    }
  }
  h.ptr[h.N] = (int)q;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  p->exec = MPKG_EXEC_BATCH;
  p->n = (int)h.N; p->nlevel = nlevel; p->valued = true; p->arith = MPKG_ARITH_FMA;
  p->nnz = nnz;
  p->rows_computed = h.N * nlevel;
  p->batch_nmat = nmat;
  int rc = cudaGetDevice(&p->device) == cudaSuccess ? kOk : fail(kECuda, "cudaGetDevice failed");
  if (!rc && cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(kECuda, "stream creation failed");
  BatchArgs &a = p->batch;
  a.N = h.N; a.nrhs = nrhs; a.nlevel = nlevel;
  int *d_ptr = nullptr, *d_col = nullptr;
  float *d_val = nullptr;
  if (!rc) rc = dev_copy(p, &d_ptr, h.ptr.data(), h.ptr.size());
  if (!rc) rc = dev_copy(p, &d_col, h.col.data(), h.col.size());
  if (!rc) rc = dev_copy(p, &d_val, h.val.data(), h.val.size());
  if (!rc) rc = dev_alloc(p, &p->d_err, 1);
  if (!rc && cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess) rc = fail(kECuda, "memset failed");
  a.ptr = d_ptr; a.col = d_col; a.val = d_val; a.err = p->d_err;
  int nsm = 0;
  if (!rc && cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess)
    rc = fail(kECuda, "device query failed");
  // candidates: lanes x vector width covering nrhs, group budget, CTAs per
  // SM; and the staged kernel at one or two CTAs per SM
  struct Cand { int lpr, vw; long budget; int grid; bool staged; int threads; size_t smem; };
  std::vector<Cand> cands;
  for (int vw : {4, 2, 1}) {
    if (nrhs % vw) continue;
    const int lpr = nrhs / vw;
    if (lpr > 32) continue;
    int per_sm = 0;
    if (!rc && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel_for(lpr, vw), 256, 0) != cudaSuccess)
      rc = fail(kECuda, "occupancy query failed");
    if (rc || per_sm <= 0) continue;
    for (long budget : {32L << 20, 64L << 20, 1L << 40})
      for (int occ : {per_sm, std::max(1, per_sm / 2)}) {
        cands.push_back({lpr, vw, budget, std::max(1, std::min<int>(occ * nsm, (int)std::min<long>(h.N, INT32_MAX))),
                         false, 256, 0});
        if (occ == std::max(1, per_sm / 2)) break;
      }
  }
  if (!rc && nrhs % 4 == 0 && nrhs / 4 <= 32) {
    int sm_per_sm = 0, sm_optin = 0;
    if (cudaDeviceGetAttribute(&sm_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, p->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sm_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device) != cudaSuccess)
      rc = fail(kECuda, "device query failed");
    for (int ctas : {1, 2, 4}) {
      if (rc) break;
      const int threads = 1024 / ctas;
      // a window of whole rows within the SM's share, less the static part and the per-CTA reserve
      size_t smem = std::min<size_t>((size_t)sm_optin, (size_t)sm_per_sm / ctas) - 2048;
      smem -= smem % (4 * (size_t)nrhs);
      BatchKernel k = batch_stage_kernel_for(nrhs / 4, 4);
      int per_sm = 0;
      if (cudaFuncSetAttribute((const void *)k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
              cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      if (per_sm <= 0) continue;
      for (long budget : {32L << 20, 64L << 20, 1L << 40})
        cands.push_back({nrhs / 4, 4, budget, std::max(1, std::min<int>(per_sm * nsm, (int)std::min<long>(h.N, INT32_MAX))),
                         true, threads, smem});
    }
  }
  if (!rc && cands.empty()) rc = fail(kEInval, "no kernel configuration for this nrhs");
  Cand best = cands.empty() ? Cand{1, 1, 0, 1, false, 256, 0} : cands[0];
  if (!rc && tune >= MPKG_BATCH_STAGED) {  // untimed staged configuration
    const int want_threads = tune == MPKG_BATCH_STAGED ? 1024 : tune == MPKG_BATCH_STAGED2 ? 512 : 256;
    bool found = false;
    for (const Cand &c : cands)
      if (c.staged && c.threads == want_threads && c.budget == (64L << 20)) {
        best = c;
        found = true;
        break;
      }
    if (!found) rc = fail(kEInval, "no staged configuration for this nrhs and device");
  } else if (!rc && tune == MPKG_BATCH_TUNE && cands.size() > 1) {
    // time every candidate on the plan's own matrices (zero input; the
    // arithmetic does not depend on the values)
    float *scratch = nullptr;
    const size_t total = (size_t)(nlevel + 1) * h.N * nrhs;
    if (cudaMalloc(&scratch, sizeof(float) * total) != cudaSuccess) rc = fail(kENoMem, "autotune scratch");
    if (!rc && cudaMemsetAsync(scratch, 0, sizeof(float) * total, p->stream) != cudaSuccess)
      rc = fail(kECuda, "memset failed");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!rc && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
      rc = fail(kECuda, "event creation failed");
    float best_ms = 1e30f;
    auto t_start = std::chrono::steady_clock::now();
    for (const Cand &c : cands) {
      if (rc) break;
      if ((rc = batch_configure(p, h, c.lpr, c.vw, c.budget, c.grid, c.staged, c.threads, c.smem))) break;
      for (int w = 0; w < 2 && !rc; w++) rc = batch_launch_raw(p, scratch, p->stream, false);
      if (!rc && cudaEventRecord(e0, p->stream) != cudaSuccess) rc = fail(kECuda, "event record");
      for (int w = 0; w < 3 && !rc; w++) rc = batch_launch_raw(p, scratch, p->stream, false);
      if (!rc && cudaEventRecord(e1, p->stream) != cudaSuccess) rc = fail(kECuda, "event record");
      if (!rc) rc = mpkg_sync(p, p->stream);
      float ms = 0.f;
      if (!rc && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = fail(kECuda, "event time");
      if (!rc && ms < best_ms) { best_ms = ms; best = c; }
    }
    p->batch_tune_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (scratch) cudaFree(scratch);
  }
  p->batch_candidates = (int)cands.size();
  if (!rc)
    rc = batch_configure(p, h, best.lpr, best.vw, best.budget, best.grid, best.staged, best.threads, best.smem);
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

int mpkg_batch_info(const mpkg_plan *p, mpkg_batch_info_t *info) {
  if (!p || !info || p->exec != MPKG_EXEC_BATCH) return fail(kEInval, "not a batch plan");
  std::memset(info, 0, sizeof *info);
  info->nmat = p->batch_nmat;
  info->rows = p->batch.N;
  info->nnz = p->nnz;
  info->nrhs = p->batch.nrhs;
  info->nlevel = p->nlevel;
  info->lanes_per_row = p->batch_lpr;
  info->vector_width = p->batch_vw;
  info->group_bytes = p->batch_group_bytes;
  info->ngroup = p->batch.ngroup;
  info->grid = p->batch.nblk;
  info->graph = p->graph_ok ? 1 : 0;
  info->candidates = p->batch_candidates;
  info->tune_ms = p->batch_tune_ms;
  info->device_bytes = p->device_bytes;
  info->staged = p->batch_staged ? 1 : 0;
  info->threads = p->batch_threads;
  info->window_bytes = (long)p->batch_smem;
  return kOk;
}

int mpkg_exec_batch_device(mpkg_plan *p, float *d_vb, void *stream) {
  clear_error();
  if (!p || !d_vb || p->exec != MPKG_EXEC_BATCH) return fail(kEInval, "bad plan or buffer");
  if (((uintptr_t)d_vb) % 16) return fail(kEInval, "the basis buffer must be 16-byte aligned");
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  p->launches = 1;
  const int rc = batch_launch(p, d_vb, st);
  if (rc) return rc;
  CUDA_TRY(cudaGetLastError());
  return kOk;
}

int mpkg_exec_batch_host(mpkg_plan *p, float *vb) {
  clear_error();
  if (!p || !vb || p->exec != MPKG_EXEC_BATCH) return fail(kEInval, "bad plan or buffer");
  const size_t lv = (size_t)p->batch.N * p->batch.nrhs, total = lv * (p->nlevel + 1);
  if (!p->d_fb) CUDA_TRY(cudaMalloc(&p->d_fb, sizeof(float) * total));
  float *d = p->d_fb;
  cudaStream_t st = p->stream;
  CUDA_TRY(cudaMemcpyAsync(d, vb, sizeof(float) * lv, cudaMemcpyHostToDevice, st));
  int rc = mpkg_exec_batch_device(p, d, st);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(vb + lv, d + lv, sizeof(float) * (total - lv), cudaMemcpyDeviceToHost, st));
  return mpkg_sync(p, st);
}

int mpkg_plan_pdmpk(int npart, const char *const *buf_paths, const char *const *results_paths, int arith,
                    mpkg_plan **out) {
  clear_error();
  if (!out || !buf_paths || !results_paths || npart <= 0) return fail(kEInval, "bad argument");
  *out = nullptr;
  if (arith != MPKG_ARITH_FMA && arith != MPKG_ARITH_SEPARATE)
    return fail(kEInval, "pdmpk buffers run in FP64 (fma or separate)");
  std::vector<pdmpk_gb300::Buffers> bufs(npart, pdmpk_gb300::Buffers(npart));
  int rc;
  for (int r = 0; r < npart; r++) {
    if (!buf_paths[r] || !results_paths[r]) return fail(kEInval, "null path");
    if ((rc = bufs[r].Load(buf_paths[r], results_paths[r]))) return rc;
  }
  PdExecMaps m;
  if ((rc = pd_exec_maps(bufs, &m))) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  p->exec = MPKG_EXEC_PDMPK;
  p->n = m.n; p->nlevel = m.nlevel; p->nphase = m.nbatch; p->npart = npart;
  p->arith = arith; p->valued = true;
  p->full_coverage = true;
  p->rows_computed = (long)m.row_dst.size();
  p->nnz = (long)m.gcol.size();
  rc = cudaGetDevice(&p->device) == cudaSuccess ? kOk : fail(kECuda, "cudaGetDevice failed");
  if (!rc && cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(kECuda, "stream creation failed");
  if (!rc) rc = dev_alloc(p, &p->b_vall, std::max<long>(m.mbuf_total, 1));
  if (!rc) rc = dev_copy(p, &p->b_in_dst, m.in_dst.data(), m.in_dst.size());
  if (!rc) rc = dev_copy(p, &p->b_in_src, m.in_src.data(), m.in_src.size());
  if (!rc) rc = dev_copy(p, &p->b_out_src, m.out_src.data(), m.out_src.size());
  if (!rc) rc = dev_copy(p, &p->b_out_dst, m.out_dst.data(), m.out_dst.size());
  if (!rc) rc = dev_copy(p, &p->b_cm_dst, m.cm_dst.data(), m.cm_dst.size());
  if (!rc) rc = dev_copy(p, &p->b_cm_src, m.cm_src.data(), m.cm_src.size());
  if (!rc) rc = dev_copy(p, &p->b_row_dst, m.row_dst.data(), m.row_dst.size());
  if (!rc) rc = dev_copy(p, &p->d_row_init, m.row_init.data(), m.row_init.size());
  if (!rc) rc = dev_copy(p, &p->b_row_ptr, m.row_ptr.data(), m.row_ptr.size());
  if (!rc) rc = dev_copy(p, &p->b_gcol, m.gcol.data(), m.gcol.size());
  if (!rc) rc = dev_copy(p, &p->b_gval, m.gval.data(), m.gval.size());
  if (!rc) rc = dev_alloc(p, &p->d_err, 1);
  if (!rc && cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess) rc = fail(kECuda, "memset failed");
  p->b_nin = (long)m.in_dst.size();
  p->b_nout = (long)m.out_src.size();
  p->b_cm_off = m.cm_off;
  p->pd_row_off = m.row_off;
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

int mpkg_pdmpk_prep(int n, const int *ptr, const int *col, const double *val, int npart, int nlevel,
                    int mirror_method, int weight_update_method, int partitioner, const char *const *buf_paths,
                    const char *const *results_paths) {
  clear_error();
  if (!ptr || !col || !val || !buf_paths || !results_paths || npart <= 0) return fail(kEInval, "bad argument");
  int rc = check_csr(n, ptr, col);
  if (rc) return rc;
  pdmpk_gb300::Csr csr;
  csr.n = n;
  csr.nnz = ptr[n];
  csr.ptr.assign(ptr, ptr + n + 1);
  csr.col.assign(col, col + ptr[n]);
  csr.val.assign(val, val + ptr[n]);
  pdmpk_gb300::Args args;
  args.npart = npart;
  args.nlevel = nlevel;
  args.mirror_method = mirror_method;
  args.weight_update_method = weight_update_method;
  if (partitioner == MPKG_PD_PART_BLOCKSHIFT) args.partitioner = pdmpk_gb300::BlockShiftPartitioner();
  else if (partitioner == MPKG_PD_PART_BFS) args.partitioner = pdmpk_gb300::BfsPartitioner();
  else if (partitioner == MPKG_PD_PART_METIS) args.partitioner = pdmpk_gb300::MetisPartitioner();
  else return fail(kEInval, "unknown partitioner");
  std::vector<pdmpk_gb300::Buffers> bufs;
  if ((rc = pdmpk_gb300::CommCompPatterns(csr, args, &bufs))) return rc;
  for (int r = 0; r < npart; r++) {
    if (!buf_paths[r] || !results_paths[r]) return fail(kEInval, "null path");
    if ((rc = bufs[r].Dump(buf_paths[r], results_paths[r]))) return rc;
  }
  return kOk;
}

}  // extern "C"

namespace {

template <bool STREAM>
const void *mix_wave_kernel_for(int value_type, bool rel, bool uni) {
  if (value_type == MPKG_VALUE_F32) {
    if (rel && uni) return (const void *)wave_mix_kernel<float, true, true, STREAM>;
    return rel ? (const void *)wave_mix_kernel<float, true, false, STREAM>
               : (const void *)wave_mix_kernel<float, false, false, STREAM>;
  }
  if (rel && uni) return (const void *)wave_mix_kernel<__nv_bfloat16, true, true, STREAM>;
  return rel ? (const void *)wave_mix_kernel<__nv_bfloat16, true, false, STREAM>
             : (const void *)wave_mix_kernel<__nv_bfloat16, false, false, STREAM>;
}

const void *mix_wave_kernel_ptr(int value_type, bool rel, bool uni, bool stream) {
  return stream ? mix_wave_kernel_for<true>(value_type, rel, uni) : mix_wave_kernel_for<false>(value_type, rel, uni);
}

int mixed_wave_setup(mpkg_plan *p, int n, const int *ptr, const int *col, const double *val, int nlevel,
                     int value_type) {
  mpkg_plan *w = nullptr;
  int rc = plan_wave_impl(n, ptr, col, val, nlevel, MPKG_ARITH_FMA, value_type, &w);
  if (rc) return rc;
  p->inner = w;
  int per_sm = 0, nsm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mix_wave_kernel_ptr(value_type, w->wave_rel, w->wave_uni, false), 256, 0));
  int per_sm_s = 0;  // the streaming build must cover the grid too
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_s, mix_wave_kernel_ptr(value_type, w->wave_rel, w->wave_uni, true), 256, 0));
  per_sm = std::min(per_sm, per_sm_s);
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
  if ((long)per_sm * nsm < w->wave_grid) return fail(kERange, "mixed wavefront kernel cannot cover the grid");
  const int nslice = (n + 31) / 32;
  std::vector<long> soff(nslice + 1, 0);
  for (int sl = 0; sl < nslice; sl++) {
    int wd = 0;
    for (int i = sl * 32; i < std::min(n, sl * 32 + 32); i++) wd = std::max(wd, ptr[i + 1] - ptr[i]);
    soff[sl + 1] = soff[sl] + 32L * wd;
  }
  auto fill = [&](auto conv, auto *vec) {
    vec->assign(soff[nslice], conv(0.0));
    for (int i = 0; i < n; i++) {
      const long e0 = soff[i / 32] + (i % 32);
      for (int t = 0; t < ptr[i + 1] - ptr[i]; t++) (*vec)[e0 + 32L * t] = conv(val[ptr[i] + t]);
    }
  };
  {  // values larger than L2: every level streams them from HBM anyway
    int l2 = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, p->device));
    const double vbytes = (double)soff[nslice] * (value_type == MPKG_VALUE_F32 ? 4.0 : 2.0);
    w->wave.stream_vals = vbytes > (double)l2 ? 1 : 0;
  }
  if (value_type == MPKG_VALUE_F32) {
    std::vector<float> sv;
    fill([](double v) { return (float)v; }, &sv);
    float *d = nullptr;
    if ((rc = dev_copy(p, &d, sv.data(), sv.size()))) return rc;
    p->mix_sval = d;
  } else {
    std::vector<__nv_bfloat16> sv;
    fill([](double v) { return __double2bfloat16(v); }, &sv);
    __nv_bfloat16 *d = nullptr;
    if ((rc = dev_copy(p, &d, sv.data(), sv.size()))) return rc;
    p->mix_sval = d;
  }
  return kOk;
}

}  // namespace

extern "C" {

int mpkg_plan_mixed(int n, const int *ptr, const int *col, const double *val, int nlevel, int value_type,
                    mpkg_plan **out) {
  clear_error();
  if (!out) return fail(kEInval, "out is null");
  *out = nullptr;
  if (!val) return fail(kEInval, "the mixed-precision form needs matrix values");
  if (value_type != MPKG_VALUE_F32 && value_type != MPKG_VALUE_BF16) return fail(kEInval, "unknown value type");
  int rc = check_csr(n, ptr, col);
  if (rc) return rc;
  if (nlevel <= 0 || nlevel > 31) return fail(kEInval, "nlevel must be in [1, 31]");
  Csr g;
  g.n = n;
  g.ptr.assign(ptr, ptr + n + 1);
  g.col.assign(col, col + ptr[n]);
  PipePlan pp;
  if ((rc = build_pipe_plan(g, nlevel, kPipeChunk, &pp))) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  p->exec = MPKG_EXEC_MIXED;
  p->n = n; p->nlevel = nlevel; p->npart = pp.nchunk; p->valued = true; p->arith = -1;
  p->nnz = ptr[n];
  p->rows_computed = (long)n * nlevel;
  p->mix_vt = value_type;
  rc = cudaGetDevice(&p->device) == cudaSuccess ? kOk : fail(kECuda, "cudaGetDevice failed");
  if (!rc && cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(kECuda, "stream creation failed");
  // infinity norm -> power-of-two scale
  double anorm = 0.0;
  for (int i = 0; i < n; i++) {
    double r = 0.0;
    for (int j = ptr[i]; j < ptr[i + 1]; j++) r += std::fabs(val[j]);
    anorm = std::max(anorm, r);
  }
  int e = 0;
  if (anorm > 0) e = (int)std::ceil(std::log2(anorm));
  p->mix_e = e;
  MixArgs &m = p->mix;
  m.n = n; m.nlevel = nlevel; m.chunk = kPipeChunk; m.nchunk = pp.nchunk;
  m.scale = std::ldexp(1.0f, -e);
  int maxnnz = 0;
  for (int c = 0; c < pp.nchunk; c++) {
    const int r1 = std::min(n, (c + 1) * kPipeChunk);
    maxnnz = std::max(maxnnz, ptr[r1] - ptr[c * kPipeChunk]);
  }
  m.max_chunk_nnz = std::max(maxnnz, 1);
  const size_t vsize = value_type == MPKG_VALUE_F32 ? 4 : 2;
  p->pipe_smem_bytes = pipe_smem_size(kPipeChunk, m.max_chunk_nnz, true, vsize);
  if (!rc) rc = dev_copy(p, &p->d_ptr, ptr, (size_t)n + 1);
  if (!rc) rc = dev_copy(p, &p->d_col, col, (size_t)p->nnz);
  if (!rc) {
    if (value_type == MPKG_VALUE_F32) {
      std::vector<float> v(p->nnz);
      for (long j = 0; j < p->nnz; j++) {
        v[j] = (float)val[j];
        if ((double)v[j] != val[j]) p->mix_inexact++;
      }
      float *dv;
      rc = dev_copy(p, &dv, v.data(), v.size());
      m.val = dv;
    } else {
      std::vector<__nv_bfloat16> v(p->nnz);
      for (long j = 0; j < p->nnz; j++) {
        v[j] = __double2bfloat16(val[j]);
        if ((double)__bfloat162float(v[j]) != val[j]) p->mix_inexact++;
      }
      __nv_bfloat16 *dv;
      rc = dev_copy(p, &dv, v.data(), v.size());
      m.val = dv;
    }
  }
  std::vector<int> glo(pp.nchunk), ghi(pp.nchunk);
  for (int c = 0; c < pp.nchunk; c++) { glo[c] = pp.dep_lo[c]; ghi[c] = pp.dep_hi[c]; }
  int *dlo = nullptr, *dhi = nullptr;
  unsigned *ticket = nullptr, *counts = nullptr;
  if (!rc) rc = dev_copy(p, &dlo, glo.data(), glo.size());
  if (!rc) rc = dev_copy(p, &dhi, ghi.data(), ghi.size());
  if (!rc) rc = dev_alloc(p, &ticket, 1);
  if (!rc) rc = dev_alloc(p, &counts, (size_t)(nlevel + 1) * pp.nchunk);
  if (!rc) rc = dev_alloc(p, &p->d_err, 1);
  if (!rc) {
    cudaMemset(counts, 0, sizeof(unsigned) * (size_t)(nlevel + 1) * pp.nchunk);
    cudaMemset(p->d_err, 0, sizeof(int));
    m.gdep_lo = dlo; m.gdep_hi = dhi; m.ptr = p->d_ptr; m.col = p->d_col; m.ticket = ticket; m.counts = counts;
    m.err = p->d_err;
    m.bulk_ok = true;
    p->pipe.counts = counts;  // reset path on errors
    p->pipe.ngroups = pp.nchunk;
    int maxsm = 0, per_sm = 0, nsm = 0;
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device);
    if (p->pipe_smem_bytes > (size_t)maxsm) rc = fail(kERange, "chunk rows too dense for shared memory");
    if (!rc) {
      cudaError_t e1 = value_type == MPKG_VALUE_F32
                           ? cudaFuncSetAttribute(mix_pipe_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)p->pipe_smem_bytes)
                           : cudaFuncSetAttribute(mix_pipe_kernel<__nv_bfloat16>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->pipe_smem_bytes);
      cudaError_t e2 = value_type == MPKG_VALUE_F32
                           ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mix_pipe_kernel<float>, kPipeThreads,
                                                                           p->pipe_smem_bytes)
                           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mix_pipe_kernel<__nv_bfloat16>,
                                                                           kPipeThreads, p->pipe_smem_bytes);
      if (e1 != cudaSuccess || e2 != cudaSuccess) rc = fail(kECuda, "kernel attribute set-up failed");
    }
    if (!rc) {
      const long grid = std::min<long>((long)per_sm * nsm, pp.nchunk);
      p->pipe_grid = (int)grid;
      p->pipe_reach = pp.reach;
      if (grid < pp.nchunk && grid < (long)(nlevel - 1) * pp.reach + 1)
        rc = fail(kERange, "matrix bandwidth too large for the mixed pipeline");
    }
  }
  // the wavefront schedule (preferred): its layout from an FP64 wave plan,
  // plus the values in the sliced order and the storage type
  if (!rc && mixed_wave_setup(p, n, ptr, col, val, nlevel, value_type) != kOk) {
    if (p->inner) { mpkg_plan_destroy(p->inner); p->inner = nullptr; }
    clear_error();  // keep the chunk pipeline
  }
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

namespace {
inline uint32_t rotl32(uint32_t m, int r) { return r ? (m << r) | (m >> (32 - r)) : m; }

// Bank rotation of every 32-slot group of one tile: for each warp-wide
// gather (a slice's entry t at level 1, weighted by the levels the slice
// computes) the slots it reads are grouped by 32-slot group as bit masks
// of their offsets; group q's rotation r maps offset o to bank (o + r) & 31.
// One pass over the groups picks for each the rotation that least overlaps
// the banks the other groups of the same gathers occupy (coordinate
// descent from no rotation; ties keep the current one).
void tile_rotations(const TilePlan &tp, int pt, int k, int nrow1, int nslice, int ns, std::vector<int> *rot_out) {
  const int nq = (ns + 31) / 32;
  struct Ent { int wf, q; uint32_t m; int w; };
  std::vector<Ent> ent;
  std::vector<int> wf_first;  // entries of gather i: [wf_first[i], wf_first[i+1])
  const int *sh = &tp.shell[(long)pt * (k + 1)];
  std::vector<uint32_t> qm(nq, 0u);
  std::vector<int> touched;
  for (int sl = 0; sl < nslice; sl++) {
    int w = 0;
    for (int l = 1; l <= k; l++) w += sl * 32 < sh[k - l];
    const long gs = tp.slice_off[pt] + sl;
    const int width = tp.ell_width[gs];
    for (int t = 0; t < width; t++) {
      wf_first.push_back((int)ent.size());
      touched.clear();
      for (int lane = 0; lane < 32 && sl * 32 + lane < nrow1; lane++) {
        const int c = tp.ell_col[tp.ell_off[gs] + (long)t * 32 + lane];
        if (c == 0xFFFF || c >= ns) continue;
        if (!qm[c >> 5]) touched.push_back(c >> 5);
        qm[c >> 5] |= 1u << (c & 31);
      }
      if (touched.size() > 1)  // a gather within one group never conflicts
        for (int q : touched) ent.push_back({(int)wf_first.size() - 1, q, qm[q], w});
      for (int q : touched) qm[q] = 0u;
    }
  }
  wf_first.push_back((int)ent.size());
  std::vector<std::vector<int>> byq(nq);
  for (int e = 0; e < (int)ent.size(); e++) byq[ent[e].q].push_back(e);
  std::vector<int> &rot = *rot_out;
  rot.assign(nq, 0);
  long cost[32];
  for (int q = 0; q < nq; q++) {
    if (byq[q].empty()) continue;
    std::fill(cost, cost + 32, 0L);
    for (int e : byq[q]) {
      const Ent &en = ent[e];
      uint32_t o = 0;
      for (int e2 = wf_first[en.wf]; e2 < wf_first[en.wf + 1]; e2++)
        if (e2 != e) o |= rotl32(ent[e2].m, rot[ent[e2].q]);
      for (int r = 0; r < 32; r++) cost[r] += (long)en.w * __builtin_popcount(rotl32(en.m, r) & o);
    }
    int best = rot[q];
    for (int r = 0; r < 32; r++)
      if (cost[r] < cost[best]) best = r;
    rot[q] = best;
  }
}

// The register-resident tile kernel's two images per tile (layout above
// tiles_reg_kernel), in execution order, built by all host threads.  Plans
// whose tiles do not fit (rows wider than 12 entries, more than
// kTrThreads * kTrRows computed rows, positions beyond 16-bit byte
// offsets, nlevel > 26, images beyond shared memory) keep tiles_mix_kernel;
// nothing is built for them.
int reg_tiles_setup(mpkg_plan *p, const TilePlan &tp, const int *ptr, const void *hval, int wmax) {
  const int k = p->nlevel, W = tr_width(wmax);
  const int npart = p->npart;
  const size_t vsz = p->mix_vt == MPKG_VALUE_F32 ? sizeof(float) : sizeof(__nv_bfloat16);
  const int zp = (tp.max_slots + 31) / 32 * 32;  // the zero position, past every tile's positions
  if (W == 0 || k > kTrHdrInts - 6 || 4 * (zp + 1) > kTrXBytes) return kOk;
  std::vector<long> voff(npart + 1, 0), moff(npart + 1, 0);
  std::vector<int> vbytes(npart), mbytes(npart);
  for (int q = 0; q < npart; q++) {
    const int pt = tp.order[q];
    const int ns = (int)(tp.slot_off[pt + 1] - tp.slot_off[pt]);
    const int nrow1 = tp.shell[(long)pt * (k + 1) + k - 1];
    if (nrow1 > kTrThreads * kTrRows) return kOk;
    const int nslice = (nrow1 + 31) / 32;
    if (tp.slice_off[pt + 1] - tp.slice_off[pt] != nslice) return fail(kEStruct, "tile slices disagree with shells");
    const int nq = (ns + 31) / 32;
    vbytes[q] = 4 * (kTrHdrInts + (nq + 3) / 4 * 4 + nq * 32);
    mbytes[q] = std::max<int>(16, (int)((size_t)nslice * 32 * (4 * ((W + 1) / 2) + W * vsz)));
    voff[q + 1] = voff[q] + vbytes[q];
    moff[q + 1] = moff[q] + mbytes[q];
  }
  const int max_v = *std::max_element(vbytes.begin(), vbytes.end());
  const int max_m = *std::max_element(mbytes.begin(), mbytes.end());
  const int buf_floats = kTrXBytes / 4;
  const size_t smem = 3 * (size_t)kTrXBytes + max_m + max_v;
  int maxsm = 0, nsm = 0, per_sm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device);
  if (smem > (size_t)maxsm) return kOk;
  std::vector<unsigned char> vimg(voff[npart]), mimg(moff[npart]);
  std::atomic<int> bad{0};
  auto build = [&](int q) {
    const int pt = tp.order[q];
    const long s0 = tp.slot_off[pt];
    const int ns = (int)(tp.slot_off[pt + 1] - s0);
    const int *sh = &tp.shell[(long)pt * (k + 1)];
    const int nrow1 = sh[k - 1], nslice = (nrow1 + 31) / 32, nq = (ns + 31) / 32, nqp = (nq + 3) / 4 * 4;
    std::vector<int> rot;
    tile_rotations(tp, pt, k, nrow1, nslice, ns, &rot);
    auto pos = [&](int c) { return (c & ~31) | ((c + rot[c >> 5]) & 31); };
    int *hv = reinterpret_cast<int *>(vimg.data() + voff[q]);
    hv[0] = nq * 32; hv[1] = nrow1; hv[2] = sh[0]; hv[3] = nslice;
    for (int d = 0; d <= k; d++) hv[4 + d] = sh[d];
    hv[31] = nqp;
    for (int g = 0; g < nq; g++) hv[kTrHdrInts + g] = rot[g];
    int *pv = hv + kTrHdrInts + nqp;
    for (int g = 0; g < nq * 32; g++) pv[g] = -1;
    for (int sl = 0; sl < ns; sl++) pv[pos(sl)] = tp.slot_vert[s0 + sl];
    uint16_t *mc = reinterpret_cast<uint16_t *>(mimg.data() + moff[q]);  // [slice][t / 2][lane][t & 1]
    unsigned char *mv = mimg.data() + moff[q] + (size_t)nslice * ((W + 1) / 2) * 128;
    for (int sl = 0; sl < nslice; sl++) {
      const long gs = tp.slice_off[pt] + sl;
      const int w = tp.ell_width[gs];
      for (int t = 0; t < W; t++)
        for (int lane = 0; lane < 32; lane++) {
          const int r = sl * 32 + lane;
          const size_t e = ((size_t)sl * W + t) * 32 + lane;
          const int c = (r < nrow1 && t < w) ? tp.ell_col[tp.ell_off[gs] + (long)t * 32 + lane] : 0xFFFF;
          if (c != 0xFFFF && c >= ns) { bad = 1; return; }
          mc[(((size_t)sl * ((W + 1) / 2) + t / 2) * 32 + lane) * 2 + (t & 1)] =
              (uint16_t)(4 * (c != 0xFFFF ? pos(c) : zp));
          const long j = c != 0xFFFF ? (long)ptr[tp.slot_vert[s0 + r]] + t : -1;
          if (vsz == sizeof(float)) {
            const float x = j >= 0 ? static_cast<const float *>(hval)[j] : -0.0f;
            std::memcpy(mv + e * 4, &x, 4);
          } else {
            uint16_t b = 0x8000;  // BF16 -0
            if (j >= 0) std::memcpy(&b, static_cast<const __nv_bfloat16 *>(hval) + j, 2);
            std::memcpy(mv + e * 2, &b, 2);
          }
        }
    }
  };
  const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::atomic<int> next{0};
  auto work = [&] {
    for (int q; (q = next.fetch_add(1)) < npart && !bad;) build(q);
  };
  std::vector<std::thread> pool;
  try {
    for (int t = 1; t < nth; t++) pool.emplace_back(work);
  } catch (const std::exception &) {  // no more threads: the caller's thread does the rest
  }
  work();
  for (auto &th : pool) th.join();
  if (bad) return fail(kEStruct, "tile column outside the halo");
  unsigned char *dvimg = nullptr, *dmimg = nullptr;
  long *dvoff = nullptr, *dmoff = nullptr;
  int *dvb = nullptr, *dmb = nullptr;
  int rc = dev_copy(p, &dvimg, vimg.data(), vimg.size());
  if (!rc) rc = dev_copy(p, &dmimg, mimg.data(), mimg.size());
  if (!rc) rc = dev_copy(p, &dvoff, voff.data(), (size_t)npart);
  if (!rc) rc = dev_copy(p, &dmoff, moff.data(), (size_t)npart);
  if (!rc) rc = dev_copy(p, &dvb, vbytes.data(), vbytes.size());
  if (!rc) rc = dev_copy(p, &dmb, mbytes.data(), mbytes.size());
  if (rc) return rc;
  const void *fn = reinterpret_cast<const void *>(tr_kernel_ptr(p->mix_vt, W));
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTrThreads, smem) != cudaSuccess)
    return fail(kECuda, "register tile kernel attribute set-up failed");
  if (per_sm < 1) return kOk;
  TileRegArgs &a = p->tr;
  a.n = p->n; a.nlevel = k; a.ntile = npart; a.zs = zp;
  a.vimg = dvimg; a.mimg = dmimg; a.voff = dvoff; a.moff = dmoff; a.vbytes = dvb; a.mbytes = dmb;
  a.max_vbytes = max_v; a.max_mbytes = max_m; a.buf_floats = buf_floats;
  a.scale = p->mix.scale;
  a.err = p->d_err;
  p->tr_w = W;
  p->tr_smem = smem;
  p->tr_grid = (int)std::min<long>((long)per_sm * nsm, npart);
  p->pipe_grid = p->tr_grid;
  p->tr_on = true;
  return kOk;
}
}  // namespace

int mpkg_plan_mixed_tiles(int n, const int *ptr, const int *col, const double *val, const int *part, int npart,
                          int nlevel, int value_type, mpkg_plan **out) {
  clear_error();
  if (!out) return fail(kEInval, "out is null");
  *out = nullptr;
  if (!val) return fail(kEInval, "the mixed-precision form needs matrix values");
  if (value_type != MPKG_VALUE_F32 && value_type != MPKG_VALUE_BF16) return fail(kEInval, "unknown value type");
  if (!part || npart <= 0) return fail(kEInval, "bad partition");
  int rc = check_csr(n, ptr, col);
  if (rc) return rc;
  if (nlevel <= 0 || nlevel > 31) return fail(kEInval, "nlevel must be in [1, 31]");
  std::vector<int> pv(part, part + n);
  for (int q : pv) if (q < 0 || q >= npart) return fail(kERange, "part id out of range");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  Csr g;
  g.n = n;
  g.ptr.assign(ptr, ptr + n + 1);
  g.col.assign(col, col + ptr[n]);
  TilePlan tp;
  bool on_gpu = false;
  if ((rc = build_tile_plan_gpu(g, pv, npart, nlevel, &tp, &on_gpu))) return rc;
  mpkg_plan *p = new_plan();
  if (!p) return fail(kENoMem, "plan allocation failed");
  p->exec = MPKG_EXEC_MIXED;
  p->n = n; p->nlevel = nlevel; p->npart = npart; p->valued = true; p->arith = -1;
  p->nnz = ptr[n];
  p->rows_computed = tp.total_rows;
  p->max_tile_slots = tp.max_slots;
  p->mix_vt = value_type;
  rc = cudaGetDevice(&p->device) == cudaSuccess ? kOk : fail(kECuda, "cudaGetDevice failed");
  if (!rc && cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(kECuda, "stream creation failed");
  double anorm = 0.0;  // infinity norm -> power-of-two scale, as mpkg_plan_mixed
  for (int i = 0; i < n; i++) {
    double r = 0.0;
    for (int j = ptr[i]; j < ptr[i + 1]; j++) r += std::fabs(val[j]);
    anorm = std::max(anorm, r);
  }
  p->mix_e = anorm > 0 ? (int)std::ceil(std::log2(anorm)) : 0;
  p->mix.scale = std::ldexp(1.0f, -p->mix_e);
  TileMixArgs &a = p->tm;
  a.n = n; a.nlevel = nlevel; a.npart = npart; a.max_slots = tp.max_slots; a.scale = p->mix.scale;
  int *order = nullptr, *shell = nullptr, *slot_vert = nullptr, *slot_coef = nullptr;
  long *slot_off = nullptr, *slice_off = nullptr, *ell_off = nullptr;
  uint16_t *ell_col = nullptr;
  uint8_t *ell_width = nullptr;
  if (!rc) rc = dev_copy(p, &order, tp.order.data(), tp.order.size());
  if (!rc) rc = dev_copy(p, &slot_off, tp.slot_off.data(), tp.slot_off.size());
  if (!rc) rc = dev_copy(p, &shell, tp.shell.data(), tp.shell.size());
  if (!rc) rc = dev_copy(p, &slot_vert, tp.slot_vert.data(), tp.slot_vert.size());
  if (!rc) {
    std::vector<int> sc(tp.slot_vert.size());
    for (size_t q = 0; q < sc.size(); q++) sc[q] = ptr[tp.slot_vert[q]];
    rc = dev_copy(p, &slot_coef, sc.data(), sc.size());
  }
  if (!rc) rc = dev_copy(p, &slice_off, tp.slice_off.data(), tp.slice_off.size());
  if (!rc) rc = dev_copy(p, &ell_off, tp.ell_off.data(), tp.ell_off.size());
  if (!rc) {
    std::vector<uint16_t> ec = tp.ell_col;
    if (ec.empty()) ec.push_back(0xFFFF);
    rc = dev_copy(p, &ell_col, ec.data(), ec.size());
  }
  int wmax = 0;
  if (!rc) {
    std::vector<uint8_t> ew = tp.ell_width;
    for (uint8_t w : ew) wmax = std::max(wmax, (int)w);
    if (ew.empty()) ew.push_back(0);
    rc = dev_copy(p, &ell_width, ew.data(), ew.size());
  }
  std::vector<float> v32;
  std::vector<__nv_bfloat16> v16;
  if (!rc) {
    if (value_type == MPKG_VALUE_F32) {
      v32.resize(p->nnz);
      for (long j = 0; j < p->nnz; j++) {
        v32[j] = (float)val[j];
        if ((double)v32[j] != val[j]) p->mix_inexact++;
      }
      float *dv = nullptr;
      rc = dev_copy(p, &dv, v32.data(), v32.size());
      a.val = dv;
    } else {
      v16.resize(p->nnz);
      for (long j = 0; j < p->nnz; j++) {
        v16[j] = __double2bfloat16(val[j]);
        if ((double)__bfloat162float(v16[j]) != val[j]) p->mix_inexact++;
      }
      __nv_bfloat16 *dv = nullptr;
      rc = dev_copy(p, &dv, v16.data(), v16.size());
      a.val = dv;
    }
  }
  unsigned int *ticket = nullptr;
  if (!rc) rc = dev_alloc(p, &ticket, 1);
  if (!rc) rc = dev_alloc(p, &p->d_err, 1);
  if (!rc) {
    cudaMemset(p->d_err, 0, sizeof(int));
    a.order = order; a.slot_off = slot_off; a.shell = shell; a.slot_vert = slot_vert; a.slot_coef = slot_coef;
    a.slice_off = slice_off; a.ell_off = ell_off; a.ell_col = ell_col; a.ell_width = ell_width;
    a.ticket = ticket; a.err = p->d_err;
    p->tm_w = wmax <= 8 ? 8 : wmax <= 12 ? 12 : 16;  // wider slices read their rows from L2 at each level
    p->tm_smem = 2 * (size_t)std::max(tp.max_slots, 1) * sizeof(float);
    int maxsm = 0, per_sm = 0, nsm = 0;
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device);
    if (p->tm_smem > (size_t)maxsm) rc = fail(kERange, "a tile's two level vectors exceed shared memory");
    const void *fn = reinterpret_cast<const void *>(tm_kernel_ptr(value_type, p->tm_w));
    if (!rc && (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->tm_smem) !=
                    cudaSuccess ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTmThreads, p->tm_smem) != cudaSuccess))
      rc = fail(kECuda, "tile kernel attribute set-up failed");
    if (!rc && per_sm < 1) rc = fail(kERange, "the tile kernel does not fit an SM");
    p->tm_grid = (int)std::min<long>((long)per_sm * nsm, npart);
    p->pipe_grid = p->tm_grid;
    p->tiles_smem = true;
    p->tm_on = true;
  }
  if (!rc) rc = reg_tiles_setup(p, tp, ptr, value_type == MPKG_VALUE_F32 ? (const void *)v32.data()
                                                                          : (const void *)v16.data(), wmax);
  if (rc) { mpkg_plan_destroy(p); return rc; }
  *out = p;
  return kOk;
}

int mpkg_plan_mixed_tiles_tuned(int n, const int *ptr, const int *col, const double *val, const int *coords, int dim,
                                int nlevel, int value_type, mpkg_plan **out) {
  clear_error();
  if (!out) return fail(kEInval, "out is null");
  *out = nullptr;
  if (n <= 0 || !coords || dim <= 0) return fail(kEInval, "bad coordinates");
  const std::vector<int> cvec(coords, coords + (long)n * dim);
  float *scratch = nullptr;
  if (cudaMalloc(&scratch, sizeof(float) * (size_t)n * (nlevel + 1)) != cudaSuccess)
    return fail(kENoMem, "autotune scratch");
  cudaMemset(scratch, 0, sizeof(float) * (size_t)n * (nlevel + 1));  // timing only: the values do not matter
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  mpkg_plan *best = nullptr;
  float best_ms = 0.f;
  int tried = 0, last_rc = kOk;
  std::string last_msg;
  const auto t_start = std::chrono::steady_clock::now();
  for (int rows : {384, 512, 768, 1024, 1536}) {  // part sizes, rows per part
    const int npart = std::max(1, (n + rows - 1) / rows);
    std::vector<int> part;
    if (partition_rcb(n, cvec, dim, npart, &part) != kOk) continue;
    mpkg_plan *p = nullptr;
    int rc = mpkg_plan_mixed_tiles(n, ptr, col, val, part.data(), npart, nlevel, value_type, &p);
    if (rc) {  // e.g. the tiles' level vectors exceed shared memory: the next size
      last_rc = rc;
      last_msg = mpkg_last_error();
      continue;
    }
    tried++;
    float ms = 0.f;
    for (int w = 0; w < 2 && !rc; w++) rc = mpkg_exec_mixed_device(p, scratch, p->stream);
    if (!rc && cudaEventRecord(e0, p->stream) != cudaSuccess) rc = fail(kECuda, "event record");
    for (int w = 0; w < 3 && !rc; w++) rc = mpkg_exec_mixed_device(p, scratch, p->stream);
    if (!rc && cudaEventRecord(e1, p->stream) != cudaSuccess) rc = fail(kECuda, "event record");
    if (!rc) rc = mpkg_sync(p, p->stream);
    if (!rc && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = fail(kECuda, "event time");
    if (rc) {
      mpkg_plan_destroy(p);
      if (best) mpkg_plan_destroy(best);
      best = nullptr;
      break;
    }
    if (!best || ms < best_ms) {
      if (best) mpkg_plan_destroy(best);
      best = p;
      best_ms = ms;
    } else {
      mpkg_plan_destroy(p);
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(scratch);
  if (!best) {
    if (tried == 0 && last_rc) return fail(last_rc, last_msg.c_str());
    return last_rc ? fail(last_rc, last_msg.c_str()) : fail(kERange, "no part size gives a tile plan");
  }
  best->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  best->tune_candidates = tried;
  clear_error();
  *out = best;
  return kOk;
}

int mpkg_mixed_scale(const mpkg_plan *p, int *exponent, long *inexact_values) {
  if (!p || p->exec != MPKG_EXEC_MIXED) return fail(kEInval, "not a mixed-precision plan");
  if (exponent) *exponent = p->mix_e;
  if (inexact_values) *inexact_values = p->mix_inexact;
  return kOk;
}

int mpkg_exec_mixed_device(mpkg_plan *p, float *d_vv, void *stream) {
  clear_error();
  if (!p || p->exec != MPKG_EXEC_MIXED || !d_vv) return fail(kEInval, "not a mixed-precision plan, or null vv");
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  p->epoch++;
  if (p->epoch >= (1u << 30)) {
    CUDA_TRY(cudaMemsetAsync(p->mix.counts, 0, sizeof(unsigned) * (size_t)(p->nlevel + 1) * p->mix.nchunk, st));
    p->epoch = 1;
  }
  if (p->tr_on) {  // PA1 tiles, rows in registers
    TileRegArgs a = p->tr;
    a.x = d_vv;
    a.vf = d_vv;
    tr_kernel_ptr(p->mix_vt, p->tr_w)<<<p->tr_grid, kTrThreads, p->tr_smem, st>>>(a);
    CUDA_TRY(cudaGetLastError());
    p->launches = 1;
    return kOk;
  }
  if (p->tm_on) {  // PA1 tiles
    CUDA_TRY(cudaMemsetAsync(p->tm.ticket, 0, sizeof(unsigned int), st));
    TileMixArgs a = p->tm;
    a.x = d_vv;
    a.vf = d_vv;
    tm_kernel_ptr(p->mix_vt, p->tm_w)<<<p->tm_grid, kTmThreads, p->tm_smem, st>>>(a);
    CUDA_TRY(cudaGetLastError());
    p->launches = 1;
    return kOk;
  }
  if (p->inner) {  // wavefront schedule
    WaveArgs &w = p->inner->wave;
    const unsigned step = (unsigned)p->nlevel + 1;
    if (w.base == 0 || w.base > (1u << 30)) {
      CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(unsigned int) * (size_t)w.nblk, st));
      w.base = 1;
    } else {
      w.base += step;
    }
    WaveArgs a = w;
    a.err = p->d_err;
    float scale = p->mix.scale;
    if (p->mix_vt == MPKG_VALUE_F32) {
      const float *sv = static_cast<const float *>(p->mix_sval);
      void *args[] = {&a, (void *)&sv, (void *)&d_vv, &scale};
      CUDA_TRY(cudaLaunchCooperativeKernel(mix_wave_kernel_ptr(MPKG_VALUE_F32, p->inner->wave_rel, p->inner->wave_uni, w.stream_vals != 0), dim3(w.nblk),
                                           dim3(256), args, 0, st));
    } else {
      const __nv_bfloat16 *sv = static_cast<const __nv_bfloat16 *>(p->mix_sval);
      void *args[] = {&a, (void *)&sv, (void *)&d_vv, &scale};
      CUDA_TRY(cudaLaunchCooperativeKernel(mix_wave_kernel_ptr(MPKG_VALUE_BF16, p->inner->wave_rel, p->inner->wave_uni, w.stream_vals != 0), dim3(w.nblk),
                                           dim3(256), args, 0, st));
    }
    p->launches = 1;
    return kOk;
  }
  CUDA_TRY(cudaMemsetAsync(p->mix.ticket, 0, sizeof(unsigned), st));
  MixArgs m = p->mix;
  m.vv = d_vv;
  m.epoch = p->epoch;
  if (p->mix_vt == MPKG_VALUE_F32)
    mix_pipe_kernel<float><<<p->pipe_grid, kPipeThreads, p->pipe_smem_bytes, st>>>(m);
  else
    mix_pipe_kernel<__nv_bfloat16><<<p->pipe_grid, kPipeThreads, p->pipe_smem_bytes, st>>>(m);
  CUDA_TRY(cudaGetLastError());
  p->launches = 1;
  return kOk;
}

int mpkg_debug_pipe_stall(mpkg_plan *p, int extra_levels) {
  const bool mixed_wave = p && p->exec == MPKG_EXEC_MIXED && p->inner;
  if (!p || (p->exec != MPKG_EXEC_PIPE && p->exec != MPKG_EXEC_WAVE && p->exec != MPKG_EXEC_BATCH && !mixed_wave) ||
      extra_levels < 0 || extra_levels > 1000)
    return fail(kEInval,
                "stall hook needs a pipeline, wavefront, mixed-wavefront or batched plan and 0 <= extra <= 1000");
  p->pipe.stall = (uint32_t)extra_levels;
  p->wave.stall = (uint32_t)extra_levels;
  if (mixed_wave) p->inner->wave.stall = (uint32_t)extra_levels;
  if (p->exec == MPKG_EXEC_BATCH) {  // the replayed graph holds the launch's arguments: capture again
    p->batch.stall = (uint32_t)extra_levels;
    if (p->graph_exec) { cudaGraphExecDestroy(p->graph_exec); p->graph_exec = nullptr; }
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    p->graph_ok = false;
    p->graph_key = nullptr;
  }
  return kOk;
}

int mpkg_plan_info(const mpkg_plan *p, mpkg_plan_info_t *info) {
  if (!p || !info) return fail(kEInval, "null argument");
  std::memset(info, 0, sizeof *info);
  info->n = p->n; info->nlevel = p->nlevel; info->nphase = p->nphase; info->npart = p->npart;
  info->exec = p->exec; info->arith = p->arith; info->valued = p->valued;
  info->nnz = p->nnz;
  info->rows_computed = p->rows_computed;
  info->device_bytes = p->device_bytes;
  info->launches = p->exec == MPKG_EXEC_TASKS ? p->nphase + 1
                   : p->exec == MPKG_EXEC_SPMV
                       ? p->nlevel + (p->arith == MPKG_ARITH_DF64 ? 1 : p->arith == MPKG_ARITH_FIXED ? 2 : 0)
                   : p->exec == MPKG_EXEC_BUFS ? 2 + 2 * p->nphase + 1
                   : p->exec == MPKG_EXEC_PDMPK ? 2 + 2 * p->nphase : 1;
  if (p->exec == MPKG_EXEC_WAVE) info->pipe_grid = p->wave_grid;
  if (p->exec == MPKG_EXEC_MIXED && p->inner) {  // the wavefront schedule (pipe_chunk 0)
    info->pipe_chunk = 0;
    info->pipe_grid = p->inner->wave_grid;
  }
  info->tiles_in_smem = p->tiles_smem ? 1 : 0;
  info->max_tile_slots = p->max_tile_slots;
  info->pipe_chunk = p->pipe.chunk;
  info->pipe_reach = p->pipe_reach;
  info->pipe_grid = p->pipe_grid;
  info->tile_regs = p->tr_on ? 1 : 0;
  info->tune_candidates = p->tune_candidates;
  info->tune_ms = p->tune_ms;
  return kOk;
}

int mpkg_exec_device(mpkg_plan *p, double *d_vv, void *stream) {
  clear_error();
  if (!p || !d_vv) return fail(kEInval, "null plan or vv");
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  return plan_launch(p, d_vv, st);
}

int mpkg_sync(mpkg_plan *p, void *stream) {
  if (!p) return fail(kEInval, "null plan");
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  CUDA_TRY(cudaStreamSynchronize(st));
  int err = 0;
  CUDA_TRY(cudaMemcpy(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(p->d_err, 0, sizeof(int));
    if ((p->exec == MPKG_EXEC_PIPE || p->exec == MPKG_EXEC_MIXED) && p->pipe.counts) {  // counters are
      // inconsistent after an abort
      cudaMemset(p->pipe.counts, 0, sizeof(unsigned int) * (size_t)(p->nlevel + 1) * p->pipe.ngroups);
      p->epoch = 0;
    }
    if (p->exec == MPKG_EXEC_WAVE) p->wave.base = 0;  // flags restart from zero on the next call
    if (p->inner) p->inner->wave.base = 0;
    if (p->exec == MPKG_EXEC_BATCH) p->batch.base = 0;
    if (err == kErrTimeout) return fail(kETimeout, "a device-side wait exceeded its spin limit");
    return fail(kERange, "device-side bounds check failed");
  }
  return kOk;
}

int mpkg_exec_host(mpkg_plan *p, double *vv) {
  clear_error();
  if (!p || !vv) return fail(kEInval, "null plan or vv");
  const long total = (long)p->n * (p->nlevel + 1);
  // Page-locked vv on a wavefront plan whose levels travel in the device
  // ring (double-float, fixed point): the kernel reads x and writes every
  // level straight through the host mapping, so the host<->device traffic
  // overlaps the computation instead of following it.  The FP64 forms
  // read their levels back and keep the copies below.
  if (p->exec == MPKG_EXEC_WAVE && (p->arith == MPKG_ARITH_DF64 || p->arith == MPKG_ARITH_FIXED)) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, vv) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
      int rc = plan_launch(p, static_cast<double *>(at.devicePointer), p->stream);
      if (rc) return rc;
      return mpkg_sync(p, p->stream);
    }
    cudaGetLastError();  // pageable memory: the copies below
  }
  // Page-locked vv on an FP64 wavefront plan: the kernel reads x from the
  // host mapping and writes every level both to the device copy (which
  // the next level reads) and through the mapping, so the device->host
  // traffic overlaps the computation.
  if (p->exec == MPKG_EXEC_WAVE && (p->arith == MPKG_ARITH_FMA || p->arith == MPKG_ARITH_SEPARATE)) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, vv) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
      if (!p->d_vv) CUDA_TRY(cudaMalloc(&p->d_vv, sizeof(double) * total));
      int rc = launch_wave(p, p->d_vv, p->stream, static_cast<double *>(at.devicePointer));
      if (rc) return rc;
      p->launches = 1;
      return mpkg_sync(p, p->stream);
    }
    cudaGetLastError();  // pageable memory: the copies below
  }
  if (!p->d_vv) {
    CUDA_TRY(cudaMalloc(&p->d_vv, sizeof(double) * total));
  }
  cudaStream_t st = p->stream;
  const long up = p->full_coverage ? p->n : total;
  CUDA_TRY(cudaMemcpyAsync(p->d_vv, vv, sizeof(double) * up, cudaMemcpyHostToDevice, st));
  int rc = plan_launch(p, p->d_vv, st);
  if (rc) return rc;
  // pdmpk buffers produce only the last level; the others stay untouched
  const long first = p->exec == MPKG_EXEC_PDMPK ? (long)p->n * p->nlevel : (long)p->n;
  CUDA_TRY(cudaMemcpyAsync(vv + first, p->d_vv + first, sizeof(double) * (total - first),
                           cudaMemcpyDeviceToHost, st));
  return mpkg_sync(p, st);
}

}  // extern "C"

// Peak FP64 fused multiply-add rate of the current GPU: every thread runs 8
// independent FMA chains (a contraction toward b / (1 - a), bounded), so
// the FP64 pipe, not latency, sets the time.
__global__ void __launch_bounds__(256) fp64_rate_kernel(double *sink, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int u = 0; u < 8; u++) x[u] = 1e-3 * threadIdx.x + u;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int u = 0; u < 8; u++) x[u] = __fma_rn(x[u], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int u = 0; u < 8; u++) s += x[u];
  if (s == -1.0) sink[blockIdx.x] = s;  // never true; keeps the chains live
}

extern "C" {

int mpkg_fp64_fma_rate(double *fma_per_s) {
  clear_error();
  if (!fma_per_s) return fail(kEInval, "null argument");
  int dev = 0, nsm = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = nsm * 8, iters = 4096;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  float best = 0.f;
  for (int rep = 0; rep < 6; rep++) {
    CUDA_TRY(cudaEventRecord(e0, st));
    fp64_rate_kernel<<<grid, 256, 0, st>>>(nullptr, iters, 0.9999999, 1e-3);
    CUDA_TRY(cudaEventRecord(e1, st));
    CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  *fma_per_s = (double)grid * 256 * 8 * iters / (best * 1e-3);
  return kOk;
}

int mpkg_spmv_chain_device(int n, const int *d_ptr, const int *d_col, const double *d_val,
                           int nlevel, double *d_vv, int arith, void *stream) {
  clear_error();
  if (n <= 0 || !d_ptr || !d_col || !d_vv || nlevel <= 0) return fail(kEInval, "bad arguments");
  if (!d_val) return fail(kEInval, "the stand-alone chain needs values; use mpkg_plan_spmv for 1/deg");
  if (arith != MPKG_ARITH_FMA && arith != MPKG_ARITH_SEPARATE) return fail(kEInval, "bad arith");
  return launch_spmv(n, d_ptr, d_col, d_val, true, nlevel, d_vv, arith, (cudaStream_t)stream);
}

}  // extern "C"

// ==========================================================================
// Allocation-free pipeline entry point (mpkg_pipe_noalloc)
//
// For callers that must not allocate device memory themselves: a solver
// plug-in running inside an application whose memory pool owns the whole
// device, or a time-stepping loop that cannot afford cudaMalloc's implicit
// device synchronisation.  The caller passes the matrix and vv in device
// memory; the pipeline's bookkeeping (dependency ranges, completion
// counters, ticket, error word) lives in the file-scope array below, which
// every GPU that loads this library holds until the process exits.
// ==========================================================================
namespace {

constexpr int kNoAllocMaxChunks = 16384;  // n <= 16384 * 256 = 4096 * 1024 rows
constexpr int kNoAllocMaxLevels = 16;
// word layout: [0] ticket, [1] error, [2] max chunk nnz, [3] reach,
// [4] a column outside [0, n) was seen, [5] ptr decreases somewhere or
// ptr[0] != 0, [6] the matrix has no entries, [7] unused, [8, 8+C) first dependency chunk, [8+C, 8+2C)
// last dependency chunk, then (kNoAllocMaxLevels+1) * C completion counters.
constexpr int kNoAllocHeader = 8;
constexpr long kNoAllocWords =
    kNoAllocHeader + 2L * kNoAllocMaxChunks + (long)(kNoAllocMaxLevels + 1) * kNoAllocMaxChunks;

static __device__ __align__(256) unsigned int g_noalloc_scratch[kNoAllocWords];

std::mutex g_noalloc_mu;
unsigned int *g_noalloc_addr[256];  // device address of the array, per device

// Looks up (once per device, with that device current) the device address
// of g_noalloc_scratch.
int noalloc_scratch(int dev, unsigned int **out) {
  if (dev < 0 || dev >= 256) return fail(kEInval, "device id out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(kECuda, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_addr[dev] = static_cast<unsigned int *>(addr);
  }
  *out = g_noalloc_addr[dev];
  return kOk;
}

// One CTA per chunk: first and last chunk its rows' columns fall in, its
// entry count, and the largest chunk distance (atomics into the header).
// It also validates the caller's CSR, which the host cannot read: a ptr
// that decreases (or ptr[0] != 0) sets word 5, a column outside [0, n) word
// 4, and the host launches nothing more when either is set.  Column reads
// stay inside [0, ptr[n]) even for a malformed ptr (the caller's col holds
// ptr[n] entries).
__global__ void noalloc_deps_kernel(int n, int chunk, const int *__restrict__ ptr,
                                    const int *__restrict__ col, unsigned int *scr) {
  __shared__ int s_lo, s_hi;
  const int c = blockIdx.x;
  const int r0 = c * chunk, r1 = min(n, r0 + chunk);
  if (threadIdx.x == 0) { s_lo = c; s_hi = c; }
  __syncthreads();
  bool bad_ptr = (c == 0 && threadIdx.x == 0 && ptr[0] != 0);
  if (c == 0 && threadIdx.x == 0 && ptr[n] <= 0) atomicExch(scr + 6, 1u);
  for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x) bad_ptr |= ptr[i + 1] < ptr[i];
  const int nnz = ptr[n];
  const int j0 = max(ptr[r0], 0), j1 = min(ptr[r1], nnz);
  int lo = c, hi = c;
  bool bad_col = false;
  for (int j = j0 + (int)threadIdx.x; j < j1; j += blockDim.x) {
    const int cj = col[j];
    if (cj < 0 || cj >= n) {
      bad_col = true;
      continue;
    }
    const int cc = cj / chunk;
    lo = min(lo, cc);
    hi = max(hi, cc);
  }
  if (bad_col) atomicExch(scr + 4, 1u);
  if (bad_ptr) atomicExch(scr + 5, 1u);
  atomicMin(&s_lo, lo);
  atomicMax(&s_hi, hi);
  __syncthreads();
  if (threadIdx.x == 0) {
    scr[kNoAllocHeader + c] = (unsigned)s_lo;
    scr[kNoAllocHeader + kNoAllocMaxChunks + c] = (unsigned)s_hi;
    atomicMax(scr + 2, (unsigned)max(j1 - j0, 0));
    atomicMax(scr + 3, (unsigned)max(c - s_lo, s_hi - c));
  }
}

}  // namespace

extern "C" int mpkg_pipe_noalloc(int n, const int *d_ptr, const int *d_col, const double *d_val,
                                 int nlevel, double *d_vv, void *stream) {
  clear_error();
  if (n <= 0 || !d_ptr || !d_col || !d_val || !d_vv) return fail(kEInval, "null argument or n <= 0");
  if (nlevel < 1 || nlevel > kNoAllocMaxLevels)
    return fail(kEInval, "mpkg_pipe_noalloc: nlevel must be in [1, 16]");
  const int chunk = kPipeChunk;
  const long nchunk = ((long)n + chunk - 1) / chunk;
  if (nchunk > kNoAllocMaxChunks)
    return fail(kERange, "mpkg_pipe_noalloc: n exceeds the fixed scratch limit of 4096*1024 rows");
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  unsigned int *scr = nullptr;
  int rc = noalloc_scratch(dev, &scr);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // the array keeps the previous call's contents: clear header and counters
  CUDA_TRY(cudaMemsetAsync(scr, 0, sizeof(unsigned int) * kNoAllocHeader, st));
  unsigned int *counts = scr + kNoAllocHeader + 2 * kNoAllocMaxChunks;
  CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(unsigned int) * (size_t)(nlevel + 1) * nchunk, st));
  noalloc_deps_kernel<<<(unsigned)nchunk, 256, 0, st>>>(n, chunk, d_ptr, d_col, scr);
  CUDA_TRY(cudaGetLastError());
  unsigned int info[5] = {0, 0, 0, 0, 0};
  CUDA_TRY(cudaMemcpyAsync(info, scr + 2, sizeof info, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (info[3]) return fail(kEInval, "mpkg_pipe_noalloc: ptr[0] must be 0 and ptr non-decreasing");
  if (info[4]) return fail(kEInval, "mpkg_pipe_noalloc: the matrix has no entries");
  if (info[2]) return fail(kERange, "mpkg_pipe_noalloc: column index out of range");
  const int max_nnz = std::max<int>((int)info[0], 1);
  const long reach = info[1];
  const size_t smem = pipe_smem_size(chunk, max_nnz, true, sizeof(double));
  int maxsm = 0, per_sm = 0, nsm = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem > (size_t)maxsm) return fail(kERange, "mpkg_pipe_noalloc: chunk rows too dense for shared memory");
  CUDA_TRY(cudaFuncSetAttribute(pipe_kernel<MPKG_ARITH_FMA, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pipe_kernel<MPKG_ARITH_FMA, true>,
                                                         kPipeThreads, smem));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const long grid = std::min<long>((long)per_sm * nsm, nchunk);
  if (grid < nchunk && grid < (long)(nlevel - 1) * reach + 1)
    return fail(kERange, "mpkg_pipe_noalloc: matrix bandwidth too large for the pipeline");
  PipeArgs a{};
  a.n = n;
  a.nlevel = nlevel;
  a.chunk = chunk;
  a.nchunk = (int)nchunk;
  a.ngroups = (int)nchunk;
  a.epoch = 1;
  a.stall = 0;
  a.gdep_lo = reinterpret_cast<const int *>(scr + kNoAllocHeader);
  a.gdep_hi = reinterpret_cast<const int *>(scr + kNoAllocHeader + kNoAllocMaxChunks);
  a.ptr = d_ptr;
  a.col = d_col;
  a.coef = d_val;
  a.x = d_vv;
  a.vv = d_vv;
  a.ticket = scr;
  a.counts = counts;
  a.err = reinterpret_cast<int *>(scr + 1);
  a.max_chunk_nnz = max_nnz;
  a.bulk_ok = ((uintptr_t)d_col % 16 == 0) && ((uintptr_t)d_val % 16 == 0);
  pipe_kernel<MPKG_ARITH_FMA, true><<<(unsigned)grid, kPipeThreads, smem, st>>>(a);
  CUDA_TRY(cudaGetLastError());
  int err = 0;
  CUDA_TRY(cudaMemcpyAsync(&err, scr + 1, sizeof err, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (err == kErrTimeout) return fail(kETimeout, "mpkg_pipe_noalloc: a device-side wait exceeded its spin limit");
  if (err) return fail(kERange, "mpkg_pipe_noalloc: device-side bounds check failed");
  return kOk;
}
