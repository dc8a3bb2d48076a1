// s-step conjugate gradients around the matrix powers kernel, with the
// pieces that choose its basis: Lanczos Ritz values (Newton shifts), cheap
// matrix features, and a small MLP that maps the features to shifts,
// trained and evaluated by the kernels below.  No counterpart in the
// reference's code (its only s-step material is a numpy notebook with a
// monomial basis); this is the consumer that gives the MPK basis a use.
//
// Precision: the s-step basis is FP32 (values and vectors), the Gram
// matrix Y^T Y and the small coefficient-space iteration are FP64 on the
// GPU, x and the true residual are FP64 (the residual is recomputed from x
// every outer iteration, so the FP32 basis does not limit the attainable
// accuracy).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/mpk_gb300.h"
#include "host.h"

using namespace mpkg;

#define SS_TRY(expr)                                                             \
  do {                                                                           \
    cudaError_t e_ = (expr);                                                     \
    if (e_ != cudaSuccess) return fail(kECuda, std::string(#expr ": ") + cudaGetErrorString(e_)); \
  } while (0)

namespace {

constexpr int kThreads = 256;
constexpr int kMaxS = 10;              // basis length limit (Gram pairs <= threads)
constexpr int kMaxCols = 2 * kMaxS + 1;

int check_csr(int n, const int *ptr, const int *col) {
  if (n <= 0 || !ptr || !col) return fail(kEInval, "empty matrix or null arrays");
  if (ptr[0] != 0) return fail(kEInval, "ptr[0] must be 0");
  for (int i = 0; i < n; i++)
    if (ptr[i + 1] < ptr[i]) return fail(kEInval, "ptr must be non-decreasing");
  for (long j = 0; j < ptr[n]; j++)
    if (col[j] < 0 || col[j] >= n) return fail(kERange, "column index out of range");
  return kOk;
}

int blocks_for(long n) { return (int)std::max<long>(1, std::min<long>((n + kThreads - 1) / kThreads, 1216)); }

// ---- sliced matrix layout ---------------------------------------------------
// Rows in slices of 32; entry t of row i at off[i/32] + 32 t + i%32, so a
// warp's loads of the same slot are coalesced.  Each row keeps CSR order,
// so every row sum below has the bits of the CSR loop.
struct Sell {
  const long *off;   // nslice + 1
  const int *len;    // per row
  const int *col;
  const double *val;
  const float *valf; // FP32 copy (s-step basis), or null
};

__global__ void sell_fill_kernel(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                                 const double *__restrict__ val, const long *__restrict__ off, int *__restrict__ len,
                                 int *__restrict__ scol, double *__restrict__ sval, float *__restrict__ svalf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int q0 = ptr[i], l = ptr[i + 1] - q0;
    const long e0 = off[i >> 5] + (i & 31);
    len[i] = l;
    for (int t = 0; t < l; t++) {
      scol[e0 + 32L * t] = col[q0 + t];
      sval[e0 + 32L * t] = val[q0 + t];
      if (svalf) svalf[e0 + 32L * t] = __double2float_rn(val[q0 + t]);
    }
  }
}

// ---- FP64 vector kernels -------------------------------------------------

// r = b - A x, and per-CTA partial sums of r.r (deterministic reduction).
__global__ void resid_kernel(int n, Sell a, const double *__restrict__ x, const double *__restrict__ b,
                             double *__restrict__ r, double *__restrict__ part) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    const long e0 = a.off[i >> 5] + (i & 31);
    const int l = a.len[i];
    for (int t = 0; t < l; t++) s = fma(a.val[e0 + 32L * t], x[a.col[e0 + 32L * t]], s);
    const double ri = b[i] - s;
    r[i] = ri;
    acc = fma(ri, ri, acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// y = A x (FP64), optionally y -= beta * z; partial sums of y.x
__global__ void spmv64_kernel(int n, Sell a, const double *__restrict__ x, double *__restrict__ y,
                              const double *__restrict__ z, double beta, double *__restrict__ part) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    const long e0 = a.off[i >> 5] + (i & 31);
    const int l = a.len[i];
    for (int t = 0; t < l; t++) s = fma(a.val[e0 + 32L * t], x[a.col[e0 + 32L * t]], s);
    if (z) s = fma(-beta, z[i], s);
    y[i] = s;
    acc = fma(s, x[i], acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0 && part) part[blockIdx.x] = red[0];
}

// y = y + a * x; partial sums of y.y
__global__ void axpy_norm_kernel(int n, double a, const double *__restrict__ x, double *__restrict__ y,
                                 double *__restrict__ part) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = fma(a, x[i], y[i]);
    y[i] = v;
    acc = fma(v, v, acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// y = a * x + b * y (no reduction)
__global__ void axpby_kernel(int n, double a, const double *__restrict__ x, double b, double *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = fma(a, x[i], b * y[i]);
}

// ---- s-step basis (FP32) ---------------------------------------------------

// Column c of the basis Y (column-major, n floats each).  P block: columns
// 0..s, R block: columns s+1..2s.  Start columns: p / |p| and r / |r|.
// The scalars of an outer iteration, in device memory so that the whole
// iteration replays as one graph: [0] |p|, [1] |r|, [2] 1/|p|, [3] 1/|r|,
// [4] r.r, [5] p.p.
constexpr int kScalars = 6;

// r.r and p.p from the per-CTA partial sums (one warp: lane j sums
// partials j, j+32, ... in order, then a fixed butterfly, so the same bits
// on every run), and the norms that scale the next basis.
__global__ void norms_kernel(int nb, const double *__restrict__ part, double *__restrict__ sc) {
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  double rr = 0.0, pp = 0.0;
  for (int k = lane; k < nb; k += 32) {
    rr += part[k];
    pp += part[nb + k];
  }
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_xor_sync(0xFFFFFFFFu, rr, o);
    pp += __shfl_xor_sync(0xFFFFFFFFu, pp, o);
  }
  if (lane != 0) return;
  const double pn = sqrt(pp), rn = sqrt(rr);
  sc[0] = pn;
  sc[1] = rn;
  sc[2] = 1.0 / pn;
  sc[3] = 1.0 / rn;
  sc[4] = rr;
  sc[5] = pp;
}

// The whole solve as one graph: a conditional WHILE node whose body is
// one outer iteration, ended by decide_kernel (one warp), which counts the
// iteration, records the P block of the Gram matrix for the host's
// condition number (a ring in page-locked memory, with a progress count),
// asks for a restart when p.p is not positive, and sets the loop
// condition: more iterations allowed, progress made, |r| above tol |b|.
// The count of iterations bounds the loop by max_outer.
struct LoopState {
  int outer, steps, breakdowns, restart;
};
constexpr int kCondRing = 512;

__global__ void restart_kernel(int n, const LoopState *__restrict__ st, const double *__restrict__ r,
                               double *__restrict__ p, double *__restrict__ sc) {
  if (!st->restart) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = r[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) {  // |p| = |r|, p.p = r.r
    sc[0] = sc[1];
    sc[2] = sc[3];
    sc[5] = sc[4];
  }
}

__global__ void decide_kernel(int s, int m, const int *__restrict__ flag, const double *__restrict__ sc,
                              const double *__restrict__ g, int max_outer, double rtol, LoopState *st, double *ring,
                              int *progress, cudaGraphConditionalHandle loop) {
  const int lane = threadIdx.x, mp = s + 1, o = st->outer;
  double *slot = ring + (size_t)(o % kCondRing) * mp * mp;
  for (int k = lane; k < mp * mp; k += 32) slot[k] = g[(k / mp) * m + k % mp];
  __threadfence_system();
  __syncwarp();
  if (lane != 0) return;
  const int steps = flag[1];
  st->outer = o + 1;
  st->steps += steps;
  st->breakdowns += flag[0];
  st->restart = steps > 0 && !(sc[5] > 0.0);
  const bool more = o + 1 < max_outer && steps > 0 && sqrt(sc[4]) > rtol;
  __threadfence_system();
  *(volatile int *)progress = o + 1;
  cudaGraphSetConditional(loop, more ? 1u : 0u);
}

__global__ void basis_start_kernel(int n, const double *__restrict__ p, const double *__restrict__ r,
                                   const double *__restrict__ sc, float *__restrict__ y0, float *__restrict__ yr) {
  const double ip = sc[2], ir = sc[3];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    y0[i] = (float)(p[i] * ip);
    yr[i] = (float)(r[i] * ir);
  }
}

// Row i of one Newton step of both blocks: out = (A in - theta in) / sigma,
// FP32 values and accumulation in CSR order (the R block when rout is not
// null); the row's entry t at cb[32 t] / vb[32 t] (the sliced layout, in
// global or shared memory).  Both basis builders below run this code, so
// they give the same bits.  The inputs are plain loads: the matrix-powers
// form reads levels that other CTAs wrote during the same launch.
__device__ __forceinline__ void newton_row(int i, int l, const int *cb, const float *vb, const float *pin, float *pout,
                                           const float *rin, float *rout, float theta, float rsigma) {
  float sp = 0.f, sr = 0.f;
  int t = 0;
  if (l <= 8) {  // all of a short row's loads in flight together: columns, then both gathers
    int c[8];
    float v[8], xp[8], xr[8];
#pragma unroll
    for (int u = 0; u < 8; u++)
      if (u < l) {
        c[u] = cb[32 * u];
        v[u] = vb[32 * u];
      }
#pragma unroll
    for (int u = 0; u < 8; u++)
      if (u < l) {
        xp[u] = pin[c[u]];
        xr[u] = rout ? rin[c[u]] : 0.f;
      }
#pragma unroll
    for (int u = 0; u < 8; u++)
      if (u < l) {
        sp = __fmaf_rn(v[u], xp[u], sp);
        if (rout) sr = __fmaf_rn(v[u], xr[u], sr);
      }
    t = l;
  }
  for (; t < l; t++) {
    const int c = cb[32 * t];
    const float v = vb[32 * t];
    sp = __fmaf_rn(v, pin[c], sp);
    if (rout) sr = __fmaf_rn(v, rin[c], sr);
  }
  pout[i] = __fmul_rn(__fmaf_rn(-theta, pin[i], sp), rsigma);
  if (rout) rout[i] = __fmul_rn(__fmaf_rn(-theta, rin[i], sr), rsigma);
}

// One Newton step of both blocks over all rows (one launch per step); the
// R block stops one step early.
__global__ void basis_step_kernel(int n, Sell a, const float *pin, float *pout, const float *rin, float *rout,
                                  float theta, float rsigma) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long e0 = a.off[i >> 5] + (i & 31);
    newton_row(i, a.len[i], a.col + e0, a.valf + e0, pin, pout, rin, rout, theta, rsigma);
  }
}

// The whole basis [p, rho_1(A) p, ..., rho_s(A) p, r, ..., rho_(s-1)(A) r]
// as ONE matrix powers launch (the wavefront form): CTA b owns rows
// [row_lo[b], row_lo[b+1]) (slice aligned, so no cache line holds two
// CTAs' rows) at every level, and computes level j once the CTAs owning
// the columns of its rows (an exact list) have published level j - 1.
// STAGE: the CTA's slab of the sliced matrix (columns and FP32 values) is
// copied into shared memory once and serves all s levels, so the matrix is
// read once per basis instead of once per step.  The levels are the basis
// vectors themselves, each a fresh buffer, so no CTA overwrites what
// another still reads.  Waits are bounded: a wait that gives up sets *err
// and the launch ends (the host reports MPKG_ETIMEOUT).  flags are reset
// to 0 before every launch.
struct BasisWave {
  int n, s, nblk;
  const int *row_lo;     // nblk + 1
  const int *dep_ptr;    // nblk + 1: CTA b waits for dep_idx[dep_ptr[b] .. dep_ptr[b+1])
  const int *dep_idx;
  unsigned int *flags;   // nblk: last level published
  int *err;
  unsigned int stall;    // test hook: extra levels to wait for (never published)
  float theta[kMaxS], rsig[kMaxS];
};

constexpr long kBasisSpin = 4000000;  // polls of one flag (~1 s with backoff)

__device__ __forceinline__ unsigned int acquire_u32(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <bool STAGE>
__global__ void __launch_bounds__(kThreads) basis_wave_kernel(BasisWave w, Sell a, float *Y) {
  extern __shared__ __align__(16) int bw_slab[];
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = 0;
  const int b = blockIdx.x, r0 = w.row_lo[b], r1 = w.row_lo[b + 1];
  const size_t n = (size_t)w.n;
  const long e_lo = r0 < r1 ? a.off[r0 >> 5] : 0;
  int *s_col = bw_slab;
  float *s_val = nullptr;
  if (STAGE && r0 < r1) {
    const long ne = a.off[(r1 + 31) >> 5] - e_lo;  // a multiple of 32 entries
    s_val = reinterpret_cast<float *>(bw_slab + ne);
    const int4 *gc = reinterpret_cast<const int4 *>(a.col + e_lo);
    const float4 *gv = reinterpret_cast<const float4 *>(a.valf + e_lo);
    for (long q = threadIdx.x; q < ne / 4; q += blockDim.x) {
      reinterpret_cast<int4 *>(s_col)[q] = gc[q];
      reinterpret_cast<float4 *>(s_val)[q] = gv[q];
    }
  }
  __syncthreads();
  for (int j = 1; j <= w.s; j++) {
    if (j > 1) {
      for (int k = w.dep_ptr[b] + (int)threadIdx.x; k < w.dep_ptr[b + 1]; k += blockDim.x) {
        const int c = w.dep_idx[k];
        long spins = 0;
        while (acquire_u32(w.flags + c) < (unsigned)(j - 1) + w.stall) {
          if (++spins > kBasisSpin || *((volatile int *)w.err)) {
            atomicCAS(w.err, 0, 1);
            s_abort = 1;
            break;
          }
          __nanosleep(spins < 16 ? 32 : 256);
        }
      }
      __syncthreads();
      if (s_abort) return;
    }
    const bool rstep = j < w.s;
    const float *pin = Y + (size_t)(j - 1) * n;
    float *pout = Y + (size_t)j * n;
    const float *rin = rstep ? Y + (size_t)(w.s + j) * n : nullptr;
    float *rout = rstep ? Y + (size_t)(w.s + 1 + j) * n : nullptr;
    for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x) {
      const long e0 = a.off[i >> 5] + (i & 31);
      if (STAGE)
        newton_row(i, a.len[i], s_col + (e0 - e_lo), s_val + (e0 - e_lo), pin, pout, rin, rout, w.theta[j - 1],
                   w.rsig[j - 1]);
      else
        newton_row(i, a.len[i], a.col + e0, a.valf + e0, pin, pout, rin, rout, w.theta[j - 1], w.rsig[j - 1]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(w.flags + b), "r"((unsigned)j) : "memory");
    }
  }
}

// Gram matrix G = Y^T Y of the FP32 basis.  Every product a*b of two FP32
// values is exact in FP64 (48-bit mantissa).  F64: the products are
// summed with FP64 FMAs (the FP64 Gram of the s-step method).  !F64: each
// product is split exactly into p + e (p = a*b rounded, e = fma(a, b, -p))
// and summed in double-float on the FP32 pipes (a two-sum on the high
// parts, errors and low parts added; about 2^-46 relative to the sum of
// |products|), for GB300 whose FP64 pipe runs at 1/64 of FP32.
// A CTA stages a tile of rows of all columns in shared memory; thread t
// accumulates pair t of the upper triangle with four independent sums;
// per-CTA partials (FP64) are summed in a fixed order by gram_reduce_kernel.
constexpr int kGramRows = 64;
thread_local bool g_gram_f64 = true;  // mpkg_sstep_gram: FP64 (default) or double-float Gram
thread_local bool g_device_loop = true;  // mpkg_sstep_loop: device-side (default) or host-side outer loop
thread_local bool g_basis_mpk = false;   // mpkg_sstep_basis: s launches (default) or one matrix powers launch
thread_local unsigned g_basis_stall = 0;  // mpkg_sstep_debug_stall
__device__ __forceinline__ void gram_acc(float a, float b, float &sh, float &sl) {
  const float p = __fmul_rn(a, b), e = __fmaf_rn(a, b, -p);
  const float t = __fadd_rn(sh, p), bp = __fadd_rn(t, -sh);
  const float err = __fadd_rn(__fadd_rn(sh, -__fadd_rn(t, -bp)), __fadd_rn(p, -bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

template <bool F64>
__global__ void __launch_bounds__(kThreads) gram_kernel(int n, int ncol, const float *__restrict__ y,
                                                        double *__restrict__ part) {
  // one padding word per column: the threads of a warp read up to 17
  // different columns at the same row, which would otherwise share a bank.
  // F64 stages the values already widened, so that each is converted once
  // per tile rather than once per pair (the conversion shares the FP64 pipe)
  using Stage = typename std::conditional<F64, double, float>::type;
  __shared__ Stage tile[kMaxCols][kGramRows + 1];
  const int npair = ncol * (ncol + 1) / 2;
  int pa = 0, pb = 0;
  {
    int t = threadIdx.x, a = 0;
    while (a < ncol && t >= ncol - a) { t -= ncol - a; a++; }
    pa = a;
    pb = a + t;
  }
  float h[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (long r0 = (long)blockIdx.x * kGramRows; r0 < n; r0 += (long)gridDim.x * kGramRows) {
    __syncthreads();
    for (int e = threadIdx.x; e < ncol * kGramRows; e += blockDim.x) {
      const int c = e / kGramRows, rr = e % kGramRows;
      tile[c][rr] = (Stage)(r0 + rr < n ? y[(size_t)c * n + r0 + rr] : 0.f);
    }
    __syncthreads();
    if ((int)threadIdx.x < npair) {  // four independent partial sums per thread
#pragma unroll 4
      for (int rr = 0; rr < kGramRows; rr += 4) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          if (F64) acc[u] = fma((double)tile[pa][rr + u], (double)tile[pb][rr + u], acc[u]);
          else gram_acc((float)tile[pa][rr + u], (float)tile[pb][rr + u], h[u], lo[u]);
        }
      }
    }
  }
  if ((int)threadIdx.x < npair) {
    double s = 0.0;
    for (int k = 0; k < 4; k++) s += F64 ? acc[k] : (double)h[k] + (double)lo[k];
    part[(size_t)blockIdx.x * npair + threadIdx.x] = s;
  }
}

// One warp per pair: lane j sums partials j, j+32, ... in order, then a
// fixed butterfly combines the lanes (the same bits on every run).
__global__ void gram_reduce_kernel(int nblk, int ncol, const double *__restrict__ part, double *__restrict__ g) {
  const int npair = ncol * (ncol + 1) / 2;
  const int lane = threadIdx.x & 31;
  const int t = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (t >= npair) return;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += part[(size_t)b * npair + t];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
  if (lane == 0) {
    int a = 0, u = t;
    while (u >= ncol - a) { u -= ncol - a; a++; }
    g[a * ncol + a + u] = s;
    g[(a + u) * ncol + a] = s;
  }
}

// The s inner CG steps in coefficient space (FP64, one warp; lane c holds
// coefficient c, m = 2s+1 <= 32): p = Y ph, r = Y rh, A Y = Y B on the
// columns in use.  Outputs xh, ph (and rh).  flag[0] = 1 when a breakdown
// (non-positive curvature or residual) stopped the inner loop early;
// flag[1] = steps taken.
__global__ void coeff_kernel(int s, const double *__restrict__ g, const double *__restrict__ theta,
                             const double *__restrict__ sigma, const double *__restrict__ sc, double *__restrict__ xh,
                             double *__restrict__ ph, double *__restrict__ rh, int *__restrict__ flag) {
  const double pnorm = sc[0], rnorm = sc[1];
  const int m = 2 * s + 1, c = threadIdx.x;
  const bool on = c < m;
  double p = 0.0, r = 0.0, x = 0.0;
  if (c == 0) p = pnorm;
  if (c == s + 1) r = rnorm;
  // B v: column j of the P block (j < s) maps to theta_j e_j + sigma_j e_(j+1),
  // the R block likewise up to its second-to-last column
  auto apply_b = [&](double v) {
    const double vm1 = __shfl_up_sync(0xffffffffu, v, 1);
    double out = 0.0;
    if (c < s) out += theta[c] * v;
    if (c >= 1 && c <= s) out += sigma[c - 1] * vm1;
    if (c >= s + 1 && c < 2 * s) out += theta[c - s - 1] * v;
    if (c >= s + 2 && c <= 2 * s) out += sigma[c - s - 2] * vm1;
    return on ? out : 0.0;
  };
  // lane c keeps row c of G in registers for the s steps
  double grow[kMaxCols];
#pragma unroll
  for (int b = 0; b < kMaxCols; b++) grow[b] = on && b < m ? g[c * m + b] : 0.0;
  // u^T G v, v distributed over the lanes; three independent partial sums
  // per row (the FP64 FMA latency bounds this one-warp kernel)
  auto gdot = [&](double u, double v) {
    double w[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int b = 0; b < kMaxCols; b++) {
      if (b < m) w[b % 3] = fma(grow[b], __shfl_sync(0xffffffffu, v, b), w[b % 3]);
    }
    double t = on ? u * ((w[0] + w[1]) + w[2]) : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
  };
  int steps = 0, brk = 0;
  double rr = gdot(r, r);
  for (int j = 0; j < s; j++) {
    const double bp = apply_b(p);
    const double pap = gdot(p, bp);
    if (!(pap > 0.0) || !(rr > 0.0)) { brk = 1; break; }
    const double alpha = rr / pap;
    x += alpha * p;
    const double rn = r - alpha * bp;
    const double rr2 = gdot(rn, rn);
    const double beta = rr2 / rr;
    r = rn;
    p = rn + beta * p;
    rr = rr2;
    steps++;
  }
  if (on) { xh[c] = x; ph[c] = p; rh[c] = r; }
  if (c == 0) { flag[0] = brk; flag[1] = steps; }
}

// x += Y xh and p = Y ph: the coefficient (FP64) times basis (FP32)
// products and their sums in double-float on the FP32 pipes (each
// coefficient split into two floats; products exact up to the low part's
// rounding, about 2^-46 relative), then one FP64 add into x per row.
__device__ __forceinline__ double ss_widen(float f) {  // exact float -> double in integer arithmetic
  const unsigned int u = __float_as_uint(f);
  const unsigned int e = (u >> 23) & 0xFF;
  const unsigned int sgn = u & 0x80000000u;
  const unsigned int bias = e == 0xFF ? (1792u << 20) : (896u << 20);
  const unsigned int hi = e == 0 ? sgn : (sgn | (((u >> 3) & 0x0FFFFFFFu) + bias));
  const unsigned int lo = e == 0 ? 0u : (u << 29);
  return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ void ss_mac(float ch, float cl, float v, float &sh, float &sl) {
  const float p = __fmul_rn(ch, v);
  float e = __fmaf_rn(ch, v, -p);
  e = __fmaf_rn(cl, v, e);
  const float t = __fadd_rn(sh, p), bp = __fadd_rn(t, -sh);
  const float err = __fadd_rn(__fadd_rn(sh, -__fadd_rn(t, -bp)), __fadd_rn(p, -bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// Also the per-CTA partial sums of p.p (same order and tree as
// axpy_norm_kernel on the same grid, so the same bits).
__global__ void combine_kernel(int n, int m, const float *__restrict__ y, const double *__restrict__ xh,
                               const double *__restrict__ ph, double *__restrict__ x, double *__restrict__ p,
                               double *__restrict__ part) {
  __shared__ float cxh[kMaxCols], cxl[kMaxCols], cph[kMaxCols], cpl[kMaxCols];
  __shared__ double red[kThreads];
  double acc = 0.0;
  if ((int)threadIdx.x < m) {
    const double a = xh[threadIdx.x], b = ph[threadIdx.x];
    cxh[threadIdx.x] = __double2float_rn(a);
    cxl[threadIdx.x] = __double2float_rn(a - (double)cxh[threadIdx.x]);
    cph[threadIdx.x] = __double2float_rn(b);
    cpl[threadIdx.x] = __double2float_rn(b - (double)cph[threadIdx.x]);
  }
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float xs = 0.f, xl = 0.f, ps = 0.f, pl = 0.f;
    for (int c = 0; c < m; c++) {
      const float v = y[(size_t)c * n + i];
      ss_mac(cxh[c], cxl[c], v, xs, xl);
      ss_mac(cph[c], cpl[c], v, ps, pl);
    }
    x[i] += ss_widen(xs) + ss_widen(xl);
    const double pv = ss_widen(ps) + ss_widen(pl);
    p[i] = pv;
    acc = fma(pv, pv, acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// ---- matrix features ---------------------------------------------------------
// Per row: diagonal, sum of |off-diagonals|, 2-norm, degree; per CTA
// partial min/max/sums (fixed-order final reduction on the host).
struct FeatPart {
  double glo, ghi, dmin, dmax, dsum, osum, omax, nsum, nsq, degmax, degsum, dommin, domsum;
};
__global__ void features_kernel(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                                const double *__restrict__ val, FeatPart *__restrict__ part) {
  __shared__ FeatPart red[kThreads];
  FeatPart f = {1e300, -1e300, 1e300, -1e300, 0, 0, 0, 0, 0, 0, 0, 1e300, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 0.0, o = 0.0, n2 = 0.0;
    for (int q = ptr[i]; q < ptr[i + 1]; q++) {
      const double v = val[q];
      n2 = fma(v, v, n2);
      if (col[q] == i) d += v;
      else o += fabs(v);
    }
    const double deg = ptr[i + 1] - ptr[i];
    f.glo = fmin(f.glo, d - o);
    f.ghi = fmax(f.ghi, d + o);
    f.dmin = fmin(f.dmin, d);
    f.dmax = fmax(f.dmax, d);
    f.dsum += d;
    f.osum += o;
    f.omax = fmax(f.omax, o);
    const double nr = sqrt(n2);
    f.nsum += nr;
    f.nsq += n2;
    f.degmax = fmax(f.degmax, deg);
    f.degsum += deg;
    const double dom = o > 0.0 ? fabs(d) / o : 10.0;
    f.dommin = fmin(f.dommin, dom);
    f.domsum += fmin(dom, 10.0);
  }
  red[threadIdx.x] = f;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      FeatPart &a = red[threadIdx.x];
      const FeatPart &b = red[threadIdx.x + w];
      a.glo = fmin(a.glo, b.glo); a.ghi = fmax(a.ghi, b.ghi);
      a.dmin = fmin(a.dmin, b.dmin); a.dmax = fmax(a.dmax, b.dmax);
      a.dsum += b.dsum; a.osum += b.osum; a.omax = fmax(a.omax, b.omax);
      a.nsum += b.nsum; a.nsq += b.nsq; a.degmax = fmax(a.degmax, b.degmax); a.degsum += b.degsum;
      a.dommin = fmin(a.dommin, b.dommin); a.domsum += b.domsum;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// ---- device copy of a CSR matrix ------------------------------------------
struct DevCsr {
  int n = 0;
  long nnz = 0;
  int *ptr = nullptr, *col = nullptr;
  double *val = nullptr;
  long *soff = nullptr;
  int *slen = nullptr, *scol = nullptr;
  double *sval = nullptr;
  float *svalf = nullptr;
  std::vector<long> soff_h;  // host copy of the slice offsets
  ~DevCsr() {
    cudaFree(ptr); cudaFree(col); cudaFree(val);
    cudaFree(soff); cudaFree(slen); cudaFree(scol); cudaFree(sval); cudaFree(svalf);
  }
  Sell sell() const { return Sell{soff, slen, scol, sval, svalf}; }
  int upload(int n_, const int *p, const int *c, const double *v, bool f32) {
    int rc = check_csr(n_, p, c);
    if (rc) return rc;
    n = n_;
    nnz = p[n_];
    SS_TRY(cudaMalloc(&ptr, sizeof(int) * (n + 1)));
    SS_TRY(cudaMalloc(&col, sizeof(int) * std::max<long>(nnz, 1)));
    SS_TRY(cudaMalloc(&val, sizeof(double) * std::max<long>(nnz, 1)));
    SS_TRY(cudaMemcpy(ptr, p, sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
    SS_TRY(cudaMemcpy(col, c, sizeof(int) * nnz, cudaMemcpyHostToDevice));
    SS_TRY(cudaMemcpy(val, v, sizeof(double) * nnz, cudaMemcpyHostToDevice));
    // the sliced copy, filled on the device from the CSR arrays
    const int nsl = (n + 31) / 32;
    std::vector<long> so(nsl + 1, 0);
    for (int sl = 0; sl < nsl; sl++) {
      int w = 0;
      for (int i = sl * 32; i < std::min(n, sl * 32 + 32); i++) w = std::max(w, p[i + 1] - p[i]);
      so[sl + 1] = so[sl] + 32L * w;
    }
    const size_t ne = (size_t)std::max<long>(so[nsl], 1);
    SS_TRY(cudaMalloc(&soff, sizeof(long) * (nsl + 1)));
    SS_TRY(cudaMalloc(&slen, sizeof(int) * n));
    SS_TRY(cudaMalloc(&scol, sizeof(int) * ne));
    SS_TRY(cudaMalloc(&sval, sizeof(double) * ne));
    if (f32) SS_TRY(cudaMalloc(&svalf, sizeof(float) * ne));
    SS_TRY(cudaMemcpy(soff, so.data(), sizeof(long) * (nsl + 1), cudaMemcpyHostToDevice));
    soff_h = so;
    sell_fill_kernel<<<blocks_for(n), kThreads>>>(n, ptr, col, val, soff, slen, scol, sval, svalf);
    SS_TRY(cudaGetLastError());
    return kOk;
  }
};

template <typename T>
struct DevBuf {
  T *p = nullptr;
  ~DevBuf() { cudaFree(p); }
  int alloc(size_t n) {
    SS_TRY(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)));
    return kOk;
  }
};

// A captured graph, its instance and its stream, released on scope exit.
struct GraphRun {
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~GraphRun() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (st) cudaStreamDestroy(st);
  }
};

// Page-locked, device-mapped ring of P-block Gram matrices and the
// progress count written by decide_kernel.
struct LoopHost {
  void *base = nullptr;
  double *ring = nullptr, *d_ring = nullptr;
  int *progress = nullptr, *d_progress = nullptr;
  ~LoopHost() {
    if (base) cudaFreeHost(base);
  }
  bool alloc(size_t ring_doubles) {
    const size_t bytes = sizeof(double) * ring_doubles + 64;
    void *d = nullptr;
    if (cudaHostAlloc(&base, bytes, cudaHostAllocMapped) != cudaSuccess) {
      base = nullptr;
      cudaGetLastError();
      return false;
    }
    std::memset(base, 0, bytes);
    if (cudaHostGetDevicePointer(&d, base, 0) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    ring = static_cast<double *>(base);
    progress = reinterpret_cast<int *>(static_cast<char *>(base) + sizeof(double) * ring_doubles);
    d_ring = static_cast<double *>(d);
    d_progress = reinterpret_cast<int *>(static_cast<char *>(d) + sizeof(double) * ring_doubles);
    return true;
  }
};

// A graph holding one conditional WHILE node whose body `body(stream,
// handle)` issues by stream capture.  False (and no graph) when the
// runtime refuses any step; the caller then loops on the host.
template <typename F>
bool build_device_loop(GraphRun &gr, F &&body) {
  cudaGraph_t g = nullptr, out = nullptr;
  cudaGraphConditionalHandle h;
  cudaGraphNode_t node;
  cudaGraphNodeParams np = {};
  bool ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
            cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault) == cudaSuccess;
  if (ok) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) == cudaSuccess;
  }
  if (ok) ok = cudaStreamBeginCaptureToGraph(gr.st, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    body(gr.st, h);
    ok = cudaStreamEndCapture(gr.st, &out) == cudaSuccess;
  }
  if (ok) ok = cudaGraphInstantiate(&gr.exec, g, 0) == cudaSuccess;
  if (!ok) {
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
    gr.exec = nullptr;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return false;
  }
  gr.graph = g;
  return true;
}

// The basis wavefront's layout: slice-aligned CTA row ranges of equal size
// and, per CTA, the exact list of CTAs owning the columns of its rows;
// the grid and whether the CTAs' matrix slabs fit shared memory.
struct BasisLayout {
  DevBuf<int> row_lo, dep_ptr, dep_idx, err;
  DevBuf<unsigned int> flags;
  BasisWave w{};
  bool coop = false;   // cooperative launch attribute accepted in stream capture
  bool stage = false;  // slabs staged in shared memory
  size_t smem = 0;
  int build(int n, const int *ptr, const int *col, const std::vector<long> &soff, int s,
            const std::vector<double> &th, const std::vector<double> &sg) {
    int dev = 0, nsm = 0, maxsm = 0;
    SS_TRY(cudaGetDevice(&dev));
    SS_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    SS_TRY(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const int nsl = (n + 31) / 32;
    auto split = [&](int nblk, std::vector<int> *lo) {
      lo->resize(nblk + 1);
      for (int b = 0; b <= nblk; b++) (*lo)[b] = (int)std::min<long>(n, 32L * ((long)b * nsl / nblk));
    };
    // the most CTAs per SM whose slabs fit shared memory (8 .. 1), else
    // the plain occupancy without staging
    std::vector<int> lo;
    int nblk = 0;
    for (int c = 8; c >= 1 && !stage; c--) {
      const int nb = std::max(1, std::min(c * nsm, nsl));
      split(nb, &lo);
      long maxe = 0;
      for (int b = 0; b < nb; b++)
        if (lo[b] < lo[b + 1]) maxe = std::max(maxe, soff[(lo[b + 1] + 31) / 32] - soff[lo[b] / 32]);
      const size_t bytes = (size_t)maxe * (sizeof(int) + sizeof(float));
      if (bytes > (size_t)maxsm) continue;
      int per_sm = 0;
      if (cudaFuncSetAttribute(basis_wave_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
              cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, basis_wave_kernel<true>, kThreads, bytes) !=
              cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      if ((long)per_sm * nsm < nb) continue;
      stage = true;
      smem = bytes;
      nblk = nb;
    }
    if (!stage) {
      int per_sm = 0;
      SS_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, basis_wave_kernel<false>, kThreads, 0));
      nblk = std::max(1, std::min(per_sm * nsm, nsl));
      split(nblk, &lo);
    }
    // exact dependency lists: the owners of every column of the CTA's rows
    std::vector<int> owner_of(n), dp(nblk + 1, 0), di;
    for (int b = 0; b < nblk; b++)
      for (int i = lo[b]; i < lo[b + 1]; i++) owner_of[i] = b;
    std::vector<int> mark(nblk, -1);
    for (int b = 0; b < nblk; b++) {
      for (int i = lo[b]; i < lo[b + 1]; i++)
        for (int j = ptr[i]; j < ptr[i + 1]; j++) {
          const int o = owner_of[col[j]];
          if (o != b && mark[o] != b) {
            mark[o] = b;
            di.push_back(o);
          }
        }
      std::sort(di.begin() + dp[b], di.end());
      dp[b + 1] = (int)di.size();
    }
    int rc;
    if ((rc = row_lo.alloc(nblk + 1)) || (rc = dep_ptr.alloc(nblk + 1)) || (rc = dep_idx.alloc(di.size())) ||
        (rc = flags.alloc(nblk)) || (rc = err.alloc(1)))
      return rc;
    SS_TRY(cudaMemcpy(row_lo.p, lo.data(), sizeof(int) * (nblk + 1), cudaMemcpyHostToDevice));
    SS_TRY(cudaMemcpy(dep_ptr.p, dp.data(), sizeof(int) * (nblk + 1), cudaMemcpyHostToDevice));
    if (!di.empty()) SS_TRY(cudaMemcpy(dep_idx.p, di.data(), sizeof(int) * di.size(), cudaMemcpyHostToDevice));
    SS_TRY(cudaMemset(err.p, 0, sizeof(int)));
    w.n = n; w.s = s; w.nblk = nblk; w.stall = g_basis_stall;
    w.row_lo = row_lo.p; w.dep_ptr = dep_ptr.p; w.dep_idx = dep_idx.p; w.flags = flags.p; w.err = err.p;
    for (int j = 0; j < s; j++) {
      w.theta[j] = (float)th[j];
      w.rsig[j] = (float)(1.0 / sg[j]);
    }
    return kOk;
  }
  cudaError_t launch(const Sell &a, float *Y, cudaStream_t cs) const {
    cudaError_t e = cudaMemsetAsync(flags.p, 0, sizeof(unsigned int) * (size_t)w.nblk, cs);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)w.nblk);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = stage ? smem : 0;
    cfg.stream = cs;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = coop ? 1 : 0;
    return stage ? cudaLaunchKernelEx(&cfg, basis_wave_kernel<true>, w, a, Y)
                 : cudaLaunchKernelEx(&cfg, basis_wave_kernel<false>, w, a, Y);
  }
  // Whether a cooperative launch can be captured into a graph here; if not,
  // the grid (sized by the occupancy calculator, every CTA resident on an
  // otherwise idle device) is launched plainly and the bounded waits guard it.
  void probe(const Sell &a, float *Y) {
    cudaStream_t st = nullptr;
    cudaGraph_t g = nullptr;
    coop = false;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); return; }
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      coop = true;
      const bool ok = launch(a, Y, st) == cudaSuccess;
      coop = cudaStreamEndCapture(st, &g) == cudaSuccess && ok;
    }
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(st);
    cudaGetLastError();
  }
};

// Page-locked host bytes (int-addressed), released on scope exit.
struct HostBuf {
  int *p = nullptr;
  ~HostBuf() { cudaFreeHost(p); }
  int alloc(size_t bytes) {
    SS_TRY(cudaMallocHost((void **)&p, bytes));
    return kOk;
  }
};

int sum_parts(const double *d_part, int nblk, double *out) {
  std::vector<double> h(nblk);
  SS_TRY(cudaMemcpy(h.data(), d_part, sizeof(double) * nblk, cudaMemcpyDeviceToHost));
  double s = 0.0;
  for (double v : h) s += v;
  *out = s;
  return kOk;
}

// Eigenvalues of the symmetric tridiagonal (alpha diag, beta off) by
// bisection on Sturm sequence counts, ascending.
void tridiag_eigs(int m, const double *alpha, const double *beta, double *out) {
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < m; i++) {
    const double r = (i > 0 ? std::fabs(beta[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(beta[i]) : 0.0);
    lo = std::min(lo, alpha[i] - r);
    hi = std::max(hi, alpha[i] + r);
  }
  auto count_below = [&](double x) {  // eigenvalues < x
    int c = 0;
    double d = 1.0;
    for (int i = 0; i < m; i++) {
      const double b2 = i > 0 ? beta[i - 1] * beta[i - 1] : 0.0;
      d = alpha[i] - x - (i > 0 ? b2 / d : 0.0);
      if (d == 0.0) d = -1e-300;
      if (d < 0.0) c++;
    }
    return c;
  };
  for (int k = 0; k < m; k++) {
    double a = lo, b = hi;
    for (int it = 0; it < 200 && b - a > 1e-15 * std::max(1.0, std::fabs(a) + std::fabs(b)); it++) {
      const double mid = 0.5 * (a + b);
      if (count_below(mid) > k) b = mid;
      else a = mid;
    }
    out[k] = 0.5 * (a + b);
  }
}

}  // namespace

extern "C" {

void mpkg_tridiag_eigs(int m, const double *alpha, const double *beta, double *out) {
  if (m > 0 && alpha && out && (m == 1 || beta)) tridiag_eigs(m, alpha, beta, out);
}

void mpkg_leja_order(int k, double *x) {
  if (!x || k <= 1) return;
  std::vector<double> v(x, x + k), o;
  std::vector<char> used(k, 0);
  int first = 0;
  for (int i = 1; i < k; i++)
    if (std::fabs(v[i]) > std::fabs(v[first])) first = i;
  o.push_back(v[first]);
  used[first] = 1;
  while ((int)o.size() < k) {
    int best = -1;
    double bv = -1.0;
    for (int i = 0; i < k; i++) {
      if (used[i]) continue;
      double prod = 0.0;  // log of the product of distances (robust to under/overflow)
      for (double c : o) prod += std::log(std::fabs(v[i] - c) + 1e-300);
      if (best < 0 || prod > bv) { bv = prod; best = i; }
    }
    used[best] = 1;
    o.push_back(v[best]);
  }
  std::copy(o.begin(), o.end(), x);
}

int mpkg_features(int n, const int *ptr, const int *col, const double *val, float *feat, double *glo, double *ghi) {
  clear_error();
  if (!val || !feat) return fail(kEInval, "null argument");
  DevCsr a;
  int rc = a.upload(n, ptr, col, val, false);
  if (rc) return rc;
  const int nb = blocks_for(n);
  DevBuf<FeatPart> part;
  if ((rc = part.alloc(nb))) return rc;
  features_kernel<<<nb, kThreads>>>(n, a.ptr, a.col, a.val, part.p);
  SS_TRY(cudaGetLastError());
  std::vector<FeatPart> h(nb);
  SS_TRY(cudaMemcpy(h.data(), part.p, sizeof(FeatPart) * nb, cudaMemcpyDeviceToHost));
  FeatPart f = h[0];
  for (int b = 1; b < nb; b++) {
    const FeatPart &o = h[b];
    f.glo = std::min(f.glo, o.glo); f.ghi = std::max(f.ghi, o.ghi);
    f.dmin = std::min(f.dmin, o.dmin); f.dmax = std::max(f.dmax, o.dmax);
    f.dsum += o.dsum; f.osum += o.osum; f.omax = std::max(f.omax, o.omax);
    f.nsum += o.nsum; f.nsq += o.nsq; f.degmax = std::max(f.degmax, o.degmax); f.degsum += o.degsum;
    f.dommin = std::min(f.dommin, o.dommin); f.domsum += o.domsum;
  }
  const double s = f.ghi > 0 ? f.ghi : 1.0, nn = n;
  const double nmean = f.nsum / nn, nstd = std::sqrt(std::max(0.0, f.nsq / nn - nmean * nmean));
  const double fv[MPKG_NFEAT] = {f.glo / s,           f.dsum / nn / s,    f.dmin / s,          f.dmax / s,
                                 f.osum / nn / s,     f.omax / s,         nmean / s,           nstd / s,
                                 f.degsum / nn / 32., f.degmax / 32.,     std::min(f.dommin, 10.0) / 10.,
                                 f.domsum / nn / 10.};
  for (int k = 0; k < MPKG_NFEAT; k++) feat[k] = (float)fv[k];
  if (glo) *glo = f.glo;
  if (ghi) *ghi = f.ghi;
  return kOk;
}

int mpkg_lanczos(int n, const int *ptr, const int *col, const double *val, int m, uint64_t seed, double *ritz,
                 double *alpha_out, double *beta_out) {
  clear_error();
  if (!val || !ritz || m <= 0 || m > 256 || m > n) return fail(kEInval, "bad argument");
  DevCsr a;
  int rc = a.upload(n, ptr, col, val, false);
  if (rc) return rc;
  const int nb = blocks_for(n);
  DevBuf<double> v0, v1, w, part;
  if ((rc = v0.alloc(n)) || (rc = v1.alloc(n)) || (rc = w.alloc(n)) || (rc = part.alloc(nb))) return rc;
  std::vector<double> h(n);
  uniform_vector(seed, n, h.data());
  double nrm = 0.0;
  for (double t : h) nrm += t * t;
  nrm = std::sqrt(nrm);
  for (double &t : h) t /= nrm;
  SS_TRY(cudaMemcpy(v1.p, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  SS_TRY(cudaMemset(v0.p, 0, sizeof(double) * n));
  std::vector<double> alpha(m), beta(m);
  double bprev = 0.0;
  double *vp = v0.p, *vc = v1.p;
  int steps = 0;
  for (int j = 0; j < m; j++) {
    // w = A v_j - beta_j v_(j-1);  alpha_j = w . v_j
    spmv64_kernel<<<nb, kThreads>>>(n, a.sell(), vc, w.p, j ? vp : nullptr, bprev, part.p);
    SS_TRY(cudaGetLastError());
    double al;
    if ((rc = sum_parts(part.p, nb, &al))) return rc;
    alpha[j] = al;
    steps = j + 1;
    if (j + 1 == m) break;
    // w -= alpha_j v_j;  beta_(j+1) = |w|
    axpy_norm_kernel<<<nb, kThreads>>>(n, -al, vc, w.p, part.p);
    double b2;
    if ((rc = sum_parts(part.p, nb, &b2))) return rc;
    const double bt = std::sqrt(b2);
    beta[j] = bt;
    if (!(bt > 1e-300)) break;  // invariant subspace
    // v_(j-1) <- w / beta (becomes v_(j+1))
    axpby_kernel<<<nb, kThreads>>>(n, 1.0 / bt, w.p, 0.0, vp);
    std::swap(vp, vc);
    bprev = bt;
  }
  SS_TRY(cudaDeviceSynchronize());
  std::vector<double> ev(steps);
  tridiag_eigs(steps, alpha.data(), beta.data(), ev.data());
  for (int k = 0; k < m; k++) ritz[k] = k < steps ? ev[k] : ev[steps - 1];
  if (alpha_out) std::copy(alpha.begin(), alpha.begin() + steps, alpha_out);
  if (beta_out) std::copy(beta.begin(), beta.begin() + std::max(0, steps - 1), beta_out);
  return steps == m ? kOk : kOk;
}

int mpkg_cg(int n, const int *ptr, const int *col, const double *val, const double *b, double *x, double tol,
            int max_iter, mpkg_cg_info_t *info) {
  clear_error();
  if (!val || !b || !x || max_iter <= 0) return fail(kEInval, "bad argument");
  auto t0 = std::chrono::steady_clock::now();
  DevCsr a;
  int rc = a.upload(n, ptr, col, val, false);
  if (rc) return rc;
  const int nb = blocks_for(n);
  DevBuf<double> dx, db, dr, dp, dq, part;
  if ((rc = dx.alloc(n)) || (rc = db.alloc(n)) || (rc = dr.alloc(n)) || (rc = dp.alloc(n)) || (rc = dq.alloc(n)) ||
      (rc = part.alloc(nb)))
    return rc;
  SS_TRY(cudaMemcpy(dx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice));
  SS_TRY(cudaMemcpy(db.p, b, sizeof(double) * n, cudaMemcpyHostToDevice));
  double bb = 0.0;
  for (int i = 0; i < n; i++) bb += b[i] * b[i];
  const double bnorm = std::sqrt(bb);
  resid_kernel<<<nb, kThreads>>>(n, a.sell(), dx.p, db.p, dr.p, part.p);
  double rr;
  if ((rc = sum_parts(part.p, nb, &rr))) return rc;
  SS_TRY(cudaMemcpy(dp.p, dr.p, sizeof(double) * n, cudaMemcpyDeviceToDevice));
  int it = 0;
  const auto t_loop = std::chrono::steady_clock::now();
  while (it < max_iter && std::sqrt(rr) > tol * bnorm) {
    spmv64_kernel<<<nb, kThreads>>>(n, a.sell(), dp.p, dq.p, nullptr, 0.0, part.p);
    double pq;
    if ((rc = sum_parts(part.p, nb, &pq))) return rc;
    if (!(pq > 0.0)) break;
    const double alpha = rr / pq;
    axpby_kernel<<<nb, kThreads>>>(n, alpha, dp.p, 1.0, dx.p);
    axpy_norm_kernel<<<nb, kThreads>>>(n, -alpha, dq.p, dr.p, part.p);
    double rr2;
    if ((rc = sum_parts(part.p, nb, &rr2))) return rc;
    axpby_kernel<<<nb, kThreads>>>(n, 1.0, dr.p, rr2 / rr, dp.p);
    rr = rr2;
    it++;
  }
  const auto t_loop_end = std::chrono::steady_clock::now();
  // true residual
  resid_kernel<<<nb, kThreads>>>(n, a.sell(), dx.p, db.p, dr.p, part.p);
  double rt;
  if ((rc = sum_parts(part.p, nb, &rt))) return rc;
  SS_TRY(cudaMemcpy(x, dx.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (info) {
    std::memset(info, 0, sizeof *info);
    info->iterations = it;
    info->mpk_steps = it;
    info->relres = std::sqrt(rt) / bnorm;
    info->converged = info->relres <= tol;
    info->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    info->loop_ms = std::chrono::duration<double, std::milli>(t_loop_end - t_loop).count();
  }
  return kOk;
}

int mpkg_sstep_gram(int mode) {
  clear_error();
  if (mode != MPKG_GRAM_FP64 && mode != MPKG_GRAM_DF64) return fail(kEInval, "unknown Gram mode");
  g_gram_f64 = mode == MPKG_GRAM_FP64;
  return kOk;
}

int mpkg_sstep_basis(int mode) {
  if (mode != MPKG_SSTEP_BASIS_MPK && mode != MPKG_SSTEP_BASIS_STEPS) return fail(kEInval, "unknown basis mode");
  g_basis_mpk = mode == MPKG_SSTEP_BASIS_MPK;
  return kOk;
}

int mpkg_sstep_debug_stall(int extra_levels) {
  if (extra_levels < 0 || extra_levels > 1000) return fail(kEInval, "0 <= extra_levels <= 1000");
  g_basis_stall = (unsigned)extra_levels;
  return kOk;
}

int mpkg_sstep_loop(int mode) {
  clear_error();
  if (mode != MPKG_SSTEP_DEVICE_LOOP && mode != MPKG_SSTEP_HOST_LOOP) return fail(kEInval, "unknown loop mode");
  g_device_loop = mode == MPKG_SSTEP_DEVICE_LOOP;
  return kOk;
}

int mpkg_sstep_cg(int n, const int *ptr, const int *col, const double *val, const double *b, double *x, int s,
                  const double *shifts, double scale, double tol, int max_outer, mpkg_cg_info_t *info) {
  clear_error();
  if (!val || !b || !x || s < 1 || s > kMaxS || max_outer <= 0 || !(scale > 0.0))
    return fail(kEInval, "bad argument");
  auto t0 = std::chrono::steady_clock::now();
  DevCsr a;
  int rc = a.upload(n, ptr, col, val, true);
  if (rc) return rc;
  const int nb = blocks_for(n), m = 2 * s + 1, npair = m * (m + 1) / 2;
  const int gblk = (int)std::min<long>(1216, (n + kGramRows - 1) / kGramRows);
  DevBuf<double> dx, db, dr, dp, part, gpart, dg, dth, dsg, dxh, dph, drh;
  DevBuf<float> y;
  DevBuf<int> dflag;
  HostBuf hbuf;  // page-locked: flags (8 ints), r.r and p.p, the Gram matrix, staged scalars
  const size_t hb_sc = 8 * sizeof(int), hb_g = hb_sc + 2 * sizeof(double), hb_up = hb_g + sizeof(double) * m * m;
  if ((rc = hbuf.alloc(hb_up + sizeof(double) * kScalars))) return rc;
  DevBuf<double> dsc;
  if ((rc = dsc.alloc(kScalars))) return rc;
  if ((rc = dx.alloc(n)) || (rc = db.alloc(n)) || (rc = dr.alloc(n)) || (rc = dp.alloc(n)) ||
      (rc = part.alloc(2 * (size_t)nb)) ||
      (rc = gpart.alloc((size_t)gblk * npair)) || (rc = dg.alloc(m * m)) || (rc = dth.alloc(s)) ||
      (rc = dsg.alloc(s)) || (rc = dxh.alloc(m)) || (rc = dph.alloc(m)) || (rc = drh.alloc(m)) ||
      (rc = y.alloc((size_t)m * n)) || (rc = dflag.alloc(2)))
    return rc;
  std::vector<double> th(s, 0.0), sg(s, scale);
  if (shifts) std::copy(shifts, shifts + s, th.begin());
  SS_TRY(cudaMemcpy(dth.p, th.data(), sizeof(double) * s, cudaMemcpyHostToDevice));
  SS_TRY(cudaMemcpy(dsg.p, sg.data(), sizeof(double) * s, cudaMemcpyHostToDevice));
  SS_TRY(cudaMemcpy(dx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice));
  SS_TRY(cudaMemcpy(db.p, b, sizeof(double) * n, cudaMemcpyHostToDevice));
  double bb = 0.0;
  for (int i = 0; i < n; i++) bb += b[i] * b[i];
  const double bnorm = std::sqrt(bb);
  resid_kernel<<<nb, kThreads>>>(n, a.sell(), dx.p, db.p, dr.p, part.p);
  double rr;
  if ((rc = sum_parts(part.p, nb, &rr))) return rc;
  SS_TRY(cudaMemcpy(dp.p, dr.p, sizeof(double) * n, cudaMemcpyDeviceToDevice));
  double pp = rr;
  GraphRun gr;
  SS_TRY(cudaStreamCreateWithFlags(&gr.st, cudaStreamNonBlocking));
  auto upload_scalars = [&]() -> int {  // host values of the norms, e.g. after a restart
    double *h = reinterpret_cast<double *>(reinterpret_cast<char *>(hbuf.p) + hb_up);
    const double pn = std::sqrt(pp), rn = std::sqrt(rr);
    h[0] = pn; h[1] = rn; h[2] = 1.0 / pn; h[3] = 1.0 / rn; h[4] = rr; h[5] = pp;
    SS_TRY(cudaMemcpyAsync(dsc.p, h, sizeof(double) * kScalars, cudaMemcpyHostToDevice, gr.st));
    return kOk;
  };
  if ((rc = upload_scalars())) return rc;
  // the basis as one matrix powers launch (default) or s SpMV launches
  const bool basis_mpk = g_basis_mpk;
  BasisLayout bl;
  if (basis_mpk) {
    if ((rc = bl.build(n, ptr, col, a.soff_h, s, th, sg))) return rc;
    bl.probe(a.sell(), y.p);
  }
  // one outer iteration: basis, Gram, coefficient steps, update, true
  // residual, scalars for the next iteration
  auto iteration = [&](cudaStream_t cs) {
    float *Y = y.p;
    basis_start_kernel<<<nb, kThreads, 0, cs>>>(n, dp.p, dr.p, dsc.p, Y, Y + (size_t)(s + 1) * n);
    if (basis_mpk) {
      bl.launch(a.sell(), Y, cs);
    } else for (int j = 0; j < s; j++) {
      const bool rstep = j + 1 < s;
      basis_step_kernel<<<nb, kThreads, 0, cs>>>(n, a.sell(), Y + (size_t)j * n, Y + (size_t)(j + 1) * n,
                                                 rstep ? Y + (size_t)(s + 1 + j) * n : nullptr,
                                                 rstep ? Y + (size_t)(s + 2 + j) * n : nullptr, (float)th[j],
                                                 (float)(1.0 / sg[j]));
    }
    if (g_gram_f64) gram_kernel<true><<<gblk, kThreads, 0, cs>>>(n, m, Y, gpart.p);
    else gram_kernel<false><<<gblk, kThreads, 0, cs>>>(n, m, Y, gpart.p);
    gram_reduce_kernel<<<(npair * 32 + kThreads - 1) / kThreads, kThreads, 0, cs>>>(gblk, m, gpart.p, dg.p);
    coeff_kernel<<<1, 32, 0, cs>>>(s, dg.p, dth.p, dsg.p, dsc.p, dxh.p, dph.p, drh.p, dflag.p);
    combine_kernel<<<nb, kThreads, 0, cs>>>(n, m, Y, dxh.p, dph.p, dx.p, dp.p, part.p + nb);
    resid_kernel<<<nb, kThreads, 0, cs>>>(n, a.sell(), dx.p, db.p, dr.p, part.p);
    norms_kernel<<<1, 32, 0, cs>>>(nb, part.p, dsc.p);
  };
  int outer = 0, steps = 0, breakdowns = 0;
  double cond_max = 0.0;
  // condition number of the P block (the s-step polynomial basis, (s+1)^2
  // row-major) from its Gram eigenvalues, computed on the host while the
  // GPU runs the following iterations
  auto basis_cond = [&](const double *blk) {
    const int m = s + 1;  // Jacobi sweeps on the leading (s+1) x (s+1) block
    std::vector<double> A(blk, blk + (size_t)m * m);
    for (int sweep = 0; sweep < 60; sweep++) {
      double off = 0.0;
      for (int p2 = 0; p2 < m; p2++)
        for (int q2 = p2 + 1; q2 < m; q2++) off += A[p2 * m + q2] * A[p2 * m + q2];
      if (off < 1e-30) break;
      for (int p2 = 0; p2 < m; p2++)
        for (int q2 = p2 + 1; q2 < m; q2++) {
          const double apq = A[p2 * m + q2];
          if (std::fabs(apq) < 1e-300) continue;
          const double tau = (A[q2 * m + q2] - A[p2 * m + p2]) / (2.0 * apq);
          const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
          const double c = 1.0 / std::sqrt(1.0 + t * t), sn = t * c;
          for (int k = 0; k < m; k++) {
            const double akp = A[k * m + p2], akq = A[k * m + q2];
            A[k * m + p2] = c * akp - sn * akq;
            A[k * m + q2] = sn * akp + c * akq;
          }
          for (int k = 0; k < m; k++) {
            const double apk = A[p2 * m + k], aqk = A[q2 * m + k];
            A[p2 * m + k] = c * apk - sn * aqk;
            A[q2 * m + k] = sn * apk + c * aqk;
          }
        }
    }
    double emin = 1e300, emax = 0.0;
    for (int k = 0; k < m; k++) {
      emin = std::min(emin, A[k * m + k]);
      emax = std::max(emax, A[k * m + k]);
    }
    const double cnd = emin > 0 ? std::sqrt(emax / emin) : 1e300;
    cond_max = std::max(cond_max, cnd);
  };
  const int mp2 = (s + 1) * (s + 1);
  const double rtol = tol * bnorm;
  int launches = 0;
  auto t_loop = std::chrono::steady_clock::now(), t_loop_end = t_loop;
  // Device-side loop (a conditional WHILE node), when the runtime offers it
  DevBuf<int> dstate;
  LoopHost lh;
  bool device_loop = g_device_loop && lh.alloc((size_t)kCondRing * mp2);
  if (device_loop && (rc = dstate.alloc(sizeof(LoopState) / sizeof(int)))) return rc;
  if (device_loop) {
    SS_TRY(cudaMemsetAsync(dstate.p, 0, sizeof(LoopState), gr.st));
    device_loop = build_device_loop(gr, [&](cudaStream_t cs, cudaGraphConditionalHandle h) {
      restart_kernel<<<nb, kThreads, 0, cs>>>(n, reinterpret_cast<const LoopState *>(dstate.p), dr.p, dp.p, dsc.p);
      iteration(cs);
      decide_kernel<<<1, 32, 0, cs>>>(s, m, dflag.p, dsc.p, dg.p, max_outer, rtol,
                                       reinterpret_cast<LoopState *>(dstate.p), lh.d_ring, lh.d_progress, h);
    });
  }
  if (device_loop) {
    if (std::sqrt(rr) > rtol) {
      t_loop = std::chrono::steady_clock::now();
      SS_TRY(cudaGraphLaunch(gr.exec, gr.st));
      launches = 1;
      int seen = 0;
      std::vector<double> blk(mp2);
      for (;;) {  // condition numbers of the iterations done so far, while the loop runs
        const cudaError_t q = cudaStreamQuery(gr.st);
        const int avail = __atomic_load_n(lh.progress, __ATOMIC_ACQUIRE);
        for (; seen < avail; seen++) {
          if (avail - seen > kCondRing) continue;  // overwritten before it was read
          std::memcpy(blk.data(), lh.ring + (size_t)(seen % kCondRing) * mp2, sizeof(double) * mp2);
          // the slot is rewritten by iteration seen + kCondRing: use the copy
          // only if that iteration had not reached its decision yet
          const int now = __atomic_load_n(lh.progress, __ATOMIC_ACQUIRE);
          if (info && now - seen < kCondRing) basis_cond(blk.data());
        }
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) SS_TRY(q);
        std::this_thread::yield();
      }
      LoopState hs;
      double sc[kScalars];
      SS_TRY(cudaMemcpy(&hs, dstate.p, sizeof hs, cudaMemcpyDeviceToHost));
      SS_TRY(cudaMemcpy(sc, dsc.p, sizeof sc, cudaMemcpyDeviceToHost));
      outer = hs.outer;
      steps = hs.steps;
      breakdowns = hs.breakdowns;
      rr = sc[4];
      t_loop_end = std::chrono::steady_clock::now();
    }
  } else {
    // host loop: the iteration as a graph replayed per outer iteration,
    // with one copy back of the flags, r.r, p.p and the Gram matrix
    cudaStream_t cs = gr.st;
    SS_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    iteration(cs);
    cudaMemcpyAsync(hbuf.p, dflag.p, sizeof(int) * 2, cudaMemcpyDeviceToHost, cs);
    cudaMemcpyAsync(reinterpret_cast<char *>(hbuf.p) + hb_sc, dsc.p + 4, sizeof(double) * 2, cudaMemcpyDeviceToHost,
                    cs);
    cudaMemcpyAsync(reinterpret_cast<char *>(hbuf.p) + hb_g, dg.p, sizeof(double) * m * m, cudaMemcpyDeviceToHost, cs);
    SS_TRY(cudaStreamEndCapture(cs, &gr.graph));
    SS_TRY(cudaGraphInstantiate(&gr.exec, gr.graph, 0));
    std::vector<double> blk(mp2);
    bool cond_pending = false;
    t_loop = std::chrono::steady_clock::now();
    while (outer < max_outer && std::sqrt(rr) > rtol) {
      SS_TRY(cudaGraphLaunch(gr.exec, gr.st));
      launches++;
      if (cond_pending && info) basis_cond(blk.data());
      cond_pending = false;
      SS_TRY(cudaStreamSynchronize(gr.st));
      int flag[2];
      std::memcpy(flag, hbuf.p, sizeof flag);
      const double *hs = reinterpret_cast<const double *>(reinterpret_cast<char *>(hbuf.p) + hb_sc);
      rr = hs[0];
      pp = hs[1];
      const double *hg = reinterpret_cast<const double *>(reinterpret_cast<char *>(hbuf.p) + hb_g);
      for (int k = 0; k < mp2; k++) blk[k] = hg[(k / (s + 1)) * m + k % (s + 1)];
      cond_pending = true;
      breakdowns += flag[0];
      steps += flag[1];
      outer++;
      if (flag[1] == 0 || !(pp > 0.0)) {  // no progress possible with this basis: restart from r
        SS_TRY(cudaMemcpyAsync(dp.p, dr.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, gr.st));
        pp = rr;
        if ((rc = upload_scalars())) return rc;
        if (flag[1] == 0) break;
      }
    }
    if (cond_pending && info) basis_cond(blk.data());
    SS_TRY(cudaStreamSynchronize(gr.st));
    t_loop_end = std::chrono::steady_clock::now();
  }
  SS_TRY(cudaStreamSynchronize(gr.st));
  SS_TRY(cudaMemcpy(x, dx.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (basis_mpk) {
    int werr = 0;
    SS_TRY(cudaMemcpy(&werr, bl.err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (werr) return fail(kETimeout, "s-step basis: a device-side wait exceeded its spin limit");
  }
  if (info) {
    std::memset(info, 0, sizeof *info);
    info->loop_ms = std::chrono::duration<double, std::milli>(t_loop_end - t_loop).count();
    info->loop_launches = launches;
    info->iterations = outer;
    info->mpk_steps = steps;
    info->relres = std::sqrt(rr) / bnorm;
    info->converged = info->relres <= tol;
    info->basis_cond = cond_max;
    info->breakdowns = breakdowns;
    info->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return kOk;
}

}  // extern "C"
