// A small multilayer perceptron (nin -> width -> width -> nout, ReLU
// hidden layers, linear output, mean squared error) trained and evaluated
// on the GPU by the kernels in this file: forward pass, per-sample
// back-propagation, deterministic weight-gradient reduction, Adam.  FP32.
// It maps cheap matrix features to Newton-basis shifts for s-step CG (no
// counterpart in the reference).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/mpk_gb300.h"
#include "host.h"

using namespace mpkg;

#define ML_TRY(expr)                                                             \
  do {                                                                           \
    cudaError_t e_ = (expr);                                                     \
    if (e_ != cudaSuccess) return fail(kECuda, std::string(#expr ": ") + cudaGetErrorString(e_)); \
  } while (0)

namespace {

constexpr int kMaxWidth = 256;

struct Dims {
  int nin, w, nout;
  // offsets of W1, b1, W2, b2, W3, b3 in the flat parameter vector
  __host__ __device__ int oW1() const { return 0; }
  __host__ __device__ int ob1() const { return w * nin; }
  __host__ __device__ int oW2() const { return ob1() + w; }
  __host__ __device__ int ob2() const { return oW2() + w * w; }
  __host__ __device__ int oW3() const { return ob2() + w; }
  __host__ __device__ int ob3() const { return oW3() + nout * w; }
  __host__ __device__ int total() const { return ob3() + nout; }
};

// One CTA per sample, one thread per hidden unit.  Stores the activations
// for the backward pass when h1/h2 are given.
__global__ void mlp_forward_kernel(Dims d, const float *__restrict__ prm, const float *__restrict__ X,
                                   const int *__restrict__ idx, float *__restrict__ h1, float *__restrict__ h2,
                                   float *__restrict__ Y) {
  __shared__ float xs[kMaxWidth], a1[kMaxWidth], a2[kMaxWidth];
  const int b = blockIdx.x, j = threadIdx.x;
  const int src = idx ? idx[b] : b;
  for (int f = j; f < d.nin; f += blockDim.x) xs[f] = X[(size_t)src * d.nin + f];
  __syncthreads();
  if (j < d.w) {
    float s = prm[d.ob1() + j];
    for (int f = 0; f < d.nin; f++) s = __fmaf_rn(prm[d.oW1() + j * d.nin + f], xs[f], s);
    a1[j] = fmaxf(s, 0.f);
    if (h1) h1[(size_t)b * d.w + j] = a1[j];
  }
  __syncthreads();
  if (j < d.w) {
    float s = prm[d.ob2() + j];
    for (int k = 0; k < d.w; k++) s = __fmaf_rn(prm[d.oW2() + j * d.w + k], a1[k], s);
    a2[j] = fmaxf(s, 0.f);
    if (h2) h2[(size_t)b * d.w + j] = a2[j];
  }
  __syncthreads();
  if (j < d.nout) {
    float s = prm[d.ob3() + j];
    for (int k = 0; k < d.w; k++) s = __fmaf_rn(prm[d.oW3() + j * d.w + k], a2[k], s);
    Y[(size_t)b * d.nout + j] = s;
  }
}

// Per-sample deltas of the mean squared error over nb samples x nout.
__global__ void mlp_delta_kernel(Dims d, int nb, const float *__restrict__ prm, const float *__restrict__ T,
                                 const int *__restrict__ idx, const float *__restrict__ h1,
                                 const float *__restrict__ h2, const float *__restrict__ Y, float *__restrict__ dy,
                                 float *__restrict__ dh1, float *__restrict__ dh2) {
  __shared__ float sdy[kMaxWidth], sd2[kMaxWidth];
  const int b = blockIdx.x, j = threadIdx.x;
  const int src = idx ? idx[b] : b;
  const float scale = 2.0f / (float)(nb * d.nout);
  if (j < d.nout) {
    const float e = (Y[(size_t)b * d.nout + j] - T[(size_t)src * d.nout + j]) * scale;
    sdy[j] = e;
    dy[(size_t)b * d.nout + j] = e;
  }
  __syncthreads();
  if (j < d.w) {
    float s = 0.f;
    for (int o = 0; o < d.nout; o++) s = __fmaf_rn(prm[d.oW3() + o * d.w + j], sdy[o], s);
    const float v = h2[(size_t)b * d.w + j] > 0.f ? s : 0.f;
    sd2[j] = v;
    dh2[(size_t)b * d.w + j] = v;
  }
  __syncthreads();
  if (j < d.w) {
    float s = 0.f;
    for (int k = 0; k < d.w; k++) s = __fmaf_rn(prm[d.oW2() + k * d.w + j], sd2[k], s);
    dh1[(size_t)b * d.w + j] = h1[(size_t)b * d.w + j] > 0.f ? s : 0.f;
  }
}

// Thread per parameter: sum over the samples in order (deterministic).
__global__ void mlp_grad_kernel(Dims d, int nb, const float *__restrict__ X, const int *__restrict__ idx,
                                const float *__restrict__ h1, const float *__restrict__ h2,
                                const float *__restrict__ dy, const float *__restrict__ dh1,
                                const float *__restrict__ dh2, float *__restrict__ g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.total()) return;
  float s = 0.f;
  if (t < d.ob1()) {
    const int j = t / d.nin, f = t % d.nin;
    for (int b = 0; b < nb; b++) s = __fmaf_rn(dh1[(size_t)b * d.w + j], X[(size_t)(idx ? idx[b] : b) * d.nin + f], s);
  } else if (t < d.oW2()) {
    const int j = t - d.ob1();
    for (int b = 0; b < nb; b++) s += dh1[(size_t)b * d.w + j];
  } else if (t < d.ob2()) {
    const int u = t - d.oW2(), j = u / d.w, k = u % d.w;
    for (int b = 0; b < nb; b++) s = __fmaf_rn(dh2[(size_t)b * d.w + j], h1[(size_t)b * d.w + k], s);
  } else if (t < d.oW3()) {
    const int j = t - d.ob2();
    for (int b = 0; b < nb; b++) s += dh2[(size_t)b * d.w + j];
  } else if (t < d.ob3()) {
    const int u = t - d.oW3(), o = u / d.w, k = u % d.w;
    for (int b = 0; b < nb; b++) s = __fmaf_rn(dy[(size_t)b * d.nout + o], h2[(size_t)b * d.w + k], s);
  } else {
    const int o = t - d.ob3();
    for (int b = 0; b < nb; b++) s += dy[(size_t)b * d.nout + o];
  }
  g[t] = s;
}

// Mean squared error of a batch (one CTA, fixed-order tree).
__global__ void mlp_loss_kernel(Dims d, int nb, const float *__restrict__ T, const int *__restrict__ idx,
                                const float *__restrict__ Y, float *__restrict__ loss) {
  __shared__ float red[256];
  float s = 0.f;
  for (int e = threadIdx.x; e < nb * d.nout; e += blockDim.x) {
    const int b = e / d.nout, o = e % d.nout;
    const float r = Y[e] - T[(size_t)(idx ? idx[b] : b) * d.nout + o];
    s = __fmaf_rn(r, r, s);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = red[0] / (float)(nb * d.nout);
}

__global__ void adam_kernel(int np, float *__restrict__ prm, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const float gt = g[t];
  const float mt = b1 * m[t] + (1.f - b1) * gt;
  const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
  m[t] = mt;
  v[t] = vt;
  prm[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}

}  // namespace

struct mpkg_mlp {
  Dims d{};
  float *prm = nullptr, *grad = nullptr, *am = nullptr, *av = nullptr;
  long step = 0;
  ~mpkg_mlp() {
    cudaFree(prm); cudaFree(grad); cudaFree(am); cudaFree(av);
  }
};

namespace {

struct Scratch {
  float *X = nullptr, *T = nullptr, *h1 = nullptr, *h2 = nullptr, *Y = nullptr, *dy = nullptr, *dh1 = nullptr,
        *dh2 = nullptr, *loss = nullptr;
  int *idx = nullptr;
  ~Scratch() {
    cudaFree(X); cudaFree(T); cudaFree(h1); cudaFree(h2); cudaFree(Y); cudaFree(dy); cudaFree(dh1); cudaFree(dh2);
    cudaFree(loss); cudaFree(idx);
  }
  int alloc(const Dims &d, int ns, int nb, const float *hX, const float *hT) {
    ML_TRY(cudaMalloc(&X, sizeof(float) * (size_t)ns * d.nin));
    ML_TRY(cudaMemcpy(X, hX, sizeof(float) * (size_t)ns * d.nin, cudaMemcpyHostToDevice));
    if (hT) {
      ML_TRY(cudaMalloc(&T, sizeof(float) * (size_t)ns * d.nout));
      ML_TRY(cudaMemcpy(T, hT, sizeof(float) * (size_t)ns * d.nout, cudaMemcpyHostToDevice));
    }
    ML_TRY(cudaMalloc(&h1, sizeof(float) * (size_t)nb * d.w));
    ML_TRY(cudaMalloc(&h2, sizeof(float) * (size_t)nb * d.w));
    ML_TRY(cudaMalloc(&Y, sizeof(float) * (size_t)nb * d.nout));
    ML_TRY(cudaMalloc(&dy, sizeof(float) * (size_t)nb * d.nout));
    ML_TRY(cudaMalloc(&dh1, sizeof(float) * (size_t)nb * d.w));
    ML_TRY(cudaMalloc(&dh2, sizeof(float) * (size_t)nb * d.w));
    ML_TRY(cudaMalloc(&loss, sizeof(float)));
    ML_TRY(cudaMalloc(&idx, sizeof(int) * (size_t)std::max(nb, 1)));
    return kOk;
  }
};

int threads_for(const Dims &d) { return std::max(32, ((std::max(d.w, std::max(d.nin, d.nout)) + 31) / 32) * 32); }

// forward + deltas + gradient of one batch (indices already on the device)
int batch_gradient(mpkg_mlp *m, Scratch &s, int nb, const int *didx) {
  const Dims &d = m->d;
  const int th = threads_for(d);
  mlp_forward_kernel<<<nb, th>>>(d, m->prm, s.X, didx, s.h1, s.h2, s.Y);
  mlp_delta_kernel<<<nb, th>>>(d, nb, m->prm, s.T, didx, s.h1, s.h2, s.Y, s.dy, s.dh1, s.dh2);
  mlp_grad_kernel<<<(d.total() + 255) / 256, 256>>>(d, nb, s.X, didx, s.h1, s.h2, s.dy, s.dh1, s.dh2, m->grad);
  mlp_loss_kernel<<<1, 256>>>(d, nb, s.T, didx, s.Y, s.loss);
  ML_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace

extern "C" {

int mpkg_mlp_create(int nin, int width, int nout, uint64_t seed, mpkg_mlp **out) {
  clear_error();
  if (!out || nin <= 0 || nout <= 0 || width <= 0 || nin > kMaxWidth || width > kMaxWidth || nout > kMaxWidth)
    return fail(kEInval, "bad MLP dimensions");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(kECuda, "no CUDA device");
  mpkg_mlp *m = new (std::nothrow) mpkg_mlp();
  if (!m) return fail(kENoMem, "allocation failed");
  m->d = Dims{nin, width, nout};
  const int np = m->d.total();
  // He-uniform initial weights (seeded), zero biases
  std::vector<double> u(np);
  uniform_vector(seed, np, u.data());
  std::vector<float> p(np, 0.f);
  auto fill = [&](int off, int count, int fan_in) {
    const double a = std::sqrt(6.0 / fan_in);
    for (int k = 0; k < count; k++) p[off + k] = (float)(a * u[off + k]);
  };
  fill(m->d.oW1(), width * nin, nin);
  fill(m->d.oW2(), width * width, width);
  fill(m->d.oW3(), nout * width, width);
  int rc = kOk;
  if (cudaMalloc(&m->prm, sizeof(float) * np) != cudaSuccess || cudaMalloc(&m->grad, sizeof(float) * np) != cudaSuccess ||
      cudaMalloc(&m->am, sizeof(float) * np) != cudaSuccess || cudaMalloc(&m->av, sizeof(float) * np) != cudaSuccess)
    rc = fail(kENoMem, "device allocation failed");
  if (!rc && (cudaMemcpy(m->prm, p.data(), sizeof(float) * np, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemset(m->am, 0, sizeof(float) * np) != cudaSuccess ||
              cudaMemset(m->av, 0, sizeof(float) * np) != cudaSuccess))
    rc = fail(kECuda, "upload failed");
  if (rc) { delete m; return rc; }
  *out = m;
  return kOk;
}

void mpkg_mlp_destroy(mpkg_mlp *m) { delete m; }

int mpkg_mlp_nparams(const mpkg_mlp *m) { return m ? m->d.total() : 0; }

int mpkg_mlp_get_params(const mpkg_mlp *m, float *params) {
  if (!m || !params) return fail(kEInval, "null argument");
  ML_TRY(cudaMemcpy(params, m->prm, sizeof(float) * m->d.total(), cudaMemcpyDeviceToHost));
  return kOk;
}

int mpkg_mlp_set_params(mpkg_mlp *m, const float *params) {
  if (!m || !params) return fail(kEInval, "null argument");
  ML_TRY(cudaMemcpy(m->prm, params, sizeof(float) * m->d.total(), cudaMemcpyHostToDevice));
  return kOk;
}

int mpkg_mlp_forward(mpkg_mlp *m, int ns, const float *X, float *Y) {
  clear_error();
  if (!m || ns <= 0 || !X || !Y) return fail(kEInval, "bad argument");
  Scratch s;
  int rc = s.alloc(m->d, ns, ns, X, nullptr);
  if (rc) return rc;
  mlp_forward_kernel<<<ns, threads_for(m->d)>>>(m->d, m->prm, s.X, nullptr, nullptr, nullptr, s.Y);
  ML_TRY(cudaGetLastError());
  ML_TRY(cudaMemcpy(Y, s.Y, sizeof(float) * (size_t)ns * m->d.nout, cudaMemcpyDeviceToHost));
  return kOk;
}

int mpkg_mlp_gradient(mpkg_mlp *m, int ns, const float *X, const float *T, float *grad, float *loss) {
  clear_error();
  if (!m || ns <= 0 || !X || !T || !grad) return fail(kEInval, "bad argument");
  Scratch s;
  int rc = s.alloc(m->d, ns, ns, X, T);
  if (rc) return rc;
  if ((rc = batch_gradient(m, s, ns, nullptr))) return rc;
  ML_TRY(cudaMemcpy(grad, m->grad, sizeof(float) * m->d.total(), cudaMemcpyDeviceToHost));
  if (loss) ML_TRY(cudaMemcpy(loss, s.loss, sizeof(float), cudaMemcpyDeviceToHost));
  return kOk;
}

int mpkg_mlp_train(mpkg_mlp *m, int ns, const float *X, const float *T, int epochs, int batch, float lr,
                   uint64_t seed, float *loss_curve) {
  clear_error();
  if (!m || ns <= 0 || !X || !T || epochs <= 0 || batch <= 0 || !(lr > 0.f)) return fail(kEInval, "bad argument");
  batch = std::min(batch, ns);
  Scratch s;
  int rc = s.alloc(m->d, ns, batch, X, T);
  if (rc) return rc;
  const int np = m->d.total();
  std::vector<int> order(ns);
  for (int i = 0; i < ns; i++) order[i] = i;
  uint64_t st = seed;
  auto rnd = [&st]() {
    st += 0x9E3779B97F4A7C15ULL;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  };
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ep++) {
    for (int i = ns - 1; i > 0; i--) std::swap(order[i], order[(int)(rnd() % (uint64_t)(i + 1))]);
    double lsum = 0.0;
    int nbt = 0;
    for (int b0 = 0; b0 + batch <= ns; b0 += batch) {
      ML_TRY(cudaMemcpy(s.idx, order.data() + b0, sizeof(int) * batch, cudaMemcpyHostToDevice));
      if ((rc = batch_gradient(m, s, batch, s.idx))) return rc;
      m->step++;
      const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
      adam_kernel<<<(np + 255) / 256, 256>>>(np, m->prm, m->grad, m->am, m->av, lr, b1, b2, eps, c1, c2);
      float l = 0.f;
      ML_TRY(cudaMemcpy(&l, s.loss, sizeof(float), cudaMemcpyDeviceToHost));
      lsum += l;
      nbt++;
    }
    if (loss_curve) loss_curve[ep] = (float)(lsum / std::max(nbt, 1));
  }
  ML_TRY(cudaGetLastError());
  return kOk;
}

}  // extern "C"
