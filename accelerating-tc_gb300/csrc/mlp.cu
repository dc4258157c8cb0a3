// Learned (direction, ordering, kernel) selection: a small FP32 MLP trained and run on
// the GPU by the kernels below, and the cheap graph statistics it reads.
//
// Model: x (6 log-scaled features, standardised with the training set's mean / std) ->
// 64 ReLU -> 64 ReLU -> T outputs, one predicted log-time per triple; the selector picks
// the smallest.  Loss: masked mean squared error against measured log-times (triples
// that were not measured, e.g. A-order where it is undefined, are masked out).
// Training: full-batch or mini-batch Adam.  Every kernel gives one output element to
// one thread and sums in a fixed order, so results are deterministic; tensor cores are
// not used (the layers are 6x64 and 64x64).  The networks are tiny, so the kernels
// are latency-bound by design.
//
// Parameter layout (one float buffer): W1[I][H] b1[H] W2[H][H] b2[H] W3[H][O] b3[O],
// W[i][j] the weight from input i to unit j.
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.cuh"

struct atc_mlp {
  int I = 0, H = 0, O = 0;
  int64_t nparams = 0;
  float* params = nullptr;  // device
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  int64_t step = 0;
  std::vector<float> mean, stdv;  // input standardisation
};

namespace atc {
namespace {

int64_t param_count(int I, int H, int O) { return (int64_t)I * H + H + (int64_t)H * H + H + (int64_t)H * O + O; }

struct Layout {
  float *W1, *b1, *W2, *b2, *W3, *b3;
};

Layout layout(float* p, int I, int H, int O) {
  Layout l;
  l.W1 = p;
  l.b1 = l.W1 + (int64_t)I * H;
  l.W2 = l.b1 + H;
  l.b2 = l.W2 + (int64_t)H * H;
  l.W3 = l.b2 + H;
  l.b3 = l.W3 + (int64_t)H * O;
  return l;
}

// Y[b][o] = act(b[o] + sum_i X[b][i] W[i][o])
__global__ void dense_fwd_kernel(const float* X, const float* W, const float* bias, float* Y, int B, int I, int O,
                                 int relu) {
  int64_t total = (int64_t)B * O;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int b = (int)(t / O), o = (int)(t % O);
    float acc = bias[o];
    for (int i = 0; i < I; ++i) acc += X[(int64_t)b * I + i] * W[(int64_t)i * O + o];
    Y[t] = relu && acc < 0.0f ? 0.0f : acc;
  }
}

// dX[b][i] = (A[b][i] > 0) * sum_o dY[b][o] W[i][o]   (A: the layer input, post-ReLU)
__global__ void dense_bwd_input_kernel(const float* dY, const float* W, const float* A, float* dX, int B, int I, int O) {
  int64_t total = (int64_t)B * I;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int b = (int)(t / I), i = (int)(t % I);
    float acc = 0.0f;
    if (A[t] > 0.0f)
      for (int o = 0; o < O; ++o) acc += dY[(int64_t)b * O + o] * W[(int64_t)i * O + o];
    dX[t] = acc;
  }
}

// dW[i][o] = sum_b X[b][i] dY[b][o];  db[o] = sum_b dY[b][o]  (one thread per weight)
__global__ void dense_bwd_weight_kernel(const float* X, const float* dY, float* dW, float* db, int B, int I, int O) {
  int64_t total = (int64_t)I * O + O;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    float acc = 0.0f;
    if (t < (int64_t)I * O) {
      int i = (int)(t / O), o = (int)(t % O);
      for (int b = 0; b < B; ++b) acc += X[(int64_t)b * I + i] * dY[(int64_t)b * O + o];
      dW[t] = acc;
    } else {
      int o = (int)(t - (int64_t)I * O);
      for (int b = 0; b < B; ++b) acc += dY[(int64_t)b * O + o];
      db[o] = acc;
    }
  }
}

// Masked MSE: loss = sum M (Y - T)^2 / (2 sum M); dY = M (Y - T) / sum M.  One block.
__global__ void mse_kernel(const float* Y, const float* T, const float* M, float* dY, float* loss, int64_t total) {
  __shared__ float s_err[256], s_cnt[256];
  float e = 0.0f, c = 0.0f;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x) {
    float d = Y[t] - T[t];
    e += M[t] * d * d;
    c += M[t];
  }
  s_err[threadIdx.x] = e;
  s_cnt[threadIdx.x] = c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s_err[threadIdx.x] += s_err[threadIdx.x + o];
      s_cnt[threadIdx.x] += s_cnt[threadIdx.x + o];
    }
    __syncthreads();
  }
  float cnt = s_cnt[0] > 0.0f ? s_cnt[0] : 1.0f;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x) dY[t] = M[t] * (Y[t] - T[t]) / cnt;
  if (threadIdx.x == 0) *loss = 0.5f * s_err[0] / cnt;
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    float gt = g[t];
    float mt = b1 * m[t] + (1.0f - b1) * gt;
    float vt = b2 * v[t] + (1.0f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
  }
}

__global__ void standardise_kernel(float* X, const float* mean, const float* inv_std, int B, int I) {
  int64_t total = (int64_t)B * I;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % I);
    X[t] = (X[t] - mean[i]) * inv_std[i];
  }
}

unsigned grid_small(int64_t work) { return (unsigned)std::min<int64_t>((work + 255) / 256, 4096); }

// Activations and gradients of one batch (device).
struct Scratch {
  DevBuf<float> x, a1, a2, y, t, mk, dy, d2, d1, grads, loss, mean, inv;
};

atc_status alloc_scratch(Scratch& s, const atc_mlp* net, int B, cudaStream_t st) {
  ATC_TRY(s.x.alloc((size_t)B * net->I, st));
  ATC_TRY(s.a1.alloc((size_t)B * net->H, st));
  ATC_TRY(s.a2.alloc((size_t)B * net->H, st));
  ATC_TRY(s.y.alloc((size_t)B * net->O, st));
  ATC_TRY(s.t.alloc((size_t)B * net->O, st));
  ATC_TRY(s.mk.alloc((size_t)B * net->O, st));
  ATC_TRY(s.dy.alloc((size_t)B * net->O, st));
  ATC_TRY(s.d2.alloc((size_t)B * net->H, st));
  ATC_TRY(s.d1.alloc((size_t)B * net->H, st));
  ATC_TRY(s.grads.alloc((size_t)net->nparams, st));
  ATC_TRY(s.loss.alloc(1, st));
  ATC_TRY(s.mean.alloc(net->I, st));
  ATC_TRY(s.inv.alloc(net->I, st));
  std::vector<float> inv(net->I);
  for (int i = 0; i < net->I; ++i) inv[i] = net->stdv[i] > 0 ? 1.0f / net->stdv[i] : 1.0f;
  ATC_CK(cudaMemcpyAsync(s.mean.p, net->mean.data(), sizeof(float) * net->I, cudaMemcpyHostToDevice, st));
  ATC_CK(cudaMemcpyAsync(s.inv.p, inv.data(), sizeof(float) * net->I, cudaMemcpyHostToDevice, st));
  ATC_CK(cudaStreamSynchronize(st));  // `inv` is host stack memory
  return ATC_OK;
}

// Forward pass of B rows already in s.x (standardised): fills a1, a2, y.
atc_status forward(const atc_mlp* net, Scratch& s, int B, cudaStream_t st) {
  Layout L = layout(net->params, net->I, net->H, net->O);
  dense_fwd_kernel<<<grid_small((int64_t)B * net->H), 256, 0, st>>>(s.x.p, L.W1, L.b1, s.a1.p, B, net->I, net->H, 1);
  dense_fwd_kernel<<<grid_small((int64_t)B * net->H), 256, 0, st>>>(s.a1.p, L.W2, L.b2, s.a2.p, B, net->H, net->H, 1);
  dense_fwd_kernel<<<grid_small((int64_t)B * net->O), 256, 0, st>>>(s.a2.p, L.W3, L.b3, s.y.p, B, net->H, net->O, 0);
  ATC_CK(cudaGetLastError());
  return ATC_OK;
}

// Loss and parameter gradients of B rows (targets in s.t, mask in s.mk) into s.grads.
atc_status backward(const atc_mlp* net, Scratch& s, int B, cudaStream_t st) {
  const int I = net->I, H = net->H, O = net->O;
  Layout L = layout(net->params, I, H, O);
  Layout G = layout(s.grads.p, I, H, O);
  mse_kernel<<<1, 256, 0, st>>>(s.y.p, s.t.p, s.mk.p, s.dy.p, s.loss.p, (int64_t)B * O);
  dense_bwd_weight_kernel<<<grid_small((int64_t)H * O + O), 256, 0, st>>>(s.a2.p, s.dy.p, G.W3, G.b3, B, H, O);
  dense_bwd_input_kernel<<<grid_small((int64_t)B * H), 256, 0, st>>>(s.dy.p, L.W3, s.a2.p, s.d2.p, B, H, O);
  dense_bwd_weight_kernel<<<grid_small((int64_t)H * H + H), 256, 0, st>>>(s.a1.p, s.d2.p, G.W2, G.b2, B, H, H);
  dense_bwd_input_kernel<<<grid_small((int64_t)B * H), 256, 0, st>>>(s.d2.p, L.W2, s.a1.p, s.d1.p, B, H, H);
  dense_bwd_weight_kernel<<<grid_small((int64_t)I * H + H), 256, 0, st>>>(s.x.p, s.d1.p, G.W1, G.b1, B, I, H);
  ATC_CK(cudaGetLastError());
  return ATC_OK;
}

atc_status load_rows(Scratch& s, const atc_mlp* net, const float* x, const float* t, const float* mk, int B,
                     cudaStream_t st) {
  ATC_CK(cudaMemcpyAsync(s.x.p, x, sizeof(float) * B * net->I, cudaMemcpyHostToDevice, st));
  standardise_kernel<<<grid_small((int64_t)B * net->I), 256, 0, st>>>(s.x.p, s.mean.p, s.inv.p, B, net->I);
  ATC_CK(cudaGetLastError());
  if (t) ATC_CK(cudaMemcpyAsync(s.t.p, t, sizeof(float) * B * net->O, cudaMemcpyHostToDevice, st));
  if (t) {
    if (mk) {
      ATC_CK(cudaMemcpyAsync(s.mk.p, mk, sizeof(float) * B * net->O, cudaMemcpyHostToDevice, st));
    } else {
      std::vector<float> ones((size_t)B * net->O, 1.0f);
      ATC_CK(cudaMemcpyAsync(s.mk.p, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, st));
      ATC_CK(cudaStreamSynchronize(st));
    }
  }
  return ATC_OK;
}

}  // namespace
}  // namespace atc

namespace atc {
namespace {

__global__ void gather_rows_kernel(const float* src, const int32_t* idx, float* dst, int B, int W) {
  int64_t total = (int64_t)B * W;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int b = (int)(t / W), w = (int)(t % W);
    dst[t] = src[(int64_t)idx[b] * W + w];
  }
}

// ---- graph features ------------------------------------------------------------------
__global__ void feat_deg_kernel(const int2* p, uint64_t np, int32_t* deg) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += (uint64_t)gridDim.x * blockDim.x) {
    int2 e = p[i];
    if (e.x == e.y) continue;
    atomicAdd(&deg[e.x], 1);
    atomicAdd(&deg[e.y], 1);
  }
}

// Out-degree under the degree orientation (lower degree first, ties to the larger id:
// the rule costFuncCal's degree cost and A-order use).
__global__ void feat_out_kernel(const int2* p, uint64_t np, const int32_t* deg, int32_t* dout) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += (uint64_t)gridDim.x * blockDim.x) {
    int2 e = p[i];
    if (e.x == e.y) continue;
    bool x_src = deg[e.x] < deg[e.y] || (deg[e.x] == deg[e.y] && e.x > e.y);
    atomicAdd(&dout[x_src ? e.x : e.y], 1);
  }
}

// acc: [0] sum deg, [1] sum deg^2, [2] max deg, [3] edges (non-loop pairs), [4] sum of
// out-degrees above twice the mean, [5] how many such vertices.
__global__ void feat_reduce_kernel(const int32_t* deg, const int32_t* dout, int64_t n, uint64_t m2,
                                   unsigned long long* acc) {
  unsigned long long s = 0, s2 = 0, mx = 0, tail = 0, cnt = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long d = (unsigned long long)deg[v];
    s += d;
    s2 += d * d;
    mx = d > mx ? d : mx;
    unsigned long long o = (unsigned long long)dout[v];
    if (o * (unsigned long long)n > m2) {  // dout - m/n > m/n
      tail += o;
      cnt += 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    tail += __shfl_xor_sync(0xffffffffu, tail, o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&acc[0], s);
    atomicAdd(&acc[1], s2);
    atomicMax(&acc[2], mx);
    atomicAdd(&acc[4], tail);
    atomicAdd(&acc[5], cnt);
  }
}

__global__ void feat_minmax_kernel(const int2* p, uint64_t np, int* mn, int* mx) {
  int lo = INT_MAX, hi = INT_MIN;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += (uint64_t)gridDim.x * blockDim.x) {
    lo = min(lo, min(p[i].x, p[i].y));
    hi = max(hi, max(p[i].x, p[i].y));
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mn, lo);
    atomicMax(mx, hi);
  }
}

__global__ void feat_loops_kernel(const int2* p, uint64_t np, unsigned long long* loops) {
  unsigned long long c = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += (uint64_t)gridDim.x * blockDim.x)
    c += p[i].x == p[i].y;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(loops, c);
}

}  // namespace
}  // namespace atc

using namespace atc;

extern "C" atc_status atc_mlp_create(int32_t n_in, int32_t hidden, int32_t n_out, uint64_t seed, atc_mlp** out) try {
  ATC_CHECK_ARG(out != nullptr && n_in > 0 && hidden > 0 && n_out > 0, "bad MLP shape");
  atc_mlp* net = new atc_mlp();
  net->I = n_in;
  net->H = hidden;
  net->O = n_out;
  net->nparams = param_count(n_in, hidden, n_out);
  net->mean.assign(n_in, 0.0f);
  net->stdv.assign(n_in, 1.0f);
  // He-uniform weights from a counter-based generator, zero biases
  std::vector<float> p(net->nparams, 0.0f);
  Layout L = layout(p.data(), n_in, hidden, n_out);
  uint64_t s0 = mix64(seed);
  auto fill = [&](float* w, int64_t count, int fan_in, uint64_t tag) {
    float lim = std::sqrt(6.0f / (float)fan_in);
    for (int64_t i = 0; i < count; ++i) {
      uint64_t r = mix64(s0 + (tag << 40) + (uint64_t)i * kGolden);
      w[i] = lim * (2.0f * (float)((r >> 40) * (1.0 / 16777216.0)) - 1.0f);
    }
  };
  fill(L.W1, (int64_t)n_in * hidden, n_in, 1);
  fill(L.W2, (int64_t)hidden * hidden, hidden, 2);
  fill(L.W3, (int64_t)hidden * n_out, hidden, 3);
  cudaError_t e1 = cudaMalloc(&net->params, sizeof(float) * net->nparams);
  cudaError_t e2 = cudaMalloc(&net->adam_m, sizeof(float) * net->nparams);
  cudaError_t e3 = cudaMalloc(&net->adam_v, sizeof(float) * net->nparams);
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    cudaFree(net->params);
    cudaFree(net->adam_m);
    cudaFree(net->adam_v);
    delete net;
    set_error("cudaMalloc for the MLP failed");
    return ATC_ERR_OOM;
  }
  ATC_CK(cudaMemcpy(net->params, p.data(), sizeof(float) * net->nparams, cudaMemcpyHostToDevice));
  ATC_CK(cudaMemset(net->adam_m, 0, sizeof(float) * net->nparams));
  ATC_CK(cudaMemset(net->adam_v, 0, sizeof(float) * net->nparams));
  *out = net;
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_mlp_destroy(atc_mlp* net) try {
  if (!net) return ATC_OK;
  cudaFree(net->params);
  cudaFree(net->adam_m);
  cudaFree(net->adam_v);
  delete net;
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_mlp_params(atc_mlp* net, float* get, const float* set, int64_t* count) try {
  ATC_CHECK_ARG(net != nullptr, "NULL MLP");
  if (count) *count = net->nparams;
  if (set) {
    ATC_CK(cudaMemcpy(net->params, set, sizeof(float) * net->nparams, cudaMemcpyHostToDevice));
    ATC_CK(cudaMemset(net->adam_m, 0, sizeof(float) * net->nparams));
    ATC_CK(cudaMemset(net->adam_v, 0, sizeof(float) * net->nparams));
    net->step = 0;
  }
  if (get) ATC_CK(cudaMemcpy(get, net->params, sizeof(float) * net->nparams, cudaMemcpyDeviceToHost));
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_mlp_scaling(atc_mlp* net, float* get_mean, float* get_std, const float* set_mean,
                                      const float* set_std) try {
  ATC_CHECK_ARG(net != nullptr, "NULL MLP");
  if (set_mean) memcpy(net->mean.data(), set_mean, sizeof(float) * net->I);
  if (set_std) memcpy(net->stdv.data(), set_std, sizeof(float) * net->I);
  if (get_mean) memcpy(get_mean, net->mean.data(), sizeof(float) * net->I);
  if (get_std) memcpy(get_std, net->stdv.data(), sizeof(float) * net->I);
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_mlp_forward(atc_mlp* net, const float* x, int32_t rows, float* y, atc_stream st) try {
  ATC_CHECK_ARG(net != nullptr && x != nullptr && y != nullptr && rows > 0, "bad argument");
  cudaStream_t s = as_stream(st);
  Scratch sc;
  ATC_TRY(alloc_scratch(sc, net, rows, s));
  ATC_TRY(load_rows(sc, net, x, nullptr, nullptr, rows, s));
  ATC_TRY(forward(net, sc, rows, s));
  ATC_CK(cudaMemcpyAsync(y, sc.y.p, sizeof(float) * rows * net->O, cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_mlp_gradients(atc_mlp* net, const float* x, const float* t, const float* mask, int32_t rows,
                                        float* grads, float* loss, atc_stream st) try {
  ATC_CHECK_ARG(net != nullptr && x != nullptr && t != nullptr && rows > 0, "bad argument");
  cudaStream_t s = as_stream(st);
  Scratch sc;
  ATC_TRY(alloc_scratch(sc, net, rows, s));
  ATC_TRY(load_rows(sc, net, x, t, mask, rows, s));
  ATC_TRY(forward(net, sc, rows, s));
  ATC_TRY(backward(net, sc, rows, s));
  if (grads) ATC_CK(cudaMemcpyAsync(grads, sc.grads.p, sizeof(float) * net->nparams, cudaMemcpyDeviceToHost, s));
  if (loss) ATC_CK(cudaMemcpyAsync(loss, sc.loss.p, sizeof(float), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_mlp_train(atc_mlp* net, const float* x, const float* t, const float* mask, int32_t rows,
                                    int32_t epochs, int32_t batch, float lr, uint64_t seed, float* final_loss,
                                    atc_stream st) try {
  ATC_CHECK_ARG(net != nullptr && x != nullptr && t != nullptr && rows > 0 && epochs > 0, "bad argument");
  cudaStream_t s = as_stream(st);
  const int I = net->I, O = net->O;
  if (batch <= 0 || batch > rows) batch = rows;
  // standardisation fitted on the training inputs
  for (int i = 0; i < I; ++i) {
    double mu = 0, var = 0;
    for (int r = 0; r < rows; ++r) mu += x[(int64_t)r * I + i];
    mu /= rows;
    for (int r = 0; r < rows; ++r) {
      double d = x[(int64_t)r * I + i] - mu;
      var += d * d;
    }
    net->mean[i] = (float)mu;
    net->stdv[i] = (float)std::sqrt(var / rows) > 1e-6f ? (float)std::sqrt(var / rows) : 1.0f;
  }
  Scratch sc;
  ATC_TRY(alloc_scratch(sc, net, batch, s));
  DevBuf<float> X, T, M;
  DevBuf<int32_t> idx;
  ATC_TRY(X.alloc((size_t)rows * I, s));
  ATC_TRY(T.alloc((size_t)rows * O, s));
  ATC_TRY(M.alloc((size_t)rows * O, s));
  ATC_TRY(idx.alloc(batch, s));
  ATC_CK(cudaMemcpyAsync(X.p, x, sizeof(float) * rows * I, cudaMemcpyHostToDevice, s));
  standardise_kernel<<<grid_small((int64_t)rows * I), 256, 0, s>>>(X.p, sc.mean.p, sc.inv.p, rows, I);
  ATC_CK(cudaMemcpyAsync(T.p, t, sizeof(float) * rows * O, cudaMemcpyHostToDevice, s));
  if (mask) {
    ATC_CK(cudaMemcpyAsync(M.p, mask, sizeof(float) * rows * O, cudaMemcpyHostToDevice, s));
  } else {
    std::vector<float> ones((size_t)rows * O, 1.0f);
    ATC_CK(cudaMemcpyAsync(M.p, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, s));
    ATC_CK(cudaStreamSynchronize(s));
  }
  std::vector<int32_t> order(rows), pick(batch);
  for (int r = 0; r < rows; ++r) order[r] = r;
  uint64_t rs = mix64(seed ^ 0x51ED270B27A1F3C5ull);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float last = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    for (int r = rows - 1; r > 0; --r) {  // Fisher-Yates with the counter-based generator
      rs = mix64(rs + kGolden);
      int j = (int)(rs % (uint64_t)(r + 1));
      std::swap(order[r], order[j]);
    }
    for (int b0 = 0; b0 + batch <= rows; b0 += batch) {
      std::copy(order.begin() + b0, order.begin() + b0 + batch, pick.begin());
      ATC_CK(cudaMemcpyAsync(idx.p, pick.data(), sizeof(int32_t) * batch, cudaMemcpyHostToDevice, s));
      gather_rows_kernel<<<grid_small((int64_t)batch * I), 256, 0, s>>>(X.p, idx.p, sc.x.p, batch, I);
      gather_rows_kernel<<<grid_small((int64_t)batch * O), 256, 0, s>>>(T.p, idx.p, sc.t.p, batch, O);
      gather_rows_kernel<<<grid_small((int64_t)batch * O), 256, 0, s>>>(M.p, idx.p, sc.mk.p, batch, O);
      ATC_TRY(forward(net, sc, batch, s));
      ATC_TRY(backward(net, sc, batch, s));
      ++net->step;
      float c1 = 1.0f - std::pow(b1, (float)net->step), c2 = 1.0f - std::pow(b2, (float)net->step);
      adam_kernel<<<grid_small(net->nparams), 256, 0, s>>>(net->params, sc.grads.p, net->adam_m, net->adam_v,
                                                            net->nparams, lr, b1, b2, eps, c1, c2);
      ATC_CK(cudaGetLastError());
      ATC_CK(cudaStreamSynchronize(s));  // `pick` is reused by the next step's copy
    }
    ATC_CK(cudaMemcpyAsync(&last, sc.loss.p, sizeof(float), cudaMemcpyDeviceToHost, s));
  }
  ATC_CK(cudaStreamSynchronize(s));
  if (final_loss) *final_loss = last;
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_graph_features(const int32_t* pairs_dev, uint64_t np, float* feat, atc_stream st) try {
  ATC_CHECK_ARG(feat != nullptr && (np == 0 || pairs_dev != nullptr), "bad argument");
  cudaStream_t s = as_stream(st);
  for (int i = 0; i < 6; ++i) feat[i] = 0.0f;
  if (np == 0) return ATC_OK;
  const int2* p = reinterpret_cast<const int2*>(pairs_dev);
  DevBuf<unsigned long long> acc;
  DevBuf<int> mx;
  ATC_TRY(acc.alloc(8, s));
  ATC_TRY(mx.alloc(2, s));
  ATC_CK(cudaMemsetAsync(acc.p, 0, sizeof(unsigned long long) * 8, s));
  int init[2] = {INT_MAX, INT_MIN};
  ATC_CK(cudaMemcpyAsync(mx.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
  feat_minmax_kernel<<<grid_for(np, 256), 256, 0, s>>>(p, np, mx.p, mx.p + 1);
  feat_loops_kernel<<<grid_for(np, 256), 256, 0, s>>>(p, np, acc.p + 6);
  ATC_CK(cudaGetLastError());
  int hm[2];
  unsigned long long loops = 0;
  ATC_CK(cudaMemcpyAsync(hm, mx.p, sizeof(hm), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaMemcpyAsync(&loops, acc.p + 6, sizeof(loops), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  if (hm[0] < 0) {
    set_error("negative vertex id %d", hm[0]);
    return ATC_ERR_INVALID;
  }
  const int64_t n = (int64_t)hm[1] + 1;
  const uint64_t m = np - loops;
  DevBuf<int32_t> deg, dout;
  ATC_TRY(deg.alloc(n, s));
  ATC_TRY(dout.alloc(n, s));
  ATC_CK(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * n, s));
  ATC_CK(cudaMemsetAsync(dout.p, 0, sizeof(int32_t) * n, s));
  feat_deg_kernel<<<grid_for(np, 256), 256, 0, s>>>(p, np, deg.p);
  feat_out_kernel<<<grid_for(np, 256), 256, 0, s>>>(p, np, deg.p, dout.p);
  feat_reduce_kernel<<<grid_for(n, 256), 256, 0, s>>>(deg.p, dout.p, n, 2ull * m, acc.p);
  ATC_CK(cudaGetLastError());
  unsigned long long h[6];
  ATC_CK(cudaMemcpyAsync(h, acc.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  ATC_CK(cudaStreamSynchronize(s));
  const double mean = (double)h[0] / (double)n;
  const double var = (double)h[1] / (double)n - mean * mean;
  const double avg_out = (double)m / (double)n;
  const double tail = (double)h[4] - (double)h[5] * avg_out;  // costFuncCal's tail cost, degree orientation
  feat[0] = (float)std::log1p((double)n);
  feat[1] = (float)std::log1p((double)m);
  feat[2] = (float)std::log1p(mean);
  feat[3] = (float)std::log1p(var > 0 ? var : 0.0);
  feat[4] = (float)std::log1p((double)h[2]);
  feat[5] = (float)std::log1p(tail > 0 ? tail : 0.0);
  return ATC_OK;
} ATC_CATCH

extern "C" atc_status atc_select(atc_mlp* net, const float* feat, int32_t* choice, float* predicted, atc_stream st) try {
  ATC_CHECK_ARG(net != nullptr && feat != nullptr && choice != nullptr, "bad argument");
  std::vector<float> y(net->O);
  ATC_TRY(atc_mlp_forward(net, feat, 1, y.data(), st));
  int best = 0;
  for (int o = 1; o < net->O; ++o)
    if (y[o] < y[best]) best = o;
  *choice = best;
  if (predicted) memcpy(predicted, y.data(), sizeof(float) * net->O);
  return ATC_OK;
} ATC_CATCH
