// C ABI of the BF16 MLP barrier surrogate (lmc_mlp_*): parameters, training and
// ensemble inference on one GPU. The kernels are in mlp.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <random>
#include <vector>

#include "../../include/lmc_gb300.h"
#include "abi_common.hpp"
#include "mlp.cuh"

using lmc::abi::CudaCheck;
using lmc::abi::Guard;
using lmc::abi::Require;

namespace {

template <typename T>
T *DevAlloc(size_t count, std::vector<void *> *owned) {
  void *p = nullptr;
  CudaCheck(cudaMalloc(&p, std::max<size_t>(16, count * sizeof(T))), "cudaMalloc");
  owned->push_back(p);
  return static_cast<T *>(p);
}

constexpr int kPredictChunk = 32768;

}  // namespace

struct lmc_mlp {
  int device{0};
  cudaStream_t stream{nullptr};
  lmc::MlpDev d{};
  long long num_params{0};
  float *params{nullptr}, *grad{nullptr}, *m1{nullptr}, *m2{nullptr}, *loss{nullptr};
  float label_mean{0.f}, label_std{1.f};
  int step{0};
  int path{0};  // inference: 0 automatic (tcgen05 when supported), 1 tcgen05, 2 mma.sync
  int *status{nullptr};
  int cap{0};
  lmc::MlpWork w{};
  __nv_bfloat16 *xb{nullptr}, *xt{nullptr};
  float *tb{nullptr}, *mean_tmp{nullptr}, *spread_tmp{nullptr};
  int *idx{nullptr};
  std::vector<void *> owned, work;

  ~lmc_mlp() {
    cudaSetDevice(device);
    for (void *p : work) cudaFree(p);
    for (void *p : owned) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }

  // Work buffers for batches of up to `rows` samples.
  void Reserve(int rows) {
    if (rows <= cap) return;
    for (void *p : work) cudaFree(p);
    work.clear();
    const size_t wide = static_cast<size_t>(rows) * d.members * d.hidden;
    w.z1 = DevAlloc<float>(wide, &work);
    w.z2 = DevAlloc<float>(wide, &work);
    w.h1 = DevAlloc<__nv_bfloat16>(wide, &work);
    w.h2 = DevAlloc<__nv_bfloat16>(wide, &work);
    w.h1t = DevAlloc<__nv_bfloat16>(wide, &work);
    w.dz1 = DevAlloc<__nv_bfloat16>(wide, &work);
    w.dz1t = DevAlloc<__nv_bfloat16>(wide, &work);
    w.dz2 = DevAlloc<__nv_bfloat16>(wide, &work);
    w.dz2t = DevAlloc<__nv_bfloat16>(wide, &work);
    w.y = DevAlloc<float>(static_cast<size_t>(rows) * d.members, &work);
    xb = DevAlloc<__nv_bfloat16>(static_cast<size_t>(rows) * d.in, &work);
    xt = DevAlloc<__nv_bfloat16>(static_cast<size_t>(rows) * d.in, &work);
    tb = DevAlloc<float>(rows, &work);
    mean_tmp = DevAlloc<float>(rows, &work);
    spread_tmp = DevAlloc<float>(rows, &work);
    idx = DevAlloc<int>(rows, &work);
    cap = rows;
  }

  void Cast() { CudaCheck(lmc::MlpCastWeights(d, stream), "cast weights"); }

  // A tcgen05 training GEMM whose bounded wait expired leaves its outputs unwritten.
  void CheckGemmStatus() {
    int st = 0;
    CudaCheck(cudaMemcpy(&st, d.gemm_status, sizeof(int), cudaMemcpyDeviceToHost), "D2H");
    if (st != 0) {
      CudaCheck(cudaMemset(d.gemm_status, 0, sizeof(int)), "memset");
      throw lmc::abi::LmcError(LMC_ERR_STOPPED, "surrogate training: a tensor-core wait expired");
    }
  }

  // One optimisation step on the batch already in xb / tb.
  void TrainStep(int batch, float lr) {
    CudaCheck(lmc::MlpTranspose(xb, batch, d.in, xt, stream), "transpose");
    CudaCheck(lmc::MlpForward(d, xb, batch, w, true, stream), "forward");
    CudaCheck(lmc::MlpBackward(d, xb, xt, tb, batch, w, grad, loss, stream), "backward");
    ++step;
    CudaCheck(lmc::MlpAdam(params, grad, m1, m2, num_params, lr, step, stream), "adam");
    Cast();
  }
};

namespace lmc {
// Inference queued on `stream` (the tcgen05 kernel; its status word is checked by the
// caller through lmc_mlp_status after synchronising). Returns false when the
// fused kernel does not support this network.
bool MlpPredictAsync(lmc_mlp *mlp, const uint16_t *x_dev, int64_t n, float *mean_dev, float *spread_dev,
                           cudaStream_t stream) {
  if (mlp->path == 2 || !lmc::MlpTcSupported(mlp->d)) return false;
  CudaCheck(cudaMemsetAsync(mlp->status, 0, sizeof(int), stream), "memset");
  CudaCheck(lmc::MlpTcPredict(mlp->d, reinterpret_cast<const __nv_bfloat16 *>(x_dev), n, mlp->label_mean,
                              mlp->label_std, mean_dev, spread_dev, mlp->status, stream),
            "tcgen05 inference");
  return true;
}
bool MlpFusedJumpsAsync(lmc_mlp *mlp, const FusedJumps &j, cudaStream_t stream) {
  if (mlp->path == 2 || lmc::MlpFusedChannels(mlp->d) != j.channels) return false;
  CudaCheck(cudaMemsetAsync(mlp->status, 0, sizeof(int), stream), "memset");
  CudaCheck(lmc::MlpFusedPredict(mlp->d, j, mlp->label_mean, mlp->label_std, mlp->status, stream),
            "fused surrogate kernel");
  return true;
}
const MlpDev &MlpDevOf(const lmc_mlp *mlp) { return mlp->d; }
void MlpLabelScaleOf(const lmc_mlp *mlp, float *mean, float *std_dev) {
  *mean = mlp->label_mean;
  *std_dev = mlp->label_std;
}
int MlpInputs(const lmc_mlp *mlp) { return mlp->d.in; }
const int *MlpStatusDev(const lmc_mlp *mlp) { return mlp->status; }

}  // namespace lmc

extern "C" {

int lmc_mlp_create(int device, int in_features, int hidden, int members, uint64_t seed, lmc_mlp **out) {
  return Guard([&] {
    Require(out != nullptr, LMC_ERR_INVALID_ARGUMENT, "out is null");
    Require(in_features > 0 && in_features % 64 == 0, LMC_ERR_INVALID_ARGUMENT, "in_features must be a multiple of 64");
    Require(hidden > 0 && hidden % 64 == 0, LMC_ERR_INVALID_ARGUMENT, "hidden must be a multiple of 64");
    Require(members >= 1 && members <= 16, LMC_ERR_INVALID_ARGUMENT, "members must be in [1, 16]");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
      throw lmc::abi::LmcError(LMC_ERR_NO_DEVICE, "no CUDA device");
    CudaCheck(cudaSetDevice(device), "cudaSetDevice");
    auto m = std::make_unique<lmc_mlp>();
    m->device = device;
    CudaCheck(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "stream");
    m->d.in = in_features;
    m->d.hidden = hidden;
    m->d.members = members;
    m->num_params = lmc::MlpParamCount(in_features, hidden, members);
    m->params = DevAlloc<float>(m->num_params, &m->owned);
    m->grad = DevAlloc<float>(m->num_params, &m->owned);
    m->m1 = DevAlloc<float>(m->num_params, &m->owned);
    m->m2 = DevAlloc<float>(m->num_params, &m->owned);
    m->loss = DevAlloc<float>(members, &m->owned);
    m->status = DevAlloc<int>(1, &m->owned);
    m->d.gemm_status = DevAlloc<int>(1, &m->owned);
    CudaCheck(cudaMemset(m->d.gemm_status, 0, sizeof(int)), "memset");
    m->d.gemm_mma_sync = 0;
    // split-K partials of the weight-gradient GEMMs: up to 16 splits of the largest gradient
    m->d.gemm_ws_floats = 16LL * members * hidden * std::max(hidden, in_features);
    m->d.gemm_ws = DevAlloc<float>(static_cast<size_t>(m->d.gemm_ws_floats), &m->owned);
    const long long H = hidden, M = members;
    m->d.w1 = m->params;
    m->d.b1 = m->d.w1 + M * H * in_features;
    m->d.w2 = m->d.b1 + M * H;
    m->d.b2 = m->d.w2 + M * H * H;
    m->d.w3 = m->d.b2 + M * H;
    m->d.b3 = m->d.w3 + M * H;
    m->d.w1h = DevAlloc<__nv_bfloat16>(M * H * in_features, &m->owned);
    m->d.w2h = DevAlloc<__nv_bfloat16>(M * H * H, &m->owned);
    m->d.w2t = DevAlloc<__nv_bfloat16>(M * H * H, &m->owned);
    m->d.w1_tiles = DevAlloc<__nv_bfloat16>(M * H * in_features, &m->owned);
    m->d.w2_tiles = DevAlloc<__half>(M * H * H, &m->owned);
    m->d.b2h = DevAlloc<__half>(M * H, &m->owned);
    m->d.w3h = DevAlloc<__half>(M * H, &m->owned);
    // He initialisation (normal, std sqrt(2 / fan_in)), zero biases
    std::vector<float> p(m->num_params, 0.f);
    std::mt19937_64 gen(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    const auto fill = [&](long long off, long long n, float sd) {
      for (long long i = 0; i < n; ++i) p[off + i] = sd * nd(gen);
    };
    fill(0, M * H * in_features, std::sqrt(2.f / in_features));
    fill(M * H * in_features + M * H, M * H * H, std::sqrt(2.f / hidden));
    fill(M * H * in_features + M * H + M * H * H + M * H, M * H, std::sqrt(1.f / hidden));
    CudaCheck(cudaMemcpy(m->params, p.data(), sizeof(float) * p.size(), cudaMemcpyHostToDevice), "H2D");
    CudaCheck(cudaMemset(m->m1, 0, sizeof(float) * m->num_params), "memset");
    CudaCheck(cudaMemset(m->m2, 0, sizeof(float) * m->num_params), "memset");
    m->Cast();
    CudaCheck(cudaStreamSynchronize(m->stream), "sync");
    *out = m.release();
  });
}

void lmc_mlp_destroy(lmc_mlp *mlp) { delete mlp; }

int lmc_mlp_layout(const lmc_mlp *mlp, int *in_features, int *hidden, int *members, int64_t *num_params) {
  return Guard([&] {
    Require(mlp != nullptr, LMC_ERR_INVALID_ARGUMENT, "mlp is null");
    if (in_features) *in_features = mlp->d.in;
    if (hidden) *hidden = mlp->d.hidden;
    if (members) *members = mlp->d.members;
    if (num_params) *num_params = mlp->num_params;
  });
}

int lmc_mlp_get_params(lmc_mlp *mlp, float *params) {
  return Guard([&] {
    Require(mlp && params, LMC_ERR_INVALID_ARGUMENT, "null argument");
    CudaCheck(cudaSetDevice(mlp->device), "cudaSetDevice");
    CudaCheck(cudaMemcpyAsync(params, mlp->params, sizeof(float) * mlp->num_params, cudaMemcpyDeviceToHost,
                              mlp->stream),
              "D2H");
    CudaCheck(cudaStreamSynchronize(mlp->stream), "sync");
  });
}

int lmc_mlp_set_params(lmc_mlp *mlp, const float *params) {
  return Guard([&] {
    Require(mlp && params, LMC_ERR_INVALID_ARGUMENT, "null argument");
    CudaCheck(cudaSetDevice(mlp->device), "cudaSetDevice");
    CudaCheck(cudaMemcpyAsync(mlp->params, params, sizeof(float) * mlp->num_params, cudaMemcpyHostToDevice,
                              mlp->stream),
              "H2D");
    mlp->Cast();
    CudaCheck(cudaStreamSynchronize(mlp->stream), "sync");
  });
}

int lmc_mlp_set_label_scale(lmc_mlp *mlp, float mean, float std_dev) {
  return Guard([&] {
    Require(mlp != nullptr, LMC_ERR_INVALID_ARGUMENT, "mlp is null");
    Require(std_dev > 0.f && std::isfinite(std_dev) && std::isfinite(mean), LMC_ERR_INVALID_ARGUMENT,
            "label scale must be finite with std > 0");
    mlp->label_mean = mean;
    mlp->label_std = std_dev;
  });
}

int lmc_mlp_gradients(lmc_mlp *mlp, const uint16_t *x, const float *labels, int batch, float *grad, float *loss) {
  return Guard([&] {
    Require(mlp && x && labels && grad, LMC_ERR_INVALID_ARGUMENT, "null argument");
    Require(batch > 0 && batch % 64 == 0, LMC_ERR_INVALID_ARGUMENT, "batch must be a positive multiple of 64");
    CudaCheck(cudaSetDevice(mlp->device), "cudaSetDevice");
    mlp->Reserve(batch);
    std::vector<float> t(batch);
    for (int b = 0; b < batch; ++b) t[b] = (labels[b] - mlp->label_mean) / mlp->label_std;
    CudaCheck(cudaMemcpyAsync(mlp->xb, x, sizeof(uint16_t) * batch * mlp->d.in, cudaMemcpyHostToDevice, mlp->stream),
              "H2D");
    CudaCheck(cudaMemcpyAsync(mlp->tb, t.data(), sizeof(float) * batch, cudaMemcpyHostToDevice, mlp->stream), "H2D");
    CudaCheck(cudaMemsetAsync(mlp->loss, 0, sizeof(float) * mlp->d.members, mlp->stream), "memset");
    CudaCheck(lmc::MlpTranspose(mlp->xb, batch, mlp->d.in, mlp->xt, mlp->stream), "transpose");
    CudaCheck(lmc::MlpForward(mlp->d, mlp->xb, batch, mlp->w, true, mlp->stream), "forward");
    CudaCheck(lmc::MlpBackward(mlp->d, mlp->xb, mlp->xt, mlp->tb, batch, mlp->w, mlp->grad, mlp->loss, mlp->stream),
              "backward");
    CudaCheck(cudaMemcpyAsync(grad, mlp->grad, sizeof(float) * mlp->num_params, cudaMemcpyDeviceToHost, mlp->stream),
              "D2H");
    if (loss)
      CudaCheck(cudaMemcpyAsync(loss, mlp->loss, sizeof(float) * mlp->d.members, cudaMemcpyDeviceToHost, mlp->stream),
                "D2H");
    CudaCheck(cudaStreamSynchronize(mlp->stream), "sync");
    mlp->CheckGemmStatus();
  });
}

int lmc_mlp_train(lmc_mlp *mlp, const uint16_t *x_dev, const float *labels_dev, int64_t n, int batch, int epochs,
                  float lr, uint64_t seed, float *loss) {
  return Guard([&] {
    Require(mlp && x_dev && labels_dev, LMC_ERR_INVALID_ARGUMENT, "null argument");
    Require(batch > 0 && batch % 64 == 0, LMC_ERR_INVALID_ARGUMENT, "batch must be a positive multiple of 64");
    Require(n >= batch && n < (1LL << 31), LMC_ERR_INVALID_ARGUMENT, "need batch <= n < 2^31 samples");
    Require(epochs >= 1 && lr > 0.f, LMC_ERR_INVALID_ARGUMENT, "epochs >= 1 and lr > 0");
    CudaCheck(cudaSetDevice(mlp->device), "cudaSetDevice");
    mlp->Reserve(batch);
    const auto *x = reinterpret_cast<const __nv_bfloat16 *>(x_dev);
    const long long steps_per_epoch = n / batch, total = steps_per_epoch * epochs;
    std::vector<int> perm(static_cast<size_t>(n));
    std::iota(perm.begin(), perm.end(), 0);
    std::mt19937_64 gen(seed);
    int *dperm = nullptr;
    CudaCheck(cudaMalloc(&dperm, sizeof(int) * n), "cudaMalloc");
    std::vector<float> host_loss(mlp->d.members, 0.f);
    try {
      long long k = 0;
      for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(perm.begin(), perm.end(), gen);
        CudaCheck(cudaMemcpyAsync(dperm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, mlp->stream), "H2D");
        CudaCheck(cudaMemsetAsync(mlp->loss, 0, sizeof(float) * mlp->d.members, mlp->stream), "memset");
        for (long long b = 0; b < steps_per_epoch; ++b, ++k) {
          // cosine schedule over all steps
          const float lr_k = lr * 0.5f * (1.f + std::cos(3.14159265358979f * static_cast<float>(k) / total));
          CudaCheck(lmc::MlpGather(x, labels_dev, dperm + b * batch, batch, mlp->d.in, mlp->label_mean,
                                   1.f / mlp->label_std, mlp->xb, mlp->tb, mlp->stream),
                    "gather");
          mlp->TrainStep(batch, lr_k);
        }
        CudaCheck(cudaMemcpyAsync(host_loss.data(), mlp->loss, sizeof(float) * mlp->d.members, cudaMemcpyDeviceToHost,
                                  mlp->stream),
                  "D2H");
        CudaCheck(cudaStreamSynchronize(mlp->stream), "sync");
      }
    } catch (...) {
      cudaFree(dperm);
      throw;
    }
    cudaFree(dperm);
    mlp->CheckGemmStatus();
    // mean loss per member over the last epoch, in standardised label units
    if (loss)
      for (int m = 0; m < mlp->d.members; ++m) loss[m] = host_loss[m] / static_cast<float>(steps_per_epoch);
  });
}

int lmc_mlp_set_train_path(lmc_mlp *mlp, int path) {
  return Guard([&] {
    Require(mlp != nullptr, LMC_ERR_INVALID_ARGUMENT, "mlp is null");
    Require(path == 0 || path == 1, LMC_ERR_INVALID_ARGUMENT, "path must be 0 (tcgen05) or 1 (mma.sync)");
    mlp->d.gemm_mma_sync = path;
  });
}

int lmc_mlp_set_inference_path(lmc_mlp *mlp, int path) {
  return Guard([&] {
    Require(mlp != nullptr, LMC_ERR_INVALID_ARGUMENT, "mlp is null");
    Require(path >= 0 && path <= 2, LMC_ERR_INVALID_ARGUMENT, "path must be 0, 1 or 2");
    Require(path != 1 || lmc::MlpTcSupported(mlp->d) || lmc::MlpFusedSupported(mlp->d), LMC_ERR_UNSUPPORTED,
            "the tcgen05 kernels serve hidden 256 with in_features <= 256, or 2 members of 128 / 192 -> 128");
    mlp->path = path;
  });
}

int lmc_mlp_predict(lmc_mlp *mlp, const uint16_t *x_dev, int64_t n, float *mean_dev, float *spread_dev) {
  return Guard([&] {
    Require(mlp && x_dev && mean_dev, LMC_ERR_INVALID_ARGUMENT, "null argument");
    Require(n >= 0, LMC_ERR_INVALID_ARGUMENT, "n < 0");
    CudaCheck(cudaSetDevice(mlp->device), "cudaSetDevice");
    if (mlp->path != 2 && lmc::MlpTcSupported(mlp->d)) {
      CudaCheck(cudaMemsetAsync(mlp->status, 0, sizeof(int), mlp->stream), "memset");
      CudaCheck(lmc::MlpTcPredict(mlp->d, reinterpret_cast<const __nv_bfloat16 *>(x_dev), n, mlp->label_mean,
                                  mlp->label_std, mean_dev, spread_dev, mlp->status, mlp->stream),
                "tcgen05 inference");
      int st = 0;
      CudaCheck(cudaMemcpyAsync(&st, mlp->status, sizeof(int), cudaMemcpyDeviceToHost, mlp->stream), "D2H");
      CudaCheck(cudaStreamSynchronize(mlp->stream), "sync");
      Require(st == 0, LMC_ERR_STOPPED, "tcgen05 inference: a tensor-core wait expired");
      return;
    }
    mlp->Reserve(kPredictChunk);
    const auto *x = reinterpret_cast<const __nv_bfloat16 *>(x_dev);
    for (int64_t off = 0; off < n; off += kPredictChunk) {
      const int rows = static_cast<int>(std::min<int64_t>(kPredictChunk, n - off));
      const int padded = (rows + 63) / 64 * 64;
      const __nv_bfloat16 *src = x + off * mlp->d.in;
      if (padded != rows) {
        CudaCheck(cudaMemsetAsync(mlp->xb, 0, sizeof(__nv_bfloat16) * padded * mlp->d.in, mlp->stream), "memset");
        CudaCheck(cudaMemcpyAsync(mlp->xb, src, sizeof(__nv_bfloat16) * rows * mlp->d.in, cudaMemcpyDeviceToDevice,
                                  mlp->stream),
                  "D2D");
        src = mlp->xb;
      }
      CudaCheck(lmc::MlpForward(mlp->d, src, padded, mlp->w, false, mlp->stream), "forward");
      const bool direct = padded == rows;
      CudaCheck(lmc::MlpEnsemble(mlp->w.y, padded, mlp->d.members, mlp->label_mean, mlp->label_std,
                                 direct ? mean_dev + off : mlp->mean_tmp,
                                 spread_dev ? (direct ? spread_dev + off : mlp->spread_tmp) : nullptr, mlp->stream),
                "ensemble");
      if (!direct) {
        CudaCheck(cudaMemcpyAsync(mean_dev + off, mlp->mean_tmp, sizeof(float) * rows, cudaMemcpyDeviceToDevice,
                                  mlp->stream),
                  "D2D");
        if (spread_dev)
          CudaCheck(cudaMemcpyAsync(spread_dev + off, mlp->spread_tmp, sizeof(float) * rows, cudaMemcpyDeviceToDevice,
                                    mlp->stream),
                    "D2D");
      }
    }
    CudaCheck(cudaStreamSynchronize(mlp->stream), "sync");
  });
}

}  // extern "C"
