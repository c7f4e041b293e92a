// Device side of the BF16 MLP barrier surrogate (see mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace lmc {

// GELU, tanh form (Hendrycks & Gimpel, 2016): 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))),
// with the hardware tanh approximation (relative error ~2^-11, below BF16 resolution).
#ifdef __CUDACC__
__device__ __forceinline__ float MlpTanh(float u) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return t;
}
// u = z (c0 + c1 z^2) with c0 = sqrt(2/pi), c1 = 0.044715 c0; GELU = h + h tanh(u), h = z / 2.
__device__ __forceinline__ float MlpGelu(float z) {
  const float t = MlpTanh(z * fmaf(z * z, 0.0356774081363001f, 0.7978845608028654f));
  const float h = 0.5f * z;
  return fmaf(h, t, h);
}
__device__ __forceinline__ float MlpGeluGrad(float z) {
  const float t = MlpTanh(z * fmaf(z * z, 0.0356774081363001f, 0.7978845608028654f));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * 0.7978845608028654f * fmaf(0.134145f, z * z, 1.0f);
}
#endif

// Training GEMMs: C[m][n] = sum_k A[m][k] B[n][k] (both operands K-major, BF16, FP32
// accumulate), batched over grid.z, with one of three fused epilogues.
enum Epi : int {
  kEpiStoreF32 = 0,     // C fp32 = alpha acc                            (weight gradients)
  kEpiBiasGelu = 1,     // Z = acc + bias (fp32), H = GELU(Z) (bf16), optional Ht (bf16, [n][m])
  kEpiGeluGrad = 2,     // D = acc * GELU'(Z) (bf16), optional Dt (bf16, [n][m])
};

struct GemmArgs {
  const __nv_bfloat16 *a;  // [M][K], lda
  const __nv_bfloat16 *b;  // [N][K], ldb
  int m, n, k, lda, ldb;
  long long stride_a, stride_b;  // per grid.z
  // epilogue
  float *c;              // kEpiStoreF32: [M][N] ldc; kEpiBiasGelu: Z; kEpiGeluGrad: Z (input)
  const float *bias;     // kEpiBiasGelu
  __nv_bfloat16 *h;      // kEpiBiasGelu: H; kEpiGeluGrad: D
  __nv_bfloat16 *ht;     // optional transposed copy, [N][M] with ld ldt
  int ldc, ldh, ldt;
  long long stride_c, stride_bias, stride_h, stride_ht;
  float alpha;           // scales acc (kEpiStoreF32)
  // kEpiStoreF32 on the tcgen05 path: K split over `splits` CTAs (1 = none), whose partial tiles
  // go to ws ([splits][batch][m][n]) and are summed in split order by a second kernel
  int splits;
  float *ws;
};

// The tcgen05 version of the training GEMMs (mlp_gemm_tc.cu): 128-row tiles, N tiles of 64 /
// 128 / 256, accumulators in TMEM. GemmTcFits: M a multiple of 128, N of 64, K of 32, the
// leading dimensions and epilogue strides multiples of 8. An expired wait sets *status.
bool GemmTcFits(const GemmArgs &g);
cudaError_t GemmTc(const GemmArgs &g, int epi, int batch, int *status, cudaStream_t s);

// Parameters of an ensemble (FP32 master copy, flat: W1, b1, W2, b2, w3, b3) and
// the BF16 copies the GEMMs read.
struct MlpDev {
  int in, hidden, members;
  int gemm_mma_sync;   // 1: training GEMMs on mma.sync only; 0: tcgen05 where GemmTcFits
  int *gemm_status;    // device word set by an expired tcgen05 wait
  float *gemm_ws;      // split-K partials of the weight-gradient GEMMs
  long long gemm_ws_floats;
  float *w1, *b1, *w2, *b2, *w3, *b3;
  __nv_bfloat16 *w1h, *w2h, *w2t;
  // W1 (bf16) and W2 (IEEE half: layer 2 of the tensor-core inference runs in
  // f16) again, cut into R-row x 32-K blocks stored contiguously in the tensor
  // cores' shared-memory operand layout (see mlp_tc.cu), so one bulk copy moves a
  // block. R = 256 for hidden 256 (member m, block c of W1 at (m * in / 32 + c) *
  // 8192 elements, of W2 at (m * hidden / 32 + c) * 8192) and R = 128 for hidden 128
  // (blocks of 4096 elements, same order).
  __nv_bfloat16 *w1_tiles;
  __half *w2_tiles;
  // b2 and w3 in IEEE half (the fused jump kernel's packed layer-2 epilogue). For in = 128
  // or 192 and hidden = 128 (that kernel's shapes) the tiles and b2h hold W1, W2 and b2
  // halved, and the last input column of w1_tiles holds b1 / 2 instead of W1's (unused)
  // last column: the kernel sets that feature to 1, so the layer-1 MMA adds the bias.
  __half *b2h, *w3h;
};

// Activations of one batch (sizes for batch B, M members, H hidden).
struct MlpWork {
  float *z1, *z2;                 // [B][M*H]
  __nv_bfloat16 *h1, *h2, *h1t;   // [B][M*H], h1t [M*H][B]
  __nv_bfloat16 *dz1, *dz1t, *dz2, *dz2t;
  float *y;                       // [M][B]
};

// Parameter count of an ensemble.
inline long long MlpParamCount(int in, int hidden, int members) {
  return static_cast<long long>(members) * (static_cast<long long>(hidden) * in + hidden +
                                            static_cast<long long>(hidden) * hidden + hidden + hidden + 1);
}

cudaError_t MlpForward(const MlpDev &d, const __nv_bfloat16 *x, int batch, MlpWork &w, bool keep_ht, cudaStream_t s);
// Gradients of the mean squared error of every member (flat, parameter order) and the per-member loss.
cudaError_t MlpBackward(const MlpDev &d, const __nv_bfloat16 *x, const __nv_bfloat16 *xt, const float *t, int batch,
                        MlpWork &w, float *grad, float *loss, cudaStream_t s);
cudaError_t MlpGather(const __nv_bfloat16 *x, const float *labels, const int *idx, int batch, int in, float mean,
                      float inv_std, __nv_bfloat16 *xb, float *tb, cudaStream_t s);
cudaError_t MlpTranspose(const __nv_bfloat16 *in, int rows, int cols, __nv_bfloat16 *out, cudaStream_t s);
cudaError_t MlpAdam(float *p, const float *grad, float *m1, float *m2, long long n, float lr, int step, cudaStream_t s);
cudaError_t MlpCastWeights(const MlpDev &d, cudaStream_t s);
// Fused tcgen05 inference of feature rows (mlp_tc.cu): hidden 256, in <= 256 and a multiple of 64.
bool MlpTcSupported(const MlpDev &d);
size_t MlpTcSharedBytes(int in);
cudaError_t MlpTcPredict(const MlpDev &d, const __nv_bfloat16 *x, long long n, float mean_label, float std_label,
                         float *mean, float *spread, int *status, cudaStream_t s);
cudaError_t MlpEnsemble(const float *y, int batch, int members, float mean_label, float std_label, float *mean,
                        float *spread, cudaStream_t s);

// Lattice jumps for the fused kernel (mlp_fused.cu), which gathers the solute-channel
// features itself (two channels per site for one-hot alphabets of three species, three
// for four).
struct FusedJumps {
  const int8_t *species;     // the lattice (one replica), n^3 cells
  int n;
  const long long *pairs;    // [m][2] (vacancy site, migrant site)
  long long m;
  const int *m_dev;          // nullable: the row count on the device (m is then its upper bound)
  const int8_t *mmm_off;     // [12][58][4] MMM-ordered offsets per jump direction (half units)
  const int8_t *dir_of;      // [27] 1NN direction of an offset, -1 none
  int channels;              // channels per site (2 or 3)
  uint32_t site_word[8];     // two channels: per species code, both bf16 channels as one word (0: base)
  int8_t chan[8];            // per species code: its channel, -1 none (the base, a vacancy)
  uint32_t fallback_codes;   // bit c: species code c in the environment sends the row to the plain predictor
  float *mean, *spread;      // [m] ensemble mean (eV) and spread (+inf: plain predictor)
  int *pair_status;          // kStatusBadSite / kStatusNotNeighbor of rejected pairs
  float mean_label, std_label;  // the network's label scale (the persistent KMC kernel)
};
// The fused kernel serves ensembles of 2 members, 128 or 192 inputs (2 or 3 channels per
// site), hidden 128 (weights kept in shared memory); an expired wait sets *status.
bool MlpFusedSupported(const MlpDev &d);
int MlpFusedChannels(const MlpDev &d);  // 2, 3, or 0 when the kernel does not serve the network
cudaError_t MlpFusedPredict(const MlpDev &d, const FusedJumps &j, float mean_label, float std_label, int *status,
                            cudaStream_t s);

}  // namespace lmc

// Host-side hooks of the surrogate object (surrogate.cpp) for other translation units.
struct lmc_mlp;
namespace lmc {
bool MlpPredictAsync(lmc_mlp *mlp, const uint16_t *x_dev, int64_t n, float *mean_dev, float *spread_dev,
                     cudaStream_t stream);
// The fused jump kernel queued on `stream` (status word as above); false when this network
// or the inference path setting does not allow it.
bool MlpFusedJumpsAsync(lmc_mlp *mlp, const FusedJumps &j, cudaStream_t stream);
const MlpDev &MlpDevOf(const lmc_mlp *mlp);
void MlpLabelScaleOf(const lmc_mlp *mlp, float *mean, float *std_dev);
int MlpInputs(const lmc_mlp *mlp);
const int *MlpStatusDev(const lmc_mlp *mlp);
}  // namespace lmc
