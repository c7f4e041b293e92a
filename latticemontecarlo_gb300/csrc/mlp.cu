// BF16 MLP barrier surrogate: ensemble of M members, each in -> H -> H -> 1 with
// GELU, BF16 weights and activations, FP32 accumulation, FP32 master weights and
// Adam. Every matrix product is one "NT" GEMM, C[m][n] = sum_k A[m][k] B[n][k],
// on the tensor cores (mma.sync m16n8k16 BF16, FP32 accumulate), batched over
// ensemble members with grid.z, with the bias / GELU / GELU-derivative work
// fused into the epilogues. Layouts (b = sample, per member m):
//   X   [B][K]           one-hot features (bf16)        Xt  [K][B]
//   W1  [M*H][K]  b1 [M*H]                               (layer 1 of all members in one GEMM)
//   W2  [M][H][H] b2 [M][H]      W2t [M][H][H] (transposed, for dH1 = dZ2 W2)
//   w3  [M][H]    b3 [M]
//   Z1, Z2 [B][M*H] pre-activations (fp32); H1, H2 [B][M*H] (bf16) and H1t [M*H][B]
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "mlp.cuh"

namespace lmc {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 32, kPad = 8, kGemmThreads = 128;

__device__ __forceinline__ uint32_t SmemAddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void CpAsync16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(SmemAddr(smem)), "l"(gmem));
}
__device__ __forceinline__ void CpAsyncCommit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void CpAsyncWait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void CpAsyncWait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

__device__ __forceinline__ void LdMatrixX4(uint32_t *r, const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(SmemAddr(p)));
}
__device__ __forceinline__ void Mma16816(float *c, const uint32_t *a, const uint32_t *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float Gelu(float z) { return MlpGelu(z); }
__device__ __forceinline__ float GeluGrad(float z) { return MlpGeluGrad(z); }

// C tile (kBM x kBN) per block, 4 warps of 32 x 32; K in steps of kBK with a
// two-stage cp.async pipeline. M, N multiples of 64 and K of 32 (checked on the host).
template <int kEpi>
__global__ void __launch_bounds__(kGemmThreads) gemm_nt_kernel(GemmArgs g) {
  __shared__ __align__(16) __nv_bfloat16 sa[2][kBM][kBK + kPad];
  __shared__ __align__(16) __nv_bfloat16 sb[2][kBN][kBK + kPad];
  const int z = blockIdx.z;
  const __nv_bfloat16 *A = g.a + z * g.stride_a;
  const __nv_bfloat16 *B = g.b + z * g.stride_b;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

  auto load = [&](int stage, int k0) {
    // 64 rows x 32 bf16 = 4 chunks of 16 B per row, 256 chunks per operand, 2 per thread
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int c = tid + i * kGemmThreads;
      const int row = c >> 2, col = (c & 3) * 8;
      CpAsync16(&sa[stage][row][col], A + static_cast<long long>(m0 + row) * g.lda + k0 + col);
      CpAsync16(&sb[stage][row][col], B + static_cast<long long>(n0 + row) * g.ldb + k0 + col);
    }
    CpAsyncCommit();
  };

  const int ktiles = g.k / kBK;
  load(0, 0);
  for (int kt = 0; kt < ktiles; ++kt) {
    const int stage = kt & 1;
    if (kt + 1 < ktiles) {
      load(stage ^ 1, (kt + 1) * kBK);
      CpAsyncWait1();
    } else {
      CpAsyncWait0();
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kBK; ks += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        // x4: rows 0-15 of the 16x16 A fragment, k halves
        const int r = wm + i * 16 + (lane & 15);
        const int c = ks + (lane >> 4) * 8;
        LdMatrixX4(af[i], &sa[stage][r][c]);
      }
#pragma unroll
      for (int j = 0; j < 4; j += 2) {
        // x4: two n8 tiles x two k halves of B ([n][k] rows = the col-major fragment)
        uint32_t r4[4];
        const int r = wn + j * 8 + (lane & 7) + ((lane >> 4) << 3);
        const int c = ks + ((lane >> 3) & 1) * 8;
        LdMatrixX4(r4, &sb[stage][r][c]);
        bf[j][0] = r4[0];
        bf[j][1] = r4[1];
        bf[j + 1][0] = r4[2];
        bf[j + 1][1] = r4[3];
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) Mma16816(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }

  // epilogue: fragment element q of tile (i, j) sits at row (lane / 4) + 8 * (q / 2),
  // column 2 * (lane % 4) + (q % 2)
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int row = m0 + wm + i * 16 + (lane >> 2) + 8 * (q >> 1);
        const int col = n0 + wn + j * 8 + 2 * (lane & 3) + (q & 1);
        const float v = acc[i][j][q];
        if (kEpi == kEpiStoreF32) {
          g.c[z * g.stride_c + static_cast<long long>(row) * g.ldc + col] = g.alpha * v;
        } else if (kEpi == kEpiBiasGelu) {
          const float zz = v + g.bias[z * g.stride_bias + col];
          g.c[z * g.stride_c + static_cast<long long>(row) * g.ldc + col] = zz;
          const __nv_bfloat16 hv = __float2bfloat16(Gelu(zz));
          g.h[z * g.stride_h + static_cast<long long>(row) * g.ldh + col] = hv;
          if (g.ht) g.ht[z * g.stride_ht + static_cast<long long>(col) * g.ldt + row] = hv;
        } else {
          const float zz = g.c[z * g.stride_c + static_cast<long long>(row) * g.ldc + col];
          const __nv_bfloat16 dv = __float2bfloat16(v * GeluGrad(zz));
          g.h[z * g.stride_h + static_cast<long long>(row) * g.ldh + col] = dv;
          if (g.ht) g.ht[z * g.stride_ht + static_cast<long long>(col) * g.ldt + row] = dv;
        }
      }
}

// The training GEMMs go to the tcgen05 kernel where the shape fits (unless the ensemble is set
// to mma.sync), else to the mma.sync kernel above.
template <int kEpi>
cudaError_t Gemm(const MlpDev &d, const GemmArgs &g, int batch, cudaStream_t s) {
  if (!d.gemm_mma_sync && d.gemm_status && GemmTcFits(g)) {
    GemmArgs t = g;
    t.splits = 1;
    if (kEpi == kEpiStoreF32 && d.gemm_ws) {
      // weight gradients (K = the batch): split K until the grid fills the GPU, at least 4 K
      // tiles per split, the partials within the workspace
      const int bn = g.n % 256 == 0 ? 256 : (g.n % 128 == 0 ? 128 : 64);
      const long long ctas = static_cast<long long>(g.n / bn) * (g.m / 128) * batch;
      const int ktiles = g.k / 32;
      while (t.splits < 16 && ctas * t.splits < 256 && ktiles % (2 * t.splits) == 0 &&
             ktiles / (2 * t.splits) >= 4 &&
             2LL * t.splits * batch * g.m * g.n <= d.gemm_ws_floats)
        t.splits *= 2;
      t.ws = d.gemm_ws;
    }
    return GemmTc(t, kEpi, batch, d.gemm_status, s);
  }
  if (g.m % kBM || g.n % kBN || g.k % kBK || g.m <= 0 || g.n <= 0 || g.k <= 0) return cudaErrorInvalidValue;
  const dim3 grid(g.n / kBN, g.m / kBM, batch);
  gemm_nt_kernel<kEpi><<<grid, kGemmThreads, 0, s>>>(g);
  return cudaGetLastError();
}

// Output layer of every member: y[m][b] = H2[b][m*H:(m+1)*H] . w3[m] + b3[m]; one warp per (b, m).
__global__ void output_kernel(const __nv_bfloat16 *h2, const float *w3, const float *b3, int batch, int members,
                              int hidden, float *y) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= batch * members) return;
  const int b = warp / members, m = warp % members;
  const __nv_bfloat16 *h = h2 + static_cast<long long>(b) * members * hidden + m * hidden;
  float s = 0.f;
  for (int j = lane; j < hidden; j += 32) s += __bfloat162float(h[j]) * w3[m * hidden + j];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[m * batch + b] = s + b3[m];
}

// Loss and output-layer backward. dy = 2 (y - t) / B (mean squared error per member);
// dZ2[b][m, j] = dy * w3[m][j] * GELU'(Z2), written with its transpose.
__global__ void output_backward_kernel(const float *y, const float *t, const float *z2, const float *w3, int batch,
                                       int members, int hidden, __nv_bfloat16 *dz2, __nv_bfloat16 *dz2t,
                                       float *loss) {
  const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  const long long total = static_cast<long long>(batch) * members * hidden;
  if (idx >= total) return;
  const int b = static_cast<int>(idx / (members * hidden));
  const int col = static_cast<int>(idx % (members * hidden));
  const int m = col / hidden, j = col % hidden;
  const float diff = y[m * batch + b] - t[b];
  const float dy = 2.f * diff / batch;
  const __nv_bfloat16 v = __float2bfloat16(dy * w3[m * hidden + j] * GeluGrad(z2[idx]));
  dz2[idx] = v;
  dz2t[static_cast<long long>(col) * batch + b] = v;
  if (j == 0) atomicAdd(&loss[m], diff * diff / batch);
}

// Output-layer parameter gradients: gw3[m][j] = sum_b dy[m][b] H2[b][m, j], gb3[m] = sum_b dy.
__global__ void output_param_grad_kernel(const float *y, const float *t, const __nv_bfloat16 *h2, int batch,
                                         int members, int hidden, float *gw3, float *gb3) {
  const int col = blockIdx.x;  // m * hidden + j
  const int m = col / hidden;
  float s = 0.f, sb = 0.f;
  for (int b = threadIdx.x; b < batch; b += blockDim.x) {
    const float dy = 2.f * (y[m * batch + b] - t[b]) / batch;
    s += dy * __bfloat162float(h2[static_cast<long long>(b) * members * hidden + col]);
    sb += dy;
  }
  __shared__ float red[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = s;
    red[1][threadIdx.x >> 5] = sb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, c = 0.f;
    for (int w = 0; w < (blockDim.x >> 5); ++w) {
      a += red[0][w];
      c += red[1][w];
    }
    gw3[col] = a;
    if (col % hidden == 0) gb3[m] = c;
  }
}

// Column sums of a bf16 [rows][cols] matrix given transposed ([cols][rows]): one block per column.
__global__ void column_sum_kernel(const __nv_bfloat16 *dt, int rows, float *out) {
  const __nv_bfloat16 *p = dt + static_cast<long long>(blockIdx.x) * rows;
  float s = 0.f;
  for (int r = threadIdx.x; r < rows; r += blockDim.x) s += __bfloat162float(p[r]);
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f;
    for (int w = 0; w < (blockDim.x >> 5); ++w) a += red[w];
    out[blockIdx.x] = a;
  }
}

// Adam (Kingma & Ba, 2015) on the FP32 master parameters, then the BF16 copies.
__global__ void adam_kernel(float *p, const float *grad, float *m1, float *m2, long long n, float lr, float beta1,
                            float beta2, float eps, float c1, float c2) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = grad[i];
  const float a = beta1 * m1[i] + (1.f - beta1) * g;
  const float b = beta2 * m2[i] + (1.f - beta2) * g * g;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// BF16 copies of W1, W2 and W2 transposed from the master parameters.
__global__ void cast_weights_kernel(const float *w1, long long n1, const float *w2, int members, int hidden,
                                    __nv_bfloat16 *w1h, __nv_bfloat16 *w2h, __nv_bfloat16 *w2t) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n1) w1h[i] = __float2bfloat16(w1[i]);
  const long long n2 = static_cast<long long>(members) * hidden * hidden;
  if (i < n2) {
    const int m = static_cast<int>(i / (static_cast<long long>(hidden) * hidden));
    const int r = static_cast<int>((i / hidden) % hidden), c = static_cast<int>(i % hidden);
    const __nv_bfloat16 v = __float2bfloat16(w2[i]);
    w2h[i] = v;
    w2t[static_cast<long long>(m) * hidden * hidden + static_cast<long long>(c) * hidden + r] = v;
  }
}

// Weights of [rows][k] row-major in the operand-block layout of the tcgen05 kernels:
// block (row / R, k / 32) of R x 32 elements, element (r, kk) at
// (r / 8) * 256 + (kk / 8) * 64 + (r % 8) * 8 + kk % 8 (16-bit units).
template <typename T>
__device__ __forceinline__ T FromFloat(float v);
template <>
__device__ __forceinline__ __nv_bfloat16 FromFloat<__nv_bfloat16>(float v) { return __float2bfloat16(v); }
template <>
__device__ __forceinline__ __half FromFloat<__half>(float v) { return __float2half_rn(v); }

template <typename T>
__global__ void tile_weights_kernel(const float *w, long long rows, int k, int block_rows, float scale, T *out) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= rows * k) return;
  const long long r = i / k;
  const int kk = static_cast<int>(i % k);
  const long long block = (r / block_rows) * (k / 32) + kk / 32;
  const int rr = static_cast<int>(r % block_rows), kc = kk % 32;
  out[block * block_rows * 32 + (rr >> 3) * 256 + (kc >> 3) * 64 + (rr & 7) * 8 + (kc & 7)] = FromFloat<T>(scale * w[i]);
}

// Half copies of `scale` b2 and of w3; with kt > 0 (hidden 128, kt = in / 32 K tiles),
// `scale` b1 into the last input column of the W1 tiles (row r = m * 128 + h: block
// m * kt + kt - 1, column 31 of the block).
__global__ void fused_extras_kernel(const float *b1, const float *b2, const float *w3, int n, int kt, float scale,
                                    __half *b2h, __half *w3h, __nv_bfloat16 *w1_tiles) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  b2h[i] = __float2half_rn(scale * b2[i]);
  w3h[i] = __float2half_rn(w3[i]);
  if (kt > 0) {
    const int m = i / 128, h = i % 128;
    w1_tiles[static_cast<long long>(m * kt + kt - 1) * 4096 + (h >> 3) * 256 + 3 * 64 + (h & 7) * 8 + 7] =
        __float2bfloat16(scale * b1[i]);
  }
}

// Transpose of a bf16 [rows][cols] matrix (32 x 32 tiles through shared memory).
__global__ void transpose_bf16_kernel(const __nv_bfloat16 *in, int rows, int cols, __nv_bfloat16 *out) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int c = blockIdx.x * 32 + threadIdx.x, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y)
    if (r0 + k < rows && c < cols) tile[k][threadIdx.x] = in[static_cast<long long>(r0 + k) * cols + c];
  __syncthreads();
  const int oc = r0 + threadIdx.x, orow0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y)
    if (orow0 + k < cols && oc < rows) out[static_cast<long long>(orow0 + k) * rows + oc] = tile[threadIdx.x][k];
}

// Ensemble mean and spread (max - min) per sample, in label units.
__global__ void ensemble_kernel(const float *y, int batch, int members, float mean_label, float std_label,
                                float *mean, float *spread) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  float s = 0.f, lo = 1e30f, hi = -1e30f;
  for (int m = 0; m < members; ++m) {
    const float v = y[m * batch + b];
    s += v;
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  mean[b] = mean_label + std_label * s / members;
  if (spread) spread[b] = std_label * (hi - lo);
}

// Rows idx[b] of X and standardised labels for one training batch.
__global__ void gather_kernel(const __nv_bfloat16 *x, const float *labels, const int *idx, int batch, int in,
                              float mean, float inv_std, __nv_bfloat16 *xb, float *tb) {
  const int b = blockIdx.x;
  if (b >= batch) return;
  const long long src = idx[b];
  const uint4 *from = reinterpret_cast<const uint4 *>(x + src * in);
  uint4 *to = reinterpret_cast<uint4 *>(xb + static_cast<long long>(b) * in);
  for (int i = threadIdx.x; i < in / 8; i += blockDim.x) to[i] = from[i];
  if (threadIdx.x == 0) tb[b] = (labels[src] - mean) * inv_std;
}

}  // namespace

// ---------------------------------------------------------------------------
cudaError_t MlpForward(const MlpDev &d, const __nv_bfloat16 *x, int batch, MlpWork &w, bool keep_ht,
                       cudaStream_t s) {
  const int M = d.members, H = d.hidden;
  // layer 1, all members at once: Z1 = X W1^T + b1
  GemmArgs g{};
  g.a = x;
  g.b = d.w1h;
  g.m = batch;
  g.n = M * H;
  g.k = d.in;
  g.lda = d.in;
  g.ldb = d.in;
  g.c = w.z1;
  g.bias = d.b1;
  g.h = w.h1;
  g.ht = keep_ht ? w.h1t : nullptr;
  g.ldc = g.ldh = M * H;
  g.ldt = batch;
  cudaError_t err = Gemm<kEpiBiasGelu>(d, g, 1, s);
  if (err != cudaSuccess) return err;
  // layer 2, member z: Z2[:, zH:(z+1)H] = H1[:, zH:(z+1)H] W2[z]^T + b2[z]
  GemmArgs g2{};
  g2.a = w.h1;
  g2.b = d.w2h;
  g2.m = batch;
  g2.n = H;
  g2.k = H;
  g2.lda = M * H;
  g2.ldb = H;
  g2.stride_a = H;
  g2.stride_b = static_cast<long long>(H) * H;
  g2.c = w.z2;
  g2.bias = d.b2;
  g2.h = w.h2;
  g2.ldc = g2.ldh = M * H;
  g2.stride_c = g2.stride_h = H;
  g2.stride_bias = H;
  err = Gemm<kEpiBiasGelu>(d, g2, M, s);
  if (err != cudaSuccess) return err;
  const int warps = batch * M;
  output_kernel<<<(warps * 32 + 255) / 256, 256, 0, s>>>(w.h2, d.w3, d.b3, batch, M, H, w.y);
  return cudaGetLastError();
}

cudaError_t MlpBackward(const MlpDev &d, const __nv_bfloat16 *x, const __nv_bfloat16 *xt, const float *t, int batch,
                        MlpWork &w, float *grad, float *loss, cudaStream_t s) {
  const int M = d.members, H = d.hidden;
  const long long n1 = static_cast<long long>(M) * H * d.in;
  float *gw1 = grad, *gb1 = gw1 + n1, *gw2 = gb1 + M * H, *gb2 = gw2 + static_cast<long long>(M) * H * H;
  float *gw3 = gb2 + M * H, *gb3 = gw3 + M * H;
  const long long total = static_cast<long long>(batch) * M * H;
  output_backward_kernel<<<static_cast<int>((total + 255) / 256), 256, 0, s>>>(w.y, t, w.z2, d.w3, batch, M, H,
                                                                               w.dz2, w.dz2t, loss);
  output_param_grad_kernel<<<M * H, 256, 0, s>>>(w.y, t, w.h2, batch, M, H, gw3, gb3);
  // gW2[z] = dZ2[:, z]^T H1[:, z]  ([H][B] x [H][B]^T)
  GemmArgs g{};
  g.a = w.dz2t;
  g.b = w.h1t;
  g.m = H;
  g.n = H;
  g.k = batch;
  g.lda = g.ldb = batch;
  g.stride_a = g.stride_b = static_cast<long long>(H) * batch;
  g.c = gw2;
  g.ldc = H;
  g.stride_c = static_cast<long long>(H) * H;
  g.alpha = 1.f;
  cudaError_t err = Gemm<kEpiStoreF32>(d, g, M, s);
  if (err != cudaSuccess) return err;
  column_sum_kernel<<<M * H, 256, 0, s>>>(w.dz2t, batch, gb2);
  // dZ1[:, z] = (dZ2[:, z] W2[z]) * GELU'(Z1): B operand W2[z]^T stored [in][out]
  GemmArgs g2{};
  g2.a = w.dz2;
  g2.b = d.w2t;
  g2.m = batch;
  g2.n = H;
  g2.k = H;
  g2.lda = M * H;
  g2.ldb = H;
  g2.stride_a = H;
  g2.stride_b = static_cast<long long>(H) * H;
  g2.c = w.z1;
  g2.h = w.dz1;
  g2.ht = w.dz1t;
  g2.ldc = g2.ldh = M * H;
  g2.ldt = batch;
  g2.stride_c = g2.stride_h = H;
  g2.stride_ht = static_cast<long long>(H) * batch;
  err = Gemm<kEpiGeluGrad>(d, g2, M, s);
  if (err != cudaSuccess) return err;
  column_sum_kernel<<<M * H, 256, 0, s>>>(w.dz1t, batch, gb1);
  // gW1 = dZ1^T X  ([M*H][B] x [K][B]^T)
  GemmArgs g3{};
  g3.a = w.dz1t;
  g3.b = xt;
  g3.m = M * H;
  g3.n = d.in;
  g3.k = batch;
  g3.lda = g3.ldb = batch;
  g3.c = gw1;
  g3.ldc = d.in;
  g3.alpha = 1.f;
  return Gemm<kEpiStoreF32>(d, g3, 1, s);
}

cudaError_t MlpGather(const __nv_bfloat16 *x, const float *labels, const int *idx, int batch, int in, float mean,
                      float inv_std, __nv_bfloat16 *xb, float *tb, cudaStream_t s) {
  if (in % 8) return cudaErrorInvalidValue;
  gather_kernel<<<batch, 64, 0, s>>>(x, labels, idx, batch, in, mean, inv_std, xb, tb);
  return cudaGetLastError();
}

cudaError_t MlpTranspose(const __nv_bfloat16 *in, int rows, int cols, __nv_bfloat16 *out, cudaStream_t s) {
  const dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  transpose_bf16_kernel<<<grid, dim3(32, 8), 0, s>>>(in, rows, cols, out);
  return cudaGetLastError();
}

cudaError_t MlpAdam(float *p, const float *grad, float *m1, float *m2, long long n, float lr, int step,
                    cudaStream_t s) {
  const float beta1 = 0.9f, beta2 = 0.999f;
  const float c1 = 1.f - powf(beta1, static_cast<float>(step)), c2 = 1.f - powf(beta2, static_cast<float>(step));
  adam_kernel<<<static_cast<int>((n + 255) / 256), 256, 0, s>>>(p, grad, m1, m2, n, lr, beta1, beta2, 1e-8f, c1, c2);
  return cudaGetLastError();
}

cudaError_t MlpCastWeights(const MlpDev &d, cudaStream_t s) {
  const long long n1 = static_cast<long long>(d.members) * d.hidden * d.in;
  const long long n2 = static_cast<long long>(d.members) * d.hidden * d.hidden;
  const long long n = n1 > n2 ? n1 : n2;
  cast_weights_kernel<<<static_cast<int>((n + 255) / 256), 256, 0, s>>>(d.w1, n1, d.w2, d.members, d.hidden, d.w1h,
                                                                        d.w2h, d.w2t);
  // hidden 128 with 128 or 192 inputs: the fused jump kernel's tiles, W1, b1, W2 and b2 halved (exact)
  const bool fused_shape = (d.in == 128 || d.in == 192) && d.hidden == 128;
  const float scale = fused_shape ? 0.5f : 1.0f;
  if (d.w1_tiles && (d.hidden % 256 == 0 || d.hidden == 128) && d.in % 32 == 0) {
    const int block_rows = d.hidden == 128 ? 128 : 256;
    tile_weights_kernel<__nv_bfloat16><<<static_cast<int>((n1 + 255) / 256), 256, 0, s>>>(
        d.w1, static_cast<long long>(d.members) * d.hidden, d.in, block_rows, scale, d.w1_tiles);
    tile_weights_kernel<__half><<<static_cast<int>((n2 + 255) / 256), 256, 0, s>>>(
        d.w2, static_cast<long long>(d.members) * d.hidden, d.hidden, block_rows, scale, d.w2_tiles);
  }
  if (d.b2h && d.w3h) {
    const int nh = d.members * d.hidden;
    fused_extras_kernel<<<(nh + 255) / 256, 256, 0, s>>>(d.b1, d.b2, d.w3, nh,
                                                         fused_shape && d.w1_tiles ? d.in / 32 : 0, scale, d.b2h,
                                                         d.w3h, d.w1_tiles);
  }
  return cudaGetLastError();
}

cudaError_t MlpEnsemble(const float *y, int batch, int members, float mean_label, float std_label, float *mean,
                        float *spread, cudaStream_t s) {
  ensemble_kernel<<<(batch + 255) / 256, 256, 0, s>>>(y, batch, members, mean_label, std_label, mean, spread);
  return cudaGetLastError();
}

}  // namespace lmc
