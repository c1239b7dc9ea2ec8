// BF16 tensor-core kernels for the threshold-proposal MLP (sm_103a).
//
// dgb_mlp_gemm: C[M,N] = A[M,K] B[K,N] with BF16 operands and FP32
// accumulation.  K-major products with M % 128 == 0, N % 256 == 0, K % 64 == 0
// and K <= 256 (the 256-wide hidden layers) run on the tcgen05 + TMA kernel of
// mlp_tc.cu; every other shape (K = 4 input layer, N = 1 output layer, the
// strided weight-gradient products) runs on the kernel below, which reads
// operands through arbitrary element strides (X, X^T, W, W^T, dY without
// transposed copies) on mma.sync.m16n8k16.  Both apply the same fused
// epilogue:
//   EPI_PLAIN      out32 = acc
//   EPI_BIAS       out32 = acc + bias
//   EPI_BIAS_GELU  out32 = z = acc + bias, out16 = bf16(gelu(z))
//   EPI_GELU_GRAD  out16 = bf16(acc * gelu'(aux[m,n])), out32 = the same in FP32
// GELU is the exact erf form, 0.5 z (1 + erf(z / sqrt 2)).
// Block tile 64x64, K tile 32, four warps of 32x32 each.
#include <cuda_bf16.h>

#include "common.cuh"

namespace dgb {

enum { EPI_PLAIN = 0, EPI_BIAS = 1, EPI_BIAS_GELU = 2, EPI_GELU_GRAD = 3 };

// tcgen05 + TMA kernel for K-major products (mlp_tc.cu)
bool mlp_gemm_tc_eligible(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam,
                          int64_t sak, const void* B, int64_t sbk, int64_t sbn);
bool mlp_gemm_tc_aligned(const void* bias, const void* aux, const void* out32, const void* out16);
int mlp_gemm_tc(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam, const void* B,
                int64_t sbn, const float* bias, int32_t epi, const float* aux, float* out32,
                void* out16, cudaStream_t st);

constexpr int TM = 64, TN = 64, TK = 32, PAD = 8;

__device__ __forceinline__ float gelu_f(float z) {
  return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad_f(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) +
         z * 0.3989422804014327f * expf(-0.5f * z * z);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(128) gemm_bf16_kernel(
    int M, int N, int K, const __nv_bfloat16* __restrict__ A, int64_t sam, int64_t sak,
    const __nv_bfloat16* __restrict__ B, int64_t sbk, int64_t sbn,
    const float* __restrict__ bias, int epi, const float* __restrict__ aux,
    float* __restrict__ out32, __nv_bfloat16* __restrict__ out16) {
  __shared__ __align__(16) __nv_bfloat16 As[TM][TK + PAD];  // [m][k]
  __shared__ __align__(16) __nv_bfloat16 Bs[TN][TK + PAD];  // [n][k]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < K; k0 += TK) {
    for (int e = tid; e < TM * TK; e += 128) {
      const int r = e / TK, c = e % TK;
      const int m = m0 + r, k = k0 + c;
      As[r][c] = (m < M && k < K) ? A[(int64_t)m * sam + (int64_t)k * sak] : zero;
    }
    for (int e = tid; e < TN * TK; e += 128) {
      const int r = e / TK, c = e % TK;
      const int n = n0 + r, k = k0 + c;
      Bs[r][c] = (n < N && k < K) ? B[(int64_t)k * sbk + (int64_t)n * sbn] : zero;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16 + g;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * t]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * t]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * t + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + j * 8 + g;
        bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * t]);
        bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int m = m0 + wm + i * 16 + g + (q >= 2 ? 8 : 0);
        const int n = n0 + wn + j * 8 + 2 * t + (q & 1);
        if (m >= M || n >= N) continue;
        const int64_t o = (int64_t)m * N + n;
        float v = acc[i][j][q];
        if (epi == EPI_BIAS || epi == EPI_BIAS_GELU) v += bias[n];
        if (epi == EPI_BIAS_GELU) {
          out32[o] = v;
          out16[o] = __float2bfloat16(gelu_f(v));
        } else if (epi == EPI_GELU_GRAD) {
          const float dz = v * gelu_grad_f(aux[o]);
          if (out32) out32[o] = dz;
          out16[o] = __float2bfloat16(dz);
        } else {
          out32[o] = v;
          if (out16) out16[o] = __float2bfloat16(v);
        }
      }
}

// out[n] = sum_m x[m, n], one block per 32 columns, fixed summation order.
__global__ void colsum_kernel(int M, int N, const float* __restrict__ x, float* __restrict__ out) {
  __shared__ float part[8][33];
  const int c = blockIdx.x * 32 + (threadIdx.x & 31);
  const int row = threadIdx.x >> 5;  // 8 row groups
  float s = 0.f;
  if (c < N)
    for (int m = row; m < M; m += 8) s += x[(int64_t)m * N + c];
  part[row][threadIdx.x & 31] = s;
  __syncthreads();
  if (row == 0 && c < N) {
    float tot = 0.f;
    for (int r = 0; r < 8; ++r) tot += part[r][threadIdx.x & 31];
    out[c] = tot;
  }
}

// Adam step on FP32 master weights w[K*N] (row-major [K][N]); refreshes the
// BF16 copies w16 = [K][N] and wt16 = [N][K] when given.
__global__ void adam_kernel(int64_t n_el, int N, float* __restrict__ w, const float* __restrict__ gr,
                            float* __restrict__ m1, float* __restrict__ m2, float lr, float b1,
                            float b2, float eps, float c1, float c2,
                            __nv_bfloat16* __restrict__ w16, __nv_bfloat16* __restrict__ wt16,
                            int K) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_el) return;
  const float g = gr[i];
  const float a = b1 * m1[i] + (1.f - b1) * g;
  const float b = b2 * m2[i] + (1.f - b2) * g * g;
  m1[i] = a;
  m2[i] = b;
  const float wn = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
  w[i] = wn;
  if (w16) w16[i] = __float2bfloat16(wn);
  if (wt16) {
    const int64_t k = i / N, n = i % N;
    wt16[n * K + k] = __float2bfloat16(wn);
  }
}

// dy = scale * (y - target) for the mean-squared-error loss
__global__ void mse_grad_kernel(int64_t n, const float* __restrict__ y, const float* __restrict__ tgt,
                                float scale, float* __restrict__ dy32,
                                __nv_bfloat16* __restrict__ dy16) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float d = scale * (y[i] - tgt[i]);
  if (dy32) dy32[i] = d;
  if (dy16) dy16[i] = __float2bfloat16(d);
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_mlp_gemm(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam,
                            int64_t sak, const void* B, int64_t sbk, int64_t sbn,
                            const float* bias, int32_t epi, const float* aux, float* out32,
                            void* out16, void* stream) {
  clear_error();
  DGB_REQUIRE(M >= 0 && N >= 0 && K >= 0, "sizes must be >= 0");
  DGB_REQUIRE(epi >= EPI_PLAIN && epi <= EPI_GELU_GRAD, "unknown epilogue %d", epi);
  if (M == 0 || N == 0) return DGB_OK;
  DGB_REQUIRE(A && B, "A and B must be non-null");
  DGB_REQUIRE(epi == EPI_PLAIN || epi == EPI_GELU_GRAD || bias, "bias required");
  DGB_REQUIRE(epi != EPI_BIAS_GELU || (out32 && out16), "gelu epilogue needs out32 and out16");
  DGB_REQUIRE(epi != EPI_GELU_GRAD || (aux && out16), "gelu-grad epilogue needs aux and out16");
  DGB_REQUIRE(epi == EPI_GELU_GRAD || out32, "out32 must be non-null");
  if (mlp_gemm_tc_eligible(M, N, K, A, sam, sak, B, sbk, sbn) &&
      mlp_gemm_tc_aligned(bias, aux, out32, out16))
    return mlp_gemm_tc(M, N, K, A, sam, B, sbn, bias, epi, aux, out32, out16, as_stream(stream));
  dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM);
  gemm_bf16_kernel<<<grid, 128, 0, as_stream(stream)>>>(
      M, N, K, (const __nv_bfloat16*)A, sam, sak, (const __nv_bfloat16*)B, sbk, sbn, bias, epi,
      aux, out32, (__nv_bfloat16*)out16);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_colsum(int32_t M, int32_t N, const float* x, float* out, void* stream) {
  clear_error();
  DGB_REQUIRE(M >= 0 && N >= 0 && x && out, "bad arguments");
  if (N == 0) return DGB_OK;
  colsum_kernel<<<(N + 31) / 32, 256, 0, as_stream(stream)>>>(M, N, x, out);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_adam(int64_t n, int32_t N, int32_t K, float* w, const float* grad, float* m1,
                        float* m2, float lr, float b1, float b2, float eps, int32_t step,
                        void* w16, void* wt16, void* stream) {
  clear_error();
  DGB_REQUIRE(n >= 0 && w && grad && m1 && m2 && step >= 1, "bad arguments");
  DGB_REQUIRE(!wt16 || (int64_t)N * K == n, "wt16 needs n == N*K");
  if (n == 0) return DGB_OK;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(
      n, N, w, grad, m1, m2, lr, b1, b2, eps, c1, c2, (__nv_bfloat16*)w16,
      (__nv_bfloat16*)wt16, K);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_mse_grad(int64_t n, const float* y, const float* target, float scale,
                            float* dy32, void* dy16, void* stream) {
  clear_error();
  DGB_REQUIRE(n >= 0 && y && target && (dy32 || dy16), "bad arguments");
  if (n == 0) return DGB_OK;
  mse_grad_kernel<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(
      n, y, target, scale, dy32, (__nv_bfloat16*)dy16);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}
