// Learned SNR screen: a small MLP that predicts ln(network SNR) of an event from its parameters,
// trained on SNRs that the exact kernels produce. Everything runs on the GPU: feature map, GEMM
// forward and backward passes with fused bias / SiLU epilogues, mean-squared-error loss, Adam.
// Weights are kept in FP32 (the optimiser's copy) and used in BF16 by both passes; all arithmetic
// accumulates in FP32. The hidden-to-hidden layers (both widths multiples of 16, at most 256) run on
// the tensor cores (gwf_umma.cuh: tcgen05.mma kind::f16, FP32 accumulation in tensor memory): their
// forward product, weight gradient and input gradient take BF16 operands, i.e. the activations and
// back-propagated gradients are rounded to BF16 where they enter those products. The input layer
// (11 features) and the output layer (width 1) run on the CUDA cores in FP32 with BF16 weights.
//
// Layout: layer l maps A_l [batch][K_l] to Z_l = A_l W_l + b_l, W_l [K_l][M_l] row-major;
// A_{l+1} = SiLU(Z_l) for the hidden layers, the last layer (M = 1) is linear.
//
// Feature map (11 inputs, standardised with the training set's mean and deviation):
//   ln Mc, eta, ln dL, cos theta, sin(phi - 2 pi tcoal), cos(phi - 2 pi tcoal), cos iota,
//   sin 2 psi, cos 2 psi, chi1z, chi2z
// (phi - 2 pi tcoal is the right ascension relative to the sidereal angle at coalescence, the only
// way phi and tcoal enter the SNR; Phicoal does not enter it).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "gwf_launch.h"
#include "gwf_umma.cuh"
#include "gwfast_gb300.h"

namespace gwf {
void set_last_error(const char* msg);  // gwf_api.cu
int ctx_device(const gwf_ctx* ctx);    // gwf_api.cu
}

namespace {

constexpr int kNF = 11;   // features
constexpr int kT = 64;    // GEMM tile (rows and columns)
constexpr int kTK = 16;   // GEMM tile depth

int fail(int code, const std::string& msg) {
  gwf::set_last_error(msg.c_str());
  return code;
}

#define MLP_CK(x)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (x);                                                                        \
    if (e_ != cudaSuccess) return fail(GWF_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// ---------------------------------------------------------------- kernels
__global__ void features_kernel(const double* __restrict__ p, long long ld, long long n, const float* __restrict__ mean,
                                const float* __restrict__ inv_std, float* __restrict__ X) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double tp = 6.283185307179586;
  const double ra = p[4 * ld + i] - tp * p[7 * ld + i];
  double f[kNF];
  f[0] = log(p[0 * ld + i]);
  f[1] = p[1 * ld + i];
  f[2] = log(p[2 * ld + i]);
  f[3] = cos(p[3 * ld + i]);
  f[4] = sin(ra);
  f[5] = cos(ra);
  f[6] = cos(p[5 * ld + i]);
  f[7] = sin(2.0 * p[6 * ld + i]);
  f[8] = cos(2.0 * p[6 * ld + i]);
  f[9] = p[9 * ld + i];
  f[10] = p[10 * ld + i];
  for (int k = 0; k < kNF; ++k) X[i * kNF + k] = (float)f[k];
  if (mean)
    for (int k = 0; k < kNF; ++k) X[i * kNF + k] = (X[i * kNF + k] - mean[k]) * inv_std[k];
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

template <class T> __device__ __forceinline__ float ld_f(const T* p, long long i);
template <> __device__ __forceinline__ float ld_f<float>(const float* p, long long i) { return p[i]; }
template <> __device__ __forceinline__ float ld_f<__nv_bfloat16>(const __nv_bfloat16* p, long long i) {
  return __bfloat162float(p[i]);
}

// C[m][n] = sum_k A(m, k) B(k, n) (+ bias[n]), A(m, k) = TA ? A[k lda + m] : A[m lda + k],
// B(k, n) = TB ? B[n ldb + k] : B[k ldb + n]. act: 0 none, 1 SiLU (Zout, if given, gets the
// pre-activation). 64 x 64 tile per block of 256 threads, 4 x 4 outputs per thread, FP32 sums.
template <bool TA, bool TB, class TBE>
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const float* __restrict__ A, int lda,
                                                   const TBE* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                                   const float* __restrict__ bias, int act, float* __restrict__ Zout) {
  __shared__ float As[kTK][kT + 1];
  __shared__ float Bs[kTK][kT + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * kT, n0 = blockIdx.x * kT;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
  for (int k0 = 0; k0 < K; k0 += kTK) {
    for (int e = threadIdx.x; e < kTK * kT; e += 256) {
      const int kk = e / kT, mm = e % kT;
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? (TA ? A[(long long)gk * lda + gm] : A[(long long)gm * lda + gk]) : 0.0f;
      const int gn = n0 + mm;
      Bs[kk][mm] = (gn < N && gk < K) ? (TB ? ld_f(B, (long long)gn * ldb + gk) : ld_f(B, (long long)gk * ldb + gn))
                                      : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float z = acc[i][j] + (bias ? bias[gn] : 0.0f);
      if (Zout) Zout[(long long)gm * ldc + gn] = z;
      C[(long long)gm * ldc + gn] = act == 1 ? silu(z) : z;
    }
  }
}

// dZ = dA * SiLU'(Z)
__global__ void silu_bwd_kernel(const float* __restrict__ dA, const float* __restrict__ Z, float* __restrict__ dZ,
                                long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dZ[i] = dA[i] * silu_grad(Z[i]);
}

// db[j] = sum_b dZ[b][j]
__global__ void colsum_kernel(const float* __restrict__ dZ, int B, int M, float* __restrict__ db) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  float s = 0.0f;
  for (int b = 0; b < B; ++b) s += dZ[(long long)b * M + j];
  db[j] = s;
}

// mean squared error of y against t over the batch: dY = 2 (y - t) / B, loss accumulated in FP64
__global__ void mse_kernel(const float* __restrict__ y, const float* __restrict__ t, int B, float* __restrict__ dY,
                           double* __restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (i < B) {
    const float d = y[i] - t[i];
    dY[i] = 2.0f * d / (float)B;
    v = (double)d * d / B;
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (loss && (threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(loss, v);
}

// minibatch gather: rows of X and targets at hashed indices (sampling with replacement)
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__global__ void gather_batch_kernel(const float* __restrict__ X, const float* __restrict__ T, long long n, int B,
                                    unsigned long long seed, unsigned long long step, float* __restrict__ Xb,
                                    float* __restrict__ Tb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const long long r = (long long)(mix64(seed ^ mix64(step * 1315423911ull + (unsigned long long)i)) % (unsigned long long)n);
  for (int k = 0; k < kNF; ++k) Xb[(long long)i * kNF + k] = X[r * kNF + k];
  Tb[i] = T[r];
}

// Adam on the FP32 weights; refreshes their BF16 copy
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                            float c2, __nv_bfloat16* __restrict__ wbf) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (wbf) wbf[i] = __float2bfloat16_rn(wi);
}

__global__ void to_bf16_kernel(const float* __restrict__ w, long long n, __nv_bfloat16* __restrict__ wbf) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wbf[i] = __float2bfloat16_rn(w[i]);
}

__global__ void to_double_kernel(const float* __restrict__ y, long long n, double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)y[i];
}

__global__ void to_float_kernel(const double* __restrict__ y, long long n, float* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)y[i];
}

// ---------------------------------------------------------------- fused inference on the tensor cores
// One CTA of 128 threads per 128 events; thread t owns event (and tensor-memory lane) t of the tile.
// The features and the input layer (11 -> H, FP32 with BF16 weights) run on the CUDA cores and leave
// the activations, rounded to BF16, in shared memory in the K-major core-matrix layout. Each
// hidden-to-hidden layer is one 128 x H x H product into tensor memory (its weights staged in 64-deep
// K chunks), read back by the epilogue, which applies bias and SiLU and writes the next layer's
// operand in place; the last epilogue feeds the output layer's dot product (FP32) directly, so no
// activation leaves the chip. Same arithmetic as the layer-by-layer forward pass up to the order of
// the FP32 sums.
constexpr int kMaxLayers = 17;
struct InferNet {
  int L, H;                    // layers (weight matrices) and hidden width
  long long woff[kMaxLayers];  // offsets of W_l (BF16 copy) and b_l (FP32) in the flat layout
  long long boff[kMaxLayers];
};

__host__ __device__ constexpr int infer_smem_bytes() { return 64 * 1024 + 32 * 1024 + 1024; }

__global__ void __launch_bounds__(128, 1) mlp_infer_tc_kernel(const double* __restrict__ p, long long ld, long long n,
                                                             const float* __restrict__ norm, InferNet net,
                                                             const __nv_bfloat16* __restrict__ wbf,
                                                             const float* __restrict__ w32, double* __restrict__ out,
                                                             int* __restrict__ err) {
  using namespace gwf::umma;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* sa = smem_raw;               // activations: 128 x H BF16, [row/8][k/8] core matrices
  unsigned char* sb = smem_raw + 64 * 1024;   // weights: H x 64 BF16 chunk, [n/8][k/8]
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  const int H = net.H, L = net.L;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const long long row = (long long)blockIdx.x * 128 + t;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (t == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // features of this thread's event, standardised (zero for rows past n)
  float x[kNF];
  {
    double f[kNF];
    if (row < n) {
      const double tp = 6.283185307179586;
      const double ra = p[4 * ld + row] - tp * p[7 * ld + row];
      f[0] = log(p[row]); f[1] = p[ld + row]; f[2] = log(p[2 * ld + row]); f[3] = cos(p[3 * ld + row]);
      f[4] = sin(ra); f[5] = cos(ra); f[6] = cos(p[5 * ld + row]); f[7] = sin(2.0 * p[6 * ld + row]);
      f[8] = cos(2.0 * p[6 * ld + row]); f[9] = p[9 * ld + row]; f[10] = p[10 * ld + row];
    }
#pragma unroll
    for (int k = 0; k < kNF; ++k) x[k] = row < n ? ((float)f[k] - norm[k]) * norm[kNF + k] : 0.0f;
  }
  const int kb = H / 8;                         // core matrices along K of the activation buffer
  float y = 0.0f;                               // output layer, accumulated by the last epilogue
  const float* wl = w32 + net.woff[L - 1];      // output weights (FP32 copy rounded as BF16 below)
  const __nv_bfloat16* wlb = wbf + net.woff[L - 1];
  // input layer on the CUDA cores: 8 columns at a time into one 16-byte core-matrix row
  {
    const __nv_bfloat16* W0 = wbf + net.woff[0];
    const float* b0 = w32 + net.boff[0];
    for (int j0 = 0; j0 < H; j0 += 8) {
      float a[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        float z = b0[j0 + j];
#pragma unroll
        for (int k = 0; k < kNF; ++k) z = fmaf(x[k], __bfloat162float(W0[k * H + j0 + j]), z);
        a[j] = silu_f(z);
      }
      if (L == 2) {
#pragma unroll
        for (int j = 0; j < 8; ++j) y = fmaf(a[j], __bfloat162float(wlb[j0 + j]), y);
      } else {
        *reinterpret_cast<uint4*>(sa + ((t >> 3) * kb + (j0 >> 3)) * 128 + (t & 7) * 16) =
            make_uint4(pack_bf16(a[0], a[1]), pack_bf16(a[2], a[3]), pack_bf16(a[4], a[5]), pack_bf16(a[6], a[7]));
      }
    }
  }
  (void)wl;
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tm = tmem_base;
  const uint32_t idesc = instr_desc(128, H);
  bool ok = true;
  uint32_t phase = 0;
  for (int l = 1; l <= L - 2 && ok; ++l) {
    const __nv_bfloat16* W = wbf + net.woff[l];   // [H][H] row-major: element (k, n) at k H + n
    for (int c = 0; c < H / 64 && ok; ++c) {
      // weights of K rows [64 c, 64 c + 64) as the MMA's B operand (n rows, K-major)
      for (int u = t; u < H * 8; u += 128) {
        const int nn = u % H, kg = u / H;
        uint32_t q[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const __nv_bfloat16 lo = W[(long long)(c * 64 + kg * 8 + 2 * j) * H + nn];
          const __nv_bfloat16 hi = W[(long long)(c * 64 + kg * 8 + 2 * j + 1) * H + nn];
          q[j] = (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
        }
        *reinterpret_cast<uint4*>(sb + ((nn >> 3) * 8 + kg) * 128 + (nn & 7) * 16) = make_uint4(q[0], q[1], q[2], q[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (t == 0) {
        fence_after_sync();
        const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
        for (int s = 0; s < 4; ++s)
          mma_f16(tm, smem_desc(a0 + (c * 8 + s * 2) * 128, 128, kb * 128), smem_desc(b0 + s * 2 * 128, 128, 8 * 128),
                  idesc, (c > 0 || s > 0) ? 1u : 0u);
        mma_commit(&bar);
      }
      ok = __syncthreads_and(mbar_wait(&bar, phase)) != 0;
      if (!ok) {
        if (t == 0) {
          atomicExch(err, 1);
          mbar_wait(&bar, phase);
        }
        __syncthreads();
      }
      phase ^= 1u;
      fence_after_sync();
    }
    if (!ok) break;
    // epilogue: bias and SiLU; the next layer's operand in place, or the output layer's dot product
    const float* bl = w32 + net.boff[l];
    const bool last = l == L - 2;
    for (int c0 = 0; c0 < H; c0 += 16) {
      float v[16];
      tmem_ld16(tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = silu_f(v[j] + bl[c0 + j]);
      if (last) {
#pragma unroll
        for (int j = 0; j < 16; ++j) y = fmaf(v[j], __bfloat162float(wlb[c0 + j]), y);
      } else {
#pragma unroll
        for (int h = 0; h < 2; ++h)
          *reinterpret_cast<uint4*>(sa + ((t >> 3) * kb + ((c0 >> 3) + h)) * 128 + (t & 7) * 16) =
              make_uint4(pack_bf16(v[8 * h + 0], v[8 * h + 1]), pack_bf16(v[8 * h + 2], v[8 * h + 3]),
                         pack_bf16(v[8 * h + 4], v[8 * h + 5]), pack_bf16(v[8 * h + 6], v[8 * h + 7]));
      }
    }
    fence_before_sync();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    fence_after_sync();
  }
  if (ok && row < n) out[row] = (double)(y + w32[net.boff[L - 1]]);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tm) : "memory");
}

struct Buf {
  void* p = nullptr;
  size_t cap = 0;
  bool ensure(size_t b) {
    if (b <= cap) return true;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    if (cudaMalloc(&p, b) != cudaSuccess) return false;
    cap = b;
    return true;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

struct gwf_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<int> dims;        // {11, H, ..., H, 1}
  std::vector<long long> woff;  // offsets of W_l in the flat parameter vector; biases follow all weights
  std::vector<long long> boff;
  long long nw = 0;             // weights + biases
  Buf w32, wbf, grad, adam_m, adam_v, norm;   // norm: mean[11], inv_std[11]
  Buf X, T, xb, tb, dy, loss, pred;            // data, batch, loss
  std::vector<Buf> act, pre, dact;             // per layer activations, pre-activations, gradients
  Buf tc_err;                                  // set by a tensor-core GEMM whose MMA wait timed out
  Buf tc_ws;                                   // split-K partial sums of the tensor-core weight gradients
  long long adam_t = 0;
  bool have_norm = false;
};

namespace {

template <class TBE, bool TA, bool TB>
cudaError_t gemm(cudaStream_t st, int M, int N, int K, const float* A, int lda, const TBE* B, int ldb, float* C, int ldc,
                 const float* bias, int act, float* Z) {
  dim3 grid(nblk(N, kT), nblk(M, kT));
  gemm_kernel<TA, TB, TBE><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, Z);
  return cudaGetLastError();
}

// C = op(A) op(B) (+ bias, SiLU) on the tensor cores (N a multiple of 16, at most 256). A long
// reduction (K well above the tile's rows, the weight gradients over a batch) with few row tiles is
// split over K into `ws` (splits x M x N floats, contiguous C with ldc = N, no bias or activation)
// and reduced in split order.
template <class TBE, bool TA, bool TB>
cudaError_t gemm_tc(cudaStream_t st, int M, int N, int K, const float* A, int lda, const TBE* B, int ldb, float* C,
                    int ldc, const float* bias, int act, float* Z, int* err, Buf* ws = nullptr) {
  auto k = gwf::umma::gemm_tc_kernel<TA, TB, TBE>;
  const int smem = gwf::umma::smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const unsigned mt = nblk(M, gwf::umma::kUM);
  int splits = 1;
  if (ws && !bias && act == 0 && !Z && ldc == N && mt < 32 && K >= 4 * gwf::umma::kUK) {
    splits = (int)std::min<long long>(64 / mt, (K + 2 * gwf::umma::kUK - 1) / (2 * gwf::umma::kUK));
    if (splits < 1) splits = 1;
  }
  if (splits > 1) {
    const int kspan = (int)((((long long)K + splits - 1) / splits + gwf::umma::kUK - 1) / gwf::umma::kUK) * gwf::umma::kUK;
    splits = (K + kspan - 1) / kspan;
    if (!ws->ensure((size_t)splits * M * N * sizeof(float))) return cudaErrorMemoryAllocation;
    k<<<dim3(mt, (unsigned)splits), 128, smem, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, Z, kspan,
                                                   ws->as<float>(), err);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    gwf::umma::splitk_reduce_kernel<<<nblk((long long)M * N, 256), 256, 0, st>>>(ws->as<float>(), splits,
                                                                                 (long long)M * N, C);
    return cudaGetLastError();
  }
  k<<<dim3(mt, 1), 128, smem, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act, Z, K, nullptr, err);
  return cudaGetLastError();
}

int n_layers(const gwf_mlp* m) { return (int)m->dims.size() - 1; }

// the hidden-to-hidden layers run on the tensor cores
bool tc_layer(const gwf_mlp* m, int l) {
  const int L = n_layers(m), K = m->dims[l], M = m->dims[l + 1];
  return l >= 1 && l <= L - 2 && K % 16 == 0 && M % 16 == 0 && M <= gwf::umma::kUNMax;
}

// report a tensor-core GEMM whose wait for its MMAs gave up (waits on the stream)
int check_tc(gwf_mlp* m) {
  int v = 0;
  MLP_CK(cudaMemcpyAsync(&v, m->tc_err.p, sizeof v, cudaMemcpyDeviceToHost, m->stream));
  MLP_CK(cudaStreamSynchronize(m->stream));
  if (v) return fail(GWF_ERR_TIMEOUT, "MLP tensor-core GEMM: MMA completion wait timed out");
  return GWF_OK;
}

// forward pass over rows [0, B) of X (features); with train, the activations and pre-activations are kept
int forward(gwf_mlp* m, const float* X, int B, float* out, bool train) {
  const int L = n_layers(m);
  const float* a = X;
  for (int l = 0; l < L; ++l) {
    const int K = m->dims[l], M = m->dims[l + 1];
    const bool last = l == L - 1;
    if (!m->act[l + 1].ensure((size_t)B * M * sizeof(float)) || (train && !m->pre[l].ensure((size_t)B * M * sizeof(float))))
      return fail(GWF_ERR_OOM, "device allocation failed (MLP activations)");
    float* o = last && out ? out : m->act[l + 1].as<float>();
    const __nv_bfloat16* W = m->wbf.as<__nv_bfloat16>() + m->woff[l];
    const float* b = m->w32.as<float>() + m->boff[l];
    if (tc_layer(m, l))
      MLP_CK((gemm_tc<__nv_bfloat16, false, false>(m->stream, B, M, K, a, K, W, M, o, M, b, last ? 0 : 1,
                                                   train ? m->pre[l].as<float>() : nullptr, m->tc_err.as<int>())));
    else
      MLP_CK((gemm<__nv_bfloat16, false, false>(m->stream, B, M, K, a, K, W, M, o, M, b, last ? 0 : 1,
                                                 train ? m->pre[l].as<float>() : nullptr)));
    a = o;
  }
  return GWF_OK;
}

// backward pass for the batch in act / pre, loss gradient dY [B]; gradients into m->grad
int backward(gwf_mlp* m, const float* X, int B, const float* dY) {
  const int L = n_layers(m);
  const float* dA = dY;
  for (int l = L - 1; l >= 0; --l) {
    const int K = m->dims[l], M = m->dims[l + 1];
    const bool last = l == L - 1;
    if (!m->dact[l + 1].ensure((size_t)B * M * sizeof(float)) || !m->dact[l].ensure((size_t)B * K * sizeof(float)))
      return fail(GWF_ERR_OOM, "device allocation failed (MLP gradients)");
    float* dZ = m->dact[l + 1].as<float>();
    if (last) {
      MLP_CK(cudaMemcpyAsync(dZ, dA, (size_t)B * M * sizeof(float), cudaMemcpyDeviceToDevice, m->stream));
    } else {
      silu_bwd_kernel<<<nblk((long long)B * M, 256), 256, 0, m->stream>>>(dA, m->pre[l].as<float>(), dZ,
                                                                             (long long)B * M);
      MLP_CK(cudaGetLastError());
    }
    const float* Al = l == 0 ? X : m->act[l].as<float>();
    float* gW = m->grad.as<float>() + m->woff[l];
    float* gb = m->grad.as<float>() + m->boff[l];
    // dW = A_l^T dZ  (K x M, reduction over the batch)
    const bool tc = tc_layer(m, l);
    if (tc)
      MLP_CK((gemm_tc<float, true, false>(m->stream, K, M, B, Al, K, dZ, M, gW, M, nullptr, 0, nullptr,
                                          m->tc_err.as<int>(), &m->tc_ws)));
    else
      MLP_CK((gemm<float, true, false>(m->stream, K, M, B, Al, K, dZ, M, gW, M, nullptr, 0, nullptr)));
    colsum_kernel<<<nblk(M, 128), 128, 0, m->stream>>>(dZ, B, M, gb);
    MLP_CK(cudaGetLastError());
    if (l > 0) {
      // dA_l = dZ W_l^T  (B x K)
      const __nv_bfloat16* W = m->wbf.as<__nv_bfloat16>() + m->woff[l];
      if (tc && K <= gwf::umma::kUNMax)
        MLP_CK((gemm_tc<__nv_bfloat16, false, true>(m->stream, B, K, M, dZ, M, W, M, m->dact[l].as<float>(), K, nullptr,
                                                    0, nullptr, m->tc_err.as<int>())));
      else
        MLP_CK((gemm<__nv_bfloat16, false, true>(m->stream, B, K, M, dZ, M, W, M, m->dact[l].as<float>(), K, nullptr,
                                                  0, nullptr)));
      dA = m->dact[l].as<float>();
    }
  }
  return GWF_OK;
}

// features of n events (params host or device) into m->X; with fit_norm, the standardisation is
// taken from these events first
int load_features(gwf_mlp* m, const double* params, int64_t ld, int64_t n, int mem, bool fit_norm) {
  Buf tmp;
  const double* dp = params;
  int64_t dld = ld;
  if (mem == GWF_MEM_HOST) {
    if (!tmp.ensure((size_t)kNF * n * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed (MLP input)");
    MLP_CK(cudaMemcpy2DAsync(tmp.p, n * sizeof(double), params, ld * sizeof(double), n * sizeof(double), kNF,
                             cudaMemcpyHostToDevice, m->stream));
    dp = tmp.as<double>();
    dld = n;
  }
  if (!m->X.ensure((size_t)n * kNF * sizeof(float))) { tmp.release(); return fail(GWF_ERR_OOM, "device allocation failed (MLP features)"); }
  features_kernel<<<nblk(n, 256), 256, 0, m->stream>>>(dp, dld, n, nullptr, nullptr, m->X.as<float>());
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && fit_norm) {
    std::vector<float> h((size_t)n * kNF);
    e = cudaMemcpyAsync(h.data(), m->X.p, h.size() * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess) {
      float st[2 * kNF];
      for (int k = 0; k < kNF; ++k) {
        double s = 0.0, s2 = 0.0;
        for (int64_t i = 0; i < n; ++i) { const double v = h[i * kNF + k]; s += v; s2 += v * v; }
        const double mu = s / n, var = s2 / n - mu * mu;
        st[k] = (float)mu;
        st[kNF + k] = (float)(var > 1e-20 ? 1.0 / std::sqrt(var) : 1.0);
      }
      if (!m->norm.ensure(sizeof st)) { tmp.release(); return fail(GWF_ERR_OOM, "device allocation failed (MLP)"); }
      e = cudaMemcpyAsync(m->norm.p, st, sizeof st, cudaMemcpyHostToDevice, m->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
      m->have_norm = true;
    }
  }
  if (e == cudaSuccess && m->have_norm)
    features_kernel<<<nblk(n, 256), 256, 0, m->stream>>>(dp, dld, n, m->norm.as<float>(), m->norm.as<float>() + kNF,
                                                          m->X.as<float>());
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  tmp.release();
  if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("MLP features: ") + cudaGetErrorString(e));
  return GWF_OK;
}

int load_targets(gwf_mlp* m, const double* t, int64_t n, int mem) {
  if (!m->T.ensure((size_t)n * sizeof(float))) return fail(GWF_ERR_OOM, "device allocation failed (MLP targets)");
  if (mem == GWF_MEM_HOST) {
    std::vector<float> h((size_t)n);
    for (int64_t i = 0; i < n; ++i) h[i] = (float)t[i];
    MLP_CK(cudaMemcpyAsync(m->T.p, h.data(), (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MLP_CK(cudaStreamSynchronize(m->stream));
  } else {
    to_float_kernel<<<nblk(n, 256), 256, 0, m->stream>>>(t, n, m->T.as<float>());
    MLP_CK(cudaGetLastError());
  }
  return GWF_OK;
}

int check(gwf_mlp* m) {
  if (!m) return fail(GWF_ERR_INVALID_ARG, "null MLP");
  MLP_CK(cudaSetDevice(m->device));
  return GWF_OK;
}

}  // namespace

extern "C" {

int gwf_mlp_create(gwf_ctx* ctx, int hidden, int layers, uint64_t seed, gwf_mlp** out) {
  if (!ctx || !out) return fail(GWF_ERR_INVALID_ARG, "null argument");
  if (hidden < 1 || hidden > 4096 || layers < 1 || layers > 16) return fail(GWF_ERR_INVALID_ARG, "bad MLP shape");
  const int dev = gwf::ctx_device(ctx);
  MLP_CK(cudaSetDevice(dev));
  gwf_mlp* m = new gwf_mlp();
  m->device = dev;
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete m;
    return fail(GWF_ERR_CUDA, "stream creation failed");
  }
  m->dims.push_back(kNF);
  for (int l = 0; l < layers; ++l) m->dims.push_back(hidden);
  m->dims.push_back(1);
  const int L = n_layers(m);
  long long off = 0;
  for (int l = 0; l < L; ++l) { m->woff.push_back(off); off += (long long)m->dims[l] * m->dims[l + 1]; }
  for (int l = 0; l < L; ++l) { m->boff.push_back(off); off += m->dims[l + 1]; }
  m->nw = off;
  m->act.resize(L + 1);
  m->pre.resize(L);
  m->dact.resize(L + 1);
  // initialisation: uniform(-a, a), a = sqrt(6 / fan_in) for SiLU layers, sqrt(3 / fan_in) for the output; zero biases
  std::vector<float> w((size_t)m->nw, 0.0f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < L; ++l) {
    const double a = std::sqrt((l == L - 1 ? 3.0 : 6.0) / m->dims[l]);
    std::uniform_real_distribution<double> u(-a, a);
    for (long long i = 0; i < (long long)m->dims[l] * m->dims[l + 1]; ++i) w[m->woff[l] + i] = (float)u(rng);
  }
  const size_t nb = (size_t)m->nw * sizeof(float);
  bool ok = m->w32.ensure(nb) && m->wbf.ensure((size_t)m->nw * 2) && m->grad.ensure(nb) && m->adam_m.ensure(nb) &&
            m->adam_v.ensure(nb) && m->loss.ensure(sizeof(double)) && m->tc_err.ensure(sizeof(int));
  if (ok) ok = cudaMemcpy(m->w32.p, w.data(), nb, cudaMemcpyHostToDevice) == cudaSuccess &&
               cudaMemset(m->adam_m.p, 0, nb) == cudaSuccess && cudaMemset(m->adam_v.p, 0, nb) == cudaSuccess &&
               cudaMemset(m->tc_err.p, 0, sizeof(int)) == cudaSuccess;
  if (ok) {
    to_bf16_kernel<<<nblk(m->nw, 256), 256, 0, m->stream>>>(m->w32.as<float>(), m->nw, m->wbf.as<__nv_bfloat16>());
    ok = cudaStreamSynchronize(m->stream) == cudaSuccess;
  }
  if (!ok) {
    gwf_mlp_destroy(m);
    return fail(GWF_ERR_OOM, "MLP set-up failed");
  }
  *out = m;
  return GWF_OK;
}

int gwf_mlp_destroy(gwf_mlp* m) {
  if (!m) return GWF_OK;
  cudaSetDevice(m->device);
  cudaStreamSynchronize(m->stream);
  for (Buf* b : {&m->w32, &m->wbf, &m->grad, &m->adam_m, &m->adam_v, &m->norm, &m->X, &m->T, &m->xb, &m->tb, &m->dy,
                 &m->loss, &m->pred, &m->tc_err, &m->tc_ws})
    b->release();
  for (auto* v : {&m->act, &m->pre, &m->dact})
    for (auto& b : *v) b.release();
  cudaStreamDestroy(m->stream);
  delete m;
  return GWF_OK;
}

int gwf_mlp_num_weights(gwf_mlp* m, int64_t* n) {
  int rc = check(m);
  if (rc) return rc;
  if (!n) return fail(GWF_ERR_INVALID_ARG, "null output");
  *n = m->nw;
  return GWF_OK;
}

int gwf_mlp_get_weights(gwf_mlp* m, float* w, float* norm) {
  int rc = check(m);
  if (rc) return rc;
  if (w) MLP_CK(cudaMemcpy(w, m->w32.p, (size_t)m->nw * sizeof(float), cudaMemcpyDeviceToHost));
  if (norm) {
    if (!m->have_norm) return fail(GWF_ERR_INVALID_ARG, "the MLP has no feature standardisation yet");
    MLP_CK(cudaMemcpy(norm, m->norm.p, 2 * kNF * sizeof(float), cudaMemcpyDeviceToHost));
  }
  return GWF_OK;
}

int gwf_mlp_set_weights(gwf_mlp* m, const float* w, const float* norm) {
  int rc = check(m);
  if (rc) return rc;
  if (w) {
    MLP_CK(cudaMemcpy(m->w32.p, w, (size_t)m->nw * sizeof(float), cudaMemcpyHostToDevice));
    to_bf16_kernel<<<nblk(m->nw, 256), 256, 0, m->stream>>>(m->w32.as<float>(), m->nw, m->wbf.as<__nv_bfloat16>());
    MLP_CK(cudaStreamSynchronize(m->stream));
  }
  if (norm) {
    if (!m->norm.ensure(2 * kNF * sizeof(float))) return fail(GWF_ERR_OOM, "device allocation failed (MLP)");
    MLP_CK(cudaMemcpy(m->norm.p, norm, 2 * kNF * sizeof(float), cudaMemcpyHostToDevice));
    m->have_norm = true;
  }
  return GWF_OK;
}

int gwf_mlp_gradients(gwf_mlp* m, const double* params, int64_t ld, int64_t n, const double* target, int mem,
                      double* loss, float* grad) {
  int rc = check(m);
  if (rc) return rc;
  if (!params || !target || n < 1 || n > (1 << 24) || ld < n) return fail(GWF_ERR_INVALID_ARG, "bad arguments");
  rc = load_features(m, params, ld, n, mem, !m->have_norm);
  if (!rc) rc = load_targets(m, target, n, mem);
  if (rc) return rc;
  const int B = (int)n;
  if (!m->pred.ensure((size_t)B * sizeof(float)) || !m->dy.ensure((size_t)B * sizeof(float)))
    return fail(GWF_ERR_OOM, "device allocation failed (MLP)");
  rc = forward(m, m->X.as<float>(), B, m->pred.as<float>(), true);
  if (rc) return rc;
  MLP_CK(cudaMemsetAsync(m->loss.p, 0, sizeof(double), m->stream));
  mse_kernel<<<nblk(B, 256), 256, 0, m->stream>>>(m->pred.as<float>(), m->T.as<float>(), B, m->dy.as<float>(),
                                                  m->loss.as<double>());
  MLP_CK(cudaGetLastError());
  rc = backward(m, m->X.as<float>(), B, m->dy.as<float>());
  if (rc) return rc;
  if (grad) MLP_CK(cudaMemcpyAsync(grad, m->grad.p, (size_t)m->nw * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  double l = 0.0;
  MLP_CK(cudaMemcpyAsync(&l, m->loss.p, sizeof l, cudaMemcpyDeviceToHost, m->stream));
  MLP_CK(cudaStreamSynchronize(m->stream));
  if (loss) *loss = l;
  return check_tc(m);
}

int gwf_mlp_train(gwf_mlp* m, const double* params, int64_t ld, int64_t n, const double* target, int epochs, int batch,
                  double lr, uint64_t seed, int mem, double* final_loss) {
  int rc = check(m);
  if (rc) return rc;
  if (!params || !target || n < 1 || ld < n || epochs < 1 || batch < 1 || batch > (1 << 20) || !(lr > 0.0))
    return fail(GWF_ERR_INVALID_ARG, "bad arguments");
  rc = load_features(m, params, ld, n, mem, true);
  if (!rc) rc = load_targets(m, target, n, mem);
  if (rc) return rc;
  const int B = batch;
  if (!m->xb.ensure((size_t)B * kNF * sizeof(float)) || !m->tb.ensure((size_t)B * sizeof(float)) ||
      !m->pred.ensure((size_t)B * sizeof(float)) || !m->dy.ensure((size_t)B * sizeof(float)))
    return fail(GWF_ERR_OOM, "device allocation failed (MLP batch)");
  const long long spe = (n + B - 1) / B;   // steps per epoch
  const long long steps = (long long)epochs * spe;
  const long long tail0 = steps - spe;      // the last epoch's mean loss is reported
  const float b1 = 0.9f, b2 = 0.999f;
  double last = 0.0;
  for (long long s = 0; s < steps; ++s) {
    gather_batch_kernel<<<nblk(B, 256), 256, 0, m->stream>>>(m->X.as<float>(), m->T.as<float>(), n, B, seed,
                                                             (unsigned long long)s, m->xb.as<float>(), m->tb.as<float>());
    MLP_CK(cudaGetLastError());
    rc = forward(m, m->xb.as<float>(), B, m->pred.as<float>(), true);
    if (rc) return rc;
    const bool tail = s >= tail0;
    if (s == tail0) MLP_CK(cudaMemsetAsync(m->loss.p, 0, sizeof(double), m->stream));
    mse_kernel<<<nblk(B, 256), 256, 0, m->stream>>>(m->pred.as<float>(), m->tb.as<float>(), B, m->dy.as<float>(),
                                                    tail ? m->loss.as<double>() : nullptr);
    MLP_CK(cudaGetLastError());
    rc = backward(m, m->xb.as<float>(), B, m->dy.as<float>());
    if (rc) return rc;
    ++m->adam_t;
    // cosine decay of the learning rate over the run
    const double lr_s = lr * 0.5 * (1.0 + std::cos(M_PI * (double)s / (double)steps));
    const float c1 = 1.0f - std::pow(b1, (float)m->adam_t), c2 = 1.0f - std::pow(b2, (float)m->adam_t);
    adam_kernel<<<nblk(m->nw, 256), 256, 0, m->stream>>>(m->w32.as<float>(), m->grad.as<float>(), m->adam_m.as<float>(),
                                                          m->adam_v.as<float>(), m->nw, (float)lr_s, b1, b2, 1e-8f, c1,
                                                          c2, m->wbf.as<__nv_bfloat16>());
    MLP_CK(cudaGetLastError());
  }
  MLP_CK(cudaMemcpyAsync(&last, m->loss.p, sizeof last, cudaMemcpyDeviceToHost, m->stream));
  MLP_CK(cudaStreamSynchronize(m->stream));
  if (final_loss) *final_loss = last / (double)spe;
  return check_tc(m);
}

int gwf_mlp_predict(gwf_mlp* m, const double* params, int64_t ld, int64_t n, int mem, double* out_ln_snr) {
  int rc = check(m);
  if (rc) return rc;
  if (!params || !out_ln_snr || n < 0 || ld < n) return fail(GWF_ERR_INVALID_ARG, "bad arguments");
  if (!m->have_norm) return fail(GWF_ERR_INVALID_ARG, "the MLP is not trained (no feature standardisation)");
  if (n == 0) return GWF_OK;
  const int L = n_layers(m), H = m->dims[1];
  if (L >= 2 && L <= kMaxLayers && H % 64 == 0 && H <= gwf::umma::kUNMax) {
    // fused tensor-core inference: parameters in, ln SNR out, nothing else in global memory
    Buf dpar, dout;
    const double* dp = params;
    int64_t dld = ld;
    double* d = out_ln_snr;
    cudaError_t e = cudaSuccess;
    if (mem == GWF_MEM_HOST) {
      if (!dpar.ensure((size_t)kNF * n * sizeof(double)) || !dout.ensure((size_t)n * sizeof(double)))
        return fail(GWF_ERR_OOM, "device allocation failed (MLP input)");
      e = cudaMemcpy2DAsync(dpar.p, n * sizeof(double), params, ld * sizeof(double), n * sizeof(double), kNF,
                            cudaMemcpyHostToDevice, m->stream);
      dp = dpar.as<double>();
      dld = n;
      d = dout.as<double>();
    }
    InferNet net;
    net.L = L;
    net.H = H;
    for (int l = 0; l < L; ++l) {
      net.woff[l] = m->woff[l];
      net.boff[l] = m->boff[l];
    }
    const int smem = infer_smem_bytes();
    if (e == cudaSuccess) e = cudaFuncSetAttribute(mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) {
      mlp_infer_tc_kernel<<<nblk(n, 128), 128, smem, m->stream>>>(dp, dld, n, m->norm.as<float>(), net,
                                                                  m->wbf.as<__nv_bfloat16>(), m->w32.as<float>(), d,
                                                                  m->tc_err.as<int>());
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && mem == GWF_MEM_HOST)
      e = cudaMemcpyAsync(out_ln_snr, d, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    dpar.release();
    dout.release();
    if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("MLP predict: ") + cudaGetErrorString(e));
    return check_tc(m);
  }
  rc = load_features(m, params, ld, n, mem, false);
  if (rc) return rc;
  // inference in slices that bound the activation memory
  const long long slice = 1 << 18;
  if (!m->pred.ensure((size_t)std::min<long long>(n, slice) * sizeof(float))) return fail(GWF_ERR_OOM, "device allocation failed");
  Buf dout;
  double* d = out_ln_snr;
  if (mem == GWF_MEM_HOST) {
    if (!dout.ensure((size_t)n * sizeof(double))) return fail(GWF_ERR_OOM, "device allocation failed");
    d = dout.as<double>();
  }
  for (long long s0 = 0; s0 < n; s0 += slice) {
    const int B = (int)std::min<long long>(slice, n - s0);
    rc = forward(m, m->X.as<float>() + s0 * kNF, B, m->pred.as<float>(), false);
    if (rc) { dout.release(); return rc; }
    to_double_kernel<<<nblk(B, 256), 256, 0, m->stream>>>(m->pred.as<float>(), B, d + s0);
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && mem == GWF_MEM_HOST)
    e = cudaMemcpyAsync(out_ln_snr, d, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  dout.release();
  if (e != cudaSuccess) return fail(GWF_ERR_CUDA, std::string("MLP predict: ") + cudaGetErrorString(e));
  return check_tc(m);
}

}  // extern "C"
