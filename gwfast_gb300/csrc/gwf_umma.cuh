// Tensor-core GEMM for the SNR-screen MLP on sm_100-family GPUs: tcgen05.mma (kind::f16, BF16
// operands, FP32 accumulation in tensor memory), operands staged in shared memory by the CTA's
// threads, one elected thread issuing the MMAs, completion through tcgen05.commit on an mbarrier,
// and an epilogue that reads the accumulators back with tcgen05.ld.
//
// C[M][N] = op(A)[M][K] op(B)[K][N] (+ bias[N], optional SiLU), with
//   op(A)(m, k) = TA ? A[k lda + m] : A[m lda + k]    (FP32 in global memory, rounded to BF16)
//   op(B)(k, n) = TB ? B[n ldb + k] : B[k ldb + n]    (FP32 or BF16 in global memory)
// One CTA of 128 threads computes a 128 x N tile (N <= 256, a multiple of 16) over its share of K
// (blockIdx.y of gridDim.y splits, kspan each; with more than one split the raw FP32 sums go to
// ws[split][M][N] and a reduction adds them in split order); K runs in chunks of kUK = 64
// (zero-padded past K). Shared memory holds one chunk of each operand in the canonical K-major
// layout without swizzling: 8 x 8 core matrices of 128 contiguous bytes (8 rows of 16 bytes),
// ordered [row / 8][k / 8], so adjacent core matrices are 128 bytes apart along K (leading-dimension
// offset) and (kUK / 8) x 128 bytes apart along M or N (stride-dimension offset).
//
// Every wait is bounded: if an mbarrier phase does not complete within kSpinLimit polls the kernel
// sets *err, waits once more (bounded) for its MMAs in flight, frees its tensor memory and returns
// (the host reports the error).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gwf {
namespace umma {

constexpr int kUM = 128;        // rows of a CTA tile (the MMA's M)
constexpr int kUK = 64;         // K chunk staged per MMA batch (4 MMAs of K = 16)
constexpr int kUNMax = 256;     // largest N of one tile
constexpr int kSpinLimit = 1 << 22;   // mbarrier polls (64 ns apart at least) before giving up: > 0.25 s

__host__ __device__ constexpr int a_stage_bytes() { return kUM * kUK * 2; }          // 16 KB
__host__ __device__ constexpr int b_stage_bytes() { return kUNMax * kUK * 2; }       // 32 KB
// dynamic shared memory per CTA: one operand chunk each, padded so that at most two CTAs share an SM
// (two 256-column tensor-memory allocations fill the SM's 512 columns; a third would wait for one)
__host__ __device__ constexpr int smem_bytes() { return 100 * 1024; }

// byte offset of element (row, k) of a [rows][kUK] operand chunk in the core-matrix layout
__device__ __forceinline__ uint32_t core_off(int row, int k) {
  return (uint32_t)(((row >> 3) * (kUK / 8) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor (tcgen05): start address, leading- and stride-dimension byte
// offsets (all >> 4), the fixed descriptor version 1 at bit 46, no swizzling (layout type 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N >> 3, M >> 4
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// poll the mbarrier (non-blocking test, short sleeps between polls) until the phase with the given
// parity completes; false after kSpinLimit polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (int i = 0; i < kSpinLimit; ++i) {
    uint32_t done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[desc] B[desc], M x N x 16, one issuing thread
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}

// arrive on the mbarrier once every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane (warp w reads lanes 32 w .. 32 w + 31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <class T> __device__ __forceinline__ float ldf(const T* p, long long i);
template <> __device__ __forceinline__ float ldf<float>(const float* p, long long i) { return p[i]; }
template <> __device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16* p, long long i) {
  return __bfloat162float(p[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 b = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&b);
}

// stage `rows` x kUK of an operand, element (r, k) = get(r0 + r, k0 + k) (zero outside [0, R) x [0, K)),
// as 16-byte core-matrix rows: each unit is 8 consecutive k of one row
template <class GET>
__device__ __forceinline__ void stage(unsigned char* s, int rows, int r0, int R, int k0, int K, GET get) {
  const int units = rows * (kUK / 8);
  for (int u = threadIdx.x; u < units; u += blockDim.x) {
    const int r = u % rows, kg = u / rows;   // consecutive threads take consecutive rows
    const int gr = r0 + r;
    float v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int gk = k0 + kg * 8 + j;
      v[j] = (gr < R && gk < K) ? get(gr, gk) : 0.0f;
    }
    const uint4 q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
    *reinterpret_cast<uint4*>(s + core_off(r, kg * 8)) = q;
  }
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + __expf(-z)); }

template <bool TA, bool TB, class TBE>
__global__ void __launch_bounds__(128, 1) gemm_tc_kernel(int M, int N, int K, const float* __restrict__ A, int lda,
                                                        const TBE* __restrict__ B, int ldb, float* __restrict__ C,
                                                        int ldc, const float* __restrict__ bias, int act,
                                                        float* __restrict__ Zout, int kspan, float* __restrict__ ws,
                                                        int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* sa = smem_raw;
  unsigned char* sb = smem_raw + a_stage_bytes();
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kUM;
  const int nt = (N + 15) & ~15;   // MMA N (a multiple of 16, <= 256)
  if (warp == 0) {                 // tensor memory: 256 columns (a power of two >= 32, >= nt)
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tm = tmem_base;
  const uint32_t idesc = instr_desc(kUM, nt);
  const uint32_t lbo = 128, sbo = (kUK / 8) * 128;
  bool ok = true;
  uint32_t phase = 0;
  const int kb = blockIdx.y * kspan, ke = min(K, kb + kspan);
  for (int k0 = kb; k0 < ke && ok; k0 += kUK) {
    stage(sa, kUM, m0, M, k0, ke, [&](int r, int k) { return TA ? A[(long long)k * lda + r] : A[(long long)r * lda + k]; });
    stage(sb, nt, 0, N, k0, ke, [&](int n, int k) {
      return TB ? ldf(B, (long long)n * ldb + k) : ldf(B, (long long)k * ldb + n);
    });
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic-proxy stores -> MMA reads
    __syncthreads();
    if (threadIdx.x == 0) {
      fence_after_sync();
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
      for (int s = 0; s < kUK / 16; ++s)   // K = 16 per MMA: two core matrices along K
        mma_f16(tm, smem_desc(a0 + s * 256, lbo, sbo), smem_desc(b0 + s * 256, lbo, sbo), idesc,
                (k0 > kb || s > 0) ? 1u : 0u);
      mma_commit(&bar);
    }
    // the chunk's MMAs are done: its shared memory may be overwritten (all threads agree on the outcome)
    ok = __syncthreads_and(mbar_wait(&bar, phase)) != 0;
    if (!ok) {   // give the MMAs in flight one more bounded wait before the tensor memory is freed
      if (threadIdx.x == 0) {
        atomicExch(err, 1);
        mbar_wait(&bar, phase);
      }
      __syncthreads();
    }
    phase ^= 1u;
    fence_after_sync();
  }
  if (ok && kb < ke) {   // epilogue: row m0 + 32 warp + lane of the tile, 16 columns at a time
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < nt; c0 += 16) {
      float v[16];
      tmem_ld16(tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (row < M && ws) {
        float* w = ws + ((long long)blockIdx.y * M + row) * N;
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (c0 + j < N) w[c0 + j] = v[j];
      } else if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = c0 + j;
          if (col < N) {
            const float z = v[j] + (bias ? bias[col] : 0.0f);
            if (Zout) Zout[(long long)row * ldc + col] = z;
            C[(long long)row * ldc + col] = act == 1 ? silu_f(z) : z;
          }
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tm) : "memory");
}

// C[i] = sum over splits of ws[split][i], in split order (M x N values)
__global__ void splitk_reduce_kernel(const float* __restrict__ ws, int splits, long long mn, float* __restrict__ C) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= mn) return;
  float s = 0.0f;
  for (int y = 0; y < splits; ++y) s += ws[(long long)y * mn + i];
  C[i] = s;
}

}  // namespace umma
}  // namespace gwf
