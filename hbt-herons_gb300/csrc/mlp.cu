// mlp.cu - BF16 tensor-core MLP (6 -> 64 -> 64 -> 1) of the learned warm
// start: forward (inference) and backward (training) kernels and an Adam step.
//
// Weights are one flat FP32 array (HBTG_MLP_PARAMS floats):
//   W1[6][64] (in x out), b1[64], W2[64][64] (in x out), b2[64], w3[64], b3
// Inference (hbtg_mlp_forward) runs on the tcgen05 tensor cores with TMEM
// accumulators (k_mlp_forward_tc, below).  Training (hbtg_mlp_backward)
// stages the weights in shared memory as BF16 and chains mma.sync.m16n8k16
// (BF16 operands, FP32 accumulation) over tiles of 16 rows, one tile per warp:
// the accumulator fragment of one layer is re-packed in registers as the A
// fragment of the next (the m16n8 C layout of two adjacent n-tiles is the
// m16k16 A layout), and the backward pass needs those per-warp fragments.
#include <algorithm>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/hbt_unbind_gpu.h"

namespace
{

constexpr int kIn = 6, kHid = 64;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kHid, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid,
              kB3 = kW3 + kHid, kMlpParams = kB3 + 1;
constexpr int kStride16 = 24; // padded bf16 row strides (conflict-free fragment loads)
constexpr int kStride64 = 72;

static_assert(kMlpParams == HBTG_MLP_PARAMS, "weight layout");
static_assert(kIn == HBTG_NUM_FEATURES, "feature count");

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi); // .x = lo (low half), .y = hi
  return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ uint32_t pack_pair(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
               "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared-memory copy of the weights.
//   w1t[n][k] = W1[k][n]  (k padded 6 -> 16 with zeros)   B operand of layer 1
//   w2t[n][k] = W2[k][n]                                   B operand of layer 2
//   w3t[n][k] = w3[k] for n = 0, else 0                    B operand of layer 3
//   w2r[n][k] = W2[n][k]                                   B operand of dH1 = dZ2 W2^T
struct SmemWeights
{
  __nv_bfloat16 w1t[kHid][kStride16];
  __nv_bfloat16 w2t[kHid][kStride64];
  __nv_bfloat16 w3t[8][kStride64];
  __nv_bfloat16 w2r[kHid][kStride64];
  float b1[kHid], b2[kHid], w3[kHid], b3;
};

__device__ void load_weights(SmemWeights &S, const float *__restrict__ w, bool with_w2r)
{
  for (int i = threadIdx.x; i < kHid * 16; i += blockDim.x)
  {
    const int n = i / 16, k = i % 16;
    S.w1t[n][k] = __float2bfloat16_rn(k < kIn ? w[kW1 + k * kHid + n] : 0.f);
  }
  for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x)
  {
    const int n = i / kHid, k = i % kHid;
    S.w2t[n][k] = __float2bfloat16_rn(w[kW2 + k * kHid + n]);
    if (with_w2r)
      S.w2r[n][k] = __float2bfloat16_rn(w[kW2 + n * kHid + k]);
  }
  for (int i = threadIdx.x; i < 8 * kHid; i += blockDim.x)
  {
    const int n = i / kHid, k = i % kHid;
    S.w3t[n][k] = __float2bfloat16_rn(n == 0 ? w[kW3 + k] : 0.f);
  }
  for (int i = threadIdx.x; i < kHid; i += blockDim.x)
  {
    S.b1[i] = w[kB1 + i];
    S.b2[i] = w[kB2 + i];
    S.w3[i] = __bfloat162float(__float2bfloat16_rn(w[kW3 + i]));
  }
  if (threadIdx.x == 0)
    S.b3 = w[kB3];
  __syncthreads();
}

// Forward pass of one 16-row tile.  g = lane / 4 (row), c = lane % 4.
// Keeps the post-ReLU activations h1/h2 (FP32, C layout), their BF16 A
// fragments, and the logits of rows g and g+8 (valid in every lane).
struct Tile
{
  float h1[8][4], h2[8][4];
  uint32_t a1[4], a2[4][4], a3[4][4];
  float logit_g, logit_g8;
};

__device__ __forceinline__ void forward_tile(const SmemWeights &S, const float *__restrict__ x, long long row0,
                                             long long n, Tile &T)
{
  const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
  const long long ra = row0 + g, rb = row0 + g + 8;
  auto feat = [&](long long r, int k) { return (r < n && k < kIn) ? x[r * kIn + k] : 0.f; };
  T.a1[0] = pack_bf16(feat(ra, 2 * c), feat(ra, 2 * c + 1));
  T.a1[1] = pack_bf16(feat(rb, 2 * c), feat(rb, 2 * c + 1));
  T.a1[2] = 0u; // features 8..15 are padding
  T.a1[3] = 0u;
#pragma unroll
  for (int nt = 0; nt < 8; nt++)
  {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&S.w1t[8 * nt + g][2 * c]);
    const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&S.w1t[8 * nt + g][2 * c + 8]);
    mma_bf16(d, T.a1, b0, b1);
    const float bb0 = S.b1[8 * nt + 2 * c], bb1 = S.b1[8 * nt + 2 * c + 1];
    T.h1[nt][0] = fmaxf(d[0] + bb0, 0.f);
    T.h1[nt][1] = fmaxf(d[1] + bb1, 0.f);
    T.h1[nt][2] = fmaxf(d[2] + bb0, 0.f);
    T.h1[nt][3] = fmaxf(d[3] + bb1, 0.f);
  }
#pragma unroll
  for (int kb = 0; kb < 4; kb++)
  {
    T.a2[kb][0] = pack_bf16(T.h1[2 * kb][0], T.h1[2 * kb][1]);
    T.a2[kb][1] = pack_bf16(T.h1[2 * kb][2], T.h1[2 * kb][3]);
    T.a2[kb][2] = pack_bf16(T.h1[2 * kb + 1][0], T.h1[2 * kb + 1][1]);
    T.a2[kb][3] = pack_bf16(T.h1[2 * kb + 1][2], T.h1[2 * kb + 1][3]);
  }
#pragma unroll
  for (int nt = 0; nt < 8; nt++)
  {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kb = 0; kb < 4; kb++)
    {
      const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&S.w2t[8 * nt + g][16 * kb + 2 * c]);
      const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&S.w2t[8 * nt + g][16 * kb + 2 * c + 8]);
      mma_bf16(d, T.a2[kb], b0, b1);
    }
    const float bb0 = S.b2[8 * nt + 2 * c], bb1 = S.b2[8 * nt + 2 * c + 1];
    T.h2[nt][0] = fmaxf(d[0] + bb0, 0.f);
    T.h2[nt][1] = fmaxf(d[1] + bb1, 0.f);
    T.h2[nt][2] = fmaxf(d[2] + bb0, 0.f);
    T.h2[nt][3] = fmaxf(d[3] + bb1, 0.f);
  }
#pragma unroll
  for (int kb = 0; kb < 4; kb++)
  {
    T.a3[kb][0] = pack_bf16(T.h2[2 * kb][0], T.h2[2 * kb][1]);
    T.a3[kb][1] = pack_bf16(T.h2[2 * kb][2], T.h2[2 * kb][3]);
    T.a3[kb][2] = pack_bf16(T.h2[2 * kb + 1][0], T.h2[2 * kb + 1][1]);
    T.a3[kb][3] = pack_bf16(T.h2[2 * kb + 1][2], T.h2[2 * kb + 1][3]);
  }
  // output layer: column 0 of an n8 tile
  float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int kb = 0; kb < 4; kb++)
  {
    const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&S.w3t[g][16 * kb + 2 * c]);
    const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&S.w3t[g][16 * kb + 2 * c + 8]);
    mma_bf16(d, T.a3[kb], b0, b1);
  }
  // column 0 lives in the lanes with c == 0 (d[0]: row g, d[2]: row g+8)
  T.logit_g = __shfl_sync(0xffffffffu, d[0], lane & ~3) + S.b3;
  T.logit_g8 = __shfl_sync(0xffffffffu, d[2], lane & ~3) + S.b3;
}

// ---------------------------------------------------------------------------
// Inference on the Blackwell tensor cores (tcgen05).  A CTA of four warps
// takes tiles of 128 rows.  Layer 1 (K = 16: the six features and ten zeros)
// and layer 2 (K = 64) are tcgen05.mma.kind::f16 issued by one thread: BF16
// operands in shared memory, FP32 accumulators in tensor memory (TMEM, 128
// lanes = rows; columns 0-63 layer 1, 64-127 layer 2), completion signalled
// to an mbarrier by tcgen05.commit.  The epilogues run on the CUDA cores from
// tcgen05.ld (thread t reads TMEM lane t, i.e. row t of the tile): bias,
// ReLU and BF16 rounding into layer 2's A operand; then bias, ReLU, BF16
// rounding and the output neuron's 64-term dot product with the BF16 w3 in
// FP32, and the sigmoid -- the rounding points of the mma.sync training
// kernels and of the numpy oracle.
//
// Operand layout (no swizzle, K-major): core matrices of 8 rows x 16 bytes
// (8 BF16 along K), stored row by row; the core matrices of one 8-row group
// follow each other along K (leading byte offset 128), and the 8-row groups
// are K * 16 bytes apart (stride byte offset).
//
// Every wait on the mbarrier is bounded (about one second of clock), and the
// CTA decides together (a block-wide AND) whether to go on; a CTA that gives
// up writes NaN for the rows it has not finished (a NaN probability is neither
// trusted nor left out, so the exact iteration decides those particles),
// waits once more (bounded) for the tensor core, frees its tensor memory and
// returns.
// ---------------------------------------------------------------------------
constexpr int kTcRows = 128;
constexpr int kTcThreads = 128;
constexpr uint32_t kTmemCols = 128;
constexpr size_t kTcSmemBytes = 52 * 1024; // at most 4 CTAs per SM: 4 x 128 TMEM columns = 512
constexpr long long kTcWaitCycles = 2000000000LL;

struct TcSmem
{
  __nv_bfloat16 a1[kTcRows * 16]; // A of layer 1: the features (BF16), K = 16
  __nv_bfloat16 a2[kTcRows * kHid]; // A of layer 2: relu(layer 1) in BF16, K = 64
  __nv_bfloat16 b1[kHid * 16];    // B of layer 1: W1^T (N = 64 x K = 16)
  __nv_bfloat16 b2[kHid * kHid];  // B of layer 2: W2^T (N = 64 x K = 64)
  float bias1[kHid], bias2[kHid], w3[kHid], b3;
  unsigned long long mbar;
  uint32_t tmem_base;
};
static_assert(sizeof(TcSmem) <= kTcSmemBytes, "tcgen05 forward shared memory");

// Byte offset of element (row, k) of a K-major operand with K columns.
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int K)
{
  return (uint32_t)((row >> 3) * (K * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (each encoded >> 4), descriptor version 1, no swizzling.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 64, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kHid >> 3) << 17) |
                              ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate)
{
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
               "l"(a), "l"(b), "r"(kTcIdesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

// Bounded wait for the mbarrier phase with the given parity; false on timeout.
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity)
{
  const long long t0 = clock64();
  for (;;)
  {
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(done)
                 : "r"(mbar), "r"(parity)
                 : "memory");
    if (done)
      return true;
    if (clock64() - t0 > kTcWaitCycles)
      return false;
  }
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16])
{
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
               "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                 "=r"(r[15])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; j++)
    v[j] = __uint_as_float(r[j]);
}

// Propose = false: prob[row] = p.  Propose = true (the learned call): the
// proposal byte instead, prop[row] = 1 (trusted, p >= trust), 2 (left out,
// p < leave_out) or 0 (uncertain; also for NaN).
template <bool Propose>
__global__ void __launch_bounds__(kTcThreads)
  k_mlp_forward_tc(const float *__restrict__ w, const float *__restrict__ x, float *__restrict__ prob,
                   uint8_t *__restrict__ prop, float trust, float leave_out, long long n)
{
  extern __shared__ __align__(1024) unsigned char tc_raw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(tc_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char *a1 = reinterpret_cast<unsigned char *>(S.a1), *a2 = reinterpret_cast<unsigned char *>(S.a2);
  unsigned char *b1 = reinterpret_cast<unsigned char *>(S.b1), *b2 = reinterpret_cast<unsigned char *>(S.b2);
  for (int i = tid; i < kHid * 16; i += kTcThreads)
  {
    const int nn = i >> 4, k = i & 15;
    *reinterpret_cast<__nv_bfloat16 *>(b1 + kmajor_off(nn, k, 16)) =
      __float2bfloat16_rn(k < kIn ? w[kW1 + k * kHid + nn] : 0.f);
  }
  for (int i = tid; i < kHid * kHid; i += kTcThreads)
  {
    const int nn = i >> 6, k = i & 63;
    *reinterpret_cast<__nv_bfloat16 *>(b2 + kmajor_off(nn, k, kHid)) = __float2bfloat16_rn(w[kW2 + k * kHid + nn]);
  }
  for (int i = tid; i < kHid; i += kTcThreads)
  {
    S.bias1[i] = w[kB1 + i];
    S.bias2[i] = w[kB2 + i];
    S.w3[i] = __bfloat162float(__float2bfloat16_rn(w[kW3 + i]));
  }
  if (tid == 0)
    S.b3 = w[kB3];
  // features 8..15 of layer 1's A are zero padding for every tile
  *reinterpret_cast<uint4 *>(a1 + kmajor_off(tid, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
  const uint32_t mbar = smem_u32(&S.mbar);
  if (tid == 0)
  {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0)
  {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem_base;
  const uint32_t my_lane = tmem + ((uint32_t)(warp * 32) << 16); // this warp's 32 TMEM lanes
  const uint64_t da1 = smem_desc(smem_u32(a1), 128, 16 * 16), db1 = smem_desc(smem_u32(b1), 128, 16 * 16);
  const uint32_t sa2 = smem_u32(a2), sb2 = smem_u32(b2);
  const long long tiles = (n + kTcRows - 1) / kTcRows;
  uint32_t parity = 0;
  bool ok = true;
  long long t = blockIdx.x;
  // this thread's row of a tile (zero past the end)
  auto load_row = [&](long long tile, float (&f)[kIn]) {
    const long long row = tile * kTcRows + tid;
#pragma unroll
    for (int q = 0; q < kIn; q++)
      f[q] = (tile < tiles && row < n) ? __ldg(x + row * kIn + q) : 0.f;
  };
  float f[kIn];
  load_row(t, f);
  for (; t < tiles; t += gridDim.x)
  {
    const long long row = t * kTcRows + tid;
    *reinterpret_cast<uint4 *>(a1 + kmajor_off(tid, 0, 16)) =
      make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), 0u);
    fence_async_smem();
    __syncthreads();
    if (tid == 0)
    {
      tc_fence_after();
      tc_mma(tmem, da1, db1, 0u);
      tc_commit(mbar);
    }
    load_row(t + gridDim.x, f); // the next tile's features load while the tensor core works
    ok = __syncthreads_and(tc_wait(mbar, parity)) != 0; // the whole block gives up together
    parity ^= 1u;
    if (!ok)
      break;
    tc_fence_after();
    // layer 1 epilogue: bias, ReLU, BF16 -> layer 2's A (row tid, 8 columns per 16-byte store)
#pragma unroll
    for (int c0 = 0; c0 < kHid; c0 += 16)
    {
      float v[16];
      tc_ld16(my_lane + (uint32_t)c0, v);
      uint32_t pk[8];
#pragma unroll
      for (int j = 0; j < 8; j++)
        pk[j] = pack_bf16(fmaxf(v[2 * j] + S.bias1[c0 + 2 * j], 0.f), fmaxf(v[2 * j + 1] + S.bias1[c0 + 2 * j + 1], 0.f));
      *reinterpret_cast<uint4 *>(a2 + kmajor_off(tid, c0, kHid)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      *reinterpret_cast<uint4 *>(a2 + kmajor_off(tid, c0 + 8, kHid)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
    {
      tc_fence_after();
#pragma unroll
      for (int kb = 0; kb < kHid / 16; kb++) // K steps of 16: two core matrices, 256 bytes
        tc_mma(tmem + (uint32_t)kHid, smem_desc(sa2 + 256u * kb, 128, kHid * 16),
               smem_desc(sb2 + 256u * kb, 128, kHid * 16), kb > 0 ? 1u : 0u);
      tc_commit(mbar);
    }
    ok = __syncthreads_and(tc_wait(mbar, parity)) != 0; // the whole block gives up together
    parity ^= 1u;
    if (!ok)
      break;
    tc_fence_after();
    // layer 2 epilogue and the output neuron
    float logit = 0.f;
#pragma unroll
    for (int c0 = 0; c0 < kHid; c0 += 16)
    {
      float v[16];
      tc_ld16(my_lane + (uint32_t)(kHid + c0), v);
#pragma unroll
      for (int j = 0; j < 16; j++)
      {
        const float h = __bfloat162float(__float2bfloat16_rn(fmaxf(v[j] + S.bias2[c0 + j], 0.f)));
        logit = fmaf(h, S.w3[c0 + j], logit);
      }
    }
    if (row < n)
    {
      const float p = 1.f / (1.f + __expf(-(logit + S.b3)));
      if (Propose)
        prop[row] = p >= trust ? 1 : (p < leave_out ? 2 : 0);
      else
        prob[row] = p;
    }
    tc_fence_before();
    __syncthreads();
  }
  if (!ok)
  { // gave up on a tile: NaN for it and the CTA's remaining tiles; let the
    // tensor core finish (bounded) before the memory is freed
    for (long long u = t; u < tiles; u += gridDim.x)
    {
      const long long row = u * kTcRows + tid;
      if (row < n)
      {
        if (Propose)
          prop[row] = 0;
        else
          prob[row] = __int_as_float(0x7fc00000);
      }
    }
    tc_wait(mbar, parity ^ 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
  {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// Per-warp staging of BF16 activations and deltas for the weight-gradient products.
struct WarpStage
{
  __nv_bfloat16 h1[16][kStride64];  // H1 (rows x hidden)
  __nv_bfloat16 dz2[16][kStride64]; // dZ2
  __nv_bfloat16 dz1[16][kStride64]; // dZ1
  __nv_bfloat16 x[16][kStride16];   // X (features padded to 16)
};

constexpr int kBwdWarps = 4;
constexpr size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }
constexpr size_t kBwdSmemStage = align16(sizeof(SmemWeights));
constexpr size_t kBwdSmemAcc = align16(kBwdSmemStage + kBwdWarps * sizeof(WarpStage));
constexpr size_t kBwdSmemBytes = align16(kBwdSmemAcc + sizeof(float) * (kMlpParams + 1));

// Weighted binary cross-entropy on sigmoid(logit): gradient and loss summed
// over n rows into grad / loss (zeroed by the caller).  Dynamic shared memory
// (kBwdSmemBytes): weights, per-warp staging, gradient accumulators + loss.
__global__ void __launch_bounds__(kBwdWarps * 32) k_mlp_backward(const float *__restrict__ w,
                                                                 const float *__restrict__ x,
                                                                 const float *__restrict__ y,
                                                                 const float *__restrict__ sw, long long n,
                                                                 float *__restrict__ grad, float *__restrict__ loss)
{
  extern __shared__ __align__(16) unsigned char smem[];
  SmemWeights &S = *reinterpret_cast<SmemWeights *>(smem);
  WarpStage *Wst = reinterpret_cast<WarpStage *>(smem + kBwdSmemStage);
  float *acc = reinterpret_cast<float *>(smem + kBwdSmemAcc);
  float &acc_loss = acc[kMlpParams];
  for (int i = threadIdx.x; i <= kMlpParams; i += blockDim.x)
    acc[i] = 0.f;
  load_weights(S, w, true); // ends with __syncthreads
  const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3, wi = threadIdx.x >> 5;
  WarpStage &st = Wst[wi];
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long row0 = warp * 16; row0 < n; row0 += nwarps * 16)
  {
    Tile T;
    forward_tile(S, x, row0, n, T);
    const long long ra = row0 + g, rb = row0 + g + 8;
    // dL/dlogit = weight * (sigmoid(logit) - y); loss in the stable log-sum-exp form
    float dl_g = 0.f, dl_g8 = 0.f, l = 0.f;
    if (ra < n)
    {
      const float p = 1.f / (1.f + __expf(-T.logit_g)), wt = sw ? sw[ra] : 1.f, t = y[ra];
      dl_g = wt * (p - t);
      l += wt * (fmaxf(T.logit_g, 0.f) - T.logit_g * t + log1pf(__expf(-fabsf(T.logit_g))));
    }
    if (rb < n)
    {
      const float p = 1.f / (1.f + __expf(-T.logit_g8)), wt = sw ? sw[rb] : 1.f, t = y[rb];
      dl_g8 = wt * (p - t);
      l += wt * (fmaxf(T.logit_g8, 0.f) - T.logit_g8 * t + log1pf(__expf(-fabsf(T.logit_g8))));
    }
    if (c == 0)
      atomicAdd(&acc_loss, l);
    // output layer: dw3[j] = sum_r H2[r][j] dl[r]; dZ2 = dl w3 relu'(H2)
    float dz2[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
    {
      const int j0 = 8 * nt + 2 * c;
      float s0 = T.h2[nt][0] * dl_g + T.h2[nt][2] * dl_g8;
      float s1 = T.h2[nt][1] * dl_g + T.h2[nt][3] * dl_g8;
      for (int o = 4; o < 32; o <<= 1)
      {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      }
      if (g == 0)
      {
        atomicAdd(&acc[kW3 + j0], s0);
        atomicAdd(&acc[kW3 + j0 + 1], s1);
      }
      dz2[nt][0] = T.h2[nt][0] > 0.f ? dl_g * S.w3[j0] : 0.f;
      dz2[nt][1] = T.h2[nt][1] > 0.f ? dl_g * S.w3[j0 + 1] : 0.f;
      dz2[nt][2] = T.h2[nt][2] > 0.f ? dl_g8 * S.w3[j0] : 0.f;
      dz2[nt][3] = T.h2[nt][3] > 0.f ? dl_g8 * S.w3[j0 + 1] : 0.f;
    }
    {
      float sdl = (c == 0) ? dl_g + dl_g8 : 0.f;
      for (int o = 4; o < 32; o <<= 1)
        sdl += __shfl_xor_sync(0xffffffffu, sdl, o);
      if (lane == 0)
        atomicAdd(&acc[kB3], sdl);
    }
    // dH1 = dZ2 W2^T (A = dZ2 as BF16 fragments, B = w2r)
    uint32_t adz[4][4];
#pragma unroll
    for (int kb = 0; kb < 4; kb++)
    {
      adz[kb][0] = pack_bf16(dz2[2 * kb][0], dz2[2 * kb][1]);
      adz[kb][1] = pack_bf16(dz2[2 * kb][2], dz2[2 * kb][3]);
      adz[kb][2] = pack_bf16(dz2[2 * kb + 1][0], dz2[2 * kb + 1][1]);
      adz[kb][3] = pack_bf16(dz2[2 * kb + 1][2], dz2[2 * kb + 1][3]);
    }
    float dz1[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
    {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kb = 0; kb < 4; kb++)
      {
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&S.w2r[8 * nt + g][16 * kb + 2 * c]);
        const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&S.w2r[8 * nt + g][16 * kb + 2 * c + 8]);
        mma_bf16(d, adz[kb], b0, b1);
      }
#pragma unroll
      for (int q = 0; q < 4; q++)
        dz1[nt][q] = T.h1[nt][q] > 0.f ? d[q] : 0.f;
    }
    // stage H1, dZ2, dZ1 (BF16) and X for the transposed products; bias gradients (FP32)
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
    {
      const int j0 = 8 * nt + 2 * c;
      st.h1[g][j0] = __float2bfloat16_rn(T.h1[nt][0]);
      st.h1[g][j0 + 1] = __float2bfloat16_rn(T.h1[nt][1]);
      st.h1[g + 8][j0] = __float2bfloat16_rn(T.h1[nt][2]);
      st.h1[g + 8][j0 + 1] = __float2bfloat16_rn(T.h1[nt][3]);
      st.dz2[g][j0] = __float2bfloat16_rn(dz2[nt][0]);
      st.dz2[g][j0 + 1] = __float2bfloat16_rn(dz2[nt][1]);
      st.dz2[g + 8][j0] = __float2bfloat16_rn(dz2[nt][2]);
      st.dz2[g + 8][j0 + 1] = __float2bfloat16_rn(dz2[nt][3]);
      st.dz1[g][j0] = __float2bfloat16_rn(dz1[nt][0]);
      st.dz1[g][j0 + 1] = __float2bfloat16_rn(dz1[nt][1]);
      st.dz1[g + 8][j0] = __float2bfloat16_rn(dz1[nt][2]);
      st.dz1[g + 8][j0 + 1] = __float2bfloat16_rn(dz1[nt][3]);
      float s20 = dz2[nt][0] + dz2[nt][2], s21 = dz2[nt][1] + dz2[nt][3];
      float s10 = dz1[nt][0] + dz1[nt][2], s11 = dz1[nt][1] + dz1[nt][3];
      for (int o = 4; o < 32; o <<= 1)
      {
        s20 += __shfl_xor_sync(0xffffffffu, s20, o);
        s21 += __shfl_xor_sync(0xffffffffu, s21, o);
        s10 += __shfl_xor_sync(0xffffffffu, s10, o);
        s11 += __shfl_xor_sync(0xffffffffu, s11, o);
      }
      if (g == 0)
      {
        atomicAdd(&acc[kB2 + j0], s20);
        atomicAdd(&acc[kB2 + j0 + 1], s21);
        atomicAdd(&acc[kB1 + j0], s10);
        atomicAdd(&acc[kB1 + j0 + 1], s11);
      }
    }
    for (int i = lane; i < 16 * 16; i += 32)
    {
      const int r = i / 16, k = i % 16;
      const long long row = row0 + r;
      st.x[r][k] = __float2bfloat16_rn((row < n && k < kIn) ? x[row * kIn + k] : 0.f);
    }
    __syncwarp();
    // dW2[i][j] = sum_r H1[r][i] dZ2[r][j]: A = H1^T (m = i, k = r), B = dZ2 (k = r, n = j)
#pragma unroll
    for (int mt = 0; mt < 4; mt++)
    {
      uint32_t a[4];
      a[0] = pack_pair(st.h1[2 * c][16 * mt + g], st.h1[2 * c + 1][16 * mt + g]);
      a[1] = pack_pair(st.h1[2 * c][16 * mt + g + 8], st.h1[2 * c + 1][16 * mt + g + 8]);
      a[2] = pack_pair(st.h1[2 * c + 8][16 * mt + g], st.h1[2 * c + 9][16 * mt + g]);
      a[3] = pack_pair(st.h1[2 * c + 8][16 * mt + g + 8], st.h1[2 * c + 9][16 * mt + g + 8]);
#pragma unroll
      for (int nt = 0; nt < 8; nt++)
      {
        const uint32_t b0 = pack_pair(st.dz2[2 * c][8 * nt + g], st.dz2[2 * c + 1][8 * nt + g]);
        const uint32_t b1 = pack_pair(st.dz2[2 * c + 8][8 * nt + g], st.dz2[2 * c + 9][8 * nt + g]);
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        mma_bf16(d, a, b0, b1);
        const int i0 = 16 * mt + g, j0 = 8 * nt + 2 * c;
        atomicAdd(&acc[kW2 + i0 * kHid + j0], d[0]);
        atomicAdd(&acc[kW2 + i0 * kHid + j0 + 1], d[1]);
        atomicAdd(&acc[kW2 + (i0 + 8) * kHid + j0], d[2]);
        atomicAdd(&acc[kW2 + (i0 + 8) * kHid + j0 + 1], d[3]);
      }
    }
    // dW1[k][j] = sum_r X[r][k] dZ1[r][j]: A = X^T (m = k, padded to 16), B = dZ1
    {
      uint32_t a[4];
      a[0] = pack_pair(st.x[2 * c][g], st.x[2 * c + 1][g]);
      a[1] = pack_pair(st.x[2 * c][g + 8], st.x[2 * c + 1][g + 8]);
      a[2] = pack_pair(st.x[2 * c + 8][g], st.x[2 * c + 9][g]);
      a[3] = pack_pair(st.x[2 * c + 8][g + 8], st.x[2 * c + 9][g + 8]);
#pragma unroll
      for (int nt = 0; nt < 8; nt++)
      {
        const uint32_t b0 = pack_pair(st.dz1[2 * c][8 * nt + g], st.dz1[2 * c + 1][8 * nt + g]);
        const uint32_t b1 = pack_pair(st.dz1[2 * c + 8][8 * nt + g], st.dz1[2 * c + 9][8 * nt + g]);
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        mma_bf16(d, a, b0, b1);
        const int j0 = 8 * nt + 2 * c;
        if (g < kIn) // rows g + 8 and g >= 6 are padding
        {
          atomicAdd(&acc[kW1 + g * kHid + j0], d[0]);
          atomicAdd(&acc[kW1 + g * kHid + j0 + 1], d[1]);
        }
      }
    }
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x)
    if (acc[i] != 0.f)
      atomicAdd(&grad[i], acc[i]);
  if (threadIdx.x == 0)
    atomicAdd(loss, acc_loss);
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ grad, float *__restrict__ m,
                       float *__restrict__ v, int np, float lr, float b1, float b2, float eps, float scale, int step)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np)
    return;
  const float gi = grad[i] * scale;
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  const float mh = m[i] / (1.f - powf(b1, (float)step));
  const float vh = v[i] / (1.f - powf(b2, (float)step));
  w[i] -= lr * mh / (sqrtf(vh) + eps);
}

inline int grid_for_rows(long long n, int rows_per_block)
{
  const long long b = (n + rows_per_block - 1) / rows_per_block;
  return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

template <bool Propose>
int launch_forward_tc(const float *w, const float *x, float *prob, uint8_t *prop, float trust, float leave_out,
                      long long n, cudaStream_t st)
{
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return HBTG_ERR_CUDA;
  if (cudaFuncSetAttribute(k_mlp_forward_tc<Propose>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kTcSmemBytes) != cudaSuccess)
    return HBTG_ERR_CUDA;
  const long long tiles = (n + kTcRows - 1) / kTcRows;
  const int grid = (int)std::min<long long>(tiles, 4LL * sms); // persistent: 4 CTAs per SM (TMEM: 4 x 128 columns)
  k_mlp_forward_tc<Propose><<<grid, kTcThreads, kTcSmemBytes, st>>>(w, x, prob, prop, trust, leave_out, n);
  return cudaGetLastError() == cudaSuccess ? HBTG_OK : HBTG_ERR_CUDA;
}

} // namespace

// The learned call's proposal straight from the network (not exported: the
// library's own units call it).
__attribute__((visibility("hidden"))) int hbtg_mlp_propose(const float *weights, const float *features,
                                                            uint8_t *prop, float trust, float leave_out, int64_t n,
                                                            cudaStream_t stream)
{
  if (n <= 0)
    return HBTG_OK;
  return launch_forward_tc<true>(weights, features, nullptr, prop, trust, leave_out, n, stream);
}

extern "C" int hbtg_mlp_forward(const float *weights, const float *features, float *prob, int64_t n, void *stream)
{
  if (!weights || n < 0 || (n > 0 && (!features || !prob)))
    return HBTG_ERR_INVALID;
  if (n == 0)
    return HBTG_OK;
  return launch_forward_tc<false>(weights, features, prob, nullptr, 0.f, 0.f, n, static_cast<cudaStream_t>(stream));
}

extern "C" int hbtg_mlp_backward(const float *weights, const float *features, const float *labels,
                                 const float *sample_weights, int64_t n, float *grad, float *loss, void *stream)
{
  if (!weights || !grad || !loss || n < 0 || (n > 0 && (!features || !labels)))
    return HBTG_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(grad, 0, sizeof(float) * kMlpParams, st) != cudaSuccess ||
      cudaMemsetAsync(loss, 0, sizeof(float), st) != cudaSuccess)
    return HBTG_ERR_CUDA;
  if (n == 0)
    return HBTG_OK;
  static bool attr_set = false; // the attribute belongs to the function, on every device
  if (!attr_set)
  {
    if (cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmemBytes) !=
        cudaSuccess)
      return HBTG_ERR_CUDA;
    attr_set = true;
  }
  // few resident blocks: each one flushes its whole gradient with global atomics
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return HBTG_ERR_CUDA;
  const int blocks = std::min(grid_for_rows(n, kBwdWarps * 16), 2 * sms);
  k_mlp_backward<<<blocks, kBwdWarps * 32, kBwdSmemBytes, st>>>(weights, features, labels, sample_weights, n, grad,
                                                                loss);
  return cudaGetLastError() == cudaSuccess ? HBTG_OK : HBTG_ERR_CUDA;
}

extern "C" int hbtg_adam_step(float *weights, const float *grad, float *m, float *v, int n_params, float lr,
                              float beta1, float beta2, float eps, float grad_scale, int step, void *stream)
{
  if (!weights || !grad || !m || !v || n_params <= 0 || step < 1)
    return HBTG_ERR_INVALID;
  k_adam<<<(n_params + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(weights, grad, m, v, n_params, lr,
                                                                                 beta1, beta2, eps, grad_scale, step);
  return cudaGetLastError() == cudaSuccess ? HBTG_OK : HBTG_ERR_CUDA;
}
