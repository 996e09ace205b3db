// Tensor-core kernels of the learned surrogate (a BF16 MLP with FP32
// accumulation) and its training step.
//
// k_gemm: C = epilogue(A B^T + bias) for row-major (K-major) BF16 A [M x K]
// and B [N x K].  Tiles reach shared memory by TMA (cp.async.bulk.tensor,
// 128-byte swizzle, zero fill outside the matrix) through a ring of
// mbarrier-tracked stages; one elected thread issues tcgen05.mma (M = 128,
// N = NT, K = 16 per instruction) into a TMEM accumulator; all four warps
// read it back with tcgen05.ld for the epilogue.  Every mbarrier wait is
// bounded: on timeout the kernel records an error flag, frees its TMEM and
// returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <cmath>
#include <mutex>

#include "../../include/optika_gb300.h"
#include "tc.cuh"

namespace otx {

constexpr int GEMM_STAGES = 4;
constexpr int GEMM_BK = 64;  // bf16 elements per K chunk: 128 bytes

struct GemmArgs {
  int m;        // valid rows of A / C
  int n;        // valid columns of C (rows of B)
  int k;        // valid K
  int ldo;      // elements between rows of the output (and of z)
  int ldt;      // elements between rows of the transposed copy
  int kc;       // K chunks per split (blockIdx.y selects the split)
  int vec;      // rows of out / z start 16-byte aligned and n % 16 == 0
  const float* bias;   // n entries or null
  void* out;           // bf16 (SILU, DSILU) or fp32 (BIAS_F32, F32, F32_ATOMIC)
  __nv_bfloat16* z;    // SILU: pre-activation written; DSILU: pre-activation read
  __nv_bfloat16* outT; // bf16 transposed copy of out (SILU, DSILU) or null
  int* err;            // set to 1 on a timed-out wait
};

#define OTX_EPI_SILU_BF16 0
#define OTX_EPI_BIAS_F32 1
#define OTX_EPI_F32 2
#define OTX_EPI_DSILU_BF16 3
#define OTX_EPI_F32_ATOMIC 4

__device__ __forceinline__ void store16_bf16(__nv_bfloat16* p, const float v[16], int valid,
                                             bool vec) {
  if (vec && valid == 16) {
    uint32_t w[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
      w[i] = *reinterpret_cast<uint32_t*>(&h);
    }
    reinterpret_cast<uint4*>(p)[0] = make_uint4(w[0], w[1], w[2], w[3]);
    reinterpret_cast<uint4*>(p)[1] = make_uint4(w[4], w[5], w[6], w[7]);
  } else {
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (i < valid) p[i] = __float2bfloat16_rn(v[i]);
  }
}

__device__ __forceinline__ void load16_bf16(const __nv_bfloat16* p, float v[16], int valid,
                                            bool vec) {
  if (vec && valid == 16) {
    const uint4 a = reinterpret_cast<const uint4*>(p)[0];
    const uint4 b = reinterpret_cast<const uint4*>(p)[1];
    const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w[i]);
      v[2 * i] = __low2float(h);
      v[2 * i + 1] = __high2float(h);
    }
  } else {
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = i < valid ? __bfloat162float(p[i]) : 0.f;
  }
}

template <int NT, int EPI>
__global__ void __launch_bounds__(128, 1)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
           const GemmArgs g) {
  constexpr int A_BYTES = 128 * GEMM_BK * 2;  // 16 KB
  constexpr int B_BYTES = NT * GEMM_BK * 2;
  constexpr uint32_t NCOLS = NT < 32 ? 32 : NT;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint8_t* sa = smem;
  uint8_t* sb = sa + GEMM_STAGES * A_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(sb + GEMM_STAGES * B_BYTES);
  uint64_t* empty = full + GEMM_STAGES;
  uint64_t* done = empty + GEMM_STAGES;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128;
  // this CTA's K chunks: [kb, kb + nk); the host makes every split non-empty
  const int nk_all = (g.k + GEMM_BK - 1) / GEMM_BK;
  const int kb = blockIdx.y * g.kc;
  const int nk = min(nk_all, kb + g.kc) - kb;
  if (nk <= 0) return;  // uniform over the CTA, before any barrier or TMEM use

  if (tid == 0) {
    for (int s = 0; s < GEMM_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tslot, NCOLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  int issued = 0;  // chunks whose TMA loads thread 0 started
  if (tid == 0) {
    // producer: stage s holds chunk k; reuse waits for the MMAs of chunk k - S
    for (int k = 0; k < nk; ++k) {
      const int s = k % GEMM_STAGES;
      if (k >= GEMM_STAGES) {
        if (!mbar_wait(&empty[s], ((k / GEMM_STAGES) - 1) & 1)) {
          atomicExch(g.err, 1);
          break;
        }
      }
      mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
      tma_load_2d(sa + s * A_BYTES, &ta, (kb + k) * GEMM_BK, m0, &full[s]);
      tma_load_2d(sb + s * B_BYTES, &tb, (kb + k) * GEMM_BK, 0, &full[s]);
      issued = k + 1;
    }
  } else if (tid == 32) {
    // MMA issuer
    constexpr uint32_t IDESC = idesc_bf16(128, NT);
    bool ok = true;
    for (int k = 0; k < nk; ++k) {
      const int s = k % GEMM_STAGES;
      if (!mbar_wait(&full[s], (k / GEMM_STAGES) & 1)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint64_t ad = desc_sw128(sa + s * A_BYTES);
      const uint64_t bd = desc_sw128(sb + s * B_BYTES);
#pragma unroll
      for (int kk = 0; kk < GEMM_BK / 16; ++kk)
        umma_bf16(tbase, ad + 2 * kk, bd + 2 * kk, IDESC, (k | kk) != 0);
      umma_commit(&empty[s]);
    }
    if (ok)
      umma_commit(done);
    else
      atomicExch(g.err, 1);
  }
  __syncwarp();
  const bool ok = mbar_wait(done, 0);
  tc_fence_after();
  if (!ok) {
    if (lane == 0) atomicExch(g.err, 1);
    // let the copies this CTA started land before its shared memory is
    // released (bounded, as every wait here)
    if (tid == 0) {
      for (int k = issued - GEMM_STAGES > 0 ? issued - GEMM_STAGES : 0; k < issued; ++k)
        mbar_wait(&full[k % GEMM_STAGES], (k / GEMM_STAGES) & 1);
    }
  } else {
    // epilogue: warp w owns TMEM lanes (rows) 32 w .. 32 w + 31
    const int row = m0 + warp * 32 + lane;
    const bool vec = g.vec != 0;
#pragma unroll 1
    for (int c = 0; c < NT; c += 16) {
      float v[16];
      __syncwarp();  // tcgen05.ld is warp-aligned: reconverge after the stores
      tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      const int valid = min(16, g.n - c);
      if (row >= g.m || valid <= 0) continue;
      const int64_t o = (int64_t)row * g.ldo + c;
      if (EPI == OTX_EPI_F32_ATOMIC) {
        float* p = reinterpret_cast<float*>(g.out) + o;
        if (vec && valid == 16) {
#pragma unroll
          for (int i = 0; i < 16; i += 4)
            atomicAdd(reinterpret_cast<float4*>(p + i), make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]));
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (i < valid) atomicAdd(p + i, v[i]);
        }
        continue;
      }
      if (EPI == OTX_EPI_F32 || EPI == OTX_EPI_BIAS_F32) {
        float* p = reinterpret_cast<float*>(g.out) + o;
#pragma unroll
        for (int i = 0; i < 16; ++i)
          if (i < valid) p[i] = v[i] + (EPI == OTX_EPI_BIAS_F32 ? g.bias[c + i] : 0.f);
        continue;
      }
      float r[16];
      if (EPI == OTX_EPI_SILU_BF16) {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += (g.bias && i < valid) ? g.bias[c + i] : 0.f;
#pragma unroll
        for (int i = 0; i < 16; i += 2) {
          const uint32_t w = silu2_bf16(0.5f * v[i], 0.5f * v[i + 1]);
          r[i] = __uint_as_float(w << 16);
          r[i + 1] = __uint_as_float(w & 0xffff0000u);
        }
        if (g.z) store16_bf16(g.z + o, v, valid, vec);
      } else {  // DSILU: dZ = dH silu'(z), silu'(z) = s (1 + z (1 - s)), s = sigmoid(z)
        float zz[16];
        load16_bf16(g.z + o, zz, valid, vec);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const float sg = sigmoid_tanh(zz[i]);
          r[i] = v[i] * sg * (1.f + zz[i] * (1.f - sg));
        }
      }
      store16_bf16(reinterpret_cast<__nv_bfloat16*>(g.out) + o, r, valid, vec);
      if (g.outT) {
#pragma unroll
        for (int i = 0; i < 16; ++i)
          if (i < valid) g.outT[(int64_t)(c + i) * g.ldt + row] = __float2bfloat16_rn(r[i]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, NCOLS);
}

// ---------------------------------------------------------------- elementwise

// dZ = dY * silu'(Z), silu'(z) = s (1 + z (1 - s)), s = sigmoid(z); both bf16.
__global__ void k_silu_backward(const float* __restrict__ dy, const __nv_bfloat16* __restrict__ z,
                                __nv_bfloat16* __restrict__ dz, int64_t count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float zz = __bfloat162float(z[i]);
    const float s = sigmoid_tanh(zz);
    dz[i] = __float2bfloat16_rn(dy[i] * s * (1.f + zz * (1.f - s)));
  }
}

// out[c][r] = in[r][c] for a rows x cols bf16 matrix (32 x 32 smem tiles).
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ in, int rows, int cols, int ldi,
                                 __nv_bfloat16* __restrict__ out, int ldo) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = in[(int64_t)r * ldi + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = bx + j, r = by + threadIdx.x;
    if (r < rows && c < cols) out[(int64_t)c * ldo + r] = tile[threadIdx.x][j];
  }
}

// out[c] += sum_r in[r][c] (bf16 in, fp32 out).  Each warp walks its own
// rows, one row per step with a 16-byte load per lane (8 columns), so many
// loads are in flight; the block's warps then reduce through shared memory
// and add their column sums with one atomic per column.
constexpr int COLSUM_BLOCK = 256;
constexpr int COLSUM_MAX_COLS = 256;

__global__ void __launch_bounds__(COLSUM_BLOCK)
    k_colsum_bf16(const __nv_bfloat16* __restrict__ in, int rows, int cols, int ldi,
                  float* __restrict__ out) {
  __shared__ float part[COLSUM_BLOCK / 32][COLSUM_MAX_COLS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = gridDim.x * (COLSUM_BLOCK / 32);
  const int c0 = lane * 8;
  float acc[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i] = 0.f;
  if (c0 < cols) {
    for (int r = blockIdx.x * (COLSUM_BLOCK / 32) + warp; r < rows; r += nw) {
      const uint4 q = *reinterpret_cast<const uint4*>(in + (int64_t)r * ldi + c0);
      const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        acc[2 * i] += __uint_as_float(w[i] << 16);
        acc[2 * i + 1] += __uint_as_float(w[i] & 0xffff0000u);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i)
    if (c0 + i < COLSUM_MAX_COLS) part[warp][c0 + i] = acc[i];
  __syncthreads();
  for (int c = threadIdx.x; c < cols; c += COLSUM_BLOCK) {
    float t = 0.f;
#pragma unroll
    for (int w = 0; w < COLSUM_BLOCK / 32; ++w) t += part[w][c];
    atomicAdd(out + c, t);
  }
}

// Adam (Kingma and Ba, 2015) on fp32 master weights; writes the bf16
// weights and, if given, their transpose (rows x cols -> cols x rows).
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ grad, int rows, int cols, float lr, float b1,
                       float b2, float eps, float c1, float c2, __nv_bfloat16* __restrict__ w16,
                       int ld16, __nv_bfloat16* __restrict__ w16t, int ld16t) {
  const int64_t n = (int64_t)rows * cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    w[i] = wi;
    const int r = (int)(i / cols), c = (int)(i % cols);
    if (w16) w16[(int64_t)r * ld16 + c] = __float2bfloat16_rn(wi);
    if (w16t) w16t[(int64_t)c * ld16t + r] = __float2bfloat16_rn(wi);
  }
}

// ---------------------------------------------------------------- host

template <int NT, int EPI>
static otx_status launch_gemm(const CUtensorMap& ta, const CUtensorMap& tb, const GemmArgs& g,
                              int splits, cudaStream_t st) {
  const size_t smem = 1024 + GEMM_STAGES * (128 * GEMM_BK * 2 + NT * GEMM_BK * 2) +
                      (2 * GEMM_STAGES + 2) * 8;
  // per-context function attribute: set on every launch (cheap)
  if (cudaFuncSetAttribute(k_gemm<NT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return OTX_ERR_CUDA;
  const dim3 grid((g.m + 127) / 128, splits);
  k_gemm<NT, EPI><<<grid, 128, smem, st>>>(ta, tb, g);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

template <int EPI>
static otx_status dispatch_nt(int nt, const CUtensorMap& ta, const CUtensorMap& tb,
                              const GemmArgs& g, int splits, cudaStream_t st) {
  switch (nt) {
    case 16: return launch_gemm<16, EPI>(ta, tb, g, splits, st);
    case 64: return launch_gemm<64, EPI>(ta, tb, g, splits, st);
    case 128: return launch_gemm<128, EPI>(ta, tb, g, splits, st);
    case 256: return launch_gemm<256, EPI>(ta, tb, g, splits, st);
    default: return OTX_ERR_UNSUPPORTED;
  }
}

static int grid_1d(int64_t n, int block) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 132;
  const int64_t need = (n + block - 1) / block;
  const int64_t cap = (int64_t)sms * 16;
  return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

}  // namespace otx

using namespace otx;

extern "C" {

otx_status otx_gemm_bf16(const void* a, int32_t lda, const void* b, int32_t ldb, int32_t m,
                         int32_t n, int32_t k, const float* bias, int32_t epilogue, void* out,
                         int32_t ldo, void* z, void* out_t, int32_t ldt, int32_t* err,
                         void* stream) {
  if (!a || !b || !out || !err || m < 0 || n < 1 || k < 1) return OTX_ERR_INVALID;
  if (epilogue < OTX_EPI_SILU_BF16 || epilogue > OTX_EPI_F32_ATOMIC) return OTX_ERR_INVALID;
  if (lda < k || ldb < k || ldo < n || (lda * 2) % 16 || (ldb * 2) % 16) return OTX_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) return OTX_ERR_INVALID;
  if (epilogue == OTX_EPI_BIAS_F32 && !bias) return OTX_ERR_INVALID;
  if (epilogue == OTX_EPI_DSILU_BF16 && !z) return OTX_ERR_INVALID;
  const bool bf16_out = epilogue == OTX_EPI_SILU_BF16 || epilogue == OTX_EPI_DSILU_BF16;
  if (out_t && (!bf16_out || ldt < m)) return OTX_ERR_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (epilogue == OTX_EPI_F32_ATOMIC && m > 0 &&
      cudaMemset2DAsync(out, (size_t)ldo * 4, 0, (size_t)n * 4, (size_t)m, st) != cudaSuccess)
    return OTX_ERR_CUDA;
  if (m == 0) return OTX_OK;
  int nt = 16;
  while (nt < n) nt *= 2;
  if (nt == 32) nt = 64;
  if (nt > 256) return OTX_ERR_SIZE;
  CUtensorMap ta, tb;
  if (!make_map(&ta, a, m, k, lda, 128) || !make_map(&tb, b, n, k, ldb, nt)) return OTX_ERR_CUDA;
  const int esize = bf16_out ? 2 : 4;
  const uintptr_t align = reinterpret_cast<uintptr_t>(out) |
                          (epilogue == OTX_EPI_SILU_BF16 || epilogue == OTX_EPI_DSILU_BF16
                               ? reinterpret_cast<uintptr_t>(z) : 0);
  const int vec = (n % 16 == 0) && ((ldo * esize) % 16 == 0) && (align % 16 == 0);
  const int nk_all = (k + GEMM_BK - 1) / GEMM_BK;
  int kc = nk_all, splits = 1;
  if (epilogue == OTX_EPI_F32_ATOMIC) {
    // split K so that the grid fills the GPU: every split at least 2 chunks
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 132;
    const int tiles = (m + 127) / 128;
    const int want = max(1, (2 * sms) / tiles);
    kc = max(2, (nk_all + want - 1) / want);
    splits = (nk_all + kc - 1) / kc;
  }
  GemmArgs g{m, n, k, ldo, ldt, kc, vec, bias, out, reinterpret_cast<__nv_bfloat16*>(z),
             reinterpret_cast<__nv_bfloat16*>(out_t), err};
  switch (epilogue) {
    case OTX_EPI_SILU_BF16: return dispatch_nt<OTX_EPI_SILU_BF16>(nt, ta, tb, g, splits, st);
    case OTX_EPI_BIAS_F32: return dispatch_nt<OTX_EPI_BIAS_F32>(nt, ta, tb, g, splits, st);
    case OTX_EPI_F32: return dispatch_nt<OTX_EPI_F32>(nt, ta, tb, g, splits, st);
    case OTX_EPI_DSILU_BF16: return dispatch_nt<OTX_EPI_DSILU_BF16>(nt, ta, tb, g, splits, st);
    default: return dispatch_nt<OTX_EPI_F32_ATOMIC>(nt, ta, tb, g, splits, st);
  }
}

otx_status otx_silu_backward(const float* dy, const void* z, void* dz, int64_t count,
                             void* stream) {
  if (count < 0 || (count > 0 && (!dy || !z || !dz))) return OTX_ERR_INVALID;
  if (count == 0) return OTX_OK;
  k_silu_backward<<<grid_1d(count, 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      dy, reinterpret_cast<const __nv_bfloat16*>(z), reinterpret_cast<__nv_bfloat16*>(dz), count);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

otx_status otx_transpose_bf16(const void* in, int32_t rows, int32_t cols, int32_t ldi, void* out,
                              int32_t ldo, void* stream) {
  if (!in || !out || rows < 0 || cols < 0 || ldi < cols || ldo < rows) return OTX_ERR_INVALID;
  if (rows == 0 || cols == 0) return OTX_OK;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  k_transpose_bf16<<<grid, block, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const __nv_bfloat16*>(in), rows, cols, ldi,
      reinterpret_cast<__nv_bfloat16*>(out), ldo);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

otx_status otx_colsum_bf16(const void* in, int32_t rows, int32_t cols, int32_t ldi, float* out,
                           void* stream) {
  if (!in || !out || rows < 0 || cols < 0 || ldi < cols) return OTX_ERR_INVALID;
  if (cols > COLSUM_MAX_COLS || ldi % 8 || (reinterpret_cast<uintptr_t>(in) & 15))
    return OTX_ERR_INVALID;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(out, 0, sizeof(float) * (size_t)cols, st) != cudaSuccess) return OTX_ERR_CUDA;
  if (rows == 0 || cols == 0) return OTX_OK;
  const int warps = COLSUM_BLOCK / 32;
  int grid = grid_1d((int64_t)rows, warps);  // at most 16 blocks per SM
  const int cap = (rows + 16 * warps - 1) / (16 * warps);  // at least 16 rows per warp
  if (grid > cap) grid = cap > 0 ? cap : 1;
  k_colsum_bf16<<<grid, COLSUM_BLOCK, 0, st>>>(reinterpret_cast<const __nv_bfloat16*>(in), rows,
                                               cols, ldi, out);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

otx_status otx_adam(float* w, float* m, float* v, const float* grad, int32_t rows, int32_t cols,
                    float lr, float beta1, float beta2, float eps, int32_t step, void* w16,
                    int32_t ld16, void* w16t, int32_t ld16t, void* stream) {
  if (!w || !m || !v || !grad || rows < 0 || cols < 0 || step < 1) return OTX_ERR_INVALID;
  if ((w16 && ld16 < cols) || (w16t && ld16t < rows)) return OTX_ERR_INVALID;
  const int64_t n = (int64_t)rows * cols;
  if (n == 0) return OTX_OK;
  float c1 = 1.f, c2 = 1.f;
  {
    const double p1 = std::pow((double)beta1, (double)step);
    const double p2 = std::pow((double)beta2, (double)step);
    c1 = (float)(1.0 / (1.0 - p1));
    c2 = (float)(1.0 / (1.0 - p2));
  }
  k_adam<<<grid_1d(n, 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      w, m, v, grad, rows, cols, lr, beta1, beta2, eps, c1, c2,
      reinterpret_cast<__nv_bfloat16*>(w16), ld16, reinterpret_cast<__nv_bfloat16*>(w16t), ld16t);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

}  // extern "C"
