// Image simulation with the surrogate network in one persistent
// tensor-core kernel, and the traced fallback of the rays it does not land.
//
// k_surrogate_fused: every CTA (one per SM) runs two 128-ray tiles side by
// side.  For each tile, 8 epilogue warps generate the rays (Philox, as the
// batched trace does), pack the 9 network inputs as BF16 straight into
// shared memory in the 128-byte-swizzled K-major layout the tensor cores
// read, and keep the quadratic baseline of the image position in
// registers.  One thread issues every tcgen05.mma (M = 128, FP32
// accumulators in TMEM, 256 columns per tile); another streams the weight
// matrices from L2 by TMA through a ring of 32 KB stages (the output
// layer's weights stay resident).  Each weight stage feeds both tiles'
// MMAs, so a weight byte fetched from L2 serves 256 rays.
//
// A hidden layer runs in column halves (N = 128 per MMA) and its weights in
// (column half, K half) stages, in the order (0-127, K 0-127),
// (0-127, K 128-255), (128-255, K 0-127), (128-255, K 128-255).  Four of a
// tile's epilogue warps own accumulator columns 0-127 and the other four
// columns 128-255; each group reads its half with tcgen05.ld, adds the
// bias, applies SiLU (packed BF16 tanh and FMA) and writes the next layer's
// BF16 input of the same K columns back into the tile's operand.  The
// first group starts once the third stage's MMAs have completed (the last
// ones to read K columns 0-127), so its epilogue overlaps the fourth
// stage's MMAs, and the second group's epilogue overlaps the next layer's
// first stage: the tensor cores and the epilogue warps work at the same
// time instead of in turn.  Activations never leave the SM.  After the
// output layer a
// ray of a trusted configuration whose vignetting logit is at least the
// band away from 0 lands at baseline + out_scale * network output (binned
// into its configuration's image if the logit is positive); every other
// ray is appended to its configuration's fallback list.
//
// k_surrogate_fallback traces the listed rays through the configuration's
// surfaces (staged in shared memory per configuration) and bins them.
//
// Every mbarrier wait is bounded; a wait that gives up sets the error flag,
// the CTA stops issuing work, lets its copies land and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/optika_gb300.h"
#include "surrogate_common.cuh"
#include "tc.cuh"

namespace otx {

constexpr int F_ROWS = 128;                          // rays per tile (MMA M)
constexpr int F_WIDTH = 256;                         // hidden width
constexpr int F_KC = 64;                             // K elements per 128-byte chunk
constexpr int F_A_CHUNK = F_ROWS * F_KC * 2;         // 16 KB: one K chunk of a tile
constexpr int F_A_BYTES = (F_WIDTH / F_KC) * F_A_CHUNK;  // 64 KB: a tile's operand
constexpr int F_NH = 128;                            // weight rows (N) per stage: a column half
constexpr int F_WBOX = F_NH * F_KC * 2;              // 16 KB: one TMA box, one K chunk
constexpr int F_STAGE = 2 * F_WBOX;                  // 32 KB: a K half (two chunks)
constexpr int F_STAGES = 2;
constexpr int F_OUT_N = 16;                          // output layer N (3 used)
constexpr int F_WOUT_CHUNK = F_OUT_N * F_KC * 2;     // 2 KB
constexpr int F_MAX_HIDDEN = OTX_MLP_MAX_HIDDEN;
constexpr int F_EPI_WARPS = 8;                       // per tile slot
constexpr int F_THREADS = 32 * (2 + 2 * F_EPI_WARPS);  // 576
constexpr int F_BIAS_FLOATS = F_MAX_HIDDEN * F_WIDTH + F_OUT_N;
constexpr size_t F_SMEM = 1024 + 2 * F_A_BYTES + F_STAGES * F_STAGE + (F_WIDTH / F_KC) * F_WOUT_CHUNK +
                          F_BIAS_FLOATS * 4 + 256;

struct FusedArgs {
  otx_batch b;
  otx_surrogate sg;
  otx_sensor sensor;
  otx_image img;
  int64_t first, count;
  int64_t num_pairs;      // ceil(ceil(count / 128) / 2)
  int num_hidden;
  const float* bias[OTX_MLP_MAX_HIDDEN + 1];
  int32_t* list;          // [count]: fallback rays (offsets from first), per-config regions
  uint32_t* list_count;   // [num_configs]
  unsigned long long* stats;
  int* err;
  float4* predict;        // [count] or null: {x, y, logit, 0}, position in mm
};

struct FusedMaps {
  CUtensorMap w[OTX_MLP_MAX_HIDDEN];  // layer l weights [width x in_l], boxes 256 x 64
  CUtensorMap out;                    // output layer [n_out x width], boxes 16 x 64
};

__device__ __forceinline__ bool aborted(volatile int* flag) { return *flag != 0; }

// First list slot of configuration c's region: its first ray in [first, first + count).
__device__ __forceinline__ int64_t list_region(const int64_t* offs, int c, int64_t first) {
  const int64_t o = offs[c];
  return (o > first ? o : first) - first;
}

// One block of 32 accumulator columns [c0, c0 + 32) of a row: bias, SiLU,
// BF16, stored into the row's 128-byte-swizzled operand (four 16-byte
// units, each written as soon as it is packed).
__device__ __forceinline__ void epilogue_block(const uint32_t r[32], const float* hbl, uint8_t* A,
                                               int c0, int row) {
  uint8_t* rp = A + (c0 >> 6) * F_A_CHUNK + row * 128;
  const int u0 = (c0 & 63) >> 3, sx = row & 7;
  const float* v = reinterpret_cast<const float*>(r);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float4 b0 = *reinterpret_cast<const float4*>(hbl + c0 + 8 * j);
    const float4 b1 = *reinterpret_cast<const float4*>(hbl + c0 + 8 * j + 4);
    uint4 w;
    w.x = silu2_bf16(fmaf(0.5f, v[8 * j + 0], b0.x), fmaf(0.5f, v[8 * j + 1], b0.y));
    w.y = silu2_bf16(fmaf(0.5f, v[8 * j + 2], b0.z), fmaf(0.5f, v[8 * j + 3], b0.w));
    w.z = silu2_bf16(fmaf(0.5f, v[8 * j + 4], b1.x), fmaf(0.5f, v[8 * j + 5], b1.y));
    w.w = silu2_bf16(fmaf(0.5f, v[8 * j + 6], b1.z), fmaf(0.5f, v[8 * j + 7], b1.w));
    *reinterpret_cast<uint4*>(rp + (((u0 + j) ^ sx) << 4)) = w;
  }
}

__global__ void __launch_bounds__(F_THREADS, 1)
    k_surrogate_fused(const __grid_constant__ FusedMaps maps, const __grid_constant__ FusedArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint8_t* sa = smem;                                   // 2 tiles x 64 KB
  uint8_t* sw = sa + 2 * F_A_BYTES;                     // weight ring
  uint8_t* swo = sw + F_STAGES * F_STAGE;               // output layer weights
  float* hb = reinterpret_cast<float*>(swo + (F_WIDTH / F_KC) * F_WOUT_CHUNK);  // bias / 2
  float* bout = hb + F_MAX_HIDDEN * F_WIDTH;
  uint64_t* wfull = reinterpret_cast<uint64_t*>(bout + F_OUT_N);
  uint64_t* wempty = wfull + F_STAGES;
  uint64_t* lo_ready = wempty + F_STAGES;  // [2] K columns 0-127 of a tile's operand written
  uint64_t* hi_ready = lo_ready + 2;       // [2] K columns 128-255 written
  uint64_t* acc0_full = hi_ready + 2;      // [2] accumulator columns 0-127 complete
  uint64_t* acc1_full = acc0_full + 2;     // [2] accumulator columns 128-255 complete
  uint64_t* woutfull = acc1_full + 2;
  uint64_t* mmadone = woutfull + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mmadone + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int L = a.num_hidden;

  // biases: hidden layers pre-halved (SiLU is evaluated on z / 2)
  for (int i = tid; i < L * F_WIDTH; i += F_THREADS) hb[i] = 0.5f * a.bias[i / F_WIDTH][i % F_WIDTH];
  if (tid < F_OUT_N) bout[tid] = tid < 3 ? a.bias[L][tid] : 0.f;
  if (tid == 0) {
    for (int s = 0; s < F_STAGES; ++s) {
      mbar_init(&wfull[s], 1);
      mbar_init(&wempty[s], 1);
    }
    for (int g = 0; g < 2; ++g) {
      mbar_init(&lo_ready[g], 32 * F_EPI_WARPS / 2);
      mbar_init(&hi_ready[g], 32 * F_EPI_WARPS / 2);
      mbar_init(&acc0_full[g], 1);
      mbar_init(&acc1_full[g], 1);
    }
    mbar_init(woutfull, 1);
    mbar_init(mmadone, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(tslot, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (warp == 0) {
    // ---------------------------------------------------------- producer
    if (lane == 0) {
      int64_t k = 0;  // stage loads issued
      mbar_expect_tx(woutfull, (F_WIDTH / F_KC) * F_WOUT_CHUNK);
      for (int kc = 0; kc < F_WIDTH / F_KC; ++kc)
        tma_load_2d(swo + kc * F_WOUT_CHUNK, &maps.out, kc * F_KC, 0, woutfull);
      bool ok = true;
      // stages in the issuer's order: layer 0 as two column halves (one
      // K chunk each, K = 16 used); every hidden layer as (columns 0-127,
      // K 0-127), (0-127, 128-255), (128-255, 0-127), (128-255, 128-255)
      for (int64_t p = blockIdx.x; ok && p < a.num_pairs; p += gridDim.x) {
        for (int l = 0; ok && l < L; ++l) {
          const int ns = l == 0 ? 2 : 4;
          for (int j = 0; j < ns; ++j) {
            const int s = (int)(k % F_STAGES);
            if (k >= F_STAGES &&
                (aborted(abort_flag) ||
                 !mbar_wait(&wempty[s], (uint32_t)(((k / F_STAGES) - 1) & 1)))) {
              ok = false;
              break;
            }
            uint8_t* dst = sw + s * F_STAGE;
            if (l == 0) {
              mbar_expect_tx(&wfull[s], F_WBOX);
              tma_load_2d(dst, &maps.w[0], 0, j * F_NH, &wfull[s]);
            } else {
              const int h = j >> 1, kh = j & 1;
              mbar_expect_tx(&wfull[s], F_STAGE);
              tma_load_2d(dst, &maps.w[l], kh * 2 * F_KC, h * F_NH, &wfull[s]);
              tma_load_2d(dst + F_WBOX, &maps.w[l], kh * 2 * F_KC + F_KC, h * F_NH, &wfull[s]);
            }
            ++k;
          }
        }
      }
      if (!ok) {
        *abort_flag = 1;
        atomicExch(a.err, 1);
      }
      // let every copy land before the CTA's shared memory is released
      for (int64_t j = k - F_STAGES > 0 ? k - F_STAGES : 0; j < k; ++j)
        mbar_wait(&wfull[j % F_STAGES], (uint32_t)((j / F_STAGES) & 1));
      mbar_wait(woutfull, 0);
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    if (lane == 0) {
      constexpr uint32_t ID_H = idesc_bf16(F_ROWS, F_NH);
      constexpr uint32_t ID_O = idesc_bf16(F_ROWS, F_OUT_N);
      int64_t k = 0;                          // weight stages consumed
      uint32_t lp[2] = {0u, 0u}, hp[2] = {0u, 0u};  // lo_ready / hi_ready parities
      bool ok = mbar_wait(woutfull, 0);
      // wait for both tiles' operand half (lo_ready or hi_ready)
      auto wait_half = [&](uint64_t* bars, uint32_t* par) {
        for (int g = 0; ok && g < 2; ++g) {
          if (aborted(abort_flag) || !mbar_wait(&bars[g], par[g])) {
            ok = false;
            break;
          }
          par[g] ^= 1u;
        }
        if (ok) tc_fence_after();
      };
      // one weight stage into column half h of both tiles' accumulators:
      // K chunks kc0, kc0 + 1 of the operand (nkk MMAs of K = 16 each);
      // accumulate unless `fresh` and first
      auto stage = [&](int h, int kc0, int nchunks, int nkk, bool fresh) {
        const int s = (int)(k % F_STAGES);
        if (!ok || !mbar_wait(&wfull[s], (uint32_t)((k / F_STAGES) & 1))) {
          ok = false;
          return;
        }
        tc_fence_after();
        for (int g = 0; g < 2; ++g) {
          const uint32_t acc = tbase + (uint32_t)(g * F_WIDTH + h * F_NH);
          for (int c = 0; c < nchunks; ++c) {
            const uint64_t ad = desc_sw128(sa + g * F_A_BYTES + (kc0 + c) * F_A_CHUNK);
            const uint64_t bd = desc_sw128(sw + s * F_STAGE + c * F_WBOX);
            for (int kk = 0; kk < nkk; ++kk)
              umma_bf16(acc, ad + 2 * kk, bd + 2 * kk, ID_H, !(fresh && c == 0 && kk == 0));
          }
        }
        umma_commit(&wempty[s]);
        ++k;
      };
      // Each hidden layer runs in column halves so that a half's epilogue
      // overlaps the other half's MMAs: the epilogue of columns 0-127
      // (which writes the next layer's K columns 0-127 over this layer's)
      // starts once every MMA reading K columns 0-127 has completed, while
      // the MMAs of columns 128-255 over K 128-255 still run.
      for (int64_t p = blockIdx.x; ok && p < a.num_pairs; p += gridDim.x) {
        for (int l = 0; ok && l < L; ++l) {
          if (l == 0) {
            wait_half(lo_ready, lp);  // ray inputs (K = 16, zero padded)
            stage(0, 0, 1, 1, true);
            stage(1, 0, 1, 1, true);
            if (ok) {
              umma_commit(&acc0_full[0]);
              umma_commit(&acc0_full[1]);
              umma_commit(&acc1_full[0]);
              umma_commit(&acc1_full[1]);
            }
            continue;
          }
          wait_half(lo_ready, lp);  // epilogue of columns 0-127 of layer l - 1 done
          stage(0, 0, 2, F_KC / 16, true);
          wait_half(hi_ready, hp);  // epilogue of columns 128-255 done
          stage(0, 2, 2, F_KC / 16, false);
          stage(1, 0, 2, F_KC / 16, true);
          if (ok) {  // columns 0-127 complete; K 0-127 of the operand read
            umma_commit(&acc0_full[0]);
            umma_commit(&acc0_full[1]);
          }
          stage(1, 2, 2, F_KC / 16, false);
          if (ok) {
            umma_commit(&acc1_full[0]);
            umma_commit(&acc1_full[1]);
          }
        }
        // output layer: resident weights, N = 16, into columns 0-15
        wait_half(lo_ready, lp);
        wait_half(hi_ready, hp);
        if (!ok) break;
        for (int g = 0; g < 2; ++g) {
          const uint32_t acc = tbase + (uint32_t)(g * F_WIDTH);
          for (int kc = 0; kc < F_WIDTH / F_KC; ++kc) {
            const uint64_t ad = desc_sw128(sa + g * F_A_BYTES + kc * F_A_CHUNK);
            const uint64_t bd = desc_sw128(swo + kc * F_WOUT_CHUNK);
            for (int kk = 0; kk < F_KC / 16; ++kk)
              umma_bf16(acc, ad + 2 * kk, bd + 2 * kk, ID_O, (kc | kk) != 0);
          }
        }
        umma_commit(&acc0_full[0]);
        umma_commit(&acc0_full[1]);
      }
      if (!ok) {
        *abort_flag = 1;
        atomicExch(a.err, 1);
      }
      // every MMA issued so far has finished before TMEM is freed
      umma_commit(mmadone);
      mbar_wait(mmadone, 0);
    }
  } else {
    // ---------------------------------------------------------- epilogue
    const int g = (warp - 2) / F_EPI_WARPS;       // tile slot
    const int lw = (warp - 2) % F_EPI_WARPS;
    const int ch = lw / 4;                        // column half of the hidden layers
    const int q = warp & 3;                       // TMEM lane quarter of this warp
    const int row = q * 32 + lane;
    uint8_t* A = sa + g * F_A_BYTES;
    const uint32_t tacc = tbase + (uint32_t)(g * F_WIDTH) + ((uint32_t)(q * 32) << 16);
    const int64_t* offs = reinterpret_cast<const int64_t*>(a.b.ray_offset);
    const float* cin = reinterpret_cast<const float*>(a.sg.config_inputs);
    const float* coef = reinterpret_cast<const float*>(a.sg.baseline);
    const uint8_t* trusted = reinterpret_cast<const uint8_t*>(a.sg.trusted);
    const bool bin = a.img.counts || a.img.flux;
    // this warp's column half: its accumulator barrier and the operand half
    // it writes (columns 0-127 also take the ray inputs and the output layer)
    uint64_t* my_full = ch == 0 ? &acc0_full[g] : &acc1_full[g];
    uint64_t* my_ready = ch == 0 ? &lo_ready[g] : &hi_ready[g];
    uint32_t cp = 0u;  // my_full parity
    unsigned long long n_rays = 0, n_net = 0, n_fb = 0;
    bool ok = true;
    for (int64_t p = blockIdx.x; ok && p < a.num_pairs; p += gridDim.x) {
      const int64_t t = 2 * p + g;
      const int64_t r = t * F_ROWS + row;  // offset of this row's ray from first
      const bool valid = r < a.count;
      int cfg = 0;
      float bx = 0.f, by = 0.f, wl = 0.f;
      if (ch == 0) {
        // ---- rays and network inputs of this tile
        float f[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) f[j] = 0.f;
        if (valid) {
          const int64_t gid = a.first + r;
          cfg = config_of(offs, a.b.num_configs, gid);
          const BatchInputs v = batch_inputs(a.b, cfg, gid - offs[cfg]);
          ray_features(a.b, v, f);
#pragma unroll
          for (int j = 0; j < 4; ++j) f[5 + j] = cin[cfg * 4 + j];
          baseline_xy(coef + (int64_t)cfg * 2 * OTX_SURROGATE_NBASE, f, bx, by);
          wl = v.wl;
        }
        uint32_t w[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = pack_bf16x2(f[2 * j], f[2 * j + 1]);
        uint8_t* rp = A + row * 128;
        const int sx = row & 7;
        *reinterpret_cast<uint4*>(rp + ((0 ^ sx) << 4)) = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4*>(rp + ((1 ^ sx) << 4)) = make_uint4(w[4], w[5], w[6], w[7]);
        fence_proxy_async_smem();
        tc_fence_before();
        mbar_arrive(my_ready);
      }
      // ---- hidden layers: TMEM -> bias, SiLU -> BF16 operand of the next
      // layer, this warp's column half (the next layer's K columns of the
      // same numbers)
      for (int l = 0; l < L; ++l) {
        if (aborted(abort_flag) || !mbar_wait(my_full, cp)) {
          ok = false;
          break;
        }
        cp ^= 1u;
        tc_fence_after();
        const float* hbl = hb + l * F_WIDTH;
        // four blocks of 32 columns; the TMEM load of block b + 1 is in
        // flight while block b is converted
        uint32_t ra[32], rb[32];
        __syncwarp();
        tmem_ld32_start(tacc + (uint32_t)(ch * 128), ra);
        tmem_wait32(ra);
        tmem_ld32_start(tacc + (uint32_t)(ch * 128 + 32), rb);
        epilogue_block(ra, hbl, A, ch * 128, row);
        tmem_wait32(rb);
        tmem_ld32_start(tacc + (uint32_t)(ch * 128 + 64), ra);
        epilogue_block(rb, hbl, A, ch * 128 + 32, row);
        tmem_wait32(ra);
        tmem_ld32_start(tacc + (uint32_t)(ch * 128 + 96), rb);
        epilogue_block(ra, hbl, A, ch * 128 + 64, row);
        tmem_wait32(rb);
        epilogue_block(rb, hbl, A, ch * 128 + 96, row);
        fence_proxy_async_smem();
        tc_fence_before();
        mbar_arrive(my_ready);
      }
      if (!ok) break;
      if (ch != 0) continue;
      // ---- output layer: land, bin or queue for the trace
      if (aborted(abort_flag) || !mbar_wait(my_full, cp)) {
        ok = false;
        break;
      }
      cp ^= 1u;
      tc_fence_after();
      {
        float v[16];
        __syncwarp();
        tmem_ld16(tacc, v);
        const float y0 = v[0] + bout[0], y1 = v[1] + bout[1], s = v[2] + bout[2];
        bool fb = false;
        if (valid && a.predict)
          a.predict[r] = make_float4(fmaf(a.sg.out_scale, y0, bx), fmaf(a.sg.out_scale, y1, by), s,
                                     0.f);
        if (valid && bin) {
          ++n_rays;
          const bool ok_cfg = trusted ? trusted[cfg] != 0 : true;
          if (!ok_cfg || !(fabsf(s) >= a.sg.logit_band)) {  // NaN logits are traced too
            fb = true;
          } else if (s > 0.f) {
            Ray ray;
            ray.px = fmaf(a.sg.out_scale, y0, bx);
            ray.py = fmaf(a.sg.out_scale, y1, by);
            ray.wl = wl;
            ray.inten = 1.f;
            ray.ok = true;
            if (sensor_bin(a.sensor, ray) >= 0) ++n_net;
            bin_ray(a.sensor, config_image(a.img, a.b.image_stride, cfg), ray);
          }
        }
        // append to the configuration's list, one atomic per configuration and warp
        const unsigned m = __ballot_sync(0xffffffffu, fb);
        if (m) {
          const unsigned same = __match_any_sync(0xffffffffu, fb ? cfg : -1);
          const unsigned grp = same & m;
          if (fb) {
            const int leader = __ffs(grp) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(a.list_count + cfg, (uint32_t)__popc(grp));
            base = __shfl_sync(grp, base, leader);
            const uint32_t idx = base + __popc(grp & ((1u << lane) - 1u));
            a.list[list_region(offs, cfg, a.first) + idx] = (int32_t)r;
            ++n_fb;
          }
        }
      }
    }
    if (!ok) {
      *abort_flag = 1;
      if (lane == 0) atomicExch(a.err, 1);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      n_rays += __shfl_xor_sync(0xffffffffu, n_rays, o);
      n_net += __shfl_xor_sync(0xffffffffu, n_net, o);
      n_fb += __shfl_xor_sync(0xffffffffu, n_fb, o);
    }
    if (lane == 0 && ch == 0) {
      if (n_rays) atomicAdd(a.stats + 0, n_rays);
      if (n_fb) atomicAdd(a.stats + 1, n_fb);
      if (n_net) atomicAdd(a.stats + 2, n_net);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tbase, 512);
}

constexpr int FB_BLOCK = 256;

struct FallbackArgs {
  otx_batch b;
  int64_t first, count;
  const int32_t* list;
  const uint32_t* list_count;
  otx_image img;
  unsigned long long* stats;
};

// Trace the queued rays: CTA (x, c) takes configuration c's list.
template <class... Ks>
__global__ void __launch_bounds__(FB_BLOCK)
    k_surrogate_fallback(const __grid_constant__ otx_system sys,
                         const __grid_constant__ FallbackArgs a) {
  __shared__ otx_surface surf[OTX_MAX_SURFACES];
  const int c = blockIdx.y, tid = threadIdx.x;
  const int64_t* offs = reinterpret_cast<const int64_t*>(a.b.ray_offset);
  const int64_t lo = list_region(offs, c, a.first);
  const int64_t hi_ray = offs[c + 1] - a.first;
  const int64_t cap = (hi_ray < a.count ? hi_ray : a.count) - lo;
  int64_t n = a.list_count[c];
  if (n > cap) n = cap > 0 ? cap : 0;
  if (n == 0 || (int64_t)blockIdx.x * FB_BLOCK >= n) return;  // uniform over the CTA
  const int words = sys.num_surfaces * (int)(sizeof(otx_surface) / 4);
  const int* src = reinterpret_cast<const int*>(sys.surfaces);
  int* dst = reinterpret_cast<int*>(surf);
  for (int w = tid; w < words; w += FB_BLOCK) dst[w] = src[w];
  __syncthreads();
  const otx_surface* ov = reinterpret_cast<const otx_surface*>(a.b.overrides);
  for (int j = 0; j < a.b.num_overrides; ++j) {
    const int ow = (int)(sizeof(otx_surface) / 4);
    const int* os = reinterpret_cast<const int*>(ov + (int64_t)c * a.b.num_overrides + j);
    int* od = reinterpret_cast<int*>(surf + a.b.override_index[j]);
    for (int w = tid; w < ow; w += FB_BLOCK) od[w] = os[w];
  }
  __syncthreads();
  const otx_image img = config_image(a.img, a.b.image_stride, c);
  const bool bin = img.counts || img.flux;
  int binned = 0;
  for (int64_t i = (int64_t)blockIdx.x * FB_BLOCK + tid; i < n; i += (int64_t)gridDim.x * FB_BLOCK) {
    const int64_t gid = a.first + a.list[lo + i];
    Ray ray;
    batch_ray(a.b, c, gid - offs[c], ray);
    propagate_all<Ks...>(sys, surf, ray);
    if (bin) {
      if (ray.ok && sensor_bin(sys.sensor, ray) >= 0) ++binned;
      bin_ray(sys.sensor, img, ray);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) binned += __shfl_xor_sync(0xffffffffu, binned, o);
  if ((tid & 31) == 0 && binned) atomicAdd(a.stats + 3, (unsigned long long)binned);
}

static int device_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 132;
}

}  // namespace otx

using namespace otx;

extern "C" {

int64_t otx_surrogate_image_fused_workspace(const otx_batch* batch, const otx_mlp* net,
                                            int64_t count) {
  if (!batch || !net || count < 0 || batch->num_configs < 1) return -1;
  return (count * 4 + 255) / 256 * 256 + ((int64_t)batch->num_configs * 4 + 255) / 256 * 256;
}

otx_status otx_surrogate_image_fused(const otx_system* base, const otx_batch* batch,
                                     const otx_surrogate* sg, const otx_mlp* net, int64_t first,
                                     int64_t count, const otx_image* image, float* predict,
                                     void* workspace, int64_t workspace_bytes,
                                     unsigned long long* stats, int32_t* err, void* stream) {
  if (!base || !batch || !sg || !net || !stats || !err || first < 0 || count < 0)
    return OTX_ERR_INVALID;
  if (reinterpret_cast<uintptr_t>(predict) & 15) return OTX_ERR_INVALID;
  const otx_batch& b = *batch;
  if (b.num_configs < 1 || !b.ray_offset || sg->num_configs != b.num_configs ||
      !sg->config_inputs || !sg->baseline || !(sg->out_scale > 0.f))
    return OTX_ERR_INVALID;
  // the fallback kernel's grid holds one configuration per y index (at most
  // 65535): reject larger batches before any GPU work
  if (b.num_configs > 65535) return OTX_ERR_SIZE;
  if (const otx_status vs = validate_system(base)) return vs;
  if (base->input_mode != OTX_INPUT_GRID_INFINITY) return OTX_ERR_INVALID;
  if (!(base->flags & OTX_SYS_FLAG_FINAL_IDENTITY)) return OTX_ERR_UNSUPPORTED;
  if (b.num_overrides < 0 || b.num_overrides > OTX_BATCH_MAX_OVERRIDES) return OTX_ERR_SIZE;
  for (int j = 0; j < b.num_overrides; ++j)
    if (b.override_index[j] < 0 || b.override_index[j] >= base->num_surfaces)
      return OTX_ERR_INVALID;
  if (b.num_overrides > 0 && !b.overrides) return OTX_ERR_INVALID;
  // the network this kernel is built for: 9 inputs, hidden width 256, 3 outputs
  if (net->num_hidden < 1 || net->num_hidden > OTX_MLP_MAX_HIDDEN || net->width != F_WIDTH ||
      net->num_inputs != OTX_SURROGATE_NIN || net->num_outputs != 3)
    return OTX_ERR_UNSUPPORTED;
  const int L = net->num_hidden;
  for (int l = 0; l <= L; ++l) {
    if (!net->w[l] || !net->b[l] || (net->w[l] & 15) || net->ld[l] % 8) return OTX_ERR_INVALID;
    const int in = l == 0 ? net->num_inputs : F_WIDTH;
    if (net->ld[l] < in) return OTX_ERR_INVALID;
  }
  // the network predicts no direction: no cosine moment from this path
  if (image && image->cos_moment) return OTX_ERR_UNSUPPORTED;
  const bool bin = image && (image->counts || image->flux);
  if (bin && (base->sensor.num_x < 1 || base->sensor.num_y < 1 || base->sensor.num_w < 1 ||
              !(base->sensor.width_x > 0.f) || !(base->sensor.width_y > 0.f) ||
              b.image_stride < base->sensor.num_w * base->sensor.num_x * base->sensor.num_y))
    return OTX_ERR_INVALID;
  if (count > 0x7fffffffLL) return OTX_ERR_SIZE;  // list entries are int32 offsets
  const int64_t need = otx_surrogate_image_fused_workspace(batch, net, count);
  if (!workspace || workspace_bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return OTX_ERR_INVALID;
  if (count == 0) return OTX_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

  // workspace: fallback list, per-configuration counts
  char* ws = reinterpret_cast<char*>(workspace);
  int32_t* list = reinterpret_cast<int32_t*>(ws);
  uint32_t* list_count = reinterpret_cast<uint32_t*>(ws + (count * 4 + 255) / 256 * 256);
  FusedMaps maps;
  memset(&maps, 0, sizeof(maps));
  const int sms = device_sms();
  for (int l = 0; l < L; ++l) {
    const int in = l == 0 ? net->num_inputs : F_WIDTH;
    if (!make_map(&maps.w[l], reinterpret_cast<const void*>(net->w[l]), F_WIDTH, in, net->ld[l],
                  F_NH))
      return OTX_ERR_CUDA;
  }
  if (!make_map(&maps.out, reinterpret_cast<const void*>(net->w[L]), 3, F_WIDTH, net->ld[L],
                F_OUT_N))
    return OTX_ERR_CUDA;

  otx_system sys = *base;
  otx_sensor& S = sys.sensor;
  S.inv_width_x = S.width_x > 0.f ? 1.f / S.width_x : 0.f;
  S.inv_width_y = S.width_y > 0.f ? 1.f / S.width_y : 0.f;
  S.inv_width_w = (S.w_hi > S.w_lo) ? (float)S.num_w / (S.w_hi - S.w_lo) : 0.f;

  if (cudaMemsetAsync(list_count, 0, (size_t)b.num_configs * 4, st) != cudaSuccess)
    return OTX_ERR_CUDA;

  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.b = b;
  a.sg = *sg;
  a.sensor = S;
  if (bin) a.img = *image;
  a.first = first;
  a.count = count;
  const int64_t tiles = (count + F_ROWS - 1) / F_ROWS;
  a.num_pairs = (tiles + 1) / 2;
  a.num_hidden = L;
  for (int l = 0; l <= L; ++l) a.bias[l] = reinterpret_cast<const float*>(net->b[l]);
  a.list = list;
  a.list_count = list_count;
  a.stats = stats;
  a.err = err;
  a.predict = reinterpret_cast<float4*>(predict);

  // the shared-memory limit is an attribute of the function in the current
  // device's context: set on every call (cheap), so every device a process
  // drives gets it
  if (cudaFuncSetAttribute(k_surrogate_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)F_SMEM) != cudaSuccess)
    return OTX_ERR_CUDA;
  const int64_t grid = a.num_pairs < sms ? a.num_pairs : sms;
  k_surrogate_fused<<<(unsigned)grid, F_THREADS, F_SMEM, st>>>(maps, a);
  if (cudaGetLastError() != cudaSuccess) return OTX_ERR_CUDA;
  if (!bin) return OTX_OK;  // predictions only: nothing was queued

  FallbackArgs f;
  memset(&f, 0, sizeof(f));
  f.b = b;
  f.first = first;
  f.count = count;
  f.list = list;
  f.list_count = list_count;
  if (bin) f.img = *image;
  f.stats = stats;
  const int gx = (4 * sms + b.num_configs - 1) / b.num_configs;
  const dim3 fgrid((unsigned)(gx > 0 ? gx : 1), (unsigned)b.num_configs);
  if (shape_matches<BObject, BSphere, BGrating, BSensor>(sys))
    k_surrogate_fallback<BObject, BSphere, BGrating, BSensor><<<fgrid, FB_BLOCK, 0, st>>>(sys, f);
  else
    k_surrogate_fallback<><<<fgrid, FB_BLOCK, 0, st>>>(sys, f);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}

}  // extern "C"
