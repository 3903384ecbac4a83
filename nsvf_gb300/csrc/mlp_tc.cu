// Field MLP on the Blackwell tensor cores: 32 -> 128 -> 128 -> 128 -> 128 -> 4
// (ReLU between layers), BF16 operands, FP32 accumulation in TMEM.
//
// The reference evaluates its field with nn.Linear in FP32 (cuBLAS), one
// layer at a time, materialising every hidden activation in HBM
// (fairnr/modules/renderer.py:105-111, fairnr/modules/implicit.py:42-75).
// Here a persistent CTA per SM keeps all five weight matrices in shared
// memory (108 KB) and streams 128-sample tiles through them: the hidden
// activations never leave the SM.
//
// CTA = 9 warps. Warps 0-3 and 4-7 are two epilogue warpgroups, each owning
// one tile slot (TMEM columns [256*g, 256*g + 144)) so that one slot's
// epilogue overlaps the other slot's MMAs. Warp 8 allocates TMEM and one of
// its lanes issues the tcgen05.mma instructions. Per layer:
//   epilogue g writes A (bf16, K-major) to smem -> fence.proxy.async ->
//   arrives on act_ready[g] -> MMA thread issues the K/16 MMAs ->
//   tcgen05.commit arrives on mma_done[g] -> epilogue g reads D with
//   tcgen05.ld, adds the bias, applies ReLU, rounds to bf16 -> next layer.
// Every wait is bounded; on a timeout the CTA records bit 3 in *err, stops,
// and still frees its TMEM.
#include "common.cuh"
#include "tc_common.cuh"

using namespace nsvf_tc;

namespace {

constexpr int E = 32;       // embedding width (first layer K)
constexpr int HID = 128;    // hidden width
constexpr int NOUT = 16;    // N of the last MMA (4 outputs used)
constexpr int TILE = 128;   // samples per MMA tile (M)
constexpr int kThreads = 9 * 32;
constexpr uint32_t kTmemCols = 512;

struct __align__(128) MlpSmem {
  __nv_bfloat16 w0[HID * E];
  __nv_bfloat16 wh[3][HID * HID];
  __nv_bfloat16 w4[NOUT * HID];
  __nv_bfloat16 ain[2][TILE * E];
  __nv_bfloat16 ah[2][TILE * HID];
  float bias[4][HID];
  float bias4[NOUT];
  uint64_t mma_done[2];
  uint64_t act_ready[2];
  uint32_t tmem_base;
  int abort;
};

struct MlpParams {
  const float *emb;                  // [ns, 32] fp32
  const __nv_bfloat16 *w[5];         // row-major [N, K]: 128x32, 3x 128x128, 4x128
  const float *b[5];                 // [128] x4, [4]
  float *out;                        // [ns, 4]: sigma, r, g, b
  int64_t ns;
  int32_t *err;
};

// Copy a row-major [rows, K] bf16 matrix into the K-major core-matrix layout
// (rows >= valid_rows are zero).
__device__ void stage_weights(__nv_bfloat16 *dst, const __nv_bfloat16 *src, int rows,
                              int valid_rows, int K) {
  int chunks = rows * (K / 8);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    int r = c / (K / 8), kc = c % (K / 8);
    uint4 v = make_uint4(0, 0, 0, 0);
    if (r < valid_rows) v = *reinterpret_cast<const uint4 *>(src + (size_t)r * K + kc * 8);
    *reinterpret_cast<uint4 *>(reinterpret_cast<uint8_t *>(dst) + kmajor_off(r, kc * 8, K)) = v;
  }
}

__device__ __forceinline__ void issue_layer(uint32_t d_tmem, const __nv_bfloat16 *A,
                                            const __nv_bfloat16 *B, int K, int N) {
  uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
  uint32_t sbo = (uint32_t)(K / 8) * 128u;
  uint32_t idesc = idesc_bf16_f32(TILE, N);
  for (int k = 0; k < K / 16; ++k) {
    uint64_t ad = sdesc(a0 + 256u * k, 128u, sbo);
    uint64_t bd = sdesc(b0 + 256u * k, 128u, sbo);
    mma_bf16(d_tmem, ad, bd, idesc, k > 0 ? 1u : 0u);
  }
}

__global__ void __launch_bounds__(kThreads, 1) mlp_tc_kernel(const MlpParams p) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  MlpSmem &S = *reinterpret_cast<MlpSmem *>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  stage_weights(S.w0, p.w[0], HID, HID, E);
  for (int l = 0; l < 3; ++l) stage_weights(S.wh[l], p.w[l + 1], HID, HID, HID);
  stage_weights(S.w4, p.w[4], NOUT, 4, HID);
  for (int i = tid; i < 4 * HID; i += blockDim.x) S.bias[i / HID][i % HID] = p.b[i / HID][i % HID];
  if (tid < NOUT) S.bias4[tid] = tid < 4 ? p.b[4][tid] : 0.0f;
  if (tid == 0) {
    mbar_init(&S.mma_done[0], 1);
    mbar_init(&S.mma_done[1], 1);
    mbar_init(&S.act_ready[0], 128);
    mbar_init(&S.act_ready[1], 128);
    S.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 8) tmem_alloc(&S.tmem_base, kTmemCols);
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = S.tmem_base;
  volatile int *abort = &S.abort;
  const int64_t n_tiles = (p.ns + TILE - 1) / TILE;
  const int64_t G = gridDim.x, b = blockIdx.x;

  if (warp == 8) {
    if (lane == 0) {
      uint32_t ph[2] = {0u, 0u};
      bool ok = true;
      for (int64_t i = 0; ok; ++i) {
        bool has[2] = {(2 * i) * G + b < n_tiles, (2 * i + 1) * G + b < n_tiles};
        if (!has[0]) break;
        for (int layer = 0; layer < 5 && ok; ++layer) {
          for (int g = 0; g < 2 && ok; ++g) {
            if (!has[g]) continue;
            if (!mbar_wait(&S.act_ready[g], ph[g], abort)) { ok = false; break; }
            ph[g] ^= 1u;
            fence_after_sync();
            uint32_t d = tmem + 256u * g;
            if (layer == 0) issue_layer(d, S.ain[g], S.w0, E, HID);
            else if (layer < 4) issue_layer(d, S.ah[g], S.wh[layer - 1], HID, HID);
            else issue_layer(d + 128u, S.ah[g], S.w4, HID, NOUT);
            mma_commit(&S.mma_done[g]);
          }
        }
      }
    }
    __syncwarp();
  } else {
    const int g = warp >> 2, q = warp & 3;
    const int row = q * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16) + 256u * g;
    uint8_t *ah = reinterpret_cast<uint8_t *>(S.ah[g]);
    uint8_t *ain = reinterpret_cast<uint8_t *>(S.ain[g]);
    uint32_t ph = 0;
    bool ok = true;
    for (int64_t i = 0; ok; ++i) {
      int64_t tile = (2 * i + g) * G + b;
      if (tile >= n_tiles) break;
      int64_t r = tile * TILE + row;
      // input tile: fp32 embedding row -> bf16, K-major
      {
        float4 x[8];
        if (r < p.ns) {
          const float4 *src = reinterpret_cast<const float4 *>(p.emb + r * E);
#pragma unroll
          for (int j = 0; j < 8; ++j) x[j] = __ldg(src + j);
        } else {
#pragma unroll
          for (int j = 0; j < 8; ++j) x[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          uint4 v;
          v.x = pack_bf16x2(x[2 * c].x, x[2 * c].y);
          v.y = pack_bf16x2(x[2 * c].z, x[2 * c].w);
          v.z = pack_bf16x2(x[2 * c + 1].x, x[2 * c + 1].y);
          v.w = pack_bf16x2(x[2 * c + 1].z, x[2 * c + 1].w);
          *reinterpret_cast<uint4 *>(ain + kmajor_off(row, c * 8, E)) = v;
        }
      }
      fence_async_smem();
      mbar_arrive(&S.act_ready[g]);
      for (int layer = 0; layer < 4; ++layer) {
        if (!mbar_wait(&S.mma_done[g], ph, abort)) { ok = false; break; }
        ph ^= 1u;
        fence_after_sync();
        const float *bias = S.bias[layer];
#pragma unroll 1
        for (int c = 0; c < HID; c += 16) {
          float v[16];
          tmem_ld16(tl + c, v);
          tmem_wait_ld();
          uint32_t pk[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            float a0 = fmaxf(v[2 * j] + bias[c + 2 * j], 0.0f);
            float a1 = fmaxf(v[2 * j + 1] + bias[c + 2 * j + 1], 0.0f);
            pk[j] = pack_bf16x2(a0, a1);
          }
          *reinterpret_cast<uint4 *>(ah + kmajor_off(row, c, HID)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
          *reinterpret_cast<uint4 *>(ah + kmajor_off(row, c + 8, HID)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
        fence_before_sync();
        fence_async_smem();
        mbar_arrive(&S.act_ready[g]);
      }
      if (!ok) break;
      if (!mbar_wait(&S.mma_done[g], ph, abort)) { ok = false; break; }
      ph ^= 1u;
      fence_after_sync();
      float v[16];
      tmem_ld16(tl + 128u, v);
      tmem_wait_ld();
      fence_before_sync();
      if (r < p.ns)
        reinterpret_cast<float4 *>(p.out)[r] =
            make_float4(v[0] + S.bias4[0], v[1] + S.bias4[1], v[2] + S.bias4[2], v[3] + S.bias4[3]);
    }
  }
  fence_before_sync();
  __syncthreads();
  if (tid == 0 && S.abort && p.err) atomicOr(p.err, 8);
  if (warp == 8) {
    fence_after_sync();
    tmem_dealloc(tmem, kTmemCols);
  }
}

int g_num_sms = 0;

}  // namespace

extern "C" {

int nsvf_mlp_forward_bf16(int64_t n_samples, const float *emb, const void *const weights[5],
                          const float *const biases[5], float *out, int32_t *err, void *stream) {
  if (n_samples < 0 || !weights || !biases) return NSVF_ERR_INVALID;
  if (n_samples == 0) return NSVF_OK;
  if (!emb || !out) return NSVF_ERR_INVALID;
  for (int l = 0; l < 5; ++l)
    if (!weights[l] || !biases[l] || (((uintptr_t)weights[l]) & 15)) return NSVF_ERR_INVALID;
  if ((((uintptr_t)emb) | ((uintptr_t)out)) & 15) return NSVF_ERR_INVALID;
  static bool attr_set = false;
  size_t smem = sizeof(MlpSmem) + 1024;
  if (!attr_set) {
    if (cudaFuncSetAttribute(mlp_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return NSVF_ERR_CUDA;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    attr_set = true;
  }
  MlpParams p;
  p.emb = emb;
  for (int l = 0; l < 5; ++l) {
    p.w[l] = (const __nv_bfloat16 *)weights[l];
    p.b[l] = biases[l];
  }
  p.out = out;
  p.ns = n_samples;
  p.err = err;
  int64_t n_tiles = (n_samples + TILE - 1) / TILE;
  int64_t grid = (n_tiles + 1) / 2;
  if (grid > g_num_sms) grid = g_num_sms;
  if (grid < 1) grid = 1;
  mlp_tc_kernel<<<(int)grid, kThreads, smem, (cudaStream_t)stream>>>(p);
  return nsvf_launch_status();
}

}  // extern "C"
