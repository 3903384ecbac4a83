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
constexpr int NB = 4;       // input tile ring depth
constexpr int kMmaWarp = 8;
constexpr int kLoaderWarp0 = 9;                 // warps 9..16: two loader warpgroups
constexpr int kThreads = 17 * 32;
constexpr uint32_t kTmemCols = 512;

struct __align__(128) MlpSmem {
  __nv_bfloat16 w0[HID * E];
  __nv_bfloat16 wh[3][HID * HID];
  __nv_bfloat16 w4[NOUT * HID];
  __nv_bfloat16 ain[NB][TILE * E];
  __nv_bfloat16 ah[2][TILE * HID];
  float bias[4][HID];
  float bias4[NOUT];
  uint64_t mma_done[2][5];   // per slot and layer: one phase per tile
  uint64_t act_ready[2];     // epilogue -> MMA: hidden activations written
  uint64_t in_full[NB];      // loaders -> MMA: input tile written
  uint64_t in_empty[NB];     // MMA -> loaders: first layer done reading
  uint32_t tmem_base;
  int abort;
};

// Where a tile's 128 rows come from and where their outputs go.
enum Mode : int {
  kEmbIn = 0,      // rows = embeddings emb[n, 32]; out[n] = (sigma, r, g, b)
  kSamplesIn = 1,  // rows = samples (voxel id, xyz): trilinear interpolation in
                   // the input stage; out[n] = (sigma, r, g, b)
  kPrune = 2,      // rows = bits^3 points per voxel; per-voxel score reduced
                   // with atomics into score[v]
};

struct MlpParams {
  const float *emb;                  // kEmbIn: [ns, 32] fp32
  const int32_t *vox;                // kSamplesIn: [ns] voxel ids
  const float4 *xyzd;                // kSamplesIn: [ns] (x, y, z, .)
  const float *centers;              // [n_vox, 3] voxel centres
  const int32_t *feats;              // [n_vox, 8] corner ids
  const float4 *values;              // [n_keys, 32] corner embeddings (fp32)
  int64_t n_vox, n_keys;
  float voxel_size;
  int bits;                          // kPrune: points per axis
  float step;                        // kPrune: rule 1 step
  int rule;                          // kPrune: 0 = min exp(-relu s), 1 = max 1-exp(-relu(s) step)
  unsigned int *score;               // kPrune: [n_vox] float bits
  const __nv_bfloat16 *w[5];         // row-major [N, K]: 128x32, 3x 128x128, 4x128
  const float *b[5];                 // [128] x4, [4]
  float *out;                        // [ns, 4]: sigma, r, g, b
  int64_t ns;                        // rows (the capacity when ns_dev is set)
  const int64_t *ns_dev;             // optional: row count read on the device
  int32_t *err;
};

// The trilinear weights of the interpolation kernel (interp.cu), same
// operations in the same order, so a sample's FP32 embedding is identical.
__device__ __forceinline__ float corner_weight(const float q[3], int k) {
  float a = (k & 4) ? q[0] : 1.0f - q[0];
  float b = (k & 2) ? q[1] : 1.0f - q[1];
  float c = (k & 1) ? q[2] : 1.0f - q[2];
  return a * b * c;
}

// emb[32] of a point x in voxel v (ids checked; out-of-range reads skipped).
__device__ __forceinline__ void interp_point(const MlpParams &p, int64_t v, float x, float y,
                                             float z, float (&e)[32], bool &bad) {
#pragma unroll
  for (int i = 0; i < 32; ++i) e[i] = 0.0f;
  if (v < 0 || v >= p.n_vox) { bad = true; return; }
  const float *c = p.centers + v * 3;
  float q[3] = {(x - c[0]) / p.voxel_size + 0.5f, (y - c[1]) / p.voxel_size + 0.5f,
                (z - c[2]) / p.voxel_size + 0.5f};
  const int4 f0 = reinterpret_cast<const int4 *>(p.feats)[v * 2];
  const int4 f1 = reinterpret_cast<const int4 *>(p.feats)[v * 2 + 1];
  const int keys[8] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, f1.z, f1.w};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    int64_t key = keys[k];
    if (key < 0 || key >= p.n_keys) { bad = true; continue; }
    float w = corner_weight(q, k);
    const float4 *src = p.values + key * 8;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float4 val = __ldg(src + j);
      e[4 * j + 0] = fmaf(w, val.x, e[4 * j + 0]);
      e[4 * j + 1] = fmaf(w, val.y, e[4 * j + 1]);
      e[4 * j + 2] = fmaf(w, val.z, e[4 * j + 2]);
      e[4 * j + 3] = fmaf(w, val.w, e[4 * j + 3]);
    }
  }
}

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

// bf16x2 of (relu(lo), relu(hi)) with round-to-nearest-even, one instruction
__device__ __forceinline__ uint32_t pack_relu_bf16x2(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %2, %1;\n" : "=r"(d) : "f"(lo), "f"(hi));
  return d;
}

// The input row `r` of a tile (embedding, interpolated sample or pruning
// point) as 32 FP32 values; rows >= ns are zero.
template <int MODE>
__device__ __forceinline__ void input_row(const MlpParams &p, int64_t r, int64_t ns, float (&e)[32],
                                          bool &bad) {
  if (r >= ns) {
#pragma unroll
    for (int j = 0; j < 32; ++j) e[j] = 0.0f;
    return;
  }
  if (MODE == kEmbIn) {
    const float4 *src = reinterpret_cast<const float4 *>(p.emb + r * E);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float4 x = __ldg(src + j);
      e[4 * j] = x.x; e[4 * j + 1] = x.y; e[4 * j + 2] = x.z; e[4 * j + 3] = x.w;
    }
  } else if (MODE == kSamplesIn) {
    float4 x = p.xyzd[r];
    interp_point(p, p.vox[r], x.x, x.y, x.z, e, bad);
  } else {
    // point i of voxel v: offset_points order (x slowest), offset
    // ((2 i_d + 1) - bits) / (bits - 1) times half a voxel
    int64_t P = (int64_t)p.bits * p.bits * p.bits;
    int64_t v = r / P, i = r % P;
    int ix = (int)(i / (p.bits * p.bits)), iy = (int)((i / p.bits) % p.bits), iz = (int)(i % p.bits);
    const float *c = p.centers + v * 3;
    float hv = p.voxel_size / 2.0f, den = (float)(p.bits - 1);
    float x = c[0] + ((float)(2 * ix + 1 - p.bits) / den) * hv;
    float y = c[1] + ((float)(2 * iy + 1 - p.bits) / den) * hv;
    float z = c[2] + ((float)(2 * iz + 1 - p.bits) / den) * hv;
    interp_point(p, v, x, y, z, e, bad);
  }
}

// Persistent CTA (one per SM), 17 warps:
//   warps 0-3, 4-7  epilogue warpgroups of tile slots 0 and 1 (TMEM columns
//                   [256 g, 256 g + 144)): bias + ReLU + bf16 of each hidden
//                   layer back to shared memory, and the output stage;
//   warp 8          TMEM allocation; lane 0 issues all tcgen05.mma;
//   warps 9-16      two loader warpgroups that build the input tiles (the
//                   embedding gathers and interpolation) into a ring of NB
//                   buffers ahead of the MMAs.
// The CTA's tiles are b, b + G, b + 2G, ...: local tile i uses slot i % 2,
// ring buffer i % NB and loader group i % 2. Each mbarrier completes exactly
// one phase per use and every waiter consumes it before the next phase can
// complete, so parity waits are unambiguous.
template <int MODE>
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
    for (int g = 0; g < 2; ++g) {
      for (int l = 0; l < 5; ++l) mbar_init(&S.mma_done[g][l], 1);
      mbar_init(&S.act_ready[g], 128);
    }
    for (int q = 0; q < NB; ++q) {
      mbar_init(&S.in_full[q], 128);
      mbar_init(&S.in_empty[q], 1);
    }
    S.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == kMmaWarp) tmem_alloc(&S.tmem_base, kTmemCols);
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = S.tmem_base;
  volatile int *abort = &S.abort;
  // With ns_dev the row count comes from device memory (a count produced by
  // an earlier kernel on the stream), clamped to the buffers' capacity p.ns.
  int64_t ns = p.ns;
  if (p.ns_dev) {
    int64_t d = *p.ns_dev;
    if (d > ns && tid == 0 && p.err) atomicOr(p.err, 2);
    ns = d < 0 ? 0 : (d < ns ? d : ns);
  }
  const int64_t n_tiles = (ns + TILE - 1) / TILE;
  const int64_t G = gridDim.x, b = blockIdx.x;
  auto tile_of = [&](int64_t i) { return b + i * G; };

  if (warp == kMmaWarp) {
    if (lane == 0) {
      uint32_t ph_act[2] = {0u, 0u};
      bool ok = true;
      for (int64_t i = 0; ok; i += 2) {
        bool has[2] = {tile_of(i) < n_tiles, tile_of(i + 1) < n_tiles};
        if (!has[0]) break;
        for (int layer = 0; layer < 5 && ok; ++layer) {
          for (int g = 0; g < 2 && ok; ++g) {
            if (!has[g]) continue;
            int64_t ii = i + g;
            uint32_t d = tmem + 256u * g;
            if (layer == 0) {
              int q = (int)(ii % NB);
              if (!mbar_wait(&S.in_full[q], (uint32_t)((ii / NB) & 1), abort)) { ok = false; break; }
              fence_after_sync();
              issue_layer(d, S.ain[q], S.w0, E, HID);
              mma_commit(&S.mma_done[g][0]);
              mma_commit(&S.in_empty[q]);
            } else {
              if (!mbar_wait(&S.act_ready[g], ph_act[g], abort)) { ok = false; break; }
              ph_act[g] ^= 1u;
              fence_after_sync();
              if (layer < 4) issue_layer(d, S.ah[g], S.wh[layer - 1], HID, HID);
              else issue_layer(d + 128u, S.ah[g], S.w4, HID, NOUT);
              mma_commit(&S.mma_done[g][layer]);
            }
          }
        }
      }
    }
    __syncwarp();
  } else if (warp >= kLoaderWarp0) {
    // loaders: every wait result is taken warp-uniformly
    const int L = (warp - kLoaderWarp0) >> 2;
    const int row = ((warp - kLoaderWarp0) & 3) * 32 + lane;
    for (int64_t i = L;; i += 2) {
      int64_t tile = tile_of(i);
      if (tile >= n_tiles) break;
      int q = (int)(i % NB);
      // the first round finds every buffer free (parity of the phase before
      // the barrier's first)
      uint32_t par = (uint32_t)(((i / NB) & 1) ^ 1);
      if (!__all_sync(0xffffffffu, mbar_wait(&S.in_empty[q], par, abort))) break;
      float e[32];
      bool bad = false;
      input_row<MODE>(p, tile * TILE + row, ns, e, bad);
      if (bad && p.err) atomicOr(p.err, 4);
      uint8_t *ain = reinterpret_cast<uint8_t *>(S.ain[q]);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        uint4 v;
        v.x = pack_bf16x2(e[8 * c + 0], e[8 * c + 1]);
        v.y = pack_bf16x2(e[8 * c + 2], e[8 * c + 3]);
        v.z = pack_bf16x2(e[8 * c + 4], e[8 * c + 5]);
        v.w = pack_bf16x2(e[8 * c + 6], e[8 * c + 7]);
        *reinterpret_cast<uint4 *>(ain + kmajor_off(row, c * 8, E)) = v;
      }
      fence_async_smem();
      mbar_arrive(&S.in_full[q]);
    }
  } else {
    // Epilogue warpgroups. Every wait result is taken warp-uniformly
    // (__all_sync), so the .sync.aligned tcgen05.ld and the warp shuffles
    // below always run with all 32 lanes, also when a timeout makes the CTA
    // unwind.
    const int g = warp >> 2, q4 = warp & 3;
    const int row = q4 * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(q4 * 32) << 16) + 256u * g;
    uint8_t *ah = reinterpret_cast<uint8_t *>(S.ah[g]);
    bool ok = true;
    for (int64_t i = g; ok; i += 2) {
      int64_t tile = tile_of(i);
      if (tile >= n_tiles) break;
      const uint32_t par = (uint32_t)((i >> 1) & 1);
      int64_t r = tile * TILE + row;
      for (int layer = 0; layer < 4; ++layer) {
        if (!__all_sync(0xffffffffu, mbar_wait(&S.mma_done[g][layer], par, abort))) { ok = false; break; }
        fence_after_sync();
        const float *bias = S.bias[layer];
#pragma unroll 1
        for (int c = 0; c < HID; c += 32) {
          float v[32];
          tmem_ld16(tl + c, *reinterpret_cast<float(*)[16]>(v));
          tmem_ld16(tl + c + 16, *reinterpret_cast<float(*)[16]>(v + 16));
          tmem_wait_ld();
          uint32_t pk[16];
#pragma unroll
          for (int j = 0; j < 16; ++j)
            pk[j] = pack_relu_bf16x2(v[2 * j] + bias[c + 2 * j], v[2 * j + 1] + bias[c + 2 * j + 1]);
#pragma unroll
          for (int h = 0; h < 4; ++h)
            *reinterpret_cast<uint4 *>(ah + kmajor_off(row, c + 8 * h, HID)) =
                make_uint4(pk[4 * h], pk[4 * h + 1], pk[4 * h + 2], pk[4 * h + 3]);
        }
        fence_before_sync();
        fence_async_smem();
        mbar_arrive(&S.act_ready[g]);
      }
      if (!ok) break;
      if (!__all_sync(0xffffffffu, mbar_wait(&S.mma_done[g][4], par, abort))) { ok = false; break; }
      fence_after_sync();
      float v[16];
      tmem_ld16(tl + 128u, v);
      tmem_wait_ld();
      fence_before_sync();
      float sigma = v[0] + S.bias4[0];
      if (MODE != kPrune) {
        if (r < ns)
          reinterpret_cast<float4 *>(p.out)[r] =
              make_float4(sigma, v[1] + S.bias4[1], v[2] + S.bias4[2], v[3] + S.bias4[3]);
      } else {
        // reference rule (fairnr/modules/encoder.py:610, 648): exp(-relu s),
        // reduced with min; workload rule: 1 - exp(-relu(s) * step), max.
        // Both are >= 0, so their float bits order like unsigned ints. A warp
        // whose rows all belong to one voxel reduces before its one atomic.
        bool live = r < ns;
        int64_t vv = live ? r / ((int64_t)p.bits * p.bits * p.bits) : -1;
        uint32_t val;
        if (p.rule == 0) val = __float_as_uint(expf(-fmaxf(sigma, 0.0f)));
        else val = __float_as_uint(fmaxf(1.0f - expf(-(fmaxf(sigma, 0.0f) * p.step)), 0.0f));
        int64_t v0 = __shfl_sync(0xffffffffu, vv, 0);
        if (__all_sync(0xffffffffu, vv == v0 && live)) {
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            uint32_t y = __shfl_xor_sync(0xffffffffu, val, o);
            val = (p.rule == 0) ? min(val, y) : max(val, y);
          }
          if (lane == 0) {
            if (p.rule == 0) atomicMin(p.score + v0, val);
            else atomicMax(p.score + v0, val);
          }
        } else if (live) {
          if (p.rule == 0) atomicMin(p.score + vv, val);
          else atomicMax(p.score + vv, val);
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (tid == 0 && S.abort && p.err) atomicOr(p.err, 8);
  if (warp == kMmaWarp) {
    fence_after_sync();
    tmem_dealloc(tmem, kTmemCols);
  }
}

int g_num_sms = 0;

template <int MODE>
int launch_mlp_grid(const MlpParams &p, cudaStream_t stream, int64_t grid_override);

template <int MODE>
int launch_mlp(const MlpParams &p, cudaStream_t stream) {
  return launch_mlp_grid<MODE>(p, stream, 0);
}

// grid_override < 0: one CTA per SM (the row count is only known on the
// device); 0: sized from p.ns.
template <int MODE>
int launch_mlp_grid(const MlpParams &p, cudaStream_t stream, int64_t grid_override) {
  static bool attr_set = false;
  size_t smem = sizeof(MlpSmem) + 1024;
  if (!attr_set) {
    if (cudaFuncSetAttribute(mlp_tc_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return NSVF_ERR_CUDA;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    attr_set = true;
  }
  int64_t n_tiles = (p.ns + TILE - 1) / TILE;
  int64_t grid = grid_override < 0 ? g_num_sms : (n_tiles + 1) / 2;
  if (grid > g_num_sms) grid = g_num_sms;
  if (grid < 1) grid = 1;
  mlp_tc_kernel<MODE><<<(int)grid, kThreads, smem, stream>>>(p);
  return nsvf_launch_status();
}

bool set_weights(MlpParams &p, const void *const weights[5], const float *const biases[5]) {
  if (!weights || !biases) return false;
  for (int l = 0; l < 5; ++l) {
    if (!weights[l] || !biases[l] || (((uintptr_t)weights[l]) & 15)) return false;
    p.w[l] = (const __nv_bfloat16 *)weights[l];
    p.b[l] = biases[l];
  }
  return true;
}

}  // namespace

extern "C" {

int nsvf_mlp_forward_bf16(int64_t n_samples, const float *emb, const void *const weights[5],
                          const float *const biases[5], float *out, int32_t *err, void *stream) {
  if (n_samples < 0) return NSVF_ERR_INVALID;
  if (n_samples == 0) return NSVF_OK;
  MlpParams p = {};
  if (!emb || !out || !set_weights(p, weights, biases)) return NSVF_ERR_INVALID;
  if ((((uintptr_t)emb) | ((uintptr_t)out)) & 15) return NSVF_ERR_INVALID;
  p.emb = emb;
  p.out = out;
  p.ns = n_samples;
  p.err = err;
  return launch_mlp<kEmbIn>(p, (cudaStream_t)stream);
}

int nsvf_field_samples_bf16(int64_t n_samples, const int32_t *voxel, const float *xyz_dist,
                            int64_t n_voxels, int64_t n_keys, float voxel_size,
                            const float *centers, const int32_t *feats, const float *values,
                            const void *const weights[5], const float *const biases[5],
                            float *out, int32_t *err, void *stream) {
  if (n_samples < 0 || n_voxels < 1 || n_keys < 1) return NSVF_ERR_INVALID;
  if (n_samples == 0) return NSVF_OK;
  MlpParams p = {};
  if (!voxel || !xyz_dist || !centers || !feats || !values || !out ||
      !set_weights(p, weights, biases))
    return NSVF_ERR_INVALID;
  if ((((uintptr_t)xyz_dist) | ((uintptr_t)values) | ((uintptr_t)out) | ((uintptr_t)feats)) & 15)
    return NSVF_ERR_INVALID;
  p.vox = voxel;
  p.xyzd = (const float4 *)xyz_dist;
  p.centers = centers;
  p.feats = feats;
  p.values = (const float4 *)values;
  p.n_vox = n_voxels;
  p.n_keys = n_keys;
  p.voxel_size = voxel_size;
  p.out = out;
  p.ns = n_samples;
  p.err = err;
  return launch_mlp<kSamplesIn>(p, (cudaStream_t)stream);
}

int nsvf_field_samples_bf16_dev(int64_t capacity, const int64_t *n_samples_dev,
                                const int32_t *voxel, const float *xyz_dist, int64_t n_voxels,
                                int64_t n_keys, float voxel_size, const float *centers,
                                const int32_t *feats, const float *values,
                                const void *const weights[5], const float *const biases[5],
                                float *out, int32_t *err, void *stream) {
  if (capacity < 0 || !n_samples_dev || n_voxels < 1 || n_keys < 1) return NSVF_ERR_INVALID;
  if (capacity == 0) return NSVF_OK;
  MlpParams p = {};
  if (!voxel || !xyz_dist || !centers || !feats || !values || !out ||
      !set_weights(p, weights, biases))
    return NSVF_ERR_INVALID;
  if ((((uintptr_t)xyz_dist) | ((uintptr_t)values) | ((uintptr_t)out) | ((uintptr_t)feats)) & 15)
    return NSVF_ERR_INVALID;
  p.vox = voxel;
  p.xyzd = (const float4 *)xyz_dist;
  p.centers = centers;
  p.feats = feats;
  p.values = (const float4 *)values;
  p.n_vox = n_voxels;
  p.n_keys = n_keys;
  p.voxel_size = voxel_size;
  p.out = out;
  p.ns = capacity;
  p.ns_dev = n_samples_dev;
  p.err = err;
  return launch_mlp_grid<kSamplesIn>(p, (cudaStream_t)stream, -1);
}

int nsvf_prune_scores_bf16(int64_t n_voxels, int bits, int rule, float step, int64_t n_keys,
                           float voxel_size, const float *centers, const int32_t *feats,
                           const float *values, const void *const weights[5],
                           const float *const biases[5], uint32_t *score, int32_t *err,
                           void *stream) {
  if (n_voxels < 0 || bits < 2 || bits > 64 || (rule != 0 && rule != 1) || n_keys < 1)
    return NSVF_ERR_INVALID;
  if (n_voxels == 0) return NSVF_OK;
  MlpParams p = {};
  if (!centers || !feats || !values || !score || !set_weights(p, weights, biases))
    return NSVF_ERR_INVALID;
  if ((((uintptr_t)values) | ((uintptr_t)feats)) & 15) return NSVF_ERR_INVALID;
  p.centers = centers;
  p.feats = feats;
  p.values = (const float4 *)values;
  p.n_vox = n_voxels;
  p.n_keys = n_keys;
  p.voxel_size = voxel_size;
  p.bits = bits;
  p.rule = rule;
  p.step = step;
  p.score = score;
  p.ns = n_voxels * (int64_t)bits * bits * bits;
  p.err = err;
  return launch_mlp<kPrune>(p, (cudaStream_t)stream);
}

}  // extern "C"
