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
// BF16 CTA = 19 warps, three tile slots. A slot's chain of layers is latency
// bound (each layer waits for the previous layer's epilogue), so the tensor
// pipe is kept busy by running several slots' chains at once. Tensor memory
// (512 columns) holds the three accumulators (128 columns each) and the
// activations of two slots (64 columns each); the third slot's activations
// live in shared memory, and each slot's head output reuses the first 16
// columns of its accumulator. Warps 0-7 are the epilogue: all eight work on
// one slot's layer at a time and take the slots in turn, so the other slots'
// MMAs run while one slot is converted. Warp 8 allocates TMEM; lane 0 of
// warps 8, 17 and 18 issues the tcgen05.mma instructions of slots 0, 1 and
// 2, so the slots' chains never wait on each other's issue. Warps 9-16 are
// two loader warpgroups that build the input tiles (embedding gathers and
// trilinear interpolation) into a ring of shared-memory buffers. Per layer:
//   MMA thread: a bias step (a ones block x a (hi, mid, lo) bf16 split of
//   the bias, K = 16) that starts D at the bias, then the layer's K / 16
//   MMAs with A = the previous activations -> tcgen05.commit arrives on
//   mma_done[g] -> each epilogue warp reads 64 columns of D (tcgen05.ld),
//   applies ReLU, rounds to bf16 pairs and stores them as the next layer's A
//   (tcgen05.st, or st.shared for slot 2) -> one arrival per warp on
//   act_ready[g].
// The first layer reads its A (the input tile) from shared memory. The FP8
// variant has the same structure with two slots (18 warps, the head output
// in columns of its own); its three hidden layers are E4M3
// (kind::f8f6f4, K = 32 per MMA) with A = E4M3 activations in tensor memory
// (four per column), its bias step holds bias / dq (the layer's
// dequantisation), and its epilogue scales the accumulator by dq * qs
// before rounding to E4M3 (or by dq before bf16, for the head's input).
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
constexpr uint32_t kTmemCols = 512;

// Warp roles and tile slots. Epilogue warps 0-7, loader warps 9-16, one MMA
// warp per slot (8, 17 and, for BF16, 18); each MMA warp's lane 0 issues one
// slot's MMAs.
//   BF16: three slots. Accumulator D of slot g at TMEM column 128 g; the
//   bf16 activations (HID per row, two per column: 64 columns) of slots 0
//   and 1 at 384 + 64 g, those of slot 2 in shared memory (act2). The
//   head's 16 output columns are the first 16 of D, so the slot's next tile
//   starts its first layer only after the epilogue has read the head
//   (head_free).
//   FP8: two slots of 256 columns: D at +0, head output at +128, E4M3
//   activations (four per column: 32 columns) at +160, the head's bf16
//   input at +192.
// The bias step of every layer reads its A operand (rows of (1, 1, 1, 0,
// ...)) from shared memory (ones_a).
template <bool F8>
struct Cfg {
  static constexpr int kSlots = F8 ? 2 : 3;
  static constexpr int kEpiWarps = 8;
  static constexpr int kLoaderWarp0 = kEpiWarps + 1;
  static constexpr int kMmaWarp = kEpiWarps;
  static constexpr int kMmaWarp2 = kLoaderWarp0 + 8;
  static constexpr int kMmaWarp3 = kMmaWarp2 + 1;
  static constexpr int kThreads = (16 + kSlots) * 32;
  // the head's output shares columns with D (the next tile's first layer
  // waits for the head to be read)
  static constexpr bool kHeadInD = !F8;
  __device__ static constexpr uint32_t d_col(int g) { return (F8 ? 256u : 128u) * (uint32_t)g; }
  __device__ static constexpr uint32_t head_col(int g) {
    return F8 ? 256u * (uint32_t)g + 128u : 128u * (uint32_t)g;
  }
  // bf16 activations in tensor memory: the A operand of the BF16 hidden
  // layers and of the head (BF16 slots 0 and 1; both FP8 slots)
  __device__ static constexpr uint32_t act_col(int g) {
    return F8 ? 256u * (uint32_t)g + 192u : 384u + 64u * (uint32_t)g;
  }
  // BF16 slot 2 keeps its activations in shared memory
  __device__ static constexpr bool act_in_smem(int g) { return !F8 && g == 2; }
  // FP8: E4M3 activations of slot g, the A operand of the E4M3 hidden layers
  __device__ static constexpr uint32_t act8_col(int g) { return 256u * (uint32_t)g + 160u; }
  static constexpr int kHidBytes = F8 ? HID * HID : HID * HID * 2;  // one hidden weight matrix
};

template <bool F8>
struct __align__(128) MlpSmem {
  __nv_bfloat16 w0[HID * E];
  uint8_t wh[3][Cfg<F8>::kHidBytes];       // bf16 or E4M3 hidden weights
  __nv_bfloat16 w4[NOUT * HID];
  __nv_bfloat16 ain[NB][TILE * E];
  // the bias step of each layer (an extra bf16 K = 16 MMA): B rows n =
  // (hi, mid, lo, 0, ...) with hi + mid + lo = bias[l][n] / dq[l] (three
  // bf16 terms; dq = 1 except after an FP8 layer), and the A tile that every
  // layer's bias step reads, rows (1, 1, 1, 0, ...).
  __nv_bfloat16 bias_b[4][HID * 16];
  __nv_bfloat16 ones_a[TILE * 16];
  // BF16 slot 2's activations (K-major, TILE x HID): written by the epilogue,
  // read by the slot's next layer
  __nv_bfloat16 act2[F8 ? 8 : TILE * HID];
  // per loader warp: its 32 rows' corner keys (kSkipKey = skip) and
  // trilinear weights, written by the row's lane and read by the 8 lanes
  // that gather the row
  int meta_key[8][32 * 8];
  // and its voxel (-1: no corners); the row's keys are a function of it
  int meta_vox[8][32];
  float meta_w[8][32 * 8];
  float bias[4][HID];
  float bias4[NOUT];
  uint64_t mma_done[Cfg<F8>::kSlots][5];  // per slot and layer: one phase per tile
  uint64_t act_ready[Cfg<F8>::kSlots];    // epilogue -> MMA: hidden activations written
  uint64_t head_free[Cfg<F8>::kSlots];    // epilogue -> MMA: head output read (kHeadInD)
  uint64_t in_full[NB];                   // loaders -> MMA: input tile written
  uint64_t in_empty[NB];                  // MMA -> loaders: first layer done reading
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
  // kPrune screen of the exact pruning pass (keep != NULL): with M = sum_j
  // |W4[0][j]| h_j (an extra head column), a point with sigma - c M above
  // the threshold T (>= for rule 1, > for rule 0) keeps its voxel
  // (keep[v] = 1); a point with sigma + c M >= T is undecided and its row is
  // appended to plist for the double-float pass (exact.cu)
  uint8_t *keep;
  float prune_T, prune_c;
  int64_t *plist;
  unsigned long long *n_plist;
  int64_t plist_cap;
  const __nv_bfloat16 *w[5];         // row-major [N, K]: 128x32, 3x 128x128, 4x128
  const float *b[5];                 // [128] x4, [4]
  // FP8 variant: the hidden layers 1-3 as E4M3 bytes (row-major [128, 128],
  // W * w_scale). Layer l's accumulator starts at bias / dq[l] (dq[l] =
  // 1 / (a_scale[l] * w_scale[l]), 1 for layer 0) and is multiplied by dq[l]
  // in the epilogue; the output of layer l (input of FP8 layer l + 1) is
  // also multiplied by qs[l] = a_scale[l + 1] before rounding to E4M3.
  // Layer 0 and the head stay BF16.
  const uint8_t *w8[3];
  float dq[4];
  float qs[4];
  float dqs[3];                      // dq[l] * qs[l]: FP8 outputs are relu(acc * dqs)
  float *out;                        // [ns, 4]: sigma, r, g, b
  int64_t ns;                        // rows (the capacity when ns_dev is set)
  const int64_t *ns_dev;             // optional: row count read on the device
  int32_t *err;
  // kSamplesIn, optional: samples far outside their voxel are appended to
  // outl (count *n_outl, capacity outl_cap) for the compensated pass
  int64_t *outl;
  unsigned long long *n_outl;
  int64_t outl_cap;
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

// Copy a row-major [rows, K] E4M3 matrix into the 8-bit K-major layout.
__device__ void stage_weights8(uint8_t *dst, const uint8_t *src, int rows, int K) {
  int chunks = rows * (K / 16);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    int r = c / (K / 16), kc = c % (K / 16);
    uint4 v = *reinterpret_cast<const uint4 *>(src + (size_t)r * K + kc * 16);
    *reinterpret_cast<uint4 *>(dst + kmajor_off8(r, kc * 16, K)) = v;
  }
}


// The K / 16 MMAs of one BF16 layer from precomputed descriptors. A K = 16
// step moves a no-swizzle K-major operand by 256 bytes, i.e. 16 in the
// descriptor's address field (addresses stay below 256 KB, so the field does
// not overflow). A from shared memory (ad) or, for issue_ts, from tensor
// memory at column a_tmem (two bf16 per column: 8 columns per step).
// ACC0: the first step accumulates onto D too (D holds the layer's bias).
template <int KS, bool ACC0>
__device__ __forceinline__ void issue_ss(uint32_t d_tmem, uint64_t ad, uint64_t bd, uint32_t idesc) {
#pragma unroll
  for (int k = 0; k < KS; ++k)
    mma_bf16(d_tmem, ad + 16u * k, bd + 16u * k, idesc, (ACC0 || k > 0) ? 1u : 0u);
}

template <int KS, bool ACC0>
__device__ __forceinline__ void issue_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bd,
                                         uint32_t idesc) {
#pragma unroll
  for (int k = 0; k < KS; ++k)
    mma_bf16_ts(d_tmem, a_tmem + 8u * k, bd + 16u * k, idesc, (ACC0 || k > 0) ? 1u : 0u);
}

// bf16 1.0 in the low half, and in both halves
constexpr uint32_t kOne = 0x00003F80u, kOnes2 = 0x3F803F80u;

// The bias step's operands (BF16), written once per CTA: row n of layer l's
// B block is (hi, mid, lo, 0, ...) with hi = bf16(b), mid = bf16(b - hi),
// lo = bf16(b - hi - mid) -- their sum is b to within the FP32 rounding of the
// accumulation -- and every row of the A block that all layers share is
// (1, 1, 1, 0, ...). Both are no-swizzle K-major tiles with K = 16.
__device__ __forceinline__ void stage_bias_step(__nv_bfloat16 (*bias_b)[HID * 16],
                                                __nv_bfloat16 *ones_a,
                                                const float *const *b, const float *dq, int tid,
                                                int nthreads) {
  for (int i = tid; i < 4 * HID; i += nthreads) {
    const int l = i / HID, n = i % HID;
    const float v = dq ? b[l][n] / dq[l] : b[l][n];
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(hi);
    const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
    const __nv_bfloat16 lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
    uint8_t *base = reinterpret_cast<uint8_t *>(bias_b[l]);
    const uint32_t w01 = (uint32_t)__bfloat16_as_ushort(hi) | ((uint32_t)__bfloat16_as_ushort(mid) << 16);
    const uint32_t w23 = (uint32_t)__bfloat16_as_ushort(lo);
    *reinterpret_cast<uint4 *>(base + kmajor_off(n, 0, 16)) = make_uint4(w01, w23, 0u, 0u);
    *reinterpret_cast<uint4 *>(base + kmajor_off(n, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
  }
  for (int m = tid; m < TILE; m += nthreads) {
    uint8_t *base = reinterpret_cast<uint8_t *>(ones_a);
    *reinterpret_cast<uint4 *>(base + kmajor_off(m, 0, 16)) = make_uint4(kOnes2, kOne, 0u, 0u);
    *reinterpret_cast<uint4 *>(base + kmajor_off(m, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
  }
}

// bf16x2 of (relu(lo), relu(hi)) with round-to-nearest-even, one instruction
__device__ __forceinline__ uint32_t pack_relu_bf16x2(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %2, %1;\n" : "=r"(d) : "f"(lo), "f"(hi));
  return d;
}

constexpr int kSkipKey = -1;

// Input stage, pass 1 (lane = row r): the row's voxel, its 8 corner keys and
// trilinear weights (interpolated sample or pruning point). Rows >= ns and
// invalid voxels / corner ids get kSkipKey (they contribute nothing; invalid
// ids set `bad`). The weights are the interpolation kernel's, same
// operations in the same order.
// A sample row's voxel id and position, loaded one tile ahead of its use.
struct SampleRow {
  int32_t vox;
  float4 xyz;
};

template <int MODE>
__device__ __forceinline__ SampleRow load_sample(const MlpParams &p, int64_t r, int64_t ns) {
  SampleRow s;
  s.vox = -1;
  s.xyz = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (MODE == kSamplesIn && r < ns) {
    s.vox = p.vox[r];
    s.xyz = p.xyzd[r];
  }
  return s;
}

// A row's voxel (-1: none): the sample's, or the pruning point's.
template <int MODE>
__device__ __forceinline__ int64_t row_voxel(const MlpParams &p, int64_t r, int64_t ns,
                                             const SampleRow &smp) {
  if (r >= ns) return -1;
  if (MODE == kSamplesIn) return smp.vox;
  return r / ((int64_t)p.bits * p.bits * p.bits);
}

// The voxel data a row needs, its centre and 8 corner ids. The loaders fetch
// it one tile ahead, as soon as the row's voxel id has arrived.
struct VoxRow {
  float cx, cy, cz;
  int4 f0, f1;
};

__device__ __forceinline__ VoxRow load_vox(const MlpParams &p, int64_t v) {
  VoxRow d;
  d.cx = d.cy = d.cz = 0.0f;
  d.f0 = d.f1 = make_int4(kSkipKey, kSkipKey, kSkipKey, kSkipKey);
  if (v >= 0 && v < p.n_vox) {
    d.cx = p.centers[v * 3];
    d.cy = p.centers[v * 3 + 1];
    d.cz = p.centers[v * 3 + 2];
    d.f0 = reinterpret_cast<const int4 *>(p.feats)[v * 2];
    d.f1 = reinterpret_cast<const int4 *>(p.feats)[v * 2 + 1];
  }
  return d;
}

template <int MODE>
__device__ __forceinline__ void row_meta(const MlpParams &p, int64_t r, int64_t ns,
                                         const SampleRow &smp, const VoxRow &vd,
                                         int *__restrict__ key, float *__restrict__ w,
                                         int *__restrict__ vid, bool &bad) {
  int k8[8];
  int vv = -1;
  float w8[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) { k8[k] = kSkipKey; w8[k] = 0.0f; }
  if (r < ns) {
    int64_t v;
    float x, y, z;
    if (MODE == kSamplesIn) {
      v = smp.vox;
      x = smp.xyz.x; y = smp.xyz.y; z = smp.xyz.z;
    } else {
      // point i of voxel v: offset_points order (x slowest), offset
      // ((2 i_d + 1) - bits) / (bits - 1) times half a voxel
      int64_t P = (int64_t)p.bits * p.bits * p.bits;
      v = r / P;
      int64_t i = r % P;
      int ix = (int)(i / (p.bits * p.bits)), iy = (int)((i / p.bits) % p.bits), iz = (int)(i % p.bits);
      // offset_points' FP32 operations: fl(fl(o / (bits - 1)) * hv), then
      // added to the centre (separate roundings, no contraction)
      float hv = p.voxel_size / 2.0f, den = (float)(p.bits - 1);
      x = __fadd_rn(vd.cx, __fmul_rn(__fdiv_rn((float)(2 * ix + 1 - p.bits), den), hv));
      y = __fadd_rn(vd.cy, __fmul_rn(__fdiv_rn((float)(2 * iy + 1 - p.bits), den), hv));
      z = __fadd_rn(vd.cz, __fmul_rn(__fdiv_rn((float)(2 * iz + 1 - p.bits), den), hv));
    }
    if (v < 0 || v >= p.n_vox) {
      bad = true;
    } else {
      vv = (int)v;
      float q[3] = {(x - vd.cx) / p.voxel_size + 0.5f, (y - vd.cy) / p.voxel_size + 0.5f,
                    (z - vd.cz) / p.voxel_size + 0.5f};
      if (MODE == kSamplesIn && p.n_outl && nsvf_far_outside(q[0], q[1], q[2]))
        nsvf_push_outlier(p.outl, p.n_outl, p.outl_cap, r, p.err);
      const int keys[8] = {vd.f0.x, vd.f0.y, vd.f0.z, vd.f0.w, vd.f1.x, vd.f1.y, vd.f1.z, vd.f1.w};
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (keys[k] < 0 || keys[k] >= p.n_keys) {
          bad = true;
        } else {
          k8[k] = keys[k];
          w8[k] = corner_weight(q, k);
        }
      }
    }
  }
  reinterpret_cast<int4 *>(key)[0] = make_int4(k8[0], k8[1], k8[2], k8[3]);
  reinterpret_cast<int4 *>(key)[1] = make_int4(k8[4], k8[5], k8[6], k8[7]);
  reinterpret_cast<float4 *>(w)[0] = make_float4(w8[0], w8[1], w8[2], w8[3]);
  reinterpret_cast<float4 *>(w)[1] = make_float4(w8[4], w8[5], w8[6], w8[7]);
  *vid = vv;
}

// Input stage, pass 2 (8 lanes per row, lane cb owns channels 4cb..4cb+3):
// sum_k w_k values[key_k][4cb..4cb+3] over the corners in order 0..7, one
// fused multiply-add per corner and channel -- per channel the interpolation
// kernel's exact sequence. One load instruction reads four rows' 128-byte
// corner rows whole. corner_loads issues the 8 loads of a row; a corner
// without a valid key reads zeros, and its weight is zero too, so it leaves
// the sum unchanged. corner_blend applies the weights, two channels per
// instruction (fma.rn.f32x2 rounds each lane like fmaf).
__device__ __forceinline__ void corner_loads(const MlpParams &p, int4 ka, int4 kb, int cb,
                                             float4 (&val)[8]) {
  const int keys[8] = {ka.x, ka.y, ka.z, ka.w, kb.x, kb.y, kb.z, kb.w};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    val[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (keys[k] != kSkipKey) val[k] = __ldg(p.values + (int64_t)keys[k] * 8 + cb);
  }
}

__device__ __forceinline__ uint64_t pack_f32x2(float lo, float hi) {
  uint64_t d;
  asm("mov.b64 %0, {%1, %2};\n" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}

// d = b * c + a on two FP32 lanes, each rounded once (round to nearest even)
__device__ __forceinline__ uint64_t fma_f32x2(uint64_t b, uint64_t c, uint64_t a) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;\n" : "=l"(d) : "l"(b), "l"(c), "l"(a));
  return d;
}

__device__ __forceinline__ float4 corner_blend(const float *__restrict__ w, const float4 (&val)[8]) {
  const float4 wa = reinterpret_cast<const float4 *>(w)[0];
  const float4 wb = reinterpret_cast<const float4 *>(w)[1];
  const float ws[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
  uint64_t exy = 0, ezw = 0;  // (+0, +0)
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const uint64_t wk = pack_f32x2(ws[k], ws[k]);
    exy = fma_f32x2(wk, pack_f32x2(val[k].x, val[k].y), exy);
    ezw = fma_f32x2(wk, pack_f32x2(val[k].z, val[k].w), ezw);
  }
  float4 e;
  asm("mov.b64 {%0, %1}, %2;\n" : "=f"(e.x), "=f"(e.y) : "l"(exy));
  asm("mov.b64 {%0, %1}, %2;\n" : "=f"(e.z), "=f"(e.w) : "l"(ezw));
  return e;
}

__device__ __forceinline__ void store_in4(uint8_t *ain, int row, int cb, float4 e) {
  *reinterpret_cast<uint2 *>(ain + kmajor_off(row, cb * 4, E) + (cb & 1) * 8) =
      make_uint2(pack_bf16x2(e.x, e.y), pack_bf16x2(e.z, e.w));
}

// FP8 epilogue chunk feeding an E4M3 layer: 32 columns [c, c + 32) of one
// row times dqs (the layer's dequantisation times the next layer's activation
// scale; the bias is already in the accumulator as bias / dq), ReLU and
// saturating E4M3 rounding in one cvt, four per 32-bit TMEM column (element
// k in byte k % 4) at ta8 + c / 4.
__device__ __forceinline__ void epi_chunk8(const float (&v)[32], float dqs, uint32_t ta8, int c) {
  uint32_t pk[8];
#pragma unroll
  for (int j = 0; j < 8; ++j)
    pk[j] = pack_relu_e4m3x2(v[4 * j] * dqs, v[4 * j + 1] * dqs) |
            (pack_relu_e4m3x2(v[4 * j + 2] * dqs, v[4 * j + 3] * dqs) << 16);
  tmem_st8(ta8 + (uint32_t)(c >> 2), pk);
}

// FP8 epilogue chunk after the last E4M3 layer, feeding the BF16 head: times
// dq, ReLU, bf16 pairs at ta + c / 2.
__device__ __forceinline__ void epi_chunk_dq(const float (&v)[32], float dq, uint32_t ta, int c) {
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    uint32_t pk[8];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      pk[j] = pack_relu_bf16x2(v[16 * q + 2 * j] * dq, v[16 * q + 2 * j + 1] * dq);
    tmem_st8(ta + (uint32_t)((c >> 1) + 8 * q), pk);
  }
}

// Hidden-layer epilogue of 32 columns [c, c + 32) of one row (the bias is
// already in the accumulator): ReLU, round to bf16, and store the 16 packed
// pairs into the row's activations in tensor memory (`ta`: this warp's
// lanes, the slot's activation column).
__device__ __forceinline__ void epi_chunk(const float (&v)[32], uint32_t ta, int c) {
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    uint32_t pk[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) pk[j] = pack_relu_bf16x2(v[16 * q + 2 * j], v[16 * q + 2 * j + 1]);
    tmem_st8(ta + (uint32_t)((c >> 1) + 8 * q), pk);
  }
}

// The same for activations kept in shared memory (K-major, K = HID): row
// `row`'s bf16 [c, c + 32) as four 16-byte chunks. The eight lanes of a
// quarter warp hold rows 8 j .. 8 j + 7, one core matrix: no bank conflicts.
__device__ __forceinline__ void epi_chunk_smem(const float (&v)[32], uint8_t *act, int row, int c) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint4 w = make_uint4(pack_relu_bf16x2(v[8 * q], v[8 * q + 1]),
                               pack_relu_bf16x2(v[8 * q + 2], v[8 * q + 3]),
                               pack_relu_bf16x2(v[8 * q + 4], v[8 * q + 5]),
                               pack_relu_bf16x2(v[8 * q + 6], v[8 * q + 7]));
    *reinterpret_cast<uint4 *>(act + kmajor_off(row, c + 8 * q, HID)) = w;
  }
}

// Output stage of one row (the whole warp calls it): the head's 16 TMEM
// columns at taddr, plus bias, to p.out as (sigma, r, g, b); or, for pruning,
// the row's score reduced into its voxel's.
template <int MODE>
__device__ __forceinline__ void head_store(const MlpParams &p, const float *bias4, uint32_t taddr,
                                           int64_t r, int64_t ns, int lane) {
  float v[16];
  tmem_ld16(taddr, v);
  tmem_wait_ld();
  fence_before_sync();
  float sigma = v[0] + bias4[0];
  if (MODE != kPrune) {
    if (r < ns)
      reinterpret_cast<float4 *>(p.out)[r] =
          make_float4(sigma, v[1] + bias4[1], v[2] + bias4[2], v[3] + bias4[3]);
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
    if (p.keep) {
      // exact-pass screen (whole warp): certain keeps, and undecided rows
      // appended to plist with one atomic per warp
      const float M = v[4];
      const float lo = sigma - p.prune_c * M, hi = sigma + p.prune_c * M;
      const bool certain = live && (p.rule == 1 ? lo >= p.prune_T : lo > p.prune_T);
      const bool maybe = live && !certain && hi >= p.prune_T;
      if (certain) p.keep[vv] = 1;
      const unsigned m = __ballot_sync(0xffffffffu, maybe);
      if (m) {
        const int leader = __ffs(m) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(p.n_plist, (unsigned long long)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (maybe) {
          const unsigned long long k = base + __popc(m & ((1u << lane) - 1u));
          if ((int64_t)k < p.plist_cap) p.plist[k] = r;
          else if (p.err) atomicOr(p.err, 16);
        }
      }
    }
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

// Persistent CTA (one per SM), roles as in Cfg:
//   epilogue warps  ReLU + rounding of each hidden layer into the next
//                   layer's A operand, and the output stage; all 8 warps on
//                   one slot's layer at a time, taking the slots in turn;
//   MMA warps       warp 8 allocates TMEM; lane 0 of warps 8, 17 (and 18)
//                   issues the tcgen05.mma of slots 0, 1 (and 2);
//   loader warps    two warpgroups that build the input tiles (the embedding
//                   gathers and interpolation) into a ring of NB buffers
//                   ahead of the MMAs.
// The CTA's tiles are b, b + G, b + 2G, ...: local tile i uses slot
// i % kSlots, ring buffer i % NB and loader group i % 2. Each mbarrier
// completes exactly one phase per use and every waiter consumes it before
// the next phase can complete, so parity waits are unambiguous.
template <int MODE, bool F8>
__global__ void __launch_bounds__(Cfg<F8>::kThreads, 1) mlp_tc_kernel(const MlpParams p) {
  using C = Cfg<F8>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  MlpSmem<F8> &S = *reinterpret_cast<MlpSmem<F8> *>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  stage_weights(S.w0, p.w[0], HID, HID, E);
  for (int l = 0; l < 3; ++l) {
    if (F8) stage_weights8(S.wh[l], p.w8[l], HID, HID);
    else stage_weights(reinterpret_cast<__nv_bfloat16 *>(S.wh[l]), p.w[l + 1], HID, HID, HID);
  }
  stage_weights(S.w4, p.w[4], NOUT, 4, HID);
  if (MODE == kPrune && p.keep) {
    // head row 4 = |W4[0]|: column 4 of the head output is M = sum_j
    // |W4[0][j]| h_j, the scale of sigma's BF16 rounding error
    // (each chunk written by the thread stage_weights gave it, after its
    // zero fill, so no barrier is needed in between)
    for (int c = threadIdx.x; c < NOUT * (HID / 8); c += blockDim.x) {
      if (c / (HID / 8) != 4) continue;
      const int kc = c % (HID / 8);
      uint4 v = *reinterpret_cast<const uint4 *>(p.w[4] + kc * 8);
      v.x &= 0x7fff7fffu; v.y &= 0x7fff7fffu; v.z &= 0x7fff7fffu; v.w &= 0x7fff7fffu;
      *reinterpret_cast<uint4 *>(reinterpret_cast<uint8_t *>(S.w4) + kmajor_off(4, kc * 8, HID)) = v;
    }
  }
  stage_bias_step(S.bias_b, S.ones_a, p.b, F8 ? p.dq : nullptr, tid, blockDim.x);
  for (int i = tid; i < 4 * HID; i += blockDim.x) S.bias[i / HID][i % HID] = p.b[i / HID][i % HID];
  if (tid < NOUT) S.bias4[tid] = tid < 4 ? p.b[4][tid] : 0.0f;
  if (tid == 0) {
    for (int g = 0; g < C::kSlots; ++g) {
      for (int l = 0; l < 5; ++l) mbar_init(&S.mma_done[g][l], 1);
      // one arrival per epilogue warp (lane 0, after the warp's fences and
      // a __syncwarp): all 8 warps work on each slot's layer
      mbar_init(&S.act_ready[g], C::kEpiWarps);
      // one arrival per warp of the half that reads slot g's head
      mbar_init(&S.head_free[g], 4);
    }
    for (int q = 0; q < NB; ++q) {
      mbar_init(&S.in_full[q], 4);    // one arrival per loader warp
      mbar_init(&S.in_empty[q], 1);
    }
    S.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == C::kMmaWarp) tmem_alloc(&S.tmem_base, kTmemCols);
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

  const bool mma_role = warp == C::kMmaWarp || warp == C::kMmaWarp2 ||
                        (C::kSlots > 2 && warp == C::kMmaWarp3);
  const bool loader_role = warp >= C::kLoaderWarp0 && warp < C::kLoaderWarp0 + 8;
  if (mma_role) {
    // One issuing thread per slot, so a slot whose activations are ready
    // never waits behind another slot's issue: lane 0 of kMmaWarp (slot 0),
    // kMmaWarp2 (slot 1) and kMmaWarp3 (slot 2).
    const int g = warp == C::kMmaWarp ? 0 : warp == C::kMmaWarp2 ? 1 : 2;
    if (lane == 0) {
      uint32_t ph_act = 0, ph_head = 0;
      bool ok = true;
      // Descriptors, computed once: the first layer's weights and input
      // ring buffer 0 (buffer q is 8 KB further: + 512 in the address
      // field), the first hidden layer's weights (layer l + 1: one matrix
      // further, + kHidBytes / 16; a K step of 16 bf16 or 32 E4M3 elements
      // is 256 bytes, + 16) and the head's weights.
      const uint64_t d_in0 = sdesc(smem_u32(S.ain[0]), 128u, (E / 8) * 128u);
      const uint64_t d_w0 = sdesc(smem_u32(S.w0), 128u, (E / 8) * 128u);
      const uint64_t d_wh = sdesc(smem_u32(S.wh[0]), 128u, (F8 ? HID / 16 : HID / 8) * 128u);
      constexpr uint32_t kHidStep = C::kHidBytes / 16;
      // the bias step of every layer: the ones block (A, shared memory) and
      // layer l's bias block (B; + 256 per layer)
      const uint64_t d_ones = sdesc(smem_u32(S.ones_a), 128u, 256u);
      const uint64_t d_bias = sdesc(smem_u32(S.bias_b[0]), 128u, 256u);
      const uint64_t d_w4 = sdesc(smem_u32(S.w4), 128u, (HID / 8) * 128u);
      // slot 2's shared-memory activations (BF16 only)
      const uint64_t d_act2 = sdesc(smem_u32(S.act2), 128u, (HID / 8) * 128u);
      const bool smem_act = C::act_in_smem(g);
      const uint32_t d = tmem + C::d_col(g);
      static_assert(sizeof(S.ain[0]) == 8192 && C::kHidBytes % 16 == 0, "descriptor steps");
#pragma unroll 1
      for (int64_t ii = g; ok; ii += C::kSlots) {
        if (tile_of(ii) >= n_tiles) break;
#pragma unroll 1
        for (int layer = 0; layer < 5; ++layer) {
          if (layer == 0) {
            int q = (int)(ii % NB);
            if (!mbar_wait(&S.in_full[q], (uint32_t)((ii / NB) & 1), abort)) { ok = false; break; }
            // the slot's previous head must have been read before the
            // first layer overwrites D
            if (C::kHeadInD && ii >= C::kSlots) {
              if (!mbar_wait(&S.head_free[g], ph_head, abort)) { ok = false; break; }
              ph_head ^= 1u;
            }
            fence_after_sync();
            // bias step (overwrites D), then the layer accumulating onto it
            mma_bf16(d, d_ones, d_bias, idesc_bf16_f32(TILE, HID), 0u);
            issue_ss<E / 16, true>(d, d_in0 + 512u * (uint32_t)q, d_w0, idesc_bf16_f32(TILE, HID));
            mma_commit(&S.mma_done[g][0]);
            mma_commit(&S.in_empty[q]);
          } else {
            if (!mbar_wait(&S.act_ready[g], ph_act, abort)) { ok = false; break; }
            ph_act ^= 1u;
            fence_after_sync();
            if (layer < 4) {
              // bias step (bias / dq, bf16), then the layer accumulating
              // onto it: BF16 K steps of 16 with A = the bf16 activations,
              // or E4M3 K steps of 32 with A = the E4M3 activations
              mma_bf16(d, d_ones, d_bias + 256u * (uint32_t)layer, idesc_bf16_f32(TILE, HID), 0u);
              const uint64_t bd = d_wh + kHidStep * (uint32_t)(layer - 1);
              if constexpr (F8) {
#pragma unroll
                for (int k = 0; k < HID / 32; ++k)
                  mma_e4m3_ts(d, tmem + C::act8_col(g) + 8u * k, bd + 16u * k,
                              idesc_e4m3_f32(TILE, HID), 1u);
              } else if (smem_act) {
                issue_ss<HID / 16, true>(d, d_act2, bd, idesc_bf16_f32(TILE, HID));
              } else {
                issue_ts<HID / 16, true>(d, tmem + C::act_col(g), bd, idesc_bf16_f32(TILE, HID));
              }
            } else if (smem_act) {
              issue_ss<HID / 16, false>(tmem + C::head_col(g), d_act2, d_w4,
                                        idesc_bf16_f32(TILE, NOUT));
            } else {
              issue_ts<HID / 16, false>(tmem + C::head_col(g), tmem + C::act_col(g), d_w4,
                                        idesc_bf16_f32(TILE, NOUT));
            }
            mma_commit(&S.mma_done[g][layer]);
          }
        }
      }
    }
    __syncwarp();
  } else if (loader_role) {
    // loaders: every wait result is taken warp-uniformly. Warp wq of group
    // L builds rows [32 wq, 32 wq + 32) of the group's tiles: pass 1 with
    // lane = row, pass 2 with 8 lanes per row (4 rows at a time).
    const int L = (warp - C::kLoaderWarp0) >> 2, wq = (warp - C::kLoaderWarp0) & 3;
    const int rsub = lane >> 3, cb = lane & 7;
    int *mkey = S.meta_key[warp - C::kLoaderWarp0];
    float *mw = S.meta_w[warp - C::kLoaderWarp0];
    int *mvox = S.meta_vox[warp - C::kLoaderWarp0];
    // this lane's sample row of the group's next tile, loaded a tile ahead
    SampleRow next = load_sample<MODE>(p, tile_of(L) * TILE + wq * 32 + lane, ns);
    // and its voxel's centre and corner ids, fetched once the voxel id is in
    VoxRow next_v = load_vox(p, row_voxel<MODE>(p, tile_of(L) * TILE + wq * 32 + lane, ns, next));
    for (int64_t i = L;; i += 2) {
      int64_t tile = tile_of(i);
      if (tile >= n_tiles) break;
      int q = (int)(i % NB);
      // the first round finds every buffer free (parity of the phase before
      // the barrier's first)
      uint32_t par = (uint32_t)(((i / NB) & 1) ^ 1);
      if (!__all_sync(0xffffffffu, mbar_wait(&S.in_empty[q], par, abort))) break;
      const int64_t r0 = tile * TILE + wq * 32;
      bool bad = false;
      if (MODE != kEmbIn) {
        const SampleRow cur = next;
        const VoxRow cur_v = next_v;
        next = load_sample<MODE>(p, tile_of(i + 2) * TILE + wq * 32 + lane, ns);
        row_meta<MODE>(p, r0 + lane, ns, cur, cur_v, mkey + lane * 8, mw + lane * 8, mvox + lane,
                       bad);
        __syncwarp();
      }
      uint8_t *ain = reinterpret_cast<uint8_t *>(S.ain[q]);
      if (MODE == kEmbIn) {
#pragma unroll 2
        for (int it = 0; it < 8; ++it) {
          const int row = it * 4 + rsub;
          float4 e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          if (r0 + row < ns) e = __ldg(reinterpret_cast<const float4 *>(p.emb + (r0 + row) * E) + cb);
          store_in4(ain, wq * 32 + row, cb, e);
        }
      } else {
        // Group rsub (8 lanes) walks the consecutive rows 8 rsub + ((2 rsub
        // + j) & 7), j = 0..7; the rotation makes the four groups store rows
        // with distinct row % 8 at each step. Consecutive samples of a ray
        // mostly lie in one voxel, so a row in the same voxel as the previous
        // row (hence with the same corner keys) blends the corner values
        // already in registers and loads nothing.
        const int4 *mk = reinterpret_cast<const int4 *>(mkey);
        float4 vc[8];
        int vc_id = 0;
#pragma unroll 2
        for (int j = 0; j < 8; ++j) {
          const int r = rsub * 8 + ((2 * rsub + j) & 7);
          const int id = mvox[r];
          if (j == 0 || id != vc_id) corner_loads(p, mk[r * 2], mk[r * 2 + 1], cb, vc);
          vc_id = id;
          store_in4(ain, wq * 32 + r, cb, corner_blend(mw + r * 8, vc));
        }
      }
      if (bad && p.err) atomicOr(p.err, 4);
      fence_async_smem();
      __syncwarp();                     // also orders pass 2's reads of the row table before the next pass 1
      if (lane == 0) mbar_arrive(&S.in_full[q]);
      // the group's next tile: its voxel ids (loaded before pass 1) are in by
      // now, so fetch their centres and corner ids ahead of its pass 1
      if (MODE != kEmbIn)
        next_v = load_vox(p, row_voxel<MODE>(p, tile_of(i + 2) * TILE + wq * 32 + lane, ns, next));
    }
  } else {
    // Epilogue warps. Every wait result is taken warp-uniformly
    // (__all_sync), so the .sync.aligned tcgen05.ld and the warp shuffles
    // below always run with all 32 lanes, also when a timeout makes the CTA
    // unwind.
    {
      // The 8 warps work on one slot's layer at a time (warp w: TMEM lane
      // quarter w & 3, columns [64 (w >> 2), + 64)) and take the slots in
      // turn layer by layer, so that the other slots' MMAs run while the
      // warps convert one slot's activations. The MMA lanes issue in the
      // same order (per group of kSlots tiles: layer by layer, slot by slot).
      const int q4 = warp & 3, h = warp >> 2;
      const int row = q4 * 32 + lane;
      const uint32_t tq = tmem + ((uint32_t)(q4 * 32) << 16);
      uint8_t *act2 = reinterpret_cast<uint8_t *>(S.act2);
      bool ok = true;
      for (int64_t i = 0; ok; i += C::kSlots) {
        if (tile_of(i) >= n_tiles) break;
        int ng = 1;
        while (ng < C::kSlots && tile_of(i + ng) < n_tiles) ++ng;
        const uint32_t par = (uint32_t)((i / C::kSlots) & 1);
        for (int layer = 0; layer < 4 && ok; ++layer) {
          for (int g = 0; g < ng; ++g) {
            if (!__all_sync(0xffffffffu, mbar_wait(&S.mma_done[g][layer], par, abort))) {
              ok = false;
              break;
            }
            fence_after_sync();
            const uint32_t tl = tq + C::d_col(g) + 64 * h;
            // the next layer's A operand: bf16 pairs (BF16, and the FP8
            // variant's head input) or E4M3 quadruples (FP8 hidden layers)
            const uint32_t ta = tq + C::act_col(g), ta8 = tq + C::act8_col(g);
            // two 32-column chunks: BF16 loads both before one wait; FP8
            // (more registers in its conversion) converts the first while
            // the second one's load is in flight
            float va[32], vb[32];
            tmem_ld32(tl, va);
            if (!F8) tmem_ld32(tl + 32, vb);
            tmem_wait_ld_bind(va);
            if (!F8) {
              tmem_wait_ld_bind(vb);
              if (C::act_in_smem(g)) {
                epi_chunk_smem(va, act2, row, 64 * h);
                epi_chunk_smem(vb, act2, row, 64 * h + 32);
                // the generic-proxy stores, before the MMA's async-proxy reads
                fence_async_smem();
              } else {
                epi_chunk(va, ta, 64 * h);
                epi_chunk(vb, ta, 64 * h + 32);
              }
            } else if (layer < 3) {
              tmem_ld32(tl + 32, vb);
              const float dqs = p.dqs[layer];
              epi_chunk8(va, dqs, ta8, 64 * h);
              tmem_wait_ld_bind(vb);
              epi_chunk8(vb, dqs, ta8, 64 * h + 32);
            } else {
              tmem_ld32(tl + 32, vb);
              const float dq = p.dq[layer];
              epi_chunk_dq(va, dq, ta, 64 * h);
              tmem_wait_ld_bind(vb);
              epi_chunk_dq(vb, dq, ta, 64 * h + 32);
            }
            tmem_wait_st();
            fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.act_ready[g]);
          }
        }
        if (!ok) break;
        // the head of slot g is read by the warps of half g & 1
        for (int g = h; g < ng; g += 2) {
          if (!__all_sync(0xffffffffu, mbar_wait(&S.mma_done[g][4], par, abort))) {
            ok = false;
            break;
          }
          fence_after_sync();
          head_store<MODE>(p, S.bias4, tq + C::head_col(g), tile_of(i + g) * TILE + row, ns, lane);
          if (C::kHeadInD) {
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.head_free[g]);
          }
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (tid == 0 && S.abort && p.err) atomicOr(p.err, 8);
  if (warp == C::kMmaWarp) {
    fence_after_sync();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// Shared memory per CTA (plus 1 KB for the 1024-byte alignment of the
// dynamic buffer) within the 227 KB an SM gives one block.
static_assert(sizeof(MlpSmem<false>) + 1024 <= 232448 && sizeof(MlpSmem<true>) + 1024 <= 232448,
              "shared memory");

int g_num_sms = 0;

template <int MODE, bool F8 = false>
int launch_mlp_grid(const MlpParams &p, cudaStream_t stream, int64_t grid_override);

template <int MODE, bool F8 = false>
int launch_mlp(const MlpParams &p, cudaStream_t stream) {
  return launch_mlp_grid<MODE, F8>(p, stream, 0);
}

// grid_override < 0: one CTA per SM (the row count is only known on the
// device); 0: sized from p.ns.
template <int MODE, bool F8>
int launch_mlp_grid(const MlpParams &p, cudaStream_t stream, int64_t grid_override) {
  static bool attr_set = false;
  size_t smem = sizeof(MlpSmem<F8>) + 1024;
  if (!attr_set) {
    if (cudaFuncSetAttribute(mlp_tc_kernel<MODE, F8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
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
  mlp_tc_kernel<MODE, F8><<<(int)grid, Cfg<F8>::kThreads, smem, stream>>>(p);
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

// FP8 variant: weights[0] and weights[4] bf16, weights[1..3] E4M3 bytes;
// scales = {w_scale[1..3], a_scale[1..3]} (positive, finite).
bool set_weights_fp8(MlpParams &p, const void *const weights[5], const float *const biases[5],
                     const float scales[6]) {
  if (!set_weights(p, weights, biases) || !scales) return false;
  for (int i = 0; i < 6; ++i)
    if (!(scales[i] > 0.0f) || !(scales[i] < 3.0e38f)) return false;
  for (int l = 0; l < 3; ++l) p.w8[l] = (const uint8_t *)weights[l + 1];
  p.dq[0] = 1.0f;
  for (int l = 1; l < 4; ++l) p.dq[l] = 1.0f / (scales[l - 1] * scales[3 + l - 1]);
  for (int l = 0; l < 3; ++l) p.qs[l] = scales[3 + l];
  p.qs[3] = 1.0f;
  for (int l = 0; l < 3; ++l) p.dqs[l] = p.dq[l] * p.qs[l];
  return true;
}

// One CTA waits, with the kernels' bounded wait, on an mbarrier phase that
// never completes (nothing arrives). The wait gives up after limit_ns; the
// kernel records bit 3 (8) in err, as the MLP kernels do on a timeout, and
// returns normally.
__global__ void wait_timeout_kernel(uint64_t limit_ns, int32_t *err) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  const bool ok = __all_sync(0xffffffffu, mbar_wait(&bar, 0, &abort_flag, limit_ns));
  if (!ok && threadIdx.x == 0 && err) atomicOr(err, 8);
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
                                float *out, int64_t *outliers, int64_t *n_outliers,
                                int64_t outlier_cap, int32_t *err, void *stream) {
  if (capacity < 0 || !n_samples_dev || n_voxels < 1 || n_keys < 1) return NSVF_ERR_INVALID;
  if (n_outliers && (outlier_cap < 0 || (outlier_cap > 0 && !outliers))) return NSVF_ERR_INVALID;
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
  p.outl = outliers;
  p.n_outl = (unsigned long long *)n_outliers;
  p.outl_cap = outlier_cap;
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

int nsvf_prune_screen_bf16(int64_t n_voxels, int bits, int rule, float step, float threshold,
                           float band, int64_t n_keys, float voxel_size, const float *centers,
                           const int32_t *feats, const float *values,
                           const void *const weights[5], const float *const biases[5],
                           uint32_t *score, uint8_t *keep, int64_t *list, int64_t *n_list,
                           int64_t list_cap, int32_t *err, void *stream) {
  if (n_voxels < 0 || bits < 2 || bits > 64 || (rule != 0 && rule != 1) || n_keys < 1 ||
      list_cap < 0 || !(threshold > 0.0f) || !(band >= 0.0f) || !(threshold < 3.0e38f))
    return NSVF_ERR_INVALID;
  if (n_voxels == 0) return NSVF_OK;
  MlpParams p = {};
  if (!centers || !feats || !values || !score || !keep || !n_list || (list_cap > 0 && !list) ||
      !set_weights(p, weights, biases))
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
  p.keep = keep;
  p.prune_T = threshold;
  p.prune_c = band;
  p.plist = list;
  p.n_plist = (unsigned long long *)n_list;
  p.plist_cap = list_cap;
  p.ns = n_voxels * (int64_t)bits * bits * bits;
  p.err = err;
  return launch_mlp<kPrune>(p, (cudaStream_t)stream);
}

int nsvf_field_samples_fp8_dev(int64_t capacity, const int64_t *n_samples_dev,
                               const int32_t *voxel, const float *xyz_dist, int64_t n_voxels,
                               int64_t n_keys, float voxel_size, const float *centers,
                               const int32_t *feats, const float *values,
                               const void *const weights[5], const float *const biases[5],
                               const float scales[6], float *out, int64_t *outliers,
                               int64_t *n_outliers, int64_t outlier_cap, int32_t *err,
                               void *stream) {
  if (capacity < 0 || !n_samples_dev || n_voxels < 1 || n_keys < 1) return NSVF_ERR_INVALID;
  if (n_outliers && (outlier_cap < 0 || (outlier_cap > 0 && !outliers))) return NSVF_ERR_INVALID;
  if (capacity == 0) return NSVF_OK;
  MlpParams p = {};
  if (!voxel || !xyz_dist || !centers || !feats || !values || !out ||
      !set_weights_fp8(p, weights, biases, scales))
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
  p.outl = outliers;
  p.n_outl = (unsigned long long *)n_outliers;
  p.outl_cap = outlier_cap;
  return launch_mlp_grid<kSamplesIn, true>(p, (cudaStream_t)stream, -1);
}

int nsvf_field_samples_fp8(int64_t n_samples, const int32_t *voxel, const float *xyz_dist,
                           int64_t n_voxels, int64_t n_keys, float voxel_size,
                           const float *centers, const int32_t *feats, const float *values,
                           const void *const weights[5], const float *const biases[5],
                           const float scales[6], float *out, int32_t *err, void *stream) {
  if (n_samples < 0 || n_voxels < 1 || n_keys < 1) return NSVF_ERR_INVALID;
  if (n_samples == 0) return NSVF_OK;
  MlpParams p = {};
  if (!voxel || !xyz_dist || !centers || !feats || !values || !out ||
      !set_weights_fp8(p, weights, biases, scales))
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
  return launch_mlp<kSamplesIn, true>(p, (cudaStream_t)stream);
}

int nsvf_wait_timeout_selftest(uint64_t limit_ns, int32_t *err, void *stream) {
  if (!err || limit_ns == 0 || limit_ns > 1000000000ull) return NSVF_ERR_INVALID;
  wait_timeout_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(limit_ns, err);
  return nsvf_launch_status();
}

}  // extern "C"
