// Tensor-core forward 3x3 convolution of the warm-start U-Net on the
// 5th-generation tensor cores (tcgen05): TMA-tiled operands in shared memory,
// the accumulator in tensor memory (TMEM).
//
// The convolution is the implicit GEMM  Y[p, co] = sum_{tap, ci} X[p + off(tap), ci] W[co, tap, ci]
// (M = pixels, N = co, K = 9 cin).  One CTA computes a tile of 128 pixels
// (one image row segment of 128, or 128 / W whole rows when W < 128) times
// all cout <= 256 output channels:
//   * K is consumed in chunks of one tap x 32 input channels (64-byte rows).
//     The A chunk is one 4D TMA box {32 channels, Wb, Hb, 1} of the NHWC
//     activations at (c0, x0 + dx, y0 + dy, b): the box's out-of-range
//     pixels read as zero, which is the convolution's zero padding.  The B
//     chunk is one 2D box {32, cout} of the weights [cout][9 cin].  Both land
//     in shared memory with the 64-byte swizzle, the canonical K-major
//     layout the MMA reads (8-row atoms of 512 bytes).
//   * A 4-stage ring of chunks: thread 0 issues the TMA loads (mbarrier
//     complete_tx), thread 32 issues two tcgen05.mma (M 128, N cout, K 16,
//     BF16 inputs, FP32 accumulation in TMEM) per chunk and frees the stage
//     with tcgen05.commit.
//   * Epilogue: the four warps read their 32 TMEM lanes (one pixel each) 32
//     columns at a time (tcgen05.ld 32x32b), add the bias, apply the ReLU and
//     store BF16 or FP32 rows.
// Every mbarrier wait is bounded; a wait that runs out sets the error word
// (read by lbm_nn_conv_status), the CTA drains its own copies in flight,
// waits for its issued MMAs and frees its TMEM before it returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "../../include/lbm_unet.h"
#include "bulk_copy.cuh"

namespace lbm {
namespace {

constexpr int      kTileM      = 128;   // pixels per tile = TMEM lanes
constexpr int      kChunkK     = 32;    // bf16 per K chunk: 64-byte rows
constexpr int      kStages     = 4;
constexpr uint32_t kABytes     = kTileM * kChunkK * 2;  // 8 KB
constexpr uint64_t kWaitNs     = 200000000ull;          // 0.2 s per pipeline wait
constexpr int      kThreads    = 128;

__device__ int g_conv_err = 0;

struct ConvTc {
  const float* bias;
  void*        y;
  int64_t      ldy;
  int          offy;
  int          H, W, cout;
  int          wb, hb;      // TMA box: Wb pixels x Hb rows = 128
  int          cin_chunks;  // cin / 32
  int          nchunk;      // 9 cin / 32
  uint64_t     limit_ns;    // limit of each pipeline wait
  int          starve;      // test only: the first chunk is never loaded, so the waits on it run out
};

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
               : "memory");
}

// shared-memory matrix descriptor of a K-major operand in the 64-byte swizzle:
// start address, leading offset 1 (unused for swizzled K-major), stride 512 B
// between 8-row groups, descriptor version 1, layout SWIZZLE_64B (4)
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
  uint64_t d = static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>(1) << 16;
  d |= static_cast<uint64_t>(512 >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= static_cast<uint64_t>(4) << 61;
  return d;
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at
// bits 17-22, M >> 4 at bits 24-28
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16_tmem(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive on the barrier once every tcgen05 operation this thread issued before is complete
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, "
      "%20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
        "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__host__ __device__ constexpr uint32_t tmem_cols(int n) { return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : 256u; }

__host__ __device__ constexpr uint32_t stage_bytes(int n) { return kABytes + static_cast<uint32_t>(n) * kChunkK * 2; }

// dynamic shared memory: 1 KB of alignment slack, the stage ring, then the
// barriers (full[S], empty[S], done) and the TMEM address slot
inline size_t smem_bytes(int n) { return 1024 + kStages * static_cast<size_t>(stage_bytes(n)) + 128; }

template <bool RELU, bool OUTF32>
__global__ void __launch_bounds__(kThreads) k_conv_tc(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw, ConvTc a) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw   = smem_u32(smem_raw);
  const uint32_t base  = (raw + 1023u) & ~1023u;
  const int      n     = a.cout;
  const uint32_t sbyte = stage_bytes(n);
  const uint32_t bars  = base + kStages * sbyte;  // full[s] at bars + 8 s, empty[s] at bars + 8 (S + s), done at bars + 16 S
  const uint32_t done  = bars + 16 * kStages;
  const uint32_t slot  = done + 8;
  uint8_t*       slot_ptr = smem_raw + (slot - raw);
  const int      warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = tmem_cols(n);

  if(threadIdx.x == 0) {
    for(int s = 0; s < kStages; ++s) {
      mbar_init(bars + 8 * s, 1);
      mbar_init(bars + 8 * (kStages + s), 1);
    }
    mbar_init(done, 1);
    fence_async_smem();
  }
  if(warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(slot_ptr);

  // the tile: 128 consecutive pixels of one image
  const int64_t p0  = static_cast<int64_t>(blockIdx.x) * kTileM;
  const int64_t hw  = static_cast<int64_t>(a.H) * a.W;
  const int     b   = static_cast<int>(p0 / hw);
  const int     rem = static_cast<int>(p0 - b * hw);
  const int     y0 = rem / a.W, x0 = rem - (rem / a.W) * a.W;
  bool          ok = true;

  if(threadIdx.x == 0) {
    // producer: chunk kc = tap * cin_chunks + cc into stage kc % S
    int kc = 0;
    for(; kc < a.nchunk; ++kc) {
      const int      s  = kc % kStages;
      const uint32_t st = base + s * sbyte;
      if(kc >= kStages && !mbar_wait_bounded(bars + 8 * (kStages + s), ((kc / kStages) - 1) & 1, a.limit_ns)) {
        ok = false;
        break;
      }
      if(a.starve && kc == 0) continue;  // test only: nothing arms this stage
      const int tap = kc / a.cin_chunks, cc = kc - tap * a.cin_chunks;
      const int dy = tap / 3 - 1, dx = tap - (tap / 3) * 3 - 1;
      mbar_expect_tx(bars + 8 * s, sbyte);
      tma_load_4d(st, &tx, cc * kChunkK, x0 + dx, y0 + dy, b, bars + 8 * s);
      tma_load_2d(st + kABytes, &tw, kc * kChunkK, 0, bars + 8 * s);
    }
    // every load issued lands before the CTA may leave
    for(int s = 0; s < kStages && s < kc; ++s) {
      const int last = s + ((kc - 1 - s) / kStages) * kStages;  // the last chunk issued into stage s
      if(a.starve && last == 0) continue;                        // never issued
      if(!mbar_wait_bounded(bars + 8 * s, (last / kStages) & 1, kDrainLimitNs)) ok = false;
    }
  } else if(threadIdx.x == 32) {
    // MMA issuer
    const uint32_t idesc = mma_idesc(kTileM, n);
    for(int kc = 0; kc < a.nchunk; ++kc) {
      const int      s  = kc % kStages;
      const uint32_t st = base + s * sbyte;
      if(!mbar_wait_bounded(bars + 8 * s, (kc / kStages) & 1, a.limit_ns)) {
        ok = false;
        break;
      }
      tc_fence_after();
#pragma unroll
      for(int k = 0; k < kChunkK / 16; ++k)
        mma_bf16_tmem(tmem, sw64_desc(st + 32 * k), sw64_desc(st + kABytes + 32 * k), idesc, (kc | k) != 0);
      mma_commit(bars + 8 * (kStages + s));
    }
    // always: `done` completes once every MMA issued above has
    mma_commit(done);
  }
  __syncwarp();

  // epilogue: warp w owns TMEM lanes 32 w .. 32 w + 31 (pixels of the tile)
  // warp-uniform, as the TMEM loads below are warp-collective
  const bool have = __all_sync(0xffffffffu, mbar_wait_bounded(done, 0, 2 * a.limit_ns + kDrainLimitNs));
  tc_fence_after();
  if(!have) ok = false;
  if(have) {
    const int64_t p   = p0 + warp * 32 + lane;
    const uint32_t tl = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    for(int c0 = 0; c0 < n; c0 += 32) {
      uint32_t r[32];
      tmem_ld32(tl + c0, r);
      float v[32];
#pragma unroll
      for(int j = 0; j < 32; ++j) {
        v[j] = __uint_as_float(r[j]) + __ldg(a.bias + c0 + j);
        if(RELU) v[j] = fmaxf(v[j], 0.f);
      }
      if(OUTF32) {
        float4* dst = reinterpret_cast<float4*>(static_cast<float*>(a.y) + p * a.ldy + a.offy + c0);
#pragma unroll
        for(int j = 0; j < 8; ++j) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
      } else {
        uint4* dst = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(a.y) + p * a.ldy + a.offy + c0);
#pragma unroll
        for(int j = 0; j < 4; ++j) {
          __nv_bfloat162 h[4];
#pragma unroll
          for(int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(v[8 * j + 2 * i], v[8 * j + 2 * i + 1]);
          uint4 u;
          memcpy(&u, h, sizeof(u));
          dst[j] = u;
        }
      }
    }
  }
  if(!ok) atomicExch(&g_conv_err, 1);
  tc_fence_before();
  __syncthreads();
  if(warp == 2) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static EncodeTiled fn = [] {
    void*                           p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
       q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int      g_conv_path     = 0;        // 0: tensor-core kernel where the shape qualifies; 1: never
uint64_t g_conv_limit_ns = kWaitNs;  // pipeline wait limit (lbm_nn_conv_test_wait)
int      g_conv_starve   = 0;

}  // namespace

// whether the tensor-core kernel takes this convolution
bool conv_tc_qualifies(const void* x, int ldx, const void* w, const void* y, int ldy, int offy, int B, int H, int W, int cin, int cout,
                       int out_f32) {
  if(g_conv_path != 0 || !encoder()) return false;
  if(cin % 32 || cout % 32 || cout > 256 || cout < 32 || ldx % 8 || B <= 0 || H <= 0 || W <= 0) return false;
  if(!(W % kTileM == 0 || (kTileM % W == 0 && H % (kTileM / W) == 0))) return false;
  if(!aligned16(x) || !aligned16(w) || !aligned16(y)) return false;
  if(out_f32 ? (ldy % 4 || offy % 4) : (ldy % 8 || offy % 8)) return false;
  return true;
}

int conv_tc_launch(const void* x, int ldx, const void* w, const float* bias, void* y, int ldy, int offy, int B, int H, int W, int cin, int cout,
                   int relu, int out_f32, cudaStream_t s) {
  EncodeTiled enc = encoder();
  CUtensorMap tx, tw;
  const int   wb = W >= kTileM ? kTileM : W, hb = kTileM / wb;
  {
    const cuuint64_t dims[4]    = {static_cast<cuuint64_t>(cin), static_cast<cuuint64_t>(W), static_cast<cuuint64_t>(H),
                                   static_cast<cuuint64_t>(B)};
    const cuuint64_t strides[3] = {static_cast<cuuint64_t>(ldx) * 2, static_cast<cuuint64_t>(ldx) * 2 * W,
                                   static_cast<cuuint64_t>(ldx) * 2 * W * H};
    const cuuint32_t box[4]     = {static_cast<cuuint32_t>(kChunkK), static_cast<cuuint32_t>(wb), static_cast<cuuint32_t>(hb), 1};
    const cuuint32_t estr[4]    = {1, 1, 1, 1};
    if(enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
           CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return -1;
  }
  {
    const cuuint64_t dims[2]    = {static_cast<cuuint64_t>(9) * cin, static_cast<cuuint64_t>(cout)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(9) * cin * 2};
    const cuuint32_t box[2]     = {static_cast<cuuint32_t>(kChunkK), static_cast<cuuint32_t>(cout)};
    const cuuint32_t estr[2]    = {1, 1};
    if(enc(&tw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(w), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
           CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return -1;
  }
  ConvTc a{bias, y, ldy, offy, H, W, cout, wb, hb, cin / kChunkK, 9 * cin / kChunkK, g_conv_limit_ns, g_conv_starve};
  const int64_t tiles = static_cast<int64_t>(B) * H * W / kTileM;
  const size_t  smem  = smem_bytes(cout);
  auto          kern  = relu ? (out_f32 ? k_conv_tc<true, true> : k_conv_tc<true, false>)
                             : (out_f32 ? k_conv_tc<false, true> : k_conv_tc<false, false>);
  if(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess) return -2;
  kern<<<static_cast<unsigned>(tiles), kThreads, smem, s>>>(tx, tw, a);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // namespace lbm

extern "C" {

int lbm_nn_set_conv_path(int path) {
  if(path != 0 && path != 1) return -1;
  lbm::g_conv_path = path;
  return 0;
}

int lbm_nn_conv_test_wait(int64_t limit_ns, int32_t starve) {
  if(limit_ns <= 0 || limit_ns > 500000000 || (starve != 0 && starve != 1)) return -1;
  lbm::g_conv_limit_ns = static_cast<uint64_t>(limit_ns);
  lbm::g_conv_starve   = starve;
  return 0;
}

int lbm_nn_conv_uses_tc(const void* x, int ldx, const void* w, const void* y, int ldy, int offy, int B, int H, int W, int cin, int cout,
                        int out_f32) {
  return lbm::conv_tc_qualifies(x, ldx, w, y, ldy, offy, B, H, W, cin, cout, out_f32) ? 1 : 0;
}

int lbm_nn_conv_status(void* stream) {
  cudaStream_t s   = static_cast<cudaStream_t>(stream);
  int          err = 0;
  const int    zero = 0;
  if(cudaMemcpyFromSymbolAsync(&err, lbm::g_conv_err, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess) return -2;
  if(cudaMemcpyToSymbolAsync(lbm::g_conv_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s) != cudaSuccess) return -2;
  if(cudaStreamSynchronize(s) != cudaSuccess) return -2;
  return err ? -6 : 0;
}

}  // extern "C"
