// Kernels of the learned warm start: a small convolutional U-Net trained and
// evaluated on the GPU with hand-written BF16 tensor-core kernels.
//
// Tensors are NHWC.  Activations and activation gradients are BF16; weights
// keep an FP32 master copy and a BF16 copy; every product accumulates in FP32
// (mma.sync m16n8k16, BF16 inputs, FP32 accumulators).  Every convolution is
// 3x3, stride 1, zero padding 1, with input and output channel counts that are
// multiples of 32, and is computed as an implicit GEMM:
//   forward        Y[p, co]   = sum_{tap, ci} X[p + off(tap), ci] W[co, tap, ci]      (M = pixels, N = co, K = 9 cin)
//   data gradient  dX[p, ci]  = the forward with W'[ci, tap, co] = W[co, 8 - tap, ci]  (off(8 - tap) = -off(tap))
//   weight grad    dW[co, k]  = sum_p dY[p, co] X[p + off(tap), ci],  k = tap cin + ci (M = co, N = 9 cin, K = pixels)
// The weight gradient splits the pixel sum over blocks into FP32 partials that
// a second kernel adds in a fixed order, so results are deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/lbm_unet.h"

namespace {

using bf16 = __nv_bfloat16;

constexpr int BM = 64, BN = 64, BK = 32, LDS = BK + 8;  // tile and padded shared row (bf16 elements)

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t lds32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// One 64x64 output tile per block (4 warps, 32x32 each: 2 m16 x 4 n8
// fragments), K consumed in chunks of 32 from the shared tiles As[m][k] and
// Bs[n][k] (k contiguous).
struct Frag {
  float acc[2][4][4];
};

__device__ __forceinline__ void tile_mma(const bf16 (*As)[LDS], const bf16 (*Bs)[LDS], Frag& F) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
#pragma unroll
  for(int kk = 0; kk < BK; kk += 16) {
    uint32_t a[2][4], b[4][2];
#pragma unroll
    for(int mi = 0; mi < 2; ++mi) {
      const int r = wm + mi * 16 + g;
      a[mi][0]    = lds32(&As[r][kk + 2 * t]);
      a[mi][1]    = lds32(&As[r + 8][kk + 2 * t]);
      a[mi][2]    = lds32(&As[r][kk + 2 * t + 8]);
      a[mi][3]    = lds32(&As[r + 8][kk + 2 * t + 8]);
    }
#pragma unroll
    for(int ni = 0; ni < 4; ++ni) {
      const int n = wn + ni * 8 + g;
      b[ni][0]    = lds32(&Bs[n][kk + 2 * t]);
      b[ni][1]    = lds32(&Bs[n][kk + 2 * t + 8]);
    }
#pragma unroll
    for(int mi = 0; mi < 2; ++mi)
#pragma unroll
      for(int ni = 0; ni < 4; ++ni) mma_bf16(F.acc[mi][ni], a[mi], b[ni]);
  }
}

struct ConvFwd {
  const bf16*  x;
  int          ldx;
  const bf16*  w;  // [cout][9 cin]
  const float* bias;
  void*        y;
  int          ldy, offy;
  int          B, H, W, cin, cout;
};

template <bool RELU, bool OUTF32>
__global__ void __launch_bounds__(128) k_conv_fwd(ConvFwd a) {
  __shared__ __align__(16) bf16 As[BM][LDS];
  __shared__ __align__(16) bf16 Bs[BN][LDS];
  const int     tid = threadIdx.x;
  const int64_t P   = static_cast<int64_t>(a.B) * a.H * a.W;
  const int64_t p0  = static_cast<int64_t>(blockIdx.x) * BM;
  const int     n0  = blockIdx.y * BN;
  const int     K   = 9 * a.cin;
  Frag          F;
#pragma unroll
  for(int i = 0; i < 2; ++i)
#pragma unroll
    for(int j = 0; j < 4; ++j)
#pragma unroll
      for(int k = 0; k < 4; ++k) F.acc[i][j][k] = 0.f;

  for(int k0 = 0; k0 < K; k0 += BK) {
    const int tap = k0 / a.cin, ci0 = k0 - tap * a.cin;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
    for(int it = 0; it < 2; ++it) {
      const int     idx = tid + it * 128;
      const int     r = idx >> 2, part = idx & 3;
      const int64_t p   = p0 + r;
      uint4         v   = make_uint4(0, 0, 0, 0);
      if(p < P) {
        const int64_t hw = static_cast<int64_t>(a.H) * a.W;
        const int     b  = static_cast<int>(p / hw);
        const int     rem = static_cast<int>(p - static_cast<int64_t>(b) * hw);
        const int     yy = rem / a.W + dy, xx = rem % a.W + dx;
        if(yy >= 0 && yy < a.H && xx >= 0 && xx < a.W)
          v = *reinterpret_cast<const uint4*>(a.x + ((static_cast<int64_t>(b) * a.H + yy) * a.W + xx) * a.ldx + ci0 + part * 8);
      }
      *reinterpret_cast<uint4*>(&As[r][part * 8]) = v;
      const int co = n0 + r;
      uint4     wv = make_uint4(0, 0, 0, 0);
      if(co < a.cout) wv = *reinterpret_cast<const uint4*>(a.w + static_cast<int64_t>(co) * K + k0 + part * 8);
      *reinterpret_cast<uint4*>(&Bs[r][part * 8]) = wv;
    }
    __syncthreads();
    tile_mma(As, Bs, F);
    __syncthreads();
  }
  const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
#pragma unroll
  for(int mi = 0; mi < 2; ++mi)
#pragma unroll
    for(int ni = 0; ni < 4; ++ni)
#pragma unroll
      for(int h = 0; h < 2; ++h) {
        const int64_t p  = p0 + wm + mi * 16 + g + 8 * h;
        const int     co = n0 + wn + ni * 8 + 2 * t;
        if(p >= P || co >= a.cout) continue;
        float v0 = F.acc[mi][ni][2 * h] + a.bias[co], v1 = F.acc[mi][ni][2 * h + 1] + a.bias[co + 1];
        if(RELU) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        const int64_t o = p * a.ldy + a.offy + co;
        if(OUTF32) {
          *reinterpret_cast<float2*>(static_cast<float*>(a.y) + o) = make_float2(v0, v1);
        } else {
          *reinterpret_cast<__nv_bfloat162*>(static_cast<bf16*>(a.y) + o) = __floats2bfloat162_rn(v0, v1);
        }
      }
}

struct ConvWgrad {
  const bf16* x;
  int         ldx;
  const bf16* dy;
  int         lddy;
  float*      part;  // [nsplit][cout][9 cin]
  int         B, H, W, cin, cout;
  int64_t     pix_per_split;
};

__global__ void __launch_bounds__(128) k_conv_wgrad(ConvWgrad a) {
  __shared__ __align__(16) bf16 As[BM][LDS];  // [co][pixel]
  __shared__ __align__(16) bf16 Bs[BN][LDS];  // [k][pixel]
  const int     tid = threadIdx.x;
  const int64_t P   = static_cast<int64_t>(a.B) * a.H * a.W;
  const int     m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int     K  = 9 * a.cin;
  const int64_t pa = static_cast<int64_t>(blockIdx.z) * a.pix_per_split;
  const int64_t pb = pa + a.pix_per_split < P ? pa + a.pix_per_split : P;
  const int64_t hw = static_cast<int64_t>(a.H) * a.W;
  Frag          F;
#pragma unroll
  for(int i = 0; i < 2; ++i)
#pragma unroll
    for(int j = 0; j < 4; ++j)
#pragma unroll
      for(int k = 0; k < 4; ++k) F.acc[i][j][k] = 0.f;

  for(int64_t q0 = pa; q0 < pb; q0 += BK) {
#pragma unroll
    for(int it = 0; it < 2; ++it) {
      const int     idx = tid + it * 128;  // 32 pixels x 8 chunks of 8 channels
      const int     pp = idx >> 3, ch = idx & 7;
      const int64_t p  = q0 + pp;
      // dY[p][m0 + 8 ch ..] -> As[m0 + 8 ch + j][pp]
      uint4 v = make_uint4(0, 0, 0, 0);
      if(p < pb && m0 + ch * 8 < a.cout) v = *reinterpret_cast<const uint4*>(a.dy + p * a.lddy + m0 + ch * 8);
      const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
      for(int j = 0; j < 8; ++j) As[ch * 8 + j][pp] = e[j];
      // X[p + off(tap)][ci ..] -> Bs[k - n0][pp], k = n0 + 8 ch + j
      const int k = n0 + ch * 8;
      uint4     u = make_uint4(0, 0, 0, 0);
      if(p < pb && k < K) {
        const int tap = k / a.cin, ci = k - tap * a.cin;
        const int b   = static_cast<int>(p / hw);
        const int rem = static_cast<int>(p - static_cast<int64_t>(b) * hw);
        const int yy = rem / a.W + tap / 3 - 1, xx = rem % a.W + tap % 3 - 1;
        if(yy >= 0 && yy < a.H && xx >= 0 && xx < a.W)
          u = *reinterpret_cast<const uint4*>(a.x + ((static_cast<int64_t>(b) * a.H + yy) * a.W + xx) * a.ldx + ci);
      }
      const bf16* f = reinterpret_cast<const bf16*>(&u);
#pragma unroll
      for(int j = 0; j < 8; ++j) Bs[ch * 8 + j][pp] = f[j];
    }
    __syncthreads();
    tile_mma(As, Bs, F);
    __syncthreads();
  }
  const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  float*    out = a.part + static_cast<int64_t>(blockIdx.z) * a.cout * K;
#pragma unroll
  for(int mi = 0; mi < 2; ++mi)
#pragma unroll
    for(int ni = 0; ni < 4; ++ni)
#pragma unroll
      for(int h = 0; h < 2; ++h) {
        const int co = m0 + wm + mi * 16 + g + 8 * h;
        const int k  = n0 + wn + ni * 8 + 2 * t;
        if(co >= a.cout || k >= K) continue;
        *reinterpret_cast<float2*>(out + static_cast<int64_t>(co) * K + k) = make_float2(F.acc[mi][ni][2 * h], F.acc[mi][ni][2 * h + 1]);
      }
}

// dW = sum over splits (fixed order)
__global__ void k_sum_splits(const float* part, int nsplit, int64_t n, float* out) {
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float s = 0.f;
    for(int z = 0; z < nsplit; ++z) s += part[z * n + i];
    out[i] = s;
  }
}

// bias gradient: per channel, the sum over pixels; block c sums channel c in a fixed order
__global__ void k_bias_grad(const bf16* dy, int lddy, int64_t P, int c0, float* db) {
  __shared__ float sh[32];
  const int c   = blockIdx.x;
  float     acc = 0.f;
  for(int64_t p = threadIdx.x; p < P; p += blockDim.x) acc += __bfloat162float(dy[p * lddy + c0 + c]);
#pragma unroll
  for(int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if(threadIdx.x < 32) {
    float s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if(threadIdx.x == 0) db[c] = s;
  }
}

// W'[ci][tap][co] = W[co][8 - tap][ci]
__global__ void k_flip(const bf16* w, bf16* wt, int cin, int cout) {
  const int64_t n = static_cast<int64_t>(cin) * 9 * cout;
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int co  = static_cast<int>(i % cout);
    const int tap = static_cast<int>((i / cout) % 9);
    const int ci  = static_cast<int>(i / (9 * static_cast<int64_t>(cout)));
    wt[i]         = w[(static_cast<int64_t>(co) * 9 + (8 - tap)) * cin + ci];
  }
}

// dx = dy * (y > 0) over npix x c channels (each with its own stride / offset)
__global__ void k_relu_bwd(const bf16* dy, int lddy, int offdy, const bf16* y, int ldy, int offy, bf16* dx, int lddx, int64_t npix, int c) {
  const int64_t n = npix * c;
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t p = i / c;
    const int     k = static_cast<int>(i - p * c);
    const float   g = __bfloat162float(dy[p * lddy + offdy + k]);
    dx[p * lddx + k] = __float2bfloat16_rn(__bfloat162float(y[p * ldy + offy + k]) > 0.f ? g : 0.f);
  }
}

// 2x2 max pooling; x [B,H,W] at stride ldx / offset offx, y [B,H/2,W/2,C] dense
__global__ void k_pool_fwd(const bf16* x, int ldx, int offx, bf16* y, int B, int H, int W, int C) {
  const int     h = H / 2, w = W / 2;
  const int64_t n = static_cast<int64_t>(B) * h * w * C;
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int     c  = static_cast<int>(i % C);
    const int64_t q  = i / C;
    const int     xo = static_cast<int>(q % w), yo = static_cast<int>((q / w) % h), b = static_cast<int>(q / (static_cast<int64_t>(w) * h));
    float         m  = -3.0e38f;
#pragma unroll
    for(int d = 0; d < 4; ++d) {
      const int64_t src = (static_cast<int64_t>(b) * H + 2 * yo + (d >> 1)) * W + 2 * xo + (d & 1);
      m                 = fmaxf(m, __bfloat162float(x[src * ldx + offx + c]));
    }
    y[i] = __float2bfloat16_rn(m);
  }
}

// gradient of the pooling, added into dx (stride lddx / offset offdx): the
// first maximum of each window takes the gradient
__global__ void k_pool_bwd(const bf16* x, int ldx, int offx, const bf16* dy, bf16* dx, int lddx, int offdx, int B, int H, int W, int C) {
  const int     h = H / 2, w = W / 2;
  const int64_t n = static_cast<int64_t>(B) * h * w * C;
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int     c  = static_cast<int>(i % C);
    const int64_t q  = i / C;
    const int     xo = static_cast<int>(q % w), yo = static_cast<int>((q / w) % h), b = static_cast<int>(q / (static_cast<int64_t>(w) * h));
    float         m  = -3.0e38f;
    int           am = 0;
#pragma unroll
    for(int d = 0; d < 4; ++d) {
      const int64_t src = (static_cast<int64_t>(b) * H + 2 * yo + (d >> 1)) * W + 2 * xo + (d & 1);
      const float   v   = __bfloat162float(x[src * ldx + offx + c]);
      if(v > m) {
        m  = v;
        am = d;
      }
    }
    const int64_t dst = (static_cast<int64_t>(b) * H + 2 * yo + (am >> 1)) * W + 2 * xo + (am & 1);
    bf16&         o   = dx[dst * lddx + offdx + c];
    o                 = __float2bfloat16_rn(__bfloat162float(o) + __bfloat162float(dy[i]));
  }
}

// nearest 2x upsampling: x [B,h,w,C] dense -> y [B,2h,2w] at stride ldy
__global__ void k_up_fwd(const bf16* x, bf16* y, int ldy, int B, int h, int w, int C) {
  const int64_t n = static_cast<int64_t>(B) * 4 * h * w * C;
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int     c = static_cast<int>(i % C);
    const int64_t q = i / C;
    const int     X = static_cast<int>(q % (2 * w)), Y = static_cast<int>((q / (2 * w)) % (2 * h)), b = static_cast<int>(q / (4 * static_cast<int64_t>(w) * h));
    y[q * ldy + c]  = x[((static_cast<int64_t>(b) * h + Y / 2) * w + X / 2) * C + c];
  }
}

// its gradient: each coarse cell sums its four fine cells
__global__ void k_up_bwd(const bf16* dy, int lddy, bf16* dx, int B, int h, int w, int C) {
  const int64_t n = static_cast<int64_t>(B) * h * w * C;
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int     c = static_cast<int>(i % C);
    const int64_t q = i / C;
    const int     x = static_cast<int>(q % w), y = static_cast<int>((q / w) % h), b = static_cast<int>(q / (static_cast<int64_t>(w) * h));
    float         s = 0.f;
#pragma unroll
    for(int d = 0; d < 4; ++d) s += __bfloat162float(dy[((static_cast<int64_t>(b) * 2 * h + 2 * y + (d >> 1)) * 2 * w + 2 * x + (d & 1)) * lddy + c]);
    dx[i] = __float2bfloat16_rn(s);
  }
}

// masked mean-square loss over the first `nout` channels of pred (stride ldp)
// against target [P][nout]; dpred (bf16, stride ldp, zero elsewhere) and one
// partial loss per block
__global__ void k_mse(const float* pred, int ldp, const float* target, const uint8_t* fluid, int64_t P, int nout, float inv_count,
                      bf16* dpred, float* partial) {
  __shared__ float sh[32];
  float            acc = 0.f;
  for(int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < P; p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const bool on = fluid[p] != 0;
    for(int c = 0; c < ldp; ++c) {
      float g = 0.f;
      if(c < nout && on) {
        const float d = pred[p * ldp + c] - target[p * nout + c];
        acc += d * d;
        g = 2.f * d * inv_count;
      }
      dpred[p * ldp + c] = __float2bfloat16_rn(g);
    }
  }
#pragma unroll
  for(int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if(threadIdx.x < 32) {
    float s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if(threadIdx.x == 0) partial[blockIdx.x] = s;
  }
}

// Adam on the FP32 master weights, refreshing the BF16 copy
__global__ void k_adam(float* w, bf16* w16, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i]           = mi;
    v[i]           = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    w[i]           = wi;
    if(w16) w16[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void k_to_bf16(const float* a, bf16* b, int64_t n) {
  for(int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    b[i] = __float2bfloat16_rn(a[i]);
}

unsigned blocks_for(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return static_cast<unsigned>(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

int status(cudaError_t e) { return e == cudaSuccess ? 0 : -2; }

}  // namespace

namespace lbm {
bool conv_tc_qualifies(const void* x, int ldx, const void* w, const void* y, int ldy, int offy, int B, int H, int W, int cin, int cout,
                       int out_f32);
int  conv_tc_launch(const void* x, int ldx, const void* w, const float* bias, void* y, int ldy, int offy, int B, int H, int W, int cin,
                    int cout, int relu, int out_f32, cudaStream_t s);
}  // namespace lbm

extern "C" {

int lbm_nn_conv3x3_fwd(const void* x, int ldx, const void* w, const float* bias, void* y, int ldy, int offy, int B, int H, int W, int cin,
                       int cout, int relu, int out_f32, void* stream) {
  if(cin % 32 || cout % 32 || ldx % 8 || ldx < cin || (!out_f32 && ldy % 2) || offy % 2 || B <= 0 || H <= 0 || W <= 0) return -1;
  // the tcgen05 kernel (conv_tc.cu) where the shape and alignment qualify
  if(lbm::conv_tc_qualifies(x, ldx, w, y, ldy, offy, B, H, W, cin, cout, out_f32))
    return lbm::conv_tc_launch(x, ldx, w, bias, y, ldy, offy, B, H, W, cin, cout, relu, out_f32, static_cast<cudaStream_t>(stream));
  ConvFwd a{static_cast<const bf16*>(x), ldx, static_cast<const bf16*>(w), bias, y, ldy, offy, B, H, W, cin, cout};
  const int64_t P = static_cast<int64_t>(B) * H * W;
  dim3          grid(static_cast<unsigned>((P + BM - 1) / BM), static_cast<unsigned>((cout + BN - 1) / BN));
  cudaStream_t  s = static_cast<cudaStream_t>(stream);
  if(out_f32) {
    if(relu) k_conv_fwd<true, true><<<grid, 128, 0, s>>>(a);
    else k_conv_fwd<false, true><<<grid, 128, 0, s>>>(a);
  } else {
    if(relu) k_conv_fwd<true, false><<<grid, 128, 0, s>>>(a);
    else k_conv_fwd<false, false><<<grid, 128, 0, s>>>(a);
  }
  return status(cudaGetLastError());
}

int lbm_nn_conv3x3_wgrad(const void* x, int ldx, const void* dy, int lddy, float* partial, int64_t partial_floats, float* dw, int B, int H,
                         int W, int cin, int cout, void* stream) {
  if(cin % 32 || cout % 32 || ldx % 8 || lddy % 8) return -1;
  const int64_t P      = static_cast<int64_t>(B) * H * W;
  const int64_t K      = 9 * static_cast<int64_t>(cin);
  const int64_t per    = 2048;
  int64_t       nsplit = (P + per - 1) / per;
  while(nsplit * cout * K > partial_floats && nsplit > 1) nsplit = (nsplit + 1) / 2;
  if(nsplit * cout * K > partial_floats) return -1;
  const int64_t pps = ((P + nsplit - 1) / nsplit + BK - 1) / BK * BK;
  nsplit            = (P + pps - 1) / pps;
  ConvWgrad    a{static_cast<const bf16*>(x), ldx, static_cast<const bf16*>(dy), lddy, partial, B, H, W, cin, cout, pps};
  dim3         grid(static_cast<unsigned>((cout + BM - 1) / BM), static_cast<unsigned>((K + BN - 1) / BN), static_cast<unsigned>(nsplit));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_conv_wgrad<<<grid, 128, 0, s>>>(a);
  k_sum_splits<<<blocks_for(cout * K), 256, 0, s>>>(partial, static_cast<int>(nsplit), cout * K, dw);
  return status(cudaGetLastError());
}

int lbm_nn_bias_grad(const void* dy, int lddy, int64_t npix, int c, float* db, void* stream) {
  k_bias_grad<<<c, 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(dy), lddy, npix, 0, db);
  return status(cudaGetLastError());
}

int lbm_nn_flip_weights(const void* w, void* wt, int cin, int cout, void* stream) {
  k_flip<<<blocks_for(9 * static_cast<int64_t>(cin) * cout), 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(w),
                                                                                                      static_cast<bf16*>(wt), cin, cout);
  return status(cudaGetLastError());
}

int lbm_nn_relu_bwd(const void* dy, int lddy, int offdy, const void* y, int ldy, int offy, void* dx, int lddx, int64_t npix, int c,
                    void* stream) {
  k_relu_bwd<<<blocks_for(npix * c), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(dy), lddy, offdy, static_cast<const bf16*>(y), ldy, offy, static_cast<bf16*>(dx), lddx, npix, c);
  return status(cudaGetLastError());
}

int lbm_nn_pool_fwd(const void* x, int ldx, int offx, void* y, int B, int H, int W, int C, void* stream) {
  if(H % 2 || W % 2) return -1;
  k_pool_fwd<<<blocks_for(static_cast<int64_t>(B) * H * W * C / 4), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(x), ldx, offx, static_cast<bf16*>(y), B, H, W, C);
  return status(cudaGetLastError());
}

int lbm_nn_pool_bwd(const void* x, int ldx, int offx, const void* dy, void* dx, int lddx, int offdx, int B, int H, int W, int C, void* stream) {
  if(H % 2 || W % 2) return -1;
  k_pool_bwd<<<blocks_for(static_cast<int64_t>(B) * H * W * C / 4), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(x), ldx, offx, static_cast<const bf16*>(dy), static_cast<bf16*>(dx), lddx, offdx, B, H, W, C);
  return status(cudaGetLastError());
}

int lbm_nn_up_fwd(const void* x, void* y, int ldy, int B, int h, int w, int C, void* stream) {
  k_up_fwd<<<blocks_for(static_cast<int64_t>(B) * 4 * h * w * C), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(x), static_cast<bf16*>(y), ldy, B, h, w, C);
  return status(cudaGetLastError());
}

int lbm_nn_up_bwd(const void* dy, int lddy, void* dx, int B, int h, int w, int C, void* stream) {
  k_up_bwd<<<blocks_for(static_cast<int64_t>(B) * h * w * C), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(dy), lddy, static_cast<bf16*>(dx), B, h, w, C);
  return status(cudaGetLastError());
}

int lbm_nn_mse(const float* pred, int ldp, const float* target, const uint8_t* fluid, int64_t npix, int nout, float inv_count, void* dpred,
               float* partial, int nblocks, void* stream) {
  k_mse<<<nblocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(pred, ldp, target, fluid, npix, nout, inv_count, static_cast<bf16*>(dpred),
                                                                partial);
  return status(cudaGetLastError());
}

int lbm_nn_adam(float* w, void* w16, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps, int step,
                void* stream) {
  const float c1 = 1.f / (1.f - powf(b1, static_cast<float>(step)));
  const float c2 = 1.f / (1.f - powf(b2, static_cast<float>(step)));
  k_adam<<<blocks_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(w, static_cast<bf16*>(w16), g, m, v, n, lr, b1, b2, eps, c1, c2);
  return status(cudaGetLastError());
}

int lbm_nn_to_bf16(const float* a, void* b, int64_t n, void* stream) {
  k_to_bf16<<<blocks_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(a, static_cast<bf16*>(b), n);
  return status(cudaGetLastError());
}

}  // extern "C"
