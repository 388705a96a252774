// fargo_mlp.cu -- the stencil MLP of the learned coarse-grid correction.
//
// Network (per coarse cell): 128 inputs (a 5x5 stencil of 5 channels, padded
// with 3 zeros) -> 64 (GELU) -> 64 (GELU) -> 2 outputs (the radial and azimuthal
// mass-flux corrections of the cell).  BF16 weights and activations, FP32
// accumulation, on the tensor cores with mma.sync m16n8k16 (the layers are
// K = 64..128 by N = 64: one warp holds a 16-row tile and keeps every activation
// in registers between the layers).  Training: the forward pass keeps the
// pre-activations; the backward pass forms the data gradients with the same
// fragments and the per-CTA weight gradients (X^T dZ etc.) from transposed tiles
// staged in shared memory; a fixed-order reduction over the CTAs (deterministic)
// and Adam on FP32 master weights follow.
//
// Fragment layouts of mma.m16n8k16 (.row.col, BF16 in, FP32 out; g = lane / 4,
// t = lane % 4): A 16x16 row-major: a0 (g, 2t..2t+1), a1 (g+8, 2t..), a2 (g, 2t+8..),
// a3 (g+8, 2t+8..); B 16x8 column-major: b0 (k 2t..2t+1, n g), b1 (k 2t+8.., n g);
// C 16x8: c0,c1 (g, 2t..2t+1), c2,c3 (g+8, 2t..2t+1).  The C tiles of two adjacent
// 8-column blocks are exactly the A fragment of the next layer's 16-wide k block.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "fargo_gb300.h"

#define MLP_IN 128
#define MLP_H 64
#define MLP_OUT 2
#define MLP_OUTP 8      // output columns of the last mma (the 2 outputs, zero-padded)
#define MLP_ROWS 64     // rows (cells) per CTA: 4 warps x 16
// FP32 parameter blob: W1 [128][64], b1 [64], W2 [64][64], b2 [64], W3 [64][8], b3 [8]
// (W[in][out]; the last layer's columns 2..7 stay zero)
#define MLP_OFF_W1 0
#define MLP_OFF_B1 (MLP_OFF_W1 + MLP_IN * MLP_H)
#define MLP_OFF_W2 (MLP_OFF_B1 + MLP_H)
#define MLP_OFF_B2 (MLP_OFF_W2 + MLP_H * MLP_H)
#define MLP_OFF_W3 (MLP_OFF_B2 + MLP_H)
#define MLP_OFF_B3 (MLP_OFF_W3 + MLP_H * MLP_OUTP)
#define MLP_NPARAM (MLP_OFF_B3 + MLP_OUTP)

static_assert(MLP_NPARAM == FARGO_MLP_NPARAM, "parameter blob size");

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ unsigned pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  unsigned r;
  memcpy(&r, &v, 4);
  return r;
}
__device__ __forceinline__ float2 unpack2(unsigned u) {
  __nv_bfloat162 v;
  memcpy(&v, &u, 4);
  return __bfloat1622float2(v);
}
__device__ __forceinline__ unsigned ld_u32(const bf16 *p) { return *reinterpret_cast<const unsigned *>(p); }

__device__ __forceinline__ void mma16816(float *c, const unsigned *a, const unsigned *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// GELU(z) = z Phi(z) with the error function, and its derivative
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// Shared-memory copies of the BF16 weights: WT (out-major, in contiguous: the B
// operand of x W) and W (in-major, out contiguous: the B operand of dz W^T).
struct MlpSmem {
  bf16 w1t[MLP_H][MLP_IN + 8];   // +8: row padding against bank conflicts (16 B)
  bf16 w2t[MLP_H][MLP_H + 8];
  bf16 w3t[MLP_OUTP][MLP_H + 8];
  bf16 w2[MLP_H][MLP_H + 8];
  bf16 w3[MLP_H][16];             // W3 [64][8] with k (= out) padded to 16
  float b1[MLP_H], b2[MLP_H], b3[MLP_OUTP];
};

__device__ void load_weights(MlpSmem &s, const float *__restrict__ P, int tid, int nt) {
  for (int e = tid; e < MLP_IN * MLP_H; e += nt) {
    const int k = e / MLP_H, n = e % MLP_H;
    s.w1t[n][k] = __float2bfloat16_rn(P[MLP_OFF_W1 + e]);
  }
  for (int e = tid; e < MLP_H * MLP_H; e += nt) {
    const int k = e / MLP_H, n = e % MLP_H;
    const bf16 v = __float2bfloat16_rn(P[MLP_OFF_W2 + e]);
    s.w2t[n][k] = v;
    s.w2[k][n] = v;
  }
  for (int e = tid; e < MLP_H * 16; e += nt) {
    const int k = e / 16, n = e % 16;
    const float v = n < MLP_OUTP ? P[MLP_OFF_W3 + k * MLP_OUTP + n] : 0.0f;
    s.w3[k][n] = __float2bfloat16_rn(n < MLP_OUT ? v : 0.0f);
    if (n < MLP_OUTP) s.w3t[n][k] = __float2bfloat16_rn(n < MLP_OUT ? v : 0.0f);
  }
  for (int e = tid; e < MLP_H; e += nt) {
    s.b1[e] = P[MLP_OFF_B1 + e];
    s.b2[e] = P[MLP_OFF_B2 + e];
  }
  for (int e = tid; e < MLP_OUTP; e += nt) s.b3[e] = e < MLP_OUT ? P[MLP_OFF_B3 + e] : 0.0f;
}

// A fragment of rows r0.. (16) and columns k0.. (16) of a row-major BF16 matrix
// with ld columns; rows >= n read as zero
__device__ __forceinline__ void load_a(unsigned *a, const bf16 *__restrict__ M, int ld, int r0, int k0, int n,
                                       int g, int t) {
  const int ra = r0 + g, rb = r0 + g + 8;
  a[0] = ra < n ? ld_u32(M + (size_t)ra * ld + k0 + 2 * t) : 0u;
  a[1] = rb < n ? ld_u32(M + (size_t)rb * ld + k0 + 2 * t) : 0u;
  a[2] = ra < n ? ld_u32(M + (size_t)ra * ld + k0 + 2 * t + 8) : 0u;
  a[3] = rb < n ? ld_u32(M + (size_t)rb * ld + k0 + 2 * t + 8) : 0u;
}

// One warp's 16 rows through the three layers.  z1/z2 (may be null): the
// pre-activations, BF16 [n][64]; y: FP32 [n][2].
__device__ void mlp_rows(const MlpSmem &s, const bf16 *__restrict__ X, int n, int r0, float *__restrict__ y,
                         bf16 *__restrict__ z1, bf16 *__restrict__ z2, int lane) {
  const int g = lane >> 2, t = lane & 3;
  // layer 1: 16 x 128 . 128 x 64
  float c1[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) c1[nt][0] = c1[nt][1] = c1[nt][2] = c1[nt][3] = 0.0f;
#pragma unroll
  for (int kb = 0; kb < MLP_IN / 16; kb++) {
    unsigned a[4];
    load_a(a, X, MLP_IN, r0, kb * 16, n, g, t);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const unsigned b[2] = {ld_u32(&s.w1t[nt * 8 + g][kb * 16 + 2 * t]), ld_u32(&s.w1t[nt * 8 + g][kb * 16 + 2 * t + 8])};
      mma16816(c1[nt], a, b);
    }
  }
  // bias, keep z, GELU into the next layer's A fragments
  unsigned h1[4][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int col = nt * 8 + 2 * t;
    const float za = c1[nt][0] + s.b1[col], zb = c1[nt][1] + s.b1[col + 1];
    const float zc = c1[nt][2] + s.b1[col], zd = c1[nt][3] + s.b1[col + 1];
    const unsigned zab = pack2(za, zb), zcd = pack2(zc, zd);
    if (z1) {
      if (r0 + g < n) *reinterpret_cast<unsigned *>(z1 + (size_t)(r0 + g) * MLP_H + col) = zab;
      if (r0 + g + 8 < n) *reinterpret_cast<unsigned *>(z1 + (size_t)(r0 + g + 8) * MLP_H + col) = zcd;
    }
    // the activation from the BF16-rounded pre-activation (as the backward pass sees it)
    const float2 zr = unpack2(zab), zs = unpack2(zcd);
    const int kb = nt >> 1, hi = nt & 1;
    h1[kb][hi * 2 + 0] = pack2(gelu(zr.x), gelu(zr.y));
    h1[kb][hi * 2 + 1] = pack2(gelu(zs.x), gelu(zs.y));
  }
  // layer 2: 16 x 64 . 64 x 64
  float c2[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) c2[nt][0] = c2[nt][1] = c2[nt][2] = c2[nt][3] = 0.0f;
#pragma unroll
  for (int kb = 0; kb < 4; kb++) {
    // h1[kb] holds a0 a1 (first 8 columns) then a2 a3 (next 8) in the order
    // {c0c1 of tile 2kb, c2c3 of tile 2kb, c0c1 of tile 2kb+1, c2c3 of tile 2kb+1}
    const unsigned a[4] = {h1[kb][0], h1[kb][1], h1[kb][2], h1[kb][3]};
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const unsigned b[2] = {ld_u32(&s.w2t[nt * 8 + g][kb * 16 + 2 * t]), ld_u32(&s.w2t[nt * 8 + g][kb * 16 + 2 * t + 8])};
      mma16816(c2[nt], a, b);
    }
  }
  unsigned h2[4][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int col = nt * 8 + 2 * t;
    const float za = c2[nt][0] + s.b2[col], zb = c2[nt][1] + s.b2[col + 1];
    const float zc = c2[nt][2] + s.b2[col], zd = c2[nt][3] + s.b2[col + 1];
    const unsigned zab = pack2(za, zb), zcd = pack2(zc, zd);
    if (z2) {
      if (r0 + g < n) *reinterpret_cast<unsigned *>(z2 + (size_t)(r0 + g) * MLP_H + col) = zab;
      if (r0 + g + 8 < n) *reinterpret_cast<unsigned *>(z2 + (size_t)(r0 + g + 8) * MLP_H + col) = zcd;
    }
    const float2 zr = unpack2(zab), zs = unpack2(zcd);
    const int kb = nt >> 1, hi = nt & 1;
    h2[kb][hi * 2 + 0] = pack2(gelu(zr.x), gelu(zr.y));
    h2[kb][hi * 2 + 1] = pack2(gelu(zs.x), gelu(zs.y));
  }
  // layer 3: 16 x 64 . 64 x 8
  float c3[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int kb = 0; kb < 4; kb++) {
    const unsigned a[4] = {h2[kb][0], h2[kb][1], h2[kb][2], h2[kb][3]};
    const unsigned b[2] = {ld_u32(&s.w3t[g][kb * 16 + 2 * t]), ld_u32(&s.w3t[g][kb * 16 + 2 * t + 8])};
    mma16816(c3, a, b);
  }
  if (t == 0) {  // columns 0, 1
    if (r0 + g < n) {
      y[(size_t)(r0 + g) * MLP_OUT + 0] = c3[0] + s.b3[0];
      y[(size_t)(r0 + g) * MLP_OUT + 1] = c3[1] + s.b3[1];
    }
    if (r0 + g + 8 < n) {
      y[(size_t)(r0 + g + 8) * MLP_OUT + 0] = c3[2] + s.b3[0];
      y[(size_t)(r0 + g + 8) * MLP_OUT + 1] = c3[3] + s.b3[1];
    }
  }
}

__global__ void __launch_bounds__(128) k_mlp_forward(const float *__restrict__ P, const bf16 *__restrict__ X, int n,
                                                     float *__restrict__ y, bf16 *__restrict__ z1,
                                                     bf16 *__restrict__ z2) {
  extern __shared__ __align__(16) unsigned char mlp_raw[];
  MlpSmem &s = *reinterpret_cast<MlpSmem *>(mlp_raw);
  load_weights(s, P, threadIdx.x, blockDim.x);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = blockIdx.x * MLP_ROWS + w * 16;
  if (r0 < n) mlp_rows(s, X, n, r0, y, z1, z2, lane);
}

// Backward of one CTA's 64 rows.  dy: FP32 [n][2] (dL/dy).  Per CTA partial
// gradients (FP32, MLP_NPARAM) to part[blockIdx.x].
struct MlpBwdSmem {
  MlpSmem w;
  bf16 xt[MLP_IN][MLP_ROWS + 8];    // X^T of the tile
  bf16 h1t[MLP_H][MLP_ROWS + 8];    // GELU(z1)^T
  bf16 h2t[MLP_H][MLP_ROWS + 8];    // GELU(z2)^T
  bf16 dz1t[MLP_H][MLP_ROWS + 8];   // dL/dz1, transposed
  bf16 dz2t[MLP_H][MLP_ROWS + 8];
  bf16 dyt[MLP_OUTP][MLP_ROWS + 8]; // dL/dy, transposed, columns 2..7 zero
  float db1[4][MLP_H], db2[4][MLP_H], db3[4][MLP_OUTP];  // per-warp bias sums
};

__global__ void __launch_bounds__(128) k_mlp_backward(const float *__restrict__ P, const bf16 *__restrict__ X,
                                                      const bf16 *__restrict__ z1, const bf16 *__restrict__ z2,
                                                      const float *__restrict__ dy, int n, float *__restrict__ part) {
  extern __shared__ __align__(16) unsigned char mlp_raw[];
  MlpBwdSmem &s = *reinterpret_cast<MlpBwdSmem *>(mlp_raw);
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int R0 = blockIdx.x * MLP_ROWS;
  load_weights(s.w, P, tid, blockDim.x);
  // stage X^T, GELU(z)^T and dy^T of the tile (rows >= n as zeros)
  for (int e = tid; e < MLP_ROWS * MLP_IN; e += blockDim.x) {
    const int r = e / MLP_IN, k = e % MLP_IN;
    s.xt[k][r] = R0 + r < n ? X[(size_t)(R0 + r) * MLP_IN + k] : __float2bfloat16_rn(0.0f);
  }
  for (int e = tid; e < MLP_ROWS * MLP_H; e += blockDim.x) {
    const int r = e / MLP_H, k = e % MLP_H;
    const bool in = R0 + r < n;
    s.h1t[k][r] = __float2bfloat16_rn(in ? gelu(__bfloat162float(z1[(size_t)(R0 + r) * MLP_H + k])) : 0.0f);
    s.h2t[k][r] = __float2bfloat16_rn(in ? gelu(__bfloat162float(z2[(size_t)(R0 + r) * MLP_H + k])) : 0.0f);
  }
  for (int e = tid; e < MLP_ROWS * MLP_OUTP; e += blockDim.x) {
    const int r = e / MLP_OUTP, k = e % MLP_OUTP;
    s.dyt[k][r] = __float2bfloat16_rn(R0 + r < n && k < MLP_OUT ? dy[(size_t)(R0 + r) * MLP_OUT + k] : 0.0f);
  }
  __syncthreads();
  // data gradients of this warp's 16 rows: dh2 = dy W3^T, dz2, dh1 = dz2 W2^T, dz1
  const int r0 = w * 16;  // row within the tile
  {
    // A = dy (16 x 16, columns >= 8 zero): from dyt
    unsigned a[4];
    {
      const int ra = r0 + g, rb = r0 + g + 8;
      const float2 v0 = {__bfloat162float(s.dyt[2 * t][ra]), __bfloat162float(s.dyt[2 * t + 1][ra])};
      const float2 v1 = {__bfloat162float(s.dyt[2 * t][rb]), __bfloat162float(s.dyt[2 * t + 1][rb])};
      a[0] = pack2(v0.x, v0.y);
      a[1] = pack2(v1.x, v1.y);
      a[2] = 0u;  // columns 8..15
      a[3] = 0u;
    }
    float c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
      // B(k = out, n = hidden) = W3[n][k]: w3[n][k], k contiguous
      const unsigned b[2] = {ld_u32(&s.w.w3[nt * 8 + g][2 * t]), ld_u32(&s.w.w3[nt * 8 + g][2 * t + 8])};
      mma16816(c[nt], a, b);
    }
    float db2p[8][2];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int col = nt * 8 + 2 * t, ra = r0 + g, rb = r0 + g + 8;
      const bool ina = R0 + ra < n, inb = R0 + rb < n;
      const float za0 = ina ? __bfloat162float(z2[(size_t)(R0 + ra) * MLP_H + col]) : 0.0f;
      const float za1 = ina ? __bfloat162float(z2[(size_t)(R0 + ra) * MLP_H + col + 1]) : 0.0f;
      const float zb0 = inb ? __bfloat162float(z2[(size_t)(R0 + rb) * MLP_H + col]) : 0.0f;
      const float zb1 = inb ? __bfloat162float(z2[(size_t)(R0 + rb) * MLP_H + col + 1]) : 0.0f;
      const float d00 = c[nt][0] * gelu_d(za0), d01 = c[nt][1] * gelu_d(za1);
      const float d10 = c[nt][2] * gelu_d(zb0), d11 = c[nt][3] * gelu_d(zb1);
      const float2 q0 = unpack2(pack2(d00, d01)), q1 = unpack2(pack2(d10, d11));
      s.dz2t[col][ra] = __float2bfloat16_rn(q0.x);
      s.dz2t[col + 1][ra] = __float2bfloat16_rn(q0.y);
      s.dz2t[col][rb] = __float2bfloat16_rn(q1.x);
      s.dz2t[col + 1][rb] = __float2bfloat16_rn(q1.y);
      db2p[nt][0] = q0.x + q1.x;
      db2p[nt][1] = q0.y + q1.y;
    }
    // bias gradient db2: sum over the 16 rows (8 groups g per column pair)
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        float v = db2p[nt][h];
        for (int o = 4; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (g == 0) s.db2[w][nt * 8 + 2 * t + h] = v;
      }
  }
  __syncwarp();
  {
    // dh1 = dz2 W2^T: A = dz2 (16 x 64) from dz2t, B(k = out, n = in) = W2[n][k]
    float c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
    for (int kb = 0; kb < 4; kb++) {
      const int ra = r0 + g, rb = r0 + g + 8, k = kb * 16 + 2 * t;
      unsigned a[4];
      a[0] = pack2(__bfloat162float(s.dz2t[k][ra]), __bfloat162float(s.dz2t[k + 1][ra]));
      a[1] = pack2(__bfloat162float(s.dz2t[k][rb]), __bfloat162float(s.dz2t[k + 1][rb]));
      a[2] = pack2(__bfloat162float(s.dz2t[k + 8][ra]), __bfloat162float(s.dz2t[k + 9][ra]));
      a[3] = pack2(__bfloat162float(s.dz2t[k + 8][rb]), __bfloat162float(s.dz2t[k + 9][rb]));
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const unsigned b[2] = {ld_u32(&s.w.w2[nt * 8 + g][kb * 16 + 2 * t]), ld_u32(&s.w.w2[nt * 8 + g][kb * 16 + 2 * t + 8])};
        mma16816(c[nt], a, b);
      }
    }
    float db1p[8][2];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int col = nt * 8 + 2 * t, ra = r0 + g, rb = r0 + g + 8;
      const bool ina = R0 + ra < n, inb = R0 + rb < n;
      const float za0 = ina ? __bfloat162float(z1[(size_t)(R0 + ra) * MLP_H + col]) : 0.0f;
      const float za1 = ina ? __bfloat162float(z1[(size_t)(R0 + ra) * MLP_H + col + 1]) : 0.0f;
      const float zb0 = inb ? __bfloat162float(z1[(size_t)(R0 + rb) * MLP_H + col]) : 0.0f;
      const float zb1 = inb ? __bfloat162float(z1[(size_t)(R0 + rb) * MLP_H + col + 1]) : 0.0f;
      const float d00 = c[nt][0] * gelu_d(za0), d01 = c[nt][1] * gelu_d(za1);
      const float d10 = c[nt][2] * gelu_d(zb0), d11 = c[nt][3] * gelu_d(zb1);
      const float2 q0 = unpack2(pack2(d00, d01)), q1 = unpack2(pack2(d10, d11));
      s.dz1t[col][ra] = __float2bfloat16_rn(q0.x);
      s.dz1t[col + 1][ra] = __float2bfloat16_rn(q0.y);
      s.dz1t[col][rb] = __float2bfloat16_rn(q1.x);
      s.dz1t[col + 1][rb] = __float2bfloat16_rn(q1.y);
      db1p[nt][0] = q0.x + q1.x;
      db1p[nt][1] = q0.y + q1.y;
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        float v = db1p[nt][h];
        for (int o = 4; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (g == 0) s.db1[w][nt * 8 + 2 * t + h] = v;
      }
    // db3: sum of dy over the warp's rows (lanes t == 0 hold rows g and g + 8)
    float d3[2] = {0.0f, 0.0f};
    if (t == 0) {
      const int ra = r0 + g, rb = r0 + g + 8;
      d3[0] = __bfloat162float(s.dyt[0][ra]) + __bfloat162float(s.dyt[0][rb]);
      d3[1] = __bfloat162float(s.dyt[1][ra]) + __bfloat162float(s.dyt[1][rb]);
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float v = d3[h];
      for (int o = 1; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) s.db3[w][h] = v;
    }
    if (lane < MLP_OUTP - MLP_OUT) s.db3[w][MLP_OUT + lane] = 0.0f;
  }
  __syncthreads();
  // weight gradients of the tile: dW = M^T dZ with M^T, dZ^T staged (k = tile rows)
  float *out = part + (size_t)blockIdx.x * MLP_NPARAM;
  // dW1 [128][64] = X^T dz1: 8 m-tiles x 8 n-tiles; warp w takes m-tiles 2w, 2w+1
#pragma unroll
  for (int mi = 0; mi < 2; mi++) {
    const int m0 = (2 * w + mi) * 16;
    float c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
    for (int kb = 0; kb < MLP_ROWS / 16; kb++) {
      const int k = kb * 16 + 2 * t;
      const unsigned a[4] = {ld_u32(&s.xt[m0 + g][k]), ld_u32(&s.xt[m0 + g + 8][k]), ld_u32(&s.xt[m0 + g][k + 8]),
                             ld_u32(&s.xt[m0 + g + 8][k + 8])};
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const unsigned b[2] = {ld_u32(&s.dz1t[nt * 8 + g][k]), ld_u32(&s.dz1t[nt * 8 + g][k + 8])};
        mma16816(c[nt], a, b);
      }
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int col = nt * 8 + 2 * t;
      out[MLP_OFF_W1 + (m0 + g) * MLP_H + col] = c[nt][0];
      out[MLP_OFF_W1 + (m0 + g) * MLP_H + col + 1] = c[nt][1];
      out[MLP_OFF_W1 + (m0 + g + 8) * MLP_H + col] = c[nt][2];
      out[MLP_OFF_W1 + (m0 + g + 8) * MLP_H + col + 1] = c[nt][3];
    }
  }
  // dW2 [64][64] = h1^T dz2 and dW3 [64][8] = h2^T dy: warp w takes m-tile w
  {
    const int m0 = w * 16;
    float c[8][4], c3[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
    for (int kb = 0; kb < MLP_ROWS / 16; kb++) {
      const int k = kb * 16 + 2 * t;
      const unsigned a[4] = {ld_u32(&s.h1t[m0 + g][k]), ld_u32(&s.h1t[m0 + g + 8][k]), ld_u32(&s.h1t[m0 + g][k + 8]),
                             ld_u32(&s.h1t[m0 + g + 8][k + 8])};
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const unsigned b[2] = {ld_u32(&s.dz2t[nt * 8 + g][k]), ld_u32(&s.dz2t[nt * 8 + g][k + 8])};
        mma16816(c[nt], a, b);
      }
      const unsigned a3[4] = {ld_u32(&s.h2t[m0 + g][k]), ld_u32(&s.h2t[m0 + g + 8][k]), ld_u32(&s.h2t[m0 + g][k + 8]),
                              ld_u32(&s.h2t[m0 + g + 8][k + 8])};
      const unsigned b3[2] = {ld_u32(&s.dyt[g][k]), ld_u32(&s.dyt[g][k + 8])};
      mma16816(c3, a3, b3);
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int col = nt * 8 + 2 * t;
      out[MLP_OFF_W2 + (m0 + g) * MLP_H + col] = c[nt][0];
      out[MLP_OFF_W2 + (m0 + g) * MLP_H + col + 1] = c[nt][1];
      out[MLP_OFF_W2 + (m0 + g + 8) * MLP_H + col] = c[nt][2];
      out[MLP_OFF_W2 + (m0 + g + 8) * MLP_H + col + 1] = c[nt][3];
    }
    const int col = 2 * t;
    out[MLP_OFF_W3 + (m0 + g) * MLP_OUTP + col] = col < MLP_OUT ? c3[0] : 0.0f;
    out[MLP_OFF_W3 + (m0 + g) * MLP_OUTP + col + 1] = col + 1 < MLP_OUT ? c3[1] : 0.0f;
    out[MLP_OFF_W3 + (m0 + g + 8) * MLP_OUTP + col] = col < MLP_OUT ? c3[2] : 0.0f;
    out[MLP_OFF_W3 + (m0 + g + 8) * MLP_OUTP + col + 1] = col + 1 < MLP_OUT ? c3[3] : 0.0f;
  }
  // bias partials: the four warps' sums in a fixed order
  for (int e = tid; e < MLP_H; e += blockDim.x) {
    out[MLP_OFF_B1 + e] = ((s.db1[0][e] + s.db1[1][e]) + s.db1[2][e]) + s.db1[3][e];
    out[MLP_OFF_B2 + e] = ((s.db2[0][e] + s.db2[1][e]) + s.db2[2][e]) + s.db2[3][e];
  }
  for (int e = tid; e < MLP_OUTP; e += blockDim.x)
    out[MLP_OFF_B3 + e] = ((s.db3[0][e] + s.db3[1][e]) + s.db3[2][e]) + s.db3[3][e];
}

// grad[p] = sum over CTAs c of part[c][p], in CTA order (deterministic)
__global__ void k_mlp_reduce(const float *__restrict__ part, int nparts, float *__restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_NPARAM) return;
  double acc = 0.0;
  for (int c = 0; c < nparts; c++) acc += (double)part[(size_t)c * MLP_NPARAM + p];
  grad[p] = (float)acc;
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; the padded columns of the
// last layer stay zero
__global__ void k_mlp_adam(float *__restrict__ P, const float *__restrict__ grad, float *__restrict__ m1,
                           float *__restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_NPARAM) return;
  const bool pad = (p >= MLP_OFF_W3 && p < MLP_OFF_B3 && (p - MLP_OFF_W3) % MLP_OUTP >= MLP_OUT) ||
                   (p >= MLP_OFF_B3 && p - MLP_OFF_B3 >= MLP_OUT);
  if (pad) {
    P[p] = 0.0f;
    return;
  }
  const float gr = grad[p];
  const float a = b1 * m1[p] + (1.0f - b1) * gr;
  const float v = b2 * m2[p] + (1.0f - b2) * gr * gr;
  m1[p] = a;
  m2[p] = v;
  P[p] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

}  // namespace

struct fargo_mlp {
  int cap = 0;           // rows the workspace holds
  float *P = nullptr;    // FP32 master parameters
  float *grad = nullptr;
  float *m1 = nullptr, *m2 = nullptr;
  bf16 *z1 = nullptr, *z2 = nullptr;
  float *part = nullptr;
  int steps = 0;
};

static size_t fwd_smem() { return sizeof(MlpSmem); }
static size_t bwd_smem() { return sizeof(MlpBwdSmem); }

extern "C" {

int fargo_mlp_create(int max_rows, fargo_mlp **out) {
  if (!out || max_rows <= 0) return FARGO_ERR_INVALID;
  *out = nullptr;
  fargo_mlp *m = new fargo_mlp();
  m->cap = max_rows;
  const size_t nblk = (size_t)(max_rows + MLP_ROWS - 1) / MLP_ROWS;
  cudaError_t e = cudaMalloc(&m->P, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->grad, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->m1, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->m2, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->z1, (size_t)max_rows * MLP_H * 2);
  if (e == cudaSuccess) e = cudaMalloc(&m->z2, (size_t)max_rows * MLP_H * 2);
  if (e == cudaSuccess) e = cudaMalloc(&m->part, nblk * MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMemset(m->P, 0, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMemset(m->m1, 0, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMemset(m->m2, 0, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem());
  if (e != cudaSuccess) {
    fargo_mlp_destroy(m);
    return FARGO_ERR_CUDA;
  }
  *out = m;
  return FARGO_OK;
}

void fargo_mlp_destroy(fargo_mlp *m) {
  if (!m) return;
  for (void *p : {(void *)m->P, (void *)m->grad, (void *)m->m1, (void *)m->m2, (void *)m->z1, (void *)m->z2,
                  (void *)m->part})
    if (p) cudaFree(p);
  delete m;
}

int fargo_mlp_set_params(fargo_mlp *m, const float *host) {
  if (!m || !host) return FARGO_ERR_INVALID;
  if (cudaMemcpy(m->P, host, MLP_NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess) return FARGO_ERR_CUDA;
  m->steps = 0;
  if (cudaMemset(m->m1, 0, MLP_NPARAM * 4) != cudaSuccess || cudaMemset(m->m2, 0, MLP_NPARAM * 4) != cudaSuccess)
    return FARGO_ERR_CUDA;
  return FARGO_OK;
}

int fargo_mlp_get_params(fargo_mlp *m, float *host) {
  if (!m || !host) return FARGO_ERR_INVALID;
  return cudaMemcpy(host, m->P, MLP_NPARAM * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

int fargo_mlp_get_grad(fargo_mlp *m, float *host) {
  if (!m || !host) return FARGO_ERR_INVALID;
  return cudaMemcpy(host, m->grad, MLP_NPARAM * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? FARGO_OK
                                                                                          : FARGO_ERR_CUDA;
}

int fargo_mlp_forward(fargo_mlp *m, const void *x, int n, float *y, int train, void *stream) {
  if (!m || !x || !y || n <= 0 || n > m->cap) return FARGO_ERR_INVALID;
  const cudaStream_t s = (cudaStream_t)stream;
  k_mlp_forward<<<(n + MLP_ROWS - 1) / MLP_ROWS, 128, fwd_smem(), s>>>(
      m->P, (const bf16 *)x, n, y, train ? m->z1 : nullptr, train ? m->z2 : nullptr);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

int fargo_mlp_backward(fargo_mlp *m, const void *x, int n, const float *dy, void *stream) {
  if (!m || !x || !dy || n <= 0 || n > m->cap) return FARGO_ERR_INVALID;
  const cudaStream_t s = (cudaStream_t)stream;
  const int nb = (n + MLP_ROWS - 1) / MLP_ROWS;
  k_mlp_backward<<<nb, 128, bwd_smem(), s>>>(m->P, (const bf16 *)x, m->z1, m->z2, dy, n, m->part);
  k_mlp_reduce<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(m->part, nb, m->grad);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

int fargo_mlp_adam(fargo_mlp *m, float lr, void *stream) {
  if (!m || !(lr > 0.0f)) return FARGO_ERR_INVALID;
  m->steps += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, (float)m->steps), c2 = 1.0f - powf(b2, (float)m->steps);
  k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, (cudaStream_t)stream>>>(m->P, m->grad, m->m1, m->m2, lr, b1, b2,
                                                                          1e-8f, c1, c2);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

}  // extern "C"
