// fargo_mlp.cu -- the stencil MLP of the learned coarse-grid correction.
//
// Network (per coarse cell): 128 inputs (a 5x5 stencil of 5 channels, padded
// with 3 zeros) -> 64 (GELU) -> 64 (GELU) -> 2 outputs (the radial and azimuthal
// mass-flux corrections of the cell).  BF16 weights and activations, FP32
// accumulation, on the tensor cores with mma.sync m16n8k16: the layers are
// K = 64..128 by N = 64, one warp holds a 16-row tile and keeps every activation
// in registers between the layers, so the contraction never leaves the SM.
//
// Both passes are persistent: a CTA stages the BF16 weights in shared memory once
// and then loops over row tiles.  Forward: every warp streams its own 16-row tiles
// of X through a double-buffered cp.async ring and ldmatrix.  Backward: a CTA
// takes 64-row tiles; each warp recomputes the forward pass of its 16 rows in
// registers (no pre-activations are stored between the passes), forms the data
// gradients dz2, dz1 with the same fragments, and leaves X, GELU(z1), GELU(z2),
// dz1, dz2, dy row-major in shared memory; the weight gradients dW = M^T dZ of the
// tile are then mma's over the 64 rows with both operands read transposed by
// ldmatrix.trans, accumulated in registers over all the CTA's tiles.  One FP32
// partial per CTA, a fixed-order FP64 reduction over the CTAs (deterministic for
// a given grid) and Adam on FP32 master weights follow.
//
// Fragment layouts of mma.m16n8k16 (.row.col, BF16 in, FP32 out; g = lane / 4,
// t = lane % 4): A 16x16 row-major: a0 (g, 2t..2t+1), a1 (g+8, 2t..), a2 (g, 2t+8..),
// a3 (g+8, 2t+8..); B 16x8 column-major: b0 (k 2t..2t+1, n g), b1 (k 2t+8.., n g);
// C 16x8: c0,c1 (g, 2t..2t+1), c2,c3 (g+8, 2t..2t+1).  The C tiles of two adjacent
// 8-column blocks are exactly the A fragment of the next layer's 16-wide k block.
// ldmatrix (x4) hands lane (g, t) the elements (g, 2t..2t+1) of four 8x8 blocks
// whose rows lanes 8q..8q+7 address; with .trans the elements (2t..2t+1, g).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "fargo_gb300.h"
#include "fargo_tc.cuh"

#define MLP_IN 128
#define MLP_H 64
#define MLP_OUT 2
#define MLP_OUTP 8      // output columns of the last mma (the 2 outputs, zero-padded)
#define MLP_ROWS 64     // rows of a backward tile: 4 warps x 16
#define MLP_LDX (MLP_IN + 8)  // shared row strides (BF16): rows 16-byte aligned, and
#define MLP_LDH (MLP_H + 8)   // 8 consecutive rows fall in distinct bank groups
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
__device__ __forceinline__ void st_u32(bf16 *p, unsigned v) { *reinterpret_cast<unsigned *>(p) = v; }

__device__ __forceinline__ void mma16816(float *c, const unsigned *a, const unsigned *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(unsigned *r, const bf16 *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_addr(p))
               : "memory");
}
__device__ __forceinline__ void ldsm_x4_t(unsigned *r, const bf16 *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_addr(p))
               : "memory");
}
__device__ __forceinline__ void ldsm_x2_t(unsigned *r, const bf16 *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(smem_addr(p))
               : "memory");
}

// 16 bytes global -> shared, zero-filled when !valid (nothing is read then)
__device__ __forceinline__ void cp_async16(bf16 *dst, const bf16 *src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(dst)), "l"(src),
               "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// GELU in its tanh form (Hendrycks & Gimpel 2016), z (1 + tanh u) / 2 with
// u = sqrt(2/pi) (z + 0.044715 z^3), written as z sigma(2u); and its derivative
// sigma + z sigma (1 - sigma) d(2u)/dz.  Two SFU operations per value.
__device__ __forceinline__ float gelu_sig(float z) {
  const float u2 = z * fmaf(0.0713548162726f * z, z, 1.5957691216057308f);
  return __fdividef(1.0f, 1.0f + __expf(-u2));
}
__device__ __forceinline__ float gelu(float z) { return z * gelu_sig(z); }
__device__ __forceinline__ float gelu_d(float z) {
  const float s = gelu_sig(z);
  return fmaf(z * s * (1.0f - s), fmaf(0.2140644488178f * z, z, 1.5957691216057308f), s);
}

// Shared-memory copies of the BF16 weights: WT (out-major, in contiguous: the B
// operand of x W) for the forward pass; W (in-major, out contiguous: the B
// operand of dz W^T) for the backward pass.
struct MlpFwdW {
  bf16 w1t[MLP_H][MLP_LDX];
  bf16 w2t[MLP_H][MLP_LDH];
  bf16 w3t[MLP_OUTP][MLP_LDH];
  float b1[MLP_H], b2[MLP_H], b3[MLP_OUTP];
};
struct MlpBwdW {
  bf16 w2[MLP_H][MLP_LDH];
  bf16 w3[MLP_H][24];  // W3 [64][8], k (= out) zero-padded to 16; rows of 48 bytes
};

__device__ void load_fwd_weights(MlpFwdW &s, const float *__restrict__ P, int tid, int nt) {
  for (int e = tid; e < MLP_IN * MLP_H; e += nt) {
    const int k = e / MLP_H, n = e % MLP_H;
    s.w1t[n][k] = __float2bfloat16_rn(P[MLP_OFF_W1 + e]);
  }
  for (int e = tid; e < MLP_H * MLP_H; e += nt) {
    const int k = e / MLP_H, n = e % MLP_H;
    s.w2t[n][k] = __float2bfloat16_rn(P[MLP_OFF_W2 + e]);
  }
  for (int e = tid; e < MLP_H * MLP_OUTP; e += nt) {
    const int k = e / MLP_OUTP, n = e % MLP_OUTP;
    s.w3t[n][k] = __float2bfloat16_rn(n < MLP_OUT ? P[MLP_OFF_W3 + e] : 0.0f);
  }
  for (int e = tid; e < MLP_H; e += nt) {
    s.b1[e] = P[MLP_OFF_B1 + e];
    s.b2[e] = P[MLP_OFF_B2 + e];
  }
  for (int e = tid; e < MLP_OUTP; e += nt) s.b3[e] = e < MLP_OUT ? P[MLP_OFF_B3 + e] : 0.0f;
}

__device__ void load_bwd_weights(MlpBwdW &s, const float *__restrict__ P, int tid, int nt) {
  for (int e = tid; e < MLP_H * MLP_H; e += nt) {
    const int k = e / MLP_H, n = e % MLP_H;
    s.w2[k][n] = __float2bfloat16_rn(P[MLP_OFF_W2 + e]);
  }
  for (int e = tid; e < MLP_H * 24; e += nt) {
    const int k = e / 24, n = e % 24;
    s.w3[k][n] = __float2bfloat16_rn(n < MLP_OUT ? P[MLP_OFF_W3 + k * MLP_OUTP + n] : 0.0f);
  }
}

// 16 rows of X (row r0..) into a shared [16][MLP_LDX] buffer by one warp; rows
// >= n as zeros
__device__ __forceinline__ void stage_rows16(bf16 *buf, const bf16 *__restrict__ X, int r0, int n, int lane) {
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int c = lane + 32 * i, row = c >> 4, col = (c & 15) * 8;
    const bool valid = r0 + row < n;
    cp_async16(buf + row * MLP_LDX + col, X + (size_t)(valid ? r0 + row : 0) * MLP_IN + col, valid);
  }
}

// Layers 1 and 2 of one warp's 16 rows, A fragments of X by ldmatrix from xs
// (16 rows, stride MLP_LDX).  Out: z1p/z2p, the BF16 pre-activations in C layout
// (rows g, g+8 of column pair 2t of tile nt), and h2 (GELU(z2)) as the A
// fragments of the next k blocks; GELU(z1) and GELU(z2) also stored row-major to
// h1s/h2s (stride MLP_LDH) when those are given.  LDSM_B: B fragments by ldmatrix
// (fewer instructions) or by 32-bit loads (fewer live registers: the backward pass).
template <bool LDSM_B>
__device__ __forceinline__ void layers12(const MlpFwdW &s, const bf16 *xs, int lane, unsigned (&z1p)[8][2],
                                         unsigned (&z2p)[8][2], unsigned (&h2)[4][4], bf16 *h1s, bf16 *h2s) {
  const int g = lane >> 2, t = lane & 3, q = lane >> 3, rr = lane & 7;
  const bf16 *arow = xs + (rr + 8 * (q & 1)) * MLP_LDX + 8 * (q >> 1);
  // B from WT[n][k]: blocks (n0, k0), (n0, k0+8), (n0+8, k0), (n0+8, k0+8)
  const int brow = rr + 8 * (q >> 1), bcol = 8 * (q & 1);
  float c[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
  for (int kb = 0; kb < MLP_IN / 16; kb++) {
    unsigned a[4];
    ldsm_x4(a, arow + kb * 16);
    if (LDSM_B) {
#pragma unroll
      for (int np = 0; np < 4; np++) {  // B fragments of n-tiles 2np, 2np+1
        unsigned b[4];
        ldsm_x4(b, &s.w1t[np * 16 + brow][kb * 16 + bcol]);
        mma16816(c[2 * np], a, &b[0]);
        mma16816(c[2 * np + 1], a, &b[2]);
      }
    } else {
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const unsigned b[2] = {ld_u32(&s.w1t[nt * 8 + g][kb * 16 + 2 * t]), ld_u32(&s.w1t[nt * 8 + g][kb * 16 + 2 * t + 8])};
        mma16816(c[nt], a, b);
      }
    }
  }
  // bias, keep z, GELU (of the BF16-rounded z, as the backward pass sees it)
  // into the next layer's A fragments: h[kb] = {tile 2kb rows g, g+8; tile 2kb+1 rows g, g+8}
  unsigned h1[4][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int col = nt * 8 + 2 * t;
    z1p[nt][0] = pack2(c[nt][0] + s.b1[col], c[nt][1] + s.b1[col + 1]);
    z1p[nt][1] = pack2(c[nt][2] + s.b1[col], c[nt][3] + s.b1[col + 1]);
    const float2 zr = unpack2(z1p[nt][0]), zs = unpack2(z1p[nt][1]);
    const unsigned ha = pack2(gelu(zr.x), gelu(zr.y)), hb = pack2(gelu(zs.x), gelu(zs.y));
    h1[nt >> 1][(nt & 1) * 2 + 0] = ha;
    h1[nt >> 1][(nt & 1) * 2 + 1] = hb;
    if (h1s) {
      st_u32(h1s + g * MLP_LDH + col, ha);
      st_u32(h1s + (g + 8) * MLP_LDH + col, hb);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
  for (int kb = 0; kb < 4; kb++) {
    if (LDSM_B) {
#pragma unroll
      for (int np = 0; np < 4; np++) {
        unsigned b[4];
        ldsm_x4(b, &s.w2t[np * 16 + brow][kb * 16 + bcol]);
        mma16816(c[2 * np], h1[kb], &b[0]);
        mma16816(c[2 * np + 1], h1[kb], &b[2]);
      }
    } else {
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const unsigned b[2] = {ld_u32(&s.w2t[nt * 8 + g][kb * 16 + 2 * t]), ld_u32(&s.w2t[nt * 8 + g][kb * 16 + 2 * t + 8])};
        mma16816(c[nt], h1[kb], b);
      }
    }
  }
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int col = nt * 8 + 2 * t;
    z2p[nt][0] = pack2(c[nt][0] + s.b2[col], c[nt][1] + s.b2[col + 1]);
    z2p[nt][1] = pack2(c[nt][2] + s.b2[col], c[nt][3] + s.b2[col + 1]);
    const float2 zr = unpack2(z2p[nt][0]), zs = unpack2(z2p[nt][1]);
    const unsigned ha = pack2(gelu(zr.x), gelu(zr.y)), hb = pack2(gelu(zs.x), gelu(zs.y));
    h2[nt >> 1][(nt & 1) * 2 + 0] = ha;
    h2[nt >> 1][(nt & 1) * 2 + 1] = hb;
    if (h2s) {
      st_u32(h2s + g * MLP_LDH + col, ha);
      st_u32(h2s + (g + 8) * MLP_LDH + col, hb);
    }
  }
}

struct MlpFwdSmem {
  MlpFwdW w;
  bf16 xb[4][2][16][MLP_LDX];  // per warp: a double-buffered 16-row tile of X
};

__global__ void __launch_bounds__(128) k_mlp_forward(const float *__restrict__ P, const bf16 *__restrict__ X, int n,
                                                     float *__restrict__ y) {
  extern __shared__ __align__(16) unsigned char mlp_raw[];
  MlpFwdSmem &s = *reinterpret_cast<MlpFwdSmem *>(mlp_raw);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int ntile = (n + 15) / 16, stride = gridDim.x * 4;
  int tile = blockIdx.x * 4 + w;
  if (tile < ntile) stage_rows16(&s.xb[w][0][0][0], X, tile * 16, n, lane);
  cp_async_commit();
  load_fwd_weights(s.w, P, threadIdx.x, blockDim.x);
  __syncthreads();
  for (int buf = 0; tile < ntile; tile += stride, buf ^= 1) {
    if (tile + stride < ntile) stage_rows16(&s.xb[w][buf ^ 1][0][0], X, (tile + stride) * 16, n, lane);
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    unsigned z1p[8][2], z2p[8][2], h2[4][4];
    layers12<true>(s.w, &s.xb[w][buf][0][0], lane, z1p, z2p, h2, nullptr, nullptr);
    // layer 3: 16 x 64 . 64 x 8
    float c3[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int kp = 0; kp < 2; kp++) {  // B fragments of k blocks 2kp, 2kp+1
      unsigned b[4];
      ldsm_x4(b, &s.w.w3t[lane & 7][kp * 32 + 8 * (lane >> 3)]);
      mma16816(c3, h2[2 * kp], &b[0]);
      mma16816(c3, h2[2 * kp + 1], &b[2]);
    }
    const int r0 = tile * 16;
    if (t == 0) {  // columns 0, 1
      if (r0 + g < n)
        *reinterpret_cast<float2 *>(y + (size_t)(r0 + g) * MLP_OUT) = make_float2(c3[0] + s.w.b3[0], c3[1] + s.w.b3[1]);
      if (r0 + g + 8 < n)
        *reinterpret_cast<float2 *>(y + (size_t)(r0 + g + 8) * MLP_OUT) =
            make_float2(c3[2] + s.w.b3[0], c3[3] + s.w.b3[1]);
    }
    __syncwarp();  // the buffer is refilled two tiles on
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// Forward on the 5th-generation tensor cores (tcgen05): a persistent CTA of eight
// warps takes 128-row tiles.  Per tile, one thread issues each layer's MMAs
// (M = 128 rows, N = 64, 64, 16; K = 128, 64, 64 in steps of 16) with BF16
// operands in shared memory and the FP32 accumulators in tensor memory.  Row m of
// an accumulator is read (tcgen05.ld) by the two warps of lane quarter m / 32,
// one per half of the columns; each adds the bias, rounds z to BF16, applies GELU
// and writes BF16 h into shared memory as the next layer's A operand -- the same
// arithmetic per value as the mma.sync kernel.  The next tile's X streams in by
// cp.async as soon as the current tile's first layer has read its buffer, behind
// the two hidden-layer epilogues.  Three CTAs fit an SM (74 KB of shared memory,
// 128 tensor-memory columns each).
//
// Shared-memory operands use the no-swizzle K-major layout of fargo_tc.cuh with
// the rows of a K chunk packed together: element (r, k) of an R-row operand at
// (k / 8) * (R * 16) + r * 16 + (k % 8) * 2, i.e. LBO = R * 16 (along K) and
// SBO = 128 (8-row groups), so that consecutive threads (rows) write consecutive
// 16-byte slots (no bank conflicts).
#define TCF_ROWS 128
#define TCF_THREADS 256
#define TCF_X_BYTES (TCF_ROWS * MLP_IN * 2)       // 32 KB
#define TCF_W1_BYTES (MLP_H * MLP_IN * 2)         // 16 KB
#define TCF_W2_BYTES (MLP_H * MLP_H * 2)          // 8 KB
#define TCF_N3 16                                 // the last layer's N (the 2 outputs, zero-padded)
#define TCF_W3_BYTES (TCF_N3 * MLP_H * 2)         // 2 KB
#define TCF_H_BYTES (TCF_ROWS * MLP_H * 2)        // 16 KB
#define TCF_SMEM (TCF_X_BYTES + TCF_W1_BYTES + TCF_W2_BYTES + TCF_W3_BYTES + TCF_H_BYTES)
#define TCF_TMEM_COLS 128                         // layers 1 and 2 at columns 0..63, layer 3 at 64..79

__device__ __forceinline__ uint32_t tcf_off(int r, int k, int rows) {
  return (uint32_t)(k >> 3) * (uint32_t)(rows * 16) + (uint32_t)r * 16u + (uint32_t)(k & 7) * 2u;
}

__global__ void __launch_bounds__(TCF_THREADS) k_mlp_forward_tc(const float *__restrict__ P,
                                                                const bf16 *__restrict__ X, int n,
                                                                float *__restrict__ y, int *err) {
  extern __shared__ __align__(128) unsigned char tcf_raw[];
  __shared__ uint32_t tslot;
  __shared__ __align__(8) uint64_t bar;
  __shared__ float b1[MLP_H], b2[MLP_H], b3[2];
  unsigned char *xs = tcf_raw, *w1 = xs + TCF_X_BYTES, *w2 = w1 + TCF_W1_BYTES, *w3 = w2 + TCF_W2_BYTES;
  unsigned char *hs = w3 + TCF_W3_BYTES;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, half = warp >> 2, m = 32 * quarter + lane;  // accumulator row and column half
  const int ntile = (n + TCF_ROWS - 1) / TCF_ROWS;
  // the weights as B operands (N rows = outputs, K = inputs), BF16
  for (int e = tid; e < MLP_IN * MLP_H; e += blockDim.x) {
    const int k = e / MLP_H, o = e % MLP_H;
    *reinterpret_cast<bf16 *>(w1 + tcf_off(o, k, MLP_H)) = __float2bfloat16_rn(P[MLP_OFF_W1 + e]);
  }
  for (int e = tid; e < MLP_H * MLP_H; e += blockDim.x) {
    const int k = e / MLP_H, o = e % MLP_H;
    *reinterpret_cast<bf16 *>(w2 + tcf_off(o, k, MLP_H)) = __float2bfloat16_rn(P[MLP_OFF_W2 + e]);
  }
  for (int e = tid; e < MLP_H * TCF_N3; e += blockDim.x) {
    const int k = e / TCF_N3, o = e % TCF_N3;
    *reinterpret_cast<bf16 *>(w3 + tcf_off(o, k, TCF_N3)) =
        __float2bfloat16_rn(o < MLP_OUT ? P[MLP_OFF_W3 + k * MLP_OUTP + o] : 0.0f);
  }
  for (int e = tid; e < MLP_H; e += blockDim.x) {
    b1[e] = P[MLP_OFF_B1 + e];
    b2[e] = P[MLP_OFF_B2 + e];
  }
  if (tid < 2) b3[tid] = P[MLP_OFF_B3 + tid];
  // row (tid % 128) of a tile, its half (tid / 128) of the 16 chunks of 16 bytes;
  // rows >= n as zeros
  auto stage = [&](int tile) {
    const int rr = tid & (TCF_ROWS - 1), c0 = (tid >> 7) * 8, r = tile * TCF_ROWS + rr;
    const bool valid = r < n;
    const bf16 *src = X + (size_t)(valid ? r : 0) * MLP_IN;
#pragma unroll
    for (int c = c0; c < c0 + 8; c++)
      cp_async16(reinterpret_cast<bf16 *>(xs + tcf_off(rr, 8 * c, TCF_ROWS)), src + 8 * c, valid);
    cp_async_commit();
  };
  int tile = blockIdx.x;
  if (tile < ntile) stage(tile);
  if (warp == 0) tc::alloc(&tslot, TCF_TMEM_COLS);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot, lane_addr = tmem + ((uint32_t)(32 * quarter) << 16);
  const uint32_t id64 = tc::idesc_bf16_f32(TCF_ROWS, MLP_H), id16 = tc::idesc_bf16_f32(TCF_ROWS, TCF_N3);
  uint32_t phase = 0;
  bool ok = true;
  // one layer: D (columns col..) = A (shared, 128 rows, K = k) * B^T.  Thread 0
  // issues the MMAs and alone polls their completion (false if it gave up); the
  // others wait at the barrier that follows, which costs them no issue slots
  auto layer = [&](const unsigned char *a, const unsigned char *b, int brows, int k, uint32_t col, uint32_t idesc) {
    bool done = true;
    if (tid == 0) {
      tc::fence_after_sync();
      for (int s = 0; s < k / 16; s++) {
        const uint64_t ad = tc::smem_desc(tc::smem_addr(a) + (uint32_t)s * 2 * TCF_ROWS * 16, TCF_ROWS * 16, 128);
        const uint64_t bd = tc::smem_desc(tc::smem_addr(b) + (uint32_t)s * 2 * brows * 16, brows * 16, 128);
        tc::mma_bf16(tmem + col, ad, bd, idesc, s > 0);
      }
      tc::commit(&bar);
      done = tc::mbar_wait(&bar, phase);
    }
    phase ^= 1;
    return done;
  };
  // bias, BF16 z, GELU, BF16 h of this thread's row and column half into the next
  // layer's A operand
  auto hidden = [&](const float *bias) {
    float acc[2][16];  // both loads in flight before one wait
    tc::ld16(lane_addr + (uint32_t)(half * 32), acc[0]);
    tc::ld16(lane_addr + (uint32_t)(half * 32 + 16), acc[1]);
    tc::wait_ld();
#pragma unroll
    for (int cc = 0; cc < 2; cc++) {
      const int c0 = half * 32 + cc * 16;
      uint32_t h[8];
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const float2 z =
            unpack2(pack2(acc[cc][2 * i] + bias[c0 + 2 * i], acc[cc][2 * i + 1] + bias[c0 + 2 * i + 1]));
        h[i] = pack2(gelu(z.x), gelu(z.y));
      }
      *reinterpret_cast<uint4 *>(hs + tcf_off(m, c0, TCF_ROWS)) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4 *>(hs + tcf_off(m, c0 + 8, TCF_ROWS)) = make_uint4(h[4], h[5], h[6], h[7]);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc::fence_before_sync();
    __syncthreads();
  };
  for (; tile < ntile; tile += gridDim.x) {
    cp_async_wait<0>();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc::fence_before_sync();
    __syncthreads();
    ok = layer(xs, w1, MLP_H, MLP_IN, 0, id64);
    if (!__syncthreads_and(ok)) break;
    tc::fence_after_sync();
    // the first layer has read X: the next tile streams in behind the epilogues
    if (tile + (int)gridDim.x < ntile) stage(tile + gridDim.x);
    hidden(b1);
    ok = layer(hs, w2, MLP_H, MLP_H, 0, id64);
    if (!__syncthreads_and(ok)) break;
    tc::fence_after_sync();
    hidden(b2);
    ok = layer(hs, w3, TCF_N3, MLP_H, 64, id16);
    if (!__syncthreads_and(ok)) break;
    tc::fence_after_sync();
    if (half == 0) {
      float v[16];
      tc::ld16(lane_addr + 64u, v);
      tc::wait_ld();
      const int r = tile * TCF_ROWS + m;
      if (r < n) *reinterpret_cast<float2 *>(y + (size_t)r * MLP_OUT) = make_float2(v[0] + b3[0], v[1] + b3[1]);
    }
    tc::fence_before_sync();
  }
  cp_async_wait<0>();
  if (!ok) {
    // an MMA did not complete in time (thread 0 saw it): flag it, give it one more
    // bounded wait, and free the tensor memory all the same
    atomicOr(err, 1);
    tc::mbar_wait(&bar, phase ^ 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::dealloc(tmem, TCF_TMEM_COLS);
}

// Backward: dL/dparameters of sum over rows of dy . y, per CTA (FP32 partial
// blob to part[blockIdx.x]).  dy: FP32 [n][2].
struct MlpBwdSmem {
  MlpFwdW f;
  MlpBwdW b;
  bf16 xs[MLP_ROWS][MLP_LDX];    // X of the tile
  bf16 h1s[MLP_ROWS][MLP_LDH];   // GELU(z1)
  bf16 h2s[MLP_ROWS][MLP_LDH];   // GELU(z2)
  bf16 dz1s[MLP_ROWS][MLP_LDH];  // dL/dz1 (BF16)
  bf16 dz2s[MLP_ROWS][MLP_LDH];
  bf16 dys[MLP_ROWS][8];         // dL/dy (BF16), columns 2..7 zero
};

__global__ void __launch_bounds__(128, 2) k_mlp_backward(const float *__restrict__ P, const bf16 *__restrict__ X,
                                                         const float *__restrict__ dy, int n,
                                                         float *__restrict__ part) {
  extern __shared__ __align__(16) unsigned char mlp_raw[];
  MlpBwdSmem &s = *reinterpret_cast<MlpBwdSmem *>(mlp_raw);
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int q = lane >> 3, rr = lane & 7;
  load_fwd_weights(s.f, P, tid, blockDim.x);
  load_bwd_weights(s.b, P, tid, blockDim.x);
  float acc1[2][8][4], acc2[8][4], acc3[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int nt = 0; nt < 8; nt++)
#pragma unroll
    for (int e = 0; e < 4; e++) acc1[0][nt][e] = acc1[1][nt][e] = acc2[nt][e] = 0.0f;
  float accb = 0.0f, accb3 = 0.0f;  // bias sums of the thread's column
  const int ntile = (n + MLP_ROWS - 1) / MLP_ROWS;
  const int rw = 16 * w;  // the warp's rows within the tile
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int R0 = tile * MLP_ROWS;
    for (int c = tid; c < MLP_ROWS * 16; c += blockDim.x) {
      const int row = c >> 4, col = (c & 15) * 8;
      const bool valid = R0 + row < n;
      cp_async16(&s.xs[row][col], X + (size_t)(valid ? R0 + row : 0) * MLP_IN + col, valid);
    }
    cp_async_commit();
    if (tid < MLP_ROWS) {
      const bool valid = R0 + tid < n;
      const float2 d =
          valid ? *reinterpret_cast<const float2 *>(dy + (size_t)(R0 + tid) * MLP_OUT) : make_float2(0.0f, 0.0f);
      *reinterpret_cast<uint4 *>(&s.dys[tid][0]) = make_uint4(pack2(d.x, d.y), 0u, 0u, 0u);
    }
    cp_async_wait<0>();
    __syncthreads();
    // ---- data gradients of the warp's 16 rows
    {
      unsigned z1p[8][2], z2p[8][2], h2[4][4];
      layers12<false>(s.f, &s.xs[rw][0], lane, z1p, z2p, h2, &s.h1s[rw][0], &s.h2s[rw][0]);
      // dh2 = dy W3^T: A = dy (16 x 16, columns >= 8 zero)
      const unsigned a[4] = {ld_u32(&s.dys[rw + g][2 * t]), ld_u32(&s.dys[rw + g + 8][2 * t]), 0u, 0u};
      float c[8][4];
#pragma unroll
      for (int np = 0; np < 4; np++) {
        unsigned b[4];
        ldsm_x4(b, &s.b.w3[np * 16 + rr + 8 * (q >> 1)][8 * (q & 1)]);
        c[2 * np][0] = c[2 * np][1] = c[2 * np][2] = c[2 * np][3] = 0.0f;
        c[2 * np + 1][0] = c[2 * np + 1][1] = c[2 * np + 1][2] = c[2 * np + 1][3] = 0.0f;
        mma16816(c[2 * np], a, &b[0]);
        mma16816(c[2 * np + 1], a, &b[2]);
      }
      // dz2 = dh2 GELU'(z2), BF16, as A fragments and row-major in dz2s
      unsigned d2[4][4];
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const int col = nt * 8 + 2 * t;
        const float2 zr = unpack2(z2p[nt][0]), zs = unpack2(z2p[nt][1]);
        const unsigned pa = pack2(c[nt][0] * gelu_d(zr.x), c[nt][1] * gelu_d(zr.y));
        const unsigned pb = pack2(c[nt][2] * gelu_d(zs.x), c[nt][3] * gelu_d(zs.y));
        d2[nt >> 1][(nt & 1) * 2 + 0] = pa;
        d2[nt >> 1][(nt & 1) * 2 + 1] = pb;
        st_u32(&s.dz2s[rw + g][col], pa);
        st_u32(&s.dz2s[rw + g + 8][col], pb);
      }
      // dh1 = dz2 W2^T: B(k = out, n = in) = W2[n][k]
#pragma unroll
      for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
      for (int kb = 0; kb < 4; kb++)
#pragma unroll
        for (int np = 0; np < 4; np++) {
          unsigned b[4];
          ldsm_x4(b, &s.b.w2[np * 16 + rr + 8 * (q >> 1)][kb * 16 + 8 * (q & 1)]);
          mma16816(c[2 * np], d2[kb], &b[0]);
          mma16816(c[2 * np + 1], d2[kb], &b[2]);
        }
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const int col = nt * 8 + 2 * t;
        const float2 zr = unpack2(z1p[nt][0]), zs = unpack2(z1p[nt][1]);
        st_u32(&s.dz1s[rw + g][col], pack2(c[nt][0] * gelu_d(zr.x), c[nt][1] * gelu_d(zr.y)));
        st_u32(&s.dz1s[rw + g + 8][col], pack2(c[nt][2] * gelu_d(zs.x), c[nt][3] * gelu_d(zs.y)));
      }
    }
    __syncthreads();
    // ---- weight gradients of the tile, k = the 64 rows
#pragma unroll
    for (int kk = 0; kk < MLP_ROWS / 16; kk++) {
      const int k0 = kk * 16;
      // B = dz1 (k = row, n = hidden): 8 n-tiles, two per ldmatrix
      unsigned b1[4][4];
#pragma unroll
      for (int np = 0; np < 4; np++) ldsm_x4_t(b1[np], &s.dz1s[k0 + rr + 8 * (q & 1)][np * 16 + 8 * (q >> 1)]);
      // dW1 = X^T dz1: m-tiles 2w, 2w+1 (inputs 32w..32w+31)
#pragma unroll
      for (int mi = 0; mi < 2; mi++) {
        unsigned a[4];
        ldsm_x4_t(a, &s.xs[k0 + rr + 8 * (q >> 1)][(2 * w + mi) * 16 + 8 * (q & 1)]);
#pragma unroll
        for (int np = 0; np < 4; np++) {
          mma16816(acc1[mi][2 * np], a, &b1[np][0]);
          mma16816(acc1[mi][2 * np + 1], a, &b1[np][2]);
        }
      }
      // dW2 = GELU(z1)^T dz2: m-tile w; dW3 = GELU(z2)^T dy: m-tile w
      unsigned a[4];
      ldsm_x4_t(a, &s.h1s[k0 + rr + 8 * (q >> 1)][w * 16 + 8 * (q & 1)]);
#pragma unroll
      for (int np = 0; np < 4; np++) {
        unsigned b[4];
        ldsm_x4_t(b, &s.dz2s[k0 + rr + 8 * (q & 1)][np * 16 + 8 * (q >> 1)]);
        mma16816(acc2[2 * np], a, &b[0]);
        mma16816(acc2[2 * np + 1], a, &b[2]);
      }
      ldsm_x4_t(a, &s.h2s[k0 + rr + 8 * (q >> 1)][w * 16 + 8 * (q & 1)]);
      unsigned b3[2];
      ldsm_x2_t(b3, &s.dys[k0 + rr + 8 * (q & 1)][0]);
      mma16816(acc3, a, b3);
    }
    // bias gradients: column sums over the tile's rows, in row order
    {
      const bf16(*dz)[MLP_LDH] = tid < MLP_H ? s.dz1s : s.dz2s;
      const int col = tid & (MLP_H - 1);
      float v = 0.0f;
      for (int r = 0; r < MLP_ROWS; r++) v += __bfloat162float(dz[r][col]);
      accb += v;
      if (tid < MLP_OUT) {
        float u = 0.0f;
        for (int r = 0; r < MLP_ROWS; r++) u += __bfloat162float(s.dys[r][tid]);
        accb3 += u;
      }
    }
    __syncthreads();  // the tile buffers are refilled next
  }
  float *out = part + (size_t)blockIdx.x * MLP_NPARAM;
#pragma unroll
  for (int mi = 0; mi < 2; mi++) {
    const int m0 = (2 * w + mi) * 16;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int col = nt * 8 + 2 * t;
      *reinterpret_cast<float2 *>(out + MLP_OFF_W1 + (m0 + g) * MLP_H + col) =
          make_float2(acc1[mi][nt][0], acc1[mi][nt][1]);
      *reinterpret_cast<float2 *>(out + MLP_OFF_W1 + (m0 + g + 8) * MLP_H + col) =
          make_float2(acc1[mi][nt][2], acc1[mi][nt][3]);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int col = nt * 8 + 2 * t;
    *reinterpret_cast<float2 *>(out + MLP_OFF_W2 + (w * 16 + g) * MLP_H + col) = make_float2(acc2[nt][0], acc2[nt][1]);
    *reinterpret_cast<float2 *>(out + MLP_OFF_W2 + (w * 16 + g + 8) * MLP_H + col) =
        make_float2(acc2[nt][2], acc2[nt][3]);
  }
  {
    const int col = 2 * t;  // columns 2..7 of W3 are padding: zero
    const bool live = col < MLP_OUT;
    *reinterpret_cast<float2 *>(out + MLP_OFF_W3 + (w * 16 + g) * MLP_OUTP + col) =
        live ? make_float2(acc3[0], acc3[1]) : make_float2(0.0f, 0.0f);
    *reinterpret_cast<float2 *>(out + MLP_OFF_W3 + (w * 16 + g + 8) * MLP_OUTP + col) =
        live ? make_float2(acc3[2], acc3[3]) : make_float2(0.0f, 0.0f);
  }
  out[(tid < MLP_H ? MLP_OFF_B1 : MLP_OFF_B2) + (tid & (MLP_H - 1))] = accb;
  if (tid < MLP_OUTP) out[MLP_OFF_B3 + tid] = tid < MLP_OUT ? accb3 : 0.0f;
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
  int cap = 0;           // rows a call may pass
  float *P = nullptr;    // FP32 master parameters
  float *grad = nullptr;
  float *m1 = nullptr, *m2 = nullptr;
  float *part = nullptr;            // per-CTA gradient partials of the backward pass
  int fwd_ctas = 0, bwd_ctas = 0;   // persistent grids: the device's resident CTAs
  int tc_ctas = 0;                  // the tcgen05 forward's persistent grid
  int *err = nullptr;               // device flag: an MMA of the tcgen05 forward did not complete
  int path = FARGO_MLP_MMA_SYNC;    // fargo_mlp_set_tensor_path (the faster, measured)
  int steps = 0;
};

static size_t fwd_smem() { return sizeof(MlpFwdSmem); }
static size_t bwd_smem() { return sizeof(MlpBwdSmem); }

extern "C" {

int fargo_mlp_create(int max_rows, fargo_mlp **out) {
  if (!out || max_rows <= 0) return FARGO_ERR_INVALID;
  *out = nullptr;
  fargo_mlp *m = new fargo_mlp();
  m->cap = max_rows;
  int dev = 0, sms = 0, per_fwd = 0, per_bwd = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem());
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_fwd, k_mlp_forward, 128, fwd_smem());
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_bwd, k_mlp_backward, 128, bwd_smem());
  if (e == cudaSuccess && (per_fwd < 1 || per_bwd < 1)) e = cudaErrorInvalidConfiguration;
  m->fwd_ctas = sms * per_fwd;
  m->bwd_ctas = sms * per_bwd;
  int per_tc = 0;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TCF_SMEM);
  // the largest shared-memory carveout, so that three CTAs fit an SM
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_tc, k_mlp_forward_tc, TCF_THREADS, TCF_SMEM);
  // CTAs that fit an SM by shared memory (the occupancy query reported one CTA per
  // SM for this kernel on GB300, where ncu shows three resident), and by tensor
  // memory: TCF_TMEM_COLS columns per CTA, 512 per SM
  int smem_sm = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  const int per_smem = smem_sm / (TCF_SMEM + 2048);  // + static shared memory and the per-CTA reserve
  m->tc_ctas = sms * std::max(1, std::min(std::max(per_tc, per_smem), 512 / TCF_TMEM_COLS));
  if (e == cudaSuccess) e = cudaMalloc(&m->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&m->P, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->grad, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->m1, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->m2, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->part, (size_t)m->bwd_ctas * MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMemset(m->P, 0, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMemset(m->m1, 0, MLP_NPARAM * 4);
  if (e == cudaSuccess) e = cudaMemset(m->m2, 0, MLP_NPARAM * 4);
  if (e != cudaSuccess) {
    fargo_mlp_destroy(m);
    return FARGO_ERR_CUDA;
  }
  *out = m;
  return FARGO_OK;
}

void fargo_mlp_destroy(fargo_mlp *m) {
  if (!m) return;
  for (void *p : {(void *)m->P, (void *)m->grad, (void *)m->m1, (void *)m->m2, (void *)m->part, (void *)m->err})
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

// x: BF16 rows of 256 bytes, 16-byte aligned (the cp.async staging); y, dy: 8-byte aligned
static bool rows_ok(const fargo_mlp *m, const void *x, int n, const void *v) {
  return m && x && v && n > 0 && n <= m->cap && ((uintptr_t)x & 15) == 0 && ((uintptr_t)v & 7) == 0;
}

int fargo_mlp_forward(fargo_mlp *m, const void *x, int n, float *y, int train, void *stream) {
  (void)train;  // the backward pass recomputes what it needs
  if (!rows_ok(m, x, n, y)) return FARGO_ERR_INVALID;
  if (m->path == FARGO_MLP_TCGEN05) {
    const int ctas = std::min(m->tc_ctas, (n + TCF_ROWS - 1) / TCF_ROWS);
    k_mlp_forward_tc<<<ctas, TCF_THREADS, TCF_SMEM, (cudaStream_t)stream>>>(m->P, (const bf16 *)x, n, y, m->err);
  } else {
    const int warps = (n + 15) / 16, ctas = std::min(m->fwd_ctas, (warps + 3) / 4);
    k_mlp_forward<<<ctas, 128, fwd_smem(), (cudaStream_t)stream>>>(m->P, (const bf16 *)x, n, y);
  }
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

int fargo_mlp_set_tensor_path(fargo_mlp *m, int path) {
  if (!m || (path != FARGO_MLP_TCGEN05 && path != FARGO_MLP_MMA_SYNC)) return FARGO_ERR_INVALID;
  m->path = path;
  return FARGO_OK;
}

int fargo_mlp_status(fargo_mlp *m) {
  if (!m) return FARGO_ERR_INVALID;
  int e = 0;
  if (cudaMemcpy(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return FARGO_ERR_CUDA;
  return e ? FARGO_ERR_NUMERIC : FARGO_OK;
}

int fargo_mlp_backward(fargo_mlp *m, const void *x, int n, const float *dy, void *stream) {
  if (!rows_ok(m, x, n, dy)) return FARGO_ERR_INVALID;
  const cudaStream_t s = (cudaStream_t)stream;
  const int ctas = std::min(m->bwd_ctas, (n + MLP_ROWS - 1) / MLP_ROWS);
  k_mlp_backward<<<ctas, 128, bwd_smem(), s>>>(m->P, (const bf16 *)x, dy, n, m->part);
  k_mlp_reduce<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(m->part, ctas, m->grad);
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
