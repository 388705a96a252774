// fargo_tc.cu -- self-test of the tcgen05 path (fargo_tc.cuh): one CTA computes
// D (128 x n, FP32) = A (128 x k, BF16) * B (n x k, BF16)^T with k / 16 MMAs into
// tensor memory and reads D back through tcgen05.ld.  The learned correction's
// tensor-core MLP is built from the same operand layout, descriptors and
// accumulator loads; the test pins them against a CPU product.
#include <cuda_runtime.h>

#include <cstdint>

#include "fargo_gb300.h"
#include "fargo_tc.cuh"

namespace {

__global__ void __launch_bounds__(128) k_tc_selftest(const uint16_t *__restrict__ A, const uint16_t *__restrict__ B,
                                                     int n, int k, int mode, float *__restrict__ D, int *status) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint32_t tslot;
  __shared__ __align__(8) uint64_t bar;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // memory strides of A (128 rows) and B (n rows): core matrices adjacent along K
  // (lk) and along the rows (lr) -- mode 1 puts the rows of a K chunk together
  const uint32_t a_lk = mode == 1 ? 128u * 16u : 128u, a_lr = mode == 1 ? 128u : (uint32_t)k * 16u;
  const uint32_t b_lk = mode == 1 ? (uint32_t)n * 16u : 128u, b_lr = mode == 1 ? 128u : (uint32_t)k * 16u;
  unsigned char *sa = sm, *sb = sm + (size_t)128 * k * 2;
  for (int i = tid; i < 128 * k; i += blockDim.x)
    *reinterpret_cast<uint16_t *>(sa + tc::kmajor_offset(i / k, i % k, a_lk, a_lr)) = A[i];
  for (int i = tid; i < n * k; i += blockDim.x)
    *reinterpret_cast<uint16_t *>(sb + tc::kmajor_offset(i / k, i % k, b_lk, b_lr)) = B[i];
  // the operands were written through the generic proxy; the MMA reads them
  // through the async proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const uint32_t ncols = n <= 32 ? 32 : (n <= 64 ? 64 : (n <= 128 ? 128 : 256));
  if (warp == 0) tc::alloc(&tslot, ncols);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = tslot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16_f32(128, n);
    for (int s = 0; s < k / 16; s++) {
      // descriptor: LBO = the stride along K, SBO = the stride along the rows (mode 2
      // swaps the two fields: the other reading of the descriptor)
      const uint32_t as = tc::smem_addr(sa) + (uint32_t)s * 2 * a_lk, bs = tc::smem_addr(sb) + (uint32_t)s * 2 * b_lk;
      const uint64_t ad = mode == 2 ? tc::smem_desc(as, a_lr, a_lk) : tc::smem_desc(as, a_lk, a_lr);
      const uint64_t bd = mode == 2 ? tc::smem_desc(bs, b_lr, b_lk) : tc::smem_desc(bs, b_lk, b_lr);
      tc::mma_bf16(taddr, ad, bd, idesc, s > 0);
    }
    tc::commit(&bar);
  }
  bool ok = tc::mbar_wait(&bar, 0);
  ok = __syncthreads_and(ok) != 0;
  tc::fence_after_sync();
  if (ok) {
    const uint32_t row_addr = taddr + ((uint32_t)(32 * warp) << 16);
    const int m = 32 * warp + lane;
    for (int c0 = 0; c0 < n; c0 += 16) {
      float v[16];
      tc::ld16(row_addr + (uint32_t)c0, v);
      tc::wait_ld();
      for (int i = 0; i < 16; i++) D[(size_t)m * n + c0 + i] = v[i];
    }
  } else {
    // the MMAs did not complete in time: flag it, give them one more bounded wait,
    // and free the tensor memory all the same
    if (tid == 0) *status = 1;
    tc::mbar_wait(&bar, 0);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::dealloc(taddr, ncols);
}

}  // namespace

extern "C" int fargo_tc_selftest(const unsigned short *a, const unsigned short *b, int n, int k, int mode, float *d) {
  if (!a || !b || !d || n < 16 || n > 256 || n % 16 || k < 16 || k > 128 || k % 16 || mode < 0 || mode > 2)
    return FARGO_ERR_INVALID;
  uint16_t *da = nullptr, *db = nullptr;
  float *dd = nullptr;
  int *ds = nullptr, st = 0;
  // the operands, and slack so that the MMA's reads stay inside the allocation
  // under either reading of the descriptor's two strides
  const size_t smem = (size_t)(128 + n) * k * 2 + 32768;
  int rc = FARGO_OK;
  if (cudaMalloc(&da, 128 * k * 2) != cudaSuccess || cudaMalloc(&db, (size_t)n * k * 2) != cudaSuccess ||
      cudaMalloc(&dd, (size_t)128 * n * 4) != cudaSuccess || cudaMalloc(&ds, sizeof(int)) != cudaSuccess)
    rc = FARGO_ERR_CUDA;
  if (rc == FARGO_OK && (cudaMemcpy(da, a, 128 * k * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
                         cudaMemcpy(db, b, (size_t)n * k * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
                         cudaMemset(ds, 0, sizeof(int)) != cudaSuccess ||
                         cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem) != cudaSuccess))
    rc = FARGO_ERR_CUDA;
  if (rc == FARGO_OK) {
    k_tc_selftest<<<1, 128, smem>>>(da, db, n, k, mode, dd, ds);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(d, dd, (size_t)128 * n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&st, ds, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = FARGO_ERR_CUDA;
    else if (st)
      rc = FARGO_ERR_NUMERIC;
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(dd);
  cudaFree(ds);
  return rc;
}
