/*
 * cg_tma.cuh -- bulk global -> shared copies through the Blackwell copy
 * engine (cp.async.bulk, completion counted on a shared-memory mbarrier),
 * in inline PTX.
 *
 * Rules the callers keep: both addresses 16-byte aligned, the size a
 * multiple of 16 and below 2^20 bytes (the mbarrier transaction range).
 * Every wait is bounded: stage_rows returns false when the copy has not
 * landed after CG_TMA_SPINS polls, after setting an error bit and waiting
 * (with the same bound) for the copy still in flight, so that the block can
 * leave without the engine writing into freed shared memory.
 */
#ifndef CG_TMA_CUH
#define CG_TMA_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#define CG_ERR_TMA_TIMEOUT 32u /* a bulk copy did not complete within the poll bound */
#define CG_TMA_SPINS (1u << 22)

namespace cgtma {

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  /* make the initialised barrier visible to the copy engine */
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

/* Bounded wait for phase `parity` of bar. */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
  for (unsigned i = 0; i < CG_TMA_SPINS; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

/* Copy `bytes` contiguous bytes from global src into shared dst with one
 * bulk copy issued by thread 0, every thread of the block waiting for it.
 * bar: a block-shared mbarrier used for this one copy.  Must be called by
 * all threads.  Returns false for every thread when the copy timed out
 * (err has CG_ERR_TMA_TIMEOUT set); the caller then leaves the kernel. */
__device__ __forceinline__ bool stage_rows(void *dst, const void *src, unsigned bytes, uint64_t *bar,
                                           unsigned int *err)
{
  if (threadIdx.x == 0) mbar_init(bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(bar, bytes);
    bulk_g2s(dst, src, bytes, bar);
  }
  const bool ok = mbar_wait(bar, 0);
  const bool any_late = __syncthreads_or(!ok);
  if (any_late) {
    if (threadIdx.x == 0 && err) atomicOr(err, CG_ERR_TMA_TIMEOUT);
    (void)mbar_wait(bar, 0); /* the copy may still be writing: bounded wait for it */
    __syncthreads();
    return false;
  }
  return true;
}

} /* namespace cgtma */

#endif /* CG_TMA_CUH */
