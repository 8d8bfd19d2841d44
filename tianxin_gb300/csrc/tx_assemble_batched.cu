// tx_assemble_batched.cu -- the persistent assembly kernel: CTAs take work
// items (element chunks of any block of any mesh, any element family) from
// an atomic counter, so the worksets of every block, or of many meshes, run
// in one launch.
#include "tx_assemble_body.cuh"

namespace tx {
namespace {

constexpr int kBatchThreads = 128;

// One work item of one element family, compiled out of line so that every
// family keeps its own register allocation inside the persistent kernel
// (inlined into one switch, the families' code shared one allocation of
// 238-255 registers).  The block view and parameters stay in global memory
// and are read through the pointers: copied by value into the caller, each
// thread kept its own 330-byte copy on its stack (local memory, rewritten for
// every work item and re-read inside the element loops; 7 % of the 256-mesh
// batch's time).
template <int T, int BS, int Q, int PH, typename Real, bool JAC, bool STAGE>
__device__ __noinline__ void batched_item(const BlockView* __restrict__ B, const EvalParams* __restrict__ P,
                                          int64_t e0, int64_t e1, unsigned char* smem) {
  assemble_body<T, BS, Q, PH, Real, JAC, true, kBatchThreads, STAGE, false, false, true>(*B, *P, nullptr, e0, e1, 0,
                                                                                        1, smem);
}

// Persistent kernel: CTAs take work items (element chunks of any block of
// any mesh, any family) from an atomic counter until the list is empty.
// STAGE: Jacobians through the staged, row-coalesced scatter, else each
// thread reduces its own rows.
// FP32 staged builds ask for five resident CTAs (at most 102 registers; some
// families' item functions then spill a little): the work items' gathers are
// latency-bound, and the fifth CTA takes the 256-mesh batch from 7.7 to 6.8 ms.
// FP64 builds ask for three (at most 168 registers): where shared memory
// allows a third CTA (the 256-mesh batch: FP64 48.6 -> 47.6 ms), the FP64 pipe
// gets a third warp a scheduler; the hex27 items' shared memory still allows
// two.
template <typename Real, bool JAC, bool STAGE>
__global__ void __launch_bounds__(kBatchThreads, min_blocks<Real, STAGE>() + (sizeof(Real) == 4 && STAGE ? 1 : 0) +
                                                     (sizeof(Real) == 8 ? 2 : 0))
k_assemble_batched(const BlockView* __restrict__ views, const EvalParams* __restrict__ params,
                   const WorkItem* __restrict__ items, int n_items, int* counter) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= n_items) break;
    const WorkItem w = items[it];
    switch (w.kind) {
#define TX_CASE(K, T, BS, Q, PH)                                                                     \
  case K:                                                                                            \
    batched_item<T, BS, Q, PH, Real, JAC, STAGE>(views + w.view, params + w.view, w.e0, w.e1, smem); \
    break;
      TX_FOR_EACH_KIND(TX_CASE)
#undef TX_CASE
      default:
        break;
    }
  }
}

template <typename Real, bool STAGE>
size_t smem_of_kind(int kind) {
  switch (kind) {
#define TX_SZ(K, T, BS, Q, PH) \
  case K:                      \
    return Cfg<T, BS, Q, PH, Real, kBatchThreads, STAGE, true>::SMEM;
    TX_FOR_EACH_KIND(TX_SZ)
#undef TX_SZ
    default:
      return 0;
  }
}

}  // namespace

int batched_elements_per_pass(int kind) {
  switch (kind) {
#define TX_EPB(K, T, BS, Q, PH) \
  case K:                       \
    return Cfg<T, BS, Q, PH, float, kBatchThreads>::EPB;
    TX_FOR_EACH_KIND(TX_EPB)
#undef TX_EPB
    default:
      return 1;
  }
}

size_t batched_smem_bytes(int kind, bool mixed, bool stage) {
  if (stage) return mixed ? smem_of_kind<float, true>(kind) : smem_of_kind<double, true>(kind);
  return mixed ? smem_of_kind<float, false>(kind) : smem_of_kind<double, false>(kind);
}

cudaError_t launch_assemble_batched(const BlockView* views, const EvalParams* params, const WorkItem* items,
                                    int n_items, int* counter, size_t smem, bool mixed, bool jac, bool stage,
                                    int grid, cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  auto go = [&](auto kern) -> cudaError_t {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBatchThreads, smem);
    if (err != cudaSuccess) return err;
    int g = (per_sm > 0 ? per_sm : 1) * sms;
    if (grid > 0 && grid < g) g = grid;
    if (g > n_items) g = n_items;
    kern<<<g, kBatchThreads, smem, s>>>(views, params, items, n_items, counter);
    return cudaGetLastError();
  };
  if (!jac) return mixed ? go(k_assemble_batched<float, false, false>) : go(k_assemble_batched<double, false, false>);
  if (stage) return mixed ? go(k_assemble_batched<float, true, true>) : go(k_assemble_batched<double, true, true>);
  return mixed ? go(k_assemble_batched<float, true, false>) : go(k_assemble_batched<double, true, false>);
}

}  // namespace tx
