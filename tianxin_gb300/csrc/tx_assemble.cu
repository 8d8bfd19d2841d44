// tx_assemble.cu -- per-block launches of the fused volume assembly
// (tx_assemble_body.cuh): one launch per block or workset range, or one per
// colour for the deterministic scatter; FP32 or FP64 element arithmetic,
// Residual, Jacobian or Tangent evaluation type.
#include <cstdio>

#include "tx_assemble_body.cuh"

namespace tx {
namespace {

// SCR: the first phase of the two-phase evaluation (element rows to scratch).
// FP64 hex27: the reference tables and the elements' epos read from global memory (through L1) instead of
// shared memory, which halves the CTA's shared memory (139.7 -> 97 KB) and lets two CTAs share an SM (the
// FP32 build keeps them in shared memory: there the fourth CTA's smaller L1 cost more than it gained).
template <typename Real>
constexpr bool global_ref() { return sizeof(Real) == 8; }

// tet10 (FP32): five CTAs an SM (at most 102 registers; it needs 96 without spills) rather than four: its
// gathers are latency-bound, and the fifth CTA takes the 48^3 tet10 heat block from 0.79 to about 0.68 ms.
template <int TOPO, int BASIS, int NQ, int PHYS, typename Real, bool JAC, bool ATOMIC, bool STAGE, bool TAN = false,
          bool SCR = false>
__global__ void __launch_bounds__(block_threads<TOPO, BASIS, NQ, PHYS, Real, STAGE>(),
                                  min_blocks<Real, STAGE>() +
                                      ((TOPO == TX_TOPO_TET && BASIS == TX_HGRAD_C2 && sizeof(Real) == 4) ? 1 : 0))
k_assemble(const BlockView B, const EvalParams P, const int32_t* perm, int64_t e_lo, int64_t e_hi) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int T = block_threads<TOPO, BASIS, NQ, PHYS, Real, STAGE>();
  assemble_body<TOPO, BASIS, NQ, PHYS, Real, JAC, ATOMIC, T, STAGE, TAN, SCR, global_ref<Real>()>(
      B, P, perm, e_lo, e_hi, blockIdx.x, gridDim.x, smem);
}

template <int TOPO, int BASIS, int NQ, int PHYS, typename Real, bool JAC, bool ATOMIC, bool STAGE, bool TAN = false,
          bool SCR = false>
cudaError_t launch_one(const BlockView& B, const EvalParams& P, const int32_t* perm, int64_t e_lo, int64_t e_hi,
                       cudaStream_t s, int grid_cap) {
  constexpr int T = block_threads<TOPO, BASIS, NQ, PHYS, Real, STAGE>();
  using C = Cfg<TOPO, BASIS, NQ, PHYS, Real, T, STAGE, global_ref<Real>()>;
  auto kern = k_assemble<TOPO, BASIS, NQ, PHYS, Real, JAC, ATOMIC, STAGE, TAN, SCR>;
  static int max_blocks_per_sm = -1;
  static int num_sms = 0;
  if (max_blocks_per_sm < 0) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    if (err != cudaSuccess) return err;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_blocks_per_sm, kern, T, C::SMEM);
    if (err != cudaSuccess) return err;
    if (max_blocks_per_sm < 1) max_blocks_per_sm = 1;
  }
  const int64_t n = e_hi - e_lo;
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + C::EPB - 1) / C::EPB;
  int64_t cap = (int64_t)max_blocks_per_sm * num_sms * 4;
  if (grid_cap > 0 && grid_cap < cap) cap = grid_cap;
  if (blocks > cap) blocks = cap;
  kern<<<(unsigned)blocks, T, C::SMEM, s>>>(B, P, perm, e_lo, e_hi);
  return cudaGetLastError();
}

template <int TOPO, int BASIS, int NQ, int PHYS>
cudaError_t launch_prec(const BlockView& B, const EvalParams& P, bool mixed, const int32_t* perm, int64_t e_lo,
                        int64_t e_hi, bool atomic, bool stage, cudaStream_t s, int cap) {
  const bool jac = P.vals != nullptr;
  const bool st = stage && jac;
#define TX_L(R, J, A, S) launch_one<TOPO, BASIS, NQ, PHYS, R, J, A, S>(B, P, perm, e_lo, e_hi, s, cap)
  if (P.kscr) {  // two-phase, first phase: element rows to scratch (staged kernels' register rows)
    if (!jac) return cudaErrorInvalidValue;
    return mixed ? launch_one<TOPO, BASIS, NQ, PHYS, float, true, true, true, false, true>(B, P, perm, e_lo, e_hi, s, cap)
                 : launch_one<TOPO, BASIS, NQ, PHYS, double, true, true, true, false, true>(B, P, perm, e_lo, e_hi, s,
                                                                                           cap);
  }
  if (P.tan) {  // Tangent: FP64 rows, atomic dfdp sums
    if (atomic) return launch_one<TOPO, BASIS, NQ, PHYS, double, true, true, false, true>(B, P, perm, e_lo, e_hi, s, cap);
    return launch_one<TOPO, BASIS, NQ, PHYS, double, true, false, false, true>(B, P, perm, e_lo, e_hi, s, cap);
  }
  if (st) {
    if (atomic) return mixed ? TX_L(float, true, true, true) : TX_L(double, true, true, true);
    return mixed ? TX_L(float, true, false, true) : TX_L(double, true, false, true);
  }
  if (atomic) {
    if (mixed) return jac ? TX_L(float, true, true, false) : TX_L(float, false, true, false);
    return jac ? TX_L(double, true, true, false) : TX_L(double, false, true, false);
  }
  if (mixed) return jac ? TX_L(float, true, false, false) : TX_L(float, false, false, false);
  return jac ? TX_L(double, true, false, false) : TX_L(double, false, false, false);
#undef TX_L
}

}  // namespace

int assemble_kind(int topo, int basis, int nq, int physics) {
#define TX_K(K, T, BS, Q, PH) \
  if (topo == T && basis == BS && nq == Q && physics == PH) return K;
  TX_FOR_EACH_KIND(TX_K)
#undef TX_K
  return -1;
}

cudaError_t launch_assemble(const BlockView& B, const EvalParams& P, bool mixed, const int32_t* perm, int64_t e_lo,
                            int64_t e_hi, bool atomic, bool stage, cudaStream_t s, int cap) {
  switch (assemble_kind(B.topo, B.basis, B.nq, P.physics)) {
#define TX_LAUNCH(K, T, BS, Q, PH) \
  case K:                          \
    return launch_prec<T, BS, Q, PH>(B, P, mixed, perm, e_lo, e_hi, atomic, stage, s, cap);
    TX_FOR_EACH_KIND(TX_LAUNCH)
#undef TX_LAUNCH
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace tx
