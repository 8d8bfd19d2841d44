// tx_assemble_tiles.cu -- the CTA-staged assembly kernel at other tile
// shapes: 64 or 256 threads a CTA instead of 128, i.e. half or twice the
// elements a CTA (elements per CTA = threads / threads per element, the
// element's basis count rounded up to a power of two: hex8 8 -> 8 or 32
// elements, tet10 16 -> 4 or 16, hex27 32 -> 2 or 8).  The knob plays the
// part of Panzer's team size (disc-fe/src/Panzer_HierarchicParallelism.hpp:
// 78-128) for the autotuner.  Instantiated for the families whose shape the
// tuner searches: hex8 elasticity, hex27 and tet10 heat; atomic staged
// scatter, FP32 and FP64 element arithmetic; a shape whose FP64 tables do
// not fit one CTA's shared memory (hex27 at 256 threads) is not offered.
#include "tx_assemble_body.cuh"

namespace tx {
namespace {

template <int TOPO, int BASIS, int NQ, int PHYS, typename Real, int TH>
__global__ void __launch_bounds__(TH, sizeof(Real) == 4 ? 512 / TH : 1)
k_assemble_tile(const BlockView B, const EvalParams P, int64_t e_lo, int64_t e_hi) {
  extern __shared__ __align__(16) unsigned char smem[];
  assemble_body<TOPO, BASIS, NQ, PHYS, Real, true, true, TH, true>(B, P, nullptr, e_lo, e_hi, blockIdx.x, gridDim.x,
                                                                  smem);
}

template <int TOPO, int BASIS, int NQ, int PHYS, typename Real, int TH>
cudaError_t launch_tile(const BlockView& B, const EvalParams& P, int64_t e_lo, int64_t e_hi, cudaStream_t s,
                        int grid_cap) {
  using C = Cfg<TOPO, BASIS, NQ, PHYS, Real, TH, true>;
  auto kern = k_assemble_tile<TOPO, BASIS, NQ, PHYS, Real, TH>;
  static int max_blocks_per_sm = -1;
  static int num_sms = 0;
  if (max_blocks_per_sm < 0) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    if (err != cudaSuccess) return err;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_blocks_per_sm, kern, TH, C::SMEM);
    if (err != cudaSuccess) return err;
    if (max_blocks_per_sm < 1) max_blocks_per_sm = 1;
  }
  const int64_t n = e_hi - e_lo;
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + C::EPB - 1) / C::EPB;
  int64_t cap = (int64_t)max_blocks_per_sm * num_sms * 4;
  if (grid_cap > 0 && grid_cap < cap) cap = grid_cap;
  if (blocks > cap) blocks = cap;
  kern<<<(unsigned)blocks, TH, C::SMEM, s>>>(B, P, e_lo, e_hi);
  return cudaGetLastError();
}

template <int TOPO, int BASIS, int NQ, int PHYS, int TH>
cudaError_t launch_shape(const BlockView& B, const EvalParams& P, bool mixed, int64_t e_lo, int64_t e_hi,
                         cudaStream_t s, int cap) {
  constexpr size_t kMax = 227 * 1024;
  if constexpr (Cfg<TOPO, BASIS, NQ, PHYS, float, TH, true>::SMEM <= kMax &&
                Cfg<TOPO, BASIS, NQ, PHYS, double, TH, true>::SMEM <= kMax) {
    return mixed ? launch_tile<TOPO, BASIS, NQ, PHYS, float, TH>(B, P, e_lo, e_hi, s, cap)
                 : launch_tile<TOPO, BASIS, NQ, PHYS, double, TH>(B, P, e_lo, e_hi, s, cap);
  } else {
    return cudaErrorInvalidValue;
  }
}

template <int TOPO, int BASIS, int NQ, int PHYS>
cudaError_t launch_family(const BlockView& B, const EvalParams& P, bool mixed, int threads, int64_t e_lo,
                          int64_t e_hi, cudaStream_t s, int cap) {
  if (threads == 64) return launch_shape<TOPO, BASIS, NQ, PHYS, 64>(B, P, mixed, e_lo, e_hi, s, cap);
  if (threads == 256) return launch_shape<TOPO, BASIS, NQ, PHYS, 256>(B, P, mixed, e_lo, e_hi, s, cap);
  return cudaErrorInvalidValue;
}

// Shared memory of the staged kernel of a family at a tile shape, in both
// precisions; a shape is offered only where both fit one CTA.
template <int TOPO, int BASIS, int NQ, int PHYS, int TH>
constexpr bool fits() {
  constexpr size_t kMax = 227 * 1024;
  return Cfg<TOPO, BASIS, NQ, PHYS, float, TH, true>::SMEM <= kMax &&
         Cfg<TOPO, BASIS, NQ, PHYS, double, TH, true>::SMEM <= kMax;
}

}  // namespace

bool tile_shape_supported(int kind, int threads) {
  if (threads != 64 && threads != 256) return false;
  const bool t64 = threads == 64;
  switch (kind) {
    case K_HEX8_ELAST:
      return t64 ? fits<TX_TOPO_HEX, TX_HGRAD_C1, 8, TX_PHYS_ELASTICITY, 64>()
                 : fits<TX_TOPO_HEX, TX_HGRAD_C1, 8, TX_PHYS_ELASTICITY, 256>();
    case K_HEX27_HEAT:
      return t64 ? fits<TX_TOPO_HEX, TX_HGRAD_C2, 27, TX_PHYS_HEAT, 64>()
                 : fits<TX_TOPO_HEX, TX_HGRAD_C2, 27, TX_PHYS_HEAT, 256>();
    case K_TET10_HEAT:
      return t64 ? fits<TX_TOPO_TET, TX_HGRAD_C2, 4, TX_PHYS_HEAT, 64>()
                 : fits<TX_TOPO_TET, TX_HGRAD_C2, 4, TX_PHYS_HEAT, 256>();
    default:
      return false;
  }
}

cudaError_t launch_assemble_tile(const BlockView& B, const EvalParams& P, bool mixed, int threads, int64_t e_lo,
                                 int64_t e_hi, cudaStream_t s, int grid_cap) {
  if (!P.vals || P.tan || P.kscr) return cudaErrorInvalidValue;  // Jacobian evaluations of the staged kernel
  switch (assemble_kind(B.topo, B.basis, B.nq, P.physics)) {
    case K_HEX8_ELAST:
      return launch_family<TX_TOPO_HEX, TX_HGRAD_C1, 8, TX_PHYS_ELASTICITY>(B, P, mixed, threads, e_lo, e_hi, s,
                                                                            grid_cap);
    case K_HEX27_HEAT:
      return launch_family<TX_TOPO_HEX, TX_HGRAD_C2, 27, TX_PHYS_HEAT>(B, P, mixed, threads, e_lo, e_hi, s, grid_cap);
    case K_TET10_HEAT:
      return launch_family<TX_TOPO_TET, TX_HGRAD_C2, 4, TX_PHYS_HEAT>(B, P, mixed, threads, e_lo, e_hi, s, grid_cap);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace tx
