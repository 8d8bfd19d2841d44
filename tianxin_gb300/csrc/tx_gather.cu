// tx_gather.cu -- second phase of the two-phase (gather) evaluation.
//
// The first phase (the staged assembly kernels with EvalParams::kscr set)
// leaves every element's residual and Jacobian in scratch.  Here one warp
// takes one entity row: it sums, in the fixed order of the entity's
// incidence list (blocks, elements, local basis in order), the element rows
// of the entity into a shared-memory copy of its nf CRS rows (the element
// column block b lands at its position epos[e][a][b] of the sorted row, as in
// ScatterResidual's sumIntoValues), then writes each CRS value and residual
// entry once.  No atomics and no prior zeroing: f and the CRS values are
// overwritten, and the sums have a fixed order (bitwise reproducible).
// Accumulation in FP64 whatever the element arithmetic's type.
#include "tx_device.cuh"
#include "tx_numeric.cuh"

namespace tx {
namespace {

constexpr int kGatherWarps = 8;  // 8 x 512 doubles = 32 KB of row accumulators a CTA

template <typename Real>
__global__ void __launch_bounds__(32 * kGatherWarps)
k_gather_rows(int64_t n_ent, int nf, const int64_t* __restrict__ inc_ptr, const int64_t* __restrict__ inc,
              GatherBlocks G, const int64_t* __restrict__ erp, const int64_t* __restrict__ rowptr,
              double* __restrict__ vals, double* __restrict__ f) {
  __shared__ double acc[kGatherWarps][kGatherRowMax];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double* row = acc[wid];
  const int64_t nwarps = (int64_t)gridDim.x * kGatherWarps;
  for (int64_t a = (int64_t)blockIdx.x * kGatherWarps + wid; a < n_ent; a += nwarps) {  // warp-uniform
    const int64_t deg = __ldg(erp + a + 1) - __ldg(erp + a);
    const int width = (int)(deg * nf);          // entries in one of the entity's rows
    for (int k = lane; k < width * nf; k += 32) row[k] = 0.0;
    double fr = 0.0;  // lane c < nf: residual of row c
    __syncwarp();
    const int64_t i1 = __ldg(inc_ptr + a + 1);
    for (int64_t i = __ldg(inc_ptr + a); i < i1; ++i) {
      const int64_t code = __ldg(inc + i);
      const int blk = (int)(code >> 56), la = (int)(code & 0xff);
      const int64_t e = (code >> 8) & ((int64_t(1) << 48) - 1);
      const GatherBlock& B = G.b[blk];
      const int nb = B.nb, ne = nf * nb;
      const Real* K = reinterpret_cast<const Real*>(B.k) + (e * ne + la * nf) * ne;  // rows la*nf .. la*nf+nf-1
      const uint8_t* ep = B.epos + (e * nb + la) * nb;
      for (int t = lane; t < nf * ne; t += 32) {
        const int c = t / ne, col = t - (t / ne) * ne;
        const int b = col / nf, d = col - (col / nf) * nf;
        row[c * width + nf * (int)__ldg(ep + b) + d] += widen(__ldg(K + t));  // widening off the FP64 pipe
      }
      if (lane < nf) fr += widen(__ldg(reinterpret_cast<const Real*>(B.r) + e * ne + la * nf + lane));
      __syncwarp();
    }
    for (int c = 0; c < nf; ++c) {
      double* out = vals + __ldg(rowptr + nf * a + c);
      for (int k = lane; k < width; k += 32) out[k] = row[c * width + k];
    }
    if (f && lane < nf) f[nf * a + lane] = fr;
    __syncwarp();
  }
}

}  // namespace

cudaError_t launch_gather_rows(int64_t n_ent, int nf, const int64_t* inc_ptr, const int64_t* inc,
                               const GatherBlocks& G, bool mixed, const int64_t* erp, const int64_t* rowptr,
                               double* vals, double* f, cudaStream_t s) {
  if (n_ent <= 0) return cudaSuccess;
  int64_t g = (n_ent + kGatherWarps - 1) / kGatherWarps;
  if (g > 152 * 64) g = 152 * 64;
  if (mixed)
    k_gather_rows<float><<<(unsigned)g, 32 * kGatherWarps, 0, s>>>(n_ent, nf, inc_ptr, inc, G, erp, rowptr, vals, f);
  else
    k_gather_rows<double><<<(unsigned)g, 32 * kGatherWarps, 0, s>>>(n_ent, nf, inc_ptr, inc, G, erp, rowptr, vals, f);
  return cudaGetLastError();
}

}  // namespace tx
