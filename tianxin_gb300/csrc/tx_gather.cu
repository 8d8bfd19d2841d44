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
// The mixed form (FP32 element rows) sums in FP32, as the owner-computes
// lattice kernel does: an entry takes at most a few dozen contributions, so
// the sums stay within the mixed evaluation's stated error, and they keep
// GB300's FP64 pipe (about two operations a clock an SM) out of the loop; each
// value is widened to FP64 exactly when written.  The FP64 form sums in FP64.
#include "tx_device.cuh"
#include "tx_numeric.cuh"

namespace tx {
namespace {

constexpr int kGatherWarps = 8;  // 8 x 512 accumulators a CTA

// Exact FP32 -> FP64 by integer operations for zeros and normal numbers;
// *rare is set for a subnormal, infinity or NaN (the caller converts those
// with the hardware instruction afterwards).
__device__ __forceinline__ double widen_int(float v, bool& rare) {
  const uint32_t b = __float_as_uint(v), a = b & 0x7fffffffu;
  rare |= (a != 0u) & (a - 0x00800000u >= 0x7f000000u);
  const uint32_t hi = min(a, 1u) * 0x38000000u + ((uint32_t)((int32_t)b >> 3) & 0x8fffffffu);
  return __hiloint2double((int)hi, (int)(b << 29));
}

template <typename Real>
__global__ void __launch_bounds__(32 * kGatherWarps)
k_gather_rows(int64_t n_ent, int nf, const int64_t* __restrict__ inc_ptr, const int64_t* __restrict__ inc,
              GatherBlocks G, const int64_t* __restrict__ erp, const int64_t* __restrict__ rowptr,
              double* __restrict__ vals, double* __restrict__ f) {
  __shared__ Real acc[kGatherWarps][kGatherRowMax];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  Real* row = acc[wid];
  const int64_t nwarps = (int64_t)gridDim.x * kGatherWarps;
  for (int64_t a = (int64_t)blockIdx.x * kGatherWarps + wid; a < n_ent; a += nwarps) {  // warp-uniform
    const int64_t deg = __ldg(erp + a + 1) - __ldg(erp + a);
    const int width = (int)(deg * nf);          // entries in one of the entity's rows
    for (int k = lane; k < width * nf; k += 32) row[k] = Real(0);
    Real fr = Real(0);  // lane c < nf: residual of row c
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
        row[c * width + nf * (int)__ldg(ep + b) + d] += __ldg(K + t);
      }
      if (lane < nf) fr += __ldg(reinterpret_cast<const Real*>(B.r) + e * ne + la * nf + lane);
      __syncwarp();
    }
    if constexpr (sizeof(Real) == 8) {
      for (int c = 0; c < nf; ++c) {
        double* out = vals + __ldg(rowptr + nf * a + c);
        for (int k = lane; k < width; k += 32) out[k] = row[c * width + k];
      }
      if (f && lane < nf) f[nf * a + lane] = fr;
    } else {
      bool rare = false;
      for (int c = 0; c < nf; ++c) {
        double* out = vals + __ldg(rowptr + nf * a + c);
        for (int k = lane; k < width; k += 32) out[k] = widen_int(row[c * width + k], rare);
      }
      if (f && lane < nf) f[nf * a + lane] = widen_int(fr, rare);
      if (__any_sync(0xffffffffu, rare)) {
        for (int c = 0; c < nf; ++c) {
          double* out = vals + __ldg(rowptr + nf * a + c);
          for (int k = lane; k < width; k += 32) out[k] = (double)row[c * width + k];
        }
        if (f && lane < nf) f[nf * a + lane] = (double)fr;
      }
    }
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
