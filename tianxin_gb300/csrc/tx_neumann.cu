// tx_neumann.cu -- Neumann flux on a side workset (TianXin::Flux).
//
// The reference evaluates a "Flux" Neumann condition as
//   residual(cell, b) = sum_q val * weighted_basis_scalar(cell, b, q)
// (disc-fe/src/evaluators/TianXin_Neumann_impl.hpp:146-166) on a side
// workset whose integration values are the side rule mapped into the cell:
// weighted_measure = w_q * |J t_u x J t_v| (the face measure), and
// weighted_basis_scalar = N_b(xi_q) * weighted_measure.  The Scatter then
// sums the row into f at the field's LIDs.
//
// One warp per side: lanes on the side points form J from the cell's vertex
// coordinates and the measure; lanes on the basis functions then reduce
// their row over the points (the measures are read with shuffles) and add
// it to f.  Boundary work grows with the surface, so this runs in FP64.
#include "tx_device.cuh"

namespace tx {
namespace {

constexpr int kNeumannThreads = 128;

__global__ void __launch_bounds__(kNeumannThreads)
k_neumann(const BlockView B, const double* __restrict__ coords, const int64_t* __restrict__ sides, int64_t n,
          const double* __restrict__ tables, int stride, int nqf, int nf, int field, double val,
          double* __restrict__ f) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int nv = B.nv, nb = B.nb;
  for (int64_t i = warp; i < n; i += nwarps) {  // warp-uniform: whole warps take a side
    const int64_t code = __ldg(sides + i);
    const int64_t e = code >> 3;
    const double* T = tables + (size_t)(code & 7) * stride;
    const double* Tg = T + nqf;                 // geo_grad [q][v][3]
    const double* Tv = Tg + (size_t)nqf * nv * 3;  // val [q][b]
    const double* Tt = Tv + (size_t)nqf * nb;      // t_u, t_v
    double m = 0.0;
    if (lane < nqf) {
      double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int v = 0; v < nv; ++v) {
        const int64_t node = __ldg(B.vconn + e * nv + v);
        const double* g = Tg + (lane * nv + v) * 3;
        for (int r = 0; r < 3; ++r) {
          const double xr = __ldg(coords + 3 * node + r);
          for (int c = 0; c < 3; ++c) J[3 * r + c] += xr * g[c];
        }
      }
      double a[3], b[3];
      for (int r = 0; r < 3; ++r) {
        a[r] = J[3 * r] * Tt[0] + J[3 * r + 1] * Tt[1] + J[3 * r + 2] * Tt[2];
        b[r] = J[3 * r] * Tt[3] + J[3 * r + 1] * Tt[4] + J[3 * r + 2] * Tt[5];
      }
      const double c0 = a[1] * b[2] - a[2] * b[1];
      const double c1 = a[2] * b[0] - a[0] * b[2];
      const double c2 = a[0] * b[1] - a[1] * b[0];
      m = T[lane] * sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    }
    double r = 0.0;
    for (int q = 0; q < nqf; ++q) {
      const double mq = __shfl_sync(0xffffffffu, m, q);
      if (lane < nb) r += val * (Tv[q * nb + lane] * mq);
    }
    if (lane < nb && r != 0.0) atomicAdd(f + (int64_t)nf * __ldg(B.dconn + e * nb + lane) + field, r);
  }
}

}  // namespace

cudaError_t launch_neumann(const BlockView& B, const double* coords, const int64_t* sides, int64_t n_sides,
                           const double* tables, int stride, int nqf, int nf, int field, double val, double* f,
                           cudaStream_t s) {
  if (n_sides <= 0) return cudaSuccess;
  if (nqf > 32 || B.nb > 32) return cudaErrorInvalidValue;
  const int64_t per_block = kNeumannThreads / 32;
  int64_t blocks = (n_sides + per_block - 1) / per_block;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_neumann<<<(unsigned)blocks, kNeumannThreads, 0, s>>>(B, coords, sides, n_sides, tables, stride, nqf, nf, field,
                                                         val, f);
  return cudaGetLastError();
}

}  // namespace tx
