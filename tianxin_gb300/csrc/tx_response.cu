// tx_response.cu -- integral responses over element blocks.
//
// value = sum_cells sum_q integrand(q) * w_q * s * det J_q, s the sign of the
// cell's first det J (computeCellMeasure, the weighted measure TianXin's
// Response_Integral multiplies its integrand by: disc-fe/src/responses/
// TianXin_Response_Integral_impl.hpp:106-130), and the gradient of value with
// respect to the field's DOFs (panzer's functional response derivative,
// Panzer_ResponseScatterEvaluator_Functional_impl.hpp:143-171).
//
// One warp per cell: lanes on the cubature points build J, J^-1, u, grad u
// and the exact solution there, keep the point quantities in shared memory,
// and reduce the cell value with shuffles; lanes on the basis functions then
// form the cell gradient.  Each CTA writes one partial sum; a one-CTA kernel
// adds the partials in a fixed order, so a value has the same bits on every
// call.  FP64 throughout: a response is evaluated once per solve.
#include "tx_device.cuh"

namespace tx {
namespace {

constexpr int kRespWarps = 4;
constexpr int kMaxRespQ = 64;   // 4 x 4 x 4 Gauss points
constexpr int kPerQ = 14;       // wm, e, de[3], Jinv[9]

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(32 * kRespWarps)
k_response(const BlockView B, int nq, const double* __restrict__ coords, const double* __restrict__ x, int nf,
           int field, int integrand, double* __restrict__ partial, double* __restrict__ dgdx) {
  __shared__ double sq[kRespWarps][kMaxRespQ][kPerQ];
  __shared__ double swarp[kRespWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nv = B.nv, nb = B.nb;
  const double* w = B.ref;
  const double* gval = w + nq;                         // geo_val [q][v]
  const double* ggrad = gval + (size_t)nq * nv;        // geo_grad [q][v][3]
  const double* val = ggrad + (size_t)nq * nv * 3;     // val [q][b]
  const double* grad = val + (size_t)nq * nb;          // grad [q][b][3]
  const double pi = 3.14159265358979323846;
  double acc = 0.0;
  const int64_t nwarps = (int64_t)gridDim.x * kRespWarps;
  for (int64_t e = (int64_t)blockIdx.x * kRespWarps + wid; e < B.n_elem; e += nwarps) {  // warp-uniform
    double cell = 0.0, sgn = 1.0;
    for (int q0 = 0; q0 < nq; q0 += 32) {
      const int q = q0 + lane;
      double contrib = 0.0, det = 0.0;
      if (q < nq) {
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, xq[3] = {0, 0, 0};
        for (int v = 0; v < nv; ++v) {
          const int64_t node = __ldg(B.vconn + e * nv + v);
          const double* g = ggrad + (q * nv + v) * 3;
          const double gv = gval[q * nv + v];
          for (int r = 0; r < 3; ++r) {
            const double xr = __ldg(coords + 3 * node + r);
            xq[r] += gv * xr;
            for (int c = 0; c < 3; ++c) J[3 * r + c] += xr * g[c];
          }
        }
        const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8], c02 = J[3] * J[7] - J[4] * J[6];
        det = J[0] * c00 + J[1] * c01 + J[2] * c02;
        double Ji[9];
        Ji[0] = c00 / det; Ji[1] = (J[2] * J[7] - J[1] * J[8]) / det; Ji[2] = (J[1] * J[5] - J[2] * J[4]) / det;
        Ji[3] = c01 / det; Ji[4] = (J[0] * J[8] - J[2] * J[6]) / det; Ji[5] = (J[2] * J[3] - J[0] * J[5]) / det;
        Ji[6] = c02 / det; Ji[7] = (J[1] * J[6] - J[0] * J[7]) / det; Ji[8] = (J[0] * J[4] - J[1] * J[3]) / det;
        double u = 0.0, gr[3] = {0, 0, 0};
        for (int b = 0; b < nb; ++b) {
          const double ub = __ldg(x + (int64_t)nf * __ldg(B.dconn + e * nb + b) + field);
          u += val[q * nb + b] * ub;
          for (int c = 0; c < 3; ++c) gr[c] += grad[(q * nb + b) * 3 + c] * ub;
        }
        double gu[3];  // grad u = J^-T grad^ u
        for (int i = 0; i < 3; ++i) gu[i] = Ji[i] * gr[0] + Ji[3 + i] * gr[1] + Ji[6 + i] * gr[2];
        double ev = u, de[3] = {0, 0, 0};
        if (integrand != TX_INTEGRAND_FIELD) {
          const double sx = sin(pi * xq[0]), sy = sin(pi * xq[1]), sz = sin(pi * xq[2]);
          const double cx = cos(pi * xq[0]), cy = cos(pi * xq[1]), cz = cos(pi * xq[2]);
          ev = u - sx * sy * sz;
          if (integrand == TX_INTEGRAND_H1_ERROR) {
            de[0] = gu[0] - pi * cx * sy * sz;
            de[1] = gu[1] - pi * sx * cy * sz;
            de[2] = gu[2] - pi * sx * sy * cz;
          }
        }
        double integ = integrand == TX_INTEGRAND_FIELD ? ev : ev * ev;
        if (integrand == TX_INTEGRAND_H1_ERROR) integ += de[0] * de[0] + de[1] * de[1] + de[2] * de[2];
        double* P = sq[wid][q];
        P[0] = w[q] * det;  // the sign is applied below
        P[1] = ev;
        for (int c = 0; c < 3; ++c) P[2 + c] = de[c];
        for (int k = 0; k < 9; ++k) P[5 + k] = Ji[k];
        contrib = integ * P[0];
      }
      if (q0 == 0) sgn = __shfl_sync(0xffffffffu, det, 0) < 0.0 ? -1.0 : 1.0;
      cell += warp_sum(contrib);
    }
    cell *= sgn;
    if (lane == 0) acc += cell;
    __syncwarp();
    if (dgdx) {
      for (int b = lane; b < nb; b += 32) {
        double d = 0.0;
        for (int q = 0; q < nq; ++q) {
          const double* P = sq[wid][q];
          const double wm = sgn * P[0];
          const double N = val[q * nb + b];
          if (integrand == TX_INTEGRAND_FIELD) {
            d += N * wm;
          } else {
            double t = 2.0 * P[1] * N;
            if (integrand == TX_INTEGRAND_H1_ERROR) {
              const double* g = grad + (q * nb + b) * 3;
              const double* Ji = P + 5;
              for (int i = 0; i < 3; ++i)
                t += 2.0 * P[2 + i] * (Ji[i] * g[0] + Ji[3 + i] * g[1] + Ji[6 + i] * g[2]);
            }
            d += t * wm;
          }
        }
        atomicAdd(dgdx + (int64_t)nf * __ldg(B.dconn + e * nb + b) + field, d);
      }
    }
    __syncwarp();
  }
  if (lane == 0) swarp[wid] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kRespWarps; ++k) s += swarp[k];
    partial[blockIdx.x] = s;
  }
}

// value = sum of n partials in index order
__global__ void k_response_sum(const double* __restrict__ partial, int64_t n, double* __restrict__ value) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += partial[i];
    *value = s;
  }
}

}  // namespace

int response_grid(int64_t n_elem) {
  const int64_t need = (n_elem + kRespWarps - 1) / kRespWarps;
  return (int)(need < kResponseCtas ? (need > 0 ? need : 1) : kResponseCtas);
}

cudaError_t launch_response(const BlockView& B, int nq, const double* coords, const double* x, int nf, int field,
                            int integrand, double* partial, double* dgdx, cudaStream_t s) {
  if (nq > kMaxRespQ || B.nb > 32) return cudaErrorInvalidValue;
  k_response<<<response_grid(B.n_elem), 32 * kRespWarps, 0, s>>>(B, nq, coords, x, nf, field, integrand, partial,
                                                                   dgdx);
  return cudaGetLastError();
}

cudaError_t launch_response_sum(const double* partial, int64_t n, double* value, cudaStream_t s) {
  k_response_sum<<<1, 32, 0, s>>>(partial, n, value);
  return cudaGetLastError();
}

}  // namespace tx
