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

// ExtremeValue: lanes on the cubature points form u(q) = sum_b N_b(q) u_b;
// each cell's extreme and the CTA's best (value, key) go to one partial, key
// = block << 48 | cell << 6 | point, so that among equal values the lowest
// (block, cell, point) wins whatever the traversal order.
__device__ __forceinline__ bool extreme_better(double v1, int64_t k1, double v2, int64_t k2, bool use_max) {
  if (k2 < 0) return k1 >= 0;
  if (k1 < 0) return false;
  if (v1 != v2) return use_max ? v1 > v2 : v1 < v2;
  return k1 < k2;
}

__global__ void __launch_bounds__(32 * kRespWarps)
k_response_extreme(const BlockView B, int nq, const double* __restrict__ x, int nf, int field, int use_max,
                   int64_t blk_key, double* __restrict__ pval, int64_t* __restrict__ pidx) {
  __shared__ double sv[kRespWarps];
  __shared__ int64_t sk[kRespWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nb = B.nb;
  const double* val = B.ref + nq + (size_t)nq * B.nv + (size_t)nq * B.nv * 3;  // val [q][b]
  double best = 0.0;
  int64_t bkey = -1;
  const int64_t nwarps = (int64_t)gridDim.x * kRespWarps;
  for (int64_t e = (int64_t)blockIdx.x * kRespWarps + wid; e < B.n_elem; e += nwarps) {  // warp-uniform
    for (int q0 = 0; q0 < nq; q0 += 32) {
      const int q = q0 + lane;
      double u = 0.0;
      int64_t k = -1;
      if (q < nq) {
        for (int b = 0; b < nb; ++b)
          u += val[q * nb + b] * __ldg(x + (int64_t)nf * __ldg(B.dconn + e * nb + b) + field);
        k = (blk_key << 48) | (e << 6) | q;
      }
      if (extreme_better(u, k, best, bkey, use_max != 0)) { best = u; bkey = k; }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, best, o);
    const int64_t ok = __shfl_xor_sync(0xffffffffu, bkey, o);
    if (extreme_better(ov, ok, best, bkey, use_max != 0)) { best = ov; bkey = ok; }
  }
  if (lane == 0) { sv[wid] = best; sk[wid] = bkey; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kRespWarps; ++k)
      if (extreme_better(sv[k], sk[k], best, bkey, use_max != 0)) { best = sv[k]; bkey = sk[k]; }
    pval[blockIdx.x] = best;
    pidx[blockIdx.x] = bkey;
  }
}

// the winner over all partials, in index order
__global__ void k_response_extreme_final(const double* __restrict__ pval, const int64_t* __restrict__ pidx,
                                         int64_t n, int use_max, double* __restrict__ value,
                                         int64_t* __restrict__ winner) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double best = 0.0;
    int64_t bkey = -1;
    for (int64_t i = 0; i < n; ++i)
      if (extreme_better(pval[i], pidx[i], best, bkey, use_max != 0)) { best = pval[i]; bkey = pidx[i]; }
    *value = best;
    *winner = bkey;
  }
}

// dgdx += N_b(q*) at the winning cell's field DOFs, when the winner is in this block
__global__ void k_response_extreme_grad(const BlockView B, int nq, int64_t blk_key, const int64_t* __restrict__ winner,
                                        int nf, int field, double* __restrict__ dgdx) {
  const int64_t w = *winner;
  if (w < 0 || (w >> 48) != blk_key) return;
  const int64_t e = (w >> 6) & ((int64_t(1) << 42) - 1);
  const int q = (int)(w & 63);
  const double* val = B.ref + nq + (size_t)nq * B.nv + (size_t)nq * B.nv * 3;
  for (int b = threadIdx.x; b < B.nb; b += blockDim.x)
    dgdx[(int64_t)nf * __ldg(B.dconn + e * B.nb + b) + field] += val[q * B.nb + b];
}

// Integral of the field over a side workset: one warp per side (the side
// measure as in the Neumann flux), lanes on the side points form u(q); each
// CTA writes one partial; the gradient adds N_b w |J t_u x J t_v|.
__global__ void __launch_bounds__(32 * kRespWarps)
k_response_side(const BlockView B, const double* __restrict__ coords, const int64_t* __restrict__ sides, int64_t n,
                const double* __restrict__ tables, int stride, int nqf, const double* __restrict__ x, int nf,
                int field, double* __restrict__ partial, double* __restrict__ dgdx) {
  __shared__ double swarp[kRespWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nv = B.nv, nb = B.nb;
  double acc = 0.0;
  const int64_t nwarps = (int64_t)gridDim.x * kRespWarps;
  for (int64_t i = (int64_t)blockIdx.x * kRespWarps + wid; i < n; i += nwarps) {  // warp-uniform
    const int64_t code = __ldg(sides + i);
    const int64_t e = code >> 3;
    const double* T = tables + (size_t)(code & 7) * stride;
    const double* Tg = T + nqf;
    const double* Tv = Tg + (size_t)nqf * nv * 3;
    const double* Tt = Tv + (size_t)nqf * nb;
    double m = 0.0, contrib = 0.0;
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
      double a[3], bt[3];
      for (int r = 0; r < 3; ++r) {
        a[r] = J[3 * r] * Tt[0] + J[3 * r + 1] * Tt[1] + J[3 * r + 2] * Tt[2];
        bt[r] = J[3 * r] * Tt[3] + J[3 * r + 1] * Tt[4] + J[3 * r + 2] * Tt[5];
      }
      const double c0 = a[1] * bt[2] - a[2] * bt[1], c1 = a[2] * bt[0] - a[0] * bt[2], c2 = a[0] * bt[1] - a[1] * bt[0];
      m = T[lane] * sqrt(c0 * c0 + c1 * c1 + c2 * c2);
      double u = 0.0;
      for (int b = 0; b < nb; ++b)
        u += Tv[lane * nb + b] * __ldg(x + (int64_t)nf * __ldg(B.dconn + e * nb + b) + field);
      contrib = u * m;
    }
    const double side = warp_sum(contrib);
    if (lane == 0) acc += side;
    if (dgdx) {
      double d = 0.0;
      for (int q = 0; q < nqf; ++q) {
        const double mq = __shfl_sync(0xffffffffu, m, q);
        if (lane < nb) d += Tv[q * nb + lane] * mq;
      }
      if (lane < nb) atomicAdd(dgdx + (int64_t)nf * __ldg(B.dconn + e * nb + lane) + field, d);
    }
  }
  if (lane == 0) swarp[wid] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kRespWarps; ++k) s += swarp[k];
    partial[blockIdx.x] = s;
  }
}

// Probe: value = sum_b N_b u(lid_b) in basis order; dgdx[lid_b] += N_b.
__global__ void k_response_probe(const int32_t* __restrict__ lids, const double* __restrict__ N, int nb,
                                 const double* __restrict__ x, double* __restrict__ value, double* __restrict__ dgdx) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double u = 0.0;
    for (int b = 0; b < nb; ++b) {
      u += N[b] * x[lids[b]];
      if (dgdx) dgdx[lids[b]] += N[b];
    }
    *value = u;
  }
}

// IPCoordinates: xyz[(e * nq + q) * 3 + r] = sum_v N^geo_v(q) X_v[r].
__global__ void k_ip_coordinates(const BlockView B, int nq, const double* __restrict__ coords,
                                 double* __restrict__ xyz) {
  const double* gval = B.ref + nq;  // geo_val [q][v]
  const int64_t n = B.n_elem * nq;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / nq;
    const int q = (int)(i - e * nq);
    double p[3] = {0, 0, 0};
    for (int v = 0; v < B.nv; ++v) {
      const int64_t node = __ldg(B.vconn + e * B.nv + v);
      const double g = gval[q * B.nv + v];
      for (int r = 0; r < 3; ++r) p[r] += g * __ldg(coords + 3 * node + r);
    }
    for (int r = 0; r < 3; ++r) xyz[3 * i + r] = p[r];
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

cudaError_t launch_response_extreme(const BlockView& B, int nq, const double* x, int nf, int field, bool use_max,
                                    int blk_key, double* pval, int64_t* pidx, cudaStream_t s) {
  if (nq > kMaxRespQ) return cudaErrorInvalidValue;
  k_response_extreme<<<response_grid(B.n_elem), 32 * kRespWarps, 0, s>>>(B, nq, x, nf, field, use_max ? 1 : 0,
                                                                           (int64_t)blk_key, pval, pidx);
  return cudaGetLastError();
}
cudaError_t launch_response_extreme_final(const double* pval, const int64_t* pidx, int64_t n, bool use_max,
                                          double* value, int64_t* winner, cudaStream_t s) {
  k_response_extreme_final<<<1, 32, 0, s>>>(pval, pidx, n, use_max ? 1 : 0, value, winner);
  return cudaGetLastError();
}
cudaError_t launch_response_extreme_grad(const BlockView& B, int nq, int blk_key, const int64_t* winner, int nf,
                                         int field, double* dgdx, cudaStream_t s) {
  k_response_extreme_grad<<<1, 32, 0, s>>>(B, nq, (int64_t)blk_key, winner, nf, field, dgdx);
  return cudaGetLastError();
}
cudaError_t launch_response_side(const BlockView& B, const double* coords, const int64_t* sides, int64_t n,
                                 const double* tables, int stride, int nqf, const double* x, int nf, int field,
                                 double* partial, double* dgdx, cudaStream_t s) {
  if (nqf > 32 || B.nb > 32) return cudaErrorInvalidValue;
  k_response_side<<<response_grid(n), 32 * kRespWarps, 0, s>>>(B, coords, sides, n, tables, stride, nqf, x, nf, field,
                                                                partial, dgdx);
  return cudaGetLastError();
}
cudaError_t launch_response_probe(const int32_t* lids, const double* N, int nb, const double* x, double* value,
                                  double* dgdx, cudaStream_t s) {
  k_response_probe<<<1, 32, 0, s>>>(lids, N, nb, x, value, dgdx);
  return cudaGetLastError();
}
cudaError_t launch_ip_coordinates(const BlockView& B, int nq, const double* coords, double* xyz, cudaStream_t s) {
  const int64_t n = B.n_elem * nq;
  if (n <= 0) return cudaSuccess;
  int64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  k_ip_coordinates<<<(unsigned)g, 256, 0, s>>>(B, nq, coords, xyz);
  return cudaGetLastError();
}

cudaError_t launch_response_sum(const double* partial, int64_t n, double* value, cudaStream_t s) {
  k_response_sum<<<1, 32, 0, s>>>(partial, n, value);
  return cudaGetLastError();
}

}  // namespace tx
