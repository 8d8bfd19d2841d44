// tx_assemble_wpe.cu -- warp-per-element mixed assembly for hex8 elasticity.
//
// The same element arithmetic as k_assemble (GatherSolution -> IntegrationValues2 /
// BasisValues2 -> GradBasisDotVector with the stress closure + the mass term ->
// ScatterResidual / ScatterJacobian), laid out for occupancy: a warp owns one
// element at a time and synchronises only with itself, its working set is a few
// kB of shared memory, and the 64 (a, b) block pairs of the element Jacobian are
// spread over the lanes (two each), so no thread holds a whole block-row in
// registers.  Many more warps stay resident per SM than in the CTA-wide kernel,
// which is issue- and latency-bound.
//
// Per element (lane l):
//   gather   l < 24: vertex coordinate differences (FP64, narrowed), DOF values,
//            row starts; l < 16: the element's 64 epos bytes as words
//   geometry l < 8: J, J^-1, w det at point l; then all lanes: the 64 physical
//            (grad N, N) 4-vectors
//   fluxes   l < 8: displacement gradient -> stress, inertia minus body force
//   residual l < 24: row (a, c), summed into f
//   Jacobian pairs p = l, l + 32: K_ab (3 x 3) staged in shared memory
//   scatter  row by row, lanes on the 24 columns: one red.global.add.f64
//            instruction per CRS row segment.
#include "tx_device.cuh"
#include "tx_numeric.cuh"

namespace tx {
namespace {

constexpr int kWarps = 4;          // warps (elements in flight) per CTA
constexpr int NV = 8, NB = 8, NQ = 8, NF = 3, NE = 24, KRS = 25;
constexpr int GQS = NB * 4 + 4;    // floats per point in the (grad N, N) table

struct WarpSmem {
  float g[NQ * GQS];               // (gx, gy, gz, N) per point and basis
  float wg[NQ * GQS];              // the same times the weighted measure
  float k[NE * KRS];               // staged element Jacobian rows
  float ji[NQ * 9];                // J^-1 per point
  float qf[NQ * 9];                // stress (6) and inertia minus body force (3)
  float dx[NV * 3];                // vertex coordinates minus vertex 0
  float u[NF * NB], ud[NF * NB];   // DOF values [c][b]
  float w[NQ];                     // weighted measure
  long long rp[NE];                // CRS row starts of the element rows
  unsigned int ep[NB * NB / 4];    // epos bytes
  int la[NB];                      // entity LIDs
};

struct RefSmem {
  float w[NQ];
  float geo_grad[NQ * NV * 3];
  float val[NQ * NB];
  float grad[NQ * NB * 3];
};

// Eight resident CTAs (32 warps per SM): at most 64 registers a thread.
template <bool JAC>
__global__ void __launch_bounds__(32 * kWarps, 8)
k_assemble_wpe(const BlockView B, const EvalParams P, int64_t e_lo, int64_t e_hi) {
  __shared__ __align__(16) WarpSmem wsm[kWarps];
  __shared__ RefSmem ref;
  {
    const double* r = B.ref;  // [w | geo_val | geo_grad | val | grad]
    // integer narrowing keeps these conversions off the FP64 pipe
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) ref.w[i] = narrow(r[i]);
    r += NQ + NQ * NV;
    for (int i = threadIdx.x; i < NQ * NV * 3; i += blockDim.x) ref.geo_grad[i] = narrow(r[i]);
    r += NQ * NV * 3;
    for (int i = threadIdx.x; i < NQ * NB; i += blockDim.x) ref.val[i] = narrow(r[i]);
    r += NQ * NB;
    for (int i = threadIdx.x; i < NQ * NB * 3; i += blockDim.x) ref.grad[i] = narrow(r[i]);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  WarpSmem& S = wsm[threadIdx.x >> 5];
  const float lam = narrow(P.lam), mu = narrow(P.mu), beta = narrow(P.beta), alpha = narrow(P.alpha);
  const float rho = narrow(P.p[5]);
  const float bf[3] = {narrow(P.p[2]), narrow(P.p[3]), narrow(P.p[4])};
  const int64_t stride = (int64_t)gridDim.x * kWarps;
  for (int64_t e = e_lo + (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5); e < e_hi; e += stride) {
    // ------------------------------------------------------------ gather
    if (lane < 24) {
      const int v = lane / 3, d = lane - (lane / 3) * 3;
      const int64_t n = __ldg(B.vconn + e * NV + v), n0 = __ldg(B.vconn + e * NV);
      S.dx[lane] = narrow(__ldg(P.coords + 3 * n + d) - __ldg(P.coords + 3 * n0 + d));
      const int b = v, c = d;  // the same lane also gathers DOF (b, c)
      const int64_t ent = __ldg(B.dconn + e * NB + b);
      S.u[c * NB + b] = narrow(__ldg(P.x + NF * ent + c));
      S.ud[c * NB + b] = P.xdot ? narrow(__ldg(P.xdot + NF * ent + c)) : 0.0f;
      if (c == 0) S.la[b] = (int)ent;
      if (JAC) S.rp[lane] = __ldg(P.rowptr + NF * ent + c);
    }
    if (JAC && lane < 16) S.ep[lane] = __ldg(reinterpret_cast<const unsigned int*>(B.epos + e * NB * NB) + lane);
    __syncwarp();
    // ---------------------------------------------------------- geometry
    float det = 0.0f;
    if (lane < NQ) {
      const int q = lane;
      float J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float x0 = S.dx[3 * v], x1 = S.dx[3 * v + 1], x2 = S.dx[3 * v + 2];
        const float* g = ref.geo_grad + (q * NV + v) * 3;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          J[j] += x0 * g[j];
          J[3 + j] += x1 * g[j];
          J[6 + j] += x2 * g[j];
        }
      }
      const float c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8], c02 = J[3] * J[7] - J[4] * J[6];
      det = J[0] * c00 + J[1] * c01 + J[2] * c02;
      const float id = 1.0f / det;
      float* ji = S.ji + 9 * q;
      ji[0] = c00 * id; ji[1] = (J[2] * J[7] - J[1] * J[8]) * id; ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
      ji[3] = c01 * id; ji[4] = (J[0] * J[8] - J[2] * J[6]) * id; ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
      ji[6] = c02 * id; ji[7] = (J[1] * J[6] - J[0] * J[7]) * id; ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
    }
    // computeCellMeasure: |.| by the sign of the first point's det
    const float sgn = __shfl_sync(0xffffffffu, det, 0) < 0.0f ? -1.0f : 1.0f;
    if (lane < NQ) S.w[lane] = ref.w[lane] * det * sgn;
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int it = lane + 32 * k, q = it >> 3, b = it & 7;
      const float* ji = S.ji + 9 * q;
      const float* gr = ref.grad + (q * NB + b) * 3;
      const float g0 = gr[0], g1 = gr[1], g2 = gr[2];
      const float px = ji[0] * g0 + ji[3] * g1 + ji[6] * g2, py = ji[1] * g0 + ji[4] * g1 + ji[7] * g2;
      const float pz = ji[2] * g0 + ji[5] * g1 + ji[8] * g2, nv = ref.val[q * NB + b];
      const float wq = S.w[q];
      st4(S.g + q * GQS + b * 4, px, py, pz, nv);
      st4(S.wg + q * GQS + b * 4, wq * px, wq * py, wq * pz, wq * nv);
    }
    __syncwarp();
    // ------------------------------------------------------- point fluxes
    if (lane < NQ) {
      const int q = lane;
      float Gu[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, acc[3] = {0, 0, 0};
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        const R4<float> gb = ld4(S.g + q * GQS + b * 4);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float ub = S.u[c * NB + b];
          Gu[3 * c] += gb.x * ub;
          Gu[3 * c + 1] += gb.y * ub;
          Gu[3 * c + 2] += gb.z * ub;
          acc[c] += gb.w * S.ud[c * NB + b];
        }
      }
      const float tr = Gu[0] + Gu[4] + Gu[8];
      float* qf = S.qf + 9 * q;
      qf[0] = mu * (Gu[0] + Gu[0]) + lam * tr;
      qf[1] = mu * (Gu[4] + Gu[4]) + lam * tr;
      qf[2] = mu * (Gu[8] + Gu[8]) + lam * tr;
      qf[3] = mu * (Gu[1] + Gu[3]);
      qf[4] = mu * (Gu[2] + Gu[6]);
      qf[5] = mu * (Gu[5] + Gu[7]);
      qf[6] = rho * acc[0] - bf[0];
      qf[7] = rho * acc[1] - bf[1];
      qf[8] = rho * acc[2] - bf[2];
    }
    __syncwarp();
    // ---------------------------------------------------------- residual
    if (P.f && lane < NE) {
      const int a = lane / 3, c = lane - (lane / 3) * 3;
      // stress row c as (s_c0, s_c1, s_c2): symmetric storage 0 1 2 | 3=01 4=02 5=12
      const int i0 = c == 0 ? 0 : (c == 1 ? 3 : 4);
      const int i1 = c == 0 ? 3 : (c == 1 ? 1 : 5);
      const int i2 = c == 0 ? 4 : (c == 1 ? 5 : 2);
      float r = 0.0f;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const R4<float> wa = ld4(S.wg + q * GQS + a * 4);
        const float* qf = S.qf + 9 * q;
        r += wa.x * qf[i0] + wa.y * qf[i1] + wa.z * qf[i2] + wa.w * qf[6 + c];
      }
      atomicAdd(P.f + (int64_t)NF * S.la[a] + c, widen(r));
    }
    if constexpr (JAC) {
      // ------------------------------------------------- Jacobian pairs
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int p = lane + 32 * k, a = p >> 3, b = p & 7;
        float Pm[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, M = 0.0f;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const R4<float> wa = ld4(S.wg + q * GQS + a * 4);
          const R4<float> gb = ld4(S.g + q * GQS + b * 4);
          Pm[0] += wa.x * gb.x; Pm[1] += wa.x * gb.y; Pm[2] += wa.x * gb.z;
          Pm[3] += wa.y * gb.x; Pm[4] += wa.y * gb.y; Pm[5] += wa.y * gb.z;
          Pm[6] += wa.z * gb.x; Pm[7] += wa.z * gb.y; Pm[8] += wa.z * gb.z;
          M += wa.w * gb.w;
        }
        const float trP = Pm[0] + Pm[4] + Pm[8];
        const float diag = beta * mu * trP + alpha * rho * M;
        float* kr = S.k + (a * NF) * KRS + b * NF;
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int d = 0; d < 3; ++d)
            kr[c * KRS + d] = beta * (lam * Pm[3 * c + d] + mu * Pm[3 * d + c]) + (c == d ? diag : 0.0f);
      }
      __syncwarp();
      // ------------------------------------------------------- scatter
      if (lane < NE) {
        const int cb = lane / 3, cd = lane - (lane / 3) * 3;
        const unsigned char* ep = reinterpret_cast<const unsigned char*>(S.ep);
        double* vals = P.vals + cd;
#pragma unroll
        for (int r = 0; r < NE; ++r) {
          const int64_t addr = S.rp[r] + (int64_t)NF * ep[(r / NF) * NB + cb];
          atomicAdd(vals + addr, widen(S.k[r * KRS + lane]));
        }
      }
    }
    __syncwarp();
  }
}

template <bool JAC>
cudaError_t launch_jac(const BlockView& B, const EvalParams& P, int64_t e_lo, int64_t e_hi, cudaStream_t s,
                       int grid_cap) {
  static int per_sm = -1, sms = 0;
  if (per_sm < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_assemble_wpe<JAC>, 32 * kWarps, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
  }
  const int64_t n = e_hi - e_lo;
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + kWarps - 1) / kWarps;
  int64_t cap = (int64_t)per_sm * sms * 4;
  if (grid_cap > 0 && grid_cap < cap) cap = grid_cap;
  if (blocks > cap) blocks = cap;
  k_assemble_wpe<JAC><<<(unsigned)blocks, 32 * kWarps, 0, s>>>(B, P, e_lo, e_hi);
  return cudaGetLastError();
}

}  // namespace

bool wpe_supported(const BlockView& B, const EvalParams& P) {
  return B.topo == TX_TOPO_HEX && B.basis == TX_HGRAD_C1 && B.nq == NQ && P.physics == TX_PHYS_ELASTICITY &&
         P.tan == nullptr;
}

cudaError_t launch_assemble_wpe(const BlockView& B, const EvalParams& P, int64_t e_lo, int64_t e_hi, cudaStream_t s,
                                int grid_cap) {
  if (!wpe_supported(B, P)) return cudaErrorInvalidValue;
  return P.vals ? launch_jac<true>(B, P, e_lo, e_hi, s, grid_cap) : launch_jac<false>(B, P, e_lo, e_hi, s, grid_cap);
}

}  // namespace tx
