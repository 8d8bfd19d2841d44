// tx_assemble_body.cuh -- the fused volume assembly of one element (shared by
// the per-block kernels, tx_assemble.cu, and the persistent kernel,
// tx_assemble_batched.cu).
//
// One launch replaces the reference's per-workset evaluator chain
// (AssemblyEngine::evaluateVolume, disc-fe/src/Panzer_AssemblyEngine_impl.hpp:
// 134-182) for the Residual and Jacobian evaluation types:
//   GatherSolution_Tpetra      x, x_dot -> element values (LID gather)
//   IntegrationValues2         J, det J, J^-1, weighted measure
//   BasisValues2               grad N = J^-T grad N^, H(curl) J^-T / J/det
//   DOF / DOFGradient / DOFCurl values at the cubature points
//   Integrator_GradBasisDotVector, Integrator_BasisTimesScalar,
//   Integrator_CurlBasisDotVector (+ the mass terms on the time-derivative
//   vector)
//   ScatterResidual_Tpetra     f += r, A(row, cols) += dr/du
// The reference obtains dr/du by forward-mode AD (seed beta on x and alpha on
// x_dot in the same derivative slot); here the element matrices are the
// closed forms of those derivatives, so W = beta dR/dx + alpha dR/dx_dot.
//
// Work decomposition: TPE threads (next power of two >= basis count) per
// element, EPB elements per CTA, grid-stride over the block's elements.
// Phase 1 gathers vertex coordinates and DOF values, phase 2 builds the
// geometry and physical basis tables of each cubature point in shared
// memory, phase 3 evaluates the point fluxes, phase 4 gives each thread one
// basis function a: it forms residual row a and the Jacobian block-row
// (a, :) and scatters them with FP64 reductions at
//   rowptr[nf*entity(a)+c] + nf*epos[e][a][b] + d
// where epos is the precomputed position of entity b in the sorted row of
// entity a (the element-to-row map; no column search on the GPU).
//
// Real = double: the FP64 path.  Real = float (TX_EVAL_MIXED): element
// geometry and contractions in FP32 (vertex coordinates are differenced in
// FP64 first), accumulation into f and the CRS in FP64.
#pragma once
#include <cstdio>
#include <type_traits>

#include "tx_device.cuh"
#include "tx_numeric.cuh"

namespace tx {
namespace {

constexpr int pow2ceil(int n) { return n <= 4 ? 4 : n <= 8 ? 8 : n <= 16 ? 16 : 32; }

template <int TOPO, int BASIS>
struct Family;
template <> struct Family<TX_TOPO_HEX, TX_HGRAD_C1> { static constexpr int NV = 8, NB = 8; };
template <> struct Family<TX_TOPO_HEX, TX_HGRAD_C2> { static constexpr int NV = 8, NB = 27; };
template <> struct Family<TX_TOPO_TET, TX_HGRAD_C1> { static constexpr int NV = 4, NB = 4; };
template <> struct Family<TX_TOPO_TET, TX_HGRAD_C2> { static constexpr int NV = 4, NB = 10; };
template <> struct Family<TX_TOPO_HEX, TX_HCURL_I1> { static constexpr int NV = 8, NB = 12; };

constexpr size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

// STAGE_: element residual/Jacobian staged in shared memory, then scattered
// by the whole CTA with consecutive threads on consecutive entries of a CRS
// row (few L2 sectors per warp reduction) instead of one row per thread.
// GREF_: the persistent kernel's form, whose shared memory is sized for the
// largest family of the launch (hex27 tables in global memory: see RG).
template <int TOPO, int BASIS, int NQ, int PHYS, typename Real, int THREADS_ = (Family<TOPO, BASIS>::NB > 16 ? 128 : 256),
          bool STAGE_ = false, bool GREF_ = false>
struct Cfg {
  static constexpr int NV = Family<TOPO, BASIS>::NV;
  static constexpr int NB = Family<TOPO, BASIS>::NB;
  static constexpr bool HC = BASIS == TX_HCURL_I1;
  static constexpr int NF = PHYS == TX_PHYS_ELASTICITY ? 3 : 1;
  static constexpr int TPE = pow2ceil(NB);
  static constexpr int THREADS = THREADS_;
  static constexpr int EPB = THREADS / TPE;
  static constexpr int NQF = PHYS == TX_PHYS_ELASTICITY ? 9 : PHYS == TX_PHYS_HEAT ? 8 : PHYS == TX_PHYS_MAXWELL ? 6 : 4;
  static constexpr int NVAL = HC ? 3 : 1;
  // odd word strides: threads that write one row/point each spread over all banks
  // sG/sV: per point q and basis b one 4-vector (x, y, z, N) at q * GQS + b * 4;
  // GQS / 4 odd: the quarter-warp of a 128-bit access covers all banks
  static constexpr int GQS = NB * 4 + (NB % 2 == 0 ? 4 : 0);  // NB float4 slots, padded to an odd count
  static_assert((GQS / 4) % 2 == 1, "odd point stride in float4 slots");
  static constexpr int NE_ = (PHYS == TX_PHYS_ELASTICITY ? 3 : 1) * NB;
  static constexpr int KRS = NE_ | 1;       // sK:    [row * KRS + col]
  // hex27 (27 basis functions at 27 points) in the persistent kernel: the
  // reference tables and the element's epos stay in global memory (read
  // through L1), so that a CTA's shared memory (four elements' point tables,
  // 54 KB) lets four CTAs share an SM, for the hex27 items and for the other
  // families' items of the same launch.  (The per-block kernel keeps them in
  // shared memory: at three CTAs an SM its L1 holds more of the gathers.)
  static constexpr bool RG = GREF_ && NB > 16;
  // shared: reference part (geometry values only where sources need absolute coordinates)
  static constexpr size_t R_GEO_GRAD = 0;
  static constexpr size_t R_GEO_VAL = align16(R_GEO_GRAD + (RG ? 0 : sizeof(Real) * NQ * NV * 3));
  static constexpr size_t R_W =
      align16(R_GEO_VAL + (RG && PHYS != TX_PHYS_POISSON ? 0 : sizeof(double) * NQ * NV));
  static constexpr size_t R_VAL = align16(R_W + sizeof(Real) * NQ);
  static constexpr size_t R_GRAD = align16(R_VAL + (RG ? 0 : sizeof(Real) * NQ * NB * NVAL));
  static constexpr size_t R_END = align16(R_GRAD + (RG ? 0 : sizeof(Real) * NQ * NB * 3));
  // shared: per element part
  static constexpr bool XABS = PHYS == TX_PHYS_POISSON;                // sources need absolute coordinates
  static constexpr size_t E_X = 0;                                      // vertex coordinates (FP64)
  static constexpr size_t E_DX = align16(E_X + sizeof(double) * (XABS ? NV * 3 : 0));  // X[v] - X[0] (Real)
  static constexpr size_t E_U = align16(E_DX + sizeof(Real) * NV * 3);
  static constexpr size_t E_UD = align16(E_U + sizeof(Real) * NF * NB);
  static constexpr size_t E_AUX = align16(E_UD + sizeof(Real) * NF * NB);
  static constexpr size_t E_SG = align16(E_AUX + sizeof(Real) * (HC ? NB : 0));
  static constexpr size_t E_G = align16(E_SG + sizeof(Real) * (HC ? NB : 0));
  static constexpr size_t E_V = align16(E_G + sizeof(Real) * NQ * GQS);
  static constexpr size_t E_W = align16(E_V + sizeof(Real) * (HC ? NQ * GQS : 0));
  static constexpr size_t E_QF = align16(E_W + sizeof(Real) * NQ);
  static constexpr size_t E_SIGN = align16(E_QF + sizeof(Real) * NQ * NQF);
  static constexpr bool STAGE = STAGE_;
  static constexpr int NE = NF * NB;  // element DOFs
  // The staged Jacobian reuses the point tables (sG .. sSign): it is written
  // from registers after every thread has finished reading them.
  static constexpr size_t E_WORK_END = align16(E_SIGN + sizeof(Real));
  static constexpr size_t E_K = E_G;
  static constexpr size_t E_K_END = align16(E_K + sizeof(Real) * (STAGE ? NE * KRS : 0));
  static constexpr size_t E_R = E_K_END > E_WORK_END ? E_K_END : E_WORK_END;
  static constexpr size_t E_RP = align16(E_R + sizeof(Real) * (STAGE ? NE : 0));
  static constexpr size_t E_LA = align16(E_RP + sizeof(int64_t) * (STAGE ? NE : 0));
  static constexpr size_t E_EP = align16(E_LA + sizeof(int32_t) * (STAGE ? NB : 0));
  // per-element stride = 32 B past a multiple of 128 B: the four elements of a
  // warp start 8 banks apart, so same-offset accesses do not conflict
  static constexpr size_t E_RAW = align16(E_EP + (STAGE && !RG ? NB * NB : 0));
  static constexpr size_t E_END = ((E_RAW + 127 - 32) / 128) * 128 + 32;
  static constexpr size_t SMEM = R_END + EPB * E_END;
};


template <typename Real>
__device__ __forceinline__ Real source_at(int kind, double c, double s0, const double ip[3]) {
  if (kind == TX_SOURCE_SINE) {
    const double pi = 3.14159265358979323846;
    return (Real)(3.0 * pi * pi * sin(pi * ip[0]) * sin(pi * ip[1]) * sin(pi * ip[2]));
  }
  if (kind == TX_SOURCE_AFFINE) return (Real)(c * (1.0 + ip[0] + 2.0 * ip[1] + 3.0 * ip[2]));
  return (Real)s0;
}

// Elements [e_lo, e_hi) of a block (through perm if given), element groups
// g = grp0, grp0 + grp_stride, ... of EPB elements each.  ATOMIC=false is
// the coloured (deterministic) scatter: no two elements processed by one
// launch share a row, so plain read-modify-write is race free.
template <int TOPO, int BASIS, int NQ, int PHYS, typename Real, bool JAC, bool ATOMIC, int THREADS,
          bool STAGE = false, bool TAN = false, bool SCR = false, bool GREF = false>
__device__ __forceinline__ void assemble_body(const BlockView& B, const EvalParams& P, const int32_t* perm,
                                              int64_t e_lo, int64_t e_hi, int64_t grp0, int64_t grp_stride,
                                              unsigned char* smem) {
  using C = Cfg<TOPO, BASIS, NQ, PHYS, Real, THREADS, STAGE, GREF>;
  constexpr int NV = C::NV, NB = C::NB, NF = C::NF, TPE = C::TPE, EPB = C::EPB, NQF = C::NQF, NE = C::NE;
  constexpr int GQS = C::GQS, KRS = C::KRS;
  constexpr bool HC = C::HC;
  Real* r_w = reinterpret_cast<Real*>(smem + C::R_W);
  double* r_geo_val = reinterpret_cast<double*>(smem + C::R_GEO_VAL);
  const Real* r_geo_grad;
  const Real* r_val;
  const Real* r_grad;
  if constexpr (C::RG) {
    // the packed tables in global memory, in the arithmetic's type
    const Real* g;
    if constexpr (sizeof(Real) == 4) g = reinterpret_cast<const Real*>(B.ref32);
    else g = reinterpret_cast<const Real*>(B.ref);
    r_geo_grad = g + NQ + NQ * NV;
    r_val = r_geo_grad + NQ * NV * 3;
    r_grad = r_val + NQ * NB * C::NVAL;
  } else {
    r_geo_grad = reinterpret_cast<const Real*>(smem + C::R_GEO_GRAD);
    r_val = reinterpret_cast<const Real*>(smem + C::R_VAL);
    r_grad = reinterpret_cast<const Real*>(smem + C::R_GRAD);
  }

  // reference tables: [w | geo_val | geo_grad | val | grad] in FP64
  {
    const double* ref = B.ref;
    // FP32 copies by integer narrowing (off the FP64 pipe)
    for (int i = threadIdx.x; i < NQ; i += blockDim.x) r_w[i] = to_real<Real>(ref[i]);
    ref += NQ;
    if constexpr (!C::RG || C::XABS)
      for (int i = threadIdx.x; i < NQ * NV; i += blockDim.x) r_geo_val[i] = ref[i];
    ref += NQ * NV;
    if constexpr (!C::RG) {
      Real* s_geo_grad = reinterpret_cast<Real*>(smem + C::R_GEO_GRAD);
      Real* s_val = reinterpret_cast<Real*>(smem + C::R_VAL);
      Real* s_grad = reinterpret_cast<Real*>(smem + C::R_GRAD);
      for (int i = threadIdx.x; i < NQ * NV * 3; i += blockDim.x) s_geo_grad[i] = to_real<Real>(ref[i]);
      ref += NQ * NV * 3;
      for (int i = threadIdx.x; i < NQ * NB * C::NVAL; i += blockDim.x) s_val[i] = to_real<Real>(ref[i]);
      ref += NQ * NB * C::NVAL;
      for (int i = threadIdx.x; i < NQ * NB * 3; i += blockDim.x) s_grad[i] = to_real<Real>(ref[i]);
    }
  }

  const int le = threadIdx.x / TPE;
  const int t = threadIdx.x % TPE;
  unsigned char* eb = smem + C::R_END + (size_t)le * C::E_END;
  double* sX = reinterpret_cast<double*>(eb + C::E_X);
  Real* sDX = reinterpret_cast<Real*>(eb + C::E_DX);
  Real* sU = reinterpret_cast<Real*>(eb + C::E_U);
  Real* sUD = reinterpret_cast<Real*>(eb + C::E_UD);
  Real* sAUX = reinterpret_cast<Real*>(eb + C::E_AUX);
  Real* sSG = reinterpret_cast<Real*>(eb + C::E_SG);
  Real* sG = reinterpret_cast<Real*>(eb + C::E_G);    // [q][b][3] grad (HGRAD) or curl (HCURL)
  Real* sV = reinterpret_cast<Real*>(eb + C::E_V);    // [q][b][3] HCURL values
  Real* sW = reinterpret_cast<Real*>(eb + C::E_W);
  Real* sQF = reinterpret_cast<Real*>(eb + C::E_QF);
  Real* sSign = reinterpret_cast<Real*>(eb + C::E_SIGN);
  Real* sK = reinterpret_cast<Real*>(eb + C::E_K);          // [a*NF+c][b*NF+d] staged Jacobian
  Real* sR = reinterpret_cast<Real*>(eb + C::E_R);          // [a*NF+c] staged residual
  int64_t* sRP = reinterpret_cast<int64_t*>(eb + C::E_RP);  // addresses of the rows' first values
  int32_t* sLA = reinterpret_cast<int32_t*>(eb + C::E_LA);  // entity LIDs
  uint8_t* sEP = reinterpret_cast<uint8_t*>(eb + C::E_EP);  // epos transposed: [b][a]
  __syncthreads();

  // parameters in the element arithmetic's type, once per thread
  Real pr[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) pr[i] = to_real<Real>(P.p[i]);
  const Real lam = to_real<Real>(P.lam), mu = to_real<Real>(P.mu);
  const Real beta = to_real<Real>(P.beta), alpha = to_real<Real>(P.alpha);
  for (int64_t g0 = e_lo + grp0 * EPB; g0 < e_hi; g0 += grp_stride * EPB) {
    const int64_t ei = g0 + le;
    const bool valid = ei < e_hi;
    const int64_t e = (perm && valid) ? (int64_t)__ldg(perm + ei) : ei;
    // ---------------------------------------------------------- 1 gather
    if (valid) {
      const int64_t n0 = __ldg(B.vconn + e * NV);
      for (int v = t; v < NV; v += TPE) {
        const int64_t n = __ldg(B.vconn + e * NV + v);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const double xv = __ldg(P.coords + 3 * n + d);
          if constexpr (C::XABS) sX[3 * v + d] = xv;
          // differencing in FP64, once per vertex, keeps the mixed J accurate
          sDX[3 * v + d] = to_real<Real>(xv - __ldg(P.coords + 3 * n0 + d));
        }
      }
      for (int b = t; b < NB; b += TPE) {
        const int64_t ent = __ldg(B.dconn + e * NB + b);
#pragma unroll
        for (int c = 0; c < NF; ++c) {
          sU[c * NB + b] = to_real<Real>(__ldg(P.x + NF * ent + c));
          sUD[c * NB + b] = P.xdot ? to_real<Real>(__ldg(P.xdot + NF * ent + c)) : Real(0);
        }
        if constexpr (HC) {
          sAUX[b] = P.aux ? to_real<Real>(__ldg(P.aux + ent)) : Real(0);
          sSG[b] = (Real)__ldg(B.esign + e * NB + b);
        }
        if constexpr (STAGE) {
          sLA[b] = (int32_t)ent;
          if constexpr (JAC) {
            // row starts as final addresses into the CRS values; epos transposed so
            // that the scatter's lane (column block k) finds its row positions together
#pragma unroll
            for (int c = 0; c < NF; ++c) sRP[b * NF + c] = (int64_t)(P.vals + __ldg(P.rowptr + NF * ent + c));
            if constexpr (!C::RG)
              for (int k = 0; k < NB; ++k) sEP[k * NB + b] = __ldg(B.epos + (e * NB + b) * NB + k);
          }
        }
      }
    }
    __syncthreads();
    // ---------------------------------------------------------- 2 geometry
    if (valid) {
      for (int q = t; q < NQ; q += TPE) {
        Real J[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) J[k] = Real(0);
#pragma unroll
        for (int v = 1; v < NV; ++v) {  // X[0] - X[0] = 0: vertex 0 adds nothing
          const Real dx = sDX[3 * v + 0], dy = sDX[3 * v + 1], dz = sDX[3 * v + 2];
          const Real* gg = r_geo_grad + (q * NV + v) * 3;
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const Real g = gg[j];
            J[0 + j] += dx * g;
            J[3 + j] += dy * g;
            J[6 + j] += dz * g;
          }
        }
        const Real c00 = J[4] * J[8] - J[5] * J[7];
        const Real c01 = J[5] * J[6] - J[3] * J[8];
        const Real c02 = J[3] * J[7] - J[4] * J[6];
        const Real det = J[0] * c00 + J[1] * c01 + J[2] * c02;
        const Real id = Real(1) / det;
        Real Ji[9];
        Ji[0] = c00 * id; Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id; Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
        Ji[3] = c01 * id; Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id; Ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
        Ji[6] = c02 * id; Ji[7] = (J[1] * J[6] - J[0] * J[7]) * id; Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
        sW[q] = r_w[q] * det;
        if (q == 0) *sSign = det < Real(0) ? Real(-1) : Real(1);
#pragma unroll 4
        for (int b = 0; b < NB; ++b) {
          const Real* gr = r_grad + (q * NB + b) * 3;
          const Real g0 = gr[0], g1 = gr[1], g2 = gr[2];
          if constexpr (!HC) {
            // grad_i = sum_j Jinv(j,i) grad^_j
            st4(sG + q * GQS + b * 4, Ji[0] * g0 + Ji[3] * g1 + Ji[6] * g2, Ji[1] * g0 + Ji[4] * g1 + Ji[7] * g2,
                Ji[2] * g0 + Ji[5] * g1 + Ji[8] * g2, r_val[q * NB + b]);
          } else {
            const Real s = sSG[b];
            const Real* vr = r_val + (q * NB + b) * 3;
            st4(sV + q * GQS + b * 4, s * (Ji[0] * vr[0] + Ji[3] * vr[1] + Ji[6] * vr[2]),
                s * (Ji[1] * vr[0] + Ji[4] * vr[1] + Ji[7] * vr[2]), s * (Ji[2] * vr[0] + Ji[5] * vr[1] + Ji[8] * vr[2]),
                Real(0));
            const Real sd = s * id;  // curl = J curl^ / det
            st4(sG + q * GQS + b * 4, sd * (J[0] * g0 + J[1] * g1 + J[2] * g2), sd * (J[3] * g0 + J[4] * g1 + J[5] * g2),
                sd * (J[6] * g0 + J[7] * g1 + J[8] * g2), Real(0));
          }
        }
      }
    }
    __syncthreads();
    // ---------------------------------------------------------- 3 point fluxes
    if (valid) {
      for (int q = t; q < NQ; q += TPE) {
        sW[q] *= *sSign;  // computeCellMeasure: |.| by the sign of the first point
        Real* qf = sQF + q * NQF;
        if constexpr (PHYS == TX_PHYS_POISSON || PHYS == TX_PHYS_HEAT) {
          Real u = 0, ud = 0, g[3] = {0, 0, 0};
          // the time derivative only when one is given (its values are zeros otherwise)
          auto values = [&](auto td) {
            for (int b = 0; b < NB; ++b) {
              const R4<Real> gq = ld4(sG + q * GQS + b * 4);
              const Real ub = sU[b];
              u += gq.w * ub;
              if constexpr (decltype(td)::value) ud += gq.w * sUD[b];
              g[0] += gq.x * ub;
              g[1] += gq.y * ub;
              g[2] += gq.z * ub;
            }
          };
          if (P.xdot) values(std::true_type{});
          else values(std::false_type{});
          if constexpr (PHYS == TX_PHYS_POISSON) {
            const Real k = pr[0], c = pr[1], m = pr[2];
            Real s = pr[3];
            if (P.source_kind != TX_SOURCE_CONST) {
              double ip[3] = {0, 0, 0};
              for (int v = 0; v < NV; ++v) {
                const double nv = r_geo_val[q * NV + v];
                ip[0] += nv * sX[3 * v]; ip[1] += nv * sX[3 * v + 1]; ip[2] += nv * sX[3 * v + 2];
              }
              s = source_at<Real>(P.source_kind, P.p[1], P.p[3], ip);
            }
            qf[0] = k * g[0]; qf[1] = k * g[1]; qf[2] = k * g[2];
            qf[3] = c * u + m * ud - s;
          } else {
            const Real k = pr[0] + pr[1] * u * u;
            const Real dk = Real(2) * pr[1] * u;
            qf[0] = k * g[0]; qf[1] = k * g[1]; qf[2] = k * g[2];
            qf[3] = -pr[2];
            qf[4] = dk * g[0]; qf[5] = dk * g[1]; qf[6] = dk * g[2];
            qf[7] = k;
          }
        } else if constexpr (PHYS == TX_PHYS_ELASTICITY) {
          Real Gu[9], acc[3] = {0, 0, 0};
#pragma unroll
          for (int k = 0; k < 9; ++k) Gu[k] = 0;
          // the acceleration only when a time derivative is given (its values are zeros otherwise)
          auto values = [&](auto td) {
            for (int b = 0; b < NB; ++b) {
              const R4<Real> gb = ld4(sG + q * GQS + b * 4);
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const Real ub = sU[c * NB + b];
                Gu[3 * c + 0] += gb.x * ub;
                Gu[3 * c + 1] += gb.y * ub;
                Gu[3 * c + 2] += gb.z * ub;
                if constexpr (decltype(td)::value) acc[c] += gb.w * sUD[c * NB + b];
              }
            }
          };
          if (P.xdot) values(std::true_type{});
          else values(std::false_type{});
          const Real tr = Gu[0] + Gu[4] + Gu[8];
          qf[0] = mu * (Gu[0] + Gu[0]) + lam * tr;  // s00
          qf[1] = mu * (Gu[4] + Gu[4]) + lam * tr;  // s11
          qf[2] = mu * (Gu[8] + Gu[8]) + lam * tr;  // s22
          qf[3] = mu * (Gu[1] + Gu[3]);             // s01
          qf[4] = mu * (Gu[2] + Gu[6]);             // s02
          qf[5] = mu * (Gu[5] + Gu[7]);             // s12
          const Real rho = pr[5];
          qf[6] = rho * acc[0] - pr[2];
          qf[7] = rho * acc[1] - pr[3];
          qf[8] = rho * acc[2] - pr[4];
        } else {  // MAXWELL
          Real Ev[3] = {0, 0, 0}, cE[3] = {0, 0, 0}, Jv[3] = {0, 0, 0};
          for (int b = 0; b < NB; ++b) {
            const Real ub = sU[b], jb = sAUX[b];
            const Real* vb = sV + q * GQS + b * 4;
            const Real* cb = sG + q * GQS + b * 4;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              Ev[i] += vb[i] * ub;
              Jv[i] += vb[i] * jb;
              cE[i] += cb[i] * ub;
            }
          }
          const Real imu = pr[0], sig = pr[1];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            qf[i] = imu * cE[i];
            qf[3 + i] = sig * Ev[i] - Jv[i];
          }
        }
      }
    }
    __syncthreads();
    // ---------------------------------------------------------- 4 rows + scatter
    // staged form: this thread's Jacobian block-row waits in registers until
    // every thread of the CTA has finished reading the point tables it reuses.
    // SYM (FP64): the element matrix of elasticity and of Poisson is
    // symmetric (K_ba = K_ab^T), so row a forms only the blocks of b = a,
    // a + 1, ..., a + NB / 2 (mod NB; the last one for a < NB / 2 only),
    // NB / 2 + 1 of NB, and the staging writes each block and its transpose.
    // The FP32 build forms every block, so that all its kernel forms (staged,
    // coloured, direct, warp per element) give the same element matrices bit
    // for bit; K_ab^T and a separately formed K_ba differ by rounding.
    constexpr bool SYM = sizeof(Real) == 8 && STAGE && JAC && !TAN && !SCR && NB % 2 == 0 &&
                         (((PHYS == TX_PHYS_ELASTICITY || PHYS == TX_PHYS_POISSON) && NQ <= 8 && !HC) ||
                          PHYS == TX_PHYS_MAXWELL);
    constexpr int NSLOT = SYM ? NB / 2 + 1 : NB;  // blocks a row forms
    // HSYM (FP64 heat): K_ab = S_ab + N_b . s_a with S_ab = sum_q k W grad
    // N_a . grad N_b symmetric and s_a(q) = W dk/dT grad T . grad N_a; row a
    // forms S for b = a, ..., a + NB / 2 (mod NB; for NB even the last one
    // for a < NB / 2 only: every pair once) and the N_b term for every
    // column (hex27: 69 instead of 108 FMAs a point; tet10: 12 x 6 + 4 x 10
    // instead of 16 x 10 an element row), and the staging adds each S entry
    // to both of its places.
    constexpr bool HSYM = sizeof(Real) == 8 && STAGE && JAC && !TAN && !SCR && PHYS == TX_PHYS_HEAT;
    constexpr int NSH = NB / 2 + 1;
    Real kreg[STAGE && JAC ? NF * NE : 1];
    Real ksym[HSYM ? NSH : 1];
    const int my_a = (valid && t < NB) ? t : -1;
    if (valid) {
      for (int a = t; a < NB; a += TPE) {
        const int64_t la = __ldg(B.dconn + e * NB + a);
        // The thread's own weighted gradient W_q grad N_a(q) and W_q N_a(q):
        // kept in registers for small rules, read from shared memory otherwise.
        constexpr bool CACHE = NQ <= 8 && !HC;
        Real wg[CACHE ? NQ : 1][3], wn[CACHE ? NQ : 1];
        if constexpr (CACHE) {
#pragma unroll
          for (int q = 0; q < NQ; ++q) {
            const Real w = sW[q];
            const R4<Real> ga = ld4(sG + q * GQS + a * 4);
            wg[q][0] = w * ga.x; wg[q][1] = w * ga.y; wg[q][2] = w * ga.z;
            wn[q] = w * ga.w;
          }
        }
        auto WG = [&](int q, int i) -> Real {
          if constexpr (CACHE) return wg[q][i];
          else return sW[q] * sG[q * GQS + a * 4 + i];
        };
        auto WN = [&](int q) -> Real {
          if constexpr (CACHE) return wn[q];
          else return sW[q] * sG[q * GQS + a * 4 + 3];
        };
        // residual row a (per field)
        Real r[NF];
#pragma unroll
        for (int c = 0; c < NF; ++c) r[c] = 0;
#pragma unroll(CACHE ? NQ : 1)
        for (int q = 0; q < NQ; ++q) {
          const Real* qf = sQF + q * NQF;
          if constexpr (PHYS == TX_PHYS_POISSON || PHYS == TX_PHYS_HEAT) {
            // FMA chains: four operations a point and row instead of five
            r[0] += WG(q, 0) * qf[0]; r[0] += WG(q, 1) * qf[1]; r[0] += WG(q, 2) * qf[2]; r[0] += WN(q) * qf[3];
          } else if constexpr (PHYS == TX_PHYS_ELASTICITY) {
            const Real g0 = WG(q, 0), g1 = WG(q, 1), g2 = WG(q, 2), n = WN(q);
            r[0] += g0 * qf[0]; r[0] += g1 * qf[3]; r[0] += g2 * qf[4]; r[0] += n * qf[6];
            r[1] += g0 * qf[3]; r[1] += g1 * qf[1]; r[1] += g2 * qf[5]; r[1] += n * qf[7];
            r[2] += g0 * qf[4]; r[2] += g1 * qf[5]; r[2] += g2 * qf[2]; r[2] += n * qf[8];
          } else {
            const Real w = sW[q];
            const Real* ga = sG + q * GQS + a * 4;
            const Real* va = sV + q * GQS + a * 4;
            r[0] += w * (ga[0] * qf[0] + ga[1] * qf[1] + ga[2] * qf[2] + va[0] * qf[3] + va[1] * qf[4] + va[2] * qf[5]);
          }
        }
        // heat Jacobian entries, k(T) W grad N_a . grad N_b + N_b W (dk/dT grad T . grad N_a): the row's point
        // factors (k(T) W grad N_a, W dk/dT grad T . grad N_a) formed once a point, so that an entry takes four
        // FMAs a point; in registers for small rules (the row's gradients are dead after the residual)
        constexpr bool HCACHE = CACHE && PHYS == TX_PHYS_HEAT;
        Real hq[HCACHE ? NQ : 1][4];
        if constexpr (HCACHE) {
#pragma unroll
          for (int q = 0; q < NQ; ++q) {
            const Real* qf = sQF + q * NQF;
            const Real g0 = WG(q, 0), g1 = WG(q, 1), g2 = WG(q, 2);
            hq[q][0] = qf[7] * g0; hq[q][1] = qf[7] * g1; hq[q][2] = qf[7] * g2;
            hq[q][3] = g0 * qf[4] + g1 * qf[5] + g2 * qf[6];
          }
        }
        auto HQ = [&](int q, int i) -> Real {
          if constexpr (HCACHE) return hq[q][i];
          else {
            const Real* qf = sQF + q * NQF;
            return i < 3 ? qf[7] * WG(q, i) : WG(q, 0) * qf[4] + WG(q, 1) * qf[5] + WG(q, 2) * qf[6];
          }
        };
        if constexpr (STAGE) {
          if constexpr (SCR) {  // two-phase: the element residual to scratch
#pragma unroll
            for (int c = 0; c < NF; ++c) reinterpret_cast<Real*>(P.rscr)[e * NE + a * NF + c] = r[c];
          } else {
#pragma unroll
            for (int c = 0; c < NF; ++c) sR[a * NF + c] = r[c];
          }
        } else if (P.f) {
#pragma unroll
          for (int c = 0; c < NF; ++c) accumulate<ATOMIC>(P.f + NF * la + c, widen(r[c]));
        }
        if constexpr (JAC) {
          int64_t rp[NF];
          const uint8_t* ep = B.epos + (e * NB + a) * NB;
          if constexpr (!STAGE && !TAN) {
#pragma unroll
            for (int c = 0; c < NF; ++c) rp[c] = __ldg(P.rowptr + NF * la + c);
          }
          // Tangent: the row's products with the tangent directions (GatherSolution<Tangent>
          // seeds dx(i) from them; ScatterResidual<Tangent> sums dx(i) into dfdp_i)
          double rt[TAN ? kMaxTangents : 1][TAN ? NF : 1];
          if constexpr (TAN) {
#pragma unroll
            for (int i = 0; i < kMaxTangents; ++i)
#pragma unroll
              for (int c = 0; c < NF; ++c) rt[i][c] = 0.0;
          }
          int64_t eb = 0;  // entity of column basis b (tangent gather)
          // Jacobian entry (row a,c; column b,d): reduce now, or stage for the CTA-wide scatter
          auto put = [&](int c, int b, int d, int64_t pb, Real v) {
            if constexpr (TAN) {
              for (int i = 0; i < P.ntan; ++i)
                rt[i][c] += (double)v * __ldg(P.tan + (int64_t)i * P.n + NF * eb + d);
            } else if constexpr (STAGE) {
              kreg[c * NE + b * NF + d] = v;
            } else {
              accumulate<ATOMIC>(P.vals + rp[c] + pb + d, widen(v));
            }
          };
          // Scalar physics whose point tables stay in shared memory (hex27: 27 x
          // 27 entries over 27 points; H(curl): 12 x 12 over 8): the point loop
          // outside, so the row's own weighted gradient (or curl and value) and
          // the point's flux factors are read once a point and the NB entries
          // of the row accumulate in registers (one or two broadcast loads and
          // four to eight FMAs an entry and point instead of about ten loads);
          // each entry's sum still runs over the points in order.
          constexpr bool QOUTER = !CACHE && (PHYS == TX_PHYS_POISSON || PHYS == TX_PHYS_HEAT || PHYS == TX_PHYS_MAXWELL);
          if constexpr (QOUTER) {
            // SYM (FP64 Maxwell): accumulator j holds the entry of b = a + j (mod NB), NB / 2 + 1 of them
            Real kg[NB], km[NB];
#pragma unroll
            for (int b = 0; b < NB; ++b) kg[b] = km[b] = Real(0);
            for (int q = 0; q < NQ; ++q) {
              if constexpr (PHYS == TX_PHYS_MAXWELL) {
                // curl-curl and mass entries: the row's curl and value at q read once
                const Real w = sW[q];
                const R4<Real> ca = ld4(sG + q * GQS + a * 4), va = ld4(sV + q * GQS + a * 4);
                const Real c0 = w * ca.x, c1 = w * ca.y, c2 = w * ca.z;
                const Real v0 = w * va.x, v1 = w * va.y, v2 = w * va.z;
#pragma unroll
                for (int b = 0; b < NSLOT; ++b) {
                  const int bc = SYM ? (a + b < NB ? a + b : a + b - NB) : b;
                  const R4<Real> cb = ld4(sG + q * GQS + bc * 4), vb = ld4(sV + q * GQS + bc * 4);
                  Real sc = kg[b], sv = km[b];
                  sc += c0 * cb.x; sc += c1 * cb.y; sc += c2 * cb.z;
                  sv += v0 * vb.x; sv += v1 * vb.y; sv += v2 * vb.z;
                  kg[b] = sc;
                  km[b] = sv;
                }
                continue;
              }
              const Real g0 = WG(q, 0), g1 = WG(q, 1), g2 = WG(q, 2);
              if constexpr (PHYS == TX_PHYS_HEAT) {
                // k(T) grad N_a . grad N_b + N_b (dk/dT grad T . grad N_a): the point's factors applied to the
                // row's gradient once, then four FMAs an entry
                const Real* qf = sQF + q * NQF;
                const Real k7 = qf[7], sa = g0 * qf[4] + g1 * qf[5] + g2 * qf[6];
                const Real h0 = k7 * g0, h1 = k7 * g1, h2 = k7 * g2;
                if constexpr (HSYM) {
                  // km[j]: S of b = a + j; kg[b]: the N_b term
#pragma unroll
                  for (int j = 0; j < NSH; ++j) {
                    const int bc = a + j < NB ? a + j : a + j - NB;
                    const R4<Real> gb = ld4(sG + q * GQS + bc * 4);
                    Real s = km[j];
                    s += h0 * gb.x; s += h1 * gb.y; s += h2 * gb.z;
                    km[j] = s;
                  }
#pragma unroll
                  for (int b = 0; b < NB; ++b) kg[b] += sa * sG[q * GQS + b * 4 + 3];
                } else {
#pragma unroll
                  for (int b = 0; b < NB; ++b) {
                    const R4<Real> gb = ld4(sG + q * GQS + b * 4);
                    Real s = kg[b];
                    s += h0 * gb.x; s += h1 * gb.y; s += h2 * gb.z; s += sa * gb.w;
                    kg[b] = s;
                  }
                }
              } else {
                const Real wn = WN(q);
#pragma unroll
                for (int b = 0; b < NB; ++b) {
                  const R4<Real> gb = ld4(sG + q * GQS + b * 4);
                  Real s = kg[b];
                  s += g0 * gb.x; s += g1 * gb.y; s += g2 * gb.z;
                  kg[b] = s;
                  km[b] += wn * gb.w;
                }
              }
            }
#pragma unroll
            for (int b = 0; b < NB; ++b) {
              if constexpr (SYM) {  // Maxwell: the formed entries, in accumulator order
                if (b < NSLOT) kreg[b] = beta * (pr[0] * kg[b] + pr[1] * km[b]);
                continue;
              }
              const int64_t pb = (STAGE || TAN) ? 0 : (int64_t)NF * __ldg(ep + b);
              if constexpr (TAN) eb = __ldg(B.dconn + e * NB + b);
              if constexpr (PHYS == TX_PHYS_HEAT) {
                put(0, b, 0, pb, beta * kg[b]);
                if constexpr (HSYM) {
                  if (b < NSH) ksym[b] = beta * km[b];
                }
              } else if constexpr (PHYS == TX_PHYS_MAXWELL) {
                put(0, b, 0, pb, beta * (pr[0] * kg[b] + pr[1] * km[b]));
              } else {
                put(0, b, 0, pb, (beta * pr[0]) * kg[b] + (beta * pr[1] + alpha * pr[2]) * km[b]);
              }
            }
          }
#pragma unroll(STAGE ? NSLOT : 1)
          for (int sl = 0; sl < (QOUTER ? 0 : NSLOT); ++sl) {
            if (SYM && sl == NB / 2 && a >= NB / 2) continue;  // the opposite block: formed by the lower row
            const int b = SYM ? (a + sl < NB ? a + sl : a + sl - NB) : sl;
            const int64_t pb = (STAGE || TAN) ? 0 : (int64_t)NF * __ldg(ep + b);
            if constexpr (TAN) eb = __ldg(B.dconn + e * NB + b);
            if constexpr (PHYS == TX_PHYS_POISSON) {
              const Real ca = beta * pr[0];
              const Real cm = beta * pr[1] + alpha * pr[2];
              Real kg = 0, km = 0;
#pragma unroll(CACHE ? NQ : 1)
              for (int q = 0; q < NQ; ++q) {
                const R4<Real> gb = ld4(sG + q * GQS + b * 4);
                kg += WG(q, 0) * gb.x; kg += WG(q, 1) * gb.y; kg += WG(q, 2) * gb.z;
                km += WN(q) * gb.w;
              }
              if constexpr (SYM) kreg[sl] = ca * kg + cm * km;
              else put(0, b, 0, pb, ca * kg + cm * km);
            } else if constexpr (PHYS == TX_PHYS_HEAT) {
              if constexpr (HSYM) {
                // the N_b term of every column; the rows' symmetric part once, with the first column
                Real kn = 0;
#pragma unroll(CACHE ? NQ : 1)
                for (int q = 0; q < NQ; ++q) kn += HQ(q, 3) * sG[q * GQS + b * 4 + 3];
                put(0, b, 0, pb, beta * kn);
                if (sl == 0) {
#pragma unroll
                  for (int j = 0; j < NSH; ++j) {
                    const int bc = a + j < NB ? a + j : a + j - NB;
                    Real ks = 0;
#pragma unroll(CACHE ? NQ : 1)
                    for (int q = 0; q < NQ; ++q) {
                      const R4<Real> gb = ld4(sG + q * GQS + bc * 4);
                      ks += HQ(q, 0) * gb.x; ks += HQ(q, 1) * gb.y; ks += HQ(q, 2) * gb.z;
                    }
                    ksym[j] = beta * ks;
                  }
                }
              } else {
                Real kab = 0;
#pragma unroll(CACHE ? NQ : 1)
                for (int q = 0; q < NQ; ++q) {
                  const R4<Real> gb = ld4(sG + q * GQS + b * 4);
                  kab += HQ(q, 0) * gb.x; kab += HQ(q, 1) * gb.y; kab += HQ(q, 2) * gb.z; kab += HQ(q, 3) * gb.w;
                }
                put(0, b, 0, pb, beta * kab);
              }
            } else if constexpr (PHYS == TX_PHYS_ELASTICITY) {
              Real Pm[9], M = 0;
#pragma unroll
              for (int k = 0; k < 9; ++k) Pm[k] = 0;
              // FP64: the mass entries only where they contribute (alpha rho != 0), one FMA in ten fewer on the
              // FP64 pipe otherwise (the 128^3 elasticity FP64 kernel 39.4 -> 35.7 ms with the folded coefficients
              // below); the FP32 build keeps one loop (two cost its staged kernel 2 %)
              auto contract = [&](auto with_mass) {
#pragma unroll(CACHE ? NQ : 1)
                for (int q = 0; q < NQ; ++q) {
                  const R4<Real> gb = ld4(sG + q * GQS + b * 4);
                  const Real b0 = gb.x, b1 = gb.y, b2 = gb.z;
                  const Real wa0 = WG(q, 0), wa1 = WG(q, 1), wa2 = WG(q, 2);
                  Pm[0] += wa0 * b0; Pm[1] += wa0 * b1; Pm[2] += wa0 * b2;
                  Pm[3] += wa1 * b0; Pm[4] += wa1 * b1; Pm[5] += wa1 * b2;
                  Pm[6] += wa2 * b0; Pm[7] += wa2 * b1; Pm[8] += wa2 * b2;
                  if constexpr (decltype(with_mass)::value) M += WN(q) * gb.w;
                }
              };
              if (sizeof(Real) == 4 || alpha * pr[5] != Real(0)) contract(std::true_type{});
              else contract(std::false_type{});
              // beta (lam P + mu P^T + mu tr(P) I) + alpha rho M I with the coefficients folded: two
              // operations an entry
              const Real bl = beta * lam, bm = beta * mu;
              const Real dg = bm * (Pm[0] + Pm[4] + Pm[8]) + alpha * pr[5] * M;
#pragma unroll
              for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                  Real k = bl * Pm[3 * c + d] + bm * Pm[3 * d + c];
                  if (c == d) k += dg;
                  if constexpr (SYM) kreg[sl * 9 + 3 * c + d] = k;
                  else put(c, b, d, pb, k);
                }
            } else {  // MAXWELL
              const Real imu = pr[0], sig = pr[1];
              Real kc = 0, kv = 0;
              for (int q = 0; q < NQ; ++q) {
                const Real* ca = sG + q * GQS + a * 4;
                const Real* cb = sG + q * GQS + b * 4;
                const Real* va = sV + q * GQS + a * 4;
                const Real* vb = sV + q * GQS + b * 4;
                kc += sW[q] * (ca[0] * cb[0] + ca[1] * cb[1] + ca[2] * cb[2]);
                kv += sW[q] * (va[0] * vb[0] + va[1] * vb[1] + va[2] * vb[2]);
              }
              put(0, b, 0, pb, beta * (imu * kc + sig * kv));
            }
          }
          if constexpr (TAN) {
            for (int i = 0; i < P.ntan; ++i)
#pragma unroll
              for (int c = 0; c < NF; ++c) accumulate<ATOMIC>(P.dfdp + (int64_t)i * P.n + NF * la + c, rt[i][c]);
          }
        }
      }
    }
    if constexpr (SCR && STAGE && JAC) {
      {
        // ---------------------------------------------------- 5 two-phase: rows to scratch
        // the thread's NF consecutive element rows (a * NF .. a * NF + NF - 1), NF * NE values
        if (my_a >= 0) {
          Real* dst = reinterpret_cast<Real*>(P.kscr) + (e * NE + my_a * NF) * NE;
          if constexpr (sizeof(Real) == 4 && (NE * NE) % 4 == 0 && (NF * NE) % 4 == 0) {
            float4* d4 = reinterpret_cast<float4*>(dst);  // 16-byte aligned: rows start at multiples of 4 values
#pragma unroll
            for (int k = 0; k < NF * NE / 4; ++k)
              d4[k] = make_float4(kreg[4 * k], kreg[4 * k + 1], kreg[4 * k + 2], kreg[4 * k + 3]);
          } else if constexpr (sizeof(Real) == 8 && (NE * NE) % 2 == 0 && (NF * NE) % 2 == 0) {
            double2* d2 = reinterpret_cast<double2*>(dst);
#pragma unroll
            for (int k = 0; k < NF * NE / 2; ++k) d2[k] = make_double2(kreg[2 * k], kreg[2 * k + 1]);
          } else {
#pragma unroll
            for (int k = 0; k < NF * NE; ++k) dst[k] = kreg[k];
          }
        }
        __syncthreads();
        continue;
      }
    }
    if constexpr (STAGE) {
      // ------------------------------------------------------ 5 CTA-wide scatter
      if constexpr (JAC) {
        __syncthreads();  // point tables are dead from here: the staged rows overwrite them
        if (my_a >= 0) {
          if constexpr (SYM) {
#pragma unroll
            for (int sl = 0; sl < NSLOT; ++sl) {
              if (sl == NB / 2 && my_a >= NB / 2) continue;
              const int b = my_a + sl < NB ? my_a + sl : my_a + sl - NB;
#pragma unroll
              for (int c = 0; c < NF; ++c)
#pragma unroll
                for (int d = 0; d < NF; ++d) {
                  const Real v = kreg[(sl * NF + c) * NF + d];
                  sK[(my_a * NF + c) * KRS + b * NF + d] = v;
                  if (sl != 0) sK[(b * NF + d) * KRS + my_a * NF + c] = v;  // K_ba = K_ab^T
                }
            }
          } else {
#pragma unroll
            for (int c = 0; c < NF; ++c)
#pragma unroll
              for (int k = 0; k < NE; ++k) sK[(my_a * NF + c) * KRS + k] = kreg[c * NE + k];
            if constexpr (HSYM) sK[my_a * KRS + my_a] += ksym[0];  // the diagonal's S (this thread's own entry)
          }
        }
        if constexpr (HSYM) {
          __syncthreads();  // every row's N_b terms are in place
          if (my_a >= 0) {
#pragma unroll
            for (int j = 1; j < NSH; ++j) {
              if (NB % 2 == 0 && j == NB / 2 && my_a >= NB / 2) continue;  // the opposite column: the lower row's
              const int b = my_a + j < NB ? my_a + j : my_a + j - NB;
              sK[my_a * KRS + b] += ksym[j];  // S_ab, and S_ba = S_ab: no other row adds to either
              sK[b * KRS + my_a] += ksym[j];
            }
          }
        }
      }
      // consecutive threads take consecutive entries of an element row
      __syncthreads();
      const int nval = (int)(e_hi - g0 < EPB ? e_hi - g0 : EPB);
      unsigned char* base = smem + C::R_END;
      if (P.f) {
        for (int i = threadIdx.x; i < nval * NE; i += blockDim.x) {
          const int l2 = i / NE, row = i - l2 * NE;
          const unsigned char* e2 = base + (size_t)l2 * C::E_END;
          const int32_t la = reinterpret_cast<const int32_t*>(e2 + C::E_LA)[row / NF];
          accumulate<ATOMIC>(P.f + (int64_t)NF * la + row % NF,
                             widen(reinterpret_cast<const Real*>(e2 + C::E_R)[row]));
        }
      }
      if constexpr (JAC) {
        // a warp walks whole elements; its lanes sit on the columns of RPW rows
        constexpr int RL = NE <= 4 ? 4 : NE <= 8 ? 8 : NE <= 16 ? 16 : 32;  // lanes per row
        constexpr int RPW = 32 / RL;                                          // rows per pass
        const int lane = threadIdx.x & 31;
        const int col = lane % RL, sub = lane / RL;
        const int cb = col / NF, cd = col - (col / NF) * NF;  // column's basis and field
        constexpr int NR = (NE + RPW - 1) / RPW;  // passes over an element's rows
        if (col < NE) {
          for (int l2 = threadIdx.x >> 5; l2 < nval; l2 += blockDim.x >> 5) {
            const unsigned char* e2 = base + (size_t)l2 * C::E_END;
            const int64_t* rps = reinterpret_cast<const int64_t*>(e2 + C::E_RP) + sub;
            const uint8_t* eps = reinterpret_cast<const uint8_t*>(e2 + C::E_EP) + cb * NB;
            const Real* kk = reinterpret_cast<const Real*>(e2 + C::E_K) + sub * KRS + col;
            // hex27: the element's epos from global memory, column cb of row a at epos[e][a][cb]
            const uint8_t* epg = nullptr;
            if constexpr (C::RG) {
              const int64_t ei2 = g0 + l2;
              epg = B.epos + ((perm ? (int64_t)__ldg(perm + ei2) : ei2) * NB) * NB + cb;
            }
            if constexpr (RPW == 1 && NB == 8) {
              // one pass per row: the lane's 8 byte offsets (one per row vertex) in registers
              const uint2 w = *reinterpret_cast<const uint2*>(eps);
              uint32_t off[NB];
#pragma unroll
              for (int a2 = 0; a2 < NB; ++a2)
                off[a2] = 8u * (NF * (((a2 < 4 ? w.x : w.y) >> (8 * (a2 & 3))) & 0xffu) + cd);
#pragma unroll
              for (int row = 0; row < NE; ++row) {
                double* p = reinterpret_cast<double*>(rps[row] + off[row / NF]);
                if constexpr (ATOMIC) red_global(p, widen(kk[row * KRS]));
                else *p += widen(kk[row * KRS]);
              }
            } else {
#pragma unroll
              for (int k = 0; k < NR; ++k) {
                const int row = sub + k * RPW;
                if (NE % RPW == 0 || row < NE) {
                  const int pos = C::RG ? (int)__ldg(epg + (row / NF) * NB) : (int)eps[row / NF];
                  double* p = reinterpret_cast<double*>(rps[k * RPW]) + (NF * pos + cd);
                  if constexpr (ATOMIC) red_global(p, widen(kk[k * RPW * KRS]));
                  else *p += widen(kk[k * RPW * KRS]);
                }
              }
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- launch shape
template <int TOPO, int BASIS, int NQ, int PHYS, typename Real, bool STAGE>
constexpr int block_threads() {
  return STAGE ? 128 : Cfg<TOPO, BASIS, NQ, PHYS, Real>::THREADS;
}

// Staged FP32 kernels ask for four resident CTAs (at most 128 registers a
// thread): the register-staged Jacobian rows otherwise cap residency at three.
template <typename Real, bool STAGE>
constexpr int min_blocks() {
  return STAGE && sizeof(Real) == 4 ? 4 : 1;
}

// ------------------------------------------------------------- families
// The element families the kernels are instantiated for.
enum Kind {
  K_HEX8_POISSON, K_HEX8_ELAST, K_HEX8_HEAT, K_HEX27_POISSON, K_HEX27_HEAT, K_TET4_POISSON, K_TET4_ELAST,
  K_TET4_HEAT, K_TET10_POISSON, K_TET10_HEAT, K_NED_MAXWELL, K_COUNT
};

#define TX_FOR_EACH_KIND(X)                                         \
  X(K_HEX8_POISSON, TX_TOPO_HEX, TX_HGRAD_C1, 8, TX_PHYS_POISSON)    \
  X(K_HEX8_ELAST, TX_TOPO_HEX, TX_HGRAD_C1, 8, TX_PHYS_ELASTICITY)   \
  X(K_HEX8_HEAT, TX_TOPO_HEX, TX_HGRAD_C1, 8, TX_PHYS_HEAT)          \
  X(K_HEX27_POISSON, TX_TOPO_HEX, TX_HGRAD_C2, 27, TX_PHYS_POISSON)  \
  X(K_HEX27_HEAT, TX_TOPO_HEX, TX_HGRAD_C2, 27, TX_PHYS_HEAT)        \
  X(K_TET4_POISSON, TX_TOPO_TET, TX_HGRAD_C1, 4, TX_PHYS_POISSON)    \
  X(K_TET4_ELAST, TX_TOPO_TET, TX_HGRAD_C1, 4, TX_PHYS_ELASTICITY)   \
  X(K_TET4_HEAT, TX_TOPO_TET, TX_HGRAD_C1, 4, TX_PHYS_HEAT)          \
  X(K_TET10_POISSON, TX_TOPO_TET, TX_HGRAD_C2, 4, TX_PHYS_POISSON)   \
  X(K_TET10_HEAT, TX_TOPO_TET, TX_HGRAD_C2, 4, TX_PHYS_HEAT)         \
  X(K_NED_MAXWELL, TX_TOPO_HEX, TX_HCURL_I1, 8, TX_PHYS_MAXWELL)

}  // namespace
}  // namespace tx
