// tx_assemble_tc.cu -- mixed R+J of hex8 elasticity with the element
// contraction on the tensor cores (tcgen05, TF32 with hi/lo splitting).
//
// The reference forms the element Jacobian block-rows by forward-mode AD
// through Integrator_GradBasisDotVector (disc-fe/src/evaluators/
// Panzer_Integrator_GradBasisDotVector_impl.hpp:225-294) and the mass terms
// through Integrator_BasisTimesScalar (Panzer_Integrator_BasisTimesScalar_
// impl.hpp:215-270), then scatters them with atomic sumIntoValues
// (Panzer_ScatterResidual_Tpetra_impl.hpp:390-439).  Here the closed form of
// that derivative is K_ab = beta (lam P_ab + mu P_ab^T + mu tr(P_ab) I) +
// alpha rho M_ab with
//   P_ab[i][j] = sum_q W_q dN_a/dx_i(q) dN_b/dx_j(q),  M_ab = sum_q W_q N_a(q) N_b(q),
// and both contractions of an element are one tensor-core product: with the
// element's 8 points as the K dimension,
//   A (rows 3a + i: W_q dN_a/dx_i; rows 24 + a: W_q N_a) times
//   B (rows 3b + j: dN_b/dx_j;     rows 24 + b: N_b)
// gives D = A B^T with P in D[0:24, 0:24] and M in D[24:32, 24:32].
//
// A CTA of four warps takes four elements at a time, warp w element w.  The
// A operand is one 128-row tile (rows 32 w .. 32 w + 31 of warp w); warp w
// multiplies the whole tile by its own B (32 rows) into its 32 tensor-memory
// columns and reads back only its own 32 lanes, so the rows of the other
// warps' elements in its D are never read (the tile shape's M = 128 is four
// times the rows one element needs).  Each product is three TF32 MMAs,
// A_hi B_hi + A_hi B_lo + A_lo B_hi, with FP32 accumulation in tensor memory:
// x = hi + lo with hi and lo TF32, the dropped A_lo B_lo term ~2^-22 of x.
// Geometry, the point stresses and the residual rows stay on the CUDA cores
// (FP32, vertex coordinates differenced in FP64); the Jacobian and residual
// go to f and the CRS values by FP64 reductions, consecutive lanes on the
// three consecutive entries of each neighbour block of a row.
//
// Every mbarrier wait is bounded: a wait that gives up sets bit 0 of the
// status word (reported as TX_ETIMEDOUT by tx_synchronize) and the kernel
// skips that element's results and carries on to free its tensor memory.
#include <algorithm>
#include <cstdint>

#include "tx_device.cuh"
#include "tx_numeric.cuh"
#include "tx_tcgen05.cuh"

namespace tx {
namespace {

constexpr int kThreads = 128;                // four warps, one element each
constexpr uint32_t kTmemCols = 128;          // D of the four warps: 32 columns each
constexpr uint32_t kMaxPolls = 1u << 22;     // mbarrier polls before a wait gives up
constexpr int kTile = 4096;                  // 128 rows x 8 TF32
constexpr int kBTile = 1024;                 // 32 rows x 8 TF32
constexpr int kPRow = 25;                    // staged P rows (odd word stride)

// shared memory (bytes)
constexpr int kSmAhi = 0;
constexpr int kSmAlo = kSmAhi + kTile;
constexpr int kSmB = kSmAlo + kTile;                             // per warp: B hi, B lo
constexpr int kSmP = kSmB + 4 * 2 * kBTile;                      // per warp: P [24][25], M [8][9]
constexpr int kPBytes = ((24 * kPRow + 8 * 9) * 4 + 15) / 16 * 16;
constexpr int kSmRef = kSmP + 4 * kPBytes;                       // [q][v] float4 (dN^/dxi, N), w[q]
constexpr int kSmBar = kSmRef + 64 * 16 + 8 * 4;                 // four mbarriers
constexpr int kSmTmem = kSmBar + 4 * 8;
constexpr int kSmUsed = kSmTmem + 16;
// at most four CTAs an SM (4 x 128 tensor-memory columns): ask for more than
// a fifth of the SM's 228 KB
constexpr int kSmBytes = kSmUsed > 48 * 1024 ? kSmUsed : 48 * 1024;
static_assert(kSmBar % 8 == 0, "mbarrier alignment");

__device__ __forceinline__ void put_split(unsigned char* hi, unsigned char* lo, uint32_t off, float v) {
  const float h = tc::to_tf32(v);
  *reinterpret_cast<float*>(hi + off) = h;
  *reinterpret_cast<float*>(lo + off) = tc::to_tf32(v - h);
}

__global__ void __launch_bounds__(kThreads, 4)
    k_assemble_tc(const BlockView B, const EvalParams P, int64_t e_lo, int64_t e_hi, int* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int t = threadIdx.x, w = t >> 5, l = t & 31;
  float4* rg = reinterpret_cast<float4*>(smem + kSmRef);
  float* rw = reinterpret_cast<float*>(smem + kSmRef + 64 * 16);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kSmBar) + w;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kSmTmem);
  {
    // reference tables [w | geo_val | geo_grad | val | grad]: (dN^/dxi, N) of basis v at point q
    const double* ref = B.ref;
    for (int i = t; i < 64; i += kThreads) {
      const double* gr = ref + 8 + 64 + 192 + 64 + 3 * i;
      rg[i] = make_float4(narrow(gr[0]), narrow(gr[1]), narrow(gr[2]), narrow(ref[8 + 64 + 192 + i]));
    }
    if (t < 8) rw[t] = narrow(ref[t]);
  }
  if (t == 0) {
    for (int i = 0; i < 4; ++i) tc::mbar_init(reinterpret_cast<uint64_t*>(smem + kSmBar) + i, 1);
    tc::mbar_init_fence();
  }
  __syncwarp();  // the allocation and the loads below are warp-collective (.sync.aligned)
  if (w == 0) tc::tmem_alloc(tslot, kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t d_w = tmem + 32u * w;                      // this warp's D columns (lane field 0)
  const uint32_t d_ld = tmem + ((32u * w) << 16) + 32u * w;  // its 32 lanes of them

  unsigned char* Ahi = smem + kSmAhi;
  unsigned char* Alo = smem + kSmAlo;
  unsigned char* Bhi = smem + kSmB + w * 2 * kBTile;
  unsigned char* Blo = Bhi + kBTile;
  float* sP = reinterpret_cast<float*>(smem + kSmP + w * kPBytes);
  float* sM = sP + 24 * kPRow;
  const uint32_t idesc = tc::idesc_tf32(128, 32);
  const uint64_t dAhi = tc::smem_desc(tc::smem_addr(Ahi)), dAlo = tc::smem_desc(tc::smem_addr(Alo));
  const uint64_t dBhi = tc::smem_desc(tc::smem_addr(Bhi)), dBlo = tc::smem_desc(tc::smem_addr(Blo));

  const float lam = narrow(P.lam), mu = narrow(P.mu), rho = narrow(P.p[5]);
  const float bx = narrow(P.p[2]), by = narrow(P.p[3]), bz = narrow(P.p[4]);
  const float bl = narrow(P.beta * P.lam), bm = narrow(P.beta * P.mu), am = narrow(P.alpha * P.p[5]);
  const int q = l & 7, vg = l >> 3, b0 = 2 * vg, b1 = b0 + 1;  // geometry roles
  uint32_t phase = 0;

  for (int64_t g = blockIdx.x; e_lo + 4 * g < e_hi; g += gridDim.x) {
    const int64_t e = e_lo + 4 * g + w;
    if (e >= e_hi) continue;  // the warp's slot is past the end (uniform over the warp)
    // ------------------------------------------------------------ gather
    float dxl = 0.f;  // lane 3 v + d: x_v[d] - x_0[d]
    int64_t rs = 0;   // lane 3 a + c: first CRS value of row (a, c)
    int32_t ent = 0;  // lane b < 8: entity LID of basis b
    float u[3] = {0.f, 0.f, 0.f}, ud[3] = {0.f, 0.f, 0.f};
    if (l < 8) {
      ent = __ldg(B.dconn + e * 8 + l);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        u[c] = narrow(__ldg(P.x + 3 * (int64_t)ent + c));
        ud[c] = P.xdot ? narrow(__ldg(P.xdot + 3 * (int64_t)ent + c)) : 0.f;
      }
    }
    {
      const int v = l < 24 ? l / 3 : 0, d = l < 24 ? l % 3 : 0;
      const double xv = __ldg(P.coords + 3 * (int64_t)__ldg(B.vconn + e * 8 + v) + d);
      const double x0 = __shfl_sync(0xffffffffu, xv, d);
      dxl = l < 24 ? narrow(xv - x0) : 0.f;
      const int32_t ea = __shfl_sync(0xffffffffu, ent, v);
      if (l < 24) rs = __ldg(P.rowptr + 3 * (int64_t)ea + d);
    }
    // ------------------------------------------------------------ geometry at point q
    float J[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) J[k] = 0.f;
#pragma unroll
    for (int v = 1; v < 8; ++v) {
      const float4 gr = rg[q * 8 + v];
      const float dx = __shfl_sync(0xffffffffu, dxl, 3 * v), dy = __shfl_sync(0xffffffffu, dxl, 3 * v + 1);
      const float dz = __shfl_sync(0xffffffffu, dxl, 3 * v + 2);
      J[0] += dx * gr.x; J[1] += dx * gr.y; J[2] += dx * gr.z;
      J[3] += dy * gr.x; J[4] += dy * gr.y; J[5] += dy * gr.z;
      J[6] += dz * gr.x; J[7] += dz * gr.y; J[8] += dz * gr.z;
    }
    const float c00 = J[4] * J[8] - J[5] * J[7];
    const float c01 = J[5] * J[6] - J[3] * J[8];
    const float c02 = J[3] * J[7] - J[4] * J[6];
    const float det = J[0] * c00 + J[1] * c01 + J[2] * c02;
    const float id = 1.0f / det;
    float Ji[9];
    Ji[0] = c00 * id; Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id; Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
    Ji[3] = c01 * id; Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id; Ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
    Ji[6] = c02 * id; Ji[7] = (J[1] * J[6] - J[0] * J[7]) * id; Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
    // computeCellMeasure: the weights take the sign of det J at the first point (lane 0)
    const float det0 = __shfl_sync(0xffffffffu, det, 0);
    const float W = rw[q] * det * (det0 < 0.f ? -1.f : 1.f);
    float gb[2][3], nb[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const float4 gr = rg[q * 8 + b0 + s];
      gb[s][0] = Ji[0] * gr.x + Ji[3] * gr.y + Ji[6] * gr.z;
      gb[s][1] = Ji[1] * gr.x + Ji[4] * gr.y + Ji[7] * gr.z;
      gb[s][2] = Ji[2] * gr.x + Ji[5] * gr.y + Ji[8] * gr.z;
      nb[s] = gr.w;
      const int b = b0 + s;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        put_split(Ahi, Alo, tc::operand_offset(32 * w + 3 * b + i, q), W * gb[s][i]);
        put_split(Bhi, Blo, tc::operand_offset(3 * b + i, q), gb[s][i]);
      }
      put_split(Ahi, Alo, tc::operand_offset(32 * w + 24 + b, q), W * nb[s]);
      put_split(Bhi, Blo, tc::operand_offset(24 + b, q), nb[s]);
    }
    // the tiles are complete once every lane's stores are visible to the tensor cores
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncwarp();
    if (l == 0) {
      tc::fence_after_sync();
      tc::mma_tf32(d_w, dAhi, dBhi, idesc, false);
      tc::mma_tf32(d_w, dAhi, dBlo, idesc, true);
      tc::mma_tf32(d_w, dAlo, dBhi, idesc, true);
      tc::mma_commit(bar);
    }
    // ------------------------------------------------------------ residual rows (CUDA cores, meanwhile)
    {
      float Gu[9], acc[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float u0 = __shfl_sync(0xffffffffu, u[c], b0), u1 = __shfl_sync(0xffffffffu, u[c], b1);
        const float v0 = __shfl_sync(0xffffffffu, ud[c], b0), v1 = __shfl_sync(0xffffffffu, ud[c], b1);
#pragma unroll
        for (int i = 0; i < 3; ++i) Gu[3 * c + i] = gb[0][i] * u0 + gb[1][i] * u1;
        acc[c] = nb[0] * v0 + nb[1] * v1;
      }
      // the four vertex pairs of point q: lanes q, q + 8, q + 16, q + 24
#pragma unroll
      for (int o = 8; o < 32; o <<= 1) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Gu[k] += __shfl_xor_sync(0xffffffffu, Gu[k], o);
#pragma unroll
        for (int c = 0; c < 3; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
      }
      const float tr = Gu[0] + Gu[4] + Gu[8];
      const float s00 = W * (mu * (Gu[0] + Gu[0]) + lam * tr), s11 = W * (mu * (Gu[4] + Gu[4]) + lam * tr);
      const float s22 = W * (mu * (Gu[8] + Gu[8]) + lam * tr), s01 = W * (mu * (Gu[1] + Gu[3]));
      const float s02 = W * (mu * (Gu[2] + Gu[6])), s12 = W * (mu * (Gu[5] + Gu[7]));
      const float f0 = W * (rho * acc[0] - bx), f1 = W * (rho * acc[1] - by), f2 = W * (rho * acc[2] - bz);
      float r[2][3];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        r[s][0] = gb[s][0] * s00 + gb[s][1] * s01 + gb[s][2] * s02 + nb[s] * f0;
        r[s][1] = gb[s][0] * s01 + gb[s][1] * s11 + gb[s][2] * s12 + nb[s] * f1;
        r[s][2] = gb[s][0] * s02 + gb[s][1] * s12 + gb[s][2] * s22 + nb[s] * f2;
      }
      // sum over the eight points: lanes 8 vg .. 8 vg + 7
#pragma unroll
      for (int o = 1; o < 8; o <<= 1)
#pragma unroll
        for (int s = 0; s < 2; ++s)
#pragma unroll
          for (int c = 0; c < 3; ++c) r[s][c] += __shfl_xor_sync(0xffffffffu, r[s][c], o);
      const int32_t e0 = __shfl_sync(0xffffffffu, ent, b0), e1 = __shfl_sync(0xffffffffu, ent, b1);
      if (q == 0 && P.f) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          atomicAdd(P.f + 3 * (int64_t)e0 + c, widen(r[0][c]));
          atomicAdd(P.f + 3 * (int64_t)e1 + c, widen(r[1][c]));
        }
      }
    }
    // ------------------------------------------------------------ contraction results
    // one verdict for the warp: the reads below are warp-collective
    const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(bar, phase & 1u, kMaxPolls));
    ++phase;
    if (!ok) {
      if (l == 0) atomicOr(status, 1);
      continue;
    }
    tc::fence_after_sync();
    {
      float v[4][8];
#pragma unroll
      for (int c = 0; c < 4; ++c) tc::tmem_ld8(d_ld + 8u * c, v[c]);
      if (l < 24) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int i = 0; i < 8; ++i) sP[l * kPRow + 8 * c + i] = v[c][i];
      } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) sM[(l - 24) * 9 + i] = v[3][i];
      }
    }
    tc::fence_before_sync();
    __syncwarp();
    // ------------------------------------------------------------ Jacobian rows to the CRS
    if (P.vals && l < 24) {
      const int b = l / 3, d = l % 3;
#pragma unroll 1
      for (int row = 0; row < 24; ++row) {
        const int a = row / 3, c = row % 3;
        const int64_t start = __shfl_sync(0x00ffffffu, rs, row);
        const float* pa = sP + 3 * a * kPRow + 3 * b;
        float k = bl * pa[c * kPRow + d] + bm * pa[d * kPRow + c];
        if (c == d) k += bm * (pa[0] + pa[kPRow + 1] + pa[2 * kPRow + 2]) + am * sM[a * 9 + b];
        const int pos = __ldg(B.epos + (e * 8 + a) * 8 + b);
        atomicAdd(P.vals + start + 3 * pos + d, widen(k));
      }
    }
    __syncwarp();
  }
  // every warp's last tensor-memory read is done before the allocation goes
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) {
    tc::fence_after_sync();
    __syncwarp();
    tc::tmem_free(tmem, kTmemCols);
  }
}

// A wait on an mbarrier nothing arrives at: the bounded wait gives up after
// max_polls polls and sets bit 0 of *status, as the assembly kernel does.
__global__ void k_wait_selftest(int* status, uint32_t max_polls) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_init_fence();
  }
  __syncthreads();
  const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(&bar, 0, max_polls));
  if (!ok && threadIdx.x == 0) atomicOr(status, 1);
}

}  // namespace

cudaError_t launch_wait_selftest(int* status, cudaStream_t s) {
  k_wait_selftest<<<1, 32, 0, s>>>(status, 1u << 12);
  return cudaGetLastError();
}

bool tc_supported(const BlockView& B, const EvalParams& P) {
  return B.topo == TX_TOPO_HEX && B.basis == TX_HGRAD_C1 && B.nq == 8 && B.nb == 8 && B.nv == 8 &&
         P.physics == TX_PHYS_ELASTICITY && !P.tan && !P.kscr;
}

cudaError_t launch_assemble_tc(const BlockView& B, const EvalParams& P, int64_t e_lo, int64_t e_hi, int* status,
                               cudaStream_t s, int grid_cap) {
  if (!tc_supported(B, P)) return cudaErrorInvalidValue;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_assemble_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int64_t n = e_hi - e_lo;
  if (n <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t grid = std::min<int64_t>((n + 3) / 4, 4 * (int64_t)sms);
  if (grid_cap > 0 && grid_cap < grid) grid = grid_cap;
  k_assemble_tc<<<(unsigned)grid, kThreads, kSmBytes, s>>>(B, P, e_lo, e_hi, status);
  return cudaGetLastError();
}

}  // namespace tx
