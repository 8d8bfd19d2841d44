// tx_lattice.cu -- owner-computes ("gather") assembly of a brick-lattice hex8
// block: every CRS row of a node is summed inside one CTA and written once.
//
// The reference scatters every element's rows into the Tpetra CRS with
// atomic sumIntoValues (disc-fe/src/evaluators/Panzer_ScatterResidual_Tpetra_
// impl.hpp:390-439) after zeroing f and the matrix (Panzer_ModelEvaluator_
// impl.hpp:1788-1789).  On the brick lattice of a CartesianConnManager block
// the elements around a node are known from its lattice position, so here
// the rows are gathered instead: a CTA owns a 4 x 4 column of nodes and
// walks it up the z axis one node layer at a time.  At layer k it
//
//   1. computes the geometry, physical gradients and residual rows of the
//      5 x 5 elements of element layer k (its own 4 x 4 and a one-element
//      halo) into a ring of two element layers in shared memory (1 KB an
//      element; four lanes an element, two points each as the two halves of
//      packed FP32x2 FMAs, the residual shares summed across the four lanes);
//   2. assembles the rows of its 16 nodes of layer k from the 8 elements
//      around each node (element layers k - 1 and k): eight lanes per node,
//      one element each; each lane forms its element's 3 x 24 block-row of
//      the node (the closed form of the AD Jacobian, as in the per-element
//      kernel) one 3 x 3 block at a time, and the eight lanes sum the blocks
//      that land on the same neighbour with up to three butterfly exchanges
//      (x, y, z: a fixed order) before the next block is formed, so one
//      block is live in registers (three CTAs of 128 threads a SM);
//   3. stages the node's 3 rows (81 values each in the interior) in shared
//      memory in CRS order and writes them with coalesced 16-byte stores.
//
// f and the CRS values are written exactly once (no zeroing, no atomics, no
// read-modify-write of the 4 GB matrix) and every run gives the same bits.
// Halo elements are recomputed by the neighbouring columns (25 element
// geometries per 16 nodes); the Jacobian rows themselves are formed once.
// Tasks (a node column's z chunk) go to the CTAs round-robin; the chunk
// length is picked at launch for the grid.
//
// Precision: the mixed evaluation type (TX_EVAL_MIXED): FP32 geometry,
// stresses and contractions; the eight element contributions of an entry
// are summed in FP32 (at most three roundings) and widened to FP64 exactly.
// Vertex coordinates enter as FP32 hi/lo pairs split on the host, so the
// element edge vectors keep their FP64 accuracy.  The point sums of the
// contraction run as two interleaved partial sums (even and odd points) in
// packed FP32x2 FMAs (fma.rn.f32x2: two IEEE FMAs per instruction).
#include <algorithm>
#include <cstdint>

#include "tx_device.cuh"
#include "tx_numeric.cuh"

namespace tx {
namespace {

constexpr int kTile = 4;                    // owned nodes per CTA along x and y
constexpr int kPlane = kTile + 2;           // node plane of a step: owned nodes, halo on both sides
constexpr int kElem = kTile + 1;            // element columns of a step along x and y
constexpr int kElems = kElem * kElem;       // 25 elements per layer
constexpr int kNodes = kTile * kTile;       // 16 owned nodes per layer
constexpr int kThreads = kNodes * 8;        // eight lanes per node
constexpr int kRowMax = 243;                // 3 rows x 81 entries (interior node)
constexpr int kStageRow = 248;              // staged floats a node: one parity slot, 243 entries, float4 tail

// Element record in shared memory, 1 KB.  Points go in pairs p = (2 qp,
// 2 qp + 1); vertex B (lattice bits x | y << 1 | z << 2) of pair qp sits in
// slot 9 qp + B, so for a fixed pair the eight vertices (the eight lanes of a
// node read eight different ones) and for a fixed vertex the four pairs fall
// in different bank groups, and every address is a lane base plus an
// immediate.
//   XY: (gx_q0, gx_q1, gy_q0, gy_q1) physical gradients, float4 slots;
//   Z:  (gz_q0, gz_q1), float2 slot 8 qp + B, 64 bytes further on in
//       elements of odd lattice x (two nodes of a warp read the same slot of
//       two x-neighbouring elements in one 64-bit load: 16 banks apart);
//   R:  float4 slot B: the element's residual row of vertex B (summed over
//       the points) and, in .w, the signed weight W_q = s w_q det J_q of point
//       q = B ^ rot, rot the parity bits of the element's lattice position (s
//       the sign of det J at the first point): the eight elements around a
//       node have eight different parities, so the eight lanes of a node read
//       W_q from eight different slots.
constexpr int kRecXY = 0;
constexpr int kRecZ = kRecXY + 36 * 16;
constexpr int kRecR = kRecZ + 32 * 8 + 64;
constexpr int kRecBytes = ((kRecR + 8 * 16) + 127) / 128 * 128;
static_assert(kRecBytes == 1024, "element record");

// Node record of a plane: coordinates (FP32 hi, lo), u, u_dot.
struct __align__(16) PlaneNode {
  float4 xh, xl, u, ud;
};

// shared memory layout
constexpr int kSmRefP = 0;  // [qp][B] 2 float4 (gx_q0, gx_q1, gy_q0, gy_q1), (gz_q0, gz_q1, N_q0, N_q1), slots 2 (9 qp + B)
constexpr int kSmRefN = kSmRefP + 72 * 16;                       // [qp][B] float2 (N(q0), N(q1)), slot 9 qp + B
constexpr int kSmRefW = kSmRefN + 36 * 8;                        // [q] w_q
constexpr int kSmPlane = kSmRefW + 8 * 4;                        // 2 x 36 PlaneNode
constexpr int kSmPlaneInfo = kSmPlane + 2 * kPlane * kPlane * 64;  // owned-node info of the 2 planes
constexpr int kInfoBytes = 48;                                   // rowstart (8) lid (4) nnb (4) npos (32)
constexpr int kSmElem = kSmPlaneInfo + 2 * kNodes * kInfoBytes;
constexpr int kSmStage = kSmElem + 2 * kElems * kRecBytes;       // [node][243] float
constexpr int kSmBytes = kSmStage + kNodes * kStageRow * 4;

// Which lane writes which exchanged slot (bit 8 e + c): every neighbour block
// is held by 2^(zero bits of c) lanes after the butterflies; this table picks
// one of them so that no lane writes more than four blocks of the 27.
constexpr unsigned long long kWriters = 0x92c2a4e08cc9b8e8ull;

// shards Hexahedron<8> vertex v <-> lattice offset bits (x | y << 1 | z << 2);
// the map is an involution on these eight codes
__device__ __forceinline__ int vbits(int v) {
  constexpr unsigned kTab = 0u | (1u << 3) | (3u << 6) | (2u << 9) | (4u << 12) | (5u << 15) | (7u << 18) | (6u << 21);
  return (kTab >> (3 * v)) & 7;
}

__device__ __forceinline__ float4 f4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }

// Two IEEE FP32 FMAs in one instruction: (a.x b.x + c.x, a.y b.y + c.y).
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;"
      : "=l"(r)
      : "l"(*reinterpret_cast<unsigned long long*>(&a)), "l"(*reinterpret_cast<unsigned long long*>(&b)),
        "l"(*reinterpret_cast<unsigned long long*>(&c)));
  return *reinterpret_cast<float2*>(&r);
}

// Loads plane node records of node layer kk for the task's 6 x 6 window and
// the owned nodes' row information.
__device__ __forceinline__ void load_plane(const LatticeArgs& A, int64_t i0, int64_t j0, int64_t kk,
                                           unsigned char* smem, int slot) {
  PlaneNode* pl = reinterpret_cast<PlaneNode*>(smem + kSmPlane) + slot * kPlane * kPlane;
  const int t = threadIdx.x;
  if (t < kPlane * kPlane) {
    const int64_t i = i0 - 1 + t % kPlane, j = j0 - 1 + t / kPlane;
    PlaneNode p{f4(0, 0, 0, 0), f4(0, 0, 0, 0), f4(0, 0, 0, 0), f4(0, 0, 0, 0)};
    if (i >= 0 && i <= A.nx && j >= 0 && j <= A.ny && kk >= 0 && kk <= A.nz) {
      const int64_t g = i + (A.nx + 1) * (j + (A.ny + 1) * kk);
      const LatticeNode& n = A.nodes[g];
      p.xh = f4(n.xh[0], n.xh[1], n.xh[2], 0.f);
      p.xl = f4(n.xl[0], n.xl[1], n.xl[2], 0.f);
      p.u = reinterpret_cast<const float4*>(A.u)[g];
      p.ud = A.ud ? reinterpret_cast<const float4*>(A.ud)[g] : f4(0, 0, 0, 0);
    }
    pl[t] = p;
  } else if (t >= 64 && t < 64 + kNodes) {
    const int ln = t - 64;
    const int64_t i = i0 + (ln & 3), j = j0 + (ln >> 2);
    unsigned char* info = smem + kSmPlaneInfo + (slot * kNodes + ln) * kInfoBytes;
    if (i <= A.nx && j <= A.ny && kk >= 0 && kk <= A.nz) {
      const int64_t g = i + (A.nx + 1) * (j + (A.ny + 1) * kk);
      const LatticeNode& n = A.nodes[g];
      *reinterpret_cast<int64_t*>(info) = n.rowstart;
      reinterpret_cast<int32_t*>(info)[2] = n.lid;
      const int nnb = (1 + (i > 0) + (i < A.nx)) * (1 + (j > 0) + (j < A.ny)) * (1 + (kk > 0) + (kk < A.nz));
      reinterpret_cast<int32_t*>(info)[3] = nnb;
      const uint4* src = reinterpret_cast<const uint4*>(n.npos);
      reinterpret_cast<uint4*>(info + 16)[0] = src[0];
      reinterpret_cast<uint4*>(info + 16)[1] = src[1];
    } else {
      reinterpret_cast<int32_t*>(info)[3] = 0;  // no node
    }
  }
}

// Geometry, physical gradients and residual rows of the 5 x 5 elements of
// element layer ek (vertices in plane slots ek & 1 and (ek + 1) & 1); one
// thread per (element, point pair), the four threads of an element adjacent
// lanes of one warp, the pair's two points the two halves of packed FP32x2
// FMAs.  Each thread forms its two points' share of the element's 8 x 3
// residual rows, W_q (grad N_B . sigma_q + N_B (rho acc_q - b)), and two
// halving exchanges over the four lanes sum the shares.
template <bool MASS>
__device__ __forceinline__ void element_layer(const LatticeArgs& A, int64_t i0, int64_t j0, int64_t ek,
                                              unsigned char* smem) {
  if (ek < 0 || ek >= A.nz) return;
  const float* rw = reinterpret_cast<const float*>(smem + kSmRefW);
  const PlaneNode* plo = reinterpret_cast<const PlaneNode*>(smem + kSmPlane) + (int)(ek & 1) * kPlane * kPlane;
  const PlaneNode* phi = reinterpret_cast<const PlaneNode*>(smem + kSmPlane) + (int)((ek + 1) & 1) * kPlane * kPlane;
  unsigned char* rec0 = smem + kSmElem + (int)(ek & 1) * kElems * kRecBytes;
  const int task = threadIdx.x;
  if (task >= kElems * 4) return;
  const int el = task >> 2, qp = task & 3;
  const int ex = el % kElem, ey = el / kElem;
  const int64_t gx = i0 - 1 + ex, gy = j0 - 1 + ey;
  if (gx < 0 || gx >= A.nx || gy < 0 || gy >= A.ny) return;  // the element's four lanes alike
  const unsigned m4 = 0xfu << (threadIdx.x & 28);              // those four lanes
  const int rot = (int)(gx & 1) | ((int)(gy & 1) << 1) | ((int)(ek & 1) << 2);
  unsigned char* rec = rec0 + el * kRecBytes;
  // vertex with lattice bits B at plane (ex + Bx, ey + By), layer Bz
  float dX[8][3], U[8][3], UD[8][3];
  float x0h[3], x0l[3];
#pragma unroll
  for (int B = 0; B < 8; ++B) {
    const PlaneNode& p = ((B >> 2) ? phi : plo)[(ex + (B & 1)) + kPlane * (ey + ((B >> 1) & 1))];
    const float4 h = p.xh, l = p.xl, u = p.u;
    if (B == 0) {
      x0h[0] = h.x; x0h[1] = h.y; x0h[2] = h.z;
      x0l[0] = l.x; x0l[1] = l.y; x0l[2] = l.z;
    }
    dX[B][0] = (h.x - x0h[0]) + (l.x - x0l[0]);
    dX[B][1] = (h.y - x0h[1]) + (l.y - x0l[1]);
    dX[B][2] = (h.z - x0h[2]) + (l.z - x0l[2]);
    U[B][0] = u.x; U[B][1] = u.y; U[B][2] = u.z;
    if constexpr (MASS) {
      const float4 ud = p.ud;
      UD[B][0] = ud.x; UD[B][1] = ud.y; UD[B][2] = ud.z;
    }
  }
  // The two points of the pair run as the two halves of packed FP32x2 FMAs
  // (fma.rn.f32x2); per vertex B the reference table holds (gx, gy | gz, N)
  // of both points.
  const float4* rp = reinterpret_cast<const float4*>(smem + kSmRefP) + 2 * 9 * qp;
  const float2 zero2 = make_float2(0.f, 0.f);
  float2 J2[9], acc2[3] = {zero2, zero2, zero2};
#pragma unroll
  for (int k = 0; k < 9; ++k) J2[k] = zero2;
#pragma unroll
  for (int B = 0; B < 8; ++B) {
    const float4 p0 = rp[2 * B], p1 = rp[2 * B + 1];
    const float2 gx = make_float2(p0.x, p0.y), gy = make_float2(p0.z, p0.w), gz = make_float2(p1.x, p1.y);
    if (B > 0) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float2 d = make_float2(dX[B][i], dX[B][i]);
        J2[3 * i + 0] = ffma2(d, gx, J2[3 * i + 0]);
        J2[3 * i + 1] = ffma2(d, gy, J2[3 * i + 1]);
        J2[3 * i + 2] = ffma2(d, gz, J2[3 * i + 2]);
      }
    }
    if constexpr (MASS) {
      const float2 nn = make_float2(p1.z, p1.w);
#pragma unroll
      for (int c = 0; c < 3; ++c) acc2[c] = ffma2(nn, make_float2(UD[B][c], UD[B][c]), acc2[c]);
    }
  }
  float2 Ji2[9];
  float det[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float J[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) J[k] = h ? J2[k].y : J2[k].x;
    const float c00 = J[4] * J[8] - J[5] * J[7];
    const float c01 = J[5] * J[6] - J[3] * J[8];
    const float c02 = J[3] * J[7] - J[4] * J[6];
    det[h] = J[0] * c00 + J[1] * c01 + J[2] * c02;
    const float id = 1.0f / det[h];
    float Ji[9];
    Ji[0] = c00 * id; Ji[1] = (J[2] * J[7] - J[1] * J[8]) * id; Ji[2] = (J[1] * J[5] - J[2] * J[4]) * id;
    Ji[3] = c01 * id; Ji[4] = (J[0] * J[8] - J[2] * J[6]) * id; Ji[5] = (J[2] * J[3] - J[0] * J[5]) * id;
    Ji[6] = c02 * id; Ji[7] = (J[1] * J[6] - J[0] * J[7]) * id; Ji[8] = (J[0] * J[4] - J[1] * J[3]) * id;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      if (h == 0) Ji2[k].x = Ji[k];
      else Ji2[k].y = Ji[k];
    }
  }
  // physical gradients grad_i = sum_j Jinv(j, i) grad^_j of both points, stored as
  // slots 9 qp + B (gx_q0, gx_q1, gy_q0, gy_q1) and 8 qp + B (gz_q0, gz_q1);
  // displacement gradients Gu[3 c + i] = du_c / dx_i
  float4* XY = reinterpret_cast<float4*>(rec + kRecXY) + 9 * qp;
  float2* Z = reinterpret_cast<float2*>(rec + kRecZ + 64 * (int)(gx & 1)) + 8 * qp;
  float2 Gu2[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Gu2[k] = zero2;
#pragma unroll
  for (int B = 0; B < 8; ++B) {
    const float4 p0 = rp[2 * B], p1 = rp[2 * B + 1];
    const float2 hx = make_float2(p0.x, p0.y), hy = make_float2(p0.z, p0.w), hz = make_float2(p1.x, p1.y);
    float2 g[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) g[i] = ffma2(Ji2[i], hx, ffma2(Ji2[3 + i], hy, ffma2(Ji2[6 + i], hz, zero2)));
    XY[B] = f4(g[0].x, g[0].y, g[1].x, g[1].y);
    Z[B] = g[2];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 uu = make_float2(U[B][c], U[B][c]);
      Gu2[3 * c + 0] = ffma2(g[0], uu, Gu2[3 * c + 0]);
      Gu2[3 * c + 1] = ffma2(g[1], uu, Gu2[3 * c + 1]);
      Gu2[3 * c + 2] = ffma2(g[2], uu, Gu2[3 * c + 2]);
    }
  }
  // W-scaled stress rows and point force (rho acc - b), both points
  float wd[2];  // w_q det J_q at the two points
  float2 S[3][3], F[3];
  const float lam = A.lam, mu = A.mu;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float Gu[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Gu[k] = h ? Gu2[k].y : Gu2[k].x;
    const float w = rw[2 * qp + h] * det[h];
    wd[h] = w;
    const float tr = Gu[0] + Gu[4] + Gu[8];
    float s[3][3];
    s[0][0] = w * (mu * (Gu[0] + Gu[0]) + lam * tr);
    s[1][1] = w * (mu * (Gu[4] + Gu[4]) + lam * tr);
    s[2][2] = w * (mu * (Gu[8] + Gu[8]) + lam * tr);
    s[0][1] = s[1][0] = w * (mu * (Gu[1] + Gu[3]));
    s[0][2] = s[2][0] = w * (mu * (Gu[2] + Gu[6]));
    s[1][2] = s[2][1] = w * (mu * (Gu[5] + Gu[7]));
    const float a[3] = {h ? acc2[0].y : acc2[0].x, h ? acc2[1].y : acc2[1].x, h ? acc2[2].y : acc2[2].x};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        if (h == 0) S[c][i].x = s[c][i];
        else S[c][i].y = s[c][i];
      }
      const float fc = w * (A.rho * a[c] - A.body[c]);
      if (h == 0) F[c].x = fc;
      else F[c].y = fc;
    }
  }
  // the two points' share of the residual rows: grad N_B . sigma_c + N_B f_c,
  // gradients read back from the record, the halves summed
  float res[8][3];
#pragma unroll
  for (int B = 0; B < 8; ++B) {
    const float4 xy = XY[B];
    const float2 z = Z[B];
    const float4 p1 = rp[2 * B + 1];
    const float2 g0 = make_float2(xy.x, xy.y), g1 = make_float2(xy.z, xy.w), nn = make_float2(p1.z, p1.w);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 t = ffma2(g0, S[c][0], ffma2(g1, S[c][1], ffma2(z, S[c][2], ffma2(nn, F[c], zero2))));
      res[B][c] = t.x + t.y;
    }
  }
  // computeCellMeasure: the weights take the sign of the first point's det J
  const int l0 = threadIdx.x & 28;
  const float sg = __shfl_sync(m4, wd[0], l0) < 0.f ? -1.f : 1.f;
  // sum the four point pairs' shares (lanes 4 el .. 4 el + 3) by halving
  // exchanges: across lane bit 1 the lane keeps vertices 0-3 or 4-7, across
  // bit 0 the lower or upper two of those, so lane qp ends with the sums of
  // vertices 2 qp and 2 qp + 1
  float h4[4][3];
  {
    const bool up = qp & 2;
#pragma unroll
    for (int B = 0; B < 4; ++B)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float keep = up ? res[B + 4][c] : res[B][c], send = up ? res[B][c] : res[B + 4][c];
        h4[B][c] = keep + __shfl_xor_sync(m4, send, 2);
      }
  }
  float h2[2][3];
  {
    const bool up = qp & 1;
#pragma unroll
    for (int B = 0; B < 2; ++B)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float keep = up ? h4[B + 2][c] : h4[B][c], send = up ? h4[B][c] : h4[B + 2][c];
        h2[B][c] = keep + __shfl_xor_sync(m4, send, 1);
      }
  }
  // slots 2 qp and 2 qp + 1 hold W of points 2 qp ^ rot and (2 qp ^ rot) ^ 1,
  // both held by lane 4 el + ((2 qp ^ rot) >> 1)
  const int src = l0 + (((2 * qp) ^ rot) >> 1);
  const float wa = sg * __shfl_sync(m4, wd[0], src), wb = sg * __shfl_sync(m4, wd[1], src);
  const bool odd = rot & 1;
  float4* R = reinterpret_cast<float4*>(rec + kRecR);
  R[2 * qp] = f4(sg * h2[0][0], sg * h2[0][1], sg * h2[0][2], odd ? wb : wa);
  R[2 * qp + 1] = f4(sg * h2[1][0], sg * h2[1][1], sg * h2[1][2], odd ? wa : wb);
}

// The rows of the 16 owned nodes of node layer k.
template <bool MASS>
__device__ __forceinline__ void node_layer(const LatticeArgs& A, int64_t i0, int64_t j0, int64_t k,
                                           unsigned char* smem) {
  const float2* rn = reinterpret_cast<const float2*>(smem + kSmRefN);
  const int lane = threadIdx.x & 31;
  const int ln = threadIdx.x >> 3;     // owned node of this lane
  const int e = threadIdx.x & 7;       // element around it: offset bits (x | y << 1 | z << 2)
  const int ex = e & 1, ey = (e >> 1) & 1, ez = e >> 2;
  const int lx = ln & 3, ly = ln >> 2;
  const unsigned char* info = smem + kSmPlaneInfo + ((int)(k & 1) * kNodes + ln) * kInfoBytes;
  const int nnb = reinterpret_cast<const int32_t*>(info)[3];
  const int64_t gx = i0 + lx - 1 + ex, gy = j0 + ly - 1 + ey, gz = k - 1 + ez;
  const bool valid = nnb > 0 && gx >= 0 && gx < A.nx && gy >= 0 && gy < A.ny && gz >= 0 && gz < A.nz;
  // the node's own vertex: lattice bits complement to the element's offset
  const int lbits = 7 - e;
  const int rot = (int)(gx & 1) | ((int)(gy & 1) << 1) | ((int)(gz & 1) << 2);
  const unsigned char* rec =
      smem + kSmElem + ((int)((k - 1 + ez) & 1) * kElems + (lx + ex) + kElem * (ly + ey)) * kRecBytes;
  const float4* XY = reinterpret_cast<const float4*>(rec + kRecXY);
  const float2* Z = reinterpret_cast<const float2*>(rec + kRecZ + 64 * (int)(gx & 1));
  const float4* R = reinterpret_cast<const float4*>(rec + kRecR);

  float r[3] = {0.f, 0.f, 0.f};
  // the lane's own weighted gradients and values as point pairs:
  // wg[qp][i] = (W grad_i N_a)(q0, q1), wn[qp] = (W N_a)(q0, q1)
  float2 wg[4][3], wn[4];
  if (valid) {
    float Wq[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) Wq[q] = R[q ^ rot].w;  // W_q sits in slot q ^ rot: eight lanes, eight slots
#pragma unroll
    for (int qp = 0; qp < 4; ++qp) {
      const float4 xy = XY[9 * qp + lbits];
      const float2 z = Z[8 * qp + lbits];
      const float w0 = Wq[2 * qp], w1 = Wq[2 * qp + 1];
      wg[qp][0] = make_float2(w0 * xy.x, w1 * xy.y);
      wg[qp][1] = make_float2(w0 * xy.z, w1 * xy.w);
      wg[qp][2] = make_float2(w0 * z.x, w1 * z.y);
      if constexpr (MASS) {
        const float2 na = rn[9 * qp + lbits];
        wn[qp] = make_float2(w0 * na.x, w1 * na.y);
      }
    }
    const float4 ra = R[lbits];  // the element's residual row of the node's vertex
    r[0] = ra.x; r[1] = ra.y; r[2] = ra.z;
  }
  const float bl = A.beta * A.lam, bm = A.beta * A.mu, am = A.alpha * A.rho;
  // entries start at float (rowstart & 1) of the node's stage row, so that
  // stage float4 j maps to an even, 16-byte aligned pair of FP64 entries
  const int so = (int)(*reinterpret_cast<const int64_t*>(info) & 1);
  float* stage = reinterpret_cast<float*>(smem + kSmStage) + ln * kStageRow + so;
  const uint8_t* npos = info + 16;
  const int rl = 3 * nnb;  // entries of one row
  // zeros around the node's entries: the parity slot and the float4 tail
  if (e == 7 && nnb > 0) {
    if (so) stage[-1] = 0.f;  // (the slot no writer touches)
    stage[9 * nnb] = 0.f;
    stage[9 * nnb + 1] = 0.f;
    stage[9 * nnb + 2] = 0.f;
  }
  const unsigned wmask = nnb > 0 ? (unsigned)(kWriters >> (8 * e)) & 0xffu : 0u;
  // slot c holds the block of the element vertex with bits c ^ lbits (bit per
  // axis: 0 = the node's own lattice line, 1 = this element's neighbour line)
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    float kv[9];
    if (valid) {
      const int bb = c ^ lbits;
      const float4* xyb = XY + bb;
      const float2* zb = Z + bb;
      float2 P[9], M = make_float2(0.f, 0.f);
#pragma unroll
      for (int t = 0; t < 9; ++t) P[t] = make_float2(0.f, 0.f);
#pragma unroll
      for (int qp = 0; qp < 4; ++qp) {
        const float4 xy = xyb[9 * qp];
        const float2 z = zb[8 * qp];
        const float2 gxp = make_float2(xy.x, xy.y), gyp = make_float2(xy.z, xy.w);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          P[3 * i + 0] = ffma2(wg[qp][i], gxp, P[3 * i + 0]);
          P[3 * i + 1] = ffma2(wg[qp][i], gyp, P[3 * i + 1]);
          P[3 * i + 2] = ffma2(wg[qp][i], z, P[3 * i + 2]);
        }
        if constexpr (MASS) M = ffma2(wn[qp], rn[9 * qp + bb], M);
      }
      float Ps[9];
#pragma unroll
      for (int t = 0; t < 9; ++t) Ps[t] = P[t].x + P[t].y;
      const float tp = Ps[0] + Ps[4] + Ps[8];
      const float md = MASS ? am * (M.x + M.y) : 0.f;
#pragma unroll
      for (int cc = 0; cc < 3; ++cc)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          float v = bl * Ps[3 * cc + d] + bm * Ps[3 * d + cc];
          if (cc == d) v += bm * tp + md;
          kv[3 * cc + d] = v;
        }
    } else {
#pragma unroll
      for (int t = 0; t < 9; ++t) kv[t] = 0.f;
    }
    // butterflies, x then y then z: on each axis where slot c has bit 0 (the
    // neighbour on the node's own line) the block is shared by the two
    // elements on either side; both lanes end with the same sum (a + b == b + a
    // in IEEE arithmetic)
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      if (c & (1 << ax)) continue;
#pragma unroll
      for (int t = 0; t < 9; ++t) kv[t] += __shfl_xor_sync(0xffffffffu, kv[t], 1 << ax);
    }
    // stage slot c: neighbour offset d_a = 0 (bit 0) or 2 e_a - 1 (bit 1);
    // kWriters names the lane that writes it
    if ((wmask >> c) & 1u) {
      const int dx = (c & 1) ? 2 * ex - 1 : 0, dy = (c & 2) ? 2 * ey - 1 : 0, dz = (c & 4) ? 2 * ez - 1 : 0;
      const int p = npos[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)];
      if (p != 0xff) {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
#pragma unroll
          for (int d = 0; d < 3; ++d) stage[cc * rl + 3 * p + d] = kv[3 * cc + d];
      }
    }
  }
#pragma unroll
  for (int ax = 0; ax < 3; ++ax)
#pragma unroll
    for (int t = 0; t < 3; ++t) r[t] += __shfl_xor_sync(0xffffffffu, r[t], 1 << ax);
  if (nnb > 0 && e == 0 && A.f) {
    const int32_t lid = reinterpret_cast<const int32_t*>(info)[2];
#pragma unroll
    for (int t = 0; t < 3; ++t) A.f[3 * (int64_t)lid + t] = widen(r[t]);
  }
  __syncwarp();
  // the warp's four nodes: coalesced FP64 stores of each node's 3 rows, a
  // float4 of the stage (four entries, two 16-byte stores) per lane and step
  const int wn0 = (threadIdx.x >> 5) * 4;
  // two nodes' loads and stores in flight
#pragma unroll 2
  for (int m = 0; m < 4; ++m) {
    const unsigned char* inf = smem + kSmPlaneInfo + ((int)(k & 1) * kNodes + wn0 + m) * kInfoBytes;
    const int nb = reinterpret_cast<const int32_t*>(inf)[3];
    if (nb == 0) continue;
    const int64_t rs = *reinterpret_cast<const int64_t*>(inf);
    const int o = (int)(rs & 1), n = 9 * nb, end = o + n;
    double* dst = A.vals + (rs - o);  // even: 16-byte aligned
    const float4* src = reinterpret_cast<const float4*>(smem + kSmStage + (wn0 + m) * kStageRow * 4);
    // exact FP32 -> FP64 widening: one entry of four by the hardware
    // conversion (on the FP64 pipe, which this kernel leaves idle; more than
    // one in four makes it the bottleneck), three by integer operations for
    // zeros and normal numbers: the exponent rebiased (not for a zero: times
    // min(|b|, 1)), the fraction moved up; a subnormal, infinity or NaN among
    // those (lane extremes of |b| and |b| - 1, one vote a node) sends them
    // through the hardware conversion afterwards.  The stage holds zeros
    // around the node's entries, so the extremes need no range test.
    uint32_t mx = 0u, mn = 0xffffffffu;
    for (int j = lane; 4 * j < end; j += 32) {
      const float4 v4 = src[j];
      const float v[4] = {v4.x, v4.y, v4.z, v4.w};
      double d[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (i == 0) {
          d[0] = (double)v[0];
          continue;
        }
        const uint32_t b = __float_as_uint(v[i]);
        const uint32_t a = b & 0x7fffffffu;  // zeros around the entries
        mx = max(mx, a);
        mn = min(mn, a - 1u);
        const uint32_t hi = min(a, 1u) * 0x38000000u + ((uint32_t)((int32_t)b >> 3) & 0x8fffffffu);
        d[i] = __hiloint2double((int)hi, (int)(b << 29));
      }
      if (4 * j >= o && 4 * j + 4 <= end) {
        __stcs(reinterpret_cast<double2*>(dst) + 2 * j, make_double2(d[0], d[1]));
        __stcs(reinterpret_cast<double2*>(dst) + 2 * j + 1, make_double2(d[2], d[3]));
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (4 * j + i >= o && 4 * j + i < end) __stcs(dst + 4 * j + i, d[i]);
      }
    }
    if (__any_sync(0xffffffffu, mx >= 0x7f800000u || mn < 0x007fffffu)) {
      const float* sf = reinterpret_cast<const float*>(src);
      for (int p = o + lane; p < end; p += 32) {
        const float v = sf[p];
        const uint32_t a = __float_as_uint(v) & 0x7fffffffu;
        if (a >= 0x7f800000u || (a != 0u && a < 0x00800000u)) __stcs(dst + p, (double)v);
      }
    }
  }
}

template <bool MASS>
__global__ void __launch_bounds__(kThreads, 3) k_lattice_gather(LatticeArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  // reference tables (hex8, 2 x 2 x 2 Gauss) from the packed FP64 tables
  // [w | geo_val | geo_grad | val | grad]: (dN^/dxi, N) of the vertex with
  // lattice bits B at point q, the values N at point pairs, and w_q
  {
    const double* ref = A.ref;
    float* rp = reinterpret_cast<float*>(smem + kSmRefP);
    float* rn = reinterpret_cast<float*>(smem + kSmRefN);
    float* rw = reinterpret_cast<float*>(smem + kSmRefW);
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {  // i = q * 8 + v (shards vertex v)
      const int q = i >> 3, B = vbits(i & 7), h = q & 1;
      const double* gr = ref + 8 + 64 + 192 + 64 + 3 * i;
      const float n = narrow(ref[8 + 64 + 192 + i]);
      float* slot = rp + 8 * (9 * (q >> 1) + B);  // two float4: x x y y | z z N N, point h in the h-th of each pair
      slot[h] = narrow(gr[0]);
      slot[2 + h] = narrow(gr[1]);
      slot[4 + h] = narrow(gr[2]);
      slot[6 + h] = n;
      rn[2 * (9 * (q >> 1) + B) + h] = n;
    }
    for (int i = threadIdx.x; i < 8; i += blockDim.x) rw[i] = narrow(ref[i]);
  }
  const int64_t tx_n = (A.nx + kTile) / kTile, ty_n = (A.ny + kTile) / kTile;  // node tiles: nx + 1 nodes
  const int64_t tz_n = (A.nz + A.zchunk) / A.zchunk;
  const int64_t ntask = tx_n * ty_n * tz_n;
  for (int64_t task = blockIdx.x; task < ntask; task += gridDim.x) {
    const int64_t tz = task / (tx_n * ty_n), rem = task - tz * tx_n * ty_n;
    const int64_t i0 = (rem % tx_n) * kTile, j0 = (rem / tx_n) * kTile;
    const int64_t k0 = tz * A.zchunk;
    const int64_t k1 = k0 + A.zchunk < A.nz + 1 ? k0 + A.zchunk : A.nz + 1;
    __syncthreads();  // the previous task's last reads of the rings are done
    // prologue: planes k0 - 1 and k0, element layer k0 - 1
    load_plane(A, i0, j0, k0 - 1, smem, (int)((k0 - 1) & 1));
    load_plane(A, i0, j0, k0, smem, (int)(k0 & 1));
    __syncthreads();
    element_layer<MASS>(A, i0, j0, k0 - 1, smem);
    for (int64_t k = k0; k < k1; ++k) {
      __syncthreads();  // node layer k - 1 done with plane slot (k + 1) & 1
      load_plane(A, i0, j0, k + 1, smem, (int)((k + 1) & 1));
      __syncthreads();
      element_layer<MASS>(A, i0, j0, k, smem);
      __syncthreads();
      node_layer<MASS>(A, i0, j0, k, smem);
    }
  }
}

// u and u_dot of every lattice node, FP32, in node GID order (x, y, z, 0).
__global__ void k_lattice_gather_u(const LatticeNode* nodes, int64_t n, const double* x, const double* xdot,
                                   float4* u, float4* ud) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = 3 * (int64_t)nodes[g].lid;
    u[g] = f4(narrow(x[l]), narrow(x[l + 1]), narrow(x[l + 2]), 0.f);
    if (xdot) ud[g] = f4(narrow(xdot[l]), narrow(xdot[l + 1]), narrow(xdot[l + 2]), 0.f);
  }
}

// Node layers per task: tasks (a node column's z chunk) go to the CTAs
// round-robin, so the kernel lasts as long as the CTA with the most tasks;
// each task adds one prologue element layer (about half a node layer's
// work).  Picks the chunk with the fewest half-layers on the heaviest CTA,
// the longer chunk on a tie.
int64_t choose_zchunk(int64_t nx, int64_t ny, int64_t nz, int64_t grid) {
  const int64_t cols = ((nx + kTile) / kTile) * ((ny + kTile) / kTile), layers = nz + 1;
  int64_t best = layers, best_cost = -1;
  for (int64_t zc = 1; zc <= layers; ++zc) {
    const int64_t ntask = cols * ((layers + zc - 1) / zc);
    const int64_t g = std::min<int64_t>(std::max<int64_t>(grid, 1), ntask);
    const int64_t cost = (ntask + g - 1) / g * (2 * zc + 1);
    if (best_cost < 0 || cost <= best_cost) best_cost = cost, best = zc;
  }
  return best;
}

template <bool MASS>
cudaError_t launch_main(const LatticeArgs& A, int sms, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_lattice_gather<MASS>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lattice_gather<MASS>, kThreads, kSmBytes);
  if (e != cudaSuccess) return e;
  int64_t grid = (int64_t)(per_sm > 0 ? per_sm : 1) * sms;
  if (A.grid > 0 && A.grid < grid) grid = A.grid;
  LatticeArgs B = A;
  B.zchunk = choose_zchunk(A.nx, A.ny, A.nz, grid);
  const int64_t ntask = ((A.nx + kTile) / kTile) * ((A.ny + kTile) / kTile) * ((A.nz + B.zchunk) / B.zchunk);
  if (grid > ntask) grid = ntask;
  k_lattice_gather<MASS><<<(unsigned)grid, kThreads, kSmBytes, s>>>(B);
  return cudaGetLastError();
}

}  // namespace

size_t lattice_gather_smem() { return kSmBytes; }

cudaError_t launch_lattice_gather(LatticeArgs A, float4* u_work, float4* ud_work, const double* x, const double* xdot,
                                  cudaStream_t s) {
  const int64_t n_nodes = (A.nx + 1) * (A.ny + 1) * (A.nz + 1);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  {
    const int64_t blocks = std::min<int64_t>((n_nodes + 255) / 256, (int64_t)sms * 8);
    k_lattice_gather_u<<<(unsigned)blocks, 256, 0, s>>>(A.nodes, n_nodes, x, xdot, u_work, xdot ? ud_work : nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  A.u = reinterpret_cast<const float*>(u_work);
  A.ud = xdot ? reinterpret_cast<const float*>(ud_work) : nullptr;
  // the time-derivative (mass) terms only where they contribute
  const bool mass = A.rho != 0.f && (A.alpha != 0.f || xdot != nullptr);
  return mass ? launch_main<true>(A, sms, s) : launch_main<false>(A, sms, s);
}

}  // namespace tx
