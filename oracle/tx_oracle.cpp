// tx_oracle.cpp -- CPU restatement of the Tianxin/Panzer FE assembly path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU library is
// checked against: only tests/, __graft_entry__.smoke() and the bench's
// cpu_baseline leg load it.  Nothing in the product links or calls it.
//
// It restates, in plain C++ and FP64, what the reference computes on one
// rank (Kokkos Serial/OpenMP semantics):
//   * Cartesian topology and entity GIDs
//       dof-mgr/test/cartesian_topology/CartesianConnManager.cpp:159-331,744-890
//   * GUN numbering, element GIDs, owned_ first-touch order, LIDs, offsets
//       dof-mgr/src/Panzer_DOFManager.cpp:474-716, 719-866, 869-975, 1261-1372
//       dof-mgr/src/Panzer_FieldAggPattern.cpp:204-246, 369-413
//   * CRS graph (union of element cliques, columns ascending)
//       disc-fe/src/lof/Panzer_TpetraLinearObjFactory_impl.hpp:559-651
//   * Geometry (J, det, inverse, weighted measure) and basis transforms
//       disc-fe/src/Panzer_IntegrationValues2.cpp:946-1182
//       disc-fe/src/Panzer_BasisValues2_impl.hpp:1036-1515, 1670-1815
//   * Gather with forward-mode AD seeds (x: beta, x_dot: alpha, derivative
//     slot = element offset)
//       disc-fe/src/evaluators/Panzer_GatherSolution_Tpetra_impl.hpp:548-649
//   * Integrators  GradBasisDotVector (..._impl.hpp:225-294),
//     BasisTimesScalar (..._impl.hpp:215-270)
//   * Scatter: atomic f += r.val(); sumIntoValues(row, lids, r.dx())
//       disc-fe/src/evaluators/Panzer_ScatterResidual_Tpetra_impl.hpp:390-439
//   * Dirichlet: f = x - g, Jacobian row -> unit row
//       disc-fe/src/evaluators/TianXin_Dirichlet_impl.hpp:55-81,
//       disc-fe/src/lof/Panzer_TpetraLinearObjContainer.hpp:228-238,306-318
//   * Integral responses: sum of integrand * weighted measure over a block
//     (TianXin Response_Integral, disc-fe/src/responses/
//     TianXin_Response_Integral_impl.hpp:106-130) and its gradient (panzer
//     functional, Panzer_ResponseScatterEvaluator_Functional_impl.hpp:143-171);
//     L2/H1 error integrands of adapters-stk/example/PoissonExample/
//     Example_ClosureModel_Factory_impl.hpp:147-230 for u* = sin sin sin
//   * Neumann flux: residual(cell, b) += val * N_b * w * |face normal| on the
//     side workset of a block (TianXin::Flux, disc-fe/src/evaluators/
//     TianXin_Neumann_impl.hpp:146-166; side worksets adapters-stk/src/
//     Panzer_STK_SetupUtilities.cpp:306-392)
//
// Definitions the reference leaves to Intrepid2 (not in the reference tree)
// are restated from the mathematics: tensor Gauss-Legendre cubature with the
// 1-D points in descending order (pinned by the reference's first IP at
// ((1+1/sqrt3)/2, ...), disc-fe/test/core_tests/integration_values2.cpp:
// 103-110), x-fastest tensor ordering (unpinned), shards node/edge/face
// order, hex27 sub-cell map (pinned by dof-mgr/test/dofmngr_test/
// tIntrepidFieldPattern.cpp:527-573), lowest-order Nedelec hex functions
// with edge signs from vertex GIDs.  Elasticity, k(T) heat and the mass
// term on the time-derivative vector have no equation set in the reference
// and are defined here from the same integrators.
//
// Build: see oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/tianxin_gb300.h"

namespace orc {

typedef int64_t GO;
typedef int32_t LO;

// ------------------------------------------------------------------ RNG
// Jitter: counter-based splitmix64 of (seed, vertex GID, component), mapped
// to a double in [-1, 1).  The GPU library generates the same lattice.
static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline double jitter_unit(uint64_t seed, GO vertex, int comp) {
  uint64_t h = mix64(seed ^ mix64((uint64_t)vertex * 3ull + (uint64_t)comp));
  double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);  // [0,1)
  return 2.0 * u - 1.0;
}

// ---------------------------------------------------------- brick tables
// shards Hexahedron<8> vertices on [-1,1]^3
static const int kHexVert[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                   {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
// shards hex edges (vertex pairs, first -> second is the local direction)
static const int kHexEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                    {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// shards hex faces
static const int kHexFace[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6},
                                   {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
// brick -> 6 tets (CartesianConnManager.cpp:220-227)
static const int kTetInHex[6][4] = {{0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6},
                                    {0, 5, 6, 4}, {1, 5, 6, 0}, {1, 6, 2, 0}};
// tet edges in brick-edge ids; 12..17 face diagonals, 18 body diagonal (:232-239)
static const int kTetEdgeInHex[6][6] = {{16, 2, 3, 18, 10, 14}, {3, 11, 15, 18, 14, 6},
                                        {15, 7, 8, 18, 6, 17},  {12, 5, 18, 8, 4, 17},
                                        {9, 5, 13, 0, 12, 18},  {13, 10, 1, 0, 18, 16}};
// tet faces in brick-face ids (:243-250)
static const int kTetFaceInHex[6][4] = {{12, 4, 13, 8}, {13, 5, 14, 7}, {14, 10, 15, 6},
                                        {1, 11, 15, 16}, {0, 16, 17, 2}, {17, 12, 9, 3}};
// shards Tetrahedron<4> edges
static const int kTetEdge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
static const int kTetFace[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 2, 3}, {0, 1, 2}};

// --------------------------------------------------------- reference elem
// Basis: number of functions and the sub-cell -> basis-index map
// (Intrepid2 DOF tags as seen by Panzer's IntrepidFieldPattern).
struct BasisDef {
  int topo = 0, kind = 0;  // topology, tx_basis
  int nb = 0;
  int nsub[4] = {0, 0, 0, 0};
  std::vector<int> sub[4];  // basis index per sub-cell, -1 if none
  bool hcurl = false;
};

static BasisDef make_basis(int topo, int kind) {
  BasisDef b;
  b.topo = topo;
  b.kind = kind;
  if (topo == TX_TOPO_HEX) {
    b.nsub[0] = 8; b.nsub[1] = 12; b.nsub[2] = 6; b.nsub[3] = 1;
  } else {
    b.nsub[0] = 4; b.nsub[1] = 6; b.nsub[2] = 4; b.nsub[3] = 1;
  }
  for (int d = 0; d < 4; ++d) b.sub[d].assign(b.nsub[d], -1);
  if (topo == TX_TOPO_HEX && kind == TX_HGRAD_C1) {
    b.nb = 8;
    for (int i = 0; i < 8; ++i) b.sub[0][i] = i;
  } else if (topo == TX_TOPO_HEX && kind == TX_HGRAD_C2) {
    b.nb = 27;
    for (int i = 0; i < 8; ++i) b.sub[0][i] = i;
    const int edge_node[12] = {8, 9, 10, 11, 16, 17, 18, 19, 12, 13, 14, 15};
    for (int i = 0; i < 12; ++i) b.sub[1][i] = edge_node[i];
    const int face_node[6] = {25, 24, 26, 23, 21, 22};
    for (int i = 0; i < 6; ++i) b.sub[2][i] = face_node[i];
    b.sub[3][0] = 20;
  } else if (topo == TX_TOPO_TET && kind == TX_HGRAD_C1) {
    b.nb = 4;
    for (int i = 0; i < 4; ++i) b.sub[0][i] = i;
  } else if (topo == TX_TOPO_TET && kind == TX_HGRAD_C2) {
    b.nb = 10;
    for (int i = 0; i < 4; ++i) b.sub[0][i] = i;
    for (int i = 0; i < 6; ++i) b.sub[1][i] = 4 + i;
  } else if (topo == TX_TOPO_HEX && kind == TX_HCURL_I1) {
    b.nb = 12;
    b.hcurl = true;
    for (int i = 0; i < 12; ++i) b.sub[1][i] = i;
  } else {
    throw std::runtime_error("unsupported topology/basis combination");
  }
  return b;
}

// hex27 node positions on [-1,1]^3 (shards Hexahedron<27>)
static void hex27_node(int n, int p[3]) {
  if (n < 8) { for (int d = 0; d < 3; ++d) p[d] = kHexVert[n][d]; return; }
  if (n == 20) { p[0] = p[1] = p[2] = 0; return; }
  if (n >= 21) {
    static const int face_of[6] = {4, 5, 3, 1, 0, 2};  // node 21..26 -> shards face
    const int* f = kHexFace[face_of[n - 21]];
    for (int d = 0; d < 3; ++d)
      p[d] = (kHexVert[f[0]][d] + kHexVert[f[1]][d] + kHexVert[f[2]][d] + kHexVert[f[3]][d]) / 4;
    return;
  }
  static const int edge_of[12] = {0, 1, 2, 3, 8, 9, 10, 11, 4, 5, 6, 7};  // node 8..19 -> edge
  const int* e = kHexEdge[edge_of[n - 8]];
  for (int d = 0; d < 3; ++d) p[d] = (kHexVert[e[0]][d] + kHexVert[e[1]][d]) / 2;
}

static inline double lag1(int a, double s) { return 0.5 * (1.0 + a * s); }
static inline double dlag1(int a, double) { return 0.5 * a; }
static inline double lag2(int a, double s) {
  return a == 0 ? 1.0 - s * s : 0.5 * s * (s + a);
}
static inline double dlag2(int a, double s) { return a == 0 ? -2.0 * s : s + 0.5 * a; }

// Scalar HGRAD basis values and reference gradients at point xi.
static void eval_hgrad(const BasisDef& B, const double xi[3], double* N, double (*dN)[3]) {
  if (B.topo == TX_TOPO_HEX && B.kind == TX_HGRAD_C1) {
    for (int n = 0; n < 8; ++n) {
      const int* v = kHexVert[n];
      double a = lag1(v[0], xi[0]), b = lag1(v[1], xi[1]), c = lag1(v[2], xi[2]);
      N[n] = a * b * c;
      dN[n][0] = dlag1(v[0], xi[0]) * b * c;
      dN[n][1] = a * dlag1(v[1], xi[1]) * c;
      dN[n][2] = a * b * dlag1(v[2], xi[2]);
    }
  } else if (B.topo == TX_TOPO_HEX && B.kind == TX_HGRAD_C2) {
    for (int n = 0; n < 27; ++n) {
      int p[3];
      hex27_node(n, p);
      double a = lag2(p[0], xi[0]), b = lag2(p[1], xi[1]), c = lag2(p[2], xi[2]);
      N[n] = a * b * c;
      dN[n][0] = dlag2(p[0], xi[0]) * b * c;
      dN[n][1] = a * dlag2(p[1], xi[1]) * c;
      dN[n][2] = a * b * dlag2(p[2], xi[2]);
    }
  } else if (B.topo == TX_TOPO_TET) {
    double L[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
    const double dL[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    if (B.kind == TX_HGRAD_C1) {
      for (int n = 0; n < 4; ++n) {
        N[n] = L[n];
        for (int d = 0; d < 3; ++d) dN[n][d] = dL[n][d];
      }
    } else {
      for (int n = 0; n < 4; ++n) {
        N[n] = L[n] * (2.0 * L[n] - 1.0);
        for (int d = 0; d < 3; ++d) dN[n][d] = (4.0 * L[n] - 1.0) * dL[n][d];
      }
      for (int e = 0; e < 6; ++e) {
        int i = kTetEdge[e][0], j = kTetEdge[e][1];
        N[4 + e] = 4.0 * L[i] * L[j];
        for (int d = 0; d < 3; ++d) dN[4 + e][d] = 4.0 * (dL[i][d] * L[j] + L[i] * dL[j][d]);
      }
    }
  } else {
    throw std::runtime_error("eval_hgrad: not an HGRAD basis");
  }
}

// Lowest-order Nedelec hex: values and reference curls at xi.  Function i
// is tangential to shards edge i, oriented first->second vertex, dual to the
// degrees of freedom L_j(u) = u(m_j) . t_j, m_j the midpoint of edge j and t_j
// its reference tangent (half the edge vector, a unit vector on [-1,1]^3).
// That is the quadrilateral convention the reference pins
// (disc-fe/test/core_tests/basis_values2.cpp:404-406: value -0.5 (y - 1) and
// curl 0.5 for quad edge 0), and it makes the tangential trace of every hex
// function on a face the quadrilateral function of that face's edge:
// function 0 = (1 - y)(1 - z)/4 e_x restricted to z = -1 is 0.5 (1 - y) e_x.
static void eval_hcurl_hex(const double xi[3], double (*V)[3], double (*C)[3]) {
  const double x = xi[0], y = xi[1], z = xi[2];
  for (int i = 0; i < 12; ++i)
    for (int d = 0; d < 3; ++d) V[i][d] = C[i][d] = 0.0;
  // x-directed edges 0 (y-,z-,+x) 2 (y+,z-,-x) 4 (y-,z+,+x) 6 (y+,z+,-x)
  const int xe[4] = {0, 2, 4, 6};
  const int xs[4][3] = {{-1, -1, 1}, {1, -1, -1}, {-1, 1, 1}, {1, 1, -1}};  // sy, sz, direction
  for (int k = 0; k < 4; ++k) {
    double sy = xs[k][0], sz = xs[k][1], dir = xs[k][2];
    V[xe[k]][0] = dir * (1 + sy * y) * (1 + sz * z) / 4.0;
    // curl of (f,0,0) = (0, df/dz, -df/dy)
    C[xe[k]][1] = dir * (1 + sy * y) * sz / 4.0;
    C[xe[k]][2] = -dir * sy * (1 + sz * z) / 4.0;
  }
  // y-directed edges 1 (x+,z-,+y) 3 (x-,z-,-y) 5 (x+,z+,+y) 7 (x-,z+,-y)
  const int ye[4] = {1, 3, 5, 7};
  const int ys[4][3] = {{1, -1, 1}, {-1, -1, -1}, {1, 1, 1}, {-1, 1, -1}};  // sx, sz, direction
  for (int k = 0; k < 4; ++k) {
    double sx = ys[k][0], sz = ys[k][1], dir = ys[k][2];
    V[ye[k]][1] = dir * (1 + sx * x) * (1 + sz * z) / 4.0;
    // curl of (0,g,0) = (-dg/dz, 0, dg/dx)
    C[ye[k]][0] = -dir * (1 + sx * x) * sz / 4.0;
    C[ye[k]][2] = dir * sx * (1 + sz * z) / 4.0;
  }
  // z-directed edges 8..11 at (x,y) = (-,-), (+,-), (+,+), (-,+), all +z
  const int zs[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  for (int k = 0; k < 4; ++k) {
    double sx = zs[k][0], sy = zs[k][1];
    V[8 + k][2] = (1 + sx * x) * (1 + sy * y) / 4.0;
    // curl of (0,0,h) = (dh/dy, -dh/dx, 0)
    C[8 + k][0] = (1 + sx * x) * sy / 4.0;
    C[8 + k][1] = -sx * (1 + sy * y) / 4.0;
  }
}

// ------------------------------------------------------------- cubature
static void gauss_1d(int n, std::vector<double>& p, std::vector<double>& w) {
  // descending order (+ .. -)
  p.clear(); w.clear();
  switch (n) {
    case 1: p = {0.0}; w = {2.0}; break;
    case 2: { double a = 1.0 / std::sqrt(3.0); p = {a, -a}; w = {1.0, 1.0}; } break;
    case 3: { double a = std::sqrt(0.6); p = {a, 0.0, -a}; w = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0}; } break;
    case 4: {
      double a = std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * std::sqrt(1.2));
      double b = std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * std::sqrt(1.2));
      double wa = (18.0 - std::sqrt(30.0)) / 36.0, wb = (18.0 + std::sqrt(30.0)) / 36.0;
      p = {a, b, -b, -a}; w = {wa, wb, wb, wa};
    } break;
    default: throw std::runtime_error("gauss_1d: unsupported point count");
  }
}

struct Cubature { int np = 0; std::vector<double> xi; std::vector<double> w; };

static Cubature make_cubature(int topo, int degree) {
  Cubature c;
  if (topo == TX_TOPO_HEX) {
    int n = degree / 2 + 1;
    std::vector<double> p, w;
    gauss_1d(n, p, w);
    c.np = n * n * n;
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          c.xi.push_back(p[i]); c.xi.push_back(p[j]); c.xi.push_back(p[k]);
          c.w.push_back(w[i] * w[j] * w[k]);
        }
  } else {
    if (degree <= 1) {
      c.np = 1; c.xi = {0.25, 0.25, 0.25}; c.w = {1.0 / 6.0};
    } else if (degree == 2) {
      const double a = 0.5854101966249685, b = 0.1381966011250105;
      c.np = 4;
      c.xi = {b, b, b, a, b, b, b, a, b, b, b, a};
      c.w = {1.0 / 24, 1.0 / 24, 1.0 / 24, 1.0 / 24};
    } else {
      throw std::runtime_error("tet cubature degree > 2 not provided");
    }
  }
  return c;
}

static int default_degree(int topo, int basis) {
  if (topo == TX_TOPO_HEX && basis == TX_HGRAD_C2) return 4;
  return 2;
}

// -------------------------------------------------------------- topology
// One-rank CartesianConnManager with a topology per block.
struct Topology {
  GO NX, NY, NZ;           // bricks
  int nx, ny, nz, bx, by, bz;
  int nblocks;
  int block_topo[TX_MAX_BLOCKS];
  GO totalNodes, hexEdges, hexFaces, bricks;
  double lx, ly, lz, jitter;
  uint64_t seed;
  // element enumeration
  std::vector<GO> elem_brick;           // element -> brick
  std::vector<int> elem_sub;            // element -> sub element
  std::vector<std::vector<LO>> block_elems;

  int brick_block(GO I, GO J, GO K) const {
    int bi = (int)(I / nx), bj = (int)(J / ny), bk = (int)(K / nz);
    return (bi * by + bj) * bz + bk;
  }
  void brick_ijk(GO b, GO& I, GO& J, GO& K) const {
    K = b / (NX * NY); J = (b - K * NX * NY) / NX; I = b - K * NX * NY - J * NX;
  }
  GO node_gid(GO I, GO J, GO K, int n) const {
    return (NX + 1) * (NY + 1) * (K + (n >= 4)) + (NX + 1) * (J + (n == 2 || n == 3 || n == 6 || n == 7)) +
           I + (n == 1 || n == 2 || n == 5 || n == 6);
  }
  // brick-level edge ids 0..11 hex, 12..18 tet diagonals (updateConnectivity_3d, subcellDim==1)
  GO edge_gid(GO I, GO J, GO K, int e) const {
    GO kshift = (NX + 1) * NY + NX * (NY + 1) + (NX + 1) * (NY + 1);
    GO base = I + J * (2 * NX + 1) + K * kshift;
    GO g = totalNodes + base;
    if (e == 0) g += 0;
    if (e == 1) g += NX + 1;
    if (e == 2) g += 2 * NX + 1;
    if (e == 3) g += NX;
    if (e == 4) g += kshift;
    if (e == 5) g += kshift + NX + 1;
    if (e == 6) g += kshift + 2 * NX + 1;
    if (e == 7) g += kshift + NX;
    if (e >= 8 && e <= 11) {
      g += (NX + 1) * NY + NX * (NY + 1) - J * NX;
      if (e == 9) g += 1;
      if (e == 10) g += NX + 2;
      if (e == 11) g += NX + 1;
    }
    if (e >= 12 && e <= 17) {
      GO fk = NX * NY + (NX + 1) * NY + NX * (NY + 1);
      g = totalNodes + hexEdges + I + J * NX + K * fk;
      if (e >= 12 && e <= 15) {
        g += NX * NY + (J + 1) * (NX + 1);
        if (e == 12) g += -NX - 1;
        if (e == 14) g += NX;
        if (e == 15) g += -1;
      }
      if (e == 17) g += fk;
    }
    if (e == 18) g = totalNodes + hexEdges + hexFaces + (I + NX * J + NX * NY * K);
    return g;
  }
  GO hexface_gid(GO I, GO J, GO K, int f) const {
    GO fk = NX * NY + (NX + 1) * NY + NX * (NY + 1);
    GO g = totalNodes + hexEdges + I + J * NX + K * fk;
    if (f <= 3) {
      g += NX * NY + (J + 1) * (NX + 1);
      if (f == 0) g += -NX - 1;
      if (f == 2) g += NX;
      if (f == 3) g += -1;
    }
    if (f == 5) g += fk;
    return g;
  }
  GO tetface_gid(GO I, GO J, GO K, int f) const {
    GO fk = NX * NY + (NX + 1) * NY + NX * (NY + 1);
    GO base = I + J * NX + K * fk;
    GO tetEdges = hexEdges + hexFaces + bricks;
    GO g = totalNodes + tetEdges + 2 * base;
    if (f < 8) {
      g += 2 * (NX * NY + (J + 1) * (NX + 1));
      const GO off[8] = {-2 * (NX + 1), -2 * (NX + 1) + 1, 0, 1, 2 * NX, 2 * NX + 1, -2, -1};
      g += off[f];
    }
    if (f == 9) g += 1;
    if (f == 10) g += 2 * fk;
    if (f == 11) g += 2 * fk + 1;
    if (f >= 12) g = totalNodes + tetEdges + 2 * hexFaces + 6 * (I + NX * J + NX * NY * K) + (f - 12);
    return g;
  }
  GO cell_gid(GO I, GO J, GO K, int topo, int sub) const {
    GO b = I + NX * J + NX * NY * K;
    if (topo == TX_TOPO_HEX) return totalNodes + hexEdges + hexFaces + b;
    return totalNodes + (hexEdges + hexFaces + bricks) + (2 * hexFaces + 6 * bricks) + 6 * b + sub;
  }
  // GID of sub-cell (dim, c) of element e
  GO entity_gid(LO e, int dim, int c) const {
    GO I, J, K;
    brick_ijk(elem_brick[e], I, J, K);
    int topo = block_topo[brick_block(I, J, K)];
    int sub = elem_sub[e];
    if (dim == 0) return node_gid(I, J, K, topo == TX_TOPO_HEX ? c : kTetInHex[sub][c]);
    if (dim == 1) return edge_gid(I, J, K, topo == TX_TOPO_HEX ? c : kTetEdgeInHex[sub][c]);
    if (dim == 2) return topo == TX_TOPO_HEX ? hexface_gid(I, J, K, c) : tetface_gid(I, J, K, kTetFaceInHex[sub][c]);
    return cell_gid(I, J, K, topo, sub);
  }
  int elem_topo(LO e) const {
    GO I, J, K;
    brick_ijk(elem_brick[e], I, J, K);
    return block_topo[brick_block(I, J, K)];
  }
  // local vertex -> brick vertex
  int brick_vertex(LO e, int v) const { return elem_topo(e) == TX_TOPO_HEX ? v : kTetInHex[elem_sub[e]][v]; }
  void vertex_lattice(GO I, GO J, GO K, int n, GO& i, GO& j, GO& k) const {
    i = I + (n == 1 || n == 2 || n == 5 || n == 6);
    j = J + (n == 2 || n == 3 || n == 6 || n == 7);
    k = K + (n >= 4);
  }
  void vertex_xyz(GO i, GO j, GO k, double x[3]) const {
    GO g = (NX + 1) * (NY + 1) * k + (NX + 1) * j + i;
    const double h[3] = {lx / NX, ly / NY, lz / NZ};
    const GO ii[3] = {i, j, k};
    const GO nn[3] = {NX, NY, NZ};
    bool interior = i > 0 && i < NX && j > 0 && j < NY && k > 0 && k < NZ;
    for (int d = 0; d < 3; ++d) {
      x[d] = (double)ii[d] * h[d];
      if (interior && jitter != 0.0) x[d] = x[d] + jitter * h[d] * jitter_unit(seed, g, d);
      (void)nn;
    }
  }
  void elem_vertices(LO e, int nv, double* xyz) const {
    GO I, J, K;
    brick_ijk(elem_brick[e], I, J, K);
    for (int v = 0; v < nv; ++v) {
      GO i, j, k;
      vertex_lattice(I, J, K, brick_vertex(e, v), i, j, k);
      vertex_xyz(i, j, k, xyz + 3 * v);
    }
  }
};

static void build_topology(Topology& T, const tx_mesh_desc& d) {
  if (d.nx <= 0 || d.ny <= 0 || d.nz <= 0 || d.bx <= 0 || d.by <= 0 || d.bz <= 0)
    throw std::runtime_error("mesh: non-positive size");
  T.nx = d.nx; T.ny = d.ny; T.nz = d.nz; T.bx = d.bx; T.by = d.by; T.bz = d.bz;
  T.nblocks = d.bx * d.by * d.bz;
  if (T.nblocks > TX_MAX_BLOCKS) throw std::runtime_error("mesh: too many blocks");
  for (int b = 0; b < T.nblocks; ++b) T.block_topo[b] = d.block_topology[b];
  T.NX = (GO)d.nx * d.bx; T.NY = (GO)d.ny * d.by; T.NZ = (GO)d.nz * d.bz;
  T.totalNodes = (T.NX + 1) * (T.NY + 1) * (T.NZ + 1);
  T.hexEdges = (T.NX + 1) * T.NY * (T.NZ + 1) + T.NX * (T.NY + 1) * (T.NZ + 1) + (T.NX + 1) * (T.NY + 1) * T.NZ;
  T.hexFaces = T.NX * T.NY * (T.NZ + 1) + T.NX * (T.NY + 1) * T.NZ + (T.NX + 1) * T.NY * T.NZ;
  T.bricks = T.NX * T.NY * T.NZ;
  T.lx = d.lx; T.ly = d.ly; T.lz = d.lz; T.jitter = d.jitter; T.seed = d.seed;
  T.block_elems.assign(T.nblocks, {});
  for (GO b = 0; b < T.bricks; ++b) {
    GO I, J, K;
    T.brick_ijk(b, I, J, K);
    int blk = T.brick_block(I, J, K);
    int nsub = T.block_topo[blk] == TX_TOPO_HEX ? 1 : 6;
    for (int s = 0; s < nsub; ++s) {
      T.block_elems[blk].push_back((LO)T.elem_brick.size());
      T.elem_brick.push_back(b);
      T.elem_sub.push_back(s);
    }
  }
}

// -------------------------------------------------------------- physics
static int physics_nfields(int phys) { return phys == TX_PHYS_ELASTICITY ? 3 : 1; }

// ----------------------------------------------------------- DOF manager
struct DofManager {
  int nfields = 0;
  std::vector<BasisDef> block_basis;      // per block
  std::vector<int> block_degree;
  // geometric aggregate pattern per block: (dim, subcell) included
  std::vector<std::vector<std::pair<int, int>>> geom;    // per block
  std::vector<std::vector<int>> geom_ndof;               // per block per geom id: dofs per field
  std::vector<std::vector<GO>> conn;                      // per element
  std::vector<std::vector<GO>> elementGIDs;               // per element
  std::vector<std::vector<LO>> elementLIDs;
  std::vector<std::vector<std::vector<int>>> offsets;    // [block][field][basis]
  std::vector<GO> owned;                                  // LID -> GID
  std::vector<LO> g2l;                                    // GID -> LID (GIDs are 0..N-1 on one rank)
  // graph
  std::vector<int64_t> rowptr;
  std::vector<LO> colind;
  // per element, orientation signs for HCURL edges
  std::vector<std::vector<signed char>> edge_sign;
};

static void build_dofs(const Topology& T, DofManager& D, const tx_equation_set_desc& q) {
  D.nfields = physics_nfields(q.physics);
  const int nf = D.nfields;
  const GO nelem = (GO)T.elem_brick.size();
  D.block_basis.clear();
  D.block_degree.clear();
  bool need_orient = false;
  for (int b = 0; b < T.nblocks; ++b) {
    D.block_basis.push_back(make_basis(T.block_topo[b], q.block_basis[b]));
    int deg = q.integration_order[b] > 0 ? q.integration_order[b] : default_degree(T.block_topo[b], q.block_basis[b]);
    D.block_degree.push_back(deg);
    if (D.block_basis.back().hcurl) need_orient = true;
  }
  if (q.physics == TX_PHYS_MAXWELL) {
    for (int b = 0; b < T.nblocks; ++b)
      if (!D.block_basis[b].hcurl) throw std::runtime_error("MAXWELL needs an HCURL basis");
  } else {
    for (int b = 0; b < T.nblocks; ++b)
      if (D.block_basis[b].hcurl) throw std::runtime_error("HCURL basis needs MAXWELL physics");
  }
  // GeometricAggFieldPattern: sub-cells carrying ids (all fields share the
  // block basis); nodes added when orientations are required
  // (Panzer_DOFManager.cpp:452-456).
  D.geom.assign(T.nblocks, {});
  D.geom_ndof.assign(T.nblocks, {});
  for (int b = 0; b < T.nblocks; ++b) {
    const BasisDef& B = D.block_basis[b];
    for (int dim = 0; dim < 4; ++dim)
      for (int c = 0; c < B.nsub[dim]; ++c) {
        bool has = B.sub[dim][c] >= 0 || (need_orient && dim == 0);
        if (has) {
          D.geom[b].push_back({dim, c});
          D.geom_ndof[b].push_back(B.sub[dim][c] >= 0 ? 1 : 0);
        }
      }
  }
  // connectivity (CartesianConnManager::buildConnectivity)
  D.conn.assign(nelem, {});
  for (int b = 0; b < T.nblocks; ++b)
    for (LO e : T.block_elems[b])
      for (auto& dc : D.geom[b]) D.conn[e].push_back(T.entity_gid(e, dc.first, dc.second));
  // overlap map: sorted unique entity GIDs (buildOverlapMapFromElements)
  std::vector<GO> overlap;
  for (GO e = 0; e < nelem; ++e) overlap.insert(overlap.end(), D.conn[e].begin(), D.conn[e].end());
  std::sort(overlap.begin(), overlap.end());
  overlap.erase(std::unique(overlap.begin(), overlap.end()), overlap.end());
  auto ov_index = [&](GO g) { return (size_t)(std::lower_bound(overlap.begin(), overlap.end(), g) - overlap.begin()); };
  // tagged multivector: max over elements of DOFs per (entity, field)
  std::vector<GO> tagged(overlap.size() * nf, 0);
  for (int b = 0; b < T.nblocks; ++b)
    for (LO e : T.block_elems[b])
      for (size_t c = 0; c < D.conn[e].size(); ++c) {
        size_t lid = ov_index(D.conn[e][c]);
        for (int f = 0; f < nf; ++f) {
          GO cnt = D.geom_ndof[b][c];
          if (cnt > tagged[lid * nf + f]) tagged[lid * nf + f] = cnt;
        }
      }
  // GUN GID assignment (Panzer_DOFManager.cpp:827-843): entity-major, field-minor
  std::vector<GO> base(overlap.size() * nf, -1);
  GO which = 0;
  for (size_t i = 0; i < overlap.size(); ++i)
    for (int f = 0; f < nf; ++f)
      if (tagged[i * nf + f] != 0) {
        base[i * nf + f] = which;
        which += tagged[i * nf + f];
      }
  // element GIDs (fillGIDsFromOverlappedMV)
  D.elementGIDs.assign(nelem, {});
  for (int b = 0; b < T.nblocks; ++b) {
    const std::vector<LO>& be = T.block_elems[b];
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < be.size(); ++i) {
      const LO e = be[i];
      auto& g = D.elementGIDs[e];
      for (size_t c = 0; c < D.conn[e].size(); ++c) {
        size_t lid = ov_index(D.conn[e][c]);
        for (int f = 0; f < nf; ++f)
          for (int k = 0; k < D.geom_ndof[b][c]; ++k) g.push_back(base[lid * nf + f] + k);
      }
    }
  }
  // offsets per field (FieldAggPattern::localOffsets_build)
  D.offsets.assign(T.nblocks, std::vector<std::vector<int>>(nf));
  for (int b = 0; b < T.nblocks; ++b) {
    const BasisDef& B = D.block_basis[b];
    int pos = 0;
    for (int f = 0; f < nf; ++f) D.offsets[b][f].assign(B.nb, -1);
    for (size_t c = 0; c < D.geom[b].size(); ++c) {
      int dim = D.geom[b][c].first, sc = D.geom[b][c].second;
      for (int f = 0; f < nf; ++f)
        for (int k = 0; k < D.geom_ndof[b][c]; ++k) D.offsets[b][f][B.sub[dim][sc]] = pos++;
    }
  }
  // owned_: first touch in block order, element order, GID order
  std::vector<unsigned char> seen((size_t)which, 0);
  D.owned.clear();
  for (int b = 0; b < T.nblocks; ++b)
    for (LO e : T.block_elems[b])
      for (GO g : D.elementGIDs[e])
        if (!seen[g]) {
          seen[g] = 1;
          D.owned.push_back(g);
        }
  if ((GO)D.owned.size() != which) throw std::runtime_error("numbering failure: owned count mismatch");
  D.g2l.assign((size_t)which, -1);
  for (size_t i = 0; i < D.owned.size(); ++i) D.g2l[D.owned[i]] = (LO)i;
  D.elementLIDs.assign(nelem, {});
#pragma omp parallel for schedule(static)
  for (GO e = 0; e < nelem; ++e)
    for (GO g : D.elementGIDs[e]) D.elementLIDs[e].push_back(D.g2l[g]);
  // edge orientations (lowest-order HCURL): +1 if the local edge direction
  // runs from the lower to the higher vertex GID
  D.edge_sign.assign(nelem, {});
  if (need_orient)
    for (int b = 0; b < T.nblocks; ++b)
      for (LO e : T.block_elems[b]) {
        for (int k = 0; k < 12; ++k) {
          GO g0 = T.entity_gid(e, 0, kHexEdge[k][0]);
          GO g1 = T.entity_gid(e, 0, kHexEdge[k][1]);
          D.edge_sign[e].push_back(g0 < g1 ? 1 : -1);
        }
      }
  // graph: union of element cliques, columns ascending LID
  const GO N = (GO)D.owned.size();
  std::vector<std::vector<LO>> rows(N);
  for (int b = 0; b < T.nblocks; ++b)
    for (LO e : T.block_elems[b]) {
      const auto& l = D.elementLIDs[e];
      for (LO r : l) rows[r].insert(rows[r].end(), l.begin(), l.end());
    }
  D.rowptr.assign(N + 1, 0);
#pragma omp parallel for schedule(dynamic, 4096)
  for (GO r = 0; r < N; ++r) {
    auto& v = rows[r];
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  for (GO r = 0; r < N; ++r) D.rowptr[r + 1] = D.rowptr[r] + (int64_t)rows[r].size();
  D.colind.assign((size_t)D.rowptr[N], 0);
#pragma omp parallel for schedule(dynamic, 4096)
  for (GO r = 0; r < N; ++r) {
    std::copy(rows[r].begin(), rows[r].end(), D.colind.begin() + D.rowptr[r]);
    std::vector<LO>().swap(rows[r]);
  }
}

// ------------------------------------------------------------ Fad type
// Forward-mode dual number with a fixed derivative length (Sacado SFad
// semantics; DFad in the reference has the element GID count as length).
template <int NDER>
struct Fad {
  double v;
  double d[NDER];
  Fad() : v(0.0) { for (int i = 0; i < NDER; ++i) d[i] = 0.0; }
  explicit Fad(double a) : v(a) { for (int i = 0; i < NDER; ++i) d[i] = 0.0; }
};
template <int N> static inline Fad<N> operator+(const Fad<N>& a, const Fad<N>& b) {
  Fad<N> r; r.v = a.v + b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r;
}
template <int N> static inline Fad<N> operator-(const Fad<N>& a, const Fad<N>& b) {
  Fad<N> r; r.v = a.v - b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r;
}
template <int N> static inline Fad<N> operator*(const Fad<N>& a, const Fad<N>& b) {
  Fad<N> r; r.v = a.v * b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r;
}
template <int N> static inline Fad<N> operator*(double s, const Fad<N>& a) {
  Fad<N> r; r.v = s * a.v; for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i]; return r;
}
template <int N> static inline Fad<N> operator*(const Fad<N>& a, double s) { return s * a; }
template <int N> static inline Fad<N> operator+(const Fad<N>& a, double s) { Fad<N> r = a; r.v += s; return r; }
template <int N> static inline void operator+=(Fad<N>& a, const Fad<N>& b) {
  a.v += b.v; for (int i = 0; i < N; ++i) a.d[i] += b.d[i];
}

// ------------------------------------------------------------ problem
struct Problem {
  Topology T;
  DofManager D;
  tx_equation_set_desc eq;
  std::vector<Cubature> cub;                 // per block
  std::string err;
};

// Element geometry at the cubature points of a block
struct ElemGeom {
  int np = 0;
  std::vector<double> J, Jinv, det, wdet, ip;  // [q][3][3], [q], [q][3]
};

static void geom_basis(int topo, BasisDef& G) { G = make_basis(topo, TX_HGRAD_C1); }

static void compute_geometry(int topo, const double* X, const Cubature& C, ElemGeom& g) {
  BasisDef G;
  geom_basis(topo, G);
  int nv = G.nb;
  g.np = C.np;
  g.J.assign(C.np * 9, 0.0); g.Jinv.assign(C.np * 9, 0.0);
  g.det.assign(C.np, 0.0); g.wdet.assign(C.np, 0.0); g.ip.assign(C.np * 3, 0.0);
  std::vector<double> N(nv);
  std::vector<double> dN(nv * 3);
  for (int q = 0; q < C.np; ++q) {
    eval_hgrad(G, &C.xi[3 * q], N.data(), (double(*)[3])dN.data());
    double* J = &g.J[9 * q];
    for (int n = 0; n < nv; ++n)
      for (int i = 0; i < 3; ++i) {
        g.ip[3 * q + i] += X[3 * n + i] * N[n];
        for (int j = 0; j < 3; ++j) J[3 * i + j] += X[3 * n + i] * dN[3 * n + j];
      }
    double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                 J[2] * (J[3] * J[7] - J[4] * J[6]);
    g.det[q] = det;
    double* Ji = &g.Jinv[9 * q];
    Ji[0] = (J[4] * J[8] - J[5] * J[7]) / det;
    Ji[1] = (J[2] * J[7] - J[1] * J[8]) / det;
    Ji[2] = (J[1] * J[5] - J[2] * J[4]) / det;
    Ji[3] = (J[5] * J[6] - J[3] * J[8]) / det;
    Ji[4] = (J[0] * J[8] - J[2] * J[6]) / det;
    Ji[5] = (J[2] * J[3] - J[0] * J[5]) / det;
    Ji[6] = (J[3] * J[7] - J[4] * J[6]) / det;
    Ji[7] = (J[1] * J[6] - J[0] * J[7]) / det;
    Ji[8] = (J[0] * J[4] - J[1] * J[3]) / det;
  }
  // computeCellMeasure: w*det, sign flipped per cell by the first point's det
  double s = g.det[0] < 0.0 ? -1.0 : 1.0;
  for (int q = 0; q < C.np; ++q) g.wdet[q] = s * g.det[q] * C.w[q];
}

static inline double source_value(int kind, double c, double s0, const double* x) {
  if (kind == TX_SOURCE_SINE) {
    const double pi = 3.14159265358979323846;
    return 3.0 * pi * pi * std::sin(pi * x[0]) * std::sin(pi * x[1]) * std::sin(pi * x[2]);
  }
  if (kind == TX_SOURCE_AFFINE) return c * (1.0 + x[0] + 2.0 * x[1] + 3.0 * x[2]);
  return s0;
}

struct EvalIn {
  const double* x; const double* xdot; const double* aux;
  double alpha, beta, t;
  double* f; double* vals;
};

static inline void atomic_add(double* p, double v) {
#ifdef _OPENMP
#pragma omp atomic
#endif
  *p += v;
}

// sumIntoValues: binary search of each column in the (sorted) row
static inline void sum_into(const DofManager& D, double* vals, LO row, LO col, double v) {
  const LO* b = D.colind.data() + D.rowptr[row];
  const LO* e = D.colind.data() + D.rowptr[row + 1];
  const LO* p = std::lower_bound(b, e, col);
  if (p == e || *p != col) throw std::runtime_error("sumIntoValues: column not in graph");
  atomic_add(vals + (p - D.colind.data()), v);
}

template <int NDER>
static void eval_element(const Problem& P, int blk, LO e, const EvalIn& in) {
  typedef Fad<NDER> F;
  const Topology& T = P.T;
  const DofManager& D = P.D;
  const BasisDef& B = D.block_basis[blk];
  const Cubature& C = P.cub[blk];
  const int topo = T.block_topo[blk];
  const int nf = D.nfields;
  const int nb = B.nb;
  const auto& lids = D.elementLIDs[e];
  const int ndof = (int)lids.size();
  if (ndof > NDER) throw std::runtime_error("derivative dimension too small");
  const bool jac = in.vals != nullptr;
  // ---- gather (GatherSolution_Tpetra<Jacobian>): seed dx(offset) = beta / alpha
  std::vector<F> u(nf * nb), ud(nf * nb);
  for (int f = 0; f < nf; ++f)
    for (int b = 0; b < nb; ++b) {
      int off = D.offsets[blk][f][b];
      F a(in.x[lids[off]]);
      if (jac && in.beta != 0.0) a.d[off] = in.beta;
      u[f * nb + b] = a;
      F c(in.xdot ? in.xdot[lids[off]] : 0.0);
      if (jac && in.alpha != 0.0) c.d[off] = in.alpha;
      ud[f * nb + b] = c;
    }
  // ---- IntegrationValues2
  int nv = topo == TX_TOPO_HEX ? 8 : 4;
  double X[24];
  T.elem_vertices(e, nv, X);
  ElemGeom g;
  compute_geometry(topo, X, C, g);
  const int np = C.np;
  // ---- BasisValues2 (physical): weighted values and gradients
  std::vector<double> N(nb), dNr(nb * 3);
  std::vector<double> bv(np * nb), gb(np * nb * 3), wbv(np * nb), wgb(np * nb * 3);
  std::vector<double> hv(np * nb * 3), hc(np * nb * 3), whv(np * nb * 3), whc(np * nb * 3);
  for (int q = 0; q < np; ++q) {
    const double* Ji = &g.Jinv[9 * q];
    const double* J = &g.J[9 * q];
    if (!B.hcurl) {
      eval_hgrad(B, &C.xi[3 * q], N.data(), (double(*)[3])dNr.data());
      for (int b = 0; b < nb; ++b) {
        bv[q * nb + b] = N[b];
        wbv[q * nb + b] = N[b] * g.wdet[q];
        for (int i = 0; i < 3; ++i) {
          // HGRADtransformGRAD: grad_i = sum_j Jinv(j,i) refgrad_j
          double s = 0.0;
          for (int j = 0; j < 3; ++j) s += Ji[3 * j + i] * dNr[3 * b + j];
          gb[(q * nb + b) * 3 + i] = s;
          wgb[(q * nb + b) * 3 + i] = s * g.wdet[q];
        }
      }
    } else {
      double V[12][3], Cu[12][3];
      eval_hcurl_hex(&C.xi[3 * q], V, Cu);
      for (int b = 0; b < nb; ++b) {
        double sgn = D.edge_sign[e][b];
        for (int i = 0; i < 3; ++i) {
          // HCURLtransformVALUE: Jinv^T v;  HCURLtransformCURL: J c / det
          double sv = 0.0, sc = 0.0;
          for (int j = 0; j < 3; ++j) {
            sv += Ji[3 * j + i] * V[b][j];
            sc += J[3 * i + j] * Cu[b][j];
          }
          sv *= sgn;
          sc = sgn * sc / g.det[q];
          hv[(q * nb + b) * 3 + i] = sv;
          hc[(q * nb + b) * 3 + i] = sc;
          whv[(q * nb + b) * 3 + i] = sv * g.wdet[q];
          whc[(q * nb + b) * 3 + i] = sc * g.wdet[q];
        }
      }
    }
  }
  // ---- physics: residual fields r[f][b]
  std::vector<F> r(nf * nb);
  const double* pr = P.eq.params;
  if (P.eq.physics == TX_PHYS_POISSON || P.eq.physics == TX_PHYS_HEAT) {
    for (int q = 0; q < np; ++q) {
      // DOF / DOFGradient
      F uq, udq, gq[3];
      for (int b = 0; b < nb; ++b) {
        uq += bv[q * nb + b] * u[b];
        udq += bv[q * nb + b] * ud[b];
        for (int i = 0; i < 3; ++i) gq[i] += gb[(q * nb + b) * 3 + i] * u[b];
      }
      if (P.eq.physics == TX_PHYS_POISSON) {
        double k = pr[0], c = pr[1], m = pr[2];
        double s = source_value(P.eq.source_kind, c, pr[3], &g.ip[3 * q]);
        for (int b = 0; b < nb; ++b) {
          F& rb = r[b];
          for (int i = 0; i < 3; ++i) rb += wgb[(q * nb + b) * 3 + i] * k * gq[i];  // GradBasisDotVector
          if (c != 0.0) rb += wbv[q * nb + b] * c * uq;                            // BasisTimesScalar(u)
          if (m != 0.0) rb += wbv[q * nb + b] * m * udq;                           // BasisTimesScalar(DXDT)
          rb.v += wbv[q * nb + b] * (-1.0) * s;                                    // BasisTimesScalar(-1 src)
        }
      } else {
        double k0 = pr[0], k2 = pr[1], qs = pr[2];
        F kq = k2 * (uq * uq) + k0;  // field multiplier k(T)
        for (int b = 0; b < nb; ++b) {
          F& rb = r[b];
          for (int i = 0; i < 3; ++i) rb += (wgb[(q * nb + b) * 3 + i] * 1.0) * (gq[i] * kq);
          rb.v += wbv[q * nb + b] * (-1.0) * qs;
        }
      }
    }
  } else if (P.eq.physics == TX_PHYS_ELASTICITY) {
    const double E = pr[0], nu = pr[1];
    const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = E / (2.0 * (1.0 + nu));
    const double rho = pr[5];
    for (int q = 0; q < np; ++q) {
      F G[3][3], acc[3];
      for (int c = 0; c < 3; ++c)
        for (int b = 0; b < nb; ++b) {
          for (int i = 0; i < 3; ++i) G[c][i] += gb[(q * nb + b) * 3 + i] * u[c * nb + b];
          if (rho != 0.0) acc[c] += bv[q * nb + b] * ud[c * nb + b];
        }
      F tr = G[0][0] + G[1][1] + G[2][2];
      F S[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          S[i][j] = mu * (G[i][j] + G[j][i]);
          if (i == j) S[i][j] += lam * tr;
        }
      for (int c = 0; c < 3; ++c)
        for (int b = 0; b < nb; ++b) {
          F& rb = r[c * nb + b];
          for (int i = 0; i < 3; ++i) rb += wgb[(q * nb + b) * 3 + i] * S[c][i];
          if (rho != 0.0) rb += wbv[q * nb + b] * rho * acc[c];
          rb.v += wbv[q * nb + b] * (-1.0) * pr[2 + c];
        }
    }
  } else if (P.eq.physics == TX_PHYS_MAXWELL) {
    const double inv_mu = pr[0], sigma = pr[1];
    for (int q = 0; q < np; ++q) {
      F Eq[3], Cq[3];
      double Jq[3] = {0, 0, 0};
      for (int b = 0; b < nb; ++b) {
        double jb = in.aux ? in.aux[lids[D.offsets[blk][0][b]]] : 0.0;
        for (int i = 0; i < 3; ++i) {
          Eq[i] += hv[(q * nb + b) * 3 + i] * u[b];
          Cq[i] += hc[(q * nb + b) * 3 + i] * u[b];
          Jq[i] += hv[(q * nb + b) * 3 + i] * jb;
        }
      }
      for (int b = 0; b < nb; ++b) {
        F& rb = r[b];
        for (int i = 0; i < 3; ++i) {
          rb += whc[(q * nb + b) * 3 + i] * inv_mu * Cq[i];
          rb += whv[(q * nb + b) * 3 + i] * sigma * Eq[i];
          rb.v += whv[(q * nb + b) * 3 + i] * (-1.0) * Jq[i];
        }
      }
    }
  }
  // ---- scatter (ScatterResidual_Tpetra<Jacobian>)
  for (int f = 0; f < nf; ++f)
    for (int b = 0; b < nb; ++b) {
      const F& rb = r[f * nb + b];
      LO row = lids[D.offsets[blk][f][b]];
      if (in.f) atomic_add(in.f + row, rb.v);
      if (jac)
        for (int k = 0; k < ndof; ++k) sum_into(D, in.vals, row, lids[k], rb.d[k]);
    }
}

static void eval_range(const Problem& P, int blk, int64_t e0, int64_t e1, const EvalIn& in, int nthreads) {
  const auto& elems = P.T.block_elems[blk];
  int nd = P.D.elementLIDs.empty() ? 0 : (int)P.D.elementLIDs[elems.empty() ? 0 : elems[0]].size();
  if (e1 < 0 || e1 > (int64_t)elems.size()) e1 = (int64_t)elems.size();
  auto body = [&](int64_t i) {
    LO e = elems[i];
    if (nd <= 4) eval_element<4>(P, blk, e, in);
    else if (nd <= 8) eval_element<8>(P, blk, e, in);
    else if (nd <= 12) eval_element<12>(P, blk, e, in);
    else if (nd <= 24) eval_element<24>(P, blk, e, in);
    else if (nd <= 27) eval_element<27>(P, blk, e, in);
    else throw std::runtime_error("element GID count > 27 not provided");
  };
#ifdef _OPENMP
  if (nthreads > 1) {
    std::string err;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 32)
    for (int64_t i = e0; i < e1; ++i) {
      try { body(i); } catch (std::exception& ex) {
#pragma omp critical
        err = ex.what();
      }
    }
    if (!err.empty()) throw std::runtime_error(err);
    return;
  }
#endif
  (void)nthreads;
  for (int64_t i = e0; i < e1; ++i) body(i);
}

// side test for an entity given its brick vertices
static bool on_sides(const Topology& T, GO I, GO J, GO K, const int* bv, int n, uint32_t mask) {
  for (int s = 0; s < 6; ++s) {
    if (!(mask & (1u << s))) continue;
    bool all = true;
    for (int k = 0; k < n; ++k) {
      GO i, j, kk;
      T.vertex_lattice(I, J, K, bv[k], i, j, kk);
      GO c = s < 2 ? i : (s < 4 ? j : kk);
      GO lim = s == 0 || s == 2 || s == 4 ? 0 : (s == 1 ? T.NX : (s == 3 ? T.NY : T.NZ));
      if (c != lim) { all = false; break; }
    }
    if (all) return true;
  }
  return false;
}

static std::vector<LO> dirichlet_dofs(const Problem& P, uint32_t side_mask, uint32_t field_mask) {
  const Topology& T = P.T;
  const DofManager& D = P.D;
  // brick-edge vertex pairs for ids 0..18
  int edgev[19][2];
  for (int k = 0; k < 12; ++k) { edgev[k][0] = kHexEdge[k][0]; edgev[k][1] = kHexEdge[k][1]; }
  for (int t = 0; t < 6; ++t)
    for (int k = 0; k < 6; ++k) {
      int id = kTetEdgeInHex[t][k];
      edgev[id][0] = kTetInHex[t][kTetEdge[k][0]];
      edgev[id][1] = kTetInHex[t][kTetEdge[k][1]];
    }
  std::set<LO> ids;
  for (int blk = 0; blk < T.nblocks; ++blk) {
    const BasisDef& B = D.block_basis[blk];
    int topo = T.block_topo[blk];
    for (LO e : T.block_elems[blk]) {
      GO I, J, K;
      T.brick_ijk(T.elem_brick[e], I, J, K);
      int sub = T.elem_sub[e];
      for (int dim = 0; dim < 3; ++dim)
        for (int c = 0; c < B.nsub[dim]; ++c) {
          int bidx = B.sub[dim][c];
          if (bidx < 0) continue;
          int bv[4], n = 0;
          if (dim == 0) { bv[0] = topo == TX_TOPO_HEX ? c : kTetInHex[sub][c]; n = 1; }
          else if (dim == 1) {
            int id = topo == TX_TOPO_HEX ? c : kTetEdgeInHex[sub][c];
            bv[0] = edgev[id][0]; bv[1] = edgev[id][1]; n = 2;
          } else {
            if (topo != TX_TOPO_HEX) continue;
            for (int k = 0; k < 4; ++k) bv[k] = kHexFace[c][k];
            n = 4;
          }
          if (!on_sides(T, I, J, K, bv, n, side_mask)) continue;
          for (int f = 0; f < D.nfields; ++f)
            if (field_mask & (1u << f)) ids.insert(D.elementLIDs[e][D.offsets[blk][f][bidx]]);
        }
    }
  }
  return std::vector<LO>(ids.begin(), ids.end());
}

// ------------------------------------------------------------- Neumann
// shards Tetrahedron<4> sides with their node order
static const int kTetSideNodes[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};

// Reference side rule mapped into the cell (CellTools::mapToReferenceSubcell)
// and the side's two reference tangents.  Quad sides: Gauss n x n on
// [-1,1]^2, x(u,v) = centre + u t_u + v t_v (the hex faces are
// parallelograms in reference space, so this is their bilinear map).
// Triangle sides: the 3-point degree-2 rule on the unit triangle,
// x(u,v) = V0 + u (V1 - V0) + v (V2 - V0).
static void side_rule(int topo, int degree, int s, std::vector<double>& xi, std::vector<double>& w,
                      double tu[3], double tv[3]) {
  xi.clear(); w.clear();
  if (topo == TX_TOPO_HEX) {
    const int* F = kHexFace[s];
    std::vector<double> p, pw;
    gauss_1d(degree / 2 + 1, p, pw);
    const int n = (int)p.size();
    double ctr[3];
    for (int d = 0; d < 3; ++d) {
      tu[d] = (kHexVert[F[1]][d] - kHexVert[F[0]][d]) / 2.0;
      tv[d] = (kHexVert[F[3]][d] - kHexVert[F[0]][d]) / 2.0;
      ctr[d] = (kHexVert[F[0]][d] + kHexVert[F[1]][d] + kHexVert[F[2]][d] + kHexVert[F[3]][d]) / 4.0;
    }
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        for (int d = 0; d < 3; ++d) xi.push_back(ctr[d] + p[i] * tu[d] + p[j] * tv[d]);
        w.push_back(pw[i] * pw[j]);
      }
  } else {
    static const double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const int* F = kTetSideNodes[s];
    for (int d = 0; d < 3; ++d) { tu[d] = V[F[1]][d] - V[F[0]][d]; tv[d] = V[F[2]][d] - V[F[0]][d]; }
    if (degree > 2) throw std::runtime_error("triangle side rule: degree <= 2");
    const double uv[3][2] = {{1.0 / 6, 1.0 / 6}, {2.0 / 3, 1.0 / 6}, {1.0 / 6, 2.0 / 3}};
    for (int q = 0; q < 3; ++q) {
      for (int d = 0; d < 3; ++d) xi.push_back(V[F[0]][d] + uv[q][0] * tu[d] + uv[q][1] * tv[d]);
      w.push_back(1.0 / 6);
    }
  }
}

// f[LID(cell, field, b)] += val * sum_q N_b(xi_q) * w_q * |(J t_u) x (J t_v)|
// over the cells of `blk` with a side on the box sides of side_mask.
static int64_t neumann_flux(const Problem& P, int blk, uint32_t side_mask, int field, double val, double* f) {
  const Topology& T = P.T;
  const DofManager& D = P.D;
  const BasisDef& B = D.block_basis[blk];
  if (B.hcurl) throw std::runtime_error("Neumann flux: scalar basis only");
  const int topo = T.block_topo[blk];
  const int nsides = topo == TX_TOPO_HEX ? 6 : 4;
  const int nvs = topo == TX_TOPO_HEX ? 4 : 3;
  BasisDef G;
  geom_basis(topo, G);
  const int nv = G.nb;
  int64_t count = 0;
  std::vector<double> xi, w, X(3 * nv), N(B.nb), dN(3 * B.nb), Ng(nv), dNg(3 * nv);
  for (LO e : T.block_elems[blk]) {
    GO I, J, K;
    T.brick_ijk(T.elem_brick[e], I, J, K);
    const int sub = T.elem_sub[e];
    for (int s = 0; s < nsides; ++s) {
      int bv[4];
      for (int k = 0; k < nvs; ++k)
        bv[k] = topo == TX_TOPO_HEX ? kHexFace[s][k] : kTetInHex[sub][kTetSideNodes[s][k]];
      if (!on_sides(T, I, J, K, bv, nvs, side_mask)) continue;
      ++count;
      double tu[3], tv[3];
      side_rule(topo, D.block_degree[blk], s, xi, w, tu, tv);
      T.elem_vertices(e, nv, X.data());
      std::vector<double> R(B.nb, 0.0);
      for (size_t q = 0; q < w.size(); ++q) {
        eval_hgrad(G, &xi[3 * q], Ng.data(), (double(*)[3])dNg.data());
        double Jm[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int n = 0; n < nv; ++n)
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Jm[3 * i + j] += X[3 * n + i] * dNg[3 * n + j];
        double a[3], b[3];
        for (int i = 0; i < 3; ++i) {
          a[i] = Jm[3 * i] * tu[0] + Jm[3 * i + 1] * tu[1] + Jm[3 * i + 2] * tu[2];
          b[i] = Jm[3 * i] * tv[0] + Jm[3 * i + 1] * tv[1] + Jm[3 * i + 2] * tv[2];
        }
        const double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
        const double wm = w[q] * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        eval_hgrad(B, &xi[3 * q], N.data(), (double(*)[3])dN.data());
        for (int bb = 0; bb < B.nb; ++bb) R[bb] += val * (N[bb] * wm);
      }
      for (int bb = 0; bb < B.nb; ++bb) f[D.elementLIDs[e][D.offsets[blk][field][bb]]] += R[bb];
    }
  }
  return count;
}

// ------------------------------------------------------------ responses
// value += sum over the cells of block blk (all blocks: blk < 0) of
// sum_q integrand(q) * wdet(q); dgdx (optional) += d value / d x.
static void response_integral(const Problem& P, int blk_sel, int field, int integrand, int degree, const double* x,
                              double* value, double* dgdx) {
  const Topology& T = P.T;
  const DofManager& D = P.D;
  const double pi = 3.14159265358979323846;
  double total = 0.0;
  for (int blk = 0; blk < T.nblocks; ++blk) {
    if (blk_sel >= 0 && blk != blk_sel) continue;
    const BasisDef& B = D.block_basis[blk];
    if (B.hcurl) throw std::runtime_error("response: scalar basis only");
    const int topo = T.block_topo[blk];
    const Cubature C = make_cubature(topo, degree > 0 ? degree : D.block_degree[blk]);
    const int nv = topo == TX_TOPO_HEX ? 8 : 4;
    std::vector<double> X(3 * nv), N(B.nb), dN(3 * B.nb);
    ElemGeom g;
    for (LO e : T.block_elems[blk]) {
      T.elem_vertices(e, nv, X.data());
      compute_geometry(topo, X.data(), C, g);
      std::vector<double> ub(B.nb), grad_e(B.nb, 0.0);
      std::vector<LO> lid(B.nb);
      for (int b = 0; b < B.nb; ++b) {
        lid[b] = D.elementLIDs[e][D.offsets[blk][field][b]];
        ub[b] = x[lid[b]];
      }
      double cell = 0.0;
      for (int q = 0; q < C.np; ++q) {
        eval_hgrad(B, &C.xi[3 * q], N.data(), (double(*)[3])dN.data());
        const double* Ji = &g.Jinv[9 * q];
        double u = 0.0, gr[3] = {0, 0, 0};
        for (int b = 0; b < B.nb; ++b) {
          u += N[b] * ub[b];
          for (int c = 0; c < 3; ++c) gr[c] += dN[3 * b + c] * ub[b];
        }
        double gu[3];
        for (int i = 0; i < 3; ++i) gu[i] = Ji[i] * gr[0] + Ji[3 + i] * gr[1] + Ji[6 + i] * gr[2];
        const double* xq = &g.ip[3 * q];
        double ev = u, de[3] = {0, 0, 0};
        if (integrand != TX_INTEGRAND_FIELD) {
          const double sx = std::sin(pi * xq[0]), sy = std::sin(pi * xq[1]), sz = std::sin(pi * xq[2]);
          ev = u - sx * sy * sz;
          if (integrand == TX_INTEGRAND_H1_ERROR) {
            de[0] = gu[0] - pi * std::cos(pi * xq[0]) * sy * sz;
            de[1] = gu[1] - pi * sx * std::cos(pi * xq[1]) * sz;
            de[2] = gu[2] - pi * sx * sy * std::cos(pi * xq[2]);
          }
        }
        double integ = integrand == TX_INTEGRAND_FIELD ? ev : ev * ev;
        if (integrand == TX_INTEGRAND_H1_ERROR) integ += de[0] * de[0] + de[1] * de[1] + de[2] * de[2];
        const double wm = g.wdet[q];
        cell += integ * wm;
        if (dgdx) {
          for (int b = 0; b < B.nb; ++b) {
            double t = integrand == TX_INTEGRAND_FIELD ? N[b] : 2.0 * ev * N[b];
            if (integrand == TX_INTEGRAND_H1_ERROR)
              for (int i = 0; i < 3; ++i)
                t += 2.0 * de[i] * (Ji[i] * dN[3 * b] + Ji[3 + i] * dN[3 * b + 1] + Ji[6 + i] * dN[3 * b + 2]);
            grad_e[b] += t * wm;
          }
        }
      }
      total += cell;
      if (dgdx)
        for (int b = 0; b < B.nb; ++b) dgdx[lid[b]] += grad_e[b];
    }
  }
  *value = total;
}

// ExtremeValue (disc-fe/src/responses/Panzer_ResponseScatterEvaluator_ExtremeValue_impl.hpp:136-146 over
// CellExtreme's per-cell extreme of the field at the cubature points): the max (use_max) or min of u(q) over
// the cells of the selected blocks (block order, cell order, point order); the first point reaching the
// extreme wins.  dgdx += d value / d x = N_b(q*) at the winning cell's field DOFs.
static void response_extreme(const Problem& P, int blk_sel, int field, bool use_max, int degree, const double* x,
                             double* value, double* dgdx) {
  const Topology& T = P.T;
  const DofManager& D = P.D;
  bool have = false;
  double best = 0.0;
  int best_blk = -1, best_q = -1;
  LO best_e = -1;
  for (int blk = 0; blk < T.nblocks; ++blk) {
    if (blk_sel >= 0 && blk != blk_sel) continue;
    const BasisDef& B = D.block_basis[blk];
    if (B.hcurl) throw std::runtime_error("response: scalar basis only");
    const Cubature C = make_cubature(T.block_topo[blk], degree > 0 ? degree : D.block_degree[blk]);
    std::vector<double> N(B.nb), dN(3 * B.nb);
    for (LO e : T.block_elems[blk])
      for (int q = 0; q < C.np; ++q) {
        eval_hgrad(B, &C.xi[3 * q], N.data(), (double(*)[3])dN.data());
        double u = 0.0;
        for (int b = 0; b < B.nb; ++b) u += N[b] * x[D.elementLIDs[e][D.offsets[blk][field][b]]];
        if (!have || (use_max ? u > best : u < best)) {
          have = true; best = u; best_blk = blk; best_e = e; best_q = q;
        }
      }
  }
  *value = best;
  if (dgdx && have) {
    const BasisDef& B = D.block_basis[best_blk];
    const Cubature C = make_cubature(T.block_topo[best_blk], degree > 0 ? degree : D.block_degree[best_blk]);
    std::vector<double> N(B.nb), dN(3 * B.nb);
    eval_hgrad(B, &C.xi[3 * best_q], N.data(), (double(*)[3])dN.data());
    for (int b = 0; b < B.nb; ++b) dgdx[D.elementLIDs[best_e][D.offsets[best_blk][field][b]]] += N[b];
  }
}

// Integral of the field over the sides of the selected blocks on the box sides of side_mask: sum over
// (cell, side) of sum_q w_q |J t_u x J t_v| u(xi_q) (the side rule of neumann_flux); dgdx += N_b w |.|.
static void response_side(const Problem& P, int blk_sel, uint32_t side_mask, int field, const double* x,
                          double* value, double* dgdx) {
  const Topology& T = P.T;
  const DofManager& D = P.D;
  double total = 0.0;
  for (int blk = 0; blk < T.nblocks; ++blk) {
    if (blk_sel >= 0 && blk != blk_sel) continue;
    const BasisDef& B = D.block_basis[blk];
    if (B.hcurl) throw std::runtime_error("response: scalar basis only");
    const int topo = T.block_topo[blk];
    const int nsides = topo == TX_TOPO_HEX ? 6 : 4, nvs = topo == TX_TOPO_HEX ? 4 : 3;
    BasisDef G;
    geom_basis(topo, G);
    const int nv = G.nb;
    std::vector<double> xi, w, X(3 * nv), N(B.nb), dN(3 * B.nb), Ng(nv), dNg(3 * nv);
    for (LO e : T.block_elems[blk]) {
      GO I, J, K;
      T.brick_ijk(T.elem_brick[e], I, J, K);
      const int sub = T.elem_sub[e];
      for (int s = 0; s < nsides; ++s) {
        int bv[4];
        for (int k = 0; k < nvs; ++k)
          bv[k] = topo == TX_TOPO_HEX ? kHexFace[s][k] : kTetInHex[sub][kTetSideNodes[s][k]];
        if (!on_sides(T, I, J, K, bv, nvs, side_mask)) continue;
        double tu[3], tv[3];
        side_rule(topo, D.block_degree[blk], s, xi, w, tu, tv);
        T.elem_vertices(e, nv, X.data());
        for (size_t q = 0; q < w.size(); ++q) {
          eval_hgrad(G, &xi[3 * q], Ng.data(), (double(*)[3])dNg.data());
          double Jm[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
          for (int n = 0; n < nv; ++n)
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j) Jm[3 * i + j] += X[3 * n + i] * dNg[3 * n + j];
          double a[3], bb[3];
          for (int i = 0; i < 3; ++i) {
            a[i] = Jm[3 * i] * tu[0] + Jm[3 * i + 1] * tu[1] + Jm[3 * i + 2] * tu[2];
            bb[i] = Jm[3 * i] * tv[0] + Jm[3 * i + 1] * tv[1] + Jm[3 * i + 2] * tv[2];
          }
          const double c[3] = {a[1] * bb[2] - a[2] * bb[1], a[2] * bb[0] - a[0] * bb[2], a[0] * bb[1] - a[1] * bb[0]};
          const double wm = w[q] * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
          eval_hgrad(B, &xi[3 * q], N.data(), (double(*)[3])dN.data());
          double u = 0.0;
          for (int b = 0; b < B.nb; ++b) u += N[b] * x[D.elementLIDs[e][D.offsets[blk][field][b]]];
          total += u * wm;
          if (dgdx)
            for (int b = 0; b < B.nb; ++b) dgdx[D.elementLIDs[e][D.offsets[blk][field][b]]] += N[b] * wm;
        }
      }
    }
  }
  *value = total;
}

// Probe (disc-fe/src/responses/Panzer_ResponseScatterEvaluator_Probe_impl.hpp: the cell holding the point,
// its reference coordinates by CellTools::mapToReferenceFrame, the basis there): the first cell (block
// order, cell order) whose inverse geometry map puts the point inside the reference cell (tolerance 1e-10);
// value = sum_b N_b(xi) u_b, dgdx += N_b(xi).  Returns the mesh element, or -1 when no cell holds it.
static LO response_probe(const Problem& P, const double pt[3], int field, const double* x, double* value,
                         double* dgdx) {
  const Topology& T = P.T;
  const DofManager& D = P.D;
  for (int blk = 0; blk < T.nblocks; ++blk) {
    const BasisDef& B = D.block_basis[blk];
    const int topo = T.block_topo[blk];
    BasisDef G;
    geom_basis(topo, G);
    const int nv = G.nb;
    std::vector<double> X(3 * nv), Ng(nv), dNg(3 * nv), N(B.nb), dN(3 * B.nb);
    for (LO e : T.block_elems[blk]) {
      T.elem_vertices(e, nv, X.data());
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      for (int n = 0; n < nv; ++n)
        for (int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], X[3 * n + d]); hi[d] = std::max(hi[d], X[3 * n + d]); }
      bool box = true;
      for (int d = 0; d < 3; ++d) box = box && pt[d] >= lo[d] - 1e-12 && pt[d] <= hi[d] + 1e-12;
      if (!box) continue;
      double xi[3] = {0.0, 0.0, 0.0};
      if (topo == TX_TOPO_TET) xi[0] = xi[1] = xi[2] = 0.25;
      for (int it = 0; it < 50; ++it) {  // Newton on x(xi) = pt
        eval_hgrad(G, xi, Ng.data(), (double(*)[3])dNg.data());
        double r[3] = {-pt[0], -pt[1], -pt[2]}, Jm[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int n = 0; n < nv; ++n)
          for (int i = 0; i < 3; ++i) {
            r[i] += Ng[n] * X[3 * n + i];
            for (int j = 0; j < 3; ++j) Jm[3 * i + j] += X[3 * n + i] * dNg[3 * n + j];
          }
        const double c00 = Jm[4] * Jm[8] - Jm[5] * Jm[7], c01 = Jm[5] * Jm[6] - Jm[3] * Jm[8];
        const double c02 = Jm[3] * Jm[7] - Jm[4] * Jm[6];
        const double det = Jm[0] * c00 + Jm[1] * c01 + Jm[2] * c02;
        const double Ji[9] = {c00 / det, (Jm[2] * Jm[7] - Jm[1] * Jm[8]) / det, (Jm[1] * Jm[5] - Jm[2] * Jm[4]) / det,
                              c01 / det, (Jm[0] * Jm[8] - Jm[2] * Jm[6]) / det, (Jm[2] * Jm[3] - Jm[0] * Jm[5]) / det,
                              c02 / det, (Jm[1] * Jm[6] - Jm[0] * Jm[7]) / det, (Jm[0] * Jm[4] - Jm[1] * Jm[3]) / det};
        double step = 0.0;
        for (int i = 0; i < 3; ++i) {
          const double d = Ji[3 * i] * r[0] + Ji[3 * i + 1] * r[1] + Ji[3 * i + 2] * r[2];
          xi[i] -= d;
          step = std::max(step, std::fabs(d));
        }
        if (step < 1e-15) break;
      }
      const double tol = 1e-10;
      bool inside;
      if (topo == TX_TOPO_HEX)
        inside = std::fabs(xi[0]) <= 1 + tol && std::fabs(xi[1]) <= 1 + tol && std::fabs(xi[2]) <= 1 + tol;
      else
        inside = xi[0] >= -tol && xi[1] >= -tol && xi[2] >= -tol && xi[0] + xi[1] + xi[2] <= 1 + tol;
      if (!inside) continue;
      eval_hgrad(B, xi, N.data(), (double(*)[3])dN.data());
      double u = 0.0;
      for (int b = 0; b < B.nb; ++b) {
        const LO lid = D.elementLIDs[e][D.offsets[blk][field][b]];
        u += N[b] * x[lid];
        if (dgdx) dgdx[lid] += N[b];
      }
      *value = u;
      return e;
    }
  }
  return -1;
}

}  // namespace orc

// ====================================================================== C API
using namespace orc;

extern "C" {

void* orc_create(const tx_mesh_desc* m, const tx_equation_set_desc* q, char* errbuf, int errlen) {
  Problem* P = new Problem;
  try {
    build_topology(P->T, *m);
    P->eq = *q;
    build_dofs(P->T, P->D, *q);
    for (int b = 0; b < P->T.nblocks; ++b) P->cub.push_back(make_cubature(P->T.block_topo[b], P->D.block_degree[b]));
  } catch (std::exception& ex) {
    if (errbuf && errlen > 0) { strncpy(errbuf, ex.what(), errlen - 1); errbuf[errlen - 1] = 0; }
    delete P;
    return nullptr;
  }
  return P;
}
void orc_destroy(void* h) { delete (Problem*)h; }

int64_t orc_n_dofs(void* h) { return (int64_t)((Problem*)h)->D.owned.size(); }
int64_t orc_nnz(void* h) { return (int64_t)((Problem*)h)->D.colind.size(); }
int orc_n_blocks(void* h) { return ((Problem*)h)->T.nblocks; }
int orc_n_fields(void* h) { return ((Problem*)h)->D.nfields; }
int64_t orc_n_elements(void* h) { return (int64_t)((Problem*)h)->T.elem_brick.size(); }
int64_t orc_block_n_elems(void* h, int b) { return (int64_t)((Problem*)h)->T.block_elems[b].size(); }
int orc_block_gid_count(void* h, int b) {
  Problem* P = (Problem*)h;
  if (P->T.block_elems[b].empty()) return 0;
  return (int)P->D.elementGIDs[P->T.block_elems[b][0]].size();
}
void orc_block_elements(void* h, int b, int64_t* out) {
  Problem* P = (Problem*)h;
  for (size_t i = 0; i < P->T.block_elems[b].size(); ++i) out[i] = P->T.block_elems[b][i];
}
void orc_owned_gids(void* h, int64_t* out) {
  Problem* P = (Problem*)h;
  std::copy(P->D.owned.begin(), P->D.owned.end(), out);
}
void orc_element_gids(void* h, int b, int64_t* out) {
  Problem* P = (Problem*)h;
  size_t k = 0;
  for (LO e : P->T.block_elems[b])
    for (GO g : P->D.elementGIDs[e]) out[k++] = g;
}
void orc_element_lids(void* h, int b, int32_t* out) {
  Problem* P = (Problem*)h;
  size_t k = 0;
  for (LO e : P->T.block_elems[b])
    for (LO l : P->D.elementLIDs[e]) out[k++] = l;
}
void orc_element_conn(void* h, int64_t e, int64_t* out, int* n) {
  Problem* P = (Problem*)h;
  *n = (int)P->D.conn[e].size();
  for (int i = 0; i < *n; ++i) out[i] = P->D.conn[e][i];
}
int orc_field_offsets(void* h, int b, int f, int32_t* out) {
  Problem* P = (Problem*)h;
  const auto& o = P->D.offsets[b][f];
  for (size_t i = 0; i < o.size(); ++i) out[i] = o[i];
  return (int)o.size();
}
void orc_graph(void* h, int64_t* rowptr, int32_t* colind) {
  Problem* P = (Problem*)h;
  std::copy(P->D.rowptr.begin(), P->D.rowptr.end(), rowptr);
  std::copy(P->D.colind.begin(), P->D.colind.end(), colind);
}
void orc_coordinates(void* h, double* xyz) {
  Problem* P = (Problem*)h;
  const Topology& T = P->T;
  for (GO k = 0; k <= T.NZ; ++k)
    for (GO j = 0; j <= T.NY; ++j)
      for (GO i = 0; i <= T.NX; ++i) {
        GO g = (T.NX + 1) * (T.NY + 1) * k + (T.NX + 1) * j + i;
        T.vertex_xyz(i, j, k, xyz + 3 * g);
      }
}
// Position of each DOF's entity (vertex / edge midpoint / face or cell centre), LID order.
void orc_dof_coordinates(void* h, double* xyz) {
  Problem* P = (Problem*)h;
  const Topology& T = P->T;
  const DofManager& D = P->D;
  for (int blk = 0; blk < T.nblocks; ++blk) {
    const BasisDef& B = D.block_basis[blk];
    int topo = T.block_topo[blk];
    int nv = topo == TX_TOPO_HEX ? 8 : 4;
    for (LO e : T.block_elems[blk]) {
      double X[24];
      T.elem_vertices(e, nv, X);
      for (int b = 0; b < B.nb; ++b) {
        double p[3] = {0, 0, 0};
        if (topo == TX_TOPO_HEX && B.kind == TX_HGRAD_C2) {
          int ip[3]; hex27_node(b, ip);
          double xi[3] = {(double)ip[0], (double)ip[1], (double)ip[2]};
          double N[8], dN[8][3];
          BasisDef G = make_basis(TX_TOPO_HEX, TX_HGRAD_C1);
          eval_hgrad(G, xi, N, dN);
          for (int n = 0; n < 8; ++n) for (int d = 0; d < 3; ++d) p[d] += N[n] * X[3 * n + d];
        } else if (topo == TX_TOPO_TET && B.kind == TX_HGRAD_C2 && b >= 4) {
          int i = kTetEdge[b - 4][0], j = kTetEdge[b - 4][1];
          for (int d = 0; d < 3; ++d) p[d] = 0.5 * (X[3 * i + d] + X[3 * j + d]);
        } else if (B.hcurl) {
          for (int d = 0; d < 3; ++d) p[d] = 0.5 * (X[3 * kHexEdge[b][0] + d] + X[3 * kHexEdge[b][1] + d]);
        } else {
          for (int d = 0; d < 3; ++d) p[d] = X[3 * b + d];
        }
        for (int f = 0; f < D.nfields; ++f) {
          LO l = D.elementLIDs[e][D.offsets[blk][f][b]];
          for (int d = 0; d < 3; ++d) xyz[3 * l + d] = p[d];
        }
      }
    }
  }
}

int orc_eval(void* h, const double* x, const double* xdot, const double* aux, double alpha, double beta, double t,
             double* f, double* vals, int block, int64_t e0, int64_t e1, int nthreads, char* errbuf, int errlen) {
  Problem* P = (Problem*)h;
  EvalIn in{x, xdot, aux, alpha, beta, t, f, vals};
  try {
    if (block < 0) {
      for (int b = 0; b < P->T.nblocks; ++b) eval_range(*P, b, 0, -1, in, nthreads);
    } else {
      eval_range(*P, block, e0, e1, in, nthreads);
    }
  } catch (std::exception& ex) {
    if (errbuf && errlen > 0) { strncpy(errbuf, ex.what(), errlen - 1); errbuf[errlen - 1] = 0; }
    return 1;
  }
  return 0;
}

int64_t orc_dirichlet_dofs(void* h, uint32_t side_mask, uint32_t field_mask, int32_t* out) {
  Problem* P = (Problem*)h;
  auto v = dirichlet_dofs(*P, side_mask, field_mask);
  if (out) std::copy(v.begin(), v.end(), out);
  return (int64_t)v.size();
}

// TpetraLinearObjContainer::applyDirichletBoundaryCondition (disc-fe/src/lof/Panzer_TpetraLinearObjContainer.hpp:
// 228-238): with a residual, f[d] = x[d] - g and the Jacobian rows become unit rows
// (applyDirichletBoundaryConditionToLocalMatrixRows); without one (f == NULL), rows and columns are cleared with
// 1 on the diagonal (applyDirichletBoundaryConditionToLocalMatrixRowsAndColumns).
void orc_dirichlet_apply(void* h, int64_t n, const int32_t* lids, const double* g, const double* x, double* f,
                         double* vals) {
  Problem* P = (Problem*)h;
  for (int64_t i = 0; i < n; ++i) {
    LO d = lids[i];
    if (f) f[d] = x[d] - (g ? g[i] : 0.0);
    if (vals)
      for (int64_t k = P->D.rowptr[d]; k < P->D.rowptr[d + 1]; ++k) vals[k] = P->D.colind[k] == d ? 1.0 : 0.0;
  }
  if (vals && !f) {
    const int64_t N = (int64_t)P->D.rowptr.size() - 1;
    std::vector<char> on(N, 0);
    for (int64_t i = 0; i < n; ++i) on[lids[i]] = 1;
    for (int64_t r = 0; r < N; ++r)
      for (int64_t k = P->D.rowptr[r]; k < P->D.rowptr[r + 1]; ++k)
        if (on[P->D.colind[k]] && P->D.colind[k] != r) vals[k] = 0.0;
  }
}

void orc_spmv(int64_t n, const int64_t* rowptr, const int32_t* colind, const double* vals, const double* x,
              double* y, double alpha, double beta) {
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    double s = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) s += vals[k] * x[colind[k]];
    y[r] = alpha * s + (beta == 0.0 ? 0.0 : beta * y[r]);
  }
}

// Jacobi-preconditioned CG in FP64 (Belos stand-in).  Returns iterations.
int orc_cg(int64_t n, const int64_t* rowptr, const int32_t* colind, const double* vals, const double* b, double* x,
           double rtol, int maxit, double* relres) {
  std::vector<double> r(n), z(n), p(n), q(n), dinv(n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double d = 0.0;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (colind[k] == i) d = vals[k];
    dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
  }
  orc_spmv(n, rowptr, colind, vals, x, q.data(), 1.0, 0.0);
  double bn = 0.0, rz = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : bn, rz)
  for (int64_t i = 0; i < n; ++i) {
    r[i] = b[i] - q[i];
    z[i] = dinv[i] * r[i];
    p[i] = z[i];
    rz += r[i] * z[i];
    bn += b[i] * b[i];
  }
  bn = std::sqrt(bn);
  if (bn == 0.0) bn = 1.0;
  int it = 0;
  double rn = 0.0;
  for (; it < maxit; ++it) {
    rn = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rn)
    for (int64_t i = 0; i < n; ++i) rn += r[i] * r[i];
    if (std::sqrt(rn) <= rtol * bn) break;
    orc_spmv(n, rowptr, colind, vals, p.data(), q.data(), 1.0, 0.0);
    double pq = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : pq)
    for (int64_t i = 0; i < n; ++i) pq += p[i] * q[i];
    double a = rz / pq;
    double rz2 = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rz2)
    for (int64_t i = 0; i < n; ++i) {
      x[i] += a * p[i];
      r[i] -= a * q[i];
      z[i] = dinv[i] * r[i];
      rz2 += r[i] * z[i];
    }
    double be = rz2 / rz;
    rz = rz2;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) p[i] = z[i] + be * p[i];
  }
  rn = 0.0;
  orc_spmv(n, rowptr, colind, vals, x, q.data(), 1.0, 0.0);
#pragma omp parallel for schedule(static) reduction(+ : rn)
  for (int64_t i = 0; i < n; ++i) rn += (b[i] - q[i]) * (b[i] - q[i]);
  if (relres) *relres = std::sqrt(rn) / bn;
  return it;
}

// ---- reference-element queries used by the known-answer tests
int orc_cubature(int topo, int degree, double* xi, double* w) {
  Cubature c = make_cubature(topo, degree);
  if (xi) std::copy(c.xi.begin(), c.xi.end(), xi);
  if (w) std::copy(c.w.begin(), c.w.end(), w);
  return c.np;
}
// Weighted measure and integration-point coordinates of one cell
int orc_cell_values(int topo, int degree, const double* X, double* wdet, double* ip) {
  Cubature c = make_cubature(topo, degree);
  ElemGeom g;
  compute_geometry(topo, X, c, g);
  if (wdet) std::copy(g.wdet.begin(), g.wdet.end(), wdet);
  if (ip) std::copy(g.ip.begin(), g.ip.end(), ip);
  return c.np;
}
// basis index carried by sub-cell (dim, c) of a (topology, basis) pair, -1 if none
int orc_basis_subcell(int topo, int basis, int dim, int c) {
  BasisDef b = make_basis(topo, basis);
  if (c < 0 || c >= b.nsub[dim]) return -2;
  return b.sub[dim][c];
}
// reference basis values (nb) and gradients (nb*3) / HCURL values and curls at xi
int orc_basis_eval(int topo, int basis, const double* xi, double* val, double* grad) {
  BasisDef b = make_basis(topo, basis);
  if (b.hcurl) {
    double V[12][3], C[12][3];
    eval_hcurl_hex(xi, V, C);
    for (int i = 0; i < 12; ++i)
      for (int d = 0; d < 3; ++d) { val[3 * i + d] = V[i][d]; grad[3 * i + d] = C[i][d]; }
  } else {
    eval_hgrad(b, xi, val, (double(*)[3])grad);
  }
  return b.nb;
}
// f += the Neumann flux of value val on block blk's sides in side_mask; returns
// the number of (cell, side) pairs, or -1 on error.
int64_t orc_neumann(void* h, int blk, uint32_t side_mask, int field, double val, double* f) {
  try {
    return neumann_flux(*(Problem*)h, blk, side_mask, field, val, f);
  } catch (std::exception&) {
    return -1;
  }
}

// *value = the integral response; dgdx (may be NULL) += its gradient.  0 or -1.
int orc_response(void* h, int blk, int field, int integrand, int degree, const double* x, double* value,
                 double* dgdx) {
  try {
    response_integral(*(Problem*)h, blk, field, integrand, degree, x, value, dgdx);
    return 0;
  } catch (std::exception&) {
    return -1;
  }
}

// ExtremeValue (use_max 1: max, 0: min), side-set integral over box sides, probe: 0 (probe: the element
// holding the point) or -1.
int orc_response_extreme(void* h, int blk, int field, int use_max, int degree, const double* x, double* value,
                         double* dgdx) {
  try {
    response_extreme(*(Problem*)h, blk, field, use_max != 0, degree, x, value, dgdx);
    return 0;
  } catch (std::exception&) {
    return -1;
  }
}
int orc_response_side(void* h, int blk, uint32_t side_mask, int field, const double* x, double* value, double* dgdx) {
  try {
    response_side(*(Problem*)h, blk, side_mask, field, x, value, dgdx);
    return 0;
  } catch (std::exception&) {
    return -1;
  }
}
int64_t orc_response_probe(void* h, const double* pt, int field, const double* x, double* value, double* dgdx) {
  try {
    return (int64_t)response_probe(*(Problem*)h, pt, field, x, value, dgdx);
  } catch (std::exception&) {
    return -1;
  }
}

int orc_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
