// tx_setup.cpp -- host-side set-up of the assembly path: brick lattice,
// entity ids, DOF numbering, entity graph, element-to-row maps and the
// reference-element tables.  Runs once per mesh (the reference does the
// same work on the host: DOFManager::buildGlobalUnknowns,
// TpetraLinearObjFactory::buildGhostedGraph, panzer::buildWorksets).
//
// Numbering equals the reference's one-rank result bit for bit:
//   * entity GIDs of the Cartesian lattice as in CartesianConnManager::
//     updateConnectivity_3d (dof-mgr/test/cartesian_topology/
//     CartesianConnManager.cpp:744-890), written here per entity family;
//   * DOF GIDs: entities in ascending entity GID, fields interleaved per
//     entity (GUN, dof-mgr/src/Panzer_DOFManager.cpp:827-843), computed as
//     a prefix sum over a dense entity-GID array instead of Tpetra maps;
//   * LIDs: first touch over blocks / elements / element GIDs
//     (Panzer_DOFManager.cpp:602-660).  Because every DOF-carrying entity
//     holds one DOF per field and its DOFs are consecutive in the element
//     GID vector, first touch of an entity numbers all its DOFs at once:
//     LID(entity, f) = nf * entityLID + f;
//   * graph rows by LID, columns ascending LID (Tpetra fillComplete).  The
//     graph is kept at entity level (an nf x nf block pattern); the DOF-level
//     Tpetra arrays are expanded on the GPU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>

#include "tx_internal.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace tx {

// ------------------------------------------------------------ brick tables
// Brick vertex n -> lattice offset, shards Hexahedron<8> order.
static const int kVtx[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                               {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
// Brick edges 0..11 (shards order) as (first, second) brick vertices.
static const int kEdgeVtx[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                    {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// Brick faces 0..5 (shards order) as their 4 vertices.
static const int kFaceVtx[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6},
                                   {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
// The six-tet split of a brick and the brick-edge ids of each tet's edges
// (ids 12..17 = diagonal of brick face id-12, 18 = body diagonal).  These
// tables fix the tet mesh and must equal the reference's
// (CartesianConnManager.cpp:220-239).
static const int kTets[6][4] = {{0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6},
                                {0, 5, 6, 4}, {1, 5, 6, 0}, {1, 6, 2, 0}};
static const int kTetEdges[6][6] = {{16, 2, 3, 18, 10, 14}, {3, 11, 15, 18, 14, 6},
                                    {15, 7, 8, 18, 6, 17},  {12, 5, 18, 8, 4, 17},
                                    {9, 5, 13, 0, 12, 18},  {13, 10, 1, 0, 18, 16}};
static const int kTetEdgeVtx[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};

// ------------------------------------------------------------ lattice ids
// An entity of the brick lattice in doubled coordinates: vertices at even
// positions, edge midpoints odd in one coordinate, faces odd in two, brick
// centres odd in all three.  Tet face diagonals and body diagonals share
// the position (and the GID) of the brick face / brick they bisect.
struct Lattice {
  int64_t NX, NY, NZ;
  int64_t nodes, hexEdges, hexFaces;
  int64_t edgeLayer, edgeLevel;  // horizontal edges per level, edges per level
  int64_t faceLevel;             // faces per level
  void init(int64_t nx, int64_t ny, int64_t nz) {
    NX = nx; NY = ny; NZ = nz;
    nodes = (NX + 1) * (NY + 1) * (NZ + 1);
    edgeLayer = (NX + 1) * NY + NX * (NY + 1);
    edgeLevel = edgeLayer + (NX + 1) * (NY + 1);
    faceLevel = NX * NY + (NX + 1) * NY + NX * (NY + 1);
    hexEdges = edgeLevel * NZ + edgeLayer;
    hexFaces = faceLevel * NZ + NX * NY;
  }
  // GID from doubled coordinates (a, b, c)
  int64_t gid(int64_t a, int64_t b, int64_t c) const {
    int64_t i = a >> 1, j = b >> 1, k = c >> 1;
    int odd = (int)(a & 1) + 2 * (int)(b & 1) + 4 * (int)(c & 1);
    switch (odd) {
      case 0: return ((NY + 1) * k + j) * (NX + 1) + i;                                  // vertex
      case 1: return nodes + k * edgeLevel + j * (2 * NX + 1) + i;                       // x-edge
      case 2: return nodes + k * edgeLevel + j * (2 * NX + 1) + NX + i;                  // y-edge
      case 4: return nodes + k * edgeLevel + edgeLayer + j * (NX + 1) + i;               // z-edge
      case 3: return nodes + hexEdges + k * faceLevel + j * NX + i;                      // z-normal face
      case 5: return nodes + hexEdges + k * faceLevel + NX * NY + j * (2 * NX + 1) + i;  // y-normal face
      case 6: return nodes + hexEdges + k * faceLevel + NX * NY + j * (2 * NX + 1) + NX + i;  // x-normal
      default: return nodes + hexEdges + hexFaces + (k * NY + j) * NX + i;                   // brick
    }
  }
};

// Doubled-coordinate offset (within a brick, 0..2 per axis) of a sub-cell of
// a brick element: dim 0 vertex n, dim 1 brick edge id (0..18), dim 2 hex
// face, dim 3 the brick.
static void brick_entity_offset(int dim, int id, int o[3]) {
  if (dim == 0) { for (int d = 0; d < 3; ++d) o[d] = 2 * kVtx[id][d]; return; }
  if (dim == 1 && id < 12) {
    for (int d = 0; d < 3; ++d) o[d] = kVtx[kEdgeVtx[id][0]][d] + kVtx[kEdgeVtx[id][1]][d];
    return;
  }
  if (dim == 1 && id < 18) { brick_entity_offset(2, id - 12, o); return; }
  if (dim == 1 || dim == 3) { o[0] = o[1] = o[2] = 1; return; }
  for (int d = 0; d < 3; ++d) {
    int s = 0;
    for (int k = 0; k < 4; ++k) s += kVtx[kFaceVtx[id][k]][d];
    o[d] = s / 2;
  }
}

// ------------------------------------------------------------ reference
int default_degree(int topo, int basis) { return (topo == TX_TOPO_HEX && basis == TX_HGRAD_C2) ? 4 : 2; }

static int n_basis(int topo, int basis) {
  if (topo == TX_TOPO_HEX) return basis == TX_HGRAD_C1 ? 8 : basis == TX_HGRAD_C2 ? 27 : 12;
  return basis == TX_HGRAD_C1 ? 4 : basis == TX_HGRAD_C2 ? 10 : -1;
}

// Basis index carried by sub-cell (dim, c); -1 if none (Intrepid2 DOF tags:
// HEX_C2 edge/face nodes in shards Hexahedron<27> order).
static int subcell_basis(int topo, int basis, int dim, int c) {
  if (basis == TX_HCURL_I1) return dim == 1 ? c : -1;
  if (dim == 0) return c;
  if (basis == TX_HGRAD_C1) return -1;
  if (topo == TX_TOPO_TET) return dim == 1 ? 4 + c : -1;
  if (dim == 1) return c < 4 ? 8 + c : (c < 8 ? 12 + c : c + 4);
  if (dim == 2) { static const int fn[6] = {25, 24, 26, 23, 21, 22}; return fn[c]; }
  return 20;
}

// Reference position of HEX_C2 node b in {-1,0,1}^3.
static void hex27_position(int b, int p[3]) {
  for (int dim = 0; dim < 4; ++dim) {
    int nsc = dim == 0 ? 8 : dim == 1 ? 12 : dim == 2 ? 6 : 1;
    for (int c = 0; c < nsc; ++c)
      if (subcell_basis(TX_TOPO_HEX, TX_HGRAD_C2, dim, c) == b) {
        int o[3];
        brick_entity_offset(dim, dim == 3 ? 18 : c, o);
        for (int d = 0; d < 3; ++d) p[d] = o[d] - 1;
        return;
      }
  }
  throw std::runtime_error("hex27_position");
}

static void gauss_points(int n, double* p, double* w) {
  // Gauss-Legendre on [-1,1], points listed from +1 towards -1
  if (n == 1) { p[0] = 0.0; w[0] = 2.0; return; }
  if (n == 2) { p[0] = std::sqrt(1.0 / 3.0); p[1] = -p[0]; w[0] = w[1] = 1.0; return; }
  if (n == 3) {
    p[0] = std::sqrt(3.0 / 5.0); p[1] = 0.0; p[2] = -p[0];
    w[0] = w[2] = 5.0 / 9.0; w[1] = 8.0 / 9.0;
    return;
  }
  if (n == 4) {  // roots of P4: sqrt(3/7 -+ 2/7 sqrt(6/5)), weights (18 +- sqrt(30)) / 36
    const double a = std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * std::sqrt(1.2));
    const double b = std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * std::sqrt(1.2));
    p[0] = a; p[1] = b; p[2] = -b; p[3] = -a;
    w[0] = w[3] = (18.0 - std::sqrt(30.0)) / 36.0;
    w[1] = w[2] = (18.0 + std::sqrt(30.0)) / 36.0;
    return;
  }
  throw std::runtime_error("gauss_points: 1 to 4 points per direction (degree <= 7)");
}

std::vector<double> RefTables::packed() const {
  std::vector<double> out;
  out.insert(out.end(), w.begin(), w.end());
  out.insert(out.end(), geo_val.begin(), geo_val.end());
  out.insert(out.end(), geo_grad.begin(), geo_grad.end());
  out.insert(out.end(), val.begin(), val.end());
  out.insert(out.end(), grad.begin(), grad.end());
  return out;
}

static void eval_tables(RefTables& R);

static RefTables blank_tables(int topo, int basis, int degree) {
  RefTables R;
  R.topo = topo; R.basis = basis; R.degree = degree;
  R.nb = n_basis(topo, basis);
  if (R.nb < 0) throw std::runtime_error("unsupported topology/basis");
  R.hcurl = basis == TX_HCURL_I1;
  R.nv = topo == TX_TOPO_HEX ? 8 : 4;
  return R;
}

RefTables make_ref_tables(int topo, int basis, int degree) {
  RefTables R = blank_tables(topo, basis, degree);
  if (topo == TX_TOPO_HEX) {
    int n = degree / 2 + 1;
    double p[4], w[4];
    gauss_points(n, p, w);
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          R.xi.insert(R.xi.end(), {p[i], p[j], p[k]});
          R.w.push_back(w[i] * w[j] * w[k]);
        }
  } else {
    if (degree != 2) throw std::runtime_error("tet cubature: only degree 2 (4 points)");
    const double a = 0.5854101966249685, b = 0.1381966011250105;
    R.xi = {b, b, b, a, b, b, b, a, b, b, b, a};
    R.w.assign(4, 1.0 / 24.0);
  }
  eval_tables(R);
  return R;
}

RefTables tables_at(int topo, int basis, const double* xi, int n) {
  RefTables R = blank_tables(topo, basis, 0);
  R.xi.assign(xi, xi + 3 * n);
  R.w.assign(n, 0.0);
  eval_tables(R);
  return R;
}

bool locate_point(const Mesh& m, const Dofs& D, const double p[3], int& block, int64_t& elem, double xi[3]) {
  for (int b = 0; b < m.nblocks; ++b) {
    const BlockDofs& B = D.blocks[b];
    const int nv = B.nv, topo = B.topo;
    const int64_t E = (int64_t)m.block_elems[b].size();
    for (int64_t i = 0; i < E; ++i) {
      const int32_t* vc = &B.vconn[i * nv];
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      for (int v = 0; v < nv; ++v)
        for (int d = 0; d < 3; ++d) {
          lo[d] = std::min(lo[d], m.coords[3 * vc[v] + d]);
          hi[d] = std::max(hi[d], m.coords[3 * vc[v] + d]);
        }
      bool box = true;
      for (int d = 0; d < 3; ++d) box = box && p[d] >= lo[d] - 1e-12 && p[d] <= hi[d] + 1e-12;
      if (!box) continue;
      // Newton on x(xi) = p with the geometry basis (trilinear hex, linear tet)
      double z[3] = {0.0, 0.0, 0.0};
      if (topo == TX_TOPO_TET) z[0] = z[1] = z[2] = 0.25;
      for (int it = 0; it < 50; ++it) {
        const RefTables G = tables_at(topo, TX_HGRAD_C1, z, 1);
        double r[3] = {-p[0], -p[1], -p[2]}, J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int v = 0; v < nv; ++v)
          for (int a = 0; a < 3; ++a) {
            const double xa = m.coords[3 * vc[v] + a];
            r[a] += G.geo_val[v] * xa;
            for (int c = 0; c < 3; ++c) J[3 * a + c] += xa * G.geo_grad[3 * v + c];
          }
        const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[5] * J[6] - J[3] * J[8], c02 = J[3] * J[7] - J[4] * J[6];
        const double det = J[0] * c00 + J[1] * c01 + J[2] * c02;
        if (det == 0.0) break;
        const double Ji[9] = {c00 / det, (J[2] * J[7] - J[1] * J[8]) / det, (J[1] * J[5] - J[2] * J[4]) / det,
                              c01 / det, (J[0] * J[8] - J[2] * J[6]) / det, (J[2] * J[3] - J[0] * J[5]) / det,
                              c02 / det, (J[1] * J[6] - J[0] * J[7]) / det, (J[0] * J[4] - J[1] * J[3]) / det};
        double step = 0.0;
        for (int a = 0; a < 3; ++a) {
          const double d = Ji[3 * a] * r[0] + Ji[3 * a + 1] * r[1] + Ji[3 * a + 2] * r[2];
          z[a] -= d;
          step = std::max(step, std::fabs(d));
        }
        if (step < 1e-15) break;
      }
      const double tol = 1e-10;
      const bool inside = topo == TX_TOPO_HEX
                              ? std::fabs(z[0]) <= 1 + tol && std::fabs(z[1]) <= 1 + tol && std::fabs(z[2]) <= 1 + tol
                              : z[0] >= -tol && z[1] >= -tol && z[2] >= -tol && z[0] + z[1] + z[2] <= 1 + tol;
      if (!inside) continue;
      block = b; elem = i;
      xi[0] = z[0]; xi[1] = z[1]; xi[2] = z[2];
      return true;
    }
  }
  return false;
}

// shards Tetrahedron<4> side (face) node order
static const int kTetSideVtx[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};

// Side rules: the reference side's cubature of the block's degree mapped to
// the element's reference coordinates (CellTools::mapToReferenceSubcell).
// Hex faces: n x n Gauss points on [-1,1]^2 (n = degree/2 + 1, u fastest),
// x(u,v) = c + u t_u + v t_v with c the face centre and t_u = (V1 - V0)/2,
// t_v = (V3 - V0)/2 over the face's vertices in shards order (the faces are
// parallelograms, so this is the bilinear side map, and the face's fixed
// coordinate stays exactly +-1).  Tet faces: 3-point degree-2 triangle rule
// ((1/6,1/6), (2/3,1/6), (1/6,2/3), weights 1/6), x(u,v) = V0 + u (V1-V0) +
// v (V2-V0).  For these flat reference sides the tangents are constants.
SideTables make_side_tables(int topo, int basis, int degree) {
  SideTables S;
  S.nsides = topo == TX_TOPO_HEX ? 6 : 4;
  if (basis == TX_HCURL_I1) throw std::runtime_error("side tables: HGRAD bases only");
  for (int s = 0; s < S.nsides; ++s) {
    RefTables R = blank_tables(topo, basis, degree);
    double tu[3], tv[3];
    if (topo == TX_TOPO_HEX) {
      double V[4][3];
      for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) V[k][d] = kVtx[kFaceVtx[s][k]][d] ? 1.0 : -1.0;
      double c[3];
      for (int d = 0; d < 3; ++d) {
        tu[d] = 0.5 * (V[1][d] - V[0][d]);
        tv[d] = 0.5 * (V[3][d] - V[0][d]);
        c[d] = 0.25 * (V[0][d] + V[1][d] + V[2][d] + V[3][d]);
      }
      const int n = degree / 2 + 1;
      double p[4], w[4];
      gauss_points(n, p, w);
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          for (int d = 0; d < 3; ++d) R.xi.push_back(c[d] + p[i] * tu[d] + p[j] * tv[d]);
          R.w.push_back(w[i] * w[j]);
        }
    } else {
      if (degree != 2) throw std::runtime_error("tet side cubature: only degree 2");
      static const double ref[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      const double* V0 = ref[kTetSideVtx[s][0]];
      const double* V1 = ref[kTetSideVtx[s][1]];
      const double* V2 = ref[kTetSideVtx[s][2]];
      for (int d = 0; d < 3; ++d) { tu[d] = V1[d] - V0[d]; tv[d] = V2[d] - V0[d]; }
      const double uv[3][2] = {{1.0 / 6, 1.0 / 6}, {2.0 / 3, 1.0 / 6}, {1.0 / 6, 2.0 / 3}};
      for (int q = 0; q < 3; ++q) {
        for (int d = 0; d < 3; ++d) R.xi.push_back(V0[d] + uv[q][0] * tu[d] + uv[q][1] * tv[d]);
        R.w.push_back(1.0 / 6);
      }
    }
    eval_tables(R);
    if (s == 0) {
      S.nqf = R.nq; S.nb = R.nb; S.nv = R.nv;
      S.stride = S.nqf * (1 + 3 * S.nv + S.nb) + 6;
      S.packed.assign((size_t)S.nsides * S.stride, 0.0);
    }
    double* o = S.packed.data() + (size_t)s * S.stride;
    o = std::copy(R.w.begin(), R.w.end(), o);
    o = std::copy(R.geo_grad.begin(), R.geo_grad.end(), o);
    o = std::copy(R.val.begin(), R.val.end(), o);
    for (int d = 0; d < 3; ++d) *o++ = tu[d];
    for (int d = 0; d < 3; ++d) *o++ = tv[d];
  }
  return S;
}

std::vector<int64_t> side_workset(const Mesh& m, int block, uint32_t side_mask) {
  if (m.is_explicit) throw std::invalid_argument("box sides are not defined on an explicit mesh; use a side set");
  std::vector<int64_t> out;
  const int topo = m.desc.block_topology[block];
  const int nsides = topo == TX_TOPO_HEX ? 6 : 4;
  const int64_t lim[3] = {m.NX, m.NY, m.NZ};
  const std::vector<int64_t>& elems = m.block_elems[block];
  for (int64_t i = 0; i < (int64_t)elems.size(); ++i) {
    const int64_t e = elems[i];
    const int64_t b = m.elem_brick[e];
    const int64_t ijk[3] = {b % m.NX, (b / m.NX) % m.NY, b / (m.NX * m.NY)};
    const int sub = m.elem_sub[e];
    for (int s = 0; s < nsides; ++s) {
      int bv[4], n = topo == TX_TOPO_HEX ? 4 : 3;
      for (int k = 0; k < n; ++k) bv[k] = topo == TX_TOPO_HEX ? kFaceVtx[s][k] : kTets[sub][kTetSideVtx[s][k]];
      bool on = false;
      for (int side = 0; side < 6 && !on; ++side) {
        if (!(side_mask & (1u << side))) continue;
        const int axis = side / 2;
        const int64_t want = (side & 1) ? lim[axis] : 0;
        bool all = true;
        for (int k = 0; k < n && all; ++k) all = ijk[axis] + kVtx[bv[k]][axis] == want;
        on = all;
      }
      if (on) out.push_back(i * 8 + s);
    }
  }
  return out;
}

static void eval_tables(RefTables& R) {
  const int topo = R.topo, basis = R.basis;
  R.nq = (int)R.w.size();
  const int nq = R.nq, nb = R.nb, nv = R.nv;
  R.geo_val.assign(nq * nv, 0.0);
  R.geo_grad.assign(nq * nv * 3, 0.0);
  R.val.assign(nq * nb * (R.hcurl ? 3 : 1), 0.0);
  R.grad.assign(nq * nb * 3, 0.0);
  for (int q = 0; q < nq; ++q) {
    const double* x = &R.xi[3 * q];
    // geometry basis: trilinear hex / linear tet
    for (int v = 0; v < nv; ++v) {
      double val, g[3];
      if (topo == TX_TOPO_HEX) {
        double f[3], df[3];
        for (int d = 0; d < 3; ++d) {
          double s = kVtx[v][d] ? 1.0 : -1.0;
          f[d] = 0.5 * (1.0 + s * x[d]);
          df[d] = 0.5 * s;
        }
        val = f[0] * f[1] * f[2];
        g[0] = df[0] * f[1] * f[2]; g[1] = f[0] * df[1] * f[2]; g[2] = f[0] * f[1] * df[2];
      } else {
        val = v == 0 ? 1.0 - x[0] - x[1] - x[2] : x[v - 1];
        for (int d = 0; d < 3; ++d) g[d] = v == 0 ? -1.0 : (d == v - 1 ? 1.0 : 0.0);
      }
      R.geo_val[q * nv + v] = val;
      for (int d = 0; d < 3; ++d) R.geo_grad[(q * nv + v) * 3 + d] = g[d];
    }
    if (R.hcurl) {
      // lowest-order Nedelec: edge k along axis a, tangent sign s,
      // phi = s * prod_{d != a} (1 + c_d x_d) / 4 * e_a,  curl_i = eps_{i j a} d_j phi_a;
      // dual to u(edge midpoint) . (half edge vector), the quadrilateral I1
      // convention extended so that face traces are the quadrilateral functions
      for (int e = 0; e < 12; ++e) {
        const int* v0 = kVtx[kEdgeVtx[e][0]];
        const int* v1 = kVtx[kEdgeVtx[e][1]];
        int a = 0;
        for (int d = 0; d < 3; ++d) if (v0[d] != v1[d]) a = d;
        double s = v1[a] > v0[a] ? 1.0 : -1.0;
        double c[3], fac[3];
        for (int d = 0; d < 3; ++d) { c[d] = v0[d] ? 1.0 : -1.0; fac[d] = d == a ? 1.0 : 1.0 + c[d] * x[d]; }
        double phi = s * fac[0] * fac[1] * fac[2] / 4.0;
        double dphi[3];
        for (int j = 0; j < 3; ++j) {
          if (j == a) { dphi[j] = 0.0; continue; }
          double prod = s / 4.0;
          for (int d = 0; d < 3; ++d) prod *= (d == j) ? c[d] : fac[d];
          dphi[j] = prod;
        }
        R.val[(q * nb + e) * 3 + a] = phi;
        for (int i = 0; i < 3; ++i) {
          double cu = 0.0;
          for (int j = 0; j < 3; ++j) {
            // Levi-Civita eps_{i j a}
            int eps = 0;
            if (i != j && j != a && i != a) eps = ((j - i + 3) % 3 == 1) ? 1 : -1;
            cu += eps * dphi[j];
          }
          R.grad[(q * nb + e) * 3 + i] = cu;
        }
      }
    } else if (topo == TX_TOPO_HEX) {
      for (int b = 0; b < nb; ++b) {
        int pos[3];
        if (basis == TX_HGRAD_C1) { for (int d = 0; d < 3; ++d) pos[d] = kVtx[b][d] ? 1 : -1; }
        else hex27_position(b, pos);
        double f[3], df[3];
        for (int d = 0; d < 3; ++d) {
          double s = x[d];
          if (basis == TX_HGRAD_C1) { f[d] = 0.5 * (1.0 + pos[d] * s); df[d] = 0.5 * pos[d]; }
          else if (pos[d] == 0) { f[d] = (1.0 - s) * (1.0 + s); df[d] = -2.0 * s; }
          else { f[d] = 0.5 * s * (s + pos[d]); df[d] = s + 0.5 * pos[d]; }
        }
        R.val[q * nb + b] = f[0] * f[1] * f[2];
        R.grad[(q * nb + b) * 3 + 0] = df[0] * f[1] * f[2];
        R.grad[(q * nb + b) * 3 + 1] = f[0] * df[1] * f[2];
        R.grad[(q * nb + b) * 3 + 2] = f[0] * f[1] * df[2];
      }
    } else {
      double lam[4] = {1.0 - x[0] - x[1] - x[2], x[0], x[1], x[2]};
      double dl[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      for (int b = 0; b < nb; ++b) {
        double v, g[3];
        if (b < 4 && basis == TX_HGRAD_C1) {
          v = lam[b];
          for (int d = 0; d < 3; ++d) g[d] = dl[b][d];
        } else if (b < 4) {
          v = lam[b] * (2.0 * lam[b] - 1.0);
          for (int d = 0; d < 3; ++d) g[d] = (4.0 * lam[b] - 1.0) * dl[b][d];
        } else {
          int i = kTetEdgeVtx[b - 4][0], j = kTetEdgeVtx[b - 4][1];
          v = 4.0 * lam[i] * lam[j];
          for (int d = 0; d < 3; ++d) g[d] = 4.0 * (dl[i][d] * lam[j] + lam[i] * dl[j][d]);
        }
        R.val[q * nb + b] = v;
        for (int d = 0; d < 3; ++d) R.grad[(q * nb + b) * 3 + d] = g[d];
      }
    }
  }
}

// ------------------------------------------------------------------ mesh
static inline uint64_t splitmix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void build_mesh(Mesh& m, const tx_mesh_desc& d) {
  if (d.nx < 1 || d.ny < 1 || d.nz < 1 || d.bx < 1 || d.by < 1 || d.bz < 1)
    throw std::invalid_argument("tx_mesh_create: sizes must be >= 1");
  if (d.bx * d.by * d.bz > TX_MAX_BLOCKS) throw std::invalid_argument("tx_mesh_create: too many blocks");
  if (!(d.lx > 0 && d.ly > 0 && d.lz > 0)) throw std::invalid_argument("tx_mesh_create: lengths must be > 0");
  m.desc = d;
  m.NX = (int64_t)d.nx * d.bx; m.NY = (int64_t)d.ny * d.by; m.NZ = (int64_t)d.nz * d.bz;
  m.nblocks = d.bx * d.by * d.bz;
  for (int b = 0; b < m.nblocks; ++b)
    if (d.block_topology[b] != TX_TOPO_HEX && d.block_topology[b] != TX_TOPO_TET)
      throw std::invalid_argument("tx_mesh_create: unknown topology");
  Lattice L;
  L.init(m.NX, m.NY, m.NZ);
  m.n_nodes = L.nodes; m.n_hex_edges = L.hexEdges; m.n_hex_faces = L.hexFaces;
  m.n_bricks = m.NX * m.NY * m.NZ;
  if (m.n_nodes >= (int64_t)INT32_MAX) throw std::invalid_argument("tx_mesh_create: more than 2^31 vertices");
  // elements: bricks in x-fastest order, each expanding to its block's
  // sub-elements (1 hex or 6 tets); block element lists ascending
  m.block_elems.assign(m.nblocks, {});
  m.elem_brick.clear(); m.elem_sub.clear();
  for (int64_t b = 0; b < m.n_bricks; ++b) {
    int64_t I = b % m.NX, J = (b / m.NX) % m.NY, K = b / (m.NX * m.NY);
    int blk = ((int)(I / d.nx) * d.by + (int)(J / d.ny)) * d.bz + (int)(K / d.nz);
    int nsub = d.block_topology[blk] == TX_TOPO_HEX ? 1 : 6;
    for (int s = 0; s < nsub; ++s) {
      m.block_elems[blk].push_back((int64_t)m.elem_brick.size());
      m.elem_brick.push_back(b);
      m.elem_sub.push_back((int8_t)s);
    }
  }
  m.n_elements = (int64_t)m.elem_brick.size();
  // vertex coordinates with seeded interior jitter
  m.coords.assign(3 * m.n_nodes, 0.0);
  const double h[3] = {d.lx / m.NX, d.ly / m.NY, d.lz / m.NZ};
  const int64_t n[3] = {m.NX, m.NY, m.NZ};
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < m.n_nodes; ++g) {
    int64_t ijk[3] = {g % (m.NX + 1), (g / (m.NX + 1)) % (m.NY + 1), g / ((m.NX + 1) * (m.NY + 1))};
    bool inside = true;
    for (int c = 0; c < 3; ++c) inside = inside && ijk[c] > 0 && ijk[c] < n[c];
    for (int c = 0; c < 3; ++c) {
      double x = (double)ijk[c] * h[c];
      if (inside && d.jitter != 0.0) {
        uint64_t r = splitmix(d.seed ^ splitmix((uint64_t)g * 3ull + (uint64_t)c));
        double u = 2.0 * ((double)(r >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
        x = x + d.jitter * h[c] * u;
      }
      m.coords[3 * g + c] = x;
    }
  }
}

void build_mesh_explicit(Mesh& m, ExplicitMesh&& x) {
  const int nb = (int)x.blocks.size();
  if (nb < 1 || nb > TX_MAX_BLOCKS) throw std::invalid_argument("explicit mesh: 1 to 8 element blocks");
  if (x.n_nodes < 1 || x.n_nodes >= (int64_t)INT32_MAX) throw std::invalid_argument("explicit mesh: node count");
  if ((int64_t)x.coords.size() != 3 * x.n_nodes) throw std::invalid_argument("explicit mesh: coordinates");
  m = Mesh();
  m.is_explicit = true;
  m.nblocks = nb;
  m.n_nodes = x.n_nodes;
  m.block_elems.assign(nb, {});
  m.block_first.assign(nb, 0);
  int64_t ne = 0;
  for (int b = 0; b < nb; ++b) {
    const ExplicitBlock& B = x.blocks[b];
    if (B.topology != TX_TOPO_HEX && B.topology != TX_TOPO_TET)
      throw std::invalid_argument("explicit mesh: blocks are hex8 or tet4");
    const int nv = B.topology == TX_TOPO_HEX ? 8 : 4, nq = B.topology == TX_TOPO_HEX ? 27 : 10;
    if (B.npe == 0) x.blocks[b].npe = nv;
    const int npe = x.blocks[b].npe;
    if (npe != nv && npe != nq) throw std::invalid_argument("explicit mesh: nodes per element (vertices or quadratic)");
    if (B.n_elem < 0 || (int64_t)B.conn.size() != B.n_elem * npe)
      throw std::invalid_argument("explicit mesh: connectivity size");
    for (int64_t v : B.conn)
      if (v < 0 || v >= x.n_nodes) throw std::invalid_argument("explicit mesh: node number out of range");
    m.desc.block_topology[b] = B.topology;
    m.block_first[b] = ne;
    for (int64_t i = 0; i < B.n_elem; ++i) m.block_elems[b].push_back(ne + i);
    ne += B.n_elem;
  }
  m.n_elements = ne;
  for (const ExplicitSet& S : x.side_sets) {
    if (S.entries.size() % 2) throw std::invalid_argument("explicit mesh: side set entries come in pairs");
    for (size_t i = 0; i < S.entries.size(); i += 2) {
      const int64_t e = S.entries[i], s = S.entries[i + 1];
      if (e < 0 || e >= ne) throw std::invalid_argument("explicit mesh: side set element out of range");
      int b = nb - 1;
      while (b > 0 && m.block_first[b] > e) --b;
      if (s < 0 || s >= (x.blocks[b].topology == TX_TOPO_HEX ? 6 : 4))
        throw std::invalid_argument("explicit mesh: side ordinal out of range");
    }
  }
  for (const ExplicitSet& S : x.node_sets)
    for (int64_t v : S.entries)
      if (v < 0 || v >= x.n_nodes) throw std::invalid_argument("explicit mesh: node set node out of range");
  m.coords = x.coords;
  m.ex = std::move(x);
}

std::vector<int64_t> side_set_workset(const Mesh& m, int block, int side_set) {
  if (!m.is_explicit || side_set < 0 || side_set >= (int)m.ex.side_sets.size())
    throw std::out_of_range("side set out of range");
  const int64_t lo = m.block_first[block], hi = lo + (int64_t)m.block_elems[block].size();
  const std::vector<int64_t>& en = m.ex.side_sets[side_set].entries;
  std::vector<int64_t> out;
  for (size_t i = 0; i < en.size(); i += 2)
    if (en[i] >= lo && en[i] < hi) out.push_back((en[i] - lo) * 8 + en[i + 1]);
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return out;
}

std::vector<int32_t> node_set_dofs(const Dofs& D, const Mesh& m, int node_set, uint32_t field_mask) {
  if (!m.is_explicit || node_set < 0 || node_set >= (int)m.ex.node_sets.size())
    throw std::out_of_range("node set out of range");
  std::vector<int32_t> lid(m.n_nodes, -1);
  for (int64_t e = 0; e < D.n_entities; ++e) lid[D.ent_gid[e]] = (int32_t)e;
  std::vector<int32_t> out;
  for (int64_t v : m.ex.node_sets[node_set].entries) {
    if (lid[v] < 0) continue;
    for (int f = 0; f < D.nf; ++f)
      if (field_mask & (1u << f)) out.push_back(lid[v] * D.nf + f);
  }
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return out;
}

int element_vertices(const Mesh& m, int block, int64_t* out) {
  const int topo = m.desc.block_topology[block];
  const int nv = topo == TX_TOPO_HEX ? 8 : 4;
  const std::vector<int64_t>& el = m.block_elems[block];
  if (m.is_explicit) {
    const ExplicitBlock& B = m.ex.blocks[block];
    for (int64_t i = 0; i < B.n_elem; ++i)
      for (int v = 0; v < nv; ++v) out[i * nv + v] = B.conn[i * B.npe + v];
    return nv;
  }
  Lattice L;
  L.init(m.NX, m.NY, m.NZ);
  for (size_t i = 0; i < el.size(); ++i) {
    const int64_t br = m.elem_brick[el[i]];
    const int64_t I = br % m.NX, J = (br / m.NX) % m.NY, K = br / (m.NX * m.NY);
    for (int v = 0; v < nv; ++v) {
      const int bv = topo == TX_TOPO_HEX ? v : kTets[m.elem_sub[el[i]]][v];
      out[i * nv + v] = L.gid(2 * (I + kVtx[bv][0]), 2 * (J + kVtx[bv][1]), 2 * (K + kVtx[bv][2]));
    }
  }
  return nv;
}

// ------------------------------------------------------------------ dofs
static void color_block(BlockDofs& B, int64_t E, int64_t n_entities);

void build_dofs(const Mesh& m, Dofs& D, const tx_equation_set_desc& q) {
  D.eq = q;
  D.nf = q.physics == TX_PHYS_ELASTICITY ? 3 : 1;
  if (q.physics != TX_PHYS_POISSON && q.physics != TX_PHYS_ELASTICITY && q.physics != TX_PHYS_HEAT &&
      q.physics != TX_PHYS_MAXWELL)
    throw std::invalid_argument("tx_dof_build: unknown physics");
  const int nf = D.nf;
  const bool ex = m.is_explicit;
  Lattice L;
  if (!ex) L.init(m.NX, m.NY, m.NZ);
  const int64_t gid_space = ex ? m.n_nodes : L.nodes + L.hexEdges + L.hexFaces + m.n_bricks;
  bool orient = false;
  D.blocks.assign(m.nblocks, BlockDofs());
  for (int b = 0; b < m.nblocks; ++b) {
    BlockDofs& B = D.blocks[b];
    B.topo = m.desc.block_topology[b];
    B.basis = q.block_basis[b];
    if ((B.basis == TX_HCURL_I1) != (q.physics == TX_PHYS_MAXWELL))
      throw std::invalid_argument("tx_dof_build: HCURL basis goes with MAXWELL physics only");
    if (B.basis == TX_HCURL_I1 && B.topo != TX_TOPO_HEX)
      throw std::invalid_argument("tx_dof_build: HCURL is provided on hexahedra only");
    if (ex && B.basis != TX_HGRAD_C1 && B.basis != TX_HGRAD_C2)
      throw std::invalid_argument("tx_dof_build: explicit meshes carry nodal (HGRAD) fields only");
    if (ex && B.basis == TX_HGRAD_C2 && m.ex.blocks[b].npe != n_basis(B.topo, B.basis))
      throw std::invalid_argument("tx_dof_build: quadratic fields need quadratic (hex27 / tet10) connectivity");
    B.degree = q.integration_order[b] > 0 ? q.integration_order[b] : default_degree(B.topo, B.basis);
    B.ref = make_ref_tables(B.topo, B.basis, B.degree);
    B.nb = B.ref.nb; B.nv = B.ref.nv;
    if (B.basis == TX_HCURL_I1) orient = true;
  }
  // geometric pattern per block: DOF-carrying sub-cells in (dim, subcell)
  // order, plus vertices when orientations are needed
  for (int b = 0; b < m.nblocks; ++b) {
    BlockDofs& B = D.blocks[b];
    const int nsc[4] = {B.topo == TX_TOPO_HEX ? 8 : 4, B.topo == TX_TOPO_HEX ? 12 : 6, B.topo == TX_TOPO_HEX ? 6 : 4, 1};
    B.geom_dim.clear(); B.geom_sub.clear(); B.geom_basis.clear();
    B.basis_pos.assign(B.nb, -1);
    int pos = 0;
    for (int dim = 0; dim < 4; ++dim)
      for (int c = 0; c < nsc[dim]; ++c) {
        int bi = subcell_basis(B.topo, B.basis, dim, c);
        if (bi < 0 && !(orient && dim == 0)) continue;
        B.geom_dim.push_back(dim); B.geom_sub.push_back(c); B.geom_basis.push_back(bi);
        if (bi >= 0) B.basis_pos[bi] = pos++;
      }
  }
  // per element: lattice position of each basis' entity; mark DOF entities
  std::vector<uint8_t> has(gid_space, 0);
  std::vector<std::vector<int64_t>> egid(m.nblocks);  // [E][nb] entity GIDs in basis order
  std::vector<std::vector<int32_t>> epos3(m.nblocks); // doubled lattice positions [E][nb][3]
  for (int b = 0; b < m.nblocks; ++b) {
    BlockDofs& B = D.blocks[b];
    const auto& el = m.block_elems[b];
    const int64_t E = (int64_t)el.size();
    egid[b].assign(E * B.nb, -1);
    epos3[b].assign(E * B.nb * 3, 0);
    B.vconn.assign(E * B.nv, 0);
    if (ex) {  // node numbers are the GIDs; basis b lives on the element's node b (shards order)
      const std::vector<int64_t>& cn = m.ex.blocks[b].conn;
      const int npe = m.ex.blocks[b].npe;
      for (int64_t i = 0; i < E; ++i) {
        for (int v = 0; v < B.nv; ++v) B.vconn[i * B.nv + v] = (int32_t)cn[i * npe + v];
        for (int bi = 0; bi < B.nb; ++bi) egid[b][i * B.nb + bi] = cn[i * npe + bi];
      }
      for (int64_t k = 0; k < E * B.nb; ++k) has[egid[b][k]] = 1;
      continue;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < E; ++i) {
      int64_t e = el[i];
      int64_t br = m.elem_brick[e];
      int64_t I = br % m.NX, J = (br / m.NX) % m.NY, K = br / (m.NX * m.NY);
      int sub = m.elem_sub[e];
      for (int v = 0; v < B.nv; ++v) {
        int bv = B.topo == TX_TOPO_HEX ? v : kTets[sub][v];
        B.vconn[i * B.nv + v] = (int32_t)L.gid(2 * (I + kVtx[bv][0]), 2 * (J + kVtx[bv][1]), 2 * (K + kVtx[bv][2]));
      }
      for (size_t g = 0; g < B.geom_dim.size(); ++g) {
        int bi = B.geom_basis[g];
        if (bi < 0) continue;
        int dim = B.geom_dim[g], c = B.geom_sub[g];
        int id = c;
        if (B.topo == TX_TOPO_TET && dim == 0) id = kTets[sub][c];
        if (B.topo == TX_TOPO_TET && dim == 1) id = kTetEdges[sub][c];
        if (B.topo == TX_TOPO_TET && dim >= 2) throw std::runtime_error("tet face/cell DOFs not provided");
        int o[3];
        brick_entity_offset(dim, dim == 3 ? 18 : id, o);
        int64_t a = 2 * I + o[0], bb = 2 * J + o[1], cc = 2 * K + o[2];
        egid[b][i * B.nb + bi] = L.gid(a, bb, cc);
        epos3[b][(i * B.nb + bi) * 3 + 0] = (int32_t)a;
        epos3[b][(i * B.nb + bi) * 3 + 1] = (int32_t)bb;
        epos3[b][(i * B.nb + bi) * 3 + 2] = (int32_t)cc;
      }
    }
    for (int64_t k = 0; k < E * B.nb; ++k) has[egid[b][k]] = 1;
  }
  // DOF GIDs: ascending entity GID, nf consecutive per entity
  std::vector<int64_t> first_gid(gid_space, -1);
  int64_t ng = 0;
  for (int64_t g = 0; g < gid_space; ++g)
    if (has[g]) { first_gid[g] = ng; ng += nf; }
  D.n_dofs = ng;
  if (ng >= (int64_t)INT32_MAX) throw std::invalid_argument("tx_dof_build: more than 2^31 DOFs");
  // first touch: blocks in order, elements in block order, entities in
  // geometric order
  std::vector<int32_t> ent_lid(gid_space, -1);
  D.ent_gid.clear(); D.ent_first_gid.clear(); D.ent_lattice.clear();
  for (int b = 0; b < m.nblocks; ++b) {
    BlockDofs& B = D.blocks[b];
    const int64_t E = (int64_t)m.block_elems[b].size();
    B.dconn.assign(E * B.nb, 0);
    for (int64_t i = 0; i < E; ++i)
      for (size_t g = 0; g < B.geom_dim.size(); ++g) {
        int bi = B.geom_basis[g];
        if (bi < 0) continue;
        int64_t G = egid[b][i * B.nb + bi];
        if (ent_lid[G] < 0) {
          ent_lid[G] = (int32_t)D.ent_gid.size();
          D.ent_gid.push_back(G);
          D.ent_first_gid.push_back(first_gid[G]);
          for (int d = 0; d < 3; ++d) D.ent_lattice.push_back(epos3[b][(i * B.nb + bi) * 3 + d]);
        }
        B.dconn[i * B.nb + bi] = ent_lid[G];
      }
  }
  D.n_entities = (int64_t)D.ent_gid.size();
  if (D.n_entities * nf != D.n_dofs) throw std::runtime_error("numbering failure: owned count mismatch");
  // HCURL edge signs: + when the local edge runs from the lower to the higher vertex GID
  for (int b = 0; b < m.nblocks; ++b) {
    BlockDofs& B = D.blocks[b];
    B.esign.clear();
    if (B.basis != TX_HCURL_I1) continue;
    const int64_t E = (int64_t)m.block_elems[b].size();
    B.esign.assign(E * 12, 1);
    for (int64_t i = 0; i < E; ++i)
      for (int k = 0; k < 12; ++k)
        B.esign[i * 12 + k] = B.vconn[i * 8 + kEdgeVtx[k][0]] < B.vconn[i * 8 + kEdgeVtx[k][1]] ? 1 : -1;
  }
  // entity graph: union of element cliques (rows/cols = entity LIDs)
  const int64_t NE = D.n_entities;
  std::vector<int64_t> cnt(NE + 1, 0);
  for (int b = 0; b < m.nblocks; ++b) {
    const BlockDofs& B = D.blocks[b];
    const int64_t E = (int64_t)m.block_elems[b].size();
    for (int64_t i = 0; i < E * B.nb; ++i) cnt[B.dconn[i] + 1] += B.nb;
  }
  for (int64_t r = 0; r < NE; ++r) cnt[r + 1] += cnt[r];
  std::vector<int32_t> raw(cnt[NE]);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  for (int b = 0; b < m.nblocks; ++b) {
    const BlockDofs& B = D.blocks[b];
    const int64_t E = (int64_t)m.block_elems[b].size();
    for (int64_t i = 0; i < E; ++i) {
      const int32_t* dc = &B.dconn[i * B.nb];
      for (int a = 0; a < B.nb; ++a) {
        int64_t p = fill[dc[a]];
        std::memcpy(&raw[p], dc, sizeof(int32_t) * B.nb);
        fill[dc[a]] = p + B.nb;
      }
    }
  }
  std::vector<int64_t> deg(NE, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t r = 0; r < NE; ++r) {
    int32_t* s = &raw[cnt[r]];
    int32_t* e = &raw[cnt[r + 1]];
    std::sort(s, e);
    deg[r] = std::unique(s, e) - s;
  }
  D.erowptr.assign(NE + 1, 0);
  for (int64_t r = 0; r < NE; ++r) D.erowptr[r + 1] = D.erowptr[r] + deg[r];
  D.ecol.assign(D.erowptr[NE], 0);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < NE; ++r) std::memcpy(&D.ecol[D.erowptr[r]], &raw[cnt[r]], sizeof(int32_t) * deg[r]);
  D.nnz = D.erowptr[NE] * (int64_t)nf * nf;
  // element-to-row map: position of entity b in the sorted row of entity a
  for (int b = 0; b < m.nblocks; ++b) {
    BlockDofs& B = D.blocks[b];
    const int64_t E = (int64_t)m.block_elems[b].size();
    B.epos.assign(E * B.nb * B.nb, 0);
    bool overflow = false;
#pragma omp parallel for schedule(static) reduction(|| : overflow)
    for (int64_t i = 0; i < E; ++i) {
      const int32_t* dc = &B.dconn[i * B.nb];
      for (int a = 0; a < B.nb; ++a) {
        const int32_t* rs = &D.ecol[D.erowptr[dc[a]]];
        const int32_t* re = &D.ecol[D.erowptr[dc[a] + 1]];
        for (int c = 0; c < B.nb; ++c) {
          int64_t p = std::lower_bound(rs, re, dc[c]) - rs;
          if (p > 255) overflow = true;
          B.epos[(i * B.nb + a) * B.nb + c] = (uint8_t)p;
        }
      }
    }
    if (overflow) throw std::runtime_error("tx_dof_build: entity row longer than 256 blocks");
    color_block(B, E, D.n_entities);
  }
}

// Greedy element colouring per block (first fit in element order): elements
// of one colour share no DOF entity, so a launch over one colour can scatter
// with plain read-modify-writes.  Lattice blocks give 8 colours (hex) or
// about 48 (tet split).
static void color_block(BlockDofs& B, int64_t E, int64_t n_entities) {
  std::vector<uint64_t> used(n_entities, 0);
  std::vector<int> color(E, 0);
  int ncolors = 0;
  for (int64_t i = 0; i < E; ++i) {
    uint64_t m = 0;
    for (int a = 0; a < B.nb; ++a) m |= used[B.dconn[i * B.nb + a]];
    if (~m == 0) throw std::runtime_error("element colouring needs more than 64 colours");
    int c = 0;
    while (m & (1ull << c)) ++c;
    color[i] = c;
    ncolors = std::max(ncolors, c + 1);
    for (int a = 0; a < B.nb; ++a) used[B.dconn[i * B.nb + a]] |= 1ull << c;
  }
  B.color_offsets.assign(ncolors + 1, 0);
  for (int64_t i = 0; i < E; ++i) B.color_offsets[color[i] + 1]++;
  for (int c = 0; c < ncolors; ++c) B.color_offsets[c + 1] += B.color_offsets[c];
  std::vector<int64_t> pos(B.color_offsets.begin(), B.color_offsets.end() - 1);
  B.color_perm.assign(E, 0);
  for (int64_t i = 0; i < E; ++i) B.color_perm[pos[color[i]]++] = (int32_t)i;
}

std::vector<int64_t> workset_bounds(int64_t n_elem, int64_t min_size, int64_t max_size, uint64_t seed) {
  std::vector<int64_t> b{0};
  if (min_size < 1) min_size = 1;
  if (max_size < min_size) max_size = min_size;
  uint64_t st = seed;
  while (b.back() < n_elem) {
    st = splitmix(st);
    int64_t sz = min_size + (int64_t)(st % (uint64_t)(max_size - min_size + 1));
    b.push_back(std::min(n_elem, b.back() + sz));
  }
  return b;
}

void dof_owned_gids(const Dofs& D, int64_t* out) {
  for (int64_t e = 0; e < D.n_entities; ++e)
    for (int f = 0; f < D.nf; ++f) out[e * D.nf + f] = D.ent_first_gid[e] + f;
}

int dof_block_gid_count(const Dofs& D, int block) {
  const BlockDofs& B = D.blocks[block];
  int n = 0;
  for (int bi : B.geom_basis) n += bi >= 0 ? D.nf : 0;
  return n;
}

// element GID / LID vectors in the reference's geometric order:
// DOF entities in (dim, subcell) order, fields interleaved per entity
template <typename T, typename F>
static void element_vectors(const Mesh& m, const Dofs& D, int block, T* out, F map) {
  const BlockDofs& B = D.blocks[block];
  const int64_t E = (int64_t)m.block_elems[block].size();
  const int n = dof_block_gid_count(D, block);
  for (int64_t i = 0; i < E; ++i) {
    int k = 0;
    for (size_t g = 0; g < B.geom_dim.size(); ++g) {
      int bi = B.geom_basis[g];
      if (bi < 0) continue;
      int32_t ent = B.dconn[i * B.nb + bi];
      for (int f = 0; f < D.nf; ++f) out[i * n + k++] = map(ent, f);
    }
  }
}

void dof_element_gids(const Mesh& m, const Dofs& D, int block, int64_t* out) {
  element_vectors(m, D, block, out, [&](int32_t ent, int f) { return (int64_t)(D.ent_first_gid[ent] + f); });
}
void dof_element_lids(const Mesh& m, const Dofs& D, int block, int32_t* out) {
  element_vectors(m, D, block, out, [&](int32_t ent, int f) { return (int32_t)(ent * D.nf + f); });
}

int dof_field_offsets(const Dofs& D, int block, int field, int32_t* out) {
  const BlockDofs& B = D.blocks[block];
  for (int b = 0; b < B.nb; ++b) out[b] = B.basis_pos[b] * D.nf + field;
  return B.nb;
}

std::vector<int32_t> dirichlet_dofs(const Dofs& D, const Mesh& m, uint32_t side_mask, uint32_t field_mask) {
  if (m.is_explicit) throw std::invalid_argument("box sides are not defined on an explicit mesh; use a node set");
  std::vector<int32_t> out;
  const int64_t lim[3] = {2 * m.NX, 2 * m.NY, 2 * m.NZ};
  for (int64_t e = 0; e < D.n_entities; ++e) {
    const int32_t* p = &D.ent_lattice[3 * e];
    bool on = false;
    for (int s = 0; s < 6 && !on; ++s)
      if (side_mask & (1u << s)) on = p[s / 2] == ((s & 1) ? lim[s / 2] : 0);
    if (!on) continue;
    for (int f = 0; f < D.nf; ++f)
      if (field_mask & (1u << f)) out.push_back((int32_t)(e * D.nf + f));
  }
  return out;  // ascending: entity LIDs ascending, fields ascending
}

}  // namespace tx
