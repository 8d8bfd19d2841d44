// tx_internal.h -- shared host/device declarations of libtianxin_gb300.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tianxin_gb300.h"

namespace tx {

// Maximum sizes of the element families the kernels are instantiated for.
constexpr int kMaxNB = 27;   // basis functions per element (hex27)
constexpr int kMaxNQ = 27;   // cubature points per element
constexpr int kMaxNV = 8;    // geometric vertices per element

// Reference element of one block: cubature and basis tables, FP64.
//   w[q]; geo_val[q][v]; geo_grad[q][v][3]; val[q][b] (HGRAD) or
//   val[q][b][3] (HCURL); grad[q][b][3] (HGRAD gradient / HCURL curl).
struct RefTables {
  int topo = 0, basis = 0, degree = 0;
  int nq = 0, nb = 0, nv = 0;
  bool hcurl = false;
  std::vector<double> xi, w, geo_val, geo_grad, val, grad;
  // pack into one contiguous array: [w | geo_val | geo_grad | val | grad]
  std::vector<double> packed() const;
};

RefTables make_ref_tables(int topo, int basis, int degree);
// Basis and geometry tables at n given reference points (weights zero).
RefTables tables_at(int topo, int basis, const double* xi, int n);
int default_degree(int topo, int basis);

// Side cubature tables of a block's reference element, one group per local
// side ordinal s (6 hex faces, 4 tet faces), each [w | geo_grad | val | tu |
// tv]: weights of the reference side rule, geometry-basis gradients and
// basis values at the side points mapped into the element, and the two
// constant tangents of the side's parametrisation.
struct SideTables {
  int nsides = 0, nqf = 0, nb = 0, nv = 0, stride = 0;
  std::vector<double> packed;  // [nsides][stride]
};
SideTables make_side_tables(int topo, int basis, int degree);

// Device view of one block, passed by value to kernels.
struct BlockView {
  int topo, basis, nq, nb, nv;
  int64_t n_elem;
  const int32_t* vconn;   // [E][nv]  vertex (node GID) per geometric vertex
  const int32_t* dconn;   // [E][nb]  entity LID of the entity carrying basis b
  const uint8_t* epos;    // [E][nb][nb] block position of entity b in row of entity a
  const int8_t* esign;    // [E][nb]  HCURL edge signs (nullptr otherwise)
  const double* ref;      // packed RefTables
  const float* ref32 = nullptr;  // the same tables in FP32 (read from global memory by the hex27 kernels)
};

struct Handle;  // defined in tx_api.cu

// ----------------------------------------------------------------- setup
// An explicit (unstructured) mesh: nodes, hex8 / tet4 blocks of node
// connectivity (0-based node numbers, Exodus/shards vertex order), side sets
// of (element, side) pairs (element numbered over the whole mesh, blocks in
// order; 0-based shards side ordinal) and node sets.
struct ExplicitBlock {
  int topology = 0;
  int npe = 0;                // nodes an element: the vertices (8 / 4) or quadratic (27 / 10)
  int64_t n_elem = 0, id = 0;
  std::string name;
  std::vector<int64_t> conn;  // [n_elem][npe], shards node order
};
struct ExplicitSet {
  int64_t id = 0;
  std::string name;
  std::vector<int64_t> entries;  // side sets: (element, side) pairs; node sets: nodes
};
struct ExplicitMesh {
  int64_t n_nodes = 0;
  std::vector<double> coords;  // [n_nodes][3]
  std::vector<ExplicitBlock> blocks;
  std::vector<ExplicitSet> side_sets, node_sets;
};
struct ExodusSummary {
  int version = 0;
  int64_t dim = 0, n_nodes = 0, n_elem = 0, n_blocks = 0, n_side_sets = 0, n_node_sets = 0;
};
// tx_exodus.cpp
ExodusSummary exodus_summary(const std::string& path);
ExplicitMesh read_exodus(const std::string& path, bool linear);

// Host-side mesh + numbering state (built by tx_setup.cpp).
struct Mesh {
  tx_mesh_desc desc{};
  int64_t NX = 0, NY = 0, NZ = 0;
  int nblocks = 0;
  int64_t n_nodes = 0, n_hex_edges = 0, n_hex_faces = 0, n_bricks = 0;
  int64_t n_elements = 0;
  std::vector<int64_t> elem_brick;        // element -> brick
  std::vector<int8_t> elem_sub;           // element -> sub-element (tet)
  std::vector<std::vector<int64_t>> block_elems;
  std::vector<double> coords;             // node GID order, xyz
  // explicit meshes: node numbers are the vertex GIDs; no lattice
  bool is_explicit = false;
  ExplicitMesh ex;
  std::vector<int64_t> block_first;       // first mesh element of each block
};

struct BlockDofs {
  int topo = 0, basis = 0, degree = 0, nb = 0, nv = 0;
  RefTables ref;
  std::vector<int32_t> vconn, dconn;      // [E][nv], [E][nb]
  std::vector<uint8_t> epos;              // [E][nb][nb]
  std::vector<int8_t> esign;              // [E][nb] (HCURL)
  std::vector<int> geom_dim, geom_sub;    // geometric pattern (dim, subcell) in order
  std::vector<int> geom_basis;            // basis index on that sub-cell, -1 none
  std::vector<int> basis_pos;             // basis b -> position among DOF entities
  // greedy colouring: elements of one colour share no DOF entity
  std::vector<int32_t> color_perm;        // block elements ordered by colour
  std::vector<int64_t> color_offsets;     // [ncolors + 1]
};

struct Dofs {
  tx_equation_set_desc eq{};
  int nf = 0;
  int64_t n_entities = 0;                 // DOF-carrying entities
  int64_t n_dofs = 0;
  std::vector<BlockDofs> blocks;
  std::vector<int64_t> ent_gid;           // entity LID -> entity GID (mesh entity id)
  std::vector<int64_t> ent_first_gid;     // entity LID -> first DOF GID
  std::vector<int32_t> ent_lattice;       // entity LID -> doubled lattice position (3)
  std::vector<int64_t> erowptr;           // entity graph
  std::vector<int32_t> ecol;
  int64_t nnz = 0;
};

void build_mesh(Mesh& m, const tx_mesh_desc& d);
void build_mesh_explicit(Mesh& m, ExplicitMesh&& x);
// Vertex node numbers of a block's elements [E][nv] (shards order); returns nv.
int element_vertices(const Mesh& m, int block, int64_t* out);
void build_dofs(const Mesh& m, Dofs& D, const tx_equation_set_desc& q);
// owned GIDs (LID order), element GIDs/LIDs of a block (reference geometric order)
void dof_owned_gids(const Dofs& D, int64_t* out);
void dof_element_gids(const Mesh& m, const Dofs& D, int block, int64_t* out);
void dof_element_lids(const Mesh& m, const Dofs& D, int block, int32_t* out);
int dof_block_gid_count(const Dofs& D, int block);
int dof_field_offsets(const Dofs& D, int block, int field, int32_t* out);
std::vector<int32_t> dirichlet_dofs(const Dofs& D, const Mesh& m, uint32_t side_mask, uint32_t field_mask);
// Side workset of a block on the box sides in side_mask: (block element << 3
// | local side ordinal) for every local side lying on one of the sides, in
// block element order, then side ordinal.
std::vector<int64_t> side_workset(const Mesh& m, int block, uint32_t side_mask);
// The first element (blocks in order, block elements in order) whose inverse
// geometry map puts p inside the reference cell (tolerance 1e-10): its block,
// block-local index and reference coordinates.
bool locate_point(const Mesh& m, const Dofs& D, const double p[3], int& block, int64_t& elem, double xi[3]);
// Side workset of a block from side set k of an explicit mesh (same encoding,
// ascending).
std::vector<int64_t> side_set_workset(const Mesh& m, int block, int side_set);
// DOF LIDs of the fields in field_mask at the nodes of node set k of an
// explicit mesh (ascending; nodes without DOFs are skipped).
std::vector<int32_t> node_set_dofs(const Dofs& D, const Mesh& m, int node_set, uint32_t field_mask);
// Worksets of a block: consecutive element ranges with sizes drawn uniformly
// in [min_size, max_size] from a seeded generator (min == max: even split).
std::vector<int64_t> workset_bounds(int64_t n_elem, int64_t min_size, int64_t max_size, uint64_t seed);

}  // namespace tx
