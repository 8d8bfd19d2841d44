// tx_exodus.cpp -- Exodus II mesh input (STK_ExodusReaderFactory's role,
// adapters-stk/src/Panzer_STK_ExodusReaderFactory.cpp), read from the NetCDF
// classic container (CDF-1, CDF-2 and CDF-5; HDF5-based NetCDF-4 files are
// refused) without the NetCDF or Exodus libraries.
//
// NetCDF classic, as published by Unidata: big-endian; a header of magic
// "CDF" + version, the record count, then tagged lists of dimensions (tag
// 0x0A), global attributes (0x0C) and variables (0x0B).  A variable is its
// name, dimension ids, attributes, type, size and the file offset of its
// data; names and attribute values are padded to 4 bytes; counts are 4 bytes
// (8 in CDF-5) and offsets 4 bytes (CDF-1) or 8 (CDF-2/5).  Mesh variables
// are fixed-size, so record variables are not read.
//
// Exodus II names used: dimensions num_dim, num_nodes, num_el_blk,
// num_el_in_blk<k>, num_nod_per_el<k>, num_side_sets, num_side_ss<k>,
// num_node_sets, num_nod_ns<k>; variables coordx/coordy/coordz (or coord),
// connect<k> (attribute elem_type), eb_prop1, eb_names, elem_ss<k>,
// side_ss<k>, ss_prop1, ss_names, node_ns<k>, ns_prop1, ns_names and the
// optional node_num_map.  Element and node numbers in the file are 1-based;
// side ordinals are 1-based in the shards face order.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "tx_internal.h"

namespace tx {
namespace {

enum NcType { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6, NC_UBYTE = 7,
              NC_USHORT = 8, NC_UINT = 9, NC_INT64 = 10, NC_UINT64 = 11 };

int type_size(int t) {
  switch (t) {
    case NC_BYTE: case NC_CHAR: case NC_UBYTE: return 1;
    case NC_SHORT: case NC_USHORT: return 2;
    case NC_INT: case NC_FLOAT: case NC_UINT: return 4;
    case NC_DOUBLE: case NC_INT64: case NC_UINT64: return 8;
    default: throw std::runtime_error("NetCDF: unknown type " + std::to_string(t));
  }
}

struct NcVar {
  std::string name;
  std::vector<int> dims;
  int type = 0;
  uint64_t begin = 0;
  std::map<std::string, std::string> text;  // character attributes
};

class NcFile {
 public:
  explicit NcFile(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::invalid_argument("cannot open " + path);
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf_.resize(n > 0 ? (size_t)n : 0);
    const size_t got = buf_.empty() ? 0 : std::fread(buf_.data(), 1, buf_.size(), f);
    std::fclose(f);
    if (got != buf_.size()) throw std::runtime_error("short read of " + path);
    parse();
  }

  int version() const { return version_; }
  bool has_dim(const std::string& n) const { return dim_index(n) >= 0; }
  int64_t dim(const std::string& n) const {
    const int i = dim_index(n);
    if (i < 0) throw std::invalid_argument("Exodus: missing dimension " + n);
    return dims_[i].second;
  }
  int64_t dim_or(const std::string& n, int64_t v) const { return has_dim(n) ? dim(n) : v; }
  const NcVar* var(const std::string& n) const {
    for (const NcVar& v : vars_)
      if (v.name == n) return &v;
    return nullptr;
  }
  int64_t count(const NcVar& v) const {
    int64_t c = 1;
    for (int d : v.dims) c *= dims_[d].second;
    return c;
  }
  // all values of a numeric variable, converted
  template <typename T>
  std::vector<T> read(const std::string& n) const {
    const NcVar* v = var(n);
    if (!v) throw std::invalid_argument("Exodus: missing variable " + n);
    const int64_t c = count(*v);
    const int ts = type_size(v->type);
    if (v->begin + (uint64_t)c * ts > buf_.size()) throw std::runtime_error("NetCDF: variable " + n + " past end");
    std::vector<T> out((size_t)c);
    const uint8_t* p = buf_.data() + v->begin;
    for (int64_t i = 0; i < c; ++i, p += ts) {
      switch (v->type) {
        case NC_BYTE: out[i] = (T)(int8_t)p[0]; break;
        case NC_UBYTE: out[i] = (T)p[0]; break;
        case NC_SHORT: out[i] = (T)(int16_t)be(p, 2); break;
        case NC_USHORT: out[i] = (T)(uint16_t)be(p, 2); break;
        case NC_INT: out[i] = (T)(int32_t)be(p, 4); break;
        case NC_UINT: out[i] = (T)(uint32_t)be(p, 4); break;
        case NC_INT64: out[i] = (T)(int64_t)be(p, 8); break;
        case NC_UINT64: out[i] = (T)be(p, 8); break;
        case NC_FLOAT: { uint32_t u = (uint32_t)be(p, 4); float x; std::memcpy(&x, &u, 4); out[i] = (T)x; break; }
        case NC_DOUBLE: { uint64_t u = be(p, 8); double x; std::memcpy(&x, &u, 8); out[i] = (T)x; break; }
        default: throw std::runtime_error("NetCDF: variable " + n + " is not numeric");
      }
    }
    return out;
  }
  // rows of a 2-D character variable (names), trailing NULs and blanks dropped
  std::vector<std::string> names(const std::string& n, int64_t rows) const {
    std::vector<std::string> out(rows);
    const NcVar* v = var(n);
    if (!v || v->type != NC_CHAR || v->dims.size() != 2) return out;
    const int64_t len = dims_[v->dims[1]].second;
    const int64_t r = std::min<int64_t>(rows, dims_[v->dims[0]].second);
    if (v->begin + (uint64_t)(r * len) > buf_.size()) return out;
    for (int64_t i = 0; i < r; ++i) {
      const char* s = (const char*)buf_.data() + v->begin + i * len;
      std::string t(s, strnlen(s, (size_t)len));
      while (!t.empty() && t.back() == ' ') t.pop_back();
      out[i] = t;
    }
    return out;
  }

 private:
  std::vector<uint8_t> buf_;
  size_t pos_ = 0;
  int version_ = 0;
  std::vector<std::pair<std::string, int64_t>> dims_;
  std::vector<NcVar> vars_;

  static uint64_t be(const uint8_t* p, int n) {
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v = (v << 8) | p[i];
    return v;
  }
  uint64_t take(int n) {
    if (pos_ + n > buf_.size()) throw std::runtime_error("NetCDF: header past end of file");
    const uint64_t v = be(buf_.data() + pos_, n);
    pos_ += n;
    return v;
  }
  int64_t count_field() { return (int64_t)take(version_ == 5 ? 8 : 4); }
  std::string name() {
    const int64_t n = count_field();
    if (n < 0 || pos_ + (size_t)n > buf_.size()) throw std::runtime_error("NetCDF: bad name");
    std::string s((const char*)buf_.data() + pos_, (size_t)n);
    pos_ += (size_t)((n + 3) / 4 * 4);
    return s;
  }
  void attributes(std::map<std::string, std::string>* text) {
    const uint64_t tag = take(4);
    const int64_t n = count_field();
    if (tag == 0 && n == 0) return;
    if (tag != 0x0C) throw std::runtime_error("NetCDF: expected an attribute list");
    for (int64_t i = 0; i < n; ++i) {
      const std::string an = name();
      const int t = (int)take(4);
      const int64_t m = count_field();
      const size_t bytes = (size_t)(m * type_size(t));
      if (pos_ + bytes > buf_.size()) throw std::runtime_error("NetCDF: attribute past end");
      if (text && t == NC_CHAR) {
        const char* s = (const char*)buf_.data() + pos_;
        (*text)[an] = std::string(s, strnlen(s, bytes));
      }
      pos_ += (bytes + 3) / 4 * 4;
    }
  }
  void parse() {
    if (buf_.size() >= 4 && buf_[0] == 0x89 && buf_[1] == 'H' && buf_[2] == 'D' && buf_[3] == 'F')
      throw std::invalid_argument("Exodus: HDF5-based (NetCDF-4) files are not read; convert to NetCDF classic");
    if (buf_.size() < 8 || buf_[0] != 'C' || buf_[1] != 'D' || buf_[2] != 'F')
      throw std::invalid_argument("Exodus: not a NetCDF classic file");
    version_ = buf_[3];
    if (version_ != 1 && version_ != 2 && version_ != 5) throw std::invalid_argument("NetCDF: unknown version");
    pos_ = 4;
    count_field();  // number of records
    uint64_t tag = take(4);
    int64_t n = count_field();
    if (!(tag == 0 && n == 0)) {
      if (tag != 0x0A) throw std::runtime_error("NetCDF: expected a dimension list");
      for (int64_t i = 0; i < n; ++i) {
        std::string dn = name();
        dims_.emplace_back(dn, count_field());
      }
    }
    attributes(nullptr);  // global attributes
    tag = take(4);
    n = count_field();
    if (tag == 0 && n == 0) return;
    if (tag != 0x0B) throw std::runtime_error("NetCDF: expected a variable list");
    for (int64_t i = 0; i < n; ++i) {
      NcVar v;
      v.name = name();
      const int64_t nd = count_field();
      for (int64_t k = 0; k < nd; ++k) {
        const int64_t d = count_field();
        if (d < 0 || d >= (int64_t)dims_.size()) throw std::runtime_error("NetCDF: bad dimension id");
        v.dims.push_back((int)d);
      }
      attributes(&v.text);
      v.type = (int)take(4);
      count_field();  // vsize
      v.begin = take(version_ == 1 ? 4 : 8);
      vars_.push_back(v);
    }
  }
  int dim_index(const std::string& n) const {
    for (size_t i = 0; i < dims_.size(); ++i)
      if (dims_[i].first == n) return (int)i;
    return -1;
  }
};

std::string upper(std::string s) {
  for (char& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

}  // namespace

ExodusSummary exodus_summary(const std::string& path) {
  NcFile f(path);
  ExodusSummary s;
  s.version = f.version();
  s.dim = f.dim("num_dim");
  s.n_nodes = f.dim("num_nodes");
  s.n_elem = f.dim_or("num_elem", 0);
  s.n_blocks = f.dim_or("num_el_blk", 0);
  s.n_side_sets = f.dim_or("num_side_sets", 0);
  s.n_node_sets = f.dim_or("num_node_sets", 0);
  return s;
}

// Reads a 3-D Exodus mesh into an explicit mesh description.  linear: keep
// the vertex nodes of HEX20/HEX27/TETRA10 elements (the quadratic-to-linear
// conversion of Panzer_STK_QuadraticToLinearMeshFactory).  Node numbers
// follow node_num_map ascending when the file has one.
ExplicitMesh read_exodus(const std::string& path, bool linear) {
  NcFile f(path);
  ExplicitMesh M;
  if (f.dim("num_dim") != 3) throw std::invalid_argument("Exodus: only 3-D meshes are built");
  const int64_t nn = f.dim("num_nodes");
  std::vector<double> x, y, z;
  if (f.var("coordx")) {
    x = f.read<double>("coordx"); y = f.read<double>("coordy"); z = f.read<double>("coordz");
  } else {
    std::vector<double> c = f.read<double>("coord");
    x.assign(c.begin(), c.begin() + nn); y.assign(c.begin() + nn, c.begin() + 2 * nn);
    z.assign(c.begin() + 2 * nn, c.begin() + 3 * nn);
  }
  // node order: ascending global id (node_num_map) or file order
  std::vector<int64_t> rank(nn);
  std::iota(rank.begin(), rank.end(), 0);
  if (f.var("node_num_map")) {
    std::vector<int64_t> gid = f.read<int64_t>("node_num_map");
    std::vector<int64_t> order(nn);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return gid[a] < gid[b]; });
    for (int64_t r = 0; r < nn; ++r) rank[order[r]] = r;
  }
  M.n_nodes = nn;
  M.coords.assign(3 * nn, 0.0);
  for (int64_t i = 0; i < nn; ++i) {
    M.coords[3 * rank[i]] = x[i]; M.coords[3 * rank[i] + 1] = y[i]; M.coords[3 * rank[i] + 2] = z[i];
  }
  const int64_t nblk = f.dim_or("num_el_blk", 0);
  std::vector<int64_t> ids = nblk > 0 && f.var("eb_prop1") ? f.read<int64_t>("eb_prop1") : std::vector<int64_t>();
  std::vector<std::string> bnames = f.names("eb_names", nblk);
  for (int64_t k = 1; k <= nblk; ++k) {
    ExplicitBlock B;
    B.id = k - 1 < (int64_t)ids.size() ? ids[k - 1] : k;
    B.name = bnames[k - 1].empty() ? "block_" + std::to_string(B.id) : bnames[k - 1];
    const int64_t ne = f.dim_or("num_el_in_blk" + std::to_string(k), 0);
    const std::string cv = "connect" + std::to_string(k);
    const NcVar* v = f.var(cv);
    std::string et = v && v->text.count("elem_type") ? upper(v->text.at("elem_type")) : "";
    const int64_t npe = f.dim_or("num_nod_per_el" + std::to_string(k), 0);
    int nv = 0;
    if (et.rfind("HEX", 0) == 0) { B.topology = TX_TOPO_HEX; nv = 8; }
    else if (et.rfind("TET", 0) == 0) { B.topology = TX_TOPO_TET; nv = 4; }
    else if (ne > 0) throw std::invalid_argument("Exodus: element type '" + et + "' is not provided (hex or tet)");
    else { B.topology = TX_TOPO_HEX; nv = 8; }
    if (ne > 0 && npe < nv) throw std::invalid_argument("Exodus: too few nodes per element for " + et);
    // kept nodes: the vertices (linear elements, or linear=true), or every node of HEX27 / TETRA10
    const int quad = B.topology == TX_TOPO_HEX ? 27 : 10;
    int keep = nv;
    if (ne > 0 && npe != nv) {
      if (!linear && npe != quad)
        throw std::invalid_argument("Exodus: " + et + " elements are read with linear=true (their vertex nodes)");
      keep = linear ? nv : quad;
    }
    B.npe = keep;
    B.conn.reserve((size_t)(ne * keep));
    if (ne > 0) {
      std::vector<int64_t> c = f.read<int64_t>(cv);
      for (int64_t e = 0; e < ne; ++e)
        for (int a = 0; a < keep; ++a) {
          const int64_t node = c[e * npe + a] - 1;
          if (node < 0 || node >= nn) throw std::invalid_argument("Exodus: node number out of range in " + cv);
          B.conn.push_back(rank[node]);
        }
    }
    B.n_elem = ne;
    M.blocks.push_back(std::move(B));
  }
  const int64_t nss = f.dim_or("num_side_sets", 0);
  std::vector<int64_t> ssid = nss > 0 && f.var("ss_prop1") ? f.read<int64_t>("ss_prop1") : std::vector<int64_t>();
  std::vector<std::string> ssn = f.names("ss_names", nss);
  for (int64_t k = 1; k <= nss; ++k) {
    ExplicitSet S;
    S.id = k - 1 < (int64_t)ssid.size() ? ssid[k - 1] : k;
    S.name = ssn[k - 1].empty() ? "surface_" + std::to_string(S.id) : ssn[k - 1];
    if (f.dim_or("num_side_ss" + std::to_string(k), 0) > 0) {
      std::vector<int64_t> el = f.read<int64_t>("elem_ss" + std::to_string(k));
      std::vector<int64_t> sd = f.read<int64_t>("side_ss" + std::to_string(k));
      for (size_t i = 0; i < el.size(); ++i) { S.entries.push_back(el[i] - 1); S.entries.push_back(sd[i] - 1); }
    }
    M.side_sets.push_back(std::move(S));
  }
  const int64_t nns = f.dim_or("num_node_sets", 0);
  std::vector<int64_t> nsid = nns > 0 && f.var("ns_prop1") ? f.read<int64_t>("ns_prop1") : std::vector<int64_t>();
  std::vector<std::string> nsn = f.names("ns_names", nns);
  for (int64_t k = 1; k <= nns; ++k) {
    ExplicitSet S;
    S.id = k - 1 < (int64_t)nsid.size() ? nsid[k - 1] : k;
    S.name = nsn[k - 1].empty() ? "nodelist_" + std::to_string(S.id) : nsn[k - 1];
    if (f.dim_or("num_nod_ns" + std::to_string(k), 0) > 0)
      for (int64_t node : f.read<int64_t>("node_ns" + std::to_string(k))) {
        if (node < 1 || node > nn) throw std::invalid_argument("Exodus: node set node out of range");
        S.entries.push_back(rank[node - 1]);
      }
    M.node_sets.push_back(std::move(S));
  }
  return M;
}

}  // namespace tx
