// tx_blocked.cu -- the blocked linear-object layout of
// BlockedTpetraLinearObjFactory (disc-fe/src/lof/Panzer_BlockedTpetraLinearObjFactory_impl.hpp):
// the fields are grouped into field blocks, block i numbers its DOFs
// nb_i * entity + k (k = the field's place in its block, entities in the
// interleaved numbering's first-touch order), and the operator is the block
// matrix [A_ij] whose block (i, j) holds, in row (entity r, field k), the
// nb_j columns nb_j * m + l of every neighbour entity m of r in ascending
// order: the entity graph expanded by nb_i x nb_j, as the interleaved graph is
// the entity graph expanded by nf x nf.  Because of that the blocked objects
// are an index permutation of the interleaved ones; these kernels move values
// between the two layouts and expand the block graphs.
#include "tx_device.cuh"

namespace tx {
namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int per_block, int64_t cap = 152 * 32) {
  int64_t b = (n + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

// row (entity r, field k) of block (i, j) starts at bi*bj*erp[r] + k*bj*deg(r)
__global__ void k_block_rowptr(const int64_t* __restrict__ erp, int64_t n_ent, int bi, int bj,
                               int64_t* __restrict__ rp) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_ent; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = erp[r], deg = erp[r + 1] - b;
    for (int k = 0; k < bi; ++k) rp[bi * r + k] = (int64_t)bi * bj * b + (int64_t)k * bj * deg;
    if (r == n_ent - 1) rp[bi * n_ent] = (int64_t)bi * bj * erp[n_ent];
  }
}

// one warp per entity row; lanes write consecutive column indices
__global__ void k_block_colind(const int64_t* __restrict__ erp, const int32_t* __restrict__ ecol, int64_t n_ent,
                               int bi, int bj, const int64_t* __restrict__ rp, int32_t* __restrict__ col) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_ent; r += nwarps) {
    const int64_t b = erp[r], len = (erp[r + 1] - b) * bj;
    for (int k = 0; k < bi; ++k) {
      int32_t* out = col + rp[bi * r + k];
      for (int64_t t = lane; t < len; t += 32) out[t] = bj * ecol[b + t / bj] + (int32_t)(t % bj);
    }
  }
}

// interleaved DOF g = nf*e + f  <->  block vector fblock[f] at bnf * e + fpos[f]
template <bool SPLIT>
__global__ void k_block_vector(int64_t n_ent, BlockedMap M, const double* __restrict__ src, BlockPtrs blocks,
                               double* __restrict__ dst) {
  const int64_t n = n_ent * M.nf;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = g / M.nf;
    const int f = (int)(g - e * M.nf);
    const int bk = M.fblock[f];
    const int64_t at = (int64_t)M.bnf[bk] * e + M.fpos[f];
    if (SPLIT) blocks.p[bk][at] = src[g];
    else dst[g] = blocks.p[bk][at];
  }
}

// Interleaved CRS values -> block CRS values: one warp per entity row r; the
// interleaved row (r, c) holds nf*deg entries (neighbour j, field d) in
// order, which go to block (fblock[c], fblock[d]) at row (r, fpos[c]),
// column position bnf_j * j + fpos[d].  Null block pointers (excluded pairs)
// are skipped.
__global__ void k_block_split_matrix(const int64_t* __restrict__ erp, int64_t n_ent, BlockedMap M,
                                     const double* __restrict__ vals, BlockPtrs blk) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int nf = M.nf, nb = M.nb;
  for (int64_t r = warp; r < n_ent; r += nwarps) {
    const int64_t b = erp[r], deg = erp[r + 1] - b;
    for (int c = 0; c < nf; ++c) {
      const int bi = M.fblock[c], ni = M.bnf[bi];
      const double* src = vals + (int64_t)nf * nf * b + (int64_t)c * nf * deg;
      for (int64_t t = lane; t < nf * deg; t += 32) {
        const int64_t j = t / nf;
        const int d = (int)(t - j * nf);
        const int bj = M.fblock[d], nj = M.bnf[bj];
        double* out = blk.p[bi * nb + bj];
        if (!out) continue;
        const int64_t row0 = (int64_t)ni * nj * b + (int64_t)M.fpos[c] * nj * deg;
        out[row0 + (int64_t)nj * j + M.fpos[d]] = src[t];
      }
    }
  }
}

}  // namespace

cudaError_t launch_block_graph(const int64_t* erp, const int32_t* ecol, int64_t n_ent, int bi, int bj, int64_t* rp,
                               int32_t* col, cudaStream_t s) {
  if (n_ent <= 0) return cudaSuccess;
  k_block_rowptr<<<grid_for(n_ent, kThreads), kThreads, 0, s>>>(erp, n_ent, bi, bj, rp);
  k_block_colind<<<grid_for(n_ent, kThreads / 32), kThreads, 0, s>>>(erp, ecol, n_ent, bi, bj, rp, col);
  return cudaGetLastError();
}

cudaError_t launch_block_vector(int64_t n_ent, const BlockedMap& M, const double* src, BlockPtrs blocks, double* dst,
                                bool split, cudaStream_t s) {
  if (n_ent <= 0) return cudaSuccess;
  const unsigned g = grid_for(n_ent * M.nf, kThreads);
  if (split) k_block_vector<true><<<g, kThreads, 0, s>>>(n_ent, M, src, blocks, dst);
  else k_block_vector<false><<<g, kThreads, 0, s>>>(n_ent, M, src, blocks, dst);
  return cudaGetLastError();
}

cudaError_t launch_block_split_matrix(const int64_t* erp, int64_t n_ent, const BlockedMap& M, const double* vals,
                                      BlockPtrs blk, cudaStream_t s) {
  if (n_ent <= 0) return cudaSuccess;
  k_block_split_matrix<<<grid_for(n_ent, kThreads / 32), kThreads, 0, s>>>(erp, n_ent, M, vals, blk);
  return cudaGetLastError();
}

}  // namespace tx
