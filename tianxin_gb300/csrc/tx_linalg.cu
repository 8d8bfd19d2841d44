// tx_linalg.cu -- Tpetra-layout graph expansion, Dirichlet rows, CRS SpMV
// and the FP64-refined FP32 Jacobi-CG used for the Newton-Krylov solve.
//
//   graph expansion   the DOF-level CRS of TpetraLinearObjFactory::
//                     buildGhostedGraph (disc-fe/src/lof/Panzer_TpetraLinear
//                     ObjFactory_impl.hpp:559-651) from the entity graph: row
//                     (entity r, field c) holds, for every neighbour entity m
//                     in ascending LID, the nf columns nf*m .. nf*m+nf-1
//   Dirichlet         TpetraLinearObjContainer::applyDirichletBoundaryCondition
//                     (disc-fe/src/lof/Panzer_TpetraLinearObjContainer.hpp:
//                     228-238, 306-318): f[d] = x[d] - g, row d = e_d
//   SpMV              Tpetra::CrsMatrix::apply (y = alpha A x + beta y)
//   CG + refinement   Belos' role in adapters-stk/example/PoissonExample/
//                     main.cpp:402-419, re-designed: FP32 Jacobi-PCG inner
//                     solve on an FP32 copy of A with symmetric Dirichlet
//                     elimination, FP64 outer residual and update.
#include <cmath>
#include <cstdio>
#include <string>

#include "tx_device.cuh"
#include "tx_numeric.cuh"

namespace tx {
namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int per_block, int64_t cap = 152 * 32) {
  int64_t b = (n + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

__global__ void k_expand_rowptr(const int64_t* __restrict__ erp, int64_t n_ent, int nf, int64_t* __restrict__ rp) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_ent; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = erp[r], deg = erp[r + 1] - b;
    for (int c = 0; c < nf; ++c) rp[nf * r + c] = (int64_t)nf * nf * b + (int64_t)c * nf * deg;
    if (r == n_ent - 1) rp[nf * n_ent] = (int64_t)nf * nf * erp[n_ent];
  }
}

// one warp per entity row; lanes write consecutive column indices
__global__ void k_expand_colind(const int64_t* __restrict__ erp, const int32_t* __restrict__ ecol, int64_t n_ent,
                                int nf, const int64_t* __restrict__ rp, int32_t* __restrict__ col) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n_ent; r += nwarps) {
    const int64_t b = erp[r], deg = erp[r + 1] - b;
    const int64_t len = deg * nf;
    for (int c = 0; c < nf; ++c) {
      int32_t* out = col + rp[nf * r + c];
      for (int64_t k = lane; k < len; k += 32) out[k] = nf * ecol[b + k / nf] + (int32_t)(k % nf);
    }
  }
}

// position of entity r in the sorted entity row of m (the pattern is
// symmetric: r is in m's row when m is in r's)
__device__ __forceinline__ int64_t entity_pos(const int64_t* __restrict__ erp, const int32_t* __restrict__ ecol,
                                              int64_t m, int32_t r) {
  int64_t lo = erp[m], hi = erp[m + 1];
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (ecol[mid] < r) lo = mid + 1; else hi = mid;
  }
  return lo - erp[m];
}

// one warp per Dirichlet DOF d = nf*r + c: zero row d, put 1 on the
// diagonal, whose block position is that of entity r in its own sorted
// entity row.  Without a residual (f == NULL) the columns go too, as the
// reference container's applyDirichletBoundaryConditionToLocalMatrixRowsAndColumns
// does: entry (j, d) of every row j = nf*m + c' of a neighbour entity m,
// j != d, is set to zero.  Two Dirichlet DOFs may both write an entry (j, d)
// with j and d Dirichlet: both write zero; diagonals only their own row writes.
__global__ void k_dirichlet(int64_t n, const int32_t* __restrict__ lids, const double* __restrict__ g,
                            const double* __restrict__ x, double* __restrict__ f, const int64_t* __restrict__ rp,
                            const int64_t* __restrict__ erp, const int32_t* __restrict__ ecol, int nf,
                            double* __restrict__ vals) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < n; i += nwarps) {
    const int32_t d = lids[i];
    if (f && lane == 0) f[d] = x[d] - (g ? g[i] : 0.0);
    if (vals) {
      const int32_t r = d / nf, c = d - (d / nf) * nf;
      int64_t lo = erp[r], hi = erp[r + 1];
      while (lo < hi) {  // lower_bound of r in its row
        const int64_t mid = (lo + hi) >> 1;
        if (ecol[mid] < r) lo = mid + 1; else hi = mid;
      }
      const int64_t diag = rp[d] + (int64_t)nf * (lo - erp[r]) + c;
      for (int64_t k = rp[d] + lane; k < rp[d + 1]; k += 32) vals[k] = k == diag ? 1.0 : 0.0;
      if (!f) {  // rows and columns
        const int64_t b0 = erp[r], deg = erp[r + 1] - b0;
        for (int64_t t = lane; t < deg * nf; t += 32) {
          const int64_t m = ecol[b0 + t / nf];
          const int cc = (int)(t - (t / nf) * nf);
          const int64_t j = (int64_t)nf * m + cc;
          if (j != d) vals[rp[j] + (int64_t)nf * entity_pos(erp, ecol, m, r) + c] = 0.0;
        }
      }
    }
  }
}

// One lane's share of a CSR row product: entries b+sub, b+sub+LANES, ...
// U entries per pass are loaded together (values and column indices
// streamed past L1/L2, x through the read-only path) before any x gather
// issues, so a lane keeps 2U independent loads in flight.  Entries past the
// row end read column 0 with value 0.
// 16-byte chunks of values and column indices: 2 FP64 or 4 FP32 entries.
template <typename T> struct Chunk;
template <> struct Chunk<double> {
  using V = double2; using I = int2; static constexpr int N = 2;
  static __device__ __forceinline__ double at(const V& v, int t) { return t == 0 ? v.x : v.y; }
  static __device__ __forceinline__ int at(const I& v, int t) { return t == 0 ? v.x : v.y; }
};
template <> struct Chunk<float> {
  using V = float4; using I = int4; static constexpr int N = 4;
  static __device__ __forceinline__ float at(const V& v, int t) { return t == 0 ? v.x : t == 1 ? v.y : t == 2 ? v.z : v.w; }
  static __device__ __forceinline__ int at(const I& v, int t) { return t == 0 ? v.x : t == 1 ? v.y : t == 2 ? v.z : v.w; }
};
constexpr int kSpmvVector = 16;  // the shape's "unroll" value of the chunked form

template <typename T, int LANES, int U>
__device__ __forceinline__ T row_dot(int64_t b, int64_t e, int sub, const int32_t* __restrict__ col,
                                     const T* __restrict__ vals, const T* __restrict__ x) {
  T s = T(0);
  if constexpr (U == kSpmvVector) {
    // Chunked form: the 16-byte chunks lying wholly inside the row are read
    // with one vector load of values and one of column indices per lane; the
    // row's unaligned head and tail (fewer than N entries each) are read singly.
    // Needs vals and col 16-byte / (4N)-byte aligned (checked by the caller).
    using CH = Chunk<T>;
    constexpr int N = CH::N;
    const int64_t ja = (b + N - 1) / N, jb = e / N;  // whole chunks [ja, jb)
    if (ja >= jb) {
      for (int64_t k = b + sub; k < e; k += LANES) s += __ldcs(vals + k) * __ldg(x + __ldcs(col + k));
      return s;
    }
    if (b + sub < ja * N) s += __ldcs(vals + b + sub) * __ldg(x + __ldcs(col + b + sub));
    if (jb * N + sub < e) s += __ldcs(vals + jb * N + sub) * __ldg(x + __ldcs(col + jb * N + sub));
    for (int64_t j = ja + sub; j < jb; j += LANES) {
      const typename CH::V v = __ldcs(reinterpret_cast<const typename CH::V*>(vals) + j);
      const typename CH::I c = __ldcs(reinterpret_cast<const typename CH::I*>(col) + j);
#pragma unroll
      for (int t = 0; t < N; ++t) s += CH::at(v, t) * __ldg(x + CH::at(c, t));
    }
    return s;
  } else {
    for (int64_t k = b + sub; k < e; k += LANES * U) {
      T v[U];
      int32_t c[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t kk = k + u * LANES;
        v[u] = kk < e ? __ldcs(vals + kk) : T(0);
        c[u] = kk < e ? __ldcs(col + kk) : 0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) s += v[u] * __ldg(x + c[u]);
    }
    return s;
  }
}

// Vector CSR: LANES threads per row, strided over the row, shuffle reduction.
// The row loop advances per warp (its trip count is warp-uniform) so every
// lane reaches the full-mask shuffles; rows past n are predicated off.
template <typename T, int LANES, int U>
__global__ void __launch_bounds__(kThreads) k_spmv(int64_t n, const int64_t* __restrict__ rp,
                                                   const int32_t* __restrict__ col, const T* __restrict__ vals,
                                                   const T* __restrict__ x, T* __restrict__ y, T alpha, T beta) {
  constexpr int GPW = 32 / LANES;  // row groups per warp
  const int sub = threadIdx.x % LANES;
  const int g = (threadIdx.x & 31) / LANES;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * GPW; base < n; base += nwarps * GPW) {
    const int64_t r = base + g;
    T s = T(0);
    if (r < n) {
      s = row_dot<T, LANES, U>(__ldg(rp + r), __ldg(rp + r + 1), sub, col, vals, x);
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LANES);
    if (r < n && sub == 0) y[r] = beta == T(0) ? alpha * s : alpha * s + beta * y[r];
  }
}

// Entity-block form of the product on the graph this library expands: row
// nf*r + c holds, for each neighbour entity m of r in ascending order, the nf
// columns nf*m .. nf*m+nf-1, so the nf rows of entity r share one column
// pattern, and row c's values start at nf*nf*erp[r] + c*nf*deg(r).  G lanes
// take one entity; lane sub walks the blocks j = sub, sub+G, ..., reads the
// block's one column index ecol[erp[r]+j] and its nf values of x, and applies
// them to the block's nf x nf entries in all nf rows.  Index traffic falls
// from 4 bytes an entry to 4/nf^2, and x is read once a block, not once an
// entry.  U blocks per pass are loaded before any x gather issues.  Every
// load address lies inside its array whatever the data: a pass slot past the
// row end re-reads block j and zeroes its x values (a select, not an FP64
// multiply: GB300's FP64 pipe is the scarce unit here, one FMA an entry), and
// a column index outside [0, n_ent) reads entity 0.
// One pass of UU blocks a lane (blocks j, j + G, ..., j + (UU - 1) G); CHECK:
// slots may lie past the row end (the last pass of a row).
template <typename T, int NF, int G, int UU, bool CHECK>
__device__ __forceinline__ void entity_pass(int64_t j, int64_t b, int64_t deg, int64_t rs,
                                            const int32_t* __restrict__ ecol, const T* __restrict__ v0,
                                            const T* __restrict__ x, int64_t n_ent, T (&s)[NF]) {
  bool in[UU];
  int64_t m[UU];
  T v[UU][NF][NF];
#pragma unroll
  for (int u = 0; u < UU; ++u) {
    const int64_t jj = j + u * G;
    in[u] = !CHECK || jj < deg;
    const int64_t jc = in[u] ? jj : j;
    const uint32_t mm = (uint32_t)__ldcs(ecol + b + jc);
    m[u] = (uint64_t)mm < (uint64_t)n_ent ? (int64_t)mm : 0;
#pragma unroll
    for (int c = 0; c < NF; ++c)
#pragma unroll
      for (int d = 0; d < NF; ++d) v[u][c][d] = __ldcs(v0 + c * rs + NF * jc + d);
  }
#pragma unroll
  for (int u = 0; u < UU; ++u) {
    T xm[NF];
#pragma unroll
    for (int d = 0; d < NF; ++d) xm[d] = __ldg(x + NF * m[u] + d);
    if (in[u]) {  // a pass slot past the row end issues no FMAs
#pragma unroll
      for (int c = 0; c < NF; ++c)
#pragma unroll
        for (int d = 0; d < NF; ++d) s[c] += v[u][c][d] * xm[d];
    }
  }
}

// Full passes of U blocks a lane while the whole pass lies inside the row,
// then one last pass of just enough blocks a lane for the rest: an interior
// elasticity entity (27 blocks) on 4 lanes x 4 blocks takes 16 + 12 slots
// instead of 16 + 16, so the FP64 pipe (one FMA a lane-slot) idles on one
// slot in 28 rather than five in 32.  Every load address lies inside its
// array whatever the data: a slot past the row end re-reads block j (and
// issues no FMAs), and a column index outside [0, n_ent) reads entity 0.
template <typename T, int NF, int G, int U>
__device__ __forceinline__ void entity_dot(int64_t b, int64_t deg, int sub, const int32_t* __restrict__ ecol,
                                           const T* __restrict__ vals, const T* __restrict__ x, int64_t n_ent,
                                           T (&s)[NF]) {
  const T* v0 = vals + (int64_t)NF * NF * b;
  const int64_t rs = (int64_t)NF * deg;  // distance between the entity's rows
  const int64_t full = deg / (G * U) * (G * U);
  int64_t j = sub;
  for (; j < full; j += G * U) entity_pass<T, NF, G, U, false>(j, b, deg, rs, ecol, v0, x, n_ent, s);
  const int64_t rest = deg - full;  // blocks left for the last pass: fewer than G * U
  if (rest <= 0) return;
  const int64_t uu = (rest + G - 1) / G;
  if constexpr (U >= 4) {
    if (uu >= 4) { entity_pass<T, NF, G, 4, true>(j, b, deg, rs, ecol, v0, x, n_ent, s); return; }
  }
  if constexpr (U >= 3) {
    if (uu == 3) { entity_pass<T, NF, G, 3, true>(j, b, deg, rs, ecol, v0, x, n_ent, s); return; }
  }
  if constexpr (U >= 2) {
    if (uu == 2) { entity_pass<T, NF, G, 2, true>(j, b, deg, rs, ecol, v0, x, n_ent, s); return; }
  }
  entity_pass<T, NF, G, 1, true>(j, b, deg, rs, ecol, v0, x, n_ent, s);
}

// Sums the G lanes' partial rows of one entity (NF = 3) by reduce-scatter:
// with the rows padded to 4, an exchange across lane bit 1 leaves each lane
// two rows (sub & 2 picks which), one across bit 0 leaves one row (sub & 3),
// and butterflies over the G/4 lanes sharing a row finish it: 3 + log2(G/4)
// additions a lane instead of 3 log2(G) for three butterflies.  Lane sub < 3
// returns row sub.  G >= 4.
template <typename T, int NF, int G>
__device__ __forceinline__ T entity_reduce(const T (&s)[NF], int sub) {
  static_assert(NF == 3 && (G == 3 || G >= 4), "reduce-scatter of three rows over three or at least four lanes");
  if constexpr (G == 3) {
    // three lanes, three rows: lane sub keeps row sub and takes it from the two
    // other lanes of its group, each of which sends the row its receiver keeps
    const int base = (threadIdx.x & 31) - sub;
    T k = sub == 0 ? s[0] : sub == 1 ? s[1] : s[2];
#pragma unroll
    for (int o = 1; o < 3; ++o) {
      const int want = sub >= o ? sub - o : sub + 3 - o;  // the row of the lane this one sends to
      const T send = want == 0 ? s[0] : want == 1 ? s[1] : s[2];
      k += __shfl_sync(0xffffffffu, send, base + (sub + o < 3 ? sub + o : sub + o - 3));
    }
    return k;
  }
  const bool hi = (sub & 2) != 0, lo = (sub & 1) != 0;
  T a0 = hi ? s[2] : s[0];
  T a1 = hi ? T(0) : s[1];
  const T b0 = hi ? s[0] : s[2];
  const T b1 = hi ? s[1] : T(0);
  a0 += __shfl_xor_sync(0xffffffffu, b0, 2, G);
  a1 += __shfl_xor_sync(0xffffffffu, b1, 2, G);
  T k = lo ? a1 : a0;
  k += __shfl_xor_sync(0xffffffffu, lo ? a0 : a1, 1, G);
#pragma unroll
  for (int o = 4; o < G; o <<= 1) k += __shfl_xor_sync(0xffffffffu, k, o, G);
  return k;
}

// Six resident CTAs an SM (40 registers) for up to 16 lanes an entity; four
// (64 registers) for 32 lanes and for three lanes with three blocks a pass,
// whose FP64 forms would spill at 40.
constexpr int entity_min_blocks(int G, int U, int bytes = 4) {
  if (U >= 4) return bytes == 8 ? 3 : 4;  // four blocks in flight: 36 values a lane in registers
  return G >= 32 || (G < 4 && U >= 3) ? 4 : 6;
}

// y = alpha A x + beta y in the entity-block form; entity loop per warp as in
// k_spmv (warp-uniform trip count for the full-mask shuffles).
template <typename T, int NF, int G, int U>
__global__ void __launch_bounds__(kThreads, entity_min_blocks(G, U, sizeof(T))) k_spmv_eb(int64_t n_ent, const int64_t* __restrict__ erp,
                                                      const int32_t* __restrict__ ecol, const T* __restrict__ vals,
                                                      const T* __restrict__ x, T* __restrict__ y, T alpha, T beta) {
  constexpr int GPW = 32 / G;  // entities per warp (G = 3: ten, lanes 30 and 31 idle)
  const int lane = threadIdx.x & 31;
  const int g = lane / G < GPW ? lane / G : GPW;  // GPW: an idle lane
  const int sub = lane - (lane / G) * G;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * GPW; base < n_ent; base += nwarps * GPW) {
    const int64_t r = g < GPW ? base + g : n_ent;  // idle lanes take no entity
    T s[NF];
#pragma unroll
    for (int c = 0; c < NF; ++c) s[c] = T(0);
    const int64_t rc = r < n_ent ? r : n_ent - 1;  // rows past the end read the last entity's bounds
    const int64_t b = __ldg(erp + rc);
    entity_dot<T, NF, G, U>(b, r < n_ent ? __ldg(erp + rc + 1) - b : 0, sub, ecol, vals, x, n_ent, s);
    const T sc = entity_reduce<T, NF, G>(s, sub);
    if (r < n_ent && sub < NF) {
      const int64_t row = (int64_t)NF * r + sub;
      // y = A x needs no multiply (each FP64 operation costs a pipe slot here)
      y[row] = beta == T(0) ? (alpha == T(1) ? sc : alpha * sc) : alpha * sc + beta * y[row];
    }
  }
}

// The automatic shape, from timings of every shape on the 128^3 elasticity
// operator (80 entries a row): narrow row groups win (8 lanes, FP64 1.52 ms
// against 3.84 ms for a warp per row), FP32 gains from four loads per lane.
SpmvShape resolve_shape(SpmvShape sh, int64_t n, int64_t nnz_hint, bool f32) {
  if (sh.lanes > 0 && sh.unroll > 0) return sh;
  const double avg = nnz_hint > 0 && n > 0 ? (double)nnz_hint / (double)n : 32.0;
  sh.lanes = avg <= 12 ? 4 : avg <= 128 ? 8 : 16;
  sh.unroll = f32 ? 4 : 1;
  return sh;
}

// The chunked form reads values and column indices as aligned 16-byte vectors.
template <typename T>
bool chunk_aligned(const T* vals, const int32_t* col) {
  return ((uintptr_t)vals % 16) == 0 && ((uintptr_t)col % (4 * Chunk<T>::N)) == 0;
}

// Calls F.template run<LANES, U>() for the shape's template arguments.
template <typename F>
cudaError_t with_shape(SpmvShape sh, F&& f) {
#define TX_SHAPE(L, U) \
  if (sh.lanes == L && sh.unroll == U) return f.template run<L, U>();
  TX_SHAPE(4, 1) TX_SHAPE(4, 2) TX_SHAPE(4, 4)
  TX_SHAPE(8, 1) TX_SHAPE(8, 2) TX_SHAPE(8, 4)
  TX_SHAPE(16, 1) TX_SHAPE(16, 2) TX_SHAPE(16, 4)
  TX_SHAPE(32, 1) TX_SHAPE(32, 2) TX_SHAPE(32, 4)
  TX_SHAPE(4, kSpmvVector) TX_SHAPE(8, kSpmvVector) TX_SHAPE(16, kSpmvVector) TX_SHAPE(32, kSpmvVector)
#undef TX_SHAPE
  return cudaErrorInvalidValue;
}

template <typename T>
struct SpmvLaunch {
  int64_t n; const int64_t* rp; const int32_t* col; const T* vals; const T* x; T* y; T a, b; cudaStream_t s;
  template <int L, int U>
  cudaError_t run() const {
    k_spmv<T, L, U><<<grid_for(n, kThreads / L, 152 * 64), kThreads, 0, s>>>(n, rp, col, vals, x, y, a, b);
    return cudaGetLastError();
  }
};

template <typename T>
cudaError_t spmv_dispatch(int64_t n, const int64_t* rp, const int32_t* col, const T* vals, const T* x, T* y, T a,
                          T b, int64_t nnz_hint, cudaStream_t s, SpmvShape shape) {
  if (n <= 0) return cudaSuccess;
  SpmvShape sh = resolve_shape(shape, n, nnz_hint, sizeof(T) == 4);
  if (sh.unroll == kSpmvVector && !chunk_aligned<T>(vals, col)) sh.unroll = 1;
  return with_shape(sh, SpmvLaunch<T>{n, rp, col, vals, x, y, a, b, s});
}

// Entity-block shapes: lanes per entity 3 (blocks per lane pass 1-3), 4/8
// (1/2/4), 16/32 (1/2).  {0, 0}: FP64 4 lanes, 4 blocks: GB300's FP64 pipe
// (about two FMAs a clock an SM) bounds the FP64 product, 4 lanes waste few
// FMA slots on the 27 blocks of an interior entity (two passes of 16) and on
// the row sums, and four blocks a lane keep 36 values in flight; FP32 16
// lanes, 2 blocks.  Both the fastest of their precision on the 128^3
// elasticity operator.
SpmvShape resolve_entity_shape(SpmvShape sh, bool f32) {
  if (sh.lanes > 0 && sh.unroll > 0) return sh;
  return f32 ? SpmvShape{16, 2} : SpmvShape{4, 4};
}

template <typename F>
cudaError_t with_entity_shape(SpmvShape sh, F&& f) {
#define TX_ESHAPE(L, U) \
  if (sh.lanes == L && sh.unroll == U) return f.template run<L, U>();
  TX_ESHAPE(3, 1) TX_ESHAPE(3, 2) TX_ESHAPE(3, 3)
  TX_ESHAPE(4, 1) TX_ESHAPE(4, 2) TX_ESHAPE(4, 4) TX_ESHAPE(8, 1) TX_ESHAPE(8, 2) TX_ESHAPE(8, 4)
  TX_ESHAPE(16, 1) TX_ESHAPE(16, 2) TX_ESHAPE(32, 1) TX_ESHAPE(32, 2)
#undef TX_ESHAPE
  return cudaErrorInvalidValue;
}

template <typename T>
struct EntitySpmvLaunch {
  EntityGraph eg; const T* vals; const T* x; T* y; T a, b; cudaStream_t s;
  template <int L, int U>
  cudaError_t run() const {
    k_spmv_eb<T, kEntityNf, L, U><<<grid_for(eg.n_ent, (kThreads / 32) * (32 / L), 152 * 64), kThreads, 0, s>>>(
        eg.n_ent, eg.erp, eg.ecol, vals, x, y, a, b);
    return cudaGetLastError();
  }
};

// ------------------------------------------------------------ reductions
// Block partial sums into red[slot * kRedBlocks + block]; a one-block
// finalize kernel writes the total.  Order is fixed: results are
// reproducible run to run.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block_sum with the total in every thread.
__device__ __forceinline__ double block_sum_all(double v, double* sh) {
  v = block_sum(v, sh);
  __syncthreads();  // every read of sh in block_sum is done
  if (threadIdx.x == 0) sh[0] = v;
  __syncthreads();
  return sh[0];
}

// The sum of nparts partials in every thread, in one fixed order: every CTA
// that reduces the same partials gets the same bits.
__device__ __forceinline__ double partials_sum(const double* __restrict__ part, int nparts, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += part[i];
  return block_sum_all(v, sh);
}

// Sums the first nparts partials of each of nslots slots.
__global__ void k_finalize(const double* __restrict__ red, int nslots, double* __restrict__ out,
                           int nparts = kRedBlocks) {
  __shared__ double sh[32];
  for (int s = 0; s < nslots; ++s) {
    double v = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += red[s * kRedBlocks + i];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) out[s] = v;
    __syncthreads();
  }
}

__global__ void k_norm2sq(const double* __restrict__ x, int64_t n, double* __restrict__ red) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += x[i] * x[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) red[blockIdx.x] = s;
}

__global__ void k_fill(double* p, double v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}
__global__ void k_axpby(double* y, const double* x, double a, double b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

__global__ void k_scaled_diff(double* out, const double* x, const double* xp, double c, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = c * (x[i] - xp[i]);
}

// ------------------------------------------------------------ CG kernels
// FP32 copy of A with symmetric Dirichlet elimination + Jacobi diagonal.
__global__ void k_make_f32(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                           const double* __restrict__ v64, const uint8_t* __restrict__ mask, float* __restrict__ v32,
                           float* __restrict__ dinv) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < n; r += nwarps) {
    const bool dr = mask[r];
    double diag = 0.0;
    for (int64_t k = rp[r] + lane; k < rp[r + 1]; k += 32) {
      const int32_t c = col[k];
      double v = v64[k];
      if (dr || mask[c]) v = (c == r) ? 1.0 : 0.0;
      v32[k] = (float)v;
      if (c == r) diag = v;
    }
    for (int o = 16; o > 0; o >>= 1) diag += __shfl_xor_sync(0xffffffffu, diag, o);
    if (lane == 0) dinv[r] = diag != 0.0 ? (float)(1.0 / diag) : 1.0f;
  }
}

// Block Jacobi: per entity the inverse of its 3x3 diagonal block (row (r, c),
// neighbour r, field d at rp[3r + c] + 3 j0 + d, j0 = r's place in its own
// row), with Dirichlet rows and columns made identity as in k_make_f32;
// inverted in FP64 by cofactors, a singular block falls back to its diagonal.
__global__ void k_make_binv(int64_t n_ent, const int64_t* __restrict__ erp, const int32_t* __restrict__ ecol,
                            const int64_t* __restrict__ rp, const double* __restrict__ v64,
                            const uint8_t* __restrict__ mask, float* __restrict__ binv) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_ent; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t j0 = -1;
    for (int64_t k = erp[r]; k < erp[r + 1]; ++k)
      if (ecol[k] == r) { j0 = k - erp[r]; break; }
    double B[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double v = j0 >= 0 ? v64[rp[3 * r + c] + 3 * j0 + d] : (c == d ? 1.0 : 0.0);
        if (mask[3 * r + c] || mask[3 * r + d]) v = c == d ? 1.0 : 0.0;
        B[c][d] = v;
      }
    const double c00 = B[1][1] * B[2][2] - B[1][2] * B[2][1], c01 = B[1][2] * B[2][0] - B[1][0] * B[2][2],
                 c02 = B[1][0] * B[2][1] - B[1][1] * B[2][0];
    const double det = B[0][0] * c00 + B[0][1] * c01 + B[0][2] * c02;
    float* o = binv + 9 * r;
    const double scale = fabs(B[0][0]) + fabs(B[1][1]) + fabs(B[2][2]);
    if (det != 0.0 && isfinite(det) && fabs(det) > 1e-30 * scale * scale * scale) {
      const double id = 1.0 / det;
      o[0] = (float)(c00 * id);
      o[1] = (float)((B[0][2] * B[2][1] - B[0][1] * B[2][2]) * id);
      o[2] = (float)((B[0][1] * B[1][2] - B[0][2] * B[1][1]) * id);
      o[3] = (float)(c01 * id);
      o[4] = (float)((B[0][0] * B[2][2] - B[0][2] * B[2][0]) * id);
      o[5] = (float)((B[0][2] * B[1][0] - B[0][0] * B[1][2]) * id);
      o[6] = (float)(c02 * id);
      o[7] = (float)((B[0][1] * B[2][0] - B[0][0] * B[2][1]) * id);
      o[8] = (float)((B[0][0] * B[1][1] - B[0][1] * B[1][0]) * id);
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) o[k] = 0.0f;
#pragma unroll
      for (int c = 0; c < 3; ++c) o[4 * c] = B[c][c] != 0.0 ? (float)(1.0 / B[c][c]) : 1.0f;
    }
  }
}

__global__ void k_mask(int64_t n, const int32_t* lids, uint8_t* mask) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    mask[lids[i]] = 1;
}

// The CG's dot products are exact products of FP32 values summed in FP64
// (the same bits as converting with the hardware); the FP32 -> FP64
// conversions are integer operations (widen), so each term costs one DFMA
// on GB300's narrow FP64 pipe instead of two conversions and a DFMA there.
// r32 = r64 (Dirichlet rows zero), z = dinv r, p = z, d = 0; partials rz, rr
__global__ void k_cg_init(int64_t n, const double* __restrict__ r64, const uint8_t* __restrict__ mask,
                          const float* __restrict__ dinv, float* r, float* z, float* p, float* d, double* red) {
  __shared__ double sh[32];
  double rz = 0.0, rr = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float ri = mask[i] ? 0.0f : (float)r64[i];
    const float zi = dinv[i] * ri;
    r[i] = ri; z[i] = zi; p[i] = zi; d[i] = 0.0f;
    const double rd = widen(ri);
    rz += rd * widen(zi);
    rr += rd * rd;
  }
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) red[0 * kRedBlocks + blockIdx.x] = rz;
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) red[1 * kRedBlocks + blockIdx.x] = rr;
}

// Block-Jacobi forms of k_cg_init / k_cg_update: one thread per entity, z = B^-1 r on its three DOFs.
__device__ __forceinline__ void block_apply(const float* __restrict__ bi, const float (&r)[3], float (&z)[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) z[c] = bi[3 * c] * r[0] + bi[3 * c + 1] * r[1] + bi[3 * c + 2] * r[2];
}

__global__ void k_cg_init_b(int64_t n_ent, const double* __restrict__ r64, const uint8_t* __restrict__ mask,
                            const float* __restrict__ binv, float* r, float* z, float* p, float* d, double* red) {
  __shared__ double sh[32];
  double rz = 0.0, rr = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_ent; e += (int64_t)gridDim.x * blockDim.x) {
    float ri[3], zi[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) ri[c] = mask[3 * e + c] ? 0.0f : (float)r64[3 * e + c];
    block_apply(binv + 9 * e, ri, zi);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t i = 3 * e + c;
      r[i] = ri[c]; z[i] = zi[c]; p[i] = zi[c]; d[i] = 0.0f;
      const double rd = widen(ri[c]);
      rz += rd * widen(zi[c]);
      rr += rd * rd;
    }
  }
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) red[0 * kRedBlocks + blockIdx.x] = rz;
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) red[1 * kRedBlocks + blockIdx.x] = rr;
}

__global__ void k_cg_update_b(int64_t n_ent, const double* __restrict__ rz_in, const double* __restrict__ pq_part,
                              int pq_parts, const float* __restrict__ binv, const float* __restrict__ p,
                              const float* __restrict__ q, float* r, float* z, float* d, double* red) {
  __shared__ double sh[32];
  const double pq = partials_sum(pq_part, pq_parts, sh);
  const float a = pq != 0.0 ? (float)(*rz_in / pq) : 0.0f;
  double rz = 0.0, rr = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_ent; e += (int64_t)gridDim.x * blockDim.x) {
    float ri[3], zi[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t i = 3 * e + c;
      d[i] += a * p[i];
      ri[c] = r[i] - a * q[i];
    }
    block_apply(binv + 9 * e, ri, zi);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t i = 3 * e + c;
      r[i] = ri[c]; z[i] = zi[c];
      const double rd = widen(ri[c]);
      rz += rd * widen(zi[c]);
      rr += rd * rd;
    }
  }
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) red[3 * kRedBlocks + blockIdx.x] = rz;
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) red[1 * kRedBlocks + blockIdx.x] = rr;
}

// q = A p and partial dot(p, q)
template <int LANES, int U>
__global__ void __launch_bounds__(kThreads) k_spmv_dot(int64_t n, const int64_t* __restrict__ rp,
                                                       const int32_t* __restrict__ col, const float* __restrict__ vals,
                                                       const float* __restrict__ p, float* __restrict__ q,
                                                       double* __restrict__ red) {
  __shared__ double sh[32];
  constexpr int GPW = 32 / LANES;
  const int sub = threadIdx.x % LANES;
  const int g = (threadIdx.x & 31) / LANES;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double pq = 0.0;
  for (int64_t base = warp * GPW; base < n; base += nwarps * GPW) {  // warp-uniform trip count
    const int64_t r = base + g;
    float s = 0.0f;
    if (r < n) {
      s = row_dot<float, LANES, U>(__ldg(rp + r), __ldg(rp + r + 1), sub, col, vals, p);
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LANES);
    if (r < n && sub == 0) {
      q[r] = s;
      pq += widen(s) * widen(p[r]);
    }
  }
  pq = block_sum(pq, sh);
  if (threadIdx.x == 0) red[2 * kRedBlocks + blockIdx.x] = pq;
}

// q = A p and partial dot(p, q) in the entity-block form
template <int NF, int G, int U>
__global__ void __launch_bounds__(kThreads, entity_min_blocks(G, U)) k_spmv_dot_eb(int64_t n_ent, const int64_t* __restrict__ erp,
                                                          const int32_t* __restrict__ ecol,
                                                          const float* __restrict__ vals, const float* __restrict__ p,
                                                          float* __restrict__ q, double* __restrict__ red) {
  __shared__ double sh[32];
  constexpr int GPW = 32 / G;
  const int lane = threadIdx.x & 31;
  const int g = lane / G < GPW ? lane / G : GPW;  // GPW: an idle lane
  const int sub = lane - (lane / G) * G;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double pq = 0.0;
  for (int64_t base = warp * GPW; base < n_ent; base += nwarps * GPW) {  // warp-uniform trip count
    const int64_t r = g < GPW ? base + g : n_ent;  // idle lanes take no entity
    float s[NF];
#pragma unroll
    for (int c = 0; c < NF; ++c) s[c] = 0.0f;
    const int64_t rc = r < n_ent ? r : n_ent - 1;
    const int64_t b = __ldg(erp + rc);
    entity_dot<float, NF, G, U>(b, r < n_ent ? __ldg(erp + rc + 1) - b : 0, sub, ecol, vals, p, n_ent, s);
    const float sc = entity_reduce<float, NF, G>(s, sub);
    if (r < n_ent && sub < NF) {
      const int64_t row = (int64_t)NF * r + sub;
      q[row] = sc;
      pq += widen(sc) * widen(p[row]);
    }
  }
  pq = block_sum(pq, sh);
  if (threadIdx.x == 0) red[2 * kRedBlocks + blockIdx.x] = pq;
}

// a = rz / pq (pq from the SpMV's partials, reduced by every CTA); d += a p,
// r -= a q, z = dinv r; partials of rz' and rr'
__global__ void k_cg_update(int64_t n, const double* __restrict__ rz_in, const double* __restrict__ pq_part,
                            int pq_parts, const float* __restrict__ dinv, const float* __restrict__ p,
                            const float* __restrict__ q, float* r, float* z, float* d, double* red) {
  __shared__ double sh[32];
  const double pq = partials_sum(pq_part, pq_parts, sh);
  const float a = pq != 0.0 ? (float)(*rz_in / pq) : 0.0f;
  double rz = 0.0, rr = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    d[i] += a * p[i];
    const float ri = r[i] - a * q[i];
    const float zi = dinv[i] * ri;
    r[i] = ri; z[i] = zi;
    const double rd = widen(ri);
    rz += rd * widen(zi);
    rr += rd * rd;
  }
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) red[3 * kRedBlocks + blockIdx.x] = rz;
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) red[1 * kRedBlocks + blockIdx.x] = rr;
}

// rz' = sum of the update's slot-3 partials (reduced by every CTA), beta =
// rz' / rz; p = z + beta p.  CTA 0 stores rz' in the other parity's slot
// (rz_out; every CTA reads rz from rz_in, which nothing writes here) and rr'
// for the host's convergence check.
__global__ void k_cg_pupdate(int64_t n, const double* __restrict__ rz_in, const double* __restrict__ red,
                             double* __restrict__ rz_out, double* __restrict__ rr_out, const float* __restrict__ z,
                             float* p) {
  __shared__ double sh[32];
  const double rz = partials_sum(red + 3 * kRedBlocks, kRedBlocks, sh);
  const double rzo = *rz_in;
  const float be = rzo != 0.0 ? (float)(rz / rzo) : 0.0f;
  if (blockIdx.x == 0) {
    const double rr = partials_sum(red + 1 * kRedBlocks, kRedBlocks, sh);
    if (threadIdx.x == 0) { *rz_out = rz; *rr_out = rr; }
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + be * p[i];
}

__global__ void k_add_f32(int64_t n, double* x, const float* d) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += (double)d[i];
}

template <typename T>
cudaError_t cmalloc(T*& p, size_t n) {
  return cudaMalloc((void**)&p, sizeof(T) * (n > 0 ? n : 1));
}

}  // namespace

cudaError_t launch_expand_rowptr(const int64_t* erp, int64_t n_ent, int nf, int64_t* rp, cudaStream_t s) {
  if (n_ent <= 0) return cudaSuccess;
  k_expand_rowptr<<<grid_for(n_ent, kThreads), kThreads, 0, s>>>(erp, n_ent, nf, rp);
  return cudaGetLastError();
}
cudaError_t launch_expand_colind(const int64_t* erp, const int32_t* ecol, int64_t n_ent, int nf, const int64_t* rp,
                                 int32_t* col, cudaStream_t s) {
  if (n_ent <= 0) return cudaSuccess;
  k_expand_colind<<<grid_for(n_ent, kThreads / 32), kThreads, 0, s>>>(erp, ecol, n_ent, nf, rp, col);
  return cudaGetLastError();
}
cudaError_t launch_dirichlet(int64_t n, const int32_t* lids, const double* g, const double* x, double* f,
                             const int64_t* rp, const int64_t* erp, const int32_t* ecol, int nf, double* vals,
                             cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_dirichlet<<<grid_for(n, kThreads / 32), kThreads, 0, s>>>(n, lids, g, x, f, rp, erp, ecol, nf, vals);
  return cudaGetLastError();
}
bool spmv_shape_valid(SpmvShape sh) {
  if (sh.lanes == 0 && sh.unroll == 0) return true;
  const bool l = sh.lanes == 4 || sh.lanes == 8 || sh.lanes == 16 || sh.lanes == 32;
  const bool u = sh.unroll == 1 || sh.unroll == 2 || sh.unroll == 4 || sh.unroll == kSpmvVector;
  return l && u;
}
bool entity_shape_valid(SpmvShape sh) {
  if (sh.lanes == 0 && sh.unroll == 0) return true;
  if (sh.lanes == 3) return sh.unroll >= 1 && sh.unroll <= 3;
  const bool l = sh.lanes == 4 || sh.lanes == 8 || sh.lanes == 16 || sh.lanes == 32;
  return l && (sh.unroll == 1 || sh.unroll == 2 || (sh.unroll == 4 && sh.lanes <= 8));
}
cudaError_t launch_spmv_entity_f64(const EntityGraph& eg, const double* vals, const double* x, double* y, double a,
                                   double b, cudaStream_t s, SpmvShape shape) {
  if (eg.n_ent <= 0) return cudaSuccess;
  return with_entity_shape(resolve_entity_shape(shape, false), EntitySpmvLaunch<double>{eg, vals, x, y, a, b, s});
}
cudaError_t launch_spmv_entity_f32(const EntityGraph& eg, const float* vals, const float* x, float* y, float a,
                                   float b, cudaStream_t s, SpmvShape shape) {
  if (eg.n_ent <= 0) return cudaSuccess;
  return with_entity_shape(resolve_entity_shape(shape, true), EntitySpmvLaunch<float>{eg, vals, x, y, a, b, s});
}
cudaError_t launch_spmv_f64(int64_t n, const int64_t* rp, const int32_t* col, const double* vals, const double* x,
                            double* y, double a, double b, int64_t nnz_hint, cudaStream_t s, SpmvShape shape) {
  return spmv_dispatch<double>(n, rp, col, vals, x, y, a, b, nnz_hint, s, shape);
}
cudaError_t launch_spmv_f32(int64_t n, const int64_t* rp, const int32_t* col, const float* vals, const float* x,
                            float* y, float a, float b, int64_t nnz_hint, cudaStream_t s, SpmvShape shape) {
  return spmv_dispatch<float>(n, rp, col, vals, x, y, a, b, nnz_hint, s, shape);
}
cudaError_t launch_fill(double* p, double v, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_fill<<<grid_for(n, kThreads), kThreads, 0, s>>>(p, v, n);
  return cudaGetLastError();
}
cudaError_t launch_axpby(double* y, const double* x, double a, double b, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_axpby<<<grid_for(n, kThreads), kThreads, 0, s>>>(y, x, a, b, n);
  return cudaGetLastError();
}
cudaError_t launch_scaled_diff(double* out, const double* x, const double* xp, double c, int64_t n,
                               cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_scaled_diff<<<grid_for(n, kThreads), kThreads, 0, s>>>(out, x, xp, c, n);
  return cudaGetLastError();
}
cudaError_t launch_norm2sq(const double* x, int64_t n, double* red, double* out, cudaStream_t s) {
  cudaMemsetAsync(red, 0, sizeof(double) * kRedBlocks, s);
  k_norm2sq<<<kRedBlocks, kThreads, 0, s>>>(x, n, red);
  k_finalize<<<1, 1024, 0, s>>>(red, 1, out);
  return cudaGetLastError();
}

cudaError_t solver_alloc(SolverWork& w, int64_t n, int64_t nnz) {
  if (w.n == n && w.nnz == nnz && w.vals32) return cudaSuccess;
  solver_free(w);
  cudaError_t e;
  if ((e = cmalloc(w.vals32, nnz)) != cudaSuccess) return e;
  if ((e = cmalloc(w.dinv, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.binv, 3 * n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.r, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.z, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.p, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.q, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.d, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.r64, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.xdw, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.mask, n)) != cudaSuccess) return e;
  if ((e = cmalloc(w.red, (size_t)kRedSlots * kRedBlocks)) != cudaSuccess) return e;
  if ((e = cmalloc(w.scal, 8)) != cudaSuccess) return e;
  if ((e = cudaMallocHost((void**)&w.host_scal, sizeof(double) * 8)) != cudaSuccess) return e;
  cudaMemset(w.red, 0, sizeof(double) * kRedSlots * kRedBlocks);
  w.n = n; w.nnz = nnz;
  return cudaSuccess;
}

void solver_free(SolverWork& w) {
  cudaFree(w.vals32); cudaFree(w.dinv); cudaFree(w.binv); cudaFree(w.r); cudaFree(w.z); cudaFree(w.p); cudaFree(w.q);
  cudaFree(w.d); cudaFree(w.r64); cudaFree(w.xdw); cudaFree(w.mask); cudaFree(w.red); cudaFree(w.scal);
  if (w.host_scal) cudaFreeHost(w.host_scal);
  w = SolverWork();
}

__global__ void k_fixed_stats(const double* scal, int outer, int inner, double* out) {
  // scal[4] = ||r_final||^2, scal[5] = ||r_0||^2
  const double r0 = sqrt(scal[5]);
  out[0] = outer;
  out[1] = (double)outer * inner;
  out[2] = r0 > 0.0 ? sqrt(scal[4]) / r0 : 0.0;
  out[3] = r0;
}

// q = A p with dot(p, q) partials, in the solver's SpMV shape
struct DotLaunch {
  int64_t n; const int64_t* rp; const int32_t* col; const SolverWork* w; unsigned gb; cudaStream_t s;
  template <int L, int U>
  cudaError_t run() const {
    k_spmv_dot<L, U><<<gb, kThreads, 0, s>>>(n, rp, col, w->vals32, w->p, w->q, w->red);
    return cudaSuccess;
  }
};

// resident CTAs an SM of the SpMV+dot kernel of a shape
struct DotOccupancy {
  int* per;
  template <int L, int U>
  cudaError_t run() const {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, k_spmv_dot<L, U>, kThreads, 0);
  }
};
struct DotEntityOccupancy {
  int* per;
  template <int L, int U>
  cudaError_t run() const {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, k_spmv_dot_eb<kEntityNf, L, U>, kThreads, 0);
  }
};

// the same in the entity-block form
struct DotEntityLaunch {
  EntityGraph eg; const SolverWork* w; unsigned gb; cudaStream_t s;
  template <int L, int U>
  cudaError_t run() const {
    k_spmv_dot_eb<kEntityNf, L, U><<<gb, kThreads, 0, s>>>(eg.n_ent, eg.erp, eg.ecol, w->vals32, w->p, w->q, w->red);
    return cudaSuccess;
  }
};

int solve_cg_ir(SolverWork& w, const int64_t* rp, const int32_t* col, const double* vals, int64_t n_dir,
                const int32_t* dir, double* x, ResidualFn resid, void* ctx, double rtol, double inner_rtol,
                int max_outer, int max_inner, double* stats, cudaStream_t s, std::string& err, bool fixed,
                bool reuse_op, double* stats_dev, const EntityGraph* eg, bool block_jacobi) {
  const int64_t n = w.n;
  const unsigned gb = kRedBlocks;
  auto cuda_fail = [&](cudaError_t e, const char* where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return TX_ECUDA;
  };
  cudaError_t e;
  // FP32 operator with symmetric Dirichlet elimination
  if (!reuse_op) {
    cudaMemsetAsync(w.mask, 0, n, s);
    if (n_dir > 0) k_mask<<<grid_for(n_dir, kThreads), kThreads, 0, s>>>(n_dir, dir, w.mask);
    k_make_f32<<<grid_for(n, kThreads / 32), kThreads, 0, s>>>(n, rp, col, vals, w.mask, w.vals32, w.dinv);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "cg: make_f32");
    w.binv_valid = false;
  }
  // block Jacobi: the entity-block form's three-field rows only
  const bool blk = block_jacobi && eg && n == 3 * eg->n_ent;
  if (blk && !w.binv_valid) {
    k_make_binv<<<grid_for(eg->n_ent, kThreads), kThreads, 0, s>>>(eg->n_ent, eg->erp, eg->ecol, rp, vals, w.mask,
                                                                   w.binv);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "cg: make_binv");
    w.binv_valid = true;
  }
  auto cg_init = [&]() {
    if (blk) k_cg_init_b<<<gb, kThreads, 0, s>>>(eg->n_ent, w.r64, w.mask, w.binv, w.r, w.z, w.p, w.d, w.red);
    else k_cg_init<<<gb, kThreads, 0, s>>>(n, w.r64, w.mask, w.dinv, w.r, w.z, w.p, w.d, w.red);
  };
  SpmvShape shape = resolve_shape(w.spmv, n, w.nnz, true);
  if (shape.unroll == kSpmvVector && !chunk_aligned<float>(w.vals32, col)) shape.unroll = 1;
  const SpmvShape eshape = resolve_entity_shape(w.spmv_eb, true);
  // The SpMV+dot grid is one full wave of resident CTAs (at most kRedBlocks
  // partials): with 1024 CTAs and six resident an SM, a second wave of 112
  // CTAs ran on 12 % of the GPU and nearly doubled the product's time.
  unsigned gd = gb;
  {
    int per = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (eg) with_entity_shape(eshape, DotEntityOccupancy{&per});
    else with_shape(shape, DotOccupancy{&per});
    if (per > 0 && sms > 0 && per * sms < (int)gb) gd = (unsigned)(per * sms);
  }
  auto spmv_dot = [&]() {
    if (eg) with_entity_shape(eshape, DotEntityLaunch{*eg, &w, gd, s});
    else with_shape(shape, DotLaunch{n, rp, col, &w, gd, s});
  };
  // Three launches an iteration: SpMV + dot partials, the update (reducing the
  // dot itself), the p update (reducing rz' itself).  rz alternates between
  // scal[0] and scal[6] by iteration parity, so no CTA reads a slot another
  // CTA of the same launch writes; an inner solve starts at parity 0 (the
  // initialisation's rz in scal[0]); rr is in scal[1].
  int par = 0;
  auto rz_slot = [&](int q) { return w.scal + (q ? 6 : 0); };
  auto cg_iteration = [&]() {
    spmv_dot();
    const double* pq_part = w.red + 2 * kRedBlocks;
    if (blk)
      k_cg_update_b<<<gb, kThreads, 0, s>>>(eg->n_ent, rz_slot(par), pq_part, (int)gd, w.binv, w.p, w.q, w.r, w.z,
                                            w.d, w.red);
    else
      k_cg_update<<<gb, kThreads, 0, s>>>(n, rz_slot(par), pq_part, (int)gd, w.dinv, w.p, w.q, w.r, w.z, w.d, w.red);
    k_cg_pupdate<<<gb, kThreads, 0, s>>>(n, rz_slot(par), w.red, rz_slot(par ^ 1), w.scal + 1, w.z, w.p);
    par ^= 1;
  };
  if (fixed) {
    // Capturable form: exact iteration counts, no host reads; statistics
    // land in stats_dev (device) when given.
    for (int outer = 0; outer < max_outer; ++outer) {
      int rc = resid(ctx, x, w.r64);
      if (rc) { err = "cg: residual evaluation failed"; return rc; }
      if (outer == 0 && (e = launch_norm2sq(w.r64, n, w.red, w.scal + 5, s)) != cudaSuccess)
        return cuda_fail(e, "cg: norm");
      cg_init();
      k_finalize<<<1, 1024, 0, s>>>(w.red, 2, w.scal);
      par = 0;
      for (int it = 0; it < max_inner; ++it) cg_iteration();
      k_add_f32<<<grid_for(n, kThreads), kThreads, 0, s>>>(n, x, w.d);
    }
    int rc = resid(ctx, x, w.r64);
    if (rc) { err = "cg: residual evaluation failed"; return rc; }
    if ((e = launch_norm2sq(w.r64, n, w.red, w.scal + 4, s)) != cudaSuccess) return cuda_fail(e, "cg: norm");
    if (stats_dev) k_fixed_stats<<<1, 1, 0, s>>>(w.scal, max_outer, max_inner, stats_dev);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "cg: fixed iterations");
    return TX_OK;
  }
  double r0 = -1.0, rn = 0.0;
  int outer = 0, inner_total = 0;
  for (;; ++outer) {
    int rc = resid(ctx, x, w.r64);
    if (rc) { err = "cg: residual evaluation failed"; return rc; }
    if ((e = launch_norm2sq(w.r64, n, w.red, w.scal + 4, s)) != cudaSuccess) return cuda_fail(e, "cg: norm");
    cudaMemcpyAsync(w.host_scal, w.scal + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "cg: sync");
    rn = std::sqrt(w.host_scal[0]);
    if (r0 < 0.0) r0 = rn > 0.0 ? rn : 1.0;
    if (rn <= rtol * r0 || outer >= max_outer) break;
    // inner FP32 Jacobi-PCG on A32 d = r
    cg_init();
    k_finalize<<<1, 1024, 0, s>>>(w.red, 2, w.scal);  // scal[0] = rz, scal[1] = rr
    par = 0;
    cudaMemcpyAsync(w.host_scal, w.scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "cg: init");
    const double rr0 = w.host_scal[1];
    const double target = inner_rtol * inner_rtol * rr0;
    int it = 0;
    const int check = 16;
    while (it < max_inner) {
      for (int k = 0; k < check && it < max_inner; ++k, ++it) cg_iteration();
      cudaMemcpyAsync(w.host_scal, w.scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, s);
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "cg: iterate");
      if (!(w.host_scal[1] > target)) break;  // also stops on NaN
    }
    inner_total += it;
    k_add_f32<<<grid_for(n, kThreads), kThreads, 0, s>>>(n, x, w.d);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "cg: update");
  }
  if (stats) {
    stats[0] = outer;
    stats[1] = inner_total;
    stats[2] = rn / r0;
    stats[3] = r0;
  }
  return (rn <= rtol * r0) ? TX_OK : TX_ETIMEDOUT;
}

}  // namespace tx
