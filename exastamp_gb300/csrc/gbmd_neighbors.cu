// gbmd_neighbors.cu -- cell grid, cell sort and full neighbour list on sm_103a.
//
// Restates exaNBody's move_particles (periodic wrap, rebinning) and
// chunk_neighbors with chunk_size 1 (data/config/config_move_particles.msp
// L54-68).  The pair set is the one the reference decodes in
// src/debug/atom_neighbors_stats.cpp L169-228: every (i, j, image n) with
// d2 <= (rcut_max + skin)^2, d2 computed in FP64 from ((x_j + n*L) - x_i)
// without contraction.  Candidates are screened in FP32 on home-cell-relative
// coordinates; only those within 2^-12 of the radius are re-tested in FP64,
// so the list is bit-identical to an all-FP64 build.
//
// Kernels (per rebuild):
//   k_wrap_bin    wrap into [lo,hi), bin, count per cell        HBM: 24 B r/w + 8 B
//   k_scan_*      exclusive scan of cell counts                 negligible
//   k_scatter     atoms -> cell segments (atomic slot)          HBM: 12 B
//   k_cell_rank   canonical (id, upload index) order per cell   L1-resident
//   k_gather      permute the FP64 state into cell order        HBM: ~130 B r/w
//   k_posf        FP32 local + FP64 packed gather copies        HBM: 24 B r, 48 B w
//   k_build_list_cells  warp per home cell over the 27-cell candidates, ballot
//                 compaction in canonical order                 HBM: 4 B per entry
//
// Every kernel of the chain takes a `gate` word: when it is non-null and
// holds 0 the kernel returns at once.  The displacement-triggered step
// (particle_displ_over, config_move_particles.msp L19-22, L116-118) sets the
// gate on the device and launches the chain unconditionally, so the decision
// to rebuild never goes through the host and the chain can sit inside a CUDA
// graph.  That variant gathers into the spare buffers and copies back, so the
// buffer parity the captured pointers rely on does not depend on the outcome.
#include <cstdio>
#include <cstring>
#include <utility>

#include "gbmd_internal.cuh"

namespace gbmd {

int grid_dims(const double lo[3], const double hi[3], double R, int nc[3]) {
  for (int d = 0; d < 3; ++d) {
    const double L = hi[d] - lo[d];
    if (!(L > 0.0) || !(R > 0.0)) return -1;
    double q = floor(L / (R * (1.0 + 0x1p-40)));
    if (q < 1.0) return -2;
    if (q > 1024.0) q = 1024.0;
    nc[d] = (int)q;
  }
  return 0;
}

struct BoxArgs {
  double lo[3], hi[3], L[3], inv_h[3];
  int nc[3];
};

__global__ void k_wrap_bin(int64_t n, double* __restrict__ x, double* __restrict__ y,
                           double* __restrict__ z, BoxArgs b, int32_t* __restrict__ cell_of,
                           int32_t* __restrict__ cell_count, int* __restrict__ err, const int* __restrict__ gate) {
  if (gate && !*gate) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
  double* r[3] = {x, y, z};
  int c[3];
  bool lost = false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double v = r[d][i];
    if (v < b.lo[d]) v = __dadd_rn(v, b.L[d]);
    else if (v >= b.hi[d]) v = __dsub_rn(v, b.L[d]);
    if (!(v >= b.lo[d] && v < b.hi[d])) lost = true;
    r[d][i] = v;
    int q = (int)__dmul_rn(__dsub_rn(v, b.lo[d]), b.inv_h[d]);
    q = q < 0 ? 0 : (q > b.nc[d] - 1 ? b.nc[d] - 1 : q);
    c[d] = q;
  }
  if (lost) {
    atomicAdd(&err[ERRW_LOST], 1);
    atomicOr(&err[ERRW_FLAGS], GBMD_DEVERR_LOST_ATOM);
  }
  const int32_t lin = (int32_t)(((int64_t)c[2] * b.nc[1] + c[1]) * b.nc[0] + c[0]);
  cell_of[i] = lin;
  // atoms stay cell-sorted between rebuilds, so a warp's 32 atoms fall into
  // a few cells: one atomic per cell and warp
  const unsigned peers = __match_any_sync(__activemask(), lin);
  if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&cell_count[lin], __popc(peers));
  }
}

// --- exclusive scan (256 threads x 8 items per block) ----------------------
constexpr int SCAN_T = 256, SCAN_I = 8, SCAN_B = SCAN_T * SCAN_I;

__device__ __forceinline__ int block_exclusive(int v, int* smem, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) smem[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? smem[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < (int)(blockDim.x >> 5)) smem[lane] = wi - w;
    if (lane == 31) smem[32] = wi;
  }
  __syncthreads();
  total = smem[32];
  const int r = smem[wid] + inc - v;
  __syncthreads();
  return r;
}

// in[0..n) -> out[0..n] exclusive (out[n] = total when this block holds n)
__global__ void k_scan_block(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                             int32_t* __restrict__ sums, const int* __restrict__ gate) {
  if (gate && !*gate) return;  // uniform per block
  __shared__ int smem[33];
  const int64_t base = (int64_t)blockIdx.x * SCAN_B + (int64_t)threadIdx.x * SCAN_I;
  int it[SCAN_I];
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_I; ++k) {
    const int64_t q = base + k;
    it[k] = q < n ? in[q] : 0;
    s += it[k];
  }
  int total;
  int off = block_exclusive(s, smem, total);
#pragma unroll
  for (int k = 0; k < SCAN_I; ++k) {
    const int64_t q = base + k;
    if (q <= n) out[q] = off;
    off += it[k];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int32_t* sums, int nb, const int* __restrict__ gate) {
  if (gate && !*gate) return;
  __shared__ int smem[33];
  int carry = 0;
  for (int base = 0; base < nb; base += SCAN_B) {
    int it[SCAN_I];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k) {
      const int q = base + threadIdx.x * SCAN_I + k;
      it[k] = q < nb ? sums[q] : 0;
      s += it[k];
    }
    int total;
    int off = block_exclusive(s, smem, total);
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k) {
      const int q = base + threadIdx.x * SCAN_I + k;
      if (q < nb) sums[q] = off + carry;
      off += it[k];
    }
    carry += total;
  }
}

__global__ void k_scan_add(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ sums,
                           const int* __restrict__ gate) {
  if (gate && !*gate) return;
  const int64_t base = (int64_t)blockIdx.x * SCAN_B;
  const int add = sums[blockIdx.x];
  for (int k = threadIdx.x; k < SCAN_B; k += blockDim.x) {
    const int64_t q = base + k;
    if (q <= n) out[q] += add;
  }
}

static int scan(gbmd_context* c, const int32_t* in, int32_t* out, int64_t n, const int* gate) {
  const int64_t nb = (n + 1 + SCAN_B - 1) / SCAN_B;
  if (c->scan_cap < nb) {
    if (c->scan_tmp) cudaFree(c->scan_tmp);
    GBMD_CUDA(c, cudaMalloc(&c->scan_tmp, sizeof(int32_t) * nb));
    c->scan_cap = nb;
  }
  k_scan_block<<<(unsigned)nb, SCAN_T, 0, c->stream>>>(in, out, n, c->scan_tmp, gate);
  k_scan_sums<<<1, SCAN_T, 0, c->stream>>>(c->scan_tmp, (int)nb, gate);
  k_scan_add<<<(unsigned)nb, SCAN_T, 0, c->stream>>>(out, n, c->scan_tmp, gate);
  return GBMD_OK;
}

__global__ void k_scatter(int64_t n, const int32_t* __restrict__ cell_of, const int32_t* __restrict__ cstart,
                          int32_t* __restrict__ fill, int32_t* __restrict__ order, const int* __restrict__ gate) {
  if (gate && !*gate) return;
  const int lane = threadIdx.x & 31;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t cl = cell_of[i];
    // one atomic per cell and warp; the order inside a cell is fixed later
    // by k_cell_rank, so any slot assignment will do
    const unsigned peers = __match_any_sync(__activemask(), cl);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&fill[cl], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    order[cstart[cl] + base + __popc(peers & ((1u << lane) - 1u))] = (int32_t)i;
  }
}

// one warp per cell: rank by (id, upload index) -> src[new] = old
__global__ void k_cell_rank(int64_t ncells, const int32_t* __restrict__ cstart, const int32_t* __restrict__ order,
                            const uint64_t* __restrict__ id, const int32_t* __restrict__ user,
                            int32_t* __restrict__ src, const int* __restrict__ gate) {
  const int lane = threadIdx.x & 31;
  if (gate && !*gate) return;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t cell = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; cell < ncells; cell += warps) {
  const int beg = cstart[cell], m = cstart[cell + 1] - beg;
  if (m <= 32) {
    // keys in registers, compared through shuffles
    int32_t a = 0, ua = 0;
    uint64_t ka = 0;
    if (lane < m) {
      a = order[beg + lane];
      ka = id[a];
      ua = user[a];
    }
    int rank = 0;
    for (int f = 0; f < m; ++f) {
      const uint64_t kb = __shfl_sync(0xffffffffu, ka, f);
      const int32_t ub = __shfl_sync(0xffffffffu, ua, f);
      rank += (kb < ka) || (kb == ka && ub < ua);
    }
    if (lane < m) src[beg + rank] = a;
    continue;
  }
  for (int e = lane; e < m; e += 32) {
    const int32_t a = order[beg + e];
    const uint64_t ka = id[a];
    const int32_t ua = user[a];
    int rank = 0;
    for (int f = 0; f < m; ++f) {
      const int32_t b = order[beg + f];
      const uint64_t kb = id[b];
      rank += (kb < ka) || (kb == ka && user[b] < ua);
    }
    src[beg + rank] = a;
  }
  }
}

struct GatherArgs {
  const double *r0, *v0, *a0;
  double *r1, *v1, *a1;
  const uint8_t* t0;
  uint8_t* t1;
  const uint64_t* i0;
  uint64_t* i1;
  const int32_t* u0;
  int32_t* u1;
  const double* ep0;
  double* ep1;
  int64_t cap;
};

__global__ void k_gather(int64_t n, const int32_t* __restrict__ src, GatherArgs g,
                         const int32_t* __restrict__ cell_of, int ncx, int ncy,
                         int32_t* __restrict__ cellpack, const int* __restrict__ gate) {
  if (gate && !*gate) return;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
  const int64_t o = src[p];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    g.r1[d * g.cap + p] = g.r0[d * g.cap + o];
    g.v1[d * g.cap + p] = g.v0[d * g.cap + o];
    g.a1[d * g.cap + p] = g.a0[d * g.cap + o];
  }
  g.t1[p] = g.t0[o];
  g.i1[p] = g.i0[o];
  g.u1[p] = g.u0[o];
  g.ep1[p] = g.ep0[o];
  const int32_t lin = cell_of[o];
  const int cx = lin % ncx, cy = (lin / ncx) % ncy, cz = lin / (ncx * ncy);
  cellpack[p] = cx | (cy << 10) | (cz << 20);
  }
}

// gated variant only: the sorted state, gathered into the spare buffers, is
// copied back so the current buffer index does not change
__global__ void k_copy_back(int64_t n, GatherArgs g, const int* __restrict__ gate) {
  if (!*gate) return;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
  double* r0 = const_cast<double*>(g.r0);
  double* v0 = const_cast<double*>(g.v0);
  double* a0 = const_cast<double*>(g.a0);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    r0[d * g.cap + p] = g.r1[d * g.cap + p];
    v0[d * g.cap + p] = g.v1[d * g.cap + p];
    a0[d * g.cap + p] = g.a1[d * g.cap + p];
  }
  const_cast<uint8_t*>(g.t0)[p] = g.t1[p];
  const_cast<uint64_t*>(g.i0)[p] = g.i1[p];
  const_cast<int32_t*>(g.u0)[p] = g.u1[p];
  const_cast<double*>(g.ep0)[p] = g.ep1[p];
  }
}

__global__ void k_fill_gated(int32_t* __restrict__ p, int64_t n, const int* __restrict__ gate) {
  if (!*gate) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = 0;
}

__global__ void k_posf(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                       const double* __restrict__ z, const uint8_t* __restrict__ type,
                       const int32_t* __restrict__ cellpack, Grid g, float4* __restrict__ pf,
                       double4_32a* __restrict__ pd, const int* __restrict__ gate) {
  if (gate && !*gate) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
  const int cp = cellpack[i];
  const double cx = (double)(cp & 1023), cy = (double)((cp >> 10) & 1023), cz = (double)(cp >> 20);
  const double xi = x[i], yi = y[i], zi = z[i];
  const int t = type[i];
  pf[i] = make_float4((float)(xi - cx * g.h[0] - g.lo[0]), (float)(yi - cy * g.h[1] - g.lo[1]),
                      (float)(zi - cz * g.h[2] - g.lo[2]), __int_as_float(t));
  pd[i] = make_double4_32a(xi, yi, zi, (double)t);
  }
}

// FP64 re-test of a candidate whose FP32 d2 fell within 2^-12 of R^2.  Out of
// line so the compiler cannot predicate it into every iteration of the
// candidate loop (it runs for ~1e-4 of the candidates).
__device__ __noinline__ bool exact_within(const double* __restrict__ x, const double* __restrict__ y,
                                          const double* __restrict__ z, int64_t i, int64_t k, uint32_t code,
                                          int cx, int cy, int cz, const Grid g, double R2) {
  const int nxi = image_of(cx, int(code & 3u) - 1, g.nc[0]);
  const int nyi = image_of(cy, int((code >> 2) & 3u) - 1, g.nc[1]);
  const int nzi = image_of(cz, int((code >> 4) & 3u) - 1, g.nc[2]);
  double a, b, c;
  return exact_d2(x[i], y[i], z[i], x[k], y[k], z[k], (double)nxi * g.L[0], (double)nyi * g.L[1],
                  (double)nzi * g.L[2], a, b, c) <= R2;
}

constexpr int BUILD_CHUNK = 64;  // candidates staged per chunk
constexpr int BUILD_WARPS = 4;   // warps per block

// Per-warp state of the candidate walk shared by both groupings.
struct BuildCell {
  int cx, cy, cz, total, hb, nh;
  int s_start, s_pre;
  uint32_t s_code;
  float s_sx, s_sy, s_sz;
};

// Stage candidates q0 .. q0+63 (position shifted into the home cell's frame,
// index | stencil code << 26) into this warp's shared-memory buffer, keeping
// in order only those within reach of the home group's bounding box
// [blo, bhi] (box distance^2 <= R2keep); the rest cannot pair with any home
// atom of the group (about a quarter of the candidates: the far parts of the
// edge and corner cells).  Returns the number kept; stage[kept] is a sentinel.
__device__ __forceinline__ int build_stage(const BuildCell& B, const float4* __restrict__ pf, int q0,
                                           float4* stage, int lane, const float3& blo, const float3& bhi,
                                           float R2keep) {
  const unsigned FULL = 0xffffffffu;
  const float FAR = 1e18f;
  int kept = 0;
#pragma unroll
  for (int r = 0; r < BUILD_CHUNK / 32; ++r) {
    const int q = q0 + r * 32 + lane;
    // stencil cell of candidate q: largest s with s_pre(s) <= q (5-step search)
    int sc = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int t = min(sc + step, 26);
      const int pv = __shfl_sync(FULL, B.s_pre, t);
      if (sc + step <= 26 && pv <= q) sc = t;
    }
    const int k = __shfl_sync(FULL, B.s_start, sc) + (q - __shfl_sync(FULL, B.s_pre, sc));
    const uint32_t code = __shfl_sync(FULL, B.s_code, sc);
    const float sx = __shfl_sync(FULL, B.s_sx, sc), sy = __shfl_sync(FULL, B.s_sy, sc),
                sz = __shfl_sync(FULL, B.s_sz, sc);
    float4 e = make_float4(FAR, FAR, FAR, __uint_as_float(0xffffffffu));
    bool keep = false;
    if (q < B.total) {
      const float4 pj = pf[k];
      e = make_float4(__fadd_rn(pj.x, sx), __fadd_rn(pj.y, sy), __fadd_rn(pj.z, sz),
                      __uint_as_float((uint32_t)k | (code << GBMD_IDX_BITS)));
      const float bx = fmaxf(0.f, fmaxf(blo.x - e.x, e.x - bhi.x));
      const float by = fmaxf(0.f, fmaxf(blo.y - e.y, e.y - bhi.y));
      const float bz = fmaxf(0.f, fmaxf(blo.z - e.z, e.z - bhi.z));
      keep = fmaf(bx, bx, fmaf(by, by, bz * bz)) <= R2keep;
    }
    const unsigned km = __ballot_sync(FULL, keep);
    if (keep) stage[kept + __popc(km & ((1u << lane) - 1u))] = e;
    kept += __popc(km);
  }
  if (lane == 0) stage[kept] = make_float4(FAR, FAR, FAR, __uint_as_float(0xffffffffu));
  return kept;
}

// Deferred FP64 re-test of an atom's band entries: recompute each entry's
// FP32 d2 with the rounded operations of the staging and the walk, re-test
// the band ones and compact the row in place.  Returns the entries dropped.
__device__ __noinline__ int build_retest_row(uint32_t* row, int nkeep, int wsh, int W, int64_t stride,
                                             const float4* __restrict__ pf, float4 pi, const double* __restrict__ x,
                                             const double* __restrict__ y, const double* __restrict__ z, int i,
                                             int cx, int cy, int cz, const Grid g, double R2, float R2lo) {
  int wpos = 0;
  for (int p = 0; p < nkeep; ++p) {
    const uint32_t w = row[(size_t)(p >> wsh) * stride + (p & (W - 1))];
    const int k = (int)(w & GBMD_IDX_MASK);
    const uint32_t code = w >> GBMD_IDX_BITS;
    const float4 pj = pf[k];
    const float sx = __fmul_rn((float)((int)(code & 3u) - 1), g.hf[0]);
    const float sy = __fmul_rn((float)((int)((code >> 2) & 3u) - 1), g.hf[1]);
    const float sz = __fmul_rn((float)((int)(code >> 4) - 1), g.hf[2]);
    const float dx = __fsub_rn(__fadd_rn(pj.x, sx), pi.x);
    const float dy = __fsub_rn(__fadd_rn(pj.y, sy), pi.y);
    const float dz = __fsub_rn(__fadd_rn(pj.z, sz), pi.z);
    const float d2f = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
    bool keepit = true;
    if (d2f >= R2lo) keepit = exact_within(x, y, z, i, k, code, cx, cy, cz, g, R2);
    if (keepit) {
      row[(size_t)(wpos >> wsh) * stride + (wpos & (W - 1))] = w;
      ++wpos;
    }
  }
  return nkeep - wpos;
}

// The walk for home groups of G atoms: G = 32, one home atom per lane and one
// candidate per step; G = 16, lanes l and l+16 hold the same home atom and a
// step tests candidates 2t (low half) and 2t+1 (high half), the two lanes
// exchanging their hit with one shuffle so both append in candidate order.
// HALF keeps only candidates after the home atom in cell order (k > i): each
// unordered pair once, for the Newton-3 force kernels.
template <int G, bool HALF>
__device__ __forceinline__ int build_walk(const BuildCell& B, const float4* __restrict__ pf,
                                          const double* __restrict__ x, const double* __restrict__ y,
                                          const double* __restrict__ z, const Grid& g, double R2, float R2lo,
                                          float R2hi, uint32_t* __restrict__ nbr, int32_t* __restrict__ nnb,
                                          int maxnb, int W, int wsh, int64_t stride, int* __restrict__ err,
                                          float4* stage, int lane) {
  const unsigned FULL = 0xffffffffu;
  const float FAR = 1e18f;
  const int half = G == 16 ? (lane >> 4) : 0;
  const int hl = G == 16 ? (lane & 15) : lane;
  // box distance bound with a margin far above the FP32 rounding of the
  // walk's d2, so no candidate the walk would keep is dropped
  const float R2keep = R2hi * (1.0f + 0x1p-10f);
  int warp_max = 0;
  for (int h0 = 0; h0 < B.nh; h0 += G) {
    const bool hv = h0 + hl < B.nh;
    const int i = B.hb + h0 + hl;
    float4 pi = make_float4(FAR, FAR, FAR, 0.f);
    if (hv) pi = pf[i];
    // bounding box of the group's home atoms (cell frame)
    float3 blo = make_float3(hv ? pi.x : FAR, hv ? pi.y : FAR, hv ? pi.z : FAR);
    float3 bhi = make_float3(hv ? pi.x : -FAR, hv ? pi.y : -FAR, hv ? pi.z : -FAR);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      blo.x = fminf(blo.x, __shfl_xor_sync(FULL, blo.x, o));
      blo.y = fminf(blo.y, __shfl_xor_sync(FULL, blo.y, o));
      blo.z = fminf(blo.z, __shfl_xor_sync(FULL, blo.z, o));
      bhi.x = fmaxf(bhi.x, __shfl_xor_sync(FULL, bhi.x, o));
      bhi.y = fmaxf(bhi.y, __shfl_xor_sync(FULL, bhi.y, o));
      bhi.z = fmaxf(bhi.z, __shfl_xor_sync(FULL, bhi.z, o));
    }
    uint32_t* row = nbr + (size_t)i * W;  // slot k at row[(k >> wsh) * stride + (k & (W - 1))]
    int cnt = 0;
    bool unc = false;
    for (int q0 = 0; q0 < B.total; q0 += BUILD_CHUNK) {
      __syncwarp();
      const int m = build_stage(B, pf, q0, stage, lane, blo, bhi, R2keep);
      __syncwarp();
#pragma unroll 8
      for (int t = 0; t < m; t += (G == 16 ? 2 : 1)) {
        const float4 e = stage[t + half];
        const uint32_t w = __float_as_uint(e.w);
        const float dx = __fsub_rn(e.x, pi.x);
        const float dy = __fsub_rn(e.y, pi.y);
        const float dz = __fsub_rn(e.z, pi.z);
        const float d2f = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
        // an atom never pairs with itself: its images sit at least one box
        // edge >= R away, so k == i only ever matters in the home cell.
        // Keep d2 <= R^2 (1 + 2^-12); flag the atom when d2 >= R^2 (1 - 2^-12).
        const int k = (int)(w & GBMD_IDX_MASK);
        const bool in = hv && (HALF ? k > i : k != i) && d2f <= R2hi;
        unc |= in && d2f >= R2lo;
        // the slot address is formed on every step and only the store is
        // conditional, so the walk stays one straight-line block
        if (G == 16) {
          const int other = __shfl_xor_sync(FULL, (int)in, 16);
          const int pos = cnt + (half & other);  // candidate 2t goes first
          uint32_t* dst = row + (size_t)(pos >> wsh) * stride + (pos & (W - 1));
          if (in && pos < maxnb) *dst = w;
          cnt += (int)in + other;
        } else {
          uint32_t* dst = row + (size_t)(cnt >> wsh) * stride + (cnt & (W - 1));
          if (in && cnt < maxnb) *dst = w;
          cnt += (int)in;
        }
      }
    }
    if (G == 16) {
      // the shuffle runs on every lane (a short-circuit here would skip it)
      const int partner_unc = __shfl_xor_sync(FULL, (int)unc, 16);
      unc = unc || partner_unc != 0;
      __syncwarp();  // the high-half lanes' entries are visible to the low half
      if (half == 0 && unc) cnt -= build_retest_row(row, min(cnt, maxnb), wsh, W, stride, pf, pi, x, y, z, i,
                                                    B.cx, B.cy, B.cz, g, R2, R2lo);
      cnt = __shfl_sync(FULL, cnt, hl);  // the high-half lane takes the corrected count
    } else if (unc) {
      cnt -= build_retest_row(row, min(cnt, maxnb), wsh, W, stride, pf, pi, x, y, z, i, B.cx, B.cy, B.cz, g,
                              R2, R2lo);
    }
    if (hv && half == 0) {
      nnb[i] = cnt;
      if (cnt > maxnb) atomicOr(&err[ERRW_FLAGS], GBMD_DEVERR_NBR_OVERFLOW);
      warp_max = max(warp_max, cnt);
    }
  }
  return warp_max;
}

// One warp per home cell.  Lane s < 27 describes stencil cell s (start,
// count, code, FP32 shift); the 27 candidate ranges are concatenated in
// stencil order and staged 64 at a time in shared memory, every candidate is
// read as a shared-memory broadcast and tested against the home atoms held
// in the lanes, hits are appended in candidate order -- the canonical order
// (stencil code, then cell order) -- straight to the atoms' list rows.  Cells
// of at most 16 atoms use the 16-atom grouping (two candidates per step),
// fuller cells the 32-atom one.  The walk keeps every candidate with FP32
// d2 <= R^2 (1 + 2^-12) and flags the atom when one lies above
// R^2 (1 - 2^-12); flagged atoms (a few per cent) rescan their row, re-test
// those entries in FP64 and compact, so the walk has no call and no
// divergent branch.
template <bool LOOP, bool HALF>
__global__ void __launch_bounds__(BUILD_WARPS * 32) k_build_list_cells(
    int64_t ncells, const float4* __restrict__ pf, const double* __restrict__ x, const double* __restrict__ y,
    const double* __restrict__ z, const int32_t* __restrict__ cstart, Grid g, double R2, float R2lo, float R2hi,
    uint32_t* __restrict__ nbr, int32_t* __restrict__ nnb, int maxnb, int W, int64_t stride,
    int* __restrict__ err, const int* __restrict__ gate) {
  const int lane = threadIdx.x & 31;
  if (gate && !*gate) return;
  const unsigned FULL = 0xffffffffu;
  __shared__ float4 stage_all[BUILD_WARPS][BUILD_CHUNK + 1];
  float4* stage = stage_all[threadIdx.x >> 5];
  int wsh = 0;
  while ((1 << wsh) < W) ++wsh;
  // one cell per warp (LOOP: and per iteration, striding over the cells;
  // used by the gated launch with its capped grid)
  const int64_t warps = LOOP ? (int64_t)gridDim.x * (blockDim.x >> 5) : ncells;
  for (int64_t cell = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cell < ncells; cell += warps) {
  BuildCell B;
  B.cx = (int)(cell % g.nc[0]);
  B.cy = (int)((cell / g.nc[0]) % g.nc[1]);
  B.cz = (int)(cell / ((int64_t)g.nc[0] * g.nc[1]));
  // stencil cell of this lane
  int s_cnt = 0;
  B.s_start = 0;
  B.s_code = 0;
  B.s_sx = B.s_sy = B.s_sz = 0.f;
  if (lane < 27) {
    const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
    const int nx = image_of(B.cx, dx, g.nc[0]), ny = image_of(B.cy, dy, g.nc[1]), nz = image_of(B.cz, dz, g.nc[2]);
    const int64_t cj = ((int64_t)(B.cz + dz - nz * g.nc[2]) * g.nc[1] + (B.cy + dy - ny * g.nc[1])) * g.nc[0] +
                       (B.cx + dx - nx * g.nc[0]);
    B.s_start = cstart[cj];
    s_cnt = cstart[cj + 1] - B.s_start;
    B.s_code = (uint32_t)(dx + 1) | ((uint32_t)(dy + 1) << 2) | ((uint32_t)(dz + 1) << 4);
    B.s_sx = __fmul_rn((float)dx, g.hf[0]);
    B.s_sy = __fmul_rn((float)dy, g.hf[1]);
    B.s_sz = __fmul_rn((float)dz, g.hf[2]);
  }
  int incl = s_cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  B.s_pre = incl - s_cnt;  // exclusive prefix of this lane's stencil cell
  B.total = __shfl_sync(FULL, incl, 26);
  B.hb = cstart[cell];
  B.nh = cstart[cell + 1] - B.hb;
  int warp_max;
  if (B.nh <= 16)
    warp_max = build_walk<16, HALF>(B, pf, x, y, z, g, R2, R2lo, R2hi, nbr, nnb, maxnb, W, wsh, stride, err, stage, lane);
  else
    warp_max = build_walk<32, HALF>(B, pf, x, y, z, g, R2, R2lo, R2hi, nbr, nnb, maxnb, W, wsh, stride, err, stage, lane);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) warp_max = max(warp_max, __shfl_xor_sync(FULL, warp_max, o));
  if (lane == 0 && warp_max > 0) atomicMax(&err[ERRW_MAXNB], warp_max);
  __syncwarp();  // the next cell restages this warp's buffer
  }
}

static inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

// Blocks of a rebuild-chain launch.  Ungated launches cover the data once;
// gated ones (launched every step, mostly to find the gate closed) get at most
// per_sm blocks per SM (no more than fit at once) and stride over the data,
// so a closed gate costs a few microseconds instead of a full grid of empty
// blocks.
unsigned chain_blocks(const gbmd_context* c, int64_t items, int per_block, const int* gate, int per_sm) {
  const unsigned full = nblk(items, per_block);
  if (!gate || c->full_chain_grids) return full;
  const unsigned cap = (unsigned)(per_sm * (c->nsm > 0 ? c->nsm : 1));
  return full < cap ? full : cap;
}

void launch_posf(gbmd_context* c, const int* gate) {
  if (c->n == 0) return;
  k_posf<<<chain_blocks(c, c->n, 256, gate, 8), 256, 0, c->stream>>>(c->n, c->X(), c->Y(), c->Z(), c->TYPE(),
                                                                   c->cellpack, c->grid, c->POSF(), c->POSD(),
                                                                   gate);
}

static int build_list(gbmd_context* c, const int* gate) {
  const double R = c->rlist;
  const double R2 = R * R;
  const float R2lo = (float)(R2 * (1.0 - 0x1p-12));
  const float R2hi = (float)(R2 * (1.0 + 0x1p-12));
  const int64_t npad = ((c->n + 31) / 32) * 32;
  const int W = list_width(c);
  const int64_t stride = npad * W;
  const int64_t need = (int64_t)(c->maxnb / W) * stride;
  if (need > c->nbr_cap) {
    if (c->nbr) cudaFree(c->nbr);
    c->nbr = nullptr;
    GBMD_CUDA(c, cudaMalloc(&c->nbr, sizeof(uint32_t) * (size_t)need));
    c->nbr_cap = need;
  }
  c->npad = npad;
  if (!gate) GBMD_CUDA(c, cudaMemsetAsync(c->d_err + ERRW_MAXNB, 0, sizeof(int), c->stream));
  const bool loop = gate && !c->full_chain_grids;  // capped grid striding over the cells (five blocks per SM fit)
  const unsigned blocks = loop ? chain_blocks(c, c->grid.ncells, BUILD_WARPS, gate, 5) : nblk(c->grid.ncells, BUILD_WARPS);
  auto kern = loop ? (c->newton3 ? k_build_list_cells<true, true> : k_build_list_cells<true, false>)
                   : (c->newton3 ? k_build_list_cells<false, true> : k_build_list_cells<false, false>);
  kern<<<blocks, 32 * BUILD_WARPS, 0, c->stream>>>(c->grid.ncells, c->POSF(), c->X(), c->Y(), c->Z(), c->cell_start,
                                                  c->grid, R2, R2lo, R2hi, c->nbr, c->nnb, c->maxnb, W, stride,
                                                  c->d_err, gate);
  return GBMD_OK;
}

// The rebuild chain for the list in c->nbr / c->nnb / c->maxnb at radius
// c->rlist (the outer list's buffers and radius while an OuterScope holds).
static int rebuild_chain(gbmd_context* c, bool check_capacity, const int* gate) {
  if (gate && (!c->list_valid || !c->grid_valid || c->maxnb <= 0))
    return set_error(c, GBMD_ERR_INVALID, "gated rebuild needs a built list");
  if (!c->box_set) return set_error(c, GBMD_ERR_INVALID, "box not set");
  if (c->pot == GBMD_POT_NONE) return set_error(c, GBMD_ERR_INVALID, "no potential set");
  if (c->n == 0) {
    c->list_valid = true;
    return GBMD_OK;
  }
  const double R = c->rlist;
  if (!c->grid_valid) {
    int nc[3];
    const int rc = grid_dims(c->lo, c->hi, R, nc);
    if (rc != 0)
      return set_error(c, GBMD_ERR_INVALID, "box edge shorter than neighbour radius %g%s", R,
                       c->list_buffer > 0.0 ? " (list radius + list buffer)" : "");
    Grid& g = c->grid;
    g.ncells = (int64_t)nc[0] * nc[1] * nc[2];
    if (g.ncells > (1ll << 27)) return set_error(c, GBMD_ERR_TOO_LARGE, "too many cells");
    for (int d = 0; d < 3; ++d) {
      g.nc[d] = nc[d];
      g.L[d] = c->hi[d] - c->lo[d];
      g.h[d] = g.L[d] / nc[d];
      g.hf[d] = (float)g.h[d];
      g.lo[d] = c->lo[d];
    }
    if (c->cells_cap < g.ncells + 1) {
      if (c->cell_start) cudaFree(c->cell_start);
      if (c->cell_fill) cudaFree(c->cell_fill);
      GBMD_CUDA(c, cudaMalloc(&c->cell_start, sizeof(int32_t) * (g.ncells + 1)));
      GBMD_CUDA(c, cudaMalloc(&c->cell_fill, sizeof(int32_t) * (g.ncells + 1)));
      c->cells_cap = g.ncells + 1;
    }
    c->grid_valid = true;
  }
  Grid& g = c->grid;
  BoxArgs b;
  for (int d = 0; d < 3; ++d) {
    b.lo[d] = c->lo[d];
    b.hi[d] = c->hi[d];
    b.L[d] = g.L[d];
    b.inv_h[d] = (double)g.nc[d] / g.L[d];
    b.nc[d] = g.nc[d];
  }
  const int64_t n = c->n;
  cudaStream_t s = c->stream;
  auto zero_fill = [&]() -> int {
    if (gate) k_fill_gated<<<chain_blocks(c, g.ncells + 1, 256, gate, 8), 256, 0, s>>>(c->cell_fill, g.ncells + 1, gate);
    else GBMD_CUDA(c, cudaMemsetAsync(c->cell_fill, 0, sizeof(int32_t) * (g.ncells + 1), s));
    return GBMD_OK;
  };
  int rc = zero_fill();
  if (rc) return rc;
  k_wrap_bin<<<chain_blocks(c, n, 256, gate, 8), 256, 0, s>>>(n, c->X(), c->Y(), c->Z(), b, c->cell_of, c->cell_fill,
                                                            c->d_err, gate);
  if ((rc = scan(c, c->cell_fill, c->cell_start, g.ncells, gate))) return rc;
  if ((rc = zero_fill())) return rc;
  k_scatter<<<chain_blocks(c, n, 256, gate, 8), 256, 0, s>>>(n, c->cell_of, c->cell_start, c->cell_fill, c->order,
                                                           gate);
  k_cell_rank<<<chain_blocks(c, g.ncells * 32, 256, gate, 8), 256, 0, s>>>(g.ncells, c->cell_start, c->order, c->ID(),
                                                                       c->USER(),
                                                        c->src, gate);
  GatherArgs ga;
  const int o = c->cur, os = c->cur_s;
  ga.r0 = c->rbuf[o]; ga.r1 = c->rbuf[o ^ 1];
  ga.v0 = c->vbuf[os]; ga.v1 = c->vbuf[os ^ 1];
  ga.a0 = c->abuf[os]; ga.a1 = c->abuf[os ^ 1];
  ga.t0 = c->typeb[os]; ga.t1 = c->typeb[os ^ 1];
  ga.i0 = c->idb[os]; ga.i1 = c->idb[os ^ 1];
  ga.u0 = c->userb[os]; ga.u1 = c->userb[os ^ 1];
  ga.ep0 = c->ep; ga.ep1 = c->stage;
  ga.cap = c->cap;
  k_gather<<<chain_blocks(c, n, 256, gate, 8), 256, 0, s>>>(n, c->src, ga, c->cell_of, g.nc[0], g.nc[1], c->cellpack,
                                                          gate);
  if (gate) {
    k_copy_back<<<chain_blocks(c, n, 256, gate, 8), 256, 0, s>>>(n, ga, gate);
  } else {
    GBMD_CUDA(c, cudaMemcpyAsync(c->ep, c->stage, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    c->cur ^= 1;
    c->cur_s ^= 1;
  }
  launch_posf(c, gate);
  if (c->maxnb <= 0) {
    // first estimate: 1.35x the mean count of an ideal gas at this density
    const double V = g.L[0] * g.L[1] * g.L[2];
    const double mean = (double)n / V * 4.18879020478639 * R * R * R;
    int m = (int)(mean * 1.35) + 16;
    c->maxnb = ((m + list_width(c) - 1) / list_width(c)) * list_width(c);
  }
  rc = build_list(c, gate);
  if (rc) return rc;
  c->list_valid = true;
  if (check_capacity) {
    rc = sync_error_word(c);
    if (c->h_err[ERRW_FLAGS] & GBMD_DEVERR_LOST_ATOM)
      return set_error(c, GBMD_ERR_LOST_ATOM, "%d atoms left the box by more than one image",
                       c->h_err[ERRW_LOST]);
    const int maxc = c->h_err[ERRW_MAXNB];
    if (maxc > c->maxnb) {
      int m = (int)(maxc * 1.2) + 8;
      c->maxnb = ((m + list_width(c) - 1) / list_width(c)) * list_width(c);
      GBMD_CUDA(c, cudaMemsetAsync(c->d_err + ERRW_FLAGS, 0, sizeof(int) * 2, s));  // flags, max count
      rc = build_list(c, nullptr);
      if (rc) return rc;
      rc = sync_error_word(c);
      if (c->h_err[ERRW_FLAGS] & GBMD_DEVERR_NBR_OVERFLOW)
        return set_error(c, GBMD_ERR_NEIGHBOR_OVERFLOW, "neighbour list overflow after regrow");
    }
  }
  return GBMD_OK;
}

// --- two-level list ---------------------------------------------------------
//
// With a list buffer d set, the sort into cells and the cell walk build an
// outer list of radius R + d (R = rcut + skin), and every rebuild filters the
// list the pair kernels read (radius R) from it: the outer row's entries that
// lie within R now, in the outer row's order.  The filter is complete while
// no atom has moved more than d/2 since the outer build: a pair within R now
// was then within R + d.  So a rebuild first tests every atom against d/2
// from its position at the outer build and runs the outer build again only
// when one moved that far.  Between outer builds the atoms keep their cells
// and are not wrapped into the box, so the cell-relative FP32 copies, the
// stencil codes and the FP64 band re-test all see continuous coordinates.
// The filtered list holds the same pairs as a fresh build; its rows follow
// the cell order of the outer build.

bool two_level(const gbmd_context* c) { return c->list_buffer > 0.0; }

void free_outer(gbmd_context* c) {
  cudaFree(c->rout);
  cudaFree(c->nnb_out);
  c->rout = nullptr;
  c->nnb_out = nullptr;
  c->outer_cap = 0;
  c->outer_valid = false;
}

static int ensure_outer(gbmd_context* c) {
  if (c->rout && c->outer_cap >= c->cap) return GBMD_OK;
  free_outer(c);
  GBMD_CUDA(c, cudaMalloc(&c->rout, sizeof(double) * 3 * c->cap));
  GBMD_CUDA(c, cudaMalloc(&c->nnb_out, sizeof(int32_t) * c->cap));
  c->outer_cap = c->cap;
  return GBMD_OK;
}

// The outer list's buffers and radius in the fields the rebuild chain uses.
struct OuterScope {
  gbmd_context* c;
  double saved;
  explicit OuterScope(gbmd_context* ctx) : c(ctx), saved(ctx->rlist) {
    swap();
    c->rlist = saved + c->list_buffer;
  }
  ~OuterScope() {
    c->rlist = saved;
    swap();
  }
  void swap() {
    std::swap(c->nbr, c->nbr_out);
    std::swap(c->nnb, c->nnb_out);
    std::swap(c->nbr_cap, c->nbr_out_cap);
    std::swap(c->maxnb, c->maxnb_out);
  }
};

// flag = 1 when some atom moved more than sqrt(thr2) since the outer build
// (|dr|^2 summed x, y, z without contraction); with a gate, only when *gate
__global__ void k_outer_check(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                              const double* __restrict__ z, const double* __restrict__ rout, int64_t cap,
                              double thr2, const int* __restrict__ gate, int* __restrict__ flag) {
  if (gate && !*gate) return;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const double dx = __dsub_rn(x[p], rout[p]), dy = __dsub_rn(y[p], rout[cap + p]),
                 dz = __dsub_rn(z[p], rout[2 * cap + p]);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (d2 > thr2) *flag = 1;
  }
}

// positions at a gated outer build; thread 0 counts the build
__global__ void k_save_outer(int64_t n, const double* __restrict__ r, double* __restrict__ rout, int64_t cap,
                             const int* __restrict__ gate, int* __restrict__ count) {
  if (!*gate) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(count, 1);
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int d = 0; d < 3; ++d) rout[d * cap + p] = r[d * cap + p];
  }
}

// One thread per atom: the entries of its outer row within R now, in order.
// The FP32 distance of the cell-relative copies (the builder's expression)
// decides outside the band R^2 (1 -+ 2^-12); band entries are re-tested in
// FP64 with the pair-set rounding.  A row never grows, so the list has the
// outer list's capacity.  V4 (rows interleaved in groups of a multiple of 4
// entries): the row is read 4 entries per 16-byte load with the next load in
// flight, and the 4 neighbour positions are gathered together.
struct FilterArgs {
  int64_t n;
  const float4* pf;
  const double *x, *y, *z;
  const int32_t* cellpack;
  const uint32_t* outer;
  const int32_t* nnb_out;
  uint32_t* nbr;
  int32_t* nnb;
  int maxnb_out, W, wsh;
  int64_t stride;
  double R2;
  float R2lo, R2hi;
};

__device__ __forceinline__ bool filter_keep(const FilterArgs& A, const Grid& g, int64_t i, const float4& pi,
                                            uint32_t w, const float4& pj, int cx, int cy, int cz) {
  const uint32_t code = w >> GBMD_IDX_BITS;
  const float sx = __fmul_rn((float)((int)(code & 3u) - 1), g.hf[0]);
  const float sy = __fmul_rn((float)((int)((code >> 2) & 3u) - 1), g.hf[1]);
  const float sz = __fmul_rn((float)((int)(code >> 4) - 1), g.hf[2]);
  const float dx = __fsub_rn(__fadd_rn(pj.x, sx), pi.x);
  const float dy = __fsub_rn(__fadd_rn(pj.y, sy), pi.y);
  const float dz = __fsub_rn(__fadd_rn(pj.z, sz), pi.z);
  const float d2f = fmaf(dx, dx, fmaf(dy, dy, __fmul_rn(dz, dz)));
  if (d2f > A.R2hi) return false;
  if (d2f < A.R2lo) return true;
  return exact_within(A.x, A.y, A.z, i, (int64_t)(w & GBMD_IDX_MASK), code, cx, cy, cz, g, A.R2);
}

template <bool V4>
__global__ void __launch_bounds__(256) k_filter_list(FilterArgs A, Grid g, const int* __restrict__ gate) {
  if (gate && !*gate) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int nn = min(A.nnb_out[i], A.maxnb_out);
    const float4 pi = A.pf[i];
    const int cp = A.cellpack[i];
    const int cx = cp & 1023, cy = (cp >> 10) & 1023, cz = cp >> 20;
    const uint32_t* orow = A.outer + (size_t)i * A.W;
    uint32_t* row = A.nbr + (size_t)i * A.W;
    int cnt = 0;
    auto put = [&](uint32_t w) {
      row[(size_t)(cnt >> A.wsh) * A.stride + (cnt & (A.W - 1))] = w;
      ++cnt;
    };
    if (V4) {
      // slot k at orow[(k >> wsh) * stride + (k & (W - 1))]; W is a multiple
      // of 4, so 4 consecutive slots from a multiple of 4 are one aligned uint4
      // (rows hold maxnb_out slots, a multiple of W: the last load stays in)
      auto group = [&](int k) {
        return *reinterpret_cast<const uint4*>(orow + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
      };
      const int ng = (nn + 3) >> 2;
      uint4 cur = ng > 0 ? group(0) : make_uint4(0u, 0u, 0u, 0u);
      for (int t = 0; t < ng; ++t) {
        const int k0 = t << 2;
        uint4 nxt = cur;
        if (t + 1 < ng) nxt = group(k0 + 4);
        const uint32_t e[4] = {cur.x, cur.y, cur.z, cur.w};
        float4 pj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) pj[q] = A.pf[k0 + q < nn ? (int64_t)(e[q] & GBMD_IDX_MASK) : i];
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (k0 + q < nn && filter_keep(A, g, i, pi, e[q], pj[q], cx, cy, cz)) put(e[q]);
        cur = nxt;
      }
    } else {
      for (int k = 0; k < nn; ++k) {
        const uint32_t w = orow[(size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1))];
        const float4 pj = A.pf[w & GBMD_IDX_MASK];
        if (filter_keep(A, g, i, pi, w, pj, cx, cy, cz)) put(w);
      }
    }
    A.nnb[i] = cnt;
  }
}

// The outer list: the rebuild chain at radius R + d into the outer buffers,
// then the positions it leaves saved for the displacement test.
static int outer_chain(gbmd_context* c, bool check_capacity, const int* gate) {
  int rc;
  if (!gate) {
    if ((rc = ensure_outer(c))) return rc;
  } else if (!c->rout || c->outer_cap < c->n) {
    return set_error(c, GBMD_ERR_INVALID, "gated rebuild needs an outer list");
  }
  {
    const OuterScope on(c);
    rc = rebuild_chain(c, check_capacity, gate);
  }
  if (rc) return rc;
  if (gate) {
    k_save_outer<<<chain_blocks(c, c->n, 256, gate, 8), 256, 0, c->stream>>>(c->n, c->rbuf[c->cur], c->rout, c->cap,
                                                                          gate, c->d_err + ERRW_OUTER_BUILDS);
  } else {
    for (int d = 0; d < 3; ++d)
      GBMD_CUDA(c, cudaMemcpyAsync(c->rout + d * c->cap, c->rbuf[c->cur] + d * c->cap, sizeof(double) * c->n,
                                   cudaMemcpyDeviceToDevice, c->stream));
    c->outer_builds++;
    c->outer_valid = true;
  }
  return GBMD_OK;
}

static int filter_list(gbmd_context* c, const int* gate) {
  const int W = list_width(c);
  int wsh = 0;
  while ((1 << wsh) < W) ++wsh;
  const int64_t stride = c->npad * W;
  const int64_t need = (int64_t)(c->maxnb_out / W) * stride;
  if (need > c->nbr_cap) {
    if (gate || c->capturing) return set_error(c, GBMD_ERR_INVALID, "the list outgrew its buffer in a gated rebuild");
    if (c->nbr) cudaFree(c->nbr);
    c->nbr = nullptr;
    c->nbr_cap = 0;
    GBMD_CUDA(c, cudaMalloc(&c->nbr, sizeof(uint32_t) * (size_t)need));
    c->nbr_cap = need;
  }
  c->maxnb = c->maxnb_out;
  const double R2 = c->rlist * c->rlist;
  const float R2lo = (float)(R2 * (1.0 - 0x1p-12));
  const float R2hi = (float)(R2 * (1.0 + 0x1p-12));
  FilterArgs A;
  A.n = c->n;
  A.pf = c->POSF();
  A.x = c->X(); A.y = c->Y(); A.z = c->Z();
  A.cellpack = c->cellpack;
  A.outer = c->nbr_out;
  A.nnb_out = c->nnb_out;
  A.nbr = c->nbr;
  A.nnb = c->nnb;
  A.maxnb_out = c->maxnb_out;
  A.W = W;
  A.wsh = wsh;
  A.stride = stride;
  A.R2 = R2;
  A.R2lo = R2lo;
  A.R2hi = R2hi;
  const unsigned blocks = gate ? chain_blocks(c, c->n, 256, gate, 8) : nblk(c->n, 256);
  if (W % 4 == 0) k_filter_list<true><<<blocks, 256, 0, c->stream>>>(A, c->grid, gate);
  else k_filter_list<false><<<blocks, 256, 0, c->stream>>>(A, c->grid, gate);
  c->list_valid = true;
  if (!gate) c->list_builds++;
  return GBMD_OK;
}

int rebuild(gbmd_context* c, bool check_capacity, const int* gate) {
  if (c->n == 0 || !two_level(c)) {
    const int rc = rebuild_chain(c, check_capacity, gate);
    if (rc == GBMD_OK && !gate) c->list_builds++;
    return rc;
  }
  if (gate && !c->outer_valid) return set_error(c, GBMD_ERR_INVALID, "gated rebuild needs an outer list");
  const int rc = outer_chain(c, check_capacity, gate);
  if (rc) return rc;
  return filter_list(c, gate);
}

static int outer_body(gbmd_context* c, const int* flag) {
  c->full_chain_grids = true;
  const int rc = outer_chain(c, false, flag);
  c->full_chain_grids = false;
  return rc;
}

int rebuild_two_level(gbmd_context* c, bool check_capacity, const int* gate) {
  if (c->n == 0 || !c->outer_valid || !c->list_valid || !c->grid_valid) {
    if (gate || c->capturing) return set_error(c, GBMD_ERR_INVALID, "gated or captured rebuild needs an outer list");
    return rebuild(c, check_capacity, nullptr);
  }
  int* flag = c->d_err + ERRW_OUTER;
  cudaStream_t s = c->stream;
  GBMD_CUDA(c, cudaMemsetAsync(flag, 0, sizeof(int), s));
  const double h = 0.5 * c->list_buffer;
  const double thr2 = h * h * (1.0 - 0x1p-20);  // a margin far above the rounding of the test
  const unsigned blocks = gate ? chain_blocks(c, c->n, 256, gate, 8) : nblk(c->n, 256);
  k_outer_check<<<blocks, 256, 0, s>>>(c->n, c->X(), c->Y(), c->Z(), c->rout, c->cap, thr2, gate, flag);
  int rc;
  if (gate) {
    // the flag stays 0 unless the gate is open: it gates the outer chain
    rc = outer_chain(c, false, flag);
  } else if (c->capturing) {
    rc = capture_if(c, flag, outer_body);
  } else {
    if ((rc = sync_error_word(c))) return rc;
    rc = c->h_err[ERRW_OUTER] ? outer_chain(c, check_capacity, nullptr) : GBMD_OK;
  }
  if (rc) return rc;
  return filter_list(c, gate);
}

int export_pairs(gbmd_context* c, int64_t cap, uint64_t* id_i, uint64_t* id_j, int8_t* img, int64_t* count) {
  if (!c->list_valid) {
    int rc = rebuild(c, true);
    if (rc) return rc;
  }
  const int64_t n = c->n;
  std::vector<int32_t> nnb(n), cp(n);
  std::vector<uint64_t> ids(n);
  GBMD_CUDA(c, cudaMemcpyAsync(nnb.data(), c->nnb, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
  GBMD_CUDA(c, cudaMemcpyAsync(cp.data(), c->cellpack, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
  GBMD_CUDA(c, cudaMemcpyAsync(ids.data(), c->ID(), sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, c->stream));
  GBMD_CUDA(c, cudaStreamSynchronize(c->stream));
  int64_t total = 0;
  for (int64_t i = 0; i < n; ++i) total += nnb[i];
  *count = total;
  if (cap < total || !id_i) return GBMD_OK;
  const int W = list_width(c);
  const int64_t stride = c->npad * W;
  std::vector<uint32_t> nb((size_t)c->nbr_cap);
  GBMD_CUDA(c, cudaMemcpy(nb.data(), c->nbr, sizeof(uint32_t) * c->nbr_cap, cudaMemcpyDeviceToHost));
  int64_t row = 0;
  const Grid& g = c->grid;
  for (int64_t i = 0; i < n; ++i) {
    const int cx = cp[i] & 1023, cy = (cp[i] >> 10) & 1023, cz = cp[i] >> 20;
    for (int k = 0; k < nnb[i] && k < c->maxnb; ++k) {
      const uint32_t e = nb[(size_t)(k / W) * stride + (size_t)i * W + (k % W)];
      const uint32_t j = e & GBMD_IDX_MASK, code = e >> GBMD_IDX_BITS;
      const int d[3] = {int(code & 3) - 1, int((code >> 2) & 3) - 1, int((code >> 4) & 3) - 1};
      const int cc[3] = {cx + d[0], cy + d[1], cz + d[2]};
      id_i[row] = ids[i];
      id_j[row] = ids[j];
      for (int q = 0; q < 3; ++q) img[3 * row + q] = (int8_t)(cc[q] < 0 ? -1 : (cc[q] >= g.nc[q] ? 1 : 0));
      ++row;
    }
  }
  return GBMD_OK;
}

}  // namespace gbmd
