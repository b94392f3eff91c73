// gbmd_mixed.cu -- mixed-precision pair kernels (FP32 pair arithmetic, FP64
// state) for sm_103a: lj_compute_force / lj_multi_force, and the eam_alloy
// density+embedding and force passes.
//
// Same functions as the FP64 kernels (lennard_jones.h L41-50,
// force_op_impl2.hxx L33-68, pair_potential_force_op_multiparam.h L92-118,
// eam_alloy.h L198-313, eam_force_op_multimat.h L114-343), evaluated on
// home-cell-relative FP32 coordinates: dr = (p_j - p_i) + s*h with s the
// stencil offset of j's cell, exact to ~1e-7 relative.  Forces, densities
// and energies are summed with compensated (Kahan) FP32 sums; per-atom
// results are converted to FP64 once.  Cutoff membership matches FP64
// exactly: pairs with FP32 d2 within 2^-12 of rcut^2 are re-tested in FP64.
//
// Loop structure: each lane reads V list entries with one coalesced load
// (V = 4: 16 B per lane, streamed past L1 so the gathers keep it), the next
// row already in flight; per entry one 16 B position gather (single-element
// EAM force pass: the position carries F'(rho_j) in w), one 16 B spline-knot
// gather per table; branch-free except the rare FP64 re-test.  The V terms
// of a row are added in FP32, the row sum goes into the compensated sum.
// 1/r and r come from one rsqrt; the stencil offset decodes to an exact
// float in two integer/FP ops per axis.
#include <algorithm>
#include <cmath>

#include "gbmd_pair_common.cuh"

namespace gbmd {

struct GeomF {
  float dx, dy, dz, d2;
};

// Exact FP64 cutoff test of a pair whose FP32 d2 fell in the ambiguous band:
// d2 <= rc2 and, for per-pair cutoffs, sqrt(d2) <= rc_pair (the reference's
// two-stage test).  Kept out of line: it runs for ~1e-4 of the pairs.
__device__ __noinline__ bool exact_inside(const double4_32a* __restrict__ posd, int64_t i, uint32_t j,
                                          uint32_t code, int cp, const Grid g, double rc2, double rc_pair) {
  int cx, cy, cz;
  unpack_cell(cp, cx, cy, cz);
  double Sx, Sy, Sz, a, b, c;
  image_shift(g, cx, cy, cz, code, Sx, Sy, Sz);
  const double4_32a di = posd[i], dj = posd[j];
  const double d2 = exact_d2(di.x, di.y, di.z, dj.x, dj.y, dj.z, Sx, Sy, Sz, a, b, c);
  if (!(d2 <= rc2)) return false;
  return rc_pair <= 0.0 || sqrt(d2) <= rc_pair;
}

// {0,1,2} -> -1.f, 0.f, +1.f exactly (small integer through the 2^23 mantissa
// trick); the separation shift is then one FMA per axis.
__device__ __forceinline__ float unit_of(uint32_t b) { return __int_as_float(0x4B000000u | b) - 8388609.0f; }

__device__ __forceinline__ GeomF geom_f(uint32_t ent, const float4& pj, const float4& pi, const Grid& g) {
  GeomF r;
  r.dx = fmaf(unit_of((ent >> 26) & 3u), g.hf[0], pj.x - pi.x);
  r.dy = fmaf(unit_of((ent >> 28) & 3u), g.hf[1], pj.y - pi.y);
  r.dz = fmaf(unit_of(ent >> 30), g.hf[2], pj.z - pi.z);
  r.d2 = fmaf(r.dx, r.dx, fmaf(r.dy, r.dy, r.dz * r.dz));
  return r;
}

// Two list entries at once in packed FP32 (sm_100 float2 arithmetic: one
// instruction per pair of lanes' worth of FADD / FMUL / FFMA).  Each half is
// geom_f of its entry, operation for operation: (p_j - p_i) is p_j + (-p_i),
// which rounds identically.  npi = (-p_i) in both halves of each axis.
struct GeomF2 {
  float2 dx, dy, dz, d2;
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

__device__ __forceinline__ GeomF2 geom_f2(uint32_t ea, uint32_t eb, const float4& pa, const float4& pb,
                                          const float2& npx, const float2& npy, const float2& npz, const float2& hx,
                                          const float2& hy, const float2& hz) {
  GeomF2 r;
  r.dx = __ffma2_rn(f2(unit_of((ea >> 26) & 3u), unit_of((eb >> 26) & 3u)), hx, __fadd2_rn(f2(pa.x, pb.x), npx));
  r.dy = __ffma2_rn(f2(unit_of((ea >> 28) & 3u), unit_of((eb >> 28) & 3u)), hy, __fadd2_rn(f2(pa.y, pb.y), npy));
  r.dz = __ffma2_rn(f2(unit_of(ea >> 30), unit_of(eb >> 30)), hz, __fadd2_rn(f2(pa.z, pb.z), npz));
  r.d2 = __ffma2_rn(r.dx, r.dx, __ffma2_rn(r.dy, r.dy, __fmul2_rn(r.dz, r.dz)));
  return r;
}

// The per-atom constants of geom_f2: -p_i and the cell edges, packed.
struct PairFrame {
  float2 npx, npy, npz, hx, hy, hz;
  __device__ __forceinline__ PairFrame(const float4& pi, const Grid& g)
      : npx(f2(-pi.x, -pi.x)), npy(f2(-pi.y, -pi.y)), npz(f2(-pi.z, -pi.z)), hx(f2(g.hf[0], g.hf[0])),
        hy(f2(g.hf[1], g.hf[1])), hz(f2(g.hf[2], g.hf[2])) {}
  __device__ __forceinline__ GeomF2 geom(uint32_t ea, uint32_t eb, const float4& pa, const float4& pb) const {
    return geom_f2(ea, eb, pa, pb, npx, npy, npz, hx, hy, hz);
  }
};

__device__ __forceinline__ void reduce6(float* v, int T) {
  for (int off = T / 2; off > 0; off >>= 1)
#pragma unroll
    for (int q = 0; q < 6; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
}

__device__ __forceinline__ void vir9(const float* v, double* o) {
  // symmetric pair virial: xx yy zz xy xz yz -> row-major 3x3
  o[0] = v[0]; o[1] = v[3]; o[2] = v[4];
  o[3] = v[3]; o[4] = v[1]; o[5] = v[5];
  o[6] = v[4]; o[7] = v[5]; o[8] = v[2];
}

// The V list entries of lane `lane` in row r of atom i, read with one load
// that bypasses L1 (each entry is used once per kernel).  Entries at or
// beyond nn are replaced by a harmless stand-in: j = i seen through the +x
// stencil offset, a separation of one cell edge (>= rcut + skin), which no
// cutoff test accepts.
template <int T, int V>
struct ListRows {
  static constexpr int W = T * V;
  const uint32_t* p;  // nbr + i*W + lane*V
  int64_t stride;
  int nrow, k0, nn;
  uint32_t standin;
  __device__ __forceinline__ ListRows(const uint32_t* nbr, int64_t i, int lane, int64_t stride_, int nn_)
      : p(nbr + (size_t)i * W + lane * V), stride(stride_), nn(nn_) {
    k0 = lane * V;
    nrow = nn > k0 ? (nn - k0 + W - 1) / W : 0;
    standin = (uint32_t)i | ((2u | (1u << 2) | (1u << 4)) << GBMD_IDX_BITS);
  }
  __device__ __forceinline__ void load(int r, uint32_t (&e)[V]) const {
    const uint32_t* q = p + (size_t)r * stride;
    if constexpr (V == 4) {
      // read once per kernel: keep it out of L1, which serves the gathers
      asm("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
          : "=r"(e[0]), "=r"(e[1]), "=r"(e[2]), "=r"(e[3])
          : "l"(q));
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v) e[v] = __ldcs(q + v);
    }
  }
  __device__ __forceinline__ bool valid(int r, int v) const { return r * W + k0 + v < nn; }
};

// ---------------------------------------------------------------------------
// Neighbour-position sources.  GlobalFetch gathers position j from the
// cell-sorted array; StagedFetch reads it from the block's shared-memory copy
// of the cells around its home cells (see stage_cells): the list entry's
// stencil row (dy, dz) picks one of nine staged row segments, each at most
// two contiguous global ranges (a row wraps at most once in x).
// ---------------------------------------------------------------------------
struct GlobalFetch {
  const float4* __restrict__ P;
  __device__ __forceinline__ float4 operator()(uint32_t ent, uint32_t j) const {
    float4 v;
    asm("ld.global.nc.L1::evict_last.v4.f32 {%0,%1,%2,%3}, [%4];"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(P + j));
    return v;
  }
};

struct StagedFetch {
  const float4* pos;   // staged positions (shared memory)
  const int4* rows;    // 16 entries by (dy+1) | (dz+1) << 2: {delta0, g1, n1, delta1}
  __device__ __forceinline__ float4 operator()(uint32_t ent, uint32_t j) const {
    const int4 t = rows[(ent >> 28) & 15u];
    const int jj = (int)j;
    const int slot = jj - ((unsigned)(jj - t.y) < (unsigned)t.z ? t.w : t.x);
    return pos[slot];
  }
};

// Stage, for the block's K home cells (x0 .. x0+K-1 of row (y, z), taken
// from blockIdx), the positions of every atom of the cells x0-1 .. x0+K in
// the nine rows (y+dy, z+dz) into `pos` and the translation table into
// `rows`; a0 / a1 receive the block's home atom range.  Returns false (then
// the block gathers from global memory) when they exceed `cap` atoms.
__device__ bool stage_cells(const Grid& g, const int32_t* __restrict__ cstart, const float4* __restrict__ src,
                            int K, int cap, float4* pos, int4* rows, int* sh, int64_t& a0, int64_t& a1) {
  const int ncx = g.nc[0], ncy = g.nc[1], ncz = g.nc[2];
  const int x0 = blockIdx.x * K, y = blockIdx.y, z = blockIdx.z;
  const int x1 = min(x0 + K, ncx);  // exclusive
  const int64_t rowbase = ((int64_t)z * ncy + y) * ncx;
  a0 = cstart[rowbase + x0];
  a1 = cstart[rowbase + x1];
  // sh[0..35]: per row s = 0..8, global start / count of range A and B
  if (threadIdx.x < 9) {
    const int s = threadIdx.x, dy = s % 3 - 1, dz = s / 3 - 1;
    const int yy = (y + dy + ncy) % ncy, zz = (z + dz + ncz) % ncz;
    const int64_t rb = ((int64_t)zz * ncy + yy) * ncx;
    int la = 0, ha = ncx - 1, lb = 0, hb = -1;  // inclusive cell ranges; B empty
    if (ncx > x1 - x0 + 2) {
      const int xs = x0 - 1, xe = x1;
      if (xs < 0) { la = ncx - 1; ha = ncx - 1; lb = 0; hb = xe; }
      else if (xe >= ncx) { la = xs; ha = ncx - 1; lb = 0; hb = 0; }
      else { la = xs; ha = xe; }
    }
    const int ga = cstart[rb + la], na = cstart[rb + ha + 1] - ga;
    const int gb = hb >= lb ? cstart[rb + lb] : 0, nb = hb >= lb ? cstart[rb + hb + 1] - gb : 0;
    sh[4 * s] = ga; sh[4 * s + 1] = na; sh[4 * s + 2] = gb; sh[4 * s + 3] = nb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int off = 0;
    for (int q = 0; q < 16; ++q) rows[q] = make_int4(0, 0, 0, 0);
    for (int s = 0; s < 9; ++s) {
      const int ga = sh[4 * s], na = sh[4 * s + 1], gb = sh[4 * s + 2], nb = sh[4 * s + 3];
      const int oa = off, ob = off + na;
      off += na + nb;
      const int key = (s % 3) | ((s / 3) << 2);
      rows[key] = make_int4(ga - oa, gb, nb, gb - ob);
      sh[36 + 2 * s] = oa;
      sh[36 + 2 * s + 1] = ob;
    }
    sh[54] = off;
  }
  __syncthreads();
  const int total = sh[54];
  if (total > cap) return false;  // uniform
  // all copies in flight at once: slot u belongs to the last segment starting
  // at or before it (18 segments A0 B0 A1 B1 ... in staging order)
  for (int u = threadIdx.x; u < total; u += blockDim.x) {
    int seg = 0;
#pragma unroll
    for (int q = 1; q < 18; ++q)
      if (sh[36 + q] <= u) seg = q;
    const int s = seg >> 1, b = seg & 1;
    const int g0 = sh[4 * s + 2 * b];
    const float4* from = &src[g0 + (u - sh[36 + seg])];
    const unsigned to = (unsigned)__cvta_generic_to_shared(&pos[u]);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(to), "l"(from) : "memory");
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  return true;
}

// ---------------------------------------------------------------------------
// Lennard-Jones
// ---------------------------------------------------------------------------
struct LJF {
  float sig2, eps24, eps4, ecut, rc2lo, rc2hi;
  double rc2, rc;
};

struct LJTabSmem {
  float4 a[GBMD_MAX_TYPES * GBMD_MAX_TYPES];   // sig2, eps24, eps4, ecut
  float2 b[GBMD_MAX_TYPES * GBMD_MAX_TYPES];   // rc2lo, rc2hi
  double r[GBMD_MAX_TYPES * GBMD_MAX_TYPES];   // rc
};

__device__ __forceinline__ void lj_load_table(LJTabSmem& t, const LJPair* __restrict__ tab, int ntypes) {
  for (int q = threadIdx.x; q < ntypes * ntypes; q += blockDim.x) {
    const LJPair& p = tab[q];
    t.a[q] = make_float4(p.sig2f, p.eps24f, p.eps4f, p.ecutf);
    t.b[q] = make_float2(p.rc2lo, p.rc2hi);
    t.r[q] = p.rc;
  }
  __syncthreads();
}

template <int T, int V, bool EV, bool MULTI, class Fetch>
__device__ __forceinline__ void lj_atom(const PairArgs& A, const LJF& P, const LJTabSmem& tab, int ntypes,
                                        double rcmax2, int64_t i, int lane, bool live, const Fetch& fetch) {
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  const float4 pi = live ? A.posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int cp = live ? A.cellpack[i] : 0;
  const int ti = __float_as_int(pi.w);
  float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const ListRows<T, V> L(A.nbr, i, lane, A.stride, nn);
  uint32_t ent[V], nxt[V];
  if (L.nrow > 0) L.load(0, ent);
  for (int r = 0; r < L.nrow; ++r) {
    if (r + 1 < L.nrow) L.load(r + 1, nxt);
    float4 pj[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      if (!L.valid(r, q)) ent[q] = L.standin;
      pj[q] = fetch(ent[q], ent[q] & GBMD_IDX_MASK);
    }
    float rx = 0.f, ry = 0.f, rz = 0.f, re = 0.f;
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const uint32_t j = ent[q] & GBMD_IDX_MASK;
      const GeomF G = geom_f(ent[q], pj[q], pi, A.g);
      float sig2, eps24, eps4, ecut, rlo, rhi;
      int pid = 0;
      if (MULTI) {
        pid = ti * ntypes + __float_as_int(pj[q].w);
        const float4 a = tab.a[pid];
        const float2 b = tab.b[pid];
        sig2 = a.x; eps24 = a.y; eps4 = a.z; ecut = a.w; rlo = b.x; rhi = b.y;
      } else {
        sig2 = P.sig2; eps24 = P.eps24; eps4 = P.eps4; ecut = P.ecut; rlo = P.rc2lo; rhi = P.rc2hi;
      }
      bool in = G.d2 < rlo;
      if (!in && G.d2 <= rhi && L.valid(r, q))  // rare: the FP64 per-pair cutoff only here
        in = exact_inside(A.posd, i, j, ent[q] >> GBMD_IDX_BITS, cp, A.g, MULTI ? rcmax2 : P.rc2,
                          MULTI ? tab.r[pid] : 0.0);
      // hardware reciprocal (within 1 ulp): the pair term's error budget is
      // ~1e-7 relative against a 1e-5 force tolerance
      float r2i;
      asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r2i) : "f"(G.d2));
      const float s2 = sig2 * r2i;
      const float s6 = s2 * s2 * s2;
      const float s12 = s6 * s6;
      const float fpair = in ? eps24 * fmaf(2.f, s12, -s6) * r2i : 0.f;  // -(dE/dr)/r
      rx = fmaf(-fpair, G.dx, rx);
      ry = fmaf(-fpair, G.dy, ry);
      rz = fmaf(-fpair, G.dz, rz);
      if (EV) {
        re += in ? 0.5f * fmaf(eps4, s12 - s6, -ecut) : 0.f;
        const float h = 0.5f * fpair;
        v[0] = fmaf(h * G.dx, G.dx, v[0]);
        v[1] = fmaf(h * G.dy, G.dy, v[1]);
        v[2] = fmaf(h * G.dz, G.dz, v[2]);
        v[3] = fmaf(h * G.dx, G.dy, v[3]);
        v[4] = fmaf(h * G.dx, G.dz, v[4]);
        v[5] = fmaf(h * G.dy, G.dz, v[5]);
      }
    }
    kahan_add(fx, cfx, rx);
    kahan_add(fy, cfy, ry);
    kahan_add(fz, cfz, rz);
    if (EV) kahan_add(e, ce, re);
#pragma unroll
    for (int q = 0; q < V; ++q) ent[q] = nxt[q];
  }
  group_reduce_kahan<T>(fx, cfx);
  group_reduce_kahan<T>(fy, cfy);
  group_reduce_kahan<T>(fz, cfz);
  if (EV) {
    group_reduce_kahan<T>(e, ce);
    reduce6(v, T);
  }
  if (live && lane == 0) {
    const float im = A.inv_massf[ti];
    double o[9];
    if (EV) vir9(v, o);
    atom_epilogue<true>(A, i, ti, 0., 0., 0., (fx - cfx) * im, (fy - cfy) * im, (fz - cfz) * im,
                        EV ? (double)(e - ce) : 0.0, EV ? o : nullptr);
  }
}

// PIECE: the launch covers atoms [A.i0, A.n) only (a separate instantiation:
// the offset costs registers that the full-range kernel, at the 64-register
// cap, would spill).
template <int T, int V, bool EV, bool MULTI, bool PIECE>
__global__ void __launch_bounds__(256, 4) k_lj_mixed(PairArgs A, LJF P, const LJPair* __restrict__ tab, int ntypes,
                                                  double rcmax2) {
  __shared__ LJTabSmem t;
  if (MULTI) lj_load_table(t, tab, ntypes);
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = PIECE ? A.i0 + gt / T : gt / T;
  lj_atom<T, V, EV, MULTI>(A, P, t, ntypes, rcmax2, i, (int)(gt % T), i < A.n, GlobalFetch{A.posf});
}

// One lane per atom, 4 entries per load, neighbour positions from the
// block's staged cells.
template <bool EV, bool MULTI>
__global__ void __launch_bounds__(256) k_lj_staged(PairArgs A, LJF P, const LJPair* __restrict__ tab, int ntypes,
                                                   double rcmax2, const int32_t* __restrict__ cstart, int K,
                                                   int cap) {
  __shared__ LJTabSmem t;
  __shared__ int4 rows[16];
  __shared__ int sh[56];
  extern __shared__ float4 staged_pos[];
  if (MULTI) lj_load_table(t, tab, ntypes);
  int64_t a0, a1;
  const bool ok = stage_cells(A.g, cstart, A.posf, K, cap, staged_pos, rows, sh, a0, a1);
  for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    if (ok) lj_atom<1, 4, EV, MULTI>(A, P, t, ntypes, rcmax2, i, 0, true, StagedFetch{staged_pos, rows});
    else lj_atom<1, 4, EV, MULTI>(A, P, t, ntypes, rcmax2, i, 0, true, GlobalFetch{A.posf});
  }
}

// ---------------------------------------------------------------------------
// eam_alloy
// ---------------------------------------------------------------------------
__device__ __forceinline__ int knot_f(float r, float rdr, int nr, float& q) {
  float t = fmaf(r, rdr, 1.0f);
  const int m = min((int)t, nr - 1);
  q = fminf(t - (float)m, 1.0f);
  return m;
}

__device__ __forceinline__ float spline_val(const float4& c, float q) {
  return fmaf(fmaf(fmaf(c.x, q, c.y), q, c.z), q, c.w);
}

__device__ __forceinline__ float spline_der(const float4& c, float q, float rd) {
  return fmaf(fmaf(3.f * c.x, q, 2.f * c.y), q, c.z) * rd;
}

// Density + embedding.  SINGLE (one element): also writes pfp[i] = (position,
// F'(rho_i)) so the force pass gathers both in one 16 B load.
template <int T, int V, bool EV, bool SINGLE, class Fetch>
__device__ __forceinline__ void eam_rho_atom(const PairArgs& A, const EamDev& E, float* __restrict__ fpf,
                                             float* __restrict__ epf, float4* __restrict__ pfp, int64_t i,
                                             int lane, bool live, const Fetch& fetch) {
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  const float4 pi = live ? A.posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int cp = live ? A.cellpack[i] : 0;
  const int ti = SINGLE ? 0 : __float_as_int(pi.w);
  const int nr = E.nr, nr1 = E.nr + 1;
  const float rdr = E.rdrf;
  float rho = 0.f, crho = 0.f;
  const PairFrame PF(pi, A.g);
  const ListRows<T, V> L(A.nbr, i, lane, A.stride, nn);
  uint32_t ent[V], nxt[V];
  if (L.nrow > 0) L.load(0, ent);
  for (int r = 0; r < L.nrow; ++r) {
    if (r + 1 < L.nrow) L.load(r + 1, nxt);
    float4 pj[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      if (!L.valid(r, q)) ent[q] = L.standin;
      pj[q] = fetch(ent[q], ent[q] & GBMD_IDX_MASK);
    }
    float rr = 0.f;
    if constexpr (V == 4) {
      // entries (0, 1) and (2, 3) in packed FP32; the rows' partial sums
      // stay packed until the row is added to the compensated sum
      float2 rr2 = f2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < V; q += 2) {
        const GeomF2 G = PF.geom(ent[q], ent[q + 1], pj[q], pj[q + 1]);
        bool ina = G.d2.x < E.rc2lo, inb = G.d2.y < E.rc2lo;
        if (!ina && G.d2.x <= E.rc2hi && L.valid(r, q))
          ina = exact_inside(A.posd, i, ent[q] & GBMD_IDX_MASK, ent[q] >> GBMD_IDX_BITS, cp, A.g, E.rcut2, 0.0);
        if (!inb && G.d2.y <= E.rc2hi && L.valid(r, q + 1))
          inb = exact_inside(A.posd, i, ent[q + 1] & GBMD_IDX_MASK, ent[q + 1] >> GBMD_IDX_BITS, cp, A.g, E.rcut2,
                             0.0);
        const float2 rd = __fmul2_rn(G.d2, f2(rsqrtf(G.d2.x), rsqrtf(G.d2.y)));
        const float2 tt = __ffma2_rn(rd, f2(rdr, rdr), f2(1.0f, 1.0f));
        const int ma = min((int)tt.x, nr - 1), mb = min((int)tt.y, nr - 1);
        const float2 qq0 = __fadd2_rn(tt, f2(-(float)ma, -(float)mb));
        const float2 qq = f2(fminf(qq0.x, 1.0f), fminf(qq0.y, 1.0f));
        const float4 ca = __ldg(&E.rhor4[SINGLE ? ma : __float_as_int(pj[q].w) * nr1 + ma]);
        const float4 cb = __ldg(&E.rhor4[SINGLE ? mb : __float_as_int(pj[q + 1].w) * nr1 + mb]);
        const float2 val = __ffma2_rn(__ffma2_rn(__ffma2_rn(f2(ca.x, cb.x), qq, f2(ca.y, cb.y)), qq, f2(ca.z, cb.z)),
                                      qq, f2(ca.w, cb.w));
        rr2 = __fadd2_rn(rr2, f2(ina ? val.x : 0.f, inb ? val.y : 0.f));
      }
      rr = rr2.x + rr2.y;
    } else {
#pragma unroll
      for (int q = 0; q < V; ++q) {
        const uint32_t j = ent[q] & GBMD_IDX_MASK;
        const GeomF G = geom_f(ent[q], pj[q], pi, A.g);
        bool in = G.d2 < E.rc2lo;
        if (!in && G.d2 <= E.rc2hi && L.valid(r, q))
          in = exact_inside(A.posd, i, j, ent[q] >> GBMD_IDX_BITS, cp, A.g, E.rcut2, 0.0);
        const float rd = G.d2 * rsqrtf(G.d2);
        float t;
        const int m = knot_f(rd, rdr, nr, t);
        const float4 c = __ldg(&E.rhor4[SINGLE ? m : __float_as_int(pj[q].w) * nr1 + m]);
        rr += in ? spline_val(c, t) : 0.f;
      }
    }
    kahan_add(rho, crho, rr);
#pragma unroll
    for (int q = 0; q < V; ++q) ent[q] = nxt[q];
  }
  group_reduce_kahan<T>(rho, crho);
  if (live && lane == 0) {
    // Rho2EmbOp / eam_alloy_fEmbed: F'(rho) (and F(rho) on energy steps),
    // linear continuation above rhomax
    const float R = rho - crho;
    float q = fmaf(R, E.rdrhof, 1.0f);
    int m = (int)q;
    m = max(1, min(m, E.nrho - 1));
    q = fminf(q - (float)m, 1.0f);
    const float4 c = __ldg(&E.frho4[(SINGLE ? 0 : ti * (E.nrho + 1)) + m]);
    const float fp = spline_der(c, q, E.rdrhof);
    fpf[i] = fp;
    if (SINGLE) pfp[i] = make_float4(pi.x, pi.y, pi.z, fp);
    if (EV) {
      float phi = spline_val(c, q);
      if (R > E.rhomaxf) phi = fmaf(fp, R - E.rhomaxf, phi);
      epf[i] = phi;
    }
  }
}

template <int T, int V, bool EV, bool SINGLE, bool PIECE>
__global__ void __launch_bounds__(256) k_eam_rho_mixed(PairArgs A, EamDev E, float* __restrict__ fpf,
                                                       float* __restrict__ epf, float4* __restrict__ pfp) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = PIECE ? A.i0 + gt / T : gt / T;
  eam_rho_atom<T, V, EV, SINGLE>(A, E, fpf, epf, pfp, i, (int)(gt % T), i < A.n, GlobalFetch{A.posf});
}

template <bool EV>
__global__ void __launch_bounds__(256) k_eam_rho_staged(PairArgs A, EamDev E, float* __restrict__ fpf,
                                                        float* __restrict__ epf, float4* __restrict__ pfp,
                                                        const int32_t* __restrict__ cstart, int K, int cap) {
  __shared__ int4 rows[16];
  __shared__ int sh[56];
  extern __shared__ float4 staged_pos[];
  int64_t a0, a1;
  const bool ok = stage_cells(A.g, cstart, A.posf, K, cap, staged_pos, rows, sh, a0, a1);
  for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    if (ok) eam_rho_atom<1, 4, EV, true>(A, E, fpf, epf, pfp, i, 0, true, StagedFetch{staged_pos, rows});
    else eam_rho_atom<1, 4, EV, true>(A, E, fpf, epf, pfp, i, 0, true, GlobalFetch{A.posf});
  }
}

// One 32-byte load of a knot's two float4 (rho' and z2r coefficients of the
// interleaved one-element table; the address is 32-byte aligned).
__device__ __forceinline__ void ldg_knot_pair(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

__device__ __forceinline__ int z2r_index_d(int a, int b) {
  const int irow = a > b ? a : b, icol = a > b ? b : a;
  return irow * (irow + 1) / 2 + icol;
}

// Force pass: f_i = sum_j u_ij (F'_i rho_j'(r) + F'_j rho_i'(r) + phi'(r)),
// then force_to_accel and the fused Verlet halves.  SINGLE reads (position,
// F'_j) through `fetch` from pfp; otherwise position (type in w) and fpf.
template <int T, int V, bool EV, bool SINGLE, class Fetch>
__device__ __forceinline__ void eam_force_atom(const PairArgs& A, const EamDev& E, const float* __restrict__ fpf,
                                               const float* __restrict__ epf, int64_t i, int lane, bool live,
                                               const Fetch& fetch) {
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  const float4 pi = live ? A.posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int cp = live ? A.cellpack[i] : 0;
  const float fpi = live ? fpf[i] : 0.f;
  const int ti = SINGLE ? 0 : __float_as_int(pi.w);
  const int nr = E.nr, nr1 = E.nr + 1;
  const float rdr = E.rdrf;
  float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const ListRows<T, V> L(A.nbr, i, lane, A.stride, nn);
  uint32_t ent[V], nxt[V];
  if (L.nrow > 0) L.load(0, ent);
  for (int r = 0; r < L.nrow; ++r) {
    if (r + 1 < L.nrow) L.load(r + 1, nxt);
    float4 pj[V];
    float fpj[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      if (!L.valid(r, q)) ent[q] = L.standin;
      const uint32_t j = ent[q] & GBMD_IDX_MASK;
      pj[q] = fetch(ent[q], j);
      fpj[q] = SINGLE ? pj[q].w : __ldg(&fpf[j]);
    }
    float rx = 0.f, ry = 0.f, rz = 0.f, re = 0.f;
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const uint32_t j = ent[q] & GBMD_IDX_MASK;
      const GeomF G = geom_f(ent[q], pj[q], pi, A.g);
      bool in = G.d2 < E.rc2lo;
      if (!in && G.d2 <= E.rc2hi && L.valid(r, q))
        in = exact_inside(A.posd, i, j, ent[q] >> GBMD_IDX_BITS, cp, A.g, E.rcut2, 0.0);
      const float rs = rsqrtf(G.d2);
      const float rd = G.d2 * rs;
      float t;
      const int m = knot_f(rd, rdr, nr, t);
      const int tj = SINGLE ? 0 : __float_as_int(pj[q].w);
      // rho'(r) from the pre-scaled derivative table: (3c3/dr, 2c4/dr, c5/dr);
      // one element: rho' and z2r knots interleaved, read in one 32 B load
      float4 dj, cz;
      if (SINGLE) {
        ldg_knot_pair(&E.fz8[2 * m], dj, cz);
      } else {
        dj = __ldg(&E.rhod4[tj * nr1 + m]);
        cz = __ldg(&E.z2r4[z2r_index_d(ti, tj) * nr1 + m]);
      }
      const float rhojp = fmaf(fmaf(dj.x, t, dj.y), t, dj.z);
      float rhoip = rhojp;
      if (!SINGLE && ti != tj) {
        const float4 di = __ldg(&E.rhod4[ti * nr1 + m]);
        rhoip = fmaf(fmaf(di.x, t, di.y), t, di.z);
      }
      const float t1 = fmaf(cz.x, t, cz.y);
      const float z2 = fmaf(fmaf(t1, t, cz.z), t, cz.w);          // z2r tables carry conv_z2r
      const float z2d = fmaf(fmaf(cz.x, t, t1 + t1), t, cz.z);     // d z2 / d t
      const float phi = z2 * rs;
      const float phip = fmaf(z2d * rdr, rs, -phi * rs);
      const float psip = fmaf(fpi, rhojp, fmaf(fpj[q], rhoip, phip));
      const float fpair = in ? psip * rs : 0.f;
      rx = fmaf(G.dx, fpair, rx);
      ry = fmaf(G.dy, fpair, ry);
      rz = fmaf(G.dz, fpair, rz);
      if (EV) {
        re += in ? 0.5f * phi : 0.f;
        const float h = -0.5f * fpair;
        v[0] = fmaf(h * G.dx, G.dx, v[0]);
        v[1] = fmaf(h * G.dy, G.dy, v[1]);
        v[2] = fmaf(h * G.dz, G.dz, v[2]);
        v[3] = fmaf(h * G.dx, G.dy, v[3]);
        v[4] = fmaf(h * G.dx, G.dz, v[4]);
        v[5] = fmaf(h * G.dy, G.dz, v[5]);
      }
    }
    kahan_add(fx, cfx, rx);
    kahan_add(fy, cfy, ry);
    kahan_add(fz, cfz, rz);
    if (EV) kahan_add(e, ce, re);
#pragma unroll
    for (int q = 0; q < V; ++q) ent[q] = nxt[q];
  }
  group_reduce_kahan<T>(fx, cfx);
  group_reduce_kahan<T>(fy, cfy);
  group_reduce_kahan<T>(fz, cfz);
  if (EV) {
    group_reduce_kahan<T>(e, ce);
    reduce6(v, T);
  }
  if (live && lane == 0) {
    const float im = A.inv_massf[ti];
    double o[9];
    if (EV) vir9(v, o);
    const double epv = EV ? (double)epf[i] + (double)(e - ce) : 0.0;
    atom_epilogue<true>(A, i, ti, 0., 0., 0., (fx - cfx) * im, (fy - cfy) * im, (fz - cfz) * im, epv,
                        EV ? o : nullptr);
  }
}

template <int T, int V, bool EV, bool SINGLE, bool PIECE>
__global__ void __launch_bounds__(256, 4) k_eam_force_mixed(PairArgs A, EamDev E, const float* __restrict__ fpf,
                                                         const float* __restrict__ epf,
                                                         const float4* __restrict__ pfp) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = PIECE ? A.i0 + gt / T : gt / T;
  eam_force_atom<T, V, EV, SINGLE>(A, E, fpf, epf, i, (int)(gt % T), i < A.n,
                                   GlobalFetch{SINGLE ? pfp : A.posf});
}

template <bool EV>
__global__ void __launch_bounds__(256) k_eam_force_staged(PairArgs A, EamDev E, const float* __restrict__ fpf,
                                                          const float* __restrict__ epf,
                                                          const float4* __restrict__ pfp,
                                                          const int32_t* __restrict__ cstart, int K, int cap) {
  __shared__ int4 rows[16];
  __shared__ int sh[56];
  extern __shared__ float4 staged_pos[];
  int64_t a0, a1;
  const bool ok = stage_cells(A.g, cstart, pfp, K, cap, staged_pos, rows, sh, a0, a1);
  for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    if (ok) eam_force_atom<1, 4, EV, true>(A, E, fpf, epf, i, 0, true, StagedFetch{staged_pos, rows});
    else eam_force_atom<1, 4, EV, true>(A, E, fpf, epf, i, 0, true, GlobalFetch{pfp});
  }
}

// ---------------------------------------------------------------------------
// Newton-3 LJ (lj_compute_force_symetric, pair_potential_singlemat_symetric.cpp
// L230-320): every unordered pair once, from the half list (j after i in cell
// order).  The pair's force, half its energy and half its virial go to i's
// register sums and -- the force negated -- to j's accumulators (the
// reference takes a spin lock on j); i's own sums are added to its
// accumulators once at the end, since other threads add to them as well.
//
// The accumulators are 64-bit fixed-point integers, so the sums do not depend
// on the order the additions arrive in and the results are the same from run
// to run.  Ten planes of `cap`: f (3), ep, virial xx yy zz xy xz yz.  A value
// x is stored as round(x * 2^38 / b), b a power of two bounding its kind (24
// eps/sigma for forces, 4 eps for energies, that force times rcut for
// virials): x * 2^38 / b is exact in FP32 and the rounding is deterministic.
// A pair's contribution must stay below 2^16 b, i's own sum below 2^24 b, so
// that 512 of them cannot overflow 2^63; a larger one raises
// GBMD_DEVERR_RANGE.  k_h3_epilogue turns the sums into the acceleration
// (and the fused Verlet half steps) and clears them for the next pass.
// ---------------------------------------------------------------------------
struct FixScale {
  float f, e, v, r;    // 2^38 / bound for forces, energies, virials, EAM densities
  double inv_f, inv_e, inv_v, inv_r;
  int* err;
};

constexpr float FIX_PAIR_LIMIT = 0x1p54f;  // |x * scale| of one pair's contribution
constexpr float FIX_SUM_LIMIT = 0x1p62f;   // |x * scale| of an atom's own sum

__device__ __forceinline__ long long fix_q(float x, float scale, float limit, int* err) {
  float y = x * scale;
  if (!(fabsf(y) <= limit)) {
    atomicOr(err, GBMD_DEVERR_RANGE);
    y = y != y ? 0.f : copysignf(limit, y);
  }
  return __float2ll_rn(y);
}

__device__ __forceinline__ void fix_add(long long* p, long long q) {
  // two's complement: the unsigned sum is the signed one modulo 2^64
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)q);
}

template <bool EV, bool MULTI>
__global__ void __launch_bounds__(256, EV ? 1 : 4) k_lj_half(PairArgs A, LJF P, const LJPair* __restrict__ tab, int ntypes,
                                                 double rcmax2, long long* __restrict__ acc, int64_t cap,
                                                 FixScale X) {
  __shared__ LJTabSmem tb;
  if (MULTI) lj_load_table(tb, tab, ntypes);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const int nn = min(A.nnb[i], A.maxnb);
  const float4 pi = A.posf[i];
  const int cp = A.cellpack[i];
  const int ti = __float_as_int(pi.w);
  float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const ListRows<1, 4> L(A.nbr, i, 0, A.stride, nn);
  const GlobalFetch fetch{A.posf};
  uint32_t ent[4], nxt[4];
  if (L.nrow > 0) L.load(0, ent);
  for (int r = 0; r < L.nrow; ++r) {
    if (r + 1 < L.nrow) L.load(r + 1, nxt);
    float4 pj[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (!L.valid(r, q)) ent[q] = L.standin;
      pj[q] = fetch(ent[q], ent[q] & GBMD_IDX_MASK);
    }
    float rx = 0.f, ry = 0.f, rz = 0.f, re = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t j = ent[q] & GBMD_IDX_MASK;
      const GeomF G = geom_f(ent[q], pj[q], pi, A.g);
      float sig2, eps24, eps4, ecut, rlo, rhi;
      int pid = 0;
      if (MULTI) {
        pid = ti * ntypes + __float_as_int(pj[q].w);
        const float4 a = tb.a[pid];
        const float2 b = tb.b[pid];
        sig2 = a.x; eps24 = a.y; eps4 = a.z; ecut = a.w; rlo = b.x; rhi = b.y;
      } else {
        sig2 = P.sig2; eps24 = P.eps24; eps4 = P.eps4; ecut = P.ecut; rlo = P.rc2lo; rhi = P.rc2hi;
      }
      bool in = G.d2 < rlo;
      if (!in && G.d2 <= rhi && L.valid(r, q))
        in = exact_inside(A.posd, i, j, ent[q] >> GBMD_IDX_BITS, cp, A.g, MULTI ? rcmax2 : P.rc2,
                          MULTI ? tb.r[pid] : 0.0);
      float r2i;
      asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r2i) : "f"(G.d2));
      const float s2 = sig2 * r2i;
      const float s6 = s2 * s2 * s2;
      const float s12 = s6 * s6;
      const float fpair = eps24 * fmaf(2.f, s12, -s6) * r2i;  // -(dE/dr)/r
      if (in) {
        const float gx = fpair * G.dx, gy = fpair * G.dy, gz = fpair * G.dz;
        rx -= gx;
        ry -= gy;
        rz -= gz;
        fix_add(acc + j, fix_q(gx, X.f, FIX_PAIR_LIMIT, X.err));
        fix_add(acc + cap + j, fix_q(gy, X.f, FIX_PAIR_LIMIT, X.err));
        fix_add(acc + 2 * cap + j, fix_q(gz, X.f, FIX_PAIR_LIMIT, X.err));
        if (EV) {
          const float eh = 0.5f * fmaf(eps4, s12 - s6, -ecut);
          const float h = 0.5f * fpair;
          const float w[6] = {h * G.dx * G.dx, h * G.dy * G.dy, h * G.dz * G.dz,
                              h * G.dx * G.dy, h * G.dx * G.dz, h * G.dy * G.dz};
          re += eh;
          fix_add(acc + 3 * cap + j, fix_q(eh, X.e, FIX_PAIR_LIMIT, X.err));
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            v[k] += w[k];
            fix_add(acc + (4 + k) * cap + j, fix_q(w[k], X.v, FIX_PAIR_LIMIT, X.err));
          }
        }
      }
    }
    kahan_add(fx, cfx, rx);
    kahan_add(fy, cfy, ry);
    kahan_add(fz, cfz, rz);
    if (EV) kahan_add(e, ce, re);
#pragma unroll
    for (int q = 0; q < 4; ++q) ent[q] = nxt[q];
  }
  fix_add(acc + i, fix_q(fx - cfx, X.f, FIX_SUM_LIMIT, X.err));
  fix_add(acc + cap + i, fix_q(fy - cfy, X.f, FIX_SUM_LIMIT, X.err));
  fix_add(acc + 2 * cap + i, fix_q(fz - cfz, X.f, FIX_SUM_LIMIT, X.err));
  if (EV) {
    fix_add(acc + 3 * cap + i, fix_q(e - ce, X.e, FIX_SUM_LIMIT, X.err));
#pragma unroll
    for (int k = 0; k < 6; ++k) fix_add(acc + (4 + k) * cap + i, fix_q(v[k], X.v, FIX_SUM_LIMIT, X.err));
  }
}

template <bool EV>
__global__ void __launch_bounds__(256) k_h3_epilogue(PairArgs A, long long* __restrict__ acc, int64_t cap,
                                                     FixScale X, const float* __restrict__ epf) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  double f[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    f[d] = (double)acc[d * cap + i] * X.inv_f;
    acc[d * cap + i] = 0;
  }
  const int t = __float_as_int(A.posf[i].w);
  const float im = A.inv_massf[t];
  double o[9];
  double epv = 0.0;
  if (EV) {
    epv = (double)acc[3 * cap + i] * X.inv_e + (epf ? (double)epf[i] : 0.0);
    acc[3 * cap + i] = 0;
    float v[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      v[k] = (float)((double)acc[(4 + k) * cap + i] * X.inv_v);
      acc[(4 + k) * cap + i] = 0;
    }
    vir9(v, o);
  }
  atom_epilogue<true>(A, i, t, 0., 0., 0., (float)f[0] * im, (float)f[1] * im, (float)f[2] * im, epv,
                      EV ? o : nullptr);
}

// Newton-3 eam_alloy (eam_symmetry: eam_force_op_multimat.h L162-169 rho_j
// scatter, L305-338 reaction force): the same per-pair FP32 expressions as
// k_eam_rho_mixed / k_eam_force_mixed on the half list.  The density pass
// adds rho_tj(r) to i's own sum and rho_ti(r) to j's fixed-point plane (the
// energy plane, free until the force pass); k_eam_embed_half turns the sums
// into F'(rho) (and F(rho)); the force pass adds u_ij psi'_ij / r to i and
// its opposite to j, half of phi to both, the pair virial to both.
template <bool SINGLE>
__global__ void __launch_bounds__(256, 4) k_eam_rho_half(PairArgs A, EamDev E, long long* __restrict__ racc,
                                                         FixScale X) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const int nn = min(A.nnb[i], A.maxnb);
  const float4 pi = A.posf[i];
  const int cp = A.cellpack[i];
  const int ti = SINGLE ? 0 : __float_as_int(pi.w);
  const int nr = E.nr, nr1 = E.nr + 1;
  float rho = 0.f, crho = 0.f;
  const ListRows<1, 4> L(A.nbr, i, 0, A.stride, nn);
  const GlobalFetch fetch{A.posf};
  uint32_t ent[4], nxt[4];
  if (L.nrow > 0) L.load(0, ent);
  for (int r = 0; r < L.nrow; ++r) {
    if (r + 1 < L.nrow) L.load(r + 1, nxt);
    float4 pj[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (!L.valid(r, q)) ent[q] = L.standin;
      pj[q] = fetch(ent[q], ent[q] & GBMD_IDX_MASK);
    }
    float rr = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t j = ent[q] & GBMD_IDX_MASK;
      const GeomF G = geom_f(ent[q], pj[q], pi, A.g);
      bool in = G.d2 < E.rc2lo;
      if (!in && G.d2 <= E.rc2hi && L.valid(r, q))
        in = exact_inside(A.posd, i, j, ent[q] >> GBMD_IDX_BITS, cp, A.g, E.rcut2, 0.0);
      const float rd = G.d2 * rsqrtf(G.d2);
      float t;
      const int m = knot_f(rd, E.rdrf, nr, t);
      const int tj = SINGLE ? 0 : __float_as_int(pj[q].w);
      const float vj = spline_val(__ldg(&E.rhor4[tj * nr1 + m]), t);
      const float vi = (SINGLE || ti == tj) ? vj : spline_val(__ldg(&E.rhor4[ti * nr1 + m]), t);
      rr += in ? vj : 0.f;
      if (in) fix_add(racc + j, fix_q(vi, X.r, FIX_PAIR_LIMIT, X.err));
    }
    kahan_add(rho, crho, rr);
#pragma unroll
    for (int q = 0; q < 4; ++q) ent[q] = nxt[q];
  }
  fix_add(racc + i, fix_q(rho - crho, X.r, FIX_SUM_LIMIT, X.err));
}

// Rho2EmbOp / eam_alloy_fEmbed on the summed densities (the embedding of
// eam_rho_atom): F'(rho), F(rho) on energy steps, linear continuation above
// rhomax; the density plane is cleared for the energies of the force pass.
template <bool EV, bool SINGLE>
__global__ void __launch_bounds__(256) k_eam_embed_half(PairArgs A, EamDev E, long long* __restrict__ racc,
                                                        FixScale X, float* __restrict__ fpf, float* __restrict__ epf,
                                                        float4* __restrict__ pfp) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const float R = (float)((double)racc[i] * X.inv_r);
  racc[i] = 0;
  const float4 pi = A.posf[i];
  const int ti = SINGLE ? 0 : __float_as_int(pi.w);
  float q = fmaf(R, E.rdrhof, 1.0f);
  int m = (int)q;
  m = max(1, min(m, E.nrho - 1));
  q = fminf(q - (float)m, 1.0f);
  const float4 c = __ldg(&E.frho4[(SINGLE ? 0 : ti * (E.nrho + 1)) + m]);
  const float fp = spline_der(c, q, E.rdrhof);
  fpf[i] = fp;
  if (SINGLE) pfp[i] = make_float4(pi.x, pi.y, pi.z, fp);
  if (EV) {
    float phi = spline_val(c, q);
    if (R > E.rhomaxf) phi = fmaf(fp, R - E.rhomaxf, phi);
    epf[i] = phi;
  }
}

template <bool EV, bool SINGLE>
__global__ void __launch_bounds__(256, EV ? 1 : 4) k_eam_force_half(PairArgs A, EamDev E,
                                                                    const float* __restrict__ fpf,
                                                                    const float4* __restrict__ pfp,
                                                                    long long* __restrict__ acc, int64_t cap,
                                                                    FixScale X) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const int nn = min(A.nnb[i], A.maxnb);
  const float4 pi = A.posf[i];
  const int cp = A.cellpack[i];
  const float fpi = fpf[i];
  const int ti = SINGLE ? 0 : __float_as_int(pi.w);
  const int nr = E.nr, nr1 = E.nr + 1;
  const float rdr = E.rdrf;
  float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const ListRows<1, 4> L(A.nbr, i, 0, A.stride, nn);
  const GlobalFetch fetch{SINGLE ? pfp : A.posf};
  uint32_t ent[4], nxt[4];
  if (L.nrow > 0) L.load(0, ent);
  for (int r = 0; r < L.nrow; ++r) {
    if (r + 1 < L.nrow) L.load(r + 1, nxt);
    float4 pj[4];
    float fpj[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (!L.valid(r, q)) ent[q] = L.standin;
      const uint32_t j = ent[q] & GBMD_IDX_MASK;
      pj[q] = fetch(ent[q], j);
      fpj[q] = SINGLE ? pj[q].w : __ldg(&fpf[j]);
    }
    float rx = 0.f, ry = 0.f, rz = 0.f, re = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t j = ent[q] & GBMD_IDX_MASK;
      const GeomF G = geom_f(ent[q], pj[q], pi, A.g);
      bool in = G.d2 < E.rc2lo;
      if (!in && G.d2 <= E.rc2hi && L.valid(r, q))
        in = exact_inside(A.posd, i, j, ent[q] >> GBMD_IDX_BITS, cp, A.g, E.rcut2, 0.0);
      const float rs = rsqrtf(G.d2);
      const float rd = G.d2 * rs;
      float t;
      const int m = knot_f(rd, rdr, nr, t);
      const int tj = SINGLE ? 0 : __float_as_int(pj[q].w);
      const float4 dj = __ldg(&E.rhod4[tj * nr1 + m]);
      const float4 cz = __ldg(&E.z2r4[z2r_index_d(ti, tj) * nr1 + m]);
      const float rhojp = fmaf(fmaf(dj.x, t, dj.y), t, dj.z);
      float rhoip = rhojp;
      if (!SINGLE && ti != tj) {
        const float4 di = __ldg(&E.rhod4[ti * nr1 + m]);
        rhoip = fmaf(fmaf(di.x, t, di.y), t, di.z);
      }
      const float t1 = fmaf(cz.x, t, cz.y);
      const float z2 = fmaf(fmaf(t1, t, cz.z), t, cz.w);
      const float z2d = fmaf(fmaf(cz.x, t, t1 + t1), t, cz.z);
      const float phi = z2 * rs;
      const float phip = fmaf(z2d * rdr, rs, -phi * rs);
      const float psip = fmaf(fpi, rhojp, fmaf(fpj[q], rhoip, phip));
      const float fpair = in ? psip * rs : 0.f;
      const float gx = G.dx * fpair, gy = G.dy * fpair, gz = G.dz * fpair;
      rx += gx;
      ry += gy;
      rz += gz;
      if (in) {
        fix_add(acc + j, fix_q(-gx, X.f, FIX_PAIR_LIMIT, X.err));
        fix_add(acc + cap + j, fix_q(-gy, X.f, FIX_PAIR_LIMIT, X.err));
        fix_add(acc + 2 * cap + j, fix_q(-gz, X.f, FIX_PAIR_LIMIT, X.err));
        if (EV) {
          const float eh = 0.5f * phi;
          const float h = -0.5f * fpair;
          const float w[6] = {h * G.dx * G.dx, h * G.dy * G.dy, h * G.dz * G.dz,
                              h * G.dx * G.dy, h * G.dx * G.dz, h * G.dy * G.dz};
          re += eh;
          fix_add(acc + 3 * cap + j, fix_q(eh, X.e, FIX_PAIR_LIMIT, X.err));
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            v[k] += w[k];
            fix_add(acc + (4 + k) * cap + j, fix_q(w[k], X.v, FIX_PAIR_LIMIT, X.err));
          }
        }
      }
    }
    kahan_add(fx, cfx, rx);
    kahan_add(fy, cfy, ry);
    kahan_add(fz, cfz, rz);
    if (EV) kahan_add(e, ce, re);
#pragma unroll
    for (int q = 0; q < 4; ++q) ent[q] = nxt[q];
  }
  fix_add(acc + i, fix_q(fx - cfx, X.f, FIX_SUM_LIMIT, X.err));
  fix_add(acc + cap + i, fix_q(fy - cfy, X.f, FIX_SUM_LIMIT, X.err));
  fix_add(acc + 2 * cap + i, fix_q(fz - cfz, X.f, FIX_SUM_LIMIT, X.err));
  if (EV) {
    fix_add(acc + 3 * cap + i, fix_q(e - ce, X.e, FIX_SUM_LIMIT, X.err));
#pragma unroll
    for (int k = 0; k < 6; ++k) fix_add(acc + (4 + k) * cap + i, fix_q(v[k], X.v, FIX_SUM_LIMIT, X.err));
  }
}

// the power of two at or above x (at least 2^-60, which keeps the FP32
// scales finite: all-zero tables give zero contributions at any scale)
static double pow2_at_least(double x) {
  return std::ldexp(1.0, (int)std::ceil(std::log2(std::max(x, 0x1p-60))));
}

// Power-of-two fixed-point scales of the bounds above, from the LJ table.
static FixScale fix_scales(const gbmd_context* c) {
  double fmax = 0.0, emax = 0.0;
  const int nt = c->pot == GBMD_POT_LJ ? 1 : c->lj.ntypes;
  for (int a = 0; a < nt * nt; ++a) {
    const LJPair& q = c->lj.p[a];
    fmax = std::max(fmax, 24.0 * std::fabs(q.eps) / q.sig);
    emax = std::max(emax, 4.0 * std::fabs(q.eps));
  }
  const double vmax = fmax * c->lj.rcut_max;
  const double bf = pow2_at_least(fmax), be = pow2_at_least(emax), bv = pow2_at_least(vmax);
  FixScale X;
  X.f = (float)std::ldexp(1.0 / bf, 38);
  X.e = (float)std::ldexp(1.0 / be, 38);
  X.v = (float)std::ldexp(1.0 / bv, 38);
  X.inv_f = std::ldexp(bf, -38);
  X.inv_e = std::ldexp(be, -38);
  X.inv_v = std::ldexp(bv, -38);
  X.r = 1.f;
  X.inv_r = 1.0;
  X.err = c->d_err + ERRW_FLAGS;
  return X;
}

// eam_alloy: bounds from the host spline copies over the knots from 0.3 rcut
// to rcut (closer pairs are far from any physical state; their
// contributions still fit below 2^16 times the bounds unless they are
// extreme).  Knot m holds the spline on [m dr, (m+1) dr) with value s[6]
// and slope s[5] / dr at its start.  |psi'| <= 2 max|F'| max|rho'| +
// max|phi'|, doubled; energies half phi; virials that force times rcut.
static FixScale eam_fix_scales(gbmd_context* c) {
  if (!c->eam_fix_ok) {
    const EamDev& E = c->eam;
    const double dr = 1.0 / E.rdr, drho = 1.0 / E.rdrho;
    const size_t kr = (size_t)E.nr + 1, kp = (size_t)E.nrho + 1;
    const size_t m0 = std::max<size_t>(1, (size_t)(0.3 * E.rcut / dr));
    const size_t m1 = std::min(kr - 1, (size_t)(E.rcut / dr) + 1);
    double rho = 0.0, rhop = 0.0, phi = 0.0, phip = 0.0, fp = 0.0;
    for (int e = 0; e < E.nel; ++e) {
      for (size_t m = m0; m <= m1; ++m) {
        const double* s = &c->eam_host_rhor[((size_t)e * kr + m) * 8];
        rho = std::max(rho, std::fabs(s[6]));
        rhop = std::max(rhop, std::fabs(s[5]) / dr);
      }
      for (size_t m = 0; m < kp; ++m)
        fp = std::max(fp, std::fabs(c->eam_host_frho[((size_t)e * kp + m) * 8 + 5]) / drho * E.conv_frho);
    }
    for (int p = 0; p < E.npairs; ++p)
      for (size_t m = m0; m <= m1; ++m) {
        const double* s = &c->eam_host_z2r[((size_t)p * kr + m) * 8];
        const double r = (double)m * dr, z2 = s[6] * E.conv_z2r, z2d = s[5] / dr * E.conv_z2r;
        phi = std::max(phi, std::fabs(z2 / r));
        phip = std::max(phip, std::fabs((z2d - z2 / r) / r));
      }
    const double f = 2.0 * (2.0 * fp * rhop + phip);
    c->eam_fix_bound[0] = pow2_at_least(2.0 * rho);
    c->eam_fix_bound[1] = pow2_at_least(f);
    c->eam_fix_bound[2] = pow2_at_least(phi);
    c->eam_fix_bound[3] = pow2_at_least(f * E.rcut);
    c->eam_fix_ok = true;
  }
  const double* b = c->eam_fix_bound;
  FixScale X;
  X.r = (float)std::ldexp(1.0 / b[0], 38);
  X.f = (float)std::ldexp(1.0 / b[1], 38);
  X.e = (float)std::ldexp(1.0 / b[2], 38);
  X.v = (float)std::ldexp(1.0 / b[3], 38);
  X.inv_r = std::ldexp(b[0], -38);
  X.inv_f = std::ldexp(b[1], -38);
  X.inv_e = std::ldexp(b[2], -38);
  X.inv_v = std::ldexp(b[3], -38);
  X.err = c->d_err + ERRW_FLAGS;
  return X;
}

template <bool EV, bool SINGLE>
static void launch_eam_newton3(gbmd_context* c, const PairArgs& A, int part, unsigned grid, int B) {
  cudaStream_t s = c->stream;
  const FixScale X = eam_fix_scales(c);
  long long* racc = c->h3acc + 3 * c->cap;  // the energy plane, free until the force pass
  if (part != 2) {
    k_eam_rho_half<SINGLE><<<grid, B, 0, s>>>(A, c->eam, racc, X);
    k_eam_embed_half<EV, SINGLE><<<grid, B, 0, s>>>(A, c->eam, racc, X, c->fpf, c->epf, c->pfp);
  }
  if (part != 1) {
    k_eam_force_half<EV, SINGLE><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->pfp, c->h3acc, c->cap, X);
    k_h3_epilogue<EV><<<grid, B, 0, s>>>(A, c->h3acc, c->cap, X, EV ? c->epf : nullptr);
  }
}

template <bool EV>
static int launch_newton3(gbmd_context* c, const PairArgs& A, int part) {
  if (A.n == 0) return GBMD_OK;
  const int B = 256;
  const unsigned grid = (unsigned)((A.n + B - 1) / B);
  if (c->pot == GBMD_POT_EAM_ALLOY) {
    if (c->eam.nel == 1) launch_eam_newton3<EV, true>(c, A, part, grid, B);
    else launch_eam_newton3<EV, false>(c, A, part, grid, B);
    return GBMD_OK;
  }
  if (part == 1) return GBMD_OK;
  cudaStream_t s = c->stream;
  const FixScale X = fix_scales(c);
  if (c->pot == GBMD_POT_LJ) {
    const LJPair& q = c->lj.p[0];
    LJF P{q.sig2f, q.eps24f, q.eps4f, q.ecutf, q.rc2lo, q.rc2hi, q.rc2, q.rc};
    k_lj_half<EV, false><<<grid, B, 0, s>>>(A, P, nullptr, 1, c->lj.rcut_max2, c->h3acc, c->cap, X);
  } else {
    LJF P{};
    k_lj_half<EV, true><<<grid, B, 0, s>>>(A, P, c->lj_tab_d, c->lj.ntypes, c->lj.rcut_max2, c->h3acc, c->cap, X);
  }
  k_h3_epilogue<EV><<<grid, B, 0, s>>>(A, c->h3acc, c->cap, X, nullptr);
  return GBMD_OK;
}

// ---------------------------------------------------------------------------
// dispatch
// ---------------------------------------------------------------------------
template <int T, int V, bool EV, bool PIECE>
static void launch_mixed_TV(gbmd_context* c, const PairArgs& A, int part) {
  const int B = c->block;
  const unsigned grid = (unsigned)(((A.n - A.i0) * T + B - 1) / B);
  const int Bd = c->block_rho ? c->block_rho : B;  // density kernels
  const unsigned gridd = (unsigned)(((A.n - A.i0) * T + Bd - 1) / Bd);
  cudaStream_t s = c->stream;
  if (c->pot == GBMD_POT_LJ) {
    if (part == 1) return;
    const LJPair& q = c->lj.p[0];
    LJF P{q.sig2f, q.eps24f, q.eps4f, q.ecutf, q.rc2lo, q.rc2hi, q.rc2, q.rc};
    k_lj_mixed<T, V, EV, false, PIECE><<<grid, B, 0, s>>>(A, P, nullptr, 1, c->lj.rcut_max2);
  } else if (c->pot == GBMD_POT_LJ_MULTI) {
    if (part == 1) return;
    LJF P{};
    k_lj_mixed<T, V, EV, true, PIECE><<<grid, B, 0, s>>>(A, P, c->lj_tab_d, c->lj.ntypes, c->lj.rcut_max2);
  } else if (c->eam.nel == 1) {
    if (part != 2) k_eam_rho_mixed<T, V, EV, true, PIECE><<<gridd, Bd, 0, s>>>(A, c->eam, c->fpf, c->epf, c->pfp);
    if (part != 1) k_eam_force_mixed<T, V, EV, true, PIECE><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->epf, c->pfp);
  } else {
    if (part != 2) k_eam_rho_mixed<T, V, EV, false, PIECE><<<gridd, Bd, 0, s>>>(A, c->eam, c->fpf, c->epf, c->pfp);
    if (part != 1) k_eam_force_mixed<T, V, EV, false, PIECE><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->epf, c->pfp);
  }
}

// Staged launch (one lane per atom, 4 entries per load): blocks of K home
// cells along x; K gives about 0.8 * block atoms per block, and the staged
// capacity is 1.4 times the mean neighbourhood of (K+2) x 3 x 3 cells (a
// denser block falls back to global gathers).
// Raise the dynamic shared-memory limit of the staged kernels once, outside
// any stream capture (the attribute is per kernel, not per launch).
static constexpr int STAGED_MAX_SMEM = 200 * 1024;

int configure_staged_kernels() {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void* f) {
    const cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, STAGED_MAX_SMEM);
    if (r != cudaSuccess) e = r;
  };
  set((const void*)k_lj_staged<false, false>);
  set((const void*)k_lj_staged<true, false>);
  set((const void*)k_lj_staged<false, true>);
  set((const void*)k_lj_staged<true, true>);
  set((const void*)k_eam_rho_staged<false>);
  set((const void*)k_eam_rho_staged<true>);
  set((const void*)k_eam_force_staged<false>);
  set((const void*)k_eam_force_staged<true>);
  return e == cudaSuccess ? GBMD_OK : GBMD_ERR_CUDA;
}

template <bool EV>
static bool launch_staged(gbmd_context* c, const PairArgs& A, int part) {
  const bool lj = c->pot == GBMD_POT_LJ || c->pot == GBMD_POT_LJ_MULTI;
  if (!lj && !(c->pot == GBMD_POT_EAM_ALLOY && c->eam.nel == 1)) return false;
  const Grid& g = c->grid;
  const double per_cell = (double)A.n / (double)g.ncells;
  const int B = c->block;
  int K = (int)(0.8 * B / (per_cell > 0.5 ? per_cell : 0.5));
  K = K < 1 ? 1 : (K > g.nc[0] ? g.nc[0] : K);
  int cap = (int)(1.4 * per_cell * 9 * (K + 2)) + 64;
  const int max_cap = STAGED_MAX_SMEM / (int)sizeof(float4);
  if (cap > max_cap) cap = max_cap;
  const size_t smem = (size_t)cap * sizeof(float4);
  const dim3 grid((unsigned)((g.nc[0] + K - 1) / K), (unsigned)g.nc[1], (unsigned)g.nc[2]);
  cudaStream_t s = c->stream;
  if (c->pot == GBMD_POT_LJ) {
    if (part == 1) return true;
    const LJPair& q = c->lj.p[0];
    LJF P{q.sig2f, q.eps24f, q.eps4f, q.ecutf, q.rc2lo, q.rc2hi, q.rc2, q.rc};
    k_lj_staged<EV, false><<<grid, B, smem, s>>>(A, P, nullptr, 1, c->lj.rcut_max2, c->cell_start, K, cap);
  } else if (c->pot == GBMD_POT_LJ_MULTI) {
    if (part == 1) return true;
    LJF P{};
    k_lj_staged<EV, true><<<grid, B, smem, s>>>(A, P, c->lj_tab_d, c->lj.ntypes, c->lj.rcut_max2, c->cell_start,
                                                 K, cap);
  } else {
    if (part != 2)
      k_eam_rho_staged<EV><<<grid, B, smem, s>>>(A, c->eam, c->fpf, c->epf, c->pfp, c->cell_start, K, cap);
    if (part != 1)
      k_eam_force_staged<EV><<<grid, B, smem, s>>>(A, c->eam, c->fpf, c->epf, c->pfp, c->cell_start, K, cap);
  }
  return true;
}

template <bool EV, bool PIECE>
static int launch_mixed_shape(gbmd_context* c, const PairArgs& A, int part) {
  const int key = c->tpa * 8 + c->vec;
  switch (key) {
    case 1 * 8 + 1: launch_mixed_TV<1, 1, EV, PIECE>(c, A, part); break;
    case 1 * 8 + 4: launch_mixed_TV<1, 4, EV, PIECE>(c, A, part); break;
    case 2 * 8 + 1: launch_mixed_TV<2, 1, EV, PIECE>(c, A, part); break;
    case 2 * 8 + 4: launch_mixed_TV<2, 4, EV, PIECE>(c, A, part); break;
    case 4 * 8 + 1: launch_mixed_TV<4, 1, EV, PIECE>(c, A, part); break;
    case 4 * 8 + 4: launch_mixed_TV<4, 4, EV, PIECE>(c, A, part); break;
    case 8 * 8 + 1: launch_mixed_TV<8, 1, EV, PIECE>(c, A, part); break;
    case 16 * 8 + 1: launch_mixed_TV<16, 1, EV, PIECE>(c, A, part); break;
    default:
      return set_error(c, GBMD_ERR_INVALID, "unsupported launch: %d lanes x %d entries per atom", c->tpa, c->vec);
  }
  return GBMD_OK;
}

template <bool EV>
static int launch_mixed_E(gbmd_context* c, const PairArgs& A, int part) {
  if (c->newton3) {
    // the half list is laid out as one lane x 4 entries per load
    if (c->tpa != 1 || c->vec != 4)
      return set_error(c, GBMD_ERR_UNSUPPORTED, "Newton-3 half lists need the 1 lane x 4 entries launch");
    return launch_newton3<EV>(c, A, part);
  }
  if (c->staged && c->tpa == 1 && c->vec == 4 && launch_staged<EV>(c, A, part)) return GBMD_OK;
  return launch_mixed_shape<EV, false>(c, A, part);
}

int launch_mixed(gbmd_context* c, const PairArgs& A, int part, bool ev) {
  // a piece of the cell order (the host-step pipeline: no energies, full
  // list, no staging, checked by launch_forces)
  if (A.i0 != 0 || A.n != c->n) {
    if (ev) return set_error(c, GBMD_ERR_INVALID, "atom ranges: no energies or virials");
    return launch_mixed_shape<false, true>(c, A, part);
  }
  return ev ? launch_mixed_E<true>(c, A, part) : launch_mixed_E<false>(c, A, part);
}

}  // namespace gbmd
