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
// Loop structure (per list entry): one coalesced 4 B list load, one 16 B
// position gather (plus 4 B F'(rho_j) for the EAM force pass), one 16 B
// spline-knot gather per table; branch-free except the rare FP64 re-test.
// 1/r and r come from one rsqrt; the stencil offset decodes to an exact
// float in two integer/FP ops per axis.
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

// List-entry prefetch: each thread streams its own list slots through a
// ring of LIST_RING words in shared memory with cp.async (4 B, L1-cached),
// LIST_RING - 1 entries ahead of the one being processed.  The slot refilled
// at iteration `it` is the one consumed at `it - 1`, whose value is already
// in a register.  Ring layout [slot][thread]: conflict-free.
constexpr int LIST_RING = 8;

__device__ __forceinline__ void cp_async4(uint32_t* smem, const uint32_t* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_ring() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(LIST_RING - 2) : "memory");
}
__device__ __forceinline__ void cp_async_drain() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

static_assert((LIST_RING & (LIST_RING - 1)) == 0, "ring size must be a power of two");

struct ListStream {
  uint32_t* ring;          // this thread's column: ring[slot * blockDim.x]
  const uint32_t* p;       // this thread's first list slot, then the next slot to prefetch
  int64_t stride;
  int niter;
  __device__ __forceinline__ void start() {
#pragma unroll
    for (int d = 0; d < LIST_RING - 1; ++d) {
      if (d < niter) cp_async4(ring + d * blockDim.x, p);
      cp_async_commit();
      p += stride;
    }
  }
  __device__ __forceinline__ uint32_t next(int it) {
    cp_async_wait_ring();
    const unsigned u = (unsigned)it;
    const uint32_t e = ring[(u & (LIST_RING - 1)) * blockDim.x];
    if ((int)(u + LIST_RING - 1) < niter) cp_async4(ring + ((u - 1) & (LIST_RING - 1)) * blockDim.x, p);
    cp_async_commit();
    p += stride;
    return e;
  }
};

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

// ---------------------------------------------------------------------------
// Lennard-Jones
// ---------------------------------------------------------------------------
struct LJF {
  float sig2, eps24, eps4, ecut, rc2lo, rc2hi;
  double rc2, rc;
};

template <int T, bool EV, bool MULTI>
__global__ void __launch_bounds__(256) k_lj_mixed(PairArgs A, LJF P, const LJPair* __restrict__ tab, int ntypes,
                                                  double rcmax2) {
  __shared__ float4 sfa[MULTI ? GBMD_MAX_TYPES * GBMD_MAX_TYPES : 1];   // sig2, eps24, eps4, ecut
  __shared__ float2 sfb[MULTI ? GBMD_MAX_TYPES * GBMD_MAX_TYPES : 1];   // rc2lo, rc2hi
  __shared__ double sfr[MULTI ? GBMD_MAX_TYPES * GBMD_MAX_TYPES : 1];   // rc
  if (MULTI) {
    for (int q = threadIdx.x; q < ntypes * ntypes; q += blockDim.x) {
      const LJPair& p = tab[q];
      sfa[q] = make_float4(p.sig2f, p.eps24f, p.eps4f, p.ecutf);
      sfb[q] = make_float2(p.rc2lo, p.rc2hi);
      sfr[q] = p.rc;
    }
    __syncthreads();
  }
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  const float4 pi = live ? A.posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int cp = live ? A.cellpack[i] : 0;
  const int ti = __float_as_int(pi.w);
  float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  __shared__ uint32_t ring_sm[LIST_RING * 256];
  ListStream ls{ring_sm + threadIdx.x, A.nbr + (size_t)i * T + lane, A.stride, nn > lane ? (nn - lane + T - 1) / T : 0};
  ls.start();
#pragma unroll 2
  for (int it = 0; it < ls.niter; ++it) {
    const uint32_t ent = ls.next(it);
    const uint32_t j = ent & GBMD_IDX_MASK;
    const float4 pj = __ldg(&A.posf[j]);
    const GeomF G = geom_f(ent, pj, pi, A.g);
    float sig2, eps24, eps4, ecut, rlo, rhi;
    double rcp = 0.0, rc2 = P.rc2;
    if (MULTI) {
      const int pid = ti * ntypes + __float_as_int(pj.w);
      const float4 a = sfa[pid];
      const float2 b = sfb[pid];
      sig2 = a.x; eps24 = a.y; eps4 = a.z; ecut = a.w; rlo = b.x; rhi = b.y;
      rcp = sfr[pid];
      rc2 = rcmax2;
    } else {
      sig2 = P.sig2; eps24 = P.eps24; eps4 = P.eps4; ecut = P.ecut; rlo = P.rc2lo; rhi = P.rc2hi;
    }
    bool in = G.d2 < rlo;
    if (!in && G.d2 <= rhi) in = exact_inside(A.posd, i, j, ent >> GBMD_IDX_BITS, cp, A.g, rc2, rcp);
    const float r2i = __frcp_rn(G.d2);
    const float s2 = sig2 * r2i;
    const float s6 = s2 * s2 * s2;
    const float s12 = s6 * s6;
    const float fpair = in ? eps24 * fmaf(2.f, s12, -s6) * r2i : 0.f;  // -(dE/dr)/r
    kahan_add(fx, cfx, -fpair * G.dx);
    kahan_add(fy, cfy, -fpair * G.dy);
    kahan_add(fz, cfz, -fpair * G.dz);
    if (EV) {
      kahan_add(e, ce, in ? 0.5f * fmaf(eps4, s12 - s6, -ecut) : 0.f);
      const float h = 0.5f * fpair;
      v[0] = fmaf(h * G.dx, G.dx, v[0]);
      v[1] = fmaf(h * G.dy, G.dy, v[1]);
      v[2] = fmaf(h * G.dz, G.dz, v[2]);
      v[3] = fmaf(h * G.dx, G.dy, v[3]);
      v[4] = fmaf(h * G.dx, G.dz, v[4]);
      v[5] = fmaf(h * G.dy, G.dz, v[5]);
    }
  }
  cp_async_drain();
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

template <int T, bool EV, bool SINGLE>
__global__ void __launch_bounds__(256) k_eam_rho_mixed(PairArgs A, EamDev E, float* __restrict__ fpf,
                                                       float* __restrict__ epf) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  const float4 pi = live ? A.posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int cp = live ? A.cellpack[i] : 0;
  const int ti = __float_as_int(pi.w);
  const int nr = E.nr, nr1 = E.nr + 1;
  const float rdr = E.rdrf;
  float rho = 0.f, crho = 0.f;
  __shared__ uint32_t ring_sm[LIST_RING * 256];
  ListStream ls{ring_sm + threadIdx.x, A.nbr + (size_t)i * T + lane, A.stride, nn > lane ? (nn - lane + T - 1) / T : 0};
  ls.start();
#pragma unroll 2
  for (int it = 0; it < ls.niter; ++it) {
    const uint32_t ent = ls.next(it);
    const uint32_t j = ent & GBMD_IDX_MASK;
    const float4 pj = __ldg(&A.posf[j]);
    const GeomF G = geom_f(ent, pj, pi, A.g);
    bool in = G.d2 < E.rc2lo;
    if (!in && G.d2 <= E.rc2hi) in = exact_inside(A.posd, i, j, ent >> GBMD_IDX_BITS, cp, A.g, E.rcut2, 0.0);
    const float r = G.d2 * rsqrtf(G.d2);
    float q;
    const int m = knot_f(r, rdr, nr, q);
    const float4 c = __ldg(&E.rhor4[SINGLE ? m : __float_as_int(pj.w) * nr1 + m]);
    kahan_add(rho, crho, in ? spline_val(c, q) : 0.f);
  }
  cp_async_drain();
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
    if (EV) {
      float phi = spline_val(c, q);
      if (R > E.rhomaxf) phi = fmaf(fp, R - E.rhomaxf, phi);
      epf[i] = phi;
    }
  }
}

__device__ __forceinline__ int z2r_index_d(int a, int b) {
  const int irow = a > b ? a : b, icol = a > b ? b : a;
  return irow * (irow + 1) / 2 + icol;
}

template <int T, bool EV, bool SINGLE>
__global__ void __launch_bounds__(256) k_eam_force_mixed(PairArgs A, EamDev E, const float* __restrict__ fpf,
                                                         const float* __restrict__ epf) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  const float4 pi = live ? A.posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int cp = live ? A.cellpack[i] : 0;
  const float fpi = live ? fpf[i] : 0.f;
  const int ti = __float_as_int(pi.w);
  const int nr = E.nr, nr1 = E.nr + 1;
  const float rdr = E.rdrf;
  float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  __shared__ uint32_t ring_sm[LIST_RING * 256];
  ListStream ls{ring_sm + threadIdx.x, A.nbr + (size_t)i * T + lane, A.stride, nn > lane ? (nn - lane + T - 1) / T : 0};
  ls.start();
  // the force sums take two pair terms per compensated add: the pair of
  // terms is rounded once (relative 6e-8 of the larger term), then the sum
  // is compensated
  float px = 0.f, py = 0.f, pz = 0.f;
#pragma unroll 2
  for (int it = 0; it < ls.niter; ++it) {
    const uint32_t ent = ls.next(it);
    const uint32_t j = ent & GBMD_IDX_MASK;
    const float4 pj = __ldg(&A.posf[j]);
    const float fpj = __ldg(&fpf[j]);
    const GeomF G = geom_f(ent, pj, pi, A.g);
    bool in = G.d2 < E.rc2lo;
    if (!in && G.d2 <= E.rc2hi) in = exact_inside(A.posd, i, j, ent >> GBMD_IDX_BITS, cp, A.g, E.rcut2, 0.0);
    const float rs = rsqrtf(G.d2);
    const float r = G.d2 * rs;
    float q;
    const int m = knot_f(r, rdr, nr, q);
    const int tj = __float_as_int(pj.w);
    // rho'(r) from the pre-scaled derivative table: (3c3/dr, 2c4/dr, c5/dr)
    const float4 dj = __ldg(&E.rhod4[SINGLE ? m : tj * nr1 + m]);
    const float rhojp = fmaf(fmaf(dj.x, q, dj.y), q, dj.z);
    float rhoip = rhojp;
    if (!SINGLE && ti != tj) {
      const float4 di = __ldg(&E.rhod4[ti * nr1 + m]);
      rhoip = fmaf(fmaf(di.x, q, di.y), q, di.z);
    }
    const float4 cz = __ldg(&E.z2r4[SINGLE ? m : z2r_index_d(ti, tj) * nr1 + m]);
    const float t1 = fmaf(cz.x, q, cz.y);
    const float z2 = fmaf(fmaf(t1, q, cz.z), q, cz.w);          // z2r tables carry conv_z2r
    const float z2d = fmaf(fmaf(cz.x, q, t1 + t1), q, cz.z);     // d z2 / d q
    const float phi = z2 * rs;
    const float phip = fmaf(z2d * rdr, rs, -phi * rs);
    const float psip = fmaf(fpi, rhojp, fmaf(fpj, rhoip, phip));
    const float fpair = in ? psip * rs : 0.f;
    if (it & 1) {
      kahan_add(fx, cfx, fmaf(G.dx, fpair, px));
      kahan_add(fy, cfy, fmaf(G.dy, fpair, py));
      kahan_add(fz, cfz, fmaf(G.dz, fpair, pz));
    } else {
      px = G.dx * fpair;
      py = G.dy * fpair;
      pz = G.dz * fpair;
    }
    if (EV) {
      kahan_add(e, ce, in ? 0.5f * phi : 0.f);
      const float h = -0.5f * fpair;
      v[0] = fmaf(h * G.dx, G.dx, v[0]);
      v[1] = fmaf(h * G.dy, G.dy, v[1]);
      v[2] = fmaf(h * G.dz, G.dz, v[2]);
      v[3] = fmaf(h * G.dx, G.dy, v[3]);
      v[4] = fmaf(h * G.dx, G.dz, v[4]);
      v[5] = fmaf(h * G.dy, G.dz, v[5]);
    }
  }
  if (ls.niter & 1) {  // a last unpaired term
    kahan_add(fx, cfx, px);
    kahan_add(fy, cfy, py);
    kahan_add(fz, cfz, pz);
  }
  cp_async_drain();
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

// ---------------------------------------------------------------------------
// dispatch
// ---------------------------------------------------------------------------
template <int T, bool EV>
static void launch_mixed_T(gbmd_context* c, const PairArgs& A, int part) {
  const int B = c->block;
  const unsigned grid = (unsigned)((A.n * T + B - 1) / B);
  cudaStream_t s = c->stream;
  if (c->pot == GBMD_POT_LJ) {
    if (part == 1) return;
    const LJPair& q = c->lj.p[0];
    LJF P{q.sig2f, q.eps24f, q.eps4f, q.ecutf, q.rc2lo, q.rc2hi, q.rc2, q.rc};
    k_lj_mixed<T, EV, false><<<grid, B, 0, s>>>(A, P, nullptr, 1, c->lj.rcut_max2);
  } else if (c->pot == GBMD_POT_LJ_MULTI) {
    if (part == 1) return;
    LJF P{};
    k_lj_mixed<T, EV, true><<<grid, B, 0, s>>>(A, P, c->lj_tab_d, c->lj.ntypes, c->lj.rcut_max2);
  } else if (c->eam.nel == 1) {
    if (part != 2) k_eam_rho_mixed<T, EV, true><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->epf);
    if (part != 1) k_eam_force_mixed<T, EV, true><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->epf);
  } else {
    if (part != 2) k_eam_rho_mixed<T, EV, false><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->epf);
    if (part != 1) k_eam_force_mixed<T, EV, false><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->epf);
  }
}

template <bool EV>
static int launch_mixed_E(gbmd_context* c, const PairArgs& A, int part) {
  switch (c->tpa) {
    case 1: launch_mixed_T<1, EV>(c, A, part); break;
    case 2: launch_mixed_T<2, EV>(c, A, part); break;
    case 4: launch_mixed_T<4, EV>(c, A, part); break;
    case 8: launch_mixed_T<8, EV>(c, A, part); break;
    case 16: launch_mixed_T<16, EV>(c, A, part); break;
    default: return set_error(c, GBMD_ERR_INVALID, "unsupported lanes per atom %d", c->tpa);
  }
  return GBMD_OK;
}

int launch_mixed(gbmd_context* c, const PairArgs& A, int part, bool ev) {
  return ev ? launch_mixed_E<true>(c, A, part) : launch_mixed_E<false>(c, A, part);
}

}  // namespace gbmd
