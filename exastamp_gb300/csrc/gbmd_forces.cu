// gbmd_forces.cu -- LJ and eam_alloy pair kernels for sm_103a.
//
// FP64 kernels restate the reference arithmetic exactly:
//   LJ       lennard_jones.h L41-50 + force_op_impl2.hxx L33-68 (e -= ecut, de /= r,
//            fe = de*dr, ep += e/2, vir += -1/2 fe (x) dr)
//   LJ multi pair_potential_force_op_multiparam.h L92-118 (r <= rcut_pair test)
//   EAM      eam_alloy.h L198-313 + eam_force_op_multimat.h L114-343
// Mixed kernels evaluate the same functions in FP32 on home-cell-relative
// coordinates (dr = (p_j - p_i) + stencil shift, exact to ~1e-7 relative),
// accumulate forces, densities and energies with compensated (Kahan) FP32
// sums, and decide cutoff membership exactly as FP64 would: pairs whose FP32
// d2 lies within 2^-12 of rcut^2 are re-tested in FP64 from the FP64 state.
//
// Per-unit algorithmic work (per ordered list entry): 4 B of list, one 16 B
// (mixed) or 32 B (FP64) position gather, the cutoff test and, inside the
// cutoff, the pair function.
#include "gbmd_pair_common.cuh"

namespace gbmd {

// ---------------------------------------------------------------------------
// Lennard-Jones (single parameter set and per-type-pair tables)
// ---------------------------------------------------------------------------
struct LJSingle {
  double eps, sig, ecut, rc2;
  float sig2f, eps24f, eps4f, ecutf, rc2f, rc2lo, rc2hi;
};

struct LJShared {
  float sig2, eps24, eps4, ecut, rc2, rc2lo, rc2hi, pad;
};

template <int T, bool MIXED, bool EV, bool MULTI>
__global__ void __launch_bounds__(256) k_lj(PairArgs A, LJSingle P, const LJPair* __restrict__ tab, int ntypes,
                                            double rcmax2) {
  __shared__ LJShared sf[MULTI ? GBMD_MAX_TYPES * GBMD_MAX_TYPES : 1];
  __shared__ double sd[MULTI ? GBMD_MAX_TYPES * GBMD_MAX_TYPES * 5 : 1];
  if (MULTI) {
    for (int q = threadIdx.x; q < ntypes * ntypes; q += blockDim.x) {
      const LJPair& p = tab[q];
      sf[q] = LJShared{p.sig2f, p.eps24f, p.eps4f, p.ecutf, p.rc2f, p.rc2lo, p.rc2hi, 0.f};
      sd[5 * q + 0] = p.eps;
      sd[5 * q + 1] = p.sig;
      sd[5 * q + 2] = p.rc;
      sd[5 * q + 3] = p.ecut;
      sd[5 * q + 4] = p.rc2;
    }
    __syncthreads();
  }
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  int cx = 0, cy = 0, cz = 0, ti = 0;
  if (live) unpack_cell(A.cellpack[i], cx, cy, cz);

  if (MIXED) {
    float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
    float vxx = 0.f, vyy = 0.f, vzz = 0.f, vxy = 0.f, vxz = 0.f, vyz = 0.f;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (live) pi = A.posf[i];
    ti = __float_as_int(pi.w);
    const uint32_t* p = A.nbr + (size_t)i * T + lane;
    for (int k = lane; k < nn; k += T, p += A.stride) {
      const uint32_t ent = __ldg(p);
      const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
      const float4 pj = __ldg(&A.posf[j]);
      const float dx = (pj.x - pi.x) + code_shift(code & 3u, A.g.hf[0]);
      const float dy = (pj.y - pi.y) + code_shift((code >> 2) & 3u, A.g.hf[1]);
      const float dz = (pj.z - pi.z) + code_shift((code >> 4) & 3u, A.g.hf[2]);
      const float d2 = dx * dx + dy * dy + dz * dz;
      float sig2, eps24, eps4, ecut, rc2, rlo, rhi;
      int pid = 0;
      if (MULTI) {
        pid = ti * ntypes + __float_as_int(pj.w);
        const LJShared q = sf[pid];
        sig2 = q.sig2; eps24 = q.eps24; eps4 = q.eps4; ecut = q.ecut; rc2 = q.rc2; rlo = q.rc2lo; rhi = q.rc2hi;
      } else {
        sig2 = P.sig2f; eps24 = P.eps24f; eps4 = P.eps4f; ecut = P.ecutf; rc2 = P.rc2f; rlo = P.rc2lo; rhi = P.rc2hi;
      }
      (void)rc2;
      if (d2 > rhi) continue;
      if (d2 >= rlo) {
        const double4_32a di = A.posd[i], dj = A.posd[j];
        double Sx, Sy, Sz, a, b, c;
        image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
        const double d2x = exact_d2(di.x, di.y, di.z, dj.x, dj.y, dj.z, Sx, Sy, Sz, a, b, c);
        if (MULTI) {
          if (!(d2x <= rcmax2) || !(sqrt(d2x) <= sd[5 * pid + 2])) continue;
        } else {
          if (!(d2x <= P.rc2)) continue;
        }
      }
      const float r2inv = __frcp_rn(d2);
      const float s2 = sig2 * r2inv;
      const float s6 = s2 * s2 * s2;
      const float s12 = s6 * s6;
      const float fpair = eps24 * (2.f * s12 - s6) * r2inv;  // -(dE/dr)/r
      kahan_add(fx, cfx, -fpair * dx);
      kahan_add(fy, cfy, -fpair * dy);
      kahan_add(fz, cfz, -fpair * dz);
      if (EV) {
        kahan_add(e, ce, 0.5f * (eps4 * (s12 - s6) - ecut));
        const float h = 0.5f * fpair;
        vxx += h * dx * dx; vyy += h * dy * dy; vzz += h * dz * dz;
        vxy += h * dx * dy; vxz += h * dx * dz; vyz += h * dy * dz;
      }
    }
    group_reduce_kahan<T>(fx, cfx);
    group_reduce_kahan<T>(fy, cfy);
    group_reduce_kahan<T>(fz, cfz);
    if (EV) {
      group_reduce_kahan<T>(e, ce);
#pragma unroll
      for (int off = T / 2; off > 0; off >>= 1) {
        vxx += __shfl_xor_sync(0xffffffffu, vxx, off);
        vyy += __shfl_xor_sync(0xffffffffu, vyy, off);
        vzz += __shfl_xor_sync(0xffffffffu, vzz, off);
        vxy += __shfl_xor_sync(0xffffffffu, vxy, off);
        vxz += __shfl_xor_sync(0xffffffffu, vxz, off);
        vyz += __shfl_xor_sync(0xffffffffu, vyz, off);
      }
    }
    if (live && lane == 0) {
      const float im = A.inv_massf[ti];
      const float Fx = fx - cfx, Fy = fy - cfy, Fz = fz - cfz;
      double v9[9];
      if (EV) {
        v9[0] = vxx; v9[1] = vxy; v9[2] = vxz;
        v9[3] = vxy; v9[4] = vyy; v9[5] = vyz;
        v9[6] = vxz; v9[7] = vyz; v9[8] = vzz;
      }
      atom_epilogue<true>(A, i, ti, 0., 0., 0., Fx * im, Fy * im, Fz * im, EV ? (double)(e - ce) : 0.0,
                          EV ? v9 : nullptr);
    }
  } else {
    double fx = 0., fy = 0., fz = 0., e = 0.;
    double v[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};
    double4_32a pi = make_double4_32a(0., 0., 0., 0.);
    if (live) pi = A.posd[i];
    ti = (int)pi.w;
    const uint32_t* p = A.nbr + (size_t)i * T + lane;
    for (int k = lane; k < nn; k += T, p += A.stride) {
      const uint32_t ent = __ldg(p);
      const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
      const double4_32a pj = A.posd[j];
      double Sx, Sy, Sz, dx, dy, dz;
      image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
      const double d2 = exact_d2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, Sx, Sy, Sz, dx, dy, dz);
      double eps, sig, ecut;
      if (MULTI) {
        const int pid = ti * ntypes + (int)pj.w;
        if (!(d2 <= rcmax2)) continue;
        const double r = sqrt(d2);
        if (!(r <= sd[5 * pid + 2])) continue;
        eps = sd[5 * pid]; sig = sd[5 * pid + 1]; ecut = sd[5 * pid + 3];
      } else {
        if (!(d2 <= P.rc2)) continue;
        eps = P.eps; sig = P.sig; ecut = P.ecut;
      }
      const double r = sqrt(d2);
      const double ratio = sig / r;
      const double ratio2 = ratio * ratio;
      const double ratio6 = ratio2 * ratio2 * ratio2;
      const double ratio12 = ratio6 * ratio6;
      double ee = 4. * eps * (ratio12 - ratio6);
      double de = (-24. * eps * (2. * ratio12 - ratio6)) / r;
      ee -= ecut;
      de /= r;
      const double fex = de * dx, fey = de * dy, fez = de * dz;
      fx += fex; fy += fey; fz += fez;
      if (EV) {
        e += .5 * ee;
        v[0] += fex * dx * -0.5; v[1] += fex * dy * -0.5; v[2] += fex * dz * -0.5;
        v[3] += fey * dx * -0.5; v[4] += fey * dy * -0.5; v[5] += fey * dz * -0.5;
        v[6] += fez * dx * -0.5; v[7] += fez * dy * -0.5; v[8] += fez * dz * -0.5;
      }
    }
    fx = group_reduce_d<T>(fx);
    fy = group_reduce_d<T>(fy);
    fz = group_reduce_d<T>(fz);
    if (EV) {
      e = group_reduce_d<T>(e);
#pragma unroll
      for (int q = 0; q < 9; ++q) v[q] = group_reduce_d<T>(v[q]);
    }
    if (live && lane == 0) atom_epilogue<false>(A, i, ti, fx, fy, fz, 0.f, 0.f, 0.f, e, EV ? v : nullptr);
  }
}

// ---------------------------------------------------------------------------
// eam_alloy: density + embedding (one kernel), force (second kernel)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int r_knot_f(float r, float rdr, int nr, float& p) {
  float pp = r * rdr + 1.0f;
  int m = (int)pp;
  m = min(m, nr - 1);
  pp -= (float)m;
  p = fminf(pp, 1.0f);
  return m;
}

__device__ __forceinline__ int r_knot_d(double r, double rdr, int nr, double& p) {
  double pp = r * rdr + 1.0;
  int m = (int)pp;
  m = min(m, nr - 1);
  pp -= m;
  p = fmin(pp, 1.0);
  return m;
}

template <int T, bool MIXED, bool EV>
__global__ void __launch_bounds__(256) k_eam_rho(PairArgs A, EamDev E, float* __restrict__ fpf,
                                                 double* __restrict__ fpd, float* __restrict__ epf) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  int cx = 0, cy = 0, cz = 0;
  if (live) unpack_cell(A.cellpack[i], cx, cy, cz);
  if (MIXED) {
    float rho = 0.f, crho = 0.f;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (live) pi = A.posf[i];
    const int ti = __float_as_int(pi.w);
    const uint32_t* p = A.nbr + (size_t)i * T + lane;
    for (int k = lane; k < nn; k += T, p += A.stride) {
      const uint32_t ent = __ldg(p);
      const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
      const float4 pj = __ldg(&A.posf[j]);
      const float dx = (pj.x - pi.x) + code_shift(code & 3u, A.g.hf[0]);
      const float dy = (pj.y - pi.y) + code_shift((code >> 2) & 3u, A.g.hf[1]);
      const float dz = (pj.z - pi.z) + code_shift((code >> 4) & 3u, A.g.hf[2]);
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (d2 > E.rc2hi) continue;
      if (d2 >= E.rc2lo) {
        const double4_32a di = A.posd[i], dj = A.posd[j];
        double Sx, Sy, Sz, a, b, c;
        image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
        if (!(exact_d2(di.x, di.y, di.z, dj.x, dj.y, dj.z, Sx, Sy, Sz, a, b, c) <= E.rcut2)) continue;
      }
      const float r = sqrtf(d2);
      float q;
      const int m = r_knot_f(r, E.rdrf, E.nr, q);
      const float4 cf = __ldg(&E.rhor4[(size_t)__float_as_int(pj.w) * (E.nr + 1) + m]);
      kahan_add(rho, crho, ((cf.x * q + cf.y) * q + cf.z) * q + cf.w);
    }
    group_reduce_kahan<T>(rho, crho);
    if (live && lane == 0) {
      const float R = rho - crho;
      float q = R * E.rdrhof + 1.0f;
      int m = (int)q;
      m = max(1, min(m, E.nrho - 1));
      q -= (float)m;
      q = fminf(q, 1.0f);
      const float4 c = __ldg(&E.frho4[(size_t)ti * (E.nrho + 1) + m]);
      const float fp = ((3.f * c.x * q + 2.f * c.y) * q + c.z) * E.rdrhof;
      float phi = ((c.x * q + c.y) * q + c.z) * q + c.w;
      if (R > E.rhomaxf) phi += fp * (R - E.rhomaxf);
      fpf[i] = fp;
      if (EV) epf[i] = phi;
    }
  } else {
    double rho = 0.;
    double4_32a pi = make_double4_32a(0., 0., 0., 0.);
    if (live) pi = A.posd[i];
    const int ti = (int)pi.w;
    const uint32_t* p = A.nbr + (size_t)i * T + lane;
    for (int k = lane; k < nn; k += T, p += A.stride) {
      const uint32_t ent = __ldg(p);
      const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
      const double4_32a pj = A.posd[j];
      double Sx, Sy, Sz, dx, dy, dz;
      image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
      const double d2 = exact_d2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, Sx, Sy, Sz, dx, dy, dz);
      if (!(d2 <= E.rcut2)) continue;
      double q;
      const int m = r_knot_d(sqrt(d2), E.rdr, E.nr, q);
      const double* c = E.rhor + ((size_t)(int)pj.w * (E.nr + 1) + m) * 8;
      rho += ((c[3] * q + c[4]) * q + c[5]) * q + c[6];
    }
    rho = group_reduce_d<T>(rho);
    if (live && lane == 0) {
      double q = rho * E.rdrho + 1.0;
      int m = (int)q;
      m = max(1, min(m, E.nrho - 1));
      q -= m;
      q = fmin(q, 1.0);
      const double* c = E.frho + ((size_t)ti * (E.nrho + 1) + m) * 8;
      double fp = (c[0] * q + c[1]) * q + c[2];
      double phi = ((c[3] * q + c[4]) * q + c[5]) * q + c[6];
      if (rho > E.rhomax) phi += fp * (rho - E.rhomax);
      phi *= E.conv_frho;
      fp *= E.conv_frho;
      fpd[i] = fp;
      if (EV) A.ep[i] = phi;
    }
  }
}

__device__ __forceinline__ int z2r_index(int a, int b) {
  const int irow = a > b ? a : b, icol = a > b ? b : a;
  return irow * (irow + 1) / 2 + icol;
}

template <int T, bool MIXED, bool EV>
__global__ void __launch_bounds__(256) k_eam_force(PairArgs A, EamDev E, const float* __restrict__ fpf,
                                                   const double* __restrict__ fpd, const float* __restrict__ epf) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  int cx = 0, cy = 0, cz = 0;
  if (live) unpack_cell(A.cellpack[i], cx, cy, cz);
  if (MIXED) {
    float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
    float vxx = 0.f, vyy = 0.f, vzz = 0.f, vxy = 0.f, vxz = 0.f, vyz = 0.f;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    float fpi = 0.f;
    if (live) {
      pi = A.posf[i];
      fpi = fpf[i];
    }
    const int ti = __float_as_int(pi.w);
    const uint32_t* p = A.nbr + (size_t)i * T + lane;
    const float rdr = E.rdrf;
    for (int k = lane; k < nn; k += T, p += A.stride) {
      const uint32_t ent = __ldg(p);
      const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
      const float4 pj = __ldg(&A.posf[j]);
      const float dx = (pj.x - pi.x) + code_shift(code & 3u, A.g.hf[0]);
      const float dy = (pj.y - pi.y) + code_shift((code >> 2) & 3u, A.g.hf[1]);
      const float dz = (pj.z - pi.z) + code_shift((code >> 4) & 3u, A.g.hf[2]);
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (d2 > E.rc2hi) continue;
      if (d2 >= E.rc2lo) {
        const double4_32a di = A.posd[i], dj = A.posd[j];
        double Sx, Sy, Sz, a, b, c;
        image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
        if (!(exact_d2(di.x, di.y, di.z, dj.x, dj.y, dj.z, Sx, Sy, Sz, a, b, c) <= E.rcut2)) continue;
      }
      const int tj = __float_as_int(pj.w);
      const float r = sqrtf(d2);
      const float recip = __frcp_rn(r);
      float q;
      const int m = r_knot_f(r, rdr, E.nr, q);
      const float4 cj = __ldg(&E.rhor4[(size_t)tj * (E.nr + 1) + m]);
      const float rhojp = ((3.f * cj.x * q + 2.f * cj.y) * q + cj.z) * rdr;
      float rhoip = rhojp;
      if (E.nel > 1 && ti != tj) {
        const float4 ci = __ldg(&E.rhor4[(size_t)ti * (E.nr + 1) + m]);
        rhoip = ((3.f * ci.x * q + 2.f * ci.y) * q + ci.z) * rdr;
      }
      const float4 cz2 = __ldg(&E.z2r4[(size_t)z2r_index(ti, tj) * (E.nr + 1) + m]);
      const float z2p = ((3.f * cz2.x * q + 2.f * cz2.y) * q + cz2.z) * rdr;
      const float z2 = ((cz2.x * q + cz2.y) * q + cz2.z) * q + cz2.w;
      const float phi = z2 * recip;
      const float phip = z2p * recip - phi * recip;
      const float fpj = __ldg(&fpf[j]);
      const float psip = fpi * rhojp + fpj * rhoip + phip;
      const float fpair = psip * recip;
      kahan_add(fx, cfx, dx * fpair);
      kahan_add(fy, cfy, dy * fpair);
      kahan_add(fz, cfz, dz * fpair);
      if (EV) {
        kahan_add(e, ce, 0.5f * phi);
        const float h = -0.5f * fpair;
        vxx += h * dx * dx; vyy += h * dy * dy; vzz += h * dz * dz;
        vxy += h * dx * dy; vxz += h * dx * dz; vyz += h * dy * dz;
      }
    }
    group_reduce_kahan<T>(fx, cfx);
    group_reduce_kahan<T>(fy, cfy);
    group_reduce_kahan<T>(fz, cfz);
    if (EV) {
      group_reduce_kahan<T>(e, ce);
#pragma unroll
      for (int off = T / 2; off > 0; off >>= 1) {
        vxx += __shfl_xor_sync(0xffffffffu, vxx, off);
        vyy += __shfl_xor_sync(0xffffffffu, vyy, off);
        vzz += __shfl_xor_sync(0xffffffffu, vzz, off);
        vxy += __shfl_xor_sync(0xffffffffu, vxy, off);
        vxz += __shfl_xor_sync(0xffffffffu, vxz, off);
        vyz += __shfl_xor_sync(0xffffffffu, vyz, off);
      }
    }
    if (live && lane == 0) {
      const float im = A.inv_massf[ti];
      double v9[9];
      if (EV) {
        v9[0] = vxx; v9[1] = vxy; v9[2] = vxz;
        v9[3] = vxy; v9[4] = vyy; v9[5] = vyz;
        v9[6] = vxz; v9[7] = vyz; v9[8] = vzz;
      }
      const double epv = EV ? (double)epf[i] + (double)(e - ce) : 0.0;
      atom_epilogue<true>(A, i, ti, 0., 0., 0., (fx - cfx) * im, (fy - cfy) * im, (fz - cfz) * im, epv,
                          EV ? v9 : nullptr);
    }
  } else {
    double fx = 0., fy = 0., fz = 0., e = 0.;
    double v[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};
    double4_32a pi = make_double4_32a(0., 0., 0., 0.);
    double fpi = 0.;
    if (live) {
      pi = A.posd[i];
      fpi = fpd[i];
    }
    const int ti = (int)pi.w;
    const uint32_t* p = A.nbr + (size_t)i * T + lane;
    for (int k = lane; k < nn; k += T, p += A.stride) {
      const uint32_t ent = __ldg(p);
      const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
      const double4_32a pj = A.posd[j];
      double Sx, Sy, Sz, dx, dy, dz;
      image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
      const double d2 = exact_d2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, Sx, Sy, Sz, dx, dy, dz);
      if (!(d2 <= E.rcut2)) continue;
      const int tj = (int)pj.w;
      const double r = sqrt(d2);
      double q;
      const int m = r_knot_d(r, E.rdr, E.nr, q);
      const double* ci = E.rhor + ((size_t)ti * (E.nr + 1) + m) * 8;
      const double rhoip = (ci[0] * q + ci[1]) * q + ci[2];
      const double* cj = E.rhor + ((size_t)tj * (E.nr + 1) + m) * 8;
      const double rhojp = (cj[0] * q + cj[1]) * q + cj[2];
      const double* c = E.z2r + ((size_t)z2r_index(ti, tj) * (E.nr + 1) + m) * 8;
      const double z2p = (c[0] * q + c[1]) * q + c[2];
      const double z2 = ((c[3] * q + c[4]) * q + c[5]) * q + c[6];
      const double recip = 1.0 / r;
      double phi = z2 * recip;
      const double phip = (z2p * recip - phi * recip) * E.conv_z2r;
      phi *= E.conv_z2r;
      const double psip = fpi * rhojp + __ldg(&fpd[j]) * rhoip + phip;
      const double fpair = psip * recip;
      const double fex = dx * fpair, fey = dy * fpair, fez = dz * fpair;
      fx += fex; fy += fey; fz += fez;
      if (EV) {
        e += .5 * phi;
        v[0] += fex * dx * -0.5; v[1] += fex * dy * -0.5; v[2] += fex * dz * -0.5;
        v[3] += fey * dx * -0.5; v[4] += fey * dy * -0.5; v[5] += fey * dz * -0.5;
        v[6] += fez * dx * -0.5; v[7] += fez * dy * -0.5; v[8] += fez * dz * -0.5;
      }
    }
    fx = group_reduce_d<T>(fx);
    fy = group_reduce_d<T>(fy);
    fz = group_reduce_d<T>(fz);
    if (EV) {
      e = group_reduce_d<T>(e);
#pragma unroll
      for (int q = 0; q < 9; ++q) v[q] = group_reduce_d<T>(v[q]);
    }
    if (live && lane == 0) {
      const double epv = EV ? A.ep[i] + e : 0.0;
      atom_epilogue<false>(A, i, ti, fx, fy, fz, 0.f, 0.f, 0.f, epv, EV ? v : nullptr);
    }
  }
}

// ---------------------------------------------------------------------------
// host dispatch
// ---------------------------------------------------------------------------
static PairArgs make_args(gbmd_context* c, const ForceFlags& f) {
  PairArgs A;
  A.n = c->n;
  A.stride = c->npad * c->tpa;
  A.nbr = c->nbr;
  A.nnb = c->nnb;
  A.maxnb = c->maxnb;
  A.posf = c->POSF();
  A.posd = c->POSD();
  A.cellpack = c->cellpack;
  A.g = c->grid;
  A.x = c->X();
  A.y = c->Y();
  A.z = c->Z();
  const int o = c->cur ^ 1;
  A.xo = c->rbuf[o];
  A.yo = c->rbuf[o] + c->cap;
  A.zo = c->rbuf[o] + 2 * c->cap;
  A.posf_o = c->posf[o];
  A.posd_o = c->posd[o];
  A.vx = c->VX(); A.vy = c->VY(); A.vz = c->VZ();
  A.ax = c->AX(); A.ay = c->AY(); A.az = c->AZ();
  A.ep = c->ep;
  A.vir = c->vir;
  A.type = c->TYPE();
  for (int t = 0; t < GBMD_MAX_TYPES; ++t) {
    A.mass[t] = t < c->ntypes ? c->mass[t] : 1.0;
    A.inv_massf[t] = (float)(1.0 / A.mass[t]);
  }
  A.fuse = f.fuse;
  A.want_energy = f.energy ? 1 : 0;
  A.want_virial = f.virial ? 1 : 0;
  A.dt = f.sp.dt;
  A.dth = f.sp.dth;
  A.dt2h = f.sp.dt2h;
  A.err = c->d_err;
  return A;
}

// part: 0 = the whole force evaluation, 1 = EAM density+embedding only,
// 2 = the final pair kernel only (used by the per-kernel profiler)
template <int T, bool MIXED, bool EV>
static void launch_T(gbmd_context* c, const PairArgs& A, int part) {
  const int B = c->block;
  const unsigned grid = (unsigned)((A.n * T + B - 1) / B);
  cudaStream_t s = c->stream;
  if (c->pot != GBMD_POT_EAM_ALLOY && part == 1) return;
  if (c->pot == GBMD_POT_LJ) {
    const LJPair& p = c->lj.p[0];
    LJSingle P{p.eps, p.sig, p.ecut, p.rc2, p.sig2f, p.eps24f, p.eps4f, p.ecutf, p.rc2f, p.rc2lo, p.rc2hi};
    k_lj<T, MIXED, EV, false><<<grid, B, 0, s>>>(A, P, nullptr, 1, c->lj.rcut_max2);
  } else if (c->pot == GBMD_POT_LJ_MULTI) {
    LJSingle P{};
    k_lj<T, MIXED, EV, true><<<grid, B, 0, s>>>(A, P, c->lj_tab_d,
                                                c->lj.ntypes, c->lj.rcut_max2);
  } else {
    if (part != 2) k_eam_rho<T, MIXED, EV><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->fpd, c->epf);
    if (part != 1) k_eam_force<T, MIXED, EV><<<grid, B, 0, s>>>(A, c->eam, c->fpf, c->fpd, c->epf);
  }
}

template <bool MIXED, bool EV>
static int launch_P(gbmd_context* c, const PairArgs& A, int part) {
  switch (c->tpa) {
    case 1: launch_T<1, MIXED, EV>(c, A, part); break;
    case 2: launch_T<2, MIXED, EV>(c, A, part); break;
    case 4: launch_T<4, MIXED, EV>(c, A, part); break;
    case 8: launch_T<8, MIXED, EV>(c, A, part); break;
    case 16: launch_T<16, MIXED, EV>(c, A, part); break;
    default: return set_error(c, GBMD_ERR_INVALID, "unsupported lanes per atom %d", c->tpa);
  }
  return GBMD_OK;
}

int launch_forces(gbmd_context* c, const ForceFlags& f) {
  if (c->n == 0) return GBMD_OK;
  // every atom type must index the potential's tables (types < ntypes is
  // checked at upload)
  if (c->pot == GBMD_POT_EAM_ALLOY && c->ntypes > c->eam.nel)
    return set_error(c, GBMD_ERR_INVALID, "%d species but the setfl tables hold %d elements", c->ntypes, c->eam.nel);
  if (c->pot == GBMD_POT_LJ_MULTI && c->ntypes > c->lj.ntypes)
    return set_error(c, GBMD_ERR_INVALID, "%d species but the LJ tables cover %d types", c->ntypes, c->lj.ntypes);
  if (!c->list_valid || !c->nbr) return set_error(c, GBMD_ERR_INVALID, "neighbour list not built");
  const PairArgs A = make_args(c, f);
  const bool ev = f.energy || f.virial;
  const bool mixed = c->precision == GBMD_PRECISION_MIXED;
  const int part = f.part;
  int rc;
  if (mixed) rc = ev ? launch_P<true, true>(c, A, part) : launch_P<true, false>(c, A, part);
  else rc = ev ? launch_P<false, true>(c, A, part) : launch_P<false, false>(c, A, part);
  if (rc) return rc;
  if (f.fuse == FUSE_PUSH2_PUSH1 && part != 1) c->cur ^= 1;
  return GBMD_OK;
}

}  // namespace gbmd
