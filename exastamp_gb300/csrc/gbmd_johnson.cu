// gbmd_johnson.cu -- the analytic single-element EAM operators run by the
// mono-material two-pass template (eam_potential.cu L69-193,
// eam_force_op_singlemat.h L39-171):
//
//   pass 1 (EmbOp):   rho_i = sum_j rho(r_ij);  ep_i = F(rho_i);  F'_i kept
//   pass 2 (ForceOp): de = (rho'(r) (F'_i + F'_j) + phi'(r)) / r
//                     f_i += de * (r_j - r_i);  ep_i += phi/2;  vir_i += -f (x) dr / 2
//
// johnson_force (src/potential/eam_potentials/johnson/johnson.h L28-176):
//   phi(r) = A e^{-alpha (x-1)} / (1 + (x-kappa)^20) - B e^{-beta (x-1)} / (1 + (x-lambda)^20)
//   rho(r) = fe e^{-beta (x-1)} / (1 + (x-lambda)^20),   x = r / re
//   F(rho): cubic in (rho/rhon - 1) below rhon = 0.85 rhoe, cubic in
//           (rho/rhoe - 1) below rho0 = 1.15 rhoe, Fo (1 - ln s) s with
//           s = (rho/rhoe)^eta above.
// sutton_chen_force (src/potential/eam_potentials/sutton_chen/sutton_chen.h
// L30-67):
//   phi(r) = epsilon (a0/r)^n,  rho(r) = (a0/r)^m,  F(rho) = -c epsilon sqrt(rho)
//
// The kernels take the functions from a policy (JohnsonFns, SuttonChenFns).
// FP64 kernels use the reference's formulas in the same order; the mixed
// kernels evaluate the same functions in FP32 on the cell-relative
// coordinates of the main mixed path, with compensated sums, FP64 embedding
// and FP64 state.  Pair membership (r <= rcut) is exact in both: FP64
// directly, mixed through the FP32 screen and the FP64 re-test of the 2^-12
// band.
#include <cmath>

#include "gbmd_pair_common.cuh"

namespace gbmd {

// --------------------------------------------------------------------------
// the three functions, FP64 (johnson.h L55-176)
// --------------------------------------------------------------------------
__device__ __forceinline__ void ej_term_d(double pre, double k, double x, double c, double ire, double& v,
                                          double& dv) {
  const double c1 = pre * exp(-k * (x - 1.));
  const double c2 = x - c;
  const double c3 = pow(c2, 20);
  const double den = 1. + c3;
  const double dnum = -k * c1;
  const double dden = 20 * c3 / c2;
  v += c1 / den;
  dv += ire * (dnum * den - c1 * dden) / (den * den);
}

__device__ __forceinline__ void ej_phi_d(const JohnsonDev& p, double r, double& phi, double& dphi) {
  const double x = r / p.re, ire = 1. / p.re;
  phi = 0.;
  dphi = 0.;
  ej_term_d(p.A, p.alpha, x, p.kappa, ire, phi, dphi);
  ej_term_d(-p.B, p.beta, x, p.lambda, ire, phi, dphi);
}

__device__ __forceinline__ void ej_rho_d(const JohnsonDev& p, double r, double& rho, double& drho) {
  const double x = r / p.re, ire = 1. / p.re;
  rho = 0.;
  drho = 0.;
  ej_term_d(p.fe, p.beta, x, p.lambda, ire, rho, drho);
}

__device__ __forceinline__ void ej_embed_d(const JohnsonDev& p, double rho, double& f, double& df) {
  const double rhon = 0.85 * p.rhoe, rho0 = 1.15 * p.rhoe;
  if (rho < rhon) {
    const double t = rho / rhon - 1.;
    f = p.Fn0 + p.Fn1 * t + p.Fn2 * (t * t) + p.Fn3 * (t * (t * t));
    df = (p.Fn1 + 2. * p.Fn2 * t + 3. * p.Fn3 * (t * t)) * (1. / rhon);
  } else if (rho < rho0) {
    const double t = rho * (1. / p.rhoe) - 1.;
    f = p.F0 + p.F1 * t + p.F2 * (t * t) + p.F3 * (t * (t * t));
    df = (p.F1 + 2. * p.F2 * t + 3. * p.F3 * (t * t)) * (1. / p.rhoe);
  } else {
    const double s = rho * (1. / p.rhoe);
    const double se = pow(s, p.eta);
    const double lse = log(se);
    f = p.Fo * (1. - lse) * se;
    df = (-p.eta * se + (1. - lse) * p.eta * se) * (p.Fo * (1. / p.rhoe) / s);
  }
}

// FP32 versions of the pair functions (value and d/dr); x^20 = ((x^5)^2)^2
__device__ __forceinline__ void ej_term_f(float pre, float k, float x, float c, float ire, float& v, float& dv) {
  const float c1 = pre * expf(-k * (x - 1.f));
  const float c2 = x - c;
  const float q2 = c2 * c2;
  const float q5 = q2 * q2 * c2;
  const float q10 = q5 * q5;
  const float c3 = q10 * q10;
  const float c19 = q10 * q5 * q2 * c2 * c2;
  const float den = 1.f + c3;
  const float rden = __frcp_rn(den);
  const float dden = 20.f * c19;
  v = fmaf(c1, rden, v);
  dv = fmaf(ire * (-k * c1 * den - c1 * dden), rden * rden, dv);
}

// --------------------------------------------------------------------------
// function policies: FP64 rho/phi/F with derivatives, FP32 rho (density
// pass) and rho', phi, phi' (force pass)
// --------------------------------------------------------------------------
struct JohnsonFns {
  using Params = JohnsonDev;
  static __device__ __forceinline__ void rho_d(const Params& p, double r, double& v, double& dv) {
    ej_rho_d(p, r, v, dv);
  }
  static __device__ __forceinline__ void phi_d(const Params& p, double r, double& v, double& dv) {
    ej_phi_d(p, r, v, dv);
  }
  static __device__ __forceinline__ void embed_d(const Params& p, double rho, double& f, double& df) {
    ej_embed_d(p, rho, f, df);
  }
  static __device__ __forceinline__ float rho_f(const Params& p, float r) {
    float v = 0.f, dv = 0.f;
    ej_term_f(p.fef, p.betaf, r * p.ire_f, p.lambdaf, p.ire_f, v, dv);
    return v;
  }
  static __device__ __forceinline__ void pair_f(const Params& p, float r, float& rh, float& drh, float& ph,
                                                float& dph) {
    const float x = r * p.ire_f;
    rh = drh = ph = dph = 0.f;
    ej_term_f(p.fef, p.betaf, x, p.lambdaf, p.ire_f, rh, drh);
    ej_term_f(p.Af, p.alphaf, x, p.kappaf, p.ire_f, ph, dph);
    ej_term_f(-p.Bf, p.betaf, x, p.lambdaf, p.ire_f, ph, dph);
  }
};

// sutton_chen.h L36-67, the same operations in the same order
struct SuttonChenFns {
  using Params = SuttonChenDev;
  static __device__ __forceinline__ void rho_d(const Params& p, double r, double& v, double& dv) {
    const double ratio = p.a0 / r;
    v = pow(ratio, p.m);
    dv = -1 * p.m * v / r;
  }
  static __device__ __forceinline__ void phi_d(const Params& p, double r, double& v, double& dv) {
    const double ratio = p.a0 / r;
    v = p.epsilon * pow(ratio, p.n);
    dv = -1 * p.n * v / r;
  }
  static __device__ __forceinline__ void embed_d(const Params& p, double rho, double& f, double& df) {
    const double sq = sqrt(rho);
    f = -1. * p.c * p.epsilon * sq;
    df = 0.5 * f / (rho > 0 ? rho : 0);
  }
  static __device__ __forceinline__ float rho_f(const Params& p, float r) { return powf(p.a0f / r, p.mf); }
  static __device__ __forceinline__ void pair_f(const Params& p, float r, float& rh, float& drh, float& ph,
                                                float& dph) {
    const float ratio = p.a0f / r;
    const float ir = __frcp_rn(r);
    rh = powf(ratio, p.mf);
    drh = -p.mf * rh * ir;
    ph = p.epsf * powf(ratio, p.nf);
    dph = -p.nf * ph * ir;
  }
};

// --------------------------------------------------------------------------
// FP64 kernels
// --------------------------------------------------------------------------
template <class Fn, int T, bool EV>
__global__ void __launch_bounds__(256) k_ej_rho(PairArgs A, typename Fn::Params P, double* __restrict__ fpd) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = A.i0 + gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  int cx = 0, cy = 0, cz = 0;
  if (live) unpack_cell(A.cellpack[i], cx, cy, cz);
  double rho = 0.;
  double4_32a pi = make_double4_32a(0., 0., 0., 0.);
  if (live) pi = A.posd[i];
  const uint32_t* row = A.nbr + (size_t)i * A.W;
  for (int k = lane; k < nn; k += T) {
    const uint32_t ent = __ldg(row + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
    const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
    const double4_32a pj = A.posd[j];
    double Sx, Sy, Sz, dx, dy, dz;
    image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
    const double d2 = exact_d2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, Sx, Sy, Sz, dx, dy, dz);
    if (!(d2 <= P.rcut2)) continue;
    double v, dv;
    Fn::rho_d(P, sqrt(d2), v, dv);
    rho += v;
  }
  rho = group_reduce_d<T>(rho);
  if (live && lane == 0) {
    double f, df;
    Fn::embed_d(P, rho, f, df);
    fpd[i] = df;
    if (EV) A.ep_emb[i] = f;
  }
}

template <class Fn, int T, bool EV>
__global__ void __launch_bounds__(256) k_ej_force(PairArgs A, typename Fn::Params P,
                                                  const double* __restrict__ fpd) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = A.i0 + gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  int cx = 0, cy = 0, cz = 0;
  if (live) unpack_cell(A.cellpack[i], cx, cy, cz);
  double fx = 0., fy = 0., fz = 0., e = 0.;
  double v[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};
  double4_32a pi = make_double4_32a(0., 0., 0., 0.);
  double fpi = 0.;
  if (live) {
    pi = A.posd[i];
    fpi = fpd[i];
  }
  const int ti = (int)pi.w;
  const uint32_t* row = A.nbr + (size_t)i * A.W;
  for (int k = lane; k < nn; k += T) {
    const uint32_t ent = __ldg(row + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
    const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
    const double4_32a pj = A.posd[j];
    double Sx, Sy, Sz, dx, dy, dz;
    image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
    const double d2 = exact_d2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, Sx, Sy, Sz, dx, dy, dz);
    if (!(d2 <= P.rcut2)) continue;
    const double r = sqrt(d2);
    double rho, drho, phi, dphi;
    Fn::rho_d(P, r, rho, drho);
    Fn::phi_d(P, r, phi, dphi);
    const double de = (drho * (fpi + __ldg(&fpd[j])) + dphi) / r;
    const double fex = de * dx, fey = de * dy, fez = de * dz;
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
    const double epv = EV ? A.ep_emb[i] + e : 0.0;
    atom_epilogue<false>(A, i, ti, fx, fy, fz, 0.f, 0.f, 0.f, epv, EV ? v : nullptr);
  }
}

// --------------------------------------------------------------------------
// mixed kernels (one lane per atom, 1 list entry per load; the analytic
// functions make these arithmetic-bound rather than gather-bound)
// --------------------------------------------------------------------------
__device__ __noinline__ bool ej_exact_inside(const double4_32a* __restrict__ posd, int64_t i, uint32_t j,
                                             uint32_t code, int cp, const Grid g, double rc2) {
  int cx, cy, cz;
  unpack_cell(cp, cx, cy, cz);
  double Sx, Sy, Sz, a, b, c;
  image_shift(g, cx, cy, cz, code, Sx, Sy, Sz);
  const double4_32a di = posd[i], dj = posd[j];
  return exact_d2(di.x, di.y, di.z, dj.x, dj.y, dj.z, Sx, Sy, Sz, a, b, c) <= rc2;
}

__device__ __forceinline__ float ej_unit(uint32_t b) { return __int_as_float(0x4B000000u | b) - 8388609.0f; }

struct EjGeom {
  float dx, dy, dz, d2;
  bool in;
};

template <class Params>
__device__ __forceinline__ EjGeom ej_geom(const PairArgs& A, const Params& P, uint32_t ent, const float4& pj,
                                          const float4& pi, int64_t i, int cp) {
  EjGeom G;
  G.dx = fmaf(ej_unit((ent >> 26) & 3u), A.g.hf[0], pj.x - pi.x);
  G.dy = fmaf(ej_unit((ent >> 28) & 3u), A.g.hf[1], pj.y - pi.y);
  G.dz = fmaf(ej_unit(ent >> 30), A.g.hf[2], pj.z - pi.z);
  G.d2 = fmaf(G.dx, G.dx, fmaf(G.dy, G.dy, G.dz * G.dz));
  G.in = G.d2 < P.rc2lo;
  if (!G.in && G.d2 <= P.rc2hi)
    G.in = ej_exact_inside(A.posd, i, ent & GBMD_IDX_MASK, ent >> GBMD_IDX_BITS, cp, A.g, P.rcut2);
  return G;
}

template <class Fn, int T, bool EV>
__global__ void __launch_bounds__(256) k_ej_rho_mixed(PairArgs A, typename Fn::Params P, float* __restrict__ fpf,
                                                      float* __restrict__ epf) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = A.i0 + gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  const float4 pi = live ? A.posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int cp = live ? A.cellpack[i] : 0;
  float rho = 0.f, crho = 0.f;
  const uint32_t* row = A.nbr + (size_t)i * A.W;
  for (int k = lane; k < nn; k += T) {
    const uint32_t ent = __ldcs(row + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
    const float4 pj = __ldg(&A.posf[ent & GBMD_IDX_MASK]);
    const EjGeom G = ej_geom(A, P, ent, pj, pi, i, cp);
    const float r = G.d2 * rsqrtf(G.d2);
    const float v = Fn::rho_f(P, r);
    kahan_add(rho, crho, G.in ? v : 0.f);
  }
  group_reduce_kahan<T>(rho, crho);
  if (live && lane == 0) {
    double f, df;
    Fn::embed_d(P, (double)(rho - crho), f, df);  // per atom: FP64
    fpf[i] = (float)df;
    if (EV) epf[i] = (float)f;
  }
}

template <class Fn, int T, bool EV>
__global__ void __launch_bounds__(256) k_ej_force_mixed(PairArgs A, typename Fn::Params P,
                                                        const float* __restrict__ fpf,
                                                        const float* __restrict__ epf) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = A.i0 + gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  const float4 pi = live ? A.posf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int cp = live ? A.cellpack[i] : 0;
  const float fpi = live ? fpf[i] : 0.f;
  const int ti = __float_as_int(pi.w);
  float fx = 0.f, fy = 0.f, fz = 0.f, cfx = 0.f, cfy = 0.f, cfz = 0.f, e = 0.f, ce = 0.f;
  // virial: compensated too (its diagonal is a small difference of large
  // attractive and repulsive terms in this potential)
  float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, cv[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const uint32_t* row = A.nbr + (size_t)i * A.W;
  for (int k = lane; k < nn; k += T) {
    const uint32_t ent = __ldcs(row + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
    const uint32_t j = ent & GBMD_IDX_MASK;
    const float4 pj = __ldg(&A.posf[j]);
    const float fpj = __ldg(&fpf[j]);
    const EjGeom G = ej_geom(A, P, ent, pj, pi, i, cp);
    const float rs = rsqrtf(G.d2);
    const float r = G.d2 * rs;
    float rh, drh, ph, dph;
    Fn::pair_f(P, r, rh, drh, ph, dph);
    const float de = G.in ? fmaf(drh, fpi + fpj, dph) * rs : 0.f;
    kahan_add(fx, cfx, de * G.dx);
    kahan_add(fy, cfy, de * G.dy);
    kahan_add(fz, cfz, de * G.dz);
    if (EV) {
      kahan_add(e, ce, G.in ? 0.5f * ph : 0.f);
      const float h = -0.5f * de;
      kahan_add(v[0], cv[0], h * G.dx * G.dx);
      kahan_add(v[1], cv[1], h * G.dy * G.dy);
      kahan_add(v[2], cv[2], h * G.dz * G.dz);
      kahan_add(v[3], cv[3], h * G.dx * G.dy);
      kahan_add(v[4], cv[4], h * G.dx * G.dz);
      kahan_add(v[5], cv[5], h * G.dy * G.dz);
    }
  }
  group_reduce_kahan<T>(fx, cfx);
  group_reduce_kahan<T>(fy, cfy);
  group_reduce_kahan<T>(fz, cfz);
  if (EV) {
    group_reduce_kahan<T>(e, ce);
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      group_reduce_kahan<T>(v[q], cv[q]);
      v[q] -= cv[q];
    }
  }
  if (live && lane == 0) {
    const float im = A.inv_massf[ti];
    double o[9];
    if (EV) {
      o[0] = v[0]; o[1] = v[3]; o[2] = v[4];
      o[3] = v[3]; o[4] = v[1]; o[5] = v[5];
      o[6] = v[4]; o[7] = v[5]; o[8] = v[2];
    }
    const double epv = EV ? (double)epf[i] + (double)(e - ce) : 0.0;
    atom_epilogue<true>(A, i, ti, 0., 0., 0., (fx - cfx) * im, (fy - cfy) * im, (fz - cfz) * im, epv,
                        EV ? o : nullptr);
  }
}

// --------------------------------------------------------------------------
// dispatch
// --------------------------------------------------------------------------
template <class Fn, int T, bool EV>
static void launch_ej_T(gbmd_context* c, const PairArgs& A, const typename Fn::Params& P, int part, bool mixed) {
  const int B = c->block;
  const unsigned grid = (unsigned)(((A.n - A.i0) * T + B - 1) / B);
  cudaStream_t s = c->stream;
  if (mixed) {
    if (part != 2) k_ej_rho_mixed<Fn, T, EV><<<grid, B, 0, s>>>(A, P, c->fpf, c->epf);
    if (part != 1) k_ej_force_mixed<Fn, T, EV><<<grid, B, 0, s>>>(A, P, c->fpf, c->epf);
  } else {
    if (part != 2) k_ej_rho<Fn, T, EV><<<grid, B, 0, s>>>(A, P, c->fpd);
    if (part != 1) k_ej_force<Fn, T, EV><<<grid, B, 0, s>>>(A, P, c->fpd);
  }
}

template <class Fn, bool EV>
static int launch_ej_E(gbmd_context* c, const PairArgs& A, const typename Fn::Params& P, int part, bool mixed) {
  switch (c->tpa) {
    case 1: launch_ej_T<Fn, 1, EV>(c, A, P, part, mixed); break;
    case 2: launch_ej_T<Fn, 2, EV>(c, A, P, part, mixed); break;
    case 4: launch_ej_T<Fn, 4, EV>(c, A, P, part, mixed); break;
    case 8: launch_ej_T<Fn, 8, EV>(c, A, P, part, mixed); break;
    case 16: launch_ej_T<Fn, 16, EV>(c, A, P, part, mixed); break;
    default: return set_error(c, GBMD_ERR_INVALID, "unsupported lanes per atom %d", c->tpa);
  }
  return GBMD_OK;
}

int launch_johnson(gbmd_context* c, const PairArgs& A, int part, bool ev, bool mixed) {
  if (c->pot == GBMD_POT_EAM_SUTTON_CHEN)
    return ev ? launch_ej_E<SuttonChenFns, true>(c, A, c->esc, part, mixed)
              : launch_ej_E<SuttonChenFns, false>(c, A, c->esc, part, mixed);
  return ev ? launch_ej_E<JohnsonFns, true>(c, A, c->ej, part, mixed)
            : launch_ej_E<JohnsonFns, false>(c, A, c->ej, part, mixed);
}

}  // namespace gbmd

