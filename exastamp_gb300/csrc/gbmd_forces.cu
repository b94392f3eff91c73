// gbmd_forces.cu -- plain-FP64 LJ and eam_alloy pair kernels for sm_103a, and
// the force dispatch (FP64 here, mixed precision in gbmd_mixed.cu).
//
// The FP64 kernels restate the reference arithmetic exactly:
//   LJ       lennard_jones.h L41-50 + force_op_impl2.hxx L33-68 (e -= ecut, de /= r,
//            fe = de*dr, ep += e/2, vir += -1/2 fe (x) dr)
//   LJ multi pair_potential_force_op_multiparam.h L92-118 (r <= rcut_pair test)
//   EAM      eam_alloy.h L198-313 + eam_force_op_multimat.h L114-343
// with dr = (x_j + n*L) - x_i and d2 rounded exactly like the list builder
// and the oracle, so cutoff membership is identical.
//
// Per unit (one ordered list entry): 4 B of list, one 32 B position gather,
// the cutoff test and, inside the cutoff, the pair function.
#include "gbmd_pair_common.cuh"

namespace gbmd {

// ---------------------------------------------------------------------------
// Lennard-Jones (single parameter set and per-type-pair tables)
// ---------------------------------------------------------------------------
struct LJSingle {
  double eps, sig, ecut, rc2;
};

template <int T, bool EV, bool MULTI>
__global__ void __launch_bounds__(256) k_lj(PairArgs A, LJSingle P, const LJPair* __restrict__ tab, int ntypes,
                                            double rcmax2) {
  __shared__ double sd[MULTI ? GBMD_MAX_TYPES * GBMD_MAX_TYPES * 5 : 1];
  if (MULTI) {
    for (int q = threadIdx.x; q < ntypes * ntypes; q += blockDim.x) {
      const LJPair& p = tab[q];
      sd[5 * q + 0] = p.eps;
      sd[5 * q + 1] = p.sig;
      sd[5 * q + 2] = p.rc;
      sd[5 * q + 3] = p.ecut;
      sd[5 * q + 4] = p.rc2;
    }
    __syncthreads();
  }
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = A.i0 + gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  int cx = 0, cy = 0, cz = 0, ti = 0;
  if (live) unpack_cell(A.cellpack[i], cx, cy, cz);

  {
    double fx = 0., fy = 0., fz = 0., e = 0.;
    double v[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};
    double4_32a pi = make_double4_32a(0., 0., 0., 0.);
    if (live) pi = A.posd[i];
    ti = (int)pi.w;
    const uint32_t* row = A.nbr + (size_t)i * A.W;
    for (int k = lane; k < nn; k += T) {
      const uint32_t ent = __ldg(row + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
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
__device__ __forceinline__ int r_knot_d(double r, double rdr, int nr, double& p) {
  double pp = r * rdr + 1.0;
  int m = (int)pp;
  m = min(m, nr - 1);
  pp -= m;
  p = fmin(pp, 1.0);
  return m;
}

template <int T, bool EV>
__global__ void __launch_bounds__(256) k_eam_rho(PairArgs A, EamDev E, double* __restrict__ fpd) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = A.i0 + gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  int cx = 0, cy = 0, cz = 0;
  if (live) unpack_cell(A.cellpack[i], cx, cy, cz);
  {
    double rho = 0.;
    double4_32a pi = make_double4_32a(0., 0., 0., 0.);
    if (live) pi = A.posd[i];
    const int ti = (int)pi.w;
    const uint32_t* row = A.nbr + (size_t)i * A.W;
    for (int k = lane; k < nn; k += T) {
      const uint32_t ent = __ldg(row + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
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
      if (EV) A.ep_emb[i] = phi;
    }
  }
}

__device__ __forceinline__ int z2r_index(int a, int b) {
  const int irow = a > b ? a : b, icol = a > b ? b : a;
  return irow * (irow + 1) / 2 + icol;
}

template <int T, bool EV>
__global__ void __launch_bounds__(256) k_eam_force(PairArgs A, EamDev E, const double* __restrict__ fpd) {
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = A.i0 + gt / T;
  const int lane = (int)(gt % T);
  const bool live = i < A.n;
  const int nn = live ? min(A.nnb[i], A.maxnb) : 0;
  int cx = 0, cy = 0, cz = 0;
  if (live) unpack_cell(A.cellpack[i], cx, cy, cz);
  {
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
      const double epv = EV ? A.ep_emb[i] + e : 0.0;
      atom_epilogue<false>(A, i, ti, fx, fy, fz, 0.f, 0.f, 0.f, epv, EV ? v : nullptr);
    }
  }
}

// ---------------------------------------------------------------------------
// host dispatch
// ---------------------------------------------------------------------------
PairArgs make_args(gbmd_context* c, const ForceFlags& f) {
  PairArgs A;
  A.i0 = f.i0;
  A.n = f.i1 >= 0 ? f.i1 : c->n;
  A.W = list_width(c);
  A.wsh = 0;
  while ((1 << A.wsh) < A.W) ++A.wsh;
  A.stride = c->npad * A.W;
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
  A.vxo = f.v_out ? f.v_out : A.vx;
  A.vyo = f.v_out ? f.v_out + c->cap : A.vy;
  A.vzo = f.v_out ? f.v_out + 2 * c->cap : A.vz;
  A.ep = c->ep;
  A.ep_emb = c->epd;
  A.vir = c->vir;
  A.type = c->TYPE();
  for (int t = 0; t < GBMD_MAX_TYPES; ++t) {
    A.mass[t] = t < c->ntypes ? c->mass[t] : 1.0;
    A.inv_massf[t] = (float)(1.0 / A.mass[t]);
  }
  A.fuse = f.fuse;
  const bool test = c->fused_trigger && f.fuse == FUSE_PUSH2_PUSH1;
  A.gate = test ? c->d_err + ERRW_GATE : nullptr;
  A.rref = c->rref;
  A.rcap = c->cap;
  A.thr2 = (0.5 * c->skin) * (0.5 * c->skin);
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
template <int T, bool EV>
static void launch_fp64_T(gbmd_context* c, const PairArgs& A, int part) {
  const int B = c->block;
  const unsigned grid = (unsigned)(((A.n - A.i0) * T + B - 1) / B);
  cudaStream_t s = c->stream;
  if (c->pot != GBMD_POT_EAM_ALLOY && part == 1) return;
  if (c->pot == GBMD_POT_LJ) {
    const LJPair& p = c->lj.p[0];
    LJSingle P{p.eps, p.sig, p.ecut, p.rc2};
    k_lj<T, EV, false><<<grid, B, 0, s>>>(A, P, nullptr, 1, c->lj.rcut_max2);
  } else if (c->pot == GBMD_POT_LJ_MULTI) {
    LJSingle P{};
    k_lj<T, EV, true><<<grid, B, 0, s>>>(A, P, c->lj_tab_d, c->lj.ntypes, c->lj.rcut_max2);
  } else {
    if (part != 2) k_eam_rho<T, EV><<<grid, B, 0, s>>>(A, c->eam, c->fpd);
    if (part != 1) k_eam_force<T, EV><<<grid, B, 0, s>>>(A, c->eam, c->fpd);
  }
}

template <bool EV>
static int launch_fp64(gbmd_context* c, const PairArgs& A, int part) {
  switch (c->tpa) {
    case 1: launch_fp64_T<1, EV>(c, A, part); break;
    case 2: launch_fp64_T<2, EV>(c, A, part); break;
    case 4: launch_fp64_T<4, EV>(c, A, part); break;
    case 8: launch_fp64_T<8, EV>(c, A, part); break;
    case 16: launch_fp64_T<16, EV>(c, A, part); break;
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
  const bool piece = f.i0 != 0 || f.i1 >= 0;
  if (piece && (f.i0 < 0 || f.i1 < f.i0 || f.i1 > c->n))
    return set_error(c, GBMD_ERR_INVALID, "atom range [%lld, %lld) outside [0, %lld)", (long long)f.i0,
                     (long long)f.i1, (long long)c->n);
  if (piece && (c->newton3 || c->staged || f.fuse == FUSE_PUSH2_PUSH1))
    return set_error(c, GBMD_ERR_INVALID, "atom ranges: full-list kernels without staging or fused first half");
  const PairArgs A = make_args(c, f);
  const bool ev = f.energy || f.virial;
  const bool mixed = c->precision == GBMD_PRECISION_MIXED;
  if (c->newton3 &&
      !(mixed && (c->pot == GBMD_POT_LJ || c->pot == GBMD_POT_LJ_MULTI || c->pot == GBMD_POT_EAM_ALLOY)))
    return set_error(c, GBMD_ERR_UNSUPPORTED,
                     "Newton-3 half lists: LJ potentials and eam_alloy in mixed precision only");
  if (c->newton3 && !c->h3acc) return set_error(c, GBMD_ERR_INVALID, "Newton-3 accumulators not allocated");
  const int part = f.part;
  int rc;
  if (c->pot == GBMD_POT_EAM_JOHNSON || c->pot == GBMD_POT_EAM_SUTTON_CHEN) rc = launch_johnson(c, A, part, ev, mixed);
  else if (mixed) rc = launch_mixed(c, A, part, ev);
  else rc = ev ? launch_fp64<true>(c, A, part) : launch_fp64<false>(c, A, part);
  if (rc) return rc;
  if (f.fuse == FUSE_PUSH2_PUSH1 && part != 1) c->cur ^= 1;
  return GBMD_OK;
}

}  // namespace gbmd
