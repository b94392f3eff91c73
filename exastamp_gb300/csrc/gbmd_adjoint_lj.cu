// gbmd_adjoint_lj.cu -- parameter adjoint of lj_compute_force: the
// force-matching + energy loss of one system and its gradient with respect to
// (epsilon, sigma), recomputing every pair term instead of storing it.
//
//   L = wF sum_i |F_i - F*_i|^2 + wE sum_i (E_i - E*_i)^2
//   F_i = sum_j g(r) d_ij,  g = (de/dr)/r,  d_ij = r_j - r_i,  E_i = 1/2 sum_j (e(r) - e(rc))
//   dL/dtheta = sum_i 2 wF (F_i - F*_i) . sum_j dg/dtheta d_ij
//             + 2 wE (E_i - E*_i) 1/2 sum_j (de/dtheta - de(rc)/dtheta)
//   de/deps = e/eps, de/dsigma = 4 eps (12 s^12 - 6 s^6)/sigma,  s = sigma/r
//   (lennard_jones.h L41-50).
//
// F_i and E_i are the context's own forces and energies (mixed or FP64 as
// set); the per-pair derivative terms are FP64, one thread per atom, and the
// per-atom (loss, dL/deps, dL/dsigma) are summed in a fixed order so the
// result is reproducible.
#include "gbmd_pair_common.cuh"

namespace gbmd {

struct LJAdjArgs {
  double eps, sig, rc2, decut_deps, decut_dsig, wF, wE;
  const double *fxt, *fyt, *fzt, *et;  // targets, cell-sorted
  double* out;                         // n x 3: loss_i, dL/deps_i, dL/dsigma_i
};

__global__ void __launch_bounds__(256) k_lj_loss_grad(PairArgs A, LJAdjArgs P) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const int nn = min(A.nnb[i], A.maxnb);
  int cx, cy, cz;
  unpack_cell(A.cellpack[i], cx, cy, cz);
  const double4_32a pi = A.posd[i];
  const int ti = (int)pi.w;
  const double m = A.mass[ti];
  const double dF[3] = {A.ax[i] * m - P.fxt[i], A.ay[i] * m - P.fyt[i], A.az[i] * m - P.fzt[i]};
  const double dE = A.ep[i] - P.et[i];
  double ge = 0., gs = 0.;
  const uint32_t* row = A.nbr + (size_t)i * A.W;
  for (int k = 0; k < nn; ++k) {
    const uint32_t ent = __ldg(row + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
    const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
    const double4_32a pj = A.posd[j];
    double Sx, Sy, Sz, dx, dy, dz;
    image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
    const double d2 = exact_d2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, Sx, Sy, Sz, dx, dy, dz);
    if (!(d2 <= P.rc2)) continue;
    const double r = sqrt(d2);
    const double s = P.sig / r, s2 = s * s, s6 = s2 * s2 * s2, s12 = s6 * s6;
    const double e = 4. * P.eps * (s12 - s6);
    const double g = -24. * P.eps * (2. * s12 - s6) / d2;
    const double dg_deps = g / P.eps;
    const double dg_dsig = -24. * P.eps * (24. * s12 - 6. * s6) / (d2 * P.sig);
    const double proj = dF[0] * dx + dF[1] * dy + dF[2] * dz;
    ge += 2. * P.wF * proj * dg_deps + P.wE * dE * (e / P.eps - P.decut_deps);
    gs += 2. * P.wF * proj * dg_dsig + P.wE * dE * (4. * P.eps * (12. * s12 - 6. * s6) / P.sig - P.decut_dsig);
  }
  P.out[3 * i] = P.wF * (dF[0] * dF[0] + dF[1] * dF[1] + dF[2] * dF[2]) + P.wE * dE * dE;
  P.out[3 * i + 1] = ge;
  P.out[3 * i + 2] = gs;
}

// Fixed-order sum of n rows of 3: ADJ_BLOCKS partial rows (grid-stride in
// atom order, then a tree in shared memory), then one block over the partials.
constexpr int ADJ_BLOCKS = 592, ADJ_THREADS = 256;

__global__ void __launch_bounds__(ADJ_THREADS) k_sum3_part(int64_t n, const double* __restrict__ v,
                                                           double* __restrict__ part) {
  __shared__ double sm[3][ADJ_THREADS];
  double a[3] = {0., 0., 0.};
  for (int64_t i = blockIdx.x * (int64_t)ADJ_THREADS + threadIdx.x; i < n; i += (int64_t)ADJ_BLOCKS * ADJ_THREADS)
    for (int q = 0; q < 3; ++q) a[q] += v[3 * i + q];
  for (int q = 0; q < 3; ++q) sm[q][threadIdx.x] = a[q];
  __syncthreads();
  for (int w = ADJ_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 3; ++q) sm[q][threadIdx.x] += sm[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) part[3 * blockIdx.x + q] = sm[q][0];
}

__global__ void __launch_bounds__(ADJ_THREADS) k_sum3_final(const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double sm[3][ADJ_THREADS];
  double a[3] = {0., 0., 0.};
  for (int b = threadIdx.x; b < ADJ_BLOCKS; b += ADJ_THREADS)
    for (int q = 0; q < 3; ++q) a[q] += part[3 * b + q];
  for (int q = 0; q < 3; ++q) sm[q][threadIdx.x] = a[q];
  __syncthreads();
  for (int w = ADJ_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 3; ++q) sm[q][threadIdx.x] += sm[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) out[q] = sm[q][0];
}

// scratch: at least 3n + 3 * ADJ_BLOCKS + 3 doubles; the result (loss,
// dL/deps, dL/dsigma) lands in scratch[3n + 3 * ADJ_BLOCKS ..].
int launch_lj_loss_grad(gbmd_context* c, const PairArgs& A, const double* const targets[4], double wF, double wE,
                        double* scratch) {
  if (c->pot != GBMD_POT_LJ) return set_error(c, GBMD_ERR_INVALID, "the LJ adjoint needs lj_compute_force");
  const LJPair& q = c->lj.p[0];
  LJAdjArgs P;
  P.eps = q.eps;
  P.sig = q.sig;
  P.rc2 = q.rc2;
  const double sc = q.sig / q.rc, sc2 = sc * sc, sc6 = sc2 * sc2 * sc2, sc12 = sc6 * sc6;
  P.decut_deps = q.ecut / q.eps;
  P.decut_dsig = 4. * q.eps * (12. * sc12 - 6. * sc6) / q.sig;
  P.wF = wF;
  P.wE = wE;
  P.fxt = targets[0];
  P.fyt = targets[1];
  P.fzt = targets[2];
  P.et = targets[3];
  P.out = scratch;
  const int64_t n = A.n;
  k_lj_loss_grad<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(A, P);
  k_sum3_part<<<ADJ_BLOCKS, ADJ_THREADS, 0, c->stream>>>(n, scratch, scratch + 3 * n);
  k_sum3_final<<<1, ADJ_THREADS, 0, c->stream>>>(scratch + 3 * n, scratch + 3 * n + 3 * ADJ_BLOCKS);
  return GBMD_OK;
}

// ---------------------------------------------------------------------------
// lj_multi_force (pair_potential_force_op_multiparam.h L92-118, per-pair
// energy shift pair_potential_impl.hxx L287-324): the same loss with one
// (epsilon, sigma) per unordered type pair u = (a <= b), each shared by the
// (a, b) and (b, a) entries of the table.  A pair is inside when d2 <= rcut_max^2
// and r <= rc_ab (the reference's two-stage test); its shift is e_ab(rc_ab).
// Per atom the kernel writes K = 1 + 2 nu doubles: loss_i, dL/deps_u (u < nu),
// dL/dsigma_u (u < nu).
// ---------------------------------------------------------------------------
constexpr int LJM_MAXP = GBMD_MAX_TYPES * GBMD_MAX_TYPES;
constexpr int LJM_MAXU = GBMD_MAX_TYPES * (GBMD_MAX_TYPES + 1) / 2;

struct LJMAdjArgs {
  int ntypes, nu;
  double rcmax2, wF, wE;
  double eps[LJM_MAXP], sig[LJM_MAXP], rc[LJM_MAXP], decut_deps[LJM_MAXP], decut_dsig[LJM_MAXP];
  int8_t uid[LJM_MAXP];                // table entry -> unordered pair
  const double *fxt, *fyt, *fzt, *et;  // targets, cell-sorted
  double* out;                         // n x K
};

__global__ void __launch_bounds__(128) k_lj_multi_loss_grad(PairArgs A, const LJMAdjArgs* __restrict__ P) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const int nu = P->nu, K = 1 + 2 * nu;
  double* o = P->out + (size_t)i * K;
  for (int q = 1; q < K; ++q) o[q] = 0.0;
  const int nn = min(A.nnb[i], A.maxnb);
  int cx, cy, cz;
  unpack_cell(A.cellpack[i], cx, cy, cz);
  const double4_32a pi = A.posd[i];
  const int ti = (int)pi.w;
  const double m = A.mass[ti];
  const double dF[3] = {A.ax[i] * m - P->fxt[i], A.ay[i] * m - P->fyt[i], A.az[i] * m - P->fzt[i]};
  const double dE = A.ep[i] - P->et[i];
  const uint32_t* row = A.nbr + (size_t)i * A.W;
  for (int k = 0; k < nn; ++k) {
    const uint32_t ent = __ldg(row + (size_t)(k >> A.wsh) * A.stride + (k & (A.W - 1)));
    const uint32_t j = ent & GBMD_IDX_MASK, code = ent >> GBMD_IDX_BITS;
    const double4_32a pj = A.posd[j];
    double Sx, Sy, Sz, dx, dy, dz;
    image_shift(A.g, cx, cy, cz, code, Sx, Sy, Sz);
    const double d2 = exact_d2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, Sx, Sy, Sz, dx, dy, dz);
    if (!(d2 <= P->rcmax2)) continue;
    const int pid = ti * P->ntypes + (int)pj.w;
    const double r = sqrt(d2);
    if (!(r <= P->rc[pid])) continue;
    const double eps = P->eps[pid], sg = P->sig[pid];
    const double s = sg / r, s2 = s * s, s6 = s2 * s2 * s2, s12 = s6 * s6;
    const double e = 4. * eps * (s12 - s6);
    const double g = -24. * eps * (2. * s12 - s6) / d2;
    const double dg_deps = g / eps;
    const double dg_dsig = -24. * eps * (24. * s12 - 6. * s6) / (d2 * sg);
    const double proj = dF[0] * dx + dF[1] * dy + dF[2] * dz;
    const int u = P->uid[pid];
    o[1 + u] += 2. * P->wF * proj * dg_deps + P->wE * dE * (e / eps - P->decut_deps[pid]);
    o[1 + nu + u] += 2. * P->wF * proj * dg_dsig +
                     P->wE * dE * (4. * eps * (12. * s12 - 6. * s6) / sg - P->decut_dsig[pid]);
  }
  o[0] = P->wF * (dF[0] * dF[0] + dF[1] * dF[1] + dF[2] * dF[2]) + P->wE * dE * dE;
}

// Fixed-order sum of n rows of K columns: ADJ_BLOCKS partial rows
// (grid-stride in atom order, then a tree per column), then one block over
// the partials.
__global__ void __launch_bounds__(ADJ_THREADS) k_sumK_part(int64_t n, int K, const double* __restrict__ v,
                                                           double* __restrict__ part) {
  __shared__ double sm[ADJ_THREADS];
  for (int q = 0; q < K; ++q) {
    double a = 0.;
    for (int64_t i = blockIdx.x * (int64_t)ADJ_THREADS + threadIdx.x; i < n; i += (int64_t)ADJ_BLOCKS * ADJ_THREADS)
      a += v[(size_t)i * K + q];
    sm[threadIdx.x] = a;
    __syncthreads();
    for (int w = ADJ_THREADS / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)blockIdx.x * K + q] = sm[0];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(ADJ_THREADS) k_sumK_final(int K, const double* __restrict__ part,
                                                            double* __restrict__ out) {
  __shared__ double sm[ADJ_THREADS];
  for (int q = 0; q < K; ++q) {
    double a = 0.;
    for (int b = threadIdx.x; b < ADJ_BLOCKS; b += ADJ_THREADS) a += part[(size_t)b * K + q];
    sm[threadIdx.x] = a;
    __syncthreads();
    for (int w = ADJ_THREADS / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[q] = sm[0];
    __syncthreads();
  }
}

// args_dev: device copy of LJMAdjArgs (filled here); scratch: at least
// K n + K ADJ_BLOCKS + K doubles; the K sums land at scratch[K n + K ADJ_BLOCKS].
int launch_lj_multi_loss_grad(gbmd_context* c, const PairArgs& A, const double* const targets[4], double wF,
                              double wE, void* args_dev, double* scratch, int* nu_out) {
  if (c->pot != GBMD_POT_LJ_MULTI) return set_error(c, GBMD_ERR_INVALID, "needs lj_multi_force");
  const int nt = c->lj.ntypes;
  LJMAdjArgs P = {};
  P.ntypes = nt;
  P.rcmax2 = c->lj.rcut_max2;
  P.wF = wF;
  P.wE = wE;
  int nu = 0;
  for (int a = 0; a < nt; ++a)
    for (int b = a; b < nt; ++b) {
      P.uid[a * nt + b] = P.uid[b * nt + a] = (int8_t)nu;
      ++nu;
    }
  P.nu = nu;
  for (int pid = 0; pid < nt * nt; ++pid) {
    const LJPair& q = c->lj.p[pid];
    P.eps[pid] = q.eps;
    P.sig[pid] = q.sig;
    P.rc[pid] = q.rc;
    // e_ab(rc_ab) and its derivatives (zero for a pair that never interacts)
    if (q.eps != 0.0 && q.sig != 0.0 && q.rc > 0.0) {
      const double sc = q.sig / q.rc, sc2 = sc * sc, sc6 = sc2 * sc2 * sc2, sc12 = sc6 * sc6;
      P.decut_deps[pid] = q.ecut / q.eps;
      P.decut_dsig[pid] = 4. * q.eps * (12. * sc12 - 6. * sc6) / q.sig;
    }
  }
  P.fxt = targets[0];
  P.fyt = targets[1];
  P.fzt = targets[2];
  P.et = targets[3];
  P.out = scratch;
  GBMD_CUDA(c, cudaMemcpyAsync(args_dev, &P, sizeof(P), cudaMemcpyHostToDevice, c->stream));
  const int K = 1 + 2 * nu;
  const int64_t n = A.n;
  k_lj_multi_loss_grad<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(A, (const LJMAdjArgs*)args_dev);
  k_sumK_part<<<ADJ_BLOCKS, ADJ_THREADS, 0, c->stream>>>(n, K, scratch, scratch + (size_t)K * n);
  k_sumK_final<<<1, ADJ_THREADS, 0, c->stream>>>(K, scratch + (size_t)K * n,
                                                 scratch + (size_t)K * n + (size_t)K * ADJ_BLOCKS);
  // the host struct must outlive the copy
  GBMD_CUDA(c, cudaStreamSynchronize(c->stream));
  *nu_out = nu;
  return GBMD_OK;
}

size_t lj_multi_adj_args_size() { return sizeof(LJMAdjArgs); }

}  // namespace gbmd
