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

}  // namespace gbmd
