// gbmd_integrate.cu -- velocity-Verlet push operators and the FP64
// thermodynamic reduction.
//
// Standalone push kernels round exactly like the reference formulas evaluated
// without contraction (explicit _rn intrinsics), so they agree bit-for-bit
// with the FP64 oracle:
//   push_f_v_r  r += v*h + a*h*h/2, h = dt*dt_scale
//               (src/numerical_schemes/push_vec3_2nd_order_xform_minimization.cpp L33-38)
//   push_f_v    v += a*h
//   push_min    r += a*h*h/2 (same file L116-149; tolF > 0 clips a first)
// Every push that moves atoms also refreshes the FP32/FP64 gather copies.
//
// Thermo: simulation_thermodynamic_state (simulation_thermodynamic_state.cpp
// L101-163): 26 FP64 sums per atom, block partials in a fixed grid, then one
// block sums the partials in block order -- the result is bit-reproducible.
// Per unit: 24 B (v) + 8 B (ep) + 1 B (type) [+ 72 B virial] read per atom.
#include "gbmd_pair_common.cuh"

namespace gbmd {

static inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

__device__ __forceinline__ void refresh_gather(const Grid& g, int64_t i, int cp, int t, double x, double y,
                                               double z, float4* pf, double4_32a* pd) {
  const double cx = (double)(cp & 1023), cy = (double)((cp >> 10) & 1023), cz = (double)(cp >> 20);
  pf[i] = make_float4((float)(x - cx * g.h[0] - g.lo[0]), (float)(y - cy * g.h[1] - g.lo[1]),
                      (float)(z - cz * g.h[2] - g.lo[2]), __int_as_float(t));
  pd[i] = make_double4_32a(x, y, z, (double)t);
}

struct PushArgs {
  int64_t n;
  double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az;
  double *xo, *yo, *zo;  // position outputs (== x,y,z in place, or the other buffer)
  const uint8_t* type;
  const int32_t* cellpack;
  float4* pf;
  double4_32a* pd;
  Grid g;
  int refresh;
  int* gate;  // k_first_half under the displacement trigger (else null)
  const double* rref;
  int64_t rcap;
  double thr2;
};

__global__ void k_push_f_v_r(PushArgs P, double h, double h2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double x = __dadd_rn(P.x[i], __dadd_rn(__dmul_rn(P.vx[i], h), __dmul_rn(P.ax[i], h2)));
  const double y = __dadd_rn(P.y[i], __dadd_rn(__dmul_rn(P.vy[i], h), __dmul_rn(P.ay[i], h2)));
  const double z = __dadd_rn(P.z[i], __dadd_rn(__dmul_rn(P.vz[i], h), __dmul_rn(P.az[i], h2)));
  P.x[i] = x;
  P.y[i] = y;
  P.z[i] = z;
  if (P.refresh) refresh_gather(P.g, i, P.cellpack[i], P.type[i], x, y, z, P.pf, P.pd);
}

__global__ void k_push_f_v(PushArgs P, double h) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  P.vx[i] = __dadd_rn(P.vx[i], __dmul_rn(P.ax[i], h));
  P.vy[i] = __dadd_rn(P.vy[i], __dmul_rn(P.ay[i], h));
  P.vz[i] = __dadd_rn(P.vz[i], __dmul_rn(P.az[i], h));
}

// verlet_first_half = push_f_v_r(dt, 1) then push_f_v(dt, 0.5), one pass.
__global__ void k_first_half(PushArgs P, double h, double h2, double hv) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double vx = P.vx[i], vy = P.vy[i], vz = P.vz[i];
  const double ax = P.ax[i], ay = P.ay[i], az = P.az[i];
  const double x = __dadd_rn(P.x[i], __dadd_rn(__dmul_rn(vx, h), __dmul_rn(ax, h2)));
  const double y = __dadd_rn(P.y[i], __dadd_rn(__dmul_rn(vy, h), __dmul_rn(ay, h2)));
  const double z = __dadd_rn(P.z[i], __dadd_rn(__dmul_rn(vz, h), __dmul_rn(az, h2)));
  P.xo[i] = x;
  P.yo[i] = y;
  P.zo[i] = z;
  P.vx[i] = __dadd_rn(vx, __dmul_rn(ax, hv));
  P.vy[i] = __dadd_rn(vy, __dmul_rn(ay, hv));
  P.vz[i] = __dadd_rn(vz, __dmul_rn(az, hv));
  if (P.refresh) refresh_gather(P.g, i, P.cellpack[i], P.type[i], x, y, z, P.pf, P.pd);
  if (P.gate) displacement_test(P.gate, P.rref, P.rcap, P.thr2, i, x, y, z);
}

__global__ void k_push_min(PushArgs P, double h2, double tolF) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  double a[3] = {P.ax[i], P.ay[i], P.az[i]};
  if (tolF > 0.0) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (fabs(a[d]) > tolF) a[d] = a[d] > 0. ? tolF : -tolF;
    P.ax[i] = a[0];
    P.ay[i] = a[1];
    P.az[i] = a[2];
  }
  const double x = __dadd_rn(P.x[i], __dmul_rn(a[0], h2));
  const double y = __dadd_rn(P.y[i], __dmul_rn(a[1], h2));
  const double z = __dadd_rn(P.z[i], __dmul_rn(a[2], h2));
  P.x[i] = x;
  P.y[i] = y;
  P.z[i] = z;
  if (P.refresh) refresh_gather(P.g, i, P.cellpack[i], P.type[i], x, y, z, P.pf, P.pd);
}

static PushArgs push_args(gbmd_context* c) {
  PushArgs P;
  P.n = c->n;
  P.x = c->X(); P.y = c->Y(); P.z = c->Z();
  P.vx = c->VX(); P.vy = c->VY(); P.vz = c->VZ();
  P.ax = c->AX(); P.ay = c->AY(); P.az = c->AZ();
  P.type = c->TYPE();
  P.xo = P.x; P.yo = P.y; P.zo = P.z;
  P.cellpack = c->cellpack;
  P.pf = c->POSF();
  P.pd = c->POSD();
  P.g = c->grid;
  P.refresh = c->list_valid ? 1 : 0;
  P.gate = c->fused_trigger ? c->d_err + ERRW_GATE : nullptr;
  P.rref = c->rref;
  P.rcap = c->cap;
  P.thr2 = (0.5 * c->skin) * (0.5 * c->skin);
  return P;
}

void launch_push_f_v_r(gbmd_context* c, double dt, double dt_scale) {
  if (!c->n) return;
  const double h = dt * dt_scale;
  const double h2 = h * h * 0.5;
  k_push_f_v_r<<<nblk(c->n, 256), 256, 0, c->stream>>>(push_args(c), h, h2);
}

void launch_push_f_v(gbmd_context* c, double dt, double dt_scale) {
  if (!c->n) return;
  k_push_f_v<<<nblk(c->n, 256), 256, 0, c->stream>>>(push_args(c), dt * dt_scale);
}

void launch_first_half(gbmd_context* c, double dt) {
  if (!c->n) return;
  const double h = dt * 1.0;
  const double h2 = h * h * 0.5;
  k_first_half<<<nblk(c->n, 256), 256, 0, c->stream>>>(push_args(c), h, h2, dt * 0.5);
}

// verlet_first_half writing the new positions (and gather copies) into the
// other position buffer, then swapping: every step of the runner swaps the
// position buffers exactly once, whichever path it takes, so a captured
// chunk of steps always ends on the buffer it started from.
void launch_first_half_swap(gbmd_context* c, double dt) {
  if (!c->n) return;
  PushArgs P = push_args(c);
  const int o = c->cur ^ 1;
  P.xo = c->rbuf[o];
  P.yo = c->rbuf[o] + c->cap;
  P.zo = c->rbuf[o] + 2 * c->cap;
  P.pf = c->posf[o];
  P.pd = c->posd[o];
  const double h = dt * 1.0;
  const double h2 = h * h * 0.5;
  k_first_half<<<nblk(c->n, 256), 256, 0, c->stream>>>(P, h, h2, dt * 0.5);
  c->cur = o;
}

// gbmd_run_nve_host's upload fused with verlet_first_half: the caller's
// page-locked r, v, a (caller order, read over the host link by consecutive
// threads) are pushed by the first half -- the formulas of k_first_half --
// and written into the cell-sorted state in place (r', v', and a as given),
// with the gather copies refreshed and the skin/2 displacement test taken on
// r', as check_and_update_particles does after verlet_first_half.
struct HostState9 {
  const double* a[9];
};

// Caller indices [u0, u1), grid-stride; with `rout` the pushed positions
// also go back to the caller's arrays (in place: each thread reads its
// element before writing it).
__global__ void k_host_first_half(PushArgs P, HostState9 H, const int32_t* __restrict__ inv, double h, double h2,
                                  double hv, int64_t u0, int64_t u1, HostState9 rout) {
  for (int64_t u = u0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < u1;
       u += (int64_t)gridDim.x * blockDim.x) {
    double q[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) q[k] = H.a[k][u];
    const int64_t i = inv[u];
    const double x = __dadd_rn(q[0], __dadd_rn(__dmul_rn(q[3], h), __dmul_rn(q[6], h2)));
    const double y = __dadd_rn(q[1], __dadd_rn(__dmul_rn(q[4], h), __dmul_rn(q[7], h2)));
    const double z = __dadd_rn(q[2], __dadd_rn(__dmul_rn(q[5], h), __dmul_rn(q[8], h2)));
    P.xo[i] = x;
    P.yo[i] = y;
    P.zo[i] = z;
    P.vx[i] = __dadd_rn(q[3], __dmul_rn(q[6], hv));
    P.vy[i] = __dadd_rn(q[4], __dmul_rn(q[7], hv));
    P.vz[i] = __dadd_rn(q[5], __dmul_rn(q[8], hv));
    P.ax[i] = q[6];
    P.ay[i] = q[7];
    P.az[i] = q[8];
    if (P.refresh) refresh_gather(P.g, i, P.cellpack[i], P.type[i], x, y, z, P.pf, P.pd);
    if (P.gate) displacement_test(P.gate, P.rref, P.rcap, P.thr2, i, x, y, z);
    if (rout.a[0]) {
      const_cast<double*>(rout.a[0])[u] = x;
      const_cast<double*>(rout.a[1])[u] = y;
      const_cast<double*>(rout.a[2])[u] = z;
    }
  }
}

void launch_host_first_half(gbmd_context* c, const double* const host[9], const int32_t* inv, double dt) {
  if (!c->n) return;
  HostState9 H, none{};
  for (int k = 0; k < 9; ++k) H.a[k] = host[k];
  const double h = dt * 1.0;
  const double h2 = h * h * 0.5;
  k_host_first_half<<<nblk(c->n, 256), 256, 0, c->stream>>>(push_args(c), H, inv, h, h2, dt * 0.5, 0, c->n, none);
}

void launch_host_first_half_range(gbmd_context* c, const double* const host[9], const int32_t* inv, double dt,
                                  int64_t u0, int64_t u1, bool write_back, int blocks, int threads,
                                  cudaStream_t stream) {
  if (u1 <= u0) return;
  HostState9 H, rout{};
  for (int k = 0; k < 9; ++k) H.a[k] = host[k];
  if (write_back)
    for (int k = 0; k < 3; ++k) rout.a[k] = host[k];
  const double h = dt * 1.0;
  const double h2 = h * h * 0.5;
  const int64_t need = (u1 - u0 + threads - 1) / threads;
  const unsigned grid = (unsigned)(need < blocks ? need : blocks);
  k_host_first_half<<<grid, threads, 0, stream>>>(push_args(c), H, inv, h, h2, dt * 0.5, u0, u1, rout);
}

void launch_push_min(gbmd_context* c, double dt, double dt_scale, double tolF) {
  if (!c->n) return;
  const double h = dt * dt_scale;
  k_push_min<<<nblk(c->n, 256), 256, 0, c->stream>>>(push_args(c), h * h * 0.5, tolF);
}

// --------------------------------------------------------------------------
// thermodynamic reduction
// --------------------------------------------------------------------------
int thermo_blocks(int64_t n) {
  int64_t b = (n + TH_THREADS - 1) / TH_THREADS;
  if (b < 1) b = 1;
  if (b > TH_MAX_BLOCKS) b = TH_MAX_BLOCKS;
  return (int)b;
}

struct ThermoArgs {
  int64_t n;
  const double *vx, *vy, *vz, *ep, *vir;
  const uint8_t* type;
  int ntypes;
  double mass[GBMD_MAX_TYPES];
};

__global__ void __launch_bounds__(TH_THREADS) k_thermo_part(ThermoArgs T, double* __restrict__ part) {
  double s[26];
#pragma unroll
  for (int q = 0; q < 26; ++q) s[q] = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < T.n; i += (int64_t)gridDim.x * blockDim.x) {
    // a type outside [0, ntypes) has no mass: it makes the mass-weighted
    // sums NaN instead of reading past the table
    const unsigned ti = T.type[i];
    const double m = ti < (unsigned)T.ntypes ? T.mass[ti] : __longlong_as_double(0x7ff8000000000000ll);
    const double v[3] = {T.vx[i], T.vy[i], T.vz[i]};
    if (T.vir) {
#pragma unroll
      for (int q = 0; q < 9; ++q) s[q] += T.vir[9 * i + q];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) s[9 + 3 * a + b] += v[a] * v[b] * m;
#pragma unroll
    for (int a = 0; a < 3; ++a) s[18 + a] += v[a] * m;
#pragma unroll
    for (int a = 0; a < 3; ++a) s[21 + a] += v[a] * v[a] * m;
    if (T.ep) s[24] += T.ep[i];
    s[25] += m;
  }
  __shared__ double red[TH_THREADS / 32][26];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 26; ++q) {
    double v = s[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 26) {
    double v = 0.0;
    for (int k = 0; k < TH_THREADS / 32; ++k) v += red[k][threadIdx.x];
    part[(size_t)blockIdx.x * 26 + threadIdx.x] = v;
  }
}

// one warp per reduced quantity: lane-strided partial sums, then a fixed
// shuffle tree -- the summation order depends only on the block count
__global__ void k_thermo_final(const double* __restrict__ part, int nb, int64_t n, double* __restrict__ out) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (q >= 27) return;
  if (q == 26) {
    if (lane == 0) out[26] = (double)n;
    return;
  }
  double v = 0.0;
  for (int b = lane; b < nb; b += 32) v += part[(size_t)b * 26 + q];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) {
    if ((q >= 9 && q < 18) || (q >= 21 && q < 24)) v *= 0.5;
    out[q] = v;
  }
}

// The same two reduction kernels on caller-provided device arrays, with a
// caller-provided partial buffer of thermo_blocks(n) x 26 doubles.
void launch_thermo_raw(int64_t n, const double* vx, const double* vy, const double* vz, const double* ep,
                       const double* vir, const uint8_t* type, const double* mass, int ntypes, double* part,
                       double* out, cudaStream_t s) {
  ThermoArgs T;
  T.n = n;
  T.vx = vx; T.vy = vy; T.vz = vz;
  T.ep = ep;
  T.vir = vir;
  T.type = type;
  T.ntypes = ntypes;
  for (int t = 0; t < GBMD_MAX_TYPES; ++t) T.mass[t] = t < ntypes ? mass[t] : 1.0;
  const int nb = thermo_blocks(n);
  k_thermo_part<<<nb, TH_THREADS, 0, s>>>(T, part);
  k_thermo_final<<<1, 27 * 32, 0, s>>>(part, nb, n, out);
}

void launch_thermo(gbmd_context* c, bool with_virial) {
  ThermoArgs T;
  T.n = c->n;
  T.vx = c->VX(); T.vy = c->VY(); T.vz = c->VZ();
  T.ep = c->ep;
  T.vir = (with_virial && c->vir) ? c->vir : nullptr;
  T.type = c->TYPE();
  T.ntypes = c->ntypes > 0 ? c->ntypes : GBMD_MAX_TYPES;
  for (int t = 0; t < GBMD_MAX_TYPES; ++t) T.mass[t] = t < c->ntypes ? c->mass[t] : 1.0;
  const int nb = thermo_blocks(c->n);
  k_thermo_part<<<nb, TH_THREADS, 0, c->stream>>>(T, c->d_part);
  k_thermo_final<<<1, 27 * 32, 0, c->stream>>>(c->d_part, nb, c->n, c->d_thermo);
}

}  // namespace gbmd
