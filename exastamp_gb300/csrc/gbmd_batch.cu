// gbmd_batch.cu -- many independent periodic eam_alloy replicas of uneven
// size in one persistent launch: forward (energy, forces, virial) and the
// parameter adjoint of a force-matching + energy loss.
//
// One thread block owns one replica at a time (replicas are taken largest
// first from an atomic queue, so the launch load-balances uneven sizes).
// Everything a replica needs lives in shared memory: its cell-sorted FP32
// cell-relative positions, cell ranges, F'(rho), the loss gradients with
// respect to its per-atom forces and energies, and the adjoint
// intermediates.  Pairs are found once per replica from the (2S+1)^3 cells
// around each atom (S = 1 with cells >= rcut, or S = 2 with cells >= rcut/2;
// the autotuner picks S and the block size), with the same FP32 screen +
// FP64 re-test of the ambiguous band as the main path, so the in-cutoff pair
// set is the FP64 one; they go to a pair list in the block's own global
// scratch (128 entries per atom, slot-major), which the density, force and
// adjoint passes read.  A replica with a fuller atom walks the cells in
// every pass instead, with the same order and arithmetic.  Pair arithmetic is FP32 with compensated force and
// density sums; per-replica sums (energy, virial, loss, gradient) are FP64
// and written to the replica's own row, so results do not depend on which
// block ran which replica.
//
// Physics restated (single element, eam_alloy.h L198-313 and
// eam_force_op_multimat.h L114-343):
//   rho_i = sum_j rho(r_ij),  E_i = F(rho_i) + 1/2 sum_j phi(r_ij)
//   f_i   = sum_j u_ij (F'_i rho'(r) + F'_j rho'(r) + phi'(r))
// Adjoint (per parameter theta, derivative splines D of the tables):
//   s_ij = gF_i . u_ij,  G_i = sum_j (s_ij + s_ji) rho'_ij,
//   lam_i = gE_i F'_i + G_i F''_i
//   dL/dtheta = sum_i [gE_i dF + G_i dF'] + sum_ij [ (gE_i/2r - s_ij/r^2) dz2
//               + (s_ij/r) dz2' + s_ij (F'_i + F'_j) drho' + lam_i drho ]
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <numeric>
#include <vector>

#include "gbmd_batch_grid.h"
#include "gbmd_internal.cuh"

namespace {

constexpr int BMAX_ATOMS = 2048;   // largest replica
constexpr int BMAX_CELLS = 1024;
constexpr int SMALL_ATOMS = 512;   // replicas up to this size run in the small-block kernel
constexpr int SMALL_CELLS = 512;
constexpr int NBL_MAX = 128;       // pair-list entries per atom
constexpr int BMAX_PARAMS = 9;
constexpr int REP_ROW = 20;  // epot, virial[9], loss, grad[9]

struct BatchArgs {
  int nrep, single;
  const int64_t* off;
  const double* lo;
  const double* hi;
  const double* L;
  const double *x, *y, *z;
  double *fx, *fy, *fz, *ep;
  double* rep;  // nrep x REP_ROW
  const int* order;
  int* queue;
  int* err;
  // tables (FP32 value coefficients c3..c6, scaled by conv)
  const float4 *frho4, *rhor4, *rhod4, *z2r4;
  int nr, nrho;
  float rdr, rdrho, rhomax;
  double rcut, rcut2;
  float rc2lo, rc2hi;
  int S;
  // adjoint
  int adjoint;
  const double *Ftx, *Fty, *Ftz, *Et;
  double wF, wE;
  const float4 *dz2r4, *drhor4, *dfrho4;  // [k][knot] for the listed parameters
  int nz2, nrh, nfr;
  uint32_t* nbl;  // MAXA * NBL_MAX entries per block: the current replica's pair list
  int pz2[BMAX_PARAMS], prh[BMAX_PARAMS], pfr[BMAX_PARAMS];
};

// Shared memory of one block: a replica of up to MAXA atoms in MAXC cells.
template <int MAXA, int MAXC>
struct SmemT {
  float4 pos[MAXA];   // cell-relative FP32 position, w = local atom index bits
  float4 gfe[MAXA];   // adjoint: dL/dF (xyz) and dL/dE (w)
  int cstart[MAXC + 1];
  int cfill[MAXC];
  int cellof[MAXA];   // by local atom index
  int order[MAXA];    // slot -> local atom index
  float fp[MAXA];     // F'(rho) by slot
  float eemb[MAXA];   // F(rho) by slot
  float rho[MAXA];    // rho by slot
  float G[MAXA];      // adjoint G by slot
  int nnb[MAXA];      // pair-list length by slot
  double red[32][REP_ROW];  // block reduction
  int rep;
  int list_ok;              // every atom's pairs fit in the list
};

struct RepGeom {
  int64_t base;
  int n, nc[3], ncells;
  double lo[3], hi[3], L[3], h[3], inv_h[3];
  float hf[3];
};

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// periodic wrap with the rounding of the main path's rebuild (and the oracle)
__device__ __forceinline__ void wrap_cell(const RepGeom& g, double v, int d, double& w, int& c) {
  if (v < g.lo[d]) v = __dadd_rn(v, g.L[d]);
  else if (v >= g.hi[d]) v = __dsub_rn(v, g.L[d]);
  w = v;
  int q = (int)__dmul_rn(__dsub_rn(v, g.lo[d]), g.inv_h[d]);
  c = q < 0 ? 0 : (q > g.nc[d] - 1 ? g.nc[d] - 1 : q);
}

// Exact FP64 re-test of a pair in the ambiguous band (positions re-read and
// re-wrapped from global memory).
__device__ __noinline__ bool batch_exact(const BatchArgs& A, const RepGeom& g, int ai, int ak, int nx, int ny,
                                         int nz) {
  double wi[3], wk[3];
  int c;
  const double xi[3] = {A.x[g.base + ai], A.y[g.base + ai], A.z[g.base + ai]};
  const double xk[3] = {A.x[g.base + ak], A.y[g.base + ak], A.z[g.base + ak]};
  for (int d = 0; d < 3; ++d) {
    wrap_cell(g, xi[d], d, wi[d], c);
    wrap_cell(g, xk[d], d, wk[d], c);
  }
  double dx, dy, dz;
  return exact_d2(wi[0], wi[1], wi[2], wk[0], wk[1], wk[2], (double)nx * g.L[0], (double)ny * g.L[1],
                  (double)nz * g.L[2], dx, dy, dz) <= A.rcut2;
}

__device__ __forceinline__ float sval(const float4& c, float q) { return fmaf(fmaf(fmaf(c.x, q, c.y), q, c.z), q, c.w); }
__device__ __forceinline__ float sdq(const float4& c, float q) {  // d value / d q
  return fmaf(fmaf(3.f * c.x, q, 2.f * c.y), q, c.z);
}

__device__ __forceinline__ int knot(float t, int nmax, float& q) {
  const int m = min((int)t, nmax);
  q = fminf(t - (float)m, 1.0f);
  return m;
}

// FP32 separation of a candidate (position shifted by its cell offset) and
// its square: the one expression every pass and the list build use.
__device__ __forceinline__ float pair_d2(const float4& pi, const float4& pj, float sx, float sy, float sz,
                                         float& ddx, float& ddy, float& ddz) {
  ddx = (pj.x - pi.x) + sx;
  ddy = (pj.y - pi.y) + sy;
  ddz = (pj.z - pi.z) + sz;
  return fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz));
}

// Visit every in-cutoff neighbour of slot s from the cells around it:
// fn(k, dx, dy, dz, d2, code), code = the cell offset (dx+S) | (dy+S) << 3 | (dz+S) << 6.
template <class SM, class Fn>
__device__ __forceinline__ void for_pairs(const BatchArgs& A, const RepGeom& g, const SM& sm, int s, Fn fn) {
  const int ai = sm.order[s];
  const int c = sm.cellof[ai];
  const int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
  const float4 pi = sm.pos[s];
  const int S = A.S;
  for (int dz = -S; dz <= S; ++dz) {
    const int vz = cz + dz, nz = floor_div(vz, g.nc[2]), wz = vz - nz * g.nc[2];
    for (int dy = -S; dy <= S; ++dy) {
      const int vy = cy + dy, ny = floor_div(vy, g.nc[1]), wy = vy - ny * g.nc[1];
      for (int dx = -S; dx <= S; ++dx) {
        const int vx = cx + dx, nx = floor_div(vx, g.nc[0]), wx = vx - nx * g.nc[0];
        const int cj = (wz * g.nc[1] + wy) * g.nc[0] + wx;
        const float sx = (float)dx * g.hf[0], sy = (float)dy * g.hf[1], sz = (float)dz * g.hf[2];
        const bool self_cell = (dx | dy | dz) == 0;
        const uint32_t code = (uint32_t)(dx + S) | ((uint32_t)(dy + S) << 3) | ((uint32_t)(dz + S) << 6);
        for (int k = sm.cstart[cj]; k < sm.cstart[cj + 1]; ++k) {
          if (self_cell && k == s) continue;
          const float4 pj = sm.pos[k];
          float ddx, ddy, ddz;
          const float d2 = pair_d2(pi, pj, sx, sy, sz, ddx, ddy, ddz);
          if (d2 > A.rc2hi) continue;
          if (d2 >= A.rc2lo && !batch_exact(A, g, ai, sm.order[k], nx, ny, nz)) continue;
          fn(k, ddx, ddy, ddz, d2, code);
        }
      }
    }
  }
}

// The same neighbours, in the same order and with the same FP32 arithmetic,
// from the replica's pair list (entry: slot k | code << 11, slot-major).
template <class SM, class Fn>
__device__ __forceinline__ void for_list(const RepGeom& g, const SM& sm, const uint32_t* __restrict__ nbl,
                                         int n, int S, int s, Fn fn) {
  const float4 pi = sm.pos[s];
  const int cnt = sm.nnb[s];
  for (int q = 0; q < cnt; ++q) {
    const uint32_t e = nbl[(size_t)q * n + s];
    const int k = (int)(e & 2047u);
    const int dx = (int)((e >> 11) & 7u) - S, dy = (int)((e >> 14) & 7u) - S, dz = (int)((e >> 17) & 7u) - S;
    const float sx = (float)dx * g.hf[0], sy = (float)dy * g.hf[1], sz = (float)dz * g.hf[2];
    const float4 pj = sm.pos[k];
    float ddx, ddy, ddz;
    const float d2 = pair_d2(pi, pj, sx, sy, sz, ddx, ddy, ddz);
    fn(k, ddx, ddy, ddz, d2);
  }
}

// fn(k, dx, dy, dz, d2) over the neighbours of slot s: from the list when
// every atom's pairs fit in it, else from the cells.
template <class SM, class Fn>
__device__ __forceinline__ void visit(const BatchArgs& A, const RepGeom& g, const SM& sm,
                                      const uint32_t* nbl, int n, int s, Fn fn) {
  if (sm.list_ok)
    for_list(g, sm, nbl, n, A.S, s, fn);
  else
    for_pairs(A, g, sm, s, [&](int k, float dx, float dy, float dz, float d2, uint32_t) { fn(k, dx, dy, dz, d2); });
}

// The replica's pair list, one thread per atom walking the cells as
// for_pairs does (same FP32 screen and FP64 band re-test, same order).  A
// warp-per-cell walk with shared-memory broadcasts measured slower here: a
// replica of a few hundred atoms has too few cells to keep 16 warps busy.
template <class SM>
__device__ void build_list(const BatchArgs& A, const RepGeom& g, SM& sm, uint32_t* __restrict__ nbl, int n) {
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    int cnt = 0;
    for_pairs(A, g, sm, s, [&](int k, float, float, float, float, uint32_t code) {
      if (cnt < NBL_MAX) nbl[(size_t)cnt * n + s] = (uint32_t)k | (code << 11);
      ++cnt;
    });
    sm.nnb[s] = cnt;
    if (cnt > NBL_MAX) sm.list_ok = 0;
  }
}

template <class SM>
__device__ void block_reduce_row(SM& sm, double* v, int nv, double* out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int q = 0; q < nv; ++q) {
    double a = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) sm.red[w][q] = a;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double a = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) a += sm.red[k][threadIdx.x];
    out[threadIdx.x] = a;
  }
  __syncthreads();
}

template <int MAXA, int MAXC>
__global__ void __launch_bounds__(512, 1) k_batch(BatchArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using SM = SmemT<MAXA, MAXC>;
  SM& sm = *reinterpret_cast<SM*>(smem_raw);
  const int t = threadIdx.x, B = blockDim.x;
  // Persistent mode: take queue tickets until they run past nrep (each block
  // takes at most nrep + 1 tickets).  Single mode: exactly one replica.
  for (int iter = 0;; ++iter) {
    if (t == 0) sm.rep = A.single >= 0 ? (iter == 0 ? A.single : A.nrep) : atomicAdd(A.queue, 1);
    __syncthreads();
    const int qi = sm.rep;
    __syncthreads();
    if (qi < 0 || qi >= A.nrep) break;
    const int r = A.single >= 0 ? qi : A.order[qi];
    RepGeom g;
    g.base = A.off[r];
    g.n = (int)(A.off[r + 1] - g.base);
    for (int d = 0; d < 3; ++d) {
      g.lo[d] = A.lo[3 * r + d];
      g.L[d] = A.L[3 * r + d];
      g.hi[d] = A.hi[3 * r + d];
    }
    g.ncells = gbmd::batch_grid_dims(g.L, A.rcut, A.S, MAXC, g.nc);
    for (int d = 0; d < 3; ++d) {
      g.h[d] = g.L[d] / g.nc[d];
      g.inv_h[d] = (double)g.nc[d] / g.L[d];
      g.hf[d] = (float)g.h[d];
    }
    double* row = A.rep + (size_t)r * REP_ROW;
    if (g.n > MAXA || g.L[0] < A.rcut || g.L[1] < A.rcut || g.L[2] < A.rcut) {
      if (t == 0) {
        atomicOr(&A.err[0], 16);
        for (int q = 0; q < REP_ROW; ++q) row[q] = __longlong_as_double(0x7ff8000000000000ll);
      }
      __syncthreads();
      continue;
    }
    const int n = g.n;
    // ---- cell sort (deterministic order inside a cell: local atom index)
    for (int c = t; c < g.ncells; c += B) sm.cfill[c] = 0;
    __syncthreads();
    for (int a = t; a < n; a += B) {
      double w;
      int c3[3];
      const double xs[3] = {A.x[g.base + a], A.y[g.base + a], A.z[g.base + a]};
      for (int d = 0; d < 3; ++d) wrap_cell(g, xs[d], d, w, c3[d]);
      const int c = (c3[2] * g.nc[1] + c3[1]) * g.nc[0] + c3[0];
      sm.cellof[a] = c;
      atomicAdd(&sm.cfill[c], 1);
    }
    __syncthreads();
    if (t < 32) {  // warp scan of the cell counts
      const int per = (g.ncells + 31) / 32;
      int loc = 0;
      for (int k = 0; k < per; ++k) {
        const int c = t * per + k;
        if (c < g.ncells) loc += sm.cfill[c];
      }
      int inc = loc;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (t >= o) inc += v;
      }
      int run = inc - loc;
      for (int k = 0; k < per; ++k) {
        const int c = t * per + k;
        if (c < g.ncells) {
          sm.cstart[c] = run;
          run += sm.cfill[c];
          sm.cfill[c] = 0;
        }
      }
      if (t == 31) sm.cstart[g.ncells] = inc;
    }
    __syncthreads();
    for (int a = t; a < n; a += B) {
      const int c = sm.cellof[a];
      sm.order[sm.cstart[c] + atomicAdd(&sm.cfill[c], 1)] = a;
    }
    __syncthreads();
    for (int c = t; c < g.ncells; c += B) {  // insertion sort of the cell's atoms
      const int b = sm.cstart[c], e = sm.cstart[c + 1];
      for (int k = b + 1; k < e; ++k) {
        const int v = sm.order[k];
        int m = k - 1;
        while (m >= b && sm.order[m] > v) {
          sm.order[m + 1] = sm.order[m];
          --m;
        }
        sm.order[m + 1] = v;
      }
    }
    __syncthreads();
    for (int s = t; s < n; s += B) {
      const int a = sm.order[s], c = sm.cellof[a];
      const int c3[3] = {c % g.nc[0], (c / g.nc[0]) % g.nc[1], c / (g.nc[0] * g.nc[1])};
      const double xs[3] = {A.x[g.base + a], A.y[g.base + a], A.z[g.base + a]};
      float lp[3];
      for (int d = 0; d < 3; ++d) {
        double w;
        int cc;
        wrap_cell(g, xs[d], d, w, cc);
        lp[d] = (float)(w - (double)c3[d] * g.h[d] - g.lo[d]);
      }
      sm.pos[s] = make_float4(lp[0], lp[1], lp[2], __int_as_float(a));
    }
    if (t == 0) sm.list_ok = 1;
    __syncthreads();
    // ---- pair list: one walk over the cells (FP32 screen, FP64 band
    // re-test), then every pass below reads the list
    uint32_t* nbl = A.nbl + (A.single >= 0 ? (size_t)0 : (size_t)blockIdx.x * MAXA * NBL_MAX);
    build_list(A, g, sm, nbl, n);
    __syncthreads();
    // ---- density + embedding
    for (int s = t; s < n; s += B) {
      float acc = 0.f, comp = 0.f;
      visit(A, g, sm, nbl, n, s, [&](int k, float dx, float dy, float dz, float d2) {
        const float rr = d2 * rsqrtf(d2);
        float q;
        const int m = knot(fmaf(rr, A.rdr, 1.f), A.nr - 1, q);
        kahan_add(acc, comp, sval(A.rhor4[m], q));
      });
      const float R = acc - comp;
      float q = fmaf(R, A.rdrho, 1.f);
      int m = (int)q;
      m = max(1, min(m, A.nrho - 1));
      q = fminf(q - (float)m, 1.f);
      const float4 c = A.frho4[m];
      const float fp = sdq(c, q) * A.rdrho;
      float e = sval(c, q);
      if (R > A.rhomax) e = fmaf(fp, R - A.rhomax, e);
      sm.fp[s] = fp;
      sm.eemb[s] = e;
      sm.rho[s] = R;
    }
    __syncthreads();
    // ---- forces, energies, virial; loss residuals
    // per-thread sums: energy, virial, loss (static indices) and the
    // parameter gradient by parameter slot
    double acc_rep[REP_ROW];
    double acc_par[BMAX_PARAMS];
    for (int q = 0; q < REP_ROW; ++q) acc_rep[q] = 0.0;
    for (int q = 0; q < BMAX_PARAMS; ++q) acc_par[q] = 0.0;
    for (int s = t; s < n; s += B) {
      float fx = 0.f, fy = 0.f, fz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, ee = 0.f, ce = 0.f;
      float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      const float fpi = sm.fp[s];
      visit(A, g, sm, nbl, n, s, [&](int k, float dx, float dy, float dz, float d2) {
        const float rs = rsqrtf(d2), rr = d2 * rs;
        float q;
        const int m = knot(fmaf(rr, A.rdr, 1.f), A.nr - 1, q);
        const float4 dr = A.rhod4[m];
        const float rhop = fmaf(fmaf(dr.x, q, dr.y), q, dr.z);
        const float4 cz2 = A.z2r4[m];
        const float z2 = sval(cz2, q), z2d = sdq(cz2, q) * A.rdr;
        const float phi = z2 * rs;
        const float phip = (z2d - phi) * rs;
        const float psip = fmaf(fpi + sm.fp[k], rhop, phip);
        const float fpair = psip * rs;
        kahan_add(fx, cx, dx * fpair);
        kahan_add(fy, cy, dy * fpair);
        kahan_add(fz, cz, dz * fpair);
        kahan_add(ee, ce, 0.5f * phi);
        const float hh = -0.5f * fpair;
        v[0] = fmaf(hh * dx, dx, v[0]);
        v[1] = fmaf(hh * dy, dy, v[1]);
        v[2] = fmaf(hh * dz, dz, v[2]);
        v[3] = fmaf(hh * dx, dy, v[3]);
        v[4] = fmaf(hh * dx, dz, v[4]);
        v[5] = fmaf(hh * dy, dz, v[5]);
      });
      const int a = sm.order[s];
      const int64_t ga = g.base + a;
      const double Fx = (double)(fx - cx), Fy = (double)(fy - cy), Fz = (double)(fz - cz);
      const double E = (double)sm.eemb[s] + (double)(ee - ce);
      A.fx[ga] = Fx;
      A.fy[ga] = Fy;
      A.fz[ga] = Fz;
      A.ep[ga] = E;
      acc_rep[0] += E;
      acc_rep[1] += v[0]; acc_rep[2] += v[3]; acc_rep[3] += v[4];
      acc_rep[4] += v[3]; acc_rep[5] += v[1]; acc_rep[6] += v[5];
      acc_rep[7] += v[4]; acc_rep[8] += v[5]; acc_rep[9] += v[2];
      if (A.adjoint) {
        const double ex = Fx - A.Ftx[ga], ey = Fy - A.Fty[ga], ez = Fz - A.Ftz[ga], de = E - A.Et[ga];
        acc_rep[10] += A.wF * (ex * ex + ey * ey + ez * ez) + A.wE * de * de;
        sm.gfe[s] = make_float4((float)(2.0 * A.wF * ex), (float)(2.0 * A.wF * ey), (float)(2.0 * A.wF * ez),
                                (float)(2.0 * A.wE * de));
      }
    }
    if (A.adjoint) {
      __syncthreads();
      // ---- adjoint sweep 1: G_i, and the phi / phi' / rho' parameter terms
      for (int s = t; s < n; s += B) {
        const float4 gi = sm.gfe[s];
        const float fpi = sm.fp[s];
        float Gs = 0.f;
        // this atom's parameter terms, FP32 over its pairs (static indices:
        // registers), folded into the FP64 per-thread sums once per atom
        float gz[BMAX_PARAMS], gr[BMAX_PARAMS];
#pragma unroll
        for (int p = 0; p < BMAX_PARAMS; ++p) gz[p] = gr[p] = 0.f;
        visit(A, g, sm, nbl, n, s, [&](int k, float dx, float dy, float dz, float d2) {
          const float rs = rsqrtf(d2), rr = d2 * rs;
          float q;
          const int m = knot(fmaf(rr, A.rdr, 1.f), A.nr - 1, q);
          const float ux = dx * rs, uy = dy * rs, uz = dz * rs;
          const float4 gk = sm.gfe[k];
          const float sij = fmaf(gi.x, ux, fmaf(gi.y, uy, gi.z * uz));
          const float sji = -fmaf(gk.x, ux, fmaf(gk.y, uy, gk.z * uz));
          const float4 dr = A.rhod4[m];
          const float rhop = fmaf(fmaf(dr.x, q, dr.y), q, dr.z);
          Gs = fmaf(sij + sji, rhop, Gs);
          const float wv = (0.5f * gi.w - sij * rs) * rs;  // weight of dz2
          const float wd = sij * rs * A.rdr;              // weight of dz2/dq
          const float wr = sij * (fpi + sm.fp[k]) * A.rdr; // weight of drho/dq
#pragma unroll
          for (int p = 0; p < BMAX_PARAMS; ++p) {
            if (p < A.nz2) {
              const float4 c = A.dz2r4[(size_t)p * (A.nr + 1) + m];
              gz[p] += fmaf(wv, sval(c, q), wd * sdq(c, q));
            }
            if (p < A.nrh) {
              const float4 c = A.drhor4[(size_t)p * (A.nr + 1) + m];
              gr[p] = fmaf(wr, sdq(c, q), gr[p]);
            }
          }
        });
        sm.G[s] = Gs;
#pragma unroll
        for (int p = 0; p < BMAX_PARAMS; ++p) {
          if (p < A.nz2) acc_par[A.pz2[p]] += (double)gz[p];
          if (p < A.nrh) acc_par[A.prh[p]] += (double)gr[p];
        }
      }
      __syncthreads();
      // ---- adjoint sweep 2: embedding terms and lam_i * drho
      for (int s = t; s < n; s += B) {
        const float4 gi = sm.gfe[s];
        const float R = sm.rho[s];
        float q = fmaf(R, A.rdrho, 1.f);
        int m = (int)q;
        m = max(1, min(m, A.nrho - 1));
        q = fminf(q - (float)m, 1.f);
        const float4 c = A.frho4[m];
        const bool over = R > A.rhomax;
        const float f2 = over ? 0.f : fmaf(6.f * c.x, q, 2.f * c.y) * A.rdrho * A.rdrho;
        const float Gs = sm.G[s];
        const float lam = fmaf(gi.w, sm.fp[s], Gs * f2);
        for (int p = 0; p < A.nfr; ++p) {
          const float4 dc = A.dfrho4[(size_t)p * (A.nrho + 1) + m];
          const float dfp = sdq(dc, q) * A.rdrho;
          acc_par[A.pfr[p]] += (double)fmaf(gi.w, sval(dc, q) + (over ? dfp * (R - A.rhomax) : 0.f), Gs * dfp);
        }
        // lam_i * sum_j drho(r_ij): the pair sums in FP32, lam once per atom
        float gd[BMAX_PARAMS];
#pragma unroll
        for (int p = 0; p < BMAX_PARAMS; ++p) gd[p] = 0.f;
        visit(A, g, sm, nbl, n, s, [&](int k, float dx, float dy, float dz, float d2) {
          const float rr = d2 * rsqrtf(d2);
          float qq;
          const int mm = knot(fmaf(rr, A.rdr, 1.f), A.nr - 1, qq);
#pragma unroll
          for (int p = 0; p < BMAX_PARAMS; ++p)
            if (p < A.nrh) gd[p] += sval(A.drhor4[(size_t)p * (A.nr + 1) + mm], qq);
        });
#pragma unroll
        for (int p = 0; p < BMAX_PARAMS; ++p)
          if (p < A.nrh) acc_par[A.prh[p]] += (double)(lam * gd[p]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < BMAX_PARAMS; ++q) acc_rep[11 + q] = acc_par[q];
    block_reduce_row(sm, acc_rep, REP_ROW, row);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct gbmd_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  int nrep = 0;
  int64_t n = 0;
  int64_t *off = nullptr;
  double *lo = nullptr, *hi = nullptr, *L = nullptr, *x = nullptr, *y = nullptr, *z = nullptr;
  double *fx = nullptr, *fy = nullptr, *fz = nullptr, *ep = nullptr, *rep = nullptr;
  double *Ftx = nullptr, *Fty = nullptr, *Ftz = nullptr, *Et = nullptr;
  int *order = nullptr, *queue = nullptr, *d_err = nullptr;
  float4* tab = nullptr;
  float4* dtab = nullptr;
  BatchArgs a{};
  bool have_pot = false, have_targets = false;
  int block = 256, S = 1;
  int small_block = 128;         // threads per block of the small-replica kernel
  cudaStream_t side = nullptr;   // runs the small-replica kernel beside the large one
  cudaEvent_t fork = nullptr, join = nullptr;
  int nbig = 0;                  // replicas of more than SMALL_ATOMS atoms (first in `order`)
  std::vector<int> rep_atoms;    // atoms per replica (host copy)
  uint32_t* nbl = nullptr;       // pair-list scratch of the large-replica kernel's blocks
  size_t nbl_regions = 0;
  uint32_t* nbl_small = nullptr; // and of the small-replica kernel's blocks
  size_t nbl_small_regions = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_adjoint = -1;
};

namespace {

int berr(gbmd_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCUDA(b, call)                                                               \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) return berr((b), GBMD_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

void free_atoms(gbmd_batch* b) {
  void* ps[] = {b->off, b->lo, b->hi, b->L, b->x, b->y, b->z, b->fx, b->fy, b->fz, b->ep, b->rep,
                b->Ftx, b->Fty, b->Ftz, b->Et, b->order};
  for (void* p : ps) cudaFree(p);
  b->off = nullptr; b->lo = b->hi = b->L = b->x = b->y = b->z = nullptr;
  b->fx = b->fy = b->fz = b->ep = b->rep = nullptr;
  b->Ftx = b->Fty = b->Ftz = b->Et = nullptr;
  b->order = nullptr;
}

void drop_graph(gbmd_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

// spline a table of knot values and return its FP32 value coefficients
void table_f4(int n, double delta, const double* vals, double scale, std::vector<float4>& out) {
  std::vector<double> f(n + 1, 0.0), s((size_t)(n + 1) * 8);
  for (int k = 0; k < n; ++k) f[k + 1] = vals[k];
  gbmd::spline7(n, delta, f.data(), s.data());
  for (int m = 0; m <= n; ++m)
    out.push_back(make_float4((float)(s[m * 8 + 3] * scale), (float)(s[m * 8 + 4] * scale),
                              (float)(s[m * 8 + 5] * scale), (float)(s[m * 8 + 6] * scale)));
}

constexpr size_t SMEM_BIG = sizeof(SmemT<BMAX_ATOMS, BMAX_CELLS>);
constexpr size_t SMEM_SMALL = sizeof(SmemT<SMALL_ATOMS, SMALL_CELLS>);
auto* const K_BIG = &k_batch<BMAX_ATOMS, BMAX_CELLS>;
auto* const K_SMALL = &k_batch<SMALL_ATOMS, SMALL_CELLS>;

}  // namespace

extern "C" {

int gbmd_batch_create(gbmd_batch** out, int device, void* stream) {
  if (!out) return GBMD_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GBMD_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return GBMD_ERR_INVALID;
  gbmd_batch* b = new gbmd_batch();
  b->device = device;
  cudaSetDevice(device);
  if (stream) {
    b->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete b;
      return GBMD_ERR_CUDA;
    }
    b->own_stream = true;
  }
  if (cudaMalloc(&b->queue, sizeof(int) * 2) != cudaSuccess || cudaMalloc(&b->d_err, sizeof(int) * 4) != cudaSuccess ||
      cudaMemset(b->d_err, 0, sizeof(int) * 4) != cudaSuccess ||
      cudaFuncSetAttribute(K_BIG, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BIG) != cudaSuccess ||
      cudaFuncSetAttribute(K_SMALL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_SMALL) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess) {
    cudaFree(b->queue);
    cudaFree(b->d_err);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return GBMD_ERR_CUDA;
  }
  *out = b;
  return GBMD_OK;
}

int gbmd_batch_destroy(gbmd_batch* b) {
  if (!b) return GBMD_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  free_atoms(b);
  cudaFree(b->queue);
  cudaFree(b->d_err);
  cudaFree(b->tab);
  cudaFree(b->dtab);
  cudaFree(b->nbl);
  cudaFree(b->nbl_small);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  delete b;
  return GBMD_OK;
}

const char* gbmd_batch_last_error(const gbmd_batch* b) { return b ? b->err.c_str() : "null batch"; }

int gbmd_batch_set_eam_alloy(gbmd_batch* b, int nrho, double drho, int nr, double dr, const double* frho,
                             const double* rhor, const double* z2r, double rcut, double conv_z2r,
                             double conv_frho) {
  if (!b || nrho < 5 || nr < 5 || !(drho > 0) || !(dr > 0) || !frho || !rhor || !z2r || !(rcut > 0))
    return berr(b, GBMD_ERR_INVALID, "bad eam_alloy tables");
  std::vector<float4> h;
  table_f4(nrho, drho, frho, conv_frho, h);
  table_f4(nr, dr, rhor, 1.0, h);
  table_f4(nr, dr, z2r, conv_z2r, h);
  // rho' coefficients (3c3, 2c4, c5) / dr
  {
    std::vector<double> f(nr + 1, 0.0), s((size_t)(nr + 1) * 8);
    for (int k = 0; k < nr; ++k) f[k + 1] = rhor[k];
    gbmd::spline7(nr, dr, f.data(), s.data());
    for (int m = 0; m <= nr; ++m)
      h.push_back(make_float4((float)(3.0 * s[m * 8 + 3] / dr), (float)(2.0 * s[m * 8 + 4] / dr),
                              (float)(s[m * 8 + 5] / dr), 0.f));
  }
  cudaSetDevice(b->device);
  cudaFree(b->tab);
  b->tab = nullptr;
  BCUDA(b, cudaMalloc(&b->tab, sizeof(float4) * h.size()));
  BCUDA(b, cudaMemcpy(b->tab, h.data(), sizeof(float4) * h.size(), cudaMemcpyHostToDevice));
  BatchArgs& A = b->a;
  A.frho4 = b->tab;
  A.rhor4 = A.frho4 + (nrho + 1);
  A.z2r4 = A.rhor4 + (nr + 1);
  A.rhod4 = A.z2r4 + (nr + 1);
  A.nr = nr;
  A.nrho = nrho;
  A.rdr = (float)(1.0 / dr);
  A.rdrho = (float)(1.0 / drho);
  A.rhomax = (float)((nrho - 1) * drho);
  A.rcut = rcut;
  A.rcut2 = rcut * rcut;
  A.rc2lo = (float)(A.rcut2 * (1.0 - 0x1p-12));
  A.rc2hi = (float)(A.rcut2 * (1.0 + 0x1p-12));
  b->have_pot = true;
  A.nz2 = A.nrh = A.nfr = 0;
  drop_graph(b);
  return GBMD_OK;
}

int gbmd_batch_set_param_derivatives(gbmd_batch* b, int nparam, const double* dfrho, const double* drhor,
                                     const double* dz2r, double conv_z2r, double conv_frho) {
  if (!b || !b->have_pot || nparam < 1 || nparam > BMAX_PARAMS || !dfrho || !drhor || !dz2r)
    return berr(b, GBMD_ERR_INVALID, "bad parameter derivative tables (set the potential first)");
  BatchArgs& A = b->a;
  const int nr = A.nr, nrho = A.nrho;
  const double dr = 1.0 / (double)A.rdr, drho = 1.0 / (double)A.rdrho;
  std::vector<float4> fr, rh, zz;
  A.nz2 = A.nrh = A.nfr = 0;
  for (int p = 0; p < nparam; ++p) {
    auto nonzero = [](const double* v, int k) {
      for (int q = 0; q < k; ++q)
        if (v[q] != 0.0) return true;
      return false;
    };
    if (nonzero(dfrho + (size_t)p * nrho, nrho)) {
      table_f4(nrho, drho, dfrho + (size_t)p * nrho, conv_frho, fr);
      A.pfr[A.nfr++] = p;
    }
    if (nonzero(drhor + (size_t)p * nr, nr)) {
      table_f4(nr, dr, drhor + (size_t)p * nr, 1.0, rh);
      A.prh[A.nrh++] = p;
    }
    if (nonzero(dz2r + (size_t)p * nr, nr)) {
      table_f4(nr, dr, dz2r + (size_t)p * nr, conv_z2r, zz);
      A.pz2[A.nz2++] = p;
    }
  }
  std::vector<float4> h;
  h.insert(h.end(), fr.begin(), fr.end());
  h.insert(h.end(), rh.begin(), rh.end());
  h.insert(h.end(), zz.begin(), zz.end());
  cudaSetDevice(b->device);
  cudaFree(b->dtab);
  b->dtab = nullptr;
  BCUDA(b, cudaMalloc(&b->dtab, sizeof(float4) * (h.size() + 1)));
  BCUDA(b, cudaMemcpy(b->dtab, h.data(), sizeof(float4) * h.size(), cudaMemcpyHostToDevice));
  A.dfrho4 = b->dtab;
  A.drhor4 = A.dfrho4 + fr.size();
  A.dz2r4 = A.drhor4 + rh.size();
  drop_graph(b);
  return GBMD_OK;
}

int gbmd_batch_upload(gbmd_batch* b, int nrep, const int64_t* offsets, const double* lo, const double* hi,
                      const double* x, const double* y, const double* z) {
  if (!b || nrep < 1 || !offsets || !lo || !hi || !x || !y || !z) return berr(b, GBMD_ERR_INVALID, "bad replicas");
  if (offsets[0] != 0) return berr(b, GBMD_ERR_INVALID, "offsets[0] must be 0");
  for (int r = 0; r < nrep; ++r) {
    const int64_t m = offsets[r + 1] - offsets[r];
    if (m < 0) return berr(b, GBMD_ERR_INVALID, "offsets must be non-decreasing");
    if (m > BMAX_ATOMS) return berr(b, GBMD_ERR_TOO_LARGE, "replica %d has %lld atoms (max %d)", r, (long long)m, BMAX_ATOMS);
    if (!gbmd::batch_box_ok(lo + 3 * r, hi + 3 * r))
      return berr(b, GBMD_ERR_INVALID, "replica %d: empty or non-finite box", r);
  }
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  drop_graph(b);
  free_atoms(b);
  const int64_t n = offsets[nrep];
  b->nrep = nrep;
  b->n = n;
  std::vector<double> L(3 * (size_t)nrep);
  for (size_t q = 0; q < L.size(); ++q) L[q] = hi[q] - lo[q];
  // largest replicas first (longest-processing-time order for the queue)
  std::vector<int> ord(nrep);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) {
    return offsets[a + 1] - offsets[a] > offsets[c + 1] - offsets[c];
  });
  b->rep_atoms.resize(nrep);
  b->nbig = 0;
  for (int r = 0; r < nrep; ++r) {
    b->rep_atoms[r] = (int)(offsets[r + 1] - offsets[r]);
    if (b->rep_atoms[r] > SMALL_ATOMS) ++b->nbig;
  }
  const size_t nb = sizeof(double) * (size_t)(n > 0 ? n : 1);
  BCUDA(b, cudaMalloc(&b->off, sizeof(int64_t) * (nrep + 1)));
  BCUDA(b, cudaMalloc(&b->lo, sizeof(double) * 3 * nrep));
  BCUDA(b, cudaMalloc(&b->L, sizeof(double) * 3 * nrep));
  BCUDA(b, cudaMalloc(&b->hi, sizeof(double) * 3 * nrep));
  BCUDA(b, cudaMalloc(&b->order, sizeof(int) * nrep));
  BCUDA(b, cudaMalloc(&b->rep, sizeof(double) * REP_ROW * nrep));
  double** arrs[] = {&b->x, &b->y, &b->z, &b->fx, &b->fy, &b->fz, &b->ep, &b->Ftx, &b->Fty, &b->Ftz, &b->Et};
  for (double** p : arrs) BCUDA(b, cudaMalloc(p, nb));
  BCUDA(b, cudaMemcpy(b->off, offsets, sizeof(int64_t) * (nrep + 1), cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->lo, lo, sizeof(double) * 3 * nrep, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->L, L.data(), sizeof(double) * 3 * nrep, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->hi, hi, sizeof(double) * 3 * nrep, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->order, ord.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->x, x, nb, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->y, y, nb, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->z, z, nb, cudaMemcpyHostToDevice));
  b->have_targets = false;
  return GBMD_OK;
}

int gbmd_batch_set_targets(gbmd_batch* b, const double* fx, const double* fy, const double* fz, const double* e,
                           double wF, double wE) {
  if (!b || !b->x || !fx || !fy || !fz || !e) return berr(b, GBMD_ERR_INVALID, "bad targets (upload first)");
  const size_t nb = sizeof(double) * (size_t)b->n;
  BCUDA(b, cudaMemcpy(b->Ftx, fx, nb, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->Fty, fy, nb, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->Ftz, fz, nb, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMemcpy(b->Et, e, nb, cudaMemcpyHostToDevice));
  b->a.wF = wF;
  b->a.wE = wE;
  b->have_targets = true;
  drop_graph(b);
  return GBMD_OK;
}

int gbmd_batch_set_small_block(gbmd_batch* b, int block) {
  if (!b || block < 64 || block > 256 || block % 32) return berr(b, GBMD_ERR_INVALID, "small block in [64,256], multiple of 32");
  b->small_block = block;
  drop_graph(b);
  return GBMD_OK;
}

int gbmd_batch_set_launch(gbmd_batch* b, int block, int stencil) {
  if (!b || block < 64 || block > 512 || block % 32 || (stencil != 1 && stencil != 2))
    return berr(b, GBMD_ERR_INVALID, "block in [64,512] (multiple of 32), stencil 1 or 2");
  b->block = block;
  b->S = stencil;
  drop_graph(b);
  return GBMD_OK;
}

// Blocks of a persistent launch: as many as fit on the device at once, at
// most one per replica of its queue.  big: the large-replica kernel (the
// autotuned block), else the small-replica kernel (b->small_block threads).
static int persistent_grid(gbmd_batch* b, bool big) {
  int dev_sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, b->device);
  if (big)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, K_BIG, b->block, SMEM_BIG);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, K_SMALL, b->small_block, SMEM_SMALL);
  const int nq = big ? b->nbig : b->nrep - b->nbig;
  return std::max(1, std::min(nq, dev_sms * std::max(per_sm, 1)));
}

// pair-list scratch for `regions` blocks of each kernel (allocated outside any capture)
static int ensure_nbl(gbmd_batch* b, int regions, int small_regions) {
  if ((size_t)regions > b->nbl_regions) {
    drop_graph(b);
    cudaFree(b->nbl);
    b->nbl = nullptr;
    b->nbl_regions = 0;
    BCUDA(b, cudaMalloc(&b->nbl, sizeof(uint32_t) * BMAX_ATOMS * NBL_MAX * (size_t)regions));
    b->nbl_regions = (size_t)regions;
  }
  if ((size_t)small_regions > b->nbl_small_regions) {
    drop_graph(b);
    cudaFree(b->nbl_small);
    b->nbl_small = nullptr;
    b->nbl_small_regions = 0;
    BCUDA(b, cudaMalloc(&b->nbl_small, sizeof(uint32_t) * SMALL_ATOMS * NBL_MAX * (size_t)small_regions));
    b->nbl_small_regions = (size_t)small_regions;
  }
  return GBMD_OK;
}

// Replicas of more than SMALL_ATOMS atoms run in the large-replica kernel
// (one block of up to 512 threads and 136 KB of shared memory per SM), the
// rest in the small-replica kernel (64-256 threads, 36 KB, several blocks per
// SM); each takes its replicas from its own queue, largest first.
static int batch_launch(gbmd_batch* b, int adjoint, int per_replica) {
  BatchArgs A = b->a;
  A.nrep = b->nrep;
  A.off = b->off;
  A.lo = b->lo;
  A.hi = b->hi;
  A.L = b->L;
  A.x = b->x; A.y = b->y; A.z = b->z;
  A.fx = b->fx; A.fy = b->fy; A.fz = b->fz; A.ep = b->ep;
  A.rep = b->rep;
  A.order = b->order;
  A.queue = b->queue;
  A.err = b->d_err;
  A.S = b->S;
  A.adjoint = adjoint;
  A.Ftx = b->Ftx; A.Fty = b->Fty; A.Ftz = b->Ftz; A.Et = b->Et;
  if (per_replica) {
    for (int r = 0; r < b->nrep; ++r) {
      A.single = r;
      if (b->rep_atoms[r] > SMALL_ATOMS) {
        A.nbl = b->nbl;
        K_BIG<<<1, b->block, SMEM_BIG, b->stream>>>(A);
      } else {
        A.nbl = b->nbl_small;
        K_SMALL<<<1, b->small_block, SMEM_SMALL, b->stream>>>(A);
      }
    }
  } else {
    A.single = -1;
    BCUDA(b, cudaMemsetAsync(b->queue, 0, sizeof(int) * 2, b->stream));
    // the two size classes on two streams, so the small-replica blocks take
    // over SMs as the large-replica kernel's blocks run out of work
    const bool both = b->nbig > 0 && b->nrep > b->nbig;
    if (both) {
      BCUDA(b, cudaEventRecord(b->fork, b->stream));
      BCUDA(b, cudaStreamWaitEvent(b->side, b->fork, 0));
    }
    if (b->nbig > 0) {
      const int grid = persistent_grid(b, true);
      if ((size_t)grid > b->nbl_regions) return berr(b, GBMD_ERR_INVALID, "pair-list scratch not sized");
      BatchArgs Ab = A;
      Ab.nrep = b->nbig;
      Ab.nbl = b->nbl;
      K_BIG<<<grid, b->block, SMEM_BIG, b->stream>>>(Ab);
    }
    if (b->nrep > b->nbig) {
      const int grid = persistent_grid(b, false);
      if ((size_t)grid > b->nbl_small_regions) return berr(b, GBMD_ERR_INVALID, "pair-list scratch not sized");
      BatchArgs As = A;
      As.nrep = b->nrep - b->nbig;
      As.order = b->order + b->nbig;
      As.queue = b->queue + 1;
      As.nbl = b->nbl_small;
      K_SMALL<<<grid, b->small_block, SMEM_SMALL, both ? b->side : b->stream>>>(As);
    }
    if (both) {
      BCUDA(b, cudaEventRecord(b->join, b->side));
      BCUDA(b, cudaStreamWaitEvent(b->stream, b->join, 0));
    }
  }
  BCUDA(b, cudaGetLastError());
  return GBMD_OK;
}

int gbmd_batch_run(gbmd_batch* b, int adjoint, int per_replica, int use_graph) {
  if (!b || !b->have_pot || !b->x) return berr(b, GBMD_ERR_INVALID, "set the potential and upload replicas first");
  if (adjoint && (!b->have_targets || b->a.nz2 + b->a.nrh + b->a.nfr == 0))
    return berr(b, GBMD_ERR_INVALID, "adjoint needs targets and parameter derivatives");
  cudaSetDevice(b->device);
  {
    const int rc = per_replica ? ensure_nbl(b, 1, 1)
                               : ensure_nbl(b, b->nbig > 0 ? persistent_grid(b, true) : 0,
                                            b->nrep > b->nbig ? persistent_grid(b, false) : 0);
    if (rc) return rc;
  }
  if (use_graph && !per_replica) {
    if (!b->graph || b->graph_adjoint != adjoint) {
      drop_graph(b);
      cudaGraph_t g;
      BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      const int rc = batch_launch(b, adjoint, 0);
      cudaError_t e = cudaStreamEndCapture(b->stream, &g);
      if (rc) return rc;
      if (e != cudaSuccess) return berr(b, GBMD_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return berr(b, GBMD_ERR_CUDA, "instantiate: %s", cudaGetErrorString(e));
      b->graph_adjoint = adjoint;
    }
    BCUDA(b, cudaGraphLaunch(b->graph, b->stream));
  } else {
    const int rc = batch_launch(b, adjoint, per_replica);
    if (rc) return rc;
  }
  return GBMD_OK;
}

int gbmd_batch_synchronize(gbmd_batch* b) {
  if (!b) return GBMD_ERR_INVALID;
  BCUDA(b, cudaStreamSynchronize(b->stream));
  int h[4];
  BCUDA(b, cudaMemcpy(h, b->d_err, sizeof(h), cudaMemcpyDeviceToHost));
  if (h[0] & 16) return berr(b, GBMD_ERR_TOO_LARGE, "a replica exceeded the per-block limits (atoms or box)");
  return GBMD_OK;
}

int gbmd_batch_download(gbmd_batch* b, double* fx, double* fy, double* fz, double* ep, double* rep_energy,
                        double* rep_virial, double* loss, double* grad) {
  if (!b || !b->x) return GBMD_ERR_INVALID;
  int rc = gbmd_batch_synchronize(b);
  if (rc) return rc;
  const size_t nb = sizeof(double) * (size_t)b->n;
  if (fx) BCUDA(b, cudaMemcpy(fx, b->fx, nb, cudaMemcpyDeviceToHost));
  if (fy) BCUDA(b, cudaMemcpy(fy, b->fy, nb, cudaMemcpyDeviceToHost));
  if (fz) BCUDA(b, cudaMemcpy(fz, b->fz, nb, cudaMemcpyDeviceToHost));
  if (ep) BCUDA(b, cudaMemcpy(ep, b->ep, nb, cudaMemcpyDeviceToHost));
  std::vector<double> rows((size_t)REP_ROW * b->nrep);
  BCUDA(b, cudaMemcpy(rows.data(), b->rep, sizeof(double) * rows.size(), cudaMemcpyDeviceToHost));
  double L = 0.0, G[BMAX_PARAMS] = {0};
  for (int r = 0; r < b->nrep; ++r) {  // replica order: fixed summation order
    const double* row = &rows[(size_t)r * REP_ROW];
    if (rep_energy) rep_energy[r] = row[0];
    if (rep_virial)
      for (int q = 0; q < 9; ++q) rep_virial[9 * r + q] = row[1 + q];
    L += row[10];
    for (int q = 0; q < BMAX_PARAMS; ++q) G[q] += row[11 + q];
  }
  if (loss) *loss = L;
  if (grad)
    for (int q = 0; q < BMAX_PARAMS; ++q) grad[q] = G[q];
  return GBMD_OK;
}

}  // extern "C"
