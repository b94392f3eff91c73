// gbmd_pair_common.cuh -- pieces shared by the pair kernels (LJ, EAM).
//
// Thread mapping: T consecutive lanes own one atom i (atoms in cell order).
// The list is stored in rows of W = T*V words per atom (V entries per lane per
// load), consecutive atoms adjacent: row r of atom i is nbr[r*stride + i*W ..
// + W), so a warp reads 32*V*4 contiguous bytes per load.  Per-atom sums are reduced across the T lanes
// with shuffles; lane 0 of the group runs the epilogue.
//
// Epilogue (lane 0): a = f/m (force_to_accel), optional ep / virial stores,
// and the fused velocity-Verlet half steps:
//   fuse 1 (push2):        v += a*dt/2                              (verlet_second_half)
//   fuse 2 (push2+push1):  v += a*dt/2; r' = r + v*dt + a*dt^2/2; v += a*dt/2
//                          (second half of this step + first half of the next)
// New positions go to the other position buffer, with the FP32/FP64 gather
// copies, so no thread ever reads a position that is being rewritten.
#pragma once
#include "gbmd_internal.cuh"

namespace gbmd {

struct PairArgs {
  int64_t n;                  // atoms [i0, n) are processed (a piece of the cell order, or all)
  int64_t i0;
  int64_t stride;             // npad * W (words per list row)
  int W, wsh;                 // words per atom per row (lanes x entries per lane), log2 W
  const uint32_t* nbr;
  const int32_t* nnb;
  int maxnb;
  const float4* posf;
  const double4_32a* posd;
  const int32_t* cellpack;
  Grid g;
  const double *x, *y, *z;    // current FP64 positions
  double *xo, *yo, *zo;       // next positions (fuse 2)
  float4* posf_o;
  double4_32a* posd_o;
  double *vx, *vy, *vz, *ax, *ay, *az;
  double *vxo, *vyo, *vzo;    // velocities after the fused halves (vx.. in place, or another buffer)
  double* ep;
  double* ep_emb;             // FP64 EAM: embedding energy F(rho_i) from the density pass
  double* vir;
  const uint8_t* type;
  double mass[GBMD_MAX_TYPES];
  float inv_massf[GBMD_MAX_TYPES];
  int fuse;
  int* gate;                  // fuse 2 with the displacement trigger: set when an atom moved > skin/2
  const double* rref;         // positions at the last rebuild (3 planes of rcap)
  int64_t rcap;
  double thr2;                // (skin/2)^2
  int want_energy, want_virial;
  double dt, dth, dt2h;
  int* err;
};

// Mixed-precision pair kernels (gbmd_mixed.cu); part as in launch_forces.
int launch_mixed(gbmd_context* c, const PairArgs& A, int part, bool ev);
// Raises the shared-memory limit of the staged pair kernels (gbmd_mixed.cu);
// called when staging is switched on, never during a stream capture.
int configure_staged_kernels();
// Pair-kernel arguments for the context's current buffers (gbmd_forces.cu).
PairArgs make_args(gbmd_context* c, const ForceFlags& f);
// lj_compute_force parameter adjoint (gbmd_adjoint_lj.cu): targets are
// cell-sorted device arrays fx, fy, fz, e; scratch holds 3n + 1779 doubles and
// receives (loss, dL/deps, dL/dsigma) at its end.
// lj_multi_force adjoint (gbmd_adjoint_lj.cu): args_dev holds
// lj_multi_adj_args_size() bytes; scratch K n + K * 593 doubles with
// K = 1 + 2 nu (nu unordered type pairs, returned), sums at its end.
int launch_lj_multi_loss_grad(gbmd_context* c, const PairArgs& A, const double* const targets[4], double wF,
                              double wE, void* args_dev, double* scratch, int* nu_out);
size_t lj_multi_adj_args_size();
int launch_lj_loss_grad(gbmd_context* c, const PairArgs& A, const double* const targets[4], double wF, double wE,
                        double* scratch);
// johnson_force and sutton_chen_force kernels, both precisions (gbmd_johnson.cu).
int launch_johnson(gbmd_context* c, const PairArgs& A, int part, bool ev, bool mixed);

// Integer image of the stencil cell of `code` seen from home cell (cx,cy,cz).
__device__ __forceinline__ void image_shift(const Grid& g, int cx, int cy, int cz, uint32_t code,
                                            double& Sx, double& Sy, double& Sz) {
  Sx = (double)image_of(cx, code_dx(code), g.nc[0]) * g.L[0];
  Sy = (double)image_of(cy, code_dy(code), g.nc[1]) * g.L[1];
  Sz = (double)image_of(cz, code_dz(code), g.nc[2]) * g.L[2];
}

__device__ __forceinline__ void unpack_cell(int cp, int& cx, int& cy, int& cz) {
  cx = cp & 1023;
  cy = (cp >> 10) & 1023;
  cz = cp >> 20;
}

// Lane-0 epilogue for atom i: force -> acceleration, stores, fused push.
// fx,fy,fz are the force in FP64; mixed kernels pass accelerations computed in
// FP32 through `amixed` (then fx.. are ignored).
template <bool MIXED>
__device__ __forceinline__ void atom_epilogue(const PairArgs& A, int64_t i, int t, double fx, double fy,
                                              double fz, float afx, float afy, float afz, double epv,
                                              const double* v9) {
  double ax, ay, az;
  if (MIXED) {
    ax = (double)afx;
    ay = (double)afy;
    az = (double)afz;
  } else {
    const double m = A.mass[t];
    ax = fx / m;
    ay = fy / m;
    az = fz / m;
  }
  if (!(isfinite(ax) && isfinite(ay) && isfinite(az))) {
    atomicOr(&A.err[ERRW_FLAGS], GBMD_DEVERR_NONFINITE);
    atomicCAS(&A.err[ERRW_BADATOM], -1, (int)i);
  }
  A.ax[i] = ax;
  A.ay[i] = ay;
  A.az[i] = az;
  if (A.want_energy) A.ep[i] = epv;
  if (A.want_virial && v9) {
#pragma unroll
    for (int q = 0; q < 9; ++q) A.vir[9 * i + q] = v9[q];
  }
  if (A.fuse >= 1) {
    double vx = fma(ax, A.dth, A.vx[i]);
    double vy = fma(ay, A.dth, A.vy[i]);
    double vz = fma(az, A.dth, A.vz[i]);
    if (A.fuse == 2) {
      const double x = A.x[i] + (vx * A.dt + ax * A.dt2h);
      const double y = A.y[i] + (vy * A.dt + ay * A.dt2h);
      const double z = A.z[i] + (vz * A.dt + az * A.dt2h);
      vx = fma(ax, A.dth, vx);
      vy = fma(ay, A.dth, vy);
      vz = fma(az, A.dth, vz);
      A.xo[i] = x;
      A.yo[i] = y;
      A.zo[i] = z;
      if (A.gate) displacement_test(A.gate, A.rref, A.rcap, A.thr2, i, x, y, z);
      int cx, cy, cz;
      unpack_cell(A.cellpack[i], cx, cy, cz);
      A.posf_o[i] = make_float4((float)(x - (double)cx * A.g.h[0] - A.g.lo[0]),
                                (float)(y - (double)cy * A.g.h[1] - A.g.lo[1]),
                                (float)(z - (double)cz * A.g.h[2] - A.g.lo[2]), __int_as_float(t));
      A.posd_o[i] = make_double4_32a(x, y, z, (double)t);
    }
    A.vxo[i] = vx;
    A.vyo[i] = vy;
    A.vzo[i] = vz;
  }
}

}  // namespace gbmd
