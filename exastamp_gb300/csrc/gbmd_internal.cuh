// gbmd_internal.cuh -- shared device/host definitions of the GB300 MD hot path.
//
// Data layout in HBM (all per-atom arrays in cell-sorted order, rebuilt every
// neighbour rebuild):
//   x,y,z / vx,vy,vz / ax,ay,az / ep     FP64 SoA (positions double-buffered)
//   type (u8), id (u64), user (i32: index in the caller's upload order)
//   cellpack (i32): home cell at the last rebuild, cx | cy<<10 | cz<<20
//   posf (float4): FP32 position relative to the home-cell corner, w = type bits
//   posd (double4_32a): FP64 absolute position, w = type bits (FP64 path gathers)
//   nbr (u32): full neighbour list entries j | code<<26, code = (dx+1)|(dy+1)<<2|(dz+1)<<4
//              the stencil offset of j's cell; laid out for T lanes per atom as
//              nbr[(k/T)*(npad*T) + i*T + k%T]
//   nnb (i32): neighbours per atom
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/gbmd.h"

#define GBMD_MAX_TYPES 8
#define GBMD_IDX_BITS 26
#define GBMD_IDX_MASK ((1u << GBMD_IDX_BITS) - 1u)
#define GBMD_MAX_ATOMS (1ll << GBMD_IDX_BITS)

// device error word layout (int[ERRW_WORDS])
enum {
  ERRW_FLAGS = 0,     // bitmask of GBMD_DEVERR_*
  ERRW_MAXNB = 1,     // largest neighbour count seen by the last list build
  ERRW_LOST = 2,      // atoms found outside the box after the wrap
  ERRW_STEP = 3,      // step index of the first error (-1 none)
  ERRW_BADATOM = 4,   // first offending atom (sorted index)
  ERRW_REBUILDS = 5,  // displacement-triggered rebuilds run on the device
  ERRW_GATE = 6,      // this step's displacement trigger (gate of the rebuild chain)
  ERRW_DISPL = 7,     // displacement check of gbmd_upload_positions
  ERRW_OUTER = 8,     // two-level list: some atom moved more than half the outer buffer
  ERRW_OUTER_BUILDS = 9,  // outer lists built on the device (graph replays, gated chains)
  ERRW_WORDS = 16,
};
enum {
  GBMD_DEVERR_NBR_OVERFLOW = 1,
  GBMD_DEVERR_LOST_ATOM = 2,
  GBMD_DEVERR_NONFINITE = 4,
  GBMD_DEVERR_TABLE_RANGE = 8,
  GBMD_DEVERR_RANGE = 16,     // a Newton-3 contribution beyond the fixed-point range
};

namespace gbmd {

// Per-type-pair LJ coefficients (both precisions carried; kernels pick one).
struct LJPair {
  double eps, sig, rc, ecut;     // FP64 reference values
  double rc2;                    // rc*rc
  float sig2f, eps24f, eps4f, ecutf, rc2f, rc2lo, rc2hi, pad;
};

struct LJTable {
  int ntypes;
  double rcut_max, rcut_max2;
  LJPair p[GBMD_MAX_TYPES * GBMD_MAX_TYPES];
};

// eam_alloy tables: FP64 copies in the reference's 8-double knot layout and
// FP32 value-coefficient float4 copies (c3,c4,c5,c6) for the mixed path.
struct EamDev {
  int nel, nr, nrho, npairs;
  double rdr, rdrho, rhomax, conv_z2r, conv_frho, rcut, rcut2;
  const double* frho;  // nel x (nrho+1) x 8
  const double* rhor;  // nel x (nr+1) x 8
  const double* z2r;   // npairs x (nr+1) x 8
  const float4* frho4; // nel x (nrho+1)      F * conv_frho
  const float4* rhor4; // nel x (nr+1)
  const float4* z2r4;  // npairs x (nr+1)      z2r * conv_z2r
  const float4* rhod4; // nel x (nr+1)         rho' coefficients (3c3, 2c4, c5) / dr
  const float4* fz8;   // one element: (nr+1) x {rhod4, z2r4}, 32-byte aligned knots
  float rdrf, rdrhof, rhomaxf, rc2f, rc2lo, rc2hi;
};

// johnson_force parameters (EamJohnsonParameters order) in FP64 and FP32.
struct JohnsonDev {
  double re, fe, rhoe, alpha, beta, A, B, kappa, lambda, Fn0, Fn1, Fn2, Fn3, F0, F1, F2, F3, Fo, eta;
  double rcut, rcut2;
  float ref, ire_f, fef, alphaf, betaf, Af, Bf, kappaf, lambdaf;
  float rc2lo, rc2hi;
};

// sutton_chen_force parameters (EamSuttonChenParameters order) in FP64 and FP32.
struct SuttonChenDev {
  double c, epsilon, a0, n, m;
  double rcut, rcut2;
  float cf, epsf, a0f, nf, mf;
  float rc2lo, rc2hi;
};

struct Grid {
  int nc[3];
  double h[3], L[3], lo[3];
  float hf[3];
  int64_t ncells;
};

struct StepParams {
  double dt, dth, dt2h;     // dt, dt/2, dt*dt/2
  int64_t step;             // step index (for error records)
};

}  // namespace gbmd

struct gbmd_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  // copy streams for host<->device staging (created lazily), forked from and
  // joined back into `stream` with events
  int nsm = 0;                  // SMs of the device
  bool capturing = false;       // a gbmd_run_nve graph is being captured
  bool full_chain_grids = false;  // gated rebuild chain captured into a conditional body
  cudaStream_t cond_stream = nullptr;  // captures the conditional rebuild body
  double* stage_r = nullptr;    // 3 x cap: r in caller order, copied out during a force pass
  double* host_r_out[3] = {nullptr, nullptr, nullptr};  // gbmd_run_nve_host's r arrays
  bool r_copy_pending = false;  // copy_join[0] marks the end of that copy
  cudaStream_t copy_stream[2] = {nullptr, nullptr};
  cudaEvent_t copy_fork = nullptr, copy_join[2] = {nullptr, nullptr};
  bool own_stream = false;
  std::string err;

  // box
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  bool box_set = false;

  // species
  int ntypes = 0;
  double mass[GBMD_MAX_TYPES] = {0};

  // atoms (device, cell-sorted).  Each FP64 vector block holds x|y|z (3*cap);
  // index 0/1 double-buffer them: sorts gather into the other buffer and the
  // fused force+push kernel writes new positions there, so no kernel ever
  // reads a neighbour position that another thread is updating.
  int64_t n = 0, cap = 0;
  double* rbuf[2] = {nullptr, nullptr};
  double* vbuf[2] = {nullptr, nullptr};
  double* abuf[2] = {nullptr, nullptr};
  float4* posf[2] = {nullptr, nullptr};   // FP32 home-cell-relative coords, w = type bits
  double4_32a* posd[2] = {nullptr, nullptr};  // FP64 absolute coords, w = type bits
  uint8_t* typeb[2] = {nullptr, nullptr};
  uint64_t* idb[2] = {nullptr, nullptr};
  int32_t* userb[2] = {nullptr, nullptr};
  int cur = 0;                            // which of r/posf/posd is current
  int cur_s = 0;                          // which of v/a/type/id/user is current
  double* ep = nullptr;
  double* epd = nullptr;                  // FP64 EAM embedding energies (density pass -> force pass)
  double* vir = nullptr;                  // 9n, allocated when virials are requested
  int32_t* cellpack = nullptr;            // home cell at the last rebuild
  int32_t* cell_of = nullptr;             // scratch: linear cell per atom (pre-sort order)
  int32_t* order = nullptr;               // scratch: atoms scattered by cell
  int32_t* src = nullptr;                 // scratch: new position -> old position
  float* fpf = nullptr;                   // EAM F'(rho) FP32 (mixed)
  float4* pfp = nullptr;                  // single-element EAM: FP32 position with F'(rho) in w (mixed)
  double* adj_scratch = nullptr;          // LJ adjoint: targets + per-atom terms (lazily allocated)
  int64_t adj_cap = 0;
  double* fpd = nullptr;                  // EAM rho_dEmb FP64
  double* stage = nullptr;                // 9n staging for host<->device reorders
  double* rref = nullptr;                 // 3n positions at the last rebuild (displacement trigger)
  float* epf = nullptr;                   // EAM embedding energy FP32 (mixed energy steps)

  double* X() const { return rbuf[cur]; }
  double* Y() const { return rbuf[cur] + cap; }
  double* Z() const { return rbuf[cur] + 2 * cap; }
  double* VX() const { return vbuf[cur_s]; }
  double* VY() const { return vbuf[cur_s] + cap; }
  double* VZ() const { return vbuf[cur_s] + 2 * cap; }
  double* AX() const { return abuf[cur_s]; }
  double* AY() const { return abuf[cur_s] + cap; }
  double* AZ() const { return abuf[cur_s] + 2 * cap; }
  uint8_t* TYPE() const { return typeb[cur_s]; }
  uint64_t* ID() const { return idb[cur_s]; }
  int32_t* USER() const { return userb[cur_s]; }
  float4* POSF() const { return posf[cur]; }
  double4_32a* POSD() const { return posd[cur]; }

  // cell grid + neighbour list
  gbmd::Grid grid{};
  bool grid_valid = false;
  int32_t *cell_start = nullptr, *cell_fill = nullptr;
  int64_t cells_cap = 0;
  int32_t* scan_tmp = nullptr;
  int64_t scan_cap = 0;
  uint32_t* nbr = nullptr;
  int32_t* nnb = nullptr;
  int64_t nbr_cap = 0;          // entries allocated
  int maxnb = 0;                // per-atom capacity (multiple of tpa * vec)
  int tpa = 1;                  // lanes per atom (autotuned; default = the GB300 optimum)
  int vec = 4;                  // list entries per lane per load (1 or 4, mixed kernels; autotuned)
  bool staged = false;          // 1 lane x 4 entries: neighbour positions from shared memory
  bool fused_trigger = false;   // run_nve with the displacement trigger: kernels that move atoms test them
  bool first_half_done = false; // gbmd_run_nve_host pushed the first half while reading the state in
  bool newton3 = false;         // half list (j > i in cell order) + scattered reaction forces (LJ, mixed)
  long long* h3acc = nullptr;   // Newton-3 fixed-point accumulators, 10 planes of cap: f (3), ep, virial (6)
  double eam_fix_bound[4] = {1.0, 1.0, 1.0, 1.0};  // Newton-3 eam_alloy bounds: rho, force, energy, virial
  bool eam_fix_ok = false;      // eam_fix_bound is that of the current tables
  int block = 256;              // threads per block of the pair / force kernels (autotuned)
  int block_rho = 128;          // threads per block of the EAM density kernels (autotuned; 0 = block)
  double skin = 0.0, rlist = 0.0;
  bool list_valid = false;
  int64_t list_builds = 0;
  // two-level list (gbmd_set_list_buffer): an outer list of radius rlist +
  // list_buffer, built with the sort into cells, and the list the pair
  // kernels read (radius rlist) filtered from it at every rebuild while no
  // atom has moved more than list_buffer / 2 since the outer build
  double list_buffer = 0.0;
  uint32_t* nbr_out = nullptr;
  int32_t* nnb_out = nullptr;
  int64_t nbr_out_cap = 0;
  int maxnb_out = 0;
  double* rout = nullptr;       // 3 planes of cap: positions at the outer build
  int64_t outer_cap = 0;        // atoms rout and nnb_out hold
  bool outer_valid = false;
  int64_t outer_builds = 0;
  int64_t npad = 0;

  // potential
  int pot = GBMD_POT_NONE;
  gbmd::JohnsonDev ej{};
  gbmd::SuttonChenDev esc{};
  gbmd::LJTable lj{};
  gbmd::EamDev eam{};
  double* eam_d = nullptr;      // device FP64 tables (one allocation)
  float4* eam_f = nullptr;      // device FP32 tables (one allocation)
  gbmd::LJPair* lj_tab_d = nullptr;  // device copy of the type-pair LJ table
  std::vector<double> eam_host_frho, eam_host_rhor, eam_host_z2r;  // spline copies for the adjoint

  int precision = GBMD_PRECISION_FP64;

  // errors + reductions
  int* d_err = nullptr;
  int* h_err = nullptr;         // pinned
  double* d_part = nullptr;     // per-block thermo partials
  int64_t part_cap = 0;
  double* d_thermo = nullptr;   // 27
  double* h_thermo = nullptr;   // pinned 27
  double* d_rows = nullptr;     // thermo rows of a run (27 per row)
  int64_t rows_cap = 0;

  int64_t step = 0;
  int64_t forces_valid_step = -1;
  int64_t energy_step = -1;      // step whose per-atom energies and virials ep, vir hold (run_nve thermo steps)
  int64_t rho_valid_step = -1;   // step of the last standalone EAM density pass (-1: none valid)
  int64_t rho_builds = -1;       // list builds at that pass
  bool rho_ev = false;           // that pass stored the embedding energies

  // CUDA graphs of a chunk of steps: [0] a chunk followed by more steps,
  // [1] the chunk that ends a run (its last step keeps full velocities);
  // one per parity of the buffer indices the chunk starts from (cur, cur_s)
  struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    int rebuild_every = 0, chunk = 0, thermo_end = 0;
    double dt = 0.0;
    int cur0 = -1, cur_s0 = -1;  // buffer indices the graph starts from (positions; v/a/type/id/user)
    int swaps = 0, swaps_s = 0;  // parity of the swaps inside it
    int64_t key_n = -1;
    int key_maxnb = -1, key_tpa = -1, key_block = -1, key_prec = -1, key_vec = -1, key_staged = -1,
        key_block_rho = -1;
  };
  GraphSlot graphs[2][4];
  GraphSlot& graph_slot(int tail) { return graphs[tail][cur | (cur_s << 1)]; }

  // host-link pipeline of one gbmd_run_nve_host step (gbmd_pipeline.cu)
  int pipe_slabs = -1;          // -1 automatic, 0 off, >= 4: slabs (and caller-order chunks) per step
  int pipe_link_mode = 1;       // 0: copy engines + staging in HBM; 1: kernels on the page-locked arrays
  int pipe_link_blocks = 40, pipe_link_threads = 512;  // grid-stride shape of those kernels (mode 1)
  double* pipe_stage = nullptr; // 9 x pipe_stage_cap: r, v, a of the step in caller order (mode 0)
  int64_t pipe_stage_cap = 0;
  cudaStream_t pipe_in = nullptr, pipe_out = nullptr, pipe_r = nullptr;
  cudaEvent_t pipe_r_done = nullptr;
  cudaStream_t pipe_cs[3] = {nullptr, nullptr, nullptr};  // compute streams besides the context's
  cudaEvent_t pipe_start = nullptr, pipe_out_done = nullptr;
  cudaEvent_t pipe_in_ev[64] = {}, pipe_f_ev[64] = {}, pipe_d_ev[64] = {};
  int* pipe_dev = nullptr;      // device scratch of the slab map
  int* pipe_host = nullptr;     // its page-locked mirror
  int64_t pipe_key_builds = -1, pipe_key_n = -1;
  int pipe_key_slabs = 0;
  std::vector<int> pipe_need;          // per slab: last caller chunk holding an atom of the slab or a neighbour slab
  std::vector<uint64_t> pipe_mask;     // per caller chunk: slabs holding its atoms
  std::vector<int64_t> pipe_begin;     // slab s = cell-order atoms [begin[s], begin[s+1])
  int64_t pipe_steps = 0;              // steps that stood as pipelined (no rebuild due)
  bool pipe_expect_rebuild = false;    // the last pipelined step predicts a rebuild in the next one
  int64_t pipe_redone = 0;             // pipelined steps discarded for a rebuild nobody predicted
  // timeline of the last pipelined step (gbmd_set_host_pipeline_trace)
  bool pipe_trace = false;
  std::vector<cudaEvent_t> pipe_tr_ev;
  std::vector<int> pipe_tr_kind, pipe_tr_idx;
  int pipe_tr_n = 0;
};

// ---------------------------------------------------------------------------
// internal launch helpers (implemented in the .cu files)
// ---------------------------------------------------------------------------
namespace gbmd {

int set_error(gbmd_context* c, int code, const char* fmt, ...);
// eam_alloy.cpp L29-58: knot values f[1..n] -> (n+1) x 8 spline coefficients
void spline7(int n, double delta, const double* f, double* s);
int check_cuda(gbmd_context* c, cudaError_t e, const char* what);
int ensure_atom_capacity(gbmd_context* c, int64_t n);
int sync_error_word(gbmd_context* c);  // copies device error word, returns status

// neighbours (gbmd_neighbors.cu)
int grid_dims(const double lo[3], const double hi[3], double R, int nc[3]);
// gate: device word; non-null makes every kernel of the chain return at once
// while it holds 0, and keeps the buffer indices unchanged (see gbmd_neighbors.cu)
// A full list build: wrap, sort into cells and build the list the pair
// kernels read (with a list buffer set: the outer list, then the filter).
int rebuild(gbmd_context* c, bool check_capacity, const int* gate = nullptr);
// With a list buffer set and an outer list in place: the outer list is
// rebuilt (with the sort) only when some atom moved more than half the
// buffer since it was built, and the list is filtered from it.  `gate`
// (device word) gates the whole rebuild as in rebuild(); without a gate the
// decision is read back on the host, or put in a conditional graph node
// while the stream is being captured.
int rebuild_two_level(gbmd_context* c, bool check_capacity, const int* gate = nullptr);
bool two_level(const gbmd_context* c);
void free_outer(gbmd_context* c);
// a device-side conditional graph node around `body`, opened when *gate != 0
// (the stream must be capturing; body issues on c->stream)
int capture_if(gbmd_context* c, const int* gate, int (*body)(gbmd_context*, const int*));
void launch_posf(gbmd_context* c, const int* gate = nullptr);
// blocks for a rebuild-chain kernel over `items` (per_block per block): all
// of them ungated, at most per_sm per SM when gated (grid-stride kernels)
unsigned chain_blocks(const gbmd_context* c, int64_t items, int per_block, const int* gate, int per_sm);
int export_pairs(gbmd_context* c, int64_t cap, uint64_t* id_i, uint64_t* id_j, int8_t* img, int64_t* count);

// forces (gbmd_forces.cu)
enum FuseMode { FUSE_NONE = 0, FUSE_PUSH2 = 1, FUSE_PUSH2_PUSH1 = 2 };
struct ForceFlags {
  bool energy = false, virial = false, thermo = false;
  int fuse = FUSE_NONE;
  int part = 0;   // 0 all kernels, 1 EAM density pass only, 2 final pair kernel only
  StepParams sp{};
  int64_t i0 = 0, i1 = -1;    // cell-order atom range [i0, i1) (i1 < 0: all atoms)
  double* v_out = nullptr;    // fused halves write v here (3 planes of cap) instead of in place
};
int launch_forces(gbmd_context* c, const ForceFlags& f);

// host-link pipeline (gbmd_pipeline.cu): compute streams (the context's own
// and pipe_cs); slabs to use for this context now
// (0: the step goes the unpipelined way); one pipelined step, all streams
// synchronised at return (the displacement gate is left in the error word)
constexpr int PIPE_STREAMS = 4;
int pipe_slabs_for(const gbmd_context* c);
// host: the caller's arrays; hdev: their device addresses (page-locked)
int pipe_step(gbmd_context* c, double dt, const double* const host[9], const double* const hdev[9],
              const int32_t* inv, int slabs);
void pipe_free(gbmd_context* c);
// the last pipelined step's timeline marks (ms since its start)
int pipe_trace_read(gbmd_context* c, int cap, double* t_ms, int* kind, int* index, int* count);

// integration (gbmd_integrate.cu)
void launch_push_f_v_r(gbmd_context* c, double dt, double dt_scale);
void launch_push_f_v(gbmd_context* c, double dt, double dt_scale);
void launch_push_min(gbmd_context* c, double dt, double dt_scale, double tolF);
void launch_first_half(gbmd_context* c, double dt);
void launch_first_half_swap(gbmd_context* c, double dt);
// host: device addresses of page-locked caller arrays r, v, a (caller order);
// inv: caller index -> cell-sorted index
void launch_host_first_half(gbmd_context* c, const double* const host[9], const int32_t* inv, double dt);
// the same over caller indices [u0, u1) on `stream` with at most `blocks`
// blocks; write_back: the pushed positions also go to host[0..2]
void launch_host_first_half_range(gbmd_context* c, const double* const host[9], const int32_t* inv, double dt,
                                  int64_t u0, int64_t u1, bool write_back, int blocks, int threads,
                                  cudaStream_t stream);
void launch_thermo(gbmd_context* c, bool with_virial);
void launch_thermo_raw(int64_t n, const double* vx, const double* vy, const double* vz, const double* ep,
                       const double* vir, const uint8_t* type, const double* mass, int ntypes, double* part,
                       double* out, cudaStream_t s);
// The thermodynamic reduction runs TH_THREADS-thread blocks, at most
// TH_MAX_BLOCKS of them (about eight per SM): a fixed cap, so the summation
// order depends on the atom count only, and the partial buffer of any call
// holds at most TH_MAX_BLOCKS x 26 doubles.
constexpr int TH_THREADS = 256;
constexpr int TH_MAX_BLOCKS = 1184;
int thermo_blocks(int64_t n);

}  // namespace gbmd

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
#define GBMD_CUDA(c, call)                                  \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return gbmd::check_cuda((c), e_, #call); \
  } while (0)

// particle_displ_over for one atom at its new position: raise the gate when
// it moved more than sqrt(thr2) since the last rebuild (|dr|^2 summed x, y, z
// without contraction, as the standalone test kernel does).
__device__ __forceinline__ void displacement_test(int* gate, const double* __restrict__ rref, int64_t cap,
                                                  double thr2, int64_t i, double x, double y, double z) {
  const double dx = __dsub_rn(x, rref[i]), dy = __dsub_rn(y, rref[cap + i]), dz = __dsub_rn(z, rref[2 * cap + i]);
  const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  if (d2 > thr2) *gate = 1;
}

__device__ __forceinline__ void kahan_add(float& s, float& comp, float v) {
  const float y = v - comp;
  const float t = s + y;
  comp = (t - s) - y;
  s = t;
}

// Combine two compensated sums (s1 - c1) + (s2 - c2) with an exact two-sum.
__device__ __forceinline__ void kahan_merge(float& s, float& comp, float s2, float c2) {
  const float t = s + s2;
  const float bb = t - s;
  const float e = (s - (t - bb)) + (s2 - bb);
  comp = comp + c2 - e;
  s = t;
}

template <int T>
__device__ __forceinline__ void group_reduce_kahan(float& s, float& c) {
#pragma unroll
  for (int off = T / 2; off > 0; off >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, s, off);
    const float c2 = __shfl_xor_sync(0xffffffffu, c, off);
    kahan_merge(s, c, s2, c2);
  }
}

template <int T>
__device__ __forceinline__ double group_reduce_d(double v) {
#pragma unroll
  for (int off = T / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// stencil code -> offsets in {-1,0,1}
__device__ __forceinline__ int code_dx(uint32_t code) { return int(code & 3u) - 1; }
__device__ __forceinline__ int code_dy(uint32_t code) { return int((code >> 2) & 3u) - 1; }
__device__ __forceinline__ int code_dz(uint32_t code) { return int((code >> 4) & 3u) - 1; }

__device__ __forceinline__ float code_shift(uint32_t bits2, float h) {
  // bits2 in {0,1,2} -> -h, 0, +h
  return bits2 == 0u ? -h : (bits2 == 2u ? h : 0.0f);
}

__device__ __forceinline__ int image_of(int c, int d, int nc) {
  const int cj = c + d;
  return cj < 0 ? -1 : (cj >= nc ? 1 : 0);
}

// Exact FP64 d2 of (i, image n of j): ((xj + n*L) - xi)^2 summed left to right,
// no contraction -- the rounding of the list builder and of the oracle.
__device__ __forceinline__ double exact_d2(double xi, double yi, double zi, double xj, double yj,
                                           double zj, double sx, double sy, double sz, double& dx,
                                           double& dy, double& dz) {
  dx = __dsub_rn(__dadd_rn(xj, sx), xi);
  dy = __dsub_rn(__dadd_rn(yj, sy), yi);
  dz = __dsub_rn(__dadd_rn(zj, sz), zi);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Words per list row of one atom: the T lanes of an atom each read `vec`
// adjacent entries, so row r of atom i holds entries r*W .. r*W+W-1 at
// nbr[r * npad * W + i * W + ...].
inline int list_width(const gbmd_context* c) { return c->tpa * c->vec; }

__device__ __forceinline__ size_t nbr_slot(int64_t i, int k, int T, int64_t stride) {
  return (size_t)(k / T) * (size_t)stride + (size_t)i * T + (k % T);
}
