// gbmd_pipeline.cu -- one gbmd_run_nve_host step with the host link
// overlapped with the pair passes.
//
// The caller's page-locked r, v, a (caller order) are read over the host link
// in P chunks of the caller order on the input stream; each chunk's first
// half (k_host_first_half, verlet_first_half's formulas) is applied as it
// arrives, and its pushed positions go straight back to the caller's arrays.
// The cell-sorted atoms are cut into S slabs of whole z layers of the cell
// grid, and the caller order into as many chunks of equal atom counts.
// (Chunks cut at the slabs' atom counts, so that chunk k holds slab k's
// atoms, were measured 18 % slower at 4 M atoms.)  Cells are at least
// rcut + skin wide, so a slab's density
// pass (or the single pass of a pair potential) reads the positions of its
// own and the two neighbouring slabs only, and its force pass the densities
// of the same three slabs; the output of a caller chunk (v, a) needs the
// force pass of every slab holding one of its atoms.  A map kernel, run once
// per neighbour-list build, records for every slab the last caller chunk
// holding one of its atoms and for every chunk the set of slabs holding its
// atoms.  From these the host issues each slab's passes on the compute stream
// right after the input chunk that completes their neighbourhood, and each
// chunk's output on the output stream right after the force pass that
// completes it.  When the caller's order follows the cell order along z
// (exaNBody's grids store atoms cell by cell, z slowest) slab s waits for
// chunks s-1..s+1 only and the three streams overlap; any other order gives
// a more serial schedule and the same results: every atom runs the same
// kernels on the same data whatever the pieces.
//
// The force pieces write v(t+dt) into the spare velocity buffer, so that
// v(t+dt/2) stays in place until the step is known to need no rebuild: the
// input pieces test every atom against skin/2 as they push it, and a gated
// copy moves v(t+dt) into place only when none moved that far.  Otherwise
// the caller finishes the step without the pipeline after a rebuild, from
// the pushed state (the caller's arrays are all rewritten then).  The same
// end-of-step kernel applies the next step's first half to the state it
// returns and tests it: when the caller passes that state back unchanged,
// a step that will need a rebuild is known in advance and not pipelined.
#include "gbmd_internal.cuh"

namespace gbmd {

namespace {

constexpr int MAX_SLABS = 64;
// layout of the slab-map scratch (ints)
constexpr int OFF_ZSLAB = 0;      // slab of each z layer (<= 1024 layers)
constexpr int OFF_ZB = 1024;      // first z layer of each slab, S + 1
constexpr int OFF_NEED = 1096;    // per slab: last caller chunk of its atoms (-1: empty)
constexpr int OFF_BEGIN = 1160;   // per slab: first cell-order atom, S + 1
constexpr int OFF_MASK = 1232;    // per chunk: 64-bit slab set (8-byte aligned)
constexpr int OFF_NEXT = 1360;    // the next step will need a rebuild (k_pipe_finish)
constexpr int SCRATCH_INTS = 1536;
constexpr int TRACE_CAP = 4 * MAX_SLABS + 2;

inline int64_t chunk_begin(int64_t n, int P, int k) { return ((int64_t)k * n + P - 1) / P; }

__global__ void k_pipe_map(int64_t n, int P, const int32_t* __restrict__ cellpack, const int32_t* __restrict__ user,
                           const int32_t* __restrict__ zslab, int* __restrict__ need,
                           unsigned long long* __restrict__ mask) {
  __shared__ int sh_need[MAX_SLABS];
  __shared__ unsigned long long sh_mask[MAX_SLABS];
  for (int q = threadIdx.x; q < MAX_SLABS; q += blockDim.x) {
    sh_need[q] = -1;
    sh_mask[q] = 0ull;
  }
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int s = zslab[cellpack[i] >> 20];
    // chunk k holds caller indices [ceil(k n / P), ceil((k+1) n / P))
    const int k = (int)((int64_t)user[i] * P / n);
    atomicMax(&sh_need[s], k);
    atomicOr(&sh_mask[k], 1ull << s);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < MAX_SLABS; q += blockDim.x) {
    if (sh_need[q] >= 0) atomicMax(&need[q], sh_need[q]);
    if (sh_mask[q]) atomicOr(&mask[q], sh_mask[q]);
  }
}

__global__ void k_pipe_bounds(const int32_t* __restrict__ cstart, const int32_t* __restrict__ zb, int S,
                              int64_t nxy, int* __restrict__ begin) {
  const int s = threadIdx.x;
  if (s <= S) begin[s] = cstart[(int64_t)zb[s] * nxy];
}

struct HostOut6 {
  double* a[6];
};

// v(t+dt) and a(t+dt) of caller indices [u0, u1) into the caller's arrays.
__global__ void k_pipe_out(int64_t u0, int64_t u1, const int32_t* __restrict__ inv, const double* __restrict__ v,
                           const double* __restrict__ a, int64_t cap, HostOut6 out) {
  for (int64_t u = u0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < u1;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = inv[u];
    const double q0 = v[i], q1 = v[cap + i], q2 = v[2 * cap + i];
    const double q3 = a[i], q4 = a[cap + i], q5 = a[2 * cap + i];
    out.a[0][u] = q0;
    out.a[1][u] = q1;
    out.a[2][u] = q2;
    out.a[3][u] = q3;
    out.a[4][u] = q4;
    out.a[5][u] = q5;
  }
}

// End of a pipelined step: v(t+dt) into place unless the displacement gate
// is raised, and the next step's first half, as k_host_first_half will
// compute it from the arrays this step returns (same operations), tested
// against skin/2: `next` is set when that step will need a rebuild.
struct FinishArgs {
  int64_t n, cap;
  const double* src;        // v(t+dt), 3 planes of cap
  double* dst;              // the context's v
  const double *x, *y, *z;  // r(t+dt)
  const double *ax, *ay, *az;
  const double* rref;       // positions at the last rebuild, 3 planes of cap
  double h, h2, thr2;
  const int* gate;
  int* next;
};

// One atom per thread and many short blocks (no grid-stride loop): the
// write-back kernels on the high-priority output stream get SM slots as
// these blocks retire.
__global__ void k_pipe_finish(FinishArgs F) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (*F.gate || i >= F.n) return;
  {
    const double vx = F.src[i], vy = F.src[F.cap + i], vz = F.src[2 * F.cap + i];
    F.dst[i] = vx;
    F.dst[F.cap + i] = vy;
    F.dst[2 * F.cap + i] = vz;
    const double x = __dadd_rn(F.x[i], __dadd_rn(__dmul_rn(vx, F.h), __dmul_rn(F.ax[i], F.h2)));
    const double y = __dadd_rn(F.y[i], __dadd_rn(__dmul_rn(vy, F.h), __dmul_rn(F.ay[i], F.h2)));
    const double z = __dadd_rn(F.z[i], __dadd_rn(__dmul_rn(vz, F.h), __dmul_rn(F.az[i], F.h2)));
    const double dx = __dsub_rn(x, F.rref[i]), dy = __dsub_rn(y, F.rref[F.cap + i]),
                 dz = __dsub_rn(z, F.rref[2 * F.cap + i]);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (d2 > F.thr2) *F.next = 1;
  }
}

int ensure_pipe(gbmd_context* c) {
  if (c->pipe_in) return GBMD_OK;
  int least = 0, greatest = 0;
  GBMD_CUDA(c, cudaDeviceGetStreamPriorityRange(&least, &greatest));
  GBMD_CUDA(c, cudaStreamCreateWithPriority(&c->pipe_in, cudaStreamNonBlocking, greatest));
  GBMD_CUDA(c, cudaStreamCreateWithPriority(&c->pipe_out, cudaStreamNonBlocking, greatest));
  GBMD_CUDA(c, cudaStreamCreateWithPriority(&c->pipe_r, cudaStreamNonBlocking, greatest));
  GBMD_CUDA(c, cudaEventCreateWithFlags(&c->pipe_r_done, cudaEventDisableTiming));
  for (int q = 0; q + 1 < PIPE_STREAMS; ++q)
    GBMD_CUDA(c, cudaStreamCreateWithFlags(&c->pipe_cs[q], cudaStreamNonBlocking));
  GBMD_CUDA(c, cudaEventCreateWithFlags(&c->pipe_start, cudaEventDisableTiming));
  GBMD_CUDA(c, cudaEventCreateWithFlags(&c->pipe_out_done, cudaEventDisableTiming));
  for (int k = 0; k < MAX_SLABS; ++k) {
    GBMD_CUDA(c, cudaEventCreateWithFlags(&c->pipe_in_ev[k], cudaEventDisableTiming));
    GBMD_CUDA(c, cudaEventCreateWithFlags(&c->pipe_f_ev[k], cudaEventDisableTiming));
    GBMD_CUDA(c, cudaEventCreateWithFlags(&c->pipe_d_ev[k], cudaEventDisableTiming));
  }
  GBMD_CUDA(c, cudaMalloc(&c->pipe_dev, sizeof(int) * SCRATCH_INTS));
  GBMD_CUDA(c, cudaMallocHost(&c->pipe_host, sizeof(int) * SCRATCH_INTS));
  return GBMD_OK;
}

// First z layer of each slab: equal shares of the nz layers (zb[0] = 0,
// zb[S] = nz, every slab at least one layer).  Thinner slabs where the
// periodic z ring closes (they wait for the last chunk) were measured
// slower: the thicker chunks between them read slower under the concurrent
// passes.
void slab_layers(int nz, int S, int* zb) {
  for (int s = 0; s <= S; ++s) zb[s] = (int)((int64_t)s * nz / S);
}

// The slab map of the current cell order (stream synchronised).
int pipe_schedule(gbmd_context* c, int S) {
  const int P = S;
  const int64_t n = c->n;
  const int nz = c->grid.nc[2];
  const int64_t nxy = (int64_t)c->grid.nc[0] * c->grid.nc[1];
  int* h = c->pipe_host;
  int* d = c->pipe_dev;
  slab_layers(nz, S, h + OFF_ZB);
  if (h[OFF_ZB + S] != nz) return set_error(c, GBMD_ERR_CUDA, "slab layers: %d of %d", h[OFF_ZB + S], nz);
  for (int s = 0; s < S; ++s)
    for (int z = h[OFF_ZB + s]; z < h[OFF_ZB + s + 1]; ++z) h[OFF_ZSLAB + z] = s;
  cudaStream_t m = c->stream;
  GBMD_CUDA(c, cudaMemcpyAsync(d, h, sizeof(int) * OFF_NEED, cudaMemcpyHostToDevice, m));
  GBMD_CUDA(c, cudaMemsetAsync(d + OFF_NEED, 0xff, sizeof(int) * MAX_SLABS, m));
  GBMD_CUDA(c, cudaMemsetAsync(d + OFF_MASK, 0, sizeof(unsigned long long) * MAX_SLABS, m));
  int64_t blocks = (n + 255) / 256;
  if (blocks > 8LL * c->nsm) blocks = 8LL * c->nsm;
  if (blocks < 1) blocks = 1;
  k_pipe_map<<<(unsigned)blocks, 256, 0, m>>>(n, P, c->cellpack, c->USER(), d + OFF_ZSLAB, d + OFF_NEED,
                                              reinterpret_cast<unsigned long long*>(d + OFF_MASK));
  k_pipe_bounds<<<1, 128, 0, m>>>(c->cell_start, d + OFF_ZB, S, nxy, d + OFF_BEGIN);
  GBMD_CUDA(c, cudaMemcpyAsync(h + OFF_NEED, d + OFF_NEED, sizeof(int) * (SCRATCH_INTS - OFF_NEED),
                               cudaMemcpyDeviceToHost, m));
  GBMD_CUDA(c, cudaStreamSynchronize(m));
  const int* need = h + OFF_NEED;
  const unsigned long long* mask = reinterpret_cast<const unsigned long long*>(h + OFF_MASK);
  c->pipe_need.assign(S, 0);
  c->pipe_mask.assign(P, 0);
  c->pipe_begin.assign(S + 1, 0);
  for (int s = 0; s < S; ++s) {
    int m3 = need[s];
    m3 = need[(s + S - 1) % S] > m3 ? need[(s + S - 1) % S] : m3;
    m3 = need[(s + 1) % S] > m3 ? need[(s + 1) % S] : m3;
    c->pipe_need[s] = m3 < 0 ? 0 : m3;
  }
  for (int k = 0; k < P; ++k) c->pipe_mask[k] = mask[k];
  for (int s = 0; s <= S; ++s) c->pipe_begin[s] = h[OFF_BEGIN + s];
  if (c->pipe_begin[0] != 0 || c->pipe_begin[S] != n)
    return set_error(c, GBMD_ERR_CUDA, "slab map: cell ranges [%lld, %lld) for %lld atoms",
                     (long long)c->pipe_begin[0], (long long)c->pipe_begin[S], (long long)n);
  c->pipe_key_builds = c->list_builds;
  c->pipe_key_n = n;
  c->pipe_key_slabs = S;
  return GBMD_OK;
}

}  // namespace

int pipe_slabs_for(const gbmd_context* c) {
  if (c->pipe_slabs == 0 || c->newton3 || c->staged || !c->grid_valid || !c->list_valid || c->n == 0) return 0;
  int S = c->pipe_slabs;
  if (S < 0) {
    // below a quarter million atoms the launches of the pieces cost more
    // than the overlap saves
    if (c->n < (1 << 18)) return 0;
    S = 16;
  }
  if (S > MAX_SLABS) S = MAX_SLABS;
  if (S > c->grid.nc[2]) S = c->grid.nc[2];
  return S >= 4 ? S : 0;
}

namespace {

// One mark of the step's timeline (gbmd_get_host_pipeline_trace): an event
// with timing on `st` after the work issued there so far.
int trace_mark(gbmd_context* c, cudaStream_t st, int kind, int idx) {
  if (!c->pipe_trace) return GBMD_OK;
  if (c->pipe_tr_ev.empty()) {
    c->pipe_tr_ev.assign(TRACE_CAP, nullptr);
    for (auto& e : c->pipe_tr_ev) GBMD_CUDA(c, cudaEventCreate(&e));
    c->pipe_tr_kind.assign(TRACE_CAP, 0);
    c->pipe_tr_idx.assign(TRACE_CAP, 0);
  }
  if (c->pipe_tr_n >= TRACE_CAP) return GBMD_OK;
  GBMD_CUDA(c, cudaEventRecord(c->pipe_tr_ev[c->pipe_tr_n], st));
  c->pipe_tr_kind[c->pipe_tr_n] = kind;
  c->pipe_tr_idx[c->pipe_tr_n] = idx;
  ++c->pipe_tr_n;
  return GBMD_OK;
}

// Launches of launch_forces on another stream of the context.
struct StreamScope {
  gbmd_context* c;
  cudaStream_t saved;
  StreamScope(gbmd_context* ctx, cudaStream_t s) : c(ctx), saved(ctx->stream) { c->stream = s; }
  ~StreamScope() { c->stream = saved; }
};

int pipe_issue(gbmd_context* c, double dt, const double* const host[9], const double* const hdev[9],
               const int32_t* inv, int S) {
  int rc = ensure_pipe(c);
  if (rc) return rc;
  const bool ce = c->pipe_link_mode == 0;
  if (ce && c->pipe_stage_cap < c->cap) {
    if (c->pipe_stage) cudaFree(c->pipe_stage);
    c->pipe_stage = nullptr;
    c->pipe_stage_cap = 0;
    GBMD_CUDA(c, cudaMalloc(&c->pipe_stage, sizeof(double) * 9 * c->cap));
    c->pipe_stage_cap = c->cap;
  }
  const int64_t sc = c->pipe_stage_cap;
  const double* stage[9];
  for (int q = 0; q < 9; ++q) stage[q] = c->pipe_stage + q * sc;
  if (c->pipe_key_builds != c->list_builds || c->pipe_key_n != c->n || c->pipe_key_slabs != S) {
    if ((rc = pipe_schedule(c, S))) return rc;
  }
  const int P = S;
  const int64_t n = c->n;
  // compute pieces go round-robin over PIPE_STREAMS streams (the context's
  // own first), ordered by events only, so that independent pieces run side
  // by side and one piece's last wave overlaps the next pieces
  cudaStream_t m = c->stream;
  cudaStream_t pool[PIPE_STREAMS];
  pool[0] = m;
  for (int q = 1; q < PIPE_STREAMS; ++q) pool[q] = c->pipe_cs[q - 1];
  int next = 0;
  auto take = [&]() { const cudaStream_t st = pool[next]; next = (next + 1) % PIPE_STREAMS; return st; };
  const bool two_pass = c->pot == GBMD_POT_EAM_ALLOY || c->pot == GBMD_POT_EAM_JOHNSON ||
                        c->pot == GBMD_POT_EAM_SUTTON_CHEN;
  double* v_spare = c->vbuf[c->cur_s ^ 1];
  c->pipe_tr_n = 0;
  if ((rc = trace_mark(c, m, GBMD_PIPE_MARK_START, -1))) return rc;
  GBMD_CUDA(c, cudaEventRecord(c->pipe_start, m));
  GBMD_CUDA(c, cudaStreamWaitEvent(c->pipe_in, c->pipe_start, 0));
  GBMD_CUDA(c, cudaStreamWaitEvent(c->pipe_out, c->pipe_start, 0));
  GBMD_CUDA(c, cudaStreamWaitEvent(c->pipe_r, c->pipe_start, 0));
  for (int q = 1; q < PIPE_STREAMS; ++q) GBMD_CUDA(c, cudaStreamWaitEvent(pool[q], c->pipe_start, 0));
  const int dev_blocks = 2 * (c->nsm > 0 ? c->nsm : 1);
  for (int k = 0; k < P; ++k) {
    const int64_t u0 = chunk_begin(n, P, k), u1 = chunk_begin(n, P, k + 1);
    if (ce) {
      // the copy engines carry the chunk into the staging arrays (caller
      // order); the first half then runs from HBM and leaves r' in place,
      // from where another copy engine returns it
      const size_t bytes = sizeof(double) * (size_t)(u1 - u0);
      if (bytes) {
        for (int q = 0; q < 9; ++q)
          GBMD_CUDA(c, cudaMemcpyAsync(const_cast<double*>(stage[q]) + u0, host[q] + u0, bytes,
                                       cudaMemcpyHostToDevice, c->pipe_in));
      }
      launch_host_first_half_range(c, stage, inv, dt, u0, u1, true, dev_blocks, 256, c->pipe_in);
      GBMD_CUDA(c, cudaEventRecord(c->pipe_in_ev[k], c->pipe_in));
      if ((rc = trace_mark(c, c->pipe_in, GBMD_PIPE_MARK_CHUNK_IN, k))) return rc;
      if (bytes) {
        GBMD_CUDA(c, cudaStreamWaitEvent(c->pipe_r, c->pipe_in_ev[k], 0));
        for (int q = 0; q < 3; ++q)
          GBMD_CUDA(c, cudaMemcpyAsync(const_cast<double*>(host[q]) + u0, stage[q] + u0, bytes,
                                       cudaMemcpyDeviceToHost, c->pipe_r));
      }
    } else {
      // kernels read the page-locked arrays over the link and write r' back
      launch_host_first_half_range(c, hdev, inv, dt, u0, u1, true, c->pipe_link_blocks, c->pipe_link_threads,
                                   c->pipe_in);
      GBMD_CUDA(c, cudaEventRecord(c->pipe_in_ev[k], c->pipe_in));
      if ((rc = trace_mark(c, c->pipe_in, GBMD_PIPE_MARK_CHUNK_IN, k))) return rc;
    }
  }
  ForceFlags f;
  f.fuse = FUSE_PUSH2;
  f.sp.dt = dt;
  f.sp.dth = dt * 0.5;
  f.sp.dt2h = dt * dt * 0.5;
  f.v_out = v_spare;
  HostOut6 out;
  for (int q = 0; q < 6; ++q) out.a[q] = const_cast<double*>(ce ? stage[3 + q] : hdev[3 + q]);
  std::vector<char> dens(S, 0), forced(S, 0), outd(P, 0);
  uint64_t forced_mask = 0;
  for (int k = 0; k < P; ++k)
    if (chunk_begin(n, P, k) == chunk_begin(n, P, k + 1)) outd[k] = 1;
  auto piece = [&](int s, int part, cudaStream_t st) -> int {
    ForceFlags g = f;
    g.part = part;
    g.i0 = c->pipe_begin[s];
    g.i1 = c->pipe_begin[s + 1];
    if (g.i1 <= g.i0) return GBMD_OK;
    const StreamScope on(c, st);
    return launch_forces(c, g);
  };
  auto force_piece = [&](int s) -> int {
    const cudaStream_t st = take();
    if (two_pass) {
      for (int d = -1; d <= 1; ++d) GBMD_CUDA(c, cudaStreamWaitEvent(st, c->pipe_d_ev[(s + d + S) % S], 0));
    } else {
      GBMD_CUDA(c, cudaStreamWaitEvent(st, c->pipe_in_ev[c->pipe_need[s]], 0));
    }
    int r = piece(s, 2, st);
    if (r) return r;
    forced[s] = 1;
    forced_mask |= 1ull << s;
    GBMD_CUDA(c, cudaEventRecord(c->pipe_f_ev[s], st));
    if ((r = trace_mark(c, st, GBMD_PIPE_MARK_FORCE, s))) return r;
    bool waited = false;
    for (int k = 0; k < P; ++k) {
      if (outd[k] || (c->pipe_mask[k] & ~forced_mask)) continue;
      if (!waited) GBMD_CUDA(c, cudaStreamWaitEvent(c->pipe_out, c->pipe_f_ev[s], 0));
      waited = true;
      // the chunk's other slabs were issued earlier: on the other compute
      // stream they may still run
      for (int q = 0; q < S; ++q)
        if (q != s && ((c->pipe_mask[k] >> q) & 1)) GBMD_CUDA(c, cudaStreamWaitEvent(c->pipe_out, c->pipe_f_ev[q], 0));
      const int64_t u0 = chunk_begin(n, P, k), u1 = chunk_begin(n, P, k + 1);
      const int T = ce ? 256 : c->pipe_link_threads;
      const int B = ce ? dev_blocks : c->pipe_link_blocks;
      const int64_t need = (u1 - u0 + T - 1) / T;
      k_pipe_out<<<(unsigned)(need < B ? need : B), T, 0, c->pipe_out>>>(u0, u1, inv, v_spare, c->AX(), c->cap, out);
      if (ce) {
        // v, a gathered into the staging arrays in caller order, then out
        const size_t bytes = sizeof(double) * (size_t)(u1 - u0);
        for (int q = 0; q < 6; ++q)
          GBMD_CUDA(c, cudaMemcpyAsync(const_cast<double*>(host[3 + q]) + u0, stage[3 + q] + u0, bytes,
                                       cudaMemcpyDeviceToHost, c->pipe_out));
      }
      outd[k] = 1;
      if ((r = trace_mark(c, c->pipe_out, GBMD_PIPE_MARK_CHUNK_OUT, k))) return r;
    }
    return GBMD_OK;
  };
  for (int k = 0; k < P; ++k) {
    for (int s = 0; s < S; ++s) {
      if (c->pipe_need[s] != k) continue;
      if (two_pass) {
        const cudaStream_t st = take();
        GBMD_CUDA(c, cudaStreamWaitEvent(st, c->pipe_in_ev[k], 0));
        if ((rc = piece(s, 1, st))) return rc;
        GBMD_CUDA(c, cudaEventRecord(c->pipe_d_ev[s], st));
        if ((rc = trace_mark(c, st, GBMD_PIPE_MARK_DENSITY, s))) return rc;
        dens[s] = 1;
      } else if ((rc = force_piece(s))) {
        return rc;
      }
    }
    if (!two_pass) continue;
    for (int s = 0; s < S; ++s)
      if (!forced[s] && dens[(s + S - 1) % S] && dens[s] && dens[(s + 1) % S] && (rc = force_piece(s))) return rc;
  }
  for (int s = 0; s < S; ++s)
    if (!forced[s]) return set_error(c, GBMD_ERR_CUDA, "pipeline: slab %d never issued", s);
  for (int k = 0; k < P; ++k)
    if (!outd[k]) return set_error(c, GBMD_ERR_CUDA, "pipeline: chunk %d never written", k);
  // the gate is final once every chunk has been pushed; v(t+dt) is complete
  // once every force piece has run
  GBMD_CUDA(c, cudaStreamWaitEvent(m, c->pipe_in_ev[P - 1], 0));
  for (int s = 0; s < S; ++s) GBMD_CUDA(c, cudaStreamWaitEvent(m, c->pipe_f_ev[s], 0));
  const int64_t blocks = (n + 255) / 256;
  int* next_flag = c->pipe_dev + OFF_NEXT;
  GBMD_CUDA(c, cudaMemsetAsync(next_flag, 0, sizeof(int), m));
  FinishArgs fa;
  fa.n = n;
  fa.cap = c->cap;
  fa.src = v_spare;
  fa.dst = c->VX();
  fa.x = c->X(); fa.y = c->Y(); fa.z = c->Z();
  fa.ax = c->AX(); fa.ay = c->AY(); fa.az = c->AZ();
  fa.rref = c->rref;
  fa.h = dt * 1.0;
  fa.h2 = fa.h * fa.h * 0.5;
  fa.thr2 = (0.5 * c->skin) * (0.5 * c->skin);
  fa.gate = c->d_err + ERRW_GATE;
  fa.next = next_flag;
  k_pipe_finish<<<(unsigned)blocks, 256, 0, m>>>(fa);
  GBMD_CUDA(c, cudaMemcpyAsync(c->pipe_host + OFF_NEXT, next_flag, sizeof(int), cudaMemcpyDeviceToHost, m));
  GBMD_CUDA(c, cudaEventRecord(c->pipe_out_done, c->pipe_out));
  GBMD_CUDA(c, cudaStreamWaitEvent(m, c->pipe_out_done, 0));
  GBMD_CUDA(c, cudaEventRecord(c->pipe_r_done, c->pipe_r));
  GBMD_CUDA(c, cudaStreamWaitEvent(m, c->pipe_r_done, 0));
  if ((rc = trace_mark(c, m, GBMD_PIPE_MARK_END, -1))) return rc;
  GBMD_CUDA(c, cudaGetLastError());
  GBMD_CUDA(c, cudaStreamSynchronize(m));
  c->pipe_expect_rebuild = c->pipe_host[OFF_NEXT] != 0;
  return GBMD_OK;
}

// Every stream the step issued on has finished (errors ignored): after a
// failed launch the pieces already issued may still read and write the
// caller's arrays, and the caller may free them once the call returns.
void pipe_drain(gbmd_context* c) {
  cudaStreamSynchronize(c->stream);
  if (c->pipe_in) cudaStreamSynchronize(c->pipe_in);
  if (c->pipe_out) cudaStreamSynchronize(c->pipe_out);
  if (c->pipe_r) cudaStreamSynchronize(c->pipe_r);
  for (int q = 0; q + 1 < PIPE_STREAMS; ++q)
    if (c->pipe_cs[q]) cudaStreamSynchronize(c->pipe_cs[q]);
}

}  // namespace

int pipe_step(gbmd_context* c, double dt, const double* const host[9], const double* const hdev[9],
              const int32_t* inv, int S) {
  const int rc = pipe_issue(c, dt, host, hdev, inv, S);
  if (rc) pipe_drain(c);
  return rc;
}

int pipe_trace_read(gbmd_context* c, int cap, double* t_ms, int* kind, int* index, int* count) {
  const int n = c->pipe_tr_n;
  *count = n;
  for (int i = 0; i < n && i < cap; ++i) {
    float ms = 0.f;
    GBMD_CUDA(c, cudaEventElapsedTime(&ms, c->pipe_tr_ev[0], c->pipe_tr_ev[i]));
    if (t_ms) t_ms[i] = ms;
    if (kind) kind[i] = c->pipe_tr_kind[i];
    if (index) index[i] = c->pipe_tr_idx[i];
  }
  return GBMD_OK;
}

void pipe_free(gbmd_context* c) {
  for (auto& e : c->pipe_tr_ev)
    if (e) cudaEventDestroy(e);
  c->pipe_tr_ev.clear();
  if (c->pipe_in) cudaStreamDestroy(c->pipe_in);
  if (c->pipe_out) cudaStreamDestroy(c->pipe_out);
  if (c->pipe_r) cudaStreamDestroy(c->pipe_r);
  if (c->pipe_r_done) cudaEventDestroy(c->pipe_r_done);
  if (c->pipe_stage) cudaFree(c->pipe_stage);
  c->pipe_r = nullptr;
  c->pipe_r_done = nullptr;
  c->pipe_stage = nullptr;
  c->pipe_stage_cap = 0;
  for (int q = 0; q + 1 < PIPE_STREAMS; ++q) {
    if (c->pipe_cs[q]) cudaStreamDestroy(c->pipe_cs[q]);
    c->pipe_cs[q] = nullptr;
  }
  if (c->pipe_start) cudaEventDestroy(c->pipe_start);
  if (c->pipe_out_done) cudaEventDestroy(c->pipe_out_done);
  c->pipe_start = c->pipe_out_done = nullptr;
  for (int k = 0; k < MAX_SLABS; ++k) {
    if (c->pipe_in_ev[k]) cudaEventDestroy(c->pipe_in_ev[k]);
    if (c->pipe_f_ev[k]) cudaEventDestroy(c->pipe_f_ev[k]);
    if (c->pipe_d_ev[k]) cudaEventDestroy(c->pipe_d_ev[k]);
    c->pipe_in_ev[k] = c->pipe_f_ev[k] = c->pipe_d_ev[k] = nullptr;
  }
  if (c->pipe_dev) cudaFree(c->pipe_dev);
  if (c->pipe_host) cudaFreeHost(c->pipe_host);
  c->pipe_in = c->pipe_out = nullptr;
  c->pipe_dev = c->pipe_host = nullptr;
}

}  // namespace gbmd
