// Persistent batched sweeps: every sweep of a call, for every replica of a
// batch, in one launch of thread-block clusters (hsmc_batch_set_schedule,
// schedule 1).  The unit replicated is the reference's NVT run, hs_nvt /
// sweep_nvt (src/nvt.c:30-103, 201-209), advanced by the checkerboard sweep.
//
// The replicas of one cell capacity are packed on the host into bundles of
// about `tile` active cells per lane group of a cluster (a replica larger
// than that is a bundle of its own), largest first.  Cluster k takes bundle k
// and runs all the call's sweeps of its replicas: per sweep the cell build of
// every particle of the bundle, then the eight colour passes over the
// bundle's active cells, separated by the cluster's hardware barrier
// (barrier.cluster: release/acquire at cluster scope; every thread reaches
// every barrier, so no wait can be left unmet).  Bundles share nothing, so
// clusters never wait on one another, and a cluster that finishes early
// makes room for the next bundle.  Data written during the launch (counts,
// slots, positions) is read through L2 only.
//
// Each replica draws the same Philox counters as a single system of the same
// seed would with the replica's batch index, and the cell work is the same
// move_cell, so the chain is the flat schedule's, replica for replica.
#include <cooperative_groups.h>

#include "move_cell.cuh"

namespace cg = cooperative_groups;

namespace hsmc {

constexpr int kBundleMaxReps = 32;

// A sweep's shift and colour order of one replica (colour of pass k in
// nibble k), and the counters a block adds up for it.
struct alignas(16) RepParams {
  float sh[3];
  uint32_t perm;
};
struct RepTally {
  unsigned acc, rej_o, rej_b, rechecks;
};

struct BundleJob {
  const SysPtrs *reps;  // the class's replicas, in bundle order
  const int *rep_ids;   // their index in the batch (enters the random counters)
  const int *nstart;    // prefix sums over them of particles,
  const int *gstart;    // of active cells (an eighth of the grid)
  const int *cstart;    // and of allocated cells
  const int *bundle;    // bundle b = replicas [bundle[b], bundle[b + 1])
  int n_sweeps;
};

template <int G, int CAP>
constexpr size_t persist_smem() {
  return PassSmem<G, CAP>::bytes + kBundleMaxReps * (sizeof(RepParams) + sizeof(RepTally));
}

__device__ __forceinline__ PassEnv persist_env(const SysPtrs &p, uint32_t rep, int layout, const RepParams &rp,
                                               unsigned long long seq) {
  PassEnv e;
  const Box *bx = p.box;  // fixed for the launch (NVT)
  e.cnt = cnt_of(p, layout);
  e.slot = slot_of(p, layout);
  e.pos = p.pos;
  e.st = p.st;
  e.dr = p.st->dr_max;
  e.seed = p.st->seed;
  e.seq = seq;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    e.len[d] = bx->len[d];
    e.half[d] = bx->half[d];
    e.L32[d] = bx->len32[d];
    e.iw[d] = bx->inv_w32[d];
    e.sh[d] = rp.sh[d];
    e.nc[d] = bx->nc[d];
  }
  e.lo = 1.0f - bx->band;
  e.hi = 1.0f + bx->band;
  e.frozen = p.st->frozen;
  e.signal = false;
  e.rep = rep;
  e.trace = nullptr;
  e.trace_cap = 0;
  return e;
}

template <int G, int CAP>
__global__ void __launch_bounds__(128, PassSmem<G, CAP>::min_blocks) k_batch_persist(BundleJob job) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PassSm m = pass_smem_ptrs<G, CAP>(smem_raw);
  RepParams *rp = reinterpret_cast<RepParams *>(smem_raw + PassSmem<G, CAP>::bytes);
  RepTally *rt = reinterpret_cast<RepTally *>(rp + kBundleMaxReps);
  cg::cluster_group cluster = cg::this_cluster();
  const int cb = (int)cluster.num_blocks();
  const int b = (int)(blockIdx.x / cb);  // this cluster's bundle
  const int tid = (int)threadIdx.x;
  const int lane = tid % G, gl = tid / G, col0 = tid - lane;
  const int gbase = (tid & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int ct = (int)cluster.block_rank() * 128 + tid;  // thread within the cluster
  const int nct = cb * 128;
  const int cgroup = ct / G, ncgroups = nct / G;

  const int r0 = job.bundle[b], nr = job.bundle[b + 1] - r0;
  const int n0 = job.nstart[r0], tot_n = job.nstart[r0 + nr] - n0;
  const int g0 = job.gstart[r0], tot_g = job.gstart[r0 + nr] - g0;
  const int c0 = job.cstart[r0], tot_c = job.cstart[r0 + nr] - c0;
  if (tid < nr) rt[tid] = RepTally{0u, 0u, 0u, 0u};
  const unsigned long long base = tid < nr ? job.reps[r0 + tid].st->sweep_base : 0ull;

  for (int s = 0; s < job.n_sweeps; s++) {
    // the sweep's shift and colour order of each replica (what the cell
    // build of the flat schedule publishes for it)
    if (tid < nr) {
      const SysPtrs &p = job.reps[r0 + tid];
      const uint32_t rep = (uint32_t)job.rep_ids[r0 + tid];
      const float w[3] = {p.box->w32[0], p.box->w32[1], p.box->w32[2]};
      RepParams q;
      sweep_shift(p.st->seed, rep, base + (unsigned long long)s, w, q.sh);
      int perm[8];
      sweep_perm(p.st->seed, rep, base + (unsigned long long)s, perm);
      q.perm = 0u;
      for (int k = 0; k < 8; k++) q.perm |= (uint32_t)perm[k] << (4 * k);
      rp[tid] = q;
    }
    __syncthreads();
    // every replica of a batch has made the same number of sweeps
    const unsigned long long sweep = job.reps[r0].st->sweep_base + (unsigned long long)s;
    const int layout = (int)(sweep & 1ull);

    // (1) cell build of every particle of the bundle (k_build, sweep.cu)
    for (int i = ct; i < tot_n; i += nct) {
      const int lr = find_rep(job.nstart + r0, nr, i + n0);
      const SysPtrs &p = job.reps[r0 + lr];
      const int li = i + n0 - job.nstart[r0 + lr];
      const Box *bx = p.box;
      const double2 a = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)li));
      const double2 c2 = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)li + 2));
      int cx, cy, cz;
      float tx, ty, tz;
      axis_cell(__double2float_rn(a.y), rp[lr].sh[0], bx->len32[0], bx->inv_w32[0], bx->nc[0], cx, tx);
      axis_cell(__double2float_rn(c2.x), rp[lr].sh[1], bx->len32[1], bx->inv_w32[1], bx->nc[1], cy, ty);
      axis_cell(__double2float_rn(c2.y), rp[lr].sh[2], bx->len32[2], bx->inv_w32[2], bx->nc[2], cz, tz);
      const int c = cx + bx->nc[0] * (cy + bx->nc[1] * cz);
      const int k = atomicAdd(cnt_of(p, layout) + c, 1);
      if (k < p.cap) {
        slot_of(p, layout)[(size_t)c * p.cap + k] = Slot{tx, ty, tz, li};
      } else {
        atomicOr(&p.st->status, ST_CELL_OVERFLOW);
      }
    }
    cluster.sync();

    // (2) the eight colour passes
    for (int pass = 0; pass < 8; pass++) {
      if (pass == 0) {  // the other layout's counts, for the next sweep's build
        for (int i = ct; i < tot_c; i += nct) {
          const int lr = find_rep(job.cstart + r0, nr, i + c0);
          const SysPtrs &p = job.reps[r0 + lr];
          cnt_of(p, layout ^ 1)[i + c0 - job.cstart[r0 + lr]] = 0;
        }
      }
      // the warp's groups take their cells in step (move_pass.cu)
      for (int it = cgroup; __any_sync(0xffffffffu, it < tot_g); it += ncgroups) {
        __syncwarp();  // the previous cell's records are no longer read
        if (it >= tot_g) continue;
        const int lr = find_rep(job.gstart + r0, nr, it + g0);
        const SysPtrs &p = job.reps[r0 + lr];
        const RepParams q = rp[lr];
        const PassEnv e =
            persist_env(p, (uint32_t)job.rep_ids[r0 + lr], layout, q, sweep * 8ull + (unsigned long long)pass);
        const int colour = (int)((q.perm >> (4 * pass)) & 7u);
        const int hx = e.nc[0] >> 1, hy = e.nc[1] >> 1;
        const int ac = it + g0 - job.gstart[r0 + lr];
        const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
        PassTally t;
        bool no_wait = false;
        move_cell<G, CAP, false, true>(e, m, tid, lane, gl, col0, gmask, 2 * ax + (colour & 1),
                                       2 * ay + ((colour >> 1) & 1), 2 * az + ((colour >> 2) & 1), t, no_wait);
        if (t.acc) atomicAdd(&rt[lr].acc, t.acc);
        if (t.rej_o) atomicAdd(&rt[lr].rej_o, t.rej_o);
        if (t.rej_b) atomicAdd(&rt[lr].rej_b, t.rej_b);
        if (t.rechecks) atomicAdd(&rt[lr].rechecks, t.rechecks);
      }
      cluster.sync();
    }
  }

  // the block's counters, and the sweep index advanced once per replica
  if (tid < nr) {
    DevState *ws = job.reps[r0 + tid].st;
    if (rt[tid].acc) atomicAdd(&ws->acc, (unsigned long long)rt[tid].acc);
    if (rt[tid].rej_o) atomicAdd(&ws->rej_overlap, (unsigned long long)rt[tid].rej_o);
    if (rt[tid].rej_b) atomicAdd(&ws->rej_boundary, (unsigned long long)rt[tid].rej_b);
    if (rt[tid].rechecks) atomicAdd(&ws->rechecks, (unsigned long long)rt[tid].rechecks);
  }
  cluster.sync();  // every block has read sweep_base for its last sweep
  if (cluster.block_rank() == 0 && tid < nr) {
    // the last sweep's layout is the current one: publish its parameters as
    // the cell build does, for the observables and the other schedules
    DevState *ws = job.reps[r0 + tid].st;
    const RepParams q = rp[tid];
    ws->params.sweep = base + (unsigned long long)job.n_sweeps - 1ull;
    for (int d = 0; d < 3; d++) ws->params.shift32[d] = q.sh[d];
    for (int k = 0; k < 8; k++) ws->params.perm[k] = (int)((q.perm >> (4 * k)) & 7u);
    ws->sweep_base = base + (unsigned long long)job.n_sweeps;
  }
}

// ------------------------------------------------------ grid schedule
// Schedule 2: every sweep of a call, for every replica of one cell
// capacity, in one cooperative launch of every block the device holds.
// Per sweep: each replica's shift and colour order, the cell build of every
// particle, then the eight colour passes over every active cell of every
// replica, the phases separated by a grid-wide barrier.  A pass spreads all
// replicas' cells over the whole device, as the flat launches do, with no
// launch between phases.  The barrier waits are bounded (1 s): one that
// gives up reports ST_FLOW_TIMEOUT and makes every block leave at its next
// barrier.
struct GridJob {
  const SysPtrs *reps;                  // the class's replicas
  const int *rep_ids;                   // their index in the batch (enters the random counters)
  const int *nstart, *gstart, *cstart;  // prefix sums of particles, active cells, allocated cells
  RepParams *params;                    // the current sweep's shift and colour order per replica
  unsigned *bar;                        // barrier: arrivals, generation (zero at launch)
  int *abort;                           // set once a barrier wait gave up (zero at launch)
  unsigned *work;                       // two counters of cells handed out in a pass (zero at launch)
  int *status;                          // where that is reported
  int n_reps, n_sweeps;
};

__device__ __forceinline__ unsigned long long grid_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

// Every block arrives once per phase; the last to arrive resets the count
// and advances the generation with a release store, the others wait for it.
// The CTA barrier before and the fence make the block's writes visible
// device-wide first (data written in the launch is read through L2 only).
__device__ __forceinline__ bool grid_barrier(const GridJob &job, unsigned *reset = nullptr) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g = ld_acquire(job.bar + 1);
    __threadfence();
    if (atomicAdd(job.bar, 1u) == gridDim.x - 1u) {
      atomicExch(job.bar, 0u);
      if (reset) atomicExch(reset, 0u);  // a work counter, for its next use
      __threadfence();
      st_release(job.bar + 1, g + 1u);
    } else {
      const unsigned long long t0 = grid_clock();
      while (ld_acquire(job.bar + 1) == g) {
        if (*(volatile int *)job.abort) {
          ok = 0;
          break;
        }
        if (grid_clock() - t0 > 1000000000ull) {
          atomicOr(job.status, ST_FLOW_TIMEOUT);
          atomicExch(job.abort, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

__device__ __forceinline__ RepParams load_params(const RepParams *q) {
  const float4 v = __ldcg(reinterpret_cast<const float4 *>(q));
  RepParams r;
  r.sh[0] = v.x;
  r.sh[1] = v.y;
  r.sh[2] = v.z;
  r.perm = __float_as_uint(v.w);
  return r;
}

// The cell build of every particle of the class (k_build, sweep.cu), four
// particles a thread at a time so that their loads are issued together.  Kept
// out of line: inlined, its registers pushed the kernel's cell work to spill.
__device__ __noinline__ void grid_build(const GridJob &job, int layout, int gt, int nt, int tot_n) {
  const int nr = job.n_reps;
  constexpr int BU = 4;
  for (int i0 = gt; i0 < tot_n; i0 += BU * nt) {
    int lr[BU], c[BU];
    Slot sl[BU];
#pragma unroll
    for (int u = 0; u < BU; u++) {
      const int i = i0 + u * nt;
      lr[u] = -1;
      if (i >= tot_n) continue;
      lr[u] = find_rep(job.nstart, nr, i);
      const SysPtrs &p = job.reps[lr[u]];
      const RepParams q = load_params(job.params + lr[u]);
      const int li = i - job.nstart[lr[u]];
      const Box *bx = p.box;
      const double2 a = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)li));
      const double2 c2 = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)li + 2));
      int cx, cy, cz;
      axis_cell(__double2float_rn(a.y), q.sh[0], bx->len32[0], bx->inv_w32[0], bx->nc[0], cx, sl[u].x);
      axis_cell(__double2float_rn(c2.x), q.sh[1], bx->len32[1], bx->inv_w32[1], bx->nc[1], cy, sl[u].y);
      axis_cell(__double2float_rn(c2.y), q.sh[2], bx->len32[2], bx->inv_w32[2], bx->nc[2], cz, sl[u].z);
      sl[u].id = li;
      c[u] = cx + bx->nc[0] * (cy + bx->nc[1] * cz);
    }
#pragma unroll
    for (int u = 0; u < BU; u++) {
      if (lr[u] < 0) continue;
      const SysPtrs &p = job.reps[lr[u]];
      const int k = atomicAdd(cnt_of(p, layout) + c[u], 1);
      if (k < p.cap) {
        slot_of(p, layout)[(size_t)c[u] * p.cap + k] = sl[u];
      } else {
        atomicOr(&p.st->status, ST_CELL_OVERFLOW);
      }
    }
  }
}

template <int G, int CAP>
__global__ void __launch_bounds__(128, PassSmem<G, CAP>::min_blocks) k_batch_grid(GridJob job) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PassSm m = pass_smem_ptrs<G, CAP>(smem_raw);
  const int tid = (int)threadIdx.x;
  const int lane = tid % G, gl = tid / G, col0 = tid - lane;
  const int gbase = (tid & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int gt = (int)blockIdx.x * 128 + tid, nt = (int)gridDim.x * 128;
  const int group = gt / G, groups = nt / G;
  const int nr = job.n_reps;
  const int tot_n = job.nstart[nr], tot_g = job.gstart[nr], tot_c = job.cstart[nr];
  // every replica of a batch has made the same number of sweeps; the index
  // is advanced after the last barrier, once every block has read it
  const unsigned long long base = job.reps[0].st->sweep_base;

  for (int s = 0; s < job.n_sweeps; s++) {
    const unsigned long long sweep = base + (unsigned long long)s;
    const int layout = (int)(sweep & 1ull);
    // (1) each replica's shift and colour order, published as the cell
    // build publishes them (for the observables after the call)
    for (int r = gt; r < nr; r += nt) {
      const SysPtrs &p = job.reps[r];
      const uint32_t rep = (uint32_t)job.rep_ids[r];
      const float w[3] = {p.box->w32[0], p.box->w32[1], p.box->w32[2]};
      RepParams q;
      sweep_shift(p.st->seed, rep, sweep, w, q.sh);
      int perm[8];
      sweep_perm(p.st->seed, rep, sweep, perm);
      q.perm = 0u;
      for (int k = 0; k < 8; k++) q.perm |= (uint32_t)perm[k] << (4 * k);
      job.params[r] = q;
      DevState *ws = p.st;
      ws->params.sweep = sweep;
      for (int d = 0; d < 3; d++) ws->params.shift32[d] = q.sh[d];
      for (int k = 0; k < 8; k++) ws->params.perm[k] = perm[k];
    }
    if (!grid_barrier(job)) return;
    // (2) the cell build of every particle (k_build, sweep.cu)
    grid_build(job, layout, gt, nt, tot_n);
    if (!grid_barrier(job)) return;
    // (3) the eight colour passes
    for (int pass = 0; pass < 8; pass++) {
      if (pass == 0) {  // the other layout's counts, for the next sweep's build
        for (int i = gt; i < tot_c; i += nt) {
          const int lr = find_rep(job.cstart, nr, i);
          cnt_of(job.reps[lr], layout ^ 1)[i - job.cstart[lr]] = 0;
        }
      }
      // Each warp takes the next run of one cell per group from a counter,
      // so warps that drew light cells take more (a fixed share per warp
      // left the pass to its unluckiest warp), and its groups take their
      // cells in step (move_pass.cu).
      unsigned *counter = job.work + ((s * 8 + pass) & 1);
      const int wgroups = 32 / G;
      for (;;) {
        int base = 0;
        if ((tid & 31) == 0) base = (int)atomicAdd(counter, (unsigned)wgroups);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= tot_g) break;
        __syncwarp();  // the previous cell's records are no longer read
        const int it = base + (tid & 31) / G;
        if (it >= tot_g) continue;
        const int lr = find_rep(job.gstart, nr, it);
        const SysPtrs &p = job.reps[lr];
        const RepParams q = load_params(job.params + lr);
        const PassEnv e =
            persist_env(p, (uint32_t)job.rep_ids[lr], layout, q, sweep * 8ull + (unsigned long long)pass);
        const int colour = (int)((q.perm >> (4 * pass)) & 7u);
        const int hx = e.nc[0] >> 1, hy = e.nc[1] >> 1;
        const int ac = it - job.gstart[lr];
        const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
        PassTally t;
        bool no_wait = false;
        move_cell<G, CAP, false, true>(e, m, tid, lane, gl, col0, gmask, 2 * ax + (colour & 1),
                                       2 * ay + ((colour >> 1) & 1), 2 * az + ((colour >> 2) & 1), t, no_wait);
        DevState *ws = p.st;
        if (t.acc) atomicAdd(&ws->acc, (unsigned long long)t.acc);
        if (t.rej_o) atomicAdd(&ws->rej_overlap, (unsigned long long)t.rej_o);
        if (t.rej_b) atomicAdd(&ws->rej_boundary, (unsigned long long)t.rej_b);
        if (t.rechecks) atomicAdd(&ws->rechecks, (unsigned long long)t.rechecks);
      }
      if (!grid_barrier(job, job.work + ((s * 8 + pass + 1) & 1))) return;
    }
  }
  for (int r = gt; r < nr; r += nt) job.reps[r].st->sweep_base = base + (unsigned long long)job.n_sweeps;
}

template <int G, int CAP>
static int grid_blocks_for(int num_sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_grid<G, CAP>, 128, PassSmem<G, CAP>::bytes) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm * num_sms;
}

// Blocks of the grid schedule's launch for cell capacity cap: every block
// the device holds at once (0: none fits).
int batch_grid_blocks(int cap, int num_sms) {
  switch (cap) {
    case 8: return grid_blocks_for<2, 8>(num_sms);
    case 16: return grid_blocks_for<4, 16>(num_sms);
    default: return grid_blocks_for<8, 32>(num_sms);
  }
}

template <int G, int CAP>
static cudaError_t grid_launch(const GridJob &job, int blocks, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = PassSmem<G, CAP>::bytes;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_batch_grid<G, CAP>, job);
}

cudaError_t prepare_batch_grid() {
  cudaError_t e = cudaFuncSetAttribute(k_batch_grid<2, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)PassSmem<2, 8>::bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_batch_grid<4, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PassSmem<4, 16>::bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_batch_grid<8, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PassSmem<8, 32>::bytes);
  return e;
}

// One cooperative launch for n_sweeps sweeps of the class's replicas; bar
// (2 words), abort and work (2 words) must be zero.
cudaError_t launch_batch_grid(int cap, const SysPtrs *reps, const int *rep_ids, const int *nstart, const int *gstart,
                              const int *cstart, void *params, unsigned *bar, int *abort, unsigned *work,
                              int *status, int n_reps, int n_sweeps, int blocks, cudaStream_t s) {
  if (n_reps <= 0 || n_sweeps <= 0) return cudaSuccess;
  const GridJob job{reps, rep_ids, nstart, gstart, cstart, reinterpret_cast<RepParams *>(params),
                    bar,  abort,   work,   status, n_reps, n_sweeps};
  switch (cap) {
    case 8: return grid_launch<2, 8>(job, blocks, s);
    case 16: return grid_launch<4, 16>(job, blocks, s);
    default: return grid_launch<8, 32>(job, blocks, s);
  }
}

template <int G, int CAP>
static cudaError_t persist_prepare() {
  return cudaFuncSetAttribute(k_batch_persist<G, CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)persist_smem<G, CAP>());
}

template <int G, int CAP>
static cudaError_t persist_launch(const BundleJob &job, int n_bundles, int cluster_blocks, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(n_bundles * cluster_blocks));
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = persist_smem<G, CAP>();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster_blocks;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_batch_persist<G, CAP>, job);
}

template <int G, int CAP>
static int persist_clusters(int cluster_blocks) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cluster_blocks);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = persist_smem<G, CAP>();
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster_blocks;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_batch_persist<G, CAP>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

// Clusters of cluster_blocks blocks the device holds at once for cell
// capacity cap (0: such a cluster does not fit).
int batch_persist_max_clusters(int cap, int cluster_blocks) {
  switch (cap) {
    case 8: return persist_clusters<2, 8>(cluster_blocks);
    case 16: return persist_clusters<4, 16>(cluster_blocks);
    default: return persist_clusters<8, 32>(cluster_blocks);
  }
}

// Largest replica count per bundle, for the host's packing.
int batch_persist_max_reps() { return kBundleMaxReps; }

cudaError_t prepare_batch_persist() {
  cudaError_t e = persist_prepare<2, 8>();
  if (e == cudaSuccess) e = persist_prepare<4, 16>();
  if (e == cudaSuccess) e = persist_prepare<8, 32>();
  return e;
}

// cap 8, 16, 32 with 2, 4, 8 lanes per cell: one block's shared memory is
// the same for all three
cudaError_t launch_batch_persist(int cap, const SysPtrs *reps, const int *rep_ids, const int *nstart,
                                 const int *gstart, const int *cstart, const int *bundle, int n_bundles,
                                 int n_sweeps, int cluster_blocks, cudaStream_t s) {
  if (n_bundles <= 0 || n_sweeps <= 0) return cudaSuccess;
  const BundleJob job{reps, rep_ids, nstart, gstart, cstart, bundle, n_sweeps};
  switch (cap) {
    case 8: return persist_launch<2, 8>(job, n_bundles, cluster_blocks, s);
    case 16: return persist_launch<4, 16>(job, n_bundles, cluster_blocks, s);
    default: return persist_launch<8, 32>(job, n_bundles, cluster_blocks, s);
  }
}

}  // namespace hsmc
