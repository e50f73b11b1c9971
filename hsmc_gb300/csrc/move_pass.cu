// The colour passes of the checkerboard sweep (part_move / check_overlap,
// src/moves.c:27-80 and 157-212, for all cells of one colour at once), in
// two schedules: one launch per pass (k_move_pass; each pass a programmatic
// dependent launch of the one before) and the dataflow sweep (k_move_flow,
// all eight passes in one cooperative launch).  The per-cell work is
// move_cell (move_cell.cuh).
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "move_cell.cuh"

namespace cg = cooperative_groups;

namespace hsmc {

// One colour pass: every active cell of the colour, then a kernel boundary.
// In a batch (BATCH) the grid covers the active cells of every replica of
// one cell capacity (gstart: their prefix sums); each group finds its
// replica, whose batch index (rep_ids) enters the random counters, and the
// counters are summed per replica.  Given the pooled count arrays, the first
// pass also clears their other layout.
template <int G, int CAP, bool TRACE, bool BATCH>
__global__ void __launch_bounds__(128, PassSmem<G, CAP>::min_blocks)
    k_move_pass(SysPtrs p1, const SysPtrs *reps, const int *gstart, const int *rep_ids, int n_reps, int pass,
                int *pool0, int *pool1, long long pool_cells) {
  static_assert(G == 1 || G == 2 || G == 4 || G == 8, "group size");
  // Launched as a programmatic dependent of the previous pass (launch_gc),
  // the blocks become resident while that pass drains.  A pass after the
  // first reads its cells' own data at once (nothing before it in the sweep
  // writes that data) and waits for the previous pass to complete, and its
  // writes to be visible, only before reading the neighbours (move_cell).
  // The first pass follows the cell build, which writes everything, so it
  // waits here, as does a batch pass.  The next pass may be scheduled as
  // soon as every block of this one runs: it too touches nothing this pass
  // writes before its own wait.
  if (BATCH || pass == 0) asm volatile("griddepcontrol.wait;\n" ::: "memory");
  if (BATCH) asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PassSm m = pass_smem_ptrs<G, CAP>(smem_raw);
  const int tid = (int)threadIdx.x;
  const int lane = tid % G;
  const int gl = tid / G;  // group within the block
  const int col0 = tid - lane;
  const int group = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);
  const int gbase = (tid & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  PassTally t;

  if (!BATCH) {
    const SysPtrs &p = p1;
    const unsigned long long sweep = p.st->params.sweep;
    const int layout = (int)(sweep & 1ull);
    PassEnv e = pass_env(p, 0u, layout);
    e.seq = sweep * 8ull + (unsigned long long)pass;
    e.signal = true;
    const int colour = p.st->params.perm[pass];
    // The first pass of a sweep clears the other layout for the next build.
    if (pass == 0) {
      int *other = cnt_of(p, layout ^ 1);
      for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x)
        other[c] = 0;
    }
    bool wait_prev = pass != 0;
    const int hx = e.nc[0] >> 1, hy = e.nc[1] >> 1, hz = e.nc[2] >> 1;
    const int cx = colour & 1, cy = (colour >> 1) & 1, cz = (colour >> 2) & 1;
    // Which cells the groups take, by rounds: a group takes entry a of a
    // sequence of cells, then a + stride, while a < limit.
    //  - spatial (p.olist null): the active cells of the colour in grid order.
    //    With at most one cell per group, each block takes an equal run of
    //    consecutive active cells (a small system is spread over every SM,
    //    move_pass_grid); otherwise the groups stride over the cells.
    //  - occupancy order (schedule 3): the colour's non-empty cells, fullest
    //    first (k_order_scatter), in runs of one cell per lane group of a
    //    warp; run j goes to block j mod grid, so the fullest runs (the
    //    longest trial chains) spread over every SM.  The list was complete
    //    before the first pass of the sweep began, so a pass may read it
    //    before its wait on the previous pass.
    const bool ordered = p.olist != nullptr;
    const int *list = nullptr;
    int a, stride, limit;
    if (ordered) {
      constexpr int GPW = 32 / G;  // lane groups per warp
      limit = p.ocnt[512 + colour];
      list = p.olist + (size_t)colour * (size_t)(p.ncell_alloc / 8);
      const int nwb = (int)blockDim.x >> 5;
      a = ((int)blockIdx.x + (int)gridDim.x * (tid >> 5)) * GPW + (tid & 31) / G;
      stride = (int)gridDim.x * nwb * GPW;
    } else {
      limit = hx * hy * hz;
      const int gpb = (int)blockDim.x / G;
      a = group;
      stride = (int)((gridDim.x * blockDim.x) / G);
      if (limit <= (int)gridDim.x * gpb) {
        const int per_block = (limit + (int)gridDim.x - 1) / (int)gridDim.x;
        a = gl < per_block ? (int)blockIdx.x * per_block + gl : limit;
        stride = limit;
      }
    }
    // The warp takes its cells in step: its groups start each round together
    // (left to drift, the groups of a warp would run different phases of
    // different cells, and the warp would issue each phase once per group).
    for (; __any_sync(0xffffffffu, a < limit); a += stride) {
      __syncwarp();  // the previous cell's records are no longer read
      if (a < limit) {
        int ix, iy, iz;
        if (ordered) {
          const int c = list[a];
          const int iyz = c / e.nc[0];
          ix = c - iyz * e.nc[0];
          iy = iyz % e.nc[1];
          iz = iyz / e.nc[1];
        } else {
          const int ax = a % hx, ayz = a / hx, ay = ayz % hy, az = ayz / hy;
          ix = 2 * ax + cx;
          iy = 2 * ay + cy;
          iz = 2 * az + cz;
        }
        move_cell<G, CAP, TRACE, false>(e, m, tid, lane, gl, col0, gmask, ix, iy, iz, t, wait_prev);
      }
    }
    // A block without cells, or whose cells were all empty, has not waited
    // for the previous pass: it waits now, so that this pass completes only
    // after that one (the next pass's wait, and its launch, rely on it).
    if (wait_prev) asm volatile("griddepcontrol.wait;\n" ::: "memory");
    add_tally(t, p.st);
    return;
  }

  if (pass == 0 && pool_cells > 0) {
    const int layout0 = (int)(reps[0].st->params.sweep & 1ull);
    int *other = layout0 ? pool0 : pool1;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < pool_cells;
         c += (long long)gridDim.x * blockDim.x)
      other[c] = 0;
  }
  // One cell of replica r (within the class) by this lane group.
  auto move_rep_cell = [&](int r, int ac_or_cell, bool listed, PassTally &tt) {
    const SysPtrs p = reps[r];
    const unsigned long long sweep = p.st->params.sweep;
    PassEnv e = pass_env(p, (uint32_t)__ldg(rep_ids + r), (int)(sweep & 1ull));
    e.seq = sweep * 8ull + (unsigned long long)pass;
    int ix, iy, iz;
    if (listed) {
      const int c = ac_or_cell, iyz = c / e.nc[0];
      ix = c - iyz * e.nc[0];
      iy = iyz % e.nc[1];
      iz = iyz / e.nc[1];
    } else {
      const int colour = p.st->params.perm[pass];
      const int hx = e.nc[0] >> 1, hy = e.nc[1] >> 1;
      const int ac = ac_or_cell;
      const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
      ix = 2 * ax + (colour & 1);
      iy = 2 * ay + ((colour >> 1) & 1);
      iz = 2 * az + ((colour >> 2) & 1);
    }
    bool no_wait = false;
    move_cell<G, CAP, TRACE, false>(e, m, tid, lane, gl, col0, gmask, ix, iy, iz, tt, no_wait);
  };
  // The lanes of one replica sum their counters together (every lane of the
  // warp takes part; r < 0: no replica).
  auto add_rep_tally = [&](int r, const PassTally &tt) {
    const cg::thread_block_tile<32> tile = cg::tiled_partition<32>(cg::this_thread_block());
    const auto part = cg::labeled_partition(tile, r);
    const unsigned a = cg::reduce(part, tt.acc, cg::plus<unsigned>());
    const unsigned o = cg::reduce(part, tt.rej_o, cg::plus<unsigned>());
    const unsigned bnd = cg::reduce(part, tt.rej_b, cg::plus<unsigned>());
    const unsigned rc = cg::reduce(part, tt.rechecks, cg::plus<unsigned>());
    if (r >= 0 && part.thread_rank() == 0) {
      DevState *ws = reps[r].st;
      if (a) atomicAdd(&ws->acc, (unsigned long long)a);
      if (o) atomicAdd(&ws->rej_overlap, (unsigned long long)o);
      if (bnd) atomicAdd(&ws->rej_boundary, (unsigned long long)bnd);
      if (rc) atomicAdd(&ws->rechecks, (unsigned long long)rc);
    }
  };
  if (p1.olist != nullptr) {
    // Occupancy order (batch schedule 3): list `pass` holds the (replica,
    // cell) pairs of every replica's cells that move in this pass, fullest
    // first (k_border_scatter); runs of one cell per lane group of a warp,
    // run j to block j mod grid, as in a single system's occupancy order.
    constexpr int GPW = 32 / G;
    const int total = p1.ocnt[512 + pass];
    const int *list = p1.olist + 2 * (size_t)pass * (size_t)p1.ncell_alloc;
    const int nwb = (int)blockDim.x >> 5;
    const int stride = (int)gridDim.x * nwb * GPW;
    for (int a = ((int)blockIdx.x + (int)gridDim.x * (tid >> 5)) * GPW + (tid & 31) / G;
         __any_sync(0xffffffffu, a < total); a += stride) {
      __syncwarp();  // the previous cell's records are no longer read
      int r = -1;
      PassTally tt;
      if (a < total) {
        r = list[2 * (size_t)a];
        move_rep_cell(r, list[2 * (size_t)a + 1], true, tt);
      }
      add_rep_tally(r, tt);
    }
    return;
  }
  int r = -1;
  if (group < __ldg(gstart + n_reps)) {
    r = find_rep(gstart, n_reps, group);
    move_rep_cell(r, group - __ldg(gstart + r), false, t);
  }
  add_rep_tally(r, t);
}

// All eight passes of a sweep in one cooperative launch, without barriers
// between passes.  The grid is cut into 2x2x2 regions, one cell of each
// colour; a group owns regions and goes through its regions pass by pass.
// Before pass k of a cell it waits until the seven regions around the
// cell's own have published pass k - 1 (prog[r] = 8 sweep + passes done),
// so each cell sees its 26 neighbours exactly as after the pass barrier: the
// chain is the one of k_move_pass.  The wait is per warp (all its groups'
// neighbourhoods), so the groups of a warp stay converged.  Waits only point
// from pass k to pass k - 1 and every block is resident (cooperative launch),
// so the schedule cannot deadlock; each wait is bounded and reports
// ST_FLOW_TIMEOUT.
__device__ __forceinline__ void warp_wait(const uint32_t *prog, const int *reg, bool valid, uint32_t target,
                                          int *status) {
  uint64_t t0 = 0;
  for (;;) {
    bool ready = true;
    if (valid) {
#pragma unroll
      for (int k = 0; k < 7; k++) ready &= (int)(ld_acquire(prog + reg[k]) - target) >= 0;
    }
    if (__all_sync(0xffffffffu, ready)) break;
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    if (t0 == 0) t0 = t;
    if (__any_sync(0xffffffffu, t - t0 > 1000000000ull)) {
      if ((threadIdx.x & 31) == 0) atomicOr(status, ST_FLOW_TIMEOUT);
      break;
    }
    __nanosleep(64);
  }
  __threadfence();
}

template <int G, int CAP, bool TRACE>
__global__ void __launch_bounds__(128, PassSmem<G, CAP>::min_blocks) k_move_flow(SysPtrs p, uint32_t *prog) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PassSm m = pass_smem_ptrs<G, CAP>(smem_raw);
  const unsigned long long sweep = p.st->params.sweep;
  const int layout = (int)(sweep & 1ull);
  PassEnv e = pass_env(p, 0u, layout);

  {
    int *other = cnt_of(p, layout ^ 1);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x) other[c] = 0;
  }

  const int tid = (int)threadIdx.x;
  const int lane = tid % G;
  const int gl = tid / G;
  const int col0 = tid - lane;
  const int group = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);
  const int groups = (int)((gridDim.x * blockDim.x) / G);
  const int gbase = (tid & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int hx = e.nc[0] >> 1, hy = e.nc[1] >> 1, hz = e.nc[2] >> 1;
  const int n_active = hx * hy * hz;
  const int iters = (n_active + groups - 1) / groups;  // the same for every thread
  const uint32_t base = (uint32_t)(sweep * 8ull);
  const int hold = p.st->flow_hold;

  PassTally t;
  for (int pass = 0; pass < 8; pass++) {
    const int colour = p.st->params.perm[pass];
    const int cx = colour & 1, cy = (colour >> 1) & 1, cz = (colour >> 2) & 1;
    e.seq = sweep * 8ull + (unsigned long long)pass;
    for (int it = 0; it < iters; it++) {
      const int ac = group + it * groups;
      const bool valid = ac < n_active;
      const int acv = valid ? ac : 0;
      const int ax = acv % hx, ayz = acv / hx, ay = ayz % hy, az = ayz / hy;
      if (pass > 0) {
        // the regions holding the cell's neighbours: its own and, per axis,
        // the one on the side the cell sits
        int reg[7];
        const int bx = cx ? (ax + 1 == hx ? 0 : ax + 1) : (ax == 0 ? hx - 1 : ax - 1);
        const int by = cy ? (ay + 1 == hy ? 0 : ay + 1) : (ay == 0 ? hy - 1 : ay - 1);
        const int bz = cz ? (az + 1 == hz ? 0 : az + 1) : (az == 0 ? hz - 1 : az - 1);
#pragma unroll
        for (int q = 1; q < 8; q++) {
          const int rx = (q & 1) ? bx : ax, ry = (q & 2) ? by : ay, rz = (q & 4) ? bz : az;
          reg[q - 1] = rx + hx * (ry + hy * rz);
        }
        warp_wait(prog, reg, valid, base + (uint32_t)pass, &p.st->status);
      }
      bool no_wait = false;
      if (valid)
        move_cell<G, CAP, TRACE, true>(e, m, tid, lane, gl, col0, gmask, 2 * ax + cx, 2 * ay + cy, 2 * az + cz, t,
                                       no_wait);
      __syncwarp();
      if (valid && lane == 0 && ac != hold) {
        __threadfence();
        st_release(prog + ac, base + (uint32_t)pass + 1u);
      }
    }
  }
  add_tally(t, p.st);
}

// ------------------------------------------------------------------ launch
template <int G, int CAP>
static size_t pass_smem() {
  return PassSmem<G, CAP>::bytes;
}

static int smem_optin_limit() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

// Dynamic shared memory above 48 KB has to be allowed per kernel and device,
// before any launch is captured into a graph: prepare_move_pass does it for
// every variant that fits on the current device.
template <int G, int CAP, bool TRACE, bool BATCH>
static void allow_smem() {
  if (pass_smem<G, CAP>() > (size_t)smem_optin_limit()) return;
  cudaFuncSetAttribute(k_move_pass<G, CAP, TRACE, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)pass_smem<G, CAP>());
}

template <int G, int CAP, bool TRACE>
static void allow_flow_smem() {
  if (pass_smem<G, CAP>() > (size_t)smem_optin_limit()) return;
  cudaFuncSetAttribute(k_move_flow<G, CAP, TRACE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)pass_smem<G, CAP>());
}

template <int G, int CAP>
static void allow_all() {
  allow_smem<G, CAP, false, false>();
  allow_smem<G, CAP, true, false>();
  allow_smem<G, CAP, false, true>();
  allow_flow_smem<G, CAP, false>();
  allow_flow_smem<G, CAP, true>();
}

template <int G>
static void allow_caps() {
  allow_all<G, 8>();
  allow_all<G, 16>();
  allow_all<G, 32>();
}

void prepare_move_pass() {
  allow_caps<1>();
  allow_caps<2>();
  allow_caps<4>();
  allow_caps<8>();
}

template <int G>
static size_t smem_for_g(int cap) {
  return cap <= 8 ? PassSmem<G, 8>::bytes : (cap <= 16 ? PassSmem<G, 16>::bytes : PassSmem<G, 32>::bytes);
}

static size_t smem_for(int group, int cap) {
  switch (group) {
    case 1: return smem_for_g<1>(cap);
    case 2: return smem_for_g<2>(cap);
    case 4: return smem_for_g<4>(cap);
    default: return smem_for_g<8>(cap);
  }
}

bool move_pass_fits(int group, int cap) {
  if (group != 1 && group != 2 && group != 4 && group != 8) return false;
  return smem_for(group, cap) <= (size_t)smem_optin_limit();
}

// One group per active cell (an eighth of the grid) in full blocks, one
// wave when the occupancy allows it, grid-stride otherwise.  A system that
// fills less than half the wave is spread over every block slot instead (a
// few cells per block): the SMs' bursts of neighbour copies and trials then
// share the work, which measured 25 % faster per sweep at N = 4000, while a
// full wave of equal runs measured 1.3 % slower than full blocks at
// N = 256,000 (the free block slots let the next pass start its blocks
// early).
template <int G, int CAP>
static int pass_blocks_for(int ncell_alloc, int num_sms) {
  if (pass_smem<G, CAP>() > (size_t)smem_optin_limit()) return 0;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_move_pass<G, CAP, false, false>, 128,
                                                pass_smem<G, CAP>());
  if (per_sm < 1) per_sm = 1;
  const int active = ncell_alloc / 8;
  const long long threads = (long long)active * G;
  const int need = (int)((threads + 127) / 128);
  const int cap = per_sm * num_sms;
  if (2 * need <= cap) return active < cap ? (active > 0 ? active : 1) : cap;
  return need < cap ? (need > 0 ? need : 1) : cap;
}

template <int G>
static int pass_blocks_g(int cap, int ncell_alloc, int num_sms) {
  switch (cap) {
    case 8: return pass_blocks_for<G, 8>(ncell_alloc, num_sms);
    case 16: return pass_blocks_for<G, 16>(ncell_alloc, num_sms);
    default: return pass_blocks_for<G, 32>(ncell_alloc, num_sms);
  }
}

int move_pass_grid(int group, int cap, int ncell_alloc, int num_sms) {
  switch (group) {
    case 1: return pass_blocks_g<1>(cap, ncell_alloc, num_sms);
    case 2: return pass_blocks_g<2>(cap, ncell_alloc, num_sms);
    case 4: return pass_blocks_g<4>(cap, ncell_alloc, num_sms);
    default: return pass_blocks_g<8>(cap, ncell_alloc, num_sms);
  }
}

// A pass is a programmatic dependent launch: it may be scheduled before the
// kernel ahead of it in the stream has finished, and waits for it inside
// (griddepcontrol.wait), which hides the launch latency between passes.
template <int G, int CAP>
static void launch_gc(const SysPtrs &p, int pass, bool trace, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = pass_smem<G, CAP>();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const SysPtrs *no_reps = nullptr;
  const int *no_ints = nullptr;
  int *no_pool = nullptr;
  if (trace)
    cudaLaunchKernelEx(&cfg, k_move_pass<G, CAP, true, false>, p, no_reps, no_ints, no_ints, 0, pass, no_pool, no_pool,
                       0ll);
  else
    cudaLaunchKernelEx(&cfg, k_move_pass<G, CAP, false, false>, p, no_reps, no_ints, no_ints, 0, pass, no_pool,
                       no_pool, 0ll);
}

template <int G, int CAP>
static void launch_batch_gc(const SysPtrs *reps, const int *gstart, const int *ids, int n_reps, int tot_groups,
                            int pass, int *pool0, int *pool1, long long pool_cells, const SysPtrs &order,
                            cudaStream_t s) {
  const long long threads = (long long)tot_groups * G;
  const int grid = (int)((threads + 127) / 128);
  k_move_pass<G, CAP, false, true><<<grid > 0 ? grid : 1, 128, pass_smem<G, CAP>(), s>>>(
      order, reps, gstart, ids, n_reps, pass, pool0, pool1, pool_cells);
}

void launch_move_pass_batch(const SysPtrs *reps, const int *gstart, const int *ids, int n_reps, int tot_groups,
                            int cap, int pass, int group, int *cnt_pool0, int *cnt_pool1, long long pool_cells,
                            int *olist, int *ocnt, cudaStream_t s) {
  SysPtrs order{};  // the occupancy lists of the class (olist null: grid order)
  order.olist = olist;
  order.ocnt = ocnt;
  order.ncell_alloc = tot_groups;  // entries per pass list
#define HSMC_BATCH_CAP(G)                                                                                  \
  switch (cap) {                                                                                           \
    case 8: launch_batch_gc<G, 8>(reps, gstart, ids, n_reps, tot_groups, pass, cnt_pool0, cnt_pool1, pool_cells, order, s); break; \
    case 16: launch_batch_gc<G, 16>(reps, gstart, ids, n_reps, tot_groups, pass, cnt_pool0, cnt_pool1, pool_cells, order, s); break; \
    default: launch_batch_gc<G, 32>(reps, gstart, ids, n_reps, tot_groups, pass, cnt_pool0, cnt_pool1, pool_cells, order, s); break; \
  }
  switch (group) {
    case 1: HSMC_BATCH_CAP(1) break;
    case 2: HSMC_BATCH_CAP(2) break;
    case 4: HSMC_BATCH_CAP(4) break;
    default: HSMC_BATCH_CAP(8) break;
  }
#undef HSMC_BATCH_CAP
}

template <int G>
static void launch_g(const SysPtrs &p, int pass, bool trace, int grid, cudaStream_t s) {
  switch (p.cap) {
    case 8: launch_gc<G, 8>(p, pass, trace, grid, s); break;
    case 16: launch_gc<G, 16>(p, pass, trace, grid, s); break;
    default: launch_gc<G, 32>(p, pass, trace, grid, s); break;
  }
}

// Dataflow sweep: the grid is every block the device can hold at once (the
// cooperative launch checks it), so every group's waits can be met.
template <int G, int CAP>
static int flow_blocks_for(int num_sms) {
  if (pass_smem<G, CAP>() > (size_t)smem_optin_limit()) return 0;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_move_flow<G, CAP, false>, 128, pass_smem<G, CAP>());
  int per_sm_t = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_t, k_move_flow<G, CAP, true>, 128, pass_smem<G, CAP>());
  if (per_sm_t < per_sm) per_sm = per_sm_t;
  return per_sm * num_sms;
}

template <int G>
static int flow_blocks_g(int cap, int num_sms) {
  switch (cap) {
    case 8: return flow_blocks_for<G, 8>(num_sms);
    case 16: return flow_blocks_for<G, 16>(num_sms);
    default: return flow_blocks_for<G, 32>(num_sms);
  }
}

int move_flow_grid(int group, int cap, int ncell_alloc, int num_sms) {
  int cap_blocks = 0;
  switch (group) {
    case 1: cap_blocks = flow_blocks_g<1>(cap, num_sms); break;
    case 2: cap_blocks = flow_blocks_g<2>(cap, num_sms); break;
    case 4: cap_blocks = flow_blocks_g<4>(cap, num_sms); break;
    default: cap_blocks = flow_blocks_g<8>(cap, num_sms); break;
  }
  const long long threads = (long long)(ncell_alloc / 8) * group;  // one group per region at most
  const int need = (int)((threads + 127) / 128);
  return need < cap_blocks ? (need > 0 ? need : 1) : cap_blocks;
}

template <int G, int CAP, bool TRACE>
static cudaError_t launch_flow_gct(const SysPtrs &p, uint32_t *prog, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = pass_smem<G, CAP>();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_move_flow<G, CAP, TRACE>, p, prog);
}

template <int G>
static cudaError_t launch_flow_g(const SysPtrs &p, uint32_t *prog, bool trace, int grid, cudaStream_t s) {
  switch (p.cap) {
    case 8: return trace ? launch_flow_gct<G, 8, true>(p, prog, grid, s) : launch_flow_gct<G, 8, false>(p, prog, grid, s);
    case 16:
      return trace ? launch_flow_gct<G, 16, true>(p, prog, grid, s) : launch_flow_gct<G, 16, false>(p, prog, grid, s);
    default:
      return trace ? launch_flow_gct<G, 32, true>(p, prog, grid, s) : launch_flow_gct<G, 32, false>(p, prog, grid, s);
  }
}

cudaError_t launch_move_flow(const SysPtrs &p, uint32_t *prog, int group, bool trace, int grid, cudaStream_t s) {
  switch (group) {
    case 1: return launch_flow_g<1>(p, prog, trace, grid, s);
    case 2: return launch_flow_g<2>(p, prog, trace, grid, s);
    case 4: return launch_flow_g<4>(p, prog, trace, grid, s);
    default: return launch_flow_g<8>(p, prog, trace, grid, s);
  }
}

void launch_move_pass(const SysPtrs &p, int pass, int group, bool trace, int grid, cudaStream_t s) {
  switch (group) {
    case 1: launch_g<1>(p, pass, trace, grid, s); break;
    case 2: launch_g<2>(p, pass, trace, grid, s); break;
    case 4: launch_g<4>(p, pass, trace, grid, s); break;
    default: launch_g<8>(p, pass, trace, grid, s); break;
  }
}

}  // namespace hsmc
