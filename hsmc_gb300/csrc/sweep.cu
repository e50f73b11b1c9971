// Checkerboard sweep of the local-move hard-sphere Monte Carlo chain.
//
// One sweep = N trial moves, as sweep_nvt makes them (src/nvt.c:201-209), but
// organised for a GPU after Anderson, Jankowski, Grubb, Engel & Glotzer
// (J. Comput. Phys. 254, 27, 2013):
//   1. k_build bins every particle into a periodic grid of cells (edge > 1,
//      even count per axis) shifted by a fresh random vector: a counting sort
//      by atomic slot claims into fixed-capacity cells.
//   2. Eight k_move_pass launches (move_pass.cu), one per colour of the 2x2x2 checkerboard in
//      a random order.  Cells of one colour are more than one diameter apart,
//      so all of them move at once.  In each active cell a group of G lanes
//      makes n trial moves (n = particles in the cell), each on a particle
//      chosen uniformly in the cell; a move that leaves the cell is rejected.
// The trial position and the overlap decision use the reference's FP64
// arithmetic (part_move / check_overlap / compute_dist, src/moves.c:27-80,
// 157-212, 400-431).  A single-precision screen decides every pair whose r^2
// is farther than a guard band from 1; pairs inside the band are re-evaluated
// in FP64 exactly as the reference does, so decisions are bit-identical.
#include "engine.cuh"

namespace hsmc {

// ------------------------------------------------------------------ build
// Bins every particle into the layout of sweep s = sweep_base + offset.
// Thread 0 also publishes that sweep's shift and colour order.
// In a batch (BATCH), the grid covers every replica's particles (nstart:
// their prefix sums) and each thread finds its replica; the replica index
// enters every random counter, so replica 0 draws what a single system draws.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_build(SysPtrs p1, const SysPtrs *reps, const int *nstart, int n_reps,
                                               long long offset) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t rep = 0u;
  if (BATCH) {
    if (i >= __ldg(nstart + n_reps)) return;
    rep = (uint32_t)find_rep(nstart, n_reps, i);
    i -= __ldg(nstart + rep);
  }
  const SysPtrs p = BATCH ? reps[rep] : p1;
  // the occupancy counts of this sweep's order start from zero (k_order_count
  // adds to them once the cell build has completed)
  if (!BATCH && p.ocnt != nullptr && blockIdx.x == 0)
    for (int t = threadIdx.x; t < 256; t += blockDim.x) p.ocnt[t] = 0;
  const DevState *st = p.st;
  const Box *bx = p.box;
  const unsigned long long s = st->sweep_base + (unsigned long long)offset;
  const unsigned long long seed = st->seed;
  const float w[3] = {bx->w32[0], bx->w32[1], bx->w32[2]};
  float sh[3];
  sweep_shift(seed, rep, s, w, sh);
  const float sh0 = sh[0], sh1 = sh[1], sh2 = sh[2];
  const int layout = (int)(s & 1ull);
  if (i == 0) {
    DevState *ws = p.st;
    ws->params.sweep = s;
    ws->params.shift32[0] = sh0;
    ws->params.shift32[1] = sh1;
    ws->params.shift32[2] = sh2;
    int perm[8];
    sweep_perm(seed, rep, s, perm);
    for (int k = 0; k < 8; k++) ws->params.perm[k] = perm[k];
  }
  if (i >= p.n) return;
  const double2 a = *reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i);
  const double2 b = *reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i + 2);
  const float x32 = __double2float_rn(a.y), y32 = __double2float_rn(b.x), z32 = __double2float_rn(b.y);
  int cx, cy, cz;
  float tx, ty, tz;
  axis_cell(x32, sh0, bx->len32[0], bx->inv_w32[0], bx->nc[0], cx, tx);
  axis_cell(y32, sh1, bx->len32[1], bx->inv_w32[1], bx->nc[1], cy, ty);
  axis_cell(z32, sh2, bx->len32[2], bx->inv_w32[2], bx->nc[2], cz, tz);
  const int c = cx + bx->nc[0] * (cy + bx->nc[1] * cz);
  const int k = atomicAdd(cnt_of(p, layout) + c, 1);
  if (k < p.cap) {
    slot_of(p, layout)[(size_t)c * p.cap + k] = Slot{tx, ty, tz, i};
  } else {
    atomicOr(&p.st->status, ST_CELL_OVERFLOW);
  }
}

__global__ void k_advance(DevState *st, int n) { st->sweep_base += (unsigned long long)n; }

// ---------------------------------------------------------- occupancy order
// A colour pass gives each warp the cells of 32/G consecutive entries of
// its colour's list, and a warp makes as many trial rounds as its fullest
// cell holds particles.  Listed fullest first, a warp's cells hold the same
// number of particles (but for the few warps at the boundary of two
// occupancies), and empty cells take no lanes.  The order changes nothing in
// the chain: the cells of one colour are independent, and a cell's random
// numbers are keyed by the cell, not by the lanes that move it.
//
// Two launches after the build, 1024 cells per block: k_order_count counts
// each colour's cells by occupancy (shared-memory histogram, one global add
// per bin and block); k_order_scatter places each block's cells of one bin
// at the bin's start (the cells of more particles come first) plus the
// block's reservation from the bin's cursor.
constexpr int kOrderThreads = 256, kOrderPerThread = 4;

// Bin of cell c (colour * 32 + min(n, 32) - 1) of the current grid, or -1
// for an empty cell or one beyond the grid.
__device__ __forceinline__ int order_bin(const int *cnt, int c, int ncell, int nc0, int nc1) {
  if (c >= ncell) return -1;
  const int n = cnt[c];
  if (n <= 0) return -1;
  const int ix = c % nc0, iyz = c / nc0, iy = iyz % nc1, iz = iyz / nc1;
  return 32 * cell_colour(ix, iy, iz) + (n < 32 ? n : 32) - 1;
}

__global__ void __launch_bounds__(kOrderThreads) k_order_count(SysPtrs p) {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  __shared__ int h[256];
  const int tid = (int)threadIdx.x;
  h[tid] = 0;
  if (blockIdx.x == 0) p.ocnt[256 + tid] = 0;  // the scatter's cursors
  __syncthreads();
  const Box *bx = p.box;
  const int nc0 = bx->nc[0], nc1 = bx->nc[1], ncell = bx->ncell;
  const int *cnt = cnt_of(p, (int)(p.st->params.sweep & 1ull));
  const int c0 = (blockIdx.x * kOrderThreads + tid) * kOrderPerThread;
#pragma unroll
  for (int k = 0; k < kOrderPerThread; k++) {
    const int b = order_bin(cnt, c0 + k, ncell, nc0, nc1);
    if (b >= 0) atomicAdd(&h[b], 1);
  }
  __syncthreads();
  if (h[tid]) atomicAdd(&p.ocnt[tid], h[tid]);
}

__global__ void __launch_bounds__(kOrderThreads) k_order_scatter(SysPtrs p) {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  __shared__ int h[256], tot[256], start[256];
  const int tid = (int)threadIdx.x;
  h[tid] = 0;
  tot[tid] = p.ocnt[tid];
  __syncthreads();
  // the number of non-empty cells of each colour, for the passes
  if (blockIdx.x == 0 && tid < 8) {
    int t = 0;
    for (int m = 0; m < 32; m++) t += tot[32 * tid + m];
    p.ocnt[512 + tid] = t;
  }
  const Box *bx = p.box;
  const int nc0 = bx->nc[0], nc1 = bx->nc[1], ncell = bx->ncell;
  const int *cnt = cnt_of(p, (int)(p.st->params.sweep & 1ull));
  const int c0 = (blockIdx.x * kOrderThreads + tid) * kOrderPerThread;
  int bin[kOrderPerThread], at[kOrderPerThread];
#pragma unroll
  for (int k = 0; k < kOrderPerThread; k++) {
    bin[k] = order_bin(cnt, c0 + k, ncell, nc0, nc1);
    at[k] = bin[k] >= 0 ? atomicAdd(&h[bin[k]], 1) : 0;
  }
  __syncthreads();
  if (h[tid]) {
    // bin tid = colour * 32 + n - 1 starts after the colour's cells holding more than n
    int first = 0;
    for (int m = (tid & 31) + 1; m < 32; m++) first += tot[(tid & ~31) + m];
    start[tid] = first + atomicAdd(&p.ocnt[256 + tid], h[tid]);
  }
  __syncthreads();
  const int stride = p.ncell_alloc / 8;
#pragma unroll
  for (int k = 0; k < kOrderPerThread; k++)
    if (bin[k] >= 0) p.olist[(bin[k] >> 5) * stride + start[bin[k]] + at[k]] = c0 + k;
}

// One step of the reference's optimiser after sample j of the sampling loop
// (opt_nvt src/optimizer.c:23-64, opt_npt :83-148, opt_cavity_nvt :172-212):
// the sample's acceptance from the counters since the previous step, then
// after the first sample the step doubled or halved, after the others the
// secant step toward the target with the reference's clamps, as long as a
// sample follows (j < n_samples + 1).  The arithmetic is the reference's
// double-precision expression with no contraction.  sweep_moves: the
// particle trial moves of every sample so far.
__global__ void k_opt_step(DevState *st, int j, int n_samples, unsigned long long sweep_moves, double part_target,
                           double vol_target, int npt) {
  const unsigned long long acc = st->acc + st->cav_acc;
  const unsigned long long moves = sweep_moves + st->cav_moves;
  const double a = __ddiv_rn((double)(acc - st->opt_acc0), (double)(moves - st->opt_moves0));
  const double av = npt ? __ddiv_rn((double)(st->vol_acc - st->opt_vacc0), (double)(st->vol_moves - st->opt_vmoves0))
                        : 0.0;
  st->opt_acc0 = acc;
  st->opt_moves0 = moves;
  st->opt_vacc0 = st->vol_acc;
  st->opt_vmoves0 = st->vol_moves;
  double dr = st->dr_max, dv = st->dv_max;
  if (j == 0) {
    st->opt_d[0] = dr;
    st->opt_a[0] = a;
    dr = a > part_target ? __dmul_rn(dr, 2.0) : __ddiv_rn(dr, 2.0);
    if (npt) {
      st->opt_v[0] = dv;
      st->opt_av[0] = av;
      dv = av > vol_target ? __dmul_rn(dv, 2.0) : __ddiv_rn(dv, 2.0);
    }
  } else {
    st->opt_d[1] = dr;
    st->opt_a[1] = a;
    if (npt) {
      st->opt_v[1] = dv;
      st->opt_av[1] = av;
    }
    if (j <= n_samples) {
      const double d1 = st->opt_d[0], d2 = st->opt_d[1], a1 = st->opt_a[0], a2 = st->opt_a[1];
      dr = __dsub_rn(d2, __ddiv_rn(__dmul_rn(__dsub_rn(a2, part_target), __dsub_rn(d2, d1)), __dsub_rn(a2, a1)));
      if (npt) {
        const double v1 = st->opt_v[0], v2 = st->opt_v[1], b1 = st->opt_av[0], b2 = st->opt_av[1];
        dv = __dsub_rn(v2, __ddiv_rn(__dmul_rn(__dsub_rn(b2, vol_target), __dsub_rn(v2, v1)), __dsub_rn(b2, b1)));
        if (dr > 1.0) dr = 1.0;
        if (dr <= 0.0) {
          dr = -dr;
          if (dr > 1.0) dr = __ddiv_rn(d2, 2.0);
        }
        if (dv <= 0.0) {
          dv = -dv;
          if (dv > 0.1) dv = __ddiv_rn(v2, 2.0);
        }
        st->opt_v[0] = v2;
        st->opt_av[0] = b2;
      } else {
        if (dr > 1.0) {
          dr = 1.0;
        } else if (dr <= 0.0) {
          dr = -dr;
          if (dr > 1.0) dr = __ddiv_rn(d2, 2.0);
        }
      }
      st->opt_d[0] = d2;
      st->opt_a[0] = a2;
    }
  }
  st->dr_max = dr;
  st->dv_max = dv;
}

void launch_opt_step(const SysPtrs &p, int j, int n_samples, unsigned long long sweep_moves, double part_target,
                     double vol_target, bool npt, cudaStream_t s) {
  k_opt_step<<<1, 1, 0, s>>>(p.st, j, n_samples, sweep_moves, part_target, vol_target, npt ? 1 : 0);
}

__global__ void k_fill_u32(uint32_t *p, int n, uint32_t v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

void launch_fill_u32(uint32_t *p, int n, uint32_t v, cudaStream_t s) {
  int blocks = (n + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  k_fill_u32<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(p, n, v);
}

// ------------------------------------------------------------ volume move
// vol_move (src/moves.c:83-153) as four launches so it stays on the device:
// propose (1 thread), scaled overlap scan (N threads, early exit once an
// overlap is seen), decide and rebuild the box (1 thread), rescale (N threads).

// ln V' = ln V + (u - 1/2) dv_max; sf = (V'/V)^(1/3).
__global__ void k_vol_propose(SysPtrs p, long long offset) {
  DevState *st = p.st;
  const Box *bx = p.box;
  const unsigned long long s = st->sweep_base + (unsigned long long)offset;
  const U32x4 r = draw4(st->seed, 0u, 0u, s, TAG_VOLUME);
  double vol_new, ratio, sf;
  vol_proposal(bx->vol, r.x, st->dv_max, vol_new, ratio, sf);
  st->vol_sf = sf;
  st->vol_new = vol_new;
  st->vol_ratio = ratio;
  st->vol_u_acc = open_unit(r.y);
  st->vol_overlap = 0;
  st->vol_accept = 0;
  st->vol_moves += 1;
}

// check_overlap(i, sf, sf, sf) for every i (src/moves.c:104-112); an
// expansion clear of 1 needs no scan (vol_scan_needed).
__global__ void __launch_bounds__(256) k_vol_scan(SysPtrs p) {
  const DevState *st = p.st;
  const double sf = st->vol_sf;
  const Box *bx = p.box;
  if (!vol_scan_needed(sf, bx->len)) return;
  if (*(volatile const int *)&st->vol_overlap) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int layout = (int)(st->params.sweep & 1ull);
  const int *cnt = cnt_of(p, layout);
  const Slot *slot = slot_of(p, layout);
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const float L32[3] = {bx->len32[0], bx->len32[1], bx->len32[2]};
  const float iw[3] = {bx->inv_w32[0], bx->inv_w32[1], bx->inv_w32[2]};
  const float sh[3] = {st->params.shift32[0], st->params.shift32[1], st->params.shift32[2]};
  const int nc[3] = {bx->nc[0], bx->nc[1], bx->nc[2]};
  const float reach = (float)(1.0 / sf) + 1e-3f;
  const float sf2f = (float)(sf * sf);
  const float lo = 1.0f - 2.0f * bx->band, hi = 1.0f + 2.0f * bx->band;
  double x, y, z;
  load_xyz(p.pos, i, x, y, z);
  const float xr[3] = {__double2float_rn(x), __double2float_rn(y), __double2float_rn(z)};
  float xs[3];  // grid coordinates, as the slots hold them
  int ci[3], k[3];
  for (int d = 0; d < 3; d++) {
    axis_cell(xr[d], sh[d], L32[d], iw[d], nc[d], ci[d], xs[d]);
    k[d] = (int)ceilf(reach * iw[d] * 1.0001f);
    if (2 * k[d] + 1 > nc[d]) k[d] = -1;
  }
  bool ov = false;
  for (int a = (k[2] < 0 ? 0 : -k[2]); !ov && a <= (k[2] < 0 ? nc[2] - 1 : k[2]); a++) {
    const int cz = k[2] < 0 ? a : (ci[2] + a + nc[2]) % nc[2];
    for (int b = (k[1] < 0 ? 0 : -k[1]); !ov && b <= (k[1] < 0 ? nc[1] - 1 : k[1]); b++) {
      const int cy = k[1] < 0 ? b : (ci[1] + b + nc[1]) % nc[1];
      for (int e = (k[0] < 0 ? 0 : -k[0]); !ov && e <= (k[0] < 0 ? nc[0] - 1 : k[0]); e++) {
        const int cx = k[0] < 0 ? e : (ci[0] + e + nc[0]) % nc[0];
        const int c = cx + nc[0] * (cy + nc[1] * cz);
        const int m = cnt[c];
        const int n = m < p.cap ? m : p.cap;
        for (int q = 0; q < n && !ov; q++) {
          const Slot o = slot[(size_t)c * p.cap + q];
          if (o.id == i) continue;
          float dx = xs[0] - o.x, dy = xs[1] - o.y, dz = xs[2] - o.z;
          dx -= L32[0] * rintf(dx / L32[0]);
          dy -= L32[1] * rintf(dy / L32[1]);
          dz -= L32[2] * rintf(dz / L32[2]);
          const float r2f = dx * dx + dy * dy + dz * dz;
          if (r2f > reach * reach) continue;
          // the scaled single-precision r^2 decides outside twice the guard
          // band of contact; inside it the reference's scaled FP64 distance
          const float est = r2f * sf2f;
          if (est < lo) {
            ov = true;
            continue;
          }
          if (est > hi) continue;
          double ox, oy, oz;
          load_xyz(p.pos, o.id, ox, oy, oz);
          if (ref_r2_scaled(x, y, z, ox, oy, oz, len, sf) < 1.0) ov = true;
        }
      }
    }
  }
  if (ov) atomicOr(&p.st->vol_overlap, 1);
}

// Acceptance exp(beta P (V - V') + (N + 1) ln(V'/V)) against a fresh uniform
// (src/moves.c:114-127); on acceptance the box is rebuilt from the lattice
// counts and the new density (src/moves.c:128-132) and the device grid is
// re-derived for it.
__global__ void k_vol_decide(SysPtrs p, double margin) {
  DevState *st = p.st;
  Box *bx = p.box;
  if (st->vol_overlap) return;
  const double boltz = vol_boltz(st->pressure, bx->vol, st->vol_new, p.n, st->vol_ratio);
  if (st->vol_u_acc >= boltz) return;
  Box nb = *bx;
  if (!vol_rebuild_box(st, p.n, st->vol_new, margin, nb)) {
    atomicOr(&st->status, ST_BAD_CELL);
    return;
  }
  *bx = nb;
  st->vol_accept = 1;
  st->vol_acc += 1;
}

// Positions scaled by sf and wrapped into the new box (src/moves.c:133-140).
__global__ void __launch_bounds__(256) k_vol_apply(SysPtrs p) {
  const DevState *st = p.st;
  if (!st->vol_accept) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double sf = st->vol_sf;
  const Box *bx = p.box;
  double *q = p.pos + 4 * (size_t)i;
  for (int d = 0; d < 3; d++) {
    double v = __dmul_rn(q[1 + d], sf);
    if (gt_pos(v, bx->len[d])) v = __dsub_rn(v, bx->len[d]);
    else if (lt_zero(v)) v = __dadd_rn(v, bx->len[d]);
    q[1 + d] = v;
  }
}

void launch_volume_scan(const SysPtrs &p, cudaStream_t s) {
  const int blocks = (p.n + 255) / 256;
  k_vol_scan<<<blocks, 256, 0, s>>>(p);
}

void launch_volume_move(const SysPtrs &p, long long sweep_offset, double margin, cudaStream_t s) {
  const int blocks = (p.n + 255) / 256;
  k_vol_propose<<<1, 1, 0, s>>>(p, sweep_offset);
  k_vol_scan<<<blocks, 256, 0, s>>>(p);
  k_vol_decide<<<1, 1, 0, s>>>(p, margin);
  k_vol_apply<<<blocks, 256, 0, s>>>(p);
}

// ------------------------------------------------------------------ launch

// The checks of hsmc_gpu_upload_config on the device, where the copied
// array is read at HBM speed (a host loop over it took about as long as 4 %
// of the sweeps between an upload and a download).
__global__ void __launch_bounds__(256) k_check_config(SysPtrs p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double2 a = *reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i);
  const double2 b = *reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i + 2);
  const Box *bx = p.box;
  if (a.x != (double)i) atomicOr(&p.st->status, ST_BAD_ID);
  if (!(a.y >= 0.0 && a.y <= bx->len[0]) || !(b.x >= 0.0 && b.x <= bx->len[1]) || !(b.y >= 0.0 && b.y <= bx->len[2]))
    atomicOr(&p.st->status, ST_OUT_OF_BOX);
}

void launch_check_config(const SysPtrs &p, cudaStream_t s) {
  k_check_config<<<(p.n + 255) / 256 > 0 ? (p.n + 255) / 256 : 1, 256, 0, s>>>(p);
}

// An ordinary launch: as a programmatic dependent of the last colour pass
// (its blocks resident early, waiting for the pass's positions) the sweep
// measured 1.7 % slower.
void launch_build(const SysPtrs &p, long long sweep_offset, int num_sms, cudaStream_t s) {
  (void)num_sms;
  const int blocks = (p.n + 255) / 256;
  k_build<false><<<blocks > 0 ? blocks : 1, 256, 0, s>>>(p, nullptr, nullptr, 0, sweep_offset);
}

// Batched replicas (hsmc_batch schedule 3): one list per pass over every
// replica of one cell capacity.  A replica's cells of the colour that its
// own colour order moves in pass k go to list k as (replica within the
// class, cell) pairs, fullest first; bins are pass * 32 + occupancy - 1.
// cstart: prefix sums of the class's replicas' cells.  The counts (ocnt, the
// words of SysPtrs::ocnt) are cleared before k_border_count.
//
// What a thread needs of the replica holding its cells: the replica's end
// in the class's cell numbering, its current counts and grid, and the pass
// that moves each colour (4 bits per colour).  A thread's cells are
// consecutive, so it looks a replica up once, and again only when its cells
// cross into the next one.
struct OrderRep {
  int r = -1, first = 0, end = 0, nc0 = 1, nc1 = 1;
  const int *cnt = nullptr;
  uint32_t pass_of = 0;
};

__device__ __forceinline__ void order_rep(const SysPtrs *reps, const int *cstart, int n_reps, int x, OrderRep &v) {
  v.r = find_rep(cstart, n_reps, x);
  v.first = __ldg(cstart + v.r);
  v.end = __ldg(cstart + v.r + 1);
  const DevState *st = reps[v.r].st;
  v.cnt = (st->params.sweep & 1ull) ? reps[v.r].cnt[1] : reps[v.r].cnt[0];
  v.nc0 = reps[v.r].box->nc[0];
  v.nc1 = reps[v.r].box->nc[1];
  v.pass_of = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) v.pass_of |= (uint32_t)k << (4 * st->params.perm[k]);
}

// Bin of flat cell x of the class (pass * 32 + min(n, 32) - 1), or -1 for an
// empty cell or one beyond the class; r and c: its replica and cell.
__device__ __forceinline__ int batch_order_bin(const SysPtrs *reps, const int *cstart, int n_reps, int n_cells, int x,
                                               OrderRep &v, int &r, int &c) {
  if (x >= n_cells) return -1;
  if (v.r < 0 || x >= v.end) order_rep(reps, cstart, n_reps, x, v);
  r = v.r;
  c = x - v.first;
  const int n = v.cnt[c];
  if (n <= 0) return -1;
  const int iyz = c / v.nc0;
  const int colour = cell_colour(c - iyz * v.nc0, iyz % v.nc1, iyz / v.nc1);
  return 32 * (int)((v.pass_of >> (4 * colour)) & 7u) + (n < 32 ? n : 32) - 1;
}

__global__ void __launch_bounds__(kOrderThreads) k_border_count(const SysPtrs *reps, const int *cstart, int n_reps,
                                                                int *ocnt) {
  __shared__ int h[256];
  const int tid = (int)threadIdx.x;
  h[tid] = 0;
  __syncthreads();
  const int n_cells = __ldg(cstart + n_reps);
  const int x0 = (blockIdx.x * kOrderThreads + tid) * kOrderPerThread;
  OrderRep v;
#pragma unroll
  for (int k = 0; k < kOrderPerThread; k++) {
    int r, c;
    const int b = batch_order_bin(reps, cstart, n_reps, n_cells, x0 + k, v, r, c);
    if (b >= 0) atomicAdd(&h[b], 1);
  }
  __syncthreads();
  if (h[tid]) atomicAdd(&ocnt[tid], h[tid]);
}

__global__ void __launch_bounds__(kOrderThreads) k_border_scatter(const SysPtrs *reps, const int *cstart, int n_reps,
                                                                  int *ocnt, int *olist, int stride) {
  __shared__ int h[256], tot[256], start[256];
  const int tid = (int)threadIdx.x;
  h[tid] = 0;
  tot[tid] = ocnt[tid];
  __syncthreads();
  if (blockIdx.x == 0 && tid < 8) {
    int t = 0;
    for (int m = 0; m < 32; m++) t += tot[32 * tid + m];
    ocnt[512 + tid] = t;
  }
  const int n_cells = __ldg(cstart + n_reps);
  const int x0 = (blockIdx.x * kOrderThreads + tid) * kOrderPerThread;
  OrderRep v;
  int bin[kOrderPerThread], at[kOrderPerThread], rr[kOrderPerThread], cc[kOrderPerThread];
#pragma unroll
  for (int k = 0; k < kOrderPerThread; k++) {
    bin[k] = batch_order_bin(reps, cstart, n_reps, n_cells, x0 + k, v, rr[k], cc[k]);
    at[k] = bin[k] >= 0 ? atomicAdd(&h[bin[k]], 1) : 0;
  }
  __syncthreads();
  if (h[tid]) {
    int first = 0;
    for (int m = (tid & 31) + 1; m < 32; m++) first += tot[(tid & ~31) + m];
    start[tid] = first + atomicAdd(&ocnt[256 + tid], h[tid]);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kOrderPerThread; k++)
    if (bin[k] >= 0) {
      const size_t e = (size_t)(bin[k] >> 5) * (size_t)stride + (size_t)(start[bin[k]] + at[k]);
      olist[2 * e] = rr[k];
      olist[2 * e + 1] = cc[k];
    }
}

void launch_order_batch(const SysPtrs *reps, const int *cstart, int n_reps, long long n_cells, int *ocnt,
                        int *olist, int stride, cudaStream_t s) {
  const long long per_block = kOrderThreads * kOrderPerThread;
  const int blocks = (int)((n_cells + per_block - 1) / per_block);
  cudaMemsetAsync(ocnt, 0, sizeof(int) * (size_t)kOrderWords, s);
  k_border_count<<<blocks > 0 ? blocks : 1, kOrderThreads, 0, s>>>(reps, cstart, n_reps, ocnt);
  k_border_scatter<<<blocks > 0 ? blocks : 1, kOrderThreads, 0, s>>>(reps, cstart, n_reps, ocnt, olist, stride);
}

// Both order kernels are programmatic dependents (each waits at its start
// for the kernel before it), so their launches overlap that kernel's end.
void launch_order(const SysPtrs &p, cudaStream_t s) {
  const int cells_per_block = kOrderThreads * kOrderPerThread;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((p.ncell_alloc + cells_per_block - 1) / cells_per_block));
  cfg.blockDim = dim3(kOrderThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_order_count, p);
  cudaLaunchKernelEx(&cfg, k_order_scatter, p);
}

void launch_build_batch(const SysPtrs *reps, const int *nstart, int n_reps, int tot_n, long long sweep_offset,
                        cudaStream_t s) {
  k_build<true><<<(tot_n + 255) / 256, 256, 0, s>>>(SysPtrs{}, reps, nstart, n_reps, sweep_offset);
}

__global__ void k_advance_batch(const SysPtrs *reps, int n_reps, int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n_reps) reps[r].st->sweep_base += (unsigned long long)n;
}

void launch_advance_batch(const SysPtrs *reps, int n_reps, int n_sweeps, cudaStream_t s) {
  k_advance_batch<<<(n_reps + 127) / 128, 128, 0, s>>>(reps, n_reps, n_sweeps);
}

void launch_advance(const SysPtrs &p, int n_sweeps, cudaStream_t s) { k_advance<<<1, 1, 0, s>>>(p.st, n_sweeps); }

}  // namespace hsmc
