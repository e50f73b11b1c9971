// Geometric cluster moves (cluster_move, cluster_move_part, rotate,
// pocket_add; src/cluster_nvt.c:232-410) grown breadth-first over the GPU.
//
// The reference moves a seed particle by a rotation of pi about a line along
// a coordinate axis through a random pivot, then repeatedly takes a random
// particle of its "pocket" (particles overlapping a moved one), moves it and
// adds the particles it now overlaps.  The rotation is an isometry of the
// periodic box, so two moved particles never overlap each other and the set
// of moved particles is the connected component of the seed in the graph
// "j overlaps the image of i": the order in which the pocket is emptied
// changes neither the set nor any moved position.  The device therefore
// grows the cluster level by level, several moves in one cooperative launch:
//   - a warp takes one particle of the current level, computes its image with
//     the reference's rotate() arithmetic and single periodic wrap, writes it,
//     and tests the 27 cells around the image (one lane per cell) against the
//     particles not yet taken, with the reference's FP64 distance;
//   - a particle found overlapping is claimed by an atomic exchange of its
//     mark word (the move's epoch), so it enters the next level once;
//   - levels are separated by a grid-wide barrier whose wait is bounded.
// Particles not yet taken keep their old positions in the current cell
// layout, which is the only layout the search reads; after each move the
// launch rebuilds that layout from the moved positions.
#include "cellview.cuh"

namespace hsmc {

namespace {

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile_int(const int *p) { return *(const volatile int *)p; }

// All blocks of the (cooperative) launch meet here.  Arrivals count up in
// *arrive; the phase-th meeting waits for phase * gridDim.x arrivals.  The
// wait is bounded at 1 s: then ST_CLUSTER_TIMEOUT is raised and every block
// leaves at its next meeting.  Returns false when the search must stop.
__device__ bool grid_meet(uint32_t *arrive, uint32_t phase, int *status) {
  __shared__ int ok;
  __syncthreads();
  if (gridDim.x == 1) return true;  // one block: the block barrier is the meeting
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(arrive, 1u);
    const uint32_t target = phase * gridDim.x;
    int good = 1;
    uint64_t t0;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t0));
    while ((int)(ld_acquire_u32(arrive) - target) < 0) {
      if (ld_volatile_int(status) & ST_CLUSTER_TIMEOUT) {
        good = 0;
        break;
      }
      uint64_t t;
      asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
      if (t - t0 > 1000000000ull) {
        atomicOr(status, ST_CLUSTER_TIMEOUT);
        good = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// rotate() (src/cluster_nvt.c:342-365) by theta = pi about the line through
// the pivot a along a coordinate axis, with cos(pi) = -1 and s = sin(M_PI).
// In the reference's expression the terms multiplied by the axis components
// 0 and 1 and by 1 - cos = 2 are exact, so they fold away without changing
// the result, signed zeros included: the axis coordinate is unchanged and a
// perpendicular coordinate c becomes (2 a_c - c) + (a_o - o) s or
// (2 a_c - c) + (o - a_o) s, o being the other perpendicular coordinate.
// Four FP64 operations per perpendicular axis instead of thirty-odd;
// two_piv = 2 * pivot.
__device__ __forceinline__ void reflect_axis(double xx, double yy, double zz, const double *piv,
                                             const double *two_piv, int axis, double sint, double &xr, double &yr,
                                             double &zr) {
  if (axis == 0) {
    xr = xx;
    yr = __dadd_rn(__dsub_rn(two_piv[1], yy), __dmul_rn(__dsub_rn(piv[2], zz), sint));
    zr = __dadd_rn(__dsub_rn(two_piv[2], zz), __dmul_rn(__dsub_rn(yy, piv[1]), sint));
  } else if (axis == 1) {
    xr = __dadd_rn(__dsub_rn(two_piv[0], xx), __dmul_rn(__dsub_rn(zz, piv[2]), sint));
    yr = yy;
    zr = __dadd_rn(__dsub_rn(two_piv[2], zz), __dmul_rn(__dsub_rn(piv[0], xx), sint));
  } else {
    xr = __dadd_rn(__dsub_rn(two_piv[0], xx), __dmul_rn(__dsub_rn(piv[1], yy), sint));
    yr = __dadd_rn(__dsub_rn(two_piv[1], yy), __dmul_rn(__dsub_rn(xx, piv[0]), sint));
    zr = zz;
  }
}

// Single-precision squared minimum-image distance of two points given in
// box coordinates, for discarding far pairs before the FP64 test.
__device__ __forceinline__ float screen_r2(float ax, float ay, float az, float bx, float by, float bz,
                                           const float *L32) {
  float d[3] = {ax - bx, ay - by, az - bz};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if (d[k] > 0.5f * L32[k]) d[k] -= L32[k];
    else if (d[k] < -0.5f * L32[k]) d[k] += L32[k];
  }
  return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
}

// apply_pbc (src/moves.c:215-226): one wrap per axis.
__device__ __forceinline__ double wrap_once(double v, double len) {
  if (v > len) return __dsub_rn(v, len);
  if (v < 0.0) return __dadd_rn(v, len);
  return v;
}

// One grid-stride pass of k_build (sweep.cu) over the positions, into the
// current layout with its shift: the layout of the moved configuration.
__device__ void rebin(const SysPtrs &p, const CellView &v, int *cnt, Slot *slot) {
  const Box *bx = p.box;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x) {
    const double2 a = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i));
    const double2 b = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i + 2));
    int cx, cy, cz;
    float tx, ty, tz;
    axis_cell(__double2float_rn(a.y), v.sh[0], bx->len32[0], bx->inv_w32[0], bx->nc[0], cx, tx);
    axis_cell(__double2float_rn(b.x), v.sh[1], bx->len32[1], bx->inv_w32[1], bx->nc[1], cy, ty);
    axis_cell(__double2float_rn(b.y), v.sh[2], bx->len32[2], bx->inv_w32[2], bx->nc[2], cz, tz);
    const int c = cx + bx->nc[0] * (cy + bx->nc[1] * cz);
    const int k = atomicAdd(cnt + c, 1);
    if (k < p.cap) slot[(size_t)c * p.cap + k] = Slot{tx, ty, tz, i};
    else atomicOr(&p.st->status, ST_CELL_OVERFLOW);
  }
}

// n_moves consecutive cluster moves in one cooperative launch.  Every read
// of data that this launch writes (positions, cells, queue, marks) goes
// through L2 (ld.global.cg): the L1 of another SM may hold stale lines.
__global__ void __launch_bounds__(512) k_cluster(SysPtrs p, ClusterJob job, int n_moves) {
  const CellView v = current_view(p);
  int *cnt = const_cast<int *>(v.cnt);
  Slot *slots = const_cast<Slot *>(v.slot);
  const Box *bx = p.box;
  double len[3], half[3];
  for (int d = 0; d < 3; d++) {
    len[d] = bx->len[d];
    half[d] = bx->half[d];
  }
  int *status = &p.st->status;
  const float band = bx->band;  // bound on the single-precision error of r^2
  const int lane = (int)(threadIdx.x & 31);
  const int wid = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nw = (int)((gridDim.x * blockDim.x) >> 5);
  const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;  // lane -> one of 27 cells
  uint32_t phase = 0;

  for (int m = 0; m < n_moves; m++) {
    const uint32_t epoch = job.epoch + (uint32_t)m;
    // pivot (three uniforms times the box side), axis and seed particle
    double piv[3];
    int axis, seed_id;
    if (job.given) {
      piv[0] = job.pivot[0];
      piv[1] = job.pivot[1];
      piv[2] = job.pivot[2];
      axis = job.axis;
      seed_id = job.seed_id;
    } else {
      const unsigned long long rs = p.st->seed, seq = job.seq + (unsigned long long)m;
      const U32x4 r1 = draw4(rs, 0u, 0u, seq, TAG_CLUSTER);
      const U32x4 r2 = draw4(rs, 1u, 0u, seq, TAG_CLUSTER);
      piv[0] = __dmul_rn(open_unit(r1.x), len[0]);
      piv[1] = __dmul_rn(open_unit(r1.y), len[1]);
      piv[2] = __dmul_rn(open_unit(r1.z), len[2]);
      axis = (int)__umulhi(r1.w, 3u);
      seed_id = (int)__umul64hi(((unsigned long long)r2.x << 32) | r2.y, (unsigned long long)p.n);
    }
    const double two_piv[3] = {__dmul_rn(2.0, piv[0]), __dmul_rn(2.0, piv[1]), __dmul_rn(2.0, piv[2])};
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      job.ctr[0] = job.ctr[1] = job.ctr[2] = 0u;
      job.queue[0] = seed_id;
      atomicExch(job.mark + seed_id, epoch);
      if (job.drawn) {
        double *dm = job.drawn + 5 * (size_t)m;
        dm[0] = piv[0];
        dm[1] = piv[1];
        dm[2] = piv[2];
        dm[3] = (double)axis;
        dm[4] = (double)seed_id;
      }
    }
    if (!grid_meet(job.ctr + 3, ++phase, status)) return;

    long long base = 0;
    int ncur = 1;
    int level = 0;
    while (ncur > 0) {
      const long long next = base + ncur;
      uint32_t *push = job.ctr + (level + 1) % 3;
      // On a small grid, the level's images first, one thread per particle
      // (a warp's FP64 sequence serves 32 particles; the SMs' FP64 pipes are
      // the bottleneck there), then a meeting so every block sees them.  On
      // a large grid the extra meeting costs more than it saves: each search
      // warp computes its own particle's image.
      const bool split = gridDim.x <= 4;
      for (int k = (int)(blockIdx.x * blockDim.x + threadIdx.x); split && k < ncur;
           k += (int)(gridDim.x * blockDim.x)) {
        const int i = __ldcg(job.queue + base + k);
        const double2 a0 = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i));
        const double2 b0 = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i + 2));
        double px, py, pz;
        reflect_axis(a0.y, b0.x, b0.y, piv, two_piv, axis, job.sint, px, py, pz);
        double *q = p.pos + 4 * (size_t)i;
        q[1] = wrap_once(px, len[0]);
        q[2] = wrap_once(py, len[1]);
        q[3] = wrap_once(pz, len[2]);
      }
      if (split && !grid_meet(job.ctr + 3, ++phase, status)) return;
      // one warp per particle, lane k on neighbour cell k of its image; the
      // level's particles are all marked, so no search reads their images
      for (int k = wid; k < ncur; k += nw) {
        const int i = __ldcg(job.queue + base + k);
        const double2 a0 = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i));
        const double2 b0 = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i + 2));
        double px = a0.y, py = b0.x, pz = b0.y;
        if (!split) {
          reflect_axis(a0.y, b0.x, b0.y, piv, two_piv, axis, job.sint, px, py, pz);
          px = wrap_once(px, len[0]);
          py = wrap_once(py, len[1]);
          pz = wrap_once(pz, len[2]);
          __syncwarp();
          if (lane == 0) {
            double *q = p.pos + 4 * (size_t)i;
            q[1] = px;
            q[2] = py;
            q[3] = pz;
          }
        }
        if (lane < 27) {
          int ci[3];
          float t[3];
          axis_cell(__double2float_rn(px), v.sh[0], v.L32[0], v.iw[0], v.nc[0], ci[0], t[0]);
          axis_cell(__double2float_rn(py), v.sh[1], v.L32[1], v.iw[1], v.nc[1], ci[1], t[1]);
          axis_cell(__double2float_rn(pz), v.sh[2], v.L32[2], v.iw[2], v.nc[2], ci[2], t[2]);
          int cx = ci[0] + ox, cy = ci[1] + oy, cz = ci[2] + oz;
          cx = cx < 0 ? cx + v.nc[0] : (cx >= v.nc[0] ? cx - v.nc[0] : cx);
          cy = cy < 0 ? cy + v.nc[1] : (cy >= v.nc[1] ? cy - v.nc[1] : cy);
          cz = cz < 0 ? cz + v.nc[2] : (cz >= v.nc[2] ? cz - v.nc[2] : cz);
          const int c = cx + v.nc[0] * (cy + v.nc[1] * cz);
          const int mc = __ldcg(cnt + c);
          const int nq = mc < v.cap ? mc : v.cap;
          const float4 *sl = reinterpret_cast<const float4 *>(slots + (size_t)c * v.cap);
          for (int q = 0; q < nq; q++) {
            const float4 f = __ldcg(sl + q);
            const Slot o{f.x, f.y, f.z, __float_as_int(f.w)};
            if (o.id == i) continue;
            const float r2 = approx_r2(t[0], t[1], t[2], o, v.L32);
            if (r2 > 1.0f + band) continue;
            if (__ldcg(job.mark + o.id) == epoch) continue;
            // pocket_add: compute_dist(moved, other) < 1.0 (src/cluster_nvt.c:371-410), in
            // FP64 when the single-precision value is within the guard band of 1
            bool ov = r2 < 1.0f - band;
            if (!ov) {
              const double2 a = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)o.id));
              const double2 b = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)o.id + 2));
              ov = ref_r2(px, py, pz, a.y, b.x, b.y, len, half) < 1.0;
            }
            if (ov) {
              if (atomicExch(job.mark + o.id, epoch) != epoch) {
                const uint32_t slot = atomicAdd(push, 1u);
                job.queue[next + slot] = o.id;
              }
            }
          }
        }
      }
      // the counter two levels ahead was last read at the start of this one
      if (blockIdx.x == 0 && threadIdx.x == 0) job.ctr[(level + 2) % 3] = 0u;
      if (!grid_meet(job.ctr + 3, ++phase, status)) return;
      ncur = (int)__ldcg(push);
      base = next;
      level++;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) job.size_out[m] = base;
    // the moved configuration's layout
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x) cnt[c] = 0;
    if (!grid_meet(job.ctr + 3, ++phase, status)) return;
    rebin(p, v, cnt, slots);
    if (!grid_meet(job.ctr + 3, ++phase, status)) return;
  }
}

// ------------------------------------------------ small systems, one block
// The whole system in shared memory: FP64 positions and their FP32 roundings
// (the screen and the cell index read only these, so a level's FP64 work is
// the image of each particle), a cell list by counting sort (start offsets +
// ids), marks and the queue.  The same moves as
// k_cluster (same draws, same set, same images), with shared-memory latency
// instead of L2 round trips between the dependent steps of a level.
struct SmallSm {
  double *x, *y, *z;
  float *x32, *y32, *z32;
  uint32_t *mark, *start, *fill;
  uint16_t *ids, *queue;
  uint32_t *pc;  // [0..2] rotating level counters, [3] scan carry
};

__device__ __forceinline__ SmallSm small_sm(unsigned char *raw, int n, int ncell) {
  SmallSm m;
  m.x = reinterpret_cast<double *>(raw);
  m.y = m.x + n;
  m.z = m.y + n;
  m.x32 = reinterpret_cast<float *>(m.z + n);
  m.y32 = m.x32 + n;
  m.z32 = m.y32 + n;
  m.mark = reinterpret_cast<uint32_t *>(m.z32 + n);
  m.start = m.mark + n;
  m.fill = m.start + (ncell + 1);
  m.pc = m.fill + ncell;
  m.ids = reinterpret_cast<uint16_t *>(m.pc + 4);
  m.queue = m.ids + n;
  return m;
}

__device__ __forceinline__ int small_cell(const Box *bx, float x, float y, float z) {
  int c[3];
  float t;
  axis_cell(x, 0.0f, bx->len32[0], bx->inv_w32[0], bx->nc[0], c[0], t);
  axis_cell(y, 0.0f, bx->len32[1], bx->inv_w32[1], bx->nc[1], c[1], t);
  axis_cell(z, 0.0f, bx->len32[2], bx->inv_w32[2], bx->nc[2], c[2], t);
  return c[0] + bx->nc[0] * (c[1] + bx->nc[1] * c[2]);
}

// Counting sort of the particles into cells (start[c] .. start[c + 1]).
__device__ void small_cells(const SmallSm &m, const Box *bx, int n, int ncell) {
  const int tid = (int)threadIdx.x, nt = (int)blockDim.x;
  for (int c = tid; c < ncell; c += nt) m.fill[c] = 0u;
  __syncthreads();
  for (int i = tid; i < n; i += nt) atomicAdd(m.fill + small_cell(bx, m.x32[i], m.y32[i], m.z32[i]), 1u);
  __syncthreads();
  // exclusive scan of fill into start: a contiguous chunk per thread, then
  // a block scan of the chunk sums
  const int per = (ncell + nt - 1) / nt;
  const int c0 = tid * per, c1 = min(c0 + per, ncell);
  uint32_t sum = 0;
  for (int c = c0; c < c1; c++) sum += m.fill[c];
  const int lane = tid & 31, w = tid >> 5;
  uint32_t inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  __shared__ uint32_t wsum[32];
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t v = lane < (nt >> 5) ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    wsum[lane] = v;  // inclusive over warps
  }
  __syncthreads();
  uint32_t run = (w ? wsum[w - 1] : 0u) + inc - sum;
  for (int c = c0; c < c1; c++) {
    m.start[c] = run;
    run += m.fill[c];
  }
  if (tid == nt - 1) m.start[ncell] = (uint32_t)n;
  __syncthreads();
  for (int c = tid; c < ncell; c += nt) m.fill[c] = 0u;
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    const int c = small_cell(bx, m.x32[i], m.y32[i], m.z32[i]);
    const uint32_t k = atomicAdd(m.fill + c, 1u);
    m.ids[m.start[c] + k] = (uint16_t)i;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(512) k_cluster_small(SysPtrs p, ClusterJob job, int n_moves) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Box *bx = p.box;
  const int n = p.n, ncell = bx->ncell;
  const SmallSm m = small_sm(smem_raw, n, ncell);
  double len[3], half[3];
  for (int d = 0; d < 3; d++) {
    len[d] = bx->len[d];
    half[d] = bx->half[d];
  }
  const int nc0 = bx->nc[0], nc1 = bx->nc[1], nc2 = bx->nc[2];
  const float band = bx->band;  // bound on the single-precision error of r^2
  const int tid = (int)threadIdx.x, nt = (int)blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
  for (int i = tid; i < n; i += nt) {
    double x, y, z;
    load_xyz(p.pos, i, x, y, z);
    m.x[i] = x;
    m.y[i] = y;
    m.z[i] = z;
    m.x32[i] = __double2float_rn(x);
    m.y32[i] = __double2float_rn(y);
    m.z32[i] = __double2float_rn(z);
    m.mark[i] = 0u;
  }
  __syncthreads();
  small_cells(m, bx, n, ncell);

  for (int mv = 0; mv < n_moves; mv++) {
    const uint32_t epoch = (uint32_t)mv + 1u;
    double piv[3];
    int axis, seed_id;
    if (job.given) {
      piv[0] = job.pivot[0];
      piv[1] = job.pivot[1];
      piv[2] = job.pivot[2];
      axis = job.axis;
      seed_id = job.seed_id;
    } else {
      const unsigned long long rs = p.st->seed, seq = job.seq + (unsigned long long)mv;
      const U32x4 r1 = draw4(rs, 0u, 0u, seq, TAG_CLUSTER);
      const U32x4 r2 = draw4(rs, 1u, 0u, seq, TAG_CLUSTER);
      piv[0] = __dmul_rn(open_unit(r1.x), len[0]);
      piv[1] = __dmul_rn(open_unit(r1.y), len[1]);
      piv[2] = __dmul_rn(open_unit(r1.z), len[2]);
      axis = (int)__umulhi(r1.w, 3u);
      seed_id = (int)__umul64hi(((unsigned long long)r2.x << 32) | r2.y, (unsigned long long)n);
    }
    const double two_piv[3] = {__dmul_rn(2.0, piv[0]), __dmul_rn(2.0, piv[1]), __dmul_rn(2.0, piv[2])};
    if (tid == 0) {
      m.pc[0] = m.pc[1] = m.pc[2] = 0u;
      m.queue[0] = (uint16_t)seed_id;
      m.mark[seed_id] = epoch;
      if (job.drawn) {
        double *dm = job.drawn + 5 * (size_t)mv;
        dm[0] = piv[0];
        dm[1] = piv[1];
        dm[2] = piv[2];
        dm[3] = (double)axis;
        dm[4] = (double)seed_id;
      }
    }
    __syncthreads();
    int base = 0, ncur = 1, level = 0;
    while (ncur > 0) {
      const int next = base + ncur;
      uint32_t *push = m.pc + (level + 1) % 3;
      // the level's images, one thread per particle: a warp's FP64 sequence
      // serves 32 particles (the FP64 pipe is busy per warp instruction)
      for (int k = tid; k < ncur; k += nt) {
        const int i = m.queue[base + k];
        double px, py, pz;
        reflect_axis(m.x[i], m.y[i], m.z[i], piv, two_piv, axis, job.sint, px, py, pz);
        px = wrap_once(px, len[0]);
        py = wrap_once(py, len[1]);
        pz = wrap_once(pz, len[2]);
        m.x[i] = px;
        m.y[i] = py;
        m.z[i] = pz;
        m.x32[i] = __double2float_rn(px);
        m.y32[i] = __double2float_rn(py);
        m.z32[i] = __double2float_rn(pz);
      }
      __syncthreads();
      // then one warp per particle, lane k on neighbour cell k of its image;
      // the level's particles are all marked, so no search reads their images
      for (int k = wid; k < ncur; k += nw) {
        const int i = m.queue[base + k];
        const double px = m.x[i], py = m.y[i], pz = m.z[i];
        const float px32 = m.x32[i], py32 = m.y32[i], pz32 = m.z32[i];
        if (lane < 27) {
          int ci[3];
          float t;
          axis_cell(px32, 0.0f, bx->len32[0], bx->inv_w32[0], nc0, ci[0], t);
          axis_cell(py32, 0.0f, bx->len32[1], bx->inv_w32[1], nc1, ci[1], t);
          axis_cell(pz32, 0.0f, bx->len32[2], bx->inv_w32[2], nc2, ci[2], t);
          int cx = ci[0] + ox, cy = ci[1] + oy, cz = ci[2] + oz;
          cx = cx < 0 ? cx + nc0 : (cx >= nc0 ? cx - nc0 : cx);
          cy = cy < 0 ? cy + nc1 : (cy >= nc1 ? cy - nc1 : cy);
          cz = cz < 0 ? cz + nc2 : (cz >= nc2 ? cz - nc2 : cz);
          const int c = cx + nc0 * (cy + nc1 * cz);
          const uint32_t q1 = m.start[c + 1];
          for (uint32_t q = m.start[c]; q < q1; q++) {
            const int j = m.ids[q];
            if (j == i || m.mark[j] == epoch) continue;
            const float r2 = screen_r2(px32, py32, pz32, m.x32[j], m.y32[j], m.z32[j], bx->len32);
            if (r2 > 1.0f + band) continue;
            // pocket_add: compute_dist(moved, other) < 1.0 (src/cluster_nvt.c:371-410), in
            // FP64 when the single-precision value is within the guard band of 1
            const bool ov = r2 < 1.0f - band || ref_r2(px, py, pz, m.x[j], m.y[j], m.z[j], len, half) < 1.0;
            if (ov) {
              if (atomicExch(m.mark + j, epoch) != epoch) m.queue[next + atomicAdd(push, 1u)] = (uint16_t)j;
            }
          }
        }
      }
      if (tid == 0) m.pc[(level + 2) % 3] = 0u;
      __syncthreads();
      ncur = (int)*push;
      base = next;
      level++;
    }
    if (tid == 0) job.size_out[mv] = base;
    __syncthreads();
    small_cells(m, bx, n, ncell);
  }
  for (int i = tid; i < n; i += nt) {
    double *q = p.pos + 4 * (size_t)i;
    q[1] = m.x[i];
    q[2] = m.y[i];
    q[3] = m.z[i];
  }
}

}  // namespace

size_t cluster_small_smem(int n, int ncell) {
  if (n > 65535) return 0;
  // x, y, z (FP64 and FP32), mark, ids, queue per particle; start, fill per cell
  const size_t bytes = 44 * (size_t)n + 8 * (size_t)ncell + 4 + 16;
  return bytes <= 200 * 1024 ? bytes : 0;
}

int cluster_grid(int n, int ncell, int num_sms) {
  const size_t small = cluster_small_smem(n, ncell);
  if (small) {
    // the allowance is the kernel's, shared by every context on the device:
    // set to the most the device allows beside the kernel's static shared
    // memory, so a smaller system never lowers it below what an earlier,
    // larger one needs
    int dev = 0, optin = 0;
    cudaFuncAttributes fa{};
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess &&
        cudaFuncGetAttributes(&fa, k_cluster_small) == cudaSuccess &&
        small <= (size_t)(optin - (int)fa.sharedSizeBytes) &&
        cudaFuncSetAttribute(k_cluster_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - (int)fa.sharedSizeBytes) == cudaSuccess)
      return 0;  // the one-block shared-memory kernel
    cudaGetLastError();
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cluster, 512, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int resident = per_sm * num_sms;
  int want = (n + 2047) / 2048;  // about four particles per warp for a cluster of all of them
  if (want < 1) want = 1;
  return want < resident ? want : resident;
}

cudaError_t launch_cluster(const SysPtrs &p, const ClusterJob &job, int n_moves, int grid, int ncell,
                           cudaStream_t s) {
  if (grid == 0) {
    k_cluster_small<<<1, 512, cluster_small_smem(p.n, ncell), s>>>(p, job, n_moves);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(512);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_cluster, p, job, n_moves);
}

}  // namespace hsmc
