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
// grows the cluster level by level in one cooperative launch:
//   - a warp takes one particle of the current level, computes its image with
//     the reference's rotate() arithmetic and single periodic wrap, writes it,
//     and tests the 27 cells around the image (one lane per cell) against the
//     particles not yet taken, with the reference's FP64 distance;
//   - a particle found overlapping is claimed by an atomic exchange of its
//     mark word (the move's epoch), so it enters the next level once;
//   - levels are separated by a grid-wide barrier whose wait is bounded.
// Particles not yet taken keep their old positions in the current cell
// layout, which is the only layout the search reads; the caller rebuilds
// the layout after the move.
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

// rotate() (src/cluster_nvt.c:342-365) for the unit axis (uu, vv, ww)
// through (aa, bb, cc), in the reference's operation order without
// contraction; cost and sint are cos(M_PI) and sin(M_PI).
__device__ __forceinline__ void rotate_ref(double xx, double yy, double zz, double aa, double bb, double cc,
                                           double uu, double vv, double ww, double cost, double sint, double &xr,
                                           double &yr, double &zr) {
  const double uu2 = __dmul_rn(uu, uu), vv2 = __dmul_rn(vv, vv), ww2 = __dmul_rn(ww, ww);
  const double omc = __dsub_rn(1.0, cost);
  {
    const double s1 = __dsub_rn(
        __dsub_rn(__dsub_rn(__dadd_rn(__dmul_rn(bb, vv), __dmul_rn(cc, ww)), __dmul_rn(uu, xx)), __dmul_rn(vv, yy)),
        __dmul_rn(ww, zz));
    const double t1 = __dsub_rn(__dmul_rn(aa, __dadd_rn(vv2, ww2)), __dmul_rn(uu, s1));
    const double t2 =
        __dadd_rn(__dsub_rn(__dadd_rn(__dmul_rn(-cc, vv), __dmul_rn(bb, ww)), __dmul_rn(ww, yy)), __dmul_rn(vv, zz));
    xr = __dadd_rn(__dadd_rn(__dmul_rn(t1, omc), __dmul_rn(xx, cost)), __dmul_rn(t2, sint));
  }
  {
    const double s2 = __dsub_rn(
        __dsub_rn(__dsub_rn(__dadd_rn(__dmul_rn(aa, uu), __dmul_rn(cc, ww)), __dmul_rn(uu, xx)), __dmul_rn(vv, yy)),
        __dmul_rn(ww, zz));
    const double t3 = __dsub_rn(__dmul_rn(bb, __dadd_rn(uu2, ww2)), __dmul_rn(vv, s2));
    const double t4 =
        __dsub_rn(__dadd_rn(__dsub_rn(__dmul_rn(cc, uu), __dmul_rn(aa, ww)), __dmul_rn(ww, xx)), __dmul_rn(uu, zz));
    yr = __dadd_rn(__dadd_rn(__dmul_rn(t3, omc), __dmul_rn(yy, cost)), __dmul_rn(t4, sint));
  }
  {
    const double s3 = __dsub_rn(
        __dsub_rn(__dsub_rn(__dadd_rn(__dmul_rn(aa, uu), __dmul_rn(bb, vv)), __dmul_rn(uu, xx)), __dmul_rn(vv, yy)),
        __dmul_rn(ww, zz));
    const double t5 = __dsub_rn(__dmul_rn(cc, __dadd_rn(uu2, vv2)), __dmul_rn(ww, s3));
    const double t6 =
        __dadd_rn(__dsub_rn(__dadd_rn(__dmul_rn(-bb, uu), __dmul_rn(aa, vv)), __dmul_rn(vv, xx)), __dmul_rn(uu, yy));
    zr = __dadd_rn(__dadd_rn(__dmul_rn(t5, omc), __dmul_rn(zz, cost)), __dmul_rn(t6, sint));
  }
}

// apply_pbc (src/moves.c:215-226): one wrap per axis.
__device__ __forceinline__ double wrap_once(double v, double len) {
  if (v > len) return __dsub_rn(v, len);
  if (v < 0.0) return __dadd_rn(v, len);
  return v;
}

__global__ void __launch_bounds__(256) k_cluster(SysPtrs p, ClusterJob job) {
  const CellView v = current_view(p);
  const Box *bx = p.box;
  double len[3], half[3];
  for (int d = 0; d < 3; d++) {
    len[d] = bx->len[d];
    half[d] = bx->half[d];
  }
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
    const unsigned long long rs = p.st->seed;
    const U32x4 r1 = draw4(rs, 0u, 0u, job.seq, TAG_CLUSTER);
    const U32x4 r2 = draw4(rs, 1u, 0u, job.seq, TAG_CLUSTER);
    piv[0] = __dmul_rn(open_unit(r1.x), len[0]);
    piv[1] = __dmul_rn(open_unit(r1.y), len[1]);
    piv[2] = __dmul_rn(open_unit(r1.z), len[2]);
    axis = (int)__umulhi(r1.w, 3u);
    seed_id = (int)__umul64hi(((unsigned long long)r2.x << 32) | r2.y, (unsigned long long)p.n);
  }
  const double uu = axis == 0 ? 1.0 : 0.0, vv = axis == 1 ? 1.0 : 0.0, ww = axis == 2 ? 1.0 : 0.0;
  int *status = &p.st->status;
  const int lane = (int)(threadIdx.x & 31);
  const int wid = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nw = (int)((gridDim.x * blockDim.x) >> 5);

  if (blockIdx.x == 0 && threadIdx.x == 0) {
    job.queue[0] = seed_id;
    atomicExch(job.mark + seed_id, job.epoch);
    if (job.drawn) {
      job.drawn[0] = piv[0];
      job.drawn[1] = piv[1];
      job.drawn[2] = piv[2];
      job.drawn[3] = (double)axis;
      job.drawn[4] = (double)seed_id;
    }
  }
  uint32_t phase = 1;
  if (!grid_meet(job.ctr + 3, phase, status)) return;

  long long base = 0;
  int ncur = 1;
  int level = 0;
  // the 27 cells around an image: lane -> offsets in {-1, 0, 1}^3
  const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
  while (ncur > 0) {
    const long long next = base + ncur;
    uint32_t *push = job.ctr + (level + 1) % 3;
    for (int k = wid; k < ncur; k += nw) {
      const int i = __ldcg(job.queue + base + k);
      double x, y, z;
      load_xyz(p.pos, i, x, y, z);  // unchanged until this warp writes the image
      double px, py, pz;
      rotate_ref(x, y, z, piv[0], piv[1], piv[2], uu, vv, ww, job.cost, job.sint, px, py, pz);
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
        const int m = __ldg(v.cnt + c);
        const int nq = m < v.cap ? m : v.cap;
        const Slot *sl = v.slot + (size_t)c * v.cap;
        for (int q = 0; q < nq; q++) {
          const Slot o = sl[q];
          if (o.id == i) continue;
          if (approx_r2(t[0], t[1], t[2], o, v.L32) > 1.01f) continue;
          if (__ldcg(job.mark + o.id) == job.epoch) continue;
          const double2 a = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)o.id));
          const double2 b = __ldcg(reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)o.id + 2));
          // pocket_add: compute_dist(moved, other) < 1.0 (src/cluster_nvt.c:371-410)
          if (ref_r2(px, py, pz, a.y, b.x, b.y, len, half) < 1.0) {
            if (atomicExch(job.mark + o.id, job.epoch) != job.epoch) {
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
  if (blockIdx.x == 0 && threadIdx.x == 0) *job.size_out = base;
}

}  // namespace

int cluster_grid(int n, int num_sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cluster, 256, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int resident = per_sm * num_sms;
  int want = (n + 2047) / 2048;  // about eight particles per warp for a cluster of all of them
  if (want < 1) want = 1;
  return want < resident ? want : resident;
}

cudaError_t launch_cluster(const SysPtrs &p, const ClusterJob &job, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_cluster, p, job);
}

}  // namespace hsmc
