// Checkerboard sweep of the local-move hard-sphere Monte Carlo chain.
//
// One sweep = N trial moves, as sweep_nvt makes them (src/nvt.c:201-209), but
// organised for a GPU after Anderson, Jankowski, Grubb, Engel & Glotzer
// (J. Comput. Phys. 254, 27, 2013):
//   1. k_build bins every particle into a periodic grid of cells (edge > 1,
//      even count per axis) shifted by a fresh random vector: a counting sort
//      by atomic slot claims into fixed-capacity cells.
//   2. Eight k_move_pass launches, one per colour of the 2x2x2 checkerboard in
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
__global__ void __launch_bounds__(256) k_build(SysPtrs p, long long offset) {
  const DevState *st = p.st;
  const Box *bx = p.box;
  const unsigned long long s = st->sweep_base + (unsigned long long)offset;
  const unsigned long long seed = st->seed;
  const U32x4 rs = draw4(seed, 0u, 0u, s, TAG_SHIFT);
  const float w0 = bx->w32[0], w1 = bx->w32[1], w2 = bx->w32[2];
  const float sh0 = __fmul_rn(__uint2float_rn(rs.x >> 8) * 5.9604644775390625e-08f, w0);
  const float sh1 = __fmul_rn(__uint2float_rn(rs.y >> 8) * 5.9604644775390625e-08f, w1);
  const float sh2 = __fmul_rn(__uint2float_rn(rs.z >> 8) * 5.9604644775390625e-08f, w2);
  const int layout = (int)(s & 1ull);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    DevState *ws = p.st;
    ws->params.sweep = s;
    ws->params.shift32[0] = sh0;
    ws->params.shift32[1] = sh1;
    ws->params.shift32[2] = sh2;
    int perm[8] = {0, 1, 2, 3, 4, 5, 6, 7};
    const U32x4 ra = draw4(seed, 0u, 0u, s, TAG_PERM), rb = draw4(seed, 1u, 0u, s, TAG_PERM);
    const uint32_t r[7] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z};
    for (int k = 7; k >= 1; k--) {  // Fisher-Yates
      int j = (int)__umulhi(r[7 - k], (unsigned)(k + 1));
      int tmp = perm[k];
      perm[k] = perm[j];
      perm[j] = tmp;
    }
    for (int k = 0; k < 8; k++) ws->params.perm[k] = perm[k];
  }
  if (i >= p.n) return;
  const double2 a = *reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i);
  const double2 b = *reinterpret_cast<const double2 *>(p.pos + 4 * (size_t)i + 2);
  const float x32 = __double2float_rn(a.y), y32 = __double2float_rn(b.x), z32 = __double2float_rn(b.y);
  int cx, cy, cz;
  float t;
  axis_cell(x32, sh0, bx->len32[0], bx->inv_w32[0], bx->nc[0], cx, t);
  axis_cell(y32, sh1, bx->len32[1], bx->inv_w32[1], bx->nc[1], cy, t);
  axis_cell(z32, sh2, bx->len32[2], bx->inv_w32[2], bx->nc[2], cz, t);
  const int c = cx + bx->nc[0] * (cy + bx->nc[1] * cz);
  const int k = atomicAdd(p.cnt[layout] + c, 1);
  if (k < p.cap) {
    p.slot[layout][(size_t)c * p.cap + k] = Slot{x32, y32, z32, i};
  } else {
    atomicOr(&p.st->status, ST_CELL_OVERFLOW);
  }
}

// ------------------------------------------------------------- move pass

__device__ __forceinline__ void load_xyz(const double *pos, int id, double &x, double &y, double &z) {
  const double2 a = *reinterpret_cast<const double2 *>(pos + 4 * (size_t)id);
  const double2 b = *reinterpret_cast<const double2 *>(pos + 4 * (size_t)id + 2);
  x = a.y;
  y = b.x;
  z = b.y;
}

// Minimum-image difference of two single-precision coordinates in [0, L].
__device__ __forceinline__ float wrap_diff(float d, float len, float half) {
  if (d > half) d -= len;
  else if (d < -half) d += len;
  return d;
}

// Single-precision screen of one pair, with the FP64 re-evaluation (the
// reference's compute_dist arithmetic, mover first as in check_overlap) for
// pairs whose r^2 lies within the guard band of 1.
__device__ __forceinline__ bool screen_pair(float dx, float dy, float dz, float band, double mx, double my,
                                            double mz, const double *pos, int other, const double *len,
                                            const double *half, unsigned &rechecks) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  if (r2 < 1.0f - band) return true;
  if (r2 > 1.0f + band) return false;
  rechecks++;
  double ox, oy, oz;
  load_xyz(pos, other, ox, oy, oz);
  return ref_r2(mx, my, mz, ox, oy, oz, len, half) < 1.0;
}

// One colour pass.  A group of G lanes owns one active cell at a time; every
// lane keeps its own copy of the cell's particles (so the trial sequence
// needs no broadcasts), the 26 neighbour cells are split across the lanes,
// and the lanes agree on each decision with one ballot.
template <int G, int CAP, bool TRACE>
__global__ void __launch_bounds__(128) k_move_pass(SysPtrs p, int pass) {
  static_assert(G == 1 || G == 2 || G == 4 || G == 8, "group size");
  constexpr int NB = (26 + G - 1) / G;  // neighbour cells per lane
  // Staged neighbour particles per thread: about 27 rho w^3 / G on average;
  // a lane with more than NCL screens from the slots directly.
  constexpr int NCL = G == 1 ? 32 : (G == 2 ? 20 : (G == 4 ? 12 : 8));
  __shared__ Slot stage_mem[NCL][128];

  const DevState *st = p.st;
  const Box *bx = p.box;
  const unsigned long long sweep = st->params.sweep;
  const int layout = (int)(sweep & 1ull);
  const int colour = st->params.perm[pass];
  const float sh[3] = {st->params.shift32[0], st->params.shift32[1], st->params.shift32[2]};
  const double dr = st->dr_max;
  const unsigned long long seed = st->seed;
  const unsigned long long seq = sweep * 8ull + (unsigned long long)pass;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const float L32[3] = {bx->len32[0], bx->len32[1], bx->len32[2]};
  const float H32[3] = {0.5f * bx->len32[0], 0.5f * bx->len32[1], 0.5f * bx->len32[2]};
  const float iw[3] = {bx->inv_w32[0], bx->inv_w32[1], bx->inv_w32[2]};
  const int nc[3] = {bx->nc[0], bx->nc[1], bx->nc[2]};
  const float band = bx->band;
  const int *__restrict__ cnt = p.cnt[layout];
  Slot *__restrict__ slot = p.slot[layout];
  double *__restrict__ pos = p.pos;

  // The first pass of a sweep clears the other layout for the next build.
  if (pass == 0) {
    int *other = p.cnt[layout ^ 1];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x) other[c] = 0;
  }

  const int lane = (int)(threadIdx.x % G);
  const int group = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);
  const int groups = (int)((gridDim.x * blockDim.x) / G);
  const int gbase = (int)((threadIdx.x & 31) & ~(G - 1));
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int hx = nc[0] >> 1, hy = nc[1] >> 1, hz = nc[2] >> 1;
  const int n_active = hx * hy * hz;
  const int cx = colour & 1, cy = (colour >> 1) & 1, cz = (colour >> 2) & 1;

  unsigned acc = 0, rej_o = 0, rej_b = 0, rechecks = 0;

  Slot(*stage)[128] = stage_mem;  // [NCL][threads]: column per thread, conflict-free

  for (int ac = group; ac < n_active; ac += groups) {
    const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
    const int ix = 2 * ax + cx, iy = 2 * ay + cy, iz = 2 * az + cz;
    const int c = ix + nc[0] * (iy + nc[1] * iz);

    // Load phase, so one trial never waits on a chain of memory round trips:
    // (1) the counts of the cell and of this lane's neighbour cells, issued
    // together; (2) every slot of those cells, the neighbours' staged in this
    // thread's column of shared memory; (3) the cell's FP64 positions.
    const int xm = ix == 0 ? nc[0] - 1 : ix - 1, xp = ix == nc[0] - 1 ? 0 : ix + 1;
    const int ym = iy == 0 ? nc[1] - 1 : iy - 1, yp = iy == nc[1] - 1 ? 0 : iy + 1;
    const int zm = iz == 0 ? nc[2] - 1 : iz - 1, zp = iz == nc[2] - 1 ? 0 : iz + 1;
    int nb_c[NB], nb_n[NB];
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const int o26 = lane + q * G;
      nb_c[q] = c;
      if (o26 < 26) {
        const int o = o26 < 13 ? o26 : o26 + 1;  // the centre (13) is the cell itself
        const int a = o / 9, b = (o / 3) % 3, e = o % 3;
        const int x = a == 0 ? xm : (a == 1 ? ix : xp);
        const int y = b == 0 ? ym : (b == 1 ? iy : yp);
        const int z = e == 0 ? zm : (e == 1 ? iz : zp);
        nb_c[q] = x + nc[0] * (y + nc[1] * z);
      }
    }
    const int n = cnt[c];
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const int m = (lane + q * G < 26) ? cnt[nb_c[q]] : 0;
      nb_n[q] = m < CAP ? m : CAP;  // an overfull cell was flagged by the build
    }
    if (n == 0) continue;
    if (n > CAP) {
      if (lane == 0) atomicOr(&p.st->status, ST_CELL_OVERFLOW);
      continue;
    }

    int staged = 0;
#pragma unroll
    for (int q = 0; q < NB; q++) staged += nb_n[q];
    const bool direct = staged > NCL;  // rare: screen straight from the slots
    if (!direct) {
      int w = 0;
#pragma unroll
      for (int q = 0; q < NB; q++)
        for (int k = 0; k < nb_n[q]; k++) stage[w++][threadIdx.x] = slot[(size_t)nb_c[q] * CAP + k];
    }

    // The cell's particles, in id order so the chain does not depend on the
    // order in which the build's atomics filled the slots.
    double qx[CAP], qy[CAP], qz[CAP];
    float fx[CAP], fy[CAP], fz[CAP];
    int qid[CAP], qslot[CAP];
    for (int j = 0; j < n; j++) {
      const Slot sv = slot[(size_t)c * CAP + j];
      int at = j;
      while (at > 0 && qid[at - 1] > sv.id) {
        qid[at] = qid[at - 1];
        qslot[at] = qslot[at - 1];
        at--;
      }
      qid[at] = sv.id;
      qslot[at] = j;
    }
    for (int j = 0; j < n; j++) {
      load_xyz(pos, qid[j], qx[j], qy[j], qz[j]);
      fx[j] = __double2float_rn(qx[j]);
      fy[j] = __double2float_rn(qy[j]);
      fz[j] = __double2float_rn(qz[j]);
    }

    unsigned moved = 0;
    for (int trial = 0; trial < n; trial++) {
      const U32x4 r = draw4(seed, (uint32_t)trial, (uint32_t)c, seq, TAG_MOVE);
      const int s = (int)__umulhi(r.x, (unsigned)n);  // rank of the moving particle
      const double nx = propose_axis(qx[s], centred_offset(r.y), dr, len[0]);
      const double ny = propose_axis(qy[s], centred_offset(r.z), dr, len[1]);
      const double nz = propose_axis(qz[s], centred_offset(r.w), dr, len[2]);
      const float gx = __double2float_rn(nx), gy = __double2float_rn(ny), gz = __double2float_rn(nz);
      int c0, c1, c2;
      float t;
      axis_cell(gx, sh[0], L32[0], iw[0], nc[0], c0, t);
      axis_cell(gy, sh[1], L32[1], iw[1], nc[1], c1, t);
      axis_cell(gz, sh[2], L32[2], iw[2], nc[2], c2, t);
      const unsigned rc_before = rechecks;
      int decision;
      if (c0 != ix || c1 != iy || c2 != iz) {
        decision = 2;  // the move would leave the active cell
      } else {
        bool ov = false;
        for (int j = lane; j < n && !ov; j += G) {
          if (j == s) continue;
          const float dx = wrap_diff(gx - fx[j], L32[0], H32[0]);
          const float dy = wrap_diff(gy - fy[j], L32[1], H32[1]);
          const float dz = wrap_diff(gz - fz[j], L32[2], H32[2]);
          const float r2 = dx * dx + dy * dy + dz * dz;
          if (r2 < 1.0f - band) {
            ov = true;
          } else if (r2 <= 1.0f + band) {
            rechecks++;
            ov = ref_r2(nx, ny, nz, qx[j], qy[j], qz[j], len, half) < 1.0;
          }
        }
        if (!direct) {
          for (int j = 0; j < staged && !ov; j++) {
            const Slot o = stage[j][threadIdx.x];
            const float dx = wrap_diff(gx - o.x, L32[0], H32[0]);
            const float dy = wrap_diff(gy - o.y, L32[1], H32[1]);
            const float dz = wrap_diff(gz - o.z, L32[2], H32[2]);
            ov = screen_pair(dx, dy, dz, band, nx, ny, nz, pos, o.id, len, half, rechecks);
          }
        } else {
#pragma unroll
          for (int q = 0; q < NB; q++) {
            for (int k = 0; k < nb_n[q] && !ov; k++) {
              const Slot o = slot[(size_t)nb_c[q] * CAP + k];
              const float dx = wrap_diff(gx - o.x, L32[0], H32[0]);
              const float dy = wrap_diff(gy - o.y, L32[1], H32[1]);
              const float dz = wrap_diff(gz - o.z, L32[2], H32[2]);
              ov = screen_pair(dx, dy, dz, band, nx, ny, nz, pos, o.id, len, half, rechecks);
            }
          }
        }
        if (G > 1) ov = __ballot_sync(gmask, ov) != 0u;
        decision = ov ? 1 : 0;
      }
      if (decision == 0) {
        qx[s] = nx;
        qy[s] = ny;
        qz[s] = nz;
        fx[s] = gx;
        fy[s] = gy;
        fz[s] = gz;
        moved |= 1u << s;
      }
      if (lane == 0) {
        acc += decision == 0;
        rej_o += decision == 1;
        rej_b += decision == 2;
      }
      if (TRACE) {
        bool any_rc = rechecks != rc_before;
        if (G > 1) any_rc = __ballot_sync(gmask, any_rc) != 0u;
        if (lane == 0) {
          const unsigned long long at = atomicAdd(&p.st->trace_count, 1ull);
          if (at < p.trace_cap) {
            uint32_t *rec = p.trace + 12 * at;
            rec[0] = (uint32_t)seq;
            rec[1] = (uint32_t)c;
            rec[2] = (uint32_t)trial;
            rec[3] = (uint32_t)qid[s];
            rec[4] = r.y;
            rec[5] = r.z;
            rec[6] = r.w;
            rec[7] = (uint32_t)decision;
            rec[8] = __float_as_uint(sh[0]);
            rec[9] = __float_as_uint(sh[1]);
            rec[10] = __float_as_uint(sh[2]);
            rec[11] = any_rc ? 1u : 0u;
          } else {
            atomicOr(&p.st->status, ST_TRACE_FULL);
          }
        }
      }
    }
    if (G > 1) __syncwarp(gmask);
    for (int j = lane; j < n; j += G) {
      if (!((moved >> j) & 1u)) continue;
      double *pp = pos + 4 * (size_t)qid[j];
      pp[1] = qx[j];
      pp[2] = qy[j];
      pp[3] = qz[j];
      slot[(size_t)c * CAP + qslot[j]] = Slot{fx[j], fy[j], fz[j], qid[j]};
    }
  }

  unsigned long long a64 = warp_sum_u64(acc), o64 = warp_sum_u64(rej_o), b64 = warp_sum_u64(rej_b),
                     r64 = warp_sum_u64(rechecks);
  if ((threadIdx.x & 31) == 0) {
    DevState *ws = p.st;
    if (a64) atomicAdd(&ws->acc, a64);
    if (o64) atomicAdd(&ws->rej_overlap, o64);
    if (b64) atomicAdd(&ws->rej_boundary, b64);
    if (r64) atomicAdd(&ws->rechecks, r64);
  }
}

__global__ void k_advance(DevState *st, int n) { st->sweep_base += (unsigned long long)n; }

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
  const double vol = bx->vol;
  const double log_new = log(vol) + centred_offset(r.x) * st->dv_max;
  const double vol_new = exp(log_new);
  const double ratio = vol_new / vol;
  st->vol_sf = pow(ratio, 1. / 3.);
  st->vol_new = vol_new;
  st->vol_ratio = ratio;
  st->vol_u_acc = open_unit(r.y);
  st->vol_overlap = 0;
  st->vol_accept = 0;
  st->vol_moves += 1;
}

// check_overlap(i, sf, sf, sf) for every i (src/moves.c:104-112).  A scale
// factor >= 1 cannot bring a pair closer than it is, so nothing runs then.
__global__ void __launch_bounds__(256) k_vol_scan(SysPtrs p) {
  const DevState *st = p.st;
  const double sf = st->vol_sf;
  if (!(sf < 1.0)) return;
  if (*(volatile const int *)&st->vol_overlap) return;
  const Box *bx = p.box;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int layout = (int)(st->params.sweep & 1ull);
  const int *cnt = p.cnt[layout];
  const Slot *slot = p.slot[layout];
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const float L32[3] = {bx->len32[0], bx->len32[1], bx->len32[2]};
  const float iw[3] = {bx->inv_w32[0], bx->inv_w32[1], bx->inv_w32[2]};
  const float sh[3] = {st->params.shift32[0], st->params.shift32[1], st->params.shift32[2]};
  const int nc[3] = {bx->nc[0], bx->nc[1], bx->nc[2]};
  const float reach = (float)(1.0 / sf) + 1e-3f;
  double x, y, z;
  load_xyz(p.pos, i, x, y, z);
  const float xs[3] = {__double2float_rn(x), __double2float_rn(y), __double2float_rn(z)};
  int ci[3], k[3];
  for (int d = 0; d < 3; d++) {
    float t;
    axis_cell(xs[d], sh[d], L32[d], iw[d], nc[d], ci[d], t);
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
          if (dx * dx + dy * dy + dz * dz > reach * reach) continue;
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
  const double boltz = exp(st->pressure * (bx->vol - st->vol_new) + (p.n + 1) * log(st->vol_ratio));
  if (st->vol_u_acc >= boltz) return;
  const double rho = p.n / st->vol_new;
  const double cell_vol = st->per_cell / rho;
  const double cell_size = pow(cell_vol, 1. / 3.);
  double lmax = 0.0;
  for (int d = 0; d < 3; d++) {
    const double len = st->cells[d] * cell_size;
    int nc = 2 * (int)floor(len / (2.0 * (1.0 + margin)));
    if (nc > st->nc_alloc[d]) nc = st->nc_alloc[d];
    if (nc < 4) {
      atomicOr(&st->status, ST_BAD_CELL);
      return;
    }
    bx->len[d] = len;
    bx->half[d] = len / 2.0;
    bx->len32[d] = (float)len;
    bx->inv_w32[d] = (float)(nc / len);
    bx->w32[d] = (float)(len / nc);
    bx->nc[d] = nc;
    lmax = len > lmax ? len : lmax;
  }
  bx->ncell = bx->nc[0] * bx->nc[1] * bx->nc[2];
  bx->vol = st->cells[0] * st->cells[1] * st->cells[2] * cell_vol;
  bx->rho = rho;
  bx->band = (float)(5.9604644775390625e-08 * (48.0 * lmax + 16.0) + 1e-6);
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

void launch_build(const SysPtrs &p, long long sweep_offset, int num_sms, cudaStream_t s) {
  (void)num_sms;
  const int blocks = (p.n + 255) / 256;
  k_build<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(p, sweep_offset);
}

// Groups per pass = active cells (an eighth of the grid); one wave when the
// occupancy allows it, grid-stride otherwise.
template <int G, int CAP>
static int pass_blocks_for(int ncell_alloc, int num_sms) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_move_pass<G, CAP, false>, 128, 0);
  if (per_sm < 1) per_sm = 1;
  const long long threads = (long long)(ncell_alloc / 8) * G;
  const int need = (int)((threads + 127) / 128);
  const int cap = per_sm * num_sms;
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

template <int G, int CAP>
static void launch_gc(const SysPtrs &p, int pass, bool trace, int grid, cudaStream_t s) {
  if (trace) k_move_pass<G, CAP, true><<<grid, 128, 0, s>>>(p, pass);
  else k_move_pass<G, CAP, false><<<grid, 128, 0, s>>>(p, pass);
}

template <int G>
static void launch_g(const SysPtrs &p, int pass, bool trace, int grid, cudaStream_t s) {
  switch (p.cap) {
    case 8: launch_gc<G, 8>(p, pass, trace, grid, s); break;
    case 16: launch_gc<G, 16>(p, pass, trace, grid, s); break;
    default: launch_gc<G, 32>(p, pass, trace, grid, s); break;
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

void launch_advance(const SysPtrs &p, int n_sweeps, cudaStream_t s) { k_advance<<<1, 1, 0, s>>>(p.st, n_sweeps); }

}  // namespace hsmc
