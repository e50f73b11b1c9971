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

// One pair of the single-precision screen: d = t_mover - t_other.  Returns
// the overlap decision, re-evaluating in FP64 (reference arithmetic, mover
// first as in check_overlap) when r^2 is within the band of 1.
__device__ __forceinline__ bool pair_overlaps(float dx, float dy, float dz, float band, double mx, double my,
                                              double mz, double ox, double oy, double oz, const double *len,
                                              const double *half, unsigned long long &rechecks) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  if (r2 < 1.0f - band) return true;
  if (r2 > 1.0f + band) return false;
  rechecks++;
  return ref_r2(mx, my, mz, ox, oy, oz, len, half) < 1.0;
}

__device__ __forceinline__ void load_xyz(const double *pos, int id, double &x, double &y, double &z) {
  const double2 a = *reinterpret_cast<const double2 *>(pos + 4 * (size_t)id);
  const double2 b = *reinterpret_cast<const double2 *>(pos + 4 * (size_t)id + 2);
  x = a.y;
  y = b.x;
  z = b.y;
}

template <int G, int CAP, int NCAND, bool TRACE>
__global__ void __launch_bounds__(256) k_move_pass(SysPtrs p, int pass) {
  static_assert(CAP <= G, "each lane holds at most one particle of its cell");
  static_assert(G == 8 || G == 16 || G == 32, "group size");
  constexpr int GPB = 256 / G;               // groups per block
  constexpr int NB = (26 + G - 1) / G;        // neighbour cells per lane
  __shared__ float4 cand[GPB][NCAND];

  const DevState *st = p.st;
  const Box *bx = p.box;
  const unsigned long long sweep = st->params.sweep;
  const int layout = (int)(sweep & 1ull);
  const int colour = st->params.perm[pass];
  const float sh0 = st->params.shift32[0], sh1 = st->params.shift32[1], sh2 = st->params.shift32[2];
  const double dr = st->dr_max;
  const unsigned long long seed = st->seed;
  const unsigned long long seq = sweep * 8ull + (unsigned long long)pass;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const float L32[3] = {bx->len32[0], bx->len32[1], bx->len32[2]};
  const float iw[3] = {bx->inv_w32[0], bx->inv_w32[1], bx->inv_w32[2]};
  const int nc[3] = {bx->nc[0], bx->nc[1], bx->nc[2]};
  const float band = bx->band;
  const int *__restrict__ cnt = p.cnt[layout];
  Slot *__restrict__ slot = p.slot[layout];
  const double *__restrict__ pos = p.pos;

  // The first pass of a sweep clears the other layout for the next build.
  if (pass == 0) {
    int *other = p.cnt[layout ^ 1];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x) other[c] = 0;
  }

  const int lane = threadIdx.x % G;
  const int gib = threadIdx.x / G;
  const int gbase = (threadIdx.x & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int hx = nc[0] >> 1, hy = nc[1] >> 1, hz = nc[2] >> 1;
  const int n_active = hx * hy * hz;
  const int cx = colour & 1, cy = (colour >> 1) & 1, cz = (colour >> 2) & 1;

  unsigned long long acc = 0, rej_o = 0, rej_b = 0, rechecks = 0;

  for (int ac = blockIdx.x * GPB + gib; ac < n_active; ac += gridDim.x * GPB) {
    const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
    const int ix = 2 * ax + cx, iy = 2 * ay + cy, iz = 2 * az + cz;
    const int c = ix + nc[0] * (iy + nc[1] * iz);
    const int n = cnt[c];
    if (n == 0) continue;
    if (n > CAP) {
      if (lane == 0) atomicOr(&p.st->status, ST_CELL_OVERFLOW);
      continue;
    }

    // Own particles: lane l < n holds particle l of the cell.
    double px = 0.0, py = 0.0, pz = 0.0;
    float tx = 0.f, ty = 0.f, tz = 0.f;
    int pid = 0x7fffffff;
    if (lane < n) {
      const Slot sv = slot[(size_t)c * CAP + lane];
      pid = sv.id;
      load_xyz(pos, pid, px, py, pz);
      int ci;
      axis_cell(sv.x, sh0, L32[0], iw[0], nc[0], ci, tx);
      axis_cell(sv.y, sh1, L32[1], iw[1], nc[1], ci, ty);
      axis_cell(sv.z, sh2, L32[2], iw[2], nc[2], ci, tz);
    }
    // Moves visit the cell's particles by rank of id, so the chain does not
    // depend on the order atomics filled the slots.
    int rank = 0;
#pragma unroll
    for (int j = 0; j < G; j++) {
      const int o = __shfl_sync(gmask, pid, j, G);
      rank += (o < pid) ? 1 : 0;
    }

    // Stage the 26 neighbour cells' particles in shared memory, as grid
    // coordinates t with the periodic image already applied.
    int nb_c[NB];
    float nb_img[NB][3];
    int nb_n[NB];
    int mine = 0;
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const int o26 = lane + q * G;
      nb_n[q] = 0;
      nb_c[q] = 0;
      if (o26 < 26) {
        const int o = o26 < 13 ? o26 : o26 + 1;  // skip the centre (13)
        const int off[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
        const int base[3] = {ix, iy, iz};
        int idx[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          int v = base[d] + off[d];
          float img = 0.f;
          if (v < 0) {
            v += nc[d];
            img = -L32[d];
          } else if (v >= nc[d]) {
            v -= nc[d];
            img = L32[d];
          }
          idx[d] = v;
          nb_img[q][d] = img;
        }
        nb_c[q] = idx[0] + nc[0] * (idx[1] + nc[1] * idx[2]);
        const int m = cnt[nb_c[q]];
        nb_n[q] = m < CAP ? m : CAP;  // an overfull cell was flagged by the build
        mine += nb_n[q];
      }
    }
    int incl = mine;
#pragma unroll
    for (int d = 1; d < G; d <<= 1) {
      const int v = __shfl_up_sync(gmask, incl, d, G);
      if (lane >= d) incl += v;
    }
    const int total = __shfl_sync(gmask, incl, G - 1, G);
    const bool staged = total <= NCAND;
    if (staged) {
      int w = incl - mine;
#pragma unroll
      for (int q = 0; q < NB; q++) {
        for (int k = 0; k < nb_n[q]; k++) {
          const Slot sv = slot[(size_t)nb_c[q] * CAP + k];
          int ci;
          float a0, a1, a2;
          axis_cell(sv.x, sh0, L32[0], iw[0], nc[0], ci, a0);
          axis_cell(sv.y, sh1, L32[1], iw[1], nc[1], ci, a1);
          axis_cell(sv.z, sh2, L32[2], iw[2], nc[2], ci, a2);
          cand[gib][w++] = make_float4(__fadd_rn(a0, nb_img[q][0]), __fadd_rn(a1, nb_img[q][1]),
                                       __fadd_rn(a2, nb_img[q][2]), __int_as_float(sv.id));
        }
      }
    }
    __syncwarp(gmask);

    bool moved = false;
    for (int trial = 0; trial < n; trial++) {
      const U32x4 r = draw4(seed, (uint32_t)trial, (uint32_t)c, seq, TAG_MOVE);
      const int pick = (int)__umulhi(r.x, (unsigned)n);
      const unsigned sel = __ballot_sync(gmask, lane < n && rank == pick);
      const int ml = __ffs(sel >> gbase) - 1;
      const double mx = __shfl_sync(gmask, px, ml, G);
      const double my = __shfl_sync(gmask, py, ml, G);
      const double mz = __shfl_sync(gmask, pz, ml, G);
      const double qx = propose_axis(mx, centred_offset(r.y), dr, len[0]);
      const double qy = propose_axis(my, centred_offset(r.z), dr, len[1]);
      const double qz = propose_axis(mz, centred_offset(r.w), dr, len[2]);
      int c0, c1, c2;
      float ux, uy, uz;
      axis_cell(__double2float_rn(qx), sh0, L32[0], iw[0], nc[0], c0, ux);
      axis_cell(__double2float_rn(qy), sh1, L32[1], iw[1], nc[1], c1, uy);
      axis_cell(__double2float_rn(qz), sh2, L32[2], iw[2], nc[2], c2, uz);
      int decision;
      unsigned rc_before = (unsigned)rechecks;
      if (c0 != ix || c1 != iy || c2 != iz) {
        decision = 2;
      } else {
        bool ov = false;
        if (lane < n && lane != ml)
          ov = pair_overlaps(ux - tx, uy - ty, uz - tz, band, qx, qy, qz, px, py, pz, len, half, rechecks);
        if (staged) {
          for (int j = lane; j < total && !ov; j += G) {
            const float4 cd = cand[gib][j];
            const float dx = ux - cd.x, dy = uy - cd.y, dz = uz - cd.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < 1.0f - band) {
              ov = true;
            } else if (r2 <= 1.0f + band) {
              double ox, oy, oz;
              load_xyz(pos, __float_as_int(cd.w), ox, oy, oz);
              rechecks++;
              ov = ref_r2(qx, qy, qz, ox, oy, oz, len, half) < 1.0;
            }
          }
        } else {
          // Too many neighbours to stage: read them straight from the slots.
#pragma unroll
          for (int q = 0; q < NB; q++) {
            for (int k = 0; k < nb_n[q] && !ov; k++) {
              const Slot sv = slot[(size_t)nb_c[q] * CAP + k];
              int ci;
              float a0, a1, a2;
              axis_cell(sv.x, sh0, L32[0], iw[0], nc[0], ci, a0);
              axis_cell(sv.y, sh1, L32[1], iw[1], nc[1], ci, a1);
              axis_cell(sv.z, sh2, L32[2], iw[2], nc[2], ci, a2);
              const float dx = ux - __fadd_rn(a0, nb_img[q][0]);
              const float dy = uy - __fadd_rn(a1, nb_img[q][1]);
              const float dz = uz - __fadd_rn(a2, nb_img[q][2]);
              const float r2 = dx * dx + dy * dy + dz * dz;
              if (r2 < 1.0f - band) {
                ov = true;
              } else if (r2 <= 1.0f + band) {
                double ox, oy, oz;
                load_xyz(pos, sv.id, ox, oy, oz);
                rechecks++;
                ov = ref_r2(qx, qy, qz, ox, oy, oz, len, half) < 1.0;
              }
            }
          }
        }
        decision = __ballot_sync(gmask, ov) ? 1 : 0;
      }
      if (decision == 0 && lane == ml) {
        px = qx;
        py = qy;
        pz = qz;
        tx = ux;
        ty = uy;
        tz = uz;
        moved = true;
      }
      if (lane == 0) {
        acc += decision == 0;
        rej_o += decision == 1;
        rej_b += decision == 2;
      }
      if (TRACE) {
        const unsigned any_rc = __ballot_sync(gmask, (unsigned)rechecks != rc_before);
        const int mid = __shfl_sync(gmask, pid, ml, G);
        if (lane == 0) {
          const unsigned long long at = atomicAdd(&p.st->trace_count, 1ull);
          if (at < p.trace_cap) {
            uint32_t *rec = p.trace + 12 * at;
            rec[0] = (uint32_t)seq;
            rec[1] = (uint32_t)c;
            rec[2] = (uint32_t)trial;
            rec[3] = (uint32_t)mid;
            rec[4] = r.y;
            rec[5] = r.z;
            rec[6] = r.w;
            rec[7] = (uint32_t)decision;
            rec[8] = __float_as_uint(sh0);
            rec[9] = __float_as_uint(sh1);
            rec[10] = __float_as_uint(sh2);
            rec[11] = any_rc ? 1u : 0u;
          } else {
            atomicOr(&p.st->status, ST_TRACE_FULL);
          }
        }
      }
    }
    __syncwarp(gmask);

    if (moved) {
      double *pp = p.pos + 4 * (size_t)pid;
      pp[1] = px;
      pp[2] = py;
      pp[3] = pz;
      slot[(size_t)c * CAP + lane] = Slot{__double2float_rn(px), __double2float_rn(py), __double2float_rn(pz), pid};
    }
  }

  acc = warp_sum_u64(acc);
  rej_o = warp_sum_u64(rej_o);
  rej_b = warp_sum_u64(rej_b);
  rechecks = warp_sum_u64(rechecks);
  if ((threadIdx.x & 31) == 0) {
    DevState *ws = p.st;
    if (acc) atomicAdd(&ws->acc, acc);
    if (rej_o) atomicAdd(&ws->rej_overlap, rej_o);
    if (rej_b) atomicAdd(&ws->rej_boundary, rej_b);
    if (rechecks) atomicAdd(&ws->rechecks, rechecks);
  }
}

__global__ void k_advance(DevState *st, int n) { st->sweep_base += (unsigned long long)n; }

// ------------------------------------------------------------------ launch

void launch_build(const SysPtrs &p, long long sweep_offset, int num_sms, cudaStream_t s) {
  (void)num_sms;
  const int blocks = (p.n + 255) / 256;
  k_build<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(p, sweep_offset);
}

template <int G, int CAP, int NCAND, bool TRACE>
static int pass_blocks_for(int ncell_alloc, int num_sms) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_move_pass<G, CAP, NCAND, TRACE>, 256, 0);
  if (per_sm < 1) per_sm = 1;
  const int groups = ncell_alloc / 8;
  const int need = (groups + (256 / G) - 1) / (256 / G);
  const int cap = per_sm * num_sms;
  return need < cap ? (need > 0 ? need : 1) : cap;
}

int move_pass_grid(int group, int cap, int ncell_alloc, int num_sms) {
  (void)cap;
  switch (group) {
    case 8: return pass_blocks_for<8, 8, 48, false>(ncell_alloc, num_sms);
    case 16: return pass_blocks_for<16, 16, 96, false>(ncell_alloc, num_sms);
    default: return pass_blocks_for<32, 32, 192, false>(ncell_alloc, num_sms);
  }
}

void launch_move_pass(const SysPtrs &p, int pass, int group, bool trace, int grid, cudaStream_t s) {
  if (group == 8) {
    if (trace) k_move_pass<8, 8, 48, true><<<grid, 256, 0, s>>>(p, pass);
    else k_move_pass<8, 8, 48, false><<<grid, 256, 0, s>>>(p, pass);
  } else if (group == 16) {
    if (trace) k_move_pass<16, 16, 96, true><<<grid, 256, 0, s>>>(p, pass);
    else k_move_pass<16, 16, 96, false><<<grid, 256, 0, s>>>(p, pass);
  } else {
    if (trace) k_move_pass<32, 32, 192, true><<<grid, 256, 0, s>>>(p, pass);
    else k_move_pass<32, 32, 192, false><<<grid, 256, 0, s>>>(p, pass);
  }
}

void launch_advance(const SysPtrs &p, int n_sweeps, cudaStream_t s) { k_advance<<<1, 1, 0, s>>>(p.st, n_sweeps); }

}  // namespace hsmc
