// One colour pass of the checkerboard sweep (part_move / check_overlap,
// src/moves.c:27-80 and 157-212, for all cells of one colour at once).
//
// A group of G lanes owns one active cell at a time.  Every lane keeps its
// own copy of the cell's particles, so the trial sequence needs no
// broadcasts; the 26 neighbour cells are split across the lanes and the
// lanes agree on each decision with one ballot.  Per cell:
//   load phase  counts of the cell and of the lane's neighbour cells (issued
//               together), then every slot of those cells -- the neighbours'
//               staged in the thread's column of shared memory as grid
//               coordinates with their periodic image applied -- then the
//               cell's FP64 positions;
//   trials      n trials (n = particles in the cell), each on the particle
//               of rank floor(u n) by id: FP64 proposal, confinement to the
//               cell, single-precision screen four candidates at a time, FP64
//               re-evaluation of any pair within the guard band of contact.
#include "engine.cuh"

namespace hsmc {

// Neighbour offsets of the 26 cells around a cell, packed (dx+1) | (dy+1)<<2
// | (dz+1)<<4, in the order x-major, the cell itself left out.
__constant__ unsigned char c_nbr[26] = {
    0x00, 0x10, 0x20, 0x04, 0x14, 0x24, 0x08, 0x18, 0x28, 0x01, 0x11, 0x21, 0x05,
    0x25, 0x09, 0x19, 0x29, 0x02, 0x12, 0x22, 0x06, 0x16, 0x26, 0x0a, 0x1a, 0x2a};

// Grid coordinate of a candidate relative to the active cell: the slot's t
// plus the periodic image of the neighbour cell it sits in.
__device__ __forceinline__ float4 staged_coord(const Slot &o, float ix, float iy, float iz) {
  return make_float4(__fadd_rn(o.x, ix), __fadd_rn(o.y, iy), __fadd_rn(o.z, iz), __int_as_float(o.id));
}

__device__ __forceinline__ float dist2(float ux, float uy, float uz, const float4 &q) {
  const float dx = ux - q.x, dy = uy - q.y, dz = uz - q.z;
  return dx * dx + dy * dy + dz * dz;
}

template <int G, int CAP, bool TRACE, bool BATCH>
__global__ void __launch_bounds__(128, 4) k_move_pass(SysPtrs p1, const SysPtrs *reps, int pass) {
  // In a batch, blockIdx.y is the replica (see k_build).
  const SysPtrs p = BATCH ? reps[blockIdx.y] : p1;
  const uint32_t rep = BATCH ? blockIdx.y : 0u;
  static_assert(G == 1 || G == 2 || G == 4 || G == 8, "group size");
  constexpr int NB = (26 + G - 1) / G;  // neighbour cells per lane
  // Staged neighbour particles per thread: about 27 rho w^3 / G on average;
  // a lane with more than NCL screens from the slots directly.
  constexpr int NCL = G == 1 ? 32 : (G == 2 ? 20 : (G == 4 ? 12 : 8));
  __shared__ float4 stage[NCL][128];  // column per thread: conflict-free

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
  const float iw[3] = {bx->inv_w32[0], bx->inv_w32[1], bx->inv_w32[2]};
  const int nc[3] = {bx->nc[0], bx->nc[1], bx->nc[2]};
  const float band = bx->band;
  const float lo = 1.0f - band, hi = 1.0f + band;
  const int *__restrict__ cnt = p.cnt[layout];
  Slot *__restrict__ slot = p.slot[layout];
  double *__restrict__ pos = p.pos;

  // The first pass of a sweep clears the other layout for the next build.
  if (pass == 0) {
    int *other = p.cnt[layout ^ 1];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x) other[c] = 0;
    if (blockIdx.x == 0 && threadIdx.x < 8 * NBUCKET) (&p.st->list_len[layout ^ 1][0][0])[threadIdx.x] = 0;
  }

  const int tid = (int)threadIdx.x;
  const int lane = tid % G;
  const int group = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);
  const int groups = (int)((gridDim.x * blockDim.x) / G);
  const int gbase = (tid & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);

  unsigned acc = 0, rej_o = 0, rej_b = 0, rechecks = 0;

  // The non-empty cells of this colour, fullest first: consecutive groups
  // (the lanes of one warp) get cells with the same number of trials.
  int blen[NBUCKET];
  int n_list = 0;
#pragma unroll
  for (int b = 0; b < NBUCKET; b++) {
    blen[b] = st->list_len[layout][colour][b];
    n_list += blen[b];
  }
  const size_t seg = (size_t)(p.ncell_alloc / 8);
  const int *__restrict__ lists = p.list[layout] + (size_t)colour * NBUCKET * seg;

  for (int li = group; li < n_list; li += groups) {
    int b = NBUCKET - 1, off = li;
    while (off >= blen[b]) {
      off -= blen[b];
      b--;
    }
    const int c = lists[(size_t)b * seg + off];
    const int ix = c % nc[0], iyz = c / nc[0], iy = iyz % nc[1], iz = iyz / nc[1];

    // (1) counts of the cell and of this lane's neighbour cells, issued together
    int nb_c[NB], nb_n[NB];
    unsigned nb_code[NB];
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const int o26 = lane + q * G;
      nb_c[q] = c;
      nb_code[q] = 0x15u;  // offset (0,0,0)
      if (o26 < 26) {
        const unsigned code = c_nbr[o26];
        nb_code[q] = code;
        int x = ix + (int)(code & 3u) - 1, y = iy + (int)((code >> 2) & 3u) - 1, z = iz + (int)(code >> 4) - 1;
        x += x < 0 ? nc[0] : (x >= nc[0] ? -nc[0] : 0);
        y += y < 0 ? nc[1] : (y >= nc[1] ? -nc[1] : 0);
        z += z < 0 ? nc[2] : (z >= nc[2] ? -nc[2] : 0);
        nb_c[q] = x + nc[0] * (y + nc[1] * z);
      }
    }
    const int n = cnt[c];
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const int m = (lane + q * G < 26) ? cnt[nb_c[q]] : 0;
      nb_n[q] = m < CAP ? m : CAP;  // an overfull cell was flagged by the build
    }
    if (n > CAP) {
      if (lane == 0) atomicOr(&p.st->status, ST_CELL_OVERFLOW);
      continue;
    }

    // (2) slots: stage the neighbours with their periodic images applied
    int staged = 0;
#pragma unroll
    for (int q = 0; q < NB; q++) staged += nb_n[q];
    const bool direct = staged > NCL;  // rare: screen straight from the slots
    if (!direct) {
      int w = 0;
#pragma unroll
      for (int q = 0; q < NB; q++) {
        if (nb_n[q] == 0) continue;
        const unsigned code = nb_code[q];
        const int ox = (int)(code & 3u) - 1, oy = (int)((code >> 2) & 3u) - 1, oz = (int)(code >> 4) - 1;
        const float imx = (ix + ox < 0) ? -L32[0] : (ix + ox >= nc[0] ? L32[0] : 0.f);
        const float imy = (iy + oy < 0) ? -L32[1] : (iy + oy >= nc[1] ? L32[1] : 0.f);
        const float imz = (iz + oz < 0) ? -L32[2] : (iz + oz >= nc[2] ? L32[2] : 0.f);
        for (int k = 0; k < nb_n[q]; k++)
          stage[w++][tid] = staged_coord(slot[(size_t)nb_c[q] * CAP + k], imx, imy, imz);
      }
    }

    // (3) the cell's particles in id order (the chain must not depend on the
    // order the build's atomics filled the slots), with FP64 positions
    double qx[CAP], qy[CAP], qz[CAP];
    float tx[CAP], ty[CAP], tz[CAP];
    int qid[CAP], qslot[CAP];
    for (int j = 0; j < n; j++) {
      const Slot sv = slot[(size_t)c * CAP + j];
      int at = j;
      while (at > 0 && qid[at - 1] > sv.id) {
        qid[at] = qid[at - 1];
        qslot[at] = qslot[at - 1];
        tx[at] = tx[at - 1];
        ty[at] = ty[at - 1];
        tz[at] = tz[at - 1];
        at--;
      }
      qid[at] = sv.id;
      qslot[at] = j;
      tx[at] = sv.x;
      ty[at] = sv.y;
      tz[at] = sv.z;
    }
    for (int j = 0; j < n; j++) load_xyz(pos, qid[j], qx[j], qy[j], qz[j]);

    unsigned moved = 0;
    for (int trial = 0; trial < n; trial++) {
      const U32x4 r = draw4(seed, (rep << 8) | (uint32_t)trial, (uint32_t)c, seq, TAG_MOVE);
      const int s = (int)__umulhi(r.x, (unsigned)n);  // rank of the moving particle
      const double nx = propose_axis(qx[s], centred_offset(r.y), dr, len[0]);
      const double ny = propose_axis(qy[s], centred_offset(r.z), dr, len[1]);
      const double nz = propose_axis(qz[s], centred_offset(r.w), dr, len[2]);
      int c0, c1, c2;
      float ux, uy, uz;
      axis_cell(__double2float_rn(nx), sh[0], L32[0], iw[0], nc[0], c0, ux);
      axis_cell(__double2float_rn(ny), sh[1], L32[1], iw[1], nc[1], c1, uy);
      axis_cell(__double2float_rn(nz), sh[2], L32[2], iw[2], nc[2], c2, uz);
      const unsigned rc_before = rechecks;
      int decision;
      if (c0 != ix || c1 != iy || c2 != iz) {
        decision = 2;  // the move would leave the active cell
      } else {
        bool ov = false;
        // the rest of the cell
        for (int j = lane; j < n && !ov; j += G) {
          if (j == s) continue;
          const float dx = ux - tx[j], dy = uy - ty[j], dz = uz - tz[j];
          const float r2 = dx * dx + dy * dy + dz * dz;
          if (r2 < lo) {
            ov = true;
          } else if (r2 <= hi) {
            rechecks++;
            ov = ref_r2(nx, ny, nz, qx[j], qy[j], qz[j], len, half) < 1.0;
          }
        }
        if (!direct) {
          int j = 0;
          for (; j + 4 <= staged && !ov; j += 4) {
            const float4 a0 = stage[j][tid], a1 = stage[j + 1][tid], a2 = stage[j + 2][tid], a3 = stage[j + 3][tid];
            const float r0 = dist2(ux, uy, uz, a0), r1 = dist2(ux, uy, uz, a1);
            const float r2 = dist2(ux, uy, uz, a2), r3 = dist2(ux, uy, uz, a3);
            if (fminf(fminf(r0, r1), fminf(r2, r3)) <= hi) {
              const float rr[4] = {r0, r1, r2, r3};
              const float4 aa[4] = {a0, a1, a2, a3};
              for (int u = 0; u < 4 && !ov; u++) {
                if (rr[u] < lo) {
                  ov = true;
                } else if (rr[u] <= hi) {
                  rechecks++;
                  double ox, oy, oz;
                  load_xyz(pos, __float_as_int(aa[u].w), ox, oy, oz);
                  ov = ref_r2(nx, ny, nz, ox, oy, oz, len, half) < 1.0;
                }
              }
            }
          }
          for (; j < staged && !ov; j++) {
            const float4 a = stage[j][tid];
            const float r2 = dist2(ux, uy, uz, a);
            if (r2 < lo) {
              ov = true;
            } else if (r2 <= hi) {
              rechecks++;
              double ox, oy, oz;
              load_xyz(pos, __float_as_int(a.w), ox, oy, oz);
              ov = ref_r2(nx, ny, nz, ox, oy, oz, len, half) < 1.0;
            }
          }
        } else {
#pragma unroll
          for (int q = 0; q < NB; q++) {
            if (nb_n[q] == 0) continue;
            const unsigned code = nb_code[q];
            const int ox = (int)(code & 3u) - 1, oy = (int)((code >> 2) & 3u) - 1, oz = (int)(code >> 4) - 1;
            const float imx = (ix + ox < 0) ? -L32[0] : (ix + ox >= nc[0] ? L32[0] : 0.f);
            const float imy = (iy + oy < 0) ? -L32[1] : (iy + oy >= nc[1] ? L32[1] : 0.f);
            const float imz = (iz + oz < 0) ? -L32[2] : (iz + oz >= nc[2] ? L32[2] : 0.f);
            for (int k = 0; k < nb_n[q] && !ov; k++) {
              const float4 a = staged_coord(slot[(size_t)nb_c[q] * CAP + k], imx, imy, imz);
              const float r2 = dist2(ux, uy, uz, a);
              if (r2 < lo) {
                ov = true;
              } else if (r2 <= hi) {
                rechecks++;
                double px, py, pz;
                load_xyz(pos, __float_as_int(a.w), px, py, pz);
                ov = ref_r2(nx, ny, nz, px, py, pz, len, half) < 1.0;
              }
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
        tx[s] = ux;
        ty[s] = uy;
        tz[s] = uz;
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
      slot[(size_t)c * CAP + qslot[j]] = Slot{tx[j], ty[j], tz[j], qid[j]};
    }
  }

  const unsigned long long a64 = warp_sum_u64(acc), o64 = warp_sum_u64(rej_o), b64 = warp_sum_u64(rej_b),
                           r64 = warp_sum_u64(rechecks);
  if ((threadIdx.x & 31) == 0) {
    DevState *ws = p.st;
    if (a64) atomicAdd(&ws->acc, a64);
    if (o64) atomicAdd(&ws->rej_overlap, o64);
    if (b64) atomicAdd(&ws->rej_boundary, b64);
    if (r64) atomicAdd(&ws->rechecks, r64);
  }
}

// ------------------------------------------------------------------ launch
// Groups per pass = active cells (an eighth of the grid); one wave when the
// occupancy allows it, grid-stride otherwise.
template <int G, int CAP>
static int pass_blocks_for(int ncell_alloc, int num_sms) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_move_pass<G, CAP, false, false>, 128, 0);
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
  if (trace) k_move_pass<G, CAP, true, false><<<grid, 128, 0, s>>>(p, nullptr, pass);
  else k_move_pass<G, CAP, false, false><<<grid, 128, 0, s>>>(p, nullptr, pass);
}

template <int G, int CAP>
static void launch_batch_gc(const SysPtrs *reps, int n_reps, int pass, int grid_x, cudaStream_t s) {
  k_move_pass<G, CAP, false, true><<<dim3((unsigned)grid_x, (unsigned)n_reps), 128, 0, s>>>(SysPtrs{}, reps, pass);
}

// Blocks per replica for the batched pass: enough groups for the largest
// replica's colour list; blocks past a smaller replica's list exit at once.
int move_pass_grid_batch(int group, int max_ncell) {
  const long long threads = (long long)(max_ncell / 8) * group;
  const int x = (int)((threads + 127) / 128);
  return x > 0 ? x : 1;
}

void launch_move_pass_batch(const SysPtrs *reps, int n_reps, int cap, int pass, int group, int grid_x,
                            cudaStream_t s) {
#define HSMC_BATCH_CAP(G)                                                      \
  switch (cap) {                                                               \
    case 8: launch_batch_gc<G, 8>(reps, n_reps, pass, grid_x, s); break;       \
    case 16: launch_batch_gc<G, 16>(reps, n_reps, pass, grid_x, s); break;     \
    default: launch_batch_gc<G, 32>(reps, n_reps, pass, grid_x, s); break;     \
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

void launch_move_pass(const SysPtrs &p, int pass, int group, bool trace, int grid, cudaStream_t s) {
  switch (group) {
    case 1: launch_g<1>(p, pass, trace, grid, s); break;
    case 2: launch_g<2>(p, pass, trace, grid, s); break;
    case 4: launch_g<4>(p, pass, trace, grid, s); break;
    default: launch_g<8>(p, pass, trace, grid, s); break;
  }
}

}  // namespace hsmc
